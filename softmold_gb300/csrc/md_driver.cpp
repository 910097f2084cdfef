// The `MD <name>` drop-in driver on top of the C ABI.
//
// Same invocation, inputs, outputs and loop cadence as the reference driver
// (MD.cpp:72-755): read <name>.mpd, initial forces, the t=0 measurement or the
// restart half-kick, then the loop with .mpd/.xyz stores every storeInterval,
// measurements every measureInterval, the temperature ramp, and the MC box
// move every 8 steps; at the end resizeHist_<name>.dat, the acceptance ratio on
// stderr and kEnergyDensity_<name>.dat.  The device advances in chunks between
// those events; the state is read back only at stores and measurements.
#include <cmath>
#include <cstdio>
#include <ctime>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/softmold_gb300.h"
#include "mpd_io.h"
#include "observables.h"

namespace {

std::string last_error() {
  char buf[1024];
  smd_last_error(buf, sizeof buf);
  return buf;
}

int die(const std::string& what) {
  std::cout << "Error(MD): " << what << ": " << last_error() << "\n";
  return 1;
}

// Terms of one external-field residue, in the order the reference applies
// them (kind = the molecule type; 8 constants each):
//   BOUNDARY (Blob::doBoundaryForce, include/system.h:2335-2349): one term per
//     bead, constants {dim, centre, -, k};
//   FLOATING_BASE (doFloatingBaseForce, :2403-2422): one term per bead, the 6
//     constants of the bead's type, then the residue's first constant (the
//     potential's z offset, doFloatingBasePotential :2437);
//   ZTORQUE (doZTorqueForce, :2626-2664): one term per bond (l, l+1) of each
//     chain but its last, constants {a, b, c, z0};
//   ZPOWERPOTENTIAL (doZPowerForce, :2693-2716): one term per bead of each
//     {start, count} block, constants {c0, c1};
//   BALL (doBallForce, :1937-1971): one term per bond (the residue's first
//     bond's first bead, this bond's second), constants {r0, k, this bond's
//     first} (the potential, doBallPotential :2750-2779, takes each bond's
//     own first).
void field_terms(const smd::Molecule& m, const std::vector<int>& type, std::vector<int>& idx,
                 std::vector<double>& cs) {
  auto push = [&](int a, int b, std::initializer_list<double> c) {
    idx.insert(idx.end(), {m.type, a, b});
    std::vector<double> v(c);
    v.resize(8, 0.0);
    cs.insert(cs.end(), v.begin(), v.end());
  };
  const std::vector<double>& C = m.constants;
  for (const auto& b : m.bonds) {
    if (m.type == smd::MOL_BOUNDARY) {
      push(b[0], -1, {C[0], C[1], C[2], C[3]});
    } else if (m.type == smd::MOL_FLOATING_BASE) {
      const double* t = C.data() + 6 * type[b[0]];
      push(b[0], -1, {t[0], t[1], t[2], t[3], t[4], t[5], C[0]});
    } else if (m.type == smd::MOL_ZPOWERPOTENTIAL) {
      for (int k = b[0]; k < b[0] + b[1]; ++k) push(k, -1, {C[0], C[1]});
    } else if (m.type == smd::MOL_BALL) {
      push(m.bonds[0][0], b[1], {C[0], C[1], (double)b[0]});
    } else {
      for (int k = b[0]; k < b[0] + b[2] * b[1]; k += b[2])
        for (int l = k; l < k + b[2] - 2; ++l) push(l, l + 1, {C[0], C[1], C[2], C[3]});
    }
  }
}

}  // namespace

extern "C" int smd_md_main(const char* name_c, int precision) {
  const std::string name(name_c);
  smd::MpdSystem S;
  std::string err;
  if (smd::mpd_read_file(name + ".mpd", S, err)) {
    std::cout << err << "\n";
    return 1;
  }
  // residues on the device path
  std::vector<int> blocks;
  std::vector<double> consts;
  std::vector<int> sphere_idx, bond_idx, bend_idx;
  std::vector<double> bond_c, bend_c;
  std::vector<int> field_idx;
  std::vector<double> field_c;
  const std::vector<double>* sphere_consts = nullptr;
  bool nanocore = false;
  int n_bead_res = 0;  // BEAD and NANOCORE residues: the beadPotential_ output (dataExtraction.h:1031-1040)
  for (const smd::Molecule& m : S.mol) {
    if (m.type == smd::MOL_CHAIN) {
      for (const auto& b : m.bonds) {
        blocks.insert(blocks.end(), {b[0], b[1], b[2]});
        consts.insert(consts.end(), m.constants.begin(), m.constants.begin() + 4);
      }
    } else if (m.type == smd::MOL_BOND) {
      for (const auto& b : m.bonds) {
        bond_idx.insert(bond_idx.end(), {b[0], b[1]});
        bond_c.insert(bond_c.end(), m.constants.begin(), m.constants.begin() + 2);
      }
    } else if (m.type == smd::MOL_BEND) {
      for (const auto& b : m.bonds) {
        bend_idx.insert(bend_idx.end(), {b[0], b[1], b[2]});
        bend_c.insert(bend_c.end(), m.constants.begin(), m.constants.begin() + 2);
      }
    } else if (m.type == smd::MOL_BEAD || m.type == smd::MOL_NANOCORE) {
      if (sphere_consts) {
        std::cout << "Error(MD): more than one BEAD or NANOCORE residue is not supported on the GPU step\n";
        return 1;
      }
      for (const auto& b : m.bonds) sphere_idx.push_back(b[0]);
      sphere_consts = &m.constants;
      nanocore = (m.type == smd::MOL_NANOCORE);
      ++n_bead_res;
    } else if (m.type == smd::MOL_BOUNDARY || m.type == smd::MOL_FLOATING_BASE || m.type == smd::MOL_ZTORQUE ||
               m.type == smd::MOL_ZPOWERPOTENTIAL || m.type == smd::MOL_BALL) {
      field_terms(m, S.type, field_idx, field_c);
    } else if (m.type != smd::MOL_SOLID) {
      std::cout << "Error(MD): molecule type " << m.type
                << " is not supported on the GPU step (supported: CHAIN, BOND, BEND, BEAD, NANOCORE, "
                   "BOUNDARY, FLOATING_BASE, ZTORQUE, ZPOWERPOTENTIAL, BALL)\n";
      return 1;
    }
  }
  double gamma = S.gamma;
  bool perTypeGamma = false;
  if (!(S.gamma > 0)) {
    if (!S.present[smd::CMD_GAMMATYPE]) {
      std::cout << "Error(main): No gamma available!\n";
      return 0;
    }
    gamma = S.gammaType[0];  // the reference applies entry 0 to every bead
    perTypeGamma = true;
  }
  const int N = S.nParticles;
  const int endInt = int(S.finalTime / S.deltaT + 0.0000001);
  const int startInt = int(S.initialTime / S.deltaT + 0.0000001);
  const int storeint = int(S.storeInterval / S.deltaT + 0.0000001);
  const int measureint = int(S.measureInterval / S.deltaT + 0.0000001);
  int tempStepInt = 0;
  double tempStep = 0;
  if (S.tempStepInterval > 0) {
    tempStep = S.tempStepInterval * (S.finalTemp - S.initialTemp) / (S.finalTime - S.initialTime);
    tempStepInt = (endInt - startInt) / int((S.finalTime - S.initialTime) / (S.tempStepInterval));
  }
  if (storeint <= 0 || measureint <= 0) {
    std::cout << "Error(MD): storeInterval and measureInterval must be at least deltaT\n";
    return 1;
  }

  smd_system_desc d{};
  d.n = N;
  d.n_types = S.nTypes;
  d.pos = S.pos.data();
  d.vel = S.vel.data();
  d.type = S.type.data();
  for (int k = 0; k < 3; ++k) d.box[k] = S.size[k];
  d.cutoff = S.cutoff;
  d.fconst = S.twoBodyFconst.data();
  d.uconst = S.twoBodyUconst.data();
  d.n_chain_blocks = (int)blocks.size() / 3;
  d.chain_blocks = blocks.data();
  d.chain_consts = consts.data();
  d.n_spheres = (int)sphere_idx.size();
  d.sphere_index = sphere_idx.data();
  d.sphere_consts = sphere_consts ? sphere_consts->data() : nullptr;
  d.sphere_nanocore = nanocore ? 1 : 0;
  d.n_bonds = (int)bond_idx.size() / 2;
  d.bonds = bond_idx.data();
  d.bond_consts = bond_c.data();
  d.n_bends = (int)bend_idx.size() / 3;
  d.bends = bend_idx.data();
  d.bend_consts = bend_c.data();
  d.n_fields = (int)field_idx.size() / 3;
  d.fields = field_idx.data();
  d.field_consts = field_c.data();
  d.dt = S.deltaT;
  d.gamma = gamma;
  d.temperature = S.initialTemp;
  d.seed = (uint32_t)S.seed;
  d.tension = S.tension;
  d.delta_lxy = S.deltaLXY;
  d.resize_rate = 8;
  d.first_step = startInt;
  smd_system* h = nullptr;
  if (smd_create(&d, precision, &h)) return die("smd_create");

  smd::Observables obs(name);
  const std::string frames = "frames_" + name + ".xyz";
  std::vector<double> pos(3 * (size_t)N), vel(3 * (size_t)N);
  double box[3];

  // start-up (MD.cpp:186-308)
  smd_energy e0;
  const bool t0 = (S.initialTime == 0);
  if (smd_prepare(h, t0 ? 0 : 1, t0 ? &e0 : nullptr)) return die("smd_prepare");
  if (t0) {
    obs.compute(S, S.initialTime, S.pos.data(), S.vel.data(), S.pos.data(), e0.pair + e0.bonded + e0.sphere,
                e0.sphere, n_bead_res);
    smd::xyz_append_frame(frames, N, S.type.data(), S.pos.data(), err);
  }
  std::cerr << "starting main loop: \n";
  time_t current = time(NULL);

  auto is_store = [&](long long i) { return i % storeint == 0 && i != startInt; };
  auto is_measure = [&](long long i) { return i % measureint == 0 && i != startInt; };
  auto is_temp = [&](long long i) {
    return S.tempStepInterval > 0 && tempStepInt != 0 && i % tempStepInt == 0 && i < endInt;
  };
  long long it = startInt;
  while (it <= endInt) {
    S.initialTime = (double)it * S.deltaT;
    if (is_temp(it)) {
      S.initialTemp = S.initialTemp + tempStep;
      if (smd_set_temperature(h, -1, S.initialTemp, perTypeGamma ? 0 : 1)) return die("smd_set_temperature");
    }
    if (is_store(it)) {
      if (smd_get_state(h, pos.data(), nullptr) || smd_get_state(h, nullptr, vel.data()) ||
          smd_get_box(h, 0, box))
        return die("smd_get_state");
      for (int k = 0; k < 3; ++k) S.size[k] = box[k];
      S.pos = pos;
      S.vel = vel;
      if (smd::mpd_write_file(name + ".mpd", S, err)) std::cout << err << "\n";
      smd::xyz_append_frame(frames, N, S.type.data(), pos.data(), err);
    }
    // next iteration that needs the host before its force pass
    long long next = it + 1;
    while (next <= endInt && !is_store(next) && !is_temp(next)) ++next;
    long long m = it;
    while (m < next && !is_measure(m)) ++m;
    if (m < next && m <= endInt) {
      if (smd_advance(h, (int)(m - it + 1), SMD_STOP_AT_MEASURE)) return die("smd_advance");
      S.initialTime = (double)m * S.deltaT;
      const time_t last = current;
      current = time(NULL);
      std::cerr << S.initialTime << '\t' << current - last << std::endl;
      smd_energy e;
      if (smd_get_state(h, pos.data(), vel.data()) || smd_get_box(h, 0, box) || smd_compute_energy(h, &e))
        return die("measure");
      for (int k = 0; k < 3; ++k) S.size[k] = box[k];
      obs.compute(S, S.initialTime, pos.data(), vel.data(), pos.data(), e.pair + e.bonded + e.sphere, e.sphere,
                  n_bead_res);
      current = time(NULL);
      if (smd_advance(h, 0, 0)) return die("smd_advance");
      it = m + 1;
    } else {
      const long long stop = std::min<long long>(next, (long long)endInt + 1);
      if (smd_advance(h, (int)(stop - it), 0)) return die("smd_advance");
      it = stop;
    }
  }
  smd_mc_stats st{};
  smd_mc_stats_get(h, 0, &st);
  if (S.deltaLXY != 0) {
    const double interval = S.deltaLXY / 101.0;
    const int nIntervals = static_cast<int>(2.0 * S.deltaLXY / interval) + 1;
    std::vector<double> acc(nIntervals, 0), rej(nIntervals, 0);
    const long n = st.trials;
    std::vector<double> f(n > 0 ? n : 1);
    std::vector<int> a(n > 0 ? n : 1);
    const long got = smd_mc_log(h, 0, 0, n, f.data(), a.data());
    for (long t = 0; t < got; ++t) {
      std::vector<double>& hist = a[t] ? acc : rej;
      hist[(size_t)((f[t] + S.deltaLXY) / interval)] += 0.5;
      hist[(size_t)((f[t] + S.deltaLXY) / interval)] += 0.5;
    }
    std::string out;
    for (int i = 0; i < nIntervals; ++i)
      out += smd::fmt_default((static_cast<double>(i) * interval) - S.deltaLXY) + '\t' + smd::fmt_default(acc[i]) +
             '\t' + smd::fmt_default(rej[i]) + '\n';
    FILE* fp = std::fopen(("resizeHist_" + name + ".dat").c_str(), "w");
    if (fp) {
      std::fwrite(out.data(), 1, out.size(), fp);
      std::fclose(fp);
    }
  }
  std::cerr << "Resize acceptance ratio: " << (double)st.accepted / (double)st.trials << std::endl;
  obs.finish();
  smd_destroy(h);
  return 0;
}
