// The `MD <name>` drop-in driver on top of the C ABI.
//
// Same invocation, inputs, outputs and loop cadence as the reference driver
// (MD.cpp:72-755): read <name>.mpd, initial forces, the t=0 measurement or the
// restart half-kick, then the loop with .mpd/.xyz stores every storeInterval,
// measurements every measureInterval, the temperature ramp, and the MC box
// move every 8 steps; at the end resizeHist_<name>.dat, the acceptance ratio on
// stderr and kEnergyDensity_<name>.dat.  The device advances in chunks between
// those events.  The state is read back only at stores: a measurement reads
// back the device's reductions (smd_measure, smd_compute_energy), and from the
// first measurement after 100 tau on the device tracks each bead's
// displacement for meanSquareDisplacement_<name>.dat (MD.cpp:64, 538-539).
//
// SMD_REFERENCE_NOISE=1 (a test mode, one step per call, slow) drives the
// Langevin term with the noise of a one-thread reference run, 2 u - 1 with u
// from MTRand(seed).rand53() for each bead's x, y, z in turn
// (include/algorithms/langevin.h:284-331), through smd_set_noise_once, so
// that a run can be compared with the reference's output files line by line.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/softmold_gb300.h"
#include "mpd_desc.h"
#include "mpd_io.h"
#include "mt19937.h"
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

// Owns the device system, so that every return releases it (smd_md_main is
// also exported to callers that stay alive after an error).
struct SystemGuard {
  smd_system* h = nullptr;
  ~SystemGuard() {
    if (h) smd_destroy(h);
  }
};

}  // namespace

extern "C" int smd_md_main(const char* name_c, int precision) {
  const std::string name(name_c);
  smd::MpdSystem S;
  std::string err;
  if (smd::mpd_read_file(name + ".mpd", S, err)) {
    std::cout << err << "\n";
    return 1;
  }
  // residues on the device path, expanded as smd_mpd_load expands them
  smd::MpdResidues res;
  if (int rc = smd::mpd_residues(S, res, err)) {
    std::cout << err << "\n";
    return rc == 2 ? 0 : 1;  // the reference exits with status 0 when gamma is missing
  }
  const int n_bead_res = res.n_bead_res;
  const bool perTypeGamma = res.per_type_gamma;
  const int N = S.nParticles;
  // the step counts below are ints
  const double max_steps = 2147483647.0;
  if (!(S.deltaT > 0) || !(std::fabs(S.finalTime) / S.deltaT < max_steps) ||
      !(std::fabs(S.initialTime) / S.deltaT < max_steps) || !(std::fabs(S.storeInterval) / S.deltaT < max_steps) ||
      !(std::fabs(S.measureInterval) / S.deltaT < max_steps)) {
    std::cout << "Error(MD): deltaT must be positive and every time below 2^31 steps\n";
    return 1;
  }
  const int endInt = int(S.finalTime / S.deltaT + 0.0000001);
  const int startInt = int(S.initialTime / S.deltaT + 0.0000001);
  const int storeint = int(S.storeInterval / S.deltaT + 0.0000001);
  const int measureint = int(S.measureInterval / S.deltaT + 0.0000001);
  int tempStepInt = 0;
  double tempStep = 0;
  if (S.tempStepInterval > 0) {
    tempStep = S.tempStepInterval * (S.finalTemp - S.initialTemp) / (S.finalTime - S.initialTime);
    // no ramp step when the interval exceeds the run (the count rounds to 0);
    // a count of 2^31 or more gives a ramp every 0 steps, i.e. none, too
    const double ramps = (S.finalTime - S.initialTime) / (S.tempStepInterval);
    const int n_ramp = std::fabs(ramps) < max_steps ? int(ramps) : 0;
    tempStepInt = n_ramp > 0 ? (endInt - startInt) / n_ramp : 0;
  }
  if (storeint <= 0 || measureint <= 0) {
    std::cout << "Error(MD): storeInterval and measureInterval must be at least deltaT\n";
    return 1;
  }

  smd_system_desc d;
  smd::mpd_descriptor(S, res, d);
  SystemGuard guard;
  if (smd_create(&d, precision, &guard.h)) return die("smd_create");
  smd_system* const h = guard.h;

  smd::Observables obs(name);
  const std::string frames = "frames_" + name + ".xyz";
  std::vector<double> pos(3 * (size_t)N), vel(3 * (size_t)N);
  double box[3];
  std::vector<int> msd_off, msd_beads;
  smd::msd_groups(S, msd_off, msd_beads);
  if (smd_set_msd_groups(h, (int)S.mol.size(), msd_off.data(), msd_beads.data())) return die("smd_set_msd_groups");
  std::vector<double> msd_sum(S.mol.size() + 1, 0.0);
  bool diffusion = false;

  const char* rn = std::getenv("SMD_REFERENCE_NOISE");
  const bool ref_noise = rn && rn[0] == '1';
  smd::Mt19937 lang((uint32_t)S.seed);
  std::vector<double> psi(ref_noise ? 3 * (size_t)N : 0);
  auto feed_noise = [&]() -> int {  // one step's draws, bead by bead, x y z
    if (!ref_noise) return 0;
    for (double& q : psi) q = 2.0 * lang.rand53() - 1.0;
    return smd_set_noise_once(h, psi.data());
  };

  // start-up (MD.cpp:186-308)
  smd_energy e0;
  const bool t0 = (S.initialTime == 0);
  if (feed_noise()) return die("smd_set_noise_once");
  if (smd_prepare(h, t0 ? 0 : 1, t0 ? &e0 : nullptr)) return die("smd_prepare");
  if (t0) {
    if (obs.compute(S, S.initialTime, S.pos.data(), S.vel.data(), S.pos.data(), e0.pair + e0.bonded + e0.sphere,
                    e0.sphere, n_bead_res)) {
      std::cout << "Error(MD): a bead's kinetic energy exceeds the measurement histogram (" << smd::kMaxKeBins / 10000
                << " per bead)\n";
      return 1;
    }
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
    while (!ref_noise && next <= endInt && !is_store(next) && !is_temp(next)) ++next;
    if (feed_noise()) return die("smd_set_noise_once");
    long long m = it;
    while (m < next && !is_measure(m)) ++m;
    if (m < next && m <= endInt) {
      if (smd_advance(h, (int)(m - it + 1), SMD_STOP_AT_MEASURE)) return die("smd_advance");
      S.initialTime = (double)m * S.deltaT;
      const time_t last = current;
      current = time(NULL);
      std::cerr << S.initialTime << '\t' << current - last << std::endl;
      // dataCollection.startDiffusion() before compute() (MD.cpp:538-539)
      if (S.initialTime > 100.0 && !diffusion) {
        if (smd_start_diffusion(h)) return die("smd_start_diffusion");
        diffusion = true;
      }
      smd_energy e;
      smd_measurement dm;
      if (smd_get_box(h, 0, box) || smd_compute_energy(h, &e) || smd_measure(h, &dm, msd_sum.data()))
        return die("measure");
      for (int k = 0; k < 3; ++k) S.size[k] = box[k];
      smd::Measurement mm;
      mm.kinetic = dm.kinetic;
      for (int k = 0; k < 3; ++k) {
        mm.lo[k] = dm.lo[k];
        mm.hi[k] = dm.hi[k];
      }
      mm.lbond = dm.bond_length_sum;
      mm.n_bond = dm.n_bond;
      mm.cos_bend = dm.bend_cos_sum;
      mm.l_bend0 = dm.bend_len0_sum;
      mm.l_bend1 = dm.bend_len1_sum;
      mm.n_bend = dm.n_bend;
      mm.msd = dm.msd != 0;
      if (mm.msd) mm.msd_sum.assign(msd_sum.begin(), msd_sum.begin() + S.mol.size());
      obs.write(S, S.initialTime, e.pair + e.bonded + e.sphere, e.sphere, n_bead_res, mm);
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
      // a trial in [-deltaLXY, deltaLXY) falls in bins 0..nIntervals-1; the
      // clamp keeps one whose bin rounds up to the upper edge in the last bin
      const double q = (f[t] + S.deltaLXY) / interval;
      const size_t bin = q > 0 ? std::min((size_t)q, (size_t)nIntervals - 1) : 0;
      hist[bin] += 0.5;
      hist[bin] += 0.5;
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
  // the measurements' kinetic-energy bins: the t = 0 measurement's (host) and
  // the loop's (device)
  size_t nb = 0;
  if (smd_ke_histogram(h, nullptr, 0, &nb)) return die("smd_ke_histogram");
  std::vector<long> dev_hist(nb);
  if (nb > 0 && smd_ke_histogram(h, dev_hist.data(), nb, &nb)) return die("smd_ke_histogram");
  std::vector<long>& hist = obs.ke_histogram();
  if (hist.size() < nb) hist.resize(nb, 0);
  for (size_t k = 0; k < nb; ++k) hist[k] += dev_hist[k];
  obs.finish();
  return 0;
}
