// ORACLE — test infrastructure only (see smd_oracle.h).
//
// Restatement of the reference `MD <name>` driver (MD.cpp:72-755) on top of the
// restated kernels in smd_oracle.cpp.  Supported residues: CHAIN and BEAD, the
// two on the hot path; any other residue type is rejected with a message.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <iostream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../softmold_gb300/csrc/mpd_io.h"
#include "../softmold_gb300/csrc/observables.h"
#include "smd_oracle.h"

namespace {

using smd::MpdSystem;

struct OracleMD {
  MpdSystem sys;
  std::string name;
  int threads = 1;
  int N = 0;
  std::vector<double> acc, absPos;
  std::vector<orc_mt> thermoRng;  // one generator per thread: MTRand(seed+t) (langevin.h:125-130)
  orc_mt baroRng;                 // MTRand randNum(seed) (MD.cpp:149)
  double cachedTypeSigma = -1;

  double* pos() { return sys.pos.data(); }
  double* vel() { return sys.vel.data(); }

  // Verlet<T>::first (include/algorithms/verlet.h:288-355)
  void first() {
    const double dt = sys.deltaT, h = dt * 0.5;
    double* p = pos();
    double* v = vel();
#pragma omp parallel for num_threads(threads)
    for (int i = 0; i < N; ++i)
      if (sys.type[i] != 0)
        for (int d = 0; d < 3; ++d) v[3 * i + d] += (acc[3 * i + d] * h);
#pragma omp parallel for num_threads(threads)
    for (int i = 0; i < N; ++i)
      if (sys.type[i] != 0)
        for (int d = 0; d < 3; ++d) p[3 * i + d] += v[3 * i + d] * dt;
#pragma omp parallel for num_threads(threads)
    for (int i = 0; i < N; ++i)
      if (sys.type[i] != 0)
        for (int d = 0; d < 3; ++d) absPos[3 * i + d] += v[3 * i + d] * dt;
    for (int d = 0; d < 3; ++d) {
      const double L = sys.size[d];
#pragma omp parallel for num_threads(threads)
      for (int i = 0; i < N; ++i) {
        if (p[3 * i + d] > L) p[3 * i + d] -= L;
        if (p[3 * i + d] < 0) p[3 * i + d] += L;
      }
    }
  }
  // Verlet<T>::second (include/algorithms/verlet.h:463-491)
  void second() {
    const double h = sys.deltaT * 0.5;
    double* v = vel();
#pragma omp parallel for num_threads(threads)
    for (int i = 0; i < N; ++i)
      if (sys.type[i] != 0)
        for (int d = 0; d < 3; ++d) v[3 * i + d] += (acc[3 * i + d] * h);
  }
  // Langevin<T>::compute (include/algorithms/langevin.h:232-331); a static
  // OpenMP schedule gives thread t one contiguous block of beads.
  void thermostat(double T) {
    // With per-type gammas the reference reads entry 0 for every bead and
    // computes that sigma once, at the first call (langevin.h:235-246,257).
    const bool perType = !(sys.gamma > 0);
    const double g = perType ? sys.gammaType[0] : sys.gamma;
    if (perType && cachedTypeSigma < 0) cachedTypeSigma = std::sqrt((6.0 * T * g) / sys.deltaT);
    const double sigma = perType ? cachedTypeSigma : std::sqrt((6.0 * T * g) / sys.deltaT);
    const double* v = sys.vel.data();
#pragma omp parallel num_threads(threads)
    {
#ifdef _OPENMP
      const int t = omp_get_thread_num(), nt = omp_get_num_threads();
#else
      const int t = 0, nt = 1;
#endif
      const int q = N / nt, r = N % nt;
      const int lo = t * q + (t < r ? t : r), hi = lo + q + (t < r ? 1 : 0);
      orc_mt* g1 = &thermoRng[t];
      for (int i = lo; i < hi; ++i)
        for (int d = 0; d < 3; ++d) {
          const double psi = 2.0 * orc_mt_rand53(g1) - 1.0;
          acc[3 * i + d] += (-g * v[3 * i + d] + sigma * psi);
        }
    }
  }
  bool bonded_forces(std::string& err) {
    for (size_t k = 0; k < sys.mol.size(); ++k) {
      const smd::Molecule& m = sys.mol[k];
      if (m.type == smd::MOL_CHAIN) {
        for (const auto& b : m.bonds)
          orc_chain_force(pos(), sys.size, b[0], b[1], b[2], m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_BEAD) {
        std::vector<int> idx;
        for (const auto& b : m.bonds) idx.push_back(b[0]);
        orc_bead_force(N, pos(), sys.type.data(), sys.size, sys.nTypes, (int)idx.size(), idx.data(),
                       m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_BOND || m.type == smd::MOL_BEND) {
        const std::vector<int> L = flat_list(m);
        if (m.type == smd::MOL_BOND)
          orc_bond_force(pos(), sys.size, (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
        else
          orc_bend_force(pos(), sys.size, (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_BOUNDARY) {
        const std::vector<int> L = column(m, 1);
        orc_boundary_force(pos(), sys.size, (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_FLOATING_BASE) {
        const std::vector<int> L = column(m, 1);
        orc_floating_base_force(pos(), sys.type.data(), (int)m.bonds.size(), L.data(), m.constants.data(),
                                acc.data());
      } else if (m.type == smd::MOL_ZTORQUE) {
        const std::vector<int> L = column(m, 3);
        orc_ztorque_force(pos(), sys.size, (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_ZPOWERPOTENTIAL) {
        const std::vector<int> L = column(m, 2);
        orc_zpower_force(pos(), (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_BALL) {
        const std::vector<int> L = column(m, 2);
        orc_ball_force(pos(), sys.size, (int)m.bonds.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_NANOCORE) {
        const std::vector<int> L = column(m, 1);
        orc_nanocore_force(N, pos(), sys.size, (int)L.size(), L.data(), m.constants.data(), acc.data());
      } else if (m.type == smd::MOL_SOLID) {
      } else {
        err = "molecule type " + std::to_string(m.type) + " is not supported";
        return false;
      }
    }
    return true;
  }
  void bead_mass_divide() {
    for (const smd::Molecule& m : sys.mol) {
      if (m.type == smd::MOL_NANOCORE) {  // each core by its own 4 pi R^2 (MD.cpp:291-303)
        for (int j = (int)m.bonds.size() - 1; j >= 0; --j) {
          const double R = m.constants[22 * j + smd::kBeadRadius];
          const double mass = (4.0) * M_PI * R * R;
          for (int d = 0; d < 3; ++d) acc[3 * m.bonds[j][0] + d] /= mass;
        }
        continue;
      }
      if (m.type != smd::MOL_BEAD) continue;
      const double R = m.constants[smd::kBeadRadius];
      const double mass = (4.0) * M_PI * R * R;
      for (int j = (int)m.bonds.size() - 1; j >= 0; --j)
        for (int d = 0; d < 3; ++d) acc[3 * m.bonds[j][0] + d] /= mass;
    }
  }
  void pair_forces() {
    orc_pair_force(N, pos(), sys.type.data(), sys.size, sys.cutoff, sys.nTypes,
                   sys.twoBodyFconst.data(), acc.data());
  }
  // The first w indices of every entry of a residue, flattened.
  static std::vector<int> column(const smd::Molecule& m, int w) {
    std::vector<int> L;
    for (const auto& b : m.bonds)
      for (int q = 0; q < w; ++q) L.push_back(b[q]);
    return L;
  }
  // Index list of a BOND (pairs) or BEND (triplets) residue.
  static std::vector<int> flat_list(const smd::Molecule& m) {
    const int w = (m.type == smd::MOL_BOND) ? 2 : 3;
    std::vector<int> L;
    for (const auto& b : m.bonds)
      for (int q = 0; q < w; ++q) L.push_back(b[q]);
    return L;
  }
  double total_potential(double* beadPot, int* nBeadRes) {
    double pot = orc_pair_potential(N, pos(), sys.type.data(), sys.size, sys.cutoff, sys.nTypes,
                                    sys.twoBodyUconst.data());
    *beadPot = 0;
    *nBeadRes = 0;
    for (const smd::Molecule& m : sys.mol) {
      if (m.type == smd::MOL_CHAIN) {
        for (const auto& b : m.bonds)
          pot += orc_chain_potential(pos(), sys.size, b[0], b[1], b[2], m.constants.data());
      } else if (m.type == smd::MOL_BOND) {
        pot += orc_bond_potential(pos(), sys.size, (int)m.bonds.size(), flat_list(m).data(), m.constants.data());
      } else if (m.type == smd::MOL_BEND) {
        pot += orc_bend_potential(pos(), sys.size, (int)m.bonds.size(), flat_list(m).data(), m.constants.data());
      } else if (m.type == smd::MOL_BEAD) {
        std::vector<int> idx;
        for (const auto& b : m.bonds) idx.push_back(b[0]);
        const double bp = orc_bead_potential(N, pos(), sys.type.data(), sys.size, sys.nTypes,
                                             (int)idx.size(), idx.data(), m.constants.data());
        *beadPot += bp;
        pot += bp;
        ++*nBeadRes;
      } else if (m.type == smd::MOL_BOUNDARY) {
        pot += orc_boundary_potential(pos(), sys.size, (int)m.bonds.size(), column(m, 1).data(), m.constants.data());
      } else if (m.type == smd::MOL_FLOATING_BASE) {
        pot += orc_floating_base_potential(pos(), sys.type.data(), (int)m.bonds.size(), column(m, 1).data(),
                                           m.constants.data());
      } else if (m.type == smd::MOL_ZTORQUE) {
        pot += orc_ztorque_potential(pos(), sys.size, (int)m.bonds.size(), column(m, 3).data(), m.constants.data());
      } else if (m.type == smd::MOL_ZPOWERPOTENTIAL) {
        pot += orc_zpower_potential(pos(), (int)m.bonds.size(), column(m, 2).data(), m.constants.data());
      } else if (m.type == smd::MOL_BALL) {
        pot += orc_ball_potential(pos(), sys.size, (int)m.bonds.size(), column(m, 2).data(), m.constants.data());
      } else if (m.type == smd::MOL_NANOCORE) {
        const std::vector<int> L = column(m, 1);
        const double bp = orc_nanocore_potential(N, pos(), sys.size, (int)L.size(), L.data(), m.constants.data());
        *beadPot += bp;
        pot += bp;
        ++*nBeadRes;
      }
    }
    return pot;
  }
  double total_dpotential(const double s[3]) {
    double dp = orc_pair_dpotential(N, pos(), sys.type.data(), sys.size, sys.cutoff, sys.nTypes,
                                    sys.twoBodyUconst.data(), s);
    for (const smd::Molecule& m : sys.mol) {
      if (m.type == smd::MOL_CHAIN) {
        for (const auto& b : m.bonds)
          dp += orc_chain_dpotential(pos(), sys.size, b[0], b[1], b[2], m.constants.data(), s);
      } else if (m.type == smd::MOL_BOND) {
        dp += orc_bond_dpotential(pos(), sys.size, (int)m.bonds.size(), flat_list(m).data(), m.constants.data(), s);
      } else if (m.type == smd::MOL_BEND) {
        dp += orc_bend_dpotential(pos(), sys.size, (int)m.bonds.size(), flat_list(m).data(), m.constants.data(), s);
      } else if (m.type == smd::MOL_BEAD) {
        std::vector<int> idx;
        for (const auto& b : m.bonds) idx.push_back(b[0]);
        dp += orc_bead_dpotential(N, pos(), sys.type.data(), sys.size, sys.nTypes, (int)idx.size(),
                                  idx.data(), m.constants.data(), s);
      }
    }
    return dp;
  }
};

// A bead's kinetic energy beyond the measurement histogram ends the run.
int blown_up() {
  std::cout << "Error(MD): a bead's kinetic energy exceeds the measurement histogram ("
            << smd::kMaxKeBins / 10000 << " per bead)\n";
  return 1;
}

int run(const char* name, int threads, int timeSteps, double* elapsed) {
  OracleMD md;
  md.name = name;
  md.threads = threads < 1 ? 1 : threads;
  std::string err;
  if (smd::mpd_read_file(std::string(name) + ".mpd", md.sys, err)) {
    std::cout << err << "\n";
    return 1;
  }
  MpdSystem& S = md.sys;
  md.N = S.nParticles;
  const int N = md.N;
  md.acc.assign(3 * (size_t)N, 0.0);
  md.absPos = S.pos;
  if (!(S.gamma > 0) && S.gammaType.empty()) {
    std::cout << "Error(main): No gamma available!\n";
    return 0;
  }
  md.thermoRng.resize(md.threads);
  for (int t = 0; t < md.threads; ++t) orc_mt_seed(&md.thermoRng[t], (uint32_t)(S.seed + t));
  orc_mt_seed(&md.baroRng, (uint32_t)S.seed);
  const bool timing = timeSteps > 0;
  smd::Observables obs(name);

  std::vector<double> resizeHist, rejectHist;
  double histInterval = 0.00001;
  if (S.deltaLXY != 0) {
    histInterval = S.deltaLXY / 101.0;
    const int nIntervals = static_cast<int>(2.0 * S.deltaLXY / histInterval) + 1;
    resizeHist.assign(nIntervals, 0);
    rejectHist.assign(nIntervals, 0);
  }
  double trial = 0, accepted = 0;

  // initial forces (MD.cpp:186-262)
  md.pair_forces();
  md.thermostat(S.initialTemp);
  if (!md.bonded_forces(err)) {
    std::cout << "Error: " << err << "\n";
    return 2;
  }
  const std::string frames = std::string("frames_") + name + ".xyz";
  if (!timing) {
    if (S.initialTime == 0) {
      double bp;
      int nb;
      const double pot = md.total_potential(&bp, &nb);
      if (obs.compute(S, S.initialTime, md.pos(), md.vel(), md.absPos.data(), pot, bp, nb)) return blown_up();
      smd::xyz_append_frame(frames, N, S.type.data(), md.pos(), err);
    } else {
      md.bead_mass_divide();
      md.second();
    }
  } else if (S.initialTime != 0) {
    md.bead_mass_divide();
    md.second();
  }
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
  const int lastStep = timing ? startInt + timeSteps - 1 : endInt;
  if (!timing) std::cerr << "starting main loop: \n";
  time_t current = time(NULL);
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = startInt; i <= lastStep; ++i) {
    S.initialTime = (double)i * S.deltaT;
    // BEAD mass before first() (MD.cpp:340-355)
    for (const smd::Molecule& m : S.mol) {
      if (m.type != smd::MOL_BEAD) continue;
      const double R = m.constants[smd::kBeadRadius];
      const double mass = (4.0) * M_PI * R * R;
      for (int j = (int)m.bonds.size() - 1; j >= 0; --j)
        for (int d = 0; d < 3; ++d) md.acc[3 * m.bonds[j][0] + d] /= mass;
    }
    md.first();
    std::fill(md.acc.begin(), md.acc.end(), 0.0);
    if (S.tempStepInterval > 0)
      if (i % tempStepInt == 0 && tempStepInt != 0 && i < endInt) S.initialTemp = S.initialTemp + tempStep;
    if (!timing && i % storeint == 0 && i != startInt) {
      smd::mpd_write_file(std::string(name) + ".mpd", S, err);
      smd::xyz_append_frame(frames, N, S.type.data(), md.pos(), err);
    }
    md.thermostat(S.initialTemp);
    md.pair_forces();
    if (!md.bonded_forces(err)) {
      std::cout << "Error: " << err << "\n";
      return 2;
    }
    md.bead_mass_divide();
    md.second();
    if (!timing && i % measureint == 0 && i != startInt) {
      const time_t last = current;
      current = time(NULL);
      std::cerr << S.initialTime << '\t' << current - last << std::endl;
      if (S.initialTime > 100.0) obs.start_diffusion(S, md.absPos.data());
      double bp;
      int nb;
      const double pot = md.total_potential(&bp, &nb);
      if (obs.compute(S, S.initialTime, md.pos(), md.vel(), md.absPos.data(), pot, bp, nb)) return blown_up();
      current = time(NULL);
    }
    // MC constant-tension box move (MD.cpp:589-721)
    if (i % 8 == 0 && i != 0 && S.deltaLXY != 0) {
      const double oldSize[3] = {S.size[0], S.size[1], S.size[2]};
      double size[3] = {S.size[0], S.size[1], S.size[2]};
      double fl[3];
      fl[0] = S.deltaLXY * (2.0 * orc_mt_rand53(&md.baroRng) - 1.0);
      fl[1] = fl[0];
      fl[2] = (size[0] * size[1]) / ((size[0] + fl[0]) * (size[1] + fl[1]));
      size[0] += fl[0];
      size[1] += fl[1];
      size[2] *= fl[2];
      const double a[3] = {size[0] / oldSize[0], size[1] / oldSize[1], size[2] / oldSize[2]};
      double dPot = md.total_dpotential(a);
      if (S.tension != 0) dPot += S.tension * ((size[0] * size[1]) - (oldSize[0] * oldSize[1]));
      double D = (dPot) / S.initialTemp;
      D = std::exp(D);
      const double r = orc_mt_rand53(&md.baroRng);
      if (D >= r || -dPot <= 0) {
        double* p = md.pos();
        for (int k = 0; k < N; ++k) {
          p[3 * k] *= a[0];
          p[3 * k + 1] *= a[1];
          p[3 * k + 2] *= a[2];
        }
        if (!resizeHist.empty()) {
          resizeHist[(size_t)((fl[0] + S.deltaLXY) / histInterval)] += 0.5;
          resizeHist[(size_t)((fl[1] + S.deltaLXY) / histInterval)] += 0.5;
        }
        S.size[0] = size[0];
        S.size[1] = size[1];
        S.size[2] = size[2];
        accepted++;
      } else if (!rejectHist.empty()) {
        rejectHist[(size_t)((fl[0] + S.deltaLXY) / histInterval)] += 0.5;
        rejectHist[(size_t)((fl[1] + S.deltaLXY) / histInterval)] += 0.5;
      }
      trial++;
    }
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (elapsed) *elapsed = std::chrono::duration<double>(t1 - t0).count();
  if (timing) return 0;
  if (S.deltaLXY != 0) {
    std::string out;
    for (size_t i = 0; i < resizeHist.size(); ++i)
      out += smd::fmt_default((static_cast<double>(i) * histInterval) - S.deltaLXY) + '\t' +
             smd::fmt_default(resizeHist[i]) + '\t' + smd::fmt_default(rejectHist[i]) + '\n';
    FILE* f = std::fopen((std::string("resizeHist_") + name + ".dat").c_str(), "w");
    if (f) {
      std::fwrite(out.data(), 1, out.size(), f);
      std::fclose(f);
    }
  }
  std::cerr << "Resize acceptance ratio: " << accepted / trial << std::endl;
  obs.finish();
  return 0;
}

}  // namespace

extern "C" int orc_md_run(const char* name, int threads) { return run(name, threads, 0, nullptr); }

extern "C" double orc_md_time(const char* name, int threads, int steps) {
  double el = -1;
  if (run(name, threads, steps < 1 ? 1 : steps, &el) != 0) return -1;
  return el;
}
