#include "observables.h"

#include <cmath>
#include <fstream>
#include <sstream>

namespace smd {

void Observables::append(const std::string& prefix, const std::string& line) {
  std::ofstream f(prefix + name_ + ".dat", std::ios::app | std::ios::out);
  f << line;
}

void Observables::compute(const MpdSystem& sys, double time, const double* p, const double* v,
                          const double* ap, double pot, double bead_pot, int n_bead_res) {
  const int n = sys.nParticles;
  const double* s = sys.size;
  // BOND lengths and BEND angles (dataExtraction.h:860-940); CHAIN residues
  // contribute to neither.
  double lBond = 0;
  int nBond = 0;
  double cosBend = 0, lBend0 = 0, lBend1 = 0;
  int nBend = 0;
  auto wrap = [&](double& d, double L) {
    if (d >= L / 2.0) d -= L;
    if (d <= -L / 2.0) d += L;
  };
  for (const Molecule& m : sys.mol) {
    if (m.type == MOL_BOND) {
      double priv = 0;
      for (const auto& b : m.bonds) {
        double dx = p[3 * b[0]] - p[3 * b[1]], dy = p[3 * b[0] + 1] - p[3 * b[1] + 1],
               dz = p[3 * b[0] + 2] - p[3 * b[1] + 2];
        wrap(dx, s[0]);
        wrap(dy, s[1]);
        wrap(dz, s[2]);
        priv += std::sqrt(dx * dx + dy * dy + dz * dz);
      }
      lBond += priv;
      nBond += (int)m.bonds.size();
    } else if (m.type == MOL_BEND) {
      for (const auto& b : m.bonds) {
        double da[3], db[3];
        for (int d = 0; d < 3; ++d) {
          da[d] = p[3 * b[0] + d] - p[3 * b[1] + d];
          db[d] = p[3 * b[1] + d] - p[3 * b[2] + d];
        }
        for (int d = 0; d < 3; ++d) wrap(da[d], s[d]);
        for (int d = 0; d < 3; ++d) wrap(db[d], s[d]);
        const double ra = std::sqrt(da[0] * da[0] + da[1] * da[1] + da[2] * da[2]);
        const double rb = std::sqrt(db[0] * db[0] + db[1] * db[1] + db[2] * db[2]);
        lBend0 += ra;
        lBend1 += rb;
        cosBend += (da[0] * db[0] + da[1] * db[1] + da[2] * db[2]) / (ra * rb);
      }
      nBend += (int)m.bonds.size();
    }
  }
  {
    std::ostringstream o;
    o << time << '\t' << pot << '\n';
    append("potential_", o.str());
  }
  {
    std::ostringstream o;
    o << time << '\t' << s[0] << '\t' << s[1] << '\t' << s[2] << '\n';
    append("size_", o.str());
  }
  {
    std::ostringstream o;
    o << time << '\t' << (lBond / (double)nBond) << '\n';
    append("lBond_", o.str());
  }
  if (nBend > 1) {
    cosBend /= (double)nBend;
    lBend0 /= (double)nBend;
    lBend1 /= (double)nBend;
  }
  {
    std::ostringstream o;
    o << time << '\t' << cosBend << '\t' << lBend0 << '\t' << lBend1 << '\n';
    append("bend_", o.str());
  }
  if (n_bead_res > 0) {
    std::ostringstream o;
    o << time << '\t' << bead_pot << '\n';
    append("beadPotential_", o.str());
  }
  {
    std::ostringstream o;
    o << time << '\t' << sys.initialTemp << '\n';
    append("temp_", o.str());
  }
  {
    // Kinetic<T>::compute (include/algorithms/dataCollection.h:666-674)
    double ke = 0;
    for (int i = 0; i < n; ++i)
      ke += ((v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) / 2.0);
    std::ostringstream o;
    o << time << '\t' << ke << '\n';
    append("kinetic_", o.str());
  }
  {
    // bounding box extents (dataExtraction.h:1456-1488)
    double mn[3] = {s[0], s[1], s[2]}, mx[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        if (p[3 * i + d] < mn[d]) mn[d] = p[3 * i + d];
        if (p[3 * i + d] > mx[d]) mx[d] = p[3 * i + d];
      }
    std::ostringstream o;
    o << time << '\t' << mx[0] - mn[0] << '\t' << mx[1] - mn[1] << '\t' << mx[2] - mn[2] << '\n';
    append("flicker_", o.str());
  }
  if (ap) {
    // per-bead kinetic-energy histogram (dataExtraction.h:1509-1519)
    for (int i = 0; i < n; ++i) {
      const int part = (int)(0.5 * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                                    v[3 * i + 2] * v[3 * i + 2]) /
                             0.0001);
      while ((int)ke_hist_.size() <= part) ke_hist_.push_back(0);
      ke_hist_[part]++;
    }
  }
  if (ap && !msd_start_.empty()) {
    // mean square displacement per residue (dataExtraction.h:1524-1650)
    std::ostringstream o;
    o << time;
    auto sq = [&](int j) {
      const double dx = ap[3 * j] - msd_start_[3 * j], dy = ap[3 * j + 1] - msd_start_[3 * j + 1],
                   dz = ap[3 * j + 2] - msd_start_[3 * j + 2];
      return dx * dx + dy * dy + dz * dz;
    };
    for (const Molecule& m : sys.mol) {
      double msd = 0;
      int np = 0;
      if (m.type == MOL_BOND) {
        for (const auto& b : m.bonds) {
          msd += sq(b[0]);
          msd += sq(b[1]);
        }
        np += (int)m.bonds.size() * 2;
      } else if (m.type == MOL_BEND) {
        for (const auto& b : m.bonds) {
          msd += sq(b[0]);
          msd += sq(b[1]);
          msd += sq(b[2]);
        }
        np += (int)m.bonds.size() * 3;
      } else if (m.type == MOL_CHAIN) {
        for (const auto& b : m.bonds) {
          for (int j = b[0]; j < b[0] + b[2] * b[1]; ++j) msd += sq(j);
          np += b[2] * b[1];
        }
      } else if (m.type == MOL_BEAD || m.type == MOL_NANOCORE) {
        for (const auto& b : m.bonds) msd += sq(b[0]);
        np += (int)m.bonds.size();
      }
      if (np != 0) o << '\t' << (msd / (double)np);
    }
    o << '\n';
    append("meanSquareDisplacement_", o.str());
  }
}

void Observables::start_diffusion(const MpdSystem& sys, const double* ap) {
  if (ap && msd_start_.empty()) msd_start_.assign(ap, ap + 3 * (size_t)sys.nParticles);
}

void Observables::finish() {
  std::ofstream f("kEnergyDensity_" + name_ + ".dat", std::ios::out);
  long sum = 0;
  for (long c : ke_hist_) sum += c;
  for (size_t i = 0; i < ke_hist_.size(); ++i) {
    f << static_cast<float>(i) * 0.0001 << '\t';
    f << static_cast<float>(ke_hist_[i]) / static_cast<float>(sum) << '\n';
  }
}

}  // namespace smd
