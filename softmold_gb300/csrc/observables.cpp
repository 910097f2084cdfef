#include "observables.h"

#include <cmath>
#include <fstream>
#include <sstream>

namespace smd {

void Observables::append(const std::string& prefix, const std::string& line) {
  std::ofstream f(prefix + name_ + ".dat", std::ios::app | std::ios::out);
  f << line;
}

void msd_groups(const MpdSystem& sys, std::vector<int>& offsets, std::vector<int>& beads) {
  offsets.assign(1, 0);
  beads.clear();
  for (const Molecule& m : sys.mol) {
    if (m.type == MOL_BOND) {
      for (const auto& b : m.bonds) beads.insert(beads.end(), {b[0], b[1]});
    } else if (m.type == MOL_BEND) {
      for (const auto& b : m.bonds) beads.insert(beads.end(), {b[0], b[1], b[2]});
    } else if (m.type == MOL_CHAIN) {
      for (const auto& b : m.bonds)
        for (int j = b[0]; j < b[0] + b[2] * b[1]; ++j) beads.push_back(j);
    } else if (m.type == MOL_BEAD || m.type == MOL_NANOCORE) {
      for (const auto& b : m.bonds) beads.push_back(b[0]);
    }
    offsets.push_back((int)beads.size());
  }
}

int Observables::compute(const MpdSystem& sys, double time, const double* p, const double* v,
                         const double* ap, double pot, double bead_pot, int n_bead_res) {
  Measurement m;
  if (int rc = aggregate(sys, p, v, ap, m)) return rc;
  write(sys, time, pot, bead_pot, n_bead_res, m);
  return 0;
}

int Observables::aggregate(const MpdSystem& sys, const double* p, const double* v, const double* ap,
                            Measurement& out) {
  const int n = sys.nParticles;
  const double* s = sys.size;
  // BOND lengths and BEND angles (dataExtraction.h:860-940); CHAIN residues
  // contribute to neither.
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
      out.lbond += priv;
      out.n_bond += (int)m.bonds.size();
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
        out.l_bend0 += ra;
        out.l_bend1 += rb;
        out.cos_bend += (da[0] * db[0] + da[1] * db[1] + da[2] * db[2]) / (ra * rb);
      }
      out.n_bend += (int)m.bonds.size();
    }
  }
  // Kinetic<T>::compute (include/algorithms/dataCollection.h:666-674)
  out.kinetic = 0;
  for (int i = 0; i < n; ++i)
    out.kinetic += ((v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) / 2.0);
  // bounding box (dataExtraction.h:1456-1488)
  for (int d = 0; d < 3; ++d) {
    out.lo[d] = s[d];
    out.hi[d] = 0;
  }
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      if (p[3 * i + d] < out.lo[d]) out.lo[d] = p[3 * i + d];
      if (p[3 * i + d] > out.hi[d]) out.hi[d] = p[3 * i + d];
    }
  if (ap) {
    // per-bead kinetic-energy histogram (dataExtraction.h:1509-1519)
    for (int i = 0; i < n; ++i) {
      const double q = 0.5 * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) /
                       0.0001;
      if (!(q < (double)kMaxKeBins)) return 1;  // converted to an int only in range
    }
    for (int i = 0; i < n; ++i) {
      const int part = (int)(0.5 * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] +
                                    v[3 * i + 2] * v[3 * i + 2]) /
                             0.0001);
      while ((int)ke_hist_.size() <= part) ke_hist_.push_back(0);
      ke_hist_[part]++;
    }
  }
  out.msd = ap && !msd_start_.empty();
  if (out.msd) {
    // mean square displacement per residue (dataExtraction.h:1524-1650), in
    // the reference's order within each molecule
    if (msd_off_.empty()) msd_groups(sys, msd_off_, msd_beads_);
    out.msd_sum.assign(msd_off_.size() - 1, 0.0);
    for (size_t g = 0; g + 1 < msd_off_.size(); ++g) {
      double msd = 0;
      for (int k = msd_off_[g]; k < msd_off_[g + 1]; ++k) {
        const int j = msd_beads_[k];
        const double dx = ap[3 * j] - msd_start_[3 * j], dy = ap[3 * j + 1] - msd_start_[3 * j + 1],
                     dz = ap[3 * j + 2] - msd_start_[3 * j + 2];
        msd += dx * dx + dy * dy + dz * dz;
      }
      out.msd_sum[g] = msd;
    }
  }
  return 0;
}

void Observables::write(const MpdSystem& sys, double time, double pot, double bead_pot, int n_bead_res,
                        const Measurement& m) {
  const double* s = sys.size;
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
    o << time << '\t' << (m.lbond / (double)m.n_bond) << '\n';
    append("lBond_", o.str());
  }
  double cosBend = m.cos_bend, lBend0 = m.l_bend0, lBend1 = m.l_bend1;
  if (m.n_bend > 1) {
    cosBend /= (double)m.n_bend;
    lBend0 /= (double)m.n_bend;
    lBend1 /= (double)m.n_bend;
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
    std::ostringstream o;
    o << time << '\t' << m.kinetic << '\n';
    append("kinetic_", o.str());
  }
  {
    std::ostringstream o;
    o << time << '\t' << m.hi[0] - m.lo[0] << '\t' << m.hi[1] - m.lo[1] << '\t' << m.hi[2] - m.lo[2] << '\n';
    append("flicker_", o.str());
  }
  if (m.msd) {
    std::vector<int> off, beads;
    msd_groups(sys, off, beads);
    std::ostringstream o;
    o << time;
    for (size_t g = 0; g + 1 < off.size() && g < m.msd_sum.size(); ++g) {
      const int np = off[g + 1] - off[g];
      if (np != 0) o << '\t' << (m.msd_sum[g] / (double)np);
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
