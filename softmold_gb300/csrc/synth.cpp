#include "synth.h"

#include <cmath>

#include "mt19937.h"

namespace smd {

namespace {

constexpr double kCutoff = 2.0, kRmin = 1.0;  // generate/include.h:28-29

void add_particle(MpdSystem& s, double x, double y, double z, int type, const double v[3]) {
  // Blob::addParticle wraps into [0,size) when a size is set (include/system.h:3836-3867).
  double p[3] = {x, y, z};
  if (s.size[0] > 0 && s.size[1] > 0 && s.size[2] > 0)
    for (int d = 0; d < 3; ++d) {
      while (p[d] >= s.size[d]) p[d] -= s.size[d];
      while (p[d] < 0) p[d] += s.size[d];
    }
  s.pos.insert(s.pos.end(), p, p + 3);
  s.vel.insert(s.vel.end(), v, v + 3);
  s.type.push_back(type);
  s.nParticles++;
  s.present[CMD_NPARTICLES] = s.present[CMD_POSITIONS] = s.present[CMD_VELOCITIES] = true;
}

void random_velocity(Mt19937& r, double vrms, double v[3]) {
  const double theta = M_PI * r.rand53();
  const double phi = M_PI * 2.0 * r.rand53();
  v[0] = vrms * std::cos(phi) * std::sin(theta);
  v[1] = vrms * std::sin(phi) * std::sin(theta);
  v[2] = vrms * std::cos(theta);
}

void add_molecule(MpdSystem& s, Molecule m) {
  m.nBondAlloc = (int)m.bonds.size();
  s.mol.push_back(std::move(m));
  s.nMolecules++;
  s.present[CMD_NMOLECULES] = s.present[CMD_MOLECULE] = true;
}

MpdSystem base_system(int seed, int nTypes, double finalTime, double store, double measure) {
  MpdSystem s;
  s.gamma = 1.0;
  s.nTypes = nTypes;
  s.seed = seed;
  s.cutoff = kCutoff;
  s.initialTime = 0;
  s.finalTime = finalTime;
  s.deltaT = 0.02;
  s.storeInterval = store;
  s.measureInterval = measure;
  s.initialTemp = 3.0;
  s.finalTemp = 3.0;
  for (int c : {CMD_GAMMA, CMD_NTYPES, CMD_SEED, CMD_PERIODIC, CMD_CUTOFF, CMD_INITIALTIME, CMD_FINALTIME,
                CMD_DELTAT, CMD_STOREINTERVAL, CMD_MEASUREINTERVAL, CMD_INITIALTEMP, CMD_FINALTEMP})
    s.present[c] = true;
  return s;
}

void lipid_tables(MpdSystem& s, std::vector<double>& Umax, std::vector<double>& Umin) {
  s.twoBodyFconst = laradji_revalee_fc(Umax, Umin, kCutoff, kRmin);
  s.twoBodyUconst = laradji_revalee_pc(Umax, Umin, kCutoff, kRmin);
  s.present[CMD_TWOBODYFCONST] = s.present[CMD_TWOBODYUCONST] = true;
}

}  // namespace

std::vector<double> laradji_revalee_fc(const std::vector<double>& Umax, const std::vector<double>& Umin,
                                       double rc, double rm) {
  std::vector<double> out;
  const int nT = (int)std::sqrt((double)Umax.size());
  for (int i = 0; i < nT; ++i)
    for (int j = 0; j < nT; ++j) {
      const int g = i + j * nT;
      out.push_back(rm);
      out.push_back((2.0 * (Umax[g] - Umin[g])) / (rm * rm));
      out.push_back(0);
      out.push_back(rc);
      out.push_back((6.0 * Umin[g]) / ((rc - rm) * (rc - rm)));
      out.push_back((6.0 * Umin[g]) / ((rc - rm) * (rc - rm) * (rc - rm)));
    }
  return out;
}

std::vector<double> laradji_revalee_pc(const std::vector<double>& Umax, const std::vector<double>& Umin,
                                       double rc, double rm) {
  std::vector<double> out;
  const int nT = (int)std::sqrt((double)Umax.size());
  for (int i = 0; i < nT; ++i)
    for (int j = 0; j < nT; ++j) {
      const int g = i + j * nT;
      out.push_back(rm);
      out.push_back((Umax[g] - Umin[g]) / (rm * rm));
      out.push_back(Umin[g]);
      out.push_back(rc);
      out.push_back((3.0 * Umin[g]) / ((rc - rm) * (rc - rm)));
      out.push_back((2.0 * Umin[g]) / ((rc - rm) * (rc - rm) * (rc - rm)));
    }
  return out;
}

std::vector<double> laradji_spangler_row(double rc, double rm, double rad, double density, double Umax,
                                         double Umin) {
  std::vector<double> o;
  o.push_back(rc + rad);
  o.push_back(-7.0 / 4.0 * rm);
  o.push_back(2.0 * rm * rm);
  o.push_back(Umin * M_PI * rad * density / (rm * rm * rm));
  o.push_back(rad);
  o.push_back(rm);
  double D = density * M_PI * rad;
  const double A = Umax - Umin;
  o.push_back(-D * A / (2.0 * rm * rm));
  o.push_back(2.0 * D * A / (3.0 * rm));
  o.push_back(-D * Umin);
  o.push_back(2.0 * D * Umin * rm);
  o.push_back(D * 1.3 * Umin * rm * rm);
  D = std::pow(2.0 * M_PI * density * rad, 2.0) / (rm * rm * rm);
  o.push_back(2.0 * rad + rm);
  o.push_back(2.0 * rad + rc);
  o.push_back(Umin * D * 2.0 / 30.0);
  o.push_back(-Umin * D * 7.0 * rm / 20.0);
  o.push_back(Umin * D * rm * rm / 2.0);
  o.push_back(-D * A * rm / 20.0);
  o.push_back(D * A * rm * rm / 12.0);
  o.push_back(-D * Umin * std::pow(rm, 3.0) / 6.0);
  o.push_back(D * Umin * std::pow(rm, 4.0) / 2.0);
  o.push_back(D * 1.3 * Umin * std::pow(rm, 5.0) / 2.0);
  o.push_back(D * 13.0 * Umin * std::pow(rm, 6.0) / 60.0);
  return o;
}

MpdSystem synth_vesicle(int seed, int nLipids, double density, double box) {
  MpdSystem s = base_system(seed, 6, 50000, 1000, 100);
  const int nT = s.nTypes;
  std::vector<double> Umax(nT * nT, 100.0), Umin(nT * nT, 0.0);
  Umin[kTail + kTail * nT] = -6;
  Umax[kTail + kTail * nT] = 200;
  lipid_tables(s, Umax, Umin);
  s.size[0] = s.size[1] = s.size[2] = box;
  s.present[CMD_SIZE] = true;
  const double pos[3] = {box / 2.0, box / 2.0, box / 2.0};
  const int L = 3;
  const double bl = 0.7;
  Molecule m;
  m.type = MOL_CHAIN;
  m.bonds.push_back({s.nParticles, nLipids, L, 0});
  m.constants = {0.7, 100, 1.0, 100};
  // liposome() geometry (models/lipidModels.h:1353-1464)
  const double radius = std::sqrt(((double)nLipids / density) / (4.0 * M_PI));
  for (int d = 0; d < 3; ++d)
    s.size[d] = s.size[d] < radius + pos[d] + L * bl ? pos[d] * 2.0 : s.size[d];
  const int inner = nLipids * std::pow(radius, 2.0) /
                    (std::pow(radius, 2.0) + std::pow(radius + (double)(L * 2 - 1) * bl, 2.0));
  const int outer = nLipids - inner;
  Mt19937 rng((uint32_t)s.seed);
  const double vrms = std::sqrt(3.0 * s.initialTemp);
  for (int leaf = 0; leaf < 2; ++leaf) {
    const int count = leaf == 0 ? inner : outer;
    const double sp = 3.6 / std::sqrt(double(count));
    double length = 0;
    const double dz = 2.0 / double(count);
    double z = 1.0 - dz / 2.0;
    for (int i = 0; i < count; ++i) {
      const double r = std::sqrt(1.0 - z * z);
      for (int j = 0; j < L; ++j) {
        const double shell = leaf == 0 ? (radius + bl * (double)j) : (radius + (bl * (double)(L + j)));
        const double x = pos[0] + r * std::cos(length) * shell;
        const double y = pos[1] + r * std::sin(length) * shell;
        const double zz = pos[2] + z * shell;
        const int type = leaf == 0 ? ((j == 0) ? kHead : kTail) : ((j == L - 1) ? kHead : kTail);
        double v[3];
        random_velocity(rng, vrms, v);
        add_particle(s, x, y, zz, type, v);
      }
      z = z - dz;
      length = length + sp / r;
    }
  }
  add_molecule(s, m);
  return s;
}

MpdSystem synth_bilayer(int seed, int nLipids, double density, double zsize, double deltaLXY,
                        double tension) {
  MpdSystem s = base_system(seed, 6, 1000, 10, 1);
  if (deltaLXY != 0) {
    s.deltaLXY = deltaLXY;
    s.present[CMD_DELTALXY] = true;
  }
  const int nT = s.nTypes;
  std::vector<double> Umax(nT * nT, 100.0), Umin(nT * nT, 0.0);
  Umin[kTail + kTail * nT] = -6;
  Umax[kTail + kTail * nT] = 200;
  // anchor-head entries of generate/bilayer.cpp:67-71 (UminAnchorHead = 0 here)
  Umin[kAnchor + kHead * nT] = 0;
  Umax[kAnchor + kHead * nT] = 200;
  Umin[kHead + kAnchor * nT] = Umin[kAnchor + kHead * nT];
  Umax[kHead + kAnchor * nT] = Umax[kAnchor + kHead * nT];
  lipid_tables(s, Umax, Umin);
  s.size[0] = 0;
  s.size[1] = 0;
  s.size[2] = zsize;
  s.present[CMD_SIZE] = true;
  const double pos[3] = {0, 0, s.size[2] / 2.0};
  const int L = 3;
  const double bl = 0.7, aspect = 1.0;
  Molecule m;
  m.type = MOL_CHAIN;
  m.constants = {bl, 100, 1, 100};
  std::array<int, 4> bond{s.nParticles, 0, L, 0};
  // bilayer() geometry (models/lipidModels.h:1788-1923)
  double need[3] = {std::sqrt((double)nLipids / density) * std::sqrt(aspect),
                    std::sqrt((double)nLipids / density) / std::sqrt(aspect), pos[2] * 2.0};
  for (int d = 0; d < 3; ++d) s.size[d] = (s.size[d] < need[d]) ? need[d] : s.size[d];
  Mt19937 rng((uint32_t)s.seed);
  const double vrms = std::sqrt(3.0 * s.initialTemp);
  const double ll = std::sqrt(2.0 / density);
  const int lsx = static_cast<int>(s.size[0]) / ll + 1;
  const int lsy = static_cast<int>(s.size[1]) / ll + 1;
  for (int i = 0; i < lsx; ++i)
    for (int j = 0; j < lsy; ++j) {
      const int lipid = 2 * (j * lsx + i);
      double v[3];
      if (lipid < nLipids) {
        for (int k = 0; k < L; ++k) {
          random_velocity(rng, vrms, v);
          add_particle(s, i * ll + 0.001, j * ll + 0.001, pos[2] + bl * (L - k), (k == L - 1) ? kHead : kTail, v);
        }
        bond[1]++;
      }
      if (lipid + 1 < nLipids) {
        for (int k = 0; k < L; ++k) {
          random_velocity(rng, vrms, v);
          add_particle(s, i * ll + 0.001, j * ll + 0.001, pos[2] + bl * (L + k + 1), (k == L - 1) ? kHead : kTail, v);
        }
        bond[1]++;
      }
    }
  m.bonds.push_back(bond);
  add_molecule(s, m);
  if (tension != 0) {
    s.tension = tension;
    s.present[CMD_TENSION] = true;
  }
  return s;
}

void add_continuum_sphere(MpdSystem& s, const double pos[3], double R, double uminHead, double umaxHead,
                          double umaxOther,
                          int beadType) {
  const int nT = s.nTypes;
  std::vector<double> C;
  // laradjiSpanglerFC with Umax umaxOther / Umin 0 except the head-sphere
  // entries, rc 2, rm 1, radius R-1, density 5.88 (the generator default
  // Umax is 10, continuumSphereAndLiposome.cpp:159-169).  The table's inner
  // polynomial is a barrier only while (Umax - Umin) / 6 exceeds ~2.3 |Umin|
  // (within ~1.3 sigma of the surface); deeper it is attractive and singular.
  for (int i = 0; i < nT; ++i)
    for (int j = 0; j < nT; ++j) {
      const int g = i + j * nT;
      double umax = umaxOther, umin = 0.0;
      if (g == kHead + beadType * nT || g == beadType + kHead * nT) {
        umax = umaxHead;
        umin = uminHead;
      }
      const std::vector<double> row = laradji_spangler_row(2.0, 1.0, R - 1, 5.88, umax, umin);
      C.insert(C.end(), row.begin(), row.end());
    }
  Mt19937 rng((uint32_t)s.seed);
  const double vrms = std::sqrt(3.0 * s.initialTemp);
  double v[3];
  random_velocity(rng, vrms, v);
  add_particle(s, pos[0], pos[1], pos[2], beadType, v);
  Molecule m;
  m.type = MOL_BEAD;
  m.constants = C;
  m.bonds.push_back({s.nParticles - 1, 0, 0, 0});
  add_molecule(s, m);
}

}  // namespace smd
