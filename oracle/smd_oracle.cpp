// ORACLE — test infrastructure only (see smd_oracle.h).  Never linked into the
// product library or the product MD executable.
//
// Each function restates the reference function cited beside it, keeping the
// reference's traversal and summation order so that, on one thread, results
// are bit-identical to the reference built with g++ -O3 -ffp-contract=off.
#include "smd_oracle.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const int kMaxCellSize = 512;  // MAX_CELL_SIZE (include/algorithms/cellOpt.h:26-28)

struct V3 {
  double x, y, z;
};
struct P4 {
  double x, y, z;
  int type;
};

// ---------------------------------------------------------------- MT19937
// init_genrand / genrand_int32 / genrand_res53 of Matsumoto & Nishimura (1998).
void mt_reload(orc_mt* g) {
  uint32_t* s = g->state;
  for (int i = 0; i < 624; ++i) {
    uint32_t y = (s[i] & 0x80000000u) | (s[(i + 1) % 624] & 0x7fffffffu);
    s[i] = s[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
  }
  g->left = 624;
  g->next = 0;
}

// ---------------------------------------------------------------- cells
// CellOpt::initialize / build (include/algorithms/cellOpt.h:155-212, 510-710).
struct Cells {
  int nx, ny, nz, nt;
  double cs[3];
  std::vector<int> head, next, full;
  std::vector<int> key;
};

void cells_build(Cells& c, int n, const double* pos, const double box[3], double rc) {
  c.nx = int(box[0] / rc);
  c.ny = int(box[1] / rc);
  c.nz = int(box[2] / rc);
  c.nt = c.nx * c.ny * c.nz;
  c.cs[0] = box[0] / c.nx;
  c.cs[1] = box[1] / c.ny;
  c.cs[2] = box[2] / c.nz;
  c.head.assign(c.nt, -1);
  std::vector<char> flag(c.nt, 0);
  c.next.assign(n, -1);
  c.key.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    int x = int(pos[3 * i] / c.cs[0]);
    int y = int(pos[3 * i + 1] / c.cs[1]);
    int z = int(pos[3 * i + 2] / c.cs[2]);
    x = (x >= c.nx) ? x - 1 : x;
    y = (y >= c.ny) ? y - 1 : y;
    z = (z >= c.nz) ? z - 1 : z;
    c.key[i] = x + y * c.nx + z * c.nx * c.ny;
  }
  // LIFO linked-list push, serial in bead order (cellOpt.h:571-585).
  for (int i = 0; i < n; ++i) {
    const int k = c.key[i];
    flag[k] = 1;
    c.next[i] = c.head[k];
    c.head[k] = i;
  }
  c.full.clear();
  for (int k = 0; k < c.nt; ++k)
    if (flag[k] == 1 && c.head[k] != -1) c.full.push_back(k);
}

const int kNextBox[13][3] = {{1, 0, 0},  {0, 1, 0},  {1, 1, 0},   {0, 0, 1},  {1, 0, 1},
                             {0, 1, 1},  {1, 1, 1},  {-1, 0, 1},  {0, -1, 1}, {-1, 1, 1},
                             {1, -1, 1}, {-1, -1, 1}, {1, -1, 0}};

// Neighbour cell index and minimum-image shift for half-shell entry j
// (cellOpt.h:790-823).
inline int neighbour_cell(const Cells& c, int cell, int j, const double box[3], V3& shift) {
  const int x = cell % c.nx, y = (cell / c.nx) % c.ny, z = cell / (c.nx * c.ny);
  const int nx = x + kNextBox[j][0], ny = y + kNextBox[j][1], nz = z + kNextBox[j][2];
  shift.x = 0;
  if (nx < 0) shift.x -= box[0];
  if (nx >= c.nx) shift.x += box[0];
  shift.y = 0;
  if (ny < 0) shift.y -= box[1];
  if (ny >= c.ny) shift.y += box[1];
  shift.z = 0;
  if (nz < 0) shift.z -= box[2];
  if (nz >= c.nz) shift.z += box[2];
  return ((nx + c.nx) % c.nx) + (((ny + c.ny) % c.ny) * c.nx) + (((nz + c.nz) % c.nz) * c.nx * c.ny);
}

// Force functor (include/MD.h:795-848).
inline void pair_force(double cut2, int nT, const P4& p1, const P4& p2, V3& a1, V3& a2,
                       const double* fC) {
  double dx = p1.x - p2.x;
  double dy = p1.y - p2.y;
  double dz = p1.z - p2.z;
  double dr = dx * dx + dy * dy + dz * dz;
  if (dr < cut2) {
    dr = std::sqrt(dr);
    int ci = 6 * ((p1.type * nT) + p2.type);
    ci += (int(dr / (fC[ci])) * 3);
    double mag = fC[ci] - dr;
    mag = ((fC[ci + 1] - fC[ci + 2] * mag) * mag) / dr;
    dx *= mag;
    dy *= mag;
    dz *= mag;
    a1.x += dx;
    a1.y += dy;
    a1.z += dz;
    a2.x -= dx;
    a2.y -= dy;
    a2.z -= dz;
  }
}

// Potential functor (include/MD.h:895-930).
inline double pair_potential(double cut2, int nT, const P4& p1, const P4& p2, const double* uC) {
  double dx = p1.x - p2.x, dy = p1.y - p2.y, dz = p1.z - p2.z;
  double dr = dx * dx + dy * dy + dz * dz;
  double pot = 0;
  if (dr < cut2) {
    dr = std::sqrt(dr);
    const int ci = 6 * ((p1.type * nT) + p2.type);
    if (dr <= uC[ci]) {
      pot = uC[ci] - dr;
      pot = uC[ci + 1] * pot * pot + uC[ci + 2];
    } else {
      pot = uC[ci + 3] - dr;
      pot = pot * pot * (uC[ci + 4] - pot * uC[ci + 5]);
    }
  }
  return pot;
}

inline P4 load(const double* pos, const int* type, int i) {
  P4 p;
  p.x = pos[3 * i];
  p.y = pos[3 * i + 1];
  p.z = pos[3 * i + 2];
  p.type = type ? type[i] : 0;
  return p;
}

// CellOpt::computeForce (cellOpt.h:712-926), OpenMP over occupied cells with
// per-cell locks on write-back exactly as the reference does.
int cell_force(const Cells& c, const double* pos, const int* type, const double box[3], double rc,
               int nT, const double* fC, double* acc) {
  const double cut2 = rc * rc;
  const int nfull = (int)c.full.size();
  int overflow = 0;
#ifdef _OPENMP
  std::vector<omp_lock_t> locks(c.nt);
  for (int k = 0; k < c.nt; ++k) omp_init_lock(&locks[k]);
#pragma omp parallel for schedule(dynamic)
#endif
  for (int ijk = 0; ijk < nfull; ++ijk) {
    const int i = c.full[ijk];
    std::vector<P4> tp;
    std::vector<V3> ta;
    tp.reserve(64);
    ta.reserve(64);
    int ni = 0;
    for (int m = c.head[i]; m != -1; m = c.next[m], ++ni) {
      if (ni > kMaxCellSize) {
#pragma omp atomic write
        overflow = 1;
      }
      tp.push_back(load(pos, type, m));
      ta.push_back(V3{0, 0, 0});
      for (int j = 0; j < ni; ++j) pair_force(cut2, nT, tp[ni], tp[j], ta[ni], ta[j], fC);
    }
    for (int j = 0; j < 13; ++j) {
      V3 sh;
      const int k = neighbour_cell(c, i, j, box, sh);
      if (c.head[k] == -1) continue;
#ifdef _OPENMP
      omp_set_lock(&locks[k]);
#endif
      for (int nn = c.head[k]; nn != -1; nn = c.next[nn]) {
        P4 cp = load(pos, type, nn);
        cp.x += sh.x;
        cp.y += sh.y;
        cp.z += sh.z;
        V3 ca{0, 0, 0};
        for (int m = 0; m < ni; ++m) pair_force(cut2, nT, tp[m], cp, ta[m], ca, fC);
        acc[3 * nn] += ca.x;
        acc[3 * nn + 1] += ca.y;
        acc[3 * nn + 2] += ca.z;
      }
#ifdef _OPENMP
      omp_unset_lock(&locks[k]);
#endif
    }
#ifdef _OPENMP
    omp_set_lock(&locks[i]);
#endif
    int q = 0;
    for (int m = c.head[i]; m != -1; m = c.next[m], ++q) {
      acc[3 * m] += ta[q].x;
      acc[3 * m + 1] += ta[q].y;
      acc[3 * m + 2] += ta[q].z;
    }
#ifdef _OPENMP
    omp_unset_lock(&locks[i]);
#endif
  }
#ifdef _OPENMP
  for (int k = 0; k < c.nt; ++k) omp_destroy_lock(&locks[k]);
#endif
  return overflow ? -1 : 0;
}

// CellOpt::computePotential (cellOpt.h:928-1041) and computeDPotential
// (cellOpt.h:1043-1180); scale==nullptr selects the plain potential.
double cell_potential(const Cells& c, const double* pos, const int* type, const double box[3],
                      double rc, int nT, const double* uC, const double* scale) {
  const double cut2 = rc * rc;
  const int nfull = (int)c.full.size();
  double total = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) reduction(+ : total)
#endif
  for (int ijk = 0; ijk < nfull; ++ijk) {
    const int i = c.full[ijk];
    std::vector<P4> tp;
    tp.reserve(64);
    int ni = 0;
    auto term = [&](const P4& a, const P4& b) -> double {
      if (!scale) return pair_potential(cut2, nT, a, b, uC);
      const double oldP = pair_potential(cut2, nT, a, b, uC);
      P4 pa = a, pb = b;
      pa.x *= scale[0];
      pa.y *= scale[1];
      pa.z *= scale[2];
      pb.x *= scale[0];
      pb.y *= scale[1];
      pb.z *= scale[2];
      const double newP = pair_potential(cut2, nT, pa, pb, uC);
      return oldP - newP;
    };
    for (int m = c.head[i]; m != -1; m = c.next[m], ++ni) {
      tp.push_back(load(pos, type, m));
      for (int j = 0; j < ni; ++j) total += term(tp[ni], tp[j]);
    }
    for (int j = 0; j < 13; ++j) {
      V3 sh;
      const int k = neighbour_cell(c, i, j, box, sh);
      if (c.head[k] == -1) continue;
      for (int nn = c.head[k]; nn != -1; nn = c.next[nn]) {
        P4 cp = load(pos, type, nn);
        cp.x += sh.x;
        cp.y += sh.y;
        cp.z += sh.z;
        for (int m = 0; m < ni; ++m) total += term(tp[m], cp);
      }
    }
  }
  return total;
}

// ---------------------------------------------------------------- bonded
// Minimum image used by the bonded terms (include/system.h:1806-1832).
inline void min_image(V3& d, const double box[3]) {
  if (d.x > box[0] / 2.0) d.x -= box[0];
  if (d.x < -box[0] / 2.0) d.x += box[0];
  if (d.y > box[1] / 2.0) d.y -= box[1];
  if (d.y < -box[1] / 2.0) d.y += box[1];
  if (d.z > box[2] / 2.0) d.z -= box[2];
  if (d.z < -box[2] / 2.0) d.z += box[2];
}
inline V3 diff(const double* pos, int a, int b, const double box[3]) {
  V3 d{pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  min_image(d, box);
  return d;
}
inline void add(double* acc, int i, const V3& v) {
  acc[3 * i] += v.x;
  acc[3 * i + 1] += v.y;
  acc[3 * i + 2] += v.z;
}

// harmonicF (include/MD.h:384-403); a1 += f, a2 -= f.
inline void harmonic_force(V3 d, V3& a1, V3& a2, const double* c) {
  const double dr = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
  double mag = dr - c[0];
  mag = -mag * c[1] / dr;
  d.x *= mag;
  d.y *= mag;
  d.z *= mag;
  a1.x += d.x;
  a1.y += d.y;
  a1.z += d.z;
  a2.x -= d.x;
  a2.y -= d.y;
  a2.z -= d.z;
}
inline double harmonic_potential(V3 d, const double* c) {
  const double dr = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
  double p = dr - c[0];
  return 0.5 * c[1] * p * p;
}
// bendF (include/MD.h:683-723).
inline void bend_force(V3 da, V3 db, V3& a1, V3& a2, V3& a3, const double* c) {
  const double dra = std::sqrt(da.x * da.x + da.y * da.y + da.z * da.z);
  const double drb = std::sqrt(db.x * db.x + db.y * db.y + db.z * db.z);
  da.x /= dra;
  da.y /= dra;
  da.z /= dra;
  db.x /= drb;
  db.y /= drb;
  db.z /= drb;
  const double cs = (da.x * db.x) + (da.y * db.y) + (da.z * db.z);
  double mag = c[0] - cs;
  mag *= c[1];
  double ba = mag * (db.x - (da.x * cs)) / dra;
  double bb = mag * (da.x - (db.x * cs)) / drb;
  a1.x += ba;
  a2.x += (bb - ba);
  a3.x -= bb;
  ba = mag * (db.y - (da.y * cs)) / dra;
  bb = mag * (da.y - (db.y * cs)) / drb;
  a1.y += ba;
  a2.y += (bb - ba);
  a3.y -= bb;
  ba = mag * (db.z - (da.z * cs)) / dra;
  bb = mag * (da.z - (db.z * cs)) / drb;
  a1.z += ba;
  a2.z += (bb - ba);
  a3.z -= bb;
}
// bendP (include/MD.h:769-789).
inline double bend_potential(V3 da, V3 db, const double* c) {
  const double dra = std::sqrt(da.x * da.x + da.y * da.y + da.z * da.z);
  const double drb = std::sqrt(db.x * db.x + db.y * db.y + db.z * db.z);
  da.x /= dra;
  da.y /= dra;
  da.z /= dra;
  db.x /= drb;
  db.y /= drb;
  db.z /= drb;
  const double cs = (da.x * db.x) + (da.y * db.y) + (da.z * db.z);
  double p = c[0] - cs;
  return c[1] * p * p * 0.5;
}

inline V3 accv(double* acc, int i) { return V3{acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]}; }
inline void setv(double* acc, int i, const V3& v) {
  acc[3 * i] = v.x;
  acc[3 * i + 1] = v.y;
  acc[3 * i + 2] = v.z;
}

// One chain of the CHAIN residue (include/system.h:1800-1862).
void chain_force_one(const double* pos, const double box[3], int k, int length, const double* c,
                     double* acc) {
  for (int l = k; l < k + length - 3; ++l) {
    const V3 da = diff(pos, l, l + 1, box), db = diff(pos, l + 1, l + 2, box);
    V3 a1 = accv(acc, l), a2 = accv(acc, l + 1), a3 = accv(acc, l + 2);
    harmonic_force(da, a1, a2, c);
    bend_force(da, db, a1, a2, a3, c + 2);
    setv(acc, l, a1);
    setv(acc, l + 1, a2);
    setv(acc, l + 2, a3);
  }
  const int f = k + length - 3, s = k + length - 2, t = k + length - 1;
  const V3 da = diff(pos, f, s, box), db = diff(pos, s, t, box);
  V3 a1 = accv(acc, f), a2 = accv(acc, s), a3 = accv(acc, t);
  harmonic_force(da, a1, a2, c);
  harmonic_force(db, a2, a3, c);
  bend_force(da, db, a1, a2, a3, c + 2);
  setv(acc, f, a1);
  setv(acc, s, a2);
  setv(acc, t, a3);
}

double chain_potential_impl(const double* pos, const double box[3], int start, int nChains,
                            int length, const double* c, const double* scale) {
  double total = 0;
  for (int k = start; k < start + length * nChains; k += length) {
    auto term = [&](V3 da, V3 db, bool last) -> double {
      double oldP = harmonic_potential(da, c);
      if (last) oldP += harmonic_potential(db, c);
      oldP += bend_potential(da, db, c + 2);
      if (!scale) return oldP;
      da.x *= scale[0];
      da.y *= scale[1];
      da.z *= scale[2];
      db.x *= scale[0];
      db.y *= scale[1];
      db.z *= scale[2];
      double newP = harmonic_potential(da, c);
      if (last) newP += harmonic_potential(db, c);
      newP += bend_potential(da, db, c + 2);
      return oldP - newP;
    };
    for (int l = k; l < k + length - 3; ++l) {
      const V3 da = diff(pos, l, l + 1, box), db = diff(pos, l + 1, l + 2, box);
      if (!scale) {
        total += harmonic_potential(da, c);
        total += bend_potential(da, db, c + 2);
      } else {
        total += term(da, db, false);
      }
    }
    const int f = k + length - 3, s = k + length - 2, t = k + length - 1;
    const V3 da = diff(pos, f, s, box), db = diff(pos, s, t, box);
    if (!scale) {
      total += harmonic_potential(da, c);
      total += harmonic_potential(db, c);
      total += bend_potential(da, db, c + 2);
    } else {
      total += term(da, db, true);
    }
  }
  return total;
}

// ---------------------------------------------------------------- BEAD
// beadForce / beadPotential / beadBeadForce / beadBeadPotential (include/MD.h:165-338).
const int kBBOff = 11;  // BEADBEADOFFSET

void bead_force_fn(V3 d, V3& a1, V3& a2, const double* C, double cut2) {
  double dr = d.x * d.x + d.y * d.y + d.z * d.z;
  double mag = 0;
  const double rminD = C[4] + C[5];
  const double rminD2 = rminD * rminD;
  if (rminD2 <= dr && dr < cut2) {
    dr = std::sqrt(dr);
    const double E = C[0] - dr, E2 = E * E, E3 = E * E2;
    mag = 2.0 * (0.4 * E3 + C[1] * E2 + C[2] * E) / (dr);
    mag += 4.0 * E2 + 8.0 * C[1] * E + 6.0 * C[2];
    mag *= (E2 * C[3]) / (dr * dr);
  } else if (dr < rminD2) {
    dr = std::sqrt(dr);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
    mag = (B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
    mag += (4.0 * B3 * C[6] + 3.0 * B2 * C[7] + 2.0 * B * C[8] + C[9]);
    mag /= dr * dr;
  }
  d.x *= mag;
  d.y *= mag;
  d.z *= mag;
  a1.x += d.x;
  a1.y += d.y;
  a1.z += d.z;
  a2.x -= d.x;
  a2.y -= d.y;
  a2.z -= d.z;
}
double bead_potential_fn(V3 d, const double* C, double cut2) {
  double dr = d.x * d.x + d.y * d.y + d.z * d.z;
  const double rminD = C[4] + C[5];
  const double rminD2 = rminD * rminD;
  double pot = 0;
  if (rminD2 <= dr && dr < cut2) {
    dr = std::sqrt(dr);
    const double E = C[0] - dr, E2 = E * E, E3 = E * E2;
    pot = 2.0 * E3 * (0.4 * E2 + C[1] * E + C[2]) * C[3] / (dr);
  } else if (dr < rminD2) {
    dr = std::sqrt(dr);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
    pot = (B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
  }
  return pot;
}
void beadbead_force_fn(V3 d, V3& a1, V3& a2, const double* C, double cut2) {
  double dr = d.x * d.x + d.y * d.y + d.z * d.z;
  double mag = 0;
  const double rminD = C[0 + kBBOff], rminD2 = rminD * rminD;
  if (rminD2 <= dr && dr < cut2) {
    dr = std::sqrt(dr);
    const double E = C[1 + kBBOff] - dr, E2 = E * E, E3 = E * E2;
    mag = E3 *
          (6.0 * C[2 + kBBOff] * E2 + 5.0 * C[3 + kBBOff] * E + 4.0 * C[4 + kBBOff] +
           (C[2 + kBBOff] * E3 + C[3 + kBBOff] * E2 + C[4 + kBBOff] * E) / dr) /
          (dr * dr);
  } else if (dr < rminD2) {
    dr = std::sqrt(dr);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2, B5 = B2 * B3;
    mag = 5.0 * B4 * C[5 + kBBOff] + 4.0 * B3 * C[6 + kBBOff] + 3.0 * B2 * C[7 + kBBOff] +
          2.0 * B * C[8 + kBBOff] + C[9 + kBBOff];
    mag += (B5 * C[5 + kBBOff] + B4 * C[6 + kBBOff] + B3 * C[7 + kBBOff] + B2 * C[8 + kBBOff] +
            B * C[9 + kBBOff] + C[10 + kBBOff]) /
           (dr);
    mag /= dr * dr;
  }
  d.x *= mag;
  d.y *= mag;
  d.z *= mag;
  a1.x += d.x;
  a1.y += d.y;
  a1.z += d.z;
  a2.x -= d.x;
  a2.y -= d.y;
  a2.z -= d.z;
}
double beadbead_potential_fn(V3 d, const double* C, double cut2) {
  double dr = d.x * d.x + d.y * d.y + d.z * d.z;
  const double rminD = C[0 + kBBOff], rminD2 = rminD * rminD;
  double pot = 0;
  if (rminD2 <= dr && dr < cut2) {
    dr = std::sqrt(dr);
    const double E = C[1 + kBBOff] - dr, E2 = E * E, E4 = E2 * E2;
    pot = E4 * (C[2 + kBBOff] * E2 + C[3 + kBBOff] * E + C[4 + kBBOff]) / dr;
  } else if (dr < rminD2) {
    dr = std::sqrt(dr);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2, B5 = B2 * B3;
    pot = (B5 * C[5 + kBBOff] + B4 * C[6 + kBBOff] + B3 * C[7 + kBBOff] + B2 * C[8 + kBBOff] +
           B * C[9 + kBBOff] + C[10 + kBBOff]) /
          (dr);
  }
  return pot;
}

}  // namespace

// ================================================================ C API
namespace {
// Bonds (l, l+1) of each chain except its last (the reference's loop stops at
// length-2); d = x_l - x_{l+1} with the minimum image, z at the bond's middle
// folded into [0, Lz).
template <typename F>
void ztorque_bonds(const double* pos, const double box[3], int nb, const int* blocks, F&& f) {
  for (int j = 0; j < nb; ++j) {
    const int start = blocks[3 * j], nChains = blocks[3 * j + 1], length = blocks[3 * j + 2];
    for (int k = start; k < start + length * nChains; k += length)
      for (int l = k; l < k + length - 2; ++l) {
        const V3 d = diff(pos, l, l + 1, box);
        double zHeight = pos[3 * l + 2] + d.z / 2.0;
        while (zHeight >= box[2]) zHeight -= box[2];
        while (zHeight < 0) zHeight += box[2];
        f(l, d, zHeight);
      }
  }
}
// magnitude (include/algorithms/functions.h:250-257)
inline double magnitude3(const V3& d) {
  double sum = 0;
  sum += d.x * d.x;
  sum += d.y * d.y;
  sum += d.z * d.z;
  return std::sqrt(sum);
}
}  // namespace

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n < 1 ? 1 : n);
#else
  (void)n;
#endif
}

void orc_mt_seed(orc_mt* g, uint32_t seed) {
  g->state[0] = seed;
  for (int i = 1; i < 624; ++i)
    g->state[i] = 1812433253u * (g->state[i - 1] ^ (g->state[i - 1] >> 30)) + (uint32_t)i;
  mt_reload(g);
}

uint32_t orc_mt_u32(orc_mt* g) {
  if (g->left == 0) mt_reload(g);
  --g->left;
  uint32_t y = g->state[g->next++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  return y ^ (y >> 18);
}

double orc_mt_rand53(orc_mt* g) {
  const uint32_t a = orc_mt_u32(g) >> 5, b = orc_mt_u32(g) >> 6;
  return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0);
}

void orc_mt_fill53(uint32_t seed, int n, double* out) {
  orc_mt g;
  orc_mt_seed(&g, seed);
  for (int i = 0; i < n; ++i) out[i] = orc_mt_rand53(&g);
}

void orc_cell_keys(int n, const double* pos, const double box[3], double rc, int* keys) {
  Cells c;
  cells_build(c, n, pos, box, rc);
  std::memcpy(keys, c.key.data(), sizeof(int) * (size_t)n);
}

long orc_pair_list(int n, const double* pos, const double box[3], double rc, int* pairs, long cap) {
  Cells c;
  cells_build(c, n, pos, box, rc);
  const double cut2 = rc * rc;
  long count = 0;
  auto rec = [&](int a, const V3& pa, int b, const V3& pb) {
    const double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
    if (dx * dx + dy * dy + dz * dz < cut2) {
      if (count < cap) {
        pairs[2 * count] = a;
        pairs[2 * count + 1] = b;
      }
      ++count;
    }
  };
  for (int i : c.full) {
    std::vector<int> idx;
    for (int m = c.head[i]; m != -1; m = c.next[m]) {
      if ((int)idx.size() > kMaxCellSize) return -1;
      const V3 pm{pos[3 * m], pos[3 * m + 1], pos[3 * m + 2]};
      for (int j : idx) rec(m, pm, j, V3{pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]});
      idx.push_back(m);
    }
    for (int j = 0; j < 13; ++j) {
      V3 sh;
      const int k = neighbour_cell(c, i, j, box, sh);
      for (int nn = c.head[k]; nn != -1; nn = c.next[nn]) {
        const V3 pn{pos[3 * nn] + sh.x, pos[3 * nn + 1] + sh.y, pos[3 * nn + 2] + sh.z};
        for (int m : idx) rec(m, V3{pos[3 * m], pos[3 * m + 1], pos[3 * m + 2]}, nn, pn);
      }
    }
  }
  return count;
}

int orc_pair_force(int n, const double* pos, const int* type, const double box[3], double rc,
                   int nTypes, const double* fconst, double* acc) {
  Cells c;
  cells_build(c, n, pos, box, rc);
  return cell_force(c, pos, type, box, rc, nTypes, fconst, acc);
}

double orc_pair_potential(int n, const double* pos, const int* type, const double box[3], double rc,
                          int nTypes, const double* uconst) {
  Cells c;
  cells_build(c, n, pos, box, rc);
  return cell_potential(c, pos, type, box, rc, nTypes, uconst, nullptr);
}

double orc_pair_dpotential(int n, const double* pos, const int* type, const double box[3], double rc,
                           int nTypes, const double* uconst, const double scale[3]) {
  Cells c;
  cells_build(c, n, pos, box, rc);
  return cell_potential(c, pos, type, box, rc, nTypes, uconst, scale);
}

void orc_chain_force(const double* pos, const double box[3], int start, int nChains, int length,
                     const double* c, double* acc) {
#ifdef _OPENMP
#pragma omp parallel for
#endif
  for (int q = 0; q < nChains; ++q) chain_force_one(pos, box, start + q * length, length, c, acc);
}

double orc_chain_potential(const double* pos, const double box[3], int start, int nChains, int length,
                           const double* c) {
  return chain_potential_impl(pos, box, start, nChains, length, c, nullptr);
}

double orc_chain_dpotential(const double* pos, const double box[3], int start, int nChains,
                            int length, const double* c, const double scale[3]) {
  return chain_potential_impl(pos, box, start, nChains, length, c, scale);
}

// BOND residue: pairs list[2k], list[2k+1] with constants {l0, k}
// (Blob::doBondForce / doBondPotential / doBondDPotential,
// include/system.h:1880-1934, 2718-2745, 3399-3435).
void orc_bond_force(const double* pos, const double box[3], int nb, const int* list, const double* c,
                    double* acc) {
  for (int j = 0; j < nb; ++j) {
    const int f = list[2 * j], s = list[2 * j + 1];
    const V3 d = diff(pos, f, s, box);
    V3 a1 = accv(acc, f), a2 = accv(acc, s);
    harmonic_force(d, a1, a2, c);
    setv(acc, f, a1);
    setv(acc, s, a2);
  }
}

static double bond_energy(const double* pos, const double box[3], int nb, const int* list, const double* c,
                          const double* scale) {
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    V3 d = diff(pos, list[2 * j], list[2 * j + 1], box);
    const double oldP = harmonic_potential(d, c);
    if (!scale) {
      total += oldP;
      continue;
    }
    d.x *= scale[0];
    d.y *= scale[1];
    d.z *= scale[2];
    total += oldP - harmonic_potential(d, c);
  }
  return total;
}

double orc_bond_potential(const double* pos, const double box[3], int nb, const int* list, const double* c) {
  return bond_energy(pos, box, nb, list, c, nullptr);
}

double orc_bond_dpotential(const double* pos, const double box[3], int nb, const int* list, const double* c,
                           const double scale[3]) {
  return bond_energy(pos, box, nb, list, c, scale);
}

// BEND residue: triplets list[3k..3k+2] with constants {a, k}
// (Blob::doBendForce / doBendPotential / doBendDPotential,
// include/system.h:1975-2040, 2782-2821, 3477-3524).
void orc_bend_force(const double* pos, const double box[3], int nb, const int* list, const double* c,
                    double* acc) {
  for (int j = 0; j < nb; ++j) {
    const int f = list[3 * j], s = list[3 * j + 1], t = list[3 * j + 2];
    const V3 da = diff(pos, f, s, box), db = diff(pos, s, t, box);
    V3 a1 = accv(acc, f), a2 = accv(acc, s), a3 = accv(acc, t);
    bend_force(da, db, a1, a2, a3, c);
    setv(acc, f, a1);
    setv(acc, s, a2);
    setv(acc, t, a3);
  }
}

static double bend_energy(const double* pos, const double box[3], int nb, const int* list, const double* c,
                          const double* scale) {
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    V3 da = diff(pos, list[3 * j], list[3 * j + 1], box), db = diff(pos, list[3 * j + 1], list[3 * j + 2], box);
    const double oldP = bend_potential(da, db, c);
    if (!scale) {
      total += oldP;
      continue;
    }
    da.x *= scale[0];
    da.y *= scale[1];
    da.z *= scale[2];
    db.x *= scale[0];
    db.y *= scale[1];
    db.z *= scale[2];
    total += oldP - bend_potential(da, db, c);
  }
  return total;
}

double orc_bend_potential(const double* pos, const double box[3], int nb, const int* list, const double* c) {
  return bend_energy(pos, box, nb, list, c, nullptr);
}

double orc_bend_dpotential(const double* pos, const double box[3], int nb, const int* list, const double* c,
                           const double scale[3]) {
  return bend_energy(pos, box, nb, list, c, scale);
}

}  // extern "C"

namespace {

// The hash-cell search of the many-sphere branches (Blob::doBeadForce above
// 20 beads, include/system.h:2104-2163; doNanoCoreForce from 50 cores,
// :2264-2318), with the cell helpers of analysis/cellInclude/cell.h:
// int(L / (2 r)) cells per axis of side L / n (getCell floors p / side),
// each cell's beads in reverse index order (createIMap pushes to the front of
// a list), and the 27 neighbours of the sphere's cell with periodic wrap,
// x offset outermost (neighIndices).  With fewer than three cells along an
// axis a neighbour repeats, and its beads are visited again, as in the
// reference.
struct HashCells {
  int n[3];
  double side[3];
  std::unordered_map<int, std::vector<int>> members;  // in index order; visited back to front

  HashCells(int np, const double* pos, const double box[3], double range) {
    for (int a = 0; a < 3; ++a) {
      n[a] = int(box[a] / (range * 2.0));
      side[a] = box[a] / n[a];
    }
    for (int i = 0; i < np; ++i) members[hash_of(pos + 3 * i)].push_back(i);
  }
  int hash_of(const double* p) const {
    const int c[3] = {int(std::floor(p[0] / side[0])), int(std::floor(p[1] / side[1])),
                      int(std::floor(p[2] / side[2]))};
    return c[0] + c[1] * n[0] + c[2] * n[0] * n[1];
  }
  template <class F>
  void visit(const double* p, F&& f) const {
    const int h = hash_of(p);
    const int cx = h % n[0], cy = (h / n[0]) % n[1], cz = (h / (n[0] * n[1])) % n[2];
    for (int i = -1; i < 2; ++i)
      for (int j = -1; j < 2; ++j)
        for (int k = -1; k < 2; ++k) {
          const int key = (cx + i + n[0]) % n[0] + ((cy + j + n[1]) % n[1]) * n[0] +
                          ((cz + k + n[2]) % n[2]) * n[0] * n[1];
          const auto it = members.find(key);
          if (it == members.end()) continue;
          for (auto b = it->second.rbegin(); b != it->second.rend(); ++b) f(*b);
        }
  }
};

}  // namespace

extern "C" {

void orc_bead_force(int n, const double* pos, const int* type, const double box[3], int nT, int nb,
                    const int* idx, const double* C, double* acc) {
  // bead-bead pairs (include/system.h:2072-2098); with a single residue the
  // bead list is this residue's beads.
  for (int j = 0; j < nb; ++j) {
    for (int k = j + 1; k < nb; ++k) {
      const int f = idx[j], s = idx[k];
      const V3 d = diff(pos, f, s, box);
      const double R = C[4];
      double cut2 = R + R + 2.0;
      cut2 *= cut2;
      const int ci = 22 * ((type[f] * nT) + type[s]);
      V3 a1 = accv(acc, f), a2 = accv(acc, s);
      beadbead_force_fn(d, a1, a2, &C[ci], cut2);
      setv(acc, f, a1);
      setv(acc, s, a2);
    }
  }
  const double cutR = C[0];
  const double cut2R = cutR * cutR;
  if (nb > 20) {
    // hash-cell branch: every other bead, the other spheres included
    const HashCells cells(n, pos, box, cutR);
    for (int j = 0; j < nb; ++j) {
      const int f = idx[j];
      double ax = 0, ay = 0, az = 0;
      cells.visit(pos + 3 * f, [&](int k) {
        if (k == f) return;
        const V3 d = diff(pos, f, k, box);
        V3 ab{0, 0, 0};
        V3 a2 = accv(acc, k);
        const int ci = 22 * ((type[f] * nT) + type[k]);
        bead_force_fn(d, ab, a2, &C[ci], cut2R);
        setv(acc, k, a2);
        ax += ab.x;
        ay += ab.y;
        az += ab.z;
      });
      acc[3 * f] += ax;
      acc[3 * f + 1] += ay;
      acc[3 * f + 2] += az;
    }
    return;
  }
  // brute-force branch for <= 20 beads (include/system.h:2165-2210)
  for (int j = 0; j < nb; ++j) {
    const int f = idx[j];
    double ax = 0, ay = 0, az = 0;
    for (int k = 0; k < n; ++k) {
      bool excluded = false;
      for (int q = 0; q < nb; ++q) excluded = excluded || (idx[q] == k);
      if (excluded) continue;
      const V3 d = diff(pos, f, k, box);
      V3 ab{0, 0, 0};
      V3 a2 = accv(acc, k);
      const int ci = 22 * ((type[f] * nT) + type[k]);
      bead_force_fn(d, ab, a2, &C[ci], cut2R);
      setv(acc, k, a2);
      ax += ab.x;
      ay += ab.y;
      az += ab.z;
    }
    acc[3 * f] += ax;
    acc[3 * f + 1] += ay;
    acc[3 * f + 2] += az;
  }
}

// doBeadPotential sums each bead's inner loop under an OpenMP reduction
// (include/system.h:2967, 2999): a private sum from zero, added to the total
// at the loop's end; doBeadDPotential's pragmas are commented out, so its
// terms go straight into the total.
static double bead_energy(int n, const double* pos, const int* type, const double box[3], int nT,
                          int nb, const int* idx, const double* C, const double* scale) {
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    double part = 0;
    double& sum = scale ? total : part;
    for (int k = j + 1; k < nb; ++k) {
      const int f = idx[j], s = idx[k];
      V3 d = diff(pos, f, s, box);
      const double R = C[4];
      double cut2 = R + R + 2.0;
      cut2 *= cut2;
      const int ci = 22 * ((type[f] * nT) + type[s]);
      const double oldP = beadbead_potential_fn(d, &C[ci], cut2);
      if (!scale) {
        sum += oldP;
        continue;
      }
      d.x *= scale[0];
      d.y *= scale[1];
      d.z *= scale[2];
      sum += oldP - beadbead_potential_fn(d, &C[ci], cut2);
    }
    if (!scale) total += part;
  }
  const double cutR = C[0];
  const double cut2R = cutR * cutR;
  for (int j = 0; j < nb; ++j) {
    const int f = idx[j];
    double part = 0;
    double& sum = scale ? total : part;
    for (int k = 0; k < n; ++k) {
      if (k == f) continue;
      V3 d = diff(pos, f, k, box);
      const int ci = 22 * ((type[f] * nT) + type[k]);
      const double oldP = bead_potential_fn(d, &C[ci], cut2R);
      if (!scale) {
        sum += oldP;
        continue;
      }
      d.x *= scale[0];
      d.y *= scale[1];
      d.z *= scale[2];
      sum += oldP - bead_potential_fn(d, &C[ci], cut2R);
    }
    if (!scale) total += part;
  }
  return total;
}

double orc_bead_potential(int n, const double* pos, const int* type, const double box[3], int nT,
                          int nb, const int* idx, const double* C) {
  return bead_energy(n, pos, type, box, nT, nb, idx, C, nullptr);
}

double orc_bead_dpotential(int n, const double* pos, const int* type, const double box[3], int nT,
                           int nb, const int* idx, const double* C, const double scale[3]) {
  return bead_energy(n, pos, type, box, nT, nb, idx, C, scale);
}


// ---------------------------------------------------------------- field residues
// Expressions keep the reference's evaluation order (the oracle is built
// without FMA contraction), so a one-thread run matches it bit for bit.

void orc_boundary_force(const double* pos, const double box[3], int nb, const int* beads, const double* c,
                        double* acc) {
  const int dim = static_cast<int>(c[0]);
  for (int j = 0; j < nb; ++j) {
    const int i = beads[j];
    double d = pos[3 * i + dim] - c[1];
    d -= (d > box[dim] / 2.0) ? box[dim] : 0;
    d += (d < -box[dim] / 2.0) ? box[dim] : 0;
    const double dir = (d < 0) ? -1.0 : 1.0;
    d = std::fabs(d);
    const double d2 = d * d;
    double magnitude = 0;
    if (d2 <= 2.0) magnitude = c[3] * (4.0 / (d2 * d2 * d) - 2.0 / (d2 * d));
    acc[3 * i + dim] += magnitude * dir;
  }
}

double orc_boundary_potential(const double* pos, const double box[3], int nb, const int* beads, const double* c) {
  const int dim = static_cast<int>(c[0]);
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    const int i = beads[j];
    double d = pos[3 * i + dim] - c[1];
    d -= (d > box[dim] / 2.0) ? box[dim] : 0;
    d += (d < -box[dim] / 2.0) ? box[dim] : 0;
    d = std::fabs(d);
    double potential = 0;
    d = d * d;
    if (d <= 2.0) potential = c[3] * (1.0 / (d * d) - 1.0 / d);
    total += potential;
  }
  return total;
}

// The force reads the absolute z; the potential reads z minus the residue's
// first constant (both as in the reference).
void orc_floating_base_force(const double* pos, const int* type, int nb, const int* beads, const double* c,
                             double* acc) {
  for (int j = 0; j < nb; ++j) {
    const int i = beads[j];
    const double z = pos[3 * i + 2];
    const double* C = c + 6 * type[i];
    if (z <= C[0]) {
      acc[3 * i + 2] += C[3] * z * z * z - 2 * C[3] * C[0] * z * z + (2 * C[2] + C[3] * C[0] * C[0]) * z;
    } else if (z < C[1]) {
      const double rcz = z - C[1];
      acc[3 * i + 2] += C[5] * (rcz * rcz) *
                        (2 * z * z - (4 * C[1] - 7 * C[0]) * z + 2 * C[1] * C[1] + C[0] * (-7 * C[1] + 6 * C[0]));
    }
  }
}

double orc_floating_base_potential(const double* pos, const int* type, int nb, const int* beads, const double* c) {
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    const int i = beads[j];
    const double z = pos[3 * i + 2] - c[0];
    const double* C = c + 6 * type[i];
    double potential = 0;
    if (z <= C[0]) {
      const double rmz = C[0] - z;
      potential = C[2] * (C[0] * C[0] - z * z) + C[3] * rmz * rmz * rmz * ((C[0] / 3.0) - (1.0 / 4.0) * rmz) + C[4];
    } else if (z < C[1]) {
      const double rcz = C[1] - z;
      potential = C[5] * rcz * rcz * rcz * (rcz * ((2.0 / 5.0) * rcz - (7.0 / 4.0) * C[0]) + (2.0) * C[0] * C[0]);
    }
    total += potential;
  }
  return total;
}

void orc_zpower_force(const double* pos, int nb, const int* blocks, const double* c, double* acc) {
  for (int j = 0; j < nb; ++j)
    for (int k = blocks[2 * j]; k < blocks[2 * j] + blocks[2 * j + 1]; ++k)
      acc[3 * k + 2] += c[0] * std::pow(pos[3 * k + 2], c[1]);
}

double orc_zpower_potential(const double* pos, int nb, const int* blocks, const double* c) {
  double total = 0;
  for (int j = 0; j < nb; ++j)
    for (int k = blocks[2 * j]; k < blocks[2 * j] + blocks[2 * j + 1]; ++k)
      total += -c[0] * std::pow(pos[3 * k + 2], c[1] + 1) / (c[1] + 1);
  return total;
}


void orc_ztorque_force(const double* pos, const double box[3], int nb, const int* blocks, const double* c,
                       double* acc) {
  ztorque_bonds(pos, box, nb, blocks, [&](int l, const V3& d, double z) {
    const double mag = magnitude3(d);
    double epsilon = c[0] - c[1] * std::tanh(c[2] * (z - c[3]));
    if (z > c[3]) epsilon = 0;
    const double m = -epsilon * (d.z / (mag * mag * mag * mag));
    double* a1 = acc + 3 * l;
    double* a2 = acc + 3 * (l + 1);
    a1[0] += d.z * m * d.x;
    a1[1] += d.z * m * d.y;
    a1[2] += -m * (d.x * d.x + d.y * d.y);
    a2[0] += -d.z * m * d.x;
    a2[1] += -d.z * m * d.y;
    a2[2] += m * (d.x * d.x + d.y * d.y);
  });
}

double orc_ztorque_potential(const double* pos, const double box[3], int nb, const int* blocks, const double* c) {
  double total = 0;
  ztorque_bonds(pos, box, nb, blocks, [&](int, const V3& d, double z) {
    const double cosTheta = std::abs(d.z) / magnitude3(d);
    const double epsilon = c[0] - c[1] * std::tanh(c[2] * (z - c[3]));
    total += epsilon * (1.0 - cosTheta * cosTheta) / 2.0;
  });
  return total;
}


void orc_ball_force(const double* pos, const double box[3], int nb, const int* bonds, const double* c, double* acc) {
  if (nb <= 0) return;
  const int first = bonds[0];
  double ax = 0, ay = 0, az = 0;
  for (int j = 0; j < nb; ++j) {
    const int second = bonds[2 * j + 1];
    V3 d = diff(pos, first, second, box);
    double dr = d.x * d.x + d.y * d.y + d.z * d.z;
    V3 aFirst{0, 0, 0};
    if (dr < c[0] * c[0]) {
      dr = std::sqrt(dr);
      double magnitude = dr - c[0];
      magnitude = -magnitude * c[1] / dr;
      d.x *= magnitude;
      d.y *= magnitude;
      d.z *= magnitude;
      aFirst.x += d.x;
      aFirst.y += d.y;
      aFirst.z += d.z;
      acc[3 * second] -= d.x;
      acc[3 * second + 1] -= d.y;
      acc[3 * second + 2] -= d.z;
    }
    ax += aFirst.x;
    ay += aFirst.y;
    az += aFirst.z;
  }
  acc[3 * first] += ax;
  acc[3 * first + 1] += ay;
  acc[3 * first + 2] += az;
}

double orc_ball_potential(const double* pos, const double box[3], int nb, const int* bonds, const double* c) {
  double total = 0;
  for (int j = 0; j < nb; ++j) {
    const V3 d = diff(pos, bonds[2 * j], bonds[2 * j + 1], box);
    double dr = d.x * d.x + d.y * d.y + d.z * d.z;
    double potential = 0;
    if (dr < c[0] * c[0]) {
      dr = std::sqrt(dr);
      potential = dr - c[0];
      potential = 0.5 * c[1] * potential * potential;
    }
    total += potential;
  }
  return total;
}


void orc_nanocore_force(int n, const double* pos, const double box[3], int nb, const int* idx, const double* C,
                        double* acc) {
  if (nb >= 50) {
    // hash-cell branch: cells from the largest range, truncated to an int
    int range = 0;
    for (int j = 0; j < nb; ++j)
      if (C[22 * j] > range) range = int(C[22 * j]);
    const HashCells cells(n, pos, box, (double)range);
    for (int j = 0; j < nb; ++j) {
      const int f = idx[j];
      const double* Cj = C + 22 * j;
      const double cut2 = Cj[0] * Cj[0];
      double ax = 0, ay = 0, az = 0;
      cells.visit(pos + 3 * f, [&](int k) {
        if (k == f) return;
        const V3 d = diff(pos, f, k, box);
        V3 ab{0, 0, 0};
        V3 a2 = accv(acc, k);
        bead_force_fn(d, ab, a2, Cj, cut2);
        setv(acc, k, a2);
        ax += ab.x;
        ay += ab.y;
        az += ab.z;
      });
      acc[3 * f] += ax;
      acc[3 * f + 1] += ay;
      acc[3 * f + 2] += az;
    }
    return;
  }
  for (int j = 0; j < nb; ++j) {
    const int f = idx[j];
    const double* Cj = C + 22 * j;
    const double cutoffRad = Cj[0];
    const double cut2 = cutoffRad * cutoffRad;
    double ax = 0, ay = 0, az = 0;
    for (int k = 0; k < n; ++k) {
      if (k == f) continue;
      const V3 d = diff(pos, f, k, box);
      V3 ab{0, 0, 0};
      V3 a2 = accv(acc, k);
      bead_force_fn(d, ab, a2, Cj, cut2);
      setv(acc, k, a2);
      ax += ab.x;
      ay += ab.y;
      az += ab.z;
    }
    acc[3 * f] += ax;
    acc[3 * f + 1] += ay;
    acc[3 * f + 2] += az;
  }
}

// Each core's loop is an OpenMP reduction (include/system.h:3049): a private
// sum from zero, added to the total at its end.
double orc_nanocore_potential(int n, const double* pos, const double box[3], int nb, const int* idx,
                              const double* C) {
  double potential = 0;
  for (int j = 0; j < nb; ++j) {
    const int f = idx[j];
    const double* Cj = C + 22 * j;
    const double cutoffRad = Cj[0];
    const double cut2 = cutoffRad * cutoffRad;
    double part = 0;
    for (int k = 0; k < n; ++k) {
      if (k == f) continue;
      part += bead_potential_fn(diff(pos, f, k, box), Cj, cut2);
    }
    potential += part;
  }
  return potential;
}

}  // extern "C"
