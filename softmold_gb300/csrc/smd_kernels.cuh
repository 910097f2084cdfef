// Kernels of the GB300 membrane MD step.  See smd_device.cuh for the layout.
//
// One MD loop iteration (MD.cpp:335-729) in the steady state is
//   [k_bin, k_scan_*, k_reorder, k_nbr]   only when the Verlet list is stale
//   k_step<MIXED>                          forces + Langevin + both half-kicks + drift
// and on barostat steps
//   k_trial, k_step<STOP|DU>, k_mc, k_finish.
#pragma once

#include "smd_device.cuh"

namespace smd {

enum StepFlags {
  F_STOP = 1,       // store a and v+h*a (second half-kick) and stop before the drift
  F_DU = 2,         // accumulate U(x) - U(s*x) for the replica's trial scale
  F_EXTNOISE = 4,   // Langevin noise from P.ext_noise (file order)
  F_INIT = 8,       // start-up force: store a only, start-up noise phase
  F_FORCES = 16,    // conservative forces only, written to P.force_out (file order)
  F_PAIRONLY = 32,  // with F_FORCES: non-bonded part only
  F_ENERGY = 64     // energies only (pair, bonded, kinetic) into RepState
};

// ------------------------------------------------------------ last block
// Runs once per launch after every block has passed its atomics: folds this
// step's largest speed into the displacement bound and decides whether the
// Verlet list must be rebuilt before the next force pass.
__device__ __forceinline__ void finalize_step(const DevPtrs& P, float vmax_block, double dt, double half_skin,
                                              double mc_shift) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    if (vmax_block > 0.f) atomicMax(&P.g->vmax_bits, __float_as_uint(vmax_block));
    __threadfence();
    const unsigned int prev = atomicAdd(&P.g->blocks_done, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const float vmax = __uint_as_float(atomicExch(&P.g->vmax_bits, 0u));
    const unsigned long long sb = atomicExch(&P.g->mc_shift, 0ull);
    const double d = P.g->disp + (double)vmax * dt + __longlong_as_double((long long)sb);
    P.g->disp = d;
    P.g->rebuild = (d > half_skin) ? 1 : 0;
    P.g->blocks_done = 0u;
  }
  (void)mc_shift;
}

// ------------------------------------------------------------ list build
__device__ __forceinline__ void list_grid(const DevPtrs& P, int r, int n[3], double cs[3]) {
  const RepState& rs = P.rs[r];
  const double lc = P.tab->list_cut;
  for (int d = 0; d < 3; ++d) {
    n[d] = int(rs.box[d] / lc);
    n[d] = n[d] < 1 ? 1 : n[d];
  }
  const int cap = P.rp[r].cell_cap;
  while ((long long)n[0] * n[1] * n[2] > cap) {
    int m = 0;
    if (n[1] > n[m]) m = 1;
    if (n[2] > n[m]) m = 2;
    n[m]--;
  }
  for (int d = 0; d < 3; ++d) cs[d] = rs.box[d] / n[d];
}

__global__ void __launch_bounds__(kBlock) k_bin(DevPtrs P) {
  if (!P.g->rebuild) return;
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int r = rep_of(P, i);
  int n[3];
  double cs[3];
  list_grid(P, r, n, cs);
  const int cx = list_cell_coord(P.x[i], cs[0], n[0]);
  const int cy = list_cell_coord(P.y[i], cs[1], n[1]);
  const int cz = list_cell_coord(P.z[i], cs[2], n[2]);
  const int key = P.rp[r].cell_begin + cx + n[0] * (cy + n[1] * cz);
  P.key[i] = key;
  P.slot[i] = atomicAdd(&P.cell_count[key], 1);
  if (i == P.rp[r].bead_begin) {
    P.rs[r].ncell[0] = n[0];
    P.rs[r].ncell[1] = n[1];
    P.rs[r].ncell[2] = n[2];
  }
}

// Exclusive scan of cell_count into cell_start in three passes: tile sums,
// scan of the tile sums (one block), tile scans.
__global__ void __launch_bounds__(kBlock) k_scan_tiles(DevPtrs P) {
  if (!P.g->rebuild) return;
  const int base = blockIdx.x * kScanTile;
  int s = 0;
  for (int k = threadIdx.x; k < kScanTile; k += kBlock) {
    const int c = base + k;
    if (c < P.n_cells_total) s += P.cell_count[c];
  }
  __shared__ int sh[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kBlock / 32; ++w) t += sh[w];
    P.block_sums[blockIdx.x] = t;
  }
}

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
  // 256-thread exclusive scan through warp shuffles and shared memory.
  __shared__ int wsum[kBlock / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = (lane < kBlock / 32) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kBlock / 32) wsum[lane] = t;
  }
  __syncthreads();
  const int before = (w > 0 ? wsum[w - 1] : 0) + x - v;
  *total = wsum[kBlock / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kBlock) k_scan_sums(DevPtrs P, int n_tiles) {
  if (!P.g->rebuild) return;
  int carry = 0;
  for (int base = 0; base < n_tiles; base += kBlock) {
    const int t = base + threadIdx.x;
    const int v = (t < n_tiles) ? P.block_sums[t] : 0;
    int total;
    const int ex = block_exclusive_scan(v, &total);
    if (t < n_tiles) P.block_sums[t] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kBlock) k_scan_apply(DevPtrs P) {
  if (!P.g->rebuild) return;
  const int base = blockIdx.x * kScanTile;
  int carry = P.block_sums[blockIdx.x];
  for (int k = 0; k < kScanTile; k += kBlock) {
    const int c = base + k + threadIdx.x;
    const int v = (c < P.n_cells_total) ? P.cell_count[c] : 0;
    int total;
    const int ex = block_exclusive_scan(v, &total);
    if (c < P.n_cells_total) P.cell_start[c] = carry + ex;
    carry += total;
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) P.cell_start[P.n_cells_total] = P.n;
}

template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_reorder(DevPtrs P, int cur) {
  if (!P.g->rebuild) return;
  const int i = blockIdx.x * kBlock + threadIdx.x;
  for (int c = i; c < P.n_cells_total; c += gridDim.x * kBlock) P.cell_count[c] = 0;
  if (i >= P.n) return;
  const int nw = P.cell_start[P.key[i]] + P.slot[i];
  const double x = P.x[i], y = P.y[i], z = P.z[i];
  P.tx[nw] = x;
  P.ty[nw] = y;
  P.tz[nw] = z;
  P.tvx[nw] = P.vx[i];
  P.tvy[nw] = P.vy[i];
  P.tvz[nw] = P.vz[i];
  P.tax[nw] = P.ax[i];
  P.tay[nw] = P.ay[i];
  P.taz[nw] = P.az[i];
  const int o = P.orig[i];
  P.torig[nw] = o;
  P.tcinfo[nw] = P.cinfo[i];
  P.inv[o] = nw;
  const int r = rep_of(P, i);
  if constexpr (MIXED) {
    const RepState& rs = P.rs[r];
    const uint4 old = P.m4[cur][i];
    P.mt[nw] = make_uint4(to_frac(x, 1.0 / rs.box[0]), to_frac(y, 1.0 / rs.box[1]), to_frac(z, 1.0 / rs.box[2]),
                          old.w);
  } else {
    const double4 old = P.d4[cur][i];
    P.dt4[nw] = make_double4(x, y, z, old.w);
  }
}

// Copies the reordered state back and builds the Verlet list of bead i from
// the 27 (or fewer, for thin boxes) surrounding cells, reading the reordered
// mirror that k_reorder left in the scratch buffer.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_nbr(DevPtrs P, int cur) {
  if (!P.g->rebuild) return;
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.g->disp = 0.0;
    P.g->n_rebuilds++;
  }
  if (i >= P.n) return;
  P.x[i] = P.tx[i];
  P.y[i] = P.ty[i];
  P.z[i] = P.tz[i];
  P.vx[i] = P.tvx[i];
  P.vy[i] = P.tvy[i];
  P.vz[i] = P.tvz[i];
  P.ax[i] = P.tax[i];
  P.ay[i] = P.tay[i];
  P.az[i] = P.taz[i];
  P.orig[i] = P.torig[i];
  P.cinfo[i] = P.tcinfo[i];
  if constexpr (MIXED) P.m4[cur][i] = P.mt[i]; else P.d4[cur][i] = P.dt4[i];
  const int r = rep_of(P, i);
  const RepState& rs = P.rs[r];
  const int n0 = rs.ncell[0], n1 = rs.ncell[1], n2 = rs.ncell[2];
  const int cb = P.rp[r].cell_begin;
  double cs[3] = {rs.box[0] / n0, rs.box[1] / n1, rs.box[2] / n2};
  const double xi = P.tx[i], yi = P.ty[i], zi = P.tz[i];
  const int cx = list_cell_coord(xi, cs[0], n0), cy = list_cell_coord(yi, cs[1], n1),
            cz = list_cell_coord(zi, cs[2], n2);
  const double lc2 = P.tab->list_cut2;
  int cnt = 0;
  const int kmax = P.kmax;
  int* out = P.nbr + i;
  const int lo0 = n0 >= 3 ? -1 : 0, hi0 = n0 >= 2 ? 1 : 0;
  const int lo1 = n1 >= 3 ? -1 : 0, hi1 = n1 >= 2 ? 1 : 0;
  const int lo2 = n2 >= 3 ? -1 : 0, hi2 = n2 >= 2 ? 1 : 0;
  uint4 mi;
  double4 di;
  double sc[3];
  if constexpr (MIXED) {
    mi = P.mt[i];
    for (int d = 0; d < 3; ++d) sc[d] = rs.box[d] * (1.0 / 4294967296.0);
  } else {
    di = P.dt4[i];
  }
  for (int oz = lo2; oz <= hi2; ++oz) {
    const int zz = (cz + oz + n2) % n2;
    for (int oy = lo1; oy <= hi1; ++oy) {
      const int yy = (cy + oy + n1) % n1;
      for (int ox = lo0; ox <= hi0; ++ox) {
        const int xx = (cx + ox + n0) % n0;
        const int c = cb + xx + n0 * (yy + n1 * zz);
        const int s = P.cell_start[c], e = P.cell_start[c + 1];
        for (int j = s; j < e; ++j) {
          if (j == i) continue;
          double d2;
          if constexpr (MIXED) {
            const uint4 mj = P.mt[j];
            const double dx = frac_delta_d(mi.x, mj.x, sc[0]), dy = frac_delta_d(mi.y, mj.y, sc[1]),
                         dz = frac_delta_d(mi.z, mj.z, sc[2]);
            d2 = dx * dx + dy * dy + dz * dz;
          } else {
            const double4 dj = P.dt4[j];
            double dx = di.x - dj.x, dy = di.y - dj.y, dz = di.z - dj.z;
            dx -= rs.box[0] * rint(dx / rs.box[0]);
            dy -= rs.box[1] * rint(dy / rs.box[1]);
            dz -= rs.box[2] * rint(dz / rs.box[2]);
            d2 = dx * dx + dy * dy + dz * dz;
          }
          if (d2 < lc2) {
            if (cnt < kmax) out[(size_t)cnt * P.npad] = j;
            ++cnt;
          }
        }
      }
    }
  }
  P.nnbr[i] = cnt < kmax ? cnt : kmax;
  if (cnt > kmax) {
    atomicOr(&P.g->error, 1);
    atomicMax(&P.g->need_nbr, cnt);
  }
}

// ------------------------------------------------------------ the step
// Per-bead CHAIN terms.  The bead at chain position p takes its share of the
// bonds (p-1,p), (p,p+1) and of the bends (p-2,p-1,p), (p-1,p,p+1),
// (p,p+1,p+2), with the formulas of harmonicF and bendF (include/MD.h:384-403,
// 683-723) and the minimum image of include/system.h:1806-1832.
template <typename R>
struct Vec3 {
  R x, y, z;
};

template <typename R>
__device__ __forceinline__ void bond_term(Vec3<R> d, const R* c, R sign, Vec3<R>& f) {
  const R dr = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
  R mag = dr - c[0];
  mag = -mag * c[1] / dr;
  f.x += sign * d.x * mag;
  f.y += sign * d.y * mag;
  f.z += sign * d.z * mag;
}

// role: 0 first (gets bufa), 1 second (bufb - bufa), 2 third (-bufb)
template <typename R>
__device__ __forceinline__ void bend_term(Vec3<R> da, Vec3<R> db, const R* c, int role, Vec3<R>& f) {
  const R dra = sqrt(da.x * da.x + da.y * da.y + da.z * da.z);
  const R drb = sqrt(db.x * db.x + db.y * db.y + db.z * db.z);
  da.x /= dra;
  da.y /= dra;
  da.z /= dra;
  db.x /= drb;
  db.y /= drb;
  db.z /= drb;
  const R cs = (da.x * db.x) + (da.y * db.y) + (da.z * db.z);
  const R mag = (c[0] - cs) * c[1];
  const R ta = mag / dra, tb = mag / drb;
  const R ax = ta * (db.x - da.x * cs), ay = ta * (db.y - da.y * cs), az = ta * (db.z - da.z * cs);
  const R bx = tb * (da.x - db.x * cs), by = tb * (da.y - db.y * cs), bz = tb * (da.z - db.z * cs);
  if (role == 0) {
    f.x += ax;
    f.y += ay;
    f.z += az;
  } else if (role == 1) {
    f.x += bx - ax;
    f.y += by - ay;
    f.z += bz - az;
  } else {
    f.x -= bx;
    f.y -= by;
    f.z -= bz;
  }
}

__device__ __forceinline__ double bond_pot(Vec3<double> d, const double* c) {
  const double dr = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
  const double p = dr - c[0];
  return 0.5 * c[1] * p * p;
}
__device__ __forceinline__ double bend_pot(Vec3<double> da, Vec3<double> db, const double* c) {
  const double dra = sqrt(da.x * da.x + da.y * da.y + da.z * da.z);
  const double drb = sqrt(db.x * db.x + db.y * db.y + db.z * db.z);
  const double cs = (da.x * db.x + da.y * db.y + da.z * db.z) / (dra * drb);
  const double p = c[0] - cs;
  return c[1] * p * p * 0.5;
}

// Difference vectors e[k] = x(p-2+k) - x(p-1+k), k = 0..3, of the chain
// around bead i, as real-space vectors of type R; valid[k] marks existing ones.
template <bool MIXED, typename R>
__device__ __forceinline__ void chain_vectors(const DevPtrs& P, int cur, int i, int p, int len, const double box[3],
                                              Vec3<R> e[4], bool valid[4]) {
  const int o = P.orig[i];
  int idx[5];
  bool have[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int q = p - 2 + k;
    have[k] = (q >= 0 && q < len);
    idx[k] = (k == 2) ? i : (have[k] ? P.inv[o - 2 + k] : i);
  }
  if constexpr (MIXED) {
    uint4 m[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) m[k] = P.m4[cur][idx[k]];
    const double s0 = box[0] * (1.0 / 4294967296.0), s1 = box[1] * (1.0 / 4294967296.0),
                 s2 = box[2] * (1.0 / 4294967296.0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      valid[k] = have[k] && have[k + 1];
      e[k].x = (R)frac_delta_d(m[k].x, m[k + 1].x, s0);
      e[k].y = (R)frac_delta_d(m[k].y, m[k + 1].y, s1);
      e[k].z = (R)frac_delta_d(m[k].z, m[k + 1].z, s2);
    }
  } else {
    double4 m[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) m[k] = P.d4[cur][idx[k]];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      valid[k] = have[k] && have[k + 1];
      double d[3] = {m[k].x - m[k + 1].x, m[k].y - m[k + 1].y, m[k].z - m[k + 1].z};
      for (int a = 0; a < 3; ++a) {
        if (d[a] > box[a] / 2.0) d[a] -= box[a];
        if (d[a] < -box[a] / 2.0) d[a] += box[a];
      }
      e[k].x = (R)d[0];
      e[k].y = (R)d[1];
      e[k].z = (R)d[2];
    }
  }
}

// Sum of v over the lanes that belong to the same replica, one atomic per
// replica present in the warp.  Called by the whole warp.
__device__ __forceinline__ void warp_atomic_add(double v, double* dst, int r) {
  const unsigned int peers = __match_any_sync(0xffffffffu, r);
  const int lane = threadIdx.x & 31;
  double acc = 0.0;
  for (unsigned int rest = peers; rest; rest &= rest - 1) acc += __shfl_sync(peers, v, __ffs(rest) - 1);
  if (lane == __ffs(peers) - 1 && acc != 0.0) atomicAdd(dst, acc);
}

// The fused step.  One thread per bead (sorted order).
template <bool MIXED, int FL>
__global__ void __launch_bounds__(kBlock) k_step(DevPtrs P, int cur, long long it) {
  using R = typename std::conditional<MIXED, float, double>::type;
  __shared__ R sF[6 * kMaxTypes * kMaxTypes];
  __shared__ R sU[6 * kMaxTypes * kMaxTypes];
  const Tables& T = *P.tab;
  const int nT = T.nT;
  for (int k = threadIdx.x; k < 6 * nT * nT; k += kBlock) {
    if constexpr (MIXED) {
      sF[k] = T.fF[k];
      sU[k] = T.fU[k];
    } else {
      sF[k] = T.dF[k];
      sU[k] = T.dU[k];
    }
  }
  __syncthreads();
  const int i = blockIdx.x * kBlock + threadIdx.x;
  const bool active = i < P.n;
  const int r = active ? rep_of(P, i) : 0;
  double dU_pair = 0.0, dU_bond = 0.0, e_pair = 0.0, e_bond = 0.0, e_kin = 0.0;
  float vmax = 0.f;
  if (active) {
    const RepParams& rp = P.rp[r];
    RepState& rs = P.rs[r];
    const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
    // ---- non-bonded, from the Verlet list
    long long qx = 0, qy = 0, qz = 0;  // MIXED: fixed point
    double fxd = 0, fyd = 0, fzd = 0;  // PLAIN
    int ti;
    R sq[3];  // (s_d^2 - 1) for the size-change difference
    if constexpr ((FL & F_DU) != 0) {
      for (int d = 0; d < 3; ++d) sq[d] = (R)(rs.scale[d] * rs.scale[d] - 1.0);
    }
    const int nn = P.nnbr[i];
    const int* nb = P.nbr + i;
    if constexpr (MIXED) {
      const uint4 me = P.m4[cur][i];
      ti = me.w & 0xff;
      const float s0 = (float)(box[0] * (1.0 / 4294967296.0)), s1 = (float)(box[1] * (1.0 / 4294967296.0)),
                  s2 = (float)(box[2] * (1.0 / 4294967296.0));
      const float* rowF = sF + 6 * ti * nT;
      const float* rowU = sU + 6 * ti * nT;
      const float rc2 = T.rc2f, fs = T.fscale;
      float eacc = 0.f;
      for (int k = 0; k < nn; ++k) {
        const int j = __ldg(nb + (size_t)k * P.npad);
        const uint4 o = P.m4[cur][j];
        const float dx = frac_delta(me.x, o.x, s0), dy = frac_delta(me.y, o.y, s1), dz = frac_delta(me.z, o.z, s2);
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < rc2) {
          const int tj = o.w & 0xff;
          const float rr = sqrtf(r2);
          if constexpr ((FL & F_ENERGY) == 0) {
            const float mag = pair_mag<float>(rowF + 6 * tj, rr) * fs;
            qx += (long long)__float2int_rn(dx * mag);
            qy += (long long)__float2int_rn(dy * mag);
            qz += (long long)__float2int_rn(dz * mag);
          } else {
            eacc += pair_pot<float>(rowU + 6 * tj, rr);
          }
          if constexpr ((FL & F_DU) != 0) {
            const float q = sq[0] * dx * dx + sq[1] * dy * dy + sq[2] * dz * dz;
            const float rn = sqrtf(r2 + q);
            dU_pair += 0.5 * (double)pair_dpot_f(rowU + 6 * tj, rr, rn, q / (rn + rr), T.rcf);
          }
        } else if constexpr ((FL & F_DU) != 0) {
          // pairs just outside rc can move inside under the trial scale
          const float q = sq[0] * dx * dx + sq[1] * dy * dy + sq[2] * dz * dz;
          const float rn2 = r2 + q;
          if (rn2 < rc2) {
            const int tj = o.w & 0xff;
            dU_pair -= 0.5 * (double)pair_pot<float>(rowU + 6 * tj, sqrtf(rn2));
          }
        }
      }
      e_pair = 0.5 * (double)eacc;
    } else {
      const double4 me = P.d4[cur][i];
      ti = __double_as_longlong(me.w) & 0xff;
      const double* rowF = sF + 6 * ti * nT;
      const double* rowU = sU + 6 * ti * nT;
      const double rc2 = T.rc2;
      for (int k = 0; k < nn; ++k) {
        const int j = __ldg(nb + (size_t)k * P.npad);
        const double4 o = P.d4[cur][j];
        // minimum image applied to the neighbour first, as CellOpt shifts the
        // neighbour cell's positions (cellOpt.h:810-840)
        double ox = o.x, oy = o.y, oz = o.z;
        if (me.x - ox > box[0] / 2.0) ox += box[0];
        if (me.x - ox < -box[0] / 2.0) ox -= box[0];
        if (me.y - oy > box[1] / 2.0) oy += box[1];
        if (me.y - oy < -box[1] / 2.0) oy -= box[1];
        if (me.z - oz > box[2] / 2.0) oz += box[2];
        if (me.z - oz < -box[2] / 2.0) oz -= box[2];
        const double dx = me.x - ox, dy = me.y - oy, dz = me.z - oz;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const int tj = __double_as_longlong(o.w) & 0xff;
        if (r2 < rc2) {
          const double rr = sqrt(r2);
          if constexpr ((FL & F_ENERGY) == 0) {
            const double mag = pair_mag<double>(rowF + 6 * tj, rr);
            fxd += dx * mag;
            fyd += dy * mag;
            fzd += dz * mag;
          } else {
            e_pair += 0.5 * pair_pot<double>(rowU + 6 * tj, rr);
          }
        }
        if constexpr ((FL & F_DU) != 0) {
          const double nx = dx * rs.scale[0], ny = dy * rs.scale[1], nz = dz * rs.scale[2];
          const double rn2 = nx * nx + ny * ny + nz * nz;
          const double u0 = r2 < rc2 ? pair_pot<double>(rowU + 6 * tj, sqrt(r2)) : 0.0;
          const double u1 = rn2 < rc2 ? pair_pot<double>(rowU + 6 * tj, sqrt(rn2)) : 0.0;
          dU_pair += 0.5 * (u0 - u1);
        }
      }
    }
    // ---- CHAIN terms
    Vec3<R> fb{0, 0, 0};
    const int ci = P.cinfo[i];
    if ((FL & F_PAIRONLY) == 0 && ci < 0 && !(ci & 0x40000000)) {
      const int p = ci & 0xfff, len = (ci >> 12) & 0xfff, set = (ci >> 24) & 0x1f;
      Vec3<R> e[4];
      bool valid[4];
      chain_vectors<MIXED, R>(P, cur, i, p, len, box, e, valid);
      const R* cf;
      if constexpr (MIXED) cf = T.chainF[set]; else cf = T.chainD[set];
      if constexpr ((FL & F_ENERGY) == 0) {
        if (valid[1]) bond_term<R>(e[1], cf, (R)-1, fb);          // bond (p-1,p): second
        if (valid[2]) bond_term<R>(e[2], cf, (R)1, fb);           // bond (p,p+1): first
        if (valid[0] && valid[1]) bend_term<R>(e[0], e[1], cf + 2, 2, fb);
        if (valid[1] && valid[2]) bend_term<R>(e[1], e[2], cf + 2, 1, fb);
        if (valid[2] && valid[3]) bend_term<R>(e[2], e[3], cf + 2, 0, fb);
      }
      if constexpr ((FL & (F_DU | F_ENERGY)) != 0) {
        // energy terms owned by the first bead of each bond / bend, in FP64
        Vec3<double> a2{(double)e[2].x, (double)e[2].y, (double)e[2].z};
        Vec3<double> a3{(double)e[3].x, (double)e[3].y, (double)e[3].z};
        const double* cd = T.chainD[set];
        if constexpr ((FL & F_ENERGY) != 0) {
          if (valid[2]) e_bond += bond_pot(a2, cd);
          if (valid[2] && valid[3]) e_bond += bend_pot(a2, a3, cd + 2);
        }
        if constexpr ((FL & F_DU) != 0) {
          const Vec3<double> s2{a2.x * rs.scale[0], a2.y * rs.scale[1], a2.z * rs.scale[2]};
          const Vec3<double> s3{a3.x * rs.scale[0], a3.y * rs.scale[1], a3.z * rs.scale[2]};
          if (valid[2]) dU_bond += bond_pot(a2, cd) - bond_pot(s2, cd);
          if (valid[2] && valid[3]) dU_bond += bend_pot(a2, a3, cd + 2) - bend_pot(s2, s3, cd + 2);
        }
      }
    }
    // ---- total conservative force
    double F[3];
    if constexpr (MIXED) {
      const float fs = T.fscale;
      qx += __float2ll_rn(fb.x * fs);
      qy += __float2ll_rn(fb.y * fs);
      qz += __float2ll_rn(fb.z * fs);
      F[0] = (double)qx * T.inv_fscale;
      F[1] = (double)qy * T.inv_fscale;
      F[2] = (double)qz * T.inv_fscale;
    } else {
      F[0] = fxd + fb.x;
      F[1] = fyd + fb.y;
      F[2] = fzd + fb.z;
    }
    if constexpr ((FL & F_FORCES) != 0) {
      const int o = P.orig[i];
      P.force_out[3 * o] = F[0];
      P.force_out[3 * o + 1] = F[1];
      P.force_out[3 * o + 2] = F[2];
    } else if constexpr ((FL & F_ENERGY) != 0) {
      const double vx = P.vx[i], vy = P.vy[i], vz = P.vz[i];
      e_kin = (vx * vx + vy * vy + vz * vz) / 2.0;
    } else {
      // ---- Langevin (include/algorithms/langevin.h:284-331) and Verlet
      const int o = P.orig[i];
      double psi[3];
      if constexpr ((FL & F_EXTNOISE) != 0) {
        psi[0] = P.ext_noise[3 * o];
        psi[1] = P.ext_noise[3 * o + 1];
        psi[2] = P.ext_noise[3 * o + 2];
      } else {
        langevin_noise(rp.seed, r, o - rp.bead_begin, it, (FL & F_INIT) ? 1 : 0, psi);
      }
      double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
      double a[3];
      for (int d = 0; d < 3; ++d) a[d] = F[d] + (-rp.gamma * v[d] + rp.sigma * psi[d]);
      const bool sphere = (ci < 0) && (ci & 0x40000000);
      if constexpr ((FL & (F_STOP | F_INIT)) != 0) {
        P.ax[i] = a[0];
        P.ay[i] = a[1];
        P.az[i] = a[2];
        if constexpr ((FL & F_STOP) != 0) {
          if (ti != 0 && !sphere) {
            const double h = rp.dt * 0.5;
            P.vx[i] = v[0] + a[0] * h;
            P.vy[i] = v[1] + a[1] * h;
            P.vz[i] = v[2] + a[2] * h;
          }
        }
      } else if (!sphere) {
        double x[3] = {P.x[i], P.y[i], P.z[i]};
        if (ti != 0) {
          const double h = rp.dt * 0.5;
          for (int d = 0; d < 3; ++d) {
            v[d] += (a[d] * h);  // second() of this step
            v[d] += (a[d] * h);  // first() of the next step
            x[d] += v[d] * rp.dt;
            if (x[d] > box[d]) x[d] -= box[d];
            if (x[d] < 0) x[d] += box[d];
          }
          P.vx[i] = v[0];
          P.vy[i] = v[1];
          P.vz[i] = v[2];
          P.x[i] = x[0];
          P.y[i] = x[1];
          P.z[i] = x[2];
          vmax = (float)sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        }
        if constexpr (MIXED) {
          const uint4 me = P.m4[cur][i];
          P.m4[cur ^ 1][i] = make_uint4(to_frac(x[0], 1.0 / box[0]), to_frac(x[1], 1.0 / box[1]),
                                        to_frac(x[2], 1.0 / box[2]), me.w);
        } else {
          const double4 me = P.d4[cur][i];
          P.d4[cur ^ 1][i] = make_double4(x[0], x[1], x[2], me.w);
        }
      } else {
        P.ax[i] = a[0];
        P.ay[i] = a[1];
        P.az[i] = a[2];
      }
    }
  }
  // ---- reductions
  if constexpr ((FL & F_DU) != 0) {
    warp_atomic_add(dU_pair, &P.rs[r].dU_pair, r);
    warp_atomic_add(dU_bond, &P.rs[r].dU_bond, r);
  }
  if constexpr ((FL & F_ENERGY) != 0) {
    warp_atomic_add(e_pair, &P.rs[r].e_pair, r);
    warp_atomic_add(e_bond, &P.rs[r].e_bond, r);
    warp_atomic_add(e_kin, &P.rs[r].e_kin, r);
  }
  if constexpr ((FL & (F_STOP | F_INIT | F_FORCES | F_ENERGY)) == 0) {
    vmax = warp_max(vmax);
    __shared__ float smax[kBlock / 32];
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = vmax;
    __syncthreads();
    float bm = 0.f;
    if (threadIdx.x == 0)
      for (int w = 0; w < kBlock / 32; ++w) bm = fmaxf(bm, smax[w]);
    finalize_step(P, bm, P.rp[0].dt, P.half_skin, 0.0);
  }
}

// Barostat trial box for every replica (MD.cpp:593-611).
__global__ void k_trial(DevPtrs P, int trial) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rep) return;
  RepState& rs = P.rs[r];
  rs.dU_pair = 0.0;
  rs.dU_bond = 0.0;
  if (P.rp[r].dlxy == 0) {
    for (int d = 0; d < 3; ++d) rs.scale[d] = 1.0;
    return;
  }
  const double u1 = P.trial_u[((size_t)trial * P.n_rep + r) * 2];
  double nb[3], s[3];
  trial_box(rs.box, P.rp[r].dlxy, u1, nb, s);
  for (int d = 0; d < 3; ++d) {
    rs.trial_box[d] = nb[d];
    rs.scale[d] = s[d];
  }
  rs.dU_pair = 0.0;
  rs.dU_bond = 0.0;
}

// Metropolis decision (MD.cpp:677-720).
__global__ void k_mc(DevPtrs P, int trial) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rep) return;
  RepState& rs = P.rs[r];
  const RepParams& rp = P.rp[r];
  rs.accept = 0;
  if (rp.dlxy == 0) return;
  double dPot = rs.dU_pair + rs.dU_bond;
  if (rp.tension != 0) dPot += rp.tension * ((rs.trial_box[0] * rs.trial_box[1]) - (rs.box[0] * rs.box[1]));
  const double D = exp(dPot / rp.kT);
  const double u2 = P.trial_u[((size_t)trial * P.n_rep + r) * 2 + 1];
  rs.last_dU = dPot;
  rs.n_trial++;
  if (D >= u2 || -dPot <= 0) {
    double shift = 0.0;
    for (int d = 0; d < 3; ++d) {
      shift = fmax(shift, fabs(rs.scale[d] - 1.0) * rs.box[d]);
      rs.box[d] = rs.trial_box[d];
    }
    rs.accept = 1;
    rs.n_accept++;
    P.accept_log[(size_t)trial * P.n_rep + r] = 1;
    atomicMax((unsigned long long*)&P.g->mc_shift, (unsigned long long)__double_as_longlong(shift));
  } else {
    rs.accept = 0;
    P.accept_log[(size_t)trial * P.n_rep + r] = 0;
  }
}

// Completes a stopped step: optional restart half-kick, optional box rescale
// of an accepted MC move, then the next step's first half-kick and drift.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_finish(DevPtrs P, int cur, int do_second, int apply_mc) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  float vmax = 0.f;
  if (i < P.n) {
    const int r = rep_of(P, i);
    const RepParams& rp = P.rp[r];
    const RepState& rs = P.rs[r];
    const int ci = P.cinfo[i];
    const bool sphere = (ci < 0) && (ci & 0x40000000);
    if (!sphere) {
      int ti;
      if constexpr (MIXED) ti = P.m4[cur][i].w & 0xff; else ti = __double_as_longlong(P.d4[cur][i].w) & 0xff;
      double x[3] = {P.x[i], P.y[i], P.z[i]};
      if (apply_mc && rs.accept)
        for (int d = 0; d < 3; ++d) x[d] *= rs.scale[d];
      if (ti != 0) {
        const double h = rp.dt * 0.5;
        const double a[3] = {P.ax[i], P.ay[i], P.az[i]};
        double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
        for (int d = 0; d < 3; ++d) {
          if (do_second) v[d] += (a[d] * h);
          v[d] += (a[d] * h);
          x[d] += v[d] * rp.dt;
          if (x[d] > rs.box[d]) x[d] -= rs.box[d];
          if (x[d] < 0) x[d] += rs.box[d];
        }
        P.vx[i] = v[0];
        P.vy[i] = v[1];
        P.vz[i] = v[2];
        vmax = (float)sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      }
      P.x[i] = x[0];
      P.y[i] = x[1];
      P.z[i] = x[2];
      if constexpr (MIXED) {
        const uint4 me = P.m4[cur][i];
        P.m4[cur ^ 1][i] = make_uint4(to_frac(x[0], 1.0 / rs.box[0]), to_frac(x[1], 1.0 / rs.box[1]),
                                      to_frac(x[2], 1.0 / rs.box[2]), me.w);
      } else {
        const double4 me = P.d4[cur][i];
        P.d4[cur ^ 1][i] = make_double4(x[0], x[1], x[2], me.w);
      }
    }
  }
  vmax = warp_max(vmax);
  __shared__ float smax[kBlock / 32];
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = vmax;
  __syncthreads();
  float bm = 0.f;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlock / 32; ++w) bm = fmaxf(bm, smax[w]);
  finalize_step(P, bm, P.rp[0].dt, P.half_skin, 0.0);
}

// Mirror of the current positions in the other buffer (after set_state or a
// box change made on the host).
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_mirror(DevPtrs P, int cur) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int r = rep_of(P, i);
  const RepState& rs = P.rs[r];
  if constexpr (MIXED) {
    const uint4 me = P.m4[cur][i];
    P.m4[cur][i] = make_uint4(to_frac(P.x[i], 1.0 / rs.box[0]), to_frac(P.y[i], 1.0 / rs.box[1]),
                              to_frac(P.z[i], 1.0 / rs.box[2]), me.w);
  } else {
    const double4 me = P.d4[cur][i];
    P.d4[cur][i] = make_double4(P.x[i], P.y[i], P.z[i], me.w);
  }
}

// CellOpt keys on the reference grid nCells = int(L/rc), file order.
__global__ void __launch_bounds__(kBlock) k_ref_keys(DevPtrs P) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int r = rep_of(P, i);
  const RepState& rs = P.rs[r];
  const double rc = P.tab->rc;
  int n[3];
  double cs[3];
  for (int d = 0; d < 3; ++d) {
    n[d] = int(rs.box[d] / rc);
    cs[d] = rs.box[d] / n[d];
  }
  const int cx = cell_coord(P.x[i], cs[0], n[0]);
  const int cy = cell_coord(P.y[i], cs[1], n[1]);
  const int cz = cell_coord(P.z[i], cs[2], n[2]);
  P.key_out[P.orig[i]] = cx + cy * n[0] + cz * n[0] * n[1];
}

// Pairs (file order, i<j) within rc from the Verlet list, distances in FP64
// with the neighbour-shift minimum image of CellOpt.
__global__ void __launch_bounds__(kBlock) k_pairs(DevPtrs P, int* out, long long cap, unsigned long long* count) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int r = rep_of(P, i);
  const RepState& rs = P.rs[r];
  const double* box = rs.box;
  const double xi = P.x[i], yi = P.y[i], zi = P.z[i];
  const int oi = P.orig[i];
  for (int k = 0; k < P.nnbr[i]; ++k) {
    const int j = P.nbr[(size_t)k * P.npad + i];
    const int oj = P.orig[j];
    if (oi >= oj) continue;
    double ox = P.x[j], oy = P.y[j], oz = P.z[j];
    if (xi - ox > box[0] / 2.0) ox += box[0];
    if (xi - ox < -box[0] / 2.0) ox -= box[0];
    if (yi - oy > box[1] / 2.0) oy += box[1];
    if (yi - oy < -box[1] / 2.0) oy -= box[1];
    if (zi - oz > box[2] / 2.0) oz += box[2];
    if (zi - oz < -box[2] / 2.0) oz -= box[2];
    const double dx = xi - ox, dy = yi - oy, dz = zi - oz;
    if (dx * dx + dy * dy + dz * dz < P.tab->rc2) {
      const unsigned long long slot = atomicAdd(count, 1ull);
      if ((long long)slot < cap) {
        out[2 * slot] = oi;
        out[2 * slot + 1] = oj;
      }
    }
  }
}

}  // namespace smd
