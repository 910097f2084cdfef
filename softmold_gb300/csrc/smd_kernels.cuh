// Kernels of the GB300 membrane MD step.  See smd_device.cuh for the layout.
//
// One MD loop iteration (MD.cpp:335-729) in the steady state is
//   [k_bin, k_scan_*, k_reorder, k_nbr]   only when the Verlet list is stale
//   k_force<MIXED>                         non-bonded forces, G lanes per bead
//   k_integ<MIXED>                         CHAIN + Langevin + both half-kicks + drift
// and on barostat steps
//   k_ref_cells (with the trial), k_force<DU>, k_integ<STOP|DU>, k_mc, k_finish.
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
  F_ENERGY = 64,    // energies only (pair, bonded, kinetic) into RepState
  F_FIELDS = 128    // the system has external-field terms (their out-of-line
                    // evaluation is compiled in only with this flag)
};

// ------------------------------------------------------------ last block
// Runs once per launch after every block has passed its atomics.  The list
// stays valid while every bead is within half the skin of its build position
// (a pair now inside rc was then inside rc + skin); accepted box moves use up
// (rc + skin)|s - 1| of that margin each.  Decides whether the Verlet list
// must be rebuilt before the next force pass.
__device__ __forceinline__ void finalize_step(const DevPtrs& P, float dmax_block, StepEnd se) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    if (dmax_block > 0.f) atomicMax(&P.g->dmax_bits, __float_as_uint(dmax_block));
    __threadfence();
    const unsigned int prev = atomicAdd(&P.g->blocks_done, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const float dmax = __uint_as_float(atomicExch(&P.g->dmax_bits, 0u));
    const unsigned long long sb = atomicExch(&P.g->mc_shift, 0ull);
    const double slack = P.g->slack + __longlong_as_double((long long)sb);
    P.g->slack = slack;
    P.g->last_disp = dmax;
    const int rebuild = ((double)dmax + slack > P.half_skin) ? 1 : 0;
    P.g->rebuild = rebuild;
    if (se.advance_it) P.g->it++;
    if (se.advance_slot) P.g->trial_slot++;
    P.g->blocks_done = 0u;
    if (se.set_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)se.cond, (unsigned int)rebuild);
  }
}

// Displacement of bead i from its build position, from 32-bit fractional
// coordinates (unchanged by box rescaling), in units of the current box.
__device__ __forceinline__ float displacement(uint4 ref, unsigned int fx, unsigned int fy, unsigned int fz,
                                              const RepState& rs) {
  const float dx = frac_delta(fx, ref.x, rs.len_per_frac[0]);
  const float dy = frac_delta(fy, ref.y, rs.len_per_frac[1]);
  const float dz = frac_delta(fz, ref.z, rs.len_per_frac[2]);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// ------------------------------------------------------------ list build
// Verlet-list cell of bead i from its 32-bit fractional coordinates: the
// cell index along an axis is floor(f * n / 2^32), always in [0, n).  The
// beads are in the previous build's cell order, so the lanes of a warp mostly
// share a few cells: the lanes of one cell take their slots from one atomic
// add of the leader (the lowest lane), in lane order.
__global__ void __launch_bounds__(kBeadBlock) k_bin(DevPtrs P, int cur, int mixed, int in_graph) {
  pdl_trigger();
  if (!P.g->rebuild) return;
  const int i = blockIdx.x * kBeadBlock + threadIdx.x;
  if (in_graph && i == 0) P.g->graph_builds++;
  const bool active = i < P.n;
  const unsigned int lanes = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const int r = rep_of(P, i);
  const RepState& rs = P.rs[r];
  unsigned int f[3];
  if (mixed) {
    const uint4 m = P.m4[cur][i];
    f[0] = m.x;
    f[1] = m.y;
    f[2] = m.z;
  } else {
    f[0] = to_frac(P.x[i], rs.frac_per_len[0]);
    f[1] = to_frac(P.y[i], rs.frac_per_len[1]);
    f[2] = to_frac(P.z[i], rs.frac_per_len[2]);
  }
  const int n0 = rs.ncell[0], n1 = rs.ncell[1], n2 = rs.ncell[2];
  const int cx = __umulhi(f[0], (unsigned)n0), cy = __umulhi(f[1], (unsigned)n1), cz = __umulhi(f[2], (unsigned)n2);
  const int key = P.rp[r].cell_begin + cx + n0 * (cy + n1 * cz);
  P.key[i] = key;
  const unsigned int same = __match_any_sync(lanes, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(same) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&P.cell_count[key], __popc(same));
  base = __shfl_sync(same, base, leader);
  P.slot[i] = base + __popc(same & ((1u << lane) - 1u));
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
  if (threadIdx.x == 0) {  // k_scan_apply appends the occupied cells
    P.g->n_occ = 0;
    P.g->next_cell = 0;
  }
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
  pdl_trigger();
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
    // occupied cells, appended one warp at a time (their order is free: each
    // cell's list does not depend on when it is built)
    const unsigned int occ = __ballot_sync(0xffffffffu, v > 0);
    if (occ) {
      const int lane = threadIdx.x & 31;
      int at = 0;
      if (lane == 0) at = atomicAdd(&P.g->n_occ, __popc(occ));
      at = __shfl_sync(0xffffffffu, at, 0);
      if (v > 0) P.occ[at + __popc(occ & ((1u << lane) - 1u))] = c;
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) P.cell_start[P.n_cells_total] = P.n;
}

// The same exclusive scan in one CTA for up to kScanOneMax cells (a single
// system's grid): each of 1024 threads sums 8 consecutive counts, the block
// scans the thread sums, and each thread writes its 8 starts.
constexpr int kScanOneThreads = 1024;
constexpr int kScanOneMax = 32768;
__global__ void __launch_bounds__(kScanOneThreads) k_scan_one(DevPtrs P) {
  pdl_trigger();
  pdl_wait();  // k_bin's counts
  if (!P.g->rebuild) return;
  __shared__ int wsum[kScanOneThreads / 32], osum[kScanOneThreads / 32];
  const int n = P.n_cells_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int carry = 0, ocarry = 0;  // beads and occupied cells before the chunk
  for (int base = 0; base < n; base += kScanOneThreads * 8) {
    const int c0 = base + threadIdx.x * 8;
    int v[8];
    int s = 0, f = 0;
    if (c0 + 8 <= n) {  // two 16-byte loads (the arrays are 16-byte aligned and c0 % 8 == 0)
      const int4 a = *reinterpret_cast<const int4*>(P.cell_count + c0);
      const int4 b = *reinterpret_cast<const int4*>(P.cell_count + c0 + 4);
      v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = (c0 + k < n) ? P.cell_count[c0 + k] : 0;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      s += v[k];
      f += v[k] > 0;
    }
    int x = s, xo = f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o), yo = __shfl_up_sync(0xffffffffu, xo, o);
      if (lane >= o) {
        x += y;
        xo += yo;
      }
    }
    if (lane == 31) {
      wsum[w] = x;
      osum[w] = xo;
    }
    __syncthreads();
    if (w == 0) {
      int t = wsum[lane], to = osum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o), yo = __shfl_up_sync(0xffffffffu, to, o);
        if (lane >= o) {
          t += y;
          to += yo;
        }
      }
      wsum[lane] = t;
      osum[lane] = to;
    }
    __syncthreads();
    int ex = carry + (w > 0 ? wsum[w - 1] : 0) + x - s;
    int eo = ocarry + (w > 0 ? osum[w - 1] : 0) + xo - f;
    int st[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      st[k] = ex;
      ex += v[k];
      if (c0 + k < n && v[k] > 0) P.occ[eo++] = c0 + k;
    }
    if (c0 + 8 <= n) {  // two 16-byte stores
      *reinterpret_cast<int4*>(P.cell_start + c0) = make_int4(st[0], st[1], st[2], st[3]);
      *reinterpret_cast<int4*>(P.cell_start + c0 + 4) = make_int4(st[4], st[5], st[6], st[7]);
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (c0 + k < n) P.cell_start[c0 + k] = st[k];
    }
    carry += wsum[kScanOneThreads / 32 - 1];
    ocarry += osum[kScanOneThreads / 32 - 1];
    __syncthreads();  // wsum, osum are rewritten by the next chunk
  }
  if (threadIdx.x == 0) {
    P.cell_start[n] = P.n;
    P.g->n_occ = ocarry;
    P.g->next_cell = 0;
  }
}

template <bool MIXED>
__global__ void __launch_bounds__(kBeadBlock) k_reorder(DevPtrs P, int cur) {
  pdl_trigger();
  pdl_wait();  // the scan's cell starts
  if (!P.g->rebuild) return;
  const int i = blockIdx.x * kBeadBlock + threadIdx.x;
  for (int c = i; c < P.n_cells_total; c += gridDim.x * kBeadBlock) P.cell_count[c] = 0;
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
  P.tkey[nw] = P.key[i];
  P.inv[o] = nw;
  if constexpr (MIXED) {
    P.mt[nw] = P.m4[cur][i];
  } else {
    P.dt4[nw] = P.d4[cur][i];
  }
}

// ------------------------------------------------------------ Verlet lists
// One CTA per cell of the list grid.  The CTA copies its beads' reordered
// state back, records their build positions, stages the beads of the 27
// surrounding cells (contiguous x-rows of the cell-sorted order) in shared
// memory and appends each bead's hits with a ballot, so a bead's list is
// written contiguously (bead-major).
constexpr int kNbrMaxCell = 1024;

struct CellCtx {
  int s, e;          // bead range of the cell
  int r, cb;         // replica and its first cell
  int cx, cy, cz;    // cell coordinates
  int n0, n1, n2;    // replica grid
};

// (Called for occupied cells only: most cells of a thin membrane box are
// empty, and their CTAs should return after two loads.)
__device__ __forceinline__ CellCtx cell_ctx(const DevPtrs& P, int c, int s, int e) {
  CellCtx q;
  q.s = s;
  q.e = e;
  int lo = 0, hi = P.n_rep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (P.rp[mid].cell_begin <= c) lo = mid; else hi = mid - 1;
  }
  q.r = lo;
  q.cb = P.rp[lo].cell_begin;
  const RepState& rs = P.rs[lo];
  q.n0 = rs.ncell[0];
  q.n1 = rs.ncell[1];
  q.n2 = rs.ncell[2];
  const int local = c - q.cb;
  q.cx = local % q.n0;
  q.cy = (local / q.n0) % q.n1;
  q.cz = local / (q.n0 * q.n1);
  return q;
}

// Copies the cell's reordered state back from the scratch arrays.
template <bool MIXED, int NT>
__device__ __forceinline__ void copy_back(const DevPtrs& P, int cur, const CellCtx& q, const RepState& rs) {
  for (int i = q.s + threadIdx.x; i < q.e; i += NT) {
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
    if constexpr (MIXED) {
      P.m4[cur][i] = P.mt[i];
      P.ref[i] = P.mt[i];
    } else {
      const double4 d = P.dt4[i];
      P.d4[cur][i] = d;
      P.ref[i] = make_uint4(to_frac(d.x, rs.frac_per_len[0]), to_frac(d.y, rs.frac_per_len[1]),
                            to_frac(d.z, rs.frac_per_len[2]), 0u);
    }
  }
}

// The stencil as contiguous bead ranges with prefix sums (one thread): cells
// are ordered x-fastest, so each (dy,dz) row of 3 cells is one range unless
// it wraps in x.  Axes with fewer than 3 cells take every cell once.
__device__ __forceinline__ int stencil_segments(const DevPtrs& P, const CellCtx& q, int* seg_s, int* seg_p) {
  int nseg = 0;
  const int lo1 = q.n1 >= 3 ? -1 : 0, hi1 = q.n1 >= 2 ? 1 : 0;
  const int lo2 = q.n2 >= 3 ? -1 : 0, hi2 = q.n2 >= 2 ? 1 : 0;
  int xa = q.cx - 1, xb = q.cx + 1;
  if (q.n0 < 3) {
    xa = 0;
    xb = q.n0 - 1;
  }
  int acc = 0;
  for (int oz = lo2; oz <= hi2; ++oz) {
    const int zz = (q.cz + oz + q.n2) % q.n2;
    for (int oy = lo1; oy <= hi1; ++oy) {
      const int yy = (q.cy + oy + q.n1) % q.n1;
      const int row = q.cb + q.n0 * (yy + q.n1 * zz);
      int a0, a1, b0 = 0, b1 = 0;
      if (xa >= 0 && xb < q.n0) {
        a0 = row + xa;
        a1 = row + xb + 1;
      } else if (xa < 0) {  // cells n0-1 | 0..xb
        a0 = row + q.n0 - 1;
        a1 = row + q.n0;
        b0 = row;
        b1 = row + xb + 1;
      } else {  // cells xa..n0-1 | 0
        a0 = row + xa;
        a1 = row + q.n0;
        b0 = row;
        b1 = row + 1;
      }
      seg_s[nseg] = P.cell_start[a0];
      seg_p[nseg] = acc;
      acc += P.cell_start[a1] - seg_s[nseg];
      ++nseg;
      if (b1 > b0) {
        seg_s[nseg] = P.cell_start[b0];
        seg_p[nseg] = acc;
        acc += P.cell_start[b1] - seg_s[nseg];
        ++nseg;
      }
    }
  }
  seg_p[nseg] = acc;
  return nseg;
}

// Bead of staged position g.
__device__ __forceinline__ int seg_bead(const int* seg_s, const int* seg_p, int nseg, int g) {
  int q = 0;
  while (q + 1 < nseg && seg_p[q + 1] <= g) ++q;
  return seg_s[q] + (g - seg_p[q]);
}

__device__ __forceinline__ void list_counts(const DevPtrs& P, const CellCtx& q, const int* cnt, int nt) {
  for (int b = threadIdx.x; b < q.e - q.s; b += nt) {
    const int count = cnt[b];
    P.nnbr[q.s + b] = count < P.kmax ? count : P.kmax;
    if (count > *(volatile int*)&P.g->max_nbr) atomicMax(&P.g->max_nbr, count);
    if (count > P.kmax) {
      atomicOr(&P.g->error, 1);
      atomicMax(&P.g->need_nbr, count);
    }
  }
}

// Occupied cells of this CTA for the list kernels: round 0 takes
// occ[blockIdx.x] without a claim; when the occupied cells outnumber the CTAs,
// later rounds take the rest from a device work queue, one at a time, which
// balances the very uneven cell occupancy.  -1 when none is left.  Every
// thread of the CTA gets the same cell.
__device__ __forceinline__ int list_cell(const DevPtrs& P, int round) {
  __shared__ int cell;
  const int n_occ = P.g->n_occ;
  if (round == 0) return (int)blockIdx.x < n_occ ? P.occ[blockIdx.x] : -1;
  if ((int)gridDim.x >= n_occ) return -1;
  __syncthreads();  // every thread has read the previous cell
  if (threadIdx.x == 0) {
    const int k = (int)gridDim.x + atomicAdd(&P.g->next_cell, 1);
    cell = k < n_occ ? P.occ[k] : -1;
  }
  __syncthreads();
  return cell;
}

__device__ __forceinline__ void list_build_begin(const DevPtrs& P) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.g->slack = 0.0;
    P.g->n_rebuilds++;
  }
}

// ---- FP64 form: each warp takes one bead of the cell at a time and tests
// 32 staged candidates per round with the minimum image of the box.
constexpr int kNbrThreads = 128;
constexpr int kNbrChunkD = 768;  // 24 KB of staged double4

__device__ __forceinline__ void nbr_cell_plain(const DevPtrs& P, int cur, int c) {
  const int s0 = P.cell_start[c], e0 = P.cell_start[c + 1];
  if (s0 >= e0) return;
  const CellCtx q = cell_ctx(P, c, s0, e0);
  const RepState& rs = P.rs[q.r];
  copy_back<false, kNbrThreads>(P, cur, q, rs);
  __shared__ int seg_s[18], seg_p[19];
  __shared__ int nseg_sh;
  __shared__ int cnt[kNbrMaxCell];
  __shared__ int cidx[kNbrChunkD];
  __shared__ double4 cposd[kNbrChunkD];
  __syncthreads();  // the previous cell of this CTA is done with the shared arrays
  const int nb = q.e - q.s;
  if (nb > kNbrMaxCell) {
    if (threadIdx.x == 0) atomicOr(&P.g->error, 2);
    return;
  }
  if (threadIdx.x == 0) nseg_sh = stencil_segments(P, q, seg_s, seg_p);
  for (int k = threadIdx.x; k < nb; k += kNbrThreads) cnt[k] = 0;
  __syncthreads();
  const int nseg = nseg_sh;
  const int M = seg_p[nseg];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned int below = (1u << lane) - 1u;
  const int kmax = P.kmax;
  const double lc2 = P.tab->list_cut2;
  for (int base = 0; base < M; base += kNbrChunkD) {
    const int m = min(kNbrChunkD, M - base);
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += kNbrThreads) {
      const int j = seg_bead(seg_s, seg_p, nseg, base + k);
      cidx[k] = j;
      cposd[k] = P.dt4[j];
    }
    __syncthreads();
    for (int b = warp; b < nb; b += kNbrThreads / 32) {
      const int i = q.s + b;
      int count = cnt[b];
      int* out = P.nbr + (size_t)i * kmax;
      const double4 di = P.dt4[i];
      for (int k0 = 0; k0 < m; k0 += 32) {
        const int k = k0 + lane;
        bool hit = false;
        if (k < m) {
          const double4 dj = cposd[k];
          double dx = di.x - dj.x, dy = di.y - dj.y, dz = di.z - dj.z;
          dx -= rs.box[0] * rint(dx * (1.0 / 4294967296.0) * rs.frac_per_len[0]);
          dy -= rs.box[1] * rint(dy * (1.0 / 4294967296.0) * rs.frac_per_len[1]);
          dz -= rs.box[2] * rint(dz * (1.0 / 4294967296.0) * rs.frac_per_len[2]);
          hit = (dx * dx + dy * dy + dz * dz < lc2) && (cidx[k] != i);
        }
        const unsigned int hits = __ballot_sync(0xffffffffu, hit);
        if (hit) {
          const int slot = count + __popc(hits & below);
          if (slot < kmax) out[slot] = cidx[k];
        }
        count += __popc(hits);
      }
      if (lane == 0) cnt[b] = count;
    }
  }
  __syncthreads();
  list_counts(P, q, cnt, kNbrThreads);
}

__global__ void __launch_bounds__(kNbrThreads) k_nbr_cells_plain(DevPtrs P, int cur) {
  pdl_wait();  // the reordered state
  if (!P.g->rebuild) return;
  list_build_begin(P);
  for (int r = 0, c = list_cell(P, 0); c >= 0; c = list_cell(P, ++r)) nbr_cell_plain(P, cur, c);
}

// ---- Mixed form, octant-filtered.  Candidates are staged as FP32 offsets
// from the cell centre (exact 32-bit fractional differences, scaled once),
// segment by segment; while staging, each warp appends its 32 candidates to
// the list of every octant of the cell whose box they lie within list_cut of
// (about 45 % of the stencil per octant), with one ballot per octant.  Each
// bead then scans only its octant's list, padded to rounds of 32 with a far
// sentinel.  The list cut carries a 1e-4 sigma margin over the FP32
// rounding of the offsets, so the list is a superset of the exact one.
constexpr int kOctThreads = 256;
constexpr int kOctChunk = 1024;  // staged candidates per pass (16 KB)

__device__ __forceinline__ unsigned int cell_centre_frac(int c, int n) {
  return (unsigned int)((((unsigned long long)(2 * c + 1)) << 32) / (unsigned long long)(2 * n));
}

// Row segments of the stencil computed by nine threads at once: row t
// (dy, dz) gives slots 2t and 2t+1 (the second is empty unless the row
// wraps in x); thread 0 then forms the prefix sums.
__device__ __forceinline__ void stencil_rows(const DevPtrs& P, const CellCtx& q, int* seg_s, int* seg_len) {
  const int t = threadIdx.x;
  if (t >= 9) return;
  const int oy = t % 3 - 1, oz = t / 3 - 1;
  const int lo1 = q.n1 >= 3 ? -1 : 0, hi1 = q.n1 >= 2 ? 1 : 0;
  const int lo2 = q.n2 >= 3 ? -1 : 0, hi2 = q.n2 >= 2 ? 1 : 0;
  seg_len[2 * t] = 0;
  seg_len[2 * t + 1] = 0;
  seg_s[2 * t] = 0;
  seg_s[2 * t + 1] = 0;
  if (oy < lo1 || oy > hi1 || oz < lo2 || oz > hi2) return;
  int xa = q.cx - 1, xb = q.cx + 1;
  if (q.n0 < 3) {
    xa = 0;
    xb = q.n0 - 1;
  }
  const int zz = (q.cz + oz + q.n2) % q.n2, yy = (q.cy + oy + q.n1) % q.n1;
  const int row = q.cb + q.n0 * (yy + q.n1 * zz);
  int a0, a1, b0 = 0, b1 = 0;
  if (xa >= 0 && xb < q.n0) {
    a0 = row + xa;
    a1 = row + xb + 1;
  } else if (xa < 0) {
    a0 = row + q.n0 - 1;
    a1 = row + q.n0;
    b0 = row;
    b1 = row + xb + 1;
  } else {
    a0 = row + xa;
    a1 = row + q.n0;
    b0 = row;
    b1 = row + 1;
  }
  const int sa = P.cell_start[a0], ea = P.cell_start[a1];
  seg_s[2 * t] = sa;
  seg_len[2 * t] = ea - sa;
  if (b1 > b0) {
    const int sb = P.cell_start[b0], eb = P.cell_start[b1];
    seg_s[2 * t + 1] = sb;
    seg_len[2 * t + 1] = eb - sb;
  }
}

// The same row segments formed by one warp: lane l < 18 takes half-row l
// (row t = l / 2; the second half is empty unless the row wraps in x), and
// the non-empty halves are compacted in lane order with their stencil-slot
// prefix sums (ballot and shuffles), the count going to seg_len[0].
__device__ __forceinline__ void stencil_warp(const DevPtrs& P, const CellCtx& q, int* seg_s, int* seg_p,
                                             int* seg_len) {
  const int lane = threadIdx.x & 31;
  int start = 0, len = 0;
  if (lane < 18) {
    const int t = lane >> 1, half = lane & 1;
    const int oy = t % 3 - 1, oz = t / 3 - 1;
    const int lo1 = q.n1 >= 3 ? -1 : 0, hi1 = q.n1 >= 2 ? 1 : 0;
    const int lo2 = q.n2 >= 3 ? -1 : 0, hi2 = q.n2 >= 2 ? 1 : 0;
    if (oy >= lo1 && oy <= hi1 && oz >= lo2 && oz <= hi2) {
      int xa = q.cx - 1, xb = q.cx + 1;
      if (q.n0 < 3) {
        xa = 0;
        xb = q.n0 - 1;
      }
      const int zz = (q.cz + oz + q.n2) % q.n2, yy = (q.cy + oy + q.n1) % q.n1;
      const int row = q.cb + q.n0 * (yy + q.n1 * zz);
      int a0, a1, b0 = 0, b1 = 0;
      if (xa >= 0 && xb < q.n0) {
        a0 = row + xa;
        a1 = row + xb + 1;
      } else if (xa < 0) {
        a0 = row + q.n0 - 1;
        a1 = row + q.n0;
        b0 = row;
        b1 = row + xb + 1;
      } else {
        a0 = row + xa;
        a1 = row + q.n0;
        b0 = row;
        b1 = row + 1;
      }
      const int u0 = half ? b0 : a0, u1 = half ? b1 : a1;
      if (u1 > u0) {
        start = P.cell_start[u0];
        len = P.cell_start[u1] - start;
      }
    }
  }
  const unsigned int full = __ballot_sync(0xffffffffu, len > 0);
  int incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (len > 0) {
    const int k = __popc(full & ((1u << lane) - 1u));
    seg_s[k] = start;
    seg_p[k] = incl - len;
  }
  if (lane == 31) {
    seg_p[__popc(full)] = incl;
    seg_len[0] = __popc(full);
  }
}

__device__ __forceinline__ void nbr_cell_oct(const DevPtrs& P, int cur, int c) {
  const int s0 = P.cell_start[c], e0 = P.cell_start[c + 1];
  if (s0 >= e0) return;
  __shared__ CellCtx qs;
  __shared__ unsigned int cr_s[3];
  __shared__ float h_s[3];
  __shared__ int seg_s[18], seg_len[18], seg_p[19];
  __shared__ int oct_c[8];
  __shared__ int cnt[kNbrMaxCell];
  __shared__ float4 stage[kOctChunk + 1];  // + one far sentinel
  __shared__ unsigned short clist[8][kOctChunk + 32];
  __syncthreads();  // the previous cell of this CTA is done with the shared arrays
  if (threadIdx.x == 0) {
    const CellCtx q0 = cell_ctx(P, c, s0, e0);
    qs = q0;
    const RepState& r0 = P.rs[q0.r];
    cr_s[0] = cell_centre_frac(q0.cx, q0.n0);
    cr_s[1] = cell_centre_frac(q0.cy, q0.n1);
    cr_s[2] = cell_centre_frac(q0.cz, q0.n2);
    // octant boxes: half a cell wide, centred a quarter cell off the cell centre
    h_s[0] = (float)(0.25 * r0.box[0] / q0.n0) + 1e-4f;
    h_s[1] = (float)(0.25 * r0.box[1] / q0.n1) + 1e-4f;
    h_s[2] = (float)(0.25 * r0.box[2] / q0.n2) + 1e-4f;
  }
  __syncthreads();
  const CellCtx q = qs;
  const RepState& rs = P.rs[q.r];
  const int nb = q.e - q.s;
  if (nb > kNbrMaxCell) {
    if (threadIdx.x == 0) atomicOr(&P.g->error, 2);
    return;
  }
  copy_back<true, kOctThreads>(P, cur, q, rs);
  stencil_rows(P, q, seg_s, seg_len);
  for (int b = threadIdx.x; b < nb; b += kOctThreads) cnt[b] = 0;
  if (threadIdx.x == 0) stage[kOctChunk] = make_float4(1e30f, 1e30f, 1e30f, __int_as_float(-1));
  __syncthreads();
  if (threadIdx.x == 0) {  // prefix sums over the 18 slots, empty ones dropped
    int k = 0, acc = 0;
    for (int t = 0; t < 18; ++t) {
      if (seg_len[t] == 0) continue;
      seg_s[k] = seg_s[t];
      seg_p[k] = acc;
      acc += seg_len[t];
      ++k;
    }
    seg_p[k] = acc;
    seg_len[0] = k;
  }
  __syncthreads();
  const int nseg = seg_len[0];
  const int M = seg_p[nseg];
  const unsigned int crx = cr_s[0], cry = cr_s[1], crz = cr_s[2];
  const float hx = h_s[0], hy = h_s[1], hz = h_s[2];
  const float sx = rs.len_per_frac[0], sy = rs.len_per_frac[1], sz = rs.len_per_frac[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned int below = (1u << lane) - 1u;
  const int kmax = P.kmax;
  const float lcut = P.tab->list_cut_f + 1e-4f;
  const float lc2 = lcut * lcut;
  // thin boxes (fewer than 3 cells on an axis) take the flat scan with the
  // minimum image per pair; the octant filter assumes a full stencil
  const bool thin = q.n0 < 3 || q.n1 < 3 || q.n2 < 3;
  const float bx = sx * 4294967296.0f, by = sy * 4294967296.0f, bz = sz * 4294967296.0f;
  for (int base = 0; base < M; base += kOctChunk) {
    const int m = min(kOctChunk, M - base);
    if (base > 0) __syncthreads();  // every warp is done with the previous chunk
    if (threadIdx.x < 8) oct_c[threadIdx.x] = 0;
    __syncthreads();
    // stage every segment with all threads, then let each warp append its
    // 32 staged candidates to the list of every octant box they lie within
    // list_cut of
    for (int t = 0; t < nseg; ++t) {
      const int ps = seg_p[t];
      const int lo = max(ps, base), hi = min(seg_p[t + 1], base + m);
      for (int g = lo + threadIdx.x; g < hi; g += kOctThreads) {
        const int j = seg_s[t] + (g - ps);
        const uint4 mj = P.mt[j];
        stage[g - base] = make_float4((float)(int)(mj.x - crx) * sx, (float)(int)(mj.y - cry) * sy,
                                      (float)(int)(mj.z - crz) * sz, __int_as_float(j));
      }
    }
    __syncthreads();
    for (int k0 = warp * 32; k0 < m; k0 += kOctThreads) {
      const int k = k0 + lane;
      unsigned int pass = 0;
      if (k < m) {
        if (thin) {
          pass = 0xffu;
        } else {
          const float4 cj = stage[k];
          const float x = cj.x, y = cj.y, z = cj.z;
          const float xl = fmaxf(fabsf(x + hx) - hx, 0.f), xu = fmaxf(fabsf(x - hx) - hx, 0.f);
          const float yl = fmaxf(fabsf(y + hy) - hy, 0.f), yu = fmaxf(fabsf(y - hy) - hy, 0.f);
          const float zl = fmaxf(fabsf(z + hz) - hz, 0.f), zu = fmaxf(fabsf(z - hz) - hz, 0.f);
          const float x0 = xl * xl, x1 = xu * xu;
          const float yz0 = yl * yl + zl * zl, yz1 = yu * yu + zl * zl, yz2 = yl * yl + zu * zu,
                      yz3 = yu * yu + zu * zu;
          pass = (x0 + yz0 < lc2 ? 1u : 0u) | (x1 + yz0 < lc2 ? 2u : 0u) | (x0 + yz1 < lc2 ? 4u : 0u) |
                 (x1 + yz1 < lc2 ? 8u : 0u) | (x0 + yz2 < lc2 ? 16u : 0u) | (x1 + yz2 < lc2 ? 32u : 0u) |
                 (x0 + yz3 < lc2 ? 64u : 0u) | (x1 + yz3 < lc2 ? 128u : 0u);
        }
      }
#pragma unroll
      for (int o = 0; o < 8; ++o) {
        const unsigned int bal = __ballot_sync(0xffffffffu, (pass >> o) & 1u);
        if (bal == 0) continue;
        int at = 0;
        if (lane == 0) at = atomicAdd(&oct_c[o], __popc(bal));
        at = __shfl_sync(0xffffffffu, at, 0);
        if ((pass >> o) & 1u) clist[o][at + __popc(bal & below)] = (unsigned short)k;
      }
    }
    __syncthreads();
    // pad every octant list to a multiple of 32 with the sentinel slot
    for (int o = warp; o < 8; o += kOctThreads / 32) {
      const int nc = oct_c[o], ncp = (nc + 31) & ~31;
      if (nc + lane < ncp) clist[o][nc + lane] = (unsigned short)kOctChunk;
    }
    __syncthreads();
    for (int b = warp; b < nb; b += kOctThreads / 32) {
      const int i = q.s + b;
      const uint4 mi = P.mt[i];
      const int o = ((int)(mi.x - crx) >= 0 ? 1 : 0) | ((int)(mi.y - cry) >= 0 ? 2 : 0) |
                    ((int)(mi.z - crz) >= 0 ? 4 : 0);
      const float xi = (float)(int)(mi.x - crx) * sx, yi = (float)(int)(mi.y - cry) * sy,
                  zi = (float)(int)(mi.z - crz) * sz;
      const int ncp = (oct_c[o] + 31) & ~31;
      const unsigned short* cl = clist[o];
      int count = cnt[b];
      int* out = P.nbr + (size_t)i * kmax;
#pragma unroll 4
      for (int k0 = 0; k0 < ncp; k0 += 32) {
        const float4 cj = stage[cl[k0 + lane]];
        float dx = xi - cj.x, dy = yi - cj.y, dz = zi - cj.z;
        if (thin) {
          dx -= bx * rintf(dx / bx);
          dy -= by * rintf(dy / by);
          dz -= bz * rintf(dz / bz);
        }
        const int j = __float_as_int(cj.w);
        const bool hit = (dx * dx + dy * dy + dz * dz < lc2) & (j != i) & (j >= 0);
        const unsigned int hits = __ballot_sync(0xffffffffu, hit);
        if (hits) {
          const int slot = count + __popc(hits & below);
          if (hit && slot < kmax) out[slot] = j;
          count += __popc(hits);
        }
      }
      if (lane == 0) cnt[b] = count;
    }
  }
  __syncthreads();
  list_counts(P, q, cnt, kOctThreads);
}

__global__ void __launch_bounds__(kOctThreads) k_nbr_cells_oct(DevPtrs P, int cur) {
  pdl_wait();  // the reordered state
  if (!P.g->rebuild) return;
  list_build_begin(P);
  for (int r = 0, c = list_cell(P, 0); c >= 0; c = list_cell(P, ++r)) nbr_cell_oct(P, cur, c);
}

// ---- Mixed form, flat stencil.  The CTA stages the stencil's beads as FP32
// offsets from the cell centre (exact 32-bit fractional differences, scaled
// once), one x-row segment after another with no per-candidate search, and
// each warp tests one bead of the cell against every staged candidate.  Few
// barriers and 16 KB of shared memory per CTA: at the ~30 beads of an
// occupied membrane cell this costs fewer instructions than filtering the
// stencil per octant first.
constexpr int kFlatChunk = 1024;  // staged candidates per pass (16 KB)

// One bead (one warp) against mpad staged candidates (a multiple of 32):
// appends the hits within lc2 to the bead's list from position count.
template <bool THIN>
__device__ __forceinline__ int flat_scan(const float4* stage, int mpad, float xi, float yi, float zi, int i,
                                         float lc2, float bx, float by, float bz, int* out, int count, int kmax,
                                         int lane) {
  const unsigned int below = (1u << lane) - 1u;
#pragma unroll 4
  for (int k0 = 0; k0 < mpad; k0 += 32) {
    const float4 cj = stage[k0 + lane];
    float dx = xi - cj.x, dy = yi - cj.y, dz = zi - cj.z;
    if constexpr (THIN) {  // fewer than 3 cells on an axis: minimum image per pair
      dx -= bx * rintf(dx / bx);
      dy -= by * rintf(dy / by);
      dz -= bz * rintf(dz / bz);
    }
    const int j = __float_as_int(cj.w);
    bool hit = (dx * dx + dy * dy + dz * dz < lc2) & (j != i);
    if constexpr (THIN) hit = hit & (j >= 0);  // the minimum image can fold a sentinel back
    const unsigned int hits = __ballot_sync(0xffffffffu, hit);
    if (hits) {
      const int slot = count + __popc(hits & below);
      if (hit && slot < kmax) out[slot] = j;
      count += __popc(hits);
    }
  }
  return count;
}

// Two beads (one warp) against the same staged candidates: one shared load
// and one loop step serve both.  Appends as flat_scan does, per bead.
template <bool THIN>
__device__ __forceinline__ void flat_scan2(const float4* stage, int mpad, float xa, float ya, float za, int ia,
                                           float xb, float yb, float zb, int ib, float lc2, float bx, float by,
                                           float bz, int* outa, int* outb, int& ca, int& cb, int kmax, int lane) {
  const unsigned int below = (1u << lane) - 1u;
#pragma unroll 2
  for (int k0 = 0; k0 < mpad; k0 += 32) {
    const float4 cj = stage[k0 + lane];
    const int j = __float_as_int(cj.w);
    float dx = xa - cj.x, dy = ya - cj.y, dz = za - cj.z;
    float ex = xb - cj.x, ey = yb - cj.y, ez = zb - cj.z;
    if constexpr (THIN) {
      dx -= bx * rintf(dx / bx);
      dy -= by * rintf(dy / by);
      dz -= bz * rintf(dz / bz);
      ex -= bx * rintf(ex / bx);
      ey -= by * rintf(ey / by);
      ez -= bz * rintf(ez / bz);
    }
    bool ha = (dx * dx + dy * dy + dz * dz < lc2) & (j != ia);
    bool hb = (ex * ex + ey * ey + ez * ez < lc2) & (j != ib);
    if constexpr (THIN) {
      ha = ha & (j >= 0);
      hb = hb & (j >= 0);
    }
    const unsigned int hitsa = __ballot_sync(0xffffffffu, ha), hitsb = __ballot_sync(0xffffffffu, hb);
    if (hitsa | hitsb) {
      const int sa = ca + __popc(hitsa & below), sb = cb + __popc(hitsb & below);
      if (ha && sa < kmax) outa[sa] = j;
      if (hb && sb < kmax) outb[sb] = j;
      ca += __popc(hitsa);
      cb += __popc(hitsb);
    }
  }
}

template <int NT>
__device__ __forceinline__ void nbr_cell_flat(const DevPtrs& P, int cur, int c) {
  const int s0 = P.cell_start[c], e0 = P.cell_start[c + 1];
  if (s0 >= e0) return;
  __shared__ int seg_s[18], seg_len[18], seg_p[19];
  __shared__ int cnt[kNbrMaxCell];
  __shared__ float4 stage[kFlatChunk];
  // every thread derives the cell's context itself (the same few loads)
  const CellCtx q = cell_ctx(P, c, s0, e0);
  const RepState& rs = P.rs[q.r];
  const int nb = q.e - q.s;
  if (nb > kNbrMaxCell) {
    if (threadIdx.x == 0) atomicOr(&P.g->error, 2);
    return;
  }
  const unsigned int crx = cell_centre_frac(q.cx, q.n0), cry = cell_centre_frac(q.cy, q.n1),
                     crz = cell_centre_frac(q.cz, q.n2);
  __syncthreads();  // the previous cell of this CTA is done with the shared arrays
  copy_back<true, NT>(P, cur, q, rs);
  if (threadIdx.x < 32) stencil_warp(P, q, seg_s, seg_p, seg_len);
  for (int b = threadIdx.x; b < nb; b += NT) cnt[b] = 0;
  __syncthreads();
  const int nseg = seg_len[0];
  const int M = seg_p[nseg];
  const float sx = rs.len_per_frac[0], sy = rs.len_per_frac[1], sz = rs.len_per_frac[2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int kmax = P.kmax;
  const float lcut = P.tab->list_cut_f + 1e-4f;
  const float lc2 = lcut * lcut;
  const bool thin = q.n0 < 3 || q.n1 < 3 || q.n2 < 3;
  const float bx = sx * 4294967296.0f, by = sy * 4294967296.0f, bz = sz * 4294967296.0f;
  for (int base = 0; base < M; base += kFlatChunk) {
    const int m = min(kFlatChunk, M - base);
    const int mpad = (m + 31) & ~31;
    if (base > 0) __syncthreads();  // every warp is done with the previous chunk
    // stage the chunk: thread t takes slots base + t, + NT, ...; the bead of a
    // slot comes from the segment table, and four loads are issued together
    // (a small system has few cells per SM, so their latency is not hidden
    // by other CTAs)
    {
      constexpr int kBatch = 4;
      int t = 0;  // segment of this thread's next slot (slots only increase)
      for (int k0 = threadIdx.x; k0 < m; k0 += kBatch * NT) {
        int jj[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const int g = base + k0 + u * NT;
          jj[u] = -1;
          if (k0 + u * NT < m) {
            while (seg_p[t + 1] <= g) ++t;
            jj[u] = seg_s[t] + (g - seg_p[t]);
          }
        }
        uint4 mj[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
          if (jj[u] >= 0) mj[u] = P.mt[jj[u]];
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
          if (jj[u] >= 0)
            stage[k0 + u * NT] = make_float4((float)(int)(mj[u].x - crx) * sx, (float)(int)(mj[u].y - cry) * sy,
                                             (float)(int)(mj[u].z - crz) * sz, __int_as_float(jj[u]));
      }
    }
    // far sentinels complete the last round of 32 (index -1 matches no bead)
    for (int k = m + threadIdx.x; k < mpad; k += NT) stage[k] = make_float4(1e30f, 1e30f, 1e30f, __int_as_float(-1));
    __syncthreads();
    // beads in pairs (b, b + NT/32): warp w takes 2w, 2w+1 of every 2*NT/32
    for (int b = 2 * warp; b < nb; b += 2 * (NT / 32)) {
      const int i = q.s + b;
      const uint4 mi = P.mt[i];
      const float xi = (float)(int)(mi.x - crx) * sx, yi = (float)(int)(mi.y - cry) * sy,
                  zi = (float)(int)(mi.z - crz) * sz;
      int* out = P.nbr + (size_t)i * kmax;
      if (b + 1 < nb) {
        const int i2 = i + 1;
        const uint4 m2 = P.mt[i2];
        const float x2 = (float)(int)(m2.x - crx) * sx, y2 = (float)(int)(m2.y - cry) * sy,
                    z2 = (float)(int)(m2.z - crz) * sz;
        int ca = cnt[b], cb = cnt[b + 1];
        if (thin)
          flat_scan2<true>(stage, mpad, xi, yi, zi, i, x2, y2, z2, i2, lc2, bx, by, bz, out, out + kmax, ca, cb, kmax,
                           lane);
        else
          flat_scan2<false>(stage, mpad, xi, yi, zi, i, x2, y2, z2, i2, lc2, bx, by, bz, out, out + kmax, ca, cb, kmax,
                            lane);
        if (lane == 0) {
          cnt[b] = ca;
          cnt[b + 1] = cb;
        }
      } else {
        const int count = thin ? flat_scan<true>(stage, mpad, xi, yi, zi, i, lc2, bx, by, bz, out, cnt[b], kmax, lane)
                               : flat_scan<false>(stage, mpad, xi, yi, zi, i, lc2, bx, by, bz, out, cnt[b], kmax, lane);
        if (lane == 0) cnt[b] = count;
      }
    }
  }
  __syncthreads();
  list_counts(P, q, cnt, NT);
}

template <int NT>
__global__ void __launch_bounds__(NT, 768 / NT) k_nbr_cells_flat(DevPtrs P, int cur) {
  pdl_wait();  // the reordered state
  if (!P.g->rebuild) return;
  list_build_begin(P);
  for (int r = 0, c = list_cell(P, 0); c >= 0; c = list_cell(P, ++r)) nbr_cell_flat<NT>(P, cur, c);
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

// Size-change differences U(d) - U(s d) of the bonded terms in FP32 for the
// mixed form, with sq[k] = s_k^2 - 1.  Both are factored through the exact
// small quantities q = sum sq_k d_k^2 (= r'^2 - r^2) and its bend analogues,
// so a scale near 1 cancels nothing:
//   bond  1/2 k (r - l)^2:  (r - l)^2 - (r' - l)^2 = (r - r')(r + r' - 2l),
//                           r - r' = -q / (r + r');
//   bend  1/2 k (a - c)^2:  (a - c)^2 - (a - c')^2 = (c' - c)(2a - c - c'),
//         c = p / (|da||db|), c' - c = (dp |da||db| + p (|da||db| - |da'||db'|)) / (|da||db||da'||db'|),
//         |da||db| - |da'||db'| = -(da^2 qb + db^2 qa + qa qb) / (|da||db| + |da'||db'|).
__device__ __forceinline__ float bond_dpot_f(Vec3<float> d, const float sq[3], const float* c) {
  const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
  const float q = sq[0] * d.x * d.x + sq[1] * d.y * d.y + sq[2] * d.z * d.z;
  const float r = sqrtf(r2), rn = sqrtf(r2 + q);
  const float dr = -q / (r + rn);
  return 0.5f * c[1] * dr * (r + rn - 2.f * c[0]);
}
__device__ __forceinline__ float bend_dpot_f(Vec3<float> da, Vec3<float> db, const float sq[3], const float* c) {
  const float a2 = da.x * da.x + da.y * da.y + da.z * da.z, b2 = db.x * db.x + db.y * db.y + db.z * db.z;
  const float p = da.x * db.x + da.y * db.y + da.z * db.z;
  const float qa = sq[0] * da.x * da.x + sq[1] * da.y * da.y + sq[2] * da.z * da.z;
  const float qb = sq[0] * db.x * db.x + sq[1] * db.y * db.y + sq[2] * db.z * db.z;
  const float dp = sq[0] * da.x * db.x + sq[1] * da.y * db.y + sq[2] * da.z * db.z;
  const float ab = sqrtf(a2 * b2), abn = sqrtf((a2 + qa) * (b2 + qb));
  const float dab = -(a2 * qb + b2 * qa + qa * qb) / (ab + abn);
  const float cs = p / ab;
  const float dc = (dp * ab + p * dab) / (ab * abn);
  return 0.5f * c[1] * dc * (2.f * (c[0] - cs) - dc);
}

// float -> int64 rounded to nearest, the same value as __float2ll_rn: values
// below 2^31 in magnitude (nearly every pair term) take the 32-bit conversion.
__device__ __forceinline__ long long f2ll_rn(float y) {
  // y = a 2^16 + b exactly, a = rint(y 2^-16) and |b| <= 2^15 (for |y| >= 2^16
  // a 2^16 is within a factor two of y, so the subtraction is exact; below,
  // a = 0): two 32-bit conversions instead of the 64-bit one.  a 2^16 is an
  // even integer, so rounding b to nearest even rounds y so.  Exact for
  // |y| < 2^46.
  const float a = rintf(y * (1.0f / 65536.0f));
  const float b = fmaf(-a, 65536.0f, y);
  return ((long long)__float2int_rn(a) << 16) + (long long)__float2int_rn(b);
}

// Difference vectors e[k] = x(p-2+k) - x(p-1+k), k = 0..3, of the chain
// around bead i; valid[k] marks existing ones.  MIXED: exact from the 32-bit
// fractional mirror (in FP64); PLAIN: FP64 with the bonded minimum image.
template <bool MIXED, typename RT>
__device__ __forceinline__ void chain_vectors(const DevPtrs& P, int cur, int i, int p, int len, const double box[3],
                                              Vec3<RT> e[4], bool valid[4]) {
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
    RT s0, s1, s2;
    if constexpr (std::is_same<RT, float>::value) {
      const RepState& rs = P.rs[rep_of(P, i)];
      s0 = rs.len_per_frac[0];
      s1 = rs.len_per_frac[1];
      s2 = rs.len_per_frac[2];
    } else {
      s0 = box[0] * (1.0 / 4294967296.0);
      s1 = box[1] * (1.0 / 4294967296.0);
      s2 = box[2] * (1.0 / 4294967296.0);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      valid[k] = have[k] && have[k + 1];
      e[k].x = (RT)(int)(m[k].x - m[k + 1].x) * s0;
      e[k].y = (RT)(int)(m[k].y - m[k + 1].y) * s1;
      e[k].z = (RT)(int)(m[k].z - m[k + 1].z) * s2;
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
      e[k].x = (RT)d[0];
      e[k].y = (RT)d[1];
      e[k].z = (RT)d[2];
    }
  }
}

// x(a) - x(b) for global (file-order) bead indices of a BOND / BEND term
// (include/system.h:1897-1906, 1992-2011).  MIXED: exact from the 32-bit
// fractional mirror; PLAIN: FP64 with the reference's half-box shift.
template <bool MIXED, typename RT>
__device__ __forceinline__ Vec3<RT> term_vec(const DevPtrs& P, int cur, int a, int b, const double box[3],
                                             const RepState& rs) {
  const int ia = P.inv[a], ib = P.inv[b];
  if constexpr (MIXED) {
    const uint4 ma = P.m4[cur][ia], mb = P.m4[cur][ib];
    RT s0, s1, s2;
    if constexpr (std::is_same<RT, float>::value) {
      s0 = rs.len_per_frac[0];
      s1 = rs.len_per_frac[1];
      s2 = rs.len_per_frac[2];
    } else {
      s0 = box[0] * (1.0 / 4294967296.0);
      s1 = box[1] * (1.0 / 4294967296.0);
      s2 = box[2] * (1.0 / 4294967296.0);
    }
    return Vec3<RT>{(RT)(int)(ma.x - mb.x) * s0, (RT)(int)(ma.y - mb.y) * s1, (RT)(int)(ma.z - mb.z) * s2};
  } else {
    const double4 ma = P.d4[cur][ia], mb = P.d4[cur][ib];
    double d[3] = {ma.x - mb.x, ma.y - mb.y, ma.z - mb.z};
    for (int k = 0; k < 3; ++k) {
      if (d[k] > box[k] / 2.0) d[k] -= box[k];
      if (d[k] < -box[k] / 2.0) d[k] += box[k];
    }
    return Vec3<RT>{(RT)d[0], (RT)d[1], (RT)d[2]};
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

__device__ __forceinline__ void warp_atomic_add_q(long long v, long long* dst, int r) {
  const unsigned int peers = __match_any_sync(0xffffffffu, r);
  const int lane = threadIdx.x & 31;
  long long acc = 0;
  for (unsigned int rest = peers; rest; rest &= rest - 1) acc += __shfl_sync(peers, v, __ffs(rest) - 1);
  if (lane == __ffs(peers) - 1 && acc != 0)
    atomicAdd((unsigned long long*)dst, (unsigned long long)acc);
}

// Hash-cell counts of the reference's many-sphere branches for the current
// box: int(box / grid_len) per axis, at least 1 (the reference divides by
// zero below that; smd_create refuses such a box).
__device__ __forceinline__ void sphere_grid_dims(const SphereDev* S, const double box[3], int n[3]) {
  for (int a = 0; a < 3; ++a) {
    const double q = box[a] / S->grid_len;
    n[a] = q >= 1.0 ? (q < 1048576.0 ? (int)q : 1048576) : 1;
  }
}

// How often the reference's 27 neighbour cells visit the cell of a partner
// (getCell and neighIndices, analysis/cellInclude/cell.h:36-101): along an
// axis of one cell all three offsets land on it, along an axis of two cells
// the other cell is reached by two offsets and the own cell by one, and with
// three or more cells a partner in range lies in exactly one neighbour.
// Cells are packed 10 bits per axis and computed only for axes below three.
__device__ __forceinline__ int sphere_cells(const double x[3], const double box[3], const int n[3]) {
  int packed = 0;
  for (int a = 0; a < 3; ++a) {
    if (n[a] != 2) continue;
    const double c = floor(x[a] / (box[a] / n[a]));
    packed |= (c >= 1.0 ? 1 : 0) << (10 * a);
  }
  return packed;
}
__device__ __forceinline__ int sphere_multiplicity(int cell_a, int cell_b, const int n[3]) {
  int m = 1;
  for (int a = 0; a < 3; ++a) {
    if (n[a] == 1) m *= 3;
    else if (n[a] == 2) m *= (((cell_a >> (10 * a)) & 1) == ((cell_b >> (10 * a)) & 1)) ? 1 : 2;
  }
  return m;
}

// Per-block copy of the spheres, in dynamic shared memory of
// sphere_stage_bytes(n, MIXED): the position word (MIXED: the 32-bit
// fractional uint4, PLAIN: the double4) of each sphere, then its file index
// and hash cell.  One dependent load chain per block instead of one per
// sphere and warp.
__host__ __device__ constexpr size_t sphere_stage_bytes(int n, bool mixed) {
  return (size_t)n * ((mixed ? sizeof(uint4) : sizeof(double4)) + sizeof(int2));
}
extern __shared__ uint4 smd_sphere_stage[];

template <bool MIXED>
__device__ __forceinline__ void stage_spheres(const DevPtrs& P, int cur, const double box[3], const int gn[3]) {
  const SphereDev* S = P.sph;
  const int n = P.n_sph;
  int2* info = reinterpret_cast<int2*>(reinterpret_cast<unsigned char*>(smd_sphere_stage) +
                                        (size_t)n * (MIXED ? sizeof(uint4) : sizeof(double4)));
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const int os = S->orig[s], js = P.inv[os];
    if constexpr (MIXED) smd_sphere_stage[s] = P.m4[cur][js];
    else reinterpret_cast<double4*>(smd_sphere_stage)[s] = P.d4[cur][js];
    int cell = 0;
    if (S->grid) {
      const double x[3] = {P.x[js], P.y[js], P.z[js]};
      cell = sphere_cells(x, box, gn);
    }
    info[s] = make_int2(os, cell);
  }
  __syncthreads();
}

// Sphere <-> bead terms of bead i for every sphere of a BEAD or NANOCORE
// residue (Blob::doBeadForce, include/system.h:2043-2212, doNanoCoreForce,
// :2216-2318, and doBeadPotential / doBeadDPotential / doNanoCorePotential):
// the force on the bead into fs, and the reaction on each sphere summed over
// the warp into the sphere's accumulator (MIXED: int64 in units of 2^-32,
// exact in any order).  Energies and size-change differences take every bead
// k != sphere; forces take the partners of the reference's branch for the
// residue's size (SphereDev), each term repeated as often as the hash-cell
// branch visits it.  The separation d = x_sphere - x_bead takes the minimum
// image (MIXED: exact from the 32-bit fractional mirror; PLAIN: the
// reference's half-box shift).  Called by whole blocks after stage_spheres.
template <bool MIXED, int FL>
__device__ __forceinline__ void sphere_terms(const DevPtrs& P, int cur, int i, bool active, Vec3<double>& fs,
                                             double& e_sph, double& du_sph) {
  SphereDev* S = P.sph;
  const int nT = P.tab->nT;
  const RepState& rs = P.rs[0];
  const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
  int gn[3] = {3, 3, 3};
  if (S->grid) sphere_grid_dims(S, box, gn);
  stage_spheres<MIXED>(P, cur, box, gn);
  const int n_sph = P.n_sph;
  const int2* info = reinterpret_cast<const int2*>(reinterpret_cast<const unsigned char*>(smd_sphere_stage) +
                                                   (size_t)n_sph * (MIXED ? sizeof(uint4) : sizeof(double4)));
  const bool me_sphere = active && (P.cinfo[i] < 0) && (P.cinfo[i] & 0x40000000);
  const bool repeats = S->grid && (gn[0] < 3 || gn[1] < 3 || gn[2] < 3);
  int ti = 0, my_cell = 0;
  uint4 mu = make_uint4(0, 0, 0, 0);
  double4 md = make_double4(0, 0, 0, 0);
  if (active) {
    if constexpr (MIXED) {
      mu = P.m4[cur][i];
      ti = mu.w & 0xff;
    } else {
      md = P.d4[cur][i];
      ti = __double_as_longlong(md.w) & 0xff;
    }
    if (repeats) {
      const double x[3] = {P.x[i], P.y[i], P.z[i]};
      my_cell = sphere_cells(x, box, gn);
    }
  }
  const int o = active ? P.orig[i] : -1;
  const bool force_partner = !me_sphere || S->all_partners;
  for (int s = 0; s < n_sph; ++s) {
    const int2 si = info[s];
    double r[3] = {0.0, 0.0, 0.0};
    if (active && o != si.x) {
      double d[3];
      int ts;
      bool near;
      if constexpr (MIXED) {
        const uint4 ms = smd_sphere_stage[s];
        ts = ms.w & 0xff;
        // FP32 range test first; FP64 from the exact fractional differences
        const float fx = frac_delta(ms.x, mu.x, rs.len_per_frac[0]);
        const float fy = frac_delta(ms.y, mu.y, rs.len_per_frac[1]);
        const float fz = frac_delta(ms.z, mu.z, rs.len_per_frac[2]);
        near = (fx * fx + fy * fy + fz * fz) < (float)S->cut2[s] * 1.001f + 0.01f;
        if (near) {
          d[0] = frac_delta_d(ms.x, mu.x, box[0] * (1.0 / 4294967296.0));
          d[1] = frac_delta_d(ms.y, mu.y, box[1] * (1.0 / 4294967296.0));
          d[2] = frac_delta_d(ms.z, mu.z, box[2] * (1.0 / 4294967296.0));
        }
      } else {
        const double4 ms = reinterpret_cast<const double4*>(smd_sphere_stage)[s];
        ts = __double_as_longlong(ms.w) & 0xff;
        d[0] = ms.x - md.x;
        d[1] = ms.y - md.y;
        d[2] = ms.z - md.z;
        for (int a = 0; a < 3; ++a) {
          if (d[a] > box[a] / 2.0) d[a] -= box[a];
          if (d[a] < -box[a] / 2.0) d[a] += box[a];
        }
        near = true;
      }
      if (near) {
        const double* row = S->nanocore ? P.sphC + kBeadConst * s : P.sphC + kBeadConst * (ts * nT + ti);
        const double cut2 = S->cut2[s];
        const double dr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if constexpr ((FL & F_ENERGY) != 0) e_sph += bead_pot(dr2, row, cut2);
        if constexpr ((FL & F_DU) != 0) {
          // the reference's barostat drops the NANOCORE difference (MD.cpp:657-661)
          if (!S->nanocore) {
            const double e0 = d[0] * rs.scale[0], e1 = d[1] * rs.scale[1], e2 = d[2] * rs.scale[2];
            du_sph += bead_pot(dr2, row, cut2) - bead_pot(e0 * e0 + e1 * e1 + e2 * e2, row, cut2);
          }
        }
        if constexpr ((FL & F_ENERGY) == 0) {
          if (force_partner) {
            double mag = bead_mag(dr2, row, cut2);
            if (repeats) mag *= (double)sphere_multiplicity(my_cell, si.y, gn);
            for (int a = 0; a < 3; ++a) r[a] = d[a] * mag;
            fs.x -= r[0];
            fs.y -= r[1];
            fs.z -= r[2];
          }
        }
      }
    }
    if constexpr ((FL & F_ENERGY) == 0) {
      if constexpr (MIXED) {
        long long q[3];
        for (int a = 0; a < 3; ++a) q[a] = __double2ll_rn(r[a] * 4294967296.0);
        if (__any_sync(0xffffffffu, (q[0] | q[1] | q[2]) != 0)) {
          for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int w = 16; w > 0; w >>= 1) q[a] += __shfl_xor_sync(0xffffffffu, q[a], w);
          }
          if ((threadIdx.x & 31) == 0)
            for (int a = 0; a < 3; ++a)
              if (q[a]) atomicAdd((unsigned long long*)&S->fq[s][a], (unsigned long long)q[a]);
        }
      } else {
        if (__any_sync(0xffffffffu, (r[0] != 0.0) || (r[1] != 0.0) || (r[2] != 0.0))) {
          for (int a = 0; a < 3; ++a) r[a] = warp_sum(r[a]);
          if ((threadIdx.x & 31) == 0)
            for (int a = 0; a < 3; ++a)
              if (r[a] != 0.0) atomicAdd(&S->fd[s][a], r[a]);
        }
      }
    }
  }
  // a sphere's terms as the other spheres' partner (their reactions on it)
  // join its own sum, which k_sphere integrates
  if constexpr ((FL & F_ENERGY) == 0) {
    if (me_sphere && S->all_partners) {
      const int me = P.cinfo[i] & 0xffff;
      const double f[3] = {fs.x, fs.y, fs.z};
      for (int a = 0; a < 3; ++a) {
        if constexpr (MIXED)
          atomicAdd((unsigned long long*)&S->fq[me][a], (unsigned long long)__double2ll_rn(f[a] * 4294967296.0));
        else
          atomicAdd(&S->fd[me][a], f[a]);
      }
    }
  }
}

// ---------------------------------------------------------------- external fields
// BOUNDARY, FLOATING_BASE, ZTORQUE, ZPOWERPOTENTIAL and BALL residues, in FP64
// in both forms (steep walls; few beads), with the reference's formulas and
// quirks (boundaryF/P, floatingBaseForce/Potential, zTorqueForce/Potential,
// zPowerForce/Potential, harmonicHalfF/P, include/MD.h:458-617, 1116-1222).  A bead's own
// terms read its master position (before this thread moves it); the two
// beads of a ZTORQUE or BALL term read the current mirror, which no thread
// writes during the step, so both see the same bond.
template <bool MIXED>
__device__ __forceinline__ Vec3<double> mirror_pos(const DevPtrs& P, int cur, int s, const double box[3]) {
  if constexpr (MIXED) {
    const uint4 m = P.m4[cur][s];
    return Vec3<double>{(double)m.x * (box[0] * (1.0 / 4294967296.0)), (double)m.y * (box[1] * (1.0 / 4294967296.0)),
                        (double)m.z * (box[2] * (1.0 / 4294967296.0))};
  } else {
    const double4 m = P.d4[cur][s];
    return Vec3<double>{m.x, m.y, m.z};
  }
}

// ZTORQUE bond of file-order beads (a, b): d = x_a - x_b (minimum image) and
// the height of its middle folded into [0, Lz).
template <bool MIXED>
__device__ __forceinline__ void ztorque_bond(const DevPtrs& P, int cur, int a, int b, const double box[3],
                                             Vec3<double>& d, double& z) {
  const int sa = P.inv[a], sb = P.inv[b];
  const Vec3<double> pa = mirror_pos<MIXED>(P, cur, sa, box);
  if constexpr (MIXED) {
    const uint4 ma = P.m4[cur][sa], mb = P.m4[cur][sb];
    d = Vec3<double>{frac_delta_d(ma.x, mb.x, box[0] * (1.0 / 4294967296.0)),
                     frac_delta_d(ma.y, mb.y, box[1] * (1.0 / 4294967296.0)),
                     frac_delta_d(ma.z, mb.z, box[2] * (1.0 / 4294967296.0))};
  } else {
    const Vec3<double> pb = mirror_pos<MIXED>(P, cur, sb, box);
    double e[3] = {pa.x - pb.x, pa.y - pb.y, pa.z - pb.z};
    for (int k = 0; k < 3; ++k) {
      if (e[k] > box[k] / 2.0) e[k] -= box[k];
      if (e[k] < -box[k] / 2.0) e[k] += box[k];
    }
    d = Vec3<double>{e[0], e[1], e[2]};
  }
  z = pa.z + d.z / 2.0;
  while (z >= box[2]) z -= box[2];
  while (z < 0) z += box[2];
}

template <bool MIXED>
__device__ __noinline__ void field_force(const DevPtrs& P, int cur, int i, const int4 t, const double box[3],
                                         Vec3<double>& ff) {
  const double* c = P.tab->fieldD[term_set(t.x)];
  const int kind = term_kind(t.x);
  if (kind == kTermBall) {  // harmonicHalfF: pushes the centre and the bead apart inside r0
    Vec3<double> d;
    double z;
    ztorque_bond<MIXED>(P, cur, t.y, t.z, box, d, z);
    double dr = d.x * d.x + d.y * d.y + d.z * d.z;
    if (dr < c[0] * c[0]) {
      dr = sqrt(dr);
      const double m = -(dr - c[0]) * c[1] / dr;
      const double sg = term_role(t.x) == 0 ? 1.0 : -1.0;
      ff.x += sg * (d.x * m);
      ff.y += sg * (d.y * m);
      ff.z += sg * (d.z * m);
    }
    return;
  }
  if (kind == kTermZTorque) {
    Vec3<double> d;
    double z;
    ztorque_bond<MIXED>(P, cur, t.y, t.z, box, d, z);
    const double mag = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    double eps = c[0] - c[1] * tanh(c[2] * (z - c[3]));
    if (z > c[3]) eps = 0;
    const double m = -eps * (d.z / (mag * mag * mag * mag));
    const double sg = term_role(t.x) == 0 ? 1.0 : -1.0;
    ff.x += sg * (d.z * m * d.x);
    ff.y += sg * (d.z * m * d.y);
    ff.z += sg * (-m * (d.x * d.x + d.y * d.y));
    return;
  }
  const double pos[3] = {P.x[i], P.y[i], P.z[i]};
  if (kind == kTermBoundary) {
    const int dim = (int)c[0];
    double d = pos[dim] - c[1];
    d -= (d > box[dim] / 2.0) ? box[dim] : 0;
    d += (d < -box[dim] / 2.0) ? box[dim] : 0;
    const double dir = (d < 0) ? -1.0 : 1.0;
    d = fabs(d);
    const double d2 = d * d;
    const double mag = (d2 <= 2.0) ? c[3] * (4.0 / (d2 * d2 * d) - 2.0 / (d2 * d)) : 0.0;
    (dim == 0 ? ff.x : (dim == 1 ? ff.y : ff.z)) += mag * dir;
  } else if (kind == kTermFloating) {
    const double z = pos[2];
    if (z <= c[0]) {
      ff.z += c[3] * z * z * z - 2 * c[3] * c[0] * z * z + (2 * c[2] + c[3] * c[0] * c[0]) * z;
    } else if (z < c[1]) {
      const double rcz = z - c[1];
      ff.z += c[5] * (rcz * rcz) * (2 * z * z - (4 * c[1] - 7 * c[0]) * z + 2 * c[1] * c[1] + c[0] * (-7 * c[1] + 6 * c[0]));
    }
  } else if (kind == kTermZPower) {
    ff.z += c[0] * pow(pos[2], c[1]);
  }
}

// Potential of a term owned by this bead (one-bead terms; ZTORQUE: its
// first bead).  The FLOATING_BASE potential subtracts the residue's first
// constant (c[6]) from z and the ZTORQUE potential has no height cut-off, as
// in the reference.  Both are out of line: they run only for systems with
// field residues and keep their registers out of the common pass.
template <bool MIXED>
__device__ __noinline__ double field_potential(const DevPtrs& P, int cur, int i, const int4 t, const double box[3]) {
  const double* c = P.tab->fieldD[term_set(t.x)];
  const int kind = term_kind(t.x);
  if (kind == kTermBall) {  // between the bond's own first bead (constant 2) and the second
    Vec3<double> d;
    double z;
    ztorque_bond<MIXED>(P, cur, (int)c[2], t.z, box, d, z);
    double dr = d.x * d.x + d.y * d.y + d.z * d.z;
    if (!(dr < c[0] * c[0])) return 0.0;
    dr = sqrt(dr) - c[0];
    return 0.5 * c[1] * dr * dr;
  }
  if (kind == kTermZTorque) {
    Vec3<double> d;
    double z;
    ztorque_bond<MIXED>(P, cur, t.y, t.z, box, d, z);
    const double cs = fabs(d.z) / sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    const double eps = c[0] - c[1] * tanh(c[2] * (z - c[3]));
    return eps * (1.0 - cs * cs) / 2.0;
  }
  const double pos[3] = {P.x[i], P.y[i], P.z[i]};
  if (kind == kTermBoundary) {
    const int dim = (int)c[0];
    double d = pos[dim] - c[1];
    d -= (d > box[dim] / 2.0) ? box[dim] : 0;
    d += (d < -box[dim] / 2.0) ? box[dim] : 0;
    d = fabs(d);
    d = d * d;
    return (d <= 2.0) ? c[3] * (1.0 / (d * d) - 1.0 / d) : 0.0;
  }
  if (kind == kTermFloating) {
    const double z = pos[2] - c[6];
    if (z <= c[0]) {
      const double rmz = c[0] - z;
      return c[2] * (c[0] * c[0] - z * z) + c[3] * rmz * rmz * rmz * ((c[0] / 3.0) - (1.0 / 4.0) * rmz) + c[4];
    }
    if (z < c[1]) {
      const double rcz = c[1] - z;
      return c[5] * rcz * rcz * rcz * (rcz * ((2.0 / 5.0) * rcz - (7.0 / 4.0) * c[0]) + (2.0) * c[0] * c[0]);
    }
    return 0.0;
  }
  if (kind == kTermZPower) return -c[0] * pow(pos[2], c[1] + 1) / (c[1] + 1);
  return 0.0;
}

// Bonded force on bead i: its share of the CHAIN bonds and bends (the bead
// at chain position p takes bonds (p-1,p), (p,p+1) and bends (p-2..p),
// (p-1..p+1), (p..p+2)), then its BOND / BEND residue terms in entry order.
// FP32 in the mixed form (vectors exact from the fractional mirror), FP64 in
// the plain form; an external-field term's force is evaluated in FP64 and
// added in R.  Every step variant takes its bonded force from here.
template <bool MIXED, bool FIELDS>
__device__ __forceinline__ Vec3<typename std::conditional<MIXED, float, double>::type> bonded_force(
    const DevPtrs& P, int cur, int i, int ci, const double box[3], const RepState& rs) {
  using R = typename std::conditional<MIXED, float, double>::type;
  const Tables& T = *P.tab;
  Vec3<R> fb{0, 0, 0};
  if (ci < 0 && !(ci & 0x40000000)) {
    const int p = ci & 0xfff, len = (ci >> 12) & 0xfff, set = (ci >> 24) & 0x1f;
    Vec3<R> er[4];
    bool valid[4];
    chain_vectors<MIXED, R>(P, cur, i, p, len, box, er, valid);
    const R* cf;
    if constexpr (MIXED) cf = T.chainF[set]; else cf = T.chainD[set];
    if (valid[1]) bond_term<R>(er[1], cf, (R)-1, fb);  // bond (p-1,p): second
    if (valid[2]) bond_term<R>(er[2], cf, (R)1, fb);   // bond (p,p+1): first
    if (valid[0] && valid[1]) bend_term<R>(er[0], er[1], cf + 2, 2, fb);
    if (valid[1] && valid[2]) bend_term<R>(er[1], er[2], cf + 2, 1, fb);
    if (valid[2] && valid[3]) bend_term<R>(er[2], er[3], cf + 2, 0, fb);
  }
  if (P.n_terms > 0) {
    const int o = P.orig[i];
    const int e1 = P.term_off[o + 1];
    for (int e = P.term_off[o]; e < e1; ++e) {
      const int4 t = P.terms[e];
      const int kind = term_kind(t.x), role = term_role(t.x), set = term_set(t.x);
      if (kind > kTermBend) {
        if constexpr (FIELDS) {
          Vec3<double> f1{0.0, 0.0, 0.0};
          field_force<MIXED>(P, cur, i, t, box, f1);
          fb.x += (R)f1.x;
          fb.y += (R)f1.y;
          fb.z += (R)f1.z;
        }
        continue;
      }
      const R* cf;
      if constexpr (MIXED) cf = T.termF[set]; else cf = T.termD[set];
      if (kind == kTermBond)  // bond (first, second): the bead's force is mag (x_self - x_other)
        bond_term<R>(term_vec<MIXED, R>(P, cur, o, role == 0 ? t.z : t.y, box, rs), cf, (R)1, fb);
      else  // bend (first, second, third): da = x1 - x2, db = x2 - x3
        bend_term<R>(term_vec<MIXED, R>(P, cur, t.y, t.z, box, rs), term_vec<MIXED, R>(P, cur, t.z, t.w, box, rs),
                     cf, role, fb);
    }
  }
  return fb;
}

// Non-bonded pass: G lanes per bead walk the bead's Verlet-list entries
// (bead-major, so a group reads G consecutive indices per round) and reduce
// with shuffles.  MIXED: FP32 pair arithmetic, each pair force rounded to a
// 32-bit fixed-point value and summed in int64, so the result does not depend
// on the order of the pairs; PLAIN: FP64 with the reference's neighbour-shift
// minimum image.  Writes the per-bead pair force (fixed point or FP64) and,
// with F_DU / F_ENERGY, the replica's pair U(x)-U(s x) / pair energy.
constexpr int kGather = 4;  // neighbour gathers in flight per lane (mixed pair pass)
// Cells of the reference's grid (nCells = int(L/rc) per axis, at least 3)
// for every bead before a size-change pass: CellOpt::computeDPotential visits
// only pairs of one cell and its 26 neighbours
// (include/algorithms/cellOpt.h:1043-1180), so a pair farther than one cell
// apart that the box rescale would bring within rc adds nothing to the
// reference's difference.  The cell of each axis is the reference's
// int(x / cellSize) with the x >= n -> n-1 correction, packed in 21 bits.
// The quotient is formed in FP32 from a reciprocal: three roundings of
// 2^-24 put it within 1.8e-7 q of x / cs, below 7.4e-4 for q < 4096, so a
// quotient more than 1e-3 from an integer has the reference's integer part;
// the others (and larger quotients) take the FP64 division.
__device__ __forceinline__ int ref_cell_coord(double x, double cs, float inv_cs, int n) {
  const float q = (float)x * inv_cs;
  const float fr = q - floorf(q);
  if (fr < 1e-3f || fr > 1.f - 1e-3f || !(q < 4096.f)) return cell_coord(x, cs, n);
  const int c = (int)q;
  return c >= n ? n - 1 : (c < 0 ? 0 : c);
}
__device__ __forceinline__ void trial_replica(const DevPtrs& P, int r);

// trial = 1: also the barostat trial of every replica (trial box, scale
// factors and cleared size-change sums, one thread per replica), so that the
// barostat step launches one kernel for both; the cells do not depend on it.
__global__ void __launch_bounds__(kBlock) k_ref_cells(DevPtrs P, int trial) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (trial && i < P.n_rep) trial_replica(P, i);
  if (i >= P.n) return;
  const RepState& rs = P.rs[rep_of(P, i)];
  const double x[3] = {P.x[i], P.y[i], P.z[i]};
  unsigned long long key = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int n = rs.refn[d];
    key |= (unsigned long long)(ref_cell_coord(x[d], rs.ref_cs[d], rs.ref_inv_cs[d], n) & 0x1fffff) << (21 * d);
  }
  P.refcell[i] = key;
}

// Whether beads a and b (sorted indices) lie in the same or neighbouring
// cells of the reference's grid (periodic).  The size-change passes ask this
// only for pairs beyond rc at the current positions (pairs within rc are
// always neighbours).
__device__ __forceinline__ bool ref_cells_adjacent(const DevPtrs& P, const RepState& rs, int a, int b) {
  const unsigned long long ka = P.refcell[a], kb = P.refcell[b];
  bool adj = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int dd = (int)((ka >> (21 * d)) & 0x1fffff) - (int)((kb >> (21 * d)) & 0x1fffff);
    dd = dd < 0 ? -dd : dd;
    adj = adj && (dd <= 1 || dd == rs.refn[d] - 1);
  }
  return adj;
}

// Mixed-form pair sums of bead i over its Verlet list, lane `sub` of its G
// lanes: each pair force rounded to fixed point and summed in int32 per lane
// (flushed to int64 every 32 terms), with F_DU the size-change difference
// (fixed point) and with F_ENERGY the pair energy.  sF, sU: the FP32 tables
// in shared memory.
template <int FL, int G>
__device__ __forceinline__ void pair_sum_q(const DevPtrs& P, int cur, int i, int sub, const RepState& rs,
                                           const float* sF, const float* sU, int nT, long long& qx, long long& qy,
                                           long long& qz, long long& dq, float& eacc) {
  const Tables& T = *P.tab;
  const int nn = P.nnbr[i];
  const int* nb = P.nbr + (size_t)i * P.kmax;
  const uint4 me = P.m4[cur][i];
  const int ti = me.w & 0xff;
  const float s0 = rs.len_per_frac[0], s1 = rs.len_per_frac[1], s2 = rs.len_per_frac[2];
  float sq0 = 0.f, sq1 = 0.f, sq2 = 0.f;
  if constexpr ((FL & F_DU) != 0) {
    sq0 = rs.sq_f[0];
    sq1 = rs.sq_f[1];
    sq2 = rs.sq_f[2];
  }
  const float* rowF = sF + 6 * ti * nT;
  const float* rowU = sU + 6 * ti * nT;
  const float rc2 = T.rc2f, fs = T.fscale;
  // pair forces: branch-free (out-of-range entries add an exact 0), summed
  // per lane in int32 and flushed to int64 every 32 entries: one pair is
  // below 2^26 in fixed point, so 32 of them cannot overflow
  int ax = 0, ay = 0, az = 0;
  auto pair_force_q = [&](float dx, float dy, float dz, float r2, int tj) {
    const float* c = rowF + 6 * tj;
    const float rinv = rsqrtf(r2), r = r2 * rinv;
    const int ci = (r >= c[0]) ? 3 : 0;
    const float m = c[ci] - r;
    float mag = ((c[ci + 1] - c[ci + 2] * m) * m) * rinv * fs;
    mag = (r2 < rc2) ? mag : 0.f;
    ax += __float2int_rn(dx * mag);
    ay += __float2int_rn(dy * mag);
    az += __float2int_rn(dz * mag);
  };
  // distances and size-change terms rounded explicitly: a pair gives the
  // same bits in every unrolled copy of the loop and in the second pass below
  auto dist2 = [](float dx, float dy, float dz) { return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))); };
  auto dscale = [&](float dx, float dy, float dz) {  // sum (s_d^2 - 1) d_d^2
    return __fmaf_rn(sq2, __fmul_rn(dz, dz), __fmaf_rn(sq1, __fmul_rn(dy, dy), __fmul_rn(sq0, __fmul_rn(dx, dx))));
  };
  auto du_q = [&](float r2, float q, float rn2, int tj) -> long long {
    const float rr = __fmul_rn(r2, rsqrtf(r2)), rs2 = __fmul_rn(rn2, rsqrtf(rn2));
    return f2ll_rn(__fmul_rn(pair_dpot_f(rowU + 6 * tj, rr, rs2, __fdividef(q, __fadd_rn(rs2, rr)), T.rcf),
                             4294967296.0f));
  };
  bool entered = false;  // a pair beyond rc that the scale brings within rc
  int k = sub;
  int rounds = 0;
  // kGather independent gathers in flight per lane; batch() takes the terms
  // of one batch in list order.  The force pass loads the next batch's list
  // entries one batch ahead, so a gather waits only on itself; the
  // size-change pass does not (the registers this takes would cost it a CTA
  // per SM and spill)
  auto batch = [&](const uint4 (&og)[kGather], const int (&jg)[kGather]) {
#pragma unroll
    for (int u = 0; u < kGather; ++u) {
      const uint4 o = og[u];
      const float dx = frac_delta(me.x, o.x, s0), dy = frac_delta(me.y, o.y, s1), dz = frac_delta(me.z, o.z, s2);
      const float r2 = dist2(dx, dy, dz);
      if constexpr ((FL & F_DU) != 0) {
        // each pair once, from its lower-index bead (the term is even in d)
        const float q = dscale(dx, dy, dz);
        const float rn2 = __fadd_rn(r2, q);
        if (jg[u] > i && (r2 < rc2 || rn2 < rc2)) {
          dq += du_q(r2, q, rn2, o.w & 0xff);
          entered = entered || !(r2 < rc2);
        }
      }
      if constexpr ((FL & F_ENERGY) == 0) {
        pair_force_q(dx, dy, dz, r2, o.w & 0xff);
      } else {
        if (r2 < rc2) eacc += pair_pot<float>(rowU + 6 * (o.w & 0xff), sqrtf(r2));
      }
    }
    if (++rounds == 32 / kGather) {  // at most 32 pair terms per int32 sum
      qx += ax;
      qy += ay;
      qz += az;
      ax = ay = az = 0;
      rounds = 0;
    }
  };
  if constexpr ((FL & F_DU) == 0) {
    int jn[kGather];
    bool more = k + (kGather - 1) * G < nn;
    if (more) {
#pragma unroll
      for (int u = 0; u < kGather; ++u) jn[u] = __ldg(nb + k + u * G);
    }
    for (; more; k += kGather * G) {
      uint4 og[kGather];
      int jg[kGather];
#pragma unroll
      for (int u = 0; u < kGather; ++u) {
        jg[u] = jn[u];
        og[u] = P.m4[cur][jg[u]];
      }
      more = k + (2 * kGather - 1) * G < nn;
      if (more) {
#pragma unroll
        for (int u = 0; u < kGather; ++u) jn[u] = __ldg(nb + k + (kGather + u) * G);
      }
      batch(og, jg);
    }
  } else {
    for (; k + (kGather - 1) * G < nn; k += kGather * G) {
      uint4 og[kGather];
      int jg[kGather];
#pragma unroll
      for (int u = 0; u < kGather; ++u) {
        jg[u] = __ldg(nb + k + u * G);
        og[u] = P.m4[cur][jg[u]];
      }
      batch(og, jg);
    }
  }
  if (k < nn) {
    // the last entries (fewer than kGather): their gathers issued together,
    // then the terms in list order (an int32 sum holds at most 31 terms here)
    uint4 og[kGather - 1];
    int jg[kGather - 1];
#pragma unroll
    for (int u = 0; u < kGather - 1; ++u) {
      const bool ok = k + u * G < nn;
      jg[u] = ok ? __ldg(nb + k + u * G) : -1;
      og[u] = P.m4[cur][ok ? jg[u] : i];
    }
#pragma unroll
    for (int u = 0; u < kGather - 1; ++u) {
      if (jg[u] < 0) break;
      const int j = jg[u];
      const uint4 o = og[u];
      const float dx = frac_delta(me.x, o.x, s0), dy = frac_delta(me.y, o.y, s1), dz = frac_delta(me.z, o.z, s2);
      const float r2 = dist2(dx, dy, dz);
      if constexpr ((FL & F_DU) != 0) {
        const float q = dscale(dx, dy, dz);
        const float rn2 = __fadd_rn(r2, q);
        if (j > i && (r2 < rc2 || rn2 < rc2)) {
          dq += du_q(r2, q, rn2, o.w & 0xff);
          entered = entered || !(r2 < rc2);
        }
      }
      if constexpr ((FL & F_ENERGY) == 0) {
        pair_force_q(dx, dy, dz, r2, o.w & 0xff);
      } else {
        if (r2 < rc2) eacc += pair_pot<float>(rowU + 6 * (o.w & 0xff), sqrtf(r2));
      }
    }
  }
  qx += ax;
  qy += ay;
  qz += az;
  if constexpr ((FL & F_DU) != 0) {
    // Rare second pass: of the pairs that only the scale brings within rc,
    // the reference counts those in neighbouring cells of its grid
    // (ref_cells_adjacent); take the others' terms back out, bit for bit.
    if (entered) {
      for (int k2 = sub; k2 < nn; k2 += G) {
        const int j = __ldg(nb + k2);
        const uint4 o = P.m4[cur][j];
        const float dx = frac_delta(me.x, o.x, s0), dy = frac_delta(me.y, o.y, s1), dz = frac_delta(me.z, o.z, s2);
        const float r2 = dist2(dx, dy, dz);
        const float q = dscale(dx, dy, dz);
        const float rn2 = __fadd_rn(r2, q);
        if (j > i && !(r2 < rc2) && rn2 < rc2 && !ref_cells_adjacent(P, rs, i, j)) dq -= du_q(r2, q, rn2, o.w & 0xff);
      }
    }
  }
}

template <bool MIXED, int FL, int G>
__global__ void __launch_bounds__(kBlock) k_force(DevPtrs P, int cur) {
  pdl_trigger();
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
  const int t = blockIdx.x * kBlock + threadIdx.x;
  const int i = t / G, sub = t % G;
  const bool active = i < P.n;
  const int r = active ? rep_of(P, i) : 0;
  double dU = 0.0, ep = 0.0;
  long long qx = 0, qy = 0, qz = 0, dq = 0;
  double fx = 0, fy = 0, fz = 0;
  if (active) {
    const RepState& rs = P.rs[r];
    const int nn = P.nnbr[i];
    const int* nb = P.nbr + (size_t)i * P.kmax;
    if constexpr (MIXED) {
      float eacc = 0.f;
      pair_sum_q<FL, G>(P, cur, i, sub, rs, sF, sU, nT, qx, qy, qz, dq, eacc);
      ep = 0.5 * (double)eacc;
    } else {
      const double4 me = P.d4[cur][i];
      const int ti = __double_as_longlong(me.w) & 0xff;
      const double* rowF = sF + 6 * ti * nT;
      const double* rowU = sU + 6 * ti * nT;
      const double rc2 = T.rc2;
      const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
      for (int k = sub; k < nn; k += G) {
        const int j = __ldg(nb + k);
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
            fx += dx * mag;
            fy += dy * mag;
            fz += dz * mag;
          } else {
            ep += 0.5 * pair_pot<double>(rowU + 6 * tj, rr);
          }
        }
        if constexpr ((FL & F_DU) != 0) {
          const double nx = dx * rs.scale[0], ny = dy * rs.scale[1], nz = dz * rs.scale[2];
          const double rn2 = nx * nx + ny * ny + nz * nz;
          const double u0 = r2 < rc2 ? pair_pot<double>(rowU + 6 * tj, sqrt(r2)) : 0.0;
          const double u1 = (rn2 < rc2 && (r2 < rc2 || ref_cells_adjacent(P, rs, i, j)))
                                ? pair_pot<double>(rowU + 6 * tj, sqrt(rn2)) : 0.0;
          dU += 0.5 * (u0 - u1);
        }
      }
    }
  }
  // group reduction (integer sums are exact in any order)
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    if constexpr (MIXED) {
      qx += __shfl_xor_sync(0xffffffffu, qx, o);
      qy += __shfl_xor_sync(0xffffffffu, qy, o);
      qz += __shfl_xor_sync(0xffffffffu, qz, o);
    } else {
      fx += __shfl_xor_sync(0xffffffffu, fx, o);
      fy += __shfl_xor_sync(0xffffffffu, fy, o);
      fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
  }
  if (active && sub == 0 && (FL & F_ENERGY) == 0) {
    if constexpr (MIXED) {
      P.fq[i] = qx;
      P.fq[i + P.n] = qy;
      P.fq[i + 2 * P.n] = qz;
    } else {
      P.fp[i] = fx;
      P.fp[i + P.n] = fy;
      P.fp[i + 2 * P.n] = fz;
    }
  }
  if constexpr ((FL & F_DU) != 0) {
    if constexpr (MIXED) warp_atomic_add_q(dq, &P.rs[r].dUq_pair, r);
    else warp_atomic_add(dU, &P.rs[r].dU_pair, r);
  }
  if constexpr ((FL & F_ENERGY) != 0) warp_atomic_add(ep, &P.rs[r].e_pair, r);
}

// Per-bead pass after k_force: CHAIN terms, the total force, the Langevin
// term (include/algorithms/langevin.h:284-331) and the velocity-Verlet
// updates (include/algorithms/verlet.h:288-355, 463-491): second half-kick of
// this step, first half-kick and drift of the next, periodic wrap, and the
// position mirror for the next force pass.  Flags select the stopped,
// start-up, force-only and energy-only variants.
// One bead's part of the per-bead pass: bonded terms, the total force, the
// Langevin term and the velocity-Verlet updates, the next mirror and the
// displacement from the list build.  The bead's pair force (P.fq in fixed
// point in the mixed form, P.fp in the plain form) is read after pdl_wait;
// fs is its sphere force; the energy and size-change sums and the
// displacement accumulate into the caller's variables.
template <bool MIXED, int FL>
__device__ __forceinline__ void integ_bead(const DevPtrs& P, int cur, int i, int r, long long it,
                                           const Vec3<double>& fs, double& dU_bond, double& e_bond, double& e_kin,
                                           float& vmax) {
  const Tables& T = *P.tab;
  const RepParams& rp = P.rp[r];
  const RepState& rs = P.rs[r];
  const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
  int ti;
  if constexpr (MIXED) ti = P.m4[cur][i].w & 0xff; else ti = __double_as_longlong(P.d4[cur][i].w) & 0xff;
  // ---- CHAIN terms (FP32 in the mixed form, from exact FP64 differences)
  using R = typename std::conditional<MIXED, float, double>::type;
  Vec3<R> fb{0, 0, 0};
  const int ci = P.cinfo[i];
  const bool sphere = (ci < 0) && (ci & 0x40000000);  // integrated by k_sphere
  // bonded forces: one function for every step variant, so stopped and
  // running steps round them alike
  if constexpr ((FL & (F_PAIRONLY | F_ENERGY)) == 0) fb = bonded_force<MIXED, (FL & F_FIELDS) != 0>(P, cur, i, ci, box, rs);
  if ((FL & F_PAIRONLY) == 0 && (FL & (F_DU | F_ENERGY)) != 0 && ci < 0 && !(ci & 0x40000000)) {
    const int p = ci & 0xfff, len = (ci >> 12) & 0xfff, set = (ci >> 24) & 0x1f;
    // the chain's difference vectors in R (exact from the fractional
    // mirror in the mixed form)
    Vec3<R> er[4];
    bool valid[4];
    chain_vectors<MIXED, R>(P, cur, i, p, len, box, er, valid);
    // terms owned by the first bead of each bond / bend: energies in FP64;
    // size-change differences in FP64 (plain) or factored FP32 (mixed)
    if constexpr (MIXED && (FL & F_DU) != 0) {
      const float* cf = T.chainF[set];
      const float sq[3] = {rs.sq_f[0], rs.sq_f[1], rs.sq_f[2]};
      float du = 0.f;
      if (valid[2]) du += bond_dpot_f(er[2], sq, cf);
      if (valid[2] && valid[3]) du += bend_dpot_f(er[2], er[3], sq, cf + 2);
      dU_bond += (double)du;
    }
    if constexpr ((FL & F_ENERGY) != 0 || (!MIXED && (FL & F_DU) != 0)) {
      Vec3<double> e[4];
      if constexpr (MIXED) {
        chain_vectors<MIXED, double>(P, cur, i, p, len, box, e, valid);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) e[k] = Vec3<double>{er[k].x, er[k].y, er[k].z};
      }
      const double* cd = T.chainD[set];
      if constexpr ((FL & F_ENERGY) != 0) {
        if (valid[2]) e_bond += bond_pot(e[2], cd);
        if (valid[2] && valid[3]) e_bond += bend_pot(e[2], e[3], cd + 2);
      }
      if constexpr (!MIXED && (FL & F_DU) != 0) {
        const Vec3<double> s2{e[2].x * rs.scale[0], e[2].y * rs.scale[1], e[2].z * rs.scale[2]};
        const Vec3<double> s3{e[3].x * rs.scale[0], e[3].y * rs.scale[1], e[3].z * rs.scale[2]};
        if (valid[2]) dU_bond += bond_pot(e[2], cd) - bond_pot(s2, cd);
        if (valid[2] && valid[3]) dU_bond += bend_pot(e[2], e[3], cd + 2) - bend_pot(s2, s3, cd + 2);
      }
    }
  }
  // ---- BOND / BEND residue terms of this bead: energies and differences
  // (their forces are in bonded_force)
  if constexpr ((FL & F_PAIRONLY) == 0 && (FL & (F_DU | F_ENERGY)) != 0) {
    if (P.n_terms > 0) {
      const int o = P.orig[i];
      const int e1 = P.term_off[o + 1];
      const float sq_f[3] = {rs.sq_f[0], rs.sq_f[1], rs.sq_f[2]};
      for (int e = P.term_off[o]; e < e1; ++e) {
        const int4 t = P.terms[e];
        const int kind = term_kind(t.x), role = term_role(t.x), set = term_set(t.x);
        if (kind > kTermBend) {  // external fields: energy only (no size-change term in the reference)
          if constexpr ((FL & F_ENERGY) != 0 && (FL & F_FIELDS) != 0)
            if (role == 0) e_bond += field_potential<MIXED>(P, cur, i, t, box);
          continue;
        }
        const double* cd = T.termD[set];
        if (kind == kTermBond) {  // bond (first, second): the bead's force is mag (x_self - x_other)
          if constexpr ((FL & (F_DU | F_ENERGY)) != 0) {
            if (role == 0) {  // energy terms owned by the first bead
              if constexpr (MIXED && (FL & F_DU) != 0)
                dU_bond += (double)bond_dpot_f(term_vec<MIXED, float>(P, cur, t.y, t.z, box, rs), sq_f,
                                               T.termF[set]);
              if constexpr ((FL & F_ENERGY) != 0 || (!MIXED && (FL & F_DU) != 0)) {
                const Vec3<double> d = term_vec<MIXED, double>(P, cur, t.y, t.z, box, rs);
                if constexpr ((FL & F_ENERGY) != 0) e_bond += bond_pot(d, cd);
                if constexpr (!MIXED && (FL & F_DU) != 0) {
                  const Vec3<double> sd{d.x * rs.scale[0], d.y * rs.scale[1], d.z * rs.scale[2]};
                  dU_bond += bond_pot(d, cd) - bond_pot(sd, cd);
                }
              }
            }
          }
        } else {  // bend (first, second, third): da = x1 - x2, db = x2 - x3
          if constexpr ((FL & (F_DU | F_ENERGY)) != 0) {
            if (role == 0) {
              if constexpr (MIXED && (FL & F_DU) != 0)
                dU_bond += (double)bend_dpot_f(term_vec<MIXED, float>(P, cur, t.y, t.z, box, rs),
                                               term_vec<MIXED, float>(P, cur, t.z, t.w, box, rs), sq_f,
                                               T.termF[set]);
              if constexpr ((FL & F_ENERGY) != 0 || (!MIXED && (FL & F_DU) != 0)) {
                const Vec3<double> da = term_vec<MIXED, double>(P, cur, t.y, t.z, box, rs);
                const Vec3<double> db = term_vec<MIXED, double>(P, cur, t.z, t.w, box, rs);
                if constexpr ((FL & F_ENERGY) != 0) e_bond += bend_pot(da, db, cd);
                if constexpr (!MIXED && (FL & F_DU) != 0) {
                  const Vec3<double> sa{da.x * rs.scale[0], da.y * rs.scale[1], da.z * rs.scale[2]};
                  const Vec3<double> sb{db.x * rs.scale[0], db.y * rs.scale[1], db.z * rs.scale[2]};
                  dU_bond += bend_pot(da, db, cd) - bend_pot(sa, sb, cd);
                }
              }
            }
          }
        }
      }
    }
  }
  if constexpr ((FL & F_ENERGY) != 0) {
    const double vx = P.vx[i], vy = P.vy[i], vz = P.vz[i];
    e_kin = (vx * vx + vy * vy + vz * vz) / 2.0;
  } else {
    // The pair pass's forces are read only from here on, after the wait for
    // that kernel (this one is its programmatic dependent): the bonded
    // terms, the noise and the state loads above and below run while the
    // pair pass's last CTAs still do.
    auto total_force = [&](double F[3]) {
      pdl_wait();
      if constexpr (MIXED) {
        F[0] = (double)P.fq[i] * T.inv_fscale + (double)fb.x;
        F[1] = (double)P.fq[i + P.n] * T.inv_fscale + (double)fb.y;
        F[2] = (double)P.fq[i + 2 * P.n] * T.inv_fscale + (double)fb.z;
      } else {
        F[0] = P.fp[i] + fb.x;
        F[1] = P.fp[i + P.n] + fb.y;
        F[2] = P.fp[i + 2 * P.n] + fb.z;
      }
      if (P.n_sph > 0) {
        F[0] += fs.x;
        F[1] += fs.y;
        F[2] += fs.z;
      }
    };
    if constexpr ((FL & F_FORCES) != 0) {
      if (!sphere) {
        double F[3];
        total_force(F);
        const int o = P.orig[i];
        P.force_out[3 * o] = F[0];
        P.force_out[3 * o + 1] = F[1];
        P.force_out[3 * o + 2] = F[2];
      }
    } else if (!sphere) {
      const int o = P.orig[i];
      double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
      double x0[3] = {0.0, 0.0, 0.0};
      if constexpr ((FL & (F_STOP | F_INIT)) == 0) {  // the drift's positions, loaded before the wait
        x0[0] = P.x[i];
        x0[1] = P.y[i];
        x0[2] = P.z[i];
      }
      double a[3];
      if constexpr (MIXED && (FL & F_EXTNOISE) == 0) {
        // CHAIN force and noise summed in FP32 (both force terms of the
        // mixed form), the pair force exact from its fixed-point sum:
        // a = -gamma v + (q 2^-k + (f_chain + sigma psi))
        float nf[3];
        langevin_noise_f(rp.seed, o - rp.bead_begin, it, (FL & F_INIT) ? 1 : 0, rp.sig31f, nf);
        double e[3] = {(double)(fb.x + nf[0]), (double)(fb.y + nf[1]), (double)(fb.z + nf[2])};
        if (P.n_sph > 0) {
          e[0] += fs.x;
          e[1] += fs.y;
          e[2] += fs.z;
        }
        pdl_wait();
        const long long q[3] = {P.fq[i], P.fq[i + P.n], P.fq[i + 2 * P.n]};
        for (int d = 0; d < 3; ++d)
          a[d] = fma(-rp.gamma, v[d], fma((double)q[d], T.inv_fscale, e[d]));
      } else {
        double noise[3];  // sigma * psi
        if constexpr ((FL & F_EXTNOISE) != 0) {
          for (int d = 0; d < 3; ++d) noise[d] = rp.sigma * P.ext_noise[3 * o + d];
        } else {
          langevin_noise(rp.seed, o - rp.bead_begin, it, (FL & F_INIT) ? 1 : 0, rp.sig31, noise);
        }
        double F[3];
        total_force(F);
        for (int d = 0; d < 3; ++d) a[d] = fma(-rp.gamma, v[d], F[d]) + noise[d];
      }
      if constexpr ((FL & (F_STOP | F_INIT)) != 0) {
        P.ax[i] = a[0];
        P.ay[i] = a[1];
        P.az[i] = a[2];
        if constexpr ((FL & F_STOP) != 0) {
          if (ti != 0) {
            const double h = rp.dt * 0.5;
            P.vx[i] = fma(a[0], h, v[0]);
            P.vy[i] = fma(a[1], h, v[1]);
            P.vz[i] = fma(a[2], h, v[2]);
          }
        }
      } else {
        double x[3] = {x0[0], x0[1], x0[2]};
        if (ti != 0) {
          if constexpr (MIXED) {
            // second() of this step and first() of the next, rounded as the
            // stopped step and k_finish round them, so that a replica's
            // trajectory does not depend on where other replicas stop
            const double h = rp.dt * 0.5;
            for (int d = 0; d < 3; ++d) {
              v[d] = fma(a[d], h, fma(a[d], h, v[d]));
              x[d] = fma(v[d], rp.dt, x[d]);
              if (x[d] > box[d]) x[d] -= box[d];
              if (x[d] < 0) x[d] += box[d];
            }
          } else {
            const double h = rp.dt * 0.5;
            for (int d = 0; d < 3; ++d) {
              v[d] += (a[d] * h);  // second() of this step
              v[d] += (a[d] * h);  // first() of the next step
              x[d] += v[d] * rp.dt;
              if (x[d] > box[d]) x[d] -= box[d];
              if (x[d] < 0) x[d] += box[d];
            }
          }
          P.vx[i] = v[0];
          P.vy[i] = v[1];
          P.vz[i] = v[2];
          P.x[i] = x[0];
          P.y[i] = x[1];
          P.z[i] = x[2];
        }
        const unsigned int fx = to_frac(x[0], rs.frac_per_len[0]), fy = to_frac(x[1], rs.frac_per_len[1]),
                           fz = to_frac(x[2], rs.frac_per_len[2]);
        vmax = displacement(P.ref[i], fx, fy, fz, rs);
        if constexpr (MIXED) {
          const uint4 me = P.m4[cur][i];
          P.m4[cur ^ 1][i] = make_uint4(fx, fy, fz, me.w);
        } else {
          const double4 me = P.d4[cur][i];
          P.d4[cur ^ 1][i] = make_double4(x[0], x[1], x[2], me.w);
        }
      }
    }
  }
}

template <bool MIXED, int FL>
__global__ void __launch_bounds__(kBeadBlock) k_integ(DevPtrs P, int cur, StepEnd se) {
  // No wait here: integ_bead waits for the pair pass right before it reads
  // the pair forces, and every thread waits before the step's sums.
  const long long it = P.g->it;
  const int i = blockIdx.x * kBeadBlock + threadIdx.x;
  const bool active = i < P.n;
  const int r = active ? rep_of(P, i) : 0;
  double dU_bond = 0.0, e_bond = 0.0, e_kin = 0.0;
  float vmax = 0.f;
  // sphere <-> bead terms (BEAD residues; whole warps)
  Vec3<double> fs{0.0, 0.0, 0.0};
  double e_sph = 0.0, du_sph = 0.0;
  if constexpr ((FL & F_PAIRONLY) == 0) {
    if (P.n_sph > 0) sphere_terms<MIXED, FL>(P, cur, i, active, fs, e_sph, du_sph);
  }
  dU_bond += du_sph;
  if (active) integ_bead<MIXED, FL>(P, cur, i, r, it, fs, dU_bond, e_bond, e_kin, vmax);
  pdl_wait();  // returns at once where integ_bead has waited
  if constexpr ((FL & F_DU) != 0) {
    if constexpr (MIXED) warp_atomic_add_q(__double2ll_rn(dU_bond * 4294967296.0), &P.rs[r].dUq_bond, r);
    else warp_atomic_add(dU_bond, &P.rs[r].dU_bond, r);
  }
  if constexpr ((FL & F_ENERGY) != 0) {
    warp_atomic_add(e_bond, &P.rs[r].e_bond, r);
    warp_atomic_add(e_kin, &P.rs[r].e_kin, r);
    if (P.n_sph > 0) warp_atomic_add(e_sph, &P.rs[r].e_sphere, r);
  }
  if constexpr ((FL & (F_STOP | F_INIT | F_FORCES | F_ENERGY)) == 0) {
    vmax = warp_max(vmax);
    __shared__ float smax[kBeadBlock / 32];
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = vmax;
    __syncthreads();
    float bm = 0.f;
    if (threadIdx.x == 0)
      for (int w = 0; w < kBeadBlock / 32; ++w) bm = fmaxf(bm, smax[w]);
    if (P.n_sph > 0) {
      // k_sphere completes the step once the spheres have moved
      if (threadIdx.x == 0 && bm > 0.f) atomicMax(&P.g->dmax_bits, __float_as_uint(bm));
    } else {
      finalize_step(P, bm, se);
    }
  }
}

// Barostat trial box of replica r (MD.cpp:593-611), drawn by k_ref_cells.
__device__ __forceinline__ void trial_replica(const DevPtrs& P, int r) {
  const int trial = P.g->trial_slot;
  RepState& rs = P.rs[r];
  rs.dU_pair = 0.0;
  rs.dU_bond = 0.0;
  rs.dUq_pair = 0;
  rs.dUq_bond = 0;
  if (P.rp[r].dlxy == 0) {
    const double one[3] = {1.0, 1.0, 1.0};
    set_scale(rs, one);
    return;
  }
  const double u1 = P.trial_u[((size_t)trial * P.n_rep + r) * 2];
  double nb[3], s[3];
  trial_box(rs.box, P.rp[r].dlxy, u1, nb, s);
  for (int d = 0; d < 3; ++d) rs.trial_box[d] = nb[d];
  set_scale(rs, s);
  rs.dU_pair = 0.0;
  rs.dU_bond = 0.0;
  rs.dUq_pair = 0;
  rs.dUq_bond = 0;
}

// Metropolis decision (MD.cpp:677-720).
__global__ void k_mc(DevPtrs P) {
  const int trial = P.g->trial_slot;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rep) return;
  RepState& rs = P.rs[r];
  const RepParams& rp = P.rp[r];
  rs.accept = 0;
  if (rp.dlxy == 0) return;
  double dPot = rep_dU(rs);
  if (rp.tension != 0) dPot += rp.tension * ((rs.trial_box[0] * rs.trial_box[1]) - (rs.box[0] * rs.box[1]));
  const double u2 = P.trial_u[((size_t)trial * P.n_rep + r) * 2 + 1];
  rs.last_dU = dPot;
  rs.n_trial++;
  // MD.cpp's test D >= u2 || -dPot <= 0 with D = exp(dPot / kT); the
  // exponential is needed only when the second clause fails
  if (-dPot <= 0 || exp(dPot / rp.kT) >= u2) {
    double shift = 0.0;  // pair distances within rc + skin change by at most this
    for (int d = 0; d < 3; ++d) {
      shift = fmax(shift, fabs(rs.scale[d] - 1.0) * P.tab->list_cut);
      rs.box[d] = rs.trial_box[d];
    }
    derive_box(rs, rp.cell_cap, P.tab->list_cut, P.tab->rc);
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
// mode bit 0: restart half-kick (MD.cpp:300-308); bit 1: the stopped step was
// a loop step.  A sphere's stored acceleration is its undivided force.  The
// reference divides a BEAD sphere's by its mass after the forces and again
// before first() (MD.cpp:340-355, 480-509), so a first half-kick that follows
// a second one uses a / m^2, the one of a fresh start a / m.  A NANOCORE
// core is divided after the forces only (MD.cpp:291-303, 495-507): a / m
// after a second half-kick, the undivided a at a fresh start.
template <bool MIXED>
__global__ void __launch_bounds__(kBeadBlock) k_finish(DevPtrs P, int cur, int mode, int apply_mc, StepEnd se) {
  const int i = blockIdx.x * kBeadBlock + threadIdx.x;
  const int do_second = mode & 1;
  float vmax = 0.f;
  if (i < P.n) {
    const int r = rep_of(P, i);
    const RepParams& rp = P.rp[r];
    const RepState& rs = P.rs[r];
    const int ci = P.cinfo[i];
    const bool sphere = (ci < 0) && (ci & 0x40000000);
    int ti;
    if constexpr (MIXED) ti = P.m4[cur][i].w & 0xff; else ti = __double_as_longlong(P.d4[cur][i].w) & 0xff;
    double x[3] = {P.x[i], P.y[i], P.z[i]};
    if (apply_mc && rs.accept)
      for (int d = 0; d < 3; ++d) x[d] *= rs.scale[d];
    if (ti != 0) {
      const double h = rp.dt * 0.5;
      double a[3] = {P.ax[i], P.ay[i], P.az[i]};
      double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
      double af[3] = {a[0], a[1], a[2]};
      if (sphere) {
        const double m = P.sph->mass[P.cinfo[i] & 0xffff];
        const bool core = P.sph->nanocore;
        for (int d = 0; d < 3; ++d) {
          const double a0 = a[d];
          a[d] = a0 / m;
          if (mode & 3) af[d] = core ? a[d] : a[d] / m;
          else af[d] = core ? a0 : a[d];
        }
      }
      for (int d = 0; d < 3; ++d) {
        if (do_second) v[d] = fma(a[d], h, v[d]);
        v[d] = fma(af[d], h, v[d]);
        x[d] = fma(v[d], rp.dt, x[d]);
        if (x[d] > rs.box[d]) x[d] -= rs.box[d];
        if (x[d] < 0) x[d] += rs.box[d];
      }
      P.vx[i] = v[0];
      P.vy[i] = v[1];
      P.vz[i] = v[2];
    }
    P.x[i] = x[0];
    P.y[i] = x[1];
    P.z[i] = x[2];
    const unsigned int fx = to_frac(x[0], rs.frac_per_len[0]), fy = to_frac(x[1], rs.frac_per_len[1]),
                       fz = to_frac(x[2], rs.frac_per_len[2]);
    vmax = displacement(P.ref[i], fx, fy, fz, rs);
    if constexpr (MIXED) {
      const uint4 me = P.m4[cur][i];
      P.m4[cur ^ 1][i] = make_uint4(fx, fy, fz, me.w);
    } else {
      const double4 me = P.d4[cur][i];
      P.d4[cur ^ 1][i] = make_double4(x[0], x[1], x[2], me.w);
    }
  }
  vmax = warp_max(vmax);
  __shared__ float smax[kBeadBlock / 32];
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = vmax;
  __syncthreads();
  float bm = 0.f;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBeadBlock / 32; ++w) bm = fmaxf(bm, smax[w]);
  finalize_step(P, bm, se);
}

// BEAD spheres and NANOCORE cores after k_integ (one block, one sphere per
// thread): the total force on each sphere (its non-bonded force, the reactions
// gathered in k_integ and the BEAD sphere-sphere terms,
// include/system.h:2072-2098, or the cores' terms on each other), its
// Langevin term, the mass division of MD.cpp:480-509 and, in a loop step, both half-kicks,
// the drift and the wrap; then the step's list-rebuild decision.  The same
// flags as k_integ select the variant.
template <bool MIXED, int FL>
__global__ void __launch_bounds__(kMaxSpheres) k_sphere(DevPtrs P, int cur, StepEnd se) {
  SphereDev* S = P.sph;
  const int s = threadIdx.x;
  // every sphere's position word, so that the sphere-sphere loop reads
  // shared memory instead of a dependent load chain per partner
  using Word = typename std::conditional<MIXED, uint4, double4>::type;
  __shared__ Word pos_s[kMaxSpheres];
  if (s < S->n) {
    const int js = P.inv[S->orig[s]];
    if constexpr (MIXED) pos_s[s] = P.m4[cur][js]; else pos_s[s] = P.d4[cur][js];
  }
  __syncthreads();
  const long long it = P.g->it;
  const Tables& T = *P.tab;
  const RepParams& rp = P.rp[0];
  const RepState& rs = P.rs[0];
  const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
  float vmax = 0.f;
  double e = 0.0, du = 0.0;
  if (s < S->n) {
    const int o = S->orig[s], j = P.inv[o];
    int ti;
    if constexpr (MIXED) ti = pos_s[s].w & 0xff; else ti = __double_as_longlong(pos_s[s].w) & 0xff;
    double F[3] = {0.0, 0.0, 0.0};
    if constexpr ((FL & F_ENERGY) == 0) {
      for (int d = 0; d < 3; ++d) {
        if constexpr (MIXED) F[d] = (double)P.fq[j + d * P.n] * T.inv_fscale;
        else F[d] = P.fp[j + d * P.n];
      }
      if constexpr ((FL & F_PAIRONLY) == 0) {
        for (int d = 0; d < 3; ++d) {
          if constexpr (MIXED) F[d] += (double)S->fq[s][d] * (1.0 / 4294967296.0);
          else F[d] += S->fd[s][d];
        }
      }
    }
    if constexpr ((FL & F_PAIRONLY) == 0) {
      for (int t = 0; t < S->n && !S->nanocore; ++t) {  // BEAD sphere-sphere terms
        if (t == s) continue;
        double d[3];
        int tt;
        if constexpr (MIXED) {
          const uint4 a = pos_s[s], b = pos_s[t];
          tt = b.w & 0xff;
          d[0] = frac_delta_d(a.x, b.x, box[0] * (1.0 / 4294967296.0));
          d[1] = frac_delta_d(a.y, b.y, box[1] * (1.0 / 4294967296.0));
          d[2] = frac_delta_d(a.z, b.z, box[2] * (1.0 / 4294967296.0));
        } else {
          const double4 a = pos_s[s], b = pos_s[t];
          tt = __double_as_longlong(b.w) & 0xff;
          d[0] = a.x - b.x;
          d[1] = a.y - b.y;
          d[2] = a.z - b.z;
          for (int q = 0; q < 3; ++q) {
            if (d[q] > box[q] / 2.0) d[q] -= box[q];
            if (d[q] < -box[q] / 2.0) d[q] += box[q];
          }
        }
        // the pair's row is (type of the earlier bead of the residue, later)
        const double* row = P.sphC + kBeadConst * ((s < t) ? (ti * T.nT + tt) : (tt * T.nT + ti));
        const double dr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if constexpr ((FL & F_ENERGY) == 0) {
          const double mag = beadbead_mag(dr2, row, S->bb_cut2);
          for (int q = 0; q < 3; ++q) F[q] += mag * d[q];
        }
        if (t > s) {
          if constexpr ((FL & F_ENERGY) != 0) e += beadbead_pot(dr2, row, S->bb_cut2);
          if constexpr ((FL & F_DU) != 0) {
            const double e0 = d[0] * rs.scale[0], e1 = d[1] * rs.scale[1], e2 = d[2] * rs.scale[2];
            du += beadbead_pot(dr2, row, S->bb_cut2) - beadbead_pot(e0 * e0 + e1 * e1 + e2 * e2, row, S->bb_cut2);
          }
        }
      }
    }
    if constexpr ((FL & F_FORCES) != 0) {
      for (int d = 0; d < 3; ++d) P.force_out[3 * o + d] = F[d];
    } else if constexpr ((FL & F_ENERGY) == 0) {
      double noise[3];
      if constexpr ((FL & F_EXTNOISE) != 0) {
        for (int d = 0; d < 3; ++d) noise[d] = rp.sigma * P.ext_noise[3 * o + d];
      } else {
        langevin_noise(rp.seed, o - rp.bead_begin, it, (FL & F_INIT) ? 1 : 0, rp.sig31, noise);
      }
      double v[3] = {P.vx[j], P.vy[j], P.vz[j]};
      double a[3];
      for (int d = 0; d < 3; ++d) a[d] = fma(-rp.gamma, v[d], F[d]) + noise[d];
      const double m = S->mass[s], h = rp.dt * 0.5;
      if constexpr ((FL & (F_STOP | F_INIT)) != 0) {
        P.ax[j] = a[0];
        P.ay[j] = a[1];
        P.az[j] = a[2];
        if constexpr ((FL & F_STOP) != 0) {
          if (ti != 0) {
            P.vx[j] = fma(a[0] / m, h, v[0]);
            P.vy[j] = fma(a[1] / m, h, v[1]);
            P.vz[j] = fma(a[2] / m, h, v[2]);
          }
        }
      } else {
        double x[3] = {P.x[j], P.y[j], P.z[j]};
        if (ti != 0) {
          for (int d = 0; d < 3; ++d) {
            // the next first() half-kick: a BEAD sphere's divided again, a core's not
            const double a1 = a[d] / m, a2 = S->nanocore ? a1 : a1 / m;
            if constexpr (MIXED) {
              v[d] = fma(a2, h, fma(a1, h, v[d]));
              x[d] = fma(v[d], rp.dt, x[d]);
            } else {
              v[d] += a1 * h;
              v[d] += a2 * h;
              x[d] += v[d] * rp.dt;
            }
            if (x[d] > box[d]) x[d] -= box[d];
            if (x[d] < 0) x[d] += box[d];
          }
          P.vx[j] = v[0];
          P.vy[j] = v[1];
          P.vz[j] = v[2];
          P.x[j] = x[0];
          P.y[j] = x[1];
          P.z[j] = x[2];
        }
        const unsigned int fx = to_frac(x[0], rs.frac_per_len[0]), fy = to_frac(x[1], rs.frac_per_len[1]),
                           fz = to_frac(x[2], rs.frac_per_len[2]);
        vmax = displacement(P.ref[j], fx, fy, fz, rs);
        if constexpr (MIXED) P.m4[cur ^ 1][j] = make_uint4(fx, fy, fz, pos_s[s].w);
        else P.d4[cur ^ 1][j] = make_double4(x[0], x[1], x[2], pos_s[s].w);
      }
    }
  }
  // each thread has read its own accumulator: clear it for the next pass
  if (s < S->n)
    for (int d = 0; d < 3; ++d) {
      S->fq[s][d] = 0;
      S->fd[s][d] = 0.0;
    }
  // block sums in a fixed order (warps, then warp 0 over them)
  __shared__ double red_d[kMaxSpheres / 32];
  __shared__ long long red_q[kMaxSpheres / 32];
  __shared__ float red_f[kMaxSpheres / 32];
  const int lane = s & 31, warp = s >> 5, nw = blockDim.x >> 5;
  if constexpr ((FL & F_ENERGY) != 0) {
    e = warp_sum(e);
    if (lane == 0) red_d[warp] = e;
    __syncthreads();
    if (s == 0) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += red_d[w];
      if (t != 0.0) atomicAdd(&P.rs[0].e_sphere, t);
    }
  }
  if constexpr ((FL & F_DU) != 0) {
    if constexpr (MIXED) {
      long long q = __double2ll_rn(du * 4294967296.0);
#pragma unroll
      for (int w = 16; w > 0; w >>= 1) q += __shfl_xor_sync(0xffffffffu, q, w);
      if (lane == 0) red_q[warp] = q;
      __syncthreads();
      if (s == 0) {
        long long t = 0;
        for (int w = 0; w < nw; ++w) t += red_q[w];
        if (t != 0) atomicAdd((unsigned long long*)&P.rs[0].dUq_bond, (unsigned long long)t);
      }
    } else {
      du = warp_sum(du);
      if (lane == 0) red_d[warp] = du;
      __syncthreads();
      if (s == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += red_d[w];
        if (t != 0.0) atomicAdd(&P.rs[0].dU_bond, t);
      }
    }
  }
  if constexpr ((FL & (F_STOP | F_INIT | F_FORCES | F_ENERGY)) == 0) {
    vmax = warp_max(vmax);
    if (lane == 0) red_f[warp] = vmax;
    __syncthreads();
    float bm = 0.f;
    if (s == 0)
      for (int w = 0; w < nw; ++w) bm = fmaxf(bm, red_f[w]);
    finalize_step(P, bm, se);
  }
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
    P.m4[cur][i] = make_uint4(to_frac(P.x[i], rs.frac_per_len[0]), to_frac(P.y[i], rs.frac_per_len[1]),
                              to_frac(P.z[i], rs.frac_per_len[2]), me.w);
  } else {
    const double4 me = P.d4[cur][i];
    P.d4[cur][i] = make_double4(P.x[i], P.y[i], P.z[i], me.w);
  }
}

// State in file order (x0 y0 z0 x1 ..., the order of the input's beads) from
// the sorted device arrays: a gather through orig, so the host copy is one
// contiguous block per array.  Either output may be null.
__global__ void __launch_bounds__(kBlock) k_state_save(DevPtrs P, double* xs, double* vs) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int o = P.orig[i];
  if (xs) {
    xs[3 * o] = P.x[i];
    xs[3 * o + 1] = P.y[i];
    xs[3 * o + 2] = P.z[i];
  }
  if (vs) {
    vs[3 * o] = P.vx[i];
    vs[3 * o + 1] = P.vy[i];
    vs[3 * o + 2] = P.vz[i];
  }
}

// The inverse scatter: file-order positions and / or velocities into the
// sorted device arrays (the caller refreshes the mirror after positions).
// Checks a state staged for smd_set_state (file order): every position
// inside its replica's box and every velocity finite, else bit 2 of the
// error word.  It runs before the state is loaded, so a refused state
// leaves the handle's own untouched.
__global__ void __launch_bounds__(kBlock) k_state_check(DevPtrs P, const double* xs, const double* vs) {
  const int o = blockIdx.x * kBlock + threadIdx.x;
  if (o >= P.n) return;
  bool bad = false;
  if (xs) {
    const RepState& rs = P.rs[rep_of(P, o)];
    for (int k = 0; k < 3; ++k) {
      const double x = xs[3 * o + k];
      bad = bad || !(x >= 0.0 && x <= rs.box[k]);
    }
  }
  if (vs)
    for (int k = 0; k < 3; ++k) bad = bad || !isfinite(vs[3 * o + k]);
  if (bad) atomicOr(&P.g->error, 4);
}

__global__ void __launch_bounds__(kBlock) k_state_load(DevPtrs P, const double* xs, const double* vs) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int o = P.orig[i];
  if (xs) {
    P.x[i] = xs[3 * o];
    P.y[i] = xs[3 * o + 1];
    P.z[i] = xs[3 * o + 2];
  }
  if (vs) {
    P.vx[i] = vs[3 * o];
    P.vy[i] = vs[3 * o + 1];
    P.vz[i] = vs[3 * o + 2];
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
    const int j = P.nbr[(size_t)i * P.kmax + k];
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

// ------------------------------------------------------------ measurement
// Displacement since diffusion tracking started, file order: the reference's
// absolute positions aP advance by v dt in every first() for beads of nonzero
// type (include/algorithms/verlet.h:317-326) and box moves do not rescale
// them (MD.cpp:555), so aP - aPStart (dataExtraction.h:790-800, 1524-1650) is
// the sum of the drifts since the start.  Runs after every drift while
// tracking: v is the half-step velocity the drift used.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_track(DevPtrs P, int cur) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  int ti;
  if constexpr (MIXED) ti = P.m4[cur][i].w & 0xff; else ti = __double_as_longlong(P.d4[cur][i].w) & 0xff;
  if (ti == 0) return;
  const double dt = P.rp[rep_of(P, i)].dt;
  double* d = P.disp + 3 * (size_t)P.orig[i];
  d[0] = __dadd_rn(d[0], __dmul_rn(P.vx[i], dt));
  d[1] = __dadd_rn(d[1], __dmul_rn(P.vy[i], dt));
  d[2] = __dadd_rn(d[2], __dmul_rn(P.vz[i], dt));
}

__device__ __forceinline__ double measure_wrap(double d, double L) {
  if (d >= L / 2.0) d -= L;
  if (d <= -L / 2.0) d += L;
  return d;
}
__device__ __forceinline__ double dot_rn(const double a[3], const double b[3]) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

// One measure step's reductions on the stopped state (positions of the step,
// velocities after its second half-kick), with the reference's expressions
// rounded alike (no contraction into FMA): sum v^2/2 (Kinetic::compute,
// include/algorithms/dataCollection.h:666-674), the smallest and largest
// coordinate per axis (dataExtraction.h:1456-1488), BOND lengths and BEND
// angles of the BOND / BEND residues (dataExtraction.h:860-940), and each
// bead's kinetic-energy bin int(0.5 v^2 / 1e-4) into the run's histogram
// (dataExtraction.h:1509-1519).  Single-system handles.
__global__ void __launch_bounds__(kBlock) k_measure(DevPtrs P, MeasureAcc* acc, unsigned int* hist, int cap) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  double ke = 0.0, lb = 0.0, cb = 0.0, l0 = 0.0, l1 = 0.0;
  int nb = 0, ne = 0;
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
  if (i < P.n) {
    const double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
    const double v2 = dot_rn(v, v);
    ke = __ddiv_rn(v2, 2.0);
    const int bin = (int)__ddiv_rn(__dmul_rn(0.5, v2), 0.0001);
    if (bin >= 0 && bin < cap) atomicAdd(hist + bin, 1u);
    else atomicMax(&acc->max_bin, bin < 0 ? 0x7fffffff : bin);
    const double x[3] = {P.x[i], P.y[i], P.z[i]};
    for (int d = 0; d < 3; ++d) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(x[d] + 0.0);  // -0 -> +0
      lo[d] = b;
      hi[d] = b;
    }
    const RepState& rs = P.rs[0];
    const int o = P.orig[i];
    if (P.n_terms > 0) {
      for (int k = P.term_off[o]; k < P.term_off[o + 1]; ++k) {
        const int4 t = P.terms[k];
        if (term_role(t.x) != 0) continue;
        const int kind = term_kind(t.x);
        if (kind != kTermBond && kind != kTermBend) continue;
        const int a = P.inv[t.y], b = P.inv[t.z];
        const double pa[3] = {P.x[a], P.y[a], P.z[a]}, pb[3] = {P.x[b], P.y[b], P.z[b]};
        double da[3];
        for (int d = 0; d < 3; ++d) da[d] = measure_wrap(pa[d] - pb[d], rs.box[d]);
        if (kind == kTermBond) {
          lb += sqrt(dot_rn(da, da));
          ++nb;
        } else {
          const int c = P.inv[t.w];
          const double pc[3] = {P.x[c], P.y[c], P.z[c]};
          double db[3];
          for (int d = 0; d < 3; ++d) db[d] = measure_wrap(pb[d] - pc[d], rs.box[d]);
          const double ra = sqrt(dot_rn(da, da)), rb = sqrt(dot_rn(db, db));
          l0 += ra;
          l1 += rb;
          cb += __ddiv_rn(dot_rn(da, db), __dmul_rn(ra, rb));
          ++ne;
        }
      }
    }
  }
  // block reductions, then one atomic per block and quantity
  __shared__ double sh[kBlock / 32];
  block_sum_atomic(ke, &acc->kinetic, sh);
  if (P.n_terms > 0) {
    block_sum_atomic(lb, &acc->lbond, sh);
    block_sum_atomic(cb, &acc->cos_bend, sh);
    block_sum_atomic(l0, &acc->l_bend0, sh);
    block_sum_atomic(l1, &acc->l_bend1, sh);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
    for (int d = 0; d < 3; ++d) {
      lo[d] = min(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = max(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    if (nb) atomicAdd(&acc->n_bond, nb);
    if (ne) atomicAdd(&acc->n_bend, ne);
    for (int d = 0; d < 3; ++d) {
      atomicMin(&acc->lo[d], lo[d]);
      atomicMax(&acc->hi[d], hi[d]);
    }
  }
}

// Kinetic-energy bins of a measure step that fell beyond the histogram's
// previous capacity [from, cap), after the histogram has grown.
__global__ void __launch_bounds__(kBlock) k_measure_bins(DevPtrs P, unsigned int* hist, int from, int cap) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const double v[3] = {P.vx[i], P.vy[i], P.vz[i]};
  const int bin = (int)__ddiv_rn(__dmul_rn(0.5, dot_rn(v, v)), 0.0001);
  if (bin >= from && bin < cap) atomicAdd(hist + bin, 1u);
}

// Sum of squared displacements of each measurement group (blockIdx.y): the
// entries [off[g], off[g+1]) of file-order beads, kMsdChunk per block.
constexpr int kMsdChunk = 4096;
__global__ void __launch_bounds__(kBlock) k_msd(DevPtrs P, const int* off, const int* beads, double* out) {
  const int g = blockIdx.y;
  const int a = off[g] + blockIdx.x * kMsdChunk, e = min(off[g + 1], a + kMsdChunk);
  double s = 0.0;
  for (int k = a + (int)threadIdx.x; k < e; k += kBlock) {
    const double* d = P.disp + 3 * (size_t)beads[k];
    const double dd[3] = {d[0], d[1], d[2]};
    s += dot_rn(dd, dd);
  }
  __shared__ double sh[kBlock / 32];
  block_sum_atomic(s, out + g, sh);
}

}  // namespace smd
