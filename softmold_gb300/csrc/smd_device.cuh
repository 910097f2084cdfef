// Device data layout and kernels of the GB300 membrane MD step.
//
// Per-bead state lives in HBM in cell-sorted order (beads of one replica are
// contiguous; within a replica they are ordered by Verlet-list cell), FP64 SoA:
//   x,y,z  vx,vy,vz  ax,ay,az        master state (8 B each)
//   mirror[2]                        double-buffered 16 B position mirror read
//                                    by the pair loop: MIXED = uint4 of 32-bit
//                                    fractional coordinates + (type | replica<<8),
//                                    PLAIN = double4 (x,y,z,type bits)
//   orig / inv                       sorted -> file order and back
//   cinfo                            CHAIN role of the bead (position, length, set)
// The Verlet list is bead-major: nbr[i * kmax + k] is neighbour k of bead i.
// Between the two passes of a step the non-bonded force of each bead is held
// as int64 fixed point (MIXED, fq) or FP64 (PLAIN, fp), SoA x | y | z.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace smd {

constexpr int kMaxTypes = 8;
constexpr int kMaxChainSets = 32;
constexpr int kMaxTermSets = 64;  // distinct constant pairs of BOND / BEND residues
constexpr int kMaxFieldSets = 64; // distinct constant sets of external-field terms
constexpr int kFieldConst = 8;    // constants per external-field term set

// Residue term entries (per bead, file order): x = kind | role << 3 | set << 5,
// then the term's beads (file order; -1 where absent).  role: the bead's place
// in the term.  Sets index termD/termF (BOND, BEND) or fieldD (the rest).
enum TermKind {
  kTermBond = 0, kTermBend = 1,        // BOND {first, second}, BEND {first, second, third}
  kTermBoundary = 2, kTermFloating = 3, // BOUNDARY {bead}, FLOATING_BASE {bead}
  kTermZTorque = 4, kTermZPower = 5,    // ZTORQUE {first, second}, ZPOWERPOTENTIAL {bead}
  kTermBall = 6                         // BALL {centre, second}
};
__host__ __device__ inline int term_pack(int kind, int role, int set) { return kind | (role << 3) | (set << 5); }
__host__ __device__ inline int term_kind(int x) { return x & 7; }
__host__ __device__ inline int term_role(int x) { return (x >> 3) & 3; }
__host__ __device__ inline int term_set(int x) { return x >> 5; }
constexpr int kBlock = 256;
// threads per CTA of the per-bead step kernels (bin, reorder, integrator):
// small CTAs spread a small system over every SM
constexpr int kBeadBlock = 128;
constexpr int kScanTile = 2048;  // cells per scan block (256 threads x 8)
constexpr long long kMaxGridCells = 1LL << 28;  // list cells of one handle, all replicas together
constexpr int kLanes = 8;        // lanes per bead in the list build and the pair pass
constexpr int kMaxSpheres = 256; // BEAD or NANOCORE beads of one handle (one k_sphere block)
constexpr int kBeadBrute = 20;   // BEAD residues up to this size take the brute-force branch
constexpr int kCoreBrute = 49;   // NANOCORE residues up to this size take the brute-force branch
constexpr int kBeadConst = 22;   // constants per ordered type pair of a BEAD residue (nBEADCONST)
constexpr int kBeadBeadOff = 11; // BEADBEADOFFSET: bead-bead constants within a row

// cinfo word: bit 31 chain member, bits 0..11 position in chain, bits 12..23
// chain length, bits 24..28 chain-constant set; bit 30 marks a BEAD sphere.
__host__ __device__ inline int cinfo_pack(int p, int len, int set) {
  return (int)(0x80000000u | (unsigned)(p & 0xfff) | ((unsigned)(len & 0xfff) << 12) |
               ((unsigned)(set & 0x1f) << 24));
}

struct RepParams {  // per replica, fixed
  double dt, gamma, kT, sigma, tension, dlxy;
  double sig31;      // sigma * 2^-31: noise amplitude per unit of a signed 32-bit draw
  float sig31f;      // the same in FP32 (the mixed form's noise is a force term, FP32)
  uint32_t seed;
  int resize_rate;
  int bead_begin, bead_end;
  int cell_begin, cell_cap;
};

// BEAD residue of a single-system handle (include/system.h:2043-2212), or a
// NANOCORE residue (:2216-2263, each core with its own 22-constant row): the
// spheres' file-order indices, masses 4 pi R^2 (MD.cpp:280-303, 340-355) and
// the sums of the other beads' reactions on each sphere, gathered during
// k_integ and used by k_sphere.  MIXED sums are int64 in units of 2^-32
// (order-independent).
//
// Which partners a sphere's force takes follows the reference's two branches.
// Brute force (BEAD up to 20 beads, NANOCORE up to 49 cores): every bead
// except the residue's own spheres (BEAD, system.h:2165-2210) or except the
// core itself (NANOCORE, :2221-2261).  Hash cells (more beads or cores,
// :2104-2163 and :2264-2318): every bead except the sphere itself, found
// through cells of side box / int(box / grid_len) and their 27 periodic
// neighbours, so that along an axis of one cell every neighbour is the same
// cell (visited 3 times) and along an axis of two cells the other cell is
// visited twice.  Energies and size-change differences take every bead except
// the sphere itself in both branches (:2936-3074, 3584-3700).
struct SphereDev {
  int n;
  int nanocore;     // 1: a NANOCORE residue (per-sphere rows, no sphere-sphere term, no dU)
  int all_partners; // 1: forces between spheres as bead partners (NANOCORE; BEAD hash-cell branch)
  int grid;         // 1: the hash-cell branch, whose repeated neighbour cells multiply terms
  double grid_len;  // cell side floor: BEAD 2 C[0]; NANOCORE 2 int(max C[0]) (system.h:2265-2277)
  int orig[kMaxSpheres];
  double mass[kMaxSpheres];   // 4 pi R^2 of each sphere
  double cut2[kMaxSpheres];   // bead-sphere range of each sphere (its row's constant 0, squared)
  double bb_cut2;   // (2R + 2)^2: sphere-sphere range (BEAD)
  long long fq[kMaxSpheres][3];
  double fd[kMaxSpheres][3];
};

struct RepState {  // per replica, updated on the device
  double box[3];
  double frac_per_len[3];  // 2^32 / box: real -> 32-bit fractional coordinate
  float len_per_frac[3];   // box / 2^32
  float pad_f;
  double trial_box[3];
  double scale[3];   // scale of the last accepted / current trial
  float sq_f[3];     // fma(scale, scale, -1) in FP32, set with scale (the mixed size-change terms)
  float pad_sq;
  double dU_pair, dU_bond;  // FP64 form: U(x) - U(s x) summed in any order
  long long dUq_pair, dUq_bond;  // mixed form: the same in units of 2^-32, summed exactly
  double e_pair, e_bond, e_kin, e_sphere;
  double last_dU;
  long long n_trial, n_accept;
  int accept;
  int ncell[3];
  int refn[3];       // the reference's cells per axis, int(L / rc) (the size-change passes' grid)
  int pad;
  double ref_cs[3];  // its cell sides L / refn
  float ref_inv_cs[3];
  float pad_r;
};

// Sets a replica's trial scale and its FP32 factors s^2 - 1 (one rounding of
// the exact s^2 - 1, on the host and the device alike).
__host__ __device__ inline void set_scale(RepState& rs, const double s[3]) {
  for (int d = 0; d < 3; ++d) {
    rs.scale[d] = s[d];
    rs.sq_f[d] = (float)fma(s[d], s[d], -1.0);
  }
}

// Size-change energy of a replica's current trial.  The mixed form rounds
// each pair term (once per pair) and each bead's bonded term to 2^-32 before
// summing, so the total, and with it every Metropolis decision, is the same
// whatever the pair order or the replicas sharing a launch.
__host__ __device__ inline double rep_dU(const RepState& rs) {
  const double q = (double)rs.dUq_pair + (double)rs.dUq_bond;
  return rs.dU_pair + rs.dU_bond + q * (1.0 / 4294967296.0);
}

struct Global {  // single instance
  double slack;                // list-distance slack used up by accepted box moves since the build
  unsigned long long mc_shift; // slack of this step's accepted box moves (double bits, max over replicas)
  long long n_rebuilds;
  unsigned int dmax_bits;      // largest bead displacement from its build position (float bits)
  float last_disp;
  unsigned int blocks_done;    // last-block counter
  int rebuild;                 // 1: rebuild the Verlet list before the next force pass
  int error;                   // bit 0: list overflow, bit 1: cell overflow (>kMaxCell), bit 2: refused set_state input
  int need_nbr;                // largest neighbour count seen on overflow
  int max_nbr;                 // largest neighbour count of any list build so far
  int trial_slot;              // staged barostat trial used by the next MC step
  long long it;                // loop step (the Langevin noise key); advanced by the step's last kernel
  long long graph_builds;      // list builds run inside graph conditional bodies
  int n_occ;                   // occupied list cells of the current build
  int next_cell;               // work queue of the list kernels over occ[]
};

// Bookkeeping of the kernel that completes a step (its last block): advance
// the step counter and the trial slot, and in a graph hand the rebuild
// decision to the next step's conditional node.
struct StepEnd {
  unsigned long long cond;  // cudaGraphConditionalHandle of the next step's rebuild node
  int set_cond;
  int advance_it;
  int advance_slot;
  int pad;
};

struct Tables {  // force/potential tables (float and double) in constant-like memory
  int nT;
  int n_sets;
  float rc2f, rcf;
  double rc2, rc;
  double list_cut2;  // (rc+skin)^2
  double list_cut;
  float list_cut_f;
  float fscale;      // fixed-point scale of one pair force (2^k)
  double inv_fscale;
  float fF[6 * kMaxTypes * kMaxTypes];
  float fU[6 * kMaxTypes * kMaxTypes];
  double dF[6 * kMaxTypes * kMaxTypes];
  double dU[6 * kMaxTypes * kMaxTypes];
  float chainF[kMaxChainSets][4];
  double chainD[kMaxChainSets][4];
  float termF[kMaxTermSets][2];   // BOND {l0, k} / BEND {a, k} constant sets
  double termD[kMaxTermSets][2];
  double fieldD[kMaxFieldSets][kFieldConst];  // external-field term constants (FP64)
};

// Reductions of one measure step (single-system handles): positions enter as
// the bit patterns of non-negative doubles, which order as unsigned integers.
struct MeasureAcc {
  double kinetic;
  unsigned long long lo[3], hi[3];
  double lbond;
  double cos_bend, l_bend0, l_bend1;
  int n_bond, n_bend;
  int max_bin;  // largest kinetic-energy bin beyond the histogram's capacity (-1: none)
  int pad;
};

// All device pointers of one handle.
struct DevPtrs {
  int n, npad, n_rep, kmax, n_cells_total;
  double half_skin;
  double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az;
  uint4* m4[2];
  double4* d4[2];
  uint4* ref;        // fractional position of each bead at the last list build
  int *orig, *inv, *cinfo;
  // rebuild scratch
  uint4* mt;
  double4* dt4;
  double *tx, *ty, *tz, *tvx, *tvy, *tvz, *tax, *tay, *taz;
  int *torig, *tcinfo;
  int *key, *slot, *tkey;
  int *cell_count, *cell_start, *block_sums;
  int* occ;          // occupied list cells of the last build (count in Global::n_occ)
  int *nbr, *nnbr;
  long long* fq;     // MIXED pair force, fixed point, 3*n (x | y | z)
  double* fp;        // PLAIN pair force, 3*n
  RepParams* rp;
  RepState* rs;
  Global* g;
  const Tables* tab;
  double* trial_u;   // 2 draws per barostat trial, per replica: [trial][rep][2]
  int* accept_log;   // decision of each staged trial: [trial][rep]
  double* ext_noise; // n*3 noise in sorted order (test hook)
  double* force_out; // n*3 scratch for host reads (file order)
  int* key_out;
  unsigned long long* refcell;  // reference-grid cell of each bead (sorted order, x | y << 21 | z << 42),
                                // set before each size-change pass
  double* disp;      // n*3 displacement since diffusion tracking started (file order; null: not tracking)
  // BOND / BEND residue terms of each bead, file order: entries
  // terms[term_off[o] .. term_off[o+1]) of bead o; an entry is {kind | role<<1
  // | set<<3, first, second, third} (kind 0 bond, 1 bend; role = the bead's
  // position in the term; global bead indices, third -1 for a bond)
  int n_terms;
  const int* term_off;
  const int4* terms;
  int n_sph;         // BEAD beads (0: none)
  SphereDev* sph;
  const double* sphC;  // kBeadConst * nT^2 BEAD constants
  const float* sphCf;  // the same in FP32
};

// ------------------------------------------------------------------ helpers
// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while the kernel before it drains: it calls
// pdl_wait() before reading anything that kernel wrote (the wait returns once
// that grid has completed and its writes are visible).  The kernel before it
// calls pdl_trigger() to let it launch early.  Both are no-ops in an ordinary
// launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ int rep_of(const DevPtrs& P, int i) {
  // replicas are contiguous ranges; linear scan is fine for the few replicas
  // of a batch, binary search for many.
  int lo = 0, hi = P.n_rep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (P.rp[mid].bead_begin <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// CellOpt cell coordinate: int(p/cellSize) with the x>=n -> n-1 correction
// (include/algorithms/cellOpt.h:532-539).  IEEE FP64 division, no fast-math.
__device__ __forceinline__ int cell_coord(double p, double cs, int n) {
  int c = int(p / cs);
  c = (c >= n) ? c - 1 : c;
  return c;
}

// Cell coordinate on the Verlet-list grid, clamped into [0, n) so that a bead
// outside the box (a blown-up run) can never index outside the cell arrays.
__device__ __forceinline__ int list_cell_coord(double p, double cs, int n) {
  int c = cell_coord(p, cs, n);
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

__device__ __forceinline__ unsigned int to_frac(double x, double frac_per_len) {
  // 32-bit fractional coordinate; x == L wraps to 0 like any periodic image.
  return (unsigned int)(long long)(x * frac_per_len);
}

// Derived box quantities of a replica: fractional scales, the Verlet-list
// grid (cells of at least list_cut, at most cap cells) and the reference's
// cell grid (cells of at least rc).  Computed on the host
// at creation and on the device when a box move is accepted; the same IEEE
// arithmetic gives the same grid on both.
__host__ __device__ inline void derive_box(RepState& rs, int cap, double list_cut, double rc) {
  for (int d = 0; d < 3; ++d) {
    rs.frac_per_len[d] = 4294967296.0 / rs.box[d];
    rs.len_per_frac[d] = (float)(rs.box[d] * (1.0 / 4294967296.0));
    int n = int(rs.box[d] / list_cut);
    rs.ncell[d] = n < 1 ? 1 : n;
    const int m = int(rs.box[d] / rc);
    rs.refn[d] = m < 1 ? 1 : m;
    rs.ref_cs[d] = rs.box[d] / rs.refn[d];
    rs.ref_inv_cs[d] = (float)(1.0 / rs.ref_cs[d]);
  }
  while ((long long)rs.ncell[0] * rs.ncell[1] * rs.ncell[2] > cap) {
    int m = 0;
    if (rs.ncell[1] > rs.ncell[m]) m = 1;
    if (rs.ncell[2] > rs.ncell[m]) m = 2;
    rs.ncell[m]--;
  }
}

__device__ __forceinline__ float frac_delta(unsigned int a, unsigned int b, float scale) {
  return (float)(int)(a - b) * scale;  // two's-complement wrap = minimum image
}

__device__ __forceinline__ double frac_delta_d(unsigned int a, unsigned int b, double scale) {
  return (double)(int)(a - b) * scale;
}

// Philox4x32-10 counter-based generator (J. K. Salmon, M. A. Moraes,
// R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11), restated from the publication.
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned int hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const unsigned int hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Langevin noise sigma*psi with psi uniform in (-1,1) (the reference draws
// 2u-1, include/algorithms/langevin.h:309-314) for bead `orig` (index within
// its replica) at loop step `it`; phase 1 is the start-up thermostat call.
// The stream depends on the replica's seed only, not on its position in a
// batch, so a replica evolves the same alone or batched.  A draw r gives
// psi = (signed(r - 2^31) + 1/2) 2^-31, so sigma*psi is one FMA with
// sig31 = sigma 2^-31.
__device__ __forceinline__ void langevin_noise(uint32_t seed, int orig, long long it, int phase, double sig31,
                                               double out[3]) {
  const uint4 c = make_uint4((unsigned)orig, (unsigned)(it & 0xffffffff),
                             (unsigned)((unsigned long long)it >> 32) ^ ((unsigned)phase << 31), 0x6D2Bu);
  const uint4 r = philox4x32(c, make_uint2(seed, 0x5A17u));
  const double half = 0.5 * sig31;
  out[0] = fma((double)(int)(r.x ^ 0x80000000u), sig31, half);
  out[1] = fma((double)(int)(r.y ^ 0x80000000u), sig31, half);
  out[2] = fma((double)(int)(r.z ^ 0x80000000u), sig31, half);
}

// The same draws in FP32 for the mixed form, where the noise is summed with
// the other FP32 force terms: psi keeps 24 of its 32 bits.
__device__ __forceinline__ void langevin_noise_f(uint32_t seed, int orig, long long it, int phase, float sig31f,
                                                 float out[3]) {
  const uint4 c = make_uint4((unsigned)orig, (unsigned)(it & 0xffffffff),
                             (unsigned)((unsigned long long)it >> 32) ^ ((unsigned)phase << 31), 0x6D2Bu);
  const uint4 r = philox4x32(c, make_uint2(seed, 0x5A17u));
  const float half = 0.5f * sig31f;
  out[0] = fmaf((float)(int)(r.x ^ 0x80000000u), sig31f, half);
  out[1] = fmaf((float)(int)(r.y ^ 0x80000000u), sig31f, half);
  out[2] = fmaf((float)(int)(r.z ^ 0x80000000u), sig31f, half);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of a per-thread double into *dst (one atomic per block).
__device__ __forceinline__ void block_sum_atomic(double v, double* dst, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0 && t != 0.0) atomicAdd(dst, t);
  }
  __syncthreads();
}

// Box of replica r after the MC trial drawn from u1 (MD.cpp:593-611).
__device__ __forceinline__ void trial_box(const double box[3], double dlxy, double u1, double nb[3],
                                          double s[3]) {
  const double fx = dlxy * (2.0 * u1 - 1.0), fy = fx;
  const double fz = (box[0] * box[1]) / ((box[0] + fx) * (box[1] + fy));
  nb[0] = box[0] + fx;
  nb[1] = box[1] + fy;
  nb[2] = box[2] * fz;
  s[0] = nb[0] / box[0];
  s[1] = nb[1] / box[1];
  s[2] = nb[2] / box[2];
}

// ------------------------------------------------------------------ potentials
// Pair force magnitude with the reference's table index trick
// (include/MD.h:811-825): force on i = mag * d.
template <typename R>
__device__ __forceinline__ R pair_mag(const R* c, R r) {
  int ci = int(r / c[0]) * 3;
  ci = ci > 3 ? 3 : ci;  // rows hold two segments; the tables use rc = 2 rm
  R m = c[ci] - r;
  return ((c[ci + 1] - c[ci + 2] * m) * m) / r;
}
// Pair potential (include/MD.h:913-926).
template <typename R>
__device__ __forceinline__ R pair_pot(const R* c, R r) {
  if (r <= c[0]) {
    const R m = c[0] - r;
    return c[1] * m * m + c[2];
  }
  const R m = c[3] - r;
  return m * m * (c[4] - m * c[5]);
}
// U(r) - U(r') with r' = r + dr, written so that a small dr does not cancel:
// each branch's polynomial difference is factored through dr.  rc bounds the
// interaction range of both arguments.  Every operation is rounded
// explicitly (no contraction left to the compiler), so a pair's term has the
// same bits wherever it is evaluated.
__device__ __forceinline__ float pot_f(const float* c, float r) {
  if (r <= c[0]) {
    const float m = __fsub_rn(c[0], r);
    return __fmaf_rn(__fmul_rn(c[1], m), m, c[2]);
  }
  const float m = __fsub_rn(c[3], r);
  return __fmul_rn(__fmul_rn(m, m), __fmaf_rn(-m, c[5], c[4]));
}
__device__ __forceinline__ float pair_dpot_f(const float* c, float r, float rn, float dr, float rc) {
  const bool in0 = r < rc, in1 = rn < rc;
  if (!in0 && !in1) return 0.f;
  if (in0 && in1 && ((r <= c[0]) == (rn <= c[0]))) {
    if (r <= c[0]) {
      // C1[(rm-r)^2-(rm-r')^2] = C1 dr (2 rm - r - r')
      return __fmul_rn(__fmul_rn(c[1], dr), __fsub_rn(__fsub_rn(__fmul_rn(2.f, c[0]), r), rn));
    }
    const float m = __fsub_rn(c[3], r), mn = __fsub_rn(c[3], rn);  // mn = m - dr
    // m^2(C4 - C5 m) - mn^2(C4 - C5 mn) = dr[C4 (m+mn) - C5 (m^2 + m mn + mn^2)]
    const float sq = __fmaf_rn(mn, mn, __fmaf_rn(m, mn, __fmul_rn(m, m)));
    return __fmul_rn(dr, __fmaf_rn(-c[5], sq, __fmul_rn(c[4], __fadd_rn(m, mn))));
  }
  const float u0 = in0 ? pot_f(c, r) : 0.f;
  const float u1 = in1 ? pot_f(c, rn) : 0.f;
  return __fsub_rn(u0, u1);
}

// ------------------------------------------------------------------ BEAD
// Continuum sphere <-> bead force and potential (beadForce / beadPotential,
// include/MD.h:165-231) for d = x_sphere - x_bead and one 22-constant row C:
// an outer well on E = C0 - r for r >= C4 + C5 and an inner polynomial in
// B = C4 + C5 - r below it.  Returns mag with force mag*d on the sphere and
// -mag*d on the bead.
__device__ __forceinline__ double bead_mag(double dr2, const double* C, double cut2) {
  const double rminD = C[4] + C[5];
  const double rminD2 = rminD * rminD;
  double mag = 0.0;
  if (rminD2 <= dr2 && dr2 < cut2) {
    const double dr = sqrt(dr2);
    const double E = C[0] - dr, E2 = E * E, E3 = E * E2;
    mag = 2.0 * (0.4 * E3 + C[1] * E2 + C[2] * E) / (dr);
    mag += 4.0 * E2 + 8.0 * C[1] * E + 6.0 * C[2];
    mag *= (E2 * C[3]) / (dr * dr);
  } else if (dr2 < rminD2) {
    const double dr = sqrt(dr2);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
    mag = (B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
    mag += (4.0 * B3 * C[6] + 3.0 * B2 * C[7] + 2.0 * B * C[8] + C[9]);
    mag /= dr * dr;
  }
  return mag;
}
__device__ __forceinline__ double bead_pot(double dr2, const double* C, double cut2) {
  const double rminD = C[4] + C[5];
  const double rminD2 = rminD * rminD;
  if (rminD2 <= dr2 && dr2 < cut2) {
    const double dr = sqrt(dr2);
    const double E = C[0] - dr, E2 = E * E, E3 = E * E2;
    return 2.0 * E3 * (0.4 * E2 + C[1] * E + C[2]) * C[3] / (dr);
  } else if (dr2 < rminD2) {
    const double dr = sqrt(dr2);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
    return (B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
  }
  return 0.0;
}
// Sphere <-> sphere (beadBeadForce / beadBeadPotential, include/MD.h:233-338)
// from the row's constants at kBeadBeadOff; d = x_first - x_second, force
// mag*d on the first.
__device__ __forceinline__ double beadbead_mag(double dr2, const double* Cr, double cut2) {
  const double* C = Cr + kBeadBeadOff;
  const double rminD = C[0], rminD2 = rminD * rminD;
  double mag = 0.0;
  if (rminD2 <= dr2 && dr2 < cut2) {
    const double dr = sqrt(dr2);
    const double E = C[1] - dr, E2 = E * E, E3 = E * E2;
    mag = E3 * (6.0 * C[2] * E2 + 5.0 * C[3] * E + 4.0 * C[4] + (C[2] * E3 + C[3] * E2 + C[4] * E) / dr) /
          (dr * dr);
  } else if (dr2 < rminD2) {
    const double dr = sqrt(dr2);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2, B5 = B2 * B3;
    mag = 5.0 * B4 * C[5] + 4.0 * B3 * C[6] + 3.0 * B2 * C[7] + 2.0 * B * C[8] + C[9];
    mag += (B5 * C[5] + B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
    mag /= dr * dr;
  }
  return mag;
}
__device__ __forceinline__ double beadbead_pot(double dr2, const double* Cr, double cut2) {
  const double* C = Cr + kBeadBeadOff;
  const double rminD = C[0], rminD2 = rminD * rminD;
  if (rminD2 <= dr2 && dr2 < cut2) {
    const double dr = sqrt(dr2);
    const double E = C[1] - dr, E2 = E * E, E4 = E2 * E2;
    return E4 * (C[2] * E2 + C[3] * E + C[4]) / dr;
  } else if (dr2 < rminD2) {
    const double dr = sqrt(dr2);
    const double B = rminD - dr, B2 = B * B, B3 = B2 * B, B4 = B2 * B2, B5 = B2 * B3;
    return (B5 * C[5] + B4 * C[6] + B3 * C[7] + B2 * C[8] + B * C[9] + C[10]) / (dr);
  }
  return 0.0;
}

}  // namespace smd
