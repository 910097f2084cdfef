// Non-bonded forces without any device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while another framework
// owns the device memory through its own pool, or a latency-critical loop in
// which cudaMalloc's implicit device-wide synchronisation is not allowed.
// smd_pair_forces_static serves them: the caller passes device pointers for
// the inputs and the output, and the scratch of the cell list lives in the
// file-scope array below, reserved once on every GPU that loads the library
// (SMD_STATIC_MAX_BEADS / SMD_STATIC_MAX_CELLS bound what fits; about 640 KB).
//
// The array is shared by every call and keeps the last call's contents, so
// each call clears the cell counts before use; calls whose kernels overlap on
// the GPU (different streams, or different host threads on one device) race on
// it and must be serialised by the caller.  The first call on a device looks
// up the array's device address (cudaGetSymbolAddress); make that first call
// before any stream capture.  The cached address belongs to the CUDA context
// it was looked up in: after cudaDeviceReset of a device, this entry point
// must not be called on that device again in the same process.
//
// The inputs come from another framework and are not checked on the host.
// Every index the kernels derive from them stays inside the arrays whatever
// their values (smd_static_cell.h): cell coordinates are clamped into the
// grid and types are range-checked before any table lookup.  A bead whose
// position is not finite, or whose type or a neighbour's type is outside
// [0, n_types), gets a NaN force.  Positions must be wrapped into [0, L] for
// the forces to be those of the reference.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <atomic>
#include <cmath>
#include <string>

#include "../../include/softmold_gb300.h"
#include "smd_static_cell.h"

namespace smd {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kMaxBeads = SMD_STATIC_MAX_BEADS;
constexpr int kMaxCells = SMD_STATIC_MAX_CELLS;
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

// [cell counts | cell starts (+1) | bead keys | bead slots | sorted beads]
constexpr size_t kScratchInts = (size_t)kMaxCells + (kMaxCells + 1) + 3 * (size_t)kMaxBeads;
static __device__ __align__(256) int g_scratch[kScratchInts];

// Host side: device address of g_scratch, looked up once per device.  Two
// host threads making a first call on one device at the same time both look
// it up and store the same value.
std::atomic<int*> g_scratch_addr[kMaxDevices];

struct Grid {
  int n[3];
  double cs[3];
  double box[3];
};

__global__ void k_static_clear(int* count, int ncells) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) count[c] = 0;
}

// CellOpt key with the reference's formula (int(p/cellSize), x>=n -> n-1),
// clamped into the grid (smd_static_cell.h): the key is always < ncells.
__global__ void k_static_bin(const double* pos, int n, Grid g, int* key, int* slot, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
  int flags = 0;
  const int k = smd_static::cell_key(p, g.cs, g.n, &flags);
  key[i] = k;
  slot[i] = atomicAdd(&count[k], 1);
}

// Exclusive scan of the counts, one block.
__global__ void k_static_scan(const int* count, int* start, int ncells) {
  __shared__ int warp_sums[kThreads / 32];
  int carry = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < ncells; base += kThreads) {
    const int c = base + threadIdx.x;
    const int v = c < ncells ? count[c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    int before = 0, total = 0;
    for (int q = 0; q < kThreads / 32; ++q) {
      if (q < w) before += warp_sums[q];
      total += warp_sums[q];
    }
    if (c < ncells) start[c] = carry + before + x - v;
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) start[ncells] = carry;
}

__global__ void k_static_scatter(const int* key, const int* slot, const int* start, int* sorted, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sorted[start[key[i]] + slot[i]] = i;
}

// FP64 non-bonded force on bead i from the 27 surrounding cells, with the
// Force functor of include/MD.h:795-848 and the neighbour-shift minimum image.
// The table row is int(r/C0) (0 or 3 for the reference's tables, rc = 2 rm),
// taken as r/C0 >= 1 so that no table value can move the lookup outside the
// pair's 6 constants.  A bead with a non-finite position or a type outside
// [0, nT), or with a neighbour within rc whose type is outside it, gets NaN.
__global__ void k_static_force(const double* pos, const int* type, int n, Grid g, double rc2, int nT,
                               const double* fC, const int* key, const int* start, const int* sorted,
                               double* force) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = key[i];
  const int cx = k % g.n[0], cy = (k / g.n[0]) % g.n[1], cz = k / (g.n[0] * g.n[1]);
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const int ti = type[i];
  int flags = 0;
  {
    const double p[3] = {xi, yi, zi};
    smd_static::cell_key(p, g.cs, g.n, &flags);
    if (!smd_static::type_ok(ti, nT)) flags |= smd_static::kStaticBadType;
  }
  double fx = 0, fy = 0, fz = 0;
  if (flags == 0) {
    for (int oz = -1; oz <= 1; ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          const int c = ((cx + ox + g.n[0]) % g.n[0]) + ((cy + oy + g.n[1]) % g.n[1]) * g.n[0] +
                        ((cz + oz + g.n[2]) % g.n[2]) * g.n[0] * g.n[1];
          for (int q = start[c]; q < start[c + 1]; ++q) {
            const int j = sorted[q];
            if (j == i) continue;
            double px = pos[3 * j], py = pos[3 * j + 1], pz = pos[3 * j + 2];
            if (xi - px > g.box[0] / 2.0) px += g.box[0];
            if (xi - px < -g.box[0] / 2.0) px -= g.box[0];
            if (yi - py > g.box[1] / 2.0) py += g.box[1];
            if (yi - py < -g.box[1] / 2.0) py -= g.box[1];
            if (zi - pz > g.box[2] / 2.0) pz += g.box[2];
            if (zi - pz < -g.box[2] / 2.0) pz -= g.box[2];
            const double dx = xi - px, dy = yi - py, dz = zi - pz;
            double dr = dx * dx + dy * dy + dz * dz;
            if (dr < rc2) {  // false for a neighbour whose position is not finite
              const int tj = type[j];
              if (!smd_static::type_ok(tj, nT)) {
                flags |= smd_static::kStaticBadType;
                continue;
              }
              dr = sqrt(dr);
              int ci = 6 * (ti * nT + tj);
              ci += (dr / fC[ci] >= 1.0) ? 3 : 0;
              double mag = fC[ci] - dr;
              mag = ((fC[ci + 1] - fC[ci + 2] * mag) * mag) / dr;
              fx += dx * mag;
              fy += dy * mag;
              fz += dz * mag;
            }
          }
        }
  }
  if (flags != 0) fx = fy = fz = CUDART_NAN;
  force[3 * i] = fx;
  force[3 * i + 1] = fy;
  force[3 * i + 2] = fz;
}

int error(int code, const std::string& msg) {
  smd::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" int smd_pair_forces_static(const double* d_pos, const int* d_type, int n, const double box[3],
                                      double cutoff, int n_types, const double* d_fconst, double* d_force,
                                      void* stream) {
  if (!d_pos || !d_type || !d_fconst || !d_force || !box || n < 0)
    return error(1, "smd_pair_forces_static: null pointer or negative size");
  if (n > kMaxBeads)
    return error(1, "smd_pair_forces_static: " + std::to_string(n) + " beads exceed the static maximum of " +
                        std::to_string(kMaxBeads));
  if (!(cutoff > 0) || !std::isfinite(cutoff) || n_types <= 0)
    return error(1, "smd_pair_forces_static: bad cutoff or n_types");
  Grid g;
  long long cells = 1;
  for (int d = 0; d < 3; ++d) {
    if (!std::isfinite(box[d]) || !(box[d] > 0))
      return error(1, "smd_pair_forces_static: box edges must be finite and positive");
    const double per_axis = box[d] / cutoff;  // compared before any conversion to int
    if (!(per_axis < (double)kMaxCells + 1.0))
      return error(1, "smd_pair_forces_static: box edge / cutoff exceeds the static maximum of " +
                          std::to_string(kMaxCells) + " cells");
    g.box[d] = box[d];
    g.n[d] = int(per_axis);
    if (g.n[d] < 3) return error(1, "smd_pair_forces_static: box edge shorter than 3 cutoffs");
    g.cs[d] = box[d] / g.n[d];
    cells *= g.n[d];
    if (cells > kMaxCells)
      return error(1, "smd_pair_forces_static: the grid's cells exceed the static maximum of " +
                          std::to_string(kMaxCells));
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // reported here, not by the caller's next launch check
    return error(100 + (int)e, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return error(1, "smd_pair_forces_static: device index out of range");
  int* count = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!count) {
    e = cudaGetSymbolAddress((void**)&count, g_scratch);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return error(100 + (int)e, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    g_scratch_addr[dev].store(count, std::memory_order_release);
  }
  if (n == 0) return 0;
  int* start = count + kMaxCells;
  int* key = start + kMaxCells + 1;
  int* slot = key + kMaxBeads;
  int* sorted = slot + kMaxBeads;
  cudaStream_t s = (cudaStream_t)stream;
  const int nc = (int)cells;
  const int gb = (n + kThreads - 1) / kThreads;
  k_static_clear<<<(nc + kThreads - 1) / kThreads, kThreads, 0, s>>>(count, nc);
  k_static_bin<<<gb, kThreads, 0, s>>>(d_pos, n, g, key, slot, count);
  k_static_scan<<<1, kThreads, 0, s>>>(count, start, nc);
  k_static_scatter<<<gb, kThreads, 0, s>>>(key, slot, start, sorted, n);
  k_static_force<<<gb, kThreads, 0, s>>>(d_pos, d_type, n, g, cutoff * cutoff, n_types, d_fconst, key, start,
                                         sorted, d_force);
  e = cudaGetLastError();
  if (e != cudaSuccess) return error(200 + (int)e, std::string("kernel launch: ") + cudaGetErrorString(e));
  return 0;
}
