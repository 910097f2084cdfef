// Host orchestration and C ABI of the GB300 membrane MD step.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <tuple>
#include <memory>
#include <string>
#include <vector>

#include "../../include/softmold_gb300.h"
#include "mt19937.h"
#include "smd_adjoint.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

// A failed call also leaves its error as the runtime's last error, which the
// next launch check would report as its own: it is read off here.
#define SMD_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      (void)cudaGetLastError();                                                              \
      return fail(100 + (int)e_, std::string(#call) + ": " + cudaGetErrorString(e_));        \
    }                                                                                        \
  } while (0)

constexpr int kTrialChunk = 1024;  // barostat trials staged per upload
constexpr int kBeadRadiusConst = 4;  // BEADRADIUS: the radius within a BEAD constant row

}  // namespace

using namespace smd;

namespace smd {
// Lets other translation units of the library report through smd_last_error.
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace smd

struct smd_system {
  bool mixed = true;
  int n = 0, n_rep = 0, npad = 0, kmax = 0, n_cells = 0, n_tiles = 0;
  int n_sph = 0;  // BEAD sphere beads
  int sph_threads = 32;  // k_sphere block: the spheres rounded up to whole warps
  size_t sph_stage = 0;  // k_integ's dynamic shared memory: the spheres' copy
  int n_terms = 0;  // BOND / BEND and external-field term entries
  bool has_fields = false;  // any external-field term entry
  long long n_chains = 0;  // CHAIN molecules (lipids)
  // adjoint work arrays (allocated by the first adjoint call)
  struct Adj {
    double *w0 = nullptr, *w1 = nullptr, *xbar = nullptr, *hbar = nullptr, *kw = nullptr, *fpair = nullptr;
    double *out = nullptr;
    double4* ws = nullptr;
    AdjAcc* acc = nullptr;
    AdjTables* tab = nullptr;
  } adj;
  // measurement on the device (smd_measure, smd_start_diffusion)
  struct Meas {
    MeasureAcc* acc = nullptr;
    unsigned int* hist = nullptr;  // kinetic-energy bins of the run so far
    int cap = 0;
    int* off = nullptr;            // meanSquareDisplacement_ groups
    int* beads = nullptr;
    int n_groups = 0, max_group = 0;
    double* msd = nullptr;
    bool tracking = false;         // the drifts add to P.disp
  } meas;
  int cur = 0;
  long long it = 0;         // current loop step
  bool at_measure = false;  // stopped after the second half-kick of step `it`
  bool pending_trial = false;
  bool ext_noise_pending = false;
  double skin = 0.5, dt = 0, half_skin = 0;
  bool barostat = false;
  int resize_rate = 8;
  std::vector<RepParams> rp;
  std::vector<Mt19937> baro;  // one MTRand(seed) stream per replica (MD.cpp:149)
  std::vector<int> first_step;
  Tables tab{};
  DevPtrs P{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<void*> allocs;
  long launches = 0;
  bool profile = false;
  double step_ms = 0;
  long step_launches = 0;
  std::vector<cudaEvent_t> prof_events;  // pairs around step-kernel launches
  size_t prof_used = 0;
  std::vector<double> trial_host;
  int trials_staged = 0, trials_used = 0;
  std::vector<std::vector<double>> mc_fluct;  // per replica, every trial so far
  std::vector<std::vector<int>> mc_accept;
  std::vector<int> log_host;
  // one MC period of the loop as a CUDA graph (per parity of the mirror
  // buffer): the list build of each step is a conditional node, set by the
  // previous step's last block, so idle rebuild kernels are never launched
  struct PeriodGraph {
    cudaGraphExec_t exec = nullptr;
    int kernels = 0;  // kernel nodes outside the conditional bodies
  } graph[2];
  bool use_graphs = true;
  // launch configuration chosen by the autotuner (mixed form): lanes per bead
  // of the pair pass and the list-build kernel (0 flat/128, 1 flat/256,
  // 2 octant/256); every choice gives bitwise the same trajectory
  struct Tune {
    int lanes = kLanes;
    int list = 0;
    bool done = false;
    float ms_list[3] = {0, 0, 0};
    float ms_force[3] = {0, 0, 0};
  } tune;
  cudaStream_t side = nullptr;  // captures the conditional bodies
  long long graph_builds = 0;   // device count of list builds run inside graphs
  double* xfer = nullptr;       // 6n doubles: file-order positions and velocities for host copies

  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();  // not the next launch's error
      return fail(100 + (int)e, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    e = cudaMemset(q, 0, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      cudaFree(q);
      return fail(100 + (int)e, std::string("cudaMemset: ") + cudaGetErrorString(e));
    }
    allocs.push_back(q);
    *p = (T*)q;
    return 0;
  }
  ~smd_system() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto& g : graph)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    if (side) cudaStreamDestroy(side);
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    for (void* q : allocs) cudaFree(q);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  int grid() const { return (n + kBlock - 1) / kBlock; }
  int bead_grid() const { return (n + kBeadBlock - 1) / kBeadBlock; }
  int grid_lanes(int g = kLanes) const { return (int)(((long long)n * g + kBlock - 1) / kBlock); }
  int sms = 152;
  // list build: CTA b builds occupied cell b, and cells beyond the grid come
  // from a device work queue.  The grid follows the occupied-cell count of
  // the last build read back (+25 %): sparse boxes have far more cells than
  // occupied ones, and every idle CTA costs launch time.
  int occ_est = 0;
  int nbr_grid() const {
    const int want = occ_est > 0 ? occ_est + occ_est / 4 + 64 : sms * 32;
    return std::max(1, std::min(n_cells, want));
  }
};

namespace {

int check_launch(smd_system* h) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(200 + (int)e, std::string("kernel launch: ") + cudaGetErrorString(e));
  h->launches++;
  return 0;
}

// Launch with programmatic stream serialization: the kernel may start while
// the previous kernel in the stream drains (it waits for that kernel's
// results on the device).  Kernel nodes captured this way keep the
// programmatic edge in the graph.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl_smem(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st,
                            Args... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
  return launch_pdl_smem(kern, grid, block, 0, st, args...);
}

#define SMD_LAUNCH(h, ...)               \
  do {                                   \
    __VA_ARGS__;                         \
    int rc_ = check_launch(h);           \
    if (rc_) return rc_;                 \
  } while (0)

#define SMD_PDL(h, ...)                                                                          \
  do {                                                                                           \
    const cudaError_t e_ = launch_pdl(__VA_ARGS__);                                              \
    if (e_ != cudaSuccess) {                                                                     \
      (void)cudaGetLastError();                                                                  \
      return fail(200 + (int)e_, std::string("kernel launch: ") + cudaGetErrorString(e_));       \
    }                                                                                            \
    int rc_ = check_launch(h);                                                                   \
    if (rc_) return rc_;                                                                         \
  } while (0)

// k_integ: the spheres' shared-memory copy when the system has any
#define SMD_PDL_INTEG(h, kern)                                                                   \
  do {                                                                                           \
    const cudaError_t e_ = launch_pdl_smem(kern, h->bead_grid(), kBeadBlock, h->sph_stage, h->stream, P, h->cur, se); \
    if (e_ != cudaSuccess) {                                                                     \
      (void)cudaGetLastError();                                                                  \
      return fail(200 + (int)e_, std::string("kernel launch: ") + cudaGetErrorString(e_));       \
    }                                                                                            \
    int rc_ = check_launch(h);                                                                   \
    if (rc_) return rc_;                                                                         \
  } while (0)

__global__ void k_set_rebuild(Global* g, int v) { g->rebuild = v; }

// Clears every replica's energy sums before an energy pass.
__global__ void k_clear_energy(DevPtrs P) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.n_rep) return;
  RepState& rs = P.rs[r];
  rs.e_pair = rs.e_bond = rs.e_kin = rs.e_sphere = 0.0;
}

__global__ void k_set_counters(Global* g, long long it, int set_it, int slot, int set_slot) {
  if (set_it) g->it = it;
  if (set_slot) g->trial_slot = slot;
}

// First node of a period graph: the rebuild decision of the step before it.
__global__ void k_graph_cond(const Global* g, unsigned long long cond) {
  cudaGraphSetConditional((cudaGraphConditionalHandle)cond, g->rebuild ? 1u : 0u);
}

// The list kernels run only when the device flag asks for a rebuild.  API
// calls outside the loop clear the flag afterwards; in the loop the step's
// last block recomputes it from the displacement bound.
int launch_rebuild(smd_system* h, cudaStream_t st, int cur, int in_graph) {
  auto& P = h->P;
  const int gb = h->bead_grid();
  SMD_LAUNCH(h, k_bin<<<gb, kBeadBlock, 0, st>>>(P, cur, h->mixed ? 1 : 0, in_graph));
  if (h->n_cells <= kScanOneMax) {
    SMD_PDL(h, k_scan_one, 1, kScanOneThreads, st, P);
  } else {
    SMD_LAUNCH(h, k_scan_tiles<<<h->n_tiles, kBlock, 0, st>>>(P));
    SMD_LAUNCH(h, k_scan_sums<<<1, kBlock, 0, st>>>(P, h->n_tiles));
    SMD_LAUNCH(h, k_scan_apply<<<h->n_tiles, kBlock, 0, st>>>(P));
  }
  if (h->mixed) {
    SMD_PDL(h, k_reorder<true>, gb, kBeadBlock, st, P, cur);
    switch (h->tune.list) {
      case 1: SMD_PDL(h, k_nbr_cells_flat<256>, h->nbr_grid(), 256, st, P, cur); break;
      case 2: SMD_PDL(h, k_nbr_cells_oct, h->nbr_grid(), kOctThreads, st, P, cur); break;
      default: SMD_PDL(h, k_nbr_cells_flat<128>, h->nbr_grid(), 128, st, P, cur); break;
    }
  } else {
    SMD_PDL(h, k_reorder<false>, gb, kBeadBlock, st, P, cur);
    SMD_PDL(h, k_nbr_cells_plain, h->nbr_grid(), kNbrThreads, st, P, cur);
  }
  return 0;
}
// kernels of one list build
int rebuild_kernels(const smd_system* h) { return h->n_cells <= kScanOneMax ? 4 : 6; }

int rebuild_if_needed(smd_system* h, bool clear_after = false) {
  if (int rc = launch_rebuild(h, h->stream, h->cur, 0)) return rc;
  if (clear_after) SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(h->P.g, 0));
  return 0;
}

int force_rebuild(smd_system* h) {
  SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(h->P.g, 1));
  return rebuild_if_needed(h, true);
}

// Sums the elapsed time of the recorded event pairs (after a stream sync).
int collect_profile(smd_system* h) {
  for (size_t k = 0; k + 1 < h->prof_used; k += 2) {
    float ms = 0;
    SMD_CUDA(cudaEventElapsedTime(&ms, h->prof_events[k], h->prof_events[k + 1]));
    h->step_ms += ms;
    h->step_launches++;
  }
  h->prof_used = 0;
  return 0;
}

int prof_mark(smd_system* h) {
  if (h->prof_used == h->prof_events.size()) {
    if (h->prof_used >= 8192) {  // bound the pool: drain what was recorded
      SMD_CUDA(cudaStreamSynchronize(h->stream));
      if (int rc = collect_profile(h)) return rc;
    } else {
      cudaEvent_t e;
      SMD_CUDA(cudaEventCreate(&e));
      h->prof_events.push_back(e);
    }
  }
  SMD_CUDA(cudaEventRecord(h->prof_events[h->prof_used++], h->stream));
  return 0;
}

template <int FL>
int launch_step(smd_system* h, StepEnd se = StepEnd{0, 0, 1, 0, 0}) {
  auto& P = h->P;
  constexpr bool kLoopStep = (FL & (F_FORCES | F_ENERGY | F_INIT)) == 0;
  // the loop's two integrator variants also come without the field-term
  // call, whose out-of-line ABI costs them registers and a stack frame
  constexpr bool kHot = FL == 0 || FL == (F_STOP | F_DU);
  if (kLoopStep && h->profile) {
    if (int rc = prof_mark(h)) return rc;
  }
  const int gl = h->grid_lanes();
  if constexpr ((FL & F_DU) != 0) {  // the reference-grid cells the size-change pass asks about
    // (and, in the loop's barostat step, the replicas' trial)
    SMD_LAUNCH(h, k_ref_cells<<<h->grid(), kBlock, 0, h->stream>>>(P, (FL & F_STOP) != 0 ? 1 : 0));
  }
  if (h->mixed) {
    if constexpr (FL == 0 || FL == (F_STOP | F_DU)) {  // the loop's pair passes follow the tuner
      switch (h->tune.lanes) {
        case 4:
          SMD_LAUNCH(h, (k_force<true, FL, 4><<<h->grid_lanes(4), kBlock, 0, h->stream>>>(P, h->cur)));
          break;
        case 16:
          SMD_LAUNCH(h, (k_force<true, FL, 16><<<h->grid_lanes(16), kBlock, 0, h->stream>>>(P, h->cur)));
          break;
        default:
          SMD_LAUNCH(h, (k_force<true, FL, kLanes><<<gl, kBlock, 0, h->stream>>>(P, h->cur)));
      }
    } else {
      SMD_LAUNCH(h, (k_force<true, FL, kLanes><<<gl, kBlock, 0, h->stream>>>(P, h->cur)));
    }
    if constexpr (kHot) {
      if (!h->has_fields)
        SMD_PDL_INTEG(h, (k_integ<true, FL>));
      else
        SMD_PDL_INTEG(h, (k_integ<true, FL | F_FIELDS>));
    } else {
      SMD_PDL_INTEG(h, (k_integ<true, FL | F_FIELDS>));
    }
    if (h->n_sph) SMD_LAUNCH(h, (k_sphere<true, FL><<<1, h->sph_threads, 0, h->stream>>>(P, h->cur, se)));
  } else {
    SMD_LAUNCH(h, (k_force<false, FL, kLanes><<<gl, kBlock, 0, h->stream>>>(P, h->cur)));
    if constexpr (kHot) {
      if (!h->has_fields)
        SMD_PDL_INTEG(h, (k_integ<false, FL>));
      else
        SMD_PDL_INTEG(h, (k_integ<false, FL | F_FIELDS>));
    } else {
      SMD_PDL_INTEG(h, (k_integ<false, FL | F_FIELDS>));
    }
    if (h->n_sph) SMD_LAUNCH(h, (k_sphere<false, FL><<<1, h->sph_threads, 0, h->stream>>>(P, h->cur, se)));
  }
  if (kLoopStep && h->profile) {
    if (int rc = prof_mark(h)) return rc;
  }
  // diffusion tracking: the drift of a step that ran through
  if constexpr (kLoopStep && (FL & F_STOP) == 0) {
    if (h->meas.tracking) {
      if (h->mixed) SMD_LAUNCH(h, k_track<true><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
      else SMD_LAUNCH(h, k_track<false><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
    }
  }
  return 0;
}

// The loop's pair pass alone (its output is scratch until k_integ reads it).
int launch_force_only(smd_system* h) {
  auto& P = h->P;
  switch (h->tune.lanes) {
    case 4: SMD_LAUNCH(h, (k_force<true, 0, 4><<<h->grid_lanes(4), kBlock, 0, h->stream>>>(P, h->cur))); break;
    case 16: SMD_LAUNCH(h, (k_force<true, 0, 16><<<h->grid_lanes(16), kBlock, 0, h->stream>>>(P, h->cur))); break;
    default: SMD_LAUNCH(h, (k_force<true, 0, kLanes><<<h->grid_lanes(), kBlock, 0, h->stream>>>(P, h->cur)));
  }
  return 0;
}

// mode bit 0: restart half-kick; bit 1: completes a stopped loop step.
int launch_finish(smd_system* h, int mode, int apply_mc, StepEnd se) {
  auto& P = h->P;
  if (h->mixed)
    SMD_LAUNCH(h, k_finish<true><<<h->bead_grid(), kBeadBlock, 0, h->stream>>>(P, h->cur, mode, apply_mc, se));
  else
    SMD_LAUNCH(h, k_finish<false><<<h->bead_grid(), kBeadBlock, 0, h->stream>>>(P, h->cur, mode, apply_mc, se));
  if (h->meas.tracking) {  // k_finish drifts
    if (h->mixed) SMD_LAUNCH(h, k_track<true><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
    else SMD_LAUNCH(h, k_track<false><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
  }
  h->cur ^= 1;
  return 0;
}

bool is_trial_step(const smd_system* h, long long it) {
  return h->barostat && (it % h->resize_rate) == 0 && it != 0;
}

// Counts the barostat trials among the next `steps` iterations, draws their
// two uniforms per replica from the MT19937 streams, and stages them.
// Appends the decisions of the trials run from the staged buffer to the host
// log (called once the stream has drained).
int flush_mc_log(smd_system* h) {
  if (h->trials_used == 0) return 0;
  const size_t n = (size_t)h->trials_used * h->n_rep;
  h->log_host.resize(n);
  SMD_CUDA(cudaMemcpyAsync(h->log_host.data(), h->P.accept_log, n * sizeof(int), cudaMemcpyDeviceToHost,
                           h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  for (int t = 0; t < h->trials_used; ++t)
    for (int r = 0; r < h->n_rep; ++r) {
      if (h->rp[r].dlxy == 0) continue;
      const double u1 = h->trial_host[((size_t)t * h->n_rep + r) * 2];
      h->mc_fluct[r].push_back(h->rp[r].dlxy * (2.0 * u1 - 1.0));
      h->mc_accept[r].push_back(h->log_host[(size_t)t * h->n_rep + r]);
    }
  h->trials_used = 0;
  h->trials_staged = 0;
  return 0;
}

int stage_trials(smd_system* h, long long from, int steps) {
  int count = 0;
  for (long long k = from; k < from + steps; ++k)
    if (is_trial_step(h, k)) ++count;
  if (count == 0) return 0;
  if (count > kTrialChunk) return fail(3, "internal: too many barostat trials staged at once");
  if (int rc = flush_mc_log(h)) return rc;
  h->trial_host.assign((size_t)count * h->n_rep * 2, 0.0);
  for (int t = 0; t < count; ++t)
    for (int r = 0; r < h->n_rep; ++r) {
      h->trial_host[((size_t)t * h->n_rep + r) * 2] = h->baro[r].rand53();
      h->trial_host[((size_t)t * h->n_rep + r) * 2 + 1] = h->baro[r].rand53();
    }
  // pageable source: the copy is staged before cudaMemcpyAsync returns
  SMD_CUDA(cudaMemcpyAsync(h->P.trial_u, h->trial_host.data(), h->trial_host.size() * sizeof(double),
                           cudaMemcpyHostToDevice, h->stream));
  SMD_LAUNCH(h, k_set_counters<<<1, 1, 0, h->stream>>>(h->P.g, 0, 0, 0, 1));
  h->trials_staged = count;
  h->trials_used = 0;
  return 0;
}

int complete_pending(smd_system* h) {
  if (!h->at_measure) return 0;
  const int apply = h->pending_trial ? 1 : 0;
  if (h->pending_trial) {
    SMD_LAUNCH(h, k_mc<<<(h->n_rep + 63) / 64, 64, 0, h->stream>>>(h->P));
  }
  int rc = launch_finish(h, 2, apply, StepEnd{0, 0, 1, apply, 0});
  if (rc) return rc;
  h->at_measure = false;
  h->pending_trial = false;
  h->it++;
  return 0;
}

// List capacity for a largest neighbour count `need` (entries per bead).
int list_capacity(int need) { return std::max(((int)(need * 2.0) + 64 + 7) / 8 * 8, 192); }

// Grows the Verlet list to list_capacity(need) (the stream is idle): a new
// buffer, graphs re-captured on their next use (they hold the old pointer),
// and a rebuild.
int grow_list(smd_system* h, int need) {
  const int kmax = list_capacity(need);
  int* nbr = nullptr;
  SMD_CUDA(cudaMalloc(&nbr, (size_t)kmax * h->n * sizeof(int)));
  for (auto& q : h->allocs)
    if (q == (void*)h->P.nbr) {
      cudaFree(q);
      q = nbr;
    }
  h->P.nbr = nbr;
  h->P.kmax = h->kmax = kmax;
  for (auto& gr : h->graph)
    if (gr.exec) {
      cudaGraphExecDestroy(gr.exec);
      gr.exec = nullptr;
    }
  SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(h->P.g, 1));
  return rebuild_if_needed(h, true);
}

// Device staging for the state copies: the host side moves one contiguous
// file-order block per array and the permutation runs on the device.
int xfer_buffer(smd_system* h) {
  if (h->xfer) return 0;
  return h->alloc(&h->xfer, (size_t)h->n * 6);
}

int read_error(smd_system* h) {
  Global g;
  SMD_CUDA(cudaMemcpyAsync(&g, h->P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  h->graph_builds = g.graph_builds;
  if (g.n_occ > 0) h->occ_est = g.n_occ;
  if (g.error & 2) return fail(8, "a Verlet-list cell holds more than 1024 beads (collapsed system)");
  if (g.error & 1) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "Verlet list overflow: a bead has %d neighbours within rc+skin, capacity %d "
                  "(system density grew far beyond the start configuration)",
                  g.need_nbr, h->kmax);
    return fail(7, buf);
  }
  // between calls: grow the list before a denser state can overflow it
  if (g.max_nbr > h->kmax * 4 / 5 && !h->at_measure) {
    if (int rc = grow_list(h, g.max_nbr)) return rc;
    SMD_CUDA(cudaStreamSynchronize(h->stream));
  }
  return 0;
}

// Range of the reference's hash cells for a residue above the brute-force
// size (cells of side >= twice it): a BEAD residue's C[0]; for NANOCORE the
// largest C[0] of its cores, truncated to an integer as the reference's
// int accumulator does (include/system.h:2265-2271).
double sphere_grid_range(const smd_system_desc& d) {
  if (!d.sphere_nanocore) return d.sphere_consts[0];
  int r = 0;
  for (int k = 0; k < d.n_spheres; ++k) {
    const double c = d.sphere_consts[kBeadConst * k];
    if (c > r) r = c < 2147483647.0 ? (int)c : 2147483647;
  }
  return (double)r;
}

int validate(const smd_system_desc& d, std::string& why) {
  if (d.n <= 0) return why = "n must be positive", 1;
  if (d.n_types <= 0 || d.n_types > kMaxTypes) return why = "n_types must be in 1..8", 1;
  if (!d.pos || !d.vel || !d.type || !d.fconst || !d.uconst) return why = "null array in descriptor", 1;
  if (!(d.cutoff > 0) || !std::isfinite(d.cutoff)) return why = "cutoff must be positive and finite", 1;
  if (!std::isfinite(d.skin)) return why = "skin not finite", 1;
  for (int k = 0; k < 3; ++k) {
    if (!(d.box[k] > 0) || !std::isfinite(d.box[k])) return why = "box must be positive and finite", 1;
    // bounds the cell grid (and the int conversions below) before any product
    if (!(d.box[k] / d.cutoff < (double)kMaxGridCells))
      return why = "box edge above " + std::to_string(kMaxGridCells) + " cutoffs", 1;
    if (int(d.box[k] / d.cutoff) < 3)
      return why = "box edge shorter than 3 cutoffs: the reference cell traversal double-counts there", 1;
  }
  for (int i = 0; i < d.n; ++i) {
    if (d.type[i] < 0 || d.type[i] >= d.n_types) return why = "bead type out of range", 1;
    for (int k = 0; k < 3; ++k) {
      const double x = d.pos[3 * i + k];
      if (!(x >= 0 && x <= d.box[k])) return why = "position out of the box", 1;
      if (!std::isfinite(d.vel[3 * i + k])) return why = "velocity not finite", 1;
    }
  }
  const auto finite = [](const double* a, long long m) {
    for (long long k = 0; k < m; ++k)
      if (!std::isfinite(a[k])) return false;
    return true;
  };
  const long long ntab = 6LL * d.n_types * d.n_types;
  if (!finite(d.fconst, ntab) || !finite(d.uconst, ntab)) return why = "pair table value not finite", 1;
  if (d.n_chain_blocks > 0 && !finite(d.chain_consts, 4LL * d.n_chain_blocks))
    return why = "CHAIN constant not finite", 1;
  if (!std::isfinite(d.dt) || !std::isfinite(d.gamma) || !(d.gamma >= 0) || !std::isfinite(d.temperature) ||
      !(d.temperature >= 0) || !std::isfinite(d.tension) || !std::isfinite(d.delta_lxy))
    return why = "dt, gamma, temperature, tension or deltaLXY not finite (or gamma / temperature negative)", 1;
  for (int b = 0; b < d.n_chain_blocks; ++b) {
    const int s = d.chain_blocks[3 * b], c = d.chain_blocks[3 * b + 1], l = d.chain_blocks[3 * b + 2];
    if (l < 3 || l > 4095) return why = "CHAIN length must be in 3..4095", 1;
    if (s < 0 || (long long)s + (long long)c * l > d.n) return why = "CHAIN block out of range", 1;
  }
  if (d.n_spheres < 0 || d.n_spheres > kMaxSpheres)
    return why = "at most " + std::to_string(kMaxSpheres) + " BEAD or NANOCORE beads per system", 1;
  if (d.n_spheres > 0) {
    if (!d.sphere_index || !d.sphere_consts) return why = "null BEAD array in descriptor", 1;
    for (int k = 0; k < d.n_spheres; ++k) {
      if (d.sphere_index[k] < 0 || d.sphere_index[k] >= d.n) return why = "BEAD bead index out of range", 1;
      for (int q = 0; q < k; ++q)
        if (d.sphere_index[q] == d.sphere_index[k]) return why = "BEAD bead listed twice", 1;
    }
    if (d.sphere_nanocore) {
      for (int k = 0; k < d.n_spheres; ++k)
        if (!(d.sphere_consts[kBeadConst * k + kBeadRadiusConst] > 0)) return why = "NANOCORE radius must be positive", 1;
    } else if (!(d.sphere_consts[kBeadRadiusConst] > 0)) {
      return why = "BEAD radius must be positive", 1;
    }
    const bool grid = d.sphere_nanocore ? d.n_spheres > kCoreBrute : d.n_spheres > kBeadBrute;
    if (grid) {
      // the reference's cell count int(L / 2r) must be at least one per axis
      const double len = 2.0 * sphere_grid_range(d);
      if (!(len > 0) || !(d.box[0] >= len && d.box[1] >= len && d.box[2] >= len))
        return why = "box below one hash cell (twice the sphere range) of the many-sphere branch", 1;
    }
  }
  if (d.n_bonds < 0 || d.n_bends < 0) return why = "negative BOND / BEND term count", 1;
  if (d.n_bonds > 0 && (!d.bonds || !d.bond_consts)) return why = "null BOND array in descriptor", 1;
  if (d.n_bends > 0 && (!d.bends || !d.bend_consts)) return why = "null BEND array in descriptor", 1;
  for (int k = 0; k < 2 * d.n_bonds; ++k)
    if (d.bonds[k] < 0 || d.bonds[k] >= d.n) return why = "BOND bead index out of range", 1;
  for (int k = 0; k < 3 * d.n_bends; ++k)
    if (d.bends[k] < 0 || d.bends[k] >= d.n) return why = "BEND bead index out of range", 1;
  if (d.n_fields < 0) return why = "negative field term count", 1;
  if (d.n_fields > 0 && (!d.fields || !d.field_consts)) return why = "null field array in descriptor", 1;
  for (int k = 0; k < d.n_fields; ++k) {
    const int kind = d.fields[3 * k], a = d.fields[3 * k + 1], b = d.fields[3 * k + 2];
    if (kind != 11 && kind != 15 && kind != 16 && kind != 17 && kind != 19)
      return why = "field term kind must be 11, 15, 16, 17 or 19 (BOUNDARY, FLOATING_BASE, ZTORQUE, "
                   "ZPOWERPOTENTIAL, BALL)", 1;
    const bool pair = (kind == 16 || kind == 19);
    if (a < 0 || a >= d.n || (pair ? (b < 0 || b >= d.n || b == a) : b != -1))
      return why = "field term bead index out of range", 1;
    if (kind == 19) {
      const double own = d.field_consts[8 * k + 2];
      if (!(own >= 0 && own < d.n && own == (double)(int)own)) return why = "BALL term's own first bead out of range", 1;
    }
    if (kind == 11 && !(d.field_consts[8 * k] == 0 || d.field_consts[8 * k] == 1 || d.field_consts[8 * k] == 2))
      return why = "BOUNDARY dimension must be 0, 1 or 2", 1;
  }
  if (d.n_bonds > 0 && !finite(d.bond_consts, 2LL * d.n_bonds)) return why = "BOND constant not finite", 1;
  if (d.n_bends > 0 && !finite(d.bend_consts, 2LL * d.n_bends)) return why = "BEND constant not finite", 1;
  if (d.n_fields > 0 && !finite(d.field_consts, 8LL * d.n_fields)) return why = "field constant not finite", 1;
  if (d.n_spheres > 0 &&
      !finite(d.sphere_consts, d.sphere_nanocore ? (long long)kBeadConst * d.n_spheres
                                                  : (long long)kBeadConst * d.n_types * d.n_types))
    return why = "BEAD / NANOCORE constant not finite", 1;
  if (!(d.dt > 0)) return why = "dt must be positive", 1;
  return 0;
}

}  // namespace

extern "C" {

int smd_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return (int)g_last_error.size();
}

int smd_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int smd_create(const smd_system_desc* desc, int precision, smd_system** out) {
  return smd_create_batch(desc, 1, precision, out);
}

int smd_create_batch(const smd_system_desc* descs, int n_rep, int precision, smd_system** out) {
  if (!descs || n_rep <= 0 || !out) return fail(1, "smd_create_batch: bad arguments");
  if (precision != SMD_PLAIN_FP64 && precision != SMD_MIXED) return fail(1, "unknown precision");
  *out = nullptr;
  // descriptors first (host checks only), then the device
  std::string why;
  for (int r = 0; r < n_rep; ++r)
    if (validate(descs[r], why)) return fail(1, "replica " + std::to_string(r) + ": " + why);
  const smd_system_desc& d0 = descs[0];
  for (int r = 0; r < n_rep; ++r)
    if (n_rep > 1 && descs[r].n_spheres > 0)
      return fail(1, "BEAD and NANOCORE residues are supported in single-system handles, not in batches");
  for (int r = 1; r < n_rep; ++r) {
    const smd_system_desc& d = descs[r];
    if (d.n_types != d0.n_types || d.cutoff != d0.cutoff || d.dt != d0.dt)
      return fail(1, "replicas of a batch must share n_types, cutoff and dt");
    for (int k = 0; k < 6 * d0.n_types * d0.n_types; ++k)
      if (d.fconst[k] != d0.fconst[k] || d.uconst[k] != d0.uconst[k])
        return fail(1, "replicas of a batch must share the pair tables");
  }
  // the list-cell grid of each replica (cells of side cutoff + skin, one
  // extra per axis: a growing box coarsens the grid in derive_box), sized on
  // the host before the device.  validate keeps each axis below kMaxGridCells
  // cells; checked after each product (at most 2^56 + 2^28), the total stays
  // an int.
  const double skin = d0.skin > 0 ? d0.skin : 0.5;
  std::vector<int> cell_caps(n_rep);
  long long grid_cells = 0;
  for (int r = 0; r < n_rep; ++r) {
    long long cap = 1;
    for (int k = 0; k < 3 && cap <= kMaxGridCells; ++k)
      cap *= std::max(1LL, (long long)(descs[r].box[k] / (d0.cutoff + skin))) + 1;
    if (cap > kMaxGridCells - grid_cells)
      return fail(1, "replica " + std::to_string(r) + ": the cell grid of the handle exceeds " +
                         std::to_string(kMaxGridCells) + " cells (box edges / (cutoff + skin))");
    cell_caps[r] = (int)cap;
    grid_cells += cap;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(2, "no CUDA device: the GB300 step has no CPU fallback");
  std::unique_ptr<smd_system> h(new smd_system());
  h->mixed = (precision == SMD_MIXED);
  h->n_rep = n_rep;
  h->dt = d0.dt;
  h->skin = skin;
  h->half_skin = 0.5 * h->skin;
  h->resize_rate = d0.resize_rate > 0 ? d0.resize_rate : 8;
  int total = 0;
  for (int r = 0; r < n_rep; ++r) total += descs[r].n;
  h->n = total;
  h->npad = (total + 31) / 32 * 32;
  // ---- tables
  Tables& T = h->tab;
  T.nT = d0.n_types;
  T.rc = d0.cutoff;
  T.rc2 = d0.cutoff * d0.cutoff;
  T.rcf = (float)d0.cutoff;
  T.rc2f = (float)(d0.cutoff * d0.cutoff);
  T.list_cut = d0.cutoff + h->skin;
  T.list_cut2 = T.list_cut * T.list_cut;
  T.list_cut_f = (float)T.list_cut;
  double maxF = 1.0;
  for (int k = 0; k < d0.n_types * d0.n_types; ++k) {
    const double* c = d0.fconst + 6 * k;
    T.dF[6 * k + 0] = c[0];
    for (int q = 0; q < 6; ++q) {
      T.dF[6 * k + q] = c[q];
      T.fF[6 * k + q] = (float)c[q];
      T.dU[6 * k + q] = d0.uconst[6 * k + q];
      T.fU[6 * k + q] = (float)d0.uconst[6 * k + q];
    }
    // |F| = |mag| r: inner segment at most C1*rm, outer sampled on [rm, rc]
    maxF = std::max(maxF, std::fabs(c[1] * c[0]));
    for (int s = 0; s <= 64; ++s) {
      const double r = c[0] + (d0.cutoff - c[0]) * s / 64.0;
      const double m = c[3] - r;
      maxF = std::max(maxF, std::fabs((c[4] - c[5] * m) * m) * 1.05);
    }
  }
  // one pair force must stay below 2^26 after scaling, so that the pair pass
  // can sum 32 of them per lane in int32 before widening to int64
  T.fscale = (float)std::ldexp(1.0, (int)std::floor(std::log2(67108864.0 / maxF)));
  T.inv_fscale = 1.0 / (double)T.fscale;
  // chain constant sets
  std::vector<std::array<double, 4>> sets;
  std::vector<std::array<double, 2>> tsets;
  std::vector<std::array<double, kFieldConst>> fsets;
  std::vector<std::vector<int4>> bead_terms(total);
  std::vector<int> cinfo(total, 0);
  std::vector<int> type(total, 0);
  h->rp.resize(n_rep);
  h->first_step.resize(n_rep);
  int bead = 0, cells = 0;
  for (int r = 0; r < n_rep; ++r) {
    const smd_system_desc& d = descs[r];
    RepParams& p = h->rp[r];
    p.dt = d.dt;
    p.gamma = d.gamma;
    p.kT = d.temperature;
    p.sigma = std::sqrt((6.0 * d.temperature * d.gamma) / d.dt);
    p.sig31 = p.sigma * (1.0 / 2147483648.0);
    p.sig31f = (float)p.sig31;
    p.tension = d.tension;
    p.dlxy = d.delta_lxy;
    p.seed = d.seed;
    p.resize_rate = h->resize_rate;
    p.bead_begin = bead;
    p.bead_end = bead + d.n;
    if (d.delta_lxy != 0) h->barostat = true;
    // one extra cell per axis: a growing box coarsens the grid in derive_box
    const int cap = cell_caps[r];
    p.cell_begin = cells;
    p.cell_cap = cap;
    cells += cap;
    h->baro.emplace_back((uint32_t)d.seed);
    h->first_step[r] = d.first_step;
    for (int i = 0; i < d.n; ++i) type[bead + i] = d.type[i];
    for (int b = 0; b < d.n_chain_blocks; ++b) {
      std::array<double, 4> c = {d.chain_consts[4 * b], d.chain_consts[4 * b + 1], d.chain_consts[4 * b + 2],
                                 d.chain_consts[4 * b + 3]};
      int set = -1;
      for (size_t q = 0; q < sets.size(); ++q)
        if (sets[q] == c) set = (int)q;
      if (set < 0) {
        if ((int)sets.size() >= kMaxChainSets) return fail(1, "too many distinct CHAIN constant sets");
        sets.push_back(c);
        set = (int)sets.size() - 1;
      }
      const int s = d.chain_blocks[3 * b], nc = d.chain_blocks[3 * b + 1], l = d.chain_blocks[3 * b + 2];
      h->n_chains += nc;
      for (int c2 = 0; c2 < nc; ++c2)
        for (int q = 0; q < l; ++q) cinfo[bead + s + c2 * l + q] = cinfo_pack(q, l, set);
    }
    for (int k = 0; k < d.n_spheres; ++k) {
      if (cinfo[bead + d.sphere_index[k]] != 0) return fail(1, "a BEAD or NANOCORE bead is also a CHAIN member");
      cinfo[bead + d.sphere_index[k]] = (int)(0xC0000000u | (unsigned)k);
    }
    // BOND / BEND terms: per-bead entries (file order), constant sets shared
    auto term_set = [&](double c0, double c1) -> int {
      const std::array<double, 2> c = {c0, c1};
      for (size_t q = 0; q < tsets.size(); ++q)
        if (tsets[q] == c) return (int)q;
      if ((int)tsets.size() >= kMaxTermSets) return -1;
      tsets.push_back(c);
      return (int)tsets.size() - 1;
    };
    for (int k = 0; k < d.n_bonds; ++k) {
      const int set = term_set(d.bond_consts[2 * k], d.bond_consts[2 * k + 1]);
      if (set < 0) return fail(1, "too many distinct BOND / BEND constant sets");
      const int a = bead + d.bonds[2 * k], b = bead + d.bonds[2 * k + 1];
      bead_terms[a].push_back(make_int4(term_pack(kTermBond, 0, set), a, b, -1));
      bead_terms[b].push_back(make_int4(term_pack(kTermBond, 1, set), a, b, -1));
    }
    for (int k = 0; k < d.n_bends; ++k) {
      const int set = term_set(d.bend_consts[2 * k], d.bend_consts[2 * k + 1]);
      if (set < 0) return fail(1, "too many distinct BOND / BEND constant sets");
      const int a = bead + d.bends[3 * k], b = bead + d.bends[3 * k + 1], c = bead + d.bends[3 * k + 2];
      for (int role = 0; role < 3; ++role)
        bead_terms[role == 0 ? a : (role == 1 ? b : c)].push_back(
            make_int4(term_pack(kTermBend, role, set), a, b, c));
    }
    // external-field terms: the same per-bead entries, constant sets in fieldD
    for (int k = 0; k < d.n_fields; ++k) {
      std::array<double, kFieldConst> c;
      for (int q = 0; q < kFieldConst; ++q) c[q] = d.field_consts[kFieldConst * k + q];
      const int kind = d.fields[3 * k], a = bead + d.fields[3 * k + 1];
      const int tk = kind == 11 ? kTermBoundary
                     : (kind == 15 ? kTermFloating : (kind == 16 ? kTermZTorque : (kind == 19 ? kTermBall : kTermZPower)));
      if (tk == kTermBall) c[2] += bead;  // the potential's own first bead, a global index like the others
      int set = -1;
      for (size_t q = 0; q < fsets.size() && set < 0; ++q)
        if (fsets[q] == c) set = (int)q;
      if (set < 0) {
        if ((int)fsets.size() >= kMaxFieldSets) return fail(1, "too many distinct external-field constant sets");
        fsets.push_back(c);
        set = (int)fsets.size() - 1;
      }
      if (tk == kTermZTorque || tk == kTermBall) {
        const int b = bead + d.fields[3 * k + 2];
        bead_terms[a].push_back(make_int4(term_pack(tk, 0, set), a, b, -1));
        bead_terms[b].push_back(make_int4(term_pack(tk, 1, set), a, b, -1));
      } else {
        bead_terms[a].push_back(make_int4(term_pack(tk, 0, set), a, -1, -1));
      }
    }
    bead += d.n;
  }
  for (int r = 1; r < n_rep; ++r)
    if (h->first_step[r] != h->first_step[0]) return fail(1, "replicas of a batch must start at the same step");
  h->it = h->first_step[0];
  T.n_sets = (int)sets.size();
  for (size_t q = 0; q < tsets.size(); ++q)
    for (int k = 0; k < 2; ++k) {
      T.termD[q][k] = tsets[q][k];
      T.termF[q][k] = (float)tsets[q][k];
    }
  for (size_t q = 0; q < fsets.size(); ++q)
    for (int k = 0; k < kFieldConst; ++k) T.fieldD[q][k] = fsets[q][k];
  for (size_t q = 0; q < sets.size(); ++q)
    for (int k = 0; k < 4; ++k) {
      T.chainD[q][k] = sets[q][k];
      T.chainF[q][k] = (float)sets[q][k];
    }
  h->n_cells = cells;
  h->n_tiles = (cells + kScanTile - 1) / kScanTile;
  // ---- device memory
  {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0)
      h->sms = sms;
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(2, "cudaStreamCreate failed");
  h->own_stream = true;
  DevPtrs& P = h->P;
  P.n = total;
  P.npad = h->npad;
  P.n_rep = n_rep;
  P.n_cells_total = cells;
  P.half_skin = h->half_skin;
  int rc = 0;
  double** dbl[] = {&P.x, &P.y, &P.z, &P.vx, &P.vy, &P.vz, &P.ax, &P.ay, &P.az,
                    &P.tx, &P.ty, &P.tz, &P.tvx, &P.tvy, &P.tvz, &P.tax, &P.tay, &P.taz};
  for (double** q : dbl)
    if ((rc = h->alloc(q, total))) return rc;
  if (h->mixed) {
    if ((rc = h->alloc(&P.m4[0], total)) || (rc = h->alloc(&P.m4[1], total)) || (rc = h->alloc(&P.mt, total)))
      return rc;
  } else {
    if ((rc = h->alloc(&P.d4[0], total)) || (rc = h->alloc(&P.d4[1], total)) || (rc = h->alloc(&P.dt4, total)))
      return rc;
  }
  if ((rc = h->alloc(&P.ref, total)) || (rc = h->alloc(&P.refcell, total))) return rc;
  int** ints[] = {&P.orig, &P.inv, &P.cinfo, &P.torig, &P.tcinfo, &P.key, &P.slot, &P.tkey, &P.nnbr, &P.key_out};
  for (int** q : ints)
    if ((rc = h->alloc(q, total))) return rc;
  if (h->mixed) {
    if ((rc = h->alloc(&P.fq, 3 * (size_t)total))) return rc;
  } else {
    if ((rc = h->alloc(&P.fp, 3 * (size_t)total))) return rc;
  }
  if ((rc = h->alloc(&P.cell_count, cells)) || (rc = h->alloc(&P.cell_start, cells + 1)) ||
      (rc = h->alloc(&P.block_sums, h->n_tiles)) || (rc = h->alloc(&P.occ, cells)))
    return rc;
  if ((rc = h->alloc(&P.rp, n_rep)) || (rc = h->alloc(&P.rs, n_rep)) || (rc = h->alloc(&P.g, 1))) return rc;
  Tables* tdev = nullptr;
  if ((rc = h->alloc(&tdev, 1))) return rc;
  P.tab = tdev;
  if ((rc = h->alloc(&P.accept_log, (size_t)kTrialChunk * n_rep))) return rc;
  h->mc_fluct.resize(n_rep);
  h->mc_accept.resize(n_rep);
  if ((rc = h->alloc(&P.trial_u, (size_t)kTrialChunk * n_rep * 2)) || (rc = h->alloc(&P.ext_noise, 3 * total)) ||
      (rc = h->alloc(&P.force_out, 3 * total)))
    return rc;
  // ---- BEAD spheres (single-system handles)
  if (d0.n_spheres > 0) {
    // BEAD: one row per ordered type pair; NANOCORE: one row per core
    const int nc = d0.sphere_nanocore ? kBeadConst * d0.n_spheres : kBeadConst * d0.n_types * d0.n_types;
    double* dC = nullptr;
    float* fC = nullptr;
    if ((rc = h->alloc(&P.sph, 1)) || (rc = h->alloc(&dC, nc)) || (rc = h->alloc(&fC, nc))) return rc;
    std::vector<float> cf(nc);
    for (int k = 0; k < nc; ++k) cf[k] = (float)d0.sphere_consts[k];
    SphereDev sd;
    std::memset(&sd, 0, sizeof sd);
    sd.n = d0.n_spheres;
    sd.nanocore = d0.sphere_nanocore ? 1 : 0;
    for (int k = 0; k < sd.n; ++k) {
      sd.orig[k] = d0.sphere_index[k];
      // its row: BEAD row 0 (constant 0 is the range, constant 4 the radius);
      // NANOCORE its own (MD.cpp:280-303)
      const double* C = d0.sphere_consts + (sd.nanocore ? kBeadConst * k : 0);
      const double R = C[kBeadRadiusConst];
      sd.mass[k] = 4.0 * M_PI * R * R;
      sd.cut2[k] = C[0] * C[0];
    }
    const double R = d0.sphere_consts[kBeadRadiusConst];
    sd.bb_cut2 = (R + R + 2.0) * (R + R + 2.0);
    // the reference's branch for this residue size (brute force or hash cells)
    sd.all_partners = (sd.nanocore || sd.n > kBeadBrute) ? 1 : 0;
    sd.grid = sd.nanocore ? (sd.n > kCoreBrute ? 1 : 0) : (sd.n > kBeadBrute ? 1 : 0);
    sd.grid_len = 2.0 * sphere_grid_range(d0);
    SMD_CUDA(cudaMemcpy(P.sph, &sd, sizeof sd, cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(dC, d0.sphere_consts, nc * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(fC, cf.data(), nc * sizeof(float), cudaMemcpyHostToDevice));
    P.sphC = dC;
    P.sphCf = fC;
    P.n_sph = sd.n;
    h->n_sph = sd.n;
    h->sph_threads = (sd.n + 31) / 32 * 32;
    h->sph_stage = sphere_stage_bytes(sd.n, h->mixed);
  }
  // ---- BOND / BEND term entries
  {
    std::vector<int> off(total + 1, 0);
    std::vector<int4> flat;
    for (int b = 0; b < total; ++b) {
      off[b] = (int)flat.size();
      flat.insert(flat.end(), bead_terms[b].begin(), bead_terms[b].end());
    }
    off[total] = (int)flat.size();
    if (!flat.empty()) {
      int* doff = nullptr;
      int4* dterms = nullptr;
      if ((rc = h->alloc(&doff, total + 1)) || (rc = h->alloc(&dterms, flat.size()))) return rc;
      SMD_CUDA(cudaMemcpy(doff, off.data(), (total + 1) * sizeof(int), cudaMemcpyHostToDevice));
      SMD_CUDA(cudaMemcpy(dterms, flat.data(), flat.size() * sizeof(int4), cudaMemcpyHostToDevice));
      P.term_off = doff;
      P.terms = dterms;
      P.n_terms = (int)flat.size();
      h->n_terms = P.n_terms;
      for (const int4& t : flat) h->has_fields = h->has_fields || term_kind(t.x) > kTermBend;
    }
  }
  // ---- upload state (sorted order = file order until the first build)
  {
    std::vector<double> hx(total), hy(total), hz(total), hvx(total), hvy(total), hvz(total);
    std::vector<int> orig(total);
    std::vector<uint4> m4(h->mixed ? total : 0);
    std::vector<double4> d4(h->mixed ? 0 : total);
    std::vector<RepState> rs(n_rep);
    int b = 0;
    for (int r = 0; r < n_rep; ++r) {
      const smd_system_desc& d = descs[r];
      std::memset(&rs[r], 0, sizeof(RepState));
      const double one[3] = {1.0, 1.0, 1.0};
      for (int k = 0; k < 3; ++k) rs[r].box[k] = d.box[k];
      set_scale(rs[r], one);
      derive_box(rs[r], h->rp[r].cell_cap, T.list_cut, T.rc);
      for (int i = 0; i < d.n; ++i, ++b) {
        hx[b] = d.pos[3 * i];
        hy[b] = d.pos[3 * i + 1];
        hz[b] = d.pos[3 * i + 2];
        hvx[b] = d.vel[3 * i];
        hvy[b] = d.vel[3 * i + 1];
        hvz[b] = d.vel[3 * i + 2];
        orig[b] = b;
        const unsigned w = (unsigned)type[b] | ((unsigned)r << 8);
        if (h->mixed) {
          auto fr = [](double x, double L) { return (unsigned int)(long long)(x * (1.0 / L) * 4294967296.0); };
          m4[b] = make_uint4(fr(hx[b], d.box[0]), fr(hy[b], d.box[1]), fr(hz[b], d.box[2]), w);
        } else {
          long long wb = (long long)w;
          double wd;
          std::memcpy(&wd, &wb, sizeof wd);
          d4[b] = make_double4(hx[b], hy[b], hz[b], wd);
        }
      }
    }
    SMD_CUDA(cudaMemcpy(P.x, hx.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.y, hy.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.z, hz.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.vx, hvx.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.vy, hvy.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.vz, hvz.data(), total * sizeof(double), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.orig, orig.data(), total * sizeof(int), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.inv, orig.data(), total * sizeof(int), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.cinfo, cinfo.data(), total * sizeof(int), cudaMemcpyHostToDevice));
    if (h->mixed)
      SMD_CUDA(cudaMemcpy(P.m4[0], m4.data(), total * sizeof(uint4), cudaMemcpyHostToDevice));
    else
      SMD_CUDA(cudaMemcpy(P.d4[0], d4.data(), total * sizeof(double4), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.rp, h->rp.data(), n_rep * sizeof(RepParams), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(P.rs, rs.data(), n_rep * sizeof(RepState), cudaMemcpyHostToDevice));
    SMD_CUDA(cudaMemcpy(tdev, &T, sizeof(Tables), cudaMemcpyHostToDevice));
  }
  // ---- size the Verlet list: count pass with zero capacity, then the build
  P.kmax = 0;
  if ((rc = force_rebuild(h.get()))) return rc;
  Global g;
  SMD_CUDA(cudaMemcpyAsync(&g, P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  const int need = std::max(g.need_nbr, 1);
  h->kmax = list_capacity(need);
  P.kmax = h->kmax;
  if ((rc = h->alloc(&P.nbr, (size_t)h->kmax * total))) return rc;
  g.error = 0;
  g.need_nbr = 0;
  g.max_nbr = 0;
  g.rebuild = 1;
  g.n_rebuilds = 0;
  g.it = h->it;
  g.trial_slot = 0;
  g.graph_builds = 0;
  SMD_CUDA(cudaMemcpy(P.g, &g, sizeof(Global), cudaMemcpyHostToDevice));
  if ((rc = rebuild_if_needed(h.get()))) return rc;
  if ((rc = read_error(h.get()))) return rc;
  *out = h.release();
  return 0;
}

void smd_destroy(smd_system* h) { delete h; }

int smd_set_stream(smd_system* h, void* s) {
  if (!h) return fail(1, "null handle");
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  h->own_stream = (s == nullptr);
  if (s == nullptr) {
    SMD_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  } else {
    h->stream = (cudaStream_t)s;
  }
  return 0;
}

int smd_get_state(smd_system* h, double* pos, double* vel) {
  if (!h) return fail(1, "null handle");
  if (!pos && !vel) return 0;
  if (int rc = xfer_buffer(h)) return rc;
  const size_t n3 = (size_t)h->n * 3;
  double* xs = h->xfer;
  double* vs = h->xfer + n3;
  SMD_LAUNCH(h, k_state_save<<<h->grid(), kBlock, 0, h->stream>>>(h->P, pos ? xs : nullptr, vel ? vs : nullptr));
  if (pos) SMD_CUDA(cudaMemcpyAsync(pos, xs, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (vel) SMD_CUDA(cudaMemcpyAsync(vel, vs, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return 0;
}

int smd_set_state(smd_system* h, const double* pos, const double* vel) {
  if (!h) return fail(1, "null handle");
  if (!pos && !vel) return 0;
  if (int rc = xfer_buffer(h)) return rc;
  auto& P = h->P;
  const size_t n3 = (size_t)h->n * 3;
  double* xs = h->xfer;
  double* vs = h->xfer + n3;
  if (pos) SMD_CUDA(cudaMemcpyAsync(xs, pos, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (vel) SMD_CUDA(cudaMemcpyAsync(vs, vel, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SMD_LAUNCH(h, k_state_check<<<h->grid(), kBlock, 0, h->stream>>>(P, pos ? xs : nullptr, vel ? vs : nullptr));
  {
    Global g;
    SMD_CUDA(cudaMemcpyAsync(&g, P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream));
    SMD_CUDA(cudaStreamSynchronize(h->stream));
    if (g.error & 4) {
      g.error &= ~4;
      SMD_CUDA(cudaMemcpy(P.g, &g, sizeof(Global), cudaMemcpyHostToDevice));
      return fail(9, "smd_set_state: a position outside its replica's box or not finite, or a velocity that is "
                     "not finite (the handle's state is unchanged)");
    }
  }
  SMD_LAUNCH(h, k_state_load<<<h->grid(), kBlock, 0, h->stream>>>(P, pos ? xs : nullptr, vel ? vs : nullptr));
  if (pos) {
    if (h->mixed)
      SMD_LAUNCH(h, k_mirror<true><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
    else
      SMD_LAUNCH(h, k_mirror<false><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur));
    SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(P.g, 1));
  }
  if (pos) {
    // a new configuration may be denser than the list was sized for: build,
    // and if a bead overflowed, grow the list to its count and build again
    if (int rc = force_rebuild(h)) return rc;
    Global g;
    SMD_CUDA(cudaMemcpyAsync(&g, P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream));
    SMD_CUDA(cudaStreamSynchronize(h->stream));
    if (g.error & 1) {
      const int need = std::max(g.need_nbr, g.max_nbr);
      g.error &= ~1;
      g.need_nbr = 0;
      SMD_CUDA(cudaMemcpy(P.g, &g, sizeof(Global), cudaMemcpyHostToDevice));
      if (int rc = grow_list(h, need)) return rc;
    }
  }
  return read_error(h);  // synchronises the stream
}

int smd_get_box(smd_system* h, int replica, double box[3]) {
  if (!h || !box || replica < 0 || replica >= h->n_rep) return fail(1, "bad arguments");
  RepState rs;
  SMD_CUDA(cudaMemcpyAsync(&rs, h->P.rs + replica, sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 3; ++k) box[k] = rs.box[k];
  return 0;
}

int smd_set_box(smd_system* h, int replica, const double box[3]) {
  if (!h || !box || replica < 0 || replica >= h->n_rep) return fail(1, "bad arguments");
  for (int k = 0; k < 3; ++k)
    if (!(box[k] > 0) || !std::isfinite(box[k]) || int(box[k] / h->tab.rc) < 3)
      return fail(1, "box edge not finite or shorter than 3 cutoffs");
  RepState rs;
  SMD_CUDA(cudaMemcpyAsync(&rs, h->P.rs + replica, sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 3; ++k) rs.box[k] = box[k];
  derive_box(rs, h->rp[replica].cell_cap, h->tab.list_cut, h->tab.rc);
  SMD_CUDA(cudaMemcpyAsync(h->P.rs + replica, &rs, sizeof(RepState), cudaMemcpyHostToDevice, h->stream));
  if (h->mixed)
    SMD_LAUNCH(h, k_mirror<true><<<h->grid(), kBlock, 0, h->stream>>>(h->P, h->cur));
  else
    SMD_LAUNCH(h, k_mirror<false><<<h->grid(), kBlock, 0, h->stream>>>(h->P, h->cur));
  SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(h->P.g, 1));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return 0;
}

static int compute_forces_impl(smd_system* h, double* out, bool pair_only) {
  if (!h || !out) return fail(1, "bad arguments");
  int rc = rebuild_if_needed(h, true);
  if (rc) return rc;
  rc = pair_only ? launch_step<F_FORCES | F_PAIRONLY>(h) : launch_step<F_FORCES>(h);
  if (rc) return rc;
  SMD_CUDA(cudaMemcpyAsync(out, h->P.force_out, 3 * h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return read_error(h);
}

int smd_compute_forces(smd_system* h, double* out) { return compute_forces_impl(h, out, false); }
int smd_compute_pair_forces(smd_system* h, double* out) { return compute_forces_impl(h, out, true); }

int smd_compute_energy(smd_system* h, smd_energy* e) {
  if (!h || !e) return fail(1, "bad arguments");
  int rc = rebuild_if_needed(h, true);
  if (rc) return rc;
  // the energy sums are cleared on the device: no host round trip before the pass
  SMD_LAUNCH(h, k_clear_energy<<<(h->n_rep + 63) / 64, 64, 0, h->stream>>>(h->P));
  if ((rc = launch_step<F_ENERGY>(h))) return rc;
  std::vector<RepState> rs(h->n_rep);
  SMD_CUDA(cudaMemcpyAsync(rs.data(), h->P.rs, h->n_rep * sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  if ((rc = read_error(h))) return rc;  // its synchronisation also completes the copy above
  for (int r = 0; r < h->n_rep; ++r) {
    e[r].pair = rs[r].e_pair;
    e[r].bonded = rs[r].e_bond;
    e[r].sphere = rs[r].e_sphere;
    e[r].kinetic = rs[r].e_kin;
  }
  return 0;
}

int smd_compute_dU(smd_system* h, const double scale[3], double* dU) {
  if (!h || !scale || !dU) return fail(1, "bad arguments");
  int rc = rebuild_if_needed(h, true);
  if (rc) return rc;
  std::vector<RepState> rs(h->n_rep);
  SMD_CUDA(cudaMemcpyAsync(rs.data(), h->P.rs, h->n_rep * sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<RepState> saved = rs;
  for (auto& s : rs) {
    s.dU_pair = s.dU_bond = 0;
    s.dUq_pair = s.dUq_bond = 0;
    set_scale(s, scale);
  }
  SMD_CUDA(cudaMemcpyAsync(h->P.rs, rs.data(), h->n_rep * sizeof(RepState), cudaMemcpyHostToDevice, h->stream));
  if ((rc = launch_step<F_DU | F_ENERGY>(h))) return rc;
  SMD_CUDA(cudaMemcpyAsync(rs.data(), h->P.rs, h->n_rep * sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  for (int r = 0; r < h->n_rep; ++r) dU[r] = rep_dU(rs[r]);
  SMD_CUDA(cudaMemcpyAsync(h->P.rs, saved.data(), h->n_rep * sizeof(RepState), cudaMemcpyHostToDevice, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return read_error(h);
}

int smd_cell_keys(smd_system* h, int* keys) {
  if (!h || !keys) return fail(1, "bad arguments");
  SMD_LAUNCH(h, k_ref_keys<<<h->grid(), kBlock, 0, h->stream>>>(h->P));
  SMD_CUDA(cudaMemcpyAsync(keys, h->P.key_out, h->n * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return 0;
}

int smd_pair_list(smd_system* h, int* pairs, size_t cap, size_t* count) {
  if (!h || !count) return fail(1, "bad arguments");
  int rc = rebuild_if_needed(h, true);
  if (rc) return rc;
  int* dpairs = nullptr;
  unsigned long long* dcount = nullptr;
  SMD_CUDA(cudaMallocAsync((void**)&dpairs, std::max<size_t>(cap, 1) * 2 * sizeof(int), h->stream));
  SMD_CUDA(cudaMallocAsync((void**)&dcount, sizeof(unsigned long long), h->stream));
  SMD_CUDA(cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), h->stream));
  SMD_LAUNCH(h, k_pairs<<<h->grid(), kBlock, 0, h->stream>>>(h->P, dpairs, (long long)cap, dcount));
  unsigned long long c = 0;
  SMD_CUDA(cudaMemcpyAsync(&c, dcount, sizeof c, cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (pairs && cap)
    SMD_CUDA(cudaMemcpy(pairs, dpairs, std::min<size_t>(cap, c) * 2 * sizeof(int), cudaMemcpyDeviceToHost));
  SMD_CUDA(cudaFreeAsync(dpairs, h->stream));
  SMD_CUDA(cudaFreeAsync(dcount, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  *count = (size_t)c;
  return 0;
}

int smd_set_noise_once(smd_system* h, const double* psi) {
  if (!h || !psi) return fail(1, "bad arguments");
  // on the handle's stream: a step launched with SMD_ASYNC may still be
  // reading the previous draws (the stream does not wait for the legacy one)
  SMD_CUDA(cudaMemcpyAsync(h->P.ext_noise, psi, 3 * h->n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  h->ext_noise_pending = true;
  return 0;
}

int smd_prepare(smd_system* h, int do_second, smd_energy* energy_out) {
  if (!h) return fail(1, "null handle");
  SMD_LAUNCH(h, k_set_counters<<<1, 1, 0, h->stream>>>(h->P.g, h->it, 1, 0, 0));
  int rc = force_rebuild(h);
  if (rc) return rc;
  if (h->ext_noise_pending) {
    rc = launch_step<F_INIT | F_EXTNOISE>(h);
    h->ext_noise_pending = false;
  } else {
    rc = launch_step<F_INIT>(h);
  }
  if (rc) return rc;
  if (energy_out && (rc = smd_compute_energy(h, energy_out))) return rc;
  if ((rc = launch_finish(h, do_second ? 1 : 0, 0, StepEnd{0, 0, 0, 0, 0}))) return rc;
  h->at_measure = false;
  h->it = h->first_step[0];
  SMD_LAUNCH(h, k_set_counters<<<1, 1, 0, h->stream>>>(h->P.g, h->it, 1, 0, 0));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return read_error(h);
}

// Captures one MC period (resize_rate steps, the trial step last) as a graph
// for mirror parity cur0.  Step s: IF(rebuild) { list build } then the step
// kernels; the kernel completing step s sets the condition of step s+1.
int capture_period(smd_system* h, int cur0) {
  const int G = h->resize_rate;
  auto& P = h->P;
  if (!h->side) SMD_CUDA(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
  const long saved_launches = h->launches;
  const int saved_cur = h->cur;
  cudaStream_t st = h->stream;
  SMD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  cudaGraph_t graph = nullptr;
  auto body = [&]() -> int {
    cudaStreamCaptureStatus status;
    SMD_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, &graph, nullptr, nullptr, nullptr));
    std::vector<cudaGraphConditionalHandle> cond(G);
    for (int k = 0; k < G; ++k) SMD_CUDA(cudaGraphConditionalHandleCreate(&cond[k], graph, 0, 0));
    SMD_LAUNCH(h, k_graph_cond<<<1, 1, 0, st>>>(P.g, (unsigned long long)cond[0]));
    for (int k = 0; k < G; ++k) {
      const int cur = cur0 ^ (k & 1);
      const cudaGraphNode_t* deps = nullptr;
      size_t ndeps = 0;
      SMD_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, &graph, &deps, nullptr, &ndeps));
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = cond[k];
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      SMD_CUDA(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
      cudaGraph_t build = cp.conditional.phGraph_out[0];
      SMD_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
      SMD_CUDA(cudaStreamBeginCaptureToGraph(h->side, build, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      const int rc1 = launch_rebuild(h, h->side, cur, 1);
      SMD_CUDA(cudaStreamEndCapture(h->side, &build));
      if (rc1) return rc1;
      h->cur = cur;
      const bool last = (k == G - 1);
      const StepEnd se{last ? 0ull : (unsigned long long)cond[k + 1], last ? 0 : 1, 1, 0, 0};
      if (last && h->barostat) {
        if (int r = launch_step<F_STOP | F_DU>(h)) return r;  // the trial is drawn in its first kernel
        SMD_LAUNCH(h, k_mc<<<(h->n_rep + 63) / 64, 64, 0, st>>>(P));
        if (int r = launch_finish(h, 2, 1, StepEnd{0, 0, 1, 1, 0})) return r;
      } else {
        if (int r = launch_step<0>(h, se)) return r;
      }
    }
    return 0;
  };
  rc = body();
  cudaGraph_t done = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &done);
  h->cur = saved_cur;
  const long kernels = h->launches - saved_launches - (long)G * rebuild_kernels(h);
  h->launches = saved_launches;
  if (rc) {
    if (done) cudaGraphDestroy(done);
    return rc;
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // reported here, not by the next launch check
    return fail(100 + (int)e, std::string("graph capture: ") + cudaGetErrorString(e));
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e2 = cudaGraphInstantiate(&exec, done, 0);
  cudaGraphDestroy(done);
  if (e2 != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(100 + (int)e2, std::string("graph instantiate: ") + cudaGetErrorString(e2));
  }
  h->graph[cur0].exec = exec;
  h->graph[cur0].kernels = (int)kernels;
  return 0;
}

// ------------------------------------------------------------ autotuner
// Times the list-build variants (whole rebuild sequence) and the pair pass at
// 4, 8 and 16 lanes per bead on the handle's own state with CUDA events and
// keeps the fastest of each.  Both are safe to repeat on a live state: a
// rebuild re-sorts the same positions, the pair pass only writes its scratch
// accumulator.  Choices are cached per device and system shape.
struct TuneKey {
  int dev, n, n_rep, n_cells;
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, n, n_rep, n_cells) < std::tie(o.dev, o.n, o.n_rep, o.n_cells);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tune_cache;

int time_ms(smd_system* h, const std::function<int()>& work, int reps, float* best) {
  cudaEvent_t a, b;
  SMD_CUDA(cudaEventCreate(&a));
  SMD_CUDA(cudaEventCreate(&b));
  float m = 1e30f;
  int rc = 0;
  for (int k = 0; k < reps && !rc; ++k) {
    cudaEventRecord(a, h->stream);
    rc = work();
    cudaEventRecord(b, h->stream);
    if (cudaEventSynchronize(b) != cudaSuccess) rc = fail(2, "autotune: event synchronisation failed");
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    m = std::min(m, t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *best = m;
  return rc;
}

void drop_graphs(smd_system* h) {
  for (auto& gr : h->graph)
    if (gr.exec) {
      cudaGraphExecDestroy(gr.exec);
      gr.exec = nullptr;
    }
}

int autotune(smd_system* h, bool force) {
  if (!h->mixed || (h->tune.done && !force)) return 0;
  int dev = 0;
  SMD_CUDA(cudaGetDevice(&dev));
  const TuneKey key{dev, h->n, h->n_rep, h->n_cells};
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      h->tune.lanes = it->second.first;
      h->tune.list = it->second.second;
      h->tune.done = true;
      drop_graphs(h);
      return 0;
    }
  }
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (int rc = complete_pending(h)) return rc;
  const long saved = h->launches;
  auto& P = h->P;
  // the tuning rebuilds are not list rebuilds of the run: keep the count
  long long rebuilds0 = 0;
  SMD_CUDA(cudaMemcpy(&rebuilds0, &P.g->n_rebuilds, sizeof rebuilds0, cudaMemcpyDeviceToHost));
  int best_list = 0;
  for (int v = 0; v < 3; ++v) {
    h->tune.list = v;
    int rc = time_ms(h, [&]() -> int {
      SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(P.g, 1));
      return rebuild_if_needed(h, true);
    }, 3, &h->tune.ms_list[v]);
    if (rc) return rc;
    if (h->tune.ms_list[v] < h->tune.ms_list[best_list]) best_list = v;
  }
  h->tune.list = best_list;
  // leave a list built by the chosen kernel
  SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(P.g, 1));
  if (int rc = rebuild_if_needed(h, true)) return rc;
  const int lanes[3] = {4, 8, 16};
  int best_lanes = 1;
  for (int v = 0; v < 3; ++v) {
    h->tune.lanes = lanes[v];
    int rc = time_ms(h, [&]() -> int { return launch_force_only(h); }, 5, &h->tune.ms_force[v]);
    if (rc) return rc;
    if (h->tune.ms_force[v] < h->tune.ms_force[best_lanes]) best_lanes = v;
  }
  h->tune.lanes = lanes[best_lanes];
  h->tune.done = true;
  h->launches = saved;  // tuning launches are not step work
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  SMD_CUDA(cudaMemcpy(&P.g->n_rebuilds, &rebuilds0, sizeof rebuilds0, cudaMemcpyHostToDevice));
  drop_graphs(h);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {h->tune.lanes, h->tune.list};
  }
  return read_error(h);
}

bool autotune_enabled() {
  const char* e = std::getenv("SMD_AUTOTUNE");
  return !(e && e[0] == '0');
}

// A period graph can run from step `it` when its trial step (the last) is a
// barostat step of the reference loop, i.e. it % resize_rate == 1.
bool graph_fits(const smd_system* h, long long it, int left) {
  const int G = h->resize_rate;
  if (!h->use_graphs || h->profile || h->ext_noise_pending || G < 2 || (G & 1) || left < G) return false;
  if (h->stream == nullptr) return false;  // the legacy stream cannot be captured
  return (it % G) == 1;
}

int smd_advance(smd_system* h, int steps, int flags) {
  if (!h || steps < 0) return fail(1, "bad arguments");
  const bool stop_at_measure = (flags & SMD_STOP_AT_MEASURE) != 0;
  const bool async = (flags & SMD_ASYNC) != 0;
  int rc = complete_pending(h);
  if (rc) return rc;
  // tune once the system has relaxed from its start (a lattice start is far
  // sparser than the running membrane and favours other kernels)
  if (!h->tune.done && h->it - h->first_step[0] >= 256 && autotune_enabled() && (rc = autotune(h, false)))
    return rc;
  int done = 0;
  while (done < steps) {
    const int chunk = std::min(steps - done, kTrialChunk * std::max(1, h->resize_rate) / 2);
    if ((rc = stage_trials(h, h->it, chunk))) return rc;
    for (int s = 0; s < chunk; ++s) {
      // the last step of a stopping call runs alone (it stops after its second half-kick)
      const int left = chunk - s - ((stop_at_measure && done + chunk == steps) ? 1 : 0);
      if (graph_fits(h, h->it, left)) {
        auto& g = h->graph[h->cur];
        if (!g.exec && (rc = capture_period(h, h->cur))) return rc;
        SMD_CUDA(cudaGraphLaunch(g.exec, h->stream));
        h->launches += g.kernels;
        h->it += h->resize_rate;
        if (h->barostat) h->trials_used++;
        s += h->resize_rate - 1;
        continue;
      }
      if ((rc = rebuild_if_needed(h))) return rc;
      const bool trial = is_trial_step(h, h->it);
      const bool stop = stop_at_measure && (done + s == steps - 1);
      const bool ext = h->ext_noise_pending;
      h->ext_noise_pending = false;
      if (!trial && !stop) {
        rc = ext ? launch_step<F_EXTNOISE>(h) : launch_step<0>(h);
        if (rc) return rc;
        h->cur ^= 1;
        h->it++;
        continue;
      }
      if (trial) {
        h->trials_used++;
        rc = ext ? launch_step<F_STOP | F_DU | F_EXTNOISE>(h) : launch_step<F_STOP | F_DU>(h);
      } else {
        rc = ext ? launch_step<F_STOP | F_EXTNOISE>(h) : launch_step<F_STOP>(h);
      }
      if (rc) return rc;
      h->at_measure = true;
      h->pending_trial = trial;
      if (stop) break;
      if ((rc = complete_pending(h))) return rc;
    }
    done += chunk;
  }
  if (async) return 0;
  return smd_sync(h);
}

int smd_autotune(smd_system* h, int force, int* lanes, int* list_kernel, float* ms) {
  if (!h) return fail(1, "null handle");
  if (int rc = autotune(h, force != 0)) return rc;
  if (lanes) *lanes = h->tune.lanes;
  if (list_kernel) *list_kernel = h->tune.list;
  if (ms)
    for (int k = 0; k < 3; ++k) {
      ms[k] = h->tune.ms_list[k];
      ms[3 + k] = h->tune.ms_force[k];
    }
  return 0;
}

int smd_set_tuning(smd_system* h, int lanes, int list_kernel) {
  if (!h) return fail(1, "null handle");
  if (!(lanes == 4 || lanes == 8 || lanes == 16) || list_kernel < 0 || list_kernel > 2)
    return fail(1, "lanes must be 4, 8 or 16 and list_kernel 0, 1 or 2");
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  h->tune.lanes = lanes;
  h->tune.list = list_kernel;
  h->tune.done = true;
  drop_graphs(h);
  return 0;
}

int smd_use_graphs(smd_system* h, int on) {
  if (!h) return fail(1, "null handle");
  h->use_graphs = on != 0;
  return 0;
}

int smd_sync(smd_system* h) {
  if (!h) return fail(1, "null handle");
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (int rc = collect_profile(h)) return rc;
  if (!h->at_measure || !h->pending_trial) {
    if (int e = flush_mc_log(h)) return e;
  }
  return read_error(h);
}

int smd_profile(smd_system* h, int on) {
  if (!h) return fail(1, "null handle");
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (int rc = collect_profile(h)) return rc;
  h->profile = on != 0;
  h->step_ms = 0;
  h->step_launches = 0;
  return 0;
}

int smd_mc_stats_get(smd_system* h, int replica, smd_mc_stats* out) {
  if (!h || !out || replica < 0 || replica >= h->n_rep) return fail(1, "bad arguments");
  RepState rs;
  SMD_CUDA(cudaMemcpyAsync(&rs, h->P.rs + replica, sizeof(RepState), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  out->trials = (long)rs.n_trial;
  out->accepted = (long)rs.n_accept;
  out->last_dU = rs.last_dU;
  return 0;
}

long smd_mc_log(smd_system* h, int replica, long start, long max, double* fluct, int* accepted) {
  if (!h || replica < 0 || replica >= h->n_rep || start < 0 || max < 0) return -fail(1, "bad arguments");
  if (!h->at_measure || !h->pending_trial) {
    if (flush_mc_log(h)) return -1;
  }
  const auto& f = h->mc_fluct[replica];
  const auto& a = h->mc_accept[replica];
  long n = 0;
  for (long k = start; k < (long)f.size() && n < max; ++k, ++n) {
    if (fluct) fluct[n] = f[k];
    if (accepted) accepted[n] = a[k];
  }
  return n;
}

int smd_set_temperature(smd_system* h, int replica, double kT, int update_sigma) {
  if (!h || replica < -1 || replica >= h->n_rep) return fail(1, "bad arguments");
  if (!std::isfinite(kT) || kT < 0) return fail(1, "temperature must be finite and not negative");
  for (int r = 0; r < h->n_rep; ++r) {
    if (replica >= 0 && r != replica) continue;
    h->rp[r].kT = kT;
    if (update_sigma) {
      h->rp[r].sigma = std::sqrt((6.0 * kT * h->rp[r].gamma) / h->rp[r].dt);
      h->rp[r].sig31 = h->rp[r].sigma * (1.0 / 2147483648.0);
      h->rp[r].sig31f = (float)h->rp[r].sig31;
    }
  }
  SMD_CUDA(cudaMemcpyAsync(h->P.rp, h->rp.data(), h->n_rep * sizeof(RepParams), cudaMemcpyHostToDevice,
                           h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return 0;
}

int smd_last_timing(smd_system* h, double* ms, long* step_launches, long* launches) {
  if (!h) return fail(1, "null handle");
  if (ms) *ms = h->step_ms;
  if (step_launches) *step_launches = h->step_launches;
  // list-build kernels that ran inside graph conditional bodies count too
  if (launches) *launches = h->launches + (long)(h->graph_builds * rebuild_kernels(h));
  return 0;
}

int smd_list_state(smd_system* h, double* max_disp, double* slack) {
  if (!h) return fail(1, "null handle");
  Global g;
  SMD_CUDA(cudaMemcpyAsync(&g, h->P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (max_disp) *max_disp = g.last_disp;
  if (slack) *slack = g.slack;
  return 0;
}

long smd_rebuild_count(smd_system* h) {
  if (!h) return -1;
  Global g;
  if (cudaMemcpyAsync(&g, h->P.g, sizeof(Global), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return -1;
  return (long)g.n_rebuilds;
}

int smd_start_diffusion(smd_system* h) {
  if (!h) return fail(1, "null handle");
  auto& M = h->meas;
  if (!h->P.disp) {
    double* d = nullptr;
    if (int rc = h->alloc(&d, 3 * (size_t)h->n)) return rc;
    h->P.disp = d;
  }
  SMD_CUDA(cudaMemsetAsync(h->P.disp, 0, 3 * sizeof(double) * (size_t)h->n, h->stream));
  if (!M.tracking) {
    M.tracking = true;
    drop_graphs(h);  // the captured periods have no tracking kernel
  }
  return 0;
}

int smd_set_msd_groups(smd_system* h, int n_groups, const int* offsets, const int* beads) {
  if (!h) return fail(1, "null handle");
  if (n_groups < 0 || (n_groups > 0 && !offsets)) return fail(1, "bad measurement groups");
  auto& M = h->meas;
  const int total = n_groups > 0 ? offsets[n_groups] : 0;
  if (n_groups > 0 && (offsets[0] != 0 || total < 0 || (total > 0 && !beads)))
    return fail(1, "measurement group offsets must start at 0");
  int widest = 0;
  for (int g = 0; g < n_groups; ++g) {
    if (offsets[g + 1] < offsets[g]) return fail(1, "measurement group offsets must not decrease");
    widest = std::max(widest, offsets[g + 1] - offsets[g]);
  }
  for (int k = 0; k < total; ++k)
    if (beads[k] < 0 || beads[k] >= h->n) return fail(1, "measurement group bead index out of range");
  if (n_groups > 0) {
    int* off = nullptr;
    int* bd = nullptr;
    double* out = nullptr;
    if (int rc = h->alloc(&off, (size_t)n_groups + 1)) return rc;
    if (int rc = h->alloc(&bd, (size_t)std::max(total, 1))) return rc;
    if (int rc = h->alloc(&out, (size_t)n_groups)) return rc;
    SMD_CUDA(cudaMemcpy(off, offsets, sizeof(int) * ((size_t)n_groups + 1), cudaMemcpyHostToDevice));
    if (total > 0) SMD_CUDA(cudaMemcpy(bd, beads, sizeof(int) * (size_t)total, cudaMemcpyHostToDevice));
    M.off = off;
    M.beads = bd;
    M.msd = out;
  }
  M.n_groups = n_groups;
  M.max_group = widest;
  return 0;
}

int smd_measure(smd_system* h, smd_measurement* out, double* msd_sum) {
  if (!h || !out) return fail(1, "bad arguments");
  if (h->n_rep != 1) return fail(1, "smd_measure runs on single-system handles");
  auto& M = h->meas;
  auto& P = h->P;
  if (!M.acc) {
    if (int rc = h->alloc(&M.acc, 1)) return rc;
    M.cap = 1 << 20;  // kinetic energies below 104.8576 per bead
    if (int rc = h->alloc(&M.hist, (size_t)M.cap)) return rc;
  }
  MeasureAcc a{};
  for (int d = 0; d < 3; ++d) {
    a.lo[d] = ~0ull;
    a.hi[d] = 0ull;
  }
  a.max_bin = -1;
  SMD_CUDA(cudaMemcpyAsync(M.acc, &a, sizeof a, cudaMemcpyHostToDevice, h->stream));
  SMD_LAUNCH(h, k_measure<<<h->grid(), kBlock, 0, h->stream>>>(P, M.acc, M.hist, M.cap));
  const bool msd = M.tracking && M.n_groups > 0 && msd_sum;
  if (msd) {
    SMD_CUDA(cudaMemsetAsync(M.msd, 0, sizeof(double) * (size_t)M.n_groups, h->stream));
    const dim3 grid((unsigned)std::max(1, (M.max_group + kMsdChunk - 1) / kMsdChunk), (unsigned)M.n_groups);
    SMD_LAUNCH(h, k_msd<<<grid, kBlock, 0, h->stream>>>(P, M.off, M.beads, M.msd));
  }
  SMD_CUDA(cudaMemcpyAsync(&a, M.acc, sizeof a, cudaMemcpyDeviceToHost, h->stream));
  if (msd)
    SMD_CUDA(cudaMemcpyAsync(msd_sum, M.msd, sizeof(double) * (size_t)M.n_groups, cudaMemcpyDeviceToHost,
                             h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  if (a.max_bin >= M.cap) {  // grow the histogram and add the bins that did not fit
    constexpr int kMaxBins = 1 << 26;
    if (a.max_bin >= kMaxBins)
      return fail(10, "a bead's kinetic energy exceeds the measurement histogram (" +
                          std::to_string(kMaxBins / 10000) + " per bead): the run has blown up");
    int cap = M.cap;
    while (cap <= a.max_bin) cap *= 2;
    unsigned int* nh = nullptr;
    if (int rc = h->alloc(&nh, (size_t)cap)) return rc;
    SMD_CUDA(cudaMemcpyAsync(nh, M.hist, sizeof(unsigned int) * (size_t)M.cap, cudaMemcpyDeviceToDevice, h->stream));
    SMD_LAUNCH(h, k_measure_bins<<<h->grid(), kBlock, 0, h->stream>>>(P, nh, M.cap, cap));
    SMD_CUDA(cudaStreamSynchronize(h->stream));
    for (auto& q : h->allocs)
      if (q == (void*)M.hist) {
        cudaFree(q);
        q = nullptr;
      }
    M.hist = nh;
    M.cap = cap;
  }
  out->kinetic = a.kinetic;
  for (int d = 0; d < 3; ++d) {
    std::memcpy(&out->lo[d], &a.lo[d], sizeof(double));
    std::memcpy(&out->hi[d], &a.hi[d], sizeof(double));
  }
  out->bond_length_sum = a.lbond;
  out->n_bond = a.n_bond;
  out->bend_cos_sum = a.cos_bend;
  out->bend_len0_sum = a.l_bend0;
  out->bend_len1_sum = a.l_bend1;
  out->n_bend = a.n_bend;
  out->msd = msd ? 1 : 0;
  return 0;
}

int smd_ke_histogram(smd_system* h, long* counts, size_t cap, size_t* n_bins) {
  if (!h || !n_bins) return fail(1, "bad arguments");
  auto& M = h->meas;
  *n_bins = 0;
  if (!M.hist) return 0;
  std::vector<unsigned int> hc((size_t)M.cap);
  SMD_CUDA(cudaMemcpyAsync(hc.data(), M.hist, sizeof(unsigned int) * hc.size(), cudaMemcpyDeviceToHost,
                           h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  size_t nb = hc.size();
  while (nb > 0 && hc[nb - 1] == 0) --nb;
  *n_bins = nb;
  if (counts)
    for (size_t k = 0; k < std::min(cap, nb); ++k) counts[k] = (long)hc[k];
  return 0;
}

}  // extern "C"

// ------------------------------------------------------------------ adjoint
namespace {

int adj_alloc(smd_system* h) {
  auto& A = h->adj;
  if (A.acc) return 0;
  const size_t n3 = 3 * (size_t)h->n;
  int rc;
  if ((rc = h->alloc(&A.w0, n3)) || (rc = h->alloc(&A.w1, n3)) || (rc = h->alloc(&A.xbar, n3)) ||
      (rc = h->alloc(&A.hbar, n3)) || (rc = h->alloc(&A.kw, n3)) || (rc = h->alloc(&A.fpair, n3)) ||
      (rc = h->alloc(&A.out, n3)) || (rc = h->alloc(&A.ws, (size_t)h->n)) || (rc = h->alloc(&A.acc, 1)) ||
      (rc = h->alloc(&A.tab, 1)))
    return rc;
  return 0;
}

// K w (pair part into adj.kw, forces into adj.fpair) at the current
// positions for w in file order on the device; adds to the accumulators.
int adj_pair_pass(smd_system* h, const double* w, double dt, double invT) {
  auto& P = h->P;
  auto& A = h->adj;
  const int g = h->grid(), gl = h->grid_lanes();
  if (h->mixed) {
    float4* ws = reinterpret_cast<float4*>(A.ws);
    SMD_LAUNCH(h, k_adj_wsort<float4><<<g, kBlock, 0, h->stream>>>(P, w, ws));
    SMD_LAUNCH(h, (k_adj_pair<true, kLanes><<<gl, kBlock, 0, h->stream>>>(P, h->cur, A.tab, ws, A.kw, A.fpair,
                                                                            A.acc, dt, invT)));
  } else {
    SMD_LAUNCH(h, k_adj_wsort<double4><<<g, kBlock, 0, h->stream>>>(P, w, A.ws));
    SMD_LAUNCH(h, (k_adj_pair<false, kLanes><<<gl, kBlock, 0, h->stream>>>(P, h->cur, A.tab, A.ws, A.kw,
                                                                             A.fpair, A.acc, dt, invT)));
  }
  return 0;
}

// Positions (and velocities) in file order into the handle; the list is
// rebuilt when they moved too far from its build positions (force: always).
int adj_load(smd_system* h, const double* xs, const double* vs, bool force) {
  auto& P = h->P;
  if (h->mixed)
    SMD_LAUNCH(h, k_adj_load<true><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur, xs, vs));
  else
    SMD_LAUNCH(h, k_adj_load<false><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur, xs, vs));
  if (force) SMD_LAUNCH(h, k_set_rebuild<<<1, 1, 0, h->stream>>>(P.g, 1));
  return rebuild_if_needed(h, true);
}

int adj_check_handle(smd_system* h) {
  if (!h) return fail(1, "null handle");
  if (h->n_rep != 1) return fail(1, "the adjoint runs on single-system handles");
  if (h->n_sph) return fail(1, "the adjoint does not cover BEAD or NANOCORE residues");
  if (h->n_terms) return fail(1, "the adjoint does not cover BOND / BEND or external-field residues");
  return 0;
}

}  // namespace

extern "C" {

int smd_hessian_vector(smd_system* h, const double* w, double* kw) {
  if (int rc = adj_check_handle(h)) return rc;
  if (!w || !kw) return fail(1, "bad arguments");
  if (int rc = complete_pending(h)) return rc;
  if (int rc = adj_alloc(h)) return rc;
  auto& A = h->adj;
  const size_t n3 = 3 * (size_t)h->n;
  if (int rc = rebuild_if_needed(h, true)) return rc;
  SMD_CUDA(cudaMemcpyAsync(A.w0, w, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (int rc = adj_pair_pass(h, A.w0, 0.0, 0.0)) return rc;
  if (h->mixed)
    SMD_LAUNCH(h, k_adj_hvp_out<true><<<h->grid(), kBlock, 0, h->stream>>>(h->P, h->cur, A.w0, A.kw, A.out));
  else
    SMD_LAUNCH(h, k_adj_hvp_out<false><<<h->grid(), kBlock, 0, h->stream>>>(h->P, h->cur, A.w0, A.kw, A.out));
  SMD_CUDA(cudaMemcpyAsync(kw, A.out, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SMD_CUDA(cudaStreamSynchronize(h->stream));
  return read_error(h);
}

int smd_adjoint(smd_system* h, const smd_adjoint_spec* spec, smd_adjoint_result* out) {
  if (int rc = adj_check_handle(h)) return rc;
  if (!spec || !out || spec->steps < 1 || spec->checkpoint_every < 1) return fail(1, "bad adjoint spec");
  const int nT = h->tab.nT;
  const int ta = spec->umin_types[0], tb = spec->umin_types[1];
  if (ta < 0 || tb < 0 || ta >= nT || tb >= nT) return fail(1, "Umin type pair out of range");
  if (h->barostat) return fail(1, "the adjoint holds the box fixed: switch the barostat off (delta_lxy 0)");
  if (int rc = complete_pending(h)) return rc;
  if (int rc = adj_alloc(h)) return rc;
  auto& P = h->P;
  auto& A = h->adj;
  const int T = spec->steps, K = spec->checkpoint_every;
  const int ncp = (int)(((long long)T + K - 1) / K);
  const size_t n3 = 3 * (size_t)h->n;
  const double dt = h->dt, invT = 1.0 / T;
  // derivative rows of Umin(a, b): the tables are linear in Umin
  {
    AdjTables at;
    std::memset(&at, 0, sizeof at);
    for (int q = 0; q < 2; ++q) {
      const int row = q == 0 ? (ta * nT + tb) : (tb * nT + ta);
      const double rm = h->tab.dF[6 * row], rc = h->tab.dF[6 * row + 3], w = rc - rm;
      const double dF[6] = {rm, -2.0 / (rm * rm), 0.0, rc, 6.0 / (w * w), 6.0 / (w * w * w)};
      const double dU[6] = {rm, -1.0 / (rm * rm), 1.0, rc, 3.0 / (w * w), 2.0 / (w * w * w)};
      for (int k = 0; k < 6; ++k) {
        at.dF[6 * row + k] = dF[k];
        at.dU[6 * row + k] = dU[k];
        at.fF[6 * row + k] = (float)dF[k];
        at.fU[6 * row + k] = (float)dU[k];
      }
    }
    SMD_CUDA(cudaMemcpyAsync(A.tab, &at, sizeof at, cudaMemcpyHostToDevice, h->stream));
    SMD_CUDA(cudaStreamSynchronize(h->stream));
  }
  // storage of this call: checkpoints (x, h), one segment of positions, the end state
  double *cp = nullptr, *seg = nullptr, *fin = nullptr;
  auto release = [&]() {
    if (cp) cudaFree(cp);
    if (seg) cudaFree(seg);
    if (fin) cudaFree(fin);
  };
  if (cudaMalloc(&cp, (size_t)ncp * 2 * n3 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&seg, (size_t)K * n3 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&fin, 2 * n3 * sizeof(double)) != cudaSuccess) {
    (void)cudaGetLastError();  // an allocation failure is not the next launch's error
    release();
    return fail(2, "cudaMalloc of the adjoint checkpoints failed");
  }
  std::vector<long long> cp_it(ncp);
  int rc = 0;
  auto body = [&]() -> int {
    // ---- forward: the state at the start of every segment
    for (int c = 0; c < ncp; ++c) {
      double* x = cp + (size_t)c * 2 * n3;
      SMD_LAUNCH(h, k_state_save<<<h->grid(), kBlock, 0, h->stream>>>(P, x, x + n3));
      cp_it[c] = h->it;
      const int len = std::min(K, T - c * K);
      if (int r = smd_advance(h, len, SMD_ASYNC)) return r;
    }
    SMD_LAUNCH(h, k_state_save<<<h->grid(), kBlock, 0, h->stream>>>(P, fin, fin + n3));
    const long long it_end = h->it;
    SMD_CUDA(cudaMemsetAsync(A.w0, 0, n3 * sizeof(double), h->stream));
    SMD_CUDA(cudaMemsetAsync(A.xbar, 0, n3 * sizeof(double), h->stream));
    SMD_CUDA(cudaMemsetAsync(A.hbar, 0, n3 * sizeof(double), h->stream));
    SMD_CUDA(cudaMemsetAsync(A.acc, 0, sizeof(AdjAcc), h->stream));
    double* w = A.w0;
    double* wn = A.w1;
    // ---- backward, segment by segment
    for (int c = ncp - 1; c >= 0; --c) {
      const int len = std::min(K, T - c * K);
      const double* x = cp + (size_t)c * 2 * n3;
      if (spec->segment_local && c != ncp - 1) {
        SMD_CUDA(cudaMemsetAsync(w, 0, n3 * sizeof(double), h->stream));
        SMD_CUDA(cudaMemsetAsync(A.xbar, 0, n3 * sizeof(double), h->stream));
        SMD_CUDA(cudaMemsetAsync(A.hbar, 0, n3 * sizeof(double), h->stream));
      }
      if (int r = adj_load(h, x, x + n3, true)) return r;
      h->it = cp_it[c];
      SMD_LAUNCH(h, k_set_counters<<<1, 1, 0, h->stream>>>(P.g, h->it, 1, 0, 0));
      for (int m = 0; m < len; ++m) {  // recompute x_n of the segment
        SMD_LAUNCH(h, k_state_save<<<h->grid(), kBlock, 0, h->stream>>>(P, seg + (size_t)m * n3, nullptr));
        if (m + 1 < len)
          if (int r = smd_advance(h, 1, SMD_ASYNC)) return r;
      }
      for (int m = len - 1; m >= 0; --m) {
        if (int r = adj_load(h, seg + (size_t)m * n3, nullptr, false)) return r;
        if (int r = adj_pair_pass(h, w, dt, invT)) return r;
        if (h->mixed)
          SMD_LAUNCH(h, k_adj_chain<true><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur, w, wn, A.xbar, A.hbar,
                                                                               A.kw, A.fpair, A.acc, dt, invT));
        else
          SMD_LAUNCH(h, k_adj_chain<false><<<h->grid(), kBlock, 0, h->stream>>>(P, h->cur, w, wn, A.xbar, A.hbar,
                                                                                A.kw, A.fpair, A.acc, dt, invT));
        std::swap(w, wn);
      }
    }
    // ---- the state after the T steps
    if (int r = adj_load(h, fin, fin + n3, true)) return r;
    h->it = it_end;
    SMD_LAUNCH(h, k_set_counters<<<1, 1, 0, h->stream>>>(P.g, h->it, 1, 0, 0));
    return 0;
  };
  rc = body();
  const cudaError_t se = cudaStreamSynchronize(h->stream);
  release();
  if (rc) return rc;
  if (se != cudaSuccess) return fail(100 + (int)se, std::string("adjoint: ") + cudaGetErrorString(se));
  AdjAcc acc;
  SMD_CUDA(cudaMemcpy(&acc, A.acc, sizeof acc, cudaMemcpyDeviceToHost));
  double box[3];
  if (int r = smd_get_box(h, 0, box)) return r;
  out->mean_potential = acc.J;
  for (int k = 0; k < 3; ++k) {
    out->grad[k] = acc.grad[k];
    out->grad_area[k] = 0.0;
  }
  out->mean_area_per_lipid = h->n_chains > 0 ? box[0] * box[1] / (0.5 * (double)h->n_chains) : 0.0;
  return read_error(h);
}

}  // extern "C"
