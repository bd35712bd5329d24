// C ABI of the step library (include/imexlb.h).
//
// Device state of one handle (one rank, one GPU):
//   fb[2]   two SoA population buffers, Q*N doubles each. After iteration n
//           the buffer `cur` holds the reference's post-BC fb of iteration n
//           on every slot a pull reads: fluid nodes (post-collision), obstacle
//           cells (b_user) and the ghost slots fluid nodes pull from; solid
//           slots keep their uploaded values in both buffers.
//   f,p,u   the reference's f, p, u (SoA); authoritative right after an
//           upload, rebuilt from fb[cur] by imexlb_download.
//   mask    one byte per padded cell (fluid / inlet / outlet).
//   fill    (dst, src) slot pairs that rebuild the boundary slots after each
//           collision; src may lie in the other buffer (an obstacle slot's
//           value from before this iteration's BC).
#include "imexlb.h"
#include "imexlb_host.h"
#include "imexlb_testing.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "batch.h"
#include "bcmap.h"
#include "fused_plan.h"
#include "kernels.h"
#include "lattice.h"

namespace {

thread_local std::string g_create_error;

enum State { kEmpty = 0, kFresh = 1, kPiped = 2 };

}  // namespace

namespace imx {
void set_thread_error(const char* msg) { g_create_error = msg; }
}  // namespace imx

struct imexlb_s {
  imexlb_desc d{};
  imx::GridLayout g;
  int dim = 2, Q = 9;
  int64_t N = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // geometry
  bool have_geom = false;
  int64_t size_fluid = 0;
  imx::BoundaryMap bmap;
  std::vector<uint8_t> mask;
  imx::DevGrid dg{};
  imx::DevCoef dc{};
  imx::DevCoefLP dcf{};  // minimal-operation update (reduced precision, fast FP64)
  imx::CoefFix dcx{};    // fixed-point update (IMEXLB_FIX64)
  // BF16 / FP16: the step kernel that stages tiles in shared memory with bulk
  // copies; its status word is mapped host memory (1: a bounded wait of the
  // kernel gave up)
  bool staged = true;
  int* stage_status = nullptr;
  int* d_stage_status = nullptr;
  cudaStream_t side = nullptr;  // the staged kernel's boundary groups run on it
  cudaEvent_t fork = nullptr, join = nullptr;
  // kStageGroup-cell groups from id_lo with a wall, periodic-face or record
  // node (the fused boundary handling's general pull; -1: not made)
  uint32_t* d_groups = nullptr;
  int64_t n_groups = -1;
  unsigned long long stage_wait_ns = 2000000000ull;  // 2 s per wait
  bool stage_stall = false;                         // failure injection (testing)
  bool exact = true;       // reference-order FP64 kernels
  int split = 0;           // step-kernel variant (identical results), set at create
  bool rho_one = true;
  int store = imx::kStoreF64;  // population storage kind
  size_t esz = 8;              // bytes per stored population

  // device memory
  uint8_t* d_mask = nullptr;
  void* d_fb[2] = {nullptr, nullptr};
  double* d_f = nullptr;
  double* d_p = nullptr;
  double* d_u = nullptr;
  double* d_stage = nullptr;
  double* d_inlet = nullptr;
  double* d_tq = nullptr;                // t by direction
  int64_t* d_offq = nullptr;             // pull offset by direction
  int64_t* d_offq_kind = nullptr;        // ... per fused boundary-node kind (27 tables)
  void* d_fill = nullptr;  // DevFill32 (fill_narrow) or DevFill entries
  int64_t n_fill = 0;
  bool fill_narrow = false;
  // the same copies folded into the step kernel (boundary_fused.cuh)
  uint32_t* d_bnd = nullptr;            // per flagged node: Q source slots + push word
  uint32_t* d_bnd_at = nullptr;         // node -> record
  imx::DevFill32* d_push = nullptr;     // obstacle copies, grouped by the node that runs them
  bool fused_ok = false;                // the plan exists for this geometry
  int64_t pshift = 0;                   // periodic y faces (3D): L1 * dy
  int64_t n_records = 0;                // nodes with a source row or obstacle copies
  int fill_mode = IMEXLB_FILL_FUSED;    // requested mode (default set at create)
  bool ghosts_stale = false;            // fused steps left the pulled ghost slots unwritten
  int* d_bl = nullptr;
  int* d_br = nullptr;
  int nl = 0, nr = 0;
  unsigned long long* d_mon = nullptr;
  int mon_cap = 0;
  bool watchdog = false;  // imexlb_set_watchdog: a non-finite Monitor value fails the step call
  int64_t device_bytes = 0;

  // momentum-exchange links and reduction scratch
  imx::DevLink* d_links = nullptr;
  int64_t n_links = 0;
  double* d_mass_partials = nullptr;
  double* d_obs = nullptr;        // 4 doubles: F[3], mass
  double* d_force_log = nullptr;
  int64_t force_cap = 0;

  // ghost slots rebuilt on download (built on first use)
  void* d_ghost = nullptr;
  int64_t n_ghost = -1;

  int cur = 0;
  int state = kEmpty;

  // rank of a multi-rank run (local_start / local_length not the whole
  // lattice): stepped by its imexlb_group, which resolves PassF across ranks
  bool member = false;
  imexlb_group_t* group = nullptr;
  std::vector<int> h_bl, h_br, h_bu, h_bd, h_user;  // the lists, for a group

  // runs of plain iterations from fb[0] back to fb[0], captured as graphs
  cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};  // kGraphLen[k] iterations from fb[0]

  // kernel accounting
  imexlb_profile prof{};
  bool timing = false;
  struct Pending { int kind; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
};

namespace {

int fail(imexlb_t* h, int code, const std::string& msg) {
  h->err = msg;
  return code;
}

int cuda_fail(imexlb_t* h, cudaError_t e, const char* what) {
  h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return IMEXLB_ERR_CUDA;
}

#define CK(h, call)                                  \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

template <class T>
int dalloc(imexlb_t* h, T** p, size_t count) {
  if (*p) return IMEXLB_OK;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    *p = nullptr;
    h->err = std::string("cudaMalloc of ") + std::to_string(sizeof(T) * count) +
             " bytes failed: " + cudaGetErrorString(e);
    return IMEXLB_ERR_NOMEM;
  }
  h->device_bytes += (int64_t)(sizeof(T) * count);
  return IMEXLB_OK;
}

template <class T>
void dfree(T** p) {
  if (*p) cudaFree(*p);
  *p = nullptr;
}

#define TRY(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != IMEXLB_OK) return r_; \
  } while (0)

cudaEvent_t take_event(imexlb_t* h) {
  if (!h->event_pool.empty()) {
    cudaEvent_t e = h->event_pool.back();
    h->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Launch through `fn` on the handle's stream, counting it under `kind` and,
// with timing on, bracketing it with events.
template <class F>
int run_kernel(imexlb_t* h, int kind, F&& fn) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (h->timing) {
    a = take_event(h);
    b = take_event(h);
    if (!a || !b) return fail(h, IMEXLB_ERR_CUDA, "cudaEventCreate failed");
    CK(h, cudaEventRecord(a, h->stream));
  }
  cudaError_t e = fn();
  if (e != cudaSuccess) return cuda_fail(h, e, "kernel launch");
  if (h->timing) {
    CK(h, cudaEventRecord(b, h->stream));
    h->pending.push_back({kind, a, b});
  }
  h->prof.launches[kind]++;
  return IMEXLB_OK;
}

// After a stream synchronize: fold the recorded launch times into the profile.
int collect_times(imexlb_t* h) {
  for (auto& pd : h->pending) {
    float ms = 0.f;
    CK(h, cudaEventElapsedTime(&ms, pd.a, pd.b));
    h->prof.ms[pd.kind] += ms;
    h->event_pool.push_back(pd.a);
    h->event_pool.push_back(pd.b);
  }
  h->pending.clear();
  return IMEXLB_OK;
}

// Boundary copies inside the step kernel for this handle's next steps (for
// the FP64 path: compiled for the default kernel variant).
bool fused_fill(const imexlb_t* h) {
  return h->fused_ok && h->fill_mode == IMEXLB_FILL_FUSED &&
         (!h->exact || !h->rho_one || h->split == imx::step_split_default(h->dim));
}

// Device state of the step kernels.
imx::DevState step_state(const imexlb_t* h) {
  imx::DevState st{h->d_mask, h->d_inlet, h->d_tq, h->d_offq};
  if (fused_fill(h)) {
    st.bnd = h->d_bnd;
    st.bnd_at = h->d_bnd_at;
    st.push = h->d_push;
    st.pshift = h->pshift;
    st.offq_kind = h->d_offq_kind;
  }
  return st;
}

// The step kernel of the handle's kind, fin -> fout.
cudaError_t launch_step_kind(imexlb_t* h, const imx::DevState& st, void* fin, void* fout,
                             unsigned long long* mon) {
  if (h->exact)
    return imx::launch_step(h->dim, h->rho_one, h->dg, h->dc, st, (const double*)fin,
                            (double*)fout, mon, h->stream, h->split);
  const imx::DevPlanes pl = imx::make_planes(h->dg, h->Q, h->esz, fin, fout);
  if (h->store == imx::kStoreFix) return imx::launch_step_fx(h->dim, h->dg, h->dcx, st, pl, mon, h->stream);
  const imx::StagedArgs sa{h->d_stage_status, h->d_groups, h->n_groups, h->stage_wait_ns,
                           h->stage_stall ? 1 : 0, h->side, h->fork, h->join};
  return imx::launch_step_lp(h->dim, h->store, h->dg, h->dcf, st, pl, mon, h->stream,
                             h->staged ? &sa : nullptr);
}

// Enqueue one plain iteration (no Monitor) from fb[src] into fb[1-src].
cudaError_t enqueue_plain_iteration(imexlb_t* h, int src) {
  const imx::DevState st = step_state(h);
  void* fin = h->d_fb[src];
  void* fout = h->d_fb[1 - src];
  cudaError_t e = launch_step_kind(h, st, fin, fout, nullptr);
  if (e != cudaSuccess || fused_fill(h)) return e;
  return imx::launch_fill(h->store, h->d_fill, h->fill_narrow, h->n_fill, fout, fin, h->stream);
}

// Write the boundary slots the last fused steps left out (the pulled ghost
// slots) into the current buffer, for kernels that pull from it outside a
// step (download, mass, sample): the separate fill list once.
int sync_ghosts(imexlb_t* h) {
  if (!h->ghosts_stale) return IMEXLB_OK;
  TRY(run_kernel(h, IMEXLB_KERNEL_FILL, [&] {
    return imx::launch_fill(h->store, h->d_fill, h->fill_narrow, h->n_fill, h->d_fb[h->cur],
                            h->d_fb[1 - h->cur], h->stream);
  }));
  h->ghosts_stale = false;
  return IMEXLB_OK;
}

// Lengths of the captured runs of plain iterations (even: they start and end
// in fb[0]); short iterations are launch-bound, so longer runs replay more of
// them per graph launch.
constexpr int kGraphLen[2] = {2, 8};

// Drop the captured graphs (the kernel variant, fill mode or geometry changed).
int drop_graphs(imexlb_t* h) {
  for (cudaGraphExec_t& g : h->graph_exec) {
    if (!g) continue;
    CK(h, cudaStreamSynchronize(h->stream));
    cudaGraphExecDestroy(g);
    g = nullptr;
  }
  return IMEXLB_OK;
}

// Capture (once per geometry) the graph of kGraphLen[k] plain iterations
// starting in fb[0].
int ensure_graph(imexlb_t* h, int k) {
  if (h->graph_exec[k]) return IMEXLB_OK;
  cudaGraph_t graph = nullptr;
  CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < kGraphLen[k] && e == cudaSuccess; ++i) e = enqueue_plain_iteration(h, i & 1);
  const cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return cuda_fail(h, e != cudaSuccess ? e : e2, "graph capture");
  }
  e = cudaGraphInstantiate(&h->graph_exec[k], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    h->graph_exec[k] = nullptr;
    return cuda_fail(h, e, "cudaGraphInstantiate");
  }
  return IMEXLB_OK;
}

bool lattice_matches(const imexlb_desc* d) {
  for (int iq = 0; iq < d->nq; ++iq)
    for (int k = 0; k < d->dim; ++k) {
      int ref = d->dim == 2 ? imx::Lattice<2>::e(iq, k) : imx::Lattice<3>::e(iq, k);
      if (d->e[iq * d->dim + k] != ref) return false;
    }
  return true;
}

// Inlet velocity of PostProcessing by padded row (2D) / plane (3D):
// uu*rho0*4*y*(ny-y)/ny**2 with integer y (lbm.f90:188-189, lbm_3d.f90:190-191).
std::vector<double> inlet_profile(const imexlb_desc& d) {
  const int n = d.dim == 2 ? d.ny : d.nz;
  const int rows = (d.dim == 2 ? d.local_length[1] : d.local_length[2]) + 2 * imx::kGhost;
  const int start = d.dim == 2 ? d.local_start[1] : d.local_start[2];
  std::vector<double> v((size_t)rows);
  for (int r = 0; r < rows; ++r) {
    const int y = r - imx::kGhost + start;
    v[(size_t)r] = d.uu * d.rho0 * 4.0 * y * (double)(n - y) / (double)(n * n);
  }
  return v;
}

int ensure_stage(imexlb_t* h) { return dalloc(h, &h->d_stage, (size_t)(h->N * h->Q)); }

// host AoS [N*K] (double) -> device SoA [K*N] of storage kind `store`
int upload_field(imexlb_t* h, const double* host, void* dev, int K, int store = imx::kStoreF64) {
  if (K == 1 && store == imx::kStoreF64) {
    CK(h, cudaMemcpyAsync(dev, host, sizeof(double) * h->N, cudaMemcpyHostToDevice, h->stream));
    return IMEXLB_OK;
  }
  TRY(ensure_stage(h));
  CK(h, cudaMemcpyAsync(h->d_stage, host, sizeof(double) * h->N * K, cudaMemcpyHostToDevice,
                        h->stream));
  TRY(run_kernel(h, IMEXLB_KERNEL_OTHER,
                 [&] { return imx::launch_aos_to_soa(store, h->d_stage, dev, h->N, K, h->stream); }));
  return IMEXLB_OK;
}

// device SoA of storage kind `store` -> host AoS (double)
int download_field(imexlb_t* h, const void* dev, double* host, int K, int store = imx::kStoreF64) {
  if (K == 1 && store == imx::kStoreF64) {
    CK(h, cudaMemcpyAsync(host, dev, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
    return IMEXLB_OK;
  }
  TRY(ensure_stage(h));
  TRY(run_kernel(h, IMEXLB_KERNEL_OTHER,
                 [&] { return imx::launch_soa_to_aos(store, dev, h->d_stage, h->N, K, h->stream); }));
  CK(h, cudaMemcpyAsync(host, h->d_stage, sizeof(double) * h->N * K, cudaMemcpyDeviceToHost,
                        h->stream));
  return IMEXLB_OK;
}

// Copy a fill list to the device, sorted by destination slot (coalesced
// writes) and with 32-bit indices when Q*N < 2^31.
int upload_fill(imexlb_t* h, std::vector<imx::DevFill>& v, void** dptr) {
  std::sort(v.begin(), v.end(),
            [](const imx::DevFill& a, const imx::DevFill& b) { return a.dst < b.dst; });
  if (h->fill_narrow) {
    std::vector<imx::DevFill32> w(v.size());
    for (size_t i = 0; i < v.size(); ++i)
      w[i] = imx::DevFill32{(uint32_t)v[i].dst,
                            v[i].src == imx::kFillNaN ? imx::kFillNaN32 : (int32_t)v[i].src};
    TRY(dalloc(h, (imx::DevFill32**)dptr, w.size()));
    if (!w.empty())
      CK(h, cudaMemcpy(*dptr, w.data(), sizeof(imx::DevFill32) * w.size(), cudaMemcpyHostToDevice));
  } else {
    TRY(dalloc(h, (imx::DevFill**)dptr, v.size()));
    if (!v.empty())
      CK(h, cudaMemcpy(*dptr, v.data(), sizeof(imx::DevFill) * v.size(), cudaMemcpyHostToDevice));
  }
  return IMEXLB_OK;
}

// The boundary copies of `fill` folded into the step kernel (fused_plan.h,
// boundary_fused.cuh): plan, upload, and the plan's bits in h->mask. Leaves
// fused_ok false (the separate fill kernel) for a geometry the plan does not
// cover, or when the slots need 64-bit indices.
// The kStageGroup-cell groups from id_lo that hold a fluid node whose fused
// pull is more than the inlet / outlet form (PullFix::other of
// boundary_fused.cuh): the staged step kernel leaves them to a second kernel.
int build_boundary_groups(imexlb_t* h) {
  using namespace imx;
  std::vector<uint32_t> w;
  const int64_t lo = h->dg.id_lo, hi = h->dg.id_hi;
  const uint32_t xf = kMaskInlet | kMaskOutlet;
  constexpr int64_t W = kStageGroup;
  for (int64_t c0 = lo; c0 < hi; c0 += W) {
    bool any = false;
    for (int64_t id = c0; id < c0 + W && id < hi && !any; ++id) {
      const uint8_t m = h->mask[(size_t)id];
      if (!(m & kMaskFluid)) continue;
      uint32_t b = (uint32_t)(m & ~kMaskFluid);
      if (b & kMaskRecord) b = kMaskRecord;
      any = (b & ~xf) != 0u || (b & xf) == xf;
    }
    if (any) w.push_back((uint32_t)((c0 - lo) / W));
  }
  dfree(&h->d_groups);
  TRY(dalloc(h, &h->d_groups, std::max<size_t>(w.size(), 1)));
  if (!w.empty())
    CK(h, cudaMemcpy(h->d_groups, w.data(), sizeof(uint32_t) * w.size(), cudaMemcpyHostToDevice));
  h->n_groups = (int64_t)w.size();
  return IMEXLB_OK;
}

int build_fused(imexlb_t* h, const std::vector<imx::DevFill>& fill) {
  h->fused_ok = false;
  h->n_groups = -1;
  h->n_records = 0;
  dfree(&h->d_bnd);
  dfree(&h->d_bnd_at);
  dfree(&h->d_push);
  imx::FusedPlan plan;
  if (!h->fill_narrow || h->member || fill.empty() ||
      !imx::plan_fused(h->g, h->dg, h->mask, h->bmap, fill, plan))
    return IMEXLB_OK;
  std::vector<uint32_t> at((size_t)h->N, 0u);
  for (size_t k = 0; k < plan.nodes.size(); ++k) at[(size_t)plan.nodes[k]] = (uint32_t)k;
  TRY(dalloc(h, &h->d_bnd_at, (size_t)h->N));
  TRY(dalloc(h, &h->d_bnd, std::max<size_t>(plan.rec.size(), 1)));
  TRY(dalloc(h, &h->d_push, std::max<size_t>(plan.ent.size(), 1)));
  CK(h, cudaMemcpy(h->d_bnd_at, at.data(), sizeof(uint32_t) * at.size(), cudaMemcpyHostToDevice));
  if (!plan.rec.empty())
    CK(h, cudaMemcpy(h->d_bnd, plan.rec.data(), sizeof(uint32_t) * plan.rec.size(), cudaMemcpyHostToDevice));
  if (!plan.ent.empty())
    CK(h, cudaMemcpy(h->d_push, plan.ent.data(), sizeof(imx::DevFill32) * plan.ent.size(),
                     cudaMemcpyHostToDevice));
  imx::apply_plan_bits(plan, h->mask);
  h->pshift = plan.pshift;
  h->n_records = (int64_t)plan.nodes.size();
  h->fused_ok = true;
  return build_boundary_groups(h);
}

// Device list that rebuilds every ghost slot of the current buffer as the
// reference's BoundaryCondition leaves it (download only).
int build_ghost_fill(imexlb_t* h) {
  if (h->n_ghost >= 0) return IMEXLB_OK;
  const imx::GridLayout& g = h->g;
  const int Q = h->Q;
  const int64_t N = h->N;
  const int PZ = h->dim == 3 ? g.L[2] + 2 * imx::kGhost : 1;
  const int PY = g.L[1] + 2 * imx::kGhost, PX = g.L[0] + 2 * imx::kGhost;
  std::vector<imx::DevFill> v;
  for (int Z = 0; Z < PZ; ++Z)
    for (int Y = 0; Y < PY; ++Y)
      for (int X = 0; X < PX; ++X) {
        const int64_t c = X + g.dy * Y + g.dz * Z;
        if (!g.is_ghost(c)) {
          X = g.L[0] + imx::kGhost - 1;  // skip the interior part of this row
          continue;
        }
        for (int iq = 0; iq < Q; ++iq) {
          const int64_t r = h->bmap.resolve(c * Q + iq);
          const int64_t dst = (int64_t)iq * N + c;
          const imx::SrcKind k = h->bmap.kind_of(r);
          int64_t src;
          if (k == imx::kSrcPoison) src = imx::kFillNaN;
          else {
            const int64_t soa = (r % Q) * N + r / Q;
            src = k == imx::kSrcUser ? ~soa : soa;
          }
          v.push_back(imx::DevFill{dst, src});
        }
      }
  TRY(upload_fill(h, v, &h->d_ghost));
  h->n_ghost = (int64_t)v.size();
  return IMEXLB_OK;
}

// ---------------------------------------------------------------------------
// Multi-rank runs (cart_mpi.f90) on one device: every rank is a handle with
// its own local box; the group resolves each rank's boundary program over
// (rank, slot) names (PassF reads the owner rank's interior cells) and
// refreshes all ranks' boundary slots with one launch per iteration.

}  // namespace

struct imexlb_group_s {
  std::vector<imexlb_t*> ranks;
  int dim = 2, nprocs = 0, device = 0;
  int np[3] = {1, 1, 1}, gl[3] = {1, 1, 1};
  cudaStream_t stream = nullptr;
  imx::GroupBoundary gb;
  imx::DevGroupFill* d_fill = nullptr;
  int64_t n_fill = 0;
  imx::DevGroupFill* d_ghost = nullptr;  // every ghost slot (downloads)
  int64_t n_ghost = -1;
  double** d_bufs = nullptr;             // fb[0], fb[1] of every rank
  unsigned long long* d_mon = nullptr;
  int mon_cap = 0;
  bool ghost_dirty = false;
  std::string err;
};

namespace {

int gfail(imexlb_group_t* g, int code, const std::string& m) {
  g->err = m;
  return code;
}

#define GCK(g, call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return gfail(g, IMEXLB_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// The resolved refresh lists of every rank in device form (SoA indices).
int group_upload(imexlb_group_t* g, bool complete, imx::DevGroupFill** dptr, int64_t* n) {
  std::vector<imx::DevGroupFill> v;
  std::vector<imx::GroupFillEntry> e;
  std::string err;
  for (int a = 0; a < g->nprocs; ++a) {
    if (!g->gb.fill(a, complete, e, err)) return gfail(g, IMEXLB_ERR_GEOMETRY, err);
    const imexlb_t* ha = g->ranks[(size_t)a];
    const int Q = ha->Q;
    for (const imx::GroupFillEntry& x : e) {
      imx::DevGroupFill d{};
      d.dst = (x.dst % Q) * ha->N + x.dst / Q;
      d.dst_rank = a;
      if (x.kind == imx::kSrcPoison) {
        d.src = 0;
        d.src_code = -1;
      } else {
        const imexlb_t* hb = g->ranks[(size_t)x.src_rank];
        d.src = (x.src % Q) * hb->N + x.src / Q;
        d.src_code = x.src_rank | (x.kind == imx::kSrcUser ? imx::kGroupPrev : 0);
      }
      v.push_back(d);
    }
  }
  if (*dptr) {
    cudaFree(*dptr);
    *dptr = nullptr;
  }
  GCK(g, cudaMalloc((void**)dptr, sizeof(imx::DevGroupFill) * (v.empty() ? 1 : v.size())));
  if (!v.empty())
    GCK(g, cudaMemcpy(*dptr, v.data(), sizeof(imx::DevGroupFill) * v.size(), cudaMemcpyHostToDevice));
  *n = (int64_t)v.size();
  return IMEXLB_OK;
}

// Download of a rank: every ghost slot of every rank as PassF and the copies
// leave them (the pipeline only keeps the slots a fluid node pulls).
int group_sync_ghosts(imexlb_t* h) {
  imexlb_group_t* g = h->group;
  if (!g) return fail(h, IMEXLB_ERR_STATE, "a rank of a multi-rank run is downloaded within its group");
  if (!g->ghost_dirty) return IMEXLB_OK;
  if (g->n_ghost < 0 && group_upload(g, true, &g->d_ghost, &g->n_ghost) != IMEXLB_OK)
    return fail(h, IMEXLB_ERR_GEOMETRY, g->err);
  TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
    return imx::launch_fill_group(g->d_ghost, g->n_ghost, g->d_bufs, h->cur, h->stream);
  }));
  g->ghost_dirty = false;
  return IMEXLB_OK;
}

}  // namespace

extern "C" {

const char* imexlb_version(void) {
  static const char* v = "1.0 (sm_103a, FP64 reference-order kernels)";
  return v;
}

const char* imexlb_last_error(const imexlb_t* h) {
  return h ? h->err.c_str() : g_create_error.c_str();
}

int imexlb_create(imexlb_t** out, const imexlb_desc* d) {
  g_create_error.clear();
  if (!out || !d) {
    g_create_error = "imexlb_create: null argument";
    return IMEXLB_ERR_ARG;
  }
  *out = nullptr;
  auto bad = [&](const std::string& m, int code = IMEXLB_ERR_ARG) {
    g_create_error = m;
    return code;
  };
  if (d->dim != 2 && d->dim != 3) return bad("dim must be 2 or 3");
  if (d->nq != (d->dim == 2 ? 9 : 27)) return bad("nq must be 9 (dim=2) or 27 (dim=3)");
  if (d->ghost != imx::kGhost) return bad("ghost must be 3");
  if (d->precision != IMEXLB_FP64 && d->precision != IMEXLB_FP64_FAST &&
      d->precision != IMEXLB_FP32 && d->precision != IMEXLB_BF16 && d->precision != IMEXLB_FP16 &&
      d->precision != IMEXLB_FIX64)
    return bad("unsupported precision", IMEXLB_ERR_UNSUPPORTED);
  if (d->precision == IMEXLB_FIX64 && (d->rho0 != 1.0 || !(d->ome > 0.0 && d->ome < 2.0)))
    return bad("IMEXLB_FIX64 needs rho0 = 1 and 0 < ome < 2", IMEXLB_ERR_UNSUPPORTED);
  const int n[3] = {d->nx, d->ny, d->dim == 3 ? d->nz : 0};
  bool member = false;
  for (int k = 0; k < d->dim; ++k) {
    if (d->local_start[k] < 0 || d->local_start[k] + d->local_length[k] > n[k] + 1)
      return bad("local box outside the global lattice (local_start + local_length > n+1)");
    if (d->local_length[k] < imx::kGhost) return bad("local_length < ghost");
    member = member || d->local_start[k] != 0 || d->local_length[k] != n[k] + 1;
  }
  if (member && d->precision != IMEXLB_FP64)
    return bad("a rank of a multi-rank run (imexlb_group) needs IMEXLB_FP64",
               IMEXLB_ERR_UNSUPPORTED);
  const int64_t dy = d->local_length[0] + 2 * imx::kGhost;
  if (d->dy != dy) return bad("dy must be local_length(1)+2*ghost");
  if (d->dim == 3 && d->dz != dy * (d->local_length[1] + 2 * imx::kGhost))
    return bad("dz must be dy*(local_length(2)+2*ghost)");
  if (!lattice_matches(d)) return bad("lattice velocities are not in InitLattice order");
  if (!std::isfinite(d->ome) || !std::isfinite(d->rho0) || !std::isfinite(d->uu) || d->rho0 == 0.0)
    return bad("ome, rho0, uu must be finite and rho0 non-zero");
  if (d->dim == 2 ? d->ny == 0 : d->nz == 0) return bad("ny (2D) / nz (3D) must be non-zero");

  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return bad(std::string("no CUDA device: ") + cudaGetErrorString(e), IMEXLB_ERR_CUDA);
  if (d->device < 0 || d->device >= ndev) return bad("device ordinal out of range");
  e = cudaSetDevice(d->device);
  if (e != cudaSuccess) return bad(std::string("cudaSetDevice: ") + cudaGetErrorString(e), IMEXLB_ERR_CUDA);

  imexlb_t* h = new (std::nothrow) imexlb_s();
  if (!h) return bad("out of host memory", IMEXLB_ERR_NOMEM);
  h->d = *d;
  h->dim = d->dim;
  h->Q = d->nq;
  h->device = d->device;
  h->member = member;
  imx::GridLayout& g = h->g;
  g.dim = d->dim;
  g.Q = d->nq;
  for (int k = 0; k < 3; ++k) g.L[k] = k < d->dim ? d->local_length[k] : 1;
  g.dy = dy;
  g.dz = d->dim == 3 ? d->dz : 0;
  g.N = dy * (d->local_length[1] + 2 * imx::kGhost);
  if (d->dim == 3) g.N *= (d->local_length[2] + 2 * imx::kGhost);
  std::memcpy(g.e, d->e, sizeof(int) * d->nq * d->dim);
  h->N = g.N;

  e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return bad(std::string("cudaStreamCreate: ") + cudaGetErrorString(e), IMEXLB_ERR_CUDA);
  }
  if (cudaHostAlloc((void**)&h->stage_status, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&h->d_stage_status, h->stage_status, 0) != cudaSuccess) {
    e = cudaGetLastError();
    if (h->stage_status) cudaFreeHost(h->stage_status);
    cudaStreamDestroy(h->stream);
    delete h;
    return bad(std::string("mapped status word: ") + cudaGetErrorString(e), IMEXLB_ERR_CUDA);
  }
  *h->stage_status = 0;
  if (cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->join, cudaEventDisableTiming) != cudaSuccess) {
    e = cudaGetLastError();
    if (h->join) cudaEventDestroy(h->join);
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->side) cudaStreamDestroy(h->side);
    cudaFreeHost(h->stage_status);
    cudaStreamDestroy(h->stream);
    delete h;
    return bad(std::string("second stream: ") + cudaGetErrorString(e), IMEXLB_ERR_CUDA);
  }
  imx::prepare_step_lp();

  imx::DevGrid& dg = h->dg;
  dg.N = g.N;
  dg.dy = g.dy;
  dg.dz = g.dz;
  const int64_t G = imx::kGhost;
  dg.id_lo = G + g.dy * G + g.dz * G;
  dg.id_hi = (g.L[0] + G - 1) + g.dy * (g.L[1] + G - 1) + (d->dim == 3 ? g.dz * (g.L[2] + G - 1) : 0) + 1;
  for (int iq = 0; iq < d->nq; ++iq) dg.off[iq] = g.off(iq, 1);
  dg.skip_id = -1;
  imx::DevCoef& dc = h->dc;
  for (int iq = 0; iq < d->nq; ++iq) dc.t[iq] = d->t[iq];
  dc.ome = d->ome;
  dc.om1 = 1.0 - d->ome;  // (1-ome), lbm.f90:71
  dc.rho0 = d->rho0;
  dc.one = 1.0;
  dc.mone = -1.0;
  dc.mzero = -0.0;
  h->rho_one = d->rho0 == 1.0;
  h->store = d->precision == IMEXLB_FP32   ? imx::kStoreF32
             : d->precision == IMEXLB_BF16 ? imx::kStoreBF16
             : d->precision == IMEXLB_FP16 ? imx::kStoreF16
             : d->precision == IMEXLB_FIX64 ? imx::kStoreFix
                                           : imx::kStoreF64;
  h->esz = imx::store_bytes(h->store);
  h->exact = d->precision == IMEXLB_FP64;
  h->split = imx::step_split_default(d->dim);
  // boundary copies inside the step kernel: one launch per iteration
  h->fill_mode = IMEXLB_FILL_FUSED;
  imx::DevCoefLP& cf = h->dcf;
  for (int iq = 0; iq < d->nq; ++iq) {
    cf.d.k[iq] = d->ome * d->t[iq] * d->rho0;
    cf.f.k[iq] = (float)cf.d.k[iq];
  }
  cf.d.om1 = 1.0 - d->ome;
  cf.d.inv_rho0 = 1.0 / d->rho0;
  cf.f.om1 = (float)cf.d.om1;
  cf.f.inv_rho0 = (float)cf.d.inv_rho0;
  // Q0.63 constants of the fixed-point kind: the doubles ome*t_i and 1-ome
  // scaled by 2^63 (exact; |value| < 1)
  for (int iq = 0; iq < d->nq; ++iq) h->dcx.k[iq] = std::llround(std::ldexp(cf.d.k[iq], 63));
  h->dcx.om1 = std::llround(std::ldexp(cf.d.om1, 63));
  *out = h;
  return IMEXLB_OK;
}

int imexlb_set_geometry(imexlb_t* h, const int* geo, const int* fluid_id, int size_fluid,
                        const int* bl, int l_size, const int* br, int r_size, const int* bu,
                        int u_size, const int* bd, int d_size, const int* b_user, int user_size) {
  if (!h) return IMEXLB_ERR_ARG;
  if (!geo || (size_fluid > 0 && !fluid_id) || size_fluid < 0)
    return fail(h, IMEXLB_ERR_ARG, "geo / fluid_id missing");
  CK(h, cudaSetDevice(h->device));
  const imx::GridLayout& g = h->g;
  h->mask.assign((size_t)h->N, 0);
  for (int i = 0; i < size_fluid; ++i) {
    const int64_t id = fluid_id[i];
    if (id < 0 || id >= h->N || g.is_ghost(id))
      return fail(h, IMEXLB_ERR_GEOMETRY, "fluid_id[" + std::to_string(i) + "] is not an interior node");
    if (geo[id] != 1)
      return fail(h, IMEXLB_ERR_GEOMETRY, "fluid_id[" + std::to_string(i) + "] has geo != 1");
    if (h->mask[(size_t)id]) return fail(h, IMEXLB_ERR_GEOMETRY, "fluid_id lists a node twice");
    h->mask[(size_t)id] = imx::kMaskFluid;
  }
  for (int i = 0; i < l_size; ++i) {
    const int64_t id = (int64_t)bl[i] + 1;
    if (id >= 0 && id < h->N && (h->mask[(size_t)id] & imx::kMaskFluid)) h->mask[(size_t)id] |= imx::kMaskInlet;
  }
  for (int i = 0; i < r_size; ++i) {
    const int64_t id = (int64_t)br[i] - 1;
    if (id >= 0 && id < h->N && (h->mask[(size_t)id] & imx::kMaskFluid)) h->mask[(size_t)id] |= imx::kMaskOutlet;
  }
  for (int i = 0; i < l_size; ++i)
    if ((int64_t)bl[i] + 1 < 0 || (int64_t)bl[i] + 1 >= h->N)
      return fail(h, IMEXLB_ERR_GEOMETRY, "bl entry + 1 is outside the array");
  for (int i = 0; i < r_size; ++i)
    if ((int64_t)br[i] - 1 < 0 || (int64_t)br[i] - 1 >= h->N)
      return fail(h, IMEXLB_ERR_GEOMETRY, "br entry - 1 is outside the array");

  imx::BoundaryLists lists;
  lists.fluid_mask = h->mask.data();
  lists.bl = bl; lists.nl = l_size;
  lists.br = br; lists.nr = r_size;
  lists.bu = bu; lists.nu = u_size;
  lists.bd = bd; lists.nd = d_size;
  lists.user = b_user; lists.nuser = user_size;
  std::string err;
  if (h->group) return fail(h, IMEXLB_ERR_STATE, "the handle is a rank of a group");
  auto keep = [](std::vector<int>& v, const int* p, int n) {
    if (n > 0) v.assign(p, p + n);
    else v.clear();
  };
  keep(h->h_bl, bl, l_size);
  keep(h->h_br, br, r_size);
  keep(h->h_bu, bu, u_size);
  keep(h->h_bd, bd, d_size);
  keep(h->h_user, b_user, user_size);
  // a rank of a multi-rank run: PassF crosses ranks, its group resolves the
  // boundary program
  if (!h->member && !h->bmap.build(g, lists, err)) return fail(h, IMEXLB_ERR_GEOMETRY, err);
  // bmap keeps a pointer to the mask; the mask must be binary fluid there.
  // kind_of only tests non-zero, which inlet/outlet bits preserve.

  const int Q = h->Q;
  const int64_t N = h->N;
  std::vector<imx::DevFill> fill;
  const std::vector<imx::FillEntry> no_fill;
  const std::vector<imx::FillEntry>& fes = h->member ? no_fill : h->bmap.fill();
  fill.reserve(fes.size());
  for (const imx::FillEntry& fe : fes) {
    const int64_t dcell = fe.dst / Q, dq = fe.dst % Q;
    const int64_t scell = fe.src / Q, sq = fe.src % Q;
    const int64_t dsoa = dq * N + dcell, ssoa = sq * N + scell;
    fill.push_back(imx::DevFill{dsoa, fe.src_prev ? ~ssoa : ssoa});
  }

  // Momentum-exchange links: fluid node x -> interior solid node x + e_iq.
  std::vector<imx::DevLink> links;
  for (int i = 0; i < size_fluid; ++i) {
    const int64_t x = fluid_id[i];
    for (int iq = 0; iq < Q; ++iq) {
      const int64_t sn = x + g.off(iq, 1);
      if (g.is_ghost(sn) || h->mask[(size_t)sn]) continue;
      links.push_back(imx::DevLink{(int64_t)iq * N + x, (int64_t)(Q - 1 - iq) * N + sn, iq, 0});
    }
  }

  // (Re)allocate device state.
  dfree(&h->d_links);
  dfree((uint8_t**)&h->d_fill);
  dfree(&h->d_bl);
  dfree(&h->d_br);
  dfree(&h->d_inlet);
  dfree((uint8_t**)&h->d_ghost);
  h->n_ghost = -1;
  TRY(drop_graphs(h));
  TRY(dalloc(h, &h->d_mask, (size_t)N));
  TRY(dalloc(h, (uint8_t**)&h->d_fb[0], (size_t)(N * Q) * h->esz));
  TRY(dalloc(h, (uint8_t**)&h->d_fb[1], (size_t)(N * Q) * h->esz));
  TRY(dalloc(h, &h->d_f, (size_t)(N * Q)));
  TRY(dalloc(h, &h->d_p, (size_t)N));
  TRY(dalloc(h, &h->d_u, (size_t)(N * h->dim)));
  h->fill_narrow = N * Q < (int64_t)INT32_MAX;
  TRY(upload_fill(h, fill, &h->d_fill));
  TRY(build_fused(h, fill));
  TRY(dalloc(h, &h->d_links, links.size()));
  TRY(dalloc(h, &h->d_mass_partials, (size_t)imx::mass_partials_size(h->dg)));
  TRY(dalloc(h, &h->d_obs, 4));
  TRY(dalloc(h, &h->d_tq, (size_t)Q));
  TRY(dalloc(h, &h->d_offq, (size_t)Q));
  CK(h, cudaMemcpyAsync(h->d_tq, h->dc.t, sizeof(double) * Q, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->d_offq, h->dg.off, sizeof(int64_t) * Q, cudaMemcpyHostToDevice, h->stream));
  {
    // pull offsets of the fused boundary-node kinds (boundary_fused.cuh)
    std::vector<int64_t> kinds;
    imx::fused_kind_offsets(h->g, h->dg, h->dim == 3 ? (int64_t)h->g.L[1] * h->g.dy : 0, kinds);
    TRY(dalloc(h, &h->d_offq_kind, kinds.size()));
    CK(h, cudaMemcpy(h->d_offq_kind, kinds.data(), sizeof(int64_t) * kinds.size(), cudaMemcpyHostToDevice));
  }
  TRY(dalloc(h, &h->d_bl, (size_t)l_size));
  TRY(dalloc(h, &h->d_br, (size_t)r_size));
  std::vector<double> inlet = inlet_profile(h->d);
  TRY(dalloc(h, &h->d_inlet, inlet.size()));
  CK(h, cudaMemcpyAsync(h->d_mask, h->mask.data(), (size_t)N, cudaMemcpyHostToDevice, h->stream));
  if (!links.empty())
    CK(h, cudaMemcpyAsync(h->d_links, links.data(), sizeof(imx::DevLink) * links.size(),
                          cudaMemcpyHostToDevice, h->stream));
  if (l_size) CK(h, cudaMemcpyAsync(h->d_bl, bl, sizeof(int) * l_size, cudaMemcpyHostToDevice, h->stream));
  if (r_size) CK(h, cudaMemcpyAsync(h->d_br, br, sizeof(int) * r_size, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->d_inlet, inlet.data(), sizeof(double) * inlet.size(),
                        cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->n_fill = (int64_t)fill.size();
  h->n_links = (int64_t)links.size();
  h->nl = l_size;
  h->nr = r_size;
  h->size_fluid = size_fluid;
  h->dg.skip_id = size_fluid > 0 ? fluid_id[0] : -1;
  h->have_geom = true;
  h->state = kEmpty;
  return IMEXLB_OK;
}

int imexlb_upload(imexlb_t* h, const double* f, const double* fb, const double* p, const double* u) {
  if (!h) return IMEXLB_ERR_ARG;
  if (!h->have_geom) return fail(h, IMEXLB_ERR_STATE, "imexlb_set_geometry must come first");
  if (!f || !fb || !p || !u) return fail(h, IMEXLB_ERR_ARG, "f, fb, p, u are all required");
  CK(h, cudaSetDevice(h->device));
  TRY(upload_field(h, f, h->d_f, h->Q));
  TRY(upload_field(h, fb, h->d_fb[0], h->Q, h->store));
  CK(h, cudaMemcpyAsync(h->d_fb[1], h->d_fb[0], h->esz * h->N * h->Q, cudaMemcpyDeviceToDevice,
                        h->stream));
  TRY(upload_field(h, p, h->d_p, 1));
  TRY(upload_field(h, u, h->d_u, h->dim));
  CK(h, cudaStreamSynchronize(h->stream));
  h->state = kFresh;
  h->cur = 0;
  return IMEXLB_OK;
}

int imexlb_init_state(imexlb_t* h, const double* r_vec) {
  if (!h) return IMEXLB_ERR_ARG;
  if (!h->have_geom) return fail(h, IMEXLB_ERR_STATE, "imexlb_set_geometry must come first");
  CK(h, cudaSetDevice(h->device));
  // fresh allocation: f and fb zero (the reference's fb stays zero on solid cells)
  CK(h, cudaMemsetAsync(h->d_f, 0, sizeof(double) * h->N * h->Q, h->stream));
  CK(h, cudaMemsetAsync(h->d_fb[0], 0, h->esz * h->N * h->Q, h->stream));
  CK(h, cudaMemsetAsync(h->d_fb[1], 0, h->esz * h->N * h->Q, h->stream));
  CK(h, cudaMemsetAsync(h->d_p, 0, sizeof(double) * h->N, h->stream));
  CK(h, cudaMemsetAsync(h->d_u, 0, sizeof(double) * h->N * h->dim, h->stream));
  if (r_vec) {
    imx::RVec rv;
    std::memcpy(rv.v, r_vec, sizeof rv.v);
    const int n = h->dim == 2 ? h->d.ny : h->d.nz;
    const int start = h->dim == 2 ? h->d.local_start[1] : h->d.local_start[2];
    TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
      return imx::launch_init_up(h->dim, h->dg, h->d_mask, rv, h->d.uu, n, start, h->d_u, h->stream);
    }));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  TRY(collect_times(h));
  h->state = kFresh;
  h->cur = 0;
  return IMEXLB_OK;
}

int imexlb_init_pdf(imexlb_t* h) {
  if (!h) return IMEXLB_ERR_ARG;
  if (h->state != kFresh) return fail(h, IMEXLB_ERR_STATE, "imexlb_init_pdf needs a fresh upload");
  CK(h, cudaSetDevice(h->device));
  TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
    return imx::launch_init_pdf(h->dim, h->rho_one, h->dg, h->dc,
                                imx::DevState{h->d_mask, h->d_inlet}, h->d_p, h->d_u, h->d_f,
                                h->stream);
  }));
  CK(h, cudaStreamSynchronize(h->stream));
  TRY(collect_times(h));
  return IMEXLB_OK;
}

static int step_impl(imexlb_t* h, int iter0, int nsteps, int interv, double* umax_log, int every,
                     double* force_log) {
  if (!h) return IMEXLB_ERR_ARG;
  if (h->member)
    return fail(h, IMEXLB_ERR_STATE, "a rank of a multi-rank run is stepped by imexlb_group_step");
  if (h->state == kEmpty) return fail(h, IMEXLB_ERR_STATE, "imexlb_upload must come first");
  if (nsteps < 0) return fail(h, IMEXLB_ERR_ARG, "nsteps < 0");
  CK(h, cudaSetDevice(h->device));
  int nmon = 0;
  if (interv > 0)
    for (int it = iter0; it < iter0 + nsteps; ++it)
      if (it % interv == 0) ++nmon;
  if (nmon > h->mon_cap) {
    dfree(&h->d_mon);
    TRY(dalloc(h, &h->d_mon, (size_t)nmon));
    h->mon_cap = nmon;
  }
  if (nmon) CK(h, cudaMemsetAsync(h->d_mon, 0, sizeof(unsigned long long) * nmon, h->stream));
  int nobs = 0;
  if (every > 0)
    for (int it = iter0; it < iter0 + nsteps; ++it)
      if (it % every == 0) ++nobs;
  const int64_t need = (int64_t)nobs * h->dim;
  if (need > h->force_cap) {
    dfree(&h->d_force_log);
    TRY(dalloc(h, &h->d_force_log, (size_t)need));
    h->force_cap = need;
  }
  int ob = 0;
  const imx::DevState st = step_state(h);
  const bool fused = fused_fill(h);
  // steps with the separate kernel pull the ghost slots fused steps left out
  // (after a change of fill mode or FP64 variant)
  if (!fused) TRY(sync_ghosts(h));
  auto plain = [&](int it) {
    return !(interv > 0 && it % interv == 0) && !(every > 0 && it % every == 0);
  };
  int m = 0;
  for (int it = iter0; it < iter0 + nsteps; ++it) {
    // A run of plain iterations starting from fb[0]: replay the longest
    // captured graph that fits (per-launch timing needs individual launches,
    // so not when timing).
    if (!h->timing && h->state == kPiped && h->cur == 0) {
      int k = 1;
      for (; k >= 0; --k) {
        const int len = kGraphLen[k];
        bool ok = it + len <= iter0 + nsteps;
        for (int j = 0; ok && j < len; ++j) ok = plain(it + j);
        if (ok) break;
      }
      if (k >= 0) {
        TRY(ensure_graph(h, k));
        CK(h, cudaGraphLaunch(h->graph_exec[k], h->stream));
        h->prof.launches[IMEXLB_KERNEL_STEP] += kGraphLen[k];
        if (!fused) h->prof.launches[IMEXLB_KERNEL_FILL] += kGraphLen[k];
        h->ghosts_stale = fused;
        it += kGraphLen[k] - 1;
        continue;
      }
    }
    unsigned long long* mon = (interv > 0 && it % interv == 0) ? h->d_mon + m++ : nullptr;
    if (h->state == kFresh) {
      TRY(run_kernel(h, IMEXLB_KERNEL_FIRST, [&] {
        if (h->exact)
          return imx::launch_collide_fpu(h->dim, h->rho_one, h->dg, h->dc, st, h->d_f, h->d_p,
                                         h->d_u, (double*)h->d_fb[0], mon, h->stream);
        return imx::launch_collide_fpu_lp(h->dim, h->store, h->dg, h->dcf, st, h->d_f, h->d_p,
                                          h->d_u, h->d_fb[0], mon, h->stream);
      }));
      TRY(run_kernel(h, IMEXLB_KERNEL_FILL, [&] {
        return imx::launch_fill(h->store, h->d_fill, h->fill_narrow, h->n_fill, h->d_fb[0], h->d_fb[1], h->stream);
      }));
      h->cur = 0;
      h->state = kPiped;
      h->ghosts_stale = false;
    } else {
      void* fin = h->d_fb[h->cur];
      void* fout = h->d_fb[1 - h->cur];
      TRY(run_kernel(h, IMEXLB_KERNEL_STEP, [&] { return launch_step_kind(h, st, fin, fout, mon); }));
      if (!fused)
        TRY(run_kernel(h, IMEXLB_KERNEL_FILL, [&] {
          return imx::launch_fill(h->store, h->d_fill, h->fill_narrow, h->n_fill, fout, fin, h->stream);
        }));
      h->cur = 1 - h->cur;
      h->ghosts_stale = fused;
    }
    if (every > 0 && it % every == 0) {
      double* dst = h->d_force_log + (int64_t)(ob++) * h->dim;
      TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
        return imx::launch_forces(h->dim, h->store, h->d_links, h->n_links, h->d_fb[h->cur], dst,
                                  h->stream);
      }));
    }
  }
  std::vector<double> mon_values;
  if (nmon && (umax_log || h->watchdog)) {
    std::vector<unsigned long long> bits((size_t)nmon);
    CK(h, cudaMemcpyAsync(bits.data(), h->d_mon, sizeof(unsigned long long) * nmon,
                          cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    mon_values.resize((size_t)nmon);
    for (int i = 0; i < nmon; ++i) std::memcpy(&mon_values[(size_t)i], &bits[(size_t)i], sizeof(double));
    if (umax_log) std::copy(mon_values.begin(), mon_values.end(), umax_log);
  } else {
    CK(h, cudaStreamSynchronize(h->stream));
  }
  if (nobs && force_log)
    CK(h, cudaMemcpy(force_log, h->d_force_log, sizeof(double) * (size_t)need, cudaMemcpyDeviceToHost));
  TRY(collect_times(h));
  if (*(volatile int*)h->stage_status) {
    *(volatile int*)h->stage_status = 0;
    return fail(h, IMEXLB_ERR_TIMEOUT,
                "the staged step kernel gave up waiting for its bulk copies (the state of this "
                "call's iterations is not valid)");
  }
  if (h->watchdog) {
    // the Monitor maximum orders NaN above every finite value, so one
    // diverged fluid node makes its iteration's value non-finite
    int k = 0;
    for (int it = iter0; it < iter0 + nsteps && interv > 0; ++it) {
      if (it % interv != 0) continue;
      const double v = mon_values[(size_t)k++];
      if (!std::isfinite(v)) {
        char msg[160];
        std::snprintf(msg, sizeof msg,
                      "diverged: the Monitor value of iteration %d is %s (the state holds the "
                      "iterations of this call)", it, std::isnan(v) ? "NaN" : "infinite");
        return fail(h, IMEXLB_ERR_DIVERGED, msg);
      }
    }
  }
  return IMEXLB_OK;
}

int imexlb_step(imexlb_t* h, int iter0, int nsteps, int interv, double* umax_log) {
  return step_impl(h, iter0, nsteps, interv, umax_log, 0, nullptr);
}

int imexlb_step_observed(imexlb_t* h, int iter0, int nsteps, int interv, double* umax_log,
                         int every, double* force_log) {
  return step_impl(h, iter0, nsteps, interv, umax_log, every, force_log);
}

int imexlb_observe(imexlb_t* h, double* force, double* mass) {
  if (!h) return IMEXLB_ERR_ARG;
  if (h->state == kEmpty) return fail(h, IMEXLB_ERR_STATE, "nothing uploaded");
  CK(h, cudaSetDevice(h->device));
  // After an upload the state is the uploaded f (already propagated) and fb;
  // otherwise f is pulled from the current post-BC buffer.
  const bool fresh = h->state == kFresh;
  const void* fb = fresh ? h->d_fb[0] : h->d_fb[h->cur];
  if (force)
    TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
      return imx::launch_forces(h->dim, h->store, h->d_links, h->n_links, fb, h->d_obs, h->stream);
    }));
  if (mass) {
    if (!fresh) TRY(sync_ghosts(h));  // the mass sum pulls
    imx::DevGrid g = h->dg;
    const void* src = fb;
    int store = h->store;
    if (fresh) {
      for (int iq = 0; iq < h->Q; ++iq) g.off[iq] = 0;  // read f in place
      src = h->d_f;
      store = imx::kStoreF64;
    }
    TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
      return imx::launch_mass(h->dim, store, g, imx::DevState{h->d_mask, h->d_inlet}, src,
                              h->d_mass_partials, h->d_obs + 3, h->stream);
    }));
  }
  double obs[4] = {0, 0, 0, 0};
  CK(h, cudaMemcpyAsync(obs, h->d_obs, sizeof obs, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (force)
    for (int k = 0; k < h->dim; ++k) force[k] = obs[k];
  if (mass) *mass = obs[3];
  return collect_times(h);
}

int imexlb_download(imexlb_t* h, double* f, double* fb, double* p, double* u) {
  if (!h) return IMEXLB_ERR_ARG;
  if (h->state == kEmpty) return fail(h, IMEXLB_ERR_STATE, "nothing uploaded");
  CK(h, cudaSetDevice(h->device));
  const int Q = h->Q;
  if (h->state == kPiped) {
    TRY(sync_ghosts(h));
    // Propagation + PostProcessing of the last iteration.
    const imx::DevState st{h->d_mask, h->d_inlet};
    TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
      if (h->exact)
        return imx::launch_finalize(h->dim, h->rho_one, h->dg, h->dc, st,
                                    (const double*)h->d_fb[h->cur], h->d_f, h->d_p, h->d_u,
                                    h->stream);
      return imx::launch_finalize_lp(h->dim, h->store, h->dg, h->dcf, st, h->d_fb[h->cur], h->d_f,
                                     h->d_p, h->d_u, h->stream);
    }));
    TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
      return imx::launch_columns(h->dim, h->dg, h->d_bl, h->nl, h->d_br, h->nr, h->d_inlet,
                                 h->d_p, h->d_u, h->stream);
    }));
    if (fb && h->member) {
      // every rank's ghost slots, from the ranks that own them
      TRY(group_sync_ghosts(h));
    } else if (fb) {
      // Every ghost slot of fb as the last BoundaryCondition left it; the
      // pipeline itself only keeps the slots a fluid node pulls.
      TRY(build_ghost_fill(h));
      TRY(run_kernel(h, IMEXLB_KERNEL_OTHER, [&] {
        return imx::launch_fill(h->store, h->d_ghost, h->fill_narrow, h->n_ghost, h->d_fb[h->cur],
                                h->d_fb[1 - h->cur], h->stream);
      }));
    }
  }
  if (f) TRY(download_field(h, h->d_f, f, Q));
  if (p) TRY(download_field(h, h->d_p, p, 1));
  if (u) TRY(download_field(h, h->d_u, u, h->dim));
  if (fb) TRY(download_field(h, h->d_fb[h->cur], fb, Q, h->store));
  CK(h, cudaStreamSynchronize(h->stream));
  return collect_times(h);
}

int imexlb_profile_reset(imexlb_t* h, int timing) {
  if (!h) return IMEXLB_ERR_ARG;
  if (!h->pending.empty()) {
    CK(h, cudaStreamSynchronize(h->stream));
    TRY(collect_times(h));
  }
  h->prof = imexlb_profile{};
  h->timing = timing != 0;
  return IMEXLB_OK;
}

int imexlb_profile_read(const imexlb_t* h, imexlb_profile* out) {
  if (!h || !out) return IMEXLB_ERR_ARG;
  *out = h->prof;
  return IMEXLB_OK;
}

int imexlb_get_info(const imexlb_t* h, imexlb_info* info) {
  if (!h || !info) return IMEXLB_ERR_ARG;
  info->array_size = h->N;
  int64_t interior = 1;
  for (int k = 0; k < h->dim; ++k) interior *= h->g.L[k];
  info->interior = interior;
  info->size_fluid = h->size_fluid;
  info->n_fill = h->n_fill;
  info->n_user = (int64_t)h->bmap.user_cells().size();
  info->n_links = h->n_links;
  info->device_bytes = h->device_bytes;
  return IMEXLB_OK;
}

int imexlb_fp64_fma_rate(int device, double* fma_per_s) {
  if (!fma_per_s) return IMEXLB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return IMEXLB_ERR_CUDA;
  return imx::measure_dfma_rate(fma_per_s) == cudaSuccess ? IMEXLB_OK : IMEXLB_ERR_CUDA;
}

int imexlb_fp64_splits(void) { return imx::step_splits(); }

int imexlb_set_fp64_split(imexlb_t* h, int split) {
  if (!h) return IMEXLB_ERR_ARG;
  if (split < 0 || split >= imx::step_splits()) return fail(h, IMEXLB_ERR_ARG, "fp64 split out of range");
  if (split == h->split) return IMEXLB_OK;
  TRY(drop_graphs(h));  // captured with the previous kernel variant
  h->split = split;
  return IMEXLB_OK;
}

int imexlb_set_fill_mode(imexlb_t* h, int mode) {
  if (!h) return IMEXLB_ERR_ARG;
  if (mode != IMEXLB_FILL_KERNEL && mode != IMEXLB_FILL_FUSED)
    return fail(h, IMEXLB_ERR_ARG, "fill mode must be IMEXLB_FILL_KERNEL or IMEXLB_FILL_FUSED");
  if (mode == IMEXLB_FILL_FUSED && h->have_geom && !h->fused_ok)
    return fail(h, IMEXLB_ERR_UNSUPPORTED, "this geometry's boundary copies need the separate fill kernel");
  if (mode == h->fill_mode) return IMEXLB_OK;
  TRY(drop_graphs(h));  // captured with the previous mode
  // the separate kernel's steps pull the ghost slots the fused ones left out
  TRY(sync_ghosts(h));
  h->fill_mode = mode;
  return IMEXLB_OK;
}

int imexlb_get_fill_mode(const imexlb_t* h, int* mode) {
  if (!h || !mode) return IMEXLB_ERR_ARG;
  *mode = fused_fill(h) ? IMEXLB_FILL_FUSED : IMEXLB_FILL_KERNEL;
  return IMEXLB_OK;
}

int imexlb_set_watchdog(imexlb_t* h, int on) {
  if (!h) return IMEXLB_ERR_ARG;
  h->watchdog = on != 0;
  return IMEXLB_OK;
}

int imexlb_get_stream(const imexlb_t* h, void** stream) {
  if (!h || !stream) return IMEXLB_ERR_ARG;
  *stream = (void*)h->stream;
  return IMEXLB_OK;
}

void imexlb_destroy(imexlb_t* h) {
  if (!h) return;
  if (h->group)  // the group reports the missing rank instead of using it
    for (imexlb_t*& r : h->group->ranks)
      if (r == h) r = nullptr;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  dfree(&h->d_mask);
  dfree(&h->d_groups);
  dfree((uint8_t**)&h->d_fb[0]);
  dfree((uint8_t**)&h->d_fb[1]);
  dfree(&h->d_f);
  dfree(&h->d_p);
  dfree(&h->d_u);
  dfree(&h->d_stage);
  dfree(&h->d_inlet);
  dfree((uint8_t**)&h->d_fill);
  dfree(&h->d_bnd);
  dfree(&h->d_bnd_at);
  dfree(&h->d_push);
  dfree(&h->d_bl);
  dfree(&h->d_br);
  dfree(&h->d_mon);
  dfree((uint8_t**)&h->d_ghost);
  dfree(&h->d_links);
  dfree(&h->d_mass_partials);
  dfree(&h->d_obs);
  dfree(&h->d_tq);
  dfree(&h->d_offq);
  dfree(&h->d_offq_kind);
  dfree(&h->d_force_log);
  for (auto& pd : h->pending) {
    cudaEventDestroy(pd.a);
    cudaEventDestroy(pd.b);
  }
  for (cudaEvent_t e : h->event_pool) cudaEventDestroy(e);
  for (cudaGraphExec_t g : h->graph_exec)
    if (g) cudaGraphExecDestroy(g);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->join) cudaEventDestroy(h->join);
  if (h->fork) cudaEventDestroy(h->fork);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->stage_status) cudaFreeHost(h->stage_status);
  delete h;
}

int imexlb_sample(imexlb_t* h, int W, int H, float* out) {
  if (!h || !out || W <= 0 || H <= 0) return IMEXLB_ERR_ARG;
  if (h->dim != 2) return fail(h, IMEXLB_ERR_UNSUPPORTED, "imexlb_sample: 2D only");
  if (h->state != kPiped) return fail(h, IMEXLB_ERR_STATE, "imexlb_sample: step at least once after upload");
  CK(h, cudaSetDevice(h->device));
  TRY(sync_ghosts(h));
  float* d = nullptr;
  CK(h, cudaMallocAsync((void**)&d, sizeof(float) * 4 * (size_t)W * H, h->stream));
  cudaError_t e = imx::launch_sample(h->store, h->dg, h->dcf, imx::DevState{h->d_mask, h->d_inlet},
                                     h->g.L[0], h->g.L[1], h->d_fb[h->cur], W, H, d, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d, sizeof(float) * 4 * (size_t)W * H, cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(d, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "imexlb_sample");
  h->prof.launches[IMEXLB_KERNEL_OTHER]++;
  return IMEXLB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Ensembles
// ---------------------------------------------------------------------------

struct imexlb_batch_s {
  std::vector<imexlb_t*> cases;
  int dim = 2, store = imx::kStoreF32, device = 0;
  cudaStream_t stream = nullptr;
  std::vector<imx::BatchCase> table;
  imx::BatchCase* d_table = nullptr;
  uint16_t* d_block_case = nullptr;
  int64_t nblocks = 0;
  uint16_t* d_fill_case = nullptr;
  int64_t nfill_blocks = 0;
  int* d_counter = nullptr;
  int shape = 1;
  cudaGraphExec_t exec = nullptr;  // kGraphIters captured iterations
  std::string err;
  // persistent stepping (batch_persist.cu): one cooperative launch per call
  int mode = IMEXLB_BATCH_LOCKSTEP;
  int persist_blocks = 0;
  int* d_order = nullptr;
  long long* d_tile_pre = nullptr;
  long long* d_fill_pre = nullptr;
  long long* d_iter_start = nullptr;
  int* d_active = nullptr;
  int iter_cap = 0;
  unsigned long long* d_next = nullptr;  // work counter, then per case done_step, done_fill
  unsigned* d_done = nullptr;
  int* d_status = nullptr;               // status, info[3]
  unsigned long long wait_budget_ns = 2000000000ull;
  int stall_case = -1;
};

namespace {

constexpr int kGraphIters = 8;

int bfail(imexlb_batch_t* b, int code, const std::string& m) {
  b->err = m;
  return code;
}

#define BCK(b, call)                                                                 \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return bfail(b, IMEXLB_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

void batch_free_tables(imexlb_batch_t* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  if (b->d_block_case) cudaFree(b->d_block_case);
  if (b->d_fill_case) cudaFree(b->d_fill_case);
  b->d_block_case = nullptr;
  b->d_fill_case = nullptr;
}

// Block -> case tables for launch shape `shape`.
int batch_build_tables(imexlb_batch_t* b, int shape) {
  batch_free_tables(b);
  const imx::BatchShape sh = imx::kBatchShapes[shape];
  std::vector<uint16_t> bc, fc;
  for (size_t i = 0; i < b->cases.size(); ++i) {
    imexlb_t* h = b->cases[i];
    imx::BatchCase& t = b->table[i];
    const int64_t span = h->dg.id_hi - h->dg.id_lo;
    const int64_t per = (int64_t)sh.block * sh.cpt;
    t.block0 = (int64_t)bc.size();
    bc.insert(bc.end(), (size_t)((span + per - 1) / per), (uint16_t)i);
    t.fill_block0 = (int64_t)fc.size();
    fc.insert(fc.end(), (size_t)((h->n_fill + 255) / 256), (uint16_t)i);
  }
  b->nblocks = (int64_t)bc.size();
  b->nfill_blocks = (int64_t)fc.size();
  BCK(b, cudaMalloc((void**)&b->d_block_case, sizeof(uint16_t) * (bc.size() + 1)));
  BCK(b, cudaMalloc((void**)&b->d_fill_case, sizeof(uint16_t) * (fc.size() + 1)));
  BCK(b, cudaMemcpy(b->d_block_case, bc.data(), sizeof(uint16_t) * bc.size(), cudaMemcpyHostToDevice));
  if (!fc.empty())
    BCK(b, cudaMemcpy(b->d_fill_case, fc.data(), sizeof(uint16_t) * fc.size(), cudaMemcpyHostToDevice));
  b->shape = shape;
  return IMEXLB_OK;
}

cudaError_t batch_iteration(imexlb_batch_t* b) {
  return imx::launch_batch_iteration(b->dim, b->store, b->shape, b->d_table, b->d_block_case,
                                     b->nblocks, b->d_fill_case, b->nfill_blocks, b->d_counter,
                                     b->stream);
}

// Load per-case parity and budgets, reset the counter. A batch runs each
// case's fill list after every step (the batched kernel keeps the plain
// pull: its several-nodes-per-thread shapes need the registers), so a case
// first gets the ghost slots its own fused steps left out.
int batch_prepare(imexlb_batch_t* b, const std::vector<int>& steps) {
  for (size_t i = 0; i < b->cases.size(); ++i) {
    imexlb_t* h = b->cases[i];
    if (h->ghosts_stale && steps[i] > 0) {
      const int rc = sync_ghosts(h);
      if (rc) return bfail(b, rc, h->err);
      BCK(b, cudaStreamSynchronize(h->stream));
    }
    b->table[i].parity0 = h->cur;
    b->table[i].nsteps = steps[i];
  }
  BCK(b, cudaMemcpyAsync(b->d_table, b->table.data(), sizeof(imx::BatchCase) * b->table.size(),
                         cudaMemcpyHostToDevice, b->stream));
  BCK(b, cudaMemsetAsync(b->d_counter, 0, sizeof(int), b->stream));
  return IMEXLB_OK;
}

void batch_finish(imexlb_batch_t* b, const std::vector<int>& steps) {
  for (size_t i = 0; i < b->cases.size(); ++i) {
    imexlb_t* h = b->cases[i];
    h->cur = (h->cur + steps[i]) & 1;
    h->prof.launches[IMEXLB_KERNEL_STEP] += steps[i];
    h->prof.launches[IMEXLB_KERNEL_FILL] += steps[i];
  }
}

// Run max(steps) lockstep iterations (graph replay for whole groups).
int batch_run(imexlb_batch_t* b, const std::vector<int>& steps) {
  int most = 0;
  for (int v : steps) most = v > most ? v : most;
  int rc = batch_prepare(b, steps);
  if (rc) return rc;
  int done = 0;
  if (most >= kGraphIters) {
    if (!b->exec) {
      cudaGraph_t graph = nullptr;
      BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaSuccess;
      for (int k = 0; k < kGraphIters && e == cudaSuccess; ++k) e = batch_iteration(b);
      cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return bfail(b, IMEXLB_ERR_CUDA, std::string("batch graph capture: ") +
                                             cudaGetErrorString(e != cudaSuccess ? e : e2));
      }
      e = cudaGraphInstantiate(&b->exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        b->exec = nullptr;
        return bfail(b, IMEXLB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      }
    }
    for (; done + kGraphIters <= most; done += kGraphIters) BCK(b, cudaGraphLaunch(b->exec, b->stream));
  }
  for (; done < most; ++done) BCK(b, batch_iteration(b));
  BCK(b, cudaStreamSynchronize(b->stream));
  batch_finish(b, steps);
  return IMEXLB_OK;
}

// Allocate the persistent schedule's device arrays for up to `iters`
// iterations per call.
int persist_reserve(imexlb_batch_t* b, int iters) {
  const size_t nc = b->cases.size();
  if (!b->d_order) {
    BCK(b, cudaMalloc((void**)&b->d_order, sizeof(int) * nc));
    BCK(b, cudaMalloc((void**)&b->d_tile_pre, sizeof(long long) * (nc + 1)));
    BCK(b, cudaMalloc((void**)&b->d_fill_pre, sizeof(long long) * (nc + 1)));
    BCK(b, cudaMalloc((void**)&b->d_next, sizeof(unsigned long long)));
    BCK(b, cudaMalloc((void**)&b->d_done, sizeof(unsigned) * 2 * nc));
    BCK(b, cudaMalloc((void**)&b->d_status, sizeof(int) * 4));
    BCK(b, imx::persistent_grid(b->dim, b->store, (int)nc, &b->persist_blocks));
    if (b->persist_blocks <= 0) return bfail(b, IMEXLB_ERR_CUDA, "persistent kernel: no resident block");
  }
  if (iters > b->iter_cap) {
    if (b->d_iter_start) cudaFree(b->d_iter_start);
    if (b->d_active) cudaFree(b->d_active);
    b->d_iter_start = nullptr;
    b->d_active = nullptr;
    b->iter_cap = 0;
    BCK(b, cudaMalloc((void**)&b->d_iter_start, sizeof(long long) * ((size_t)iters + 1)));
    BCK(b, cudaMalloc((void**)&b->d_active, sizeof(int) * (size_t)iters));
    b->iter_cap = iters;
  }
  return IMEXLB_OK;
}

// All iterations of a call in one cooperative launch of the persistent
// kernel: work items numbered iteration-major (step tiles, then fill chunks
// of the cases still running), taken in order by the resident blocks.
int batch_run_persistent(imexlb_batch_t* b, const std::vector<int>& steps) {
  int most = 0;
  for (int v : steps) most = v > most ? v : most;
  int rc = batch_prepare(b, steps);
  if (rc) return rc;
  if (most == 0) return IMEXLB_OK;
  rc = persist_reserve(b, most);
  if (rc) return rc;
  const int nc = (int)b->cases.size();
  std::vector<int> order((size_t)nc);
  for (int i = 0; i < nc; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return steps[(size_t)x] > steps[(size_t)y]; });
  std::vector<long long> tile_pre((size_t)nc + 1, 0), fill_pre((size_t)nc + 1, 0);
  for (int k = 0; k < nc; ++k) {
    const imexlb_t* h = b->cases[(size_t)order[(size_t)k]];
    const int64_t span = h->dg.id_hi - h->dg.id_lo;
    tile_pre[(size_t)k + 1] = tile_pre[(size_t)k] + (span + imx::kPersistTile - 1) / imx::kPersistTile;
    fill_pre[(size_t)k + 1] =
        fill_pre[(size_t)k] + (h->n_fill + imx::kPersistFillChunk - 1) / imx::kPersistFillChunk;
  }
  std::vector<int> active((size_t)most);
  std::vector<long long> iter_start((size_t)most + 1, 0);
  int a = nc;
  for (int n = 0; n < most; ++n) {
    while (a > 0 && steps[(size_t)order[(size_t)a - 1]] <= n) --a;
    active[(size_t)n] = a;
    iter_start[(size_t)n + 1] = iter_start[(size_t)n] + tile_pre[(size_t)a] + fill_pre[(size_t)a];
  }
  cudaStream_t st = b->stream;
  BCK(b, cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * (size_t)nc, cudaMemcpyHostToDevice, st));
  BCK(b, cudaMemcpyAsync(b->d_tile_pre, tile_pre.data(), sizeof(long long) * ((size_t)nc + 1),
                         cudaMemcpyHostToDevice, st));
  BCK(b, cudaMemcpyAsync(b->d_fill_pre, fill_pre.data(), sizeof(long long) * ((size_t)nc + 1),
                         cudaMemcpyHostToDevice, st));
  BCK(b, cudaMemcpyAsync(b->d_iter_start, iter_start.data(), sizeof(long long) * ((size_t)most + 1),
                         cudaMemcpyHostToDevice, st));
  BCK(b, cudaMemcpyAsync(b->d_active, active.data(), sizeof(int) * (size_t)most,
                         cudaMemcpyHostToDevice, st));
  BCK(b, cudaMemsetAsync(b->d_next, 0, sizeof(unsigned long long), st));
  BCK(b, cudaMemsetAsync(b->d_done, 0, sizeof(unsigned) * 2 * (size_t)nc, st));
  BCK(b, cudaMemsetAsync(b->d_status, 0, sizeof(int) * 4, st));
  imx::PersistSched ps{};
  ps.cases = b->d_table;
  ps.order = b->d_order;
  ps.tile_pre = b->d_tile_pre;
  ps.fill_pre = b->d_fill_pre;
  ps.iter_start = b->d_iter_start;
  ps.active = b->d_active;
  ps.nitems = iter_start[(size_t)most];
  ps.ncases = nc;
  ps.next = b->d_next;
  ps.done_step = b->d_done;
  ps.done_fill = b->d_done + nc;
  ps.status = b->d_status;
  ps.info = b->d_status + 1;
  ps.budget_ns = b->wait_budget_ns;
  ps.stall_case = b->stall_case;
  BCK(b, imx::launch_batch_persistent(b->dim, b->store, b->persist_blocks, ps, st));
  int status[4] = {0, 0, 0, 0};
  BCK(b, cudaMemcpyAsync(status, b->d_status, sizeof status, cudaMemcpyDeviceToHost, st));
  BCK(b, cudaStreamSynchronize(st));
  if (status[0] != 0) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "persistent batch: a wait gave up after %.3f s (case %d, iteration %d of the "
                  "call, waiting for its %s); the cases' states are undefined",
                  (double)b->wait_budget_ns * 1e-9, status[1], status[2],
                  status[3] == 0 ? "boundary copies" : "step tiles");
    return bfail(b, IMEXLB_ERR_TIMEOUT, msg);
  }
  batch_finish(b, steps);
  return IMEXLB_OK;
}

}  // namespace

extern "C" {

const char* imexlb_batch_last_error(const imexlb_batch_t* b) { return b ? b->err.c_str() : ""; }

int imexlb_batch_set_mode(imexlb_batch_t* b, int mode) {
  if (!b || (mode != IMEXLB_BATCH_LOCKSTEP && mode != IMEXLB_BATCH_PERSISTENT)) return IMEXLB_ERR_ARG;
  if (mode == IMEXLB_BATCH_PERSISTENT && b->cases.size() > 2048)
    return bfail(b, IMEXLB_ERR_UNSUPPORTED, "persistent mode takes at most 2048 cases");
  b->mode = mode;
  return IMEXLB_OK;
}

int imexlb_testing_stage_stall(imexlb_t* h, double budget_s) {
  if (!h || !(budget_s <= 60.0)) return IMEXLB_ERR_ARG;
  h->stage_stall = budget_s > 0.0;
  h->stage_wait_ns = h->stage_stall ? (unsigned long long)(budget_s * 1e9) : 2000000000ull;
  TRY(drop_graphs(h));  // captured iterations hold the previous plan
  return IMEXLB_OK;
}

int imexlb_testing_set_staged_kernel(imexlb_t* h, int on) {
  if (!h) return IMEXLB_ERR_ARG;
  h->staged = on != 0;
  TRY(drop_graphs(h));  // captured iterations hold the previous kernel
  return IMEXLB_OK;
}

int imexlb_testing_batch_stall(imexlb_batch_t* b, int case_index, double budget_s) {
  if (!b || case_index >= (int)b->cases.size() || !(budget_s > 0.0)) return IMEXLB_ERR_ARG;
  b->stall_case = case_index < 0 ? -1 : case_index;
  b->wait_budget_ns = (unsigned long long)(budget_s * 1e9);
  return IMEXLB_OK;
}

int imexlb_batch_create(imexlb_batch_t** out, imexlb_t* const* cases, int ncases) {
  if (!out || !cases || ncases <= 0) return IMEXLB_ERR_ARG;
  *out = nullptr;
  if (ncases > 65535) return IMEXLB_ERR_ARG;
  imexlb_batch_t* b = new (std::nothrow) imexlb_batch_s();
  if (!b) return IMEXLB_ERR_NOMEM;
  auto reject = [&](int code) {
    delete b;
    return code;
  };
  for (int i = 0; i < ncases; ++i) {
    imexlb_t* h = cases[i];
    if (!h || !h->have_geom) return reject(IMEXLB_ERR_ARG);
    if (h->state != kPiped) return reject(IMEXLB_ERR_STATE);
    if (h->store == imx::kStoreF64 || h->store == imx::kStoreFix)
      return reject(IMEXLB_ERR_UNSUPPORTED);  // narrow kinds only
    if (i > 0 && (h->device != cases[0]->device || h->dim != cases[0]->dim ||
                  h->store != cases[0]->store))
      return reject(IMEXLB_ERR_ARG);
    b->cases.push_back(h);
  }
  b->dim = cases[0]->dim;
  b->store = cases[0]->store;
  b->device = cases[0]->device;
  if (cudaSetDevice(b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return reject(IMEXLB_ERR_CUDA);
  b->table.resize((size_t)ncases);
  for (int i = 0; i < ncases; ++i) {
    imexlb_t* h = cases[i];
    imx::BatchCase& t = b->table[(size_t)i];
    t = imx::BatchCase{};
    t.g = h->dg;
    t.c = h->dcf.f;
    t.mask = h->d_mask;
    t.inlet = h->d_inlet;
    t.fb[0] = h->d_fb[0];
    t.fb[1] = h->d_fb[1];
    t.fill = h->d_fill;
    t.n_fill = h->n_fill;
    t.fill_narrow = h->fill_narrow ? 1 : 0;
  }
  if (cudaMalloc((void**)&b->d_table, sizeof(imx::BatchCase) * (size_t)ncases) != cudaSuccess ||
      cudaMalloc((void**)&b->d_counter, sizeof(int)) != cudaSuccess) {
    imexlb_batch_destroy(b);
    return IMEXLB_ERR_NOMEM;
  }
  if (batch_build_tables(b, 1) != IMEXLB_OK) {
    imexlb_batch_destroy(b);
    return IMEXLB_ERR_CUDA;
  }
  *out = b;
  return IMEXLB_OK;
}

int imexlb_batch_tune(imexlb_batch_t* b, int trial, int* shape) {
  if (!b || trial <= 0) return IMEXLB_ERR_ARG;
  BCK(b, cudaSetDevice(b->device));
  cudaEvent_t e0, e1;
  BCK(b, cudaEventCreate(&e0));
  BCK(b, cudaEventCreate(&e1));
  float best = 1e30f;
  int best_shape = b->shape;
  std::vector<int> steps(b->cases.size(), trial);
  for (int sh = 0; sh < imx::kNumBatchShapes; ++sh) {
    int rc = batch_build_tables(b, sh);
    if (!rc) rc = batch_prepare(b, steps);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    BCK(b, cudaEventRecord(e0, b->stream));
    for (int k = 0; k < trial; ++k) BCK(b, batch_iteration(b));
    BCK(b, cudaEventRecord(e1, b->stream));
    BCK(b, cudaEventSynchronize(e1));
    float ms = 0.f;
    BCK(b, cudaEventElapsedTime(&ms, e0, e1));
    batch_finish(b, steps);
    if (ms < best) {
      best = ms;
      best_shape = sh;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int rc = batch_build_tables(b, best_shape);
  if (rc) return rc;
  if (shape) *shape = best_shape;
  return IMEXLB_OK;
}

int imexlb_batch_step(imexlb_batch_t* b, int nsteps, const int* steps) {
  if (!b) return IMEXLB_ERR_ARG;
  BCK(b, cudaSetDevice(b->device));
  std::vector<int> s(b->cases.size());
  for (size_t i = 0; i < s.size(); ++i) {
    s[i] = steps ? steps[i] : nsteps;
    if (s[i] < 0) return bfail(b, IMEXLB_ERR_ARG, "negative iteration count");
  }
  return b->mode == IMEXLB_BATCH_PERSISTENT ? batch_run_persistent(b, s) : batch_run(b, s);
}

const char* imexlb_group_last_error(const imexlb_group_t* g) { return g ? g->err.c_str() : ""; }

int imexlb_group_create(imexlb_group_t** out, imexlb_t* const* ranks, int nprocs) {
  if (!out || !ranks || nprocs < 1) return IMEXLB_ERR_ARG;
  *out = nullptr;
  imexlb_t* h0 = ranks[0];
  if (!h0) return IMEXLB_ERR_ARG;
  auto reject = [&](int code, const std::string& m) {
    imx::set_thread_error(m.c_str());
    return code;
  };
  const imexlb_desc& d0 = h0->d;
  const int dim = d0.dim;
  const int gl[3] = {d0.nx + 1, d0.ny + 1, dim == 3 ? d0.nz + 1 : 1};
  int np[3] = {1, 1, 1};
  if (imexlb_host_decompose(dim, gl, nprocs, np) != IMEXLB_OK)
    return reject(IMEXLB_ERR_ARG, "imexlb_group_create: no decomposition");
  for (int a = 0; a < nprocs; ++a) {
    imexlb_t* h = ranks[a];
    if (!h) return reject(IMEXLB_ERR_ARG, "imexlb_group_create: null rank");
    if (h->group) return reject(IMEXLB_ERR_STATE, "imexlb_group_create: a rank is already grouped");
    if (!h->have_geom) return reject(IMEXLB_ERR_STATE, "imexlb_group_create: a rank has no geometry");
    if (!h->exact) return reject(IMEXLB_ERR_UNSUPPORTED, "imexlb_group_create: ranks need IMEXLB_FP64");
    const imexlb_desc& d = h->d;
    if (d.dim != dim || d.nx != d0.nx || d.ny != d0.ny || (dim == 3 && d.nz != d0.nz) ||
        d.device != d0.device || d.ome != d0.ome || d.rho0 != d0.rho0 || d.uu != d0.uu)
      return reject(IMEXLB_ERR_ARG, "imexlb_group_create: ranks of different runs");
    // the box SetLocalLength gives MPI rank a (row-major Cartesian coordinates)
    int cc[3] = {0, 0, 0};
    if (dim == 2) {
      cc[0] = a / np[1];
      cc[1] = a % np[1];
    } else {
      cc[0] = a / (np[1] * np[2]);
      cc[1] = (a / np[2]) % np[1];
      cc[2] = a % np[2];
    }
    for (int k = 0; k < dim; ++k) {
      int st = 0;
      for (int q = 0; q < cc[k]; ++q) st += gl[k] / np[k] + (q < gl[k] % np[k] ? 1 : 0);
      const int len = gl[k] / np[k] + (cc[k] < gl[k] % np[k] ? 1 : 0);
      if (d.local_start[k] != st || d.local_length[k] != len)
        return reject(IMEXLB_ERR_ARG, "imexlb_group_create: rank " + std::to_string(a) +
                                          " does not have the box of its MPI rank");
    }
  }
  imexlb_group_t* g = new (std::nothrow) imexlb_group_s();
  if (!g) return reject(IMEXLB_ERR_NOMEM, "out of host memory");
  g->ranks.assign(ranks, ranks + nprocs);
  g->dim = dim;
  g->nprocs = nprocs;
  g->device = d0.device;
  for (int k = 0; k < 3; ++k) {
    g->np[k] = np[k];
    g->gl[k] = gl[k];
  }
  auto bail = [&](int rc) {
    imx::set_thread_error(g->err.c_str());
    imexlb_group_destroy(g);
    return rc;
  };
  if (cudaSetDevice(g->device) != cudaSuccess) return bail(gfail(g, IMEXLB_ERR_CUDA, "cudaSetDevice"));
  std::vector<imx::RankGeometry> rg((size_t)nprocs);
  for (int a = 0; a < nprocs; ++a) {
    imexlb_t* h = ranks[a];
    imx::RankGeometry& r = rg[(size_t)a];
    r.g = h->g;
    for (int k = 0; k < 3; ++k) r.start[k] = k < dim ? h->d.local_start[k] : 0;
    r.fluid_mask = h->mask.data();
    r.lists.fluid_mask = h->mask.data();
    r.lists.bl = h->h_bl.data(); r.lists.nl = (int)h->h_bl.size();
    r.lists.br = h->h_br.data(); r.lists.nr = (int)h->h_br.size();
    r.lists.bu = h->h_bu.data(); r.lists.nu = (int)h->h_bu.size();
    r.lists.bd = h->h_bd.data(); r.lists.nd = (int)h->h_bd.size();
    r.lists.user = h->h_user.data(); r.lists.nuser = (int)h->h_user.size();
  }
  std::string err;
  if (!g->gb.build(rg, gl, np, err)) return bail(gfail(g, IMEXLB_ERR_GEOMETRY, err));
  int rc = group_upload(g, false, &g->d_fill, &g->n_fill);
  if (rc != IMEXLB_OK) return bail(rc);
  std::vector<double*> bufs((size_t)(2 * nprocs));
  for (int a = 0; a < nprocs; ++a) {
    bufs[(size_t)(2 * a)] = (double*)ranks[a]->d_fb[0];
    bufs[(size_t)(2 * a + 1)] = (double*)ranks[a]->d_fb[1];
  }
  if (cudaMalloc((void**)&g->d_bufs, sizeof(double*) * bufs.size()) != cudaSuccess ||
      cudaMemcpy(g->d_bufs, bufs.data(), sizeof(double*) * bufs.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(gfail(g, IMEXLB_ERR_CUDA, "group allocation"));
  for (imexlb_t* h : g->ranks) h->group = g;
  *out = g;
  return IMEXLB_OK;
}

int imexlb_group_step(imexlb_group_t* g, int iter0, int nsteps, int interv, double* umax_log) {
  if (!g) return IMEXLB_ERR_ARG;
  if (nsteps < 0) return gfail(g, IMEXLB_ERR_ARG, "nsteps < 0");
  GCK(g, cudaSetDevice(g->device));
  for (imexlb_t* h : g->ranks)
    if (!h) return gfail(g, IMEXLB_ERR_STATE, "a rank of the group was destroyed");
  const int state = g->ranks[0]->state, cur = g->ranks[0]->cur;
  for (imexlb_t* h : g->ranks) {
    if (h->state == kEmpty) return gfail(g, IMEXLB_ERR_STATE, "every rank needs imexlb_upload first");
    if (h->state != state || h->cur != cur)
      return gfail(g, IMEXLB_ERR_STATE, "the ranks are not at the same iteration");
    GCK(g, cudaStreamSynchronize(h->stream));  // uploads and InitPDF
  }
  int nmon = 0;
  if (interv > 0)
    for (int it = iter0; it < iter0 + nsteps; ++it)
      if (it % interv == 0) ++nmon;
  if (nmon > g->mon_cap) {
    if (g->d_mon) cudaFree(g->d_mon);
    g->d_mon = nullptr;
    GCK(g, cudaMalloc((void**)&g->d_mon, sizeof(unsigned long long) * nmon));
    g->mon_cap = nmon;
  }
  if (nmon) GCK(g, cudaMemsetAsync(g->d_mon, 0, sizeof(unsigned long long) * nmon, g->stream));
  int st = state, c = cur, m = 0;
  for (int it = iter0; it < iter0 + nsteps; ++it) {
    // one Monitor slot for all ranks: the maximum over ranks (MPI_REDUCE MAX)
    unsigned long long* mon = (interv > 0 && it % interv == 0) ? g->d_mon + m++ : nullptr;
    for (imexlb_t* h : g->ranks) {
      const imx::DevState dst{h->d_mask, h->d_inlet, h->d_tq, h->d_offq};
      cudaError_t e;
      if (st == kFresh)
        e = imx::launch_collide_fpu(h->dim, h->rho_one, h->dg, h->dc, dst, h->d_f, h->d_p, h->d_u,
                                    (double*)h->d_fb[0], mon, g->stream);
      else
        e = imx::launch_step(h->dim, h->rho_one, h->dg, h->dc, dst, (const double*)h->d_fb[c],
                             (double*)h->d_fb[1 - c], mon, g->stream, h->split);
      if (e != cudaSuccess) return gfail(g, IMEXLB_ERR_CUDA, std::string("step: ") + cudaGetErrorString(e));
    }
    const int out_parity = st == kFresh ? 0 : 1 - c;
    GCK(g, imx::launch_fill_group(g->d_fill, g->n_fill, g->d_bufs, out_parity, g->stream));
    c = out_parity;
    st = kPiped;
  }
  for (imexlb_t* h : g->ranks) {
    h->state = st;
    h->cur = c;
  }
  if (nsteps > 0) g->ghost_dirty = true;
  if (nmon && umax_log) {
    std::vector<unsigned long long> bits((size_t)nmon);
    GCK(g, cudaMemcpyAsync(bits.data(), g->d_mon, sizeof(unsigned long long) * nmon,
                           cudaMemcpyDeviceToHost, g->stream));
    GCK(g, cudaStreamSynchronize(g->stream));
    for (int i = 0; i < nmon; ++i) std::memcpy(&umax_log[i], &bits[(size_t)i], sizeof(double));
  }
  GCK(g, cudaStreamSynchronize(g->stream));
  return IMEXLB_OK;
}

void imexlb_group_destroy(imexlb_group_t* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (imexlb_t* h : g->ranks)
    if (h && h->group == g) h->group = nullptr;
  if (g->d_fill) cudaFree(g->d_fill);
  if (g->d_ghost) cudaFree(g->d_ghost);
  if (g->d_bufs) cudaFree(g->d_bufs);
  if (g->d_mon) cudaFree(g->d_mon);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

void imexlb_batch_destroy(imexlb_batch_t* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free_tables(b);
  if (b->d_table) cudaFree(b->d_table);
  if (b->d_counter) cudaFree(b->d_counter);
  for (void* p : {(void*)b->d_order, (void*)b->d_tile_pre, (void*)b->d_fill_pre,
                  (void*)b->d_iter_start, (void*)b->d_active, (void*)b->d_next, (void*)b->d_done,
                  (void*)b->d_status})
    if (p) cudaFree(p);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
