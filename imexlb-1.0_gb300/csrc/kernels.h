// Device-side entry points of the step library (launchers for kernels.cu).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace imx {

// Storage type of the population buffers.
enum StoreKind : int {
  kStoreF64 = 0,   // IEEE double (reference arithmetic)
  kStoreF32 = 2,   // float, FP32 arithmetic
  kStoreBF16 = 3,  // bfloat16, FP32 arithmetic
  kStoreF16 = 4,   // half, FP32 arithmetic
  kStoreFix = 5,   // Q3.60 fixed point (fixed64.cuh), integer arithmetic
};
inline size_t store_bytes(int store) {
  return (store == kStoreF64 || store == kStoreFix) ? 8 : (store == kStoreF32 ? 4 : 2);
}

// Per-node flag bits of the device mask (one byte per padded cell).
enum : uint8_t {
  kMaskFluid = 1,   // listed in fluid_id: collided, streamed, post-processed
  kMaskInlet = 2,   // fluid node bl(i)+1: Dirichlet velocity (lbm.f90:186-191)
  kMaskOutlet = 4,  // fluid node br(i)-1: zero pressure (lbm.f90:195-198)
  // Fused boundary (boundary_fused.cuh), fluid nodes next to the rim or an
  // obstacle: a record (source row and obstacle copies), or closed forms.
  kMaskRecord = 8,
  kMaskWallLo = 16,  // next to the wall at -1 of the wall axis (z in 3D, y in 2D)
  kMaskWallHi = 32,  // next to the wall at n+1 of the wall axis
  kMaskPerLo = 64,   // 3D: next to the periodic face at y = -1
  kMaskPerHi = 128,  // 3D: next to the periodic face at y = ny+1
};

// Geometry of the padded grid as the kernels see it. Populations are stored
// structure-of-arrays: value (cell id, direction iq) at [iq*N + id].
struct DevGrid {
  int64_t N;             // padded cells
  int64_t id_lo, id_hi;  // linear range covering the interior
  int64_t dy, dz;        // strides (dz = 0 in 2D)
  int64_t skip_id;       // fluid_id(0): not part of Monitor (lbm.f90:213)
  int64_t off[27];       // pull offset of direction iq: e_x + dy*e_y + dz*e_z
};

// BGK coefficients (input.in line 3, InitLattice weights).
struct DevCoef {
  double t[27];
  double ome, om1, rho0;  // om1 = 1 - ome, formed on the host as the reference does
  // 1, -1 and -0: a*1+b, b*(-1)+a and a*b+(-0) as fused multiply-adds are
  // exactly a+b, a-b and a*b (one rounding of an exact value, the same signed
  // zeros). Kernel parameters, so that no compiler folds them back.
  double one, mone, mzero;
};

// One boundary slot refreshed after a collision: fout[dst] = src >= 0 ?
// fout[src] : fin[~src]  (SoA indices).
struct DevFill {
  int64_t dst;
  int64_t src;
};
// src value that stores a quiet NaN (a slot the reference fills from outside
// its arrays).
constexpr int64_t kFillNaN = INT64_MIN;

// The same entry with 32-bit slot indices (used when Q*N < 2^31).
struct DevFill32 {
  uint32_t dst;
  int32_t src;
};
constexpr int32_t kFillNaN32 = INT32_MIN;

struct DevState {
  const uint8_t* mask;
  const double* inlet;  // Dirichlet u_x by padded row (2D) / plane (3D)
  // Per-direction weight t and pull offset (DevCoef::t, DevGrid::off) in
  // device memory, for kernels that index them with a run-time direction.
  const double* tq = nullptr;
  const int64_t* offq = nullptr;
  // Boundary copies inside the step kernel (boundary_fused.cuh); null: the
  // separate fill kernel keeps the boundary slots. A node flagged
  // kMaskRecord owns the record bnd[bnd_at[id] * (Q+1) ...]: Q source slots
  // (kNoRedirect: plain pull) and one word, first push entry << 8 | count.
  const uint32_t* bnd = nullptr;
  const uint32_t* bnd_at = nullptr;
  const DevFill32* push = nullptr;
  int64_t pshift = 0;  // periodic y faces: L1 * dy
  // offq with the closed forms of a boundary node applied (the slot read for
  // direction i is i*N + id - offq_kind[kind*Q + i]), one table per kind:
  // kind = x + 3*w + 9*y with x, w, y = 0 (none), 1 (inlet / low face),
  // 2 (outlet / high face) of the x faces, the wall axis and the periodic y
  // faces (boundary_fused.cuh)
  const int64_t* offq_kind = nullptr;
};
constexpr uint32_t kNoRedirect = 0xffffffffu;  // a row entry without a redirect

// One momentum-exchange link from a fluid node x to an interior solid node
// s = x + e_iq: a = SoA slot of (x, iq), b = SoA slot of (s, nq-1-iq).
struct DevLink {
  int64_t a, b;
  int32_t iq, pad;
};

// All launchers enqueue on `s` and return the launch status.
// Collision from stored f, p, u (first iteration after an upload); monitor
// (optional) receives max |(ux,uy)| of the stored u as ordered bits.
cudaError_t launch_collide_fpu(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                               const DevState& st, const double* f, const double* p,
                               const double* u, double* fout, unsigned long long* monitor,
                               cudaStream_t s);

// Fused iteration: pull fin (post-BC of the previous iteration) -> moments ->
// inlet/outlet Dirichlet -> [Monitor] -> collision -> fout. `split` in
// [0, step_splits()) selects how many FP64 operations run in integer
// emulation (same results for every value; rho0 = 1 only, else ignored).
cudaError_t launch_step(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                        const DevState& st, const double* fin, double* fout,
                        unsigned long long* monitor, cudaStream_t s, int split = 0);
int step_splits();
int step_split_default(int dim);  // the fastest variant, used unless a host picks another
// The rho0 = 1 step kernels by split index (step_split2.cu, step_split3.cu).
cudaError_t launch_step_split2(int split, unsigned grid, const DevGrid& g, const DevCoef& c,
                               const DevState& st, const double* fin, double* fout,
                               unsigned long long* monitor, cudaStream_t s);
cudaError_t launch_step_split3(int split, unsigned grid, const DevGrid& g, const DevCoef& c,
                               const DevState& st, const double* fin, double* fout,
                               unsigned long long* monitor, cudaStream_t s);
// The default variant with the boundary copies folded in (st.bnd set).
cudaError_t launch_step_fused(int dim, bool rho_one, unsigned grid, const DevGrid& g,
                              const DevCoef& c, const DevState& st, const double* fin,
                              double* fout, unsigned long long* monitor, cudaStream_t s);

// Boundary refresh of a rank group (FP64): entry i writes rank dst_rank's
// slot dst (SoA index) with rank (src_code & 0xffff)'s slot src, read from
// that rank's buffer of this iteration or, with kGroupPrev, of the previous
// one; src_code < 0 stores NaN. bufs holds two pointers per rank (fb[0],
// fb[1]); out_parity selects the buffer being written.
struct DevGroupFill {
  int64_t dst;
  int64_t src;
  int32_t dst_rank;
  int32_t src_code;
};
constexpr int32_t kGroupPrev = 1 << 30;
cudaError_t launch_fill_group(const DevGroupFill* fill, int64_t n, double* const* bufs,
                              int out_parity, cudaStream_t s);

// Boundary refresh after a collision into fout (any storage kind); `fill` is
// DevFill32[n] when narrow, DevFill[n] otherwise.
cudaError_t launch_fill(int store, const void* fill, bool narrow, int64_t n, void* fout,
                        const void* fin, cudaStream_t s);

// Propagation + PostProcessing of the last iteration into f, p, u.
cudaError_t launch_finalize(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                            const DevState& st, const double* fin, double* f, double* p,
                            double* u, cudaStream_t s);

// PostProcessing's inlet / outlet loops over the bl / br lists (all rows).
cudaError_t launch_columns(int dim, const DevGrid& g, const int* bl, int nl, const int* br,
                           int nr, const double* inlet, double* p, double* u, cudaStream_t s);

// InitPDF: f = feq(p, u) on fluid nodes.
// InitUP on the device (initialization.f90:259-282, initialization_3d.f90:
// 282-308) for the fluid nodes of the mask: u_x = uu*4*y*(n-y)/n**2*r with
// y = local row (2D) or plane (3D) + start, r = 1 + (r_vec(mod(id,100)) -
// 0.5)*2*0.2; p and the other components are left as they are (zero).
struct RVec {
  double v[100];
};
cudaError_t launch_init_up(int dim, const DevGrid& g, const uint8_t* mask, const RVec& rv,
                           double uu, int n, int start, double* u, cudaStream_t s);

cudaError_t launch_init_pdf(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                            const DevState& st, const double* p, const double* u, double* f,
                            cudaStream_t s);

// F = sum over links of e_iq * (fb[a] + fb[b]) in double-double, one block,
// fixed reduction order; out[0..dim) receives F.
cudaError_t launch_forces(int dim, int store, const DevLink* links, int64_t n, const void* fb,
                          double* out, cudaStream_t s);

// Mass deviation sum(f) over fluid nodes of the state whose post-BC fb is
// `fin` (f = the pulled populations), double-double, deterministic.
// partials needs mass_partials_size(g) doubles.
int64_t mass_partials_size(const DevGrid& g);
cudaError_t launch_mass(int dim, int store, const DevGrid& g, const DevState& st, const void* fin,
                        double* partials, double* out, cudaStream_t s);

// Layout conversion between the reference's AoS [id*K+k] (double) and SoA
// [k*N+id] of the given storage kind (round to nearest even when narrowing).
cudaError_t launch_aos_to_soa(int store, const double* aos, void* soa, int64_t N, int K,
                              cudaStream_t s);
cudaError_t launch_soa_to_aos(int store, const void* soa, double* aos, int64_t N, int K,
                              cudaStream_t s);

// ---- FP32-arithmetic kernels for the reduced-precision storage kinds
// (kernels_lp.cu). Same contracts as the FP64 launchers above.
template <class R>
struct CoefR {
  R k[27];          // ome * t_i * rho0
  R om1, inv_rho0;  // 1 - ome, 1 / rho0
};

// Coefficients of the minimal-operation BGK update in float and double.
struct DevCoefLP {
  CoefR<float> f;
  CoefR<double> d;
  template <class R>
  const CoefR<R>& get() const {
    if constexpr (sizeof(R) == 8) return d;
    else return f;
  }
};

// Per-direction plane pointers of one iteration: in[iq] already offset by the
// pull shift (value pulled by node id is in[iq][id]), out[iq][id] the
// post-collision value of node id.
struct DevPlanes {
  const void* in[27];
  void* out[27];
};
DevPlanes make_planes(const DevGrid& g, int nq, size_t esz, const void* fin, void* fout);

// Bilinear sample of (fluid fraction, p, ux, uy) of a 2D state at W x H pixel
// centres; `fin` is the post-BC buffer (the pulled populations are the state).
cudaError_t launch_sample(int store, const DevGrid& g, const DevCoefLP& c, const DevState& st,
                          int L0, int L1, const void* fin, int W, int H, float* out,
                          cudaStream_t s);

cudaError_t launch_collide_fpu_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                                  const DevState& st, const double* f, const double* p,
                                  const double* u, void* fout, unsigned long long* monitor,
                                  cudaStream_t s);
// The kernel that stages each tile's pulled runs in shared memory with bulk
// copies (BF16 / FP16 storage):
// Cells per consumer warp of the staged kernel (two per thread): the unit in
// which it leaves boundary cells to a second kernel.
constexpr int kStageGroup = 64;

struct StagedArgs {
  int* status;              // host-visible word, set to 1 if a bounded wait gives up
  const uint32_t* groups;   // with the fused boundary handling: the
  int64_t n_groups;         // kStageGroup-cell groups from id_lo that hold a
                            // wall, periodic-face or record node (a second
                            // kernel updates them)
  unsigned long long wait_ns;  // budget of each of the kernel's waits
  int stall;                // failure injection: a block's first tile starts no copies
  cudaStream_t side;        // second stream and the two events (no timing) that
  cudaEvent_t fork, join;   // run the boundary groups beside the staged kernel
};
// staged non-null: the BF16 / FP16 kinds on D3Q27 run the staged kernel
// where the lattice's ghost layers cover its copies; null (or otherwise: D2Q9,
// FP32 / FP64 storage) the kernel that loads every population into
// registers. Identical results.
cudaError_t launch_step_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                           const DevState& st, const DevPlanes& pl, unsigned long long* monitor,
                           cudaStream_t s, const StagedArgs* staged = nullptr);
// Sets up the staged kernel (shared-memory limit, resident blocks) on the
// current device, once per process (the devices a process uses are taken to
// be alike); call it outside any stream capture.
void prepare_step_lp();
cudaError_t launch_finalize_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                               const DevState& st, const void* fin, double* f, double* p,
                               double* u, cudaStream_t s);

// ---- Fixed-point kind (kernels_fx.cu): populations in Q3.60, the node
// update on the integer pipes (node_fixed.cuh); rho0 = 1.
struct CoefFix {
  long long k[27];  // ome * t_i in Q0.63
  long long om1;    // 1 - ome in Q0.63
};
cudaError_t launch_step_fx(int dim, const DevGrid& g, const CoefFix& c, const DevState& st,
                           const DevPlanes& pl, unsigned long long* monitor, cudaStream_t s);

// FP64 fused multiply-adds per second of the current device (a short
// throughput kernel, ~40 ms).
cudaError_t measure_dfma_rate(double* fma_per_s);

}  // namespace imx
