// FP64 lattice Boltzmann kernels for sm_103a with the reference's rounding.
//
// Every floating-point operation is an explicit round-to-nearest intrinsic in
// the evaluation order of lbm.f90 (Collision lbm.f90:64-72, PostProcessing
// lbm.f90:166-179), so no multiply-add is ever fused and results equal the
// reference's serial build. Terms the reference multiplies by an integer
// lattice component in {-1,0,1} are added, subtracted or skipped; that is
// exact (it can change only the sign of an exact zero). A +/- direction pair
// shares |e.u|, e.u squared and 4.5(e.u)^2, which are exactly equal for the
// two members (e_opp = -e).
//
// GB300 has ~0.5 T FP64 add/mul per second against ~7 TB/s of HBM, so these
// kernels are bound by FP64 issue, not memory; the work per node is kept to
// the reference's own operation count.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "exact_node.cuh"
#include "kernels.h"
#include "lattice.h"
#include "storage.cuh"

namespace imx {
namespace {

template <int DIM, bool RHO1, bool MON>
__global__ void __launch_bounds__(kBlock) k_collide_fpu(DevGrid g, DevCoef c, DevState st,
                                                         const double* __restrict__ fs,
                                                         const double* __restrict__ ps,
                                                         const double* __restrict__ us,
                                                         double* __restrict__ fout,
                                                         unsigned long long* monitor) {
  using N_ = Node<DIM, RHO1>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlock + threadIdx.x;
  double um = 0.0;
  if (id < g.id_hi) {
    const uint8_t m = st.mask[id];
    if (m & kMaskFluid) {
      double f[N_::Q];
      sfor<0, N_::Q>([&](auto I) { f[I] = fs[(int64_t)I * g.N + id]; });
      double u[DIM];
      sfor<0, DIM>([&](auto K) { u[K] = us[(int64_t)K * g.N + id]; });
      const double p = ps[id];
      if constexpr (MON) {
        if (id != g.skip_id) um = speed2d(u[0], u[1]);
      }
      N_::collide(f, p, u, c, fout, g.N, id);
    }
  }
  if constexpr (MON) block_max_to(um, monitor);
}

template <int DIM, bool RHO1>
__global__ void __launch_bounds__(kBlock) k_finalize(DevGrid g, DevCoef c, DevState st,
                                                      const double* __restrict__ fin,
                                                      double* __restrict__ fs,
                                                      double* __restrict__ ps,
                                                      double* __restrict__ us) {
  using N_ = Node<DIM, RHO1>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (id >= g.id_hi) return;
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) return;
  double f[N_::Q];
  N_::pull(fin, g, id, f);
  double p, u[DIM];
  N_::moments(f, p, u, c);
  N_::dirichlet(m, id, g, st.inlet, p, u);
  sfor<0, N_::Q>([&](auto I) { fs[(int64_t)I * g.N + id] = f[I]; });
  sfor<0, DIM>([&](auto K) { us[(int64_t)K * g.N + id] = u[K]; });
  ps[id] = p;
}

template <int DIM, bool RHO1>
__global__ void __launch_bounds__(kBlock) k_init_pdf(DevGrid g, DevCoef c, DevState st,
                                                      const double* __restrict__ ps,
                                                      const double* __restrict__ us,
                                                      double* __restrict__ fs) {
  using N_ = Node<DIM, RHO1>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (id >= g.id_hi) return;
  if (!(st.mask[id] & kMaskFluid)) return;
  double u[DIM];
  sfor<0, DIM>([&](auto K) { u[K] = us[(int64_t)K * g.N + id]; });
  N_::equilibria(ps[id], u, c, [&](int i, double fe) { fs[(int64_t)i * g.N + id] = fe; });
}

template <class T, class E>
__global__ void k_fill(const E* __restrict__ fill, int64_t n, T* fout, const T* __restrict__ fin) {
  constexpr auto kNaN = sizeof(E) == sizeof(DevFill32) ? (int64_t)kFillNaN32 : kFillNaN;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const E e = fill[i];
    const int64_t src = e.src;
    T v;
    if (src >= 0) v = fout[src];
    else if (src != kNaN) v = fin[~src];
    else v = Store<T>::nan();
    fout[e.dst] = v;
  }
}

template <int DIM>
__global__ void k_columns(DevGrid g, const int* __restrict__ bl, int nl,
                          const int* __restrict__ br, int nr, const double* __restrict__ inlet,
                          double* p, double* u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nl) {
    const int64_t id = (int64_t)bl[i] + 1;
    const int64_t r = DIM == 2 ? id / g.dy : id / g.dz;
    u[id] = inlet[r];
    u[g.N + id] = 0.0;
  }
  if (i < nr) p[(int64_t)br[i] - 1] = 0.0;
}

// ---- double-double accumulation (error-free TwoSum), used for the force and
// mass sums so that the result does not depend on the summation order to
// within ~1e-30 relative.
struct DD {
  double hi, lo;
};

__device__ IMX_FI DD dd_add(DD a, double x) {
  const double s = __dadd_rn(a.hi, x);
  const double bp = __dsub_rn(s, a.hi);
  const double e = __dadd_rn(__dsub_rn(a.hi, __dsub_rn(s, bp)), __dsub_rn(x, bp));
  return DD{s, __dadd_rn(a.lo, e)};
}

__device__ IMX_FI DD dd_add(DD a, DD b) {
  DD r = dd_add(a, b.hi);
  r.lo = __dadd_rn(r.lo, b.lo);
  // renormalise (Fast2Sum, |hi| >= |lo|)
  const double s = __dadd_rn(r.hi, r.lo);
  const double e = __dsub_rn(r.lo, __dsub_rn(s, r.hi));
  return DD{s, e};
}

constexpr int kRedThreads = 512;

// Fixed-shape tree reduction of one DD per component across the block.
template <int NC>
__device__ IMX_FI void block_dd_reduce(DD (&v)[NC], DD (*sh)[NC]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int c = 0; c < NC; ++c) sh[t][c] = v[c];
  __syncthreads();
  for (int stride = kRedThreads / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
#pragma unroll
      for (int c = 0; c < NC; ++c) sh[t][c] = dd_add(sh[t][c], sh[t + stride][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) v[c] = sh[0][c];
}

template <int DIM, class T>
__global__ void __launch_bounds__(kRedThreads) k_forces(const DevLink* __restrict__ links,
                                                         int64_t n, const T* __restrict__ fb,
                                                         double* out) {
  using Lat = Lattice<DIM>;
  __shared__ DD sh[kRedThreads][DIM];
  DD acc[DIM];
#pragma unroll
  for (int c = 0; c < DIM; ++c) acc[c] = DD{0.0, 0.0};
  for (int64_t i = threadIdx.x; i < n; i += kRedThreads) {
    const DevLink L = links[i];
    const double v = __dadd_rn(Store<T>::to_d(fb[L.a]), Store<T>::to_d(fb[L.b]));
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const int e = Lat::e(L.iq, c);
      if (e > 0) acc[c] = dd_add(acc[c], v);
      else if (e < 0) acc[c] = dd_add(acc[c], -v);
    }
  }
  block_dd_reduce<DIM>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < DIM; ++c) out[c] = __dadd_rn(acc[c].hi, acc[c].lo);
  }
}

constexpr int kMassBlock = 256;

template <int DIM, class T>
__global__ void __launch_bounds__(kMassBlock) k_mass_partial(DevGrid g, DevState st,
                                                              const T* __restrict__ fin,
                                                              double* partials) {
  using Lat = Lattice<DIM>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kMassBlock + threadIdx.x;
  DD acc{0.0, 0.0};
  if (id < g.id_hi && (st.mask[id] & kMaskFluid)) {
    sfor<0, Lat::Q>([&](auto I) {
      acc = dd_add(acc, Store<T>::to_d(fin[(int64_t)I * g.N + id - g.off[I]]));
    });
  }
  // fixed-shape block tree
  __shared__ DD sh[kMassBlock];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int stride = kMassBlock / 2; stride > 0; stride >>= 1) {
    if (threadIdx.x < stride) sh[threadIdx.x] = dd_add(sh[threadIdx.x], sh[threadIdx.x + stride]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sh[0].hi;
    partials[2 * blockIdx.x + 1] = sh[0].lo;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_mass_final(const double* __restrict__ partials,
                                                             int64_t nb, double* out) {
  __shared__ DD sh[kRedThreads][1];
  DD acc[1] = {DD{0.0, 0.0}};
  for (int64_t i = threadIdx.x; i < nb; i += kRedThreads)
    acc[0] = dd_add(acc[0], DD{partials[2 * i], partials[2 * i + 1]});
  block_dd_reduce<1>(acc, sh);
  if (threadIdx.x == 0) out[0] = __dadd_rn(acc[0].hi, acc[0].lo);
}

constexpr int kTile = 32;  // cells per transpose tile

template <class T>
__global__ void k_aos_to_soa(const double* __restrict__ aos, T* __restrict__ soa, int64_t N,
                             int K) {
  extern __shared__ double tile[];
  const int64_t c0 = (int64_t)blockIdx.x * kTile;
  const int ncell = (int)((N - c0) < kTile ? (N - c0) : kTile);
  for (int j = threadIdx.x; j < ncell * K; j += blockDim.x) tile[j] = aos[c0 * K + j];
  __syncthreads();
  for (int j = threadIdx.x; j < ncell * K; j += blockDim.x) {
    const int k = j / ncell, c = j - k * ncell;
    soa[(int64_t)k * N + c0 + c] = Store<T>::from_d(tile[c * K + k]);
  }
}

template <class T>
__global__ void k_soa_to_aos(const T* __restrict__ soa, double* __restrict__ aos, int64_t N,
                             int K) {
  extern __shared__ double tile[];
  const int64_t c0 = (int64_t)blockIdx.x * kTile;
  const int ncell = (int)((N - c0) < kTile ? (N - c0) : kTile);
  for (int j = threadIdx.x; j < ncell * K; j += blockDim.x) {
    const int k = j / ncell, c = j - k * ncell;
    tile[c * K + k] = Store<T>::to_d(soa[(int64_t)k * N + c0 + c]);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < ncell * K; j += blockDim.x) aos[c0 * K + j] = tile[j];
}

inline unsigned grid_for(const DevGrid& g) {
  return (unsigned)((g.id_hi - g.id_lo + kBlock - 1) / kBlock);
}

}  // namespace

cudaError_t launch_collide_fpu(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                               const DevState& st, const double* f, const double* p,
                               const double* u, double* fout, unsigned long long* monitor,
                               cudaStream_t s) {
  const unsigned grid = grid_for(g);
  const bool mon = monitor != nullptr;
#define L_(D, R, M) k_collide_fpu<D, R, M><<<grid, kBlock, 0, s>>>(g, c, st, f, p, u, fout, monitor)
  if (dim == 2) {
    if (rho_one) { if (mon) L_(2, true, true); else L_(2, true, false); }
    else { if (mon) L_(2, false, true); else L_(2, false, false); }
  } else {
    if (rho_one) { if (mon) L_(3, true, true); else L_(3, true, false); }
    else { if (mon) L_(3, false, true); else L_(3, false, false); }
  }
#undef L_
  return cudaGetLastError();
}

// FP64 fused multiply-add throughput: eight independent chains per thread
// (x = x*y + z with y < 1, so the values stay bounded); the result is kept
// live through one conditional store.
__global__ void __launch_bounds__(256) k_dfma_rate(double* out, double y, double z, int iters) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = (double)(threadIdx.x + j);
#pragma unroll 1
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], y, z);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  if (s == -1.0) out[0] = s;
}

int step_splits() { return Splits<3>::n; }
int step_split_default(int dim) { return dim == 2 ? Splits<2>::kDefault : Splits<3>::kDefault; }

cudaError_t launch_step(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                        const DevState& st, const double* fin, double* fout,
                        unsigned long long* monitor, cudaStream_t s, int split) {
  const unsigned grid = grid_for(g);
  const bool mon = monitor != nullptr;
  if (split < 0 || split >= step_splits()) return cudaErrorInvalidValue;
  if (st.bnd) {  // boundary copies folded in: the default variant only
    if (rho_one && split != step_split_default(dim)) return cudaErrorInvalidValue;
    return launch_step_fused(dim, rho_one, grid, g, c, st, fin, fout, monitor, s);
  }
  if (rho_one) {
    return dim == 2 ? launch_step_split2(split, grid, g, c, st, fin, fout, monitor, s)
                    : launch_step_split3(split, grid, g, c, st, fin, fout, monitor, s);
  }
#define L_(D, M) k_step<D, false, M><<<grid, kBlock, 0, s>>>(g, c, st, fin, fout, monitor)
  if (dim == 2) { if (mon) L_(2, true); else L_(2, false); }
  else { if (mon) L_(3, true); else L_(3, false); }
#undef L_
  return cudaGetLastError();
}

namespace {

__global__ void k_fill_group(const DevGroupFill* __restrict__ fill, int64_t n,
                             double* const* __restrict__ bufs, int out_parity) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const DevGroupFill e = fill[i];
    double v;
    if (e.src_code < 0) {
      v = __longlong_as_double(0x7ff8000000000000ll);
    } else {
      const int r = e.src_code & 0xffff;
      const int k = (e.src_code & kGroupPrev) ? 1 - out_parity : out_parity;
      v = bufs[2 * r + k][e.src];
    }
    bufs[2 * e.dst_rank + out_parity][e.dst] = v;
  }
}

}  // namespace

namespace {

// The arithmetic of the reference's InitUP in its order:
// ((((uu*4)*y)*(n-y))/n**2)*geo*r, r = 1 + ((r_vec - 0.5)*2)*0.2.
template <int DIM>
__global__ void k_init_up(DevGrid g, const uint8_t* __restrict__ mask, RVec rv, double uu, int n,
                          int start, double* __restrict__ u) {
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= g.id_hi || !(mask[id] & kMaskFluid)) return;
  const int64_t row = DIM == 2 ? id / g.dy : id / g.dz;
  const double y = (double)(row - kGhost + start);
  const double r = __dadd_rn(1.0, __dmul_rn(__dmul_rn(__dsub_rn(rv.v[id % 100], 0.5), 2.0), 0.2));
  double v = __dmul_rn(__dmul_rn(uu, 4.0), y);
  v = __dmul_rn(v, __dsub_rn((double)n, y));
  v = __ddiv_rn(v, (double)(n * n));
  u[id] = __dmul_rn(__dmul_rn(v, 1.0), r);  // *geo(id) = *1 on fluid nodes, then *r
}

}  // namespace

cudaError_t launch_init_up(int dim, const DevGrid& g, const uint8_t* mask, const RVec& rv,
                           double uu, int n, int start, double* u, cudaStream_t s) {
  const int64_t cells = g.id_hi - g.id_lo;
  if (cells <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((cells + 255) / 256);
  if (dim == 2) k_init_up<2><<<grid, 256, 0, s>>>(g, mask, rv, uu, n, start, u);
  else k_init_up<3><<<grid, 256, 0, s>>>(g, mask, rv, uu, n, start, u);
  return cudaGetLastError();
}

cudaError_t launch_fill_group(const DevGroupFill* fill, int64_t n, double* const* bufs,
                              int out_parity, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  k_fill_group<<<(unsigned)blocks, 256, 0, s>>>(fill, n, bufs, out_parity);
  return cudaGetLastError();
}

cudaError_t launch_fill(int store, const void* fill, bool narrow, int64_t n, void* fout,
                        const void* fin, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    if (narrow)
      k_fill<T, DevFill32><<<(unsigned)blocks, 256, 0, s>>>((const DevFill32*)fill, n, (T*)fout,
                                                          (const T*)fin);
    else
      k_fill<T, DevFill><<<(unsigned)blocks, 256, 0, s>>>((const DevFill*)fill, n, (T*)fout,
                                                        (const T*)fin);
    return cudaGetLastError();
  });
}

cudaError_t launch_finalize(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                            const DevState& st, const double* fin, double* f, double* p,
                            double* u, cudaStream_t s) {
  const unsigned grid = grid_for(g);
#define L_(D, R) k_finalize<D, R><<<grid, kBlock, 0, s>>>(g, c, st, fin, f, p, u)
  if (dim == 2) { if (rho_one) L_(2, true); else L_(2, false); }
  else { if (rho_one) L_(3, true); else L_(3, false); }
#undef L_
  return cudaGetLastError();
}

cudaError_t launch_columns(int dim, const DevGrid& g, const int* bl, int nl, const int* br,
                           int nr, const double* inlet, double* p, double* u, cudaStream_t s) {
  const int n = nl > nr ? nl : nr;
  if (n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (dim == 2) k_columns<2><<<grid, 256, 0, s>>>(g, bl, nl, br, nr, inlet, p, u);
  else k_columns<3><<<grid, 256, 0, s>>>(g, bl, nl, br, nr, inlet, p, u);
  return cudaGetLastError();
}

cudaError_t launch_init_pdf(int dim, bool rho_one, const DevGrid& g, const DevCoef& c,
                            const DevState& st, const double* p, const double* u, double* f,
                            cudaStream_t s) {
  const unsigned grid = grid_for(g);
#define L_(D, R) k_init_pdf<D, R><<<grid, kBlock, 0, s>>>(g, c, st, p, u, f)
  if (dim == 2) { if (rho_one) L_(2, true); else L_(2, false); }
  else { if (rho_one) L_(3, true); else L_(3, false); }
#undef L_
  return cudaGetLastError();
}

cudaError_t launch_forces(int dim, int store, const DevLink* links, int64_t n, const void* fb,
                          double* out, cudaStream_t s) {
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    if (dim == 2) k_forces<2, T><<<1, kRedThreads, 0, s>>>(links, n, (const T*)fb, out);
    else k_forces<3, T><<<1, kRedThreads, 0, s>>>(links, n, (const T*)fb, out);
    return cudaGetLastError();
  });
}

int64_t mass_partials_size(const DevGrid& g) {
  return 2 * ((g.id_hi - g.id_lo + kMassBlock - 1) / kMassBlock);
}

cudaError_t launch_mass(int dim, int store, const DevGrid& g, const DevState& st, const void* fin,
                        double* partials, double* out, cudaStream_t s) {
  const int64_t nb = (g.id_hi - g.id_lo + kMassBlock - 1) / kMassBlock;
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    if (dim == 2) k_mass_partial<2, T><<<(unsigned)nb, kMassBlock, 0, s>>>(g, st, (const T*)fin, partials);
    else k_mass_partial<3, T><<<(unsigned)nb, kMassBlock, 0, s>>>(g, st, (const T*)fin, partials);
    k_mass_final<<<1, kRedThreads, 0, s>>>(partials, nb, out);
    return cudaGetLastError();
  });
}

cudaError_t launch_aos_to_soa(int store, const double* aos, void* soa, int64_t N, int K,
                              cudaStream_t s) {
  const unsigned grid = (unsigned)((N + kTile - 1) / kTile);
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    k_aos_to_soa<T><<<grid, 256, sizeof(double) * kTile * K, s>>>(aos, (T*)soa, N, K);
    return cudaGetLastError();
  });
}

cudaError_t launch_soa_to_aos(int store, const void* soa, double* aos, int64_t N, int K,
                              cudaStream_t s) {
  const unsigned grid = (unsigned)((N + kTile - 1) / kTile);
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    k_soa_to_aos<T><<<grid, 256, sizeof(double) * kTile * K, s>>>((const T*)soa, aos, N, K);
    return cudaGetLastError();
  });
}

cudaError_t measure_dfma_rate(double* fma_per_s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  double* out = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  e = cudaMalloc((void**)&out, sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const unsigned grid = (unsigned)sms * 16;
  const int iters = 2048;
  if (e == cudaSuccess) {
    k_dfma_rate<<<grid, 256>>>(out, 0.999999, 1e-3, 64);  // warm-up
    cudaEventRecord(a);
    k_dfma_rate<<<grid, 256>>>(out, 0.999999, 1e-3, iters);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
  }
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && ms > 0.f) *fma_per_s = (double)grid * 256.0 * 8.0 * iters / (ms * 1e-3);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (out) cudaFree(out);
  return e;
}

}  // namespace imx
