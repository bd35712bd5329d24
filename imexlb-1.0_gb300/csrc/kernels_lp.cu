// Reduced-precision LBM kernels: populations stored as FP32, BF16 or FP16,
// collision arithmetic in FP32 (fused multiply-adds allowed); with double
// storage and double arithmetic the same kernels are the fast FP64 option
// (minimal operation count, not the reference's rounding).
//
// The stored value is the reference's own f, which is already the deviation
// f_i - t_i*rho0 from the rest state (its equilibrium has no t*rho0 term,
// lbm.f90:44), so narrow storage keeps full relative precision near rest.
// Same algorithm and boundary handling as the FP64 kernels (kernels.cu);
// these are HBM-bound: 2*Q*sizeof(T) bytes per node update.
#include <cstdint>
#include <utility>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "boundary_fused.cuh"
#include "kernels.h"
#include "lattice.h"
#include "node_fast.cuh"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kBlockLP = 256;

// Max over the block of non-negative values (their bit patterns order like
// the values), one atomicMax per block.
__device__ IMX_FI void block_max_lp(double v, unsigned long long* dst) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  __shared__ unsigned long long wmax[kBlockLP / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wmax[w] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = wmax[0];
    for (int i = 1; i < kBlockLP / 32; ++i) m = wmax[i] > m ? wmax[i] : m;
    atomicMax(dst, m);
  }
}

template <class T, class R>
__device__ IMX_FI R load_as(const T* p) {
  if constexpr (sizeof(R) == 8) return Store<T>::to_d(*p);
  else return Store<T>::to_f(*p);
}

template <class T, class R>
__device__ IMX_FI T store_as(R v) {
  if constexpr (sizeof(R) == 8) return Store<T>::from_d(v);
  else return Store<T>::from_f(v);
}

// Resident blocks per SM the step kernel is compiled for. The 2-byte kinds
// are latency-bound (few bytes per load): capping registers at 40 gives six
// 256-thread blocks per SM instead of five, 5% faster on D3Q27 (measured on
// 256x128x128: 0.117 vs 0.123 ms); FP32 and FP64 gain nothing from it. 0 = no
// minimum.
template <int DIM, class T>
constexpr int lp_min_blocks() {
  return DIM == 3 ? (sizeof(T) == 2 ? 6 : (sizeof(T) == 4 ? 5 : 0)) : 0;
}

template <int DIM, class T, class R, bool MON>
__global__ void __launch_bounds__(kBlockLP, lp_min_blocks<DIM, T>()) k_step_lp(DevGrid g, CoefR<R> c, DevState st,
                                                       DevPlanes pl,
                                                       unsigned long long* monitor) {
  using N_ = NodeFast<DIM, R>;
  using L = Lattice<DIM>;
  constexpr int Q = N_::Q;
  // 32-bit node index: every plane pointer already carries its direction's offset
  const uint32_t id = (uint32_t)(g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x);
  double um = 0.0;  // R-precision |u| (exact in double)
  const uint8_t m = (int64_t)id < g.id_hi ? st.mask[id] : (uint8_t)0;
  const PullFix fx = PullFix::make(st, (m & kMaskFluid) ? m : (uint8_t)0);
  // warps with a node on a wall or periodic face or with a record take the
  // general pull; the inlet / outlet forms cost every node one add per
  // e_x = -1 direction
  const bool bwarp = __any_sync(0xffffffffu, fx.other());
  if (m & kMaskFluid) {
    R f[Q];
    // plane 0 of each buffer starts at its base (the input plane pointer
    // carries the pull shift -off[0])
    const T* fin = (const T*)pl.in[0] + g.off[0];
    T* fout = (T*)pl.out[0];
    if (!bwarp) {
      const uint32_t id_in = id + fx.inl(), o = fx.outl();
      sfor<0, Q>([&](auto I) {
        constexpr int ex = L::ex(I);
        const uint32_t a = ex == 1 ? id_in : (ex == -1 ? id + o * (uint32_t)g.off[I] : id);
        f[I] = load_as<T, R>((const T*)pl.in[I] + a);
      });
    } else if (!fx.record()) {
      sfor<0, Q>([&](auto I) {
        constexpr int i = I;
        bool opp;
        int64_t sh;
        fx.form<DIM>(L::ex(i), L::ey(i), L::ez(i), g.off[i], st.pshift, opp, sh);
        const T* base = (const T*)(opp ? pl.in[Q - 1 - i] : pl.in[i]);
        f[I] = load_as<T, R>(base + (uint32_t)(id + (uint32_t)sh));
      });
    } else {
      const uint32_t* row = PullFix::row<Q>(st, id);
      sfor<0, Q>([&](auto I) {
        const uint32_t r = row[I];
        f[I] = load_as<T, R>(r != kNoRedirect ? fin + r : (const T*)pl.in[I] + id);
      });
    }
    R u[DIM];
    R S3 = N_::moments(f, u, c.inv_rho0);
    N_::dirichlet(m, id, g, st.inlet, S3, u);
    if constexpr (MON) {
      if (id != g.skip_id) um = (double)sqrt(u[0] * u[0] + u[1] * u[1]);
    }
    N_::collide(f, S3, u, c, [&](int i, R v) { ((T*)pl.out[i])[id] = store_as<T, R>(v); });
    if (fx.record()) push_copies(st.push, PullFix::row<Q>(st, id)[Q], fin, fout);
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

template <int DIM, class T, class R, bool MON>
__global__ void __launch_bounds__(kBlockLP) k_collide_fpu_lp(DevGrid g, CoefR<R> c, DevState st,
                                                              const double* __restrict__ fs,
                                                              const double* __restrict__ ps,
                                                              const double* __restrict__ us,
                                                              T* __restrict__ fout,
                                                              unsigned long long* monitor) {
  using N_ = NodeFast<DIM, R>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  double um = 0.0;  // R-precision |u| (exact in double)
  if (id < g.id_hi) {
    const uint8_t m = st.mask[id];
    if (m & kMaskFluid) {
      R f[N_::Q];
      sfor<0, N_::Q>([&](auto I) { f[I] = (R)fs[(int64_t)I * g.N + id]; });
      R u[DIM];
      sfor<0, DIM>([&](auto K) { u[K] = (R)us[(int64_t)K * g.N + id]; });
      const R S3 = R(3) * (R)ps[id];
      if constexpr (MON) {
        if (id != g.skip_id) um = (double)sqrt(u[0] * u[0] + u[1] * u[1]);
      }
      N_::collide(f, S3, u, c, [&](int i, R v) { fout[(int64_t)i * g.N + id] = store_as<T, R>(v); });
    }
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

template <int DIM, class T, class R>
__global__ void __launch_bounds__(kBlockLP) k_finalize_lp(DevGrid g, CoefR<R> c, DevState st,
                                                           const T* __restrict__ fin,
                                                           double* __restrict__ fs,
                                                           double* __restrict__ ps,
                                                           double* __restrict__ us) {
  using N_ = NodeFast<DIM, R>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  if (id >= g.id_hi) return;
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) return;
  R f[N_::Q];
  sfor<0, N_::Q>([&](auto I) { f[I] = load_as<T, R>(fin + (int64_t)I * g.N + id - g.off[I]); });
  R u[DIM];
  R S3 = N_::moments(f, u, c.inv_rho0);
  N_::dirichlet(m, id, g, st.inlet, S3, u);
  sfor<0, N_::Q>([&](auto I) { fs[(int64_t)I * g.N + id] = (double)f[I]; });
  sfor<0, DIM>([&](auto K) { us[(int64_t)K * g.N + id] = (double)u[K]; });
  ps[id] = (double)(S3 / R(3));
}

// Node value (fluid indicator, p, ux, uy) of a 2D node at (x, y).
template <class T>
__device__ IMX_FI void node_fields(const DevGrid& g, const CoefR<float>& c, const DevState& st,
                                   const T* __restrict__ fin, int x, int y, float (&v)[4]) {
  const int64_t id = (x + kGhost) + g.dy * (y + kGhost);
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) {
    v[0] = v[1] = v[2] = v[3] = 0.0f;
    return;
  }
  using N_ = NodeFast<2, float>;
  float f[9];
  sfor<0, 9>([&](auto I) { f[I] = Store<T>::to_f(fin[(int64_t)I * g.N + id - g.off[I]]); });
  float u[2];
  float S3 = N_::moments(f, u, c.inv_rho0);
  N_::dirichlet(m, id, g, st.inlet, S3, u);
  v[0] = 1.0f;
  v[1] = S3 * (1.0f / 3.0f);
  v[2] = u[0];
  v[3] = u[1];
}

template <class T>
__global__ void k_sample(DevGrid g, CoefR<float> c, DevState st, int L0, int L1,
                         const T* __restrict__ fin, int W, int H, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= W || j >= H) return;
  float X = (i + 0.5f) * (float)L0 / (float)W - 0.5f;
  float Y = (j + 0.5f) * (float)L1 / (float)H - 0.5f;
  X = fminf(fmaxf(X, 0.0f), (float)(L0 - 1));
  Y = fminf(fmaxf(Y, 0.0f), (float)(L1 - 1));
  const int x0 = min((int)X, L0 - 2 < 0 ? 0 : L0 - 2), y0 = min((int)Y, L1 - 2 < 0 ? 0 : L1 - 2);
  const float fx = X - x0, fy = Y - y0;
  float a[4], b[4], cc[4], d[4];
  node_fields(g, c, st, fin, x0, y0, a);
  node_fields(g, c, st, fin, x0 + 1, y0, b);
  node_fields(g, c, st, fin, x0, y0 + 1, cc);
  node_fields(g, c, st, fin, x0 + 1, y0 + 1, d);
  const int64_t plane = (int64_t)W * H, o = (int64_t)j * W + i;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    out[k * plane + o] = (1 - fy) * ((1 - fx) * a[k] + fx * b[k]) + fy * ((1 - fx) * cc[k] + fx * d[k]);
}

inline unsigned grid_lp(const DevGrid& g) {
  return (unsigned)((g.id_hi - g.id_lo + kBlockLP - 1) / kBlockLP);
}

// fn(T{}, R{}) for the storage kind: narrow kinds compute in float, double
// storage (the fast FP64 option) in double.
template <class F>
cudaError_t dispatch_lp(int store, F&& fn) {
  switch (store) {
    case kStoreF32: return fn(float{}, float{});
    case kStoreBF16: return fn(__nv_bfloat16{}, float{});
    case kStoreF16: return fn(__half{}, float{});
    case kStoreF64: return fn(double{}, double{});
    default: return cudaErrorInvalidValue;
  }
}

// dispatch_lp for the kernels outside the step (first collision after an
// upload, finalize on download), which also serve the fixed-point kind with
// double arithmetic; its step kernel is kernels_fx.cu's.
template <class F>
cudaError_t dispatch_lp_aux(int store, F&& fn) {
  if (store == kStoreFix) return fn(Fix64{}, double{});
  return dispatch_lp(store, std::forward<F>(fn));
}

}  // namespace

cudaError_t launch_collide_fpu_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                                  const DevState& st, const double* f, const double* p,
                                  const double* u, void* fout, unsigned long long* monitor,
                                  cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp_aux(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    T* o = (T*)fout;
    if (dim == 2) {
      if (monitor) k_collide_fpu_lp<2, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<2, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
    } else {
      if (monitor) k_collide_fpu_lp<3, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<3, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_step_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                           const DevState& st, const DevPlanes& pl, unsigned long long* monitor,
                           cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    if (dim == 2) {
      if (monitor) k_step_lp<2, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
      else k_step_lp<2, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
    } else {
      if (monitor) k_step_lp<3, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
      else k_step_lp<3, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_finalize_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                               const DevState& st, const void* fin, double* f, double* p,
                               double* u, cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp_aux(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    if (dim == 2) k_finalize_lp<2, T, R><<<grid, kBlockLP, 0, s>>>(g, cr, st, (const T*)fin, f, p, u);
    else k_finalize_lp<3, T, R><<<grid, kBlockLP, 0, s>>>(g, cr, st, (const T*)fin, f, p, u);
    return cudaGetLastError();
  });
}

cudaError_t launch_sample(int store, const DevGrid& g, const DevCoefLP& c, const DevState& st,
                          int L0, int L1, const void* fin, int W, int H, float* out,
                          cudaStream_t s) {
  const dim3 grid((unsigned)((W + 127) / 128), (unsigned)H);
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    k_sample<T><<<grid, 128, 0, s>>>(g, c.f, st, L0, L1, (const T*)fin, W, H, out);
    return cudaGetLastError();
  });
}

DevPlanes make_planes(const DevGrid& g, int nq, size_t esz, const void* fin, void* fout) {
  DevPlanes pl{};
  for (int i = 0; i < nq; ++i) {
    pl.in[i] = (const char*)fin + ((int64_t)i * g.N - g.off[i]) * (int64_t)esz;
    pl.out[i] = (char*)fout + (int64_t)i * g.N * (int64_t)esz;
  }
  return pl;
}

}  // namespace imx
