// Reduced-precision LBM kernels: populations stored as FP32, BF16 or FP16,
// collision arithmetic in FP32 (fused multiply-adds allowed).
//
// The stored value is the reference's own f, which is already the deviation
// f_i - t_i*rho0 from the rest state (its equilibrium has no t*rho0 term,
// lbm.f90:44), so narrow storage keeps full relative precision near rest.
// Same algorithm and boundary handling as the FP64 kernels (kernels.cu);
// these are HBM-bound: 2*Q*sizeof(T) bytes per node update.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "kernels.h"
#include "lattice.h"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kBlockLP = 256;

template <int DIM>
struct NodeF {
  using Lat = Lattice<DIM>;
  static constexpr int Q = Lat::Q;

  __device__ static IMX_FI void moments(const float (&f)[Q], float& p, float (&u)[DIM],
                                        const DevCoefF& c) {
    float s = f[0];
    sfor<1, Q>([&](auto I) { s += f[I]; });
    p = s * (1.0f / 3.0f);
    sfor<0, DIM>([&](auto K) {
      constexpr int k = K;
      constexpr int i0 = Lat::first_nz(k);
      float m = Lat::e(i0, k) > 0 ? f[i0] : -f[i0];
      sfor<i0 + 1, Q>([&](auto I) {
        constexpr int cc = Lat::e(I, k);
        if constexpr (cc > 0) m += f[I];
        else if constexpr (cc < 0) m -= f[I];
      });
      u[k] = m * c.inv_rho0;
    });
  }

  template <int I>
  __device__ static IMX_FI float edu(const float (&u)[DIM]) {
    constexpr int k0 = Lat::first_comp(I);
    float s = u[k0];
    sfor<k0 + 1, DIM>([&](auto K) {
      constexpr int cc = Lat::e(I, K);
      if constexpr (cc > 0) s += u[K];
      else if constexpr (cc < 0) s -= u[K];
    });
    return s;
  }

  // fn(iq, feq) for every direction; feq = t*(3p + rho0*(3eu + 4.5eu^2 - 1.5uu))
  template <class F>
  __device__ static IMX_FI void equilibria(float p, const float (&u)[DIM], const DevCoefF& c,
                                           F&& fn) {
    float uu = u[0] * u[0] + u[1] * u[1];
    if constexpr (DIM == 3) uu += u[2] * u[2];
    const float p3 = 3.0f * p;
    const float h = 1.5f * uu;
    fn(Lat::REST, c.t[Lat::REST] * (p3 - c.rho0 * h));
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        const float e = edu<i>(u);
        const float a = 3.0f * e;
        const float q = 4.5f * e * e - h;
        fn(i, c.t[i] * (p3 + c.rho0 * (q + a)));
        fn(o, c.t[o] * (p3 + c.rho0 * (q - a)));
      }
    });
  }

  template <class T>
  __device__ static IMX_FI void collide(const float (&f)[Q], float p, const float (&u)[DIM],
                                        const DevCoefF& c, T* __restrict__ out, int64_t N,
                                        int64_t id) {
    equilibria(p, u, c, [&](int i, float fe) {
      out[(int64_t)i * N + id] = Store<T>::from_f(c.om1 * f[i] + c.ome * fe);
    });
  }

  template <class T>
  __device__ static IMX_FI void pull(const T* __restrict__ fin, const DevGrid& g, int64_t id,
                                     float (&f)[Q]) {
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      f[i] = Store<T>::to_f(fin[(int64_t)i * g.N + id - g.off[i]]);
    });
  }

  __device__ static IMX_FI void dirichlet(uint8_t m, int64_t id, const DevGrid& g,
                                          const double* inlet, float& p, float (&u)[DIM]) {
    if (m & kMaskInlet) {
      const int64_t r = DIM == 2 ? id / g.dy : id / g.dz;
      u[0] = (float)inlet[r];
      u[1] = 0.0f;
    }
    if (m & kMaskOutlet) p = 0.0f;
  }
};

__device__ IMX_FI void block_max_lp(float v, unsigned long long* dst) {
  unsigned long long b = (unsigned long long)__double_as_longlong((double)v);
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

template <int DIM, class T, bool MON>
__global__ void __launch_bounds__(kBlockLP) k_step_lp(DevGrid g, DevCoefF c, DevState st,
                                                       DevPlanes pl,
                                                       unsigned long long* monitor) {
  using N_ = NodeF<DIM>;
  constexpr int Q = N_::Q;
  // 32-bit node index: every plane pointer already carries its direction's offset
  const uint32_t id = (uint32_t)(g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x);
  float um = 0.0f;
  if ((int64_t)id < g.id_hi) {
    const uint8_t m = st.mask[id];
    if (m & kMaskFluid) {
      float f[Q];
      sfor<0, Q>([&](auto I) { f[I] = Store<T>::to_f(((const T*)pl.in[I])[id]); });
      float p, u[DIM];
      N_::moments(f, p, u, c);
      N_::dirichlet(m, id, g, st.inlet, p, u);
      if constexpr (MON) {
        if (id != g.skip_id) um = sqrtf(u[0] * u[0] + u[1] * u[1]);
      }
      N_::equilibria(p, u, c, [&](int i, float fe) {
        ((T*)pl.out[i])[id] = Store<T>::from_f(c.om1 * f[i] + c.ome * fe);
      });
    }
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

template <int DIM, class T, bool MON>
__global__ void __launch_bounds__(kBlockLP) k_collide_fpu_lp(DevGrid g, DevCoefF c, DevState st,
                                                              const double* __restrict__ fs,
                                                              const double* __restrict__ ps,
                                                              const double* __restrict__ us,
                                                              T* __restrict__ fout,
                                                              unsigned long long* monitor) {
  using N_ = NodeF<DIM>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  float um = 0.0f;
  if (id < g.id_hi) {
    const uint8_t m = st.mask[id];
    if (m & kMaskFluid) {
      float f[N_::Q];
      sfor<0, N_::Q>([&](auto I) { f[I] = (float)fs[(int64_t)I * g.N + id]; });
      float u[DIM];
      sfor<0, DIM>([&](auto K) { u[K] = (float)us[(int64_t)K * g.N + id]; });
      const float p = (float)ps[id];
      if constexpr (MON) {
        if (id != g.skip_id) um = sqrtf(u[0] * u[0] + u[1] * u[1]);
      }
      N_::collide(f, p, u, c, fout, g.N, id);
    }
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

template <int DIM, class T>
__global__ void __launch_bounds__(kBlockLP) k_finalize_lp(DevGrid g, DevCoefF c, DevState st,
                                                           const T* __restrict__ fin,
                                                           double* __restrict__ fs,
                                                           double* __restrict__ ps,
                                                           double* __restrict__ us) {
  using N_ = NodeF<DIM>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  if (id >= g.id_hi) return;
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) return;
  float f[N_::Q];
  N_::pull(fin, g, id, f);
  float p, u[DIM];
  N_::moments(f, p, u, c);
  N_::dirichlet(m, id, g, st.inlet, p, u);
  sfor<0, N_::Q>([&](auto I) { fs[(int64_t)I * g.N + id] = f[I]; });
  sfor<0, DIM>([&](auto K) { us[(int64_t)K * g.N + id] = u[K]; });
  ps[id] = p;
}

// Node value (fluid indicator, p, ux, uy) of a 2D node at (x, y).
template <class T>
__device__ IMX_FI void node_fields(const DevGrid& g, const DevCoefF& c, const DevState& st,
                                   const T* __restrict__ fin, int x, int y, float (&v)[4]) {
  const int64_t id = (x + kGhost) + g.dy * (y + kGhost);
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) {
    v[0] = v[1] = v[2] = v[3] = 0.0f;
    return;
  }
  using N_ = NodeF<2>;
  float f[9];
  sfor<0, 9>([&](auto I) { f[I] = Store<T>::to_f(fin[(int64_t)I * g.N + id - g.off[I]]); });
  float p, u[2];
  N_::moments(f, p, u, c);
  N_::dirichlet(m, id, g, st.inlet, p, u);
  v[0] = 1.0f;
  v[1] = p;
  v[2] = u[0];
  v[3] = u[1];
}

template <class T>
__global__ void k_sample(DevGrid g, DevCoefF c, DevState st, int L0, int L1,
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

template <class F>
cudaError_t dispatch_lp(int store, F&& fn) {
  switch (store) {
    case kStoreF32: return fn(float{});
    case kStoreBF16: return fn(__nv_bfloat16{});
    case kStoreF16: return fn(__half{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_collide_fpu_lp(int dim, int store, const DevGrid& g, const DevCoefF& c,
                                  const DevState& st, const double* f, const double* p,
                                  const double* u, void* fout, unsigned long long* monitor,
                                  cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp(store, [&](auto tag) {
    using T = decltype(tag);
    T* o = (T*)fout;
    if (dim == 2) {
      if (monitor) k_collide_fpu_lp<2, T, true><<<grid, kBlockLP, 0, s>>>(g, c, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<2, T, false><<<grid, kBlockLP, 0, s>>>(g, c, st, f, p, u, o, monitor);
    } else {
      if (monitor) k_collide_fpu_lp<3, T, true><<<grid, kBlockLP, 0, s>>>(g, c, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<3, T, false><<<grid, kBlockLP, 0, s>>>(g, c, st, f, p, u, o, monitor);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_sample(int store, const DevGrid& g, const DevCoefF& c, const DevState& st,
                          int L0, int L1, const void* fin, int W, int H, float* out,
                          cudaStream_t s) {
  const dim3 grid((unsigned)((W + 127) / 128), (unsigned)H);
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    k_sample<T><<<grid, 128, 0, s>>>(g, c, st, L0, L1, (const T*)fin, W, H, out);
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

cudaError_t launch_step_lp(int dim, int store, const DevGrid& g, const DevCoefF& c,
                           const DevState& st, const DevPlanes& pl, unsigned long long* monitor,
                           cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp(store, [&](auto tag) {
    using T = decltype(tag);
    if (dim == 2) {
      if (monitor) k_step_lp<2, T, true><<<grid, kBlockLP, 0, s>>>(g, c, st, pl, monitor);
      else k_step_lp<2, T, false><<<grid, kBlockLP, 0, s>>>(g, c, st, pl, monitor);
    } else {
      if (monitor) k_step_lp<3, T, true><<<grid, kBlockLP, 0, s>>>(g, c, st, pl, monitor);
      else k_step_lp<3, T, false><<<grid, kBlockLP, 0, s>>>(g, c, st, pl, monitor);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_finalize_lp(int dim, int store, const DevGrid& g, const DevCoefF& c,
                               const DevState& st, const void* fin, double* f, double* p,
                               double* u, cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp(store, [&](auto tag) {
    using T = decltype(tag);
    if (dim == 2) k_finalize_lp<2, T><<<grid, kBlockLP, 0, s>>>(g, c, st, (const T*)fin, f, p, u);
    else k_finalize_lp<3, T><<<grid, kBlockLP, 0, s>>>(g, c, st, (const T*)fin, f, p, u);
    return cudaGetLastError();
  });
}

}  // namespace imx
