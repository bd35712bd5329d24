// Lockstep stepping of many independent cases (an ensemble of lattices) with
// one launch per iteration for the collide kernel and one for the boundary
// refresh. Each case keeps its own geometry, buffers and boundary fill list;
// a block -> case table maps the launch onto them, and a device counter
// (advanced by a one-thread kernel after every iteration) lets a captured CUDA
// graph replay iterations while cases with a smaller budget drop out.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "batch.h"
#include "lattice.h"
#include "storage.cuh"

namespace imx {
namespace {

// FP32 node arithmetic shared with kernels_lp.cu (same formulas).
template <int DIM>
struct NodeB {
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

  template <class T>
  __device__ static IMX_FI void collide(const float (&f)[Q], float p, const float (&u)[DIM],
                                        const DevCoefF& c, T* __restrict__ out, int64_t N,
                                        int64_t id) {
    float uu = u[0] * u[0] + u[1] * u[1];
    if constexpr (DIM == 3) uu += u[2] * u[2];
    const float p3 = 3.0f * p, h = 1.5f * uu;
    auto put = [&](int i, float fe) {
      out[(int64_t)i * N + id] = Store<T>::from_f(c.om1 * f[i] + c.ome * fe);
    };
    put(Lat::REST, c.t[Lat::REST] * (p3 - c.rho0 * h));
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        const float e = edu<i>(u);
        const float a = 3.0f * e;
        const float q = 4.5f * e * e - h;
        put(i, c.t[i] * (p3 + c.rho0 * (q + a)));
        put(o, c.t[o] * (p3 + c.rho0 * (q - a)));
      }
    });
  }
};

template <int DIM, class T>
__device__ IMX_FI void update_node(const BatchCase& cs, int64_t id, const T* __restrict__ fin,
                                   T* __restrict__ fout) {
  using N_ = NodeB<DIM>;
  if (id >= cs.g.id_hi) return;
  const uint8_t m = cs.mask[id];
  if (!(m & kMaskFluid)) return;
  float f[N_::Q];
  sfor<0, N_::Q>([&](auto I) {
    f[I] = Store<T>::to_f(fin[(int64_t)I * cs.g.N + id - cs.g.off[I]]);
  });
  float p, u[DIM];
  N_::moments(f, p, u, cs.c);
  if (m & kMaskInlet) {
    const int64_t r = DIM == 2 ? id / cs.g.dy : id / cs.g.dz;
    u[0] = (float)cs.inlet[r];
    u[1] = 0.0f;
  }
  if (m & kMaskOutlet) p = 0.0f;
  N_::collide(f, p, u, cs.c, fout, cs.g.N, id);
}

// One iteration for every active case: block b serves case block_case[b],
// tile (b - cs.block0) of BLOCK*CPT cells.
template <int DIM, class T, int BLOCK, int CPT>
__global__ void __launch_bounds__(BLOCK) k_step_batch(const BatchCase* __restrict__ cases,
                                                       const uint16_t* __restrict__ block_case,
                                                       const int* __restrict__ counter) {
  const BatchCase& cs = cases[block_case[blockIdx.x]];
  const int it = *counter;
  if (it >= cs.nsteps) return;
  const int par = (cs.parity0 + it) & 1;
  const T* fin = (const T*)cs.fb[par];
  T* fout = (T*)cs.fb[1 - par];
  const int64_t base = cs.g.id_lo + (int64_t)(blockIdx.x - cs.block0) * (BLOCK * CPT);
#pragma unroll
  for (int k = 0; k < CPT; ++k) update_node<DIM, T>(cs, base + k * BLOCK + threadIdx.x, fin, fout);
}

// Boundary refresh for every active case: block b serves case fill_case[b],
// entries (b - cs.fill_block0) * 256 + [0, 256) of its fill list.
template <class T>
__global__ void __launch_bounds__(256) k_fill_batch(const BatchCase* __restrict__ cases,
                                                     const uint16_t* __restrict__ fill_case,
                                                     const int* __restrict__ counter) {
  const BatchCase& cs = cases[fill_case[blockIdx.x]];
  const int it = *counter;
  if (it >= cs.nsteps) return;
  const int par = (cs.parity0 + it) & 1;
  const T* fin = (const T*)cs.fb[par];
  T* fout = (T*)cs.fb[1 - par];
  const int64_t i = (int64_t)(blockIdx.x - cs.fill_block0) * 256 + threadIdx.x;
  if (i >= cs.n_fill) return;
  int64_t dst, src;
  if (cs.fill_narrow) {
    const DevFill32 e = ((const DevFill32*)cs.fill)[i];
    dst = e.dst;
    src = e.src == kFillNaN32 ? kFillNaN : (int64_t)e.src;
  } else {
    const DevFill e = ((const DevFill*)cs.fill)[i];
    dst = e.dst;
    src = e.src;
  }
  T v;
  if (src >= 0) v = fout[src];
  else if (src != kFillNaN) v = fin[~src];
  else v = Store<T>::nan();
  fout[dst] = v;
}

__global__ void k_tick(int* counter) { *counter += 1; }

template <class F>
cudaError_t dispatch_lp_b(int store, F&& fn) {
  switch (store) {
    case kStoreF32: return fn(float{});
    case kStoreBF16: return fn(__nv_bfloat16{});
    case kStoreF16: return fn(__half{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

const BatchShape kBatchShapes[kNumBatchShapes] = {
    {128, 1}, {256, 1}, {512, 1}, {128, 2}, {256, 2}, {128, 4}};

cudaError_t launch_batch_iteration(int dim, int store, int shape, const BatchCase* cases,
                                   const uint16_t* block_case, int64_t nblocks,
                                   const uint16_t* fill_case, int64_t nfill_blocks, int* counter,
                                   cudaStream_t s) {
  const BatchShape sh = kBatchShapes[shape];
  cudaError_t e = dispatch_lp_b(store, [&](auto tag) {
    using T = decltype(tag);
#define L_(D, B, C) k_step_batch<D, T, B, C><<<(unsigned)nblocks, B, 0, s>>>(cases, block_case, counter)
    if (dim == 2) {
      if (sh.block == 128 && sh.cpt == 1) L_(2, 128, 1);
      else if (sh.block == 256 && sh.cpt == 1) L_(2, 256, 1);
      else if (sh.block == 512 && sh.cpt == 1) L_(2, 512, 1);
      else if (sh.block == 128 && sh.cpt == 2) L_(2, 128, 2);
      else if (sh.block == 256 && sh.cpt == 2) L_(2, 256, 2);
      else L_(2, 128, 4);
    } else {
      if (sh.block == 128 && sh.cpt == 1) L_(3, 128, 1);
      else if (sh.block == 256 && sh.cpt == 1) L_(3, 256, 1);
      else if (sh.block == 512 && sh.cpt == 1) L_(3, 512, 1);
      else if (sh.block == 128 && sh.cpt == 2) L_(3, 128, 2);
      else if (sh.block == 256 && sh.cpt == 2) L_(3, 256, 2);
      else L_(3, 128, 4);
    }
#undef L_
    const cudaError_t e1 = cudaGetLastError();
    if (e1 != cudaSuccess) return e1;
    if (nfill_blocks > 0)
      k_fill_batch<T><<<(unsigned)nfill_blocks, 256, 0, s>>>(cases, fill_case, counter);
    return cudaGetLastError();
  });
  if (e != cudaSuccess) return e;
  k_tick<<<1, 1, 0, s>>>(counter);
  return cudaGetLastError();
}

}  // namespace imx
