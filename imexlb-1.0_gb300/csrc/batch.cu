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
#include "node_fast.cuh"
#include "storage.cuh"

namespace imx {
namespace {

template <int DIM, class T>
__device__ IMX_FI void update_node(const BatchCase& cs, int64_t id, const T* __restrict__ fin,
                                   T* __restrict__ fout) {
  using N_ = NodeFast<DIM, float>;
  if (id >= cs.g.id_hi) return;
  const uint8_t m = cs.mask[id];
  if (!(m & kMaskFluid)) return;
  float f[N_::Q];
  sfor<0, N_::Q>([&](auto I) {
    f[I] = Store<T>::to_f(fin[(int64_t)I * cs.g.N + id - cs.g.off[I]]);
  });
  float u[DIM];
  float S3 = N_::moments(f, u, cs.c.inv_rho0);
  N_::dirichlet(m, id, cs.g, cs.inlet, S3, u);
  N_::collide(f, S3, u, cs.c, [&](int i, float v) {
    fout[(int64_t)i * cs.g.N + id] = Store<T>::from_f(v);
  });
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
