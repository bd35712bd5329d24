// Persistent stepping of an ensemble: one cooperative launch advances every
// case of a batch through all the iterations of a call.
//
// Each case's iteration n is a set of work items: step tiles (the pull,
// moments, Dirichlet conditions and collision of lbm.f90:52-201 for
// kPersistTile consecutive cells) and then fill chunks (the case's resolved
// BoundaryCondition copies, lbm.f90:96-155). The items of the whole call are
// numbered iteration-major (for every n: the step tiles of the cases still
// running, then their fill chunks), and the resident blocks take them in that
// order from one atomic counter. An item waits only for items numbered
// before it:
//   step tile (c, n) needs every fill chunk of (c, n-1): its pulls read the
//     boundary slots, and it overwrites the buffer those chunks read;
//   fill chunk (c, n) needs every step tile of (c, n).
// The block that took the earliest unfinished item therefore never waits
// for an unfinished item, so the launch always progresses; every block is
// resident (a cooperative launch refuses a grid that does not fit).
//
// Every wait is bounded: a block polls its case's counter for at most
// budget_ns of the device's global timer, then records where it gave up in
// the status word and returns; the other blocks see the status and return
// too. The host reads the status after the launch.
//
// Populations written by other blocks of the same launch are read with
// L2-only loads (ld.global.cg): the L1 of an SM is not coherent with other
// SMs' stores.
#include <cstdint>
#include <type_traits>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "batch.h"
#include "lattice.h"
#include "node_fast.cuh"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kPB = 256;  // threads per block

template <class T>
__device__ __forceinline__ float ld_cg_f(const T* p) {
  if constexpr (sizeof(T) == 4) {
    return __ldcg((const float*)p);
  } else {
    const unsigned short b = __ldcg((const unsigned short*)p);
    if constexpr (std::is_same<T, __half>::value) return __half2float(__ushort_as_half(b));
    else return __bfloat162float(__ushort_as_bfloat16(b));
  }
}

template <class T>
__device__ __forceinline__ T ld_cg_raw(const T* p) {
  if constexpr (sizeof(T) == 4) {
    return __int_as_float(__ldcg((const int*)p));
  } else {
    const unsigned short b = __ldcg((const unsigned short*)p);
    if constexpr (std::is_same<T, __half>::value) return __ushort_as_half(b);
    else return __ushort_as_bfloat16(b);
  }
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_status(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Thread 0: wait until *ctr >= target. False when the budget ran out (the
// status then says where) or another block gave up.
__device__ bool wait_geq(const unsigned* ctr, unsigned target, const PersistSched& s, int c, int n,
                         int kind) {
  if (ld_acquire(ctr) >= target) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (ld_acquire(ctr) >= target) return true;
    if (ld_status(s.status) != 0) return false;
    if (global_ns() - t0 > s.budget_ns) {
      if (atomicCAS(s.status, 0, kPersistTimeout) == 0) {
        s.info[0] = c;
        s.info[1] = n;
        s.info[2] = kind;
      }
      return false;
    }
    __nanosleep(256);
  }
}

template <int DIM, class T>
__device__ __forceinline__ void step_node(const BatchCase& cs, int64_t id, const T* __restrict__ fin,
                                          T* __restrict__ fout) {
  using N_ = NodeFast<DIM, float>;
  if (id >= cs.g.id_hi) return;
  const uint8_t m = cs.mask[id];
  if (!(m & kMaskFluid)) return;
  float f[N_::Q];
  sfor<0, N_::Q>([&](auto I) { f[I] = ld_cg_f(fin + ((int64_t)I * cs.g.N + id - cs.g.off[I])); });
  float u[DIM];
  float S3 = N_::moments(f, u, cs.c.inv_rho0);
  N_::dirichlet(m, id, cs.g, cs.inlet, S3, u);
  N_::collide(f, S3, u, cs.c, [&](int i, float v) {
    fout[(int64_t)i * cs.g.N + id] = Store<T>::from_f(v);
  });
}

template <class T>
__device__ __forceinline__ void fill_entry(const BatchCase& cs, int64_t i, const T* fin, T* fout) {
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
  if (src >= 0) v = ld_cg_raw(fout + src);
  else if (src != kFillNaN) v = ld_cg_raw(fin + ~src);
  else v = Store<T>::nan();
  fout[dst] = v;
}

// Largest k in [0, n) with pre[k] <= x (pre ascending, pre[0] = 0).
__device__ __forceinline__ int upper_index(const long long* pre, int n, long long x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int DIM, class T, int CPT>
__global__ void __launch_bounds__(kPB) k_batch_persistent(PersistSched s) {
  // the case tables in shared memory: decoding an item is a binary search
  extern __shared__ long long sm_tab[];
  const int nc = s.ncases;
  long long* tpre = sm_tab;
  long long* fpre = sm_tab + nc + 1;
  int* ord = (int*)(sm_tab + 2 * (nc + 1));
  for (int i = threadIdx.x; i <= nc; i += kPB) {
    tpre[i] = s.tile_pre[i];
    fpre[i] = s.fill_pre[i];
    if (i < nc) ord[i] = s.order[i];
  }
  __shared__ long long s_item;
  __shared__ int s_go;
  if (threadIdx.x == 0) s_item = (long long)atomicAdd(s.next, 1ull);
  __syncthreads();
  int n = 0;  // iteration of the last item (a block's items come in increasing order)
  for (;;) {
    const long long item = s_item;
    if (item >= s.nitems) return;  // uniform: every thread read the same s_item
    while (__ldg(s.iter_start + n + 1) <= item) ++n;
    const int A = __ldg(s.active + n);  // cases still running at iteration n (a prefix of `ord`)
    const long long l = item - __ldg(s.iter_start + n);
    const long long nstep = tpre[A];
    const bool is_step = l < nstep;
    const long long x = is_step ? l : l - nstep;
    const int k = upper_index(is_step ? tpre : fpre, A + 1, x);
    const int c = ord[k];
    const BatchCase& cs = s.cases[c];
    const long long sub = x - (is_step ? tpre[k] : fpre[k]);
    const unsigned ntile = (unsigned)(tpre[k + 1] - tpre[k]);
    const unsigned nfill = (unsigned)(fpre[k + 1] - fpre[k]);
    long long next_item = 0;
    if (threadIdx.x == 0) {
      bool ok = ld_status(s.status) == 0;
      if (ok) {
        if (is_step) {
          unsigned target = (unsigned)n * nfill;
          if (c == s.stall_case && n > 0) target += 1u;  // testing: a count nothing reaches
          ok = wait_geq(s.done_fill + c, target, s, c, n, 0);
        } else {
          ok = wait_geq(s.done_step + c, (unsigned)(n + 1) * ntile, s, c, n, 1);
        }
      }
      if (ok) {
        __threadfence();
        // claim the next item now; its latency overlaps this item's work
        next_item = (long long)atomicAdd(s.next, 1ull);
      }
      s_go = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_go) return;
    const int par = (cs.parity0 + n) & 1;
    const T* fin = (const T*)cs.fb[par];
    T* fout = (T*)cs.fb[1 - par];
    if (is_step) {
      const int64_t base = cs.g.id_lo + sub * (int64_t)(kPB * CPT);
#pragma unroll
      for (int q = 0; q < CPT; ++q) step_node<DIM, T>(cs, base + q * kPB + threadIdx.x, fin, fout);
    } else {
      const int64_t i0 = sub * (int64_t)kPersistFillChunk;
      for (int64_t i = i0 + threadIdx.x; i < i0 + kPersistFillChunk && i < cs.n_fill; i += kPB)
        fill_entry<T>(cs, i, fin, fout);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(is_step ? s.done_step + c : s.done_fill + c, 1u);
      s_item = next_item;
    }
    __syncthreads();
  }
}

template <class F>
cudaError_t dispatch_narrow(int store, F&& fn) {
  switch (store) {
    case kStoreF32: return fn(float{});
    case kStoreBF16: return fn(__nv_bfloat16{});
    case kStoreF16: return fn(__half{});
    default: return cudaErrorInvalidValue;
  }
}

template <int DIM, class T>
const void* persistent_kernel() {
  return (const void*)&k_batch_persistent<DIM, T, kPersistCPT>;
}

}  // namespace

size_t persistent_smem(int ncases) {
  return sizeof(long long) * 2 * ((size_t)ncases + 1) + sizeof(int) * (size_t)ncases;
}

cudaError_t persistent_grid(int dim, int store, int ncases, int* blocks) {
  return dispatch_narrow(store, [&](auto tag) {
    using T = decltype(tag);
    const void* k = dim == 2 ? persistent_kernel<2, T>() : persistent_kernel<3, T>();
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, kPB, persistent_smem(ncases));
    *blocks = sms * per;
    return e;
  });
}

cudaError_t launch_batch_persistent(int dim, int store, int blocks, const PersistSched& s,
                                    cudaStream_t st) {
  return dispatch_narrow(store, [&](auto tag) {
    using T = decltype(tag);
    const void* k = dim == 2 ? persistent_kernel<2, T>() : persistent_kernel<3, T>();
    PersistSched arg = s;
    void* args[] = {&arg};
    return cudaLaunchCooperativeKernel(k, dim3((unsigned)blocks), dim3(kPB), args,
                                       persistent_smem(s.ncases), st);
  });
}

}  // namespace imx
