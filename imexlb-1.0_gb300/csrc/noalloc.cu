// Monitor reduction that allocates nothing (imexlb_monitor_noalloc).
//
// Some hosts cannot let a library call cudaMalloc: a Fortran host whose u
// and fluid_id live in device memory mapped by its OpenMP offload runtime
// (reached with use_device_ptr) runs under that runtime's memory
// management, and an application that reserves device memory up front for
// its own pool has none left to give. For such callers this entry point
// computes the reference's Monitor value, max sqrt(ux^2+uy^2) over
// fluid_id(1:) (lbm.f90:205-217), directly on their device arrays. Its
// scratch (one partial maximum per thread block) is the file-scope array
// below, which every GPU that loads the library holds until the process
// exits.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "imexlb.h"

namespace imx {
void set_thread_error(const char* msg);  // imexlb.cpp: text for imexlb_last_error(NULL)
}

namespace {

constexpr int kThreads = 256;
constexpr int kItemsPerThread = 8;
constexpr int kChunk = kThreads * kItemsPerThread;  // fluid entries per block
constexpr int kMaxBlocks = IMEXLB_NOALLOC_MAX_FLUID / kChunk;
static_assert(IMEXLB_NOALLOC_MAX_FLUID % kChunk == 0, "limit must be whole blocks");

// Scratch shared by every call on a device: one partial maximum (as ordered
// bits of a non-negative double) per block. Host code must not use this name
// as an address; it takes the device address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned long long g_monitor_partials[kMaxBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct Cached {
  unsigned long long ctx_id = 0;  // context the address belongs to (0: none yet)
  void* addr = nullptr;
};
Cached g_partials[kMaxDevices];

// The current context's unique id (CUDA driver, reached through the
// runtime's entry-point query so the library needs no libcuda link); 0 when
// no context is current or the driver lacks the query.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) ==
            cudaSuccess && qa == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
            cudaSuccess && qb == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<GetCurrent>(a);
      get_id = reinterpret_cast<GetId>(b);
    }
    looked_up = true;
  }
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Set-up, once per device and context, with that device current: the device
// address of the scratch array. A device reset creates a new context whose
// module copy holds the array at a new address, so the cache is keyed on the
// context's id; without an id the address is looked up on every call.
int partials_address(int device, unsigned long long** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  Cached& c = g_partials[device];
  const unsigned long long id = current_context_id();
  if (!c.addr || id == 0 || id != c.ctx_id) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_monitor_partials) != cudaSuccess || !p) return IMEXLB_ERR_CUDA;
    c.addr = p;
    c.ctx_id = current_context_id();  // the lookup made the primary context current
  }
  *out = static_cast<unsigned long long*>(c.addr);
  return IMEXLB_OK;
}

__device__ __forceinline__ unsigned long long umax_bits(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

__device__ __forceinline__ unsigned long long block_max(unsigned long long b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = umax_bits(b, __shfl_xor_sync(0xffffffffu, b, o));
  __shared__ unsigned long long w[kThreads / 32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    b = threadIdx.x < kThreads / 32 ? w[threadIdx.x] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = umax_bits(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  return b;
}

// Block b reduces fluid entries [b*kChunk, (b+1)*kChunk) (entry 0 excluded)
// and stores its maximum in partials[b]; every block writes its own slot, so
// no slot has to be cleared between calls.
__global__ void __launch_bounds__(kThreads)
k_monitor_partial(const double* __restrict__ u, const int* __restrict__ fluid_id, int n, int dim,
                  unsigned long long* __restrict__ partials) {
  const int64_t base = (int64_t)blockIdx.x * kChunk;
  unsigned long long m = 0ull;  // bits of +0.0
#pragma unroll
  for (int k = 0; k < kItemsPerThread; ++k) {
    const int64_t idn = base + (int64_t)k * kThreads + threadIdx.x;
    if (idn >= 1 && idn < n) {
      const int64_t id = fluid_id[idn];
      const double ux = u[id * dim], uy = u[id * dim + 1];
      const double v = __dsqrt_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)));
      m = umax_bits(m, (unsigned long long)__double_as_longlong(v));
    }
  }
  m = block_max(m);
  if (threadIdx.x == 0) partials[blockIdx.x] = m;
}

__global__ void __launch_bounds__(kThreads)
k_monitor_final(const unsigned long long* __restrict__ partials, int nblocks, double* out) {
  unsigned long long m = 0ull;
  for (int i = threadIdx.x; i < nblocks; i += kThreads) m = umax_bits(m, partials[i]);
  m = block_max(m);
  if (threadIdx.x == 0) *out = __longlong_as_double((long long)m);
}

}  // namespace

extern "C" int imexlb_monitor_noalloc(int dim, const double* u, const int* fluid_id,
                                      int size_fluid, double* umax, void* stream) {
  if ((dim != 2 && dim != 3) || !u || !fluid_id || !umax || size_fluid < 0) {
    imx::set_thread_error("imexlb_monitor_noalloc: bad argument");
    return IMEXLB_ERR_ARG;
  }
  if (size_fluid > IMEXLB_NOALLOC_MAX_FLUID) {
    imx::set_thread_error(
        "imexlb_monitor_noalloc: size_fluid exceeds IMEXLB_NOALLOC_MAX_FLUID (16777216), the "
        "capacity of its fixed scratch array");
    return IMEXLB_ERR_ARG;
  }
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) {
    imx::set_thread_error("imexlb_monitor_noalloc: no current CUDA device");
    return IMEXLB_ERR_CUDA;
  }
  if (device < 0 || device >= kMaxDevices) {
    imx::set_thread_error("imexlb_monitor_noalloc: device ordinal above 63");
    return IMEXLB_ERR_UNSUPPORTED;
  }
  unsigned long long* partials = nullptr;
  if (partials_address(device, &partials) != IMEXLB_OK) {
    imx::set_thread_error("imexlb_monitor_noalloc: cudaGetSymbolAddress of the scratch array failed");
    return IMEXLB_ERR_CUDA;
  }
  // An error the caller's own work left pending is not this call's: leave it
  // in place (cudaGetLastError would clear it) and report it.
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    const std::string msg = std::string("imexlb_monitor_noalloc: an earlier CUDA error is pending (") +
          cudaGetErrorString(pending) + "); nothing was launched";
    imx::set_thread_error(msg.c_str());
    return IMEXLB_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = size_fluid > 0 ? (size_fluid + kChunk - 1) / kChunk : 1;
  k_monitor_partial<<<nblocks, kThreads, 0, s>>>(u, fluid_id, size_fluid, dim, partials);
  if (cudaGetLastError() != cudaSuccess) {
    imx::set_thread_error("imexlb_monitor_noalloc: launch of k_monitor_partial failed");
    return IMEXLB_ERR_CUDA;
  }
  k_monitor_final<<<1, kThreads, 0, s>>>(partials, nblocks, umax);
  if (cudaGetLastError() != cudaSuccess) {
    imx::set_thread_error("imexlb_monitor_noalloc: launch of k_monitor_final failed");
    return IMEXLB_ERR_CUDA;
  }
  return IMEXLB_OK;
}
