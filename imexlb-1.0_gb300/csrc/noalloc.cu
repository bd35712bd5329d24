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
void* g_partials_addr[kMaxDevices] = {};

// Set-up, once per device, with that device current.
int partials_address(int device, unsigned long long** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_partials_addr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_monitor_partials) != cudaSuccess || !p) return IMEXLB_ERR_CUDA;
    g_partials_addr[device] = p;
  }
  *out = static_cast<unsigned long long*>(g_partials_addr[device]);
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
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = size_fluid > 0 ? (size_fluid + kChunk - 1) / kChunk : 1;
  k_monitor_partial<<<nblocks, kThreads, 0, s>>>(u, fluid_id, size_fluid, dim, partials);
  k_monitor_final<<<1, kThreads, 0, s>>>(partials, nblocks, umax);
  if (cudaGetLastError() != cudaSuccess) {
    imx::set_thread_error("imexlb_monitor_noalloc: kernel launch failed");
    return IMEXLB_ERR_CUDA;
  }
  return IMEXLB_OK;
}
