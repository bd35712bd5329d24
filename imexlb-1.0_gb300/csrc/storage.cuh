// Storage types of the population buffers and their conversions. Narrowing
// conversions round to nearest even.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "fixed64.cuh"
#include "kernels.h"

namespace imx {

template <class T>
struct Store;

template <>
struct Store<double> {
  __device__ static __forceinline__ double to_d(double v) { return v; }
  __device__ static __forceinline__ double from_d(double v) { return v; }
  __device__ static __forceinline__ float to_f(double v) { return (float)v; }
  __device__ static __forceinline__ double from_f(float v) { return (double)v; }
  __device__ static __forceinline__ double nan() { return __longlong_as_double(0x7ff8000000000000LL); }
};

template <>
struct Store<float> {
  __device__ static __forceinline__ double to_d(float v) { return (double)v; }
  __device__ static __forceinline__ float from_d(double v) { return __double2float_rn(v); }
  __device__ static __forceinline__ float to_f(float v) { return v; }
  __device__ static __forceinline__ float from_f(float v) { return v; }
  __device__ static __forceinline__ float nan() { return __int_as_float(0x7fc00000); }
};

template <>
struct Store<__nv_bfloat16> {
  __device__ static __forceinline__ double to_d(__nv_bfloat16 v) { return (double)__bfloat162float(v); }
  __device__ static __forceinline__ __nv_bfloat16 from_d(double v) { return __double2bfloat16(v); }
  __device__ static __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
  __device__ static __forceinline__ __nv_bfloat16 from_f(float v) { return __float2bfloat16_rn(v); }
  __device__ static __forceinline__ __nv_bfloat16 nan() { return __ushort_as_bfloat16((unsigned short)0x7fc0); }
};

template <>
struct Store<__half> {
  __device__ static __forceinline__ double to_d(__half v) { return (double)__half2float(v); }
  __device__ static __forceinline__ __half from_d(double v) { return __double2half(v); }
  __device__ static __forceinline__ float to_f(__half v) { return __half2float(v); }
  __device__ static __forceinline__ __half from_f(float v) { return __float2half_rn(v); }
  __device__ static __forceinline__ __half nan() { return __ushort_as_half((unsigned short)0x7e00); }
};

// Q3.60 fixed point (fixed64.cuh); the reserved value stands for NaN.
template <>
struct Store<Fix64> {
  __device__ static __forceinline__ double to_d(Fix64 v) { return fix_to_double(v.v); }
  __device__ static __forceinline__ Fix64 from_d(double v) { return Fix64{fix_from_double(v)}; }
  __device__ static __forceinline__ float to_f(Fix64 v) { return (float)fix_to_double(v.v); }
  __device__ static __forceinline__ Fix64 from_f(float v) { return Fix64{fix_from_double((double)v)}; }
  __device__ static __forceinline__ Fix64 nan() { return Fix64{kFixInvalid}; }
};

// Call fn(T{}) with the storage type of `store`.
template <class F>
inline cudaError_t dispatch_store(int store, F&& fn) {
  switch (store) {
    case kStoreF64: return fn(double{});
    case kStoreF32: return fn(float{});
    case kStoreBF16: return fn(__nv_bfloat16{});
    case kStoreF16: return fn(__half{});
    case kStoreFix: return fn(Fix64{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace imx
