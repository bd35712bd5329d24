// Convolution kernels of the warm-start neural operator: 3x3 convolutions
// (stride 1 or 2, optional nearest x2 upsampling of the input) on NHWC
// bfloat16 activations with FP32 accumulation on the tensor cores
// (mma.sync m16n8k16 bf16), their data and weight gradients, and Adam.
//
// All three products are one implicit GEMM, C[M x N] = A[M x K] B[K x N],
// with the operands gathered on the fly:
//   forward      M = output pixels, K = 9*Cin (tap-major), N = Cout
//   data grad    M = input pixels of the (upsampled) grid, K = 9*Cout, N = Cin
//   weight grad  M = Cout, K = output pixels, N = 9*Cin   (K split over blocks)
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "imexlb_nn.h"

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct Geo {
  int n, hin, win, cin, hout, wout, cout, stride, up;
  // size of the grid the 3x3 stencil runs on (the input, upsampled when up)
  __device__ __forceinline__ int hg() const { return up ? 2 * hin : hin; }
  __device__ __forceinline__ int wg() const { return up ? 2 * win : win; }
};

// x value of the stencil grid at (img, gy, gx, c); 0 outside.
__device__ __forceinline__ bf16 grid_val(const Geo& g, const bf16* __restrict__ x, int img, int gy,
                                         int gx, int c) {
  if (gy < 0 || gx < 0 || gy >= g.hg() || gx >= g.wg()) return __float2bfloat16(0.0f);
  const int sy = g.up ? gy >> 1 : gy, sx = g.up ? gx >> 1 : gx;
  return x[(((int64_t)img * g.hin + sy) * g.win + sx) * g.cin + c];
}

// ---- operand loaders: pair (k, k+1) at row m of A, or at column n of B ----

// Forward A: im2col of x; k = tap*Cin + ci (Cin even, so a pair never splits a tap).
struct FwdA {
  Geo g;
  const bf16* x;
  __device__ __forceinline__ uint32_t pair(int m, int k) const {
    const int hw = g.hout * g.wout;
    const int img = m / hw, r = m - img * hw, oy = r / g.wout, ox = r - oy * g.wout;
    const int tap = k / g.cin, ci = k - tap * g.cin;
    const int gy = oy * g.stride + tap / 3 - 1, gx = ox * g.stride + tap % 3 - 1;
    if (gy < 0 || gx < 0 || gy >= g.hg() || gx >= g.wg()) return 0u;
    const int sy = g.up ? gy >> 1 : gy, sx = g.up ? gx >> 1 : gx;
    return *(const uint32_t*)(x + (((int64_t)img * g.hin + sy) * g.win + sx) * g.cin + ci);
  }
};
// Forward B: weights w[co][tap*Cin + ci].
struct FwdB {
  const bf16* w;
  int K;
  __device__ __forceinline__ uint32_t pair(int k, int n) const {
    return *(const uint32_t*)(w + (int64_t)n * K + k);
  }
};

// Data-grad A: dz gathered through the transposed stencil; m = stencil-grid
// pixel, k = tap*Cout + co; the output pixel reading grid (gy, gx) through
// tap (ky, kx) is ((gy + 1 - ky)/s, (gx + 1 - kx)/s) when that divides.
struct DgradA {
  Geo g;
  const bf16* dz;
  __device__ __forceinline__ uint32_t pair(int m, int k) const {
    const int hw = g.hg() * g.wg();
    const int img = m / hw, r = m - img * hw, gy = r / g.wg(), gx = r - gy * g.wg();
    const int tap = k / g.cout, co = k - tap * g.cout;
    int ty = gy + 1 - tap / 3, tx = gx + 1 - tap % 3;
    if (ty < 0 || tx < 0) return 0u;
    if (g.stride == 2) {
      if ((ty | tx) & 1) return 0u;
      ty >>= 1;
      tx >>= 1;
    }
    if (ty >= g.hout || tx >= g.wout) return 0u;
    return *(const uint32_t*)(dz + (((int64_t)img * g.hout + ty) * g.wout + tx) * g.cout + co);
  }
};
// Data-grad B: wt[ci][tap*Cout + co] (transposed weights).
struct DgradB {
  const bf16* wt;
  int K;
  __device__ __forceinline__ uint32_t pair(int k, int n) const {
    return *(const uint32_t*)(wt + (int64_t)n * K + k);
  }
};

// Weight-grad A: dz^T, row co, column = output pixel (pairs are two pixels).
struct WgradA {
  const bf16* dz;
  int cout, M;  // M = number of output pixels
  __device__ __forceinline__ uint32_t pair(int co, int p) const {
    const bf16 a = p < M ? dz[(int64_t)p * cout + co] : __float2bfloat16(0.0f);
    const bf16 b = p + 1 < M ? dz[(int64_t)(p + 1) * cout + co] : __float2bfloat16(0.0f);
    return pack2(a, b);
  }
};
// Weight-grad B: im2col(x), row = output pixel p, column = tap*Cin + ci.
struct WgradB {
  Geo g;
  const bf16* x;
  int M;
  __device__ __forceinline__ bf16 one(int p, int k) const {
    if (p >= M) return __float2bfloat16(0.0f);
    const int hw = g.hout * g.wout;
    const int img = p / hw, r = p - img * hw, oy = r / g.wout, ox = r - oy * g.wout;
    const int tap = k / g.cin, ci = k - tap * g.cin;
    return grid_val(g, x, img, oy * g.stride + tap / 3 - 1, ox * g.stride + tap % 3 - 1, ci);
  }
  __device__ __forceinline__ uint32_t pair(int p, int k) const { return pack2(one(p, k), one(p + 1, k)); }
};

// One warp computes a 16 x (8*NF) tile of C over k in [k0, k1).
template <int NF, class LA, class LB>
__device__ __forceinline__ void warp_tile(const LA& la, const LB& lb, int m0, int n0, int k0, int k1,
                                          int M, float (&acc)[NF][4]) {
  const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
  const int r0 = m0 + gid, r1 = m0 + gid + 8;
  for (int k = k0; k < k1; k += 16) {
    uint32_t a[4];
    const int c0 = k + 2 * tig, c1 = k + 2 * tig + 8;
    a[0] = r0 < M ? la.pair(r0, c0) : 0u;
    a[1] = r1 < M ? la.pair(r1, c0) : 0u;
    a[2] = r0 < M ? la.pair(r0, c1) : 0u;
    a[3] = r1 < M ? la.pair(r1, c1) : 0u;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      uint32_t b[2];
      const int n = n0 + f * 8 + gid;
      b[0] = lb.pair(c0, n);
      b[1] = lb.pair(c1, n);
      mma16816(acc[f], a, b);
    }
  }
}

constexpr int kWarps = 4;

// Forward / data-grad: C rows = pixels, all N columns (N = 8*NF) per warp.
// Epilogue: + bias, ReLU, store bf16 (or f32) NHWC.
template <int NF, class LA, class LB>
__global__ void __launch_bounds__(32 * kWarps) k_gemm_rows(LA la, LB lb, int M, int K,
                                                            const float* __restrict__ bias,
                                                            int relu, bf16* out_b, float* out_f,
                                                            int ncols_store) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = (blockIdx.x * kWarps + warp) * 16;
  if (m0 >= M) return;
  float acc[NF][4];
#pragma unroll
  for (int f = 0; f < NF; ++f) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.0f;
  warp_tile<NF>(la, lb, m0, 0, 0, K, M, acc);
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int f = 0; f < NF; ++f)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = m0 + gid + 8 * h;
      if (row >= M) continue;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int col = f * 8 + 2 * tig + j;
        if (col >= ncols_store) continue;
        float v = acc[f][2 * h + j] + (bias ? bias[col] : 0.0f);
        if (relu) v = fmaxf(v, 0.0f);
        if (out_f) out_f[(int64_t)row * ncols_store + col] = v;
        else out_b[(int64_t)row * ncols_store + col] = __float2bfloat16(v);
      }
    }
}

// Weight gradient: C = dz^T (Cout x P) * im2col (P x 9Cin); grid.x over
// 8*NF-column groups of 9Cin, grid.y over Cout/16, grid.z over pixel slices.
template <int NF>
__global__ void __launch_bounds__(32 * kWarps) k_wgrad(WgradA la, WgradB lb, int P, int N,
                                                        int slice, float* __restrict__ dw) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = (blockIdx.x * kWarps + warp) * 8 * NF;
  const int m0 = blockIdx.y * 16;
  const int p0 = blockIdx.z * slice, p1 = min(P, p0 + slice);
  if (n0 >= N) return;
  float acc[NF][4];
#pragma unroll
  for (int f = 0; f < NF; ++f) acc[f][0] = acc[f][1] = acc[f][2] = acc[f][3] = 0.0f;
  // pixels are the GEMM's K: p0 is a multiple of 16 (slice is)
  warp_tile<NF>(la, lb, m0, n0, p0, p0 + ((p1 - p0 + 15) / 16) * 16, la.cout, acc);
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int f = 0; f < NF; ++f)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = m0 + gid + 8 * h;
      if (co >= la.cout) continue;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int col = n0 + f * 8 + 2 * tig + j;
        if (col < N) atomicAdd(&dw[(int64_t)co * N + col], acc[f][2 * h + j]);
      }
    }
}

// dz = bf16(dy * relu'(y)) over n = pixels*c values, and the bias gradient
// (per-channel sums of dz): block sums in shared memory, one global atomic
// per block and channel.
__global__ void k_act_grad(const float* __restrict__ dy, const bf16* __restrict__ y, int64_t n,
                           int c, int relu, bf16* __restrict__ dz, float* __restrict__ dbias) {
  __shared__ float part[64];
  for (int i = threadIdx.x; i < c; i += blockDim.x) part[i] = 0.0f;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float g = dy[i];
    if (relu && __bfloat162float(y[i]) <= 0.0f) g = 0.0f;
    dz[i] = __float2bfloat16(g);
    if (dbias) atomicAdd(&part[i % c], g);
  }
  __syncthreads();
  if (dbias)
    for (int i = threadIdx.x; i < c; i += blockDim.x) atomicAdd(&dbias[i], part[i]);
}

// Sum the 2x2 children of each pixel of an upsampled grid (data grad of the
// nearest x2 upsampling).
__global__ void k_down_sum(const float* __restrict__ du, int n, int h, int w, int c,
                           float* __restrict__ dx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)n * h * w * c;
  if (i >= total) return;
  const int ch = (int)(i % c);
  int64_t r = i / c;
  const int x = (int)(r % w);
  r /= w;
  const int y = (int)(r % h);
  const int img = (int)(r / h);
  float s = 0.0f;
  for (int dy2 = 0; dy2 < 2; ++dy2)
    for (int dx2 = 0; dx2 < 2; ++dx2)
      s += du[(((int64_t)img * 2 * h + 2 * y + dy2) * (2 * w) + 2 * x + dx2) * c + ch];
  dx[i] = s;
}

// wt[ci][tap*Cout + co] = w[co][tap*Cin + ci]
__global__ void k_transpose_w(const bf16* __restrict__ w, int cout, int cin, bf16* __restrict__ wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cout * 9 * cin) return;
  const int co = i / (9 * cin), r = i - co * 9 * cin, tap = r / cin, ci = r - tap * cin;
  wt[((int64_t)ci * 9 + tap) * cout + co] = w[i];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, bf16* __restrict__ pb, int64_t n, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, float wd) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * p[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  p[i] = pi;
  if (pb) pb[i] = __float2bfloat16(pi);
}

// Mean squared error over the first `used` of `c` channels per pixel, with
// optional per-pixel weights; dy (c channels per pixel, padding channels
// zero) receives d(loss)/dy. Loss partial sums by block into *loss (atomic).
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t,
                      const float* __restrict__ w, int64_t npix, int c, int used, float inv_count,
                      float* __restrict__ dy, float* __restrict__ loss) {
  __shared__ float part[256];
  float acc = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix * c;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t px = i / c;
    const int ch = (int)(i - px * c);
    float g = 0.0f;
    if (ch < used) {
      const float wt = w ? w[px] : 1.0f;
      const float d = y[i] - t[px * used + ch];
      acc += wt * d * d;
      g = 2.0f * wt * d * inv_count;
    }
    dy[i] = g;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) part[threadIdx.x] += part[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, part[0] * inv_count);
}

Geo geo_of(const imexlb_conv_desc* d) {
  return Geo{d->n, d->hin, d->win, d->cin, d->hout, d->wout, d->cout, d->stride, d->upsample};
}

bool valid(const imexlb_conv_desc* d) {
  if (!d || d->n <= 0 || d->cin <= 0 || d->cin % 16 || d->cout <= 0 || d->cout % 16 || d->cout > 64)
    return false;
  if (d->cout_store < 0 || d->cout_store > d->cout) return false;
  if (d->stride != 1 && d->stride != 2) return false;
  const int hg = d->upsample ? 2 * d->hin : d->hin, wg = d->upsample ? 2 * d->win : d->win;
  return d->hout == (hg - 1) / d->stride + 1 && d->wout == (wg - 1) / d->stride + 1;
}

template <class LA, class LB>
cudaError_t rows_gemm(int ncols, LA la, LB lb, int M, int K, const float* bias, int relu, bf16* ob,
                      float* of, int store_cols, cudaStream_t s) {
  const unsigned grid = (unsigned)((M + 16 * kWarps - 1) / (16 * kWarps));
  switch ((ncols + 7) / 8) {
    case 2: k_gemm_rows<2><<<grid, 32 * kWarps, 0, s>>>(la, lb, M, K, bias, relu, ob, of, store_cols); break;
    case 4: k_gemm_rows<4><<<grid, 32 * kWarps, 0, s>>>(la, lb, M, K, bias, relu, ob, of, store_cols); break;
    case 6: k_gemm_rows<6><<<grid, 32 * kWarps, 0, s>>>(la, lb, M, K, bias, relu, ob, of, store_cols); break;
    case 8: k_gemm_rows<8><<<grid, 32 * kWarps, 0, s>>>(la, lb, M, K, bias, relu, ob, of, store_cols); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int imexlb_nn_conv_fwd(const imexlb_conv_desc* d, const void* x, const void* w, const float* bias,
                       int relu, void* y_bf16, float* y_f32, void* stream) {
  if (!valid(d) || !x || !w || (!y_bf16 && !y_f32)) return -1;
  const Geo g = geo_of(d);
  const int M = d->n * d->hout * d->wout, K = 9 * d->cin;
  cudaError_t e = rows_gemm(d->cout, FwdA{g, (const bf16*)x}, FwdB{(const bf16*)w, K}, M, K, bias,
                            relu, (bf16*)y_bf16, y_f32, d->cout_store ? d->cout_store : d->cout,
                            (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : -2;
}

int imexlb_nn_act_grad(const float* dy, const void* y, long long n, int c, int relu, void* dz,
                       float* dbias, void* stream) {
  if (!dy || !dz || n < 0 || c <= 0 || c > 64 || (relu && !y)) return -1;
  if (n == 0) return 0;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_act_grad<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(dy, (const bf16*)y, n, c, relu,
                                                                  (bf16*)dz, dbias);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int imexlb_nn_conv_bwd_data(const imexlb_conv_desc* d, const void* dz, const void* w, void* wt_scratch,
                            float* dgrid, float* dx, void* stream) {
  if (!valid(d) || !dz || !w || !wt_scratch || !dgrid) return -1;
  cudaStream_t s = (cudaStream_t)stream;
  const int total_w = d->cout * 9 * d->cin;
  k_transpose_w<<<(total_w + 255) / 256, 256, 0, s>>>((const bf16*)w, d->cout, d->cin, (bf16*)wt_scratch);
  const Geo g = geo_of(d);
  const int hg = d->upsample ? 2 * d->hin : d->hin, wg = d->upsample ? 2 * d->win : d->win;
  const int M = d->n * hg * wg, K = 9 * d->cout;
  cudaError_t e = rows_gemm(d->cin, DgradA{g, (const bf16*)dz}, DgradB{(const bf16*)wt_scratch, K},
                            M, K, nullptr, 0, nullptr, dgrid, d->cin, s);
  if (e != cudaSuccess) return -2;
  if (d->upsample) {
    if (!dx) return -1;
    const int64_t n = (int64_t)d->n * d->hin * d->win * d->cin;
    k_down_sum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dgrid, d->n, d->hin, d->win, d->cin, dx);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int imexlb_nn_conv_bwd_weight(const imexlb_conv_desc* d, const void* x, const void* dz, float* dw,
                              void* stream) {
  if (!valid(d) || !x || !dz || !dw) return -1;
  const Geo g = geo_of(d);
  const int P = d->n * d->hout * d->wout, N = 9 * d->cin;
  const int slice = 4096;  // pixels per block (multiple of 16)
  constexpr int NF = 6;
  dim3 grid((unsigned)((N + 8 * NF * kWarps - 1) / (8 * NF * kWarps)), (unsigned)((d->cout + 15) / 16),
            (unsigned)((P + slice - 1) / slice));
  k_wgrad<NF><<<grid, 32 * kWarps, 0, (cudaStream_t)stream>>>(
      WgradA{(const bf16*)dz, d->cout, P}, WgradB{g, (const bf16*)x, P}, P, N, slice, dw);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int imexlb_nn_mse(const float* y, const float* target, const float* weight, long long npix, int c,
                  int used, float* dy, float* loss, void* stream) {
  if (!y || !target || !dy || !loss || npix < 0 || c <= 0 || used <= 0 || used > c) return -1;
  if (npix == 0) return 0;
  int64_t blocks = (npix * c + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_mse<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(y, target, weight, npix, c, used,
                                                            1.0f / (float)(npix * used), dy, loss);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int imexlb_nn_adam(float* p, const float* g, float* m, float* v, void* p_bf16, long long n, float lr,
                   float beta1, float beta2, float eps, int t, float weight_decay, void* stream) {
  if (!p || !g || !m || !v || n < 0 || t < 1) return -1;
  if (n == 0) return 0;
  const float bc1 = 1.0f - powf(beta1, (float)t), bc2 = 1.0f - powf(beta2, (float)t);
  k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      p, g, m, v, (bf16*)p_bf16, n, lr, beta1, beta2, eps, bc1, bc2, weight_decay);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // extern "C"
