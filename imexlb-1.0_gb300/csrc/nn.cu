// Convolution kernels of the warm-start neural operator: 3x3 convolutions
// (stride 1 or 2, optional nearest x2 upsampling of the input) on NHWC
// bfloat16 activations, their data and weight gradients, and Adam.
//
// The products run on the 5th-generation tensor cores (tcgen05.mma, bf16
// operands in shared memory, FP32 accumulators in tensor memory), each an
// implicit GEMM whose operands are gathered from the activations:
//   forward      C[P x Cout]  = im2col(x)[P x 9Cin] * W^T        (P output pixels)
//   data grad    C[G x Cin]   = dz~[G x 9Cout] * Wt^T            (G stencil-grid pixels)
//   weight grad  C[9Cin x Cout] = im2col(x)^T[9Cin x P] * dz[P x Cout]
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "imexlb_nn.h"
#include "umma.cuh"

namespace {

namespace umma = imx::umma;
typedef __nv_bfloat16 bf16;

struct Geo {
  int n, hin, win, cin, hout, wout, cout, stride, up;
  // size of the grid the 3x3 stencil runs on (the input, upsampled when up)
  __device__ __forceinline__ int hg() const { return up ? 2 * hin : hin; }
  __device__ __forceinline__ int wg() const { return up ? 2 * win : win; }
};

// ---- tcgen05 implicit GEMMs -------------------------------------------------
//
// 16-byte chunk gathers: chunk (m, c) holds elements k = 8c .. 8c+7 of row m
// of the GEMM operand A (8 channels of one tap: Cin and Cout are multiples
// of 16, so a chunk never straddles two taps); nullptr where the stencil
// reads outside the grid (zero).

// Forward A: im2col of x; row m = output pixel, k = tap*Cin + ci.
struct FwdChunk {
  Geo g;
  const bf16* x;
  __device__ __forceinline__ const bf16* at(int m, int c) const {
    const int hw = g.hout * g.wout;
    const int img = m / hw, r = m - img * hw, oy = r / g.wout, ox = r - oy * g.wout;
    const int k = c * 8, tap = k / g.cin, ci = k - tap * g.cin;
    const int gy = oy * g.stride + tap / 3 - 1, gx = ox * g.stride + tap % 3 - 1;
    if (gy < 0 || gx < 0 || gy >= g.hg() || gx >= g.wg()) return nullptr;
    const int sy = g.up ? gy >> 1 : gy, sx = g.up ? gx >> 1 : gx;
    return x + (((int64_t)img * g.hin + sy) * g.win + sx) * g.cin + ci;
  }
};

// Data-grad A: dz through the transposed stencil; row m = stencil-grid
// pixel, k = tap*Cout + co; output pixel ((gy+1-ky)/s, (gx+1-kx)/s) when
// that divides.
struct DgradChunk {
  Geo g;
  const bf16* dz;
  __device__ __forceinline__ const bf16* at(int m, int c) const {
    const int hw = g.hg() * g.wg();
    const int img = m / hw, r = m - img * hw, gy = r / g.wg(), gx = r - gy * g.wg();
    const int k = c * 8, tap = k / g.cout, co = k - tap * g.cout;
    int ty = gy + 1 - tap / 3, tx = gx + 1 - tap % 3;
    if (ty < 0 || tx < 0) return nullptr;
    if (g.stride == 2) {
      if ((ty | tx) & 1) return nullptr;
      ty >>= 1;
      tx >>= 1;
    }
    if (ty >= g.hout || tx >= g.wout) return nullptr;
    return dz + (((int64_t)img * g.hout + ty) * g.wout + tx) * g.cout + co;
  }
};

constexpr int kTM = 128;      // GEMM rows per tile: the MMA's M
constexpr int kTThreads = 128;      // weight-gradient blocks
constexpr int kRowsThreads = 256;   // forward / data-gradient blocks: two threads per row
constexpr int kTmemCols = 64;  // accumulator columns (N <= 64)
constexpr int kWaitTries = 1 << 24;

// Status of the last kernels: 0, or 1 when an MMA completion wait gave up.
__device__ int g_nn_status = 0;

__device__ __forceinline__ uint4 ld16(const bf16* p) {
  return p ? *(const uint4*)p : make_uint4(0u, 0u, 0u, 0u);
}

// C[M x N] = A[M x K] * B^T with B[N x K] (row-major, K contiguous), both
// bf16, FP32 accumulation in TMEM. Persistent over 128-row tiles: B is
// staged once per block; per tile every thread gathers its row of A into the
// core-matrix layout, one thread issues the K/16 MMAs, and after their
// completion each warp reads its 32 rows of the accumulator for the
// epilogue (+ bias, ReLU, bf16 or f32 store of ncols_store columns).
template <int N, class G>
__global__ void __launch_bounds__(kRowsThreads) k_tc_rows(G gather, const bf16* __restrict__ B, int M,
                                                      int K, const float* __restrict__ bias,
                                                      int relu, bf16* out_b, float* out_f,
                                                      int ncols_store) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int sb_bytes = ((N * K * 2 + 1023) / 1024) * 1024;
  bf16* sB = (bf16*)smem;
  bf16* sA = (bf16*)(smem + sb_bytes);
  __shared__ uint32_t tmem_base;
  __shared__ __align__(8) uint64_t mbar;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int kc_n = K / 8;
  for (int i = tid; i < N * kc_n; i += kRowsThreads) {
    const int n = i / kc_n, c = i - n * kc_n;
    *(uint4*)(sB + umma::cm_off(n, c * 8, N)) = *(const uint4*)(B + (int64_t)n * K + c * 8);
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, kTmemCols);
  if (tid == 0) umma::mbar_init(&mbar);
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t aaddr = umma::smem_addr(sA), baddr = umma::smem_addr(sB);
  constexpr uint32_t idesc = umma::idesc_bf16_f32(kTM, N);
  const int ntiles = (M + kTM - 1) / kTM;
  uint32_t phase = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int m = t * kTM + (tid & (kTM - 1));
    // gather: thread (row, c0) loads chunks c0, c0 + kG, ... of its row, kU
    // loads in flight before their stores
    constexpr int kG = kRowsThreads / kTM, kU = 6;
    for (int c = tid / kTM; c < kc_n; c += kG * kU) {
      uint4 v[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int cc = c + u * kG;
        v[u] = cc < kc_n ? ld16(m < M ? gather.at(m, cc) : nullptr) : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int cc = c + u * kG;
        if (cc < kc_n) *(uint4*)(sA + umma::cm_off(tid & (kTM - 1), cc * 8, kTM)) = v[u];
      }
    }
    umma::fence_smem_async();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after();
      for (int s = 0; s < K / 16; ++s)
        umma::mma_bf16(tmem, umma::slice_desc(aaddr, kTM, s), umma::slice_desc(baddr, N, s), idesc,
                       s > 0);
      umma::mma_commit(&mbar);
    }
    ok = umma::mbar_wait(&mbar, phase, kWaitTries);
    phase ^= 1u;
    umma::fence_after();
    if (ok && warp < kTM / 32) {
#pragma unroll
      for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (m < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = c0 + j;
            if (col >= ncols_store) break;
            float x = v[j] + (bias ? bias[col] : 0.0f);
            if (relu) x = fmaxf(x, 0.0f);
            if (out_f) out_f[(int64_t)m * ncols_store + col] = x;
            else out_b[(int64_t)m * ncols_store + col] = __float2bfloat16(x);
          }
        }
      }
    } else if (tid == 0) {
      atomicExch(&g_nn_status, 1);
    }
    umma::fence_before();
    __syncthreads();
  }
  if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
}

// Weight gradient as C^T[9Cin x Cout] = im2col(x)^T (9Cin x P) * dz (P x Cout):
// block (mt, slice) owns rows [128 mt, 128 mt + 128) of 9Cin and a slice of
// output pixels, taken 64 at a time (four K steps of 16 pixels): the tile of
// im2col^T and the tile of dz^T are written transposed into the core-matrix
// layout (8 bf16 of one 16-byte load go to 8 rows), then the MMAs run and
// accumulate in TMEM over the whole slice; the partial C^T is added to dw
// (f32 atomics) as dw[co][row].
template <int N>
__global__ void __launch_bounds__(kTThreads) k_tc_wgrad(Geo g, const bf16* __restrict__ x,
                                                       const bf16* __restrict__ dz, int P,
                                                       int slice, float* __restrict__ dw) {
  constexpr int kPix = 64;
  __shared__ __align__(1024) bf16 sA[kTM * kPix];
  __shared__ __align__(1024) bf16 sB[64 * kPix];
  __shared__ uint32_t tmem_base;
  __shared__ __align__(8) uint64_t mbar;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rows = 9 * g.cin, row0 = blockIdx.x * kTM;
  const int p0 = blockIdx.y * slice, p1 = min(P, p0 + slice);
  if (warp == 0) umma::tmem_alloc(&tmem_base, kTmemCols);
  if (tid == 0) umma::mbar_init(&mbar);
  umma::fence_before();
  __syncthreads();
  umma::fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t aaddr = umma::smem_addr(sA), baddr = umma::smem_addr(sB);
  constexpr uint32_t idesc = umma::idesc_bf16_f32(kTM, N);
  const int hw = g.hout * g.wout;
  uint32_t phase = 0;
  bool ok = true, first = true;
  for (int pc = p0; pc < p1 && ok; pc += kPix) {
    // A^T: 16 row groups (8 channels of one tap) x 64 pixels
    for (int i = tid; i < (kTM / 8) * kPix; i += kTThreads) {
      const int grp = i / kPix, pl = i - grp * kPix, p = pc + pl, r = row0 + grp * 8;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (p < p1 && r < rows) {
        const int img = p / hw, rr = p - img * hw, oy = rr / g.wout, ox = rr - oy * g.wout;
        const int tap = r / g.cin, ci = r - tap * g.cin;
        const int gy = oy * g.stride + tap / 3 - 1, gx = ox * g.stride + tap % 3 - 1;
        if (gy >= 0 && gx >= 0 && gy < g.hg() && gx < g.wg()) {
          const int sy = g.up ? gy >> 1 : gy, sx = g.up ? gx >> 1 : gx;
          v = *(const uint4*)(x + (((int64_t)img * g.hin + sy) * g.win + sx) * g.cin + ci);
        }
      }
      const bf16* e = (const bf16*)&v;
#pragma unroll
      for (int j = 0; j < 8; ++j) sA[umma::cm_off(grp * 8 + j, pl, kTM)] = e[j];
    }
    // dz^T: N/8 groups of 8 output channels x 64 pixels
    for (int i = tid; i < (N / 8) * kPix; i += kTThreads) {
      const int grp = i / kPix, pl = i - grp * kPix, p = pc + pl;
      const uint4 v = p < p1 ? *(const uint4*)(dz + (int64_t)p * g.cout + grp * 8)
                             : make_uint4(0u, 0u, 0u, 0u);
      const bf16* e = (const bf16*)&v;
#pragma unroll
      for (int j = 0; j < 8; ++j) sB[umma::cm_off(grp * 8 + j, pl, N)] = e[j];
    }
    umma::fence_smem_async();
    __syncthreads();
    if (tid == 0) {
      umma::fence_after();
#pragma unroll
      for (int s = 0; s < kPix / 16; ++s)
        umma::mma_bf16(tmem, umma::slice_desc(aaddr, kTM, s), umma::slice_desc(baddr, N, s), idesc,
                       !(first && s == 0));
      umma::mma_commit(&mbar);
    }
    first = false;
    ok = umma::mbar_wait(&mbar, phase, kWaitTries);
    phase ^= 1u;
    umma::fence_after();
    __syncthreads();  // the next chunk overwrites sA / sB
  }
  if (!ok && tid == 0) atomicExch(&g_nn_status, 1);
  if (ok && !first) {
    const int r = row0 + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (r < rows) {
#pragma unroll
        for (int j = 0; j < 16; ++j) atomicAdd(&dw[(int64_t)(c0 + j) * rows + r], v[j]);
      }
    }
  }
  umma::fence_before();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, kTmemCols);
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

// Launch k_tc_rows for N columns: one block per SM (or fewer, for few
// tiles), looping over the 128-row tiles.
template <class G>
cudaError_t tc_rows(int N, G gather, const bf16* B, int M, int K, const float* bias, int relu,
                    bf16* ob, float* of, int store_cols, cudaStream_t s) {
  const int smem = ((N * K * 2 + 1023) / 1024) * 1024 + kTM * K * 2;
  const int tiles = (M + kTM - 1) / kTM;
  auto launch = [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kRowsThreads, smem);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(tiles, sms * std::max(per, 1)));
    kern<<<grid, kRowsThreads, smem, s>>>(gather, B, M, K, bias, relu, ob, of, store_cols);
    return cudaGetLastError();
  };
  switch (N) {
    case 16: return launch(k_tc_rows<16, G>);
    case 32: return launch(k_tc_rows<32, G>);
    case 48: return launch(k_tc_rows<48, G>);
    case 64: return launch(k_tc_rows<64, G>);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

extern "C" {

int imexlb_nn_conv_fwd(const imexlb_conv_desc* d, const void* x, const void* w, const float* bias,
                       int relu, void* y_bf16, float* y_f32, void* stream) {
  if (!valid(d) || !x || !w || (!y_bf16 && !y_f32)) return -1;
  const Geo g = geo_of(d);
  const int M = d->n * d->hout * d->wout, K = 9 * d->cin;
  cudaError_t e = tc_rows(d->cout, FwdChunk{g, (const bf16*)x}, (const bf16*)w, M, K, bias, relu,
                          (bf16*)y_bf16, y_f32, d->cout_store ? d->cout_store : d->cout,
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
  cudaError_t e = tc_rows(d->cin, DgradChunk{g, (const bf16*)dz}, (const bf16*)wt_scratch, M, K,
                          nullptr, 0, nullptr, dgrid, d->cin, s);
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
  const int P = d->n * d->hout * d->wout, rows = 9 * d->cin;
  const int slice = 4096;  // output pixels per block (a multiple of 64)
  const dim3 grid((unsigned)((rows + kTM - 1) / kTM), (unsigned)((P + slice - 1) / slice));
  cudaStream_t s = (cudaStream_t)stream;
  switch (d->cout) {
    case 16: k_tc_wgrad<16><<<grid, kTThreads, 0, s>>>(g, (const bf16*)x, (const bf16*)dz, P, slice, dw); break;
    case 32: k_tc_wgrad<32><<<grid, kTThreads, 0, s>>>(g, (const bf16*)x, (const bf16*)dz, P, slice, dw); break;
    case 48: k_tc_wgrad<48><<<grid, kTThreads, 0, s>>>(g, (const bf16*)x, (const bf16*)dz, P, slice, dw); break;
    case 64: k_tc_wgrad<64><<<grid, kTThreads, 0, s>>>(g, (const bf16*)x, (const bf16*)dz, P, slice, dw); break;
    default: return -1;
  }
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

int imexlb_nn_status(int* status) {
  if (!status) return -1;
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_nn_status, sizeof(int)) != cudaSuccess) return -2;
  *status = v;
  if (v) {
    const int zero = 0;
    if (cudaMemcpyToSymbol(g_nn_status, &zero, sizeof(int)) != cudaSuccess) return -2;
  }
  return 0;
}

}  // extern "C"
