// SetGeometry on the device (imexlb_device_set_geometry): the reference's
// geometry of one rank's box (initialization.f90:167-255,
// initialization_3d.f90:170-279) computed by kernels, for hosts that set up
// many cases (an ensemble generator) and would otherwise loop over every
// padded cell on the CPU. Same outputs, bit for bit, as
// imexlb_host_set_geometry (host_setup.cpp):
//   - geo: 1 where (x-pos)^2 + (y-ny/2-yoff)^2 [+ (z-nz/2)^2] > radius^2 on
//     the interior (the reference's double arithmetic, nothing contracted),
//     the ghost layers filled by the one-rank PassInt (a periodic wrap);
//   - fluid_id and the rim lists bl, br, bu, bd (bf, bb in 3D) in the
//     reference's loop order (z, then y, then x fastest), which is the order
//     of the cell index: ordered stream compaction;
//   - b_user: in every x-row the first solid cell whose probe
//     geo(id + e_x + dy*(iq*dim+1) [+ dz*(iq*dim+2)]) is fluid for some iq
//     (initialization.f90:232-253): one thread per row.
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "imexlb.h"
#include "imexlb_host.h"
#include "lattice.h"

namespace imx {
void set_thread_error(const char* msg);  // imexlb.cpp: text for imexlb_last_error(NULL)
}

namespace {

constexpr int G = imx::kGhost;
constexpr int kLists = 7;  // fluid_id, bl, br, bu, bd, bf, bb
constexpr int kThreads = 256;
constexpr int kItems = 8;  // loop cells per thread and block pass
constexpr int kChunk = kThreads * kItems;

struct GeoBox {
  int dim, L0, L1, L2, s0, s1, s2, nx, ny, nz;
  long long dy, dz, N;
  double pos, cy, cz, r2max;  // cy = ny/2 + yoff, cz = nz/2, r2max = radius^2
  long long loop_cells;       // (L0+3)(L1+3)[(L2+3)]: the reference's loop box
};

__device__ __forceinline__ int wrapc(int c, int L) { return c < G ? c + L : (c >= L + G ? c - L : c); }

// geo of the interior cell at padded coordinates (X, Y, Z)
__device__ __forceinline__ int fluid_at(const GeoBox& b, int X, int Y, int Z) {
  const int x = X - G + b.s0, y = Y - G + b.s1, z = Z - G + b.s2;
  const double ax = __dsub_rn((double)x, b.pos), ay = __dsub_rn((double)y, b.cy);
  double r2 = __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
  if (b.dim == 3) {
    const double az = __dsub_rn((double)z, b.cz);
    r2 = __dadd_rn(r2, __dmul_rn(az, az));
  }
  return r2 > b.r2max ? 1 : 0;
}

// Every padded cell: interior cells from the obstacle test, ghost cells from
// the interior cell one period away (PassInt with one periodic rank).
__global__ void k_geo(GeoBox b, int* __restrict__ geo) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= b.N) return;
  int X, Y, Z = 0;
  if (b.dim == 3) {
    Z = (int)(id / b.dz);
    const long long r = id - (long long)Z * b.dz;
    Y = (int)(r / b.dy);
    X = (int)(r - (long long)Y * b.dy);
  } else {
    Y = (int)(id / b.dy);
    X = (int)(id - (long long)Y * b.dy);
  }
  geo[id] = fluid_at(b, wrapc(X, b.L0), wrapc(Y, b.L1), b.dim == 3 ? wrapc(Z, b.L2) : 0);
}

// Loop position q (x fastest over L0+3, then y over L1+3, then z) -> cell id
// and list memberships (bit m: list m).
__device__ __forceinline__ unsigned flags_at(const GeoBox& b, const int* __restrict__ geo,
                                             long long q, long long* id_out) {
  const int PX = b.L0 + 3, PY = b.L1 + 3;
  const int i = (int)(q % PX);
  const long long t = q / PX;
  const int j = (int)(t % PY);
  const int k = (int)(t / PY);
  const long long id = (long long)(i - 1 + G) + b.dy * (j - 1 + G) + (b.dim == 3 ? b.dz * (k - 1 + G) : 0);
  *id_out = id;
  const int x = i - 1 + b.s0, y = j - 1 + b.s1, z = k - 1 + b.s2;
  const bool inside = i >= 1 && i <= b.L0 && j >= 1 && j <= b.L1 && (b.dim == 2 || (k >= 1 && k <= b.L2));
  if (inside) return geo[id] ? 1u : 0u;
  unsigned f = 0;
  if (x == -1) f |= 1u << 1;
  if (x == b.nx + 1) f |= 1u << 2;
  if (b.dim == 2) {
    if (y == b.ny + 1) f |= 1u << 3;
    if (y == -1) f |= 1u << 4;
  } else {
    if (y == -1) f |= 1u << 5;
    if (y == b.ny + 1) f |= 1u << 6;
    if (z == -1) f |= 1u << 4;
    if (z == b.nz + 1) f |= 1u << 3;
  }
  return f;
}

// Pass 1: members of each list per block of kChunk loop cells.
__global__ void __launch_bounds__(kThreads) k_list_count(GeoBox b, const int* __restrict__ geo,
                                                         int nblocks, int* __restrict__ counts) {
  __shared__ int c[kLists];
  if (threadIdx.x < kLists) c[threadIdx.x] = 0;
  __syncthreads();
  int mine[kLists] = {0, 0, 0, 0, 0, 0, 0};
  for (int it = 0; it < kItems; ++it) {
    const long long q = (long long)blockIdx.x * kChunk + (long long)it * kThreads + threadIdx.x;
    if (q >= b.loop_cells) break;
    long long id;
    const unsigned f = flags_at(b, geo, q, &id);
#pragma unroll
    for (int m = 0; m < kLists; ++m) mine[m] += (f >> m) & 1u;
  }
#pragma unroll
  for (int m = 0; m < kLists; ++m)
    if (mine[m]) atomicAdd(&c[m], mine[m]);
  __syncthreads();
  if (threadIdx.x < kLists) counts[threadIdx.x * nblocks + blockIdx.x] = c[threadIdx.x];
}

// Exclusive scan of each list's block counts (one block; lists in turn).
__global__ void __launch_bounds__(1024) k_list_scan(int* __restrict__ counts, int nblocks,
                                                    int* __restrict__ totals) {
  __shared__ int warp_sum[32];
  __shared__ int carry;
  for (int m = 0; m < kLists; ++m) {
    int* c = counts + (long long)m * nblocks;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += 1024) {
      const int i = base + threadIdx.x;
      const int v = i < nblocks ? c[i] : 0;
      int x = v;  // inclusive warp scan
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= o) x += y;
      }
      if ((threadIdx.x & 31) == 31) warp_sum[threadIdx.x >> 5] = x;
      __syncthreads();
      if (threadIdx.x < 32) {
        int w = warp_sum[threadIdx.x];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, w, o);
          if (threadIdx.x >= o) w += y;
        }
        warp_sum[threadIdx.x] = w;  // inclusive over warps
      }
      __syncthreads();
      const int before = (threadIdx.x >= 32 ? warp_sum[(threadIdx.x >> 5) - 1] : 0) + x - v;
      if (i < nblocks) c[i] = carry + before;
      __syncthreads();
      if (threadIdx.x == 1023) carry += warp_sum[31];
      __syncthreads();
    }
    if (threadIdx.x == 0) totals[m] = carry;
    __syncthreads();
  }
}

struct ListOut {
  int* p[kLists];
};

// Pass 2: write each list's members in loop order from the block's offset.
__global__ void __launch_bounds__(kThreads) k_list_write(GeoBox b, const int* __restrict__ geo,
                                                         int nblocks, const int* __restrict__ offs,
                                                         ListOut out) {
  __shared__ int wsum[kLists][kThreads / 32];
  __shared__ int run[kLists];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x < kLists) run[threadIdx.x] = offs[threadIdx.x * nblocks + blockIdx.x];
  __syncthreads();
  for (int it = 0; it < kItems; ++it) {
    const long long q = (long long)blockIdx.x * kChunk + (long long)it * kThreads + threadIdx.x;
    long long id = 0;
    const unsigned f = q < b.loop_cells ? flags_at(b, geo, q, &id) : 0u;
    unsigned bal[kLists];
#pragma unroll
    for (int m = 0; m < kLists; ++m) {
      bal[m] = __ballot_sync(0xffffffffu, (f >> m) & 1u);
      if (lane == 0) wsum[m][w] = __popc(bal[m]);
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < kLists; ++m) {
      if ((f >> m) & 1u) {
        int before = run[m];
        for (int v = 0; v < w; ++v) before += wsum[m][v];
        before += __popc(bal[m] & ((1u << lane) - 1u));
        out.p[m][before] = (int)id;
      }
    }
    __syncthreads();
    if (threadIdx.x < kLists) {
      int s = 0;
      for (int v = 0; v < kThreads / 32; ++v) s += wsum[threadIdx.x][v];
      run[threadIdx.x] += s;
    }
    __syncthreads();
  }
}

// The obstacle scan, one thread per x-row of the loop box: the first solid
// cell whose probe reads a fluid cell, or -1; *oob is set when a probe
// leaves the geo array (the reference reads undefined memory there).
__global__ void k_obstacle_rows(GeoBox b, const int* __restrict__ geo, const int* __restrict__ e,
                                int nq, int* __restrict__ row_hit, int* __restrict__ oob) {
  const int PY = b.L1 + 3;
  const int rows = PY * (b.dim == 3 ? b.L2 + 3 : 1);
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int j = r % PY, k = r / PY;
  int hit_id = -1;
  for (int i = 0; i <= b.L0 + 2 && hit_id < 0; ++i) {
    const long long id = (long long)(i - 1 + G) + b.dy * (j - 1 + G) + (b.dim == 3 ? b.dz * (k - 1 + G) : 0);
    if (geo[id] != 0) continue;
    for (int iq = 0; iq < nq; ++iq) {
      long long pr = id + e[iq * b.dim] + b.dy * (long long)(iq * b.dim + 1);
      if (b.dim == 3) pr += b.dz * (long long)(iq * b.dim + 2);
      if (pr < 0 || pr >= b.N) {
        atomicOr(oob, 1);
        continue;
      }
      if (geo[pr] == 1) {
        hit_id = (int)id;
        break;
      }
    }
  }
  row_hit[r] = hit_id;
}

}  // namespace

extern "C" int imexlb_device_set_geometry(const imexlb_config* c, int device, int* geo,
                                          int* fluid_id, int* bl, int* br, int* bu, int* bd,
                                          int* bf, int* bb, int* b_user, int sizes[8]) {
  if (!c || !geo || !fluid_id || !bl || !br || !bu || !bd || !b_user || !sizes ||
      (c->dim != 2 && c->dim != 3) || (c->dim == 3 && (!bf || !bb))) {
    imx::set_thread_error("imexlb_device_set_geometry: bad argument");
    return IMEXLB_ERR_ARG;
  }
  long long caps[8];
  imexlb_host_list_capacity(c, caps);
  GeoBox b{};
  b.dim = c->dim;
  b.L0 = c->local_length[0];
  b.L1 = c->local_length[1];
  b.L2 = c->dim == 3 ? c->local_length[2] : 1;
  b.s0 = c->local_start[0];
  b.s1 = c->local_start[1];
  b.s2 = c->dim == 3 ? c->local_start[2] : 0;
  b.nx = c->nx;
  b.ny = c->ny;
  b.nz = c->nz;
  b.dy = c->dy;
  b.dz = c->dim == 3 ? c->dz : 0;
  b.N = c->array_size;
  b.pos = c->pos;
  b.cy = c->ny / 2.0 + c->yoff;  // as the host set-up forms it
  b.cz = c->nz / 2.0;
  b.r2max = c->radius * c->radius;
  b.loop_cells = (long long)(b.L0 + 3) * (b.L1 + 3) * (c->dim == 3 ? b.L2 + 3 : 1);
  const int nq = c->dim == 2 ? 9 : 27;
  double t[27];
  int e[81];
  imexlb_host_lattice(c->dim, t, e);
  const int nblocks = (int)((b.loop_cells + kChunk - 1) / kChunk);
  const int rows = (b.L1 + 3) * (c->dim == 3 ? b.L2 + 3 : 1);

  int prev = 0;
  cudaGetDevice(&prev);
  if (cudaSetDevice(device) != cudaSuccess) {
    imx::set_thread_error("imexlb_device_set_geometry: cudaSetDevice failed");
    return IMEXLB_ERR_CUDA;
  }
  int* d_geo = nullptr;
  int* d_counts = nullptr;
  int* d_tot = nullptr;
  int* d_e = nullptr;
  int* d_rows = nullptr;
  int* d_oob = nullptr;
  int* d_lists[kLists] = {};
  int rc = IMEXLB_OK;
  const char* what = nullptr;
  auto ck = [&](cudaError_t err, const char* w) {
    if (err != cudaSuccess && rc == IMEXLB_OK) {
      rc = IMEXLB_ERR_CUDA;
      what = w;
    }
    return rc == IMEXLB_OK;
  };
  int tot[kLists] = {};
  std::vector<int> row_hit((size_t)rows);
  int oob = 0;
  if (ck(cudaMalloc(&d_geo, sizeof(int) * (size_t)b.N), "cudaMalloc") &&
      ck(cudaMalloc(&d_counts, sizeof(int) * (size_t)kLists * nblocks), "cudaMalloc") &&
      ck(cudaMalloc(&d_tot, sizeof(int) * kLists), "cudaMalloc") &&
      ck(cudaMalloc(&d_e, sizeof(int) * 81), "cudaMalloc") &&
      ck(cudaMalloc(&d_rows, sizeof(int) * (size_t)rows), "cudaMalloc") &&
      ck(cudaMalloc(&d_oob, sizeof(int)), "cudaMalloc")) {
    for (int m = 0; m < kLists && rc == IMEXLB_OK; ++m)
      ck(cudaMalloc(&d_lists[m], sizeof(int) * (size_t)(caps[m] > 0 ? caps[m] : 1)), "cudaMalloc");
  }
  if (rc == IMEXLB_OK) {
    ListOut lo;
    for (int m = 0; m < kLists; ++m) lo.p[m] = d_lists[m];
    ck(cudaMemcpy(d_e, e, sizeof(int) * 81, cudaMemcpyHostToDevice), "cudaMemcpy") &&
        ck(cudaMemset(d_oob, 0, sizeof(int)), "cudaMemset");
    if (rc == IMEXLB_OK) {
      k_geo<<<(unsigned)((b.N + 255) / 256), 256>>>(b, d_geo);
      k_list_count<<<nblocks, kThreads>>>(b, d_geo, nblocks, d_counts);
      k_list_scan<<<1, 1024>>>(d_counts, nblocks, d_tot);
      k_list_write<<<nblocks, kThreads>>>(b, d_geo, nblocks, d_counts, lo);
      k_obstacle_rows<<<(rows + 127) / 128, 128>>>(b, d_geo, d_e, nq, d_rows, d_oob);
      ck(cudaGetLastError(), "kernel launch") && ck(cudaDeviceSynchronize(), "kernel");
    }
  }
  if (rc == IMEXLB_OK &&
      ck(cudaMemcpy(tot, d_tot, sizeof(tot), cudaMemcpyDeviceToHost), "cudaMemcpy") &&
      ck(cudaMemcpy(geo, d_geo, sizeof(int) * (size_t)b.N, cudaMemcpyDeviceToHost), "cudaMemcpy") &&
      ck(cudaMemcpy(row_hit.data(), d_rows, sizeof(int) * (size_t)rows, cudaMemcpyDeviceToHost),
         "cudaMemcpy") &&
      ck(cudaMemcpy(&oob, d_oob, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy")) {
    int* dst[kLists] = {fluid_id, bl, br, bu, bd, bf, bb};
    for (int m = 0; m < kLists && rc == IMEXLB_OK; ++m) {
      if (tot[m] > caps[m]) {
        rc = IMEXLB_ERR_ARG;
        what = "list longer than its capacity";
        break;
      }
      if (tot[m] > 0)
        ck(cudaMemcpy(dst[m], d_lists[m], sizeof(int) * (size_t)tot[m], cudaMemcpyDeviceToHost),
           "cudaMemcpy");
      sizes[m] = tot[m];
    }
  }
  cudaFree(d_geo);
  cudaFree(d_counts);
  cudaFree(d_tot);
  cudaFree(d_e);
  cudaFree(d_rows);
  cudaFree(d_oob);
  for (int m = 0; m < kLists; ++m) cudaFree(d_lists[m]);
  cudaSetDevice(prev);
  if (rc != IMEXLB_OK) {
    imx::set_thread_error(what ? what : "imexlb_device_set_geometry failed");
    return rc;
  }
  int n = 0;
  for (int r = 0; r < rows; ++r)
    if (row_hit[(size_t)r] >= 0) b_user[n++] = row_hit[(size_t)r];
  sizes[7] = n;
  return oob ? IMEXLB_ERR_GEOMETRY : IMEXLB_OK;
}
