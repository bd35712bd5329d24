// Reduced-precision LBM kernels: populations stored as FP32, BF16 or FP16,
// collision arithmetic in FP32 with every rounding explicit (node_fast.cuh);
// with double storage and double arithmetic the same kernels are the fast
// FP64 option (minimal operation count, not the reference's rounding).
//
// The stored value is the reference's own f, which is already the deviation
// f_i - t_i*rho0 from the rest state (its equilibrium has no t*rho0 term,
// lbm.f90:44), so narrow storage keeps full relative precision near rest.
// Same algorithm and boundary handling as the FP64 kernels (kernels.cu);
// 2*Q*sizeof(T) bytes per node update.
#include <cstdint>
#include <cstring>
#include <utility>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "boundary_fused.cuh"
#include "kernels.h"
#include "lattice.h"
#include "f32x2.cuh"
#include "node_fast.cuh"
#include "staged.cuh"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kBlockLP = 256;

// Max over the block of non-negative values (their bit patterns order like
// the values), one atomicMax per block.
__device__ IMX_FI void block_max_lp(double v, unsigned long long* dst) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
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

template <class T, class R>
__device__ IMX_FI R load_as(const T* p) {
  if constexpr (sizeof(R) == 8) return Store<T>::to_d(*p);
  else return Store<T>::to_f(*p);
}

template <class T, class R>
__device__ IMX_FI T store_as(R v) {
  if constexpr (sizeof(R) == 8) return Store<T>::from_d(v);
  else return Store<T>::from_f(v);
}

// Resident blocks per SM the step kernel is compiled for. The 2-byte kinds
// are latency-bound (few bytes per load): capping registers at 40 gives six
// 256-thread blocks per SM instead of five, 5% faster on D3Q27 (measured on
// 256x128x128: 0.117 vs 0.123 ms); FP32 and FP64 gain nothing from it. 0 = no
// minimum.
template <int DIM, class T>
constexpr int lp_min_blocks() {
  return DIM == 3 ? (sizeof(T) == 2 ? 6 : (sizeof(T) == 4 ? 5 : 0)) : 0;
}

template <int DIM, class T, class R, bool MON>
__global__ void __launch_bounds__(kBlockLP, lp_min_blocks<DIM, T>()) k_step_lp(DevGrid g, CoefR<R> c, DevState st,
                                                       DevPlanes pl,
                                                       unsigned long long* monitor) {
  using N_ = NodeFast<DIM, R>;
  using L = Lattice<DIM>;
  constexpr int Q = N_::Q;
  // 32-bit node index: every plane pointer already carries its direction's offset
  const uint32_t id = (uint32_t)(g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x);
  double um = 0.0;  // R-precision |u| (exact in double)
  const uint8_t m = (int64_t)id < g.id_hi ? st.mask[id] : (uint8_t)0;
  const PullFix fx = PullFix::make(st, (m & kMaskFluid) ? m : (uint8_t)0);
  // warps with a node on a wall or periodic face or with a record take the
  // general pull; the inlet / outlet forms cost every node one add per
  // e_x = -1 direction
  const bool bwarp = __any_sync(0xffffffffu, fx.other());
  if (m & kMaskFluid) {
    R f[Q];
    // plane 0 of each buffer starts at its base (the input plane pointer
    // carries the pull shift -off[0])
    const T* fin = (const T*)pl.in[0] + g.off[0];
    T* fout = (T*)pl.out[0];
    if (!bwarp) {
      const uint32_t id_in = id + fx.inl(), o = fx.outl();
      sfor<0, Q>([&](auto I) {
        constexpr int ex = L::ex(I);
        const uint32_t a = ex == 1 ? id_in : (ex == -1 ? id + o * (uint32_t)g.off[I] : id);
        f[I] = load_as<T, R>((const T*)pl.in[I] + a);
      });
    } else if (!fx.record()) {
      sfor<0, Q>([&](auto I) {
        constexpr int i = I;
        bool opp;
        int64_t sh;
        fx.form<DIM>(L::ex(i), L::ey(i), L::ez(i), g.off[i], st.pshift, opp, sh);
        const T* base = (const T*)(opp ? pl.in[Q - 1 - i] : pl.in[i]);
        f[I] = load_as<T, R>(base + (uint32_t)(id + (uint32_t)sh));
      });
    } else {
      const uint32_t* row = PullFix::row<Q>(st, id);
      sfor<0, Q>([&](auto I) {
        const uint32_t r = row[I];
        f[I] = load_as<T, R>(r != kNoRedirect ? fin + r : (const T*)pl.in[I] + id);
      });
    }
    R u[DIM];
    R S3 = N_::moments(f, u, c.inv_rho0);
    N_::dirichlet(m, id, g, st.inlet, S3, u);
    if constexpr (MON) {
      if (id != g.skip_id) um = (double)N_::speed(u);
    }
    N_::collide(f, S3, u, c, [&](int i, R v) { ((T*)pl.out[i])[id] = store_as<T, R>(v); });
    if (fx.record()) push_copies(st.push, PullFix::row<Q>(st, id)[Q], fin, fout);
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

// max of two non-negative values (or NaN) through their bit patterns: NaN
// stays the maximum, as in the block reduction
__device__ __forceinline__ double bitmax(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  return __longlong_as_double((long long)(x > y ? x : y));
}

// The per-node update of k_step_lp for one fluid cell with the general pull
// (closed forms, or its record's source row).
template <int DIM, class T, bool MON>
__device__ __forceinline__ void lp_node_general(const DevGrid& g, const CoefR<float>& c,
                                                const DevState& st, const DevPlanes& pl,
                                                uint32_t id, uint8_t m, const PullFix& fx,
                                                double& um) {
  using N_ = NodeFast<DIM, float>;
  using L = Lattice<DIM>;
  constexpr int Q = N_::Q;
  float f[Q];
  const T* fin = (const T*)pl.in[0] + g.off[0];
  T* fout = (T*)pl.out[0];
  if (!fx.record()) {
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      bool opp;
      int64_t sh;
      fx.form<DIM>(L::ex(i), L::ey(i), L::ez(i), g.off[i], st.pshift, opp, sh);
      const T* base = (const T*)(opp ? pl.in[Q - 1 - i] : pl.in[i]);
      f[I] = load_as<T, float>(base + (uint32_t)(id + (uint32_t)sh));
    });
  } else {
    const uint32_t* row = PullFix::row<Q>(st, id);
    sfor<0, Q>([&](auto I) {
      const uint32_t r = row[I];
      f[I] = load_as<T, float>(r != kNoRedirect ? fin + r : (const T*)pl.in[I] + id);
    });
  }
  float u[DIM];
  float S3 = N_::moments(f, u, c.inv_rho0);
  N_::dirichlet(m, id, g, st.inlet, S3, u);
  if constexpr (MON) {
    if (id != g.skip_id) um = bitmax(um, (double)N_::speed(u));
  }
  N_::collide(f, S3, u, c, [&](int i, float v) { ((T*)pl.out[i])[id] = store_as<T, float>(v); });
  if (fx.record()) push_copies(st.push, PullFix::row<Q>(st, id)[Q], fin, fout);
}

// ---- Tiles staged in shared memory by the bulk-copy engine ----------------
//
// BF16 / FP16 on D3Q27 (staged.cuh has the tiles, copies, barriers and bounded
// waits): 1024-cell tiles, one producer and sixteen consumer warps per block,
// one block per SM. Each consumer thread updates two cells (64 w + l and
// 64 w + l + 32 of the tile, warp w) with packed f32x2 arithmetic: the same
// rounded float operations per cell for about half the instructions. Loads in
// flight hold no registers, so an SM keeps ~3x the bytes in flight of the
// register-staged k_step_lp. Outlet cells read their e_x = -1 slots from
// global memory. Groups with a wall, periodic-face or record node (a list the
// host makes once per geometry) are left to k_step_bgroups, which runs
// k_step_lp's general pull for them on a second stream, concurrently.
// (Measured on 256x128x128 FP16: in the consumers that pull stalled the
// pipeline on global loads, 132 us; in the producer, between its issues,
// 171 us; as a following kernel on the same stream it added a latency-bound
// 20 us to the staged kernel's 105.)
constexpr int kStageTile = 1024;
// stages per block: 3 of 55.4 KB (D3Q27), one block of 16 consumer warps
// per SM. Measured on 512x256x256 FP16 (ms per iteration; blocks per SM x
// consumer warps): 256-cell tiles, 4 stages (3 x 4) 0.868; 512-cell tiles,
// 2 stages (3 x 4) 0.797, 3 stages (2 x 4) 0.844, 2 stages (2 x 8) 0.780,
// 3 stages (2 x 8) 0.767; 768-cell tiles, 2 stages (2 x 4) 0.801;
// 1024-cell tiles (1 x 16): 2 stages 0.813, 3 stages 0.747, 4 stages 0.818.
// Below ~1 KB per copy the bulk-copy engine's cost per request dominates.
template <class T>
__host__ __device__ constexpr int stage_count() { return 3; }
// consumer warps, each two cells per thread (a kStageGroup-cell group) per
// pass, kStagePasses passes a tile; warp kStageConsumers produces
constexpr int kStageConsumers = 16;
constexpr int kStagePasses = kStageTile / (kStageGroup * kStageConsumers);
constexpr int kStageThreads = 32 * (kStageConsumers + 1);

// The first direction of weight class |e|^2 = n2 (its K_i stands for the
// class's).
template <int DIM>
__host__ __device__ constexpr int class_rep(int n2) {
  for (int i = 0; i < Lattice<DIM>::Q; ++i) {
    const int ex = Lattice<DIM>::ex(i), ey = Lattice<DIM>::ey(i), ez = Lattice<DIM>::ez(i);
    if (ex * ex + ey * ey + ez * ez == n2) return i;
  }
  return -1;
}

// The boundary groups of a staged step: warps 2j and 2j+1 of the grid update
// the cells id_lo + kStageGroup groups[j] + (0 .. kStageGroup-1), a group
// with a wall, periodic-face or record node (the staged kernel skips it), one
// thread per cell with k_step_lp's general pull. It runs on a second stream
// beside the staged kernel, in blocks of 256 threads (four groups, at most 48
// registers). Blocks of 32 or 64 threads, which fit beside the staged block
// in every register-file partition, measured the same.
template <int DIM, class T, bool MON>
__global__ void __launch_bounds__(kBlockLP, 5)  // <= 51 registers
    k_step_bgroups(DevGrid g, CoefR<float> c, DevState st, DevPlanes pl, const uint32_t* groups,
                   int64_t n, unsigned long long* monitor) {
  const int64_t t = (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  const int64_t j = t / kStageGroup;
  double um = 0.0;
  if (j < n) {
    const uint32_t id = (uint32_t)(g.id_lo + (int64_t)groups[j] * kStageGroup + t % kStageGroup);
    const uint8_t m = (int64_t)id < g.id_hi ? st.mask[id] : (uint8_t)0;
    if (m & kMaskFluid) lp_node_general<DIM, T, MON>(g, c, st, pl, id, m, PullFix::make(st, m), um);
  }
  if constexpr (MON) {
    unsigned long long b = (unsigned long long)__double_as_longlong(um);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
      b = x > b ? x : b;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(monitor, b);
  }
}

template <int DIM, class T, bool MON>
__global__ void __launch_bounds__(kStageThreads, 1)
    k_step_staged(const __grid_constant__ DevGrid g, const __grid_constant__ CoefR<float> c,
                  const __grid_constant__ DevState st, const __grid_constant__ DevPlanes pl,
                  const __grid_constant__ StagePlan sp, unsigned long long* monitor) {
  using N_ = NodeFast<DIM, float>;
  using L = Lattice<DIM>;
  constexpr int Q = N_::Q;
  constexpr uint32_t kStage = stage_bytes(Q, kStageTile, sizeof(T));
  constexpr uint32_t kStages = stage_count<T>();
  extern __shared__ __align__(128) uint8_t stage_smem[];
  __shared__ uint64_t full[kStages], empty[kStages];
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    stage_init(full, empty, kStages, kStageConsumers);
    abort_flag = 0;
  }
  __syncthreads();
  const int64_t G = gridDim.x, t0 = blockIdx.x;
  // tiles of this block: t0 + k G for k = 0, 1, ...; tile k uses stage
  // k % kStages in its phase k / kStages
  const uint32_t ntiles = (uint32_t)((sp.ntiles - t0 + G - 1) / G);
  volatile int* abort_v = &abort_flag;

  if (warp == kStageConsumers) {
    stage_produce<Q>(sp, stage_smem, kStage, kStages, kStage, full, empty, ntiles, t0, G, lane,
                     abort_v);
    return;
  }

  // consumers: lane l of warp w updates the tile cells 64 w + l (A, the low
  // half of every F2) and that + 32 (B, the high half); a tile longer than
  // 64 kStageConsumers cells would take kStagePasses such passes
  using N2 = NodeFast<DIM, F2>;
  CoefR<F2> c2;
  {
    // the node update's coefficients as pairs: K_i takes one value per
    // weight class |e_i|^2 (the host checks that the four are exact)
    F2 kc[4];
    sfor<0, Q>([&](auto I) {
      constexpr int n2 = L::ex(I) * L::ex(I) + L::ey(I) * L::ey(I) + L::ez(I) * L::ez(I);
      constexpr int rep = class_rep<DIM>(n2);
      if constexpr (rep == (int)I) kc[n2] = F2(c.k[I]);
    });
    sfor<0, Q>([&](auto I) {
      constexpr int n2 = L::ex(I) * L::ex(I) + L::ey(I) * L::ey(I) + L::ez(I) * L::ez(I);
      c2.k[I] = kc[n2];
    });
    c2.om1 = F2(c.om1);
    c2.inv_rho0 = F2(c.inv_rho0);
  }
  const uint32_t ca = (uint32_t)(kStageGroup * warp + lane);
  double um = 0.0;
  uint32_t s = 0, phase = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < ntiles; ++k) {
    // (the warp goes on only if all its lanes saw the copies land: the
    // update below has warp-wide votes)
    const bool ok = __all_sync(0xffffffffu, stage_wait(&full[s], phase, sp.wait_ns));
    if (!ok) {
      if (lane == 0) stage_give_up(abort_v, sp.status);
      break;
    }
    if (__any_sync(0xffffffffu, *abort_v)) break;
#pragma unroll 1
    for (uint32_t pass = 0; pass < (uint32_t)kStagePasses; ++pass) {
      const uint32_t cp = ca + pass * (uint32_t)(kStageGroup * kStageConsumers);
      // opaque to the compiler, so that the per-direction addresses are formed
      // per tile (hoisted out of the loop they would take ~80 registers)
      uint32_t ida = (uint32_t)(g.id_lo + (t0 + (int64_t)k * G) * kStageTile + cp);
      const uint8_t* sb = stage_smem + s * kStage + cp * sizeof(T);
      asm volatile("" : "+r"(ida), "+l"(sb));
      const uint32_t idb = ida + 32u;
      const uint8_t* sm = stage_smem + s * kStage + sp.mpos + cp;
      const uint8_t ma = (int64_t)ida < g.id_hi ? sm[0] : (uint8_t)0;
      const uint8_t mb = (int64_t)idb < g.id_hi ? sm[32] : (uint8_t)0;
      const bool fla = (ma & kMaskFluid) != 0, flb = (mb & kMaskFluid) != 0;
      const PullFix fxa = PullFix::make(st, fla ? ma : (uint8_t)0);
      const PullFix fxb = PullFix::make(st, flb ? mb : (uint8_t)0);
      const bool bwarp = __any_sync(0xffffffffu, fxa.other() || fxb.other());
      // a group with a wall, periodic-face or record node is k_step_bgroups'
      // part; the cells of a pair that are not fluid run on values that are
      // never stored
      if ((fla || flb) && !bwarp) {
        F2 f[Q];
        const uint32_t inla = fxa.inl(), oa = fxa.outl(), inlb = fxb.inl(), ob = fxb.outl();
        sfor<0, Q>([&](auto I) {
          constexpr int ex = L::ex(I);
          const T* q = (const T*)(sb + sp.pos[I]);
          float va, vb;
          if constexpr (ex == 1) {
            va = load_as<T, float>(q + inla);
            vb = load_as<T, float>(q + 32 + inlb);
          } else if constexpr (ex == -1) {
            const T* own = (const T*)pl.in[I] + (uint32_t)(ida + (uint32_t)g.off[I]);
            va = oa ? load_as<T, float>(own) : load_as<T, float>(q);
            vb = ob ? load_as<T, float>(own + 32) : load_as<T, float>(q + 32);
          } else {
            va = load_as<T, float>(q);
            vb = load_as<T, float>(q + 32);
          }
          f[I] = F2(va, vb);
        });
        F2 u[DIM];
        F2 S3 = N2::moments(f, u, c2.inv_rho0);
        if (((ma | mb) & (kMaskInlet | kMaskOutlet)) != 0) {
          // PostProcessing's Dirichlet conditions per cell, as NodeFast's
          float sa = S3.lo(), sbv = S3.hi(), ua[DIM], ub[DIM];
  #pragma unroll
          for (int d = 0; d < DIM; ++d) {
            ua[d] = u[d].lo();
            ub[d] = u[d].hi();
          }
          NodeFast<DIM, float>::dirichlet(ma, ida, g, st.inlet, sa, ua);
          NodeFast<DIM, float>::dirichlet(mb, idb, g, st.inlet, sbv, ub);
          S3 = F2(sa, sbv);
  #pragma unroll
          for (int d = 0; d < DIM; ++d) u[d] = F2(ua[d], ub[d]);
        }
        if constexpr (MON) {
          const F2 v = N2::speed(u);
          if (fla && ida != g.skip_id) um = bitmax(um, (double)v.lo());
          if (flb && idb != g.skip_id) um = bitmax(um, (double)v.hi());
        }
        N2::collide(f, S3, u, c2, [&](int i, F2 v) {
          T* o = (T*)pl.out[i] + ida;
          if (fla) o[0] = store_as<T, float>(v.lo());
          if (flb) o[32] = store_as<T, float>(v.hi());
        });
      }
    }
    // this warp is done with stage s
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
    if (++s == kStages) {
      s = 0;
      phase ^= 1u;
    }
  }
  if constexpr (MON) {
    // max over the warp, one atomicMax per warp (the bit patterns of
    // non-negative values order like the values)
    unsigned long long b = (unsigned long long)__double_as_longlong(um);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
      b = x > b ? x : b;
    }
    if (lane == 0) atomicMax(monitor, b);
  }
}

template <int DIM, class T, class R, bool MON>
__global__ void __launch_bounds__(kBlockLP) k_collide_fpu_lp(DevGrid g, CoefR<R> c, DevState st,
                                                              const double* __restrict__ fs,
                                                              const double* __restrict__ ps,
                                                              const double* __restrict__ us,
                                                              T* __restrict__ fout,
                                                              unsigned long long* monitor) {
  using N_ = NodeFast<DIM, R>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  double um = 0.0;  // R-precision |u| (exact in double)
  if (id < g.id_hi) {
    const uint8_t m = st.mask[id];
    if (m & kMaskFluid) {
      R f[N_::Q];
      sfor<0, N_::Q>([&](auto I) { f[I] = (R)fs[(int64_t)I * g.N + id]; });
      R u[DIM];
      sfor<0, DIM>([&](auto K) { u[K] = (R)us[(int64_t)K * g.N + id]; });
      const R S3 = R(3) * (R)ps[id];
      if constexpr (MON) {
        if (id != g.skip_id) um = (double)N_::speed(u);
      }
      N_::collide(f, S3, u, c, [&](int i, R v) { fout[(int64_t)i * g.N + id] = store_as<T, R>(v); });
    }
  }
  if constexpr (MON) block_max_lp(um, monitor);
}

template <int DIM, class T, class R>
__global__ void __launch_bounds__(kBlockLP) k_finalize_lp(DevGrid g, CoefR<R> c, DevState st,
                                                           const T* __restrict__ fin,
                                                           double* __restrict__ fs,
                                                           double* __restrict__ ps,
                                                           double* __restrict__ us) {
  using N_ = NodeFast<DIM, R>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlockLP + threadIdx.x;
  if (id >= g.id_hi) return;
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) return;
  R f[N_::Q];
  sfor<0, N_::Q>([&](auto I) { f[I] = load_as<T, R>(fin + (int64_t)I * g.N + id - g.off[I]); });
  R u[DIM];
  R S3 = N_::moments(f, u, c.inv_rho0);
  N_::dirichlet(m, id, g, st.inlet, S3, u);
  sfor<0, N_::Q>([&](auto I) { fs[(int64_t)I * g.N + id] = (double)f[I]; });
  sfor<0, DIM>([&](auto K) { us[(int64_t)K * g.N + id] = (double)u[K]; });
  ps[id] = (double)(S3 / R(3));
}

// Node value (fluid indicator, p, ux, uy) of a 2D node at (x, y).
template <class T>
__device__ IMX_FI void node_fields(const DevGrid& g, const CoefR<float>& c, const DevState& st,
                                   const T* __restrict__ fin, int x, int y, float (&v)[4]) {
  const int64_t id = (x + kGhost) + g.dy * (y + kGhost);
  const uint8_t m = st.mask[id];
  if (!(m & kMaskFluid)) {
    v[0] = v[1] = v[2] = v[3] = 0.0f;
    return;
  }
  using N_ = NodeFast<2, float>;
  float f[9];
  sfor<0, 9>([&](auto I) { f[I] = Store<T>::to_f(fin[(int64_t)I * g.N + id - g.off[I]]); });
  float u[2];
  float S3 = N_::moments(f, u, c.inv_rho0);
  N_::dirichlet(m, id, g, st.inlet, S3, u);
  v[0] = 1.0f;
  v[1] = S3 * (1.0f / 3.0f);
  v[2] = u[0];
  v[3] = u[1];
}

template <class T>
__global__ void k_sample(DevGrid g, CoefR<float> c, DevState st, int L0, int L1,
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

// fn(T{}, R{}) for the storage kind: narrow kinds compute in float, double
// storage (the fast FP64 option) in double.
template <class F>
cudaError_t dispatch_lp(int store, F&& fn) {
  switch (store) {
    case kStoreF32: return fn(float{}, float{});
    case kStoreBF16: return fn(__nv_bfloat16{}, float{});
    case kStoreF16: return fn(__half{}, float{});
    case kStoreF64: return fn(double{}, double{});
    default: return cudaErrorInvalidValue;
  }
}

// dispatch_lp for the kernels outside the step (first collision after an
// upload, finalize on download), which also serve the fixed-point kind with
// double arithmetic; its step kernel is kernels_fx.cu's.
template <class F>
cudaError_t dispatch_lp_aux(int store, F&& fn) {
  if (store == kStoreFix) return fn(Fix64{}, double{});
  return dispatch_lp(store, std::forward<F>(fn));
}

}  // namespace

cudaError_t launch_collide_fpu_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                                  const DevState& st, const double* f, const double* p,
                                  const double* u, void* fout, unsigned long long* monitor,
                                  cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp_aux(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    T* o = (T*)fout;
    if (dim == 2) {
      if (monitor) k_collide_fpu_lp<2, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<2, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
    } else {
      if (monitor) k_collide_fpu_lp<3, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
      else k_collide_fpu_lp<3, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, f, p, u, o, monitor);
    }
    return cudaGetLastError();
  });
}

namespace {

// Resident k_step_staged blocks on the device (blocks per SM x SMs); 0 when
// the kernel cannot be set up. Set once, outside any stream capture, by
// prepare_step_lp.
template <int DIM, class T, bool MON>
int staged_blocks() {
  static const int n = [] {
    constexpr int Q = NodeFast<DIM, float>::Q;
    const int smem = stage_count<T>() * (int)stage_bytes(Q, kStageTile, sizeof(T));
    auto k = k_step_staged<DIM, T, MON>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return 0;
    int per_sm = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kStageThreads, smem) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
    return per_sm * sms;
  }();
  return n;
}

template <int DIM, class T>
void prepare_staged() {
  (void)staged_blocks<DIM, T, false>();
  (void)staged_blocks<DIM, T, true>();
}

template <int DIM, class T, bool MON>
cudaError_t launch_staged(const DevGrid& g, const CoefR<float>& c, const DevState& st,
                          const DevPlanes& pl, const StagedArgs& sa, unsigned long long* monitor,
                          cudaStream_t s, bool& launched) {
  constexpr int Q = NodeFast<DIM, float>::Q;
  const int blocks = staged_blocks<DIM, T, MON>();
  // the kernel pairs the coefficients by weight class: K_i must be one value
  // per class (it is, from equal weights t_i)
  bool classes = true;
  for (int i = 0; i < Q; ++i) {
    const int n2 = Lattice<DIM>::ex(i) * Lattice<DIM>::ex(i) + Lattice<DIM>::ey(i) * Lattice<DIM>::ey(i) +
                   Lattice<DIM>::ez(i) * Lattice<DIM>::ez(i);
    classes = classes && std::memcmp(&c.k[i], &c.k[class_rep<DIM>(n2)], sizeof(float)) == 0;
  }
  launched = blocks > 0 && classes;
  if (!launched) return cudaSuccess;
  const StagePlan sp = make_stage_plan<Q>(g, st, pl, sa, kStageTile, sizeof(T));

  const unsigned grid = (unsigned)(sp.ntiles < blocks ? sp.ntiles : blocks);
  const bool bgroups = st.bnd && sa.n_groups > 0;  // (only the fused boundary handling has them)
  cudaError_t e = cudaSuccess;
  if (bgroups) e = cudaEventRecord(sa.fork, s);
  if (e != cudaSuccess) return e;
  k_step_staged<DIM, T, MON><<<grid, kStageThreads, stage_count<T>() * stage_bytes(Q, kStageTile, sizeof(T)), s>>>(
      g, c, st, pl, sp, monitor);
  if (bgroups) {
    // beside the staged kernel on the second stream, joined before the step ends
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamWaitEvent(sa.side, sa.fork, 0)) != cudaSuccess)
      return e;
    constexpr int per_block = kBlockLP / kStageGroup;
    k_step_bgroups<DIM, T, MON>
        <<<(unsigned)((sa.n_groups + per_block - 1) / per_block), kBlockLP, 0, sa.side>>>(
            g, c, st, pl, sa.groups, sa.n_groups, monitor);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaEventRecord(sa.join, sa.side)) != cudaSuccess)
      return e;
    return cudaStreamWaitEvent(s, sa.join, 0);
  }
  return cudaGetLastError();
}

}  // namespace

void prepare_step_lp() {
  prepare_staged<3, __half>();
  prepare_staged<3, __nv_bfloat16>();
}


cudaError_t launch_step_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                           const DevState& st, const DevPlanes& pl, unsigned long long* monitor,
                           cudaStream_t s, const StagedArgs* sa) {
  const unsigned grid = grid_lp(g);
  // D3Q27 only: on D2Q9 lattices (9 runs a tile) the register kernel is as
  // fast (cylinder 1024x512 FP16: 0.0117 against 0.0121 ms). A fused step
  // needs the boundary-group list (n_groups < 0: not made).
  const bool staged =
      dim == 3 && sa != nullptr && stage_fits(g, kStageTile) && (!st.bnd || sa->n_groups >= 0);
  return dispatch_lp(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    if constexpr (sizeof(T) == 2) {
      if (staged) {
        bool launched = false;
        const cudaError_t e =
            monitor ? launch_staged<3, T, true>(g, cr, st, pl, *sa, monitor, s, launched)
                    : launch_staged<3, T, false>(g, cr, st, pl, *sa, monitor, s, launched);
        if (e != cudaSuccess || launched) return e;
      }
    }
    if (dim == 2) {
      if (monitor) k_step_lp<2, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
      else k_step_lp<2, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
    } else {
      if (monitor) k_step_lp<3, T, R, true><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
      else k_step_lp<3, T, R, false><<<grid, kBlockLP, 0, s>>>(g, cr, st, pl, monitor);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_finalize_lp(int dim, int store, const DevGrid& g, const DevCoefLP& c,
                               const DevState& st, const void* fin, double* f, double* p,
                               double* u, cudaStream_t s) {
  const unsigned grid = grid_lp(g);
  return dispatch_lp_aux(store, [&](auto tag, auto rtag) {
    using T = decltype(tag);
    using R = decltype(rtag);
    const CoefR<R>& cr = c.get<R>();
    if (dim == 2) k_finalize_lp<2, T, R><<<grid, kBlockLP, 0, s>>>(g, cr, st, (const T*)fin, f, p, u);
    else k_finalize_lp<3, T, R><<<grid, kBlockLP, 0, s>>>(g, cr, st, (const T*)fin, f, p, u);
    return cudaGetLastError();
  });
}

cudaError_t launch_sample(int store, const DevGrid& g, const DevCoefLP& c, const DevState& st,
                          int L0, int L1, const void* fin, int W, int H, float* out,
                          cudaStream_t s) {
  const dim3 grid((unsigned)((W + 127) / 128), (unsigned)H);
  return dispatch_store(store, [&](auto tag) {
    using T = decltype(tag);
    k_sample<T><<<grid, 128, 0, s>>>(g, c.f, st, L0, L1, (const T*)fin, W, H, out);
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

}  // namespace imx
