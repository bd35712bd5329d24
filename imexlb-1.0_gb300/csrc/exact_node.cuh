// Reference-rounding FP64 node update and the fused step kernel, shared by
// the translation units that instantiate it (kernels.cu; step_split2.cu and
// step_split3.cu hold the variants that move FP64 work to the integer pipes).
//
// Every floating-point operation is an explicit round-to-nearest operation in
// the evaluation order of lbm.f90 (Collision lbm.f90:64-72, PostProcessing
// lbm.f90:166-179), so no multiply-add is ever fused and results equal the
// reference's serial build. Terms the reference multiplies by an integer
// lattice component in {-1,0,1} are added, subtracted or skipped; that is
// exact (it can change only the sign of an exact zero). A +/- direction pair
// shares |e.u|, e.u squared and 4.5(e.u)^2, which are exactly equal for the
// two members (e_opp = -e).
//
// GB300 has ~0.5 T FP64 add/mul per second against ~7 TB/s of HBM, so these
// kernels are bound by FP64 issue, not memory; the work per node is kept to
// the reference's own operation count, and part of it can run as integer
// emulation of the same IEEE operations (fp64_emu.cuh).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "fp64_emu.cuh"
#include "kernels.h"
#include "lattice.h"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kBlock = 128;

// Which FP64 operations of the node update run on the integer pipes
// (fp64_emu.cuh): bit j (j < 13) = the operations of direction pair j (e.u,
// its square terms, both equilibria and both collisions), then the rest
// direction, the density sum, the three momentum sums, and u.u with 3p and
// 1.5 u.u, and the division by 3 of the density sum. kEmMulsOnly /
// kEmAddsOnly restrict the pair, rest and u.u groups to their
// multiplications / additions. With kFmaForm the operations left on the FP64
// pipe are issued as fused multiply-adds with the exact operands of DevCoef
// (GB300 issues DFMA about 19% faster than DADD or DMUL). The results are the
// same bits for every mask.
constexpr uint32_t kEmRest = 1u << 13;
constexpr uint32_t kEmP = 1u << 14;
constexpr uint32_t kEmU = 1u << 15;  // << k for component k
constexpr uint32_t kEmUdu = 1u << 18;
constexpr uint32_t kEmMulsOnly = 1u << 19;
constexpr uint32_t kEmAddsOnly = 1u << 20;
constexpr uint32_t kEmDiv3 = 1u << 21;  // p = sum / 3
constexpr uint32_t kFmaForm = 1u << 22;  // FP64 adds and multiplies not emulated run as DFMA
constexpr uint32_t kEmConstMuls = 1u << 23;  // every multiplication by 3, 1.5 or 4.5
constexpr uint32_t kReloadF = 1u << 24;  // collision re-reads f (L1) instead of holding it
constexpr uint32_t kMinBlocks6 = 1u << 25;  // register cap for 6 resident blocks per SM
constexpr uint32_t kMinBlocks8 = 1u << 26;  // register cap for 8 resident blocks per SM
// Warp split: the last n warps of each block (n = (EM >> 27) & 3) compute
// their nodes entirely in integer emulation while the others use the FP64
// pipe with the rest of the mask.
constexpr uint32_t kEmWarpShift = 27;
template <int DIM>
constexpr uint32_t kFullEmu = (DIM == 3 ? 0x1fffu : 0xfu) | kEmRest | kEmUdu | kEmP | (7u << 15) | kEmDiv3 | kReloadF;

template <int DIM, bool RHO1, uint32_t EM = 0>
struct Node {
  using Lat = Lattice<DIM>;
  static constexpr int Q = Lat::Q;

  IMX_HD static constexpr bool em(uint32_t bit) { return (EM & bit) != 0u; }
  // Index of the +/- pair of direction iq among the representatives.
  IMX_HD static constexpr int pair_of(int iq) {
    const int r = Lat::is_rep(iq) ? iq : Lat::opp(iq);
    int n = 0;
    for (int k = 0; k < r; ++k) n += Lat::is_rep(k) ? 1 : 0;
    return n;
  }
  IMX_HD static constexpr uint32_t flag_of(int iq) { return iq == Lat::REST ? kEmRest : 1u << pair_of(iq); }

  template <bool E>
  __device__ static IMX_FI double add(const DevCoef& c, double a, double b) {
    if constexpr (E) return emu::dadd(a, b);
    else if constexpr (em(kFmaForm)) return __fma_rn(a, c.one, b);
    else return __dadd_rn(a, b);
  }
  template <bool E>
  __device__ static IMX_FI double sub(const DevCoef& c, double a, double b) {
    if constexpr (E) return emu::dsub(a, b);
    else if constexpr (em(kFmaForm)) return __fma_rn(b, c.mone, a);
    else return __dsub_rn(a, b);
  }
  template <bool E>
  __device__ static IMX_FI double mul(const DevCoef& c, double a, double b) {
    if constexpr (E) return emu::dmul(a, b);
    else if constexpr (em(kFmaForm)) return __fma_rn(a, b, c.mzero);
    else return __dmul_rn(a, b);
  }
  // the same inside the pair, rest and u.u groups
  template <bool E>
  __device__ static IMX_FI double gadd(const DevCoef& c, double a, double b) {
    return add<E && !em(kEmMulsOnly)>(c, a, b);
  }
  template <bool E>
  __device__ static IMX_FI double gsub(const DevCoef& c, double a, double b) {
    return sub<E && !em(kEmMulsOnly)>(c, a, b);
  }
  template <bool E>
  __device__ static IMX_FI double gmul(const DevCoef& c, double a, double b) {
    return mul<E && !em(kEmAddsOnly)>(c, a, b);
  }
  // x * (K * 2^S) (3, 1.5, 4.5) inside the groups
  template <bool E, int K, int S>
  __device__ static IMX_FI double gmulc(const DevCoef& c, double x) {
    if constexpr ((E && !em(kEmAddsOnly)) || em(kEmConstMuls)) {
      return emu::mul_small<K, S>(x);
    } else {
      constexpr double k = S >= 0 ? (double)(K << (S >= 0 ? S : 0)) : (double)K / (double)(1 << (S < 0 ? -S : 0));
      return mul<false>(c, k, x);
    }
  }

  // PostProcessing moments of one node (lbm.f90:166-179): p = sum(f)/3,
  // u_k = sum(f*e_k)/rho0, summed in iq order; *geo(id) = *1 on fluid nodes.
  __device__ static IMX_FI void moments(const double (&f)[Q], double& p, double (&u)[DIM],
                                        const DevCoef& c) {
    constexpr bool EP = em(kEmP);
    double s = f[0];
    sfor<1, Q>([&](auto I) { s = add<EP>(c, s, f[I]); });
    if constexpr (em(kEmDiv3)) p = emu::div3(s);
    else p = __ddiv_rn(s, 3.0);
    sfor<0, DIM>([&](auto K) {
      constexpr int k = K;
      constexpr bool EU = em(kEmU << k);
      constexpr int i0 = Lat::first_nz(k);
      double m = Lat::e(i0, k) > 0 ? f[i0] : -f[i0];
      sfor<i0 + 1, Q>([&](auto I) {
        constexpr int ck = Lat::e(I, k);
        if constexpr (ck > 0) m = add<EU>(c, m, f[I]);
        else if constexpr (ck < 0) m = sub<EU>(c, m, f[I]);
      });
      if constexpr (!RHO1) m = __ddiv_rn(m, c.rho0);
      u[k] = m;
    });
  }

  // e.u for a representative direction (first non-zero component +1),
  // summed in component order as edu = edu + e(iq*dim+ind)*u(...) does.
  template <int I, bool E>
  __device__ static IMX_FI double edu(const DevCoef& c, const double (&u)[DIM]) {
    constexpr int k0 = Lat::first_comp(I);
    double s = u[k0];
    sfor<k0 + 1, DIM>([&](auto K) {
      constexpr int ck = Lat::e(I, K);
      if constexpr (ck > 0) s = gadd<E>(c, s, u[K]);
      else if constexpr (ck < 0) s = gsub<E>(c, s, u[K]);
    });
    return s;
  }

  template <bool E>
  __device__ static IMX_FI double udu(const DevCoef& c, const double (&u)[DIM]) {
    double s = gmul<E>(c, u[0], u[0]);
    s = gadd<E>(c, s, gmul<E>(c, u[1], u[1]));
    if constexpr (DIM == 3) s = gadd<E>(c, s, gmul<E>(c, u[2], u[2]));
    return s;
  }

  // feq = t*(p*3 + rho0*((3*edu + 4.5*edu^2) - 1.5*udu)), given
  // s = 3*edu + 4.5*edu^2 (lbm.f90:70).
  template <bool E>
  __device__ static IMX_FI double feq(const DevCoef& c, double t, double p3, double h, double s) {
    double v = gsub<E>(c, s, h);
    if constexpr (!RHO1) v = gmul<E>(c, c.rho0, v);
    return gmul<E>(c, t, gadd<E>(c, p3, v));
  }

  // Visit every direction with its equilibrium value: fn(IC<iq>, feq).
  template <class F>
  __device__ static IMX_FI void equilibria(double p, const double (&u)[DIM], const DevCoef& c,
                                           F&& fn) {
    constexpr bool EH = em(kEmUdu);
    const double p3 = gmulc<EH, 3, 0>(c, p);
    const double h = gmulc<EH, 3, -1>(c, udu<EH>(c, u));
    {  // rest direction: edu = +0, so 3*edu + 4.5*edu^2 - 1.5*udu = -h
      constexpr int r = Lat::REST;
      constexpr bool ER = em(kEmRest);
      double v = -h;
      if constexpr (!RHO1) v = gmul<ER>(c, c.rho0, v);
      fn(IC<r>{}, gmul<ER>(c, c.t[r], gadd<ER>(c, p3, v)));
    }
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        constexpr bool E = em(flag_of(i));
        const double e = edu<i, E>(c, u);
        const double a = gmulc<E, 3, 0>(c, e);
        const double q = gmulc<E, 9, -1>(c, gmul<E>(c, e, e));
        fn(IC<i>{}, feq<E>(c, c.t[i], p3, h, gadd<E>(c, a, q)));
        fn(IC<o>{}, feq<E>(c, c.t[o], p3, h, gsub<E>(c, q, a)));  // (-3edu) + 4.5edu^2
      }
    });
  }

  // Collision (lbm.f90:71): fb = (1-ome)*f + ome*feq, stored SoA.
  __device__ static IMX_FI void collide(const double (&f)[Q], double p, const double (&u)[DIM],
                                        const DevCoef& c, double* __restrict__ out, int64_t N,
                                        int64_t id) {
    equilibria(p, u, c, [&](auto I, double fe) {
      constexpr int i = I;
      constexpr bool E = em(flag_of(i));
      out[(int64_t)i * N + id] = gadd<E>(c, gmul<E>(c, c.om1, f[i]), gmul<E>(c, c.ome, fe));
    });
  }

  // The same with each f_i read again from memory (an L1 / L2 hit: the pull
  // read it a moment before), so that the 27 values need no registers
  // through the equilibrium arithmetic.
  __device__ static IMX_FI void collide_reload(double p, const double (&u)[DIM], const DevCoef& c,
                                               const double* __restrict__ fin, const DevGrid& g,
                                               double* __restrict__ out, int64_t id) {
    equilibria(p, u, c, [&](auto I, double fe) {
      constexpr int i = I;
      constexpr bool E = em(flag_of(i));
      double fi;
      asm volatile("ld.global.ca.f64 %0, [%1];" : "=d"(fi) : "l"(fin + ((int64_t)i * g.N + id - g.off[i])));
      out[(int64_t)i * g.N + id] = gadd<E>(c, gmul<E>(c, c.om1, fi), gmul<E>(c, c.ome, fe));
    });
  }

  __device__ static IMX_FI void pull(const double* __restrict__ fin, const DevGrid& g, int64_t id,
                                     double (&f)[Q]) {
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      f[i] = fin[(int64_t)i * g.N + id - g.off[i]];
    });
  }

  // Dirichlet conditions of PostProcessing (lbm.f90:185-198) on a fluid node.
  __device__ static IMX_FI void dirichlet(uint8_t m, int64_t id, const DevGrid& g,
                                          const double* inlet, double& p, double (&u)[DIM]) {
    if (m & kMaskInlet) {
      const int64_t r = DIM == 2 ? id / g.dy : id / g.dz;
      u[0] = inlet[r];
      u[1] = 0.0;
    }
    if (m & kMaskOutlet) p = 0.0;
  }
};

// Non-negative doubles order like their bit patterns (NaN above +inf).
template <int NT = kBlock>
__device__ IMX_FI void block_max_bits(unsigned long long b, unsigned long long* dst) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  __shared__ unsigned long long wmax[NT / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wmax[w] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = wmax[0];
    for (int i = 1; i < NT / 32; ++i) m = wmax[i] > m ? wmax[i] : m;
    atomicMax(dst, m);
  }
}

__device__ IMX_FI void block_max_to(double v, unsigned long long* dst) {
  block_max_bits<kBlock>((unsigned long long)__double_as_longlong(v), dst);
}

__device__ IMX_FI double speed2d(double ux, double uy) {
  return __dsqrt_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)));
}

template <uint32_t EM>
constexpr int min_blocks() {
  return (EM & kMinBlocks8) ? 8 : (EM & kMinBlocks6) ? 6 : 0;  // 0: no minimum
}

// One node of the fused iteration; returns its Monitor speed (or 0).
template <int DIM, bool RHO1, bool MON, uint32_t EM>
__device__ IMX_FI double step_node(const DevGrid& g, const DevCoef& c, const DevState& st,
                                   const double* __restrict__ fin, double* __restrict__ fout,
                                   int64_t id) {
  using N_ = Node<DIM, RHO1, EM>;
  double um = 0.0;
  const uint8_t m = st.mask[id];
  if (m & kMaskFluid) {
    double f[N_::Q];
    N_::pull(fin, g, id, f);
    double p, u[DIM];
    N_::moments(f, p, u, c);
    N_::dirichlet(m, id, g, st.inlet, p, u);
    if constexpr (MON) {
      if (id != g.skip_id) um = speed2d(u[0], u[1]);
    }
    if constexpr ((EM & kReloadF) != 0u) N_::collide_reload(p, u, c, fin, g, fout, id);
    else N_::collide(f, p, u, c, fout, g.N, id);
  }
  return um;
}

template <int DIM, bool RHO1, bool MON, uint32_t EM = 0>
__global__ void __launch_bounds__(kBlock, min_blocks<EM>()) k_step(DevGrid g, DevCoef c, DevState st,
                                                  const double* __restrict__ fin,
                                                  double* __restrict__ fout,
                                                  unsigned long long* monitor) {
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlock + threadIdx.x;
  constexpr int kEmuWarps = (int)((EM >> kEmWarpShift) & 3u);
  constexpr uint32_t kHw = EM & ~(3u << kEmWarpShift);
  double um = 0.0;
  if (id < g.id_hi) {
    if constexpr (kEmuWarps > 0) {
      if ((int)(threadIdx.x >> 5) >= kBlock / 32 - kEmuWarps)
        um = step_node<DIM, RHO1, MON, kFullEmu<DIM>>(g, c, st, fin, fout, id);
      else
        um = step_node<DIM, RHO1, MON, kHw>(g, c, st, fin, fout, id);
    } else {
      um = step_node<DIM, RHO1, MON, kHw>(g, c, st, fin, fout, id);
    }
  }
  if constexpr (MON) block_max_to(um, monitor);
}

// Persistent form: a grid of resident blocks whose warps take 32-node chunks
// until none is left. With kEmWarps n > 0, the last n warps of each block
// compute their chunks entirely in integer emulation (kFullEmu) and the
// others on the FP64 pipe, so both kinds of pipe work at once; every warp
// runs at its own pace. One 64-bit word counts the chunks taken from the
// front (low half, FP64 warps) and from the back (high half, emulating
// warps); a chunk is valid while front + back < nchunks, so the two ends
// never overlap and every chunk is taken once. Emulating warps stop while
// `reserve` chunks remain, leaving the tail to the faster FP64 warps. The
// last warp to finish zeroes the counters for the next launch.
constexpr uint32_t kPersist = 1u << 29;
constexpr int kPBlock = 256;
constexpr int kEmuRetries = 64;  // bounded compare-and-swap attempts per fetch

template <int DIM, bool MON, uint32_t EM>
__global__ void __launch_bounds__(kPBlock, 2) k_step_persist(DevGrid g, DevCoef c, DevState st,
                                                          const double* __restrict__ fin,
                                                          double* __restrict__ fout,
                                                          unsigned long long* monitor,
                                                          uint32_t nchunks, uint32_t reserve) {
  constexpr int kEW = (int)((EM >> kEmWarpShift) & 3u);
  constexpr uint32_t kHw = EM & ~((3u << kEmWarpShift) | kPersist);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long* work = st.work;
  unsigned long long ub = 0;  // Monitor: bit-pattern max of the node speeds
  if (warp >= kPBlock / 32 - kEW) {
    for (;;) {
      long long chunk = -1;
      if (lane == 0) {
        unsigned long long old = atomicAdd(work, 0ull);
        for (int r = 0; r < kEmuRetries; ++r) {
          const uint32_t F = (uint32_t)old, B = (uint32_t)(old >> 32);
          if ((uint64_t)F + B + reserve >= nchunks) break;
          const unsigned long long seen = atomicCAS(work, old, old + (1ull << 32));
          if (seen == old) {
            chunk = (long long)nchunks - 1 - B;
            break;
          }
          old = seen;
        }
      }
      chunk = __shfl_sync(0xffffffffu, chunk, 0);
      if (chunk < 0) break;
      const int64_t id = g.id_lo + chunk * 32 + lane;
      if (id < g.id_hi) {
        const double v = step_node<DIM, true, MON, kFullEmu<DIM>>(g, c, st, fin, fout, id);
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        ub = b > ub ? b : ub;
      }
    }
  } else {
    for (;;) {
      long long chunk = -1;
      if (lane == 0) {
        const unsigned long long old = atomicAdd(work, 1ull);
        const uint32_t F = (uint32_t)old, B = (uint32_t)(old >> 32);
        if ((uint64_t)F + B < nchunks) chunk = F;
      }
      chunk = __shfl_sync(0xffffffffu, chunk, 0);
      if (chunk < 0) break;
      const int64_t id = g.id_lo + chunk * 32 + lane;
      if (id < g.id_hi) {
        const double v = step_node<DIM, true, MON, kHw>(g, c, st, fin, fout, id);
        const unsigned long long b = (unsigned long long)__double_as_longlong(v);
        ub = b > ub ? b : ub;
      }
    }
  }
  if (lane == 0) {
    __threadfence();
    const unsigned long long nwarps = (unsigned long long)gridDim.x * (kPBlock / 32);
    if (atomicAdd(work + 1, 1ull) == nwarps - 1) {
      work[0] = 0ull;
      work[1] = 0ull;
      __threadfence();
    }
  }
  if constexpr (MON) block_max_bits<kPBlock>(ub, monitor);
}

template <int DIM, bool MON, uint32_t EM>
cudaError_t launch_persist(const DevGrid& g, const DevCoef& c, const DevState& st, const double* fin,
                           double* fout, unsigned long long* monitor, cudaStream_t s) {
  if (st.work == nullptr) return cudaErrorInvalidValue;
  const int64_t nodes = g.id_hi - g.id_lo;
  const int64_t nchunks = (nodes + 31) / 32;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_persist<DIM, MON, EM>, kPBlock, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (int64_t)sms * per_sm;
  const int64_t needed = (nchunks + kPBlock / 32 - 1) / (kPBlock / 32);
  if (blocks > needed) blocks = needed;
  if (blocks < 1) blocks = 1;
  // counters: front + back stays below 2^32 (each warp overshoots by at most one)
  if (nchunks + blocks * (kPBlock / 32) >= (int64_t)UINT32_MAX) return cudaErrorInvalidValue;
  constexpr int kEW = (int)((EM >> kEmWarpShift) & 3u);
  const uint32_t reserve = (uint32_t)(blocks * (kPBlock / 32 - kEW));
  k_step_persist<DIM, MON, EM><<<(unsigned)blocks, kPBlock, 0, s>>>(g, c, st, fin, fout, monitor,
                                                                    (uint32_t)nchunks, reserve);
  return cudaGetLastError();
}

// Masks of the step-kernel variants, by split index (rho0 = 1).
template <int DIM>
struct Splits {
  static constexpr uint32_t kPairs = DIM == 3 ? 0x1fffu : 0xfu;
  static constexpr uint32_t kAll = kPairs | kEmRest | kEmUdu;
  static constexpr uint32_t F = kFmaForm, D = kEmDiv3, M = kEmMulsOnly;
  static constexpr uint32_t AM = F | D | kAll | M;  // every multiplication emulated
  static constexpr uint32_t v[] = {0u,
                                   F | D,
                                   AM,
                                   D | kAll | M,
                                   AM | kReloadF,
                                   D | kAll | M | kReloadF,
                                   AM | kMinBlocks6,
                                   AM | kReloadF | kMinBlocks6,
                                   AM | kReloadF | kMinBlocks8,
                                   kPersist | AM,
                                   AM | kEmP,
                                   AM | kEmU};
  static constexpr int n = 12;
  // fastest on GB300 (D3Q27 256x128x128 and D2Q9 1024x512 sweeps)
  static constexpr int kDefault = 2;  // AM
};
static_assert(Splits<2>::n == Splits<3>::n, "one split index space");

// Launch variant `split` (recursion over the compile-time table).
template <int DIM, bool MON, int V = 0>
cudaError_t launch_step_variant(int split, unsigned grid, const DevGrid& g, const DevCoef& c,
                                const DevState& st, const double* fin, double* fout,
                                unsigned long long* monitor, cudaStream_t s) {
  if constexpr (V < Splits<DIM>::n) {
    if (split != V)
      return launch_step_variant<DIM, MON, V + 1>(split, grid, g, c, st, fin, fout, monitor, s);
    constexpr uint32_t em = Splits<DIM>::v[V];
    if constexpr ((em & kPersist) != 0u) {
      return launch_persist<DIM, MON, em>(g, c, st, fin, fout, monitor, s);
    } else {
      k_step<DIM, true, MON, em><<<grid, kBlock, 0, s>>>(g, c, st, fin, fout, monitor);
      return cudaGetLastError();
    }
  } else {
    return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace imx
