// Reference-rounding FP64 node update and the fused step kernel, shared by
// the translation units that instantiate it (kernels.cu; step_split2.cu and
// step_split3.cu hold the variants that move FP64 work off the FP64 pipe).
//
// Every floating-point operation is an explicit round-to-nearest operation in
// the evaluation order of lbm.f90 (Collision lbm.f90:64-72, PostProcessing
// lbm.f90:166-179), so nothing is contracted and results equal the
// reference's serial build. Terms the reference multiplies by an integer
// lattice component in {-1,0,1} are added, subtracted or skipped; that is
// exact (it can change only the sign of an exact zero). A +/- direction pair
// shares |e.u|, e.u squared and 4.5(e.u)^2, which are exactly equal for the
// two members (e_opp = -e).
//
// GB300 issues ~0.5 T FP64 add/mul (0.6 T fused multiply-add) per second
// against ~7 TB/s of HBM, so these kernels are bound by the FP64 pipe, not by
// memory. Three exact devices move work off it without changing a bit:
//  - kFmaForm: additions and multiplications left on the FP64 pipe are
//    issued as fused multiply-adds with exact operands (a*1+b, b*(-1)+a,
//    a*b+(-0); DevCoef::one, mone, mzero), which GB300 issues ~19% faster;
//  - group emulation (bits 0-18, kEmDiv3): operations computed by the
//    integer IEEE emulation of fp64_emu.cuh (multiplications only under
//    kEmMulsOnly; emulated additions cost more than they save);
//  - kLoopPairs: the collision of the direction pairs as a run-time loop,
//    so that the long emulated multiplications are not unrolled Q/2 times
//    past the instruction cache.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "boundary_fused.cuh"
#include "fp64_emu.cuh"
#include "kernels.h"
#include "lattice.h"
#include "storage.cuh"

namespace imx {
namespace {

constexpr int kBlock = 128;

// Mask bits of a step-kernel variant. Bit j (j < 13): the operations of
// direction pair j (e.u, its square terms, both equilibria and both
// collisions; with kLoopPairs bit 0 stands for every pair); then the rest
// direction, the density sum, the three momentum sums, and u.u with 3p and
// 1.5 u.u. The results are the same bits for every mask.
constexpr uint32_t kEmRest = 1u << 13;
constexpr uint32_t kEmP = 1u << 14;
constexpr uint32_t kEmU = 1u << 15;  // << k for component k
constexpr uint32_t kEmUdu = 1u << 18;
constexpr uint32_t kEmMulsOnly = 1u << 19;  // groups emulate their multiplications only
constexpr uint32_t kEmDiv3 = 1u << 20;      // p = sum / 3 in integer arithmetic
constexpr uint32_t kFmaForm = 1u << 21;     // FP64-pipe operations issued as DFMA
constexpr uint32_t kLoopPairs = 1u << 22;   // run-time loop over the direction pairs

// -x as a flip of the sign bit on the integer pipe (IEEE negation is exactly
// that). Written as integer PTX so that it does not become an FP64
// instruction on the busy FP64 pipe.
__device__ IMX_FI double neg(double x) {
  double r;
  asm("{\n\t.reg .b32 lo, hi;\n\tmov.b64 {lo, hi}, %1;\n\txor.b32 hi, hi, 0x80000000;\n\t"
      "mov.b64 %0, {lo, hi};\n\t}"
      : "=d"(r)
      : "d"(x));
  return r;
}

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
  IMX_HD static constexpr uint32_t flag_of(int iq) {
    return iq == Lat::REST ? kEmRest : 1u << pair_of(iq);
  }

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
  // additions inside an emulated group stay on the FP64 pipe under kEmMulsOnly
  template <bool E>
  __device__ static IMX_FI double gadd(const DevCoef& c, double a, double b) {
    return add<E && !em(kEmMulsOnly)>(c, a, b);
  }
  template <bool E>
  __device__ static IMX_FI double gsub(const DevCoef& c, double a, double b) {
    return sub<E && !em(kEmMulsOnly)>(c, a, b);
  }
  // x * (K * 2^S): the constants 3, 1.5 and 4.5
  template <bool E, int K, int S>
  __device__ static IMX_FI double mulc(const DevCoef& c, double x) {
    if constexpr (E) {
      return emu::mul_small<K, S>(x);
    } else {
      constexpr double k = S >= 0 ? (double)(K << (S >= 0 ? S : 0))
                                  : (double)K / (double)(1 << (S < 0 ? -S : 0));
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
      double m = Lat::e(i0, k) > 0 ? f[i0] : neg(f[i0]);
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
    double s = mul<E>(c, u[0], u[0]);
    s = gadd<E>(c, s, mul<E>(c, u[1], u[1]));
    if constexpr (DIM == 3) s = gadd<E>(c, s, mul<E>(c, u[2], u[2]));
    return s;
  }

  // feq = t*(p*3 + rho0*((3*edu + 4.5*edu^2) - 1.5*udu)), given
  // s = 3*edu + 4.5*edu^2 (lbm.f90:70).
  template <bool E>
  __device__ static IMX_FI double feq(const DevCoef& c, double t, double p3, double h, double s) {
    double v = gsub<E>(c, s, h);
    if constexpr (!RHO1) v = mul<E>(c, c.rho0, v);
    return mul<E>(c, t, gadd<E>(c, p3, v));
  }

  // 3p and 1.5 u.u, shared by every direction.
  __device__ static IMX_FI void common(double p, const double (&u)[DIM], const DevCoef& c,
                                       double& p3, double& h) {
    constexpr bool EH = em(kEmUdu);
    p3 = mulc<EH, 3, 0>(c, p);
    h = mulc<EH, 3, -1>(c, udu<EH>(c, u));
  }

  // rest direction: edu = +0, so 3*edu + 4.5*edu^2 - 1.5*udu = -h, and
  // p3 + (-h) is p3 - h
  __device__ static IMX_FI double feq_rest(const DevCoef& c, double p3, double h) {
    constexpr int r = Lat::REST;
    constexpr bool ER = em(kEmRest);
    if constexpr (!RHO1) return mul<ER>(c, c.t[r], gadd<ER>(c, p3, mul<ER>(c, c.rho0, neg(h))));
    else return mul<ER>(c, c.t[r], gsub<ER>(c, p3, h));
  }

  // Visit every direction with its equilibrium value: fn(IC<iq>, feq).
  template <class F>
  __device__ static IMX_FI void equilibria(double p, const double (&u)[DIM], const DevCoef& c,
                                           F&& fn) {
    double p3, h;
    common(p, u, c, p3, h);
    fn(IC<Lat::REST>{}, feq_rest(c, p3, h));
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        constexpr bool E = em(flag_of(i));
        const double e = edu<i, E>(c, u);
        const double a = mulc<E, 3, 0>(c, e);
        const double q = mulc<E, 9, -1>(c, mul<E>(c, e, e));
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
      out[(int64_t)i * N + id] = gadd<E>(c, mul<E>(c, c.om1, f[i]), mul<E>(c, c.ome, fe));
    });
  }

  // The collision as a run-time loop over the +/- pairs (kLoopPairs): one
  // compact body instead of Q/2 unrolled copies. The loop visits one member
  // i of every pair (the upper half of the ordering; any member works: e.u
  // of the other is exactly -e.u, so its 3e.u + 4.5(e.u)^2 is q - a). Its
  // weight and pull offset come from per-handle tables (warp-uniform
  // loads); f_i is read again (an L1 / L2 hit: the pull read it a moment
  // before) rather than kept in 27 registers; e.u is built with the exact
  // operations of edu() (adding -u is subtracting u).
  // FX: boundary copies folded into the step (boundary_fused.cuh); f_i is
  // read again where the fused pull read it.
  template <bool FX>
  __device__ static IMX_FI void collide_loop(double p, const double (&u)[DIM], const DevCoef& c,
                                             const DevState& st, const double* __restrict__ fin,
                                             const DevGrid& g, double* __restrict__ out,
                                             int64_t id, const PullFix& fx) {
    constexpr bool E = em(1u);
    constexpr bool ER = em(kEmRest);
    double p3, h;
    common(p, u, c, p3, h);
    // closed-form boundary nodes read their pull offsets from the table of
    // their kind (no extra work in the loop); record nodes from their row
    const int64_t* oq = st.offq;
    const uint32_t* row = nullptr;
    if constexpr (FX) {
      if (fx.record()) row = PullFix::row<Q>(st, id);
      else if (fx.bits) oq = st.offq_kind + fx.kind() * Q;
    }
    auto reload = [&](int i, int64_t off) {
      int64_t a = (int64_t)i * g.N + id - off;
      if constexpr (FX) {
        if (row) {
          const uint32_t r = row[i];
          if (r != kNoRedirect) a = r;
        }
      }
      double v;
      asm volatile("ld.global.ca.f64 %0, [%1];" : "=d"(v) : "l"(fin + a));
      return v;
    };
    {
      constexpr int r = Lat::REST;
      const double fr = reload(r, g.off[r]);
      out[(int64_t)r * g.N + id] =
          gadd<ER>(c, mul<ER>(c, c.om1, fr), mul<ER>(c, c.ome, feq_rest(c, p3, h)));
    }
    // one member i of a pair per call (one pair per loop iteration: two or
    // three per iteration were measured slower)
    auto pair = [&](int i) {
      const int o = Q - 1 - i;
      double e = 0.0;
      bool started = false;
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const int ek = Lat::e(i, k);
        if (ek != 0) {
          const double v = ek > 0 ? u[k] : neg(u[k]);
          e = started ? gadd<E>(c, e, v) : v;
          started = true;
        }
      }
      const double t = __ldg(st.tq + i);
      const double a = mulc<E, 3, 0>(c, e);
      const double q = mulc<E, 9, -1>(c, mul<E>(c, e, e));
      const double fei = feq<E>(c, t, p3, h, gadd<E>(c, a, q));
      const double feo = feq<E>(c, t, p3, h, gsub<E>(c, q, a));
      const double fi = reload(i, __ldg(oq + i));
      const double fo = reload(o, __ldg(oq + o));
      out[(int64_t)i * g.N + id] = gadd<E>(c, mul<E>(c, c.om1, fi), mul<E>(c, c.ome, fei));
      out[(int64_t)o * g.N + id] = gadd<E>(c, mul<E>(c, c.om1, fo), mul<E>(c, c.ome, feo));
    };
#pragma unroll 1
    for (int i = Lat::REST + 1; i < Q; ++i) pair(i);
  }

  __device__ static IMX_FI void pull(const double* __restrict__ fin, const DevGrid& g, int64_t id,
                                     double (&f)[Q]) {
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      f[i] = fin[(int64_t)i * g.N + id - g.off[i]];
    });
  }

  // The pull of a step with the boundary copies folded in (boundary_fused.cuh).
  // `bwarp`: some node of the warp is next to the rim or an obstacle; then
  // every node of the warp reads its offsets from a table (the plain one, or
  // the one of its kind) or its record's row, else the plain pull.
  __device__ static IMX_FI void pull_fixed(const double* __restrict__ fin, const DevGrid& g,
                                           const DevState& st, int64_t id, const PullFix& fx,
                                           bool bwarp, double (&f)[Q]) {
    if (!bwarp) {
      pull(fin, g, id, f);
    } else if (!fx.record()) {
      const int64_t* oq = fx.bits ? st.offq_kind + fx.kind() * Q : st.offq;
      sfor<0, Q>([&](auto I) {
        constexpr int i = I;
        f[i] = fin[(int64_t)i * g.N + id - __ldg(oq + i)];
      });
    } else {
      const uint32_t* row = PullFix::row<Q>(st, id);
      sfor<0, Q>([&](auto I) {
        constexpr int i = I;
        const uint32_t r = row[i];
        f[i] = fin[r != kNoRedirect ? (int64_t)r : (int64_t)i * g.N + id - g.off[i]];
      });
    }
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
__device__ IMX_FI void block_max_to(double v, unsigned long long* dst) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  __shared__ unsigned long long wmax[kBlock / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wmax[w] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = wmax[0];
    for (int i = 1; i < kBlock / 32; ++i) m = wmax[i] > m ? wmax[i] : m;
    atomicMax(dst, m);
  }
}

__device__ IMX_FI double speed2d(double ux, double uy) {
  return __dsqrt_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)));
}

// Resident blocks per SM a variant is compiled for (0: no minimum). The 3D
// pair-loop kernel with the boundary copies folded in keeps the plain
// kernel's seven.
template <uint32_t EM, bool FX, int DIM>
constexpr int min_blocks() {
  return (FX && DIM == 3 && (EM & kLoopPairs)) ? 7 : 0;
}

// One iteration: pull, moments, Dirichlet, [Monitor], collide. FX: the
// boundary copies run inside (boundary_fused.cuh) instead of in k_fill.
template <int DIM, bool RHO1, bool MON, uint32_t EM = 0, bool FX = false>
__global__ void __launch_bounds__(kBlock, (min_blocks<EM, FX, DIM>())) k_step(DevGrid g, DevCoef c,
                                                                   DevState st,
                                                                   const double* __restrict__ fin,
                                                                   double* __restrict__ fout,
                                                                   unsigned long long* monitor) {
  using N_ = Node<DIM, RHO1, EM>;
  const int64_t id = g.id_lo + (int64_t)blockIdx.x * kBlock + threadIdx.x;
  double um = 0.0;
  if constexpr (!FX) {
    if (id < g.id_hi) {
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
        if constexpr ((EM & kLoopPairs) != 0u)
          N_::template collide_loop<false>(p, u, c, st, fin, g, fout, id, PullFix{0u});
        else N_::collide(f, p, u, c, fout, g.N, id);
      }
    }
  } else {
    const uint8_t m = id < g.id_hi ? st.mask[id] : (uint8_t)0;
    const PullFix fx = PullFix::make(st, (m & kMaskFluid) ? m : (uint8_t)0);
    // warps with a node next to the rim or an obstacle take the table pull
    const bool bwarp = __any_sync(0xffffffffu, fx.bits != 0u);
    if (m & kMaskFluid) {
      double f[N_::Q];
      N_::pull_fixed(fin, g, st, id, fx, bwarp, f);
      double p, u[DIM];
      N_::moments(f, p, u, c);
      N_::dirichlet(m, id, g, st.inlet, p, u);
      if constexpr (MON) {
        if (id != g.skip_id) um = speed2d(u[0], u[1]);
      }
      if constexpr ((EM & kLoopPairs) != 0u)
        N_::template collide_loop<true>(p, u, c, st, fin, g, fout, id, fx);
      else N_::collide(f, p, u, c, fout, g.N, id);
      if (fx.record()) push_copies(st.push, PullFix::row<N_::Q>(st, id)[N_::Q], fin, fout);
    }
  }
  if constexpr (MON) block_max_to(um, monitor);
}

// Masks of the step-kernel variants by split index (rho0 = 1): the FP64
// instructions as the reference writes them (the plain form, kept as the
// simplest kernel to check the others against) and the fastest measured on
// GB300 (D3Q27 256x128x128 sphere, D2Q9 1024x512 cylinder): DFMA form, exact
// integer /3, every multiplication emulated, a run-time pair loop. Five other
// masks measured slower were dropped.
template <int DIM>
struct Splits {
  static constexpr uint32_t F = kFmaForm, D = kEmDiv3, M = kEmMulsOnly;
  static constexpr uint32_t v[] = {
      0u,                                              // DADD / DMUL / DDIV
      F | D | M | 1u | kEmRest | kEmUdu | kLoopPairs,  // the default
  };
  static constexpr int n = sizeof(v) / sizeof(v[0]);
  static constexpr int kDefault = 1;
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
    k_step<DIM, true, MON, Splits<DIM>::v[V]><<<grid, kBlock, 0, s>>>(g, c, st, fin, fout, monitor);
    return cudaGetLastError();
  } else {
    return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace imx
