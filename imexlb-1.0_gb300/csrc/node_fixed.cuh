// BGK node update in 64-bit fixed point (IMEXLB_FIX64), on the integer pipes.
//
// The same update as the reference's Collision / PostProcessing
// (lbm.f90:52-76, 159-201) written for rho0 = 1:
//   S = sum f_i (= 3p),  u = sum f_i e_i,  X = S - 1.5 u.u,
//   fb_i = (1 - ome) f_i + K_i (X + 4.5 (e_i.u)^2 + 3 e_i.u),  K_i = ome t_i,
// with every value in Q3.60 (fixed64.cuh). Sums are exact. The products of
// two velocity components are formed once (six in D3Q27, three in D2Q9) and
// rounded to Q.59, so that 1.5 u.u and 4.5 (e.u)^2 are exact integer
// multiples (3 and 9 times a Q.59 value, read as Q.60); every (e.u)^2 is an
// exact combination of those products. The remaining products by the
// constants K_i and 1 - ome round to nearest, so no operation is biased and
// the mass sum does not drift from rounding. A +/- direction pair shares
// K (X + 4.5 (e.u)^2) and K 3 e.u.
//
// Range: a node whose populations reach |f| >= 4, or whose moments reach
// |S| >= 2 or |u_k| >= 0.25 (far outside a stable lattice Boltzmann state),
// is marked invalid: all its outputs become kFixInvalid (NaN on download),
// which the Monitor value reports.
#pragma once

#include <cstdint>

#include "fixed64.cuh"
#include "kernels.h"
#include "lattice.h"

namespace imx {

template <int DIM>
struct NodeFixed {
  using Lat = Lattice<DIM>;
  static constexpr int Q = Lat::Q;

  // S = sum F and J_k = sum e_k F over the z columns (x columns in 2D),
  // sharing partial sums as NodeFast does; exact integer additions.
  __device__ static __forceinline__ long long moments(const long long (&F)[Q], long long (&J)[DIM]) {
    if constexpr (DIM == 2) {
      const long long gm = F[0] + F[1] + F[2], g0 = F[3] + F[4] + F[5], gp = F[6] + F[7] + F[8];
      J[0] = gp - gm;
      J[1] = (F[2] + F[5] + F[8]) - (F[0] + F[3] + F[6]);
      return gm + g0 + gp;
    } else {
      long long gs[9], gd[9];
#pragma unroll
      for (int b = 0; b < 9; ++b) {
        gs[b] = F[b] + F[b + 9] + F[b + 18];
        gd[b] = F[b + 18] - F[b];
      }
      const long long xm = gs[0] + gs[1] + gs[2], x0 = gs[3] + gs[4] + gs[5], xp = gs[6] + gs[7] + gs[8];
      J[0] = xp - xm;
      J[1] = (gs[2] + gs[5] + gs[8]) - (gs[0] + gs[3] + gs[6]);
      long long z = gd[0];
#pragma unroll
      for (int b = 1; b < 9; ++b) z += gd[b];
      J[2] = z;
      return xm + x0 + xp;
    }
  }

  // Populations below 4 in magnitude (and none invalid), S below 2, every
  // velocity component below 0.25.
  __device__ static __forceinline__ bool in_range(const long long (&F)[Q], long long S,
                                                  const long long (&J)[DIM]) {
    unsigned acc = 0u;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const int hi = (int)(F[i] >> 32);
      acc |= (unsigned)(hi ^ (hi >> 31));
    }
    bool ok = acc < (1u << 30) && fix_below(S, kFixFrac + 1);
#pragma unroll
    for (int k = 0; k < DIM; ++k) ok = ok && fix_below(J[k], kFixFrac - 2);
    return ok;
  }

  // e_i . u of direction I as an exact sum of components
  template <int I>
  __device__ static __forceinline__ long long edu(const long long (&J)[DIM]) {
    long long s = 0;
    sfor<0, DIM>([&](auto K) {
      constexpr int cc = Lat::e(I, K);
      if constexpr (cc > 0) s += J[K];
      else if constexpr (cc < 0) s -= J[K];
    });
    return s;
  }

  // (e_i . u)^2 in Q.59 from the products P (Q.59; P[a][b], a <= b)
  template <int I>
  __device__ static __forceinline__ long long sq(const long long (&P)[DIM][DIM]) {
    long long s = 0;
    sfor<0, DIM>([&](auto A) {
      constexpr int ea = Lat::e(I, A);
      if constexpr (ea != 0) s += P[A][A];
      sfor<A + 1, DIM>([&](auto B) {
        constexpr int eb = Lat::e(I, B);
        if constexpr (ea * eb > 0) s += P[A][B] << 1;
        else if constexpr (ea * eb < 0) s -= P[A][B] << 1;
      });
    });
    return s;
  }

  // fn(iq, post-collision value) for every direction. k[i] = ome t_i and
  // om1 = 1 - ome in Q0.63.
  template <class Fn>
  __device__ static __forceinline__ void collide(const long long (&F)[Q], long long S,
                                                 const long long (&J)[DIM], const long long* k,
                                                 long long om1, Fn&& fn) {
    long long P[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a) {
      const long long J4 = J[a] * 4;  // Q.62
#pragma unroll
      for (int b = a; b < DIM; ++b) P[a][b] = fix_mul(J4, J[b]);
    }
    long long uu = P[0][0] + P[1][1];
    if constexpr (DIM == 3) uu += P[2][2];
    const long long X = S - 3 * uu;
    fn(Lat::REST, fix_mul(F[Lat::REST], om1) + fix_mul(X, k[Lat::REST]));
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        const long long A = X + 9 * sq<i>(P);
        const long long B = 3 * edu<i>(J);
        const long long KA = fix_mul(A, k[i]), KB = fix_mul(B, k[i]);
        fn(i, fix_mul(F[i], om1) + (KA + KB));
        fn(o, fix_mul(F[o], om1) + (KA - KB));
      }
    });
  }
};

}  // namespace imx
