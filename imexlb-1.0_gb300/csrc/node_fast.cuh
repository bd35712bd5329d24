// BGK node update with a minimal operation count (not the reference's
// evaluation order): used by the FP32-arithmetic kernels and by the FP64
// option that trades bit-exactness for speed.
//
// Moments: the populations are summed in the nine (x, y) columns of three z
// values (D3Q27; columns of three y values in D2Q9), so p and u share their
// partial sums: 49 additions in D3Q27 instead of 77, 14 instead of 18 in D2Q9.
//
// Collision: with K_i = ome * t_i * rho0 and X = 3p/rho0 - 1.5 u.u,
//   fb_i = (1-ome) f_i + K_i (X + e(3 + 4.5 e)),  e = e_i.u,
// and the opposite direction uses e(4.5e - 3) = e(3 + 4.5e) - 6e, so a
// +/- pair costs 9 operations. Every multiply, add and fused multiply-add is
// written out with its rounding (the _rn intrinsics, which the compiler does
// not contract or reorder), so every kernel that inlines this update gives
// the same bits for the same inputs, whatever code surrounds it.
#pragma once

#include <cstdint>

#include "kernels.h"
#include "lattice.h"

namespace imx {

// Explicitly rounded operations in R = float or double.
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double r_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float r_sqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double r_sqrt(double a) { return ::sqrt(a); }

template <int DIM, class R>
struct NodeFast {
  using Lat = Lattice<DIM>;
  static constexpr int Q = Lat::Q;

  // Returns S = sum(f) (= 3p before the outlet condition) and u.
  __device__ static IMX_FI R moments(const R (&f)[Q], R (&u)[DIM], R inv_rho0) {
    if constexpr (DIM == 2) {
      // iq = (i+1)*3 + (j+1): columns of fixed x
      const R gm = f[0] + f[1] + f[2], g0 = f[3] + f[4] + f[5], gp = f[6] + f[7] + f[8];
      const R s = gm + g0 + gp;
      u[0] = r_mul(gp - gm, inv_rho0);
      u[1] = r_mul((f[2] + f[5] + f[8]) - (f[0] + f[3] + f[6]), inv_rho0);
      return s;
    } else {
      // iq = (k+1)*9 + b, b = (i+1)*3 + (j+1): z-sum and z-difference per b
      R gs[9], gd[9];
#pragma unroll
      for (int b = 0; b < 9; ++b) {
        gs[b] = f[b] + f[b + 9] + f[b + 18];
        gd[b] = f[b + 18] - f[b];
      }
      const R xm = gs[0] + gs[1] + gs[2], x0 = gs[3] + gs[4] + gs[5], xp = gs[6] + gs[7] + gs[8];
      const R s = xm + x0 + xp;
      u[0] = r_mul(xp - xm, inv_rho0);
      u[1] = r_mul((gs[2] + gs[5] + gs[8]) - (gs[0] + gs[3] + gs[6]), inv_rho0);
      R z = gd[0];
#pragma unroll
      for (int b = 1; b < 9; ++b) z += gd[b];
      u[2] = r_mul(z, inv_rho0);
      return s;
    }
  }

  template <int I>
  __device__ static IMX_FI R edu(const R (&u)[DIM]) {
    constexpr int k0 = Lat::first_comp(I);
    R s = u[k0];
    sfor<k0 + 1, DIM>([&](auto K) {
      constexpr int cc = Lat::e(I, K);
      if constexpr (cc > 0) s += u[K];
      else if constexpr (cc < 0) s -= u[K];
    });
    return s;
  }

  // fn(iq, post-collision value). S3 = 3p (the moment sum, or 0 at the outlet).
  // |(u_x, u_y)|, the quantity Monitor reduces
  __device__ static IMX_FI R speed(const R (&u)[DIM]) {
    return r_sqrt(r_fma(u[1], u[1], r_mul(u[0], u[0])));
  }

  template <class F>
  __device__ static IMX_FI void collide(const R (&f)[Q], R S3, const R (&u)[DIM],
                                        const CoefR<R>& c, F&& fn) {
    R uu = r_fma(u[1], u[1], r_mul(u[0], u[0]));
    if constexpr (DIM == 3) uu = r_fma(u[2], u[2], uu);
    const R X = r_fma(R(-1.5), uu, r_mul(S3, c.inv_rho0));
    fn(Lat::REST, r_fma(c.om1, f[Lat::REST], r_mul(c.k[Lat::REST], X)));
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      if constexpr (Lat::is_rep(i)) {
        constexpr int o = Lat::opp(i);
        const R e = edu<i>(u);
        const R gp = r_mul(e, r_fma(R(4.5), e, R(3)));
        const R gm = r_fma(R(-6), e, gp);
        fn(i, r_fma(c.om1, f[i], r_mul(c.k[i], r_add(X, gp))));
        fn(o, r_fma(c.om1, f[o], r_mul(c.k[o], r_add(X, gm))));
      }
    });
  }

  // PostProcessing's Dirichlet conditions on a fluid node (lbm.f90:185-198).
  __device__ static IMX_FI void dirichlet(uint8_t m, int64_t id, const DevGrid& g,
                                          const double* inlet, R& S3, R (&u)[DIM]) {
    if (m & kMaskInlet) {
      const int64_t r = DIM == 2 ? id / g.dy : id / g.dz;
      u[0] = (R)inlet[r];
      u[1] = R(0);
    }
    if (m & kMaskOutlet) S3 = R(0);
  }
};

}  // namespace imx
