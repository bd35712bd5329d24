// Lattice tables for D2Q9 and D3Q27 in the reference ordering, usable as
// compile-time constants in host and device code.
//
// Reference ordering (initialization.f90:115-121, initialization_3d.f90:111-120):
//   D2Q9:  iq = (i+1)*3 + (j+1),            e(iq) = (i, j)
//   D3Q27: iq = (k+1)*9 + (i+1)*3 + (j+1),  e(iq) = (i, j, k)
// so the opposite direction of iq is nq-1-iq and the rest direction is nq/2.
#pragma once

#include <type_traits>
#include <utility>

#if defined(__CUDACC__)
#define IMX_HD __host__ __device__
#define IMX_FI __forceinline__
#else
#define IMX_HD
#define IMX_FI inline
#endif

namespace imx {

constexpr int kGhost = 3;  // cart_mpi.f90:10

template <int DIM>
struct Lattice {
  static_assert(DIM == 2 || DIM == 3, "D2Q9 or D3Q27");
  static constexpr int Q = DIM == 2 ? 9 : 27;
  static constexpr int REST = Q / 2;
  IMX_HD static constexpr int ex(int iq) { return DIM == 2 ? iq / 3 - 1 : (iq / 3) % 3 - 1; }
  IMX_HD static constexpr int ey(int iq) { return iq % 3 - 1; }
  IMX_HD static constexpr int ez(int iq) { return DIM == 2 ? 0 : iq / 9 - 1; }
  IMX_HD static constexpr int e(int iq, int k) { return k == 0 ? ex(iq) : (k == 1 ? ey(iq) : ez(iq)); }
  IMX_HD static constexpr int opp(int iq) { return Q - 1 - iq; }
  // The direction of a +/- pair whose first non-zero component is +1.
  IMX_HD static constexpr bool is_rep(int iq) {
    return iq != REST && (ex(iq) > 0 || (ex(iq) == 0 && (ey(iq) > 0 || (ey(iq) == 0 && ez(iq) > 0))));
  }
  // First direction with a non-zero k-th component (start of the moment sum).
  IMX_HD static constexpr int first_nz(int k) {
    for (int i = 0; i < Q; ++i)
      if (e(i, k) != 0) return i;
    return -1;
  }
  // First non-zero component of direction iq.
  IMX_HD static constexpr int first_comp(int iq) {
    for (int k = 0; k < DIM; ++k)
      if (e(iq, k) != 0) return k;
    return -1;
  }
};

// Integer constant usable as a template argument inside device lambdas.
template <int V>
struct IC {
  static constexpr int value = V;
  IMX_HD constexpr operator int() const { return V; }
};

// Compile-time loop: fn(IC<I>) for I in [B, E).
template <int B, int E, class F>
IMX_HD IMX_FI constexpr void sfor(F&& fn) {
  if constexpr (B < E) {
    fn(IC<B>{});
    sfor<B + 1, E>(std::forward<F>(fn));
  }
}

}  // namespace imx
