// Step kernel of the fixed-point kind (IMEXLB_FIX64): populations stored as
// Q3.60 integers, the whole node update on the integer pipes
// (node_fixed.cuh). Pull, boundary handling and obstacle copies are those of
// the other step kernels (kernels_lp.cu, boundary_fused.cuh): one thread per
// padded interior cell, the pulled population of direction i read from the
// direction's plane shifted by its pull offset (Propagation, lbm.f90:80-92),
// the moments and Dirichlet conditions of PostProcessing (lbm.f90:159-201),
// Monitor (lbm.f90:205-227) and Collision (lbm.f90:52-76).
#include <cstdint>

#include <cuda_runtime.h>

#include "boundary_fused.cuh"
#include "fixed64.cuh"
#include "kernels.h"
#include "lattice.h"
#include "node_fixed.cuh"

namespace imx {
namespace {

constexpr int kBlockFx = 256;

// Max over the block of non-negative values or NaN (their bit patterns order
// like the values, NaN above all), one atomicMax per block.
__device__ __forceinline__ void block_max_fx(double v, unsigned long long* dst) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  __shared__ unsigned long long wmax[kBlockFx / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wmax[w] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = wmax[0];
    for (int i = 1; i < kBlockFx / 32; ++i) m = wmax[i] > m ? wmax[i] : m;
    atomicMax(dst, m);
  }
}

// max of two non-negative values (or NaN) through their bit patterns: NaN
// stays the maximum, as in the block reduction
__device__ __forceinline__ double fx_bitmax(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long y = (unsigned long long)__double_as_longlong(b);
  return __longlong_as_double((long long)(x > y ? x : y));
}

// The node update after the pull: moments, PostProcessing's inlet velocity
// (lbm.f90:186-191) and zero outlet pressure (lbm.f90:195-198), the range
// check, [Monitor: um takes the max with |(u_x, u_y)|], Collision, stores.
// (k: the coefficients ome t_i of CoefFix, om1 = 1 - ome)
template <int DIM, bool MON>
__device__ __forceinline__ void fx_node_finish(const long long (&F)[Lattice<DIM>::Q],
                                               const DevGrid& g, const long long* k,
                                               long long om1, const DevState& st,
                                               const DevPlanes& pl, uint32_t id, uint8_t m,
                                               double& um) {
  using NF = NodeFixed<DIM>;
  constexpr int Q = Lattice<DIM>::Q;
  long long J[DIM];
  long long S = NF::moments(F, J);
  if (m & kMaskInlet) {
    const int64_t r = DIM == 2 ? (int64_t)id / g.dy : (int64_t)id / g.dz;
    J[0] = fix_from_double(st.inlet[r]);
    J[1] = 0;
  }
  if (m & kMaskOutlet) S = 0;
  const bool ok = NF::in_range(F, S, J);
  if constexpr (MON) {
    if (id != g.skip_id) {
      const double ux = fix_to_double(J[0]), uy = fix_to_double(J[1]);
      um = fx_bitmax(um, ok ? sqrt(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)))
                            : __longlong_as_double(0x7ff8000000000000LL));
    }
  }
  if (ok) {
    NF::collide(F, S, J, k, om1, [&](int i, long long v) { ((long long*)pl.out[i])[id] = v; });
  } else {
#pragma unroll
    for (int i = 0; i < Q; ++i) ((long long*)pl.out[i])[id] = kFixInvalid;
  }
}

// The general pull of one fluid cell (closed forms of its boundary bits, or
// its record's source row), the node update, and the record's push copies.
template <int DIM, bool MON>
__device__ __forceinline__ void fx_node_general(const DevGrid& g, const CoefFix& c,
                                                const DevState& st, const DevPlanes& pl,
                                                uint32_t id, uint8_t m, const PullFix& fx,
                                                double& um) {
  using L = Lattice<DIM>;
  constexpr int Q = L::Q;
  long long F[Q];
  const long long* fin = (const long long*)pl.in[0] + g.off[0];
  long long* fout = (long long*)pl.out[0];
  if (!fx.record()) {
    sfor<0, Q>([&](auto I) {
      constexpr int i = I;
      bool opp;
      int64_t sh;
      fx.form<DIM>(L::ex(i), L::ey(i), L::ez(i), g.off[i], st.pshift, opp, sh);
      const long long* base = (const long long*)(opp ? pl.in[Q - 1 - i] : pl.in[i]);
      F[I] = base[(uint32_t)(id + (uint32_t)sh)];
    });
  } else {
    const uint32_t* row = PullFix::row<Q>(st, id);
    sfor<0, Q>([&](auto I) {
      const uint32_t r = row[I];
      F[I] = r != kNoRedirect ? fin[r] : ((const long long*)pl.in[I])[id];
    });
  }
  fx_node_finish<DIM, MON>(F, g, c.k, c.om1, st, pl, id, m, um);
  if (fx.record()) push_copies(st.push, PullFix::row<Q>(st, id)[Q], fin, fout);
}

template <int DIM, bool MON>
__global__ void __launch_bounds__(kBlockFx) k_step_fx(DevGrid g, CoefFix c, DevState st,
                                                      DevPlanes pl, unsigned long long* monitor) {
  using L = Lattice<DIM>;
  constexpr int Q = L::Q;
  const uint32_t id = (uint32_t)(g.id_lo + (int64_t)blockIdx.x * kBlockFx + threadIdx.x);
  double um = 0.0;
  const uint8_t m = (int64_t)id < g.id_hi ? st.mask[id] : (uint8_t)0;
  const PullFix fx = PullFix::make(st, (m & kMaskFluid) ? m : (uint8_t)0);
  const bool bwarp = __any_sync(0xffffffffu, fx.other());
  if (m & kMaskFluid) {
    if (!bwarp) {
      long long F[Q];
      const uint32_t id_in = id + fx.inl(), o = fx.outl();
      sfor<0, Q>([&](auto I) {
        constexpr int ex = L::ex(I);
        const uint32_t a = ex == 1 ? id_in : (ex == -1 ? id + o * (uint32_t)g.off[I] : id);
        F[I] = ((const long long*)pl.in[I])[a];
      });
      fx_node_finish<DIM, MON>(F, g, c.k, c.om1, st, pl, id, m, um);
    } else {
      fx_node_general<DIM, MON>(g, c, st, pl, id, m, fx, um);
    }
  }
  if constexpr (MON) block_max_fx(um, monitor);
}

}  // namespace

cudaError_t launch_step_fx(int dim, const DevGrid& g, const CoefFix& c, const DevState& st,
                           const DevPlanes& pl, unsigned long long* monitor, cudaStream_t s) {
  const unsigned grid = (unsigned)((g.id_hi - g.id_lo + kBlockFx - 1) / kBlockFx);
  if (dim == 2) {
    if (monitor) k_step_fx<2, true><<<grid, kBlockFx, 0, s>>>(g, c, st, pl, monitor);
    else k_step_fx<2, false><<<grid, kBlockFx, 0, s>>>(g, c, st, pl, monitor);
  } else {
    if (monitor) k_step_fx<3, true><<<grid, kBlockFx, 0, s>>>(g, c, st, pl, monitor);
    else k_step_fx<3, false><<<grid, kBlockFx, 0, s>>>(g, c, st, pl, monitor);
  }
  return cudaGetLastError();
}

}  // namespace imx
