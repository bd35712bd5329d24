// The reference's BoundaryCondition (lbm.f90:96-155, lbm_3d.f90:96-157)
// inside the step kernel.
//
// Resolved on the host, the boundary program is a list of slot copies
// fb[dst] = fb[src] in which no source is another copy's destination. The
// step kernel pulls f_q(x) = fb(x - e_q, q); where that slot is a boundary
// slot the kernel needs its copy's source instead. Two kinds of destination:
//  - ghost slots (the rim around the lattice). They are never stored: the
//    fluid node that pulls one reads the copy's source from the input buffer
//    (a slot the previous step's collision wrote, or one no step writes).
//    On the faces the source has a closed form in the node's own pulls:
//      inlet (fb(id) = fb(id+1), lbm.f90:137-143): e_x = +1 directions read
//        one cell further in x;
//      outlet (fb(id) = fb(id+e), lbm.f90:146-153): e_x = -1 directions read
//        the node's own slot;
//      wall (bounce-back from two cells in, lbm.f90:105-123): directions
//        pointing away from the wall read the opposite direction's pull;
//      periodic y faces in 3D (PassF): directions crossing the face read the
//        opposite face, L1 * dy away.
//    The forms add up on edges where the program composes them; every node
//    whose sources the host cannot match with them carries a row of Q source
//    slots instead (kMaskRecord).
//  - obstacle slots. Their values carry over between iterations, so they
//    are stored: each copy runs in the thread that has just written its
//    source (a slot of its own cell, visible to it in program order), or,
//    when the source does not change during the step, in a nearby thread.
// The host checks every pulled boundary slot of the geometry against these
// rules and otherwise leaves the separate fill kernel in place.
#pragma once

#include <cstdint>

#include "kernels.h"
#include "lattice.h"

namespace imx {

// The obstacle copies run by this thread: `word` = first entry << 8 | count;
// fout[dst] = src >= 0 ? fout[src] : fin[~src]. Eight at a time: their entry
// loads, then their source loads, then their stores.
template <class T>
__device__ __forceinline__ void push_copies(const DevFill32* __restrict__ ent, uint32_t word,
                                            const T* fin, T* fout) {
  constexpr uint32_t kW = 8;
  const DevFill32* e = ent + (word >> 8);
  const uint32_t n = word & 0xffu;
#pragma unroll 1
  for (uint32_t k0 = 0; k0 < n; k0 += kW) {
    DevFill32 x[kW];
    T v[kW];
#pragma unroll
    for (uint32_t j = 0; j < kW; ++j)
      if (k0 + j < n) x[j] = e[k0 + j];
#pragma unroll
    for (uint32_t j = 0; j < kW; ++j)
      if (k0 + j < n) v[j] = x[j].src >= 0 ? fout[x[j].src] : fin[~x[j].src];
#pragma unroll
    for (uint32_t j = 0; j < kW; ++j)
      if (k0 + j < n) fout[x[j].dst] = v[j];
  }
}

// Boundary flags of one fluid node in fused mode (0 otherwise): a record
// node uses its row, the others the closed forms their bits select.
struct PullFix {
  uint32_t bits;

  __device__ __forceinline__ static PullFix make(const DevState& st, uint8_t m) {
    uint32_t b = st.bnd ? (uint32_t)(m & ~kMaskFluid) : 0u;
    return PullFix{(b & kMaskRecord) ? (uint32_t)kMaskRecord : b};
  }
  __device__ __forceinline__ bool record() const { return (bits & kMaskRecord) != 0u; }
  // 1 on an inlet node without a record: its e_x = +1 pulls read one cell on
  __device__ __forceinline__ uint32_t inl() const { return (bits & kMaskInlet) ? 1u : 0u; }
  // 1 on an outlet node without a record: its e_x = -1 pulls read its own
  // slot, off[q] cells from the plain pull
  __device__ __forceinline__ uint32_t outl() const { return (bits & kMaskOutlet) ? 1u : 0u; }
  // bits beyond a single inlet or outlet form: walls, periodic faces,
  // records, or both x forms at once
  __device__ __forceinline__ bool other() const {
    return (bits & ~(uint32_t)(kMaskInlet | kMaskOutlet)) != 0u ||
           (bits & (kMaskInlet | kMaskOutlet)) == (kMaskInlet | kMaskOutlet);
  }
  // index of the node's offset table in DevState::offq_kind (a node without
  // a record has at most one bit of each pair: the host makes the others
  // records)
  __device__ __forceinline__ int kind() const {
    const int x = (bits & kMaskInlet) ? 1 : ((bits & kMaskOutlet) ? 2 : 0);
    const int w = (bits & kMaskWallLo) ? 1 : ((bits & kMaskWallHi) ? 2 : 0);
    const int y = (bits & kMaskPerLo) ? 1 : ((bits & kMaskPerHi) ? 2 : 0);
    return x + 3 * w + 9 * y;
  }
  // closed forms of direction (ex, ey, ez): `opp` = read the opposite
  // direction's pull, `shift` = cells added to the pull index
  template <int DIM>
  __device__ __forceinline__ void form(int ex, int ey, int ez, int64_t off, int64_t pshift,
                                       bool& opp, int64_t& shift) const {
    const int ew = DIM == 3 ? ez : ey;
    opp = (ew == 1 && (bits & kMaskWallLo)) || (ew == -1 && (bits & kMaskWallHi));
    shift = 0;
    if (ex == 1 && (bits & kMaskInlet)) shift += 1;
    if (ex == -1 && (bits & kMaskOutlet)) shift += off;
    if (DIM == 3) {
      if (ey == 1 && (bits & kMaskPerLo)) shift += pshift;
      if (ey == -1 && (bits & kMaskPerHi)) shift -= pshift;
    }
  }
  // the node's record: Q source slots, then the push word
  template <int Q>
  __device__ __forceinline__ static const uint32_t* row(const DevState& st, int64_t id) {
    return st.bnd + (size_t)st.bnd_at[id] * (Q + 1);
  }
};

}  // namespace imx
