// Host side of the boundary copies folded into the step kernel
// (boundary_fused.cuh): which fluid node reads which source, and which node
// runs which obstacle copy.
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

#include "bcmap.h"
#include "kernels.h"

namespace imx {

struct FusedPlan {
  std::vector<int64_t> nodes;                      // record nodes, ascending
  std::vector<uint32_t> rec;                       // (Q+1) words per record node
  std::vector<DevFill32> ent;                      // obstacle copies grouped by node
  std::vector<std::pair<int64_t, uint8_t>> face;   // closed-form nodes, their face bits
  int64_t pshift = 0;                              // periodic y faces (3D): L1 * dy
};

// Builds the plan from the step's fill list (SoA slots; ~src = previous
// buffer) and the node mask (fluid, inlet, outlet bits). Returns false when
// the geometry keeps the separate fill kernel: a ghost slot copies an
// obstacle slot of the previous iteration, or a node would run more than 255
// obstacle copies.
bool plan_fused(const GridLayout& gl, const DevGrid& g, const std::vector<uint8_t>& mask,
                const BoundaryMap& bmap, const std::vector<DevFill>& fill, FusedPlan& out);

// The plan's bits (kMaskRecord, face bits) added to a node mask.
void apply_plan_bits(const FusedPlan& p, std::vector<uint8_t>& mask);

// The slot a closed-form node with boundary bits `bits` pulls direction q
// from (the device's PullFix::form).
int64_t fused_form(const GridLayout& gl, const DevGrid& g, int64_t pshift, int64_t p,
                   uint32_t bits, int q);

// The pull-offset tables of the 27 node kinds (DevState::offq_kind):
// out[kind*Q + q] = q*N + p - fused_form(p, bits of kind, q), the same for
// every node p.
void fused_kind_offsets(const GridLayout& gl, const DevGrid& g, int64_t pshift,
                        std::vector<int64_t>& out);

}  // namespace imx
