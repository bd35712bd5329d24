// Tiles staged in shared memory by the bulk-copy engine: the copy plan, the
// stage barriers, the bounded waits and the producer loop of a staged step
// kernel (k_step_staged in kernels_lp.cu, BF16 / FP16 storage on D3Q27).
//
// A persistent block walks tiles of TILE consecutive cells from id_lo. One
// warp (the producer) starts, per tile, Q + 1 bulk copies (cp.async.bulk,
// global -> shared, completion counted in bytes on the stage's `full`
// mbarrier): each direction's pulled run and the tile's mask bytes. A run
// starts at any element; its copy starts at the 16-byte boundary below it
// and takes TILE * sizeof(T) + 16 bytes, which holds the run and the
// element after it (the inlet pulls). A tile is a multiple of 16 bytes in
// every plane, so a run's place inside its copy is the same for every tile:
// the host passes the copies of tile 0 and their stride (StagePlan).
// Consumer warps read the tile from shared memory and release the stage on
// its `empty` mbarrier (one arrival per warp); the producer refills a stage
// once all consumers released it. No block-wide barrier: a warp waits only
// for its data, and loads in flight hold no registers.
//
// Every wait is bounded (StagePlan::wait_ns of the global timer, 2 s unless
// a test injects a stall). A warp that gives up writes 1 to StagePlan::status
// and raises the block's abort flag; the other warps stop at their next tile
// (or when their own bounded wait gives up), and the producer waits (bounded
// again) for the copies it still has in flight before the block returns. The
// host reads the status after the step call.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "kernels.h"

namespace imx {

// One stage's copies: entry l <= Q (lane l of the producer warp starts it)
// moves size[l] bytes from src0[l] + t step[l] (tile t) to byte dst[l] of the
// stage; the runs are entries 0 .. Q-1, the mask bytes entry Q.
struct StagePlan {
  uint64_t src0[28];
  uint32_t step[28];
  uint32_t dst[28];
  uint32_t size[28];
  uint32_t pos[27];  // byte offset of direction i's run (its first element) in a stage
  uint32_t mpos;     // byte offset of the tile's first mask byte
  int64_t ntiles;
  int* status;       // host-visible word: 1 when a wait gave up
  unsigned long long wait_ns;  // budget of every wait
  int stall;         // failure injection: the first tile of a block starts no copies
};

// bytes of one run's copy and of one stage (Q runs and the mask bytes)
__host__ __device__ constexpr uint32_t stage_run_bytes(int tile, int esz) {
  return (uint32_t)(tile * esz + 16);
}
__host__ __device__ constexpr uint32_t stage_bytes(int q, int tile, int esz) {
  return (uint32_t)q * stage_run_bytes(tile, esz) + (uint32_t)(tile + 16);
}

// The copies reach TILE * esz + 16 bytes past a tile's first pulled element
// and the last plane's pull shift is up to 1 + dy + dz cells: the trailing
// ghost layers must cover both (and the tile's mask bytes).
inline bool stage_fits(const DevGrid& g, int tile) {
  return g.N - g.id_hi >= tile + 16 + g.dy + g.dz;
}

// The plan of a step from fin's plane pointers (pl) and the cell mask.
template <int Q>
inline StagePlan make_stage_plan(const DevGrid& g, const DevState& st, const DevPlanes& pl,
                                 const StagedArgs& sa, int tile, int esz) {
  const uint32_t run = stage_run_bytes(tile, esz);
  StagePlan sp{};
  for (int i = 0; i < Q; ++i) {
    const uint64_t a = (uint64_t)(uintptr_t)pl.in[i] + (uint64_t)esz * (uint64_t)g.id_lo;
    sp.src0[i] = a & ~(uint64_t)15;
    sp.step[i] = (uint32_t)(tile * esz);
    sp.dst[i] = (uint32_t)i * run;
    sp.size[i] = run;
    sp.pos[i] = (uint32_t)(i * run + (a & 15u));
  }
  const uint64_t am = (uint64_t)(uintptr_t)st.mask + (uint64_t)g.id_lo;
  sp.src0[Q] = am & ~(uint64_t)15;
  sp.step[Q] = (uint32_t)tile;
  sp.dst[Q] = (uint32_t)Q * run;
  sp.size[Q] = (uint32_t)(tile + 16);
  sp.mpos = (uint32_t)(Q * run + (am & 15u));
  sp.ntiles = (g.id_hi - g.id_lo + tile - 1) / tile;
  sp.status = sa.status;
  sp.wait_ns = sa.wait_ns;
  sp.stall = sa.stall;
  return sp;
}

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for phase `parity` of a stage barrier; false when it gave up.
// Each try suspends the warp until the phase completes or kStageSuspendNs
// pass (the suspend-time hint), so a waiting warp takes no issue slots.
constexpr uint32_t kStageSuspendNs = 100000;
__device__ __forceinline__ bool stage_wait(uint64_t* bar, uint32_t parity,
                                           unsigned long long budget_ns) {
  unsigned long long t0 = 0;
  for (uint32_t n = 0;; ++n) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kStageSuspendNs)
        : "memory");
    if (done) return true;
    const unsigned long long t = global_ns();
    if (n == 0) t0 = t;
    else if (t - t0 > budget_ns) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Barriers of a block's kStages stages (thread 0, before the block's first
// __syncthreads): `full` takes the producer's arrival, `empty` one arrival per
// consumer warp.
__device__ __forceinline__ void stage_init(uint64_t* full, uint64_t* empty, uint32_t stages,
                                           uint32_t consumers) {
  for (uint32_t s = 0; s < stages; ++s) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[s])), "r"(1)
                 : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&empty[s])),
                 "r"(consumers)
                 : "memory");
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The producer warp starts the copies of tile t into stage buffer `dst`
// (barrier bar, `bytes` in all).
template <int Q>
__device__ __forceinline__ void stage_issue(const StagePlan& sp, int64_t t, uint8_t* dst,
                                            uint64_t* bar, int lane, uint32_t bytes) {
  if (lane == 0) {
    // the block's reads of this buffer (generic proxy) come before the copies
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
  }
  __syncwarp();
  if (lane <= Q && !(sp.stall && t == (int64_t)blockIdx.x)) {
    const uint64_t src = sp.src0[lane] + (uint64_t)t * sp.step[lane];
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst + sp.dst[lane])),
        "l"(src), "r"(sp.size[lane]), "r"(smem_u32(bar))
        : "memory");
  }
}

// A wait that gave up: the block's abort flag and the host's status word.
__device__ __forceinline__ void stage_give_up(volatile int* abort_v, int* status) {
  *abort_v = 1;
  *(volatile int*)status = 1;
}

// The producer warp's loop: tile k (t0 + k G) into stage k % stages once the
// consumers released its previous tile; then, after an abort, the wait
// (bounded) for the copies still in flight, the last `stages` tiles issued.
template <int Q>
__device__ __forceinline__ void stage_produce(const StagePlan& sp, uint8_t* smem, uint32_t stage,
                                              uint32_t stages, uint32_t bytes, uint64_t* full,
                                              uint64_t* empty, uint32_t ntiles, int64_t t0,
                                              int64_t G, int lane, volatile int* abort_v) {
  uint32_t k = 0, s = 0, phase = 0;
#pragma unroll 1
  for (; k < ntiles; ++k) {
    if (__any_sync(0xffffffffu, *abort_v)) break;
    // the stage's previous tile (k - stages) released by every consumer
    bool ok = true;
    if (k >= stages) ok = stage_wait(&empty[s], phase ^ 1u, sp.wait_ns);
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) {
      if (lane == 0) stage_give_up(abort_v, sp.status);
      break;
    }
    stage_issue<Q>(sp, t0 + (int64_t)k * G, smem + s * stage, &full[s], lane, bytes);
    if (++s == stages) {
      s = 0;
      phase ^= 1u;
    }
  }
  if (*abort_v && lane == 0)
    for (uint32_t j = k > stages ? k - stages : 0; j < k; ++j)
      stage_wait(&full[j % stages], (j / stages) & 1u, sp.wait_ns);
}

#endif  // __CUDACC__

}  // namespace imx
