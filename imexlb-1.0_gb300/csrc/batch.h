// Device-side description of one case of an ensemble stepped in lockstep.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "kernels.h"

namespace imx {

struct BatchCase {
  DevGrid g;
  CoefR<float> c;
  const uint8_t* mask;
  const double* inlet;
  void* fb[2];          // population buffers of the case
  const void* fill;     // its boundary fill list (DevFill32 if fill_narrow)
  int64_t n_fill;
  int fill_narrow;
  int parity0;          // buffer holding the post-BC state when the call starts
  int nsteps;           // iterations this case takes in the call
  int pad;
  int64_t block0;       // first step block of the case
  int64_t fill_block0;  // first fill block of the case
};

// Step-kernel launch shapes the autotuner chooses from: threads per block and
// lattice nodes per thread.
struct BatchShape {
  int block, cpt;
};
constexpr int kNumBatchShapes = 6;
extern const BatchShape kBatchShapes[kNumBatchShapes];

// One lockstep iteration of every case with counter < nsteps, then counter++.
cudaError_t launch_batch_iteration(int dim, int store, int shape, const BatchCase* cases,
                                   const uint16_t* block_case, int64_t nblocks,
                                   const uint16_t* fill_case, int64_t nfill_blocks, int* counter,
                                   cudaStream_t s);

// ---- Persistent stepping (batch_persist.cu): one cooperative launch per
// call; work items are step tiles and fill chunks of each case's iterations.
constexpr int kPersistCPT = 4;                   // cells per thread of a step tile
constexpr int kPersistTile = 256 * kPersistCPT;  // cells per step tile
constexpr int kPersistFillChunk = 1024;          // fill entries per chunk
constexpr int kPersistTimeout = 1;               // status: a wait ran out of budget

struct PersistSched {
  const BatchCase* cases;
  const int* order;             // cases by descending iteration budget
  const long long* tile_pre;    // [ncases + 1] prefix sums of step tiles in `order`
  const long long* fill_pre;    // [ncases + 1] prefix sums of fill chunks in `order`
  const long long* iter_start;  // [niters + 1] first item of each iteration
  const int* active;            // [niters] cases still running at each iteration
  long long nitems;
  int ncases;
  unsigned long long* next;     // work counter (zero at launch)
  unsigned* done_step;          // per case: step tiles finished in this call
  unsigned* done_fill;          // per case: fill chunks finished in this call
  int* status;                  // 0, or kPersistTimeout
  int* info;                    // case, iteration, kind (0 step, 1 fill) of the wait that gave up
  unsigned long long budget_ns; // bound of every wait (device global timer)
  int stall_case;               // testing: this case's step tiles after its first iteration
                                // wait for a count nothing reaches (-1: none)
};

// Resident blocks of the persistent kernel for this device (SMs x blocks per
// SM) for a batch of ncases cases, and its dynamic shared memory.
cudaError_t persistent_grid(int dim, int store, int ncases, int* blocks);
size_t persistent_smem(int ncases);
cudaError_t launch_batch_persistent(int dim, int store, int blocks, const PersistSched& s,
                                    cudaStream_t st);

}  // namespace imx
