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

}  // namespace imx
