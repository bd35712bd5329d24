/*
 * imexlb_testing.h -- host-only hooks that expose libimexlb's boundary
 * resolution for verification without a GPU.
 */
#ifndef IMEXLB_TESTING_H
#define IMEXLB_TESTING_H

#include "imexlb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Apply the boundary map the library builds in imexlb_set_geometry to a
 * host array laid out like fb: out[s] = in[r(s)] for every slot s, where r(s)
 * is the slot whose value s holds after the reference's BoundaryCondition
 * (lbm.f90:96-155 with PassF of one rank, cart_mpi.f90:240-277); NaN where
 * the reference reads outside its arrays. Returns the number of boundary
 * slots the step kernels refresh per iteration (>= 0) or an IMEXLB_ERR_*
 * code. */
long long imexlb_testing_resolve_bc(const imexlb_desc* d, const int* fluid_id, int size_fluid,
                                    const int* bl, int l_size, const int* br, int r_size,
                                    const int* bu, int u_size, const int* bd, int d_size,
                                    const int* b_user, int user_size, const double* in,
                                    double* out);

/* The pulls of one step, with the boundary copies run as the separate
 * program (IMEXLB_FILL_KERNEL) and as the plan of IMEXLB_FILL_FUSED, on host
 * arrays in the device's layout (value of cell id, direction q at q*N + id;
 * N padded cells). `cur` is the buffer the step's collision has just written
 * (fluid slots) and holds every other slot's earlier value; `prev` is the
 * other buffer. For every fluid node and direction, out_kernel and out_fused
 * receive the value the next step pulls (other slots 0). Returns 1 when the
 * geometry gets a fused plan (n_records: the nodes with a source row or
 * obstacle copies), 0 when it keeps the separate kernel (out_fused zero), or
 * an IMEXLB_ERR_* code. */
long long imexlb_testing_fused_pull(const imexlb_desc* d, const int* fluid_id, int size_fluid,
                                    const int* bl, int l_size, const int* br, int r_size,
                                    const int* bu, int u_size, const int* bd, int d_size,
                                    const int* b_user, int user_size, const double* cur,
                                    const double* prev, double* out_kernel, double* out_fused,
                                    long long* n_records);

/* Step kernel of the BF16 and FP16 storage kinds: on != 0 (the default) the
 * kernel that stages each tile's pulled runs in shared memory with bulk
 * copies and updates two cells per thread with packed FP32 arithmetic (where
 * the lattice's ghost layers cover its copies), 0 the kernel that loads
 * every population into registers. Same node update, same bits; for
 * comparing the two. */
int imexlb_testing_set_staged_kernel(imexlb_t* h, int on);

/* Failure injection for the staged step kernel: with budget_s > 0 every wait
 * of the kernel gives up after budget_s seconds and the first tile of every
 * block starts no copies, so that its wait runs out: the kernel writes its
 * status word, drains the copies it has in flight and returns, and the step
 * call returns IMEXLB_ERR_TIMEOUT (the state of that call's iterations is not
 * valid). budget_s = 0 restores the normal kernel (2 s per wait). */
int imexlb_testing_stage_stall(imexlb_t* h, double budget_s);

/* Failure injection for the persistent batch (IMEXLB_BATCH_PERSISTENT): set
 * every device-side wait's budget to budget_s seconds and, with case_index
 * >= 0, make that case's step tiles after its first iteration wait for a
 * count no block ever reaches, so the wait runs out and the call returns
 * IMEXLB_ERR_TIMEOUT. case_index -1 removes the stall (the budget stays). No
 * kernel faults: the blocks return and the context stays usable. */
int imexlb_testing_batch_stall(imexlb_batch_t* b, int case_index, double budget_s);

#ifdef __cplusplus
}
#endif
#endif /* IMEXLB_TESTING_H */
