/*
 * imexlb_host.h -- host-side setup for C and C++ callers of libimexlb.
 *
 * A Fortran host keeps its own DataInput / InitLattice / SetGeometry / InitUP
 * (initialization.f90) and only binds imexlb.h. These functions give a C or
 * C++ host the same setup, producing the arrays imexlb_set_geometry and
 * imexlb_upload take, in the reference layout. They run on the CPU only.
 */
#ifndef IMEXLB_HOST_H
#define IMEXLB_HOST_H

#include "imexlb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The four input.in lines (input.in:1-4) and the values DataInput derives
 * from them (initialization.f90:59-102), plus the single-rank layout of
 * MPISetup (cart_mpi.f90:57-138). */
typedef struct imexlb_config {
  int dim;                        /* 2 or 3 */
  int nx, ny, nz;                 /* line 1 */
  double charlength_in, xpos_in;  /* line 2, in units of nx */
  double re;
  double ome, dt, rho0;           /* line 3 */
  double max_t, inter;            /* line 4 */
  /* derived */
  double charlength, pos, nu, t_intv, uu, tau, ma, radius;
  int interv, max_step;
  int local_length[3], local_start[3];
  int dy, dz;
  long long array_size;
  /* Extension (no reference counterpart): obstacle centre y = ny/2 + yoff.
   * 0 (the default of imexlb_host_read_input) reproduces the reference. */
  double yoff;
} imexlb_config;

/* DataInput: parse input.in (2D) / input_3d.in (3D) with Fortran list-directed
 * rules (one READ per record, values may continue on the next record) and
 * derive the rest. Returns 0 or an IMEXLB_ERR_* code. */
int imexlb_host_read_input(const char* path, int dim, imexlb_config* c);

/* Derive the DataInput quantities and the one-rank layout from the raw
 * input fields already set in *c. Returns IMEXLB_ERR_ARG when a local length
 * is below the ghost width (cart_mpi.f90:107-110). */
int imexlb_host_derive(imexlb_config* c);

/* InitLattice (initialization.f90:112-123, initialization_3d.f90:108-122). */
int imexlb_host_lattice(int dim, double* t /* nq */, int* e /* nq*dim */);

/* Capacities the caller allocates for SetGeometry's outputs, in the order
 * fluid_id, bl, br, bu, bd, bf, bb, b_user (AllocateArrays). */
int imexlb_host_list_capacity(const imexlb_config* c, long long caps[8]);

/* SetGeometry (initialization.f90:167-255, initialization_3d.f90:170-279),
 * including the periodic geo halo and the reference's obstacle-cell rule.
 * geo has array_size entries; sizes[8] receives the list lengths in the
 * order of imexlb_host_list_capacity. bf/bb may be NULL in 2D. Returns
 * IMEXLB_ERR_GEOMETRY when an obstacle probe leaves the geo array (where the
 * reference reads undefined memory). */
int imexlb_host_set_geometry(const imexlb_config* c, int* geo, int* fluid_id, int* bl, int* br,
                             int* bu, int* bd, int* bf, int* bb, int* b_user, int sizes[8]);

/* imexlb_host_set_geometry computed by kernels on CUDA device `device` (the
 * interior test, PassInt's periodic wrap, ordered compaction of fluid_id and
 * the rim lists, one thread per x-row for the obstacle scan) and copied into
 * the same host arrays with the same sizes: identical results, without a
 * host loop over every padded cell. For hosts that set up many cases (an
 * ensemble generator). Returns IMEXLB_ERR_CUDA (message in
 * imexlb_last_error(NULL)) when the device work fails. No counterpart in the
 * reference. */
int imexlb_device_set_geometry(const imexlb_config* c, int device, int* geo, int* fluid_id,
                               int* bl, int* br, int* bu, int* bd, int* bf, int* bb,
                               int* b_user, int sizes[8]);

/* SetGeometry in the stages a multi-rank host needs (initialization.f90:
 * 167-255): the geometry and wall lists of this rank's box without PassInt
 * (sizes[7] in the order fluid_id, bl, br, bu, bd, bf, bb); PassInt(geo)
 * across the ranks of a group (geo[r] is rank r's array, boxes from
 * imexlb_host_rank_layout); and the reference's obstacle scan on a geo whose
 * ghost layers are filled (IMEXLB_ERR_GEOMETRY when a probe leaves the
 * array). imexlb_host_set_geometry is the three with one periodic rank. */
int imexlb_host_geometry_lists(const imexlb_config* c, int* geo, int* fluid_id, int* bl, int* br,
                               int* bu, int* bd, int* bf, int* bb, int sizes[7]);
int imexlb_host_group_pass_int(const imexlb_config* c, const int np[3], int nprocs,
                               int* const* geo);
int imexlb_host_obstacle_scan(const imexlb_config* c, const int* geo, int* b_user, int* n_user);

/* SetCartesian (cart_mpi.f90:57-103, cart_mpi_3d.f90:57-103): ranks per
 * dimension for nprocs ranks and global lengths gl = n+1. */
int imexlb_host_decompose(int dim, const int gl[3], int nprocs, int np[3]);

/* SetLocalLength (cart_mpi.f90:105-136) for MPI rank `rank` of the np grid
 * (row-major Cartesian coordinates, as MPI_Cart_coords without
 * reordering): sets local_length, local_start, dy, dz, array_size of a
 * derived config. IMEXLB_ERR_ARG when a length is below the ghost width. */
int imexlb_host_rank_layout(imexlb_config* c, const int np[3], int rank);

/* Obstacle cells for the corrected-physics mode (no counterpart in the
 * reference, which keeps at most one cell per x-row and probes
 * geo(id + e_x + dy*(iq*dim+1)), initialization.f90:232-253): every
 * interior solid cell with a fluid neighbour id + e_x + dy*e_y + dz*e_z,
 * in x-fastest order. Replaces SetGeometry's b_user list when a host wants
 * every solid link bounced; results then differ from the reference's.
 * b_user needs array_size entries. */
int imexlb_host_obstacle_cells(const imexlb_config* c, const int* geo, int* b_user, int* n_user);

/* 100 perturbation draws: splitmix64(seed) -> 53-bit uniforms in [0,1).
 * A Fortran host passes its own random_number draws instead. */
void imexlb_host_r_vec(unsigned long long seed, double* r_vec /* 100 */);

/* InitUP (initialization.f90:259-282, initialization_3d.f90:282-308) into
 * p[array_size], u[array_size*dim]; other entries are left as they are. */
int imexlb_host_init_up(const imexlb_config* c, const int* geo, const double* r_vec, double* p,
                        double* u);

/* WriteBinary with one rank (lbm.f90:231-413, lbm_3d.f90:233-449): the
 * Tecplot #!TDV112 binary file of x, y[, z], p, ux, uy[, uz] in the
 * reference's units (lengths / charlength, p * charlength / t_intv^2,
 * u / (charlength * t_intv)), zone "ZONE nnn" with nnn = count, solution time
 * iter / t_intv, min/max over fluid_id(1:). p and u in the reference layout. */
int imexlb_host_write_plt(const imexlb_config* c, const char* path, int count, int iter,
                          const double* p, const double* u, const int* fluid_id, int size_fluid);

/* Fill an imexlb_desc from the configuration. */
int imexlb_host_make_desc(const imexlb_config* c, int precision, int device, imexlb_desc* d);

#ifdef __cplusplus
}
#endif
#endif /* IMEXLB_HOST_H */
