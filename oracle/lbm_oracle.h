/*
 * CPU oracle for the IMEXLB-1.0 single-rank lattice Boltzmann step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark compare against. Nothing in
 * the product library links, loads or calls it.
 *
 * PARITY UNPINNED by the reference: the reference ships no tests, fixtures or
 * golden data, and it cannot be built here (Fortran + MPI). This restatement
 * is pinned instead by known-answer tests derived from the reference's
 * formulas and input files, and by a second, independently written numpy
 * restatement that must agree with it bit for bit (tests/golden/).
 *
 * It restates, in plain C, the serial (CPU-build) semantics of the Fortran
 * reference with one MPI rank:
 *   initialization.f90:59-102 / initialization_3d.f90:60-103   DataInput
 *   initialization.f90:112-123 / initialization_3d.f90:108-122 InitLattice
 *   initialization.f90:167-255 / initialization_3d.f90:170-279 SetGeometry
 *   initialization.f90:259-282 / initialization_3d.f90:282-308 InitUP
 *   lbm.f90:24-48     InitPDF          lbm.f90:52-76   Collision
 *   lbm.f90:96-155    BoundaryCondition (cart_mpi.f90:240-277 PassF, one rank)
 *   lbm.f90:80-92     Propagation      lbm.f90:159-201 PostProcessing
 *   lbm.f90:205-227   Monitor          main.f90:48-63  step order
 * (the _3d files at the same places for D3Q27). Arrays keep the reference
 * layout: padded, 0-based, array-of-structures (f[id*nq+iq], u[id*dim+k]).
 *
 * Arithmetic follows the reference's evaluation order in IEEE double with no
 * contraction (build with -ffp-contract=off). Reads the reference would make
 * outside its arrays return NaN and are counted in oob_reads; the reference's
 * own result there is undefined.
 *
 * Parity status: the reference ships no tests or golden data and cannot be
 * compiled in this environment (Fortran + MPI), so this oracle is pinned by
 * known-answer tests derived from the reference's formulas and input files.
 */
#ifndef IMEXLB_ORACLE_H
#define IMEXLB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_GHOST 3

/* The four lines of input.in (input.in:1-4) plus the dimension. */
typedef struct orc_input {
  int dim;                 /* 2 (D2Q9) or 3 (D3Q27) */
  int nx, ny, nz;          /* line 1 */
  double charlength, xpos, re;   /* line 2, in units of nx */
  double ome, dt, rho0;          /* line 3 */
  double max_t, inter;           /* line 4 */
} orc_input;

typedef struct orc_state {
  int dim, nq;
  int nx, ny, nz;
  /* DataInput results (lattice units) */
  double charlength, pos, re, uu, ma, radius;
  double nu, rho0, dt, ome, tau, t_intv, inter, max_t;
  int max_step, interv;
  /* single-rank Cartesian layout (cart_mpi.f90:63-64,105-136) */
  int L[3];                /* local_length = n+1 nodes per dimension */
  int dy, dz;
  long long array_size;
  /* lattice */
  double t[27];
  int e[81];
  /* fields, reference layout */
  double *f, *fb, *p, *u;
  int *geo, *fluid_id, *bl, *br, *bu, *bd, *bf, *bb, *b_user;
  int size_fluid, l_size, r_size, u_size, d_size, f_size, b_size, user_size;
  /* diagnostics */
  long long oob_reads;     /* fb reads outside the array made by the BC loops */
  int geom_error;          /* 1: obstacle-cell probe left the geo array */
  int nthreads;            /* OpenMP threads for the per-cell loops (0 = runtime default) */
  int start[3];            /* local_start: global position of local node 0 (0 with one rank) */
} orc_state;

/* The reference run with nprocs MPI ranks (cart_mpi.f90, cart_mpi_3d.f90):
 * the Cartesian decomposition of SetCartesian / SetLocalLength, one state per
 * rank with its own local arrays, lists and obstacle scan, PassInt / PassF as
 * exchanges of the 3-deep ghost layers between the rank arrays, Monitor as
 * the maximum over the ranks' own Monitor values. Rank r has the
 * row-major Cartesian coordinates of MPI_Cart_coords (no reordering). */
typedef struct orc_group {
  int dim, nprocs;
  int np[3];               /* ranks per dimension (cart_num_procs) */
  int gl[3];               /* global_length = n+1 */
  int (*cc)[3];            /* Cartesian coordinates of each rank */
  orc_state* r;            /* the ranks' states */
} orc_group;

/* DataInput: parse an input.in / input_3d.in file. Returns 0 on success. */
int orc_read_input(const char* path, int dim, orc_input* in);

/* DataInput (derived quantities) + MPISetup (one rank) + InitLattice +
 * AllocateArrays (zero-filled) + SetGeometry. Returns 0 on success. */
int orc_setup(orc_state* s, const orc_input* in);
void orc_free(orc_state* s);

/* Replace b_user with the corrected-physics obstacle list: every interior
 * solid node with a fluid neighbour x + e_iq (proper dy*e_y + dz*e_z
 * offsets), instead of the reference's first-per-x-row rule. */
void orc_corrected_obstacles(orc_state* s);

/* InitUP with the 100 perturbation draws supplied by the caller. */
void orc_init_up(orc_state* s, const double* r_vec);
void orc_init_pdf(orc_state* s);

void orc_collision(orc_state* s);
void orc_pass_f(orc_state* s, double* a);         /* PassF with one periodic rank */
void orc_bc_copies(orc_state* s, double* a);      /* BoundaryCondition after PassF */
void orc_boundary_condition(orc_state* s);
void orc_propagation(orc_state* s);
void orc_post_processing(orc_state* s);
double orc_monitor(const orc_state* s);           /* max |(ux,uy)| over fluid_id(1:) */

/* Iterations iter0 .. iter0+nsteps-1 of main.f90:48-63. Monitor runs before
 * Collision when iter % interv == 0 (interv <= 0: never); its values go to
 * umax_log (may be NULL). Returns the number of Monitor values. */
int orc_run(orc_state* s, int iter0, int nsteps, int interv, double* umax_log);

/* Apply only the BoundaryCondition copy program (PassF wrap, Up, Down, User,
 * Inlet, Outlet) to an arbitrary array laid out like fb. */
void orc_apply_bc(orc_state* s, double* a);

/* Momentum-exchange force on the obstacle from the post-BC fb of the last
 * iteration (no reference counterpart): over every link from a fluid node x
 * to an interior solid node s = x + e_i,
 *   F += e_i * (fb(x, i) + fb(s, nq-1-i)),
 * accumulated in double-double in fluid_id / iq order. F has dim entries;
 * returns the number of links. */
int orc_forces(const orc_state* s, double* F);

/* Sum of f over all fluid nodes (the mass deviation 3*sum(p)), accumulated
 * in double-double in fluid_id / iq order. */
double orc_mass(const orc_state* s);

/* Deterministic perturbation draws used when no Fortran random_number stream
 * is supplied: splitmix64(seed) -> 53-bit uniforms in [0,1). */
void orc_r_vec(unsigned long long seed, double* r_vec /* 100 */);

/* SetCartesian (cart_mpi.f90:57-103, cart_mpi_3d.f90:57-103): the ranks per
 * dimension chosen for nprocs ranks and the global lengths gl. */
void orc_decompose(int dim, const int gl[3], int nprocs, int np[3]);

/* SetLocalLength (cart_mpi.f90:105-136): local length and start of the rank
 * at Cartesian coordinates cc. Returns -3 if a length is below the ghost
 * width (the reference aborts). */
int orc_local_box(int dim, const int gl[3], const int np[3], const int cc[3], int L[3],
                  int start[3]);

/* One rank of a multi-rank run on its own (for a driver that exchanges the
 * ghost layers itself): DataInput, the local box, InitLattice,
 * AllocateArrays and SetGeometry up to PassInt(geo); after the caller has
 * filled geo's ghost layers, orc_obstacle_scan finishes SetGeometry
 * (returns -2 if a probe left the geo array). */
int orc_setup_rank(orc_state* s, const orc_input* in, const int L[3], const int start[3]);
int orc_obstacle_scan(orc_state* s);

/* Rank group: DataInput + MPISetup + InitLattice + AllocateArrays +
 * SetGeometry (with PassInt(geo) between the ranks) for nprocs ranks.
 * Returns 0, -2 (an obstacle probe left some rank's geo array), -3 (a local
 * length below the ghost width) or another negative code. */
int orc_group_setup(orc_group* g, const orc_input* in, int nprocs);
void orc_group_free(orc_group* g);
/* PassF between the ranks on array fb (every rank's ghost layers receive the
 * owner's interior cells at the globally periodic position). */
void orc_group_pass_f(orc_group* g);
/* InitUP on every rank; r_vecs holds 100 draws per rank (each rank calls
 * random_number itself in the reference). */
void orc_group_init_up(orc_group* g, const double* r_vecs);
void orc_group_init_pdf(orc_group* g);
double orc_group_monitor(const orc_group* g);
/* main.f90:48-63 on every rank, with PassF between Collision and the
 * boundary copies. Returns the number of Monitor values. */
int orc_group_run(orc_group* g, int iter0, int nsteps, int interv, double* umax_log);

#ifdef __cplusplus
}
#endif
#endif
