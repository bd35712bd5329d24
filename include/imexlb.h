/*
 * imexlb.h -- C ABI of the GB300 lattice Boltzmann step library (libimexlb).
 *
 * The library replaces the per-timestep part of IMEXLB-1.0's time loop for one
 * MPI rank on one GPU: Collision, BoundaryCondition (including PassF's halo
 * copy), Propagation, PostProcessing and Monitor (main.f90:48-63). The host
 * keeps the reference's setup (DataInput, MPISetup, InitLattice,
 * AllocateArrays, SetGeometry, InitUP) and hands its arrays over in the
 * reference layout: padded 0-based 1-D arrays, f(id*nq+iq), u(id*dim+k),
 * id = (x+3) + dy*(y+3) [+ dz*(z+3)] (initialization.f90:33-53,171-183).
 *
 * Conventions
 *   - Every function returns 0 (IMEXLB_OK) or a negative IMEXLB_ERR_* code;
 *     imexlb_last_error() then holds a message. Nothing unwinds across the ABI.
 *   - Host arrays belong to the caller and are only read or written during the
 *     call. Device memory belongs to the handle.
 *   - Fortran callers bind these with ISO_C_BINDING: integer = c_int,
 *     double precision = c_double, arrays passed by reference.
 *   - One handle is used by one host thread; calls are ordered on the handle's
 *     own CUDA stream and return after the work they describe is complete.
 */
#ifndef IMEXLB_H
#define IMEXLB_H

#ifdef __cplusplus
extern "C" {
#endif

#define IMEXLB_VERSION_MAJOR 1
#define IMEXLB_VERSION_MINOR 0

enum {
  IMEXLB_OK = 0,
  IMEXLB_ERR_ARG = -1,         /* bad argument or descriptor */
  IMEXLB_ERR_CUDA = -2,        /* CUDA runtime error */
  IMEXLB_ERR_STATE = -3,       /* call out of order (e.g. step before upload) */
  IMEXLB_ERR_GEOMETRY = -4,    /* geometry the reference itself leaves undefined */
  IMEXLB_ERR_UNSUPPORTED = -5, /* e.g. a multi-rank decomposition */
  IMEXLB_ERR_NOMEM = -6,       /* host or device allocation failed */
  IMEXLB_ERR_DIVERGED = -7,    /* watchdog: a Monitor value is NaN or infinite */
  IMEXLB_ERR_TIMEOUT = -8      /* a bounded device-side wait gave up */
};

/* Arithmetic / storage of the populations. The reduced-precision kinds store
 * the reference's f (already the deviation f_i - t_i*rho0 from rest) in a
 * narrow type and collide in FP32; forces and mass stay FP64. They are not
 * bit-compatible with the reference. */
enum {
  IMEXLB_FP64 = 0, /* reference arithmetic: IEEE double, reference evaluation order, no FMA */
  IMEXLB_FP64_FAST = 1, /* double storage and arithmetic, minimal operation count with fused
                           multiply-adds: agrees with the reference to rounding, not bitwise */
  IMEXLB_FP32 = 2, /* FP32 storage, FP32 arithmetic */
  IMEXLB_BF16 = 3, /* bfloat16 storage, FP32 arithmetic */
  IMEXLB_FP16 = 4, /* IEEE half storage, FP32 arithmetic */
  IMEXLB_FIX64 = 5 /* 64-bit fixed-point storage (value * 2^60 as a signed integer) and
                      integer arithmetic with round-to-nearest products: the FP64 drop-in's
                      accuracy (agrees with the reference within 1e-12 relative) on the
                      integer pipes. Needs rho0 = 1 and 0 < ome < 2; a node whose populations
                      reach |f| >= 4 or moments |S| >= 2, |u_k| >= 0.25 turns NaN. */
};

/* Everything the reference's lbm module reads from module globals
 * (initialization.f90:14-53, cart_mpi.f90:10-43). */
typedef struct imexlb_desc {
  int dim;              /* 2 (D2Q9) or 3 (D3Q27): cart_mpi.f90:10 */
  int nq;               /* 9 or 27 */
  int ghost;            /* must be 3: cart_mpi.f90:10 */
  int nx, ny, nz;       /* lattice extents; nodes 0..n per dimension (nz ignored in 2D) */
  int local_length[3];  /* cart_mpi.f90:105-111; one rank: n+1 */
  int local_start[3];   /* cart_mpi.f90:125-126; one rank: 0 */
  int dy, dz;           /* index strides: initialization.f90:171, initialization_3d.f90:175-176 */
  double ome;           /* relaxation parameter (input.in line 3) */
  double rho0;          /* reference density (input.in line 3) */
  double uu;            /* peak inlet velocity: initialization.f90:78 */
  double t[27];         /* lattice weights, InitLattice order */
  int e[81];            /* lattice velocities, e[iq*dim+k] */
  int precision;        /* IMEXLB_FP64, IMEXLB_FP64_FAST, IMEXLB_FP32, IMEXLB_BF16, IMEXLB_FP16,
                           IMEXLB_FIX64 */
  int device;           /* CUDA device ordinal, e.g. mod(rank, ndev) as main.f90:31 */
} imexlb_desc;

typedef struct imexlb_s imexlb_t;

/* Sizes of the device-side state, for diagnostics and benchmarks. */
typedef struct imexlb_info {
  long long array_size;   /* padded cells */
  long long interior;     /* (nx+1)(ny+1)[(nz+1)] lattice nodes */
  long long size_fluid;   /* fluid nodes */
  long long n_fill;       /* copies of the boundary program per iteration */
  long long n_user;       /* obstacle (b_user) cells */
  long long n_links;      /* fluid->obstacle links of the force sum */
  long long device_bytes; /* device memory held by the handle */
} imexlb_info;

/* Create a handle on desc->device. Replaces the device mapping of
 * main.f90:31-33. Only the single-rank layout is accepted. */
int imexlb_create(imexlb_t** h, const imexlb_desc* d);

/* Geometry from SetGeometry (initialization.f90:167-255): geo[array_size],
 * the fluid index list and the boundary index lists bl, br, bu, bd, b_user
 * with their lengths (2D: bu/bd are the y walls; 3D: the z walls, y is
 * periodic). The library runs the reference's BoundaryCondition copy program
 * once over slot names and stores, for every boundary slot a fluid node
 * pulls, the slot whose post-collision value it holds (lbm.f90:96-155,
 * cart_mpi.f90:240-277). Returns IMEXLB_ERR_GEOMETRY when such a slot would
 * take a value the reference reads outside its arrays. */
int imexlb_set_geometry(imexlb_t* h, const int* geo, const int* fluid_id, int size_fluid,
                        const int* bl, int l_size, const int* br, int r_size,
                        const int* bu, int u_size, const int* bd, int d_size,
                        const int* b_user, int user_size);

/* Copy f, fb, p, u (reference layout, host) to the device. This is the state
 * after InitUP + InitPDF, or any state the reference holds between two
 * iterations of main.f90:48-63. fb matters where the step never writes it:
 * obstacle cells (b_user, lbm.f90:126-133) and solid cells. */
int imexlb_upload(imexlb_t* h, const double* f, const double* fb, const double* p, const double* u);

/* The initial state computed on the device instead of uploaded: f = fb = 0
 * (the reference's fresh allocation) and, with r_vec (100 draws), InitUP
 * (initialization.f90:259-282, initialization_3d.f90:282-308) for this
 * handle's box: p = 0, u_x = uu*4*y*(n-y)/n**2*r on fluid nodes, the other
 * components 0; with r_vec == NULL the rest state p = u = 0. Same bits as
 * imexlb_host_init_up + imexlb_upload of zero f and fb, without copying four
 * full arrays from the host (an ensemble sets up hundreds of cases). Follow
 * with imexlb_init_pdf. No counterpart in the reference. */
int imexlb_init_state(imexlb_t* h, const double* r_vec);

/* InitPDF on the device: f = feq(p, u) on fluid nodes (lbm.f90:24-48). */
int imexlb_init_pdf(imexlb_t* h);

/* Advance iterations iter0 .. iter0+nsteps-1 of main.f90:48-63: for each,
 * Monitor when interv > 0 and iter % interv == 0 (max |(ux,uy)| over
 * fluid_id(1:), lbm.f90:205-227, unscaled), then Collision, BoundaryCondition,
 * Propagation, PostProcessing. umax_log (may be NULL) receives one value per
 * Monitor call in order. */
int imexlb_step(imexlb_t* h, int iter0, int nsteps, int interv, double* umax_log);

/* Additions with no reference counterpart (Cd/Cl and mass monitoring).
 *
 * imexlb_observe: from the current state (after the last iteration's
 * BoundaryCondition, or as uploaded), the momentum-exchange force on the
 * obstacle, F = sum over links from a fluid node x to an interior solid node
 * s = x + e_i of e_i * (fb(x,i) + fb(s, nq-1-i)) (dim values), and the mass
 * deviation sum(f) over fluid nodes. Both are accumulated in double-double
 * with a fixed reduction order. Either pointer may be NULL.
 *
 * imexlb_step_observed: imexlb_step that also records F after the
 * BoundaryCondition of every iteration with iter % every == 0 (every > 0)
 * into force_log (dim values per sample, in order). */
int imexlb_observe(imexlb_t* h, double* force, double* mass);
int imexlb_step_observed(imexlb_t* h, int iter0, int nsteps, int interv, double* umax_log,
                         int every, double* force_log);

/* ---- Ensembles (no reference counterpart) ----------------------------------
 * Many independent cases advanced together, e.g. a data-generation ensemble
 * of cylinder flows of different sizes. Each case is an ordinary handle
 * (geometry set, state uploaded, at least one iteration taken with
 * imexlb_step); all cases share one device, dimension and reduced-precision
 * storage kind (IMEXLB_FP32/BF16/FP16). A batch advances every case with one
 * collide launch and one boundary launch per iteration (whatever the cases'
 * imexlb_set_fill_mode), replayed from a CUDA graph; cases with a smaller
 * iteration budget drop out along the way.
 * Monitor and force sampling are not recorded inside a batch call; the cases'
 * handles remain usable (download, observe, step) between calls. */
typedef struct imexlb_batch_s imexlb_batch_t;
int imexlb_batch_create(imexlb_batch_t** b, imexlb_t* const* cases, int ncases);
/* Time every launch shape (threads per block x nodes per thread) over `trial`
 * iterations of all cases (the cases advance by them) and keep the fastest;
 * *shape (may be NULL) receives its index. */
int imexlb_batch_tune(imexlb_batch_t* b, int trial, int* shape);
/* Advance case i by steps[i] iterations (steps NULL: every case by nsteps). */
int imexlb_batch_step(imexlb_batch_t* b, int nsteps, const int* steps);
/* How imexlb_batch_step runs a call. LOCKSTEP (the default): one collide and
 * one boundary launch per iteration, replayed from a CUDA graph.
 * PERSISTENT: one cooperative launch of resident blocks runs every iteration
 * of the call; each case advances as soon as its own previous iteration's
 * boundary copies are done (no grid-wide step between iterations). Its
 * device-side waits are bounded (2 s each): a wait that runs out makes the
 * call return IMEXLB_ERR_TIMEOUT, and the cases' states are then undefined.
 * PERSISTENT takes at most 2048 cases. Both modes give the same results up to
 * the compiler's choice of fused multiply-adds in the two kernels. */
#define IMEXLB_BATCH_LOCKSTEP 0
#define IMEXLB_BATCH_PERSISTENT 1
int imexlb_batch_set_mode(imexlb_batch_t* b, int mode);
void imexlb_batch_destroy(imexlb_batch_t* b);
const char* imexlb_batch_last_error(const imexlb_batch_t* b);

/* Fields of the current state of a 2D handle sampled at the W x H pixel
 * centres of the node lattice (bilinear between nodes; solid nodes count as
 * p = u = 0): out[0:WH) fluid fraction, then p, ux, uy (each W*H, x fastest).
 * Needs at least one iteration since the last upload. */
int imexlb_sample(imexlb_t* h, int W, int H, float* out);

/* Copy the state back in the reference layout: f, p, u after the last
 * PostProcessing and fb after the last BoundaryCondition. Any pointer may be
 * NULL. fb slots that the reference fills from outside its arrays are NaN. */
int imexlb_download(imexlb_t* h, double* f, double* fb, double* p, double* u);

/* Sizes of the device state. */
int imexlb_get_info(const imexlb_t* h, imexlb_info* info);

/* Kernel accounting of imexlb_step: launches of each kernel kind since the
 * last imexlb_profile_reset, and (when timing is on) their summed device time
 * from CUDA events recorded around each launch on the handle's stream. */
enum {
  IMEXLB_KERNEL_STEP = 0,    /* fused pull-collide iteration */
  IMEXLB_KERNEL_FILL = 1,    /* boundary-slot refresh after a collision */
  IMEXLB_KERNEL_FIRST = 2,   /* collision from uploaded f, p, u */
  IMEXLB_KERNEL_OTHER = 3,   /* layout conversion, finalize, init */
  IMEXLB_KERNEL_KINDS = 4
};
typedef struct imexlb_profile {
  long long launches[IMEXLB_KERNEL_KINDS];
  double ms[IMEXLB_KERNEL_KINDS];  /* 0 unless timing was on */
} imexlb_profile;
int imexlb_profile_reset(imexlb_t* h, int timing);
int imexlb_profile_read(const imexlb_t* h, imexlb_profile* out);

/* Divergence watchdog (no counterpart in the reference, whose Monitor prints
 * NaN and carries on, lbm.f90:212-226). With on != 0, imexlb_step and
 * imexlb_step_observed return IMEXLB_ERR_DIVERGED when a Monitor value of
 * the call (interv > 0) is NaN or infinite; imexlb_last_error names the
 * first such iteration. The call's iterations have all run and umax_log is
 * filled, so the caller can download the state for inspection. Off by
 * default. */
int imexlb_set_watchdog(imexlb_t* h, int on);

/* The cudaStream_t all work of the handle is ordered on (for host timing). */
int imexlb_get_stream(const imexlb_t* h, void** stream);

/* Diagnostics: the FP64 fused multiply-add throughput of a device (per
 * second), measured by a short kernel with independent chains; the bound of
 * the IMEXLB_FP64 step kernel, whose additions run as exact fused
 * multiply-adds. No counterpart in the reference. */
int imexlb_fp64_fma_rate(int device, double* fma_per_s);

/* Variants of the reference-rounding (IMEXLB_FP64) step kernel. They differ
 * only in how each IEEE round-to-nearest operation is issued, never in its
 * result. Variant 0 issues the DADD/DMUL/DDIV instructions as the reference
 * writes them; variant 1, the default and the fastest measured on GB300,
 * issues the additions as fused multiply-adds with exact operands (a*1+b,
 * b*(-1)+a, a*b+(-0)) and the division by 3 of the density and every
 * multiplication as an integer emulation that returns the hardware's bits.
 * Applies when rho0 == 1 (the reference's value); other rho0 use variant 0.
 * No counterpart in the reference. imexlb_fp64_splits() is the number of
 * variants; imexlb_set_fp64_split() takes effect at the next imexlb_step. */
int imexlb_fp64_splits(void);
int imexlb_set_fp64_split(imexlb_t* h, int split);

/* Where the boundary copies of each iteration run (the reference's
 * BoundaryCondition, lbm.f90:96-155 / lbm_3d.f90:96-157, which
 * imexlb_set_geometry resolves into slot-to-slot copies).
 * IMEXLB_FILL_FUSED: inside the step kernel, one launch per iteration. A
 * fluid node that pulls a ghost slot reads that copy's source instead
 * (closed forms on the inlet, outlet, wall and periodic faces, a per-node
 * source row on edges), and obstacle slots are written by the thread that
 * has just written their source. IMEXLB_FILL_KERNEL: a separate kernel after
 * each step writes every pulled boundary slot. Results are identical. The
 * default is FUSED (faster for every kernel on GB300); IMEXLB_FP64 fuses its
 * default kernel variant (imexlb_set_fp64_split) only.
 * FUSED needs 32-bit slot indices (nq * cells < 2^31), a single-rank handle
 * (the ranks of an imexlb_group run their group's copy program) and a
 * boundary program whose ghost slots do not copy an obstacle slot of the
 * previous iteration; otherwise imexlb_set_fill_mode(FUSED) returns
 * IMEXLB_ERR_UNSUPPORTED and the handle keeps the separate kernel. Takes effect at the next
 * imexlb_step; imexlb_get_fill_mode reports the mode the next step uses.
 * No counterpart in the reference. */
#define IMEXLB_FILL_KERNEL 0
#define IMEXLB_FILL_FUSED 1
int imexlb_set_fill_mode(imexlb_t* h, int mode);
int imexlb_get_fill_mode(const imexlb_t* h, int* mode);

void imexlb_destroy(imexlb_t* h);

/* Multi-rank runs (cart_mpi.f90 with nprocs MPI ranks) on one device. The
 * reference's results depend on the rank count: every rank runs SetGeometry
 * (its own obstacle scan), InitUP (r_vec indexed by local id), the boundary
 * copies and Monitor's fluid_id(0) skip on its own array, and PassF fills
 * its ghost layers from the neighbour ranks. Each rank is a handle created
 * with its rank's local_start / local_length (SetLocalLength of the
 * SetCartesian decomposition, see imexlb_host_decompose and
 * imexlb_host_rank_layout; MPI rank r has row-major Cartesian coordinates)
 * and given its own lists with imexlb_set_geometry; ranks[r] is MPI rank r.
 * imexlb_group_step advances all ranks; its Monitor values are the maximum
 * over the ranks (MPI_REDUCE MAX). Upload, InitPDF and download stay per
 * rank (a download completes every rank's ghost slots first). A rank handle
 * cannot be stepped alone, and IMEXLB_FP64 only. Destroy the group before
 * its ranks. No counterpart in the reference (it is the MPI program's
 * single-device form). */
typedef struct imexlb_group_s imexlb_group_t;
int imexlb_group_create(imexlb_group_t** g, imexlb_t* const* ranks, int nprocs);
int imexlb_group_step(imexlb_group_t* g, int iter0, int nsteps, int interv, double* umax_log);
void imexlb_group_destroy(imexlb_group_t* g);
const char* imexlb_group_last_error(const imexlb_group_t* g);

/* Largest fluid_id list imexlb_monitor_noalloc accepts. */
#define IMEXLB_NOALLOC_MAX_FLUID 16777216

/* Monitor without any allocation. No counterpart in the reference: it is an
 * addition for hosts that cannot let a library call cudaMalloc, such as a
 * Fortran host whose u and fluid_id live in device memory mapped by its
 * OpenMP offload runtime (use_device_ptr), or an application that has
 * reserved the device memory for its own pool.
 *
 * Computes the value Monitor reduces (lbm.f90:211-217): the maximum of
 * sqrt(u(id*dim)**2 + u(id*dim+1)**2) over fluid_id(1 : size_fluid-1), on the
 * caller's device arrays in the reference layout (u[id*dim+k], fluid_id as
 * SetGeometry builds it), and stores it to the device double *umax. Work is
 * enqueued on `stream` (NULL: the default stream) of the calling thread's
 * current device; the call does not wait for it.
 *
 * Scratch is a fixed 64 KB array in device memory that every GPU loading the
 * library holds until the process exits; it limits size_fluid to
 * IMEXLB_NOALLOC_MAX_FLUID (larger lists return IMEXLB_ERR_ARG). The first
 * call on a device looks up that array's address (cudaGetSymbolAddress); make
 * that first call before any stream capture. The address is kept per device
 * and context: after a device reset the next call looks it up again (make
 * that call outside stream capture too). All calls on a device share the
 * array: calls whose work overlaps on the GPU race and must be ordered by the
 * caller (e.g. one stream). Each call rewrites every scratch entry it reads,
 * so nothing needs clearing between calls. A CUDA error already pending when
 * the call starts is left in place and returned as IMEXLB_ERR_CUDA with
 * nothing launched. */
int imexlb_monitor_noalloc(int dim, const double* u, const int* fluid_id, int size_fluid,
                           double* umax, void* stream);

/* Message of the last failed call on h (h may be NULL for imexlb_create and
 * imexlb_monitor_noalloc). */
const char* imexlb_last_error(const imexlb_t* h);

/* "major.minor (build info)". */
const char* imexlb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* IMEXLB_H */
