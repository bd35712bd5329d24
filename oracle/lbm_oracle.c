/*
 * CPU oracle for the IMEXLB-1.0 single-rank lattice Boltzmann step.
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h): the checker for the CUDA path.
 * Parity unpinned by the reference (no reference tests or outputs exist);
 * pinned by known-answer tests and an independent numpy restatement.
 *
 * Every routine follows the serial semantics of the Fortran reference; the
 * file:line given with each function is the reference code it restates.
 * Build with -ffp-contract=off so that a*b+c is never fused.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define G ORC_GHOST

/* ------------------------------------------------------------------------ */
/* DataInput file parsing: Fortran list-directed READ, one READ per record.  */
/* initialization.f90:61-75                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  FILE* fp;
  char line[4096];
  char* cur;
  int have_line;
} rd_t;

static int rd_next_record(rd_t* r) {
  if (!fgets(r->line, sizeof r->line, r->fp)) return 0;
  r->cur = r->line;
  r->have_line = 1;
  return 1;
}

/* Next value token; continues onto following records when the current one is
 * exhausted, as list-directed input does. */
static int rd_token(rd_t* r, char* tok, size_t n) {
  for (;;) {
    if (!r->have_line && !rd_next_record(r)) return 0;
    while (*r->cur && (isspace((unsigned char)*r->cur) || *r->cur == ',')) r->cur++;
    if (*r->cur == '\0') { r->have_line = 0; continue; }
    size_t k = 0;
    while (*r->cur && !isspace((unsigned char)*r->cur) && *r->cur != ',') {
      if (k + 1 < n) tok[k++] = *r->cur;
      r->cur++;
    }
    tok[k] = '\0';
    return 1;
  }
}

static int rd_int(rd_t* r, int* v) {
  char tok[256], *end;
  if (!rd_token(r, tok, sizeof tok)) return 0;
  long x = strtol(tok, &end, 10);
  if (*end != '\0') return 0;
  *v = (int)x;
  return 1;
}

static int rd_dbl(rd_t* r, double* v) {
  char tok[256], *end;
  if (!rd_token(r, tok, sizeof tok)) return 0;
  for (char* c = tok; *c; ++c)
    if (*c == 'd' || *c == 'D' || *c == 'q' || *c == 'Q') *c = 'e';
  *v = strtod(tok, &end);
  return *end == '\0';
}

/* Each READ statement starts on a fresh record. */
static void rd_new_statement(rd_t* r) { r->have_line = 0; }

int orc_read_input(const char* path, int dim, orc_input* in) {
  rd_t r;
  memset(&r, 0, sizeof r);
  memset(in, 0, sizeof *in);
  in->dim = dim;
  r.fp = fopen(path, "r");
  if (!r.fp) return -1;
  int ok = 1;
  rd_new_statement(&r);
  ok = ok && rd_int(&r, &in->nx) && rd_int(&r, &in->ny);
  if (dim == 3) ok = ok && rd_int(&r, &in->nz);
  rd_new_statement(&r);
  ok = ok && rd_dbl(&r, &in->charlength) && rd_dbl(&r, &in->xpos) && rd_dbl(&r, &in->re);
  rd_new_statement(&r);
  ok = ok && rd_dbl(&r, &in->ome) && rd_dbl(&r, &in->dt) && rd_dbl(&r, &in->rho0);
  rd_new_statement(&r);
  ok = ok && rd_dbl(&r, &in->max_t) && rd_dbl(&r, &in->inter);
  fclose(r.fp);
  return ok ? 0 : -2;
}

/* ------------------------------------------------------------------------ */
/* helpers                                                                   */
/* ------------------------------------------------------------------------ */

static inline int wrap_c(int c, int L) {
  /* periodic image of a padded coordinate in the single-rank PassF */
  if (c < G) return c + L;
  if (c >= L + G) return c - L;
  return c;
}

static inline int is_ghost(const orc_state* s, int X, int Y, int Z) {
  if (X < G || X >= s->L[0] + G) return 1;
  if (Y < G || Y >= s->L[1] + G) return 1;
  if (s->dim == 3 && (Z < G || Z >= s->L[2] + G)) return 1;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* DataInput derived values, MPISetup (1 rank), InitLattice, Allocate,       */
/* SetGeometry                                                               */
/* ------------------------------------------------------------------------ */

/* initialization.f90:112-123 (2D), initialization_3d.f90:108-122 (3D) */
static void init_lattice(orc_state* s) {
  if (s->dim == 2) {
    for (int j = -1; j <= 1; ++j)
      for (int i = -1; i <= 1; ++i) {
        int iq = (i + 1) * 3 + (j + 1);
        s->e[iq * 2] = i;
        s->e[iq * 2 + 1] = j;
        /* 0.75 is a default-real literal: the product is formed in single
         * precision (exactly) and divided by 9 in double. */
        float a = 4.0f * (1.0f - 0.75f * (float)(i * i));
        a = a * (1.0f - 0.75f * (float)(j * j));
        s->t[iq] = (double)a / 9.0;
      }
  } else {
    for (int j = -1; j <= 1; ++j)
      for (int i = -1; i <= 1; ++i)
        for (int k = -1; k <= 1; ++k) {
          int iq = (k + 1) * 9 + (i + 1) * 3 + (j + 1);
          s->e[iq * 3] = i;
          s->e[iq * 3 + 1] = j;
          s->e[iq * 3 + 2] = k;
          int n = abs(i) + abs(j) + abs(k);
          double p4 = 1.0;
          for (int m = 0; m < n; ++m) p4 = p4 * 4.0;
          s->t[iq] = 8.0 / p4 / 27.0;
        }
  }
}

/* PassInt / PassF with one rank: every ghost cell receives the interior cell
 * one period away (cart_mpi.f90:142-277; send slabs are interior, receive
 * slabs are the 3-deep ghost layers, so the order of the messages does not
 * matter). */
static void wrap_int(orc_state* s, int* a) {
  int PX = s->L[0] + 2 * G, PY = s->L[1] + 2 * G, PZ = s->dim == 3 ? s->L[2] + 2 * G : 1;
  for (int Z = 0; Z < PZ; ++Z)
    for (int Y = 0; Y < PY; ++Y)
      for (int X = 0; X < PX; ++X) {
        if (!is_ghost(s, X, Y, Z)) continue;
        int sx = wrap_c(X, s->L[0]), sy = wrap_c(Y, s->L[1]);
        int sz = s->dim == 3 ? wrap_c(Z, s->L[2]) : 0;
        long long dst = X + (long long)s->dy * Y + (long long)s->dz * Z;
        long long src = sx + (long long)s->dy * sy + (long long)s->dz * sz;
        a[dst] = a[src];
      }
}

void orc_pass_f(orc_state* s, double* a) {
  int nq = s->nq;
  int PX = s->L[0] + 2 * G, PY = s->L[1] + 2 * G, PZ = s->dim == 3 ? s->L[2] + 2 * G : 1;
  for (int Z = 0; Z < PZ; ++Z)
    for (int Y = 0; Y < PY; ++Y)
      for (int X = 0; X < PX; ++X) {
        if (!is_ghost(s, X, Y, Z)) continue;
        int sx = wrap_c(X, s->L[0]), sy = wrap_c(Y, s->L[1]);
        int sz = s->dim == 3 ? wrap_c(Z, s->L[2]) : 0;
        long long dst = X + (long long)s->dy * Y + (long long)s->dz * Z;
        long long src = sx + (long long)s->dy * sy + (long long)s->dz * sz;
        memcpy(a + dst * nq, a + src * nq, sizeof(double) * nq);
      }
}

/* SetGeometry up to PassInt: initialization.f90:167-226,
 * initialization_3d.f90:170-247. Coordinates are global (local + start). */
static void geometry_local(orc_state* s) {
  const int dim = s->dim;
  const int L0 = s->L[0], L1 = s->L[1], L2 = dim == 3 ? s->L[2] : 1;
  int idn = 0, idl = 0, idr = 0, idu = 0, idd = 0, idf = 0, idb = 0;
  const int kmax = dim == 3 ? L2 + 2 : 0;
  for (int k = 0; k <= kmax; ++k)
    for (int j = 0; j <= L1 + 2; ++j)
      for (int i = 0; i <= L0 + 2; ++i) {
        int x = i - 1, y = j - 1, z = k - 1;
        long long id = (i - 1 + G) + (long long)s->dy * (j - 1 + G);
        if (dim == 3) id += (long long)s->dz * (k - 1 + G);
        int inside = x >= 0 && x < L0 && y >= 0 && y < L1;
        if (dim == 3) inside = inside && z >= 0 && z < L2;
        x += s->start[0];
        y += s->start[1];
        z += s->start[2];
        if (inside) {
          s->geo[id] = 0;
          double ax = (double)x - s->pos;
          double ay = (double)y - s->ny / 2.0;
          double r2;
          if (dim == 2) {
            r2 = ax * ax + ay * ay;
          } else {
            double az = (double)z - s->nz / 2.0;
            r2 = ax * ax + ay * ay + az * az;
          }
          if (r2 > s->radius * s->radius) {
            s->geo[id] = 1;
            s->fluid_id[idn++] = (int)id;
          }
        } else {
          if (x == -1) s->bl[idl++] = (int)id;
          if (x == s->nx + 1) s->br[idr++] = (int)id;
          if (dim == 2) {
            if (y == -1) s->bd[idd++] = (int)id;
            if (y == s->ny + 1) s->bu[idu++] = (int)id;
          } else {
            if (y == -1) s->bf[idf++] = (int)id;
            if (y == s->ny + 1) s->bb[idb++] = (int)id;
            if (z == -1) s->bd[idd++] = (int)id;
            if (z == s->nz + 1) s->bu[idu++] = (int)id;
          }
        }
      }
  s->size_fluid = idn;
  s->l_size = idl;
  s->r_size = idr;
  s->u_size = idu;
  s->d_size = idd;
  s->f_size = idf;
  s->b_size = idb;
}

/* SetGeometry after PassInt(geo): the obstacle cells,
 * initialization.f90:232-253, initialization_3d.f90:253-277. */
static void obstacle_scan(orc_state* s) {
  const int dim = s->dim, nq = s->nq;
  const int L0 = s->L[0], L1 = s->L[1], L2 = dim == 3 ? s->L[2] : 1;
  const int kmax = dim == 3 ? L2 + 2 : 0;
  /* Obstacle cells: per x-row, the first solid cell whose probe cell
   * geo(id + e_x + dy*(iq*dim+1) [+ dz*(iq*dim+2)]) is fluid, probes taken in
   * iq order (initialization.f90:232-253, initialization_3d.f90:253-277). */
  int id_user = 0;
  for (int k = 0; k <= kmax; ++k)
    for (int j = 0; j <= L1 + 2; ++j)
      for (int i = 0; i <= L0 + 2; ++i) {
        long long id = (i - 1 + G) + (long long)s->dy * (j - 1 + G);
        if (dim == 3) id += (long long)s->dz * (k - 1 + G);
        int found = 0;
        if (s->geo[id] == 0) {
          for (int iq = 0; iq < nq; ++iq) {
            long long pr = id + s->e[iq * dim] + (long long)s->dy * (iq * dim + 1);
            if (dim == 3) pr += (long long)s->dz * (iq * dim + 2);
            if (pr < 0 || pr >= s->array_size) {
              s->geom_error = 1;
              continue;
            }
            if (s->geo[pr] == 1) {
              s->b_user[id_user++] = (int)id;
              found = 1;
              break;
            }
          }
        }
        if (found) break;
      }
  s->user_size = id_user;
}

/* Corrected-physics obstacle list (not the reference's rule): every
 * interior solid node (x, y[, z]) in 0..n with a fluid node at x + e_iq for
 * some iq, scanned z, y, x. Clears the reference rule's probe error, which
 * concerns only that rule. */
void orc_corrected_obstacles(orc_state* s) {
  const int dim = s->dim, nq = s->nq;
  const int nzl = dim == 3 ? s->nz : 0;
  int n = 0;
  for (int z = 0; z <= nzl; ++z)
    for (int y = 0; y <= s->ny; ++y)
      for (int x = 0; x <= s->nx; ++x) {
        long long id = (x + G) + (long long)s->dy * (y + G);
        if (dim == 3) id += (long long)s->dz * (z + G);
        if (s->geo[id] != 0) continue;
        int wet = 0;
        for (int iq = 0; iq < nq && !wet; ++iq) {
          long long nb = id + s->e[iq * dim] + (long long)s->dy * s->e[iq * dim + 1];
          if (dim == 3) nb += (long long)s->dz * s->e[iq * dim + 2];
          wet = s->geo[nb] == 1;
        }
        if (wet) s->b_user[n++] = (int)id;
      }
  s->user_size = n;
  s->geom_error = 0;
}

void orc_free(orc_state* s) {
  free(s->f); free(s->fb); free(s->p); free(s->u);
  free(s->geo); free(s->fluid_id);
  free(s->bl); free(s->br); free(s->bu); free(s->bd); free(s->bf); free(s->bb);
  free(s->b_user);
  memset(s, 0, sizeof *s);
}

/* DataInput derived values, initialization.f90:65-81 */
static int data_input(orc_state* s, const orc_input* in) {
  memset(s, 0, sizeof *s);
  if (in->dim != 2 && in->dim != 3) return -1;
  s->dim = in->dim;
  s->nq = in->dim == 2 ? 9 : 27;
  s->nx = in->nx;
  s->ny = in->ny;
  s->nz = in->dim == 3 ? in->nz : 0;
  s->charlength = in->charlength * s->nx;
  s->pos = in->xpos * s->nx;
  s->re = in->re;
  s->ome = in->ome;
  s->dt = in->dt;
  s->rho0 = in->rho0;
  s->max_t = in->max_t;
  s->inter = in->inter;
  s->nu = (2.0 - s->ome) * s->dt / (6.0 * s->ome);
  s->t_intv = s->charlength * s->charlength / s->nu;
  s->interv = (int)(s->inter * s->t_intv);
  s->max_step = (int)(s->max_t * s->t_intv);
  s->uu = s->re * s->nu / s->charlength;
  s->tau = 3 * s->nu;
  s->ma = s->uu * sqrt(3.0);
  s->radius = s->charlength * 0.5;
  return 0;
}

/* Local layout (cart_mpi.f90:105-136) + InitLattice + AllocateArrays
 * (zero-filled) + SetGeometry up to PassInt, for the box L at start. */
static int setup_box(orc_state* s, const int L[3], const int start[3]) {
  for (int d = 0; d < 3; ++d) {
    s->L[d] = d < s->dim ? L[d] : 1;
    s->start[d] = d < s->dim ? start[d] : 0;
  }
  for (int d = 0; d < s->dim; ++d)
    if (s->L[d] < G) return -3;
  s->dy = s->L[0] + 2 * G;
  s->dz = s->dim == 3 ? s->dy * (s->L[1] + 2 * G) : 0;
  s->array_size = (long long)(s->L[0] + 2 * G) * (s->L[1] + 2 * G);
  if (s->dim == 3) s->array_size *= (s->L[2] + 2 * G);

  init_lattice(s);

  long long n = s->array_size;
  s->f = (double*)calloc((size_t)(n * s->nq), sizeof(double));
  s->fb = (double*)calloc((size_t)(n * s->nq), sizeof(double));
  s->p = (double*)calloc((size_t)n, sizeof(double));
  s->u = (double*)calloc((size_t)(n * s->dim), sizeof(double));
  s->geo = (int*)calloc((size_t)n, sizeof(int));
  s->fluid_id = (int*)calloc((size_t)n, sizeof(int));
  s->b_user = (int*)calloc((size_t)n, sizeof(int));
  long long face = (long long)(s->L[0] + 2 * G) * (s->L[1] + 2 * G);
  long long facey = s->dim == 3 ? (long long)(s->L[1] + 2 * G) * (s->L[2] + 2 * G) : s->L[1] + 2 * G;
  long long facex = s->dim == 3 ? (long long)(s->L[0] + 2 * G) * (s->L[2] + 2 * G) : s->L[0] + 2 * G;
  long long facez = s->dim == 3 ? face : s->L[0] + 2 * G;
  s->bl = (int*)calloc((size_t)facey + 1, sizeof(int));
  s->br = (int*)calloc((size_t)facey + 1, sizeof(int));
  s->bu = (int*)calloc((size_t)facez + 1, sizeof(int));
  s->bd = (int*)calloc((size_t)facez + 1, sizeof(int));
  s->bf = (int*)calloc((size_t)facex + 1, sizeof(int));
  s->bb = (int*)calloc((size_t)facex + 1, sizeof(int));
  if (!s->f || !s->fb || !s->p || !s->u || !s->geo || !s->fluid_id || !s->b_user || !s->bl ||
      !s->br || !s->bu || !s->bd || !s->bf || !s->bb) {
    orc_free(s);
    return -4;
  }
  geometry_local(s);
  return 0;
}

int orc_setup(orc_state* s, const orc_input* in) {
  int rc = data_input(s, in);
  if (rc) return rc;
  /* SetLocalLength with one rank, cart_mpi.f90:63-64,105-111,133-136 */
  const int L[3] = {s->nx + 1, s->ny + 1, s->dim == 3 ? s->nz + 1 : 1};
  const int start[3] = {0, 0, 0};
  rc = setup_box(s, L, start);
  if (rc) return rc;
  wrap_int(s, s->geo); /* PassInt(geo), one periodic rank */
  obstacle_scan(s);
  return s->geom_error ? -2 : 0;
}

/* ------------------------------------------------------------------------ */
/* InitUP: initialization.f90:259-282, initialization_3d.f90:282-308         */
/* ------------------------------------------------------------------------ */
void orc_init_up(orc_state* s, const double* r_vec) {
  const double uu = s->uu;
  if (s->dim == 2) {
    const int ny = s->ny;
    for (int j = 0; j < s->L[1]; ++j)
      for (int i = 0; i < s->L[0]; ++i) {
        long long id = i + G + (long long)s->dy * (j + G);
        double r = 1.0 + (r_vec[id % 100] - 0.5) * 2.0 * 0.2;
        double y = (double)(j + s->start[1]);
        s->p[id] = 0.0;
        s->u[id * 2] = uu * 4.0 * y * (ny - y) / (double)(ny * ny) * (double)s->geo[id] * r;
        s->u[id * 2 + 1] = 0.0;
      }
  } else {
    const int nz = s->nz;
    for (int k = 0; k < s->L[2]; ++k)
      for (int j = 0; j < s->L[1]; ++j)
        for (int i = 0; i < s->L[0]; ++i) {
          long long id = i + G + (long long)s->dy * (j + G) + (long long)s->dz * (k + G);
          double r = 1.0 + (r_vec[id % 100] - 0.5) * 2.0 * 0.2;
          double z = (double)(k + s->start[2]);
          s->p[id] = 0.0;
          s->u[id * 3] = uu * 4.0 * z * (nz - z) / (double)(nz * nz) * r * (double)s->geo[id];
          s->u[id * 3 + 1] = 0.0;
          s->u[id * 3 + 2] = 0.0;
        }
  }
}

/* ------------------------------------------------------------------------ */
/* Equilibrium as written at lbm.f90:44 and lbm.f90:70                       */
/* ------------------------------------------------------------------------ */
static inline double feq_of(const orc_state* s, long long id, int iq, double udu) {
  const int dim = s->dim;
  double edu = 0.0;
  for (int ind = 0; ind < dim; ++ind) edu = edu + (double)s->e[iq * dim + ind] * s->u[id * dim + ind];
  return s->t[iq] * (s->p[id] * 3.0 + s->rho0 * (3.0 * edu + 4.5 * (edu * edu) - 1.5 * udu));
}

static inline double udu_of(const orc_state* s, long long id) {
  double udu = 0.0;
  for (int ind = 0; ind < s->dim; ++ind) udu = udu + s->u[id * s->dim + ind] * s->u[id * s->dim + ind];
  return udu;
}

#define NT(s) ((s)->nthreads > 0 ? (s)->nthreads : 0)

/* InitPDF, lbm.f90:24-48 */
void orc_init_pdf(orc_state* s) {
  const int nq = s->nq;
  const int nf = s->size_fluid;
#ifdef _OPENMP
  int nt = NT(s) ? NT(s) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int idn = 0; idn < nf; ++idn) {
    long long id = s->fluid_id[idn];
    double udu = udu_of(s, id);
    for (int iq = 0; iq < nq; ++iq) s->f[id * nq + iq] = feq_of(s, id, iq, udu);
  }
}

/* Collision, lbm.f90:52-76 */
void orc_collision(orc_state* s) {
  const int nq = s->nq;
  const int nf = s->size_fluid;
  const double ome = s->ome;
#ifdef _OPENMP
  int nt = NT(s) ? NT(s) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int idn = 0; idn < nf; ++idn) {
    long long id = s->fluid_id[idn];
    double udu = udu_of(s, id);
    for (int iq = 0; iq < nq; ++iq) {
      double feq = feq_of(s, id, iq, udu);
      s->fb[id * nq + iq] = (1.0 - ome) * s->f[id * nq + iq] + ome * feq;
    }
  }
}

/* Propagation, lbm.f90:80-92 */
void orc_propagation(orc_state* s) {
  const int nq = s->nq, dim = s->dim;
  const int nf = s->size_fluid;
#ifdef _OPENMP
  int nt = NT(s) ? NT(s) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int idn = 0; idn < nf; ++idn) {
    long long id = s->fluid_id[idn];
    for (int iq = 0; iq < nq; ++iq) {
      long long nb = id - s->e[iq * dim] - (long long)s->dy * s->e[iq * dim + 1];
      if (dim == 3) nb -= (long long)s->dz * s->e[iq * dim + 2];
      s->f[id * nq + iq] = s->fb[nb * nq + iq];
    }
  }
}

/* Bounds-checked read inside the BC copy program. */
static inline double bc_read(orc_state* s, const double* a, long long idx) {
  if (idx < 0 || idx >= s->array_size * s->nq) {
    s->oob_reads++;
    return NAN;
  }
  return a[idx];
}

static inline long long ofs(const orc_state* s, int iq, int mult) {
  const int dim = s->dim;
  long long o = (long long)mult * s->e[iq * dim] + (long long)mult * s->dy * s->e[iq * dim + 1];
  if (dim == 3) o += (long long)mult * s->dz * s->e[iq * dim + 2];
  return o;
}

/* The copy program of BoundaryCondition, lbm.f90:96-155 (lbm_3d.f90:96-157)
 * applied to array a, in the reference's serial order. */
void orc_apply_bc(orc_state* s, double* a) {
  orc_pass_f(s, a);
  orc_bc_copies(s, a);
}

/* BoundaryCondition after PassF: the wall, obstacle, inlet and outlet
 * copies of lbm.f90:105-153 on this rank's own array. */
void orc_bc_copies(orc_state* s, double* a) {
  const int nq = s->nq;
  /* Up wall, Down wall, User boundary: fb(id,iq) = fb(id+2e_iq, nq-1-iq) */
  const int* lists[3] = {s->bu, s->bd, s->b_user};
  const int sizes[3] = {s->u_size, s->d_size, s->user_size};
  for (int l = 0; l < 3; ++l)
    for (int idn = 0; idn < sizes[l]; ++idn) {
      long long id = lists[l][idn];
      for (int iq = 0; iq < nq; ++iq)
        a[id * nq + iq] = bc_read(s, a, (id + ofs(s, iq, 2)) * nq + nq - 1 - iq);
    }
  /* Inlet: fb(id,iq) = fb(id+1,iq) */
  for (int idn = 0; idn < s->l_size; ++idn) {
    long long id = s->bl[idn];
    for (int iq = 0; iq < nq; ++iq) a[id * nq + iq] = bc_read(s, a, (id + 1) * nq + iq);
  }
  /* Outlet: fb(id,iq) = fb(id+e_iq,iq) */
  for (int idn = 0; idn < s->r_size; ++idn) {
    long long id = s->br[idn];
    for (int iq = 0; iq < nq; ++iq) a[id * nq + iq] = bc_read(s, a, (id + ofs(s, iq, 1)) * nq + iq);
  }
}

void orc_boundary_condition(orc_state* s) { orc_apply_bc(s, s->fb); }

/* PostProcessing, lbm.f90:159-201 (lbm_3d.f90:161-203) */
void orc_post_processing(orc_state* s) {
  const int nq = s->nq, dim = s->dim;
  const int nf = s->size_fluid;
  const double rho0 = s->rho0;
#ifdef _OPENMP
  int nt = NT(s) ? NT(s) : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int idn = 0; idn < nf; ++idn) {
    long long id = s->fluid_id[idn];
    double p = 0.0;
    double u[3] = {0.0, 0.0, 0.0};
    for (int iq = 0; iq < nq; ++iq) {
      double fv = s->f[id * nq + iq];
      p = p + fv;
      for (int ind = 0; ind < dim; ++ind) u[ind] = u[ind] + fv * (double)s->e[iq * dim + ind];
    }
    for (int ind = 0; ind < dim; ++ind) s->u[id * dim + ind] = u[ind] / rho0 * (double)s->geo[id];
    s->p[id] = p / 3.0 * (double)s->geo[id];
  }
  /* Dirichlet inlet velocity on column x=0 (rows of bl, ghost rows included) */
  for (int idn = 0; idn < s->l_size; ++idn) {
    long long id = s->bl[idn] + 1;
    if (dim == 2) {
      int y = (int)(id / s->dy) - G + s->start[1];
      s->u[id * 2] = s->uu * rho0 * 4.0 * y * (double)(s->ny - y) / (double)(s->ny * s->ny);
      s->u[id * 2 + 1] = 0.0;
    } else {
      int z = (int)(id / s->dz) - G + s->start[2];
      s->u[id * 3] = s->uu * rho0 * 4.0 * z * (double)(s->nz - z) / (double)(s->nz * s->nz);
      s->u[id * 3 + 1] = 0.0;
    }
  }
  /* zero pressure on column x=nx */
  for (int idn = 0; idn < s->r_size; ++idn) s->p[s->br[idn] - 1] = 0.0;
}

/* Monitor, lbm.f90:205-227: skips fluid_id(0), uses only ux, uy. */
double orc_monitor(const orc_state* s) {
  const int dim = s->dim;
  double um = 0.0;
  for (int idn = 1; idn < s->size_fluid; ++idn) {
    long long id = s->fluid_id[idn];
    double v = sqrt(s->u[id * dim] * s->u[id * dim] + s->u[id * dim + 1] * s->u[id * dim + 1]);
    if (v > um) um = v;
  }
  return um;
}

/* main.f90:48-63 */
int orc_run(orc_state* s, int iter0, int nsteps, int interv, double* umax_log) {
  int m = 0;
  for (int iter = iter0; iter < iter0 + nsteps; ++iter) {
    if (interv > 0 && iter % interv == 0) {
      double um = orc_monitor(s);
      if (umax_log) umax_log[m] = um;
      m++;
    }
    orc_collision(s);
    orc_boundary_condition(s);
    orc_propagation(s);
    orc_post_processing(s);
  }
  return m;
}

/* double-double accumulation (Knuth's TwoSum on the high word) */
static inline void dd_add(double* hi, double* lo, double x) {
  double s = *hi + x;
  double bp = s - *hi;
  double e = (*hi - (s - bp)) + (x - bp);
  *hi = s;
  *lo += e;
}

int orc_forces(const orc_state* s, double* F) {
  const int nq = s->nq, dim = s->dim;
  double hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
  int links = 0;
  for (int idn = 0; idn < s->size_fluid; ++idn) {
    long long x = s->fluid_id[idn];
    for (int iq = 0; iq < nq; ++iq) {
      long long nb = x + ofs(s, iq, 1);
      int X = (int)(nb % s->dy), Y, Z;
      if (dim == 2) {
        Y = (int)(nb / s->dy);
        Z = G;
      } else {
        Z = (int)(nb / s->dz);
        Y = (int)((nb - (long long)Z * s->dz) / s->dy);
      }
      if (is_ghost(s, X, Y, Z) || s->geo[nb] != 0) continue;
      double v = s->fb[x * nq + iq] + s->fb[nb * nq + nq - 1 - iq];
      for (int k = 0; k < dim; ++k) {
        int c = s->e[iq * dim + k];
        if (c) dd_add(&hi[k], &lo[k], c > 0 ? v : -v);
      }
      links++;
    }
  }
  for (int k = 0; k < dim; ++k) F[k] = hi[k] + lo[k];
  return links;
}

double orc_mass(const orc_state* s) {
  const int nq = s->nq;
  double hi = 0, lo = 0;
  for (int idn = 0; idn < s->size_fluid; ++idn) {
    long long x = s->fluid_id[idn];
    for (int iq = 0; iq < nq; ++iq) dd_add(&hi, &lo, s->f[x * nq + iq]);
  }
  return hi + lo;
}

void orc_r_vec(unsigned long long seed, double* r_vec) {
  unsigned long long x = seed;
  for (int i = 0; i < 100; ++i) {
    x += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    r_vec[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
}

/* ------------------------------------------------------------------------ */
/* Multi-rank runs: cart_mpi.f90 / cart_mpi_3d.f90                           */
/* ------------------------------------------------------------------------ */

void orc_decompose(int dim, const int gl[3], int nprocs, int np[3]) {
  double max_e = 0.0;
  np[0] = np[1] = np[2] = 1;
  for (int i = 1; i <= nprocs; ++i) {
    if (nprocs % i != 0) continue;
    const int px = i;
    if (dim == 2) {
      const int py = nprocs / i;
      /* integer arithmetic as written, then 1.d0/(...) */
      const int den = 2 * (gl[1] * (px - 1) / py + gl[0] * (py - 1) / px);
      const double e = 1.0 / (double)den; /* +Inf for one rank, as in IEEE Fortran */
      if (e >= max_e) {
        max_e = e;
        np[0] = px;
        np[1] = py;
      }
    } else {
      const int pyz = nprocs / i;
      for (int j = 1; j <= pyz; ++j) {
        if (pyz % j != 0) continue;
        const int py = j, pz = pyz / j;
        if (gl[2] == 2 && pz > 1) continue;
        const int den = 2 * (gl[1] * (px - 1) * gl[2] / py / pz + gl[0] * (py - 1) * gl[2] / px / pz +
                             gl[0] * gl[1] * (pz - 1) / px / py);
        const double e = 1.0 / (double)den;
        if (e >= max_e) {
          max_e = e;
          np[0] = px;
          np[1] = py;
          np[2] = pz;
        }
      }
    }
  }
}

int orc_local_box(int dim, const int gl[3], const int np[3], const int cc[3], int L[3],
                  int start[3]) {
  for (int d = 0; d < 3; ++d) {
    L[d] = 1;
    start[d] = 0;
  }
  for (int d = 0; d < dim; ++d) {
    /* gl/np + (1 - sign(1, cc - mod(gl, np)))/2, start = sum of the
     * lengths before it along the same dimension */
    int st = 0;
    for (int c = 0; c < cc[d]; ++c) st += gl[d] / np[d] + (c < gl[d] % np[d] ? 1 : 0);
    L[d] = gl[d] / np[d] + (cc[d] < gl[d] % np[d] ? 1 : 0);
    start[d] = st;
    if (L[d] < G) return -3;
  }
  return 0;
}

static int group_rank_of(const orc_group* g, const int c[3]) {
  if (g->dim == 2) return c[0] * g->np[1] + c[1];
  return (c[0] * g->np[1] + c[1]) * g->np[2] + c[2];
}

/* Owner rank and its padded cell of the globally periodic position of rank
 * a's padded cell (X, Y, Z). */
static long long group_source(const orc_group* g, int a, int X, int Y, int Z, int* owner) {
  const orc_state* s = &g->r[a];
  int P[3] = {X, Y, Z}, oc[3] = {0, 0, 0}, loc[3] = {G, G, G};
  for (int d = 0; d < g->dim; ++d) {
    int gx = P[d] - G + s->start[d];
    gx = ((gx % g->gl[d]) + g->gl[d]) % g->gl[d];
    int c = 0, st = 0;
    for (;;) {
      int len = g->gl[d] / g->np[d] + (c < g->gl[d] % g->np[d] ? 1 : 0);
      if (gx < st + len) break;
      st += len;
      ++c;
    }
    oc[d] = c;
    loc[d] = gx - st + G;
  }
  *owner = group_rank_of(g, oc);
  const orc_state* o = &g->r[*owner];
  return loc[0] + (long long)o->dy * loc[1] + (g->dim == 3 ? (long long)o->dz * loc[2] : 0);
}

/* PassInt / PassF between ranks: the messages go from interior cells to
 * ghost cells, so their order does not matter. width = values per cell. */
static void group_exchange(orc_group* g, int is_geo) {
  for (int a = 0; a < g->nprocs; ++a) {
    orc_state* s = &g->r[a];
    const int PX = s->L[0] + 2 * G, PY = s->L[1] + 2 * G, PZ = g->dim == 3 ? s->L[2] + 2 * G : 1;
    for (int Z = 0; Z < PZ; ++Z)
      for (int Y = 0; Y < PY; ++Y)
        for (int X = 0; X < PX; ++X) {
          if (!is_ghost(s, X, Y, Z)) continue;
          int owner;
          const long long src = group_source(g, a, X, Y, Z, &owner);
          const long long dst = X + (long long)s->dy * Y + (long long)s->dz * Z;
          const orc_state* o = &g->r[owner];
          if (is_geo) s->geo[dst] = o->geo[src];
          else memcpy(s->fb + dst * s->nq, o->fb + src * s->nq, sizeof(double) * s->nq);
        }
  }
}

void orc_group_pass_f(orc_group* g) { group_exchange(g, 0); }

void orc_group_free(orc_group* g) {
  if (g->r)
    for (int a = 0; a < g->nprocs; ++a) orc_free(&g->r[a]);
  free(g->r);
  free(g->cc);
  memset(g, 0, sizeof *g);
}

int orc_setup_rank(orc_state* s, const orc_input* in, const int L[3], const int start[3]) {
  int rc = data_input(s, in);
  return rc ? rc : setup_box(s, L, start);
}

int orc_obstacle_scan(orc_state* s) {
  obstacle_scan(s);
  return s->geom_error ? -2 : 0;
}

int orc_group_setup(orc_group* g, const orc_input* in, int nprocs) {
  memset(g, 0, sizeof *g);
  if (nprocs < 1 || (in->dim != 2 && in->dim != 3)) return -1;
  g->dim = in->dim;
  g->nprocs = nprocs;
  g->gl[0] = in->nx + 1;
  g->gl[1] = in->ny + 1;
  g->gl[2] = in->dim == 3 ? in->nz + 1 : 1;
  orc_decompose(g->dim, g->gl, nprocs, g->np);
  g->r = (orc_state*)calloc((size_t)nprocs, sizeof(orc_state));
  g->cc = (int(*)[3])calloc((size_t)nprocs, sizeof(int[3]));
  if (!g->r || !g->cc) {
    orc_group_free(g);
    return -4;
  }
  int rc = 0;
  for (int a = 0; a < nprocs; ++a) {
    int* c = g->cc[a];
    if (g->dim == 2) {
      c[0] = a / g->np[1];
      c[1] = a % g->np[1];
      c[2] = 0;
    } else {
      c[0] = a / (g->np[1] * g->np[2]);
      c[1] = (a / g->np[2]) % g->np[1];
      c[2] = a % g->np[2];
    }
    int L[3], start[3];
    rc = orc_local_box(g->dim, g->gl, g->np, c, L, start);
    if (!rc) rc = data_input(&g->r[a], in);
    if (!rc) rc = setup_box(&g->r[a], L, start);
    if (rc) {
      orc_group_free(g);
      return rc;
    }
  }
  group_exchange(g, 1); /* PassInt(geo) */
  int geom = 0;
  for (int a = 0; a < nprocs; ++a) {
    obstacle_scan(&g->r[a]);
    geom |= g->r[a].geom_error;
  }
  return geom ? -2 : 0;
}

void orc_group_init_up(orc_group* g, const double* r_vecs) {
  for (int a = 0; a < g->nprocs; ++a) orc_init_up(&g->r[a], r_vecs + 100 * a);
}

void orc_group_init_pdf(orc_group* g) {
  for (int a = 0; a < g->nprocs; ++a) orc_init_pdf(&g->r[a]);
}

/* MPI_REDUCE(MPI_MAX) of the ranks' Monitor values (lbm.f90:209-220). */
double orc_group_monitor(const orc_group* g) {
  double um = 0.0;
  for (int a = 0; a < g->nprocs; ++a) {
    const double v = orc_monitor(&g->r[a]);
    if (v > um) um = v;
  }
  return um;
}

int orc_group_run(orc_group* g, int iter0, int nsteps, int interv, double* umax_log) {
  int m = 0;
  for (int iter = iter0; iter < iter0 + nsteps; ++iter) {
    if (interv > 0 && iter % interv == 0) {
      const double um = orc_group_monitor(g);
      if (umax_log) umax_log[m] = um;
      m++;
    }
    for (int a = 0; a < g->nprocs; ++a) orc_collision(&g->r[a]);
    orc_group_pass_f(g);
    for (int a = 0; a < g->nprocs; ++a) orc_bc_copies(&g->r[a], g->r[a].fb);
    for (int a = 0; a < g->nprocs; ++a) {
      orc_propagation(&g->r[a]);
      orc_post_processing(&g->r[a]);
    }
  }
  return m;
}
