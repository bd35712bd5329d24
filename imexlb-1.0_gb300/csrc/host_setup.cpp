// Host-side setup for C/C++ callers (include/imexlb_host.h): the parts of
// initialization.f90 / initialization_3d.f90 and cart_mpi.f90 a host needs
// before handing arrays to the step library. Built with -ffp-contract=off so
// derived values round exactly as the reference's serial build.
#include "imexlb_host.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "lattice.h"

namespace {

constexpr int G = imx::kGhost;

// Fortran list-directed input: each READ starts on a new record and takes
// values (separated by blanks or commas) from as many records as it needs.
class ListReader {
 public:
  explicit ListReader(std::istream& in) : in_(in) {}
  void next_statement() { toks_.clear(); pos_ = 0; }
  bool value(std::string& out) {
    while (pos_ >= toks_.size()) {
      std::string line;
      if (!std::getline(in_, line)) return false;
      toks_.clear();
      pos_ = 0;
      std::string cur;
      for (char ch : line) {
        if (std::isspace((unsigned char)ch) || ch == ',') {
          if (!cur.empty()) toks_.push_back(cur), cur.clear();
        } else {
          cur.push_back(ch);
        }
      }
      if (!cur.empty()) toks_.push_back(cur);
    }
    out = toks_[pos_++];
    return true;
  }
  bool integer(int& v) {
    std::string s;
    if (!value(s)) return false;
    char* end = nullptr;
    long x = std::strtol(s.c_str(), &end, 10);
    if (*end) return false;
    v = (int)x;
    return true;
  }
  bool real(double& v) {
    std::string s;
    if (!value(s)) return false;
    for (char& ch : s)
      if (ch == 'd' || ch == 'D' || ch == 'q' || ch == 'Q') ch = 'e';
    char* end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return *end == '\0';
  }

 private:
  std::istream& in_;
  std::vector<std::string> toks_;
  size_t pos_ = 0;
};

inline long long cell_id(const imexlb_config* c, int i, int j, int k) {
  // id for loop indices i,j,k in 0..L+2 (position x = i-1 etc.)
  long long id = (i - 1 + G) + (long long)c->dy * (j - 1 + G);
  if (c->dim == 3) id += (long long)c->dz * (k - 1 + G);
  return id;
}

int wrapc(int c, int L) { return c < G ? c + L : (c >= L + G ? c - L : c); }

}  // namespace

extern "C" {

int imexlb_host_derive(imexlb_config* c) {
  if (!c || (c->dim != 2 && c->dim != 3)) return IMEXLB_ERR_ARG;
  // initialization.f90:65-81
  c->charlength = c->charlength_in * c->nx;
  c->pos = c->xpos_in * c->nx;
  c->nu = (2.0 - c->ome) * c->dt / (6.0 * c->ome);
  c->t_intv = c->charlength * c->charlength / c->nu;
  c->interv = (int)(c->inter * c->t_intv);
  c->max_step = (int)(c->max_t * c->t_intv);
  c->uu = c->re * c->nu / c->charlength;
  c->tau = 3 * c->nu;
  c->ma = c->uu * std::sqrt(3.0);
  c->radius = c->charlength * 0.5;
  // cart_mpi.f90:63-64,105-136 with one rank
  const int n[3] = {c->nx, c->ny, c->dim == 3 ? c->nz : 0};
  for (int k = 0; k < 3; ++k) {
    c->local_start[k] = 0;
    c->local_length[k] = k < c->dim ? n[k] + 1 : 1;
    if (k < c->dim && c->local_length[k] < G) return IMEXLB_ERR_ARG;
  }
  c->dy = c->local_length[0] + 2 * G;
  c->dz = c->dim == 3 ? c->dy * (c->local_length[1] + 2 * G) : 0;
  c->array_size = (long long)c->dy * (c->local_length[1] + 2 * G);
  if (c->dim == 3) c->array_size *= (c->local_length[2] + 2 * G);
  return IMEXLB_OK;
}

int imexlb_host_read_input(const char* path, int dim, imexlb_config* c) {
  if (!path || !c || (dim != 2 && dim != 3)) return IMEXLB_ERR_ARG;
  std::memset(c, 0, sizeof *c);
  c->dim = dim;
  std::ifstream in(path);
  if (!in) return IMEXLB_ERR_ARG;
  ListReader r(in);
  bool ok = true;
  r.next_statement();
  ok = ok && r.integer(c->nx) && r.integer(c->ny) && (dim == 2 || r.integer(c->nz));
  r.next_statement();
  ok = ok && r.real(c->charlength_in) && r.real(c->xpos_in) && r.real(c->re);
  r.next_statement();
  ok = ok && r.real(c->ome) && r.real(c->dt) && r.real(c->rho0);
  r.next_statement();
  ok = ok && r.real(c->max_t) && r.real(c->inter);
  if (!ok) return IMEXLB_ERR_ARG;
  return imexlb_host_derive(c);
}

int imexlb_host_lattice(int dim, double* t, int* e) {
  if (!t || !e || (dim != 2 && dim != 3)) return IMEXLB_ERR_ARG;
  if (dim == 2) {
    for (int iq = 0; iq < 9; ++iq) {
      const int i = imx::Lattice<2>::ex(iq), j = imx::Lattice<2>::ey(iq);
      e[iq * 2] = i;
      e[iq * 2 + 1] = j;
      // 4*(1-0.75*i**2)*(1-0.75*j**2)/9.d0: single-precision product (exact), double divide
      const float w = 4.0f * (1.0f - 0.75f * (float)(i * i)) * (1.0f - 0.75f * (float)(j * j));
      t[iq] = (double)w / 9.0;
    }
  } else {
    for (int iq = 0; iq < 27; ++iq) {
      const int i = imx::Lattice<3>::ex(iq), j = imx::Lattice<3>::ey(iq), k = imx::Lattice<3>::ez(iq);
      e[iq * 3] = i;
      e[iq * 3 + 1] = j;
      e[iq * 3 + 2] = k;
      double p4 = 1.0;
      for (int m = 0; m < std::abs(i) + std::abs(j) + std::abs(k); ++m) p4 *= 4.0;
      t[iq] = 8.0 / p4 / 27.0;  // 8.d0/4.d0**(|i|+|j|+|k|)/27.d0
    }
  }
  return IMEXLB_OK;
}

int imexlb_host_list_capacity(const imexlb_config* c, long long caps[8]) {
  if (!c || !caps) return IMEXLB_ERR_ARG;
  const long long PX = c->local_length[0] + 2 * G, PY = c->local_length[1] + 2 * G;
  const long long PZ = c->dim == 3 ? c->local_length[2] + 2 * G : 1;
  caps[0] = c->array_size;                       // fluid_id
  caps[1] = caps[2] = c->dim == 3 ? PY * PZ + 1 : PY;  // bl, br
  caps[3] = caps[4] = c->dim == 3 ? PX * PY + 1 : PX;  // bu, bd
  caps[5] = caps[6] = c->dim == 3 ? PX * PZ + 1 : 0;   // bf, bb
  caps[7] = c->array_size;                       // b_user
  return IMEXLB_OK;
}

int imexlb_host_geometry_lists(const imexlb_config* c, int* geo, int* fluid_id, int* bl, int* br,
                               int* bu, int* bd, int* bf, int* bb, int sizes[7]) {
  if (!c || !geo || !fluid_id || !bl || !br || !bu || !bd || !sizes) return IMEXLB_ERR_ARG;
  if (c->dim == 3 && (!bf || !bb)) return IMEXLB_ERR_ARG;
  const int dim = c->dim;
  const int L0 = c->local_length[0], L1 = c->local_length[1], L2 = c->local_length[2];
  const int kmax = dim == 3 ? L2 + 2 : 0;
  int n[7] = {0, 0, 0, 0, 0, 0, 0};
  const double r2max = c->radius * c->radius;
  for (int k = 0; k <= kmax; ++k)
    for (int j = 0; j <= L1 + 2; ++j)
      for (int i = 0; i <= L0 + 2; ++i) {
        const int x = i - 1 + c->local_start[0], y = j - 1 + c->local_start[1];
        const int z = k - 1 + c->local_start[2];
        const long long id = cell_id(c, i, j, k);
        const bool inside = i >= 1 && i <= L0 && j >= 1 && j <= L1 && (dim == 2 || (k >= 1 && k <= L2));
        if (inside) {
          const double ax = (double)x - c->pos, ay = (double)y - (c->ny / 2.0 + c->yoff);
          double r2 = ax * ax + ay * ay;
          if (dim == 3) {
            const double az = (double)z - c->nz / 2.0;
            r2 = r2 + az * az;
          }
          geo[id] = r2 > r2max ? 1 : 0;
          if (geo[id]) fluid_id[n[0]++] = (int)id;
        } else {
          if (x == -1) bl[n[1]++] = (int)id;
          if (x == c->nx + 1) br[n[2]++] = (int)id;
          if (dim == 2) {
            if (y == c->ny + 1) bu[n[3]++] = (int)id;
            if (y == -1) bd[n[4]++] = (int)id;
          } else {
            if (y == -1) bf[n[5]++] = (int)id;
            if (y == c->ny + 1) bb[n[6]++] = (int)id;
            if (z == -1) bd[n[4]++] = (int)id;
            if (z == c->nz + 1) bu[n[3]++] = (int)id;
          }
        }
      }
  for (int m = 0; m < 7; ++m) sizes[m] = n[m];
  return IMEXLB_OK;
}

int imexlb_host_obstacle_scan(const imexlb_config* c, const int* geo, int* b_user, int* n_user) {
  if (!c || !geo || !b_user || !n_user) return IMEXLB_ERR_ARG;
  const int dim = c->dim, nq = dim == 2 ? 9 : 27;
  const int L0 = c->local_length[0], L1 = c->local_length[1], L2 = c->local_length[2];
  const int kmax = dim == 3 ? L2 + 2 : 0;
  double t[27];
  int e[81];
  imexlb_host_lattice(dim, t, e);
  bool probe_oob = false;
  int n = 0;
  for (int k = 0; k <= kmax; ++k)
    for (int j = 0; j <= L1 + 2; ++j)
      for (int i = 0; i <= L0 + 2; ++i) {
        const long long id = cell_id(c, i, j, k);
        if (geo[id] != 0) continue;
        bool hit = false;
        for (int iq = 0; iq < nq && !hit; ++iq) {
          long long pr = id + e[iq * dim] + (long long)c->dy * (iq * dim + 1);
          if (dim == 3) pr += (long long)c->dz * (iq * dim + 2);
          if (pr < 0 || pr >= c->array_size) {
            probe_oob = true;
            continue;
          }
          hit = geo[pr] == 1;
        }
        if (hit) {
          b_user[n++] = (int)id;
          break;  // next x-row
        }
      }
  *n_user = n;
  return probe_oob ? IMEXLB_ERR_GEOMETRY : IMEXLB_OK;
}

int imexlb_host_set_geometry(const imexlb_config* c, int* geo, int* fluid_id, int* bl, int* br,
                             int* bu, int* bd, int* bf, int* bb, int* b_user, int sizes[8]) {
  if (!b_user || !sizes) return IMEXLB_ERR_ARG;
  const int rc = imexlb_host_geometry_lists(c, geo, fluid_id, bl, br, bu, bd, bf, bb, sizes);
  if (rc != IMEXLB_OK) return rc;
  const int dim = c->dim;
  const int L0 = c->local_length[0], L1 = c->local_length[1], L2 = c->local_length[2];
  // PassInt(geo) with one periodic rank
  const int PX = L0 + 2 * G, PY = L1 + 2 * G, PZ = dim == 3 ? L2 + 2 * G : 1;
  for (int Z = 0; Z < PZ; ++Z)
    for (int Y = 0; Y < PY; ++Y)
      for (int X = 0; X < PX; ++X) {
        const bool ghost = X < G || X >= L0 + G || Y < G || Y >= L1 + G ||
                           (dim == 3 && (Z < G || Z >= L2 + G));
        if (!ghost) continue;
        const long long dst = X + (long long)c->dy * Y + (long long)c->dz * Z;
        const long long src = wrapc(X, L0) + (long long)c->dy * wrapc(Y, L1) +
                              (dim == 3 ? (long long)c->dz * wrapc(Z, L2) : 0);
        geo[dst] = geo[src];
      }
  // Obstacle cells: the first solid cell of each x-row whose probe
  // geo(id + e_x + dy*(iq*dim+1) [+ dz*(iq*dim+2)]) is fluid, probing iq in
  // order (initialization.f90:232-253, initialization_3d.f90:253-277).
  return imexlb_host_obstacle_scan(c, geo, b_user, &sizes[7]);
}

// SetCartesian (cart_mpi.f90:57-103, cart_mpi_3d.f90:57-103): integer
// arithmetic as written, 1.d0/(...) compared with .ge., so the last of equal
// candidates wins.
int imexlb_host_decompose(int dim, const int gl[3], int nprocs, int np[3]) {
  if ((dim != 2 && dim != 3) || !gl || !np || nprocs < 1) return IMEXLB_ERR_ARG;
  double max_e = 0.0;
  np[0] = np[1] = np[2] = 1;
  for (int i = 1; i <= nprocs; ++i) {
    if (nprocs % i != 0) continue;
    const int px = i;
    if (dim == 2) {
      const int py = nprocs / i;
      const int den = 2 * (gl[1] * (px - 1) / py + gl[0] * (py - 1) / px);
      const double e = den == 0 ? INFINITY : 1.0 / (double)den;
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
        const double e = den == 0 ? INFINITY : 1.0 / (double)den;
        if (e >= max_e) {
          max_e = e;
          np[0] = px;
          np[1] = py;
          np[2] = pz;
        }
      }
    }
  }
  return IMEXLB_OK;
}

// MPI_Cart_coords without reordering: row-major, the last dimension fastest.
static void rank_coords(int dim, const int np[3], int rank, int cc[3]) {
  cc[0] = cc[1] = cc[2] = 0;
  if (dim == 2) {
    cc[0] = rank / np[1];
    cc[1] = rank % np[1];
  } else {
    cc[0] = rank / (np[1] * np[2]);
    cc[1] = (rank / np[2]) % np[1];
    cc[2] = rank % np[2];
  }
}

int imexlb_host_rank_layout(imexlb_config* c, const int np[3], int rank) {
  if (!c || !np || (c->dim != 2 && c->dim != 3)) return IMEXLB_ERR_ARG;
  const int dim = c->dim;
  int nprocs = 1;
  for (int k = 0; k < dim; ++k) nprocs *= np[k];
  if (rank < 0 || rank >= nprocs) return IMEXLB_ERR_ARG;
  const int gl[3] = {c->nx + 1, c->ny + 1, dim == 3 ? c->nz + 1 : 1};
  int cc[3];
  rank_coords(dim, np, rank, cc);
  // SetLocalLength (cart_mpi.f90:105-136)
  for (int k = 0; k < 3; ++k) {
    c->local_length[k] = 1;
    c->local_start[k] = 0;
  }
  for (int k = 0; k < dim; ++k) {
    int st = 0;
    for (int q = 0; q < cc[k]; ++q) st += gl[k] / np[k] + (q < gl[k] % np[k] ? 1 : 0);
    c->local_start[k] = st;
    c->local_length[k] = gl[k] / np[k] + (cc[k] < gl[k] % np[k] ? 1 : 0);
    if (c->local_length[k] < G) return IMEXLB_ERR_ARG;
  }
  c->dy = c->local_length[0] + 2 * G;
  c->dz = dim == 3 ? c->dy * (c->local_length[1] + 2 * G) : 0;
  c->array_size = (long long)c->dy * (c->local_length[1] + 2 * G);
  if (dim == 3) c->array_size *= (c->local_length[2] + 2 * G);
  return IMEXLB_OK;
}

int imexlb_host_group_pass_int(const imexlb_config* c, const int np[3], int nprocs,
                               int* const* geo) {
  if (!c || !np || !geo || nprocs < 1) return IMEXLB_ERR_ARG;
  const int dim = c->dim;
  int count = 1;
  for (int k = 0; k < dim; ++k) count *= np[k];
  if (count != nprocs) return IMEXLB_ERR_ARG;
  std::vector<imexlb_config> r((size_t)nprocs, *c);
  for (int a = 0; a < nprocs; ++a) {
    if (!geo[a]) return IMEXLB_ERR_ARG;
    const int rc = imexlb_host_rank_layout(&r[(size_t)a], np, a);
    if (rc != IMEXLB_OK) return rc;
  }
  const int gl[3] = {c->nx + 1, c->ny + 1, dim == 3 ? c->nz + 1 : 1};
  // interior cells go to ghost cells, so the order of the copies does not matter
  for (int a = 0; a < nprocs; ++a) {
    const imexlb_config& s = r[(size_t)a];
    const int P[3] = {s.local_length[0] + 2 * G, s.local_length[1] + 2 * G,
                      dim == 3 ? s.local_length[2] + 2 * G : 1};
    for (int Z = 0; Z < P[2]; ++Z)
      for (int Y = 0; Y < P[1]; ++Y)
        for (int X = 0; X < P[0]; ++X) {
          const int pc[3] = {X, Y, Z};
          bool ghost = false;
          for (int k = 0; k < dim; ++k) ghost = ghost || pc[k] < G || pc[k] >= s.local_length[k] + G;
          if (!ghost) continue;
          int oc[3] = {0, 0, 0}, loc[3] = {G, G, G};
          for (int k = 0; k < dim; ++k) {
            int gx = pc[k] - G + s.local_start[k];
            gx = ((gx % gl[k]) + gl[k]) % gl[k];
            int q = 0, st = 0;
            for (;;) {
              const int len = gl[k] / np[k] + (q < gl[k] % np[k] ? 1 : 0);
              if (gx < st + len) break;
              st += len;
              ++q;
            }
            oc[k] = q;
            loc[k] = gx - st + G;
          }
          const int b = dim == 2 ? oc[0] * np[1] + oc[1] : (oc[0] * np[1] + oc[1]) * np[2] + oc[2];
          const imexlb_config& o = r[(size_t)b];
          const long long src = loc[0] + (long long)o.dy * loc[1] + (dim == 3 ? (long long)o.dz * loc[2] : 0);
          const long long dst = X + (long long)s.dy * Y + (long long)s.dz * Z;
          geo[a][dst] = geo[b][src];
        }
  }
  return IMEXLB_OK;
}

int imexlb_host_obstacle_cells(const imexlb_config* c, const int* geo, int* b_user, int* n_user) {
  if (!c || !geo || !b_user || !n_user || (c->dim != 2 && c->dim != 3)) return IMEXLB_ERR_ARG;
  const int dim = c->dim, nq = dim == 2 ? 9 : 27;
  double t[27];
  int e[81];
  imexlb_host_lattice(dim, t, e);
  long long off[27];
  for (int iq = 0; iq < nq; ++iq)
    off[iq] = e[iq * dim] + (long long)c->dy * e[iq * dim + 1] +
              (dim == 3 ? (long long)c->dz * e[iq * dim + 2] : 0);
  const int L0 = c->local_length[0], L1 = c->local_length[1];
  const int L2 = dim == 3 ? c->local_length[2] : 1;
  int n = 0;
  for (int k = 0; k < L2; ++k)
    for (int j = 0; j < L1; ++j)
      for (int i = 0; i < L0; ++i) {
        const long long id = (i + G) + (long long)c->dy * (j + G) +
                             (dim == 3 ? (long long)c->dz * (k + G) : 0);
        if (geo[id] != 0) continue;
        for (int iq = 0; iq < nq; ++iq)
          if (geo[id + off[iq]] == 1) {
            b_user[n++] = (int)id;
            break;
          }
      }
  *n_user = n;
  return IMEXLB_OK;
}

void imexlb_host_r_vec(unsigned long long seed, double* r_vec) {
  unsigned long long x = seed;
  for (int i = 0; i < 100; ++i) {
    x += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    r_vec[i] = (double)(z >> 11) * 0x1.0p-53;
  }
}

int imexlb_host_init_up(const imexlb_config* c, const int* geo, const double* r_vec, double* p,
                        double* u) {
  if (!c || !geo || !r_vec || !p || !u) return IMEXLB_ERR_ARG;
  const int dim = c->dim;
  const int L0 = c->local_length[0], L1 = c->local_length[1];
  const int L2 = dim == 3 ? c->local_length[2] : 1;
  for (int k = 0; k < L2; ++k)
    for (int j = 0; j < L1; ++j)
      for (int i = 0; i < L0; ++i) {
        long long id = i + G + (long long)c->dy * (j + G);
        if (dim == 3) id += (long long)c->dz * (k + G);
        const double r = 1.0 + (r_vec[id % 100] - 0.5) * 2.0 * 0.2;
        p[id] = 0.0;
        if (dim == 2) {
          const double y = (double)(j + c->local_start[1]);
          u[id * 2] = c->uu * 4.0 * y * (c->ny - y) / (double)(c->ny * c->ny) * (double)geo[id] * r;
          u[id * 2 + 1] = 0.0;
        } else {
          const double z = (double)(k + c->local_start[2]);
          u[id * 3] = c->uu * 4.0 * z * (c->nz - z) / (double)(c->nz * c->nz) * r * (double)geo[id];
          u[id * 3 + 1] = 0.0;
          u[id * 3 + 2] = 0.0;
        }
      }
  return IMEXLB_OK;
}

int imexlb_host_make_desc(const imexlb_config* c, int precision, int device, imexlb_desc* d) {
  if (!c || !d) return IMEXLB_ERR_ARG;
  std::memset(d, 0, sizeof *d);
  d->dim = c->dim;
  d->nq = c->dim == 2 ? 9 : 27;
  d->ghost = G;
  d->nx = c->nx;
  d->ny = c->ny;
  d->nz = c->dim == 3 ? c->nz : 0;
  for (int k = 0; k < 3; ++k) {
    d->local_length[k] = c->local_length[k];
    d->local_start[k] = c->local_start[k];
  }
  d->dy = c->dy;
  d->dz = c->dz;
  d->ome = c->ome;
  d->rho0 = c->rho0;
  d->uu = c->uu;
  imexlb_host_lattice(c->dim, d->t, d->e);
  d->precision = precision;
  d->device = device;
  return IMEXLB_OK;
}

}  // extern "C"
