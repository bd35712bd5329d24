// Host-only verification hooks (include/imexlb_testing.h).
#include "imexlb_testing.h"

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bcmap.h"
#include "lattice.h"

extern "C" long long imexlb_testing_resolve_bc(const imexlb_desc* d, const int* fluid_id,
                                               int size_fluid, const int* bl, int l_size,
                                               const int* br, int r_size, const int* bu,
                                               int u_size, const int* bd, int d_size,
                                               const int* b_user, int user_size,
                                               const double* in, double* out) {
  if (!d || !in || !out || (d->dim != 2 && d->dim != 3)) return IMEXLB_ERR_ARG;
  imx::GridLayout g;
  g.dim = d->dim;
  g.Q = d->nq;
  for (int k = 0; k < 3; ++k) g.L[k] = k < d->dim ? d->local_length[k] : 1;
  g.dy = d->dy;
  g.dz = d->dim == 3 ? d->dz : 0;
  g.N = (int64_t)d->dy * (g.L[1] + 2 * imx::kGhost);
  if (d->dim == 3) g.N *= (g.L[2] + 2 * imx::kGhost);
  std::memcpy(g.e, d->e, sizeof(int) * d->nq * d->dim);
  std::vector<uint8_t> mask((size_t)g.N, 0);
  for (int i = 0; i < size_fluid; ++i) {
    if (fluid_id[i] < 0 || fluid_id[i] >= g.N) return IMEXLB_ERR_GEOMETRY;
    mask[(size_t)fluid_id[i]] = 1;
  }
  imx::BoundaryLists b;
  b.fluid_mask = mask.data();
  b.bl = bl; b.nl = l_size;
  b.br = br; b.nr = r_size;
  b.bu = bu; b.nu = u_size;
  b.bd = bd; b.nd = d_size;
  b.user = b_user; b.nuser = user_size;
  imx::BoundaryMap m;
  std::string err;
  const bool ok = m.build(g, b, err);
  // Resolution of every slot is defined even when a pulled slot is poisoned.
  const int64_t NQ = g.N * g.Q;
  for (int64_t s = 0; s < NQ; ++s) {
    const int64_t r = m.resolve(s);
    out[s] = r == imx::kPoison ? std::nan("") : in[r];
  }
  return ok ? (long long)m.fill().size() : IMEXLB_ERR_GEOMETRY;
}
