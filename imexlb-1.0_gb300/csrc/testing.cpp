// Host-only verification hooks (include/imexlb_testing.h).
#include "imexlb_testing.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bcmap.h"
#include "fused_plan.h"
#include "kernels.h"
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
  return ok ? (long long)m.fill().size() : (long long)IMEXLB_ERR_GEOMETRY;
}

extern "C" long long imexlb_testing_fused_pull(const imexlb_desc* d, const int* fluid_id,
                                               int size_fluid, const int* bl, int l_size,
                                               const int* br, int r_size, const int* bu,
                                               int u_size, const int* bd, int d_size,
                                               const int* b_user, int user_size,
                                               const double* cur, const double* prev,
                                               double* out_kernel, double* out_fused,
                                               long long* n_records) {
  if (!d || !cur || !prev || !out_kernel || !out_fused || (d->dim != 2 && d->dim != 3))
    return IMEXLB_ERR_ARG;
  imx::GridLayout g;
  g.dim = d->dim;
  g.Q = d->nq;
  for (int k = 0; k < 3; ++k) g.L[k] = k < d->dim ? d->local_length[k] : 1;
  g.dy = d->dy;
  g.dz = d->dim == 3 ? d->dz : 0;
  g.N = (int64_t)d->dy * (g.L[1] + 2 * imx::kGhost);
  if (d->dim == 3) g.N *= (g.L[2] + 2 * imx::kGhost);
  std::memcpy(g.e, d->e, sizeof(int) * d->nq * d->dim);
  const int Q = g.Q;
  const int64_t N = g.N, G = imx::kGhost;
  imx::DevGrid dg{};
  dg.N = N;
  dg.dy = g.dy;
  dg.dz = g.dz;
  dg.id_lo = G + g.dy * G + g.dz * G;
  dg.id_hi = (g.L[0] + G - 1) + g.dy * (g.L[1] + G - 1) + (d->dim == 3 ? g.dz * (g.L[2] + G - 1) : 0) + 1;
  for (int q = 0; q < Q; ++q) dg.off[q] = g.off(q, 1);
  // node mask as imexlb_set_geometry builds it
  std::vector<uint8_t> mask((size_t)N, 0);
  for (int i = 0; i < size_fluid; ++i) {
    if (fluid_id[i] < 0 || fluid_id[i] >= N || g.is_ghost(fluid_id[i])) return IMEXLB_ERR_GEOMETRY;
    mask[(size_t)fluid_id[i]] = imx::kMaskFluid;
  }
  for (int i = 0; i < l_size; ++i) {
    const int64_t id = (int64_t)bl[i] + 1;
    if (id >= 0 && id < N && (mask[(size_t)id] & imx::kMaskFluid)) mask[(size_t)id] |= imx::kMaskInlet;
  }
  for (int i = 0; i < r_size; ++i) {
    const int64_t id = (int64_t)br[i] - 1;
    if (id >= 0 && id < N && (mask[(size_t)id] & imx::kMaskFluid)) mask[(size_t)id] |= imx::kMaskOutlet;
  }
  std::vector<uint8_t> fluid01((size_t)N, 0);
  for (int64_t c = 0; c < N; ++c) fluid01[(size_t)c] = (mask[(size_t)c] & imx::kMaskFluid) ? 1 : 0;
  imx::BoundaryLists b;
  b.fluid_mask = fluid01.data();
  b.bl = bl; b.nl = l_size;
  b.br = br; b.nr = r_size;
  b.bu = bu; b.nu = u_size;
  b.bd = bd; b.nd = d_size;
  b.user = b_user; b.nuser = user_size;
  imx::BoundaryMap m;
  std::string err;
  if (!m.build(g, b, err)) return IMEXLB_ERR_GEOMETRY;
  std::vector<imx::DevFill> fill;
  for (const imx::FillEntry& fe : m.fill()) {
    const int64_t dsoa = (fe.dst % Q) * N + fe.dst / Q, ssoa = (fe.src % Q) * N + fe.src / Q;
    fill.push_back(imx::DevFill{dsoa, fe.src_prev ? ~ssoa : ssoa});
  }
  const size_t NQ = (size_t)N * Q;
  std::fill(out_kernel, out_kernel + NQ, 0.0);
  std::fill(out_fused, out_fused + NQ, 0.0);
  auto src_val = [&](const std::vector<double>& b2, int64_t s) { return s >= 0 ? b2[(size_t)s] : prev[(size_t)~s]; };
  // separate program: every copy, then the plain pull
  std::vector<double> B(cur, cur + NQ);
  const std::vector<double> C(cur, cur + NQ);
  for (const imx::DevFill& e : fill) B[(size_t)e.dst] = src_val(C, e.src);
  for (int64_t p = dg.id_lo; p < dg.id_hi; ++p)
    if (mask[(size_t)p] & imx::kMaskFluid)
      for (int q = 0; q < Q; ++q) out_kernel[(size_t)(q * N + p)] = B[(size_t)(q * N + p - dg.off[q])];
  imx::FusedPlan plan;
  if (N * Q >= (int64_t)INT32_MAX || !imx::plan_fused(g, dg, mask, m, fill, plan)) return 0;
  if (n_records) *n_records = (long long)plan.nodes.size();
  imx::apply_plan_bits(plan, mask);
  // fused: obstacle copies, then the pulls with closed forms or rows
  std::vector<double> F(cur, cur + NQ);
  std::vector<int64_t> rec_at((size_t)N, -1);
  for (size_t k = 0; k < plan.nodes.size(); ++k) {
    rec_at[(size_t)plan.nodes[k]] = (int64_t)k;
    const uint32_t w = plan.rec[k * (Q + 1) + Q];
    for (uint32_t j = 0; j < (w & 255u); ++j) {
      const imx::DevFill32& e = plan.ent[(w >> 8) + j];
      F[e.dst] = e.src >= 0 ? C[(size_t)e.src] : prev[(size_t)~(int64_t)e.src];
    }
  }
  for (int64_t p = dg.id_lo; p < dg.id_hi; ++p) {
    const uint8_t mk = mask[(size_t)p];
    if (!(mk & imx::kMaskFluid)) continue;
    for (int q = 0; q < Q; ++q) {
      int64_t a;
      if (mk & imx::kMaskRecord) {
        const uint32_t r = plan.rec[(size_t)rec_at[(size_t)p] * (Q + 1) + q];
        a = r != imx::kNoRedirect ? (int64_t)r : q * N + p - dg.off[q];
      } else {
        a = imx::fused_form(g, dg, plan.pshift, p, mk & ~imx::kMaskFluid, q);
      }
      out_fused[(size_t)(q * N + p)] = F[(size_t)a];
    }
  }
  return 1;
}
