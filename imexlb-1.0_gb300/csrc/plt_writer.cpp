// WriteBinary for one rank: the reference's Tecplot binary (#!TDV112) file
// (lbm.f90:231-413, lbm_3d.f90:233-449), written from host arrays in the
// reference layout. Same records in the same order: magic, header integers
// (title and variable names as one integer per character), format 299.0,
// zone record, solution time iter/t_intv, ordered-zone sizes, 357.0 299.0,
// variable formats (all double), the min/max of every variable, then one
// block of (nx+1)(ny+1)[(nz+1)] doubles per variable in x-fastest order.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "imexlb_host.h"

namespace {

void put_chars(std::vector<int>& v, const char* s, int n) {
  for (int i = 0; i < n; ++i) v.push_back((unsigned char)s[i]);
}

}  // namespace

extern "C" int imexlb_host_write_plt(const imexlb_config* c, const char* path, int count, int iter,
                                     const double* p, const double* u, const int* fluid_id,
                                     int size_fluid) {
  if (!c || !path || !p || !u || (size_fluid > 0 && !fluid_id) || count < 0 || count > 999)
    return IMEXLB_ERR_ARG;
  const int dim = c->dim;
  const int numvars = dim == 2 ? 5 : 7;
  const double L = c->charlength, ti = c->t_intv;
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return IMEXLB_ERR_ARG;
  auto wi = [&](const std::vector<int>& v) { std::fwrite(v.data(), sizeof(int), v.size(), fp); };
  auto wf = [&](float x) { std::fwrite(&x, sizeof x, 1, fp); };
  auto wd = [&](const std::vector<double>& v) { std::fwrite(v.data(), sizeof(double), v.size(), fp); };

  std::fwrite("#!TDV112", 1, 8, fp);
  std::vector<int> h = {1, 0};
  if (dim == 2) put_chars(h, "Cylinder", 8);
  else put_chars(h, "Sphere", 6);
  h.push_back(0);
  h.push_back(numvars);
  const char* names2[] = {"x", "y", "p", "ux", "uy"};
  const char* names3[] = {"x", "y", "z", "p", "ux", "uy", "uz"};
  for (int k = 0; k < numvars; ++k) {
    const char* nm = dim == 2 ? names2[k] : names3[k];
    put_chars(h, nm, (int)std::strlen(nm));
    h.push_back(0);
  }
  wi(h);
  wf(299.0f);
  char num[8];
  std::snprintf(num, sizeof num, "%03d", count);
  std::string zone = std::string("ZONE ") + num;
  std::vector<int> z;
  put_chars(z, zone.c_str(), 8);
  z.insert(z.end(), {0, -1, 0});
  wi(z);
  wd({iter / ti});
  wi({-1, 0, 0, 0, 0, c->nx + 1, c->ny + 1, dim == 2 ? 1 : c->nz + 1, 0});
  wf(357.0f);
  wf(299.0f);
  std::vector<int> fmt((size_t)numvars, 2);
  fmt.insert(fmt.end(), {0, 0, -1});
  wi(fmt);

  // min/max over fluid_id(1:size_fluid-1), starting from 0 (lbm.f90:306-323)
  double umax[3] = {0, 0, 0}, umin[3] = {0, 0, 0}, pmax = 0, pmin = 0;
  for (int idn = 1; idn < size_fluid; ++idn) {
    const long long id = fluid_id[idn];
    for (int k = 0; k < dim; ++k) {
      const double v = u[id * dim + k];
      if (v > umax[k]) umax[k] = v;
      if (v < umin[k]) umin[k] = v;
    }
    if (p[id] > pmax) pmax = p[id];
    if (p[id] < pmin) pmin = p[id];
  }
  std::vector<double> lim = {0.0, c->nx / L, 0.0, c->ny / L};
  if (dim == 3) lim.insert(lim.end(), {0.0, c->nz / L});
  lim.push_back(pmin * L / (ti * ti));
  lim.push_back(pmax * L / (ti * ti));
  for (int k = 0; k < dim; ++k) {
    lim.push_back(umin[k] / (L * ti));
    lim.push_back(umax[k] / (L * ti));
  }
  wd(lim);

  const int L0 = c->local_length[0], L1 = c->local_length[1], L2 = dim == 3 ? c->local_length[2] : 1;
  const size_t n = (size_t)L0 * L1 * L2;
  std::vector<double> buf(n);
  auto block = [&](auto fn) {
    size_t q = 0;
    for (int k = 0; k < L2; ++k)
      for (int j = 0; j < L1; ++j)
        for (int i = 0; i < L0; ++i) buf[q++] = fn(i, j, k);
    wd(buf);
  };
  auto idx = [&](int i, int j, int k) {
    long long id = (i + 3) + (long long)c->dy * (j + 3);
    if (dim == 3) id += (long long)c->dz * (k + 3);
    return id;
  };
  block([&](int i, int, int) { return (c->local_start[0] + i) / L; });
  block([&](int, int j, int) { return (c->local_start[1] + j) / L; });
  if (dim == 3) block([&](int, int, int k) { return (c->local_start[2] + k) / L; });
  block([&](int i, int j, int k) { return p[idx(i, j, k)] * L / (ti * ti); });
  for (int d = 0; d < dim; ++d)
    block([&](int i, int j, int k) { return u[idx(i, j, k) * dim + d] / (L * ti); });
  const bool ok = std::ferror(fp) == 0;
  std::fclose(fp);
  return ok ? IMEXLB_OK : IMEXLB_ERR_ARG;
}
