// imexlb_run: single-rank driver with the structure of main.f90, on the GPU.
//
//   imexlb_run <input.in> [--dim 2|3] [--steps N] [--interv I] [--seed S] [--device D]
//              [--plt 0|1]
//
// DataInput -> MPISetup (one rank) -> InitLattice -> AllocateArrays ->
// SetGeometry -> device mapping -> InitUP -> InitPDF -> time loop
// (Monitor every interv iterations, then Collision, BoundaryCondition,
// Propagation, PostProcessing) -> elapsed time -> WriteBinary
// (output_<count>.plt, count = number of Monitor calls) (main.f90:14-73). The loop
// runs max_step+1 iterations as `do iter=0,max_step` does, unless --steps is
// given. Prints the same quantities as DataInput (initialization.f90:84-100)
// and Monitor (lbm.f90:222-226).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "imexlb.h"
#include "imexlb_host.h"

static int die(const char* what, int rc, imexlb_t* h) {
  std::fprintf(stderr, "imexlb_run: %s failed (%d): %s\n", what, rc, imexlb_last_error(h));
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <input.in> [--dim 2|3] [--steps N] [--interv I] [--seed S] [--device D]\n",
                 argv[0]);
    return 2;
  }
  const char* path = argv[1];
  int dim = 2, steps = -1, interv = -1, device = 0, plt = 1;
  unsigned long long seed = 12345ULL;
  for (int i = 2; i + 1 < argc; i += 2) {
    if (!std::strcmp(argv[i], "--dim")) dim = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "--steps")) steps = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "--interv")) interv = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "--seed")) seed = std::strtoull(argv[i + 1], nullptr, 10);
    else if (!std::strcmp(argv[i], "--device")) device = std::atoi(argv[i + 1]);
    else if (!std::strcmp(argv[i], "--plt")) plt = std::atoi(argv[i + 1]);
  }

  imexlb_config c;
  int rc = imexlb_host_read_input(path, dim, &c);
  if (rc) {
    std::fprintf(stderr, "imexlb_run: cannot read %s\n", path);
    return 1;
  }
  std::printf("%24s%6.2f\n", "Reynolds Number      :", c.re);
  std::printf("%24s%6.2f\n", "Characteristic Length:", c.charlength);
  std::printf("%24s%6.2f\n", "Ma                   :", c.ma);
  std::printf("%24s%6.2f\n", "Kinematic Viscosity  :", c.nu);
  std::printf("%24s%6.2f\n", "Relaxation Parameter :", c.ome);
  std::printf("%24s%6.2f\n", "Relaxation Time      :", c.tau);
  std::printf("%24s%4.1f\n", "Density              :", c.rho0);
  std::printf("%24s%8d\n", "Maximum # of Steps   :", c.max_step);
  std::printf("%24s%8d\n", "Interval Size        :", c.interv);
  std::printf(" =============================\n");

  const int nq = dim == 2 ? 9 : 27;
  const size_t N = (size_t)c.array_size;
  long long caps[8];
  imexlb_host_list_capacity(&c, caps);
  std::vector<int> geo(N), fluid_id((size_t)caps[0]), bl((size_t)caps[1]), br((size_t)caps[2]),
      bu((size_t)caps[3]), bd((size_t)caps[4]), bf((size_t)caps[5] + 1), bb((size_t)caps[6] + 1),
      b_user((size_t)caps[7]);
  int sizes[8];
  rc = imexlb_host_set_geometry(&c, geo.data(), fluid_id.data(), bl.data(), br.data(), bu.data(),
                                bd.data(), bf.data(), bb.data(), b_user.data(), sizes);
  if (rc) {
    std::fprintf(stderr, "imexlb_run: SetGeometry failed (%d)\n", rc);
    return 1;
  }
  std::vector<double> f(N * nq, 0.0), fb(N * nq, 0.0), p(N, 0.0), u(N * dim, 0.0), r_vec(100);
  imexlb_host_r_vec(seed, r_vec.data());
  imexlb_host_init_up(&c, geo.data(), r_vec.data(), p.data(), u.data());

  imexlb_desc d;
  imexlb_host_make_desc(&c, IMEXLB_FP64, device, &d);
  imexlb_t* h = nullptr;
  if ((rc = imexlb_create(&h, &d))) return die("imexlb_create", rc, nullptr);
  if ((rc = imexlb_set_geometry(h, geo.data(), fluid_id.data(), sizes[0], bl.data(), sizes[1],
                                br.data(), sizes[2], bu.data(), sizes[3], bd.data(), sizes[4],
                                b_user.data(), sizes[7])))
    return die("imexlb_set_geometry", rc, h);
  if ((rc = imexlb_upload(h, f.data(), fb.data(), p.data(), u.data()))) return die("imexlb_upload", rc, h);
  if ((rc = imexlb_init_pdf(h))) return die("imexlb_init_pdf", rc, h);

  const int nsteps = steps >= 0 ? steps : c.max_step + 1;
  const int iv = interv >= 0 ? interv : c.interv;
  // Monitor output is printed per interval; advance interval by interval.
  const int chunk = iv > 0 ? iv : nsteps;
  const auto t0 = std::chrono::steady_clock::now();
  int count = 0;
  for (int it = 0; it < nsteps; it += chunk) {
    const int n = std::min(chunk, nsteps - it);
    double um[1] = {0.0};
    if ((rc = imexlb_step(h, it, n, iv, um))) return die("imexlb_step", rc, h);
    if (iv > 0) {
      std::printf(" T= %.15g\n Umax= %.15g\n -------------------\n", it / c.t_intv,
                  um[0] / (c.charlength * c.t_intv));
      ++count;
    }
  }
  const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  imexlb_info info;
  imexlb_get_info(h, &info);
  std::printf(" Elapsed time:  %.6f\n", el);
  std::printf(" MLUPS: %.2f (nodes %lld, fluid %lld, steps %d)\n", (double)info.interior * nsteps / el / 1e6,
              info.interior, info.size_fluid, nsteps);
  if (plt) {
    if ((rc = imexlb_download(h, f.data(), fb.data(), p.data(), u.data())))
      return die("imexlb_download", rc, h);
    char name[32];
    std::snprintf(name, sizeof name, "output_%03d.plt", count);
    // the Fortran loop variable is max_step+1 after "do iter=0,max_step"
    if (imexlb_host_write_plt(&c, name, count, nsteps, p.data(), u.data(), fluid_id.data(),
                              sizes[0]))
      std::fprintf(stderr, "imexlb_run: cannot write %s\n", name);
  }
  imexlb_destroy(h);
  return 0;
}
