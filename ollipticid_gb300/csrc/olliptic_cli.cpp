// olliptic_cli.cpp -- Olliptic_gpu.x, the reference's Olliptic.x command line
// on the GB300 solver.
//
// The reference reads its parameters from argv only (interface::read_console,
// src/interface.cc:366-800; a pars/ file is a shell line running Olliptic.x
// with flags), so a pars/ file runs unchanged with Olliptic.x replaced by this
// program.  Flags of the puncture FAS path are read with the reference's names
// and defaults; flags outside it (output, printing, symmetry, MPI) are accepted
// and ignored, as the reference ignores unknown flags.  Equations other than
// Punctures / Punctures_scalar_field are refused.
//
// Extra flags of this program (no reference counterpart):
//   -gpu-mixed yes|no   mixed-precision cycles (FP32 correction around FP64)
//   -gpu-device N       CUDA device (default: the current one)
//   -plan yes           print the box hierarchy (no GPU needed) and exit
//
// Output: the hierarchy, one line per V-cycle with its norm, and the ADM
// masses in the reference's "ADM mass[i] = ..." form (src/elliptic.cc:2466-
// 2469).  Exit status 0 on success; otherwise the C ABI's status with its
// message on stderr.
#include "olgpu.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct Args {
  std::map<std::string, std::string> kv;   // first value of each flag

  Args(int argc, char **argv)
  {
    for (int i = 1; i + 1 < argc; i++)
      if (argv[i][0] == '-' && !kv.count(argv[i])) kv[argv[i]] = argv[i + 1];
  }
  const char *find(std::initializer_list<const char *> names) const
  {
    for (const char *n : names) {
      auto it = kv.find(n);
      if (it != kv.end()) return it->second.c_str();
    }
    return nullptr;
  }
  double num(std::initializer_list<const char *> names, double def) const
  {
    const char *v = find(names);
    return v ? std::strtod(v, nullptr) : def;
  }
  int integer(std::initializer_list<const char *> names, int def) const
  {
    const char *v = find(names);
    return v ? (int)std::strtol(v, nullptr, 10) : def;
  }
  bool yes(std::initializer_list<const char *> names) const
  {
    const char *v = find(names);
    return v && (!std::strcmp(v, "yes") || !std::strcmp(v, "YES") || !std::strcmp(v, "true"));
  }
};

int fail(olgpu_status st, const char *what)
{
  std::fprintf(stderr, "Olliptic_gpu.x: %s: %s (status %d)\n", what, olgpu_last_error(), (int)st);
  return (int)st;
}

}  // namespace

int main(int argc, char **argv)
{
  for (int i = 1; i < argc; i++)
    if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) {
      std::printf("Olliptic_gpu.x: the Olliptic.x command line on the GB300 puncture FAS solver\n"
                  "  -eq Punctures|Punctures_scalar_field -NumBH n -bhmp<i> -bhx<i> -bhy<i> -bhz<i>\n"
                  "  -bhpx<i> -bhpy<i> -bhpz<i> -bhsx<i> -bhsy<i> -bhsz<i> -N n -L length -O order\n"
                  "  -l levels -nu1 n -nu2 n -s tol [-psc -phi0 -r0 -sigma -a2]\n"
                  "  -gpu-mixed yes|no  -gpu-device N  -plan yes\n");
      return 0;
    }
  const Args A(argc, argv);
  olgpu_problem p;
  olgpu_problem_defaults(&p);
  const char *eq = A.find({"-eq", "--equation"});
  const std::string equation = eq ? eq : "Punctures";
  if (equation == "Punctures") p.equation = OLGPU_EQ_PUNCTURES;
  else if (equation == "Punctures_scalar_field") p.equation = OLGPU_EQ_PUNCTURES_SCALAR;
  else {
    std::fprintf(stderr, "Olliptic_gpu.x: equation %s is not on the puncture FAS path\n", equation.c_str());
    return (int)OLGPU_ERR_INVALID_ARG;
  }
  p.numbh = A.integer({"-NumBH", "--num-bh"}, 1);
  if (p.numbh < 1 || p.numbh > OLGPU_MAX_BH) {
    std::fprintf(stderr, "Olliptic_gpu.x: NumBH must be 1..%d\n", OLGPU_MAX_BH);
    return (int)OLGPU_ERR_INVALID_ARG;
  }
  for (int i = 0; i < p.numbh; i++) {
    auto flag = [&](const char *base) { return std::string(base) + std::to_string(i + 1); };
    auto get = [&](const char *base) {
      const std::string f = flag(base);
      auto it = A.kv.find(f);
      return it == A.kv.end() ? 0.0 : std::strtod(it->second.c_str(), nullptr);
    };
    p.mp[i] = get("-bhmp");
    p.x[i] = get("-bhx");
    p.y[i] = get("-bhy");
    p.z[i] = get("-bhz");
    p.px[i] = get("-bhpx");
    p.py[i] = get("-bhpy");
    p.pz[i] = get("-bhpz");
    p.sx[i] = get("-bhsx");
    p.sy[i] = get("-bhsy");
    p.sz[i] = get("-bhsz");
  }
  p.n = A.integer({"-N", "-n"}, 30);
  p.L = A.num({"-L", "--length"}, 2.0);
  p.order = A.integer({"-O", "--order"}, 4);
  p.levels = A.integer({"-l", "--levels"}, 1);
  p.nu1 = A.integer({"-nu1", "--pre-smooth"}, 3);
  p.nu2 = A.integer({"-nu2", "--post-smooth"}, 3);
  p.tol = A.num({"-s", "--tolerance"}, 1e-8);
  p.ps_case = A.integer({"-psc", "-ps_case"}, 1);
  p.ps_phi0 = A.num({"-phi0", "--phi0_sf"}, 0.025);
  p.ps_r0 = A.num({"-r0", "--radius_sf_r0"}, 120.0);
  p.ps_sigma = A.num({"-sigma", "--sigma_sf"}, 8.0);
  p.ps_a2 = A.num({"-a2", "--a2_sf"}, 1.0);

  // the hierarchy (host only)
  std::vector<olgpu_box_info> boxes(1024);
  int nb = 0, nl = 0, mg = 0;
  olgpu_status st = olgpu_plan_boxes(&p, boxes.data(), (int)boxes.size(), &nb, &nl, &mg);
  if (st != OLGPU_OK) return fail(st, "grid set-up");
  std::printf("Olliptic_gpu.x: %s, NumBH %d, order %d, N %d, L %g, %d levels (%d multigrid), %d boxes\n",
              equation.c_str(), p.numbh, p.order, p.n, p.L, nl, mg, nb);
  for (int g = 0; g < nb; g++)
    std::printf("  box %2d level %2d  %d x %d x %d  origin (%g, %g, %g)  dx %g\n", g, boxes[g].level, boxes[g].nx,
                boxes[g].ny, boxes[g].nz, boxes[g].xi, boxes[g].yi, boxes[g].zi, boxes[g].dx);
  if (A.yes({"-plan"})) return 0;

  olgpu_hierarchy *h = nullptr;
  st = olgpu_hierarchy_create(&p, A.integer({"-gpu-device"}, -1), &h);
  if (st != OLGPU_OK) return fail(st, "hierarchy");
  if (A.yes({"-gpu-mixed"})) {
    st = olgpu_set_precision(h, OLGPU_PREC_MIXED);
    if (st != OLGPU_OK) {
      olgpu_hierarchy_destroy(h);
      return fail(st, "mixed precision");
    }
  }
  olgpu_report rep;
  st = olgpu_solve(h, nullptr, &rep);   // the reference stop rule
  for (int c = 0; c < rep.cycles && c < 256; c++) std::printf("  V-cycle %3d  norm %.6e\n", c + 1, rep.res[c]);
  if (st != OLGPU_OK) {
    olgpu_hierarchy_destroy(h);
    return fail(st, "solve");
  }
  std::printf("Solved in %d V-cycles, norm %.6e, %.3f ms on the device\n", rep.cycles, rep.final_res,
              olgpu_last_device_ms(h));
  std::printf("Puncure method: \n");
  double adm[OLGPU_MAX_BH];
  olgpu_adm_mass(h, adm);
  for (int i = 0; i < p.numbh; i++) std::printf("ADM mass[%d] = %.17g\n", i, adm[i]);
  olgpu_hierarchy_destroy(h);
  return 0;
}
