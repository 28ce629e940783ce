// olliptic_cli.cpp -- Olliptic_gpu.x, the reference's Olliptic.x command line
// on the GB300 solver.
//
// The reference reads its parameters from argv only (interface::read_console,
// src/interface.cc:366-800; a pars/ file is a shell line running Olliptic.x
// with flags), so a pars/ file runs unchanged with Olliptic.x replaced by this
// program.  Flags of the puncture FAS path are read with the reference's names
// and defaults; flags outside it (output, printing, symmetry, MPI) are accepted
// and ignored, as the reference ignores unknown flags.  Equations other than
// Punctures / Punctures_scalar_field, the reference's test equations Poisson
// (the Gaussian test), Boundary-test and Multibox-test, and Bowen-York (its
// variables V1, V2, V3, lambda printed each as the reference prints u) are
// refused, and so are boundary conditions other than Robin and Dirichlet (the
// reference's default).
//
// Methods (-m): Vcycle (the default, and, as in the reference, what a name it
// does not know means), Wcycle (every level repeated until its own norm
// meets the tolerance, elliptic::Wcycle; FP64) and AppPuncture (the analytic
// approximation alone, elliptic::ApproximateID); Gauss-Seidel and
// Full-Multigrid are refused.
//
// Extra flags of this program (no reference counterpart):
//   -gpu-mixed yes|no   mixed-precision cycles (FP32 correction around FP64)
//   -gpu-guess approx   start the V-cycles from the analytic approximation
//                       (the same fixed point, fewer cycles) instead of u = 0
//   -gpu-device N       CUDA device (default: the current one)
//   -plan yes           print the box hierarchy (no GPU needed) and exit
//
// Output: the hierarchy, one line per top-level cycle with its norm, and the ADM
// masses in the reference's "ADM mass[i] = ..." form (src/elliptic.cc:2466-
// 2469) on stdout; in the output directory (-o, default Output) the files of
// elliptic::Print_Solution (src/output.cc:624-700) for the puncture path:
// the per-box cuts u-l<l>b<i>-0.{x,y,z} (-p1d, ffunction::Print_1D,
// src/ffunction.cc:819-960) and the interpolated cuts u.X, u.Y, u.Z and the
// plane u.XY (-pint, multigrid::Print_Interpol_1D / _2D, src/multigrid.cc:
// 151-880), with the reference's number formats, the cycle number and norm
// of every pre-smoothing step as Loo.gp (-so yes, elliptic::Print_Pre_Cycle,
// src/output.cc:1355-1460), the banner and the per-cycle norms as
// stdout0.out (Print_Info, Print_Pre_Cycle / Print_Post_Cycle) and the
// command line as <dir>.run.  The directory is rotated like the reference's
// (interface.cc:1470-1538): an existing <dir> becomes <dir>_prev, replacing
// an older <dir>_prev.  -p2d yes adds the per-box planes u-l<l>b<i>-0.{yz,xz,xy}
// (ffunction::Print_2D) and -p3d yes the dumps u-l<l>b<i>-0.xyz of every point
// in the reference's storage order (ffunction::Print_3D).
// Exit status 0 on success; otherwise the C ABI's status with its message on
// stderr.
#include "olgpu.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <map>
#include <string>
#include <system_error>
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
  // a logic parameter with the reference's default when absent
  bool logic(std::initializer_list<const char *> names, bool def) const
  {
    return find(names) ? yes(names) : def;
  }
};

// The geometry of one box as the output needs it (domain::Get_x, is_in).
struct BoxGeom {
  olgpu_box_info b;
  double lo(int a) const { return a == 0 ? b.xi : a == 1 ? b.yi : b.zi; }
  double hi(int a) const { return a == 0 ? b.xf : a == 1 ? b.yf : b.zf; }
  double d(int a) const { return a == 0 ? b.dx : a == 1 ? b.dy : b.dz; }
  int n(int a) const { return a == 0 ? b.nx : a == 1 ? b.ny : b.nz; }
  double coord(int a, int i) const { return lo(a) + (double)i * d(a); }
  bool is_in_axis(int a, double x) const { return lo(a) - d(a) * 0.1 <= x && x <= hi(a) + d(a) * 0.1; }
  // domain::Get_i: the first node at or after x
  int locate(int a, double x) const
  {
    const int np = n(a);
    int lo_i = 0, hi_i = np, i;
    if (lo(a) - x < 0.0 && x - hi(a) < 0.0) {
      i = np % 2 == 0 ? np / 2 : (np - 1) / 2;
      do {
        const double xi = coord(a, i);
        if (xi > x || std::fabs(xi - x) <= 3 * 2.220446049250313080847e-16)
          hi_i = i;
        else
          lo_i = i;
        i = (hi_i + lo_i) / 2;
      } while (lo_i + 1 < hi_i);
    } else {
      i = (lo(a) >= x) ? 0 : np - 2;
    }
    return i + 1;
  }
};

// interface.cc:1470-1538: <dir>_prev is removed, <dir> moved to it, <dir>
// made afresh, and the command line written to <dir>/<dir>.run.
bool prepare_output_dir(const std::string &name, int argc, char **argv)
{
  namespace fs = std::filesystem;
  std::error_code ec;
  const fs::path dir(name), prev(name + "_prev");
  if (fs::exists(dir, ec)) {
    fs::remove_all(prev, ec);
    fs::rename(dir, prev, ec);
  }
  fs::create_directories(dir, ec);
  if (!fs::is_directory(dir, ec)) return false;
  const std::string run = name + "/" + fs::path(name).filename().string() + ".run";
  FILE *f = std::fopen(run.c_str(), "w");
  if (!f) return false;
  for (int i = 0; i < argc; i++) std::fprintf(f, "%s%s", i ? " " : "", argv[i]);
  std::fprintf(f, "\n");
  std::fclose(f);
  fs::permissions(run, fs::perms::owner_exec | fs::perms::group_exec | fs::perms::others_exec,
                  fs::perm_options::add, ec);
  return true;
}

// elliptic::Print_Info (src/output.cc:1030-1345) into <dir>stdout0.out: the
// run's parameters and every box (ffunction::Print_Info with the domain's
// stream form, src/domain.cc:1759-1790), then "Init Multigrid iteration".
// `levels` and `mg` are the hierarchy's; the analytic method's hierarchy has
// no multigrid grids, so its listing starts at the base.
void write_banner(FILE *f, const olgpu_problem &p, const char *equation_str, const char *method_str,
                  const char *boundary_str, const std::string &dir, const std::vector<olgpu_box_info> &boxes, int nb,
                  int nl, int mg, bool skip_mg)
{
  const double eps_coarse = 2 * 2.220446049250313080847e-16;
  const double eps_solv = p.tol < eps_coarse ? eps_coarse : p.tol;
  static const char *orders[5] = {"", "2nd", "4th", "6th", "8th"};
  std::fprintf(f, " ---------------------------- Olliptic -----------------------------\n");
  std::fprintf(f, "Equation\t:\t%s\nMethod\t\t:\t%s\n", equation_str, method_str);
  std::fprintf(f, "Tolerance \n Fine grid\t:\t%g\n Coarse grid\t:\t%g\n", eps_solv, eps_coarse);
  std::fprintf(f, "Smooth sweeps \n Pre\t\t:\t%d\n Post\t\t:\t%d\n", p.nu1, p.nu2);
  std::fprintf(f, "Levels\t\t:\t%d\nBoxes\t\t:\t%d\nOrder\t\t:\t%s\n\n", nl - mg, p.numbh,
               p.order >= 2 && p.order <= 8 ? orders[p.order / 2] : "");
  std::fprintf(f, "Boundary\t:\t%s\nSymmetry\t:\tFull domain\n\nOutput to\t:\t%s*\n", boundary_str, dir.c_str());
  std::vector<int> in_level(nl, 0);
  for (int l = skip_mg ? mg : 0; l < nl; l++)
    for (int g = 0; g < nb; g++) {
      if (boxes[g].level != l) continue;
      const olgpu_box_info &b = boxes[g];
      std::fprintf(f, "\n  __________________________________________________________________\n");
      std::fprintf(f, "  level: %d | box: %d | Interpolation: %d\n", l - (skip_mg ? mg : 0), in_level[l]++, b.order);
      std::fprintf(f, "  ------------------------------------------------------------------\n");
      std::fprintf(f, "  nx = %d, \t\tny = %d, \t\tnz = %d\n", b.nx, b.ny, b.nz);
      std::fprintf(f, "  dx = %.3e, \tdy = %.3e, \tdz = %.3e\n", b.dx, b.dy, b.dz);
      std::fprintf(f, "  lx = %.2f, \t\tly = %.2f, \t\tlz = %.2f\n", b.xf - b.xi, b.yf - b.yi, b.zf - b.zi);
      std::fprintf(f, "  x-->[%.2f,%.2f]\ty-->[%.2f,%.2f]\tz-->[%.2f,%.2f]\n", b.xi, b.xf, b.yi, b.yf, b.zi, b.zf);
    }
  std::fprintf(f, "--------------------------------------------------------------------\n  Init Multigrid iteration\n");
}

// The cycle tables of <dir>stdout0.out (elliptic::Print_Pre_Cycle /
// Print_Post_Cycle, src/output.cc:1355-1605), one indented "|Loo[k] : norm"
// line per call of the solve: a cycle header and a rule before the top
// level's pre-smoothing line, a rule and the norm against the tolerance
// after its post-smoothing line.
void write_cycle_tables(FILE *f, const std::vector<olgpu_cycle_event> &ev, int nl, double eps_solv)
{
  const int top = nl - 1;
  auto rule = [&]() {
    for (int j = 0; j <= top; j++) std::fprintf(f, "========================");
    std::fprintf(f, "\n");
  };
  for (const olgpu_cycle_event &e : ev) {
    if (!e.post && e.level == top) {
      std::fprintf(f, "\n\nCycle: %lld\n", e.cycle);
      rule();
    }
    for (int j = 0; j < e.level; j++) std::fprintf(f, "|\t\t\t");
    std::fprintf(f, "|Loo[%d] : %.8e", e.level, e.norm);
    for (int j = e.level + 1; j <= top + 1; j++) std::fprintf(f, "|\t\t\t");
    std::fprintf(f, "\n");
    if (e.post && e.level == top) {
      rule();
      std::fprintf(f, "%.8e  -->  %.8e\n", e.norm, eps_solv);
    }
  }
}

// ffunction::Print_1D of one box and one axis: at every node along `axis`
// (ghosts included) through the other coordinates 0 when the box holds them,
// else through its middle node; the value is interpolated (Lagrange, order+1)
// when `interpolate`, else the node value.  "%.12e\t%.12e\t" lines, then a
// blank line.
olgpu_status print_box_cut(olgpu_hierarchy *h, const char *var, const BoxGeom &B, int g, int axis, bool interpolate,
                           int ord, const std::string &file)
{
  int node[3];
  double at[3];
  for (int a = 0; a < 3; a++) {
    const int m = B.n(a) % 2 == 0 ? B.n(a) / 2 : (B.n(a) - 1) / 2;
    node[a] = m;
    at[a] = B.coord(a, m);
    if (a == axis) continue;
    if (B.is_in_axis(a, 0.0)) {
      if (interpolate)
        at[a] = 0.0;
      else {
        node[a] = B.locate(a, 0.0);
        at[a] = B.coord(a, node[a]);
      }
    }
  }
  const int np = B.n(axis);
  std::vector<double> pts(3 * (size_t)np), val(np);
  for (int i = 0; i < np; i++) {
    for (int a = 0; a < 3; a++) pts[3 * i + a] = at[a];
    pts[3 * i + axis] = B.coord(axis, i);
  }
  if (interpolate) {
    const olgpu_status st = olgpu_interpolate_field(h, var, g, 0, pts.data(), np, ord, val.data());
    if (st != OLGPU_OK) return st;
  } else {
    std::vector<double> u((size_t)B.b.nx * B.b.ny * B.b.nz);
    const olgpu_status st = olgpu_download(h, g, var, u.data());
    if (st != OLGPU_OK) return st;
    for (int i = 0; i < np; i++) {
      int ijk[3] = {node[0], node[1], node[2]};
      ijk[axis] = i;
      val[i] = u[((size_t)ijk[2] * B.b.ny + ijk[1]) * B.b.nx + ijk[0]];
    }
  }
  FILE *f = std::fopen(file.c_str(), "a");
  if (!f) return OLGPU_ERR_INVALID_ARG;
  for (int i = 0; i < np; i++) std::fprintf(f, "%.12e\t%.12e\t\n", B.coord(axis, i), val[i]);
  std::fprintf(f, "\n");
  std::fclose(f);
  return OLGPU_OK;
}

// ffunction::Print_2D of one box (src/ffunction.cc:477-735, called by
// multigrid::Print_2D with the Lagrange order 2): the plane through the
// normal coordinate 0 when the box holds it and the values are interpolated,
// else through the box's middle node; every node of the other two axes, the
// lower axis outer; "%.12e\t%.12e\t%.12e\t" lines, a blank line after each
// outer index and one more at the end.
olgpu_status print_box_plane(olgpu_hierarchy *h, const char *var, const BoxGeom &B, int g, int normal,
                             bool interpolate, const std::string &file)
{
  const int a1 = normal == 0 ? 1 : 0, a2 = normal == 2 ? 1 : 2;   // in-plane axes, a1 < a2
  const int nm = B.n(normal) % 2 == 0 ? B.n(normal) / 2 : (B.n(normal) - 1) / 2;
  double at = B.coord(normal, nm);
  if (interpolate && B.is_in_axis(normal, 0.0)) at = 0.0;
  const int n1 = B.n(a1), n2 = B.n(a2);
  std::vector<double> pts(3 * (size_t)n1 * n2), val((size_t)n1 * n2);
  for (int p = 0; p < n1; p++)
    for (int q = 0; q < n2; q++) {
      double *x = &pts[3 * ((size_t)p * n2 + q)];
      x[normal] = at;
      x[a1] = B.coord(a1, p);
      x[a2] = B.coord(a2, q);
    }
  if (interpolate) {
    const olgpu_status st = olgpu_interpolate_field(h, var, g, 0, pts.data(), (long long)val.size(), 2, val.data());
    if (st != OLGPU_OK) return st;
  } else {
    std::vector<double> u((size_t)B.b.nx * B.b.ny * B.b.nz);
    const olgpu_status st = olgpu_download(h, g, var, u.data());
    if (st != OLGPU_OK) return st;
    for (int p = 0; p < n1; p++)
      for (int q = 0; q < n2; q++) {
        int ijk[3];
        ijk[normal] = nm;
        ijk[a1] = p;
        ijk[a2] = q;
        val[(size_t)p * n2 + q] = u[((size_t)ijk[2] * B.b.ny + ijk[1]) * B.b.nx + ijk[0]];
      }
  }
  FILE *f = std::fopen(file.c_str(), "a");
  if (!f) return OLGPU_ERR_INVALID_ARG;
  for (int p = 0; p < n1; p++) {
    for (int q = 0; q < n2; q++) {
      const size_t r = (size_t)p * n2 + q;
      std::fprintf(f, "%.12e\t%.12e\t%.12e\t\n", pts[3 * r + a1], pts[3 * r + a2], val[r]);
    }
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "\n");
  std::fclose(f);
  return OLGPU_OK;
}

// ffunction::Print_3D of one box (src/ffunction.cc:412-475): every point in
// the reference's storage order (olgpu_storage_order), "%.12e\t" x, y, z and
// the node value of u, then a line end; no blank line at the end.
olgpu_status print_box_3d(olgpu_hierarchy *h, const char *var, const BoxGeom &B, int g, const std::string &file)
{
  const size_t np = (size_t)B.b.nx * B.b.ny * B.b.nz;
  std::vector<double> u(np);
  std::vector<long long> order(np);
  olgpu_status st = olgpu_download(h, g, var, u.data());
  if (st == OLGPU_OK) st = olgpu_storage_order(&B.b, order.data());
  if (st != OLGPU_OK) return st;
  FILE *f = std::fopen(file.c_str(), "a");
  if (!f) return OLGPU_ERR_INVALID_ARG;
  for (long long q : order) {
    const int i = (int)(q % B.b.nx), j = (int)((q / B.b.nx) % B.b.ny), k = (int)(q / ((long long)B.b.nx * B.b.ny));
    std::fprintf(f, "%.12e\t%.12e\t%.12e\t%.12e\t\n", B.coord(0, i), B.coord(1, j), B.coord(2, k), u[(size_t)q]);
  }
  std::fclose(f);
  return OLGPU_OK;
}

// multigrid::Print_Interpol_1D along one axis: from -LD/2 by D (LD/1000 when
// D <= 0) while <= LD/2, the other coordinates 0, points outside the largest
// box skipped; "%.18e\t%.18e" lines, then a blank line.
olgpu_status print_interpol_1d(olgpu_hierarchy *h, const char *var, int axis, double LD, double D, int ord,
                               int first_level, const std::string &file)
{
  const double xi = -0.5 * LD, xf = 0.5 * LD, Dx = D > 0.0 ? D : LD / 1000;
  std::vector<double> pts, xs;
  for (double x = xi; x <= xf; x += Dx) {
    double p[3] = {0.0, 0.0, 0.0};
    p[axis] = x;
    pts.insert(pts.end(), p, p + 3);
    xs.push_back(x);
  }
  std::vector<double> val(xs.size());
  const olgpu_status st =
      olgpu_interpolate_field(h, var, -1, first_level, pts.data(), (long long)xs.size(), ord, val.data());
  if (st != OLGPU_OK) return st;
  FILE *f = std::fopen(file.c_str(), "a");
  if (!f) return OLGPU_ERR_INVALID_ARG;
  for (size_t i = 0; i < xs.size(); i++)
    if (!std::isnan(val[i])) std::fprintf(f, "%.18e\t%.18e\n", xs[i], val[i]);
  std::fprintf(f, "\n");
  std::fclose(f);
  return OLGPU_OK;
}

// multigrid::Print_Interpol_2D, the z = 0 plane: x and y from -L/4 by L/200
// while <= L/4; "%.18e\t%.18e\t%.18e" lines, a blank line after each x and
// one more at the end.
olgpu_status print_interpol_xy(olgpu_hierarchy *h, const char *var, double LD1, double LD2, int ord,
                               int first_level, const std::string &file)
{
  const double x1i = -0.25 * LD1, x2i = -0.25 * LD2, x1f = 0.25 * LD1, x2f = 0.25 * LD2;
  const double Dx1 = LD1 / 200, Dx2 = LD2 / 200;
  std::vector<double> pts, xs, ys;
  std::vector<int> row_end;
  for (double x = x1i; x <= x1f; x += Dx1) {
    for (double y = x2i; y <= x2f; y += Dx2) {
      const double p[3] = {x, y, 0.0};
      pts.insert(pts.end(), p, p + 3);
      xs.push_back(x);
      ys.push_back(y);
    }
    row_end.push_back((int)xs.size());
  }
  std::vector<double> val(xs.size());
  const olgpu_status st =
      olgpu_interpolate_field(h, var, -1, first_level, pts.data(), (long long)xs.size(), ord, val.data());
  if (st != OLGPU_OK) return st;
  FILE *f = std::fopen(file.c_str(), "a");
  if (!f) return OLGPU_ERR_INVALID_ARG;
  size_t q = 0;
  for (int e : row_end) {
    for (; q < (size_t)e; q++) std::fprintf(f, "%.18e\t%.18e\t%.18e\n", xs[q], ys[q], val[q]);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "\n");
  std::fclose(f);
  return OLGPU_OK;
}

int fail(olgpu_status st, const char *what)
{
  std::fprintf(stderr, "Olliptic_gpu.x: %s: %s (status %d)\n", what, olgpu_last_error(), (int)st);
  return (int)st;
}

bool file_exists(const std::string &name)
{
  FILE *f = std::fopen(name.c_str(), "r");
  if (f) std::fclose(f);
  return f != nullptr;
}

bool read_file(const std::string &name, std::string &text)
{
  FILE *f = std::fopen(name.c_str(), "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  text.clear();
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  std::fclose(f);
  return true;
}

// Reads the next number the way `stream >> double` does (leading white space
// skipped); false at the end of the text or on a token that is no number.
bool next_number(const std::string &t, size_t &pos, double &v)
{
  while (pos < t.size() && std::isspace((unsigned char)t[pos])) pos++;
  if (pos >= t.size()) return false;
  char *end = nullptr;
  v = std::strtod(t.c_str() + pos, &end);
  if (end == t.c_str() + pos) return false;
  pos = (size_t)(end - t.c_str());
  return true;
}

// u at the points, each point checked against the largest box as the
// exporters do ("bam grid bigger than Olliptic grid": exit status 1).
int export_values(olgpu_hierarchy *h, int ord, const std::vector<double> &xyz, std::vector<double> &val)
{
  val.assign(xyz.size() / 3, 0.0);
  if (val.empty()) return 0;
  const olgpu_status st = olgpu_interpolate(h, -1, 0, xyz.data(), (long long)val.size(), ord, val.data());
  if (st != OLGPU_OK) return fail(st, "export");
  for (size_t q = 0; q < val.size(); q++)
    if (std::isnan(val[q])) {
      std::printf("X: %e\tY: %e\tZ: %e\n", xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]);
      std::printf("Error: bam grid bigger than Olliptic grid\n");
      return 1;
    }
  return 0;
}

// elliptic::IO_bam (src/output.cc:377-410) and multigrid::Print_IO_BAM
// (src/multigrid.cc:990-1120): the files <prefix><level><"", a..e> that exist,
// level by level until a level has none; in each, every record "x y z val" is
// rewritten in place, from the record's first byte, as x, y, z (%16.9e,
// %17.9e, %17.9e) and u there (%24.15e), and reading resumes one byte after
// the old value.  A file with a point outside the largest box is left as it
// was (the reference has rewritten the records before that point when it
// stops).
int export_bam(olgpu_hierarchy *h, int ord, const std::string &prefix)
{
  static const char *ending[6] = {"", "a", "b", "c", "d", "e"};
  std::vector<std::string> files;
  for (int level = 0;; level++) {
    int found = 0;
    for (const char *e : ending) {
      const std::string f = prefix + std::to_string(level) + e;
      if (file_exists(f)) {
        std::printf("File found: %s\n", f.c_str());
        files.push_back(f);
        found++;
      }
    }
    if (!found) break;
  }
  for (const std::string &name : files) {
    std::string t;
    if (!read_file(name, t)) continue;
    std::printf("reading from: %s\n", name.c_str());
    // the records and where each starts and ends, read as the exporter does:
    // the positions do not move when a rewrite has another length
    std::vector<size_t> start, after;
    std::vector<double> xyz;
    size_t pos = 0;
    for (;;) {
      const size_t r1 = pos;
      double x, y, z, v;
      size_t q = pos;
      if (!next_number(t, q, x) || !next_number(t, q, y) || !next_number(t, q, z) || !next_number(t, q, v)) break;
      start.push_back(r1);
      after.push_back(q);
      xyz.insert(xyz.end(), {x, y, z});
      pos = q + 1;
      if (pos > t.size()) break;
    }
    std::vector<double> val;
    const int rc = export_values(h, ord, xyz, val);
    if (rc) return rc;
    // rewrite record by record; a later record is read from the text as the
    // earlier rewrites left it, as the reference's in-place stream does
    std::string out = t;
    pos = 0;
    for (size_t rrec = 0;; rrec++) {
      const size_t r1 = pos;
      double x, y, z, v;
      size_t q = pos;
      if (!next_number(out, q, x) || !next_number(out, q, y) || !next_number(out, q, z) || !next_number(out, q, v))
        break;
      double u = rrec < val.size() && x == xyz[3 * rrec] && y == xyz[3 * rrec + 1] && z == xyz[3 * rrec + 2]
                     ? val[rrec]
                     : std::nan("");
      if (std::isnan(u)) {   // the text changed under the rewrite: read this point afresh
        std::vector<double> p1 = {x, y, z}, v1;
        const int rc1 = export_values(h, ord, p1, v1);
        if (rc1) return rc1;
        u = v1[0];
      }
      char rec[160];
      const int n = std::snprintf(rec, sizeof rec, "%16.9e%17.9e%17.9e%24.15e", x, y, z, u);
      if (r1 + n > out.size()) out.resize(r1 + n, ' ');
      out.replace(r1, n, rec, n);
      pos = q + 1;
      if (pos > out.size()) break;
    }
    FILE *f = std::fopen(name.c_str(), "wb");
    if (!f) return (int)OLGPU_ERR_INVALID_ARG;
    std::fwrite(out.data(), 1, out.size(), f);
    std::fclose(f);
  }
  return 0;
}

// elliptic::IO_Zcode (src/output.cc:412-618) and multigrid::Print_IO_Zcode
// (src/multigrid.cc:1123-1180): the files <prefix><LL>-0<b>.mgid (two-digit
// level, b = 0..5) level by level until a level has none, then the shells
// <prefix>SH-{xm,xp,ym,yp,zm,zp}.mgid; each record "x y z val" becomes the
// line "x y z u" (%.16e) of <file>_m.  The reference's read loop ends on the
// end-of-file flag, so when the last record is followed by white space it
// is written twice; that is kept.
int export_zcode(olgpu_hierarchy *h, int ord, const std::string &prefix)
{
  std::vector<std::string> files;
  for (int level = 0;; level++) {
    int found = 0;
    for (int b = 0; b < 6; b++) {
      char f[32];
      std::snprintf(f, sizeof f, "%s%d-0%d.mgid", level < 10 ? "0" : "", level, b);
      const std::string name = prefix + f;
      if (file_exists(name)) {
        std::printf("File found: %s\n", name.c_str());
        files.push_back(name);
        found++;
      }
    }
    if (!found) break;
  }
  for (const char *sh : {"SH-xm.mgid", "SH-xp.mgid", "SH-ym.mgid", "SH-yp.mgid", "SH-zm.mgid", "SH-zp.mgid"})
    if (file_exists(prefix + sh)) {
      std::printf("File found: %s\n", (prefix + sh).c_str());
      files.push_back(prefix + sh);
    }
  for (const std::string &name : files) {
    std::string t;
    if (!read_file(name, t)) continue;
    std::printf("reading from: %s\n", name.c_str());
    std::vector<double> xyz;
    size_t pos = 0;
    bool trailing = false;   // white space after the last record
    for (;;) {
      double x, y, z, v;
      size_t q = pos;
      if (!next_number(t, q, x) || !next_number(t, q, y) || !next_number(t, q, z) || !next_number(t, q, v)) break;
      xyz.insert(xyz.end(), {x, y, z});
      pos = q;
      trailing = pos < t.size();
    }
    if (!xyz.empty() && trailing) xyz.insert(xyz.end(), xyz.end() - 3, xyz.end());
    std::vector<double> val;
    const int rc = export_values(h, ord, xyz, val);
    if (rc) return rc;
    FILE *f = std::fopen((name + "_m").c_str(), "w");
    if (!f) return (int)OLGPU_ERR_INVALID_ARG;
    for (size_t q = 0; q < val.size(); q++)
      std::fprintf(f, "%.16e %.16e %.16e %.16e\n", xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2], val[q]);
    std::fclose(f);
  }
  return 0;
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
  else if (equation == "Poisson") p.equation = OLGPU_EQ_POISSON;
  else if (equation == "Boundary-test") p.equation = OLGPU_EQ_BOUNDARY_TEST;
  else if (equation == "Multibox-test") p.equation = OLGPU_EQ_MULTIBOX_TEST;
  else if (equation == "Bowen-York") p.equation = OLGPU_EQ_BOWEN_YORK;
  else {
    std::fprintf(stderr, "Olliptic_gpu.x: equation %s is not on the puncture FAS path\n", equation.c_str());
    return (int)OLGPU_ERR_INVALID_ARG;
  }
  // elliptic::Set_Method (src/elliptic.cc:229-294): V-cycles, W-cycles, or
  // the analytic approximation alone (AppPuncture, elliptic::ApproximateID).
  // Like interface.cc:1333-1354 a name it does not know means Vcycle;
  // Gauss-Seidel (elliptic::Gauss_Seidel, src/elliptic.cc:1389-1454) is not
  // built, and Full-Multigrid is an empty member in the reference
  // (include/elliptic.h:323-325: it leaves u at the initial guess), so both
  // are refused rather than replaced.
  const char *me = A.find({"-m", "--method"});
  const std::string method = me ? me : "Vcycle";
  const bool approx_only = method == "AppPuncture";
  if (method == "Wcycle") p.method = OLGPU_METHOD_WCYCLE;
  else if (method == "Gauss-Seidel" || method == "Full-Multigrid") {
    std::fprintf(stderr, "Olliptic_gpu.x: method %s is not on the puncture FAS path\n", method.c_str());
    return (int)OLGPU_ERR_INVALID_ARG;
  }
  // the boundary condition (interface.cc:272, Dirichlet without -B): Robin
  // (what every pars/ file passes) or Dirichlet; another is refused rather
  // than replaced
  const char *bc = A.find({"-B", "--boundary"});
  const std::string boundary = bc ? bc : "Dirichlet";
  if (boundary == "Robin") p.boundary = OLGPU_BC_ROBIN;
  else if (boundary == "Dirichlet") p.boundary = OLGPU_BC_DIRICHLET;
  else {
    std::fprintf(stderr, "Olliptic_gpu.x: boundary %s is not on the GPU path\n", boundary.c_str());
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

  {   // interface.cc:1168-1176: -iob needs -iof
    const char *iof = A.find({"-iof", "--io-bam-file"});
    if (A.yes({"-iob", "--io-bam"}) && (!iof || !std::strcmp(iof, "none"))) {
      std::printf("\n\n*** Error: Missing file.\n");
      return 1;
    }
  }
  // the output directory exists from start-up on, as the reference's
  const char *o = A.find({"-o", "--out-dir"});
  const std::string out = o ? o : "Output";
  if (!prepare_output_dir(out, argc, argv)) {
    std::fprintf(stderr, "Olliptic_gpu.x: cannot create the output directory %s\n", out.c_str());
    return (int)OLGPU_ERR_INVALID_ARG;
  }
  const std::string dir = out + "/";
  const char *so = A.find({"-so", "--std-output"});
  const bool std_output = !so || !std::strcmp(so, "yes");
  const bool std_partial = so && !std::strcmp(so, "partial");
  {   // stdout0.out: the banner now (main.cc:111), the cycles after the solve
    FILE *f = std::fopen((dir + "stdout0.out").c_str(), "a");
    if (f && (std_output || std_partial)) {
      const char *eq_str = p.equation == OLGPU_EQ_PUNCTURES        ? "Punctures ID"
                           : p.equation == OLGPU_EQ_POISSON        ? "Poisson"
                           : p.equation == OLGPU_EQ_BOUNDARY_TEST  ? "Robin boundary test"
                           : p.equation == OLGPU_EQ_MULTIBOX_TEST  ? "Multibox test"
                           : p.equation == OLGPU_EQ_BOWEN_YORK     ? "Bowen-York momentum constrain test"
                                                                   : "";   // the scalar field has no name there
      write_banner(f, p, eq_str,
                   approx_only                          ? "Analitical Approximate"
                   : p.method == OLGPU_METHOD_WCYCLE    ? "Multigrid W-Cycle"
                                                        : "Multigrid V-Cycles",
                   p.boundary == OLGPU_BC_ROBIN ? "Robin" : "Dirichlet", dir, boxes, nb, nl, mg, approx_only);
    }
    if (f) std::fclose(f);
  }

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
  const char *guess = A.find({"-gpu-guess"});
  if (approx_only || (guess && !std::strcmp(guess, "approx"))) {
    st = olgpu_approximate_id(h, approx_only ? 0 : 1);
    if (st != OLGPU_OK) {
      olgpu_hierarchy_destroy(h);
      return fail(st, "approximate initial data");
    }
  }
  if (approx_only) {
    // elliptic::Get_Puncture_App (src/elliptic.cc:2232-2444): u at the node
    // at or after each puncture, added over the finest boxes that hold it
    std::vector<double> up(p.numbh, 0.0);
    for (int g = 0; g < nb; g++) {
      if (boxes[g].level != nl - 1) continue;
      const BoxGeom B{boxes[g]};
      for (int j = 0; j < p.numbh; j++) {
        const double q[3] = {p.x[j], p.y[j], p.z[j]};
        if (!(B.is_in_axis(0, q[0]) && B.is_in_axis(1, q[1]) && B.is_in_axis(2, q[2]))) continue;
        double node[3], v = 0;
        for (int a = 0; a < 3; a++) node[a] = B.coord(a, B.locate(a, q[a]));
        st = olgpu_interpolate(h, g, 0, node, 1, 1, &v);
        if (st != OLGPU_OK) {
          olgpu_hierarchy_destroy(h);
          return fail(st, "approximate initial data");
        }
        up[j] += v;
      }
    }
    for (int i = 0; i < p.numbh; i++)
      std::printf(" == Approximate ID: puncture %d\n x : %.7e\t y : %.7e\t z : %.7e\t u : %.7e\n", i, p.x[i], p.y[i],
                  p.z[i], up[i]);
  }
  olgpu_report rep{};
  if (!approx_only) {
    st = olgpu_solve(h, nullptr, &rep);   // the reference stop rule
    const char *cyc = p.method == OLGPU_METHOD_WCYCLE ? "W-cycle" : "V-cycle";
    for (int c = 0; c < rep.cycles && c < 256; c++) std::printf("  %s %3d  norm %.6e\n", cyc, c + 1, rep.res[c]);
    if (st != OLGPU_OK) {
      olgpu_hierarchy_destroy(h);
      return fail(st, "solve");
    }
    std::printf("Solved in %d %ss, norm %.6e, %.3f ms on the device\n", rep.cycles, cyc, rep.final_res,
                olgpu_last_device_ms(h));
  }
  // every Print_Pre_Cycle / Print_Post_Cycle call of the solve
  std::vector<olgpu_cycle_event> events;
  if (std_output && !approx_only) {
    long long total = 0;
    if (olgpu_cycle_events(h, 0, 0, nullptr, &total) == OLGPU_OK && total > 0) {
      events.resize((size_t)total);
      if (olgpu_cycle_events(h, 0, (int)total, events.data(), &total) != OLGPU_OK) events.clear();
    }
  }
  if (std_output && !approx_only) {   // stdout0.out: the cycle tables
    FILE *f = std::fopen((dir + "stdout0.out").c_str(), "a");
    const double eps_coarse = 2 * 2.220446049250313080847e-16;
    if (f) write_cycle_tables(f, events, nl, p.tol < eps_coarse ? eps_coarse : p.tol);
    if (f) std::fclose(f);
  }
  // Loo.gp: the cycle number and norm of every pre-smoothing step and
  // coarsest solve (Print_Pre_Cycle)
  if (std_output && !approx_only) {
    FILE *f = std::fopen((dir + "Loo.gp").c_str(), "a");
    for (const olgpu_cycle_event &e : events)
      if (f && !e.post) std::fprintf(f, "%lld\t%.18e\n", e.cycle, e.norm);
    if (f) std::fclose(f);
  }
  if (!approx_only && p.equation < OLGPU_EQ_POISSON) {   // Vcycle prints ADM for punctures only
    std::printf("Puncure method: \n");
    double adm[OLGPU_MAX_BH];
    olgpu_adm_mass(h, adm);
    for (int i = 0; i < p.numbh; i++) std::printf("ADM mass[%d] = %.17g\n", i, adm[i]);
  }

  // elliptic::Print_Solution (src/output.cc:624-730): each variable (u, or
  // Bowen-York's V1, V2, V3, lambda) in turn
  const bool print_1d = A.logic({"-p1d", "--print-1d"}, true);
  const bool print_2d = A.logic({"-p2d", "--print-2d"}, false);
  const bool print_3d = A.logic({"-p3d", "--print-3d"}, false);
  const bool print_interpol = A.logic({"-pint", "--print-interpol"}, true);
  const bool interpol_output = A.logic({"-int", "--interpol-output"}, true);
  if (print_1d || print_2d || print_3d || print_interpol) {
    const int ord = p.order + 1;
    std::printf("Printing...\n");
    olgpu_status ps = OLGPU_OK;
    // the analytic method's hierarchy has no multigrid coarse grids: its
    // levels are the refinement levels, numbered from the base
    const int l0 = approx_only ? mg : 0;
    static const char *by_vars[4] = {"V1", "V2", "V3", "lambda"};
    const bool by = p.equation == OLGPU_EQ_BOWEN_YORK;
    for (int iv = 0; iv < (by ? 4 : 1) && ps == OLGPU_OK; iv++) {
      const char *var = by ? by_vars[iv] : "u";
      const std::string vs = var;
      if (print_1d) {
        std::vector<int> in_level(nl, 0);
        static const char *ext[3] = {".x", ".y", ".z"};
        for (int l = l0; l < nl && ps == OLGPU_OK; l++)
          for (int g = 0; g < nb && ps == OLGPU_OK; g++) {
            if (boxes[g].level != l) continue;
            const BoxGeom B{boxes[g]};
            const std::string stem =
                dir + vs + "-l" + std::to_string(l - l0) + "b" + std::to_string(in_level[l]++) + "-0";
            for (int a = 0; a < 3 && ps == OLGPU_OK; a++)
              ps = print_box_cut(h, var, B, g, a, interpol_output, ord, stem + ext[a]);
          }
      }
      if (print_2d) {   // the planes .yz, .xz, .xy of every box, level by level
        std::vector<int> in_level(nl, 0);
        static const char *ext[3] = {".yz", ".xz", ".xy"};
        for (int l = l0; l < nl && ps == OLGPU_OK; l++)
          for (int g = 0; g < nb && ps == OLGPU_OK; g++) {
            if (boxes[g].level != l) continue;
            const BoxGeom B{boxes[g]};
            const std::string stem =
                dir + vs + "-l" + std::to_string(l - l0) + "b" + std::to_string(in_level[l]++) + "-0";
            for (int a = 0; a < 3 && ps == OLGPU_OK; a++)
              ps = print_box_plane(h, var, B, g, a, interpol_output, stem + ext[a]);
          }
      }
      if (print_3d) {   // every point of every box, level by level
        std::vector<int> in_level(nl, 0);
        for (int l = l0; l < nl && ps == OLGPU_OK; l++)
          for (int g = 0; g < nb && ps == OLGPU_OK; g++) {
            if (boxes[g].level != l) continue;
            const BoxGeom B{boxes[g]};
            const std::string file =
                dir + vs + "-l" + std::to_string(l - l0) + "b" + std::to_string(in_level[l]++) + "-0.xyz";
            ps = print_box_3d(h, var, B, g, file);
          }
      }
      if (print_interpol && ps == OLGPU_OK) {
        const double Dp = A.num({"-Dp", "--d-print"}, -1.0);
        const double Lx = A.num({"-Lx", "--length-x"}, p.L), Ly = A.num({"-Ly", "--length-y"}, p.L),
                     Lz = A.num({"-Lz", "--length-z"}, p.L);
        static const char *ext[3] = {".X", ".Y", ".Z"};
        const double LD[3] = {Lx, Ly, Lz};
        for (int a = 0; a < 3 && ps == OLGPU_OK; a++)
          ps = print_interpol_1d(h, var, a, LD[a], Dp, ord, l0, dir + vs + ext[a]);
        if (ps == OLGPU_OK) ps = print_interpol_xy(h, var, Lx, Ly, ord, l0, dir + vs + ".XY");
      }
    }
    if (ps != OLGPU_OK) {
      olgpu_hierarchy_destroy(h);
      return fail(ps, "output");
    }
    std::printf("done\n");
  }
  // initial data for other codes (main.cc:133-141): u at their grid points
  const char *iof = A.find({"-iof", "--io-bam-file"});
  int rc = 0;
  if (A.yes({"-iob", "--io-bam"})) rc = export_bam(h, p.order + 1, iof);
  if (!rc && A.yes({"-ioZ", "--io-Zcode"})) rc = export_zcode(h, p.order + 1, iof ? iof : "none");
  olgpu_hierarchy_destroy(h);
  return rc;
}
