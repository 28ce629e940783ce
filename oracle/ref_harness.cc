// ref_harness.cc -- test infrastructure only.
//
// Drives the UNMODIFIED reference solver (WuShichao/OllipticID, compiled from
// its own sources by oracle/Makefile into oracle/_ref/) and dumps what the
// parity tests need: per-box geometry, coefficient fields, the solution on
// every box (u, or every variable of a system: V1, V2, V3, lambda for
// Bowen-York, b<box>_<name>.f64), per-cycle residual norms and the ADM masses
// at 17 digits.
//
// The reference keeps its solver internals private; this harness opens them
// (access specifiers only, no behaviour change) so that it can call
// elliptic::FASN (src/elliptic.cc:1468) cycle by cycle and read multigrid
// fields (include/multigrid.h:98).  Construction follows src/main.cc:101-118.
//
// Usage:
//   ref_harness <mode> <outdir> -- <Olliptic.x arguments...>
// modes:
//   coeff           dump geometry + b, c (and d, e, rho0 if present)
//   cycles:K        run exactly K FAS V-cycles from the initial guess
//   solve           run elliptic::Solve (the CLI stop rule, src/elliptic.cc:1330)
//   fixed:TOL:MAXC  Solve(), then more V-cycles until max|du| <= TOL on every
//                   box or MAXC extra cycles ran
#include <iostream>
#include <iomanip>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <valarray>
#include <map>
#include <cmath>
#include <limits>
#include <cstdlib>
#include <cstring>
#include <sys/stat.h>

#include <algorithm>
#include <list>
#include <set>
#define private public
#define protected public
#define class struct
#include "elliptic.h"
#undef class
#undef private
#undef protected

static void dump_field(const std::string &path, ffunction *F)
{
  domain *D = F->Get_domain();
  const size_t nx = D->Get_Nx(), ny = D->Get_Ny(), nz = D->Get_Nz();
  std::vector<double> buf(nx * ny * nz);
  size_t p = 0;
  for (size_t k = 0; k < nz; k++)
    for (size_t j = 0; j < ny; j++)
      for (size_t i = 0; i < nx; i++)
        buf[p++] = F->Get_val((int)i, (int)j, (int)k);
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) { perror(path.c_str()); exit(2); }
  fwrite(buf.data(), sizeof(double), buf.size(), fp);
  fclose(fp);
}

static bool has_field(elliptic &E, size_t l, const std::string &name)
{
  for (size_t i = 0; i < E.total_names.size(); i++)
    if (E.total_names[i] == name) return true;
  return false;
}

// every variable of the equation (elliptic::var_names) on every box
static void snapshot_u(elliptic &E, std::vector<std::vector<double> > &snap)
{
  snap.clear();
  for (size_t l = 0; l < E.levels; l++)
    for (size_t b = 0; b < E.vars.Get_num_dom(l); b++)
      for (size_t iv = 0; iv < E.var_names.size(); iv++) {
        ffunction *U = E.vars.Get_ffunction(l, b, E.var_names[iv]);
        domain *D = U->Get_domain();
        const size_t n = D->Get_Nx() * D->Get_Ny() * D->Get_Nz();
        std::vector<double> v(n);
        for (size_t i = 0; i < n; i++) v[i] = U->Get_val((int)i);
        snap.push_back(v);
      }
}

static double max_delta(elliptic &E, const std::vector<std::vector<double> > &prev)
{
  std::vector<std::vector<double> > cur;
  snapshot_u(E, cur);
  double m = 0;
  for (size_t b = 0; b < cur.size(); b++)
    for (size_t i = 0; i < cur[b].size(); i++) {
      double d = fabs(cur[b][i] - prev[b][i]);
      if (d > m || d != d) m = d;
    }
  return m;
}

int main(int argc, char **argv)
{
  if (argc < 4 || std::string(argv[3]) != "--") {
    std::cerr << "usage: ref_harness <mode> <outdir> -- <Olliptic args>\n";
    return 2;
  }
  std::string mode = argv[1];
  std::string outdir = argv[2];
  mkdir(outdir.c_str(), 0755);

  // argv for the reference: program name + the remaining arguments
  std::vector<char *> rargv;
  rargv.push_back(argv[0]);
  for (int i = 4; i < argc; i++) rargv.push_back(argv[i]);

  interface Oll((int)rargv.size(), rargv.data());
  elliptic E(&Oll);
  std::cout.precision(17);

  std::vector<double> norms, deltas;
  int ncycles = 0;
  if (mode == "coeff") {
    // nothing to run
  } else if (mode.compare(0, 7, "cycles:") == 0) {
    int K = atoi(mode.c_str() + 7);
    for (int c = 0; c < K; c++) {
      std::vector<std::vector<double> > prev;
      snapshot_u(E, prev);
      double res = E.FASN(E.levels - 1, E.levels - 1, false, c);
      norms.push_back(res);
      deltas.push_back(max_delta(E, prev));
      ncycles++;
    }
  } else if (mode == "solve") {
    E.Solve();
  } else if (mode.compare(0, 6, "fixed:") == 0) {
    double tol = atof(mode.c_str() + 6);
    const char *c2 = strchr(mode.c_str() + 6, ':');
    int maxc = c2 ? atoi(c2 + 1) : 200;
    E.Solve();
    for (int c = 0; c < maxc; c++) {
      std::vector<std::vector<double> > prev;
      snapshot_u(E, prev);
      double res = E.FASN(E.levels - 1, E.levels - 1, false, 1000 + c);
      norms.push_back(res);
      double d = max_delta(E, prev);
      deltas.push_back(d);
      ncycles++;
      if (d <= tol) break;
    }
  } else {
    std::cerr << "unknown mode " << mode << "\n";
    return 2;
  }

  // ---- meta -------------------------------------------------------------
  std::ofstream meta((outdir + "/meta.txt").c_str());
  meta.precision(17);
  meta << "levels " << E.levels << "\n";
  meta << "mgrid_levels " << E.mgrid_levels << "\n";
  meta << "order " << E.order << "\n";
  meta << "numbh " << E.NumBH << "\n";
  meta << "ncycles " << ncycles << "\n";
  for (size_t i = 0; i < norms.size(); i++)
    meta << "cycle " << i << " " << norms[i] << " " << deltas[i] << "\n";
  for (size_t i = 0; i < E.ADM_mass.size(); i++)
    meta << "adm " << i << " " << E.ADM_mass[i] << "\n";
  size_t gb = 0;
  for (size_t l = 0; l < E.levels; l++)
    for (size_t b = 0; b < E.vars.Get_num_dom(l); b++, gb++) {
      ffunction *U = E.vars.Get_ffunction(l, b, E.var_names[0]);
      domain *D = U->Get_domain();
      meta << "box " << gb << " level " << l << " ibox " << b
           << " n " << D->Get_Nx() << " " << D->Get_Ny() << " " << D->Get_Nz()
           << " buf " << D->Get_buffer_x() << " ord " << D->Get_order()
           << " x0 " << D->Get_xi() << " " << D->Get_yi() << " " << D->Get_zi()
           << " x1 " << D->Get_xf() << " " << D->Get_yf() << " " << D->Get_zf()
           << " d " << D->Get_dx() << " " << D->Get_dy() << " " << D->Get_dz()
           << " c " << D->Get_Center_x() << " " << D->Get_Center_y() << " " << D->Get_Center_z()
           << " g0 " << D->gxi << " " << D->gyi << " " << D->gzi
           << " g1 " << D->gxf << " " << D->gyf << " " << D->gzf
           << " bound " << D->Get_Bound_Xi() << "\n";
      std::ostringstream pre;
      pre << outdir << "/b" << gb << "_";
      for (size_t iv = 0; iv < E.var_names.size(); iv++)
        dump_field(pre.str() + E.var_names[iv] + ".f64", E.vars.Get_ffunction(l, b, E.var_names[iv]));
      if (mode == "coeff") {
        const char *names[] = {"b", "c", "d", "e", "rho0", "rho1", "rho2", "rho3"};
        for (int f = 0; f < 8; f++)
          if (has_field(E, l, names[f]))
            dump_field(pre.str() + names[f] + ".f64", E.vars.Get_ffunction(l, b, names[f]));
      }
    }
  meta.close();
  return 0;
}
