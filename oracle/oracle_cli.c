/* oracle_cli.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Command-line driver for the CPU restatement (olliptic_oracle.c).  It reads
 * the reference's Olliptic.x flags that matter for the puncture FAS path
 * (src/interface.cc:73-273, 748-856; unknown flags are ignored, as in the
 * reference) and writes the same dump format as ref_harness.cc, so that the
 * two can be compared file by file.
 *
 *   oracle_cli <mode> <outdir> -- <Olliptic.x arguments...>
 *   modes: coeff | cycles:K | solve | fixed:TOL:MAXC | time:K (no dump)
 */
#define _GNU_SOURCE
#include "olliptic_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

static int parse_args(int argc, char **argv, orc_problem *p)
{
  orc_problem_defaults(p);
  p->mp[0] = 0;
  for (int i = 0; i + 1 < argc; i++) {
    const char *a = argv[i], *v = argv[i + 1];
    if (!strcmp(a, "-eq") || !strcmp(a, "--equation")) {
      if (!strcmp(v, "Punctures")) p->equation = 0;
      else if (!strcmp(v, "Punctures_scalar_field")) p->equation = 1;
      else return -1;
    } else if (!strcmp(a, "-NumBH") || !strcmp(a, "--num-bh")) p->numbh = atoi(v);
    else if (!strcmp(a, "-L") || !strcmp(a, "--length")) p->L = atof(v);
    else if (!strcmp(a, "-N") || !strcmp(a, "-n")) p->n = atoi(v);
    else if (!strcmp(a, "-O") || !strcmp(a, "--order")) p->order = atoi(v);
    else if (!strcmp(a, "-l") || !strcmp(a, "--levels")) p->levels = atoi(v);
    else if (!strcmp(a, "-s") || !strcmp(a, "--tolerance")) p->tol = atof(v);
    else if (!strcmp(a, "-nu1") || !strcmp(a, "--pre-smooth")) p->nu1 = atoi(v);
    else if (!strcmp(a, "-nu2") || !strcmp(a, "--post-smooth")) p->nu2 = atoi(v);
    else if (!strcmp(a, "-psc") || !strcmp(a, "-ps_case")) p->ps_case = atoi(v);
    else if (!strcmp(a, "-phi0") || !strcmp(a, "--phi0_sf")) p->ps_phi0 = atof(v);
    else if (!strcmp(a, "-r0") || !strcmp(a, "--radius_sf_r0")) p->ps_r0 = atof(v);
    else if (!strcmp(a, "-sigma") || !strcmp(a, "--sigma_sf")) p->ps_sigma = atof(v);
    else if (!strcmp(a, "-a2") || !strcmp(a, "--a2_sf")) p->ps_a2 = atof(v);
  }
  if (p->numbh < 1 || p->numbh > ORC_MAX_BH) return -1;
  for (int i = 0; i + 1 < argc; i++) {
    for (int j = 0; j < p->numbh; j++) {
      char key[32];
      double v = atof(argv[i + 1]);
#define KEY(name, dst) snprintf(key, sizeof key, "-" name "%d", j + 1); if (!strcmp(argv[i], key)) dst[j] = v;
      KEY("bhmp", p->mp) KEY("bhx", p->x) KEY("bhy", p->y) KEY("bhz", p->z)
      KEY("bhpx", p->px) KEY("bhpy", p->py) KEY("bhpz", p->pz)
      KEY("bhsx", p->sx) KEY("bhsy", p->sy) KEY("bhsz", p->sz)
#undef KEY
    }
  }
  return 0;
}

static void dump(const char *dir, orc_solver *s, const char *name, int g, long n)
{
  char path[1024];
  snprintf(path, sizeof path, "%s/b%d_%s.f64", dir, g, name);
  double *buf = (double *)malloc(sizeof(double) * n);
  orc_get_field(s, g, name, buf);
  FILE *fp = fopen(path, "wb");
  if (!fp) { perror(path); exit(2); }
  fwrite(buf, sizeof(double), n, fp);
  fclose(fp);
  free(buf);
}

static double now(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

int main(int argc, char **argv)
{
  if (argc < 4 || strcmp(argv[3], "--")) {
    fprintf(stderr, "usage: oracle_cli <mode> <outdir> -- <Olliptic args>\n");
    return 2;
  }
  const char *mode = argv[1], *out = argv[2];
  orc_problem P;
  if (parse_args(argc - 4, argv + 4, &P)) { fprintf(stderr, "bad arguments\n"); return 2; }
  orc_solver *s = orc_create(&P);
  if (!s) { fprintf(stderr, "could not build the hierarchy\n"); return 2; }
  int nb = orc_num_boxes(s);
  double norms[4096], deltas[4096];
  int nc = 0;
  if (!strncmp(mode, "time:", 5)) {
    int K = atoi(mode + 5);
    double t0 = now();
    double res = 0;
    for (int c = 0; c < K; c++) res = orc_vcycle(s);
    double t1 = now();
    printf("{\"cycles\": %d, \"seconds\": %.6f, \"res\": %.17g}\n", K, t1 - t0, res);
    orc_destroy(s);
    return 0;
  }
  mkdir(out, 0755);
  if (!strcmp(mode, "coeff")) {
  } else if (!strncmp(mode, "cycles:", 7)) {
    int K = atoi(mode + 7);
    for (int c = 0; c < K && c < 4096; c++) {
      norms[nc] = orc_vcycle(s);
      deltas[nc] = 0;
      nc++;
    }
  } else if (!strcmp(mode, "solve")) {
    double res;
    orc_solve(s, 100000, &res);
  } else if (!strncmp(mode, "fixed:", 6)) {
    double tol = atof(mode + 6);
    const char *c2 = strchr(mode + 6, ':');
    int maxc = c2 ? atoi(c2 + 1) : 200;
    double res;
    orc_solve(s, 100000, &res);
    for (int c = 0; c < maxc && nc < 4096; c++) {
      /* max |du| over every box */
      double m = 0;
      double **prev = (double **)malloc(sizeof(double *) * nb);
      for (int g = 0; g < nb; g++) {
        orc_box_info bi;
        orc_box(s, g, &bi);
        long n = (long)bi.nx * bi.ny * bi.nz;
        prev[g] = (double *)malloc(sizeof(double) * n);
        orc_get_field(s, g, "u", prev[g]);
      }
      norms[nc] = orc_vcycle(s);
      for (int g = 0; g < nb; g++) {
        orc_box_info bi;
        orc_box(s, g, &bi);
        long n = (long)bi.nx * bi.ny * bi.nz;
        double *cur = (double *)malloc(sizeof(double) * n);
        orc_get_field(s, g, "u", cur);
        for (long q = 0; q < n; q++) {
          double d = fabs(cur[q] - prev[g][q]);
          if (d > m || d != d) m = d;
        }
        free(cur);
        free(prev[g]);
      }
      free(prev);
      deltas[nc++] = m;
      if (m <= tol) break;
    }
  } else {
    fprintf(stderr, "unknown mode\n");
    return 2;
  }
  char path[1024];
  snprintf(path, sizeof path, "%s/meta.txt", out);
  FILE *fp = fopen(path, "w");
  fprintf(fp, "levels %d\nmgrid_levels %d\norder %d\nnumbh %d\nncycles %d\n", orc_num_levels(s),
          orc_mgrid_levels(s), P.order, P.numbh, nc);
  for (int i = 0; i < nc; i++) fprintf(fp, "cycle %d %.17g %.17g\n", i, norms[i], deltas[i]);
  double adm[ORC_MAX_BH];
  orc_adm(s, adm);
  for (int i = 0; i < P.numbh; i++) fprintf(fp, "adm %d %.17g\n", i, adm[i]);
  for (int g = 0; g < nb; g++) {
    orc_box_info b;
    orc_box(s, g, &b);
    fprintf(fp, "box %d level %d n %d %d %d buf %d ord %d x0 %.17g %.17g %.17g x1 %.17g %.17g %.17g "
                "d %.17g %.17g %.17g c %.17g %.17g %.17g\n",
            g, b.level, b.nx, b.ny, b.nz, b.buf, b.order, b.xi, b.yi, b.zi, b.xf, b.yf, b.zf, b.dx,
            b.dy, b.dz, b.cx, b.cy, b.cz);
    long n = (long)b.nx * b.ny * b.nz;
    dump(out, s, "u", g, n);
    if (!strcmp(mode, "coeff")) {
      dump(out, s, "b", g, n);
      dump(out, s, "c", g, n);
      if (P.equation == 1) {
        dump(out, s, "d", g, n);
        dump(out, s, "e", g, n);
      }
    }
  }
  fclose(fp);
  orc_destroy(s);
  return 0;
}
