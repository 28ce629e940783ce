/* olliptic_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of the reference's (WuShichao/OllipticID) FAS
 * multigrid solve of the puncture Hamiltonian constraint on nested boxes.
 * Used by tests/ (parity checker), __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg; never by the GPU product path.
 *
 * Layout: every box stores each field lexicographically, i fastest, ghost
 * layers included (the reference stores the same points in a permuted order,
 * include/domain.h:581-586; the permutation only matters for the order in
 * which its iterators visit points, which is reproduced below where it
 * matters: interior points in lexicographic order, Robin layers inner to
 * outer, src/domain.cc:574-1388).
 *
 * Floating-point expressions are written in the reference's evaluation order
 * (build with -ffp-contract=off) so that the iterates match the reference
 * bit for bit on the same host.
 *
 * Bowen-York (four unknowns V1, V2, V3, lambda, include/elliptic.h:772-803)
 * is restated as its fixed point, not its iterates: the reference smooths
 * and transfers the four together, this oracle solves V1, V2, V3 (each a
 * Poisson problem with its own source) and then lambda with the divergence
 * of the solved V as its source (orc_set_divergence_source).  The discrete
 * system, and so its fixed point, is the same; it is pinned against the
 * reference's own fixed point (tests/golden/bowen_york).
 */
#define _GNU_SOURCE
#include "olliptic_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EPS DBL_EPSILON
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* geometry: domain (include/domain.h, src/domain.cc)                        */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n[3];          /* points per axis, ghosts included                    */
  int buf;           /* ghost width max(order/2,1), src/domain.cc:531-538   */
  int order;
  int level;
  double d[3];       /* spacing                                            */
  double c[3];       /* centre                                             */
  double lo[3], hi[3];   /* per-rank extents xi..xf                          */
  double glo[3], ghi[3]; /* global extents gxi..gxf                          */
} odom;

/* Valid_N, src/interface.cc:883-945 */
static const int valid_sizes[63] = {
  3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 17, 19, 21,
  23, 25, 27, 29, 33, 37, 41, 45, 49, 53, 57, 65, 73, 81, 89, 97,
  105, 113, 129, 145, 161, 177, 193, 209, 225, 257, 289, 321, 353, 385, 417, 449,
  513, 577, 641, 705, 769, 833, 897, 1153, 1281, 1409, 1665, 1793, 2305, 2817, 3329};

int orc_valid_n(int N)
{
  for (int j = 0; j < 63; j++)
    if (valid_sizes[j] == N) return N;
  int lo = valid_sizes[61], hi = valid_sizes[62];
  int i = 0;
  while (i < 63 && valid_sizes[i] < N) {
    lo = valid_sizes[i];
    hi = (i + 1 < 63) ? valid_sizes[i + 1] : valid_sizes[62];
    i++;
  }
  return (N - lo < hi - N) ? lo : hi;
}

/* Set_Boundary for one rank covering the whole axis (size == 1, k == 0,
 * c == 1, no symmetry): src/domain.cc:450-525 */
static void set_boundary_axis(double *ti, double *tf, int *Nt, double gti,
                              double gtf, double dt)
{
  double lti = gti + 0.0;   /* gti + k*Lt/c with k = 0 */
  double ltf = gtf - 0.0;   /* gtf - (c-1-k)*Lt/c       */
  while (*ti + (double)(*Nt - 1) * dt > ltf) (*Nt)--;
  if (*ti + (double)(*Nt - 1) * dt < ltf - 0.5 * dt) (*Nt)++;
  *tf = *ti + (double)(*Nt - 1) * dt;
  while (*tf - (double)(*Nt - 1) * dt < lti) (*Nt)--;
  if (*tf - (double)(*Nt - 1) * dt > lti + 0.5 * dt) (*Nt)++;
  *ti = *tf - (double)(*Nt - 1) * dt;
}

/* domain::Make -> Set, Set_Buffer, Set_N (src/domain.cc:26-99, 292-445) */
static void dom_make(odom *D, int Nx, int Ny, int Nz, double dx, double dy,
                     double dz, double cx, double cy, double cz, int ord)
{
  int N[3] = {Nx, Ny, Nz};
  D->order = ord;
  D->level = 0;
  D->d[0] = dx; D->d[1] = dy; D->d[2] = dz;
  D->c[0] = cx; D->c[1] = cy; D->c[2] = cz;
  D->buf = ord / 2 >= 1 ? ord / 2 : 1;
  for (int a = 0; a < 3; a++) {
    int n = orc_valid_n(N[a]);
    double d = D->d[a];
    double gi = D->c[a] - 0.5 * (double)(n - 1) * d - (double)(D->buf - 1) * d;
    n += D->buf - 1;
    double gf = gi + (double)(n - 1) * d + (double)(D->buf - 1) * d;
    n += D->buf - 1;
    D->glo[a] = gi;
    D->ghi[a] = gf;
    double ti = gi, tf = gf;
    set_boundary_axis(&ti, &tf, &n, gi, gf, d);
    D->lo[a] = ti;
    D->hi[a] = tf;
    D->n[a] = n;
  }
}

static inline double dom_coord(const odom *D, int a, int i)
{
  return D->lo[a] + (double)i * D->d[a];   /* include/domain.h:714-727 */
}

static inline int dcomp(double x, double y)   /* include/domain.h:871-875 */
{
  return fabs(x - y) <= 3 * EPS;
}

/* Get_i / Get_j / Get_k binary search, src/domain.cc:1492-1675 */
static int dom_locate(const odom *D, int a, double x)
{
  const int nx = D->n[a];
  int i = 0;
  int sup = nx, inf = 0;
  int mid = nx % 2 == 0 ? nx / 2 : (nx - 1) / 2;
  if (D->lo[a] - x < 0.0 && x - D->hi[a] < 0.0) {
    i = mid;
    do {
      double xi = D->lo[a] + (double)i * D->d[a];
      if (xi > x || dcomp(xi, x)) {
        sup = i;
        i = (sup + inf) % 2 == 0 ? (sup + inf) / 2 : (sup + inf - 1) / 2;
      } else {
        inf = i;
        i = (sup + inf) % 2 == 0 ? (sup + inf) / 2 : (sup + inf - 1) / 2;
      }
    } while (inf + 1 < sup);
  } else {
    i = (D->lo[a] >= x) ? 0 : nx - 2;
  }
  return i + 1;
}

/* Is_In, include/domain.h:767-775 */
static int dom_is_in(const odom *D, double x, double y, double z)
{
  const double p[3] = {x, y, z};
  for (int a = 0; a < 3; a++)
    if (!(D->lo[a] - D->d[a] * 0.1 <= p[a] && p[a] <= D->hi[a] + D->d[a] * 0.1)) return 0;
  return 1;
}

/* is_in_nb, include/domain.h:839-850 */
static int dom_is_in_nb(const odom *D, double x, double y, double z)
{
  const double p[3] = {x, y, z};
  for (int a = 0; a < 3; a++) {
    double m = D->d[a] * ((double)D->buf - 0.1);
    if (!(D->lo[a] + m < p[a] && p[a] < D->hi[a] - m)) return 0;
  }
  return 1;
}

/* operator&& (A && B == B >= B - A), src/domain.cc:1877-1922, 1984-2005 */
static int dom_touch(const odom *A, const odom *B)
{
  for (int a = 0; a < 3; a++) {
    double ci = A->lo[a] > B->lo[a] ? A->lo[a] : B->lo[a];   /* max(B.xi, A.xi) */
    double cf = B->hi[a] < A->hi[a] ? B->hi[a] : A->hi[a];   /* min(B.xf, A.xf) */
    double di = ci < cf ? ci : cf;
    double df = ci < cf ? cf : ci;
    if (!(B->lo[a] <= di && df <= B->hi[a])) return 0;
  }
  return 1;
}

/* operator+, src/domain.cc:1810-1871 */
static void dom_plus(odom *C, const odom *A, const odom *B)
{
  double lo[3], hi[3], c[3];
  int n[3];
  for (int a = 0; a < 3; a++) {
    lo[a] = A->glo[a] < B->glo[a] ? A->glo[a] : B->glo[a];
    hi[a] = A->ghi[a] < B->ghi[a] ? B->ghi[a] : A->ghi[a];
    c[a] = 0.5 * (lo[a] + hi[a]);
    n[a] = (int)(size_t)((hi[a] - lo[a]) / A->d[a] + 1);
  }
  odom T;
  dom_make(&T, n[0], n[1], n[2], A->d[0], A->d[1], A->d[2], c[0], c[1], c[2], A->order);
  *C = T;
}

/* ------------------------------------------------------------------------ */
/* boxes and fields                                                          */
/* ------------------------------------------------------------------------ */
enum { F_U, F_B, F_C, F_D, F_E, F_RHO, F_R, F_W, F_WW, F_V, F_NUM };
static const char *field_names[F_NUM] = {"u", "b", "c", "d", "e", "rho", "r", "w", "ww", "v"};

typedef struct {
  odom D;
  long npts;
  double *f[F_NUM];
  double idx[3], idx2[3];
} obox;

struct orc_solver {
  orc_problem P;
  int nboxes;
  int levels;        /* total levels incl. multigrid coarse grids */
  int mgrid_levels;
  int *ndl;          /* boxes per level */
  int *first;        /* first box index per level */
  obox *box;
  double eps_solv, eps_coarse;
  double adm[ORC_MAX_BH];
  /* scalar field constants, src/elliptic.cc:71-81 */
  double ps_isigma, ps_phi0, ps_d1, ps_e1, ps_e2, ps_de1;
  int nan_flag;
  /* checker options (not part of the reference algorithm) */
  int multicolor;    /* 1: visit points by colour (i+j+k) mod (buf+1), as the GPU does */
  long coarse_cap;   /* cap on coarsest-grid sweeps per V-cycle */
  long coarse_iters; /* sweeps used by the last coarse solve */
  int wsmooth;       /* 1: full-weight W over INSIDE points before its transfer */
  double coarse_omega; /* over-relaxation of the coarsest-solve sweeps (1 = reference) */
  double coarse_rtol;  /* also stop once the sweep norm <= rtol * first sweep norm (0 = off) */
  int extra_coarse;    /* checker option: keep coarsening below 12 points (down to >= 5) */
  double lnorm[64][2]; /* last cycle: smoother norms per level (pre, post) */
  double coarse_norm;
  long ncycles;        /* top-level cycles run (the cycle count each starts from) */
  /* every Print_Pre_Cycle / Print_Post_Cycle call of the solve, in order */
  orc_event *ev;
  long nev, cap_ev;
  long w_cap;          /* checker guard: iterations of one level's W loop (the reference has none) */
};

static void log_event(orc_solver *S, int level, int post, long cycle, double norm)
{
  if (S->nev == S->cap_ev) {
    const long cap = S->cap_ev ? 2 * S->cap_ev : 256;
    orc_event *ev = (orc_event *)realloc(S->ev, sizeof(orc_event) * cap);
    if (!ev) return;
    S->ev = ev;
    S->cap_ev = cap;
  }
  S->ev[S->nev].level = level;
  S->ev[S->nev].post = post;
  S->ev[S->nev].cycle = cycle;
  S->ev[S->nev].norm = norm;
  S->nev++;
}

static inline long IDX(const obox *B, int i, int j, int k)
{
  return ((long)k * B->D.n[1] + j) * B->D.n[0] + i;
}

/* ------------------------------------------------------------------------ */
/* hierarchy: elliptic::Set_Grids, src/elliptic.cc:299-921                  */
/* ------------------------------------------------------------------------ */
typedef struct {
  odom *v;
  int n, cap;
} domvec;

static void dv_push(domvec *V, const odom *D)
{
  if (V->n == V->cap) {
    V->cap = V->cap ? 2 * V->cap : 16;
    V->v = (odom *)realloc(V->v, sizeof(odom) * V->cap);
  }
  V->v[V->n++] = *D;
}

static void dv_erase(domvec *V, int k)
{
  memmove(V->v + k, V->v + k + 1, sizeof(odom) * (V->n - k - 1));
  V->n--;
}

static int set_grids(orc_solver *S, domvec *Dv, int **ndl_out, int *nlev_out)
{
  const orc_problem *P = &S->P;
  int Nx = orc_valid_n(P->n);
  double Dx = fabs(P->L) / (double)(Nx - 1.0);   /* src/interface.cc:1061 */
  int base = S->extra_coarse ? 5 : 12;             /* full domain, :502-506 */
  int cap = 64;
  int *nx = (int *)malloc(sizeof(int) * cap);
  double *dxs = (double *)malloc(sizeof(double) * cap);
  int nl = 1;
  nx[0] = Nx;
  dxs[0] = Dx;
  /* multigrid coarsening, :510-651 (same for y and z: cubic problem) */
  for (;;) {
    int ntmp = (nx[nl - 1] + 1) / 2;
    if (ntmp < base) break;               /* limit reached on all axes */
    if (nl == cap) return -1;
    nx[nl] = ntmp;
    dxs[nl] = dxs[nl - 1] * 2.0;
    nl++;
  }
  if (nl <= 1) { free(nx); free(dxs); return -1; }
  int mg = nl - 1;
  S->mgrid_levels = mg;
  int levels = P->levels + mg;
  int *ndl = (int *)calloc(levels, sizeof(int));
  Dv->n = 0;
  for (int l = mg; l >= 0; l--) {            /* :686-701 */
    odom D;
    int gz = l == 0 ? P->order : 2;
    dom_make(&D, nx[l], nx[l], nx[l], dxs[l], dxs[l], dxs[l], 0, 0, 0, gz);
    dv_push(Dv, &D);
    ndl[mg - l] = 1;
  }
  /* refinement boxes, :712-828 */
  const odom *Db = &Dv->v[mg];
  for (int l = mg + 1; l < levels; l++) {
    for (int ib = 0; ib < P->numbh; ib++) {
      double pot = l - mg;
      double dl = Dx / pow(2.0, pot);
      double bh[3] = {P->x[ib], P->y[ib], P->z[ib]};
      double cc[3];
      for (int a = 0; a < 3; a++) {
        int i = dom_locate(&Dv->v[mg], a, bh[a]);
        double xi = dom_coord(&Dv->v[mg], a, i - 1);
        double xf = dom_coord(&Dv->v[mg], a, i);
        if (dcomp(xi, bh[a]) || dcomp(xf, bh[a]))
          cc[a] = bh[a];
        else {
          while (xi + dl < bh[a]) xi += dl;
          while (xf - dl > bh[a]) xf -= dl;
          cc[a] = fabs(xi - bh[a]) < fabs(xf - bh[a]) ? xi : xf;
        }
      }
      odom D;
      dom_make(&D, Nx, Nx, Nx, dl, dl, dl, cc[0], cc[1], cc[2], P->order);
      dv_push(Dv, &D);
      Db = &Dv->v[mg];
    }
    ndl[l] = P->numbh;
  }
  (void)Db;
  /* merge touching boxes of a level, :833-896 */
  for (int l = mg + 1; l < levels; l++) {
    int restore = 0;
    for (int i = 0; i < ndl[l]; i++)
      for (int j = 0; j < ndl[l]; j++)
        if (i != j) {
          int ibox = 0, jbox = 0;
          for (int ll = 0; ll < l; ll++) ibox += ndl[ll];
          ibox += i;
          for (int ll = 0; ll < l; ll++) jbox += ndl[ll];
          jbox += j;
          if (dom_touch(&Dv->v[ibox], &Dv->v[jbox])) {
            odom C;
            dom_plus(&C, &Dv->v[ibox], &Dv->v[jbox]);
            Dv->v[ibox] = C;
            dv_erase(Dv, jbox);
            ndl[l]--;
            restore = 1;
          }
        }
    if (restore) l--;
  }
  int g = 0;
  for (int l = 0; l < levels; l++)
    for (int i = 0; i < ndl[l]; i++) Dv->v[g++].level = l;
  free(nx);
  free(dxs);
  *ndl_out = ndl;
  *nlev_out = levels;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* coefficients: src/operator.cc:752-868, 2193-2380; include/elliptic.h      */
/* ------------------------------------------------------------------------ */
static double punctures_c(const orc_problem *P, double X, double Y, double Z)
{
  double cval = 1;
  for (int i = 0; i < P->numbh; i++) {
    double x = X - P->x[i], y = Y - P->y[i], z = Z - P->z[i];
    double r = sqrt(x * x + y * y + z * z);
    if (r < 2 * EPS) r = 2 * EPS;
    cval += 0.5 * P->mp[i] / r;
  }
  return cval;
}

static double punctures_b(const orc_problem *P, double X, double Y, double Z)
{
  double A[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = 0.0;
  for (int i = 0; i < P->numbh; i++) {
    double x = X - P->x[i], y = Y - P->y[i], z = Z - P->z[i];
    double x2 = x * x, y2 = y * y, z2 = z * z;
    double r2 = x2 + y2 + z2;
    if (r2 < 2 * EPS) r2 = 2 * EPS;
    double r = sqrt(r2);
    double ir5 = 1.0 / (r2 * r2 * r);
    const double px = P->px[i], py = P->py[i], pz = P->pz[i];
    const double sx = P->sx[i], sy = P->sy[i], sz = P->sz[i];
    A[0][0] += 1.5 * ir5 * (px * x * (x2 + r2) + py * y * (x2 - r2) + pz * z * (x2 - r2) +
                            4.0 * x * (sy * z - sz * y));
    A[1][1] += 1.5 * ir5 * (px * x * (y2 - r2) + py * y * (y2 + r2) + pz * z * (y2 - r2) +
                            4.0 * y * (sz * x - sx * z));
    A[2][2] += 1.5 * ir5 * (px * x * (z2 - r2) + py * y * (z2 - r2) + pz * z * (z2 + r2) +
                            4.0 * z * (sx * y - sy * x));
    A[0][1] += 1.5 * ir5 * (px * y * (r2 + x2) + py * x * (r2 + y2) + pz * x * y * z -
                            2.0 * sx * x * z + 2.0 * sy * y * z + 2.0 * sz * (x2 - y2));
    A[0][2] += 1.5 * ir5 * (px * z * (r2 + x2) + py * x * y * z + pz * x * (r2 + z2) +
                            2.0 * sx * x * y + 2.0 * sy * (z2 - x2) - 2.0 * sz * y * z);
    A[1][2] += 1.5 * ir5 * (px * x * y * z + py * z * (r2 + y2) + pz * y * (r2 + z2) +
                            2.0 * sx * (y2 - z2) - 2.0 * sy * x * y + 2.0 * sz * x * z);
  }
  A[1][0] = A[0][1];
  A[2][0] = A[0][2];
  A[2][1] = A[1][2];
  double bval = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) bval += A[i][j] * A[i][j];
  return 0.125 * bval;
}

/* scalar-field profiles, include/elliptic.h:1099-1147 */
static double phi_cII(const orc_solver *S, double r)
{
  return S->ps_phi0 * exp(-(r - S->P.ps_r0) * (r - S->P.ps_r0) * S->ps_isigma);
}
static double phi_ground(double x)
{
  double l2 = 0.6;
  return (0.0481646 * exp(-0.0581545 * (x - 1.8039e-08) * (x - 1.8039e-08) / (l2)) +
          0.298408 * exp(-0.111412 * (x + 9.6741e-09) * (x + 9.6741e-09) / l2) +
          0.42755 * exp(-0.207156 * (x - 1.09822e-08) * (x - 1.09822e-08) / l2) +
          0.204229 * exp(-0.37742 * (x + 2.13778e-08) * (x + 2.13778e-08) / l2) +
          0.021649 * exp(-0.68406 * (x - 8.78608e-08) * (x - 8.78608e-08) / l2)) * l2;
}
static double phi_cIV(const orc_solver *S, double r)
{
  return S->ps_phi0 * 0.5 * (tanh((r + S->P.ps_r0) * S->ps_isigma) - tanh((r - S->P.ps_r0) * S->ps_isigma));
}
static double dphi_cI(const orc_solver *S, double r)
{
  return S->ps_d1 / pow(cosh((r - S->P.ps_r0) * S->ps_isigma), 4);
}
static double dphi_cII(const orc_solver *S, double r)
{
  double r0 = S->P.ps_r0;
  return S->ps_de1 * (r - r0) * (r - r0) * exp(-2 * S->ps_isigma * (r - r0) * (r - r0));
}
static double dphi_ground(double x)
{
  double l2 = 10000;
  return M_PI * pow(-2 * (0.0581545 * (x - 1.8039e-08) * 0.0481646 * exp(-0.0581545 * (x - 1.8039e-08) * (x - 1.8039e-08) / (l2)) +
                          0.111412 * (x + 9.6741e-09) * 0.298408 * exp(-0.111412 * (x + 9.6741e-09) * (x + 9.6741e-09) / l2) +
                          0.207156 * (x - 1.09822e-08) * 0.42755 * exp(-0.207156 * (x - 1.09822e-08) * (x - 1.09822e-08) / l2) +
                          0.37742 * (x + 2.13778e-08) * 0.204229 * exp(-0.37742 * (x + 2.13778e-08) * (x + 2.13778e-08) / l2) +
                          0.68406 * (x - 8.78608e-08) * 0.021649 * exp(-0.68406 * (x - 8.78608e-08) * (x - 8.78608e-08) / l2)) /
                        (l2 * l2), 2);
}
static double dphi_cIV(const orc_solver *S, double r)
{
  double r0 = S->P.ps_r0, is = S->ps_isigma;
  return S->ps_de1 * 0.25 * pow(pow(1. / cosh((r + r0) * is), 2) - pow(1. / cosh((r - r0) * is), 2), 2);
}
/* punctures_scalar_d / _e, src/operator.cc:2339-2380 */
static double scalar_d(const orc_solver *S, double X, double Y, double Z)
{
  double r = sqrt(X * X + Y * Y + Z * Z);
  switch (S->P.ps_case) {
  case 1: return dphi_cI(S, r);
  case 2: return dphi_cII(S, r);
  case 3: return dphi_ground(r);
  default: return dphi_cIV(S, r);
  }
}
static double scalar_e(const orc_solver *S, double X, double Y, double Z)
{
  int c = S->P.ps_case;
  if (c == 2 || c == 3 || c == 4) {
    double r = sqrt(X * X + Y * Y + Z * Z);
    double ff = 0;
    if (c == 2) ff = S->ps_e2 * phi_cII(S, r);
    if (c == 3) ff = S->ps_e2 * phi_ground(r);
    if (c == 4) ff = S->ps_e2 * phi_cIV(S, r);
    return S->ps_e1 * (1 - exp(ff)) * (1 - exp(ff)) * exp(-2 * ff);
  }
  return 0.0;
}

/* ------------------------------------------------------------------------ */
/* stencils: include/ffunction.h:1290-1524, src/diff_{2nd,4th,8th}.cc        */
/* ------------------------------------------------------------------------ */
static inline double lap_at(const obox *B, const double *u, int i, int j, int k)
{
  const long sx = 1, sy = B->D.n[0], sz = (long)B->D.n[0] * B->D.n[1];
  const long p = IDX(B, i, j, k);
  const double c = u[p];
  const double ix2 = B->idx2[0], iy2 = B->idx2[1], iz2 = B->idx2[2];
  switch (B->D.order) {
  case 2:
    return ((u[p + sx] - 2.0 * c + u[p - sx]) * ix2 +
            (u[p + sy] - 2.0 * c + u[p - sy]) * iy2 +
            (u[p + sz] - 2.0 * c + u[p - sz]) * iz2);
  case 4:
    return (((-(u[p + 2 * sx] + u[p - 2 * sx]) + 16.0 * (u[p + sx] + u[p - sx]) - 30.0 * c) * ix2 +
             (-(u[p + 2 * sy] + u[p - 2 * sy]) + 16.0 * (u[p + sy] + u[p - sy]) - 30.0 * c) * iy2 +
             (-(u[p + 2 * sz] + u[p - 2 * sz]) + 16.0 * (u[p + sz] + u[p - sz]) - 30.0 * c) * iz2) / 12.0);
  case 6: {
    const double i180 = 1.0 / 180;
    return (2.0 * (u[p + 3 * sx] + u[p - 3 * sx]) -
            27.0 * (u[p + 2 * sx] + u[p - 2 * sx] - 10.0 * (u[p + sx] + u[p - sx])) - 490.0 * c) * ix2 * i180 +
           (2.0 * (u[p + 3 * sy] + u[p - 3 * sy]) -
            27.0 * (u[p + 2 * sy] + u[p - 2 * sy] - 10.0 * (u[p + sy] + u[p - sy])) - 490.0 * c) * iy2 * i180 +
           (2.0 * (u[p + 3 * sz] + u[p - 3 * sz]) -
            27.0 * (u[p + 2 * sz] + u[p - 2 * sz] - 10.0 * (u[p + sz] + u[p - sz])) - 490.0 * c) * iz2 * i180;
  }
  default: /* 8 */
    return ((-9.0 * (u[p + 4 * sx] + u[p - 4 * sx]) + 128.0 * (u[p + 3 * sx] + u[p - 3 * sx]) -
             1008.0 * (u[p + 2 * sx] + u[p - 2 * sx]) + 8064.0 * (u[p + sx] + u[p - sx]) - 14350.0 * c) * ix2 / 5040.0 +
            (-9.0 * (u[p + 4 * sy] + u[p - 4 * sy]) + 128.0 * (u[p + 3 * sy] + u[p - 3 * sy]) -
             1008.0 * (u[p + 2 * sy] + u[p - 2 * sy]) + 8064.0 * (u[p + sy] + u[p - sy]) - 14350.0 * c) * iy2 / 5040.0 +
            (-9.0 * (u[p + 4 * sz] + u[p - 4 * sz]) + 128.0 * (u[p + 3 * sz] + u[p - 3 * sz]) -
             1008.0 * (u[p + 2 * sz] + u[p - 2 * sz]) + 8064.0 * (u[p + sz] + u[p - sz]) - 14350.0 * c) * iz2 / 5040.0);
  }
}

static inline double dulap(const obox *B)
{
  const double s = B->idx2[0] + B->idx2[1] + B->idx2[2];
  switch (B->D.order) {
  case 2: return -2.0 * s;
  case 4: return -2.5 * s;
  case 6: return -490 * s * (1.0 / 180);
  default: return -205 * s / 72.0;
  }
}

/* first derivative along axis a: dx2 (src/diff_2nd.cc:238-295) for order 2,
 * dx4 (src/diff_4th.cc:6-57) for orders 4/6/8 (src/ffunction.cc:197-282) */
static inline double deriv(const obox *B, const double *u, int a, int i, int j, int k)
{
  const int ijk[3] = {i, j, k};
  const long st[3] = {1, B->D.n[0], (long)B->D.n[0] * B->D.n[1]};
  const long s = st[a];
  const int n = B->D.n[a];
  const long p = IDX(B, i, j, k);
  const double id = B->idx[a];
  if (B->D.order == 2) {
    if (ijk[a] == 0) return (-3.0 * u[p] + 4.0 * u[p + s] - u[p + 2 * s]) * 0.5 * id;
    if (ijk[a] == n - 1) return (3.0 * u[p] - 4.0 * u[p - s] + u[p - 2 * s]) * 0.5 * id;
    return (u[p + s] - u[p - s]) * 0.5 * id;
  }
  const int nm = n % 2 == 0 ? n / 2 : (n - 1) / 2;
  if (ijk[a] <= nm)
    return (-(25 * u[p] - 48 * u[p + s] + 36 * u[p + 2 * s] - 16 * u[p + 3 * s] + 3 * u[p + 4 * s]) * id / 12.0);
  return ((25 * u[p] - 48 * u[p - s] + 36 * u[p - 2 * s] - 16 * u[p - 3 * s] + 3 * u[p - 4 * s]) * id / 12.0);
}

static inline double du_deriv(const obox *B, int a, int i, int j, int k)
{
  const int ijk[3] = {i, j, k};
  const int n = B->D.n[a];
  const double id = B->idx[a];
  if (B->D.order == 2) {
    if (ijk[a] == 0) return -3.0 * 0.5 * id;
    if (ijk[a] == n - 1) return 3.0 * 0.5 * id;
    return 0.0;
  }
  const int nm = n % 2 == 0 ? n / 2 : (n - 1) / 2;
  if (ijk[a] <= nm) return -25 * id / 12.0;
  return 25 * id / 12.0;
}

/* The Gaussian test, src/operator.cc:1865-1887: u = a exp(-r^2 / 2) solves
 * Lap u + u^2 = a exp(-r^2) (a + exp(r^2 / 2) (r^2 - 3)), a = 0.004. */
static double gaussian_source(double x, double y, double z)
{
  double r2 = x * x + y * y + z * z;
  double a = 0.004;
  return (a * exp(-r2) * (a + exp(0.5 * r2) * (r2 - 3.0)));
}

static double gaussian(double x, double y, double z)
{
  double r2 = x * x + y * y + z * z;
  double a = 0.004;
  return (a * exp(-0.5 * r2));
}

/* Boundary-test and Multibox-test, src/operator.cc:1772-1857 (the source is
 * of the Laplacian alone, as the reference writes it) */
static int dcomp0(double r) { return fabs(r) <= 3 * DBL_EPSILON; }

static double test_boundary(double x, double y, double z)
{
  double r = sqrt(x * x + y * y + z * z);
  return !dcomp0(r) ? (0.004 * tanh(r) / r) : (0.004);
}

static double test_boundary_source(double x, double y, double z)
{
  double r = sqrt(x * x + y * y + z * z);
  return !dcomp0(r) ? (-2.0 * 0.004 * tanh(r) / (r * cosh(r) * cosh(r))) : (-2.0 * 0.004);
}

static double test_mfunct(const orc_problem *p, double x, double y, double z)
{
  double r2_1 = (x - p->x[0]) * (x - p->x[0]) + y * y + z * z;
  double r2_2 = (x - p->x[1]) * (x - p->x[1]) + y * y + z * z;
  double a = 0.05;
  return (exp(-a * r2_1) + exp(-a * r2_2));
}

static double test_mfunct_source(const orc_problem *p, double x, double y, double z)
{
  double r2_1 = (x - p->x[0]) * (x - p->x[0]) + y * y + z * z;
  double r2_2 = (x - p->x[1]) * (x - p->x[1]) + y * y + z * z;
  double a = 0.05;
  return (2.0 * a * exp(-a * r2_1) * ((2 * a * r2_1 - 3)) + 2.0 * a * exp(-a * r2_2) * ((2 * a * r2_2 - 3)));
}

/* Bowen_York_rho0/1/2 (src/operator.cc:3313-3408): the momentum component
 * `comp` of every puncture within one cell diagonal dr of the point, spread
 * as 3 p / (4 pi dr^3) (a unit-volume ball of radius dr). */
static double by_rho(const orc_problem *p, int comp, double X, double Y, double Z, double dx, double dy, double dz)
{
  double cval = 0;
  for (int i = 0; i < p->numbh; i++) {
    const double x = X - p->x[i], y = Y - p->y[i], z = Z - p->z[i];
    const double r = sqrt(x * x + y * y + z * z);
    const double dr = sqrt(dx * dx + dy * dy + dz * dz);
    const double pc = comp == 0 ? p->px[i] : comp == 1 ? p->py[i] : p->pz[i];
    if (r <= dr) cval += 3 * pc / (4 * M_PI * dr * dr * dr);
  }
  return cval;
}

/* ------------------------------------------------------------------------ */
/* pointwise operator: include/elliptic.h:405-445                            */
/* ------------------------------------------------------------------------ */
static inline double op_at(const orc_solver *S, const obox *B, long p, double lap)
{
  const double *u = B->f[F_U], *b = B->f[F_B], *c = B->f[F_C];
  if (S->P.equation == 5) return lap;                 /* BowenYork_OP_X/Y/Z, include/elliptic.h:772-793 */
  if (S->P.equation >= 2) return lap + u[p] * u[p];   /* poisson_OP, include/elliptic.h:359-362 */
  if (S->P.equation == 0) return lap + b[p] / pow(c[p] + u[p], 7);
  const double *d = B->f[F_D], *e = B->f[F_E];
  return lap + b[p] / pow(c[p] + u[p], 7) + d[p] * (c[p] + u[p]) + e[p] * pow(c[p] + u[p], 5);
}

static inline double duop_at(const orc_solver *S, const obox *B, long p, double dl)
{
  const double *u = B->f[F_U], *b = B->f[F_B], *c = B->f[F_C];
  if (S->P.equation == 5) return dl;                /* BowenYork_duOP_* */
  if (S->P.equation >= 2) return dl + 2.0 * u[p];   /* poisson_duOP */
  if (S->P.equation == 0) return dl - 7.0 * b[p] / pow(c[p] + u[p], 8);
  const double *d = B->f[F_D], *e = B->f[F_E];
  return dl - 7.0 * b[p] / pow(c[p] + u[p], 8) + d[p] + 5 * e[p] * pow(c[p] + u[p], 4);
}

/* elliptic::Smooth, src/elliptic.cc:1126-1242: lexicographic nonlinear
 * Gauss-Seidel-Newton over INSIDE points; returns the max over the nu sweeps
 * of the L-infinity norm of the pre-update point residuals. */
static double smooth_box_w(orc_solver *S, obox *B, int nu, double omega);
static double smooth_box(orc_solver *S, obox *B, int nu) { return smooth_box_w(S, B, nu, 1.0); }
static double smooth_box_w(orc_solver *S, obox *B, int nu, double omega)
{
  double gLinf = 0;
  const int b = B->D.buf;
  const int nx = B->D.n[0], ny = B->D.n[1], nz = B->D.n[2];
  double *u = B->f[F_U], *R = B->f[F_R];
  const double *rho = B->f[F_RHO];
  const double dl = dulap(B);
  /* multicolor: bit 0 = multigrid levels above the coarsest (Robin boxes),
   * bit 1 = coarsest solve, bit 2 = refinement levels */
  const int lv = B->D.level;
  const int mc = lv == 0 ? (S->multicolor >> 1) & 1
                         : (lv <= S->mgrid_levels ? S->multicolor & 1 : (S->multicolor >> 2) & 1);
  const int NC = mc ? b + 1 : 1;
  for (int kk = 0; kk < nu; kk++) {
    double Linf = 0;
    for (int color = 0; color < NC; color++)
    for (int k = b; k < nz - b; k++)
      for (int j = b; j < ny - b; j++)
        for (int i = b; i < nx - b; i++) {
          if (NC > 1 && (i + j + k) % NC != color) continue;
          long p = IDX(B, i, j, k);
          double r = op_at(S, B, p, lap_at(B, u, i, j, k)) - rho[p];
          R[p] = r;
          double dr = duop_at(S, B, p, dl);
          u[p] = omega == 1.0 ? u[p] - R[p] / dr : u[p] - omega * (R[p] / dr);
          double f = fabs(R[p]);
          if (Linf < f) Linf = f;
          if (!(u[p] == u[p])) S->nan_flag = 1;
        }
    gLinf = Linf > gLinf ? Linf : gLinf;
  }
  return gLinf;
}

/* ------------------------------------------------------------------------ */
/* Robin boundary: src/boundary.cc:447-800, 915-1101 (update) and           */
/* 1118-1535, 1544-1710 (operator value into R)                              */
/* ------------------------------------------------------------------------ */
/* One Robin point.  mask selects the derivative axes: one bit on a face
 * (Boundary_Face: F = r2*ipn*Dx/x + u - S), two on an edge and three on a
 * corner (Boundary_Edge/Corner: F = r2*ipn*(Dx/x + Dy/y [+ Dz/z]) + u - S),
 * with each expression grouped as in src/boundary.cc:947-950, 1011-1016,
 * 1079-1086.  Returns the term without u and S; *dF gets dF/du. */
static inline double robin_F(const orc_solver *S, const obox *B, const double *u, int mask, int i, int j, int k,
                             double *dF)
{
  const double x = dom_coord(&B->D, 0, i), y = dom_coord(&B->D, 1, j), z = dom_coord(&B->D, 2, k);
  const double x2 = x * x, y2 = y * y, z2 = z * z;
  const double r2 = x2 + y2 + z2;
  /* falloff n = 1 (src/operator.cc:789), 2 for Bowen-York's variables (1393-1399) */
  const double ipn = 1.0 / (double)(S->P.equation == 5 ? 2 : 1);
  const double crd[3] = {x, y, z};
  int ax[3], na = 0;
  for (int a = 0; a < 3; a++)
    if (mask & (1 << a)) ax[na++] = a;
  if (na == 1) {
    *dF = r2 * ipn * du_deriv(B, ax[0], i, j, k) / crd[ax[0]] + 1.0;
    return r2 * ipn * deriv(B, u, ax[0], i, j, k) / crd[ax[0]];
  }
  double t = deriv(B, u, ax[0], i, j, k) / crd[ax[0]] + deriv(B, u, ax[1], i, j, k) / crd[ax[1]];
  double dt = du_deriv(B, ax[0], i, j, k) / crd[ax[0]] + du_deriv(B, ax[1], i, j, k) / crd[ax[1]];
  if (na == 3) {
    t = t + deriv(B, u, ax[2], i, j, k) / crd[ax[2]];
    dt = dt + du_deriv(B, ax[2], i, j, k) / crd[ax[2]];
  }
  *dF = r2 * ipn * dt + 1.0;
  return r2 * ipn * t;
}

typedef void (*robin_pt_fn)(orc_solver *, obox *, int mask, int i, int j, int k);

static void robin_update_pt(orc_solver *S, obox *B, int mask, int i, int j, int k)
{
  double *u = B->f[F_U];
  const double *rho = B->f[F_RHO];
  long p = IDX(B, i, j, k);
  if (S->P.boundary == 1) {   /* Dirichlet: u = S on the BOUNDARY points, src/boundary.cc:800-812 */
    u[p] = rho[p];
    return;
  }
  double dF;
  double t = robin_F(S, B, u, mask, i, j, k, &dF);
  double F = t + u[p] - rho[p];
  u[p] = u[p] - F / dF;
}

static void robin_operator_pt(orc_solver *S, obox *B, int mask, int i, int j, int k)
{
  const double *u = B->f[F_U];
  long p = IDX(B, i, j, k);
  if (S->P.boundary == 1) {   /* Dirichlet: R = u on the BOUNDARY points, src/boundary.cc:1481-1490 */
    B->f[F_R][p] = u[p];
    return;
  }
  double dF;
  double t = robin_F(S, B, u, mask, i, j, k, &dF);
  B->f[F_R][p] = t + u[p];
}

/* Layer index lists for the ghost band of an axis: the low side walks
 * b-1 .. 0 and the high side n-b .. n-1, i.e. inner to outer
 * (src/domain.cc:614-1352). */
static int side_layers(int n, int b, int hi, int *out)
{
  for (int t = 0; t < b; t++) out[t] = hi ? n - b + t : b - 1 - t;
  return b;
}

/* Faces -> edges -> corners in App_Bound's order. */
static void robin_walk(orc_solver *S, obox *B, robin_pt_fn fn)
{
  const int b = B->D.buf;
  const int n[3] = {B->D.n[0], B->D.n[1], B->D.n[2]};
  int L0[8], L1[8], L2[8];
  /* faces Xi, Xf, Yi, Yf, Zi, Zf */
  for (int a = 0; a < 3; a++)
    for (int hi = 0; hi < 2; hi++) {
      side_layers(n[a], b, hi, L0);
      const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
      for (int t = 0; t < b; t++)
        for (int q = b; q < n[a2] - b; q++)
          for (int r = b; r < n[a1] - b; r++) {
            int ijk[3];
            ijk[a] = L0[t]; ijk[a1] = r; ijk[a2] = q;
            fn(S, B, 1 << a, ijk[0], ijk[1], ijk[2]);
          }
    }
  /* edges: XY (4), XZ (4), YZ (4); inner-to-outer in both ghost axes */
  const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int pi = 0; pi < 3; pi++) {
    const int a = pairs[pi][0], c = pairs[pi][1];
    const int free_ax = 3 - a - c;
    for (int ha = 0; ha < 2; ha++)
      for (int hc = 0; hc < 2; hc++) {
        side_layers(n[a], b, ha, L0);
        side_layers(n[c], b, hc, L1);
        for (int ta = 0; ta < b; ta++)
          for (int tc = 0; tc < b; tc++)
            for (int q = b; q < n[free_ax] - b; q++) {
              int ijk[3];
              ijk[a] = L0[ta]; ijk[c] = L1[tc]; ijk[free_ax] = q;
              fn(S, B, (1 << a) | (1 << c), ijk[0], ijk[1], ijk[2]);
            }
      }
  }
  /* corners XiYiZi, XiYiZf, XfYiZi, XfYiZf, XiYfZi, XiYfZf, XfYfZi, XfYfZf */
  for (int hy = 0; hy < 2; hy++)
    for (int hx = 0; hx < 2; hx++)
      for (int hz = 0; hz < 2; hz++) {
        side_layers(n[0], b, hx, L0);
        side_layers(n[1], b, hy, L1);
        side_layers(n[2], b, hz, L2);
        for (int tk = 0; tk < b; tk++)
          for (int tj = 0; tj < b; tj++)
            for (int ti = 0; ti < b; ti++)
              fn(S, B, 7, L0[ti], L1[tj], L2[tk]);
      }
}

/* ------------------------------------------------------------------------ */
/* interpolation: src/interpolation.cc:124-375                               */
/* ------------------------------------------------------------------------ */
static double lagrange_poly(const odom *D, int a, double t, int i, int ni, int nf)
{
  double lp = 1.0;
  const double ti = dom_coord(D, a, i);
  for (int j = ni; j < i; j++) lp *= (t - dom_coord(D, a, j)) / (ti - dom_coord(D, a, j));
  for (int j = i + 1; j <= nf; j++) lp *= (t - dom_coord(D, a, j)) / (ti - dom_coord(D, a, j));
  return lp;
}

static double interp_lagrange(const obox *B, const double *f, int ord, double x, double y, double z)
{
  const odom *D = &B->D;
  int i = dom_locate(D, 0, x), j = dom_locate(D, 1, y), k = dom_locate(D, 2, z);
  if (dcomp(x, dom_coord(D, 0, i)) && dcomp(y, dom_coord(D, 1, j)) && dcomp(z, dom_coord(D, 2, k)))
    return f[IDX(B, i, j, k)];
  int st[3];
  const int c3[3] = {i, j, k};
  for (int a = 0; a < 3; a++) {
    int s = ord % 2 == 0 ? c3[a] - ord / 2 : c3[a] - (ord + 1) / 2;
    if (s < 0) s = 0;
    else if (s + ord >= D->n[a]) s = D->n[a] - ord - 1;
    st[a] = s;
  }
  double uk[16][16];
  for (int I = 0; I <= ord; I++)
    for (int J = 0; J <= ord; J++) {
      uk[I][J] = 0;
      for (int K = 0; K <= ord; K++)
        uk[I][J] += f[IDX(B, st[0] + I, st[1] + J, st[2] + K)] *
                    lagrange_poly(D, 2, z, st[2] + K, st[2], st[2] + ord);
    }
  double ujk[16];
  for (int I = 0; I <= ord; I++) {
    ujk[I] = 0;
    for (int J = 0; J <= ord; J++)
      ujk[I] += uk[I][J] * lagrange_poly(D, 1, y, st[1] + J, st[1], st[1] + ord);
  }
  double fxyz = 0;
  for (int I = 0; I <= ord; I++) fxyz += ujk[I] * lagrange_poly(D, 0, x, st[0] + I, st[0], st[0] + ord);
  return fxyz;
}

static double interp_linear(const obox *B, const double *f, double x, double y, double z)
{
  const odom *D = &B->D;
  int i = dom_locate(D, 0, x), j = dom_locate(D, 1, y), k = dom_locate(D, 2, z);
  if (dcomp(x, dom_coord(D, 0, i)) && dcomp(y, dom_coord(D, 1, j)) && dcomp(z, dom_coord(D, 2, k)))
    return f[IDX(B, i, j, k)];
  i = i == 0 ? 1 : i;
  j = j == 0 ? 1 : j;
  k = k == 0 ? 1 : k;
  double dxf = (x - dom_coord(D, 0, i - 1)) * B->idx[0];
  double dyf = (y - dom_coord(D, 1, j - 1)) * B->idx[1];
  double dzf = (z - dom_coord(D, 2, k - 1)) * B->idx[2];
  double dxi = (1 - dxf), dyi = (1 - dyf), dzi = (1 - dzf);
#define V(a, b, c) f[IDX(B, a, b, c)]
  return (((V(i - 1, j - 1, k - 1) * dxi + V(i, j - 1, k - 1) * dxf) * dyi +
           (V(i - 1, j, k - 1) * dxi + V(i, j, k - 1) * dxf) * dyf) * dzi +
          ((V(i - 1, j - 1, k) * dxi + V(i, j - 1, k) * dxf) * dyi +
           (V(i - 1, j, k) * dxi + V(i, j, k) * dxf) * dyf) * dzf);
#undef V
}

/* ------------------------------------------------------------------------ */
/* transfers: ffunction::Transferir (src/ffunction.cc:2435-2478),            */
/* multigrid::Transferir (src/multigrid.cc:121-141), Set_In (2807-2849)      */
/* ------------------------------------------------------------------------ */
enum { IT_ALL, IT_INSIDE, IT_BOUNDARY };
enum { M_LINEAR, M_LAGRANGE };

static inline int in_iter(const obox *B, int it, int i, int j, int k)
{
  if (it == IT_ALL) return 1;
  const int b = B->D.buf;
  int inside = i >= b && i < B->D.n[0] - b && j >= b && j < B->D.n[1] - b && k >= b && k < B->D.n[2] - b;
  return it == IT_INSIDE ? inside : !inside;
}

static void transfer_box(obox *T, int tf, const obox *Sb, int sf, int it, int method, int ord, int all, int to_zero)
{
  double *dst = T->f[tf];
  const double *src = Sb->f[sf];
  for (int k = 0; k < T->D.n[2]; k++)
    for (int j = 0; j < T->D.n[1]; j++)
      for (int i = 0; i < T->D.n[0]; i++) {
        if (!in_iter(T, it, i, j, k)) continue;
        double x = dom_coord(&T->D, 0, i), y = dom_coord(&T->D, 1, j), z = dom_coord(&T->D, 2, k);
        long p = IDX(T, i, j, k);
        if (dom_is_in_nb(&Sb->D, x, y, z) || (all && dom_is_in(&Sb->D, x, y, z)))
          dst[p] = method == M_LAGRANGE ? interp_lagrange(Sb, src, ord, x, y, z) : interp_linear(Sb, src, x, y, z);
        else if (to_zero)
          dst[p] = 0.0;
      }
}

static void transferir(orc_solver *S, int from, int ff, int to, int tf, int it, int method, int ord, int all, int to_zero)
{
  from = from < S->levels ? from : S->levels - 1;
  to = to < S->levels ? to : S->levels - 1;
  for (int ib = 0; ib < S->ndl[from]; ib++)
    for (int jb = 0; jb < S->ndl[to]; jb++)
      transfer_box(&S->box[S->first[to] + jb], tf, &S->box[S->first[from] + ib], ff, it, method, ord, all, to_zero);
}

static void set_in(obox *Sb, const obox *Wb, const odom *Dom)
{
  double *s = Sb->f[F_RHO];
  const double *w = Wb->f[F_W];
  for (int k = 0; k < Sb->D.n[2]; k++)
    for (int j = 0; j < Sb->D.n[1]; j++)
      for (int i = 0; i < Sb->D.n[0]; i++) {
        double x = dom_coord(&Sb->D, 0, i), y = dom_coord(&Sb->D, 1, j), z = dom_coord(&Sb->D, 2, k);
        if (dom_is_in_nb(&Wb->D, x, y, z) && dom_is_in_nb(Dom, x, y, z))
          s[IDX(Sb, i, j, k)] = interp_linear(Wb, w, x, y, z);
      }
}

/* elliptic::App_Ell_Operator, src/elliptic.cc:943-991 */
static void app_ell_operator(orc_solver *S, obox *B)
{
  const int b = B->D.buf;
  const int nx = B->D.n[0], ny = B->D.n[1], nz = B->D.n[2];
  for (int k = b; k < nz - b; k++)
    for (int j = b; j < ny - b; j++)
      for (int i = b; i < nx - b; i++) {
        long p = IDX(B, i, j, k);
        B->f[F_R][p] = op_at(S, B, p, lap_at(B, B->f[F_U], i, j, k));
      }
}

/* elliptic::Compute_ADM_Mass, puncture part, src/elliptic.cc:2447-2469 */
static void compute_adm(orc_solver *S)
{
  const orc_problem *P = &S->P;
  const int top = S->levels - 1;
  for (int i = 0; i < P->numbh; i++) {
    int bi = S->first[top] + (i < S->ndl[top] ? i : 0);   /* Get_dom_index */
    const obox *B = &S->box[bi];
    double bhmj = 0;
    for (int j = 0; j < P->numbh; j++)
      if (j != i)
        bhmj += 0.5 * P->mp[j] / sqrt((P->x[i] - P->x[j]) * (P->x[i] - P->x[j]) +
                                      (P->y[i] - P->y[j]) * (P->y[i] - P->y[j]) +
                                      (P->z[i] - P->z[j]) * (P->z[i] - P->z[j]));
    S->adm[i] = P->mp[i] * (1 + bhmj + interp_lagrange(B, B->f[F_U], 4, P->x[i], P->y[i], P->z[i]));
  }
}

static void axpy_all(obox *B, int dst, int a, double sa, int b)   /* dst = a + sa*b over ALL points */
{
  for (long p = 0; p < B->npts; p++) B->f[dst][p] = B->f[a][p] + sa * B->f[b][p];
}

/* Checker option: replace W on the INSIDE points of a box by its
 * (1,2,1)^3/64 average, where a neighbour outside INSIDE contributes the
 * centre value.  W vanishes at the fixed point, so this changes the path of
 * the iteration, not its fixed point. */
static void full_weight_w(obox *B)
{
  const int b = B->D.buf, nx = B->D.n[0], ny = B->D.n[1], nz = B->D.n[2];
  double *w = B->f[F_W];
  double *t = (double *)malloc(sizeof(double) * B->npts);
  memcpy(t, w, sizeof(double) * B->npts);
  for (int k = b; k < nz - b; k++)
    for (int j = b; j < ny - b; j++)
      for (int i = b; i < nx - b; i++) {
        const double c = t[IDX(B, i, j, k)];
        double acc = 0;
        for (int dk = -1; dk <= 1; dk++)
          for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++) {
              const int ii = i + di, jj = j + dj, kk = k + dk;
              const double wt = (double)((2 - di * di) * (2 - dj * dj) * (2 - dk * dk)) / 64.0;
              const int in = ii >= b && ii < nx - b && jj >= b && jj < ny - b && kk >= b && kk < nz - b;
              acc += wt * (in ? t[IDX(B, ii, jj, kk)] : c);
            }
        w[IDX(B, i, j, k)] = acc;
      }
  free(t);
}

/* elliptic::FASN, src/elliptic.cc:1468-1968.  With wcycle the level repeats
 * its body (and so every coarser level its own loop) while its
 * post-smoothing norm is above eps_solv (1956); `cycle` counts the
 * iterations from the caller's count and is what Print_Pre_Cycle /
 * Print_Post_Cycle print (1499, 1535, 1818, 1936, 1948). */
static double fasn(orc_solver *S, int k, int k_top, int wcycle, long icycle)
{
  const int mg = S->mgrid_levels;
  const int order = S->P.order;
  double norm_k = 0, norm_km1 = 0;
  obox *Bk = &S->box[S->first[k]];
  obox *Bc = &S->box[S->first[k - 1]];
  const int nk = S->ndl[k], nc = S->ndl[k - 1];
  long cycle = icycle, iters = 0;

  do {
    norm_k = 0;
    for (int i = 0; i < nk; i++) {                                  /* 1518-1533 */
      if (k <= mg) robin_walk(S, &Bk[i], robin_update_pt);
      double n = smooth_box(S, &Bk[i], S->P.nu1);
      norm_k = n > norm_k ? n : norm_k;
    }
    if (k < 64) S->lnorm[k][0] = norm_k;
    log_event(S, k, 0, cycle, norm_k);                              /* 1535 */
    transferir(S, k, F_U, k - 1, F_U, IT_INSIDE, M_LAGRANGE, 3, 0, 0);   /* 1543-1546 */
    for (int j = 0; j < nc; j++) {                                  /* 1582-1594 */
      app_ell_operator(S, &Bc[j]);
      if (k <= mg) robin_walk(S, &Bc[j], robin_operator_pt);
    }
    for (int i = 0; i < nk; i++) {                                  /* 1603-1614 */
      app_ell_operator(S, &Bk[i]);
      if (k <= mg) robin_walk(S, &Bk[i], robin_operator_pt);
    }
    for (int i = 0; i < nk; i++)                                    /* 1625-1649 */
      for (long p = 0; p < Bk[i].npts; p++) Bk[i].f[F_W][p] = Bk[i].f[F_RHO][p] - Bk[i].f[F_R][p];
    if (S->wsmooth)
      for (int i = 0; i < nk; i++) full_weight_w(&Bk[i]);
    if (k - 1 <= mg)                                                /* 1660-1676 */
      transferir(S, k, F_W, k - 1, F_W, IT_ALL, M_LAGRANGE, 2, 1, 0);
    else
      transferir(S, k, F_W, k - 1, F_W, IT_ALL, M_LAGRANGE, 2, 0, 0);
    for (int j = 0; j < nc; j++) {                                  /* 1692-1747 */
      if (k <= mg)
        axpy_all(&Bc[j], F_RHO, F_W, 1.0, F_R);
      else {
        for (long p = 0; p < Bc[j].npts; p++) Bc[j].f[F_W][p] = Bc[j].f[F_W][p] + Bc[j].f[F_R][p];
        for (int i = 0; i < nk; i++) set_in(&Bc[j], &Bc[j], &Bk[i].D);
      }
    }
    for (int j = 0; j < nc; j++)                                    /* 1756-1775 */
      memcpy(Bc[j].f[F_WW], Bc[j].f[F_U], sizeof(double) * Bc[j].npts);
    if (k == 1) {                                                   /* 1782-1816 */
      for (int j = 0; j < nc; j++) {
        double norm_prev;
        norm_km1 = 1;
        long guard = 0;
        double first = -1.0;
        do {
          norm_prev = norm_km1;
          robin_walk(S, &Bc[j], robin_update_pt);
          norm_km1 = smooth_box_w(S, &Bc[j], 1, S->coarse_omega);
          if (first < 0) first = norm_km1;
          ++guard;
          if (S->nan_flag) break;
          if (S->coarse_rtol > 0 && norm_km1 <= S->coarse_rtol * first) break;
        } while (norm_km1 > S->eps_coarse && norm_prev != norm_km1 && guard < S->coarse_cap);
        S->coarse_iters = guard;
        S->coarse_norm = norm_km1;
      }
      log_event(S, 0, 0, cycle, norm_km1);                          /* 1818 */
    } else {
      norm_km1 = fasn(S, k - 1, k_top, wcycle, cycle);
    }
    (void)norm_km1;
    for (int j = 0; j < nc; j++) axpy_all(&Bc[j], F_V, F_U, -1.0, F_WW);   /* 1827-1850 */
    if (k <= mg)                                                    /* 1857-1885 */
      transferir(S, k - 1, F_V, k, F_V, IT_ALL, M_LINEAR, 3, 1, 1);
    else
      transferir(S, k - 1, F_V, k, F_V, IT_INSIDE, M_LINEAR, order + 1, 1, 0);
    for (int i = 0; i < nk; i++)                                    /* 1890-1903 */
      for (long p = 0; p < Bk[i].npts; p++) Bk[i].f[F_U][p] = Bk[i].f[F_U][p] + Bk[i].f[F_V][p];
    if (k > mg)                                                     /* 1905-1908 */
      transferir(S, k - 1, F_U, k, F_U, IT_BOUNDARY, M_LAGRANGE, order + 1, 1, 0);
    norm_k = 0;                                                     /* 1917-1932 */
    for (int i = 0; i < nk; i++) {
      if (k <= mg) robin_walk(S, &Bk[i], robin_update_pt);
      double n = smooth_box(S, &Bk[i], S->P.nu2);
      norm_k = n > norm_k ? n : norm_k;
    }
    if (k < 64) S->lnorm[k][1] = norm_k;
    log_event(S, k, 1, cycle, norm_k);                              /* 1936 */
    if (k == k_top) compute_adm(S);                                 /* 1939-1941 */
    cycle++;
    iters++;
  } while (wcycle && norm_k > S->eps_solv && !S->nan_flag && iters < S->w_cap);   /* 1956 */
  return norm_k;
}

/* Dx V1 + Dy V2 + Dz V3 into lambda's source on INSIDE points: the
 * reference's BowenYork_OP_L (include/elliptic.h:796-800) takes the
 * derivatives with the order's first-derivative stencil (dx2, or dx4 for
 * orders 4-8: src/ffunction.cc:197-282) and sums them in this order. */
void orc_set_divergence_source(orc_solver *lam, const orc_solver *v1, const orc_solver *v2, const orc_solver *v3)
{
  const orc_solver *V[3] = {v1, v2, v3};
  for (int g = 0; g < lam->nboxes; g++) {
    obox *B = &lam->box[g];
    const int b = B->D.buf;
    for (int k = b; k < B->D.n[2] - b; k++)
      for (int j = b; j < B->D.n[1] - b; j++)
        for (int i = b; i < B->D.n[0] - b; i++) {
          double d[3];
          for (int a = 0; a < 3; a++) d[a] = deriv(&V[a]->box[g], V[a]->box[g].f[F_U], a, i, j, k);
          B->f[F_RHO][IDX(B, i, j, k)] = d[0] + d[1] + d[2];
        }
  }
}

/* ------------------------------------------------------------------------ */
/* public API                                                                */
/* ------------------------------------------------------------------------ */
void orc_problem_defaults(orc_problem *p)
{
  memset(p, 0, sizeof(*p));
  p->numbh = 1;
  p->mp[0] = 1.0;          /* bhmp default is set by the caller */
  p->n = 30;
  p->L = 2.0;
  p->order = 4;
  p->levels = 1;
  p->nu1 = 3;
  p->nu2 = 3;
  p->tol = 1e-8;
  p->ps_case = 1;
  p->ps_phi0 = 0.025;
  p->ps_r0 = 120;
  p->ps_sigma = 8;
  p->ps_a2 = 1;
}

static orc_solver *orc_create_opt(const orc_problem *p, int extra_coarse);
orc_solver *orc_create(const orc_problem *p) { return orc_create_opt(p, 0); }
orc_solver *orc_create_extra_coarse(const orc_problem *p) { return orc_create_opt(p, 1); }
static orc_solver *orc_create_opt(const orc_problem *p, int extra_coarse)
{
  if (p->numbh < 1 || p->numbh > ORC_MAX_BH) return NULL;
  if (!(p->order == 2 || p->order == 4 || p->order == 6 || p->order == 8)) return NULL;
  orc_solver *S = (orc_solver *)calloc(1, sizeof(orc_solver));
  S->P = *p;
  S->extra_coarse = extra_coarse;
  S->eps_coarse = 2 * EPS;                          /* src/elliptic.cc:62 */
  S->coarse_cap = 1000000000L;
  S->w_cap = 1000000000L;
  S->coarse_omega = 1.0;
  S->eps_solv = p->tol < S->eps_coarse ? S->eps_coarse : p->tol;
  S->ps_isigma = 1 / p->ps_sigma;                   /* src/elliptic.cc:71-81 */
  double a2 = p->ps_a2;
  S->ps_phi0 = (a2 * a2 / (1 + a2 * a2)) * p->ps_phi0;
  S->ps_d1 = M_PI * S->ps_phi0 * S->ps_phi0 * S->ps_isigma * S->ps_isigma;
  S->ps_e1 = 1 / (16 * p->ps_a2);
  S->ps_e2 = 4 * sqrt(M_PI / 3);
  S->ps_de1 = 4 * M_PI * S->ps_phi0 * S->ps_phi0 * S->ps_isigma * S->ps_isigma;

  domvec Dv = {0, 0, 0};
  int *ndl = NULL, nlev = 0;
  if (set_grids(S, &Dv, &ndl, &nlev) != 0) { free(Dv.v); free(S); return NULL; }
  S->levels = nlev;
  S->ndl = ndl;
  S->first = (int *)calloc(nlev, sizeof(int));
  for (int l = 1; l < nlev; l++) S->first[l] = S->first[l - 1] + ndl[l - 1];
  S->nboxes = Dv.n;
  S->box = (obox *)calloc(Dv.n, sizeof(obox));
  for (int g = 0; g < Dv.n; g++) {
    obox *B = &S->box[g];
    B->D = Dv.v[g];
    B->npts = (long)B->D.n[0] * B->D.n[1] * B->D.n[2];
    for (int f = 0; f < F_NUM; f++) B->f[f] = (double *)calloc(B->npts, sizeof(double));
    for (int a = 0; a < 3; a++) {
      B->idx[a] = 1.0 / B->D.d[a];
      B->idx2[a] = B->idx[a] * B->idx[a];
    }
    /* Set_Coefficients, src/operator.cc:752-868; rho0 = 0 (test_ps returns 0) */
    for (int k = 0; k < B->D.n[2]; k++)
      for (int j = 0; j < B->D.n[1]; j++)
        for (int i = 0; i < B->D.n[0]; i++) {
          double x = dom_coord(&B->D, 0, i), y = dom_coord(&B->D, 1, j), z = dom_coord(&B->D, 2, k);
          long q = IDX(B, i, j, k);
          if (p->equation >= 2) {
            /* the test equations (src/operator.cc:640-673, 1145-1175): rho0
             * = the source on every point, then the boundary value on the
             * BOUNDARY points (Set_Boundary, src/boundary.cc:8-78: Robin's
             * coefficient 0, or Dirichlet's boundary function), and u = the
             * boundary function on every point as the initial guess */
            const int bb = B->D.buf;
            const int ghost = i < bb || j < bb || k < bb || i >= B->D.n[0] - bb || j >= B->D.n[1] - bb ||
                              k >= B->D.n[2] - bb;
            double g, src;
            if (p->equation == 5) {   /* zero boundary function (src/operator.cc:1380-1386) */
              g = 0.0;
              src = p->by_var < 3 ? by_rho(p, p->by_var, x, y, z, B->D.d[0], B->D.d[1], B->D.d[2]) : 0.0;
            } else if (p->equation == 3) {
              g = test_boundary(x, y, z);
              src = test_boundary_source(x, y, z);
            } else if (p->equation == 4) {
              g = test_mfunct(p, x, y, z);
              src = test_mfunct_source(p, x, y, z);
            } else {
              g = gaussian(x, y, z);
              src = gaussian_source(x, y, z);
            }
            B->f[F_RHO][q] = ghost ? (p->boundary == 1 ? g : 0.0) : src;
            B->f[F_U][q] = g;
            continue;
          }
          B->f[F_B][q] = punctures_b(p, x, y, z);
          B->f[F_C][q] = punctures_c(p, x, y, z);
          if (p->equation == 1) {
            B->f[F_D][q] = scalar_d(S, x, y, z);
            B->f[F_E][q] = scalar_e(S, x, y, z);
          }
        }
  }
  free(Dv.v);
  return S;
}

/* elliptic::ApproximateID, src/elliptic.cc:1977-2226: u on every point of
 * every box := the sum over the punctures of the perturbative spin,
 * momentum and cross terms, in the reference's operation order. */
static double approx_u(const orc_problem *p, double x, double y, double z)
{
  double u = 0.0;
  for (int i = 0; i < p->numbh && p->mp[i] != 0.0; i++) {
    double sbl = sqrt(p->sx[i] * p->sx[i] + p->sy[i] * p->sy[i] + p->sz[i] * p->sz[i]);
    double imass = 1.0 / p->mp[i];
    double imass2 = imass * imass;
    double Jx = 4.0 * p->sx[i] * imass2, Jy = 4.0 * p->sy[i] * imass2, Jz = 4.0 * p->sz[i] * imass2;
    double J2 = Jx * Jx + Jy * Jy + Jz * Jz;
    double pbl = sqrt(p->px[i] * p->px[i] + p->py[i] * p->py[i] + p->pz[i] * p->pz[i]);
    double Px = 2.0 * p->px[i] * imass, Py = 2.0 * p->py[i] * imass, Pz = 2.0 * p->pz[i] * imass;
    double P2 = Px * Px + Py * Py + Pz * Pz;
    double xi = x - p->x[i], yi = y - p->y[i], zi = z - p->z[i];
    double r = sqrt(xi * xi + yi * yi + zi * zi);
    if (fabs(r) <= 0.00000000001) r = 0.0000000001;
    double Rx = 2.0 * xi * imass, Ry = 2.0 * yi * imass, Rz = 2.0 * zi * imass;
    double R = 2.0 * r * imass;
    double l1 = 1.0 / (1.0 + R), l2 = l1 * l1, l3 = l2 * l1, l4 = l3 * l1, l5 = l4 * l1;
    double u0j = 0.025 * (l1 + l2 + l3 - 4.0 * l4 + 2.0 * l5);
    double u2j = -0.05 * l5;
    double muj = (sbl != 0.0 && r != 0.0) ? (p->sx[i] * xi + p->sy[i] * yi + p->sz[i] * zi) / (r * sbl) : 0.0;
    double PL2j = 0.5 * (3.0 * muj * muj - 1.0);
    double uj = J2 * (u0j + u2j * R * R * PL2j);
    double u0p = 0.15625 * (l1 - 2.0 * l2 + 2.0 * l3 - l4 + 0.2 * l5);
    double u2p = 0.0125 * (15.0 * l1 + 132.0 * l2 + 53.0 * l3 + 96.0 * l4 + 82 * l5 + 84.0 * (l5 + log(l1) / R) / R) / R;
    double mup = (pbl != 0.0 && r != 0.0) ? (p->px[i] * xi + p->py[i] * yi + p->pz[i] * zi) / (r * pbl) : 0.0;
    double PL2p = 0.5 * (3.0 * mup * mup - 1.0);
    double up = P2 * (u0p + u2p * PL2p);
    double X0 = Py * Jz - Pz * Jy, X1 = Pz * Jx - Px * Jz, X2 = Px * Jy - Py * Jx;
    double uc = 0.0125 * (X0 * Rx + X1 * Ry + X2 * Rz) * (1.0 + 5.0 * R + 10.0 * R * R) * l5;
    u += uj + up + uc;
  }
  return u;
}

void orc_approximate_id(orc_solver *S)
{
  for (int g = 0; g < S->nboxes; g++) {
    obox *B = &S->box[g];
    for (int k = 0; k < B->D.n[2]; k++)
      for (int j = 0; j < B->D.n[1]; j++)
        for (int i = 0; i < B->D.n[0]; i++)
          B->f[F_U][IDX(B, i, j, k)] =
              approx_u(&S->P, dom_coord(&B->D, 0, i), dom_coord(&B->D, 1, j), dom_coord(&B->D, 2, k));
  }
}

void orc_destroy(orc_solver *S)
{
  if (!S) return;
  for (int g = 0; g < S->nboxes; g++)
    for (int f = 0; f < F_NUM; f++) free(S->box[g].f[f]);
  free(S->box);
  free(S->ndl);
  free(S->first);
  free(S->ev);
  free(S);
}

int orc_num_boxes(const orc_solver *S) { return S->nboxes; }
int orc_num_levels(const orc_solver *S) { return S->levels; }
int orc_mgrid_levels(const orc_solver *S) { return S->mgrid_levels; }

void orc_box(const orc_solver *S, int g, orc_box_info *o)
{
  const odom *D = &S->box[g].D;
  o->level = D->level;
  o->nx = D->n[0]; o->ny = D->n[1]; o->nz = D->n[2];
  o->buf = D->buf; o->order = D->order;
  o->xi = D->lo[0]; o->yi = D->lo[1]; o->zi = D->lo[2];
  o->xf = D->hi[0]; o->yf = D->hi[1]; o->zf = D->hi[2];
  o->dx = D->d[0]; o->dy = D->d[1]; o->dz = D->d[2];
  o->cx = D->c[0]; o->cy = D->c[1]; o->cz = D->c[2];
  o->gxi = D->glo[0]; o->gyi = D->glo[1]; o->gzi = D->glo[2];
  o->gxf = D->ghi[0]; o->gyf = D->ghi[1]; o->gzf = D->ghi[2];
}

static int field_id(const char *name)
{
  for (int f = 0; f < F_NUM; f++)
    if (strcmp(name, field_names[f]) == 0) return f;
  return -1;
}

int orc_get_field(const orc_solver *S, int g, const char *name, double *out)
{
  int f = field_id(name);
  if (f < 0 || g < 0 || g >= S->nboxes) return -1;
  memcpy(out, S->box[g].f[f], sizeof(double) * S->box[g].npts);
  return 0;
}

int orc_set_field(orc_solver *S, int g, const char *name, const double *in)
{
  int f = field_id(name);
  if (f < 0 || g < 0 || g >= S->nboxes) return -1;
  memcpy(S->box[g].f[f], in, sizeof(double) * S->box[g].npts);
  return 0;
}

/* u at arbitrary points as the reference prints it.  box < 0: the rule of
 * multigrid::Print_Interpol_1D / _2D (src/multigrid.cc:151-261, 555-880):
 * the largest box l0 (multigrid::multigrid, src/multigrid.cc:40-48, with
 * domain::operator<, src/domain.cc:1947-1954), a point outside it is not
 * printed (NaN here), otherwise the last box in level order whose interior
 * holds it (is_in_nb), l0 when none does.  box >= 0: that box, as
 * ffunction::Print_1D (src/ffunction.cc:819-960).  The value is
 * Lagrange_Interpol_In with ord+1 nodes per axis. */
int orc_interpolate(const orc_solver *S, int box, int first_level, const double *xyz, long npts, int ord,
                    double *out)
{
  if (box >= S->nboxes || ord < 1 || ord > 15 || first_level < 0 || first_level >= S->levels) return -1;
  const int first = S->first[first_level];
  int l0 = first;
  for (int g = first + 1; g < S->nboxes; g++) {
    const odom *A = &S->box[l0].D, *B = &S->box[g].D;
    int inside = 1;
    for (int a = 0; a < 3; a++) inside = inside && B->lo[a] < A->lo[a] && A->hi[a] < B->hi[a];
    if (inside) l0 = g;
  }
  for (long q = 0; q < npts; q++) {
    const double x = xyz[3 * q], y = xyz[3 * q + 1], z = xyz[3 * q + 2];
    int g = box;
    if (g < 0) {
      if (!dom_is_in(&S->box[l0].D, x, y, z)) {
        out[q] = NAN;
        continue;
      }
      g = l0;
      for (int b = first; b < S->nboxes; b++)
        if (dom_is_in_nb(&S->box[b].D, x, y, z)) g = b;
    }
    out[q] = interp_lagrange(&S->box[g], S->box[g].f[F_U], ord, x, y, z);
  }
  return 0;
}

double orc_vcycle(orc_solver *S)
{
  return fasn(S, S->levels - 1, S->levels - 1, 0, S->ncycles++);
}

/* elliptic::Vcycle, src/elliptic.cc:1251-1342 */
int orc_solve(orc_solver *S, int max_cycles, double *final_res)
{
  double res = 1e12, res_prev;
  int c = 0;
  do {
    res_prev = res;
    res = orc_vcycle(S);
    c++;
    if (S->nan_flag) break;
  } while (res > S->eps_solv && res < res_prev && c < max_cycles);
  if (final_res) *final_res = res;
  return S->nan_flag ? -c : c;
}

/* elliptic::Wcycle, src/elliptic.cc:1348-1380: W-cycles from the top level
 * while res > eps && res < res_prev; each one repeats every level until its
 * norm is <= eps_solv */
int orc_solve_wcycle(orc_solver *S, int max_cycles, double *final_res)
{
  double res = 1e12, res_prev;
  int c = 0;
  do {
    res_prev = res;
    res = fasn(S, S->levels - 1, S->levels - 1, 1, S->ncycles++);
    c++;
    if (S->nan_flag) break;
  } while (res > S->eps_solv && res < res_prev && c < max_cycles);
  if (final_res) *final_res = res;
  return S->nan_flag ? -c : c;
}

long orc_events(const orc_solver *S, long first, long cap, orc_event *out)
{
  for (long i = 0; i < cap && first + i < S->nev; i++) out[i] = S->ev[first + i];
  return S->nev;
}

void orc_set_wcycle_cap(orc_solver *S, long cap) { S->w_cap = cap > 0 ? cap : 1000000000L; }

void orc_adm(const orc_solver *S, double *out)
{
  for (int i = 0; i < S->P.numbh; i++) out[i] = S->adm[i];
}

double orc_smooth(orc_solver *S, int level, int ibox, int nu)
{
  return smooth_box(S, &S->box[S->first[level] + ibox], nu);
}

void orc_set_multicolor(orc_solver *S, int on) { S->multicolor = on; }
void orc_set_wsmooth(orc_solver *S, int on) { S->wsmooth = on; }
void orc_set_coarse_omega(orc_solver *S, double w) { S->coarse_omega = w; }
void orc_set_coarse_rtol(orc_solver *S, double r) { S->coarse_rtol = r; }
void orc_set_coarse_cap(orc_solver *S, long cap) { S->coarse_cap = cap > 0 ? cap : 1000000000L; }
long orc_coarse_iters(const orc_solver *S) { return S->coarse_iters; }
double orc_level_norm(const orc_solver *S, int level, int post)
{
  if (level == 0) return S->coarse_norm;
  return (level > 0 && level < 64) ? S->lnorm[level][post ? 1 : 0] : -1.0;
}

void orc_robin(orc_solver *S, int level, int ibox)
{
  robin_walk(S, &S->box[S->first[level] + ibox], robin_update_pt);
}
