/* olliptic_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's (WuShichao/OllipticID) FAS multigrid
 * solve of the puncture Hamiltonian constraint.  It is the checker for the
 * GPU library: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load it.  The product (libolgpu) never links or calls it.
 *
 * Every routine follows the reference's arithmetic in the same order, so that
 * on the same host it reproduces the reference's iterates (pinned against the
 * reference itself by tests/golden/, which oracle/ref_harness.cc generated).
 */
#ifndef OLLIPTIC_ORACLE_H
#define OLLIPTIC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_BH 16

typedef struct {
  int equation;            /* 0 Punctures, 1 Punctures_scalar_field, 2 Poisson (Gaussian test),
                              3 Boundary-test, 4 Multibox-test, 5 Bowen-York (one variable of
                              the system, by_var) */
  int numbh;
  double mp[ORC_MAX_BH];
  double x[ORC_MAX_BH], y[ORC_MAX_BH], z[ORC_MAX_BH];
  double px[ORC_MAX_BH], py[ORC_MAX_BH], pz[ORC_MAX_BH];
  double sx[ORC_MAX_BH], sy[ORC_MAX_BH], sz[ORC_MAX_BH];
  int n;                   /* -N  (snapped by Valid_N)                      */
  double L;                /* -L  full domain length                        */
  int order;               /* -O  2/4/6/8                                   */
  int levels;              /* -l  refinement levels incl. the base grid     */
  int nu1, nu2;            /* -nu1 / -nu2                                   */
  double tol;              /* -s                                            */
  /* scalar field (-psc -phi0 -r0 -sigma -a2) */
  int ps_case;
  double ps_phi0, ps_r0, ps_sigma, ps_a2;
  int boundary;            /* -B: 0 Robin, 1 Dirichlet (the reference's default) */
  int by_var;              /* Bowen-York: 0..2 V1..V3 (source rho0..rho2), 3 lambda (source
                              set by orc_set_divergence_source) */
} orc_problem;

typedef struct orc_solver orc_solver;

typedef struct {
  int level, nx, ny, nz, buf, order;
  double xi, yi, zi, xf, yf, zf, dx, dy, dz, cx, cy, cz;
  double gxi, gyi, gzi, gxf, gyf, gzf;
} orc_box_info;

void orc_problem_defaults(orc_problem *p);
orc_solver *orc_create(const orc_problem *p);
/* checker variant: multigrid coarsening continues below 12 points (to >= 5) */
orc_solver *orc_create_extra_coarse(const orc_problem *p);
void orc_destroy(orc_solver *s);
int orc_num_boxes(const orc_solver *s);
int orc_num_levels(const orc_solver *s);
int orc_mgrid_levels(const orc_solver *s);
void orc_box(const orc_solver *s, int box, orc_box_info *out);
/* field names: "u" "b" "c" "d" "e" "rho" "r" "w" "ww" "v"; lexicographic, i fastest */
int orc_get_field(const orc_solver *s, int box, const char *name, double *out);
int orc_set_field(orc_solver *s, int box, const char *name, const double *in);
/* u at npts (x, y, z) points (xyz, 3*npts doubles): box < 0 follows the
 * reference's printed-cut rule (finest box whose interior holds the point,
 * NaN outside the largest box) over the boxes of levels >= first_level
 * (the analytic method's hierarchy has no multigrid grids), box >= 0 reads
 * that box; ord+1 Lagrange nodes per axis.  Returns 0, or -1 on a bad argument. */
int orc_interpolate(const orc_solver *s, int box, int first_level, const double *xyz, long npts, int ord,
                    double *out);
/* elliptic::ApproximateID: u := the perturbative puncture solution on every box */
void orc_approximate_id(orc_solver *s);
/* one FAS V-cycle from the top level (elliptic::FASN); returns the top-level norm */
double orc_vcycle(orc_solver *s);
/* elliptic::Vcycle: cycles while res > eps && res < res_prev; returns cycles run */
int orc_solve(orc_solver *s, int max_cycles, double *final_res);
/* elliptic::Wcycle: W-cycles (every level repeated until its norm <= eps)
 * while res > eps && res < res_prev; returns top-level cycles run */
int orc_solve_wcycle(orc_solver *s, int max_cycles, double *final_res);
/* One elliptic::Print_Pre_Cycle (post = 0) or Print_Post_Cycle (post = 1)
 * call: the level (0: the coarsest solve), the cycle number it prints and
 * the norm.  orc_events copies events [first, first+cap) and returns how many
 * the solver has logged since it was created. */
typedef struct {
  int level;
  int post;
  long cycle;
  double norm;
} orc_event;
long orc_events(const orc_solver *s, long first, long cap, orc_event *out);
/* checker guard on one level's W loop (the reference has none) */
void orc_set_wcycle_cap(orc_solver *s, long cap);
/* ADM masses computed at the end of every top-level cycle */
void orc_adm(const orc_solver *s, double *out);
/* Single-box building blocks, exposed for unit tests. */
double orc_smooth(orc_solver *s, int level, int ibox, int nu);
void orc_robin(orc_solver *s, int level, int ibox);
/* Checker options outside the reference algorithm: visit smoother points by
 * colour (i+j+k) mod (ghost width + 1) like the GPU, and cap the coarsest-grid
 * sweeps per V-cycle.  Neither changes the discrete fixed point. */
void orc_set_multicolor(orc_solver *s, int on);
void orc_set_coarse_cap(orc_solver *s, long cap);
void orc_set_wsmooth(orc_solver *s, int on);
void orc_set_coarse_omega(orc_solver *s, double omega);
void orc_set_coarse_rtol(orc_solver *s, double rtol);
long orc_coarse_iters(const orc_solver *s);
/* last cycle's smoother norm on a level (post = 0 pre-, 1 post-smoothing);
 * level 0 gives the coarsest-solve norm */
double orc_level_norm(const orc_solver *s, int level, int post);
/* Bowen-York's lambda equation, Lap lambda - (Dx V1 + Dy V2 + Dz V3) = 0
 * (include/elliptic.h:796-800), with the divergence moved into the source:
 * rho of every INSIDE point of every box of `lam` := Dx V1 + Dy V2 + Dz V3
 * of the hierarchies v1, v2, v3 (same problem, by_var 0..2).  The FAS
 * equations of every level are the same (the divergence of the level's V
 * enters both sides of the tau correction and cancels), so the fixed point
 * is the system's. */
void orc_set_divergence_source(orc_solver *lam, const orc_solver *v1, const orc_solver *v2, const orc_solver *v3);
/* Valid_N restated (src/interface.cc:883-945) */
int orc_valid_n(int n);

#ifdef __cplusplus
}
#endif
#endif
