/* olgpu.h -- C ABI of the GB300 puncture FAS solver (libolgpu.so).
 *
 * Plain C types only: no C++ types and no exceptions cross this boundary.
 * Every call returns an olgpu_status; olgpu_last_error() describes the last
 * failure of the calling thread.  A hierarchy handle owns all of its device
 * memory, is bound to one CUDA stream and must be used by one host thread at
 * a time.  Host buffers are owned by the caller and only touched during the
 * call that receives them.
 *
 * Reference interfaces replaced (WuShichao/OllipticID):
 *   olgpu_hierarchy_create  elliptic::elliptic(interface*) -> Make, Set_Grids,
 *                           Set_Equation, Set_Coefficients
 *                           (src/elliptic.cc:30-221, 299-921;
 *                            src/operator.cc:22-621, 629-1668)
 *   olgpu_box / olgpu_num_*  multigrid::Get_num_dom, domain getters
 *                           (include/multigrid.h:246, include/domain.h:457-727)
 *   olgpu_upload/download   multigrid::Get_ffunction(level, box, name) field
 *                           access (include/multigrid.h:98)
 *   olgpu_vcycle            elliptic::FASN(levels-1, levels-1, false, c)
 *                           (src/elliptic.cc:1468-1968)
 *   olgpu_solve             elliptic::Solve -> elliptic::Vcycle
 *                           (include/elliptic.h:331-334, src/elliptic.cc:1251-1342)
 *   olgpu_adm_mass          elliptic::Compute_ADM_Mass, puncture part
 *                           (src/elliptic.cc:2447-2469)
 */
#ifndef OLGPU_H
#define OLGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define OLGPU_MAX_BH 16

typedef enum {
  OLGPU_OK = 0,
  OLGPU_ERR_INVALID_ARG = 1,
  OLGPU_ERR_OOM = 2,
  OLGPU_ERR_CUDA = 3,
  OLGPU_ERR_NAN = 4,          /* the smoother produced NaN (reference: exit(0)) */
  OLGPU_ERR_DIVERGED = 5,
  OLGPU_ERR_TIMEOUT = 6,
  OLGPU_ERR_GEOMETRY = 7,     /* too few points for multigrid (reference: exit(1)) */
  OLGPU_ERR_NO_DEVICE = 8
} olgpu_status;

/* The reference's test equations, Lap u + u^2 = source (poisson_OP,
 * include/elliptic.h:359-366), run on the same FAS path in FP64:
 * OLGPU_EQ_POISSON, the Gaussian test (-eq Poisson, src/operator.cc:640-655,
 * 1865-1887): source a e^{-r^2}(a + e^{r^2/2}(r^2 - 3)), whose solution
 * u = a e^{-r^2/2} (a = 0.004) is known (a known-answer test);
 * OLGPU_EQ_BOUNDARY_TEST (-eq Boundary-test, 661-673, 1772-1816): source
 * -2a tanh(r) / (r cosh^2 r), boundary function a tanh(r) / r;
 * OLGPU_EQ_MULTIBOX_TEST (-eq Multibox-test, 1145-1175, 1820-1857): two
 * Gaussians e^{-0.05 r_i^2} centred at x = bhx1, bhx2 (NumBH >= 2).
 * OLGPU_EQ_BOWEN_YORK, the momentum-constraint test (-eq Bowen-York,
 * include/elliptic.h:772-803, src/operator.cc:370-398, 1320-1408, 3313-3408):
 * four unknowns, Lap V_i = rho_i (the momenta p_i of the punctures spread as
 * 3 p_i / (4 pi dr^3) over the points within one cell diagonal dr) and
 * Lap lambda - (Dx V1 + Dy V2 + Dz V3) = 0, each with the Robin falloff
 * n = 2.  olgpu_solve solves V1, V2, V3 and then lambda (the V equations do
 * not involve lambda: the same fixed point as the reference's joint
 * iteration); olgpu_download reads them as "V1", "V2", "V3", "lambda" ("u"
 * is the one being solved).  FP64, olgpu_solve only (not olgpu_solve_many,
 * a batch or the server). */
typedef enum {
  OLGPU_EQ_PUNCTURES = 0,
  OLGPU_EQ_PUNCTURES_SCALAR = 1,
  OLGPU_EQ_POISSON = 2,
  OLGPU_EQ_BOUNDARY_TEST = 3,
  OLGPU_EQ_MULTIBOX_TEST = 4,
  OLGPU_EQ_BOWEN_YORK = 5
} olgpu_equation;

/* The outer boundary condition (-B, src/boundary.cc:447-1535): Robin, u ~
 * u_inf + C / r^n (what the puncture pars/ files use), or Dirichlet, u fixed
 * to the boundary function on the outer ghost layers (the reference's
 * default without -B).  olgpu_problem_defaults picks Robin. */
typedef enum { OLGPU_BC_ROBIN = 0, OLGPU_BC_DIRICHLET = 1 } olgpu_boundary;

/* The cycle olgpu_solve runs (-m, elliptic::Set_Method, src/elliptic.cc:229-294):
 * V-cycles (elliptic::Vcycle, 1251-1342), or W-cycles (elliptic::Wcycle,
 * 1348-1380), where FASN repeats every level, each time through its own
 * coarser levels, until that level's post-smoothing norm is <= tol
 * (src/elliptic.cc:1956).  A W-cycle runs in FP64, from olgpu_solve only;
 * the mixed-precision cycle, olgpu_cycle_launch, olgpu_solve_many and the
 * server take V-cycles. */
typedef enum { OLGPU_METHOD_VCYCLE = 0, OLGPU_METHOD_WCYCLE = 1 } olgpu_method;

/* The Olliptic.x parameters of the puncture problem (src/interface.cc:73-273,
 * 748-856); -L is the full domain length and dx = L/(N-1). */
typedef struct {
  int equation;                 /* olgpu_equation                       */
  int numbh;                    /* -NumBH                               */
  double mp[OLGPU_MAX_BH];      /* -bhmp<i>                             */
  double x[OLGPU_MAX_BH], y[OLGPU_MAX_BH], z[OLGPU_MAX_BH];      /* -bhx<i> ... */
  double px[OLGPU_MAX_BH], py[OLGPU_MAX_BH], pz[OLGPU_MAX_BH];   /* -bhpx<i> ...*/
  double sx[OLGPU_MAX_BH], sy[OLGPU_MAX_BH], sz[OLGPU_MAX_BH];   /* -bhsx<i> ...*/
  int n;                        /* -N                                   */
  double L;                     /* -L                                   */
  int order;                    /* -O  2, 4, 6 or 8                     */
  int levels;                   /* -l                                   */
  int nu1, nu2;                 /* -nu1, -nu2                           */
  double tol;                   /* -s                                   */
  int ps_case;                  /* -psc                                 */
  double ps_phi0, ps_r0, ps_sigma, ps_a2;   /* -phi0 -r0 -sigma -a2     */
  int boundary;                 /* -B: olgpu_boundary                   */
  int method;                   /* -m: olgpu_method                     */
} olgpu_problem;

typedef struct {
  int level, nx, ny, nz;        /* points per axis, ghost layers included */
  int buf;                      /* ghost width max(order/2, 1)            */
  int order;                    /* stencil order of this box              */
  double xi, yi, zi;            /* coordinate of point (0,0,0)            */
  double dx, dy, dz;
  double cx, cy, cz;            /* box centre                             */
  double xf, yf, zf;            /* coordinate of the last point (domain xf) */
} olgpu_box_info;

/* Stop rules for olgpu_solve.  The reference stops on the top level's
 * residual alone; on nested boxes the coarser levels can still be moving
 * then (u 1e-9 from the fixed point at a 1e-11 residual), so
 * OLGPU_STOP_ERROR also bounds the cycle's largest change of u on every
 * point the discrete system fixes: with the cycle's contraction rate below
 * one half that change bounds the distance of u from the fixed point.  For
 * mixed precision the residual part is the finest FP64 defect.  V-cycles
 * only. */
typedef enum {
  OLGPU_STOP_REFERENCE = 0,     /* while res > tol && res < res_prev (src/elliptic.cc:1330) */
  OLGPU_STOP_TOLERANCE = 1,     /* while res > tol                                          */
  OLGPU_STOP_FIXED = 2,         /* exactly max_cycles cycles                                */
  OLGPU_STOP_ERROR = 3          /* while res > tol || max |du| > du_tol                     */
} olgpu_stop_kind;

typedef struct {
  int stop;                     /* olgpu_stop_kind                        */
  int max_cycles;               /* hard cap on V-cycles (> 0)             */
  double tol;                   /* <= 0: the problem's -s tolerance       */
  double du_tol;                /* OLGPU_STOP_ERROR's bound on the cycle's
                                   largest change of u; <= 0: tol         */
} olgpu_stop_rule;

typedef struct {
  int cycles;                   /* top-level cycles run                   */
  int status;                   /* olgpu_status of the solve              */
  double final_res;             /* top-level residual norm of the last cycle */
  double adm[OLGPU_MAX_BH];     /* ADM masses after the last cycle        */
  double res[256];              /* per-cycle top-level norms (first 256)  */
  double final_du;              /* the last cycle's largest change of u on
                                   the points the discrete system fixes   */
  double final_part;            /* the last cycle's residual part: FP64, the
                                   top-level norm (= final_res); mixed, the
                                   finest FP64 defect (final_res is the larger
                                   of it and the cycle's largest correction) */
} olgpu_report;

typedef struct olgpu_hierarchy olgpu_hierarchy;

/* Default parameter values of Olliptic.x. */
void olgpu_problem_defaults(olgpu_problem *p);

/* Geometry only, no GPU needed: the boxes elliptic::Set_Grids builds for p
 * (src/elliptic.cc:299-921), level-major.  Writes up to cap entries into out
 * (out may be NULL) and the totals into the non-NULL count pointers. */
olgpu_status olgpu_plan_boxes(const olgpu_problem *p, olgpu_box_info *out, int cap, int *nboxes,
                              int *nlevels, int *mgrid_levels);

/* Builds the nested-box hierarchy of the problem (Set_Grids), allocates every
 * field in device memory, evaluates the coefficients and the initial guess
 * u = 0 on the device.  device < 0 keeps the current device. */
olgpu_status olgpu_hierarchy_create(const olgpu_problem *p, int device, olgpu_hierarchy **out);
olgpu_status olgpu_hierarchy_destroy(olgpu_hierarchy *h);

int olgpu_num_boxes(const olgpu_hierarchy *h);
int olgpu_num_levels(const olgpu_hierarchy *h);
int olgpu_mgrid_levels(const olgpu_hierarchy *h);
olgpu_status olgpu_box(const olgpu_hierarchy *h, int box, olgpu_box_info *out);

/* The reference's storage order of a box's points (domain::Fix_Points,
 * src/domain.cc:574-1388: corners, edges, faces, interior), the order its
 * iterators and its 3-D dumps visit them: out receives nx*ny*nz indices
 * into the lexicographic layout of the box (i fastest).  Host only. */
olgpu_status olgpu_storage_order(const olgpu_box_info *box, long long *out);

/* Field access by reference name: "u" "b" "c" "d" "e" "rho" (the source
 * rho0), "r", "w", "ww", "v", and the solver's work fields "t" (the
 * full-weighted W) and "up" (u as the last cycle found it).  Host arrays
 * hold nx*ny*nz doubles in lexicographic order, i fastest. */
olgpu_status olgpu_upload(olgpu_hierarchy *h, int box, const char *field, const double *host);
olgpu_status olgpu_download(olgpu_hierarchy *h, int box, const char *field, double *host);

/* One FAS V-cycle from the finest level; *res receives the top-level norm. */
olgpu_status olgpu_vcycle(olgpu_hierarchy *h, double *res);
/* Repeated cycles of the problem's method under a stop rule; rule NULL =
 * the reference's rule.  For W-cycles the rule stops the top-level calls
 * (normally one: its own loop meets tol), and the iterations of each level's
 * loop in one call are capped at min(max_cycles, OLGPU_WCYCLE_LEVEL_CAP)
 * (the reference has no cap and repeats forever where a level's norm levels
 * off above tol); a level that reaches the cap without meeting tol ends the
 * solve with OLGPU_ERR_DIVERGED. */
#define OLGPU_WCYCLE_LEVEL_CAP 500
olgpu_status olgpu_solve(olgpu_hierarchy *h, const olgpu_stop_rule *rule, olgpu_report *out);
olgpu_status olgpu_adm_mass(olgpu_hierarchy *h, double *out);
/* The parts of the last finished cycle's norm (either pointer may be NULL):
 * *res its residual (FP64: the top level's post-smoothing norm, the
 * reference's; mixed: the finest FP64 defect) and *du its largest change of
 * u on the points the discrete system fixes (every point of the solution
 * levels, the INSIDE points of the multigrid coarse levels).  No reference
 * counterpart. */
olgpu_status olgpu_last_cycle(const olgpu_hierarchy *h, double *res, double *du);

/* Smoother norms of one cycle of the current solve (0 = its first cycle;
 * olgpu_solve / olgpu_solve_many start a new history): pre[l] and post[l],
 * l = 0 .. olgpu_num_levels - 1, the L-infinity norms the smoother of level
 * l reported before and after the cycle's correction (the reference's
 * "Loo[l]" lines, elliptic::Print_Pre_Cycle / Print_Post_Cycle,
 * src/output.cc:1355-1605); level 0
 * holds the coarsest solve's norm.  In mixed precision they are the norms
 * of the FP32 correction cycle. */
olgpu_status olgpu_level_norms(const olgpu_hierarchy *h, int cycle, double *pre, double *post);

/* Every elliptic::Print_Pre_Cycle (post = 0) and Print_Post_Cycle (post = 1)
 * call of the current solve, in the reference's order: the level (0: the
 * coarsest solve, logged as a pre call), the cycle number it prints (the
 * per-level count of FASN, src/elliptic.cc:1499, 1935) and the norm.  Loo.gp
 * holds the pre calls' (cycle, norm); stdout0.out's tables all of them.  A
 * V-cycle logs levels-1 .. 1 pre, 0, 1 .. levels-1 post, all with the cycle's
 * number; a W-cycle logs each level iteration as it runs.  Copies calls
 * [first, first + cap) into out (NULL when cap is 0) and writes how many the
 * solve has logged into *total. */
typedef struct {
  int level;
  int post;
  long long cycle;
  double norm;
} olgpu_cycle_event;
olgpu_status olgpu_cycle_events(const olgpu_hierarchy *h, long long first, int cap, olgpu_cycle_event *out,
                                long long *total);

/* u at arbitrary points, as the reference prints and exports it
 * (multigrid::Print_Interpol_1D / _2D, src/multigrid.cc:151-261 and 555-880;
 * ffunction::Print_1D, src/ffunction.cc:819-960; the Lagrange sum of
 * ffunction::Lagrange_Interpol_In, src/interpolation.cc:188-375).
 * box < 0: each point is read from the last box, in level order, whose
 * interior (no ghost layers) holds it, from the largest box when none does,
 * and is NaN outside the largest box (the reference prints no line there);
 * box >= 0: every point is read from that box.  With box < 0 only the boxes
 * of levels >= first_level take part: 0 as the V-cycle's hierarchy prints;
 * olgpu_mgrid_levels() for the analytic method's (elliptic::ApproximateID),
 * whose hierarchy has no multigrid coarse grids.  The value is the node value
 * where the point coincides with a node, else the Lagrange sum over ord+1
 * nodes per axis (the reference prints with ord = order + 1), window clamped
 * to the box.  xyz holds npts (x, y, z) triples and out npts values, both
 * host memory; the gather runs on the device, ordered after the cycles
 * already enqueued. */
olgpu_status olgpu_interpolate(olgpu_hierarchy *h, int box, int first_level, const double *xyz, long long npts,
                               int ord, double *out);
/* The same for any field olgpu_download reads (Bowen-York's "V1", "V2",
 * "V3", "lambda" among them: the reference prints each variable this way,
 * src/output.cc:624-730); olgpu_interpolate is this with "u". */
olgpu_status olgpu_interpolate_field(olgpu_hierarchy *h, const char *field, int box, int first_level,
                                     const double *xyz, long long npts, int ord, double *out);

/* Asynchronous stepping, for hosts that drive several solves at once (each
 * hierarchy has its own CUDA stream, so cycles of different hierarchies run
 * concurrently on the GPU).  olgpu_cycle_launch enqueues one V-cycle and
 * returns; olgpu_cycle_poll reports whether it finished (wait != 0 blocks)
 * and then its norm (*res) -- the same norm olgpu_vcycle returns. */
olgpu_status olgpu_cycle_launch(olgpu_hierarchy *h);
olgpu_status olgpu_cycle_poll(olgpu_hierarchy *h, int wait, int *done, double *res);
/* Solves n problems concurrently, each under the same stop rule (rule NULL =
 * the reference's), stepping every unfinished one each round; reports[i]
 * (may be NULL) gets the i-th problem's report.  Returns the first failure
 * status, if any. */
olgpu_status olgpu_solve_many(olgpu_hierarchy **hs, int n, const olgpu_stop_rule *rule, olgpu_report *reports);

/* Arithmetic of the V-cycle.  OLGPU_PREC_FP64 runs the reference's FAS
 * cycle in FP64 throughout.  OLGPU_PREC_MIXED keeps u, the defect, the
 * singular puncture terms b/(c+u)^7 and 1/(c+u), the update and the
 * convergence norm in FP64 and runs the V-cycle itself (smoothing, Robin
 * updates, transfers, coarse solve) in FP32 on a correction e to u; it
 * converges to the same FP64 fixed point.  In mixed mode the cycle's norm
 * (stop rule, report) is the larger of the FP64 L-infinity defect of the
 * finest level after the update and the largest correction |e| applied to a
 * point the discrete system fixes, so that stopping at tol also bounds the
 * remaining error in u on every level. */
typedef enum { OLGPU_PREC_FP64 = 0, OLGPU_PREC_MIXED = 1 } olgpu_precision;
olgpu_status olgpu_set_precision(olgpu_hierarchy *h, int precision);
/* Anderson acceleration of the mixed-precision outer iteration with a
 * history of `depth` corrections (0 = off, 1..4; default 4).  Each cycle's
 * update becomes u + f - (dU + dF) gamma with gamma the least-squares fit of
 * the newest correction f by the last `depth` correction differences; the
 * fixed point is unchanged.  Applies to OLGPU_PREC_MIXED only. */
olgpu_status olgpu_set_acceleration(olgpu_hierarchy *h, int depth);
/* The same Anderson mixing for the plain FP64 V-cycle, with its history and
 * sums in FP64 (depth 0..4; default 0: the reference's iteration).  Each
 * cycle's change u - u_before is mixed with the last `depth` changes; the
 * fixed point is the FP64 cycle's, reached in fewer cycles (the multicolour
 * FAS cycle's slow smooth mode is damped).  V-cycles of one hierarchy; a
 * change of depth re-captures the cycle and clears the history.  No
 * reference counterpart. */
olgpu_status olgpu_set_fp64_acceleration(olgpu_hierarchy *h, int depth);

/* Pre- and post-smoothing sweeps of the FP32 correction cycle of
 * OLGPU_PREC_MIXED (default: the problem's nu1 / nu2).  No reference
 * counterpart: the reference has no inner cycle.  The FP64 fixed point does
 * not depend on them, only the work per outer cycle and the number of outer
 * cycles do.  Re-captures the mixed cycle if it is built and clears the
 * acceleration history; call between solves.  0 <= nu1 <= 64, 1 <= nu2 <= 64. */
olgpu_status olgpu_set_inner_sweeps(olgpu_hierarchy *h, int nu1, int nu2);

/* Largest thread-block cluster (8..16 blocks) that keeps a box's FP32
 * correction resident through all sweeps of the mixed cycle's smoother, or 0
 * for one launch per colour and sweep (default 16).  No reference
 * counterpart.  Smaller clusters leave more of the GPU to other solves; the
 * result is the same bit for bit.  Re-captures the mixed cycle if built. */
olgpu_status olgpu_set_smoother_blocks(olgpu_hierarchy *h, int max_blocks);

/* Reset u to the initial guess (0) and the work fields, keeping the geometry
 * and coefficients, so that one hierarchy can serve repeated solves. */
olgpu_status olgpu_reset(olgpu_hierarchy *h);

/* Serving: continuous batching of puncture solves on one GPU (no reference
 * counterpart; the reference runs one solve per process).  Requests are
 * admitted in arrival order while a slot (max_active) and their device
 * footprint (from the host-only plan) fit in mem_budget; builder threads
 * make their hierarchies while a scheduler thread keeps every admitted solve's
 * next cycle queued on its own stream (olgpu_cycle_launch / _poll), so the
 * work of different requests overlaps on the device; a finished solve frees
 * its memory at once and the next request takes its place.  A request whose
 * footprint exceeds mem_budget is refused with OLGPU_ERR_OOM.  Each result is
 * the one the same problem gives solved alone, bit for bit.  With
 * batch_max >= 2 the requests admitted together (up to batch_max, once as
 * many wait or the oldest has waited batch_window) are solved as one batch
 * (olgpu_batch_*: one launch per FASN step over all of them) on a builder
 * thread, several batches at once; each result is reported when its batch
 * ends, and keep_solutions is refused.
 * olgpu_server_submit and olgpu_server_poll may be called from any thread. */
typedef struct olgpu_server olgpu_server;

typedef struct {
  int device;                   /* CUDA device (-1: the current one)          */
  long long mem_budget;         /* device bytes the admitted solves may hold   */
  int max_active;               /* solves on the GPU (or being built) at once  */
  int precision;                /* olgpu_precision of every solve              */
  int stop;                     /* olgpu_stop_kind of every solve              */
  int max_cycles;               /* cap on V-cycles per solve (> 0)             */
  double tol;                   /* <= 0: each problem's -s tolerance           */
  int builders;                 /* host threads building hierarchies (>= 1)    */
  int nu1, nu2;                 /* FP32 cycle sweeps (mixed); nu1 < 0: the problem's */
  int blocks;                   /* FP32 smoother cluster blocks; < 0: follow the load */
  int busy;                     /* with blocks < 0: per-colour launches while fewer
                                   solves are on the GPU, clusters of 16 beyond */
  int keep_solutions;           /* != 0: a finished solve's hierarchy is handed
                                   to the caller in olgpu_server_result.h      */
  double du_tol;                /* OLGPU_STOP_ERROR's bound on a cycle's change
                                   of u; <= 0: the tolerance                   */
  int batch_max;                /* >= 2: admitted requests are solved together as
                                   batches (olgpu_batch_*) of up to batch_max;
                                   0 or 1: one hierarchy per request           */
  double batch_window;          /* batching: seconds the oldest waiting request
                                   waits for a batch to fill before it is
                                   admitted with those waiting beside it       */
} olgpu_server_config;

typedef struct {
  long long id;                 /* the request                                */
  int status;                   /* olgpu_status of the request                */
  int cycles;                   /* V-cycles run                               */
  double final_res;             /* norm of the last cycle                     */
  double adm[OLGPU_MAX_BH];     /* ADM masses after the last cycle            */
  double queue_s;               /* arrival (submit) to admission              */
  double latency_s;             /* arrival to the end of the last cycle       */
  olgpu_hierarchy *h;           /* keep_solutions: the solved hierarchy, now the
                                   caller's (destroy it); else NULL            */
  double final_du;              /* the last cycle's largest change of u       */
} olgpu_server_result;

void olgpu_server_config_defaults(olgpu_server_config *c);
olgpu_status olgpu_server_create(const olgpu_server_config *c, olgpu_server **out);
/* Queues one problem; *id identifies its result. */
olgpu_status olgpu_server_submit(olgpu_server *s, const olgpu_problem *p, long long *id);
/* *done = 1 and *out filled once request id has finished (its result is then
 * released; a second poll of the same id is an error); wait != 0 blocks until
 * it has.  Returns the call's status; the request's own is out->status. */
olgpu_status olgpu_server_poll(olgpu_server *s, long long id, int wait, int *done, olgpu_server_result *out);
/* Solves on the GPU, being built or waiting, and the peak of the first. */
olgpu_status olgpu_server_stats(olgpu_server *s, int *active, int *building, int *waiting, int *peak_active);
/* Stops the threads, finishes nothing more and frees every hierarchy it holds
 * (results not yet polled included).  No other call on s may be running or
 * waiting when it is called. */
olgpu_status olgpu_server_destroy(olgpu_server *s);

/* Batching (no reference counterpart; the reference runs one solve per
 * process): uneven puncture solves stepped together on one GPU, every FASN
 * step of a level one launch over the boxes of all the solves at that level.
 * The solves are grouped into unions -- the same equation, order, boundary,
 * sweep counts and refinement depth (levels above the base grid) -- whose
 * levels are aligned from the finest down, so that a solve with fewer levels
 * reaches its coarsest solve earlier while the others descend further; each
 * union holds its solves' fields in one device arena and steps them with one
 * captured cycle, a solve that meets its stop rule drops out of every launch
 * (its boxes are skipped) and the others go on.  A union of several solves
 * runs each FASN step as one launch where the solves alone would run one
 * launch each; the arithmetic of every point is the solve's own, so each
 * result is the same, bit for bit, as the problem solved alone
 * (olgpu_solve) under the same rule and precision.  V-cycles; mixed precision
 * for the puncture equations with the Robin boundary. */
typedef struct olgpu_batch olgpu_batch;

typedef struct {
  int device;                   /* CUDA device (-1: the current one)            */
  int precision;                /* olgpu_precision of every solve               */
  int nu1, nu2;                 /* FP32 cycle sweeps (mixed); < 0: the problems' */
  int blocks;                   /* FP32 smoother cluster blocks (0: one launch per
                                   colour and sweep); < 0: the default (16)     */
} olgpu_batch_config;

void olgpu_batch_config_defaults(olgpu_batch_config *c);
/* Plans, groups and sets up n problems (initial guess u = 0). */
olgpu_status olgpu_batch_create(const olgpu_problem *ps, int n, const olgpu_batch_config *c, olgpu_batch **out);
/* Solves every problem of the batch under the same stop rule (NULL: the
 * reference's); reports[i] (may be NULL) gets problem i's report.  Returns
 * the first failure status, if any (each report holds its own). */
olgpu_status olgpu_batch_solve(olgpu_batch *b, const olgpu_stop_rule *rule, olgpu_report *reports);
/* u = 0 again for every problem (repeated solves of the same batch). */
olgpu_status olgpu_batch_reset(olgpu_batch *b);
/* Problem i's hierarchy, for olgpu_download / olgpu_box / olgpu_adm_mass /
 * olgpu_level_norms (owned by the batch: do not destroy or solve it). */
olgpu_hierarchy *olgpu_batch_member(olgpu_batch *b, int i);
int olgpu_batch_size(const olgpu_batch *b);
/* Unions the problems were grouped into, and their kernel launches per cycle. */
int olgpu_batch_unions(const olgpu_batch *b);
int olgpu_batch_kernels_per_cycle(const olgpu_batch *b);
/* Host wall-clock time of the last olgpu_batch_solve in ms. */
double olgpu_batch_last_ms(const olgpu_batch *b);
olgpu_status olgpu_batch_destroy(olgpu_batch *b);

/* elliptic::ApproximateID (src/elliptic.cc:1977-2226, the reference's
 * "-m AppPuncture" method): u on every point of every box becomes the
 * perturbative puncture solution (spin, momentum and cross terms summed over
 * the punctures), the work fields are reset as by olgpu_reset.  as_guess = 0
 * evaluates the formula as the reference writes it (what -m AppPuncture
 * prints); as_guess != 0 takes the momentum term's small-distance limit from
 * its series (the formula cancels to rounding noise of order 1e10 on a
 * puncture that sits on a grid node).  As a start for olgpu_solve it leaves
 * the fixed point unchanged and takes cycles off. */
olgpu_status olgpu_approximate_id(olgpu_hierarchy *h, int as_guess);

/* Timing aids. */
/* device time of the last olgpu_solve / olgpu_vcycle in ms */
double olgpu_last_device_ms(const olgpu_hierarchy *h);
/* kernel launches in one V-cycle (the captured graph's kernel nodes) */
int olgpu_kernels_per_cycle(const olgpu_hierarchy *h);
/* iterations of the coarsest-level solve in the last finished cycle (the
 * reference prints no such count; diagnostic only) */
int olgpu_last_coarse_iters(const olgpu_hierarchy *h);
/* INSIDE points of a level, summed over its boxes (algorithmic work unit) */
long long olgpu_level_interior_points(const olgpu_hierarchy *h, int level);
/* Times `sweeps` full smoother sweeps (every colour pass) on one level with
 * CUDA events on the hierarchy's stream; *ms gets the elapsed device time and
 * *launches the number of smoother kernels it launched.  Changes u (FP64
 * precision) or the FP32 correction e (mixed precision: its smoother). */
olgpu_status olgpu_time_smoother(olgpu_hierarchy *h, int level, int sweeps, double *ms, int *launches);
/* The same for n hierarchies at once (no reference counterpart): each one's
 * sweeps on its own stream, all started together; *ms is the device time
 * from the common start to the last one's end.  Measures the smoother's rate
 * when many solves share the GPU. */
olgpu_status olgpu_time_smoother_many(olgpu_hierarchy *const *hs, int n, int level, int sweeps, double *ms);
/* Device memory of the library's hierarchies and batches on one device (no
 * reference counterpart): they allocate from one stream-ordered pool per
 * device, so that a finished solve frees its memory without waiting for the
 * GPU and the next one reuses it.  *reserved: bytes the pool holds from the
 * device; *used: bytes handed out to live hierarchies.  The pool keeps its
 * memory while any hierarchy is alive and gives it back when the last one
 * is destroyed. */
olgpu_status olgpu_device_pool_bytes(int device, long long *reserved, long long *used);
/* Measured issue rate of dependent-free fused multiply-adds on the current
 * device (no reference counterpart): every SM runs eight 256-thread blocks,
 * each thread eight independent FMA chains of `iters` steps, timed with CUDA
 * events; *tflops = 2 * FMAs / time.  precision: OLGPU_PREC_FP64 (double
 * FMA) or OLGPU_PREC_MIXED (float FMA).  The stencil kernels' instruction
 * roofline is taken against it. */
olgpu_status olgpu_fma_peak(int precision, int iters, double *tflops);

/* One box whose fields the caller already holds in device memory (all
 * nx*ny*nz doubles, lexicographic, i fastest, ghost layers included). */
typedef struct {
  double *u;                    /* in/out: the solution                   */
  const double *b, *c;          /* puncture coefficients                  */
  const double *s;              /* source (the reference's rho0 / tau)    */
  const double *d, *e;          /* scalar-field coefficients, or both NULL */
  int nx, ny, nz;
  int order;                    /* 2, 4, 6 or 8; ghost width max(order/2,1) */
  double dx, dy, dz;
} olgpu_box_fields;

#define OLGPU_NOALLOC_MAX_SWEEPS 64

/* Non-allocating variant of the multicolour Gauss-Seidel-Newton smoother
 * (no counterpart in the reference).  Some callers cannot call cudaMalloc:
 * host codes that hand out all device memory from their own pre-reserved
 * pool, or serving processes that fix their memory budget at start-up and
 * must not grow it per request.  This entry point allocates nothing: the
 * caller passes the box's fields, and the kernel's scratch (the box
 * descriptor, one residual-norm accumulator per sweep and a NaN flag) lives
 * in a fixed 2 KiB array in the library's device memory, which every GPU that
 * loads the library holds until the process exits.
 *   sweeps: 1..OLGPU_NOALLOC_MAX_SWEEPS (64); more is rejected with
 *           OLGPU_ERR_INVALID_ARG.
 *   norms:  host array of `sweeps` doubles, the L-infinity norm of the
 *           pre-update point residuals of each sweep (may be NULL).
 *   stream: cudaStream_t to run on (NULL = the default stream); the call
 *           returns after that stream has finished the sweeps.
 * The first call on a device looks up the scratch array's device address
 * (set-up once per device); make that first call before any stream capture.
 * A device reset (cudaDeviceReset) makes that address stale: a call that
 * meets a CUDA error forgets it and the next call looks it up again, so
 * after a reset call once outside any capture before relying on it.
 * Every call on a device shares the one scratch array, and the call clears
 * the parts that must start at zero: calls that overlap on the GPU (from
 * several host threads or streams) race on it and must be serialised by the
 * caller. */
olgpu_status olgpu_smooth_box_noalloc(const olgpu_box_fields *f, int sweeps, double *norms, void *stream);

const char *olgpu_last_error(void);
const char *olgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OLGPU_H */
