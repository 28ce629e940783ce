// olgpu.cu -- C ABI of the GB300 puncture FAS solver and its host driver.
//
// The driver mirrors elliptic::FASN (WuShichao/OllipticID,
// src/elliptic.cc:1468-1968) step by step, but every step is a device kernel
// over all boxes of a level, and the whole V-cycle is recorded once into a
// CUDA graph that is replayed for every cycle.  Host work per cycle: one graph
// launch and one small device-to-host copy of the cycle's norms.
#include "../../include/olgpu.h"
#include "device.cuh"
#include "grid.h"
#include "kernels.cuh"
#include "coarse_cluster.cuh"
#include "mixed.cuh"
#include "smooth_cluster.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <thread>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

using namespace olgpu;

namespace {

thread_local std::string g_last_error;

olgpu_status fail(olgpu_status s, const std::string &msg)
{
  g_last_error = msg;
  return s;
}

#define CUDA_TRY(expr)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (expr);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail(e_ == cudaErrorMemoryAllocation ? OLGPU_ERR_OOM : OLGPU_ERR_CUDA,          \
                  std::string(#expr) + ": " + cudaGetErrorString(e_));                       \
  } while (0)

constexpr int kThreads = 256;
// blocks of the per-colour smoothers: one colour of a level is about one
// wave of 256-thread blocks, so smaller blocks spread it more evenly
constexpr int kSmoothThreads = 128;
constexpr size_t kCoarseSmemMax = 200 * 1024;   // dynamic shared memory of the coarse solves
constexpr size_t kCoarse32ClusterSmem = 96 * 1024;   // ... of a block of k_coarse32_cluster
// iterations of one W-cycle level's loop in one call (OLGPU_WCYCLE_LEVEL_CAP)
constexpr int kWcycleLevelCap = OLGPU_WCYCLE_LEVEL_CAP;

// ---------------------------------------------------------------------------
// Device memory of hierarchies and batches: one stream-ordered pool per
// device.  cudaFree waits for the whole device, so in a server (or under
// solve_many) every finished solve freed that way would hold up every other
// solve's queued cycles; cudaFreeAsync on the owner's stream returns at once,
// the memory goes back to the pool when the stream gets there, and the next
// hierarchy's allocations are served from it.  The pool keeps what it holds
// (no release threshold) while any hierarchy of the process is alive and is
// trimmed when the last one is destroyed.  The pinned host copies of the
// stats are recycled the same way (cudaFreeHost waits for the device too).
// ---------------------------------------------------------------------------
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};
int g_live[kMaxDevices] = {};
std::vector<Stats *> g_pinned_stats;

cudaMemPool_t device_pool(int dev)
{
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> g(g_pool_mu);
  if (g_pools[dev]) {   // still valid (a device reset by the host destroys it)
    unsigned long long thr = 0;
    if (cudaMemPoolGetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &thr) != cudaSuccess) {
      cudaGetLastError();
      g_pools[dev] = nullptr;
      g_live[dev] = 0;
    }
  }
  if (!g_pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
  }
  return g_pools[dev];
}

// bytes of device memory in stream order on s (usable on s at once, on other
// streams once s has reached this point)
cudaError_t dev_alloc(void **p, size_t bytes, int dev, cudaStream_t s)
{
  *p = nullptr;
  if (bytes == 0) return cudaSuccess;
  cudaMemPool_t pool = device_pool(dev);
  if (!pool) return cudaErrorMemoryAllocation;
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

void dev_free(void *p, cudaStream_t s)
{
  if (p) cudaFreeAsync(p, s);
}

Stats *pinned_stats_get()
{
  {
    std::lock_guard<std::mutex> g(g_pool_mu);
    while (!g_pinned_stats.empty()) {
      Stats *p = g_pinned_stats.back();
      g_pinned_stats.pop_back();
      // a device reset by the host frees pinned memory too: reuse only what
      // is still registered
      cudaPointerAttributes pa{};
      if (cudaPointerGetAttributes(&pa, p) == cudaSuccess && pa.type == cudaMemoryTypeHost) return p;
      cudaGetLastError();
    }
  }
  Stats *p = nullptr;
  return cudaMallocHost(&p, sizeof(Stats)) == cudaSuccess ? p : nullptr;
}

void pinned_stats_put(Stats *p)
{
  if (!p) return;
  std::lock_guard<std::mutex> g(g_pool_mu);
  g_pinned_stats.push_back(p);
}

void live_add(int dev)
{
  if (dev < 0 || dev >= kMaxDevices) return;
  std::lock_guard<std::mutex> g(g_pool_mu);
  g_live[dev]++;
}

// one hierarchy fewer; true for the device's last one
bool live_remove(int dev)
{
  if (dev < 0 || dev >= kMaxDevices) return false;
  std::lock_guard<std::mutex> g(g_pool_mu);
  return --g_live[dev] == 0;
}

// the pool's unused memory back to the device
void pool_trim(int dev)
{
  cudaMemPool_t pool = device_pool(dev);
  if (pool) cudaMemPoolTrimTo(pool, 0);
}

// Host copy of one transfer: its jobs, their block prefix and the device copy.
struct Transfer {
  std::vector<XferJob> jobs;
  long long blocks = 0;
  long long row_blocks = 0;         // blocks of the row kernel (k_xfer_rows)
  long long pair_blocks = 0;        // blocks of the pair kernel (k_prolong_correct)
  int width = 0;                    // kernel variant (xfer_width of the jobs)
  bool rows = false;                // run on k_xfer_rows
  bool strided = false;             // every job is a strided copy
  XferJob *d_jobs = nullptr;
};

}  // namespace

struct olgpu_hierarchy {
  olgpu_problem P{};
  hierarchy_geometry G;
  int device = 0;
  int equation = 0;
  // Bowen-York (four unknowns): the variable u holds now (0..2 V1..V3, 3
  // lambda) and V1, V2, V3 as solved (3 x total_pts, the arena's layout)
  int by_var = 0;
  double *d_by = nullptr;
  std::vector<DevBox> hboxes;
  long long total_pts = 0;
  DevBox *d_boxes = nullptr;
  double *d_arena = nullptr;
  DevFields F{};
  std::vector<double> hcoords;
  double *d_coords = nullptr;
  std::vector<AxisEntry> htab;
  AxisEntry *d_tab = nullptr;
  // per level k >= 1
  std::vector<Transfer> restrict_u, xfer_w, set_in, prolong_v, ghost_u;
  std::vector<Transfer> ghost_lo;   // cubic ghost fills (the FP32 cycle's correction may use them)
  std::vector<AdmJob> hadm;
  AdmJob *d_adm = nullptr;
  Stats *d_stats = nullptr;
  Stats *h_stats = nullptr;         // pinned
  Stats *d_stats0 = nullptr;        // what DevBox::solve indexes (d_stats alone)
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_cycle = nullptr;   // end of the last enqueued cycle
  double last_ms = 0.0;
  double adm[OLGPU_MAX_BH] = {0};
  int coarse_max_iters = 2000;
  int coarse_ncta = 0;            // blocks of the coarse-solve cluster (0: one block)
  int coarse_bal = 0;             // its slab layout: 1 the balanced one (cslab_begin_bal)
  size_t coarse_cluster_smem = 0;
  double coarse_omega = 1.9;
  double coarse_rtol = 1e-4;
  double eps_solv = 0, eps_coarse = 0;
  int launches = 0;               // kernels emitted while capturing the V-cycle
  // mixed precision (FP32 correction cycle around the FP64 state)
  int precision = OLGPU_PREC_FP64;
  float *d_arena32 = nullptr;
  DevFields32 F32{};
  float2 *d_aq = nullptr;           // (A, 1/(c+u)) colour-packed for the cluster smoother
  std::vector<Transfer> restrict_e, xfer_w32, set_in32, prolong_v32, ghost_e;
  cudaGraphExec_t graph_mixed = nullptr;
  int launches_mixed = 0;
  double last_defect = 0, last_correction = 0;   // parts of the last mixed cycle's norm
  // the last finished cycle: its residual (FP64: the top level's post-
  // smoothing norm; mixed: the finest FP64 defect) and its largest change of
  // u on the fixed points
  double last_res = 0, last_du = 0;
  // smoother norms of every cycle since the solve began: per cycle, levels
  // pre-smoothing norms then levels post-smoothing norms (level 0: the
  // coarsest solve's)
  std::vector<double> norm_hist;
  // every Print_Pre_Cycle / Print_Post_Cycle call of the current solve
  std::vector<olgpu_cycle_event> events;
  // W-cycle: per level k >= 1 FASN's descent (smoothing down to the saved
  // coarse u) and ascent (correction and smoothing), and the coarsest solve,
  // each captured alone so that the host can repeat every level (built on
  // the first W-cycle solve)
  std::vector<cudaGraphExec_t> graph_down, graph_up;
  cudaGraphExec_t graph_coarse = nullptr;
  // Anderson acceleration of the mixed outer iteration
  int anderson_m = kAndDefault;
  // Anderson acceleration of the FP64 cycle (0: the reference's iteration)
  int anderson64_m = 0;
  double *d_and64 = nullptr;            // DU[m], DF[m], fprev (FP64, total_pts each)
  AndersonState *d_and64_state = nullptr;
  double *d_and64_part = nullptr;
  float *d_and = nullptr;               // DU[m], DF[m], fprev (FP32, total_pts each)
  unsigned char *d_pinned = nullptr;    // points the discrete system fixes
  AndersonState *d_and_state = nullptr;
  double *d_and_part = nullptr;         // per-block partial sums of the Anderson fit
  // per level: blocks of the cluster that keeps e resident through all sweeps
  // of the FP32 smoother (0: one launch per colour and sweep) and its shared
  // memory per block
  std::vector<int> sc_ncta;
  std::vector<size_t> sc_smem;
  // per level, bit q: box q of the smoother's box list (level_list order)
  // runs in the cluster launch; the others take one launch per colour
  std::vector<unsigned long long> sc_fit;
  // pre-/post-smoothing sweeps of the FP32 correction cycle (-1: nu1/nu2)
  int inner_nu1 = -1, inner_nu2 = -1;
  int sc_max = 16;   // largest cluster for the FP32 smoother (0: per-colour launches)
  // structural fast paths of the transfers (strided copies, folded full
  // weighting / Set_In operator, fused prolong-and-correct); off only to test
  // them against the plain steps
  bool fast_paths = !std::getenv("OLGPU_XFER_POINTS");
  // smoother launches as programmatic dependents (overlap launch with the
  // previous kernel's tail); off with OLGPU_NO_PDL
  bool pdl = !std::getenv("OLGPU_NO_PDL");
  // the Robin walk as separate face, edge and corner launches (off: one
  // launch of a cluster per box); the two give the same bits
  bool robin_split = std::getenv("OLGPU_ROBIN_SPLIT") != nullptr;
  // FP64 smoother points per thread (1 or 2: OLGPU_SMOOTH_PTS); the same bits
  int smooth_pts = std::getenv("OLGPU_SMOOTH_PTS") && std::atoi(std::getenv("OLGPU_SMOOTH_PTS")) == 2 ? 2 : 1;
  // points of a row a thread in the per-colour FP32 smoother (1, or 2 with
  // OLGPU_SMOOTH32_PTS=2: the same bits, 2-5 % slower with many solves)
  int smooth32_pts = std::getenv("OLGPU_SMOOTH32_PTS") && std::atoi(std::getenv("OLGPU_SMOOTH32_PTS")) == 2 ? 2 : 1;
  // The solves this hierarchy steps: alone, one (itself); a union of solves
  // (olgpu_batch) steps every member's boxes in shared launches, their levels
  // aligned from the top (a member's level k is the union's level k + off).
  struct Member {
    olgpu_hierarchy *h = nullptr;   // the member's own hierarchy (plans, host state)
    int off = 0;                    // the union level of its level 0
    int coarse_box = 0;             // its level-0 box in this box table
    int box_base = 0;               // its first box in this box table
    long long pt_base = 0;          // its first point in this arena
    Stats *d_stats = nullptr;       // its stats (this table's stats[solve])
    AdmJob *d_adm = nullptr;        // its ADM jobs, box indices of this table
    int nadm = 0;
    int coarse_ncta = 0;            // its coarsest solve: cluster blocks, layout and shared memory
    int coarse_bal = 0;
    size_t coarse_smem = 0;
  };
  std::vector<Member> members;
  // union: per level the boxes of the members for which it is not the
  // coarsest level (the fine side of a FASN step); alone, every box
  std::vector<int> fine_count;
  bool is_union = false;
  bool mixed_ready = false;         // FP32 fields, plans and Anderson history are set up
  bool coarse32_clusters = false;   // FP32 coarsest solves may run as clusters (k_coarse32_cluster)
  bool owns_arena = true, owns_arena32 = true, owns_stats = true;
  bool pooled_hstats = false;   // h_stats from the recycled pinned records (one Stats)
  bool live = false;            // counted among the device's live hierarchies
};

namespace {

// A launch's box list: the given boxes (indices into the hierarchy's box
// table) with their block prefix sums.
BoxList box_list(const std::vector<DevBox> &hboxes, const int *boxes, int count,
                 long long (*blocks_of)(const DevBox &))
{
  BoxList L{};
  L.count = count;
  long long acc = 0;
  for (int b = 0; b < count; b++) {
    L.box[b] = boxes[b];
    L.blk[b] = (int)acc;
    acc += blocks_of(hboxes[boxes[b]]);
  }
  L.blk[count] = (int)acc;
  return L;
}

// The boxes of a level a launch covers: alone, all of them; in a union of
// solves, the fine side of a FASN step -- the members for which the level is
// not their coarsest, which come first in the level's boxes -- or, with
// whole, every box of the level (the coarse side of a step, per-level
// passes).
BoxList level_list(const olgpu_hierarchy *h, int level, long long (*blocks_of)(const DevBox &), bool whole = false)
{
  int boxes[kMaxBoxesPerLevel];
  const int n = whole || h->fine_count.empty() ? h->G.boxes_in_level[level] : h->fine_count[level];
  for (int b = 0; b < n; b++) boxes[b] = h->G.first_box[level] + b;
  return box_list(h->hboxes, boxes, n, blocks_of);
}

// The boxes q of level_list(h, level, ...) whose bit q is (set) / is not
// (!set) in mask.
BoxList level_list_mask(const olgpu_hierarchy *h, int level, long long (*blocks_of)(const DevBox &),
                        unsigned long long mask, bool set)
{
  const BoxList A = level_list(h, level, blocks_of);
  int boxes[kMaxBoxesPerLevel];
  int n = 0;
  for (int q = 0; q < A.count; q++)
    if (((mask >> q) & 1ull) == (set ? 1ull : 0ull)) boxes[n++] = A.box[q];
  return box_list(h->hboxes, boxes, n, blocks_of);
}

long long cdiv(long long a, long long b) { return (a + b - 1) / b; }

long long blocks_all(const DevBox &B) { return cdiv((long long)B.n[0] * B.n[1] * B.n[2], kThreads); }

long long blocks_inside(const DevBox &B)
{
  const int b = B.buf;
  return cdiv((long long)(B.n[0] - 2 * b) * (B.n[1] - 2 * b) * (B.n[2] - 2 * b), kThreads);
}

long long blocks_color(const DevBox &B)
{
  const int b = B.buf;
  const int nc = b + 1;   // colours: order/2 + 1 (2 for the order-2 boxes)
  const long long H = (B.n[0] - 2 * b + nc - 1) / nc;
  return cdiv(H * (B.n[1] - 2 * b) * (B.n[2] - 2 * b), kSmoothThreads);
}

long long blocks_color2(const DevBox &B)   // two points of a row per thread
{
  const int b = B.buf;
  const int nc = b + 1;
  const long long H = (B.n[0] - 2 * b + nc - 1) / nc;
  return cdiv((H + 1) / 2 * (B.n[1] - 2 * b) * (B.n[2] - 2 * b), kSmoothThreads);
}

long long blocks_boundary(const DevBox &B)   // every ghost item: face columns, edge points, corners
{
  return cdiv(robin_face_items(B) + robin_edge_items(B) + 8, kThreads);
}

long long blocks_faces(const DevBox &B)
{
  const int b = B.buf;
  long long cols = 0;
  for (int a = 0; a < 3; a++) cols += 2LL * (B.n[(a + 1) % 3] - 2 * b) * (B.n[(a + 2) % 3] - 2 * b);
  return cdiv(cols, kThreads);   // one thread per normal column of each face
}

// The stencil terms of a box descriptor, shared by the hierarchy's boxes and
// the single caller-owned box of olgpu_smooth_box_noalloc: the spacing, 1/dx
// and 1/dx^2 per axis, whether every axis has the same spacing, and the
// diagonal of the order's Laplacian (duLapc2/4/6/8, include/ffunction.h:
// 1310-1313, 1382-1385, 1466-1469, 1521-1524).
void set_box_stencil(DevBox &B, int order, const double d[3])
{
  B.order = order;
  for (int a = 0; a < 3; a++) {
    B.d[a] = d[a];
    B.idx[a] = 1.0 / d[a];
    B.idx2[a] = B.idx[a] * B.idx[a];
  }
  B.iso = B.idx2[0] == B.idx2[1] && B.idx2[1] == B.idx2[2];
  B.lscale = order == 2 ? B.idx2[0] : B.idx2[0] * (1.0 / 12.0);
  const double s = B.idx2[0] + B.idx2[1] + B.idx2[2];
  switch (order) {
  case 2: B.dulap = -2.0 * s; break;
  case 4: B.dulap = -2.5 * s; break;
  case 6: B.dulap = -490 * s * (1.0 / 180); break;
  default: B.dulap = -205 * s / 72.0; break;
  }
}

PunctureParams puncture_params(const olgpu_problem *p)
{
  PunctureParams PP{};
  PP.numbh = p->numbh;
  PP.equation = p->equation;
  PP.ps_case = p->ps_case;
  for (int i = 0; i < p->numbh; i++) {
    PP.mp[i] = p->mp[i]; PP.x[i] = p->x[i]; PP.y[i] = p->y[i]; PP.z[i] = p->z[i];
    PP.px[i] = p->px[i]; PP.py[i] = p->py[i]; PP.pz[i] = p->pz[i];
    PP.sx[i] = p->sx[i]; PP.sy[i] = p->sy[i]; PP.sz[i] = p->sz[i];
  }
  // scalar-field constants (src/elliptic.cc:71-81)
  PP.ps_r0 = p->ps_r0;
  PP.ps_isigma = 1 / p->ps_sigma;
  const double a2 = p->ps_a2;
  PP.ps_phi0 = (a2 * a2 / (1 + a2 * a2)) * p->ps_phi0;
  PP.ps_d1 = M_PI * PP.ps_phi0 * PP.ps_phi0 * PP.ps_isigma * PP.ps_isigma;
  PP.ps_e1 = 1 / (16 * p->ps_a2);
  PP.ps_e2 = 4 * std::sqrt(M_PI / 3);
  PP.ps_de1 = 4 * M_PI * PP.ps_phi0 * PP.ps_phi0 * PP.ps_isigma * PP.ps_isigma;
  return PP;
}

// LagrangePoly (src/interpolation.cc:308-375)
double lagrange_poly(const domain &D, int a, double t, int i, int ni, int nf)
{
  double lp = 1.0;
  const double ti = D.coord(a, i);
  for (int j = ni; j < i; j++) lp *= (t - D.coord(a, j)) / (ti - D.coord(a, j));
  for (int j = i + 1; j <= nf; j++) lp *= (t - D.coord(a, j)) / (ti - D.coord(a, j));
  return lp;
}

// Interpolation table of target axis a for source box S; returns its offset.
int build_axis(olgpu_hierarchy *h, const domain &T, const domain &S, int a, int method, int ord, bool all,
               const domain *mask_fine)
{
  const int off = (int)h->htab.size();
  for (int t = 0; t < T.n[a]; t++) {
    AxisEntry e{};
    const double x = T.coord(a, t);
    if (method == XM_COPY) {
      // Set_In: inside the box's own nb region and the fine box's nb region
      e.sel = S.is_in_nb_axis(a, x) && mask_fine && mask_fine->is_in_nb_axis(a, x);
      e.exact = 1;
      e.node = t;
      e.start = t;
    } else {
      e.sel = all ? S.is_in_axis(a, x) : S.is_in_nb_axis(a, x);
      const int node = S.locate(a, x);
      e.node = node;
      e.exact = dcomp(x, S.coord(a, node));
      if (method == XM_LAGRANGE) {
        int s = ord % 2 == 0 ? node - ord / 2 : node - (ord + 1) / 2;
        if (s < 0) s = 0;
        else if (s + ord >= S.n[a]) s = S.n[a] - ord - 1;
        e.start = s;
        for (int I = 0; I <= ord; I++) e.w[I] = lagrange_poly(S, a, x, s + I, s, s + ord);
        e.lo = 0;
        e.hi = ord;
        int ones = 0, nonzero = 0, at = 0;
        for (int I = 0; I <= ord; I++) {
          if (e.w[I] != 0.0) nonzero++;
          if (e.w[I] == 1.0) { ones++; at = I; }
        }
        if (ones == 1 && nonzero == 1) e.lo = e.hi = at;
      } else {
        const int nn = node == 0 ? 1 : node;
        e.start = nn - 1;
        const double dxf = (x - S.coord(a, nn - 1)) * (1.0 / S.d[a]);
        e.w[0] = 1 - dxf;
        e.w[1] = dxf;
      }
    }
    h->htab.push_back(e);
  }
  return off;
}

void add_region_jobs(Transfer &X, XferJob base, const domain &T, const int sel_lo[3], const int sel_hi[3])
{
  const int b = T.buf;
  const int *n = T.n;
  std::vector<std::pair<std::array<int, 3>, std::array<int, 3>>> regs;
  auto box = [&](int i0, int i1, int j0, int j1, int k0, int k1) {
    regs.push_back({{i0, j0, k0}, {i1, j1, k1}});
  };
  if (base.to_zero || base.iter == IT_ALL) {
    box(0, n[0], 0, n[1], 0, n[2]);
  } else if (base.iter == IT_INSIDE) {
    box(b, n[0] - b, b, n[1] - b, b, n[2] - b);
  } else {   // the ghost shell as six slabs
    box(0, n[0], 0, n[1], 0, b);
    box(0, n[0], 0, n[1], n[2] - b, n[2]);
    box(0, n[0], 0, b, b, n[2] - b);
    box(0, n[0], n[1] - b, n[1], b, n[2] - b);
    box(0, b, b, n[1] - b, b, n[2] - b);
    box(n[0] - b, n[0], b, n[1] - b, b, n[2] - b);
  }
  for (auto &r : regs) {
    XferJob J = base;
    bool empty = false;
    for (int a = 0; a < 3; a++) {
      J.r0[a] = r.first[a];
      J.r1[a] = r.second[a];
      if (!base.to_zero) {
        J.r0[a] = std::max(J.r0[a], sel_lo[a]);
        J.r1[a] = std::min(J.r1[a], sel_hi[a]);
      }
      if (J.r1[a] <= J.r0[a]) empty = true;
    }
    if (empty) continue;
    const long long e0 = J.r1[0] - J.r0[0], e1 = J.r1[1] - J.r0[1], e2 = J.r1[2] - J.r0[2];
    J.blk0 = X.blocks;
    X.blocks += cdiv(e0 * e1 * e2, kThreads);
    // rows for the row kernel: along the longer of x and y
    J.row_axis = e0 >= e1 ? 0 : 1;
    J.rblk0 = X.row_blocks;
    X.row_blocks += cdiv((J.row_axis == 0 ? e1 : e0) * e2, kRowWarps);
    J.pblk0 = X.pair_blocks;
    X.pair_blocks += cdiv(cdiv(e0, 2) * e1 * e2, kThreads);
    X.jobs.push_back(J);
  }
}

// Marks the jobs of X whose every target is selected and coincides with a
// source node that moves by a constant step along each axis (the exact-copy
// branch of the transfer for all of them) as strided copies.
void stride_jobs(const olgpu_hierarchy *h, Transfer &X)
{
  for (XferJob &J : X.jobs) {
    if (J.method != XM_LAGRANGE && J.method != XM_COPY) continue;
    bool ok = true;
    for (int a = 0; a < 3 && ok; a++) {
      const AxisEntry *e = h->htab.data() + J.tab[a];
      const int r0 = J.r0[a], r1 = J.r1[a];
      const int step = r1 - r0 > 1 ? e[r0 + 1].node - e[r0].node : 1;
      for (int t = r0; t < r1 && ok; t++)
        ok = e[t].sel && (J.method == XM_COPY || e[t].exact) && e[t].node == e[r0].node + step * (t - r0);
      J.sstart[a] = e[r0].node;
      J.sstep[a] = step;
    }
    if (ok) J.method = XM_STRIDED;
  }
}

// Marks the linear jobs of X whose axis tables repeat with period two (2:1
// prolongation): every target selected and, along each axis, the entry of
// r0 + 2m + q equal to that of r0 + q with start and node moved by m.  The
// prolong-and-correct kernel then forms the entries instead of loading them.
void periodic_linear_jobs(const olgpu_hierarchy *h, Transfer &X)
{
  for (XferJob &J : X.jobs) {
    if (J.method != XM_LINEAR) continue;
    bool ok = true;
    for (int a = 0; a < 3 && ok; a++) {
      const AxisEntry *e = h->htab.data() + J.tab[a];
      const int r0 = J.r0[a], r1 = J.r1[a];
      for (int q = 0; q < 2; q++) {
        const AxisEntry &b = e[std::min(r0 + q, r1 - 1)];
        J.lstart[a][q] = b.start;
        J.lnode[a][q] = b.node;
        J.lexact[a][q] = b.exact;
        J.lw0[a][q] = b.w[0];
        J.lw1[a][q] = b.w[1];
      }
      for (int t = r0; t < r1 && ok; t++) {
        const int q = (t - r0) & 1, m = (t - r0) >> 1;
        const AxisEntry &b = e[r0 + q];
        ok = e[t].sel && e[t].exact == b.exact && e[t].start == b.start + m && e[t].node == b.node + m &&
             e[t].w[0] == b.w[0] && e[t].w[1] == b.w[1];
      }
    }
    J.lin2 = ok ? 1 : 0;
  }
}

// Transferir(from, sfield, to, tfield, iter, method, ord, all, to_zero):
// every (source box, target box) pair of the two levels.
Transfer make_transfer(olgpu_hierarchy *h, int from, int sfield, int to, int tfield, int iter, int method, int ord,
                       bool all, bool to_zero)
{
  Transfer X;
  const auto &G = h->G;
  for (int sb = 0; sb < G.boxes_in_level[from]; sb++)
    for (int tb = 0; tb < G.boxes_in_level[to]; tb++) {
      const int gs = G.first_box[from] + sb, gt = G.first_box[to] + tb;
      const domain &S = G.boxes[gs], &T = G.boxes[gt];
      XferJob J{};
      J.tbox = gt;
      J.sbox = gs;
      J.tfield = tfield;
      J.sfield = sfield;
      J.method = method;
      J.ord = ord;
      J.to_zero = to_zero;
      J.iter = iter;
      int lo[3], hi[3];
      for (int a = 0; a < 3; a++) {
        J.tab[a] = build_axis(h, T, S, a, method, ord, all, nullptr);
        lo[a] = T.n[a];
        hi[a] = 0;
        for (int t = 0; t < T.n[a]; t++)
          if (h->htab[J.tab[a] + t].sel) {
            lo[a] = std::min(lo[a], t);
            hi[a] = std::max(hi[a], t + 1);
          }
      }
      add_region_jobs(X, J, T, lo, hi);
    }
  if (!std::getenv("OLGPU_XFER_POINTS")) {
    stride_jobs(h, X);
    periodic_linear_jobs(h, X);
  }
  X.width = xfer_width(X.jobs.data(), X.jobs.size());
  X.rows = xfer_rows(X.jobs.data(), X.jobs.size(), X.width) && !std::getenv("OLGPU_XFER_POINTS");
  X.strided = !X.jobs.empty() && std::all_of(X.jobs.begin(), X.jobs.end(),
                                             [](const XferJob &J) { return J.method == XM_STRIDED; });
  return X;
}

// S.Set_In(W, fine box, false) for every coarse box and fine box of level k.
Transfer make_set_in(olgpu_hierarchy *h, int k)
{
  Transfer X;
  const auto &G = h->G;
  for (int cb = 0; cb < G.boxes_in_level[k - 1]; cb++) {
    const int gc = G.first_box[k - 1] + cb;
    const domain &C = G.boxes[gc];
    for (int fb = 0; fb < G.boxes_in_level[k]; fb++) {
      const domain &Fd = G.boxes[G.first_box[k] + fb];
      XferJob J{};
      J.tbox = gc;
      J.sbox = gc;
      J.tfield = F_RHO;
      J.sfield = F_W;
      J.method = XM_COPY;
      J.iter = IT_ALL;
      int lo[3], hi[3];
      for (int a = 0; a < 3; a++) {
        J.tab[a] = build_axis(h, C, C, a, XM_COPY, 0, false, &Fd);
        lo[a] = C.n[a];
        hi[a] = 0;
        for (int t = 0; t < C.n[a]; t++)
          if (h->htab[J.tab[a] + t].sel) {
            lo[a] = std::min(lo[a], t);
            hi[a] = std::max(hi[a], t + 1);
          }
      }
      add_region_jobs(X, J, C, lo, hi);
    }
  }
  if (!std::getenv("OLGPU_XFER_POINTS")) {
    stride_jobs(h, X);
    periodic_linear_jobs(h, X);
  }
  X.width = xfer_width(X.jobs.data(), X.jobs.size());
  X.rows = xfer_rows(X.jobs.data(), X.jobs.size(), X.width) && !std::getenv("OLGPU_XFER_POINTS");
  X.strided = !X.jobs.empty() && std::all_of(X.jobs.begin(), X.jobs.end(),
                                             [](const XferJob &J) { return J.method == XM_STRIDED; });
  return X;
}

// Launches a kernel as a programmatic dependent of the previous work in the
// stream (the kernel waits on griddep_wait() before reading anything).
template <class... KArgs, class... Args>
void launch_pdl(olgpu_hierarchy *h, void (*kern)(KArgs...), unsigned grid, unsigned block, Args... args)
{
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(block, 1, 1);
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = h->pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// Launches a kernel as clusters of `ncta` blocks on the hierarchy's stream.
template <class... KArgs, class... Args>
void launch_clusters(olgpu_hierarchy *h, void (*kern)(KArgs...), unsigned grid, unsigned block, unsigned ncta,
                     Args... args)
{
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(block, 1, 1);
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ncta;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

template <int ORD, int EQ>
void launch_smooth(olgpu_hierarchy *h, int level, int nu, int slot)
{
  const bool two = h->smooth_pts == 2;   // two points of a row per thread
  const BoxList L = level_list(h, level, two ? blocks_color2 : blocks_color);
  const int nb = L.blk[L.count];
  for (int s = 0; s < nu; s++)
    for (int color = 0; color < num_colors<ORD>(); color++) {
      if (two)
        launch_pdl(h, k_smooth_color<ORD, EQ, 2>, (unsigned)nb, (unsigned)kSmoothThreads, L,
                   (const DevBox *)h->d_boxes, h->F, color, h->d_stats0, slot - 2 * level);
      else
        launch_pdl(h, k_smooth_color<ORD, EQ, 1>, (unsigned)nb, (unsigned)kSmoothThreads, L,
                   (const DevBox *)h->d_boxes, h->F, color, h->d_stats0, slot - 2 * level);
      h->launches++;
    }
}

template <int ORD, int EQ>
void launch_apply_op(olgpu_hierarchy *h, int level, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_inside, whole);
  k_apply_op<ORD, EQ><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F);
  h->launches++;
}

template <int ORD>
void launch_robin(olgpu_hierarchy *h, int level, int mode, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_faces, whole);
  if (!h->robin_split) {
    if (mode == 1 || mode == 3) {   // the operator only reads u: every ghost point in one launch
      const BoxList LA = level_list(h, level, blocks_boundary, whole);
      k_robin_all<ORD><<<LA.blk[LA.count], kThreads, 0, h->stream>>>(LA, h->d_boxes, h->F, h->d_coords, mode);
      h->launches++;
      return;
    }
    // the update: the faces over the whole GPU, then edges and corners, a cluster per box
    k_robin_faces<ORD><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F, h->d_coords, mode);
    launch_clusters(h, k_robin_ec_cluster<ORD>, (unsigned)(L.count * kRobinCluster), kThreads, kRobinCluster, L,
                    (const DevBox *)h->d_boxes, h->F, (const double *)h->d_coords, mode);
    h->launches += 2;
    return;
  }
  k_robin_faces<ORD><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F, h->d_coords, mode);
  k_robin_edges_corners<ORD><<<12 * L.count, 64, 0, h->stream>>>(L, h->d_boxes, h->F, h->d_coords, mode, 0);
  k_robin_edges_corners<ORD><<<L.count, 32, 0, h->stream>>>(L, h->d_boxes, h->F, h->d_coords, mode, 1);
  h->launches += 3;
}

void launch_ew(olgpu_hierarchy *h, int level, int op, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_all, whole);
  k_elementwise<<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F, op);
  h->launches++;
}

// Launches k_xfer for plan X on fields F (double or float fields).
template <class V, class Fields>
void launch_xfer(olgpu_hierarchy *h, const Transfer &X, const Fields &F)
{
  if (X.jobs.empty()) return;
  const int nj = (int)X.jobs.size();
  if (X.rows) {
    const unsigned nr = (unsigned)X.row_blocks;
    const int th = 32 * kRowWarps;
    switch (X.width) {
    case 4: k_xfer_rows<V, Fields, 4><<<nr, th, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
    case 6: k_xfer_rows<V, Fields, 6><<<nr, th, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
    case 8: k_xfer_rows<V, Fields, 8><<<nr, th, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
    default: k_xfer_rows<V, Fields, 10><<<nr, th, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
    }
    return;
  }
  const unsigned nb = (unsigned)X.blocks;
  switch (X.width) {
  case 0: k_xfer<V, Fields, 0><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  case 3: k_xfer<V, Fields, 3><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  case 4: k_xfer<V, Fields, 4><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  case 6: k_xfer<V, Fields, 6><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  case 8: k_xfer<V, Fields, 8><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  case 10: k_xfer<V, Fields, 10><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  default: k_xfer<V, Fields, -1><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, F, h->d_tab); break;
  }
}

void launch_transfer(olgpu_hierarchy *h, const Transfer &X)
{
  if (X.jobs.empty()) return;
  launch_xfer<double>(h, X, h->F);
  h->launches++;
}

int level_order(const olgpu_hierarchy *h, int level) { return h->G.boxes[h->G.first_box[level]].order; }

template <int EQ>
void dispatch_smooth(olgpu_hierarchy *h, int level, int nu, int slot)
{
  switch (level_order(h, level)) {
  case 2: launch_smooth<2, EQ>(h, level, nu, slot); break;
  case 4: launch_smooth<4, EQ>(h, level, nu, slot); break;
  case 6: launch_smooth<6, EQ>(h, level, nu, slot); break;
  default: launch_smooth<8, EQ>(h, level, nu, slot); break;
  }
}

template <int EQ>
void dispatch_apply_op(olgpu_hierarchy *h, int level, bool whole = false)
{
  switch (level_order(h, level)) {
  case 2: launch_apply_op<2, EQ>(h, level, whole); break;
  case 4: launch_apply_op<4, EQ>(h, level, whole); break;
  case 6: launch_apply_op<6, EQ>(h, level, whole); break;
  default: launch_apply_op<8, EQ>(h, level, whole); break;
  }
}

void dispatch_robin(olgpu_hierarchy *h, int level, int mode, bool whole = false)
{
  // the Dirichlet condition runs through the same boundary walk: modes 2, 3
  if (h->P.boundary == OLGPU_BC_DIRICHLET) mode += 2;
  if (level_order(h, level) == 2) launch_robin<2>(h, level, mode, whole);
  else launch_robin<4>(h, level, mode, whole);   // orders 4, 6, 8 share dx4 (src/ffunction.cc:197-282)
}

template <int EQ, int NCTA>
cudaError_t launch_coarse_cluster_n(olgpu_hierarchy *h, const olgpu_hierarchy::Member &M)
{
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(NCTA, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = M.coarse_smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = NCTA;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_coarse_cluster<EQ, NCTA>, (const DevBox *)h->d_boxes, M.coarse_box, h->F,
                            (const double *)h->d_coords, h->eps_coarse, h->coarse_max_iters, h->coarse_omega,
                            h->coarse_rtol, &M.d_stats->coarse_norm, &M.d_stats->coarse_iters,
                            &M.d_stats->nan_flag, h->P.boundary == OLGPU_BC_DIRICHLET ? 1 : 0, M.coarse_bal);
}

template <int EQ>
void launch_coarse_cluster(olgpu_hierarchy *h, const olgpu_hierarchy::Member &M)
{
  if (M.coarse_ncta == 16) launch_coarse_cluster_n<EQ, 16>(h, M);
  else launch_coarse_cluster_n<EQ, 8>(h, M);
}

// Largest supported cluster for the coarse solve: 16 blocks (non-portable
// size), else 8, else 0 (one block).
template <int EQ, int NCTA>
bool cluster_fits(olgpu_hierarchy *h, size_t smem)
{
  auto kern = k_coarse_cluster<EQ, NCTA>;
  if (NCTA > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  // the limit is per kernel and process-wide: always the device's maximum,
  // so that a hierarchy with a smaller coarsest grid never lowers it below
  // what another one's captured cycle launches with
  int optin = 0;
  cudaFuncAttributes fa{};
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, (const void *)kern) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const int lim = optin - (int)fa.sharedSizeBytes;   // the dynamic part beside the kernel's static arrays
  if (lim < (int)smem || cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(NCTA, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = NCTA;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n >= 1;
}

// The coarse solve's cluster: of 8 or 16 blocks (non-portable size) in the
// plain or the balanced slab layout, the one whose busiest block has the
// least FP64 work between two barriers -- its interior planes, plus a
// quarter plane for the z-face Robin points of blocks 0 and ncta-1 -- and
// of equal ones the fewer blocks, then the plain layout.  OLGPU_COARSE_BAL=0
// keeps the plain layout.
void choose_coarse_cluster(olgpu_hierarchy *h)
{
  const DevBox &B = h->hboxes[h->G.first_box[0]];
  if (B.n[2] > 64 || B.n[2] < 6 || B.buf != 1) return;
  const int n2 = B.n[2];
  auto work = [&](int ncta, int bal) {
    double m = 0;
    for (int r = 0; r < ncta; r++) {
      const int a = std::max(cslab_at(r, n2, ncta, bal), 1), b = std::min(cslab_at(r + 1, n2, ncta, bal), n2 - 1);
      m = std::max(m, (b > a ? b - a : 0) + (r == 0 || r == ncta - 1 ? 0.25 : 0.0));
    }
    return m;
  };
  const char *bal_env = std::getenv("OLGPU_COARSE_BAL");
  const bool allow_bal = !(bal_env && std::atoi(bal_env) == 0);
  struct Cand {
    int ncta, bal;
    double w;
  };
  std::vector<Cand> cands;
  for (int ncta : {8, 16})
    for (int bal : {0, 1})
      if (!bal || allow_bal) cands.push_back({ncta, bal, work(ncta, bal)});
  std::stable_sort(cands.begin(), cands.end(), [](const Cand &x, const Cand &y) { return x.w < y.w; });
  for (const Cand &c : cands) {
    int planes = 0;
    for (int r = 0; r < c.ncta; r++)
      planes = std::max(planes, cslab_at(r + 1, n2, c.ncta, c.bal) - cslab_at(r, n2, c.ncta, c.bal));
    const size_t smem = sizeof(double) * (size_t)planes * B.n[0] * B.n[1];
    const bool ok = c.ncta == 16 ? (cluster_fits<0, 16>(h, smem) && cluster_fits<1, 16>(h, smem) &&
                                    cluster_fits<2, 16>(h, smem))
                                 : (cluster_fits<0, 8>(h, smem) && cluster_fits<1, 8>(h, smem) &&
                                    cluster_fits<2, 8>(h, smem));
    if (ok) {
      h->coarse_ncta = c.ncta;
      h->coarse_bal = c.bal;
      h->coarse_cluster_smem = smem;
      return;
    }
  }
}

// FASN's descent on level k (src/elliptic.cc:1518-1775): boundary and
// pre-smoothing, u restricted, the coarse level's source with tau, the
// coarse u saved in ww
template <int EQ>
void emit_fasn_down(olgpu_hierarchy *h, int k)
{
  const int mg = h->G.mgrid_levels;
  if (k <= mg) dispatch_robin(h, k, 0);
  dispatch_smooth<EQ>(h, k, h->P.nu1, 2 * k);
  launch_transfer(h, h->restrict_u[k]);
  // on a refinement level the coarse operator is only needed where Set_In
  // copies (k_set_in_op forms it there)
  const bool fold_set_in = k > mg && h->set_in[k].strided;
  if (!fold_set_in) dispatch_apply_op<EQ>(h, k - 1, true);
  if (k <= mg) dispatch_robin(h, k - 1, 1, true);
  dispatch_apply_op<EQ>(h, k);
  if (k <= mg) dispatch_robin(h, k, 1);
  launch_ew(h, k, EW_W_EQ_S_MINUS_R);
  if (h->xfer_w[k].strided) {   // full weighting folded into the transfer
    const Transfer &X = h->xfer_w[k];
    k_xfer_fw<double, DevFields, false><<<(unsigned)X.blocks, kThreads, 0, h->stream>>>(
        X.d_jobs, (int)X.jobs.size(), h->d_boxes, h->F, F_W, F_W);
    h->launches++;
  } else {
    const BoxList L = level_list(h, k, blocks_all);
    k_full_weight<<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F);
    h->launches++;
    launch_transfer(h, h->xfer_w[k]);
  }
  if (k <= mg) {
    launch_ew(h, k - 1, EW_S_EQ_W_PLUS_R, true);
  } else if (fold_set_in) {
    const Transfer &X = h->set_in[k];
    const unsigned nb = (unsigned)X.blocks;
    const int nj = (int)X.jobs.size();
    switch (level_order(h, k - 1)) {
    case 2: k_set_in_op<2, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F); break;
    case 4: k_set_in_op<4, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F); break;
    case 6: k_set_in_op<6, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F); break;
    default: k_set_in_op<8, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F); break;
    }
    h->launches++;
  } else {
    launch_ew(h, k - 1, EW_W_PLUS_EQ_R, true);
    launch_transfer(h, h->set_in[k]);
  }
  launch_ew(h, k - 1, EW_WW_EQ_U, true);
}

// the coarsest solve (src/elliptic.cc:1782-1816)
template <int EQ>
void emit_coarse(olgpu_hierarchy *h, const olgpu_hierarchy::Member &M)
{
  const DevBox &B = h->hboxes[M.coarse_box];
  const size_t smem = sizeof(double) * (size_t)B.n[0] * B.n[1] * B.n[2];
  if (M.coarse_ncta > 0)
    launch_coarse_cluster<EQ>(h, M);
  else
    k_coarse_solve<EQ><<<1, 1024, smem, h->stream>>>(h->d_boxes, M.coarse_box, h->F, h->d_coords,
                                                     h->eps_coarse, h->coarse_max_iters, h->coarse_omega,
                                                     h->coarse_rtol, &M.d_stats->coarse_norm,
                                                     &M.d_stats->coarse_iters, &M.d_stats->nan_flag,
                                                     h->P.boundary == OLGPU_BC_DIRICHLET ? 1 : 0);
  h->launches++;
}

// The correction of a refinement level's INSIDE points and the ghost fill of
// its BOUNDARY points in one launch (k_prolong_ghost), when both plans take
// their fast forms; returns false (nothing launched) otherwise.
template <class V, class Fields>
bool launch_prolong_ghost(olgpu_hierarchy *h, const Transfer &Pv, const Transfer &Gh, const Fields &F, int fe, int fww)
{
  if (!h->fast_paths || Pv.jobs.empty() || Gh.jobs.empty() || !Gh.rows) return false;
  const unsigned nb = (unsigned)((Pv.pair_blocks + 1) / 2 + Gh.row_blocks);
  const int np = (int)Pv.jobs.size(), ng = (int)Gh.jobs.size();
  const unsigned th = 32 * kRowWarps;
  switch (Gh.width) {
  case 4: k_prolong_ghost<V, Fields, 4><<<nb, th, 0, h->stream>>>(Pv.d_jobs, np, Pv.pair_blocks, Gh.d_jobs, ng,
                                                                  h->d_boxes, F, h->d_tab, fe, fww); break;
  case 6: k_prolong_ghost<V, Fields, 6><<<nb, th, 0, h->stream>>>(Pv.d_jobs, np, Pv.pair_blocks, Gh.d_jobs, ng,
                                                                  h->d_boxes, F, h->d_tab, fe, fww); break;
  case 8: k_prolong_ghost<V, Fields, 8><<<nb, th, 0, h->stream>>>(Pv.d_jobs, np, Pv.pair_blocks, Gh.d_jobs, ng,
                                                                  h->d_boxes, F, h->d_tab, fe, fww); break;
  default: k_prolong_ghost<V, Fields, 10><<<nb, th, 0, h->stream>>>(Pv.d_jobs, np, Pv.pair_blocks, Gh.d_jobs, ng,
                                                                    h->d_boxes, F, h->d_tab, fe, fww); break;
  }
  return true;
}

// FASN's ascent on level k (src/elliptic.cc:1827-1941): the coarse
// correction prolonged and added, ghosts refilled, boundary and
// post-smoothing, the ADM integrand on the top level
template <int EQ>
void emit_fasn_up(olgpu_hierarchy *h, int k, int top)
{
  const int mg = h->G.mgrid_levels;
  if (k > mg && launch_prolong_ghost<double>(h, h->prolong_v[k], h->ghost_u[k], h->F, F_U, F_WW)) {
    h->launches++;   // correction and ghost fill of a refinement level in one launch
  } else {
    if (h->fast_paths) {   // u_fine += P(u - ww) in one pass
      const Transfer &X = h->prolong_v[k];
      if (!X.jobs.empty()) {
        k_prolong_correct<double, DevFields><<<(unsigned)X.pair_blocks, kThreads, 0, h->stream>>>(
            X.d_jobs, (int)X.jobs.size(), h->d_boxes, h->F, h->d_tab, F_U, F_WW);
        h->launches++;
      }
    } else {
      launch_ew(h, k - 1, EW_V_EQ_U_MINUS_WW, true);
      launch_transfer(h, h->prolong_v[k]);
      launch_ew(h, k, EW_U_PLUS_EQ_V);
    }
    if (k > mg) launch_transfer(h, h->ghost_u[k]);
  }
  if (k <= mg) dispatch_robin(h, k, 0);
  dispatch_smooth<EQ>(h, k, h->P.nu2, 2 * k + 1);
  if (k == top && h->anderson64_m == 0)   // with FP64 acceleration: after the update
    for (const auto &M : h->members)
      if (M.nadm > 0) {
        k_adm<<<1, 32, 0, h->stream>>>(M.d_adm, M.nadm, h->d_boxes, h->F, M.d_stats->adm_u);
        h->launches++;
      }
}

// elliptic::FASN with Wcycle = false (src/elliptic.cc:1468-1968)
template <int EQ>
// (a union: a member whose coarsest level is k - 1 solves it there, the
// others descend further)
void emit_fasn(olgpu_hierarchy *h, int k, int top)
{
  emit_fasn_down<EQ>(h, k);
  bool deeper = false;
  for (const auto &M : h->members) {
    if (M.off == k - 1) emit_coarse<EQ>(h, M);
    else if (M.off < k - 1) deeper = true;
  }
  if (deeper) emit_fasn<EQ>(h, k - 1, top);
  emit_fasn_up<EQ>(h, k, top);
}

// The cycle's largest change of u on the points the discrete system fixes:
// u as the cycle finds it is copied to F_UP first, max |u - up| ends the
// cycle.  With the residual it bounds how far u still is from the fixed
// point (OLGPU_STOP_ERROR).
void emit_du_begin(olgpu_hierarchy *h)
{
  cudaMemcpyAsync(h->F.f[F_UP], h->F.f[F_U], sizeof(double) * (size_t)h->total_pts, cudaMemcpyDeviceToDevice,
                  h->stream);
}

int emit_du_end(olgpu_hierarchy *h)
{
  for (const auto &M : h->members)   // each solve's own points and slot
    k_du_max<<<152 * 4, kThreads, 0, h->stream>>>(M.h->total_pts, h->F.f[F_U] + M.pt_base, h->F.f[F_UP] + M.pt_base,
                                                  M.h->d_pinned, &M.d_stats->slots[kSlotDu],
                                                  (const DevBox *)h->d_boxes + M.box_base);
  return (int)h->members.size();
}

// ---------------------------------------------------------------------------
// mixed precision: FP64 preparation, FP32 correction cycle, FP64 update
// ---------------------------------------------------------------------------
void launch_transfer32(olgpu_hierarchy *h, const Transfer &X)
{
  if (X.jobs.empty()) return;
  launch_xfer<float>(h, X, h->F32);
  h->launches_mixed++;
}

void launch_ew32(olgpu_hierarchy *h, int level, int op, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_all, whole);
  k_elementwise32<<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F32, op);
  h->launches_mixed++;
}

template <int ORD, int EQ>
void launch_mx_defect(olgpu_hierarchy *h, int level, int slot)
{
  const BoxList L = level_list(h, level, blocks_all);
  k_mx_defect<ORD, EQ><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F, h->F32, h->d_stats0, slot);
  h->launches_mixed++;
}

template <int EQ>
void dispatch_mx_defect(olgpu_hierarchy *h, int level, int slot)
{
  switch (level_order(h, level)) {
  case 2: launch_mx_defect<2, EQ>(h, level, slot); break;
  case 4: launch_mx_defect<4, EQ>(h, level, slot); break;
  case 6: launch_mx_defect<6, EQ>(h, level, slot); break;
  default: launch_mx_defect<8, EQ>(h, level, slot); break;
  }
}

template <int ORD, int EQ>
void launch_smooth32(olgpu_hierarchy *h, const BoxList &L, int nu)
{
  if (L.count == 0) return;
  for (int s = 0; s < nu; s++)
    for (int color = 0; color < num_colors<ORD>(); color++) {
      if (h->smooth32_pts == 2)
        launch_pdl(h, k_smooth32<ORD, EQ, 2>, (unsigned)L.blk[L.count], (unsigned)kSmoothThreads, L,
                   (const DevBox *)h->d_boxes, h->F32, (const float2 *)h->d_aq, color, h->d_stats0);
      else
        launch_pdl(h, k_smooth32<ORD, EQ, 1>, (unsigned)L.blk[L.count], (unsigned)kSmoothThreads, L,
                   (const DevBox *)h->d_boxes, h->F32, (const float2 *)h->d_aq, color, h->d_stats0);
      h->launches_mixed++;
    }
}

template <int ORD, int EQ>
void launch_apply_op32(olgpu_hierarchy *h, int level, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_inside, whole);
  k_apply_op32<ORD, EQ><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F32);
  h->launches_mixed++;
}

template <int ORD, int EQ>
void launch_smooth32_cluster(olgpu_hierarchy *h, int level, int nu)
{
  const int ncta = h->sc_ncta[level];
  // one cluster per box of the list that fits one
  const BoxList L = level_list_mask(h, level, blocks_all, h->sc_fit[level], true);
  if (L.count == 0) return;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(ncta * L.count), 1, 1);
  cfg.blockDim = dim3(kSmoothClusterThreads, 1, 1);
  cfg.dynamicSmemBytes = h->sc_smem[level];
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ncta;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_smooth32_cluster<ORD, EQ>, (const DevBox *)h->d_boxes, L, h->F32,
                     (const float2 *)h->d_aq, nu, h->d_stats0);
  h->launches_mixed++;
}

// Whether a cluster of ncta blocks of `threads` threads with `smem` bytes of
// dynamic shared memory each can be resident for kernel `kern`; also raises
// the kernel's shared-memory limit to the device's opt-in maximum.
bool cluster_launchable(const void *kern, int ncta, int threads, size_t smem)
{
  cudaFuncAttributes fa{};
  int dev = 0, optin = 0;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const size_t limit = (size_t)optin - fa.sharedSizeBytes;
  if (smem > limit) return false;
  if ((ncta > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) ||
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(ncta, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ncta;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n >= 1;
}

const void *smooth32_cluster_kernel(int ord, int eq)
{
  switch (ord) {
  case 2: return eq ? (const void *)k_smooth32_cluster<2, 1> : (const void *)k_smooth32_cluster<2, 0>;
  case 4: return eq ? (const void *)k_smooth32_cluster<4, 1> : (const void *)k_smooth32_cluster<4, 0>;
  case 6: return eq ? (const void *)k_smooth32_cluster<6, 1> : (const void *)k_smooth32_cluster<6, 0>;
  default: return eq ? (const void *)k_smooth32_cluster<8, 1> : (const void *)k_smooth32_cluster<8, 0>;
  }
}

// Per level: the cluster that keeps e resident through the FP32 smoother, or
// none.  A box fits a cluster of ncta blocks when its ghost band is at least
// as wide as the stencil's reach, it has at most kMaxClusterPlanes planes and
// one interior plane per block, and its largest slab fits in a block's
// shared memory.  The cluster is used when every box of the level fits it:
// splitting a level (the boxes that fit in a cluster launch, the others in
// per-colour launches after it on the same stream) was measured 4 % slower
// on the batched binaries, whose union levels put the largest problems'
// boxes beside smaller ones (the cluster launch, on a few SMs, lengthens
// the level's chain).  Of the sizes 8..16 whose largest share of interior
// planes is smallest (the critical path between two barriers), the fewest
// blocks are taken: the other SMs stay free for other work.
void choose_smooth_clusters(olgpu_hierarchy *h)
{
  const int L = h->G.levels;
  h->sc_ncta.assign(L, 0);
  h->sc_smem.assign(L, 0);
  h->sc_fit.assign(L, 0ull);
  if (std::getenv("OLGPU_SMOOTH32_LAUNCHES") || h->sc_max < 8) return;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  for (int l = 0; l < L; l++) {
    const int ord = level_order(h, l);
    const void *kern = smooth32_cluster_kernel(ord, h->equation);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    const size_t limit = (size_t)optin - fa.sharedSizeBytes;
    const BoxList FL = level_list(h, l, blocks_all);   // the boxes the smoother runs on
    int best = 0, best_share = 1 << 30;
    long long best_pts = 0;
    size_t best_smem = 0;
    unsigned long long best_fit = 0ull;
    for (int ncta = std::min(h->sc_max, 16); ncta >= 8; ncta--) {
      size_t smem = 0;
      int share = 0;
      long long pts = 0;
      unsigned long long fit = 0ull;
      for (int q = 0; q < FL.count; q++) {
        const DevBox &B = h->hboxes[FL.box[q]];
        const int m2 = B.n[2] - 2 * B.buf;
        if (m2 < ncta || B.n[2] > kMaxClusterPlanes || B.buf < ord / 2 || B.order != ord) continue;
        const size_t sb = sizeof(float) * (size_t)slab_max_planes(B.n[2], B.buf, ncta) * B.n[0] * B.n[1];
        if (sb > limit) continue;
        fit |= 1ull << q;
        share = std::max(share, (m2 + ncta - 1) / ncta);
        smem = std::max(smem, sb);
        pts += (long long)(B.n[0] - 2 * B.buf) * (B.n[1] - 2 * B.buf) * m2;
      }
      const unsigned long long all = FL.count >= 64 ? ~0ull : (1ull << FL.count) - 1;
      if (fit != all || FL.count == 0 || pts < best_pts || (pts == best_pts && share > best_share)) continue;
      if (!cluster_launchable(kern, ncta, kSmoothClusterThreads, smem)) continue;
      best = ncta;
      best_share = share;
      best_smem = smem;
      best_pts = pts;
      best_fit = fit;
    }
    h->sc_ncta[l] = best;
    h->sc_smem[l] = best_smem;
    h->sc_fit[l] = best_fit;
    if (std::getenv("OLGPU_VERBOSE"))
      std::fprintf(stderr, "olgpu: level %d FP32 smoother: %d of %d boxes cluster-resident (%d blocks, %zu B shared "
                   "memory per block)\n", l, __builtin_popcountll(best_fit), FL.count, best, best_smem);
  }
}

template <int EQ>
void dispatch_smooth32(olgpu_hierarchy *h, int level, int nu)
{
  if (nu <= 0) return;
  const unsigned long long fit = h->sc_ncta[level] > 0 ? h->sc_fit[level] : 0ull;
  if (fit) {
    switch (level_order(h, level)) {
    case 2: launch_smooth32_cluster<2, EQ>(h, level, nu); break;
    case 4: launch_smooth32_cluster<4, EQ>(h, level, nu); break;
    case 6: launch_smooth32_cluster<6, EQ>(h, level, nu); break;
    default: launch_smooth32_cluster<8, EQ>(h, level, nu); break;
    }
  }
  // the boxes no cluster holds: one launch per colour and sweep
  const BoxList R = level_list_mask(h, level, h->smooth32_pts == 2 ? blocks_color2 : blocks_color, fit, false);
  switch (level_order(h, level)) {
  case 2: launch_smooth32<2, EQ>(h, R, nu); break;
  case 4: launch_smooth32<4, EQ>(h, R, nu); break;
  case 6: launch_smooth32<6, EQ>(h, R, nu); break;
  default: launch_smooth32<8, EQ>(h, R, nu); break;
  }
}

template <int EQ>
void dispatch_apply_op32(olgpu_hierarchy *h, int level, bool whole = false)
{
  switch (level_order(h, level)) {
  case 2: launch_apply_op32<2, EQ>(h, level, whole); break;
  case 4: launch_apply_op32<4, EQ>(h, level, whole); break;
  case 6: launch_apply_op32<6, EQ>(h, level, whole); break;
  default: launch_apply_op32<8, EQ>(h, level, whole); break;
  }
}

template <int ORD>
void launch_robin32(olgpu_hierarchy *h, int level, int mode, bool whole = false)
{
  const BoxList L = level_list(h, level, blocks_faces, whole);
  if (!h->robin_split) {
    if (mode == 1) {   // the operator only reads e: every ghost point in one launch
      const BoxList LA = level_list(h, level, blocks_boundary, whole);
      k_robin32_all<ORD><<<LA.blk[LA.count], kThreads, 0, h->stream>>>(LA, h->d_boxes, h->F32, h->d_coords, mode);
      h->launches_mixed++;
      return;
    }
    k_robin32_faces<ORD><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F32, h->d_coords, mode);
    launch_clusters(h, k_robin32_ec_cluster<ORD>, (unsigned)(L.count * kRobinCluster), kThreads, kRobinCluster, L,
                    (const DevBox *)h->d_boxes, h->F32, (const double *)h->d_coords, mode);
    h->launches_mixed += 2;
    return;
  }
  k_robin32_faces<ORD><<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F32, h->d_coords, mode);
  k_robin32_edges_corners<ORD><<<12 * L.count, 64, 0, h->stream>>>(L, h->d_boxes, h->F32, h->d_coords, mode, 0);
  k_robin32_edges_corners<ORD><<<L.count, 32, 0, h->stream>>>(L, h->d_boxes, h->F32, h->d_coords, mode, 1);
  h->launches_mixed += 3;
}

void dispatch_robin32(olgpu_hierarchy *h, int level, int mode, bool whole = false)
{
  if (level_order(h, level) == 2) launch_robin32<2>(h, level, mode, whole);
  else launch_robin32<4>(h, level, mode, whole);
}

// Whether k_coarse32_cluster<EQ> runs here: its shared-memory limit set (the
// same for every hierarchy, so that none lowers it below what another's
// captured cycle launches with) and one cluster resident.
template <int EQ>
bool coarse32_cluster_fits()
{
  auto kern = k_coarse32_cluster<EQ, kCoarse32Ncta>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCoarse32ClusterSmem) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(kCoarse32Ncta, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = kCoarse32ClusterSmem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCoarse32Ncta;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n >= 1;
}

// Shared memory of a block of k_coarse32_cluster for a coarsest box, or 0
// where the kernel does not take it (one ghost layer, 6..64 planes, rows of
// at most 64 points, arrays within kCoarse32ClusterSmem).
size_t coarse32_cluster_smem(const DevBox &B, int eq)
{
  if (B.buf != 1 || B.n[2] < 6 || B.n[0] > 64 || B.n[1] > 64 || B.n[2] > 64) return 0;
  const size_t bytes =
      sizeof(float) * (size_t)coarse32_cluster_slab(B.n[0], B.n[1], B.n[2], kCoarse32Ncta) * (eq == 1 ? 6 : 4);
  return bytes <= kCoarse32ClusterSmem ? bytes : 0;
}

template <int EQ>
void emit_fasn32(olgpu_hierarchy *h, int k)
{
  const int mg = h->G.mgrid_levels;
  if (k <= mg) dispatch_robin32(h, k, 0);
  dispatch_smooth32<EQ>(h, k, h->inner_nu1 >= 0 ? h->inner_nu1 : h->P.nu1);
  launch_transfer32(h, h->restrict_e[k]);
  // on a refinement level the coarse operator is only needed where Set_In
  // copies (k_set_in_op32 forms it there)
  const bool fold_set_in = k > mg && h->set_in32[k].strided;
  if (!fold_set_in) dispatch_apply_op32<EQ>(h, k - 1, true);
  if (k <= mg) dispatch_robin32(h, k - 1, 1, true);
  dispatch_apply_op32<EQ>(h, k);
  if (k <= mg) dispatch_robin32(h, k, 1);
  if (h->xfer_w32[k].strided) {   // full weighting of S - R folded into the transfer
    const Transfer &X = h->xfer_w32[k];
    k_xfer_fw<float, DevFields32, true><<<(unsigned)X.blocks, kThreads, 0, h->stream>>>(
        X.d_jobs, (int)X.jobs.size(), h->d_boxes, h->F32, G_S, G_R);
    h->launches_mixed++;
  } else {
    const BoxList L = level_list(h, k, blocks_all);
    k_full_weight32<<<L.blk[L.count], kThreads, 0, h->stream>>>(L, h->d_boxes, h->F32);
    h->launches_mixed++;
    launch_transfer32(h, h->xfer_w32[k]);
  }
  if (k <= mg) {
    launch_ew32(h, k - 1, EW32_S_EQ_W_PLUS_R_WW_EQ_E, true);
  } else if (fold_set_in) {
    launch_ew32(h, k - 1, EW32_WW_EQ_E, true);
    const Transfer &X = h->set_in32[k];
    const unsigned nb = (unsigned)X.blocks;
    const int nj = (int)X.jobs.size();
    switch (level_order(h, k - 1)) {
    case 2: k_set_in_op32<2, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F32); break;
    case 4: k_set_in_op32<4, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F32); break;
    case 6: k_set_in_op32<6, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F32); break;
    default: k_set_in_op32<8, EQ><<<nb, kThreads, 0, h->stream>>>(X.d_jobs, nj, h->d_boxes, h->F32); break;
    }
    h->launches_mixed++;
  } else {
    launch_ew32(h, k - 1, EW32_W_PLUS_EQ_R_WW_EQ_E, true);   // WW = E: nothing writes E before set_in
    launch_transfer32(h, h->set_in32[k]);
  }
  // a union: members whose coarsest level is k - 1 solve it, side by side:
  // one launch of a cluster per box for the boxes k_coarse32_cluster takes,
  // one of a block per box for those whose coefficients fit in shared memory
  // beside e, one for the others; the other members descend
  bool deeper = false;
  BoxList Ls{}, Lg{}, Lc{};
  size_t smem_s = 0, smem_g = 0, smem_c = 0;
  auto flush_cluster = [&]() {   // one cluster of kCoarse32Ncta blocks per box
    if (Lc.count == 0) return;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(Lc.count * kCoarse32Ncta), 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = smem_c;
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kCoarse32Ncta;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_coarse32_cluster<EQ, kCoarse32Ncta>, (const DevBox *)h->d_boxes, Lc, h->F32,
                       (const double *)h->d_coords, h->coarse_max_iters, (float)h->coarse_omega, 1e-4f,
                       h->d_stats0);
    h->launches_mixed++;
    Lc.count = 0;
    smem_c = 0;
  };
  auto flush = [&](BoxList &BL, size_t smem, bool staged_coeffs) {
    if (BL.count == 0) return;
    if (staged_coeffs)
      k_coarse32<EQ, true><<<BL.count, 1024, smem, h->stream>>>(h->d_boxes, BL, h->F32, h->d_coords,
                                                                 h->coarse_max_iters, (float)h->coarse_omega, 1e-4f,
                                                                 h->d_stats0);
    else
      k_coarse32<EQ, false><<<BL.count, 1024, smem, h->stream>>>(h->d_boxes, BL, h->F32, h->d_coords,
                                                                  h->coarse_max_iters, (float)h->coarse_omega, 1e-4f,
                                                                  h->d_stats0);
    h->launches_mixed++;
    BL.count = 0;
  };
  for (const auto &M : h->members) {
    if (M.off != k - 1) {
      deeper = deeper || M.off < k - 1;
      continue;
    }
    const DevBox &B = h->hboxes[M.coarse_box];
    const size_t csm = h->coarse32_clusters ? coarse32_cluster_smem(B, EQ) : 0;
    if (csm > 0) {   // every box the cluster kernel takes runs there, alone or in a batch
      Lc.box[Lc.count++] = M.coarse_box;
      smem_c = std::max(smem_c, csm);
      if (Lc.count == kMaxBoxesPerLevel) flush_cluster();
      continue;
    }
    const size_t np = (size_t)B.n[0] * B.n[1] * B.n[2];
    const size_t staged = sizeof(float) * np * (EQ == 1 ? 6 : 4);
    const bool st = staged <= kCoarseSmemMax;
    BoxList &BL = st ? Ls : Lg;
    size_t &sm = st ? smem_s : smem_g;
    BL.box[BL.count++] = M.coarse_box;
    sm = std::max(sm, st ? staged : sizeof(float) * np);
    if (BL.count == kMaxBoxesPerLevel) flush(BL, sm, st);
  }
  flush(Ls, smem_s, true);
  flush(Lg, smem_g, false);
  flush_cluster();
  if (deeper) emit_fasn32<EQ>(h, k - 1);
  if (k > mg && launch_prolong_ghost<float>(h, h->prolong_v32[k], h->ghost_e[k], h->F32, G_E, G_WW)) {
    h->launches_mixed++;
  } else {
    if (h->fast_paths) {   // e_fine += P(e - ww) in one pass
      const Transfer &X = h->prolong_v32[k];
      if (!X.jobs.empty()) {
        k_prolong_correct<float, DevFields32><<<(unsigned)X.pair_blocks, kThreads, 0, h->stream>>>(
            X.d_jobs, (int)X.jobs.size(), h->d_boxes, h->F32, h->d_tab, G_E, G_WW);
        h->launches_mixed++;
      }
    } else {
      launch_ew32(h, k - 1, EW32_V_EQ_E_MINUS_WW, true);
      launch_transfer32(h, h->prolong_v32[k]);
      launch_ew32(h, k, EW32_E_PLUS_EQ_V);
    }
    if (k > mg) launch_transfer32(h, h->ghost_e[k]);
  }
  if (k <= mg) dispatch_robin32(h, k, 0);
  dispatch_smooth32<EQ>(h, k, h->inner_nu2 >= 0 ? h->inner_nu2 : h->P.nu2);
}

template <int EQ>
void emit_mixed_cycle(olgpu_hierarchy *h)
{
  const int L = h->G.levels, top = L - 1, mg = h->G.mgrid_levels;
  // FP64: restrict u top-down and refill refinement ghosts bottom-up, so that
  // the FP32 cycle's transfers of e are exact corrections of those of u
  const int fp64_before = h->launches;
  for (int k = top; k >= 1; k--) launch_transfer(h, h->restrict_u[k]);
  for (int k = mg + 1; k <= top; k++) launch_transfer(h, h->ghost_u[k]);
  h->launches_mixed += h->launches - fp64_before;
  h->launches = fp64_before;
  // FP64: coefficients of the correction operator and the defect source
  for (int l = 0; l < L; l++) {
    const BoxList BL = level_list(h, l, blocks_all, true);
    // the cluster smoother reads (A, 1/(c+u)) colour-packed
    float2 *aq = h->d_aq;   // both FP32 smoothers read the colour-packed copy
    switch (level_order(h, l)) {
    case 2: k_mx_prep<2, EQ><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, aq); break;
    case 4: k_mx_prep<4, EQ><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, aq); break;
    case 6: k_mx_prep<6, EQ><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, aq); break;
    default: k_mx_prep<8, EQ><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, aq); break;
    }
    if (l <= mg) {
      if (level_order(h, l) == 2)
        k_mx_robin_defect<2><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, h->d_coords);
      else
        k_mx_robin_defect<4><<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, h->d_coords);
      h->launches_mixed++;
    }
    h->launches_mixed++;
  }
  const size_t n32 = sizeof(float) * (size_t)h->total_pts;
  for (int f : {G_E, G_R, G_V})
    if (f != G_V || !h->fast_paths) cudaMemsetAsync(h->F32.f[f], 0, n32, h->stream);
  // FP32 correction V-cycle
  emit_fasn32<EQ>(h, top);
  // FP64 update and the FP64 defect of the finest level as the cycle's norm
  if (h->anderson_m > 0) {
    for (const auto &M : h->members) {   // each solve's own history, points and slot
      const olgpu_hierarchy *m = M.h;
      const long long n = m->total_pts;
      float *DU = m->d_and, *DF = m->d_and + (size_t)kAndMax * n, *fprev = m->d_and + (size_t)2 * kAndMax * n;
      const DevBox *gate = (const DevBox *)h->d_boxes + M.box_base;
      const int nblk = 152 * 4;
      k_and_reduce<<<nblk, kThreads, 0, h->stream>>>(n, h->F32.f[G_E] + M.pt_base, fprev, DF, m->d_pinned,
                                                      m->d_and_state, m->d_and_part, &M.d_stats->slots[kSlotCorr],
                                                      gate);
      k_and_solve<<<1, 32 * kAndSolveWarps, 0, h->stream>>>(m->d_and_state, m->d_and_part, nblk, gate);
      k_and_update<<<nblk, kThreads, 0, h->stream>>>(n, h->F.f[F_U] + M.pt_base, h->F32.f[G_E] + M.pt_base, DU, DF,
                                                      m->d_and_state, gate);
      h->launches_mixed += 3;
    }
  } else {
    for (int l = 0; l < L; l++) {
      const BoxList BL = level_list(h, l, blocks_all, true);
      k_mx_update<<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->F32, h->d_stats0);
      h->launches_mixed++;
    }
  }
  dispatch_mx_defect<EQ>(h, top, kSlotDefect);
  for (const auto &M : h->members)
    if (M.nadm > 0) {
      k_adm<<<1, 32, 0, h->stream>>>(M.d_adm, M.nadm, h->d_boxes, h->F, M.d_stats->adm_u);
      h->launches_mixed++;
    }
}

Transfer remap(const Transfer &X, int sfield, int tfield)
{
  Transfer Y;
  Y.jobs = X.jobs;
  Y.blocks = X.blocks;
  Y.width = X.width;
  Y.rows = X.rows;
  Y.strided = X.strided;
  Y.row_blocks = X.row_blocks;
  Y.pair_blocks = X.pair_blocks;
  for (auto &J : Y.jobs) {
    J.sfield = sfield;
    J.tfield = tfield;
  }
  return Y;
}

olgpu_status reset_anderson(olgpu_hierarchy *h)
{
  if (h->d_and_state) {
    AndersonState st{};
    st.m = h->anderson_m > 0 ? h->anderson_m : 1;
    CUDA_TRY(cudaMemcpyAsync(h->d_and_state, &st, sizeof(st), cudaMemcpyHostToDevice, h->stream));
  }
  if (h->d_and64_state) {
    AndersonState st{};
    st.m = h->anderson64_m > 0 ? h->anderson64_m : 1;
    CUDA_TRY(cudaMemcpyAsync(h->d_and64_state, &st, sizeof(st), cudaMemcpyHostToDevice, h->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return OLGPU_OK;
}

// FP64 acceleration of the FP64 cycle after its last kernel: each solve's
// mixing over its own points, then its ADM integrand from the mixed u.
void emit_anderson64(olgpu_hierarchy *h)
{
  for (const auto &M : h->members) {
    const olgpu_hierarchy *m = M.h;
    const long long n = m->total_pts;
    double *DU = m->d_and64, *DF = m->d_and64 + (size_t)kAndMax * n, *fprev = m->d_and64 + (size_t)2 * kAndMax * n;
    const DevBox *gate = (const DevBox *)h->d_boxes + M.box_base;
    double *u = h->F.f[F_U] + M.pt_base;
    const double *up = h->F.f[F_UP] + M.pt_base;
    const int nblk = 152 * 4;
    k_and_reduce64<<<nblk, kThreads, 0, h->stream>>>(n, u, up, fprev, DF, m->d_pinned, m->d_and64_state,
                                                      m->d_and64_part, &M.d_stats->slots[kSlotCorr], gate);
    k_and_solve<<<1, 32 * kAndSolveWarps, 0, h->stream>>>(m->d_and64_state, m->d_and64_part, nblk, gate);
    k_and_update64<<<nblk, kThreads, 0, h->stream>>>(n, u, up, DU, DF, m->d_and64_state, gate);
    h->launches += 3;
    if (M.nadm > 0) {
      k_adm<<<1, 32, 0, h->stream>>>(M.d_adm, M.nadm, h->d_boxes, h->F, M.d_stats->adm_u);
      h->launches++;
    }
  }
}

olgpu_status capture_mixed(olgpu_hierarchy *h);

// Allocates the FP32 fields and plans and captures the mixed cycle (once).
// The FP32 fields, plans and Anderson history of the mixed cycle (once).  A
// union's member gets arena32 (its FP32 field g at arena32 + g * stride +
// base, inside the union's arena) and keeps only its Anderson history; the
// union itself has no history of its own (each member's is used).
olgpu_status prepare_mixed(olgpu_hierarchy *h, float *arena32, long long stride, long long base)
{
  if (h->mixed_ready) return OLGPU_OK;
  const bool member = arena32 != nullptr;
  if (!member) {
    const size_t bytes = sizeof(float) * (size_t)h->total_pts * G_NUM;
    if (dev_alloc((void **)&h->d_arena32, bytes, h->device, h->stream) != cudaSuccess ||
        dev_alloc((void **)&h->d_aq, sizeof(float2) * (size_t)h->total_pts, h->device, h->stream) != cudaSuccess)
      return fail(OLGPU_ERR_OOM, "FP32 arena allocation failed");
    CUDA_TRY(cudaMemsetAsync(h->d_arena32, 0, bytes, h->stream));
    arena32 = h->d_arena32;
    stride = h->total_pts;
    base = 0;
  } else {
    h->owns_arena32 = false;
  }
  for (int f = 0; f < G_NUM; f++) h->F32.f[f] = arena32 + (size_t)f * stride + base;
  const int L = h->G.levels;
  h->restrict_e.resize(L);
  h->xfer_w32.resize(L);
  h->set_in32.resize(L);
  h->prolong_v32.resize(L);
  h->ghost_e.resize(L);
  for (int k = 1; k < L; k++) {
    h->restrict_e[k] = remap(h->restrict_u[k], G_E, G_E);
    h->xfer_w32[k] = remap(h->xfer_w[k], G_T, G_W);
    h->set_in32[k] = remap(h->set_in[k], G_W, G_S);
    h->prolong_v32[k] = remap(h->prolong_v[k], G_V, G_V);
    // the correction's ghosts: cubic Lagrange (the FP64 ghosts of u keep order+1)
    h->ghost_e[k] = remap(h->ghost_lo[k], G_E, G_E);
  }
  for (auto *vec : {&h->restrict_e, &h->xfer_w32, &h->set_in32, &h->prolong_v32, &h->ghost_e})
    for (auto &X : *vec) {
      if (X.jobs.empty() || member) continue;   // a member's FP32 steps run in the union's plans
      if (dev_alloc((void **)&X.d_jobs, sizeof(XferJob) * X.jobs.size(), h->device, h->stream) != cudaSuccess)
        return fail(OLGPU_ERR_OOM, "transfer plan allocation failed");
      CUDA_TRY(cudaMemcpyAsync(X.d_jobs, X.jobs.data(), sizeof(XferJob) * X.jobs.size(), cudaMemcpyHostToDevice,
                               h->stream));
    }
  if (!h->is_union) {
    const size_t n = (size_t)h->total_pts;
    if (dev_alloc((void **)&h->d_and, sizeof(float) * n * (2 * kAndMax + 1), h->device, h->stream) != cudaSuccess ||
        dev_alloc((void **)&h->d_and_state, sizeof(AndersonState), h->device, h->stream) != cudaSuccess ||
        dev_alloc((void **)&h->d_and_part, sizeof(double) * 152 * 4 * kAndPart, h->device, h->stream) !=
            cudaSuccess)
      return fail(OLGPU_ERR_OOM, "Anderson history allocation failed");
    CUDA_TRY(cudaMemsetAsync(h->d_and, 0, sizeof(float) * n * (2 * kAndMax + 1), h->stream));
    olgpu_status st = reset_anderson(h);
    if (st != OLGPU_OK) return st;
  }
  for (const void *kern : {(const void *)k_coarse32<0, true>, (const void *)k_coarse32<1, true>,
                           (const void *)k_coarse32<0, false>, (const void *)k_coarse32<1, false>})
    CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCoarseSmemMax));
  if (!member) {
    choose_smooth_clusters(h);
    h->coarse32_clusters =
        !std::getenv("OLGPU_COARSE32_ONE_BLOCK") && coarse32_cluster_fits<0>() && coarse32_cluster_fits<1>();
  }
  h->mixed_ready = true;
  return OLGPU_OK;
}

// Prepares and captures the mixed cycle (once).
olgpu_status build_mixed(olgpu_hierarchy *h)
{
  if (h->graph_mixed) return OLGPU_OK;
  olgpu_status st = prepare_mixed(h, nullptr, 0, 0);
  return st != OLGPU_OK ? st : capture_mixed(h);
}

// Captures the mixed cycle into h->graph_mixed (replacing an earlier one).
olgpu_status capture_mixed(olgpu_hierarchy *h)
{
  if (h->graph_mixed) {
    CUDA_TRY(cudaGraphExecDestroy(h->graph_mixed));
    h->graph_mixed = nullptr;
  }
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(h->d_stats, 0, sizeof(Stats) * h->members.size(), h->stream);   // a union: every member's
  h->launches_mixed = 0;
  emit_du_begin(h);
  if (h->equation == 1) emit_mixed_cycle<1>(h);
  else emit_mixed_cycle<0>(h);
  h->launches_mixed += emit_du_end(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("mixed graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph_mixed, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("mixed graph instantiate: ") + cudaGetErrorString(e));
  return OLGPU_OK;
}

olgpu_status build_graph(olgpu_hierarchy *h)
{
  const int top = h->G.levels - 1;
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(h->d_stats, 0, sizeof(Stats) * h->members.size(), h->stream);   // a union: every member's
  h->launches = 0;
  emit_du_begin(h);
  if (h->equation == 1) emit_fasn<1>(h, top, top);
  else if (h->equation >= 2) emit_fasn<2>(h, top, top);   // the test equations share one operator
  else emit_fasn<0>(h, top, top);
  if (h->anderson64_m > 0) emit_anderson64(h);
  h->launches += emit_du_end(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return OLGPU_OK;
}

// Captures what emit() enqueues on the hierarchy's stream as one graph.
template <class Emit>
olgpu_status capture_piece(olgpu_hierarchy *h, Emit emit, cudaGraphExec_t *out, const char *what)
{
  cudaGraph_t g;
  CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  emit();
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string(what) + " capture: " + cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string(what) + " instantiate: " + cudaGetErrorString(e));
  return OLGPU_OK;
}

template <int EQ>
olgpu_status build_wgraphs_eq(olgpu_hierarchy *h)
{
  const int top = h->G.levels - 1;
  const int saved = h->launches;   // the V-cycle's kernel count stays the reported one
  for (auto *vec : {&h->graph_down, &h->graph_up})   // pieces of an earlier attempt that failed
    for (cudaGraphExec_t g : *vec)
      if (g) cudaGraphExecDestroy(g);
  h->graph_down.assign(top + 1, nullptr);
  h->graph_up.assign(top + 1, nullptr);
  olgpu_status st = OLGPU_OK;
  for (int k = 1; k <= top && st == OLGPU_OK; k++) {
    unsigned long long *pre = &h->d_stats->slots[2 * k], *post = &h->d_stats->slots[2 * k + 1];
    st = capture_piece(h, [&] {
      cudaMemsetAsync(pre, 0, sizeof(*pre), h->stream);   // the smoother max-reduces into its slot
      emit_fasn_down<EQ>(h, k);
    }, &h->graph_down[k], "W-cycle descent");
    if (st != OLGPU_OK) break;
    st = capture_piece(h, [&] {
      cudaMemsetAsync(post, 0, sizeof(*post), h->stream);
      emit_fasn_up<EQ>(h, k, top);
    }, &h->graph_up[k], "W-cycle ascent");
  }
  if (st == OLGPU_OK)
    st = capture_piece(h, [&] { emit_coarse<EQ>(h, h->members[0]); }, &h->graph_coarse, "W-cycle coarse solve");
  h->launches = saved;
  return st;
}

olgpu_status build_wgraphs(olgpu_hierarchy *h)
{
  if (h->graph_coarse) return OLGPU_OK;
  if (h->equation == 1) return build_wgraphs_eq<1>(h);
  if (h->equation >= 2) return build_wgraphs_eq<2>(h);
  return build_wgraphs_eq<0>(h);
}

int field_id(const char *name)
{
  static const char *names[F_NUM] = {"u", "b", "c", "d", "e", "rho", "r", "w", "ww", "v", "t", "up"};
  if (!name) return -1;
  for (int f = 0; f < F_NUM; f++)
    if (!std::strcmp(name, names[f])) return f;
  return -1;
}

double elapsed_ms(cudaEvent_t a, cudaEvent_t b)
{
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char *olgpu_last_error(void) { return g_last_error.c_str(); }
const char *olgpu_version(void)
{
  return "olgpu 0.3 (sm_103a, FP64 FAS; FP32/FP64 mixed precision; Robin and Dirichlet boundaries; point gather; "
         "continuous-batching server)";
}

void olgpu_problem_defaults(olgpu_problem *p)
{
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->equation = OLGPU_EQ_PUNCTURES;
  p->numbh = 1;
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

static void fill_box_info(const domain &D, olgpu_box_info *o)
{
  o->level = D.level;
  o->nx = D.n[0];
  o->ny = D.n[1];
  o->nz = D.n[2];
  o->buf = D.buf;
  o->order = D.order;
  o->xi = D.lo[0];
  o->yi = D.lo[1];
  o->zi = D.lo[2];
  o->dx = D.d[0];
  o->dy = D.d[1];
  o->dz = D.d[2];
  o->cx = D.c[0];
  o->cy = D.c[1];
  o->cz = D.c[2];
  o->xf = D.hi[0];
  o->yf = D.hi[1];
  o->zf = D.hi[2];
}

// domain::Fix_Points (src/domain.cc:574-1388): the 8 corner blocks, the 12
// edge blocks, the 6 face blocks and the interior, each a triple loop whose
// axes run over the low ghost band inward-out (b-1 .. 0), the high band
// (n-b .. n-1) or the interior (b .. n-b-1).  One row per block: the
// outer, middle and inner axis, and the band of x, y, z (L, H, I).
olgpu_status olgpu_storage_order(const olgpu_box_info *box, long long *out)
{
  if (!box || !out) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  struct Block {
    int axis[3];    // loop axes, outer to inner (0 = x, 1 = y, 2 = z)
    char band[4];   // band of x, y, z
  };
  static const Block blocks[27] = {
      {{2, 1, 0}, "LLL"}, {{2, 1, 0}, "LLH"}, {{2, 1, 0}, "HLL"}, {{2, 1, 0}, "HLH"},   // corners
      {{2, 1, 0}, "LHL"}, {{2, 1, 0}, "LHH"}, {{2, 1, 0}, "HHL"}, {{2, 1, 0}, "HHH"},
      {{0, 1, 2}, "LLI"}, {{0, 1, 2}, "LHI"}, {{0, 1, 2}, "HLI"}, {{0, 1, 2}, "HHI"},   // edges along z
      {{0, 2, 1}, "LIL"}, {{0, 2, 1}, "LIH"}, {{0, 2, 1}, "HIL"}, {{0, 2, 1}, "HIH"},   // edges along y
      {{2, 1, 0}, "ILL"}, {{2, 1, 0}, "ILH"}, {{2, 1, 0}, "IHL"}, {{2, 1, 0}, "IHH"},   // edges along x
      {{0, 2, 1}, "LII"}, {{0, 2, 1}, "HII"}, {{1, 2, 0}, "ILI"}, {{1, 2, 0}, "IHI"},   // faces
      {{2, 1, 0}, "IIL"}, {{2, 1, 0}, "IIH"},
      {{2, 1, 0}, "III"}};                                                               // interior
  const int n[3] = {box->nx, box->ny, box->nz}, b = box->buf;
  for (int a = 0; a < 3; a++)
    if (n[a] < 2 * b + 1 || b < 1) return fail(OLGPU_ERR_INVALID_ARG, "box smaller than its ghost bands");
  // the values an axis takes in a band, in loop order
  auto band = [&](int a, char c, std::vector<int> &v) {
    v.clear();
    if (c == 'L')
      for (int t = b - 1; t >= 0; t--) v.push_back(t);
    else if (c == 'H')
      for (int t = n[a] - b; t < n[a]; t++) v.push_back(t);
    else
      for (int t = b; t < n[a] - b; t++) v.push_back(t);
  };
  long long q = 0;
  std::vector<int> r[3];
  for (const Block &B : blocks) {
    for (int a = 0; a < 3; a++) band(a, B.band[a], r[a]);
    const int A0 = B.axis[0], A1 = B.axis[1], A2 = B.axis[2];
    int ijk[3];
    for (int v0 : r[A0]) {
      ijk[A0] = v0;
      for (int v1 : r[A1]) {
        ijk[A1] = v1;
        for (int v2 : r[A2]) {
          ijk[A2] = v2;
          out[q++] = ((long long)ijk[2] * n[1] + ijk[1]) * n[0] + ijk[0];
        }
      }
    }
  }
  return OLGPU_OK;
}

olgpu_status olgpu_plan_boxes(const olgpu_problem *p, olgpu_box_info *out, int cap, int *nboxes, int *nlevels,
                              int *mgrid_levels)
{
  if (!p) return fail(OLGPU_ERR_INVALID_ARG, "null problem");
  if (p->numbh < 1 || p->numbh > OLGPU_MAX_BH) return fail(OLGPU_ERR_INVALID_ARG, "numbh out of range 1..16");
  if (!(p->order == 2 || p->order == 4 || p->order == 6 || p->order == 8))
    return fail(OLGPU_ERR_INVALID_ARG, "order must be 2, 4, 6 or 8");
  if (p->levels < 1) return fail(OLGPU_ERR_INVALID_ARG, "levels must be >= 1");
  hierarchy_geometry G;
  puncture_set bh{p->numbh, p->x, p->y, p->z};
  if (!set_grids(p->n, p->L, p->order, p->levels, bh, G))
    return fail(OLGPU_ERR_GEOMETRY, "not enough grid points for multigrid");
  if (nboxes) *nboxes = (int)G.boxes.size();
  if (nlevels) *nlevels = G.levels;
  if (mgrid_levels) *mgrid_levels = G.mgrid_levels;
  if (out)
    for (int g = 0; g < (int)G.boxes.size() && g < cap; g++) fill_box_info(G.boxes[g], &out[g]);
  return OLGPU_OK;
}

// The problem's parameters are ones the solver takes.
static olgpu_status validate_problem(const olgpu_problem *p)
{
  if (p->numbh < 1 || p->numbh > OLGPU_MAX_BH) return fail(OLGPU_ERR_INVALID_ARG, "numbh out of range 1..16");
  if (!(p->order == 2 || p->order == 4 || p->order == 6 || p->order == 8))
    return fail(OLGPU_ERR_INVALID_ARG, "order must be 2, 4, 6 or 8");
  if (p->levels < 1) return fail(OLGPU_ERR_INVALID_ARG, "levels must be >= 1");
  if (p->nu1 < 0 || p->nu2 < 0) return fail(OLGPU_ERR_INVALID_ARG, "negative sweep count");
  if (p->equation < 0 || p->equation > OLGPU_EQ_BOWEN_YORK) return fail(OLGPU_ERR_INVALID_ARG, "unknown equation");
  if (p->equation == OLGPU_EQ_MULTIBOX_TEST && p->numbh < 2)
    return fail(OLGPU_ERR_INVALID_ARG, "the multibox test takes its two centres from bhx1 and bhx2");
  if (p->boundary != OLGPU_BC_ROBIN && p->boundary != OLGPU_BC_DIRICHLET)
    return fail(OLGPU_ERR_INVALID_ARG, "boundary must be Robin or Dirichlet");
  if (p->method != OLGPU_METHOD_VCYCLE && p->method != OLGPU_METHOD_WCYCLE)
    return fail(OLGPU_ERR_INVALID_ARG, "method must be Vcycle or Wcycle");
  if (p->equation == 1 && !(p->ps_case >= 1 && p->ps_case <= 4))
    return fail(OLGPU_ERR_INVALID_ARG, "ps_case must be 1..4");
  return OLGPU_OK;
}

// Host planning of a hierarchy: the geometry (elliptic::Set_Grids), the box
// table, the coordinate tables, every transfer plan and the ADM jobs.
// Nothing on the device yet.
static olgpu_status plan_hierarchy(const olgpu_problem *p, olgpu_hierarchy *h)
{
  h->P = *p;
  h->equation = p->equation;
  CUDA_TRY(cudaGetDevice(&h->device));
  h->eps_coarse = 2 * 2.220446049250313e-16;
  h->eps_solv = p->tol < h->eps_coarse ? h->eps_coarse : p->tol;
  puncture_set bh{p->numbh, p->x, p->y, p->z};
  if (!set_grids(p->n, p->L, p->order, p->levels, bh, h->G)) {
    return fail(OLGPU_ERR_GEOMETRY, "not enough grid points for multigrid");
  }
  if (h->G.levels > 60) {   // norm slots 0..119 (2 a level); 120..127 hold the cycle's other norms
    return fail(OLGPU_ERR_INVALID_ARG, "too many levels");
  }
  for (int l = 0; l < h->G.levels; l++)
    if (h->G.boxes_in_level[l] > kMaxBoxesPerLevel) {
        return fail(OLGPU_ERR_INVALID_ARG, "too many boxes on one level");
    }
  // device box table and coordinate tables
  long long off = 0;
  int coff = 0;
  for (const domain &D : h->G.boxes) {
    DevBox B{};
    for (int a = 0; a < 3; a++) B.n[a] = D.n[a];
    B.buf = D.buf;
    B.level = D.level;
    B.off = off;
    B.coord_off = coff;
    B.solve = 0;
    B.active = 1;
    B.mg_coarse = D.level < h->G.mgrid_levels ? 1 : 0;
    B.falloff = h->equation == OLGPU_EQ_BOWEN_YORK ? 2 : 1;   // src/operator.cc:789, 1393-1399
    set_box_stencil(B, D.order, D.d);
    // x, y, z of the box's nodes, then their reciprocals (ghost nodes lie on
    // the outer faces; a node at 0 gets 0, it is never a Robin point)
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < D.n[a]; i++) h->hcoords.push_back(D.coord(a, i));
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < D.n[a]; i++) {
        const double x = D.coord(a, i);
        h->hcoords.push_back(x != 0.0 ? 1.0 / x : 0.0);
      }
    coff += 2 * (D.n[0] + D.n[1] + D.n[2]);
    off += D.npts();
    h->hboxes.push_back(B);
  }
  h->total_pts = off;
  // transfer plans for every level k >= 1 (FASN steps 2, 5, 6, 10, 12)
  const int L = h->G.levels, mg = h->G.mgrid_levels, order = p->order;
  h->restrict_u.resize(L);
  h->xfer_w.resize(L);
  h->set_in.resize(L);
  h->prolong_v.resize(L);
  h->ghost_u.resize(L);
  h->ghost_lo.resize(L);
  for (int k = 1; k < L; k++) {
    h->restrict_u[k] = make_transfer(h, k, F_U, k - 1, F_U, IT_INSIDE, XM_LAGRANGE, 3, false, false);
    h->xfer_w[k] = make_transfer(h, k, F_T, k - 1, F_W, IT_ALL, XM_LAGRANGE, 2, k - 1 <= mg, false);
    if (k > mg) h->set_in[k] = make_set_in(h, k);
    if (k <= mg)
      h->prolong_v[k] = make_transfer(h, k - 1, F_V, k, F_V, IT_ALL, XM_LINEAR, 1, true, true);
    else
      h->prolong_v[k] = make_transfer(h, k - 1, F_V, k, F_V, IT_INSIDE, XM_LINEAR, 1, true, false);
    if (k > mg) h->ghost_u[k] = make_transfer(h, k - 1, F_U, k, F_U, IT_BOUNDARY, XM_LAGRANGE, order + 1, true, false);
    if (k > mg) h->ghost_lo[k] = make_transfer(h, k - 1, F_U, k, F_U, IT_BOUNDARY, XM_LAGRANGE, 3, true, false);
  }
  // ADM: 4th-order Lagrange at each puncture on finest box i (box 0 if absent)
  {
    const int top = L - 1;
    for (int i = 0; i < p->numbh; i++) {
      const int g = h->G.first_box[top] + (i < h->G.boxes_in_level[top] ? i : 0);
      const domain &S = h->G.boxes[g];
      AdmJob J{};
      J.box = g;
      const double pt[3] = {p->x[i], p->y[i], p->z[i]};
      int ex = 1;
      for (int a = 0; a < 3; a++) {
        const int node = S.locate(a, pt[a]);
        J.node[a] = node;
        ex = ex && dcomp(pt[a], S.coord(a, node));
        int s = node - 2;
        if (s < 0) s = 0;
        else if (s + 4 >= S.n[a]) s = S.n[a] - 5;
        J.start[a] = s;
        for (int I = 0; I <= 4; I++) J.w[a][I] = lagrange_poly(S, a, pt[a], s + I, s, s + 4);
      }
      J.exact = ex;
      h->hadm.push_back(J);
    }
  }
  return OLGPU_OK;
}

// Device set-up of a planned hierarchy: stream and events, the field arena
// (its own when arena is NULL, else field f at arena + f * stride + base),
// the tables and plans, the stats (its own when stats is NULL), the
// coefficients and initial state, and (capture) its captured V-cycle.
static olgpu_status setup_device(olgpu_hierarchy *h, double *arena, long long stride, long long base, Stats *stats,
                                 Stats *hstats, bool capture)
{
  olgpu_status st = OLGPU_OK;
  auto cleanup = [&](olgpu_status s) { return s; };   // the caller destroys h
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_cycle, cudaEventDisableTiming) != cudaSuccess)
    return cleanup(fail(OLGPU_ERR_CUDA, "stream/event creation failed"));
  live_add(h->device);
  h->live = true;
  cudaError_t e = cudaSuccess;
  if (!arena) {   // its own arena
    e = dev_alloc((void **)&h->d_arena, sizeof(double) * (size_t)h->total_pts * F_NUM, h->device, h->stream);
    if (e != cudaSuccess) return cleanup(fail(OLGPU_ERR_OOM, "device arena allocation failed"));
    arena = h->d_arena;
    stride = h->total_pts;
    base = 0;
  } else {
    h->owns_arena = false;
  }
  for (int f = 0; f < F_NUM; f++) h->F.f[f] = arena + (size_t)f * stride + base;
  if (h->equation != 1) h->F.f[F_D] = h->F.f[F_E] = nullptr;
  auto up = [&](void **dst, const void *src, size_t bytes) -> bool {
    if (bytes == 0) return true;
    if (dev_alloc(dst, bytes, h->device, h->stream) != cudaSuccess) return false;
    return cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, h->stream) == cudaSuccess;
  };
  bool ok = up((void **)&h->d_boxes, h->hboxes.data(), sizeof(DevBox) * h->hboxes.size()) &&
            up((void **)&h->d_coords, h->hcoords.data(), sizeof(double) * h->hcoords.size()) &&
            up((void **)&h->d_tab, h->htab.data(), sizeof(AxisEntry) * h->htab.size()) &&
            up((void **)&h->d_adm, h->hadm.data(), sizeof(AdmJob) * h->hadm.size());
  for (auto *vec : {&h->restrict_u, &h->xfer_w, &h->set_in, &h->prolong_v, &h->ghost_u, &h->ghost_lo})
    for (auto &X : *vec)
      ok = ok && up((void **)&X.d_jobs, X.jobs.data(), sizeof(XferJob) * X.jobs.size());
  if (stats) {   // a member of a union: its stats are the union's
    h->owns_stats = false;
    h->d_stats = stats;
    h->h_stats = hstats;
  } else {
    ok = ok && dev_alloc((void **)&h->d_stats, sizeof(Stats), h->device, h->stream) == cudaSuccess &&
         (h->h_stats = pinned_stats_get()) != nullptr;
    h->pooled_hstats = true;
  }
  h->d_stats0 = h->d_stats;
  if (!ok) return cleanup(fail(OLGPU_ERR_OOM, "device allocation failed"));
  // the points the discrete system fixes: every point of the solution levels,
  // the INSIDE points of the multigrid coarse levels (their ghost layers keep
  // whatever the iteration leaves there once W vanishes)
  {
    std::vector<unsigned char> pin((size_t)h->total_pts, 1);
    for (const DevBox &B : h->hboxes) {
      if (B.level >= h->G.mgrid_levels) continue;
      for (int k = 0; k < B.n[2]; k++)
        for (int j = 0; j < B.n[1]; j++)
          for (int i = 0; i < B.n[0]; i++) {
            const bool in = i >= B.buf && i < B.n[0] - B.buf && j >= B.buf && j < B.n[1] - B.buf && k >= B.buf &&
                            k < B.n[2] - B.buf;
            if (!in) pin[B.off + ((size_t)k * B.n[1] + j) * B.n[0] + i] = 0;
          }
    }
    if (!up((void **)&h->d_pinned, pin.data(), pin.size()))
      return cleanup(fail(OLGPU_ERR_OOM, "device allocation failed"));
  }
  // coarsest box must fit in shared memory
  {
    const DevBox &B0 = h->hboxes[h->G.first_box[0]];
    const size_t smem = sizeof(double) * (size_t)B0.n[0] * B0.n[1] * B0.n[2];
    if (smem > kCoarseSmemMax || B0.n[0] > 64 || B0.n[1] > 64 || B0.n[2] > 64)
      return cleanup(fail(OLGPU_ERR_INVALID_ARG, "coarsest grid too large"));
    // the limit is per kernel and process-wide: always the same maximum, so
    // hierarchies with different coarse grids never lower it for each other
    const int lim = (int)kCoarseSmemMax;
    cudaError_t e1 = cudaFuncSetAttribute(k_coarse_solve<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaError_t e2 = cudaFuncSetAttribute(k_coarse_solve<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaError_t e3 = cudaFuncSetAttribute(k_coarse_solve<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess)
      return cleanup(fail(OLGPU_ERR_CUDA, "shared memory opt-in failed"));
  }
  if (!std::getenv("OLGPU_COARSE_ONE_BLOCK")) choose_coarse_cluster(h);
  // coarsest-solve tuning knobs (over-relaxation, relative stop): they change
  // the work per cycle and how well the coarse problem is solved, not the
  // fixed point of the cycle
  if (const char *v = std::getenv("OLGPU_COARSE_OMEGA")) h->coarse_omega = std::atof(v);
  if (const char *v = std::getenv("OLGPU_COARSE_RTOL")) h->coarse_rtol = std::atof(v);
  if (h->equation == OLGPU_EQ_BOWEN_YORK &&
      dev_alloc((void **)&h->d_by, sizeof(double) * 3 * (size_t)h->total_pts, h->device, h->stream) != cudaSuccess)
    return cleanup(fail(OLGPU_ERR_OOM, "Bowen-York variable allocation failed"));
  st = olgpu_reset(h);
  if (st != OLGPU_OK) return cleanup(st);
  // coefficients on the device
  {
    const PunctureParams PP = puncture_params(&h->P);
    for (int l = 0; l < h->G.levels; l++) {
      const BoxList BL = level_list(h, l, blocks_all, true);
      k_coefficients<<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->d_coords, PP);
    }
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cleanup(fail(OLGPU_ERR_CUDA, std::string("coefficients: ") + cudaGetErrorString(e)));
  }
  h->members.assign(1, olgpu_hierarchy::Member{});
  {
    olgpu_hierarchy::Member &M = h->members[0];
    M.h = h;
    M.off = 0;
    M.coarse_box = h->G.first_box[0];
    M.box_base = 0;
    M.pt_base = 0;
    M.d_stats = h->d_stats;
    M.d_adm = h->d_adm;
    M.nadm = (int)h->hadm.size();
    M.coarse_ncta = h->coarse_ncta;
    M.coarse_bal = h->coarse_bal;
    M.coarse_smem = h->coarse_cluster_smem;
  }
  if (capture) {
    st = build_graph(h);
    if (st != OLGPU_OK) return cleanup(st);
  }
  return OLGPU_OK;
}


olgpu_status olgpu_hierarchy_create(const olgpu_problem *p, int device, olgpu_hierarchy **out)
{
  if (!p || !out) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  olgpu_status st = validate_problem(p);
  if (st != OLGPU_OK) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(OLGPU_ERR_NO_DEVICE, "no CUDA device");
  if (device >= 0) CUDA_TRY(cudaSetDevice(device));

  auto *h = new olgpu_hierarchy();
  const auto t0 = std::chrono::steady_clock::now();
  st = plan_hierarchy(p, h);
  const auto t1 = std::chrono::steady_clock::now();
  if (st == OLGPU_OK) st = setup_device(h, nullptr, 0, 0, nullptr, nullptr, true);
  if (std::getenv("OLGPU_VERBOSE")) {
    const auto t2 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "olgpu: hierarchy of %lld points: plan %.1f ms, device set-up and capture %.1f ms\n",
                 h->total_pts, std::chrono::duration<double, std::milli>(t1 - t0).count(),
                 std::chrono::duration<double, std::milli>(t2 - t1).count());
  }
  if (st != OLGPU_OK) {
    olgpu_hierarchy_destroy(h);
    return st;
  }
  *out = h;
  return OLGPU_OK;
}

olgpu_status olgpu_hierarchy_destroy(olgpu_hierarchy *h)
{
  if (!h) return OLGPU_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->graph_mixed) cudaGraphExecDestroy(h->graph_mixed);
  for (auto *vec : {&h->graph_down, &h->graph_up})
    for (cudaGraphExec_t g : *vec)
      if (g) cudaGraphExecDestroy(g);
  if (h->graph_coarse) cudaGraphExecDestroy(h->graph_coarse);
  // device memory back to the pool in the stream's order (no device-wide wait)
  cudaStream_t s = h->stream;
  for (auto *vec : {&h->restrict_e, &h->xfer_w32, &h->set_in32, &h->prolong_v32, &h->ghost_e})
    for (auto &X : *vec) dev_free(X.d_jobs, s);
  if (h->owns_arena32) dev_free(h->d_arena32, s);
  dev_free(h->d_aq, s);
  dev_free(h->d_and, s);
  dev_free(h->d_pinned, s);
  dev_free(h->d_and_state, s);
  dev_free(h->d_and_part, s);
  dev_free(h->d_and64, s);
  dev_free(h->d_and64_state, s);
  dev_free(h->d_and64_part, s);
  dev_free(h->d_by, s);
  for (auto *vec : {&h->restrict_u, &h->xfer_w, &h->set_in, &h->prolong_v, &h->ghost_u, &h->ghost_lo})
    for (auto &X : *vec) dev_free(X.d_jobs, s);
  if (h->owns_arena) dev_free(h->d_arena, s);
  dev_free(h->d_boxes, s);
  dev_free(h->d_coords, s);
  dev_free(h->d_tab, s);
  dev_free(h->d_adm, s);
  if (h->is_union)   // a union owns its members and their ADM job copies
    for (auto &M : h->members) {
      dev_free(M.d_adm, s);
      olgpu_hierarchy_destroy(M.h);
    }
  if (h->owns_stats) {
    dev_free(h->d_stats, s);
    if (h->pooled_hstats)
      pinned_stats_put(h->h_stats);
    else if (h->h_stats)
      cudaFreeHost(h->h_stats);
  }
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_cycle) cudaEventDestroy(h->ev_cycle);
  // the frees complete before the stream goes: a completed free is what the
  // pool hands to the next allocation on any stream (a pending one on a
  // destroyed stream would leave the pool growing instead)
  if (s) cudaStreamSynchronize(s);
  if (h->live && live_remove(h->device)) pool_trim(h->device);   // the last one: the pool gives its memory back
  if (s) cudaStreamDestroy(s);
  if (prev >= 0) cudaSetDevice(prev);
  delete h;
  return OLGPU_OK;
}

int olgpu_num_boxes(const olgpu_hierarchy *h) { return h ? (int)h->G.boxes.size() : 0; }
int olgpu_num_levels(const olgpu_hierarchy *h) { return h ? h->G.levels : 0; }
int olgpu_mgrid_levels(const olgpu_hierarchy *h) { return h ? h->G.mgrid_levels : 0; }

olgpu_status olgpu_box(const olgpu_hierarchy *h, int box, olgpu_box_info *o)
{
  if (!h || !o || box < 0 || box >= (int)h->G.boxes.size()) return fail(OLGPU_ERR_INVALID_ARG, "bad box");
  fill_box_info(h->G.boxes[box], o);
  return OLGPU_OK;
}

// Bowen-York's variables by name: the one being solved is u, the V solved
// before it are in d_by; -1 for any other name
static int by_var_id(const char *field)
{
  static const char *names[4] = {"V1", "V2", "V3", "lambda"};
  for (int v = 0; v < 4; v++)
    if (field && std::strcmp(field, names[v]) == 0) return v;
  return -1;
}

// The device field of every box (laid out like the arena's) for a field
// name, or nullptr after fail() for an unknown one or a Bowen-York variable
// not solved yet.
static double *field_base(olgpu_hierarchy *h, const char *field)
{
  const int bv = h->equation == OLGPU_EQ_BOWEN_YORK ? by_var_id(field) : -1;
  const int f = bv >= 0 ? F_U : field_id(field);
  if (f < 0 || !h->F.f[f]) {
    fail(OLGPU_ERR_INVALID_ARG, std::string("unknown field ") + (field ? field : ""));
    return nullptr;
  }
  if (bv > h->by_var) {
    fail(OLGPU_ERR_INVALID_ARG, std::string(field) + " is not solved yet");
    return nullptr;
  }
  return bv >= 0 && bv < h->by_var ? h->d_by + (size_t)bv * h->total_pts : h->F.f[f];
}

static olgpu_status field_copy(olgpu_hierarchy *h, int box, const char *field, void *host, bool upload)
{
  if (!h || !host || box < 0 || box >= (int)h->G.boxes.size()) return fail(OLGPU_ERR_INVALID_ARG, "bad box");
  double *base = field_base(h, field);
  if (!base) return OLGPU_ERR_INVALID_ARG;
  CUDA_TRY(cudaSetDevice(h->device));
  const DevBox &B = h->hboxes[box];
  double *d = base + B.off;
  const size_t bytes = sizeof(double) * (size_t)B.n[0] * B.n[1] * B.n[2];
  if (upload)
    CUDA_TRY(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, h->stream));
  else
    CUDA_TRY(cudaMemcpyAsync(host, d, bytes, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return OLGPU_OK;
}

olgpu_status olgpu_upload(olgpu_hierarchy *h, int box, const char *field, const double *host)
{
  return field_copy(h, box, field, const_cast<double *>(host), true);
}

olgpu_status olgpu_download(olgpu_hierarchy *h, int box, const char *field, double *host)
{
  return field_copy(h, box, field, host, false);
}

// The initial state of the solve: u and the FAS work fields cleared, a test
// equation's initial u and source; for Bowen-York those of variable
// h->by_var (lambda's source: the divergence of the solved V).
static olgpu_status init_solve_state(olgpu_hierarchy *h)
{
  CUDA_TRY(cudaSetDevice(h->device));
  const size_t n = sizeof(double) * (size_t)h->total_pts;
  for (int f : {F_U, F_RHO, F_R, F_W, F_WW, F_V, F_T}) CUDA_TRY(cudaMemsetAsync(h->F.f[f], 0, n, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  std::fill(h->adm, h->adm + OLGPU_MAX_BH, 0.0);
  if (h->equation >= OLGPU_EQ_POISSON) {   // a test equation's initial u and source
    PunctureParams PP = puncture_params(&h->P);
    PP.var = h->by_var;
    for (int l = 0; l < h->G.levels; l++) {
      const BoxList BL = level_list(h, l, blocks_all);
      k_test_init<<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->d_coords, PP,
                                                                h->P.boundary == OLGPU_BC_DIRICHLET ? 1 : 0);
      if (h->equation == OLGPU_EQ_BOWEN_YORK && h->by_var == 3)
        k_by_divergence<<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->d_by,
                                                                      h->total_pts);
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->stream));
  }
  return reset_anderson(h);
}

olgpu_status olgpu_reset(olgpu_hierarchy *h)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  h->by_var = 0;
  return init_solve_state(h);
}

// Enqueues one cycle (graph + copy of its norms to pinned host memory) and
// records h->ev_cycle after it; returns at once.
static olgpu_status cycle_enqueue(olgpu_hierarchy *h)
{
  const bool mixed = h->precision == OLGPU_PREC_MIXED;
  CUDA_TRY(cudaGraphLaunch(mixed ? h->graph_mixed : h->graph, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->h_stats, h->d_stats, sizeof(Stats) * h->members.size(), cudaMemcpyDeviceToHost,
                           h->stream));   // a union: every member's
  CUDA_TRY(cudaEventRecord(h->ev_cycle, h->stream));
  return OLGPU_OK;
}

static olgpu_status finish_adm(olgpu_hierarchy *h);

// Reads a finished cycle's norms: the cycle's norm, the ADM masses, NaN.
static olgpu_status cycle_finish(olgpu_hierarchy *h, double *res)
{
  const bool mixed = h->precision == OLGPU_PREC_MIXED;
  const int top = h->G.levels - 1;
  std::memcpy(res, &h->h_stats->slots[mixed ? kSlotDefect : 2 * top + 1], sizeof(double));
  h->last_res = *res;
  std::memcpy(&h->last_du, &h->h_stats->slots[kSlotDu], sizeof(double));
  if (mixed) {   // norm of a mixed cycle: max(finest FP64 defect, max |correction|)
    double corr;
    std::memcpy(&corr, &h->h_stats->slots[kSlotCorr], sizeof(double));
    h->last_defect = *res;
    h->last_correction = corr;
    if (corr > *res) *res = corr;
  }
  const long long c = (long long)(h->norm_hist.size() / (2 * (top + 1)));
  for (int post = 0; post < 2; post++)
    for (int l = 0; l <= top; l++) {
      double v = h->h_stats->coarse_norm;
      if (l > 0) std::memcpy(&v, &h->h_stats->slots[2 * l + post], sizeof(double));
      h->norm_hist.push_back(v);
    }
  // the cycle's print calls: pre-smoothing from the top down, the coarsest
  // solve, post-smoothing back up
  const double *pre = &h->norm_hist[h->norm_hist.size() - 2 * (top + 1)], *post = pre + top + 1;
  for (int l = top; l >= 0; l--) h->events.push_back(olgpu_cycle_event{l, 0, c, pre[l]});
  for (int l = 1; l <= top; l++) h->events.push_back(olgpu_cycle_event{l, 1, c, post[l]});
  return finish_adm(h);
}

// The ADM masses from the last cycle's integrals (elliptic::Compute_ADM_Mass,
// src/elliptic.cc:2447-2611) and the NaN check.
static olgpu_status finish_adm(olgpu_hierarchy *h)
{
  const olgpu_problem &P = h->P;
  for (int i = 0; i < P.numbh; i++) {
    double bhmj = 0;
    for (int j = 0; j < P.numbh; j++)
      if (j != i)
        bhmj += 0.5 * P.mp[j] / std::sqrt((P.x[i] - P.x[j]) * (P.x[i] - P.x[j]) + (P.y[i] - P.y[j]) * (P.y[i] - P.y[j]) +
                                          (P.z[i] - P.z[j]) * (P.z[i] - P.z[j]));
    h->adm[i] = P.mp[i] * (1 + bhmj + h->h_stats->adm_u[i]);
  }
  if (h->h_stats->nan_flag) return fail(OLGPU_ERR_NAN, "NaN in the smoother");
  return OLGPU_OK;
}

static olgpu_status run_cycle(olgpu_hierarchy *h, double *res)
{
  olgpu_status st = cycle_enqueue(h);
  if (st != OLGPU_OK) return st;
  CUDA_TRY(cudaEventSynchronize(h->ev_cycle));
  return cycle_finish(h, res);
}

// Stop-rule bookkeeping shared by olgpu_solve and olgpu_solve_many.
struct SolveTrack {
  olgpu_stop_rule R;
  double tol, du_tol;
  double res = 1e12, res_prev = 1e12;
  double du = 0, part = 0;
  int cycles = 0;
  bool done = false;
  olgpu_status status = OLGPU_OK;
  olgpu_report rep{};

  // Records one finished cycle (r: its norm; part: its residual part;
  // change: its largest change of u); returns true once the rule stops the
  // solve.
  bool step(olgpu_status s, double r, double part_, double change)
  {
    res_prev = res;
    res = r;
    du = change;
    part = part_;
    if (cycles < 256) rep.res[cycles] = r;
    cycles++;
    status = s;
    if (s != OLGPU_OK || cycles >= R.max_cycles) return true;
    if (R.stop == OLGPU_STOP_FIXED) return false;
    if (R.stop == OLGPU_STOP_ERROR) return part_ <= tol && change <= du_tol;   // a NaN never stops it
    if (!(res > tol)) return true;
    if (R.stop == OLGPU_STOP_REFERENCE && !(res < res_prev)) return true;
    return false;
  }
  bool step(olgpu_hierarchy *h, olgpu_status s, double r) { return step(s, r, h->last_res, h->last_du); }
};

olgpu_status olgpu_vcycle(olgpu_hierarchy *h, double *res)
{
  if (!h || !res) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  olgpu_status s = run_cycle(h, res);
  cudaEventRecord(h->ev1, h->stream);
  cudaEventSynchronize(h->ev1);
  h->last_ms = elapsed_ms(h->ev0, h->ev1);
  return s;
}

static olgpu_status make_track(olgpu_hierarchy *h, const olgpu_stop_rule *rule, SolveTrack &T)
{
  T.R = olgpu_stop_rule{OLGPU_STOP_REFERENCE, 100000, 0.0, 0.0};
  if (rule) T.R = *rule;
  if (T.R.max_cycles <= 0) return fail(OLGPU_ERR_INVALID_ARG, "max_cycles must be > 0");
  if (T.R.stop < OLGPU_STOP_REFERENCE || T.R.stop > OLGPU_STOP_ERROR) return fail(OLGPU_ERR_INVALID_ARG, "unknown stop rule");
  if (T.R.stop == OLGPU_STOP_ERROR && h->P.method != OLGPU_METHOD_VCYCLE)
    return fail(OLGPU_ERR_INVALID_ARG, "OLGPU_STOP_ERROR is a V-cycle rule");
  T.tol = T.R.tol > 0 ? T.R.tol : h->eps_solv;
  T.du_tol = T.R.du_tol > 0 ? T.R.du_tol : T.tol;
  h->norm_hist.clear();
  h->events.clear();
  return OLGPU_OK;
}

static void close_track(olgpu_hierarchy *h, SolveTrack &T, olgpu_report *out)
{
  T.rep.cycles = T.cycles;
  T.rep.status = T.status;
  T.rep.final_res = T.res;
  T.rep.final_du = T.du;
  T.rep.final_part = T.part;
  for (int i = 0; i < h->P.numbh; i++) T.rep.adm[i] = h->adm[i];
  if (out) *out = T.rep;
}

// elliptic::FASN with Wcycle = true (src/elliptic.cc:1468-1968): level k
// repeats its descent, the coarser levels' own loop (the coarsest solve
// below level 1) and its ascent while its post-smoothing norm is above tol,
// at most `cap` times.  One host sync per iteration reads the level's norms
// (and the coarsest solve's): the loop's test needs them.
static olgpu_status wcycle_level(olgpu_hierarchy *h, int k, long long icycle, double tol, int cap, double *norm_k)
{
  long long cycle = icycle;
  int iters = 0;
  do {
    const size_t pre = h->events.size();
    h->events.push_back(olgpu_cycle_event{k, 0, cycle, 0.0});   // its norm is read after the sync below
    CUDA_TRY(cudaGraphLaunch(h->graph_down[k], h->stream));
    if (k == 1) {
      h->events.push_back(olgpu_cycle_event{0, 0, cycle, 0.0});
      CUDA_TRY(cudaGraphLaunch(h->graph_coarse, h->stream));
    } else {
      double inner = 0;
      olgpu_status st = wcycle_level(h, k - 1, cycle, tol, cap, &inner);
      if (st != OLGPU_OK) return st;
    }
    CUDA_TRY(cudaGraphLaunch(h->graph_up[k], h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->h_stats, h->d_stats, sizeof(Stats), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    std::memcpy(&h->events[pre].norm, &h->h_stats->slots[2 * k], sizeof(double));
    if (k == 1) h->events[pre + 1].norm = h->h_stats->coarse_norm;
    std::memcpy(norm_k, &h->h_stats->slots[2 * k + 1], sizeof(double));
    h->events.push_back(olgpu_cycle_event{k, 1, cycle, *norm_k});
    if (h->h_stats->nan_flag) return fail(OLGPU_ERR_NAN, "NaN in the smoother");
    cycle++;
    iters++;
  } while (*norm_k > tol && iters < cap);
  if (*norm_k > tol)
    return fail(OLGPU_ERR_DIVERGED, "W-cycle: level " + std::to_string(k) + " did not reach the tolerance in " +
                                        std::to_string(cap) + " iterations");
  return OLGPU_OK;
}

// elliptic::Wcycle (src/elliptic.cc:1348-1380) under the stop rule: each
// top-level call runs the top level's own loop.
static void solve_wcycle(olgpu_hierarchy *h, SolveTrack &T)
{
  const int top = h->G.levels - 1;
  olgpu_status st = top >= 1 ? build_wgraphs(h) : fail(OLGPU_ERR_GEOMETRY, "W-cycle: no coarser level");
  if (st == OLGPU_OK && cudaMemsetAsync(h->d_stats, 0, sizeof(Stats), h->stream) != cudaSuccess)
    st = fail(OLGPU_ERR_CUDA, "W-cycle: clearing the norms");
  if (st != OLGPU_OK) {
    T.step(st, 0.0, 0.0, 0.0);
    return;
  }
  // each level's own loop is capped separately (the reference has no cap):
  // a coarse level whose norm levels off above tol would otherwise repeat
  // max_cycles times inside every iteration of the levels above it
  const int level_cap = std::min(T.R.max_cycles, kWcycleLevelCap);
  for (;;) {
    double r = 0;
    olgpu_status s = wcycle_level(h, top, T.cycles, T.tol, level_cap, &r);
    if (s == OLGPU_OK || s == OLGPU_ERR_DIVERGED) {
      for (int post = 0; post < 2; post++)   // the latest norms of every level, as a V-cycle's
        for (int l = 0; l <= top; l++) {
          double v = h->h_stats->coarse_norm;
          if (l > 0) std::memcpy(&v, &h->h_stats->slots[2 * l + post], sizeof(double));
          h->norm_hist.push_back(v);
        }
      const olgpu_status a = finish_adm(h);
      if (s == OLGPU_OK) s = a;
    }
    if (T.step(s, r, r, 0.0)) break;
  }
}

static void solve_loop(olgpu_hierarchy *h, SolveTrack &T)
{
  if (h->P.method == OLGPU_METHOD_WCYCLE) {
    solve_wcycle(h, T);
  } else {
    for (;;) {
      double r = 0;
      olgpu_status s = run_cycle(h, &r);
      if (T.step(h, s, r)) break;
    }
  }
}

// Bowen-York (include/elliptic.h:772-803): V1, V2, V3 and then lambda, each
// solved under the rule from the state it is in (the one in u continues, the
// later ones start from zero), V kept in d_by as it is solved; lambda's
// source is the divergence of the solved V.  The reference advances the
// four together (elliptic::Smooth and every transfer loop over var_names);
// the equations for V do not involve lambda, so solving them first reaches
// the same fixed point.  The report: the cycles of all four, the largest
// final norm and change, the first failure; res[] holds their norms in turn.
static void solve_bowen_york(olgpu_hierarchy *h, SolveTrack &All)
{
  for (;;) {
    SolveTrack T;
    T.R = All.R;
    T.tol = All.tol;
    T.du_tol = All.du_tol;
    solve_loop(h, T);
    for (int c = 0; c < T.cycles && All.cycles + c < 256; c++) All.rep.res[All.cycles + c] = T.rep.res[c];
    All.cycles += T.cycles;
    All.res = std::max(All.cycles == T.cycles ? 0.0 : All.res, T.res);
    All.du = std::max(All.du, T.du);
    All.part = std::max(All.part, T.part);
    All.status = T.status;
    if (T.status != OLGPU_OK || h->by_var == 3) return;
    const size_t n = sizeof(double) * (size_t)h->total_pts;
    olgpu_status st = OLGPU_OK;
    if (cudaMemcpyAsync(h->d_by + (size_t)h->by_var * h->total_pts, h->F.f[F_U], n, cudaMemcpyDeviceToDevice,
                        h->stream) != cudaSuccess)
      st = fail(OLGPU_ERR_CUDA, "Bowen-York: keeping a solved V");
    if (st == OLGPU_OK) {
      h->by_var++;
      st = init_solve_state(h);
    }
    if (st != OLGPU_OK) {
      All.status = st;
      return;
    }
  }
}

olgpu_status olgpu_solve(olgpu_hierarchy *h, const olgpu_stop_rule *rule, olgpu_report *out)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  SolveTrack T;
  olgpu_status st = make_track(h, rule, T);
  if (st != OLGPU_OK) return st;
  CUDA_TRY(cudaSetDevice(h->device));
  CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  if (h->equation == OLGPU_EQ_BOWEN_YORK)
    solve_bowen_york(h, T);
  else
    solve_loop(h, T);
  cudaEventRecord(h->ev1, h->stream);
  cudaEventSynchronize(h->ev1);
  h->last_ms = elapsed_ms(h->ev0, h->ev1);
  close_track(h, T, out);
  return T.status;
}

olgpu_status olgpu_cycle_launch(olgpu_hierarchy *h)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (h->P.method != OLGPU_METHOD_VCYCLE) return fail(OLGPU_ERR_INVALID_ARG, "W-cycles run from olgpu_solve only");
  CUDA_TRY(cudaSetDevice(h->device));
  return cycle_enqueue(h);
}

olgpu_status olgpu_cycle_poll(olgpu_hierarchy *h, int wait, int *done, double *res)
{
  if (!h || !done || !res) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(h->device));
  *done = 0;
  if (wait) {
    CUDA_TRY(cudaEventSynchronize(h->ev_cycle));
  } else {
    const cudaError_t e = cudaEventQuery(h->ev_cycle);
    if (e == cudaErrorNotReady) return OLGPU_OK;
    if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("cycle: ") + cudaGetErrorString(e));
  }
  *done = 1;
  return cycle_finish(h, res);
}

olgpu_status olgpu_solve_many(olgpu_hierarchy **hs, int n, const olgpu_stop_rule *rule, olgpu_report *reports)
{
  if (!hs || n <= 0) return fail(OLGPU_ERR_INVALID_ARG, "no hierarchies");
  std::vector<SolveTrack> T(n);
  for (int i = 0; i < n; i++) {
    if (!hs[i]) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy in the set");
    if (hs[i]->P.method != OLGPU_METHOD_VCYCLE) return fail(OLGPU_ERR_INVALID_ARG, "W-cycles run from olgpu_solve only");
    if (hs[i]->equation == OLGPU_EQ_BOWEN_YORK)
      return fail(OLGPU_ERR_INVALID_ARG, "Bowen-York solves its variables in turn: olgpu_solve");
    olgpu_status st = make_track(hs[i], rule, T[i]);
    if (st != OLGPU_OK) return st;
  }
  olgpu_status worst = OLGPU_OK;
  // Every solve has its own stream; a solve's next cycle is enqueued as soon
  // as its last one has finished (no lockstep rounds), so the GPU always has
  // the other solves' work queued while the host reads one cycle's norms.
  int active = 0;
  for (int i = 0; i < n; i++) {
    olgpu_status st = olgpu_cycle_launch(hs[i]);
    if (st != OLGPU_OK) return st;
    active++;
  }
  while (active > 0) {
    bool progressed = false;
    for (int i = 0; i < n; i++) {
      if (T[i].done) continue;
      int done = 0;
      double r = 0;
      olgpu_status s = olgpu_cycle_poll(hs[i], 0, &done, &r);
      if (!done && s == OLGPU_OK) continue;
      progressed = true;
      if (T[i].step(hs[i], s, r)) {
        T[i].done = true;
        active--;
        if (s != OLGPU_OK) worst = s;
        continue;
      }
      olgpu_status st = olgpu_cycle_launch(hs[i]);
      if (st != OLGPU_OK) return st;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  for (int i = 0; i < n; i++) close_track(hs[i], T[i], reports ? &reports[i] : nullptr);
  return worst;
}

olgpu_status olgpu_last_cycle(const olgpu_hierarchy *h, double *res, double *du)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (res) *res = h->last_res;
  if (du) *du = h->last_du;
  return OLGPU_OK;
}

olgpu_status olgpu_adm_mass(olgpu_hierarchy *h, double *out)
{
  if (!h || !out) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  for (int i = 0; i < h->P.numbh; i++) out[i] = h->adm[i];
  return OLGPU_OK;
}

// u at arbitrary points (the printed cuts and exports; k_interp_points).
olgpu_status olgpu_interpolate(olgpu_hierarchy *h, int box, int first_level, const double *xyz, long long npts,
                               int ord, double *out)
{
  return olgpu_interpolate_field(h, "u", box, first_level, xyz, npts, ord, out);
}

olgpu_status olgpu_interpolate_field(olgpu_hierarchy *h, const char *field, int box, int first_level,
                                     const double *xyz, long long npts, int ord, double *out)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  const double *src = field_base(h, field);
  if (!src) return OLGPU_ERR_INVALID_ARG;
  if (npts < 0 || (npts > 0 && (!xyz || !out))) return fail(OLGPU_ERR_INVALID_ARG, "null or negative point array");
  if (ord < 1 || ord > kMaxInterpOrd) return fail(OLGPU_ERR_INVALID_ARG, "interpolation order must be 1..15");
  const int nb = (int)h->G.boxes.size();
  if (box >= nb) return fail(OLGPU_ERR_INVALID_ARG, "box index out of range");
  if (first_level < 0 || first_level >= h->G.levels) return fail(OLGPU_ERR_INVALID_ARG, "no such level");
  const int first = h->G.first_box[first_level];   // boxes are level-major
  if (npts == 0) return OLGPU_OK;
  if (npts > 128LL * 0x7fffffffLL) return fail(OLGPU_ERR_INVALID_ARG, "too many points for one call");
  if (box >= 0) {
    for (int a = 0; a < 3; a++)
      if (h->G.boxes[box].n[a] < ord + 1) return fail(OLGPU_ERR_INVALID_ARG, "box smaller than the window");
  } else {
    for (const domain &D : h->G.boxes)
      for (int a = 0; a < 3; a++)
        if (D.n[a] < ord + 1) return fail(OLGPU_ERR_INVALID_ARG, "a box is smaller than the window");
  }
  std::vector<InterpBox> ib(nb);
  int base = first;   // multigrid::multigrid: the box that strictly holds every box scanned before it
  for (int g = 0; g < nb; g++) {
    const domain &D = h->G.boxes[g];
    InterpBox &B = ib[g];
    for (int a = 0; a < 3; a++) {
      B.lo[a] = D.lo[a];
      B.hi[a] = D.hi[a];
      B.d[a] = D.d[a];
      B.n[a] = D.n[a];
    }
    B.buf = D.buf;
    B.off = h->hboxes[g].off;
    const domain &C = h->G.boxes[base];
    bool holds = true;   // domain::operator< (src/domain.cc:1947-1954): C strictly inside D
    for (int a = 0; a < 3; a++) holds = holds && D.lo[a] < C.lo[a] && C.hi[a] < D.hi[a];
    if (g > first && holds) base = g;
  }
  CUDA_TRY(cudaSetDevice(h->device));
  InterpBox *d_b = nullptr;
  double *d_xyz = nullptr, *d_out = nullptr;
  auto release = [&]() {
    dev_free(d_b, h->stream);
    dev_free(d_xyz, h->stream);
    dev_free(d_out, h->stream);
  };
  cudaError_t e = dev_alloc((void **)&d_b, sizeof(InterpBox) * nb, h->device, h->stream);
  if (e == cudaSuccess) e = dev_alloc((void **)&d_xyz, sizeof(double) * 3 * (size_t)npts, h->device, h->stream);
  if (e == cudaSuccess) e = dev_alloc((void **)&d_out, sizeof(double) * (size_t)npts, h->device, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_b, ib.data(), sizeof(InterpBox) * nb, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * (size_t)npts, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) {
    const long long blocks = cdiv(npts, 128);
    k_interp_points<<<(unsigned)blocks, 128, 0, h->stream>>>(d_b, first, nb, base, box, src, d_xyz, npts, ord,
                                                             d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)npts, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  release();
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? OLGPU_ERR_OOM : OLGPU_ERR_CUDA,
                std::string("olgpu_interpolate: ") + cudaGetErrorString(e));
  return OLGPU_OK;
}

// elliptic::ApproximateID: u = the perturbative puncture solution on every
// point of every box, the work fields and the acceleration history reset
// (k_approx_id).
olgpu_status olgpu_approximate_id(olgpu_hierarchy *h, int as_guess)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (h->equation >= OLGPU_EQ_POISSON) return fail(OLGPU_ERR_INVALID_ARG, "the approximation is for punctures");
  olgpu_status st = olgpu_reset(h);
  if (st != OLGPU_OK) return st;
  const PunctureParams PP = puncture_params(&h->P);
  for (int l = 0; l < h->G.levels; l++) {
    const BoxList BL = level_list(h, l, blocks_all);
    k_approx_id<<<BL.blk[BL.count], kThreads, 0, h->stream>>>(BL, h->d_boxes, h->F, h->d_coords, PP,
                                                              as_guess ? 1 : 0);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return OLGPU_OK;
}

olgpu_status olgpu_cycle_events(const olgpu_hierarchy *h, long long first, int cap, olgpu_cycle_event *out,
                                long long *total)
{
  if (!h || first < 0 || cap < 0 || (cap > 0 && !out)) return fail(OLGPU_ERR_INVALID_ARG, "bad argument");
  const long long n = (long long)h->events.size();
  for (long long i = 0; i < cap && first + i < n; i++) out[i] = h->events[first + i];
  if (total) *total = n;
  return OLGPU_OK;
}

olgpu_status olgpu_level_norms(const olgpu_hierarchy *h, int cycle, double *pre, double *post)
{
  if (!h || !pre || !post) return fail(OLGPU_ERR_INVALID_ARG, "null argument");
  const int L = h->G.levels;
  const int cycles = (int)(h->norm_hist.size() / (2 * (size_t)L));
  if (cycle < 0 || cycle >= cycles) return fail(OLGPU_ERR_INVALID_ARG, "no such cycle in this solve");
  const double *v = h->norm_hist.data() + (size_t)cycle * 2 * L;
  for (int l = 0; l < L; l++) {
    pre[l] = v[l];
    post[l] = v[L + l];
  }
  return OLGPU_OK;
}

double olgpu_last_device_ms(const olgpu_hierarchy *h) { return h ? h->last_ms : 0.0; }

int olgpu_kernels_per_cycle(const olgpu_hierarchy *h)
{
  if (!h) return 0;
  return h->precision == OLGPU_PREC_MIXED ? h->launches_mixed : h->launches;
}

olgpu_status olgpu_set_acceleration(olgpu_hierarchy *h, int depth)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (depth < 0 || depth > kAndMax) return fail(OLGPU_ERR_INVALID_ARG, "acceleration depth must be 0..4");
  CUDA_TRY(cudaSetDevice(h->device));
  if (h->graph_mixed && (depth > 0) != (h->anderson_m > 0)) {   // the graph's shape changes
    cudaGraphExecDestroy(h->graph_mixed);
    h->graph_mixed = nullptr;
    h->anderson_m = depth;
    for (auto *vec : {&h->restrict_e, &h->xfer_w32, &h->set_in32, &h->prolong_v32, &h->ghost_e})
      for (auto &X : *vec) { dev_free(X.d_jobs, h->stream); X.d_jobs = nullptr; }
    dev_free(h->d_arena32, h->stream); h->d_arena32 = nullptr;
    dev_free(h->d_aq, h->stream); h->d_aq = nullptr;
    h->mixed_ready = false;
    dev_free(h->d_and, h->stream); h->d_and = nullptr;
    dev_free(h->d_and_state, h->stream); h->d_and_state = nullptr;
    dev_free(h->d_and_part, h->stream); h->d_and_part = nullptr;
    if (h->precision == OLGPU_PREC_MIXED) {
      olgpu_status st = build_mixed(h);
      if (st != OLGPU_OK) return st;
    }
    return OLGPU_OK;
  }
  h->anderson_m = depth;
  return reset_anderson(h);
}

olgpu_status olgpu_set_fp64_acceleration(olgpu_hierarchy *h, int depth)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (depth < 0 || depth > kAndMax) return fail(OLGPU_ERR_INVALID_ARG, "acceleration depth must be 0..4");
  if (h->is_union || h->P.method != OLGPU_METHOD_VCYCLE)
    return fail(OLGPU_ERR_INVALID_ARG, "FP64 acceleration is built for the V-cycle of one hierarchy");
  CUDA_TRY(cudaSetDevice(h->device));
  if (depth > 0 && !h->d_and64) {
    const size_t n = (size_t)h->total_pts;
    if (dev_alloc((void **)&h->d_and64, sizeof(double) * n * (2 * kAndMax + 1), h->device, h->stream) !=
            cudaSuccess ||
        dev_alloc((void **)&h->d_and64_state, sizeof(AndersonState), h->device, h->stream) != cudaSuccess ||
        dev_alloc((void **)&h->d_and64_part, sizeof(double) * 152 * 4 * kAndPart, h->device, h->stream) !=
            cudaSuccess)
      return fail(OLGPU_ERR_OOM, "FP64 Anderson history allocation failed");
    CUDA_TRY(cudaMemsetAsync(h->d_and64, 0, sizeof(double) * n * (2 * kAndMax + 1), h->stream));
  }
  const bool shape = (depth > 0) != (h->anderson64_m > 0);
  h->anderson64_m = depth;
  olgpu_status st = reset_anderson(h);
  if (st != OLGPU_OK || !shape) return st;
  if (h->graph) {   // the FP64 cycle's graph gains or loses the mixing
    CUDA_TRY(cudaGraphExecDestroy(h->graph));
    h->graph = nullptr;
  }
  return build_graph(h);
}

olgpu_status olgpu_set_precision(olgpu_hierarchy *h, int precision)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (precision != OLGPU_PREC_FP64 && precision != OLGPU_PREC_MIXED)
    return fail(OLGPU_ERR_INVALID_ARG, "precision must be OLGPU_PREC_FP64 or OLGPU_PREC_MIXED");
  CUDA_TRY(cudaSetDevice(h->device));
  if (precision == OLGPU_PREC_MIXED) {
    if (h->equation >= OLGPU_EQ_POISSON)
      return fail(OLGPU_ERR_INVALID_ARG, "mixed precision is built for the puncture equations");
    if (h->P.boundary != OLGPU_BC_ROBIN)
      return fail(OLGPU_ERR_INVALID_ARG, "mixed precision is built for the Robin boundary");
    if (h->P.method != OLGPU_METHOD_VCYCLE)
      return fail(OLGPU_ERR_INVALID_ARG, "the W-cycle runs in FP64");
    olgpu_status st = build_mixed(h);
    if (st != OLGPU_OK) return st;
  }
  h->precision = precision;
  return OLGPU_OK;
}

olgpu_status olgpu_set_inner_sweeps(olgpu_hierarchy *h, int nu1, int nu2)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (nu1 < 0 || nu1 > 64 || nu2 < 1 || nu2 > 64)
    return fail(OLGPU_ERR_INVALID_ARG, "inner sweeps must satisfy 0 <= nu1 <= 64, 1 <= nu2 <= 64");
  CUDA_TRY(cudaSetDevice(h->device));
  h->inner_nu1 = nu1;
  h->inner_nu2 = nu2;
  if (!h->graph_mixed) return OLGPU_OK;   // used when the mixed cycle is built
  olgpu_status st = capture_mixed(h);
  if (st != OLGPU_OK) return st;
  return reset_anderson(h);
}

olgpu_status olgpu_set_smoother_blocks(olgpu_hierarchy *h, int max_blocks)
{
  if (!h) return fail(OLGPU_ERR_INVALID_ARG, "null hierarchy");
  if (max_blocks != 0 && (max_blocks < 8 || max_blocks > 16))
    return fail(OLGPU_ERR_INVALID_ARG, "smoother blocks must be 0 or 8..16");
  CUDA_TRY(cudaSetDevice(h->device));
  h->sc_max = max_blocks;
  if (!h->graph_mixed) return OLGPU_OK;   // used when the mixed cycle is built
  choose_smooth_clusters(h);
  return capture_mixed(h);
}

int olgpu_last_coarse_iters(const olgpu_hierarchy *h) { return h && h->h_stats ? h->h_stats->coarse_iters : 0; }

long long olgpu_level_interior_points(const olgpu_hierarchy *h, int level)
{
  if (!h || level < 0 || level >= h->G.levels) return 0;
  long long n = 0;
  for (int i = 0; i < h->G.boxes_in_level[level]; i++) {
    const domain &D = h->G.boxes[h->G.first_box[level] + i];
    n += (long long)(D.n[0] - 2 * D.buf) * (D.n[1] - 2 * D.buf) * (D.n[2] - 2 * D.buf);
  }
  return n;
}

olgpu_status olgpu_time_smoother(olgpu_hierarchy *h, int level, int sweeps, double *ms, int *launches)
{
  if (!h || !ms || level < 1 || level >= h->G.levels || sweeps < 1)
    return fail(OLGPU_ERR_INVALID_ARG, "bad smoother timing request");
  CUDA_TRY(cudaSetDevice(h->device));
  const bool mixed = h->precision == OLGPU_PREC_MIXED;
  int &count = mixed ? h->launches_mixed : h->launches;
  const int before = count;
  CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  if (mixed) {   // the FP32 correction smoother on e
    if (h->equation == 1) dispatch_smooth32<1>(h, level, sweeps);
    else dispatch_smooth32<0>(h, level, sweeps);
  } else {
    if (h->equation == 1) dispatch_smooth<1>(h, level, sweeps, 0);
    else if (h->equation >= 2) dispatch_smooth<2>(h, level, sweeps, 0);
    else dispatch_smooth<0>(h, level, sweeps, 0);
  }
  CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  CUDA_TRY(cudaEventSynchronize(h->ev1));
  CUDA_TRY(cudaGetLastError());
  *ms = elapsed_ms(h->ev0, h->ev1);
  if (launches) *launches = count - before;
  count = before;
  return OLGPU_OK;
}

olgpu_status olgpu_device_pool_bytes(int device, long long *reserved, long long *used)
{
  if (!reserved || !used) return fail(OLGPU_ERR_INVALID_ARG, "null output");
  *reserved = *used = 0;
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> g(g_pool_mu);
    if (device >= 0 && device < kMaxDevices) pool = g_pools[device];
  }
  if (!pool) return OLGPU_OK;   // nothing allocated on this device yet
  unsigned long long r = 0, u = 0;
  CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
  CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
  *reserved = (long long)r;
  *used = (long long)u;
  return OLGPU_OK;
}

olgpu_status olgpu_time_smoother_many(olgpu_hierarchy *const *hs, int n, int level, int sweeps, double *ms)
{
  if (!hs || n < 1 || !ms || sweeps < 1) return fail(OLGPU_ERR_INVALID_ARG, "bad smoother timing request");
  for (int i = 0; i < n; i++)
    if (!hs[i] || hs[i]->is_union || hs[i]->device != hs[0]->device || level < 1 || level >= hs[i]->G.levels)
      return fail(OLGPU_ERR_INVALID_ARG, "bad smoother timing request");
  CUDA_TRY(cudaSetDevice(hs[0]->device));
  std::vector<cudaEvent_t> done(n, nullptr);
  cudaEvent_t end = nullptr;
  auto release = [&]() {
    for (cudaEvent_t e : done)
      if (e) cudaEventDestroy(e);
    if (end) cudaEventDestroy(end);
  };
  cudaError_t e = cudaEventCreate(&end);
  for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
  cudaStream_t s0 = hs[0]->stream;
  // every stream starts after the start event of the first; the end event
  // waits for the last smoother of every stream
  if (e == cudaSuccess) e = cudaEventRecord(hs[0]->ev0, s0);
  for (int i = 1; i < n && e == cudaSuccess; i++) e = cudaStreamWaitEvent(hs[i]->stream, hs[0]->ev0, 0);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    olgpu_hierarchy *h = hs[i];
    const bool mixed = h->precision == OLGPU_PREC_MIXED;
    int &count = mixed ? h->launches_mixed : h->launches;
    const int before = count;
    if (mixed) {
      if (h->equation == 1) dispatch_smooth32<1>(h, level, sweeps);
      else dispatch_smooth32<0>(h, level, sweeps);
    } else {
      if (h->equation == 1) dispatch_smooth<1>(h, level, sweeps, 0);
      else if (h->equation >= 2) dispatch_smooth<2>(h, level, sweeps, 0);
      else dispatch_smooth<0>(h, level, sweeps, 0);
    }
    count = before;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(done[i], h->stream);
    if (e == cudaSuccess && i > 0) e = cudaStreamWaitEvent(s0, done[i], 0);
  }
  if (e == cudaSuccess) e = cudaEventRecord(end, s0);
  if (e == cudaSuccess) e = cudaEventSynchronize(end);
  if (e == cudaSuccess) *ms = elapsed_ms(hs[0]->ev0, end);
  release();
  CUDA_TRY(e);
  return OLGPU_OK;
}

olgpu_status olgpu_fma_peak(int precision, int iters, double *tflops)
{
  if (!tflops || iters < 1 || (precision != OLGPU_PREC_FP64 && precision != OLGPU_PREC_MIXED))
    return fail(OLGPU_ERR_INVALID_ARG, "olgpu_fma_peak: bad argument");
  int dev = 0, sms = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t st;
  CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t a, b;
  CUDA_TRY(cudaEventCreate(&a));
  CUDA_TRY(cudaEventCreate(&b));
  const int blocks = 8 * sms, threads = 256;
  double *sink = nullptr;
  cudaError_t e = cudaMalloc(&sink, sizeof(double));
  double best = 0.0;
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
    cudaEventRecord(a, st);
    if (precision == OLGPU_PREC_FP64) k_fma_peak<double><<<blocks, threads, 0, st>>>(iters, sink);
    else k_fma_peak<float><<<blocks, threads, 0, st>>>(iters, reinterpret_cast<float *>(sink));
    cudaEventRecord(b, st);
    e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (rep == 0) continue;   // warm-up launch
    const double ms = elapsed_ms(a, b);
    const double fmas = (double)blocks * threads * kFmaChains * (double)iters;
    if (ms > 0) best = std::max(best, 2.0 * fmas / (ms * 1e-3) / 1e12);
  }
  cudaFree(sink);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(st);
  if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("olgpu_fma_peak: ") + cudaGetErrorString(e));
  *tflops = best;
  return OLGPU_OK;
}

}  // extern "C"

// ============================================================================
// Batches of solves (olgpu_batch_*): every FASN step of a level is one launch
// over the boxes of all the solves at that level
// ============================================================================
namespace {

// Appends a member's transfer plan to a union's: box indices through map (the
// member's box -> the union's), axis-table offsets moved by tab_base, and the
// plan's block offsets moved past the jobs already there.
void append_plan(Transfer &U, const Transfer &X, const std::vector<int> &map, int tab_base)
{
  for (XferJob J : X.jobs) {
    J.tbox = map[J.tbox];
    J.sbox = map[J.sbox];
    for (int a = 0; a < 3; a++) J.tab[a] += tab_base;
    J.blk0 += U.blocks;
    J.rblk0 += U.row_blocks;
    J.pblk0 += U.pair_blocks;
    U.jobs.push_back(J);
  }
  U.blocks += X.blocks;
  U.row_blocks += X.row_blocks;
  U.pair_blocks += X.pair_blocks;
}

void finish_plan(Transfer &U)
{
  U.width = xfer_width(U.jobs.data(), U.jobs.size());
  U.rows = xfer_rows(U.jobs.data(), U.jobs.size(), U.width) && !std::getenv("OLGPU_XFER_POINTS");
  U.strided = !U.jobs.empty() && std::all_of(U.jobs.begin(), U.jobs.end(),
                                             [](const XferJob &J) { return J.method == XM_STRIDED; });
}

// Members that can share one union: the same equation, order, refinement
// depth (levels above the base grid: with levels aligned from the top, their
// multigrid levels then line up), boundary and sweep counts.
struct UnionKey {
  int eq, order, depth, boundary, nu1, nu2;
  bool operator<(const UnionKey &o) const
  {
    return std::tie(eq, order, depth, boundary, nu1, nu2) < std::tie(o.eq, o.order, o.depth, o.boundary, o.nu1, o.nu2);
  }
};

}  // namespace

struct olgpu_batch {
  std::vector<olgpu_hierarchy *> members;    // in the caller's order
  std::vector<olgpu_hierarchy *> unions;
  std::vector<std::pair<int, int>> where;   // member -> (union, index in the union)
  int precision = OLGPU_PREC_FP64;
  double last_ms = 0.0;
};

// Builds one union of planned members (each with no device state yet),
// ordered by decreasing levels, and everything it launches.
static olgpu_status build_union(std::vector<olgpu_hierarchy *> ms, int precision, int nu1, int nu2, int blocks,
                                olgpu_hierarchy **out)
{
  auto *U = new olgpu_hierarchy();
  U->is_union = true;
  U->P = ms[0]->P;
  U->equation = ms[0]->equation;
  U->device = ms[0]->device;
  U->eps_coarse = ms[0]->eps_coarse;
  U->eps_solv = ms[0]->eps_solv;
  U->inner_nu1 = nu1;
  U->inner_nu2 = nu2;
  if (blocks >= 0) U->sc_max = blocks;
  const int n = (int)ms.size();
  int Lmax = 0;
  long long total = 0;
  for (auto *m : ms) Lmax = std::max(Lmax, m->G.levels);
  std::vector<int> off(n);
  std::vector<long long> base(n);
  for (int i = 0; i < n; i++) {
    off[i] = Lmax - ms[i]->G.levels;
    base[i] = total;
    total += ms[i]->total_pts;
  }
  U->total_pts = total;
  U->G.levels = Lmax;
  U->G.mgrid_levels = ms[0]->G.mgrid_levels + off[0];
  auto fail_u = [&](olgpu_status st) {
    for (auto *m : ms)
      if (std::find_if(U->members.begin(), U->members.end(),
                       [&](const olgpu_hierarchy::Member &M) { return M.h == m; }) == U->members.end())
        olgpu_hierarchy_destroy(m);
    olgpu_hierarchy_destroy(U);
    return st;
  };
  // device: the union's arena and stats, then each member inside them
  if (cudaStreamCreateWithFlags(&U->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&U->ev0) != cudaSuccess || cudaEventCreate(&U->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&U->ev_cycle, cudaEventDisableTiming) != cudaSuccess)
    return fail_u(fail(OLGPU_ERR_CUDA, "batch: stream/event creation failed"));
  live_add(U->device);
  U->live = true;
  if (dev_alloc((void **)&U->d_arena, sizeof(double) * (size_t)total * F_NUM, U->device, U->stream) !=
          cudaSuccess ||
      dev_alloc((void **)&U->d_stats, sizeof(Stats) * n, U->device, U->stream) != cudaSuccess ||
      cudaMallocHost(&U->h_stats, sizeof(Stats) * n) != cudaSuccess)
    return fail_u(fail(OLGPU_ERR_OOM, "batch: device allocation failed"));
  // the members set themselves up on their own streams inside this memory
  if (cudaStreamSynchronize(U->stream) != cudaSuccess) return fail_u(fail(OLGPU_ERR_CUDA, "batch: allocation failed"));
  U->d_stats0 = U->d_stats;
  for (int f = 0; f < F_NUM; f++) U->F.f[f] = U->d_arena + (size_t)f * total;
  if (U->equation != 1) U->F.f[F_D] = U->F.f[F_E] = nullptr;
  U->members.resize(n);
  for (int i = 0; i < n; i++) {
    olgpu_status st = setup_device(ms[i], U->d_arena, total, base[i], U->d_stats + i, U->h_stats + i, false);
    U->members[i].h = ms[i];   // owned by the union from here on
    if (st != OLGPU_OK) return fail_u(st);
    ms[i]->precision = precision;
  }
  // the union's tables: level-major, members in order inside a level, so that
  // the members for which a level is not the coarsest come first
  std::vector<std::vector<int>> map(n);
  std::vector<int> coord_base(n), tab_base(n);
  for (int i = 0; i < n; i++) {
    map[i].assign(ms[i]->hboxes.size(), -1);
    coord_base[i] = (int)U->hcoords.size();
    U->hcoords.insert(U->hcoords.end(), ms[i]->hcoords.begin(), ms[i]->hcoords.end());
    tab_base[i] = (int)U->htab.size();
    U->htab.insert(U->htab.end(), ms[i]->htab.begin(), ms[i]->htab.end());
  }
  U->G.boxes_in_level.assign(Lmax, 0);
  U->G.first_box.assign(Lmax, 0);
  U->fine_count.assign(Lmax, 0);
  for (int A = 0; A < Lmax; A++) {
    U->G.first_box[A] = (int)U->hboxes.size();
    for (int i = 0; i < n; i++) {
      const int k = A - off[i];
      if (k < 0) continue;
      const auto &Gm = ms[i]->G;
      for (int b = 0; b < Gm.boxes_in_level[k]; b++) {
        const int g = Gm.first_box[k] + b;
        DevBox B = ms[i]->hboxes[g];
        B.off += base[i];
        B.coord_off += coord_base[i];
        B.solve = i;
        B.active = 1;
        map[i][g] = (int)U->hboxes.size();
        U->hboxes.push_back(B);
        U->G.boxes.push_back(Gm.boxes[g]);
        U->G.boxes_in_level[A]++;
        if (off[i] < A) U->fine_count[A]++;
      }
    }
    if (U->G.boxes_in_level[A] > kMaxBoxesPerLevel)
      return fail_u(fail(OLGPU_ERR_INVALID_ARG, "batch: too many boxes on one level"));
  }
  // the union's plans: each level's members (those for which it is not the
  // coarsest level) in order
  const int L = Lmax;
  for (auto *vec : {&U->restrict_u, &U->xfer_w, &U->set_in, &U->prolong_v, &U->ghost_u, &U->ghost_lo})
    vec->assign(L, Transfer{});
  for (int A = 1; A < L; A++) {
    for (int i = 0; i < n; i++) {
      const int k = A - off[i];
      if (k < 1) continue;
      olgpu_hierarchy *m = ms[i];
      append_plan(U->restrict_u[A], m->restrict_u[k], map[i], tab_base[i]);
      append_plan(U->xfer_w[A], m->xfer_w[k], map[i], tab_base[i]);
      append_plan(U->set_in[A], m->set_in[k], map[i], tab_base[i]);
      append_plan(U->prolong_v[A], m->prolong_v[k], map[i], tab_base[i]);
      append_plan(U->ghost_u[A], m->ghost_u[k], map[i], tab_base[i]);
      append_plan(U->ghost_lo[A], m->ghost_lo[k], map[i], tab_base[i]);
    }
    for (auto *vec : {&U->restrict_u, &U->xfer_w, &U->set_in, &U->prolong_v, &U->ghost_u, &U->ghost_lo})
      finish_plan((*vec)[A]);
    if (std::getenv("OLGPU_VERBOSE")) {
      auto flags = [](const Transfer &X) {
        return std::to_string(X.jobs.size()) + (X.strided ? "s" : "") + (X.rows ? "r" : "") + std::to_string(X.width);
      };
      std::fprintf(stderr, "olgpu union level %d: restrict %s xfer_w %s set_in %s prolong %s ghost %s |", A,
                   flags(U->restrict_u[A]).c_str(), flags(U->xfer_w[A]).c_str(), flags(U->set_in[A]).c_str(),
                   flags(U->prolong_v[A]).c_str(), flags(U->ghost_u[A]).c_str());
      for (int i = 0; i < n; i++) {
        const int k = A - off[i];
        if (k < 1) continue;
        std::fprintf(stderr, " m%d k%d: %s %s %s %s %s", i, k, flags(ms[i]->restrict_u[k]).c_str(),
                     flags(ms[i]->xfer_w[k]).c_str(), flags(ms[i]->set_in[k]).c_str(),
                     flags(ms[i]->prolong_v[k]).c_str(), flags(ms[i]->ghost_u[k]).c_str());
      }
      std::fprintf(stderr, "\n");
    }
  }
  auto upload = [&](void **dst, const void *src, size_t bytes) -> bool {
    if (bytes == 0) return true;
    if (dev_alloc(dst, bytes, U->device, U->stream) != cudaSuccess) return false;
    return cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, U->stream) == cudaSuccess;
  };
  bool ok = upload((void **)&U->d_boxes, U->hboxes.data(), sizeof(DevBox) * U->hboxes.size()) &&
            upload((void **)&U->d_coords, U->hcoords.data(), sizeof(double) * U->hcoords.size()) &&
            upload((void **)&U->d_tab, U->htab.data(), sizeof(AxisEntry) * U->htab.size());
  for (auto *vec : {&U->restrict_u, &U->xfer_w, &U->set_in, &U->prolong_v, &U->ghost_u, &U->ghost_lo})
    for (auto &X : *vec) ok = ok && upload((void **)&X.d_jobs, X.jobs.data(), sizeof(XferJob) * X.jobs.size());
  if (!ok) return fail_u(fail(OLGPU_ERR_OOM, "batch: device allocation failed"));
  // the members' records
  for (int i = 0; i < n; i++) {
    olgpu_hierarchy::Member &M = U->members[i];
    olgpu_hierarchy *m = ms[i];
    M.off = off[i];
    M.coarse_box = map[i][m->G.first_box[0]];
    M.box_base = M.coarse_box;
    M.pt_base = base[i];
    M.d_stats = U->d_stats + i;
    M.coarse_ncta = m->coarse_ncta;
    M.coarse_bal = m->coarse_bal;
    M.coarse_smem = m->coarse_cluster_smem;
    std::vector<AdmJob> adm = m->hadm;
    for (auto &J : adm) J.box = map[i][J.box];
    M.nadm = (int)adm.size();
    if (!upload((void **)&M.d_adm, adm.data(), sizeof(AdmJob) * adm.size()))
      return fail_u(fail(OLGPU_ERR_OOM, "batch: device allocation failed"));
  }
  for (int i = 0; i < n; i++)   // the members' set-up ran on their own streams
    if (cudaStreamSynchronize(ms[i]->stream) != cudaSuccess)
      return fail_u(fail(OLGPU_ERR_CUDA, "batch: member set-up failed"));
  olgpu_status st = OLGPU_OK;
  if (precision == OLGPU_PREC_MIXED) {
    st = prepare_mixed(U, nullptr, 0, 0);
    for (int i = 0; i < n && st == OLGPU_OK; i++) st = prepare_mixed(ms[i], U->d_arena32, total, base[i]);
    if (st == OLGPU_OK) st = capture_mixed(U);
  } else {
    st = build_graph(U);
  }
  if (st != OLGPU_OK) return fail_u(st);
  U->precision = precision;
  *out = U;
  return OLGPU_OK;
}

extern "C" {

void olgpu_batch_config_defaults(olgpu_batch_config *c)
{
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->device = -1;
  c->precision = OLGPU_PREC_MIXED;
  c->nu1 = -1;
  c->nu2 = -1;
  c->blocks = -1;
}

olgpu_status olgpu_batch_create(const olgpu_problem *ps, int n, const olgpu_batch_config *cfg, olgpu_batch **out)
{
  if (!ps || n < 1 || !out) return fail(OLGPU_ERR_INVALID_ARG, "batch: no problems");
  *out = nullptr;
  olgpu_batch_config c;
  olgpu_batch_config_defaults(&c);
  if (cfg) c = *cfg;
  if (c.precision != OLGPU_PREC_FP64 && c.precision != OLGPU_PREC_MIXED)
    return fail(OLGPU_ERR_INVALID_ARG, "batch: precision must be OLGPU_PREC_FP64 or OLGPU_PREC_MIXED");
  if ((c.nu1 >= 0) != (c.nu2 >= 0) || c.nu1 > 64 || c.nu2 > 64 || (c.nu2 >= 0 && c.nu2 < 1))
    return fail(OLGPU_ERR_INVALID_ARG, "batch: inner sweeps must be 0 <= nu1 <= 64, 1 <= nu2 <= 64 (or both < 0)");
  for (int i = 0; i < n; i++) {
    olgpu_status st = validate_problem(&ps[i]);
    if (st != OLGPU_OK) return st;
    if (ps[i].method != OLGPU_METHOD_VCYCLE) return fail(OLGPU_ERR_INVALID_ARG, "batch: V-cycles only");
    if (c.precision == OLGPU_PREC_MIXED &&
        (ps[i].equation >= OLGPU_EQ_POISSON || ps[i].boundary != OLGPU_BC_ROBIN))
      return fail(OLGPU_ERR_INVALID_ARG, "batch: mixed precision is built for the puncture equations, Robin");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(OLGPU_ERR_NO_DEVICE, "no CUDA device");
  if (c.device >= 0) CUDA_TRY(cudaSetDevice(c.device));
  auto *b = new olgpu_batch();
  b->precision = c.precision;
  // plan every member, then group them into unions
  std::map<UnionKey, std::vector<int>> groups;
  for (int i = 0; i < n; i++) {
    auto *m = new olgpu_hierarchy();
    olgpu_status st = plan_hierarchy(&ps[i], m);
    if (st != OLGPU_OK) {
      olgpu_hierarchy_destroy(m);
      for (auto *x : b->members) olgpu_hierarchy_destroy(x);
      delete b;
      return st;
    }
    b->members.push_back(m);
    const UnionKey key{m->equation >= OLGPU_EQ_POISSON ? 2 : m->equation, m->P.order,
                       m->G.levels - m->G.mgrid_levels, m->P.boundary, m->P.nu1, m->P.nu2};
    groups[key].push_back(i);
  }
  b->where.assign(n, {-1, -1});
  olgpu_status st = OLGPU_OK;
  std::vector<bool> owned(n, false);   // handed to a union (which destroys it)
  for (auto &kv : groups) {
    std::vector<int> idx = kv.second;   // deepest first: its boxes open every level
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int x, int y) { return b->members[x]->G.levels > b->members[y]->G.levels; });
    // chunks whose every level fits one launch's box list
    size_t at = 0;
    while (at < idx.size() && st == OLGPU_OK) {
      std::vector<int> chunk;
      std::vector<int> per_level;
      for (; at < idx.size(); at++) {
        const olgpu_hierarchy *m = b->members[idx[at]];
        const int Lm = m->G.levels;
        const int Lmax = chunk.empty() ? Lm : b->members[chunk[0]]->G.levels;
        std::vector<int> trial = per_level;
        trial.resize(Lmax, 0);
        for (int k = 0; k < Lm; k++) trial[k + Lmax - Lm] += m->G.boxes_in_level[k];
        if (!chunk.empty() && *std::max_element(trial.begin(), trial.end()) > kMaxBoxesPerLevel) break;
        per_level = trial;
        chunk.push_back(idx[at]);
      }
      std::vector<olgpu_hierarchy *> ms;
      for (int i : chunk) {
        ms.push_back(b->members[i]);
        owned[i] = true;
      }
      olgpu_hierarchy *U = nullptr;
      st = build_union(ms, c.precision, c.nu1, c.nu2, c.blocks, &U);
      if (st != OLGPU_OK) break;
      for (size_t q = 0; q < chunk.size(); q++) b->where[chunk[q]] = {(int)b->unions.size(), (int)q};
      b->unions.push_back(U);
    }
    if (st != OLGPU_OK) break;
  }
  if (st != OLGPU_OK) {
    for (int i = 0; i < n; i++)
      if (!owned[i]) olgpu_hierarchy_destroy(b->members[i]);
    for (auto *U : b->unions) olgpu_hierarchy_destroy(U);
    delete b;
    return st;
  }
  *out = b;
  return OLGPU_OK;
}

olgpu_status olgpu_batch_destroy(olgpu_batch *b)
{
  if (!b) return OLGPU_OK;
  for (auto *U : b->unions) olgpu_hierarchy_destroy(U);
  delete b;
  return OLGPU_OK;
}

int olgpu_batch_size(const olgpu_batch *b) { return b ? (int)b->members.size() : 0; }
int olgpu_batch_unions(const olgpu_batch *b) { return b ? (int)b->unions.size() : 0; }

int olgpu_batch_kernels_per_cycle(const olgpu_batch *b)
{
  if (!b) return 0;
  int k = 0;
  for (auto *U : b->unions) k += b->precision == OLGPU_PREC_MIXED ? U->launches_mixed : U->launches;
  return k;
}

olgpu_hierarchy *olgpu_batch_member(olgpu_batch *b, int i)
{
  return b && i >= 0 && i < (int)b->members.size() ? b->members[i] : nullptr;
}

olgpu_status olgpu_batch_reset(olgpu_batch *b)
{
  if (!b) return fail(OLGPU_ERR_INVALID_ARG, "null batch");
  for (auto *m : b->members) {
    olgpu_status st = olgpu_reset(m);
    if (st != OLGPU_OK) return st;
  }
  return OLGPU_OK;
}

olgpu_status olgpu_batch_solve(olgpu_batch *b, const olgpu_stop_rule *rule, olgpu_report *reports)
{
  if (!b) return fail(OLGPU_ERR_INVALID_ARG, "null batch");
  const int n = (int)b->members.size();
  std::vector<SolveTrack> T(n);
  for (int i = 0; i < n; i++) {
    olgpu_status st = make_track(b->members[i], rule, T[i]);
    if (st != OLGPU_OK) return st;
  }
  const auto t0 = std::chrono::steady_clock::now();
  olgpu_status worst = OLGPU_OK;
  std::vector<int> live(b->unions.size(), 0);
  for (size_t u = 0; u < b->unions.size(); u++) {   // every box active, then the first cycle
    olgpu_hierarchy *U = b->unions[u];
    CUDA_TRY(cudaSetDevice(U->device));
    for (auto &B : U->hboxes) B.active = 1;
    CUDA_TRY(cudaMemcpyAsync(U->d_boxes, U->hboxes.data(), sizeof(DevBox) * U->hboxes.size(), cudaMemcpyHostToDevice,
                             U->stream));
    live[u] = (int)U->members.size();
    olgpu_status st = cycle_enqueue(U);
    if (st != OLGPU_OK) return st;
  }
  int remaining = n;
  while (remaining > 0) {
    bool progressed = false;
    for (size_t u = 0; u < b->unions.size(); u++) {
      if (live[u] == 0) continue;
      olgpu_hierarchy *U = b->unions[u];
      const cudaError_t e = cudaEventQuery(U->ev_cycle);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) return fail(OLGPU_ERR_CUDA, std::string("batch cycle: ") + cudaGetErrorString(e));
      progressed = true;
      bool dirty = false;
      for (int q = 0; q < (int)U->members.size(); q++) {
        olgpu_hierarchy *m = U->members[q].h;
        const int i = (int)(std::find(b->members.begin(), b->members.end(), m) - b->members.begin());
        if (T[i].done) continue;
        double r = 0;
        const olgpu_status s = cycle_finish(m, &r);
        if (!T[i].step(m, s, r)) continue;
        T[i].done = true;   // this solve stops: its boxes are left as they are from now on
        if (s != OLGPU_OK) worst = s;
        for (auto &B : U->hboxes)
          if (B.solve == q) B.active = 0;
        dirty = true;
        live[u]--;
        remaining--;
      }
      if (live[u] == 0) continue;
      if (dirty)
        CUDA_TRY(cudaMemcpyAsync(U->d_boxes, U->hboxes.data(), sizeof(DevBox) * U->hboxes.size(),
                                 cudaMemcpyHostToDevice, U->stream));
      olgpu_status st = cycle_enqueue(U);
      if (st != OLGPU_OK) return st;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  for (auto *U : b->unions) CUDA_TRY(cudaStreamSynchronize(U->stream));
  b->last_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < n; i++) close_track(b->members[i], T[i], reports ? &reports[i] : nullptr);
  return worst;
}

double olgpu_batch_last_ms(const olgpu_batch *b) { return b ? b->last_ms : 0.0; }

}  // extern "C"

// ============================================================================
// Non-allocating single-box smoother (olgpu_smooth_box_noalloc)
//
// Its scratch is one fixed file-scope device array: the box descriptor the
// kernel reads and a Stats record (the norm accumulator of sweep s in
// slots[s], the NaN flag).  In host code
// the symbol is only a stand-in, so each device's address of it is looked up
// once with cudaGetSymbolAddress (with that device current) and passed to the
// kernels.
// ============================================================================
namespace {

constexpr int kNoAllocWords = 256;                    // 2 KiB
constexpr int kNoAllocBoxWords = 32;                  // DevBox, rounded up
constexpr int kNoAllocStatsOff = kNoAllocBoxWords;    // then one Stats record
static_assert(sizeof(DevBox) <= kNoAllocBoxWords * sizeof(unsigned long long), "box slot too small");
static_assert(kNoAllocStatsOff * sizeof(unsigned long long) + sizeof(Stats) <=
                  kNoAllocWords * sizeof(unsigned long long), "scratch too small");
static_assert(OLGPU_NOALLOC_MAX_SWEEPS <= kSlotDu, "one norm slot per sweep");

static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocWords];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned long long *g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (set-up once;
// dropped again by noalloc_forget after a CUDA error, so that a call after a
// device reset looks it up anew).
olgpu_status noalloc_scratch(unsigned long long **out)
{
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(OLGPU_ERR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(OLGPU_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_addr[dev] = static_cast<unsigned long long *>(p);
  }
  *out = g_noalloc_addr[dev];
  return OLGPU_OK;
}

void noalloc_forget()
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  g_noalloc_addr[dev] = nullptr;
}

// CUDA_TRY for the non-allocating entry point: a failed CUDA call also drops
// the cached scratch address of the current device.
#define NOALLOC_TRY(expr)                                                                    \
  do {                                                                                       \
    cudaError_t e_ = (expr);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      noalloc_forget();                                                                      \
      return fail(OLGPU_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));       \
    }                                                                                        \
  } while (0)

template <int ORD, int EQ>
void noalloc_sweeps(const BoxList &L, const DevBox *box, const DevFields &F, int sweeps, unsigned long long *scr,
                    cudaStream_t st)
{
  for (int s = 0; s < sweeps; s++)
    for (int color = 0; color < num_colors<ORD>(); color++)
      k_smooth_color<ORD, EQ><<<L.blk[L.count], kSmoothThreads, 0, st>>>(
          L, box, F, color, reinterpret_cast<Stats *>(scr + kNoAllocStatsOff), s);   // level 0: slots[s]
}

template <int EQ>
void noalloc_dispatch(int order, const BoxList &L, const DevBox *box, const DevFields &F, int sweeps,
                      unsigned long long *scr, cudaStream_t st)
{
  switch (order) {
  case 2: noalloc_sweeps<2, EQ>(L, box, F, sweeps, scr, st); break;
  case 4: noalloc_sweeps<4, EQ>(L, box, F, sweeps, scr, st); break;
  case 6: noalloc_sweeps<6, EQ>(L, box, F, sweeps, scr, st); break;
  default: noalloc_sweeps<8, EQ>(L, box, F, sweeps, scr, st); break;
  }
}

}  // namespace

extern "C" olgpu_status olgpu_smooth_box_noalloc(const olgpu_box_fields *f, int sweeps, double *norms, void *stream)
{
  if (!f || !f->u || !f->b || !f->c || !f->s) return fail(OLGPU_ERR_INVALID_ARG, "null field pointer");
  if (!(f->order == 2 || f->order == 4 || f->order == 6 || f->order == 8))
    return fail(OLGPU_ERR_INVALID_ARG, "order must be 2, 4, 6 or 8");
  if ((f->d == nullptr) != (f->e == nullptr))
    return fail(OLGPU_ERR_INVALID_ARG, "d and e must both be given (scalar field) or both be NULL");
  if (sweeps < 1 || sweeps > OLGPU_NOALLOC_MAX_SWEEPS)
    return fail(OLGPU_ERR_INVALID_ARG, "sweeps must be 1.." + std::to_string(OLGPU_NOALLOC_MAX_SWEEPS) +
                                           ": the fixed scratch holds one norm accumulator per sweep");
  const int buf = f->order / 2;
  if (f->nx < 2 * buf + 1 || f->ny < 2 * buf + 1 || f->nz < 2 * buf + 1)
    return fail(OLGPU_ERR_INVALID_ARG, "box has no interior point for this order");
  if (!(f->dx > 0 && f->dy > 0 && f->dz > 0)) return fail(OLGPU_ERR_INVALID_ARG, "spacing must be > 0");
  unsigned long long *scr = nullptr;
  olgpu_status st = noalloc_scratch(&scr);
  if (st != OLGPU_OK) return st;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);

  DevBox B{};
  B.n[0] = f->nx;
  B.n[1] = f->ny;
  B.n[2] = f->nz;
  B.buf = buf;
  B.off = 0;
  B.level = 0;
  B.solve = 0;
  B.active = 1;
  B.falloff = 1;
  const double d[3] = {f->dx, f->dy, f->dz};
  set_box_stencil(B, f->order, d);
  // the descriptor and the zeroed accumulators go into the fixed scratch
  NOALLOC_TRY(cudaMemcpyAsync(scr, &B, sizeof(DevBox), cudaMemcpyHostToDevice, cs));
  NOALLOC_TRY(cudaMemsetAsync(scr + kNoAllocStatsOff, 0, sizeof(Stats), cs));
  DevFields F{};
  F.f[F_U] = f->u;
  F.f[F_B] = const_cast<double *>(f->b);
  F.f[F_C] = const_cast<double *>(f->c);
  F.f[F_RHO] = const_cast<double *>(f->s);
  F.f[F_D] = const_cast<double *>(f->d);
  F.f[F_E] = const_cast<double *>(f->e);
  BoxList L{};
  L.count = 1;
  L.box[0] = 0;
  L.blk[0] = 0;
  L.blk[1] = (int)blocks_color(B);
  const DevBox *dbox = reinterpret_cast<const DevBox *>(scr);
  if (f->d) noalloc_dispatch<1>(f->order, L, dbox, F, sweeps, scr, cs);
  else noalloc_dispatch<0>(f->order, L, dbox, F, sweeps, scr, cs);
  NOALLOC_TRY(cudaGetLastError());
  Stats host;
  NOALLOC_TRY(cudaMemcpyAsync(&host, scr + kNoAllocStatsOff, sizeof(Stats), cudaMemcpyDeviceToHost, cs));
  NOALLOC_TRY(cudaStreamSynchronize(cs));
  if (norms)
    for (int s = 0; s < sweeps; s++) std::memcpy(&norms[s], &host.slots[s], sizeof(double));
  const int nan_flag = host.nan_flag;
  if (nan_flag) return fail(OLGPU_ERR_NAN, "NaN in the smoother");
  return OLGPU_OK;
}
