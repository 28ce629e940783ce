// mixed.cuh -- FP32 inner V-cycle of the mixed-precision solve.
//
// The FP64 state u is frozen during a cycle; the cycle solves in FP32 for a
// correction e on every level with the reference's FAS algorithm
// (src/elliptic.cc:1468-1968) applied to the correction problem
//     N(u + e) - N(u) = S - N(u),
// whose right-hand side (the FP64 defect) and whose per-point coefficients
// A = b/(c+u)^7 and 1/(c+u) are evaluated in FP64 before the cycle.  With
// x = e/(c+u) and y = 1/(1+x) the puncture term of the correction operator is
//     A [(1+x)^-7 - 1] = -A x y (1 + y + ... + y^6),
// which has no cancellation for small x, so FP32 resolves the correction to
// FP32 precision relative to the correction itself; the FP64 update u += e
// then converges to the FP64 fixed point.  The singular factor b/(c+u)^7 is
// only ever formed in FP64 (at a puncture on a node c+u ~ 1e14 and its 7th
// power overflows FP32).
#pragma once

#include "kernels.cuh"

namespace olgpu {

// FP32 work fields of the correction cycle.
enum Field32 { G_E = 0, G_S, G_A, G_IQ, G_R, G_W, G_WW, G_V, G_T, G_D, G_E5, G_NUM };

struct DevFields32 {
  float *f[G_NUM];
};

// Laplacian of e on one point from an accessor at(axis, offset) of its
// neighbours.  Every FP32 stencil (global or shared-memory resident, one
// launch per colour or every sweep in a cluster) evaluates this one
// expression, and every operation is an explicitly rounded intrinsic: the
// compiler may not fuse or reorder any of it, so kernels of different shapes
// get the same bits (plain expressions were seen to differ between two
// kernels after an unrelated branch was added to one of them).
template <int ORD, class Acc>
__device__ __forceinline__ float lapf_acc(float c, Acc at, float ix2, float iy2, float iz2)
{
  // the axes' terms scaled and summed by explicit multiply-adds
  auto sum3 = [&](float a0, float a1, float a2) {
    return __fmaf_rn(a2, iz2, __fmaf_rn(a1, iy2, __fmul_rn(a0, ix2)));
  };
  auto pair = [&](int a, int d) { return __fadd_rn(at(a, d), at(a, -d)); };
  if (ORD == 2) {
    auto ax = [&](int a) { return __fadd_rn(__fmaf_rn(-2.0f, c, at(a, 1)), at(a, -1)); };
    return sum3(ax(0), ax(1), ax(2));
  } else if (ORD == 4) {
    auto ax = [&](int a) { return __fmaf_rn(-30.0f, c, __fmaf_rn(16.0f, pair(a, 1), -pair(a, 2))); };
    return __fmul_rn(sum3(ax(0), ax(1), ax(2)), 1.0f / 12.0f);
  } else if (ORD == 6) {
    auto ax = [&](int a) {
      const float v = __fmaf_rn(-27.0f, pair(a, 2), __fmul_rn(2.0f, pair(a, 3)));
      return __fmaf_rn(-490.0f, c, __fmaf_rn(270.0f, pair(a, 1), v));
    };
    return __fmul_rn(sum3(ax(0), ax(1), ax(2)), 1.0f / 180.0f);
  } else {
    auto ax = [&](int a) {
      float v = __fmaf_rn(128.0f, pair(a, 3), __fmul_rn(-9.0f, pair(a, 4)));
      v = __fmaf_rn(-1008.0f, pair(a, 2), v);
      v = __fmaf_rn(8064.0f, pair(a, 1), v);
      return __fmaf_rn(-14350.0f, c, v);
    };
    return __fmul_rn(sum3(ax(0), ax(1), ax(2)), 1.0f / 5040.0f);
  }
}

template <int ORD>
__device__ __forceinline__ float lapf(const float *__restrict__ u, long long p, long long sy, long long sz,
                                      const DevBox &B)
{
  const long long st[3] = {1, sy, sz};
  return lapf_acc<ORD>(u[p], [&](int a, int d) { return u[p + d * st[a]]; }, (float)B.idx2[0], (float)B.idx2[1],
                       (float)B.idx2[2]);
}


// Correction operator N(u+e) - N(u) at one point and its derivative in e.
template <int EQ>
__device__ __forceinline__ void corr_op(float lapv, float dl, float e, float A, float iq, float D, float E5,
                                        float &op, float &dop)
{
  // explicitly rounded operations and multiply-adds throughout (see lapf_acc)
  const float x = __fmul_rn(e, iq);
  const float y = rcp_fast(__fadd_rn(1.0f, x));
  const float y2 = __fmul_rn(y, y), y4 = __fmul_rn(y2, y2);
  float s = __fadd_rn(__fadd_rn(1.0f, y), y2);                     // sum_{k=0..6} y^k
  s = __fadd_rn(__fmaf_rn(y2, y, s), y4);
  s = __fmaf_rn(y4, y2, __fmaf_rn(y4, y, s));
  op = __fmaf_rn(-__fmul_rn(__fmul_rn(A, x), y), s, lapv);                        // A ((1+x)^-7 - 1)
  dop = __fmaf_rn(-__fmul_rn(__fmul_rn(7.0f, A), iq), __fmul_rn(y4, y4), dl);    // -7 A iq (1+x)^-8
  if (EQ == 1) {
    // d e + E5 ((1+x)^5 - 1),  E5 = e_coef (c+u)^5
    float p = __fadd_rn(5.0f, x);
    p = __fmaf_rn(x, p, 10.0f);
    p = __fmaf_rn(x, p, 10.0f);
    p = __fmaf_rn(x, p, 5.0f);
    op = __fadd_rn(op, __fmaf_rn(D, e, __fmul_rn(__fmul_rn(E5, x), p)));
    const float x1 = __fadd_rn(1.0f, x), x2 = __fmul_rn(x1, x1);
    dop = __fadd_rn(dop, __fmaf_rn(__fmul_rn(__fmul_rn(5.0f, E5), iq), __fmul_rn(x2, x2), D));
  }
}

// One point's smoother update e - (op - S) / dop, one explicit multiply-add: every
// FP32 smoother (per colour, cluster-resident) forms it here.
__device__ __forceinline__ float corr_update(float e, float op, float dop, float S)
{
  return __fmaf_rn(-__fsub_rn(op, S), rcp_fast(dop), e);
}

// ---------------------------------------------------------------------------
// FP64 preparation (coefficients and defect: k_mx_prep below) and the FP64
// defect of the finest level after the update (the cycle's norm)
// ---------------------------------------------------------------------------

// FP64 defect S - OP(u) on INSIDE points into the FP32 source; the other
// points get S (the operator value there is written by the Robin kernels in
// mode 2 on boxes with a physical boundary, and stays 0 on refinement ghosts,
// as the reference's r field does).  Optionally (slot >= 0) the L-infinity
// norm, into stats[B.solve].slots[slot].
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_mx_defect(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                   DevFields32 G, Stats *stats, int slot)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;   // the whole block (one box a block)
  unsigned long long *norm_slot = slot >= 0 ? &stats[B.solve].slots[slot] : nullptr;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  double rabs = 0.0;
  if (t < n) {
    const int b = B.buf;
    const int i = ((int)t % B.n[0]);
    const int r = (int)t / B.n[0];
    const int j = (r % B.n[1]), k = (r / B.n[1]);
    const bool inside = i >= b && i < B.n[0] - b && j >= b && j < B.n[1] - b && k >= b && k < B.n[2] - b;
    const double *u = F.f[F_U] + B.off;
    double d = F.f[F_RHO][B.off + t];
    if (inside) {
      const double lv = lap<ORD>(u, t, B.n[0], (long long)B.n[0] * B.n[1], B);
      double op, dop;
      point_op<EQ>(lv, B.dulap, u[t], F.f[F_B][B.off + t], F.f[F_C][B.off + t],
                   EQ == 1 ? F.f[F_D][B.off + t] : 0.0, EQ == 1 ? F.f[F_E][B.off + t] : 0.0, op, dop);
      d = d - op;
      rabs = fabs(d);
    }
    G.f[G_S][B.off + t] = (float)d;
  }
  if (norm_slot) block_max_atomic(rabs, norm_slot);
}

// Colour-packed position of INSIDE point (i, j, k) of a box: the points of
// colour c = (i + j + k) mod NC, row by row (plane k, row j), in the order the
// colour pass visits them (ih = the point's index among its row's colour-c
// points), so that a colour pass reads its points' coefficients contiguously.
// Every index is below NC * m2 * m1 * ceil(m0 / NC) <= the box's points.
template <int ORD>
__host__ __device__ __forceinline__ long long packed_index(const DevBox &B, int i, int j, int k)
{
  constexpr int NC = ORD / 2 + 1;
  const int b = B.buf;
  const int m0 = B.n[0] - 2 * b, m1 = B.n[1] - 2 * b, m2 = B.n[2] - 2 * b;
  const int H = (m0 + NC - 1) / NC;
  const int c = (i + j + k) % NC;
  return (((long long)c * m2 + (k - b)) * m1 + (j - b)) * H + (i - b) / NC;
}

// The FP64 preparation of one level in one pass: on INSIDE points the
// coefficients of the correction operator, A = b/(c+u)^7 and 1/(c+u) (and d,
// E5 = e (c+u)^5 for the scalar field; nothing reads them on the ghosts) and
// the source S32 = S - OP(u), sharing 1/(c+u); S on the other points (as
// k_mx_defect).
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_mx_prep(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                 DevFields32 G, float2 *__restrict__ aq)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const long long p = B.off + t;
  const int b = B.buf;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const bool inside = i >= b && i < B.n[0] - b && j >= b && j < B.n[1] - b && k >= b && k < B.n[2] - b;
  if (!inside) {   // the FP32 cycle reads the coefficients on INSIDE points only
    G.f[G_S][p] = (float)F.f[F_RHO][p];
    return;
  }
  const double *u = F.f[F_U] + B.off;
  const double uu = u[t], bb = F.f[F_B][p];
  const double q = F.f[F_C][p] + uu;
  const double iq = rcp_newton(q);
  const double iq2 = iq * iq, iq4 = iq2 * iq2;
  const double t7 = bb * (iq4 * iq2 * iq);   // b / (c+u)^7
  G.f[G_A][p] = (float)t7;
  G.f[G_IQ][p] = (float)iq;
  if (aq) aq[B.off + packed_index<ORD>(B, i, j, k)] = make_float2((float)t7, (float)iq);
  double q4 = 0.0;
  if (EQ == 1) {
    const double q2 = q * q;
    q4 = q2 * q2;
    G.f[G_D][p] = (float)F.f[F_D][p];
    G.f[G_E5][p] = (float)(F.f[F_E][p] * (q4 * q));
  }
  double nl = t7;   // OP - Lap u
  if (EQ == 1) nl = nl + F.f[F_D][p] * q + F.f[F_E][p] * (q4 * q);
  // S = rho - OP(u), the Laplacian's scale and the addition in one multiply-add
  G.f[G_S][p] = (float)-lap_acc<ORD>(u, t, B.n[0], (long long)B.n[0] * B.n[1], B, nl - F.f[F_RHO][p]);
}

// Robin defect on the physical boundary: S32 = S - (term(u) + u) (FP64).
template <int ORD>
__device__ __forceinline__ void mx_robin_defect_point(const DevBox &B, const DevFields &F, const DevFields32 &G,
                                                      const double *__restrict__ crd, int mask, int i, int j, int k)
{
  const double *u = F.f[F_U] + B.off;
  const long long p = pidx(B, i, j, k);
  double dF;
  const double t = robin_term<ORD>(u, B, crd, mask, i, j, k, dF);
  G.f[G_S][B.off + p] = (float)(F.f[F_RHO][B.off + p] - (t + u[p]));
}

template <int ORD>
__global__ void __launch_bounds__(256) k_mx_robin_defect(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                         DevFields32 G, const double *__restrict__ crd)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const int b = B.buf;
  // every ghost point of the box: classify by how many axes are in the band
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const int ijk[3] = {i, j, k};
  int mask = 0;
  for (int a = 0; a < 3; a++)
    if (ijk[a] < b || ijk[a] >= B.n[a] - b) mask |= 1 << a;
  if (mask) mx_robin_defect_point<ORD>(B, F, G, crd, mask, i, j, k);
}

// u += e over ALL points (the FP64 outer update), and max |e| over the points
// the discrete system fixes (every point of the solution levels, the interior
// of the multigrid coarse levels, whose ghost values are not fixed), into
// stats[B.solve].slots[kSlotCorr].
__global__ void __launch_bounds__(256) k_mx_update(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                   DevFields32 G, Stats *stats)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;   // the whole block (one box a block)
  unsigned long long *norm_slot = &stats[B.solve].slots[kSlotCorr];
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  double eabs = 0.0;
  if (t < n) {
    const long long p = B.off + t;
    const double e = (double)G.f[G_E][p];
    F.f[F_U][p] = F.f[F_U][p] + e;
    bool pinned = !B.mg_coarse;
    if (!pinned) {
      const int b = B.buf;
      const int i = ((int)t % B.n[0]);
      const int r = (int)t / B.n[0];
      const int j = (r % B.n[1]), k = (r / B.n[1]);
      pinned = i >= b && i < B.n[0] - b && j >= b && j < B.n[1] - b && k >= b && k < B.n[2] - b;
    }
    if (pinned) eabs = fabs(e);
  }
  block_max_atomic(eabs, norm_slot);
}

// ---------------------------------------------------------------------------
// FP32 correction cycle
// ---------------------------------------------------------------------------
template <int EQ>
__device__ __forceinline__ void corr_at(const DevBox &B, const DevFields32 &G, long long p, float lv, float &op,
                                        float &dop)
{
  const long long q = B.off + p;
  corr_op<EQ>(lv, (float)B.dulap, G.f[G_E][q], G.f[G_A][q], G.f[G_IQ][q], EQ == 1 ? G.f[G_D][q] : 0.0f,
              EQ == 1 ? G.f[G_E5][q] : 0.0f, op, dop);
}

// One multicolour pass on e (colour (i+j+k) mod (order/2+1)), PTS points of
// a row's colour a thread (their loads first, then the updates: points of
// one colour do not read each other, so any PTS gives the same bits).  Held
// to 32 registers at order 4 with one point a thread (no spills there), so
// that 16 of its 128-thread blocks fit an SM: the pass waits on loads, and
// at 40 registers (12 blocks) it ran 4 % slower; the other forms get the
// registers they need without spilling.  A and 1/(c+u)
// come colour-packed from aq (one float2 per point, the pass's points
// contiguous: packed_index) when the hierarchy keeps that copy, else from the
// lexicographic fields; the values, and so the bits, are the same.  Each is
// used once, so aq is read through L2 (ld.global.cg).
template <int ORD, int EQ, int PTS = 1>
__global__ void __launch_bounds__(256, PTS == 1 ? (ORD == 4 ? 8 : 6) : 4)
    k_smooth32(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G, const float2 *aq, int color, Stats *stats)
{
  constexpr int NC = num_colors<ORD>();
  griddep_wait();                 // launched as a programmatic dependent
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  int *nan_flag = &stats[B.solve].nan_flag;
  const int b = B.buf;
  const int m0 = B.n[0] - 2 * b, m1 = B.n[1] - 2 * b, m2 = B.n[2] - 2 * b;
  const int H = (m0 + NC - 1) / NC;
  const int HP = (H + PTS - 1) / PTS;
  const long long t = lb * blockDim.x + threadIdx.x;
  if (t >= (long long)HP * m1 * m2) return;
  const int ihp = ((int)t % HP);
  const int r = (int)t / HP;
  const int j = b + (r % m1);
  const int k = b + (r / m1);
  const int delta = (((color - b - j - k) % NC) + NC) % NC;
  float *e = G.f[G_E] + B.off;
  const long long sy = B.n[0], sz = (long long)B.n[0] * B.n[1];
  const long long prow = aq ? B.off + (((long long)color * m2 + (k - b)) * m1 + (j - b)) * H : 0;
  float en[PTS];
  long long pp[PTS];
  bool ok[PTS];
#pragma unroll
  for (int q = 0; q < PTS; q++) {
    const int ih = ihp * PTS + q;
    const int i = b + delta + NC * ih;
    ok[q] = i < B.n[0] - b;
    const int ihq = ok[q] ? ih : 0;   // a point past the row's end repeats the row's first point
    const long long p = pidx(B, b + delta + NC * ihq, j, k);
    pp[q] = p;
    const float lv = lapf<ORD>(e, p, sy, sz, B);
    float op, dop;
    if (aq) {
      const float2 a = __ldcg(aq + prow + ihq);
      const long long g = B.off + p;
      corr_op<EQ>(lv, (float)B.dulap, e[p], a.x, a.y, EQ == 1 ? G.f[G_D][g] : 0.0f, EQ == 1 ? G.f[G_E5][g] : 0.0f,
                  op, dop);
    } else {
      corr_at<EQ>(B, G, p, lv, op, dop);
    }
    en[q] = corr_update(e[p], op, dop, G.f[G_S][B.off + p]);
  }
#pragma unroll
  for (int q = 0; q < PTS; q++)
    if (ok[q]) {
      e[pp[q]] = en[q];
      if (!(en[q] == en[q])) atomicOr(nan_flag, 1);
    }
}

// R = N^u(e) on INSIDE points
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_apply_op32(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const int b = B.buf;
  const int m0 = B.n[0] - 2 * b, m1 = B.n[1] - 2 * b, m2 = B.n[2] - 2 * b;
  const long long t = lb * blockDim.x + threadIdx.x;
  if (t >= (long long)m0 * m1 * m2) return;
  const int i = b + ((int)t % m0);
  const int r = (int)t / m0;
  const int j = b + (r % m1);
  const int k = b + (r / m1);
  const long long p = pidx(B, i, j, k);
  const float lv = lapf<ORD>(G.f[G_E] + B.off, p, B.n[0], (long long)B.n[0] * B.n[1], B);
  float op, dop;
  corr_at<EQ>(B, G, p, lv, op, dop);
  G.f[G_R][B.off + p] = op;
}

// one-sided derivative of e along an axis (dx2 for order 2, dx4 otherwise)
template <int ORD>
__device__ __forceinline__ float derivf(const float *__restrict__ u, long long p, long long s, int i, int n,
                                        float id, float &du)
{
  if (ORD == 2) {
    if (i == 0) {
      du = -1.5f * id;
      return (-3.0f * u[p] + 4.0f * u[p + s] - u[p + 2 * s]) * 0.5f * id;
    }
    if (i == n - 1) {
      du = 1.5f * id;
      return (3.0f * u[p] - 4.0f * u[p - s] + u[p - 2 * s]) * 0.5f * id;
    }
    du = 0.0f;
    return (u[p + s] - u[p - s]) * 0.5f * id;
  } else {
    const int nm = n % 2 == 0 ? n / 2 : (n - 1) / 2;
    if (i <= nm) {
      du = -25.0f * id * (1.0f / 12.0f);
      return -(25.0f * u[p] - 48.0f * u[p + s] + 36.0f * u[p + 2 * s] - 16.0f * u[p + 3 * s] + 3.0f * u[p + 4 * s]) *
             id * (1.0f / 12.0f);
    }
    du = 25.0f * id * (1.0f / 12.0f);
    return (25.0f * u[p] - 48.0f * u[p - s] + 36.0f * u[p - 2 * s] - 16.0f * u[p - 3 * s] + 3.0f * u[p - 4 * s]) *
           id * (1.0f / 12.0f);
  }
}

// Robin on e: mode 0 Newton update with source G_S, mode 1 operator into G_R.
// The condition is linear, so its correction form is the condition itself.
template <int ORD>
__device__ __forceinline__ void robin32_point(const DevBox &B, const DevFields32 &G, const double *__restrict__ crd,
                                              int mode, int mask, int i, int j, int k)
{
  float *e = G.f[G_E] + B.off;
  const double *c = crd + B.coord_off, *ic = c + (B.n[0] + B.n[1] + B.n[2]);   // coordinates, reciprocals
  const float x = (float)c[i];
  const float y = (float)c[B.n[0] + j];
  const float z = (float)c[B.n[0] + B.n[1] + k];
  const float r2 = x * x + y * y + z * z;
  const long long p = pidx(B, i, j, k);
  const long long st[3] = {1, (long long)B.n[0], (long long)B.n[0] * B.n[1]};
  const int ijk[3] = {i, j, k};
  const float ixyz[3] = {(float)ic[i], (float)ic[B.n[0] + j], (float)ic[B.n[0] + B.n[1] + k]};
  float t = 0.0f, dt = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!(mask & (1 << a))) continue;
    float du;
    const float dv = derivf<ORD>(e, p, st[a], ijk[a], B.n[a], (float)B.idx[a], du);
    t += dv * ixyz[a];
    dt += du * ixyz[a];
  }
  if (mode == 0) {
    const float Fv = r2 * t + e[p] - G.f[G_S][B.off + p];
    e[p] = e[p] - Fv * rcp_fast(r2 * dt + 1.0f);
  } else {
    G.f[G_R][B.off + p] = r2 * t + e[p];
  }
}

template <int ORD>
__global__ void __launch_bounds__(256) k_robin32_faces(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G,
                                                       const double *__restrict__ crd, int mode)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const int b = B.buf;
  long long t = lb * blockDim.x + threadIdx.x;
  for (int f = 0; f < 6; f++) {
    const int a = f >> 1, hi = f & 1;
    const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
    const int m1 = B.n[a1] - 2 * b, m2 = B.n[a2] - 2 * b;
    const long long cols = (long long)m1 * m2;
    if (t < cols) {
      int ijk[3];
      ijk[a1] = b + ((int)t % m1);
      ijk[a2] = b + (int)t / m1;
      for (int l = 0; l < b; l++) {
        ijk[a] = hi ? B.n[a] - b + l : b - 1 - l;
        robin32_point<ORD>(B, G, crd, mode, 1 << a, ijk[0], ijk[1], ijk[2]);
      }
      return;
    }
    t -= cols;
  }
}

template <int ORD>
__global__ void __launch_bounds__(64) k_robin32_edges_corners(BoxList L, const DevBox *__restrict__ boxes, DevFields32 F,
                                            const double *__restrict__ crd, int mode, int part)
{
  if (part == 0) {
    // one block per (box, edge): 12 edges a box, (a, c) the edge's ghost axes
    const DevBox B = boxes[L.box[blockIdx.x / 12]];
    if (!B.active) return;
    const int e12 = blockIdx.x % 12, pi = e12 >> 2, e = e12 & 3;
    const int a = pi == 2 ? 1 : 0, c = pi == 0 ? 1 : 2, fa = 3 - a - c;
    const int b = B.buf, m = B.n[fa] - 2 * b;
    const int ha = e >> 1, hc = e & 1;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      int ijk[3];
      ijk[fa] = b + q;
      for (int ta = 0; ta < b; ta++)
        for (int tc = 0; tc < b; tc++) {
          ijk[a] = ha ? B.n[a] - b + ta : b - 1 - ta;
          ijk[c] = hc ? B.n[c] - b + tc : b - 1 - tc;
          robin32_point<ORD>(B, F, crd, mode, (1 << a) | (1 << c), ijk[0], ijk[1], ijk[2]);
        }
    }
    return;
  }
  // corners, after every edge (a launch of their own), one block per box
  const DevBox B = boxes[L.box[blockIdx.x]];
  if (!B.active) return;
  const int b = B.buf;
  if (threadIdx.x < 8) {
    const int hx = threadIdx.x & 1, hy = (threadIdx.x >> 1) & 1, hz = threadIdx.x >> 2;
    for (int tk = 0; tk < b; tk++)
      for (int tj = 0; tj < b; tj++)
        for (int ti = 0; ti < b; ti++) {
          const int i = hx ? B.n[0] - b + ti : b - 1 - ti;
          const int j = hy ? B.n[1] - b + tj : b - 1 - tj;
          const int k = hz ? B.n[2] - b + tk : b - 1 - tk;
          robin32_point<ORD>(B, F, crd, mode, 7, i, j, k);
        }
  }
}

// FP32 Robin of the correction in fewer launches (as k_robin_ec_cluster and
// k_robin_all): the edges and corners of the update in one cluster launch
// per box after the faces' launch, the operator in one flat launch.
template <int ORD>
__global__ void __launch_bounds__(256) k_robin32_ec_cluster(BoxList L, const DevBox *__restrict__ boxes,
                                                            DevFields32 G, const double *__restrict__ crd, int mode)
{
  namespace cg = cooperative_groups;
  const unsigned ncta = cg::this_cluster().num_blocks();
  if ((int)(blockIdx.x / ncta) >= L.count) return;   // the whole cluster: one box a cluster
  const DevBox B = boxes[L.box[blockIdx.x / ncta]];
  if (!B.active) return;   // every block of the cluster reads the same box: all leave
  robin_ec_walk(B, cg::this_cluster().block_rank(), ncta,
                [&](int mask, int i, int j, int k) { robin32_point<ORD>(B, G, crd, mode, mask, i, j, k); });
}

template <int ORD>
__global__ void __launch_bounds__(256) k_robin32_all(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G,
                                                     const double *__restrict__ crd, int mode)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  long long t = lb * blockDim.x + threadIdx.x;
  auto pt = [&](int mask, int i, int j, int k) { robin32_point<ORD>(B, G, crd, mode, mask, i, j, k); };
  const long long nf = robin_face_items(B), ne = robin_edge_items(B);
  if (t < nf) robin_face_item(B, t, pt);
  else if ((t -= nf) < ne) robin_edge_item(B, t, pt);
  else if ((t -= ne) < 8) robin_corner_item(B, (int)t, pt);
}

enum Ew32Op { EW32_W_EQ_S_MINUS_R = 0, EW32_S_EQ_W_PLUS_R, EW32_W_PLUS_EQ_R, EW32_WW_EQ_E, EW32_V_EQ_E_MINUS_WW,
              EW32_E_PLUS_EQ_V, EW32_S_EQ_W_PLUS_R_WW_EQ_E, EW32_W_PLUS_EQ_R_WW_EQ_E };

__global__ void __launch_bounds__(256) k_elementwise32(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G,
                                                       int op)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const long long p = B.off + t;
  switch (op) {
  case EW32_W_EQ_S_MINUS_R: G.f[G_W][p] = G.f[G_S][p] - G.f[G_R][p]; break;
  case EW32_S_EQ_W_PLUS_R: G.f[G_S][p] = G.f[G_W][p] + G.f[G_R][p]; break;
  case EW32_W_PLUS_EQ_R: G.f[G_W][p] = G.f[G_W][p] + G.f[G_R][p]; break;
  case EW32_WW_EQ_E: G.f[G_WW][p] = G.f[G_E][p]; break;
  case EW32_V_EQ_E_MINUS_WW: G.f[G_V][p] = G.f[G_E][p] - G.f[G_WW][p]; break;
  case EW32_E_PLUS_EQ_V: G.f[G_E][p] = G.f[G_E][p] + G.f[G_V][p]; break;
  case EW32_S_EQ_W_PLUS_R_WW_EQ_E:   // two steps of one level in one pass
    G.f[G_S][p] = G.f[G_W][p] + G.f[G_R][p];
    G.f[G_WW][p] = G.f[G_E][p];
    break;
  case EW32_W_PLUS_EQ_R_WW_EQ_E:
    G.f[G_W][p] = G.f[G_W][p] + G.f[G_R][p];
    G.f[G_WW][p] = G.f[G_E][p];
    break;
  }
}

// T = (1,2,1)^3/64 average of W = S - R on INSIDE points (see k_full_weight),
// W formed where it is read (it is needed for nothing else)
__global__ void __launch_bounds__(256) k_full_weight32(BoxList L, const DevBox *__restrict__ boxes, DevFields32 G)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int b = B.buf;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const float *gs = G.f[G_S] + B.off, *gr = G.f[G_R] + B.off;
  auto w = [&](long long q) { return gs[q] - gr[q]; };
  const float c = w(t);
  const bool inside = i >= b && i < B.n[0] - b && j >= b && j < B.n[1] - b && k >= b && k < B.n[2] - b;
  if (!inside) {
    G.f[G_T][B.off + t] = c;
    return;
  }
  G.f[G_T][B.off + t] = fw_sum<float>(w, c, B, i, j, k, t);
}

// Set_In of a refinement level with the coarse operator folded in: at every
// target of the (strided, same-box) Set_In plan S = W + N(e), N evaluated as
// k_apply_op32 does on INSIDE points and 0 on the ghosts (where R is 0 on a
// refinement level).  The coarse R is needed nowhere else, so it is formed
// only where Set_In copies, not on the whole level.
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_set_in_op32(const XferJob *__restrict__ jobs, int njobs,
                                                     const DevBox *__restrict__ boxes, DevFields32 G)
{
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].blk0 <= (long long)blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const XferJob &J = jobs[lo];
  if (!boxes[J.tbox].active) return;   // the target's solve has stopped (whole block: one job)
  const long long t = ((long long)blockIdx.x - J.blk0) * blockDim.x + threadIdx.x;
  const int e0 = J.r1[0] - J.r0[0], e1 = J.r1[1] - J.r0[1], e2 = J.r1[2] - J.r0[2];
  if (t >= (long long)e0 * e1 * e2) return;
  const int i = J.r0[0] + ((int)t % e0);
  const int r = (int)t / e0;
  const int j = J.r0[1] + (r % e1);
  const int k = J.r0[2] + (r / e1);
  const DevBox T = boxes[J.tbox];
  const DevBox &S = boxes[J.sbox];
  const long long sp = pidx(S, J.sstart[0] + J.sstep[0] * (i - J.r0[0]), J.sstart[1] + J.sstep[1] * (j - J.r0[1]),
                            J.sstart[2] + J.sstep[2] * (k - J.r0[2]));
  const long long tp = pidx(T, i, j, k);
  const int b = T.buf;
  float rr = 0.0f;
  if (i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b) {
    const float lv = lapf<ORD>(G.f[G_E] + T.off, tp, T.n[0], (long long)T.n[0] * T.n[1], T);
    float op, dop;
    corr_at<EQ>(T, G, tp, lv, op, dop);
    rr = op;
  }
  G.f[G_S][T.off + tp] = G.f[G_W][S.off + sp] + rr;
}

// Coarsest correction problem of one solve in one CTA: repeat { Robin; one
// red-black SOR sweep } until the sweep norm <= rtol * first, stops
// changing, or max_it.  e lives in shared memory; with SMEM the read-only
// coefficients (A, 1/(c+u), source, and d, E5 for the scalar field) are
// staged there too, so an iteration touches no global memory.  Block b
// solves box L.box[b], so the coarsest problems of every solve of a batch
// that ends at this level run side by side in one launch; the iteration
// count and NaN flag go to that box's solve (stats[B.solve]).
template <int EQ, bool SMEM>
__global__ void __launch_bounds__(1024) k_coarse32(const DevBox *__restrict__ boxes, BoxList L, DevFields32 G,
                                                   const double *__restrict__ crd, int max_it, float omega, float rtol,
                                                   Stats *stats)
{
  extern __shared__ float4 s_coarse4[];
  float *se = reinterpret_cast<float *>(s_coarse4);
  __shared__ float red[32];
  __shared__ float s_norm;
  __shared__ int s_nan;
  __shared__ float s_x[3][64], s_ix[3][64];   // node coordinates and their reciprocals
  if ((int)blockIdx.x >= L.count) return;
  const DevBox B = boxes[L.box[blockIdx.x]];
  if (!B.active) return;   // the whole block
  int *iters_out = &stats[B.solve].coarse_iters, *nan_flag = &stats[B.solve].nan_flag;
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
  const int np = n0 * n1 * n2;
  float *ge = G.f[G_E] + B.off;
  const float *gs = G.f[G_S] + B.off, *ga = G.f[G_A] + B.off, *giq = G.f[G_IQ] + B.off;
  const float *gd = EQ == 1 ? G.f[G_D] + B.off : nullptr, *ge5 = EQ == 1 ? G.f[G_E5] + B.off : nullptr;
  float *cs = se + np, *ca = se + 2 * np, *ciq = se + 3 * np, *cd = se + 4 * np, *ce5 = se + 5 * np;
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    se[p] = ge[p];
    if (SMEM) {
      cs[p] = gs[p];
      ca[p] = ga[p];
      ciq[p] = giq[p];
      if (EQ) {
        cd[p] = gd[p];
        ce5[p] = ge5[p];
      }
    }
  }
  const float *S_ = SMEM ? cs : gs, *A_ = SMEM ? ca : ga, *IQ_ = SMEM ? ciq : giq;
  const float *D_ = SMEM ? cd : gd, *E5_ = SMEM ? ce5 : ge5;
  for (int t = threadIdx.x; t < n0 + n1 + n2; t += blockDim.x) {
    const int a = t < n0 ? 0 : t < n0 + n1 ? 1 : 2;
    const int i = t - (a == 0 ? 0 : a == 1 ? n0 : n0 + n1);
    const float x = (float)crd[B.coord_off + t];
    s_x[a][i] = x;
    s_ix[a][i] = x != 0.0f ? rcp_fast(x) : 0.0f;
  }
  __syncthreads();
  const int m0 = n0 - 2, m1 = n1 - 2, m2 = n2 - 2;
  const int sy = n0, sz = n0 * n1;
  const float dl = (float)B.dulap;
  const float ix2 = (float)B.idx2[0], iy2 = (float)B.idx2[1], iz2 = (float)B.idx2[2];
  const float idx[3] = {(float)B.idx[0], (float)B.idx[1], (float)B.idx[2]};
  const int nn[3] = {n0, n1, n2};
  const int st[3] = {1, sy, sz};
  auto robin = [&](int mask, int i, int j, int k) {
    const int ijk[3] = {i, j, k};
    const float r2 = s_x[0][i] * s_x[0][i] + s_x[1][j] * s_x[1][j] + s_x[2][k] * s_x[2][k];
    const int p = (k * n1 + j) * n0 + i;
    float t = 0.0f, dt = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (!(mask & (1 << a))) continue;
      float du;
      const float dv = derivf<2>(se, p, st[a], ijk[a], nn[a], idx[a], du);
      t += dv * s_ix[a][ijk[a]];
      dt += du * s_ix[a][ijk[a]];
    }
    const float Fv = r2 * t + se[p] - S_[p];
    se[p] = se[p] - Fv * rcp_fast(r2 * dt + 1.0f);
  };
  auto nof = [&](int a) { return a == 0 ? n0 : a == 1 ? n1 : n2; };
  // point with coordinate va on axis a, vb on axis b2, vc on the third
  auto at = [&](int a, int va, int b2, int vb, int vc, int mask) {
    const int i = a == 0 ? va : b2 == 0 ? vb : vc;
    const int j = a == 1 ? va : b2 == 1 ? vb : vc;
    const int k = a == 2 ? va : b2 == 2 ? vb : vc;
    robin(mask, i, j, k);
  };
  float norm = 1.0f, prev, first = -1.0f;
  int it = 0;
  do {
    prev = norm;
    // faces (2 per axis), then edges, then corners
    {
      const int f0 = m1 * m2, f1 = m0 * m2, f2 = m0 * m1;
      for (int t = threadIdx.x; t < 2 * (f0 + f1 + f2); t += blockDim.x) {
        int q = t, a;
        if (q < 2 * f0) a = 0;
        else if ((q -= 2 * f0) < 2 * f1) a = 1;
        else {
          q -= 2 * f1;
          a = 2;
        }
        const int cnt = a == 0 ? f0 : a == 1 ? f1 : f2;
        const int hi = q >= cnt ? 1 : 0;
        q -= hi * cnt;
        const int a1 = a == 2 ? 0 : a + 1;
        const int c1 = nof(a1) - 2;
        at(a, hi ? nof(a) - 1 : 0, a1, 1 + q % c1, 1 + q / c1, 1 << a);
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 4 * (m0 + m1 + m2); t += blockDim.x) {
      // edges along axis fa (4 each): XY edges (fa = 2), XZ (1), YZ (0)
      int q = t, fa;
      if (q < 4 * m2) fa = 2;
      else if ((q -= 4 * m2) < 4 * m1) fa = 1;
      else {
        q -= 4 * m1;
        fa = 0;
      }
      const int m = nof(fa) - 2;
      const int e = q / m, r = q % m;
      const int a = fa == 0 ? 1 : 0, c = fa == 2 ? 1 : 2;
      at(a, (e >> 1) ? nof(a) - 1 : 0, c, (e & 1) ? nof(c) - 1 : 0, 1 + r, (1 << a) | (1 << c));
    }
    __syncthreads();
    if (threadIdx.x < 8)
      robin(7, (threadIdx.x & 1) ? n0 - 1 : 0, ((threadIdx.x >> 1) & 1) ? n1 - 1 : 0, (threadIdx.x >> 2) ? n2 - 1 : 0);
    __syncthreads();
    float rmax = 0.0f;
    int nan_seen = 0;
    const int H = (m0 + 1) / 2;
    for (int color = 0; color < 2; color++) {
      for (int t = threadIdx.x; t < H * m1 * m2; t += blockDim.x) {
        const int ih = t % H, r = t / H;
        const int j = 1 + r % m1, k = 1 + r / m1;
        const int i = 1 + ((color + 1 + j + k) & 1) + 2 * ih;
        if (i >= n0 - 1) continue;
        const int p = (k * n1 + j) * n0 + i;
        const float c0 = se[p];
        const float lv = (se[p + 1] - 2.0f * c0 + se[p - 1]) * ix2 + (se[p + sy] - 2.0f * c0 + se[p - sy]) * iy2 +
                         (se[p + sz] - 2.0f * c0 + se[p - sz]) * iz2;
        float op, dop;
        corr_op<EQ>(lv, dl, c0, A_[p], IQ_[p], EQ == 1 ? D_[p] : 0.0f, EQ == 1 ? E5_[p] : 0.0f, op, dop);
        const float R = op - S_[p];
        const float en = c0 - omega * (R * rcp_fast(dop));
        se[p] = en;
        rmax = fmaxf(rmax, fabsf(R));
        if (!(en == en)) nan_seen = 1;
      }
      __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    nan_seen = __syncthreads_or(nan_seen);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = rmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      float m = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
      s_norm = m;
      s_nan = nan_seen;
      if (nan_seen) atomicOr(nan_flag, 1);
    }
    __syncthreads();
    norm = s_norm;
    const int stop_nan = s_nan;
    __syncthreads();
    it++;
    if (first < 0.0f) first = norm;
    if (stop_nan) break;
    if (norm <= rtol * first) break;
  } while (norm > 0.0f && prev != norm && it < max_it);
  for (int p = threadIdx.x; p < np; p += blockDim.x) ge[p] = se[p];
  if (threadIdx.x == 0) *iters_out = it;
}

// Blocks of k_coarse32_cluster's clusters (portable size).
constexpr int kCoarse32Ncta = 8;

// Points of the largest slab of k_coarse32_cluster on a box: each of its
// shared arrays (e and the staged S, A, 1/(c+u), and d, E5) holds that many
// floats in every block.
__host__ __device__ inline int coarse32_cluster_slab(int n0, int n1, int n2, int ncta)
{
  int smax = 0;
  for (int r = 0; r < ncta; r++) {
    const int planes = cslab_begin(r + 1, n2, ncta) - cslab_begin(r, n2, ncta);
    smax = planes * n0 * n1 > smax ? planes * n0 * n1 : smax;
  }
  return smax;
}

// k_coarse32's iteration with the box spread over a cluster of NCTA blocks,
// one cluster per box (the coarsest problems of a batch's solves side by
// side): the z-planes split as in k_coarse_cluster (block 0 owns the low
// ghost plane and the two interior planes above it, the last block the
// mirror image, so the Robin update -- faces, edges, corners -- stays inside
// a block), e in the blocks' shared memory with the other blocks' planes read
// through distributed shared memory, and each block's S, A, 1/(c+u) (d, E5)
// staged beside its slab.  A sweep needs a cluster barrier after colour 0
// (colour 1 reads its z neighbours) and one after colour 1 (the norm, and the
// next colour 0).  Every block reads every block's partial norm in the same
// order, so all take the same stop decision.  The updates are k_coarse32's.
template <int EQ, int NCTA>
__global__ void __launch_bounds__(256) k_coarse32_cluster(const DevBox *__restrict__ boxes, BoxList L, DevFields32 G,
                                                          const double *__restrict__ crd, int max_it, float omega,
                                                          float rtol, Stats *stats)
{
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ float4 s_c32[];
  float *se = reinterpret_cast<float *>(s_c32);
  __shared__ float *plane[64];
  __shared__ float red[8];               // one slot per warp (256 threads)
  __shared__ int red_nan[8];
  __shared__ float s_part[2][2];         // per iteration parity: max |R| of this block, NaN seen
  __shared__ float s_x[3][64], s_ix[3][64];

  if ((int)(blockIdx.x / NCTA) >= L.count) return;   // the whole cluster: one box a cluster
  const DevBox B = boxes[L.box[blockIdx.x / NCTA]];
  if (!B.active) return;   // every block of the cluster reads the same box: all leave
  int *iters_out = &stats[B.solve].coarse_iters, *nan_flag = &stats[B.solve].nan_flag;
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
  const int n01 = n0 * n1;
  const int kz0 = cslab_begin(rank, n2, NCTA), kz1 = cslab_begin(rank + 1, n2, NCTA);
  const int slab = (kz1 - kz0) * n01;
  const int smax = coarse32_cluster_slab(n0, n1, n2, NCTA);
  float *cs = se + smax, *ca = se + 2 * smax, *ciq = se + 3 * smax;
  float *cd = se + 4 * smax, *ce5 = se + 5 * smax;   // scalar field only
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    int r = 0;
    while (cslab_begin(r + 1, n2, NCTA) <= k) r++;
    plane[k] = cl.map_shared_rank(se, r) + (k - cslab_begin(r, n2, NCTA)) * n01;
  }
  float *ge = G.f[G_E] + B.off;
  const long long g0 = (long long)kz0 * n01;
  for (int p = threadIdx.x; p < slab; p += blockDim.x) {
    se[p] = ge[g0 + p];
    cs[p] = G.f[G_S][B.off + g0 + p];
    ca[p] = G.f[G_A][B.off + g0 + p];
    ciq[p] = G.f[G_IQ][B.off + g0 + p];
    if (EQ == 1) {
      cd[p] = G.f[G_D][B.off + g0 + p];
      ce5[p] = G.f[G_E5][B.off + g0 + p];
    }
  }
  for (int t = threadIdx.x; t < n0 + n1 + n2; t += blockDim.x) {
    const int a = t < n0 ? 0 : t < n0 + n1 ? 1 : 2;
    const int i = t - (a == 0 ? 0 : a == 1 ? n0 : n0 + n1);
    const float x = (float)crd[B.coord_off + t];
    s_x[a][i] = x;
    s_ix[a][i] = x != 0.0f ? rcp_fast(x) : 0.0f;
  }
  cl.sync();   // every block's slab and plane table are in place

  auto E = [&](int i, int j, int k) -> float & { return plane[k][j * n0 + i]; };
  auto own = [&](int i, int j, int k) { return (k - kz0) * n01 + j * n0 + i; };   // this block's staged arrays
  const float dl = (float)B.dulap;
  const float ix2 = (float)B.idx2[0], iy2 = (float)B.idx2[1], iz2 = (float)B.idx2[2];
  const float idx[3] = {(float)B.idx[0], (float)B.idx[1], (float)B.idx[2]};
  // derivf<2> at a ghost position: one-sided, pointing inward
  auto d1 = [&](int a, int i, int j, int k, float &du) -> float {
    const int ijk[3] = {i, j, k};
    const int s = ijk[a] == 0 ? 1 : -1;
    int p1[3] = {i, j, k}, p2[3] = {i, j, k};
    p1[a] += s;
    p2[a] += 2 * s;
    const float u0 = E(i, j, k), u1 = E(p1[0], p1[1], p1[2]), u2 = E(p2[0], p2[1], p2[2]);
    if (ijk[a] == 0) {
      du = -1.5f * idx[a];
      return (-3.0f * u0 + 4.0f * u1 - u2) * 0.5f * idx[a];
    }
    du = 1.5f * idx[a];
    return (3.0f * u0 - 4.0f * u1 + u2) * 0.5f * idx[a];
  };
  auto robin = [&](int mask, int i, int j, int k) {
    const int ijk[3] = {i, j, k};
    const float r2 = s_x[0][i] * s_x[0][i] + s_x[1][j] * s_x[1][j] + s_x[2][k] * s_x[2][k];
    float t = 0.0f, dt = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (!(mask & (1 << a))) continue;
      float du;
      const float dv = d1(a, i, j, k, du);
      t += dv * s_ix[a][ijk[a]];
      dt += du * s_ix[a][ijk[a]];
    }
    float &ee = E(i, j, k);
    const float Fv = r2 * t + ee - cs[own(i, j, k)];
    ee = ee - Fv * rcp_fast(r2 * dt + 1.0f);
  };

  float norm = 1.0f, prev, first = -1.0f;
  int it = 0;
  const int mi0 = n0 - 2, mi1 = n1 - 2;
  do {
    prev = norm;
    // Robin update of this block's planes: faces, then edges, then corners
    for (int k = kz0; k < kz1; k++) {
      if (k == 0 || k == n2 - 1) {
        for (int t = threadIdx.x; t < mi0 * mi1; t += blockDim.x) robin(4, 1 + t % mi0, 1 + t / mi0, k);
      } else {
        for (int t = threadIdx.x; t < 2 * mi1 + 2 * mi0; t += blockDim.x) {
          if (t < 2 * mi1) robin(1, (t & 1) ? n0 - 1 : 0, 1 + (t >> 1), k);
          else {
            const int q = t - 2 * mi1;
            robin(2, 1 + (q >> 1), (q & 1) ? n1 - 1 : 0, k);
          }
        }
      }
    }
    __syncthreads();
    for (int k = kz0; k < kz1; k++) {
      if (k == 0 || k == n2 - 1) {
        for (int t = threadIdx.x; t < 2 * mi1 + 2 * mi0; t += blockDim.x) {
          if (t < 2 * mi1) robin(5, (t & 1) ? n0 - 1 : 0, 1 + (t >> 1), k);   // x-z edges
          else {
            const int q = t - 2 * mi1;
            robin(6, 1 + (q >> 1), (q & 1) ? n1 - 1 : 0, k);                   // y-z edges
          }
        }
      } else if (threadIdx.x < 4) {
        robin(3, (threadIdx.x & 1) ? n0 - 1 : 0, (threadIdx.x & 2) ? n1 - 1 : 0, k);   // x-y edges
      }
    }
    __syncthreads();
    for (int k = kz0; k < kz1; k++)
      if ((k == 0 || k == n2 - 1) && threadIdx.x < 4)
        robin(7, (threadIdx.x & 1) ? n0 - 1 : 0, (threadIdx.x & 2) ? n1 - 1 : 0, k);
    __syncthreads();
    // one red-black SOR sweep over the interior points of this block's planes
    float rmax = 0.0f;
    int nan_seen = 0;
    const int ka = kz0 > 1 ? kz0 : 1, kb = kz1 < n2 - 1 ? kz1 : n2 - 1;
    const int H = (mi0 + 1) / 2;
    const int work = H * mi1 * (kb > ka ? kb - ka : 0);
    for (int color = 0; color < 2; color++) {
      for (int t = threadIdx.x; t < work; t += blockDim.x) {
        const int ih = t % H, r = t / H;
        const int j = 1 + r % mi1, k = ka + r / mi1;
        const int i = 1 + ((color + 1 + j + k) & 1) + 2 * ih;
        if (i >= n0 - 1) continue;
        const float c0 = E(i, j, k);
        const float lv = (E(i + 1, j, k) - 2.0f * c0 + E(i - 1, j, k)) * ix2 +
                         (E(i, j + 1, k) - 2.0f * c0 + E(i, j - 1, k)) * iy2 +
                         (E(i, j, k + 1) - 2.0f * c0 + E(i, j, k - 1)) * iz2;
        const int q = own(i, j, k);
        float op, dop;
        corr_op<EQ>(lv, dl, c0, ca[q], ciq[q], EQ == 1 ? cd[q] : 0.0f, EQ == 1 ? ce5[q] : 0.0f, op, dop);
        const float R = op - cs[q];
        const float en = c0 - omega * (R * rcp_fast(dop));
        E(i, j, k) = en;
        rmax = fmaxf(rmax, fabsf(R));
        if (!(en == en)) nan_seen = 1;
      }
      if (color == 0) cl.sync();   // colour 1 reads colour 0 of the neighbouring blocks
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
      nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = rmax;
      red_nan[threadIdx.x >> 5] = nan_seen;
    }
    __syncthreads();
    const int par = it & 1;
    if (threadIdx.x == 0) {
      float m = 0.0f;
      int nn = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        m = fmaxf(m, red[w]);
        nn |= red_nan[w];
      }
      s_part[par][0] = m;
      s_part[par][1] = nn ? 1.0f : 0.0f;
    }
    cl.sync();   // every block's colour 1 and partial norm are done
    // the slot of this parity is written again two iterations later, after
    // two more cluster barriers that this block must reach first
    float m = 0.0f, nanv = 0.0f;
#pragma unroll
    for (int r = 0; r < NCTA; r++) {
      const float *pr = cl.map_shared_rank(&s_part[par][0], r);
      m = fmaxf(m, pr[0]);
      nanv = fmaxf(nanv, pr[1]);
    }
    norm = m;
    it++;
    if (first < 0.0f) first = norm;
    if (nanv > 0.0f) {
      if (rank == 0 && threadIdx.x == 0) atomicOr(nan_flag, 1);
      break;                                       // the same decision in every block
    }
    if (norm <= rtol * first) break;
  } while (norm > 0.0f && prev != norm && it < max_it);
  cl.sync();   // every block is done reading the others' shared memory
  for (int p = threadIdx.x; p < slab; p += blockDim.x) ge[g0 + p] = se[p];
  if (rank == 0 && threadIdx.x == 0) *iters_out = it;
}

}  // namespace olgpu

namespace olgpu {

// ---------------------------------------------------------------------------
// Anderson acceleration of the outer iteration u_{k+1} = Phi(u_k) (one mixed
// cycle).  With f_k = Phi(u_k) - u_k (the cycle's correction e) and the last
// m differences dU_j = u_j - u_{j-1}, dF_j = f_j - f_{j-1}:
//     gamma = argmin || f_k - dF gamma ||_2   (over the pinned points)
//     u_{k+1} = u_k + f_k - (dU + dF) gamma.
// A fixed point of Phi is a fixed point of this iteration, so the solution is
// the same; the slow smooth mode of the FAS-FAC cycle (about 0.65 per cycle
// on the coarse levels under the refinement boxes) is damped much faster.
// Differences are stored in FP32 (they are correction-sized); sums in FP64.
// ---------------------------------------------------------------------------
constexpr int kAndMax = 4;   // largest history depth (deeper histories did not cut cycles)
constexpr int kAndDefault = 4;

struct AndersonState {
  int k;            // outer iterations done since the last reset
  int m;            // history depth (<= kAndMax)
  int k_used;       // iteration the last solve was for
  int pad;
  double gram[kAndMax * kAndMax];
  double rhs[kAndMax];
  double gamma[kAndMax];
};

// dF_k = f_k - f_{k-1} into its ring slot, f_prev = f_k, and the normal
// equations (dF^T dF, dF^T f_k) over pinned points; also max |f_k| pinned.
// Per-block partial sums go to part[blockIdx.x * kAndPart + ...] and are added
// in block order by k_and_solve, so the result does not depend on scheduling.
constexpr int kAndPart = kAndMax * (kAndMax + 1) / 2 + kAndMax;

__global__ void __launch_bounds__(256) k_and_reduce(long long n, const float *__restrict__ f, float *fprev,
                                                    float *DF, const unsigned char *__restrict__ pinned,
                                                    const AndersonState *st, double *part,
                                                    unsigned long long *fmax_slot, const DevBox *__restrict__ gate)
{
  if (!gate->active) return;   // the solve has stopped (batch): the whole grid leaves
  const int k = st->k, m = st->m;
  const int nc = k < m ? k : m;
  const int newest = (k + m - 1) % m;   // ring slot of dF_k (k >= 1)
  // column i of the fit is dF at ring slot (newest - i) mod m
  const float *dfc[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax; i++) dfc[i] = DF + (long long)((newest - i + 2 * kAndMax * m) % m) * n;
  float *dfw = DF + (long long)newest * n;
  // a thread's products are summed in FP32 (a few dozen points each), the
  // thread partials in FP64
  float g[kAndMax * (kAndMax + 1) / 2], r[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax * (kAndMax + 1) / 2; i++) g[i] = 0.0f;
#pragma unroll
  for (int i = 0; i < kAndMax; i++) r[i] = 0.0f;
  float fm = 0.0f;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const float fk = f[p];
    if (k >= 1) dfw[p] = fk - fprev[p];
    fprev[p] = fk;
    if (!pinned[p]) continue;
    fm = fmaxf(fm, fabsf(fk));
    float c[kAndMax];
#pragma unroll
    for (int i = 0; i < kAndMax; i++) {
      c[i] = i < nc ? dfc[i][p] : 0.0f;
      r[i] += c[i] * fk;
    }
    int q = 0;
#pragma unroll
    for (int i = 0; i < kAndMax; i++)
#pragma unroll
      for (int j = 0; j <= i; j++) g[q++] += c[i] * c[j];
  }
  __shared__ double red[32];
  auto block_sum = [&](double v) -> double {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    __syncthreads();
    return s;
  };
  double *mine = part + (long long)blockIdx.x * kAndPart;
  int q = 0;
#pragma unroll
  for (int i = 0; i < kAndMax; i++) {
    const double s = block_sum((double)r[i]);
    if (threadIdx.x == 0) mine[kAndMax * (kAndMax + 1) / 2 + i] = s;
#pragma unroll
    for (int j = 0; j <= i; j++) {
      const double t = block_sum((double)g[q]);
      if (threadIdx.x == 0) mine[q] = t;
      q++;
    }
  }
  block_max_atomic((double)fm, fmax_slot);
}

// Solves the regularised normal equations for gamma.  Launched with
// kAndSolveWarps warps: warp w adds partials w, w + kAndSolveWarps, ... of
// every block (lane l takes blocks l, l + 32, ...; then a fixed butterfly),
// so the sums do not depend on scheduling; thread 0 then eliminates.
constexpr int kAndSolveWarps = kAndPart < 32 ? kAndPart : 32;

__global__ void __launch_bounds__(32 * kAndSolveWarps) k_and_solve(AndersonState *st, const double *__restrict__ part,
                                                                   int nblocks, const DevBox *__restrict__ gate)
{
  if (!gate->active) return;
  __shared__ double tot[kAndPart];
  const int lane = threadIdx.x & 31;
  for (int v = threadIdx.x >> 5; v < kAndPart; v += kAndSolveWarps) {
    double s = 0.0;
    for (int blk = lane; blk < nblocks; blk += 32) s += part[(long long)blk * kAndPart + v];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tot[v] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int k = st->k, m = st->m;
  const int nc = k < m ? k : m;
  double A[kAndMax][kAndMax], b[kAndMax];
  double tr = 0.0;
  int q = 0;
  for (int i = 0; i < nc; i++) {
    b[i] = tot[kAndMax * (kAndMax + 1) / 2 + i];
    for (int j = 0; j <= i; j++) {
      A[i][j] = A[j][i] = tot[q];
      q++;
    }
    tr += A[i][i];
  }
  for (int i = 0; i < nc; i++) A[i][i] += 1e-10 * tr / (nc > 0 ? nc : 1);
  bool ok = nc > 0 && tr > 0.0;
  for (int c = 0; c < nc && ok; c++) {           // Gaussian elimination, partial pivoting
    int piv = c;
    for (int i = c + 1; i < nc; i++)
      if (fabs(A[i][c]) > fabs(A[piv][c])) piv = i;
    if (!(fabs(A[piv][c]) > 1e-300)) { ok = false; break; }
    for (int j = 0; j < nc; j++) { const double t = A[c][j]; A[c][j] = A[piv][j]; A[piv][j] = t; }
    { const double t = b[c]; b[c] = b[piv]; b[piv] = t; }
    for (int i = c + 1; i < nc; i++) {
      const double fct = A[i][c] / A[c][c];
      for (int j = c; j < nc; j++) A[i][j] -= fct * A[c][j];
      b[i] -= fct * b[c];
    }
  }
  for (int i = nc - 1; i >= 0 && ok; i--) {
    double s = b[i];
    for (int j = i + 1; j < nc; j++) s -= A[i][j] * st->gamma[j];
    st->gamma[i] = s / A[i][i];
    if (!(st->gamma[i] == st->gamma[i])) ok = false;
  }
  if (!ok)
    for (int i = 0; i < kAndMax; i++) st->gamma[i] = 0.0;
  for (int i = nc; i < kAndMax; i++) st->gamma[i] = 0.0;
  st->k_used = k;
  for (int i = 0; i < kAndMax * kAndMax; i++) st->gram[i] = 0.0;
  for (int i = 0; i < kAndMax; i++) st->rhs[i] = 0.0;
  st->k = k + 1;
}

// u_{k+1} = u_k + f_k - sum gamma_i (dU_i + dF_i); stores dU_{k+1}.
__global__ void __launch_bounds__(256) k_and_update(long long n, double *u, const float *__restrict__ f, float *DU,
                                                    const float *__restrict__ DF, const AndersonState *st,
                                                    const DevBox *__restrict__ gate)
{
  if (!gate->active) return;
  const int k = st->k_used, m = st->m;
  const int nc = k < m ? k : m;
  const int newest = (k + m - 1) % m;
  float *du_out = DU + (long long)(k % m) * n;   // ring slot of dU_{k+1}
  const float *duc[kAndMax], *dfc[kAndMax];
  float gam[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax; i++) {
    const long long slot = (newest - i + 2 * kAndMax * m) % m;
    duc[i] = DU + slot * n;
    dfc[i] = DF + slot * n;
    gam[i] = i < nc ? (float)st->gamma[i] : 0.0f;
  }
  // the step is a correction: FP32 is enough for it; u accumulates in FP64
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    float step = f[p];
#pragma unroll
    for (int i = 0; i < kAndMax; i++)
      if (i < nc) step -= gam[i] * (duc[i][p] + dfc[i][p]);
    u[p] = u[p] + (double)step;
    du_out[p] = step;
  }
}

// The same acceleration of the plain FP64 cycle, with its history in FP64:
// f_k = u - up (up: u as the cycle found it), u_{k+1} = up + f_k - (dU + dF)
// gamma.  Every stored quantity and every sum is FP64, so the iteration stays
// FP64 throughout; its fixed point is the FP64 cycle's.
__global__ void __launch_bounds__(256) k_and_reduce64(long long n, const double *__restrict__ u,
                                                      const double *__restrict__ up, double *fprev, double *DF,
                                                      const unsigned char *__restrict__ pinned, const AndersonState *st,
                                                      double *part, unsigned long long *fmax_slot,
                                                      const DevBox *__restrict__ gate)
{
  if (!gate->active) return;   // the solve has stopped (batch): the whole grid leaves
  const int k = st->k, m = st->m;
  const int nc = k < m ? k : m;
  const int newest = (k + m - 1) % m;
  const double *dfc[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax; i++) dfc[i] = DF + (long long)((newest - i + 2 * kAndMax * m) % m) * n;
  double *dfw = DF + (long long)newest * n;
  double g[kAndMax * (kAndMax + 1) / 2], r[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax * (kAndMax + 1) / 2; i++) g[i] = 0.0;
#pragma unroll
  for (int i = 0; i < kAndMax; i++) r[i] = 0.0;
  double fm = 0.0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const double fk = u[p] - up[p];
    if (k >= 1) dfw[p] = fk - fprev[p];
    fprev[p] = fk;
    if (!pinned[p]) continue;
    fm = fmax(fm, fabs(fk));
    double c[kAndMax];
#pragma unroll
    for (int i = 0; i < kAndMax; i++) {
      c[i] = i < nc ? dfc[i][p] : 0.0;
      r[i] += c[i] * fk;
    }
    int q = 0;
#pragma unroll
    for (int i = 0; i < kAndMax; i++)
#pragma unroll
      for (int j = 0; j <= i; j++) g[q++] += c[i] * c[j];
  }
  __shared__ double red[32];
  auto block_sum = [&](double v) -> double {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    __syncthreads();
    return s;
  };
  double *mine = part + (long long)blockIdx.x * kAndPart;
  int q = 0;
#pragma unroll
  for (int i = 0; i < kAndMax; i++) {
    const double s = block_sum(r[i]);
    if (threadIdx.x == 0) mine[kAndMax * (kAndMax + 1) / 2 + i] = s;
#pragma unroll
    for (int j = 0; j <= i; j++) {
      const double t = block_sum(g[q]);
      if (threadIdx.x == 0) mine[q] = t;
      q++;
    }
  }
  block_max_atomic(fm, fmax_slot);
}

__global__ void __launch_bounds__(256) k_and_update64(long long n, double *u, const double *__restrict__ up,
                                                      double *DU, const double *__restrict__ DF,
                                                      const AndersonState *st, const DevBox *__restrict__ gate)
{
  if (!gate->active) return;
  const int k = st->k_used, m = st->m;
  const int nc = k < m ? k : m;
  const int newest = (k + m - 1) % m;
  double *du_out = DU + (long long)(k % m) * n;
  const double *duc[kAndMax], *dfc[kAndMax];
  double gam[kAndMax];
#pragma unroll
  for (int i = 0; i < kAndMax; i++) {
    const long long slot = (newest - i + 2 * kAndMax * m) % m;
    duc[i] = DU + slot * n;
    dfc[i] = DF + slot * n;
    gam[i] = i < nc ? st->gamma[i] : 0.0;
  }
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    double step = u[p] - up[p];
#pragma unroll
    for (int i = 0; i < kAndMax; i++)
      if (i < nc) step -= gam[i] * (duc[i][p] + dfc[i][p]);
    u[p] = up[p] + step;
    du_out[p] = step;
  }
}

}  // namespace olgpu
