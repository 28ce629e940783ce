// kernels.cuh -- sm_103a kernels of the FP64 puncture FAS V-cycle.
//
// Reference path (WuShichao/OllipticID):
//   smoother          elliptic::Smooth              src/elliptic.cc:1126-1242
//   operator          puncture_OP / puncture_duOP   include/elliptic.h:405-445
//   stencils          Lapc2/4/6/8, duLapc*          include/ffunction.h:1290-1524,
//                                                   src/diff_4th.cc:392-410, src/diff_8th.cc:596-674
//   Robin boundary    App_Bound, Boundary_*         src/boundary.cc:447-1101
//   Robin operator    App_Boundary_Operator         src/boundary.cc:1118-1710
//   one-sided d/dx    dx2, dx4 (+ du*)              src/diff_2nd.cc:238-335, src/diff_4th.cc:6-89
//   residual          App_Ell_Operator              src/elliptic.cc:943-991
//   transfers         Transferir, Set_In            src/ffunction.cc:2435-2849
//   interpolation     Lagrange/Linear_Interpol_In   src/interpolation.cc:124-375
//   coefficients      punctures_b/_c, scalar d/e    src/operator.cc:2193-2380
//
// The smoother is multicolour (red-black for order 2) instead of
// lexicographic: every colour pass updates its points in parallel.  That
// changes the iterates but not the discrete fixed point, which is what the
// solver is compared on.
#pragma once

#include "device.cuh"

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cfloat>

namespace olgpu {

__device__ __forceinline__ long long pidx(const DevBox &B, int i, int j, int k)
{
  return ((long long)k * B.n[1] + j) * B.n[0] + i;
}

// Finds the box of this block inside a BoxList launch (the last entry whose
// first block is <= blockIdx.x).
__device__ __forceinline__ int list_box(const BoxList &L, long long &local_block)
{
  int lo = 0, hi = L.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long long)blockIdx.x >= L.blk[mid]) lo = mid;
    else hi = mid - 1;
  }
  local_block = (long long)blockIdx.x - L.blk[lo];
  return L.box[lo];
}

// ----------------------------------------------------------------------------
// stencils
// ----------------------------------------------------------------------------
// The reference divides by 12 (order 4) and by 5040 (order 8, once per
// axis); here those are multiplications by the rounded reciprocal -- a
// 1-ulp difference, where an FP64 division costs the GB300 FP64 pipe about as
// much as the rest of the stencil.
// Equal spacing, orders 2 and 4: the axes share one scale (B.lscale), so the
// neighbour sums are added first and the centre enters once (fewer FP64
// instructions; the value differs from the per-axis form by rounding only).
// This is the sum before that scale.
template <int ORD>
__device__ __forceinline__ double lap_sum_iso(const double *__restrict__ u, long long p, long long sy, long long sz)
{
  const double c = u[p];
  if (ORD == 2) return (u[p + 1] + u[p - 1]) + (u[p + sy] + u[p - sy]) + (u[p + sz] + u[p - sz]) - 6.0 * c;
  const double s1 = (u[p + 1] + u[p - 1]) + (u[p + sy] + u[p - sy]) + (u[p + sz] + u[p - sz]);
  const double s2 = (u[p + 2] + u[p - 2]) + (u[p + 2 * sy] + u[p - 2 * sy]) + (u[p + 2 * sz] + u[p - 2 * sz]);
  return 16.0 * s1 - s2 - 90.0 * c;
}

template <int ORD>
__device__ __forceinline__ double lap(const double *__restrict__ u, long long p, long long sy,
                                      long long sz, const DevBox &B)
{
  const double c = u[p];
  const double ix2 = B.idx2[0], iy2 = B.idx2[1], iz2 = B.idx2[2];
  if (ORD <= 4 && B.iso) return lap_sum_iso<ORD>(u, p, sy, sz) * B.lscale;
  if (ORD == 2) {
    return (u[p + 1] - 2.0 * c + u[p - 1]) * ix2 + (u[p + sy] - 2.0 * c + u[p - sy]) * iy2 +
           (u[p + sz] - 2.0 * c + u[p - sz]) * iz2;
  } else if (ORD == 4) {
    return ((-(u[p + 2] + u[p - 2]) + 16.0 * (u[p + 1] + u[p - 1]) - 30.0 * c) * ix2 +
            (-(u[p + 2 * sy] + u[p - 2 * sy]) + 16.0 * (u[p + sy] + u[p - sy]) - 30.0 * c) * iy2 +
            (-(u[p + 2 * sz] + u[p - 2 * sz]) + 16.0 * (u[p + sz] + u[p - sz]) - 30.0 * c) * iz2) *
           (1.0 / 12.0);
  } else if (ORD == 6) {
    const double i180 = 1.0 / 180;
    return (2.0 * (u[p + 3] + u[p - 3]) - 27.0 * (u[p + 2] + u[p - 2] - 10.0 * (u[p + 1] + u[p - 1])) -
            490.0 * c) * ix2 * i180 +
           (2.0 * (u[p + 3 * sy] + u[p - 3 * sy]) -
            27.0 * (u[p + 2 * sy] + u[p - 2 * sy] - 10.0 * (u[p + sy] + u[p - sy])) - 490.0 * c) * iy2 * i180 +
           (2.0 * (u[p + 3 * sz] + u[p - 3 * sz]) -
            27.0 * (u[p + 2 * sz] + u[p - 2 * sz] - 10.0 * (u[p + sz] + u[p - sz])) - 490.0 * c) * iz2 * i180;
  } else {
    return ((-9.0 * (u[p + 4] + u[p - 4]) + 128.0 * (u[p + 3] + u[p - 3]) - 1008.0 * (u[p + 2] + u[p - 2]) +
             8064.0 * (u[p + 1] + u[p - 1]) - 14350.0 * c) * ix2 +
            (-9.0 * (u[p + 4 * sy] + u[p - 4 * sy]) + 128.0 * (u[p + 3 * sy] + u[p - 3 * sy]) -
             1008.0 * (u[p + 2 * sy] + u[p - 2 * sy]) + 8064.0 * (u[p + sy] + u[p - sy]) - 14350.0 * c) * iy2 +
            (-9.0 * (u[p + 4 * sz] + u[p - 4 * sz]) + 128.0 * (u[p + 3 * sz] + u[p - 3 * sz]) -
             1008.0 * (u[p + 2 * sz] + u[p - 2 * sz]) + 8064.0 * (u[p + sz] + u[p - sz]) - 14350.0 * c) * iz2) *
           (1.0 / 5040.0);
  }
}

// Lap u + a, with the scale of the equal-spacing forms and the addition in
// one multiply-add.
template <int ORD>
__device__ __forceinline__ double lap_acc(const double *__restrict__ u, long long p, long long sy, long long sz,
                                          const DevBox &B, double a)
{
  if (ORD <= 4 && B.iso) return fma(lap_sum_iso<ORD>(u, p, sy, sz), B.lscale, a);
  return lap<ORD>(u, p, sy, sz, B) + a;
}

// NaN test on the bits (integer pipe).
__device__ __forceinline__ bool is_nan_bits(double x)
{
  return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

// Hardware approximate FP32 reciprocal (PTX rcp.approx.ftz.f32, error within
// about one ulp).
__device__ __forceinline__ float rcp_fast(float x)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Approximate FP64 reciprocal (PTX rcp.approx.ftz.f64: about 20 correct
// bits, one special-function instruction, no FP32 round trip).
__device__ __forceinline__ double rcp_approx64(double x)
{
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}

// 1/q in FP64: the approximate reciprocal r (relative error e = 1 - q r of
// about 1e-6) refined by one third-order step, 1/q = r / (1 - e) =
// r (1 + e + e^2 + ...) ~ r + r (e + e^2), whose truncation e^3 (about 1e-18)
// is below the FP64 rounding level.  Three FP64 multiply-adds instead of a
// correctly rounded reciprocal; the result is within about an ulp of it.
__device__ __forceinline__ double rcp_newton(double q)
{
  const double r = rcp_approx64(q);
  const double e = fma(-q, r, 1.0);
  return fma(r, fma(e, e, e), r);
}

// Pointwise operator value and its derivative in u (puncture, optionally with
// the scalar-field terms d (c+u) + e (c+u)^5).  Integer powers by products of
// one reciprocal (rcp_newton).
template <int EQ>
__device__ __forceinline__ void point_op(double lapv, double dl, double uu, double bb, double cc,
                                         double dd, double ee, double &op, double &dop)
{
  const double q = cc + uu;
  const double iq = rcp_newton(q);
  const double iq2 = iq * iq;
  const double iq4 = iq2 * iq2;
  const double t7 = bb * (iq4 * iq2 * iq);   // b / (c+u)^7
  op = lapv + t7;
  dop = dl - 7.0 * t7 * iq;                  // -7 b / (c+u)^8
  if (EQ == 2) {   // the test equations: poisson_OP / _duOP, include/elliptic.h:359-366, with b (1, or 0
                   // for Bowen-York's Laplacians, 772-803) the factor of u^2
    const double bu = bb * uu;
    op = lapv + bu * uu;
    dop = dl + 2.0 * bu;
    return;
  }
  if (EQ == 1) {
    const double q2 = q * q;
    const double q4 = q2 * q2;
    op = op + dd * q + ee * (q4 * q);
    dop = dop + dd + 5.0 * ee * q4;
  }
}

// The pointwise part of the operator, nl = OP - Lap u, and duOP, for the
// smoothers, which add nl - rho to the Laplacian in one multiply-add
// (lap_acc).  The same terms as point_op.
template <int EQ>
__device__ __forceinline__ void point_terms(double dl, double uu, double bb, double cc, double dd, double ee,
                                            double &nl, double &dop)
{
  if (EQ == 2) {
    const double bu = bb * uu;
    nl = bu * uu;
    dop = dl + 2.0 * bu;
    return;
  }
  const double q = cc + uu;
  const double iq = rcp_newton(q);
  const double iq2 = iq * iq;
  const double iq4 = iq2 * iq2;
  const double t7 = bb * (iq4 * iq2 * iq);   // b / (c+u)^7
  nl = t7;
  dop = dl - 7.0 * t7 * iq;                  // -7 b / (c+u)^8
  if (EQ == 1) {
    const double q2 = q * q;
    const double q4 = q2 * q2;
    nl = nl + dd * q + ee * (q4 * q);
    dop = dop + dd + 5.0 * ee * q4;
  }
}

// One-sided first derivative for the Robin condition: dx2 for order 2
// (one-sided 2nd order at the ends, centred inside), dx4 for orders 4/6/8
// (5-point one-sided pointing inward).
template <int ORD>
__device__ __forceinline__ double deriv(const double *__restrict__ u, long long p, long long s, int i,
                                        int n, double id, double &du)
{
  if (ORD == 2) {
    if (i == 0) {
      du = -3.0 * 0.5 * id;
      return (-3.0 * u[p] + 4.0 * u[p + s] - u[p + 2 * s]) * 0.5 * id;
    }
    if (i == n - 1) {
      du = 3.0 * 0.5 * id;
      return (3.0 * u[p] - 4.0 * u[p - s] + u[p - 2 * s]) * 0.5 * id;
    }
    du = 0.0;
    return (u[p + s] - u[p - s]) * 0.5 * id;
  } else {
    const int nm = n % 2 == 0 ? n / 2 : (n - 1) / 2;
    if (i <= nm) {
      du = -25 * id / 12.0;
      return (-(25 * u[p] - 48 * u[p + s] + 36 * u[p + 2 * s] - 16 * u[p + 3 * s] + 3 * u[p + 4 * s]) * id / 12.0);
    }
    du = 25 * id / 12.0;
    return ((25 * u[p] - 48 * u[p - s] + 36 * u[p - 2 * s] - 16 * u[p - 3 * s] + 3 * u[p - 4 * s]) * id / 12.0);
  }
}

// Robin term r^2/n * sum_a (du/dx_a)/x_a for the axes in mask (n = B.falloff), grouped
// like Boundary_Face (one axis) and Boundary_Edge/Corner (two/three axes).
// A box's coordinate table holds x, y, z and then 1/x, 1/y, 1/z: the
// divisions by the coordinate are products with its reciprocal (within an
// ulp of the quotient; an FP64 division costs GB300 about ten FP64
// instructions).
template <int ORD>
__device__ __forceinline__ double robin_term(const double *__restrict__ u, const DevBox &B,
                                             const double *__restrict__ crd, int mask, int i, int j,
                                             int k, double &dF)
{
  const double *c = crd + B.coord_off, *ic = c + (B.n[0] + B.n[1] + B.n[2]);
  const double x = c[i], y = c[B.n[0] + j], z = c[B.n[0] + B.n[1] + k];
  // r^2 / n (the falloff; the halving is exact, so the grouping of r2 * ipn * D
  // in src/boundary.cc:947-950 gives the same bits)
  const double r2 = B.falloff == 2 ? 0.5 * (x * x + y * y + z * z) : x * x + y * y + z * z;
  const long long p = pidx(B, i, j, k);
  const long long st[3] = {1, (long long)B.n[0], (long long)B.n[0] * B.n[1]};
  const int ijk[3] = {i, j, k};
  const double ixyz[3] = {ic[i], ic[B.n[0] + j], ic[B.n[0] + B.n[1] + k]};
  double t = 0.0, dt = 0.0;
  int na = 0;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!(mask & (1 << a))) continue;
    double du;
    const double dv = deriv<ORD>(u, p, st[a], ijk[a], B.n[a], B.idx[a], du);
    if (na == 0 && mask == (1 << a)) {          // face
      dF = r2 * du * ixyz[a] + 1.0;
      return r2 * dv * ixyz[a];
    }
    t = na == 0 ? dv * ixyz[a] : t + dv * ixyz[a];
    dt = na == 0 ? du * ixyz[a] : dt + du * ixyz[a];
    na++;
  }
  dF = r2 * dt + 1.0;
  return r2 * t;
}

// mode 0: Newton update u -= F/dF with F = term + u - S   (App_Bound)
// mode 1: R = term + u                                     (App_Boundary_Operator)
template <int ORD>
__device__ __forceinline__ void robin_point(const DevBox &B, const DevFields &F,
                                            const double *__restrict__ crd, int mode, int mask, int i,
                                            int j, int k)
{
  double *u = F.f[F_U] + B.off;
  const long long p = pidx(B, i, j, k);
  if (mode >= 2) {   // Dirichlet (src/boundary.cc:800-812, 1481-1490): u = S, and R = u
    if (mode == 2) u[p] = F.f[F_RHO][B.off + p];
    else F.f[F_R][B.off + p] = u[p];
    return;
  }
  double dF;
  const double t = robin_term<ORD>(u, B, crd, mask, i, j, k, dF);
  if (mode == 0) {   // the step's divisor only sizes the step: F = 0 stays the solution
    const double Fv = t + u[p] - F.f[F_RHO][B.off + p];
    u[p] = u[p] - Fv * rcp_approx64(dF);
  } else {
    F.f[F_R][B.off + p] = t + u[p];
  }
}

// ----------------------------------------------------------------------------
// programmatic dependent launch: a kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may be scheduled while
// its predecessor in the stream is still running; it must not read anything
// the predecessor writes before griddep_wait() returns (then all of the
// predecessor's memory operations are complete and visible).
// griddep_launch_dependents() lets the next such kernel be scheduled early.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents()
{
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ----------------------------------------------------------------------------
// reductions
// ----------------------------------------------------------------------------
// v >= 0: a non-negative double orders like its bit pattern read as an
// unsigned integer, so the block maximum is taken on the bits with integer
// instructions and the FP64 pipe (the smoothers' bottleneck on GB300) stays
// free.  A NaN compares above every finite value and reaches the slot.
__device__ __forceinline__ void block_max_atomic_bits(unsigned long long m, unsigned long long *slot)
{
  __shared__ unsigned long long red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = m;
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    m = lane < nw ? red[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
      m = x > m ? x : m;
    }
    if (lane == 0 && m > 0ull) atomicMax(slot, m);
  }
}

__device__ __forceinline__ void block_max_atomic(double v, unsigned long long *slot)
{
  block_max_atomic_bits((unsigned long long)__double_as_longlong(v), slot);
}


// Largest change of u over one cycle, max |u - up| over the points the
// discrete system fixes (pinned[p] != 0: every point of the solution levels,
// the INSIDE points of the multigrid coarse levels), into *slot as a bit
// pattern.  A NaN difference wins the maximum.  n = the solve's points (its
// part of the arena); gate = one of its boxes.
__global__ void __launch_bounds__(256) k_du_max(long long n, const double *__restrict__ u,
                                                const double *__restrict__ up,
                                                const unsigned char *__restrict__ pinned,
                                                unsigned long long *slot, const DevBox *__restrict__ gate)
{
  if (!gate->active) return;   // the solve has stopped (batch); the whole grid leaves
  double m = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride)
    if (pinned[p]) {
      const double d = fabs(u[p] - up[p]);
      if (d > m || is_nan_bits(d)) m = d;
      if (is_nan_bits(m)) break;
    }
  block_max_atomic(m, slot);
}

// FMA issue-rate probe (olgpu_fma_peak): kFmaChains independent chains per
// thread, x <- x * a + c, which stays near c / (1 - a) = 1 (no overflow, no
// subnormals).  The result is stored only if it is impossible (x > 1e30), so
// the loop is kept and nothing is written.
constexpr int kFmaChains = 8;

template <class T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T *sink)
{
  T x[kFmaChains];
#pragma unroll
  for (int c = 0; c < kFmaChains; c++) x[c] = T(threadIdx.x + c) * T(1e-3);
  const T a = T(0.999), k = T(1e-3);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kFmaChains; c++) x[c] = fma(x[c], a, k);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kFmaChains; c++) s += x[c];
  if (s > T(1e30)) *sink = s;
}

// Inverse of the Newton diagonal dOP/du for the smoother's step.  The step
// u -= R / dOP only needs the diagonal approximately: a relative error of
// about 1e-6 in it scales the step by 1 +- 1e-6 and leaves the fixed point
// (R = 0) where it is, so one approximate reciprocal replaces an FP64
// division (the FP64 pipe is the bottleneck of this kernel on GB300).
__device__ __forceinline__ double step_inverse(double dop)
{
  return rcp_approx64(dop);
}

// ----------------------------------------------------------------------------
// K1: multicolour nonlinear Gauss-Seidel-Newton pass.  Colour of a point is
// (i + j + k) mod NC with NC = ORD/2 + 1, so that no two points of a colour
// are within the stencil reach of each other: a colour pass is a true
// Gauss-Seidel pass in any thread order (red-black for order 2).
// ----------------------------------------------------------------------------
template <int ORD>
__host__ __device__ constexpr int num_colors() { return ORD / 2 + 1; }

// The pass's residual maximum goes to stats[B.solve].slots[2 * B.level +
// post] (the level's pre- or post-smoothing norm), a NaN to its nan_flag.
// PTS points of a row per thread (its colour's points ih*PTS .. ih*PTS+PTS-1):
// every point's loads and arithmetic before any store -- points of one
// colour do not read each other -- so the latencies of the points overlap;
// each point's update is the same expression, so any PTS gives the same bits.
template <int ORD, int EQ, int PTS = 1>
__global__ void __launch_bounds__(256) k_smooth_color(BoxList L, const DevBox *__restrict__ boxes,
                                                      DevFields F, int color, Stats *stats, int post)
{
  constexpr int NC = num_colors<ORD>();
  griddep_wait();                 // launched as a programmatic dependent
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;          // the whole block leaves (one box a block)
  unsigned long long *norm_slot = &stats[B.solve].slots[2 * B.level + post];
  int *nan_flag = &stats[B.solve].nan_flag;
  const int b = B.buf;
  const int m0 = B.n[0] - 2 * b, m1 = B.n[1] - 2 * b, m2 = B.n[2] - 2 * b;
  const int H = (m0 + NC - 1) / NC;
  const int HP = (H + PTS - 1) / PTS;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long total = (long long)HP * m1 * m2;
  unsigned long long rabs = 0ull;   // max |R| as its bit pattern (integer compares)
  if (t < total) {
    const int ihp = ((int)t % HP);
    const int r = (int)t / HP;
    const int j = b + (r % m1);
    const int k = b + (r / m1);
    const int delta = (((color - b - j - k) % NC) + NC) % NC;
    double *u = F.f[F_U] + B.off;
    const long long sy = B.n[0], sz = (long long)B.n[0] * B.n[1];
    double un[PTS];
    long long pp[PTS];
    bool ok[PTS];
#pragma unroll
    for (int q = 0; q < PTS; q++) {
      const int i = b + delta + NC * (ihp * PTS + q);
      ok[q] = i < B.n[0] - b;
      pp[q] = pidx(B, ok[q] ? i : b + delta, j, k);   // a point past the row's end repeats its first point
      const long long p = pp[q];
      const double up = u[p];
      double nl, dop;
      point_terms<EQ>(B.dulap, up, F.f[F_B][B.off + p], F.f[F_C][B.off + p],
                      EQ == 1 ? F.f[F_D][B.off + p] : 0.0, EQ == 1 ? F.f[F_E][B.off + p] : 0.0, nl, dop);
      const double R = lap_acc<ORD>(u, p, sy, sz, B, nl - F.f[F_RHO][B.off + p]);
      un[q] = up - R * step_inverse(dop);
      // |R| on the bits: non-negative doubles order as their patterns, and a
      // NaN's pattern is above infinity's, so a NaN stays the maximum
      const unsigned long long a = (unsigned long long)__double_as_longlong(R) & 0x7fffffffffffffffull;
      if (ok[q] && a > rabs) rabs = a;
    }
#pragma unroll
    for (int q = 0; q < PTS; q++)
      if (ok[q]) {
        u[pp[q]] = un[q];
        if (is_nan_bits(un[q])) atomicOr(nan_flag, 1);
      }
  }
  block_max_atomic_bits(rabs, norm_slot);
}

// R = OP(u) on the INSIDE points (App_Ell_Operator).
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_apply_op(BoxList L, const DevBox *__restrict__ boxes, DevFields F)
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
  const double *u = F.f[F_U] + B.off;
  const long long p = pidx(B, i, j, k);
  const double lv = lap<ORD>(u, p, B.n[0], (long long)B.n[0] * B.n[1], B);
  double op, dop;
  point_op<EQ>(lv, B.dulap, u[p], F.f[F_B][B.off + p], F.f[F_C][B.off + p],
               EQ == 1 ? F.f[F_D][B.off + p] : 0.0, EQ == 1 ? F.f[F_E][B.off + p] : 0.0, op, dop);
  F.f[F_R][B.off + p] = op;
}

// ----------------------------------------------------------------------------
// Robin boundary: faces (one thread per normal column, layers inner -> outer)
// ----------------------------------------------------------------------------
template <int ORD>
__global__ void __launch_bounds__(256) k_robin_faces(BoxList L, const DevBox *__restrict__ boxes,
                                                     DevFields F, const double *__restrict__ crd, int mode)
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
        robin_point<ORD>(B, F, crd, mode, 1 << a, ijk[0], ijk[1], ijk[2]);
      }
      return;
    }
    t -= cols;
  }
}

// Robin points on the ghost edges (part 0) or corners (part 1; launched
// after the edges, whose values the corners read).
template <int ORD>
__global__ void __launch_bounds__(64) k_robin_edges_corners(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
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
          robin_point<ORD>(B, F, crd, mode, (1 << a) | (1 << c), ijk[0], ijk[1], ijk[2]);
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
          robin_point<ORD>(B, F, crd, mode, 7, i, j, k);
        }
  }
}

// ----------------------------------------------------------------------------
// Robin boundary in fewer launches.  The Newton update (mode 0) must see the
// faces done before the edges and the edges before the corners (the
// reference's order: faces, edges, corners; src/boundary.cc:447-907): the
// faces keep their launch over the whole GPU (k_robin_faces), and the edges
// and corners of a box follow in one launch of a thread-block cluster per box
// whose barrier separates them (k_robin_ec_cluster).  The operator value
// (mode 1, src/boundary.cc:1118-1535) only reads u, so every ghost point of
// a level -- faces, edges and corners -- is one flat launch (k_robin_all).
// The point updates and their dependency order are those of the separate
// face, edge and corner launches above, so the results are the same bits.
// pt(mask, i, j, k) updates one ghost point.
// ----------------------------------------------------------------------------
constexpr int kRobinCluster = 8;

// Ghost points of a box's 12 edges, counted along the edges (each item: the
// edge's b x b points at one position).
__host__ __device__ __forceinline__ long long robin_edge_items(const DevBox &B)
{
  long long n = 0;
  for (int e12 = 0; e12 < 12; e12++) {
    const int pi = e12 >> 2, a = pi == 2 ? 1 : 0, c = pi == 0 ? 1 : 2;
    n += B.n[3 - a - c] - 2 * B.buf;
  }
  return n;
}

// Normal columns of a box's six faces (each item: the column's b points).
__host__ __device__ __forceinline__ long long robin_face_items(const DevBox &B)
{
  const int b = B.buf;
  long long cols = 0;
  for (int a = 0; a < 3; a++) cols += 2LL * (B.n[(a + 1) % 3] - 2 * b) * (B.n[(a + 2) % 3] - 2 * b);
  return cols;
}

template <class PointFn>
__device__ __forceinline__ void robin_face_item(const DevBox &B, long long t, PointFn pt)
{
  const int b = B.buf;
  for (int f = 0; f < 6; f++) {
    const int a = f >> 1, hi = f & 1;
    const int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
    const int m1 = B.n[a1] - 2 * b, m2 = B.n[a2] - 2 * b;
    const long long cols = (long long)m1 * m2;
    if (t < cols) {
      int ijk[3];
      ijk[a1] = b + (int)(t % m1);
      ijk[a2] = b + (int)(t / m1);
      for (int l = 0; l < b; l++) {
        ijk[a] = hi ? B.n[a] - b + l : b - 1 - l;
        pt(1 << a, ijk[0], ijk[1], ijk[2]);
      }
      return;
    }
    t -= cols;
  }
}

template <class PointFn>
__device__ __forceinline__ void robin_edge_item(const DevBox &B, long long t, PointFn pt)
{
  const int b = B.buf;
  for (int e12 = 0; e12 < 12; e12++) {
    const int pi = e12 >> 2, e = e12 & 3;
    const int a = pi == 2 ? 1 : 0, c = pi == 0 ? 1 : 2, fa = 3 - a - c;
    const int m = B.n[fa] - 2 * b;
    if (t < m) {
      const int ha = e >> 1, hc = e & 1;
      int ijk[3];
      ijk[fa] = b + (int)t;
      for (int ta = 0; ta < b; ta++)
        for (int tc = 0; tc < b; tc++) {
          ijk[a] = ha ? B.n[a] - b + ta : b - 1 - ta;
          ijk[c] = hc ? B.n[c] - b + tc : b - 1 - tc;
          pt((1 << a) | (1 << c), ijk[0], ijk[1], ijk[2]);
        }
      return;
    }
    t -= m;
  }
}

template <class PointFn>
__device__ __forceinline__ void robin_corner_item(const DevBox &B, int corner, PointFn pt)
{
  const int b = B.buf;
  const int hx = corner & 1, hy = (corner >> 1) & 1, hz = corner >> 2;
  for (int tk = 0; tk < b; tk++)
    for (int tj = 0; tj < b; tj++)
      for (int ti = 0; ti < b; ti++)
        pt(7, hx ? B.n[0] - b + ti : b - 1 - ti, hy ? B.n[1] - b + tj : b - 1 - tj, hz ? B.n[2] - b + tk : b - 1 - tk);
}

// Edges, then (cluster barrier) corners of one box by a cluster of ncta blocks.
template <class PointFn>
__device__ __forceinline__ void robin_ec_walk(const DevBox &B, unsigned rank, unsigned ncta, PointFn pt)
{
  namespace cg = cooperative_groups;
  const long long tid = (long long)rank * blockDim.x + threadIdx.x, nth = (long long)ncta * blockDim.x;
  const long long ne = robin_edge_items(B);
  for (long long t = tid; t < ne; t += nth) robin_edge_item(B, t, pt);
  cg::this_cluster().sync();   // every edge is done (global writes visible in the cluster)
  if (tid < 8) robin_corner_item(B, (int)tid, pt);
}

template <int ORD>
__global__ void __launch_bounds__(256) k_robin_ec_cluster(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                          const double *__restrict__ crd, int mode)
{
  namespace cg = cooperative_groups;
  const unsigned ncta = cg::this_cluster().num_blocks();
  if ((int)(blockIdx.x / ncta) >= L.count) return;   // the whole cluster: one box a cluster
  const DevBox B = boxes[L.box[blockIdx.x / ncta]];
  if (!B.active) return;   // every block of the cluster reads the same box: all leave
  robin_ec_walk(B, cg::this_cluster().block_rank(), ncta,
                [&](int mask, int i, int j, int k) { robin_point<ORD>(B, F, crd, mode, mask, i, j, k); });
}

// Every ghost point of the boxes of L in one launch, for the modes that only
// read u (1: the Robin operator, 3: the Dirichlet one).
template <int ORD>
__global__ void __launch_bounds__(256) k_robin_all(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                   const double *__restrict__ crd, int mode)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  long long t = lb * blockDim.x + threadIdx.x;
  auto pt = [&](int mask, int i, int j, int k) { robin_point<ORD>(B, F, crd, mode, mask, i, j, k); };
  const long long nf = robin_face_items(B), ne = robin_edge_items(B);
  if (t < nf) robin_face_item(B, t, pt);
  else if ((t -= nf) < ne) robin_edge_item(B, t, pt);
  else if ((t -= ne) < 8) robin_corner_item(B, (int)t, pt);
}

// ----------------------------------------------------------------------------
// element-wise field updates over ALL points of a level
// ----------------------------------------------------------------------------
enum EwOp { EW_W_EQ_S_MINUS_R = 0, EW_S_EQ_W_PLUS_R, EW_W_PLUS_EQ_R, EW_WW_EQ_U, EW_V_EQ_U_MINUS_WW,
            EW_U_PLUS_EQ_V };

__global__ void __launch_bounds__(256) k_elementwise(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
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
  case EW_W_EQ_S_MINUS_R: F.f[F_W][p] = F.f[F_RHO][p] - F.f[F_R][p]; break;
  case EW_S_EQ_W_PLUS_R: F.f[F_RHO][p] = F.f[F_W][p] + F.f[F_R][p]; break;
  case EW_W_PLUS_EQ_R: F.f[F_W][p] = F.f[F_W][p] + F.f[F_R][p]; break;
  case EW_WW_EQ_U: F.f[F_WW][p] = F.f[F_U][p]; break;
  case EW_V_EQ_U_MINUS_WW: F.f[F_V][p] = F.f[F_U][p] - F.f[F_WW][p]; break;
  case EW_U_PLUS_EQ_V: F.f[F_U][p] = F.f[F_U][p] + F.f[F_V][p]; break;
  }
}

// ----------------------------------------------------------------------------
// T = W averaged with (1,2,1)^3/64 weights on INSIDE points (a neighbour
// outside INSIDE contributes the centre value), T = W elsewhere.  The tau
// defect W is then moved to the coarse level from T: with a multicolour
// smoother the defect alternates in sign between colours, and the reference's
// injection would hand the coarse level a single colour.  W vanishes at the
// fixed point, so the averaging changes the path, not the solution.
// ----------------------------------------------------------------------------
// The (1,2,1)^3/64 average of w around (i, j, k), a neighbour outside the
// INSIDE range taking the centre value c: summed separably, rows along x
// first ((v[-1] + 2 v[0]) + v[+1]), then those rows along y, then the
// planes along z, and scaled by 1/64 once.  The factors are powers of two,
// so only the additions round; every kernel that forms the weighting uses
// this one order, so the fused and the plain steps agree bit for bit.  The
// INSIDE test of a neighbour is the product of three per-axis tests.
template <class V, class W>
__device__ __forceinline__ V fw_sum(const W &w, V c, const DevBox &B, int i, int j, int k, long long p)
{
  const int b = B.buf;
  const long long sy = B.n[0], sz = (long long)B.n[0] * B.n[1];
  const bool xin[3] = {i - 1 >= b, true, i + 1 < B.n[0] - b};
  const bool yin[3] = {j - 1 >= b, true, j + 1 < B.n[1] - b};
  const bool zin[3] = {k - 1 >= b, true, k + 1 < B.n[2] - b};
  V plane[3];
#pragma unroll
  for (int dk = 0; dk < 3; dk++) {
    V row[3];
#pragma unroll
    for (int dj = 0; dj < 3; dj++) {
      const long long q = p + (long long)(dk - 1) * sz + (long long)(dj - 1) * sy;
      const bool yz = yin[dj] && zin[dk];
      const V vm = (yz && xin[0]) ? w(q - 1) : c;
      const V v0 = yz ? w(q) : c;
      const V vp = (yz && xin[2]) ? w(q + 1) : c;
      row[dj] = (vm + V(2) * v0) + vp;
    }
    plane[dk] = (row[0] + V(2) * row[1]) + row[2];
  }
  return ((plane[0] + V(2) * plane[1]) + plane[2]) * (V(1) / V(64));
}

__global__ void __launch_bounds__(256) k_full_weight(BoxList L, const DevBox *__restrict__ boxes, DevFields F)
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
  const double *w = F.f[F_W] + B.off;
  const double c = w[t];
  const bool inside = i >= b && i < B.n[0] - b && j >= b && j < B.n[1] - b && k >= b && k < B.n[2] - b;
  if (!inside) {
    F.f[F_T][B.off + t] = c;
    return;
  }
  F.f[F_T][B.off + t] = fw_sum<double>([&](long long q) { return w[q]; }, c, B, i, j, k, t);
}

// ----------------------------------------------------------------------------
// generic inter-box transfer (restriction, tau transfer, prolongation, ghost
// fill, tau mask) driven by host-built per-axis interpolation tables
// ----------------------------------------------------------------------------
// Tensor Lagrange sum over the window at `base`: z innermost, then y, then x
// (the reference's order); the terms of an axis outside its [lo, hi] (all but
// one where the weights are exactly one-hot) are skipped, which leaves the sum
// unchanged bit for bit.  P points per axis are unrolled at compile time, so
// the window's loads are independent and issue together instead of one per
// accumulation step.
template <class T, int P>
__device__ __forceinline__ T tensor_sum(const T *__restrict__ base, long long sy, long long sz, const AxisEntry &ax,
                                        const AxisEntry &ay, const AxisEntry &az)
{
  T wz[P];
#pragma unroll
  for (int K = 0; K < P; K++) wz[K] = (T)az.w[K];
  T fx = T(0);
#pragma unroll
  for (int I = 0; I < P; I++) {
    if (I < ax.lo || I > ax.hi) continue;
    T uy = T(0);
#pragma unroll
    for (int Jj = 0; Jj < P; Jj++) {
      if (Jj < ay.lo || Jj > ay.hi) continue;
      const T *col = base + I + Jj * sy;
      T uz = T(0);
#pragma unroll
      for (int K = 0; K < P; K++)
        if (K >= az.lo && K <= az.hi) uz += col[K * sz] * wz[K];
      uy += uz * (T)ay.w[Jj];
    }
    fx += uy * (T)ax.w[I];
  }
  return fx;
}

// The same sum for any window width (at most kMaxInterpPoints).
template <class T>
__device__ __forceinline__ T tensor_sum_any(const T *__restrict__ base, long long sy, long long sz,
                                            const AxisEntry &ax, const AxisEntry &ay, const AxisEntry &az)
{
  T fx = T(0);
  for (int I = ax.lo; I <= ax.hi; I++) {
    T uy = T(0);
    for (int Jj = ay.lo; Jj <= ay.hi; Jj++) {
      const T *col = base + I + Jj * sy;
      T uz = T(0);
      for (int K = az.lo; K <= az.hi; K++) uz += col[K * sz] * (T)az.w[K];
      uy += uz * (T)ay.w[Jj];
    }
    fx += uy * (T)ax.w[I];
  }
  return fx;
}

// One launch runs every job of a transfer plan; V is the field type (double
// for the FP64 fields, float for the FP32 correction fields).  P is the
// plan's Lagrange window width (0: the plan has copy / linear jobs only, -1:
// a width without its own instantiation), so each width is a kernel of its
// own with its own register budget.
template <class V, class Fields, int P>
__global__ void __launch_bounds__(256) k_xfer(const XferJob *__restrict__ jobs, int njobs,
                                              const DevBox *__restrict__ boxes, Fields F,
                                              const AxisEntry *__restrict__ tab)
{
  int jb = 0;
  {
    int lo = 0, hi = njobs - 1;   // last job with blk0 <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].blk0 <= (long long)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    jb = lo;
  }
  const XferJob &J = jobs[jb];
  if (!boxes[J.tbox].active) return;   // the target's solve has stopped (whole block: one job)
  const long long t = ((long long)blockIdx.x - J.blk0) * blockDim.x + threadIdx.x;
  const int e0 = J.r1[0] - J.r0[0], e1 = J.r1[1] - J.r0[1], e2 = J.r1[2] - J.r0[2];
  if (t >= (long long)e0 * e1 * e2) return;
  const int i = J.r0[0] + ((int)t % e0);
  const int r = (int)t / e0;
  const int j = J.r0[1] + (r % e1);
  const int k = J.r0[2] + (r / e1);
  const DevBox T = boxes[J.tbox];
  if (J.iter != IT_ALL) {
    const int b = T.buf;
    const bool inside = i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b;
    if ((J.iter == IT_INSIDE) != inside) return;
  }
  V *dst = F.f[J.tfield] + T.off;
  const long long tp = pidx(T, i, j, k);
  if (J.method == XM_STRIDED) {   // every target coincides with a node: no table lookups
    const DevBox &S = boxes[J.sbox];
    dst[tp] = F.f[J.sfield][S.off + pidx(S, J.sstart[0] + J.sstep[0] * (i - J.r0[0]),
                                          J.sstart[1] + J.sstep[1] * (j - J.r0[1]),
                                          J.sstart[2] + J.sstep[2] * (k - J.r0[2]))];
    return;
  }
  const AxisEntry &ax = tab[J.tab[0] + i];
  const AxisEntry &ay = tab[J.tab[1] + j];
  const AxisEntry &az = tab[J.tab[2] + k];
  if (!(ax.sel && ay.sel && az.sel)) {
    if (J.to_zero) dst[tp] = V(0);
    return;
  }
  const DevBox S = boxes[J.sbox];
  const V *src = F.f[J.sfield] + S.off;
  if (J.method == XM_COPY || (ax.exact && ay.exact && az.exact)) {
    dst[tp] = src[pidx(S, ax.node, ay.node, az.node)];
    return;
  }
  if (J.method == XM_LINEAR || P == 0) {
    // ((v000 dxi + v100 dxf) dyi + (v010 dxi + v110 dxf) dyf) dzi + (...) dzf
    const int i0 = ax.start, j0 = ay.start, k0 = az.start;
    const V dxi = (V)ax.w[0], dxf = (V)ax.w[1], dyi = (V)ay.w[0], dyf = (V)ay.w[1], dzi = (V)az.w[0],
            dzf = (V)az.w[1];
    const V v000 = src[pidx(S, i0, j0, k0)], v100 = src[pidx(S, i0 + 1, j0, k0)];
    const V v010 = src[pidx(S, i0, j0 + 1, k0)], v110 = src[pidx(S, i0 + 1, j0 + 1, k0)];
    const V v001 = src[pidx(S, i0, j0, k0 + 1)], v101 = src[pidx(S, i0 + 1, j0, k0 + 1)];
    const V v011 = src[pidx(S, i0, j0 + 1, k0 + 1)], v111 = src[pidx(S, i0 + 1, j0 + 1, k0 + 1)];
    dst[tp] = ((v000 * dxi + v100 * dxf) * dyi + (v010 * dxi + v110 * dxf) * dyf) * dzi +
              ((v001 * dxi + v101 * dxf) * dyi + (v011 * dxi + v111 * dxf) * dyf) * dzf;
    return;
  }
  const V *base = src + pidx(S, ax.start, ay.start, az.start);
  const long long sy = S.n[0], sz = (long long)S.n[0] * S.n[1];
  if (P > 0) dst[tp] = tensor_sum<V, (P > 0 ? P : 1)>(base, sy, sz, ax, ay, az);
  else dst[tp] = tensor_sum_any<V>(base, sy, sz, ax, ay, az);
}

// ----------------------------------------------------------------------------
// Separable form of the tensor Lagrange transfer, one warp per target row.
// Along a row in x (fixed j, k) every target shares ay and az, so the inner
// sums of the tensor sum, uy(I') = sum_J wy_J sum_K wz_K src(I', J, K), are
// the same for every target that reaches source column I'; the warp forms
// them once per column in shared memory and each target then adds its x
// terms, fx = sum_I wx_I uy(start_x + I).  Along a row in y (the two-wide
// x-slabs of a ghost shell) the targets share ax and az: the warp forms
// uz(I, J') = sum_K wz_K src(start_x + I, J', K) and each target adds
// sum_I wx_I sum_J wy_J uz(I, start_y + J).  The terms, their order and
// their rounding are those of tensor_sum, so the result is the same bit for
// bit, with about P/2 instead of P^3 multiply-adds per target.
// ----------------------------------------------------------------------------
// 16 rows per block: the kernel is latency-bound with few rows, so packing
// them onto fewer SMs costs little time and leaves the other SMs to other work
constexpr int kRowWarps = 16;    // rows in flight per block
constexpr int kRowBuf = 320;     // shared partial sums per row (else direct sums)

// The body of k_xfer_rows for block rb of its plan (32 * kRowWarps threads).
template <class V, class Fields, int P>
__device__ __forceinline__ void xfer_rows_body(long long rb, const XferJob *__restrict__ jobs, int njobs,
                                               const DevBox *__restrict__ boxes, Fields F,
                                               const AxisEntry *__restrict__ tab)
{
  __shared__ V sbuf[kRowWarps][kRowBuf];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int lo = 0, hi = njobs - 1;   // last job with rblk0 <= rb
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].rblk0 <= rb) lo = mid;
    else hi = mid - 1;
  }
  const XferJob &J = jobs[lo];
  if (!boxes[J.tbox].active) return;   // the target's solve has stopped (whole block: one job)
  const int e0 = J.r1[0] - J.r0[0], e1 = J.r1[1] - J.r0[1];
  const int ra = J.row_axis;
  const long long row = (rb - J.rblk0) * kRowWarps + warp;
  const int across = ra == 0 ? e1 : e0;   // rows per plane
  if (row >= (long long)across * (J.r1[2] - J.r0[2])) return;   // the whole warp leaves together
  const int k = J.r0[2] + (int)row / across;
  const int fixed = (ra == 0 ? J.r0[1] : J.r0[0]) + (int)row % across;
  const int len = ra == 0 ? e0 : e1, first = ra == 0 ? J.r0[0] : J.r0[1];
  const DevBox T = boxes[J.tbox], S = boxes[J.sbox];
  V *dst = F.f[J.tfield] + T.off;
  const V *src = F.f[J.sfield] + S.off;
  const long long sy = S.n[0], sz = (long long)S.n[0] * S.n[1];
  const AxisEntry &az = tab[J.tab[2] + k];
  const AxisEntry &af = tab[J.tab[ra == 0 ? 1 : 0] + fixed];   // the row's fixed x or y entry
  V *buf = sbuf[warp];

  // pass 0: copies, zeros and the source span of the targets that need a sum
  int smin = 1 << 30, smax = -1;
  for (int t = lane; t < len; t += 32) {
    const int i = ra == 0 ? first + t : fixed, j = ra == 0 ? fixed : first + t;
    if (J.iter != IT_ALL) {
      const int b = T.buf;
      const bool inside = i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b;
      if ((J.iter == IT_INSIDE) != inside) continue;
    }
    const AxisEntry &ax = tab[J.tab[0] + i];
    const AxisEntry &ay = tab[J.tab[1] + j];
    const long long tp = pidx(T, i, j, k);
    if (!(ax.sel && ay.sel && az.sel)) {
      if (J.to_zero) dst[tp] = V(0);
      continue;
    }
    if (J.method == XM_COPY || (ax.exact && ay.exact && az.exact)) {
      dst[tp] = src[pidx(S, ax.node, ay.node, az.node)];
      continue;
    }
    const AxisEntry &ar = ra == 0 ? ax : ay;
    smin = min(smin, ar.start + ar.lo);
    smax = max(smax, ar.start + ar.hi);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    smin = min(smin, __shfl_xor_sync(0xffffffffu, smin, o));
    smax = max(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  }
  if (smax < smin) return;
  const int span = smax - smin + 1;
  const int nI = ra == 0 ? 1 : af.hi - af.lo + 1;
  const bool shared = span * nI <= kRowBuf;

  // pass 1: the shared partial sums
  if (shared) {
    if (ra == 0) {
      for (int c = lane; c < span; c += 32) {
        const V *col0 = src + (long long)(smin + c) + (long long)af.start * sy + (long long)az.start * sz;
        V uy = V(0);
        for (int Jj = af.lo; Jj <= af.hi; Jj++) {
          const V *col = col0 + Jj * sy;
          V uz = V(0);
          for (int K = az.lo; K <= az.hi; K++) uz += col[K * sz] * (V)az.w[K];
          uy += uz * (V)af.w[Jj];
        }
        buf[c] = uy;
      }
    } else {
      for (int q = lane; q < span * nI; q += 32) {
        const int I = af.lo + q / span, c = q % span;
        const V *col = src + (long long)(af.start + I) + (long long)(smin + c) * sy + (long long)az.start * sz;
        V uz = V(0);
        for (int K = az.lo; K <= az.hi; K++) uz += col[K * sz] * (V)az.w[K];
        buf[q] = uz;
      }
    }
  }
  __syncwarp();

  // pass 2: every target's own terms
  for (int t = lane; t < len; t += 32) {
    const int i = ra == 0 ? first + t : fixed, j = ra == 0 ? fixed : first + t;
    if (J.iter != IT_ALL) {
      const int b = T.buf;
      const bool inside = i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b;
      if ((J.iter == IT_INSIDE) != inside) continue;
    }
    const AxisEntry &ax = tab[J.tab[0] + i];
    const AxisEntry &ay = tab[J.tab[1] + j];
    if (!(ax.sel && ay.sel && az.sel) || J.method == XM_COPY || (ax.exact && ay.exact && az.exact)) continue;
    const long long tp = pidx(T, i, j, k);
    if (!shared) {
      dst[tp] = tensor_sum_any<V>(src + pidx(S, ax.start, ay.start, az.start), sy, sz, ax, ay, az);
      continue;
    }
    V fx = V(0);
    if (ra == 0) {
      for (int I = ax.lo; I <= ax.hi; I++) fx += buf[ax.start + I - smin] * (V)ax.w[I];
    } else {
      for (int I = ax.lo; I <= ax.hi; I++) {
        const V *uzI = buf + (I - ax.lo) * span - smin;
        V uy = V(0);
        for (int Jj = ay.lo; Jj <= ay.hi; Jj++) uy += uzI[ay.start + Jj] * (V)ay.w[Jj];
        fx += uy * (V)ax.w[I];
      }
    }
    dst[tp] = fx;
  }
}

template <class V, class Fields, int P>
__global__ void __launch_bounds__(32 * kRowWarps) k_xfer_rows(const XferJob *__restrict__ jobs, int njobs,
                                                              const DevBox *__restrict__ boxes, Fields F,
                                                              const AxisEntry *__restrict__ tab)
{
  xfer_rows_body<V, Fields, P>(blockIdx.x, jobs, njobs, boxes, F, tab);
}

// Window width P of a plan's kernel: 0 without Lagrange jobs, the Lagrange
// order + 1 when it has an instantiation, else -1.
inline int xfer_width(const XferJob *jobs, size_t n)
{
  int w = 0;
  for (size_t q = 0; q < n; q++) {
    if (jobs[q].method != XM_LAGRANGE) continue;
    const int p = jobs[q].ord + 1;
    const int pw = (p == 3 || p == 4 || p == 6 || p == 8 || p == 10) ? p : -1;
    if (w == 0) w = pw;
    else if (w != pw) w = -1;
  }
  return w;
}

// Whether a plan runs on the row kernel: Lagrange jobs only, with a window of
// at least 4 points (the order 3 restriction and the order+1 ghost fills).
inline bool xfer_rows(const XferJob *jobs, size_t n, int width)
{
  if (width < 4) return false;
  for (size_t q = 0; q < n; q++)
    if (jobs[q].method != XM_LAGRANGE) return false;
  return true;
}

// The tau transfer with the full weighting folded in: every job of the plan
// is a strided copy from the fine level, so the (1,2,1)^3/64 average of W is
// formed only at the fine nodes that are read (one in eight), with
// k_full_weight's terms and order (fw_sum).  DIFF: W = f[fa] - f[fb] (the FP32 cycle
// forms S - R where it is read), else W = f[fa].
template <class V, class Fields, bool DIFF>
__global__ void __launch_bounds__(256) k_xfer_fw(const XferJob *__restrict__ jobs, int njobs,
                                                 const DevBox *__restrict__ boxes, Fields F, int fa, int fb)
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
  const DevBox &T = boxes[J.tbox];
  if (J.iter != IT_ALL) {
    const int b = T.buf;
    const bool inside = i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b;
    if ((J.iter == IT_INSIDE) != inside) return;
  }
  const DevBox &S = boxes[J.sbox];
  const int si = J.sstart[0] + J.sstep[0] * (i - J.r0[0]);
  const int sj = J.sstart[1] + J.sstep[1] * (j - J.r0[1]);
  const int sk = J.sstart[2] + J.sstep[2] * (k - J.r0[2]);
  const V *wa = F.f[fa] + S.off;
  const V *wb = DIFF ? F.f[fb] + S.off : nullptr;
  auto w = [&](long long q) -> V { return DIFF ? wa[q] - wb[q] : wa[q]; };
  const long long sp = pidx(S, si, sj, sk);
  const V c = w(sp);
  const int b = S.buf;
  V val = c;
  if (si >= b && si < S.n[0] - b && sj >= b && sj < S.n[1] - b && sk >= b && sk < S.n[2] - b)
    val = fw_sum<V>(w, c, S, si, sj, sk, sp);
  F.f[J.tfield][T.off + pidx(T, i, j, k)] = val;
}

// The coarse-to-fine correction of one level in one pass: for every target
// of the (trilinear) prolongation plan, E_fine += P(E_coarse - WW_coarse),
// the difference formed at each source node as it is read (fe, fww: the
// solution / correction field and its copy from before the coarse solve).
// The same terms in the same order as V = E - WW, V_fine = P V,
// E += V_fine; targets the plan zeroes get a zero correction and are left
// as they are.
// The body of k_prolong_correct for virtual block vb of its plan: thread vtid
// of a block of vdim threads (the plan's pair blocks are 256 threads).
template <class V, class Fields>
__device__ __forceinline__ void prolong_correct_body(long long vb, int vtid, int vdim, const XferJob *__restrict__ jobs,
                                                     int njobs, const DevBox *__restrict__ boxes, Fields F,
                                                     const AxisEntry *__restrict__ tab, int fe, int fww)
{
  // two x-neighbour targets per thread: the job search, the index split, the
  // y and z axis entries and the boxes are shared by both
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].pblk0 <= vb) lo = mid;
    else hi = mid - 1;
  }
  const XferJob &J = jobs[lo];
  if (!boxes[J.tbox].active) return;   // the target's solve has stopped (whole block: one job)
  const long long t = (vb - J.pblk0) * vdim + vtid;
  const int e0 = J.r1[0] - J.r0[0], e1 = J.r1[1] - J.r0[1], e2 = J.r1[2] - J.r0[2];
  const int h0 = (e0 + 1) >> 1;
  if (t >= (long long)h0 * e1 * e2) return;
  const int ih = (int)t % h0;
  const int r = (int)t / h0;
  const int j = J.r0[1] + (r % e1);
  const int k = J.r0[2] + (r / e1);
  const DevBox T = boxes[J.tbox];
  const DevBox S = boxes[J.sbox];
  const int b = T.buf;
  const bool yz_inside = j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b;
  // y and z entries: from the job's per-parity entries on a periodic job,
  // else from the tables
  int sy_, sz_, ny, nz, ey, ez;
  double wy0, wy1, wz0, wz1;
  bool yz_sel = true;
  if (J.lin2) {
    const int qj = (j - J.r0[1]) & 1, qk = (k - J.r0[2]) & 1;
    const int mj = (j - J.r0[1]) >> 1, mk = (k - J.r0[2]) >> 1;
    sy_ = J.lstart[1][qj] + mj, sz_ = J.lstart[2][qk] + mk;
    ny = J.lnode[1][qj] + mj, nz = J.lnode[2][qk] + mk;
    ey = J.lexact[1][qj], ez = J.lexact[2][qk];
    wy0 = J.lw0[1][qj], wy1 = J.lw1[1][qj], wz0 = J.lw0[2][qk], wz1 = J.lw1[2][qk];
  } else {
    const AxisEntry &ay = tab[J.tab[1] + j];
    const AxisEntry &az = tab[J.tab[2] + k];
    yz_sel = ay.sel && az.sel;
    sy_ = ay.start, sz_ = az.start, ny = ay.node, nz = az.node;
    ey = ay.exact, ez = az.exact;
    wy0 = ay.w[0], wy1 = ay.w[1], wz0 = az.w[0], wz1 = az.w[1];
  }
  if (!yz_sel) return;
  const V *ec = F.f[fe] + S.off, *wc = F.f[fww] + S.off;
  V *ef = F.f[fe] + T.off;
  auto v = [&](long long q) -> V { return ec[q] - wc[q]; };
#pragma unroll
  for (int d = 0; d < 2; d++) {
    const int i = J.r0[0] + 2 * ih + d;
    if (i >= J.r1[0]) break;
    if (J.iter != IT_ALL) {
      const bool inside = yz_inside && i >= b && i < T.n[0] - b;
      if ((J.iter == IT_INSIDE) != inside) continue;
    }
    int sx, nx, ex;
    double wx0, wx1;
    if (J.lin2) {
      const int qi = (i - J.r0[0]) & 1, mi = (i - J.r0[0]) >> 1;
      sx = J.lstart[0][qi] + mi, nx = J.lnode[0][qi] + mi, ex = J.lexact[0][qi];
      wx0 = J.lw0[0][qi], wx1 = J.lw1[0][qi];
    } else {
      const AxisEntry &ax = tab[J.tab[0] + i];
      if (!ax.sel) continue;
      sx = ax.start, nx = ax.node, ex = ax.exact;
      wx0 = ax.w[0], wx1 = ax.w[1];
    }
    V vf;
    if (ex && ey && ez) {
      vf = v(pidx(S, nx, ny, nz));
    } else {
      const int i0 = sx, j0 = sy_, k0 = sz_;
      const V dxi = (V)wx0, dxf = (V)wx1, dyi = (V)wy0, dyf = (V)wy1, dzi = (V)wz0, dzf = (V)wz1;
      const V v000 = v(pidx(S, i0, j0, k0)), v100 = v(pidx(S, i0 + 1, j0, k0));
      const V v010 = v(pidx(S, i0, j0 + 1, k0)), v110 = v(pidx(S, i0 + 1, j0 + 1, k0));
      const V v001 = v(pidx(S, i0, j0, k0 + 1)), v101 = v(pidx(S, i0 + 1, j0, k0 + 1));
      const V v011 = v(pidx(S, i0, j0 + 1, k0 + 1)), v111 = v(pidx(S, i0 + 1, j0 + 1, k0 + 1));
      vf = ((v000 * dxi + v100 * dxf) * dyi + (v010 * dxi + v110 * dxf) * dyf) * dzi +
           ((v001 * dxi + v101 * dxf) * dyi + (v011 * dxi + v111 * dxf) * dyf) * dzf;
    }
    const long long tp = pidx(T, i, j, k);
    ef[tp] = ef[tp] + vf;
  }
}

template <class V, class Fields>
__global__ void __launch_bounds__(256) k_prolong_correct(const XferJob *__restrict__ jobs, int njobs,
                                                         const DevBox *__restrict__ boxes, Fields F,
                                                         const AxisEntry *__restrict__ tab, int fe, int fww)
{
  prolong_correct_body<V, Fields>(blockIdx.x, threadIdx.x, blockDim.x, jobs, njobs, boxes, F, tab, fe, fww);
}

// A refinement level's coarse-to-fine step in one launch: the correction of
// its INSIDE points (prolong_correct_body, two 256-thread pair blocks per
// block) and the ghost fill of its BOUNDARY points from the corrected coarse
// level (xfer_rows_body, the order+1 Lagrange rows).  The two write disjoint
// points and read only the coarse level, so running them side by side gives
// the bits of the two launches in a row.
template <class V, class Fields, int P>
__global__ void __launch_bounds__(32 * kRowWarps) k_prolong_ghost(const XferJob *__restrict__ pjobs, int npjobs,
                                                                  long long ppairs, const XferJob *__restrict__ gjobs,
                                                                  int ngjobs, const DevBox *__restrict__ boxes,
                                                                  Fields F, const AxisEntry *__restrict__ tab, int fe,
                                                                  int fww)
{
  static_assert(32 * kRowWarps == 512, "two pair blocks of 256 threads per block");
  const long long pblocks = (ppairs + 1) >> 1;
  if ((long long)blockIdx.x < pblocks) {
    const long long vb = 2 * (long long)blockIdx.x + (threadIdx.x >> 8);
    if (vb < ppairs) prolong_correct_body<V, Fields>(vb, threadIdx.x & 255, 256, pjobs, npjobs, boxes, F, tab, fe, fww);
    return;
  }
  xfer_rows_body<V, Fields, P>((long long)blockIdx.x - pblocks, gjobs, ngjobs, boxes, F, tab);
}

// Set_In of a refinement level with the coarse FP64 operator folded in:
// RHO = W + OP(u) at every target of the (strided, same-box) Set_In plan, OP
// evaluated as k_apply_op does on INSIDE points and 0 on the ghosts (R is 0
// there on a refinement level).  The coarse R is needed nowhere else.
template <int ORD, int EQ>
__global__ void __launch_bounds__(256) k_set_in_op(const XferJob *__restrict__ jobs, int njobs,
                                                   const DevBox *__restrict__ boxes, DevFields F)
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
  double rr = 0.0;
  if (i >= b && i < T.n[0] - b && j >= b && j < T.n[1] - b && k >= b && k < T.n[2] - b) {
    const double *u = F.f[F_U] + T.off;
    const double lv = lap<ORD>(u, tp, T.n[0], (long long)T.n[0] * T.n[1], T);
    double op, dop;
    point_op<EQ>(lv, T.dulap, u[tp], F.f[F_B][T.off + tp], F.f[F_C][T.off + tp],
                 EQ == 1 ? F.f[F_D][T.off + tp] : 0.0, EQ == 1 ? F.f[F_E][T.off + tp] : 0.0, op, dop);
    rr = op;
  }
  F.f[F_RHO][T.off + tp] = F.f[F_W][S.off + sp] + rr;
}

// ----------------------------------------------------------------------------
// K5: coarsest-grid solve in one CTA: repeat { Robin; one red-black sweep }
// until the sweep norm <= eps or stops changing (src/elliptic.cc:1782-1816),
// or drops below rtol times the first sweep's norm, or max_it sweeps ran.
// The interior update is over-relaxed (red-black SOR): only the coarse
// problem's solution enters the V-cycle, not the sweep that reaches it.
// u lives in shared memory; b, c, S (and d, e) are read through L1.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void cs_robin_point(const DevBox &B, double *u, const double *rho,
                                               const double *crd, int mask, int i, int j, int k,
                                               bool dirichlet)
{
  const long long p = pidx(B, i, j, k);
  if (dirichlet) {   // u = S on the boundary points
    u[p] = rho[p];
    return;
  }
  double dF;
  const double t = robin_term<2>(u, B, crd, mask, i, j, k, dF);
  const double Fv = t + u[p] - rho[p];
  u[p] = u[p] - Fv * rcp_approx64(dF);   // the divisor only sizes the step
}

template <int EQ>
__global__ void __launch_bounds__(1024) k_coarse_solve(const DevBox *__restrict__ boxes, int box, DevFields F,
                                                       const double *__restrict__ crd, double eps, int max_it,
                                                       double omega, double rtol, double *norm_out,
                                                       int *iters_out, int *nan_flag, int dirichlet)
{
  extern __shared__ double su[];
  __shared__ double red[32];
  __shared__ double s_norm;
  __shared__ int s_nan;
  const DevBox B = boxes[box];
  if (!B.active) return;   // one block
  const long long np = (long long)B.n[0] * B.n[1] * B.n[2];
  double *gu = F.f[F_U] + B.off;
  const double *gb = F.f[F_B] + B.off, *gc = F.f[F_C] + B.off, *gs = F.f[F_RHO] + B.off;
  const double *gd = EQ == 1 ? F.f[F_D] + B.off : nullptr, *ge = EQ == 1 ? F.f[F_E] + B.off : nullptr;
  for (long long p = threadIdx.x; p < np; p += blockDim.x) su[p] = gu[p];
  __syncthreads();
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
  const int m0 = n0 - 2, m1 = n1 - 2, m2 = n2 - 2;   // ghost width 1 on coarse grids
  const long long sy = n0, sz = (long long)n0 * n1;
  double norm = 1.0, prev, first = -1.0;
  int it = 0;
  do {
    prev = norm;
    // Robin update: faces, edges, corners
    for (int f = 0; f < 6; f++) {
      const int a = f >> 1, hi = f & 1, a1 = (a + 1) % 3, a2 = (a + 2) % 3;
      const int c1 = B.n[a1] - 2, c2 = B.n[a2] - 2;
      for (int t = threadIdx.x; t < c1 * c2; t += blockDim.x) {
        int ijk[3];
        ijk[a] = hi ? B.n[a] - 1 : 0;
        ijk[a1] = 1 + t % c1;
        ijk[a2] = 1 + t / c1;
        cs_robin_point(B, su, gs, crd, 1 << a, ijk[0], ijk[1], ijk[2], dirichlet);
      }
    }
    __syncthreads();
    {
      const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
      for (int pi = 0; pi < 3; pi++) {
        const int a = pairs[pi][0], c = pairs[pi][1], fa = 3 - a - c;
        const int m = B.n[fa] - 2;
        for (int t = threadIdx.x; t < 4 * m; t += blockDim.x) {
          const int e = t / m, q = t % m;
          int ijk[3];
          ijk[fa] = 1 + q;
          ijk[a] = (e >> 1) ? B.n[a] - 1 : 0;
          ijk[c] = (e & 1) ? B.n[c] - 1 : 0;
          cs_robin_point(B, su, gs, crd, (1 << a) | (1 << c), ijk[0], ijk[1], ijk[2], dirichlet);
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 8) {
      const int i = (threadIdx.x & 1) ? n0 - 1 : 0;
      const int j = ((threadIdx.x >> 1) & 1) ? n1 - 1 : 0;
      const int k = (threadIdx.x >> 2) ? n2 - 1 : 0;
      cs_robin_point(B, su, gs, crd, 7, i, j, k, dirichlet);
    }
    __syncthreads();
    // one red-black sweep
    double rmax = 0.0;
    const int H = (m0 + 1) / 2;
    for (int color = 0; color < 2; color++) {
      for (int t = threadIdx.x; t < H * m1 * m2; t += blockDim.x) {
        const int ih = t % H, r = t / H;
        const int j = 1 + r % m1, k = 1 + r / m1;
        const int i = 1 + ((color + 1 + j + k) & 1) + 2 * ih;
        if (i >= n0 - 1) continue;
        const long long p = pidx(B, i, j, k);
        const double lv = lap<2>(su, p, sy, sz, B);
        double op, dop;
        point_op<EQ>(lv, B.dulap, su[p], gb[p], gc[p], EQ == 1 ? gd[p] : 0.0, EQ == 1 ? ge[p] : 0.0, op, dop);
        const double R = op - gs[p];
        su[p] = su[p] - omega * (R * step_inverse(dop));
        rmax = fmax(rmax, fabs(R));
        if (!(su[p] == su[p])) atomicOr(nan_flag, 1);
      }
      __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = rmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmax(m, red[w]);
      s_norm = m;
      s_nan = *(volatile int *)nan_flag;
    }
    __syncthreads();
    norm = s_norm;
    const int stop_nan = s_nan;
    __syncthreads();
    it++;
    if (first < 0.0) first = norm;
    if (stop_nan) break;                           // uniform across the block
    if (rtol > 0.0 && norm <= rtol * first) break;
  } while (norm > eps && prev != norm && it < max_it);
  for (long long p = threadIdx.x; p < np; p += blockDim.x) gu[p] = su[p];
  if (threadIdx.x == 0) {
    *norm_out = norm;
    *iters_out = it;
  }
}

// ----------------------------------------------------------------------------
// K6: coefficients b, c (and d, e) at every point of every box
// ----------------------------------------------------------------------------
__device__ double dev_punctures_c(const PunctureParams &P, double X, double Y, double Z)
{
  double cval = 1;
  for (int i = 0; i < P.numbh; i++) {
    const double x = X - P.x[i], y = Y - P.y[i], z = Z - P.z[i];
    double r = sqrt(x * x + y * y + z * z);
    if (r < 2 * 2.220446049250313e-16) r = 2 * 2.220446049250313e-16;
    cval += 0.5 * P.mp[i] / r;
  }
  return cval;
}

__device__ double dev_punctures_b(const PunctureParams &P, double X, double Y, double Z)
{
  double A00 = 0, A11 = 0, A22 = 0, A01 = 0, A02 = 0, A12 = 0;
  for (int i = 0; i < P.numbh; i++) {
    const double x = X - P.x[i], y = Y - P.y[i], z = Z - P.z[i];
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    double r2 = x2 + y2 + z2;
    if (r2 < 2 * 2.220446049250313e-16) r2 = 2 * 2.220446049250313e-16;
    const double r = sqrt(r2);
    const double ir5 = 1.0 / (r2 * r2 * r);
    const double px = P.px[i], py = P.py[i], pz = P.pz[i], sx = P.sx[i], sy = P.sy[i], sz = P.sz[i];
    A00 += 1.5 * ir5 * (px * x * (x2 + r2) + py * y * (x2 - r2) + pz * z * (x2 - r2) + 4.0 * x * (sy * z - sz * y));
    A11 += 1.5 * ir5 * (px * x * (y2 - r2) + py * y * (y2 + r2) + pz * z * (y2 - r2) + 4.0 * y * (sz * x - sx * z));
    A22 += 1.5 * ir5 * (px * x * (z2 - r2) + py * y * (z2 - r2) + pz * z * (z2 + r2) + 4.0 * z * (sx * y - sy * x));
    A01 += 1.5 * ir5 * (px * y * (r2 + x2) + py * x * (r2 + y2) + pz * x * y * z - 2.0 * sx * x * z +
                        2.0 * sy * y * z + 2.0 * sz * (x2 - y2));
    A02 += 1.5 * ir5 * (px * z * (r2 + x2) + py * x * y * z + pz * x * (r2 + z2) + 2.0 * sx * x * y +
                        2.0 * sy * (z2 - x2) - 2.0 * sz * y * z);
    A12 += 1.5 * ir5 * (px * x * y * z + py * z * (r2 + y2) + pz * y * (r2 + z2) + 2.0 * sx * (y2 - z2) -
                        2.0 * sy * x * y + 2.0 * sz * x * z);
  }
  // sum over i,j of A_ij^2 in row-major order
  double bval = 0.0;
  bval += A00 * A00; bval += A01 * A01; bval += A02 * A02;
  bval += A01 * A01; bval += A11 * A11; bval += A12 * A12;
  bval += A02 * A02; bval += A12 * A12; bval += A22 * A22;
  return 0.125 * bval;
}

__device__ double dev_scalar_d(const PunctureParams &P, double X, double Y, double Z)
{
  const double r = sqrt(X * X + Y * Y + Z * Z);
  const double r0 = P.ps_r0, is = P.ps_isigma;
  switch (P.ps_case) {
  case 1: return P.ps_d1 / pow(cosh((r - r0) * is), 4.0);
  case 2: return P.ps_de1 * (r - r0) * (r - r0) * exp(-2 * is * (r - r0) * (r - r0));
  case 3: {
    const double l2 = 10000, x = r;
    const double s = 0.0581545 * (x - 1.8039e-08) * 0.0481646 * exp(-0.0581545 * (x - 1.8039e-08) * (x - 1.8039e-08) / l2) +
                     0.111412 * (x + 9.6741e-09) * 0.298408 * exp(-0.111412 * (x + 9.6741e-09) * (x + 9.6741e-09) / l2) +
                     0.207156 * (x - 1.09822e-08) * 0.42755 * exp(-0.207156 * (x - 1.09822e-08) * (x - 1.09822e-08) / l2) +
                     0.37742 * (x + 2.13778e-08) * 0.204229 * exp(-0.37742 * (x + 2.13778e-08) * (x + 2.13778e-08) / l2) +
                     0.68406 * (x - 8.78608e-08) * 0.021649 * exp(-0.68406 * (x - 8.78608e-08) * (x - 8.78608e-08) / l2);
    const double g = -2 * s / (l2 * l2);
    return CUDART_PI * g * g;
  }
  default: {
    const double a = 1. / cosh((r + r0) * is), c = 1. / cosh((r - r0) * is);
    const double q = a * a - c * c;
    return P.ps_de1 * 0.25 * q * q;
  }
  }
}

__device__ double dev_scalar_e(const PunctureParams &P, double X, double Y, double Z)
{
  const int c = P.ps_case;
  if (c == 2 || c == 3 || c == 4) {
    const double r = sqrt(X * X + Y * Y + Z * Z);
    const double r0 = P.ps_r0, is = P.ps_isigma;
    double phi;
    if (c == 2) {
      phi = P.ps_phi0 * exp(-(r - r0) * (r - r0) * is);
    } else if (c == 3) {
      const double l2 = 0.6, x = r;
      phi = (0.0481646 * exp(-0.0581545 * (x - 1.8039e-08) * (x - 1.8039e-08) / (l2)) +
             0.298408 * exp(-0.111412 * (x + 9.6741e-09) * (x + 9.6741e-09) / l2) +
             0.42755 * exp(-0.207156 * (x - 1.09822e-08) * (x - 1.09822e-08) / l2) +
             0.204229 * exp(-0.37742 * (x + 2.13778e-08) * (x + 2.13778e-08) / l2) +
             0.021649 * exp(-0.68406 * (x - 8.78608e-08) * (x - 8.78608e-08) / l2)) * l2;
    } else {
      phi = P.ps_phi0 * 0.5 * (tanh((r + r0) * is) - tanh((r - r0) * is));
    }
    const double ff = P.ps_e2 * phi;
    const double g = 1 - exp(ff);
    return P.ps_e1 * g * g * exp(-2 * ff);
  }
  return 0.0;
}

__global__ void __launch_bounds__(256) k_coefficients(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                      const double *__restrict__ crd, PunctureParams P)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const double x = crd[B.coord_off + i], y = crd[B.coord_off + B.n[0] + j],
               z = crd[B.coord_off + B.n[0] + B.n[1] + k];
  if (P.equation >= 2) {   // the test equations: b is the factor of u^2 (none for Bowen-York)
    F.f[F_B][B.off + t] = P.equation == 5 ? 0.0 : 1.0;
    F.f[F_C][B.off + t] = 0.0;
    return;
  }
  F.f[F_B][B.off + t] = dev_punctures_b(P, x, y, z);
  F.f[F_C][B.off + t] = dev_punctures_c(P, x, y, z);
  if (P.equation == 1) {
    F.f[F_D][B.off + t] = dev_scalar_d(P, x, y, z);
    F.f[F_E][B.off + t] = dev_scalar_e(P, x, y, z);
  }
}

// ----------------------------------------------------------------------------
// The reference's test equations (Lap u + u^2 = source) and their boundary
// functions, src/operator.cc:1772-1887: the Gaussian test (Poisson: u = a
// e^{-r^2/2}, which solves it), Boundary-test (a tanh(r)/r) and
// Multibox-test (two Gaussians centred at x = bhx1, bhx2).  Initial state
// (Set_Coefficients, Set_Boundary, src/boundary.cc:8-78): rho0 = the source
// on every point, then the boundary value on the BOUNDARY (ghost) points of
// every box (0 for Robin, the boundary function for Dirichlet); u = the
// boundary function on every point.
// ----------------------------------------------------------------------------
__device__ __forceinline__ bool dev_dcomp0(double r) { return fabs(r) <= 3 * DBL_EPSILON; }

__device__ double dev_test_function(const PunctureParams &P, double x, double y, double z)
{
  if (P.equation == 3) {   // test_boundary
    const double r = sqrt(x * x + y * y + z * z);
    return !dev_dcomp0(r) ? 0.004 * tanh(r) / r : 0.004;
  }
  if (P.equation == 4) {   // test_mfunct
    const double r2_1 = (x - P.x[0]) * (x - P.x[0]) + y * y + z * z;
    const double r2_2 = (x - P.x[1]) * (x - P.x[1]) + y * y + z * z;
    const double a = 0.05;
    return exp(-a * r2_1) + exp(-a * r2_2);
  }
  const double r2 = x * x + y * y + z * z;   // Gaussian
  return 0.004 * exp(-0.5 * r2);
}

__device__ double dev_test_source(const PunctureParams &P, double x, double y, double z)
{
  if (P.equation == 3) {   // test_boundary_source
    const double r = sqrt(x * x + y * y + z * z);
    return !dev_dcomp0(r) ? -2.0 * 0.004 * tanh(r) / (r * cosh(r) * cosh(r)) : -2.0 * 0.004;
  }
  if (P.equation == 4) {   // test_mfunct_source
    const double r2_1 = (x - P.x[0]) * (x - P.x[0]) + y * y + z * z;
    const double r2_2 = (x - P.x[1]) * (x - P.x[1]) + y * y + z * z;
    const double a = 0.05;
    return 2.0 * a * exp(-a * r2_1) * ((2 * a * r2_1 - 3)) + 2.0 * a * exp(-a * r2_2) * ((2 * a * r2_2 - 3));
  }
  const double r2 = x * x + y * y + z * z;   // Gaussian_source
  const double a = 0.004;
  return a * exp(-r2) * (a + exp(0.5 * r2) * (r2 - 3.0));
}

// Bowen_York_rho0/1/2 (src/operator.cc:3313-3408): momentum component `comp`
// of every puncture within one cell diagonal dr of the point, spread as
// 3 p / (4 pi dr^3).  Rounded operation by operation (no contraction): which
// points lie in a ball is decided by r <= dr, as in the reference.
__device__ double dev_by_source(const PunctureParams &P, int comp, double X, double Y, double Z, const DevBox &B)
{
  double cval = 0.0;
  const double dr = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(B.d[0], B.d[0]), __dmul_rn(B.d[1], B.d[1])),
                                         __dmul_rn(B.d[2], B.d[2])));
  const double vol = __dmul_rn(__dmul_rn(__dmul_rn(4.0 * M_PI, dr), dr), dr);
  for (int i = 0; i < P.numbh; i++) {
    const double x = __dsub_rn(X, P.x[i]), y = __dsub_rn(Y, P.y[i]), z = __dsub_rn(Z, P.z[i]);
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    const double pc = comp == 0 ? P.px[i] : comp == 1 ? P.py[i] : P.pz[i];
    if (r <= dr) cval = __dadd_rn(cval, __ddiv_rn(__dmul_rn(3.0, pc), vol));
  }
  return cval;
}

__global__ void __launch_bounds__(256) k_test_init(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                   const double *__restrict__ crd, PunctureParams P, int dirichlet)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const double x = crd[B.coord_off + i], y = crd[B.coord_off + B.n[0] + j],
               z = crd[B.coord_off + B.n[0] + B.n[1] + k];
  const int b = B.buf;
  const bool ghost = i < b || j < b || k < b || i >= B.n[0] - b || j >= B.n[1] - b || k >= B.n[2] - b;
  if (P.equation == 5) {   // Bowen-York: zero boundary function and initial guess; lambda's source
                           // is the divergence of V (k_by_divergence)
    F.f[F_RHO][B.off + t] = ghost || P.var == 3 ? 0.0 : dev_by_source(P, P.var, x, y, z, B);
    F.f[F_U][B.off + t] = 0.0;
    return;
  }
  const double g = dev_test_function(P, x, y, z);
  F.f[F_RHO][B.off + t] = ghost ? (dirichlet ? g : 0.0) : dev_test_source(P, x, y, z);
  F.f[F_U][B.off + t] = g;
}

// Bowen-York's lambda equation, Lap lambda - (Dx V1 + Dy V2 + Dz V3) = 0
// (include/elliptic.h:796-800), with the divergence in the source: rho of
// every INSIDE point := Dx V1 + Dy V2 + Dz V3 of the solved V (v: V1, V2, V3
// one after another, each laid out like a field of the arena, stride
// `total`), with the order's first-derivative stencil (dx2, or dx4 for
// orders 4-8).  The divergence of each level's V enters both sides of that
// level's FAS tau correction and cancels, so the fixed point is the system's.
__global__ void __launch_bounds__(256) k_by_divergence(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                       const double *__restrict__ v, long long total)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const int b = B.buf;
  if (i < b || j < b || k < b || i >= B.n[0] - b || j >= B.n[1] - b || k >= B.n[2] - b) return;
  const long long st[3] = {1, (long long)B.n[0], (long long)B.n[0] * B.n[1]};
  const int ijk[3] = {i, j, k};
  double d[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double *va = v + a * total + B.off;
    double du;
    d[a] = B.order == 2 ? deriv<2>(va, t, st[a], ijk[a], B.n[a], B.idx[a], du)
                        : deriv<4>(va, t, st[a], ijk[a], B.n[a], B.idx[a], du);
  }
  F.f[F_RHO][B.off + t] = d[0] + d[1] + d[2];
}

// ----------------------------------------------------------------------------
// elliptic::ApproximateID (src/elliptic.cc:1977-2226): the perturbative
// puncture solution, summed over the punctures on every point of every box:
// with R = 2 r / m and l = 1 / (1 + R), the spin part
//   J^2 (u0j + u2j R^2 P2(mu_S)),  u0j = (l + l^2 + l^3 - 4 l^4 + 2 l^5) / 40,
//   u2j = -l^5 / 20,  J = 4 S / m^2,
// the momentum part
//   P^2 (u0p + u2p P2(mu_P)),  P = 2 p / m,
//   u0p = (5/32) (l - 2 l^2 + 2 l^3 - l^4 + l^5 / 5),
//   u2p = (15 l + 132 l^2 + 53 l^3 + 96 l^4 + 82 l^5 + 84 (l^5 + ln(l) / R) / R) / (80 R),
// and the cross term (P x J) . (2 x / m) (1 + 5 R + 10 R^2) l^5 / 80; P2 is
// the Legendre polynomial of the cosine between the point's direction and
// the spin (momentum), 0 where that vector vanishes; r below 1e-11 is taken
// as 1e-10.  Products, quotients and sums are rounded one by one in the
// reference's order; near a puncture the u2p bracket cancels (about 1/R^2
// amplification of rounding), so its value there is only as good as that.
// With `stable` (a starting guess rather than the reference's printout) u2p
// below R = 1e-3 takes the leading term of its series instead: the bracket
// is R^3 / 5 + O(R^4), so u2p = R^2 / 400 + O(R^3), where the formula as
// written returns rounding noise of order 1e10 on a puncture that sits on
// a grid node (r clamped to 1e-10).
// ----------------------------------------------------------------------------
__device__ double dev_approx_u(const PunctureParams &P, double x, double y, double z, bool stable)
{
  double u = 0.0;
  for (int i = 0; i < P.numbh && P.mp[i] != 0.0; i++) {
    const double sbl = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(P.sx[i], P.sx[i]), __dmul_rn(P.sy[i], P.sy[i])),
                                            __dmul_rn(P.sz[i], P.sz[i])));
    const double imass = __ddiv_rn(1.0, P.mp[i]);
    const double imass2 = __dmul_rn(imass, imass);
    const double Jx = __dmul_rn(__dmul_rn(4.0, P.sx[i]), imass2);
    const double Jy = __dmul_rn(__dmul_rn(4.0, P.sy[i]), imass2);
    const double Jz = __dmul_rn(__dmul_rn(4.0, P.sz[i]), imass2);
    const double J2 = __dadd_rn(__dadd_rn(__dmul_rn(Jx, Jx), __dmul_rn(Jy, Jy)), __dmul_rn(Jz, Jz));
    const double pbl = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(P.px[i], P.px[i]), __dmul_rn(P.py[i], P.py[i])),
                                            __dmul_rn(P.pz[i], P.pz[i])));
    const double Px = __dmul_rn(__dmul_rn(2.0, P.px[i]), imass);
    const double Py = __dmul_rn(__dmul_rn(2.0, P.py[i]), imass);
    const double Pz = __dmul_rn(__dmul_rn(2.0, P.pz[i]), imass);
    const double P2 = __dadd_rn(__dadd_rn(__dmul_rn(Px, Px), __dmul_rn(Py, Py)), __dmul_rn(Pz, Pz));
    const double xi = __dsub_rn(x, P.x[i]), yi = __dsub_rn(y, P.y[i]), zi = __dsub_rn(z, P.z[i]);
    double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(xi, xi), __dmul_rn(yi, yi)), __dmul_rn(zi, zi)));
    if (fabs(r) <= 0.00000000001) r = 0.0000000001;
    const double Rx = __dmul_rn(__dmul_rn(2.0, xi), imass);
    const double Ry = __dmul_rn(__dmul_rn(2.0, yi), imass);
    const double Rz = __dmul_rn(__dmul_rn(2.0, zi), imass);
    const double R = __dmul_rn(__dmul_rn(2.0, r), imass);
    const double l1 = __ddiv_rn(1.0, __dadd_rn(1.0, R));
    const double l2 = __dmul_rn(l1, l1), l3 = __dmul_rn(l2, l1), l4 = __dmul_rn(l3, l1), l5 = __dmul_rn(l4, l1);
    const double u0j = __dmul_rn(
        0.025, __dadd_rn(__dsub_rn(__dadd_rn(__dadd_rn(l1, l2), l3), __dmul_rn(4.0, l4)), __dmul_rn(2.0, l5)));
    const double u2j = __dmul_rn(-0.05, l5);
    double muj = 0.0;
    if (sbl != 0.0 && r != 0.0)
      muj = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(P.sx[i], xi), __dmul_rn(P.sy[i], yi)), __dmul_rn(P.sz[i], zi)),
                      __dmul_rn(r, sbl));
    const double PL2j = __dmul_rn(0.5, __dsub_rn(__dmul_rn(__dmul_rn(3.0, muj), muj), 1.0));
    const double uj = __dmul_rn(J2, __dadd_rn(u0j, __dmul_rn(__dmul_rn(__dmul_rn(u2j, R), R), PL2j)));
    const double u0p = __dmul_rn(
        0.15625, __dadd_rn(__dsub_rn(__dadd_rn(__dsub_rn(l1, __dmul_rn(2.0, l2)), __dmul_rn(2.0, l3)), l4),
                           __dmul_rn(0.2, l5)));
    double br = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(15.0, l1), __dmul_rn(132.0, l2)),
                                              __dmul_rn(53.0, l3)), __dmul_rn(96.0, l4)), __dmul_rn(82.0, l5));
    br = __dadd_rn(br, __ddiv_rn(__dmul_rn(84.0, __dadd_rn(l5, __ddiv_rn(log(l1), R))), R));
    double u2p = __ddiv_rn(__dmul_rn(0.0125, br), R);
    if (stable && R < 1e-3) u2p = __dmul_rn(0.0025, __dmul_rn(R, R));
    double mup = 0.0;
    if (pbl != 0.0 && r != 0.0)
      mup = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(P.px[i], xi), __dmul_rn(P.py[i], yi)), __dmul_rn(P.pz[i], zi)),
                      __dmul_rn(r, pbl));
    const double PL2p = __dmul_rn(0.5, __dsub_rn(__dmul_rn(__dmul_rn(3.0, mup), mup), 1.0));
    const double up = __dmul_rn(P2, __dadd_rn(u0p, __dmul_rn(u2p, PL2p)));
    const double X0 = __dsub_rn(__dmul_rn(Py, Jz), __dmul_rn(Pz, Jy));
    const double X1 = __dsub_rn(__dmul_rn(Pz, Jx), __dmul_rn(Px, Jz));
    const double X2 = __dsub_rn(__dmul_rn(Px, Jy), __dmul_rn(Py, Jx));
    const double dotr = __dadd_rn(__dadd_rn(__dmul_rn(X0, Rx), __dmul_rn(X1, Ry)), __dmul_rn(X2, Rz));
    const double poly = __dadd_rn(__dadd_rn(1.0, __dmul_rn(5.0, R)), __dmul_rn(__dmul_rn(10.0, R), R));
    const double uc = __dmul_rn(__dmul_rn(__dmul_rn(0.0125, dotr), poly), l5);
    u = __dadd_rn(u, __dadd_rn(__dadd_rn(uj, up), uc));
  }
  return u;
}

__global__ void __launch_bounds__(256) k_approx_id(BoxList L, const DevBox *__restrict__ boxes, DevFields F,
                                                   const double *__restrict__ crd, PunctureParams P, int stable)
{
  long long lb;
  const DevBox B = boxes[list_box(L, lb)];
  if (!B.active) return;
  const long long t = lb * blockDim.x + threadIdx.x;
  const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
  if (t >= n) return;
  const int i = ((int)t % B.n[0]);
  const int r = (int)t / B.n[0];
  const int j = (r % B.n[1]), k = (r / B.n[1]);
  const double x = crd[B.coord_off + i], y = crd[B.coord_off + B.n[0] + j],
               z = crd[B.coord_off + B.n[0] + B.n[1] + k];
  F.f[F_U][B.off + t] = dev_approx_u(P, x, y, z, stable != 0);
}

// ----------------------------------------------------------------------------
// K7: u at each puncture by 4th-order Lagrange on the finest box (ADM mass)
// ----------------------------------------------------------------------------
struct AdmJob {
  int box;
  int exact;
  int node[3];
  int start[3];
  double w[3][5];
};

__global__ void k_adm(const AdmJob *__restrict__ jobs, int n, const DevBox *__restrict__ boxes, DevFields F,
                      double *out)
{
  const int q = threadIdx.x;
  if (q >= n) return;
  const AdmJob J = jobs[q];
  const DevBox S = boxes[J.box];
  if (!S.active) return;
  const double *u = F.f[F_U] + S.off;
  if (J.exact) {
    out[q] = u[pidx(S, J.node[0], J.node[1], J.node[2])];
    return;
  }
  double fx = 0.0;
  for (int I = 0; I <= 4; I++) {
    double uy = 0.0;
    for (int Jj = 0; Jj <= 4; Jj++) {
      double uz = 0.0;
      for (int K = 0; K <= 4; K++) uz += u[pidx(S, J.start[0] + I, J.start[1] + Jj, J.start[2] + K)] * J.w[2][K];
      uy += uz * J.w[1][Jj];
    }
    fx += uy * J.w[0][I];
  }
  out[q] = fx;
}

// ----------------------------------------------------------------------------
// u at arbitrary points: the reference's printed cuts and exports.
// multigrid::Print_Interpol_1D / _2D (src/multigrid.cc:151-261, 555-880) read
// each point from the last box, in level order, whose interior holds it
// (domain::is_in_nb, include/domain.h:839-850), the largest box when none
// does, and print nothing for a point outside the largest box (domain::is_in);
// ffunction::Print_1D (src/ffunction.cc:819-960) reads one given box.  The
// value is ffunction::Lagrange_Interpol_In (src/interpolation.cc:188-375):
// the node value where the point coincides with a node on every axis (the
// 3-epsilon test), else the tensor Lagrange sum over ord+1 nodes per axis,
// the window clamped to the box, summed over z, then y, then x.  Every
// product, quotient and sum is rounded on its own (no fused multiply-add), in
// the reference's order, so the result is the host's bit for bit.
// ----------------------------------------------------------------------------
struct InterpBox {
  double lo[3], hi[3], d[3];
  int n[3];
  int buf;
  long long off;
};

constexpr int kMaxInterpOrd = 15;

__device__ __forceinline__ double ib_coord(const InterpBox &B, int a, int i)
{
  return __dadd_rn(B.lo[a], __dmul_rn((double)i, B.d[a]));   // domain::Get_x: xi + i dx
}

__device__ __forceinline__ bool ib_dcomp(double x, double y) { return fabs(__dsub_rn(x, y)) <= 3 * DBL_EPSILON; }

// domain::Get_i: the first node at or after x (binary search)
__device__ int ib_locate(const InterpBox &B, int a, double x)
{
  const int np = B.n[a];
  int lo_i = 0, hi_i = np, i;
  if (__dsub_rn(B.lo[a], x) < 0.0 && __dsub_rn(x, B.hi[a]) < 0.0) {
    i = np % 2 == 0 ? np / 2 : (np - 1) / 2;
    do {
      const double xi = ib_coord(B, a, i);
      if (xi > x || ib_dcomp(xi, x))
        hi_i = i;
      else
        lo_i = i;
      i = (hi_i + lo_i) / 2;
    } while (lo_i + 1 < hi_i);
  } else {
    i = (B.lo[a] >= x) ? 0 : np - 2;
  }
  return i + 1;
}

__device__ __forceinline__ bool ib_is_in(const InterpBox &B, const double p[3])
{
  for (int a = 0; a < 3; a++) {
    const double m = __dmul_rn(B.d[a], 0.1);
    if (!(__dsub_rn(B.lo[a], m) <= p[a] && p[a] <= __dadd_rn(B.hi[a], m))) return false;
  }
  return true;
}

__device__ __forceinline__ bool ib_is_in_nb(const InterpBox &B, const double p[3])
{
  for (int a = 0; a < 3; a++) {
    const double m = __dmul_rn(B.d[a], __dsub_rn((double)B.buf, 0.1));
    if (!(__dadd_rn(B.lo[a], m) < p[a] && p[a] < __dsub_rn(B.hi[a], m))) return false;
  }
  return true;
}

// LagrangePoly (src/interpolation.cc:308-375)
__device__ double ib_lagrange(const InterpBox &B, int a, double t, int i, int ni, int nf)
{
  double lp = 1.0;
  const double ti = ib_coord(B, a, i);
  for (int j = ni; j < i; j++) {
    const double cj = ib_coord(B, a, j);
    lp = __dmul_rn(lp, __ddiv_rn(__dsub_rn(t, cj), __dsub_rn(ti, cj)));
  }
  for (int j = i + 1; j <= nf; j++) {
    const double cj = ib_coord(B, a, j);
    lp = __dmul_rn(lp, __ddiv_rn(__dsub_rn(t, cj), __dsub_rn(ti, cj)));
  }
  return lp;
}

// One thread per point.  box >= 0: that box; box < 0: the printed-cut rule
// over boxes first .. nboxes-1 with `base` the largest (NaN outside it).
__global__ void __launch_bounds__(128) k_interp_points(const InterpBox *__restrict__ boxes, int first, int nboxes,
                                                       int base, int box, const double *__restrict__ u,
                                                       const double *__restrict__ xyz, long long npts, int ord,
                                                       double *__restrict__ out)
{
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npts) return;
  const double p[3] = {xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]};
  int g = box;
  if (g < 0) {
    if (!ib_is_in(boxes[base], p)) {
      out[q] = __longlong_as_double(0x7ff8000000000000LL);
      return;
    }
    g = base;
    for (int b = first; b < nboxes; b++)
      if (ib_is_in_nb(boxes[b], p)) g = b;
  }
  const InterpBox B = boxes[g];
  const double *f = u + B.off;
  const long long sy = B.n[0], sz = (long long)B.n[0] * B.n[1];
  int node[3], st[3];
  bool exact = true;
  for (int a = 0; a < 3; a++) {
    node[a] = ib_locate(B, a, p[a]);
    exact = exact && node[a] < B.n[a] && ib_dcomp(p[a], ib_coord(B, a, node[a]));
    int s = ord % 2 == 0 ? node[a] - ord / 2 : node[a] - (ord + 1) / 2;
    if (s < 0) s = 0;
    else if (s + ord >= B.n[a]) s = B.n[a] - ord - 1;
    st[a] = s;
  }
  if (exact) {
    out[q] = f[node[0] + node[1] * sy + node[2] * sz];
    return;
  }
  double wy[kMaxInterpOrd + 1], wz[kMaxInterpOrd + 1];
  for (int J = 0; J <= ord; J++) wy[J] = ib_lagrange(B, 1, p[1], st[1] + J, st[1], st[1] + ord);
  for (int K = 0; K <= ord; K++) wz[K] = ib_lagrange(B, 2, p[2], st[2] + K, st[2], st[2] + ord);
  double fx = 0.0;
  for (int I = 0; I <= ord; I++) {
    double uy = 0.0;
    for (int J = 0; J <= ord; J++) {
      const double *col = f + (st[0] + I) + (st[1] + J) * sy + st[2] * sz;
      double uz = 0.0;
      for (int K = 0; K <= ord; K++) uz = __dadd_rn(uz, __dmul_rn(col[K * sz], wz[K]));
      uy = __dadd_rn(uy, __dmul_rn(uz, wy[J]));
    }
    fx = __dadd_rn(fx, __dmul_rn(uy, ib_lagrange(B, 0, p[0], st[0] + I, st[0], st[0] + ord)));
  }
  out[q] = fx;
}

}  // namespace olgpu
