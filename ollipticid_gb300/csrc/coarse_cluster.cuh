// coarse_cluster.cuh -- the coarsest-grid solve spread over one thread-block
// cluster.
//
// Same iteration as k_coarse_solve (src/elliptic.cc:1782-1816 semantics:
// repeat { Robin update; one red-black sweep } until the norm is <= eps or
// stops changing, plus the relative stop and SOR of the device solver), but
// the box's z-planes are split between the NCTA blocks of one cluster, each
// holding its slab of u in shared memory.  Stencil reads of neighbouring
// planes go to the owning block's shared memory through distributed shared
// memory; every write is to the writer's own slab.  On GB300 one SM issues
// only a few FP64 FMAs per clock, so the sweeps are spread over the cluster.
//
// Ownership keeps the Robin update local: block 0 owns the low ghost plane
// and the two interior planes above it, the last block the mirror image, and
// the others share the planes in between (cslab_begin; the balanced layout,
// cslab_begin_bal, moves one of those planes to the next block and separates
// the Robin phases by cluster barriers instead).  A face point reads interior points
// of its own plane (or, on a z face, the two planes next to it); an edge
// point reads face points, a corner edge points, all in planes its block
// owns.  So faces -> edges -> corners need only block barriers, and since
// the Robin update writes no interior point, colour 0 may follow at once.
// Two cluster barriers per iteration remain: after colour 0 (colour 1 reads
// its z neighbours) and after colour 1 (the norm, and the next iteration's
// colour 0).  The updates are the same as with one barrier per phase.
#pragma once

#include "kernels.cuh"

#include <cooperative_groups.h>

namespace olgpu {

// First plane of block r: block 0 holds [0, 3), block ncta-1 holds
// [n2-3, n2), blocks 1..ncta-2 share [3, n2-3) evenly.  Needs n2 >= 6, a
// ghost band of one plane and ncta >= 3.
__host__ __device__ inline int cslab_begin(int r, int n2, int ncta)
{
  if (r <= 0) return 0;
  if (r >= ncta) return n2;
  if (r == ncta - 1) return n2 - 3;
  const int m = n2 - 6, k = ncta - 2, rr = r - 1;
  const int base = m / k, rem = m % k;
  return 3 + rr * base + (rr < rem ? rr : rem);
}

// The balanced layout (bal = 1): block 0 holds [0, 2), the ghost plane and
// one interior plane, block ncta-1 [n2-2, n2), blocks 1..ncta-2 share
// [2, n2-2) evenly, so that on 16 blocks no block sweeps more than about one
// plane.  A z-face Robin point then reads plane 2 (n2-3) of the next block,
// and the edges and corners beside it read that block's face and edge
// points: faces, edges and corners are separated by cluster barriers
// instead of block barriers.  The updates are the same.
__host__ __device__ inline int cslab_begin_bal(int r, int n2, int ncta)
{
  if (r <= 0) return 0;
  if (r >= ncta) return n2;
  if (r == ncta - 1) return n2 - 2;
  const int m = n2 - 4, k = ncta - 2, rr = r - 1;
  const int base = m / k, rem = m % k;
  return 2 + rr * base + (rr < rem ? rr : rem);
}

__host__ __device__ inline int cslab_at(int r, int n2, int ncta, int bal)
{
  return bal ? cslab_begin_bal(r, n2, ncta) : cslab_begin(r, n2, ncta);
}

template <int EQ, int NCTA>
__global__ void __launch_bounds__(256) k_coarse_cluster(const DevBox *__restrict__ boxes, int box, DevFields F,
                                                        const double *__restrict__ crd, double eps, int max_it,
                                                        double omega, double rtol, double *norm_out,
                                                        int *iters_out, int *nan_flag, int dirichlet, int bal)
{
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ double su[];
  __shared__ double *plane[64];
  __shared__ double red[8];                // one slot per warp (256 threads)
  __shared__ int red_nan[8];
  __shared__ double s_part[2][2];          // per iteration parity: [0] max |R| of this block, [1] NaN seen
  __shared__ double s_x[3][64], s_ix[3][64];   // node coordinates and their reciprocals

  const DevBox B = boxes[box];
  if (!B.active) return;   // every block of the cluster reads the same box: all leave
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
  const int n01 = n0 * n1;
  const int kz0 = cslab_at(rank, n2, NCTA, bal), kz1 = cslab_at(rank + 1, n2, NCTA, bal);
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    int r = 0;
    while (cslab_at(r + 1, n2, NCTA, bal) <= k) r++;
    plane[k] = cl.map_shared_rank(su, r) + (k - cslab_at(r, n2, NCTA, bal)) * n01;
  }
  double *gu = F.f[F_U] + B.off;
  const double *gb = F.f[F_B] + B.off, *gc = F.f[F_C] + B.off, *gs = F.f[F_RHO] + B.off;
  const double *gd = EQ == 1 ? F.f[F_D] + B.off : nullptr, *ge = EQ == 1 ? F.f[F_E] + B.off : nullptr;
  for (int p = threadIdx.x; p < (kz1 - kz0) * n01; p += blockDim.x) su[p] = gu[(long long)kz0 * n01 + p];
  for (int t = threadIdx.x; t < n0 + n1 + n2; t += blockDim.x) {
    const int a = t < n0 ? 0 : t < n0 + n1 ? 1 : 2;
    const int i = t - (a == 0 ? 0 : a == 1 ? n0 : n0 + n1);
    const double x = crd[B.coord_off + t];
    s_x[a][i] = x;
    s_ix[a][i] = 1.0 / x;   // ghost nodes lie on the outer faces, never at 0
  }
  cl.sync();

  auto U = [&](int i, int j, int k) -> double & { return plane[k][j * n0 + i]; };
  // one-sided order-2 derivative along axis a at a ghost position
  auto d1 = [&](int a, int i, int j, int k, double &du) -> double {
    const int idx[3] = {i, j, k};
    const double id = B.idx[a];
    const int s = idx[a] == 0 ? 1 : -1;
    int p1[3] = {i, j, k}, p2[3] = {i, j, k};
    p1[a] += s;
    p2[a] += 2 * s;
    const double u0 = U(i, j, k), u1 = U(p1[0], p1[1], p1[2]), u2 = U(p2[0], p2[1], p2[2]);
    if (idx[a] == 0) {
      du = -3.0 * 0.5 * id;
      return (-3.0 * u0 + 4.0 * u1 - u2) * 0.5 * id;
    }
    du = 3.0 * 0.5 * id;
    return (3.0 * u0 - 4.0 * u1 + u2) * 0.5 * id;
  };
  // Newton update of one Robin point (Boundary_Face/Edge/Corner grouping).
  // The divisions by the coordinate are products with its reciprocal (within
  // an ulp); the Newton step divides by an approximate reciprocal of the
  // derivative, which only sizes the step (F = 0 stays the solution).
  auto robin = [&](int mask, int i, int j, int k) {
    if (dirichlet) {   // u = S on the boundary points
      U(i, j, k) = gs[((long long)k * n1 + j) * n0 + i];
      return;
    }
    const double r2s = s_x[0][i] * s_x[0][i] + s_x[1][j] * s_x[1][j] + s_x[2][k] * s_x[2][k];
    const double r2 = B.falloff == 2 ? 0.5 * r2s : r2s;   // r^2 / n
    const int ijk[3] = {i, j, k};
    double tF = 0.0, dF = 1.0, t = 0.0, dt = 0.0;
    int na = 0;
    const bool face = mask == 1 || mask == 2 || mask == 4;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      if (!(mask & (1 << a))) continue;
      double du;
      const double dv = d1(a, i, j, k, du);
      const double ia = s_ix[a][ijk[a]];
      if (face) {
        tF = r2 * dv * ia;
        dF = r2 * du * ia + 1.0;
      } else {
        t = na == 0 ? dv * ia : t + dv * ia;
        dt = na == 0 ? du * ia : dt + du * ia;
        na++;
      }
    }
    if (!face) {
      tF = r2 * t;
      dF = r2 * dt + 1.0;
    }
    double &uu = U(i, j, k);
    const double Fv = tF + uu - gs[((long long)k * n1 + j) * n0 + i];
    uu = uu - Fv * rcp_approx64(dF);
  };

  double norm = 1.0, prev, first = -1.0;
  int it = 0;
  const int mi0 = n0 - 2, mi1 = n1 - 2;
  do {
    prev = norm;
    // Robin update of this block's planes: faces, edges, corners
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
    if (bal) cl.sync();   // the edges at a z face read the next block's faces
    else __syncthreads();
    for (int k = kz0; k < kz1; k++) {
      if (k == 0 || k == n2 - 1) {
        for (int t = threadIdx.x; t < 2 * mi1 + 2 * mi0; t += blockDim.x) {
          if (t < 2 * mi1) robin(5, (t & 1) ? n0 - 1 : 0, 1 + (t >> 1), k);   // XZ edges
          else {
            const int q = t - 2 * mi1;
            robin(6, 1 + (q >> 1), (q & 1) ? n1 - 1 : 0, k);                   // YZ edges
          }
        }
      } else if (threadIdx.x < 4) {
        robin(3, (threadIdx.x & 1) ? n0 - 1 : 0, (threadIdx.x & 2) ? n1 - 1 : 0, k);   // XY edges
      }
    }
    if (bal) cl.sync();   // the corners at a z face read the next block's edges
    else __syncthreads();
    for (int k = kz0; k < kz1; k++)
      if ((k == 0 || k == n2 - 1) && threadIdx.x < 4)
        robin(7, (threadIdx.x & 1) ? n0 - 1 : 0, (threadIdx.x & 2) ? n1 - 1 : 0, k);
    __syncthreads();
    // one red-black SOR sweep over the interior points of this block's planes
    unsigned long long rbits = 0ull;
    int nan_seen = 0;
    const int ka = kz0 > 1 ? kz0 : 1, kb = kz1 < n2 - 1 ? kz1 : n2 - 1;
    const int H = (mi0 + 1) / 2;
    for (int color = 0; color < 2; color++) {
      for (int t = threadIdx.x; t < H * mi1 * (kb > ka ? kb - ka : 0); t += blockDim.x) {
        const int ih = t % H, r = t / H;
        const int j = 1 + r % mi1, k = ka + r / mi1;
        const int i = 1 + ((color + 1 + j + k) & 1) + 2 * ih;
        if (i >= n0 - 1) continue;
        const double c0 = U(i, j, k);
        const long long p = ((long long)k * n1 + j) * n0 + i;
        double nl, dop;
        point_terms<EQ>(B.dulap, c0, gb[p], gc[p], EQ == 1 ? gd[p] : 0.0, EQ == 1 ? ge[p] : 0.0, nl, dop);
        double R;
        if (B.iso) {   // equal spacing: the neighbour sum, its scale and the pointwise terms in one multiply-add
          const double sum = (U(i + 1, j, k) + U(i - 1, j, k)) + (U(i, j + 1, k) + U(i, j - 1, k)) +
                             (U(i, j, k + 1) + U(i, j, k - 1)) - 6.0 * c0;
          R = fma(sum, B.lscale, nl - gs[p]);
        } else {
          const double lapv = (U(i + 1, j, k) - 2.0 * c0 + U(i - 1, j, k)) * B.idx2[0] +
                              (U(i, j + 1, k) - 2.0 * c0 + U(i, j - 1, k)) * B.idx2[1] +
                              (U(i, j, k + 1) - 2.0 * c0 + U(i, j, k - 1)) * B.idx2[2];
          R = lapv + (nl - gs[p]);
        }
        const double un = c0 - R * (omega * step_inverse(dop));
        U(i, j, k) = un;
        // |R| on the bits (the integer pipe); a NaN's pattern is above infinity's
        rbits = max(rbits, (unsigned long long)__double_as_longlong(R) & 0x7fffffffffffffffull);
        if (is_nan_bits(un)) nan_seen = 1;
      }
      if (color == 0) cl.sync();   // colour 1 reads colour 0 of the neighbouring blocks
    }
    // this block's partial norm into the slot of this iteration's parity
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      rbits = max(rbits, __shfl_xor_sync(0xffffffffu, rbits, o));
      nan_seen |= __shfl_xor_sync(0xffffffffu, nan_seen, o);
    }
    const double rmax = __longlong_as_double((long long)rbits);
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = rmax;
      red_nan[threadIdx.x >> 5] = nan_seen;
    }
    __syncthreads();
    const int par = it & 1;
    if (threadIdx.x == 0) {
      double m = 0.0;
      int nn = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        m = fmax(m, red[w]);
        nn |= red_nan[w];
      }
      s_part[par][0] = m;
      s_part[par][1] = nn ? 1.0 : 0.0;
    }
    cl.sync();   // every block's colour 1 and partial norm are done
    // Every block reads all partials of this parity in the same order, so all
    // take the same decision.  The slot is written again two iterations later,
    // after two more cluster barriers this block must reach first.
    double m = 0.0, nn = 0.0;
#pragma unroll
    for (int r = 0; r < NCTA; r++) {
      const double *pr = cl.map_shared_rank(&s_part[par][0], r);
      m = fmax(m, pr[0]);
      nn = fmax(nn, pr[1]);
    }
    norm = m;
    if (nn > 0.0 && rank == 0 && threadIdx.x == 0) atomicOr(nan_flag, 1);
    it++;
    if (first < 0.0) first = norm;
    if (nn > 0.0) break;                           // the same decision in every block
    if (rtol > 0.0 && norm <= rtol * first) break;
  } while (norm > eps && prev != norm && it < max_it);
  cl.sync();   // every block is done reading its neighbours' shared memory
  for (int p = threadIdx.x; p < (kz1 - kz0) * n01; p += blockDim.x) gu[(long long)kz0 * n01 + p] = su[p];
  if (rank == 0 && threadIdx.x == 0) {
    *norm_out = norm;
    *iters_out = it;
  }
}

}  // namespace olgpu
