// coarse_cluster.cuh -- the coarsest-grid solve spread over one thread-block
// cluster.
//
// Same iteration as k_coarse_solve (src/elliptic.cc:1782-1816 semantics:
// repeat { Robin update; one red-black sweep } until the norm is <= eps or
// stops changing, plus the relative stop and SOR of the device solver), but
// the box's z-planes are split between the NCTA blocks of one cluster, each
// holding its slab of u in shared memory.  Stencil reads of neighbouring
// planes go to the owning block's shared memory through distributed shared
// memory; every write is to the writer's own slab.  Phases are separated by
// cluster barriers.  On GB300 one SM issues only a few FP64 FMAs per clock, so
// a 17^3 FP64 sweep in one block is ~60 us; sixteen blocks divide that.
#pragma once

#include "kernels.cuh"

#include <cooperative_groups.h>

namespace olgpu {

template <int EQ, int NCTA>
__global__ void __launch_bounds__(256) k_coarse_cluster(const DevBox *__restrict__ boxes, int box, DevFields F,
                                                        const double *__restrict__ crd, double eps, int max_it,
                                                        double omega, double rtol, double *norm_out,
                                                        int *iters_out, int *nan_flag)
{
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ double su[];
  __shared__ double *slab[NCTA];
  __shared__ int z0s[NCTA + 1];
  __shared__ unsigned char owner[64];
  __shared__ double red[8], red_nan[8];   // one slot per warp (256 threads)
  __shared__ double s_part[2];   // [0] this block's max |R|, [1] NaN seen (0/1)
  __shared__ double s_norm;
  __shared__ int s_stop;

  const DevBox B = boxes[box];
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2];
  const int n01 = n0 * n1;
  if (threadIdx.x == 0) {
    const int base = n2 / NCTA, rem = n2 % NCTA;
    int z = 0;
    for (int r = 0; r < NCTA; r++) {
      z0s[r] = z;
      const int cnt = base + (r < rem ? 1 : 0);
      for (int k = z; k < z + cnt; k++) owner[k] = (unsigned char)r;
      z += cnt;
    }
    z0s[NCTA] = z;
  }
  if (threadIdx.x < NCTA) slab[threadIdx.x] = cl.map_shared_rank(su, (int)threadIdx.x);
  __syncthreads();
  const int kz0 = z0s[rank], kz1 = z0s[rank + 1];
  double *gu = F.f[F_U] + B.off;
  const double *gb = F.f[F_B] + B.off, *gc = F.f[F_C] + B.off, *gs = F.f[F_RHO] + B.off;
  const double *gd = EQ ? F.f[F_D] + B.off : nullptr, *ge = EQ ? F.f[F_E] + B.off : nullptr;
  for (int p = threadIdx.x; p < (kz1 - kz0) * n01; p += blockDim.x) su[p] = gu[(long long)kz0 * n01 + p];
  cl.sync();

  auto U = [&](int i, int j, int k) -> double & {
    const int r = owner[k];
    return slab[r][(k - z0s[r]) * n01 + j * n0 + i];
  };
  const double *cx = crd + B.coord_off, *cy = cx + n0, *cz = cy + n1;
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
  // Newton update of one Robin point (Boundary_Face/Edge/Corner grouping)
  auto robin = [&](int mask, int i, int j, int k) {
    const double x = cx[i], y = cy[j], z = cz[k];
    const double r2 = x * x + y * y + z * z;
    const double xyz[3] = {x, y, z};
    double t = 0.0, dt = 0.0, tF = 0.0, dF = 0.0;
    int na = 0;
    for (int a = 0; a < 3; a++) {
      if (!(mask & (1 << a))) continue;
      double du;
      const double dv = d1(a, i, j, k, du);
      if (mask == (1 << a)) {
        tF = r2 * dv / xyz[a];
        dF = r2 * du / xyz[a] + 1.0;
      }
      t = na == 0 ? dv / xyz[a] : t + dv / xyz[a];
      dt = na == 0 ? du / xyz[a] : dt + du / xyz[a];
      na++;
    }
    if (na > 1) {
      tF = r2 * t;
      dF = r2 * dt + 1.0;
    }
    double &uu = U(i, j, k);
    const double Fv = tF + uu - gs[((long long)k * n1 + j) * n0 + i];
    uu = uu - Fv / dF;
  };

  double norm = 1.0, prev, first = -1.0;
  int it = 0;
  const int mi0 = n0 - 2, mi1 = n1 - 2;
  do {
    prev = norm;
    // faces
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
    cl.sync();
    // edges
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
    cl.sync();
    // corners
    for (int k = kz0; k < kz1; k++)
      if ((k == 0 || k == n2 - 1) && threadIdx.x < 4)
        robin(7, (threadIdx.x & 1) ? n0 - 1 : 0, (threadIdx.x & 2) ? n1 - 1 : 0, k);
    cl.sync();
    // one red-black SOR sweep over the interior points of this block's planes
    double rmax = 0.0, nan_seen = 0.0;
    const int ka = kz0 > 1 ? kz0 : 1, kb = kz1 < n2 - 1 ? kz1 : n2 - 1;
    const int H = (mi0 + 1) / 2;
    for (int color = 0; color < 2; color++) {
      for (int t = threadIdx.x; t < H * mi1 * (kb > ka ? kb - ka : 0); t += blockDim.x) {
        const int ih = t % H, r = t / H;
        const int j = 1 + r % mi1, k = ka + r / mi1;
        const int i = 1 + ((color + 1 + j + k) & 1) + 2 * ih;
        if (i >= n0 - 1) continue;
        const double c0 = U(i, j, k);
        const double lapv = (U(i + 1, j, k) - 2.0 * c0 + U(i - 1, j, k)) * B.idx2[0] +
                            (U(i, j + 1, k) - 2.0 * c0 + U(i, j - 1, k)) * B.idx2[1] +
                            (U(i, j, k + 1) - 2.0 * c0 + U(i, j, k - 1)) * B.idx2[2];
        const long long p = ((long long)k * n1 + j) * n0 + i;
        double op, dop;
        point_op<EQ>(lapv, B.dulap, c0, gb[p], gc[p], EQ ? gd[p] : 0.0, EQ ? ge[p] : 0.0, op, dop);
        const double R = op - gs[p];
        const double un = c0 - omega * (R * step_inverse(dop));
        U(i, j, k) = un;
        rmax = fmax(rmax, fabs(R));
        if (!(un == un)) nan_seen = 1.0;
      }
      cl.sync();
    }
    // cluster-wide max of the sweep norm and of the NaN flag
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
      nan_seen = fmax(nan_seen, __shfl_xor_sync(0xffffffffu, nan_seen, o));
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = rmax;
      red_nan[threadIdx.x >> 5] = nan_seen;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0, nn = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        m = fmax(m, red[w]);
        nn = fmax(nn, red_nan[w]);
      }
      s_part[0] = m;
      s_part[1] = nn;
    }
    cl.sync();
    if (threadIdx.x == 0) {
      double m = 0.0, nn = 0.0;
      for (int r = 0; r < NCTA; r++) {
        const double *pr = cl.map_shared_rank(s_part, r);
        m = fmax(m, pr[0]);
        nn = fmax(nn, pr[1]);
      }
      s_norm = m;
      s_stop = nn > 0.0;
      if (nn > 0.0 && rank == 0) atomicOr(nan_flag, 1);
    }
    __syncthreads();
    norm = s_norm;
    const int stop_nan = s_stop;
    it++;
    if (first < 0.0) first = norm;
    if (stop_nan) break;                           // the same decision in every block
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
