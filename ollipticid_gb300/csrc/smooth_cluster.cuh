// smooth_cluster.cuh -- every sweep of the FP32 correction smoother of one
// level in one launch.
//
// One thread-block cluster per box.  The box's correction e (ghosts
// included) is split into z-slabs, one per block, and stays in the blocks'
// shared memory for all sweeps: x/y neighbours are read from the block's own
// slab, z neighbours through a per-plane pointer table that maps every plane
// of the box to its owner's shared memory (distributed shared memory for the
// planes of other blocks).  The colours of a sweep are separated by cluster
// barriers, so a sweep costs no kernel launch and no HBM round trip of e; the
// read-only coefficients (A, 1/(c+u), source) come from L2.  The update of a
// point is the same explicitly rounded expression as in k_smooth32 (lapf_acc,
// corr_op, corr_update), so the result equals the per-colour launches' bit
// for bit.
//
// The interior planes are split evenly (the ghost planes, which are read but
// not updated, go with the first and the last block), so every block has the
// same share of updates between two barriers.  The cluster size is a launch
// parameter (8..16 blocks).  One 512-thread block per SM: held to 64
// registers so that two fit, the kernel moved 5 % more bytes with 16 solves
// sharing the GPU but a solve alone held half the SMs, and 16 copies of the
// benchmark binary ran 4 % slower (71.7 against 75.1 solves/s).
#pragma once

#include "mixed.cuh"

#include <cooperative_groups.h>

namespace olgpu {

constexpr int kSmoothClusterThreads = 512;
constexpr int kMaxClusterPlanes = 160;

// First plane of block r of a cluster of ncta blocks over a box of n2 planes
// with b ghost planes on each side: the n2 - 2b interior planes are dealt out
// evenly (the first (n2 - 2b) % ncta blocks take one more), block 0 also
// holds the low ghost planes and block ncta-1 the high ones.
__host__ __device__ inline int slab_begin(int r, int n2, int b, int ncta)
{
  if (r <= 0) return 0;
  if (r >= ncta) return n2;
  const int m2 = n2 - 2 * b, base = m2 / ncta, rem = m2 % ncta;
  return b + r * base + (r < rem ? r : rem);
}

// Planes of the largest slab (the shared memory a block needs, in planes).
__host__ __device__ inline int slab_max_planes(int n2, int b, int ncta)
{
  int m = 0;
  for (int r = 0; r < ncta; r++) {
    const int p = slab_begin(r + 1, n2, b, ncta) - slab_begin(r, n2, b, ncta);
    m = p > m ? p : m;
  }
  return m;
}

template <int ORD, int EQ>
__global__ void __launch_bounds__(kSmoothClusterThreads, 1)
    k_smooth32_cluster(const DevBox *__restrict__ boxes, BoxList L, DevFields32 G, const float2 *__restrict__ aq,
                       int sweeps, Stats *stats)
{
  namespace cg = cooperative_groups;
  constexpr int NC = num_colors<ORD>();
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), ncta = (int)cl.num_blocks();
  extern __shared__ float4 s_slab4[];
  float *se = reinterpret_cast<float *>(s_slab4);
  __shared__ const float *plane[kMaxClusterPlanes];

  if ((int)blockIdx.x / ncta >= L.count) return;   // the whole cluster: one box a cluster
  const DevBox B = boxes[L.box[(int)blockIdx.x / ncta]];
  if (!B.active) return;   // every block of the cluster reads the same box: all leave
  int *nan_flag = &stats[B.solve].nan_flag;
  const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2], b = B.buf;
  const int n01 = n0 * n1;
  const int z0 = slab_begin(rank, n2, b, ncta), z1 = slab_begin(rank + 1, n2, b, ncta);
  for (int k = threadIdx.x; k < n2; k += blockDim.x) {
    int r = 0;
    while (slab_begin(r + 1, n2, b, ncta) <= k) r++;
    plane[k] = cl.map_shared_rank(se, r) + (k - slab_begin(r, n2, b, ncta)) * n01;
  }
  float *ge = G.f[G_E] + B.off;
  const int slab = (z1 - z0) * n01;
  for (int p = threadIdx.x; p < slab; p += blockDim.x) se[p] = ge[z0 * n01 + p];
  cl.sync();

  const float ix2 = (float)B.idx2[0], iy2 = (float)B.idx2[1], iz2 = (float)B.idx2[2];
  const float dl = (float)B.dulap;
  const float *gs = G.f[G_S] + B.off;
  const float2 *gaq = aq + B.off;   // (A, 1/(c+u)) colour-packed (packed_index)
  const float *gd = EQ == 1 ? G.f[G_D] + B.off : nullptr, *ge5 = EQ == 1 ? G.f[G_E5] + B.off : nullptr;
  const int m0 = n0 - 2 * b, m1 = n1 - 2 * b, m2 = n2 - 2 * b;
  const int ka = z0 > b ? z0 : b, kb = z1 < n2 - b ? z1 : n2 - b;
  const int nk = kb > ka ? kb - ka : 0;
  const int H = (m0 + NC - 1) / NC;
  const int total = H * m1 * nk;
  // A thread's points are t = threadIdx.x + u * blockDim.x: their (ih, row,
  // plane) coordinates advance by the decomposed stride with one carry each,
  // so the sweep loop has no integer division.  U points are updated per
  // step, all loads first and then all stores (points of one colour do not
  // read each other); a point past the end reads the slab's first interior
  // point instead and is not stored, so the loads need no branch.
  constexpr int U = 4;
  const int S = blockDim.x;
  const int s_ih = S % H, s_j = (S / H) % m1, s_k = S / (H * m1);
  const int t0 = threadIdx.x;
  const int ih0 = t0 % H, j0 = (t0 / H) % m1, k0 = t0 / (H * m1);
  int nan_seen = 0;
  for (int s = 0; s < sweeps; s++) {
    for (int color = 0; color < NC; color++) {
      int ih = ih0, jr = j0, kr = k0;
      for (int t = t0; t < total; t += U * S) {
        float en[U];
        int qq[U], kk[U];
        int pk[U];   // the point's colour-packed position
        bool ok[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int j = b + jr, k = ka + kr;
          const int delta = (((color - b - j - k) % NC) + NC) % NC;
          const int i = b + delta + NC * ih;
          ok[u] = t + u * S < total && i < n0 - b;
          kk[u] = ok[u] ? k : ka;
          qq[u] = ok[u] ? j * n0 + i : b * n0 + b;
          pk[u] = ok[u] ? ((color * m2 + (k - b)) * m1 + jr) * H + ih : 0;
          ih += s_ih;
          jr += s_j;
          kr += s_k;
          if (ih >= H) {
            ih -= H;
            jr++;
          }
          if (jr >= m1) {
            jr -= m1;
            kr++;
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int q = qq[u], k = kk[u];
          const float *pl = se + (k - z0) * n01;
          const float c = pl[q];
          const float lv = lapf_acc<ORD>(
              c, [&](int a, int d) -> float { return a == 0 ? pl[q + d] : a == 1 ? pl[q + d * n0] : plane[k + d][q]; },
              ix2, iy2, iz2);
          const int p = k * n01 + q;
          float op, dop;
          const float2 aqv = __ldg(gaq + pk[u]);
          corr_op<EQ>(lv, dl, c, aqv.x, aqv.y, EQ == 1 ? __ldg(gd + p) : 0.0f, EQ == 1 ? __ldg(ge5 + p) : 0.0f,
                      op, dop);
          en[u] = corr_update(c, op, dop, __ldg(gs + p));
        }
#pragma unroll
        for (int u = 0; u < U; u++)
          if (ok[u]) {
            se[(kk[u] - z0) * n01 + qq[u]] = en[u];
            if (!(en[u] == en[u])) nan_seen = 1;
          }
      }
      cl.sync();
    }
  }
  for (int p = threadIdx.x; p < slab; p += blockDim.x) ge[z0 * n01 + p] = se[p];
  if (nan_seen) atomicOr(nan_flag, 1);
}

}  // namespace olgpu
