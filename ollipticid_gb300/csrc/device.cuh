// device.cuh -- data layout shared by the host driver and the kernels.
//
// Every field of every box lives in one device arena: field f of box g
// starts at arena + f * total_points + box[g].off and is stored
// lexicographically (i fastest) with the ghost layers included, so that a
// point's neighbours along x, y, z are at +-1, +-nx, +-nx*ny.
#pragma once

#include <cstdint>

namespace olgpu {

// F_T and F_UP are work fields of the device solver, not reference fields:
// F_T holds the full-weighted W, F_UP u as the current cycle found it (the
// cycle's largest change of u is measured against it).
enum Field { F_U = 0, F_B, F_C, F_D, F_E, F_RHO, F_R, F_W, F_WW, F_V, F_T, F_UP, F_NUM };

// boxes one launch covers: a level's boxes, or those of the same level of
// every solve of a batch
constexpr int kMaxBoxesPerLevel = 64;
constexpr int kMaxInterpPoints = 10;   // Lagrange order 9 (order 8 ghosts)

struct DevBox {
  int n[3];
  int buf;
  int order;
  int level;
  long long off;        // element offset inside each field arena
  int coord_off;        // offset of this box's x, y, z tables in coords[]
  int iso;              // the same spacing on every axis (1/dx^2 equal)
  double idx[3];        // 1/dx
  double idx2[3];       // 1/dx^2
  double dulap;         // diagonal of the Laplacian stencil
  double lscale;        // equal spacing, orders 2 and 4: the factor of the
                        // Laplacian's neighbour sum (1/dx^2, 1/(12 dx^2))
  int solve;            // the box's solve in a batch (0 alone): its norm slots
                        // are stats[solve]
  int active;           // 0: the box's solve has stopped; every kernel leaves it as it is
  int mg_coarse;        // 1: a multigrid coarse level (level < the solve's
                        // mgrid levels), whose ghost layers the discrete system
                        // does not fix
  int falloff;          // the Robin condition's falloff n (u ~ u_inf + C / r^n):
                        // 2 for the Bowen-York variables, else 1
  double d[3];          // spacing dx, dy, dz
};

struct DevFields {
  double *f[F_NUM];
};

// Boxes handled by one launch (indices into the box table); blocks are split
// between them by the prefix sums in blk.
struct BoxList {
  int count;
  int box[kMaxBoxesPerLevel];
  int blk[kMaxBoxesPerLevel + 1];
};

// Interpolation table entry for one target index along one axis.
struct AxisEntry {
  int sel;        // the target coordinate is inside the source (nb or all)
  int exact;      // coincides with source node `node` (3-epsilon test)
  int node;       // source node for the exact copy
  int start;      // first source index of the interpolation window
  int lo, hi;     // window terms [lo, hi] to sum: one term when the weights
                  // are exactly one-hot (then the sum equals that term bit for bit)
  int pad[2];
  double w[kMaxInterpPoints];
};

// XM_STRIDED: a job whose every target coincides with a source node that
// moves by a fixed step per target index (restriction and tau transfer at
// coinciding points, Set_In): a strided copy, found when the plan is built.
enum XferMethod { XM_LINEAR = 0, XM_LAGRANGE = 1, XM_COPY = 2, XM_STRIDED = 3 };
enum IterKind { IT_ALL = 0, IT_INSIDE = 1, IT_BOUNDARY = 2 };

// One (target box, source box, target sub-region) piece of a transfer.
struct XferJob {
  int tbox, sbox;
  int tfield, sfield;
  int method, ord, to_zero, iter;
  int r0[3], r1[3];     // visited target index box [r0, r1)
  int tab[3];           // AxisEntry offset of target index 0 on each axis
  long long blk0;       // first block of this job in the launch
  int row_axis;         // row kernel: rows run along x (0) or y (1)
  int pad_;
  long long rblk0;      // row kernel: first block of this job
  long long pblk0;      // pair kernel (two x-neighbour targets a thread): first block of this job
  int sstart[3], sstep[3];   // XM_STRIDED: source node of target r0 and its step
  // periodic linear jobs (lin2 = 1): along each axis the table entries of the
  // targets r0 + 2m + q are those of r0 + q with window start and node moved
  // by m; these are the entries of r0 and r0 + 1
  int lin2;
  int lstart[3][2], lnode[3][2], lexact[3][2];
  double lw0[3][2], lw1[3][2];
};

// Norm slots of a cycle beside the smoothers' (2 a level, pre/post): the
// cycle's largest change of u on the fixed points, the mixed cycle's largest
// correction and its finest FP64 defect.
constexpr int kSlotDu = 125, kSlotCorr = 126, kSlotDefect = 127;

// Device scalars of one solve, read back after each cycle (a batch holds one
// per solve, indexed by DevBox::solve).  Norms are kept as the bit patterns
// of non-negative doubles (atomicMax).
struct Stats {
  unsigned long long slots[128];    // smoother norms, 2 per level (pre/post), then kSlot*
  double coarse_norm;
  int coarse_iters;
  int nan_flag;
  double adm_u[16];
};

struct PunctureParams {
  int numbh;
  int equation;
  int ps_case;
  int var;              // Bowen-York: the variable k_test_init sets up (0..2 V1..V3, 3 lambda)
  double mp[16], x[16], y[16], z[16];
  double px[16], py[16], pz[16], sx[16], sy[16], sz[16];
  double ps_phi0, ps_r0, ps_isigma, ps_d1, ps_e1, ps_e2, ps_de1;
};

}  // namespace olgpu
