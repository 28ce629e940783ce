// grid.h -- host-side geometry of the nested-box hierarchy.
//
// The device solver needs the exact same boxes, coordinates and point
// classifications as the reference, because injection, Lagrange windows and
// the tau masks all depend on floating-point coordinate tests.  This header
// keeps the reference's `domain` vocabulary (include/domain.h) for the parts
// of the class the hot path uses; storage on the device is plain
// lexicographic, so the permuted index tables of domain::Fix_Points are not
// reproduced.
#pragma once

#include <cfloat>
#include <cmath>
#include <vector>

namespace olgpu {

int valid_n(int n);   // interface.cc Valid_N: snap to the allowed sizes

struct domain {
  int n[3] = {0, 0, 0};     // points per axis, ghosts included
  int buf = 1;              // ghost width max(order/2, 1)
  int order = 2;
  int level = 0;
  double d[3] = {0, 0, 0};  // spacing
  double c[3] = {0, 0, 0};  // centre
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};    // xi..xf (one rank)
  double glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};  // gxi..gxf

  static domain make(const int N[3], const double dx[3], const double cc[3], int ord);

  double coord(int a, int i) const { return lo[a] + (double)i * d[a]; }
  long npts() const { return (long)n[0] * n[1] * n[2]; }
  // Get_i / Get_j / Get_k: first node at or after x (binary search)
  int locate(int a, double x) const;
  bool is_in_axis(int a, double x) const;      // Is_In along one axis
  bool is_in_nb_axis(int a, double x) const;   // is_in_nb along one axis
  bool is_in(double x, double y, double z) const;
  bool is_in_nb(double x, double y, double z) const;
  bool touches(const domain &other) const;     // *this && other
  static domain merge(const domain &A, const domain &B);   // A + B
};

// 3-epsilon absolute coordinate comparison (include/domain.h:871-875)
inline bool dcomp(double x, double y) { return std::fabs(x - y) <= 3 * DBL_EPSILON; }

struct hierarchy_geometry {
  std::vector<domain> boxes;        // level-major, as the reference orders them
  std::vector<int> boxes_in_level;  // num_dom_in_level
  std::vector<int> first_box;       // index of the first box of each level
  int levels = 0;                   // total, multigrid coarse grids included
  int mgrid_levels = 0;
};

struct puncture_set {
  int numbh = 0;
  const double *x = nullptr, *y = nullptr, *z = nullptr;
};

// elliptic::Set_Grids for a full (no symmetry) cubic domain.  Returns false
// when there are too few points for a multigrid coarse grid.
bool set_grids(int N, double L, int order, int levels, const puncture_set &bh,
               hierarchy_geometry &out);

}  // namespace olgpu
