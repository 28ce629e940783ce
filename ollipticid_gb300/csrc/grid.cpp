// grid.cpp -- nested-box hierarchy construction (host, one time per solve).
//
// Reference: WuShichao/OllipticID, src/elliptic.cc:299-921 (Set_Grids),
// src/domain.cc:26-525 (domain::Make, Set_N, Set_Boundary), 1492-1706
// (Get_i/j/k, Find_cell_xyz), 1810-2005 (operator+, operator&&),
// src/interface.cc:883-945 (Valid_N).  The floating-point steps are kept in
// the reference's order: the coordinates of the points decide which coarse
// and fine points coincide (3-epsilon absolute test), so a different rounding
// would change the discrete system.  Compile with -ffp-contract=off.
#include "grid.h"

#include <cfloat>
#include <cmath>
#include <cstddef>

namespace olgpu {

static const int kValidSizes[63] = {
    3,   4,   5,   6,   7,   8,   9,   10,  11,  12,  13,  14,  15,  17,  19,  21,
    23,  25,  27,  29,  33,  37,  41,  45,  49,  53,  57,  65,  73,  81,  89,  97,
    105, 113, 129, 145, 161, 177, 193, 209, 225, 257, 289, 321, 353, 385, 417, 449,
    513, 577, 641, 705, 769, 833, 897, 1153, 1281, 1409, 1665, 1793, 2305, 2817, 3329};

int valid_n(int n)
{
  for (int s : kValidSizes)
    if (s == n) return n;
  int below = kValidSizes[61], above = kValidSizes[62];
  for (int i = 0; i < 63 && kValidSizes[i] < n; i++) {
    below = kValidSizes[i];
    above = kValidSizes[i + 1 < 63 ? i + 1 : 62];
  }
  return (n - below < above - n) ? below : above;   // ties go up
}

domain domain::make(const int N[3], const double dx[3], const double cc[3], int ord)
{
  domain D;
  D.order = ord;
  D.buf = ord / 2 >= 1 ? ord / 2 : 1;
  for (int a = 0; a < 3; a++) {
    D.d[a] = dx[a];
    D.c[a] = cc[a];
    int npts = valid_n(N[a]);
    const double h = dx[a];
    // global extent with b-1 extra ghost layers per side (Set_N)
    const double g0 = cc[a] - 0.5 * (double)(npts - 1) * h - (double)(D.buf - 1) * h;
    npts += D.buf - 1;
    const double g1 = g0 + (double)(npts - 1) * h + (double)(D.buf - 1) * h;
    npts += D.buf - 1;
    D.glo[a] = g0;
    D.ghi[a] = g1;
    // single-rank Set_Boundary: re-derive both ends from the point count
    double t0 = g0, t1;
    while (t0 + (double)(npts - 1) * h > g1) npts--;
    if (t0 + (double)(npts - 1) * h < g1 - 0.5 * h) npts++;
    t1 = t0 + (double)(npts - 1) * h;
    while (t1 - (double)(npts - 1) * h < g0) npts--;
    if (t1 - (double)(npts - 1) * h > g0 + 0.5 * h) npts++;
    t0 = t1 - (double)(npts - 1) * h;
    D.lo[a] = t0;
    D.hi[a] = t1;
    D.n[a] = npts;
  }
  return D;
}

int domain::locate(int a, double x) const
{
  const int np = n[a];
  int lo_i = 0, hi_i = np;
  int i;
  if (lo[a] - x < 0.0 && x - hi[a] < 0.0) {
    i = np % 2 == 0 ? np / 2 : (np - 1) / 2;
    do {
      const double xi = lo[a] + (double)i * d[a];
      if (xi > x || dcomp(xi, x))
        hi_i = i;
      else
        lo_i = i;
      i = (hi_i + lo_i) / 2;
    } while (lo_i + 1 < hi_i);
  } else {
    i = (lo[a] >= x) ? 0 : np - 2;
  }
  return i + 1;
}

bool domain::is_in_axis(int a, double x) const
{
  return lo[a] - d[a] * 0.1 <= x && x <= hi[a] + d[a] * 0.1;
}

bool domain::is_in_nb_axis(int a, double x) const
{
  const double m = d[a] * ((double)buf - 0.1);
  return lo[a] + m < x && x < hi[a] - m;
}

bool domain::is_in(double x, double y, double z) const
{
  return is_in_axis(0, x) && is_in_axis(1, y) && is_in_axis(2, z);
}

bool domain::is_in_nb(double x, double y, double z) const
{
  return is_in_nb_axis(0, x) && is_in_nb_axis(1, y) && is_in_nb_axis(2, z);
}

// A && B: the (possibly empty) overlap of the extents lies inside B
bool domain::touches(const domain &B) const
{
  for (int a = 0; a < 3; a++) {
    const double s = lo[a] > B.lo[a] ? lo[a] : B.lo[a];
    const double e = B.hi[a] < hi[a] ? B.hi[a] : hi[a];
    const double p = s < e ? s : e, q = s < e ? e : s;
    if (!(B.lo[a] <= p && q <= B.hi[a])) return false;
  }
  return true;
}

domain domain::merge(const domain &A, const domain &B)
{
  int N[3];
  double cc[3];
  for (int a = 0; a < 3; a++) {
    const double g0 = A.glo[a] < B.glo[a] ? A.glo[a] : B.glo[a];
    const double g1 = A.ghi[a] < B.ghi[a] ? B.ghi[a] : A.ghi[a];
    cc[a] = 0.5 * (g0 + g1);
    N[a] = (int)(size_t)((g1 - g0) / A.d[a] + 1);
  }
  return make(N, A.d, cc, A.order);
}

bool set_grids(int N, double L, int order, int levels, const puncture_set &bh,
               hierarchy_geometry &out)
{
  const int n0 = valid_n(N);
  const double h0 = std::fabs(L) / (double)(n0 - 1.0);
  // multigrid coarse grids: n -> (n+1)/2 while >= 12 (full domain)
  std::vector<int> mg_n(1, n0);
  std::vector<double> mg_h(1, h0);
  for (;;) {
    const int nt = (mg_n.back() + 1) / 2;
    if (nt < 12) break;
    mg_n.push_back(nt);
    mg_h.push_back(mg_h.back() * 2.0);
  }
  if (mg_n.size() <= 1) return false;
  const int mg = (int)mg_n.size() - 1;
  const int total = levels + mg;
  std::vector<domain> D;
  std::vector<int> ndl(total, 0);
  const double origin[3] = {0, 0, 0};
  for (int l = mg; l >= 0; l--) {
    const int nn[3] = {mg_n[l], mg_n[l], mg_n[l]};
    const double hh[3] = {mg_h[l], mg_h[l], mg_h[l]};
    D.push_back(domain::make(nn, hh, origin, l == 0 ? order : 2));
    ndl[mg - l] = 1;
  }
  // one box of the base size per puncture and refinement level, centred on
  // the level's lattice point nearest the puncture (Find_cell_xyz walk)
  for (int l = mg + 1; l < total; l++) {
    for (int ib = 0; ib < bh.numbh; ib++) {
      const double hl = h0 / std::pow(2.0, (double)(l - mg));
      const double p[3] = {bh.x[ib], bh.y[ib], bh.z[ib]};
      double cc[3];
      const domain &base = D[mg];
      for (int a = 0; a < 3; a++) {
        const int i = base.locate(a, p[a]);
        double x0 = base.coord(a, i - 1), x1 = base.coord(a, i);
        if (dcomp(x0, p[a]) || dcomp(x1, p[a])) {
          cc[a] = p[a];
        } else {
          while (x0 + hl < p[a]) x0 += hl;
          while (x1 - hl > p[a]) x1 -= hl;
          cc[a] = std::fabs(x0 - p[a]) < std::fabs(x1 - p[a]) ? x0 : x1;
        }
      }
      const int nn[3] = {n0, n0, n0};
      const double hh[3] = {hl, hl, hl};
      D.push_back(domain::make(nn, hh, cc, order));
    }
    ndl[l] = bh.numbh;
  }
  // merge overlapping or touching boxes of a level and rescan the level
  for (int l = mg + 1; l < total; l++) {
    bool again = false;
    for (int i = 0; i < ndl[l]; i++)
      for (int j = 0; j < ndl[l]; j++) {
        if (i == j) continue;
        int base_idx = 0;
        for (int ll = 0; ll < l; ll++) base_idx += ndl[ll];
        const int bi = base_idx + i, bj = base_idx + j;
        if (D[bi].touches(D[bj])) {
          D[bi] = domain::merge(D[bi], D[bj]);
          D.erase(D.begin() + bj);
          ndl[l]--;
          again = true;
        }
      }
    if (again) l--;
  }
  out.boxes = D;
  out.boxes_in_level = ndl;
  out.levels = total;
  out.mgrid_levels = mg;
  out.first_box.assign(total, 0);
  for (int l = 1; l < total; l++) out.first_box[l] = out.first_box[l - 1] + ndl[l - 1];
  int g = 0;
  for (int l = 0; l < total; l++)
    for (int i = 0; i < ndl[l]; i++) out.boxes[g++].level = l;
  return true;
}

}  // namespace olgpu
