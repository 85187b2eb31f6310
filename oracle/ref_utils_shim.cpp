// Test infrastructure only: C entry points over the reference's own box and link-list code,
// compiled from the reference tree by oracle/ref_build.sh into oracle/_ref/libref_utils.so
// (with oracle/boost_shim standing in for the two Boost headers Utils.hpp includes). The
// geometry golden vectors (tests/golden/make_geometry_golden.py) come from these calls, and
// the oracle's restatement (ora_geom_* in oracle/cil_oracle.cpp) must equal them bit for bit.
//
// What is called, all from the reference's Utils.hpp: Nint (173-175), MDutils::BoundingBox::
// distance / updatePos (536-566), MDutils::LinkListOrtho2D/3D get_opt_size, init/reset,
// reset_list, populate_list, get_cells (get_cellCoord) and get_cellID (872-1069).
#include <cmath>
#include <cstdint>
#include <vector>
using std::isnan;  // Utils.hpp calls isnan unqualified
#include "Utils.hpp"

namespace {

MDutils::BoundingBox make_box(int dim, const double *box, const int32_t *pbc) {
  MDutils::BoundingBox b;
  double L[3] = {0.0, 0.0, 0.0};
  bool p[3] = {false, false, false};
  for (int d = 0; d < dim; ++d) {
    L[d] = box[d];
    p[d] = pbc[d] != 0;
  }
  b.init(dim, L, p);
  return b;
}

template <class LL>
int32_t link_list(LL &ll, int dim, double rcut, const double *box, const int32_t *pbc, int32_t n, const double *r,
                  int32_t *ns_out, int32_t *head, int32_t *list, int32_t *coords, int32_t *neighbor_ids,
                  int32_t max_bins) {
  int ns[3] = {1, 1, 1};
  ll.get_opt_size(ns, rcut, box);
  bool p[3] = {false, false, false};
  for (int d = 0; d < dim; ++d) p[d] = pbc[d] != 0;
  int nneigh = 0;
  const int ncells = ll.init(nneigh, ns, box, p);
  std::vector<int> ns_now;
  ll.get_ns(ns_now);
  for (int d = 0; d < 3; ++d) ns_out[d] = d < dim ? ns_now[d] : 1;
  if (ncells > max_bins) return -ncells;
  std::vector<int> hd(ncells), lk(n > 0 ? n : 1);
  ll.reset_list(hd.data(), lk.data(), n);
  ll.populate_list(const_cast<double *>(r), hd.data(), lk.data(), n, 0);
  for (int b = 0; b < ncells; ++b) head[b] = hd[b];
  for (int i = 0; i < n; ++i) list[i] = lk[i];
  std::vector<int> cell(static_cast<size_t>(ncells) * dim), shifts(static_cast<size_t>(nneigh) * dim);
  ll.get_cells(cell.data(), shifts.data());
  for (int b = 0; b < ncells; ++b) {
    for (int d = 0; d < dim; ++d) coords[b * dim + d] = cell[b * dim + d];
    for (int k = 0; k < nneigh; ++k) neighbor_ids[b * nneigh + k] = ll.get_cellID(&cell[b * dim], &shifts[k * dim]);
  }
  return ncells;
}

}  // namespace

extern "C" {

int32_t ref_nint(double a) { return Nint(a); }

void ref_box_distance(int32_t dim, const double *box, const int32_t *pbc, int64_t n, const double *r1,
                      const double *r2, double *r12, double *d2) {
  const MDutils::BoundingBox b = make_box(dim, box, pbc);
  for (int64_t i = 0; i < n; ++i) d2[i] = b.distance(r12 + i * dim, r1 + i * dim, r2 + i * dim);
}

// dt == 0: updatePos(r, dr) with v as dr; otherwise updatePos(r, v, dt)
void ref_box_update_pos(int32_t dim, const double *box, const int32_t *pbc, int64_t n, double *r, const double *v,
                        double dt) {
  const MDutils::BoundingBox b = make_box(dim, box, pbc);
  for (int64_t i = 0; i < n; ++i) {
    if (dt == 0.0)
      b.updatePos(r + i * dim, v + i * dim);
    else
      b.updatePos(r + i * dim, v + i * dim, dt);
  }
}

int32_t ref_link_list(int32_t dim, double rcut, const double *box, const int32_t *pbc, int32_t n, const double *r,
                      int32_t *ns, int32_t *head, int32_t *list, int32_t *coords, int32_t *neighbor_ids,
                      int32_t max_bins) {
  if (dim == 2) {
    MDutils::LinkListOrtho2D ll;
    return link_list(ll, 2, rcut, box, pbc, n, r, ns, head, list, coords, neighbor_ids, max_bins);
  }
  MDutils::LinkListOrtho3D ll;
  return link_list(ll, 3, rcut, box, pbc, n, r, ns, head, list, coords, neighbor_ids, max_bins);
}

}  // extern "C"
