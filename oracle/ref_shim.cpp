// extern "C" shim over LLNL/axom's own SEQ spatial-query path.
//
// Test infrastructure only: compiled by oracle/build_ref.py against the
// reference sources into oracle/_ref/libaxom_ref.so, and used by the CPU test
// suite to pin the CPU restatement (oracle/gsq_oracle.cpp) and to generate the
// golden fixtures in tests/golden/.  Every entry point calls the reference's
// public API (or, for the internals export, its namespace-level build steps):
//   spin::BVH<3,SEQ_EXEC,double>::initialize / findBoundingBoxes / findPoints /
//     findRays / getBounds / getTraverser      (src/axom/spin/BVH.hpp:129-568)
//   spin::internal::linear_bvh::build_radix_tree
//     (src/axom/spin/internal/linear_bvh/build_radix_tree.hpp:579-611)
//   quest::SignedDistance<3,SEQ_EXEC> ctor / computeDistances
//     (src/axom/quest/SignedDistance.hpp:410-605)
#include "axom/config.hpp"
#include "axom/core.hpp"
#include "axom/slic.hpp"
#include "axom/primal/operators/closest_point.hpp"
#include "axom/primal/operators/squared_distance.hpp"
#include "axom/mint/mesh/UnstructuredMesh.hpp"
#include "axom/spin/BVH.hpp"
#include "axom/spin/internal/linear_bvh/build_radix_tree.hpp"
#include "axom/quest/SignedDistance.hpp"
#include "axom/quest/readers/STLReader.hpp"

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace
{
using BoxType = axom::primal::BoundingBox<double, 3>;
using PointType = axom::primal::Point<double, 3>;
using VectorType = axom::primal::Vector<double, 3>;
using RayType = axom::primal::Ray<double, 3>;
using TriType = axom::primal::Triangle<double, 3>;
using BVHType = axom::spin::BVH<3, axom::SEQ_EXEC, double>;
using UMesh = axom::mint::UnstructuredMesh<axom::mint::SINGLE_SHAPE>;
using SDType = axom::quest::SignedDistance<3, axom::SEQ_EXEC>;

static_assert(sizeof(PointType) == 3 * sizeof(double), "Point<double,3> must be 3 packed doubles");
static_assert(sizeof(VectorType) == 3 * sizeof(double), "Vector<double,3> must be 3 packed doubles");

void ensure_logger()
{
  static bool init = false;
  if(!init)
  {
    axom::slic::initialize();
    axom::slic::setLoggingMsgLevel(axom::slic::message::Error);
    init = true;
  }
}

std::vector<BoxType> to_boxes(const double* b, int n)
{
  std::vector<BoxType> out;
  out.reserve(n);
  for(int i = 0; i < n; ++i)
  {
    // Construct without fixing bounds so that invalid boxes stay invalid,
    // exactly as a caller-built BoundingBox{min,max,false} would.
    out.emplace_back(PointType {b[6 * i + 0], b[6 * i + 1], b[6 * i + 2]},
                     PointType {b[6 * i + 3], b[6 * i + 4], b[6 * i + 5]},
                     false);
  }
  return out;
}

void put_box(const BoxType& bb, double* dst)
{
  for(int d = 0; d < 3; ++d)
  {
    dst[d] = bb.getMin()[d];
    dst[3 + d] = bb.getMax()[d];
  }
}

long long copy_candidates(const axom::Array<axom::IndexType>& c, int** out)
{
  const long long total = c.size();
  *out = static_cast<int*>(std::malloc(sizeof(int) * (total > 0 ? total : 1)));
  for(long long i = 0; i < total; ++i) (*out)[i] = c[i];
  return total;
}

struct SDHandle
{
  std::vector<double> x, y, z;
  std::vector<axom::IndexType> conn;
  UMesh* mesh {nullptr};
  SDType* sd {nullptr};
};
}  // namespace

extern "C" {

void ref_free(void* p) { std::free(p); }

// ---- spin::BVH -----------------------------------------------------------
void* ref_bvh_create(const double* boxes, int n, double scale)
{
  ensure_logger();
  auto* bvh = new BVHType();
  bvh->setScaleFactor(scale);
  std::vector<BoxType> bx = to_boxes(boxes, n);
  bvh->initialize(bx.data(), n);
  return bvh;
}

void ref_bvh_destroy(void* h) { delete static_cast<BVHType*>(h); }

void ref_bvh_bounds(void* h, double* out6) { put_box(static_cast<BVHType*>(h)->getBounds(), out6); }

long long ref_bvh_find_boxes(void* h, const double* q, int m, int* offsets, int* counts, int** cands)
{
  auto* bvh = static_cast<BVHType*>(h);
  std::vector<BoxType> qb = to_boxes(q, m);
  axom::ArrayView<axom::IndexType> off(offsets, m), cnt(counts, m);
  axom::Array<axom::IndexType> c;
  bvh->findBoundingBoxes(off, cnt, c, m, qb.data());
  return copy_candidates(c, cands);
}

// Instrumented findBoundingBoxes: per query, the number of box-predicate
// calls the BVH's own traverser makes (its generic, no-preference overload,
// spin/policy/LinearBVH.hpp:91-103, as findBoundingBoxes uses).
void ref_bvh_find_boxes_counts(void* h, const double* q, int m, int* box_tests)
{
  auto* bvh = static_cast<BVHType*>(h);
  auto it = bvh->getTraverser();
  std::vector<BoxType> qb = to_boxes(q, m);
  for(int i = 0; i < m; ++i)
  {
    int nb = 0;
    auto leaf = [](std::int32_t, const std::int32_t*) {};
    auto pred = [&](const BoxType& query, const BoxType& bb) -> bool {
      ++nb;
      return query.intersectsWith(bb);
    };
    it.traverse_tree(qb[i], leaf, pred);
    box_tests[i] = nb;
  }
}

long long ref_bvh_find_points(void* h, const double* p, int m, int* offsets, int* counts, int** cands)
{
  auto* bvh = static_cast<BVHType*>(h);
  const PointType* pts = reinterpret_cast<const PointType*>(p);
  axom::ArrayView<axom::IndexType> off(offsets, m), cnt(counts, m);
  axom::Array<axom::IndexType> c;
  bvh->findPoints(off, cnt, c, m, pts);
  return copy_candidates(c, cands);
}

// Rays are built with primal::Ray(origin, direction), which normalises the
// direction; the normalised directions are written to dir_out (nullable).
long long ref_bvh_find_rays(void* h,
                            const double* o,
                            const double* d,
                            int m,
                            int* offsets,
                            int* counts,
                            int** cands,
                            double* dir_out)
{
  auto* bvh = static_cast<BVHType*>(h);
  std::vector<RayType> rays;
  rays.reserve(m);
  for(int i = 0; i < m; ++i)
  {
    rays.emplace_back(PointType {o[3 * i], o[3 * i + 1], o[3 * i + 2]},
                      VectorType {d[3 * i], d[3 * i + 1], d[3 * i + 2]});
    if(dir_out)
      for(int k = 0; k < 3; ++k) dir_out[3 * i + k] = rays.back().direction()[k];
  }
  axom::ArrayView<axom::IndexType> off(offsets, m), cnt(counts, m);
  axom::Array<axom::IndexType> c;
  bvh->findRays(off, cnt, c, m, rays.data());
  return copy_candidates(c, cands);
}

// Re-runs the reference build steps (transform, reduce, Morton, stable sort,
// reorder, Karras tree, refit) on n >= 2 boxes and exports the RadixTree.
//   codes[n]        sorted Morton codes        perm[n]     sorted -> original id
//   lchild/rchild[n-1] children (>= n-1 means leaf n-1+k)   parents[2n-1]
//   inner[(n-1)*6]  inner node boxes            leaf[n*6]   sorted scaled leaf boxes
//   bounds[6]       global bounds of the scaled boxes
int ref_bvh_internals(const double* boxes,
                      int n,
                      double scale,
                      std::uint32_t* codes,
                      int* perm,
                      int* lchild,
                      int* rchild,
                      int* parents,
                      double* inner,
                      double* leaf,
                      double* bounds)
{
  ensure_logger();
  if(n < 2) return -1;
  namespace lbvh = axom::spin::internal::linear_bvh;
  std::vector<BoxType> bx = to_boxes(boxes, n);
  lbvh::RadixTree<double, 3> tree;
  BoxType gb;
  const int alloc = axom::execution_space<axom::SEQ_EXEC>::allocatorID();
  lbvh::build_radix_tree<axom::SEQ_EXEC>(bx.data(), n, gb, tree, scale, alloc);
  for(int i = 0; i < n; ++i)
  {
    codes[i] = tree.m_mcodes[i];
    perm[i] = tree.m_leafs[i];
    put_box(tree.m_leaf_aabbs[i], leaf + 6 * i);
  }
  for(int i = 0; i < n - 1; ++i)
  {
    lchild[i] = tree.m_left_children[i];
    rchild[i] = tree.m_right_children[i];
    put_box(tree.m_inner_aabbs[i], inner + 6 * i);
  }
  for(int i = 0; i < 2 * n - 1; ++i) parents[i] = tree.m_parents[i];
  put_box(gb, bounds);
  return 0;
}

// ---- quest::SignedDistance ---------------------------------------------
void* ref_sdf_create(const double* x,
                     const double* y,
                     const double* z,
                     int nverts,
                     const int* cells,
                     int ncells,
                     int nodes_per_cell,
                     int watertight,
                     int compute_sign)
{
  ensure_logger();
  auto* h = new SDHandle();
  h->x.assign(x, x + nverts);
  h->y.assign(y, y + nverts);
  h->z.assign(z, z + nverts);
  h->conn.assign(cells, cells + (long long)nodes_per_cell * ncells);
  h->mesh = new UMesh(nodes_per_cell == 4 ? axom::mint::QUAD : axom::mint::TRIANGLE,
                      ncells,
                      h->conn.data(),
                      nverts,
                      h->x.data(),
                      h->y.data(),
                      h->z.data());
  h->sd = new SDType(h->mesh, watertight != 0, compute_sign != 0);
  return h;
}

void ref_sdf_destroy(void* hv)
{
  auto* h = static_cast<SDHandle*>(hv);
  delete h->sd;
  delete h->mesh;
  delete h;
}

// q, cp, normals are AoS (m x 3).  cp / normals nullable.  The const
// computeDistances is called on contiguous sub-ranges from nthreads threads.
void ref_sdf_eval(void* hv, const double* q, int m, double* out, double* cp, double* normals, int nthreads)
{
  auto* h = static_cast<SDHandle*>(hv);
  const PointType* pts = reinterpret_cast<const PointType*>(q);
  PointType* cps = reinterpret_cast<PointType*>(cp);
  VectorType* nrm = reinterpret_cast<VectorType*>(normals);
  if(nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
  {
    int t = 0, nt = 1;
#ifdef _OPENMP
    t = omp_get_thread_num();
    nt = omp_get_num_threads();
#endif
    const long long lo = (long long)m * t / nt, hi = (long long)m * (t + 1) / nt;
    if(hi > lo)
      h->sd->computeDistances(int(hi - lo),
                              pts + lo,
                              out + lo,
                              cps ? cps + lo : nullptr,
                              nrm ? nrm + lo : nullptr);
  }
}

// Instrumented traversal: per query, the number of box-predicate calls and
// leaf (triangle) tests made by the SignedDistance traversal, using the BVH's
// own traverser with the SignedDistance predicate and minimum update.
void ref_sdf_counts(void* hv, const double* q, int m, int* box_tests, int* leaf_tests, int nthreads)
{
  auto* h = static_cast<SDHandle*>(hv);
  auto it = h->sd->getBVHTree().getTraverser();
  if(nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
  for(int i = 0; i < m; ++i)
  {
    PointType qpt {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    double minSq = axom::numerics::floating_point_limits<double>::max();
    int nb = 0, nl = 0;
    auto leaf = [&](std::int32_t node, const std::int32_t* leaves) {
      const int c = leaves[node];
      const axom::IndexType* t = &h->conn[3 * (long long)c];
      TriType tri {PointType {h->x[t[0]], h->y[t[0]], h->z[t[0]]},
                   PointType {h->x[t[1]], h->y[t[1]], h->z[t[1]]},
                   PointType {h->x[t[2]], h->y[t[2]], h->z[t[2]]}};
      int loc;
      PointType cpt = axom::primal::closest_point(qpt, tri, &loc, 1e-12);
      const double sq = axom::primal::squared_distance(qpt, cpt);
      if(sq < minSq) minSq = sq;
      ++nl;
    };
    auto pred = [&](const PointType& p, const BoxType& bb) -> bool {
      ++nb;
      return axom::primal::squared_distance(p, bb) <= minSq;
    };
    it.traverse_tree(qpt, leaf, pred);
    box_tests[i] = nb;
    leaf_tests[i] = nl;
  }
}

void ref_sdf_mesh_bounds(void* hv, double* out6)
{
  // SignedDistance keeps the mesh box private; rebuild it the way setMesh's
  // SEQ branch does (BoundingBox::addPoint over the nodes, SD:483-486).
  auto* h = static_cast<SDHandle*>(hv);
  BoxType bb;
  for(size_t i = 0; i < h->x.size(); ++i) bb.addPoint(PointType {h->x[i], h->y[i], h->z[i]});
  put_box(bb, out6);
}

// ---- quest::STLReader (quest/readers/STLReader.cpp) --------------------------
// Reads the file and copies the mesh STLReader::getMesh builds: coordinates
// (AoS, 3 per node) and connectivity (3 per triangle).  Returns the number of
// triangles, or -1 if read() failed; the arrays are malloc'd (ref_free).
int ref_stl_read(const char* path, double** xyz, int* nnodes, int** conn)
{
  ensure_logger();
  axom::quest::STLReader reader;
  reader.setFileName(path);
  if(reader.read() != 0) return -1;
  UMesh mesh(3, axom::mint::TRIANGLE);
  reader.getMesh(&mesh);
  const int nn = (int)mesh.getNumberOfNodes(), nc = (int)mesh.getNumberOfCells();
  *nnodes = nn;
  *xyz = static_cast<double*>(std::malloc(sizeof(double) * 3 * std::max(nn, 1)));
  *conn = static_cast<int*>(std::malloc(sizeof(int) * 3 * std::max(nc, 1)));
  const double* x = mesh.getCoordinateArray(axom::mint::X_COORDINATE);
  const double* y = mesh.getCoordinateArray(axom::mint::Y_COORDINATE);
  const double* z = mesh.getCoordinateArray(axom::mint::Z_COORDINATE);
  for(int i = 0; i < nn; ++i)
  {
    (*xyz)[3 * i] = x[i];
    (*xyz)[3 * i + 1] = y[i];
    (*xyz)[3 * i + 2] = z[i];
  }
  const axom::IndexType* c = mesh.getCellNodesArray();
  for(int i = 0; i < 3 * nc; ++i) (*conn)[i] = (int)c[i];
  return nc;
}

// ---- the local closest-point query of quest::DistributedClosestPoint --------
// DistributedClosestPoint itself needs MPI and conduit; its local step
// (computeLocalClosestPoints, quest/detail/DistributedClosestPointImpl.hpp:
// 883-901 and 1002-1050) is a BVH over one degenerate box per object point
// and a traverse_tree call per query point.  This drives the reference's own
// BVH and traverser with a leaf action and predicate that behave as that
// step's (no earlier rank's candidate).
struct CPHandle
{
  BVHType bvh;
  std::vector<PointType> pts;
  std::vector<int> dom;
};

void* ref_cp_create(const double* p, int n, const int* domains)
{
  ensure_logger();
  auto* h = new CPHandle();
  h->pts.resize(n);
  h->dom.resize(n);
  std::vector<BoxType> boxes(n);
  for(int i = 0; i < n; ++i)
  {
    h->pts[i] = PointType {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
    h->dom[i] = domains ? domains[i] : 0;
    boxes[i] = BoxType {h->pts[i]};
  }
  h->bvh.initialize(boxes.data(), n);
  return h;
}

void ref_cp_destroy(void* h) { delete static_cast<CPHandle*>(h); }

void ref_cp_query(void* hv, const double* q, int m, double sq_threshold, int* idx, int* dom, double* pos, double* dist,
                  int nthreads)
{
  auto* h = static_cast<CPHandle*>(hv);
  auto it = h->bvh.getTraverser();
  const double nan = std::numeric_limits<double>::quiet_NaN();
  if(nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
  for(int i = 0; i < m; ++i)
  {
    PointType qpt {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    double best = axom::numerics::floating_point_limits<double>::max();
    int bi = -1, bd = -1;
    auto leaf = [&](std::int32_t node, const std::int32_t* leaves) {
      const int c = leaves[node];
      const double sq = axom::primal::squared_distance(qpt, h->pts[c]);
      if(sq < best)
      {
        best = sq;
        bi = c;
        bd = h->dom[c];
      }
    };
    auto pred = [&](const PointType& pt, const BoxType& bb) -> bool {
      const double sq = axom::primal::squared_distance(pt, bb);
      return sq <= best && sq <= sq_threshold;
    };
    if(!h->pts.empty()) it.traverse_tree(qpt, leaf, pred);
    idx[i] = bi;
    dom[i] = bd;
    for(int d = 0; d < 3; ++d) pos[3 * i + d] = (bi >= 0) ? h->pts[bi][d] : nan;
    dist[i] = (bi >= 0) ? std::sqrt(best) : nan;
  }
}

}  // extern "C"
