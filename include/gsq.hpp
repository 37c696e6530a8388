// gsq.hpp -- header-only C++ mirror of axom's spin::BVH and
// quest::SignedDistance over the C ABI in gsq.h.
//
// A caller of the reference switches by changing the namespace:
//   axom::spin::BVH<3, axom::CUDA_EXEC<256>, double>   -> gsq::spin::BVH<3, double>
//   axom::quest::SignedDistance<3, axom::CUDA_EXEC<>>  -> gsq::quest::SignedDistance<3>
// Method names, argument meaning and the candidate (offsets, counts,
// candidates) convention follow spin/BVH.hpp:129-568 and
// quest/SignedDistance.hpp:147-605.  Where the reference aborts through
// SLIC_ERROR, these methods throw gsq::Error.
#ifndef GSQ_HPP_
#define GSQ_HPP_

#include <cfloat>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gsq.h"
#include "gsq_quest.h"

namespace gsq
{
struct Error : std::runtime_error
{
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) { }
};

inline void check(int rc)
{
  if(rc != GSQ_OK) throw Error(rc, gsq_last_error());
}

// primal::BoundingBox<double,3> / Point / Ray layouts (6, 3, 3+3 doubles).
struct BoundingBox
{
  double min[3], max[3];
};
struct Point
{
  double x[3];
};
struct Ray
{
  double origin[3];
  double direction[3];  // stored normalised, as primal::Ray does (Ray.hpp:123-128)
  Ray() = default;
  Ray(const Point& o, const double* d)
  {
    for(int k = 0; k < 3; ++k) origin[k] = o.x[k];
    check(gsq_ray_normalize(d, 1, direction));
  }
};

// Candidate arrays as findPoints / findRays / findBoundingBoxes return them.
struct Candidates
{
  std::vector<int32_t> offsets, counts, candidates;
};

namespace spin
{
constexpr int BVH_BUILD_OK = 0;
constexpr int BVH_BUILD_FAILED = -1;

template <int NDIMS, typename FloatType = double>
class BVH
{
  static_assert(NDIMS == 3, "gsq implements the 3D BVH");
  static_assert(sizeof(FloatType) == 8, "gsq implements the double-precision BVH");

public:
  BVH() { check(gsq_bvh_create(&m_h)); }
  BVH(const BoundingBox* boxes, int32_t n) : BVH() { initialize(boxes, n); }
  ~BVH()
  {
    if(m_owned) gsq_bvh_destroy(m_h);
  }
  BVH(const BVH&) = delete;
  BVH& operator=(const BVH&) = delete;

  // BVH::initialize (spin/BVH.hpp:424-477)
  int initialize(const BoundingBox* boxes, int32_t n, void* stream = nullptr)
  {
    return gsq_bvh_build(m_h, reinterpret_cast<const double*>(boxes), n, stream) == GSQ_OK ? BVH_BUILD_OK
                                                                                             : BVH_BUILD_FAILED;
  }
  void setScaleFactor(double s) { check(gsq_bvh_set_scale_factor(m_h, s)); }
  double getScaleFactor() const
  {
    double s;
    check(gsq_bvh_get_scale_factor(m_h, &s));
    return s;
  }
  void setTolerance(double t) { check(gsq_bvh_set_tolerance(m_h, t)); }
  double getTolerance() const
  {
    double t;
    check(gsq_bvh_get_tolerance(m_h, &t));
    return t;
  }
  BoundingBox getBounds() const
  {
    BoundingBox b;
    check(gsq_bvh_bounds(m_h, b.min, b.max));
    return b;
  }

  // Host-array forms of findPoints / findRays / findBoundingBoxes
  // (spin/BVH.hpp:480-568).
  void findPoints(Candidates& c, int32_t n, const Point* pts) const
  {
    find(c, n, [&](int32_t* off, int32_t* cnt, int32_t** cand, int64_t* tot) {
      return gsq_bvh_find_points(m_h, reinterpret_cast<const double*>(pts), n, off, cnt, cand, tot, nullptr);
    });
  }
  void findBoundingBoxes(Candidates& c, int32_t n, const BoundingBox* boxes) const
  {
    find(c, n, [&](int32_t* off, int32_t* cnt, int32_t** cand, int64_t* tot) {
      return gsq_bvh_find_boxes(m_h, reinterpret_cast<const double*>(boxes), n, off, cnt, cand, tot, nullptr);
    });
  }
  void findRays(Candidates& c, int32_t n, const Ray* rays) const
  {
    std::vector<double> o(3 * (size_t)n), d(3 * (size_t)n);
    for(int32_t i = 0; i < n; ++i)
      for(int k = 0; k < 3; ++k)
      {
        o[3 * i + k] = rays[i].origin[k];
        d[3 * i + k] = rays[i].direction[k];
      }
    find(c, n, [&](int32_t* off, int32_t* cnt, int32_t** cand, int64_t* tot) {
      return gsq_bvh_find_rays(m_h, o.data(), d.data(), n, off, cnt, cand, tot, nullptr);
    });
  }

  // Device-array form: offsets/counts and the query array in device memory;
  // *candidates is a device allocation released with gsq_free.
  int findPointsDevice(int32_t* offsets, int32_t* counts, int32_t** candidates, int32_t n, const double* pts,
                       void* stream = nullptr) const
  {
    int64_t total = 0;
    return gsq_bvh_find_points(m_h, pts, n, offsets, counts, candidates, &total, stream);
  }

  const gsq_bvh* handle() const { return m_h; }
  static BVH borrowed(const gsq_bvh* h) { return BVH(const_cast<gsq_bvh*>(h), false); }

private:
  BVH(gsq_bvh* h, bool owned) : m_h(h), m_owned(owned) { }
  template <class F>
  void find(Candidates& c, int32_t n, F&& f) const
  {
    c.offsets.resize(n);
    c.counts.resize(n);
    int32_t* cand = nullptr;
    int64_t total = 0;
    check(f(c.offsets.data(), c.counts.data(), &cand, &total));
    c.candidates.assign(cand, cand + total);
    gsq_free(cand);
  }
  gsq_bvh* m_h = nullptr;
  bool m_owned = true;
};
}  // namespace spin

namespace quest
{
// An unstructured single-shape surface mesh (the data SignedDistance reads
// from mint::Mesh: SignedDistance.cpp:16-45).
struct SurfaceMesh
{
  std::vector<double> x, y, z;
  std::vector<int32_t> cells;
  int32_t nodes_per_cell = 3;  // 3 triangles, 4 quads
  int32_t numCells() const { return (int32_t)(cells.size() / nodes_per_cell); }
};

template <int NDIMS>
class SignedDistance
{
  static_assert(NDIMS == 3, "gsq implements the 3D signed distance");

public:
  // SignedDistance(mesh, isWatertight, computeSign) (quest/SignedDistance.hpp:410-424)
  SignedDistance(const SurfaceMesh& mesh, bool isWatertight, bool computeSign = true,
                 int32_t precision = GSQ_PRECISION_FP64)
  {
    gsq_sdf_opts o;
    check(gsq_sdf_opts_init(&o));
    o.precision = precision;
    check(gsq_sdf_create(&m_h, mesh.x.data(), mesh.y.data(), mesh.z.data(), (int32_t)mesh.x.size(),
                         mesh.cells.data(), mesh.numCells(), mesh.nodes_per_cell, isWatertight, computeSign, &o,
                         nullptr));
  }
  ~SignedDistance() { gsq_sdf_destroy(m_h); }
  SignedDistance(const SignedDistance&) = delete;
  SignedDistance& operator=(const SignedDistance&) = delete;

  // computeDistance (SD:507-524)
  double computeDistance(const Point& p) const
  {
    double d;
    check(gsq_sdf_eval(m_h, p.x, p.x + 1, p.x + 2, 3, 1, &d, nullptr, nullptr, nullptr));
    return d;
  }
  double computeDistance(const Point& p, Point& closest, double* normal) const
  {
    double d;
    check(gsq_sdf_eval(m_h, p.x, p.x + 1, p.x + 2, 3, 1, &d, closest.x, normal, nullptr));
    return d;
  }
  // computeDistances (SD:527-605): points host or device, outputs alike.
  void computeDistances(int32_t n, const Point* pts, double* out, Point* closest = nullptr,
                        double* normals = nullptr, void* stream = nullptr) const
  {
    const double* q = reinterpret_cast<const double*>(pts);
    check(gsq_sdf_eval(m_h, q, q + 1, q + 2, 3, n, out, reinterpret_cast<double*>(closest), normals, stream));
  }
  // signed_distance_evaluate(x, y, z, n, phi) form (quest/interface/signed_distance.hpp:290)
  void computeDistances(int32_t n, const double* x, const double* y, const double* z, double* out,
                        void* stream = nullptr) const
  {
    check(gsq_sdf_eval(m_h, x, y, z, 1, n, out, nullptr, nullptr, stream));
  }
  BoundingBox getMeshBounds() const
  {
    BoundingBox b;
    check(gsq_sdf_mesh_bounds(m_h, b.min, b.max));
    return b;
  }
  const gsq_sdf* handle() const { return m_h; }

private:
  gsq_sdf* m_h = nullptr;
};

// STLReader (quest/readers/STLReader.hpp): setFileName, read, getMesh.
class STLReader
{
public:
  void setFileName(const std::string& name) { m_file = name; }
  // read() (STLReader.cpp:190-202): 0 on success, -1 otherwise
  int read()
  {
    double* xyz = nullptr;
    int32_t* cells = nullptr;
    int32_t nn = 0, nc = 0;
    if(gsq_stl_read(m_file.c_str(), &xyz, &nn, &cells, &nc) != GSQ_OK) return -1;
    m_mesh.x.resize(nn);
    m_mesh.y.resize(nn);
    m_mesh.z.resize(nn);
    for(int32_t i = 0; i < nn; ++i)
    {
      m_mesh.x[i] = xyz[3 * i];
      m_mesh.y[i] = xyz[3 * i + 1];
      m_mesh.z[i] = xyz[3 * i + 2];
    }
    m_mesh.cells.assign(cells, cells + 3 * (size_t)nc);
    m_mesh.nodes_per_cell = 3;
    gsq_free(xyz);
    gsq_free(cells);
    return 0;
  }
  // getMesh (STLReader.cpp:205-250): three nodes per triangle, in file order
  void getMesh(SurfaceMesh& mesh) const { mesh = m_mesh; }

private:
  std::string m_file;
  SurfaceMesh m_mesh;
};

// The local step of DistributedClosestPoint
// (quest/detail/DistributedClosestPointImpl.hpp:883-901, 1002-1050).
class ClosestPoint
{
public:
  // the object points (generateBVHTree) and their domain ids (nullable)
  ClosestPoint(int32_t n, const Point* pts, const int32_t* domain_ids = nullptr, void* stream = nullptr)
  {
    check(gsq_cpq_create(&m_h, reinterpret_cast<const double*>(pts), n, domain_ids, stream));
  }
  ~ClosestPoint() { gsq_cpq_destroy(m_h); }
  ClosestPoint(const ClosestPoint&) = delete;
  ClosestPoint& operator=(const ClosestPoint&) = delete;
  // setDistanceThreshold (DistributedClosestPoint.cpp:125-130) stores t * t
  void setDistanceThreshold(double t) { m_sq_threshold = t * t; }
  // per query point: closest object point index and domain (-1 if none),
  // its coordinates and distance (NaN if none)
  void computeClosestPoints(int32_t m, const Point* queries, int32_t* idx, int32_t* dom, Point* pos, double* dist,
                            int32_t precision = GSQ_PRECISION_MIXED, void* stream = nullptr) const
  {
    check(gsq_cpq_query(m_h, reinterpret_cast<const double*>(queries), m, m_sq_threshold, precision, idx, dom,
                        reinterpret_cast<double*>(pos), dist, stream));
  }

private:
  gsq_cpq* m_h = nullptr;
  double m_sq_threshold = DBL_MAX;
};

// The C-style interface of quest/interface/signed_distance.hpp:88-319 (a
// global query object), over the QUEST_signed_distance_* entry points of
// gsq_quest.h.  As in the reference, misuse (options after init, evaluate
// before init, null buffers, a dimension other than 3) aborts the process.
enum class SignedDistExec
{
  CPU = QUEST_SignedDistExec_CPU,
  OpenMP = QUEST_SignedDistExec_OpenMP,
  GPU = QUEST_SignedDistExec_GPU
};

// signed_distance_init(file) (signed_distance.hpp:117) and (mesh) (:137): 0, or -1
inline int signed_distance_init(const std::string& file) { return QUEST_signed_distance_init_serial(file.c_str()); }
inline int signed_distance_init(const SurfaceMesh* m)
{
  // triangles only: -1 for other cells, where the reference aborts
  // (signed_distance.cpp:174-175)
  if(m->nodes_per_cell != 3) return -1;
  return gsq_quest_init_mesh(m->x.data(), m->y.data(), m->z.data(), (int32_t)m->x.size(), m->cells.data(),
                             m->numCells());
}
inline bool signed_distance_initialized() { return QUEST_signed_distance_initialized(); }
inline void signed_distance_set_dimension(int dim) { QUEST_signed_distance_set_dimension(dim); }
inline void signed_distance_set_closed_surface(bool status) { QUEST_signed_distance_set_closed_surface(status); }
inline void signed_distance_set_compute_signs(bool computeSign)
{
  QUEST_signed_distance_set_compute_signs(computeSign);
}
inline void signed_distance_set_allocator(int allocatorID) { QUEST_signed_distance_set_allocator(allocatorID); }
inline void signed_distance_set_verbose(bool status) { QUEST_signed_distance_set_verbose(status); }
inline void signed_distance_use_shared_memory(bool status) { QUEST_signed_distance_use_shared_memory(status); }
inline void signed_distance_set_execution_space(SignedDistExec s)
{
  QUEST_signed_distance_set_execution_space((int)s);
}
// signed_distance_evaluate (:248, :266, :290)
inline double signed_distance_evaluate(double x, double y, double z = 0.0)
{
  return QUEST_signed_distance_evaluate_0(x, y, z);
}
inline double signed_distance_evaluate(double x, double y, double z, double& cp_x, double& cp_y, double& cp_z,
                                       double& n_x, double& n_y, double& n_z)
{
  return QUEST_signed_distance_evaluate_1(x, y, z, &cp_x, &cp_y, &cp_z, &n_x, &n_y, &n_z);
}
inline void signed_distance_evaluate(const double* x, const double* y, const double* z, int npoints, double* phi)
{
  gsq_quest_evaluate_points(x, y, z, npoints, phi);
}
inline void signed_distance_get_mesh_bounds(double* lo, double* hi) { QUEST_signed_distance_get_mesh_bounds(lo, hi); }
inline void signed_distance_finalize() { QUEST_signed_distance_finalize(); }
}  // namespace quest
}  // namespace gsq

#endif  // GSQ_HPP_
