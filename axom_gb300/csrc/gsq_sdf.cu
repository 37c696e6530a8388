// Signed distance to a surface mesh on the GPU (quest::SignedDistance
// replacement).
//
// Set-up (replaces SignedDistance::setMesh, quest/SignedDistance.hpp:427-504):
// the mesh is copied to the device, the mesh box is folded (SD:483-486), one
// box per cell is built (getCellBoundingBox, SD:608-633) and the BVH is built
// over them.  Then one "leaf record" per sorted BVH leaf is written with the
// cell's vertex coordinates inline, so a leaf test is one contiguous 80-byte
// (triangle) or 112-byte (quad) read instead of id -> connectivity -> vertex
// gathers.
//
// Query (replaces computeDistances, SD:527-605): one thread per point runs
// the reference traversal (bvh_traverse.hpp:66-154) with the point
// traverser's nearer-centroid-first order (policy/LinearBVH.hpp:72-85), the
// min-distance predicate (SD:576-578) and checkCandidate (SD:636-737), all in
// FP64 with the reference's operation order, so distances, closest points and
// signs are bit-identical to the reference.  Queries may be processed in
// Morton order of the point (results are per point, so order does not change
// them) for warp coherence and cache reuse.
#include "gsq_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

namespace gsq
{
const BvhDev* bvh_dev(const gsq_bvh* h);
gsq_bvh* bvh_new_internal(int device);
int bvh_build_internal(gsq_bvh* h, const double* d_boxes, int n, cudaStream_t s);
int node_bounds(const double* x, const double* y, const double* z, int nv, double* out6, cudaStream_t s);

template <int NPC>
struct LeafRec;
template <>
struct __align__(16) LeafRec<3>
{
  double v[9];
  int cell;
  int pad;
};
template <>
struct __align__(16) LeafRec<4>
{
  double v[12];
  int cell;
  int pad[3];
};
static_assert(sizeof(LeafRec<3>) == 80, "triangle leaf record is 80 bytes");
static_assert(sizeof(LeafRec<4>) == 112, "quad leaf record is 112 bytes");

namespace
{
constexpr double CP_EPS = 1e-12;  // SD:665

__device__ __forceinline__ double sqdist_pp(const double* a, const double* b)
{
  // squared_distance(Point A, Point B) (squared_distance.hpp:62-67): |B - A|^2
  const double v0 = b[0] - a[0], v1 = b[1] - a[1], v2 = b[2] - a[2];
  return dot3(v0, v1, v2, v0, v1, v2);
}

__device__ __forceinline__ bool is_leq(double x, double y) { return !((x > y) && !near_eq(x, y, CP_EPS)); }
__device__ __forceinline__ bool is_geq(double x, double y) { return !((x < y) && !near_eq(x, y, CP_EPS)); }

// closest_point(Point, Triangle, loc, EPS) (primal/operators/closest_point.hpp:162-290)
__device__ __forceinline__ int closest_point(const double* P, const double* A, const double* B, const double* C,
                                             double* out)
{
  const double ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const double ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const double ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const double d1 = dot3(ab0, ab1, ab2, ap0, ap1, ap2);
  const double d2 = dot3(ac0, ac1, ac2, ap0, ap1, ap2);
  if(is_leq(d1, 0.0) && is_leq(d2, 0.0))
  {
    out[0] = A[0], out[1] = A[1], out[2] = A[2];
    return 0;
  }
  const double bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const double d3 = dot3(ab0, ab1, ab2, bp0, bp1, bp2);
  const double d4 = dot3(ac0, ac1, ac2, bp0, bp1, bp2);
  if(is_geq(d3, 0.0) && is_leq(d4, d3))
  {
    out[0] = B[0], out[1] = B[1], out[2] = B[2];
    return 1;
  }
  const double vc = d1 * d4 - d3 * d2;
  if(is_leq(vc, 0.0) && is_geq(d1, 0.0) && is_leq(d3, 0.0) && !near_eq(d1, d3, CP_EPS))
  {
    const double v = d1 / (d1 - d3);
    out[0] = A[0] + ab0 * v, out[1] = A[1] + ab1 * v, out[2] = A[2] + ab2 * v;
    return -1;
  }
  const double cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const double d5 = dot3(ab0, ab1, ab2, cp0, cp1, cp2);
  const double d6 = dot3(ac0, ac1, ac2, cp0, cp1, cp2);
  if(is_geq(d6, 0.0) && is_leq(d5, d6))
  {
    out[0] = C[0], out[1] = C[1], out[2] = C[2];
    return 2;
  }
  const double vb = d5 * d2 - d1 * d6;
  if(is_leq(vb, 0.0) && is_geq(d2, 0.0) && is_leq(d6, 0.0))
  {
    const double w = d2 / (d2 - d6);
    out[0] = A[0] + ac0 * w, out[1] = A[1] + ac1 * w, out[2] = A[2] + ac2 * w;
    return -3;
  }
  const double va = d3 * d6 - d5 * d4;
  if(is_leq(va, 0.0) && is_geq(d4 - d3, 0.0) && is_geq(d5 - d6, 0.0))
  {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    out[0] = B[0] + (C[0] - B[0]) * w, out[1] = B[1] + (C[1] - B[1]) * w, out[2] = B[2] + (C[2] - B[2]) * w;
    return -2;
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom, w = vc * denom;
  const double n0 = ab0 * v + ac0 * w, n1 = ab1 * v + ac1 * w, n2 = ab2 * v + ac2 * w;
  out[0] = A[0] + n0, out[1] = A[1] + n1, out[2] = A[2] + n2;
  return 3;
}

// Triangle::normal (Triangle.hpp:98-102) = cross(B - A, C - A) through
// numerics::determinant (Vector.hpp:563-570).
__device__ __forceinline__ void tri_normal(const double* A, const double* B, const double* C, double* n)
{
  const double u0 = B[0] - A[0], u1 = B[1] - A[1], u2 = B[2] - A[2];
  const double v0 = C[0] - A[0], v1 = C[1] - A[1], v2 = C[2] - A[2];
  n[0] = u1 * v2 - v1 * u2;
  n[1] = v0 * u2 - u0 * v2;
  n[2] = u0 * v1 - v0 * u1;
}

// Vector::unitVector (Vector.hpp:477-493)
__device__ __forceinline__ void unit3(const double* v, double* o)
{
  const double l2 = dot3(v[0], v[1], v[2], v[0], v[1], v[2]);
  if(l2 >= 1e-50)
  {
    const double s = 1.0 / sqrt(l2);
    o[0] = v[0] * s, o[1] = v[1] * s, o[2] = v[2] * s;
  }
  else
    o[0] = 1.0, o[1] = 0.0, o[2] = 0.0;
}

// Triangle::angle (Triangle.hpp:385-400)
__device__ __forceinline__ double tri_angle(const double* const* T, int idx)
{
  const double* pt = T[idx];
  const double* p1 = T[(idx + 1) % 3];
  const double* p2 = T[(idx + 2) % 3];
  const double a[3] = {p1[0] - pt[0], p1[1] - pt[1], p1[2] - pt[2]};
  const double b[3] = {p2[0] - pt[0], p2[1] - pt[1], p2[2] - pt[2]};
  double u1[3], u2[3];
  unit3(a, u1);
  unit3(b, u2);
  double dp = dot3(u1[0], u1[1], u1[2], u2[0], u2[1], u2[2]);
  dp = (dp < -1.0) ? -1.0 : (dp > 1.0) ? 1.0 : dp;
  return acos(dp);
}

// Triangle::degenerate (Triangle.hpp:327-330): |0.5 |n| - 0| <= 1e-12
__device__ __forceinline__ bool tri_degenerate(const double* A, const double* B, const double* C)
{
  double n[3];
  tri_normal(A, B, C, n);
  const double area = 0.5 * sqrt(dot3(n[0], n[1], n[2], n[0], n[1], n[2]));
  return near_eq(area, 0.0, 1.0e-12);
}

// MinCandidate (SD:159-175); the closest element's geometry is kept as its
// leaf position and sub-triangle and reloaded at the end.
struct MinCand
{
  double minSq;
  double mp[3];
  double sn[3];
  int type;  // -1 uninitialized, 0 vertex, 1 edge, 2 face (SD:110-137)
  int leaf;
  int sub;
};

// checkCandidate for one triangle (SD:667-736)
__device__ __forceinline__ void check_triangle(const double* q, MinCand& m, const double* const* T, int leafpos,
                                               int sub, bool computeNormal)
{
  double cp[3];
  const int loc = closest_point(q, T[0], T[1], T[2], cp);
  const double sq = sqdist_pp(q, cp);
  const int ty = (loc < 0) ? 1 : (loc <= 2) ? 0 : 2;
  const bool shared = (ty != 2);
  bool upd;
  if(sq < m.minSq)
  {
    const bool clear = !shared || (m.type != ty) || !near_eq(sqdist_pp(cp, m.mp), 0.0, CP_EPS);
    m.minSq = sq;
    m.mp[0] = cp[0], m.mp[1] = cp[1], m.mp[2] = cp[2];
    m.type = ty;
    m.leaf = leafpos;
    m.sub = sub;
    if(computeNormal && clear) m.sn[0] = m.sn[1] = m.sn[2] = 0.0;
    upd = computeNormal && shared;
  }
  else
    upd = computeNormal && shared && (m.type == ty) && near_eq(sqdist_pp(cp, m.mp), 0.0, CP_EPS);
  if(upd)
  {
    if(ty == 1)
    {
      double n[3], u[3];
      tri_normal(T[0], T[1], T[2], n);
      unit3(n, u);
      m.sn[0] = m.sn[0] + u[0], m.sn[1] = m.sn[1] + u[1], m.sn[2] = m.sn[2] + u[2];
    }
    else if(!tri_degenerate(T[0], T[1], T[2]))
    {
      const double alpha = tri_angle(T, loc);
      double n[3], u[3];
      tri_normal(T[0], T[1], T[2], n);
      unit3(n, u);
      m.sn[0] = m.sn[0] + u[0] * alpha, m.sn[1] = m.sn[1] + u[1] * alpha, m.sn[2] = m.sn[2] + u[2] * alpha;
    }
  }
}

template <int NPC>
__device__ __forceinline__ void load_leaf(const LeafRec<NPC>* __restrict__ leaves, int leafpos, double* v)
{
  const double2* r = reinterpret_cast<const double2*>(leaves + leafpos);
#pragma unroll
  for(int k = 0; k < (3 * NPC) / 2; ++k)
  {
    const double2 t = __ldg(r + k);
    v[2 * k] = t.x;
    v[2 * k + 1] = t.y;
  }
  if((3 * NPC) % 2) v[3 * NPC - 1] = __ldg(&leaves[leafpos].v[3 * NPC - 1]);
}

// squared_distance(Point, BoundingBox) (squared_distance.hpp:77-102)
__device__ __forceinline__ double sqdist_pb(const double* p, const double* lo, const double* hi)
{
  if(!box_valid(lo, hi)) return DBL_MAX;
  if(!(p[0] < lo[0] || p[0] > hi[0] || p[1] < lo[1] || p[1] > hi[1] || p[2] < lo[2] || p[2] > hi[2])) return 0.0;
  double c[3];
  for(int d = 0; d < 3; ++d) c[d] = (p[d] < lo[d]) ? lo[d] : (p[d] > hi[d]) ? hi[d] : p[d];
  return sqdist_pp(p, c);
}

struct SdfParams
{
  double domain[6];  // mesh box (SD:483-486)
  int watertight;
  int sign;
};

struct QueryPts
{
  const double* x;
  const double* y;
  const double* z;
  int stride;
};

template <int NPC>
__global__ void __launch_bounds__(128) k_sdf_fp64(const NodeRec64* __restrict__ nodes,
                                                  const LeafRec<NPC>* __restrict__ leaves,
                                                  QueryPts qp,
                                                  int m,
                                                  const int* __restrict__ order,
                                                  SdfParams prm,
                                                  double* __restrict__ out,
                                                  double* __restrict__ out_cp,
                                                  double* __restrict__ out_n,
                                                  int* err)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  const int idx = order ? __ldg(order + t) : t;
  const double q[3] = {qp.x[(size_t)idx * qp.stride], qp.y[(size_t)idx * qp.stride], qp.z[(size_t)idx * qp.stride]};
  const bool computeNormal = prm.sign != 0;
  MinCand mc;
  mc.minSq = DBL_MAX;
  mc.mp[0] = mc.mp[1] = mc.mp[2] = 0.0;
  mc.sn[0] = mc.sn[1] = mc.sn[2] = 0.0;
  mc.type = -1;
  mc.leaf = -1;
  mc.sub = 0;

  auto leaf_action = [&](int leafpos) {
    double v[3 * NPC];
    load_leaf<NPC>(leaves, leafpos, v);
    const double* T0[3] = {v, v + 3, v + 6};
    check_triangle(q, mc, T0, leafpos, 0, computeNormal);
    if constexpr(NPC == 4)
    {
      const double* T1[3] = {v, v + 6, v + 9};
      check_triangle(q, mc, T1, leafpos, 1, computeNormal);
    }
  };

  // bvh_traverse with the point preference; pruning uses the running minimum.
  int todo[STACK_SIZE];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0, cur = 0;
  bool overflow = false;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      const double2* r = reinterpret_cast<const double2*>(nodes + cur);
      double b[12];
#pragma unroll
      for(int k = 0; k < 6; ++k)
      {
        const double2 v = __ldg(r + k);
        b[2 * k] = v.x;
        b[2 * k + 1] = v.y;
      }
      const int2 ch = __ldg(reinterpret_cast<const int2*>(nodes[cur].child));
      const bool inL = box_valid(b, b + 3) ? (sqdist_pb(q, b, b + 3) <= mc.minSq) : false;
      const bool inR = box_valid(b + 6, b + 9) ? (sqdist_pb(q, b + 6, b + 9) <= mc.minSq) : false;
      if(!inL && !inR)
        cur = (sp >= 0) ? todo[sp--] : BARRIER;
      else
      {
        cur = inL ? ch.x : ch.y;
        int rc = ch.y;
        if(inL && inR)
        {
          // traversePref (LB:75-82): swap when the left centroid is farther.
          const double cl[3] = {0.5 * (b[0] + b[3]), 0.5 * (b[1] + b[4]), 0.5 * (b[2] + b[5])};
          const double cr[3] = {0.5 * (b[6] + b[9]), 0.5 * (b[7] + b[10]), 0.5 * (b[8] + b[11])};
          const double sl = sqdist_pp(q, cl);
          const double sr = sqdist_pp(q, cr);  // right box is valid here
          if(sl > sr)
          {
            const int tmp = cur;
            cur = rc;
            rc = tmp;
          }
          if(sp + 1 >= STACK_SIZE)
          {
            overflow = true;
            break;
          }
          todo[++sp] = rc;
        }
      }
      if(cur < 0 && !(found < 0))
      {
        found = cur;
        if(cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
      }
    }
    if(overflow) break;
    while(found < 0 && found != BARRIER)
    {
      leaf_action(-found - 1);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
    }
    found = 0;
  }
  if(overflow) atomicOr(err, DEVERR_STACK);

  // Sign (SD:583-592) and outputs (SD:594-603).
  double nrm[3] = {mc.sn[0], mc.sn[1], mc.sn[2]};
  if(mc.type == 2)
  {
    double v[3 * NPC];
    load_leaf<NPC>(leaves, mc.leaf, v);
    if(NPC == 4 && mc.sub == 1)
      tri_normal(v, v + 6, v + 9, nrm);
    else
      tri_normal(v, v + 3, v + 6, nrm);
  }
  double sgn = 1.0;
  if(prm.sign)
  {
    const double* D = prm.domain;
    const bool inside_box = !(mc.mp[0] < D[0] || mc.mp[0] > D[3] || mc.mp[1] < D[1] || mc.mp[1] > D[4] ||
                              mc.mp[2] < D[2] || mc.mp[2] > D[5]);
    if(!(prm.watertight && !inside_box))
    {
      const double r0 = q[0] - mc.mp[0], r1 = q[1] - mc.mp[1], r2 = q[2] - mc.mp[2];
      sgn = (dot3(r0, r1, r2, nrm[0], nrm[1], nrm[2]) >= 0.0) ? 1.0 : -1.0;
    }
  }
  out[idx] = sqrt(mc.minSq) * sgn;
  if(out_cp)
  {
    out_cp[3 * (size_t)idx + 0] = mc.mp[0];
    out_cp[3 * (size_t)idx + 1] = mc.mp[1];
    out_cp[3 * (size_t)idx + 2] = mc.mp[2];
  }
  if(out_n)
  {
    double u[3];
    unit3(nrm, u);
    out_n[3 * (size_t)idx + 0] = u[0];
    out_n[3 * (size_t)idx + 1] = u[1];
    out_n[3 * (size_t)idx + 2] = u[2];
  }
}

// Per-cell bounding boxes (getCellBoundingBox, SD:608-633): addPoint of each
// node into an invalid box.
__global__ void k_cell_boxes(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                             const int* __restrict__ cells, int ncells, int npc, int nverts, double* __restrict__ boxes,
                             int* err)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if(c >= ncells) return;
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for(int k = 0; k < npc; ++k)
  {
    int v = cells[(size_t)c * npc + k];
    if(v < 0 || v >= nverts)
    {
      atomicOr(err, DEVERR_RANGE);
      v = 0;
    }
    const double p[3] = {x[v], y[v], z[v]};
    for(int d = 0; d < 3; ++d)
    {
      if(p[d] < lo[d]) lo[d] = p[d];
      if(p[d] > hi[d]) hi[d] = p[d];
    }
  }
  for(int d = 0; d < 3; ++d)
  {
    boxes[6 * (size_t)c + d] = lo[d];
    boxes[6 * (size_t)c + 3 + d] = hi[d];
  }
}

// One record per sorted leaf: the cell's vertex coordinates inline.  Padding
// leaves (cell id >= ncells, from BVH::initialize's 0/1-box padding) are
// never reached by a traversal; they get zero coordinates.
template <int NPC>
__global__ void k_leaf_records(const int* __restrict__ perm, int nleaves, const double* __restrict__ x,
                               const double* __restrict__ y, const double* __restrict__ z,
                               const int* __restrict__ cells, int ncells, int nverts, LeafRec<NPC>* __restrict__ recs)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k >= nleaves) return;
  const int c = perm[k];
  LeafRec<NPC> r;
  for(int j = 0; j < NPC; ++j)
  {
    int v = (c < ncells) ? cells[(size_t)c * NPC + j] : -1;
    const bool ok = (v >= 0 && v < nverts);
    r.v[3 * j + 0] = ok ? x[v] : 0.0;
    r.v[3 * j + 1] = ok ? y[v] : 0.0;
    r.v[3 * j + 2] = ok ? z[v] : 0.0;
  }
  r.cell = c;
  recs[k] = r;
}

// 30-bit Morton code of each query point in the given box (processing order
// only; results do not depend on it).
__global__ void k_query_codes(QueryPts qp, int m, double lx, double ly, double lz, double sx, double sy, double sz,
                              uint32_t* __restrict__ codes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  const double c[3] = {(qp.x[(size_t)i * qp.stride] - lx) * sx, (qp.y[(size_t)i * qp.stride] - ly) * sy,
                       (qp.z[(size_t)i * qp.stride] - lz) * sz};
  uint32_t u[3];
  for(int d = 0; d < 3; ++d)
  {
    const double f = fmin(fmax(c[d] * 1024.0, 0.0), 1023.0);
    u[d] = (uint32_t)(int)f;
  }
  auto spread = [](uint32_t v) {
    v = (v | (v << 16)) & 0xFF0000FFu;
    v = (v | (v << 8)) & 0x0F00F00Fu;
    v = (v | (v << 4)) & 0xC30C30C3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
  };
  codes[i] = spread(u[0]) | (spread(u[1]) << 1) | (spread(u[2]) << 2);
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

}  // namespace
}  // namespace gsq

using namespace gsq;

// =============================================================================
// C ABI: quest::SignedDistance
// =============================================================================
struct gsq_sdf
{
  int device = 0;
  gsq_sdf_opts opts;
  int watertight = 1, sign = 1;
  int nverts = 0, ncells = 0, npc = 3;
  double* d_x = nullptr;  // device copies of the mesh (x, y, z, cells in one block)
  double* d_y = nullptr;
  double* d_z = nullptr;
  int* d_cells = nullptr;
  void* mesh_block = nullptr;
  double domain[6];
  gsq_bvh* bvh = nullptr;
  void* leaves = nullptr;
  int* d_err = nullptr;
  float eval_ms = 0.f;
};

namespace
{
void sdf_release(gsq_sdf* h)
{
  if(h->mesh_block) cudaFree(h->mesh_block);
  if(h->leaves) cudaFree(h->leaves);
  if(h->d_err) cudaFree(h->d_err);
  if(h->bvh) gsq_bvh_destroy(h->bvh);
  delete h;
}

int stage_queries(const double* qx, const double* qy, const double* qz, int stride, int m, cudaStream_t s,
                  InBuf* bufs, QueryPts& qp)
{
  qp.stride = stride;
  const size_t span = sizeof(double) * ((size_t)(m - 1) * stride + 1);
  const bool aos = (stride == 3 && qy == qx + 1 && qz == qx + 2);
  if(aos)
  {
    GSQ_CUDA_TRY(bufs[0].stage(qx, sizeof(double) * 3 * (size_t)m, s));
    qp.x = static_cast<const double*>(bufs[0].dev);
    qp.y = qp.x + 1;
    qp.z = qp.x + 2;
    return GSQ_OK;
  }
  GSQ_CUDA_TRY(bufs[0].stage(qx, span, s));
  GSQ_CUDA_TRY(bufs[1].stage(qy, span, s));
  GSQ_CUDA_TRY(bufs[2].stage(qz, span, s));
  qp.x = static_cast<const double*>(bufs[0].dev);
  qp.y = static_cast<const double*>(bufs[1].dev);
  qp.z = static_cast<const double*>(bufs[2].dev);
  return GSQ_OK;
}
}  // namespace

extern "C" {

int gsq_sdf_opts_init(gsq_sdf_opts* o)
{
  if(!o) return fail(GSQ_ERR_INVALID, "null opts");
  std::memset(o, 0, sizeof(*o));
  o->precision = GSQ_PRECISION_FP64;
  o->sort_queries = 1;
  o->block_size = 0;
  return GSQ_OK;
}

int gsq_sdf_create(gsq_sdf** out, const double* x, const double* y, const double* z, int32_t nverts,
                   const int32_t* cells, int32_t ncells, int32_t npc, int32_t watertight, int32_t compute_sign,
                   const gsq_sdf_opts* opts, void* stream)
{
  if(!out) return fail(GSQ_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if(nverts < 0 || ncells < 0 || (npc != 3 && npc != 4)) return fail(GSQ_ERR_INVALID, "invalid mesh sizes");
  if((nverts > 0 && (!x || !y || !z)) || (ncells > 0 && !cells)) return fail(GSQ_ERR_INVALID, "null mesh arrays");
  if(ncells >= (1 << 30)) return fail(GSQ_ERR_INVALID, "at most 2^30-1 cells");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* h = new(std::nothrow) gsq_sdf();
  if(!h) return fail(GSQ_ERR_NOMEM, "handle allocation failed");
  gsq_sdf_opts_init(&h->opts);
  if(opts) h->opts = *opts;
  h->watertight = watertight ? 1 : 0;
  h->sign = compute_sign ? 1 : 0;
  h->nverts = nverts;
  h->ncells = ncells;
  h->npc = npc;
  auto bail = [&](int rc) {
    sdf_release(h);
    return rc;
  };
  cudaError_t e = cudaGetDevice(&h->device);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_err, sizeof(int));
  if(e == cudaSuccess) e = cudaMemsetAsync(h->d_err, 0, sizeof(int), s);
  const size_t vbytes = sizeof(double) * std::max(nverts, 1);
  const size_t cbytes = sizeof(int) * (size_t)std::max(ncells, 1) * npc;
  const size_t vpad = (vbytes + 255) & ~size_t(255);
  if(e == cudaSuccess) e = cudaMalloc(&h->mesh_block, 3 * vpad + cbytes);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create"));
  char* mb = static_cast<char*>(h->mesh_block);
  h->d_x = reinterpret_cast<double*>(mb);
  h->d_y = reinterpret_cast<double*>(mb + vpad);
  h->d_z = reinterpret_cast<double*>(mb + 2 * vpad);
  h->d_cells = reinterpret_cast<int*>(mb + 3 * vpad);
  auto kind = [](const void* p) { return is_device_ptr(p) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; };
  if(nverts > 0)
  {
    e = cudaMemcpyAsync(h->d_x, x, sizeof(double) * nverts, kind(x), s);
    if(e == cudaSuccess) e = cudaMemcpyAsync(h->d_y, y, sizeof(double) * nverts, kind(y), s);
    if(e == cudaSuccess) e = cudaMemcpyAsync(h->d_z, z, sizeof(double) * nverts, kind(z), s);
  }
  if(e == cudaSuccess && ncells > 0)
    e = cudaMemcpyAsync(h->d_cells, cells, sizeof(int) * (size_t)ncells * npc, kind(cells), s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: mesh upload"));

  int rc = node_bounds(h->d_x, h->d_y, h->d_z, nverts, h->domain, s);
  if(rc) return bail(rc);

  Scratch boxes;
  e = boxes.alloc(sizeof(double) * 6 * (size_t)std::max(ncells, 1), s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: boxes"));
  if(ncells > 0)
    count_launch();
  if(ncells > 0)
    k_cell_boxes<<<grid_for(ncells, 256), 256, 0, s>>>(h->d_x, h->d_y, h->d_z, h->d_cells, ncells, npc, nverts,
                                                       boxes.as<double>(), h->d_err);
  h->bvh = bvh_new_internal(h->device);
  if(!h->bvh) return bail(GSQ_ERR_NOMEM);
  rc = bvh_build_internal(h->bvh, boxes.as<double>(), ncells, s);
  if(rc) return bail(rc);
  const BvhDev* B = bvh_dev(h->bvh);
  count_launch();
  const size_t rec = (npc == 3) ? sizeof(LeafRec<3>) : sizeof(LeafRec<4>);
  e = cudaMalloc(&h->leaves, rec * B->n);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: leaf records"));
  if(npc == 3)
    k_leaf_records<3><<<grid_for(B->n, 256), 256, 0, s>>>(B->perm, B->n, h->d_x, h->d_y, h->d_z, h->d_cells, ncells,
                                                         nverts, static_cast<LeafRec<3>*>(h->leaves));
  else
    k_leaf_records<4><<<grid_for(B->n, 256), 256, 0, s>>>(B->perm, B->n, h->d_x, h->d_y, h->d_z, h->d_cells, ncells,
                                                         nverts, static_cast<LeafRec<4>*>(h->leaves));
  e = cudaGetLastError();
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create"));
  rc = check_device_error(h->d_err, s, "gsq_sdf_create");
  if(rc) return bail(rc);
  *out = h;
  return GSQ_OK;
}

int gsq_sdf_destroy(gsq_sdf* h)
{
  if(h) sdf_release(h);
  return GSQ_OK;
}

int gsq_sdf_set_opts(gsq_sdf* h, const gsq_sdf_opts* o)
{
  if(!h || !o) return fail(GSQ_ERR_INVALID, "null argument");
  if(o->precision != GSQ_PRECISION_FP64 && o->precision != GSQ_PRECISION_MIXED)
    return fail(GSQ_ERR_INVALID, "unknown precision");
  h->opts = *o;
  return GSQ_OK;
}

int gsq_sdf_mesh_bounds(const gsq_sdf* h, double* lo, double* hi)
{
  if(!h || !lo || !hi) return fail(GSQ_ERR_INVALID, "null argument");
  for(int d = 0; d < 3; ++d)
  {
    lo[d] = h->domain[d];
    hi[d] = h->domain[3 + d];
  }
  return GSQ_OK;
}

int gsq_sdf_get_bvh(const gsq_sdf* h, const gsq_bvh** b)
{
  if(!h || !b) return fail(GSQ_ERR_INVALID, "null argument");
  *b = h->bvh;
  return GSQ_OK;
}

int gsq_sdf_last_eval_ms(const gsq_sdf* h, float* ms)
{
  if(!h || !ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->eval_ms;
  return GSQ_OK;
}

int gsq_sdf_eval(const gsq_sdf* hc, const double* qx, const double* qy, const double* qz, int32_t stride, int32_t m,
                 double* out, double* closest, double* normals, void* stream)
{
  gsq_sdf* h = const_cast<gsq_sdf*>(hc);
  if(!h) return fail(GSQ_ERR_INVALID, "null sdf handle");
  if(m < 0 || stride < 1) return fail(GSQ_ERR_INVALID, "invalid query count or stride");
  if(m == 0) return GSQ_OK;
  if(!qx || !qy || !qz || !out) return fail(GSQ_ERR_INVALID, "null query or output array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  InBuf qb[3];
  QueryPts qp;
  int rc = stage_queries(qx, qy, qz, stride, m, s, qb, qp);
  if(rc) return rc;
  OutBuf ob, cb, nb;
  GSQ_CUDA_TRY(ob.prepare(out, sizeof(double) * (size_t)m, s));
  GSQ_CUDA_TRY(cb.prepare(closest, sizeof(double) * 3 * (size_t)m, s));
  GSQ_CUDA_TRY(nb.prepare(normals, sizeof(double) * 3 * (size_t)m, s));

  const BvhDev* B = bvh_dev(h->bvh);
  Scratch order_buf;
  const int* order = nullptr;
  if(h->opts.sort_queries && m > 1)
  {
    GSQ_CUDA_TRY(order_buf.alloc(4 * sizeof(uint32_t) * (size_t)m, s));
    uint32_t* keys[2] = {order_buf.as<uint32_t>(), order_buf.as<uint32_t>() + m};
    int* vals[2] = {reinterpret_cast<int*>(order_buf.as<uint32_t>() + 2 * (size_t)m),
                    reinterpret_cast<int*>(order_buf.as<uint32_t>() + 3 * (size_t)m)};
    const double* b = B->bounds;
    double sc[3];
    for(int d = 0; d < 3; ++d)
    {
      const double ext = b[3 + d] - b[d];
      sc[d] = (ext > 0.0) ? 1.0 / ext : 0.0;
    }
    count_launch();
    k_query_codes<<<grid_for(m, 256), 256, 0, s>>>(qp, m, b[0], b[1], b[2], sc[0], sc[1], sc[2], keys[0]);
    const int which = radix_sort_pairs(keys, vals, m, 30, true, s, h->d_err);
    if(which < 0) return which;
    order = vals[which];
  }

  SdfParams prm;
  std::memcpy(prm.domain, h->domain, sizeof(prm.domain));
  prm.watertight = h->watertight;
  prm.sign = h->sign;
  const int threads = 128;
  count_launch();
  cudaEvent_t e0, e1;
  GSQ_CUDA_TRY(cudaEventCreate(&e0));
  GSQ_CUDA_TRY(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  if(h->npc == 3)
    k_sdf_fp64<3><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<3>*>(h->leaves), qp, m,
                                                          order, prm, static_cast<double*>(ob.dev),
                                                          static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                                                          h->d_err);
  else
    k_sdf_fp64<4><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<4>*>(h->leaves), qp, m,
                                                          order, prm, static_cast<double*>(ob.dev),
                                                          static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                                                          h->d_err);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaGetLastError();
  if(e == cudaSuccess) e = ob.flush(s);
  if(e == cudaSuccess) e = cb.flush(s);
  if(e == cudaSuccess) e = nb.flush(s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaEventElapsedTime(&h->eval_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(e != cudaSuccess) return cuda_fail(e, "gsq_sdf_eval");
  return check_device_error(h->d_err, s, "gsq_sdf_eval");
}

}  // extern "C"
