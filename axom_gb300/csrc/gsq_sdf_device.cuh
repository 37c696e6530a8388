// FP64 device primitives of the signed-distance query, shared by the FP64
// and mixed-precision kernels.  Each restates an axom primitive with the same
// operation order (cited per function); compiled with -fmad=false.
#pragma once

#include "gsq_internal.cuh"

namespace gsq
{
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

namespace sdf
{
constexpr double CP_EPS = 1e-12;  // SD:665

__device__ __forceinline__ double sqdist_pp(const double* a, const double* b)
{
  // squared_distance(Point A, Point B) (squared_distance.hpp:62-67): |B - A|^2
  const double v0 = b[0] - a[0], v1 = b[1] - a[1], v2 = b[2] - a[2];
  return dot3(v0, v1, v2, v0, v1, v2);
}

__device__ __forceinline__ bool is_leq(double x, double y)
{
  return !(ok_gt(okey(x), okey(y)) && !abs_le_eps(x - y));
}
__device__ __forceinline__ bool is_geq(double x, double y)
{
  return !(ok_lt(okey(x), okey(y)) && !abs_le_eps(x - y));
}
// The same predicates in one comparison, given d = x - y rounded: x > y makes
// the rounded difference positive (FP64 keeps subnormals), so "x > y and
// |x - y| > EPS" is "d > EPS", and "x < y and |x - y| > EPS" is "d < -EPS";
// NaNs give true as in is_leq/is_geq.  For y = 0, d is x itself.
// KEYS: the comparison on the integer pipe (for the FP64-pipe-bound
// one-thread-per-point kernels) or as an FP64 comparison (for the mixed
// kernels' converged FP64 batches, where the integer form measured slower).
template <bool KEYS = true>
__device__ __forceinline__ bool leq_d(double d)
{
  if constexpr(KEYS)
    return !gt_eps(d);
  else
    return !(d > CP_EPS);
}
template <bool KEYS = true>
__device__ __forceinline__ bool geq_d(double d)
{
  if constexpr(KEYS)
    return !lt_neg_eps(d);
  else
    return !(d < -CP_EPS);
}

// closest_point(Point, Triangle, loc, EPS) (primal/operators/closest_point.hpp:162-290)
template <bool KEYS = true>
__device__ __forceinline__ int closest_point(const double* P, const double* A, const double* B, const double* C,
                                             double* out)
{
  const double ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const double ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const double ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const double d1 = dot3(ab0, ab1, ab2, ap0, ap1, ap2);
  const double d2 = dot3(ac0, ac1, ac2, ap0, ap1, ap2);
  if(leq_d<KEYS>(d1) && leq_d<KEYS>(d2))  // is_leq(d1, 0) && is_leq(d2, 0)
  {
    out[0] = A[0], out[1] = A[1], out[2] = A[2];
    return 0;
  }
  const double bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const double d3 = dot3(ab0, ab1, ab2, bp0, bp1, bp2);
  const double d4 = dot3(ac0, ac1, ac2, bp0, bp1, bp2);
  if(geq_d<KEYS>(d3) && leq_d<KEYS>(d4 - d3))  // is_geq(d3, 0) && is_leq(d4, d3)
  {
    out[0] = B[0], out[1] = B[1], out[2] = B[2];
    return 1;
  }
  const double vc = d1 * d4 - d3 * d2;
  if(leq_d<KEYS>(vc) && geq_d<KEYS>(d1) && leq_d<KEYS>(d3) && !abs_le_eps(d1 - d3))
  {
    const double v = d1 / (d1 - d3);
    out[0] = A[0] + ab0 * v, out[1] = A[1] + ab1 * v, out[2] = A[2] + ab2 * v;
    return -1;
  }
  const double cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const double d5 = dot3(ab0, ab1, ab2, cp0, cp1, cp2);
  const double d6 = dot3(ac0, ac1, ac2, cp0, cp1, cp2);
  if(geq_d<KEYS>(d6) && leq_d<KEYS>(d5 - d6))  // is_geq(d6, 0) && is_leq(d5, d6)
  {
    out[0] = C[0], out[1] = C[1], out[2] = C[2];
    return 2;
  }
  const double vb = d5 * d2 - d1 * d6;
  if(leq_d<KEYS>(vb) && geq_d<KEYS>(d2) && leq_d<KEYS>(d6))
  {
    const double w = d2 / (d2 - d6);
    out[0] = A[0] + ac0 * w, out[1] = A[1] + ac1 * w, out[2] = A[2] + ac2 * w;
    return -3;
  }
  const double va = d3 * d6 - d5 * d4;
  if(leq_d<KEYS>(va) && geq_d<KEYS>(d4 - d3) && geq_d<KEYS>(d5 - d6))
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
  return abs_le_eps(area);  // isNearlyEqual(area, 0, 1e-12)
}

// MinCandidate (SD:159-175); the closest element's geometry is kept as its
// leaf position and sub-triangle and reloaded at the end.
//
// The pseudo-normal sum is accumulated lazily: checkCandidate's contributions
// (SD:709-736) are recorded in order and only evaluated when the sum is needed
// (flush_normals) or the list is full.  A clear (a strictly closer point that
// is not the same shared vertex or edge) drops the list unevaluated.  The sum
// is formed from the same terms in the same order, so it equals the eager
// sum bit for bit; most contributions of far points are cleared later, and
// each costs a normal, a square root and (for vertices) an arccosine in FP64.
constexpr int NPEND = 8;
struct MinCand
{
  double minSq;
  double mp[3];
  double sn[3];  // the sum of the contributions evaluated so far
  int type;      // -1 uninitialized, 0 vertex, 1 edge, 2 face (SD:110-137)
  int leaf;
  int sub;
  int npend;           // contributions recorded after those in sn
  int pend[NPEND];     // leafpos * 8 + sub * 4 + (vertex index 0..2, or 3 for an edge)
};

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

// One recorded contribution to the pseudo-normal sum (SD:709-736).
template <int NPC>
__device__ __forceinline__ void add_normal(MinCand& m, const LeafRec<NPC>* __restrict__ leaves, int code)
{
  double v[3 * NPC];
  load_leaf<NPC>(leaves, code >> 3, v);
  const int s = (code >> 2) & 1;
  const double* T[3] = {v, v + 3 * (s + 1), v + 3 * (s + 2)};
  const int k = code & 3;
  if(k == 3)
  {
    double n[3], u[3];
    tri_normal(T[0], T[1], T[2], n);
    unit3(n, u);
    m.sn[0] = m.sn[0] + u[0], m.sn[1] = m.sn[1] + u[1], m.sn[2] = m.sn[2] + u[2];
  }
  else if(!tri_degenerate(T[0], T[1], T[2]))
  {
    const double alpha = tri_angle(T, k);
    double n[3], u[3];
    tri_normal(T[0], T[1], T[2], n);
    unit3(n, u);
    m.sn[0] = m.sn[0] + u[0] * alpha, m.sn[1] = m.sn[1] + u[1] * alpha, m.sn[2] = m.sn[2] + u[2] * alpha;
  }
}

// Evaluates the recorded contributions into sn, in order.
template <int NPC>
__device__ __forceinline__ void flush_normals(MinCand& m, const LeafRec<NPC>* __restrict__ leaves)
{
  for(int i = 0; i < m.npend; ++i) add_normal<NPC>(m, leaves, m.pend[i]);
  m.npend = 0;
}

// checkCandidate's state update (SD:675-736) for a triangle whose closest
// point cp (location loc, squared distance sq) is already known; sub-triangle
// `sub` of leaf `leafpos`.
template <int NPC>
__device__ __forceinline__ void apply_candidate(const double* cp, double sq, int loc, MinCand& m,
                                                const LeafRec<NPC>* __restrict__ leaves, int leafpos, int sub,
                                                bool computeNormal)
{
  const int ty = (loc < 0) ? 1 : (loc <= 2) ? 0 : 2;
  const bool shared = (ty != 2);
  bool upd;
  if(ok_lt(okey(sq), okey(m.minSq)))
  {
    const bool clear = !shared || (m.type != ty) || !abs_le_eps(sqdist_pp(cp, m.mp));
    m.minSq = sq;
    m.mp[0] = cp[0], m.mp[1] = cp[1], m.mp[2] = cp[2];
    m.type = ty;
    m.leaf = leafpos;
    m.sub = sub;
    if(computeNormal && clear)
    {
      m.sn[0] = m.sn[1] = m.sn[2] = 0.0;
      m.npend = 0;
    }
    upd = computeNormal && shared;
  }
  else
    upd = computeNormal && shared && (m.type == ty) && abs_le_eps(sqdist_pp(cp, m.mp));
  if(upd)
  {
    if(m.npend == NPEND) flush_normals<NPC>(m, leaves);
    m.pend[m.npend++] = leafpos * 8 + sub * 4 + (ty == 1 ? 3 : loc);
  }
}

// checkCandidate for one triangle (SD:667-736); sub-triangle `sub` of leaf
// `leafpos` with vertices T.
template <int NPC, bool KEYS = true>
__device__ __forceinline__ void check_triangle(const double* q, MinCand& m, const double* const* T,
                                               const LeafRec<NPC>* __restrict__ leaves, int leafpos, int sub,
                                               bool computeNormal)
{
  double cp[3];
  const int loc = closest_point<KEYS>(q, T[0], T[1], T[2], cp);
  apply_candidate<NPC>(cp, sqdist_pp(q, cp), loc, m, leaves, leafpos, sub, computeNormal);
}

// squared_distance(Point, BoundingBox) (squared_distance.hpp:77-102)
// (its comparisons on the integer pipe, OKey, with the FP64 outcomes; keys
// are formed one axis at a time, so that few stay live)
__device__ __forceinline__ bool box_valid_i(const double* lo, const double* hi)
{
  bool ok = true;
#pragma unroll
  for(int d = 0; d < 3; ++d) ok = ok && !ok_gt(okey(lo[d]), okey(hi[d]));
  return ok;
}
__device__ __forceinline__ double sqdist_pb(const double* p, const double* lo, const double* hi)
{
  if(!box_valid_i(lo, hi)) return DBL_MAX;
  bool out = false;
  double c[3];
#pragma unroll
  for(int d = 0; d < 3; ++d)
  {
    const OKey kp = okey(p[d]);
    const bool below = ok_lt(kp, okey(lo[d])), above = ok_gt(kp, okey(hi[d]));
    out = out || below || above;
    c[d] = below ? lo[d] : above ? hi[d] : p[d];
  }
  if(!out) return 0.0;
  return sqdist_pp(p, c);
}
// The same with FP64 comparisons (fewer registers), for code that runs only
// in converged FP64 batches.
__device__ __forceinline__ double sqdist_pb_d(const double* p, const double* lo, const double* hi)
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

__device__ __forceinline__ void init_min(MinCand& mc)
{
  mc.minSq = DBL_MAX;
  mc.mp[0] = mc.mp[1] = mc.mp[2] = 0.0;
  mc.sn[0] = mc.sn[1] = mc.sn[2] = 0.0;
  mc.type = -1;
  mc.leaf = -1;
  mc.sub = 0;
  mc.npend = 0;
}

// Sign (SD:583-592) and outputs (SD:594-603) of one query.  sign_hint() may
// return the certain outcome of the sign test (+1 or -1; 0 when unknown); it
// is asked only when the sign is needed and no normal is written, and then
// saves the FP64 pseudo-normal.
template <int NPC, class SignHint>
__device__ __forceinline__ void finish_query(const double* q, const MinCand& mc, const LeafRec<NPC>* __restrict__ leaves,
                                             const SdfParams& prm, int idx, double* __restrict__ out,
                                             double* __restrict__ out_cp, double* __restrict__ out_n,
                                             SignHint sign_hint)
{
  // getSurfaceNormal (SD:740-748); the recorded pseudo-normal terms are
  // evaluated only when the normal is used
  double nrm[3] = {mc.sn[0], mc.sn[1], mc.sn[2]};
  const double* D = prm.domain;
  const bool inside_box = !(mc.mp[0] < D[0] || mc.mp[0] > D[3] || mc.mp[1] < D[1] || mc.mp[1] > D[4] ||
                            mc.mp[2] < D[2] || mc.mp[2] > D[5]);
  const bool want_sign = prm.sign && !(prm.watertight && !inside_box);
  const double hint = (want_sign && !out_n) ? sign_hint() : 0.0;
  if(hint == 0.0 && mc.type == 2)
  {
    double v[3 * NPC];
    load_leaf<NPC>(leaves, mc.leaf, v);
    if(NPC == 4 && mc.sub == 1)
      tri_normal(v, v + 6, v + 9, nrm);
    else
      tri_normal(v, v + 3, v + 6, nrm);
  }
  else if(hint == 0.0 && mc.npend > 0 && (want_sign || out_n))
  {
    MinCand m = mc;
    flush_normals<NPC>(m, leaves);
    nrm[0] = m.sn[0], nrm[1] = m.sn[1], nrm[2] = m.sn[2];
  }
  double sgn = 1.0;
  if(hint != 0.0)
    sgn = hint;
  else if(want_sign)
  {
    // computeSign (SD:751-763)
    const double r0 = q[0] - mc.mp[0], r1 = q[1] - mc.mp[1], r2 = q[2] - mc.mp[2];
    sgn = (dot3(r0, r1, r2, nrm[0], nrm[1], nrm[2]) >= 0.0) ? 1.0 : -1.0;
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

template <int NPC>
__device__ __forceinline__ void finish_query(const double* q, const MinCand& mc, const LeafRec<NPC>* __restrict__ leaves,
                                             const SdfParams& prm, int idx, double* __restrict__ out,
                                             double* __restrict__ out_cp, double* __restrict__ out_n)
{
  finish_query<NPC>(q, mc, leaves, prm, idx, out, out_cp, out_n, [] { return 0.0; });
}

// computeSign's outcome (SD:751-763) in FP64, as finish_query forms it when the
// sign is needed (used to audit certified signs).
template <int NPC>
__device__ __forceinline__ double sign64(const double* q, const MinCand& mc, const LeafRec<NPC>* __restrict__ leaves)
{
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
  else if(mc.npend > 0)
  {
    MinCand m = mc;
    flush_normals<NPC>(m, leaves);
    nrm[0] = m.sn[0], nrm[1] = m.sn[1], nrm[2] = m.sn[2];
  }
  const double r0 = q[0] - mc.mp[0], r1 = q[1] - mc.mp[1], r2 = q[2] - mc.mp[2];
  return (dot3(r0, r1, r2, nrm[0], nrm[1], nrm[2]) >= 0.0) ? 1.0 : -1.0;
}

// Leaf action of the reference (the searchMinDist lambda, SD:570-574) on one
// leaf record: checkCandidate for its one or two triangles.
template <int NPC>
__device__ __forceinline__ void check_leaf(const double* q, MinCand& mc, const LeafRec<NPC>* __restrict__ leaves,
                                           int leafpos, bool computeNormal)
{
  double v[3 * NPC];
  load_leaf<NPC>(leaves, leafpos, v);
  const double* T0[3] = {v, v + 3, v + 6};
  check_triangle<NPC>(q, mc, T0, leaves, leafpos, 0, computeNormal);
  if constexpr(NPC == 4)
  {
    const double* T1[3] = {v, v + 6, v + 9};
    check_triangle<NPC>(q, mc, T1, leaves, leafpos, 1, computeNormal);
  }
}

// One node visit of the point traverser in FP64 (bvh_traverse.hpp:93-99 with
// the traversePref of policy/LinearBVH.hpp:75-82): child predicates and, when
// both children pass, whether to swap.
template <bool KEYS = true>
__device__ __forceinline__ void visit_fp64(const NodeRec64* __restrict__ nodes, int cur, const double* q, double minSq,
                                           bool& inL, bool& inR, bool& swap)
{
  const double2* r = reinterpret_cast<const double2*>(nodes + cur);
  // 96 bytes of child boxes; the links are read by the caller
  double b[12];
#pragma unroll
  for(int k = 0; k < 6; ++k)
  {
    const double2 t = __ldg(r + k);
    b[2 * k] = t.x;
    b[2 * k + 1] = t.y;
  }
  if constexpr(KEYS)
  {
    inL = box_valid_i(b, b + 3) ? ok_le(okey(sqdist_pb(q, b, b + 3)), okey(minSq)) : false;
    inR = box_valid_i(b + 6, b + 9) ? ok_le(okey(sqdist_pb(q, b + 6, b + 9)), okey(minSq)) : false;
  }
  else
  {
    inL = box_valid(b, b + 3) ? (sqdist_pb_d(q, b, b + 3) <= minSq) : false;
    inR = box_valid(b + 6, b + 9) ? (sqdist_pb_d(q, b + 6, b + 9) <= minSq) : false;
  }
  swap = false;
  if(inL && inR)
  {
    const double cl[3] = {0.5 * (b[0] + b[3]), 0.5 * (b[1] + b[4]), 0.5 * (b[2] + b[5])};
    const double cr[3] = {0.5 * (b[6] + b[9]), 0.5 * (b[7] + b[10]), 0.5 * (b[8] + b[11])};
    if constexpr(KEYS)
      swap = ok_gt(okey(sqdist_pp(q, cl)), okey(sqdist_pp(q, cr)));
    else
      swap = sqdist_pp(q, cl) > sqdist_pp(q, cr);
  }
}

// bvh_traverse (bvh_traverse.hpp:66-154): stack descent with the reference's
// deferred leaf actions (a found leaf waits until a second one is found or
// the stack runs out).  visit(cur, inL, inR, swap, children) evaluates one
// node and returns its two child links; leaf(leafpos) is the leaf action.
// Returns false on stack overflow.
template <class Visit, class Leaf>
__device__ __forceinline__ bool traverse_point(Visit& visit, Leaf& leaf)
{
  int todo[STACK_SIZE];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0, cur = 0;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      int2 ch;
      bool inL, inR, swap;
      visit(cur, inL, inR, swap, ch);
      if(!inL && !inR)
        cur = (sp >= 0) ? todo[sp--] : BARRIER;
      else
      {
        cur = inL ? ch.x : ch.y;
        int rc = ch.y;
        if(inL && inR)
        {
          if(swap)
          {
            const int tmp = cur;
            cur = rc;
            rc = tmp;
          }
          if(sp + 1 >= STACK_SIZE) return false;
          todo[++sp] = rc;
        }
      }
      if(cur < 0 && !(found < 0))
      {
        found = cur;
        if(cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
      }
    }
    while(found < 0 && found != BARRIER)
    {
      leaf(-found - 1);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
    }
    found = 0;
  }
  return true;
}

}  // namespace sdf
}  // namespace gsq
