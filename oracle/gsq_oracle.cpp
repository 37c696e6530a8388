// CPU restatement ("port") of axom v0.11.0's spatial-query hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and bench.py's CPU-baseline leg call it as the checker or as
// the timed CPU baseline; the product (axom_gb300/, libgsq.so) never links or
// calls it.  Parity of this restatement is pinned against the reference
// itself (oracle/_ref/libaxom_ref.so, built from the reference sources by
// oracle/build_ref.py) and against the committed golden fixtures.
//
// Every routine restates one reference routine, cited by file:line relative to
// the axom source tree.  Floating-point expressions keep the reference's
// operation order; the file is compiled with -ffp-contract=off so that no
// multiply-add is fused (the reference oracle is built the same way).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{
struct Box
{
  double lo[3], hi[3];
};

constexpr double INVALID_MIN = DBL_MAX;   // BoundingBox.hpp:72
constexpr double INVALID_MAX = -DBL_MAX;  // BoundingBox.hpp:73

inline Box invalid_box()
{
  Box b;
  for(int d = 0; d < 3; ++d)
  {
    b.lo[d] = INVALID_MIN;
    b.hi[d] = INVALID_MAX;
  }
  return b;
}

// BoundingBox::isValid  (primal/geometry/BoundingBox.hpp:451-460)
inline bool valid(const Box& b)
{
  for(int d = 0; d < 3; ++d)
    if(b.lo[d] > b.hi[d]) return false;
  return true;
}

// BoundingBox::addPoint  (BoundingBox.hpp:466-482)
inline void add_point(Box& b, const double* p)
{
  for(int d = 0; d < 3; ++d)
  {
    if(p[d] < b.lo[d]) b.lo[d] = p[d];
    if(p[d] > b.hi[d]) b.hi[d] = p[d];
  }
}

// BoundingBox::addBox  (BoundingBox.hpp:487-505)
inline void add_box(Box& acc, const Box& o)
{
  if(valid(acc))
  {
    if(valid(o))
    {
      add_point(acc, o.lo);
      add_point(acc, o.hi);
    }
  }
  else
    acc = o;
}

// BoundingBox::scale + checkAndFixBounds  (BoundingBox.hpp:548-561, 575-585)
inline void scale_box(Box& b, double s)
{
  if(!valid(b)) return;
  const double half = s * 0.5;
  for(int d = 0; d < 3; ++d)
  {
    const double mid = 0.5 * (b.lo[d] + b.hi[d]);
    const double r = (b.hi[d] - b.lo[d]) * half;
    b.lo[d] = mid - r;
    b.hi[d] = mid + r;
  }
  for(int d = 0; d < 3; ++d)
    if(b.lo[d] > b.hi[d]) std::swap(b.lo[d], b.hi[d]);
}

// 10-bit-per-axis Morton interleave (MortonIndex.hpp:446-466 with the
// expandBits loop at 151-159, Ericson's magic-number spread).
inline std::uint32_t spread10(std::uint32_t x)
{
  x = (x | (x << 16)) & 0xFF0000FFu;
  x = (x | (x << 8)) & 0x0F00F00Fu;
  x = (x | (x << 4)) & 0xC30C30C3u;
  x = (x | (x << 2)) & 0x49249249u;
  return x;
}

// morton32_encode  (spin/internal/linear_bvh/build_radix_tree.hpp:48-65)
inline std::uint32_t morton30(const double c[3])
{
  std::int32_t q[3];
  for(int d = 0; d < 3; ++d) q[d] = (std::int32_t)std::fmin(std::fmax(c[d] * 1024.0, 0.0), 1023.0);
  return spread10((std::uint32_t)q[0]) | (spread10((std::uint32_t)q[1]) << 1) |
    (spread10((std::uint32_t)q[2]) << 2);
}

// delta  (build_radix_tree.hpp:265-287)
inline int delta(int a, int b, int inner, const std::uint32_t* codes)
{
  const bool oor = (b < 0 || b > inner);
  const int bb = oor ? 0 : b;
  std::uint32_t x = codes[a] ^ codes[bb];
  const bool tie = (x == 0);
  if(tie) x = std::uint32_t(a) ^ std::uint32_t(bb);
  int c = x == 0 ? 32 : __builtin_clz(x);
  if(tie) c += 32;
  return oor ? -1 : c;
}

struct Tree
{
  int n = 0;                        // number of leaves (after 0/1 padding)
  Box bounds;                       // global bounds of the scaled boxes
  std::vector<std::uint32_t> codes; // sorted Morton codes
  std::vector<int> perm;            // sorted position -> original id (m_leafs)
  std::vector<int> lchild, rchild, parent;
  std::vector<Box> leaf;            // scaled, sorted leaf boxes
  std::vector<Box> inner;           // inner node boxes
  // Final linear layout (policy/LinearBVH.hpp:170-182, 225-266)
  std::vector<Box> nodes;           // 2*(n-1) child boxes
  std::vector<int> children;        // 2*(n-1): 2*c for inner, -(leafpos+1) for leaf
};

// build_radix_tree  (build_radix_tree.hpp:579-611) and emit_bvh_parents
// (policy/LinearBVH.hpp:191-269), for n >= 2 boxes.
void build(Tree& t, const Box* in, int n, double scale)
{
  t.n = n;
  const int inner = n - 1;
  t.leaf.assign(in, in + n);
  for(auto& b : t.leaf) scale_box(b, scale);  // transform_boxes 85-99

  // reduce, SEQ branch (134-141): fold of addBox from an invalid box
  Box gb = invalid_box();
  for(int i = 0; i < n; ++i) add_box(gb, t.leaf[i]);
  t.bounds = gb;

  // get_mcodes  (146-176)
  double minc[3], inv[3];
  for(int d = 0; d < 3; ++d)
  {
    const double ext = gb.hi[d] - gb.lo[d];
    minc[d] = gb.lo[d];
    inv[d] = (std::fabs(ext - 0.0) <= 1.0e-8) ? 0.0 : 1.0 / ext;
  }
  std::vector<std::uint32_t> raw(n);
  for(int i = 0; i < n; ++i)
  {
    double c[3];
    for(int d = 0; d < 3; ++d)
    {
      const double mid = 0.5 * (t.leaf[i].lo[d] + t.leaf[i].hi[d]);
      c[d] = (mid - minc[d]) * inv[d];
    }
    raw[i] = morton30(c);
  }
  // sort_mcodes: stable sort of indices by code, then reorder (242-260)
  t.perm.resize(n);
  std::iota(t.perm.begin(), t.perm.end(), 0);
  std::stable_sort(t.perm.begin(), t.perm.end(), [&](int a, int b) { return raw[a] < raw[b]; });
  t.codes.resize(n);
  std::vector<Box> sorted(n);
  for(int i = 0; i < n; ++i)
  {
    t.codes[i] = raw[t.perm[i]];
    sorted[i] = t.leaf[t.perm[i]];
  }
  t.leaf.swap(sorted);

  // build_tree (290-384): Karras 2012
  const std::uint32_t* mc = t.codes.data();
  t.lchild.assign(inner, 0);
  t.rchild.assign(inner, 0);
  t.parent.assign(2 * n - 1, 0);
  for(int i = 0; i < inner; ++i)
  {
    const int dir = (delta(i, i + 1, inner, mc) - delta(i, i - 1, inner, mc)) < 0 ? -1 : 1;
    const int dmin = delta(i, i - dir, inner, mc);
    int lmax = 2;
    while(delta(i, i + lmax * dir, inner, mc) > dmin) lmax *= 2;
    int l = 0;
    for(int s = lmax / 2; s >= 1; s /= 2)
      if(delta(i, i + (l + s) * dir, inner, mc) > dmin) l += s;
    const int j = i + l * dir;
    const int dnode = delta(i, j, inner, mc);
    int s = 0;
    double div = 2.0;
    for(int st = (int)std::ceil(double(float(l)) / div);; div *= 2, st = (int)std::ceil(double(float(l)) / div))
    {
      if(delta(i, i + (s + st) * dir, inner, mc) > dnode) s += st;
      if(st == 1) break;
    }
    const int split = i + s * dir + std::min(dir, 0);
    if(std::min(i, j) == split)
    {
      t.parent[split + inner] = i;
      t.lchild[i] = split + inner;
    }
    else
    {
      t.parent[split] = i;
      t.lchild[i] = split;
    }
    if(std::max(i, j) == split + 1)
    {
      t.parent[split + inner + 1] = i;
      t.rchild[i] = split + inner + 1;
    }
    else
    {
      t.parent[split + 1] = i;
      t.rchild[i] = split + 1;
    }
    if(i == 0) t.parent[0] = -1;
  }

  // propagate_aabbs (505-576), SEQ order.  Leaves are walked in increasing
  // order and the second visitor of a node continues; that visitor always
  // comes from the right child, so box(node) = addBox(box(right), box(left)).
  t.inner.assign(inner, invalid_box());
  std::vector<int> counter(inner, 0);
  for(int i = 0; i < n; ++i)
  {
    Box acc = t.leaf[i];
    int last = inner + i;
    int cur = t.parent[inner + i];
    while(cur != -1)
    {
      if(counter[cur]++ == 0) break;
      const int other = (t.lchild[cur] == last) ? t.rchild[cur] : t.lchild[cur];
      const Box& ob = (other >= inner) ? t.leaf[other - inner] : t.inner[other];
      add_box(acc, ob);
      t.inner[cur] = acc;
      last = cur;
      cur = t.parent[cur];
    }
  }

  // emit_bvh_parents  (LinearBVH.hpp:225-264)
  t.nodes.resize(2 * inner);
  t.children.resize(2 * inner);
  for(int i = 0; i < inner; ++i)
  {
    int lc = t.lchild[i], rc = t.rchild[i];
    Box lb, rb;
    if(lc >= inner)
    {
      lb = t.leaf[lc - inner];
      lc = -(lc - inner + 1);
    }
    else
    {
      lb = t.inner[lc];
      lc *= 2;
    }
    if(rc >= inner)
    {
      rb = t.leaf[rc - inner];
      rc = -(rc - inner + 1);
    }
    else
    {
      rb = t.inner[rc];
      rc *= 2;
    }
    t.nodes[2 * i] = lb;
    t.nodes[2 * i + 1] = rb;
    t.children[2 * i] = lc;
    t.children[2 * i + 1] = rc;
  }
}

// BVH::initialize  (spin/BVH.hpp:424-477): 0 or 1 boxes are padded to 2, the
// second one invalid.
void initialize(Tree& t, const Box* in, int n, double scale)
{
  if(n <= 1)
  {
    Box pad[2] = {invalid_box(), invalid_box()};
    if(n == 1) pad[0] = in[0];
    build(t, pad, 2, scale);
  }
  else
    build(t, in, n, scale);
}

// bvh_traverse  (spin/internal/linear_bvh/bvh_traverse.hpp:66-154): stack
// descent with deferred leaf actions (two found leaves, then act).
template <typename Pred, typename Leaf, typename Pref>
inline void traverse(const Tree& t, Pred&& B, Leaf&& A, Pref&& Comp)
{
  constexpr int BARRIER = -2000000000;
  int todo[64];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0;
  int cur = 0;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      const Box& L = t.nodes[cur];
      const Box& R = t.nodes[cur + 1];
      const bool inL = valid(L) ? B(L) : false;
      const bool inR = valid(R) ? B(R) : false;
      const int lc = t.children[cur];
      int rc = t.children[cur + 1];
      const bool swp = Comp(L, R);
      if(!inL && !inR)
        cur = todo[sp--];
      else
      {
        cur = inL ? lc : rc;
        if(inL && inR)
        {
          if(swp) std::swap(cur, rc);
          todo[++sp] = rc;
        }
      }
      if(cur < 0 && !(found < 0))
      {
        found = cur;
        if(cur != BARRIER) cur = todo[sp--];
      }
    }
    while(found < 0 && found != BARRIER)
    {
      A(-found - 1);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = todo[sp--];
    }
    found = 0;
  }
}

// ---- geometric primitives (primal) -------------------------------------
inline double dot3(const double* u, const double* v)
{
  // Vector::dot_product (primal/geometry/Vector.hpp:544-553): res starts at 0
  double r = 0.0;
  r += u[0] * v[0];
  r += u[1] * v[1];
  r += u[2] * v[2];
  return r;
}

inline void sub3(const double* h, const double* tl, double* o)
{
  for(int d = 0; d < 3; ++d) o[d] = h[d] - tl[d];
}

// squared_distance(Point, Point)  (primal/operators/squared_distance.hpp:62-67)
inline double sq_dist_pp(const double* a, const double* b)
{
  double v[3];
  sub3(b, a, v);
  return dot3(v, v);
}

// BoundingBox::contains(Point)  (BoundingBox.hpp:388-401)
inline bool contains(const Box& b, const double* p)
{
  for(int d = 0; d < 3; ++d)
    if(p[d] < b.lo[d] || p[d] > b.hi[d]) return false;
  return true;
}

// squared_distance(Point, BoundingBox)  (squared_distance.hpp:77-102)
inline double sq_dist_pb(const double* p, const Box& b)
{
  if(!valid(b)) return DBL_MAX;
  if(contains(b, p)) return 0.0;
  double cp[3];
  for(int d = 0; d < 3; ++d) cp[d] = (p[d] < b.lo[d]) ? b.lo[d] : (p[d] > b.hi[d]) ? b.hi[d] : p[d];
  return sq_dist_pp(p, cp);
}

// fuzzy comparators  (primal/operators/detail/fuzzy_comparators.hpp:24-44)
inline bool near_eq(double a, double b, double eps) { return std::fabs(a - b) <= eps; }
inline bool is_leq(double x, double y, double eps) { return !((x > y) && !near_eq(x, y, eps)); }
inline bool is_geq(double x, double y, double eps) { return !((x < y) && !near_eq(x, y, eps)); }

// closest_point(Point, Triangle, loc, EPS)  (primal/operators/closest_point.hpp:162-290)
inline void closest_point(const double* P, const double* A, const double* B, const double* C, double eps,
                          double* out, int* loc)
{
  double ab[3], ac[3], ap[3];
  sub3(B, A, ab);
  sub3(C, A, ac);
  sub3(P, A, ap);
  const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if(is_leq(d1, 0.0, eps) && is_leq(d2, 0.0, eps))
  {
    *loc = 0;
    std::memcpy(out, A, 24);
    return;
  }
  double bp[3];
  sub3(P, B, bp);
  const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if(is_geq(d3, 0.0, eps) && is_leq(d4, d3, eps))
  {
    *loc = 1;
    std::memcpy(out, B, 24);
    return;
  }
  const double vc = d1 * d4 - d3 * d2;
  if(is_leq(vc, 0.0, eps) && is_geq(d1, 0.0, eps) && is_leq(d3, 0.0, eps) && !near_eq(d1, d3, eps))
  {
    const double v = d1 / (d1 - d3);
    for(int d = 0; d < 3; ++d) out[d] = A[d] + ab[d] * v;
    *loc = -1;
    return;
  }
  double cpv[3];
  sub3(P, C, cpv);
  const double d5 = dot3(ab, cpv), d6 = dot3(ac, cpv);
  if(is_geq(d6, 0.0, eps) && is_leq(d5, d6, eps))
  {
    *loc = 2;
    std::memcpy(out, C, 24);
    return;
  }
  const double vb = d5 * d2 - d1 * d6;
  if(is_leq(vb, 0.0, eps) && is_geq(d2, 0.0, eps) && is_leq(d6, 0.0, eps))
  {
    const double w = d2 / (d2 - d6);
    for(int d = 0; d < 3; ++d) out[d] = A[d] + ac[d] * w;
    *loc = -3;
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if(is_leq(va, 0.0, eps) && is_geq(d4 - d3, 0.0, eps) && is_geq(d5 - d6, 0.0, eps))
  {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    double bc[3];
    sub3(C, B, bc);
    for(int d = 0; d < 3; ++d) out[d] = B[d] + bc[d] * w;
    *loc = -2;
    return;
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom, w = vc * denom;
  for(int d = 0; d < 3; ++d)
  {
    const double nd = ab[d] * v + ac[d] * w;
    out[d] = A[d] + nd;
  }
  *loc = 3;
}

// Vector::cross_product  (Vector.hpp:563-570) via numerics::determinant
inline void cross3(const double* u, const double* v, double* o)
{
  o[0] = u[1] * v[2] - v[1] * u[2];
  o[1] = v[0] * u[2] - u[0] * v[2];
  o[2] = u[0] * v[1] - v[0] * u[1];
}

// Triangle::normal  (primal/geometry/Triangle.hpp:98-102)
inline void tri_normal(const double* A, const double* B, const double* C, double* n)
{
  double u[3], v[3];
  sub3(B, A, u);
  sub3(C, A, v);
  cross3(u, v, n);
}

// Vector::unitVector  (Vector.hpp:477-493), PRIMAL_TINY = 1e-50
inline void unit3(const double* v, double* o)
{
  const double l2 = dot3(v, v);
  if(l2 >= 1e-50)
  {
    const double s = 1.0 / std::sqrt(l2);
    for(int d = 0; d < 3; ++d) o[d] = v[d] * s;
  }
  else
  {
    o[0] = 1.0;
    o[1] = 0.0;
    o[2] = 0.0;
  }
}

// Triangle::angle  (Triangle.hpp:385-400)
inline double tri_angle(const double* const* P, int idx)
{
  const double* pt = P[idx];
  double a[3], b[3], u1[3], u2[3];
  sub3(P[(idx + 1) % 3], pt, a);
  sub3(P[(idx + 2) % 3], pt, b);
  unit3(a, u1);
  unit3(b, u2);
  double dp = dot3(u1, u2);
  dp = (dp < -1.0) ? -1.0 : (dp > 1.0) ? 1.0 : dp;
  return std::acos(dp);
}

// Triangle::degenerate  (Triangle.hpp:327-330) with area (Triangle.hpp:105-109)
inline bool tri_degenerate(const double* A, const double* B, const double* C)
{
  double n[3];
  tri_normal(A, B, C, n);
  const double area = 0.5 * std::sqrt(dot3(n, n));
  return near_eq(area, 0.0, 1.0e-12);
}

struct Mesh
{
  std::vector<double> x, y, z;
  std::vector<int> cells;
  int npc = 3;  // nodes per cell: 3 (triangle) or 4 (quad)
  int ncells = 0;
  bool watertight = true, sign = true;
  Box domain;
  Tree tree;
  void node(int i, double* p) const
  {
    p[0] = x[i];
    p[1] = y[i];
    p[2] = z[i];
  }
};

// MinCandidate  (quest/SignedDistance.hpp:159-175)
struct MinCand
{
  double minSq = DBL_MAX;
  double minPt[3] = {0, 0, 0};
  int minType = -1;  // -1 uninitialized, 0 vertex, 1 edge, 2 face
  int minElem = 0;
  double tri[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double sumN[3] = {0, 0, 0};
  int count = 0;
};

// getClosestPointLocType  (SignedDistance.hpp:119-137)
inline int loc_type(int loc) { return (loc < 0) ? 1 : (loc <= 2) ? 0 : 2; }

// checkCandidate  (SignedDistance.hpp:636-737)
inline void check_candidate(const double* q, MinCand& m, int cell, const Mesh& M, bool computeNormal)
{
  const int* nodes = &M.cells[(long long)cell * M.npc];
  double P[4][3];
  for(int k = 0; k < M.npc; ++k) M.node(nodes[k], P[k]);
  const int ntri = (M.npc == 4) ? 2 : 1;
  const double* tris[2][3] = {{P[0], P[1], P[2]}, {P[0], P[2], P[3]}};
  for(int e = 0; e < ntri; ++e)
  {
    const double* const* T = tris[e];
    int loc;
    double cp[3];
    closest_point(q, T[0], T[1], T[2], 1e-12, cp, &loc);
    const double sq = sq_dist_pp(q, cp);
    const int ty = loc_type(loc);
    const bool shared = (ty != 2);
    bool upd = false;
    if(sq < m.minSq)
    {
      const bool clear = !shared || (m.minType != ty) || !near_eq(sq_dist_pp(cp, m.minPt), 0.0, 1e-12);
      m.minSq = sq;
      std::memcpy(m.minPt, cp, 24);
      m.minType = ty;
      m.minElem = cell;
      for(int k = 0; k < 3; ++k) std::memcpy(m.tri[k], T[k], 24);
      if(computeNormal && clear)
      {
        m.sumN[0] = m.sumN[1] = m.sumN[2] = 0.0;
        m.count = 0;
      }
      upd = computeNormal && shared;
    }
    else
      upd = computeNormal && shared && (m.minType == ty) && near_eq(sq_dist_pp(cp, m.minPt), 0.0, 1e-12);
    if(upd)
    {
      ++m.count;
      double n[3], u[3];
      if(ty == 1)
      {
        tri_normal(T[0], T[1], T[2], n);
        unit3(n, u);
        for(int d = 0; d < 3; ++d) m.sumN[d] += u[d];
      }
      else if(ty == 0)
      {
        if(!tri_degenerate(T[0], T[1], T[2]))
        {
          const double alpha = tri_angle(T, loc);
          tri_normal(T[0], T[1], T[2], n);
          unit3(n, u);
          for(int d = 0; d < 3; ++d) m.sumN[d] += u[d] * alpha;
        }
      }
    }
  }
}

// getSurfaceNormal  (SignedDistance.hpp:740-748)
inline void surface_normal(const MinCand& m, double* n)
{
  if(m.minType == 2)
    tri_normal(m.tri[0], m.tri[1], m.tri[2], n);
  else
    std::memcpy(n, m.sumN, 24);
}

// computeDistances per-point body  (SignedDistance.hpp:563-604), with the
// point traverser's nearer-centroid-first preference (policy/LinearBVH.hpp:72-85).
inline void sdf_point(const Mesh& M, const double* q, double* out, double* cpo, double* no, int* nb, int* nl)
{
  MinCand m;
  int boxes = 0, leaves = 0;
  auto pred = [&](const Box& bb) {
    ++boxes;
    return sq_dist_pb(q, bb) <= m.minSq;
  };
  auto leaf = [&](int leafpos) {
    ++leaves;
    check_candidate(q, m, M.tree.perm[leafpos], M, M.sign);
  };
  auto pref = [&](const Box& l, const Box& r) {
    double cl[3], cr[3];
    for(int d = 0; d < 3; ++d) cl[d] = 0.5 * (l.lo[d] + l.hi[d]);
    const double sl = sq_dist_pp(q, cl);
    double sr = DBL_MAX;
    if(valid(r))
    {
      for(int d = 0; d < 3; ++d) cr[d] = 0.5 * (r.lo[d] + r.hi[d]);
      sr = sq_dist_pp(q, cr);
    }
    return sl > sr;
  };
  traverse(M.tree, pred, leaf, pref);
  double sgn = 1.0;
  if(M.sign)
  {
    if(!(M.watertight && !contains(M.domain, m.minPt)))
    {
      double n[3], r[3];
      surface_normal(m, n);
      sub3(q, m.minPt, r);
      sgn = (dot3(r, n) >= 0.0) ? 1.0 : -1.0;
    }
  }
  *out = std::sqrt(m.minSq) * sgn;
  if(cpo) std::memcpy(cpo, m.minPt, 24);
  if(no)
  {
    double n[3];
    surface_normal(m, n);
    unit3(n, no);
  }
  if(nb) *nb = boxes;
  if(nl) *nl = leaves;
}

inline Box read_box(const double* b)
{
  Box o;
  for(int d = 0; d < 3; ++d)
  {
    o.lo[d] = b[d];
    o.hi[d] = b[3 + d];
  }
  return o;
}

inline void write_box(const Box& b, double* o)
{
  for(int d = 0; d < 3; ++d)
  {
    o[d] = b.lo[d];
    o[3 + d] = b.hi[d];
  }
}

template <typename Pred>
long long find_candidates(const Tree& t, int m, Pred&& pred_of, int* offsets, int* counts, int** cands)
{
  // findCandidatesImpl, single-pass SEQ branch  (policy/LinearBVH.hpp:368-401)
  std::vector<int> out;
  long long cur = 0;
  for(int i = 0; i < m; ++i)
  {
    offsets[i] = (int)cur;
    int c = 0;
    auto pred = pred_of(i);
    traverse(
      t, pred,
      [&](int leafpos) {
        out.push_back(t.perm[leafpos]);
        ++c;
        ++cur;
      },
      [](const Box&, const Box&) { return false; });
    counts[i] = c;
  }
  *cands = static_cast<int*>(std::malloc(sizeof(int) * (out.empty() ? 1 : out.size())));
  if(!out.empty()) std::memcpy(*cands, out.data(), sizeof(int) * out.size());
  return (long long)out.size();
}

}  // namespace orc

using namespace orc;

extern "C" {

void orc_free(void* p) { std::free(p); }

void* orc_bvh_create(const double* boxes, int n, double scale)
{
  auto* t = new Tree();
  std::vector<Box> in(n > 0 ? n : 0);
  for(int i = 0; i < n; ++i) in[i] = read_box(boxes + 6 * i);
  initialize(*t, in.data(), n, scale);
  return t;
}

void orc_bvh_destroy(void* h) { delete static_cast<Tree*>(h); }

void orc_bvh_bounds(void* h, double* out6) { write_box(static_cast<Tree*>(h)->bounds, out6); }

int orc_bvh_size(void* h) { return static_cast<Tree*>(h)->n; }

// Final linear layout: nodes[2(n-1)*6], children[2(n-1)], leaf ids[n].
void orc_bvh_layout(void* h, double* nodes, int* children, int* leaf_ids)
{
  const Tree& t = *static_cast<Tree*>(h);
  for(size_t i = 0; i < t.nodes.size(); ++i) write_box(t.nodes[i], nodes + 6 * i);
  std::memcpy(children, t.children.data(), sizeof(int) * t.children.size());
  std::memcpy(leaf_ids, t.perm.data(), sizeof(int) * t.perm.size());
}

int orc_bvh_internals(const double* boxes, int n, double scale, std::uint32_t* codes, int* perm, int* lchild,
                      int* rchild, int* parents, double* inner, double* leaf, double* bounds)
{
  if(n < 2) return -1;
  Tree t;
  std::vector<Box> in(n);
  for(int i = 0; i < n; ++i) in[i] = read_box(boxes + 6 * i);
  build(t, in.data(), n, scale);
  std::memcpy(codes, t.codes.data(), 4 * n);
  std::memcpy(perm, t.perm.data(), 4 * n);
  std::memcpy(lchild, t.lchild.data(), 4 * (n - 1));
  std::memcpy(rchild, t.rchild.data(), 4 * (n - 1));
  std::memcpy(parents, t.parent.data(), 4 * (2 * n - 1));
  for(int i = 0; i < n - 1; ++i) write_box(t.inner[i], inner + 6 * i);
  for(int i = 0; i < n; ++i) write_box(t.leaf[i], leaf + 6 * i);
  write_box(t.bounds, bounds);
  return 0;
}

long long orc_bvh_find_boxes(void* h, const double* q, int m, int* offsets, int* counts, int** cands)
{
  const Tree& t = *static_cast<Tree*>(h);
  return find_candidates(
    t, m,
    [&](int i) {
      const Box qb = read_box(q + 6 * i);
      // BoundingBox::intersectsWith + intersect_bbox_bbox (BoundingBox.hpp:432-447,
      // primal/operators/detail/intersect_bounding_box_impl.hpp:35-41)
      return [qb](const Box& bb) {
        for(int d = 0; d < 3; ++d)
          if(!(qb.hi[d] >= bb.lo[d] && qb.lo[d] <= bb.hi[d])) return false;
        return true;
      };
    },
    offsets, counts, cands);
}

// findBoundingBoxes from nthreads threads over contiguous sub-ranges of the
// queries (each range as the SEQ branch does it), concatenated in query order:
// the same CSR as orc_bvh_find_boxes.
long long orc_bvh_find_boxes_mt(void* h, const double* q, int m, int* offsets, int* counts, int** cands,
                                int nthreads)
{
  if(nthreads < 1) nthreads = 1;
  std::vector<int*> part(nthreads, nullptr);
  std::vector<long long> size(nthreads, 0), lo(nthreads + 1, 0);
  for(int t = 0; t <= nthreads; ++t) lo[t] = (long long)m * t / nthreads;
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
  for(int t = 0; t < nthreads; ++t)
    size[t] = orc_bvh_find_boxes(h, q + 6 * lo[t], int(lo[t + 1] - lo[t]), offsets + lo[t], counts + lo[t], &part[t]);
  long long total = 0;
  for(int t = 0; t < nthreads; ++t) total += size[t];
  *cands = static_cast<int*>(std::malloc(sizeof(int) * (total ? total : 1)));
  long long at = 0;
  for(int t = 0; t < nthreads; ++t)
  {
    for(long long i = lo[t]; i < lo[t + 1]; ++i) offsets[i] += (int)at;
    if(size[t]) std::memcpy(*cands + at, part[t], sizeof(int) * size[t]);
    at += size[t];
    std::free(part[t]);
  }
  return total;
}

// Instrumented findBoundingBoxes: per query, the number of box-predicate calls
// of the traversal (the roofline numerator counts N_node = calls / 2).
void orc_bvh_find_boxes_counts(void* h, const double* q, int m, int* box_tests)
{
  const Tree& t = *static_cast<Tree*>(h);
  for(int i = 0; i < m; ++i)
  {
    const Box qb = read_box(q + 6 * i);
    int nb = 0;
    auto pred = [&](const Box& bb) {
      ++nb;
      for(int d = 0; d < 3; ++d)
        if(!(qb.hi[d] >= bb.lo[d] && qb.lo[d] <= bb.hi[d])) return false;
      return true;
    };
    traverse(t, pred, [](int) {}, [](const Box&, const Box&) { return false; });
    box_tests[i] = nb;
  }
}

long long orc_bvh_find_points(void* h, const double* p, int m, int* offsets, int* counts, int** cands)
{
  const Tree& t = *static_cast<Tree*>(h);
  return find_candidates(
    t, m,
    [&](int i) {
      const double* pt = p + 3 * i;
      return [pt](const Box& bb) { return contains(bb, pt); };
    },
    offsets, counts, cands);
}

// primal::Ray stores a unit direction (Ray.hpp:123-128); this restates the
// normalisation so callers can build the stored directions.
void orc_ray_normalize(const double* d, int m, double* out)
{
  for(int i = 0; i < m; ++i) unit3(d + 3 * i, out + 3 * i);
}

// dirs are the rays' stored (unit) directions.
long long orc_bvh_find_rays(void* h, const double* o, const double* dirs, int m, double tol, int* offsets,
                            int* counts, int** cands)
{
  const Tree& t = *static_cast<Tree*>(h);
  return find_candidates(
    t, m,
    [&](int i) {
      const double* x0 = o + 3 * i;
      const double* n = dirs + 3 * i;
      // intersect_ray(Ray, BoundingBox, Point&, EPS) and intersect_ray_bbox_test
      // (primal/operators/detail/intersect_ray_impl.hpp:151-186, 321-351)
      return [x0, n, tol](const Box& bb) {
        double tmin = DBL_MIN, tmax = DBL_MAX;
        for(int d = 0; d < 3; ++d)
        {
          bool ok;
          if(std::fabs(n[d] - 0.0) <= tol)
            ok = !((x0[d] < bb.lo[d]) || (x0[d] > bb.hi[d]));
          else
          {
            const double inv = 1.0 / n[d];
            double t1 = (bb.lo[d] - x0[d]) * inv;
            double t2 = (bb.hi[d] - x0[d]) * inv;
            if(t1 > t2) std::swap(t1, t2);
            tmin = (t1 < tmin) ? tmin : t1;
            tmax = (t2 < tmax) ? t2 : tmax;
            ok = !(tmin > tmax);
          }
          if(!ok) return false;
        }
        return true;
      };
    },
    offsets, counts, cands);
}

// SignedDistance ctor / setMesh  (quest/SignedDistance.hpp:410-504)
void* orc_sdf_create(const double* x, const double* y, const double* z, int nverts, const int* cells, int ncells,
                     int nodes_per_cell, int watertight, int compute_sign)
{
  auto* M = new Mesh();
  M->x.assign(x, x + nverts);
  M->y.assign(y, y + nverts);
  M->z.assign(z, z + nverts);
  M->npc = nodes_per_cell;
  M->ncells = ncells;
  M->cells.assign(cells, cells + (long long)ncells * nodes_per_cell);
  M->watertight = watertight != 0;
  M->sign = compute_sign != 0;
  M->domain = invalid_box();
  for(int i = 0; i < nverts; ++i)
  {
    double p[3];
    M->node(i, p);
    add_point(M->domain, p);
  }
  std::vector<Box> boxes(ncells);
  for(int c = 0; c < ncells; ++c)  // getCellBoundingBox (SignedDistance.hpp:608-633)
  {
    Box b = invalid_box();
    for(int k = 0; k < nodes_per_cell; ++k)
    {
      double p[3];
      M->node(M->cells[(long long)c * nodes_per_cell + k], p);
      add_point(b, p);
    }
    boxes[c] = b;
  }
  initialize(M->tree, boxes.data(), ncells, 1.000123);  // BVH.hpp:410
  return M;
}

void orc_sdf_destroy(void* h) { delete static_cast<Mesh*>(h); }

void* orc_sdf_tree(void* h) { return &static_cast<Mesh*>(h)->tree; }

void orc_sdf_mesh_bounds(void* h, double* out6) { write_box(static_cast<Mesh*>(h)->domain, out6); }

void orc_sdf_eval(void* h, const double* q, int m, double* out, double* cp, double* normals, int nthreads)
{
  const Mesh& M = *static_cast<Mesh*>(h);
  if(nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
  for(int i = 0; i < m; ++i)
    sdf_point(M, q + 3 * (long long)i, out + i, cp ? cp + 3 * (long long)i : nullptr,
              normals ? normals + 3 * (long long)i : nullptr, nullptr, nullptr);
}

void orc_sdf_counts(void* h, const double* q, int m, int* box_tests, int* leaf_tests, int nthreads)
{
  const Mesh& M = *static_cast<Mesh*>(h);
  if(nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
  for(int i = 0; i < m; ++i)
  {
    double d;
    sdf_point(M, q + 3 * (long long)i, &d, nullptr, nullptr, box_tests + i, leaf_tests + i);
  }
}

// ---- closest object point (DistributedClosestPoint's local query) ----------
// The object points, one degenerate box each (BoxType{point},
// quest/detail/DistributedClosestPointImpl.hpp:883-901), in a BVH with the
// default scale factor.
struct PointCloud
{
  Tree tree;
  std::vector<double> xyz;
  std::vector<int> dom;
};

void* orc_cp_create(const double* pts, int n, const int* domains)
{
  auto* P = new PointCloud();
  P->xyz.assign(pts, pts + 3 * (long long)std::max(n, 0));
  P->dom.resize(std::max(n, 0));
  for(int i = 0; i < n; ++i) P->dom[i] = domains ? domains[i] : 0;
  std::vector<Box> boxes(std::max(n, 0));
  for(int i = 0; i < n; ++i)
    for(int d = 0; d < 3; ++d) boxes[i].lo[d] = boxes[i].hi[d] = pts[3 * (long long)i + d];
  initialize(P->tree, boxes.data(), n, 1.000123);  // BVH.hpp:410
  return P;
}

void orc_cp_destroy(void* h) { delete static_cast<PointCloud*>(h); }

// computeLocalClosestPoints per query point with no earlier candidate
// (DistributedClosestPointImpl.hpp:1002-1050): the point traverser (nearer
// centroid first, LinearBVH.hpp:72-85), a branch is entered when its box is
// within both the best squared distance so far and the threshold, and a point
// replaces the best only if strictly closer.  Not found: index and domain -1,
// position and distance NaN.
void orc_cp_query(void* h, const double* q, int m, double sq_threshold, int* idx, int* dom, double* pos, double* dist,
                  int nthreads)
{
  const PointCloud& P = *static_cast<PointCloud*>(h);
  if(nthreads < 1) nthreads = 1;
  const double nan = std::numeric_limits<double>::quiet_NaN();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
  for(int i = 0; i < m; ++i)
  {
    const double* p = q + 3 * (long long)i;
    double best = DBL_MAX;
    int bi = -1, bd = -1;
    auto pred = [&](const Box& bb) {
      const double sq = sq_dist_pb(p, bb);
      return sq <= best && sq <= sq_threshold;
    };
    auto leaf = [&](int leafpos) {
      const int c = P.tree.perm[leafpos];
      if(c >= (int)P.dom.size()) return;  // padding of a 0/1-point cloud
      const double sq = sq_dist_pp(p, &P.xyz[3 * (long long)c]);
      if(sq < best)
      {
        best = sq;
        bi = c;
        bd = P.dom[c];
      }
    };
    auto pref = [&](const Box& l, const Box& r) {
      double cl[3], cr[3];
      for(int d = 0; d < 3; ++d) cl[d] = 0.5 * (l.lo[d] + l.hi[d]);
      const double sl = sq_dist_pp(p, cl);
      double sr = DBL_MAX;
      if(valid(r))
      {
        for(int d = 0; d < 3; ++d) cr[d] = 0.5 * (r.lo[d] + r.hi[d]);
        sr = sq_dist_pp(p, cr);
      }
      return sl > sr;
    };
    traverse(P.tree, pred, leaf, pref);
    idx[i] = bi;
    dom[i] = bd;
    for(int d = 0; d < 3; ++d) pos[3 * (long long)i + d] = (bi >= 0) ? P.xyz[3 * (long long)bi + d] : nan;
    dist[i] = (bi >= 0) ? std::sqrt(best) : nan;
  }
}

}  // extern "C"
