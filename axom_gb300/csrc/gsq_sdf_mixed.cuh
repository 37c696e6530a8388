// FP32 records and the certified traversal of the mixed-precision signed
// distance, shared by the mixed query kernel and the adjoint kernel.
#pragma once

#include "gsq_sdf_device.cuh"
#include "gsq_sign.cuh"

namespace gsq
{
template <int NPC>
struct LeafRec32;
// FP32 triangle(s) of one leaf: vertices rounded to nearest, and per
// triangle the error factor ec = 256 * 2^-24 * kappa and max edge length lt
// (triangles also carry fz, the bound on the reference's fuzzy closest-point
// displacement; quads compute it from ec and lt).
template <>
struct __align__(16) LeafRec32<3>
{
  float v[9];
  float ec;
  float lt;
  float fz;
};
template <>
struct __align__(16) LeafRec32<4>
{
  float v[12];
  float ec[2];
  float lt[2];
};
static_assert(sizeof(LeafRec32<3>) == 48, "fp32 triangle leaf is 48 bytes");
static_assert(sizeof(LeafRec32<4>) == 64, "fp32 quad leaf is 64 bytes");

// Per-mesh entry of a query launch: where the mesh's node and leaf records
// start in the shared arrays, its node box and coordinate bound.
struct MeshInfo
{
  long long node_off;
  long long leaf_off;
  double domain[6];
  float mesh_max;
  int pad;
};

namespace sdf
{
// FP32 dot product with fused operations (one rounding per multiply-add):
// the error bounds used with these FP32 evaluations count at least one
// rounding per operation, which fused operations meet.
__device__ __forceinline__ float dot3f(float a0, float b0, float a1, float b1, float a2, float b2)
{
  return __fmaf_rn(a2, b2, __fmaf_rn(a1, b1, a0 * b0));
}

// True when every fuzzy comparison of the reference's closest_point
// (closest_point.hpp:181-282: d1..d6, d4 - d3, d5 - d6, d1 - d3 and vc, vb, va
// against 0 with EPS = 1e-12) certainly has the outcome of the exact
// comparison.  The reference's point is then the exact closest point up to
// FP64 rounding, and its fuzzy displacement bound is not needed.
// Q bounds |q| per coordinate, M the mesh's coordinates.  Every dot is of an
// edge e (ab or ac: two vertices rounded to FP32, then subtracted) and an
// offset p (ap, bp or cp: the rounded point minus a rounded vertex).  Per
// coordinate, e is within 2^-23 M + 2^-24 |e_d| of the exact edge and p within
// 2^-24 (Q + M) + 2^-24 |p_d| of the exact offset (to a factor 1 + 2^-23), and
// the fused dot rounds three times, so with E1 = max |e|_1, P1 = max |p|_1
//   err_d = 1.02 (2^-23 M P1 + 2^-24 (Q + M) E1 + 5 2^-24 E1 P1 + 2^-44 (Q + M)^2)
// bounds every dot's error (the last term: products of two coordinate
// errors); a product difference a b - c d is then within 4 D err_d + 2 err_d^2
// + 2^-22 D^2 (D the largest |d| plus err_d), a difference of two dots within
// 2 err_d + 2^-23 D.  Each value must exceed twice its bound plus 2 EPS: then
// the FP64 value, whose own rounding error is below 2^-28 of the FP32 bound,
// is beyond EPS with the exact value's sign, and so is the exact value for the
// rounded inputs (the FP32 region is the exact region for both).
__device__ __forceinline__ bool crisp_regions(const float* P, const float* A, const float* B, const float* C, float Q,
                                              float M)
{
  constexpr float EPS = 1e-12f;
  const float ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const float ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const float ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const float bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const float cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const float d1 = dot3f(ab0, ap0, ab1, ap1, ab2, ap2);
  const float d2 = dot3f(ac0, ap0, ac1, ap1, ac2, ap2);
  const float d3 = dot3f(ab0, bp0, ab1, bp1, ab2, bp2);
  const float d4 = dot3f(ac0, bp0, ac1, bp1, ac2, bp2);
  const float d5 = dot3f(ab0, cp0, ab1, cp1, ab2, cp2);
  const float d6 = dot3f(ac0, cp0, ac1, cp1, ac2, cp2);
  const float vc = __fmaf_rn(d1, d4, -(d3 * d2));
  const float vb = __fmaf_rn(d5, d2, -(d1 * d6));
  const float va = __fmaf_rn(d3, d6, -(d5 * d4));
  auto n1 = [](float x, float y, float z) { return fabsf(x) + fabsf(y) + fabsf(z); };
  const float E1 = fmaxf(n1(ab0, ab1, ab2), n1(ac0, ac1, ac2));
  const float P1 = fmaxf(n1(ap0, ap1, ap2), fmaxf(n1(bp0, bp1, bp2), n1(cp0, cp1, cp2)));
  const float QM = __fadd_ru(Q, M);
  const float err_d =
      __fmul_ru(1.02f, __fadd_ru(__fadd_ru(__fmul_ru(0x1p-23f * M, P1), __fmul_ru(0x1p-24f * QM, E1)),
                                 __fadd_ru(__fmul_ru(5.f * 0x1p-24f, __fmul_ru(E1, P1)),
                                           __fmul_ru(0x1p-44f * QM, QM))));
  const float D = __fadd_ru(fmaxf(fmaxf(fmaxf(fabsf(d1), fabsf(d2)), fmaxf(fabsf(d3), fabsf(d4))),
                                  fmaxf(fabsf(d5), fabsf(d6))),
                            err_d);
  const float err_v = __fmul_ru(1.01f, __fadd_ru(__fadd_ru(__fmul_ru(4.f * D, err_d), 2.f * err_d * err_d),
                                                 __fmul_ru(0x1p-22f, __fmul_ru(D, D))));
  const float err_s = __fmul_ru(1.01f, __fadd_ru(2.f * err_d, __fmul_ru(0x1p-23f, D)));
  auto clear = [&](float x, float e) { return fabsf(x) > __fadd_ru(2.f * e, 2.f * EPS); };
  return clear(d1, err_d) && clear(d2, err_d) && clear(d3, err_d) && clear(d4, err_d) && clear(d5, err_d) &&
         clear(d6, err_d) && clear(d4 - d3, err_s) && clear(d5 - d6, err_s) && clear(d1 - d3, err_s) &&
         clear(vc, err_v) && clear(vb, err_v) && clear(va, err_v);
}

// Squared point-triangle distance in FP32 by Voronoi regions (Ericson,
// Real-Time Collision Detection 5.1.5), measured from P; off receives P - cp,
// the offset from the closest point.  The region tests run in Ericson's order
// and each region keeps its formula, but the results are selected instead of
// branched to, so that the lanes of a warp testing different triangles do not
// diverge.  One division serves every region (its operands are selected); the
// offset is base - v e1 - w e2 with fused operations.  kind receives the
// region: 0 a vertex, 1 the edge AB or AC, 2 the edge BC or the face.
__device__ __forceinline__ float dist2_f32_flat(const float* P, const float* A, const float* B, const float* C,
                                               float* off, int& kind)
{
  const float ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const float ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const float bc0 = C[0] - B[0], bc1 = C[1] - B[1], bc2 = C[2] - B[2];
  const float ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const float bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const float cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const float d1 = dot3f(ab0, ap0, ab1, ap1, ab2, ap2);
  const float d2 = dot3f(ac0, ap0, ac1, ap1, ac2, ap2);
  const float d3 = dot3f(ab0, bp0, ab1, bp1, ab2, bp2);
  const float d4 = dot3f(ac0, bp0, ac1, bp1, ac2, bp2);
  const float d5 = dot3f(ab0, cp0, ab1, cp1, ab2, cp2);
  const float d6 = dot3f(ac0, cp0, ac1, cp1, ac2, cp2);
  const float vc = __fmaf_rn(d1, d4, -(d3 * d2));
  const float vb = __fmaf_rn(d5, d2, -(d1 * d6));
  const float va = __fmaf_rn(d3, d6, -(d5 * d4));
  const bool rA = d1 <= 0.f && d2 <= 0.f;
  const bool rB = !rA && d3 >= 0.f && d4 <= d3;
  const bool rAB = !rA && !rB && vc <= 0.f && d1 >= 0.f && d3 <= 0.f;
  const bool rC = !rA && !rB && !rAB && d6 >= 0.f && d5 <= d6;
  const bool rAC = !rA && !rB && !rAB && !rC && vb <= 0.f && d2 >= 0.f && d6 <= 0.f;
  const bool rBC = !rA && !rB && !rAB && !rC && !rAC && va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f;
  const bool rF = !rA && !rB && !rAB && !rC && !rAC && !rBC;
  kind = (rA || rB || rC) ? 0 : (rAB || rAC) ? 1 : 2;
  const float num = rAB ? d1 : rAC ? d2 : rBC ? (d4 - d3) : 1.f;
  const float den = rAB ? (d1 - d3) : rAC ? (d2 - d6) : rBC ? ((d4 - d3) + (d5 - d6)) : rF ? (va + vb + vc) : 1.f;
  const float t = num / den;
  const float v = rAB ? t : rF ? vb * t : 0.f;
  const float w = (rAC || rBC) ? t : rF ? vc * t : 0.f;
  // base and directions per region: A, AB, AC, face from A; B, BC from B; C from C
  const bool fromB = rB || rBC, fromC = rC;
  const float b0 = fromB ? bp0 : fromC ? cp0 : ap0, b1 = fromB ? bp1 : fromC ? cp1 : ap1,
              b2 = fromB ? bp2 : fromC ? cp2 : ap2;
  const float e0 = rBC ? bc0 : ac0, e1 = rBC ? bc1 : ac1, e2 = rBC ? bc2 : ac2;
  off[0] = __fmaf_rn(-w, e0, __fmaf_rn(-v, ab0, b0));
  off[1] = __fmaf_rn(-w, e1, __fmaf_rn(-v, ab1, b1));
  off[2] = __fmaf_rn(-w, e2, __fmaf_rn(-v, ab2, b2));
  return dot3f(off[0], off[0], off[1], off[1], off[2], off[2]);
}

// Per-query constants of the FP32 certificates.
struct QCtx
{
  float qf[3];           // the point rounded to nearest
  float eq;              // bound on the point's rounding (per axis)
  float lip;             // coordinate-rounding part of the triangle distance error
  float t_true, t_false; // box predicate thresholds from the interval holding minSq
  float thr_leaf;        // sqrt(upper end of that interval) + 1e-6, rounded up
};

__device__ __forceinline__ void qctx_init(QCtx& c, const double* q, float mesh_max)
{
  float qabs = 0.f;
  for(int d = 0; d < 3; ++d)
  {
    c.qf[d] = __double2float_rn(q[d]);
    qabs = fmaxf(qabs, fabsf(c.qf[d]));
  }
  // |qf - q| <= 2^-24 |qf| (round to nearest; the absolute term covers
  // subnormals); the subtraction in a gap is exact or contributes at most
  // 2^-24 of the gap, which the relative term of box_decide covers
  c.eq = __fadd_ru(__fmul_ru(0x1p-24f, qabs), 0x1p-149f);
  // the point-triangle distance is 1-Lipschitz in the point and the vertices
  c.lip = __fmul_ru(0x1p-21f, __fadd_ru(qabs, mesh_max));
}

// Thresholds for an exact minimum known to lie in the FP32 interval [lo, hi]:
// t_true <= minSq (1 - 2^-40) and t_false >= minSq (1 + 2^-40) with room for
// the FP64 predicate's own rounding; thr_leaf >= sqrt(minSq) + 1e-6.  No FP64
// arithmetic.
__device__ __forceinline__ void qctx_set32(QCtx& c, float lo, float hi)
{
  c.t_true = __fmul_rd(lo, 1.f - 0x1p-22f);
  c.t_false = __fmul_ru(hi, 1.f + 0x1p-22f);
  c.thr_leaf = __fadd_ru(__fsqrt_ru(hi), 1.0001e-6f);
}

// The same for an exactly known FP64 minimum.
__device__ __forceinline__ void qctx_update(QCtx& c, double minSq)
{
  qctx_set32(c, __double2float_rd(minSq), __double2float_ru(minSq));
}

// squared_distance(p, box) <= minSq decided in FP32 (SD:576-578).  s is the
// per-axis signed gap to the outward-rounded box in round-to-nearest (> 0
// outside); it differs from the exact signed gap to the FP64 box by at most
// del = slack + eq plus 2^-24 |s|.  An axis with s < -del (plus that term) has
// an exact gap of 0 and contributes no error; the others contribute
// 2 del g + del^2, and 2^-21 sum g^2 covers the relative terms and the FP32
// rounding of the sum.  0: certainly false, 1: certainly true, 2: undecided.
__device__ __forceinline__ int box_decide(const float* lo, const float* hi, float slack, const QCtx& c)
{
  const float del = slack + c.eq;
  const float s0 = fmaxf(lo[0] - c.qf[0], c.qf[0] - hi[0]);
  const float s1 = fmaxf(lo[1] - c.qf[1], c.qf[1] - hi[1]);
  const float s2 = fmaxf(lo[2] - c.qf[2], c.qf[2] - hi[2]);
  const float g0 = fmaxf(s0, 0.f), g1 = fmaxf(s1, 0.f), g2 = fmaxf(s2, 0.f);
  const float lim = -1.01f * del;
  const float n0 = (s0 * 0.999f < lim) ? 0.f : 1.f;
  const float n1 = (s1 * 0.999f < lim) ? 0.f : 1.f;
  const float n2 = (s2 * 0.999f < lim) ? 0.f : 1.f;
  const float d2 = dot3f(g0, g0, g1, g1, g2, g2);
  const float err = __fmaf_rn(0x1p-21f, d2, __fmaf_rn(1.01f * del * del, n0 + n1 + n2, 2.02f * del * (g0 + g1 + g2)));
  if(!(err < INFINITY)) return 2;
  if(__fsub_rd(d2, err) > c.t_false) return 0;
  if(__fadd_ru(d2, err) <= c.t_true) return 1;
  return 2;
}

// One node visit decided in FP32.  Returns false if some decision is not
// certain (the caller then decides the whole visit in FP64 with visit_fp64).
// The child order (the nearer centroid first, LinearBVH.hpp:72-85) is the
// sign of 4 (|c_L - q|^2 - |c_R - q|^2) = sum_d a_d b_d, built from the gaps
// lo - q and q - hi the box tests use: per child u = (lo - q) - (q - hi) =
// 2 (c - q), a = u_L - u_R, b = u_L + u_R.  Against the exact values of the
// FP64 boxes and point, per axis (r the sum of the four |gaps|, s_L, s_R the
// boxes' rounding slacks, eq the point's):
//   |da| <= 2 (s_L + s_R) + 2^-22 r          (the point cancels in a)
//   |db| <= 2 (s_L + s_R) + 4 eq + 2^-22 r
// (three roundings of at most 2^-24 of a gap sum each), so the dot is within
//   (c0 + 4 eq) A1 + c0 B1 + 2^-22 sum r (|a| + |b|) + 2^-21 sum |a b|
//   + 6 (c0 + 4 eq)^2 + 2^-43 sum r^2,      c0 = 2 (s_L + s_R),
// A1 = sum |a|, B1 = sum |b| (the fused dot rounds three times).  The FP64
// comparison of the rounded centroids' squared distances is within
// 2^-50 Mq sum r (Mq the largest coordinate, below 2^21 lip) of the exact one.
__device__ __forceinline__ bool visit32(const NodeRec32* __restrict__ nodes32, int cur, const QCtx& c, bool& inL,
                                        bool& inR, bool& swap, int2& ch)
{
  const float4* r = reinterpret_cast<const float4*>(nodes32 + cur);
  const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
  const int4 lk = __ldg(reinterpret_cast<const int4*>(r + 3));
  ch = make_int2(lk.x, lk.y);
  const float lo_l[3] = {a.x, a.y, a.z}, hi_l[3] = {a.w, b.x, b.y};
  const float lo_r[3] = {b.z, b.w, cc.x}, hi_r[3] = {cc.y, cc.z, cc.w};
  const float sl_ = __int_as_float(lk.z), sr_ = __int_as_float(lk.w);
  // an invalid box is stored as [+inf, -inf]: its gap is +inf, box_decide
  // leaves it undecided and the FP64 visit applies the validity rule
  const int dl = box_decide(lo_l, hi_l, sl_, c);
  const int dr = box_decide(lo_r, hi_r, sr_, c);
  if(dl == 2 || dr == 2) return false;
  swap = false;
  if(dl == 1 && dr == 1)
  {
    float dot = 0.f, A1 = 0.f, B1 = 0.f, es = 0.f, rr = 0.f, R1 = 0.f, prod = 0.f;
#pragma unroll
    for(int d = 0; d < 3; ++d)
    {
      const float gll = lo_l[d] - c.qf[d], ghl = c.qf[d] - hi_l[d];
      const float glr = lo_r[d] - c.qf[d], ghr = c.qf[d] - hi_r[d];
      const float uL = gll - ghl, uR = glr - ghr;
      const float av = uL - uR, bv = uL + uR;
      dot = __fmaf_rn(av, bv, dot);
      const float aa = fabsf(av), bb = fabsf(bv);
      const float r = (fabsf(gll) + fabsf(ghl)) + (fabsf(glr) + fabsf(ghr));
      A1 += aa;
      B1 += bb;
      R1 += r;
      es = __fmaf_rn(r, aa + bb, es);
      rr = __fmaf_rn(r, r, rr);
      prod = __fmaf_rn(aa, bb, prod);
    }
    const float c0 = 2.f * (sl_ + sr_), c04 = c0 + 4.f * c.eq;
    const float bound = 1.02f * (c04 * A1 + c0 * B1 + 0x1p-22f * es + 0x1p-21f * prod + 6.f * c04 * c04 +
                                 0x1p-43f * rr + 0x1p-29f * c.lip * R1);
    if(!(bound < INFINITY)) return false;
    if(dot > bound)
      swap = true;
    else if(!(dot < -bound))
      return false;
  }
  inL = (dl == 1);
  inR = (dr == 1);
  return true;
}

// FP32 certificate of the leaf action: bit s of the result is set when
// triangle s may change the running minimum or the pseudo-normal sum and so
// needs the FP64 checkCandidate.
template <int NPC>
__device__ __forceinline__ int leaf_prefilter(const LeafRec32<NPC>* __restrict__ leaves32, int leafpos, const QCtx& c)
{
  const float4* r = reinterpret_cast<const float4*>(leaves32 + leafpos);
  float v[3 * NPC];
  float ec[2], lt[2];
  if constexpr(NPC == 3)
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    ec[0] = cc.y, lt[0] = cc.z;
  }
  else
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2), d4 = __ldg(r + 3);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    v[9] = cc.y, v[10] = cc.z, v[11] = cc.w;
    ec[0] = d4.x, ec[1] = d4.y, lt[0] = d4.z, lt[1] = d4.w;
  }
  int need = 0;
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    const float* A = v;
    const float* B = v + 3 * (s + 1);
    const float* C = v + 3 * (s + 2);
    float off[3];
    int kind;
    const float d2 = dist2_f32_flat(c.qf, A, B, C, off, kind);
    const float ap = fmaxf(fabsf(c.qf[0] - A[0]), fmaxf(fabsf(c.qf[1] - A[1]), fabsf(c.qf[2] - A[2])));
    const float E = __fadd_ru(c.lip, __fmul_ru(ec[s], __fadd_ru(ap, lt[s])));
    const float lim = __fadd_ru(c.thr_leaf, E);
    if(!(d2 > __fmul_ru(__fmul_ru(lim, lim), 1.0f + 0x1p-20f))) need |= 1 << s;
  }
  return need;
}

// Error of the FP32 distance sqrt(d2) = sd of dist2_f32_flat when its region
// is certain (crisp_regions) and not the edge BC or the face.  u = 2^-24.
// Rounding the point and the vertices moves the exact distance by at most
// u sqrt(3) (|q|_inf + M) (it is 1-Lipschitz in them), below lip / 4.
//  * vertex V: off = fl(qf - Vf) exactly as the offset, within u |off| of
//    qf - Vf: sd is within lip / 4 + 2^-23 sd of |q - V|, and the FP64 point
//    is V itself;
//  * edge AB (AC alike): t = d1 / (d1 - d3) and off = fl(ap - t ab).  With
//    dots of rounded differences within 5.01 u |e| |p| of the exact ones,
//    |t - t*| <= 5.1 u (2 |ap| + |bp|) / |ab| + 2 u to first order, and
//    |off - off*| <= u (|off| + 16.3 |ap|_2 + 8.1 |ab|) with |ap|_2 <=
//    sqrt(3) ap (ap the largest coordinate of qf - A) and |ab| <= lt:
//    lip / 4 + 2^-23 sd + 2^-19 ap + 2^-20 lt.  First order holds while the
//    relative error of d1 - d3 is small: every edge is at least lt / kappa
//    long (kappa = ec 2^16), so ap ec <= lt / 16 keeps |ap|_2 / |ab| below
//    7100 and that error below 1/200, which the constants' margins cover.
// The FP64 routine's point is within 2^-36 M of the exact projection, far
// inside either bound.  Returns +inf where no bound applies.
__device__ __forceinline__ float region_error(int kind, float lip, float sd, float ap, float lt, float ec)
{
  const float base = __fadd_ru(__fmul_ru(0.25f, lip), __fmul_ru(0x1p-23f, sd));
  if(kind == 0) return base;
  if(kind == 1 && __fmul_ru(ap, ec) <= 0.0625f * lt)
    return __fadd_ru(base, __fadd_ru(__fmul_ru(0x1p-19f, ap), __fmul_ru(0x1p-20f, lt)));
  return INFINITY;
}

// leaf_prefilter that also bounds, for the triangles it keeps, the squared
// distance the FP64 checkCandidate will compute: [lo2, hi2] holds the minimum
// over the kept triangles.  The FP64 point always lies on the triangle, so the
// lower end needs only the FP32 error.  The upper end adds the FP64 routine's
// own departure from the exact closest point: its fuzzy region tests
// (closest_point.hpp:181-282) use a fixed EPS = 1e-12 on dot products
// (length^2), which moves the point by at most 1e-12 / (shortest edge)
// <= 1e-12 kappa / L, and on the products vc, vb, va (length^4), which moves
// it by at most 1e-12 / (edge |n|) <= 1e-12 kappa^2 / L^3 (for the small
// triangles of fine meshes this is ~1e-6, far above rounding); both doubled.
// mesh_max bounds the mesh's coordinates (rounded up).
template <int NPC>
__device__ __forceinline__ int leaf_prefilter_bounds(const LeafRec32<NPC>* __restrict__ leaves32, int leafpos,
                                                     const QCtx& c, float mesh_max, float& lo2, float& hi2, float* cpf,
                                                     float& rad)
{
  const float4* r = reinterpret_cast<const float4*>(leaves32 + leafpos);
  float v[3 * NPC];
  float ec[2], lt[2];
  float fzt = 0.f;
  if constexpr(NPC == 3)
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    ec[0] = cc.y, lt[0] = cc.z, fzt = cc.w;
  }
  else
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2), d4 = __ldg(r + 3);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    v[9] = cc.y, v[10] = cc.z, v[11] = cc.w;
    ec[0] = d4.x, ec[1] = d4.y, lt[0] = d4.z, lt[1] = d4.w;
  }
  int need = 0;
  lo2 = INFINITY;
  hi2 = INFINITY;
  rad = INFINITY;
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    const float* A = v;
    const float* B = v + 3 * (s + 1);
    const float* C = v + 3 * (s + 2);
    float off[3];
    int kind;
    const float d2 = dist2_f32_flat(c.qf, A, B, C, off, kind);
    const float ap = fmaxf(fabsf(c.qf[0] - A[0]), fmaxf(fabsf(c.qf[1] - A[1]), fabsf(c.qf[2] - A[2])));
    float E = __fadd_ru(c.lip, __fmul_ru(ec[s], __fadd_ru(ap, lt[s])));
    const float lim = __fadd_ru(c.thr_leaf, E);
    if(!(d2 > __fmul_ru(__fmul_ru(lim, lim), 1.0f + 0x1p-20f)))
    {
      need |= 1 << s;
      float fz;
      if constexpr(NPC == 3)
        fz = fzt;  // stored with the triangle
      else
      {
        const float kappa = ec[s] * (1.f / (256.f * 0x1p-24f));
        const float kl = __fdiv_ru(kappa, lt[s]);
        fz = __fmul_ru(2e-12f, __fadd_ru(kl, __fdiv_ru(__fmul_ru(kl, kl), lt[s])));
      }
      // sqrt(d2 (1 -+ 2^-20)) from the correctly rounded sqrt(d2): the factor
      // 1 -+ 2^-20 covers both the 2^-21 of the square root of the margin and
      // the 2^-24 rounding of sqrtf
      const float sd = sqrtf(d2);
      // no fuzzy displacement when every region test is clear of its EPS band;
      // the region is then certain, and a vertex or an edge at A has a
      // tighter error than the general one
      // (eq 2^24 bounds the point's largest coordinate)
      if(crisp_regions(c.qf, A, B, C, c.eq * 0x1p24f, mesh_max))
      {
        fz = 0.f;
        E = fminf(E, region_error(kind, c.lip, sd, ap, lt[s], ec[s]));
      }
      const float dl = fmaxf(__fsub_rd(__fmul_rd(sd, 1.f - 0x1p-20f), E), 0.f);
      const float dh = __fadd_ru(__fadd_ru(__fmul_ru(sd, 1.f + 0x1p-20f), E), fz);
      const float l2 = __fmul_rd(dl, dl), h2 = __fmul_ru(dh, dh);
      lo2 = (d2 == d2) ? fminf(lo2, l2) : 0.f;
      hi2 = (d2 == d2 && h2 == h2) ? fminf(hi2, h2) : hi2;
      // closest point estimate: the exact projection is 1-Lipschitz, so the
      // FP64 point lies within 2 (E + fz) of qf - off
      for(int d = 0; d < 3; ++d) cpf[d] = c.qf[d] - off[d];
      rad = __fmul_ru(2.f, __fadd_ru(E, fz));
    }
  }
  return need;
}

// The roundings the sign certificate asks for, as device intrinsics (the
// certificate is evaluated on the device; the host checker supplies its own).
struct SignOps
{
#ifdef __CUDA_ARCH__
  __host__ __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  __host__ __device__ static float add_ru(float a, float b) { return __fadd_ru(a, b); }
  __host__ __device__ static float add_rd(float a, float b) { return __fadd_rd(a, b); }
  __host__ __device__ static float sub_rd(float a, float b) { return __fsub_rd(a, b); }
  __host__ __device__ static float mul_ru(float a, float b) { return __fmul_ru(a, b); }
  __host__ __device__ static float mul_rd(float a, float b) { return __fmul_rd(a, b); }
  __host__ __device__ static float div_ru(float a, float b) { return __fdiv_ru(a, b); }
  __host__ __device__ static float rsqrt(float a) { return __frsqrt_rn(a); }
  __host__ __device__ static float acos(float a) { return acosf(a); }
  __host__ __device__ static float to_float(double a) { return __double2float_rn(a); }
#else
  static float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static float add_ru(float a, float b) { return nextafterf(a + b, INFINITY); }
  static float add_rd(float a, float b) { return nextafterf(a + b, -INFINITY); }
  static float sub_rd(float a, float b) { return nextafterf(a - b, -INFINITY); }
  static float mul_ru(float a, float b) { return nextafterf(a * b, INFINITY); }
  static float mul_rd(float a, float b) { return nextafterf(a * b, -INFINITY); }
  static float div_ru(float a, float b) { return nextafterf(a / b, INFINITY); }
  static float rsqrt(float a) { return (float)(1.0 / sqrt((double)a)); }
  static float acos(float a) { return (float)::acos((double)a); }
  static float to_float(double a) { return (float)a; }
#endif
};

// FP32 certificate of computeSign (SD:751-763) for one finished query (see
// gsq_sign.cuh): +1 or -1 when the FP64 dot(q - cp, N) >= 0 of finish_query
// certainly has that outcome, 0 when not certain (the caller then evaluates
// the pseudo-normal in FP64).  The triangles come from the FP32 leaf records:
// the closest face (type 2) or the recorded pseudo-normal contributions.
template <int NPC>
__device__ __forceinline__ double sign32(const double* q, const MinCand& mc, const LeafRec32<NPC>* __restrict__ leaves32,
                                         float M)
{
  const float r[3] = {__double2float_rn(q[0] - mc.mp[0]), __double2float_rn(q[1] - mc.mp[1]),
                      __double2float_rn(q[2] - mc.mp[2])};
  auto rec_tri = [&](int leaf, int sub, const float*& A, const float*& B, const float*& C, float& L) {
    const LeafRec32<NPC>& rec = leaves32[leaf];
    A = rec.v;
    B = rec.v + 3 * (sub + 1);
    C = rec.v + 3 * (sub + 2);
    if constexpr(NPC == 3)
      L = rec.lt;
    else
      L = rec.lt[sub];
  };
  if(mc.type == 2)
  {
    auto face_tri = [&](int, const float*& A, const float*& B, const float*& C, float& L, int& k) {
      k = 0;
      rec_tri(mc.leaf, mc.sub, A, B, C, L);
    };
    return sign_certificate<SignOps>(r, true, mc.sn, 1, face_tri, M);
  }
  auto pend_tri = [&](int i, const float*& A, const float*& B, const float*& C, float& L, int& k) {
    const int code = mc.pend[i];
    k = code & 3;
    rec_tri(code >> 3, (code >> 2) & 1, A, B, C, L);
  };
  return sign_certificate<SignOps>(r, false, mc.sn, mc.npend, pend_tri, M);
}

// Audit of a skipped triangle: counts it if the FP64 distance contradicts
// the certificate (it would lie within sqrt(minSq) + 1e-6).
template <int NPC>
__device__ __forceinline__ int leaf_audit(const LeafRec<NPC>* __restrict__ leaves64, int leafpos, int skip_mask,
                                          const double* q, double minSq)
{
  double w[3 * NPC];
  load_leaf<NPC>(leaves64, leafpos, w);
  int bad = 0;
  for(int s = 0; s < NPC - 2; ++s)
  {
    if(!(skip_mask & (1 << s))) continue;
    double cp[3];
    closest_point(q, w, w + 3 * (s + 1), w + 3 * (s + 2), cp);
    const double lim64 = sqrt(minSq) + 1e-6;
    if(sqdist_pp(q, cp) <= lim64 * lim64) ++bad;
  }
  return bad;
}

// Audit: two checkCandidate states are the same (pseudo-normal sums evaluated).
template <int NPC>
__device__ __forceinline__ bool same_state(MinCand a, MinCand b, const LeafRec<NPC>* __restrict__ leaves64)
{
  flush_normals<NPC>(a, leaves64);
  flush_normals<NPC>(b, leaves64);
  return a.minSq == b.minSq && a.type == b.type && a.leaf == b.leaf && a.sub == b.sub && a.mp[0] == b.mp[0] &&
         a.mp[1] == b.mp[1] && a.mp[2] == b.mp[2] && a.sn[0] == b.sn[0] && a.sn[1] == b.sn[1] && a.sn[2] == b.sn[2];
}

// FP64 checkCandidate on the triangles of `need`, in the reference's order.
template <int NPC>
__device__ __forceinline__ void leaf_refine(const LeafRec<NPC>* __restrict__ leaves64, int leafpos, int need,
                                            const double* q, MinCand& mc, bool computeNormal)
{
  double w[3 * NPC];
  load_leaf<NPC>(leaves64, leafpos, w);
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    if(!(need & (1 << s))) continue;
    const double* T[3] = {w, w + 3 * (s + 1), w + 3 * (s + 2)};
    check_triangle<NPC>(q, mc, T, leaves64, leafpos, s, computeNormal);
  }
}

// The certified traversal for one point, one thread at a time (used by the
// adjoint).  mc must be initialised.  Returns false on stack overflow.  With
// AUDIT, stats[0..3] accumulate contradictions, FP64 node decisions, FP64
// leaf checks and skips.
template <int NPC, bool AUDIT>
__device__ __forceinline__ bool mixed_traverse(const double* q, MinCand& mc, const NodeRec64* __restrict__ nodes64,
                                               const NodeRec32* __restrict__ nodes32,
                                               const LeafRec<NPC>* __restrict__ leaves64,
                                               const LeafRec32<NPC>* __restrict__ leaves32, float mesh_max,
                                               bool computeNormal, unsigned long long* stats)
{
  QCtx c;
  qctx_init(c, q, mesh_max);
  qctx_update(c, mc.minSq);
  auto visit = [&](int cur, bool& inL, bool& inR, bool& swap, int2& ch) {
    if(visit32(nodes32, cur, c, inL, inR, swap, ch))
    {
      if(AUDIT)
      {
        bool a2, b2, w2;
        visit_fp64(nodes64, cur, q, mc.minSq, a2, b2, w2);
        if(a2 != inL || b2 != inR || (inL && inR && w2 != swap)) ++stats[0];
      }
      return;
    }
    if(AUDIT) ++stats[1];
    visit_fp64(nodes64, cur, q, mc.minSq, inL, inR, swap);
  };
  auto leaf = [&](int leafpos) {
    const int need = leaf_prefilter<NPC>(leaves32, leafpos, c);
    const int all = (1 << (NPC - 2)) - 1;
    if(AUDIT)
    {
      if(need == 0) ++stats[3];
      stats[0] += leaf_audit<NPC>(leaves64, leafpos, all & ~need, q, mc.minSq);
    }
    if(need == 0) return;
    if(AUDIT) ++stats[2];
    const double before = mc.minSq;
    leaf_refine<NPC>(leaves64, leafpos, need, q, mc, computeNormal);
    if(mc.minSq != before) qctx_update(c, mc.minSq);
  };
  return traverse_point(visit, leaf);
}
}  // namespace sdf
}  // namespace gsq
