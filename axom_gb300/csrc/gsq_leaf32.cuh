// The FP32 certificates of the mixed signed distance: the per-query context;
// for the leaves, the point-triangle distance evaluated in FP32, its error
// bounds, the test that the reference's fuzzy region tests take their exact
// outcomes, and the per-triangle error terms stored in the FP32 leaf records;
// for the nodes, the outward-rounded child boxes of the FP32 node records, the
// box test and the child order.
//
// The functions compile for the device (the query kernels) and for the host
// (checkers in the tests compare them with the oracle's FP64 closest point and
// node visit).
// fp:: names the roundings: on the device they are the CUDA intrinsics; on
// the host round-to-nearest operations are the same IEEE operations, and a
// directed rounding is the nearest result moved one ulp outward, never tighter
// than the device's.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define GSQ_HD __host__ __device__ __forceinline__
#else
#define GSQ_HD inline
#endif

namespace gsq
{
namespace fp
{
#ifdef __CUDA_ARCH__
GSQ_HD float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
GSQ_HD float add_ru(float a, float b) { return __fadd_ru(a, b); }
GSQ_HD float add_rd(float a, float b) { return __fadd_rd(a, b); }
GSQ_HD float sub_rd(float a, float b) { return __fsub_rd(a, b); }
GSQ_HD float mul_ru(float a, float b) { return __fmul_ru(a, b); }
GSQ_HD float mul_rd(float a, float b) { return __fmul_rd(a, b); }
GSQ_HD float div_ru(float a, float b) { return __fdiv_ru(a, b); }
GSQ_HD float sqrt_ru(float a) { return __fsqrt_ru(a); }
GSQ_HD float sqrt_rd(float a) { return __fsqrt_rd(a); }
GSQ_HD float f_rn(double a) { return __double2float_rn(a); }
GSQ_HD float f_ru(double a) { return __double2float_ru(a); }
GSQ_HD float f_rd(double a) { return __double2float_rd(a); }
#else
GSQ_HD float fma(float a, float b, float c) { return std::fmaf(a, b, c); }
GSQ_HD float add_ru(float a, float b) { return std::nextafterf(a + b, INFINITY); }
GSQ_HD float add_rd(float a, float b) { return std::nextafterf(a + b, -INFINITY); }
GSQ_HD float sub_rd(float a, float b) { return std::nextafterf(a - b, -INFINITY); }
GSQ_HD float mul_ru(float a, float b) { return std::nextafterf(a * b, INFINITY); }
GSQ_HD float mul_rd(float a, float b) { return std::nextafterf(a * b, -INFINITY); }
GSQ_HD float div_ru(float a, float b) { return std::nextafterf(a / b, INFINITY); }
GSQ_HD float sqrt_ru(float a)
{
  const float s = std::sqrt(a);
  return ((double)s * (double)s < (double)a) ? std::nextafterf(s, INFINITY) : s;
}
GSQ_HD float sqrt_rd(float a)
{
  const float s = std::sqrt(a);
  return ((double)s * (double)s > (double)a) ? std::nextafterf(s, -INFINITY) : s;
}
GSQ_HD float f_rn(double a) { return (float)a; }
GSQ_HD float f_ru(double a)
{
  const float f = (float)a;
  return ((double)f < a) ? std::nextafterf(f, INFINITY) : f;
}
GSQ_HD float f_rd(double a)
{
  const float f = (float)a;
  return ((double)f > a) ? std::nextafterf(f, -INFINITY) : f;
}
#endif
}  // namespace fp

namespace sdf
{
// FP32 dot product with fused operations (one rounding per multiply-add):
// the error bounds used with these FP32 evaluations count at least one
// rounding per operation, which fused operations meet.
GSQ_HD float dot3f(float a0, float b0, float a1, float b1, float a2, float b2)
{
  return fp::fma(a2, b2, fp::fma(a1, b1, a0 * b0));
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
GSQ_HD bool crisp_regions(const float* P, const float* A, const float* B, const float* C, float Q, float M)
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
  const float vc = fp::fma(d1, d4, -(d3 * d2));
  const float vb = fp::fma(d5, d2, -(d1 * d6));
  const float va = fp::fma(d3, d6, -(d5 * d4));
  auto n1 = [](float x, float y, float z) { return fabsf(x) + fabsf(y) + fabsf(z); };
  const float E1 = fmaxf(n1(ab0, ab1, ab2), n1(ac0, ac1, ac2));
  const float P1 = fmaxf(n1(ap0, ap1, ap2), fmaxf(n1(bp0, bp1, bp2), n1(cp0, cp1, cp2)));
  const float QM = fp::add_ru(Q, M);
  const float err_d =
      fp::mul_ru(1.02f, fp::add_ru(fp::add_ru(fp::mul_ru(0x1p-23f * M, P1), fp::mul_ru(0x1p-24f * QM, E1)),
                                 fp::add_ru(fp::mul_ru(5.f * 0x1p-24f, fp::mul_ru(E1, P1)),
                                           fp::mul_ru(0x1p-44f * QM, QM))));
  const float D = fp::add_ru(fmaxf(fmaxf(fmaxf(fabsf(d1), fabsf(d2)), fmaxf(fabsf(d3), fabsf(d4))),
                                  fmaxf(fabsf(d5), fabsf(d6))),
                            err_d);
  const float err_v = fp::mul_ru(1.01f, fp::add_ru(fp::add_ru(fp::mul_ru(4.f * D, err_d), 2.f * err_d * err_d),
                                                 fp::mul_ru(0x1p-22f, fp::mul_ru(D, D))));
  const float err_s = fp::mul_ru(1.01f, fp::add_ru(2.f * err_d, fp::mul_ru(0x1p-23f, D)));
  auto clear = [&](float x, float e) { return fabsf(x) > fp::add_ru(2.f * e, 2.f * EPS); };
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
GSQ_HD float dist2_f32_flat(const float* P, const float* A, const float* B, const float* C, float* off,
                             int& kind)
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
  const float vc = fp::fma(d1, d4, -(d3 * d2));
  const float vb = fp::fma(d5, d2, -(d1 * d6));
  const float va = fp::fma(d3, d6, -(d5 * d4));
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
  off[0] = fp::fma(-w, e0, fp::fma(-v, ab0, b0));
  off[1] = fp::fma(-w, e1, fp::fma(-v, ab1, b1));
  off[2] = fp::fma(-w, e2, fp::fma(-v, ab2, b2));
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

GSQ_HD void qctx_init(QCtx& c, const double* q, float mesh_max)
{
  float qabs = 0.f;
  for(int d = 0; d < 3; ++d)
  {
    c.qf[d] = fp::f_rn(q[d]);
    qabs = fmaxf(qabs, fabsf(c.qf[d]));
  }
  // |qf - q| <= 2^-24 |qf| (round to nearest; the absolute term covers
  // subnormals); the subtraction in a gap is exact or contributes at most
  // 2^-24 of the gap, which the relative term of box_decide covers
  c.eq = fp::add_ru(fp::mul_ru(0x1p-24f, qabs), 0x1p-149f);
  // the point-triangle distance is 1-Lipschitz in the point and the vertices
  c.lip = fp::mul_ru(0x1p-21f, fp::add_ru(qabs, mesh_max));
}

// Thresholds for an exact minimum known to lie in the FP32 interval [lo, hi]:
// t_true <= minSq (1 - 2^-40) and t_false >= minSq (1 + 2^-40) with room for
// the FP64 predicate's own rounding; thr_leaf >= sqrt(minSq) + 1e-6.  No FP64
// arithmetic.
GSQ_HD void qctx_set32(QCtx& c, float lo, float hi)
{
  c.t_true = fp::mul_rd(lo, 1.f - 0x1p-22f);
  c.t_false = fp::mul_ru(hi, 1.f + 0x1p-22f);
  c.thr_leaf = fp::add_ru(fp::sqrt_ru(hi), 1.0001e-6f);
}

// The same for an exactly known FP64 minimum.
GSQ_HD void qctx_update(QCtx& c, double minSq)
{
  qctx_set32(c, fp::f_rd(minSq), fp::f_ru(minSq));
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
GSQ_HD float region_error(int kind, float lip, float sd, float ap, float lt, float ec)
{
  const float base = fp::add_ru(fp::mul_ru(0.25f, lip), fp::mul_ru(0x1p-23f, sd));
  if(kind == 0) return base;
  if(kind == 1 && fp::mul_ru(ap, ec) <= 0.0625f * lt)
    return fp::add_ru(base, fp::add_ru(fp::mul_ru(0x1p-19f, ap), fp::mul_ru(0x1p-20f, lt)));
  return INFINITY;
}

// Per triangle: ec = 256 * 2^-24 * kappa (kappa = L^2 / |n|, L the longest
// edge), lt = L, and fz = 2e-12 (kappa / L + kappa^2 / L^3), the bound on how
// far the reference's fuzzy region tests move its closest point; all rounded
// up with a margin.
GSQ_HD void tri_error_terms(const double* A, const double* B, const double* C, float& ec, float& lt,
                                                float* fz = nullptr)
{
  const double ab[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
  const double ac[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
  const double bc[3] = {C[0] - B[0], C[1] - B[1], C[2] - B[2]};
  const double n[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
  const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double L = fmax(sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]),
                        fmax(sqrt(ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2]),
                             sqrt(bc[0] * bc[0] + bc[1] * bc[1] + bc[2] * bc[2])));
  const double kappa = (nn > 0.0 && nn == nn) ? (L * L) / nn : INFINITY;
  ec = fp::f_ru(256.0 * 0x1p-24 * kappa * 1.01);
  // The reference's fuzzy dot tests (EPS = 1e-12 on d1..d6) can leave its
  // point up to EPS / (shortest edge) <= 1e-12 kappa / L off the triangle (an
  // edge parameter d1 / (d1 - d3) with d1 in [-EPS, 0)), nearer the query than
  // the exact distance.  The coordinate term lip of the FP32 error bound holds
  // 0.78 lip >= 2^-22 M of slack beyond the rounding it covers; where the
  // overshoot could exceed 2^-22 times the triangle's largest coordinate (tiny
  // triangles), the conditioning factor is made infinite, so that the
  // triangle is never skipped and its bounds come from FP64.
  const double mt = fmax(fmax(fmax(fabs(A[0]), fabs(A[1])), fmax(fabs(A[2]), fabs(B[0]))),
                         fmax(fmax(fabs(B[1]), fabs(B[2])), fmax(fmax(fabs(C[0]), fabs(C[1])), fabs(C[2]))));
  if(!(2.06e-12 * kappa / L <= 0x1p-22 * mt)) ec = INFINITY;
  // The conditioning factor is the FP64 triangle's; the FP32 one has its
  // vertices moved by up to d = sqrt(3) 2^-24 mt, which changes the cross
  // product by about 4 d L, i.e. its altitude h = |n| / L by 4 d.  Slivers
  // narrower than 64 d (their rounded form can be far thinner, even flipped)
  // get an infinite factor too: never skipped, bounds from FP64.
  if(!(64.0 * 1.7320508075688774 * 0x1p-24 * mt * L <= nn)) ec = INFINITY;
  lt = fp::f_ru(L * 1.0001);
  if(fz)
  {
    const double kl = kappa / L;
    const double f = 2e-12 * (kl + kl * kappa / (L * L)) * 1.03;
    *fz = (f == f) ? fp::f_ru(f) : INFINITY;
  }
}


// The certificate for one triangle A, B, C of an FP32 leaf record, with the
// stored ec and lt (and fz for triangle meshes; a quad's triangle derives it
// from ec and lt): false when its FP64 distance certainly exceeds
// c.thr_leaf, so that checkCandidate can change neither the minimum nor the
// pseudo-normal sum; else true with d2 (the FP32 squared distance), [l2, h2]
// holding the FP64 squared distance checkCandidate will compute, and the
// estimate cpf of the FP64 closest point with a radius rad around it.
// The FP64 point lies on the triangle, or at most the fuzzy overshoot off it
// (see tri_error_terms), so the lower end needs only the FP32 error.  The
// upper end adds the FP64 routine's own departure from the exact closest
// point: its fuzzy region tests (closest_point.hpp:181-282) use a fixed
// EPS = 1e-12 on dot products (length^2), which moves the point by at most
// 1e-12 / (shortest edge) <= 1e-12 kappa / L, and on the products vc, vb, va
// (length^4), which moves it by at most 1e-12 / (edge |n|) <= 1e-12 kappa^2 / L^3
// (for the small triangles of fine meshes this is ~1e-6, far above rounding);
// both doubled.  Where every region test is clear of its EPS band the region
// is certain: no displacement, and a vertex or an edge at A has a tighter
// error than the general one.  mesh_max bounds the mesh's coordinates
// (rounded up).
// The general error is lip + ec (ap + L) cond(kappa), cond = max(1, kappa/16):
// the face region's weights are ratios of products of dots over |n|^2, whose
// error grows as kappa^2 (measured: within 0.46 u kappa (ap + L) for
// kappa < 8, about 0.2 u kappa^2 (ap + L) for slivers).
// The closest point's error is not the distance's: moving the vertices by d
// (their rounding, u sqrt(3) M) turns an edge or the plane, and the foot of a
// point at |ap| moves by up to d (1 + 2 |ap| / shortest edge) <= d (1 + 3.5 ap
// kappa / L), while the distance moves only by d; the face region's weights
// add 8 u kappa^2 (ap + L).  So the FP64 point lies within
//   2 (E + fz + 16 u (|q| + M) (1 + ap kappa / L) + 8 u kappa^2 (ap + L))
// of cpf = qf - off (measured up to 1.6x the bracket without the factors 2,
// 16 and 8).
template <bool QUAD>
GSQ_HD bool tri_bounds(const QCtx& c, float mesh_max, const float* A, const float* B, const float* C, float ec,
                       float lt, float fz_stored, float& d2, float& l2, float& h2, float* cpf, float& rad)
{
  float off[3];
  int kind;
  d2 = dist2_f32_flat(c.qf, A, B, C, off, kind);
  const float ap = fmaxf(fabsf(c.qf[0] - A[0]), fmaxf(fabsf(c.qf[1] - A[1]), fabsf(c.qf[2] - A[2])));
  const float kap = ec * 65536.f;  // >= kappa (ec = 2^-16 kappa, rounded up)
  float E = fp::add_ru(c.lip, fp::mul_ru(fp::mul_ru(ec, fmaxf(1.f, kap * 0.0625f)), fp::add_ru(ap, lt)));
  const float lim = fp::add_ru(c.thr_leaf, E);
  if(d2 > fp::mul_ru(fp::mul_ru(lim, lim), 1.0f + 0x1p-20f)) return false;
  float fz;
  if constexpr(!QUAD)
    fz = fz_stored;
  else
  {
    const float kappa = ec * (1.f / (256.f * 0x1p-24f));
    const float kl = fp::div_ru(kappa, lt);
    fz = fp::mul_ru(2e-12f, fp::add_ru(kl, fp::div_ru(fp::mul_ru(kl, kl), lt)));
  }
  // sqrt(d2 (1 -+ 2^-20)) from the correctly rounded sqrt(d2): the factor
  // 1 -+ 2^-20 covers both the 2^-21 of the square root of the margin and
  // the 2^-24 rounding of sqrtf
  const float sd = sqrtf(d2);
  // (eq 2^24 bounds the point's largest coordinate)
  if(crisp_regions(c.qf, A, B, C, c.eq * 0x1p24f, mesh_max))
  {
    fz = 0.f;
    E = fminf(E, region_error(kind, c.lip, sd, ap, lt, ec));
  }
  const float dl = fmaxf(fp::sub_rd(fp::mul_rd(sd, 1.f - 0x1p-20f), E), 0.f);
  const float dh = fp::add_ru(fp::add_ru(fp::mul_ru(sd, 1.f + 0x1p-20f), E), fz);
  l2 = fp::mul_rd(dl, dl);
  h2 = fp::mul_ru(dh, dh);
  for(int d = 0; d < 3; ++d) cpf[d] = c.qf[d] - off[d];
  const float QM = fp::add_ru(c.eq * 0x1p24f, mesh_max);
  const float lever = fp::mul_ru(16.f * 0x1p-24f, fp::mul_ru(QM, fp::add_ru(1.f, fp::div_ru(fp::mul_ru(ap, kap), lt))));
  const float arith = fp::mul_ru(8.f * 0x1p-24f, fp::mul_ru(fp::mul_ru(kap, kap), fp::add_ru(ap, lt)));
  rad = fp::mul_ru(2.f, fp::add_ru(fp::add_ru(E, fz), fp::add_ru(lever, arith)));
  if(!(d2 == d2)) rad = INFINITY;  // no estimate (a degenerate FP32 triangle)
  return true;
}
// squared_distance(p, box) <= minSq decided in FP32 (SD:576-578).  s is the
// per-axis signed gap to the outward-rounded box in round-to-nearest (> 0
// outside); it differs from the exact signed gap to the FP64 box by at most
// del = slack + eq plus 2^-24 |s|.  An axis with s < -del (plus that term) has
// an exact gap of 0 and contributes no error; the others contribute
// 2 del g + del^2, and 2^-21 sum g^2 covers the relative terms and the FP32
// rounding of the sum.  0: certainly false, 1: certainly true, 2: undecided.
GSQ_HD int box_decide(const float* lo, const float* hi, float slack, const QCtx& c)
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
  const float err = fp::fma(0x1p-21f, d2, fp::fma(1.01f * del * del, n0 + n1 + n2, 2.02f * del * (g0 + g1 + g2)));
  if(!(err < INFINITY)) return 2;
  if(fp::sub_rd(d2, err) > c.t_false) return 0;
  if(fp::add_ru(d2, err) <= c.t_true) return 1;
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
GSQ_HD bool visit32_core(const float* lo_l, const float* hi_l, const float* lo_r, const float* hi_r, float sl_,
                         float sr_, const QCtx& c, bool& inL, bool& inR, bool& swap)
{
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
      dot = fp::fma(av, bv, dot);
      const float aa = fabsf(av), bb = fabsf(bv);
      const float r = (fabsf(gll) + fabsf(ghl)) + (fabsf(glr) + fabsf(ghr));
      A1 += aa;
      B1 += bb;
      R1 += r;
      es = fp::fma(r, aa + bb, es);
      rr = fp::fma(r, r, rr);
      prod = fp::fma(aa, bb, prod);
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


// FP32 enclosure [lo2, hi2] of the FP64 squared distance the reference
// computes between the query and an object point (squared_distance(Point,
// Point), primal/operators/squared_distance.hpp:62-67), from the query
// context (qf rounded to nearest, lip = 2^-21 (max|qf| + M)) and the object
// point rounded to nearest (pf, |p| <= M).  With u = 2^-24: per coordinate
// the rounded difference qf - pf is within u (max|qf| + M) of q - p, so
// |q - p| is within sqrt(3) u (max|qf| + M) < lip / 4 of |qf - pf|; the FP32
// offsets o = fl(qf - pf) are within u |o| of qf - pf and the fused dot d2 is
// within 3.01 u of |o|^2, so |q - p| lies in sqrt(d2) (1 -+ 2.52 u) -+ lip / 4,
// widened here to (1 -+ 4 u).  The FP64 evaluation rounds within 2^-50 of
// |q - p|^2, covered by a further factor (1 -+ 2^-22).  Distances too small
// for these FP32 bounds (or too large) give [0, inf): undecided.
GSQ_HD void point_bounds32(const QCtx& c, const float* pf, float& lo2, float& hi2)
{
  const float o0 = c.qf[0] - pf[0], o1 = c.qf[1] - pf[1], o2 = c.qf[2] - pf[2];
  const float d2 = dot3f(o0, o0, o1, o1, o2, o2);
  const float e = fp::mul_ru(0.25f, c.lip);
  const float slo = fp::sub_rd(fp::mul_rd(fp::sqrt_rd(d2), 1.f - 0x1p-22f), e);
  const float shi = fp::add_ru(fp::mul_ru(fp::sqrt_ru(d2), 1.f + 0x1p-22f), e);
  if(!(shi > 0x1p-60f && shi < 0x1p60f))
  {
    lo2 = 0.f;
    hi2 = INFINITY;
    return;
  }
  const float l = fmaxf(slo, 0.f);
  lo2 = fp::mul_rd(fp::mul_rd(l, l), 1.f - 0x1p-22f);
  hi2 = fp::mul_ru(fp::mul_ru(shi, shi), 1.f + 0x1p-22f);
}

// One child box of an FP64 node record as the FP32 node records hold it
// (k_nodes32): lo rounded down, hi rounded up, and the returned slack (the
// largest rounding distance, rounded up); an invalid box (BoundingBox::isValid,
// primal/geometry/BoundingBox.hpp:451-460) becomes [+inf, -inf] with slack 0.
GSQ_HD float node_box32(const double* b, float* o)
{
  if(b[0] > b[3] || b[1] > b[4] || b[2] > b[5])
  {
    for(int d = 0; d < 3; ++d)
    {
      o[d] = INFINITY;
      o[3 + d] = -INFINITY;
    }
    return 0.f;
  }
  double s = 0.0;
  for(int d = 0; d < 3; ++d)
  {
    o[d] = fp::f_rd(b[d]);
    o[3 + d] = fp::f_ru(b[3 + d]);
    s = fmax(s, fmax(b[d] - (double)o[d], (double)o[3 + d] - b[3 + d]));
  }
  return (s == s) ? fp::f_ru(s) : INFINITY;
}

}  // namespace sdf
}  // namespace gsq
