// FP32 certificate of the signed distance's sign test (computeSign,
// quest/SignedDistance.hpp:751-763): the FP64 test is dot(q - cp, N) >= 0 with
// N the closest face's normal, or for a shared vertex or edge the
// pseudo-normal sum (SD:709-736) in its recorded order.  The certificate
// rebuilds N in FP32 from the rounded vertices with error bounds and returns
// +1 or -1 when the FP64 test certainly has that outcome, 0 otherwise.
//
// The arithmetic is written once for the device and for a host checker: Ops
// supplies the fused multiply-add, the directed roundings, the reciprocal
// square root and the arccosine.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define GSQ_SIGN_HD __host__ __device__ __forceinline__
#else
#define GSQ_SIGN_HD inline
#endif

namespace gsq
{
// r: q - cp formed in FP64 as the reference forms it, rounded to nearest.
// face: N is the normal of triangle 0; else N = sn (the FP64 sum of the
// contributions already evaluated) plus contributions 0..count-1.
// tri(i, A, B, C, L, k): triangle i's FP32 vertices (rounded to nearest), an
// upper bound L on its longest edge, and the contribution's kind k (0..2:
// the angle-weighted unit normal at vertex k; 3: the unit normal, an edge).
// M bounds every coordinate of the mesh.
// Error terms (u = 2^-24):
//  * an edge of rounded vertices is within de = 2^-23 M + u L per coordinate;
//  * a cross product of two edges within dn = 3 (4 de L + 2 de^2 + 2^-22 L^2)
//    in L1 (two products and a fused subtraction per coordinate);
//  * a normalised vector v within 2 |dv| / (|v| - |dv|) + 4u (direction of a
//    perturbed vector, then the correctly rounded 1/sqrt and the scaling);
//  * the angle acos(ua . ub) within w(ddp) + 2^-21: ddp bounds the dot's
//    error, w(t) = t / sqrt(1 - (|x| + t)^2) away from +-1 and pi sqrt(t / 2)
//    everywhere (acos's modulus of continuity), 2^-21 the 2 ulp of acosf;
//  * FP32 sums round at most u per term and addition;
//  * r is within u of q - cp per coordinate.
// The FP64 evaluation's own rounding is below 2^-40 of these bounds.
template <class Ops, class Tri>
GSQ_SIGN_HD double sign_certificate(const float* r, bool face, const double* sn, int count, Tri tri, float M)
{
  constexpr float U = 0x1p-24f;
  auto dot3 = [](float a0, float b0, float a1, float b1, float a2, float b2) {
    return Ops::fma(a2, b2, Ops::fma(a1, b1, a0 * b0));
  };
  // cross(B - A, C - A) and the L1 bound on its error
  auto normal = [&](const float* A, const float* B, const float* C, float L, float* n) {
    const float e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    const float e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    n[0] = Ops::fma(e1[1], e2[2], -(e2[1] * e1[2]));
    n[1] = Ops::fma(e2[0], e1[2], -(e1[0] * e2[2]));
    n[2] = Ops::fma(e1[0], e2[1], -(e2[0] * e1[1]));
    const float de = Ops::add_ru(0x1p-23f * M, Ops::mul_ru(U, L));
    return Ops::mul_ru(3.f, Ops::add_ru(Ops::add_ru(Ops::mul_ru(4.f * de, L), Ops::mul_ru(2.f * de, de)),
                                        Ops::mul_ru(0x1p-22f, Ops::mul_ru(L, L))));
  };
  // v / |v| and the L2 bound on its error given |dv|_2 <= dv; false if v is
  // too short to bound
  auto unit = [&](const float* v, float dv, float* o, float& du) {
    const float l2 = dot3(v[0], v[0], v[1], v[1], v[2], v[2]);
    const float len = sqrtf(l2);
    const float gap = Ops::sub_rd(Ops::mul_rd(len, 1.f - 0x1p-21f), dv);
    if(!(gap > 0x1p-100f) || !(gap > dv)) return false;
    const float s = Ops::rsqrt(l2);
    o[0] = v[0] * s, o[1] = v[1] * s, o[2] = v[2] * s;
    du = Ops::add_ru(Ops::div_ru(2.f * dv, gap), 4.f * U);
    return true;
  };
  float n[3], en;
  if(face)
  {
    const float *A, *B, *C;
    float L;
    int k;
    tri(0, A, B, C, L, k);
    en = normal(A, B, C, L, n);
  }
  else
  {
    n[0] = Ops::to_float(sn[0]), n[1] = Ops::to_float(sn[1]), n[2] = Ops::to_float(sn[2]);
    float mag = fabsf(n[0]) + fabsf(n[1]) + fabsf(n[2]);
    en = Ops::mul_ru(U, mag);
    for(int i = 0; i < count; ++i)
    {
      const float *A, *B, *C;
      float L;
      int k;
      tri(i, A, B, C, L, k);
      float nt[3], u[3], du;
      const float dn = normal(A, B, C, L, nt);
      if(k != 3)
      {
        // degenerate (Triangle.hpp:327-330): area = |n| / 2 <= 1e-12
        const float len = sqrtf(dot3(nt[0], nt[0], nt[1], nt[1], nt[2], nt[2]));
        const float lo = Ops::mul_rd(Ops::sub_rd(len, dn), 0.5f - 0x1p-22f);
        const float hi = Ops::mul_ru(Ops::add_ru(len, dn), 0.5f + 0x1p-22f);
        if(hi < 0.999e-12f) continue;  // certainly degenerate: no contribution
        if(!(lo > 1.001e-12f)) return 0.0;
      }
      if(!unit(nt, dn, u, du)) return 0.0;
      float c[3], ec;
      if(k == 3)
      {
        c[0] = u[0], c[1] = u[1], c[2] = u[2];
        ec = Ops::mul_ru(1.7321f, du);
      }
      else
      {
        // Triangle::angle (Triangle.hpp:385-400) at vertex k
        const float* V[3] = {A, B, C};
        const float* pt = V[k];
        const float* p1 = V[(k + 1) % 3];
        const float* p2 = V[(k + 2) % 3];
        const float a[3] = {p1[0] - pt[0], p1[1] - pt[1], p1[2] - pt[2]};
        const float b[3] = {p2[0] - pt[0], p2[1] - pt[1], p2[2] - pt[2]};
        const float de = Ops::mul_ru(1.7321f, Ops::add_ru(0x1p-23f * M, Ops::mul_ru(U, L)));
        float ua[3], ub[3], dua, dub;
        if(!unit(a, de, ua, dua) || !unit(b, de, ub, dub)) return 0.0;
        const float dp = fminf(fmaxf(dot3(ua[0], ub[0], ua[1], ub[1], ua[2], ub[2]), -1.f), 1.f);
        const float ddp = Ops::add_ru(Ops::add_ru(dua, dub), Ops::add_ru(Ops::mul_ru(dua, dub), 4.f * U));
        float dal = Ops::mul_ru(3.1416f, sqrtf(Ops::mul_ru(0.5f, ddp)) * (1.f + 0x1p-20f));
        const float x = Ops::add_ru(fabsf(dp), ddp);
        if(x < 1.f)
          dal = fminf(dal, Ops::div_ru(ddp, Ops::mul_rd(sqrtf(Ops::mul_rd(Ops::sub_rd(1.f, x), Ops::add_rd(1.f, x))),
                                                        1.f - 0x1p-20f)));
        dal = Ops::add_ru(dal, 0x1p-21f);
        const float al = Ops::acos(dp);
        c[0] = u[0] * al, c[1] = u[1] * al, c[2] = u[2] * al;
        // |d(al u)|_1 <= sqrt(3) (dal + (al + dal) du) plus the products' rounding
        ec = Ops::mul_ru(1.7321f, Ops::add_ru(Ops::add_ru(dal, Ops::mul_ru(Ops::add_ru(al, dal), du)), Ops::mul_ru(U, al)));
      }
      n[0] += c[0], n[1] += c[1], n[2] += c[2];
      mag = Ops::add_ru(mag, fabsf(c[0]) + fabsf(c[1]) + fabsf(c[2]));
      // this term's error and the rounding of the running sum
      en = Ops::add_ru(en, Ops::add_ru(ec, Ops::mul_ru(2.f * U, mag)));
    }
  }
  const float s = dot3(r[0], n[0], r[1], n[1], r[2], n[2]);
  const float rmax = fmaxf(fabsf(r[0]), fmaxf(fabsf(r[1]), fabsf(r[2])));
  const float rn = Ops::add_ru(Ops::add_ru(fabsf(r[0] * n[0]), fabsf(r[1] * n[1])), fabsf(r[2] * n[2]));
  const float err = Ops::mul_ru(1.05f, Ops::add_ru(Ops::mul_ru(rmax, en), Ops::mul_ru(5.f * U, rn)));
  if(!(err < INFINITY)) return 0.0;
  if(s > err) return 1.0;
  if(s < -err) return -1.0;
  return 0.0;
}
}  // namespace gsq
