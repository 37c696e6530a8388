// Host check of the FP32 leaf certificate of the mixed signed distance
// (axom_gb300/csrc/gsq_leaf32.cuh: the leaf records' error terms, the query
// context, tri_bounds) against the oracle's FP64 closest_point (the reference's
// algorithm restated, oracle/gsq_oracle.cpp) and an exact long-double distance.
//
// The certificate's FP32 arithmetic runs here with the same round-to-nearest
// operations as on the device (-ffp-contract=off; fmaf is the correctly
// rounded fused multiply-add); its directed roundings are emulated one ulp
// outward, never tighter than the device's.  For every case:
//   skipped (false)  =>  the FP64 distance exceeds thr_leaf;
//   kept (true)      =>  l2 <= FP64 squared distance <= h2 and
//                        |cpf - FP64 closest point| <= rad.
// Usage: leaf_check <cases> <seed> [mode]; mode 0 mixed sizes, 1 coordinates
// up to 1e3, 2 triangles of 1e-6..1e-4, 3 points up to 1e2 away, 4 triangles
// of 1e-6..1e-4 at coordinates up to 1e3.  Prints counts and exits 1 on a
// violation.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../oracle/gsq_oracle.cpp"
#include "../../axom_gb300/csrc/gsq_leaf32.cuh"

namespace
{
typedef long double LD;

LD seg_dist2(const LD* p, const LD* a, const LD* b)
{
  LD e[3], v[3];
  for(int d = 0; d < 3; ++d) e[d] = b[d] - a[d], v[d] = p[d] - a[d];
  const LD ee = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
  LD t = ee > 0 ? (v[0] * e[0] + v[1] * e[1] + v[2] * e[2]) / ee : 0;
  t = t < 0 ? 0 : t > 1 ? 1 : t;
  LD s = 0;
  for(int d = 0; d < 3; ++d)
  {
    const LD w = v[d] - t * e[d];
    s += w * w;
  }
  return s;
}

// exact distance (long double) from p to the triangle abc
LD exact_dist(const double* pd, const double* ad, const double* bd, const double* cd)
{
  LD p[3], a[3], b[3], c[3];
  for(int d = 0; d < 3; ++d) p[d] = pd[d], a[d] = ad[d], b[d] = bd[d], c[d] = cd[d];
  LD e1[3], e2[3], v[3];
  for(int d = 0; d < 3; ++d) e1[d] = b[d] - a[d], e2[d] = c[d] - a[d], v[d] = p[d] - a[d];
  const LD d11 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  const LD d12 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
  const LD d22 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
  const LD dv1 = v[0] * e1[0] + v[1] * e1[1] + v[2] * e1[2];
  const LD dv2 = v[0] * e2[0] + v[1] * e2[1] + v[2] * e2[2];
  const LD den = d11 * d22 - d12 * d12;
  LD best = seg_dist2(p, a, b);
  best = std::min(best, seg_dist2(p, a, c));
  best = std::min(best, seg_dist2(p, b, c));
  if(den > 0)
  {
    const LD s = (d22 * dv1 - d12 * dv2) / den, t = (d11 * dv2 - d12 * dv1) / den;
    if(s >= 0 && t >= 0 && s + t <= 1)
    {
      LD w2 = 0;
      for(int d = 0; d < 3; ++d)
      {
        const LD w = v[d] - s * e1[d] - t * e2[d];
        w2 += w * w;
      }
      best = std::min(best, w2);
    }
  }
  return std::sqrt(best);
}

}  // namespace

int main(int argc, char** argv)
{
  using namespace gsq::sdf;
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 200000;
  const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1;
  const int mode = argc > 3 ? std::atoi(argv[3]) : 0;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U01(0.0, 1.0);
  auto unif = [&](double a, double b) { return a + (b - a) * U01(rng); };
  long long skipped = 0, kept = 0, bad_skip = 0, bad_lo = 0, bad_hi = 0, bad_cp = 0, tight = 0;
  double max_cp = 0, min_lo = 1e300, min_hi = 1e300;
  for(long long k = 0; k < cases; ++k)
  {
    // a triangle: small (fine meshes), unit-sized, or a sliver, at a random place
    const int kind = (int)(k % 4);
    double scale = kind == 2 ? unif(0.1, 1.0) : std::pow(10.0, unif(-3.5, -1.5));
    if(mode == 2 || mode == 4) scale = std::pow(10.0, unif(-6, -4));
    const double R = (mode == 1 || mode == 4) ? std::pow(10.0, unif(0, 3)) : unif(0.0, 2.0);
    double A[3], B[3], C[3];
    for(int d = 0; d < 3; ++d) A[d] = unif(-R, R);
    for(int d = 0; d < 3; ++d) B[d] = A[d] + scale * unif(-1, 1);
    if(kind == 3)
    {
      const double t = unif(-0.2, 1.2), off = scale * std::pow(10.0, unif(-7, -2));
      for(int d = 0; d < 3; ++d) C[d] = A[d] + t * (B[d] - A[d]) + off * unif(-1, 1);
    }
    else
      for(int d = 0; d < 3; ++d) C[d] = A[d] + scale * unif(-1, 1);
    // a point: far, near the plane over the triangle, or in its plane
    const int pk = (int)((k / 4) % 3);
    double q[3];
    if(pk == 0)
    {
      const double D = std::pow(10.0, mode == 3 ? unif(-1, 2) : unif(-3, 0));
      for(int d = 0; d < 3; ++d) q[d] = A[d] + D * unif(-1, 1);
    }
    else
    {
      const double n[3] = {(B[1] - A[1]) * (C[2] - A[2]) - (B[2] - A[2]) * (C[1] - A[1]),
                           (B[2] - A[2]) * (C[0] - A[0]) - (B[0] - A[0]) * (C[2] - A[2]),
                           (B[0] - A[0]) * (C[1] - A[1]) - (B[1] - A[1]) * (C[0] - A[0])};
      const double ln = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if(!(ln > 0)) continue;
      const double s = unif(-0.3, 1.1), t = unif(-0.3, 1.1);
      const double h = (pk == 1) ? (unif(0, 1) < 0.5 ? -1 : 1) * std::pow(10.0, unif(-9, -2)) : 0.0;
      for(int d = 0; d < 3; ++d) q[d] = A[d] + s * (B[d] - A[d]) + t * (C[d] - A[d]) + h * n[d] / ln;
    }
    // the FP32 record as the leaf records hold it, and the query context
    const double* V[3] = {A, B, C};
    float v[9];
    double Mx = 0;
    for(int j = 0; j < 3; ++j)
      for(int d = 0; d < 3; ++d)
      {
        v[3 * j + d] = (float)V[j][d];
        Mx = std::max(Mx, std::fabs(V[j][d]));
      }
    const float M = gsq::fp::f_ru(Mx);
    float ec, lt, fz;
    tri_error_terms(A, B, C, ec, lt, &fz);
    QCtx c;
    qctx_init(c, q, M);
    // the FP64 reference and the exact distance
    double cp[3];
    int loc = 0;
    orc::closest_point(q, A, B, C, 1e-12, cp, &loc);
    const double sq64 = orc::sq_dist_pp(q, cp);
    const LD dex = exact_dist(q, A, B, C);
    // a minimum near this triangle's distance, so both outcomes occur
    const double rel = (unif(0, 1) < 0.5 ? -1 : 1) * std::pow(10.0, unif(-8, -0.5));
    const double mind = std::max(0.0, (double)dex * (1.0 + rel) - 1e-6 * unif(0, 2));
    const float hi = gsq::fp::f_ru(mind * mind);
    qctx_set32(c, gsq::fp::f_rd(mind * mind * (1 - 1e-6)), hi);
    float d2, l2, h2, cpf[3], rad;
    const bool quad = (k / 12) % 2 == 1;  // a quad's triangle derives fz from ec and lt
    const bool keep = quad ? tri_bounds<true>(c, M, v, v + 3, v + 6, ec, lt, 0.f, d2, l2, h2, cpf, rad)
                           : tri_bounds<false>(c, M, v, v + 3, v + 6, ec, lt, fz, d2, l2, h2, cpf, rad);
    if(!keep)
    {
      ++skipped;
      if(!(std::sqrt(sq64) > (double)c.thr_leaf))
      {
        if(bad_skip < 5) std::printf("skip violation: d64 %.17g thr %.9g\n", std::sqrt(sq64), (double)c.thr_leaf);
        ++bad_skip;
      }
      continue;
    }
    ++kept;
    // as the kernel combines them: a NaN distance gives [0, inf), a NaN upper
    // end inf, and an infinite radius certifies nothing
    if(!(d2 == d2)) l2 = 0.f;
    if(!(d2 == d2 && h2 == h2)) h2 = INFINITY;
    if(!((double)l2 <= sq64))
    {
      if(bad_lo < 5) std::printf("lo violation: l2 %.9g sq64 %.17g kind %d\n", (double)l2, sq64, kind);
      ++bad_lo;
    }
    if(!(sq64 <= (double)h2))
    {
      if(bad_hi < 5) std::printf("hi violation: h2 %.9g sq64 %.17g kind %d\n", (double)h2, sq64, kind);
      ++bad_hi;
    }
    const double e = std::sqrt((cpf[0] - cp[0]) * (cpf[0] - cp[0]) + (cpf[1] - cp[1]) * (cpf[1] - cp[1]) +
                               (cpf[2] - cp[2]) * (cpf[2] - cp[2]));
    if(rad < INFINITY) max_cp = std::max(max_cp, e / (double)rad);
    {
      const double d64 = std::sqrt(sq64), lo = std::sqrt((double)l2), hi = std::sqrt((double)h2);
      if(hi < INFINITY && hi > lo && d64 > 0)
      {
        min_lo = std::min(min_lo, (d64 - lo) / (hi - lo));
        min_hi = std::min(min_hi, (hi - d64) / (hi - lo));
      }
    }
    if(rad < INFINITY && !(e <= (double)rad))
    {
      if(bad_cp < 5) std::printf("rad violation: |cpf - cp64| %.9g rad %.9g kind %d\n", e, (double)rad, kind);
      ++bad_cp;
    }
    if(h2 < INFINITY && (double)h2 - (double)l2 < 1e-3 * (double)h2) ++tight;
  }
  std::printf("cases %lld skipped %lld kept %lld (interval within 0.1%%: %lld) | violations: skip %lld lo %lld hi %lld "
              "rad %lld\n",
              cases, skipped, kept, tight, bad_skip, bad_lo, bad_hi, bad_cp);
  std::printf("smallest margins (fraction of the interval): below %.3g above %.3g; largest |cpf - cp| / rad %.3g\n",
              min_lo, min_hi, max_cp);
  return (bad_skip || bad_lo || bad_hi || bad_cp) ? 1 : 0;
}
