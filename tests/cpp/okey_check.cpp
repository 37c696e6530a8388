// Host check of the exact FP64 comparisons on the integer pipe
// (axom_gb300/csrc/gsq_internal.cuh: okey and ok_lt / ok_gt / ok_le / ok_ge /
// ok_eq / box_valid_k and the comparisons with +-1e-12 gt_eps / lt_neg_eps /
// abs_le_eps, which the BVH build, the candidate queries and the
// signed-distance kernels use in place of FP64 comparisons): every result must
// equal the IEEE comparison of the two doubles, on special values (signed
// zeros, subnormals, the extremes, infinities, NaNs with either sign and any
// payload) and on random bit patterns, near and far apart.
// Usage: okey_check <cases> <seed>.  Prints counts and exits 1 on a mismatch.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../../axom_gb300/csrc/gsq_internal.cuh"

static double from_bits(uint64_t u)
{
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

int main(int argc, char** argv)
{
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 10000000;
  std::mt19937_64 g(argc > 2 ? std::atoi(argv[2]) : 1);
  long long bad = 0, checked = 0;
  auto check = [&](double a, double b) {
    const gsq::OKey x = gsq::okey(a), y = gsq::okey(b);
    ++checked;
    if(gsq::ok_lt(x, y) != (a < b) || gsq::ok_gt(x, y) != (a > b) || gsq::ok_le(x, y) != (a <= b) ||
       gsq::ok_ge(x, y) != (a >= b) || gsq::ok_eq(x, y) != (a == b))
    {
      if(bad < 5) std::printf("mismatch: %a %a\n", a, b);
      ++bad;
    }
  };
  const double sp[] = {0.0, -0.0, 1.0, -1.0, DBL_MIN, -DBL_MIN, 4.9e-324, -4.9e-324, DBL_MAX, -DBL_MAX, INFINITY,
                       -INFINITY, NAN, -NAN, from_bits(0x7FF0000000000001ull), from_bits(0xFFF0000000000001ull),
                       from_bits(0x7FF8000000000000ull), 1e-12, -1e-12, 3.0, std::nextafter(3.0, 4.0),
                       std::nextafter(-3.0, -4.0), from_bits(0x00000000FFFFFFFFull), from_bits(0x0000000100000000ull)};
  for(double a : sp)
    for(double b : sp) check(a, b);
  for(long long i = 0; i < cases; ++i)
  {
    const uint64_t u = g();
    uint64_t v;
    switch(i % 4)
    {
    case 0: v = g(); break;                                    // unrelated
    case 1: v = u + (g() % 7) - 3; break;                      // adjacent
    case 2: v = u ^ (1ull << (g() % 64)); break;               // one bit apart (sign, high/low word)
    default: v = (u & 0xFFFFFFFF00000000ull) | (g() & 0xFFFFFFFFull);  // same high word
    }
    check(from_bits(u), from_bits(v));
  }
  // the comparisons with +-1e-12 of closest_point's fuzzy tests
  const double eps = 1e-12;
  auto check_eps = [&](double x) {
    ++checked;
    if(gsq::gt_eps(x) != (x > eps) || gsq::lt_neg_eps(x) != (x < -eps) || gsq::abs_le_eps(x) != (std::fabs(x) <= eps))
    {
      if(bad < 5) std::printf("eps mismatch: %a\n", x);
      ++bad;
    }
  };
  for(double a : sp) check_eps(a);
  for(double a : {eps, -eps, std::nextafter(eps, 1.0), std::nextafter(eps, 0.0), -std::nextafter(eps, 1.0),
                  -std::nextafter(eps, 0.0)})
    check_eps(a);
  for(long long i = 0; i < cases; ++i)
  {
    check_eps(from_bits(g()));
    check_eps(std::ldexp((double)(g() % 2001) / 1000.0 - 1.0, -(int)(g() % 80)));
  }
  // box_valid_k against BoundingBox::isValid's "no lo > hi"
  for(long long i = 0; i < cases / 10; ++i)
  {
    double lo[3], hi[3];
    gsq::OKey kl[3], kh[3];
    for(int d = 0; d < 3; ++d)
    {
      lo[d] = (g() % 5 == 0) ? sp[g() % (sizeof(sp) / sizeof(sp[0]))] : from_bits(g());
      hi[d] = (g() % 3 == 0) ? lo[d] : from_bits(g());
      kl[d] = gsq::okey(lo[d]);
      kh[d] = gsq::okey(hi[d]);
    }
    ++checked;
    if(gsq::box_valid_k(kl, kh) != gsq::box_valid(lo, hi))
    {
      if(bad < 5) std::printf("box mismatch\n");
      ++bad;
    }
  }
  std::printf("checked %lld mismatches %lld\n", checked, bad);
  return bad ? 1 : 0;
}
