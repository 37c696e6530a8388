// Host check of the FP32 enclosure of a query-to-object-point squared
// distance (axom_gb300/csrc/gsq_leaf32.cuh: qctx_init and point_bounds32, the
// code the mixed closest-point kernel runs) against the FP64 squared distance
// the reference computes (squared_distance(Point, Point): the oracle's
// sq_dist_pp, oracle/gsq_oracle.cpp) and its exact long-double value.
//
// The certificate's FP32 arithmetic runs here with the same round-to-nearest
// operations as on the device (-ffp-contract=off; fmaf is the correctly
// rounded fused multiply-add); its directed roundings are emulated one ulp
// outward, never tighter than the device's.  For every case the FP64 value
// must lie in [lo2, hi2].  M, the bound on the object points' coordinates, is
// the tightest the library uses (max |p| times 1 + 1e-6).
// Usage: point_check <cases> <seed> <mode>; mode 0 unit-sized scenes, 1
// coordinates up to 1e3 with nearby points, 2 points within 1e-20..1e-5 of the
// query or on it, 3 queries up to 1e2 away.  Prints counts and exits 1 on a
// violation.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../oracle/gsq_oracle.cpp"
#include "../../axom_gb300/csrc/gsq_leaf32.cuh"

int main(int argc, char** argv)
{
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 1000000;
  const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1;
  const int mode = argc > 3 ? std::atoi(argv[3]) : 0;
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0), E(0.0, 1.0);
  long long bad = 0, decided = 0, tight = 0;
  double worst = 0.0;
  for(long long k = 0; k < cases; ++k)
  {
    double q[3], p[3];
    const double scale = (mode == 1) ? std::pow(10.0, 3.0 * E(g)) : 1.0;
    for(int d = 0; d < 3; ++d) q[d] = U(g) * scale;
    if(mode == 0)
      for(int d = 0; d < 3; ++d) p[d] = U(g);
    else if(mode == 1)
    {
      const double off = std::pow(10.0, -8.0 + 8.0 * E(g));
      for(int d = 0; d < 3; ++d) p[d] = q[d] + U(g) * off * scale;
    }
    else if(mode == 2)
    {
      const double off = (k % 10 == 0) ? 0.0 : std::pow(10.0, -20.0 + 15.0 * E(g));
      for(int d = 0; d < 3; ++d) p[d] = q[d] + U(g) * off;
    }
    else
    {
      for(int d = 0; d < 3; ++d) q[d] = U(g) * 100.0;
      for(int d = 0; d < 3; ++d) p[d] = U(g);
    }
    double M = 0.0;
    for(int d = 0; d < 3; ++d) M = std::fmax(M, std::fabs(p[d]));
    gsq::sdf::QCtx c;
    gsq::sdf::qctx_init(c, q, (float)(M * (1.0 + 1e-6)));
    const float pf[3] = {(float)p[0], (float)p[1], (float)p[2]};
    float lo2, hi2;
    gsq::sdf::point_bounds32(c, pf, lo2, hi2);
    const double sq = orc::sq_dist_pp(q, p);
    long double ex = 0;
    for(int d = 0; d < 3; ++d) ex += ((long double)p[d] - q[d]) * ((long double)p[d] - q[d]);
    if(!((long double)lo2 <= (long double)sq && (long double)sq <= (long double)hi2 && (long double)lo2 <= ex &&
         ex <= (long double)hi2))
    {
      if(bad < 5)
        std::printf("violation: q %.17g %.17g %.17g p %.17g %.17g %.17g sq %.17g [%.9g, %.9g]\n", q[0], q[1], q[2],
                    p[0], p[1], p[2], sq, lo2, hi2);
      ++bad;
    }
    if(hi2 < INFINITY)
    {
      ++decided;
      if(sq > 0.0)
      {
        const double w = ((double)hi2 - (double)lo2) / sq;
        worst = std::fmax(worst, w);
        if(w < 1e-5) ++tight;
      }
    }
  }
  std::printf("cases %lld bounded %lld tight %lld violations %lld | widest relative %.3g\n", cases, decided, tight, bad,
              worst);
  return bad ? 1 : 0;
}
