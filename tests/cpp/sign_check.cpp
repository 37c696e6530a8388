// Host check of the FP32 sign certificate (axom_gb300/csrc/gsq_sign.cuh)
// against the sign test of the oracle (oracle/gsq_oracle.cpp, the reference's
// algorithm restated): dot(q - cp, N) >= 0 with N the closest face's normal,
// or the pseudo-normal sum of a shared vertex (angle-weighted unit normals,
// degenerate triangles skipped) or edge (unit normals), in order.
//
// The certificate's FP32 arithmetic runs here with the same round-to-nearest
// operations as on the device (-ffp-contract=off; fmaf is the correctly
// rounded fused multiply-add); its directed roundings are emulated one ulp
// outward, never tighter than the device's, and the reciprocal square root and
// arccosine are evaluated in FP64 and rounded.  Whenever the certificate gives
// a sign it must be the FP64 test's.
// Usage: sign_check <cases> <seed> [mode]; mode 1 places the geometry at
// coordinates up to 1e3 (default: up to 2).  Prints counts, exits 1 on a
// violation.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <cstring>
#include <random>
#include <vector>

#include "../../oracle/gsq_oracle.cpp"
#include "../../axom_gb300/csrc/gsq_sign.cuh"

namespace
{
struct HostOps
{
  static float fma(float a, float b, float c) { return std::fmaf(a, b, c); }
  static float add_ru(float a, float b) { return std::nextafterf(a + b, INFINITY); }
  static float add_rd(float a, float b) { return std::nextafterf(a + b, -INFINITY); }
  static float sub_rd(float a, float b) { return std::nextafterf(a - b, -INFINITY); }
  static float mul_ru(float a, float b) { return std::nextafterf(a * b, INFINITY); }
  static float mul_rd(float a, float b) { return std::nextafterf(a * b, -INFINITY); }
  static float div_ru(float a, float b) { return std::nextafterf(a / b, INFINITY); }
  static float rsqrt(float a) { return (float)(1.0 / std::sqrt((double)a)); }
  static float acos(float a) { return (float)std::acos((double)a); }
  static float to_float(double a) { return (float)a; }
};

// one triangle as the FP32 leaf records hold it
struct Tri32
{
  float v[9];
  float L;  // longest edge * 1.0001, rounded up
  int k;    // contribution kind: vertex index 0..2, or 3 for an edge
};

Tri32 make_tri(const double* A, const double* B, const double* C, int k)
{
  Tri32 t;
  const double* P[3] = {A, B, C};
  for(int j = 0; j < 3; ++j)
    for(int d = 0; d < 3; ++d) t.v[3 * j + d] = (float)P[j][d];
  double L = 0;
  for(int j = 0; j < 3; ++j)
  {
    const double* a = P[j];
    const double* b = P[(j + 1) % 3];
    L = std::max(L, std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                              (a[2] - b[2]) * (a[2] - b[2])));
  }
  t.L = std::nextafterf((float)(L * 1.0001), INFINITY);
  t.k = k;
  return t;
}
}  // namespace

int main(int argc, char** argv)
{
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 100000;
  const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1;
  const int mode = argc > 3 ? std::atoi(argv[3]) : 0;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U01(0.0, 1.0);
  std::normal_distribution<double> G(0.0, 1.0);
  auto unif = [&](double a, double b) { return a + (b - a) * U01(rng); };
  auto normalize = [](double* v) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for(int d = 0; d < 3; ++d) v[d] /= l;
  };
  long long certified[3] = {0, 0, 0}, total[3] = {0, 0, 0}, bad = 0;
  for(long long c = 0; c < cases; ++c)
  {
    const int kind = (int)(c % 3);  // 0 face, 1 shared vertex, 2 shared edge
    const double R = mode == 1 ? std::pow(10.0, unif(0, 3)) : unif(0.0, 2.0);
    double V[3], e1[3], e2[3], e3[3], g[3];
    for(int d = 0; d < 3; ++d) V[d] = unif(-R, R), e3[d] = G(rng), g[d] = G(rng);
    normalize(e3);
    orc::cross3(e3, g, e1);
    normalize(e1);
    orc::cross3(e3, e1, e2);
    const double scale = std::pow(10.0, unif(-4, -0.5));
    double P[10][3];          // vertices
    std::vector<Tri32> tris;  // the triangles the certificate reads
    std::vector<std::array<double, 3>> terms;  // FP64 pseudo-normal terms, in order
    double N[3] = {0, 0, 0}, cp[3];
    bool face = false;
    if(kind == 0)
    {
      // a face: N is the triangle's normal, cp the FP64 closest point
      for(int d = 0; d < 3; ++d)
      {
        P[0][d] = V[d];
        P[1][d] = V[d] + scale * G(rng);
        P[2][d] = V[d] + scale * G(rng);
      }
      orc::tri_normal(P[0], P[1], P[2], N);
      tris.push_back(make_tri(P[0], P[1], P[2], 0));
      face = true;
    }
    else if(kind == 1)
    {
      // a closed fan of m triangles around V, V at a random index of each
      // (angle-weighted unit normals; slivers and near-degenerate triangles)
      const int m = 3 + (int)(rng() % 6);
      std::vector<double> th(m);
      for(int i = 0; i < m; ++i) th[i] = unif(0, 2 * M_PI);
      std::sort(th.begin(), th.end());
      if(rng() % 4 == 0) th[1] = th[0] + std::pow(10.0, unif(-12, -3));
      std::memcpy(P[0], V, 24);
      for(int i = 0; i < m; ++i)
      {
        const double rho = scale * std::pow(10.0, unif(-1, 0));
        const double h = (rng() % 2 ? 1 : -1) * std::pow(10.0, unif(-7, 0)) * rho;
        for(int d = 0; d < 3; ++d)
          P[i + 1][d] = V[d] + rho * (std::cos(th[i]) * e1[d] + std::sin(th[i]) * e2[d]) + h * e3[d];
      }
      for(int i = 0; i < m; ++i)
      {
        const int rot = (int)(rng() % 3);
        const double* cyc[3] = {P[0], P[1 + i], P[1 + (i + 1) % m]};
        const double* T[3];
        for(int j = 0; j < 3; ++j) T[j] = cyc[(j + 3 - rot) % 3];
        tris.push_back(make_tri(T[0], T[1], T[2], rot));
        std::array<double, 3> t = {0, 0, 0};
        if(!orc::tri_degenerate(T[0], T[1], T[2]))
        {
          const double alpha = orc::tri_angle(T, rot);
          double n[3], u[3];
          orc::tri_normal(T[0], T[1], T[2], n);
          orc::unit3(n, u);
          for(int d = 0; d < 3; ++d) t[d] = u[d] * alpha;
          terms.push_back(t);
        }
        else
          terms.push_back({NAN, 0, 0});  // skipped by the reference
      }
      std::memcpy(cp, V, 24);
    }
    else
    {
      // an edge V..Q shared by two triangles (opposite orientations along it,
      // third vertices on either side, bent out of plane): unit normals
      double* Q = P[1];
      double* R1 = P[2];
      double* R2 = P[3];
      for(int d = 0; d < 3; ++d)
      {
        Q[d] = V[d] + scale * e1[d];
        R1[d] = V[d] + scale * (0.5 * e1[d] + unif(0.1, 1) * e2[d] + unif(-1, 1) * std::pow(10.0, unif(-6, 0.3)) * e3[d]);
        R2[d] = V[d] + scale * (0.5 * e1[d] - unif(0.1, 1) * e2[d] + unif(-1, 1) * std::pow(10.0, unif(-6, 0.3)) * e3[d]);
      }
      std::memcpy(P[0], V, 24);
      for(int i = 0; i < 2; ++i)
      {
        const double* cyc[3] = {i == 0 ? P[0] : Q, i == 0 ? Q : P[0], i == 0 ? R1 : R2};
        const int rot = (int)(rng() % 3);
        const double* T[3];
        for(int j = 0; j < 3; ++j) T[j] = cyc[(j + 3 - rot) % 3];
        tris.push_back(make_tri(T[0], T[1], T[2], 3));
        double n[3], u[3];
        orc::tri_normal(T[0], T[1], T[2], n);
        orc::unit3(n, u);
        terms.push_back({u[0], u[1], u[2]});
      }
      const double t = unif(0.01, 0.99);
      for(int d = 0; d < 3; ++d) cp[d] = V[d] + t * (Q[d] - V[d]);
    }
    // the FP64 pseudo-normal: the terms summed in order; the first `first`
    // are in sn (evaluated earlier), the rest pending for the certificate
    int first = 0;
    double sn[3] = {0, 0, 0};
    if(!face)
    {
      first = (int)(rng() % (terms.size() + 1));
      for(size_t i = 0; i < terms.size(); ++i)
      {
        if(std::isnan(terms[i][0])) continue;
        for(int d = 0; d < 3; ++d) N[d] = N[d] + terms[i][d];
        if((int)i + 1 == first)
          for(int d = 0; d < 3; ++d) sn[d] = N[d];
      }
      if(first > 0 && std::isnan(terms[first - 1][0]))
      {
        // sn is the sum of the evaluated terms before `first`
        double acc[3] = {0, 0, 0};
        for(int i = 0; i < first; ++i)
          if(!std::isnan(terms[i][0]))
            for(int d = 0; d < 3; ++d) acc[d] = acc[d] + terms[i][d];
        std::memcpy(sn, acc, 24);
      }
    }
    // the query: from cp along a direction between the normal and the
    // tangent plane, at distances 1e-9..1 times the scale
    double q[3], dir[3];
    const double tilt = std::pow(10.0, unif(-8, 0));
    const double sgnq = rng() % 2 ? 1.0 : -1.0;
    for(int d = 0; d < 3; ++d) dir[d] = sgnq * e3[d] + tilt * (G(rng) * e1[d] + G(rng) * e2[d]) * 10;
    normalize(dir);
    const double D = scale * std::pow(10.0, unif(-9, 1));
    for(int d = 0; d < 3; ++d) q[d] = cp[d] + D * dir[d];
    if(face)
    {
      int loc;
      orc::closest_point(q, P[0], P[1], P[2], 1e-12, cp, &loc);
    }
    // FP64 test (SD:751-763) and the certificate
    const double r64[3] = {q[0] - cp[0], q[1] - cp[1], q[2] - cp[2]};
    const double s64 = (orc::dot3(r64, N) >= 0.0) ? 1.0 : -1.0;
    const float r32[3] = {(float)r64[0], (float)r64[1], (float)r64[2]};
    double Mx = 0;
    for(const Tri32& t : tris)
      for(int j = 0; j < 9; ++j) Mx = std::max(Mx, std::fabs((double)t.v[j]));
    const float M = std::nextafterf((float)(Mx * 1.0000001), INFINITY);
    auto tri = [&](int i, const float*& A, const float*& B, const float*& C, float& L, int& k) {
      const Tri32& t = tris[face ? 0 : first + i];
      A = t.v, B = t.v + 3, C = t.v + 6, L = t.L, k = t.k;
    };
    const int count = face ? 1 : (int)tris.size() - first;
    const double s32 = gsq::sign_certificate<HostOps>(r32, face, sn, count, tri, M);
    ++total[kind];
    if(s32 != 0.0)
    {
      ++certified[kind];
      if(s32 != s64)
      {
        if(bad < 5) std::printf("violation: kind %d certified %+.0f FP64 %+.0f (|r| %.3g)\n", kind, s32, s64, D);
        ++bad;
      }
    }
  }
  std::printf("certified: face %lld/%lld vertex %lld/%lld edge %lld/%lld | violations %lld\n", certified[0], total[0],
              certified[1], total[1], certified[2], total[2], bad);
  return bad ? 1 : 0;
}
