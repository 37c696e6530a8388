// Host check of the FP32 node-visit certificate of the mixed signed distance
// (axom_gb300/csrc/gsq_leaf32.cuh: node_box32, the FP32 child boxes the node
// records hold; qctx_init / qctx_set32, the query context; box_decide and
// visit32_core, the visit the query kernels run) against the FP64 visit
// (squared_distance(Point, BoundingBox) <= minSq per child, the nearer centroid
// first: oracle/gsq_oracle.cpp, the reference's algorithm restated) and exact
// long-double values.
//
// The certificate's FP32 arithmetic runs here with the same round-to-nearest
// operations as on the device (-ffp-contract=off; fmaf is the correctly
// rounded fused multiply-add); its directed roundings are emulated one ulp
// outward, never tighter than the device's.  A context holds an FP32 interval
// [lo, hi] known to contain minSq.  For every certified visit (visit32_core
// returns true) and both children:
//   entered      =>  the box is valid and its FP64 squared distance is <= lo
//                    (the FP64 predicate holds for every minSq in the
//                    interval), with room 2^-45 for any FP64 evaluation order;
//   not entered  =>  the box is invalid or its FP64 squared distance is > hi;
//   both entered =>  swap equals the FP64 centroid comparison, evaluated with
//                    and without fused multiply-adds, and the exact difference
//                    of the FP64 centroids' squared distances has that sign
//                    with room 2^-48 of their sum.
// Usage: node_check <cases> <seed> [mode]; mode 0 unit-sized scenes, 1
// coordinates up to 1e3, 2 boxes of 1e-7..1e-4, 3 points up to 1e2 away.
// Prints counts and exits 1 on a violation.
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

// exact squared distance (long double: 64-bit significand, products of
// doubles' differences exact to 2^-63) from p to a valid box
LD exact_pb(const double* p, const orc::Box& b)
{
  LD s = 0;
  for(int d = 0; d < 3; ++d)
  {
    LD g = 0;
    if(p[d] < b.lo[d]) g = (LD)b.lo[d] - (LD)p[d];
    if(p[d] > b.hi[d]) g = (LD)p[d] - (LD)b.hi[d];
    s += g * g;
  }
  return s;
}

// the FP64 centroid comparison with the device's fused products
// (sqdist_pp: fma(v0, v0, fma(v1, v1, v2 * v2)))
bool pref_fma(const double* q, const orc::Box& l, const orc::Box& r)
{
  double sl, sr;
  {
    const double v0 = 0.5 * (l.lo[0] + l.hi[0]) - q[0], v1 = 0.5 * (l.lo[1] + l.hi[1]) - q[1],
                 v2 = 0.5 * (l.lo[2] + l.hi[2]) - q[2];
    sl = std::fma(v0, v0, std::fma(v1, v1, v2 * v2));
  }
  {
    const double v0 = 0.5 * (r.lo[0] + r.hi[0]) - q[0], v1 = 0.5 * (r.lo[1] + r.hi[1]) - q[1],
                 v2 = 0.5 * (r.lo[2] + r.hi[2]) - q[2];
    sr = std::fma(v0, v0, std::fma(v1, v1, v2 * v2));
  }
  return sl > sr;
}

bool pref_plain(const double* q, const orc::Box& l, const orc::Box& r)
{
  double cl[3], cr[3];
  for(int d = 0; d < 3; ++d) cl[d] = 0.5 * (l.lo[d] + l.hi[d]), cr[d] = 0.5 * (r.lo[d] + r.hi[d]);
  return orc::sq_dist_pp(q, cl) > orc::sq_dist_pp(q, cr);
}

// exact |c_L - q|^2 - |c_R - q|^2 of the FP64 centroids, and their sum
LD exact_pref(const double* q, const orc::Box& l, const orc::Box& r, LD& sum)
{
  LD sl = 0, sr = 0;
  for(int d = 0; d < 3; ++d)
  {
    const LD vl = (LD)(0.5 * (l.lo[d] + l.hi[d])) - (LD)q[d];
    const LD vr = (LD)(0.5 * (r.lo[d] + r.hi[d])) - (LD)q[d];
    sl += vl * vl;
    sr += vr * vr;
  }
  sum = sl + sr;
  return sl - sr;
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
  auto sgn = [&]() { return U01(rng) < 0.5 ? -1.0 : 1.0; };
  long long certified = 0, undecided = 0, both = 0, swaps = 0, entered = 0, excluded = 0, near_tie = 0,
            near_tie_cert = 0;
  long long bad_box = 0, bad_in = 0, bad_out = 0, bad_swap = 0;
  LD m_in = 1e30L, m_out = 1e30L, m_ord = 1e30L;  // smallest certified relative margins
  for(long long k = 0; k < cases; ++k)
  {
    const double R = mode == 1 ? std::pow(10.0, unif(0, 3)) : unif(0.0, 2.0);
    const double s = mode == 2 ? std::pow(10.0, unif(-7, -4)) : std::pow(10.0, unif(-4, 0));
    // the left child: a box of half extents up to s (flat on an axis now and then)
    orc::Box L, Rb;
    double cl[3];
    for(int d = 0; d < 3; ++d)
    {
      cl[d] = unif(-R, R);
      const double h = U01(rng) < 0.125 ? 0.0 : s * unif(0, 1);
      L.lo[d] = cl[d] - h;
      L.hi[d] = cl[d] + h;
    }
    // the point: near the boxes, on a face of L, inside L, or just off a face
    const int qk = (int)((k / 4) % 4);
    double q[3];
    const int ax = (int)(k % 3);
    for(int d = 0; d < 3; ++d)
    {
      if(qk == 0)
      {
        const double D = mode == 3 ? std::pow(10.0, unif(-1, 2)) : s * std::pow(10.0, unif(-1, 1));
        q[d] = cl[d] + D * unif(-1, 1);
      }
      else
        q[d] = L.lo[d] + (L.hi[d] - L.lo[d]) * unif(0, 1);
    }
    if(qk == 1) q[ax] = U01(rng) < 0.5 ? L.lo[ax] : L.hi[ax];
    if(qk == 3) q[ax] = L.hi[ax] + sgn() * s * std::pow(10.0, unif(-12, -3));
    // the right child: a nearby box, a sibling sharing a face, the mirror
    // image of L through a plane through the point (centroids all but
    // equidistant), or a box inside L; invalid boxes now and then
    const int rk = (int)(k % 4);
    for(int d = 0; d < 3; ++d)
    {
      const double h = U01(rng) < 0.125 ? 0.0 : s * unif(0, 1);
      const double c = cl[d] + s * unif(-2, 2);
      Rb.lo[d] = c - h;
      Rb.hi[d] = c + h;
    }
    if(rk == 1)
    {
      const double w = s * unif(0, 1);
      Rb.lo[ax] = L.hi[ax];
      Rb.hi[ax] = L.hi[ax] + w;
    }
    else if(rk == 2)
    {
      double n[3], nn = 0;
      for(int d = 0; d < 3; ++d) n[d] = unif(-1, 1), nn += n[d] * n[d];
      nn = std::sqrt(nn);
      double t = 0;
      for(int d = 0; d < 3; ++d) n[d] /= nn, t += (cl[d] - q[d]) * n[d];
      const double eps = s * std::pow(10.0, unif(-16, -3)) * sgn();
      for(int d = 0; d < 3; ++d)
      {
        const double c = cl[d] - 2 * t * n[d] + eps * unif(-1, 1);
        const double h = 0.5 * (L.hi[d] - L.lo[d]) * unif(0.5, 1.0);
        Rb.lo[d] = c - h;
        Rb.hi[d] = c + h;
      }
    }
    else if(rk == 3)
    {
      for(int d = 0; d < 3; ++d)
      {
        const double a = unif(0, 1), b = unif(0, 1);
        Rb.lo[d] = L.lo[d] + (L.hi[d] - L.lo[d]) * std::min(a, b);
        Rb.hi[d] = L.lo[d] + (L.hi[d] - L.lo[d]) * std::max(a, b);
      }
      if(U01(rng) < 0.3) std::swap(Rb.lo[ax], Rb.hi[ax]);
    }
    if(k % 16 == 5) std::swap(L.lo[(ax + 1) % 3], L.hi[(ax + 1) % 3]);
    if(rk == 0 && k % 16 == 8) Rb = orc::invalid_box();
    // the FP32 node record and the query context
    double b64[12];
    for(int d = 0; d < 3; ++d)
      b64[d] = L.lo[d], b64[3 + d] = L.hi[d], b64[6 + d] = Rb.lo[d], b64[9 + d] = Rb.hi[d];
    float o[12];
    const float sl = node_box32(b64, o), sr = node_box32(b64 + 6, o + 6);
    double mx = 0;
    for(int side = 0; side < 2; ++side)
    {
      const orc::Box& B = side ? Rb : L;
      if(!orc::valid(B)) continue;
      const float* ob = o + 6 * side;
      const float sla = side ? sr : sl;
      for(int d = 0; d < 6; ++d)
      {
        const double v = d < 3 ? B.lo[d] : B.hi[d - 3];
        mx = std::max(mx, std::fabs(v));
        const bool out = d < 3 ? ((double)ob[d] <= v) : ((double)ob[d] >= v);
        if(!out || std::fabs((double)ob[d] - v) > (double)sla) ++bad_box;
      }
    }
    const float mesh_max = gsq::fp::f_ru(mx * unif(1.0, 2.0));
    QCtx c;
    qctx_init(c, q, mesh_max);
    // the interval: round a target (a child's FP64 distance, moved a little)
    // outward as the FP64 refine does, widen it as the lazy queue does, leave
    // it open above, or start from no minimum at all
    const int ik = (int)((k / 16) % 5);
    const double s64 = orc::sq_dist_pb(q, (k / 80) % 2 ? Rb : L);
    double target = s64 == DBL_MAX ? orc::sq_dist_pb(q, (k / 80) % 2 ? L : Rb) : s64;
    if(target == DBL_MAX) target = 1.0;
    if(U01(rng) < 0.7) target *= 1.0 + sgn() * std::pow(10.0, unif(-12, -1));
    float lo = gsq::fp::f_rd(target), hi = gsq::fp::f_ru(target);
    if(ik == 2)
    {
      const double w = std::pow(10.0, unif(-6, -1));
      lo = gsq::fp::f_rd(target * (1 - w));
      hi = gsq::fp::f_ru(target * (1 + w));
    }
    if(ik == 3) hi = INFINITY;
    if(ik == 4)
    {
      qctx_update(c, DBL_MAX);
      lo = gsq::fp::f_rd(DBL_MAX);
      hi = INFINITY;
    }
    else
      qctx_set32(c, lo, hi);
    bool inL = false, inR = false, swap = false;
    if(!visit32_core(o, o + 3, o + 6, o + 9, sl, sr, c, inL, inR, swap))
    {
      ++undecided;
      continue;
    }
    ++certified;
    for(int side = 0; side < 2; ++side)
    {
      const orc::Box& B = side ? Rb : L;
      const bool in = side ? inR : inL;
      const double f64 = orc::sq_dist_pb(q, B);
      if(in)
      {
        ++entered;
        const bool ok = orc::valid(B) && f64 <= (double)lo && exact_pb(q, B) * (1 + 0x1p-45L) <= (LD)lo;
        if(lo > 0) m_in = std::min(m_in, ((LD)lo - exact_pb(q, B)) / (LD)lo);
        if(!ok && bad_in++ < 5)
          std::printf("entered violation: side %d f64 %.17g lo %.9g hi %.9g\n", side, f64, (double)lo, (double)hi);
      }
      else
      {
        ++excluded;
        const bool ok = !orc::valid(B) || (f64 > (double)hi && exact_pb(q, B) * (1 - 0x1p-45L) > (LD)hi);
        if(orc::valid(B) && hi > 0) m_out = std::min(m_out, (exact_pb(q, B) - (LD)hi) / (LD)hi);
        if(!ok && bad_out++ < 5)
          std::printf("excluded violation: side %d f64 %.17g lo %.9g hi %.9g\n", side, f64, (double)lo, (double)hi);
      }
    }
    LD sum = 0;
    const LD dx = exact_pref(q, L, Rb, sum);
    const bool tie = std::fabs(dx) <= 1e-6L * sum;
    if(rk == 2) near_tie += tie;
    if(inL && inR)
    {
      ++both;
      swaps += swap;
      near_tie_cert += (rk == 2 && tie);
      if(sum > 0) m_ord = std::min(m_ord, std::fabs(dx) / sum);
      const bool ok = swap == pref_plain(q, L, Rb) && swap == pref_fma(q, L, Rb) &&
                      (swap ? dx > 0x1p-48L * sum : -dx > 0x1p-48L * sum);
      if(!ok && bad_swap++ < 5)
        std::printf("order violation: swap %d exact difference %.6Lg of %.6Lg\n", (int)swap, dx, sum);
    }
  }
  std::printf("cases %lld certified %lld undecided %lld both %lld swaps %lld entered %lld excluded %lld "
              "mirror near-ties %lld (certified with both children %lld) | violations: box %lld entered %lld "
              "excluded %lld order %lld\n",
              cases, certified, undecided, both, swaps, entered, excluded, near_tie, near_tie_cert, bad_box, bad_in,
              bad_out, bad_swap);
  std::printf("smallest certified margins (relative): entered %.3Lg excluded %.3Lg order %.3Lg\n", m_in, m_out,
              m_ord);
  return (bad_box || bad_in || bad_out || bad_swap) ? 1 : 0;
}
