// Mixed-precision signed distance: FP32 certified traversal, FP64 refine.
//
// The kernel replays the reference's per-point traversal (bvh_traverse.hpp:
// 66-154 with the point preference of policy/LinearBVH.hpp:72-85 and
// checkCandidate, quest/SignedDistance.hpp:636-737) in the same order, but
// decides each step in FP32 interval arithmetic where the decision is certain:
//   * child predicate  squared_distance(p, box) <= minSq  (SD:576-578): the
//     FP32 copies of the boxes are rounded outward (lo down, hi up) and carry
//     their rounding slack, so a lower bound L and an upper bound H of the
//     FP64 box distance follow with directed rounding; L > minSq(1+2^-40) is
//     certainly false, H <= minSq(1-2^-40) certainly true;
//   * child order      |c_L - p|^2 > |c_R - p|^2: decided in FP32 when the gap
//     exceeds a bound on the FP32 error;
//   * leaf action      a triangle whose distance certainly exceeds
//     sqrt(minSq) + 1e-6 can neither lower the minimum nor join the
//     pseudo-normal sum (that needs |cp - minPt| <= 1e-6, SD:690, 709), so
//     checkCandidate would leave the state unchanged: it is skipped.  The
//     certificate is the FP32 point-triangle distance minus an error bound
//     (coordinate rounding plus a conditioning term kappa = L^2 / |n| stored
//     per triangle).
// Anything not certain is evaluated exactly as the FP64 kernel does, from the
// FP64 node and leaf records.  Every state change therefore happens in FP64
// on the same inputs in the same order as the reference, and distances,
// closest points and signs equal the FP64 path bit for bit.
#include "gsq_sdf_device.cuh"

#include <algorithm>

namespace gsq
{
template <int NPC>
struct LeafRec32;
// FP32 triangle(s) of one leaf: vertices rounded to nearest, and per
// triangle the error factor ec = 256 * 2^-24 * kappa and max edge length lt.
template <>
struct __align__(16) LeafRec32<3>
{
  float v[9];
  float ec;
  float lt;
  float pad;
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

namespace
{
using namespace sdf;

// FP64 node records -> FP32 records with outward rounding.  Invalid boxes
// become (+inf, -inf) so that validity stays exact; pad[k] holds the slack
// (max rounding distance) of child k's box as float bits.
__global__ void k_nodes32(const NodeRec64* __restrict__ in, int n_inner, NodeRec32* __restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n_inner) return;
  NodeRec32 r;
  for(int side = 0; side < 2; ++side)
  {
    const double* b = in[i].b + 6 * side;
    float* o = r.b + 6 * side;
    float slack = 0.f;
    if(!box_valid(b, b + 3))
    {
      for(int d = 0; d < 3; ++d)
      {
        o[d] = INFINITY;
        o[3 + d] = -INFINITY;
      }
    }
    else
    {
      double s = 0.0;
      for(int d = 0; d < 3; ++d)
      {
        o[d] = __double2float_rd(b[d]);
        o[3 + d] = __double2float_ru(b[3 + d]);
        s = fmax(s, fmax(b[d] - (double)o[d], (double)o[3 + d] - b[3 + d]));
      }
      slack = (s == s) ? __double2float_ru(s) : INFINITY;
    }
    r.pad[side] = __float_as_int(slack);
  }
  r.child[0] = in[i].child[0];
  r.child[1] = in[i].child[1];
  out[i] = r;
}

__device__ __forceinline__ void tri_error_terms(const double* A, const double* B, const double* C, float& ec, float& lt)
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
  ec = __double2float_ru(256.0 * 0x1p-24 * kappa * 1.01);
  lt = __double2float_ru(L * 1.0001);
}

template <int NPC>
__global__ void k_leaves32(const LeafRec<NPC>* __restrict__ in, int n, LeafRec32<NPC>* __restrict__ out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k >= n) return;
  const double* v = in[k].v;
  LeafRec32<NPC> r;
  for(int j = 0; j < 3 * NPC; ++j) r.v[j] = (float)v[j];
  if constexpr(NPC == 3)
  {
    tri_error_terms(v, v + 3, v + 6, r.ec, r.lt);
    r.pad = 0.f;
  }
  else
  {
    tri_error_terms(v, v + 3, v + 6, r.ec[0], r.lt[0]);
    tri_error_terms(v, v + 6, v + 9, r.ec[1], r.lt[1]);
  }
  out[k] = r;
}

// Squared point-triangle distance in FP32 by Voronoi regions (Ericson,
// Real-Time Collision Detection 5.1.5), measured from P.
__device__ __forceinline__ float dist2_f32(const float* P, const float* A, const float* B, const float* C)
{
  const float ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const float ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const float ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const float d1 = ab0 * ap0 + ab1 * ap1 + ab2 * ap2;
  const float d2 = ac0 * ap0 + ac1 * ap1 + ac2 * ap2;
  if(d1 <= 0.f && d2 <= 0.f) return ap0 * ap0 + ap1 * ap1 + ap2 * ap2;
  const float bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const float d3 = ab0 * bp0 + ab1 * bp1 + ab2 * bp2;
  const float d4 = ac0 * bp0 + ac1 * bp1 + ac2 * bp2;
  if(d3 >= 0.f && d4 <= d3) return bp0 * bp0 + bp1 * bp1 + bp2 * bp2;
  const float vc = d1 * d4 - d3 * d2;
  if(vc <= 0.f && d1 >= 0.f && d3 <= 0.f)
  {
    const float v = d1 / (d1 - d3);
    const float x = ap0 - v * ab0, y = ap1 - v * ab1, z = ap2 - v * ab2;
    return x * x + y * y + z * z;
  }
  const float cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const float d5 = ab0 * cp0 + ab1 * cp1 + ab2 * cp2;
  const float d6 = ac0 * cp0 + ac1 * cp1 + ac2 * cp2;
  if(d6 >= 0.f && d5 <= d6) return cp0 * cp0 + cp1 * cp1 + cp2 * cp2;
  const float vb = d5 * d2 - d1 * d6;
  if(vb <= 0.f && d2 >= 0.f && d6 <= 0.f)
  {
    const float w = d2 / (d2 - d6);
    const float x = ap0 - w * ac0, y = ap1 - w * ac1, z = ap2 - w * ac2;
    return x * x + y * y + z * z;
  }
  const float va = d3 * d6 - d5 * d4;
  if(va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
  {
    const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    const float x = bp0 - w * (C[0] - B[0]), y = bp1 - w * (C[1] - B[1]), z = bp2 - w * (C[2] - B[2]);
    return x * x + y * y + z * z;
  }
  const float denom = 1.f / (va + vb + vc);
  const float v = vb * denom, w = vc * denom;
  const float x = ap0 - v * ab0 - w * ac0, y = ap1 - v * ab1 - w * ac1, z = ap2 - v * ab2 - w * ac2;
  return x * x + y * y + z * z;
}

// 0: certainly false, 1: certainly true, 2: undecided.
__device__ __forceinline__ int box_decide(const float* lo, const float* hi, float slack, const float* qlo,
                                          const float* qhi, float t_true, float t_false)
{
  float L = 0.f, H = 0.f;
#pragma unroll
  for(int d = 0; d < 3; ++d)
  {
    const float gl = fmaxf(fmaxf(__fsub_rd(lo[d], qhi[d]), __fsub_rd(qlo[d], hi[d])), 0.f);
    const float gh = fmaxf(fmaxf(__fadd_ru(__fsub_ru(lo[d], qlo[d]), slack), __fadd_ru(__fsub_ru(qhi[d], hi[d]), slack)),
                           0.f);
    L = __fadd_rd(L, __fmul_rd(gl, gl));
    H = __fadd_ru(H, __fmul_ru(gh, gh));
  }
  if(!(slack < INFINITY)) H = INFINITY;
  if(L > t_false) return 0;
  if(H <= t_true) return 1;
  return 2;
}

struct MixedStats
{
  unsigned long long* c;  // [0] audit violations [1] node FP64 fallbacks [2] leaf FP64 checks [3] leaf skips
};

template <int NPC, bool AUDIT>
__global__ void __launch_bounds__(128) k_sdf_mixed(const NodeRec64* __restrict__ nodes64,
                                                   const NodeRec32* __restrict__ nodes32,
                                                   const LeafRec<NPC>* __restrict__ leaves64,
                                                   const LeafRec32<NPC>* __restrict__ leaves32,
                                                   QueryPts qp,
                                                   int m,
                                                   const int* __restrict__ order,
                                                   SdfParams prm,
                                                   float mesh_max,
                                                   double* __restrict__ out,
                                                   double* __restrict__ out_cp,
                                                   double* __restrict__ out_n,
                                                   int* err,
                                                   MixedStats stats)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  const int idx = order ? __ldg(order + t) : t;
  const double q[3] = {qp.x[(size_t)idx * qp.stride], qp.y[(size_t)idx * qp.stride], qp.z[(size_t)idx * qp.stride]};
  const bool computeNormal = prm.sign != 0;
  float qf[3], qlo[3], qhi[3];
  float qabs = 0.f;
  for(int d = 0; d < 3; ++d)
  {
    qf[d] = __double2float_rn(q[d]);
    qlo[d] = __double2float_rd(q[d]);
    qhi[d] = __double2float_ru(q[d]);
    qabs = fmaxf(qabs, fmaxf(fabsf(qlo[d]), fabsf(qhi[d])));
  }
  const float Mq = fmaxf(qabs, mesh_max);
  // centroid-order error: e bounds |(c_f - q_f) - (c - q)| per axis
  const float e = __fmul_ru(0x1p-20f, Mq);
  const float e2 = __fmul_ru(3.5f, e);
  const float e3 = __fmul_ru(3.f * e, e);
  // coordinate-rounding part of the triangle distance error (1-Lipschitz)
  const float lip = __fmul_ru(0x1p-21f, __fadd_ru(qabs, mesh_max));

  MinCand mc;
  init_min(mc);
  float t_true, t_false, thr_leaf;
  auto update = [&]() {
    t_true = __double2float_rd(mc.minSq * (1.0 - 0x1p-40));
    t_false = __double2float_ru(mc.minSq * (1.0 + 0x1p-40));
    thr_leaf = __fadd_ru(__double2float_ru(sqrt(mc.minSq)), 1.0001e-6f);
  };
  update();
  unsigned long long n_node64 = 0, n_leaf64 = 0, n_skip = 0, n_bad = 0;

  auto visit = [&](int cur, bool& inL, bool& inR, bool& swap, int2& ch) {
    const float4* r = reinterpret_cast<const float4*>(nodes32 + cur);
    const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
    const int4 lk = __ldg(reinterpret_cast<const int4*>(r + 3));
    ch = make_int2(lk.x, lk.y);
    const float lo_l[3] = {a.x, a.y, a.z}, hi_l[3] = {a.w, b.x, b.y};
    const float lo_r[3] = {b.z, b.w, c.x}, hi_r[3] = {c.y, c.z, c.w};
    const bool vl = lo_l[0] <= hi_l[0] && lo_l[1] <= hi_l[1] && lo_l[2] <= hi_l[2];
    const bool vr = lo_r[0] <= hi_r[0] && lo_r[1] <= hi_r[1] && lo_r[2] <= hi_r[2];
    const int dl = vl ? box_decide(lo_l, hi_l, __int_as_float(lk.z), qlo, qhi, t_true, t_false) : 0;
    const int dr = vr ? box_decide(lo_r, hi_r, __int_as_float(lk.w), qlo, qhi, t_true, t_false) : 0;
    bool certain = (dl != 2 && dr != 2);
    swap = false;
    if(certain && dl == 1 && dr == 1)
    {
      float sl = 0.f, sr = 0.f;
#pragma unroll
      for(int d = 0; d < 3; ++d)
      {
        const float xl = 0.5f * (lo_l[d] + hi_l[d]) - qf[d];
        const float xr = 0.5f * (lo_r[d] + hi_r[d]) - qf[d];
        sl += xl * xl;
        sr += xr * xr;
      }
      const float bound = e2 * (sqrtf(sl) + sqrtf(sr)) + 2.f * e3 + 0x1p-20f * (sl + sr);
      if(sl - sr > bound)
        swap = true;
      else if(!(sr - sl > bound))
        certain = false;
    }
    if(certain)
    {
      inL = (dl == 1);
      inR = (dr == 1);
      return;
    }
    if(AUDIT) ++n_node64;
    visit_fp64(nodes64, cur, q, mc.minSq, inL, inR, swap);
  };

  auto leaf = [&](int leafpos) {
    const float4* r = reinterpret_cast<const float4*>(leaves32 + leafpos);
    float v[3 * NPC];
    float ec[2], lt[2];
    if constexpr(NPC == 3)
    {
      const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
      v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = c.x;
      ec[0] = c.y, lt[0] = c.z;
    }
    else
    {
      const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), d4 = __ldg(r + 3);
      v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = c.x;
      v[9] = c.y, v[10] = c.z, v[11] = c.w;
      ec[0] = d4.x, ec[1] = d4.y, lt[0] = d4.z, lt[1] = d4.w;
    }
    bool need[2] = {false, false};
#pragma unroll
    for(int s = 0; s < NPC - 2; ++s)
    {
      const float* A = v;
      const float* B = v + 3 * (s + 1);
      const float* C = v + 3 * (s + 2);
      const float d2 = dist2_f32(qf, A, B, C);
      const float ap = fmaxf(fabsf(qf[0] - A[0]), fmaxf(fabsf(qf[1] - A[1]), fabsf(qf[2] - A[2])));
      const float E = __fadd_ru(lip, __fmul_ru(ec[s], __fadd_ru(ap, lt[s])));
      const float lim = __fadd_ru(thr_leaf, E);
      need[s] = !(d2 > __fmul_ru(__fmul_ru(lim, lim), 1.0f + 0x1p-20f));
    }
    if(!need[0] && !need[1])
    {
      if(AUDIT)
      {
        // prove the skip: checkCandidate must be a no-op for every triangle
        ++n_skip;
        double w[3 * NPC];
        load_leaf<NPC>(leaves64, leafpos, w);
        for(int s = 0; s < NPC - 2; ++s)
        {
          double cp[3];
          closest_point(q, w, w + 3 * (s + 1), w + 3 * (s + 2), cp);
          const double lim64 = sqrt(mc.minSq) + 1e-6;
          if(sqdist_pp(q, cp) <= lim64 * lim64) ++n_bad;
        }
      }
      return;
    }
    if(AUDIT) ++n_leaf64;
    double w[3 * NPC];
    load_leaf<NPC>(leaves64, leafpos, w);
    const double before = mc.minSq;
#pragma unroll
    for(int s = 0; s < NPC - 2; ++s)
    {
      if(!need[s])
      {
        if(AUDIT)
        {
          double cp[3];
          closest_point(q, w, w + 3 * (s + 1), w + 3 * (s + 2), cp);
          const double lim64 = sqrt(mc.minSq) + 1e-6;
          if(sqdist_pp(q, cp) <= lim64 * lim64) ++n_bad;
        }
        continue;
      }
      const double* T[3] = {w, w + 3 * (s + 1), w + 3 * (s + 2)};
      check_triangle(q, mc, T, leafpos, s, computeNormal);
    }
    if(mc.minSq != before) update();
  };

  if(!traverse_point(visit, leaf)) atomicOr(err, DEVERR_STACK);
  finish_query<NPC>(q, mc, leaves64, prm, idx, out, out_cp, out_n);
  if(AUDIT)
  {
    atomicAdd(stats.c + 0, n_bad);
    atomicAdd(stats.c + 1, n_node64);
    atomicAdd(stats.c + 2, n_leaf64);
    atomicAdd(stats.c + 3, n_skip);
  }
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }
}  // namespace

size_t mixed_leaf_bytes(int npc) { return npc == 3 ? sizeof(LeafRec32<3>) : sizeof(LeafRec32<4>); }

// FP32 node and leaf records from the FP64 ones.
int mixed_prepare(const NodeRec64* nodes64, int n_inner, const void* leaves64, int nleaves, int npc, NodeRec32* nodes32,
                  void* leaves32, cudaStream_t s)
{
  k_nodes32<<<grid_for(n_inner, 256), 256, 0, s>>>(nodes64, n_inner, nodes32);
  if(npc == 3)
    k_leaves32<3><<<grid_for(nleaves, 256), 256, 0, s>>>(static_cast<const LeafRec<3>*>(leaves64), nleaves,
                                                         static_cast<LeafRec32<3>*>(leaves32));
  else
    k_leaves32<4><<<grid_for(nleaves, 256), 256, 0, s>>>(static_cast<const LeafRec<4>*>(leaves64), nleaves,
                                                         static_cast<LeafRec32<4>*>(leaves32));
  count_launch(2);
  GSQ_CUDA_TRY(cudaGetLastError());
  return GSQ_OK;
}

int mixed_launch(int npc, const NodeRec64* nodes64, const NodeRec32* nodes32, const void* leaves64,
                 const void* leaves32, const sdf::QueryPts& qp, int m, const int* order, const sdf::SdfParams& prm,
                 float mesh_max, double* out, double* out_cp, double* out_n, int* err, unsigned long long* audit,
                 cudaStream_t s)
{
  const int threads = 128;
  MixedStats st {audit};
  const int g = grid_for(m, threads);
#define GSQ_MIXED(NPC, AUD)                                                                                       \
  k_sdf_mixed<NPC, AUD><<<g, threads, 0, s>>>(nodes64, nodes32, static_cast<const LeafRec<NPC>*>(leaves64),      \
                                              static_cast<const LeafRec32<NPC>*>(leaves32), qp, m, order, prm,    \
                                              mesh_max, out, out_cp, out_n, err, st)
  if(npc == 3)
  {
    if(audit)
      GSQ_MIXED(3, true);
    else
      GSQ_MIXED(3, false);
  }
  else
  {
    if(audit)
      GSQ_MIXED(4, true);
    else
      GSQ_MIXED(4, false);
  }
#undef GSQ_MIXED
  count_launch();
  GSQ_CUDA_TRY(cudaGetLastError());
  return GSQ_OK;
}

}  // namespace gsq
