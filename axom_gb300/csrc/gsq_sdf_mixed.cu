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
#include "gsq_sdf_mixed.cuh"

#include <algorithm>

namespace gsq
{
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

struct MixedStats
{
  unsigned long long* c;  // [0] audit violations [1] node FP64 fallbacks [2] leaf FP64 checks [3] leaf skips
};

// Persistent warp loop over a work queue of Morton-ordered points.  Each lane
// runs one point's traversal as a resumable state machine, one FP32 step per
// iteration.  Leaves that the FP32 certificate cannot skip are queued (up to
// QCAP per lane) instead of being refined at once: until they are refined the
// exact running minimum is only known to lie in an interval (the resolved
// minimum and certified bounds of the queued candidates' FP64 distances), and
// every later decision is certified against the whole interval.  A lane parks
// when its queue is full, when a node decision is uncertain, or at its end;
// once every live lane of the warp is parked (or BATCH_MIN are) the warp
// replays the parked lanes' queues in order in FP64, converged.  The FP64 state
// therefore evolves through exactly the reference's checkCandidate calls on
// exactly the reference's candidates.  Finished lanes take the next point from
// the queue of Morton-ordered points with one warp-aggregated atomic.
constexpr int BATCH_MIN = 20;

template <int NPC, bool AUDIT, int QCAP>
__global__ void __launch_bounds__(128, 5) k_sdf_mixed(const NodeRec64* __restrict__ nodes64,
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
                                                   MixedStats stats,
                                                   int* __restrict__ work)
{
  constexpr unsigned FULL = 0xFFFFFFFFu;
  constexpr int M_DESCEND = 0, M_LEAF = 1, M_IDLE = 2;
  constexpr int P_NONE = 0, P_NODE = 1, P_FLUSH = 2, P_FINISH = 3;
  constexpr int ALL = (1 << (NPC - 2)) - 1;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const bool computeNormal = prm.sign != 0;

  int idx = 0;
  double q[3] = {0.0, 0.0, 0.0};
  QCtx c;
  MinCand mc;
  init_min(mc);
  int todo[STACK_SIZE];
  todo[0] = BARRIER;
  int pq[QCAP];  // queued leaves: leafpos * 4 + mask of triangles to refine
  float aq[AUDIT ? 2 * QCAP : 1];  // audit only: the bounds each queued entry was given
  int np = 0;
  float plo = INFINITY, phi = INFINITY;  // bounds on the queued candidates' best FP64 distance^2
  float mlo = INFINITY, mhi = INFINITY;  // the resolved minSq rounded down and up
  float qcp[3 * QCAP], qrad[QCAP];        // queued candidates' FP32 closest points and their error radii
  float mpf[3] = {0.f, 0.f, 0.f};         // the resolved closest point in FP32
  bool mvalid = false;                    // the resolved state holds a closest point
  bool reset = false;                     // a queued candidate superseded the resolved state
  int sp = 0, found = 0, cur = 0;
  int mode = M_IDLE, pend = P_NONE;
  int2 pch = make_int2(0, 0);
  bool open = true;
  unsigned long long st[4] = {0, 0, 0, 0};

  auto set_thresholds = [&]() {
    qctx_set32(c, fminf(reset ? INFINITY : mlo, plo), fminf(reset ? INFINITY : mhi, phi));
  };
  auto resolved = [&]() {
    qctx_update(c, mc.minSq);
    mlo = __double2float_rd(mc.minSq);
    mhi = __double2float_ru(mc.minSq);
    mvalid = mc.minSq < DBL_MAX;
    for(int d = 0; d < 3; ++d) mpf[d] = (float)mc.mp[d];
    reset = false;
  };
  // |a - b| > 1e-6 + r for certain: the candidate's point is farther than the
  // pseudo-normal window from b, so checkCandidate clears (SD:684-690)
  auto far = [&](const float* a, const float* b, float r) {
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    const float lim = __fadd_ru(1.0001e-6f, r);
    return __fmul_rd(0.999f, dx * dx + dy * dy + dz * dz) > __fmul_ru(lim, lim);
  };
  // transitions of the reference traversal (bvh_traverse.hpp:100-133, 140-151)
  auto pop = [&]() { return (sp >= 0) ? todo[sp--] : BARRIER; };
  auto apply_visit = [&](bool inL, bool inR, bool swap, int2 ch) {
    if(!inL && !inR)
      cur = pop();
    else
    {
      cur = inL ? ch.x : ch.y;
      int rc = ch.y;
      if(inL && inR)
      {
        if(swap)
        {
          const int tmp = cur;
          cur = rc;
          rc = tmp;
        }
        if(sp + 1 >= STACK_SIZE)
        {
          atomicOr(err, DEVERR_STACK);
          pend = P_FINISH;
          return;
        }
        todo[++sp] = rc;
      }
    }
    if(cur < 0 && !(found < 0))
    {
      found = cur;
      if(cur != BARRIER) cur = pop();
    }
  };
  auto after_leaf = [&]() {
    found = cur;
    if(cur < 0 && cur != BARRIER) cur = pop();
  };

  while(true)
  {
    const unsigned want = __ballot_sync(FULL, mode == M_IDLE && open);
    if(want)
    {
      const int leader = __ffs(want) - 1;
      int base = 0;
      if(lane == leader) base = atomicAdd(work, __popc(want));
      base = __shfl_sync(FULL, base, leader);
      if(mode == M_IDLE && open)
      {
        const int t = base + __popc(want & lt_mask);
        if(t < m)
        {
          idx = order ? __ldg(order + t) : t;
          q[0] = qp.x[(size_t)idx * qp.stride];
          q[1] = qp.y[(size_t)idx * qp.stride];
          q[2] = qp.z[(size_t)idx * qp.stride];
          qctx_init(c, q, mesh_max);
          init_min(mc);
          np = 0;
          plo = phi = INFINITY;
          resolved();
          sp = 0;
          todo[0] = BARRIER;
          found = 0;
          cur = 0;
          mode = M_DESCEND;
          pend = P_NONE;
        }
        else
          open = false;
      }
    }
    const unsigned live = __ballot_sync(FULL, mode != M_IDLE);
    if(live == 0) break;
    const unsigned parked = __ballot_sync(FULL, pend != P_NONE);
    if(parked && (parked == live || __popc(parked) >= BATCH_MIN))
    {
      // converged FP64 work of the parked lanes: replay the queue in order
      const int p = pend;
      pend = P_NONE;
      if(p != P_NONE)
      {
        if(reset) init_min(mc);
        if(AUDIT)
        {
          // every queued bound must hold for the FP64 distance it stood for
          for(int j = 0; j < np; ++j)
          {
            double w[3 * NPC];
            load_leaf<NPC>(leaves64, pq[j] >> 2, w);
            double best = DBL_MAX;
            for(int t2 = 0; t2 < NPC - 2; ++t2)
              if((pq[j] & 3) & (1 << t2))
              {
                double cp[3];
                closest_point(q, w, w + 3 * (t2 + 1), w + 3 * (t2 + 2), cp);
                best = fmin(best, sqdist_pp(q, cp));
              }
            if(!(best >= (double)aq[2 * j] && best <= (double)aq[2 * j + 1])) ++st[0];
          }
        }
        for(int j = 0; j < np; ++j)
          leaf_refine<NPC>(leaves64, pq[j] >> 2, pq[j] & 3, q, mc, computeNormal);
        if(AUDIT) st[2] += np;
        np = 0;
        plo = phi = INFINITY;
        resolved();
      }
      if(p == P_NODE)
      {
        bool inL, inR, swap;
        visit_fp64(nodes64, cur, q, mc.minSq, inL, inR, swap);
        if(AUDIT) ++st[1];
        apply_visit(inL, inR, swap, pch);
      }
      else if(p == P_FINISH)
      {
        finish_query<NPC>(q, mc, leaves64, prm, idx, out, out_cp, out_n);
        mode = M_IDLE;
      }
      continue;
    }
    if(mode == M_IDLE || pend != P_NONE) continue;
    // one FP32 step
    if(mode == M_DESCEND)
    {
      if(cur >= 0)
      {
        bool inL, inR, swap;
        int2 ch;
        if(visit32(nodes32, cur, c, inL, inR, swap, ch))
          apply_visit(inL, inR, swap, ch);
        else
        {
          pend = P_NODE;
          pch = ch;
        }
      }
      else
        mode = M_LEAF;
    }
    else
    {
      if(found < 0 && found != BARRIER)
      {
        const int lp = -found - 1;
        float lo2, hi2, cpf[3], rad;
        const int need = leaf_prefilter_bounds<NPC>(leaves32, lp, c, lo2, hi2, cpf, rad);
        if(AUDIT)
        {
          if(need == 0) ++st[3];
          st[0] += leaf_audit<NPC>(leaves64, lp, ALL & ~need, q, fmin(mc.minSq, (double)phi));
          if(np > 0 && !(mc.minSq >= (double)mlo && mc.minSq <= (double)mhi)) ++st[0];
        }
        if(need)
        {
          // A candidate that certainly lowers the minimum below everything
          // before it and certainly clears (its point is far from every earlier
          // closest point) leaves the state of checkCandidate independent of
          // all earlier candidates: they are dropped unevaluated.
          bool noop = false;
          if(need == 1 || need == 2)
          {
            // certainly no update (lo2 >= every possible minimum) and certainly
            // no pseudo-normal accumulation (far from every possible closest
            // point): checkCandidate would leave the state unchanged
            noop = lo2 >= fminf(reset ? INFINITY : mhi, phi) && (reset || np > 0 || mvalid);
            if(noop && !reset && mvalid) noop = far(cpf, mpf, __fadd_ru(rad, __fmul_ru(0x1p-22f, mesh_max)));
            for(int j = 0; noop && j < np; ++j) noop = far(cpf, qcp + 3 * j, __fadd_ru(rad, qrad[j]));
            if(AUDIT && noop)
            {
              MinCand s1 = mc;
              if(reset) init_min(s1);
              for(int j = 0; j < np; ++j) leaf_refine<NPC>(leaves64, pq[j] >> 2, pq[j] & 3, q, s1, computeNormal);
              MinCand s2 = s1;
              leaf_refine<NPC>(leaves64, lp, need, q, s2, computeNormal);
              const bool same = s1.minSq == s2.minSq && s1.type == s2.type && s1.leaf == s2.leaf &&
                                s1.sub == s2.sub && s1.mp[0] == s2.mp[0] && s1.mp[1] == s2.mp[1] &&
                                s1.mp[2] == s2.mp[2] && s1.sn[0] == s2.sn[0] && s1.sn[1] == s2.sn[1] &&
                                s1.sn[2] == s2.sn[2];
              if(!same) ++st[0];
            }
          }
          if(noop)
          {
            if(AUDIT) ++st[3];
          }
          else
          {
          if(need == 1 || need == 2)
          {
            bool sup = hi2 < fminf(reset ? INFINITY : mlo, plo);
            if(sup && !reset && mvalid) sup = far(cpf, mpf, __fadd_ru(rad, __fmul_ru(0x1p-22f, mesh_max)));
            for(int j = 0; sup && j < np; ++j) sup = far(cpf, qcp + 3 * j, __fadd_ru(rad, qrad[j]));
            if(sup)
            {
              if(AUDIT)
              {
                MinCand s1 = mc, s2;
                if(reset) init_min(s1);
                for(int j = 0; j < np; ++j) leaf_refine<NPC>(leaves64, pq[j] >> 2, pq[j] & 3, q, s1, computeNormal);
                leaf_refine<NPC>(leaves64, lp, need, q, s1, computeNormal);
                init_min(s2);
                leaf_refine<NPC>(leaves64, lp, need, q, s2, computeNormal);
                const bool same = s1.minSq == s2.minSq && s1.type == s2.type && s1.leaf == s2.leaf &&
                                  s1.sub == s2.sub && s1.mp[0] == s2.mp[0] && s1.mp[1] == s2.mp[1] &&
                                  s1.mp[2] == s2.mp[2] && s1.sn[0] == s2.sn[0] && s1.sn[1] == s2.sn[1] &&
                                  s1.sn[2] == s2.sn[2];
                if(!same) ++st[0];
              }
              np = 0;
              plo = phi = INFINITY;
              reset = true;
            }
          }
          if(AUDIT)
          {
            aq[2 * np] = lo2;
            aq[2 * np + 1] = hi2;
          }
          for(int d = 0; d < 3; ++d) qcp[3 * np + d] = cpf[d];
          qrad[np] = rad;
          pq[np++] = lp * 4 + need;
          if(np == QCAP)
            pend = P_FLUSH;
          else
          {
            plo = fminf(plo, lo2);
            phi = fminf(phi, hi2);
            set_thresholds();
          }
          }
        }
        after_leaf();
      }
      else
      {
        found = 0;
        if(cur == BARRIER)
          pend = P_FINISH;
        else
          mode = M_DESCEND;
      }
    }
  }
  if(AUDIT)
    for(int k = 0; k < 4; ++k)
      if(st[k]) atomicAdd(stats.c + k, st[k]);
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
                 int* work, int block, int depth, cudaStream_t s)
{
  if(depth != 1 && depth != 16) depth = 4;
  const int threads = (block >= 32 && block <= 128) ? (block / 32) * 32 : 128;
  MixedStats st {audit};
  int dev = 0, sms = 0;
  GSQ_CUDA_TRY(cudaGetDevice(&dev));
  GSQ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GSQ_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), s));
  int per_sm = 0;
#define GSQ_MIXED3(NPC, AUD, QC)                                                                                    \
  do                                                                                                                \
  {                                                                                                                 \
    GSQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sdf_mixed<NPC, AUD, QC>, threads, 0));   \
    const long long need = ((long long)m + threads - 1) / threads;                                                  \
    const int g = (int)std::max<long long>(1, std::min<long long>((long long)sms * std::max(per_sm, 1), need));     \
    k_sdf_mixed<NPC, AUD, QC><<<g, threads, 0, s>>>(nodes64, nodes32, static_cast<const LeafRec<NPC>*>(leaves64),   \
                                                    static_cast<const LeafRec32<NPC>*>(leaves32), qp, m, order,     \
                                                    prm, mesh_max, out, out_cp, out_n, err, st, work);              \
  } while(0)
#define GSQ_MIXED(NPC, AUD)        \
  do                               \
  {                                \
    if(depth == 16)                \
      GSQ_MIXED3(NPC, AUD, 16);    \
    else if(depth == 4)            \
      GSQ_MIXED3(NPC, AUD, 4);     \
    else                           \
      GSQ_MIXED3(NPC, AUD, 1);     \
  } while(0)
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
#undef GSQ_MIXED3
#undef GSQ_MIXED
  count_launch();
  GSQ_CUDA_TRY(cudaGetLastError());
  return GSQ_OK;
}

}  // namespace gsq
