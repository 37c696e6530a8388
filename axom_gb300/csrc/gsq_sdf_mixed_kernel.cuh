// The persistent mixed-precision query kernel, shared by the single-mesh
// query (gsq_sdf_mixed.cu) and the batched form (gsq_batch.cu).  Each
// translation unit instantiates the variants it launches.
#pragma once

#include "gsq_sdf_mixed.cuh"

#include <algorithm>

namespace gsq
{
namespace
{
using namespace sdf;

struct MixedStats
{
  unsigned long long* c;  // [0] audit violations [1] node FP64 fallbacks [2] leaf FP64 checks [3] leaf skips
};

// Persistent warp loop over a work queue of Morton-ordered points.  Each lane
// runs one point's traversal as a resumable state machine; an iteration takes
// the deferred leaf where the descent stopped (if any), then one node visit,
// both decided in FP32.  Leaves that the FP32 certificate cannot skip are queued (up to
// QCAP per lane) instead of being refined at once: until they are refined the
// exact running minimum is only known to lie in an interval (the resolved
// minimum and certified bounds of the queued candidates' FP64 distances), and
// every later decision is certified against the whole interval.  A lane parks
// when its queue is full, when a node decision is uncertain, or at its end;
// once every live lane of the warp is parked (or enough are, see below) the
// warp replays the parked lanes' queues in order in FP64, converged.  The FP64 state
// therefore evolves through exactly the reference's checkCandidate calls on
// exactly the reference's candidates.  Finished lanes take the next point from
// the queue of Morton-ordered points, which a warp takes 32 at a time.
//
// STK is the traversal stack depth (the reference's 64, or 32 where every
// tree is shallow enough).  MULTI: the points belong to several meshes (point
// ranges qoff[k].. of mesh k, whose records start at meshes[k]'s offsets);
// otherwise to the one mesh meshes[0] with its node box in prm_all.
//
// Batch size: a batch costs about the same whatever its lanes, and a parked
// lane idles until the batch, so with parks arriving at rate lam per iteration
// the cost per park C / N + N / (2 lam) is least at N ~ sqrt(2 C lam).  Each
// warp tracks lam (a moving average of parked lanes per iteration between
// batches) and fires at N = 38.5 sqrt(lam) parked lanes, clamped to 8..24 (the
// constant measured: about 12 for uniform points, 24 near the surface).
constexpr float BATCH_K = 38.5f, BATCH_LAM0 = 0.1f;
constexpr int BATCH_LO = 8, BATCH_HI = 24;
//
// LEAF: also write each point's closest triangle to out_leaf: c for triangle
// cell c, 2c or 2c + 1 for the first or second triangle of quad cell c, -1
// when there is none (for the adjoint).

template <int NPC, bool AUDIT, int QCAP, int STK, bool MULTI, bool LEAF = false>
__global__ void __launch_bounds__(128, 5) k_sdf_mixed(const NodeRec64* __restrict__ nodes64_all,
                                                   const NodeRec32* __restrict__ nodes32_all,
                                                   const LeafRec<NPC>* __restrict__ leaves64_all,
                                                   const LeafRec32<NPC>* __restrict__ leaves32_all,
                                                   const MeshInfo* __restrict__ meshes,
                                                   int nmeshes,
                                                   const long long* __restrict__ qoff,
                                                   QueryPts qp,
                                                   int m,
                                                   const int* __restrict__ order,
                                                   SdfParams prm_all,
                                                   double* __restrict__ out,
                                                   double* __restrict__ out_cp,
                                                   double* __restrict__ out_n,
                                                   int* err,
                                                   MixedStats stats,
                                                   int* __restrict__ work,
                                                   int* __restrict__ out_leaf)
{
  constexpr unsigned FULL = 0xFFFFFFFFu;
  constexpr int M_DESCEND = 0, M_LEAF = 1, M_IDLE = 2;
  constexpr int P_NONE = 0, P_NODE = 1, P_FLUSH = 2, P_FINISH = 3;
  constexpr int ALL = (1 << (NPC - 2)) - 1;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const bool computeNormal = prm_all.sign != 0;

  // the current point's mesh (several meshes share one launch in the batched form)
  int noff = 0, loff = 0;  // the point's mesh: its first node and leaf record
  auto mesh_of = [&](int i) {
    int lo = 0, hi = nmeshes;  // last mesh whose first point is <= i
    while(hi - lo > 1)
    {
      const int mid = (lo + hi) >> 1;
      if(__ldg(qoff + mid) <= i)
        lo = mid;
      else
        hi = mid;
    }
    return lo;
  };
  float mesh_max = 0.f;
#define nodes64 (nodes64_all + noff)
#define nodes32 (nodes32_all + noff)
#define leaves64 (leaves64_all + loff)
#define leaves32 (leaves32_all + loff)
  int idx = 0;
  double q[3] = {0.0, 0.0, 0.0};
  QCtx c;
  MinCand mc;
  init_min(mc);
  int todo[STK];
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
  float lam = BATCH_LAM0;  // parks per iteration (warp-uniform moving average)
  int bmin = 12, since = 0;
  unsigned long long st[4] = {0, 0, 0, 0};

  auto set_thresholds = [&]() {
    qctx_set32(c, fminf(reset ? INFINITY : mlo, plo), fminf(reset ? INFINITY : mhi, phi));
  };
  auto resolved = [&]() {
    // thresholds from the FP32 enclosure of the exact minimum (no FP64 math:
    // FP64 instructions are the scarcest resource of this GPU)
    mlo = __double2float_rd(mc.minSq);
    mhi = __double2float_ru(mc.minSq);
    qctx_set32(c, mlo, mhi);
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
        if(sp + 1 >= STK)
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

  // Work comes in runs of 32 consecutive (Morton-ordered) points per warp,
  // [cb, ce): the lanes of a warp work on neighbouring points, which share
  // most of their node and leaf records (16M uniform points: 468 instead of
  // 482 ms; runs of 64 lost more near the surface than they gained).
  int cb = 0, ce = 0;
  while(true)
  {
    const unsigned want = __ballot_sync(FULL, mode == M_IDLE && open);
    if(want)
    {
      const int leader = __ffs(want) - 1;
      const int nw = __popc(want), avail = ce - cb;
      int nb = 0;
      if(avail < nw)  // the run's rest, then a new run of 32 (nw - avail <= 32)
      {
        if(lane == leader) nb = atomicAdd(work, 32);
        nb = __shfl_sync(FULL, nb, leader);
      }
      const int rk = __popc(want & lt_mask);
      const int tk = (rk < avail) ? cb + rk : nb + (rk - avail);
      if(avail < nw)
      {
        cb = nb + (nw - avail);
        ce = nb + 32;
      }
      else
        cb += nw;
      if(mode == M_IDLE && open)
      {
        const int t = tk;
        if(t < m)
        {
          idx = order ? __ldg(order + t) : t;
          if constexpr(MULTI)
          {
            const MeshInfo& mi = meshes[mesh_of(idx)];
            noff = (int)mi.node_off;
            loff = (int)mi.leaf_off;
            mesh_max = mi.mesh_max;
          }
          else
            mesh_max = meshes[0].mesh_max;
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
    ++since;
    if(parked && (parked == live || __popc(parked) >= bmin))
    {
      lam = 0.875f * lam + 0.125f * (float)__popc(parked) / (float)since;
      bmin = (int)fminf(fmaxf(BATCH_K * sqrtf(lam), (float)BATCH_LO), (float)BATCH_HI);
      since = 0;
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
        visit_fp64<false>(nodes64, cur, q, mc.minSq, inL, inR, swap);
        if(AUDIT) ++st[1];
        apply_visit(inL, inR, swap, pch);
      }
      else if(p == P_FINISH)
      {
        // the sign certified in FP32 where possible (the FP64 pseudo-normal
        // is then not formed); the audit checks it against FP64
        auto hint = [&] {
          const double h = sign32<NPC>(q, mc, leaves32, mesh_max);
          if(AUDIT && h != 0.0 && h != sign64<NPC>(q, mc, leaves64)) ++st[0];
          return h;
        };
        if constexpr(MULTI)
        {
          SdfParams prm = prm_all;
          const MeshInfo& mi = meshes[mesh_of(idx)];
          for(int d = 0; d < 6; ++d) prm.domain[d] = mi.domain[d];
          finish_query<NPC>(q, mc, leaves64, prm, idx, out, out_cp, out_n, hint);
        }
        else
          finish_query<NPC>(q, mc, leaves64, prm_all, idx, out, out_cp, out_n, hint);
        if constexpr(LEAF)
        {
          const int cell = (mc.leaf < 0) ? -1 : __ldg(&leaves64[mc.leaf].cell);
          out_leaf[idx] = (cell < 0) ? -1 : (NPC == 3 ? cell : 2 * cell + mc.sub);
        }
        mode = M_IDLE;
      }
      continue;
    }
    if(mode == M_IDLE || pend != P_NONE) continue;
    // One FP32 step: the deferred leaf where the descent has stopped at one,
    // then one node visit, in the reference's order (bvh_traverse.hpp:100-151).
    if(mode == M_DESCEND && cur < 0) mode = M_LEAF;
    if(mode == M_LEAF)
    {
      if(found < 0 && found != BARRIER)
      {
        const int lp = -found - 1;
        float lo2, hi2, cpf[3], rad;
        const int need = leaf_prefilter_bounds<NPC>(leaves32, lp, c, mesh_max, lo2, hi2, cpf, rad);
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
              if(!same_state<NPC>(s1, s2, leaves64)) ++st[0];
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
                if(!same_state<NPC>(s1, s2, leaves64)) ++st[0];
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
      if(pend == P_NONE && !(found < 0 && found != BARRIER))
      {
        // the run of deferred leaves is over
        found = 0;
        if(cur == BARRIER)
          pend = P_FINISH;
        else
          mode = M_DESCEND;
      }
    }
    if(mode == M_DESCEND && pend == P_NONE && cur >= 0)
    {
      bool inL, inR, swap;
      int2 ch;
      if(visit32(nodes32, cur, c, inL, inR, swap, ch))
      {
        if(AUDIT)
        {
          // the FP64 visit at the exact minimum (the queue refined on a copy)
          // must take the same decisions
          MinCand s1 = mc;
          if(reset) init_min(s1);
          for(int j = 0; j < np; ++j) leaf_refine<NPC>(leaves64, pq[j] >> 2, pq[j] & 3, q, s1, computeNormal);
          bool a2, b2, w2;
          visit_fp64<false>(nodes64, cur, q, s1.minSq, a2, b2, w2);
          if(a2 != inL || b2 != inR || (inL && inR && w2 != swap)) ++st[0];
        }
        apply_visit(inL, inR, swap, ch);
      }
      else
      {
        pend = P_NODE;
        pch = ch;
      }
    }
  }
  if(AUDIT)
    for(int k = 0; k < 4; ++k)
      if(st[k]) atomicAdd(stats.c + k, st[k]);
#undef nodes64
#undef nodes32
#undef leaves64
#undef leaves32
}


// Grid of the persistent kernel: as many blocks as fit on the device, at most
// one per `threads` points.
template <class K>
cudaError_t mixed_grid(K kernel, int threads, long long m, int* grid)
{
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if(e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if(e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  const long long need = (m + threads - 1) / threads;
  *grid = (int)std::max<long long>(1, std::min<long long>((long long)sms * std::max(per_sm, 1), need));
  return e;
}

template <int NPC, bool AUDIT, int QCAP, int STK, bool MULTI, bool LEAF = false>
cudaError_t launch_mixed(int threads, cudaStream_t s, const NodeRec64* nodes64, const NodeRec32* nodes32,
                         const void* leaves64, const void* leaves32, const MeshInfo* meshes, int nmeshes,
                         const long long* qoff, const QueryPts& qp, int m, const int* order, const SdfParams& prm,
                         double* out, double* out_cp, double* out_n, int* err, MixedStats st, int* work,
                         int* out_leaf = nullptr)
{
  auto kernel = k_sdf_mixed<NPC, AUDIT, QCAP, STK, MULTI, LEAF>;
  int g = 1;
  cudaError_t e = mixed_grid(kernel, threads, m, &g);
  if(e != cudaSuccess) return e;
  kernel<<<g, threads, 0, s>>>(nodes64, nodes32, static_cast<const LeafRec<NPC>*>(leaves64),
                               static_cast<const LeafRec32<NPC>*>(leaves32), meshes, nmeshes, qoff, qp, m, order, prm,
                               out, out_cp, out_n, err, st, work, out_leaf);
  return cudaGetLastError();
}
}  // namespace
}  // namespace gsq
