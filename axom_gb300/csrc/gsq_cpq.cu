// Closest object point: the local query of quest::DistributedClosestPoint on
// the GPU.
//
// Reference: quest/detail/DistributedClosestPointImpl.hpp.  The object points
// become one degenerate box each in a spin::BVH with the default scale
// factor (generateBVHTreeImpl, 883-901); computeLocalClosestPoints (1002-1050)
// then runs, per query point, the point traverser (nearer centroid first,
// spin/policy/LinearBVH.hpp:72-85) with the predicate
//   squared_distance(p, box) <= best && squared_distance(p, box) <= threshold
// and the leaf action "replace the best if strictly closer" (the first point
// found wins ties).  Not found: index and domain -1, position and distance NaN.
//
// Two forms, equal bit for bit: FP64 (every decision in FP64, the reference's
// operation order), and mixed: a persistent warp loop (k_cpq_persist) whose
// node decisions are certified in FP32 on outward rounded boxes and whose
// leaf actions are certified on FP32 enclosures of the points' FP64 squared
// distances; what FP32 cannot decide runs in FP64, converged across the warp.
#include "gsq_sdf_handle.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

namespace gsq
{
gsq_bvh* bvh_new_internal(int device);
int bvh_build_internal(gsq_bvh* h, const double* d_boxes, int n, cudaStream_t s);

namespace
{
using namespace sdf;

// One sorted leaf: the object point, its index and its domain id.
struct __align__(16) PointRec
{
  double p[3];
  int id;
  int dom;
};
static_assert(sizeof(PointRec) == 32, "point record is 32 bytes");

// The same leaf for the FP32 certificate: the point rounded to nearest and
// its index (-1 for the padding leaf of a 0/1-point cloud).
struct __align__(16) PointRec32
{
  float p[3];
  int id;
};
static_assert(sizeof(PointRec32) == 16, "fp32 point record is 16 bytes");

__global__ void k_point_boxes(const double* __restrict__ pts, int n, double* __restrict__ boxes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  for(int d = 0; d < 3; ++d)
  {
    const double v = pts[3 * (size_t)i + d];
    boxes[6 * (size_t)i + d] = v;
    boxes[6 * (size_t)i + 3 + d] = v;
  }
}

__global__ void k_point_records(const int* __restrict__ perm, int nleaves, const double* __restrict__ pts,
                                const int* __restrict__ dom, int n, PointRec* __restrict__ recs)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k >= nleaves) return;
  const int c = perm[k];
  PointRec r;
  const bool ok = c < n;  // padding leaves of a 0/1-point cloud are never reached
  for(int d = 0; d < 3; ++d) r.p[d] = ok ? pts[3 * (size_t)c + d] : 0.0;
  r.id = ok ? c : -1;
  r.dom = (ok && dom) ? dom[c] : (ok ? 0 : -1);
  recs[k] = r;
}

__global__ void k_point_records32(const PointRec* __restrict__ recs, int nleaves, PointRec32* __restrict__ out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k >= nleaves) return;
  const PointRec r = recs[k];
  PointRec32 o;
  for(int d = 0; d < 3; ++d) o.p[d] = __double2float_rn(r.p[d]);
  o.id = r.id;
  out[k] = o;
}

__global__ void k_cpq_codes(const double* __restrict__ q, int m, const double* b, uint32_t* __restrict__ codes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  uint32_t u[3];
  for(int d = 0; d < 3; ++d)
  {
    // the object points' box grown by a quarter of its extent on every side,
    // so that queries just outside it keep distinct codes
    const double ext = b[3 + d] - b[d];
    const double sc = (ext > 0.0) ? 1.0 / (1.5 * ext) : 0.0;
    u[d] = (uint32_t)(int)fmin(fmax((q[3 * (size_t)i + d] - (b[d] - 0.25 * ext)) * sc * 1024.0, 0.0), 1023.0);
  }
  auto spread = [](uint32_t x) {
    x = (x | (x << 16)) & 0xFF0000FFu;
    x = (x | (x << 8)) & 0x0F00F00Fu;
    x = (x | (x << 4)) & 0xC30C30C3u;
    x = (x | (x << 2)) & 0x49249249u;
    return x;
  };
  codes[i] = spread(u[0]) | (spread(u[1]) << 1) | (spread(u[2]) << 2);
}

// The point traverser's FP64 node step with the closest-point predicate.
// KEYS: the comparisons on the integer pipe (OKey, the FP64 outcomes), for the
// one-thread-per-query FP64 kernel, which the FP64 pipe bounds; the persistent
// kernel runs this step only in converged batches and keeps FP64 comparisons,
// which need fewer registers.
template <bool KEYS>
__device__ __forceinline__ void cpq_visit_fp64(const NodeRec64* __restrict__ nodes, int cur, const double* q,
                                               double best, double thr, bool& inL, bool& inR, bool& swap)
{
  const double2* r = reinterpret_cast<const double2*>(nodes + cur);
  double b[12];
#pragma unroll
  for(int k = 0; k < 6; ++k)
  {
    const double2 t = __ldg(r + k);
    b[2 * k] = t.x;
    b[2 * k + 1] = t.y;
  }
  inL = false;
  inR = false;
  for(int side = 0; side < 2; ++side)
  {
    const double* lo = b + 6 * side;
    const double* hi = lo + 3;
    bool in = false;
    if constexpr(KEYS)
    {
      if(box_valid_i(lo, hi))
      {
        const OKey ks = okey(sqdist_pb(q, lo, hi));
        in = ok_le(ks, okey(best)) && ok_le(ks, okey(thr));
      }
    }
    else if(box_valid(lo, hi))
    {
      const double sq = sqdist_pb_d(q, lo, hi);
      in = sq <= best && sq <= thr;
    }
    (side ? inR : inL) = in;
  }
  swap = false;
  if(inL && inR)
  {
    const double cl[3] = {0.5 * (b[0] + b[3]), 0.5 * (b[1] + b[4]), 0.5 * (b[2] + b[5])};
    const double cr[3] = {0.5 * (b[6] + b[9]), 0.5 * (b[7] + b[10]), 0.5 * (b[8] + b[11])};
    if constexpr(KEYS)
      swap = ok_gt(okey(sqdist_pp(q, cl)), okey(sqdist_pp(q, cr)));
    else
      swap = sqdist_pp(q, cl) > sqdist_pp(q, cr);
  }
}

// The FP64 form: one thread per query, every decision in FP64.
__global__ void __launch_bounds__(128) k_cpq(const NodeRec64* __restrict__ nodes64,
                                             const PointRec* __restrict__ recs,
                                             const double* __restrict__ qs,
                                             int m,
                                             const int* __restrict__ order,
                                             double thr,
                                             int* __restrict__ out_idx,
                                             int* __restrict__ out_dom,
                                             double* __restrict__ out_pos,
                                             double* __restrict__ out_dist,
                                             int* err)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  const int i = order ? __ldg(order + t) : t;
  const double q[3] = {qs[3 * (size_t)i], qs[3 * (size_t)i + 1], qs[3 * (size_t)i + 2]};
  double best = DBL_MAX;
  int bleaf = -1;
  auto visit = [&](int cur, bool& inL, bool& inR, bool& swap, int2& ch) {
    ch = __ldg(reinterpret_cast<const int2*>(nodes64[cur].child));
    cpq_visit_fp64<true>(nodes64, cur, q, best, thr, inL, inR, swap);
  };
  auto leaf = [&](int leafpos) {
    const PointRec r = recs[leafpos];
    if(r.id < 0) return;
    const double sq = sqdist_pp(q, r.p);
    if(ok_lt(okey(sq), okey(best)))
    {
      best = sq;
      bleaf = leafpos;
    }
  };
  if(!traverse_point(visit, leaf)) atomicOr(err, DEVERR_STACK);
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  const PointRec* r = (bleaf >= 0) ? recs + bleaf : nullptr;
  out_idx[i] = r ? r->id : -1;
  out_dom[i] = r ? r->dom : -1;
  for(int d = 0; d < 3; ++d) out_pos[3 * (size_t)i + d] = r ? r->p[d] : nan;
  out_dist[i] = r ? sqrt(best) : nan;
}

// The mixed form as a persistent warp loop over Morton-ordered queries.  Each
// lane runs one query's traversal (the reference's point traverser, deferred
// leaves included) as a resumable state machine; an iteration takes the
// deferred leaf where the descent stopped, then one node visit, both decided
// in FP32 where FP32 can prove the FP64 outcome:
//  * node: visit32 against an FP32 interval holding min(best, threshold);
//  * leaf: the point's FP64 squared distance lies in [lo2, hi2]
//    (point_bounds32).  lo2 >= the interval's top: "sq < best" is certainly
//    false, nothing happens.  Otherwise the leaf is queued (up to QC per
//    lane) and the interval narrows to the minimum over the resolved best
//    and the queue; a leaf with hi2 below the interval's bottom is certainly
//    closer than everything before it and supersedes the queue and the
//    resolved best (replaying them would end in this leaf anyway).
// A lane parks when a node decision is uncertain, its queue is full, or its
// traversal ends; once enough lanes are parked (the batch size rule of the
// signed-distance kernel) the warp replays the parked lanes' queues in FP64
// in order ("replace the best if strictly closer"), runs their uncertain node
// visits in FP64 and writes finished queries, converged.
constexpr float CPQ_BATCH_K = 38.5f, CPQ_LAM0 = 0.1f;
constexpr int CPQ_BATCH_LO = 8, CPQ_BATCH_HI = 24;

template <int QC>
__global__ void __launch_bounds__(128) k_cpq_persist(const NodeRec64* __restrict__ nodes64,
                                                     const NodeRec32* __restrict__ nodes32,
                                                     const PointRec* __restrict__ recs,
                                                     const PointRec32* __restrict__ recs32,
                                                     const double* __restrict__ qs,
                                                     int m,
                                                     const int* __restrict__ order,
                                                     double thr,
                                                     float coord_max,
                                                     int* __restrict__ out_idx,
                                                     int* __restrict__ out_dom,
                                                     double* __restrict__ out_pos,
                                                     double* __restrict__ out_dist,
                                                     int* err,
                                                     int* __restrict__ work)
{
  constexpr unsigned FULL = 0xFFFFFFFFu;
  constexpr int M_DESCEND = 0, M_LEAF = 1, M_IDLE = 2;
  constexpr int P_NONE = 0, P_NODE = 1, P_FLUSH = 2, P_FINISH = 3;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float thr_lo = fp::f_rd(thr), thr_hi = fp::f_ru(thr);
  int idx = 0;
  double q[3] = {0.0, 0.0, 0.0};
  QCtx c;
  double best = DBL_MAX;  // the resolved state: best squared distance and its leaf
  int bleaf = -1;
  float blo = FLT_MAX, bhi = INFINITY;  // best rounded down and up
  int pq[QC];                           // queued leaves, in traversal order
  int np = 0;
  float plo = INFINITY, phi = INFINITY;  // bounds on the queued leaves' smallest squared distance
  bool reset = false;                    // a queued leaf superseded the resolved state
  int todo[STACK_SIZE];
  todo[0] = BARRIER;
  int sp = 0, found = 0, cur = 0;
  int mode = M_IDLE, pend = P_NONE;
  int2 pch = make_int2(0, 0);
  bool open = true;
  float lam = CPQ_LAM0;
  int bmin = 12, since = 0;

  auto set_thresholds = [&]() {
    const float lo = fminf(reset ? INFINITY : blo, plo), hi = fminf(reset ? INFINITY : bhi, phi);
    qctx_set32(c, fminf(lo, thr_lo), fminf(hi, thr_hi));
  };
  auto resolved = [&]() {
    blo = fp::f_rd(best);
    bhi = fp::f_ru(best);
    reset = false;
    np = 0;
    plo = phi = INFINITY;
    set_thresholds();
  };
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
          for(int d = 0; d < 3; ++d) q[d] = qs[3 * (size_t)idx + d];
          qctx_init(c, q, coord_max);
          best = DBL_MAX;
          bleaf = -1;
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
      bmin = (int)fminf(fmaxf(CPQ_BATCH_K * sqrtf(lam), (float)CPQ_BATCH_LO), (float)CPQ_BATCH_HI);
      since = 0;
      const int p = pend;
      pend = P_NONE;
      if(p != P_NONE)
      {
        // the queued leaf actions in FP64, in order (DistributedClosestPointImpl.hpp:1031-1040)
        if(reset)
        {
          best = DBL_MAX;
          bleaf = -1;
        }
        for(int j = 0; j < np; ++j)
        {
          const PointRec r = recs[pq[j]];
          if(r.id < 0) continue;
          const double sq = sqdist_pp(q, r.p);
          if(sq < best)
          {
            best = sq;
            bleaf = pq[j];
          }
        }
        resolved();
      }
      if(p == P_NODE)
      {
        bool inL, inR, swap;
        cpq_visit_fp64<false>(nodes64, cur, q, best, thr, inL, inR, swap);
        apply_visit(inL, inR, swap, pch);
      }
      else if(p == P_FINISH)
      {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        const PointRec* r = (bleaf >= 0) ? recs + bleaf : nullptr;
        out_idx[idx] = r ? r->id : -1;
        out_dom[idx] = r ? r->dom : -1;
        for(int d = 0; d < 3; ++d) out_pos[3 * (size_t)idx + d] = r ? r->p[d] : nan;
        out_dist[idx] = r ? sqrt(best) : nan;
        mode = M_IDLE;
      }
      continue;
    }
    if(mode == M_IDLE || pend != P_NONE) continue;
    if(mode == M_DESCEND && cur < 0) mode = M_LEAF;
    if(mode == M_LEAF)
    {
      if(found < 0 && found != BARRIER)
      {
        const int lp = -found - 1;
        const float4 rv = __ldg(reinterpret_cast<const float4*>(recs32 + lp));
        if(__float_as_int(rv.w) >= 0)
        {
          const float pf[3] = {rv.x, rv.y, rv.z};
          float lo2, hi2;
          point_bounds32(c, pf, lo2, hi2);
          const float cur_lo = fminf(reset ? INFINITY : blo, plo), cur_hi = fminf(reset ? INFINITY : bhi, phi);
          if(!(lo2 >= cur_hi))
          {
            if(hi2 < cur_lo)
            {
              np = 0;
              plo = phi = INFINITY;
              reset = true;
            }
            pq[np++] = lp;
            if(np == QC)
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
        apply_visit(inL, inR, swap, ch);
      else
      {
        pend = P_NODE;
        pch = ch;
      }
    }
  }
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

// Grid of the persistent kernel: as many blocks as fit on the device, at most
// one per `threads` queries.
template <class K>
cudaError_t persist_grid(K kernel, int threads, long long m, int* grid)
{
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if(e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if(e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  *grid = (int)std::max<long long>(1, std::min<long long>((long long)sms * std::max(per_sm, 1), (m + threads - 1) / threads));
  return e;
}
}  // namespace
}  // namespace gsq

using namespace gsq;

struct gsq_cpq
{
  int device = 0;
  int n = 0;
  gsq_bvh* bvh = nullptr;
  PointRec* recs = nullptr;
  PointRec32* recs32 = nullptr;
  NodeRec32* nodes32 = nullptr;
  int* d_work = nullptr;  // work-queue counter of the persistent query kernel
  double* d_bounds = nullptr;
  float coord_max = 0.f;
  int* d_err = nullptr;
  float eval_ms = 0.f;
};

namespace
{
void cpq_release(gsq_cpq* h)
{
  if(h->recs) cudaFree(h->recs);
  if(h->recs32) cudaFree(h->recs32);
  if(h->d_work) cudaFree(h->d_work);
  if(h->nodes32) cudaFree(h->nodes32);
  if(h->d_bounds) cudaFree(h->d_bounds);
  if(h->d_err) cudaFree(h->d_err);
  if(h->bvh) gsq_bvh_destroy(h->bvh);
  delete h;
}
}  // namespace

extern "C" {

int gsq_cpq_create(gsq_cpq** out, const double* points, int32_t n, const int32_t* domain_ids, void* stream)
{
  if(!out) return fail(GSQ_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if(n < 0 || n >= (1 << 30)) return fail(GSQ_ERR_INVALID, "number of points must be 0..2^30-1");
  if(n > 0 && !points) return fail(GSQ_ERR_INVALID, "null point array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* h = new(std::nothrow) gsq_cpq();
  if(!h) return fail(GSQ_ERR_NOMEM, "handle allocation failed");
  auto bail = [&](int rc) {
    cpq_release(h);
    return rc;
  };
  h->n = n;
  cudaError_t e = cudaGetDevice(&h->device);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_err, sizeof(int));
  if(e == cudaSuccess) e = cudaMemsetAsync(h->d_err, 0, sizeof(int), s);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_bounds, 6 * sizeof(double));
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_cpq_create"));
  InBuf pb, db;
  e = pb.stage(points, sizeof(double) * 3 * (size_t)n, s);
  if(e == cudaSuccess) e = db.stage(domain_ids, domain_ids ? sizeof(int) * (size_t)n : 0, s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_cpq_create: points"));
  Scratch boxes;
  e = boxes.alloc(sizeof(double) * 6 * (size_t)std::max(n, 1), s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_cpq_create: boxes"));
  if(n > 0)
  {
    k_point_boxes<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const double*>(pb.dev), n, boxes.as<double>());
    count_launch();
  }
  h->bvh = bvh_new_internal(h->device);
  if(!h->bvh) return bail(GSQ_ERR_NOMEM);
  int rc = bvh_build_internal(h->bvh, boxes.as<double>(), n, s);
  if(rc) return bail(rc);
  const BvhDev* B = bvh_dev(h->bvh);
  e = cudaMalloc(&h->recs, sizeof(PointRec) * B->n);
  if(e == cudaSuccess) e = cudaMalloc(&h->recs32, sizeof(PointRec32) * B->n);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_work, sizeof(int));
  if(e == cudaSuccess) e = cudaMalloc(&h->nodes32, sizeof(NodeRec32) * std::max(B->n - 1, 1));
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_cpq_create: records"));
  k_point_records<<<grid_for(B->n, 256), 256, 0, s>>>(B->perm, B->n, static_cast<const double*>(pb.dev),
                                                      static_cast<const int*>(db.dev), n, h->recs);
  k_point_records32<<<grid_for(B->n, 256), 256, 0, s>>>(h->recs, B->n, h->recs32);
  count_launch(2);
  rc = mixed_prepare(B->nodes, B->n - 1, nullptr, 0, 3, h->nodes32, nullptr, s);
  if(rc) return bail(rc);
  double mm = 0.0;
  for(int d = 0; d < 6; ++d)
    if(std::fabs(B->bounds[d]) < DBL_MAX) mm = std::max(mm, std::fabs(B->bounds[d]));
  h->coord_max = (float)(mm * (1.0 + 1e-6));
  e = cudaMemcpyAsync(h->d_bounds, B->bounds, 6 * sizeof(double), cudaMemcpyHostToDevice, s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_cpq_create"));
  rc = check_device_error(h->d_err, s, "gsq_cpq_create");
  if(rc) return bail(rc);
  *out = h;
  return GSQ_OK;
}

int gsq_cpq_destroy(gsq_cpq* h)
{
  if(h) cpq_release(h);
  return GSQ_OK;
}

int gsq_cpq_query(const gsq_cpq* hc, const double* points, int32_t m, double sq_threshold, int32_t precision,
                  int32_t* idx, int32_t* dom, double* pos, double* dist, void* stream)
{
  gsq_cpq* h = const_cast<gsq_cpq*>(hc);
  if(!h) return fail(GSQ_ERR_INVALID, "null closest-point handle");
  if(m < 0) return fail(GSQ_ERR_INVALID, "negative point count");
  if(m == 0) return GSQ_OK;
  if(!points || !idx || !dom || !pos || !dist) return fail(GSQ_ERR_INVALID, "null point or output array");
  if(precision != GSQ_PRECISION_FP64 && precision != GSQ_PRECISION_MIXED)
    return fail(GSQ_ERR_INVALID, "unknown precision");
  if(!(sq_threshold >= 0.0)) return fail(GSQ_ERR_INVALID, "the squared threshold must be >= 0");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  InBuf qb;
  GSQ_CUDA_TRY(qb.stage(points, sizeof(double) * 3 * (size_t)m, s));
  OutBuf ib, dmb, pb, sb;
  GSQ_CUDA_TRY(ib.prepare(idx, sizeof(int) * (size_t)m, s));
  GSQ_CUDA_TRY(dmb.prepare(dom, sizeof(int) * (size_t)m, s));
  GSQ_CUDA_TRY(pb.prepare(pos, sizeof(double) * 3 * (size_t)m, s));
  GSQ_CUDA_TRY(sb.prepare(dist, sizeof(double) * (size_t)m, s));
  const double* q = static_cast<const double*>(qb.dev);

  // Morton order of the query points (processing order only)
  Scratch ob;
  const int* order = nullptr;
  if(m > 1)
  {
    GSQ_CUDA_TRY(ob.alloc(4 * sizeof(uint32_t) * (size_t)m, s));
    uint32_t* keys[2] = {ob.as<uint32_t>(), ob.as<uint32_t>() + m};
    int* vals[2] = {reinterpret_cast<int*>(ob.as<uint32_t>() + 2 * (size_t)m),
                    reinterpret_cast<int*>(ob.as<uint32_t>() + 3 * (size_t)m)};
    k_cpq_codes<<<grid_for(m, 256), 256, 0, s>>>(q, m, h->d_bounds, keys[0]);
    count_launch();
    const int which = radix_sort_pairs(keys, vals, m, 30, true, s, h->d_err);
    if(which < 0) return which;
    order = vals[which];
  }
  const BvhDev* B = bvh_dev(h->bvh);
  cudaEvent_t e0, e1;
  GSQ_CUDA_TRY(cudaEventCreate(&e0));
  GSQ_CUDA_TRY(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  if(precision == GSQ_PRECISION_MIXED)
  {
    auto kernel = k_cpq_persist<2>;
    int g = 1;
    GSQ_CUDA_TRY(persist_grid(kernel, 128, m, &g));
    GSQ_CUDA_TRY(cudaMemsetAsync(h->d_work, 0, sizeof(int), s));
    kernel<<<g, 128, 0, s>>>(B->nodes, h->nodes32, h->recs, h->recs32, q, m, order, sq_threshold, h->coord_max,
                             static_cast<int*>(ib.dev), static_cast<int*>(dmb.dev), static_cast<double*>(pb.dev),
                             static_cast<double*>(sb.dev), h->d_err, h->d_work);
  }
  else
    k_cpq<<<grid_for(m, 128), 128, 0, s>>>(B->nodes, h->recs, q, m, order, sq_threshold, static_cast<int*>(ib.dev),
                                           static_cast<int*>(dmb.dev), static_cast<double*>(pb.dev),
                                           static_cast<double*>(sb.dev), h->d_err);
  count_launch();
  cudaEventRecord(e1, s);
  cudaError_t e = cudaGetLastError();
  if(e == cudaSuccess) e = ib.flush(s);
  if(e == cudaSuccess) e = dmb.flush(s);
  if(e == cudaSuccess) e = pb.flush(s);
  if(e == cudaSuccess) e = sb.flush(s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e == cudaSuccess) e = cudaEventElapsedTime(&h->eval_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(e != cudaSuccess) return cuda_fail(e, "gsq_cpq_query");
  return check_device_error(h->d_err, s, "gsq_cpq_query");
}

int gsq_cpq_last_ms(const gsq_cpq* h, float* ms)
{
  if(!h || !ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->eval_ms;
  return GSQ_OK;
}

}  // extern "C"
