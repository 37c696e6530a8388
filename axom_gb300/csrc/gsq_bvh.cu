// Linear BVH build and candidate queries on the GPU (spin::BVH replacement).
//
// Build pipeline (replaces build_radix_tree + emit_bvh_parents,
// spin/internal/linear_bvh/build_radix_tree.hpp:579-611 and
// spin/policy/LinearBVH.hpp:191-269):
//   k_leaf_bounds   scale each box about its midpoint (transform_boxes,
//                   BR:85-99) and fold the global bounds (reduce, BR:102-143);
//                   the last block to finish merges the blocks' folds
//   k_morton        30-bit Morton code of each scaled box centroid (get_mcodes,
//                   BR:146-176), written into the tree's code array
//   radix sort      stable (key, index) sort (sort_mcodes, BR:225-260) in
//                   place: four passes end in the tree's code and permutation
//                   arrays
//   k_karras        Karras 2012 hierarchy, identical tie-breaking (build_tree,
//                   BR:265-384); also zeroes the refit's counters
//   k_refit_persist bottom-up boxes with one atomic per node; the second
//                   arrival continues (propagate_aabbs, BR:505-576), writing each
//                   box straight into its parent's 128-byte node record (the
//                   emit step fused in); persistent lanes take the next leaf
//                   when their chain ends.  No thread ever waits on another.
// Queries (replace findCandidatesImpl, LinearBVH.hpp:271-402): one thread per
// query runs the reference traversal state machine (bvh_traverse.hpp:66-154);
// pass 1 keeps up to CAP candidates per query in scratch and counts all of
// them, a scan gives the CSR offsets, and pass 2 copies, re-traversing only
// the queries with more than CAP candidates.
#include "gsq_build.cuh"

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

using namespace gsq;

namespace gsq
{
namespace
{
constexpr int BUILD_THREADS = 256;

using lbvh::ArgV;
using lbvh::Fold;
using lbvh::fold_block;
using lbvh::fold_init;
using lbvh::fold_merge;
using lbvh::take_max;
using lbvh::take_min;

// Scaled leaf boxes and the bounds (transform_boxes, BR:85-99, and reduce,
// BR:102-143): each block folds its boxes and publishes the fold; the last
// block to finish (one counter, which it resets) merges every block's fold
// and writes params: bounds lo[3] hi[3], then Morton min[3], inv_extent[3].
// The merge is commutative (it keeps the leftmost extreme), so the order in
// which blocks finish does not matter.
__device__ __forceinline__ Fold load_fold_cg(const Fold* p)
{
  Fold f;
  for(int d = 0; d < 3; ++d)
  {
    f.lo[d] = ArgV {__ldcg(&p->lo[d].v), __ldcg(&p->lo[d].i)};
    f.hi[d] = ArgV {__ldcg(&p->hi[d].v), __ldcg(&p->hi[d].i)};
  }
  f.first_valid = __ldcg(&p->first_valid);
  return f;
}

__global__ void __launch_bounds__(BUILD_THREADS) k_leaf_bounds(const double* __restrict__ in,
                                                                 int n,
                                                                 double scale,
                                                                 double* __restrict__ leaf,
                                                                 Fold* __restrict__ partials,
                                                                 int* __restrict__ done,
                                                                 double* __restrict__ params)
{
  Fold f;
  fold_init(f);
  const double half = scale * 0.5;
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    double lo[3], hi[3];
    for(int d = 0; d < 3; ++d)
    {
      lo[d] = in[6 * (size_t)i + d];
      hi[d] = in[6 * (size_t)i + 3 + d];
    }
    if(lbvh::scale_box(lo, hi, half)) lbvh::fold_add_box(f, lo, hi, i);
    for(int d = 0; d < 3; ++d)
    {
      leaf[6 * (size_t)i + d] = lo[d];
      leaf[6 * (size_t)i + 3 + d] = hi[d];
    }
  }
  const Fold a = fold_block(f);
  __shared__ bool s_last;
  if(threadIdx.x == 0)
  {
    partials[blockIdx.x] = a;
    __threadfence();
    s_last = (atomicAdd(done, 1) == (int)gridDim.x - 1);
  }
  __syncthreads();
  if(!s_last) return;
  __threadfence();
  Fold g;
  fold_init(g);
  for(int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) fold_merge(g, load_fold_cg(partials + b));
  const Fold t = fold_block(g);
  if(threadIdx.x == 0)
  {
    lbvh::bounds_params(t, leaf, n - 1, params);
    *done = 0;
  }
}

__global__ void __launch_bounds__(BUILD_THREADS) k_morton(const double* __restrict__ leaf,
                                                            int n,
                                                            const double* __restrict__ params,
                                                            uint32_t* __restrict__ codes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n) return;
  codes[i] = lbvh::box_morton(leaf + 6 * (size_t)i, params);
}

__global__ void __launch_bounds__(BUILD_THREADS) k_karras(const uint32_t* __restrict__ codes,
                                                            int n,
                                                            int* __restrict__ lchild,
                                                            int* __restrict__ rchild,
                                                            int* __restrict__ parent,
                                                            NodeRec64* __restrict__ nodes,
                                                            int* __restrict__ counters)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= n - 1) return;
  // the refit's node counters and (counters[n - 1]) its work counter
  counters[i] = 0;
  if(i == 0) counters[n - 1] = 0;
  lbvh::karras_node(i, codes, n, lchild, rchild, parent, nodes);
}

// The refit as a persistent loop: every lane takes the next sorted leaf from
// a work counter (one warp-aggregated atomic) when its previous chain has
// ended, then climbs one level per iteration (lbvh::refit_step).  One thread
// per leaf leaves warps on a few lanes after the first levels (half the
// threads stop at each level); here the lanes stay busy.  Nothing waits: a
// lane's chain ends at its first first-arrival or at the root.
__global__ void __launch_bounds__(BUILD_THREADS) k_refit_persist(const double* __restrict__ leaf,
                                                                   const int* __restrict__ perm,
                                                                   int n,
                                                                   const int* __restrict__ parent,
                                                                   int* __restrict__ counters,
                                                                   NodeRec64* nodes,
                                                                   double* __restrict__ root_box,
                                                                   int* __restrict__ work)
{
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int inner = n - 1;
  bool active = false, open = true;
  int pcode = 0;
  double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {0.0, 0.0, 0.0};
  while(true)
  {
    const unsigned want = __ballot_sync(FULL, !active && open);
    if(want)
    {
      const int leader = __ffs(want) - 1;
      int base = 0;
      if(lane == leader) base = atomicAdd(work, __popc(want));
      base = __shfl_sync(FULL, base, leader);
      if(!active && open)
      {
        const int k = base + __popc(want & lt_mask);
        if(k < n)
        {
          const int id = perm[k];
          for(int d = 0; d < 3; ++d)
          {
            lo[d] = leaf[6 * (size_t)id + d];
            hi[d] = leaf[6 * (size_t)id + 3 + d];
          }
          pcode = parent[inner + k];
          active = true;
        }
        else
          open = false;
      }
    }
    if(__ballot_sync(FULL, active || open) == 0) break;
    if(active) active = lbvh::refit_step(pcode, lo, hi, parent, counters, nodes, root_box);
  }
}

// ---- traversal --------------------------------------------------------------
// bvh_traverse (bvh_traverse.hpp:66-154) with the generic traverser's
// no-preference order (LB:92-103).  pred(b, k) tests one child box given as
// its six doubles (lo, hi) and their comparison keys; leaf receives the sorted
// leaf position.  Returns false on stack overflow.  Every comparison of the
// visit runs on the integer pipe (OKey), with the FP64 results.
template <class Pred, class Leaf>
__device__ __forceinline__ bool traverse_nopref(const NodeRec64* __restrict__ nodes, Pred& pred, Leaf& leaf)
{
  int todo[STACK_SIZE];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0, cur = 0;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      const double2* r = reinterpret_cast<const double2*>(nodes + cur);
      double b[12];
      OKey k[12];
#pragma unroll
      for(int j = 0; j < 6; ++j)
      {
        const double2 v = __ldg(r + j);
        b[2 * j] = v.x;
        b[2 * j + 1] = v.y;
        k[2 * j] = okey(v.x);
        k[2 * j + 1] = okey(v.y);
      }
      const int2 ch = __ldg(reinterpret_cast<const int2*>(nodes[cur].child));
      const bool inL = box_valid_k(k, k + 3) ? pred(b, k) : false;
      const bool inR = box_valid_k(k + 6, k + 9) ? pred(b + 6, k + 6) : false;
      if(!inL && !inR)
        cur = (sp >= 0) ? todo[sp--] : BARRIER;
      else
      {
        cur = inL ? ch.x : ch.y;
        if(inL && inR)
        {
          if(sp + 1 >= STACK_SIZE) return false;
          todo[++sp] = ch.y;
        }
      }
      if(cur < 0 && !(found < 0))
      {
        found = cur;
        if(cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
      }
    }
    while(found < 0 && found != BARRIER)
    {
      leaf(-found - 1);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
    }
    found = 0;
  }
  return true;
}

// Comparison keys of a node record's two child boxes (the OKey words of its
// twelve coordinates, FP64 order as 32-bit integer order), for the box and
// point finds, whose predicates only compare.  A box is valid when lo <= hi
// on every axis, so a valid box has no NaN coordinate and its keys need no
// NaN flag; an invalid box is never entered.  128 bytes per inner node, made
// from the node records on the first such find after a build: each visit then
// loads its keys instead of forming them from the doubles.
struct __align__(16) NodeKeyRec
{
  int hi[12];
  unsigned lo[12];
  int child[2];
  int valid;  // bit 0: left box valid, bit 1: right box valid
  int pad[5];
};
static_assert(sizeof(NodeKeyRec) == 128, "key record must be one 128-byte line");

__global__ void __launch_bounds__(BUILD_THREADS) k_node_keys(const NodeRec64* __restrict__ nodes, int inner,
                                                              NodeKeyRec* __restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= inner) return;
  const double2* r = reinterpret_cast<const double2*>(nodes + i);
  OKey k[12];
#pragma unroll
  for(int j = 0; j < 6; ++j)
  {
    const double2 v = __ldg(r + j);
    k[2 * j] = okey(v.x);
    k[2 * j + 1] = okey(v.y);
  }
  NodeKeyRec o;
#pragma unroll
  for(int j = 0; j < 12; ++j)
  {
    o.hi[j] = k[j].hi;
    o.lo[j] = k[j].lo;
  }
  const int2 ch = __ldg(reinterpret_cast<const int2*>(nodes[i].child));
  o.child[0] = ch.x;
  o.child[1] = ch.y;
  o.valid = (box_valid_k(k, k + 3) ? 1 : 0) | (box_valid_k(k + 6, k + 9) ? 2 : 0);
  for(int j = 0; j < 5; ++j) o.pad[j] = 0;
  int4* dst = reinterpret_cast<int4*>(out + i);
  const int4* src = reinterpret_cast<const int4*>(&o);
#pragma unroll
  for(int j = 0; j < 8; ++j) dst[j] = src[j];
}

// traverse_nopref over the key records: the same visits, leaves and order.
template <class Pred, class Leaf>
__device__ __forceinline__ bool traverse_keys(const NodeKeyRec* __restrict__ nk, Pred& pred, Leaf& leaf)
{
  int todo[STACK_SIZE];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0, cur = 0;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      const int4* r = reinterpret_cast<const int4*>(nk + cur);
      int w[28];
#pragma unroll
      for(int j = 0; j < 7; ++j)
      {
        const int4 v = __ldg(r + j);
        w[4 * j] = v.x;
        w[4 * j + 1] = v.y;
        w[4 * j + 2] = v.z;
        w[4 * j + 3] = v.w;
      }
      OKey k[12];
#pragma unroll
      for(int j = 0; j < 12; ++j)
      {
        k[j].hi = w[j];
        k[j].lo = (unsigned)w[12 + j];
        k[j].nan = false;
      }
      const int2 ch = make_int2(w[24], w[25]);
      const int valid = w[26];
      const bool inL = (valid & 1) ? pred(nullptr, k) : false;
      const bool inR = (valid & 2) ? pred(nullptr, k + 6) : false;
      if(!inL && !inR)
        cur = (sp >= 0) ? todo[sp--] : BARRIER;
      else
      {
        cur = inL ? ch.x : ch.y;
        if(inL && inR)
        {
          if(sp + 1 >= STACK_SIZE) return false;
          todo[++sp] = ch.y;
        }
      }
      if(cur < 0 && !(found < 0))
      {
        found = cur;
        if(cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
      }
    }
    while(found < 0 && found != BARRIER)
    {
      leaf(-found - 1);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
    }
    found = 0;
  }
  return true;
}

// Query primitives.  Boxes: BoundingBox::intersectsWith with
// intersect_bbox_bbox (BoundingBox.hpp:432-447, intersect_bounding_box_impl.hpp:35-41).
struct BoxQuery
{
  OKey lo[3], hi[3];
  __device__ bool operator()(const double*, const OKey* k) const
  {
    for(int d = 0; d < 3; ++d)
      if(!(ok_ge(hi[d], k[d]) && ok_le(lo[d], k[3 + d]))) return false;
    return true;
  }
};
// Points: BoundingBox::contains(Point) (BoundingBox.hpp:388-401).
struct PointQuery
{
  OKey p[3];
  __device__ bool operator()(const double*, const OKey* k) const
  {
    for(int d = 0; d < 3; ++d)
      if(ok_lt(p[d], k[d]) || ok_gt(p[d], k[3 + d])) return false;
    return true;
  }
};
// Rays: intersect_ray(Ray, BoundingBox, Point&, EPS) and
// intersect_ray_bbox_test (intersect_ray_impl.hpp:151-186, 321-351).  The
// per-axis reciprocal 1 / n_d and the near-zero test |n_d - 0| <= EPS depend
// on the ray only, so they are evaluated once per ray (the same values the
// per-box evaluation gives).
struct RayQuery
{
  double o[3], inv[3];
  OKey ko[3];
  bool flat[3];
  __device__ bool operator()(const double* b, const OKey* k) const
  {
    double tmin = DBL_MIN, tmax = DBL_MAX;
    for(int d = 0; d < 3; ++d)
    {
      bool ok;
      if(flat[d])
        ok = !(ok_lt(ko[d], k[d]) || ok_gt(ko[d], k[3 + d]));
      else
      {
        double t1 = (b[d] - o[d]) * inv[d];
        double t2 = (b[3 + d] - o[d]) * inv[d];
        OKey k1 = okey(t1), k2 = okey(t2);
        if(ok_gt(k1, k2))
        {
          const double t = t1;
          t1 = t2;
          t2 = t;
          const OKey kt = k1;
          k1 = k2;
          k2 = kt;
        }
        tmin = ok_lt(k1, okey(tmin)) ? tmin : t1;
        tmax = ok_lt(k2, okey(tmax)) ? t2 : tmax;
        ok = !ok_gt(okey(tmin), okey(tmax));
      }
      if(!ok) return false;
    }
    return true;
  }
};

enum QueryKind
{
  Q_BOXES = 0,
  Q_POINTS = 1,
  Q_RAYS = 2
};

struct QueryArgs
{
  const double* a;  // boxes (m x 6), points (m x 3) or ray origins (m x 3)
  const double* b;  // ray directions (m x 3)
  double eps;
};

template <int KIND>
__device__ __forceinline__ auto make_query(const QueryArgs& q, int i)
{
  if constexpr(KIND == Q_BOXES)
  {
    BoxQuery bq;
    for(int d = 0; d < 3; ++d)
    {
      bq.lo[d] = okey(q.a[6 * (size_t)i + d]);
      bq.hi[d] = okey(q.a[6 * (size_t)i + 3 + d]);
    }
    return bq;
  }
  else if constexpr(KIND == Q_POINTS)
  {
    PointQuery pq;
    for(int d = 0; d < 3; ++d) pq.p[d] = okey(q.a[3 * (size_t)i + d]);
    return pq;
  }
  else
  {
    RayQuery rq;
    for(int d = 0; d < 3; ++d)
    {
      rq.o[d] = q.a[3 * (size_t)i + d];
      rq.ko[d] = okey(rq.o[d]);
      const double n = q.b[3 * (size_t)i + d];
      rq.flat[d] = fabs(n - 0.0) <= q.eps;
      rq.inv[d] = rq.flat[d] ? 0.0 : 1.0 / n;
    }
    return rq;
  }
}

constexpr int FIND_THREADS = 128;
constexpr int FIND_CAP = 8;  // candidates kept per query by pass 1

// Boxes and points traverse the key records, rays the node records (their
// slab test needs the coordinates).
template <int KIND, class Pred, class Leaf>
__device__ __forceinline__ bool find_traverse(const NodeRec64* __restrict__ nodes, const NodeKeyRec* __restrict__ nk,
                                              Pred& pred, Leaf& leaf)
{
  if constexpr(KIND == Q_RAYS)
    return traverse_nopref(nodes, pred, leaf);
  else
    return traverse_keys(nk, pred, leaf);
}

template <int KIND>
__global__ void __launch_bounds__(FIND_THREADS) k_find_pass1(const NodeRec64* __restrict__ nodes,
                                                               const NodeKeyRec* __restrict__ nk,
                                                               const int* __restrict__ perm,
                                                               QueryArgs qa,
                                                               int m,
                                                               int* __restrict__ counts,
                                                               int* __restrict__ keep,
                                                               int* err)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  auto pred = make_query<KIND>(qa, i);
  int c = 0;
  int* mine = keep + (size_t)i * FIND_CAP;
  auto leaf = [&](int leafpos) {
    if(c < FIND_CAP) mine[c] = __ldg(perm + leafpos);
    ++c;
  };
  if(!find_traverse<KIND>(nodes, nk, pred, leaf)) atomicOr(err, DEVERR_STACK);
  counts[i] = c;
}

template <int KIND>
__global__ void __launch_bounds__(FIND_THREADS) k_find_pass2(const NodeRec64* __restrict__ nodes,
                                                               const NodeKeyRec* __restrict__ nk,
                                                               const int* __restrict__ perm,
                                                               QueryArgs qa,
                                                               int m,
                                                               const int* __restrict__ counts,
                                                               const int* __restrict__ offsets,
                                                               const int* __restrict__ keep,
                                                               int* __restrict__ cand)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  const int c = counts[i];
  int* out = cand + offsets[i];
  if(c <= FIND_CAP)
  {
    for(int k = 0; k < c; ++k) out[k] = keep[(size_t)i * FIND_CAP + k];
    return;
  }
  auto pred = make_query<KIND>(qa, i);
  int w = 0;
  auto leaf = [&](int leafpos) {
    if(w < c) out[w] = __ldg(perm + leafpos);
    ++w;
  };
  find_traverse<KIND>(nodes, nk, pred, leaf);
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

// Mesh box: BoundingBox::addPoint over the nodes in order from an invalid box
// (quest/SignedDistance.hpp:483-486) = per axis leftmost min and leftmost max.
__global__ void __launch_bounds__(BUILD_THREADS) k_node_fold(const double* __restrict__ x,
                                                               const double* __restrict__ y,
                                                               const double* __restrict__ z,
                                                               int nv,
                                                               Fold* __restrict__ partials)
{
  Fold f;
  fold_init(f);
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
  {
    const double p[3] = {x[i], y[i], z[i]};
    for(int d = 0; d < 3; ++d)
    {
      if(okey(p[d]).nan) continue;  // addPoint's comparisons are false for a NaN
      take_min(f.lo[d], ArgV {p[d], i});
      take_max(f.hi[d], ArgV {p[d], i});
    }
  }
  const Fold a = fold_block(f);
  if(threadIdx.x == 0) partials[blockIdx.x] = a;
}

__global__ void __launch_bounds__(BUILD_THREADS) k_node_final(const Fold* __restrict__ partials, int nb,
                                                                double* __restrict__ out)
{
  Fold f;
  fold_init(f);
  for(int b = threadIdx.x; b < nb; b += blockDim.x) fold_merge(f, partials[b]);
  const Fold a = fold_block(f);
  if(threadIdx.x != 0) return;
  for(int d = 0; d < 3; ++d)
  {
    out[d] = (a.lo[d].i == INT_MAX) ? DBL_MAX : a.lo[d].v;
    out[3 + d] = (a.hi[d].i == INT_MAX) ? -DBL_MAX : a.hi[d].v;
  }
}

}  // namespace

int node_bounds(const double* x, const double* y, const double* z, int nv, double* out6, cudaStream_t s)
{
  const int nb = std::min(grid_for(std::max(nv, 1), BUILD_THREADS), 4 * 152);
  Scratch work;
  GSQ_CUDA_TRY(work.alloc(sizeof(Fold) * nb + 256, s));
  Fold* folds = work.as<Fold>();
  double* d_out = reinterpret_cast<double*>(reinterpret_cast<char*>(folds) + ((sizeof(Fold) * nb + 15) & ~size_t(15)));
  k_node_fold<<<nb, BUILD_THREADS, 0, s>>>(x, y, z, nv, folds);
  k_node_final<<<1, BUILD_THREADS, 0, s>>>(folds, nb, d_out);
  count_launch(2);
  GSQ_CUDA_TRY(cudaGetLastError());
  GSQ_CUDA_TRY(cudaMemcpyAsync(out6, d_out, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  return GSQ_OK;
}

void BvhDev::drop_graph()
{
  if(exec) cudaGraphExecDestroy(exec);
  exec = nullptr;
  graph_kernels = 0;
  key_n = -1;
}

void BvhDev::release()
{
  drop_graph();
  if(block) cudaFree(block);
  if(work) cudaFree(work);
  if(stage) cudaFree(stage);
  if(pad) cudaFree(pad);
  if(cs) cudaStreamDestroy(cs);
  block = work = stage = nullptr;
  pad = nullptr;
  cs = nullptr;
  block_bytes = work_bytes = stage_bytes = 0;
  nodes = nullptr;
  perm = nullptr;
  codes = nullptr;
  lchild = rchild = nullptr;
  n = 0;
}

namespace
{

// Scratch of one build over n boxes.
constexpr size_t BUILD_FIXED_BYTES = 256;

struct BuildScratch
{
  int* fold_done;
  double* leaf;
  double* params;
  uint32_t* keys[2];
  int* vals[2];
  int* parent;
  int* counters;
  Fold* folds;
  void* sort_work;
  size_t sort_bytes;
  int fold_blocks;
};

size_t build_scratch_layout(int n, char* base, BuildScratch* out)
{
  const int inner = n - 1;
  const int fold_blocks = std::min(grid_for(n, BUILD_THREADS), 4 * 152);
  const size_t sz_leaf = align256(sizeof(double) * 6 * (size_t)n);
  const size_t sz_params = align256(sizeof(double) * 18);
  const size_t sz_u32 = align256(sizeof(uint32_t) * n);
  const size_t sz_par = align256(sizeof(int) * (2 * (size_t)n - 1));
  const size_t sz_cnt = align256(sizeof(int) * (inner + 1));  // node counters, then the refit's work counter
  const size_t sz_fold = align256(sizeof(Fold) * fold_blocks);
  const size_t sz_sort = align256(radix_sort_work_bytes(n));
  // the first 256 bytes hold words whose place does not depend on n: the
  // bounds fold's block counter (zeroed once when the scratch is allocated;
  // the last block of every build resets it)
  const size_t total = BUILD_FIXED_BYTES + sz_leaf + sz_params + 4 * sz_u32 + sz_par + sz_cnt + sz_fold + sz_sort;
  if(out)
  {
    out->fold_done = reinterpret_cast<int*>(base);
    char* w = base + BUILD_FIXED_BYTES;
    out->leaf = reinterpret_cast<double*>(w);
    w += sz_leaf;
    out->params = reinterpret_cast<double*>(w);
    w += sz_params;
    out->keys[0] = reinterpret_cast<uint32_t*>(w);
    out->keys[1] = reinterpret_cast<uint32_t*>(w + sz_u32);
    w += 2 * sz_u32;
    out->vals[0] = reinterpret_cast<int*>(w);
    out->vals[1] = reinterpret_cast<int*>(w + sz_u32);
    w += 2 * sz_u32;
    out->parent = reinterpret_cast<int*>(w);
    w += sz_par;
    out->counters = reinterpret_cast<int*>(w);
    w += sz_cnt;
    out->folds = reinterpret_cast<Fold*>(w);
    w += sz_fold;
    out->sort_work = w;
    out->sort_bytes = sz_sort;
    out->fold_blocks = fold_blocks;
  }
  return total;
}

// The build's device work, with no allocation and no host synchronisation (so
// that it can be captured): transform_boxes + reduce, Morton codes, the
// stable sort, Karras hierarchy and refit.
int enqueue_build(BvhDev& B, const BuildScratch& w, const double* d_boxes, int n, double scale, cudaStream_t s,
                  int* d_err)
{
  const int inner = n - 1;
  k_leaf_bounds<<<w.fold_blocks, BUILD_THREADS, 0, s>>>(d_boxes, n, scale, w.leaf, w.folds, w.fold_done, w.params);
  // the codes and the permutation are sorted in place into the tree's arrays
  // (four passes end in the first buffer)
  k_morton<<<grid_for(n, BUILD_THREADS), BUILD_THREADS, 0, s>>>(w.leaf, n, w.params, B.codes);
  count_launch(2);
  uint32_t* keys[2] = {B.codes, w.keys[1]};
  int* vals[2] = {B.perm, w.vals[1]};
  const int which = radix_sort_pairs_prealloc(keys, vals, n, 30, true, w.sort_work, w.sort_bytes, s, d_err);
  if(which < 0) return which;
  if(which != 0)
  {
    GSQ_CUDA_TRY(cudaMemcpyAsync(B.codes, keys[which], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    GSQ_CUDA_TRY(cudaMemcpyAsync(B.perm, vals[which], sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  }
  k_karras<<<grid_for(inner, BUILD_THREADS), BUILD_THREADS, 0, s>>>(B.codes, n, B.lchild, B.rchild, w.parent, B.nodes,
                                                                   w.counters);
  int dev = 0, sms = 0, per_sm = 0;
  GSQ_CUDA_TRY(cudaGetDevice(&dev));
  GSQ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GSQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_refit_persist, BUILD_THREADS, 0));
  const int rgrid = std::max(1, std::min(sms * std::max(per_sm, 1), grid_for(n, BUILD_THREADS)));
  k_refit_persist<<<rgrid, BUILD_THREADS, 0, s>>>(w.leaf, B.perm, n, w.parent, w.counters, B.nodes, w.params + 12,
                                                  w.counters + inner);
  count_launch(2);
  GSQ_CUDA_TRY(cudaGetLastError());
  return GSQ_OK;
}
}  // namespace

int bvh_build(BvhDev& B, const double* d_boxes, int n, double scale, cudaStream_t s, int* d_err, cudaEvent_t done)
{
  if(n < 0) return fail(GSQ_ERR_INVALID, "number of boxes must be >= 0");
  // BVH::initialize (spin/BVH.hpp:436-463): 0 or 1 boxes -> 2, second invalid.
  if(n <= 1)
  {
    double h[12];
    for(int d = 0; d < 3; ++d)
    {
      h[d] = h[6 + d] = DBL_MAX;
      h[3 + d] = h[9 + d] = -DBL_MAX;
    }
    if(!B.pad) GSQ_CUDA_TRY(cudaMalloc(&B.pad, sizeof(h)));
    GSQ_CUDA_TRY(cudaMemcpyAsync(B.pad, h, sizeof(h), cudaMemcpyHostToDevice, s));
    if(n == 1) GSQ_CUDA_TRY(cudaMemcpyAsync(B.pad, d_boxes, 6 * sizeof(double), cudaMemcpyDeviceToDevice, s));
    d_boxes = B.pad;
    n = 2;
  }
  const int inner = n - 1;

  // Persistent arrays in one allocation, and the scratch (both grow-only; a
  // new allocation invalidates the captured build).
  const size_t sz_nodes = align256(sizeof(NodeRec64) * inner);
  const size_t sz_perm = align256(sizeof(int) * n);
  const size_t sz_codes = align256(sizeof(uint32_t) * n);
  const size_t sz_child = align256(sizeof(int) * inner);
  const size_t total = sz_nodes + sz_perm + sz_codes + 2 * sz_child;
  if(total > B.block_bytes)
  {
    B.drop_graph();
    if(B.block) cudaFree(B.block);
    B.block = nullptr;
    B.block_bytes = 0;
    GSQ_CUDA_TRY(cudaMalloc(&B.block, total));
    B.block_bytes = total;
  }
  const size_t wbytes = build_scratch_layout(n, nullptr, nullptr);
  if(wbytes > B.work_bytes)
  {
    B.drop_graph();
    if(B.work) cudaFree(B.work);
    B.work = nullptr;
    B.work_bytes = 0;
    GSQ_CUDA_TRY(cudaMalloc(&B.work, wbytes));
    B.work_bytes = wbytes;
    GSQ_CUDA_TRY(cudaMemsetAsync(B.work, 0, BUILD_FIXED_BYTES, s));
  }
  char* base = static_cast<char*>(B.block);
  B.n = n;
  B.nodes = reinterpret_cast<NodeRec64*>(base);
  B.perm = reinterpret_cast<int*>(base + sz_nodes);
  B.codes = reinterpret_cast<uint32_t*>(base + sz_nodes + sz_perm);
  B.lchild = reinterpret_cast<int*>(base + sz_nodes + sz_perm + sz_codes);
  B.rchild = reinterpret_cast<int*>(base + sz_nodes + sz_perm + sz_codes + sz_child);
  BuildScratch w;
  build_scratch_layout(n, static_cast<char*>(B.work), &w);

  const bool repeat = (n == B.key_n && scale == B.key_scale && d_boxes == B.key_in && d_err == B.key_err);
  if(!repeat)
  {
    // a first build with these inputs runs directly; a repeat is captured
    B.drop_graph();
    B.key_n = n;
    B.key_scale = scale;
    B.key_in = d_boxes;
    B.key_err = d_err;
    const int rc = enqueue_build(B, w, d_boxes, n, scale, s, d_err);
    if(rc) return rc;
  }
  else
  {
    if(!B.exec)
    {
      if(!B.cs) GSQ_CUDA_TRY(cudaStreamCreateWithFlags(&B.cs, cudaStreamNonBlocking));
      const int64_t before = gsq_kernel_launches();
      GSQ_CUDA_TRY(cudaStreamBeginCapture(B.cs, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_build(B, w, d_boxes, n, scale, B.cs, d_err);
      cudaGraph_t g = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(B.cs, &g);
      const int kernels = (int)(gsq_kernel_launches() - before);
      count_launch(-kernels);  // counted when the graph runs
      if(rc || ec != cudaSuccess)
      {
        if(g) cudaGraphDestroy(g);
        B.key_n = -1;
        return rc ? rc : cuda_fail(ec, "bvh build: graph capture");
      }
      const cudaError_t ei = cudaGraphInstantiate(&B.exec, g, 0);
      cudaGraphDestroy(g);
      if(ei != cudaSuccess)
      {
        B.exec = nullptr;
        B.key_n = -1;
        return cuda_fail(ei, "bvh build: graph instantiation");
      }
      B.graph_kernels = kernels;
    }
    GSQ_CUDA_TRY(cudaGraphLaunch(B.exec, s));
    count_launch(B.graph_kernels);
  }
  if(done) GSQ_CUDA_TRY(cudaEventRecord(done, s));
  GSQ_CUDA_TRY(cudaMemcpyAsync(B.bounds, w.params, sizeof(double) * 6, cudaMemcpyDeviceToHost, s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  return check_device_error(d_err, s, "bvh build");
}

}  // namespace gsq

// =============================================================================
// C ABI: spin::BVH
// =============================================================================
// What a find needs besides its inputs and outputs, kept with the handle so
// that a find allocates only its candidate array: the pass-1 candidate
// scratch, the scan's tile sums and the device total (grow-only), the timing
// events, and a pinned host word pair into which the total and the device
// error word are read back together.  The reference's find* are const and
// may run concurrently; a find that finds the cache in use by another thread
// allocates its own scratch for the call instead.
struct FindCache
{
  std::mutex busy;
  void* work = nullptr;
  size_t work_bytes = 0;
  void* cand = nullptr;  // the candidates of a find with host outputs, on the device
  size_t cand_bytes = 0;
  long long* host = nullptr;  // pinned: [0] total, [1] error word
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  void release()
  {
    if(work) cudaFree(work);
    if(cand) cudaFree(cand);
    cand = nullptr;
    cand_bytes = 0;
    if(host) cudaFreeHost(host);
    for(auto& e : ev)
      if(e) cudaEventDestroy(e);
    work = nullptr;
    host = nullptr;
    work_bytes = 0;
    for(auto& e : ev) e = nullptr;
  }
};

struct gsq_bvh
{
  int device = 0;
  double scale = gsq::DEFAULT_SCALE;
  double tol = DBL_EPSILON;
  gsq::BvhDev dev;
  bool built = false;
  float build_ms = 0.f;
  mutable float find_ms = 0.f;  // device time of the last find's two passes and scan
  mutable FindCache fc;
  int* d_err = nullptr;
  // the key records of the box and point finds: made by the first such find
  // after a build (under nk_mu; nk_ev orders later finds on other streams)
  mutable gsq::NodeKeyRec* nkeys = nullptr;
  mutable size_t nkeys_cap = 0;
  mutable bool nkeys_ok = false;
  mutable std::mutex nk_mu;
  mutable cudaEvent_t nk_ev = nullptr;
};

namespace
{
int check_bvh(const gsq_bvh* h)
{
  if(!h) return fail(GSQ_ERR_INVALID, "null bvh handle");
  if(!h->built) return fail(GSQ_ERR_STATE, "bvh has not been built");
  return GSQ_OK;
}

// The key records of the current tree, made on stream s if the tree has none.
int node_keys(const gsq_bvh* h, cudaStream_t s, const NodeKeyRec** out)
{
  std::lock_guard<std::mutex> g(h->nk_mu);
  const int inner = h->dev.n - 1;
  if(!h->nkeys_ok)
  {
    if((size_t)inner > h->nkeys_cap)
    {
      if(h->nkeys) cudaFree(h->nkeys);
      h->nkeys = nullptr;
      h->nkeys_cap = 0;
      GSQ_CUDA_TRY(cudaMalloc(&h->nkeys, sizeof(NodeKeyRec) * (size_t)inner));
      h->nkeys_cap = (size_t)inner;
    }
    if(!h->nk_ev) GSQ_CUDA_TRY(cudaEventCreateWithFlags(&h->nk_ev, cudaEventDisableTiming));
    count_launch();
    k_node_keys<<<grid_for(inner, BUILD_THREADS), BUILD_THREADS, 0, s>>>(h->dev.nodes, inner, h->nkeys);
    GSQ_CUDA_TRY(cudaGetLastError());
    GSQ_CUDA_TRY(cudaEventRecord(h->nk_ev, s));
    h->nkeys_ok = true;
  }
  else
    GSQ_CUDA_TRY(cudaStreamWaitEvent(s, h->nk_ev, 0));
  *out = h->nkeys;
  return GSQ_OK;
}

template <int KIND>
int find_impl(const gsq_bvh* h, const double* a, const double* b, int32_t m, int32_t* offsets, int32_t* counts,
              int32_t** candidates, int64_t* total_out, void* stream)
{
  int rc = check_bvh(h);
  if(rc) return rc;
  if(m < 0 || !candidates || (m > 0 && (!a || !offsets || !counts || (KIND == Q_RAYS && !b))))
    return fail(GSQ_ERR_INVALID, "invalid find arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool dev_out = offsets ? is_device_ptr(offsets) : false;
  *candidates = nullptr;
  const int width = (KIND == Q_BOXES) ? 6 : 3;
  InBuf qa_buf, qb_buf;
  GSQ_CUDA_TRY(qa_buf.stage(a, sizeof(double) * width * (size_t)m, s));
  if(KIND == Q_RAYS) GSQ_CUDA_TRY(qb_buf.stage(b, sizeof(double) * 3 * (size_t)m, s));
  // scratch: the handle's cache, or (when another thread holds it) the call's own
  const size_t keep_bytes = (sizeof(int) * FIND_CAP * (size_t)std::max(m, 1) + 255) & ~size_t(255);
  const size_t scan_bytes = (exclusive_scan_work_bytes(m) + 255) & ~size_t(255);
  const size_t csr_bytes = dev_out ? 0 : 2 * align256(sizeof(int) * (size_t)std::max(m, 1));  // host offsets, counts
  const size_t need = keep_bytes + scan_bytes + 256 + csr_bytes;
  FindCache& fc = h->fc;
  std::unique_lock<std::mutex> lock(fc.busy, std::try_to_lock);
  const bool cached = lock.owns_lock();
  Scratch own;
  Events own_ev;
  long long own_host[2];
  char* work = nullptr;
  cudaEvent_t* ev = nullptr;
  long long* hostw = own_host;
  if(cached)
  {
    if(need > fc.work_bytes)
    {
      if(fc.work) cudaFree(fc.work);
      fc.work = nullptr;
      fc.work_bytes = 0;
      GSQ_CUDA_TRY(cudaMalloc(&fc.work, need));
      fc.work_bytes = need;
    }
    if(!fc.host) GSQ_CUDA_TRY(cudaMallocHost(&fc.host, 2 * sizeof(long long)));
    for(auto& e : fc.ev)
      if(!e) GSQ_CUDA_TRY(cudaEventCreate(&e));
    work = static_cast<char*>(fc.work);
    ev = fc.ev;
    hostw = fc.host;
  }
  else
  {
    GSQ_CUDA_TRY(own.alloc(need, s));
    GSQ_CUDA_TRY(own_ev.create());
    work = own.as<char>();
    ev = own_ev.e;
  }
  int* keep = reinterpret_cast<int*>(work);
  void* scan_work = work + keep_bytes;
  long long* d_tot = reinterpret_cast<long long*>(work + keep_bytes + scan_bytes);
  char* csr = csr_bytes ? work + keep_bytes + scan_bytes + 256 : nullptr;
  OutBuf off_buf, cnt_buf;
  GSQ_CUDA_TRY(off_buf.prepare(offsets, sizeof(int) * (size_t)m, s, csr));
  GSQ_CUDA_TRY(cnt_buf.prepare(counts, sizeof(int) * (size_t)m, s, csr ? csr + csr_bytes / 2 : nullptr));
  QueryArgs qa {static_cast<const double*>(qa_buf.dev), static_cast<const double*>(qb_buf.dev), h->tol};
  int* d_cnt = static_cast<int*>(cnt_buf.dev);
  int* d_off = static_cast<int*>(off_buf.dev);
  cudaEventRecord(ev[0], s);
  const NodeKeyRec* nk = nullptr;
  if(KIND != Q_RAYS && m > 0)
  {
    rc = node_keys(h, s, &nk);
    if(rc) return rc;
  }
  if(m > 0)
  {
    count_launch();
    k_find_pass1<KIND><<<grid_for(m, FIND_THREADS), FIND_THREADS, 0, s>>>(h->dev.nodes, nk, h->dev.perm, qa, m,
                                                                          d_cnt, keep, h->d_err);
  }
  rc = exclusive_scan(d_cnt, d_off, m, d_tot, s, scan_work);
  if(rc) return rc;
  cudaEventRecord(ev[1], s);
  // the total and the device error word in one read-back
  hostw[1] = 0;
  GSQ_CUDA_TRY(cudaMemcpyAsync(hostw, d_tot, sizeof(long long), cudaMemcpyDeviceToHost, s));
  GSQ_CUDA_TRY(cudaMemcpyAsync(hostw + 1, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  const long long total = hostw[0];
  if(static_cast<int>(hostw[1]) != 0)
  {
    rc = check_device_error(h->d_err, s, "find pass 1");  // reports and clears the word
    if(rc) return rc;
  }
  if(total > INT_MAX) return fail(GSQ_ERR_INVALID, "more than 2^31-1 candidates");
  // the candidates: a new device array when the caller takes device outputs,
  // else the cache's (grow-only) before the copy to host memory
  int* d_cand = nullptr;
  const size_t cand_bytes = sizeof(int) * (size_t)std::max<long long>(total, 1);
  const bool cand_cached = cached && !dev_out;
  if(cand_cached)
  {
    if(cand_bytes > fc.cand_bytes)
    {
      if(fc.cand) cudaFree(fc.cand);
      fc.cand = nullptr;
      fc.cand_bytes = 0;
      GSQ_CUDA_TRY(cudaMalloc(&fc.cand, cand_bytes));
      fc.cand_bytes = cand_bytes;
    }
    d_cand = static_cast<int*>(fc.cand);
  }
  else
    GSQ_CUDA_TRY(cudaMalloc(&d_cand, cand_bytes));
  cudaEventRecord(ev[2], s);
  if(m > 0)
  {
    count_launch();
    k_find_pass2<KIND><<<grid_for(m, FIND_THREADS), FIND_THREADS, 0, s>>>(h->dev.nodes, nk, h->dev.perm, qa, m,
                                                                          d_cnt, d_off, keep, d_cand);
  }
  cudaEventRecord(ev[3], s);
  cudaError_t e = cudaGetLastError();
  if(e == cudaSuccess) e = off_buf.flush(s);
  if(e == cudaSuccess) e = cnt_buf.flush(s);
  if(e == cudaSuccess && !dev_out)
  {
    int* host = static_cast<int*>(std::malloc(sizeof(int) * (size_t)std::max<long long>(total, 1)));
    if(!host)
      e = cudaErrorMemoryAllocation;
    else
    {
      e = cudaMemcpyAsync(host, d_cand, sizeof(int) * (size_t)total, cudaMemcpyDeviceToHost, s);
      if(e == cudaSuccess) e = cudaStreamSynchronize(s);
      if(!cand_cached) cudaFree(d_cand);
      d_cand = nullptr;
      *candidates = host;
      if(e != cudaSuccess)
      {
        std::free(host);
        *candidates = nullptr;
      }
    }
  }
  else if(dev_out)
    *candidates = d_cand;
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess)
  {
    if(d_cand && !cand_cached) cudaFree(d_cand);
    *candidates = nullptr;
    return cuda_fail(e, "find pass 2");
  }
  if(total_out) *total_out = total;
  float t01 = 0.f, t23 = 0.f;
  cudaEventElapsedTime(&t01, ev[0], ev[1]);
  cudaEventElapsedTime(&t23, ev[2], ev[3]);
  h->find_ms = t01 + t23;
  return GSQ_OK;
}
}  // namespace

extern "C" {

int gsq_bvh_create(gsq_bvh** out)
{
  if(!out) return fail(GSQ_ERR_INVALID, "null output pointer");
  auto* h = new(std::nothrow) gsq_bvh();
  if(!h) return fail(GSQ_ERR_NOMEM, "handle allocation failed");
  cudaError_t e = cudaGetDevice(&h->device);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_err, sizeof(int));
  if(e == cudaSuccess) e = cudaMemset(h->d_err, 0, sizeof(int));
  if(e != cudaSuccess)
  {
    delete h;
    return cuda_fail(e, "gsq_bvh_create");
  }
  *out = h;
  return GSQ_OK;
}

int gsq_bvh_destroy(gsq_bvh* h)
{
  if(!h) return GSQ_OK;
  h->dev.release();
  h->fc.release();
  if(h->nkeys) cudaFree(h->nkeys);
  if(h->nk_ev) cudaEventDestroy(h->nk_ev);
  if(h->d_err) cudaFree(h->d_err);
  delete h;
  return GSQ_OK;
}

int gsq_bvh_set_scale_factor(gsq_bvh* h, double s)
{
  if(!h) return fail(GSQ_ERR_INVALID, "null bvh handle");
  h->scale = s;
  return GSQ_OK;
}
int gsq_bvh_get_scale_factor(const gsq_bvh* h, double* s)
{
  if(!h || !s) return fail(GSQ_ERR_INVALID, "null argument");
  *s = h->scale;
  return GSQ_OK;
}
int gsq_bvh_set_tolerance(gsq_bvh* h, double t)
{
  if(!h) return fail(GSQ_ERR_INVALID, "null bvh handle");
  h->tol = t;
  return GSQ_OK;
}
int gsq_bvh_get_tolerance(const gsq_bvh* h, double* t)
{
  if(!h || !t) return fail(GSQ_ERR_INVALID, "null argument");
  *t = h->tol;
  return GSQ_OK;
}

int gsq_bvh_build(gsq_bvh* h, const double* boxes, int32_t n, void* stream)
{
  if(!h) return fail(GSQ_ERR_INVALID, "null bvh handle");
  if(n < 0 || (n > 0 && !boxes)) return fail(GSQ_ERR_INVALID, "invalid boxes");
  if(n >= (1 << 30)) return fail(GSQ_ERR_INVALID, "at most 2^30-1 boxes");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  h->built = false;
  h->nkeys_ok = false;
  // host boxes go to a staging buffer kept with the handle, so that a repeated
  // build from the same host array replays the captured build
  const double* d_boxes = boxes;
  const size_t bytes = sizeof(double) * 6 * (size_t)n;
  if(n > 0 && !is_device_ptr(boxes))
  {
    if(bytes > h->dev.stage_bytes)
    {
      h->dev.drop_graph();
      if(h->dev.stage) cudaFree(h->dev.stage);
      h->dev.stage = nullptr;
      h->dev.stage_bytes = 0;
      GSQ_CUDA_TRY(cudaMalloc(&h->dev.stage, bytes));
      h->dev.stage_bytes = bytes;
    }
    GSQ_CUDA_TRY(cudaMemcpyAsync(h->dev.stage, boxes, bytes, cudaMemcpyHostToDevice, s));
    d_boxes = static_cast<const double*>(h->dev.stage);
  }
  cudaEvent_t e0, e1;
  GSQ_CUDA_TRY(cudaEventCreate(&e0));
  GSQ_CUDA_TRY(cudaEventCreate(&e1));
  // device time of the build's work: e1 is recorded once it is enqueued,
  // before the read-back of the bounds and of the error word
  cudaEventRecord(e0, s);
  const int rc = bvh_build(h->dev, d_boxes, n, h->scale, s, h->d_err, e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&h->build_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(rc) return rc;
  h->built = true;
  return GSQ_OK;
}

int gsq_bvh_bounds(const gsq_bvh* h, double* lo, double* hi)
{
  int rc = check_bvh(h);
  if(rc) return rc;
  if(!lo || !hi) return fail(GSQ_ERR_INVALID, "null argument");
  for(int d = 0; d < 3; ++d)
  {
    lo[d] = h->dev.bounds[d];
    hi[d] = h->dev.bounds[3 + d];
  }
  return GSQ_OK;
}

int gsq_bvh_num_leaves(const gsq_bvh* h, int32_t* n)
{
  int rc = check_bvh(h);
  if(rc) return rc;
  if(!n) return fail(GSQ_ERR_INVALID, "null argument");
  *n = h->dev.n;
  return GSQ_OK;
}

int gsq_bvh_last_build_ms(const gsq_bvh* h, float* ms)
{
  if(!h || !ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->build_ms;
  return GSQ_OK;
}

int gsq_bvh_last_find_ms(const gsq_bvh* h, float* ms)
{
  if(!h || !ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->find_ms;
  return GSQ_OK;
}

int gsq_bvh_find_boxes(const gsq_bvh* h, const double* q, int32_t m, int32_t* offsets, int32_t* counts,
                       int32_t** candidates, int64_t* total, void* stream)
{
  return find_impl<Q_BOXES>(h, q, nullptr, m, offsets, counts, candidates, total, stream);
}

int gsq_bvh_find_points(const gsq_bvh* h, const double* p, int32_t m, int32_t* offsets, int32_t* counts,
                        int32_t** candidates, int64_t* total, void* stream)
{
  return find_impl<Q_POINTS>(h, p, nullptr, m, offsets, counts, candidates, total, stream);
}

int gsq_bvh_find_rays(const gsq_bvh* h, const double* o, const double* d, int32_t m, int32_t* offsets,
                      int32_t* counts, int32_t** candidates, int64_t* total, void* stream)
{
  return find_impl<Q_RAYS>(h, o, d, m, offsets, counts, candidates, total, stream);
}

int gsq_bvh_get_view(const gsq_bvh* h, gsq_bvh_view* view)
{
  int rc = check_bvh(h);
  if(rc) return rc;
  if(!view) return fail(GSQ_ERR_INVALID, "null view");
  view->nodes = h->dev.nodes;
  view->leaf_ids = h->dev.perm;
  view->num_leaves = h->dev.n;
  view->reserved = 0;
  return GSQ_OK;
}

int gsq_bvh_export(const gsq_bvh* h, double* node_boxes, int32_t* children, int32_t* leaf_ids, uint32_t* codes)
{
  int rc = check_bvh(h);
  if(rc) return rc;
  const int n = h->dev.n, inner = n - 1;
  std::vector<NodeRec64> recs(inner);
  GSQ_CUDA_TRY(cudaMemcpy(recs.data(), h->dev.nodes, sizeof(NodeRec64) * inner, cudaMemcpyDeviceToHost));
  for(int i = 0; i < inner; ++i)
  {
    if(node_boxes) std::memcpy(node_boxes + 12 * (size_t)i, recs[i].b, sizeof(double) * 12);
    if(children)
      for(int k = 0; k < 2; ++k)
      {
        const int c = recs[i].child[k];
        children[2 * i + k] = (c >= 0) ? 2 * c : c;
      }
  }
  if(leaf_ids) GSQ_CUDA_TRY(cudaMemcpy(leaf_ids, h->dev.perm, sizeof(int) * n, cudaMemcpyDeviceToHost));
  if(codes) GSQ_CUDA_TRY(cudaMemcpy(codes, h->dev.codes, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
  return GSQ_OK;
}

}  // extern "C"

namespace gsq
{
// Accessor for the signed-distance translation unit.
const BvhDev* bvh_dev(const gsq_bvh* h) { return h ? &h->dev : nullptr; }
gsq_bvh* bvh_new_internal(int device)
{
  gsq_bvh* h = nullptr;
  if(gsq_bvh_create(&h) != GSQ_OK) return nullptr;
  h->device = device;
  return h;
}
int bvh_build_internal(gsq_bvh* h, const double* d_boxes, int n, cudaStream_t s)
{
  h->built = false;
  h->nkeys_ok = false;
  const int rc = bvh_build(h->dev, d_boxes, n, h->scale, s, h->d_err);
  if(rc == GSQ_OK) h->built = true;
  return rc;
}
}  // namespace gsq
