// Device pieces of the linear BVH build, shared by the single-hierarchy build
// (gsq_bvh.cu) and the segmented build of many meshes (gsq_batch.cu).  Every
// function works on one hierarchy given by base pointers and local indices,
// so a segmented build produces, per mesh, the same bits as a standalone one.
#pragma once

#include "gsq_internal.cuh"

#include <climits>

namespace gsq
{
namespace lbvh
{
// (value, index) pairs folded "leftmost wins on ties", which reproduces the
// strict-comparison updates of BoundingBox::addPoint applied in index order.
struct ArgV
{
  double v;
  int i;
};
// (comparisons on the integer pipe, OKey, with the FP64 outcomes)
__device__ __forceinline__ void take_min(ArgV& a, const ArgV& b)
{
  if(b.i == INT_MAX) return;
  const OKey kb = okey(b.v), ka = okey(a.v);
  if(a.i == INT_MAX || ok_lt(kb, ka) || (ok_eq(kb, ka) && b.i < a.i)) a = b;
}
__device__ __forceinline__ void take_max(ArgV& a, const ArgV& b)
{
  if(b.i == INT_MAX) return;
  const OKey kb = okey(b.v), ka = okey(a.v);
  if(a.i == INT_MAX || ok_gt(kb, ka) || (ok_eq(kb, ka) && b.i < a.i)) a = b;
}
__device__ __forceinline__ ArgV shfl_argv(const ArgV& a, int src)
{
  return ArgV {__shfl_sync(0xFFFFFFFFu, a.v, src), __shfl_sync(0xFFFFFFFFu, a.i, src)};
}

struct Fold
{
  ArgV lo[3], hi[3];
  int first_valid;
};

__device__ __forceinline__ void fold_init(Fold& f)
{
  for(int d = 0; d < 3; ++d)
  {
    f.lo[d] = ArgV {0.0, INT_MAX};
    f.hi[d] = ArgV {0.0, INT_MAX};
  }
  f.first_valid = INT_MAX;
}

__device__ __forceinline__ void fold_merge(Fold& a, const Fold& b)
{
  for(int d = 0; d < 3; ++d)
  {
    take_min(a.lo[d], b.lo[d]);
    take_max(a.hi[d], b.hi[d]);
  }
  a.first_valid = min(a.first_valid, b.first_valid);
}

__device__ __forceinline__ void fold_warp(Fold& f)
{
  const int lane = threadIdx.x & 31;
  for(int off = 16; off > 0; off >>= 1)
  {
    const int src = lane + off < 32 ? lane + off : lane;
    Fold o;
    for(int d = 0; d < 3; ++d)
    {
      o.lo[d] = shfl_argv(f.lo[d], src);
      o.hi[d] = shfl_argv(f.hi[d], src);
    }
    o.first_valid = __shfl_sync(0xFFFFFFFFu, f.first_valid, src);
    fold_merge(f, o);
  }
}

// Folds a whole block (blockDim.x a multiple of 32, at most 1024); the result
// is valid in thread 0.
__device__ __forceinline__ Fold fold_block(Fold f)
{
  __shared__ Fold s_f[32];
  fold_warp(f);
  if((threadIdx.x & 31) == 0) s_f[threadIdx.x >> 5] = f;
  __syncthreads();
  Fold a;
  fold_init(a);
  if(threadIdx.x < 32)
  {
    // the first warp merges the warps' folds (the merge is commutative)
    if(threadIdx.x < (blockDim.x >> 5)) a = s_f[threadIdx.x];
    fold_warp(a);
  }
  __syncthreads();
  return a;
}

// BoundingBox::scale (BoundingBox.hpp:548-561): mid = 0.5*(lo+hi),
// r = (s*0.5)*(hi-lo), lo' = mid - r, hi' = mid + r, then checkAndFixBounds.
// Invalid boxes are left as they are.  Returns the box's validity.
__device__ __forceinline__ bool scale_box(double* lo, double* hi, double half)
{
  const OKey kl[3] = {okey(lo[0]), okey(lo[1]), okey(lo[2])};
  const OKey kh[3] = {okey(hi[0]), okey(hi[1]), okey(hi[2])};
  const bool valid = box_valid_k(kl, kh);
  if(valid)
  {
    for(int d = 0; d < 3; ++d)
    {
      const double mid = 0.5 * (lo[d] + hi[d]);
      const double r = (hi[d] - lo[d]) * half;
      lo[d] = mid - r;
      hi[d] = mid + r;
    }
    for(int d = 0; d < 3; ++d)
      if(ok_gt(okey(lo[d]), okey(hi[d])))
      {
        const double t = lo[d];
        lo[d] = hi[d];
        hi[d] = t;
      }
  }
  return valid;
}

// One valid scaled box into the bounds fold.  reduce's SEQ branch (BR:134-141)
// copies the first valid box and then, for every later valid box, calls
// addPoint(lo) and addPoint(hi): per axis, strict "<" / ">" updates in that
// order.  So a later box offers the min fold lo (or hi where lo is NaN) and
// the max fold hi (lo where they are equal, so that the earlier of two equal
// values, e.g. -0 before +0, is kept, or where hi is NaN); a NaN never wins a
// comparison and is not offered.  The first valid box's own coordinates are
// applied by bounds_params, a NaN among them included (a NaN copied into the
// running box is never replaced).
__device__ __forceinline__ void fold_add_box(Fold& f, const double* lo, const double* hi, int i)
{
  for(int d = 0; d < 3; ++d)
  {
    const OKey kl = okey(lo[d]), kh = okey(hi[d]);
    const double vmin = kl.nan ? hi[d] : lo[d];
    const double vmax = kl.nan ? hi[d] : (kh.nan ? lo[d] : (ok_eq(kl, kh) ? lo[d] : hi[d]));
    if(!okey(vmin).nan) take_min(f.lo[d], ArgV {vmin, i});
    if(!okey(vmax).nan) take_max(f.hi[d], ArgV {vmax, i});
  }
  f.first_valid = min(f.first_valid, i);
}

// Bounds and Morton parameters from the folded boxes.  leaf holds the scaled
// boxes addressed by the fold's indices; last is the index of the last box
// (the fold's result when no box is valid).  params: bounds lo[3] hi[3], then
// Morton min[3], inv_extent[3].
__device__ __forceinline__ void bounds_params(const Fold& a, const double* __restrict__ leaf, int last,
                                              double* __restrict__ params)
{
  double lo[3], hi[3];
  if(a.first_valid == INT_MAX)
  {
    for(int d = 0; d < 3; ++d)
    {
      lo[d] = leaf[6 * (size_t)last + d];
      hi[d] = leaf[6 * (size_t)last + 3 + d];
    }
  }
  else
  {
    // the first valid box's coordinates start the running box: they stand
    // where they win (ties included, being first) and where they are NaN
    const double* fb = leaf + 6 * (size_t)a.first_valid;
    for(int d = 0; d < 3; ++d)
    {
      const bool lnan = okey(fb[d]).nan, hnan = okey(fb[3 + d]).nan;
      lo[d] = (lnan || a.lo[d].i == INT_MAX) ? fb[d] : a.lo[d].v;
      hi[d] = (hnan || a.hi[d].i == INT_MAX || a.hi[d].i == a.first_valid) ? fb[3 + d] : a.hi[d].v;
    }
  }
  for(int d = 0; d < 3; ++d)
  {
    params[d] = lo[d];
    params[3 + d] = hi[d];
    // get_mcodes (BR:154-163): inv_extent = isNearlyEqual(extent, 0) ? 0 : 1/extent
    const double ext = hi[d] - lo[d];
    params[6 + d] = lo[d];
    params[9 + d] = (fabs(ext - 0.0) <= 1.0e-8) ? 0.0 : 1.0 / ext;
  }
}

// 10-bit spread for a 3D Morton interleave (Ericson's magic numbers; the
// reference's Mortonizer<int32,int32,3>::expandBits, spin/MortonIndex.hpp:151-159).
__host__ __device__ __forceinline__ uint32_t spread10(uint32_t x)
{
  x = (x | (x << 16)) & 0xFF0000FFu;
  x = (x | (x << 8)) & 0x0F00F00Fu;
  x = (x | (x << 4)) & 0xC30C30C3u;
  x = (x | (x << 2)) & 0x49249249u;
  return x;
}

// morton32_encode (BR:48-65) of the normalised centroid (BR:165-175).
__device__ __forceinline__ uint32_t box_morton(const double* __restrict__ box, const double* __restrict__ params)
{
  uint32_t q[3];
  for(int d = 0; d < 3; ++d)
  {
    const double mid = 0.5 * (box[d] + box[3 + d]);
    const double c = (mid - params[6 + d]) * params[9 + d];
    q[d] = (uint32_t)(int)fmin(fmax(c * 1024.0, 0.0), 1023.0);
  }
  return spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
}

// delta (BR:265-287); ca is codes[a], loaded once by the caller
__device__ __forceinline__ int delta(int a, uint32_t ca, int b, int inner, const uint32_t* __restrict__ codes)
{
  const bool oor = (b < 0 || b > inner);
  const int bb = oor ? 0 : b;
  uint32_t x = ca ^ __ldg(codes + bb);
  const bool tie = (x == 0);
  if(tie) x = (uint32_t)a ^ (uint32_t)bb;
  int c = __clz(x);
  if(tie) c += 32;
  return oor ? -1 : c;
}

// build_tree (BR:290-384) for inner node i of a hierarchy over n sorted codes;
// also writes the child links of the node record.  Leaf j has node id
// inner + j in lchild/rchild/parent; parent[x] holds the parent's id times two
// plus the side of x (0 left, 1 right), -1 at the root.
__device__ __forceinline__ void karras_node(int i, const uint32_t* __restrict__ codes, int n, int* __restrict__ lchild,
                                            int* __restrict__ rchild, int* __restrict__ parent,
                                            NodeRec64* __restrict__ nodes)
{
  const int inner = n - 1;
  const uint32_t ci = __ldg(codes + i);
  const int dir = (delta(i, ci, i + 1, inner, codes) - delta(i, ci, i - 1, inner, codes)) < 0 ? -1 : 1;
  const int dmin = delta(i, ci, i - dir, inner, codes);
  int lmax = 2;
  while(delta(i, ci, i + lmax * dir, inner, codes) > dmin) lmax *= 2;
  int l = 0;
  for(int s = lmax / 2; s >= 1; s /= 2)
    if(delta(i, ci, i + (l + s) * dir, inner, codes) > dmin) l += s;
  const int j = i + l * dir;
  const int dnode = delta(i, ci, j, inner, codes);
  int s = 0;
  // The reference's step is ceil(float32(l) / div) in FloatType = double with
  // div = 2, 4, 8, ...: float32(l) is an integer L and dividing it by a power
  // of two is exact, so the step is ceil(L / 2^k) = (L + 2^k - 1) >> k,
  // computed here without FP64 arithmetic (scarce on this GPU).
  const long long L = (long long)(float)l;
  for(int k = 1;; ++k)
  {
    const int st = (int)((L + (1LL << k) - 1) >> k);
    if(delta(i, ci, i + (s + st) * dir, inner, codes) > dnode) s += st;
    if(st == 1) break;
  }
  const int split = i + s * dir + min(dir, 0);
  int lc, rc;
  if(min(i, j) == split)
  {
    parent[split + inner] = 2 * i;
    lc = split + inner;
  }
  else
  {
    parent[split] = 2 * i;
    lc = split;
  }
  if(max(i, j) == split + 1)
  {
    parent[split + inner + 1] = 2 * i + 1;
    rc = split + inner + 1;
  }
  else
  {
    parent[split + 1] = 2 * i + 1;
    rc = split + 1;
  }
  lchild[i] = lc;
  rchild[i] = rc;
  nodes[i].child[0] = (lc >= inner) ? -(lc - inner + 1) : lc;
  nodes[i].child[1] = (rc >= inner) ? -(rc - inner + 1) : rc;
  if(i == 0) parent[0] = -1;
}

// BoundingBox::addBox (BoundingBox.hpp:487-505) into acc (comparisons on the
// integer pipe, OKey, with the FP64 outcomes).
__device__ __forceinline__ void add_box(double* alo, double* ahi, const double* lo, const double* hi)
{
  OKey ka[3], kb[3], kl[3], kh[3];
  for(int d = 0; d < 3; ++d)
  {
    ka[d] = okey(alo[d]);
    kb[d] = okey(ahi[d]);
    kl[d] = okey(lo[d]);
    kh[d] = okey(hi[d]);
  }
  if(box_valid_k(ka, kb))
  {
    if(box_valid_k(kl, kh))
    {
      for(int d = 0; d < 3; ++d)
      {
        if(ok_lt(kl[d], ka[d]))
        {
          alo[d] = lo[d];
          ka[d] = kl[d];
        }
        if(ok_gt(kl[d], kb[d]))
        {
          ahi[d] = lo[d];
          kb[d] = kl[d];
        }
      }
      for(int d = 0; d < 3; ++d)
      {
        if(ok_lt(kh[d], ka[d])) alo[d] = hi[d];
        if(ok_gt(kh[d], kb[d])) ahi[d] = hi[d];
      }
    }
  }
  else
    for(int d = 0; d < 3; ++d)
    {
      alo[d] = lo[d];
      ahi[d] = hi[d];
    }
}

// atomicAdd with acquire-release ordering at device scope: the caller's
// earlier stores are visible to whoever reads the counter's new value, and
// the caller sees the stores of the threads whose increments it read.
__device__ __forceinline__ int atomic_add_acq_rel(int* p, int v)
{
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// propagate_aabbs (BR:505-576) fused with emit_bvh_parents (LB:225-264), one
// level at a time: a thread stores its node's box into the parent's record and
// bumps the parent's counter with an acquire-release atomic (the store is
// visible to the second arrival, which sees the first arrival's box); the first
// arrival stops and the second combines the two child boxes as the reference's
// SEQ order does (box(node) = addBox(box(right), box(left))) and moves up.  No
// thread ever waits on another.
// One level of the refit for the node with box (lo, hi) and parent code pcode
// (parent id * 2 + side).  The parent's own code is read before the atomic,
// so that its latency overlaps the atomic's; the second arrival reads only
// its sibling's box back.  Returns true when this thread continues: (lo, hi)
// is then the parent's box and pcode the parent's code.  At the root the box
// goes to root_box and it returns false.
__device__ __forceinline__ bool refit_step(int& pcode, double* lo, double* hi, const int* __restrict__ parent,
                                           int* __restrict__ counters, NodeRec64* nodes, double* __restrict__ root_box)
{
  const int node = pcode >> 1, side = pcode & 1;
  const int next = __ldg(parent + node);
  double* b = nodes[node].b;
  for(int d = 0; d < 3; ++d)
  {
    b[6 * side + d] = lo[d];
    b[6 * side + 3 + d] = hi[d];
  }
  if(atomic_add_acq_rel(&counters[node], 1) == 0) return false;
  double slo[3], shi[3];
  for(int d = 0; d < 3; ++d)
  {
    slo[d] = __ldcg(b + 6 * (1 - side) + d);
    shi[d] = __ldcg(b + 6 * (1 - side) + 3 + d);
  }
  if(side == 0)
  {
    // this thread holds the left box: start from the right (sibling's) box
    add_box(slo, shi, lo, hi);
    for(int d = 0; d < 3; ++d)
    {
      lo[d] = slo[d];
      hi[d] = shi[d];
    }
  }
  else
    add_box(lo, hi, slo, shi);
  pcode = next;
  if(next < 0)
  {
    if(root_box)
      for(int d = 0; d < 3; ++d)
      {
        root_box[d] = lo[d];
        root_box[3 + d] = hi[d];
      }
    return false;
  }
  return true;
}

}  // namespace lbvh
}  // namespace gsq
