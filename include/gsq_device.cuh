// Device-side traversal of a gsq BVH from user kernels.
//
// Replaces spin::BVH::getTraverser and LinearBVHTraverser::traverse_tree
// (spin/BVH.hpp:319, spin/policy/LinearBVH.hpp:57-109) for code that writes
// its own kernels over the tree, as quest's two-pass example does
// (quest/examples/quest_bvh_two_pass.cpp:143-200).  Obtain a view of a built
// BVH on the host with gsq_bvh_get_view (gsq.h), pass it to the kernel by
// value and call gsq::device::traverse_tree.  The traversal is the
// reference's (bvh_traverse.hpp:66-154): a 64-entry stack, leaf actions
// deferred until a second leaf is found or the stack runs out, and the
// leaves' original box ids handed to the leaf action.
#pragma once

#include <cfloat>
#include <cstdint>

#include "gsq.h"

namespace gsq
{
namespace device
{
// The node record behind gsq_bvh_view::nodes: the boxes of the two children
// (lo, hi of the left, then of the right) and their links (>= 0: an inner
// node, < 0: -(sorted leaf position + 1)).
struct __align__(16) Node
{
  double b[12];
  int32_t child[2];
  int32_t pad[6];
};
static_assert(sizeof(Node) == 128, "node record is 128 bytes");

__device__ __forceinline__ bool box_is_valid(const double* lo, const double* hi)
{
  return !(lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]);
}

// predicate(lo, hi) -> bool: descend into the child box [lo, hi] (called only
// for valid boxes).  leaf(id): the leaf action, with the box's index in the
// array the BVH was built from.  swap(lo_l, hi_l, lo_r, hi_r) -> bool: when
// both children pass, visit the right one first (the reference's traversal
// preference; return false for none).  Returns false if the stack overflowed
// (the traversal then stops).
template <class Pred, class Leaf, class Swap>
__device__ bool traverse_tree(const gsq_bvh_view& view, Pred&& predicate, Leaf&& leaf, Swap&& swap)
{
  constexpr int STACK = 64;
  constexpr int BARRIER = -2000000000;
  const Node* nodes = static_cast<const Node*>(view.nodes);
  int todo[STACK];
  int sp = 0;
  todo[0] = BARRIER;
  int found = 0, cur = 0;
  while(cur != BARRIER)
  {
    while(cur >= 0)
    {
      const Node& n = nodes[cur];
      const bool inL = box_is_valid(n.b, n.b + 3) && predicate(n.b, n.b + 3);
      const bool inR = box_is_valid(n.b + 6, n.b + 9) && predicate(n.b + 6, n.b + 9);
      if(!inL && !inR)
        cur = (sp >= 0) ? todo[sp--] : BARRIER;
      else
      {
        cur = inL ? n.child[0] : n.child[1];
        int rc = n.child[1];
        if(inL && inR)
        {
          if(swap(n.b, n.b + 3, n.b + 6, n.b + 9))
          {
            const int t = cur;
            cur = rc;
            rc = t;
          }
          if(sp + 1 >= STACK) return false;
          todo[++sp] = rc;
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
      leaf(view.leaf_ids[-found - 1]);
      found = cur;
      if(cur < 0 && cur != BARRIER) cur = (sp >= 0) ? todo[sp--] : BARRIER;
    }
    found = 0;
  }
  return true;
}

// The traversal without a preference (the generic traverser, LinearBVH.hpp:92-103).
template <class Pred, class Leaf>
__device__ bool traverse_tree(const gsq_bvh_view& view, Pred&& predicate, Leaf&& leaf)
{
  return traverse_tree(view, predicate, leaf, [](const double*, const double*, const double*, const double*) {
    return false;
  });
}

// The point traverser's preference (LinearBVH.hpp:72-85): nearer centroid first.
struct NearerCentroid
{
  double p[3];
  __device__ bool operator()(const double* lol, const double* hil, const double* lor, const double* hir) const
  {
    double sl = 0.0, sr = 0.0;
    for(int d = 0; d < 3; ++d)
    {
      const double cl = 0.5 * (lol[d] + hil[d]) - p[d];
      const double cr = 0.5 * (lor[d] + hir[d]) - p[d];
      sl = sl + cl * cl;
      sr = sr + cr * cr;
    }
    return sl > sr;
  }
};
}  // namespace device
}  // namespace gsq
