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
#include "gsq_sdf_mixed_kernel.cuh"

#include <algorithm>
#include <type_traits>

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
    r.pad[side] = __float_as_int(node_box32(in[i].b + 6 * side, r.b + 6 * side));
  }
  r.child[0] = in[i].child[0];
  r.child[1] = in[i].child[1];
  out[i] = r;
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
    tri_error_terms(v, v + 3, v + 6, r.ec, r.lt, &r.fz);
  }
  else
  {
    tri_error_terms(v, v + 3, v + 6, r.ec[0], r.lt[0]);
    tri_error_terms(v, v + 6, v + 9, r.ec[1], r.lt[1]);
  }
  out[k] = r;
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
                 const void* leaves32, const MeshInfo* meshes, const sdf::QueryPts& qp, int m, const int* order,
                 const sdf::SdfParams& prm, double* out, double* out_cp, double* out_n, int* err,
                 unsigned long long* audit, int* work, int block, int depth, cudaStream_t s)
{
  if(depth != 1 && depth != 16) depth = 4;
  const int threads = (block >= 32 && block <= 128) ? (block / 32) * 32 : 128;
  GSQ_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), s));
  auto go = [&](auto npc_c, auto audit_c, auto depth_c) {
    return launch_mixed<decltype(npc_c)::value, decltype(audit_c)::value, decltype(depth_c)::value, STACK_SIZE,
                        false>(threads, s, nodes64, nodes32, leaves64, leaves32, meshes, 1, nullptr, qp, m, order,
                               prm, out, out_cp, out_n, err, MixedStats {audit}, work);
  };
  auto by_depth = [&](auto npc_c, auto audit_c) {
    if(depth == 16) return go(npc_c, audit_c, std::integral_constant<int, 16> {});
    if(depth == 4) return go(npc_c, audit_c, std::integral_constant<int, 4> {});
    return go(npc_c, audit_c, std::integral_constant<int, 1> {});
  };
  auto by_audit = [&](auto npc_c) {
    return audit ? by_depth(npc_c, std::true_type {}) : by_depth(npc_c, std::false_type {});
  };
  const cudaError_t e = (npc == 3) ? by_audit(std::integral_constant<int, 3> {})
                                   : by_audit(std::integral_constant<int, 4> {});
  count_launch();
  GSQ_CUDA_TRY(e);
  return GSQ_OK;
}

}  // namespace gsq
