// Adjoint of the signed distance: gradients of a loss L(d) with respect to
// the query points and the mesh vertices.  The reference has no gradient; the
// forward value it differentiates is computeDistances (quest/SignedDistance.hpp:
// 527-605).
//
// For a point q whose closest point cp lies on triangle (V0, V1, V2) with
// barycentric weights b (from the Voronoi region of closest_point,
// primal/operators/closest_point.hpp:162-290) and sign s, d = s |q - cp|.  With
// u = (q - cp) / |q - cp| the envelope theorem gives
//   dd/dq  =  s u                 dd/dV_k = -s b_k u
// (the sign is piecewise constant; at |q - cp| = 0 both are taken as 0).
//
// The backward pass runs the persistent mixed query (the forward's traversal,
// so cp is the forward's cp bit for bit), which also writes each point's
// closest triangle; k_adjoint_apply then forms cp's barycentric weights on
// that triangle and writes dL/dq plus three vertex contributions per point,
// the sign taken from the signed distance the query wrote.  The vertex
// gradient is then reduced deterministically: the contributions are sorted by
// vertex id with a stable radix sort (ties keep point order) and each vertex's
// segment is summed by one thread in that order, so the result does not depend
// on scheduling and repeats bit for bit.
#include "gsq_sdf_handle.cuh"
#include "gsq_sdf_mixed_kernel.cuh"

#include <algorithm>
#include <cstring>

namespace gsq
{
namespace
{
using namespace sdf;

// closest_point with the barycentric weights of the returned point; the point
// itself is computed with exactly the operations of closest_point.
__device__ __forceinline__ void closest_point_bary(const double* P, const double* A, const double* B, const double* C,
                                                   double* out, double* bary)
{
  const double ab0 = B[0] - A[0], ab1 = B[1] - A[1], ab2 = B[2] - A[2];
  const double ac0 = C[0] - A[0], ac1 = C[1] - A[1], ac2 = C[2] - A[2];
  const double ap0 = P[0] - A[0], ap1 = P[1] - A[1], ap2 = P[2] - A[2];
  const double d1 = dot3(ab0, ab1, ab2, ap0, ap1, ap2);
  const double d2 = dot3(ac0, ac1, ac2, ap0, ap1, ap2);
  bary[0] = bary[1] = bary[2] = 0.0;
  if(is_leq(d1, 0.0) && is_leq(d2, 0.0))
  {
    out[0] = A[0], out[1] = A[1], out[2] = A[2];
    bary[0] = 1.0;
    return;
  }
  const double bp0 = P[0] - B[0], bp1 = P[1] - B[1], bp2 = P[2] - B[2];
  const double d3 = dot3(ab0, ab1, ab2, bp0, bp1, bp2);
  const double d4 = dot3(ac0, ac1, ac2, bp0, bp1, bp2);
  if(is_geq(d3, 0.0) && is_leq(d4, d3))
  {
    out[0] = B[0], out[1] = B[1], out[2] = B[2];
    bary[1] = 1.0;
    return;
  }
  const double vc = d1 * d4 - d3 * d2;
  if(is_leq(vc, 0.0) && is_geq(d1, 0.0) && is_leq(d3, 0.0) && !abs_le_eps(d1 - d3))
  {
    const double v = d1 / (d1 - d3);
    out[0] = A[0] + ab0 * v, out[1] = A[1] + ab1 * v, out[2] = A[2] + ab2 * v;
    bary[0] = 1.0 - v, bary[1] = v;
    return;
  }
  const double cp0 = P[0] - C[0], cp1 = P[1] - C[1], cp2 = P[2] - C[2];
  const double d5 = dot3(ab0, ab1, ab2, cp0, cp1, cp2);
  const double d6 = dot3(ac0, ac1, ac2, cp0, cp1, cp2);
  if(is_geq(d6, 0.0) && is_leq(d5, d6))
  {
    out[0] = C[0], out[1] = C[1], out[2] = C[2];
    bary[2] = 1.0;
    return;
  }
  const double vb = d5 * d2 - d1 * d6;
  if(is_leq(vb, 0.0) && is_geq(d2, 0.0) && is_leq(d6, 0.0))
  {
    const double w = d2 / (d2 - d6);
    out[0] = A[0] + ac0 * w, out[1] = A[1] + ac1 * w, out[2] = A[2] + ac2 * w;
    bary[0] = 1.0 - w, bary[2] = w;
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if(is_leq(va, 0.0) && is_geq(d4 - d3, 0.0) && is_geq(d5 - d6, 0.0))
  {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    out[0] = B[0] + (C[0] - B[0]) * w, out[1] = B[1] + (C[1] - B[1]) * w, out[2] = B[2] + (C[2] - B[2]) * w;
    bary[1] = 1.0 - w, bary[2] = w;
    return;
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom, w = vc * denom;
  const double n0 = ab0 * v + ac0 * w, n1 = ab1 * v + ac1 * w, n2 = ab2 * v + ac2 * w;
  out[0] = A[0] + n0, out[1] = A[1] + n1, out[2] = A[2] + n2;
  bary[0] = 1.0 - v - w, bary[1] = v, bary[2] = w;
}

// Per point: the gradient directions from its closest triangle (tri: c, or
// 2c / 2c + 1 within quad cell c; -1 for none), whose vertices are read from
// the mesh arrays (the values the leaf records hold), and the sign of its
// signed distance d = sqrt(minSq) * sign.
template <int NPC>
__global__ void __launch_bounds__(256) k_adjoint_apply(const double* __restrict__ x, const double* __restrict__ y,
                                                       const double* __restrict__ z, const int* __restrict__ cells,
                                                       QueryPts qp,
                                                       int m,
                                                       const double* __restrict__ dist,
                                                       const int* __restrict__ tri,
                                                       const double* __restrict__ grad_d,
                                                       double* __restrict__ grad_q,
                                                       uint32_t* __restrict__ vkeys,
                                                       double* __restrict__ vcontrib)
{
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if(idx >= m) return;
  const double q[3] = {qp.x[(size_t)idx * qp.stride], qp.y[(size_t)idx * qp.stride], qp.z[(size_t)idx * qp.stride]};
  const double sgn = signbit(dist[idx]) ? -1.0 : 1.0;
  const int t = tri[idx];
  double u[3] = {0.0, 0.0, 0.0}, bary[3] = {0.0, 0.0, 0.0};
  int vid[3] = {0, 0, 0};
  if(t >= 0)
  {
    const int cell = (NPC == 3) ? t : (t >> 1);
    const int s1 = (NPC == 4 && (t & 1)) ? 2 : 1;
    vid[0] = __ldg(cells + (size_t)cell * NPC);
    vid[1] = __ldg(cells + (size_t)cell * NPC + s1);
    vid[2] = __ldg(cells + (size_t)cell * NPC + s1 + 1);
    double v[9];
    for(int k = 0; k < 3; ++k)
    {
      v[3 * k] = __ldg(x + vid[k]);
      v[3 * k + 1] = __ldg(y + vid[k]);
      v[3 * k + 2] = __ldg(z + vid[k]);
    }
    double cp[3];
    closest_point_bary(q, v, v + 3, v + 6, cp, bary);
    const double r0 = q[0] - cp[0], r1 = q[1] - cp[1], r2 = q[2] - cp[2];
    const double len = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
    if(len > 0.0) u[0] = r0 / len, u[1] = r1 / len, u[2] = r2 / len;
  }
  const double coef = grad_d[idx] * sgn;
  if(grad_q)
    for(int c = 0; c < 3; ++c) grad_q[3 * (size_t)idx + c] = coef * u[c];
  if(vkeys)
    for(int k = 0; k < 3; ++k)
    {
      const size_t r = 3 * (size_t)idx + k;
      vkeys[r] = (uint32_t)vid[k];
      for(int c = 0; c < 3; ++c) vcontrib[3 * r + c] = -coef * bary[k] * u[c];
    }
}

// One thread per sorted record; the first record of each vertex's segment sums
// the segment in sorted (stable) order.
__global__ void k_segment_sum(const uint32_t* __restrict__ keys, const int* __restrict__ recs, long long n,
                              const double* __restrict__ contrib, double* __restrict__ grad_v, int nverts)
{
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if(p >= n) return;
  const uint32_t key = keys[p];
  if(p > 0 && keys[p - 1] == key) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for(long long j = p; j < n && keys[j] == key; ++j)
  {
    const double* c = contrib + 3 * (size_t)recs[j];
    s0 += c[0];
    s1 += c[1];
    s2 += c[2];
  }
  if((int)key < nverts)
  {
    grad_v[3 * (size_t)key + 0] = s0;
    grad_v[3 * (size_t)key + 1] = s1;
    grad_v[3 * (size_t)key + 2] = s2;
  }
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

int vertex_key_bits(int nverts)
{
  int b = 1;
  while(b < 31 && (1ll << b) < (long long)std::max(nverts, 1)) ++b;
  return b;
}
}  // namespace
}  // namespace gsq

namespace gsq
{
int mixed_launch_tri(int npc, const NodeRec64* nodes64, const NodeRec32* nodes32, const void* leaves64,
                     const void* leaves32, const MeshInfo* meshes, const sdf::QueryPts& qp, int m, const int* order,
                     const sdf::SdfParams& prm, double* out, double* out_cp, double* out_n, int* err, int* work,
                     int* tri, cudaStream_t s)
{
  GSQ_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), s));
  cudaError_t e;
  if(npc == 3)
    e = launch_mixed<3, false, 4, STACK_SIZE, false, true>(128, s, nodes64, nodes32, leaves64, leaves32, meshes, 1,
                                                            nullptr, qp, m, order, prm, out, out_cp, out_n, err,
                                                            MixedStats {nullptr}, work, tri);
  else
    e = launch_mixed<4, false, 4, STACK_SIZE, false, true>(128, s, nodes64, nodes32, leaves64, leaves32, meshes, 1,
                                                            nullptr, qp, m, order, prm, out, out_cp, out_n, err,
                                                            MixedStats {nullptr}, work, tri);
  count_launch();
  GSQ_CUDA_TRY(e);
  return GSQ_OK;
}
}  // namespace gsq

using namespace gsq;

namespace
{
// gsq_sdf_backward and gsq_sdf_backward_tri: with dist_in and tri_in null,
// the closest triangles come from the mixed query run here.
int backward_impl(const gsq_sdf* hc, const double* qx, const double* qy, const double* qz, int32_t stride, int32_t m,
                  const double* dist_in, const int32_t* tri_in, const double* grad_dist, double* grad_points,
                  double* grad_vertices, void* stream)
{
  gsq_sdf* h = const_cast<gsq_sdf*>(hc);
  if(!h) return fail(GSQ_ERR_INVALID, "null sdf handle");
  if(m < 0 || stride < 1) return fail(GSQ_ERR_INVALID, "invalid query count or stride");
  if(3ll * m >= (1ll << 30)) return fail(GSQ_ERR_INVALID, "too many points for one backward call");
  if(m > 0 && (!qx || !qy || !qz || !grad_dist)) return fail(GSQ_ERR_INVALID, "null query or gradient array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  OutBuf gq, gv;
  GSQ_CUDA_TRY(gv.prepare(grad_vertices, sizeof(double) * 3 * (size_t)h->nverts, s));
  if(gv.dev) GSQ_CUDA_TRY(cudaMemsetAsync(gv.dev, 0, sizeof(double) * 3 * (size_t)h->nverts, s));
  if(m == 0)
  {
    GSQ_CUDA_TRY(gv.flush(s));
    GSQ_CUDA_TRY(cudaStreamSynchronize(s));
    return GSQ_OK;
  }
  InBuf qb[3], gb, db, tb;
  sdf::QueryPts qp;
  int rc = stage_query_points(qx, qy, qz, stride, m, s, qb, qp);
  if(rc) return rc;
  GSQ_CUDA_TRY(gb.stage(grad_dist, sizeof(double) * (size_t)m, s));
  GSQ_CUDA_TRY(gq.prepare(grad_points, sizeof(double) * 3 * (size_t)m, s));

  const double* dist = nullptr;
  const int* tri = nullptr;
  Scratch order_buf, fwd;
  // the work counter of the mixed query: the handle's unless another thread
  // holds it (held until the stream has synchronised below)
  std::unique_lock<std::mutex> lock(h->work_busy, std::defer_lock);
  if(tri_in)
  {
    GSQ_CUDA_TRY(db.stage(dist_in, sizeof(double) * (size_t)m, s));
    GSQ_CUDA_TRY(tb.stage(tri_in, sizeof(int32_t) * (size_t)m, s));
    dist = static_cast<const double*>(db.dev);
    tri = static_cast<const int*>(tb.dev);
  }
  else
  {
    const BvhDev* B = bvh_dev(h->bvh);
    GSQ_CUDA_TRY(order_buf.alloc(4 * sizeof(uint32_t) * (size_t)m, s));
    uint32_t* okeys[2] = {order_buf.as<uint32_t>(), order_buf.as<uint32_t>() + m};
    int* ovals[2] = {reinterpret_cast<int*>(order_buf.as<uint32_t>() + 2 * (size_t)m),
                     reinterpret_cast<int*>(order_buf.as<uint32_t>() + 3 * (size_t)m)};
    const int* order = nullptr;
    rc = sdf_query_order(h, qp, m, okeys, ovals, &order, s);
    if(rc) return rc;
    GSQ_CUDA_TRY(fwd.alloc(align256(sizeof(double) * (size_t)m) + sizeof(int) * ((size_t)m + 64), s));
    double* d = fwd.as<double>();
    int* t = reinterpret_cast<int*>(fwd.as<char>() + align256(sizeof(double) * (size_t)m));
    int* work = t + m;
    if(lock.try_lock()) work = h->d_work;
    sdf::SdfParams prm;
    std::memcpy(prm.domain, h->domain, sizeof(prm.domain));
    prm.watertight = h->watertight;
    prm.sign = h->sign;
    rc = mixed_launch_tri(h->npc, B->nodes, h->nodes32, h->leaves, h->leaves32, h->d_mesh, qp, m, order, prm, d,
                          nullptr, nullptr, h->d_err, work, t, s);
    if(rc) return rc;
    dist = d;
    tri = t;
  }

  const long long nrec = gv.dev ? 3ll * m : 0;
  Scratch rec_buf;
  uint32_t* vkeys[2] = {nullptr, nullptr};
  int* vvals[2] = {nullptr, nullptr};
  double* contrib = nullptr;
  if(nrec)
  {
    GSQ_CUDA_TRY(rec_buf.alloc((sizeof(double) * 3 + 4 * sizeof(uint32_t)) * (size_t)nrec, s));
    contrib = rec_buf.as<double>();
    uint32_t* w = reinterpret_cast<uint32_t*>(contrib + 3 * (size_t)nrec);
    vkeys[0] = w;
    vkeys[1] = w + nrec;
    vvals[0] = reinterpret_cast<int*>(w + 2 * nrec);
    vvals[1] = reinterpret_cast<int*>(w + 3 * nrec);
  }
  count_launch();
  if(h->npc == 3)
    k_adjoint_apply<3><<<grid_for(m, 256), 256, 0, s>>>(h->d_x, h->d_y, h->d_z, h->d_cells, qp, m, dist, tri,
                                                        static_cast<const double*>(gb.dev),
                                                        static_cast<double*>(gq.dev), vkeys[0], contrib);
  else
    k_adjoint_apply<4><<<grid_for(m, 256), 256, 0, s>>>(h->d_x, h->d_y, h->d_z, h->d_cells, qp, m, dist, tri,
                                                        static_cast<const double*>(gb.dev),
                                                        static_cast<double*>(gq.dev), vkeys[0], contrib);
  GSQ_CUDA_TRY(cudaGetLastError());
  if(nrec)
  {
    const int which = radix_sort_pairs(vkeys, vvals, (int)nrec, vertex_key_bits(h->nverts), true, s, h->d_err);
    if(which < 0) return which;
    count_launch();
    k_segment_sum<<<grid_for(nrec, 256), 256, 0, s>>>(vkeys[which], vvals[which], nrec, contrib,
                                                      static_cast<double*>(gv.dev), h->nverts);
    GSQ_CUDA_TRY(cudaGetLastError());
  }
  GSQ_CUDA_TRY(gq.flush(s));
  GSQ_CUDA_TRY(gv.flush(s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  return check_device_error(h->d_err, s, "gsq_sdf_backward");
}
}  // namespace

extern "C" {

int gsq_sdf_backward(const gsq_sdf* h, const double* qx, const double* qy, const double* qz, int32_t stride,
                     int32_t m, const double* grad_dist, double* grad_points, double* grad_vertices, void* stream)
{
  return backward_impl(h, qx, qy, qz, stride, m, nullptr, nullptr, grad_dist, grad_points, grad_vertices, stream);
}

int gsq_sdf_backward_tri(const gsq_sdf* h, const double* qx, const double* qy, const double* qz, int32_t stride,
                         int32_t m, const double* dist, const int32_t* triangles, const double* grad_dist,
                         double* grad_points, double* grad_vertices, void* stream)
{
  if(m > 0 && (!dist || !triangles)) return fail(GSQ_ERR_INVALID, "null distance or triangle array");
  return backward_impl(h, qx, qy, qz, stride, m, dist, triangles, grad_dist, grad_points, grad_vertices, stream);
}

}  // extern "C"
