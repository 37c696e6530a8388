// Signed distance to a surface mesh on the GPU (quest::SignedDistance
// replacement).
//
// Set-up (replaces SignedDistance::setMesh, quest/SignedDistance.hpp:427-504):
// the mesh is copied to the device, the mesh box is folded (SD:483-486), one
// box per cell is built (getCellBoundingBox, SD:608-633) and the BVH is built
// over them.  Then one "leaf record" per sorted BVH leaf is written with the
// cell's vertex coordinates inline, so a leaf test is one contiguous 80-byte
// (triangle) or 112-byte (quad) read instead of id -> connectivity -> vertex
// gathers.
//
// Query (replaces computeDistances, SD:527-605): one thread per point runs
// the reference traversal (bvh_traverse.hpp:66-154) with the point
// traverser's nearer-centroid-first order (policy/LinearBVH.hpp:72-85), the
// min-distance predicate (SD:576-578) and checkCandidate (SD:636-737), all in
// FP64 with the reference's operation order, so distances, closest points and
// signs are bit-identical to the reference.  Queries may be processed in
// Morton order of the point (results are per point, so order does not change
// them) for warp coherence and cache reuse.
#include "gsq_sdf_handle.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace gsq
{
const BvhDev* bvh_dev(const gsq_bvh* h);
gsq_bvh* bvh_new_internal(int device);
int bvh_build_internal(gsq_bvh* h, const double* d_boxes, int n, cudaStream_t s);
int node_bounds(const double* x, const double* y, const double* z, int nv, double* out6, cudaStream_t s);


namespace
{
using namespace sdf;

template <int NPC>
__global__ void __launch_bounds__(128) k_sdf_fp64(const NodeRec64* __restrict__ nodes,
                                                  const LeafRec<NPC>* __restrict__ leaves,
                                                  QueryPts qp,
                                                  int m,
                                                  const int* __restrict__ order,
                                                  SdfParams prm,
                                                  double* __restrict__ out,
                                                  double* __restrict__ out_cp,
                                                  double* __restrict__ out_n,
                                                  int* __restrict__ out_tri,
                                                  int* err)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if(t >= m) return;
  const int idx = order ? __ldg(order + t) : t;
  const double q[3] = {qp.x[(size_t)idx * qp.stride], qp.y[(size_t)idx * qp.stride], qp.z[(size_t)idx * qp.stride]};
  const bool computeNormal = prm.sign != 0;
  MinCand mc;
  init_min(mc);
  auto visit = [&](int cur, bool& inL, bool& inR, bool& swap, int2& ch) {
    ch = __ldg(reinterpret_cast<const int2*>(nodes[cur].child));
    visit_fp64(nodes, cur, q, mc.minSq, inL, inR, swap);
  };
  auto leaf = [&](int leafpos) { check_leaf<NPC>(q, mc, leaves, leafpos, computeNormal); };
  if(!traverse_point(visit, leaf)) atomicOr(err, DEVERR_STACK);
  finish_query<NPC>(q, mc, leaves, prm, idx, out, out_cp, out_n);
  if(out_tri)
  {
    // the closest triangle (c, or 2c / 2c + 1 within quad cell c; -1: none)
    const int cell = (mc.leaf < 0) ? -1 : __ldg(&leaves[mc.leaf].cell);
    out_tri[idx] = (cell < 0) ? -1 : (NPC == 3 ? cell : 2 * cell + mc.sub);
  }
}

// Per-cell bounding boxes (getCellBoundingBox, SD:608-633): addPoint of each
// node into an invalid box.
__global__ void k_cell_boxes(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                             const int* __restrict__ cells, int ncells, int npc, int nverts, double* __restrict__ boxes,
                             int* err)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if(c >= ncells) return;
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  OKey klo[3], khi[3];
  for(int d = 0; d < 3; ++d)
  {
    klo[d] = okey(lo[d]);
    khi[d] = okey(hi[d]);
  }
  for(int k = 0; k < npc; ++k)
  {
    int v = cells[(size_t)c * npc + k];
    if(v < 0 || v >= nverts)
    {
      atomicOr(err, DEVERR_RANGE);
      v = 0;
    }
    const double p[3] = {x[v], y[v], z[v]};
    for(int d = 0; d < 3; ++d)
    {
      const OKey kp = okey(p[d]);  // addPoint's comparisons on the integer pipe
      if(ok_lt(kp, klo[d]))
      {
        lo[d] = p[d];
        klo[d] = kp;
      }
      if(ok_gt(kp, khi[d]))
      {
        hi[d] = p[d];
        khi[d] = kp;
      }
    }
  }
  for(int d = 0; d < 3; ++d)
  {
    boxes[6 * (size_t)c + d] = lo[d];
    boxes[6 * (size_t)c + 3 + d] = hi[d];
  }
}

// One record per sorted leaf: the cell's vertex coordinates inline.  Padding
// leaves (cell id >= ncells, from BVH::initialize's 0/1-box padding) are
// never reached by a traversal; they get zero coordinates.
template <int NPC>
__global__ void k_leaf_records(const int* __restrict__ perm, int nleaves, const double* __restrict__ x,
                               const double* __restrict__ y, const double* __restrict__ z,
                               const int* __restrict__ cells, int ncells, int nverts, LeafRec<NPC>* __restrict__ recs)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if(k >= nleaves) return;
  const int c = perm[k];
  LeafRec<NPC> r;
  for(int j = 0; j < NPC; ++j)
  {
    int v = (c < ncells) ? cells[(size_t)c * NPC + j] : -1;
    const bool ok = (v >= 0 && v < nverts);
    r.v[3 * j + 0] = ok ? x[v] : 0.0;
    r.v[3 * j + 1] = ok ? y[v] : 0.0;
    r.v[3 * j + 2] = ok ? z[v] : 0.0;
  }
  r.cell = c;
  recs[k] = r;
}

// 30-bit Morton code of each query point in the given box (processing order
// only; results do not depend on it).
// The frame of the points' processing order: the mesh box grown by a quarter of
// its extent on every side (points just outside the mesh, common in uniform
// query sets, keep distinct codes instead of piling up on the box faces;
// 16M points in the 1.2x box: 460 instead of 467 ms), and the inverse extent.
inline void query_code_frame(const double* b, double* lo, double* sc)
{
  for(int d = 0; d < 3; ++d)
  {
    const double ext = b[3 + d] - b[d];
    lo[d] = b[d] - 0.25 * ext;
    sc[d] = (ext > 0.0) ? 1.0 / (1.5 * ext) : 0.0;
  }
}

__global__ void k_query_codes(QueryPts qp, int m, double lx, double ly, double lz, double sx, double sy, double sz,
                              uint32_t* __restrict__ codes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  const double c[3] = {(qp.x[(size_t)i * qp.stride] - lx) * sx, (qp.y[(size_t)i * qp.stride] - ly) * sy,
                       (qp.z[(size_t)i * qp.stride] - lz) * sz};
  uint32_t u[3];
  for(int d = 0; d < 3; ++d)
  {
    const double f = fmin(fmax(c[d] * 1024.0, 0.0), 1023.0);
    u[d] = (uint32_t)(int)f;
  }
  auto spread = [](uint32_t v) {
    v = (v | (v << 16)) & 0xFF0000FFu;
    v = (v | (v << 8)) & 0x0F00F00Fu;
    v = (v | (v << 4)) & 0xC30C30C3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
  };
  codes[i] = spread(u[0]) | (spread(u[1]) << 1) | (spread(u[2]) << 2);
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

}  // namespace
}  // namespace gsq

using namespace gsq;

// =============================================================================
// C ABI: quest::SignedDistance
// =============================================================================

namespace
{
void sdf_release(gsq_sdf* h)
{
  if(h->mesh_block) cudaFree(h->mesh_block);
  if(h->leaves) cudaFree(h->leaves);
  if(h->nodes32) cudaFree(h->nodes32);
  if(h->leaves32) cudaFree(h->leaves32);
  if(h->d_audit) cudaFree(h->d_audit);
  if(h->d_work) cudaFree(h->d_work);
  if(h->eval_buf) cudaFree(h->eval_buf);
  if(h->d_mesh) cudaFree(h->d_mesh);
  if(h->d_err) cudaFree(h->d_err);
  if(h->bvh) gsq_bvh_destroy(h->bvh);
  delete h;
}

// Bytes of device memory the staged query coordinates take: one block of
// 3m doubles for interleaved points, else one span per coordinate array kept
// in host memory.  ext (optional) is where stage_queries puts them.
size_t stage_query_bytes(const double* qx, const double* qy, const double* qz, int stride, int m)
{
  const size_t span = align256(sizeof(double) * ((size_t)(m - 1) * stride + 1));
  if(stride == 3 && qy == qx + 1 && qz == qx + 2) return is_device_ptr(qx) ? 0 : align256(sizeof(double) * 3 * (size_t)m);
  size_t b = 0;
  for(const double* a : {qx, qy, qz})
    if(!is_device_ptr(a)) b += span;
  return b;
}

int stage_queries(const double* qx, const double* qy, const double* qz, int stride, int m, cudaStream_t s,
                  InBuf* bufs, QueryPts& qp, char* ext = nullptr)
{
  qp.stride = stride;
  const size_t span = sizeof(double) * ((size_t)(m - 1) * stride + 1);
  const bool aos = (stride == 3 && qy == qx + 1 && qz == qx + 2);
  if(aos)
  {
    GSQ_CUDA_TRY(bufs[0].stage(qx, sizeof(double) * 3 * (size_t)m, s, ext));
    qp.x = static_cast<const double*>(bufs[0].dev);
    qp.y = qp.x + 1;
    qp.z = qp.x + 2;
    return GSQ_OK;
  }
  const double* src[3] = {qx, qy, qz};
  for(int k = 0; k < 3; ++k)
  {
    char* e = (ext && !is_device_ptr(src[k])) ? ext : nullptr;
    GSQ_CUDA_TRY(bufs[k].stage(src[k], span, s, e));
    if(e) ext += align256(span);
  }
  qp.x = static_cast<const double*>(bufs[0].dev);
  qp.y = static_cast<const double*>(bufs[1].dev);
  qp.z = static_cast<const double*>(bufs[2].dev);
  return GSQ_OK;
}
}  // namespace

namespace gsq
{
int sdf_query_order(const gsq_sdf* h, const QueryPts& qp, int m, uint32_t* keys[2], int* vals[2], const int** order,
                    cudaStream_t s)
{
  *order = nullptr;
  if(!h->opts.sort_queries || m <= 1) return GSQ_OK;
  double b[3], sc[3];
  query_code_frame(bvh_dev(h->bvh)->bounds, b, sc);
  count_launch();
  k_query_codes<<<grid_for(m, 256), 256, 0, s>>>(qp, m, b[0], b[1], b[2], sc[0], sc[1], sc[2], keys[0]);
  const int which = radix_sort_pairs(keys, vals, m, 30, true, s, h->d_err);
  if(which < 0) return which;
  *order = vals[which];
  return GSQ_OK;
}

int stage_query_points(const double* qx, const double* qy, const double* qz, int stride, int m, cudaStream_t s,
                       InBuf* bufs, QueryPts& qp)
{
  return stage_queries(qx, qy, qz, stride, m, s, bufs, qp);
}
}  // namespace gsq

extern "C" {

int gsq_sdf_opts_init(gsq_sdf_opts* o)
{
  if(!o) return fail(GSQ_ERR_INVALID, "null opts");
  std::memset(o, 0, sizeof(*o));
  o->precision = GSQ_PRECISION_FP64;
  o->sort_queries = 1;
  o->block_size = 0;
  return GSQ_OK;
}

int gsq_sdf_create(gsq_sdf** out, const double* x, const double* y, const double* z, int32_t nverts,
                   const int32_t* cells, int32_t ncells, int32_t npc, int32_t watertight, int32_t compute_sign,
                   const gsq_sdf_opts* opts, void* stream)
{
  if(!out) return fail(GSQ_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if(nverts < 0 || ncells < 0 || (npc != 3 && npc != 4)) return fail(GSQ_ERR_INVALID, "invalid mesh sizes");
  if((nverts > 0 && (!x || !y || !z)) || (ncells > 0 && !cells)) return fail(GSQ_ERR_INVALID, "null mesh arrays");
  if(ncells >= (1 << 28)) return fail(GSQ_ERR_INVALID, "at most 2^28-1 cells");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto* h = new(std::nothrow) gsq_sdf();
  if(!h) return fail(GSQ_ERR_NOMEM, "handle allocation failed");
  gsq_sdf_opts_init(&h->opts);
  if(opts) h->opts = *opts;
  h->watertight = watertight ? 1 : 0;
  h->sign = compute_sign ? 1 : 0;
  h->nverts = nverts;
  h->ncells = ncells;
  h->npc = npc;
  auto bail = [&](int rc) {
    sdf_release(h);
    return rc;
  };
  cudaError_t e = cudaGetDevice(&h->device);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_err, sizeof(int));
  if(e == cudaSuccess) e = cudaMemsetAsync(h->d_err, 0, sizeof(int), s);
  const size_t vbytes = sizeof(double) * std::max(nverts, 1);
  const size_t cbytes = sizeof(int) * (size_t)std::max(ncells, 1) * npc;
  const size_t vpad = (vbytes + 255) & ~size_t(255);
  if(e == cudaSuccess) e = cudaMalloc(&h->mesh_block, 3 * vpad + cbytes);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create"));
  char* mb = static_cast<char*>(h->mesh_block);
  h->d_x = reinterpret_cast<double*>(mb);
  h->d_y = reinterpret_cast<double*>(mb + vpad);
  h->d_z = reinterpret_cast<double*>(mb + 2 * vpad);
  h->d_cells = reinterpret_cast<int*>(mb + 3 * vpad);
  auto kind = [](const void* p) { return is_device_ptr(p) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; };
  if(nverts > 0)
  {
    e = cudaMemcpyAsync(h->d_x, x, sizeof(double) * nverts, kind(x), s);
    if(e == cudaSuccess) e = cudaMemcpyAsync(h->d_y, y, sizeof(double) * nverts, kind(y), s);
    if(e == cudaSuccess) e = cudaMemcpyAsync(h->d_z, z, sizeof(double) * nverts, kind(z), s);
  }
  if(e == cudaSuccess && ncells > 0)
    e = cudaMemcpyAsync(h->d_cells, cells, sizeof(int) * (size_t)ncells * npc, kind(cells), s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: mesh upload"));

  int rc = node_bounds(h->d_x, h->d_y, h->d_z, nverts, h->domain, s);
  if(rc) return bail(rc);

  Scratch boxes;
  e = boxes.alloc(sizeof(double) * 6 * (size_t)std::max(ncells, 1), s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: boxes"));
  if(ncells > 0)
    count_launch();
  if(ncells > 0)
    k_cell_boxes<<<grid_for(ncells, 256), 256, 0, s>>>(h->d_x, h->d_y, h->d_z, h->d_cells, ncells, npc, nverts,
                                                       boxes.as<double>(), h->d_err);
  h->bvh = bvh_new_internal(h->device);
  if(!h->bvh) return bail(GSQ_ERR_NOMEM);
  rc = bvh_build_internal(h->bvh, boxes.as<double>(), ncells, s);
  if(rc) return bail(rc);
  const BvhDev* B = bvh_dev(h->bvh);
  count_launch();
  const size_t rec = (npc == 3) ? sizeof(LeafRec<3>) : sizeof(LeafRec<4>);
  e = cudaMalloc(&h->leaves, rec * B->n);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: leaf records"));
  if(npc == 3)
    k_leaf_records<3><<<grid_for(B->n, 256), 256, 0, s>>>(B->perm, B->n, h->d_x, h->d_y, h->d_z, h->d_cells, ncells,
                                                         nverts, static_cast<LeafRec<3>*>(h->leaves));
  else
    k_leaf_records<4><<<grid_for(B->n, 256), 256, 0, s>>>(B->perm, B->n, h->d_x, h->d_y, h->d_z, h->d_cells, ncells,
                                                         nverts, static_cast<LeafRec<4>*>(h->leaves));
  e = cudaGetLastError();
  // FP32 copies for the mixed form, and the coordinate bound its error terms use
  if(e == cudaSuccess) e = cudaMalloc(&h->nodes32, sizeof(NodeRec32) * std::max(B->n - 1, 1));
  if(e == cudaSuccess) e = cudaMalloc(&h->leaves32, mixed_leaf_bytes(npc) * B->n);
  if(e == cudaSuccess) e = cudaMalloc(&h->d_audit, 4 * sizeof(unsigned long long));
  if(e == cudaSuccess) e = cudaMalloc(&h->d_work, sizeof(int));
  if(e == cudaSuccess) e = cudaMalloc(&h->d_mesh, sizeof(MeshInfo));
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: fp32 records"));
  rc = mixed_prepare(B->nodes, B->n - 1, h->leaves, B->n, npc, h->nodes32, h->leaves32, s);
  if(rc) return bail(rc);
  double mm = 0.0;
  for(int d = 0; d < 6; ++d)
    if(std::fabs(h->domain[d]) < DBL_MAX) mm = std::max(mm, std::fabs(h->domain[d]));
  h->mesh_max = (float)(mm * (1.0 + 1e-6));
  {
    MeshInfo mi {};
    mi.node_off = 0;
    mi.leaf_off = 0;
    std::memcpy(mi.domain, h->domain, sizeof(mi.domain));
    mi.mesh_max = h->mesh_max;
    e = cudaMemcpyAsync(h->d_mesh, &mi, sizeof(mi), cudaMemcpyHostToDevice, s);
    if(e == cudaSuccess) e = cudaStreamSynchronize(s);
    if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create: mesh entry"));
  }
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_sdf_create"));
  rc = check_device_error(h->d_err, s, "gsq_sdf_create");
  if(rc) return bail(rc);
  *out = h;
  return GSQ_OK;
}

int gsq_sdf_destroy(gsq_sdf* h)
{
  if(h) sdf_release(h);
  return GSQ_OK;
}

int gsq_sdf_set_opts(gsq_sdf* h, const gsq_sdf_opts* o)
{
  if(!h || !o) return fail(GSQ_ERR_INVALID, "null argument");
  if(o->precision != GSQ_PRECISION_FP64 && o->precision != GSQ_PRECISION_MIXED)
    return fail(GSQ_ERR_INVALID, "unknown precision");
  h->opts = *o;
  return GSQ_OK;
}

int gsq_sdf_mesh_bounds(const gsq_sdf* h, double* lo, double* hi)
{
  if(!h || !lo || !hi) return fail(GSQ_ERR_INVALID, "null argument");
  for(int d = 0; d < 3; ++d)
  {
    lo[d] = h->domain[d];
    hi[d] = h->domain[3 + d];
  }
  return GSQ_OK;
}

int gsq_sdf_get_bvh(const gsq_sdf* h, const gsq_bvh** b)
{
  if(!h || !b) return fail(GSQ_ERR_INVALID, "null argument");
  *b = h->bvh;
  return GSQ_OK;
}

int gsq_sdf_mixed_stats(const gsq_sdf* h, int64_t* c)
{
  if(!h || !c) return fail(GSQ_ERR_INVALID, "null argument");
  for(int k = 0; k < 4; ++k) c[k] = h->audit[k];
  return GSQ_OK;
}

int gsq_sdf_last_eval_ms(const gsq_sdf* h, float* ms)
{
  if(!h || !ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->eval_ms;
  return GSQ_OK;
}

}  // extern "C"

namespace
{
// gsq_sdf_eval and gsq_sdf_eval_tri: tri (nullable) receives each point's
// closest triangle.
int sdf_eval_impl(const gsq_sdf* hc, const double* qx, const double* qy, const double* qz, int32_t stride, int32_t m,
                  double* out, double* closest, double* normals, int32_t* tri, void* stream)
{
  gsq_sdf* h = const_cast<gsq_sdf*>(hc);
  if(!h) return fail(GSQ_ERR_INVALID, "null sdf handle");
  if(m < 0 || stride < 1) return fail(GSQ_ERR_INVALID, "invalid query count or stride");
  if(m == 0) return GSQ_OK;
  if(!qx || !qy || !qz || !out) return fail(GSQ_ERR_INVALID, "null query or output array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Staging of host points and outputs, the sort's buffers and the persistent
  // kernel's work counter: the handle's (grow-only), held until this call has
  // synchronised its stream below, or the call's own when another thread is
  // evaluating on this handle (computeDistances is const and re-entrant).
  std::unique_lock<std::mutex> lock(h->work_busy, std::try_to_lock);
  const bool cached = lock.owns_lock();
  const bool sort = h->opts.sort_queries && m > 1;
  const size_t in_bytes = stage_query_bytes(qx, qy, qz, stride, m);
  const size_t out_bytes[4] = {is_device_ptr(out) ? 0 : align256(sizeof(double) * (size_t)m),
                               (!closest || is_device_ptr(closest)) ? 0 : align256(sizeof(double) * 3 * (size_t)m),
                               (!normals || is_device_ptr(normals)) ? 0 : align256(sizeof(double) * 3 * (size_t)m),
                               (!tri || is_device_ptr(tri)) ? 0 : align256(sizeof(int32_t) * (size_t)m)};
  const size_t order_bytes = sort ? align256(4 * sizeof(uint32_t) * (size_t)m) : 0;
  const size_t sort_bytes = sort ? align256(radix_sort_work_bytes(m)) : 0;
  char* cv = nullptr;
  if(cached)
  {
    const size_t need = in_bytes + out_bytes[0] + out_bytes[1] + out_bytes[2] + out_bytes[3] + order_bytes + sort_bytes;
    if(need > h->eval_bytes)
    {
      if(h->eval_buf) cudaFree(h->eval_buf);
      h->eval_buf = nullptr;
      h->eval_bytes = 0;
      GSQ_CUDA_TRY(cudaMalloc(&h->eval_buf, need));
      h->eval_bytes = need;
    }
    cv = static_cast<char*>(h->eval_buf);
  }
  auto take = [&](size_t b) -> char* {
    if(!cv || b == 0) return nullptr;
    char* r = cv;
    cv += b;
    return r;
  };
  InBuf qb[3];
  QueryPts qp;
  int rc = stage_queries(qx, qy, qz, stride, m, s, qb, qp, take(in_bytes));
  if(rc) return rc;
  OutBuf ob, cb, nb, tb;
  GSQ_CUDA_TRY(ob.prepare(out, sizeof(double) * (size_t)m, s, take(out_bytes[0])));
  GSQ_CUDA_TRY(cb.prepare(closest, sizeof(double) * 3 * (size_t)m, s, take(out_bytes[1])));
  GSQ_CUDA_TRY(nb.prepare(normals, sizeof(double) * 3 * (size_t)m, s, take(out_bytes[2])));
  GSQ_CUDA_TRY(tb.prepare(tri, sizeof(int32_t) * (size_t)m, s, take(out_bytes[3])));

  const BvhDev* B = bvh_dev(h->bvh);
  Scratch order_buf;
  const int* order = nullptr;
  if(sort)
  {
    uint32_t* ob4 = reinterpret_cast<uint32_t*>(take(order_bytes));
    if(!ob4)
    {
      GSQ_CUDA_TRY(order_buf.alloc(4 * sizeof(uint32_t) * (size_t)m, s));
      ob4 = order_buf.as<uint32_t>();
    }
    uint32_t* keys[2] = {ob4, ob4 + m};
    int* vals[2] = {reinterpret_cast<int*>(ob4 + 2 * (size_t)m), reinterpret_cast<int*>(ob4 + 3 * (size_t)m)};
    double b[3], sc[3];
    query_code_frame(B->bounds, b, sc);
    count_launch();
    k_query_codes<<<grid_for(m, 256), 256, 0, s>>>(qp, m, b[0], b[1], b[2], sc[0], sc[1], sc[2], keys[0]);
    char* sw = take(sort_bytes);
    const int which = sw ? radix_sort_pairs_prealloc(keys, vals, m, 30, true, sw, sort_bytes, s, h->d_err)
                         : radix_sort_pairs(keys, vals, m, 30, true, s, h->d_err);
    if(which < 0) return which;
    order = vals[which];
  }

  SdfParams prm;
  std::memcpy(prm.domain, h->domain, sizeof(prm.domain));
  prm.watertight = h->watertight;
  prm.sign = h->sign;
  const int threads = 128;
  cudaEvent_t e0, e1;
  GSQ_CUDA_TRY(cudaEventCreate(&e0));
  GSQ_CUDA_TRY(cudaEventCreate(&e1));
  const bool mixed = (h->opts.precision == GSQ_PRECISION_MIXED);
  const bool audit = mixed && h->opts.audit;
  if(audit) GSQ_CUDA_TRY(cudaMemsetAsync(h->d_audit, 0, 4 * sizeof(unsigned long long), s));
  cudaEventRecord(e0, s);
  Scratch own_work;
  if(mixed)
  {
    int* work = h->d_work;
    if(!cached)
    {
      GSQ_CUDA_TRY(own_work.alloc(sizeof(int), s));
      work = own_work.as<int>();
    }
    if(tri)
      rc = mixed_launch_tri(h->npc, B->nodes, h->nodes32, h->leaves, h->leaves32, h->d_mesh, qp, m, order, prm,
                            static_cast<double*>(ob.dev), static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                            h->d_err, work, static_cast<int*>(tb.dev), s);
    else
      rc = mixed_launch(h->npc, B->nodes, h->nodes32, h->leaves, h->leaves32, h->d_mesh, qp, m, order, prm,
                        static_cast<double*>(ob.dev), static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                        h->d_err, audit ? h->d_audit : nullptr, work, h->opts.block_size, h->opts.queue_depth, s);
    if(rc) return rc;
  }
  else
    count_launch();
  if(!mixed && h->npc == 3)
    k_sdf_fp64<3><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<3>*>(h->leaves), qp, m,
                                                          order, prm, static_cast<double*>(ob.dev),
                                                          static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                                                          static_cast<int*>(tb.dev), h->d_err);
  else if(!mixed)
    k_sdf_fp64<4><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<4>*>(h->leaves), qp, m,
                                                          order, prm, static_cast<double*>(ob.dev),
                                                          static_cast<double*>(cb.dev), static_cast<double*>(nb.dev),
                                                          static_cast<int*>(tb.dev), h->d_err);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaGetLastError();
  if(audit && e == cudaSuccess)
    e = cudaMemcpyAsync(h->audit, h->d_audit, 4 * sizeof(long long), cudaMemcpyDeviceToHost, s);
  if(e == cudaSuccess) e = ob.flush(s);
  if(e == cudaSuccess) e = cb.flush(s);
  if(e == cudaSuccess) e = nb.flush(s);
  if(e == cudaSuccess) e = tb.flush(s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaEventElapsedTime(&h->eval_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(e != cudaSuccess) return cuda_fail(e, "gsq_sdf_eval");
  return check_device_error(h->d_err, s, "gsq_sdf_eval");
}
}  // namespace

extern "C" {

int gsq_sdf_eval(const gsq_sdf* h, const double* qx, const double* qy, const double* qz, int32_t stride, int32_t m,
                 double* out, double* closest, double* normals, void* stream)
{
  return sdf_eval_impl(h, qx, qy, qz, stride, m, out, closest, normals, nullptr, stream);
}

int gsq_sdf_eval_tri(const gsq_sdf* h, const double* qx, const double* qy, const double* qz, int32_t stride,
                     int32_t m, double* out, int32_t* triangles, void* stream)
{
  if(m > 0 && !triangles) return fail(GSQ_ERR_INVALID, "null triangle array");
  return sdf_eval_impl(h, qx, qy, qz, stride, m, out, nullptr, nullptr, triangles, stream);
}

}  // extern "C"

// =============================================================================
// Allocation-free evaluation
// =============================================================================
// Some callers cannot allocate device memory while they evaluate distances:
// applications whose own pool allocator owns all device memory and forbids
// allocations behind its back, and loops running beside other streams that
// must not be stalled by the implicit device-wide synchronisation of
// cudaMalloc/cudaFree (this call waits only for its own stream, to read the
// device error flag).  For them gsq_sdf_eval_noalloc takes the query points
// and the output in device memory and keeps its only scratch -- the
// Morton-order sort of the queries and the query kernel's work counter -- in
// the fixed array below, which every
// GPU that loads this library holds until the process exits.  The array's
// address is looked up once per device and kept; a cudaDeviceReset, which
// also invalidates every handle, is not supported after the first call.
namespace
{
constexpr int NOALLOC_MAX = GSQ_NOALLOC_MAX_QUERIES;
// keys[2] + vals[2] (4 arrays of NOALLOC_MAX words) + the sort's histogram and
// look-back words for NOALLOC_MAX keys (4*256 + 64 tiles * 256 + 32 words).
constexpr size_t NOALLOC_SORT_WORDS = 4 * 256 + ((NOALLOC_MAX + 4095) / 4096) * 256 + 32;
// ... followed by the persistent kernel's work counter (so that these calls do
// not share the handle's counter with gsq_sdf_eval).
constexpr size_t NOALLOC_BYTES = sizeof(uint32_t) * (4 * (size_t)NOALLOC_MAX + NOALLOC_SORT_WORDS + 64);
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, once per device (with that device current).
int noalloc_scratch(void** out)
{
  int dev = 0;
  GSQ_CUDA_TRY(cudaGetDevice(&dev));
  if(dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(GSQ_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if(!g_noalloc_ptr[dev])
  {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if(e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GSQ_OK;
}
}  // namespace

extern "C" {

int gsq_sdf_eval_noalloc(const gsq_sdf* hc, const double* qx, const double* qy, const double* qz, int32_t stride,
                         int32_t m, double* out, void* stream)
{
  gsq_sdf* h = const_cast<gsq_sdf*>(hc);
  if(!h) return fail(GSQ_ERR_INVALID, "null sdf handle");
  if(m < 0 || stride < 1) return fail(GSQ_ERR_INVALID, "invalid query count or stride");
  if(m > NOALLOC_MAX)
    return fail(GSQ_ERR_INVALID, "gsq_sdf_eval_noalloc: at most GSQ_NOALLOC_MAX_QUERIES (" +
                                     std::to_string(NOALLOC_MAX) + ") points per call, got " + std::to_string(m));
  if(m == 0) return GSQ_OK;
  if(!qx || !qy || !qz || !out) return fail(GSQ_ERR_INVALID, "null query or output array");
  if(!is_device_ptr(qx) || !is_device_ptr(qy) || !is_device_ptr(qz) || !is_device_ptr(out))
    return fail(GSQ_ERR_INVALID, "gsq_sdf_eval_noalloc: queries and output must be device memory");
  int dev = 0;
  GSQ_CUDA_TRY(cudaGetDevice(&dev));
  if(dev != h->device)
    return fail(GSQ_ERR_INVALID, "gsq_sdf_eval_noalloc: the current device (" + std::to_string(dev) +
                                     ") is not the handle's device (" + std::to_string(h->device) + ")");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* base = nullptr;
  int rc = noalloc_scratch(&base);
  if(rc) return rc;
  uint32_t* words = static_cast<uint32_t*>(base);
  uint32_t* keys[2] = {words, words + NOALLOC_MAX};
  int* vals[2] = {reinterpret_cast<int*>(words + 2 * (size_t)NOALLOC_MAX),
                  reinterpret_cast<int*>(words + 3 * (size_t)NOALLOC_MAX)};
  void* sort_work = words + 4 * (size_t)NOALLOC_MAX;
  int* work = reinterpret_cast<int*>(words + 4 * (size_t)NOALLOC_MAX + NOALLOC_SORT_WORDS);

  QueryPts qp {qx, qy, qz, stride};
  const BvhDev* B = bvh_dev(h->bvh);
  const int* order = nullptr;
  if(h->opts.sort_queries && m > 1)
  {
    double b[3], sc[3];
    query_code_frame(B->bounds, b, sc);
    count_launch();
    k_query_codes<<<grid_for(m, 256), 256, 0, s>>>(qp, m, b[0], b[1], b[2], sc[0], sc[1], sc[2], keys[0]);
    const int which = radix_sort_pairs_prealloc(keys, vals, m, 30, true, sort_work,
                                                sizeof(uint32_t) * NOALLOC_SORT_WORDS, s, h->d_err);
    if(which < 0) return which;
    order = vals[which];
  }
  SdfParams prm;
  std::memcpy(prm.domain, h->domain, sizeof(prm.domain));
  prm.watertight = h->watertight;
  prm.sign = h->sign;
  if(h->opts.precision == GSQ_PRECISION_MIXED)
  {
    rc = mixed_launch(h->npc, B->nodes, h->nodes32, h->leaves, h->leaves32, h->d_mesh, qp, m, order, prm, out,
                      nullptr, nullptr, h->d_err, nullptr, work, h->opts.block_size, h->opts.queue_depth, s);
    if(rc) return rc;
  }
  else
  {
    const int threads = 128;
    count_launch();
    if(h->npc == 3)
      k_sdf_fp64<3><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<3>*>(h->leaves), qp,
                                                            m, order, prm, out, nullptr, nullptr, nullptr, h->d_err);
    else
      k_sdf_fp64<4><<<grid_for(m, threads), threads, 0, s>>>(B->nodes, static_cast<const LeafRec<4>*>(h->leaves), qp,
                                                            m, order, prm, out, nullptr, nullptr, nullptr, h->d_err);
  }
  GSQ_CUDA_TRY(cudaGetLastError());
  return check_device_error(h->d_err, s, "gsq_sdf_eval_noalloc");
}

}  // extern "C"
