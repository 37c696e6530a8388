// Batched signed distance: many meshes and point sets in one CUDA graph.
//
// Build (every kernel covers all meshes; mesh k owns cells [coff[k], coff[k+1]),
// inner nodes [coff[k]-k, coff[k+1]-k-1) and tree-node ids [2coff[k]-k, ...)):
//   k_b_leaf_boxes   cell boxes (getCellBoundingBox, quest/SignedDistance.hpp:608-633)
//                    scaled as BVH::initialize does (BoundingBox::scale)
//   k_b_mesh_bounds  one block per mesh: the mesh box (SD:483-486), the bounds
//                    and Morton parameters of its boxes (BR:102-163)
//   k_b_morton       Morton code of each cell in its mesh's bounds
//   two stable radix sorts: by code, then by mesh; within a mesh the order is
//                    (code, cell index), the single-tree sort's order
//   k_b_karras / k_b_refit_persist / k_b_leaf_records: the single-tree kernels' bodies
//                    on each mesh's slice with local indices
//   mixed_prepare    FP32 node and leaf records
// Query: each point's Morton code in its mesh's bounds, prefixed by the mesh
// id, one radix sort for the processing order, and one persistent launch of
// the mixed kernel over all points, each point using its mesh's records.
// Every per-mesh array therefore holds the bits a standalone build of that
// mesh holds, and the query is the standalone query.
#include "gsq_build.cuh"
#include "gsq_sdf_handle.cuh"
#include "gsq_sdf_mixed_kernel.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

namespace gsq
{
namespace
{
using namespace sdf;
constexpr int BT = 256;
constexpr int PARAMS = 18;  // per mesh: bounds[6], Morton min[3] inv_extent[3], root box[6]

// Last k in [0, n) with off[k] - k * sub <= i, for offsets ascending in k.
__device__ __forceinline__ int segment_of(const long long* __restrict__ off, int n, long long i, int sub = 0)
{
  int lo = 0, hi = n;
  while(hi - lo > 1)
  {
    const int mid = (lo + hi) >> 1;
    if(__ldg(off + mid) - (long long)sub * mid <= i)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(BT) k_b_leaf_boxes(const double* __restrict__ x, const double* __restrict__ y,
                                                     const double* __restrict__ z, const int* __restrict__ cells,
                                                     int npc, const long long* __restrict__ voff,
                                                     const long long* __restrict__ coff, int nm, int ncells,
                                                     double half, double* __restrict__ leafbox, int* err)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if(c >= ncells) return;
  const int k = segment_of(coff, nm, c);
  const long long v0 = voff[k];
  const long long nv = voff[k + 1] - v0;
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for(int j = 0; j < npc; ++j)
  {
    const int v = cells[(size_t)c * npc + j];
    const bool ok = (v >= 0 && v < nv);
    if(!ok) atomicOr(err, DEVERR_RANGE);
    const double p[3] = {ok ? x[v0 + v] : 0.0, ok ? y[v0 + v] : 0.0, ok ? z[v0 + v] : 0.0};
    for(int d = 0; d < 3; ++d)
    {
      if(p[d] < lo[d]) lo[d] = p[d];
      if(p[d] > hi[d]) hi[d] = p[d];
    }
  }
  lbvh::scale_box(lo, hi, half);
  for(int d = 0; d < 3; ++d)
  {
    leafbox[6 * (size_t)c + d] = lo[d];
    leafbox[6 * (size_t)c + 3 + d] = hi[d];
  }
}

// One block per mesh.  Indices in the folds are global (vertex or cell), which
// keeps each mesh's index order.
__global__ void __launch_bounds__(BT) k_b_mesh_bounds(const double* __restrict__ x, const double* __restrict__ y,
                                                      const double* __restrict__ z,
                                                      const long long* __restrict__ voff,
                                                      const long long* __restrict__ coff,
                                                      const double* __restrict__ leafbox, double* __restrict__ params,
                                                      MeshInfo* __restrict__ meshes)
{
  const int k = blockIdx.x;
  lbvh::Fold fv;
  lbvh::fold_init(fv);
  for(long long v = voff[k] + threadIdx.x; v < voff[k + 1]; v += blockDim.x)
  {
    const double p[3] = {x[v], y[v], z[v]};
    for(int d = 0; d < 3; ++d)
    {
      if(okey(p[d]).nan) continue;  // addPoint's comparisons are false for a NaN
      lbvh::take_min(fv.lo[d], lbvh::ArgV {p[d], (int)v});
      lbvh::take_max(fv.hi[d], lbvh::ArgV {p[d], (int)v});
    }
  }
  const lbvh::Fold dom = lbvh::fold_block(fv);
  lbvh::Fold fb;
  lbvh::fold_init(fb);
  const int c0 = (int)coff[k], c1 = (int)coff[k + 1];
  for(int c = c0 + threadIdx.x; c < c1; c += blockDim.x)
  {
    const double* b = leafbox + 6 * (size_t)c;
    if(box_valid(b, b + 3)) lbvh::fold_add_box(fb, b, b + 3, c);
  }
  const lbvh::Fold bb = lbvh::fold_block(fb);
  if(threadIdx.x != 0) return;
  double* pk = params + (size_t)PARAMS * k;
  lbvh::bounds_params(bb, leafbox, c1 - 1, pk);
  MeshInfo mi;
  mi.node_off = c0 - k;
  mi.leaf_off = c0;
  double mm = 0.0;
  for(int d = 0; d < 3; ++d)
  {
    mi.domain[d] = (dom.lo[d].i == INT_MAX) ? DBL_MAX : dom.lo[d].v;
    mi.domain[3 + d] = (dom.hi[d].i == INT_MAX) ? -DBL_MAX : dom.hi[d].v;
  }
  for(int d = 0; d < 6; ++d)
    if(fabs(mi.domain[d]) < DBL_MAX) mm = fmax(mm, fabs(mi.domain[d]));
  mi.mesh_max = (float)(mm * (1.0 + 1e-6));
  mi.pad = 0;
  meshes[k] = mi;
}

__global__ void __launch_bounds__(BT) k_b_morton(const double* __restrict__ leafbox, const long long* __restrict__ coff,
                                                 int nm, int ncells, const double* __restrict__ params,
                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ codes)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if(c >= ncells) return;
  const int k = segment_of(coff, nm, c);
  const uint32_t code = lbvh::box_morton(leafbox + 6 * (size_t)c, params + (size_t)PARAMS * k);
  keys[c] = code;
  codes[c] = code;
}

__global__ void __launch_bounds__(BT) k_b_mesh_keys(const int* __restrict__ ids, const long long* __restrict__ coff,
                                                    int nm, int ncells, uint32_t* __restrict__ keys)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= ncells) return;
  keys[i] = (uint32_t)segment_of(coff, nm, ids[i]);
}

__global__ void __launch_bounds__(BT) k_b_gather(const int* __restrict__ ids, const uint32_t* __restrict__ codes,
                                                 int ncells, int* __restrict__ perm, uint32_t* __restrict__ scodes)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= ncells) return;
  const int c = ids[i];
  perm[i] = c;
  scodes[i] = codes[c];
}

__global__ void __launch_bounds__(BT) k_b_karras(const uint32_t* __restrict__ scodes, const long long* __restrict__ coff,
                                                 int nm, int ninner, int* __restrict__ lchild, int* __restrict__ rchild,
                                                 int* __restrict__ parent, NodeRec64* __restrict__ nodes)
{
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if(g >= ninner) return;
  const int k = segment_of(coff, nm, g, 1);
  const long long c0 = coff[k];
  const int n = (int)(coff[k + 1] - c0);
  const long long io = c0 - k, po = 2 * c0 - k;
  lbvh::karras_node((int)(g - io), scodes + c0, n, lchild + io, rchild + io, parent + po, nodes + io);
}

// The segmented refit as a persistent loop (as the single-tree build's
// k_refit_persist): a lane takes the next cell of any mesh when its previous
// chain has ended and climbs that mesh's tree one level per iteration.
__global__ void __launch_bounds__(BT) k_b_refit_persist(const double* __restrict__ leafbox, const int* __restrict__ perm,
                                                        const long long* __restrict__ coff, int nm, int ncells,
                                                        const int* __restrict__ parent, int* __restrict__ counters,
                                                        NodeRec64* nodes, double* __restrict__ params,
                                                        int* __restrict__ work)
{
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  bool active = false, open = true;
  int pcode = 0;
  double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {0.0, 0.0, 0.0};
  const int* pa = parent;
  int* cn = counters;
  NodeRec64* nd = nodes;
  double* root = params;
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
        const int i = base + __popc(want & lt_mask);
        if(i < ncells)
        {
          const int k = segment_of(coff, nm, i);
          const long long c0 = coff[k];
          const int n = (int)(coff[k + 1] - c0);
          const long long io = c0 - k, po = 2 * c0 - k;
          pa = parent + po;
          cn = counters + io;
          nd = nodes + io;
          root = params + (size_t)PARAMS * k + 12;
          const int id = perm[i];
          for(int d = 0; d < 3; ++d)
          {
            lo[d] = leafbox[6 * (size_t)id + d];
            hi[d] = leafbox[6 * (size_t)id + 3 + d];
          }
          pcode = pa[(n - 1) + (int)(i - c0)];
          active = true;
        }
        else
          open = false;
      }
    }
    if(__ballot_sync(FULL, active || open) == 0) break;
    if(active) active = lbvh::refit_step(pcode, lo, hi, pa, cn, nd, root);
  }
}

template <int NPC>
__global__ void __launch_bounds__(BT) k_b_leaf_records(const int* __restrict__ perm, const long long* __restrict__ coff,
                                                       const long long* __restrict__ voff, int nm, int ncells,
                                                       const double* __restrict__ x, const double* __restrict__ y,
                                                       const double* __restrict__ z, const int* __restrict__ cells,
                                                       LeafRec<NPC>* __restrict__ recs)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= ncells) return;
  const int k = segment_of(coff, nm, i);
  const int c = perm[i];
  const long long v0 = voff[k], nv = voff[k + 1] - v0;
  LeafRec<NPC> r;
  for(int j = 0; j < NPC; ++j)
  {
    const int v = cells[(size_t)c * NPC + j];
    const bool ok = (v >= 0 && v < nv);
    r.v[3 * j + 0] = ok ? x[v0 + v] : 0.0;
    r.v[3 * j + 1] = ok ? y[v0 + v] : 0.0;
    r.v[3 * j + 2] = ok ? z[v0 + v] : 0.0;
  }
  r.cell = (int)(c - coff[k]);
  recs[i] = r;
}

// Depth of each leaf (edges to the root); the maximum over all trees.
__global__ void __launch_bounds__(BT) k_b_depth(const long long* __restrict__ coff, int nm, int ncells,
                                                const int* __restrict__ parent, int* __restrict__ max_depth)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= ncells) return;
  const int k = segment_of(coff, nm, i);
  const long long c0 = coff[k];
  const int n = (int)(coff[k + 1] - c0);
  const int* par = parent + (2 * c0 - k);
  int node = (n - 1) + (int)(i - c0);  // the leaf's tree-node id
  int d = 0;
  while(d < n)  // at most n - 1 edges in a tree of n leaves
  {
    const int p = par[node];
    if(p < 0) break;
    node = p >> 1;
    ++d;
  }
  atomicMax(max_depth, d);
}

// Processing-order key of each point: its mesh id above the top `bits` bits of
// its 30-bit Morton code in the mesh's bounds.
__global__ void __launch_bounds__(BT) k_b_point_keys(const double* __restrict__ q, int m,
                                                     const long long* __restrict__ qoff, int nm,
                                                     const double* __restrict__ params, int bits,
                                                     uint32_t* __restrict__ keys)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  const int k = segment_of(qoff, nm, i);
  const double* b = params + (size_t)PARAMS * k;
  uint32_t u[3];
  for(int d = 0; d < 3; ++d)
  {
    // the mesh's box grown by a quarter of its extent on every side (as the
    // single-mesh query orders its points)
    const double ext = b[3 + d] - b[d];
    const double sc = (ext > 0.0) ? 1.0 / (1.5 * ext) : 0.0;
    const double f = fmin(fmax((q[3 * (size_t)i + d] - (b[d] - 0.25 * ext)) * sc * 1024.0, 0.0), 1023.0);
    u[d] = (uint32_t)(int)f;
  }
  const uint32_t code = lbvh::spread10(u[0]) | (lbvh::spread10(u[1]) << 1) | (lbvh::spread10(u[2]) << 2);
  keys[i] = ((uint32_t)k << bits) | (code >> (30 - bits));
}

// A sample of the processing order: `chunks` runs of `len` consecutive
// positions spread evenly over the m positions.
__global__ void k_b_sample(const int* __restrict__ order, int m, int chunks, int len, int* __restrict__ out)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if(j >= chunks * len) return;
  const long long start = (long long)(j / len) * (m / chunks);
  out[j] = order[start + j % len];
}

inline int grid_for(long long n, int threads) { return (int)std::max<long long>(1, (n + threads - 1) / threads); }

int bits_for(long long v)  // bits to hold 0..v
{
  int b = 0;
  while(b < 62 && (1LL << b) <= v) ++b;
  return b;
}
}  // namespace
}  // namespace gsq

using namespace gsq;

struct gsq_batch
{
  int device = 0;
  int nm = 0, npc = 3, watertight = 1, sign = 1;
  long long nverts = 0, ncells = 0, ninner = 0, npoints = 0;
  gsq_batch_opts opts;
  bool have_vertices = false, have_points = false;
  int max_depth = -1;
  float last_ms = 0.f;

  void* block = nullptr;  // one allocation holding every array below
  double *x = nullptr, *y = nullptr, *z = nullptr;
  int* cells = nullptr;
  long long *voff = nullptr, *coff = nullptr, *qoff = nullptr;
  double* leafbox = nullptr;
  double* params = nullptr;
  MeshInfo* meshes = nullptr;
  uint32_t* codes = nullptr;
  uint32_t* keys[2] = {nullptr, nullptr};  // sort buffers, max(ncells, npoints)
  int* vals[2] = {nullptr, nullptr};
  void* sort_work = nullptr;
  size_t sort_bytes = 0;
  uint32_t* scodes = nullptr;
  int* perm = nullptr;
  int *parent = nullptr, *lchild = nullptr, *rchild = nullptr, *counters = nullptr;
  NodeRec64* nodes = nullptr;
  NodeRec32* nodes32 = nullptr;
  void* leaves = nullptr;
  void* leaves32 = nullptr;
  double* q = nullptr;
  double* out = nullptr;
  double* cp = nullptr;
  int* work = nullptr;
  int* err = nullptr;
  int* depth = nullptr;

  cudaStream_t cs = nullptr;  // capture stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_kernels = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};

namespace
{
void drop_graph(gsq_batch* h)
{
  if(h->exec) cudaGraphExecDestroy(h->exec);
  if(h->graph) cudaGraphDestroy(h->graph);
  h->exec = nullptr;
  h->graph = nullptr;
  h->graph_kernels = 0;
}

void batch_release(gsq_batch* h)
{
  drop_graph(h);
  if(h->e0) cudaEventDestroy(h->e0);
  if(h->e1) cudaEventDestroy(h->e1);
  if(h->cs) cudaStreamDestroy(h->cs);
  if(h->block) cudaFree(h->block);
  delete h;
}

int morton_bits_max(const gsq_batch* h) { return std::min(30, 32 - bits_for(h->nm - 1)); }

// Options with defaults filled in and values checked.
int normalise_opts(const gsq_batch* h, gsq_batch_opts& o)
{
  if(o.block_size == 0) o.block_size = 128;
  if(o.block_size < 32 || o.block_size > 128 || o.block_size % 32)
    return fail(GSQ_ERR_INVALID, "block_size must be 32, 64, 96 or 128");
  if(o.queue_depth == 0) o.queue_depth = 4;
  if(o.queue_depth != 1 && o.queue_depth != 4 && o.queue_depth != 16)
    return fail(GSQ_ERR_INVALID, "queue_depth must be 1, 4 or 16");
  if(o.stack_depth == 0) o.stack_depth = STACK_SIZE;
  if(o.stack_depth != 32 && o.stack_depth != 64) return fail(GSQ_ERR_INVALID, "stack_depth must be 32 or 64");
  const int mb = morton_bits_max(h);
  if(o.morton_bits == 0) o.morton_bits = mb;
  if(o.morton_bits < 1 || o.morton_bits > mb)
    return fail(GSQ_ERR_INVALID, "morton_bits must be 1.." + std::to_string(mb) + " for this many meshes");
  if(o.leaf_size == 0) o.leaf_size = 1;
  if(o.leaf_size != 1)
    return fail(GSQ_ERR_INVALID,
                "leaf_size must be 1: the reference's trees hold one box per leaf, and larger leaves change "
                "which triangles are examined (and so the pseudo-normal sums)");
  return GSQ_OK;
}

// The build of every tree, on stream s.
int enqueue_build(gsq_batch* h, cudaStream_t s)
{
  const int C = (int)h->ncells, nm = h->nm;
  k_b_leaf_boxes<<<grid_for(C, BT), BT, 0, s>>>(h->x, h->y, h->z, h->cells, h->npc, h->voff, h->coff, nm, C,
                                                DEFAULT_SCALE * 0.5, h->leafbox, h->err);
  k_b_mesh_bounds<<<nm, BT, 0, s>>>(h->x, h->y, h->z, h->voff, h->coff, h->leafbox, h->params, h->meshes);
  k_b_morton<<<grid_for(C, BT), BT, 0, s>>>(h->leafbox, h->coff, nm, C, h->params, h->keys[0], h->codes);
  count_launch(3);
  GSQ_CUDA_TRY(cudaGetLastError());
  const int w1 = radix_sort_pairs_prealloc(h->keys, h->vals, C, 30, true, h->sort_work, h->sort_bytes, s, h->err);
  if(w1 < 0) return w1;
  uint32_t* k2[2] = {h->keys[w1 ^ 1], h->keys[w1]};
  int* v2[2] = {h->vals[w1], h->vals[w1 ^ 1]};
  k_b_mesh_keys<<<grid_for(C, BT), BT, 0, s>>>(v2[0], h->coff, nm, C, k2[0]);
  count_launch();
  const int w2 = radix_sort_pairs_prealloc(k2, v2, C, std::max(1, bits_for(nm - 1)), false, h->sort_work,
                                           h->sort_bytes, s, h->err);
  if(w2 < 0) return w2;
  k_b_gather<<<grid_for(C, BT), BT, 0, s>>>(v2[w2], h->codes, C, h->perm, h->scodes);
  k_b_karras<<<grid_for(h->ninner, BT), BT, 0, s>>>(h->scodes, h->coff, nm, (int)h->ninner, h->lchild, h->rchild,
                                                    h->parent, h->nodes);
  GSQ_CUDA_TRY(cudaMemsetAsync(h->counters, 0, sizeof(int) * (h->ninner + 1), s));
  int dev = 0, sms = 0, per_sm = 0;
  GSQ_CUDA_TRY(cudaGetDevice(&dev));
  GSQ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  GSQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_b_refit_persist, BT, 0));
  const int rgrid = std::max(1, std::min(sms * std::max(per_sm, 1), grid_for(C, BT)));
  k_b_refit_persist<<<rgrid, BT, 0, s>>>(h->leafbox, h->perm, h->coff, nm, C, h->parent, h->counters, h->nodes,
                                         h->params, h->counters + h->ninner);
  if(h->npc == 3)
    k_b_leaf_records<3><<<grid_for(C, BT), BT, 0, s>>>(h->perm, h->coff, h->voff, nm, C, h->x, h->y, h->z, h->cells,
                                                       static_cast<LeafRec<3>*>(h->leaves));
  else
    k_b_leaf_records<4><<<grid_for(C, BT), BT, 0, s>>>(h->perm, h->coff, h->voff, nm, C, h->x, h->y, h->z, h->cells,
                                                       static_cast<LeafRec<4>*>(h->leaves));
  count_launch(4);
  GSQ_CUDA_TRY(cudaGetLastError());
  return mixed_prepare(h->nodes, (int)h->ninner, h->leaves, C, h->npc, h->nodes32, h->leaves32, s);
}

// The processing order of the points for the given Morton width.
int enqueue_order(gsq_batch* h, int bits, const int** order, cudaStream_t s)
{
  const int m = (int)h->npoints;
  k_b_point_keys<<<grid_for(m, BT), BT, 0, s>>>(h->q, m, h->qoff, h->nm, h->params, bits, h->keys[0]);
  count_launch();
  GSQ_CUDA_TRY(cudaGetLastError());
  const int w = radix_sort_pairs_prealloc(h->keys, h->vals, m, bits + bits_for(h->nm - 1), true, h->sort_work,
                                          h->sort_bytes, s, h->err);
  if(w < 0) return w;
  *order = h->vals[w];
  return GSQ_OK;
}

int enqueue_query(gsq_batch* h, const gsq_batch_opts& o, const int* order, int m, cudaStream_t s)
{
  SdfParams prm;
  for(int d = 0; d < 6; ++d) prm.domain[d] = 0.0;  // per mesh, from the mesh table
  prm.watertight = h->watertight;
  prm.sign = h->sign;
  QueryPts qp {h->q, h->q + 1, h->q + 2, 3};
  GSQ_CUDA_TRY(cudaMemsetAsync(h->work, 0, sizeof(int), s));
  auto go = [&](auto npc_c, auto depth_c, auto stack_c) {
    return launch_mixed<decltype(npc_c)::value, false, decltype(depth_c)::value, decltype(stack_c)::value, true>(
        o.block_size, s, h->nodes, h->nodes32, h->leaves, h->leaves32, h->meshes, h->nm, h->qoff, qp, m, order, prm,
        h->out, h->cp, nullptr, h->err, MixedStats {nullptr}, h->work);
  };
  auto by_stack = [&](auto npc_c, auto depth_c) {
    return o.stack_depth == 32 ? go(npc_c, depth_c, std::integral_constant<int, 32> {})
                               : go(npc_c, depth_c, std::integral_constant<int, STACK_SIZE> {});
  };
  auto by_depth = [&](auto npc_c) {
    if(o.queue_depth == 16) return by_stack(npc_c, std::integral_constant<int, 16> {});
    if(o.queue_depth == 1) return by_stack(npc_c, std::integral_constant<int, 1> {});
    return by_stack(npc_c, std::integral_constant<int, 4> {});
  };
  const cudaError_t e = (h->npc == 3) ? by_depth(std::integral_constant<int, 3> {})
                                      : by_depth(std::integral_constant<int, 4> {});
  count_launch();
  GSQ_CUDA_TRY(e);
  return GSQ_OK;
}

int enqueue_step(gsq_batch* h, cudaStream_t s)
{
  int rc = enqueue_build(h, s);
  if(rc) return rc;
  if(h->npoints == 0) return GSQ_OK;
  const int* order = nullptr;
  rc = enqueue_order(h, h->opts.morton_bits, &order, s);
  if(rc) return rc;
  return enqueue_query(h, h->opts, order, (int)h->npoints, s);
}

// Captures one step into a graph on the batch's own stream.
int capture(gsq_batch* h)
{
  drop_graph(h);
  const int64_t before = gsq_kernel_launches();
  GSQ_CUDA_TRY(cudaStreamBeginCapture(h->cs, cudaStreamCaptureModeRelaxed));
  const int rc = enqueue_step(h, h->cs);
  cudaGraph_t g = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(h->cs, &g);
  count_launch(-(int)(gsq_kernel_launches() - before));  // counted when the graph runs
  if(rc)
  {
    if(g) cudaGraphDestroy(g);
    return rc;
  }
  if(ec != cudaSuccess) return cuda_fail(ec, "gsq_batch: graph capture");
  h->graph = g;
  cudaError_t e = cudaGraphInstantiate(&h->exec, g, 0);
  if(e != cudaSuccess)
  {
    drop_graph(h);
    return cuda_fail(e, "gsq_batch: graph instantiation");
  }
  size_t n = 0;
  e = cudaGraphGetNodes(g, nullptr, &n);
  std::vector<cudaGraphNode_t> nodes(n);
  if(e == cudaSuccess && n) e = cudaGraphGetNodes(g, nodes.data(), &n);
  if(e != cudaSuccess) return cuda_fail(e, "gsq_batch: graph nodes");
  int kernels = 0;
  for(auto nd : nodes)
  {
    cudaGraphNodeType t;
    if(cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
  }
  h->graph_kernels = kernels;
  return GSQ_OK;
}

bool valid_offsets(const int64_t* off, int n, bool strict2)
{
  if(off[0] != 0) return false;
  for(int k = 0; k < n; ++k)
    if(off[k + 1] - off[k] < (strict2 ? 2 : 0)) return false;
  return true;
}

int copy_out(void* dst, const void* src, size_t bytes, cudaStream_t s)
{
  if(!dst || !bytes) return GSQ_OK;
  GSQ_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
  return GSQ_OK;
}

int check_batch(const gsq_batch* h)
{
  if(!h) return fail(GSQ_ERR_INVALID, "null batch handle");
  return GSQ_OK;
}
}  // namespace

extern "C" {

int gsq_batch_opts_init(gsq_batch_opts* o)
{
  if(!o) return fail(GSQ_ERR_INVALID, "null opts");
  std::memset(o, 0, sizeof(*o));
  return GSQ_OK;
}

int gsq_batch_create(gsq_batch** out, int32_t nmeshes, const int64_t* vert_offsets, const int64_t* cell_offsets,
                     const int32_t* cells, int32_t npc, const int64_t* query_offsets, int32_t watertight,
                     int32_t compute_sign, const gsq_batch_opts* opts, void* stream)
{
  if(!out) return fail(GSQ_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if(nmeshes < 1 || nmeshes > 65536) return fail(GSQ_ERR_INVALID, "nmeshes must be 1..65536");
  if(!vert_offsets || !cell_offsets || !query_offsets || !cells) return fail(GSQ_ERR_INVALID, "null array");
  if(npc != 3 && npc != 4) return fail(GSQ_ERR_INVALID, "nodes_per_cell must be 3 or 4");
  if(!valid_offsets(vert_offsets, nmeshes, false) || !valid_offsets(query_offsets, nmeshes, false))
    return fail(GSQ_ERR_INVALID, "offsets must start at 0 and not decrease");
  if(!valid_offsets(cell_offsets, nmeshes, true)) return fail(GSQ_ERR_INVALID, "every mesh needs at least 2 cells");
  for(int k = 0; k < nmeshes; ++k)
    if(cell_offsets[k + 1] - cell_offsets[k] >= (1 << 28)) return fail(GSQ_ERR_INVALID, "at most 2^28-1 cells per mesh");
  const long long V = vert_offsets[nmeshes], Cn = cell_offsets[nmeshes], M = query_offsets[nmeshes];
  if(Cn >= (1LL << 30) || M >= (1LL << 30) || V >= (1LL << 31) - 1)
    return fail(GSQ_ERR_INVALID, "batch too large (cells and points < 2^30, vertices < 2^31)");
  auto* h = new(std::nothrow) gsq_batch();
  if(!h) return fail(GSQ_ERR_NOMEM, "handle allocation failed");
  h->nm = nmeshes;
  h->npc = npc;
  h->watertight = watertight ? 1 : 0;
  h->sign = compute_sign ? 1 : 0;
  h->nverts = V;
  h->ncells = Cn;
  h->ninner = Cn - nmeshes;
  h->npoints = M;
  gsq_batch_opts_init(&h->opts);
  if(opts) h->opts = *opts;
  h->opts.closest_points = (opts && opts->closest_points) ? 1 : 0;
  int rc = normalise_opts(h, h->opts);
  if(rc)
  {
    batch_release(h);
    return rc;
  }
  auto bail = [&](int code) {
    batch_release(h);
    return code;
  };
  cudaError_t e = cudaGetDevice(&h->device);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_batch_create"));

  // one allocation, carved into 256-byte aligned arrays
  const long long SM = std::max(Cn, M);
  h->sort_bytes = radix_sort_work_bytes((int)std::max<long long>(SM, 1));
  const size_t leaf_bytes = (npc == 3) ? sizeof(LeafRec<3>) : sizeof(LeafRec<4>);
  struct Part
  {
    void** p;
    size_t bytes;
  };
  const Part parts[] = {
      {(void**)&h->x, sizeof(double) * V},
      {(void**)&h->y, sizeof(double) * V},
      {(void**)&h->z, sizeof(double) * V},
      {(void**)&h->cells, sizeof(int) * Cn * npc},
      {(void**)&h->voff, sizeof(long long) * (nmeshes + 1)},
      {(void**)&h->coff, sizeof(long long) * (nmeshes + 1)},
      {(void**)&h->qoff, sizeof(long long) * (nmeshes + 1)},
      {(void**)&h->leafbox, sizeof(double) * 6 * Cn},
      {(void**)&h->params, sizeof(double) * PARAMS * nmeshes},
      {(void**)&h->meshes, sizeof(MeshInfo) * nmeshes},
      {(void**)&h->codes, sizeof(uint32_t) * Cn},
      {(void**)&h->keys[0], sizeof(uint32_t) * SM},
      {(void**)&h->keys[1], sizeof(uint32_t) * SM},
      {(void**)&h->vals[0], sizeof(int) * SM},
      {(void**)&h->vals[1], sizeof(int) * SM},
      {(void**)&h->sort_work, h->sort_bytes},
      {(void**)&h->scodes, sizeof(uint32_t) * Cn},
      {(void**)&h->perm, sizeof(int) * Cn},
      {(void**)&h->parent, sizeof(int) * (2 * Cn - nmeshes)},
      {(void**)&h->lchild, sizeof(int) * h->ninner},
      {(void**)&h->rchild, sizeof(int) * h->ninner},
      {(void**)&h->counters, sizeof(int) * (h->ninner + 1)},  // node counters, then the refit's work counter
      {(void**)&h->nodes, sizeof(NodeRec64) * h->ninner},
      {(void**)&h->nodes32, sizeof(NodeRec32) * h->ninner},
      {(void**)&h->leaves, leaf_bytes * Cn},
      {(void**)&h->leaves32, mixed_leaf_bytes(npc) * Cn},
      {(void**)&h->q, sizeof(double) * 3 * M},
      {(void**)&h->out, sizeof(double) * M},
      {(void**)&h->cp, h->opts.closest_points ? sizeof(double) * 3 * M : 0},
      {(void**)&h->work, sizeof(int)},
      {(void**)&h->err, sizeof(int)},
      {(void**)&h->depth, sizeof(int)},
  };
  auto align = [](size_t b) { return (b + 255) & ~size_t(255); };
  size_t total = 0;
  for(const Part& p : parts) total += align(std::max<size_t>(p.bytes, 1));
  e = cudaMalloc(&h->block, total);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_batch_create: device buffers"));
  char* b = static_cast<char*>(h->block);
  for(const Part& p : parts)
  {
    *p.p = p.bytes ? b : nullptr;
    b += align(std::max<size_t>(p.bytes, 1));
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaStreamCreateWithFlags(&h->cs, cudaStreamNonBlocking);
  if(e == cudaSuccess) e = cudaEventCreate(&h->e0);
  if(e == cudaSuccess) e = cudaEventCreate(&h->e1);
  if(e == cudaSuccess) e = cudaMemcpyAsync(h->cells, cells, sizeof(int) * Cn * npc, cudaMemcpyDefault, s);
  if(e == cudaSuccess)
    e = cudaMemcpyAsync(h->voff, vert_offsets, sizeof(long long) * (nmeshes + 1), cudaMemcpyDefault, s);
  if(e == cudaSuccess)
    e = cudaMemcpyAsync(h->coff, cell_offsets, sizeof(long long) * (nmeshes + 1), cudaMemcpyDefault, s);
  if(e == cudaSuccess)
    e = cudaMemcpyAsync(h->qoff, query_offsets, sizeof(long long) * (nmeshes + 1), cudaMemcpyDefault, s);
  if(e == cudaSuccess) e = cudaMemsetAsync(h->err, 0, sizeof(int), s);
  if(e == cudaSuccess) e = cudaStreamSynchronize(s);
  if(e != cudaSuccess) return bail(cuda_fail(e, "gsq_batch_create"));
  *out = h;
  return GSQ_OK;
}

int gsq_batch_destroy(gsq_batch* h)
{
  if(h) batch_release(h);
  return GSQ_OK;
}

int gsq_batch_set_vertices(gsq_batch* h, const double* x, const double* y, const double* z, void* stream)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(h->nverts && (!x || !y || !z)) return fail(GSQ_ERR_INVALID, "null coordinate array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t bytes = sizeof(double) * h->nverts;
  if(bytes)
  {
    GSQ_CUDA_TRY(cudaMemcpyAsync(h->x, x, bytes, cudaMemcpyDefault, s));
    GSQ_CUDA_TRY(cudaMemcpyAsync(h->y, y, bytes, cudaMemcpyDefault, s));
    GSQ_CUDA_TRY(cudaMemcpyAsync(h->z, z, bytes, cudaMemcpyDefault, s));
  }
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  h->have_vertices = true;
  return GSQ_OK;
}

int gsq_batch_set_points(gsq_batch* h, const double* pts, void* stream)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(h->npoints && !pts) return fail(GSQ_ERR_INVALID, "null point array");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if(h->npoints) GSQ_CUDA_TRY(cudaMemcpyAsync(h->q, pts, sizeof(double) * 3 * h->npoints, cudaMemcpyDefault, s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  h->have_points = true;
  return GSQ_OK;
}

int gsq_batch_run(gsq_batch* h, double* out, double* closest, void* stream)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!h->have_vertices || !h->have_points) return fail(GSQ_ERR_STATE, "set vertices and points before a run");
  if(closest && !h->cp) return fail(GSQ_ERR_INVALID, "closest points need opts.closest_points at creation");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for(int attempt = 0; attempt < 2; ++attempt)
  {
    if(!h->exec)
    {
      rc = capture(h);
      if(rc) return rc;
    }
    GSQ_CUDA_TRY(cudaEventRecord(h->e0, s));
    GSQ_CUDA_TRY(cudaGraphLaunch(h->exec, s));
    GSQ_CUDA_TRY(cudaEventRecord(h->e1, s));
    count_launch(h->graph_kernels);
    int flags = 0;
    GSQ_CUDA_TRY(cudaMemcpyAsync(&flags, h->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    GSQ_CUDA_TRY(cudaStreamSynchronize(s));
    if(flags == DEVERR_STACK && h->opts.stack_depth == 32 && attempt == 0)
    {
      // a tree grew deeper than the short stack allows: repeat with the reference's depth
      GSQ_CUDA_TRY(cudaMemsetAsync(h->err, 0, sizeof(int), s));
      h->opts.stack_depth = STACK_SIZE;
      drop_graph(h);
      continue;
    }
    rc = check_device_error(h->err, s, "gsq_batch_run");
    if(rc) return rc;
    break;
  }
  GSQ_CUDA_TRY(cudaEventElapsedTime(&h->last_ms, h->e0, h->e1));
  rc = copy_out(out, h->out, sizeof(double) * h->npoints, s);
  if(rc == GSQ_OK) rc = copy_out(closest, h->cp, sizeof(double) * 3 * h->npoints, s);
  if(rc) return rc;
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  return GSQ_OK;
}

int gsq_batch_device_output(const gsq_batch* h, const double** dist, const double** closest)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(dist) *dist = h->out;
  if(closest) *closest = h->cp;
  return GSQ_OK;
}

int gsq_batch_tune(gsq_batch* h, void* stream)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!h->have_vertices || !h->have_points) return fail(GSQ_ERR_STATE, "set vertices and points before tuning");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  rc = enqueue_build(h, s);
  if(rc) return rc;
  GSQ_CUDA_TRY(cudaMemsetAsync(h->depth, 0, sizeof(int), s));
  k_b_depth<<<grid_for(h->ncells, BT), BT, 0, s>>>(h->coff, h->nm, (int)h->ncells, h->parent, h->depth);
  count_launch();
  GSQ_CUDA_TRY(cudaGetLastError());
  GSQ_CUDA_TRY(cudaMemcpyAsync(&h->max_depth, h->depth, sizeof(int), cudaMemcpyDeviceToHost, s));
  rc = check_device_error(h->err, s, "gsq_batch_tune: build");
  if(rc) return rc;
  if(h->npoints == 0) return GSQ_OK;

  // a push at a node of depth d leaves d + 1 stack entries, so depth-32 stacks
  // serve trees whose deepest leaf is at depth <= 31
  std::vector<int> stacks = {STACK_SIZE};
  if(h->max_depth <= 31) stacks.insert(stacks.begin(), 32);
  const int mb_max = morton_bits_max(h), mesh_bits = bits_for(h->nm - 1);
  std::vector<int> widths;
  for(int total : {16, 24, 32})
  {
    const int w = std::min(mb_max, total - mesh_bits);
    if(w >= 1 && std::find(widths.begin(), widths.end(), w) == widths.end()) widths.push_back(w);
  }
  const int m = (int)h->npoints;
  const int chunks = (m >= (1 << 20)) ? 64 : 1;
  const int len = (m >= (1 << 20)) ? (1 << 20) / 64 : m;
  const int S = chunks * len;
  Scratch sample;
  GSQ_CUDA_TRY(sample.alloc(sizeof(int) * S, s));

  gsq_batch_opts best = h->opts;
  float best_ms = INFINITY;
  for(int w : widths)
  {
    const int* order = nullptr;
    GSQ_CUDA_TRY(cudaEventRecord(h->e0, s));
    rc = enqueue_order(h, w, &order, s);
    if(rc) return rc;
    GSQ_CUDA_TRY(cudaEventRecord(h->e1, s));
    GSQ_CUDA_TRY(cudaEventSynchronize(h->e1));
    float sort_ms = 0.f;
    GSQ_CUDA_TRY(cudaEventElapsedTime(&sort_ms, h->e0, h->e1));
    k_b_sample<<<grid_for(S, BT), BT, 0, s>>>(order, m, chunks, len, sample.as<int>());
    count_launch();
    GSQ_CUDA_TRY(cudaGetLastError());
    for(int block : {64, 128})
      for(int depth : {1, 4, 16})
        for(int stack : stacks)
        {
          gsq_batch_opts o = h->opts;
          o.block_size = block;
          o.queue_depth = depth;
          o.stack_depth = stack;
          o.morton_bits = w;
          float ms = 0.f;
          for(int rep = 0; rep < 2; ++rep)  // the second launch is timed
          {
            GSQ_CUDA_TRY(cudaEventRecord(h->e0, s));
            rc = enqueue_query(h, o, sample.as<int>(), S, s);
            if(rc) return rc;
            GSQ_CUDA_TRY(cudaEventRecord(h->e1, s));
            GSQ_CUDA_TRY(cudaEventSynchronize(h->e1));
            GSQ_CUDA_TRY(cudaEventElapsedTime(&ms, h->e0, h->e1));
          }
          rc = check_device_error(h->err, s, "gsq_batch_tune: query");
          if(rc) return rc;
          const float est = sort_ms + ms * (float)m / (float)S;
          if(est < best_ms)
          {
            best_ms = est;
            best = o;
          }
        }
  }
  h->opts = best;
  drop_graph(h);
  return GSQ_OK;
}

int gsq_batch_get_opts(const gsq_batch* h, gsq_batch_opts* o)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!o) return fail(GSQ_ERR_INVALID, "null opts");
  *o = h->opts;
  return GSQ_OK;
}

int gsq_batch_set_opts(gsq_batch* h, const gsq_batch_opts* o)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!o) return fail(GSQ_ERR_INVALID, "null opts");
  gsq_batch_opts n = *o;
  n.closest_points = h->opts.closest_points;
  rc = normalise_opts(h, n);
  if(rc) return rc;
  h->opts = n;
  drop_graph(h);
  return GSQ_OK;
}

int gsq_batch_last_ms(const gsq_batch* h, float* ms)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!ms) return fail(GSQ_ERR_INVALID, "null argument");
  *ms = h->last_ms;
  return GSQ_OK;
}

int gsq_batch_max_depth(const gsq_batch* h, int32_t* depth)
{
  int rc = check_batch(h);
  if(rc) return rc;
  if(!depth) return fail(GSQ_ERR_INVALID, "null argument");
  *depth = h->max_depth;
  return GSQ_OK;
}

}  // extern "C"
