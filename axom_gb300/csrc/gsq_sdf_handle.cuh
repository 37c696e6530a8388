// The signed-distance handle and the interfaces between its translation
// units (gsq_sdf.cu: set-up and FP64 query; gsq_sdf_mixed.cu: mixed query;
// gsq_sdf_adjoint.cu: gradients).
#pragma once

#include "gsq_sdf_mixed.cuh"

#include <mutex>

using gsq::NodeRec32;
using gsq::NodeRec64;

struct gsq_sdf
{
  int device = 0;
  gsq_sdf_opts opts;
  int watertight = 1, sign = 1;
  int nverts = 0, ncells = 0, npc = 3;
  double* d_x = nullptr;  // device copies of the mesh (x, y, z, cells in one block)
  double* d_y = nullptr;
  double* d_z = nullptr;
  int* d_cells = nullptr;
  void* mesh_block = nullptr;
  double domain[6];
  gsq_bvh* bvh = nullptr;
  void* leaves = nullptr;
  NodeRec32* nodes32 = nullptr;  // mixed form: FP32 node records
  void* leaves32 = nullptr;      // mixed form: FP32 leaf records
  float mesh_max = 0.f;          // max |coordinate| of the mesh, rounded up
  unsigned long long* d_audit = nullptr;
  int* d_work = nullptr;          // work-queue counter of the persistent query kernel
  std::mutex work_busy;           // held by the evaluation using d_work and eval_buf
  void* eval_buf = nullptr;       // an evaluation's staging and sort scratch (grow-only)
  size_t eval_bytes = 0;
  gsq::MeshInfo* d_mesh = nullptr; // the single mesh's entry for the query kernel
  long long audit[4] = {0, 0, 0, 0};
  int* d_err = nullptr;
  float eval_ms = 0.f;
};

namespace gsq
{
size_t mixed_leaf_bytes(int npc);
int mixed_prepare(const NodeRec64* nodes64, int n_inner, const void* leaves64, int nleaves, int npc, NodeRec32* nodes32,
                  void* leaves32, cudaStream_t s);
// The persistent mixed query over one mesh (meshes[0]; its node box in prm).
int mixed_launch(int npc, const NodeRec64* nodes64, const NodeRec32* nodes32, const void* leaves64,
                 const void* leaves32, const MeshInfo* meshes, const sdf::QueryPts& qp, int m, const int* order,
                 const sdf::SdfParams& prm, double* out, double* out_cp, double* out_n, int* err,
                 unsigned long long* audit, int* work, int block, int depth, cudaStream_t s);
// The same query (128 threads, queue depth 4, no audit) also writing each
// point's closest triangle to tri (c, or 2c / 2c + 1 within quad cell c).
int mixed_launch_tri(int npc, const NodeRec64* nodes64, const NodeRec32* nodes32, const void* leaves64,
                     const void* leaves32, const MeshInfo* meshes, const sdf::QueryPts& qp, int m, const int* order,
                     const sdf::SdfParams& prm, double* out, double* out_cp, double* out_n, int* err, int* work,
                     int* tri, cudaStream_t s);
}  // namespace gsq

namespace gsq
{
const BvhDev* bvh_dev(const gsq_bvh* h);
// Morton order of the queries (sorted by the code of each point in the BVH
// bounds); keys/vals are 2 x m scratch each.  Returns the order array or null.
int sdf_query_order(const gsq_sdf* h, const sdf::QueryPts& qp, int m, uint32_t* keys[2], int* vals[2],
                    const int** order, cudaStream_t s);
// Stages (possibly host) query coordinates to the device, as gsq_sdf_eval does.
int stage_query_points(const double* qx, const double* qy, const double* qz, int stride, int m, cudaStream_t s,
                       InBuf* bufs, sdf::QueryPts& qp);
}  // namespace gsq
