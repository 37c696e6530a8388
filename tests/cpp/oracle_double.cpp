// Test double for the GPU entry points of libgsq.so, backed by the oracle
// (oracle/gsq_oracle.cpp, the reference's algorithm restated): the BVH
// (gsq_bvh_create / build / bounds / find_* / destroy and the scale and
// tolerance setters), the signed distance (gsq_sdf_opts_init, gsq_sdf_create,
// gsq_sdf_eval, gsq_sdf_mesh_bounds, gsq_sdf_destroy) and the closest object
// point (gsq_cpq_create / query / destroy), and the option and timer queries
// of the host mirrors.  Linked into an executable with
// -rdynamic, or preloaded, these definitions take the place of libgsq.so's own,
// so the host code above them (the quest interface in libgsq.so, the C++ shim
// include/gsq.hpp, the Python classes) runs on a machine without a GPU, over
// the same results the GPU path gives bit for bit.  Candidates are allocated
// with malloc, which gsq_free releases for host pointers.  Test infrastructure
// only.
#include <cfloat>
#include <cstring>
#include <vector>

#include "../../oracle/gsq_oracle.cpp"
#include "gsq.h"

extern "C" {

int gsq_sdf_opts_init(gsq_sdf_opts* o)
{
  if(!o) return GSQ_ERR_INVALID;
  std::memset(o, 0, sizeof(*o));
  return GSQ_OK;
}

int gsq_sdf_create(gsq_sdf** out, const double* x, const double* y, const double* z, int32_t nverts,
                   const int32_t* cells, int32_t ncells, int32_t nodes_per_cell, int32_t watertight,
                   int32_t compute_sign, const gsq_sdf_opts*, void*)
{
  if(!out || !x || !y || !z || !cells || nverts < 0 || ncells < 0) return GSQ_ERR_INVALID;
  *out = static_cast<gsq_sdf*>(
      orc_sdf_create(x, y, z, nverts, cells, ncells, nodes_per_cell, watertight, compute_sign));
  return GSQ_OK;
}

int gsq_sdf_destroy(gsq_sdf* h)
{
  if(h) orc_sdf_destroy(h);
  return GSQ_OK;
}

int gsq_sdf_eval(const gsq_sdf* h, const double* qx, const double* qy, const double* qz, int32_t stride, int32_t m,
                 double* out, double* closest, double* normals, void*)
{
  if(!h || m < 0 || stride < 1) return GSQ_ERR_INVALID;
  if(m == 0) return GSQ_OK;
  std::vector<double> q(3 * (size_t)m);
  for(int32_t i = 0; i < m; ++i)
  {
    q[3 * (size_t)i] = qx[(size_t)i * stride];
    q[3 * (size_t)i + 1] = qy[(size_t)i * stride];
    q[3 * (size_t)i + 2] = qz[(size_t)i * stride];
  }
  orc_sdf_eval(const_cast<gsq_sdf*>(h), q.data(), m, out, closest, normals, 1);
  return GSQ_OK;
}

int gsq_sdf_mesh_bounds(const gsq_sdf* h, double* lo, double* hi)
{
  if(!h || !lo || !hi) return GSQ_ERR_INVALID;
  double b[6];
  orc_sdf_mesh_bounds(const_cast<gsq_sdf*>(h), b);
  for(int d = 0; d < 3; ++d)
  {
    lo[d] = b[d];
    hi[d] = b[3 + d];
  }
  return GSQ_OK;
}

// ---- BVH -------------------------------------------------------------
struct gsq_bvh
{
  double scale = 1.000123;  // BVH.hpp:410
  double tol = DBL_EPSILON;  // the reference's default ray tolerance
  void* tree = nullptr;
};

int gsq_bvh_create(gsq_bvh** out)
{
  if(!out) return GSQ_ERR_INVALID;
  *out = new gsq_bvh();
  return GSQ_OK;
}

int gsq_bvh_destroy(gsq_bvh* b)
{
  if(b)
  {
    if(b->tree) orc_bvh_destroy(b->tree);
    delete b;
  }
  return GSQ_OK;
}

int gsq_bvh_set_scale_factor(gsq_bvh* b, double s)
{
  if(!b) return GSQ_ERR_INVALID;
  b->scale = s;
  return GSQ_OK;
}

int gsq_bvh_get_scale_factor(const gsq_bvh* b, double* s)
{
  if(!b || !s) return GSQ_ERR_INVALID;
  *s = b->scale;
  return GSQ_OK;
}

int gsq_bvh_set_tolerance(gsq_bvh* b, double t)
{
  if(!b) return GSQ_ERR_INVALID;
  b->tol = t;
  return GSQ_OK;
}

int gsq_bvh_get_tolerance(const gsq_bvh* b, double* t)
{
  if(!b || !t) return GSQ_ERR_INVALID;
  *t = b->tol;
  return GSQ_OK;
}

int gsq_bvh_build(gsq_bvh* b, const double* boxes, int32_t n, void*)
{
  if(!b || n < 0 || (n > 0 && !boxes)) return GSQ_ERR_INVALID;
  if(b->tree) orc_bvh_destroy(b->tree);
  b->tree = orc_bvh_create(boxes, n, b->scale);
  return GSQ_OK;
}

int gsq_bvh_bounds(const gsq_bvh* b, double* lo, double* hi)
{
  if(!b || !b->tree || !lo || !hi) return GSQ_ERR_INVALID;
  double o[6];
  orc_bvh_bounds(b->tree, o);
  for(int d = 0; d < 3; ++d) lo[d] = o[d], hi[d] = o[3 + d];
  return GSQ_OK;
}

static int csr_out(long long total, int* cand, int32_t** candidates, int64_t* tot)
{
  *candidates = cand;
  if(tot) *tot = total;
  return GSQ_OK;
}

int gsq_bvh_find_boxes(const gsq_bvh* b, const double* q, int32_t m, int32_t* off, int32_t* cnt, int32_t** cands,
                       int64_t* total, void*)
{
  if(!b || !b->tree || !off || !cnt || !cands) return GSQ_ERR_INVALID;
  int* c = nullptr;
  const long long t = orc_bvh_find_boxes(b->tree, q, m, off, cnt, &c);
  return csr_out(t, c, cands, total);
}

int gsq_bvh_find_points(const gsq_bvh* b, const double* p, int32_t m, int32_t* off, int32_t* cnt, int32_t** cands,
                        int64_t* total, void*)
{
  if(!b || !b->tree || !off || !cnt || !cands) return GSQ_ERR_INVALID;
  int* c = nullptr;
  const long long t = orc_bvh_find_points(b->tree, p, m, off, cnt, &c);
  return csr_out(t, c, cands, total);
}

int gsq_bvh_find_rays(const gsq_bvh* b, const double* o, const double* d, int32_t m, int32_t* off, int32_t* cnt,
                      int32_t** cands, int64_t* total, void*)
{
  if(!b || !b->tree || !off || !cnt || !cands) return GSQ_ERR_INVALID;
  int* c = nullptr;
  const long long t = orc_bvh_find_rays(b->tree, o, d, m, b->tol, off, cnt, &c);
  return csr_out(t, c, cands, total);
}

// ---- closest object point ----------------------------------------------
int gsq_cpq_create(gsq_cpq** out, const double* points, int32_t n, const int32_t* domain_ids, void*)
{
  if(!out || n < 0 || (n > 0 && !points)) return GSQ_ERR_INVALID;
  *out = static_cast<gsq_cpq*>(orc_cp_create(points, n, domain_ids));
  return GSQ_OK;
}

int gsq_cpq_destroy(gsq_cpq* h)
{
  if(h) orc_cp_destroy(h);
  return GSQ_OK;
}

int gsq_cpq_query(const gsq_cpq* h, const double* points, int32_t m, double sq_threshold, int32_t, int32_t* idx,
                  int32_t* dom, double* pos, double* dist, void*)
{
  if(!h || m < 0) return GSQ_ERR_INVALID;
  orc_cp_query(const_cast<gsq_cpq*>(h), points, m, sq_threshold, idx, dom, pos, dist, 1);
  return GSQ_OK;
}

// ---- options and timers the host mirrors query (no GPU work: zero time,
// no audit counters) -------------------------------------------------------
int gsq_sdf_set_opts(gsq_sdf* h, const gsq_sdf_opts* o) { return (h && o) ? GSQ_OK : GSQ_ERR_INVALID; }

int gsq_sdf_last_eval_ms(const gsq_sdf* h, float* ms)
{
  if(!h || !ms) return GSQ_ERR_INVALID;
  *ms = 0.f;
  return GSQ_OK;
}

int gsq_sdf_mixed_stats(const gsq_sdf* h, int64_t* c)
{
  if(!h || !c) return GSQ_ERR_INVALID;
  for(int k = 0; k < 4; ++k) c[k] = 0;
  return GSQ_OK;
}

int gsq_bvh_num_leaves(const gsq_bvh* b, int32_t* n)
{
  if(!b || !b->tree || !n) return GSQ_ERR_INVALID;
  *n = orc_bvh_size(b->tree);
  return GSQ_OK;
}

int gsq_bvh_last_build_ms(const gsq_bvh* b, float* ms)
{
  if(!b || !ms) return GSQ_ERR_INVALID;
  *ms = 0.f;
  return GSQ_OK;
}

int gsq_cpq_last_ms(const gsq_cpq* h, float* ms)
{
  if(!h || !ms) return GSQ_ERR_INVALID;
  *ms = 0.f;
  return GSQ_OK;
}

}  // extern "C"
