// Test double for the GPU query under the quest C interface: gsq_sdf_opts_init,
// gsq_sdf_create, gsq_sdf_eval, gsq_sdf_mesh_bounds and gsq_sdf_destroy backed
// by the oracle (oracle/gsq_oracle.cpp, the reference's algorithm restated).
// Linked into an executable with -rdynamic, these definitions take the place
// of libgsq.so's own for the library's QUEST_signed_distance_* functions, so the
// interface's option handling, init, evaluate and finalize logic (gsq_quest.cu,
// as built into libgsq.so) runs on a machine without a GPU.  Test
// infrastructure only.
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

}  // extern "C"
