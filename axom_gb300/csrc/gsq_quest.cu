// The quest signed-distance C interface: the global query object of
// quest/interface/signed_distance.cpp and the shroud C layer over it
// (quest/interface/c_fortran/wrapQUEST.h:84-129), over gsq_sdf.  Host code.
//
// The reference keeps its options in a static struct (signed_distance.cpp:
// parameters_t) and the query in a static pointer; these do the same.  Like
// the reference's interface, this state is not thread-safe: one thread
// initialises, evaluates and finalises.
#include "gsq_internal.cuh"
#include "gsq_quest.h"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace
{
struct QuestParams
{
  int dimension = 3;
  bool verbose = false;
  bool closed = true;
  bool shared_memory = false;
  bool compute_sign = true;
  int allocator = -1;
  int exec_space = QUEST_SignedDistExec_CPU;
  int32_t precision = GSQ_PRECISION_MIXED;
};

QuestParams g_params;
gsq_sdf* g_query = nullptr;

// SLIC_ERROR: the reference logs and aborts
[[noreturn]] void quest_error(const std::string& msg)
{
  gsq::set_error(msg);
  std::fprintf(stderr, "[gsq] ERROR in the quest signed distance interface: %s\n", msg.c_str());
  std::fflush(stderr);
  std::abort();
}

// SLIC_WARNING: the reference logs and goes on
void quest_warning(const std::string& msg)
{
  std::fprintf(stderr, "[gsq] WARNING in the quest signed distance interface: %s\n", msg.c_str());
}

void require_not_initialized()
{
  if(g_query) quest_error("signed distance query already initialized; setting option has no effect!");
}

void require_initialized(const char* what)
{
  if(!g_query) quest_error(std::string("signed distance query must be initialized prior to calling ") + what);
}

// the query over a triangle mesh with the current options; 0 or -1
int create_query(const double* x, const double* y, const double* z, int32_t stride, int32_t nnodes,
                 const int32_t* tris, int32_t ntris)
{
  gsq_sdf_opts o;
  gsq_sdf_opts_init(&o);
  o.precision = g_params.precision;
  gsq_sdf* h = nullptr;
  int rc;
  if(stride == 1)
    rc = gsq_sdf_create(&h, x, y, z, nnodes, tris, ntris, 3, g_params.closed, g_params.compute_sign, &o, nullptr);
  else
  {
    // interleaved coordinates (the STL reader's) split into three arrays
    std::vector<double> sx(nnodes), sy(nnodes), sz(nnodes);
    for(int32_t i = 0; i < nnodes; ++i)
    {
      sx[i] = x[(size_t)stride * i];
      sy[i] = y[(size_t)stride * i];
      sz[i] = z[(size_t)stride * i];
    }
    rc = gsq_sdf_create(&h, sx.data(), sy.data(), sz.data(), nnodes, tris, ntris, 3, g_params.closed,
                        g_params.compute_sign, &o, nullptr);
  }
  if(rc != GSQ_OK)
  {
    quest_warning(std::string("creating the signed distance query failed: ") + gsq_last_error());
    return -1;
  }
  g_query = h;
  if(g_params.verbose)
    std::fprintf(stderr, "[gsq] signed distance query initialized: %d nodes, %d triangles, %s surface\n", nnodes,
                 ntris, g_params.closed ? "closed" : "open");
  return 0;
}
}  // namespace

extern "C" {

int QUEST_signed_distance_init_serial(const char* file)
{
  // signed_distance_init(file) (signed_distance.cpp:109-160)
  if(g_params.dimension != 3)
  {
    quest_warning("the SignedDistance Query is currently only supported in 3D");
    gsq::set_error("dimension is not 3");
    return -1;
  }
  if(g_query)
  {
    // read_stl_mesh refuses to overwrite the mesh of an initialized query
    // (QuestHelpers.cpp:293-298)
    quest_warning("supplied mesh pointer is not null!");
    gsq::set_error("signed distance query already initialized");
    return -1;
  }
  if(g_params.shared_memory)
    quest_warning("Shared memory requires MPI3 and building Axom with AXOM_USE_MPI3 set to ON");
  double* xyz = nullptr;
  int32_t* cells = nullptr;
  int32_t nn = 0, nc = 0;
  if(!file || gsq_stl_read(file, &xyz, &nn, &cells, &nc) != GSQ_OK)
  {
    const std::string why = gsq_last_error();
    quest_warning(std::string("reading mesh from [") + (file ? file : "") + "] failed!");
    gsq::set_error(why);
    return -1;
  }
  const int rc = create_query(xyz, xyz + 1, xyz + 2, 3, nn, cells, nc);
  gsq_free(xyz);
  gsq_free(cells);
  return rc;
}

int QUEST_signed_distance_init_serial_bufferify(char* file, int SHT_file_len)
{
  // shroud passes a Fortran CHARACTER buffer: blank padded, not terminated
  int n = (file && SHT_file_len > 0) ? SHT_file_len : 0;
  while(n > 0 && file[n - 1] == ' ') --n;
  const std::string name = n > 0 ? std::string(file, (size_t)n) : std::string();
  return QUEST_signed_distance_init_serial(name.c_str());
}

bool QUEST_signed_distance_initialized(void) { return g_query != nullptr; }

void QUEST_signed_distance_get_mesh_bounds(double* lo, double* hi)
{
  // signed_distance.cpp:251-260
  require_initialized("get_mesh_bounds()");
  if(!lo || !hi) quest_error("supplied buffer is null");
  if(gsq_sdf_mesh_bounds(g_query, lo, hi) != GSQ_OK) quest_error(gsq_last_error());
}

void QUEST_signed_distance_set_dimension(int dim)
{
  if(dim != 3) quest_error("The signed distance query only support 3D");
  require_not_initialized();
  g_params.dimension = dim;
}

void QUEST_signed_distance_set_closed_surface(bool status)
{
  require_not_initialized();
  g_params.closed = status;
}

void QUEST_signed_distance_set_compute_signs(bool computeSign)
{
  require_not_initialized();
  g_params.compute_sign = computeSign;
}

void QUEST_signed_distance_set_allocator(int allocatorID)
{
  require_not_initialized();
  g_params.allocator = allocatorID;
}

void QUEST_signed_distance_set_verbose(bool status)
{
  require_not_initialized();
  g_params.verbose = status;
}

void QUEST_signed_distance_use_shared_memory(bool status)
{
  require_not_initialized();
  g_params.shared_memory = status;
  if(status) quest_warning("Enabling shared memory requires MPI-3. Option is ignored!");
}

void QUEST_signed_distance_set_execution_space(int execSpace)
{
  require_not_initialized();
  if(execSpace < QUEST_SignedDistExec_CPU || execSpace > QUEST_SignedDistExec_GPU)
    quest_error("Unsupported execution space");
  g_params.exec_space = execSpace;
}

double QUEST_signed_distance_evaluate_0(double x, double y, double z)
{
  // signed_distance.cpp:346-372 (computeDistance(x, y, z))
  require_initialized("evaluate()!");
  double phi = 0.0;
  if(gsq_sdf_eval(g_query, &x, &y, &z, 1, 1, &phi, nullptr, nullptr, nullptr) != GSQ_OK)
    quest_error(gsq_last_error());
  return phi;
}

double QUEST_signed_distance_evaluate_1(double x, double y, double z, double* cp_x, double* cp_y, double* cp_z,
                                        double* n_x, double* n_y, double* n_z)
{
  // signed_distance.cpp:375-429 (computeDistance(pt, closest, normal))
  require_initialized("evaluate()!");
  if(!cp_x || !cp_y || !cp_z || !n_x || !n_y || !n_z) quest_error("output buffer is null");
  double phi = 0.0, cp[3], nrm[3];
  if(gsq_sdf_eval(g_query, &x, &y, &z, 1, 1, &phi, cp, nrm, nullptr) != GSQ_OK) quest_error(gsq_last_error());
  *cp_x = cp[0];
  *cp_y = cp[1];
  *cp_z = cp[2];
  *n_x = nrm[0];
  *n_y = nrm[1];
  *n_z = nrm[2];
  return phi;
}

void QUEST_signed_distance_finalize(void)
{
  // signed_distance.cpp:468-507: the query goes, the options stay
  if(g_query) gsq_sdf_destroy(g_query);
  g_query = nullptr;
}

int gsq_quest_init_mesh(const double* x, const double* y, const double* z, int32_t nnodes, const int32_t* tris,
                        int32_t ntris)
{
  // signed_distance_init(const mint::Mesh*) (signed_distance.cpp:163-227)
  if(g_query) quest_error("signed distance query has already been initialized!");
  if(g_params.dimension != 3) quest_error("signed distance query currently only support 3-D meshes");
  return create_query(x, y, z, 1, nnodes, tris, ntris);
}

void gsq_quest_evaluate_points(const double* x, const double* y, const double* z, int32_t npoints, double* phi)
{
  // signed_distance_evaluate(x, y, z, n, phi) (signed_distance.cpp:432-465)
  require_initialized("evaluate()!");
  if(!x) quest_error("x-coords array is null");
  if(!y) quest_error("y-coords array is null");
  if(!z) quest_error("z-coords array is null");
  if(!phi) quest_error("output phi array is null");
  if(gsq_sdf_eval(g_query, x, y, z, 1, npoints, phi, nullptr, nullptr, nullptr) != GSQ_OK)
    quest_error(gsq_last_error());
}

int gsq_quest_set_precision(int32_t precision)
{
  require_not_initialized();
  if(precision != GSQ_PRECISION_FP64 && precision != GSQ_PRECISION_MIXED)
    return gsq::fail(GSQ_ERR_INVALID, "unknown precision form");
  g_params.precision = precision;
  return GSQ_OK;
}

int gsq_quest_handle(const gsq_sdf** sdf)
{
  if(!sdf) return gsq::fail(GSQ_ERR_INVALID, "null argument");
  *sdf = g_query;
  return GSQ_OK;
}

}  // extern "C"
