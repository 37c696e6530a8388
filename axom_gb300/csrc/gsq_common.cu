// Error state, pointer classification and small host helpers of libgsq.
#include "gsq_internal.cuh"

#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace gsq
{
namespace
{
thread_local std::string g_last_error;
std::atomic<long long> g_launches {0};
}  // namespace

void count_launch(int n) { g_launches += n; }

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg)
{
  set_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
  const int code = (e == cudaErrorMemoryAllocation) ? GSQ_ERR_NOMEM : GSQ_ERR_CUDA;
  return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_device_ptr(const void* ptr)
{
  if(!ptr) return false;
  cudaPointerAttributes a;
  if(cudaPointerGetAttributes(&a, ptr) != cudaSuccess)
  {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int check_device_error(int* d_err, cudaStream_t s, const char* what)
{
  int h = 0;
  GSQ_CUDA_TRY(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GSQ_CUDA_TRY(cudaStreamSynchronize(s));
  if(h == 0) return GSQ_OK;
  GSQ_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), s));
  std::string msg = std::string(what) + ": device reported";
  if(h & DEVERR_STACK) msg += " traversal stack overflow";
  if(h & DEVERR_WAIT) msg += " expired bounded wait";
  if(h & DEVERR_RANGE) msg += " index out of range";
  return fail(GSQ_ERR_DEVICE, msg);
}

}  // namespace gsq

extern "C" {

const char* gsq_last_error(void) { return gsq::g_last_error.c_str(); }

const char* gsq_version(void) { return "gsq 0.1.0 (sm_103a)"; }

int64_t gsq_kernel_launches(void) { return gsq::g_launches.load(); }

int gsq_free(void* ptr)
{
  if(!ptr) return GSQ_OK;
  if(gsq::is_device_ptr(ptr))
  {
    GSQ_CUDA_TRY(cudaFree(ptr));
  }
  else
    std::free(ptr);
  return GSQ_OK;
}

int gsq_memcpy(void* dst, const void* src, size_t bytes)
{
  if(bytes == 0) return GSQ_OK;
  if(!dst || !src) return gsq::fail(GSQ_ERR_INVALID, "null pointer");
  GSQ_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
  return GSQ_OK;
}

// Vector::unitVector (primal/geometry/Vector.hpp:477-493): v * (1/sqrt(|v|^2))
// when |v|^2 >= PRIMAL_TINY (1e-50), else (1, 0, 0).
int gsq_ray_normalize(const double* raw, int32_t m, double* unit)
{
  if(m < 0 || (m > 0 && (!raw || !unit))) return gsq::fail(GSQ_ERR_INVALID, "invalid arguments");
  for(int32_t i = 0; i < m; ++i)
  {
    const double* v = raw + 3 * (size_t)i;
    double* o = unit + 3 * (size_t)i;
    const double l2 = gsq::dot3(v[0], v[1], v[2], v[0], v[1], v[2]);
    if(l2 >= 1e-50)
    {
      const double s = 1.0 / std::sqrt(l2);
      o[0] = v[0] * s;
      o[1] = v[1] * s;
      o[2] = v[2] * s;
    }
    else
    {
      o[0] = 1.0;
      o[1] = 0.0;
      o[2] = 0.0;
    }
  }
  return GSQ_OK;
}

}  // extern "C"
