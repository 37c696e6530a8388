// Internal declarations shared by the libgsq translation units.
//
// Device-side geometry helpers here keep the operation order of the axom
// primitives they restate (cited per function); the library is compiled with
// -fmad=false so no multiply-add is contracted, which keeps FP64 results
// bit-identical to the reference's host build.
#pragma once

#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>
#include <string>

#include "gsq.h"

namespace gsq
{
// ---- error reporting ------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define GSQ_CUDA_TRY(expr)                              \
  do                                                    \
  {                                                     \
    cudaError_t e_ = (expr);                            \
    if(e_ != cudaSuccess) return ::gsq::cuda_fail(e_, #expr); \
  } while(0)

// Device-side error flags (bit set by kernels, read by the host after a sync).
enum DeviceError : int
{
  DEVERR_STACK = 1,      // traversal stack overflow
  DEVERR_WAIT = 2,       // a bounded spin-wait expired
  DEVERR_RANGE = 4,      // an index was out of range
};

// True if ptr is device (or managed) memory of some device.
bool is_device_ptr(const void* ptr);

// Adds n to the library-wide count of kernel launches (gsq_kernel_launches).
void count_launch(int n = 1);

// ---- stream-ordered scratch -----------------------------------------------
// Owns one cudaMallocAsync allocation, freed on the same stream.
struct Scratch
{
  void* p = nullptr;
  cudaStream_t s = nullptr;
  Scratch() = default;
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
  ~Scratch() { release(); }
  cudaError_t alloc(size_t bytes, cudaStream_t stream)
  {
    release();
    s = stream;
    return cudaMallocAsync(&p, bytes ? bytes : 16, stream);
  }
  void release()
  {
    if(p) cudaFreeAsync(p, s);
    p = nullptr;
  }
  template <class T>
  T* as() const
  {
    return static_cast<T*>(p);
  }
};

// Four CUDA events, destroyed with the object (timing of one call).
struct Events
{
  cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
  Events() = default;
  Events(const Events&) = delete;
  Events& operator=(const Events&) = delete;
  ~Events()
  {
    for(auto& x : e)
      if(x) cudaEventDestroy(x);
  }
  cudaError_t create()
  {
    for(auto& x : e)
    {
      const cudaError_t r = cudaEventCreate(&x);
      if(r != cudaSuccess) return r;
    }
    return cudaSuccess;
  }
};

// Device buffer that is either the caller's device pointer or a staged copy
// of the caller's host array.
struct InBuf
{
  const void* dev = nullptr;
  Scratch own;
  // ext: device memory of at least `bytes` to stage into (else allocated)
  cudaError_t stage(const void* user, size_t bytes, cudaStream_t s, void* ext = nullptr)
  {
    if(user == nullptr || bytes == 0 || is_device_ptr(user))
    {
      dev = user;
      return cudaSuccess;
    }
    void* d = ext;
    if(!d)
    {
      cudaError_t e = own.alloc(bytes, s);
      if(e != cudaSuccess) return e;
      d = own.p;
    }
    dev = d;
    return cudaMemcpyAsync(d, user, bytes, cudaMemcpyHostToDevice, s);
  }
};

// Device buffer for an output that may be host memory (copied back by flush).
struct OutBuf
{
  void* user = nullptr;
  void* dev = nullptr;
  size_t bytes = 0;
  Scratch own;
  // ext: device memory of at least `b` to use for a host output (else allocated)
  cudaError_t prepare(void* u, size_t b, cudaStream_t s, void* ext = nullptr)
  {
    user = u;
    bytes = b;
    if(u == nullptr || b == 0 || is_device_ptr(u))
    {
      dev = u;
      return cudaSuccess;
    }
    if(ext)
    {
      dev = ext;
      return cudaSuccess;
    }
    cudaError_t e = own.alloc(b, s);
    dev = own.p;
    return e;
  }
  cudaError_t flush(cudaStream_t s)
  {
    if(user && dev != user && bytes) return cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, s);
    return cudaSuccess;
  }
};

// ---- layouts ----------------------------------------------------------------
// One record per inner node i: boxes of its two children (AoS lo/hi, left
// then right) and their links: c >= 0 an inner node, -(leafpos+1) a leaf.
// 128 bytes, one cache line per node visit.
struct __align__(16) NodeRec64
{
  double b[12];  // lo_l[3] hi_l[3] lo_r[3] hi_r[3]
  int child[2];
  int pad[6];
};
static_assert(sizeof(NodeRec64) == 128, "node record must be one 128-byte line");

// FP32 copy of a node record, boxes rounded outward (lo down, hi up). 64 B.
struct __align__(16) NodeRec32
{
  float b[12];
  int child[2];
  int pad[2];
};
static_assert(sizeof(NodeRec32) == 64, "fp32 node record must be 64 bytes");

constexpr int STACK_SIZE = 64;            // bvh_traverse.hpp:79
constexpr int BARRIER = -2000000000;      // bvh_traverse.hpp:80
constexpr double DEFAULT_SCALE = 1.000123;  // spin/BVH.hpp:410

// Built hierarchy resident in device memory.
struct BvhDev
{
  int n = 0;                      // leaves (>= 2 once built)
  NodeRec64* nodes = nullptr;     // n-1 records (root = 0)
  int* perm = nullptr;            // sorted leaf position -> original id
  uint32_t* codes = nullptr;      // sorted Morton codes
  int* lchild = nullptr;          // radix tree links (kept for export)
  int* rchild = nullptr;
  double bounds[6];               // host copy of the global bounds
  void* block = nullptr;          // single allocation backing the arrays
  size_t block_bytes = 0;
  // Build scratch and staging, kept between builds (grow-only), and the
  // build captured as a CUDA graph: a build with the same inputs as the one
  // before it (count, scale, box array, error word) replays the graph.
  void* work = nullptr;
  size_t work_bytes = 0;
  void* stage = nullptr;          // host boxes copied to the device
  size_t stage_bytes = 0;
  double* pad = nullptr;          // the two boxes of a 0/1-box build
  cudaStream_t cs = nullptr;      // private stream the build is captured on
  cudaGraphExec_t exec = nullptr;
  int graph_kernels = 0;
  int key_n = -1;                 // inputs of the last build
  double key_scale = 0.0;
  const double* key_in = nullptr;
  int* key_err = nullptr;
  void drop_graph();
  void release();
};

// Builds the hierarchy over n boxes (device array, n x 6), padding 0/1 boxes
// to 2 like BVH::initialize.  `done`, when given, is recorded on s once the
// build's device work is enqueued (before the bounds are read back).  Returns
// a GSQ status.
int bvh_build(BvhDev& B, const double* d_boxes, int n, double scale, cudaStream_t s, int* d_err,
              cudaEvent_t done = nullptr);

// Stable LSD radix sort of (key, value) pairs on key bits [0, end_bit).
// Inputs in keys[0]/vals[0]; keys[1]/vals[1] are scratch of the same size.
// If vals_iota, vals[0] is ignored and the values start as 0..n-1.  Returns
// the index (0 or 1) of the buffers holding the result, or a negative GSQ
// status.  d_err gets DEVERR_WAIT if a look-back wait expired.
int radix_sort_pairs(uint32_t* keys[2], int* vals[2], int n, int end_bit, bool vals_iota, cudaStream_t s,
                     int* d_err);

// The same sort with a caller-provided workspace of at least
// radix_sort_work_bytes(n) bytes (no allocation).
size_t radix_sort_work_bytes(int n);
// x rounded up to a multiple of 256 bytes
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
int radix_sort_pairs_prealloc(uint32_t* keys[2], int* vals[2], int n, int end_bit, bool vals_iota, void* work,
                              size_t work_bytes, cudaStream_t s, int* d_err);

// Exclusive scan of m int32 counts into offsets; *d_total (device int64)
// receives the sum.
// work: exclusive_scan_work_bytes(m) bytes of device scratch, or null to
// allocate it for the call.
int exclusive_scan(const int* d_in, int* d_out, int m, long long* d_total, cudaStream_t s, void* work = nullptr);
size_t exclusive_scan_work_bytes(int m);

// Reads and clears the device error word; returns a GSQ status.
int check_device_error(int* d_err, cudaStream_t s, const char* what);

// ---- exact device geometry (restatements of axom primal) ----------------
struct DBox
{
  double lo[3], hi[3];
};

__host__ __device__ inline bool box_valid(const double* lo, const double* hi)
{
  // BoundingBox::isValid (primal/geometry/BoundingBox.hpp:451-460)
  return !(lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]);
}

// ---- exact FP64 comparisons on the integer pipe ----------------------------
// This GPU executes FP64 instructions, comparisons included, at a small
// fraction of its FP32/integer rate (and its 64-bit integer operations share
// that cost, as ncu's FP64-pipe counters show), so comparison-heavy loops (box
// tests, addBox, the bounds fold, the closest-point region tests) compare
// doubles through their bit patterns with 32-bit operations: for non-NaN x, y
// with the 64 bits b (and -0 taken as +0), the map b -> b ^ ((b >> 63) &
// INT64_MAX) is strictly increasing, so the keys' lexicographic order on
// (signed high word, unsigned low word) is the FP64 order, and equal keys mean
// equal values.  Any comparison involving a NaN is false, as in IEEE
// arithmetic; the results equal the FP64 comparisons.
struct OKey
{
  int hi;
  unsigned lo;
  bool nan;
};

__host__ __device__ inline void dwords(double x, int& hi, unsigned& lo)
{
#ifdef __CUDA_ARCH__
  hi = __double2hiint(x);
  lo = (unsigned)__double2loint(x);
#else
  unsigned long long b;
  __builtin_memcpy(&b, &x, sizeof b);
  hi = (int)(unsigned)(b >> 32);
  lo = (unsigned)b;
#endif
}

__host__ __device__ inline OKey okey(double x)
{
  int h;
  unsigned l;
  dwords(x, h, l);
  const int mag = h & 0x7FFFFFFF;
  OKey r;
  r.nan = mag > 0x7FF00000 || (mag == 0x7FF00000 && l != 0u);
  if(mag == 0 && l == 0u) h = 0;  // -0 as +0
  if(h < 0)
  {
    h ^= 0x7FFFFFFF;
    l = ~l;
  }
  r.hi = h;
  r.lo = l;
  return r;
}
__host__ __device__ inline bool ok_klt(const OKey& a, const OKey& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__host__ __device__ inline bool ok_keq(const OKey& a, const OKey& b) { return a.hi == b.hi && a.lo == b.lo; }
__host__ __device__ inline bool ok_lt(const OKey& a, const OKey& b) { return !(a.nan | b.nan) && ok_klt(a, b); }
__host__ __device__ inline bool ok_gt(const OKey& a, const OKey& b) { return !(a.nan | b.nan) && ok_klt(b, a); }
__host__ __device__ inline bool ok_le(const OKey& a, const OKey& b) { return !(a.nan | b.nan) && !ok_klt(b, a); }
__host__ __device__ inline bool ok_ge(const OKey& a, const OKey& b) { return !(a.nan | b.nan) && !ok_klt(a, b); }
__host__ __device__ inline bool ok_eq(const OKey& a, const OKey& b) { return !(a.nan | b.nan) && ok_keq(a, b); }

// Comparisons with CP_EPS on the integer pipe, in 32-bit words (the FP64
// pipe of this GPU is scarce): with (h, l) the signed high and unsigned low
// words of x, x > EPS exactly when (h, l) lies in (EPS, INF] in lexicographic
// order (negative values have h < 0; NaNs lie above INF or are negative),
// x < -EPS exactly when h < 0 and the magnitude (h & INT32_MAX, l) lies in
// (EPS, INF], and |x| <= EPS exactly when the magnitude is at most EPS.
constexpr int CP_EPS_HI = 0x3D719799;           // the words of 1e-12
constexpr unsigned CP_EPS_LO = 0x812DEA11u;
__host__ __device__ inline bool mag_gt_eps(int m, unsigned l)
{
  return m > CP_EPS_HI || (m == CP_EPS_HI && l > CP_EPS_LO);
}
__host__ __device__ inline bool mag_le_inf(int m, unsigned l) { return m < 0x7FF00000 || (m == 0x7FF00000 && l == 0u); }
__host__ __device__ inline bool gt_eps(double x)
{
  int h;
  unsigned l;
  dwords(x, h, l);
  return h >= 0 && mag_gt_eps(h, l) && mag_le_inf(h, l);
}
__host__ __device__ inline bool lt_neg_eps(double x)
{
  int h;
  unsigned l;
  dwords(x, h, l);
  const int m = h & 0x7FFFFFFF;
  return h < 0 && mag_gt_eps(m, l) && mag_le_inf(m, l);
}
__host__ __device__ inline bool abs_le_eps(double x)
{
  int h;
  unsigned l;
  dwords(x, h, l);
  return !mag_gt_eps(h & 0x7FFFFFFF, l);
}

// box_valid on keys
__host__ __device__ inline bool box_valid_k(const OKey* lo, const OKey* hi)
{
  return !(ok_gt(lo[0], hi[0]) || ok_gt(lo[1], hi[1]) || ok_gt(lo[2], hi[2]));
}

__host__ __device__ inline double dot3(double u0, double u1, double u2, double v0, double v1, double v2)
{
  // Vector::dot_product (primal/geometry/Vector.hpp:544-553): accumulator
  // starts at 0, so (0 + u0 v0) + u1 v1 + u2 v2.
  double r = 0.0;
  r = r + u0 * v0;
  r = r + u1 * v1;
  r = r + u2 * v2;
  return r;
}

__host__ __device__ inline bool near_eq(double a, double b, double eps) { return fabs(a - b) <= eps; }

}  // namespace gsq
