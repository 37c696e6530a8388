// A user kernel over a gsq BVH through the device traversal header: the
// two-pass point query of quest's example (quest/examples/
// quest_bvh_two_pass.cpp:143-200) - pass 1 counts each point's candidate
// boxes, the caller scans the counts, pass 2 writes the candidate ids.  The
// test compares the result with gsq_bvh_find_points.
#include "gsq_device.cuh"

namespace
{
struct Contains
{
  double p[3];
  __device__ bool operator()(const double* lo, const double* hi) const
  {
    for(int d = 0; d < 3; ++d)
      if(p[d] < lo[d] || p[d] > hi[d]) return false;
    return true;
  }
};

__global__ void k_count(gsq_bvh_view view, const double* pts, int m, int* counts, int* err)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  Contains c {{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}};
  int n = 0;
  if(!gsq::device::traverse_tree(view, c, [&](int) { ++n; })) atomicOr(err, 1);
  counts[i] = n;
}

__global__ void k_fill(gsq_bvh_view view, const double* pts, int m, const int* offsets, int* cands)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if(i >= m) return;
  Contains c {{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}};
  int* out = cands + offsets[i];
  int n = 0;
  gsq::device::traverse_tree(view, c, [&](int id) { out[n++] = id; });
}
}  // namespace

extern "C" {

// Device arrays; returns 0, or 1 if a traversal stack overflowed.
int two_pass_count(const gsq_bvh_view* view, const double* pts, int m, int* counts, int* err)
{
  k_count<<<(m + 127) / 128, 128>>>(*view, pts, m, counts, err);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

int two_pass_fill(const gsq_bvh_view* view, const double* pts, int m, const int* offsets, int* cands)
{
  k_fill<<<(m + 127) / 128, 128>>>(*view, pts, m, offsets, cands);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
}
