// Stable onesweep LSD radix sort of (uint32 key, int32 value) pairs and an
// exclusive scan of int32 counts.
//
// Replaces the reference's sort_mcodes (spin/internal/linear_bvh/
// build_radix_tree.hpp:225-260: RAJA::stable_sort_pairs, i.e. CUB's radix
// sort on the GPU and std::stable_sort on the host) and the
// RAJA::exclusive_scan of findCandidatesImpl (policy/LinearBVH.hpp:332-334).
//
// One launch per 8-bit digit.  Each block takes the next tile (4096 keys) from
// an atomic tile counter, ranks its keys per digit with warp-aggregated
// counting (__match_any_sync: one shared-memory update per distinct digit per
// warp row), and obtains its global offsets by a decoupled look-back over the
// tiles before it (eight predecessors read at once).  Ranks follow input
// position (warp, row, lane order), so the sort is stable, which makes the
// result identical to a stable sort of the reference.  Every look-back wait is
// bounded: after SPIN_LIMIT polls without progress the block sets
// DEVERR_WAIT and continues.
#include "gsq_internal.cuh"

#include <algorithm>

namespace gsq
{
namespace
{
constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int KPT = 16;                 // keys per thread
constexpr int TILE = THREADS * KPT;     // 4096 keys per tile
constexpr int RADIX = 256;
constexpr unsigned FLAG_AGG = 1u << 30; // tile aggregate published
constexpr unsigned FLAG_PRE = 2u << 30; // inclusive prefix published
constexpr unsigned VAL_MASK = (1u << 30) - 1;
constexpr long long SPIN_LIMIT = 1ll << 20;  // polls without progress before a look-back wait gives up
constexpr int LOOK = 8;                  // look-back window (tiles read at once)

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p)
{
  return *reinterpret_cast<const volatile unsigned*>(p);
}
__device__ __forceinline__ void st_volatile(unsigned* p, unsigned v) { *reinterpret_cast<volatile unsigned*>(p) = v; }

// Digit counts of every pass (one shared histogram per block, added into
// hist), then the exclusive prefix over the 256 digits of every pass, taken by
// the last block to finish (`done`, zeroed with hist; blockDim.x == RADIX).
__global__ void __launch_bounds__(RADIX) k_histogram(const uint32_t* __restrict__ keys, int n, int passes,
                                                     unsigned* __restrict__ hist, unsigned* __restrict__ done)
{
  __shared__ unsigned sh[4 * RADIX];
  __shared__ bool s_last;
  for(int i = threadIdx.x; i < passes * RADIX; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const uint32_t k = keys[i];
    for(int p = 0; p < passes; ++p) atomicAdd(&sh[p * RADIX + ((k >> (8 * p)) & 0xFF)], 1u);
  }
  __syncthreads();
  for(int i = threadIdx.x; i < passes * RADIX; i += blockDim.x)
    if(sh[i]) atomicAdd(&hist[i], sh[i]);
  __threadfence();
  __syncthreads();
  if(threadIdx.x == 0) s_last = (atomicAdd(done, 1u) == gridDim.x - 1);
  __syncthreads();
  if(!s_last) return;
  __threadfence();
  unsigned* s = sh;  // reused: one pass at a time
  for(int p = 0; p < passes; ++p)
  {
    const unsigned v = __ldcg(&hist[p * RADIX + threadIdx.x]);
    s[threadIdx.x] = v;
    __syncthreads();
    for(int off = 1; off < RADIX; off <<= 1)
    {
      const unsigned t = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    hist[p * RADIX + threadIdx.x] = s[threadIdx.x] - v;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(THREADS) k_onesweep(const uint32_t* __restrict__ kin,
                                                        const int* __restrict__ vin,
                                                        int iota,
                                                        uint32_t* __restrict__ kout,
                                                        int* __restrict__ vout,
                                                        int n,
                                                        int shift,
                                                        const unsigned* __restrict__ digit_offsets,
                                                        unsigned* lookback,
                                                        int* tile_counter,
                                                        int* err)
{
  __shared__ unsigned s_whist[WARPS][RADIX];
  __shared__ unsigned s_base[RADIX];
  __shared__ int s_tile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if(threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  for(int i = threadIdx.x; i < WARPS * RADIX; i += THREADS) (&s_whist[0][0])[i] = 0;
  __syncthreads();
  const int tile = s_tile;
  const long long base = (long long)tile * TILE + warp * (KPT * 32);

  uint32_t key[KPT];
  int val[KPT];
  unsigned rank[KPT];
#pragma unroll
  for(int j = 0; j < KPT; ++j)
  {
    const long long idx = base + j * 32 + lane;
    const bool ok = idx < n;
    key[j] = ok ? kin[idx] : 0u;
    val[j] = ok ? (iota ? (int)idx : vin[idx]) : 0;
  }
  const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
  for(int j = 0; j < KPT; ++j)
  {
    const long long idx = base + j * 32 + lane;
    const unsigned d = (idx < n) ? ((key[j] >> shift) & 0xFFu) : 256u;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const unsigned below = __popc(peers & lt_mask);
    const unsigned before = (d < 256u) ? s_whist[warp][d] : 0u;
    rank[j] = before + below;
    __syncwarp();
    if(d < 256u && below == 0) s_whist[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit (thread = digit): warp-exclusive prefixes and the tile total.
  const int d = threadIdx.x;
  unsigned total = 0;
#pragma unroll
  for(int w = 0; w < WARPS; ++w)
  {
    const unsigned t = s_whist[w][d];
    s_whist[w][d] = total;
    total += t;
  }
  unsigned excl = 0;
  unsigned* lb = lookback + (size_t)tile * RADIX + d;
  if(tile == 0)
    st_volatile(lb, FLAG_PRE | total);
  else
  {
    st_volatile(lb, FLAG_AGG | total);
    // LOOK tiles are read at once (independent loads), then consumed in order
    // up to the first unpublished one or the first inclusive prefix
    long long spins = 0;
    for(int k = tile - 1; k >= 0;)
    {
      unsigned v[LOOK];
#pragma unroll
      for(int u = 0; u < LOOK; ++u) v[u] = (k - u >= 0) ? ld_volatile(lookback + (size_t)(k - u) * RADIX + d) : 0u;
      int used = 0;
      bool done = false;
#pragma unroll
      for(int u = 0; u < LOOK; ++u)
      {
        if(done || used < u || k - u < 0) continue;
        const unsigned flag = v[u] & ~VAL_MASK;
        if(flag == 0u) continue;
        excl += v[u] & VAL_MASK;
        used = u + 1;
        done = (flag == FLAG_PRE);
      }
      if(done) break;
      if(used == 0 && ++spins > SPIN_LIMIT)
      {
        atomicOr(err, DEVERR_WAIT);
        break;
      }
      k -= used;
    }
    st_volatile(lb, FLAG_PRE | ((excl + total) & VAL_MASK));
  }
  s_base[d] = digit_offsets[d] + excl;
  __syncthreads();

#pragma unroll
  for(int j = 0; j < KPT; ++j)
  {
    const long long idx = base + j * 32 + lane;
    if(idx < n)
    {
      const unsigned dd = (key[j] >> shift) & 0xFFu;
      const unsigned pos = s_base[dd] + s_whist[warp][dd] + rank[j];
      if(pos < (unsigned)n)  // always true unless a look-back wait expired (flagged above)
      {
        kout[pos] = key[j];
        vout[pos] = val[j];
      }
    }
  }
}

// ---- exclusive scan ---------------------------------------------------------
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_IPT = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;

__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* total)
{
  __shared__ long long s_warp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for(int o = 1; o < 32; o <<= 1)
  {
    const long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if(lane >= o) x += y;
  }
  if(lane == 31) s_warp[warp] = x;
  __syncthreads();
  if(warp == 0)
  {
    long long w = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
    {
      const long long y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if(lane >= o) w += y;
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  const long long warp_excl = warp ? s_warp[warp - 1] : 0;
  *total = s_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_excl + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const int* __restrict__ in, int m, long long* sums)
{
  long long s = 0;
  const long long b = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
#pragma unroll
  for(int k = 0; k < SCAN_IPT; ++k)
    if(b + k < m) s += in[b + k];
  long long tot;
  block_exclusive_scan(s, &tot);
  if(threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(long long* sums, int nb, long long* d_total)
{
  long long carry = 0;
  for(int start = 0; start < nb; start += SCAN_THREADS)
  {
    const int i = start + threadIdx.x;
    const long long v = (i < nb) ? sums[i] : 0;
    long long tot;
    const long long ex = block_exclusive_scan(v, &tot);
    if(i < nb) sums[i] = carry + ex;
    carry += tot;
  }
  if(threadIdx.x == 0 && d_total) *d_total = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int* __restrict__ in,
                                                               int* __restrict__ out,
                                                               int m,
                                                               const long long* __restrict__ sums)
{
  const long long b = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
  int v[SCAN_IPT];
  long long s = 0;
#pragma unroll
  for(int k = 0; k < SCAN_IPT; ++k)
  {
    v[k] = (b + k < m) ? in[b + k] : 0;
    s += v[k];
  }
  long long tot;
  long long ex = block_exclusive_scan(s, &tot) + sums[blockIdx.x];
#pragma unroll
  for(int k = 0; k < SCAN_IPT; ++k)
    if(b + k < m)
    {
      out[b + k] = (int)ex;
      ex += v[k];
    }
}
}  // namespace

// Self-test of the bounded waits: one block runs a onesweep pass on tile 1
// of a two-tile input while tile 0 is never processed, so its look-back waits
// for a flag nothing sets.  After SPIN_LIMIT polls without progress the block
// sets DEVERR_WAIT, finishes its pass (its scatter stays inside the output)
// and the call reports GSQ_ERR_DEVICE; the context stays usable.
int sort_wait_selftest(cudaStream_t s)
{
  const int n = 2 * TILE;
  Scratch buf;
  const size_t words = 4 * (size_t)n + (size_t)2 * RADIX + 64;
  GSQ_CUDA_TRY(buf.alloc(sizeof(unsigned) * words, s));
  unsigned* w = buf.as<unsigned>();
  GSQ_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(unsigned) * words, s));
  uint32_t* kin = w;
  uint32_t* kout = w + n;
  int* vout = reinterpret_cast<int*>(w + 2 * (size_t)n);
  unsigned* offsets = w + 3 * (size_t)n;                  // RADIX zero digit offsets
  unsigned* lookback = offsets + RADIX;                    // two tiles x RADIX, never published for tile 0
  int* tile_counter = reinterpret_cast<int*>(w + 4 * (size_t)n);  // words after the look-back area
  int* err = tile_counter + 8;
  const int one = 1;  // the block takes tile 1
  GSQ_CUDA_TRY(cudaMemcpyAsync(tile_counter, &one, sizeof(int), cudaMemcpyHostToDevice, s));
  count_launch();
  k_onesweep<<<1, THREADS, 0, s>>>(kin, nullptr, 1, kout, vout, n, 0, offsets, lookback, tile_counter, err);
  GSQ_CUDA_TRY(cudaGetLastError());
  return check_device_error(err, s, "sort wait self-test");
}

int radix_sort_pairs(uint32_t* keys[2], int* vals[2], int n, int end_bit, bool vals_iota, cudaStream_t s, int* d_err)
{
  if(n <= 0) return 0;
  if(n >= (1 << 30)) return fail(GSQ_ERR_INVALID, "radix sort supports fewer than 2^30 keys");
  const int passes = (end_bit + 7) / 8;
  const int ntiles = (n + TILE - 1) / TILE;
  Scratch work;
  const size_t hist_words = 4 * RADIX;
  const size_t lb_words = (size_t)ntiles * RADIX;
  GSQ_CUDA_TRY(work.alloc(sizeof(unsigned) * (hist_words + lb_words + 32), s));
  unsigned* hist = work.as<unsigned>();
  unsigned* lookback = hist + hist_words;
  int* tile_counter = reinterpret_cast<int*>(lookback + lb_words);
  // hist and, in the first look-back word (free until the first pass clears
  // the look-back area), the histogram's block counter
  GSQ_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * (hist_words + 1), s));
  const int hblocks = (int)std::min<long long>(((long long)n + 1023) / 1024, 1024);
  k_histogram<<<hblocks, RADIX, 0, s>>>(keys[0], n, passes, hist, lookback);
  count_launch(1 + passes);
  int cur = 0;
  for(int p = 0; p < passes; ++p)
  {
    GSQ_CUDA_TRY(cudaMemsetAsync(lookback, 0, sizeof(unsigned) * (lb_words + 32), s));
    k_onesweep<<<ntiles, THREADS, 0, s>>>(keys[cur], vals[cur], (vals_iota && p == 0) ? 1 : 0, keys[cur ^ 1],
                                          vals[cur ^ 1], n, 8 * p, hist + p * RADIX, lookback, tile_counter,
                                          d_err);
    cur ^= 1;
  }
  GSQ_CUDA_TRY(cudaGetLastError());
  return cur;
}

size_t radix_sort_work_bytes(int n)
{
  const size_t ntiles = ((size_t)std::max(n, 1) + TILE - 1) / TILE;
  return sizeof(unsigned) * (4 * RADIX + ntiles * RADIX + 32);
}

int radix_sort_pairs_prealloc(uint32_t* keys[2], int* vals[2], int n, int end_bit, bool vals_iota, void* work,
                              size_t work_bytes, cudaStream_t s, int* d_err)
{
  if(n <= 0) return 0;
  if(n >= (1 << 30)) return fail(GSQ_ERR_INVALID, "radix sort supports fewer than 2^30 keys");
  if(!work || work_bytes < radix_sort_work_bytes(n)) return fail(GSQ_ERR_INVALID, "sort workspace too small");
  const int passes = (end_bit + 7) / 8;
  const int ntiles = (n + TILE - 1) / TILE;
  const size_t hist_words = 4 * RADIX;
  const size_t lb_words = (size_t)ntiles * RADIX;
  unsigned* hist = static_cast<unsigned*>(work);
  unsigned* lookback = hist + hist_words;
  int* tile_counter = reinterpret_cast<int*>(lookback + lb_words);
  // hist and, in the first look-back word (free until the first pass clears
  // the look-back area), the histogram's block counter
  GSQ_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * (hist_words + 1), s));
  const int hblocks = (int)std::min<long long>(((long long)n + 1023) / 1024, 1024);
  k_histogram<<<hblocks, RADIX, 0, s>>>(keys[0], n, passes, hist, lookback);
  count_launch(1 + passes);
  int cur = 0;
  for(int p = 0; p < passes; ++p)
  {
    GSQ_CUDA_TRY(cudaMemsetAsync(lookback, 0, sizeof(unsigned) * (lb_words + 32), s));
    k_onesweep<<<ntiles, THREADS, 0, s>>>(keys[cur], vals[cur], (vals_iota && p == 0) ? 1 : 0, keys[cur ^ 1],
                                          vals[cur ^ 1], n, 8 * p, hist + p * RADIX, lookback, tile_counter,
                                          d_err);
    cur ^= 1;
  }
  GSQ_CUDA_TRY(cudaGetLastError());
  return cur;
}

size_t exclusive_scan_work_bytes(int m)
{
  return sizeof(long long) * (size_t)std::max<long long>(1, ((long long)m + SCAN_TILE - 1) / SCAN_TILE);
}

int exclusive_scan(const int* d_in, int* d_out, int m, long long* d_total, cudaStream_t s, void* work)
{
  if(m <= 0)
  {
    if(d_total) GSQ_CUDA_TRY(cudaMemsetAsync(d_total, 0, sizeof(long long), s));
    return GSQ_OK;
  }
  const int nb = (int)(((long long)m + SCAN_TILE - 1) / SCAN_TILE);
  Scratch own;
  long long* sums = static_cast<long long*>(work);
  if(!sums)
  {
    GSQ_CUDA_TRY(own.alloc(sizeof(long long) * nb, s));
    sums = own.as<long long>();
  }
  k_scan_tiles<<<nb, SCAN_THREADS, 0, s>>>(d_in, m, sums);
  k_scan_sums<<<1, SCAN_THREADS, 0, s>>>(sums, nb, d_total);
  k_scan_apply<<<nb, SCAN_THREADS, 0, s>>>(d_in, d_out, m, sums);
  count_launch(3);
  GSQ_CUDA_TRY(cudaGetLastError());
  return GSQ_OK;
}

}  // namespace gsq

extern "C" int gsq_selftest_bounded_wait(void* stream)
{
  return gsq::sort_wait_selftest(static_cast<cudaStream_t>(stream));
}
