// FP32 records and the certified traversal of the mixed-precision signed
// distance, shared by the mixed query kernel and the adjoint kernel.
#pragma once

#include "gsq_leaf32.cuh"
#include "gsq_sdf_device.cuh"
#include "gsq_sign.cuh"

namespace gsq
{
template <int NPC>
struct LeafRec32;
// FP32 triangle(s) of one leaf: vertices rounded to nearest, and per
// triangle the error factor ec = 256 * 2^-24 * kappa and max edge length lt
// (triangles also carry fz, the bound on the reference's fuzzy closest-point
// displacement; quads compute it from ec and lt).
template <>
struct __align__(16) LeafRec32<3>
{
  float v[9];
  float ec;
  float lt;
  float fz;
};
template <>
struct __align__(16) LeafRec32<4>
{
  float v[12];
  float ec[2];
  float lt[2];
};
static_assert(sizeof(LeafRec32<3>) == 48, "fp32 triangle leaf is 48 bytes");
static_assert(sizeof(LeafRec32<4>) == 64, "fp32 quad leaf is 64 bytes");

// Per-mesh entry of a query launch: where the mesh's node and leaf records
// start in the shared arrays, its node box and coordinate bound.
struct MeshInfo
{
  long long node_off;
  long long leaf_off;
  double domain[6];
  float mesh_max;
  int pad;
};

namespace sdf
{
// One node visit of record cur decided in FP32 (visit32_core on its two child
// boxes and slacks); ch receives the record's child links.
__device__ __forceinline__ bool visit32(const NodeRec32* __restrict__ nodes32, int cur, const QCtx& c, bool& inL,
                                        bool& inR, bool& swap, int2& ch)
{
  const float4* r = reinterpret_cast<const float4*>(nodes32 + cur);
  const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
  const int4 lk = __ldg(reinterpret_cast<const int4*>(r + 3));
  ch = make_int2(lk.x, lk.y);
  const float lo_l[3] = {a.x, a.y, a.z}, hi_l[3] = {a.w, b.x, b.y};
  const float lo_r[3] = {b.z, b.w, cc.x}, hi_r[3] = {cc.y, cc.z, cc.w};
  return visit32_core(lo_l, hi_l, lo_r, hi_r, __int_as_float(lk.z), __int_as_float(lk.w), c, inL, inR, swap);
}

// FP32 certificate of the leaf action: bit s of the result is set when
// triangle s may change the running minimum or the pseudo-normal sum and so
// needs the FP64 checkCandidate.
template <int NPC>
__device__ __forceinline__ int leaf_prefilter(const LeafRec32<NPC>* __restrict__ leaves32, int leafpos, const QCtx& c)
{
  const float4* r = reinterpret_cast<const float4*>(leaves32 + leafpos);
  float v[3 * NPC];
  float ec[2], lt[2];
  if constexpr(NPC == 3)
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    ec[0] = cc.y, lt[0] = cc.z;
  }
  else
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2), d4 = __ldg(r + 3);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    v[9] = cc.y, v[10] = cc.z, v[11] = cc.w;
    ec[0] = d4.x, ec[1] = d4.y, lt[0] = d4.z, lt[1] = d4.w;
  }
  int need = 0;
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    const float* A = v;
    const float* B = v + 3 * (s + 1);
    const float* C = v + 3 * (s + 2);
    float off[3];
    int kind;
    const float d2 = dist2_f32_flat(c.qf, A, B, C, off, kind);
    const float ap = fmaxf(fabsf(c.qf[0] - A[0]), fmaxf(fabsf(c.qf[1] - A[1]), fabsf(c.qf[2] - A[2])));
    // the general error of tri_bounds (kappa^2 growth for slivers included)
    const float E =
        __fadd_ru(c.lip, __fmul_ru(__fmul_ru(ec[s], fmaxf(1.f, ec[s] * 65536.f * 0.0625f)), __fadd_ru(ap, lt[s])));
    const float lim = __fadd_ru(c.thr_leaf, E);
    if(!(d2 > __fmul_ru(__fmul_ru(lim, lim), 1.0f + 0x1p-20f))) need |= 1 << s;
  }
  return need;
}

// leaf_prefilter that also bounds, for the triangles it keeps, the squared
// distance the FP64 checkCandidate will compute (tri_bounds): [lo2, hi2] holds
// the minimum over the kept triangles, cpf and rad the last kept one's closest
// point estimate and its radius.  mesh_max bounds the mesh's coordinates.
template <int NPC>
__device__ __forceinline__ int leaf_prefilter_bounds(const LeafRec32<NPC>* __restrict__ leaves32, int leafpos,
                                                     const QCtx& c, float mesh_max, float& lo2, float& hi2, float* cpf,
                                                     float& rad)
{
  const float4* r = reinterpret_cast<const float4*>(leaves32 + leafpos);
  float v[3 * NPC];
  float ec[2], lt[2];
  float fzt = 0.f;
  if constexpr(NPC == 3)
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    ec[0] = cc.y, lt[0] = cc.z, fzt = cc.w;
  }
  else
  {
    const float4 a = __ldg(r), b = __ldg(r + 1), cc = __ldg(r + 2), d4 = __ldg(r + 3);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w, v[8] = cc.x;
    v[9] = cc.y, v[10] = cc.z, v[11] = cc.w;
    ec[0] = d4.x, ec[1] = d4.y, lt[0] = d4.z, lt[1] = d4.w;
  }
  int need = 0;
  lo2 = INFINITY;
  hi2 = INFINITY;
  rad = INFINITY;
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    float d2, l2, h2;
    if(tri_bounds<NPC == 4>(c, mesh_max, v, v + 3 * (s + 1), v + 3 * (s + 2), ec[s], lt[s], fzt, d2, l2, h2, cpf, rad))
    {
      need |= 1 << s;
      lo2 = (d2 == d2) ? fminf(lo2, l2) : 0.f;
      hi2 = (d2 == d2 && h2 == h2) ? fminf(hi2, h2) : hi2;
    }
  }
  // both triangles of a quad kept: either may set the closest point, and
  // cpf is only the second one's, so nothing may be certified far from it
  if(need == 3) rad = INFINITY;
  return need;
}

// The roundings the sign certificate asks for, as device intrinsics (the
// certificate is evaluated on the device; the host checker supplies its own).
struct SignOps
{
#ifdef __CUDA_ARCH__
  __host__ __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  __host__ __device__ static float add_ru(float a, float b) { return __fadd_ru(a, b); }
  __host__ __device__ static float add_rd(float a, float b) { return __fadd_rd(a, b); }
  __host__ __device__ static float sub_rd(float a, float b) { return __fsub_rd(a, b); }
  __host__ __device__ static float mul_ru(float a, float b) { return __fmul_ru(a, b); }
  __host__ __device__ static float mul_rd(float a, float b) { return __fmul_rd(a, b); }
  __host__ __device__ static float div_ru(float a, float b) { return __fdiv_ru(a, b); }
  __host__ __device__ static float rsqrt(float a) { return __frsqrt_rn(a); }
  __host__ __device__ static float acos(float a) { return acosf(a); }
  __host__ __device__ static float to_float(double a) { return __double2float_rn(a); }
#else
  static float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static float add_ru(float a, float b) { return nextafterf(a + b, INFINITY); }
  static float add_rd(float a, float b) { return nextafterf(a + b, -INFINITY); }
  static float sub_rd(float a, float b) { return nextafterf(a - b, -INFINITY); }
  static float mul_ru(float a, float b) { return nextafterf(a * b, INFINITY); }
  static float mul_rd(float a, float b) { return nextafterf(a * b, -INFINITY); }
  static float div_ru(float a, float b) { return nextafterf(a / b, INFINITY); }
  static float rsqrt(float a) { return (float)(1.0 / sqrt((double)a)); }
  static float acos(float a) { return (float)::acos((double)a); }
  static float to_float(double a) { return (float)a; }
#endif
};

// FP32 certificate of computeSign (SD:751-763) for one finished query (see
// gsq_sign.cuh): +1 or -1 when the FP64 dot(q - cp, N) >= 0 of finish_query
// certainly has that outcome, 0 when not certain (the caller then evaluates
// the pseudo-normal in FP64).  The triangles come from the FP32 leaf records:
// the closest face (type 2) or the recorded pseudo-normal contributions.
template <int NPC>
__device__ __forceinline__ double sign32(const double* q, const MinCand& mc, const LeafRec32<NPC>* __restrict__ leaves32,
                                         float M)
{
  const float r[3] = {__double2float_rn(q[0] - mc.mp[0]), __double2float_rn(q[1] - mc.mp[1]),
                      __double2float_rn(q[2] - mc.mp[2])};
  auto rec_tri = [&](int leaf, int sub, const float*& A, const float*& B, const float*& C, float& L) {
    const LeafRec32<NPC>& rec = leaves32[leaf];
    A = rec.v;
    B = rec.v + 3 * (sub + 1);
    C = rec.v + 3 * (sub + 2);
    if constexpr(NPC == 3)
      L = rec.lt;
    else
      L = rec.lt[sub];
  };
  if(mc.type == 2)
  {
    auto face_tri = [&](int, const float*& A, const float*& B, const float*& C, float& L, int& k) {
      k = 0;
      rec_tri(mc.leaf, mc.sub, A, B, C, L);
    };
    return sign_certificate<SignOps>(r, true, mc.sn, 1, face_tri, M);
  }
  auto pend_tri = [&](int i, const float*& A, const float*& B, const float*& C, float& L, int& k) {
    const int code = mc.pend[i];
    k = code & 3;
    rec_tri(code >> 3, (code >> 2) & 1, A, B, C, L);
  };
  return sign_certificate<SignOps>(r, false, mc.sn, mc.npend, pend_tri, M);
}

// Audit of a skipped triangle: counts it if the FP64 distance contradicts
// the certificate (it would lie within sqrt(minSq) + 1e-6).
template <int NPC>
__device__ __forceinline__ int leaf_audit(const LeafRec<NPC>* __restrict__ leaves64, int leafpos, int skip_mask,
                                          const double* q, double minSq)
{
  double w[3 * NPC];
  load_leaf<NPC>(leaves64, leafpos, w);
  int bad = 0;
  for(int s = 0; s < NPC - 2; ++s)
  {
    if(!(skip_mask & (1 << s))) continue;
    double cp[3];
    closest_point(q, w, w + 3 * (s + 1), w + 3 * (s + 2), cp);
    const double lim64 = sqrt(minSq) + 1e-6;
    if(sqdist_pp(q, cp) <= lim64 * lim64) ++bad;
  }
  return bad;
}

// Audit: two checkCandidate states are the same (pseudo-normal sums evaluated).
template <int NPC>
__device__ __forceinline__ bool same_state(MinCand a, MinCand b, const LeafRec<NPC>* __restrict__ leaves64)
{
  flush_normals<NPC>(a, leaves64);
  flush_normals<NPC>(b, leaves64);
  return a.minSq == b.minSq && a.type == b.type && a.leaf == b.leaf && a.sub == b.sub && a.mp[0] == b.mp[0] &&
         a.mp[1] == b.mp[1] && a.mp[2] == b.mp[2] && a.sn[0] == b.sn[0] && a.sn[1] == b.sn[1] && a.sn[2] == b.sn[2];
}

// FP64 checkCandidate on the triangles of `need`, in the reference's order.
template <int NPC>
__device__ __forceinline__ void leaf_refine(const LeafRec<NPC>* __restrict__ leaves64, int leafpos, int need,
                                            const double* q, MinCand& mc, bool computeNormal)
{
  double w[3 * NPC];
  load_leaf<NPC>(leaves64, leafpos, w);
#pragma unroll
  for(int s = 0; s < NPC - 2; ++s)
  {
    if(!(need & (1 << s))) continue;
    const double* T[3] = {w, w + 3 * (s + 1), w + 3 * (s + 2)};
    check_triangle<NPC, false>(q, mc, T, leaves64, leafpos, s, computeNormal);
  }
}

}  // namespace sdf
}  // namespace gsq
