// me_common.cuh -- device building blocks shared by the motion estimators:
// padded-reference geometry, packed vectors, the median predictor and the
// Lagrangian vector pick.
#pragma once

#include "vppgpu_internal.cuh"

namespace vppgpu {

// Padded 8-bit reference: every plane is stored with PAD samples of edge
// replication on each side (OverlayExtMem2Dv2::FillBoundary,
// src/ImageUtils/OverlayExtMem2Dv2.cpp:153-211, is a coordinate clamp).  48
// covers the +-31 search window, the 3-sample 6-tap margin of the sub-pel
// stages and the 16-sample macroblock overhang the reference allows.
constexpr int PAD = 48;

struct Plane8 {
    const unsigned char* p;  // top-left of the padded buffer
    int stride;              // bytes per padded row (multiple of 16)
    __device__ __forceinline__ const unsigned char* at(int x, int y) const
    {
        return p + (size_t)(y + PAD) * stride + (x + PAD);
    }
};

// Status bits written by device code.
constexpr int ST_PIXEL_RANGE = 1;
constexpr int ST_TIMEOUT = 2;

__device__ __forceinline__ int pack_mv(int x, int y) { return (int)((unsigned)(x & 0xffff) | ((unsigned)y << 16)); }
__device__ __forceinline__ int mv_x(int p) { return (int)(short)(p & 0xffff); }
__device__ __forceinline__ int mv_y(int p) { return p >> 16; }

__device__ __forceinline__ int tap6(int a, int b, int c, int d, int e, int f)
{
    return a - 5 * b + 20 * c + 20 * d - 5 * e + f;
}

// Sum over the warp (every lane gets it).
__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Median prediction (MacroBlockH264::GetMbMotionMedianPred,
// src/CodecUtils/MacroBlockH264.cpp:757-816; Median :923-936) from the
// current vectors of the left (A), above (B), above-right (C, else
// above-left D) neighbours; unavailable neighbours count as (0,0) and with
// neither B nor C both take A.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int median3(int x, int y, int z)
{
    int lo = y - z < 0 ? y : z, hi = y - z < 0 ? z : y;
    lo = x < lo ? x : lo;
    hi = x > hi ? x : hi;
    return x + y + z - lo - hi;
}

// Neighbour availability bits kept in the per-macroblock flags (position
// and slice membership, MacroBlockH264::Initialise, MacroBlockH264.cpp:319-).
constexpr int AV_A = 1 << 1;   // left
constexpr int AV_B = 1 << 2;   // above
constexpr int AV_C = 1 << 3;   // above-right
constexpr int AV_D = 1 << 4;   // above-left

__device__ __forceinline__ int neighbour_mask(const int* slice, int k, int cols, int rows)
{
    int r = k / cols, c = k - r * cols;
    int sk = slice ? slice[k] : 0;
    auto ok = [&](int rr, int cc) { return rr >= 0 && rr < rows && cc >= 0 && cc < cols && (!slice || slice[rr * cols + cc] == sk); };
    return (ok(r, c - 1) ? AV_A : 0) | (ok(r - 1, c) ? AV_B : 0) | (ok(r - 1, c + 1) ? AV_C : 0) |
           (ok(r - 1, c - 1) ? AV_D : 0);
}

// Median of the packed neighbour vectors under the availability mask.
__device__ __forceinline__ void median_from(int av, int A, int B, int C, int D, int* px, int* py)
{
    if (!(av & AV_A)) A = 0;
    if (!(av & AV_B)) B = 0;
    if (av & AV_C) {
    } else if (av & AV_D) {
        C = D;
    } else {
        C = 0;
    }
    if (!(av & AV_B) && !(av & AV_C)) B = C = A;
    *px = median3(mv_x(A), mv_x(B), mv_x(C));
    *py = median3(mv_y(A), mv_y(B), mv_y(C));
}

// Same median on packed vectors (x in the low, y in the high signed 16-bit
// half): per-half min/max, the packed result equals pack_mv(px, py).
__device__ __forceinline__ int median_packed(int av, int A, int B, int C, int D)
{
    if (!(av & AV_A)) A = 0;
    if (!(av & AV_B)) B = 0;
    C = (av & AV_C) ? C : ((av & AV_D) ? D : 0);
    if (!(av & AV_B) && !(av & AV_C)) B = C = A;
    const unsigned a = (unsigned)A, b = (unsigned)B, c = (unsigned)C;
    return (int)__vmaxs2(__vmins2(a, b), __vmins2(__vmaxs2(a, b), c));
}

// From the current vectors in global memory (L2, bypassing L1: other SMs update them).
__device__ __forceinline__ void median_pred(const int* final_mv, int av, int k, int cols, int* px, int* py)
{
    int A = (av & AV_A) ? __ldcg(final_mv + k - 1) : 0;
    int B = (av & AV_B) ? __ldcg(final_mv + k - cols) : 0;
    int C = (av & AV_C) ? __ldcg(final_mv + k - cols + 1) : 0;
    int D = (!(av & AV_C) && (av & AV_D)) ? __ldcg(final_mv + k - cols - 1) : 0;
    median_from(av, A, B, C, D, px, py);
}

// Flag word accesses ordered against the data they publish (device scope).
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Nearest full-pel prediction with C division (Full.cpp:368-380).
__device__ __forceinline__ int round_pred(int p) { return p < 0 ? (p - 2) / 4 : (p + 2) / 4; }

// GetBestVector over the Fifo slots (best, pred, zero, zero, zero)
// (include/CodecUtils/MotionEstimatorH264ImplFull.h:140-168): cost =
// D/norm + lambda*sqrt(|v-ref|^2) in IEEE double, one rounding per
// operation, strict improvement.  Returns the winning slot 0..2.
static __device__ __noinline__ int best_of3(int bx, int by, int bd, int px, int py, int pd, int zd, double lambda,
                                        double norm, int xref, int yref)
{
    auto cost = [&](int x, int y, int d) {
        double m = (double)((x - xref) * (x - xref) + (y - yref) * (y - yref));
        return __dadd_rn(__ddiv_rn((double)d, norm), __dmul_rn(lambda, __dsqrt_rn(m)));
    };
    double c0 = cost(bx, by, bd);
    int pos = 0;
    double c1 = cost(px, py, pd);
    if (c1 < c0) {
        c0 = c1;
        pos = 1;
    }
    double c2 = cost(0, 0, zd);
    if (c2 < c0) pos = 2;
    return pos;
}

// Same decision without FP64 in the common cases (norm a power of two: 256,
// or 64 for the Cross estimator).  Two costs with the same sqrt argument
// differ only in D/norm, and D/norm is exact; with |lambda| <
// 2^20 every sum stays below 2^40, where costs 1/norm apart never round
// together, so their double order is the order of the integers D.  This
// covers the most frequent near-tie, the prediction slot against a searched
// vector equal to it.  Other pairs compare in float: each float cost is
// within a few ulp of the exact real value and the double costs within 2^-50
// relative, so when a pair differs by more than 2^-18 relative both orderings
// agree with the exact one; closer pairs take the double path.
__device__ __forceinline__ int best_of3_fast(int bx, int by, int bd, int px, int py, int pd, int zd, double lambda,
                                             int xref, int yref, int norm = 256)
{
    const int m0 = (bx - xref) * (bx - xref) + (by - yref) * (by - yref);
    const int m1 = (px - xref) * (px - xref) + (py - yref) * (py - yref);
    const int m2 = xref * xref + yref * yref;
    const float lf = (float)lambda, inv = 1.0f / (float)norm;
    const float c0 = (float)bd * inv + lf * sqrtf((float)m0);
    const float c1 = (float)pd * inv + lf * sqrtf((float)m1);
    const float c2 = (float)zd * inv + lf * sqrtf((float)m2);
    bool slow = false;
    const bool small_lambda = fabs(lambda) < 1048576.0;
    // strict "cost a < cost b" in the double arithmetic of best_of3
    auto less = [&](int da, int ma, float ca, int db, int mb, float cb) {
        if (ma == mb && small_lambda) return da < db;
        if (fabsf(ca - cb) <= 4e-6f * fmaxf(fabsf(ca), fabsf(cb)) + 1e-30f) slow = true;
        return ca < cb;
    };
    int pos = less(pd, m1, c1, bd, m0, c0) ? 1 : 0;
    const bool z = pos == 0 ? less(zd, m2, c2, bd, m0, c0) : less(zd, m2, c2, pd, m1, c1);
    if (slow) return best_of3(bx, by, bd, px, py, pd, zd, lambda, (double)norm, xref, yref);
    return z ? 2 : pos;
}

// ---------------------------------------------------------------------------
// Shared-memory barriers (mbarrier) and bulk / tensor copies, for the kernels
// that stage data asynchronously.  Every wait on them is bounded by the caller.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// One arrival that also expects `bytes` of copy completions in this phase.
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// One arrival (release: this thread's earlier shared-memory accesses are
// ordered before a successful wait on the phase).
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
// True once the phase of parity `parity` has completed (acquire).
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// One bulk copy global -> shared, completion counted on `bar` (16-byte
// aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar)
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// One 2-D tensor copy global -> shared (the box of `map` at element
// coordinates (x, y)), completion counted on `bar`.  x times the element size
// must be a multiple of 16 bytes; dst 128-byte aligned.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, int x, int y, unsigned long long* bar)
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// H.263 half-pel samples of four bytes (OverlayMem2Dv2::HalfRead) from the
// samples a (the block's), b (beside it), c (below or above it) and d (both):
// the rounded mean of a and its one neighbour on the horizontal or vertical
// lines, (a + b + c + d + 2) / 4 on the diagonals, evaluated in 16-bit lanes.
__device__ __forceinline__ unsigned half4(unsigned a, unsigned b, unsigned c, unsigned d, int hx, int hy)
{
    if (!hy) return __vavgu4(a, b);
    if (!hx) return __vavgu4(a, c);
    const unsigned m = 0x00ff00ffu;
    const unsigned lo = (a & m) + (b & m) + (c & m) + (d & m) + 0x00020002u;
    const unsigned hi = ((a >> 8) & m) + ((b >> 8) & m) + ((c >> 8) & m) + ((d >> 8) & m) + 0x00020002u;
    return ((lo >> 2) & m) | (((hi >> 2) & m) << 8);
}

// Four bytes at any offset of a row (shared or global memory: the aligned word after the
// one holding p must be readable).
__device__ __forceinline__ unsigned word_at(const unsigned char* p)
{
    const unsigned* w = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
    return __funnelshift_r(w[0], w[1], sh);
}

}  // namespace vppgpu
