// me_full_common.cuh -- pieces shared by the full-search kernels (search,
// resolve, wavefront): table geometry, the search range of
// MotionEstimatorH264ImplFull::GetMotionRange and the sequential scan replay.
#pragma once

#include "me_common.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace full {

constexpr int RMAX = 31;       // table geometry: i in [-31,31] -> ii = i+31, j -> jj = j+32
constexpr int WROWS = 84;      // window rows m-34 .. m+49
constexpr int WSTRIDE = 112;   // window cols n-48 .. n+63
constexpr int H2STRIDE = 81;   // odd stride: conflict-free column walks
constexpr int TAB = 64;        // SSD table is TAB x TAB ints
constexpr int FLAG_TIE = 1;


// GetMotionRange with zero offset (Full.cpp:1029-1081).
__device__ __forceinline__ void full_range(int n, int m, int W, int H, int motion_range, int& xl, int& xr, int& yu,
                                           int& yd)
{
    // Estimate asks for range = vecRange = motion_range/4 with zero offset, so
    // both vector limits resolve to vecRange - 1 (Full.cpp:1046-1061).
    int vr = motion_range / 4;
    int lr = vr - 1, rr = vr - 1;
    const int boundary = 16;
    xl = (n - lr >= -boundary) ? -lr : -(n + boundary);
    xr = (n + rr < W) ? rr : W - n;
    yu = (m - lr >= -boundary) ? -lr : -(m + boundary);
    yd = (m + rr < H) ? rr : H - m;
}

// Sequential raster replay of the integer search over tab (ii = i+31,
// jj = j+32), one warp.  prx/pry: rounded prediction used at ties.  Returns
// the winner and sets *tie when any exact tie was decided.
template <typename TabT>
__device__ __forceinline__ void scan_table(const TabT& tab, int xl, int xr, int yu, int yd, int prx, int pry,
                                           int lane, int* omx, int* omy, int* omin, int* tie)
{
    int minD = tab(RMAX, RMAX + 1), mx = 0, my = 0, t = 0;
    for (int i = yu; i <= yd; i++) {
        for (int base = xl; base <= xr; base += 32) {
            int j = base + lane;
            bool valid = (j <= xr) && !(i == 0 && j == 0);
            int d = valid ? tab(i + RMAX, j + RMAX + 1) : 0x7fffffff;
            unsigned pending = 0xffffffffu;
            while (true) {
                bool ok = valid && d <= minD && (i + my >= yu) && (i + my <= yd) && (j + mx >= xl) && (j + mx <= xr);
                unsigned m = __ballot_sync(0xffffffffu, ok) & pending;
                if (!m) break;
                int f = __ffs(m) - 1;
                int df = __shfl_sync(0xffffffffu, d, f);
                int jf = base + f;
                bool accept = true;
                if (df == minD) {
                    t = 1;
                    int cx = mx - prx, cy = my - pry, nx = jf - prx, ny = i - pry;
                    accept = (cy * cy + cx * cx) - (ny * ny + nx * nx) >= 0;
                }
                if (accept) {
                    minD = df;
                    mx = jf;
                    my = i;
                }
                pending &= ~((2u << f) - 1u);
                if (f == 31) break;
            }
        }
    }
    *omx = mx;
    *omy = my;
    *omin = minD;
    *tie = t;
}

struct SmemTab {
    const int (*t)[TAB];
    __device__ int operator()(int r, int c) const { return t[r][c]; }
};
struct GlobalTab {
    const int* t;
    __device__ int operator()(int r, int c) const { return __ldcg(t + r * TAB + c); }
};


}  // namespace full
}  // namespace vppgpu
