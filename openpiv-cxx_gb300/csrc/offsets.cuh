// offsets.cuh -- window offsetting of the multi-pass schedule (device side).
//
// Pass k > 0 moves frame B's window of every pass-k window by the integer
// displacement D of the previous pass's window whose centre is nearest
// (index = clamp(floor((c - c0 + step/2) / step), 0, n - 1) per axis), and
// clamps the move so that the window stays inside the image.  The integer
// displacement a pass hands on is D = (px - W/2 + ox, py - W/2 + oy) for a
// window whose first peak is at (px, py) of the quadrant-swapped plane, or
// (ox, oy) when it has fewer than two peaks.  Integer peaks are identical to
// the reference's, so the whole chain is reproducible exactly.
#pragma once
#include "piv_kernels.h"

namespace opiv {

__device__ __forceinline__ int nearest_index(int c, int c0, int step, int n)
{
    if (c < c0) return 0;
    const int i = (c - c0 + step / 2) / step;
    return i < n - 1 ? i : n - 1;
}

__device__ __forceinline__ void b_offset(const PivParams& p, int W, int bx, int by, int& ox, int& oy)
{
    ox = 0;
    oy = 0;
    if (p.prev_disp == nullptr) return;
    const int ix = nearest_index(bx + W / 2, p.pgx0 + p.pw / 2, p.pgdx, p.pgnx);
    const int iy = nearest_index(by + W / 2, p.pgy0 + p.pw / 2, p.pgdy, p.pgny);
    const int32_t d = p.prev_disp[iy * p.pgnx + ix];
    const int dx = (int)(int16_t)(d & 0xffff), dy = d >> 16;
    const int lox = -bx, hix = p.img_w - W - bx, loy = -by, hiy = p.img_h - W - by;
    ox = dx < lox ? lox : (dx > hix ? hix : dx);
    oy = dy < loy ? loy : (dy > hiy ? hiy : dy);
}

__device__ __forceinline__ int32_t pack_disp(int dx, int dy)
{
    return (int32_t)(((uint32_t)dy << 16) | ((uint32_t)dx & 0xffffu));
}

}  // namespace opiv
