// Square-root-free bound of the sweep screens (used by the fused, local and
// boxed screens and the batched CTA sweep).
//
// A pair (i, c) can only be chosen if its exact delta is <= B, the best exact
// delta this thread has seen (B <= -1).  With d1 = nint d(i, c) and
// d2 = nint d(i-1, c-1), delta = d1 + d2 - e[i] - e[c] <= B and d1, d2 >= 0
// imply  d1 <= V  and  d2 <= V,  V = B + e[i] + e[c].
// For the per-edge nint,  nint(sqrt(s)) <= V  implies
//     s_approx < (V + 0.5)^2 (1 + 2^-21)
// (the correctly rounded root is below V + 0.5; the contracted sum of squares
// s_approx is within 2^-22 of the binary32 one), and that is below
//     L = RN(u * |u|),  u = V + 5,
// for every V <= 1.6e7 (here V <= 4e6: the coordinate box diagonal is below
// 2e6, so every edge is below 2e6).  A negative u makes L negative, so such
// pairs never pass.  A screen therefore needs one sum of squares per
// distance-matrix entry (each entry serves two pairs) and, per pair,
//     u = B + e[i] + 5 + e_c,  L = u * |u|,  max(s(i,c), s(i-1,c-1)) < L
// -- no square root and no MUFU work.  Pairs that pass are re-evaluated
// exactly (exact_dist), so the chosen move is still the exact lowest
// (delta, i, c).
#pragma once
#include "logo_device.cuh"

namespace logo {

__device__ __forceinline__ float sq_dist(float ax, float ay, float bx, float by) {
    const float dx = ax - bx;
    const float dy = ay - by;
    return __fmaf_rn(dy, dy, dx * dx);
}

}  // namespace logo
