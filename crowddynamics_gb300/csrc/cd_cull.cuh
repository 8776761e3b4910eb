// cd_cull.cuh -- the float32 pre-checks that skip agent pairs and wall
// segments whose float64 evaluation the reference would discard (shared by
// the step kernels and the adjoint; not part of the ABI).
//
// Soundness at any coordinates.  The pre-check records hold positions
// relative to the scenario's grid origin (float64 difference, then rounded to
// float32), walls likewise.  Rounding a coordinate of magnitude M moves it by
// at most 2^-24 M, and the tests' subtractions add as much again, so every
// agent record's extent is raised by CULL_MAG (|x| + |y|) = 8 x 2^-24 per unit
// of its own magnitude, and every wall test by WALL_MAG times the sum of its
// endpoints' magnitudes (16 x 2^-24, covering the endpoints, the tangent and
// the projection).  CULL_MARGIN covers the rounding of the tests' own
// products, relative to distances of a few metres.  Inside a grid of a few
// kilometres the raised extents differ from the bare ones by under a
// millimetre; an agent far from its grid only gets a wider cull, never a
// wrong one.
//
// Positions farther than COORD_MAX from the grid origin are reported by the
// step (ERR_RANGE): the float32 hi + lo representation of a position that the
// ThreeCircle certificates use is exact to 2^-48 of the coordinate, 3.6e-8 m
// at COORD_MAX, well inside the 1e-6 m their margins allow for it.
#pragma once
#include <cuda_runtime.h>

namespace cdk {

constexpr float CULL_MARGIN = 0.01f;           // metres
constexpr float CULL_MAG = 4.76837158e-7f;     // 2^-21
constexpr float WALL_MAG = 9.53674316e-7f;     // 2^-20
constexpr double COORD_MAX = 1e7;              // metres from the grid origin
constexpr float CULL_SIGHT = 3.0f;             // core/interactions.py:45

// Extent slack of a record at (xf, yf) (relative float32 position); 0 for a
// non-finite position, whose pairs no test certifies anyway.
__host__ __device__ __forceinline__ float cull_slack(float xf, float yf) {
    const float m = fabsf(xf) + fabsf(yf);
    return m <= 3.0e38f ? m * CULL_MAG : 0.f;
}

// True if the pair certainly has skin distance >= 3 m.  Symmetric in its
// arguments (the two extents are added first), so both agents of a pair
// agree on it.  False for NaN.
__device__ __forceinline__ bool pair_far(float4 me, float4 o) {
    const float dx = me.x - o.x, dy = me.y - o.y;
    const float lim = (me.z + o.z) + (CULL_SIGHT + CULL_MARGIN);
    return dx * dx + dy * dy > lim * lim;
}

// True if the centre-to-segment distance certainly exceeds `reach` (the
// agent's raised extent).  False for NaN.
__device__ __forceinline__ bool wall_far(float x, float y, float reach, float4 w) {
    const float dx = w.z - w.x, dy = w.w - w.y;
    const float qx = x - w.x, qy = y - w.y;
    const float dd = dx * dx + dy * dy;
    const float t = dd > 0.f ? fminf(fmaxf((qx * dx + qy * dy) / dd, 0.f), 1.f) : 0.f;
    const float rx = qx - t * dx, ry = qy - t * dy;
    const float wm = (fabsf(w.x) + fabsf(w.y)) + (fabsf(w.z) + fabsf(w.w));
    const float lim = (reach + CULL_MARGIN) + wm * WALL_MAG;
    return rx * rx + ry * ry > lim * lim;
}

}  // namespace cdk
