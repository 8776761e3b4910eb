// cd_kernels.cu -- device kernels of libcdgpu (sm_103a, float64 arithmetic).
//
// One step of the reference's MultiAgentSimulation.update()
// (crowddynamics/simulation/multiagent.py:51-55) runs as:
//   prepare  : cell key + per-cell count of every agent, per-scenario max |v|
//   dt       : adaptive timestep per scenario (core/integrator.py:29-97)
//   scan     : exclusive prefix sum of cell counts -> cell start offsets
//   scatter  : agents into cells (atomic), then a stable per-cell rank so that
//              each cell lists its agents in ascending index order
//   gather   : cell-sorted staging copy of the fields the pair loop reads, plus
//              a float32 (x, y, extent) record for the conservative pre-check
//   forces   : per agent: noise + orientation + adjusting + agent-agent +
//              agent-wall, then velocity Verlet, shoulders and reset
//
// The library is compiled without fused multiply-add contraction and uses the
// elementary functions of cd_math.h, so every float64 result rounds exactly
// as the oracle's does; agent-agent contributions are summed per agent in the
// reference's visiting order (3 x 3 cells in (dx, dy) lexicographic order,
// each cell in ascending agent order), so a step is bit-identical to the
// oracle's and multi-step rollouts stay identical.
//
// Float64 is the only arithmetic that reaches a result.  Float32 is used for
// one thing: skipping agent pairs (and wall segments) whose centre distance
// exceeds the social cut-off plus both extents by a margin far above float32
// rounding, i.e. pairs the reference evaluates to exactly no contribution.
#include <cstdint>
#include <algorithm>
#include <cmath>
#include <cuda_fp16.h>
#include "cd_internal.cuh"
#include "cd_cull.cuh"
#include "cd_math.h"
#include "cd_noise.h"

namespace cdk {

namespace {

constexpr double SIGTH_SOC = 3.0;      // core/interactions.py:45
constexpr double F_SOC_MAX = 2e3;      // core/motion/power_law.py:52
constexpr double TAU_MAX = 30.0;       // core/motion/power_law.py:243
constexpr double PI_D = 3.141592653589793;

// ---- float64 helpers restating core/vector2D.py ------------------------

// Python float modulo (numba follows CPython's float_rem).
__device__ __forceinline__ double py_mod(double x, double y) {
    double m = fmod(x, y);
    if (m != 0.0) {
        if ((y < 0) != (m < 0)) m += y;
    } else {
        m = copysign(0.0, y);
    }
    return m;
}

// wrap_to_pi, core/vector2D.py:8-36
__device__ __forceinline__ double wrap_to_pi(double rad) {
    double r = py_mod(rad, 2 * PI_D);
    if (rad < 0 && r == PI_D) return -PI_D;
    if (r > PI_D) return r - (2 * PI_D);
    return r;
}

__device__ __forceinline__ double np_sign(double x) {
    return x > 0 ? 1.0 : (x < 0 ? -1.0 : x);
}

// truncate, core/vector2D.py:166-187.  A vector whose float64 squared
// length is below 0.99 l^2 is certainly shorter than l (the sum of two
// rounded squares is within 3 units in the last place of |v|^2), so the
// exact test would leave it as it is: it is returned without the hypot.
// NaN, infinite and overflowing squares take the exact test.
__device__ __forceinline__ void truncate2(double &vx, double &vy, double l) {
    if (vx * vx + vy * vy < 0.99 * (l * l)) return;
    double vlen = cdm_hypot(vx, vy);
    if (vlen > l) {
        double s = l / vlen;
        vx = vx * s;
        vy = vy * s;
    }
}

// magnitude, core/motion/power_law.py:83-102, with 1 / tau_0 (itau_0) the
// staged records' IEEE quotient: the same value, divided once per agent
__device__ __forceinline__ double magnitude(double tau, double tau_0, double itau_0) {
    return (2.0 / tau + itau_0) * cdm_exp(-tau / tau_0) / (tau * tau);
}

// force_contact, core/motion/contact.py:12-48; t = rotate270(n) = (n.y, -n.x)
__device__ __forceinline__ void force_contact(double h, double nx, double ny,
                                              double vx, double vy, double mu,
                                              double kappa, double damping,
                                              double &cx, double &cy) {
    double tx = ny, ty = -nx;
    double vt = vx * tx + vy * ty;
    double vn = vx * nx + vy * ny;
    cx = (-h) * (mu * nx - (kappa * vt) * tx) + (damping * vn) * nx;
    cy = (-h) * (mu * ny - (kappa * vt) * ty) + (damping * vn) * ny;
}

// Ordered-bits encoding of a non-negative double for atomicMax.
__device__ __forceinline__ unsigned long long ord_bits(double v) {
    return (unsigned long long)__double_as_longlong(v);
}

__device__ __forceinline__ int axis_cell(double v, double v0, double cell, int n) {
    double q = floor((v - v0) / cell);
    if (q < 0.0) return 0;
    if (q > (double)(n - 1)) return n - 1;
    return (int)q;
}

// ---- staged agent records ----------------------------------------------

struct Circ {
    double x, y, vx, vy, r, m, k, tau0, mu, kappa, damp, itau0;   // itau0 = 1.0 / tau0
};

struct TC {
    double x[3], y[3];          // torso, left shoulder, right shoulder
    double vx, vy, rt, rs, rts, m, k, tau0, mu, kappa, damp, sn, cs, itau0;   // itau0 = 1 / tau0
};

// Register-friendly selection of part k (0 torso, 1 left, 2 right).
__device__ __forceinline__ double sel3(const double v[3], int k) {
    return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]);
}

__device__ __forceinline__ Circ load_circ(const double2 *__restrict__ st, int slot) {
    const double2 *p = st + (size_t)slot * STAGE_Q_CIRC;
    double2 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3),
            q4 = __ldg(p + 4), q5 = __ldg(p + 5);
    Circ a;
    a.x = q0.x; a.y = q0.y; a.vx = q1.x; a.vy = q1.y; a.r = q2.x; a.m = q2.y;
    a.k = q3.x; a.tau0 = q3.y; a.mu = q4.x; a.kappa = q4.y; a.damp = q5.x; a.itau0 = q5.y;
    return a;
}

__device__ __forceinline__ TC load_tc(const double2 *__restrict__ st, int slot) {
    const double2 *p = st + (size_t)slot * STAGE_Q_TC;
    double2 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3),
            q4 = __ldg(p + 4), q5 = __ldg(p + 5), q6 = __ldg(p + 6), q7 = __ldg(p + 7),
            q8 = __ldg(p + 8), q9 = __ldg(p + 9);
    TC a;
    a.x[0] = q0.x; a.y[0] = q0.y; a.x[1] = q1.x; a.y[1] = q1.y; a.x[2] = q2.x; a.y[2] = q2.y;
    a.vx = q3.x; a.vy = q3.y; a.rt = q4.x; a.rs = q4.y; a.rts = q5.x; a.m = q5.y;
    a.k = q6.x; a.tau0 = q6.y; a.mu = q7.x; a.kappa = q7.y; a.damp = q8.x; a.sn = q8.y;
    a.cs = q9.x;
    a.itau0 = q9.y;
    return a;
}

// ---- walls -------------------------------------------------------------

// distance_circle_line, core/distance.py:108-146 (wall tangent precomputed)
__device__ __forceinline__ double dist_circle_line(double x, double y, double r,
                                                   const double *w, double &nx,
                                                   double &ny) {
    double p0x = w[0], p0y = w[1], p1x = w[2], p1y = w[3];
    double tx = w[4], ty = w[5], l_w = w[6];
    double nwx = -ty, nwy = tx;                 // rotate90(t_w)
    double q0x = x - p0x, q0y = y - p0y;
    double q1x = x - p1x, q1y = y - p1y;
    double l_t = -(tx * q1x + ty * q1y) - (tx * q0x + ty * q0y);
    double d_iw;
    if (l_t > l_w) {
        d_iw = cdm_hypot(q0x, q0y);
        nx = q0x / d_iw; ny = q0y / d_iw;
    } else if (l_t < -l_w) {
        d_iw = cdm_hypot(q1x, q1y);
        nx = q1x / d_iw; ny = q1y / d_iw;
    } else {
        double l_n = nwx * q0x + nwy * q0y;
        d_iw = fabs(l_n);
        double s = np_sign(l_n);
        nx = s * nwx; ny = s * nwy;
    }
    return d_iw - r;
}

__device__ __forceinline__ void wall_circular(const Circ &A, const double *w,
                                              double &fx, double &fy) {
    double nx, ny;
    double h = dist_circle_line(A.x, A.y, A.r, w, nx, ny);
    if (h < 0) {
        double cx, cy;
        force_contact(h, nx, ny, A.vx, A.vy, A.mu, A.kappa, A.damp, cx, cy);
        fx += cx; fy += cy;
    }
}

// interaction_agent_three_circle_obstacle, core/interactions.py:123-141, with
// distance_three_circle_line, core/distance.py:149-180
__device__ __forceinline__ void wall_three_circle(const TC &A, const double *w,
                                                  double &fx, double &fy, double &tq) {
    double h_min = __longlong_as_double(0x7ff8000000000000LL);
    double nx = 0.0, ny = 0.0;
    int i_min = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double r = (i == 0) ? A.rt : A.rs;
        double mx, my;
        double h = dist_circle_line(A.x[i], A.y[i], r, w, mx, my);
        if (h < h_min || isnan(h_min)) { h_min = h; nx = mx; ny = my; i_min = i; }
    }
    if (h_min < 0) {
        double r = (i_min == 0) ? A.rt : A.rs;
        double rmx = (sel3(A.x, i_min) - r * nx) - A.x[0];
        double rmy = (sel3(A.y, i_min) - r * ny) - A.y[0];
        double cx, cy;
        force_contact(h_min, nx, ny, A.vx, A.vy, A.mu, A.kappa, A.damp, cx, cy);
        fx += cx; fy += cy;
        tq += rmx * cy - rmy * cx;
    }
}

// ---- kernels ------------------------------------------------------------

// Programmatic dependent launch, first statement of the step's chained
// kernels: wait until the kernel before this one on the stream has completed
// and its memory is visible (returns at once after an ordinary launch), then
// allow the next kernel's blocks to be scheduled beside this one's last
// blocks (they wait here in turn).

constexpr int PREP_NT = 256;                     // k_prepare's block size

__global__ void __launch_bounds__(PREP_NT) k_prepare(StepArgs a) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    // device fluctuation: this step's generator counter (read by the force stage)
    if (i == 0 && a.noise_dev && (a.nodes & N_FLUCT)) *a.rng_step += 1;
    if (i == 0 && a.fix_count) *a.fix_count = 0;   // agents the gather leaves for a redo
    int s = -1;
    double l = 0.0;
    if (i < a.n) {
        s = a.scen_of[i];
        const ScenDev sc = a.scen[s];
        double x = a.col[X][i], y = a.col[Y][i];
        int key = sc.cell_base;
        if (isfinite(x) && isfinite(y)) {
            key += axis_cell(x, sc.x0, sc.cell, sc.nx) * sc.ny + axis_cell(y, sc.y0, sc.cell, sc.ny);
            // the float32 pre-checks are sound within COORD_MAX of the origin
            if (!(fabs(x - sc.x0) <= COORD_MAX && fabs(y - sc.y0) <= COORD_MAX))
                atomicOr(a.err, ERR_RANGE);
        } else {
            atomicOr(a.err, ERR_NOT_FINITE);
        }
        a.key[i] = key;
        atomicAdd(&a.count[key], 1);
        l = cdm_hypot(a.col[VX][i], a.col[VY][i]);      // length(velocity)
    }
    // per-scenario max |v| (NaN and 0 ignored, like `if l > v_max`): one
    // atomic per block when its agents share a scenario (fmax is exact, so
    // the order does not matter)
    __shared__ int s_block;
    __shared__ double wmax[PREP_NT / 32];
    if (threadIdx.x == 0) s_block = s;
    __syncthreads();
    if (__syncthreads_and(s == s_block || s < 0)) {
        double m = (l > 0) ? l : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            const double t = __shfl_xor_sync(0xffffffffu, m, o);
            m = (t > m) ? t : m;
        }
        if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x < 32) {
            m = threadIdx.x < PREP_NT / 32 ? wmax[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) {
                const double t = __shfl_xor_sync(0xffffffffu, m, o);
                m = (t > m) ? t : m;
            }
            if (threadIdx.x == 0 && s_block >= 0 && m > 0) atomicMax(&a.vmax[s_block], ord_bits(m));
        }
    } else if (s >= 0 && l > 0) {
        atomicMax(&a.vmax[s], ord_bits(l));
    }
}

// adaptive_timestep, core/integrator.py:29-97; accumulates time_tot.
__device__ __forceinline__ void scenario_dt(const StepArgs &a, int s) {
    const ScenDev sc = a.scen[s];
    double v_max = __longlong_as_double((long long)a.vmax[s]);
    double dt;
    if (v_max == 0.0) {
        dt = sc.dt_max;
    } else {
        double c = 1.1;
        double dx_max = c * a.v0max[s] * sc.dt_max;
        double t = dx_max / v_max;
        if (t > sc.dt_max) dt = sc.dt_max;
        else if (t < sc.dt_min) dt = sc.dt_min;
        else dt = t;
    }
    a.dt[s] = dt;
    a.time_tot[s] += dt;
}

__global__ void k_dt(StepArgs a) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.n_scen) scenario_dt(a, s);
}

// Per-scenario max target_velocity (NaN if any is NaN, like numpy's max) and
// max agent extent (finite values only) in two passes: up to V0MAX_B blocks
// per scenario (about two agents per thread at the mean scenario size) write
// partials, then one warp per scenario combines them.  fmax is exact, so the
// result does not depend on the order.
constexpr int V0MAX_B = 256;

__device__ __forceinline__ double extent_tc(double x, double y, double xl, double yl,
                                            double xr, double yr, double rt, double rs);

// Wall-binning extent of an agent: ThreeCircle also counts r_ts + r_s, the
// shoulders' reach at any orientation.
__device__ __forceinline__ double extent_of(double *const *c, int body, int i) {
    if (body == 0) return c[R][i];
    const double e = extent_tc(c[X][i], c[Y][i], c[XLS][i], c[YLS][i], c[XRS][i], c[YRS][i],
                               c[RT][i], c[RS][i]);
    return fmax(e, c[RTS][i] + c[RS][i]);
}
__device__ __forceinline__ double agent_extent(const StepArgs &a, int i) {
    return extent_of(a.col, a.body, i);
}

__global__ void k_scen_max_partial(StepArgs a, double *partial) {
    const int s = blockIdx.y;
    const ScenDev sc = a.scen[s];
    __shared__ double rv[256], re[256];
    __shared__ int any_nan;
    if (threadIdx.x == 0) any_nan = 0;
    __syncthreads();
    double m = -INFINITY, e = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < sc.agent_count;
         k += gridDim.x * blockDim.x) {
        const int i = sc.agent_begin + k;
        const double v = a.col[V0][i];
        if (isnan(v)) any_nan = 1;
        else m = fmax(m, v);
        const double x = agent_extent(a, i);
        if (isfinite(x)) e = fmax(e, x);
    }
    rv[threadIdx.x] = m;
    re[threadIdx.x] = e;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            rv[threadIdx.x] = fmax(rv[threadIdx.x], rv[threadIdx.x + o]);
            re[threadIdx.x] = fmax(re[threadIdx.x], re[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *p = partial + 2 * ((size_t)s * gridDim.x + blockIdx.x);
        p[0] = any_nan ? __longlong_as_double(0x7ff8000000000000LL) : rv[0];
        p[1] = re[0];
    }
}

__global__ void k_scen_max_final(const double *partial, int nb, int n_scen, double *v0max,
                                 double *ext) {
    const int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (s >= n_scen) return;
    double m = -INFINITY, e = 0.0;
    bool nan = false;
    for (int b = lane; b < nb; b += 32) {
        const double *p = partial + 2 * ((size_t)s * nb + b);
        if (isnan(p[0])) nan = true;
        else m = fmax(m, p[0]);
        e = fmax(e, p[1]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
    }
    nan = __any_sync(0xffffffffu, nan);
    if (lane == 0) {
        v0max[s] = nan ? __longlong_as_double(0x7ff8000000000000LL) : m;
        if (ext) ext[s] = e;
    }
}

// -- exclusive scan (block-local, then block totals) --

constexpr int SCAN_NT = 1024, SCAN_IPT = 4, SCAN_TILE = SCAN_NT * SCAN_IPT;

// Up to three arrays of the same length scanned by one launch (blockIdx.y).
struct ScanSet { const int *in[3]; int *out[3]; int *sums[3]; };

__global__ void __launch_bounds__(SCAN_NT) k_scan_local(ScanSet S, int n) {
    pdl_enter();
    const int *in = S.in[blockIdx.y];
    int *out = S.out[blockIdx.y];
    int *blocksums = S.sums[blockIdx.y];
    __shared__ int wtot[SCAN_NT / 32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        sum += v[k];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wtot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = wtot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        wtot[lane] = x;
    }
    __syncthreads();
    int excl = incl - sum + (w > 0 ? wtot[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        if (base + k < n) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SCAN_NT - 1) {
        if (blocksums) blocksums[blockIdx.x] = excl;
        else out[n] = excl;           // single tile: total at out[n]
    }
}

// One block scanning n values in tiles, in turn: exclusive offsets into
// out[0, n); returns the total (the same in every thread).  Loads go through
// L2 only, so values other blocks of the same launch wrote are seen.
__device__ int scan_one_block(const int *in, int *out, int n) {
    __shared__ int wtot[SCAN_NT / 32];
    __shared__ int tile_total;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int carry = 0;
    for (int t0 = 0; t0 < n; t0 += SCAN_TILE) {
        const int base = t0 + threadIdx.x * SCAN_IPT;
        int v[SCAN_IPT];
        int sum = 0;
#pragma unroll
        for (int k = 0; k < SCAN_IPT; ++k) {
            v[k] = (base + k < n) ? __ldcg(in + base + k) : 0;
            sum += v[k];
        }
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wtot[w] = incl;
        __syncthreads();
        if (w == 0) {
            int x = wtot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += t;
            }
            wtot[lane] = x;
            if (lane == 31) tile_total = x;
        }
        __syncthreads();
        int excl = carry + incl - sum + (w > 0 ? wtot[w - 1] : 0);
#pragma unroll
        for (int k = 0; k < SCAN_IPT; ++k) {
            if (base + k < n) out[base + k] = excl;
            excl += v[k];
        }
        carry += tile_total;
        __syncthreads();                      // wtot and tile_total reused
    }
    return carry;
}

// One block scanning up to a few tiles in turn (one launch for small arrays).
__global__ void __launch_bounds__(SCAN_NT) k_scan_single(const int *in, int *out, int n) {
    pdl_enter();
    const int total = scan_one_block(in, out, n);
    if (threadIdx.x == 0) out[n] = total;
}

// Up to three arrays scanned by one launch, for the near lists: every tile
// writes its exclusive offsets relative to the tile and its total
// (sums[tile]); the last tile to finish (counted at sums[2 nb + 2]; no block
// waits for another) scans the totals into tile offsets (sums[nb + 1 + j]),
// writes the grand total at out[n] and re-arms the counter.  The near-list
// fill adds its agent's tile offset and writes the final offset back.
__global__ void __launch_bounds__(SCAN_NT) k_scan_tiles(ScanSet S, int n, int nb) {
    pdl_enter();
    const int *in = S.in[blockIdx.y];
    int *out = S.out[blockIdx.y];
    int *sums = S.sums[blockIdx.y];
    __shared__ int wtot[SCAN_NT / 32];
    __shared__ int last;
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        sum += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wtot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = wtot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        wtot[lane] = x;
    }
    __syncthreads();
    int excl = incl - sum + (w > 0 ? wtot[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        if (base + k < n) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SCAN_NT - 1) {
        sums[blockIdx.x] = excl;                        // the tile's total
        __threadfence();
        unsigned *done = reinterpret_cast<unsigned *>(sums + 2 * nb + 2);
        last = atomicAdd(done, 1u) == (unsigned)(nb - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int total = scan_one_block(sums, sums + nb + 1, nb);
    if (threadIdx.x == 0) {
        sums[nb + 1 + nb] = total;
        out[n] = total;
        sums[2 * nb + 2] = 0;
    }
}

__global__ void k_scan_add(ScanSet S, int n, int nb) {
    pdl_enter();
    int *out = S.out[blockIdx.y];
    const int *offs = S.in[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offs[i / SCAN_TILE];
    else if (i == n) out[n] = offs[nb];          // total
}

__global__ void k_scatter(StepArgs a) {
    pdl_enter();
    // the step's dt: k_prepare's max |v| is complete once this kernel runs
    // (then the max is used up: zero for the next cell list)
    if (blockIdx.x == 0)
        for (int sc = threadIdx.x; sc < a.n_scen; sc += blockDim.x) {
            if (a.nodes & N_INTEG) scenario_dt(a, sc);
            a.vmax[sc] = 0;
        }
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int c = a.key[i];
    int p = a.start[c] + atomicAdd(&a.fill[c], 1);
    a.perm_unsorted[p] = i;
}

// Extent: distance from the torso centre to the farthest skin point.
__device__ __forceinline__ double extent_tc(double x, double y, double xl, double yl,
                                            double xr, double yr, double rt, double rs) {
    double e = rt;
    double l = cdm_hypot(xl - x, yl - y) + rs;
    double r = cdm_hypot(xr - x, yr - y) + rs;
    e = (l > e) ? l : e;
    e = (r > e) ? r : e;
    return e;
}

// Velocity as two halves in one float's bits (the cull record's w): used
// only for the order of the flat pair list, never for a result.
__device__ __forceinline__ float pack_velocity(double vx, double vy) {
    const __half2 h = __floats2half2_rn((float)vx, (float)vy);
    return __uint_as_float(*reinterpret_cast<const unsigned *>(&h));
}
__device__ __forceinline__ float2 unpack_velocity(float w) {
    const unsigned u = __float_as_uint(w);
    return __half22float2(*reinterpret_cast<const __half2 *>(&u));
}

__device__ __forceinline__ float up_f(double v) {
    float f = (float)v;
    return f + fabsf(f) * 1e-6f + 1e-6f;
}

// The staged records of agent i in its cell-sorted slot s.  `part`: 0 all
// records; 1 the float32 pre-check records only (all the near-list build
// reads); 2 the float64 staged records only.
__device__ __forceinline__ void gather_agent(const StepArgs &a, const int i, const int s,
                                             const int part) {
    double *const *c = a.col;
    // pre-check records: positions relative to the scenario's grid origin
    // (cd_cull.cuh); the staged float64 records keep the reference's values
    const ScenDev *sc = a.scen + __ldg(&a.scen_of[i]);
    const double ox = __ldg(&sc->x0), oy = __ldg(&sc->y0);
    if (a.body == 0) {
        if (part != 1) {
            double2 *p = a.stage + (size_t)s * STAGE_Q_CIRC;
            p[0] = make_double2(c[X][i], c[Y][i]);
            p[1] = make_double2(c[VX][i], c[VY][i]);
            p[2] = make_double2(c[R][i], c[MASS][i]);
            p[3] = make_double2(c[K_SOC][i], c[TAU0][i]);
            p[4] = make_double2(c[MU][i], c[KAPPA][i]);
            p[5] = make_double2(c[DAMP][i], 1.0 / c[TAU0][i]);
        }
        if (part != 2) {
            const double xr = c[X][i] - ox, yr = c[Y][i] - oy;
            const float xf = (float)xr, yf = (float)yr;
            a.cull[s] = make_float4(xf, yf, up_f(c[R][i]) + cull_slack(xf, yf),
                                    pack_velocity(c[VX][i], c[VY][i]));
            // position = float hi (cull) + float lo, and the radius, for the
            // float32 pair pass (circ_pair_light)
            a.stage_f[2 * s] = make_float4((float)(xr - (double)xf), (float)(yr - (double)yf),
                                           (float)c[R][i], 0.f);
        }
    } else {
        double x = c[X][i], y = c[Y][i];
        if (part != 1) {
            double2 *p = a.stage + (size_t)s * STAGE_Q_TC;
            p[0] = make_double2(x, y);
            p[1] = make_double2(c[XLS][i], c[YLS][i]);
            p[2] = make_double2(c[XRS][i], c[YRS][i]);
            p[3] = make_double2(c[VX][i], c[VY][i]);
            p[4] = make_double2(c[RT][i], c[RS][i]);
            p[5] = make_double2(c[RTS][i], c[MASS][i]);
            p[6] = make_double2(c[K_SOC][i], c[TAU0][i]);
            p[7] = make_double2(c[MU][i], c[KAPPA][i]);
            double sn, cs;
            cdm_sincos(c[PHI][i], &sn, &cs);
            p[8] = make_double2(c[DAMP][i], sn);
            p[9] = make_double2(cs, 1.0 / c[TAU0][i]);
        }
        if (part == 2) return;
        // position relative to the grid origin = float hi + float lo;
        // shoulder centres relative to the torso
        const double xr = x - ox, yr = y - oy;
        const float xh = (float)xr, yh = (float)yr;
        const float oxl = (float)(c[XLS][i] - x), oyl = (float)(c[YLS][i] - y);
        const float oxr = (float)(c[XRS][i] - x), oyr = (float)(c[YRS][i] - y);
        const float rtf = (float)c[RT][i], rsf = (float)c[RS][i];
        a.stage_f[2 * s] = make_float4((float)(xr - (double)xh), (float)(yr - (double)yh), rtf, rsf);
        a.stage_f[2 * s + 1] = make_float4(oxl, oyl, oxr, oyr);
        // extent (extent_tc) in float32 from the same offsets: its error is
        // below 1e-6 relative, the 1e-5 added makes it an upper bound, which
        // is all the pre-check records need; raised by the position's slack
        const float ef = fmaxf(rtf, fmaxf(sqrtf(oxl * oxl + oyl * oyl) + rsf,
                                          sqrtf(oxr * oxr + oyr * oyr) + rsf));
        a.cull[s] = make_float4(xh, yh, (ef + ef * 1e-5f + 1e-5f) + cull_slack(xh, yh),
                                pack_velocity(c[VX][i], c[VY][i]));
    }
}

// One lane per agent where the slots are known (column reads coalesced, the
// staged records written whole), else one lane per slot.
__global__ void k_gather(StepArgs a, int part) {
    pdl_enter();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    int s, i;
    if (a.slot_of) { i = t; s = a.slot_of[t]; }
    else { s = t; i = a.perm[t]; }
    gather_agent(a, i, s, part);
}

// Stable order inside a cell: the rank of agent i is the number of agents of
// its cell with a smaller index.  One lane per agent (its columns read
// coalesced); with part >= 0 it also writes the agent's staged records
// (gather_agent) at its slot, so no separate gather runs.
__global__ void k_rank(StepArgs a, int part) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int c = a.key[i];
    const int b = a.start[c], e = a.start[c + 1];
    int r = 0;
    for (int q = b; q < e; ++q) r += (a.perm_unsorted[q] < i);
    const int s = b + r;
    a.perm[s] = i;
    if (a.slot_of) a.slot_of[i] = s;
    // the cell's count and fill are used up: zero for the next cell list
    if (r == 0) {
        a.count[c] = 0;
        a.fill[c] = 0;
    }
    if (part >= 0) gather_agent(a, i, s, part);
}

// Candidate enumeration over the 3 x 3 cell neighbourhood of slot s.  The
// pair (s, t) is oriented with s first iff t is later in the same cell or t's
// cell is in the forward half of the stencil (flat offset dx*ny + dy > 0).
// Calls fn(t, s_is_first) for every candidate that survives the pre-check;
// counts all candidates in *cand.
template <typename Fn>
__device__ __forceinline__ void for_candidates(const StepArgs &a, const ScenDev &sc, int s,
                                               int my_cell, float4 me, Fn fn, int *cand) {
    int local = my_cell - sc.cell_base;
    int ix = local / sc.ny, iy = local - ix * sc.ny;
    for (int dx = -1; dx <= 1; ++dx) {
        int jx = ix + dx;
        if (jx < 0 || jx >= sc.nx) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int jy = iy + dy;
            if (jy < 0 || jy >= sc.ny) continue;
            int c2 = sc.cell_base + jx * sc.ny + jy;
            int b = __ldg(&a.start[c2]), e = __ldg(&a.start[c2 + 1]);
            bool fwd = (dx > 0) || (dx == 0 && dy > 0);
            bool same = (dx == 0 && dy == 0);
            for (int t = b; t < e; ++t) {
                if (t == s) continue;
                if (cand) ++*cand;
                float4 o = __ldg(&a.cull[t]);
                if (pair_far(me, o)) continue;
                fn(t, same ? (s < t) : fwd);
            }
        }
    }
}

// ---- agent-agent evaluation in the calling agent's frame -------------------
//
// The reference evaluates pair (i, j) once with i the owner and adds force_i
// to i and force_j to j.  Each agent here evaluates its own side with
// relative quantities taken as (me - other).  Every shared quantity of the
// reference's (P, Q) frame is then either identical (a, b, c, disc, d, tau,
// h: products or sums of two negated values, sums of the same radii) or
// exactly negated (x_rel, v_rel, r_off, n, the gradient), because IEEE
// negation is exact.  Working it through the reference formulas, the calling
// agent's contribution is the same expression for both sides:
//   F = truncate((-m k) * grad_me * magnitude(tau, tau0_me)) + contact_me
//   r_moment = (X[part_me] + r_me[part_me] * n_me) - x_me_torso
// where X is the first agent's part positions (the reference takes
// r_moment1 from x0[j_min], core/distance.py:103).  Orientation therefore only
// decides the order in which the 3 x 3 sub-circle pairs are visited (first
// minimum of h, first defined root, strict "<" replacement), which follows
// the first agent's parts in the outer loop.

// Sequence position k (first agent's part k / 3, second's k % 3) to the
// calling agent's part (mine) and the other agent's part (theirs).
__device__ __forceinline__ void seq_parts(int k, bool me_first, int &mine, int &theirs) {
    int p = k / 3, q = k - 3 * (k / 3);
    mine = me_first ? p : q;
    theirs = me_first ? q : p;
}

__device__ __forceinline__ double part_r(const TC &A, int k) { return k == 0 ? A.rt : A.rs; }

// r_off contribution of one agent's contact part: +/- r_ts (sin phi, -cos phi)
// for the left / right shoulder, 0 for the torso (power_law.py:337-350).
__device__ __forceinline__ void r_off_part(const TC &A, int part, double &ox, double &oy) {
    double ex = A.rts * A.sn, ey = A.rts * (-A.cs);
    ox = part == 1 ? (0.0 + ex) : (part == 2 ? (0.0 - ex) : 0.0);
    oy = part == 1 ? (0.0 + ey) : (part == 2 ? (0.0 - ey) : 0.0);
}

// Circular pair, calling agent A, other agent B (interactions.py:51-70):
// A's force from the pair in (Fx, Fy); false when the pair does not interact
// (h >= sight_soc: the reference adds nothing).
__device__ __forceinline__ bool pair_circular_eval(const Circ &A, const Circ &B, double &Fx,
                                                   double &Fy) {
    Fx = 0.0;
    Fy = 0.0;
    double xx = A.x - B.x, xy = A.y - B.y;
    double d = cdm_hypot(xx, xy);
    double r_tot = A.r + B.r;
    double h = d - r_tot;
    if (!(h < SIGTH_SOC)) return false;
    double vrx = A.vx - B.vx, vry = A.vy - B.vy;
    double a = vrx * vrx + vry * vry;
    double b = -(xx * vrx + xy * vry);
    double c = (xx * xx + xy * xy) - r_tot * r_tot;
    double disc = b * b - a * c;
    if (disc > 0 && a != 0) {                     // isnan(d) or d == 0 or a == 0
        double dd = sqrt(disc);
        double tau = (b - dd) / a;
        if (!(tau <= 0 || tau > TAU_MAX)) {
            double gx = (vrx - (vrx * b + xx * a) / dd) / a;
            double gy = (vry - (vry * b + xy * a) / dd) / a;
            double cm = (-A.m) * A.k;
            double mag = magnitude(tau, A.tau0, A.itau0);
            Fx = (cm * gx) * mag;
            Fy = (cm * gy) * mag;
            truncate2(Fx, Fy, F_SOC_MAX);
        }
    }
    if (h < 0) {
        double nx = 0.0, ny = 0.0;
        if (d != 0.0) { nx = xx / d; ny = xy / d; }
        double cx, cy;
        force_contact(h, nx, ny, vrx, vry, A.mu, A.kappa, A.damp, cx, cy);
        Fx = Fx + cx;
        Fy = Fy + cy;
    }
    return true;
}

__device__ __forceinline__ void pair_circular_me(const Circ &A, const Circ &B, double &fx,
                                                 double &fy) {
    double Fx, Fy;
    if (pair_circular_eval(A, B, Fx, Fy)) {
        fx += Fx;
        fy += Fy;
    }
}

// Outcome of a pair evaluation: not interacting, interacting without a force
// on either side (each side's torque a signed zero), or with a force.
constexpr int RES_NONE = 0, RES_ZERO = 1, RES_FORCE = 2;
constexpr int RES_DEFER = 3;                // tc_pair_light: float64 needed

// Both forces of a Circular pair (interactions.py:51-70) with P = A the
// first agent of the pair (the lower cell-sorted slot) and Q = B: each side
// comes out exactly as pair_circular_eval computes it from that side (Q's
// relative position, velocity, tau gradient and normal are exact negations
// of P's), sharing the distance, the time-to-collision and its gradient.
// Two passes: circ_pair_decide returns RES_NONE, RES_ZERO or RES_FORCE with
// the distance, sqrt(D) and tau in a CircJob; circ_pair_force computes both
// forces from it.
struct CircJob {
    double d, dd, tau;          // |x_P - x_Q|, sqrt of the discriminant, time to collision
    bool social, contact;
};

__device__ __forceinline__ int circ_pair_decide(const Circ &A, const Circ &B, CircJob &J) {
    double xx = A.x - B.x, xy = A.y - B.y;
    double d = cdm_hypot(xx, xy);
    double r_tot = A.r + B.r;
    double h = d - r_tot;
    if (!(h < SIGTH_SOC)) return RES_NONE;
    double vrx = A.vx - B.vx, vry = A.vy - B.vy;
    double a = vrx * vrx + vry * vry;
    double b = -(xx * vrx + xy * vry);
    double c = (xx * xx + xy * xy) - r_tot * r_tot;
    double disc = b * b - a * c;
    J.d = d;
    J.dd = 0.0;
    J.tau = 0.0;
    J.social = false;
    J.contact = h < 0;
    if (disc > 0 && a != 0) {
        double dd = sqrt(disc);
        double tau = (b - dd) / a;
        if (!(tau <= 0 || tau > TAU_MAX)) {
            J.social = true;
            J.dd = dd;
            J.tau = tau;
        }
    }
    return (J.social || J.contact) ? RES_FORCE : RES_ZERO;
}

__device__ __forceinline__ void circ_pair_force(const Circ &A, const Circ &B, const CircJob &J,
                                                double &FPx, double &FPy, double &FQx,
                                                double &FQy) {
    FPx = 0.0; FPy = 0.0; FQx = 0.0; FQy = 0.0;
    double xx = A.x - B.x, xy = A.y - B.y;
    double d = J.d;
    double r_tot = A.r + B.r;
    double h = d - r_tot;
    double vrx = A.vx - B.vx, vry = A.vy - B.vy;
    if (J.social) {
        double a = vrx * vrx + vry * vry;
        double b = -(xx * vrx + xy * vry);
        double dd = J.dd, tau = J.tau;
        double gx = (vrx - (vrx * b + xx * a) / dd) / a;
        double gy = (vry - (vry * b + xy * a) / dd) / a;
        double cmp = (-A.m) * A.k, cmq = (-B.m) * B.k;
        double two_t = 2.0 / tau, tt = tau * tau;       // shared terms of magnitude()
        double magp = (two_t + A.itau0) * cdm_exp(-tau / A.tau0) / tt;
        // magnitude() depends on (tau, tau_0) only: equal tau_0, equal value
        double magq = B.tau0 == A.tau0 ? magp
                                       : (two_t + B.itau0) * cdm_exp(-tau / B.tau0) / tt;
        FPx = (cmp * gx) * magp;
        FPy = (cmp * gy) * magp;
        truncate2(FPx, FPy, F_SOC_MAX);
        FQx = (cmq * (-gx)) * magq;
        FQy = (cmq * (-gy)) * magq;
        truncate2(FQx, FQy, F_SOC_MAX);
    }
    if (h < 0) {
        double nx = 0.0, ny = 0.0, mx = 0.0, my = 0.0;
        if (d != 0.0) { nx = xx / d; ny = xy / d; mx = -nx; my = -ny; }   // (-x)/d == -(x/d)
        double cx, cy;
        force_contact(h, nx, ny, vrx, vry, A.mu, A.kappa, A.damp, cx, cy);
        FPx = FPx + cx;
        FPy = FPy + cy;
        force_contact(h, mx, my, -vrx, -vry, B.mu, B.kappa, B.damp, cx, cy);
        FQx = FQx + cx;
        FQy = FQy + cy;
    }
}

// Per-warp queue for the square root and division of the defined sub-circle
// pairs of the warp's 32 current pairs (9 slots per lane).
struct WarpQueue {
    double b[32 * 9];
    double disc[32 * 9];       // in: discriminant; out: its square root
    double tau[32 * 9];
    double a[32];
    int off[33];
};

constexpr float PRESEL_MARGIN = 1e-4f;   // metres (float32 error of h is ~1e-6 m)


// Per-warp queue of tc_pair_decide: the sub-circle pairs that may have a
// time-to-collision (9 slots per lane) and each lane's pair geometry.
constexpr int GEO_D = 19;   // P parts x[3] y[3], Q parts x[3] y[3], P rt rs, Q rt rs, vr, a
struct PairQueue {
    double b[32 * 9];
    double disc[32 * 9];        // out: square root of the discriminant, or -1
    double tau[32 * 9];
    double geo[32 * GEO_D];
    int off[33];
    unsigned char kidx[32 * 9];
};

// One ThreeCircle pair for every lane of the warp (collective: all lanes in
// `wmask` call it; `act` lanes have a pair, `me_first` its orientation):
// A's force and torque from the pair in (Fx, Fy, Tq); false when the pair
// does not interact.
__device__ __forceinline__ bool tc_pair_eval(const TC &A, const float4 meC, const float4 meF0,
                                             const float4 meF1, const StepArgs &a, bool act,
                                             int t, bool me_first, WarpQueue &q, int lane,
                                             unsigned wmask, int nlanes, double &Fx_out,
                                             double &Fy_out, double &Tq_out) {
    TC B = A;
    float4 oC = meC, oF0 = meF0, oF1 = meF1;
    if (act) {
        B = load_tc(a.stage, t);
        oC = __ldg(&a.cull[t]);
        oF0 = __ldg(&a.stage_f[2 * t]);
        oF1 = __ldg(&a.stage_f[2 * t + 1]);
    }
    // -- distance_three_circles: float32 pre-selection of the minimum --
    const float dxt = (meC.x - oC.x) + (meF0.x - oF0.x);
    const float dyt = (meC.y - oC.y) + (meF0.y - oF0.y);
    const float mox[3] = {0.f, meF1.x, meF1.z}, moy[3] = {0.f, meF1.y, meF1.w};
    const float oox[3] = {0.f, oF1.x, oF1.z}, ooy[3] = {0.f, oF1.y, oF1.w};
    const float mr[3] = {meF0.z, meF0.w, meF0.w}, orr[3] = {oF0.z, oF0.w, oF0.w};
    float hf[9];
    float hfmin = INFINITY;
    bool anynan = false;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float dx = (dxt + mox[i]) - oox[j], dy = (dyt + moy[i]) - ooy[j];
            float h = sqrtf(dx * dx + dy * dy) - (mr[i] + orr[j]);
            hf[3 * i + j] = h;
            anynan |= (h != h);
            hfmin = fminf(hfmin, h);
        }
    // candidates in visiting order (bit k: sequence position k); the margin
    // covers float32 rounding of every input and operation above (each below
    // 2^-24 of the magnitudes involved) many times over
    const float scale = fabsf(dxt) + fabsf(dyt) + fabsf(meF1.x) + fabsf(meF1.y) + fabsf(meF1.z) +
                        fabsf(meF1.w) + fabsf(oF1.x) + fabsf(oF1.y) + fabsf(oF1.z) + fabsf(oF1.w) +
                        mr[0] + mr[1] + orr[0] + orr[1];
    const float margin = PRESEL_MARGIN + 1e-6f * scale;
    unsigned seq = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        int p = k / 3, qq = k % 3;
        float hk = me_first ? hf[3 * p + qq] : hf[3 * qq + p];
        if (hk <= hfmin + margin) seq |= 1u << k;
    }
    if (anynan) seq = 0x1ffu;
    if (!act) seq = 1u;
    // exact float64 minimum over the candidates, first in visiting order wins
    double h_min = __longlong_as_double(0x7ff8000000000000LL);
    double sdx = 0.0, sdy = 0.0, sd = 0.0;
    int mine_min = 0;
    {
        int k = __ffs(seq) - 1;
        unsigned rest = seq & (seq - 1);
        int mi, ti;
        seq_parts(k, me_first, mi, ti);
        double dx = sel3(A.x, mi) - sel3(B.x, ti), dy = sel3(A.y, mi) - sel3(B.y, ti);
        double d = cdm_hypot(dx, dy);
        h_min = d - (part_r(A, mi) + part_r(B, ti));
        sdx = dx; sdy = dy; sd = d; mine_min = mi;
        while (rest) {
            k = __ffs(rest) - 1;
            rest &= rest - 1;
            seq_parts(k, me_first, mi, ti);
            dx = sel3(A.x, mi) - sel3(B.x, ti);
            dy = sel3(A.y, mi) - sel3(B.y, ti);
            d = cdm_hypot(dx, dy);
            double h = d - (part_r(A, mi) + part_r(B, ti));
            if (h < h_min || isnan(h_min)) {
                h_min = h; sdx = dx; sdy = dy; sd = d; mine_min = mi;
            }
        }
    }
    const bool inter = act && (h_min < SIGTH_SOC);
    double nx = 0.0, ny = 0.0;
    if (inter && sd != 0.0) { nx = sdx / sd; ny = sdy / sd; }
    // moment arm: (X[part_me] + r_me * n) - x_me_torso, X the first agent's parts
    double rmx, rmy;
    {
        double xs = me_first ? sel3(A.x, mine_min) : sel3(B.x, mine_min);
        double ys = me_first ? sel3(A.y, mine_min) : sel3(B.y, mine_min);
        double r = part_r(A, mine_min);
        rmx = (xs + r * nx) - A.x[0];
        rmy = (ys + r * ny) - A.y[0];
    }
    // -- force_social_three_circle --
    const double vrx = A.vx - B.vx, vry = A.vy - B.vy;
    const double av = vrx * vrx + vry * vry;
    const bool soc = inter && av != 0;
    unsigned defmask = 0;
    int cnt = 0;
    double* qb = q.b + lane * 9;
    double* qd = q.disc + lane * 9;
    if (soc) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            int mi, ti;
            seq_parts(k, me_first, mi, ti);
            double xr = sel3(A.x, mi) - sel3(B.x, ti), yr = sel3(A.y, mi) - sel3(B.y, ti);
            double r_tot = part_r(A, mi) + part_r(B, ti);
            double b = -(xr * vrx + yr * vry);
            double c = (xr * xr + yr * yr) - r_tot * r_tot;
            double disc = b * b - av * c;
            if (disc > 0) {                        // sqrt defined and non-zero
                qb[cnt] = b;
                qd[cnt] = disc;
                ++cnt;
                defmask |= 1u << k;
            }
        }
    }
    // warp exclusive scan of the item counts (active lanes are a prefix)
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(wmask, incl, o);
        if (lane >= o) incl += v;
    }
    q.off[lane] = incl - cnt;
    q.a[lane] = av;
    const int total = __shfl_sync(wmask, incl, nlanes - 1);
    if (lane == nlanes - 1) q.off[nlanes] = incl;
    __syncwarp(wmask);
    for (int base = 0; base < total; base += nlanes) {     // only nlanes lanes are live
        int it = base + lane;
        if (it < total) {
            int lo = 0, hi = nlanes - 1;        // owner: last lane with off <= it
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (q.off[mid] <= it) lo = mid; else hi = mid - 1;
            }
            int slot = lo * 9 + (it - q.off[lo]);
            double d = sqrt(q.disc[slot]);
            q.tau[slot] = (q.b[slot] - d) / q.a[lo];
            q.disc[slot] = d;
        }
    }
    __syncwarp(wmask);
    double tau = __longlong_as_double(0x7ff8000000000000LL);
    double b_min = 0.0, d_min = 0.0;
    int k_sel = 0;
    {
        int jj = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            if (defmask & (1u << k)) {
                double tau_new = q.tau[lane * 9 + jj];
                double dk = qd[jj], bk = qb[jj];
                ++jj;
                if (isnan(tau) || (0 < tau_new && tau_new < tau)) {
                    k_sel = k; tau = tau_new; b_min = bk; d_min = dk;
                }
            }
        }
    }
    __syncwarp(wmask);
    double Fx = 0.0, Fy = 0.0;
    if (soc && !(isnan(tau) || tau <= 0)) {
        int mi, ti;
        seq_parts(k_sel, me_first, mi, ti);
        double o1x, o1y, o2x, o2y;
        r_off_part(A, mi, o1x, o1y);
        r_off_part(B, ti, o2x, o2y);
        double ox = o1x - o2x, oy = o1y - o2y;
        double xr = A.x[0] - B.x[0], yr = A.y[0] - B.y[0];
        double gx = (vrx - (av * (xr + 2 * ox) + b_min * vrx) / d_min) / av;
        double gy = (vry - (av * (yr + 2 * oy) + b_min * vry) / d_min) / av;
        double cm = (-A.m) * A.k;
        double mag = magnitude(tau, A.tau0, A.itau0);
        Fx = (cm * gx) * mag;
        Fy = (cm * gy) * mag;
        truncate2(Fx, Fy, F_SOC_MAX);
    }
    if (inter && h_min < 0) {
        double cx, cy;
        force_contact(h_min, nx, ny, vrx, vry, A.mu, A.kappa, A.damp, cx, cy);
        Fx = Fx + cx;
        Fy = Fy + cy;
    }
    Fx_out = Fx;
    Fy_out = Fy;
    Tq_out = rmx * Fy - rmy * Fx;                  // cross(r_moment, force)
    return inter;
}

__device__ __forceinline__ void tc_pair_step(const TC &A, const float4 meC, const float4 meF0,
                                             const float4 meF1, const StepArgs &a, bool act,
                                             int t, bool me_first, WarpQueue &q, int lane,
                                             unsigned wmask, int nlanes, double &fx, double &fy,
                                             double &tq) {
    double Fx, Fy, Tq;
    if (tc_pair_eval(A, meC, meF0, meF1, a, act, t, me_first, q, lane, wmask, nlanes, Fx, Fy,
                     Tq)) {
        fx += Fx;
        fy += Fy;
        tq += Tq;
    }
}

// distance_three_circles (core/distance.py:50-105) in P's frame: the
// minimum skin distance over the 3 x 3 sub-circle pairs, the first in
// visiting order winning ties, with the relative position and centre
// distance of that sub-pair and the parts of P and Q at it.  tc_presel keeps,
// in float32, the sub-pairs within a certified margin of the float32 minimum
// (the margin bounds the float32 error of every h many times over);
// tc_distance_exact evaluates those in float64 in visiting order.
struct TcDist { double h, sdx, sdy, sd; int pp, qp; };
struct TcPre { unsigned seq; float hmin, margin; };

__device__ __forceinline__ TcPre tc_presel(float dxt, float dyt, const float mox[3],
                                          const float moy[3], const float oox[3],
                                          const float ooy[3], const float mr[3],
                                          const float orr[3], bool act) {
    float hf[9];
    float hfmin = INFINITY;
    bool anynan = false;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float dx = (dxt + mox[i]) - oox[j], dy = (dyt + moy[i]) - ooy[j];
            float h = sqrtf(dx * dx + dy * dy) - (mr[i] + orr[j]);
            hf[3 * i + j] = h;
            anynan |= (h != h);
            hfmin = fminf(hfmin, h);
        }
    const float scale = fabsf(dxt) + fabsf(dyt) + fabsf(mox[1]) + fabsf(moy[1]) + fabsf(mox[2]) +
                        fabsf(moy[2]) + fabsf(oox[1]) + fabsf(ooy[1]) + fabsf(oox[2]) +
                        fabsf(ooy[2]) + mr[0] + mr[1] + orr[0] + orr[1];
    TcPre P;
    P.margin = PRESEL_MARGIN + 1e-6f * scale;
    P.hmin = hfmin;
    P.seq = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k)
        if (hf[k] <= hfmin + P.margin) P.seq |= 1u << k;
    if (anynan) P.seq = 0x1ffu;
    if (!act) P.seq = 1u;
    return P;
}

// The exact float64 minimum over the pre-selected sub-pairs `seq`, the first
// in visiting order winning ties.
__device__ __forceinline__ TcDist tc_distance_exact(const TC &A, const TC &B, unsigned seq) {
    TcDist D;
    int k = __ffs(seq) - 1;
    unsigned rest = seq & (seq - 1);
    int mi = k / 3, ti = k % 3;
    double dx = sel3(A.x, mi) - sel3(B.x, ti), dy = sel3(A.y, mi) - sel3(B.y, ti);
    double d = cdm_hypot(dx, dy);
    D.h = d - (part_r(A, mi) + part_r(B, ti));
    D.sdx = dx; D.sdy = dy; D.sd = d; D.pp = mi; D.qp = ti;
    while (rest) {
        k = __ffs(rest) - 1;
        rest &= rest - 1;
        mi = k / 3; ti = k % 3;
        dx = sel3(A.x, mi) - sel3(B.x, ti);
        dy = sel3(A.y, mi) - sel3(B.y, ti);
        d = cdm_hypot(dx, dy);
        const double h = d - (part_r(A, mi) + part_r(B, ti));
        if (h < D.h || isnan(D.h)) {
            D.h = h; D.sdx = dx; D.sdy = dy; D.sd = d; D.pp = mi; D.qp = ti;
        }
    }
    return D;
}

// Unit normals of both sides at the minimum and the moment arms
// (X_P[part] + r_side * n_side) - x_side_torso, X_P the first agent's parts
// indexed by the side's own part (core/distance.py:100-103).
__device__ __forceinline__ void tc_moment_arms(const TC &A, const TC &B, const TcDist &D,
                                               double &npx, double &npy, double &nqx,
                                               double &nqy, double &rpx, double &rpy,
                                               double &rqx, double &rqy) {
    npx = 0.0; npy = 0.0; nqx = 0.0; nqy = 0.0;
    if (D.sd != 0.0) {
        npx = D.sdx / D.sd; npy = D.sdy / D.sd;
        nqx = -npx; nqy = -npy;                  // (-x)/d == -(x/d), signed zeros included
    }
    double r = part_r(A, D.pp);
    rpx = (sel3(A.x, D.pp) + r * npx) - A.x[0];
    rpy = (sel3(A.y, D.pp) + r * npy) - A.y[0];
    r = part_r(B, D.qp);
    rqx = (sel3(A.x, D.qp) + r * nqx) - B.x[0];
    rqy = (sel3(A.y, D.qp) + r * nqy) - B.y[0];
}

// Both sides of a ThreeCircle pair (interactions.py:73-101,
// power_law.py:264-363) with P = A first and Q = the pair partner, in two
// passes.  tc_pair_decide computes the distance search and the
// time-to-collision selection once (warp collective like tc_pair_eval: all 32
// lanes call it) and returns RES_NONE, RES_ZERO (no force: forces +0, torques
// signed zeros left to the gather) or RES_FORCE with what the force needs in
// a TcJob; tc_pair_force then computes each side's force, contact and torque
// exactly as tc_pair_eval computes them from that side.  k_pairs decides,
// k_pair_forces evaluates the jobs with every lane busy.
struct TcJob {
    double tau, b_min, d_min;   // selected time to collision and its root's b, sqrt(D)
    TcDist D;                   // the exact minimum sub-pair
    int k_sel;                  // selected sub-pair (3 * P part + Q part)
    bool social, contact;
};

__device__ __forceinline__ int tc_pair_decide(const TC &A, const float4 meC, const float4 meF0,
                                               const float4 meF1, const StepArgs &a, bool act,
                                               int t, PairQueue &q, int lane, TcJob &J) {
    constexpr unsigned wmask = 0xffffffffu;
    constexpr int nlanes = 32;
    // Q's staged record is loaded only where a float64 path needs it
    TC B;
    bool have_b = false;
    float4 oC = meC, oF0 = meF0, oF1 = meF1;
    double2 vq = make_double2(A.vx, A.vy);
    if (act) {
        oC = __ldg(&a.cull[t]);
        oF0 = __ldg(&a.stage_f[2 * t]);
        oF1 = __ldg(&a.stage_f[2 * t + 1]);
        vq = a.stage[(size_t)t * STAGE_Q_TC + 3];
    }
    auto need_b = [&]() {
        if (!have_b) {
            B = load_tc(a.stage, t);
            have_b = true;
        }
    };
    // float32 geometry of the sub-circles (P's frame)
    const float dxt = (meC.x - oC.x) + (meF0.x - oF0.x);
    const float dyt = (meC.y - oC.y) + (meF0.y - oF0.y);
    const float mox[3] = {0.f, meF1.x, meF1.z}, moy[3] = {0.f, meF1.y, meF1.w};
    const float oox[3] = {0.f, oF1.x, oF1.z}, ooy[3] = {0.f, oF1.y, oF1.w};
    const float mr[3] = {meF0.z, meF0.w, meF0.w}, orr[3] = {oF0.z, oF0.w, oF0.w};

    // -- distance_three_circles --
    // The exact minimum is needed for a force (normal, contact, moment arms)
    // and wherever float32 cannot decide the pair.  The torso pair's skin
    // distance bounds the minimum h from above, the enclosing circles' (radius
    // = extent, rounded up) from below: with both clear of 3 and 0 by the
    // float32 margin, the pair interacts without contact, or does not
    // interact.  Otherwise the pre-selection keeps the sub-pairs near the
    // float32 minimum; a single one with its h clear of 3 and 0 decides too,
    // and the rest take the exact float64 minimum.
    const float xe2 = dxt * dxt + dyt * dyt;
    const float xe = sqrtf(xe2);
    const float re = meC.z + oC.z;
    const float dmarg = PRESEL_MARGIN +
                        1e-6f * (fabsf(dxt) + fabsf(dyt) + fabsf(mox[1]) + fabsf(moy[1]) +
                                 fabsf(mox[2]) + fabsf(moy[2]) + fabsf(oox[1]) + fabsf(ooy[1]) +
                                 fabsf(oox[2]) + fabsf(ooy[2]) + mr[0] + mr[1] + orr[0] + orr[1]);
    const float h_lo = xe - re, h_hi = xe - (mr[0] + orr[0]);
    TcPre pre;
    pre.seq = 1u;
    bool have_pre = false;
    TcDist D;
    bool have_d = false;
    bool inter = false;
    if (act && !(h_lo - dmarg >= (float)SIGTH_SOC)) {
        if (h_hi + dmarg < (float)SIGTH_SOC && h_lo - dmarg > 0.f) {
            inter = true;
        } else {
            pre = tc_presel(dxt, dyt, mox, moy, oox, ooy, mr, orr, act);
            have_pre = true;
            const bool unique = (pre.seq & (pre.seq - 1u)) == 0u;
            const bool far_cert = pre.hmin - pre.margin >= (float)SIGTH_SOC;
            const bool near_cert =
                pre.hmin + pre.margin < (float)SIGTH_SOC && pre.hmin - pre.margin > 0.f;
            if (unique && (far_cert || near_cert)) {
                inter = near_cert;
            } else {
                need_b();
                D = tc_distance_exact(A, B, pre.seq);
                have_d = true;
                inter = D.h < SIGTH_SOC;
            }
        }
    }
    const double h_min = have_d ? D.h : 0.0;
    const bool contact = inter && have_d && h_min < 0;

    // -- force_social_three_circle (shared time-to-collision) --
    // The selected tau is positive exactly when the first sub-pair (visiting
    // order) with a defined root has a positive root: a non-positive first
    // root is never replaced.  float32 classifies each sub-pair's
    // discriminant (below -M: no root; above M: a root) and, for the first
    // sub-pair with a root, the sign of tau = (b - d) / a from the signs of b
    // and c (b < 0, or c < 0 with a|c| not negligible against b^2: the
    // float64 d exceeds b, tau < 0; b > 0 and c > 0 likewise: tau > 0).  A
    // pair certified to have no positive tau takes no float64 work here; the
    // others put their candidate sub-pairs in the warp queue, where any lane
    // evaluates the reference's float64 b, c, discriminant, root and tau from
    // the owner's geometry in shared memory, and select tau as the reference.
    const double vrx = A.vx - vq.x, vry = A.vy - vq.y;
    const float vxf = (float)vrx, vyf = (float)vry;
    double av = 0.0;
    bool have_av = false;
    bool soc = inter;
    if (inter && !(fabsf(vxf) > 1e-20f || fabsf(vyf) > 1e-20f)) {
        av = vrx * vrx + vry * vry;                      // a == 0 only for (near) zero speed
        have_av = true;
        soc = av != 0;
    }
    unsigned candmask = 0;
    int cnt = 0;
    bool least_rule = false;             // select the least positive root (first root > 0)
    if (soc) {
        const float af = vxf * vxf + vyf * vyf;
        const float e0 = 1e-6f * (1.f + fabsf(dxt) + fabsf(dyt) + fabsf(mox[1]) + fabsf(moy[1]) +
                                  fabsf(mox[2]) + fabsf(moy[2]) + fabsf(oox[1]) + fabsf(ooy[1]) +
                                  fabsf(oox[2]) + fabsf(ooy[2]));
        // Enclosing circles (radius = extent, rounded up, about the torsos)
        // contain every sub-circle.  Apart now and for all t > 0 (c > 0, and
        // b <= 0 or b^2 < a c, each with its error margin): no sub-pair ever
        // overlaps at t > 0, so every root is negative and there is no force.
        const float re = meC.z + oC.z;
        const float xe2 = dxt * dxt + dyt * dyt;
        const float be = -(dxt * vxf + dyt * vyf);
        const float ce = xe2 - re * re;
        const float mbe = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                          1e-6f * (fabsf(dxt * vxf) + fabsf(dyt * vyf));
        const float mce = 8.f * e0 * (fabsf(dxt) + fabsf(dyt) + re) + 1e-6f * (xe2 + re * re);
        const float bbe = fabsf(be) + mbe;
        const bool apart = ce - mce > 0.f && (be + mbe <= 0.f || bbe * bbe < 0.99f * af * (ce - mce));
        int first = apart ? 1 : -1;                      // class of the first sub-pair with a root
        float min_hi = INFINITY;                         // least upper bound of a certain tau > 0
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            if (apart) break;
            const int i = k / 3, j = k % 3;
            const float dx = (dxt + mox[i]) - oox[j], dy = (dyt + moy[i]) - ooy[j];
            const float rt = mr[i] + orr[j];
            const float bf = -(dx * vxf + dy * vyf);
            const float x2 = dx * dx + dy * dy;
            const float cf = x2 - rt * rt;
            const float acf = af * cf;
            const float discf = bf * bf - acf;
            const float m = 1e-5f * af * (1.f + x2 + rt * rt) + 1e-6f * (bf * bf + fabsf(acf));
            if (!(discf < -m)) {
                candmask |= 1u << k;
                const float mb = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                                 1e-6f * (fabsf(dx * vxf) + fabsf(dy * vyf));
                const float mc = 8.f * e0 * (fabsf(dx) + fabsf(dy) + rt) + 1e-6f * (x2 + rt * rt);
                const float bb = (fabsf(bf) + mb) * (fabsf(bf) + mb);
                const bool pos = discf > m && bf > mb && cf > mc &&
                                 0.99f * af * (cf - mc) > 1e-9f * bb;
                if (first < 0) {
                    // 0: decide in float64; 1: tau < 0 certain; 2: tau > 0 certain
                    first = 0;
                    if (discf > m) {
                        if (bf < -mb) first = 1;
                        else if (cf < -mc && 0.99f * af * (-cf - mc) > 1e-9f * bb) first = 1;
                        else if (pos) first = 2;
                    }
                }
                // tau = c / (b + sqrt(D)) (b > 0): an upper bound from the
                // margins of b, c and D (and 1e-5 for every rounding)
                if (pos)
                    min_hi = fminf(min_hi, (cf + mc) / ((bf - mb) + sqrtf(discf - m)) * 1.00001f);
            }
        }
        if (first == 1) candmask = 0;                     // no positive tau: no force
        if (first == 2 && (candmask & (candmask - 1u))) {
            // The first root is positive: the selected tau is the least
            // positive root (the earliest of equals).  A root certainly
            // negative, or whose lower bound exceeds another root's upper
            // bound, is never selected: not evaluated in float64.
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                if (!(candmask & (1u << k))) continue;
                const int i = k / 3, j = k % 3;
                const float dx = (dxt + mox[i]) - oox[j], dy = (dyt + moy[i]) - ooy[j];
                const float rt = mr[i] + orr[j];
                const float bf = -(dx * vxf + dy * vyf);
                const float x2 = dx * dx + dy * dy;
                const float cf = x2 - rt * rt;
                const float acf = af * cf;
                const float discf = bf * bf - acf;
                const float m = 1e-5f * af * (1.f + x2 + rt * rt) + 1e-6f * (bf * bf + fabsf(acf));
                if (!(discf > m)) continue;
                const float mb = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                                 1e-6f * (fabsf(dx * vxf) + fabsf(dy * vyf));
                const float mc = 8.f * e0 * (fabsf(dx) + fabsf(dy) + rt) + 1e-6f * (x2 + rt * rt);
                const float bb = (fabsf(bf) + mb) * (fabsf(bf) + mb);
                bool drop = bf < -mb || (cf < -mc && 0.99f * af * (-cf - mc) > 1e-9f * bb);
                if (!drop && bf > mb && cf > mc && 0.99f * af * (cf - mc) > 1e-9f * bb)
                    drop = (cf - mc) / ((bf + mb) + sqrtf(discf + m)) * 0.99999f > min_hi;
                if (drop) candmask &= ~(1u << k);
            }
        }
        least_rule = first == 2;
    }
    if (candmask) {
        if (!have_av) {
            av = vrx * vrx + vry * vry;
            have_av = true;
        }
        need_b();
        unsigned mrest = candmask;
        while (mrest) {
            const int k = __ffs(mrest) - 1;
            mrest &= mrest - 1;
            q.kidx[lane * 9 + cnt] = (unsigned char)k;
            ++cnt;
        }
        double *g = q.geo + lane * GEO_D;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g[k] = A.x[k]; g[3 + k] = A.y[k]; g[6 + k] = B.x[k]; g[9 + k] = B.y[k];
        }
        g[12] = A.rt; g[13] = A.rs; g[14] = B.rt; g[15] = B.rs;
        g[16] = vrx; g[17] = vry; g[18] = av;
    }
    double tau = __longlong_as_double(0x7ff8000000000000LL);
    double b_min = 0.0, d_min = 0.0;
    int k_sel = 0;
    // the queue (scan, float64 roots, selection) only where a lane needs it
    if (__any_sync(wmask, cnt > 0)) {
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(wmask, incl, o);
            if (lane >= o) incl += v;
        }
        q.off[lane] = incl - cnt;
        const int total = __shfl_sync(wmask, incl, nlanes - 1);
        if (lane == nlanes - 1) q.off[nlanes] = incl;
        __syncwarp(wmask);
        for (int base = 0; base < total; base += nlanes) {
            int it = base + lane;
            if (it < total) {
                int lo = 0, hi = nlanes - 1;        // owner: last lane with off <= it
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (q.off[mid] <= it) lo = mid; else hi = mid - 1;
                }
                const int slot = lo * 9 + (it - q.off[lo]);
                const int k = q.kidx[slot];
                const int i = k / 3, j = k % 3;
                const double *g = q.geo + lo * GEO_D;
                const double gvx = g[16], gvy = g[17], ga = g[18];
                const double xr = g[i] - g[6 + j], yr = g[3 + i] - g[9 + j];
                const double r_tot = g[12 + (i > 0)] + g[14 + (j > 0)];
                const double b = -(xr * gvx + yr * gvy);
                const double c = (xr * xr + yr * yr) - r_tot * r_tot;
                const double disc = b * b - ga * c;
                double d = -1.0, tau_k = 0.0;
                if (disc > 0) {                      // sqrt defined and non-zero
                    d = sqrt(disc);
                    tau_k = (b - d) / ga;
                }
                q.b[slot] = b;
                q.disc[slot] = d;                    // -1: no time-to-collision
                q.tau[slot] = tau_k;
            }
        }
        __syncwarp(wmask);
        {
            int jj = 0;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                if (candmask & (1u << k)) {
                    const int slot = lane * 9 + jj;
                    ++jj;
                    const double dk = q.disc[slot];
                    if (dk > 0) {
                        const double tau_new = q.tau[slot];
                        const bool take =
                            least_rule ? (0 < tau_new && (isnan(tau) || tau_new < tau))
                                       : (isnan(tau) || (0 < tau_new && tau_new < tau));
                        if (take) {
                            k_sel = k; tau = tau_new; b_min = q.b[slot]; d_min = dk;
                        }
                    }
                }
            }
        }
        __syncwarp(wmask);
    }
    const bool social = soc && candmask && !(isnan(tau) || tau <= 0);
    // No force on either side: forces (+0, +0), and each side's torque
    // r x (+0, +0) a signed zero that the gather needs only when the agent's
    // running torque is -0 (the agent is then redone with exact signs)
    if (!(social || contact)) return inter ? RES_ZERO : RES_NONE;
    need_b();
    if (!have_d) {
        if (!have_pre) pre = tc_presel(dxt, dyt, mox, moy, oox, ooy, mr, orr, act);
        D = tc_distance_exact(A, B, pre.seq);
    }
    J.tau = tau;
    J.b_min = b_min;
    J.d_min = d_min;
    J.D = D;
    J.k_sel = k_sel;
    J.social = social;
    J.contact = contact;
    return RES_FORCE;
}

// The forces and torques of a pair tc_pair_decide found to have a force.
// The relative velocity and a = |v|^2 are formed as tc_pair_decide forms them.
__device__ __forceinline__ void tc_pair_force(const TC &A, const TC &B, const TcJob &J,
                                              double &FPx, double &FPy, double &TP, double &FQx,
                                              double &FQy, double &TQ) {
    const double vrx = A.vx - B.vx, vry = A.vy - B.vy;
    FPx = 0.0; FPy = 0.0; FQx = 0.0; FQy = 0.0;
    if (J.social) {
        const double av = vrx * vrx + vry * vry;
        const double tau = J.tau, b_min = J.b_min, d_min = J.d_min;
        const int mi = J.k_sel / 3, ti = J.k_sel % 3;
        double o1x, o1y, o2x, o2y;
        r_off_part(A, mi, o1x, o1y);
        r_off_part(B, ti, o2x, o2y);
        double ox = o1x - o2x, oy = o1y - o2y;
        double xr = A.x[0] - B.x[0], yr = A.y[0] - B.y[0];
        double gx = (vrx - (av * (xr + 2 * ox) + b_min * vrx) / d_min) / av;
        double gy = (vry - (av * (yr + 2 * oy) + b_min * vry) / d_min) / av;
        double cmp = (-A.m) * A.k, cmq = (-B.m) * B.k;
        double two_t = 2.0 / tau, tt = tau * tau;            // shared terms of magnitude()
        double magp = (two_t + A.itau0) * cdm_exp(-tau / A.tau0) / tt;
        // magnitude() depends on (tau, tau_0) only: equal tau_0, equal value
        double magq = B.tau0 == A.tau0 ? magp
                                       : (two_t + B.itau0) * cdm_exp(-tau / B.tau0) / tt;
        FPx = (cmp * gx) * magp;
        FPy = (cmp * gy) * magp;
        truncate2(FPx, FPy, F_SOC_MAX);
        FQx = (cmq * (-gx)) * magq;             // Q's gradient is -g exactly
        FQy = (cmq * (-gy)) * magq;
        truncate2(FQx, FQy, F_SOC_MAX);
    }
    double npx, npy, nqx, nqy, rpx, rpy, rqx, rqy;
    tc_moment_arms(A, B, J.D, npx, npy, nqx, nqy, rpx, rpy, rqx, rqy);
    if (J.contact) {
        const double h_min = J.D.h;
        double cx, cy;
        force_contact(h_min, npx, npy, vrx, vry, A.mu, A.kappa, A.damp, cx, cy);
        FPx = FPx + cx;
        FPy = FPy + cy;
        force_contact(h_min, nqx, nqy, -vrx, -vry, B.mu, B.kappa, B.damp, cx, cy);
        FQx = FQx + cx;
        FQy = FQy + cy;
    }
    TP = rpx * FPy - rpy * FPx;
    TQ = rqx * FQy - rqy * FQx;
}

// The float32 part of tc_pair_decide alone, for a pair (s, t): RES_NONE or
// RES_ZERO where its certificates decide the pair (no contact, no positive
// time to collision; the same tests and margins, so the same decision), and
// RES_DEFER where tc_pair_decide would need float64 (the exact distance, the
// roots, a zero relative speed).  Reads 96 bytes of pre-check records and
// the two velocities; holds no float64 geometry.
__device__ __forceinline__ int tc_pair_light(const StepArgs &a, int s, int t) {
    const float4 meC = __ldg(&a.cull[s]), meF0 = __ldg(&a.stage_f[2 * s]),
                 meF1 = __ldg(&a.stage_f[2 * s + 1]);
    const float4 oC = __ldg(&a.cull[t]), oF0 = __ldg(&a.stage_f[2 * t]),
                 oF1 = __ldg(&a.stage_f[2 * t + 1]);
    const float dxt = (meC.x - oC.x) + (meF0.x - oF0.x);
    const float dyt = (meC.y - oC.y) + (meF0.y - oF0.y);
    const float mox[3] = {0.f, meF1.x, meF1.z}, moy[3] = {0.f, meF1.y, meF1.w};
    const float oox[3] = {0.f, oF1.x, oF1.z}, ooy[3] = {0.f, oF1.y, oF1.w};
    const float mr[3] = {meF0.z, meF0.w, meF0.w}, orr[3] = {oF0.z, oF0.w, oF0.w};
    // distance bounds (torso pair above, enclosing circles below), then the
    // pre-selection's single candidate
    const float xe2 = dxt * dxt + dyt * dyt;
    const float xe = sqrtf(xe2);
    const float re = meC.z + oC.z;
    const float dmarg = PRESEL_MARGIN +
                        1e-6f * (fabsf(dxt) + fabsf(dyt) + fabsf(mox[1]) + fabsf(moy[1]) +
                                 fabsf(mox[2]) + fabsf(moy[2]) + fabsf(oox[1]) + fabsf(ooy[1]) +
                                 fabsf(oox[2]) + fabsf(ooy[2]) + mr[0] + mr[1] + orr[0] + orr[1]);
    const float h_lo = xe - re, h_hi = xe - (mr[0] + orr[0]);
    if (h_lo - dmarg >= (float)SIGTH_SOC) return RES_NONE;
    if (!(h_hi + dmarg < (float)SIGTH_SOC && h_lo - dmarg > 0.f)) {
        const TcPre pre = tc_presel(dxt, dyt, mox, moy, oox, ooy, mr, orr, true);
        const bool unique = (pre.seq & (pre.seq - 1u)) == 0u;
        const bool far_cert = pre.hmin - pre.margin >= (float)SIGTH_SOC;
        const bool near_cert =
            pre.hmin + pre.margin < (float)SIGTH_SOC && pre.hmin - pre.margin > 0.f;
        if (!(unique && (far_cert || near_cert))) return RES_DEFER;
        if (!near_cert) return RES_NONE;
    }
    // interacting without contact: a force only from a positive time to
    // collision (the relative velocity as tc_pair_decide forms it)
    const double2 vp = __ldg(&a.stage[(size_t)s * STAGE_Q_TC + 3]);
    const double2 vq = __ldg(&a.stage[(size_t)t * STAGE_Q_TC + 3]);
    const float vxf = (float)(vp.x - vq.x), vyf = (float)(vp.y - vq.y);
    if (!(fabsf(vxf) > 1e-20f || fabsf(vyf) > 1e-20f)) return RES_DEFER;
    const float af = vxf * vxf + vyf * vyf;
    const float e0 = 1e-6f * (1.f + fabsf(dxt) + fabsf(dyt) + fabsf(mox[1]) + fabsf(moy[1]) +
                              fabsf(mox[2]) + fabsf(moy[2]) + fabsf(oox[1]) + fabsf(ooy[1]) +
                              fabsf(oox[2]) + fabsf(ooy[2]));
    {
        const float be = -(dxt * vxf + dyt * vyf);
        const float ce = xe2 - re * re;
        const float mbe = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                          1e-6f * (fabsf(dxt * vxf) + fabsf(dyt * vyf));
        const float mce = 8.f * e0 * (fabsf(dxt) + fabsf(dyt) + re) + 1e-6f * (xe2 + re * re);
        const float bbe = fabsf(be) + mbe;
        if (ce - mce > 0.f && (be + mbe <= 0.f || bbe * bbe < 0.99f * af * (ce - mce)))
            return RES_ZERO;                             // enclosing circles apart for t > 0
    }
    // the first sub-pair (visiting order) that may have a root decides:
    // a certainly negative first root, no force; anything else, float64
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int i = k / 3, j = k % 3;
        const float dx = (dxt + mox[i]) - oox[j], dy = (dyt + moy[i]) - ooy[j];
        const float rt = mr[i] + orr[j];
        const float bf = -(dx * vxf + dy * vyf);
        const float x2 = dx * dx + dy * dy;
        const float cf = x2 - rt * rt;
        const float acf = af * cf;
        const float discf = bf * bf - acf;
        const float m = 1e-5f * af * (1.f + x2 + rt * rt) + 1e-6f * (bf * bf + fabsf(acf));
        if (discf < -m) continue;
        if (!(discf > m)) return RES_DEFER;
        const float mb = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                         1e-6f * (fabsf(dx * vxf) + fabsf(dy * vyf));
        const float mc = 8.f * e0 * (fabsf(dx) + fabsf(dy) + rt) + 1e-6f * (x2 + rt * rt);
        const float bb = (fabsf(bf) + mb) * (fabsf(bf) + mb);
        if (bf < -mb) return RES_ZERO;
        if (cf < -mc && 0.99f * af * (-cf - mc) > 1e-9f * bb) return RES_ZERO;
        return RES_DEFER;
    }
    return RES_ZERO;                                     // no sub-pair has a root
}

// The first stages of tc_pair_light, which decide most pairs (the distance
// bounds, then the enclosing circles apart for t > 0): its result, or
// RES_SLOW where tc_pair_light goes on to the pre-selection or to the
// sub-pair roots (the same tests on the same values, so the same decisions).
constexpr int RES_SLOW = 4;
__device__ __forceinline__ int tc_pair_light_quick(const StepArgs &a, int s, int t) {
    const float4 meC = __ldg(&a.cull[s]), meF0 = __ldg(&a.stage_f[2 * s]),
                 meF1 = __ldg(&a.stage_f[2 * s + 1]);
    const float4 oC = __ldg(&a.cull[t]), oF0 = __ldg(&a.stage_f[2 * t]),
                 oF1 = __ldg(&a.stage_f[2 * t + 1]);
    const float dxt = (meC.x - oC.x) + (meF0.x - oF0.x);
    const float dyt = (meC.y - oC.y) + (meF0.y - oF0.y);
    const float mox1 = meF1.x, moy1 = meF1.y, mox2 = meF1.z, moy2 = meF1.w;
    const float oox1 = oF1.x, ooy1 = oF1.y, oox2 = oF1.z, ooy2 = oF1.w;
    const float xe2 = dxt * dxt + dyt * dyt;
    const float xe = sqrtf(xe2);
    const float re = meC.z + oC.z;
    const float dmarg = PRESEL_MARGIN +
                        1e-6f * (fabsf(dxt) + fabsf(dyt) + fabsf(mox1) + fabsf(moy1) +
                                 fabsf(mox2) + fabsf(moy2) + fabsf(oox1) + fabsf(ooy1) +
                                 fabsf(oox2) + fabsf(ooy2) + meF0.z + meF0.w + oF0.z + oF0.w);
    const float h_lo = xe - re, h_hi = xe - (meF0.z + oF0.z);
    if (h_lo - dmarg >= (float)SIGTH_SOC) return RES_NONE;
    if (!(h_hi + dmarg < (float)SIGTH_SOC && h_lo - dmarg > 0.f)) return RES_SLOW;
    const double2 vp = __ldg(&a.stage[(size_t)s * STAGE_Q_TC + 3]);
    const double2 vq = __ldg(&a.stage[(size_t)t * STAGE_Q_TC + 3]);
    const float vxf = (float)(vp.x - vq.x), vyf = (float)(vp.y - vq.y);
    if (!(fabsf(vxf) > 1e-20f || fabsf(vyf) > 1e-20f)) return RES_DEFER;
    const float af = vxf * vxf + vyf * vyf;
    const float e0 = 1e-6f * (1.f + fabsf(dxt) + fabsf(dyt) + fabsf(mox1) + fabsf(moy1) +
                              fabsf(mox2) + fabsf(moy2) + fabsf(oox1) + fabsf(ooy1) +
                              fabsf(oox2) + fabsf(ooy2));
    const float be = -(dxt * vxf + dyt * vyf);
    const float ce = xe2 - re * re;
    const float mbe = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                      1e-6f * (fabsf(dxt * vxf) + fabsf(dyt * vyf));
    const float mce = 8.f * e0 * (fabsf(dxt) + fabsf(dyt) + re) + 1e-6f * (xe2 + re * re);
    const float bbe = fabsf(be) + mbe;
    if (ce - mce > 0.f && (be + mbe <= 0.f || bbe * bbe < 0.99f * af * (ce - mce)))
        return RES_ZERO;
    return RES_SLOW;
}

// The float32 certificates of circ_pair_decide for a pair (s, t):
// RES_NONE where the skin distance is certainly >= 3 m, RES_ZERO where it is
// certainly in (0, 3) and the pair certainly has no time to collision in
// (0, 30] (no root; a negative root; or one beyond the 30 s cut-off, with
// a c >= 1e-9 b^2 so that the float64 root's own cancellation stays below
// 1e-6 relative), RES_DEFER otherwise (contact, the edges of 3 and 0, roots
// near 0 or 30, a zero relative speed).  The margins are those of
// tc_pair_light's sub-pairs: each bounds the float32 error of every input
// (positions as hi + lo floats relative to the grid origin, radii and the
// relative velocity rounded once) and operation many times over.
__device__ __forceinline__ int circ_pair_light(const StepArgs &a, int s, int t) {
    const float4 meC = __ldg(&a.cull[s]), meF = __ldg(&a.stage_f[2 * s]);
    const float4 oC = __ldg(&a.cull[t]), oF = __ldg(&a.stage_f[2 * t]);
    const float dx = (meC.x - oC.x) + (meF.x - oF.x);
    const float dy = (meC.y - oC.y) + (meF.y - oF.y);
    const float rt = meF.z + oF.z;
    const float x2 = dx * dx + dy * dy;
    const float h = sqrtf(x2) - rt;
    const float dmarg = PRESEL_MARGIN + 1e-6f * (fabsf(dx) + fabsf(dy) + rt);
    if (h - dmarg >= (float)SIGTH_SOC) return RES_NONE;
    if (!(h + dmarg < (float)SIGTH_SOC && h - dmarg > 0.f)) return RES_DEFER;
    // interacting without contact: a force only from a time to collision
    // in (0, 30] (the relative velocity as circ_pair_decide forms it)
    const double2 vp = __ldg(&a.stage[(size_t)s * STAGE_Q_CIRC + 1]);
    const double2 vq = __ldg(&a.stage[(size_t)t * STAGE_Q_CIRC + 1]);
    const float vxf = (float)(vp.x - vq.x), vyf = (float)(vp.y - vq.y);
    if (!(fabsf(vxf) > 1e-20f || fabsf(vyf) > 1e-20f)) return RES_DEFER;
    const float af = vxf * vxf + vyf * vyf;
    const float e0 = 1e-6f * (1.f + fabsf(dx) + fabsf(dy));
    const float bf = -(dx * vxf + dy * vyf);
    const float cf = x2 - rt * rt;
    const float acf = af * cf;
    const float discf = bf * bf - acf;
    const float m = 1e-5f * af * (1.f + x2 + rt * rt) + 1e-6f * (bf * bf + fabsf(acf));
    if (discf < -m) return RES_ZERO;                     // no root
    if (!(discf > m)) return RES_DEFER;
    const float mb = 4.f * e0 * (fabsf(vxf) + fabsf(vyf)) +
                     1e-6f * (fabsf(dx * vxf) + fabsf(dy * vyf));
    const float mc = 8.f * e0 * (fabsf(dx) + fabsf(dy) + rt) + 1e-6f * (x2 + rt * rt);
    if (bf < -mb) return RES_ZERO;                       // tau = (b - d) / a < 0
    const float bb = (fabsf(bf) + mb) * (fabsf(bf) + mb);
    if (bf > mb && cf > mc && 0.99f * af * (cf - mc) > 1e-9f * bb) {
        // tau = c / (b + d) from below
        const float lo = (cf - mc) / ((bf + mb) + sqrtf(discf + m)) * 0.99999f;
        if (lo > (float)TAU_MAX * 1.00001f) return RES_ZERO;
    }
    return RES_DEFER;
}

// Resumable candidate enumeration into the thread's list (visiting order:
// 3 x 3 cells in (dx, dy) lexicographic order, each cell ascending).
struct EnumState { int ck, t; };

template <int NT, int CAP>
__device__ __forceinline__ int enumerate_candidates(const StepArgs &a, const ScenDev &sc, int s,
                                                    int my_cell, float4 me, int *mylist,
                                                    EnumState &st) {
    int local = my_cell - sc.cell_base;
    int ix = local / sc.ny, iy = local - ix * sc.ny;
    int nl = 0;
    for (; st.ck < 9; ++st.ck, st.t = -1) {
        int dx = st.ck / 3 - 1, dy = st.ck % 3 - 1;
        int jx = ix + dx, jy = iy + dy;
        if (jx < 0 || jx >= sc.nx || jy < 0 || jy >= sc.ny) continue;
        int c2 = sc.cell_base + jx * sc.ny + jy;
        int e = __ldg(&a.start[c2 + 1]);
        if (st.t < 0) st.t = __ldg(&a.start[c2]);
        bool fwd = (dx > 0) || (dx == 0 && dy > 0);
        bool same = (dx == 0 && dy == 0);
        for (; st.t < e; ++st.t) {
            int t = st.t;
            if (t == s) continue;
            if (pair_far(me, __ldg(&a.cull[t]))) continue;
            if (nl == CAP) return nl;            // resume at this candidate
            mylist[nl * NT] = (same ? (s < t) : fwd) ? ~t : t;
            ++nl;
        }
    }
    return nl;
}

// Navigation (simulation/logic.py:152-165, core/steering/navigation.py:60-78,
// core/steering/quickest_path.py:40-43): an agent with target t in range
// takes map t's direction at ((position - origin) / step) truncated toward
// zero, (y, x) as (row, column), when inside the map.  Non-finite quotients
// leave the direction unchanged.
__device__ __forceinline__ void navigate(const StepArgs &a, const ScenDev &sc, const int i) {
    const int t = a.tgt[i];
    if (t < 0 || t >= sc.nav_targets) return;
    double *const *col = a.col;
    const double tx = trunc((col[X][i] - sc.nav_x0) / sc.nav_step);
    const double ty = trunc((col[Y][i] - sc.nav_y0) / sc.nav_step);
    if (!(tx >= 0.0 && tx < (double)sc.nav_nx && ty >= 0.0 && ty < (double)sc.nav_ny)) return;
    const double2 e = a.navmap[sc.nav_off + ((long long)t * sc.nav_ny + (long long)ty) * sc.nav_nx +
                               (long long)tx];
    col[E0X][i] = e.x;
    col[E0Y][i] = e.y;
}

// Per-agent terms before agent-agent: navigation, the force (and torque)
// array's value, fluctuation, orientation and adjusting, in the reference's
// node order.
template <int BODY>
__device__ __forceinline__ void agent_prologue(const StepArgs &a, const int i, double &fx,
                                               double &fy, double &tq, double &phi0) {
    double *const *col = a.col;
    const int nodes = a.nodes;
    if (nodes & N_NAV) navigate(a, a.scen[a.scen_of[i]], i);
    fx = col[FX][i];
    fy = col[FY][i];
    tq = (BODY == 1) ? col[TORQUE][i] : 0.0;
    // Fluctuation (simulation/logic.py:78-86): noise drawn on the host, or on
    // the device by the counter generator (cd_noise.h)
    if ((nodes & N_FLUCT) && a.noise_dev) {
        double nx, ny, nq;
        cdn_fluctuation(a.noise_seed, *a.rng_step, (uint32_t)i, col[MASS][i], col[SRF][i],
                        BODY == 1 ? col[INERTIA][i] : 0.0, BODY == 1 ? col[SRT][i] : 0.0,
                        BODY == 1, &nx, &ny, &nq);
        fx = fx + nx;
        fy = fy + ny;
        if (BODY == 1) tq = tq + nq;
    } else if ((nodes & N_FLUCT) && a.noise_f) {
        fx = fx + a.noise_f[2 * i];
        fy = fy + a.noise_f[2 * i + 1];
        if (BODY == 1 && a.noise_m) tq = tq + a.noise_m[i];
    }
    phi0 = (BODY == 1) ? col[PHI0][i] : 0.0;
    // Orientation (core/steering/orientation.py:17-21)
    if (BODY == 1 && (nodes & N_ORIENT)) phi0 = cdm_atan2(col[E0Y][i], col[E0X][i]);
    // Adjusting (core/motion/adjusting.py:16-121)
    if (nodes & N_ADJUST) {
        double k = col[MASS][i] / col[TAU_ADJ][i];
        double v0 = col[V0][i];
        fx = fx + k * (v0 * col[E0X][i] - col[VX][i]);
        fy = fy + k * (v0 * col[E0Y][i] - col[VY][i]);
        if (BODY == 1) {
            tq = tq + col[INERTIA][i] / col[TAU_ROT][i] *
                          (wrap_to_pi(phi0 - col[PHI][i]) / PI_D * col[W0][i] - col[OMEGA][i]);
        }
    }
}

// Per-agent terms after agent-agent: walls, then integration and reset.
template <int BODY>
__device__ __forceinline__ void agent_epilogue(const StepArgs &a, const int s, const int i,
                                               const int sid, const ScenDev &sc,
                                               const float4 me, const int my_cell, double fx,
                                               double fy, double tq, const double phi0,
                                               const double *old_acc = nullptr) {
    double *const *col = a.col;
    const int nodes = a.nodes;
    // Agent-wall (core/interactions.py:107-141,169-186), walls in index order
    if ((nodes & N_WALL) && sc.wall_count > 0) {
        const bool all_walls = me.z > (float)sc.wall_reach;
        int wb, we;
        if (all_walls) { wb = sc.wall_begin; we = sc.wall_begin + sc.wall_count; }
        else { wb = __ldg(&a.wall_start[my_cell]); we = __ldg(&a.wall_start[my_cell + 1]); }
        if (BODY == 0) {
            Circ A;
            bool loaded = false;
            for (int q = wb; q < we; ++q) {
                int w = all_walls ? q : __ldg(&a.wall_idx[q]);
                if (wall_far(me.x, me.y, me.z, __ldg(&a.walls_f[w]))) continue;
                if (!loaded) { A = load_circ(a.stage, s); loaded = true; }
                wall_circular(A, a.walls + (size_t)w * WALL_D, fx, fy);
            }
        } else {
            TC A;
            bool loaded = false;
            for (int q = wb; q < we; ++q) {
                int w = all_walls ? q : __ldg(&a.wall_idx[q]);
                if (wall_far(me.x, me.y, me.z, __ldg(&a.walls_f[w]))) continue;
                if (!loaded) { A = load_tc(a.stage, s); loaded = true; }
                wall_three_circle(A, a.walls + (size_t)w * WALL_D, fx, fy, tq);
            }
        }
    }

    if (BODY == 1 && (nodes & N_ORIENT)) col[PHI0][i] = phi0;

    if (nodes & N_INTEG) {
        // velocity_verlet_integrator, core/integrator.py:164-193,209-256
        const double dt = a.dt[sid];
        const double dt2 = dt * dt;
        double m = col[MASS][i];
        // the old accelerations, from k_prologue when it ran (same divisions)
        double oax = old_acc ? old_acc[0] : col[FPX][i] / m;
        double oay = old_acc ? old_acc[1] : col[FPY][i] / m;
        double nax = fx / m, nay = fy / m;
        double vx = col[VX][i] + (oax + nax) / 2 * dt;
        double vy = col[VY][i] + (oay + nay) / 2 * dt;
        double x = col[X][i] + (vx * dt + nax / 2 * dt2);
        double y = col[Y][i] + (vy * dt + nay / 2 * dt2);
        col[FPX][i] = fx; col[FPY][i] = fy;
        col[VX][i] = vx; col[VY][i] = vy;
        col[X][i] = x; col[Y][i] = y;
        if (BODY == 1) {
            double I = col[INERTIA][i];
            double oaa = old_acc ? old_acc[2] : col[TORQUE_PREV][i] / I, naa = tq / I;
            col[TORQUE_PREV][i] = tq;
            double w = col[OMEGA][i] + (oaa + naa) / 2 * dt;
            double phi = wrap_to_pi(col[PHI][i] + (w * dt + naa / 2 * dt2));
            col[OMEGA][i] = w;
            col[PHI][i] = phi;
            // shoulders, simulation/agents.py:473-486
            double rts = col[RTS][i];
            double sn, cs;
            cdm_sincos(phi, &sn, &cs);
            double ox = sn * rts, oy = (-cs) * rts;
            col[XLS][i] = x - ox; col[YLS][i] = y - oy;
            col[XRS][i] = x + ox; col[YRS][i] = y + oy;
        }
    }
    if (nodes & N_RESET) {
        // Reset.update, simulation/logic.py:59-64 (runs last)
        col[FX][i] = 0.0; col[FY][i] = 0.0;
        if (BODY == 1) col[TORQUE][i] = 0.0;
    } else {
        col[FX][i] = fx; col[FY][i] = fy;
        if (BODY == 1) col[TORQUE][i] = tq;
    }
}

// All forces on the agent in cell-sorted slot s, then its integration.
// Called by a whole warp (lanes with s >= n skip; warp collectives run over
// the lanes that take part).
template <int BODY, int NT, int CAP>
__device__ __forceinline__ void force_agent(const StepArgs &a, const int s, int *list,
                                            WarpQueue *wq) {
    const unsigned wmask = __ballot_sync(0xffffffffu, s < a.n);
    if (s >= a.n) return;
    const int lane = threadIdx.x & 31;
    const int nlanes = __popc(wmask);           // active lanes form a prefix
    const int i = a.perm[s];
    const int sid = a.scen_of[i];
    const ScenDev sc = a.scen[sid];
    const float4 me = a.cull[s];
    const int my_cell = a.key[i];

    double fx, fy, tq, phi0;
    agent_prologue<BODY>(a, i, fx, fy, tq, phi0);

    // Agent-agent (core/interactions.py:147-166), contributions summed in the
    // reference's visiting order for this agent
    if (a.nodes & N_AGENT) {
        int *mylist = list + threadIdx.x;
        EnumState st{0, -1};
        if (BODY == 0) {
            const Circ A = load_circ(a.stage, s);
            while (true) {
                int nl = enumerate_candidates<NT, CAP>(a, sc, s, my_cell, me, mylist, st);
                for (int k = 0; k < nl; ++k) {
                    int v = mylist[k * NT];
                    const Circ B = load_circ(a.stage, v < 0 ? ~v : v);
                    pair_circular_me(A, B, fx, fy);
                }
                if (st.ck >= 9) break;
            }
        } else {
            const TC A = load_tc(a.stage, s);
            const float4 meF0 = a.stage_f[2 * s], meF1 = a.stage_f[2 * s + 1];
            WarpQueue &q = wq[threadIdx.x >> 5];
            while (true) {
                int nl = enumerate_candidates<NT, CAP>(a, sc, s, my_cell, me, mylist, st);
                int kmax = __reduce_max_sync(wmask, (unsigned)nl);
                for (int k = 0; k < kmax; ++k) {
                    bool act = k < nl;
                    int v = act ? mylist[k * NT] : 0;
                    int t = v < 0 ? ~v : v;
                    tc_pair_step(A, me, meF0, meF1, a, act, t, v < 0, q, lane, wmask, nlanes,
                                 fx, fy, tq);
                }
                if (!__any_sync(wmask, st.ck < 9)) break;
            }
        }
    }
    agent_epilogue<BODY>(a, s, i, sid, sc, me, my_cell, fx, fy, tq, phi0);
}

// Lane-group form: L lanes share one agent (32 / L agents per warp).  The
// agent's candidates are the slots of its 3 x 3 neighbour cells, which in
// the reference's visiting order ((dx, dy) lexicographic, ascending within a
// cell) are three runs of consecutive slots, one per dx.  The group culls L
// candidates at a time, appends the near ones to its queue in order, and
// evaluates L queued pairs at once, one per lane; the pair forces are then
// added in queue order by every lane of the group (shuffles), so each lane
// holds the same, reference-ordered sum.  The first lane of the group then
// adds the walls and integrates.  Called by all 32 lanes of the warp.
template <int BODY, int L>
__device__ __forceinline__ void force_agent_group(const StepArgs &a, const int s,
                                                  int *gq, WarpQueue *wq) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr unsigned GMASK = L == 32 ? 0xffffffffu : ((1u << L) - 1u);
    const int lane = threadIdx.x & 31;
    const int r = lane & (L - 1);
    const int g0 = lane & ~(L - 1);              // first lane of the group
    const bool valid = s < a.n;
    int i = 0, sid = 0, my_cell = 0;
    ScenDev sc;
    float4 me = make_float4(0.f, 0.f, 0.f, 0.f);
    double fx = 0.0, fy = 0.0, tq = 0.0, phi0 = 0.0;
    if (valid) {
        i = a.perm[s];
        sid = a.scen_of[i];
        sc = a.scen[sid];
        me = a.cull[s];
        my_cell = a.key[i];
        agent_prologue<BODY>(a, i, fx, fy, tq, phi0);
    }
    if (a.nodes & N_AGENT) {
        // candidate runs, one per dx in -1, 0, 1 (empty where off the grid)
        int rb[3] = {0, 0, 0}, re[3] = {0, 0, 0};
        if (valid) {
            const int local = my_cell - sc.cell_base;
            const int ix = local / sc.ny, iy = local - ix * sc.ny;
            const int jy0 = iy > 0 ? iy - 1 : 0, jy1 = iy + 1 < sc.ny ? iy + 1 : sc.ny - 1;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int jx = ix + d - 1;
                if (jx < 0 || jx >= sc.nx) continue;
                const int c0 = sc.cell_base + jx * sc.ny;
                rb[d] = __ldg(&a.start[c0 + jy0]);
                re[d] = __ldg(&a.start[c0 + jy1 + 1]);
            }
        }
        // current run: index `run`, end `cur_e`; runs are selected without
        // dynamic array indexing so that they stay in registers
        int run = 0, cur_e = 0, p = 0;
        bool done = true;
#pragma unroll
        for (int d = 2; d >= 0; --d)
            if (rb[d] < re[d]) { run = d; p = rb[d]; cur_e = re[d]; done = false; }
        int qlen = 0;
        Circ Ac;
        TC At;
        float4 meF0 = make_float4(0.f, 0.f, 0.f, 0.f), meF1 = meF0;
        if (valid) {
            if (BODY == 0) Ac = load_circ(a.stage, s);
            else {
                At = load_tc(a.stage, s);
                meF0 = a.stage_f[2 * s];
                meF1 = a.stage_f[2 * s + 1];
            }
        }
        while (true) {
            // fill: until the group's queue holds L pairs or its candidates run out
            while (true) {
                const bool need = !done && qlen < L;
                if (!__any_sync(FULL, need)) break;
                const int t = p + r;
                const bool near = need && t < cur_e && t != s &&
                                  !pair_far(me, __ldg(&a.cull[t]));
                const unsigned gb = (__ballot_sync(FULL, near) >> g0) & GMASK;
                if (near) {
                    // orientation: the dx = +1 run follows the agent's cell, the dx = -1
                    // run precedes it, and within dx = 0 slot order decides
                    const bool me_first = run == 2 || (run == 1 && t > s);
                    gq[qlen + __popc(gb & ((1u << r) - 1u))] = me_first ? ~t : t;
                }
                if (need) {
                    qlen += __popc(gb);
                    p += L;
                    if (p >= cur_e) {                // next non-empty run, if any
                        if (run < 1 && rb[1] < re[1]) {
                            run = 1; p = rb[1]; cur_e = re[1];
                        } else if (run < 2 && rb[2] < re[2]) {
                            run = 2; p = rb[2]; cur_e = re[2];
                        } else {
                            done = true;
                        }
                    }
                }
                __syncwarp();
            }
            const int cnt = qlen < L ? qlen : L;
            const int cmax = (int)__reduce_max_sync(FULL, (unsigned)cnt);
            if (cmax == 0) break;
            const bool act = r < cnt;
            const int v = act ? gq[r] : 0;
            const int t = v < 0 ? ~v : v;
            double Fx = 0.0, Fy = 0.0, Tq = 0.0;
            bool inter = false;
            if (BODY == 0) {
                if (act) inter = pair_circular_eval(Ac, load_circ(a.stage, t), Fx, Fy);
            } else {
                inter = tc_pair_eval(At, me, meF0, meF1, a, act, t, v < 0, wq[threadIdx.x >> 5],
                                     lane, FULL, 32, Fx, Fy, Tq);
            }
            // reference-ordered sum over the group's evaluated pairs
            const unsigned ib = __ballot_sync(FULL, inter);
            for (int k = 0; k < cmax; ++k) {
                const double ax = __shfl_sync(FULL, Fx, g0 + k);
                const double ay = __shfl_sync(FULL, Fy, g0 + k);
                double aq = 0.0;
                if (BODY == 1) aq = __shfl_sync(FULL, Tq, g0 + k);
                if ((ib >> (g0 + k)) & 1u) {
                    fx = fx + ax;
                    fy = fy + ay;
                    if (BODY == 1) tq = tq + aq;
                }
            }
            // drop the evaluated pairs from the queue
            const int rest = qlen - cnt;
            const int moved = r < rest ? gq[cnt + r] : 0;
            __syncwarp();
            if (r < rest) gq[r] = moved;
            qlen = rest;
            __syncwarp();
        }
    }
    if (!valid || r != 0) return;
    agent_epilogue<BODY>(a, s, i, sid, sc, me, my_cell, fx, fy, tq, phi0);
}

// Persistent grid (resident blocks only): each warp claims 32 consecutive
// cell-sorted agents at a time from a counter, so uneven per-agent work
// spreads over all SMs without a partial last wave.  NT threads per block,
// CAP candidates staged per thread per pass (launch variants).
template <int BODY, int NT, int CAP>
__global__ void __launch_bounds__(NT) k_forces(StepArgs a) {
    extern __shared__ unsigned char smem[];
    int *list = reinterpret_cast<int *>(smem);
    WarpQueue *wq = reinterpret_cast<WarpQueue *>(smem + sizeof(int) * CAP * NT);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(a.work, 1);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        if (chunk * 32 >= a.n) return;
        force_agent<BODY, NT, CAP>(a, chunk * 32 + lane, list, wq);
        __syncwarp();
    }
}

// Persistent lane-group grid: each warp claims 32 / L consecutive cell-sorted
// agents at a time from a counter.
constexpr int NTG = 128;

template <int BODY, int L>
__global__ void __launch_bounds__(NTG) k_forces_group(StepArgs a) {
    extern __shared__ unsigned char smem[];
    int *gq_all = reinterpret_cast<int *>(smem);                 // 2L ints per group
    WarpQueue *wq = reinterpret_cast<WarpQueue *>(smem + sizeof(int) * 2 * NTG);
    int *gq = gq_all + 2 * (threadIdx.x & ~(L - 1));
    const int lane = threadIdx.x & 31;
    for (;;) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(a.work, 1);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        const int s0 = chunk * (32 / L);
        if (s0 >= a.n) return;
        force_agent_group<BODY, L>(a, s0 + lane / L, gq, wq);
        __syncwarp();
    }
}

// ---- compute-once pair pipeline --------------------------------------
//
// The reference visits every unordered pair once and adds both agents'
// forces (interactions.py:147-166); the per-thread and lane-group kernels
// instead evaluate each pair from both sides.  This pipeline evaluates each
// pair once, in the reference's orientation (the lower cell-sorted slot is
// the pair's first agent: the forward half-stencil reaches exactly the cells
// with a larger flat index), and sums each agent's pair results in its
// visiting order afterwards:
//   k_nl_count / scan / k_nl_fill: every agent's near candidates (float32
//     cull, symmetric) in ascending slot order, which is its visiting order;
//   k_pairs: for every entry with a later slot, both sides of the pair, the
//     first side into the entry, the second into the partner's entry for
//     this agent (found in the partner's earlier-slot part); a kind byte
//     per entry, a 32-byte record only for a force;
//   k_forces_gather: per agent, the entries' forces added in list order,
//     then walls and integration;
//   k_forces_fallback: the agents the gather left (a signed-zero torque
//     decides), evaluated again with exact signs.
// When the entries exceed the allocated capacity the pair kernels do
// nothing and k_forces_fallback runs the lane-group path instead; nl_off[n]
// tells the host how much to allocate.

// Agent s's candidate runs, one per dx in -1, 0, 1 (empty where off the grid).
__device__ __forceinline__ void candidate_runs(const StepArgs &a, const ScenDev &sc,
                                               int my_cell, int rb[3], int re[3]) {
    const int local = my_cell - sc.cell_base;
    const int ix = local / sc.ny, iy = local - ix * sc.ny;
    const int jy0 = iy > 0 ? iy - 1 : 0, jy1 = iy + 1 < sc.ny ? iy + 1 : sc.ny - 1;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        rb[d] = 0;
        re[d] = 0;
        const int jx = ix + d - 1;
        if (jx < 0 || jx >= sc.nx) continue;
        const int c0 = sc.cell_base + jx * sc.ny;
        rb[d] = __ldg(&a.start[c0 + jy0]);
        re[d] = __ldg(&a.start[c0 + jy1 + 1]);
    }
}

// Float32 guess that a forward pair will need the social force: within
// sight, and the two enclosing circles (radius = extent) on a collision
// course (their time-to-collision discriminant positive, and approaching or
// overlapping).  Sub-circles lie inside the enclosing circles, so a pair with
// a positive time-to-collision always passes, up to rounding.  Only the order
// of the flat pair list depends on the guess (pairs guessed so come first, so
// that warps of the pair kernel mostly take the same branches); every pair
// writes only its own two entries, so no result does.
__device__ __forceinline__ bool social_guess(float4 me, float4 o) {
    const float dx = me.x - o.x, dy = me.y - o.y;
    const float2 vm = unpack_velocity(me.w), vo = unpack_velocity(o.w);
    const float vx = vm.x - vo.x, vy = vm.y - vo.y;
    const float re = me.z + o.z;
    const float x2 = dx * dx + dy * dy;
    const float b = -(dx * vx + dy * vy);
    const float c = x2 - re * re;
    const float disc = b * b - (vx * vx + vy * vy) * c;
    const float sight = 3.0f + re;                      // skin distance below 3 m
    return x2 < sight * sight && disc > 0.0f && (b > 0.0f || c < 0.0f);
}

// Near lists in two passes over the same candidate chunks (CW consecutive
// candidates of one run per chunk: C per lane, candidate base + c L + r on
// lane r).  k_nl_count evaluates the bound check and the social-force guess,
// counts, and keeps each chunk's bits (near low 16, guessed high 16; bit j is
// candidate base + j) in the agent's mask row; k_nl_fill then places the
// entries from the masks alone.  An agent with more chunks than a row holds is
// evaluated again by the fill.
// Chunks of 16 candidates for every lane count: the per-chunk work (the run
// and its bounds, the counts, the row word) is spread over more candidates
// (4 lanes x 4 against 4 x 2: the step 0.320 -> 0.315 ms at 100k agents).
template <int L> struct NlChunk {
    static constexpr int C = L == 4 ? 4 : (L <= 8 ? 2 : 1);   // candidates per lane and chunk
    static constexpr int CW = C * L;                   // candidates per chunk, <= 16
    static constexpr unsigned CMASK = (1u << CW) - 1u;
};

// Bits of a chunk's candidates that follow slot s (bit j: candidate base + j).
template <int L>
__device__ __forceinline__ unsigned later_bits(int s, int base) {
    const int k0 = s - base + 1;
    return k0 <= 0 ? NlChunk<L>::CMASK
                   : (k0 >= NlChunk<L>::CW ? 0u : (NlChunk<L>::CMASK & ~((1u << k0) - 1u)));
}

template <int L>
__global__ void __launch_bounds__(NTG) k_nl_count(StepArgs a) {
    pdl_enter();
    static_assert(NlChunk<L>::CW <= 16, "two 16-bit masks per 32-bit word");
    constexpr int C = NlChunk<L>::C, CW = NlChunk<L>::CW;
    constexpr unsigned GMASK = (1u << L) - 1u;
    const int lane = threadIdx.x & 31;
    const int r = lane & (L - 1), g0 = lane & ~(L - 1);
    const unsigned gm = GMASK << g0;
    const int s = (int)(((long long)blockIdx.x * NTG + threadIdx.x) / L);
    const bool valid = s < a.n;                           // whole groups
    float4 me = make_float4(0.f, 0.f, 0.f, 0.f);
    int rb[3] = {0, 0, 0}, re[3] = {0, 0, 0};
    if (valid) {
        const int i = a.perm[s];
        const ScenDev sc = a.scen[a.scen_of[i]];
        me = a.cull[s];
        candidate_runs(a, sc, a.key[i], rb, re);
    }
    // The group's chunks, run after run: the agents of one cell have the
    // same runs, and the warp steps through the most chunks any of its groups
    // has, so that its ballots take all 32 lanes without divergence.
    const int n0 = (re[0] - rb[0] + CW - 1) / CW, n1 = (re[1] - rb[1] + CW - 1) / CW;
    const int mine = n0 + n1 + (re[2] - rb[2] + CW - 1) / CW;
    const int most = __reduce_max_sync(0xffffffffu, mine);
    // the group's mask row is staged in shared memory and written out whole
    __shared__ unsigned srow[(NTG / L) * NL_MASK_CHUNKS];
    unsigned *row = srow + (threadIdx.x / L) * NL_MASK_CHUNKS;
    int cnt = 0, fwd = 0, soc = 0, ch = 0;
    for (int it = 0; it < most; ++it) {
        const bool on = it < mine;
        // run d of chunk `it` (selects, so that the runs stay in registers)
        const bool r0 = it < n0, r1 = !r0 && it < n0 + n1;
        const int base = (r0 ? rb[0] : (r1 ? rb[1] : rb[2])) +
                         (it - (r0 ? 0 : (r1 ? n0 : n0 + n1))) * CW;
        const int end = r0 ? re[0] : (r1 ? re[1] : re[2]);
        unsigned nb = 0, sb = 0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int t = base + c * L + r;
            bool near = false, guess = false;
            if (on && t < end && t != s) {
                const float4 o = __ldg(&a.cull[t]);
                near = !pair_far(me, o);
                if (near && t > s) guess = social_guess(me, o);
            }
            nb |= ((__ballot_sync(0xffffffffu, near) >> g0) & GMASK) << (c * L);
            sb |= ((__ballot_sync(0xffffffffu, guess) >> g0) & GMASK) << (c * L);
        }
        if (on) {
            if (r == 0 && ch < NL_MASK_CHUNKS) row[ch] = nb | (sb << 16);
            ++ch;
            cnt += __popc(nb);
            fwd += __popc(nb & later_bits<L>(s, base));
            soc += __popc(sb);
        }
    }
    if (!valid) return;
    __syncwarp(gm);
    unsigned *mrow = a.nl_mask + (size_t)s * NL_MASK_CHUNKS;
    const int nst = ch < NL_MASK_CHUNKS ? ch : NL_MASK_CHUNKS;
    for (int c = r; c < nst; c += L) mrow[c] = row[c];
    if (r == 0) {
        a.nl_cnt[s] = cnt;
        a.fw_cnt[s] = fwd;
        a.fs_cnt[s] = soc;
        a.nl_nch[s] = ch;
    }
}

template <int L>
__global__ void __launch_bounds__(NTG) k_nl_fill(StepArgs a) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {     // k_pairs' work counter, pairs deferred,
        a.work[0] = 0;                              // jobs of the force pass
        a.work[1] = 0;
        a.work[2] = 0;
        a.work[3] = 0;
    }
    if (a.nl_off[a.n] > a.nl_cap) return;                 // over capacity: fallback
    constexpr unsigned GMASK = (1u << L) - 1u;
    const int lane = threadIdx.x & 31;
    const int r = lane & (L - 1), g0 = lane & ~(L - 1);
    const unsigned gm = GMASK << g0;
    const int s = (int)(((long long)blockIdx.x * NTG + threadIdx.x) / L);
    if (s >= a.n) return;                                 // whole groups leave together
    const int i = a.perm[s];
    const ScenDev sc = a.scen[a.scen_of[i]];
    int rb[3], re[3];
    candidate_runs(a, sc, a.key[i], rb, re);
    // the scans left offsets relative to the slot's tile: add the tile's
    // offset (written back below, once every lane of the group has read)
    const int off_at = (a.n + SCAN_TILE - 1) / SCAN_TILE + 1 + s / SCAN_TILE;
    const int nl_s = a.nl_off[s] + a.nl_scan[off_at];
    const int fw_s = a.fw_off[s] + a.fw_scan[off_at];
    const int fs_s = a.fs_off[s] + a.fs_scan[off_at];
    // entries with a later slot follow all earlier ones (ascending order)
    const int fwd0 = nl_s + (a.nl_cnt[s] - a.fw_cnt[s]);
    int pos = nl_s;
    // the flat list of pairs: first every pair guessed to need the social
    // force, then the others, each part in slot order
    int p0 = fs_s;
    int p1 = a.fs_off[a.n] + (fw_s - fs_s);
    const unsigned lower = (1u << r) - 1u;
    if (a.nl_nch[s] <= NL_MASK_CHUNKS) {
        constexpr int C = NlChunk<L>::C, CW = NlChunk<L>::CW;
        const unsigned *mrow = a.nl_mask + (size_t)s * NL_MASK_CHUNKS;
        int ch = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            for (int base = rb[d]; base < re[d]; base += CW) {
                const unsigned m = mrow[ch++];
                const unsigned nb = m & 0xffffu, sb = m >> 16;
                const unsigned fb = nb & later_bits<L>(s, base);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const int j = c * L + r;
                    const unsigned below = (1u << j) - 1u;
                    const int t = base + j;
                    if ((nb >> j) & 1u) {
                        const int e = pos + __popc(nb & below);
                        a.nl_idx[e] = t;
                        if (t > s)
                            a.fw_pairs[((sb >> j) & 1u) ? p0 + __popc(sb & below)
                                                        : p1 + __popc(fb & ~sb & below)] =
                                make_int2(s, e);
                    }
                }
                pos += __popc(nb);
                p0 += __popc(sb);
                p1 += __popc(fb & ~sb);
            }
    } else {
        const float4 me = a.cull[s];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            for (int base = rb[d]; base < re[d]; base += L) {
                const int t = base + r;
                bool near = false, guess = false;
                if (t < re[d] && t != s) {
                    const float4 o = __ldg(&a.cull[t]);
                    near = !pair_far(me, o);
                    if (near && t > s) guess = social_guess(me, o);
                }
                const unsigned gb = (__ballot_sync(gm, near) >> g0) & GMASK;
                const unsigned fb = (__ballot_sync(gm, near && t > s) >> g0) & GMASK;
                const unsigned sb = (__ballot_sync(gm, guess) >> g0) & GMASK;
                if (near) {
                    const int e = pos + __popc(gb & lower);
                    a.nl_idx[e] = t;
                    if (t > s)
                        a.fw_pairs[guess ? p0 + __popc(sb & lower)
                                         : p1 + __popc(fb & ~sb & lower)] = make_int2(s, e);
                }
                pos += __popc(gb);
                p0 += __popc(sb);
                p1 += __popc(fb & ~sb);
            }
    }
    __syncwarp(gm);
    if (r == 0) {
        a.nl_fwd[s] = fwd0;
        a.nl_off[s] = nl_s;
        a.fw_off[s] = fw_s;
        a.fs_off[s] = fs_s;
    }
}

// Entry of `s` in the earlier-slot part of `t`'s near list (s < t), or -1.
// The part is scanned 32 entries at a time with eight independent 16-byte
// loads from a 4-aligned start (one memory round trip for most lists);
// entries outside the part are ignored.  Near the end of the allocation a
// binary search replaces the wide loads.  k_pairs, bound by float64 latency,
// gains from the single round trip; the float32 pass, bound by instruction
// issue, takes the binary search (partner_entry_search: about a fifth of the
// instructions, 57 -> 45 us per step at 100k ThreeCircle agents).
__device__ __forceinline__ int partner_entry(const StepArgs &a, int t, int s) {
    int lo = __ldg(&a.nl_off[t]), hi = __ldg(&a.nl_fwd[t]);
    const int end = hi;
    for (int base = lo & ~3; base < end && base + 32 <= a.nl_cap; base += 32) {
        const int4 *p = reinterpret_cast<const int4 *>(a.nl_idx + base);
        int4 q[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) q[k] = __ldg(p + k);
        int found = -1;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int e = base + 4 * k;
            if (q[k].x == s && e >= lo && e < end) found = e;
            if (q[k].y == s && e + 1 >= lo && e + 1 < end) found = e + 1;
            if (q[k].z == s && e + 2 >= lo && e + 2 < end) found = e + 2;
            if (q[k].w == s && e + 3 >= lo && e + 3 < end) found = e + 3;
        }
        if (found >= 0) return found;
        lo = base + 32 > lo ? base + 32 : lo;
    }
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.nl_idx[mid]) < s) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && __ldg(&a.nl_idx[lo]) == s) ? lo : -1;
}

// The same by binary search over the part (slots ascending).
__device__ __forceinline__ int partner_entry_search(const StepArgs &a, int t, int s) {
    int lo = __ldg(&a.nl_off[t]), hi = __ldg(&a.nl_fwd[t]);
    const int end = hi;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.nl_idx[mid]) < s) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && __ldg(&a.nl_idx[lo]) == s) ? lo : -1;
}

// One side of a pair into its near-list entry: the entry's kind byte, and
// for a force its 32-byte record (fx, fy, torque).  A pair without a force
// contributes (+0, +0) and a signed-zero torque.
constexpr unsigned char KIND_NONE = 0, KIND_ZERO = 1, KIND_FORCE = 3;

__device__ __forceinline__ void put_pair(const StepArgs &a, int e, int res, double fx, double fy,
                                         double tq) {
    unsigned char kind = KIND_NONE;
    if (res == RES_FORCE) {
        kind = KIND_FORCE;
        double4_32a v;
        v.x = fx; v.y = fy; v.z = tq; v.w = 0.0;   // w unused (32-byte records)
        *reinterpret_cast<double4_32a *>(a.nl_res + (size_t)e * RES_D) = v;
    } else if (res == RES_ZERO) {
        kind = KIND_ZERO;
    }
    a.nl_kind[e] = kind;
}

// The reverse of a pair without a force (no contact, no time to collision
// in (0, 30]) adds nothing to either side: its entries are marked empty
// (kind 0) and k_adj_gather skips them.
__device__ __forceinline__ void put_adj_zero(const StepArgs &a, int e) { a.nl_kind[e] = 0; }

// The pairs of the flat list's second part (not guessed to need the social
// force), in float32 alone (tc_pair_light, circ_pair_light): a decided pair
// writes the kind bytes of both its entries (ADJ: marks them empty); the
// others are appended to defer_list for k_pairs (ADJ: k_adj_pairs), which
// takes them after the first part.  Few registers, so many warps per SM hide
// the loads.  Warps take 32 consecutive pairs at a time, in turn.
template <int BODY, bool ADJ = false>
__global__ void __launch_bounds__(NTG) k_pairs_light(StepArgs a) {
    pdl_enter();
    constexpr unsigned FULL = 0xffffffffu;
    if (a.nl_off[a.n] > a.nl_cap) return;
    const int lane = threadIdx.x & 31;
    const int k0 = a.fs_off[a.n], npairs = a.fw_off[a.n];
    const int warps = gridDim.x * (NTG / 32);
    // ThreeCircle: the few pairs that need the pre-selection or the sub-pair
    // roots wait in a per-warp queue and are evaluated 32 at a time, so that
    // the warps do not run those stages for one lane each
    __shared__ int slow_q[NTG / 32][64];
    int *sq = slow_q[threadIdx.x >> 5];
    int nq = 0;                                            // warp-uniform
    auto finish = [&](int k, int s, int e, int t, int res, bool on) {
        const unsigned dm = __ballot_sync(FULL, on && res == RES_DEFER);
        if (dm) {
            int d0 = 0;
            if (lane == 0) d0 = atomicAdd(a.work + 1, __popc(dm));
            d0 = __shfl_sync(FULL, d0, 0);
            if ((dm >> lane) & 1u) a.defer_list[d0 + __popc(dm & ((1u << lane) - 1u))] = k;
        }
        if (on && res != RES_DEFER) {
            const int eq = partner_entry_search(a, t, s);
            if (ADJ) {
                put_adj_zero(a, e);
                if (eq >= 0) put_adj_zero(a, eq);
            } else {
                put_pair(a, e, res, 0.0, 0.0, 0.0);
                if (eq >= 0) put_pair(a, eq, res, 0.0, 0.0, 0.0);
            }
            if (eq < 0) atomicOr(a.err, ERR_NEAR_LIST);
        }
    };
    // the queue's first `count` pairs, one per lane, through all of tc_pair_light
    auto drain = [&](int count) {
        const bool on = lane < count;
        int k = 0, s = 0, e = 0, t = 0, res = RES_NONE;
        if (on) {
            k = sq[lane];
            const int2 pe = __ldg(&a.fw_pairs[k]);
            s = pe.x;
            e = pe.y;
            t = __ldg(&a.nl_idx[e]);
            res = tc_pair_light(a, s, t);
        }
        __syncwarp(FULL);
        finish(k, s, e, t, res, on);
    };
    for (int base = k0 + (blockIdx.x * (NTG / 32) + (threadIdx.x >> 5)) * 32; base < npairs;
         base += warps * 32) {
        const int k = base + lane;
        int res = RES_NONE, s = 0, e = 0, t = 0;
        if (k < npairs) {
            const int2 pe = __ldg(&a.fw_pairs[k]);
            s = pe.x;
            e = pe.y;
            t = __ldg(&a.nl_idx[e]);
            res = BODY == 1 ? tc_pair_light_quick(a, s, t) : circ_pair_light(a, s, t);
        }
        if (BODY == 1) {
            const unsigned sm = __ballot_sync(FULL, k < npairs && res == RES_SLOW);
            if ((sm >> lane) & 1u) sq[nq + __popc(sm & ((1u << lane) - 1u))] = k;
            nq += __popc(sm);
            __syncwarp(FULL);
        }
        finish(k, s, e, t, res, k < npairs && res != RES_SLOW);
        if (BODY == 1 && nq >= 32) {
            drain(32);
            // the rest moves to the front
            const int rest = nq - 32;
            const int v = lane < rest ? sq[32 + lane] : 0;
            __syncwarp(FULL);
            if (lane < rest) sq[lane] = v;
            __syncwarp(FULL);
            nq = rest;
        }
    }
    if (BODY == 1 && nq > 0) drain(nq);
}

// Job records of the force pass (JOB_Q_TC / JOB_Q_CIRC double2 each).  Jobs
// without contact fill the buffer from the front (count work[2]), jobs with
// contact from the back (count work[3]), so that the force pass's warps take
// one kind at a time: contact is rare, and mixed in it would make nearly
// every warp run the contact arithmetic with a few lanes.
__device__ __forceinline__ int job_cap(const StepArgs &a) { return a.nl_cap / 2 + 1; }
__device__ __forceinline__ int job_record(const StepArgs &a, int j, int n_front) {
    return j < n_front ? j : job_cap(a) - 1 - (j - n_front);
}

__device__ __forceinline__ void put_job(const StepArgs &a, int j, int s, int t, int e, int eq,
                                        const TcJob &J) {
    double2 *p = a.pair_jobs + (size_t)j * JOB_Q_TC;
    *reinterpret_cast<int4 *>(p) = make_int4(s, t, e, eq);
    const long long f = (long long)J.social | ((long long)J.contact << 1) |
                        ((long long)J.k_sel << 2) | ((long long)J.D.pp << 6) |
                        ((long long)J.D.qp << 8);
    p[1] = make_double2(J.tau, J.b_min);
    p[2] = make_double2(J.d_min, J.D.h);
    p[3] = make_double2(J.D.sdx, J.D.sdy);
    p[4] = make_double2(J.D.sd, __longlong_as_double(f));
}

__device__ __forceinline__ int4 get_job(const StepArgs &a, int j, TcJob &J) {
    const double2 *p = a.pair_jobs + (size_t)j * JOB_Q_TC;
    const int4 h = __ldg(reinterpret_cast<const int4 *>(p));
    const double2 q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3), q4 = __ldg(p + 4);
    const long long f = __double_as_longlong(q4.y);
    J.tau = q1.x;
    J.b_min = q1.y;
    J.d_min = q2.x;
    J.D.h = q2.y;
    J.D.sdx = q3.x;
    J.D.sdy = q3.y;
    J.D.sd = q4.x;
    J.social = (f & 1) != 0;
    J.contact = (f & 2) != 0;
    J.k_sel = (int)((f >> 2) & 15);
    J.D.pp = (int)((f >> 6) & 3);
    J.D.qp = (int)((f >> 8) & 3);
    return h;
}

__device__ __forceinline__ void put_job(const StepArgs &a, int j, int s, int t, int e, int eq,
                                        const CircJob &J) {
    double2 *p = a.pair_jobs + (size_t)j * JOB_Q_CIRC;
    *reinterpret_cast<int4 *>(p) = make_int4(s, t, e, eq);
    p[1] = make_double2(J.d, J.dd);
    p[2] = make_double2(J.tau, __longlong_as_double((long long)J.social |
                                                    ((long long)J.contact << 1)));
}

__device__ __forceinline__ int4 get_job(const StepArgs &a, int j, CircJob &J) {
    const double2 *p = a.pair_jobs + (size_t)j * JOB_Q_CIRC;
    const int4 h = __ldg(reinterpret_cast<const int4 *>(p));
    const double2 q1 = __ldg(p + 1), q2 = __ldg(p + 2);
    J.d = q1.x;
    J.dd = q1.y;
    J.tau = q2.x;
    const long long f = __double_as_longlong(q2.y);
    J.social = (f & 1) != 0;
    J.contact = (f & 2) != 0;
    return h;
}

// Every pair of the flat list once: warps claim 32 consecutive pairs at a
// time (consecutive pairs mostly share their first agent) and decide them.
// A pair without a force writes the kind bytes of both its entries.  A pair
// with a force: its forces at once (SPLIT false), or a job of k_pair_forces
// (SPLIT true), which evaluates the jobs with its own register budget and
// with the contact jobs apart.  Which is faster depends on the workload
// (the launch variants hold both).
template <int BODY, bool SPLIT>
__global__ void __launch_bounds__(NTG, (BODY == 0 && SPLIT) ? 6 : 3) k_pairs(StepArgs a) {
    pdl_enter();
    constexpr unsigned FULL = 0xffffffffu;
    if (a.nl_off[a.n] > a.nl_cap) return;
    extern __shared__ unsigned char smem[];
    PairQueue *wq = reinterpret_cast<PairQueue *>(smem);
    const int lane = threadIdx.x & 31;
    // after k_pairs_light: the first part, then the pairs the float32 pass left
    const bool split = a.defer_list != nullptr;
    const int nfirst = split ? a.fs_off[a.n] : a.fw_off[a.n];
    const int npairs = split ? nfirst + a.work[1] : nfirst;
    // the next chunk's pair and partner are loaded before this chunk is
    // evaluated, so that their load latency overlaps its work
    auto claim = [&](int &s_, int &e_, int &t_) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(a.work, 1);
        chunk = __shfl_sync(FULL, chunk, 0);
        const int k_ = chunk * 32 + lane;
        s_ = 0; e_ = 0; t_ = 0;
        if (k_ < npairs) {
            const int kk = k_ < nfirst ? k_ : __ldg(&a.defer_list[k_ - nfirst]);
            const int2 pe = __ldg(&a.fw_pairs[kk]);
            s_ = pe.x;
            e_ = pe.y;
            t_ = __ldg(&a.nl_idx[e_]);
        }
        return chunk * 32 < npairs ? k_ : -1;
    };
    int ns, ne, nt;
    int nk = claim(ns, ne, nt);
    for (;;) {
        if (nk < 0) return;
        const int k = nk, s = ns, e = ne, t = nt;
        const bool act = k < npairs;
        nk = claim(ns, ne, nt);
        int kind = RES_NONE;
        TcJob tj;
        CircJob cj;
        bool contact = false;
        if (BODY == 0) {
            if (act) {
                kind = circ_pair_decide(load_circ(a.stage, s), load_circ(a.stage, t), cj);
                contact = kind == RES_FORCE && cj.contact;
            }
        } else {
            TC At;
            float4 me = make_float4(0.f, 0.f, 0.f, 0.f), meF0 = me, meF1 = me;
            if (act) {
                At = load_tc(a.stage, s);
                me = __ldg(&a.cull[s]);
                meF0 = __ldg(&a.stage_f[2 * s]);
                meF1 = __ldg(&a.stage_f[2 * s + 1]);
            } else {
                At = load_tc(a.stage, 0);
            }
            kind = tc_pair_decide(At, me, meF0, meF1, a, act, t, wq[threadIdx.x >> 5], lane, tj);
            contact = kind == RES_FORCE && tj.contact;
        }
        int eq = -1;
        if (act) {
            eq = partner_entry(a, t, s);
            if (eq < 0) atomicOr(a.err, ERR_NEAR_LIST);
            if (kind != RES_FORCE) {
                put_pair(a, e, kind, 0.0, 0.0, 0.0);
                if (eq >= 0) put_pair(a, eq, kind, 0.0, 0.0, 0.0);
            } else if (!SPLIT) {
                double fpx, fpy, tp = 0.0, fqx, fqy, tq = 0.0;
                if (BODY == 0)
                    circ_pair_force(load_circ(a.stage, s), load_circ(a.stage, t), cj, fpx, fpy,
                                    fqx, fqy);
                else
                    tc_pair_force(load_tc(a.stage, s), load_tc(a.stage, t), tj, fpx, fpy, tp, fqx,
                                  fqy, tq);
                put_pair(a, e, RES_FORCE, fpx, fpy, tp);
                if (eq >= 0) put_pair(a, eq, RES_FORCE, fqx, fqy, tq);
            }
        }
        if (SPLIT) {
            // jobs in warp order: without contact at the front, with it at the back
            const unsigned jm = __ballot_sync(FULL, act && kind == RES_FORCE && !contact);
            const unsigned cm = __ballot_sync(FULL, act && kind == RES_FORCE && contact);
            if (jm | cm) {
                int j0 = 0, c0 = 0;
                if (lane == 0) {
                    if (jm) j0 = atomicAdd(a.work + 2, __popc(jm));
                    if (cm) c0 = atomicAdd(a.work + 3, __popc(cm));
                }
                j0 = __shfl_sync(FULL, j0, 0);
                c0 = __shfl_sync(FULL, c0, 0);
                const unsigned below = (1u << lane) - 1u;
                int rec = -1;
                if ((jm >> lane) & 1u) rec = j0 + __popc(jm & below);
                if ((cm >> lane) & 1u) rec = job_cap(a) - 1 - (c0 + __popc(cm & below));
                if (rec >= 0) {
                    if (BODY == 0) put_job(a, rec, s, t, e, eq, cj);
                    else put_job(a, rec, s, t, e, eq, tj);
                }
            }
        }
    }
}

// The force pass: one lane per job of k_pairs, both sides' forces (and
// torques) into the pair's two entries; the jobs without contact first.
template <int BODY>
__global__ void __launch_bounds__(NTG, 5) k_pair_forces(StepArgs a) {
    pdl_enter();
    if (a.nl_off[a.n] > a.nl_cap) return;
    const int n_front = a.work[2], njobs = n_front + a.work[3];
    for (int j = blockIdx.x * NTG + threadIdx.x; j < njobs; j += gridDim.x * NTG) {
        const int rec = job_record(a, j, n_front);
        double fpx, fpy, tp = 0.0, fqx, fqy, tq = 0.0;
        int4 h;
        if (BODY == 0) {
            CircJob J;
            h = get_job(a, rec, J);
            circ_pair_force(load_circ(a.stage, h.x), load_circ(a.stage, h.y), J, fpx, fpy, fqx,
                            fqy);
        } else {
            TcJob J;
            h = get_job(a, rec, J);
            tc_pair_force(load_tc(a.stage, h.x), load_tc(a.stage, h.y), J, fpx, fpy, tp, fqx, fqy,
                          tq);
        }
        put_pair(a, h.z, RES_FORCE, fpx, fpy, tp);
        if (h.w >= 0) put_pair(a, h.w, RES_FORCE, fqx, fqy, tq);
    }
}

// Torque of slot s's side of the interacting pair (s, t) that exerts no
// force: r x (+0, +0) with the exact moment arm r, as tc_pair_force computes
// it for a pair with a force (the same distance search and arms).
__device__ __noinline__ double tc_zero_force_torque(const StepArgs &a, int s, int t) {
    const int p = s < t ? s : t, q = s < t ? t : s;
    const TC A = load_tc(a.stage, p), B = load_tc(a.stage, q);
    const float4 meC = __ldg(&a.cull[p]), meF0 = __ldg(&a.stage_f[2 * p]),
                 meF1 = __ldg(&a.stage_f[2 * p + 1]);
    const float4 oC = __ldg(&a.cull[q]), oF0 = __ldg(&a.stage_f[2 * q]),
                 oF1 = __ldg(&a.stage_f[2 * q + 1]);
    const float dxt = (meC.x - oC.x) + (meF0.x - oF0.x);
    const float dyt = (meC.y - oC.y) + (meF0.y - oF0.y);
    const float mox[3] = {0.f, meF1.x, meF1.z}, moy[3] = {0.f, meF1.y, meF1.w};
    const float oox[3] = {0.f, oF1.x, oF1.z}, ooy[3] = {0.f, oF1.y, oF1.w};
    const float mr[3] = {meF0.z, meF0.w, meF0.w}, orr[3] = {oF0.z, oF0.w, oF0.w};
    const TcPre pre = tc_presel(dxt, dyt, mox, moy, oox, ooy, mr, orr, true);
    const TcDist D = tc_distance_exact(A, B, pre.seq);
    double npx, npy, nqx, nqy, rpx, rpy, rqx, rqy;
    tc_moment_arms(A, B, D, npx, npy, nqx, nqy, rpx, rpy, rqx, rqy);
    return s == p ? rpx * 0.0 - rpy * 0.0 : rqx * 0.0 - rqy * 0.0;
}

// Agent in slot s from its near-list results: one lane per agent, entries
// added in list order (32-byte records, one sector each), then walls and
// integration at full lane occupancy.
// A record without a force adds (+0, +0) and a signed-zero torque: that
// changes a running force only from -0 to +0, and a running torque only when
// it is -0, the one case in which the torque's sign is needed.  The gather
// then leaves the agent (writing nothing) to the next kernel
// (k_forces_fallback, which otherwise has nothing to do), which runs it again
// with EXACT, evaluating those signs.
// The per-agent terms before agent-agent (navigation, fluctuation,
// orientation, adjusting) of every agent, one lane per agent, for the
// gather: they do not depend on the pairs, so they run beside the near-list
// build (which leaves the float64 pipe idle).
template <int BODY>
__device__ __forceinline__ void prologue_agent(const StepArgs &a, const int i) {
    double fx, fy, tq, phi0;
    agent_prologue<BODY>(a, i, fx, fy, tq, phi0);
    double4_32a v;
    v.x = fx; v.y = fy; v.z = tq; v.w = phi0;
    double4_32a *p = reinterpret_cast<double4_32a *>(a.pro + PRO_D * (size_t)i);
    p[0] = v;
    // the integrator's old accelerations: this step's force_prev / m and
    // torque_prev / I, inputs no kernel before the gather changes
    if (a.nodes & N_INTEG) {
        double *const *col = a.col;
        const double m = col[MASS][i];
        double4_32a w;
        w.x = col[FPX][i] / m;
        w.y = col[FPY][i] / m;
        w.z = BODY == 1 ? col[TORQUE_PREV][i] / col[INERTIA][i] : 0.0;
        w.w = 0.0;
        p[1] = w;
    }
}

template <int BODY>
__global__ void __launch_bounds__(128) k_prologue(StepArgs a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
        prologue_agent<BODY>(a, i);
}

// Bytes j of a 4-byte word of kinds with lo <= j < hi (0xff each).
__device__ __forceinline__ unsigned byte_keep(int lo, int hi) {
    unsigned m = 0xffffffffu;
    if (lo > 0) m = m << (8 * lo);                   // lo <= 3: the word holds entry lo
    if (hi < 4) m &= 0xffffffffu >> (8 * (4 - hi));  // hi >= 1: the word holds entry hi - 1
    return m;
}

// Adds agent s's near-list results to (fx, fy, tq) in list order, the lanes
// of `lanes` (every lane of the warp running an agent) together.  Each lane
// walks its kind bytes four at a time (the next word loaded while one is
// read) to its next force entry with integer work alone, so that the float64
// adds run once per force entry of the lane with the most, not once per entry
// of any lane.  Entries without a force between two forces act once: each
// turns a -0 force component into +0 (what adding +0 does), which is
// idempotent, and the torque they would need the exact sign of is the same
// for all of them.  Returns false when the torque is -0 at such an entry (the
// agent is left to the exact pass).  The kinds array has 16 bytes of padding,
// so the word holding the last entry is inside it.
template <int BODY>
__device__ __forceinline__ bool add_entries(const StepArgs &a, const int s, const unsigned lanes,
                                            double &fx, double &fy, double &tq) {
    constexpr long long NEG_ZERO = (long long)0x8000000000000000ULL;
    const double4_32a *res = reinterpret_cast<const double4_32a *>(a.nl_res);
    const unsigned *kw = reinterpret_cast<const unsigned *>(a.nl_kind);
    const int o0 = a.nl_off[s], o1 = a.nl_off[s + 1];
    int w = o0 >> 2;
    const int wend = (o1 + 3) >> 2;                  // words holding entries o0 .. o1 - 1
    unsigned fm = 0, zm = 0, nk = 0;                 // force / zero bytes left in word w
    if (w < wend) {
        const unsigned k = __ldg(kw + w);
        if (w + 1 < wend) nk = __ldg(kw + w + 1);
        const unsigned keep = byte_keep(o0 - 4 * w, o1 - 4 * w);
        fm = __vcmpeq4(k, 0x03030303u) & keep;      // KIND_FORCE
        zm = __vcmpeq4(k, 0x01010101u) & keep;      // KIND_ZERO
    }
    bool ok = true;
    for (;;) {
        int e = -1;                                  // the lane's next force entry
        for (;;) {
            if (fm) {
                const int b = __ffs(fm) - 1;         // its byte's lowest bit
                const unsigned thru = ((1u << b) - 1u) | (0xffu << b);
                if (zm & ((1u << b) - 1u)) {         // entries without a force before it
                    if (__double_as_longlong(fx) == NEG_ZERO) fx = 0.0;
                    if (__double_as_longlong(fy) == NEG_ZERO) fy = 0.0;
                    if (BODY == 1 && __double_as_longlong(tq) == NEG_ZERO) {
                        ok = false;
                        fm = zm = 0;
                        w = wend;
                        break;
                    }
                }
                fm &= ~thru;
                zm &= ~thru;
                e = 4 * w + (b >> 3);
                break;
            }
            if (zm) {
                if (__double_as_longlong(fx) == NEG_ZERO) fx = 0.0;
                if (__double_as_longlong(fy) == NEG_ZERO) fy = 0.0;
                zm = 0;
                if (BODY == 1 && __double_as_longlong(tq) == NEG_ZERO) {
                    ok = false;
                    fm = 0;
                    w = wend;
                    break;
                }
            }
            if (++w >= wend) break;
            const unsigned k = nk;
            if (w + 1 < wend) nk = __ldg(kw + w + 1);
            const unsigned keep = byte_keep(o0 - 4 * w, o1 - 4 * w);
            fm = __vcmpeq4(k, 0x03030303u) & keep;
            zm = __vcmpeq4(k, 0x01010101u) & keep;
        }
        if (!__any_sync(lanes, e >= 0)) return ok;
        if (e >= 0) {
            const double4_32a v = res[e];
            fx = fx + v.x;
            fy = fy + v.y;
            if (BODY == 1) tq = tq + v.z;
        }
    }
}

template <int BODY, bool EXACT>
__device__ __forceinline__ void gather_agent(const StepArgs &a, const int s, const int i,
                                             const unsigned lanes = 0u) {
    const int sid = a.scen_of[i];
    const ScenDev sc = a.scen[sid];
    const float4 me = a.cull[s];
    const int my_cell = a.key[i];
    double fx, fy, tq, phi0;
    if (a.pro) {                                   // k_prologue's terms
        const double4_32a v = *reinterpret_cast<const double4_32a *>(a.pro + PRO_D * (size_t)i);
        fx = v.x; fy = v.y; tq = v.z; phi0 = v.w;
    } else {
        agent_prologue<BODY>(a, i, fx, fy, tq, phi0);
    }
    if (!EXACT && (a.nodes & N_AGENT)) {
        if (!add_entries<BODY>(a, s, lanes, fx, fy, tq)) {
            a.fix_list[atomicAdd(a.fix_count, 1)] = s;
            return;
        }
    } else if (a.nodes & N_AGENT) {
        const double4_32a *res = reinterpret_cast<const double4_32a *>(a.nl_res);
        const int o1 = a.nl_off[s + 1];
        constexpr long long NEG_ZERO = (long long)0x8000000000000000ULL;
        for (int e = a.nl_off[s]; e < o1; ++e) {
            const unsigned char kind = __ldg(&a.nl_kind[e]);
            if (kind == KIND_FORCE) {
                const double4_32a v = res[e];
                fx = fx + v.x;
                fy = fy + v.y;
                if (BODY == 1) tq = tq + v.z;
            } else if (kind == KIND_ZERO) {
                if (__double_as_longlong(fx) == NEG_ZERO) fx = 0.0;
                if (__double_as_longlong(fy) == NEG_ZERO) fy = 0.0;
                if (BODY == 1 && __double_as_longlong(tq) == NEG_ZERO) {
                    if (!EXACT) {
                        a.fix_list[atomicAdd(a.fix_count, 1)] = s;
                        return;
                    }
                    tq = tq + tc_zero_force_torque(a, s, __ldg(&a.nl_idx[e]));
                }
            }
        }
    }
    agent_epilogue<BODY>(a, s, i, sid, sc, me, my_cell, fx, fy, tq, phi0,
                         a.pro ? a.pro + PRO_D * (size_t)i + 4 : nullptr);
}

// One-warp blocks; 24 resident per SM (80 registers, a few spilled): the
// float64 epilogue's latency wants the warps more than the registers.
constexpr int GATHER_NT = 32;
template <int BODY>
__global__ void __launch_bounds__(GATHER_NT, 24) k_forces_gather(StepArgs a) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.work = 0;   // k_forces_fallback's work counter
    if ((a.nodes & N_AGENT) && a.nl_off[a.n] > a.nl_cap) return;   // k_forces_fallback's step
    // one lane per slot: the entries of neighbouring lanes are neighbours
    // (launched in one-warp blocks: the float64 epilogue spreads evenly
    // over the SMs)
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int left = a.n - blockIdx.x * blockDim.x;       // agents from this warp's first
    const unsigned lanes = left >= 32 ? 0xffffffffu : (1u << left) - 1u;
    if (s < a.n) gather_agent<BODY, false>(a, s, a.perm[s], lanes);
}

// The lane-group kernel, for a step whose near lists exceeded the capacity.
template <int BODY, int L>
__global__ void __launch_bounds__(NTG) k_forces_fallback(StepArgs a) {
    pdl_enter();
    if (!((a.nodes & N_AGENT) && a.nl_off[a.n] > a.nl_cap)) {
        // the gather ran: redo the agents it left (their torque reached -0)
        if (BODY == 1) {
            const int nfix = *a.fix_count;
            for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nfix;
                 f += gridDim.x * blockDim.x) {
                const int s = a.fix_list[f];
                gather_agent<BODY, true>(a, s, a.perm[s]);
            }
        }
        return;
    }
    extern __shared__ unsigned char smem[];
    int *gq_all = reinterpret_cast<int *>(smem);
    WarpQueue *wq = reinterpret_cast<WarpQueue *>(smem + sizeof(int) * 2 * NTG);
    int *gq = gq_all + 2 * (threadIdx.x & ~(L - 1));
    const int lane = threadIdx.x & 31;
    for (;;) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(a.work, 1);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        const int s0 = chunk * (32 / L);
        if (s0 >= a.n) return;
        force_agent_group<BODY, L>(a, s0 + lane / L, gq, wq);
        __syncwarp();
    }
}

// Skin distance of a pair (same value whichever side is first).
__device__ __forceinline__ double pair_h(const StepArgs &a, int s, int t) {
    if (a.body == 0) {
        const Circ A = load_circ(a.stage, s), B = load_circ(a.stage, t);
        return cdm_hypot(A.x - B.x, A.y - B.y) - (A.r + B.r);
    }
    const TC A = load_tc(a.stage, s), B = load_tc(a.stage, t);
    double h_min = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double h = cdm_hypot(A.x[i] - B.x[j], A.y[i] - B.y[j]) -
                       ((i == 0 ? A.rt : A.rs) + (j == 0 ? B.rt : B.rs));
            if (h < h_min || isnan(h_min)) h_min = h;
        }
    return h_min;
}

// Which branches of the reference's social force the pair (s first, t
// second) takes (core/motion/power_law.py:213-259 Circular, :262-363
// ThreeCircle): `soc` the sub-pair loop runs (ThreeCircle: relative speed
// non-zero; Circular: always), `ndef` sub-pairs with a defined square root
// (Circular: defined and a != 0), `valid` a force is computed (tau > 0, and
// tau <= 30 for Circular).  Work accounting only: plain float64 arithmetic.
__device__ __forceinline__ void social_branches(const StepArgs &a, int s, int t, int &soc,
                                                int &ndef, int &valid) {
    soc = 0; ndef = 0; valid = 0;
    if (a.body == 0) {
        const Circ A = load_circ(a.stage, s), B = load_circ(a.stage, t);
        const double xr = A.x - B.x, yr = A.y - B.y, vx = A.vx - B.vx, vy = A.vy - B.vy;
        const double r = A.r + B.r;
        const double av = vx * vx + vy * vy, b = -(xr * vx + yr * vy);
        const double c = (xr * xr + yr * yr) - r * r;
        const double d = sqrt(b * b - av * c);
        soc = 1;
        if (isnan(d) || d == 0 || av == 0) return;
        ndef = 1;
        const double tau = (b - d) / av;
        valid = !(tau <= 0 || tau > 30.0);
        return;
    }
    const TC A = load_tc(a.stage, s), B = load_tc(a.stage, t);
    const double vx = A.vx - B.vx, vy = A.vy - B.vy;
    const double av = vx * vx + vy * vy;
    if (av == 0) return;
    soc = 1;
    double tau = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double xr = A.x[i] - B.x[j], yr = A.y[i] - B.y[j];
            const double r = (i == 0 ? A.rt : A.rs) + (j == 0 ? B.rt : B.rs);
            const double b = -(xr * vx + yr * vy), c = (xr * xr + yr * yr) - r * r;
            const double d = sqrt(b * b - av * c);
            if (isnan(d) || d == 0) continue;
            ++ndef;
            const double tn = (b - d) / av;
            if (isnan(tau) || (0 < tn && tn < tau)) tau = tn;
        }
    valid = !(isnan(tau) || tau <= 0);
}

// Per-agent interaction counts (diagnostics / algorithmic work accounting):
// candidates, pre-check survivors, h < 3, h < 0, walls past the pre-check,
// walls in contact; then, over the interacting pairs this agent comes first
// in (each unordered pair once), the social-force branches taken.
__global__ void k_pair_counts(StepArgs a, int *out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n) return;
    int i = a.perm[s];
    const ScenDev sc = a.scen[a.scen_of[i]];
    const float4 me = a.cull[s];
    int nc = 0, nn = 0, ni = 0, nt = 0, wn = 0, wc = 0, ns = 0, nd = 0, nv = 0;
    for_candidates(a, sc, s, a.key[i], me, [&](int t, bool s_first) {
        ++nn;
        double h = pair_h(a, s, t);
        ni += (h < SIGTH_SOC);
        nt += (h < 0);
        if (h < SIGTH_SOC && s_first) {
            int so, de, va;
            social_branches(a, s, t, so, de, va);
            ns += so; nd += de; nv += va;
        }
    }, &nc);
    if (sc.wall_count > 0) {
        const bool all_walls = me.z > (float)sc.wall_reach;
        int my_cell = a.key[i];
        int wb = all_walls ? sc.wall_begin : a.wall_start[my_cell];
        int we = all_walls ? sc.wall_begin + sc.wall_count : a.wall_start[my_cell + 1];
        for (int q = wb; q < we; ++q) {
            int w = all_walls ? q : a.wall_idx[q];
            if (wall_far(me.x, me.y, me.z, a.walls_f[w])) continue;
            ++wn;
            if (a.body == 0) {
                const Circ A = load_circ(a.stage, s);
                double nx, ny;
                wc += dist_circle_line(A.x, A.y, A.r, a.walls + (size_t)w * WALL_D, nx, ny) < 0;
            } else {
                const TC A = load_tc(a.stage, s);
                double h_min = __longlong_as_double(0x7ff8000000000000LL);
                for (int k = 0; k < 3; ++k) {
                    double nx, ny;
                    double h = dist_circle_line(A.x[k], A.y[k], k == 0 ? A.rt : A.rs,
                                                a.walls + (size_t)w * WALL_D, nx, ny);
                    if (h < h_min || isnan(h_min)) h_min = h;
                }
                wc += h_min < 0;
            }
        }
    }
    int *o = out + (size_t)i * COUNT_COLS;
    o[0] = nc; o[1] = nn; o[2] = ni; o[3] = nt; o[4] = wn; o[5] = wc;
    o[6] = ns; o[7] = nd; o[8] = nv;
}

// Float64 wall records (the tangent and length of distance_circle_line);
// the float32 pre-check records are written by the host (relative to their
// scenario's grid origin, cd_cull.cuh).
__global__ void k_wall_prep(const double *raw, double *walls, int nw) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    double p0x = raw[4 * w], p0y = raw[4 * w + 1], p1x = raw[4 * w + 2], p1y = raw[4 * w + 3];
    double dx = p1x - p0x, dy = p1y - p0y;
    double l_w = cdm_hypot(dx, dy);
    double *o = walls + (size_t)w * WALL_D;
    o[0] = p0x; o[1] = p0y; o[2] = p1x; o[3] = p1y;
    o[4] = dx / l_w; o[5] = dy / l_w; o[6] = l_w; o[7] = 0.0;
}

// -- packed host records <-> columns -------------------------------------
// Record fields are 4-byte aligned (packed numpy dtypes), so every float64 is
// moved as two 32-bit words.

struct FieldMap { int field, comp, col; };
// (CD_F_* field, vector component, column)
#define CD_MAP_CIRC                                                                      \
    {0, 0, X}, {0, 1, Y}, {1, 0, VX}, {1, 1, VY}, {2, 0, E0X}, {2, 1, E0Y},             \
    {3, 0, FX}, {3, 1, FY}, {4, 0, FPX}, {4, 1, FPY}, {5, 0, R}, {9, 0, MASS},          \
    {11, 0, V0}, {13, 0, TAU_ADJ}, {14, 0, K_SOC}, {15, 0, TAU0}, {16, 0, MU},          \
    {17, 0, KAPPA}, {18, 0, DAMP}, {19, 0, SRF}
#define CD_MAP_TC                                                                        \
    {0, 0, X}, {0, 1, Y}, {1, 0, VX}, {1, 1, VY}, {2, 0, E0X}, {2, 1, E0Y},             \
    {3, 0, FX}, {3, 1, FY}, {4, 0, FPX}, {4, 1, FPY}, {5, 0, R}, {9, 0, MASS},          \
    {11, 0, V0}, {13, 0, TAU_ADJ}, {14, 0, K_SOC}, {15, 0, TAU0}, {16, 0, MU},          \
    {17, 0, KAPPA}, {18, 0, DAMP}, {19, 0, SRF}, {28, 0, SRT},                          \
    {20, 0, XLS}, {20, 1, YLS}, {21, 0, XRS}, {21, 1, YRS}, {6, 0, RT}, {7, 0, RS},     \
    {8, 0, RTS}, {10, 0, INERTIA}, {12, 0, W0}, {22, 0, PHI}, {23, 0, OMEGA},           \
    {24, 0, PHI0}, {25, 0, TORQUE}, {26, 0, TORQUE_PREV}, {27, 0, TAU_ROT}
#define CD_OUT_CIRC X, Y, VX, VY, FX, FY, FPX, FPY, E0X, E0Y
#define CD_OUT_TC                                                                        \
    X, Y, VX, VY, FX, FY, FPX, FPY, XLS, YLS, XRS, YRS, PHI, OMEGA, PHI0, TORQUE,        \
    TORQUE_PREV, E0X, E0Y
__constant__ FieldMap kMapCirc[20] = {CD_MAP_CIRC};
__constant__ FieldMap kMapTC[36] = {CD_MAP_TC};
// Columns the step writes (downloaded back into the records).
__constant__ int kOutCirc[10] = {CD_OUT_CIRC};
__constant__ int kOutTC[19] = {CD_OUT_TC};
constexpr FieldMap hMapCirc[20] = {CD_MAP_CIRC};
constexpr FieldMap hMapTC[36] = {CD_MAP_TC};
constexpr int hOutCirc[10] = {CD_OUT_CIRC};
constexpr int hOutTC[19] = {CD_OUT_TC};

struct OffTable { long long off[32]; };
struct ColPtrs { double *p[NCOL]; };

__device__ __forceinline__ double ld_rec(const char *rec, long long off) {
    const unsigned *p = reinterpret_cast<const unsigned *>(rec + off);
    return __hiloint2double((int)p[1], (int)p[0]);
}
__device__ __forceinline__ void st_rec(char *rec, long long off, double v) {
    unsigned *p = reinterpret_cast<unsigned *>(rec + off);
    p[0] = (unsigned)__double2loint(v);
    p[1] = (unsigned)__double2hiint(v);
}

__global__ void k_aos_to_soa(const char *aos, long long itemsize, OffTable off, int n,
                             int body, ColPtrs cols) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const char *rec = aos + (size_t)i * itemsize;
    const FieldMap *map = body == 0 ? kMapCirc : kMapTC;
    int nm = body == 0 ? 20 : 36;
    for (int k = 0; k < nm; ++k) {
        long long o = off.off[map[k].field];
        if (o < 0) continue;
        cols.p[map[k].col][i] = ld_rec(rec, o + 8 * map[k].comp);
    }
}

__global__ void k_soa_to_aos(char *aos, long long itemsize, OffTable off, int n, int body,
                             ColPtrs cols) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    char *rec = aos + (size_t)i * itemsize;
    const FieldMap *map = body == 0 ? kMapCirc : kMapTC;
    const int *outs = body == 0 ? kOutCirc : kOutTC;
    int nm = body == 0 ? 20 : 36, no = body == 0 ? 10 : 19;
    for (int k = 0; k < nm; ++k) {
        bool written = false;
        for (int q = 0; q < no; ++q) written |= (outs[q] == map[k].col);
        long long o = off.off[map[k].field];
        if (!written || o < 0) continue;
        st_rec(rec, o + 8 * map[k].comp, cols.p[map[k].col][i]);
    }
}

// Integer and bool state fields of the packed records (target, active,
// is_leader, is_follower, index_leader, familiar_exit) sit at any byte offset
// (target at 2 in the reference dtypes, after two bools): read and written
// byte by byte, little-endian.
__device__ __forceinline__ long long ld_int(const char *rec, long long off, int bytes) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(rec + off);
    unsigned long long v = 0;
    for (int k = 0; k < bytes; ++k) v |= (unsigned long long)p[k] << (8 * k);
    return (long long)v;
}
__device__ __forceinline__ void st_int(char *rec, long long off, int bytes, long long v) {
    unsigned char *p = reinterpret_cast<unsigned char *>(rec + off);
    for (int k = 0; k < bytes; ++k) p[k] = (unsigned char)((unsigned long long)v >> (8 * k));
}
__device__ __forceinline__ int clamp_index(long long t) {
    return (t >= 0 && t <= 0x7fffffffLL) ? (int)t : -1;
}

// One record's state fields into the state columns (row i).
__device__ __forceinline__ void states_of_record(const char *rec, const StateOffsets &o,
                                                 const StateCols &c, int i) {
    c.target[i] = o.target >= 0 ? clamp_index(ld_int(rec, o.target, 8)) : -1;
    c.active[i] = o.active >= 0 ? (ld_int(rec, o.active, 1) != 0) : 1;
    c.leader[i] = o.leader >= 0 ? (ld_int(rec, o.leader, 1) != 0) : 0;
    c.follower[i] = o.follower >= 0 ? (ld_int(rec, o.follower, 1) != 0) : 0;
    c.index_leader[i] = o.index_leader >= 0 ? clamp_index(ld_int(rec, o.index_leader, 8)) : -1;
    c.familiar_exit[i] = o.familiar_exit >= 0 ? clamp_index(ld_int(rec, o.familiar_exit, 8)) : -1;
}

// Records moved straight between host memory the device can address (pinned,
// on this Grace-Blackwell part over the chip-to-chip link) and the columns:
// a block takes REC_BLOCK consecutive records, copies their 32-bit words with
// coalesced loads or stores into shared memory, and moves the float64 fields
// between shared memory and the columns there, so the copy and the transpose
// are one pass and no staging copy is made.
constexpr int XFER_NT = 256;
struct XferTable { int n; int word[40]; int col[40]; };   // field word offset, column

// A float64 as a key whose unsigned order is the numbers' order (-inf lowest,
// +inf highest, -0 below +0); 0 is no number, ~0 a NaN.
__device__ __forceinline__ unsigned long long order_key(double v) {
    if (isnan(v)) return ~0ull;
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(unsigned long long k, double none) {
    if (k == 0ull) return none;
    if (k == ~0ull) return __longlong_as_double(0x7ff8000000000000LL);
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

__device__ __forceinline__ unsigned long long shfl_max64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    return v;
}

__global__ void __launch_bounds__(XFER_NT)
k_records_in(const unsigned *__restrict__ src, unsigned *__restrict__ copy, int wpr, int per_block,
             int n, XferTable t, ColPtrs cols, StateOffsets so, StateCols sc, ScenMax mx) {
    extern __shared__ __align__(16) unsigned rec_sm[];
    const int i0 = blockIdx.x * per_block;
    const int nrec = min(per_block, n - i0);
    const size_t w0 = (size_t)i0 * wpr;
    const int words = nrec * wpr;
    // 16-byte words where the chunk starts on a 16-byte boundary (both
    // buffers), then the remaining 32-bit words
    int done = 0;
    if ((((uintptr_t)(src + w0) | (uintptr_t)(copy + w0)) & 15) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src + w0);
        uint4 *c4 = reinterpret_cast<uint4 *>(copy + w0);
        uint4 *m4 = reinterpret_cast<uint4 *>(rec_sm);
        const int q = words / 4;
        int w = threadIdx.x;
        for (; w + XFER_NT < q; w += 2 * XFER_NT) {
            const uint4 a = s4[w], b = s4[w + XFER_NT];
            m4[w] = a;
            m4[w + XFER_NT] = b;
            c4[w] = a;
            c4[w + XFER_NT] = b;
        }
        for (; w < q; w += XFER_NT) {
            const uint4 a = s4[w];
            m4[w] = a;
            c4[w] = a;
        }
        done = 4 * q;
    }
    for (int w = done + threadIdx.x; w < words; w += XFER_NT) {
        const unsigned v = src[w0 + w];
        rec_sm[w] = v;
        copy[w0 + w] = v;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < t.n * nrec; it += XFER_NT) {
        const int k = it / nrec, r = it - k * nrec;
        const unsigned *p = rec_sm + r * wpr + t.word[k];
        cols.p[t.col[k]][i0 + r] = __hiloint2double((int)p[1], (int)p[0]);
    }
    // the integer and bool state fields, from the same shared copy
    for (int r = threadIdx.x; r < nrec; r += XFER_NT)
        states_of_record(reinterpret_cast<const char *>(rec_sm + r * wpr), so, sc, i0 + r);
    if (!mx.key) return;
    // Per scenario: the largest target speed (a NaN wins) and the largest
    // finite extent, as order keys reduced per block (a max is exact in any
    // order), then one atomic per block and scenario; the last block to
    // finish writes them out as numbers and clears the keys for the next
    // upload.  The kernel waits on the host link: this work is hidden.
    __syncthreads();                                   // the block's columns are written
    __shared__ unsigned long long kv[XFER_NT / 32], ke[XFER_NT / 32];
    __shared__ int ks[XFER_NT / 32], last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long v = 0ull, e = 0ull;
    int sid = -1;
    if (threadIdx.x < nrec) {
        const int i = i0 + threadIdx.x;
        sid = mx.scen_of[i];
        v = order_key(cols.p[V0][i]);
        const double x = extent_of(cols.p, mx.body, i);
        e = isfinite(x) ? order_key(x) : 0ull;
    }
    const int s0 = __shfl_sync(0xffffffffu, sid, 0);
    if (__all_sync(0xffffffffu, sid == s0 || sid < 0)) {
        v = shfl_max64(v);
        e = shfl_max64(e);
        if (lane == 0) { kv[w] = v; ke[w] = e; ks[w] = s0; }
    } else {
        if (sid >= 0) {
            atomicMax(&mx.key[2 * sid], v);
            atomicMax(&mx.key[2 * sid + 1], e);
        }
        if (lane == 0) ks[w] = -1;
    }
    __threadfence();                                   // these atomics before the count below
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (nrec + 31) / 32;
        int cur = -1;
        unsigned long long cv = 0ull, ce = 0ull;
        for (int k = 0; k < nw; ++k) {                 // runs of warps of one scenario
            if (ks[k] != cur && cur >= 0) {
                atomicMax(&mx.key[2 * cur], cv);
                atomicMax(&mx.key[2 * cur + 1], ce);
                cv = 0ull; ce = 0ull;
            }
            cur = ks[k];
            if (cur >= 0) { cv = kv[k] > cv ? kv[k] : cv; ce = ke[k] > ce ? ke[k] : ce; }
        }
        if (cur >= 0) {
            atomicMax(&mx.key[2 * cur], cv);
            atomicMax(&mx.key[2 * cur + 1], ce);
        }
        __threadfence();
        last = atomicAdd(mx.blocks_done, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int k = threadIdx.x; k < mx.n_scen; k += XFER_NT) {
        const unsigned long long kvk = atomicExch(&mx.key[2 * k], 0ull);
        const unsigned long long kek = atomicExch(&mx.key[2 * k + 1], 0ull);
        mx.v0max[k] = key_value(kvk, -INFINITY);
        const double ek = key_value(kek, 0.0);
        mx.ext[k] = ek > 0.0 ? ek : 0.0;
        if (mx.ext_host) mx.ext_host[k] = ek > 0.0 ? ek : 0.0;
    }
    if (threadIdx.x == 0) *mx.blocks_done = 0;
}

__global__ void __launch_bounds__(XFER_NT)
k_records_out(unsigned *__restrict__ dst, const unsigned *__restrict__ base, int wpr,
              int per_block, int n, XferTable t, ColPtrs cols, StepStatus st) {
    extern __shared__ __align__(16) unsigned rec_sm[];
    // the status the host reads once the download is complete
    if (st.host && blockIdx.x == 0 && threadIdx.x == 0) {
        st.host[0] = *st.err;
        st.host[1] = st.need ? *st.need : 0;
    }
    const int i0 = blockIdx.x * per_block;
    const int nrec = min(per_block, n - i0);
    const size_t w0 = (size_t)i0 * wpr;
    const int words = nrec * wpr;
    int first = 0;
    if (((uintptr_t)(base + w0) & 15) == 0) {
        const uint4 *b4 = reinterpret_cast<const uint4 *>(base + w0);
        uint4 *m4 = reinterpret_cast<uint4 *>(rec_sm);
        const int q = words / 4;
        for (int w = threadIdx.x; w < q; w += XFER_NT) m4[w] = b4[w];
        first = 4 * q;
    }
    for (int w = first + threadIdx.x; w < words; w += XFER_NT) rec_sm[w] = base[w0 + w];
    __syncthreads();
    for (int it = threadIdx.x; it < t.n * nrec; it += XFER_NT) {
        const int k = it / nrec, r = it - k * nrec;
        unsigned *p = rec_sm + r * wpr + t.word[k];
        const double v = cols.p[t.col[k]][i0 + r];
        p[0] = (unsigned)__double2loint(v);
        p[1] = (unsigned)__double2hiint(v);
    }
    __syncthreads();
    int done = 0;
    if (((uintptr_t)(dst + w0) & 15) == 0) {
        uint4 *d4 = reinterpret_cast<uint4 *>(dst + w0);
        const uint4 *m4 = reinterpret_cast<const uint4 *>(rec_sm);
        const int q = words / 4;
        for (int w = threadIdx.x; w < q; w += XFER_NT) d4[w] = m4[w];
        done = 4 * q;
    }
    for (int w = done + threadIdx.x; w < words; w += XFER_NT) dst[w0 + w] = rec_sm[w];
}

__global__ void k_states_in(const char *aos, long long itemsize, StateOffsets o, int n,
                            StateCols c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    states_of_record(aos + (size_t)i * itemsize, o, c, i);
}

// The state fields the state nodes change: target, index_leader, active,
// is_follower.
__global__ void k_states_out(char *aos, long long itemsize, StateOffsets o, int n, StateCols c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    char *rec = aos + (size_t)i * itemsize;
    if (o.target >= 0) st_int(rec, o.target, 8, c.target[i]);
    if (o.index_leader >= 0) st_int(rec, o.index_leader, 8, c.index_leader[i]);
    if (o.active >= 0) st_int(rec, o.active, 1, c.active[i] ? 1 : 0);
    if (o.follower >= 0) st_int(rec, o.follower, 1, c.follower[i] ? 1 : 0);
}

__global__ void k_fp64_fma(double *out, int iters, double b, double c) {
    double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3,
           a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

inline int nblk(long long n, int nt) { return (int)((n + nt - 1) / nt); }

}  // namespace

void launch_prepare(const StepArgs &a, cudaStream_t s) {
    if (a.n > 0) k_prepare<<<nblk(a.n, PREP_NT), PREP_NT, 0, s>>>(a);
}
void launch_dt(const StepArgs &a, cudaStream_t s) {
    if (a.n_scen > 0) k_dt<<<nblk(a.n_scen, 128), 128, 0, s>>>(a);
}
int scan_launches_single(int n) { return nblk(n, SCAN_TILE) <= 4 ? 1 : 3; }
int scan_scratch_ints(int n) {
    int nb = nblk(n, SCAN_TILE);
    return nb > 1 ? 2 * (nb + 1) : 1;
}
int near_scan_ints(int n) { return 2 * (nblk(n, SCAN_TILE) + 1) + 1; }
void launch_scans(int k, const int *const *in, int *const *out, int n, int *const *scratch,
                  cudaStream_t s, bool dep) {
    const int nb = nblk(n, SCAN_TILE);
    ScanSet S{};
    for (int j = 0; j < k; ++j) {
        S.in[j] = in[j];
        S.out[j] = out[j];
        S.sums[j] = nb > 1 ? scratch[j] : nullptr;
    }
    if (nb <= 1) {
        launch_k(dep, k_scan_local, dim3(1, k), SCAN_NT, 0, s, S, n);
        return;
    }
    launch_k(dep, k_scan_local, dim3(nb, k), SCAN_NT, 0, s, S, n);
    ScanSet T{};                          // block totals, offsets after them (offs[nb] = total)
    for (int j = 0; j < k; ++j) {
        T.in[j] = scratch[j];
        T.out[j] = scratch[j] + nb + 1;
        T.sums[j] = nullptr;
    }
    launch_k(true, k_scan_local, dim3(1, k), SCAN_NT, 0, s, T, nb);
    ScanSet U{};
    for (int j = 0; j < k; ++j) {
        U.in[j] = scratch[j] + nb + 1;
        U.out[j] = out[j];
    }
    launch_k(true, k_scan_add, dim3(nblk(n + 1, 256), k), 256, 0, s, U, n, nb);
}
void launch_scan(const int *in, int *out, int n, int *scratch, cudaStream_t s, bool after_kernel) {
    if (n > SCAN_TILE && n <= 4 * SCAN_TILE) {
        launch_k(after_kernel, k_scan_single, 1, SCAN_NT, 0, s, in, out, n);
        return;
    }
    launch_scans(1, &in, &out, n, &scratch, s, after_kernel);
}
// Near, forward and guessed-social counts scanned together.
void launch_near_scans(const StepArgs &a, cudaStream_t s) {
    const int nb = nblk(a.n, SCAN_TILE);
    if (nb <= 0) return;
    const ScanSet S{{a.nl_cnt, a.fw_cnt, a.fs_cnt},
                    {a.nl_off, a.fw_off, a.fs_off},
                    {a.nl_scan, a.fw_scan, a.fs_scan}};
    launch_k(true, k_scan_tiles, dim3(nb, 3), SCAN_NT, 0, s, S, a.n, nb);   // after the count
}
void launch_scatter(const StepArgs &a, cudaStream_t s, bool after_kernel, int gather_part) {
    if (a.n <= 0) return;
    launch_k(after_kernel, k_scatter, nblk(a.n, 256), 256, 0, s, a);
    launch_k(true, k_rank, nblk(a.n, 128), 128, 0, s, a, gather_part);
}
void launch_gather(const StepArgs &a, cudaStream_t s, int part, bool after_kernel) {
    if (a.n > 0) launch_k(after_kernel, k_gather, nblk(a.n, 128), 128, 0, s, a, part);
}
// Force-kernel launch variants: the per-thread kernel (k_forces, lanes = 1)
// with NT threads per block and CAP candidates staged per thread per pass,
// the lane-group kernel (k_forces_group) with L lanes per agent, and the
// compute-once pair pipeline (near lists, k_pairs, gather) with L lanes per
// agent in the list build, its forces computed in k_pairs (pairs = 1) or in
// the separate force pass k_pair_forces (pairs = 2).
struct Variant { int nt, cap, lanes, pairs; };
constexpr Variant kVariants[N_VARIANTS] = {
    {128, 64, 1, 0}, {64, 64, 1, 0}, {128, 32, 1, 0}, {64, 32, 1, 0}, {256, 32, 1, 0},
    {NTG, 0, 4, 0},  {NTG, 0, 8, 0}, {NTG, 0, 16, 0}, {NTG, 0, 32, 0},
    {NTG, 0, 4, 1},  {NTG, 0, 8, 1}, {NTG, 0, 16, 1},
    {NTG, 0, 4, 2},  {NTG, 0, 8, 2}, {NTG, 0, 16, 2}};

size_t forces_smem_bytes(int body, int variant) {
    const Variant v = kVariants[variant];
    if (v.pairs) return 0;                                      // k_forces_gather
    size_t b = v.lanes == 1 ? sizeof(int) * (size_t)v.cap * v.nt : sizeof(int) * 2 * (size_t)NTG;
    if (body == 1) b += sizeof(WarpQueue) * (v.nt / 32);
    return b;
}

size_t pairs_smem_bytes(int body) { return body == 1 ? sizeof(PairQueue) * (NTG / 32) : 0; }

typedef void (*ForcesFn)(StepArgs);
constexpr ForcesFn kForces[2][N_VARIANTS] = {
    {k_forces<0, 128, 64>, k_forces<0, 64, 64>, k_forces<0, 128, 32>, k_forces<0, 64, 32>,
     k_forces<0, 256, 32>, k_forces_group<0, 4>, k_forces_group<0, 8>, k_forces_group<0, 16>,
     k_forces_group<0, 32>, k_forces_gather<0>, k_forces_gather<0>, k_forces_gather<0>,
     k_forces_gather<0>, k_forces_gather<0>, k_forces_gather<0>},
    {k_forces<1, 128, 64>, k_forces<1, 64, 64>, k_forces<1, 128, 32>, k_forces<1, 64, 32>,
     k_forces<1, 256, 32>, k_forces_group<1, 4>, k_forces_group<1, 8>, k_forces_group<1, 16>,
     k_forces_group<1, 32>, k_forces_gather<1>, k_forces_gather<1>, k_forces_gather<1>,
     k_forces_gather<1>, k_forces_gather<1>, k_forces_gather<1>}};

// Near-list and pair kernels of the pair-pipeline variants (by lanes 4, 8, 16).
constexpr int N_PAIR_L = 3;
constexpr ForcesFn kNlCount[N_PAIR_L] = {k_nl_count<4>, k_nl_count<8>, k_nl_count<16>};
constexpr ForcesFn kNlFill[N_PAIR_L] = {k_nl_fill<4>, k_nl_fill<8>, k_nl_fill<16>};
constexpr ForcesFn kPairs[2][2] = {{k_pairs<0, false>, k_pairs<0, true>},
                                    {k_pairs<1, false>, k_pairs<1, true>}};
constexpr ForcesFn kPairForces[2] = {k_pair_forces<0>, k_pair_forces<1>};
constexpr ForcesFn kPairsLight[2] = {k_pairs_light<0>, k_pairs_light<1>};
constexpr ForcesFn kFallback[2][N_PAIR_L] = {
    {k_forces_fallback<0, 4>, k_forces_fallback<0, 8>, k_forces_fallback<0, 16>},
    {k_forces_fallback<1, 4>, k_forces_fallback<1, 8>, k_forces_fallback<1, 16>}};
inline int pair_l_index(int lanes) { return lanes == 4 ? 0 : (lanes == 8 ? 1 : 2); }
// The lane-group variant with a pair-pipeline variant's lanes (4, 8, 16).
inline int group_twin(int variant) { return 5 + pair_l_index(kVariants[variant].lanes); }

bool variant_pairs(int variant) {
    return variant >= 0 && variant < N_VARIANTS && kVariants[variant].pairs != 0;
}

// Variant a new context starts with, from its agent count and body type
// (autotune.py refines it per workload).  Measured whole steps (ms) on GB300,
// lane groups of 16 / 32 against the pair pipeline with 16 / 8 list-build
// lanes and forces in k_pairs: Circular hallways of 400 agents 0.054 / 0.045
// against 0.065 / 0.067, 2000 agents 0.153 / 0.162 against 0.140 / 0.146,
// 5000 agents 0.276 / 0.312 against 0.176 / 0.182, 20000 agents 0.99 / 1.16
// against 0.294 / 0.295; the 2000-agent ThreeCircle room 0.237 / 0.247
// against 0.147 / 0.152.  Near the crossing it depends on the density: lane
// groups of 32 against the pipeline with 16 lanes, 1000 agents 0.062 against
// 0.079 (hallway, 1.3 per m^2) and 0.146 against 0.144 (room, 2.2 per m^2),
// 1300-1400 agents 0.075 against 0.079 and 0.201 against 0.147.  The force
// pass (variants 12-14 against 9-11, 4 / 8 / 16 list-build lanes): Circular
// 100k agents 0.347 / 0.340 / 0.369 against 0.351 / 0.344 / 0.373, 20k
// 0.302 / 0.270 / 0.270 against 0.330 / 0.298 / 0.298, 5000 0.180 / 0.163 /
// 0.157 against 0.201 / 0.181 / 0.176; ThreeCircle 100k field 0.337 / 0.340 /
// 0.366 against 0.333 / 0.335 / 0.362, 2000-agent room 0.164 / 0.150 / 0.145
// against 0.165 / 0.151 / 0.147, 4000 agents in contact 0.185 / 0.171 /
// 0.166 against 0.172 / 0.157 / 0.153.
int default_variant(long long n, int body) {
    if (n < 1200) return 8;                  // lane groups, 32 lanes per agent
    if (body == 0) return n < 16000 ? 14 : 13;   // Circular: the separate force pass
    return n < 16000 ? 11 : 9;               // ThreeCircle: forces in k_pairs
}

// The same without the pair pipeline (contexts without near-list memory).
int default_group_variant(long long n, int body) {
    const int v = default_variant(n, body);
    return kVariants[v].pairs ? group_twin(v) : v;
}

bool variant_split(int variant) {
    return variant >= 0 && variant < N_VARIANTS && kVariants[variant].pairs == 2;
}

int variant_lanes(int variant) {
    return variant >= 0 && variant < N_VARIANTS ? kVariants[variant].lanes : 0;
}
int variant_threads(int variant) {
    return variant >= 0 && variant < N_VARIANTS ? kVariants[variant].nt : 0;
}
int variant_staged(int variant) {
    return variant >= 0 && variant < N_VARIANTS ? kVariants[variant].cap : 0;
}

// Resident blocks of each force kernel variant (and pair kernel) on each device.
int g_forces_blocks[64][2][N_VARIANTS];
int g_pairs_blocks[64][2][2];             // [device][body][split]
int g_light_blocks[64][2];
int g_job_blocks[64][2];

int init_kernels() {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int body = 0; body < 2 && e == cudaSuccess; ++body)
        for (int v = 0; v < N_VARIANTS && e == cudaSuccess; ++v) {
            e = cudaFuncSetAttribute(kForces[body][v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)forces_smem_bytes(body, v));
            int nb = 0;
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &nb, kForces[body][v], kVariants[v].pairs ? GATHER_NT : kVariants[v].nt,
                    forces_smem_bytes(body, v));
            if (e == cudaSuccess && dev >= 0 && dev < 64)
                g_forces_blocks[dev][body][v] = (nb > 0 ? nb : 1) * sms;
        }
    for (int body = 0; body < 2 && e == cudaSuccess; ++body)
        for (int l = 0; l < N_PAIR_L && e == cudaSuccess; ++l)
            // the fallback kernel shares the lane-group variant's shared memory
            e = cudaFuncSetAttribute(kFallback[body][l],
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)forces_smem_bytes(body, 5 + l));
    for (int body = 0; body < 2 && e == cudaSuccess; ++body)
        for (int sp = 0; sp < 2 && e == cudaSuccess; ++sp) {
            e = cudaFuncSetAttribute(kPairs[body][sp],
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)pairs_smem_bytes(body));
            int nb = 0;
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kPairs[body][sp], NTG,
                                                                  pairs_smem_bytes(body));
            if (e == cudaSuccess && dev >= 0 && dev < 64)
                g_pairs_blocks[dev][body][sp] = (nb > 0 ? nb : 1) * sms;
        }
    for (int body = 0; body < 2 && e == cudaSuccess; ++body) {
        int nb = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kPairsLight[body], NTG, 0);
        if (e == cudaSuccess && dev >= 0 && dev < 64)
            g_light_blocks[dev][body] = (nb > 0 ? nb : 1) * sms;
        nb = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kPairForces[body], NTG, 0);
        if (e == cudaSuccess && dev >= 0 && dev < 64)
            g_job_blocks[dev][body] = (nb > 0 ? nb : 1) * sms;
    }
    return e == cudaSuccess ? 0 : (int)e;
}

void launch_prologue(const StepArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    if (a.body) k_prologue<1><<<nblk(a.n, 128), 128, 0, s>>>(a);
    else k_prologue<0><<<nblk(a.n, 128), 128, 0, s>>>(a);
}

void launch_forces(const StepArgs &a, cudaStream_t s, int variant, const cudaEvent_t *pair_ev,
                   bool captured, const Fork *fork, bool stage_deferred) {
    if (a.n <= 0) return;
    if (variant < 0 || variant >= N_VARIANTS) variant = 0;
    // the pair pipeline needs the near-list buffers: otherwise its lane-group twin
    if (kVariants[variant].pairs && !a.nl_cnt) variant = group_twin(variant);
    const Variant v = kVariants[variant];
    int dev = 0;
    cudaGetDevice(&dev);
    const int body = a.body ? 1 : 0;
    // the gather takes the prologue from k_prologue, on the second stream
    // beside the near lists when there is one
    // and, when the cell list left them, the float64 staged records first
    const bool pro = v.pairs && a.pro;
    if (pro) {
        cudaStream_t sp = s;
        if (fork) {
            cudaEventRecord(fork->fork, s);
            cudaStreamWaitEvent(fork->s2, fork->fork, 0);
            sp = fork->s2;
        }
        if (stage_deferred) {
            launch_gather(a, sp, 2);
            if (fork) cudaEventRecord(fork->join_stage, fork->s2);
        }
        launch_prologue(a, sp);
        if (fork) cudaEventRecord(fork->join, fork->s2);
    } else if (stage_deferred) {
        launch_gather(a, s, 2);
    }
    if (v.pairs && (a.nodes & N_AGENT)) {
        const int l = pair_l_index(v.lanes);
        const int nb = nblk((long long)a.n * v.lanes, NTG);
        kNlCount[l]<<<nb, NTG, 0, s>>>(a);
        launch_near_scans(a, s);
        launch_k(true, kNlFill[l], nb, NTG, 0, s, a);
        const int sp = v.pairs == 2 ? 1 : 0;
        int rp = (dev >= 0 && dev < 64) ? g_pairs_blocks[dev][body][sp] : 0;
        if (rp <= 0) rp = 152;
        // at most one warp per 32 pairs (about 16 pairs per agent): enough blocks
        if (pro && stage_deferred && fork) cudaStreamWaitEvent(s, fork->join_stage, 0);
        if (pair_ev) cudaEventRecordWithFlags(pair_ev[0], s, captured ? cudaEventRecordExternal : 0);
        if (a.defer_list) {
            int rl = (dev >= 0 && dev < 64) ? g_light_blocks[dev][body] : 0;
            if (rl <= 0) rl = 152;
            kPairsLight[body]<<<std::min(nblk((long long)a.n * 16, NTG), rl), NTG, 0, s>>>(a);
            if (pair_ev)            // the float32 pass's end (timing only)
                cudaEventRecordWithFlags(pair_ev[1], s, captured ? cudaEventRecordExternal : 0);
        }
        // after k_pairs_light: chained to it (unless an event sits between)
        launch_k(a.defer_list != nullptr && !pair_ev, kPairs[body][sp],
                 std::min(nblk((long long)a.n * 16, NTG), rp), NTG, pairs_smem_bytes(body), s, a);
        if (sp) {
            // the force pass over the jobs (their count is known on the device only)
            int rj = (dev >= 0 && dev < 64) ? g_job_blocks[dev][body] : 0;
            if (rj <= 0) rj = 152;
            launch_k(true, kPairForces[body], std::min(nblk((long long)a.n * 16, NTG), rj), NTG,
                     0, s, a);
        }
        if (pair_ev) cudaEventRecordWithFlags(pair_ev[2], s, captured ? cudaEventRecordExternal : 0);
    }
    int resident = (dev >= 0 && dev < 64) ? g_forces_blocks[dev][body][variant] : 0;
    if (resident <= 0) resident = 152;
    const long long threads = (long long)a.n * v.lanes;
    int blocks = (int)std::min<long long>((threads + v.nt - 1) / v.nt, resident);
    int nt = v.nt;
    if (v.pairs) {                                       // gather: one lane per slot, full grid
        nt = GATHER_NT;
        blocks = nblk(a.n, nt);
    }
    if (!v.pairs) cudaMemsetAsync(a.work, 0, sizeof(int), s);     // the gather zeroes it itself
    if (pro && fork) cudaStreamWaitEvent(s, fork->join, 0);
    kForces[body][variant]<<<blocks, nt, forces_smem_bytes(body, variant), s>>>(a);
    if (v.pairs && (a.nodes & N_AGENT)) {
        const int gv = group_twin(variant);
        int rg = (dev >= 0 && dev < 64) ? g_forces_blocks[dev][body][gv] : 0;
        if (rg <= 0) rg = 152;
        launch_k(true, kFallback[body][pair_l_index(v.lanes)],
                 (int)std::min<long long>((threads + NTG - 1) / NTG, rg), NTG,
                 forces_smem_bytes(body, gv), s, a);          // after the gather
    }
}

void launch_near_count(const StepArgs &a, cudaStream_t s, int variant) {
    if (a.n <= 0 || !variant_pairs(variant)) return;
    const int lanes = kVariants[variant].lanes;
    kNlCount[pair_l_index(lanes)]<<<nblk((long long)a.n * lanes, NTG), NTG, 0, s>>>(a);
    launch_near_scans(a, s);
}

void launch_near_lists(const StepArgs &a, cudaStream_t s) {
    if (a.n <= 0 || !a.nl_cnt) return;
    const int nb = nblk((long long)a.n * 8, NTG);
    kNlCount[1]<<<nb, NTG, 0, s>>>(a);
    launch_near_scans(a, s);
    launch_k(true, kNlFill[1], nb, NTG, 0, s, a);
}
void launch_adj_light(const StepArgs &a, cudaStream_t s) {
    if (a.n <= 0 || !a.nl_cnt || a.body != 0) return;
    launch_k(true, k_pairs_light<0, true>, nblk((long long)a.n * 16, NTG), NTG, 0, s, a);
}

void launch_pair_counts(const StepArgs &a, int *counts, cudaStream_t s) {
    if (a.n > 0) k_pair_counts<<<nblk(a.n, 128), 128, 0, s>>>(a, counts);
}
void launch_scen_max(const StepArgs &a, double *v0max, double *ext, double *partial,
                     cudaStream_t s) {
    if (a.n_scen <= 0) return;
    const long long mean = ((long long)a.n + a.n_scen - 1) / a.n_scen;
    const int nb = (int)std::min<long long>(V0MAX_B, std::max<long long>(1, (mean + 511) / 512));
    k_scen_max_partial<<<dim3(nb, a.n_scen), 256, 0, s>>>(a, partial);
    k_scen_max_final<<<(a.n_scen + 7) / 8, 256, 0, s>>>(partial, nb, a.n_scen, v0max, ext);
}
int scen_max_partials(int n_scen) { return 2 * V0MAX_B * (n_scen > 0 ? n_scen : 1); }
void launch_wall_prep(const double *raw, double *walls, int nw, cudaStream_t s) {
    if (nw > 0) k_wall_prep<<<nblk(nw, 128), 128, 0, s>>>(raw, walls, nw);
}
void launch_aos_to_soa(const char *aos, long long itemsize, const long long *off, int n,
                       int body, double *const *col, cudaStream_t s) {
    if (n <= 0) return;
    OffTable t;
    for (int k = 0; k < 32; ++k) t.off[k] = k < 29 ? off[k] : -1;
    ColPtrs c;
    for (int k = 0; k < NCOL; ++k) c.p[k] = col[k];
    k_aos_to_soa<<<nblk(n, 128), 128, 0, s>>>(aos, itemsize, t, n, body, c);
}
void launch_states_in(const char *aos, long long itemsize, const StateOffsets &o, int n,
                      const StateCols &c, cudaStream_t s) {
    if (n > 0) k_states_in<<<nblk(n, 256), 256, 0, s>>>(aos, itemsize, o, n, c);
}
void launch_states_out(char *aos, long long itemsize, const StateOffsets &o, int n,
                       const StateCols &c, cudaStream_t s) {
    if (n > 0) k_states_out<<<nblk(n, 256), 256, 0, s>>>(aos, itemsize, o, n, c);
}
void launch_soa_to_aos(char *aos, long long itemsize, const long long *off, int n, int body,
                       const double *const *col, cudaStream_t s) {
    if (n <= 0) return;
    OffTable t;
    for (int k = 0; k < 32; ++k) t.off[k] = k < 29 ? off[k] : -1;
    ColPtrs c;
    for (int k = 0; k < NCOL; ++k) c.p[k] = const_cast<double *>(col[k]);
    k_soa_to_aos<<<nblk(n, 128), 128, 0, s>>>(aos, itemsize, t, n, body, c);
}

int records_per_block(long long itemsize) {
    const long long r = (48 * 1024) / itemsize;
    return (int)std::min<long long>(64, r);
}

static XferTable xfer_table(const long long *off, int body, bool outputs_only) {
    XferTable t{};
    const FieldMap *map = body == 0 ? hMapCirc : hMapTC;
    const int nm = body == 0 ? 20 : 36;
    const int *outs = body == 0 ? hOutCirc : hOutTC;
    const int no = body == 0 ? 10 : 19;
    for (int k = 0; k < nm; ++k) {
        const long long o = off[map[k].field];
        if (o < 0) continue;
        bool written = false;
        for (int q = 0; q < no; ++q) written |= outs[q] == map[k].col;
        if (outputs_only && !written) continue;
        t.word[t.n] = (int)((o + 8 * map[k].comp) / 4);
        t.col[t.n] = map[k].col;
        ++t.n;
    }
    return t;
}

void launch_records_in(const void *src, char *aos, long long itemsize, const long long *off,
                       int n, int body, double *const *col, const StateOffsets &so,
                       const StateCols &sc, cudaStream_t s, const ScenMax &mx) {
    const int per = records_per_block(itemsize);
    if (n <= 0 || per <= 0) return;
    ColPtrs c;
    for (int k = 0; k < NCOL; ++k) c.p[k] = col[k];
    k_records_in<<<nblk(n, per), XFER_NT, (size_t)per * itemsize, s>>>(
        static_cast<const unsigned *>(src), reinterpret_cast<unsigned *>(aos), (int)(itemsize / 4),
        per, n, xfer_table(off, body, false), c, so, sc, mx);
}

void launch_records_out(void *dst, const char *aos, long long itemsize, const long long *off,
                        int n, int body, const double *const *col, cudaStream_t s,
                        const StepStatus &st) {
    const int per = records_per_block(itemsize);
    if (n <= 0 || per <= 0) return;
    ColPtrs c;
    for (int k = 0; k < NCOL; ++k) c.p[k] = const_cast<double *>(col[k]);
    k_records_out<<<nblk(n, per), XFER_NT, (size_t)per * itemsize, s>>>(
        static_cast<unsigned *>(dst), reinterpret_cast<const unsigned *>(aos), (int)(itemsize / 4),
        per, n, xfer_table(off, body, true), c, st);
}

double fp64_peak_gflops() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_fp64_fma<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return -1;
    double flops = 2.0 * 8 * iters * (double)blocks * threads;
    return flops / (best * 1e-3) / 1e9;
}

}  // namespace cdk
