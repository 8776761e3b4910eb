// cd_adjoint.cu -- hand-written adjoint (reverse mode) of one Circular step.
//
// Forward step (core/integrator.py:164-176 with the force nodes of
// simulation/logic.py:89-130), per agent i with state (x, v, fp):
//   F   = F_adj(v; m, tau_adj, v0, e0) + sum_j F_pair(x_i - x_j, v_i - v_j)
//         + sum_w F_wall(x_i, v_i)
//   dt  = clamp(1.1 * max(v0) * dt_max / max|v|, dt_min, dt_max)
//   v'  = v + (fp / m + F / m) / 2 * dt
//   x'  = x + v' dt + F / (2 m) dt^2
//   fp' = F
// Reverse, with incoming adjoints (lx', lv', lfp') of (x', v', fp'):
//   lvt = lv' + lx' dt                       (v' also reaches x')
//   lF  = lfp' + lvt dt / (2 m) + lx' dt^2 / (2 m)
//   lfp = lvt dt / (2 m)
//   lx  = lx' + (dF/dx)^T lF,   lv = lvt + (dF/dv)^T lF
//   ldt = sum_i lx'_i . (v'_i + F_i dt / m_i) + lvt_i . (fp_i + F_i) / (2 m_i)
// and ldt reaches max(v0) and max|v| when dt is not clamped.  The pair
// terms need both sides: agent i's force depends on x_i - x_j, and agent j's
// force on x_j - x_i, so agent i gathers (dF_i/dx_rel)^T lF_i from its own
// side and -(dF_j/dx_rel)^T lF_j from each neighbour's side; every agent sums
// in its fixed neighbour order, so the result is deterministic.
//
// Branches are differentiated where they are taken (a sub-gradient at the
// contact onset h = 0, the social cut-offs h = 3 and tau = 30, the 2000 N
// truncation and the dt clamp).
#include <algorithm>
#include <cstdint>
#include <cmath>
#include "cd_internal.cuh"
#include "cd_cull.cuh"
#include "cd_math.h"

namespace cdk {
namespace {

constexpr double SIGTH_SOC = 3.0;
constexpr double F_SOC_MAX = 2e3;
constexpr double TAU_MAX = 30.0;
constexpr int NT = 128;
constexpr int RED_NT = 256;

struct Circ {
    double x, y, vx, vy, r, m, k, tau0, mu, kappa, damp;
};

// Last-block-done: every block has written its partial (made visible by the
// fence) before it counts itself; the block that counts last returns true
// and resets the counter for the next kernel.
__device__ __forceinline__ bool last_block(int *blocks_done) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(blocks_done, 1) == (int)gridDim.x - 1;
        if (last) *blocks_done = 0;
    }
    __syncthreads();
    return last;
}

// Sum of nb partials by warp 0 in a fixed order (lane-strided sums, then a
// butterfly): deterministic for a given nb; every lane of warp 0 holds it.
__device__ __forceinline__ double ordered_sum(const double *partial, int nb) {
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += 32) s += __ldcg(partial + k);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

__device__ __forceinline__ Circ load_circ(const double2 *__restrict__ st, int slot) {
    const double2 *p = st + (size_t)slot * STAGE_Q_CIRC;
    double2 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3),
            q4 = __ldg(p + 4), q5 = __ldg(p + 5);
    Circ a;
    a.x = q0.x; a.y = q0.y; a.vx = q1.x; a.vy = q1.y; a.r = q2.x; a.m = q2.y;
    a.k = q3.x; a.tau0 = q3.y; a.mu = q4.x; a.kappa = q4.y; a.damp = q5.x;
    return a;
}

// Reverse of a sum of contact forces sharing one geometry,
//   Phi = sum_s sigma_s u_s . [-h (mu_s n - kappa_s (v.t) t) + c_s (v.n) n],
// given the combined seeds U_mu = sum sigma mu u, U_ka = sum sigma kappa u,
// U_d = sum sigma c u (h = |x| - r, n = x / |x|, t = rotate270(n) = R n);
// adds dPhi/dx and dPhi/dv.
__device__ __forceinline__ void contact_vjp3(double xx, double xy, double d0, double h,
                                             double vx, double vy, double umx, double umy,
                                             double ukx, double uky, double udx, double udy,
                                             double &gxx, double &gxy, double &gvx,
                                             double &gvy) {
    const double id0 = 1.0 / d0;
    const double nx = xx * id0, ny = xy * id0;
    const double tx = ny, ty = -nx;
    const double vt = vx * tx + vy * ty, vn = vx * nx + vy * ny;
    const double umn = umx * nx + umy * ny;
    const double ukt = ukx * tx + uky * ty;
    const double udn = udx * nx + udy * ny;
    gvx += h * ukt * tx + udn * nx;
    gvy += h * ukt * ty + udn * ny;
    const double A = -umn + vt * ukt;                        // coefficient of dh = n . dx
    const double w1x = -h * umx + udn * vx + vn * udx;       // through dn = P dx / |x|
    const double w1y = -h * umy + udn * vy + vn * udy;
    const double w2x = h * (ukt * vx + vt * ukx);            // through dt = R P dx / |x|
    const double w2y = h * (ukt * vy + vt * uky);
    const double qx = w1x - w2y, qy = w1y + w2x;             // w1 + R^T w2
    const double pq = nx * qx + ny * qy;                     // P q = q - n (n . q)
    gxx += A * nx + (qx - nx * pq) * id0;
    gxy += A * ny + (qy - ny * pq) * id0;
}

// Single contact force with seed u.
__device__ __forceinline__ void contact_vjp(double xx, double xy, double d0, double h, double vx,
                                            double vy, double mu, double kappa, double damp,
                                            double ux, double uy, double &gxx, double &gxy,
                                            double &gvx, double &gvy) {
    contact_vjp3(xx, xy, d0, h, vx, vy, mu * ux, mu * uy, kappa * ux, kappa * uy, damp * ux,
                 damp * uy, gxx, gxy, gvx, gvy);
}

// Seed of the untruncated force from the seed u of truncate(F, 2000 N)
// (vector2D.py:166-187): u itself, or (s)(I - f f^T) u above the limit.
__device__ __forceinline__ void truncate_vjp(double Fx, double Fy, double &ux, double &uy) {
    // certainly below the limit (as truncate2 decides it): the identity
    if (Fx * Fx + Fy * Fy < 0.99 * (F_SOC_MAX * F_SOC_MAX)) return;
    const double L = cdm_hypot(Fx, Fy);
    if (L > F_SOC_MAX) {
        const double iL = 1.0 / L;
        const double fx = Fx * iL, fy = Fy * iL, s = F_SOC_MAX * iL;
        const double dot = ux * fx + uy * fy;
        ux = s * (ux - dot * fx);
        uy = s * (uy - dot * fy);
    }
}

struct PairGrad {
    double gxx, gxy, gvx, gvy;                 // d/d(x_i - x_j), d/d(v_i - v_j)
    double gk, gt0;                            // d/dk_soc_i, d/dtau_0_i
};

// Social side s of a pair (power_law.py:215-259): F_s = trunc(c_s mg(tau, tau0_s)
// sigma g), c_s = -m_s k_s, sigma = +1 for agent i and -1 for agent j (tau's
// gradient in j's frame is -g).  Adds the side's seed of g to (lgx, lgy) and
// of tau to ltau; returns (l_raw . g) sigma for the k_soc / tau_0 terms.
__device__ __forceinline__ void social_side(double tau, double it, double it2, double gx,
                                            double gy, double sigma, double m, double k,
                                            double tau0, double ux, double uy, double &lgx,
                                            double &lgy, double &ltau, double *gk,
                                            double *gt0) {
    const double i0 = 1.0 / tau0;
    const double e = cdm_exp(-tau * i0);
    const double mg = (2.0 * it + i0) * e * it2;
    const double cm = (-m) * k;
    const double cms = cm * mg * sigma;
    double lx = ux, ly = uy;
    truncate_vjp(cms * gx, cms * gy, lx, ly);
    lgx += cms * lx;
    lgy += cms * ly;
    const double lgd = sigma * (lx * gx + ly * gy);
    const double lmg = cm * lgd;
    ltau -= lmg * e * it2 * (6.0 * it2 + 4.0 * it * i0 + i0 * i0);
    if (gk) {
        *gk += (-m) * mg * lgd;
        *gt0 += lmg * e * i0 * i0 * (it2 + it * i0);
    }
}

// Reverse of one pair's two forces (interactions.py:51-70): the seed is
//   Phi = u_i . F_i(x, v) + u_j . F_j(-x, -v)
// with x = x_i - x_j, v = v_i - v_j; both forces share h, tau and tau's
// gradient g, so one pass back through the geometry serves both sides.
// Adds dPhi/dx, dPhi/dv and agent i's k_soc, tau_0 terms.
__device__ __forceinline__ void pair_vjp_both(const Circ &A, const Circ &B, double uix,
                                              double uiy, double ujx, double ujy, PairGrad &G,
                                              double *gk_j = nullptr, double *gt0_j = nullptr) {
    const double xx = A.x - B.x, xy = A.y - B.y;
    const double d0 = cdm_hypot(xx, xy);
    const double r_tot = A.r + B.r;
    const double h = d0 - r_tot;
    if (!(h < SIGTH_SOC)) return;
    const double vx = A.vx - B.vx, vy = A.vy - B.vy;
    const double a = vx * vx + vy * vy;
    const double b = -(xx * vx + xy * vy);
    const double c = (xx * xx + xy * xy) - r_tot * r_tot;
    const double disc = b * b - a * c;
    if (disc > 0 && a != 0) {
        const double dd = sqrt(disc);
        const double tau = (b - dd) / a;
        if (!(tau <= 0 || tau > TAU_MAX)) {
            const double ia = 1.0 / a, idd = 1.0 / dd;
            const double gx = (vx - (vx * b + xx * a) * idd) * ia;   // grad of tau
            const double gy = (vy - (vy * b + xy * a) * idd) * ia;
            const double it = 1.0 / tau, it2 = it * it;
            double lgx = 0.0, lgy = 0.0, ltau = 0.0;
            social_side(tau, it, it2, gx, gy, 1.0, A.m, A.k, A.tau0, uix, uiy, lgx, lgy, ltau,
                        &G.gk, &G.gt0);
            social_side(tau, it, it2, gx, gy, -1.0, B.m, B.k, B.tau0, ujx, ujy, lgx, lgy, ltau,
                        gk_j, gt0_j);
            // g = v / a - b v / (a dd) - x / dd,  tau = (b - dd) / a
            double la = -(lgx * (gx + xx * idd) + lgy * (gy + xy * idd)) * ia;
            double lb = -(lgx * vx + lgy * vy) * ia * idd;
            double ldd = (lgx * (b * vx * ia + xx) + lgy * (b * vy * ia + xy)) * idd * idd;
            const double cv = ia - b * ia * idd;
            G.gvx += cv * lgx;
            G.gvy += cv * lgy;
            G.gxx -= lgx * idd;
            G.gxy -= lgy * idd;
            lb += ltau * ia;
            ldd -= ltau * ia;
            la -= ltau * tau * ia;
            const double ldisc = 0.5 * ldd * idd;                  // dd = sqrt(b^2 - a c)
            lb += 2.0 * b * ldisc;
            la -= c * ldisc;
            const double lc = -a * ldisc;
            G.gxx += 2.0 * lc * xx - lb * vx;                      // c = x.x - r^2, b = -x.v
            G.gxy += 2.0 * lc * xy - lb * vy;
            G.gvx += 2.0 * la * vx - lb * xx;                      // a = v.v
            G.gvy += 2.0 * la * vy - lb * xy;
        }
    }
    if (h < 0 && d0 != 0.0) {
        // F_i = C(p_i), F_j(-x, -v) = -C(p_j) in i's frame (interactions.py:63-66)
        contact_vjp3(xx, xy, d0, h, vx, vy, A.mu * uix - B.mu * ujx, A.mu * uiy - B.mu * ujy,
                     A.kappa * uix - B.kappa * ujx, A.kappa * uiy - B.kappa * ujy,
                     A.damp * uix - B.damp * ujx, A.damp * uiy - B.damp * ujy, G.gxx, G.gxy,
                     G.gvx, G.gvy);
    }
}

// Reverse of the Circular agent-wall contact (interactions.py:107-120,
// distance.py:108-146), seed u; adds to d/dx, d/dv.
__device__ void wall_circ_vjp(const Circ &A, const double *w, double ux, double uy, double &gxx,
                              double &gxy, double &gvx, double &gvy) {
    double p0x = w[0], p0y = w[1], p1x = w[2], p1y = w[3];
    double tx = w[4], ty = w[5], l_w = w[6];
    double nwx = -ty, nwy = tx;
    double q0x = A.x - p0x, q0y = A.y - p0y, q1x = A.x - p1x, q1y = A.y - p1y;
    double l_t = -(tx * q1x + ty * q1y) - (tx * q0x + ty * q0y);
    if (l_t > l_w || l_t < -l_w) {
        double qx = l_t > l_w ? q0x : q1x, qy = l_t > l_w ? q0y : q1y;
        double d = cdm_hypot(qx, qy);
        double h = d - A.r;
        if (h < 0 && d != 0.0)
            contact_vjp(qx, qy, d, h, A.vx, A.vy, A.mu, A.kappa, A.damp, ux, uy, gxx, gxy, gvx, gvy);
        return;
    }
    double l_n = nwx * q0x + nwy * q0y;
    double h = fabs(l_n) - A.r;
    if (!(h < 0)) return;
    double s = l_n > 0 ? 1.0 : (l_n < 0 ? -1.0 : 0.0);
    double nx = s * nwx, ny = s * nwy;                       // constant normal
    double ttx = ny, tty = -nx;
    double vt = A.vx * ttx + A.vy * tty;
    double ut = ux * ttx + uy * tty, un = ux * nx + uy * ny;
    gvx += h * A.kappa * ut * ttx + A.damp * un * nx;
    gvy += h * A.kappa * ut * tty + A.damp * un * ny;
    double Acoef = -A.mu * un + A.kappa * vt * ut;
    gxx += Acoef * nx;
    gxy += Acoef * ny;
}

__global__ void k_adj_seed(AdjArgs q) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && q.work_zero) {           // the reverse pair kernels' counters
        q.work_zero[0] = 0;
        q.work_zero[1] = 0;
        q.work_zero[2] = 0;
        q.work_zero[3] = 0;
    }
    double s = 0.0;
    if (i < q.n) {
        const double dt = *q.dt;
        const double m = q.mass[i];
        double lxx = q.lx[2 * i], lxy = q.lx[2 * i + 1];
        if (q.gtarget) {                   // the step's loss term: lx += scale 2 (x' - target)
            lxx += q.gscale * 2.0 * (q.gx[i] - q.gtarget[2 * i]);
            lxy += q.gscale * 2.0 * (q.gy[i] - q.gtarget[2 * i + 1]);
            q.lx_rw[2 * i] = lxx;
            q.lx_rw[2 * i + 1] = lxy;
        }
        double lvtx = q.lv[2 * i] + lxx * dt, lvty = q.lv[2 * i + 1] + lxy * dt;
        double c1 = dt / (2.0 * m), c2 = dt * dt / (2.0 * m);
        double Fx = q.fx[i], Fy = q.fy[i];
        q.lF[2 * i] = q.lfp[2 * i] + lvtx * c1 + lxx * c2;
        q.lF[2 * i + 1] = q.lfp[2 * i + 1] + lvty * c1 + lxy * c2;
        q.lvt[2 * i] = lvtx;
        q.lvt[2 * i + 1] = lvty;
        q.lfp_out[2 * i] = lvtx * c1;
        q.lfp_out[2 * i + 1] = lvty * c1;
        double vnx = q.vnx[i], vny = q.vny[i];
        double fpx = q.fpx[i], fpy = q.fpy[i];
        s = lxx * (vnx + Fx * dt / m) + lxy * (vny + Fy * dt / m) +
            lvtx * (fpx + Fx) / (2.0 * m) + lvty * (fpy + Fy) / (2.0 * m);
    }
    // block partial of ldt, fixed tree order
    __shared__ double red[RED_NT];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = RED_NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) q.partial[blockIdx.x] = red[0];
    // the last block: the dt adjoint, the partials summed in a fixed order
    if (last_block(q.blocks_done) && threadIdx.x < 32) {
        const double t = ordered_sum(q.partial, gridDim.x);
        if (threadIdx.x == 0) *q.ldt = t;
    }
}

// loss += scale * sum_i |x_i - target_i|^2: per block partials, summed by
// the last block in a fixed order; block 0 also copies the step's dt.
__global__ void k_loss(const double *x, const double *y, const double *target, int n,
                       double *partial, double *loss, double scale, int *blocks_done,
                       const double *dt_src, double *dt_dst) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && dt_dst) *dt_dst = *dt_src;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < n) {
        double dx = x[i] - target[2 * i], dy = y[i] - target[2 * i + 1];
        s = dx * dx + dy * dy;
    }
    __shared__ double red[RED_NT];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = RED_NT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
    if (last_block(blocks_done) && threadIdx.x < 32) {
        const double t = ordered_sum(partial, gridDim.x);
        if (threadIdx.x == 0) *loss += t * scale;
    }
}

// Adjusting term (F = (m / tau_adj) (v0 e0 - v)) and the agent's outputs.
__device__ __forceinline__ void adj_finish(const StepArgs &a, const AdjArgs &q, int i, double uxi,
                                           double uyi, PairGrad G) {
    double *const *col = a.col;
    const double m = col[MASS][i], ta = col[TAU_ADJ][i], v0 = col[V0][i];
    const double ex = col[E0X][i], ey = col[E0Y][i];
    const double kk = m / ta;
    G.gvx -= kk * uxi;
    G.gvy -= kk * uyi;
    const double g_ta =
        -(m / (ta * ta)) * (uxi * (v0 * ex - col[VX][i]) + uyi * (v0 * ey - col[VY][i]));
    const double g_v0 = kk * (uxi * ex + uyi * ey);
    q.lx_out[2 * i] = q.lx[2 * i] + G.gxx;
    q.lx_out[2 * i + 1] = q.lx[2 * i + 1] + G.gxy;
    q.lv_out[2 * i] = q.lvt[2 * i] + G.gvx;
    q.lv_out[2 * i + 1] = q.lvt[2 * i + 1] + G.gvy;
    q.grad[4 * i + 0] += g_ta;
    q.grad[4 * i + 1] += g_v0;
    q.grad[4 * i + 2] += G.gt0;
    q.grad[4 * i + 3] += G.gk;
}

// Pair, wall and adjusting terms of the reverse step.  A group of L lanes
// takes the agent in cell-sorted slot s: its 3 x 3 neighbour cells are three
// runs of consecutive slots, which the lanes stride through; the lanes'
// partial sums meet in a fixed butterfly, so the result is deterministic.
template <int L>
__global__ void __launch_bounds__(NT) k_adj_forces(StepArgs a, AdjArgs q, int only_if_over) {
    pdl_enter();
    // as the pair pipeline's fallback: only for a step whose near lists did not fit
    if (only_if_over && !(a.nl_off[a.n] > a.nl_cap)) return;
    const int r = threadIdx.x & (L - 1);
    const int s = (int)(((long long)blockIdx.x * NT + threadIdx.x) / L);
    const bool valid = s < a.n;
    PairGrad G{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int i = 0;
    double uxi = 0.0, uyi = 0.0;
    if (valid) {
        i = a.perm[s];
        const ScenDev sc = a.scen[a.scen_of[i]];
        const float4 me = a.cull[s];
        const int my_cell = a.key[i];
        const Circ A = load_circ(a.stage, s);
        uxi = q.lF[2 * i];
        uyi = q.lF[2 * i + 1];
        const int local = my_cell - sc.cell_base;
        const int ix = local / sc.ny, iy = local - ix * sc.ny;
        const int jy0 = iy > 0 ? iy - 1 : 0, jy1 = iy + 1 < sc.ny ? iy + 1 : sc.ny - 1;
        for (int jx = ix - 1; jx <= ix + 1; ++jx) {
            if (jx < 0 || jx >= sc.nx) continue;
            const int c0 = sc.cell_base + jx * sc.ny;
            const int b = __ldg(&a.start[c0 + jy0]), e = __ldg(&a.start[c0 + jy1 + 1]);
            for (int t = b + r; t < e; t += L) {
                if (t == s || pair_far(me, __ldg(&a.cull[t]))) continue;
                const Circ B = load_circ(a.stage, t);
                const int j = a.perm[t];
                pair_vjp_both(A, B, uxi, uyi, q.lF[2 * j], q.lF[2 * j + 1], G);
            }
        }
        if (sc.wall_count > 0) {
            const bool all_walls = me.z > (float)sc.wall_reach;
            const int wb = all_walls ? sc.wall_begin : __ldg(&a.wall_start[my_cell]);
            const int we = all_walls ? sc.wall_begin + sc.wall_count
                                     : __ldg(&a.wall_start[my_cell + 1]);
            for (int qw = wb + r; qw < we; qw += L) {
                const int w = all_walls ? qw : __ldg(&a.wall_idx[qw]);
                wall_circ_vjp(A, a.walls + (size_t)w * WALL_D, uxi, uyi, G.gxx, G.gxy, G.gvx,
                              G.gvy);
            }
        }
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
        G.gxx += __shfl_xor_sync(0xffffffffu, G.gxx, o);
        G.gxy += __shfl_xor_sync(0xffffffffu, G.gxy, o);
        G.gvx += __shfl_xor_sync(0xffffffffu, G.gvx, o);
        G.gvy += __shfl_xor_sync(0xffffffffu, G.gvy, o);
        G.gk += __shfl_xor_sync(0xffffffffu, G.gk, o);
        G.gt0 += __shfl_xor_sync(0xffffffffu, G.gt0, o);
    }
    if (!valid || r != 0) return;
    adj_finish(a, q, i, uxi, uyi, G);
}

// ---- compute-once form over the near lists of the forward pipeline ----
//
// Every unordered pair once (flat list of (slot, entry) with the later slot
// in the entry): G = dPhi/d(x_i - x_j), dPhi/d(v_i - v_j) of the pair's
// seed Phi goes to the first agent's entry and -G to the partner's entry for
// it, each with its own k_soc / tau_0 terms; a per-agent pass then adds the
// entries in list order (deterministic), the walls and adjusting.

__device__ __forceinline__ int partner_entry(const StepArgs &a, int t, int s) {
    int lo = __ldg(&a.nl_off[t]), hi = __ldg(&a.nl_fwd[t]);
    const int end = hi;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.nl_idx[mid]) < s) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && __ldg(&a.nl_idx[lo]) == s) ? lo : -1;
}

// An entry's adjoint record, marked present (kind 1; the float32 pass marks
// the entries of the pairs it certifies to have no force empty, kind 0).
__device__ __forceinline__ void put_adj(const StepArgs &a, int e, double gx, double gy,
                                        double gvx, double gvy, double gk, double gt0) {
    double2 *p = reinterpret_cast<double2 *>(a.nl_res + (size_t)e * ADJ_RES_D);
    p[0] = make_double2(gx, gy);
    p[1] = make_double2(gvx, gvy);
    p[2] = make_double2(gk, gt0);
    a.nl_kind[e] = 1;
}

// The flat list's first part (pairs guessed to need the social force), then
// the pairs of the second part that the float32 pass could not certify to be
// without a force; that pass marked the others' entries empty.
__global__ void __launch_bounds__(NT) k_adj_pairs(StepArgs a, AdjArgs q) {
    pdl_enter();
    if (a.nl_off[a.n] > a.nl_cap) return;
    const int nfirst = a.fs_off[a.n];
    const int npairs = nfirst + a.work[1];
    for (int kk = blockIdx.x * NT + threadIdx.x; kk < npairs; kk += gridDim.x * NT) {
        const int k = kk < nfirst ? kk : a.defer_list[kk - nfirst];
        const int2 pe = __ldg(&a.fw_pairs[k]);
        const int s = pe.x, e = pe.y;
        const int t = __ldg(&a.nl_idx[e]);
        const int i = a.perm[s], j = a.perm[t];
        PairGrad G{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        double gkj = 0.0, gt0j = 0.0;
        pair_vjp_both(load_circ(a.stage, s), load_circ(a.stage, t), q.lF[2 * i], q.lF[2 * i + 1],
                      q.lF[2 * j], q.lF[2 * j + 1], G, &gkj, &gt0j);
        put_adj(a, e, G.gxx, G.gxy, G.gvx, G.gvy, G.gk, G.gt0);
        const int eq = partner_entry(a, t, s);
        if (eq >= 0) put_adj(a, eq, -G.gxx, -G.gxy, -G.gvx, -G.gvy, gkj, gt0j);
        else atomicOr(a.err, ERR_NEAR_LIST);
    }
}

// L lanes per agent: lane r adds entries r, r + L, ... of the agent's list
// (those marked present)
// and walls r, r + L, ...; the lanes' sums meet in a fixed butterfly, so the
// result is deterministic.  One lane per agent left 5000 agents with one warp
// per SM, each lane walking about a hundred 48-byte entries in turn.  Each
// lane steps over its empty entries with integer work alone and the warp's
// lanes add their next present entries together, so that the six float64
// adds run once per present entry of the lane with the most, not at every
// entry where any lane has one (each lane keeps its own order).
template <int L>
__global__ void __launch_bounds__(NT) k_adj_gather(StepArgs a, AdjArgs q) {
    pdl_enter();
    if (a.nl_off[a.n] > a.nl_cap) return;               // k_adj_forces' step
    const int r = threadIdx.x & (L - 1);
    const int s = (int)(((long long)blockIdx.x * NT + threadIdx.x) / L);
    const bool valid = s < a.n;
    PairGrad G{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    int i = 0;
    double uxi = 0.0, uyi = 0.0;
    int e = 0, o1 = 0;
    if (valid) {
        e = a.nl_off[s] + r;
        o1 = a.nl_off[s + 1];
    }
    for (;;) {
        while (e < o1 && !a.nl_kind[e]) e += L;         // pairs without a force
        const bool has = e < o1;
        if (!__any_sync(0xffffffffu, has)) break;
        if (has) {
            const double2 *p = reinterpret_cast<const double2 *>(a.nl_res + (size_t)e * ADJ_RES_D);
            const double2 x = p[0], v = p[1], kt = p[2];
            G.gxx += x.x; G.gxy += x.y;
            G.gvx += v.x; G.gvy += v.y;
            G.gk += kt.x; G.gt0 += kt.y;
            e += L;
        }
    }
    if (valid) {
        i = a.perm[s];
        uxi = q.lF[2 * i];
        uyi = q.lF[2 * i + 1];
        const ScenDev sc = a.scen[a.scen_of[i]];
        if (sc.wall_count > 0) {
            const float4 me = a.cull[s];
            const int my_cell = a.key[i];
            const Circ A = load_circ(a.stage, s);
            const bool all_walls = me.z > (float)sc.wall_reach;
            const int wb = all_walls ? sc.wall_begin : __ldg(&a.wall_start[my_cell]);
            const int we = all_walls ? sc.wall_begin + sc.wall_count
                                     : __ldg(&a.wall_start[my_cell + 1]);
            for (int qw = wb + r; qw < we; qw += L) {
                const int w = all_walls ? qw : __ldg(&a.wall_idx[qw]);
                wall_circ_vjp(A, a.walls + (size_t)w * WALL_D, uxi, uyi, G.gxx, G.gxy, G.gvx,
                              G.gvy);
            }
        }
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
        G.gxx += __shfl_xor_sync(0xffffffffu, G.gxx, o);
        G.gxy += __shfl_xor_sync(0xffffffffu, G.gxy, o);
        G.gvx += __shfl_xor_sync(0xffffffffu, G.gvx, o);
        G.gvy += __shfl_xor_sync(0xffffffffu, G.gvy, o);
        G.gk += __shfl_xor_sync(0xffffffffu, G.gk, o);
        G.gt0 += __shfl_xor_sync(0xffffffffu, G.gt0, o);
    }
    if (!valid || r != 0) return;
    adj_finish(a, q, i, uxi, uyi, G);
}

// Copies of up to 8 state columns in one launch (checkpoint save / restore).
struct ColCopy {
    const double *src[8];
    double *dst[8];
    int ncol;
};

__global__ void k_copy_cols(ColCopy cc, int n) {
    pdl_enter();
    const int k = blockIdx.y;
    if (k >= cc.ncol) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        cc.dst[k][i] = cc.src[k][i];
}

// Copies of up to 16 device buffers in one launch (byte counts multiples of 4;
// 16-byte words where a buffer's size and both addresses allow).
struct BufCopy {
    const void *src[16];
    void *dst[16];
    long long bytes[16];
    int nbuf;
};

__global__ void k_copy_bufs(BufCopy bc) {
    const int k = blockIdx.y;
    if (k >= bc.nbuf) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long done = 0;
    if ((((uintptr_t)bc.src[k] | (uintptr_t)bc.dst[k]) & 15) == 0) {
        const uint4 *s4 = static_cast<const uint4 *>(bc.src[k]);
        uint4 *d4 = static_cast<uint4 *>(bc.dst[k]);
        const long long n4 = bc.bytes[k] / 16;
        for (long long w = t0; w < n4; w += stride) d4[w] = s4[w];
        done = n4 * 16;
    }
    const unsigned *s1 = static_cast<const unsigned *>(bc.src[k]);
    unsigned *d1 = static_cast<unsigned *>(bc.dst[k]);
    for (long long w = done / 4 + t0; w < bc.bytes[k] / 4; w += stride) d1[w] = s1[w];
}

// (value, index) of a maximum: the larger value, on ties the smaller index
// (-1 = none); NaN never wins.
__device__ __forceinline__ void better(double &v, int &j, double v2, int j2) {
    if (j2 >= 0 && (v2 > v || (v2 == v && (j < 0 || j2 < j)))) { v = v2; j = j2; }
}

// The timestep's own gradient, when dt was not clamped:
// dt = 1.1 V0 dt_max / Vm  ->  d/dV0 = dt / V0,  d/dVm = -dt / Vm.
// Warp 0 of k_adj_argmax's last block: the blocks' maxima combined (the
// largest value, on ties the first index: the same whatever the order).
__device__ __forceinline__ void adj_dt(const AdjArgs &q, double dt_min, double dt_max,
                                       const double *vx, const double *vy) {
    const int lane = threadIdx.x & 31;
    double Vm = 0.0, V0 = -INFINITY;
    int jv = -1, j0 = -1;
    for (int b = lane; b < (int)gridDim.x; b += 32) {
        better(Vm, jv, __ldcg(q.argmax_vals + 2 * b), __ldcg(q.argmax_idx + 2 * b));
        better(V0, j0, __ldcg(q.argmax_vals + 2 * b + 1), __ldcg(q.argmax_idx + 2 * b + 1));
    }
    for (int o = 16; o > 0; o >>= 1) {
        better(Vm, jv, __shfl_xor_sync(0xffffffffu, Vm, o), __shfl_xor_sync(0xffffffffu, jv, o));
        better(V0, j0, __shfl_xor_sync(0xffffffffu, V0, o), __shfl_xor_sync(0xffffffffu, j0, o));
    }
    if (lane != 0) return;
    const double dt = *q.dt, ldt = *q.ldt;
    if (!(Vm > 0) || !(dt > dt_min && dt < dt_max)) return;
    if (j0 >= 0) q.grad[4 * j0 + 1] += ldt * dt / V0;
    if (jv >= 0) {
        double c = ldt * (-dt / Vm) / Vm;
        q.lv_out[2 * jv] += c * vx[jv];
        q.lv_out[2 * jv + 1] += c * vy[jv];
    }
}

// Per block: max |v| (positive values only) and max v0 with their first
// indices, written to vals / idx [2 * block + {0, 1}]; the last block
// combines the blocks (adj_dt).  |v| = hypot(vx, vy) only where q = vx^2 + vy^2 can hold the
// block's maximum: q is within 4 ulp of |v|^2, so a lane 2^-40 below the
// block's largest q has a |v| smaller by far more than hypot's 2 ulp
// (non-finite q, and blocks whose largest q is tiny, take hypot everywhere).
__global__ void k_adj_argmax(AdjArgs aq, double dt_min, double dt_max, const double *vx,
                             const double *vy, const double *v0, int n) {
    pdl_enter();
    double *vals = aq.argmax_vals;
    int *idx = aq.argmax_idx;
    __shared__ double sq[RED_NT / 32], sv[RED_NT / 32], s0[RED_NT / 32];
    __shared__ int jv_s[RED_NT / 32], j0_s[RED_NT / 32];
    const int i = blockIdx.x * RED_NT + threadIdx.x, w = threadIdx.x >> 5;
    const bool in = i < n;
    const double x = in ? vx[i] : 0.0, y = in ? vy[i] : 0.0;
    const double q = x * x + y * y;
    double qm = (in && q > 0) ? q : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, qm, o);
        qm = (t > qm) ? t : qm;
    }
    if ((threadIdx.x & 31) == 0) sq[w] = qm;
    __syncthreads();
    qm = sq[0];
#pragma unroll
    for (int k = 1; k < RED_NT / 32; ++k) qm = (sq[k] > qm) ? sq[k] : qm;
    const double thr = !(qm >= 0x1p-900) ? 0.0
                       : (qm <= 0x1.fffffffffffffp+1023 ? qm * (1.0 - 0x1p-40)
                                                        : 0x1.fffffffffffffp+1022);
    double mv = 0.0, m0 = -INFINITY;
    int jv = -1, j0 = -1;
    if (in && !(q < thr)) {
        const double l = cdm_hypot(x, y);
        if (l > mv) { mv = l; jv = i; }
    }
    if (in && v0[i] > m0) { m0 = v0[i]; j0 = i; }
    for (int o = 16; o > 0; o >>= 1) {
        better(mv, jv, __shfl_xor_sync(0xffffffffu, mv, o), __shfl_xor_sync(0xffffffffu, jv, o));
        better(m0, j0, __shfl_xor_sync(0xffffffffu, m0, o), __shfl_xor_sync(0xffffffffu, j0, o));
    }
    if ((threadIdx.x & 31) == 0) { sv[w] = mv; jv_s[w] = jv; s0[w] = m0; j0_s[w] = j0; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < RED_NT / 32; ++k) {
            better(mv, jv, sv[k], jv_s[k]);
            better(m0, j0, s0[k], j0_s[k]);
        }
        vals[2 * blockIdx.x] = mv; vals[2 * blockIdx.x + 1] = m0;
        idx[2 * blockIdx.x] = jv; idx[2 * blockIdx.x + 1] = j0;
    }
    if (last_block(aq.blocks_done) && threadIdx.x < 32) adj_dt(aq, dt_min, dt_max, vx, vy);
}

inline int nblk(long long n, int nt) { return (int)((n + nt - 1) / nt); }

}  // namespace

int adj_partials(int n) { return nblk(n, RED_NT) > 0 ? nblk(n, RED_NT) : 1; }

void launch_adj_seed(const AdjArgs &q, cudaStream_t s) {
    launch_k(true, k_adj_seed, adj_partials(q.n), RED_NT, 0, s, q);
}
void launch_adj_forces(const StepArgs &a, const AdjArgs &q, cudaStream_t s) {
    if (a.n <= 0) return;
    const long long n = a.n;
    const int over = a.nl_cnt != nullptr;     // pair pipeline first, this as its fallback
    if (over) {
        launch_adj_light(a, s);
        launch_k(true, k_adj_pairs, nblk(n * 16, NT), NT, 0, s, a, q);
        // lanes per agent: enough warps to fill the SMs at small agent counts
        if (n < 20000) launch_k(true, k_adj_gather<16>, nblk(n * 16, NT), NT, 0, s, a, q);
        else launch_k(true, k_adj_gather<4>, nblk(n * 4, NT), NT, 0, s, a, q);
    }
    // lanes per agent: enough warps to fill the SMs at small agent counts
    if (n < 20000) launch_k(over, k_adj_forces<16>, nblk(n * 16, NT), NT, 0, s, a, q, over);
    else if (n < 80000) launch_k(over, k_adj_forces<8>, nblk(n * 8, NT), NT, 0, s, a, q, over);
    else launch_k(over, k_adj_forces<4>, nblk(n * 4, NT), NT, 0, s, a, q, over);
}
void launch_copy_cols(const double *const *src, double *const *dst, int ncol, int n,
                      cudaStream_t s, bool dep) {
    if (n <= 0 || ncol <= 0) return;
    ColCopy cc;
    for (int k = 0; k < 8; ++k) {
        cc.src[k] = k < ncol ? src[k] : nullptr;
        cc.dst[k] = k < ncol ? dst[k] : nullptr;
    }
    cc.ncol = ncol < 8 ? ncol : 8;
    int nb = nblk(n, 256);
    if (nb > 1024) nb = 1024;
    launch_k(dep, k_copy_cols, dim3(nb, cc.ncol), 256, 0, s, cc, n);
}
void launch_copy_bufs(const void *const *src, void *const *dst, const long long *bytes, int nbuf,
                      cudaStream_t s) {
    if (nbuf <= 0) return;
    BufCopy bc;
    long long most = 0;
    for (int k = 0; k < 16; ++k) {
        bc.src[k] = k < nbuf ? src[k] : nullptr;
        bc.dst[k] = k < nbuf ? dst[k] : nullptr;
        bc.bytes[k] = k < nbuf ? bytes[k] : 0;
        if (k < nbuf) most = std::max(most, bytes[k]);
    }
    bc.nbuf = nbuf < 16 ? nbuf : 16;
    int nb = (int)std::min<long long>((most / 16 + 255) / 256, 512);
    if (nb < 1) nb = 1;
    k_copy_bufs<<<dim3(nb, bc.nbuf), 256, 0, s>>>(bc);
}
void launch_adj_dt(const AdjArgs &q, double dt_min, double dt_max, const double *vx,
                   const double *vy, const double *v0, cudaStream_t s) {
    launch_k(true, k_adj_argmax, adj_partials(q.n), RED_NT, 0, s, q, dt_min, dt_max, vx, vy, v0,
             q.n);
}
void launch_loss(const double *x, const double *y, const double *target, int n, double *partial,
                 double *loss, double scale, int *blocks_done, const double *dt_src,
                 double *dt_dst, cudaStream_t s) {
    k_loss<<<adj_partials(n), RED_NT, 0, s>>>(x, y, target, n, partial, loss, scale, blocks_done,
                                              dt_src, dt_dst);
}
}  // namespace cdk
