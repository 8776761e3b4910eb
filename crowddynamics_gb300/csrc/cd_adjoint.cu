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
#include <cstdint>
#include <cmath>
#include "cd_internal.cuh"
#include "cd_math.h"

namespace cdk {
namespace {

constexpr double SIGTH_SOC = 3.0;
constexpr double F_SOC_MAX = 2e3;
constexpr double TAU_MAX = 30.0;
constexpr float CULL_MARGIN = 0.01f;
constexpr int NT = 128;
constexpr int RED_NT = 256;

struct Circ {
    double x, y, vx, vy, r, m, k, tau0, mu, kappa, damp;
};

__device__ __forceinline__ Circ load_circ(const double2 *__restrict__ st, int slot) {
    const double2 *p = st + (size_t)slot * STAGE_Q_CIRC;
    double2 q0 = __ldg(p), q1 = __ldg(p + 1), q2 = __ldg(p + 2), q3 = __ldg(p + 3),
            q4 = __ldg(p + 4), q5 = __ldg(p + 5);
    Circ a;
    a.x = q0.x; a.y = q0.y; a.vx = q1.x; a.vy = q1.y; a.r = q2.x; a.m = q2.y;
    a.k = q3.x; a.tau0 = q3.y; a.mu = q4.x; a.kappa = q4.y; a.damp = q5.x;
    return a;
}

__device__ __forceinline__ bool pair_far(float4 me, float4 o) {
    float dx = me.x - o.x, dy = me.y - o.y;
    float lim = (float)SIGTH_SOC + me.z + o.z + CULL_MARGIN;
    return dx * dx + dy * dy > lim * lim;
}

// Reverse of the contact force -h (mu n - kappa (v.t) t) + c (v.n) n with
// h = |x| - r, n = x / |x|, t = rotate270(n), seed u; adds d(u.F)/dx, /dv.
__device__ __forceinline__ void contact_vjp(double xx, double xy, double d0, double h, double vx,
                                            double vy, double mu, double kappa, double damp,
                                            double ux, double uy, double &gxx, double &gxy,
                                            double &gvx, double &gvy) {
    double nx = xx / d0, ny = xy / d0;
    double tx = ny, ty = -nx;
    double vt = vx * tx + vy * ty, vn = vx * nx + vy * ny;
    double ut = ux * tx + uy * ty, un = ux * nx + uy * ny;
    gvx += h * kappa * ut * tx + damp * un * nx;
    gvy += h * kappa * ut * ty + damp * un * ny;
    double A = -mu * un + kappa * vt * ut;                   // coefficient of dh = n . dx
    double w1x = -h * mu * ux + damp * (un * vx + vn * ux);  // through dn = P dx / |x|
    double w1y = -h * mu * uy + damp * (un * vy + vn * uy);
    double w2x = h * kappa * (ut * vx + vt * ux);            // through dt = R P dx / |x|
    double w2y = h * kappa * (ut * vy + vt * uy);
    double qx = w1x + (-w2y), qy = w1y + w2x;                // w1 + R^T w2
    double pq = nx * qx + ny * qy;                           // P q = q - n (n . q)
    gxx += A * nx + (qx - nx * pq) / d0;
    gxy += A * ny + (qy - ny * pq) / d0;
}

// Reverse of one side's Circular pair force (interactions.py:51-70 with
// power_law.py:213-259), evaluated in that side's frame (x = x_me - x_other,
// v = v_me - v_other), seed u = adjoint of the side's total force.
__device__ void pair_circ_vjp(double xx, double xy, double vx, double vy, double r_tot, double m,
                              double k, double tau0, double mu, double kappa, double damp,
                              double ux, double uy, double &gxx, double &gxy, double &gvx,
                              double &gvy, double &gk, double &gtau0) {
    double d0 = cdm_hypot(xx, xy);
    double h = d0 - r_tot;
    if (!(h < SIGTH_SOC)) return;
    double a = vx * vx + vy * vy;
    double b = -(xx * vx + xy * vy);
    double c = (xx * xx + xy * xy) - r_tot * r_tot;
    double disc = b * b - a * c;
    if (disc > 0 && a != 0) {
        double dd = sqrt(disc);
        double tau = (b - dd) / a;
        if (!(tau <= 0 || tau > TAU_MAX)) {
            double gx = (vx - (vx * b + xx * a) / dd) / a;   // grad of tau
            double gy = (vy - (vy * b + xy * a) / dd) / a;
            double cm = (-m) * k;
            double e = cdm_exp(-tau / tau0);
            double mg = (2.0 / tau + 1.0 / tau0) * e / (tau * tau);
            double Fx = (cm * gx) * mg, Fy = (cm * gy) * mg;
            double L = cdm_hypot(Fx, Fy);
            double lx = ux, ly = uy;
            if (L > F_SOC_MAX) {                             // truncate (vector2D.py:166-187)
                double fx = Fx / L, fy = Fy / L, s = F_SOC_MAX / L;
                double dot = ux * fx + uy * fy;
                lx = s * (ux - dot * fx);
                ly = s * (uy - dot * fy);
            }
            double lgx = cm * mg * lx, lgy = cm * mg * ly;   // F_raw = cm mg g
            double lgdot = lx * gx + ly * gy;
            double lmg = cm * lgdot;
            gk += mg * lgdot * (-m);
            double t2 = tau * tau, t3 = t2 * tau, t02 = tau0 * tau0;
            double dmg_dtau = -e * (6.0 / (t3 * tau) + 4.0 / (t3 * tau0) + 1.0 / (t2 * t02));
            double dmg_dtau0 = e * (1.0 / (t2 * t02) + 1.0 / (tau * t02 * tau0));
            double ltau = lmg * dmg_dtau;
            gtau0 += lmg * dmg_dtau0;
            // g = v / a - b v / (a dd) - x / dd
            double la = -(lgx * (gx + xx / dd) + lgy * (gy + xy / dd)) / a;
            double lb = -(lgx * vx + lgy * vy) / (a * dd);
            double ldd = (lgx * (b * vx / a + xx) + lgy * (b * vy / a + xy)) / (dd * dd);
            double cv = 1.0 / a - b / (a * dd);
            gvx += cv * lgx;
            gvy += cv * lgy;
            gxx += -lgx / dd;
            gxy += -lgy / dd;
            lb += ltau / a;                                  // tau = (b - dd) / a
            ldd += -ltau / a;
            la += -ltau * tau / a;
            double ldisc = ldd / (2.0 * dd);                 // dd = sqrt(b^2 - a c)
            lb += 2.0 * b * ldisc;
            la += -c * ldisc;
            double lc = -a * ldisc;
            gxx += 2.0 * lc * xx;                            // c = x.x - r^2
            gxy += 2.0 * lc * xy;
            gxx += -lb * vx;                                 // b = -x.v
            gxy += -lb * vy;
            gvx += -lb * xx;
            gvy += -lb * xy;
            gvx += 2.0 * la * vx;                            // a = v.v
            gvy += 2.0 * la * vy;
        }
    }
    if (h < 0 && d0 != 0.0)
        contact_vjp(xx, xy, d0, h, vx, vy, mu, kappa, damp, ux, uy, gxx, gxy, gvx, gvy);
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
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < q.n) {
        const double dt = *q.dt;
        const double m = q.mass[i];
        double lxx = q.lx[2 * i], lxy = q.lx[2 * i + 1];
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
}

// Sum of block partials in index order (one thread: deterministic).
__global__ void k_adj_sum(const double *partial, int nb, double *out, double scale, int accumulate) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double s = 0.0;
    for (int k = 0; k < nb; ++k) s += partial[k];
    if (accumulate) *out += s * scale;
    else *out = s * scale;
}

// Loss partials: sum_i |x_i - target_i|^2 per block.
__global__ void k_loss_partial(const double *x, const double *y, const double *target, int n,
                               double *partial) {
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
}

// lx += scale * 2 (x - target)
__global__ void k_loss_grad(const double *x, const double *y, const double *target, int n,
                            double scale, double *lx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lx[2 * i] += scale * 2.0 * (x[i] - target[2 * i]);
    lx[2 * i + 1] += scale * 2.0 * (y[i] - target[2 * i + 1]);
}

// Pair, wall and adjusting terms of the reverse step for the agent in
// cell-sorted slot s; writes lx_out, lv_out and accumulates parameter grads.
__global__ void __launch_bounds__(NT) k_adj_forces(StepArgs a, AdjArgs q) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n) return;
    const int i = a.perm[s];
    const ScenDev sc = a.scen[a.scen_of[i]];
    double *const *col = a.col;
    const float4 me = a.cull[s];
    const int my_cell = a.key[i];
    const Circ A = load_circ(a.stage, s);
    const double uxi = q.lF[2 * i], uyi = q.lF[2 * i + 1];
    double gxx = 0, gxy = 0, gvx = 0, gvy = 0, gk = 0, gt0 = 0;
    // agent-agent, both sides of every pair, in the forward visiting order
    int local = my_cell - sc.cell_base;
    int ix = local / sc.ny, iy = local - ix * sc.ny;
    for (int ck = 0; ck < 9; ++ck) {
        int jx = ix + ck / 3 - 1, jy = iy + ck % 3 - 1;
        if (jx < 0 || jx >= sc.nx || jy < 0 || jy >= sc.ny) continue;
        int c2 = sc.cell_base + jx * sc.ny + jy;
        int b = __ldg(&a.start[c2]), e = __ldg(&a.start[c2 + 1]);
        for (int t = b; t < e; ++t) {
            if (t == s) continue;
            if (pair_far(me, __ldg(&a.cull[t]))) continue;
            const Circ B = load_circ(a.stage, t);
            const int j = a.perm[t];
            // my side: F_i(x_i - x_j, v_i - v_j)
            pair_circ_vjp(A.x - B.x, A.y - B.y, A.vx - B.vx, A.vy - B.vy, A.r + B.r, A.m, A.k,
                          A.tau0, A.mu, A.kappa, A.damp, uxi, uyi, gxx, gxy, gvx, gvy, gk, gt0);
            // neighbour's side: F_j(x_j - x_i, v_j - v_i), d/dx_i = -d/dx_rel
            double hx = 0, hy = 0, hvx = 0, hvy = 0, dk = 0, dt0 = 0;
            pair_circ_vjp(B.x - A.x, B.y - A.y, B.vx - A.vx, B.vy - A.vy, B.r + A.r, B.m, B.k,
                          B.tau0, B.mu, B.kappa, B.damp, q.lF[2 * j], q.lF[2 * j + 1], hx, hy,
                          hvx, hvy, dk, dt0);
            gxx -= hx; gxy -= hy; gvx -= hvx; gvy -= hvy;
        }
    }
    // walls
    if (sc.wall_count > 0) {
        const bool all_walls = me.z > (float)sc.wall_reach;
        int wb = all_walls ? sc.wall_begin : __ldg(&a.wall_start[my_cell]);
        int we = all_walls ? sc.wall_begin + sc.wall_count : __ldg(&a.wall_start[my_cell + 1]);
        for (int qw = wb; qw < we; ++qw) {
            int w = all_walls ? qw : __ldg(&a.wall_idx[qw]);
            wall_circ_vjp(A, a.walls + (size_t)w * WALL_D, uxi, uyi, gxx, gxy, gvx, gvy);
        }
    }
    // adjusting: F = (m / tau_adj) (v0 e0 - v)
    const double m = col[MASS][i], ta = col[TAU_ADJ][i], v0 = col[V0][i];
    const double ex = col[E0X][i], ey = col[E0Y][i];
    const double kk = m / ta;
    gvx -= kk * uxi;
    gvy -= kk * uyi;
    double g_ta = -(m / (ta * ta)) * (uxi * (v0 * ex - col[VX][i]) + uyi * (v0 * ey - col[VY][i]));
    double g_v0 = kk * (uxi * ex + uyi * ey);
    q.lx_out[2 * i] = q.lx[2 * i] + gxx;
    q.lx_out[2 * i + 1] = q.lx[2 * i + 1] + gxy;
    q.lv_out[2 * i] = q.lvt[2 * i] + gvx;
    q.lv_out[2 * i + 1] = q.lvt[2 * i + 1] + gvy;
    q.grad[4 * i + 0] += g_ta;
    q.grad[4 * i + 1] += g_v0;
    q.grad[4 * i + 2] += gt0;
    q.grad[4 * i + 3] += gk;
}

// max |v| and max v0 with their first indices (single block, index order).
__global__ void k_adj_argmax(const double *vx, const double *vy, const double *v0, int n,
                             double *out_vals, int *out_idx) {
    __shared__ double bv[RED_NT], b0[RED_NT];
    __shared__ int iv[RED_NT], i0[RED_NT];
    double mv = 0.0, m0 = -INFINITY;
    int jv = -1, j0 = -1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double l = cdm_hypot(vx[i], vy[i]);
        if (l > mv) { mv = l; jv = i; }
        if (v0[i] > m0) { m0 = v0[i]; j0 = i; }
    }
    bv[threadIdx.x] = mv; iv[threadIdx.x] = jv; b0[threadIdx.x] = m0; i0[threadIdx.x] = j0;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 1; t < (int)blockDim.x; ++t) {
            if (bv[t] > mv || (bv[t] == mv && iv[t] >= 0 && iv[t] < jv)) { mv = bv[t]; jv = iv[t]; }
            if (b0[t] > m0 || (b0[t] == m0 && i0[t] >= 0 && i0[t] < j0)) { m0 = b0[t]; j0 = i0[t]; }
        }
        out_vals[0] = mv; out_vals[1] = m0;
        out_idx[0] = jv; out_idx[1] = j0;
    }
}

// The timestep's own gradient, when dt was not clamped:
// dt = 1.1 V0 dt_max / Vm  ->  d/dV0 = dt / V0,  d/dVm = -dt / Vm.
__global__ void k_adj_dt(AdjArgs q, double dt_min, double dt_max, const double *vx,
                         const double *vy) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const double dt = *q.dt, ldt = *q.ldt;
    const double Vm = q.argmax_vals[0], V0 = q.argmax_vals[1];
    if (!(Vm > 0) || !(dt > dt_min && dt < dt_max)) return;
    const int jv = q.argmax_idx[0], j0 = q.argmax_idx[1];
    if (j0 >= 0) q.grad[4 * j0 + 1] += ldt * dt / V0;
    if (jv >= 0) {
        double c = ldt * (-dt / Vm) / Vm;
        q.lv_out[2 * jv] += c * vx[jv];
        q.lv_out[2 * jv + 1] += c * vy[jv];
    }
}

inline int nblk(long long n, int nt) { return (int)((n + nt - 1) / nt); }

}  // namespace

int adj_partials(int n) { return nblk(n, RED_NT) > 0 ? nblk(n, RED_NT) : 1; }

void launch_adj_seed(const AdjArgs &q, cudaStream_t s) {
    int nb = adj_partials(q.n);
    k_adj_seed<<<nb, RED_NT, 0, s>>>(q);
    k_adj_sum<<<1, 1, 0, s>>>(q.partial, nb, q.ldt, 1.0, 0);
}
void launch_adj_forces(const StepArgs &a, const AdjArgs &q, cudaStream_t s) {
    if (a.n > 0) k_adj_forces<<<nblk(a.n, NT), NT, 0, s>>>(a, q);
}
void launch_adj_dt(const AdjArgs &q, double dt_min, double dt_max, const double *vx,
                   const double *vy, const double *v0, cudaStream_t s) {
    k_adj_argmax<<<1, RED_NT, 0, s>>>(vx, vy, v0, q.n, q.argmax_vals, q.argmax_idx);
    k_adj_dt<<<1, 1, 0, s>>>(q, dt_min, dt_max, vx, vy);
}
void launch_loss(const double *x, const double *y, const double *target, int n, double *partial,
                 double *loss, double scale, cudaStream_t s) {
    int nb = adj_partials(n);
    k_loss_partial<<<nb, RED_NT, 0, s>>>(x, y, target, n, partial);
    k_adj_sum<<<1, 1, 0, s>>>(partial, nb, loss, scale, 1);
}
void launch_loss_grad(const double *x, const double *y, const double *target, int n,
                      double scale, double *lx, cudaStream_t s) {
    if (n > 0) k_loss_grad<<<nblk(n, RED_NT), RED_NT, 0, s>>>(x, y, target, n, scale, lx);
}

}  // namespace cdk
