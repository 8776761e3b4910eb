/*
 * cd_oracle.c -- CPU restatement of crowddynamics' per-step agent update.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the device path is
 * checked against and the timed CPU baseline; nothing in the product imports
 * or links it.  Each function restates one reference function operation by
 * operation in IEEE float64 (built with -O2 -ffp-contract=off, no fast-math)
 * and cites the reference file:line it follows.  It is itself pinned against
 * the reference's own Python source (executed with stub modules) by the
 * golden fixtures under tests/golden/.
 *
 * Agent records are the reference's packed numpy structured records; fields
 * are addressed through a table of byte offsets (ORC_F_* order) so the same
 * code serves Circular and ThreeCircle arrays.
 *
 * The neighbour search restates the third-party package `cell_lists`
 * (pinned only as git+https://github.com/jaantollander/cell_lists.git, no
 * version; source absent): agents are binned on a uniform grid, grouped by
 * cell in ascending agent order, and every unordered pair of agents in the
 * same or Chebyshev-adjacent cells is visited once, oriented (owner, other)
 * with the owner cell visited in ascending flat order.  See orc_cell_list.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "cd_math.h"
#include "cd_noise.h"

/* Elementary functions: the C library's by default (the plain restatement),
 * or the shared cd_math.h implementations that the device kernels use, so
 * that device results can be compared bit for bit. */
static int g_exact_math = 0;
void orc_set_exact_math(int on) { g_exact_math = on; }
static inline double m_hypot(double x, double y) { return g_exact_math ? cdm_hypot(x, y) : hypot(x, y); }
static inline double m_exp(double x) { return g_exact_math ? cdm_exp(x) : exp(x); }
static inline double m_sin(double x) { return g_exact_math ? cdm_sin(x) : sin(x); }
static inline double m_cos(double x) { return g_exact_math ? cdm_cos(x) : cos(x); }
static inline double m_atan2(double y, double x) { return g_exact_math ? cdm_atan2(y, x) : atan2(y, x); }

enum {
    F_POSITION = 0, F_VELOCITY, F_TARGET_DIRECTION, F_FORCE, F_FORCE_PREV,
    F_RADIUS, F_R_T, F_R_S, F_R_TS, F_MASS, F_INERTIA_ROT, F_TARGET_VELOCITY,
    F_TARGET_ANGULAR_VELOCITY, F_TAU_ADJ, F_K_SOC, F_TAU_0, F_MU, F_KAPPA,
    F_DAMPING, F_STD_RAND_FORCE, F_POSITION_LS, F_POSITION_RS, F_ORIENTATION,
    F_ANGULAR_VELOCITY, F_TARGET_ORIENTATION, F_TORQUE, F_TORQUE_PREV,
    F_TAU_ROT, F_STD_RAND_TORQUE, F_TARGET, F_COUNT
};

enum { BODY_CIRCULAR = 0, BODY_THREE_CIRCLE = 1 };

enum {
    ORC_FLUCTUATION = 1, ORC_ORIENTATION = 2, ORC_ADJUSTING = 4,
    ORC_AGENT_AGENT = 8, ORC_AGENT_OBSTACLE = 16, ORC_INTEGRATE = 32,
    ORC_RESET = 64,
    ORC_NAVIGATION = 128
};

/* core/interactions.py:45 and core/motion/power_law.py:52 */
#define SIGTH_SOC 3.0
#define F_SOC_MAX 2e3
#define PI 3.141592653589793

typedef struct {
    char *base;
    int64_t itemsize;
    const int64_t *off;
} arr_t;

typedef struct { double x, y; } v2;

static inline double ld(const arr_t *A, int64_t i, int f) {
    double v;
    memcpy(&v, A->base + i * A->itemsize + A->off[f], 8);
    return v;
}
static inline v2 ld2(const arr_t *A, int64_t i, int f) {
    v2 v;
    memcpy(&v.x, A->base + i * A->itemsize + A->off[f], 8);
    memcpy(&v.y, A->base + i * A->itemsize + A->off[f] + 8, 8);
    return v;
}
static inline void st(arr_t *A, int64_t i, int f, double v) {
    memcpy(A->base + i * A->itemsize + A->off[f], &v, 8);
}
static inline void st2(arr_t *A, int64_t i, int f, v2 v) {
    memcpy(A->base + i * A->itemsize + A->off[f], &v.x, 8);
    memcpy(A->base + i * A->itemsize + A->off[f] + 8, &v.y, 8);
}

/* ---- core/vector2D.py ------------------------------------------------- */

/* Python float modulo (numba restates CPython's float_rem). */
static double py_mod(double x, double y) {
    double m = fmod(x, y);
    if (m != 0.0) {
        if ((y < 0) != (m < 0)) m += y;
    } else {
        m = copysign(0.0, y);
    }
    return m;
}

/* core/vector2D.py:8-36 */
double orc_wrap_to_pi(double rad) {
    double r = py_mod(rad, 2 * PI);
    if (rad < 0 && r == PI) return -PI;
    else if (r > PI) return r - (2 * PI);
    else return r;
}

static inline v2 sub(v2 a, v2 b) { v2 r = {a.x - b.x, a.y - b.y}; return r; }
static inline v2 add(v2 a, v2 b) { v2 r = {a.x + b.x, a.y + b.y}; return r; }
static inline v2 scale(double s, v2 a) { v2 r = {s * a.x, s * a.y}; return r; }
static inline v2 divs(v2 a, double s) { v2 r = {a.x / s, a.y / s}; return r; }
static inline double dot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }      /* :116-131 */
static inline double cross(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }    /* :134-149 */
static inline double length(v2 a) { return m_hypot(a.x, a.y); }              /* :99-113 */
static inline v2 rotate90(v2 a) { v2 r = {-a.y, a.x}; return r; }           /* :39-59 */
static inline v2 rotate270(v2 a) { v2 r = {a.y, -a.x}; return r; }          /* :62-82 */
static inline double np_sign(double x) {
    if (x > 0) return 1.0;
    if (x < 0) return -1.0;
    return x; /* 0 -> 0, nan -> nan */
}
/* core/vector2D.py:166-187 */
static inline v2 truncate(v2 v, double l) {
    double vlen = length(v);
    if (vlen > l) {
        double s = l / vlen;
        v.x = v.x * s;
        v.y = v.y * s;
    }
    return v;
}

/* ---- core/distance.py ------------------------------------------------- */

/* core/distance.py:16-47 */
static inline double distance_circles(v2 x0, double r0, v2 x1, double r1, v2 *n) {
    v2 x = sub(x0, x1);
    double d = length(x);
    double r_tot = r0 + r1;
    double h = d - r_tot;
    if (d == 0.0) { n->x = 0.0; n->y = 0.0; }
    else { *n = divs(x, d); }
    return h;
}

/* core/distance.py:50-105, including r_moment1 built from x0[j_min] (:103). */
static double distance_three_circles(const v2 x0[3], const double r0[3],
                                     const v2 x1[3], const double r1[3],
                                     v2 *normal, v2 *rm0, v2 *rm1) {
    double h_min = NAN;
    v2 nrm = {0.0, 0.0};
    int i_min = 0, j_min = 0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            v2 n;
            double h = distance_circles(x0[i], r0[i], x1[j], r1[j], &n);
            if (h < h_min || isnan(h_min)) {
                h_min = h; nrm = n; i_min = i; j_min = j;
            }
        }
    *normal = nrm;
    *rm0 = sub(add(x0[i_min], scale(r0[i_min], nrm)), x0[0]);
    *rm1 = sub(sub(x0[j_min], scale(r1[j_min], nrm)), x1[0]);
    return h_min;
}

/* core/distance.py:108-146 */
static double distance_circle_line(v2 x, double r, v2 p0, v2 p1, v2 *n_out) {
    v2 d = sub(p1, p0);
    double l_w = length(d);
    v2 t_w = divs(d, l_w);
    v2 n_w = rotate90(t_w);
    v2 q0 = sub(x, p0);
    v2 q1 = sub(x, p1);
    double l_t = -dot(t_w, q1) - dot(t_w, q0);
    double d_iw;
    v2 n_iw;
    if (l_t > l_w) {
        d_iw = length(q0);
        n_iw = divs(q0, d_iw);
    } else if (l_t < -l_w) {
        d_iw = length(q1);
        n_iw = divs(q1, d_iw);
    } else {
        double l_n = dot(n_w, q0);
        d_iw = fabs(l_n);
        n_iw = scale(np_sign(l_n), n_w);
    }
    *n_out = n_iw;
    return d_iw - r;
}

/* core/distance.py:149-180 */
static double distance_three_circle_line(const v2 x[3], const double r[3],
                                         v2 p0, v2 p1, v2 *normal, v2 *rm) {
    double h_min = NAN;
    v2 nrm = {0.0, 0.0};
    int i_min = 0;
    for (int i = 0; i < 3; ++i) {
        v2 n;
        double h = distance_circle_line(x[i], r[i], p0, p1, &n);
        if (h < h_min || isnan(h_min)) { h_min = h; nrm = n; i_min = i; }
    }
    *normal = nrm;
    *rm = sub(sub(x[i_min], scale(r[i_min], nrm)), x[0]);
    return h_min;
}

/* ---- core/motion/contact.py:12-48 ------------------------------------- */
static inline v2 force_contact(double h, v2 n, v2 v, v2 t, double mu,
                               double kappa, double damping) {
    double vt = dot(v, t), vn = dot(v, n);
    v2 r;
    r.x = (-h) * (mu * n.x - (kappa * vt) * t.x) + (damping * vn) * n.x;
    r.y = (-h) * (mu * n.y - (kappa * vt) * t.y) + (damping * vn) * n.y;
    return r;
}

/* ---- core/motion/power_law.py ----------------------------------------- */

/* :83-102 */
static inline double magnitude(double tau, double tau_0) {
    return (2.0 / tau + 1.0 / tau_0) * m_exp(-tau / tau_0) / (tau * tau);
}

/* :213-259 */
static void force_social_circular(const arr_t *A, int64_t i, int64_t j,
                                  v2 *fi, v2 *fj) {
    v2 force_i = {0.0, 0.0}, force_j = {0.0, 0.0};
    v2 x_rel = sub(ld2(A, i, F_POSITION), ld2(A, j, F_POSITION));
    v2 v_rel = sub(ld2(A, i, F_VELOCITY), ld2(A, j, F_VELOCITY));
    double r_tot = ld(A, i, F_RADIUS) + ld(A, j, F_RADIUS);
    double a = dot(v_rel, v_rel);
    double b = -dot(x_rel, v_rel);
    double c = dot(x_rel, x_rel) - r_tot * r_tot;
    double d = sqrt(b * b - a * c);
    *fi = force_i; *fj = force_j;
    if (isnan(d) || d == 0 || a == 0) return;
    double tau = (b - d) / a;
    double tau_max = 30.0;
    if (tau <= 0 || tau > tau_max) return;
    v2 grad;   /* gradient_circle_circle :105-126 */
    grad.x = (v_rel.x - (v_rel.x * b + x_rel.x * a) / d) / a;
    grad.y = (v_rel.y - (v_rel.y * b + x_rel.y * a) / d) / a;
    double ci = (-ld(A, i, F_MASS)) * ld(A, i, F_K_SOC);
    double cj = (-ld(A, j, F_MASS)) * ld(A, j, F_K_SOC);
    double mi = magnitude(tau, ld(A, i, F_TAU_0));
    double mj = magnitude(tau, ld(A, j, F_TAU_0));
    force_i.x = 0.0 + (ci * grad.x) * mi;
    force_i.y = 0.0 + (ci * grad.y) * mi;
    force_j.x = 0.0 - (cj * grad.x) * mj;
    force_j.y = 0.0 - (cj * grad.y) * mj;
    *fi = truncate(force_i, F_SOC_MAX);
    *fj = truncate(force_j, F_SOC_MAX);
}

static inline void three_parts(const arr_t *A, int64_t i, v2 x[3], double r[3]) {
    x[0] = ld2(A, i, F_POSITION);
    x[1] = ld2(A, i, F_POSITION_LS);
    x[2] = ld2(A, i, F_POSITION_RS);
    r[0] = ld(A, i, F_R_T);
    r[1] = ld(A, i, F_R_S);
    r[2] = r[1];
}

/* :262-363 (first defined root is accepted even when negative, :324;
 * no tau_max cut-off) */
static void force_social_three_circle(const arr_t *A, int64_t i, int64_t j,
                                      v2 *fi, v2 *fj) {
    v2 force_i = {0.0, 0.0}, force_j = {0.0, 0.0};
    *fi = force_i; *fj = force_j;
    v2 v_rel = sub(ld2(A, i, F_VELOCITY), ld2(A, j, F_VELOCITY));
    double a = dot(v_rel, v_rel);
    if (a == 0) return;
    v2 x_i[3], x_j[3];
    double r_i[3], r_j[3];
    three_parts(A, i, x_i, r_i);
    three_parts(A, j, x_j, r_j);
    int contact_i = 0, contact_j = 0;
    double tau = NAN, b_min = NAN, d_min = NAN;
    for (int pi = 0; pi < 3; ++pi)
        for (int pj = 0; pj < 3; ++pj) {
            v2 x_rel = sub(x_i[pi], x_j[pj]);
            double r_tot = r_i[pi] + r_j[pj];
            double b = -dot(x_rel, v_rel);
            double c = dot(x_rel, x_rel) - r_tot * r_tot;
            double d = sqrt(b * b - a * c);
            if (isnan(d) || d == 0) continue;
            double tau_new = (b - d) / a;
            if (isnan(tau) || (0 < tau_new && tau_new < tau)) {
                contact_i = pi; contact_j = pj;
                tau = tau_new; b_min = b; d_min = d;
            }
        }
    if (isnan(tau) || tau <= 0) return;
    v2 r_off_i = {0.0, 0.0}, r_off_j = {0.0, 0.0};
    if (contact_i == 1 || contact_i == 2) {
        double phi = ld(A, i, F_ORIENTATION);
        double rts = ld(A, i, F_R_TS);
        v2 e = {m_sin(phi), -m_cos(phi)};
        v2 o = {rts * e.x, rts * e.y};
        if (contact_i == 1) r_off_i = add(r_off_i, o);
        else r_off_i = sub(r_off_i, o);
    }
    if (contact_j == 1 || contact_j == 2) {
        double phi = ld(A, j, F_ORIENTATION);
        double rts = ld(A, j, F_R_TS);
        v2 e = {m_sin(phi), -m_cos(phi)};
        v2 o = {rts * e.x, rts * e.y};
        if (contact_j == 1) r_off_j = add(r_off_j, o);
        else r_off_j = sub(r_off_j, o);
    }
    v2 x_rel = sub(ld2(A, i, F_POSITION), ld2(A, j, F_POSITION));
    v2 r_off = sub(r_off_i, r_off_j);
    v2 grad;   /* gradient_three_circle :129-149 */
    grad.x = (v_rel.x - (a * (x_rel.x + 2 * r_off.x) + b_min * v_rel.x) / d_min) / a;
    grad.y = (v_rel.y - (a * (x_rel.y + 2 * r_off.y) + b_min * v_rel.y) / d_min) / a;
    double ci = (-ld(A, i, F_MASS)) * ld(A, i, F_K_SOC);
    double cj = (-ld(A, j, F_MASS)) * ld(A, j, F_K_SOC);
    double mi = magnitude(tau, ld(A, i, F_TAU_0));
    double mj = magnitude(tau, ld(A, j, F_TAU_0));
    force_i.x = 0.0 + (ci * grad.x) * mi;
    force_i.y = 0.0 + (ci * grad.y) * mi;
    force_j.x = 0.0 - (cj * grad.x) * mj;
    force_j.y = 0.0 - (cj * grad.y) * mj;
    *fi = truncate(force_i, F_SOC_MAX);
    *fj = truncate(force_j, F_SOC_MAX);
}

/* ---- core/interactions.py: pair interactions -------------------------- */

/* Outputs of one oriented pair (i, j): the force and torque each side adds. */
typedef struct { v2 fi, fj; double mi, mj; int active; } pair_out_t;

/* core/interactions.py:51-70 */
static pair_out_t pair_circular(const arr_t *A, int64_t i, int64_t j) {
    pair_out_t o;
    memset(&o, 0, sizeof o);
    v2 n;
    double h = distance_circles(ld2(A, i, F_POSITION), ld(A, i, F_RADIUS),
                                ld2(A, j, F_POSITION), ld(A, j, F_RADIUS), &n);
    if (h < SIGTH_SOC) {
        v2 fi, fj;
        force_social_circular(A, i, j, &fi, &fj);
        if (h < 0) {
            v2 t = rotate270(n);
            v2 v = sub(ld2(A, i, F_VELOCITY), ld2(A, j, F_VELOCITY));
            fi = add(fi, force_contact(h, n, v, t, ld(A, i, F_MU),
                                       ld(A, i, F_KAPPA), ld(A, i, F_DAMPING)));
            fj = sub(fj, force_contact(h, n, v, t, ld(A, j, F_MU),
                                       ld(A, j, F_KAPPA), ld(A, j, F_DAMPING)));
        }
        o.fi = fi; o.fj = fj; o.active = 1;
    }
    return o;
}

/* core/interactions.py:73-104 */
static pair_out_t pair_three_circle(const arr_t *A, int64_t i, int64_t j) {
    pair_out_t o;
    memset(&o, 0, sizeof o);
    v2 x_i[3], x_j[3];
    double r_i[3], r_j[3];
    three_parts(A, i, x_i, r_i);
    three_parts(A, j, x_j, r_j);
    v2 n, rm_i, rm_j;
    double h = distance_three_circles(x_i, r_i, x_j, r_j, &n, &rm_i, &rm_j);
    if (h < SIGTH_SOC) {
        v2 fi, fj;
        force_social_three_circle(A, i, j, &fi, &fj);
        if (h < 0) {
            v2 t = rotate270(n);
            v2 v = sub(ld2(A, i, F_VELOCITY), ld2(A, j, F_VELOCITY));
            fi = add(fi, force_contact(h, n, v, t, ld(A, i, F_MU),
                                       ld(A, i, F_KAPPA), ld(A, i, F_DAMPING)));
            fj = sub(fj, force_contact(h, n, v, t, ld(A, j, F_MU),
                                       ld(A, j, F_KAPPA), ld(A, j, F_DAMPING)));
        }
        o.fi = fi; o.fj = fj;
        o.mi = cross(rm_i, fi);
        o.mj = cross(rm_j, fj);
        o.active = 1;
    }
    return o;
}

static inline void add_force(arr_t *A, int64_t i, v2 f) {
    v2 cur = ld2(A, i, F_FORCE);
    st2(A, i, F_FORCE, add(cur, f));
}
static inline void add_torque(arr_t *A, int64_t i, double m) {
    st(A, i, F_TORQUE, ld(A, i, F_TORQUE) + m);
}

/* ---- restated cell_lists --------------------------------------------- */

typedef struct {
    double x0, y0, cell;
    int64_t nx, ny;
} grid_t;

/* Clamped cell coordinate of one axis: floor((x - x0) / cell) in [0, n-1].
 * Returns -1 for a non-finite coordinate. */
static inline int64_t axis_cell(double x, double x0, double cell, int64_t n) {
    double q = floor((x - x0) / cell);
    if (!(q == q)) return -1;
    if (q < 0.0) return 0;
    if (q > (double)(n - 1)) return n - 1;
    return (int64_t)q;
}

/* Flat cell index ix * ny + iy of every agent; -1 if its position is not
 * finite.  Returns the number of agents with a non-finite position. */
int64_t orc_cell_keys(const double *x, const double *y, int64_t n,
                      const grid_t *g, int64_t *keys) {
    int64_t bad = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t ix = axis_cell(x[i], g->x0, g->cell, g->nx);
        int64_t iy = axis_cell(y[i], g->y0, g->cell, g->ny);
        if (ix < 0 || iy < 0 || !isfinite(x[i]) || !isfinite(y[i])) {
            keys[i] = -1; ++bad;
        } else {
            keys[i] = ix * g->ny + iy;
        }
    }
    return bad;
}

/* add_to_cells restated: points_indices grouped by cell (ascending agent
 * index inside a cell), cells_count, cells_offset (exclusive prefix sum).
 * Call sites: core/interactions.py:192-194. */
int64_t orc_cell_list(const double *x, const double *y, int64_t n,
                      const grid_t *g, int64_t *keys, int64_t *points_indices,
                      int64_t *cells_count, int64_t *cells_offset) {
    int64_t ncells = g->nx * g->ny;
    int64_t bad = orc_cell_keys(x, y, n, g, keys);
    if (bad) return bad;
    memset(cells_count, 0, sizeof(int64_t) * ncells);
    for (int64_t i = 0; i < n; ++i) cells_count[keys[i]]++;
    int64_t acc = 0;
    for (int64_t c = 0; c < ncells; ++c) { cells_offset[c] = acc; acc += cells_count[c]; }
    int64_t *fill = (int64_t *)calloc((size_t)ncells, sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = keys[i];
        points_indices[cells_offset[c] + fill[c]++] = i;
    }
    free(fill);
    return 0;
}

/* Forward half of the 3x3 stencil (neighboring_cells restated): offsets in
 * (dx, dy) whose flat offset dx*ny + dy is positive, in ascending flat order. */
static const int FWD_DX[4] = {0, 1, 1, 1};
static const int FWD_DY[4] = {1, -1, 0, 1};

typedef void (*pair_fn)(void *ctx, int64_t i, int64_t j);

/* iter_nearest_neighbors restated (call sites core/interactions.py:152-165):
 * for each cell c ascending, for each agent a of c in order: pairs (a, b)
 * with b later in c, then (a, b) for b in each forward neighbour cell. */
static void iter_pairs(const grid_t *g, const int64_t *pidx, const int64_t *cnt,
                       const int64_t *off, pair_fn fn, void *ctx) {
    for (int64_t ix = 0; ix < g->nx; ++ix)
        for (int64_t iy = 0; iy < g->ny; ++iy) {
            int64_t c = ix * g->ny + iy;
            for (int64_t s = 0; s < cnt[c]; ++s) {
                int64_t a = pidx[off[c] + s];
                for (int64_t t = s + 1; t < cnt[c]; ++t) fn(ctx, a, pidx[off[c] + t]);
                for (int k = 0; k < 4; ++k) {
                    int64_t jx = ix + FWD_DX[k], jy = iy + FWD_DY[k];
                    if (jx < 0 || jx >= g->nx || jy < 0 || jy >= g->ny) continue;
                    int64_t c2 = jx * g->ny + jy;
                    for (int64_t t = 0; t < cnt[c2]; ++t) fn(ctx, a, pidx[off[c2] + t]);
                }
            }
        }
}

typedef struct { int64_t *out; int64_t k, cap; } pair_rec_t;
static void rec_pair(void *ctx, int64_t i, int64_t j) {
    pair_rec_t *r = (pair_rec_t *)ctx;
    if (r->k < r->cap) { r->out[2 * r->k] = i; r->out[2 * r->k + 1] = j; }
    r->k++;
}

/* Candidate pairs in visiting order, as (i, j) rows.  Returns the total
 * number of pairs (rows beyond `cap` are counted but not written), or -1 if
 * some position is not finite. */
int64_t orc_candidate_pairs(const double *x, const double *y, int64_t n,
                            const grid_t *g, int64_t *pairs, int64_t cap) {
    int64_t ncells = g->nx * g->ny;
    int64_t *keys = malloc(sizeof(int64_t) * (n ? n : 1));
    int64_t *pidx = malloc(sizeof(int64_t) * (n ? n : 1));
    int64_t *cnt = malloc(sizeof(int64_t) * ncells);
    int64_t *off = malloc(sizeof(int64_t) * ncells);
    int64_t res = -1;
    if (orc_cell_list(x, y, n, g, keys, pidx, cnt, off) == 0) {
        pair_rec_t r = {pairs, 0, cap};
        iter_pairs(g, pidx, cnt, off, rec_pair, &r);
        res = r.k;
    }
    free(keys); free(pidx); free(cnt); free(off);
    return res;
}

typedef struct { arr_t *A; int body; } aa_ctx_t;

static void aa_pair(void *vctx, int64_t i, int64_t j) {
    aa_ctx_t *c = (aa_ctx_t *)vctx;
    if (c->body == BODY_CIRCULAR) {
        pair_out_t o = pair_circular(c->A, i, j);
        if (o.active) { add_force(c->A, i, o.fi); add_force(c->A, j, o.fj); }
    } else {
        pair_out_t o = pair_three_circle(c->A, i, j);
        if (o.active) {
            add_force(c->A, i, o.fi); add_force(c->A, j, o.fj);
            add_torque(c->A, i, o.mi); add_torque(c->A, j, o.mj);
        }
    }
}

static void positions_soa(const arr_t *A, int64_t n, double *x, double *y) {
    for (int64_t i = 0; i < n; ++i) {
        v2 p = ld2(A, i, F_POSITION);
        x[i] = p.x; y[i] = p.y;
    }
}

/* agent_agent_block_list (core/interactions.py:191-205) over the restated
 * cell list, serial, in the reference's visiting order.  nthreads > 1 runs
 * the same pairs agent-parallel: every agent sums the pairs it belongs to,
 * each evaluated in its (owner, other) orientation, visiting the 3 x 3
 * neighbourhood in (dx, dy) lexicographic order and each cell in ascending
 * agent order.  That is exactly the order in which the serial visit adds
 * pair contributions to any one agent (the backward half-stencil cells have
 * smaller flat indices, the forward half larger), so both variants give
 * bit-identical forces.  Returns 0, or -1 for a non-finite position. */
int orc_agent_agent(char *base, int64_t n, int64_t itemsize, const int64_t *off,
                    int body, const grid_t *g, int nthreads) {
    arr_t A = {base, itemsize, off};
    int64_t ncells = g->nx * g->ny;
    double *x = malloc(sizeof(double) * (n ? n : 1));
    double *y = malloc(sizeof(double) * (n ? n : 1));
    int64_t *keys = malloc(sizeof(int64_t) * (n ? n : 1));
    int64_t *pidx = malloc(sizeof(int64_t) * (n ? n : 1));
    int64_t *cnt = malloc(sizeof(int64_t) * ncells);
    int64_t *cof = malloc(sizeof(int64_t) * ncells);
    positions_soa(&A, n, x, y);
    int rc = 0;
    if (orc_cell_list(x, y, n, g, keys, pidx, cnt, cof) != 0) {
        rc = -1;
    } else if (nthreads <= 1) {
        aa_ctx_t ctx = {&A, body};
        iter_pairs(g, pidx, cnt, cof, aa_pair, &ctx);
    } else {
        /* rank of each agent inside its cell */
        int64_t *rank = malloc(sizeof(int64_t) * (n ? n : 1));
        for (int64_t c = 0; c < ncells; ++c)
            for (int64_t s = 0; s < cnt[c]; ++s) rank[pidx[cof[c] + s]] = s;
        double *acc = calloc((size_t)(n ? n : 1) * 3, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
#endif
        for (int64_t a = 0; a < n; ++a) {
            int64_t c = keys[a], ix = c / g->ny, iy = c % g->ny;
            /* start from the agent's current force so the running sum has
             * the serial visiting order's association */
            v2 f0 = ld2(&A, a, F_FORCE);
            double fx = f0.x, fy = f0.y;
            double m = body == BODY_THREE_CIRCLE ? ld(&A, a, F_TORQUE) : 0.0;
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy) {
                    int64_t jx = ix + dx, jy = iy + dy;
                    if (jx < 0 || jx >= g->nx || jy < 0 || jy >= g->ny) continue;
                    int64_t c2 = jx * g->ny + jy;
                    int64_t flat = (int64_t)dx * g->ny + dy;  /* sign gives orientation */
                    for (int64_t t = 0; t < cnt[c2]; ++t) {
                        int64_t b = pidx[cof[c2] + t];
                        if (b == a) continue;
                        int owner = (c2 == c) ? (rank[a] < t) : (flat > 0);
                        /* neighbour offsets with flat < 0 make b the owner */
                        pair_out_t o = owner ?
                            (body == BODY_CIRCULAR ? pair_circular(&A, a, b) : pair_three_circle(&A, a, b)) :
                            (body == BODY_CIRCULAR ? pair_circular(&A, b, a) : pair_three_circle(&A, b, a));
                        if (!o.active) continue;
                        if (owner) { fx += o.fi.x; fy += o.fi.y; m += o.mi; }
                        else { fx += o.fj.x; fy += o.fj.y; m += o.mj; }
                    }
                }
            acc[3 * a] = fx; acc[3 * a + 1] = fy; acc[3 * a + 2] = m;
        }
        for (int64_t a = 0; a < n; ++a) {
            v2 f = {acc[3 * a], acc[3 * a + 1]};
            st2(&A, a, F_FORCE, f);
            if (body == BODY_THREE_CIRCLE) st(&A, a, F_TORQUE, acc[3 * a + 2]);
        }
        free(acc); free(rank);
    }
    free(x); free(y); free(keys); free(pidx); free(cnt); free(cof);
    return rc;
}

/* agent_obstacle (core/interactions.py:107-141,169-186,208-214): every agent
 * against every wall, walls in index order.  walls = W rows of (p0x, p0y,
 * p1x, p1y). */
void orc_agent_obstacle(char *base, int64_t n, int64_t itemsize, const int64_t *off,
                        int body, const double *walls, int64_t nw, int nthreads) {
    arr_t A = {base, itemsize, off};
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 1 ? nthreads : 1)
#endif
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t w = 0; w < nw; ++w) {
            v2 p0 = {walls[4 * w], walls[4 * w + 1]};
            v2 p1 = {walls[4 * w + 2], walls[4 * w + 3]};
            if (body == BODY_CIRCULAR) {
                v2 n;
                double h = distance_circle_line(ld2(&A, i, F_POSITION), ld(&A, i, F_RADIUS), p0, p1, &n);
                if (h < 0) {
                    v2 t = rotate270(n);
                    v2 v = ld2(&A, i, F_VELOCITY);
                    add_force(&A, i, force_contact(h, n, v, t, ld(&A, i, F_MU),
                                                   ld(&A, i, F_KAPPA), ld(&A, i, F_DAMPING)));
                }
            } else {
                v2 x[3], n, rm;
                double r[3];
                three_parts(&A, i, x, r);
                double h = distance_three_circle_line(x, r, p0, p1, &n, &rm);
                if (h < 0) {
                    v2 t = rotate270(n);
                    v2 v = ld2(&A, i, F_VELOCITY);
                    v2 f = force_contact(h, n, v, t, ld(&A, i, F_MU),
                                         ld(&A, i, F_KAPPA), ld(&A, i, F_DAMPING));
                    add_force(&A, i, f);
                    add_torque(&A, i, cross(rm, f));
                }
            }
        }
    }
}

/* ---- core/motion/adjusting.py ----------------------------------------- */

/* force_adjust_agents :98-108 with force_adjust :16-51 */
void orc_force_adjust_agents(char *base, int64_t n, int64_t itemsize, const int64_t *off) {
    arr_t A = {base, itemsize, off};
    for (int64_t i = 0; i < n; ++i) {
        double k = ld(&A, i, F_MASS) / ld(&A, i, F_TAU_ADJ);
        double v0 = ld(&A, i, F_TARGET_VELOCITY);
        v2 e0 = ld2(&A, i, F_TARGET_DIRECTION), v = ld2(&A, i, F_VELOCITY);
        v2 f = {k * (v0 * e0.x - v.x), k * (v0 * e0.y - v.y)};
        add_force(&A, i, f);
    }
}

/* torque_adjust_agents :111-121 with torque_adjust :54-95 */
void orc_torque_adjust_agents(char *base, int64_t n, int64_t itemsize, const int64_t *off) {
    arr_t A = {base, itemsize, off};
    for (int64_t i = 0; i < n; ++i) {
        double m = ld(&A, i, F_INERTIA_ROT) / ld(&A, i, F_TAU_ROT) *
                   (orc_wrap_to_pi(ld(&A, i, F_TARGET_ORIENTATION) - ld(&A, i, F_ORIENTATION)) / PI *
                    ld(&A, i, F_TARGET_ANGULAR_VELOCITY) - ld(&A, i, F_ANGULAR_VELOCITY));
        add_torque(&A, i, m);
    }
}

/* core/steering/orientation.py:17-21 with vector2D.angle :85-96 */
void orc_orient_towards_target_direction(char *base, int64_t n, int64_t itemsize,
                                         const int64_t *off) {
    arr_t A = {base, itemsize, off};
    for (int64_t i = 0; i < n; ++i) {
        v2 e = ld2(&A, i, F_TARGET_DIRECTION);
        st(&A, i, F_TARGET_ORIENTATION, m_atan2(e.y, e.x));
    }
}

/* ---- core/integrator.py ----------------------------------------------- */

/* adaptive_timestep :29-97 */
double orc_adaptive_timestep(char *base, int64_t n, int64_t itemsize, const int64_t *off,
                             double dt_min, double dt_max) {
    arr_t A = {base, itemsize, off};
    double v_max = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double l = length(ld2(&A, i, F_VELOCITY));
        if (l > v_max) v_max = l;
    }
    if (v_max == 0.0) return dt_max;
    double c = 1.1;
    /* np.max propagates NaN */
    double v0max = -INFINITY;
    for (int64_t i = 0; i < n; ++i) {
        double v0 = ld(&A, i, F_TARGET_VELOCITY);
        if (isnan(v0) || isnan(v0max)) v0max = NAN;
        else if (v0 > v0max) v0max = v0;
    }
    double dx_max = c * v0max * dt_max;
    double dt = dx_max / v_max;
    if (dt > dt_max) return dt_max;
    else if (dt < dt_min) return dt_min;
    else return dt;
}

/* translational_verlet :164-176 (velocity first, then position with the
 * updated velocity) */
static void translational_verlet(arr_t *A, int64_t n, double dt) {
    for (int64_t i = 0; i < n; ++i) {
        double m = ld(A, i, F_MASS);
        v2 fp = ld2(A, i, F_FORCE_PREV), f = ld2(A, i, F_FORCE);
        v2 oa = divs(fp, m), na = divs(f, m);
        st2(A, i, F_FORCE_PREV, f);
        v2 v = ld2(A, i, F_VELOCITY);
        v.x = v.x + (oa.x + na.x) / 2 * dt;
        v.y = v.y + (oa.y + na.y) / 2 * dt;
        st2(A, i, F_VELOCITY, v);
        v2 x = ld2(A, i, F_POSITION);
        x.x = x.x + (v.x * dt + na.x / 2 * (dt * dt));
        x.y = x.y + (v.y * dt + na.y / 2 * (dt * dt));
        st2(A, i, F_POSITION, x);
    }
}

/* rotational_verlet :179-193 */
static void rotational_verlet(arr_t *A, int64_t n, double dt) {
    for (int64_t i = 0; i < n; ++i) {
        double I = ld(A, i, F_INERTIA_ROT);
        double oa = ld(A, i, F_TORQUE_PREV) / I, na = ld(A, i, F_TORQUE) / I;
        st(A, i, F_TORQUE_PREV, ld(A, i, F_TORQUE));
        double w = ld(A, i, F_ANGULAR_VELOCITY) + (oa + na) / 2 * dt;
        st(A, i, F_ANGULAR_VELOCITY, w);
        double phi = ld(A, i, F_ORIENTATION) + (w * dt + na / 2 * (dt * dt));
        st(A, i, F_ORIENTATION, orc_wrap_to_pi(phi));
    }
}

/* shoulders, simulation/agents.py:473-486 */
void orc_shoulders(char *base, int64_t n, int64_t itemsize, const int64_t *off) {
    arr_t A = {base, itemsize, off};
    for (int64_t i = 0; i < n; ++i) {
        double phi = ld(&A, i, F_ORIENTATION), rts = ld(&A, i, F_R_TS);
        v2 tangent = rotate270((v2){m_cos(phi), m_sin(phi)});
        v2 offset = {tangent.x * rts, tangent.y * rts};
        v2 x = ld2(&A, i, F_POSITION);
        st2(&A, i, F_POSITION_LS, sub(x, offset));
        st2(&A, i, F_POSITION_RS, add(x, offset));
    }
}

/* velocity_verlet_integrator :209-256 */
double orc_velocity_verlet(char *base, int64_t n, int64_t itemsize, const int64_t *off,
                           int body, double dt_min, double dt_max) {
    arr_t A = {base, itemsize, off};
    double dt = orc_adaptive_timestep(base, n, itemsize, off, dt_min, dt_max);
    translational_verlet(&A, n, dt);
    if (body == BODY_THREE_CIRCLE) {
        rotational_verlet(&A, n, dt);
        orc_shoulders(base, n, itemsize, off);
    }
    return dt;
}

/* Reset.update, simulation/logic.py:59-64 */
void orc_reset(char *base, int64_t n, int64_t itemsize, const int64_t *off, int body) {
    arr_t A = {base, itemsize, off};
    v2 z = {0.0, 0.0};
    for (int64_t i = 0; i < n; ++i) {
        st2(&A, i, F_FORCE, z);
        if (body == BODY_THREE_CIRCLE) st(&A, i, F_TORQUE, 0.0);
    }
}

/* Fluctuation.update (simulation/logic.py:78-86) with host-drawn noise:
 * force += noise_f[i], torque += noise_m[i]. */
void orc_add_noise(char *base, int64_t n, int64_t itemsize, const int64_t *off, int body,
                   const double *noise_f, const double *noise_m) {
    arr_t A = {base, itemsize, off};
    for (int64_t i = 0; i < n; ++i) {
        if (noise_f) { v2 f = {noise_f[2 * i], noise_f[2 * i + 1]}; add_force(&A, i, f); }
        if (noise_m && body == BODY_THREE_CIRCLE) add_torque(&A, i, noise_m[i]);
    }
}

/* Direction maps for Navigation: n_targets maps of ny x nx (row = y) on the
 * meshgrid (minx, miny, step); set before orc_step, used while it runs. */
static struct {
    int64_t n_targets, ny, nx;
    double minx, miny, step;
    const double *dx, *dy;
} g_nav;

void orc_set_navigation(int64_t n_targets, const double *dx, const double *dy, int64_t ny,
                        int64_t nx, double minx, double miny, double step) {
    g_nav.n_targets = n_targets;
    g_nav.dx = dx;
    g_nav.dy = dy;
    g_nav.ny = ny;
    g_nav.nx = nx;
    g_nav.minx = minx;
    g_nav.miny = miny;
    g_nav.step = step;
}

/* Navigation.update (simulation/logic.py:152-165): for every target t, the
 * agents with target == t take getdefault(indices, dir_map_t, e0)
 * (core/steering/navigation.py:69-78) with indices the meshgrid indicer
 * ((position - (minx, miny)) / step).astype(int64) (core/steering/
 * quickest_path.py:40-43) flipped to (row = y, column = x); is_inside
 * (navigation.py:60-64) keeps e0 outside the map.  astype(int64) truncates
 * toward zero; non-finite quotients leave e0 unchanged (numpy on x86 maps
 * them to INT64_MIN, outside every map). */
void orc_navigation(char *base, int64_t n, int64_t itemsize, const int64_t *off) {
    arr_t A = {base, itemsize, off};
    if (off[F_TARGET] < 0) return;
    for (int64_t i = 0; i < n; ++i) {
        int64_t t;
        memcpy(&t, base + i * itemsize + off[F_TARGET], sizeof t);
        if (t < 0 || t >= g_nav.n_targets) continue;
        v2 p = ld2(&A, i, F_POSITION);
        double qx = (p.x - g_nav.minx) / g_nav.step;
        double qy = (p.y - g_nav.miny) / g_nav.step;
        double tx = trunc(qx), ty = trunc(qy);
        if (!(tx >= 0.0 && tx < (double)g_nav.nx && ty >= 0.0 && ty < (double)g_nav.ny)) continue;
        int64_t k = (t * g_nav.ny + (int64_t)ty) * g_nav.nx + (int64_t)tx;
        v2 e = {g_nav.dx[k], g_nav.dy[k]};
        st2(&A, i, F_TARGET_DIRECTION, e);
    }
}

/* Philox4x32-10 of cd_noise.h, exported for known-answer tests. */
void orc_philox4x32_10(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
    cdn_philox4x32_10(ctr, key, out);
}

/* The device's fluctuation noise of step `step` (cd_noise.h): force (n x 2)
 * and, for ThreeCircle, torque (n), from mass, std_rand_force, inertia_rot
 * and std_rand_torque (core/motion/fluctuation.py:14-62). */
void orc_device_noise(const char *base, int64_t n, int64_t itemsize, const int64_t *off, int body,
                      uint64_t seed, uint64_t step, double *force, double *torque) {
    arr_t A = {(char *)base, itemsize, off};
    const int three = body == BODY_THREE_CIRCLE;
    for (int64_t i = 0; i < n; ++i) {
        double fx, fy, tq;
        cdn_fluctuation(seed, step, (uint32_t)i, ld(&A, i, F_MASS), ld(&A, i, F_STD_RAND_FORCE),
                        three ? ld(&A, i, F_INERTIA_ROT) : 0.0,
                        three ? ld(&A, i, F_STD_RAND_TORQUE) : 0.0, three, &fx, &fy, &tq);
        force[2 * i] = fx;
        force[2 * i + 1] = fy;
        if (torque) torque[i] = tq;
    }
}

/* One MultiAgentSimulation.update() (simulation/multiagent.py:51-55) for the
 * standard tree Reset << Integrator << (Fluctuation, Adjusting << Orientation,
 * AgentAgentInteractions, AgentObstacleInteractions), post-order.  `flags`
 * selects nodes (ORC_*).  Returns dt (0 when the integrator is not run) or
 * NAN if the cell list saw a non-finite position. */
double orc_step(char *base, int64_t n, int64_t itemsize, const int64_t *off, int body,
                int flags, const grid_t *g, const double *walls, int64_t nw,
                const double *noise_f, const double *noise_m,
                double dt_min, double dt_max, int nthreads) {
    double dt = 0.0;
    if (flags & ORC_NAVIGATION) orc_navigation(base, n, itemsize, off);
    if (flags & ORC_FLUCTUATION) orc_add_noise(base, n, itemsize, off, body, noise_f, noise_m);
    if ((flags & ORC_ORIENTATION) && body == BODY_THREE_CIRCLE)
        orc_orient_towards_target_direction(base, n, itemsize, off);
    if (flags & ORC_ADJUSTING) {
        orc_force_adjust_agents(base, n, itemsize, off);
        if (body == BODY_THREE_CIRCLE) orc_torque_adjust_agents(base, n, itemsize, off);
    }
    if (flags & ORC_AGENT_AGENT)
        if (orc_agent_agent(base, n, itemsize, off, body, g, nthreads) != 0) return NAN;
    if (flags & ORC_AGENT_OBSTACLE)
        orc_agent_obstacle(base, n, itemsize, off, body, walls, nw, nthreads);
    if (flags & ORC_INTEGRATE)
        dt = orc_velocity_verlet(base, n, itemsize, off, body, dt_min, dt_max);
    if (flags & ORC_RESET) orc_reset(base, n, itemsize, off, body);
    return dt;
}

/* The shared elementary functions, exported for accuracy tests:
 * which = 0 hypot(a, b), 1 exp(a), 2 sin(a), 3 cos(a), 4 atan2(a, b). */
double orc_cdm(int which, double a, double b) {
    switch (which) {
    case 0: return cdm_hypot(a, b);
    case 1: return cdm_exp(a);
    case 2: return cdm_sin(a);
    case 3: return cdm_cos(a);
    case 4: return cdm_atan2(a, b);
    case 5: return cdm_log(a);
    default: return NAN;
    }
}

/* ---- the same pair sums evaluated in each agent's own frame -------------
 * Test support for the device kernel's formulation: every agent evaluates
 * each of its pairs with relative quantities (me - other), visiting the 3 x 3
 * sub-circle pairs in the owner-first order.  Must equal orc_agent_agent bit
 * for bit (ThreeCircle only). */
static void tc_pair_me(const arr_t *A, int64_t me, int64_t ot, int me_first,
                       double *fx, double *fy, double *tq) {
    v2 xm[3], xo[3];
    double rm[3], ro[3];
    three_parts(A, me, xm, rm);
    three_parts(A, ot, xo, ro);
    double h_min = NAN, sdx = 0, sdy = 0, sd = 0;
    int mine_min = 0;
    for (int k = 0; k < 9; ++k) {
        int p = k / 3, q = k % 3, mi = me_first ? p : q, ti = me_first ? q : p;
        double dx = xm[mi].x - xo[ti].x, dy = xm[mi].y - xo[ti].y;
        double d = m_hypot(dx, dy);
        double h = d - (rm[mi] + ro[ti]);
        if (h < h_min || isnan(h_min)) { h_min = h; sdx = dx; sdy = dy; sd = d; mine_min = mi; }
    }
    if (!(h_min < SIGTH_SOC)) return;
    double nx = 0, ny = 0;
    if (sd != 0) { nx = sdx / sd; ny = sdy / sd; }
    v2 xs = me_first ? xm[mine_min] : xo[mine_min];
    double rmx = (xs.x + rm[mine_min] * nx) - xm[0].x;
    double rmy = (xs.y + rm[mine_min] * ny) - xm[0].y;
    v2 vm = ld2(A, me, F_VELOCITY), vo = ld2(A, ot, F_VELOCITY);
    double vrx = vm.x - vo.x, vry = vm.y - vo.y;
    double a = vrx * vrx + vry * vry;
    double Fx = 0, Fy = 0;
    if (a != 0) {
        double tau = NAN, b_min = 0, d_min = 0;
        int k_sel = 0;
        for (int k = 0; k < 9; ++k) {
            int p = k / 3, q = k % 3, mi = me_first ? p : q, ti = me_first ? q : p;
            double xr = xm[mi].x - xo[ti].x, yr = xm[mi].y - xo[ti].y;
            double r_tot = rm[mi] + ro[ti];
            double b = -(xr * vrx + yr * vry);
            double c = (xr * xr + yr * yr) - r_tot * r_tot;
            double d = sqrt(b * b - a * c);
            if (isnan(d) || d == 0) continue;
            double tau_new = (b - d) / a;
            if (isnan(tau) || (0 < tau_new && tau_new < tau)) { k_sel = k; tau = tau_new; b_min = b; d_min = d; }
        }
        if (!(isnan(tau) || tau <= 0)) {
            int p = k_sel / 3, q = k_sel % 3, mi = me_first ? p : q, ti = me_first ? q : p;
            double o[2][2];
            int parts[2] = {mi, ti};
            int64_t who[2] = {me, ot};
            for (int u = 0; u < 2; ++u) {
                double phi = ld(A, who[u], F_ORIENTATION), rts = ld(A, who[u], F_R_TS);
                double ex = rts * m_sin(phi), ey = rts * (-m_cos(phi));
                o[u][0] = parts[u] == 1 ? (0.0 + ex) : (parts[u] == 2 ? (0.0 - ex) : 0.0);
                o[u][1] = parts[u] == 1 ? (0.0 + ey) : (parts[u] == 2 ? (0.0 - ey) : 0.0);
            }
            double ox = o[0][0] - o[1][0], oy = o[0][1] - o[1][1];
            double xr = xm[0].x - xo[0].x, yr = xm[0].y - xo[0].y;
            double gx = (vrx - (a * (xr + 2 * ox) + b_min * vrx) / d_min) / a;
            double gy = (vry - (a * (yr + 2 * oy) + b_min * vry) / d_min) / a;
            double cm = (-ld(A, me, F_MASS)) * ld(A, me, F_K_SOC);
            double mag = magnitude(tau, ld(A, me, F_TAU_0));
            v2 F = {(cm * gx) * mag, (cm * gy) * mag};
            F = truncate(F, F_SOC_MAX);
            Fx = F.x; Fy = F.y;
        }
    }
    if (h_min < 0) {
        v2 n = {nx, ny}, v = {vrx, vry};
        v2 c = force_contact(h_min, n, v, rotate270(n), ld(A, me, F_MU), ld(A, me, F_KAPPA), ld(A, me, F_DAMPING));
        Fx = Fx + c.x; Fy = Fy + c.y;
    }
    *fx += Fx; *fy += Fy;
    *tq += rmx * Fy - rmy * Fx;
}

int orc_agent_agent_me_frame(char *base, int64_t n, int64_t itemsize, const int64_t *off,
                             const grid_t *g) {
    arr_t A = {base, itemsize, off};
    int64_t ncells = g->nx * g->ny;
    double *x = malloc(sizeof(double) * (n ? n : 1)), *y = malloc(sizeof(double) * (n ? n : 1));
    int64_t *keys = malloc(sizeof(int64_t) * (n ? n : 1)), *pidx = malloc(sizeof(int64_t) * (n ? n : 1));
    int64_t *cnt = malloc(sizeof(int64_t) * ncells), *cof = malloc(sizeof(int64_t) * ncells);
    int64_t *rank = malloc(sizeof(int64_t) * (n ? n : 1));
    double *acc = calloc((size_t)(n ? n : 1) * 3, sizeof(double));
    positions_soa(&A, n, x, y);
    int rc = orc_cell_list(x, y, n, g, keys, pidx, cnt, cof) ? -1 : 0;
    if (!rc) {
        for (int64_t c = 0; c < ncells; ++c)
            for (int64_t s = 0; s < cnt[c]; ++s) rank[pidx[cof[c] + s]] = s;
        for (int64_t a = 0; a < n; ++a) {
            int64_t c = keys[a], ix = c / g->ny, iy = c % g->ny;
            v2 f0 = ld2(&A, a, F_FORCE);
            double fx = f0.x, fy = f0.y, m = ld(&A, a, F_TORQUE);
            for (int dx = -1; dx <= 1; ++dx)
                for (int dy = -1; dy <= 1; ++dy) {
                    int64_t jx = ix + dx, jy = iy + dy;
                    if (jx < 0 || jx >= g->nx || jy < 0 || jy >= g->ny) continue;
                    int64_t c2 = jx * g->ny + jy;
                    for (int64_t t = 0; t < cnt[c2]; ++t) {
                        int64_t b = pidx[cof[c2] + t];
                        if (b == a) continue;
                        int first = (c2 == c) ? (rank[a] < t) : ((int64_t)dx * g->ny + dy > 0);
                        tc_pair_me(&A, a, b, first, &fx, &fy, &m);
                    }
                }
            acc[3 * a] = fx; acc[3 * a + 1] = fy; acc[3 * a + 2] = m;
        }
        for (int64_t a = 0; a < n; ++a) {
            v2 f = {acc[3 * a], acc[3 * a + 1]};
            st2(&A, a, F_FORCE, f);
            st(&A, a, F_TORQUE, acc[3 * a + 2]);
        }
    }
    free(x); free(y); free(keys); free(pidx); free(cnt); free(cof); free(rank); free(acc);
    return rc;
}
