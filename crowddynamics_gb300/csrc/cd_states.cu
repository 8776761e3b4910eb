// cd_states.cu -- the per-step state nodes around the force step:
// InsideDomain and TargetReached (simulation/logic.py:343-387) and the
// leader-follower nodes with and without herding (simulation/logic.py:168-217,
// core/steering/collective_motion.py:15-279).
//
// Herding follows the reference's sequence exactly:
//  * nearest unobstructed neighbours (find_nearest_neighbors, :71-104): the
//    reference visits every unordered pair of the cell list once (cell size =
//    the follower sight) and offers the pair to both agents, each keeping its
//    size_nearest_other closest in an array whose largest entry (first
//    arg-max) is replaced.  An agent's array changes only through its own
//    offers, which it receives in its visiting order (3 x 3 cells in (dx, dy)
//    order, ascending within a cell), so one thread per agent replays them in
//    that order.  The line-of-sight test (is_obstacle_between_points over all
//    walls, with the pair's own orientation) only matters when the distance
//    would enter the array, and is only evaluated then;
//  * herding_interaction (:107-155), leader_follower_interaction_brute
//    (:158-218; leaders in increasing distance, ties by index) and the
//    combination of leader_follower[_with_herding]_interaction (:221-279),
//    one thread per follower.
// Leaders are assumed not to be followers themselves (a follower reads the
// target of the leader it follows as it was before the update).
#include <cstdint>
#include <cmath>
#include "cd_internal.cuh"
#include "cd_math.h"

namespace cdk {
namespace {

constexpr int HNT = 128;
constexpr int KMAX = 16;

__device__ __forceinline__ void normalize(double &x, double &y) {
    const double l = cdm_hypot(x, y);
    if (l != 0.0) {                              // `v / l if l else v`
        x = x / l;
        y = y / l;
    }
}

// geom2D.line_intersect (core/geom2D.py:36-59)
__device__ __forceinline__ bool line_intersect(double x0x, double x0y, double x1x, double x1y,
                                               double y0x, double y0y, double y1x, double y1y) {
    const double ux = x1x - x0x, uy = x1y - x0y;
    const double vx = y1x - y0x, vy = y1y - y0y;
    const double bx = y0x - x0x, by = y0y - x0y;
    const double d = ux * vy - uy * vx;
    if (d == 0) return false;
    const double t0 = bx * vy - by * vx;
    const double t1 = bx * uy - by * ux;
    const double s0 = t0 / d, s1 = t1 / d;
    return 0 <= s0 && s0 <= 1 && 0 <= s1 && s1 <= 1;
}

// sensory_region.is_obstacle_between_points (core/sensory_region.py:9-16)
// over a warp: lanes take the walls in turn (the result does not depend on
// the order).  Called by all 32 lanes with the same arguments.
__device__ __forceinline__ bool blocked_warp(const HerdArgs &h, const ScenDev &sc, double ax,
                                             double ay, double bx, double by, int lane) {
    bool hit = false;
    for (int w = sc.wall_begin + lane; w < sc.wall_begin + sc.wall_count && !hit; w += 32) {
        const double *p = h.walls + (size_t)w * WALL_D;
        hit = line_intersect(ax, ay, bx, by, p[0], p[1], p[2], p[3]);
    }
    return __any_sync(0xffffffffu, hit);
}

// herding_relationship (collective_motion.py:24-57): first element.
__device__ __forceinline__ bool heading_away(const HerdArgs &h, double x1x, double x1y,
                                             double x2x, double x2y, double v1x, double v1y,
                                             double v2x, double v2y) {
    if (cdm_hypot(v1x, v1y) == 0 || cdm_hypot(v2x, v2y) == 0) return false;
    double ex = x2x - x1x, ey = x2y - x1y;
    normalize(ex, ey);
    double n1x = v1x, n1y = v1y, n2x = v2x, n2y = v2y;
    normalize(n1x, n1y);
    normalize(n2x, n2y);
    const double c_i = ex * n1x + ey * n1y;
    const double c_j = -(ex * n2x + ey * n2y);
    const double cp = h.cos_phi;
    (void)c_i;                 // both branches on c_i give the same first element:
    return !(cp < c_j && c_j < 1.0);           // the other is not heading towards us
}

// One warp per agent: the lanes measure 32 candidates at a time; those
// closer than the agent's current farthest kept neighbour (which only
// shrinks) are offered in slot order with all lanes carrying the same array.
__global__ void __launch_bounds__(HNT) k_herd_neighbors(HerdArgs h) {
    const int s = (int)(((long long)blockIdx.x * HNT + threadIdx.x) / 32);
    const int lane = threadIdx.x & 31;
    if (s >= h.n) return;                                // whole warps leave together
    const int i = h.perm[s];
    const ScenDev sc = h.scen_h[h.scen_of[i]];
    const double *const *col = h.col;
    const double xi = col[X][i], yi = col[Y][i];
    int nb[KMAX];
    double dist[KMAX];
    const int K = h.K;
#pragma unroll
    for (int k = 0; k < KMAX; ++k) { nb[k] = -1; dist[k] = h.sight_f; }
    double dmax = h.sight_f;
    const int local = h.key[i] - sc.cell_base;
    const int ix = local / sc.ny, iy = local - ix * sc.ny;
    for (int ck = 0; ck < 9; ++ck) {
        const int jx = ix + ck / 3 - 1, jy = iy + ck % 3 - 1;
        if (jx < 0 || jx >= sc.nx || jy < 0 || jy >= sc.ny) continue;
        const int c2 = sc.cell_base + jx * sc.ny + jy;
        const int b = h.start[c2], e = h.start[c2 + 1];
        for (int base = b; base < e; base += 32) {
            const int t = base + lane;
            int j = -1;
            double l = INFINITY;
            if (t < e && t != s) {
                j = h.perm[t];
                l = cdm_hypot(xi - col[X][j], yi - col[Y][j]);
            }
            unsigned m = __ballot_sync(0xffffffffu, l < dmax);
            while (m) {
                const int k = __ffs(m) - 1;
                m &= m - 1;
                const double lk = __shfl_sync(0xffffffffu, l, k);
                const int jk = __shfl_sync(0xffffffffu, j, k);
                if (!(lk < dmax)) continue;
                const double xj = col[X][jk], yj = col[Y][jk];
                // the pair's first agent is the lower slot
                const bool first = s < base + k;
                if (first ? blocked_warp(h, sc, xi, yi, xj, yj, lane)
                          : blocked_warp(h, sc, xj, yj, xi, yi, lane))
                    continue;
                int am = 0;                                  // set_neighbor: first arg-max
#pragma unroll
                for (int q = 1; q < KMAX; ++q)
                    if (q < K && dist[q] > dist[am]) am = q;
#pragma unroll
                for (int q = 0; q < KMAX; ++q)
                    if (q == am) { nb[q] = jk; dist[q] = lk; }
                dmax = dist[0];
#pragma unroll
                for (int q = 1; q < KMAX; ++q)
                    if (q < K) dmax = dist[q] > dmax ? dist[q] : dmax;
            }
        }
    }
    if (lane < K) {
#pragma unroll
        for (int q = 0; q < KMAX; ++q)
            if (q == lane) h.nbr[(size_t)i * K + q] = nb[q];
    }
}

// The reference's follower loop reads the targets of leaders it may already
// have updated as followers (core/steering/collective_motion.py:186-216);
// the device reads the targets from before the update, so both roles at
// once are rejected before any state is written.
__global__ void k_check_roles(StateCols st, int n, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && st.leader[i] && st.follower[i]) atomicOr(err, ERR_LEADER_FOLLOWER);
}

__global__ void k_leader_flags(HerdArgs h, int *flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < h.n) flags[i] = h.st.leader[i] ? 1 : 0;
}

__global__ void k_leader_list(HerdArgs h, const int *pos, int *list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < h.n && h.st.leader[i]) list[pos[i]] = i;
}

__global__ void k_target_snapshot(HerdArgs h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < h.n) h.tgt_before[i] = h.st.target[i];
}

// One warp per follower: every lane carries the same values (control flow is
// uniform), the lanes share the scan for the next-nearest leader, lane 0
// writes.
__global__ void __launch_bounds__(HNT) k_herd_follow(HerdArgs h) {
    const int i = (int)(((long long)blockIdx.x * HNT + threadIdx.x) / 32);
    const int lane = threadIdx.x & 31;
    if (i >= h.n || !h.st.follower[i]) return;          // whole warps leave together
    double *const *col = h.col;
    const int sid = h.scen_of[i];
    const ScenDev sc = h.scen_h[sid];
    const double xi = col[X][i], yi = col[Y][i], vxi = col[VX][i], vyi = col[VY][i];
    // herding_interaction: average of the neighbours heading away
    double dhx = 0.0, dhy = 0.0;
    bool has_dir = false;
    if (h.with_herding) {
        double mpx = 0.0, mpy = 0.0, mvx = 0.0, mvy = 0.0;
        int num = 0;
        for (int k = 0; k < h.K; ++k) {
            const int j = h.nbr[(size_t)i * h.K + k];
            if (j < 0) continue;
            if (heading_away(h, xi, yi, col[X][j], col[Y][j], vxi, vyi, col[VX][j], col[VY][j])) {
                mpx += col[X][j];
                mpy += col[Y][j];
                mvx += col[VX][j];
                mvy += col[VY][j];
                num += 1;
            }
        }
        if (num > 0) {
            double ax = mpx / num - xi, ay = mpy / num - yi;
            normalize(ax, ay);
            double bx = mvx, by = mvy;
            normalize(bx, by);
            dhx = h.w_herd * ax + (1 - h.w_herd) * bx;
            dhy = h.w_herd * ay + (1 - h.w_herd) * by;
            normalize(dhx, dhy);
            has_dir = true;                            // target becomes NO_TARGET
        }
    }
    // leader_follower_interaction_brute: leaders from the nearest
    double dlx = 0.0, dly = 0.0;
    bool strategy = false;
    int behind = 0, away = 0;
    const int nl = *h.n_leaders;
    double pd = -INFINITY;
    int pj = -1;
    int leader_now = h.st.index_leader[i];
    int target_now = has_dir ? -1 : h.st.target[i];
    while (true) {
        double bd = INFINITY;
        int bj = 0x7fffffff;
        for (int q = lane; q < nl; q += 32) {
            const int j = h.leaders[q];
            if (h.scen_of[j] != sid) continue;
            const double d = cdm_hypot(xi - col[X][j], yi - col[Y][j]);
            const bool after = d > pd || (d == pd && j > pj);
            if (after && (d < bd || (d == bd && j < bj))) { bd = d; bj = j; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {               // nearest (distance, index) in the warp
            const double od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
            if (od < bd || (od == bd && oj < bj)) { bd = od; bj = oj; }
        }
        if (bj == 0x7fffffff || bd > h.sight_l) break;  // the rest are farther
        pd = bd;
        pj = bj;
        const int j = bj;
        if (blocked_warp(h, sc, xi, yi, col[X][j], col[Y][j], lane)) {
            const int leader = leader_now;
            if (leader != -1 && leader == j) {
                behind += 1;
                target_now = h.tgt_before[leader];
                strategy = true;
                break;
            }
            continue;
        }
        if (heading_away(h, xi, yi, col[X][j], col[Y][j], vxi, vyi, col[VX][j], col[VY][j])) {
            away += 1;
            leader_now = j;
            target_now = -1;
            double ax = col[X][j] - xi, ay = col[Y][j] - yi;
            normalize(ax, ay);
            double bx = col[VX][j], by = col[VY][j];
            normalize(bx, by);
            dlx = h.w_lead * ax + (1 - h.w_lead) * bx;
            dly = h.w_lead * ay + (1 - h.w_lead) * by;
            normalize(dlx, dly);
            strategy = true;
            break;
        }
    }
    if (behind == 0 && away == 0) {
        const int leader = leader_now;
        if (leader != -1) {
            target_now = h.tgt_before[leader];
            strategy = true;
        }
    }
    if (!(has_dir || strategy)) target_now = h.st.familiar_exit[i];   // familiar exit
    double ex = dlx, ey = dly;
    if (h.with_herding) {
        ex = h.w_dir * dlx + (1 - h.w_dir) * dhx;
        ey = h.w_dir * dly + (1 - h.w_dir) * dhy;
        normalize(ex, ey);
    }
    if (lane == 0) {
        h.st.index_leader[i] = leader_now;
        h.st.target[i] = target_now;
        col[E0X][i] = ex;
        col[E0Y][i] = ey;
    }
}

// ExitDetection (simulation/logic.py:220-237 with exit_detection,
// core/evacuation.py:139-174): the nearest door centre within the range that
// is in line of sight (agent to door); a follower that sees one takes it as
// its target and stops following.
__global__ void k_exit_detection(int begin, int count, const double *x, const double *y,
                                 const double *walls, int wall_begin, int wall_count,
                                 const double2 *doors, int n_doors, double range,
                                 StateCols st) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int i = begin + k;
    const double px = x[i], py = y[i];
    double dist = range;
    int found = -1;
    for (int c = 0; c < n_doors; ++c) {
        const double2 d = doors[c];
        bool hit = false;
        for (int w = wall_begin; w < wall_begin + wall_count && !hit; ++w) {
            const double *p = walls + (size_t)w * WALL_D;
            hit = line_intersect(px, py, d.x, d.y, p[0], p[1], p[2], p[3]);
        }
        if (hit) continue;
        const double l = cdm_hypot(d.x - px, d.y - py);
        if (l < dist) {
            dist = l;
            found = c;
        }
    }
    if (found >= 0 && st.follower[i]) {
        st.target[i] = found;
        st.follower[i] = 0;
    }
}

// Point in polygon as the reference's nodes compute it with matplotlib's
// Path.contains_points (simulation/logic.py:348-357,372-387): the "crossings
// multiply" test of E. Haines (Point in Polygon Strategies, Graphics Gems IV,
// 1994).  A ray from the point towards +x; an edge from an earlier vertex p0
// to the next p1 is a candidate when the flags (p.y >= ty) differ, and is
// crossed when ((p1.y - ty) * (p0.x - p1.x) >= (p1.x - tx) * (p0.y - p1.y))
// equals p1's flag; an odd count is inside.  The path is closed (the edge from
// the last vertex to the first is tested; a repeated first vertex only adds
// an edge of length zero) and a point with a non-finite coordinate is outside.
__device__ __forceinline__ bool inside_polygon(double tx, double ty, const double2 *v, int m) {
    bool inside = false;
    if (!(isfinite(tx) && isfinite(ty)) || m < 1) return false;
    double2 p0 = v[m - 1];
    bool y0 = p0.y >= ty;
    for (int k = 0; k < m; ++k) {
        const double2 p1 = v[k];
        const bool y1 = p1.y >= ty;
        if (y0 != y1) {
            if (((p1.y - ty) * (p0.x - p1.x) >= (p1.x - tx) * (p0.y - p1.y)) == y1)
                inside = !inside;
        }
        y0 = y1;
        p0 = p1;
    }
    return inside;
}

__global__ void k_inside_domain(int begin, int count, const double *x, const double *y,
                                int *active, const double2 *poly, int m,
                                unsigned long long *changed) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int change = 0;
    if (k < count) {
        const int i = begin + k;
        const int now = inside_polygon(x[i], y[i], poly, m) ? 1 : 0;
        change = active[i] != now;
        active[i] = now;
    }
    const unsigned b = __ballot_sync(0xffffffffu, change);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(changed, (unsigned long long)__popc(b));
}

__global__ void k_target_reached(int begin, int count, const double *x, const double *y,
                                 unsigned char *reached, const double2 *polys, const int *voff,
                                 int t, unsigned long long *counts) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int now = 0;
    if (k < count) {
        unsigned char &r = reached[k];
        if (!r && inside_polygon(x[begin + k], y[begin + k], polys + voff[t],
                                 voff[t + 1] - voff[t]))
            r = 1;
        now = r;
    }
    const unsigned b = __ballot_sync(0xffffffffu, now);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&counts[t], (unsigned long long)__popc(b));
}

inline int nblk(long long n, int nt) { return (int)((n + nt - 1) / nt); }

}  // namespace

void launch_herd_neighbors(const HerdArgs &h, cudaStream_t s) {
    if (h.n > 0 && h.with_herding)
        k_herd_neighbors<<<nblk((long long)h.n * 32, HNT), HNT, 0, s>>>(h);
}
void launch_check_roles(const StateCols &st, int n, int *err, cudaStream_t s) {
    if (n > 0) k_check_roles<<<nblk(n, 256), 256, 0, s>>>(st, n, err);
}
void launch_leaders(const HerdArgs &h, int *flags, int *pos, int *scan_scratch, int *list,
                    cudaStream_t s) {
    if (h.n <= 0) return;
    k_leader_flags<<<nblk(h.n, 256), 256, 0, s>>>(h, flags);
    launch_scan(flags, pos, h.n, scan_scratch, s);      // pos[n] = number of leaders
    k_leader_list<<<nblk(h.n, 256), 256, 0, s>>>(h, pos, list);
    k_target_snapshot<<<nblk(h.n, 256), 256, 0, s>>>(h);
}
void launch_herd_follow(const HerdArgs &h, cudaStream_t s) {
    if (h.n > 0) k_herd_follow<<<nblk((long long)h.n * 32, HNT), HNT, 0, s>>>(h);
}
void launch_inside_domain(int begin, int count, const double *x, const double *y, int *active,
                          const double2 *poly, int m, unsigned long long *changed,
                          cudaStream_t s) {
    if (count > 0 && m > 0)
        k_inside_domain<<<nblk(count, 256), 256, 0, s>>>(begin, count, x, y, active, poly, m,
                                                         changed);
}
void launch_exit_detection(int begin, int count, const double *x, const double *y,
                           const double *walls, int wall_begin, int wall_count,
                           const double2 *doors, int n_doors, double range, const StateCols &st,
                           cudaStream_t s) {
    if (count > 0)
        k_exit_detection<<<nblk(count, 256), 256, 0, s>>>(begin, count, x, y, walls, wall_begin,
                                                          wall_count, doors, n_doors, range, st);
}
void launch_target_reached(int begin, int count, const double *x, const double *y,
                           unsigned char *reached, const double2 *polys, const int *voff, int t,
                           unsigned long long *counts, cudaStream_t s) {
    if (count > 0)
        k_target_reached<<<nblk(count, 256), 256, 0, s>>>(begin, count, x, y, reached, polys, voff,
                                                          t, counts);
}

}  // namespace cdk
