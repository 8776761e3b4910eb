// cd_api.cu -- host side of the C ABI declared in include/cdgpu.h.
//
// A context owns every device buffer of one batch of scenarios; nothing is
// allocated per step, so a step (or a captured CUDA graph of one step) only
// launches kernels and memsets on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "cd_internal.cuh"
#include "cd_math.h"
#include "../../include/cdgpu.h"

using cdk::StepArgs;
using cdk::ScenDev;

static thread_local std::string g_create_error;

struct cd_ctx {
    int body = 0;
    int64_t n = 0, nw = 0, ncells = 0;
    int nscen = 0;
    std::vector<cd_scenario> scen_host;
    std::vector<ScenDev> scen_dev;
    std::vector<int> scen_of_host;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;              // beside the near-list build
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join_stage = nullptr;
    cudaEvent_t ev_read = nullptr;               // an upload has read the host records
    cudaEvent_t ev_ext = nullptr;                // an upload's extents are in ext_host
    bool ext_pending = false;                    // ext_host not yet folded into extent_max
    double *pro = nullptr;
    int device = 0;

    double *colbuf = nullptr;
    double *col[cdk::NCOL] = {};
    int *scen_of = nullptr;
    ScenDev *scen = nullptr;
    int *key = nullptr, *count = nullptr, *fill = nullptr, *start = nullptr;
    int *perm_unsorted = nullptr, *perm = nullptr, *scan_scratch = nullptr;
    double2 *stage = nullptr;
    float4 *cull = nullptr, *stage_f = nullptr;
    double *walls_raw = nullptr, *walls = nullptr;
    float4 *walls_f = nullptr;
    int *wall_start = nullptr, *wall_idx = nullptr;
    int64_t wall_idx_cap = 0;
    double *noise_f = nullptr, *noise_m = nullptr;
    bool noise_pending = false;
    bool noise_dev = false;                          // fluctuation drawn on the device
    uint64_t noise_seed = 0;
    unsigned long long *rng_step = nullptr;          // generator counter of the last step
    int *tgt = nullptr;                              // per-agent target index
    int *states = nullptr;                           // active, leader, follower, index_leader,
                                                     // familiar_exit (n each)
    bool states_dirty = false;                       // changed on the device since the upload
    // leader-follower / domain nodes (allocated on first use)
    int *herd = nullptr;                             // neighbours, flags, scan, list, targets
    int herd_k = 0;
    ScenDev *scen_h = nullptr;
    unsigned long long *counters = nullptr;          // domain changes, per-target counts
    unsigned char *reached = nullptr;                // per target x agent
    int64_t reached_targets = 0;
    double2 *polys = nullptr;
    int *poly_off = nullptr;
    int64_t poly_cap = 0;
    double2 *navmap = nullptr;                       // all scenarios' direction maps
    std::vector<std::vector<double>> nav_host;       // per scenario: x maps then y maps
    unsigned long long *vmax = nullptr;
    double *v0max = nullptr, *dt = nullptr, *time_tot = nullptr;
    double *ext = nullptr, *max_partial = nullptr;      // per-scenario max extent, scratch
    double *ext_host = nullptr;                        // pinned copy of ext
    // the direct upload's per-scenario maxima: two order keys per scenario
    // and the kernel's block counter, zero between uploads
    unsigned long long *max_key = nullptr;
    int *max_done = nullptr;
    int *status_host = nullptr;                        // pinned: error word, near-list need
    // device views of ext_host and status_host (null: copied by the stream)
    double *ext_host_dev = nullptr;
    int *status_host_dev = nullptr;
    int *err = nullptr, *work = nullptr;
    int *diag = nullptr;
    // near lists of the compute-once pair pipeline (entries allocated on use)
    int *nl_cnt = nullptr, *nl_off = nullptr, *nl_fwd = nullptr, *nl_scan = nullptr;
    unsigned *nl_mask = nullptr;
    int *nl_nch = nullptr;
    int *nl_idx = nullptr;
    double *nl_res = nullptr;
    unsigned char *nl_kind = nullptr;
    int *fix_count = nullptr, *fix_list = nullptr, *slot_of = nullptr;
    int *fw_cnt = nullptr, *fw_off = nullptr, *fw_scan = nullptr;
    int *fs_cnt = nullptr, *fs_off = nullptr, *fs_scan = nullptr;
    int2 *fw_pairs = nullptr;
    int *defer_list = nullptr;                     // the float32 pair pass's leftovers
    double2 *pair_jobs = nullptr;                  // k_pairs -> k_pair_forces
    int64_t nl_cap = 0;
    bool nl_fixed = false;              // capacity set by cd_set_near_list_capacity

    char *aos = nullptr;
    int64_t aos_bytes = 0, itemsize = 0;
    bool direct_host = true;               // pinned host records: device reads/writes them
    int64_t off[CD_F_COUNT];
    bool have_records = false;

    std::vector<double> walls_host;
    std::vector<double> extent_max;     // per scenario, from the last upload
    bool walls_dirty = true;

    cudaGraphExec_t graph = nullptr;
    int graph_nodes = -1;
    uint64_t graph_gen = 0;        // bumped whenever a graph of this context goes stale
    int variant = 0;

    cd_ctx *shadow = nullptr;      // the adjoint's recomputation context (made on first use)
    int timing = 0;                // 0 off; 1 run, step and kernel events; 2 run events only
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evs0 = nullptr, evs1 = nullptr;
    cudaEvent_t evr0 = nullptr, evr1 = nullptr;
    cudaEvent_t evp[3] = {nullptr, nullptr, nullptr};   // pair stage: start, after the
                                                         // float32 pass, end
    cudaEvent_t evsnap[CD_SNAPSHOT_SLOTS] = {};  // completion of asynchronous snapshots
    double pair_ms = 0, light_ms = 0;
    int64_t pair_launches = 0;
    double force_ms = 0, step_ms = 0, run_ms = 0;
    int64_t launches = 0, run_steps = 0;

    std::string msg;
};

namespace {

int fail(cd_ctx *c, int code, const std::string &m) {
    if (c) c->msg = m;
    else g_create_error = m;
    return code;
}

// Drop the step graph: buffers, variant or nodes changed (graphs built from
// this context's steps, its own or a group's, are stale from now on).
void drop_graph(cd_ctx *c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_nodes = -1;
    ++c->graph_gen;
}

#define CUDA_OR_FAIL(ctx, call)                                                       \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail((ctx), CD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

StepArgs args_of(cd_ctx *c, int nodes) {
    StepArgs a;
    a.n = (int)c->n;
    a.n_scen = c->nscen;
    a.n_cells = (int)c->ncells;
    a.body = c->body;
    a.nodes = nodes;
    for (int k = 0; k < cdk::NCOL; ++k) a.col[k] = c->col[k];
    a.scen_of = c->scen_of;
    a.scen = c->scen;
    a.key = c->key;
    a.count = c->count;
    a.fill = c->fill;
    a.start = c->start;
    a.perm_unsorted = c->perm_unsorted;
    a.perm = c->perm;
    a.stage = c->stage;
    a.cull = c->cull;
    a.stage_f = c->stage_f;
    a.walls = c->walls;
    a.walls_f = c->walls_f;
    a.wall_start = c->wall_start;
    a.wall_idx = c->wall_idx;
    a.noise_f = c->noise_f;
    a.noise_m = c->noise_m;
    a.noise_dev = c->noise_dev ? 1 : 0;
    a.noise_seed = c->noise_seed;
    a.rng_step = c->rng_step;
    a.tgt = c->tgt;
    a.navmap = c->navmap;
    a.vmax = c->vmax;
    a.v0max = c->v0max;
    a.dt = c->dt;
    a.time_tot = c->time_tot;
    a.err = c->err;
    a.work = c->work;
    a.nl_cnt = c->nl_cnt;
    a.nl_off = c->nl_off;
    a.nl_fwd = c->nl_fwd;
    a.nl_mask = c->nl_mask;
    a.nl_nch = c->nl_nch;
    a.nl_idx = c->nl_idx;
    a.nl_res = c->nl_res;
    a.nl_kind = c->nl_kind;
    a.fix_count = c->fix_count;
    a.fix_list = c->fix_list;
    a.slot_of = c->slot_of;
    a.pro = c->pro;
    a.nl_cap = (int)c->nl_cap;
    a.nl_scan = c->nl_scan;
    a.fw_cnt = c->fw_cnt;
    a.fw_off = c->fw_off;
    a.fw_pairs = c->fw_pairs;
    a.defer_list = c->defer_list;
    a.pair_jobs = c->pair_jobs;
    a.fw_scan = c->fw_scan;
    a.fs_cnt = c->fs_cnt;
    a.fs_off = c->fs_off;
    a.fs_scan = c->fs_scan;
    return a;
}

template <typename T>
int dalloc(cd_ctx *c, T **p, int64_t count) {
    size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(count, 1);
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess)
        return fail(c, CD_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return CD_OK;
}

void release(cd_ctx *c) {
    if (c->shadow) cd_destroy(c->shadow);
    c->shadow = nullptr;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    void *ptrs[] = {c->colbuf, c->scen_of, c->scen, c->key, c->count, c->fill, c->start,
                    c->perm_unsorted, c->perm, c->scan_scratch, c->stage, c->cull, c->stage_f,
                    c->walls_raw, c->walls, c->walls_f, c->wall_start, c->wall_idx,
                    c->noise_f, c->noise_m, c->vmax, c->v0max, c->dt, c->time_tot,
                    c->err, c->work, c->diag, c->aos, c->nl_cnt, c->nl_off, c->nl_fwd,
                    c->nl_scan, c->nl_idx, c->nl_res, c->nl_kind, c->fw_cnt, c->fw_off, c->fw_scan,
                    c->fw_pairs, c->defer_list, c->pair_jobs, c->ext, c->max_partial, c->tgt, c->navmap, c->rng_step,
                    c->states, c->herd, c->scen_h, c->counters, c->reached, c->polys,
                    c->poly_off, c->fs_cnt, c->fs_off, c->fs_scan, c->nl_mask, c->nl_nch,
                    c->fix_count, c->fix_list, c->slot_of, c->pro};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->evs0) cudaEventDestroy(c->evs0);
    if (c->evs1) cudaEventDestroy(c->evs1);
    if (c->evr0) cudaEventDestroy(c->evr0);
    if (c->evr1) cudaEventDestroy(c->evr1);
    if (c->evp[0]) cudaEventDestroy(c->evp[0]);
    if (c->evp[1]) cudaEventDestroy(c->evp[1]);
    if (c->evp[2]) cudaEventDestroy(c->evp[2]);
    for (cudaEvent_t e : c->evsnap)
        if (e) cudaEventDestroy(e);
    if (c->ext_host) cudaFreeHost(c->ext_host);
    if (c->max_key) cudaFree(c->max_key);
    if (c->max_done) cudaFree(c->max_done);
    if (c->status_host) cudaFreeHost(c->status_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_join_stage) cudaEventDestroy(c->ev_join_stage);
    if (c->ev_read) cudaEventDestroy(c->ev_read);
    if (c->ev_ext) cudaEventDestroy(c->ev_ext);
}

// Flat cell range of a coordinate interval along one axis (clamped).
inline void axis_range(double lo, double hi, double v0, double cell, int64_t n, int64_t &a,
                       int64_t &b) {
    auto f = [&](double v) -> int64_t {
        double q = std::floor((v - v0) / cell);
        if (q < 0) return 0;
        if (q > (double)(n - 1)) return n - 1;
        return (int64_t)q;
    };
    a = f(lo);
    b = f(hi);
}

// Bin every wall into the cells whose square overlaps the wall's bounding
// box grown by the scenario's agent extent (+ a margin); per-cell lists stay
// in ascending wall order, the reference's loop order.
int bin_walls(cd_ctx *c) {
    std::vector<int> cnt((size_t)c->ncells + 1, 0);
    std::vector<std::pair<int, int>> items;
    for (int s = 0; s < c->nscen; ++s) {
        const cd_scenario &sc = c->scen_host[s];
        double ext = c->extent_max.empty() ? 0.0 : c->extent_max[s];
        double reach = ext + 0.05;
        c->scen_dev[s].wall_reach = ext + 0.04;
        int64_t base = c->scen_dev[s].cell_base;
        for (int64_t w = sc.wall_begin; w < sc.wall_begin + sc.wall_count; ++w) {
            const double *p = &c->walls_host[4 * w];
            bool ok = true;
            for (int k = 0; k < 4; ++k) ok &= std::isfinite(p[k]);
            if (!ok) continue;     // the reference's distance is NaN: no contact
            int64_t x0, x1, y0, y1;
            axis_range(std::min(p[0], p[2]) - reach, std::max(p[0], p[2]) + reach, sc.x0,
                       sc.cell_size, sc.nx, x0, x1);
            axis_range(std::min(p[1], p[3]) - reach, std::max(p[1], p[3]) + reach, sc.y0,
                       sc.cell_size, sc.ny, y0, y1);
            for (int64_t ix = x0; ix <= x1; ++ix)
                for (int64_t iy = y0; iy <= y1; ++iy) {
                    int cell = (int)(base + ix * sc.ny + iy);
                    items.emplace_back(cell, (int)w);
                    cnt[cell]++;
                }
        }
    }
    std::vector<int> startv((size_t)c->ncells + 1, 0);
    for (int64_t k = 0; k < c->ncells; ++k) startv[k + 1] = startv[k] + cnt[k];
    std::vector<int> idx(items.size());
    std::vector<int> fillv((size_t)c->ncells, 0);
    for (auto &it : items) idx[startv[it.first] + fillv[it.first]++] = it.second;
    if ((int64_t)idx.size() > c->wall_idx_cap) {
        if (c->wall_idx) cudaFree(c->wall_idx);
        c->wall_idx = nullptr;
        if (int rc = dalloc(c, &c->wall_idx, (int64_t)idx.size())) return rc;
        c->wall_idx_cap = (int64_t)idx.size();
        drop_graph(c);
    }
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->wall_start, startv.data(), sizeof(int) * startv.size(),
                                    cudaMemcpyHostToDevice, c->stream));
    if (!idx.empty())
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->wall_idx, idx.data(), sizeof(int) * idx.size(),
                                        cudaMemcpyHostToDevice, c->stream));
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->scen, c->scen_dev.data(), sizeof(ScenDev) * c->nscen,
                                    cudaMemcpyHostToDevice, c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    c->walls_dirty = false;
    return CD_OK;
}

// Cell list + staging for the current state (no forces).
// `defer_stage`: only the pre-check records here; the force stage writes the
// float64 staged records beside the near-list build.
void enqueue_cells(cd_ctx *c, const StepArgs &a, bool defer_stage = false) {
    // count, fill and vmax are zero between cell lists (zeroed at creation,
    // then by k_rank and k_scatter once used)
    cdk::launch_prepare(a, c->stream);
    // dt is computed by the scatter kernel, launched only for agents
    const bool dt_kernel = (a.nodes & cdk::N_INTEG) && a.n == 0;
    if (dt_kernel) cdk::launch_dt(a, c->stream);
    // each kernel of the cell list chained to the one before it
    cdk::launch_scan(c->count, c->start, (int)c->ncells, c->scan_scratch, c->stream,
                     a.n > 0 || dt_kernel);
    cdk::launch_scatter(a, c->stream, true, defer_stage ? 1 : 0);     // rank + gather
}

// One step on the context stream.  `timed`: record the step and force-kernel
// events (cd_step).  `captured`: the sequence is being captured into a graph;
// with kernel timing (mode 1) the force-stage and pair events are then
// recorded as external event-record nodes (a plain cudaEventRecord under
// capture only marks a capture dependency); otherwise the graph holds none,
// so that every kernel of the step stays chained to the one before it.
void enqueue_step(cd_ctx *c, int nodes, bool timed, bool captured = false) {
    StepArgs a = args_of(c, nodes);
    const bool kev = captured && c->timing == 1;
    // the pair pipeline writes the float64 staged records beside the near lists
    const bool defer = cdk::variant_pairs(c->variant) && c->nl_cnt;
    if (timed) cudaEventRecord(c->evs0, c->stream);
    enqueue_cells(c, a, defer);
    if (timed) cudaEventRecord(c->ev0, c->stream);
    if (kev) cudaEventRecordWithFlags(c->ev0, c->stream, cudaEventRecordExternal);
    const cdk::Fork fork{c->stream2, c->ev_fork, c->ev_join, c->ev_join_stage};
    cdk::launch_forces(a, c->stream, c->variant, (timed || kev) ? c->evp : nullptr, captured,
                       &fork, defer);
    if (timed) cudaEventRecord(c->ev1, c->stream);
    if (kev) cudaEventRecordWithFlags(c->ev1, c->stream, cudaEventRecordExternal);
    if (timed) cudaEventRecord(c->evs1, c->stream);
}

int64_t kernels_per_step(const cd_ctx *c, int nodes) {
    if (c->n == 0) return (nodes & CD_NODE_INTEGRATE) ? 1 : 0;
    int64_t k = 4;                                      // prepare scatter(+dt) rank(+gather) forces
    k += cdk::scan_launches_single((int)c->ncells);
    if (cdk::variant_pairs(c->variant) && c->nl_cnt) k += 2;     // prologue, float64 staging
    if (cdk::variant_pairs(c->variant) && (nodes & CD_NODE_AGENT_AGENT) && c->nl_cnt)
        k += 5 + (c->defer_list ? 1 : 0) +        // count, scans, fill, (float32 pass,) pairs,
             (cdk::variant_split(c->variant) ? 1 : 0);    // (force pass,) fallback
    return k;
}

// Entries of the near lists: `need` plus a quarter (density changes between
// steps), reallocated when a step needed more than the current capacity.
int alloc_near_lists(cd_ctx *c, int64_t cap) {
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    if (c->nl_idx) cudaFree(c->nl_idx);
    if (c->nl_res) cudaFree(c->nl_res);
    if (c->nl_kind) cudaFree(c->nl_kind);
    if (c->fw_pairs) cudaFree(c->fw_pairs);
    if (c->defer_list) cudaFree(c->defer_list);
    if (c->pair_jobs) cudaFree(c->pair_jobs);
    c->defer_list = nullptr;
    c->pair_jobs = nullptr;
    c->nl_idx = nullptr;
    c->nl_res = nullptr;
    c->nl_kind = nullptr;
    c->fw_pairs = nullptr;
    c->nl_cap = 0;
    const int64_t res_d = c->body == CD_BODY_CIRCULAR ? cdk::ADJ_RES_D : cdk::RES_D;
    if (cap > 0) {
        if (int rc = dalloc(c, &c->nl_idx, cap)) return rc;
        if (int rc = dalloc(c, &c->nl_res, cap * res_d)) return rc;
        // 16 bytes past the last entry: the gather reads the kinds in 4-byte words
        if (int rc = dalloc(c, &c->nl_kind, cap + 16)) return rc;
        if (int rc = dalloc(c, &c->fw_pairs, cap)) return rc;
        if (int rc = dalloc(c, &c->defer_list, cap)) return rc;
        const int64_t job_q = c->body == CD_BODY_CIRCULAR ? cdk::JOB_Q_CIRC : cdk::JOB_Q_TC;
        if (int rc = dalloc(c, &c->pair_jobs, (cap / 2 + 1) * job_q)) return rc;
    }
    c->nl_cap = cap;
    drop_graph(c);
    return CD_OK;
}

int grow_near_lists(cd_ctx *c, int64_t need) {
    if (c->nl_fixed) return CD_OK;
    int64_t cap = need + need / 4 + 1024;
    if (cap > (int64_t)INT32_MAX / 8) cap = (int64_t)INT32_MAX / 8;
    if (cap <= c->nl_cap) return CD_OK;
    return alloc_near_lists(c, cap);
}

// Near-list entries for the current state (pair pipeline, adjoint), counted
// and allocated on first use.
int size_near_lists(cd_ctx *c) {
    if (c->n == 0 || c->nl_cap > 0 || c->nl_fixed) return CD_OK;
    StepArgs a = args_of(c, CD_NODE_AGENT_AGENT);
    enqueue_cells(c, a);
    cdk::launch_near_count(a, c->stream, cdk::variant_pairs(c->variant) ? c->variant : 10);
    int need = 0;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(&need, c->nl_off + c->n, sizeof(int), cudaMemcpyDeviceToHost,
                                    c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    return grow_near_lists(c, need);
}

int ensure_near_lists(cd_ctx *c, int nodes) {
    if (!cdk::variant_pairs(c->variant) || !(nodes & CD_NODE_AGENT_AGENT)) return CD_OK;
    return size_near_lists(c);
}

// Pair-kernel time of the step just timed (pair pipeline with agent-agent).
void add_pair_time(cd_ctx *c, int nodes) {
    if (!cdk::variant_pairs(c->variant) || !(nodes & CD_NODE_AGENT_AGENT) || c->n == 0) return;
    float pms = 0, lms = 0;
    if (cudaEventElapsedTime(&pms, c->evp[0], c->evp[2]) == cudaSuccess) {
        c->pair_ms += pms;
        c->pair_launches += 1;
        if (c->defer_list && cudaEventElapsedTime(&lms, c->evp[0], c->evp[1]) == cudaSuccess)
            c->light_ms += lms;
    }
}

// Offsets of the integer and bool fields that fit the record (-1 otherwise).
cdk::StateOffsets state_offsets(const int64_t *off, int64_t itemsize) {
    auto f = [&](int field, int bytes) -> long long {
        return (off[field] >= 0 && off[field] + bytes <= itemsize) ? off[field] : -1;
    };
    cdk::StateOffsets o;
    o.target = f(CD_F_TARGET, 8);
    o.active = f(CD_F_ACTIVE, 1);
    o.leader = f(CD_F_IS_LEADER, 1);
    o.follower = f(CD_F_IS_FOLLOWER, 1);
    o.index_leader = f(CD_F_INDEX_LEADER, 8);
    o.familiar_exit = f(CD_F_FAMILIAR_EXIT, 8);
    return o;
}

cdk::StateCols state_cols(cd_ctx *c) {
    const int64_t np = std::max<int64_t>(c->n, 1);
    cdk::StateCols k;
    k.target = c->tgt;
    k.active = c->states;
    k.leader = c->states + np;
    k.follower = c->states + 2 * np;
    k.index_leader = c->states + 3 * np;
    k.familiar_exit = c->states + 4 * np;
    return k;
}

// Enqueue the copies of the error word and the near-list need into pinned
// host memory (asynchronous; read by check_device_error after the next
// synchronisation).
int enqueue_status(cd_ctx *c) {
    c->status_host[1] = 0;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(&c->status_host[0], c->err, sizeof(int),
                                    cudaMemcpyDeviceToHost, c->stream));
    if (c->nl_cap > 0 && c->n > 0)
        CUDA_OR_FAIL(c, cudaMemcpyAsync(&c->status_host[1], c->nl_off + c->n, sizeof(int),
                                        cudaMemcpyDeviceToHost, c->stream));
    return CD_OK;
}

// `enqueued`: the caller already enqueued the status copies before its own
// synchronisation (one synchronisation for both).
// Folds the extents read back by the last upload into the wall-bin sizing;
// the bins are rebuilt before the next step when an agent grew beyond the
// extent they were built for.  This runs where the host waits for the stream
// anyway (after a step's or a download's synchronisation, before the next
// upload), so the step right after an upload always runs on the bins it
// found: an agent that outgrew them scans every wall of its scenario (its
// float32 extent exceeds the scenario's wall_reach), with the same walls
// skipped as too far, and the results do not depend on the bins.
int absorb_extent(cd_ctx *c) {
    if (!c->ext_pending) return CD_OK;
    CUDA_OR_FAIL(c, cudaEventSynchronize(c->ev_ext));
    c->ext_pending = false;
    if (c->extent_max.empty()) {
        c->extent_max.assign(c->ext_host, c->ext_host + c->nscen);
        c->walls_dirty = true;
    } else {
        bool grew = false;
        for (int s = 0; s < c->nscen; ++s) grew |= c->ext_host[s] > c->extent_max[s];
        if (grew) {
            c->walls_dirty = true;
            for (int s = 0; s < c->nscen; ++s)
                c->extent_max[s] = std::max(c->extent_max[s], c->ext_host[s]);
        }
    }
    return CD_OK;
}

int check_device_error(cd_ctx *c, bool enqueued = false) {
    CUDA_OR_FAIL(c, cudaGetLastError());
    const bool pairs = c->nl_cap > 0 && c->n > 0;       // lists in use (pair pipeline, adjoint)
    if (!enqueued) {
        if (int rc = enqueue_status(c)) return rc;
        CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    }
    if (int rc = absorb_extent(c)) return rc;       // complete: the stream was synchronised
    const int h = c->status_host[0], need = c->status_host[1];
    // the last list build did not fit: its step ran the fallback; grow for the next
    if (pairs && need > c->nl_cap)
        if (int rc = grow_near_lists(c, need)) return rc;
    if (h) {
        cudaMemsetAsync(c->err, 0, sizeof(int), c->stream);
        cudaStreamSynchronize(c->stream);
        if (h & cdk::ERR_NOT_FINITE)
            return fail(c, CD_ERR_NOT_FINITE, "an agent position is not finite");
        if (h & cdk::ERR_LEADER_FOLLOWER)
            return fail(c, CD_ERR_INVALID_VALUE,
                        "an agent is both leader and follower (is_leader and is_follower)");
        if (h & cdk::ERR_RANGE)
            return fail(c, CD_ERR_INVALID_VALUE,
                        "an agent is more than 1e7 m from its scenario's grid origin");
        if (h & cdk::ERR_NEAR_LIST)
            return fail(c, CD_ERR_CUDA, "internal error: a near list lacks a pair partner");
        return fail(c, CD_ERR_INVALID_VALUE, "device reported error bits " + std::to_string(h));
    }
    return CD_OK;
}

int prepare_step(cd_ctx *c, int nodes) {
    if (nodes & ~(CD_NODE_ALL | CD_NODE_NAVIGATION))
        return fail(c, CD_ERR_INVALID_VALUE, "unknown node flags");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if ((nodes & CD_NODE_AGENT_OBSTACLE) && c->walls_dirty && c->nw > 0) {
        if (c->walls_host.empty())
            return fail(c, CD_ERR_INVALID_VALUE, "walls declared but cd_set_walls not called");
        if (int rc = bin_walls(c)) return rc;
    }
    return ensure_near_lists(c, nodes);
}

bool aligned_field(int64_t off, int64_t itemsize, int width) {
    return off >= 0 && (off % 4) == 0 && off + 8 * width <= itemsize;
}

// The device address of host memory [p, p + bytes) when all of it is pinned
// and mapped for the device (both ends inside one mapping), else null.
const void *device_view_of_host(const void *p, int64_t bytes) {
    if (!p || bytes <= 0) return nullptr;
    cudaPointerAttributes a0{}, a1{};
    const char *last = static_cast<const char *>(p) + (bytes - 1);
    if (cudaPointerGetAttributes(&a0, p) != cudaSuccess ||
        cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer ||
        !a1.devicePointer)
        return nullptr;
    const char *d0 = static_cast<const char *>(a0.devicePointer);
    if (static_cast<const char *>(a1.devicePointer) - d0 != bytes - 1) return nullptr;
    if (reinterpret_cast<uintptr_t>(d0) % 4) return nullptr;
    return d0;
}

}  // namespace

extern "C" {

const char *cd_last_error(const cd_ctx *ctx) {
    return ctx ? ctx->msg.c_str() : g_create_error.c_str();
}

int cd_create(cd_ctx **out, int body_type, int64_t n_scenarios, const cd_scenario *scen) {
    if (!out) return fail(nullptr, CD_ERR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (body_type != CD_BODY_CIRCULAR && body_type != CD_BODY_THREE_CIRCLE)
        return fail(nullptr, CD_ERR_INVALID_TYPE, "unknown body type");
    if (n_scenarios < 1 || !scen) return fail(nullptr, CD_ERR_INVALID_VALUE, "need >= 1 scenario");
    int64_t n = 0, nw = 0, ncells = 0;
    for (int64_t s = 0; s < n_scenarios; ++s) {
        const cd_scenario &sc = scen[s];
        if (sc.agent_begin != n || sc.agent_count < 0 || sc.wall_begin != nw || sc.wall_count < 0)
            return fail(nullptr, CD_ERR_INVALID_VALUE, "agent/wall ranges must tile in order");
        if (!(sc.cell_size > 0) || !std::isfinite(sc.cell_size) || !std::isfinite(sc.x0) ||
            !std::isfinite(sc.y0) || sc.nx < 1 || sc.ny < 1)
            return fail(nullptr, CD_ERR_INVALID_VALUE, "bad cell grid");
        if (!(sc.dt_min >= 0) || !(sc.dt_max >= 0) || !std::isfinite(sc.dt_max))
            return fail(nullptr, CD_ERR_INVALID_VALUE, "bad timestep bounds");
        n += sc.agent_count;
        nw += sc.wall_count;
        ncells += sc.nx * sc.ny;
        if (sc.nx > (1 << 30) || sc.ny > (1 << 30) || ncells > (int64_t)INT32_MAX - 1)
            return fail(nullptr, CD_ERR_CAPACITY, "too many cells");
    }
    if (n > (int64_t)INT32_MAX / 16 || nw > (int64_t)INT32_MAX / 16)
        return fail(nullptr, CD_ERR_CAPACITY, "too many agents or walls");

    cd_ctx *c = new cd_ctx();
    c->body = body_type;
    c->n = n;
    c->variant = cdk::default_variant(n, body_type == CD_BODY_CIRCULAR ? 0 : 1);
    c->nw = nw;
    c->ncells = ncells;
    c->nscen = (int)n_scenarios;
    c->scen_host.assign(scen, scen + n_scenarios);
    c->scen_dev.resize(n_scenarios);
    c->nav_host.resize(n_scenarios);
    c->scen_of_host.resize(std::max<int64_t>(n, 1));
    std::fill(c->off, c->off + CD_F_COUNT, -1);
    int64_t base = 0;
    for (int64_t s = 0; s < n_scenarios; ++s) {
        const cd_scenario &sc = scen[s];
        ScenDev &d = c->scen_dev[s];
        d.x0 = sc.x0; d.y0 = sc.y0; d.cell = sc.cell_size;
        d.dt_min = sc.dt_min; d.dt_max = sc.dt_max;
        d.wall_reach = 0.0;
        d.nx = (int)sc.nx; d.ny = (int)sc.ny;
        d.cell_base = (int)base;
        d.agent_begin = (int)sc.agent_begin; d.agent_count = (int)sc.agent_count;
        d.wall_begin = (int)sc.wall_begin; d.wall_count = (int)sc.wall_count;
        d.nav_x0 = 0.0; d.nav_y0 = 0.0; d.nav_step = 1.0;
        d.nav_nx = 0; d.nav_ny = 0; d.nav_targets = 0; d.nav_off = 0;
        base += sc.nx * sc.ny;
        for (int64_t i = sc.agent_begin; i < sc.agent_begin + sc.agent_count; ++i)
            c->scen_of_host[i] = (int)s;
    }
    int rc = CD_OK;
    auto step = [&](int r) { if (r && !rc) rc = r; return rc == CD_OK; };
    cudaGetDevice(&c->device);
    if (int e = cdk::init_kernels())
        rc = fail(c, CD_ERR_CUDA, std::string("kernel attributes: ") +
                                     cudaGetErrorString((cudaError_t)e));
    // the step's critical path runs on the context stream; the second stream
    // (the prologue, the float64 staging) fills the SMs the critical path
    // leaves idle: it gets the lowest priority, the context stream the highest,
    // so that waiting blocks of the critical path are scheduled first
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->stream2, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join_stage, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_read, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_ext, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(c, CD_ERR_CUDA, "cudaStreamCreate failed");
    const int64_t npad = std::max<int64_t>(n, 1);
    if (rc == CD_OK && step(dalloc(c, &c->colbuf, npad * cdk::NCOL)))
        for (int k = 0; k < cdk::NCOL; ++k) c->col[k] = c->colbuf + k * npad;
    const int sq = body_type == CD_BODY_CIRCULAR ? cdk::STAGE_Q_CIRC : cdk::STAGE_Q_TC;
    step(dalloc(c, &c->scen_of, n));
    step(dalloc(c, &c->scen, n_scenarios));
    step(dalloc(c, &c->key, n));
    step(dalloc(c, &c->count, ncells));
    step(dalloc(c, &c->fill, ncells));
    step(dalloc(c, &c->start, ncells + 1));
    step(dalloc(c, &c->perm_unsorted, n));
    step(dalloc(c, &c->perm, n));
    step(dalloc(c, &c->scan_scratch, cdk::scan_scratch_ints((int)ncells)));
    step(dalloc(c, &c->stage, n * sq));
    step(dalloc(c, &c->cull, n));
    step(dalloc(c, &c->stage_f, 2 * n));
    step(dalloc(c, &c->walls_raw, nw * 4));
    step(dalloc(c, &c->walls, nw * cdk::WALL_D));
    step(dalloc(c, &c->walls_f, nw));
    step(dalloc(c, &c->wall_start, ncells + 1));
    step(dalloc(c, &c->noise_f, 2 * n));
    step(dalloc(c, &c->noise_m, n));
    step(dalloc(c, &c->tgt, n));
    step(dalloc(c, &c->states, 5 * npad));
    step(dalloc(c, &c->rng_step, 1));
    step(dalloc(c, &c->vmax, n_scenarios));
    step(dalloc(c, &c->v0max, n_scenarios));
    step(dalloc(c, &c->ext, n_scenarios));
    step(dalloc(c, &c->max_key, 2 * (int64_t)n_scenarios));
    step(dalloc(c, &c->max_done, 1));
    if (rc == CD_OK &&
        (cudaMemset(c->max_key, 0, sizeof(unsigned long long) * 2 * n_scenarios) != cudaSuccess ||
         cudaMemset(c->max_done, 0, sizeof(int)) != cudaSuccess))
        rc = fail(c, CD_ERR_CUDA, "cudaMemset failed");
    step(dalloc(c, &c->max_partial, cdk::scen_max_partials((int)n_scenarios)));
    if (rc == CD_OK && cudaMallocHost((void **)&c->ext_host, sizeof(double) * n_scenarios) != cudaSuccess)
        rc = fail(c, CD_ERR_CUDA, "cudaMallocHost failed");
    if (rc == CD_OK && cudaMallocHost((void **)&c->status_host, sizeof(int) * 2) != cudaSuccess)
        rc = fail(c, CD_ERR_CUDA, "cudaMallocHost failed");
    if (rc == CD_OK) {
        // the transfer kernels write these two directly where the device can
        // address them; otherwise small copies on the stream do
        if (cudaHostGetDevicePointer((void **)&c->ext_host_dev, c->ext_host, 0) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&c->status_host_dev, c->status_host, 0) != cudaSuccess) {
            c->ext_host_dev = nullptr;
            c->status_host_dev = nullptr;
            cudaGetLastError();
        }
    }
    step(dalloc(c, &c->dt, n_scenarios));
    step(dalloc(c, &c->time_tot, n_scenarios));
    step(dalloc(c, &c->err, 1));
    step(dalloc(c, &c->work, 4));
    step(dalloc(c, &c->diag, (int64_t)CD_COUNT_COLS * n));
    step(dalloc(c, &c->nl_cnt, n + 1));
    step(dalloc(c, &c->nl_off, n + 1));
    step(dalloc(c, &c->nl_fwd, n));
    step(dalloc(c, &c->fix_count, 1));
    step(dalloc(c, &c->fix_list, n));
    step(dalloc(c, &c->slot_of, n));
    step(dalloc(c, &c->pro, cdk::PRO_D * (int64_t)n));
    step(dalloc(c, &c->nl_mask, (int64_t)n * cdk::NL_MASK_CHUNKS));
    step(dalloc(c, &c->nl_nch, n + 1));
    step(dalloc(c, &c->nl_scan, cdk::near_scan_ints((int)npad)));
    step(dalloc(c, &c->fw_cnt, n + 1));
    step(dalloc(c, &c->fw_off, n + 1));
    step(dalloc(c, &c->fw_scan, cdk::near_scan_ints((int)npad)));
    step(dalloc(c, &c->fs_cnt, n + 1));
    step(dalloc(c, &c->fs_off, n + 1));
    step(dalloc(c, &c->fs_scan, cdk::near_scan_ints((int)npad)));
    if (rc == CD_OK) {
        cudaMemcpy(c->scen_of, c->scen_of_host.data(), sizeof(int) * npad, cudaMemcpyHostToDevice);
        cudaMemcpy(c->scen, c->scen_dev.data(), sizeof(ScenDev) * n_scenarios, cudaMemcpyHostToDevice);
        cudaMemset(c->colbuf, 0, sizeof(double) * npad * cdk::NCOL);
        cudaMemset(c->time_tot, 0, sizeof(double) * n_scenarios);
        cudaMemset(c->dt, 0, sizeof(double) * n_scenarios);
        cudaMemset(c->err, 0, sizeof(int));
        cudaMemset(c->rng_step, 0, sizeof(unsigned long long));
        cudaMemset(c->wall_start, 0, sizeof(int) * (ncells + 1));
        cudaMemset(c->count, 0, sizeof(int) * ncells);       // zero between cell lists
        cudaMemset(c->fill, 0, sizeof(int) * ncells);
        cudaMemset(c->vmax, 0, sizeof(unsigned long long) * n_scenarios);
        for (int *p : {c->nl_scan, c->fw_scan, c->fs_scan})   // the scans' tile counters
            cudaMemset(p, 0, sizeof(int) * cdk::near_scan_ints((int)npad));
        cudaEventCreate(&c->ev0);
        cudaEventCreate(&c->ev1);
        cudaEventCreate(&c->evs0);
        cudaEventCreate(&c->evs1);
        cudaEventCreate(&c->evr0);
        cudaEventCreate(&c->evr1);
        cudaEventCreate(&c->evp[0]);
        cudaEventCreate(&c->evp[1]);
        cudaEventCreate(&c->evp[2]);
        for (cudaEvent_t &e : c->evsnap) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = fail(c, CD_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc != CD_OK) {
        g_create_error = c->msg;
        release(c);
        delete c;
        return rc;
    }
    c->walls_dirty = nw > 0;
    *out = c;
    return CD_OK;
}

void cd_destroy(cd_ctx *ctx) {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->stream);
    release(ctx);
    delete ctx;
}

namespace {
int upload_records(cd_ctx *c, const void *records, int64_t n, int64_t itemsize,
                   const int64_t *off, bool wait_read);
}

int cd_upload_agents(cd_ctx *c, const void *records, int64_t n, int64_t itemsize,
                     const int64_t *off) {
    return upload_records(c, records, n, itemsize, off, true);
}

namespace {
// `wait_read`: return once the records have been read (cd_upload_agents);
// cd_step_records does not wait, since it returns only after the download.
int upload_records(cd_ctx *c, const void *records, int64_t n, int64_t itemsize,
                   const int64_t *off, bool wait_read) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (n != c->n) return fail(c, CD_ERR_INVALID_VALUE, "agent count differs from the context");
    if (itemsize <= 0 || !off || (n > 0 && !records))
        return fail(c, CD_ERR_INVALID_VALUE, "bad records");
    static const int need_circ[] = {CD_F_POSITION, CD_F_VELOCITY, CD_F_TARGET_DIRECTION, CD_F_FORCE,
                                    CD_F_FORCE_PREV, CD_F_RADIUS, CD_F_MASS, CD_F_TARGET_VELOCITY,
                                    CD_F_TAU_ADJ, CD_F_K_SOC, CD_F_TAU_0, CD_F_MU, CD_F_KAPPA,
                                    CD_F_DAMPING};
    static const int need_tc[] = {CD_F_R_T, CD_F_R_S, CD_F_R_TS, CD_F_INERTIA_ROT,
                                  CD_F_TARGET_ANGULAR_VELOCITY, CD_F_POSITION_LS, CD_F_POSITION_RS,
                                  CD_F_ORIENTATION, CD_F_ANGULAR_VELOCITY, CD_F_TARGET_ORIENTATION,
                                  CD_F_TORQUE, CD_F_TORQUE_PREV, CD_F_TAU_ROT};
    for (int f : need_circ) {
        int width = (f <= CD_F_FORCE_PREV) ? 2 : 1;
        if (!aligned_field(off[f], itemsize, width))
            return fail(c, CD_ERR_INVALID_TYPE, "record lacks a required, 4-byte aligned field");
    }
    if (c->body == CD_BODY_THREE_CIRCLE)
        for (int f : need_tc) {
            int width = (f == CD_F_POSITION_LS || f == CD_F_POSITION_RS) ? 2 : 1;
            if (!aligned_field(off[f], itemsize, width))
                return fail(c, CD_ERR_INVALID_TYPE, "record lacks a ThreeCircle field");
        }
    if (itemsize % 4) return fail(c, CD_ERR_INVALID_TYPE, "record size must be a multiple of 4");
    // optional float64 fields, where present, obey the same alignment
    for (int f = 0; f < CD_F_TARGET; ++f) {
        const int width = (f <= CD_F_FORCE_PREV || f == CD_F_POSITION_LS || f == CD_F_POSITION_RS) ? 2 : 1;
        if (off[f] >= 0 && !aligned_field(off[f], itemsize, width))
            return fail(c, CD_ERR_INVALID_TYPE, "float64 record field not 4-byte aligned");
    }
    // the previous upload's read-back lands in ext_host: fold it in first
    if (int rc = absorb_extent(c)) return rc;
    int64_t bytes = n * itemsize;
    if (bytes > c->aos_bytes) {
        if (c->aos) cudaFree(c->aos);
        c->aos = nullptr;
        if (int rc = dalloc(c, &c->aos, bytes)) return rc;
        c->aos_bytes = bytes;
    }
    c->itemsize = itemsize;
    std::memcpy(c->off, off, sizeof(int64_t) * CD_F_COUNT);
    bool maxima_done = false;
    if (n > 0) {
        long long offl[CD_F_COUNT];
        for (int k = 0; k < CD_F_COUNT; ++k) offl[k] = off[k];
        const void *dv = (c->direct_host && cdk::records_per_block(itemsize) > 0)
                             ? device_view_of_host(records, bytes)
                             : nullptr;
        const cdk::StateOffsets so = state_offsets(off, itemsize);
        if (dv) {
            // the per-scenario maxima in the same pass
            const cdk::ScenMax mx{c->max_key,    c->max_done,  c->scen_of,
                                  c->v0max,      c->ext,       c->ext_host_dev,
                                  (int)c->nscen, c->body == CD_BODY_CIRCULAR ? 0 : 1};
            cdk::launch_records_in(dv, c->aos, itemsize, offl, (int)n, c->body, c->col, so,
                                   state_cols(c), c->stream, mx);
            CUDA_OR_FAIL(c, cudaEventRecord(c->ev_read, c->stream));
            maxima_done = true;
        } else {
            CUDA_OR_FAIL(c, cudaMemcpyAsync(c->aos, records, bytes, cudaMemcpyHostToDevice,
                                            c->stream));
            CUDA_OR_FAIL(c, cudaEventRecord(c->ev_read, c->stream));
            cdk::launch_aos_to_soa(c->aos, itemsize, offl, (int)n, c->body, c->col, c->stream);
            cdk::launch_states_in(c->aos, itemsize, so, (int)n, state_cols(c), c->stream);
        }
        c->states_dirty = false;
    }
    if (!maxima_done) {
        StepArgs a = args_of(c, 0);
        cdk::launch_scen_max(a, c->v0max, c->ext, c->max_partial, c->stream);
    }
    if (!maxima_done || !c->ext_host_dev)   // else the upload kernel wrote ext_host itself
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->ext_host, c->ext, sizeof(double) * c->nscen,
                                        cudaMemcpyDeviceToHost, c->stream));
    CUDA_OR_FAIL(c, cudaEventRecord(c->ev_ext, c->stream));
    CUDA_OR_FAIL(c, cudaGetLastError());
    c->ext_pending = true;
    c->have_records = true;
    // The caller may reuse `records` once this returns: wait for the read of
    // them, not for the extent reduction behind it.
    if (n > 0 && wait_read) CUDA_OR_FAIL(c, cudaEventSynchronize(c->ev_read));
    // Wall bins depend on the agents' extent: the first upload sizes them.
    if (c->extent_max.empty())
        if (int rc = absorb_extent(c)) return rc;
    return CD_OK;
}
}  // namespace

int cd_download_agents(cd_ctx *c, void *records, int64_t n, int64_t itemsize, const int64_t *off) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (n != c->n || itemsize != c->itemsize || !off ||
        std::memcmp(off, c->off, sizeof(int64_t) * CD_F_COUNT) != 0)
        return fail(c, CD_ERR_INVALID_VALUE, "record layout differs from the upload");
    if (n == 0) return CD_OK;
    long long offl[CD_F_COUNT];
    for (int k = 0; k < CD_F_COUNT; ++k) offl[k] = off[k];
    if (c->states_dirty)
        cdk::launch_states_out(c->aos, itemsize, state_offsets(off, itemsize), (int)n,
                               state_cols(c), c->stream);
    void *dv = (c->direct_host && cdk::records_per_block(itemsize) > 0)
                   ? const_cast<void *>(device_view_of_host(records, n * itemsize))
                   : nullptr;
    if (dv) {
        // the download kernel also copies the status into status_host
        const cdk::StepStatus st{c->err, (c->nl_cap > 0 && c->n > 0) ? c->nl_off + c->n : nullptr,
                                 c->status_host_dev};
        cdk::launch_records_out(dv, c->aos, itemsize, offl, (int)n, c->body, c->col, c->stream,
                                st);
        if (!c->status_host_dev)
            if (int rc = enqueue_status(c)) return rc;
    } else {
        cdk::launch_soa_to_aos(c->aos, itemsize, offl, (int)n, c->body, c->col, c->stream);
        CUDA_OR_FAIL(c, cudaMemcpyAsync(records, c->aos, n * itemsize, cudaMemcpyDeviceToHost,
                                        c->stream));
        if (int rc = enqueue_status(c)) return rc;
    }
    CUDA_OR_FAIL(c, cudaGetLastError());
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    return check_device_error(c, true);
}

int cd_step_records(cd_ctx *c, void *records, int64_t n, int64_t itemsize, const int64_t *off,
                    int nodes, int64_t steps) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (steps < 0) return fail(c, CD_ERR_INVALID_VALUE, "negative step count");
    // everything enqueued at once: the records are read, stepped and written
    // back without the host waiting in between
    if (int rc = upload_records(c, records, n, itemsize, off, false)) return rc;
    if (int rc = cd_launch(c, nodes, steps)) return rc;
    return cd_download_agents(c, records, n, itemsize, off);
}

int cd_set_direct_host_access(cd_ctx *c, int enable) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    c->direct_host = enable != 0;
    return CD_OK;
}

int cd_snapshot_agents(cd_ctx *c, int slot, void *records, int64_t n, int64_t itemsize,
                       const int64_t *off, double *dt, double *time_tot) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (slot < 0 || slot >= CD_SNAPSHOT_SLOTS) return fail(c, CD_ERR_INVALID_VALUE, "bad slot");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (n != c->n || itemsize != c->itemsize || !off ||
        std::memcmp(off, c->off, sizeof(int64_t) * CD_F_COUNT) != 0)
        return fail(c, CD_ERR_INVALID_VALUE, "record layout differs from the upload");
    if (n > 0) {
        if (!records) return fail(c, CD_ERR_INVALID_VALUE, "records is NULL");
        long long offl[CD_F_COUNT];
        for (int k = 0; k < CD_F_COUNT; ++k) offl[k] = off[k];
        cdk::launch_soa_to_aos(c->aos, itemsize, offl, (int)n, c->body, c->col, c->stream);
        if (c->states_dirty)
            cdk::launch_states_out(c->aos, itemsize, state_offsets(off, itemsize), (int)n,
                                   state_cols(c), c->stream);
        CUDA_OR_FAIL(c, cudaMemcpyAsync(records, c->aos, n * itemsize, cudaMemcpyDeviceToHost,
                                        c->stream));
    }
    if (dt)
        CUDA_OR_FAIL(c, cudaMemcpyAsync(dt, c->dt, sizeof(double) * c->nscen,
                                        cudaMemcpyDeviceToHost, c->stream));
    if (time_tot)
        CUDA_OR_FAIL(c, cudaMemcpyAsync(time_tot, c->time_tot, sizeof(double) * c->nscen,
                                        cudaMemcpyDeviceToHost, c->stream));
    CUDA_OR_FAIL(c, cudaEventRecord(c->evsnap[slot], c->stream));
    CUDA_OR_FAIL(c, cudaGetLastError());
    return CD_OK;
}

int cd_snapshot_wait(cd_ctx *c, int slot) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (slot < 0 || slot >= CD_SNAPSHOT_SLOTS) return fail(c, CD_ERR_INVALID_VALUE, "bad slot");
    CUDA_OR_FAIL(c, cudaEventSynchronize(c->evsnap[slot]));
    return CD_OK;
}

int cd_set_walls(cd_ctx *c, const double *walls, int64_t n_walls) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (n_walls != c->nw) return fail(c, CD_ERR_INVALID_VALUE, "wall count differs from the context");
    if (n_walls > 0 && !walls) return fail(c, CD_ERR_INVALID_VALUE, "walls is NULL");
    c->walls_host.assign(walls, walls + 4 * n_walls);
    if (n_walls > 0) {
        // float32 pre-check records relative to the wall's scenario grid
        // origin (the agents' records are relative to the same origin)
        std::vector<float4> wf((size_t)n_walls);
        for (const cd_scenario &sc : c->scen_host)
            for (int64_t w = sc.wall_begin; w < sc.wall_begin + sc.wall_count; ++w) {
                const double *p = walls + 4 * w;
                wf[w] = make_float4((float)(p[0] - sc.x0), (float)(p[1] - sc.y0),
                                    (float)(p[2] - sc.x0), (float)(p[3] - sc.y0));
            }
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->walls_raw, walls, sizeof(double) * 4 * n_walls,
                                        cudaMemcpyHostToDevice, c->stream));
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->walls_f, wf.data(), sizeof(float4) * n_walls,
                                        cudaMemcpyHostToDevice, c->stream));
        cdk::launch_wall_prep(c->walls_raw, c->walls, (int)n_walls, c->stream);
    }
    c->walls_dirty = true;
    CUDA_OR_FAIL(c, cudaGetLastError());
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    return CD_OK;
}

int cd_herding(cd_ctx *c, int with_herding, double sight_follower, int64_t size_nearest_other,
               double sight_leader, double phi, double w_herding, double w_leader,
               double w_direction) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (with_herding && (size_nearest_other < 1 || size_nearest_other > 16))
        return fail(c, CD_ERR_INVALID_VALUE, "size_nearest_other must be in [1, 16]");
    if (!(sight_follower > 0) || !std::isfinite(sight_follower) || !(sight_leader >= 0))
        return fail(c, CD_ERR_INVALID_VALUE, "bad sight");
    const int64_t n = c->n;
    if (n == 0) return CD_OK;
    cdk::launch_check_roles(state_cols(c), (int)n, c->err, c->stream);
    if (int rc = check_device_error(c)) return rc;
    const int K = with_herding ? (int)size_nearest_other : 1;
    const int64_t scan = cdk::scan_scratch_ints((int)n);
    if (!c->herd) {
        if (int rc = dalloc(c, &c->herd, 16 * n + 2 * (n + 1) + 2 * n + scan)) return rc;
        if (int rc = dalloc(c, &c->scen_h, c->nscen)) return rc;
    }
    int *nbr = c->herd, *flags = nbr + 16 * n, *pos = flags + (n + 1), *list = pos + (n + 1);
    int *before = list + n, *scratch = before + n;
    // herding grid: the scenario's origin, cells of the follower sight
    std::vector<ScenDev> hs(c->scen_dev);
    int64_t base = 0;
    for (int s = 0; s < c->nscen; ++s) {
        const cd_scenario &sc = c->scen_host[s];
        hs[s].cell = sight_follower;
        hs[s].nx = (int)std::max<int64_t>(1, (int64_t)std::ceil(sc.nx * sc.cell_size / sight_follower));
        hs[s].ny = (int)std::max<int64_t>(1, (int64_t)std::ceil(sc.ny * sc.cell_size / sight_follower));
        hs[s].cell_base = (int)base;
        base += (int64_t)hs[s].nx * hs[s].ny;
    }
    if (with_herding && base > c->ncells)
        return fail(c, CD_ERR_CAPACITY, "follower sight smaller than the cell size");
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->scen_h, hs.data(), sizeof(ScenDev) * c->nscen,
                                    cudaMemcpyHostToDevice, c->stream));
    StepArgs a = args_of(c, 0);
    a.scen = c->scen_h;
    if (with_herding) enqueue_cells(c, a);                   // cell list on the herding grid
    cdk::HerdArgs h;
    h.n = (int)n;
    h.K = K;
    h.with_herding = with_herding ? 1 : 0;
    h.perm = c->perm;
    h.key = c->key;
    h.start = c->start;
    h.scen_of = c->scen_of;
    h.scen_h = c->scen_h;
    for (int k = 0; k < cdk::NCOL; ++k) h.col[k] = c->col[k];
    h.walls = c->walls;
    h.st = state_cols(c);
    h.nbr = nbr;
    h.leaders = list;
    h.n_leaders = pos + n;
    h.tgt_before = before;
    h.sight_f = sight_follower;
    h.sight_l = sight_leader;
    h.cos_phi = cdm_cos(phi);
    h.w_herd = w_herding;
    h.w_lead = w_leader;
    h.w_dir = w_direction;
    cdk::launch_herd_neighbors(h, c->stream);
    cdk::launch_leaders(h, flags, pos, scratch, list, c->stream);
    cdk::launch_herd_follow(h, c->stream);
    c->states_dirty = true;
    CUDA_OR_FAIL(c, cudaGetLastError());
    return check_device_error(c);
}

namespace {
int upload_polygons(cd_ctx *c, int64_t n_polys, const double *xy, const int64_t *voff) {
    const int64_t nv = voff[n_polys];
    if (nv < 0 || nv > INT32_MAX) return fail(c, CD_ERR_INVALID_VALUE, "bad vertex offsets");
    for (int64_t t = 0; t < n_polys; ++t)
        if (voff[t + 1] < voff[t]) return fail(c, CD_ERR_INVALID_VALUE, "bad vertex offsets");
    if (nv + n_polys + 1 > c->poly_cap) {
        if (c->polys) cudaFree(c->polys);
        if (c->poly_off) cudaFree(c->poly_off);
        c->polys = nullptr;
        c->poly_off = nullptr;
        c->poly_cap = 0;
        if (int rc = dalloc(c, &c->polys, nv + 1)) return rc;
        if (int rc = dalloc(c, &c->poly_off, nv + n_polys + 2)) return rc;
        c->poly_cap = nv + n_polys + 1;
    }
    std::vector<int> off(voff, voff + n_polys + 1);
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->polys, xy, sizeof(double) * 2 * nv, cudaMemcpyHostToDevice,
                                    c->stream));
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->poly_off, off.data(), sizeof(int) * off.size(),
                                    cudaMemcpyHostToDevice, c->stream));
    if (!c->counters)
        if (int rc = dalloc(c, &c->counters, 1 + 256)) return rc;
    return CD_OK;
}
}  // namespace

int cd_inside_domain(cd_ctx *c, int64_t scenario, const double *xy, int64_t n_vertices,
                     int64_t *changed) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (scenario < 0 || scenario >= c->nscen) return fail(c, CD_ERR_INVALID_VALUE, "bad scenario");
    if (n_vertices < 1 || !xy) return fail(c, CD_ERR_INVALID_VALUE, "empty polygon");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    const int64_t voff[2] = {0, n_vertices};
    if (int rc = upload_polygons(c, 1, xy, voff)) return rc;
    CUDA_OR_FAIL(c, cudaMemsetAsync(c->counters, 0, sizeof(unsigned long long), c->stream));
    const cd_scenario &sc = c->scen_host[scenario];
    cdk::launch_inside_domain((int)sc.agent_begin, (int)sc.agent_count, c->col[cdk::X],
                              c->col[cdk::Y], state_cols(c).active, c->polys, (int)n_vertices,
                              c->counters, c->stream);
    unsigned long long h = 0;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(&h, c->counters, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    c->states_dirty = true;
    if (changed) *changed = (int64_t)h;
    return check_device_error(c);
}

int cd_exit_detection(cd_ctx *c, int64_t scenario, const double *centers, int64_t n_doors,
                      double detection_range) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (scenario < 0 || scenario >= c->nscen) return fail(c, CD_ERR_INVALID_VALUE, "bad scenario");
    if (n_doors < 0 || (n_doors > 0 && !centers))
        return fail(c, CD_ERR_INVALID_VALUE, "bad door centres");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (n_doors == 0) return CD_OK;
    std::vector<int64_t> voff = {0, n_doors};
    if (int rc = upload_polygons(c, 1, centers, voff.data())) return rc;
    const cd_scenario &sc = c->scen_host[scenario];
    cdk::launch_exit_detection((int)sc.agent_begin, (int)sc.agent_count, c->col[cdk::X],
                               c->col[cdk::Y], c->walls, (int)sc.wall_begin, (int)sc.wall_count,
                               c->polys, (int)n_doors, detection_range, state_cols(c), c->stream);
    c->states_dirty = true;
    CUDA_OR_FAIL(c, cudaGetLastError());
    return check_device_error(c);
}

int cd_target_reached(cd_ctx *c, int64_t scenario, int64_t n_targets, const double *xy,
                      const int64_t *vertex_offsets, int reset, int64_t *counts) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (scenario < 0 || scenario >= c->nscen) return fail(c, CD_ERR_INVALID_VALUE, "bad scenario");
    if (n_targets < 0 || n_targets > 256) return fail(c, CD_ERR_INVALID_VALUE, "0-256 targets");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (n_targets == 0) return CD_OK;
    if (!xy || !vertex_offsets) return fail(c, CD_ERR_INVALID_VALUE, "NULL polygons");
    if (int rc = upload_polygons(c, n_targets, xy, vertex_offsets)) return rc;
    const int64_t n = std::max<int64_t>(c->n, 1);
    if (n_targets > c->reached_targets) {
        if (c->reached) cudaFree(c->reached);
        c->reached = nullptr;
        c->reached_targets = 0;
        if (int rc = dalloc(c, &c->reached, n_targets * n)) return rc;
        CUDA_OR_FAIL(c, cudaMemsetAsync(c->reached, 0, n_targets * n, c->stream));
        c->reached_targets = n_targets;
    } else if (reset) {
        CUDA_OR_FAIL(c, cudaMemsetAsync(c->reached, 0, n_targets * n, c->stream));
    }
    CUDA_OR_FAIL(c, cudaMemsetAsync(c->counters + 1, 0, sizeof(unsigned long long) * n_targets,
                                    c->stream));
    const cd_scenario &sc = c->scen_host[scenario];
    for (int t = 0; t < n_targets; ++t)
        cdk::launch_target_reached((int)sc.agent_begin, (int)sc.agent_count, c->col[cdk::X],
                                   c->col[cdk::Y], c->reached + (size_t)t * n + sc.agent_begin,
                                   c->polys, c->poly_off, t, c->counters + 1, c->stream);
    std::vector<unsigned long long> h(n_targets);
    CUDA_OR_FAIL(c, cudaMemcpyAsync(h.data(), c->counters + 1, sizeof(unsigned long long) * n_targets,
                                    cudaMemcpyDeviceToHost, c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    if (counts)
        for (int64_t t = 0; t < n_targets; ++t) counts[t] = (int64_t)h[t];
    return check_device_error(c);
}

int cd_set_direction_maps(cd_ctx *c, int64_t scenario, int64_t n_targets, const double *dir_x,
                          const double *dir_y, int64_t ny, int64_t nx, double minx, double miny,
                          double step) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (scenario < 0 || scenario >= c->nscen) return fail(c, CD_ERR_INVALID_VALUE, "bad scenario");
    if (n_targets < 0) return fail(c, CD_ERR_INVALID_VALUE, "negative target count");
    if (n_targets > 0) {
        if (!dir_x || !dir_y) return fail(c, CD_ERR_INVALID_VALUE, "NULL direction map");
        if (nx < 1 || ny < 1 || nx > INT32_MAX || ny > INT32_MAX || n_targets > INT32_MAX)
            return fail(c, CD_ERR_INVALID_VALUE, "bad direction map shape");
        if (!(step > 0) || !std::isfinite(step) || !std::isfinite(minx) || !std::isfinite(miny))
            return fail(c, CD_ERR_INVALID_VALUE, "bad meshgrid origin or step");
    }
    const int64_t cells = n_targets * ny * nx;
    std::vector<double> &h = c->nav_host[scenario];
    h.assign(dir_x, dir_x + (n_targets > 0 ? cells : 0));
    if (n_targets > 0) h.insert(h.end(), dir_y, dir_y + cells);
    ScenDev &d = c->scen_dev[scenario];
    d.nav_targets = (int)n_targets;
    d.nav_nx = n_targets > 0 ? (int)nx : 0;
    d.nav_ny = n_targets > 0 ? (int)ny : 0;
    d.nav_x0 = minx;
    d.nav_y0 = miny;
    d.nav_step = n_targets > 0 ? step : 1.0;
    // rebuild the interleaved device copy of every scenario's maps
    std::vector<double> all;
    for (int s = 0; s < c->nscen; ++s) {
        ScenDev &e = c->scen_dev[s];
        e.nav_off = (long long)(all.size() / 2);
        const std::vector<double> &m = c->nav_host[s];
        const size_t k = m.size() / 2;
        for (size_t q = 0; q < k; ++q) {
            all.push_back(m[q]);
            all.push_back(m[k + q]);
        }
    }
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    if (c->navmap) cudaFree(c->navmap);
    c->navmap = nullptr;
    if (!all.empty()) {
        if (int rc = dalloc(c, &c->navmap, (int64_t)(all.size() / 2))) return rc;
        CUDA_OR_FAIL(c, cudaMemcpy(c->navmap, all.data(), sizeof(double) * all.size(),
                                   cudaMemcpyHostToDevice));
    }
    CUDA_OR_FAIL(c, cudaMemcpy(c->scen, c->scen_dev.data(), sizeof(ScenDev) * c->nscen,
                               cudaMemcpyHostToDevice));
    drop_graph(c);
    return CD_OK;
}

int cd_set_noise_mode(cd_ctx *c, int device, uint64_t seed, uint64_t step) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    const bool dev = device != 0;
    if (dev != c->noise_dev || (dev && seed != c->noise_seed)) {
        drop_graph(c);
    }
    c->noise_dev = dev;
    c->noise_seed = seed;
    const unsigned long long st = step;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->rng_step, &st, sizeof st, cudaMemcpyHostToDevice, c->stream));
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    return CD_OK;
}

int cd_set_noise(cd_ctx *c, const double *force, const double *torque) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (c->n > 0 && !force) return fail(c, CD_ERR_INVALID_VALUE, "force noise is NULL");
    if (c->n > 0) {
        CUDA_OR_FAIL(c, cudaMemcpyAsync(c->noise_f, force, sizeof(double) * 2 * c->n,
                                        cudaMemcpyHostToDevice, c->stream));
        if (torque)
            CUDA_OR_FAIL(c, cudaMemcpyAsync(c->noise_m, torque, sizeof(double) * c->n,
                                            cudaMemcpyHostToDevice, c->stream));
        else
            CUDA_OR_FAIL(c, cudaMemsetAsync(c->noise_m, 0, sizeof(double) * c->n, c->stream));
    }
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    c->noise_pending = true;
    return CD_OK;
}

int cd_step(cd_ctx *c, int nodes, double *dt) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (int rc = prepare_step(c, nodes)) return rc;
    if ((nodes & CD_NODE_FLUCTUATION) && !c->noise_dev && !c->noise_pending)
        return fail(c, CD_ERR_INVALID_VALUE, "cd_set_noise must precede a step with fluctuation");
    enqueue_step(c, nodes, c->timing != 0);
    if ((nodes & CD_NODE_FLUCTUATION) && !c->noise_dev) c->noise_pending = false;
    CUDA_OR_FAIL(c, cudaGetLastError());
    if (c->timing) {
        CUDA_OR_FAIL(c, cudaEventSynchronize(c->evs1));
        float ms = 0, sms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        cudaEventElapsedTime(&sms, c->evs0, c->evs1);
        c->force_ms += ms;
        c->step_ms += sms;
        c->launches += 1;
        add_pair_time(c, nodes);
    }
    if (dt) {
        if (int rc = check_device_error(c)) return rc;
        CUDA_OR_FAIL(c, cudaMemcpy(dt, c->dt, sizeof(double) * c->nscen, cudaMemcpyDeviceToHost));
    }
    return CD_OK;
}

namespace {
// Capture (or reuse) the graph of one step with `nodes`.
int ensure_graph(cd_ctx *c, int nodes) {
    if ((nodes & CD_NODE_FLUCTUATION) && !c->noise_dev)
        return fail(c, CD_ERR_INVALID_VALUE,
                    "graph steps cannot consume per-step host noise (use device noise)");
    if (int rc = prepare_step(c, nodes)) return rc;
    if (!c->graph || c->graph_nodes != nodes) {
        drop_graph(c);
        cudaGraph_t g;
        CUDA_OR_FAIL(c, cudaGetLastError());
        CUDA_OR_FAIL(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(c, nodes, false, true);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return fail(c, CD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(c, CD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        c->graph_nodes = nodes;
    }
    return CD_OK;
}
}  // namespace

int cd_launch(cd_ctx *c, int nodes, int64_t steps) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (steps < 0) return fail(c, CD_ERR_INVALID_VALUE, "negative step count");
    if (int rc = ensure_graph(c, nodes)) return rc;
    for (int64_t k = 0; k < steps; ++k) CUDA_OR_FAIL(c, cudaGraphLaunch(c->graph, c->stream));
    CUDA_OR_FAIL(c, cudaGetLastError());
    return CD_OK;
}

int cd_run(cd_ctx *c, int nodes, int64_t steps) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (steps < 0) return fail(c, CD_ERR_INVALID_VALUE, "negative step count");
    if (int rc = ensure_graph(c, nodes)) return rc;
    if (c->timing) cudaEventRecord(c->evr0, c->stream);
    for (int64_t k = 0; k < steps; ++k) CUDA_OR_FAIL(c, cudaGraphLaunch(c->graph, c->stream));
    CUDA_OR_FAIL(c, cudaGetLastError());
    if (c->timing) {
        cudaEventRecord(c->evr1, c->stream);
        CUDA_OR_FAIL(c, cudaEventSynchronize(c->evr1));
        float ms = 0;
        cudaEventElapsedTime(&ms, c->evr0, c->evr1);
        c->run_ms += ms;
        c->run_steps += steps;
        if (steps == 1 && c->timing == 1) {   // the graph's own events bracket its force stage
            float fms = 0;
            cudaEventElapsedTime(&fms, c->ev0, c->ev1);
            c->force_ms += fms;
            c->launches += 1;
            add_pair_time(c, nodes);
        }
    }
    return check_device_error(c);
}

int cd_synchronize(cd_ctx *c) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int cd_get_time(cd_ctx *c, double *dt, double *time_tot) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    if (dt) CUDA_OR_FAIL(c, cudaMemcpy(dt, c->dt, sizeof(double) * c->nscen, cudaMemcpyDeviceToHost));
    if (time_tot)
        CUDA_OR_FAIL(c, cudaMemcpy(time_tot, c->time_tot, sizeof(double) * c->nscen, cudaMemcpyDeviceToHost));
    return CD_OK;
}

int cd_get_cell_list(cd_ctx *c, int64_t *keys, int64_t *order, int64_t *cells_count,
                     int64_t *cells_offset) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
    std::vector<int> k(std::max<int64_t>(c->n, 1)), p(std::max<int64_t>(c->n, 1)),
        st((size_t)c->ncells + 1);
    CUDA_OR_FAIL(c, cudaMemcpy(k.data(), c->key, sizeof(int) * c->n, cudaMemcpyDeviceToHost));
    CUDA_OR_FAIL(c, cudaMemcpy(p.data(), c->perm, sizeof(int) * c->n, cudaMemcpyDeviceToHost));
    CUDA_OR_FAIL(c, cudaMemcpy(st.data(), c->start, sizeof(int) * (c->ncells + 1), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < c->n; ++i) {
        int s = c->scen_of_host[i];
        if (keys) keys[i] = k[i] - c->scen_dev[s].cell_base;
        if (order) order[i] = p[i];
    }
    for (int64_t q = 0; q < c->ncells; ++q) {
        if (cells_count) cells_count[q] = st[q + 1] - st[q];
        if (cells_offset) cells_offset[q] = st[q];
    }
    return CD_OK;
}

static_assert(CD_COUNT_COLS == cdk::COUNT_COLS, "count columns differ");

int cd_pair_counts(cd_ctx *c, int64_t *counts) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (!c->have_records) return fail(c, CD_ERR_INVALID_VALUE, "no agents uploaded");
    if (int rc = absorb_extent(c)) return rc;
    if (c->walls_dirty && c->nw > 0) {
        if (c->walls_host.empty())
            return fail(c, CD_ERR_INVALID_VALUE, "walls declared but cd_set_walls not called");
        if (int rc = bin_walls(c)) return rc;
    }
    StepArgs a = args_of(c, CD_NODE_AGENT_AGENT | CD_NODE_AGENT_OBSTACLE);
    enqueue_cells(c, a);
    cdk::launch_pair_counts(a, c->diag, c->stream);
    CUDA_OR_FAIL(c, cudaGetLastError());
    if (int rc = check_device_error(c)) return rc;
    std::vector<int> h((size_t)CD_COUNT_COLS * std::max<int64_t>(c->n, 1));
    CUDA_OR_FAIL(c, cudaMemcpy(h.data(), c->diag, sizeof(int) * CD_COUNT_COLS * c->n,
                               cudaMemcpyDeviceToHost));
    if (counts)
        for (int64_t k = 0; k < (int64_t)CD_COUNT_COLS * c->n; ++k) counts[k] = h[k];
    return CD_OK;
}

int cd_sizes(const cd_ctx *c, int64_t *n_agents, int64_t *n_walls, int64_t *n_cells) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (n_agents) *n_agents = c->n;
    if (n_walls) *n_walls = c->nw;
    if (n_cells) *n_cells = c->ncells;
    return CD_OK;
}

int cd_set_timing(cd_ctx *c, int enable) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (enable < 0 || enable > 2) return fail(c, CD_ERR_INVALID_VALUE, "timing mode must be 0, 1 or 2");
    // the step graph holds kernel events only in mode 1
    if ((enable == 1) != (c->timing == 1)) drop_graph(c);
    c->timing = enable;
    c->force_ms = c->step_ms = c->run_ms = c->pair_ms = c->light_ms = 0;
    c->launches = c->run_steps = c->pair_launches = 0;
    return CD_OK;
}

int cd_pair_kernel_time(cd_ctx *c, double *ms, int64_t *launches) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (ms) *ms = c->pair_ms;
    if (launches) *launches = c->pair_launches;
    return CD_OK;
}

int cd_pair_kernel_times(cd_ctx *c, double *light_ms, double *pairs_ms, int64_t *launches) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (light_ms) *light_ms = c->light_ms;
    if (pairs_ms) *pairs_ms = c->pair_ms - c->light_ms;
    if (launches) *launches = c->pair_launches;
    return CD_OK;
}

int cd_pair_split(cd_ctx *c, int64_t *pairs, int64_t *first_part, int64_t *deferred) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    int v[3] = {0, 0, 0};
    if (c->n > 0 && c->nl_cap > 0) {
        CUDA_OR_FAIL(c, cudaStreamSynchronize(c->stream));
        CUDA_OR_FAIL(c, cudaMemcpy(&v[0], c->fw_off + c->n, sizeof(int), cudaMemcpyDeviceToHost));
        CUDA_OR_FAIL(c, cudaMemcpy(&v[1], c->fs_off + c->n, sizeof(int), cudaMemcpyDeviceToHost));
        if (c->defer_list)
            CUDA_OR_FAIL(c, cudaMemcpy(&v[2], c->work + 1, sizeof(int), cudaMemcpyDeviceToHost));
    }
    if (pairs) *pairs = v[0];
    if (first_part) *first_part = v[1];
    if (deferred) *deferred = v[2];
    return CD_OK;
}

int cd_kernel_time(cd_ctx *c, double *force_ms, int64_t *force_launches, double *step_ms,
                   double *run_ms, int64_t *run_steps) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (force_ms) *force_ms = c->force_ms;
    if (force_launches) *force_launches = c->launches;
    if (step_ms) *step_ms = c->step_ms;
    if (run_ms) *run_ms = c->run_ms;
    if (run_steps) *run_steps = c->run_steps;
    return CD_OK;
}

int cd_variant_count(int *count) {
    if (!count) return fail(nullptr, CD_ERR_INVALID_VALUE, "count is NULL");
    *count = cdk::N_VARIANTS;
    return CD_OK;
}

int cd_variant_shape(int variant, int *threads, int *staged, int *lanes, int *pairs) {
    if (variant < 0 || variant >= cdk::N_VARIANTS)
        return fail(nullptr, CD_ERR_INVALID_VALUE, "unknown variant");
    if (threads) *threads = cdk::variant_threads(variant);
    if (staged) *staged = cdk::variant_staged(variant);
    if (lanes) *lanes = cdk::variant_lanes(variant);
    if (pairs) *pairs = cdk::variant_pairs(variant) ? 1 : 0;
    return CD_OK;
}

int cd_set_near_list_capacity(cd_ctx *c, int64_t entries) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (entries < 0) {                  // grow from the current capacity when a step needs more
        c->nl_fixed = false;
        return CD_OK;
    }
    if (entries > (int64_t)INT32_MAX / 8)
        return fail(c, CD_ERR_CAPACITY, "near-list capacity above 2^28 entries");
    c->nl_fixed = true;
    return alloc_near_lists(c, entries);
}

int cd_set_variant(cd_ctx *c, int variant) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (variant < 0 || variant >= cdk::N_VARIANTS)
        return fail(c, CD_ERR_INVALID_VALUE, "unknown variant");
    if (variant != c->variant) drop_graph(c);
    c->variant = variant;
    return CD_OK;
}

int cd_kernels_per_step(const cd_ctx *c, int nodes, int64_t *kernels) {
    if (!c || !kernels) return fail(nullptr, CD_ERR_INVALID_VALUE, "NULL argument");
    *kernels = kernels_per_step(c, nodes);
    return CD_OK;
}

int cd_measure_fp64_peak(double *gflops) {
    if (!gflops) return fail(nullptr, CD_ERR_INVALID_VALUE, "gflops is NULL");
    double g = cdk::fp64_peak_gflops();
    if (g <= 0) return fail(nullptr, CD_ERR_CUDA, "FP64 peak measurement failed");
    *gflops = g;
    return CD_OK;
}

}  // extern "C"


// ---- differentiable rollout ------------------------------------------------

namespace {

// State snapshot: columns x, y, vx, vy, fpx, fpy of n agents.
// State a step reads: positions, velocities, previous and current force (the
// current force is zero after a reset, the array's own value before step 0).
constexpr int SNAP_COLS = 8;
constexpr int kSnapCol[SNAP_COLS] = {cdk::X,   cdk::Y,   cdk::VX, cdk::VY,
                                     cdk::FPX, cdk::FPY, cdk::FX, cdk::FY};

int copy_state(cd_ctx *c, double *snap, bool save, bool dep = false) {
    const double *src[SNAP_COLS];
    double *dst[SNAP_COLS];
    for (int k = 0; k < SNAP_COLS; ++k) {
        double *col = c->col[kSnapCol[k]], *buf = snap + (size_t)k * c->n;
        src[k] = save ? col : buf;
        dst[k] = save ? buf : col;
    }
    cdk::launch_copy_cols(src, dst, SNAP_COLS, (int)c->n, c->stream, dep);
    return CD_OK;
}

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf() { for (void *p : ptrs) cudaFree(p); }
    template <typename T> T *get(cd_ctx *c, int64_t count, int &rc) {
        void *p = nullptr;
        if (rc == CD_OK) rc = dalloc(c, reinterpret_cast<T **>(&p), count);
        if (p) ptrs.push_back(p);
        return static_cast<T *>(p);
    }
};

// The step structures a reverse step reads (cell list, staged records, near
// lists, flat pair list) as the recomputation context builds them for the
// state before each step of a segment: kept per step, the reverse pass takes
// them instead of building them again.
enum { SN_KEY, SN_PERM, SN_START, SN_STAGE, SN_CULL, SN_STAGEF, SN_NLOFF, SN_NLFWD, SN_FWOFF,
       SN_FSOFF, SN_NLIDX, SN_FWPAIRS, SN_COUNT };
struct StepSnapLayout {
    long long off[SN_COUNT], bytes[SN_COUNT], total;
};

StepSnapLayout snap_layout(const cd_ctx *b) {
    const long long n = std::max<int64_t>(b->n, 1), cells = b->ncells + 1, cap = b->nl_cap;
    const long long sq = b->body == CD_BODY_CIRCULAR ? cdk::STAGE_Q_CIRC : cdk::STAGE_Q_TC;
    // (fw_pairs: at most cap / 2 pairs of two ints)
    const long long bytes[SN_COUNT] = {4 * n,       4 * n,       4 * cells,   16 * sq * n,
                                       16 * n,      32 * n,      4 * (n + 1), 4 * n,
                                       4 * (n + 1), 4 * (n + 1), 4 * cap,     4 * cap};
    StepSnapLayout L;
    long long o = 0;
    for (int k = 0; k < SN_COUNT; ++k) {
        L.off[k] = o;
        L.bytes[k] = bytes[k];
        o += (bytes[k] + 255) / 256 * 256;
    }
    L.total = o;
    return L;
}

void snap_step(const cd_ctx *b, const StepSnapLayout &L, char *dst) {
    const void *src[SN_COUNT] = {b->key,    b->perm,   b->start,  b->stage,  b->cull,   b->stage_f,
                                 b->nl_off, b->nl_fwd, b->fw_off, b->fs_off, b->nl_idx, b->fw_pairs};
    void *to[SN_COUNT];
    for (int k = 0; k < SN_COUNT; ++k) to[k] = dst + L.off[k];
    cdk::launch_copy_bufs(src, to, L.bytes, SN_COUNT, b->stream);
}

// The reverse step's structures from a snapshot (c's own buffers for what it
// writes: entry records and kinds, the deferred list, the work counters).
void snap_args(StepArgs &a, const StepSnapLayout &L, char *sp, int64_t cap) {
    a.key = reinterpret_cast<int *>(sp + L.off[SN_KEY]);
    a.perm = reinterpret_cast<int *>(sp + L.off[SN_PERM]);
    a.start = reinterpret_cast<int *>(sp + L.off[SN_START]);
    a.stage = reinterpret_cast<double2 *>(sp + L.off[SN_STAGE]);
    a.cull = reinterpret_cast<float4 *>(sp + L.off[SN_CULL]);
    a.stage_f = reinterpret_cast<float4 *>(sp + L.off[SN_STAGEF]);
    a.nl_off = reinterpret_cast<int *>(sp + L.off[SN_NLOFF]);
    a.nl_fwd = reinterpret_cast<int *>(sp + L.off[SN_NLFWD]);
    a.fw_off = reinterpret_cast<int *>(sp + L.off[SN_FWOFF]);
    a.fs_off = reinterpret_cast<int *>(sp + L.off[SN_FSOFF]);
    a.nl_idx = reinterpret_cast<int *>(sp + L.off[SN_NLIDX]);
    a.fw_pairs = reinterpret_cast<int2 *>(sp + L.off[SN_FWPAIRS]);
    a.nl_cap = (int)cap;
}

// The adjoint's recomputation context: a copy of `c` (scenarios, walls,
// agent records, launch variant) with its own buffers, stream and step graph,
// so that the forward steps of one checkpoint segment are recomputed on its
// stream while `c` runs the reverse pass of the segment after it.  Made on
// first use; before each rollout its walls, wall bins and variant follow c's
// (the same bins, so its steps are bit-identical to c's), and the rollout
// copies c's columns, timestep maxima and agent states into it.
int sync_shadow(cd_ctx *c, int nodes) {
    cd_ctx *b = c->shadow;
    if (!b) {
        if (cd_create(&b, c->body, c->nscen, c->scen_host.data()) != CD_OK)
            return fail(c, CD_ERR_CUDA,
                        std::string("recomputation context: ") + cd_last_error(nullptr));
        std::vector<char> rec((size_t)(c->n * c->itemsize));
        int rc = cd_download_agents(c, rec.data(), c->n, c->itemsize, c->off);
        if (rc == CD_OK && cd_upload_agents(b, rec.data(), c->n, c->itemsize, c->off) != CD_OK)
            rc = fail(c, CD_ERR_CUDA, std::string("recomputation context: ") + cd_last_error(b));
        if (rc != CD_OK) {                      // no half-made context is kept
            cd_destroy(b);
            return rc;
        }
        c->shadow = b;
    }
    if (c->nw > 0 && b->walls_host != c->walls_host)
        if (cd_set_walls(b, c->walls_host.data(), c->nw) != CD_OK)
            return fail(c, CD_ERR_CUDA, std::string("recomputation context: ") + cd_last_error(b));
    if (int rc = absorb_extent(c)) return rc;
    if (int rc = absorb_extent(b)) return fail(c, rc, cd_last_error(b));
    if (b->extent_max != c->extent_max) {
        b->extent_max = c->extent_max;
        b->walls_dirty = true;
    }
    if (b->variant != c->variant && cd_set_variant(b, c->variant) != CD_OK)
        return fail(c, CD_ERR_CUDA, std::string("recomputation context: ") + cd_last_error(b));
    if (ensure_graph(b, nodes) != CD_OK)
        return fail(c, CD_ERR_CUDA, std::string("recomputation context: ") + cd_last_error(b));
    return CD_OK;
}

}  // namespace

extern "C" int cd_rollout_loss(cd_ctx *c, int64_t steps, const double *target, int64_t ckpt,
                               double *loss, double *grads, double *forward_ms, double *adjoint_ms) {
    if (!c) return fail(nullptr, CD_ERR_INVALID_VALUE, "ctx is NULL");
    if (c->body != CD_BODY_CIRCULAR)
        return fail(c, CD_ERR_INVALID_TYPE, "the adjoint covers Circular agents only");
    if (c->nscen != 1) return fail(c, CD_ERR_INVALID_VALUE, "the adjoint covers one scenario");
    if (steps < 1 || ckpt < 1 || !target || !loss)
        return fail(c, CD_ERR_INVALID_VALUE, "bad rollout arguments");
    const int nodes = CD_NODE_ADJUSTING | CD_NODE_AGENT_AGENT | CD_NODE_AGENT_OBSTACLE |
                      CD_NODE_INTEGRATE | CD_NODE_RESET;
    const int64_t n = c->n;
    if (forward_ms) *forward_ms = 0.0;
    if (adjoint_ms) *adjoint_ms = 0.0;
    if (n == 0) {                                  // nothing to differentiate: plain steps
        *loss = 0.0;
        return cd_run(c, nodes, steps);
    }
    ckpt = std::min(ckpt, steps);
    if (grads)                                      // near-list entries for the reverse pass
        if (int rc = size_near_lists(c)) return rc;  // (before the graph: sizing drops it)
    if (int rc = ensure_graph(c, nodes)) return rc;
    if (grads)
        if (int rc = sync_shadow(c, nodes)) return rc;
    const int64_t nseg = (steps + ckpt - 1) / ckpt;
    const size_t snap = (size_t)SNAP_COLS * (size_t)std::max<int64_t>(n, 1);
    int rc = CD_OK;
    DevBuf mem;
    double *tgt = mem.get<double>(c, steps * 2 * n, rc);
    double *ck = mem.get<double>(c, nseg * snap, rc);
    // two segment buffers: one being recomputed, one being reversed
    double *segbuf = grads ? mem.get<double>(c, 2 * (ckpt + 1) * snap, rc) : nullptr;
    // and, where the recomputation builds near lists, each step's structures
    // (up to 8 GiB; beyond, the reverse pass builds them itself)
    const cd_ctx *shadow = grads ? c->shadow : nullptr;
    const bool keep_steps = shadow && shadow->nl_cap > 0 && cdk::variant_pairs(shadow->variant) &&
                            c->nl_cnt && c->nl_cap > 0;
    const StepSnapLayout snl = keep_steps ? snap_layout(shadow) : StepSnapLayout{};
    const bool use_snaps = keep_steps && 2 * ckpt * snl.total <= (8LL << 30);
    char *snapbuf = use_snaps ? mem.get<char>(c, 2 * ckpt * snl.total, rc) : nullptr;
    double *fin = mem.get<double>(c, snap, rc);
    double *dts = mem.get<double>(c, steps, rc);
    double *partial = mem.get<double>(c, cdk::adj_partials((int)n), rc);
    double *scal = mem.get<double>(c, 4, rc);           // loss, ldt, saved dt, saved time
    int *blocks_done = mem.get<int>(c, 1, rc);          // the reductions' last-block counter
    double *adj = grads ? mem.get<double>(c, 16 * n + 4 * n, rc) : nullptr;
    // per block of the argmax: (max |v|, max v0) and their first indices
    int *amax = grads ? mem.get<int>(c, 2 * cdk::adj_partials((int)n), rc) : nullptr;
    double *avals = grads ? mem.get<double>(c, 2 * cdk::adj_partials((int)n), rc) : nullptr;
    if (rc) return rc;
    cudaStream_t st = c->stream;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(tgt, target, sizeof(double) * steps * 2 * n,
                                    cudaMemcpyHostToDevice, st));
    CUDA_OR_FAIL(c, cudaMemsetAsync(scal, 0, sizeof(double) * 4, st));
    CUDA_OR_FAIL(c, cudaMemsetAsync(blocks_done, 0, sizeof(int), st));
    const double scale = 1.0 / ((double)steps * (double)std::max<int64_t>(n, 1));
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaEventRecord(e0, st);
    // forward rollout with checkpoints and the loss
    for (int64_t t = 0; t < steps; ++t) {
        if (t % ckpt == 0)
            if ((rc = copy_state(c, ck + (size_t)(t / ckpt) * snap, true))) break;
        CUDA_OR_FAIL(c, cudaGraphLaunch(c->graph, st));
        // the loss term of the step, and its dt kept for the reverse pass
        cdk::launch_loss(c->col[cdk::X], c->col[cdk::Y], tgt + (size_t)t * 2 * n, (int)n, partial,
                         scal, scale, blocks_done, c->dt, dts + t, st);
    }
    if (rc) return rc;
    if ((rc = copy_state(c, fin, true))) return rc;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(scal + 2, c->dt, sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_OR_FAIL(c, cudaMemcpyAsync(scal + 3, c->time_tot, sizeof(double), cudaMemcpyDeviceToDevice, st));
    cudaEventRecord(e1, st);
    if (grads) {
        double *lx = adj, *lv = adj + 2 * n, *lfp = adj + 4 * n, *lF = adj + 6 * n;
        double *lvt = adj + 8 * n, *lfp2 = adj + 10 * n, *lx2 = adj + 12 * n, *lv2 = adj + 14 * n;
        double *g = adj + 16 * n;
        CUDA_OR_FAIL(c, cudaMemsetAsync(adj, 0, sizeof(double) * (16 * n + 4 * n), st));
        const int fnodes = CD_NODE_ADJUSTING | CD_NODE_AGENT_AGENT | CD_NODE_AGENT_OBSTACLE;
        const cd_scenario &sc = c->scen_host[0];
        // The recomputation context takes this rollout's parameters and agent
        // states; each checkpoint segment's forward steps are recomputed on
        // its stream into one of two segment buffers while this stream
        // reverses the segment after it from the other buffer.
        cd_ctx *b = c->shadow;
        const int64_t npad = std::max<int64_t>(n, 1);
        CUDA_OR_FAIL(c, cudaMemcpyAsync(b->colbuf, c->colbuf, sizeof(double) * npad * cdk::NCOL,
                                        cudaMemcpyDeviceToDevice, st));
        CUDA_OR_FAIL(c, cudaMemcpyAsync(b->v0max, c->v0max, sizeof(double) * c->nscen,
                                        cudaMemcpyDeviceToDevice, st));
        CUDA_OR_FAIL(c, cudaMemcpyAsync(b->states, c->states, sizeof(int) * 5 * npad,
                                        cudaMemcpyDeviceToDevice, st));
        cudaEvent_t ev_sync, ev_rec[2], ev_rev[2];
        cudaEventCreateWithFlags(&ev_sync, cudaEventDisableTiming);
        for (int k = 0; k < 2; ++k) {
            cudaEventCreateWithFlags(&ev_rec[k], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ev_rev[k], cudaEventDisableTiming);
        }
        CUDA_OR_FAIL(c, cudaEventRecord(ev_sync, st));
        CUDA_OR_FAIL(c, cudaStreamWaitEvent(b->stream, ev_sync, 0));
        auto seg_of = [&](int64_t sgi) { return segbuf + (size_t)(sgi & 1) * (ckpt + 1) * snap; };
        auto recompute = [&](int64_t sgi) -> int {
            const int64_t t0 = sgi * ckpt, t1 = std::min<int64_t>(t0 + ckpt, steps);
            double *seg = seg_of(sgi);
            if (int e = copy_state(b, ck + (size_t)sgi * snap, false)) return e;
            for (int64_t t = t0; t < t1; ++t) {
                if (int e = copy_state(b, seg + (size_t)(t - t0) * snap, true)) return e;
                CUDA_OR_FAIL(c, cudaGraphLaunch(b->graph, b->stream));
                if (use_snaps)
                    snap_step(b, snl, snapbuf + ((size_t)(sgi & 1) * ckpt + (t - t0)) * snl.total);
            }
            if (int e = copy_state(b, seg + (size_t)(t1 - t0) * snap, true)) return e;
            CUDA_OR_FAIL(c, cudaEventRecord(ev_rec[sgi & 1], b->stream));
            return CD_OK;
        };
        rc = recompute(nseg - 1);
        for (int64_t sgi = nseg - 1; sgi >= 0 && rc == CD_OK; --sgi) {
            const int64_t t0 = sgi * ckpt, t1 = std::min<int64_t>(t0 + ckpt, steps);
            double *seg = seg_of(sgi);
            CUDA_OR_FAIL(c, cudaStreamWaitEvent(st, ev_rec[sgi & 1], 0));
            if (sgi > 0) {
                // the buffer of segment sgi - 1 held segment sgi + 1: reversed by now
                if (sgi + 1 < nseg) CUDA_OR_FAIL(c, cudaStreamWaitEvent(b->stream, ev_rev[(sgi + 1) & 1], 0));
                if ((rc = recompute(sgi - 1))) break;
            }
            for (int64_t t = t1 - 1; t >= t0; --t) {
                const double *after = seg + (size_t)(t + 1 - t0) * snap;
                // chained to the reverse step before it; the segment's first
                // reverse step follows a wait on the other stream
                if ((rc = copy_state(c, seg + (size_t)(t - t0) * snap, false, t != t1 - 1))) break;
                StepArgs a = args_of(c, fnodes);
                if (use_snaps) {
                    // the recomputation's cell list and near lists of the state before step t
                    snap_args(a, snl, snapbuf + ((size_t)(sgi & 1) * ckpt + (t - t0)) * snl.total,
                              std::min<int64_t>(c->nl_cap, shadow->nl_cap));
                    // the work counters are zeroed by k_adj_seed (k_nl_fill does not run)
                } else {
                    enqueue_cells(c, a);                    // cell list of the state before step t
                    cdk::launch_near_lists(a, st);          // and its near lists
                }
                cdk::AdjArgs q;
                q.n = (int)n;
                q.dt = dts + t;
                q.mass = c->col[cdk::MASS];
                q.fx = after + 4 * n;                       // force_prev after the step = its force
                q.fy = after + 5 * n;
                q.vnx = after + 2 * n;
                q.vny = after + 3 * n;
                q.fpx = c->col[cdk::FPX];
                q.fpy = c->col[cdk::FPY];
                q.lx = lx; q.lv = lv; q.lfp = lfp;
                q.gx = after;                               // the step's loss term
                q.gy = after + n;
                q.gtarget = tgt + (size_t)t * 2 * n;
                q.gscale = scale;
                q.lx_rw = lx;
                q.work_zero = use_snaps ? c->work : nullptr;
                q.lF = lF; q.lvt = lvt; q.lfp_out = lfp2;
                q.lx_out = lx2; q.lv_out = lv2;
                q.partial = partial;
                q.ldt = scal + 1;
                q.grad = g;
                q.argmax_vals = avals;
                q.argmax_idx = amax;
                q.blocks_done = blocks_done;
                cdk::launch_adj_seed(q, st);
                cdk::launch_adj_forces(a, q, st);
                cdk::launch_adj_dt(q, sc.dt_min, sc.dt_max, c->col[cdk::VX], c->col[cdk::VY],
                                   c->col[cdk::V0], st);
                std::swap(lx, lx2);
                std::swap(lv, lv2);
                std::swap(lfp, lfp2);
            }
            if (rc == CD_OK) CUDA_OR_FAIL(c, cudaEventRecord(ev_rev[sgi & 1], st));
        }
        if (rc == CD_OK)
            CUDA_OR_FAIL(c, cudaMemcpyAsync(grads, g, sizeof(double) * 4 * n,
                                            cudaMemcpyDeviceToHost, st));
        cudaStreamSynchronize(b->stream);
        cudaEventDestroy(ev_sync);
        for (int k = 0; k < 2; ++k) {
            cudaEventDestroy(ev_rec[k]);
            cudaEventDestroy(ev_rev[k]);
        }
        if (rc) return rc;
        if (check_device_error(b) != CD_OK)
            return fail(c, CD_ERR_CUDA, std::string("recomputation context: ") + cd_last_error(b));
    }
    cudaEventRecord(e2, st);
    // leave the context in the rollout's final state
    if ((rc = copy_state(c, fin, false))) return rc;
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->dt, scal + 2, sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_OR_FAIL(c, cudaMemcpyAsync(c->time_tot, scal + 3, sizeof(double), cudaMemcpyDeviceToDevice, st));
    CUDA_OR_FAIL(c, cudaMemcpyAsync(loss, scal, sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_OR_FAIL(c, cudaGetLastError());
    CUDA_OR_FAIL(c, cudaStreamSynchronize(st));
    float f_ms = 0, a_ms = 0;
    cudaEventElapsedTime(&f_ms, e0, e1);
    cudaEventElapsedTime(&a_ms, e1, e2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (forward_ms) *forward_ms = f_ms;
    if (adjoint_ms) *adjoint_ms = a_ms;
    return check_device_error(c);
}

// ---- groups: several contexts' steps in one graph launch ------------------
//
// A group captures the steps of its contexts into one CUDA graph: each
// context's stream joins the capture and enqueues its own `steps_per_launch`
// steps (exactly the sequence cd_launch replays, so every result is the
// same), then joins back.  Contexts advance independently inside the graph;
// one cudaGraphLaunch advances them all.  The graph is rebuilt when a member
// context's buffers, variant or walls changed (its graph generation moved).

struct cd_group {
    std::vector<cd_ctx *> ctx;
    std::vector<uint64_t> gen;
    std::vector<cudaEvent_t> ev_ctx;       // per member: its stream before a launch / capture join
    cudaEvent_t ev_fork = nullptr, ev_done = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int nodes = 0;
    int64_t k = 1;
    int device = 0;
    std::string msg;
};

namespace {

int gfail(cd_group *g, int code, const std::string &m) {
    if (g) g->msg = m;
    else g_create_error = m;
    return code;
}

#define GCUDA_OR_FAIL(g, call)                                                        \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return gfail((g), CD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Host-side preparation of every member (wall bins, noise checks), then the
// group graph if it is missing or stale.
int group_prepare(cd_group *g) {
    for (cd_ctx *c : g->ctx) {
        if ((g->nodes & CD_NODE_FLUCTUATION) && !c->noise_dev)
            return gfail(g, CD_ERR_INVALID_VALUE,
                         "graph steps cannot consume per-step host noise (use device noise)");
        if (int rc = prepare_step(c, g->nodes)) return gfail(g, rc, c->msg);
    }
    bool stale = g->exec == nullptr;
    for (size_t i = 0; i < g->ctx.size(); ++i) stale |= g->gen[i] != g->ctx[i]->graph_gen;
    if (!stale) return CD_OK;
    if (g->exec) {                                  // launches of the old graph end first
        GCUDA_OR_FAIL(g, cudaStreamSynchronize(g->stream));
        cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
    }
    GCUDA_OR_FAIL(g, cudaGetLastError());
    GCUDA_OR_FAIL(g, cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(g->ev_fork, g->stream);
    for (size_t i = 0; i < g->ctx.size() && e == cudaSuccess; ++i) {
        cd_ctx *c = g->ctx[i];
        e = cudaStreamWaitEvent(c->stream, g->ev_fork, 0);
        for (int64_t k = 0; k < g->k && e == cudaSuccess; ++k) {
            enqueue_step(c, g->nodes, false, false);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(g->ev_ctx[i], c->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g->stream, g->ev_ctx[i], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(g->stream, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gfail(g, CD_ERR_CUDA, std::string("group graph: ") + cudaGetErrorString(e));
    }
    for (size_t i = 0; i < g->ctx.size(); ++i) g->gen[i] = g->ctx[i]->graph_gen;
    return CD_OK;
}

}  // namespace

int cd_group_create(cd_group **out, cd_ctx *const *ctxs, int64_t n_ctxs, int nodes,
                    int64_t steps_per_launch) {
    if (!out) return gfail(nullptr, CD_ERR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (n_ctxs < 1 || !ctxs) return gfail(nullptr, CD_ERR_INVALID_VALUE, "need >= 1 context");
    if (steps_per_launch < 1 || steps_per_launch > 1000)
        return gfail(nullptr, CD_ERR_INVALID_VALUE, "steps_per_launch must be in [1, 1000]");
    if (nodes & ~(CD_NODE_ALL | CD_NODE_NAVIGATION))
        return gfail(nullptr, CD_ERR_INVALID_VALUE, "unknown node flags");
    int dev = 0;
    GCUDA_OR_FAIL(nullptr, cudaGetDevice(&dev));
    for (int64_t i = 0; i < n_ctxs; ++i) {
        if (!ctxs[i]) return gfail(nullptr, CD_ERR_INVALID_VALUE, "a context is NULL");
        if (ctxs[i]->device != dev)
            return gfail(nullptr, CD_ERR_INVALID_VALUE, "contexts on another device");
        for (int64_t j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return gfail(nullptr, CD_ERR_INVALID_VALUE, "a context twice");
    }
    cd_group *g = new cd_group();
    g->ctx.assign(ctxs, ctxs + n_ctxs);
    g->gen.assign(n_ctxs, 0);
    g->ev_ctx.assign(n_ctxs, nullptr);
    g->nodes = nodes;
    g->k = steps_per_launch;
    g->device = dev;
    bool ok = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&g->ev_done, cudaEventDisableTiming) == cudaSuccess;
    for (auto &e : g->ev_ctx)
        ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cd_group_destroy(g);
        return gfail(nullptr, CD_ERR_CUDA, "cudaStreamCreate / cudaEventCreate failed");
    }
    if (int rc = group_prepare(g)) {
        const std::string m = g->msg;
        cd_group_destroy(g);
        return gfail(nullptr, rc, m);
    }
    *out = g;
    return CD_OK;
}

void cd_group_destroy(cd_group *g) {
    if (!g) return;
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    for (cudaEvent_t e : g->ev_ctx)
        if (e) cudaEventDestroy(e);
    if (g->ev_fork) cudaEventDestroy(g->ev_fork);
    if (g->ev_done) cudaEventDestroy(g->ev_done);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

const char *cd_group_last_error(const cd_group *g) {
    return g ? g->msg.c_str() : g_create_error.c_str();
}

int cd_group_launch(cd_group *g, int64_t launches) {
    if (!g) return gfail(nullptr, CD_ERR_INVALID_VALUE, "group is NULL");
    if (launches < 0) return gfail(g, CD_ERR_INVALID_VALUE, "negative launch count");
    if (int rc = group_prepare(g)) return rc;
    // after each member's earlier work; each member's later work after the launch
    for (size_t i = 0; i < g->ctx.size(); ++i) {
        GCUDA_OR_FAIL(g, cudaEventRecord(g->ev_ctx[i], g->ctx[i]->stream));
        GCUDA_OR_FAIL(g, cudaStreamWaitEvent(g->stream, g->ev_ctx[i], 0));
    }
    for (int64_t k = 0; k < launches; ++k) GCUDA_OR_FAIL(g, cudaGraphLaunch(g->exec, g->stream));
    GCUDA_OR_FAIL(g, cudaEventRecord(g->ev_done, g->stream));
    for (cd_ctx *c : g->ctx) GCUDA_OR_FAIL(g, cudaStreamWaitEvent(c->stream, g->ev_done, 0));
    GCUDA_OR_FAIL(g, cudaGetLastError());
    return CD_OK;
}

int cd_group_synchronize(cd_group *g) {
    if (!g) return gfail(nullptr, CD_ERR_INVALID_VALUE, "group is NULL");
    GCUDA_OR_FAIL(g, cudaStreamSynchronize(g->stream));
    for (cd_ctx *c : g->ctx)
        if (int rc = cd_synchronize(c)) return gfail(g, rc, c->msg);
    return CD_OK;
}

// ---- agent-agent forces without device allocation -------------------------
//
// The cell list and staging buffers of one agent-agent pass live in the
// file-scope array below, carved at fixed 256-byte-aligned offsets.  Host code
// never uses the array's name as an address: its device address comes from
// cudaGetSymbolAddress, looked up once per device.

namespace {

constexpr size_t na_align(size_t b) { return (b + 255) & ~size_t(255); }
constexpr int NA_N = CD_NOALLOC_MAX_AGENTS, NA_C = CD_NOALLOC_MAX_CELLS;
constexpr size_t NA_OFF_SCEN = 0;
constexpr size_t NA_OFF_SCEN_OF = NA_OFF_SCEN + na_align(sizeof(ScenDev));
constexpr size_t NA_OFF_KEY = NA_OFF_SCEN_OF + na_align(sizeof(int) * NA_N);
constexpr size_t NA_OFF_COUNT = NA_OFF_KEY + na_align(sizeof(int) * NA_N);
constexpr size_t NA_OFF_FILL = NA_OFF_COUNT + na_align(sizeof(int) * NA_C);
constexpr size_t NA_OFF_START = NA_OFF_FILL + na_align(sizeof(int) * NA_C);
constexpr size_t NA_OFF_PERM_U = NA_OFF_START + na_align(sizeof(int) * (NA_C + 1));
constexpr size_t NA_OFF_PERM = NA_OFF_PERM_U + na_align(sizeof(int) * NA_N);
constexpr size_t NA_OFF_SCAN = NA_OFF_PERM + na_align(sizeof(int) * NA_N);
constexpr size_t NA_SCAN_INTS = 2 * (NA_C / 4096 + 2);
constexpr size_t NA_OFF_STAGE = NA_OFF_SCAN + na_align(sizeof(int) * NA_SCAN_INTS);
constexpr size_t NA_OFF_CULL = NA_OFF_STAGE + na_align(sizeof(double2) * NA_N * cdk::STAGE_Q_TC);
constexpr size_t NA_OFF_STAGEF = NA_OFF_CULL + na_align(sizeof(float4) * NA_N);
constexpr size_t NA_OFF_VMAX = NA_OFF_STAGEF + na_align(sizeof(float4) * 2 * NA_N);
constexpr size_t NA_OFF_ERR = NA_OFF_VMAX + na_align(sizeof(unsigned long long));
constexpr size_t NA_OFF_WORK = NA_OFF_ERR + na_align(sizeof(int));
// StepArgs::work holds four ints (the force kernel's work counter, the
// float32 pair pass's deferred count, the force pass's two job counts)
constexpr size_t NA_BYTES = NA_OFF_WORK + na_align(4 * sizeof(int));
static_assert(NA_BYTES < (4u << 20), "allocation-free scratch stays below 4 MiB");

__device__ __align__(256) static unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_na_mutex;
unsigned char *g_na_base[256] = {};

// Scenario record and per-agent scenario ids (all zero) for one call.
__global__ void k_na_init(ScenDev *scen, int *scen_of, int n, double x0, double y0, double cell,
                          int nx, int ny) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        ScenDev d;
        d.x0 = x0; d.y0 = y0; d.cell = cell;
        d.dt_min = 0.0; d.dt_max = 0.0; d.wall_reach = 0.0;
        d.nx = nx; d.ny = ny; d.cell_base = 0;
        d.agent_begin = 0; d.agent_count = n; d.wall_begin = 0; d.wall_count = 0;
        *scen = d;
    }
    if (i < n) scen_of[i] = 0;
}

}  // namespace

extern "C" int cd_agent_agent_noalloc(int body_type, int64_t n, const double *cols,
                                      double *force_x, double *force_y, double *torque,
                                      double x0, double y0, double cell_size, int64_t nx,
                                      int64_t ny, void *stream_ptr) {
    if (body_type != CD_BODY_CIRCULAR && body_type != CD_BODY_THREE_CIRCLE)
        return fail(nullptr, CD_ERR_INVALID_TYPE, "unknown body type");
    if (n < 0) return fail(nullptr, CD_ERR_INVALID_VALUE, "negative agent count");
    if (n > CD_NOALLOC_MAX_AGENTS)
        return fail(nullptr, CD_ERR_CAPACITY, "cd_agent_agent_noalloc: " + std::to_string(n) +
                                                  " agents exceed CD_NOALLOC_MAX_AGENTS (" +
                                                  std::to_string(CD_NOALLOC_MAX_AGENTS) + ")");
    if (nx < 1 || ny < 1 || !(cell_size > 0) || !std::isfinite(cell_size) || !std::isfinite(x0) ||
        !std::isfinite(y0))
        return fail(nullptr, CD_ERR_INVALID_VALUE, "bad cell grid");
    if (nx > CD_NOALLOC_MAX_CELLS || ny > CD_NOALLOC_MAX_CELLS || nx * ny > CD_NOALLOC_MAX_CELLS)
        return fail(nullptr, CD_ERR_CAPACITY, "cd_agent_agent_noalloc: " + std::to_string(nx * ny) +
                                                  " cells exceed CD_NOALLOC_MAX_CELLS (" +
                                                  std::to_string(CD_NOALLOC_MAX_CELLS) + ")");
    if (n == 0) return CD_OK;
    if (!cols || !force_x || !force_y || (body_type == CD_BODY_THREE_CIRCLE && !torque))
        return fail(nullptr, CD_ERR_INVALID_VALUE, "NULL column or output pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream_ptr);
    int dev = 0;
    CUDA_OR_FAIL(nullptr, cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(nullptr, CD_ERR_INVALID_VALUE, "device ordinal out of range");
    unsigned char *base;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_base[dev]) {
            void *p = nullptr;
            CUDA_OR_FAIL(nullptr, cudaGetSymbolAddress(&p, g_noalloc_scratch));
            if (int e = cdk::init_kernels())
                return fail(nullptr, CD_ERR_CUDA, std::string("kernel attributes: ") +
                                                      cudaGetErrorString((cudaError_t)e));
            g_na_base[dev] = static_cast<unsigned char *>(p);
        }
        base = g_na_base[dev];
    }
    const int ncells = (int)(nx * ny);
    StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = (int)n;
    a.n_scen = 1;
    a.n_cells = ncells;
    a.body = body_type;
    a.nodes = cdk::N_AGENT;
    const double *c = cols;
    auto col = [&](int k) { return const_cast<double *>(c + (size_t)k * n); };
    a.col[cdk::X] = col(CD_NA_X); a.col[cdk::Y] = col(CD_NA_Y);
    a.col[cdk::VX] = col(CD_NA_VX); a.col[cdk::VY] = col(CD_NA_VY);
    a.col[cdk::MASS] = col(CD_NA_MASS); a.col[cdk::K_SOC] = col(CD_NA_K_SOC);
    a.col[cdk::TAU0] = col(CD_NA_TAU_0); a.col[cdk::MU] = col(CD_NA_MU);
    a.col[cdk::KAPPA] = col(CD_NA_KAPPA); a.col[cdk::DAMP] = col(CD_NA_DAMPING);
    a.col[cdk::FX] = force_x; a.col[cdk::FY] = force_y;
    if (body_type == CD_BODY_CIRCULAR) {
        a.col[cdk::R] = col(CD_NA_RADIUS);
    } else {
        a.col[cdk::RT] = col(CD_NA_R_T); a.col[cdk::RS] = col(CD_NA_R_S);
        a.col[cdk::RTS] = col(CD_NA_R_TS);
        a.col[cdk::XLS] = col(CD_NA_X_LS); a.col[cdk::YLS] = col(CD_NA_Y_LS);
        a.col[cdk::XRS] = col(CD_NA_X_RS); a.col[cdk::YRS] = col(CD_NA_Y_RS);
        a.col[cdk::PHI] = col(CD_NA_ORIENTATION);
        a.col[cdk::PHI0] = col(CD_NA_ORIENTATION);     // read, never written (no orientation node)
        a.col[cdk::TORQUE] = torque;
    }
    ScenDev *scen = reinterpret_cast<ScenDev *>(base + NA_OFF_SCEN);
    int *scen_of = reinterpret_cast<int *>(base + NA_OFF_SCEN_OF);
    a.scen = scen;
    a.scen_of = scen_of;
    a.key = reinterpret_cast<int *>(base + NA_OFF_KEY);
    a.count = reinterpret_cast<int *>(base + NA_OFF_COUNT);
    a.fill = reinterpret_cast<int *>(base + NA_OFF_FILL);
    a.start = reinterpret_cast<int *>(base + NA_OFF_START);
    a.perm_unsorted = reinterpret_cast<int *>(base + NA_OFF_PERM_U);
    a.perm = reinterpret_cast<int *>(base + NA_OFF_PERM);
    a.stage = reinterpret_cast<double2 *>(base + NA_OFF_STAGE);
    a.cull = reinterpret_cast<float4 *>(base + NA_OFF_CULL);
    a.stage_f = reinterpret_cast<float4 *>(base + NA_OFF_STAGEF);
    a.vmax = reinterpret_cast<unsigned long long *>(base + NA_OFF_VMAX);
    a.err = reinterpret_cast<int *>(base + NA_OFF_ERR);
    a.work = reinterpret_cast<int *>(base + NA_OFF_WORK);
    int *scan = reinterpret_cast<int *>(base + NA_OFF_SCAN);
    // the array keeps the previous call's contents: zero what must start at 0
    CUDA_OR_FAIL(nullptr, cudaMemsetAsync(a.count, 0, sizeof(int) * ncells, st));
    CUDA_OR_FAIL(nullptr, cudaMemsetAsync(a.fill, 0, sizeof(int) * ncells, st));
    CUDA_OR_FAIL(nullptr, cudaMemsetAsync(a.vmax, 0, sizeof(unsigned long long), st));
    CUDA_OR_FAIL(nullptr, cudaMemsetAsync(a.err, 0, sizeof(int), st));
    k_na_init<<<(int)((n + 255) / 256), 256, 0, st>>>(scen, scen_of, (int)n, x0, y0, cell_size,
                                                       (int)nx, (int)ny);
    cdk::launch_prepare(a, st);
    cdk::launch_scan(a.count, a.start, ncells, scan, st);
    cdk::launch_scatter(a, st, false, 0);               // rank + gather
    cdk::launch_forces(a, st, cdk::default_group_variant(n, a.body ? 1 : 0));
    CUDA_OR_FAIL(nullptr, cudaGetLastError());
    int h = 0;
    CUDA_OR_FAIL(nullptr, cudaMemcpyAsync(&h, a.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_OR_FAIL(nullptr, cudaStreamSynchronize(st));
    if (h & cdk::ERR_NOT_FINITE) return fail(nullptr, CD_ERR_NOT_FINITE, "an agent position is not finite");
    if (h & cdk::ERR_RANGE)
        return fail(nullptr, CD_ERR_INVALID_VALUE, "an agent is more than 1e7 m from the grid origin");
    return CD_OK;
}
