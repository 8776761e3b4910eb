// cd_internal.cuh -- shared device-side types of libcdgpu (not part of the ABI).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cdk {

// Primary agent state: one float64 column per field, agents in batch order.
enum Col {
    X, Y, VX, VY, FX, FY, FPX, FPY, E0X, E0Y, R, MASS, TAU_ADJ, K_SOC, TAU0,
    MU, KAPPA, DAMP, V0,
    XLS, YLS, XRS, YRS, RT, RS, RTS, INERTIA, W0, PHI, OMEGA, PHI0, TORQUE,
    TORQUE_PREV, TAU_ROT, SRF, SRT,      // std_rand_force, std_rand_torque
    NCOL
};

// Staged neighbour records (cell-sorted order), in double2 units.
constexpr int STAGE_Q_CIRC = 6;    // (x,y)(vx,vy)(r,m)(k,tau0)(mu,kappa)(damp,1/tau0)
constexpr int STAGE_Q_TC = 10;     // (x,y)(xls,yls)(xrs,yrs)(vx,vy)(rt,rs)
                                   // (rts,m)(k,tau0)(mu,kappa)(damp,sin)(cos,1/tau0)
constexpr int WALL_D = 8;          // p0x p0y p1x p1y tx ty lw -

// Device error bits (StepArgs::err).
constexpr int ERR_NOT_FINITE = 1;
// An agent farther than COORD_MAX (cd_cull.cuh) from its scenario's grid origin.
constexpr int ERR_RANGE = 4;
// A record flagged both leader and follower (cd_herding rejects it).
constexpr int ERR_LEADER_FOLLOWER = 8;

// Candidate chunks per agent whose ballots the near-list count keeps for the
// fill (an agent with more is evaluated again by the fill).
constexpr int NL_MASK_CHUNKS = 64;

// Doubles per agent of k_prologue's record (two 32-byte halves).
constexpr int PRO_D = 8;

// Columns of the per-agent interaction counts (CD_COUNT_COLS of cdgpu.h).
constexpr int COUNT_COLS = 9;

// Node flags (mirror CD_NODE_* of include/cdgpu.h).
constexpr int N_FLUCT = 1, N_ORIENT = 2, N_ADJUST = 4, N_AGENT = 8,
              N_WALL = 16, N_INTEG = 32, N_RESET = 64, N_NAV = 128;

struct ScenDev {
    double x0, y0, cell;
    double dt_min, dt_max;
    double wall_reach;          // agent extent the wall bins were built for
    int nx, ny;
    int cell_base;              // first flat cell of this scenario
    int agent_begin, agent_count;
    int wall_begin, wall_count;
    // navigation: direction maps on a meshgrid (origin, spacing), targets x ny x nx
    double nav_x0, nav_y0, nav_step;
    int nav_nx, nav_ny, nav_targets;
    long long nav_off;           // first double2 of the scenario's maps
};

struct StepArgs {
    int n, n_scen, n_cells, body, nodes;
    double *col[NCOL];
    const int *scen_of;          // scenario of every agent
    const ScenDev *scen;
    // cell list
    int *key;                    // flat cell (batch-global) per agent
    int *count, *fill, *start;   // per cell; start has n_cells + 1 entries
    int *perm_unsorted, *perm;   // slot -> agent
    // staging (cell-sorted)
    double2 *stage;
    float4 *cull;                // (x, y, extent, -) as float
    float4 *stage_f;             // ThreeCircle: 2 per slot, float32 geometry for
                                 // the sub-circle pre-selection (see k_gather)
    // walls
    const double *walls;         // WALL_D doubles per wall
    const float4 *walls_f;       // (p0x, p0y, p1x, p1y) as float
    const int *wall_start, *wall_idx;   // per-cell CSR of wall ids
    // fluctuation: host-drawn arrays, or drawn on the device (noise_dev) from
    // the counter generator with `noise_seed` at step *rng_step
    const double *noise_f, *noise_m;
    int noise_dev;
    unsigned long long noise_seed;
    unsigned long long *rng_step;
    // navigation
    const int *tgt;              // per agent: target index, -1 for none
    const double2 *navmap;       // (dir_x, dir_y) per map cell
    // timestep
    unsigned long long *vmax;    // per scenario, ordered bits of max |v|
    const double *v0max;         // per scenario max target_velocity
    double *dt, *time_tot;       // per scenario
    int *err;
    int *work;                   // [0] force-kernel work counter (zeroed per launch),
                                 // [1] pairs the float32 pair pass left to k_pairs,
                                 // [2] / [3] force-pass jobs without / with contact
    int *fix_count, *fix_list;   // agents the gather leaves to k_forces_fallback
    int *slot_of;                // per agent: its cell-sorted slot (k_rank)
    double *pro;                 // per agent PRO_D doubles: prologue fx, fy, torque, phi0;
                                 // old accelerations (force_prev / m, torque_prev / I)
    // near lists (compute-once pair pipeline): per cell-sorted slot, the
    // slots of its near candidates in ascending order (= visiting order)
    int *nl_cnt;                 // n + 1 counts (scan input)
    int *nl_off;                 // n + 1 offsets; nl_off[n] = entries needed (k_scan_tiles
                                 // leaves tile-relative offsets, k_nl_fill the final ones)
    int *nl_fwd;                 // per slot: first entry with a later slot
    unsigned *nl_mask;           // per slot NL_MASK_CHUNKS chunk ballots (k_nl_count -> k_nl_fill)
    int *nl_nch;                 // per slot: its candidate chunks
    int *nl_idx;                 // nl_cap entries
    double *nl_res;              // per entry: RES_D doubles of pair results (forces only)
    unsigned char *nl_kind;      // per entry: none / zero force (+0 or -0 torque) / force
    int nl_cap;
    int *nl_scan;                // scan scratch: tile totals, tile offsets, a tile counter
    int *fw_cnt, *fw_off;        // per slot: entries with a later slot (n + 1 each)
    int2 *fw_pairs;              // flat list of (slot, entry) for those entries
    int *defer_list;             // flat-list indices the float32 pair pass left to k_pairs
                                 // (nl_cap entries; null: no float32 pass)
    double2 *pair_jobs;          // the pairs k_pairs found to have a force, for k_pair_forces
                                 // (nl_cap / 2 + 1 records of JOB_Q_TC / JOB_Q_CIRC double2)
    int *fw_scan;                // scan scratch (as nl_scan)
    int *fs_cnt, *fs_off;        // per agent: those guessed to need the social force, scan
    int *fs_scan;                // scan scratch (as nl_scan)
};

// Pair-result record of a near-list entry with a force: (fx, fy, torque, -);
// the adjoint's records (Circular contexts) hold ADJ_RES_D doubles.
constexpr int RES_D = 4;
constexpr int ADJ_RES_D = 6;
// Force-pass job records (double2 each): ThreeCircle (s, t, e, eq), (tau, b),
// (d, h), (dx, dy), (|d|, flags); Circular (s, t, e, eq), (|x|, sqrt D), (tau, flags).
constexpr int JOB_Q_TC = 5;
constexpr int JOB_Q_CIRC = 3;
// Device error bit: a pair partner's near list lacked the pair.
constexpr int ERR_NEAR_LIST = 2;

// Integer and bool state fields: byte offsets in the records (-1 = absent)
// and their device columns (indices outside [0, 2^31) read as -1).
struct StateOffsets {
    long long target, active, leader, follower, index_leader, familiar_exit;
};
struct StateCols {
    int *target, *active, *leader, *follower, *index_leader, *familiar_exit;
};

// Leader-follower / herding arguments (cd_states.cu).  The cell list is the
// one built on the herding grid (cell = follower sight).
struct HerdArgs {
    int n, K, with_herding;
    const int *perm, *key, *start, *scen_of;
    const ScenDev *scen_h;           // herding grid per scenario (walls as in the step)
    double *col[NCOL];
    const double *walls;             // WALL_D doubles per wall
    StateCols st;
    int *nbr;                        // n x K nearest unobstructed neighbours, -1 missing
    const int *leaders;              // leader agents in ascending order
    const int *n_leaders;
    int *tgt_before;                 // targets before the update
    double sight_f, sight_l, cos_phi, w_herd, w_lead, w_dir;
};
// Sets ERR_LEADER_FOLLOWER in *err if any record is both leader and follower.
void launch_check_roles(const StateCols &st, int n, int *err, cudaStream_t s);
void launch_herd_neighbors(const HerdArgs &h, cudaStream_t s);
void launch_leaders(const HerdArgs &h, int *flags, int *pos, int *scan_scratch, int *list,
                    cudaStream_t s);
void launch_herd_follow(const HerdArgs &h, cudaStream_t s);
void launch_inside_domain(int begin, int count, const double *x, const double *y, int *active,
                          const double2 *poly, int m, unsigned long long *changed,
                          cudaStream_t s);
void launch_exit_detection(int begin, int count, const double *x, const double *y,
                           const double *walls, int wall_begin, int wall_count,
                           const double2 *doors, int n_doors, double range, const StateCols &st,
                           cudaStream_t s);
void launch_target_reached(int begin, int count, const double *x, const double *y,
                           unsigned char *reached, const double2 *polys, const int *voff, int t,
                           unsigned long long *counts, cudaStream_t s);

// Reverse-step arguments (cd_adjoint.cu); n x 2 arrays are interleaved,
// state snapshots are columns.
struct AdjArgs {
    int n;
    const double *dt;                      // this step's timestep (device scalar)
    const double *mass, *fx, *fy;          // mass, the step's total force
    const double *vnx, *vny;               // velocity after the step
    const double *fpx, *fpy;               // force_prev before the step
    const double *lx, *lv, *lfp;           // incoming adjoints of x', v', fp'
    // this step's loss term, added to the incoming x' adjoint by k_adj_seed
    // (lx += scale 2 (x' - target), written back to lx_rw = lx); gtarget null: none
    const double *gx, *gy, *gtarget;       // positions after the step, their target
    double gscale;
    double *lx_rw;
    int *work_zero;                        // StepArgs::work, zeroed by k_adj_seed (null: not)
    double *lF, *lvt, *lfp_out;            // adjoint of F, of v' incl. x', of fp
    double *lx_out, *lv_out;               // outgoing adjoints of x, v
    double *partial, *ldt;                 // dt adjoint (block partials, total)
    double *grad;                          // n x 4: tau_adj, v0, tau_0, k_soc
    double *argmax_vals;                   // per argmax block: max |v|, max v0
    int *argmax_idx;                       // their first indices
    int *blocks_done;                      // last-block counter (zero between kernels)
};

int adj_partials(int n);
void launch_adj_seed(const AdjArgs &q, cudaStream_t s);
void launch_adj_forces(const StepArgs &a, const AdjArgs &q, cudaStream_t s);
void launch_adj_dt(const AdjArgs &q, double dt_min, double dt_max, const double *vx,
                   const double *vy, const double *v0, cudaStream_t s);
// loss += scale * sum |x - target|^2 (block partials summed by the last
// block in a fixed order); also copies the step's dt (dt_src) to dt_dst.
void launch_loss(const double *x, const double *y, const double *target, int n,
                 double *partial, double *loss, double scale, int *blocks_done,
                 const double *dt_src, double *dt_dst, cudaStream_t s);
// Up to 16 device-to-device copies in one launch (byte counts multiples of 4).
void launch_copy_bufs(const void *const *src, void *const *dst, const long long *bytes, int nbuf,
                      cudaStream_t s);
// `dep`: launched as the programmatic dependent of the kernel before it.
void launch_copy_cols(const double *const *src, double *const *dst, int ncol, int n,
                      cudaStream_t s, bool dep = false);

// Programmatic dependent launch: a kernel launched by launch_k(true, ...)
// may start while the kernel before it on the stream finishes; it begins
// with pdl_enter, which waits for that kernel (its memory visible) and lets
// the next dependent start in turn.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch of kernel `k` on `s`.  `dep`: as the programmatic dependent of the
// kernel launched just before it on `s` (every such kernel starts with
// pdl_enter), so that its launch overlaps that kernel's last blocks.
template <typename... P, typename... A>
inline void launch_k(bool dep, void (*k)(P...), dim3 grid, dim3 block, size_t smem,
                     cudaStream_t s, A... args) {
    if (!dep) {
        k<<<grid, block, smem, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

// Launchers (cd_kernels.cu)
void launch_prepare(const StepArgs &a, cudaStream_t s);
void launch_dt(const StepArgs &a, cudaStream_t s);
int scan_scratch_ints(int n);
// Scratch ints of each near-list scan (tile totals, tile offsets, a counter;
// zeroed once at allocation).
int near_scan_ints(int n);
// `after_kernel`: the last operation on `s` is a kernel launch; the first
// kernel here is then launched as its programmatic dependent.
void launch_scan(const int *in, int *out, int n, int *scratch, cudaStream_t s,
                 bool after_kernel = false);
int scan_launches_single(int n);          // kernels launch_scan uses for n elements
// Agents into cells in stable order; with gather_part >= 0 the ranking kernel
// also writes the staged records of that part (as launch_gather).
void launch_scatter(const StepArgs &a, cudaStream_t s, bool after_kernel = false,
                    int gather_part = -1);
// Staged records of the cell-sorted agents: part 0 all, 1 the float32
// pre-check records, 2 the float64 records.
void launch_gather(const StepArgs &a, cudaStream_t s, int part = 0, bool after_kernel = false);
constexpr int N_VARIANTS = 15;      // launch variants of the force kernel
bool variant_pairs(int variant);
bool variant_split(int variant);     // the pair pipeline with the separate force pass
int variant_lanes(int variant);
int default_variant(long long n_agents, int body);
int default_group_variant(long long n_agents, int body);
int variant_threads(int variant);
int variant_staged(int variant);
// A second stream for work that runs beside the near-list build (fork after
// the work already on the main stream, join before the gather).
struct Fork { cudaStream_t s2; cudaEvent_t fork, join, join_stage; };
// The agent-force stage; with `pair_ev` (3 events), events recorded before
// the pair stage, after its float32 pass and after it (as external
// event-record nodes if `captured`).
void launch_forces(const StepArgs &a, cudaStream_t s, int variant,
                   const cudaEvent_t *pair_ev = nullptr, bool captured = false,
                   const Fork *fork = nullptr, bool stage_deferred = false);
// The per-agent terms before agent-agent (navigation, fluctuation,
// orientation, adjusting) and the old accelerations, into StepArgs::pro.
void launch_prologue(const StepArgs &a, cudaStream_t s);
// Near-list counts and their scan (nl_off) for the state staged in `a`.
void launch_near_count(const StepArgs &a, cudaStream_t s, int variant);
// Near lists (counts, scans, fill; 8 lanes per agent) for the state staged in `a`.
void launch_near_lists(const StepArgs &a, cudaStream_t s);
// The float32 pass of the Circular reverse step over the flat list's second
// part: the entries of the pairs without a force marked empty, the rest
// appended to the deferred list for k_adj_pairs.
void launch_adj_light(const StepArgs &a, cudaStream_t s);
void launch_pair_counts(const StepArgs &a, int *counts, cudaStream_t s);
// Per-scenario max target_velocity and (if `ext`) max agent extent;
// `partial` holds scen_max_partials(n_scen) doubles.
void launch_scen_max(const StepArgs &a, double *v0max, double *ext, double *partial,
                     cudaStream_t s);
int scen_max_partials(int n_scen);
void launch_wall_prep(const double *raw, double *walls, int nw, cudaStream_t s);
void launch_aos_to_soa(const char *aos, long long itemsize, const long long *off,
                       int n, int body, double *const *col, cudaStream_t s);
void launch_states_in(const char *aos, long long itemsize, const StateOffsets &o, int n,
                      const StateCols &c, cudaStream_t s);
// Writes target, index_leader, active and is_follower back into the records.
void launch_states_out(char *aos, long long itemsize, const StateOffsets &o, int n,
                       const StateCols &c, cudaStream_t s);
void launch_soa_to_aos(char *aos, long long itemsize, const long long *off,
                       int n, int body, const double *const *col, cudaStream_t s);
// Packed records straight from / into device-addressable host memory (the
// copy and the transpose in one pass; `aos` keeps the device copy of the
// records for the fields the step does not write).  0 records per block:
// records too large for shared memory, use the staged path.
int records_per_block(long long itemsize);
// The per-scenario maxima an upload leaves (launch_scen_max's results),
// reduced by launch_records_in in its own pass when `key` is set: `key` holds
// two order keys per scenario (zero between uploads), `blocks_done` one
// counter (zero between uploads).
struct ScenMax {
    unsigned long long *key;
    int *blocks_done;
    const int *scen_of;
    double *v0max, *ext;
    double *ext_host;            // page-locked copy of ext, written by the kernel too
    int n_scen, body;
};
// What the host reads after a download (the step status and the entries the
// last near-list build needed), written into page-locked memory by
// launch_records_out itself.
struct StepStatus {
    const int *err, *need;       // need: nl_off + n, or null without near lists
    int *host;                   // [0] err, [1] need (0 without near lists)
};
// launch_records_in also fills the state columns (as launch_states_in).
void launch_records_in(const void *src, char *aos, long long itemsize, const long long *off,
                       int n, int body, double *const *col, const StateOffsets &so,
                       const StateCols &sc, cudaStream_t s, const ScenMax &mx);
void launch_records_out(void *dst, const char *aos, long long itemsize, const long long *off,
                        int n, int body, const double *const *col, cudaStream_t s,
                        const StepStatus &st);
double fp64_peak_gflops();
// Shared-memory bytes of the force kernel (dynamic) and one-time attributes.
size_t forces_smem_bytes(int body, int variant);
int init_kernels();

}  // namespace cdk
