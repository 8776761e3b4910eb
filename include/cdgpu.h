/*
 * cdgpu.h -- C ABI of the GB300-native per-step agent update (libcdgpu.so).
 *
 * The library advances crowds of Circular or ThreeCircle agents by the
 * reference's per-step update: fluctuation (host-drawn noise), orientation,
 * adjusting force/torque, agent-agent power-law social + contact forces over
 * a uniform cell list, agent-wall contact forces, adaptive-timestep velocity
 * Verlet and reset.  All arithmetic is IEEE float64.  Plain pointers and
 * sizes only; every entry point returns CD_OK (0) or a CD_ERR_* code and
 * keeps a message for cd_last_error().
 *
 * A context owns one batch of independent scenarios (a plain simulation is
 * a batch of one).  Scenarios share a body type; each has its own agent
 * range, wall range, cell grid and timestep bounds.  Calls on one context
 * are not reentrant; one context runs on one CUDA stream of the device that
 * was current at cd_create.
 *
 * Reference interfaces each entry point replaces (paths inside the
 * crowddynamics project):
 *   cd_step / cd_run ...... MultiAgentSimulation.update()
 *                           crowddynamics/simulation/multiagent.py:51-55 with
 *                           the nodes of crowddynamics/simulation/logic.py:59-130,258-261
 *   CD_NODE_AGENT_AGENT ... agent_agent_block_list, core/interactions.py:191-205
 *   CD_NODE_AGENT_OBSTACLE  agent_obstacle, core/interactions.py:208-214
 *   CD_NODE_ADJUSTING ..... force_adjust_agents / torque_adjust_agents,
 *                           core/motion/adjusting.py:98-121
 *   CD_NODE_ORIENTATION ... orient_towards_target_direction,
 *                           core/steering/orientation.py:17-21
 *   CD_NODE_INTEGRATE ..... velocity_verlet_integrator, core/integrator.py:209-256
 *   CD_NODE_RESET ......... Reset.update, simulation/logic.py:59-64
 *   CD_NODE_FLUCTUATION ... Fluctuation.update, simulation/logic.py:78-86
 *                           (noise drawn on the host, passed by cd_set_noise)
 *   CD_NODE_NAVIGATION .... Navigation.update, simulation/logic.py:135-165, with
 *                           getdefault, core/steering/navigation.py:69-78, and the
 *                           meshgrid indicer, core/steering/quickest_path.py:40-43
 *                           (direction maps passed by cd_set_direction_maps)
 *   cd_upload_agents /
 *   cd_download_agents .... the in-place numpy structured agent arrays the
 *                           nodes read and write (simulation/agents.py:447-448)
 *   cd_set_walls .......... geom_to_linear_obstacles' obstacle_type_linear
 *                           array, core/geometry.py:99-102, core/structures.py:6-9
 */
#ifndef CDGPU_H
#define CDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define CD_OK 0
#define CD_ERR_INVALID_TYPE 1   /* body type / record layout not recognised  */
#define CD_ERR_INVALID_VALUE 2  /* bad size, range or non-finite input       */
#define CD_ERR_CUDA 3           /* a CUDA runtime call failed                 */
#define CD_ERR_NOT_FINITE 4     /* a kernel saw a non-finite agent position   */
#define CD_ERR_CAPACITY 5       /* an input exceeded a fixed capacity         */

/* ---- body types -------------------------------------------------------- */
#define CD_BODY_CIRCULAR 0
#define CD_BODY_THREE_CIRCLE 1

/* ---- logic nodes run by cd_step / cd_run (bit flags, post-order) ------- */
#define CD_NODE_FLUCTUATION 1
#define CD_NODE_ORIENTATION 2
#define CD_NODE_ADJUSTING 4
#define CD_NODE_AGENT_AGENT 8
#define CD_NODE_AGENT_OBSTACLE 16
#define CD_NODE_INTEGRATE 32
#define CD_NODE_RESET 64
#define CD_NODE_ALL 127          /* the standard tree (navigation excluded) */
#define CD_NODE_NAVIGATION 128   /* runs first: target direction from the maps */

/* ---- float64 fields of an agent record (offset-table order) ------------ */
enum {
    CD_F_POSITION = 0, CD_F_VELOCITY, CD_F_TARGET_DIRECTION, CD_F_FORCE,
    CD_F_FORCE_PREV, CD_F_RADIUS, CD_F_R_T, CD_F_R_S, CD_F_R_TS, CD_F_MASS,
    CD_F_INERTIA_ROT, CD_F_TARGET_VELOCITY, CD_F_TARGET_ANGULAR_VELOCITY,
    CD_F_TAU_ADJ, CD_F_K_SOC, CD_F_TAU_0, CD_F_MU, CD_F_KAPPA, CD_F_DAMPING,
    CD_F_STD_RAND_FORCE, CD_F_POSITION_LS, CD_F_POSITION_RS, CD_F_ORIENTATION,
    CD_F_ANGULAR_VELOCITY, CD_F_TARGET_ORIENTATION, CD_F_TORQUE,
    CD_F_TORQUE_PREV, CD_F_TAU_ROT, CD_F_STD_RAND_TORQUE,
    CD_F_TARGET,                  /* int64: target index, -1 for none */
    CD_F_ACTIVE,                  /* bool */
    CD_F_IS_LEADER,               /* bool */
    CD_F_IS_FOLLOWER,             /* bool */
    CD_F_INDEX_LEADER,            /* int64: leader agent, -1 for none */
    CD_F_FAMILIAR_EXIT,           /* int64: target, -1 for none */
    CD_F_COUNT
};

/* One scenario of a batch.  The cell grid covers [x0, x0 + nx*cell_size) x
 * [y0, y0 + ny*cell_size); an agent outside it is binned into the nearest
 * border cell, which keeps every interacting pair in adjacent cells.  The
 * reference's default cell size is sight_soc + 2 * max_agent_radius
 * (simulation/logic.py:97-116).  Coordinates may be anywhere (UTM metres,
 * say), but every agent must stay within 1e7 m of its scenario's (x0, y0) in
 * each axis: a step that finds one farther fails with CD_ERR_INVALID_VALUE
 * (the float32 pre-checks that skip non-interacting pairs work relative to
 * the grid origin and are exact only within that range). */
typedef struct {
    int64_t agent_begin, agent_count;   /* range in the batch's agent array */
    int64_t wall_begin, wall_count;     /* range in the batch's wall array  */
    double x0, y0, cell_size;           /* grid origin and cell size (m)    */
    int64_t nx, ny;                     /* grid shape (cells)               */
    double dt_min, dt_max;              /* Integrator.dt_min / dt_max (s)   */
} cd_scenario;

typedef struct cd_ctx cd_ctx;

/* Message of the last failed call on `ctx` (or of the last failed
 * cd_create when ctx is NULL). */
const char *cd_last_error(const cd_ctx *ctx);

/* Create a context for `n_scenarios` scenarios of `body_type`.  Agent and
 * wall ranges must tile [0, total) in scenario order.  Allocates all device
 * memory the step needs. */
int cd_create(cd_ctx **out, int body_type, int64_t n_scenarios,
              const cd_scenario *scenarios);
void cd_destroy(cd_ctx *ctx);

/* Copy `n` (= total agents) packed host records of `itemsize` bytes into the
 * device.  `field_offsets` holds CD_F_COUNT byte offsets (-1 = absent);
 * float64 fields must be 4-byte aligned; the integer and bool fields
 * (CD_F_TARGET and after) may sit at any offset.  Recomputes timestep maxima.
 * Returns once the records have been read: the caller may then reuse them.
 * The per-scenario maxima are computed on the context stream: by the same
 * pass that reads page-locked records, else behind the staged copy. */
int cd_upload_agents(cd_ctx *ctx, const void *records, int64_t n,
                     int64_t itemsize, const int64_t *field_offsets);
/* Write the device state back into `n` packed host records.  Whole records
 * are written: fields the device does not update keep the values of the
 * last cd_upload_agents. */
int cd_download_agents(cd_ctx *ctx, void *records, int64_t n, int64_t itemsize,
                       const int64_t *field_offsets);
/* `steps` graph steps of the host records in place: cd_upload_agents,
 * cd_launch and cd_download_agents in one call, enqueued together (the host
 * does not wait between them; the records must not be touched until it
 * returns).  The drop-in form of the reference's update() on a host array. */
int cd_step_records(cd_ctx *ctx, void *records, int64_t n, int64_t itemsize,
                    const int64_t *field_offsets, int nodes, int64_t steps);
/* Host records in pinned (page-locked, device-mapped) memory are read and
 * written by the device directly, copy and transpose in one kernel pass;
 * other host memory goes through a staged copy.  Both give the same bytes.
 * `enable` = 0 makes every transfer staged (default 1). */
int cd_set_direct_host_access(cd_ctx *ctx, int enable);

/* Asynchronous snapshot for SaveSimulationData (simulation/logic.py:264-337):
 * enqueue on the context stream, behind the steps already enqueued, the
 * copy of the agent state into `n` packed host records (layout as uploaded;
 * page-locked memory makes the copy asynchronous), and of every scenario's
 * dt and time_tot (may be NULL), then record completion in `slot` (0 ..
 * CD_SNAPSHOT_SLOTS - 1).  Returns at once.  cd_snapshot_wait blocks until
 * the snapshot of `slot` is in host memory; it may be called from another
 * host thread. */
#define CD_SNAPSHOT_SLOTS 8
int cd_snapshot_agents(cd_ctx *ctx, int slot, void *records, int64_t n, int64_t itemsize,
                       const int64_t *field_offsets, double *dt, double *time_tot);
int cd_snapshot_wait(cd_ctx *ctx, int slot);

/* ---- state nodes between steps ------------------------------------------ */
/* LeaderFollowerWithHerding (with_herding = 1; simulation/logic.py:183-217 with
 * leader_follower_with_herding_interaction, core/steering/collective_motion.py:
 * 246-279) or LeaderFollower (with_herding = 0; logic.py:168-180 with
 * leader_follower_interaction, :221-243) for every follower: the target
 * direction, target and index_leader (and, with herding, the nearest
 * `size_nearest_other` <= 16 unobstructed neighbours within `sight_follower`,
 * on a cell list of that cell size).  Reference arguments: sight_leader 20
 * (herding) or the node's sight, phi 0.45 pi, weights 0.15 (herding
 * position), 0.40 (leader position), 0.65 (leader direction).  A record
 * that is both leader and follower is rejected with CD_ERR_INVALID_VALUE
 * before any state changes (the reference's serial follower loop would read
 * targets it has already updated in that case). */
int cd_herding(cd_ctx *ctx, int with_herding, double sight_follower,
               int64_t size_nearest_other, double sight_leader, double phi,
               double w_herding, double w_leader, double w_direction);
/* InsideDomain (simulation/logic.py:343-357): `active` = position inside the
 * polygon (n_vertices (x, y) pairs, a ring) for the scenario's agents;
 * `changed` receives the number of agents whose state flipped. */
int cd_inside_domain(cd_ctx *ctx, int64_t scenario, const double *xy, int64_t n_vertices,
                     int64_t *changed);
/* ExitDetection (simulation/logic.py:220-237, core/evacuation.py:139-174): for
 * the scenario's agents, the nearest of the `n_doors` door centres (x, y
 * pairs) within `detection_range` in line of sight; a follower that detects
 * one takes it as its target and stops following. */
int cd_exit_detection(cd_ctx *ctx, int64_t scenario, const double *centers, int64_t n_doors,
                      double detection_range);
/* TargetReached (simulation/logic.py:360-387): per target polygon t (vertices
 * xy[vertex_offsets[t] .. vertex_offsets[t+1])), remember the agents found
 * inside it (since the first call, or since `reset`) and return their
 * number in counts[t].  At most 256 targets. */
int cd_target_reached(cd_ctx *ctx, int64_t scenario, int64_t n_targets, const double *xy,
                      const int64_t *vertex_offsets, int reset, int64_t *counts);

/* Replace all walls: `n_walls` rows of (p0x, p0y, p1x, p1y) float64, split
 * among scenarios by their wall ranges.  Walls are binned into the cells of
 * their scenario's grid. */
int cd_set_walls(cd_ctx *ctx, const double *walls, int64_t n_walls);

/* Direction maps of scenario `scenario` for CD_NODE_NAVIGATION: for each of
 * `n_targets` targets, dir_x and dir_y (ny x nx float64, row = y) on the
 * meshgrid with origin (minx, miny) and spacing `step`, targets stored one
 * after another.  An agent whose `target` field is t in [0, n_targets) takes
 * map t's entry at index ((position - origin) / step) truncated toward zero,
 * (y, x) as (row, column), when inside the map; other agents keep their
 * target direction.  n_targets = 0 removes the scenario's maps. */
int cd_set_direction_maps(cd_ctx *ctx, int64_t scenario, int64_t n_targets,
                          const double *dir_x, const double *dir_y, int64_t ny, int64_t nx,
                          double minx, double miny, double step);

/* Where CD_NODE_FLUCTUATION's noise comes from.  device = 0 (default): host
 * arrays passed by cd_set_noise before each such step.  device = 1: drawn on
 * the device from a Philox4x32-10 counter generator keyed by `seed`, one
 * counter value per step (the step after this call uses step + 1), one
 * stream per agent: force = mass * std_rand_force * xi * (cos phi, sin phi),
 * xi ~ N(0,1) on [0, 3], phi ~ U(0, 2 pi); torque = inertia_rot *
 * std_rand_torque * eta, eta ~ N(0,1) on [-3, 3] (Box-Muller with
 * rejection).  Device noise also runs inside cd_run / cd_launch graphs. */
int cd_set_noise_mode(cd_ctx *ctx, int device, uint64_t seed, uint64_t step);

/* Host-drawn fluctuation added by the next step that runs
 * CD_NODE_FLUCTUATION: force (n x 2) and torque (n; ignored for Circular,
 * may be NULL). */
int cd_set_noise(cd_ctx *ctx, const double *force, const double *torque);

/* Run one update with the selected nodes (CD_NODE_* flags).  If `dt` is not
 * NULL the call waits for the step and writes each scenario's timestep. */
int cd_step(cd_ctx *ctx, int nodes, double *dt);
/* Run `steps` updates with the selected nodes as one CUDA-graph launch per
 * step (captured on first use).  CD_NODE_FLUCTUATION needs device noise.
 * Waits for completion and checks the device status. */
int cd_run(cd_ctx *ctx, int nodes, int64_t steps);
/* Wait for all work of the context and report device-side errors. */
int cd_synchronize(cd_ctx *ctx);
/* Per-scenario last timestep and accumulated time (simulation.data['dt'],
 * simulation.data['time_tot']). */
int cd_get_time(cd_ctx *ctx, double *dt, double *time_tot);

/* Diagnostics: the cell list of the last step that ran CD_NODE_AGENT_AGENT
 * (keys: flat cell index per agent within its scenario's grid; order: agent
 * indices grouped by cell, ascending inside a cell; count/offset per cell of
 * all scenarios, scenarios concatenated). */
int cd_get_cell_list(cd_ctx *ctx, int64_t *keys, int64_t *order,
                     int64_t *cells_count, int64_t *cells_offset);
/* Diagnostics for the current state, per agent, CD_COUNT_COLS int64 each
 * (row-major n x CD_COUNT_COLS): candidate partners (same or adjacent cell),
 * partners that survive the conservative distance pre-check, partners with
 * skin distance h < 3 (interacting), partners with h < 0 (contact), wall
 * segments that survive the pre-check, walls in contact.  Summing one of
 * these pair columns over agents counts every unordered pair twice.  Then,
 * over the interacting pairs whose first agent (in the cell-list order) is
 * this one, so each unordered pair once: pairs whose social force runs its
 * sub-pair loop, sub-pairs with a defined time-to-collision root, pairs with
 * a valid time-to-collision (a force is computed). */
#define CD_COUNT_COLS 9
int cd_pair_counts(cd_ctx *ctx, int64_t *counts);

/* Total cells over all scenarios and agents/walls of the context. */
int cd_sizes(const cd_ctx *ctx, int64_t *n_agents, int64_t *n_walls,
             int64_t *n_cells);

/* Timing: when enabled, cd_step records CUDA events on the context stream
 * around the whole step and around the agent-force kernel, and cd_run
 * around its graph launches; cd_kernel_time returns the accumulated
 * milliseconds since the last cd_set_timing: force kernel (and its launch
 * count), whole cd_step steps, and cd_run steps (and their count).
 * `enable`: 0 off; 1 all of these, the step graph then holding event nodes
 * around the force stage and the pair stage (one-step cd_run calls accumulate
 * them); 2 cd_step's events and cd_run's around its launches only, the step
 * graph holding no event node (the kernels of a step stay chained to each
 * other, as with timing off). */
int cd_set_timing(cd_ctx *ctx, int enable);
int cd_kernel_time(cd_ctx *ctx, double *force_ms, int64_t *force_launches,
                   double *step_ms, double *run_ms, int64_t *run_steps);
/* Time and launches of the pair stage (the float32 pair pass and the pair
 * kernel; pair-pipeline variants, steps with agent-agent), accumulated like
 * cd_kernel_time (timing mode 1). */
int cd_pair_kernel_time(cd_ctx *ctx, double *ms, int64_t *launches);
/* The same split into the float32 pair pass (k_pairs_light) and the float64
 * pair kernels (k_pairs, and k_pair_forces for pair_pipeline 2); light_ms is
 * 0 without a float32 pass. */
int cd_pair_kernel_times(cd_ctx *ctx, double *light_ms, double *pairs_ms, int64_t *launches);
/* The last pair-pipeline step's flat pair list: its pairs, those in its
 * first part (guessed to need the social force) and, for ThreeCircle
 * contexts, those the float32 pass left to the float64 pair kernel (zeros
 * when no near lists are in use).  Waits for the context stream. */
int cd_pair_split(cd_ctx *ctx, int64_t *pairs, int64_t *first_part, int64_t *deferred);
/* Number of kernels one step with `nodes` launches (memsets excluded). */
int cd_kernels_per_step(const cd_ctx *ctx, int nodes, int64_t *kernels);

/* Launch variants of the agent-force kernel: threads per block, candidates
 * staged per thread per pass (lanes_per_agent == 1: one lane per agent) or
 * lanes that share one agent (lanes_per_agent > 1, staged_per_thread 0), and
 * whether the variant is the compute-once pair pipeline (pair_pipeline 1 or
 * 2: every unordered pair evaluated once into per-agent near lists, then
 * summed per agent in visiting order; 2 computes the forces of the pairs
 * that have one in a separate pass; the lists' device memory is allocated on
 * first use and grown after a step that needed more, that step falling back
 * to the lane-group kernel).  Every variant gives bit-identical results;
 * only the speed differs, so an autotuner may pick one per context (the
 * choice is applied to the next captured graph).  A new context starts with
 * a variant chosen from its agent count. */
int cd_variant_count(int *count);
int cd_variant_shape(int variant, int *threads_per_block, int *staged_per_thread,
                     int *lanes_per_agent, int *pair_pipeline);
int cd_set_variant(cd_ctx *ctx, int variant);
/* Near-list entries of the pair pipeline: `entries` >= 0 fixes the capacity
 * (no growth; steps that need more run the lane-group kernel instead, with
 * identical results); a negative value returns to automatic sizing, which
 * grows the current capacity after a step that needed more. */
int cd_set_near_list_capacity(cd_ctx *ctx, int64_t entries);

/* Enqueue `steps` CUDA-graph launches of a step with `nodes` on the context
 * stream and return at once (no host synchronisation), so several contexts
 * (for example one per body type of a mixed batch) run concurrently.  Device
 * errors surface at the next cd_synchronize / cd_run. */
int cd_launch(cd_ctx *ctx, int nodes, int64_t steps);

/* Measured FP64 FMA throughput of the current device in GFLOP/s (2 flops
 * per FMA), used as the roofline denominator. */
int cd_measure_fp64_peak(double *gflops);

/* ---- differentiable rollout (Circular agents, one scenario) -------------
 * Runs `steps` updates (adjusting, agent-agent, agent-wall, integrate,
 * reset) from the current state and writes
 *   loss = (1 / (steps * n)) * sum_t sum_i |x_i(t) - target[t][i]|^2
 * where x(t) is the position after step t and `target` holds steps x n x 2
 * float64 (host).  With `grads` non-NULL it also runs the hand-written
 * adjoint of the whole rollout -- a checkpoint of (x, v, force_prev) every
 * `checkpoint_every` steps, recomputation of each segment, and the reverse
 * step -- and writes d loss / d (tau_adj, target_velocity, tau_0, k_soc) for
 * every agent (n x 4).  The context ends in the rollout's final state.
 * Replaces nothing in the reference (which has no gradients); the forward
 * part is the same step as cd_step.  `forward_ms` / `adjoint_ms` (may be
 * NULL) receive the device time of the forward rollout and of the reverse
 * sweep (recomputation included).  The first call with `grads` makes a second
 * context inside this one (the same scenarios, walls and agents, its own
 * device buffers and stream), on which each segment is recomputed while the
 * reverse step runs the segment after it; cd_destroy releases it. */
int cd_rollout_loss(cd_ctx *ctx, int64_t steps, const double *target,
                    int64_t checkpoint_every, double *loss, double *grads,
                    double *forward_ms, double *adjoint_ms);

/* ---- groups: the steps of several contexts in one graph launch ---------
 * The batched form (several contexts, e.g. one per body type, each holding
 * many scenarios) advanced by one CUDA-graph launch: the group captures
 * `steps_per_launch` steps of `nodes` of every member into one graph, each
 * member's steps exactly as cd_launch runs them (results are the same as
 * the members stepped one by one), the members advancing independently
 * inside it.  Replaces the reference's loop of MultiAgentSimulation.update()
 * over independent simulations (simulation/multiagent.py:51-55, one call
 * per scenario and step).  The members must outlive the group; a launch is
 * ordered after work already enqueued on each member and before work
 * enqueued on them afterwards.  A member whose buffers, variant or walls
 * change is recaptured at the next launch.  cd_group_synchronize waits for
 * the launches and checks every member's status.  Errors: the group's
 * message (cd_group_last_error; the creation's with a NULL group). */
typedef struct cd_group cd_group;
int cd_group_create(cd_group **out, cd_ctx *const *ctxs, int64_t n_ctxs, int nodes,
                    int64_t steps_per_launch);
int cd_group_launch(cd_group *group, int64_t launches);
int cd_group_synchronize(cd_group *group);
const char *cd_group_last_error(const cd_group *group);
void cd_group_destroy(cd_group *group);

/* ---- agent-agent forces without any device allocation ------------------
 * No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory while they run -- for example a host
 * application that owns all device memory through its own pool, or code
 * running where cudaMalloc is not allowed.  It computes the same
 * agent-agent forces as CD_NODE_AGENT_AGENT for one scenario, but keeps its
 * cell list and staging buffers in a fixed array that the library holds on
 * every device that loads it, for the life of the process
 * (about 3.9 MB).  It calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *
 * Limits: n <= CD_NOALLOC_MAX_AGENTS and nx * ny <= CD_NOALLOC_MAX_CELLS;
 * larger inputs are rejected with CD_ERR_CAPACITY before any device work.
 * `cols` is a device array of column-major float64 columns of length n,
 * column k at cols + k * n, in CD_NA_* order (Circular reads columns 0-10,
 * ThreeCircle reads 0-9 and 11-18).  Forces are added to the device arrays
 * force_x / force_y (and the torque to `torque`, ThreeCircle only), as the
 * reference adds to agents['force'] in place.  Work runs on `stream` (a
 * cudaStream_t; NULL = default stream) and the call returns after it ends.
 *
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  The address is kept for the life of the process: after a
 * cudaDeviceReset (or any teardown of the device's primary context) it is
 * stale, and the entry point must not be called on that device again.  All
 * calls share the one array: calls whose work overlaps on the GPU (other
 * host threads, or other streams) race and must not be issued.  Positions
 * farther than 1e7 m from (x0, y0) are rejected with CD_ERR_INVALID_VALUE
 * (the step's float32 pre-checks are exact only within that range). */
#define CD_NOALLOC_MAX_AGENTS 16384
#define CD_NOALLOC_MAX_CELLS 16384
enum {
    CD_NA_X = 0, CD_NA_Y, CD_NA_VX, CD_NA_VY, CD_NA_MASS, CD_NA_K_SOC, CD_NA_TAU_0,
    CD_NA_MU, CD_NA_KAPPA, CD_NA_DAMPING, CD_NA_RADIUS, CD_NA_R_T, CD_NA_R_S,
    CD_NA_R_TS, CD_NA_X_LS, CD_NA_Y_LS, CD_NA_X_RS, CD_NA_Y_RS, CD_NA_ORIENTATION,
    CD_NA_NCOLS
};
int cd_agent_agent_noalloc(int body_type, int64_t n, const double *cols,
                           double *force_x, double *force_y, double *torque,
                           double x0, double y0, double cell_size, int64_t nx,
                           int64_t ny, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CDGPU_H */
