/*
 * kgmt.h -- C ABI of the GB300 KGMT planner (libkgmt.so).
 *
 * Drop-in for the reference planner's public surface (nipe1783/KGMT):
 *   construction           KGMT::KGMT()            src/planners/KGMT.cu:4-39,
 *                          Planner::Planner()       src/planners/Planner.cu:4-35,
 *                          compile-time config      include/config/config.h:209-307
 *                          -> kgmt_create(config)
 *   plan                   virtual void plan(float* h_initial, float* h_goal,
 *                                            float* d_obstacles_ptr,
 *                                            uint h_obstaclesCount)
 *                          include/planners/Planner.cuh:26, KGMT.cuh:12,
 *                          src/planners/KGMT.cu:41-105
 *                          -> kgmt_plan (same argument order and ownership:
 *                             host start/goal rows, caller-owned DEVICE
 *                             obstacle array of [n][6] floats min xyz, max xyz)
 *   readout                public fields h_treeSize_, h_itr_, h_pathToGoal_,
 *                          h_controlPathToGoal_, d_treeSamples_,
 *                          d_treeSamplesParentIdxs_, d_treeSampleCosts_
 *                          include/planners/Planner.cuh:31-41
 *                          -> kgmt_get_result, kgmt_copy_tree, kgmt_copy_path,
 *                             kgmt_device_tree
 *
 * Every call returns a kgmt_status; kgmt_last_error() describes the last
 * failure of the calling thread.  A planner handle is bound to one CUDA stream
 * and is not thread safe; distinct handles may be used from distinct threads.
 * There is no CPU fallback: without a CUDA device every planning call returns
 * KGMT_ERR_NO_DEVICE.
 */
#ifndef KGMT_H
#define KGMT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGMT_ABI_VERSION 1

#if defined(__GNUC__)
#define KGMT_API __attribute__((visibility("default")))
#else
#define KGMT_API
#endif

typedef enum kgmt_status {
    KGMT_OK = 0,
    KGMT_ERR_INVALID_ARG = 1,
    KGMT_ERR_OOM = 2,        /* device memory (or the configured budget) exhausted */
    KGMT_ERR_CAPACITY = 3,   /* too many queries for the batch / server slots */
    KGMT_ERR_TIMEOUT = 4,    /* a bounded device-side wait gave up; results invalid */
    KGMT_ERR_CUDA = 5,
    KGMT_ERR_NO_DEVICE = 6,
    KGMT_ERR_NOT_READY = 7,  /* nothing planned yet / result not available */
    KGMT_ERR_INTERNAL = 8
} kgmt_status;

/* dynamics models, numbered like the reference's MODEL macro (config.h,
 * statePropagator.cu:375-390) */
#define KGMT_MODEL_UNICYCLE 0        /* planar: 2-D workspace, boxes [n][4] */
#define KGMT_MODEL_DOUBLE_INTEGRATOR 1
#define KGMT_MODEL_DUBINS_AIRPLANE 2
#define KGMT_MODEL_QUADROTOR 3

/* double-integrator position update */
#define KGMT_DI_RULE_RK4 0       /* classic RK4: p += v h + a h^2 / 2         */
#define KGMT_DI_RULE_REFERENCE 1 /* statePropagator.cu:97-99: (5v + 2ah) h / 6 */

/* per-query outcome */
#define KGMT_QUERY_RUNNING 0
#define KGMT_QUERY_SUCCESS 1    /* a node reached the goal ball            */
#define KGMT_QUERY_ITER_LIMIT 2 /* max_iterations spent without the goal  */
#define KGMT_QUERY_CAPACITY 3   /* tree full before the goal was reached   */
#define KGMT_QUERY_CANCELLED 4  /* withdrawn by kgmt_server_cancel          */

#define KGMT_MAX_SAMPLE_DIM 17
#define KGMT_MAX_FINE_CELLS 64

/* Runtime replacement for the reference's config.h macros.  Workspace-only
 * region grids: coarse_len^W regions (W_R1_LENGTH), fine_len^W cells per
 * region (W_R2_LENGTH, at most 64 cells), W = 3, or 2 for the planar
 * unicycle.  Sample rows are state + control + duration (SAMPLE_DIM):
 *   unicycle          7: x y theta v | a steering dt               (statePropagator.cu:13-74)
 *   double integrator 10: x y z vx vy vz | ax ay az | k*h           (76-142)
 *   Dubins airplane   10: x y z yaw pitch v | yaw-rate pitch-rate a | k*h (147-244)
 *   quadrotor         17: 12 states | Zc Lc Mc Nc | k*h             (246-370)
 * Steps per sample k = min_steps + floor(u * (max_steps - min_steps + 1))
 * (MAX_PROPAGATION_DURATION, STEP_SIZE). */
typedef struct kgmt_config {
    int32_t model;             /* KGMT_MODEL_*                                 */
    int32_t di_rule;           /* KGMT_DI_RULE_*                               */
    uint32_t tree_capacity;    /* MAX_TREE_SIZE                                */
    uint32_t samples_per_node; /* samples per expanded frontier entry          */
    uint32_t max_iterations;   /* MAX_ITER                                     */
    uint32_t min_steps;
    uint32_t max_steps;
    float step_size;
    float goal_radius; /* GOAL_THRESH */
    float epsilon;     /* EPSILON     */
    float ws_min, ws_max;
    uint32_t coarse_len, fine_len;
    float v_min, v_max; /* V_MIN, V_MAX (not checked for the unicycle, as in the reference) */
    /* control bounds, in the reference's draw order: DI ax ay az; quad Zc Lc
     * Mc Nc; Dubins a, yaw rate, pitch rate; unicycle a, steering, dt */
    float u_min[4], u_max[4];
    float nu, mu, ix, iy, iz, gravity, mass_inv; /* quadrotor constants */
    uint64_t seed; /* Philox key of this query */
    float pitch_min, pitch_max; /* Dubins airplane pitch bounds (DUBINS_AIRPLANE_MIN/MAX_PITCH) */
    float wheelbase;            /* unicycle length (UNI_LENGTH) */
    uint32_t reserved;          /* zero */
} kgmt_config;

typedef struct kgmt_result {
    int32_t status;         /* KGMT_QUERY_*                        */
    uint32_t iterations;    /* h_itr_                              */
    uint32_t tree_size;     /* h_treeSize_                         */
    int32_t goal_index;     /* tree index of the goal node or -1   */
    uint32_t path_len;      /* nodes on goal->root path, 0 if none */
    uint32_t samples_drawn; /* samples propagated over the plan    */
    float solve_ms;         /* admission -> completion, device clock           */
    float latency_ms;       /* server: submit -> retirement, host clock        */
    uint64_t ticket; /* server ticket / batch index */
    float goal_cost; /* goal node's distance to the goal (h_costToGoal_), 0 if none */
    uint32_t reserved;
} kgmt_result;

typedef struct kgmt_planner kgmt_planner;
typedef struct kgmt_batch kgmt_batch;
typedef struct kgmt_server kgmt_server;

/* ---- library ---- */
KGMT_API const char* kgmt_version(void);
KGMT_API const char* kgmt_last_error(void);
/* Fills *out with the defaults of a model (unit cube, 8^3/2^3 grid for the
 * double integrator; 16^3/4^3 grid and scaled constants for the quadrotor). */
KGMT_API kgmt_status kgmt_config_default(int32_t model, kgmt_config* out);
KGMT_API kgmt_status kgmt_config_validate(const kgmt_config* cfg);
/* device bytes one query of this config holds (tree, frontier, region tables) */
KGMT_API size_t kgmt_query_bytes(const kgmt_config* cfg, uint32_t n_obstacles);
KGMT_API int32_t kgmt_sample_dim(int32_t model);

/* ---- single query: replaces KGMT::KGMT / KGMT::plan (KGMT.cu:4-105) ---- */
/* stream: a cudaStream_t or NULL for a stream the planner creates */
KGMT_API kgmt_status kgmt_create(const kgmt_config* cfg, void* stream, kgmt_planner** out);
KGMT_API void kgmt_destroy(kgmt_planner* p);
/* h_initial / h_goal: host rows of kgmt_sample_dim(model) floats (only the
 * first W goal components are used); d_obstacles: caller-owned device array
 * [n_obstacles][2W] = min corner, max corner (W = 3; 2 for the unicycle).
 * Blocks until the plan is done. */
KGMT_API kgmt_status kgmt_plan(kgmt_planner* p, const float* h_initial, const float* h_goal, const float* d_obstacles, uint32_t n_obstacles);
KGMT_API kgmt_status kgmt_get_result(const kgmt_planner* p, kgmt_result* out);
/* copies the first min(tree_size, max_nodes) nodes; any pointer may be NULL */
KGMT_API kgmt_status kgmt_copy_tree(kgmt_planner* p, float* h_samples, int32_t* h_parents, float* h_costs, uint32_t max_nodes);
/* goal->root rows of sample_dim floats (h_controlPathToGoal_ layout) */
KGMT_API kgmt_status kgmt_copy_path(kgmt_planner* p, float* h_rows, uint32_t max_rows, uint32_t* n_rows);
/* device pointers of the tree (d_treeSamples_, d_treeSamplesParentIdxs_,
 * d_treeSampleCosts_); valid until the next plan or destroy */
KGMT_API kgmt_status kgmt_device_tree(kgmt_planner* p, const float** d_samples, const int32_t** d_parents, const float** d_costs);

/* ---- traced plan: replaces KGMT::planBench (KGMT.cu:107-165) ----
 * What one iteration left behind, as the reference's writeDeviceVectorsToCSV
 * (KGMT.cu:405-488) dumps it after every iteration.  Host arrays owned by the
 * planner, valid during the hook only. */
typedef struct kgmt_iteration {
    uint32_t itr;                /* h_itr_: the iteration just run (1-based)                      */
    uint32_t tree_size;          /* h_treeSize_ after its append                                  */
    uint32_t frontier_size;      /* h_frontierSize_: distinct frontier nodes it expanded          */
    uint32_t expanded;           /* samples it propagated (the ExpandedNodes value)               */
    uint32_t next_frontier_size; /* distinct nodes on the next frontier                           */
    int32_t goal_index;          /* tree index of the goal node, -1 while none                    */
    uint32_t path_len;           /* goal -> root rows in path once the goal is found, else 0      */
    uint32_t capacity, sample_dim, regions;
    const float* samples;   /* [capacity][sample_dim] d_treeSamples_; rows from tree_size on are 0  */
    const int32_t* parents; /* [capacity] d_treeSamplesParentIdxs_; -1 from tree_size on           */
    const int32_t* counter; /* [regions] samples per region so far (d_counterArray_)               */
    const int32_t* valid;   /* [regions] valid samples per region (d_validCounterArray_)           */
    const float* score;     /* [regions] region scores (d_vertexScoreArray_)                       */
    const uint8_t* frontier; /* [capacity] 1: on the next frontier (d_frontier_)                   */
    const uint32_t* repeat;  /* [capacity] its entries on the next frontier (d_activeFrontierRepeatCount_) */
    const float* path;       /* [path_len][sample_dim] goal -> root (d_controlPathToGoal_)         */
} kgmt_iteration;
typedef void (*kgmt_iteration_hook)(const kgmt_iteration* it, void* user);
/* kgmt_plan, one iteration per launch pair, calling hook(it, user) after
 * every iteration with the state above; the same plan as kgmt_plan (a debug
 * and analysis path: each iteration copies the tree back).  hook may be NULL. */
KGMT_API kgmt_status kgmt_plan_traced(kgmt_planner* p, const float* h_initial, const float* h_goal, const float* d_obstacles,
                                      uint32_t n_obstacles, kgmt_iteration_hook hook, void* user);

/* ---- batched: many independent queries in one device-resident launch chain ---- */
typedef struct kgmt_batch_options {
    uint32_t max_queries;      /* slots                                          */
    uint32_t iters_per_graph;  /* iterations captured per CUDA graph replay (0: 4) */
    uint32_t propagate_block;  /* 0 = autotuned / default                        */
    uint32_t use_graph;        /* 1 = replay a captured CUDA graph                */
    uint32_t profile_kernels;  /* 1 = direct launches bracketed by CUDA events    */
} kgmt_batch_options;

/* counters of the last kgmt_plan_batch* call */
typedef struct kgmt_batch_stats {
    uint64_t kernel_launches;     /* kernels this library launched                 */
    uint64_t steps_executed;      /* RK4 steps over all propagated samples         */
    uint64_t obstacle_tests;      /* step-box x obstacle-box tests                 */
    uint64_t samples;             /* samples propagated                            */
    uint64_t fp32_ops;            /* algorithmic FP32 operations of k_propagate    */
    uint32_t iterations_launched; /* iterations launched (incl. the no-op tail)    */
    uint32_t launches_propagate, launches_tail, launches_append;
    float ms_propagate, ms_tail, ms_append; /* summed CUDA-event time (profile_kernels) */
    uint32_t iterations_tail;     /* iterations run by the persistent tail launches */
    uint32_t reserved;
    uint64_t fp32_ops_tail;       /* the part of fp32_ops the tail launches did      */
    uint64_t samples_tail;        /* the part of samples the tail launches propagated */
} kgmt_batch_stats;

KGMT_API kgmt_status kgmt_batch_create(const kgmt_batch_options* opt, void* stream, kgmt_batch** out);
KGMT_API void kgmt_batch_destroy(kgmt_batch* b);
/* Host buffers: cfgs[n], inits/goals [n][KGMT_MAX_SAMPLE_DIM], obstacles
 * [sum count][6] with per-query offset/count (in boxes).  Copies in, plans all
 * queries to completion, writes results[n].  Blocks. */
KGMT_API kgmt_status kgmt_plan_batch(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits, const float* h_goals,
                            const float* h_obstacles, const uint32_t* obs_offset, const uint32_t* obs_count, kgmt_result* results);
/* Same with inits / goals / obstacles / offsets / counts already in device
 * memory (cfgs and results stay on the host). */
KGMT_API kgmt_status kgmt_plan_batch_device(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* d_inits, const float* d_goals,
                                   const float* d_obstacles, const uint32_t* h_obs_offset, const uint32_t* h_obs_count,
                                   kgmt_result* results);
KGMT_API kgmt_status kgmt_batch_get_stats(kgmt_batch* b, kgmt_batch_stats* out);
/* tree of query i of the last batch (host copy) */
KGMT_API kgmt_status kgmt_batch_copy_tree(kgmt_batch* b, uint32_t i, float* h_samples, int32_t* h_parents, float* h_costs, uint32_t max_nodes);
KGMT_API kgmt_status kgmt_batch_copy_path(kgmt_batch* b, uint32_t i, float* h_rows, uint32_t max_rows, uint32_t* n_rows);
/* picks the propagate block size for a representative batch (sweeps 128, 256, 512) */
KGMT_API kgmt_status kgmt_batch_autotune(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits, const float* h_goals,
                                const float* h_obstacles, const uint32_t* obs_offset, const uint32_t* obs_count,
                                uint32_t* best_block);

typedef struct kgmt_autotune_result {
    uint32_t propagate_block;  /* chosen block size (now the batch's)                        */
    uint32_t samples_per_node; /* chosen samples per expanded node: set it in the configs     */
    float queries_per_s;       /* of the chosen pair (host clock around kgmt_plan_batch)      */
    float success_rate;        /* of the chosen pair                                          */
    float base_queries_per_s;  /* the configs as given, block 256                             */
    float base_success_rate;
} kgmt_autotune_result;

/* sweeps the propagate block size (128, 256, 512) and the samples per
   expanded node (2, 4, 8, 16) on a representative batch and keeps the pair
   with the most queries/s among those whose success rate is at least 95 % of
   the configs' own (samples per node changes the plans, so the caller
   decides whether to adopt it: it is returned, not written into cfgs) */
KGMT_API kgmt_status kgmt_batch_autotune_full(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits,
                                              const float* h_goals, const float* h_obstacles, const uint32_t* obs_offset,
                                              const uint32_t* obs_count, kgmt_autotune_result* out);

/* ---- served: continuous batching with memory-based admission ---- */
typedef struct kgmt_server_options {
    uint32_t max_slots;        /* queries resident at once                      */
    uint64_t memory_budget;    /* bytes of device memory for resident queries   */
    uint32_t iters_per_step;   /* iterations per kgmt_server_step (0: 1)        */
    uint32_t propagate_block;  /* 0 = default                                    */
} kgmt_server_options;

KGMT_API kgmt_status kgmt_server_create(const kgmt_server_options* opt, void* stream, kgmt_server** out);
KGMT_API void kgmt_server_destroy(kgmt_server* s);
/* queues a query (host buffers are copied); it is admitted at the next step
 * with a free slot and enough memory.  Returns its ticket. */
KGMT_API kgmt_status kgmt_server_submit(kgmt_server* s, const kgmt_config* cfg, const float* h_init, const float* h_goal,
                               const float* h_obstacles, uint32_t n_obstacles, uint64_t* ticket);
/* admits what fits, runs iterations for every resident query, retires the
 * finished ones.  *n_running / *n_queued may be NULL. */
KGMT_API kgmt_status kgmt_server_step(kgmt_server* s, uint32_t* n_running, uint32_t* n_queued);
/* takes up to max finished results (FIFO by completion) */
KGMT_API kgmt_status kgmt_server_poll(kgmt_server* s, kgmt_result* out, uint32_t max, uint32_t* n_out);
/* Withdraws a submitted query between steps: a queued one is dropped, a
 * resident one stops where its last step left it and frees its slot and
 * memory.  Either way poll returns its result with status
 * KGMT_QUERY_CANCELLED (a resident one with its iterations and tree size so
 * far).  KGMT_ERR_NOT_READY when no queued or resident query has the ticket
 * (unknown, or already finished). */
KGMT_API kgmt_status kgmt_server_cancel(kgmt_server* s, uint64_t ticket);

/* ---- single query without any allocation ----
 * No counterpart in the reference (its planner allocates everything in its
 * constructor).  For callers that cannot call cudaMalloc: processes whose
 * device memory is owned by a fixed pool set up at start-up, real-time loops
 * that must never enter the allocator, hosts that forbid allocation after
 * initialisation.  The working memory lives in a static device array of
 * KGMT_NOALLOC_SCRATCH_BYTES (32 MiB) that every GPU loading this library
 * holds until exit; its first KGMT_NOALLOC_RESERVED_BYTES hold the planner's
 * descriptors, so a query is accepted when
 *     kgmt_query_bytes(cfg, n_obstacles) + KGMT_NOALLOC_RESERVED_BYTES <= KGMT_NOALLOC_SCRATCH_BYTES
 * and rejected with KGMT_ERR_INVALID_ARG otherwise.
 * The caller passes the start / goal rows (host), the obstacles (device,
 * [n][6]) and device output buffers for up to max_nodes tree nodes
 * (samples [max_nodes][sample_dim], parents, costs) and max_path_rows path
 * rows (goal -> root); any output pointer may be NULL; a host pointer where
 * device memory is expected is rejected with KGMT_ERR_INVALID_ARG.  All calls
 * on a device share that one array and it keeps the last call's contents:
 * calls that overlap on the GPU (other threads, other streams) race and
 * corrupt each other.  The first call on a device (and the first after its
 * CUDA context is recreated) looks up the array's address; make it before
 * any stream capture begins.  Every call waits for its stream before it
 * returns; stream may be NULL. */
#define KGMT_NOALLOC_SCRATCH_BYTES (32u << 20)
#define KGMT_NOALLOC_RESERVED_BYTES 4096u
KGMT_API kgmt_status kgmt_plan_noalloc(const kgmt_config* cfg, const float* h_initial, const float* h_goal, const float* d_obstacles,
                                       uint32_t n_obstacles, float* d_samples, int32_t* d_parents, float* d_costs, uint32_t max_nodes,
                                       float* d_path, uint32_t max_path_rows, kgmt_result* result, void* stream);

/* ---- function-level kernel (tests, tooling) ---- */
/* Propagates n samples: d_x0 [n][D] parents, d_uniforms [n][8] the draws
 * (controls, steps, accept), d_obstacles [m][6].  Outputs d_x1 [n][D],
 * d_valid [n], d_r1 / d_r2 [n] (coarse region, fine cell inside it; may be
 * NULL).  stream may be NULL.  Asynchronous. */
KGMT_API kgmt_status kgmt_propagate_samples(const kgmt_config* cfg, const float* d_x0, const float* d_uniforms, const float* d_obstacles,
                                   uint32_t n_obstacles, uint32_t n, float* d_x1, uint8_t* d_valid, int32_t* d_r1, int32_t* d_r2,
                                   void* stream);

/* ---- failure-detection self-test (no counterpart in the reference) ---- */
/* Runs the planning kernels' bounded look-back wait against a predecessor
 * that never publishes, giving up after `polls` polls (1 .. 4194304).  The
 * wait must time out: returns KGMT_ERR_TIMEOUT with the device error bits in
 * *error_bits (bit 0: look-back timeout), as planning calls do when a bounded
 * wait gives up; the context stays usable.  KGMT_ERR_INTERNAL if it did not
 * time out.  Synchronous; a few kilobytes of device memory. */
KGMT_API kgmt_status kgmt_selftest_bounded_wait(uint32_t polls, uint32_t* error_bits);

#ifdef __cplusplus
}
#endif
#endif /* KGMT_H */
