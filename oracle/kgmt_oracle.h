/*
 * kgmt_oracle.h -- CPU restatement of the KGMT planning loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * planner in kgmt_gb300/ and the timed CPU baseline in bench.py.  Nothing in
 * the product links, loads or calls it.
 *
 * Reference being restated (nipe1783/KGMT):
 *   planner loop          src/planners/KGMT.cu:41-105, 167-211, 218-259, 305-403
 *   repeat expansion      src/planners/Planner.cu:52-79
 *   region ids / scores   src/graphs/Graph.cu:53-97, 99-153, 155-205, 311-358
 *   dynamics              src/statePropagator/statePropagator.cu:13-74 (unicycle),
 *                         76-142 (double integrator), 147-244 (Dubins airplane),
 *                         246-370 (quadrotor)
 *   collision             src/collisionCheck/collisionCheck.cu:3-10, 49-61
 *   goal distance         include/helper/helper.cuh:138-152
 *
 * Two numeric modes:
 *   FP32 "mirror": single precision, no contraction (-ffp-contract=off), the
 *       same operation order as the CUDA kernels -> integer results (region
 *       ids, verdicts, parents, tree sizes) are bit-exact with the GPU.
 *   FP64: the same RK4 in double with the host libm, used as the accuracy
 *       oracle for propagated states (relative 1e-5 with a per-component
 *       scale floor).
 *
 * Parity pinning: the reference's own propagate / collision / getRegion code
 * is compiled on the host by oracle/ref/Makefile and its outputs are stored as
 * fixtures in tests/golden/ (see tests/golden/make_golden.py).
 */
#ifndef KGMT_ORACLE_H
#define KGMT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KO_MODEL_UNICYCLE 0          /* reference MODEL 0 (config.h), planar */
#define KO_MODEL_DOUBLE_INTEGRATOR 1 /* reference MODEL 1 (config.h) */
#define KO_MODEL_DUBINS_AIRPLANE 2   /* reference MODEL 2 (config.h) */
#define KO_MODEL_QUADROTOR 3         /* reference MODEL 3 (config.h) */

#define KO_DI_RULE_RK4 0       /* classic RK4 position update            */
#define KO_DI_RULE_REFERENCE 1 /* statePropagator.cu:97-99 formula as is */

#define KO_STATUS_RUNNING 0
#define KO_STATUS_SUCCESS 1
#define KO_STATUS_ITER_LIMIT 2
#define KO_STATUS_CAPACITY 3

#define KO_MAX_SAMPLE_DIM 17
#define KO_SCORE_LANES 256
#define KO_NEW_NODE_REPEAT_SPARSE 15 /* KGMT.cu:336-337 */
#define KO_NEW_NODE_REPEAT_DENSE 1   /* KGMT.cu:338-339 */
#define KO_ROOT_REPEAT 5             /* KGMT.cu:67 */
#define KO_SPARSE_VALID_LIMIT 10     /* KGMT.cu:336 */

typedef struct ko_config {
    int32_t model;
    int32_t di_rule;
    uint32_t tree_capacity;
    uint32_t samples_per_node;
    uint32_t max_iterations;
    uint32_t min_steps;
    uint32_t max_steps;
    float step_size;
    float goal_radius;
    float epsilon;
    float ws_min;
    float ws_max;
    uint32_t coarse_len;
    uint32_t fine_len;
    float v_min;
    float v_max;
    float u_min[4];
    float u_max[4];
    float nu, mu, ix, iy, iz, gravity, mass_inv;
    uint64_t seed;
    float pitch_min, pitch_max; /* Dubins airplane */
    float wheelbase;            /* unicycle */
    uint32_t reserved;
} ko_config;

typedef struct ko_result {
    int32_t status;
    uint32_t iterations;
    uint32_t tree_size;
    int32_t goal_index;
    uint32_t path_len;
    uint32_t samples_drawn; /* sum over iterations of samples propagated */
} ko_result;

/* Per-iteration trace (optional) for step-by-step comparison. */
typedef struct ko_iter_trace {
    uint32_t itr;
    uint32_t tree_size_before;
    uint32_t n_samples;
    uint32_t samples_per_entry;
    uint32_t n_next;
    uint32_t n_react;
    uint32_t repeat_total;
    float f_accept;
    float score_total;
} ko_iter_trace;

/* ---- building blocks ---- */
void ko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float ko_u01(uint32_t x);
/* mismatches of the fused-multiply-add replacement of x / 6 over two binades */
long ko_check_div6(void);
void ko_sincosf(float x, float* s, float* c);
int ko_sample_dim(int32_t model);
int ko_state_dim(int32_t model);

/* draws the 8 uniforms a propagation sample consumes (two Philox blocks) */
void ko_sample_uniforms(uint64_t seed, uint32_t slot, uint32_t itr, float u[8]);
float ko_react_uniform(uint64_t seed, uint32_t node, uint32_t itr);

/* workspace dimension W: 2 for the planar unicycle, else 3.  Obstacle boxes
 * passed to the functions below are rows of 2W floats (min corner, max
 * corner), as the reference lays them out (collisionCheck.cu:53-57), except
 * in ko_plan_batch, whose rows are always 6 floats. */
int ko_ws_dims(int32_t model);
int ko_region(const ko_config* c, const float* x);
int ko_subregion(const ko_config* c, const float* x, int r1);
float ko_distance(const float* a, const float* b);             /* 3-D */
float ko_distance_w(const float* a, const float* b, int w);    /* first w components */
int ko_segment_valid(const float* p0, const float* p1, const float* obstacles, uint32_t n_obs); /* 3-D */

/* FP32 mirror propagation of n samples with explicit uniforms u[n*8].
 * x0: n*sample_dim, x1: n*sample_dim, valid: n bytes. */
void ko_propagate_f32(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs, uint32_t n,
                      float* x1, uint8_t* valid, int32_t* r1, int32_t* r2);
/* FP64 RK4 oracle.  Controls are the same float values as the FP32 path. */
void ko_propagate_f64(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs, uint32_t n,
                      double* x1, uint8_t* valid);
/* minimum distance (over steps taken in FP64) between the swept step boxes
 * and any obstacle face; used to classify verdict mismatches */
double ko_verdict_margin_f64(const ko_config* c, const float* x0, const float* u, const float* obstacles, uint32_t n_obs);

/* Region score update (Graph.cu:311-358 with the defects fixed) */
void ko_score_update(const ko_config* c, const int32_t* counter, const int32_t* valid, uint64_t* marks, uint64_t* newmarks,
                     float* score, float* total_out);
float ko_f_accept(uint32_t itr, float eps, uint32_t tree_size, uint32_t n_next, uint32_t capacity);

/* What one iteration leaves behind, for the per-iteration dump of the
 * reference's planBench (KGMT.cu:107-165, writeDeviceVectorsToCSV 405-488):
 * sizes, the cumulative region tables after the iteration's scores, and the
 * next frontier as the two index lists (re-activated nodes, then new nodes
 * each repeated 15 or 1 times).  Pointers are valid during the hook only. */
typedef struct ko_iter_view {
    uint32_t itr;
    uint32_t tree_size;     /* after the iteration's append */
    uint32_t frontier_size; /* distinct frontier nodes the iteration expanded */
    uint32_t expanded;      /* samples it propagated */
    uint32_t n_react, n_rep_new;
    int32_t goal_index;     /* -1 while none */
    uint32_t regions;
    const uint32_t* rep_old;
    const uint32_t* rep_new;
    const int32_t* counter;
    const int32_t* valid;
    const float* score;
} ko_iter_view;
typedef void (*ko_iter_hook)(const ko_iter_view* view, void* user);

/* Whole plan (FP32 mirror).  samples: capacity*sample_dim, parents/costs:
 * capacity; path: (max_iterations+2)*sample_dim rows goal->root.  trace may be
 * NULL or hold max_iterations entries. */
int ko_plan(const ko_config* c, const float* init, const float* goal, const float* obstacles, uint32_t n_obs, ko_result* res,
            float* samples, int32_t* parents, float* costs, float* path, ko_iter_trace* trace);
/* ko_plan calling hook(view, user) after every iteration */
int ko_plan_hooked(const ko_config* c, const float* init, const float* goal, const float* obstacles, uint32_t n_obs, ko_result* res,
                   float* samples, int32_t* parents, float* costs, float* path, ko_iter_trace* trace, ko_iter_hook hook, void* user);

/* n independent queries; OpenMP over queries with `threads` threads (0 = all).
 * Only results (no trees) are returned.  obstacles concatenated as rows of 6
 * floats (a planar query uses the x and y extents), obs_offset in boxes. */
int ko_plan_batch(uint32_t nq, const ko_config* cfgs, const float* inits, const float* goals, const float* obstacles,
                  const uint32_t* obs_offset, const uint32_t* obs_count, ko_result* res, int threads);
int ko_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
