// kgmt_abi.cu -- the C ABI (include/kgmt.h): single planner, batch, server
// and the function-level propagation entry.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <new>
#include <vector>

#include "../../include/kgmt.h"
#include "kgmt_engine.h"

using namespace kgmt;

namespace kgmt {
extern thread_local std::string g_last_error;
}

#define RETURN_IF(cond, code, msg) \
    do {                           \
        if(cond)                   \
            {                      \
                set_error(msg);    \
                return code;       \
            }                      \
    } while(0)

#define CHECK_ST(expr)                      \
    do {                                    \
        kgmt_status st_ = (expr);           \
        if(st_ != KGMT_OK) return st_;      \
    } while(0)

// ---------------------------------------------------------------------------
// library
// ---------------------------------------------------------------------------
extern "C" const char* kgmt_version(void) { return "kgmt-gb300 1.0 (sm_103a)"; }

extern "C" const char* kgmt_last_error(void) { return kgmt::g_last_error.c_str(); }

extern "C" int32_t kgmt_sample_dim(int32_t model)
{
    if(model < KGMT_MODEL_UNICYCLE || model > KGMT_MODEL_QUADROTOR) return -1;
    return (int32_t)sample_dim_of(model);
}

extern "C" kgmt_status kgmt_config_default(int32_t model, kgmt_config* out)
{
    RETURN_IF(!out, KGMT_ERR_INVALID_ARG, "kgmt_config_default: out is NULL");
    kgmt_config c;
    std::memset(&c, 0, sizeof(c));
    c.model = model;
    c.di_rule = KGMT_DI_RULE_RK4;
    c.epsilon = 1e-2f;
    c.ws_min = 0.0f;
    c.ws_max = 1.0f;
    c.goal_radius = 0.05f;
    c.v_min = -0.3f;
    c.v_max = 0.3f;
    c.nu = 10e-3f;
    c.mu = 2e-6f;
    c.ix = 1.0f;
    c.iy = 1.0f;
    c.iz = 2.0f;
    c.mass_inv = 1.0f;
    c.seed = 1;
    c.pitch_min = -3.14159265358979323846f / 3.0f;
    c.pitch_max = 3.14159265358979323846f / 3.0f;
    c.wheelbase = 1.0f;
    if(model == KGMT_MODEL_DOUBLE_INTEGRATOR)
        {
            c.tree_capacity = 100000;
            c.samples_per_node = 4;
            c.max_iterations = 200;
            c.min_steps = 1;
            c.max_steps = 6;
            c.step_size = 0.05f;
            c.coarse_len = 8;
            c.fine_len = 2;
            for(int i = 0; i < 3; ++i) c.u_min[i] = -1.0f, c.u_max[i] = 1.0f;
            c.gravity = -9.81f;
        }
    else if(model == KGMT_MODEL_QUADROTOR)
        {
            const float pi = 3.14159265358979323846f;
            c.tree_capacity = 2000000;
            c.samples_per_node = 8;
            c.max_iterations = 200;
            c.min_steps = 3;
            c.max_steps = 15;
            c.step_size = 0.02f;
            c.coarse_len = 16;
            c.fine_len = 4;
            c.u_min[0] = 0.0f, c.u_max[0] = 0.3f;
            for(int i = 1; i < 4; ++i) c.u_min[i] = -pi, c.u_max[i] = pi;
            c.gravity = -0.0981f;
        }
    else if(model == KGMT_MODEL_DUBINS_AIRPLANE)
        {
            // the reference's Dubins airplane block of config.h (workspace-only grid)
            const float pi = 3.14159265358979323846f;
            c.tree_capacity = 200000;
            c.samples_per_node = 4;
            c.max_iterations = 300;
            c.min_steps = 1;
            c.max_steps = 10;
            c.step_size = 0.1f;
            c.coarse_len = 8;
            c.fine_len = 2;
            c.v_min = 0.0f;
            c.v_max = 0.3f;
            c.u_min[0] = -0.3f, c.u_max[0] = 0.3f;                    // a
            c.u_min[1] = -pi / 4.0f, c.u_max[1] = pi / 4.0f;          // yaw rate
            c.u_min[2] = -pi / 4.0f, c.u_max[2] = pi / 4.0f;          // pitch rate
        }
    else if(model == KGMT_MODEL_UNICYCLE)
        {
            // the reference's unicycle constants (config.h UNI_*), planar unit square
            const float pi = 3.14159265358979323846f;
            c.tree_capacity = 100000;
            c.samples_per_node = 4;
            c.max_iterations = 200;
            c.min_steps = 1;
            c.max_steps = 10;
            c.step_size = 0.1f;
            c.coarse_len = 8;
            c.fine_len = 4;
            c.u_min[0] = -0.2f, c.u_max[0] = 0.2f;                    // a
            c.u_min[1] = -pi / 2.0f, c.u_max[1] = pi / 2.0f;          // steering
            c.u_min[2] = 0.1f, c.u_max[2] = 2.0f;                     // dt (UNI_MIN_DT, UNI_MAX_DT)
        }
    else
        {
            set_error("kgmt_config_default: unknown model");
            return KGMT_ERR_INVALID_ARG;
        }
    *out = c;
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_config_validate(const kgmt_config* cfg)
{
    RETURN_IF(!cfg, KGMT_ERR_INVALID_ARG, "config is NULL");
    return validate_config(*cfg);
}

extern "C" size_t kgmt_query_bytes(const kgmt_config* cfg, uint32_t n_obstacles)
{
    if(!cfg || validate_config(*cfg) != KGMT_OK) return 0;
    return layout_of(*cfg, n_obstacles, true).total;
}

// ---------------------------------------------------------------------------
// single planner
// ---------------------------------------------------------------------------
struct kgmt_planner {
    Engine eng;
    DeviceArena arena;
    kgmt_config cfg;
    QueryParams params;
    QueryState state;
    bool planned = false;
};

extern "C" kgmt_status kgmt_create(const kgmt_config* cfg, void* stream, kgmt_planner** out)
{
    RETURN_IF(!cfg || !out, KGMT_ERR_INVALID_ARG, "kgmt_create: NULL argument");
    *out = nullptr;
    CHECK_ST(validate_config(*cfg));
    kgmt_planner* p = new(std::nothrow) kgmt_planner();
    RETURN_IF(!p, KGMT_ERR_OOM, "kgmt_create: host allocation failed");
    p->cfg = *cfg;
    kgmt_status st = p->eng.init(1, (cudaStream_t)stream, 256, 4, true);
    if(st == KGMT_OK) st = p->arena.reserve(layout_of(*cfg, 0, true).total);
    if(st != KGMT_OK)
        {
            delete p;
            return st;
        }
    *out = p;
    return KGMT_OK;
}

extern "C" void kgmt_destroy(kgmt_planner* p) { delete p; }

// set-up shared by kgmt_plan and kgmt_plan_traced: the query's buffers in
// the planner's arena, its boxes staged, the query admitted and the first
// schedule computed (KGMT.cu:48-81)
static kgmt_status plan_setup(kgmt_planner* p, const float* h_initial, const float* h_goal, const float* d_obstacles, uint32_t n_obstacles,
                              const char* who)
{
    RETURN_IF(!p || !h_initial || !h_goal, KGMT_ERR_INVALID_ARG, std::string(who) + ": NULL argument");
    RETURN_IF(n_obstacles > 0 && !d_obstacles, KGMT_ERR_INVALID_ARG, std::string(who) + ": obstacles pointer is NULL");
    RETURN_IF(n_obstacles > 0 && !is_device_pointer(d_obstacles), KGMT_ERR_INVALID_ARG,
              std::string(who) + ": obstacles must be a device pointer (as in KGMT::plan)");
    p->planned = false;
    const QueryLayout L = layout_of(p->cfg, n_obstacles, true);
    p->arena.reset();
    CHECK_ST(p->arena.reserve(L.total));
    size_t off = 0;
    RETURN_IF(!p->arena.alloc(L.total, &off), KGMT_ERR_OOM, std::string(who) + ": arena allocation failed");
    p->params = make_params(p->cfg, h_initial, h_goal, p->arena.base() + off, L, nullptr, n_obstacles);
    CHECK_ST(cuda_status(launch_stage_obstacles(d_obstacles, p->params.obstacles, n_obstacles, (int)ws_dims_of(p->cfg.model), p->eng.stream()),
                         "stage obstacles"));
    p->eng.host_params(0) = p->params;
    p->eng.set_models(Engine::model_bit(p->cfg.model));
    p->eng.set_max_obstacles(n_obstacles);
    return p->eng.admit(0, 1, 1);
}

extern "C" kgmt_status kgmt_plan(kgmt_planner* p, const float* h_initial, const float* h_goal, const float* d_obstacles,
                                 uint32_t n_obstacles)
{
    CHECK_ST(plan_setup(p, h_initial, h_goal, d_obstacles, n_obstacles, "kgmt_plan"));
    CHECK_ST(p->eng.run_until_done(p->cfg.max_iterations));
    CHECK_ST(p->eng.extract_paths(1));
    uint32_t err = 0;
    CHECK_ST(p->eng.read_states_and_error(0, 1, &p->state, &err));
    RETURN_IF(err != 0, KGMT_ERR_TIMEOUT, "kgmt_plan: a device-side wait gave up (error bits " + std::to_string(err) + ")");
    RETURN_IF(bounds_error_take() != 0, KGMT_ERR_INTERNAL, "kgmt_plan: an index check failed (bounds-checked build)");
    p->planned = true;
    return KGMT_OK;
}

// device -> pageable host copy on the planner's stream, waited for
static kgmt_status copy_back(cudaStream_t s, void* dst, const void* src, size_t bytes, const char* what)
{
    if(bytes == 0) return KGMT_OK;
    CHECK_ST(cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s), what));
    return cuda_status(cudaStreamSynchronize(s), what);
}

// KGMT::planBench (KGMT.cu:107-165): the same plan one iteration at a time,
// with the state writeDeviceVectorsToCSV (KGMT.cu:405-488) dumps handed to
// the hook after each iteration.  Only the rows appended by the iteration are
// copied back; the next frontier's flags and repeat counts are rebuilt on the
// host from the two frontier lists.
extern "C" kgmt_status kgmt_plan_traced(kgmt_planner* p, const float* h_initial, const float* h_goal, const float* d_obstacles,
                                        uint32_t n_obstacles, kgmt_iteration_hook hook, void* user)
{
    CHECK_ST(plan_setup(p, h_initial, h_goal, d_obstacles, n_obstacles, "kgmt_plan_traced"));
    const QueryParams& prm = p->params;
    const uint32_t T = prm.capacity, D = prm.sample_dim, R1 = prm.regions;
    const cudaStream_t s = p->eng.stream();
    std::vector<float> samples((size_t)T * D, 0.0f), score(R1), path(((size_t)prm.max_iterations + 2) * D, 0.0f);
    std::vector<int32_t> parents(T, -1), counter(R1), valid(R1);
    std::vector<uint8_t> frontier(T, 0);
    std::vector<uint32_t> repeat(T, 0), list(T);
    QueryState before, after;
    uint32_t err = 0;
    CHECK_ST(p->eng.read_states_and_error(0, 1, &before, &err));
    CHECK_ST(copy_back(s, samples.data(), prm.tree, (size_t)D * 4, "copy root"));
    parents[0] = -1;
    uint32_t new_nodes = 1;  // nodes the previous iteration appended (the root before the first)
    for(uint32_t k = 0; k < prm.max_iterations + 2 && before.status == KGMT_QUERY_RUNNING; ++k)
        {
            CHECK_ST(p->eng.run_iterations(1));
            CHECK_ST(p->eng.read_states_and_error(0, 1, &after, &err));
            RETURN_IF(err != 0, KGMT_ERR_TIMEOUT, "kgmt_plan_traced: a device-side wait gave up (error bits " + std::to_string(err) + ")");
            if(after.status != KGMT_QUERY_RUNNING)
                {
                    CHECK_ST(p->eng.extract_paths(1));
                    CHECK_ST(p->eng.read_states_and_error(0, 1, &after, &err));
                }
            // rows appended by this iteration (earlier rows never change)
            const uint32_t t0 = before.tree_size, t1 = after.tree_size < T ? after.tree_size : T;
            if(t1 > t0)
                {
                    CHECK_ST(copy_back(s, samples.data() + (size_t)t0 * D, prm.tree + (size_t)t0 * D, (size_t)(t1 - t0) * D * 4, "copy rows"));
                    CHECK_ST(copy_back(s, parents.data() + t0, prm.parent + t0, (size_t)(t1 - t0) * 4, "copy parents"));
                }
            CHECK_ST(copy_back(s, counter.data(), prm.counter, (size_t)R1 * 4, "copy counters"));
            CHECK_ST(copy_back(s, valid.data(), prm.valid, (size_t)R1 * 4, "copy valid counts"));
            CHECK_ST(copy_back(s, score.data(), prm.score, (size_t)R1 * 4, "copy scores"));
            // the next frontier: re-activated nodes once each, then new nodes
            // with their repeat counts
            std::fill(frontier.begin(), frontier.end(), 0);
            std::fill(repeat.begin(), repeat.end(), 0u);
            uint32_t distinct = 0;
            const uint32_t n_old = after.n_react < T ? after.n_react : T, n_new = after.w_new < T ? after.w_new : T;
            CHECK_ST(copy_back(s, list.data(), prm.rep_old, (size_t)n_old * 4, "copy frontier"));
            for(uint32_t i = 0; i < n_old; ++i)
                if(list[i] < T) frontier[list[i]] = 1, repeat[list[i]] += 1, ++distinct;
            CHECK_ST(copy_back(s, list.data(), prm.rep_new, (size_t)n_new * 4, "copy frontier"));
            for(uint32_t i = 0; i < n_new; ++i)
                if(list[i] < T)
                    {
                        if(!frontier[list[i]]) ++distinct;
                        frontier[list[i]] = 1, repeat[list[i]] += 1;
                    }
            const uint32_t rows = after.path_len < prm.max_iterations + 2 ? after.path_len : prm.max_iterations + 2;
            if(after.status == KGMT_QUERY_SUCCESS && rows)
                CHECK_ST(copy_back(s, path.data(), prm.path, (size_t)rows * D * 4, "copy path"));
            if(hook)
                {
                    kgmt_iteration it;
                    std::memset(&it, 0, sizeof(it));
                    it.itr = before.itr;
                    it.tree_size = after.tree_size;
                    it.frontier_size = before.n_react + new_nodes;
                    it.expanded = before.n_samples;
                    it.next_frontier_size = distinct;
                    it.goal_index = after.status == KGMT_QUERY_SUCCESS ? after.goal_index : -1;
                    it.path_len = after.status == KGMT_QUERY_SUCCESS ? rows : 0;
                    it.capacity = T, it.sample_dim = D, it.regions = R1;
                    it.samples = samples.data(), it.parents = parents.data();
                    it.counter = counter.data(), it.valid = valid.data(), it.score = score.data();
                    it.frontier = frontier.data(), it.repeat = repeat.data(), it.path = path.data();
                    hook(&it, user);
                }
            new_nodes = after.tree_size - before.tree_size;
            before = after;
        }
    RETURN_IF(before.status == KGMT_QUERY_RUNNING, KGMT_ERR_INTERNAL, "kgmt_plan_traced: the query did not stop within its iteration budget");
    RETURN_IF(bounds_error_take() != 0, KGMT_ERR_INTERNAL, "kgmt_plan_traced: an index check failed (bounds-checked build)");
    p->state = before;
    p->planned = true;
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_get_result(const kgmt_planner* p, kgmt_result* out)
{
    RETURN_IF(!p || !out, KGMT_ERR_INVALID_ARG, "kgmt_get_result: NULL argument");
    RETURN_IF(!p->planned, KGMT_ERR_NOT_READY, "kgmt_get_result: no plan has completed");
    *out = to_result(p->state, 0);
    return KGMT_OK;
}

static kgmt_status copy_tree_common(const QueryParams& prm, const QueryState& st, cudaStream_t s, float* h_samples, int32_t* h_parents,
                                    float* h_costs, uint32_t max_nodes)
{
    const uint32_t n = st.tree_size < max_nodes ? st.tree_size : max_nodes;
    const size_t D = prm.sample_dim;
    if(h_samples) CHECK_ST(cuda_status(cudaMemcpyAsync(h_samples, prm.tree, n * D * 4, cudaMemcpyDeviceToHost, s), "copy tree"));
    if(h_parents) CHECK_ST(cuda_status(cudaMemcpyAsync(h_parents, prm.parent, n * 4ull, cudaMemcpyDeviceToHost, s), "copy parents"));
    if(h_costs) CHECK_ST(cuda_status(cudaMemcpyAsync(h_costs, prm.cost, n * 4ull, cudaMemcpyDeviceToHost, s), "copy costs"));
    return cuda_status(cudaStreamSynchronize(s), "sync");
}

static kgmt_status copy_path_common(const QueryParams& prm, const QueryState& st, cudaStream_t s, float* h_rows, uint32_t max_rows,
                                    uint32_t* n_rows)
{
    const uint32_t n = st.path_len < max_rows ? st.path_len : max_rows;
    if(n_rows) *n_rows = n;
    if(n && h_rows)
        {
            CHECK_ST(cuda_status(cudaMemcpyAsync(h_rows, prm.path, (size_t)n * prm.sample_dim * 4, cudaMemcpyDeviceToHost, s), "copy path"));
            return cuda_status(cudaStreamSynchronize(s), "sync");
        }
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_copy_tree(kgmt_planner* p, float* h_samples, int32_t* h_parents, float* h_costs, uint32_t max_nodes)
{
    RETURN_IF(!p, KGMT_ERR_INVALID_ARG, "kgmt_copy_tree: NULL planner");
    RETURN_IF(!p->planned, KGMT_ERR_NOT_READY, "kgmt_copy_tree: no plan has completed");
    return copy_tree_common(p->params, p->state, p->eng.stream(), h_samples, h_parents, h_costs, max_nodes);
}

extern "C" kgmt_status kgmt_copy_path(kgmt_planner* p, float* h_rows, uint32_t max_rows, uint32_t* n_rows)
{
    RETURN_IF(!p, KGMT_ERR_INVALID_ARG, "kgmt_copy_path: NULL planner");
    RETURN_IF(!p->planned, KGMT_ERR_NOT_READY, "kgmt_copy_path: no plan has completed");
    return copy_path_common(p->params, p->state, p->eng.stream(), h_rows, max_rows, n_rows);
}

extern "C" kgmt_status kgmt_device_tree(kgmt_planner* p, const float** d_samples, const int32_t** d_parents, const float** d_costs)
{
    RETURN_IF(!p, KGMT_ERR_INVALID_ARG, "kgmt_device_tree: NULL planner");
    RETURN_IF(!p->planned, KGMT_ERR_NOT_READY, "kgmt_device_tree: no plan has completed");
    if(d_samples) *d_samples = p->params.tree;
    if(d_parents) *d_parents = p->params.parent;
    if(d_costs) *d_costs = p->params.cost;
    return KGMT_OK;
}

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
struct kgmt_batch {
    Engine eng;
    DeviceArena arena;
    kgmt_batch_options opt;
    std::vector<QueryState> states;
    std::vector<QueryParams> params;
    uint32_t n_last = 0;
    kgmt_batch_stats stats{};
};

extern "C" kgmt_status kgmt_batch_create(const kgmt_batch_options* opt, void* stream, kgmt_batch** out)
{
    RETURN_IF(!opt || !out, KGMT_ERR_INVALID_ARG, "kgmt_batch_create: NULL argument");
    RETURN_IF(opt->max_queries == 0 || opt->max_queries > (1u << 20), KGMT_ERR_INVALID_ARG, "kgmt_batch_create: max_queries");
    *out = nullptr;
    kgmt_batch* b = new(std::nothrow) kgmt_batch();
    RETURN_IF(!b, KGMT_ERR_OOM, "kgmt_batch_create: host allocation failed");
    b->opt = *opt;
    kgmt_status st = b->eng.init(opt->max_queries, (cudaStream_t)stream, opt->propagate_block ? opt->propagate_block : 256,
                                 opt->iters_per_graph ? opt->iters_per_graph : 4, opt->use_graph != 0);
    if(st != KGMT_OK)
        {
            delete b;
            return st;
        }
    b->eng.set_profile(opt->profile_kernels != 0);
    *out = b;
    return KGMT_OK;
}

extern "C" void kgmt_batch_destroy(kgmt_batch* b) { delete b; }

// lays out n queries + one shared obstacle region + raw staging in the arena
static kgmt_status batch_prepare(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits, const float* h_goals,
                                 const uint32_t* obs_offset, const uint32_t* obs_count, size_t* raw_off, float4** obs_region,
                                 uint32_t* n_boxes)
{
    RETURN_IF(n == 0 || n > b->eng.slots(), KGMT_ERR_CAPACITY, "batch: query count exceeds max_queries");
    RETURN_IF(!cfgs || !obs_offset || !obs_count, KGMT_ERR_INVALID_ARG, "batch: NULL argument");
    b->eng.reset_counters();
    uint64_t boxes = 0;
    uint32_t max_iters = 0, max_obs = 0;
    size_t total = 0;
    std::vector<QueryLayout> L(n);
    for(uint32_t i = 0; i < n; ++i)
        {
            CHECK_ST(validate_config(cfgs[i]));
            L[i] = layout_of(cfgs[i], obs_count[i], false);
            total += L[i].total;
            uint64_t end = (uint64_t)obs_offset[i] + obs_count[i];
            if(end > boxes) boxes = end;
            if(obs_count[i] > max_obs) max_obs = obs_count[i];
            if(cfgs[i].max_iterations > max_iters) max_iters = cfgs[i].max_iterations;
        }
    RETURN_IF(boxes > (1ull << 31), KGMT_ERR_INVALID_ARG, "batch: too many obstacles");
    const size_t obs_bytes = ((boxes * 32 + 255) / 256) * 256;
    const size_t raw_bytes = ((boxes * 24 + 255) / 256) * 256;
    b->arena.reset();
    CHECK_ST(b->arena.reserve(total + obs_bytes + raw_bytes + 4096));
    size_t obs_off = 0, rawo = 0;
    RETURN_IF(!b->arena.alloc(obs_bytes ? obs_bytes : 256, &obs_off), KGMT_ERR_OOM, "batch: arena");
    RETURN_IF(!b->arena.alloc(raw_bytes ? raw_bytes : 256, &rawo), KGMT_ERR_OOM, "batch: arena");
    float4* region = (float4*)(b->arena.base() + obs_off);
    int models = 0;
    for(uint32_t i = 0; i < n; ++i) models |= Engine::model_bit(cfgs[i].model);
    b->eng.set_models(models);
    b->eng.set_max_obstacles(max_obs);
    b->params.resize(n);
    for(uint32_t i = 0; i < n; ++i)
        {
            size_t off = 0;
            RETURN_IF(!b->arena.alloc(L[i].total, &off), KGMT_ERR_OOM, "batch: arena");
            const float* init = h_inits ? h_inits + (size_t)i * KGMT_MAX_SAMPLE_DIM : nullptr;
            const float* goal = h_goals ? h_goals + (size_t)i * KGMT_MAX_SAMPLE_DIM : nullptr;
            b->params[i] = make_params(cfgs[i], init, goal, b->arena.base() + off, L[i], region + 2 * (size_t)obs_offset[i], obs_count[i]);
            b->eng.host_params(i) = b->params[i];
        }
    *raw_off = rawo;
    *obs_region = region;
    *n_boxes = (uint32_t)boxes;
    return KGMT_OK;
}

static kgmt_status batch_run(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* d_inits, const float* d_goals,
                             kgmt_result* results)
{
    uint32_t max_iters = 0;
    for(uint32_t i = 0; i < n; ++i)
        if(cfgs[i].max_iterations > max_iters) max_iters = cfgs[i].max_iterations;
    const uint32_t it0 = b->eng.iterations_launched();
    CHECK_ST(b->eng.admit(0, n, n, d_inits, d_goals));
    CHECK_ST(b->eng.run_until_done(max_iters));
    CHECK_ST(b->eng.extract_paths(n));
    b->states.resize(n);
    uint32_t err = 0;
    CHECK_ST(b->eng.read_states_and_error(0, n, b->states.data(), &err));
    b->n_last = n;
    RETURN_IF(err != 0, KGMT_ERR_TIMEOUT, "batch: a device-side wait gave up (error bits " + std::to_string(err) + ")");
    RETURN_IF(bounds_error_take() != 0, KGMT_ERR_INTERNAL, "batch: an index check failed (bounds-checked build)");
    // counters of this call
    kgmt_batch_stats& s = b->stats;
    std::memset(&s, 0, sizeof(s));
    s.kernel_launches = b->eng.launches();
    s.iterations_launched = b->eng.iterations_launched() - it0;
    for(uint32_t i = 0; i < n; ++i)
        {
            const QueryState& q = b->states[i];
            const uint64_t per_step = ops_per_step(cfgs[i].model);
            s.steps_executed += q.steps;
            s.obstacle_tests += q.tests;
            s.samples += q.samples_drawn;
            const uint64_t lookup = b->params[i].n_obstacles ? kOpsPerGridLookup : 0;
            s.fp32_ops += q.steps * (per_step + lookup) + q.tests * kOpsPerObstacleTest;
        }
    float ms[3];
    uint32_t cnt[3];
    CHECK_ST(b->eng.kernel_times(ms, cnt));
    s.ms_propagate = ms[0], s.ms_tail = ms[1], s.ms_append = ms[2];
    s.launches_propagate = cnt[0], s.launches_tail = cnt[1], s.launches_append = cnt[2];
    uint32_t tail_iters = 0;
    uint64_t tail_ops = 0, tail_samples = 0;
    CHECK_ST(b->eng.tail_counters(&tail_iters, &tail_ops, &tail_samples));
    s.iterations_tail = tail_iters;
    s.fp32_ops_tail = tail_ops;
    s.samples_tail = tail_samples;
    if(results)
        for(uint32_t i = 0; i < n; ++i) results[i] = to_result(b->states[i], i);
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_batch_get_stats(kgmt_batch* b, kgmt_batch_stats* out)
{
    RETURN_IF(!b || !out, KGMT_ERR_INVALID_ARG, "kgmt_batch_get_stats: NULL argument");
    *out = b->stats;
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_plan_batch(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits, const float* h_goals,
                                       const float* h_obstacles, const uint32_t* obs_offset, const uint32_t* obs_count,
                                       kgmt_result* results)
{
    RETURN_IF(!b || !h_inits || !h_goals, KGMT_ERR_INVALID_ARG, "kgmt_plan_batch: NULL argument");
    b->n_last = 0;
    size_t raw_off = 0;
    float4* region = nullptr;
    uint32_t boxes = 0;
    CHECK_ST(batch_prepare(b, n, cfgs, h_inits, h_goals, obs_offset, obs_count, &raw_off, &region, &boxes));
    RETURN_IF(boxes > 0 && !h_obstacles, KGMT_ERR_INVALID_ARG, "kgmt_plan_batch: obstacles pointer is NULL");
    cudaStream_t s = b->eng.stream();
    float* raw = (float*)(b->arena.base() + raw_off);
    if(boxes)
        {
            CHECK_ST(cuda_status(cudaMemcpyAsync(raw, h_obstacles, (size_t)boxes * 24, cudaMemcpyHostToDevice, s), "upload obstacles"));
            CHECK_ST(cuda_status(launch_stage_obstacles(raw, region, boxes, 3, s), "stage obstacles"));
            b->eng.add_launches(1);
        }
    return batch_run(b, n, cfgs, nullptr, nullptr, results);
}

extern "C" kgmt_status kgmt_plan_batch_device(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* d_inits,
                                              const float* d_goals, const float* d_obstacles, const uint32_t* h_obs_offset,
                                              const uint32_t* h_obs_count, kgmt_result* results)
{
    RETURN_IF(!b || !d_inits || !d_goals, KGMT_ERR_INVALID_ARG, "kgmt_plan_batch_device: NULL argument");
    b->n_last = 0;
    size_t raw_off = 0;
    float4* region = nullptr;
    uint32_t boxes = 0;
    CHECK_ST(batch_prepare(b, n, cfgs, nullptr, nullptr, h_obs_offset, h_obs_count, &raw_off, &region, &boxes));
    RETURN_IF(boxes > 0 && !d_obstacles, KGMT_ERR_INVALID_ARG, "kgmt_plan_batch_device: obstacles pointer is NULL");
    if(boxes)
        {
            CHECK_ST(cuda_status(launch_stage_obstacles(d_obstacles, region, boxes, 3, b->eng.stream()), "stage obstacles"));
            b->eng.add_launches(1);
        }
    return batch_run(b, n, cfgs, d_inits, d_goals, results);
}

extern "C" kgmt_status kgmt_batch_copy_tree(kgmt_batch* b, uint32_t i, float* h_samples, int32_t* h_parents, float* h_costs,
                                            uint32_t max_nodes)
{
    RETURN_IF(!b, KGMT_ERR_INVALID_ARG, "kgmt_batch_copy_tree: NULL batch");
    RETURN_IF(i >= b->n_last, KGMT_ERR_NOT_READY, "kgmt_batch_copy_tree: no such query in the last batch");
    return copy_tree_common(b->params[i], b->states[i], b->eng.stream(), h_samples, h_parents, h_costs, max_nodes);
}

extern "C" kgmt_status kgmt_batch_copy_path(kgmt_batch* b, uint32_t i, float* h_rows, uint32_t max_rows, uint32_t* n_rows)
{
    RETURN_IF(!b, KGMT_ERR_INVALID_ARG, "kgmt_batch_copy_path: NULL batch");
    RETURN_IF(i >= b->n_last, KGMT_ERR_NOT_READY, "kgmt_batch_copy_path: no such query in the last batch");
    return copy_path_common(b->params[i], b->states[i], b->eng.stream(), h_rows, max_rows, n_rows);
}

extern "C" kgmt_status kgmt_batch_autotune(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits, const float* h_goals,
                                           const float* h_obstacles, const uint32_t* obs_offset, const uint32_t* obs_count,
                                           uint32_t* best_block)
{
    RETURN_IF(!b, KGMT_ERR_INVALID_ARG, "kgmt_batch_autotune: NULL batch");
    const uint32_t blocks[3] = {128, 256, 512};
    double best_t = 1e30;
    uint32_t best = b->eng.prop_block();
    for(uint32_t blk : blocks)
        {
            CHECK_ST(b->eng.set_prop_block(blk));
            // one warm-up, then the timed run
            CHECK_ST(kgmt_plan_batch(b, n, cfgs, h_inits, h_goals, h_obstacles, obs_offset, obs_count, nullptr));
            auto t0 = std::chrono::steady_clock::now();
            CHECK_ST(kgmt_plan_batch(b, n, cfgs, h_inits, h_goals, h_obstacles, obs_offset, obs_count, nullptr));
            double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if(t < best_t)
                {
                    best_t = t;
                    best = blk;
                }
        }
    CHECK_ST(b->eng.set_prop_block(best));
    if(best_block) *best_block = best;
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_batch_autotune_full(kgmt_batch* b, uint32_t n, const kgmt_config* cfgs, const float* h_inits,
                                                const float* h_goals, const float* h_obstacles, const uint32_t* obs_offset,
                                                const uint32_t* obs_count, kgmt_autotune_result* out)
{
    RETURN_IF(!b || !cfgs || !out, KGMT_ERR_INVALID_ARG, "kgmt_batch_autotune_full: NULL argument");
    RETURN_IF(n == 0, KGMT_ERR_INVALID_ARG, "kgmt_batch_autotune_full: empty batch");
    std::vector<kgmt_config> c(cfgs, cfgs + n);
    std::vector<kgmt_result> res(n);
    // one warm-up and one timed plan of the batch at (block, samples per node; 0 = as given)
    auto trial = [&](uint32_t blk, uint32_t spn, double* qps, double* succ) -> kgmt_status {
        CHECK_ST(b->eng.set_prop_block(blk));
        for(uint32_t i = 0; i < n; ++i) c[i].samples_per_node = spn ? spn : cfgs[i].samples_per_node;
        CHECK_ST(kgmt_plan_batch(b, n, c.data(), h_inits, h_goals, h_obstacles, obs_offset, obs_count, res.data()));
        const auto t0 = std::chrono::steady_clock::now();
        CHECK_ST(kgmt_plan_batch(b, n, c.data(), h_inits, h_goals, h_obstacles, obs_offset, obs_count, res.data()));
        const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        uint32_t ok = 0;
        for(uint32_t i = 0; i < n; ++i) ok += res[i].status == KGMT_QUERY_SUCCESS ? 1u : 0u;
        *qps = t > 0.0 ? n / t : 0.0;
        *succ = (double)ok / n;
        return KGMT_OK;
    };
    double base_qps = 0.0, base_succ = 0.0;
    CHECK_ST(trial(256, 0, &base_qps, &base_succ));
    uint32_t best_blk = 256, best_spn = cfgs[0].samples_per_node;
    double best_qps = -1.0, best_succ = base_succ;
    const uint32_t blocks[3] = {128, 256, 512};
    const uint32_t spns[4] = {2, 4, 8, 16};
    for(uint32_t spn : spns)
        for(uint32_t blk : blocks)
            {
                double qps = 0.0, succ = 0.0;
                CHECK_ST(trial(blk, spn, &qps, &succ));
                if(succ >= 0.95 * base_succ && qps > best_qps)
                    {
                        best_qps = qps, best_succ = succ;
                        best_blk = blk, best_spn = spn;
                    }
            }
    if(best_qps < 0.0)
        {
            // nothing kept the success rate: the configs as given
            best_qps = base_qps;
        }
    CHECK_ST(b->eng.set_prop_block(best_blk));
    out->propagate_block = best_blk;
    out->samples_per_node = best_spn;
    out->queries_per_s = (float)best_qps;
    out->success_rate = (float)best_succ;
    out->base_queries_per_s = (float)base_qps;
    out->base_success_rate = (float)base_succ;
    return KGMT_OK;
}

// ---------------------------------------------------------------------------
// server: continuous batching with memory-based admission
//
// A step is asynchronous: it finishes the previous step (waits for its
// iterations and for the copy of the states queued behind them, then retires
// the queries they finished), admits queued queries into free slots, queues
// this step's iterations (a CUDA-graph replay) and the copy of the states
// behind them, and returns while the GPU runs.  Admission copies from pinned
// staging and admits every new query with one kernel launch.  Queries that
// fit may pass a head that does not (memory), within a window, until the head
// has waited kMaxBypass steps; then nothing passes it.
// ---------------------------------------------------------------------------
constexpr uint32_t kAdmitWindow = 64;  // queued queries one step looks at
constexpr uint32_t kMaxBypass = 16;    // steps the head may be passed before it blocks the queue

struct PendingQuery {
    uint64_t ticket;
    kgmt_config cfg;
    float init[KGMT_MAX_SAMPLE_DIM];
    float goal[KGMT_MAX_SAMPLE_DIM];
    std::vector<float> obstacles;
    std::chrono::steady_clock::time_point submitted;
    uint32_t passed = 0;  // steps in which a later query was admitted before it
};

struct ResidentQuery {
    bool used = false;
    int model_bit = 0;
    uint64_t ticket = 0;
    size_t offset = 0;
    std::chrono::steady_clock::time_point submitted;
};

// pinned host memory that grows geometrically, keeping its contents
struct PinnedBuffer {
    char* p = nullptr;
    size_t cap = 0;
    ~PinnedBuffer()
    {
        if(p) cudaFreeHost(p);
    }
    // no copy from the old buffer may be in flight when it grows
    kgmt_status reserve(size_t bytes, size_t keep)
    {
        if(bytes <= cap) return KGMT_OK;
        size_t n = cap ? cap : 65536;
        while(n < bytes) n *= 2;
        char* q = nullptr;
        CHECK_ST(cuda_status(cudaMallocHost((void**)&q, n), "cudaMallocHost(staging)"));
        if(p)
            {
                if(keep) std::memcpy(q, p, keep);
                cudaFreeHost(p);
            }
        p = q;
        cap = n;
        return KGMT_OK;
    }
};

struct kgmt_server {
    Engine eng;
    DeviceArena arena;
    kgmt_server_options opt;
    std::deque<PendingQuery> queue;
    std::vector<ResidentQuery> slots;
    std::deque<kgmt_result> done;
    uint64_t next_ticket = 1;
    uint32_t resident = 0;     // admitted and not yet retired
    uint32_t box_capacity = 0; // boxes a propagate block stages: the largest admitted so far
    bool resched = false;      // a resident query was cancelled: the next step recomputes the schedule
    // the step in flight: its iterations and the copy of states [0, copied)
    bool inflight = false;
    uint32_t copied = 0;
    cudaEvent_t ev = nullptr;
    QueryState* h_states = nullptr;  // pinned [max_slots]
    uint32_t* h_error = nullptr;     // pinned
    PinnedBuffer stage;              // params, raw boxes and the slot list of one admission
    ~kgmt_server()
    {
        if(eng.stream()) cudaStreamSynchronize(eng.stream());
        if(ev) cudaEventDestroy(ev);
        if(h_states) cudaFreeHost(h_states);
        if(h_error) cudaFreeHost(h_error);
    }
};

extern "C" kgmt_status kgmt_server_create(const kgmt_server_options* opt, void* stream, kgmt_server** out)
{
    RETURN_IF(!opt || !out, KGMT_ERR_INVALID_ARG, "kgmt_server_create: NULL argument");
    RETURN_IF(opt->max_slots == 0 || opt->max_slots > (1u << 16), KGMT_ERR_INVALID_ARG, "kgmt_server_create: max_slots");
    RETURN_IF(opt->memory_budget < (1ull << 20), KGMT_ERR_INVALID_ARG, "kgmt_server_create: memory_budget below 1 MiB");
    *out = nullptr;
    kgmt_server* s = new(std::nothrow) kgmt_server();
    RETURN_IF(!s, KGMT_ERR_OOM, "kgmt_server_create: host allocation failed");
    s->opt = *opt;
    if(s->opt.iters_per_step == 0) s->opt.iters_per_step = 1;
    // one graph replay per step: a unit of iters_per_step iterations
    kgmt_status st = s->eng.init(opt->max_slots, (cudaStream_t)stream, opt->propagate_block ? opt->propagate_block : 256, s->opt.iters_per_step, true);
    if(st == KGMT_OK) st = s->arena.reserve(opt->memory_budget);
    if(st == KGMT_OK) st = s->eng.set_active(opt->max_slots);
    if(st == KGMT_OK) st = cuda_status(cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming), "cudaEventCreate");
    if(st == KGMT_OK) st = cuda_status(cudaMallocHost((void**)&s->h_states, sizeof(QueryState) * opt->max_slots), "cudaMallocHost(states)");
    if(st == KGMT_OK) st = cuda_status(cudaMallocHost((void**)&s->h_error, sizeof(uint32_t)), "cudaMallocHost(error)");
    if(st != KGMT_OK)
        {
            delete s;
            return st;
        }
    s->slots.resize(opt->max_slots);
    *out = s;
    return KGMT_OK;
}

extern "C" void kgmt_server_destroy(kgmt_server* s) { delete s; }

extern "C" kgmt_status kgmt_server_submit(kgmt_server* s, const kgmt_config* cfg, const float* h_init, const float* h_goal,
                                          const float* h_obstacles, uint32_t n_obstacles, uint64_t* ticket)
{
    RETURN_IF(!s || !cfg || !h_init || !h_goal, KGMT_ERR_INVALID_ARG, "kgmt_server_submit: NULL argument");
    RETURN_IF(n_obstacles > 0 && !h_obstacles, KGMT_ERR_INVALID_ARG, "kgmt_server_submit: obstacles pointer is NULL");
    CHECK_ST(validate_config(*cfg));
    const QueryLayout L = layout_of(*cfg, n_obstacles, true);
    RETURN_IF(L.total + (size_t)n_obstacles * 24 + 256 > s->arena.capacity(), KGMT_ERR_OOM,
              "kgmt_server_submit: query larger than the memory budget");
    PendingQuery q;
    q.ticket = s->next_ticket++;
    q.cfg = *cfg;
    const uint32_t D = sample_dim_of(cfg->model);
    std::memset(q.init, 0, sizeof(q.init));
    std::memset(q.goal, 0, sizeof(q.goal));
    std::memcpy(q.init, h_init, D * sizeof(float));
    std::memcpy(q.goal, h_goal, 3 * sizeof(float));
    q.obstacles.assign(h_obstacles, h_obstacles + (size_t)n_obstacles * 6);
    q.submitted = std::chrono::steady_clock::now();
    s->queue.push_back(std::move(q));
    if(ticket) *ticket = s->queue.back().ticket;
    return KGMT_OK;
}

// waits for the step in flight and retires the queries it finished
static kgmt_status server_finish_step(kgmt_server* s)
{
    if(!s->inflight) return KGMT_OK;
    s->inflight = false;
    CHECK_ST(cuda_status(cudaEventSynchronize(s->ev), "cudaEventSynchronize"));
    const auto now = std::chrono::steady_clock::now();
    for(uint32_t i = 0; i < s->copied; ++i)
        {
            ResidentQuery& r = s->slots[i];
            if(!r.used) continue;
            const QueryState& qs = s->h_states[i];
            if(qs.status == KGMT_QUERY_RUNNING) continue;
            kgmt_result res = to_result(qs, r.ticket);
            res.latency_ms = (float)(std::chrono::duration<double, std::milli>(now - r.submitted).count());
            s->done.push_back(res);
            s->arena.release(r.offset);
            r.used = false;
            --s->resident;
        }
    const uint32_t err = *s->h_error;
    RETURN_IF(err != 0, KGMT_ERR_TIMEOUT, "server: a device-side wait gave up (error bits " + std::to_string(err) + ")");
    RETURN_IF(bounds_error_take() != 0, KGMT_ERR_INTERNAL, "server: an index check failed (bounds-checked build)");
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_server_step(kgmt_server* s, uint32_t* n_running, uint32_t* n_queued)
{
    RETURN_IF(!s, KGMT_ERR_INVALID_ARG, "kgmt_server_step: NULL server");
    CHECK_ST(server_finish_step(s));
    cudaStream_t st = s->eng.stream();
    // ---- admission: queued queries in order into free slots while memory
    // allows; a query that does not fit may be passed by later ones.  Each
    // admitted query's params and raw boxes go to pinned staging (the previous
    // step's copies from it are complete) ----
    struct Admit {
        uint32_t slot;
        size_t params_at, raw_at, raw_bytes;
        float* d_raw;
    };
    std::vector<Admit> adm;
    std::vector<size_t> taken;  // queue positions admitted
    size_t used = 0;
    uint32_t slot = 0;
    for(size_t pos = 0; pos < s->queue.size() && pos < kAdmitWindow; ++pos)
        {
            while(slot < s->slots.size() && s->slots[slot].used) ++slot;
            if(slot >= s->slots.size()) break;
            PendingQuery& q = s->queue[pos];
            const uint32_t n_obs = (uint32_t)(q.obstacles.size() / 6);
            const QueryLayout L = layout_of(q.cfg, n_obs, true);
            const size_t raw_at = (L.total + 255) & ~size_t(255);
            size_t off = 0;
            if(!s->arena.alloc(raw_at + (size_t)n_obs * 24 + 256, &off))
                {
                    // it waits for memory; later queries may pass it unless it
                    // is the head and has been passed kMaxBypass times
                    if(pos == 0 && q.passed >= kMaxBypass) break;
                    continue;
                }
            char* chunk = s->arena.base() + off;
            QueryParams prm = make_params(q.cfg, q.init, q.goal, chunk, L, nullptr, n_obs);
            prm.raw_obstacles = n_obs ? (const float*)(chunk + raw_at) : nullptr;
            prm.raw_w = 3;
            Admit a;
            a.slot = slot;
            a.params_at = (used + 15) & ~size_t(15);
            a.raw_at = (a.params_at + sizeof(QueryParams) + 15) & ~size_t(15);
            a.raw_bytes = (size_t)n_obs * 24;
            a.d_raw = (float*)(chunk + raw_at);
            CHECK_ST(s->stage.reserve(a.raw_at + a.raw_bytes, used));
            std::memcpy(s->stage.p + a.params_at, &prm, sizeof(QueryParams));
            if(a.raw_bytes) std::memcpy(s->stage.p + a.raw_at, q.obstacles.data(), a.raw_bytes);
            used = a.raw_at + a.raw_bytes;
            adm.push_back(a);
            taken.push_back(pos);
            for(size_t j = 0; j < pos; ++j) s->queue[j].passed += 1;
            ResidentQuery& r = s->slots[slot];
            r.used = true;
            r.model_bit = Engine::model_bit(q.cfg.model);
            r.ticket = q.ticket;
            r.offset = off;
            r.submitted = q.submitted;
            if(n_obs > s->box_capacity) s->box_capacity = n_obs;
            ++s->resident;
            ++slot;
        }
    if(!adm.empty())
        {
            const size_t list_at = (used + 15) & ~size_t(15);
            CHECK_ST(s->stage.reserve(list_at + sizeof(uint32_t) * adm.size(), used));
            uint32_t* list = (uint32_t*)(s->stage.p + list_at);
            for(size_t i = 0; i < adm.size(); ++i)
                {
                    const Admit& a = adm[i];
                    list[i] = a.slot;
                    CHECK_ST(s->eng.upload_params_async(a.slot, (const QueryParams*)(s->stage.p + a.params_at)));
                    if(a.raw_bytes)
                        CHECK_ST(cuda_status(cudaMemcpyAsync(a.d_raw, s->stage.p + a.raw_at, a.raw_bytes, cudaMemcpyHostToDevice, st),
                                             "upload obstacles"));
                }
            CHECK_ST(s->eng.admit_slot_list(list, (uint32_t)adm.size()));
            for(size_t i = taken.size(); i-- > 0;) s->queue.erase(s->queue.begin() + (std::ptrdiff_t)taken[i]);
        }
    if(!adm.empty() || s->resched)
        {
            int models = 0;
            for(size_t i = 0; i < s->slots.size(); ++i)
                if(s->slots[i].used) models |= s->slots[i].model_bit;
            s->eng.set_models(models);
            s->eng.set_max_obstacles(s->box_capacity);
            CHECK_ST(s->eng.schedule());
            s->resched = false;
        }
    // ---- this step's iterations, and the states behind them ----
    if(s->resident)
        {
            uint32_t hwm = 0;
            for(uint32_t i = 0; i < (uint32_t)s->slots.size(); ++i)
                if(s->slots[i].used) hwm = i + 1;
            CHECK_ST(s->eng.launch_units(1));
            CHECK_ST(s->eng.enqueue_state_copy(hwm, s->h_states, s->h_error));
            CHECK_ST(cuda_status(cudaEventRecord(s->ev, st), "cudaEventRecord"));
            s->copied = hwm;
            s->inflight = true;
        }
    if(n_running) *n_running = s->resident;
    if(n_queued) *n_queued = (uint32_t)s->queue.size();
    return KGMT_OK;
}

extern "C" kgmt_status kgmt_server_cancel(kgmt_server* s, uint64_t ticket)
{
    RETURN_IF(!s, KGMT_ERR_INVALID_ARG, "kgmt_server_cancel: NULL server");
    // no kernel of a step may run while a status is rewritten: finish the
    // step in flight (its finished queries retire as in a step)
    CHECK_ST(server_finish_step(s));
    const auto now = std::chrono::steady_clock::now();
    for(auto it = s->queue.begin(); it != s->queue.end(); ++it)
        if(it->ticket == ticket)
            {
                kgmt_result res;
                std::memset(&res, 0, sizeof(res));
                res.status = KGMT_QUERY_CANCELLED;
                res.goal_index = -1;
                res.ticket = ticket;
                res.latency_ms = (float)(std::chrono::duration<double, std::milli>(now - it->submitted).count());
                s->done.push_back(res);
                s->queue.erase(it);
                return KGMT_OK;
            }
    for(uint32_t i = 0; i < (uint32_t)s->slots.size(); ++i)
        {
            ResidentQuery& r = s->slots[i];
            if(!r.used || r.ticket != ticket) continue;
            // the status is final before the next step's schedule, which then
            // gives the slot no tiles
            CHECK_ST(s->eng.write_status(i, KGMT_QUERY_CANCELLED));
            QueryState qs;
            CHECK_ST(s->eng.read_states(i, 1, &qs));
            kgmt_result res = to_result(qs, ticket);
            res.latency_ms = (float)(std::chrono::duration<double, std::milli>(now - r.submitted).count());
            s->done.push_back(res);
            s->arena.release(r.offset);
            r.used = false;
            --s->resident;
            s->resched = true;
            return KGMT_OK;
        }
    set_error("kgmt_server_cancel: no queued or running query has this ticket");
    return KGMT_ERR_NOT_READY;
}

extern "C" kgmt_status kgmt_server_poll(kgmt_server* s, kgmt_result* out, uint32_t max, uint32_t* n_out)
{
    RETURN_IF(!s || (!out && max > 0), KGMT_ERR_INVALID_ARG, "kgmt_server_poll: NULL argument");
    uint32_t k = 0;
    while(k < max && !s->done.empty())
        {
            out[k++] = s->done.front();
            s->done.pop_front();
        }
    if(n_out) *n_out = k;
    return KGMT_OK;
}

// ---------------------------------------------------------------------------
// function-level propagation
// ---------------------------------------------------------------------------
extern "C" kgmt_status kgmt_propagate_samples(const kgmt_config* cfg, const float* d_x0, const float* d_uniforms, const float* d_obstacles,
                                              uint32_t n_obstacles, uint32_t n, float* d_x1, uint8_t* d_valid, int32_t* d_r1, int32_t* d_r2,
                                              void* stream)
{
    RETURN_IF(!cfg || (n > 0 && (!d_x0 || !d_uniforms || !d_x1 || !d_valid)), KGMT_ERR_INVALID_ARG, "kgmt_propagate_samples: NULL argument");
    RETURN_IF(n_obstacles > 0 && !d_obstacles, KGMT_ERR_INVALID_ARG, "kgmt_propagate_samples: obstacles pointer is NULL");
    RETURN_IF(n_obstacles > 6000, KGMT_ERR_INVALID_ARG, "kgmt_propagate_samples: at most 6000 obstacles");
    CHECK_ST(validate_config(*cfg));
    int dev_count = 0;
    if(cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
        {
            cudaGetLastError();
            set_error("no CUDA device");
            return KGMT_ERR_NO_DEVICE;
        }
    const QueryLayout L = layout_of(*cfg, 0, false);
    QueryParams p = make_params(*cfg, nullptr, nullptr, nullptr, L, nullptr, n_obstacles);
    return cuda_status(
      launch_propagate_samples(p, d_x0, d_uniforms, d_obstacles, n_obstacles, n, d_x1, d_valid, d_r1, d_r2, (cudaStream_t)stream),
      "k_propagate_samples");
}

extern "C" kgmt_status kgmt_selftest_bounded_wait(uint32_t polls, uint32_t* error_bits)
{
    RETURN_IF(!error_bits, KGMT_ERR_INVALID_ARG, "kgmt_selftest_bounded_wait: error_bits is NULL");
    RETURN_IF(polls == 0 || polls > kSpinLimit, KGMT_ERR_INVALID_ARG, "kgmt_selftest_bounded_wait: polls outside 1 .. 4194304");
    int dev_count = 0;
    if(cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
        {
            cudaGetLastError();
            set_error("no CUDA device");
            return KGMT_ERR_NO_DEVICE;
        }
    // two look-back words (tile 0 left empty) and the error word
    void* d = nullptr;
    CHECK_ST(cuda_status(cudaMalloc(&d, 3 * sizeof(unsigned long long)), "cudaMalloc"));
    unsigned long long* tiles = (unsigned long long*)d;
    uint32_t* err = (uint32_t*)(tiles + 2);
    uint32_t h_err = 0;
    cudaError_t e = cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    if(e == cudaSuccess) e = launch_selftest_wait(tiles, err, polls, nullptr);
    if(e == cudaSuccess) e = cudaMemcpy(&h_err, err, sizeof(h_err), cudaMemcpyDeviceToHost);
    cudaFree(d);
    CHECK_ST(cuda_status(e, "k_selftest_wait"));
    *error_bits = h_err;
    RETURN_IF(h_err & kErrLookbackTimeout, KGMT_ERR_TIMEOUT,
              "kgmt_selftest_bounded_wait: a device-side wait gave up (error bits " + std::to_string(h_err) + ")");
    set_error("kgmt_selftest_bounded_wait: the wait did not time out");
    return KGMT_ERR_INTERNAL;
}
