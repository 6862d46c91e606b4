// kgmt_engine.cu -- host runtime: device arena, per-query layout, parameter
// derivation and the iteration loop (direct launches or CUDA-graph replay).
//
// Reference counterparts: buffer construction of Planner::Planner / KGMT::KGMT
// (src/planners/Planner.cu:4-35, src/planners/KGMT.cu:4-39, Graph::Graph
// src/graphs/Graph.cu:5-42) and the host loop of KGMT::plan
// (src/planners/KGMT.cu:84-95), which read sizes back from the device about
// six times per iteration; here the schedule stays on the device.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include <nvtx3/nvToolsExt.h>

#include "kgmt_engine.h"

namespace kgmt {

// Names the host stages of the launch chain (admission, iteration units,
// path readout) on a profiler's timeline; without a tool attached a range
// costs a branch.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

kgmt_status cuda_status(cudaError_t e, const char* what)
{
    if(e == cudaSuccess) return KGMT_OK;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    if(e == cudaErrorMemoryAllocation) return KGMT_ERR_OOM;
    if(e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return KGMT_ERR_NO_DEVICE;
    return KGMT_ERR_CUDA;
}

// Every device allocation of the library goes through here.  With
// KGMT_FAULT_ALLOC_AFTER=n in the environment (read once), each allocation
// after the first n fails as out of memory without reaching the driver: a
// host-side fault injector for the tests of the error paths.
static cudaError_t device_alloc(void** p, size_t bytes)
{
    static const long limit = [] {
        const char* e = std::getenv("KGMT_FAULT_ALLOC_AFTER");
        return e ? std::atol(e) : -1L;
    }();
    static std::atomic<long> count{0};
    if(limit >= 0 && count.fetch_add(1) >= limit) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

bool is_device_pointer(const void* p)
{
    cudaPointerAttributes a;
    if(cudaPointerGetAttributes(&a, p) != cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

#define KGMT_CUDA(call, what)                                 \
    do {                                                      \
        kgmt_status st_ = cuda_status((call), what);          \
        if(st_ != KGMT_OK) return st_;                        \
    } while(0)

// ---------------------------------------------------------------------------
// arena
// ---------------------------------------------------------------------------
DeviceArena::~DeviceArena()
{
    if(base_) cudaFree(base_);
}

kgmt_status DeviceArena::reserve(size_t bytes)
{
    if(bytes <= cap_) return KGMT_OK;
    if(!used_.empty())
        {
            set_error("arena: cannot grow while allocations are live");
            return KGMT_ERR_INTERNAL;
        }
    if(base_) cudaFree(base_);
    base_ = nullptr;
    cap_ = 0;
    free_.clear();
    bytes = (bytes + 4095) & ~size_t(4095);
    KGMT_CUDA(device_alloc((void**)&base_, bytes), "cudaMalloc(arena)");
    cap_ = bytes;
    free_[0] = bytes;
    used_bytes_ = 0;
    return KGMT_OK;
}

bool DeviceArena::alloc(size_t bytes, size_t* offset)
{
    bytes = (bytes + 255) & ~size_t(255);
    for(auto it = free_.begin(); it != free_.end(); ++it)
        {
            if(it->second >= bytes)
                {
                    size_t off = it->first, sz = it->second;
                    free_.erase(it);
                    if(sz > bytes) free_[off + bytes] = sz - bytes;
                    used_[off] = bytes;
                    used_bytes_ += bytes;
                    *offset = off;
                    return true;
                }
        }
    return false;
}

void DeviceArena::release(size_t offset)
{
    auto it = used_.find(offset);
    if(it == used_.end()) return;
    size_t sz = it->second;
    used_.erase(it);
    used_bytes_ -= sz;
    auto nx = free_.lower_bound(offset);
    if(nx != free_.end() && offset + sz == nx->first)
        {
            sz += nx->second;
            nx = free_.erase(nx);
        }
    if(nx != free_.begin())
        {
            auto pv = std::prev(nx);
            if(pv->first + pv->second == offset)
                {
                    pv->second += sz;
                    return;
                }
        }
    free_[offset] = sz;
}

void DeviceArena::reset()
{
    used_.clear();
    free_.clear();
    used_bytes_ = 0;
    if(cap_) free_[0] = cap_;
}

// ---------------------------------------------------------------------------
// layout / params
// ---------------------------------------------------------------------------
// SAMPLE_DIM per model: unicycle 7, double integrator 10, Dubins airplane 10, quadrotor 17
uint32_t sample_dim_of(int32_t model) { return model == KGMT_MODEL_QUADROTOR ? 17u : model == KGMT_MODEL_UNICYCLE ? 7u : 10u; }
// workspace dimension W (W_DIM): 2 for the planar unicycle
uint32_t ws_dims_of(int32_t model) { return model == KGMT_MODEL_UNICYCLE ? 2u : 3u; }
uint32_t regions_of(const kgmt_config& c)
{
    return ws_dims_of(c.model) == 2 ? c.coarse_len * c.coarse_len : c.coarse_len * c.coarse_len * c.coarse_len;
}

kgmt_status validate_config(const kgmt_config& c)
{
    auto bad = [](const char* m) {
        set_error(std::string("invalid config: ") + m);
        return KGMT_ERR_INVALID_ARG;
    };
    if(c.model < KGMT_MODEL_UNICYCLE || c.model > KGMT_MODEL_QUADROTOR) return bad("model");
    if(c.di_rule != KGMT_DI_RULE_RK4 && c.di_rule != KGMT_DI_RULE_REFERENCE) return bad("di_rule");
    if(c.tree_capacity < 2 || c.tree_capacity > (1u << 28)) return bad("tree_capacity must be in [2, 2^28]");
    if(c.samples_per_node < 1 || c.samples_per_node > 1024) return bad("samples_per_node must be in [1, 1024]");
    if(c.max_iterations < 1 || c.max_iterations > 100000) return bad("max_iterations must be in [1, 100000]");
    if(c.min_steps < 1 || c.min_steps > c.max_steps || c.max_steps > 10000) return bad("need 1 <= min_steps <= max_steps <= 10000");
    if(!(c.step_size > 0.0f) || !std::isfinite(c.step_size)) return bad("step_size");
    if(!(c.ws_max > c.ws_min)) return bad("ws_max must exceed ws_min");
    if(c.coarse_len < 1 || c.coarse_len > 128) return bad("coarse_len must be in [1, 128]");
    const uint32_t fine_cells = ws_dims_of(c.model) == 2 ? c.fine_len * c.fine_len : c.fine_len * c.fine_len * c.fine_len;
    if(c.fine_len < 1 || c.fine_len > 8 || fine_cells > KGMT_MAX_FINE_CELLS) return bad("fine_len^W must be in [1, 64]");
    if(!(c.v_max >= c.v_min)) return bad("v_max < v_min");
    if(!(c.goal_radius >= 0.0f) || !(c.epsilon >= 0.0f)) return bad("goal_radius / epsilon");
    if(c.model == KGMT_MODEL_QUADROTOR && (c.ix == 0.0f || c.iy == 0.0f || c.iz == 0.0f)) return bad("inertia must be non-zero");
    if(c.model == KGMT_MODEL_DUBINS_AIRPLANE && !(c.pitch_max >= c.pitch_min)) return bad("pitch_max < pitch_min");
    if(c.model == KGMT_MODEL_UNICYCLE && (c.wheelbase == 0.0f || !std::isfinite(c.wheelbase))) return bad("wheelbase must be finite and non-zero");
    return KGMT_OK;
}

static size_t aligned(size_t& cur, size_t bytes)
{
    size_t off = cur;
    cur += (bytes + 255) & ~size_t(255);
    return off;
}

QueryLayout layout_of(const kgmt_config& c, uint32_t n_obstacles, bool inline_obstacles)
{
    QueryLayout L{};
    L.grid_budget = n_obstacles ? std::min<uint32_t>(kMaxGridItems, std::max<uint32_t>(8192u, 32u * std::min(n_obstacles, 4096u))) : 0u;
    const size_t T = c.tree_capacity, D = sample_dim_of(c.model);
    const size_t R1 = regions_of(c);
    // look-back words of the two chains, one per tile of the smallest size
    // either uses (re-activation tiles of kTileOldSmall old nodes, append
    // tiles of kTileC samples)
    constexpr uint64_t kMinTile = (uint64_t)(kTileC < kTileOldSmall ? kTileC : kTileOldSmall);
    L.tiles_per_chain = (uint32_t)((T + kMinTile - 1) / kMinTile + 1);
    size_t cur = 0;
    L.tree = aligned(cur, T * D * 4);
    L.parent = aligned(cur, T * 4);
    L.cost = aligned(cur, T * 4);
    L.node_r1 = aligned(cur, T * 4);
    L.rep_old = aligned(cur, T * 4);
    L.rep_new = aligned(cur, T * 4);
    L.us = aligned(cur, T * D * 4);
    L.up = aligned(cur, T * 4);
    L.ur1f = aligned(cur, T * 4);
    L.counter = aligned(cur, R1 * 4);
    L.valid = aligned(cur, R1 * 4);
    L.score = aligned(cur, R1 * 4);
    L.marks = aligned(cur, R1 * 8);
    L.newmarks = aligned(cur, R1 * 8);
    L.tiles_old = aligned(cur, (size_t)L.tiles_per_chain * 8);
    L.tiles_slot = aligned(cur, (size_t)L.tiles_per_chain * 8);
    L.path = aligned(cur, ((size_t)c.max_iterations + 2) * D * 4);
    L.grid_meta = aligned(cur, n_obstacles ? 16 : 0);
    L.grid_start = aligned(cur, n_obstacles ? ((size_t)kGridCells + 1) * 2 : 0);
    L.grid_items = aligned(cur, (size_t)L.grid_budget * 2);
    L.obstacles = aligned(cur, inline_obstacles ? (size_t)n_obstacles * 32 : 0);
    L.total = cur;
    return L;
}

QueryParams make_params(const kgmt_config& c, const float* init, const float* goal, char* chunk, const QueryLayout& L, float4* obstacles,
                        uint32_t n_obstacles)
{
    QueryParams p;
    std::memset(&p, 0, sizeof(p));
    p.model = c.model;
    p.di_rule = c.di_rule;
    p.capacity = c.tree_capacity;
    p.samples_per_node = c.samples_per_node;
    p.max_iterations = c.max_iterations;
    p.min_steps = c.min_steps;
    p.max_steps = c.max_steps;
    p.sample_dim = sample_dim_of(c.model);
    // derived values in float, the same operations the CPU restatement uses
    volatile float h = c.step_size;
    p.step_span = (float)(c.max_steps - c.min_steps + 1u);
    p.step_size = h;
    p.half_step = 0.5f * h;
    p.sixth_step = h / 6.0f;
    p.goal_radius = c.goal_radius;
    p.epsilon = c.epsilon;
    p.ws_min = c.ws_min;
    p.ws_max = c.ws_max;
    volatile float range = c.ws_max - c.ws_min;
    volatile float cell = range / (float)c.coarse_len;
    volatile float cell2 = cell * cell;
    p.ws_range = range;
    p.cell_size = cell;
    p.planar = ws_dims_of(c.model) == 2 ? 1 : 0;
    // W_R1_VOL: the coarse cell's measure in the workspace dimension
    p.cell_volume = p.planar ? (float)cell2 : cell2 * cell;
    // a power of two divides exactly like a multiply by its reciprocal
    auto pow2 = [](float v) {
        int e = 0;
        return v > 0.0f && std::isfinite(v) && std::frexp(v, &e) == 0.5f && e > -125 && e < 126;
    };
    p.range_pow2 = pow2(range) ? 1 : 0;
    p.cell_pow2 = pow2(cell) ? 1 : 0;
    p.inv_range = p.range_pow2 ? 1.0f / range : 0.0f;
    p.inv_cell = p.cell_pow2 ? 1.0f / cell : 0.0f;
    p.coarse_len = c.coarse_len;
    p.fine_len = c.fine_len;
    p.regions = regions_of(c);
    p.fine_cells = p.planar ? c.fine_len * c.fine_len : c.fine_len * c.fine_len * c.fine_len;
    p.v_min = c.v_min;
    p.v_max = c.v_max;
    for(int i = 0; i < 4; ++i)
        {
            p.u_min[i] = c.u_min[i];
            volatile float span = c.u_max[i] - c.u_min[i];
            p.u_span[i] = span;
        }
    p.pitch_min = c.pitch_min;
    p.pitch_max = c.pitch_max;
    p.wheelbase = c.wheelbase;
    p.nu = c.nu;
    p.mu = c.mu;
    p.gravity = c.gravity;
    p.mass_inv = c.mass_inv;
    if(c.model == KGMT_MODEL_QUADROTOR)
        {
            volatile float a = c.iy - c.iz, b = c.iz - c.ix, d = c.ix - c.iy;
            p.iix = 1.0f / c.ix;
            p.iiy = 1.0f / c.iy;
            p.iiz = 1.0f / c.iz;
            p.jx = a / c.ix;
            p.jy = b / c.iy;
            p.jz = d / c.iz;
        }
    p.seed = c.seed;
    const uint32_t D = p.sample_dim;
    if(goal)
        for(int i = 0; i < 3; ++i) p.goal[i] = goal[i];
    if(init)
        for(uint32_t i = 0; i < D; ++i) p.init[i] = init[i];
    p.n_obstacles = n_obstacles;
    p.tiles_per_chain = L.tiles_per_chain;
    p.grid_dim = kGridDim;
    p.grid_scale = (float)kGridDim / p.ws_range;
    p.grid_budget = L.grid_budget;
    if(chunk == nullptr)  // parameters only (function-level propagation): no buffers, no grid
        {
            p.obstacles = obstacles;
            return p;
        }
    p.grid_meta = n_obstacles ? (uint32_t*)(chunk + L.grid_meta) : nullptr;
    p.grid_start = n_obstacles ? (uint16_t*)(chunk + L.grid_start) : nullptr;
    p.grid_items = (uint16_t*)(chunk + L.grid_items);
    p.tree = (float*)(chunk + L.tree);
    p.parent = (int32_t*)(chunk + L.parent);
    p.cost = (float*)(chunk + L.cost);
    p.node_r1 = (int32_t*)(chunk + L.node_r1);
    p.rep_old = (uint32_t*)(chunk + L.rep_old);
    p.rep_new = (uint32_t*)(chunk + L.rep_new);
    p.us = (float*)(chunk + L.us);
    p.up = (int32_t*)(chunk + L.up);
    p.ur1f = (uint32_t*)(chunk + L.ur1f);
    p.counter = (int32_t*)(chunk + L.counter);
    p.valid = (int32_t*)(chunk + L.valid);
    p.score = (float*)(chunk + L.score);
    p.marks = (uint64_t*)(chunk + L.marks);
    p.newmarks = (uint64_t*)(chunk + L.newmarks);
    p.tiles_old = (unsigned long long*)(chunk + L.tiles_old);
    p.tiles_slot = (unsigned long long*)(chunk + L.tiles_slot);
    p.path = (float*)(chunk + L.path);
    p.obstacles = obstacles ? obstacles : (float4*)(chunk + L.obstacles);
    return p;
}

kgmt_result to_result(const QueryState& s, uint64_t ticket)
{
    kgmt_result r;
    std::memset(&r, 0, sizeof(r));
    r.status = (int32_t)s.status;
    r.iterations = s.itr;
    r.tree_size = s.tree_size;
    r.goal_index = s.status == KGMT_QUERY_SUCCESS ? s.goal_index : -1;
    r.path_len = s.path_len;
    r.samples_drawn = s.samples_drawn;
    r.solve_ms = s.t_end > s.t_start ? (float)((double)(s.t_end - s.t_start) * 1e-6) : 0.0f;
    r.ticket = ticket;
    r.goal_cost = s.status == KGMT_QUERY_SUCCESS && s.path_len > 0 ? s.goal_cost : 0.0f;
    return r;
}

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
__global__ void k_set_n_slots(Sched* sched, uint32_t n) { sched->n_slots = n; }

__global__ void k_set_endpoints(QueryParams* P, uint32_t first, uint32_t count, const float* __restrict__ inits,
                                const float* __restrict__ goals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= count) return;
    QueryParams& p = P[first + i];
    for(int j = 0; j < KGMT_MAX_SAMPLE_DIM; ++j) p.init[j] = inits[(size_t)i * KGMT_MAX_SAMPLE_DIM + j];
    for(int j = 0; j < 3; ++j) p.goal[j] = goals[(size_t)i * KGMT_MAX_SAMPLE_DIM + j];
}

Engine::~Engine()
{
    if(graph_) cudaGraphExecDestroy(graph_);
    for(auto& e : ev_)
        if(e) cudaEventDestroy(e);
    if(h_running_) cudaFreeHost(h_running_);
    if(h_stage_states_) cudaFreeHost(h_stage_states_);
    cudaFree(d_params_);
    cudaFree(d_states_);
    cudaFree(d_sched_);
    cudaFree(d_tile_a_);
    cudaFree(d_tile_c_);
    cudaFree(d_tile_old_);
    cudaFree(d_slot_list_);
    cudaFree(d_tail_);
    if(own_stream_ && stream_) cudaStreamDestroy(stream_);
}

LaunchArgs Engine::args() const { return LaunchArgs{d_params_, d_states_, d_sched_, d_tile_a_, d_tile_c_, d_tile_old_}; }

kgmt_status Engine::init(uint32_t slots, cudaStream_t stream, uint32_t prop_block, uint32_t iters_per_graph, bool use_graph)
{
    int dev_count = 0;
    if(cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
        {
            cudaGetLastError();
            set_error("no CUDA device");
            return KGMT_ERR_NO_DEVICE;
        }
    if(slots == 0)
        {
            set_error("engine needs at least one slot");
            return KGMT_ERR_INVALID_ARG;
        }
    slots_ = slots;
    if(stream) stream_ = stream;
    else
        {
            KGMT_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
            own_stream_ = true;
        }
    iters_per_graph_ = iters_per_graph ? iters_per_graph : 4;
    use_graph_ = use_graph;
    h_params_.assign(slots, QueryParams{});
    KGMT_CUDA(device_alloc((void**)&d_params_, sizeof(QueryParams) * slots), "cudaMalloc(params)");
    KGMT_CUDA(device_alloc((void**)&d_states_, sizeof(QueryState) * slots), "cudaMalloc(states)");
    KGMT_CUDA(device_alloc((void**)&d_sched_, sizeof(Sched)), "cudaMalloc(sched)");
    KGMT_CUDA(device_alloc((void**)&d_tile_a_, sizeof(uint32_t) * (slots + 1)), "cudaMalloc(tiles)");
    KGMT_CUDA(device_alloc((void**)&d_tile_c_, sizeof(uint32_t) * (slots + 1)), "cudaMalloc(tiles)");
    KGMT_CUDA(device_alloc((void**)&d_tile_old_, sizeof(uint32_t) * slots), "cudaMalloc(tiles)");
    // empty slots: zeroed params, status bytes 0xFF (kSlotEmpty), so no kernel
    // treats a slot as running before it is admitted
    KGMT_CUDA(cudaMemsetAsync(d_params_, 0, sizeof(QueryParams) * slots, stream_), "memset(params)");
    KGMT_CUDA(cudaMemsetAsync(d_states_, 0xFF, sizeof(QueryState) * slots, stream_), "memset(states)");
    KGMT_CUDA(cudaMemsetAsync(d_tile_a_, 0, sizeof(uint32_t) * (slots + 1), stream_), "memset");
    KGMT_CUDA(cudaMemsetAsync(d_tile_c_, 0, sizeof(uint32_t) * (slots + 1), stream_), "memset");
    KGMT_CUDA(cudaMemsetAsync(d_tile_old_, 0, sizeof(uint32_t) * slots, stream_), "memset");
    KGMT_CUDA(device_alloc((void**)&d_tail_, tail_scratch_bytes()), "cudaMalloc(tail)");
    KGMT_CUDA(device_alloc((void**)&d_slot_list_, sizeof(uint32_t) * slots), "cudaMalloc(slot list)");
    KGMT_CUDA(cudaMemsetAsync(d_tail_, 0, tail_scratch_bytes(), stream_), "memset(tail)");
    {
        const char* e = std::getenv("KGMT_TAIL");
        tail_on_ = !(e && e[0] == '0');
    }
    // the running count and the tail launch's report, written by the device
    // into mapped pinned memory
    KGMT_CUDA(cudaHostAlloc((void**)&h_running_, sizeof(uint32_t) * 4, cudaHostAllocMapped), "cudaHostAlloc(mapped)");
    std::memset(h_running_, 0, sizeof(uint32_t) * 4);
    KGMT_CUDA(cudaHostGetDevicePointer((void**)&d_running_, h_running_, 0), "cudaHostGetDevicePointer");
    KGMT_CUDA(cudaMallocHost((void**)&h_stage_states_, sizeof(QueryState) * slots), "cudaMallocHost(states)");
    for(auto& e : ev_) KGMT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    return set_prop_block(prop_block ? prop_block : 256);
}

kgmt_status Engine::set_prop_block(uint32_t block)
{
    if(block != 128 && block != 256 && block != 512)
        {
            set_error("propagate block must be 128, 256 or 512");
            return KGMT_ERR_INVALID_ARG;
        }
    prop_block_ = block;
    int dev = 0, sms = 0;
    KGMT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    KGMT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    for(int m : {1, 2, 4, 8, 15}) grid_a_[m] = sms * propagate_blocks_per_sm((int)block, m);
    grid_c_ = sms * append_blocks_per_sm();
    // the tail launch: one block per SM (all blocks resident for its grid-wide
    // barriers), iterations up to two samples per thread
    for(int m : {1, 2, 4, 8, 15})
        {
            const int per_sm = tail_blocks_per_sm(m);
            tail_grid_[m] = (per_sm >= 1 && sms >= 2 * kTailQueries && sms <= kTailMaxBlocks) ? sms : 0;
        }
    tail_max_samples_ = 2u * (uint32_t)sms * (uint32_t)kTailThreads;
    Sched s;
    std::memset(&s, 0, sizeof(s));
    s.prop_tile = block;
    s.prop_block = block;
    // two samples per thread once an iteration fills the resident threads of
    // the double-integrator variant twice
    s.pair_samples = 2u * (uint32_t)grid_a_[1] * block;
    s.n_sms = (uint32_t)sms;
    s.old_tile = kTileOld;
    s.host_running = d_running_;
    KGMT_CUDA(cudaMemcpyAsync(d_sched_, &s, sizeof(s), cudaMemcpyHostToDevice, stream_), "upload(sched)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "sync");
    if(graph_)
        {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
    return KGMT_OK;
}

void Engine::set_max_obstacles(uint32_t max_obs)
{
    const uint32_t boxes = smem_boxes_for(max_obs);
    if(boxes == smem_boxes_) return;
    smem_boxes_ = boxes;
    if(graph_)
        {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
}

void Engine::set_models(int mask)
{
    mask = variant_of(mask & 15);
    if(mask == models_) return;
    models_ = mask;
    if(graph_)
        {
            cudaGraphExecDestroy(graph_);
            graph_ = nullptr;
        }
}

kgmt_status Engine::upload_params(uint32_t first, uint32_t count)
{
    if(first + count > slots_)
        {
            set_error("upload_params: slot range out of bounds");
            return KGMT_ERR_INVALID_ARG;
        }
    if(count == 0) return KGMT_OK;
    // pageable source: the copy has completed when the call returns
    KGMT_CUDA(cudaMemcpyAsync(d_params_ + first, h_params_.data() + first, sizeof(QueryParams) * count, cudaMemcpyHostToDevice, stream_),
              "upload(params)");
    return KGMT_OK;
}

kgmt_status Engine::init_slots(uint32_t first, uint32_t count, const float* d_inits, const float* d_goals)
{
    if(first + count > slots_)
        {
            set_error("init_slots: slot range out of bounds");
            return KGMT_ERR_INVALID_ARG;
        }
    if(count == 0) return KGMT_OK;
    if(d_inits && d_goals)
        {
            k_set_endpoints<<<(count + 127) / 128, 128, 0, stream_>>>(d_params_, first, count, d_inits, d_goals);
            KGMT_CUDA(cudaGetLastError(), "k_set_endpoints");
            launches_ += 1;
        }
    KGMT_CUDA(launch_admit(args(), first, count, stream_), "k_admit");
    launches_ += 2;  // k_admit + k_build_grid
    return KGMT_OK;
}

kgmt_status Engine::set_active(uint32_t n_active)
{
    if(n_active > slots_)
        {
            set_error("set_active: more slots than the engine holds");
            return KGMT_ERR_INVALID_ARG;
        }
    n_active_ = n_active;
    // by value through a kernel parameter: no host memory to keep alive, no wait
    k_set_n_slots<<<1, 1, 0, stream_>>>(d_sched_, n_active);
    KGMT_CUDA(cudaGetLastError(), "k_set_n_slots");
    launches_ += 1;
    return KGMT_OK;
}

kgmt_status Engine::schedule()
{
    KGMT_CUDA(launch_schedule(args(), stream_), "k_schedule");
    launches_ += 1;
    return KGMT_OK;
}

kgmt_status Engine::admit(uint32_t first, uint32_t count, uint32_t n_active, const float* d_inits, const float* d_goals)
{
    NvtxRange r("kgmt admit");
    kgmt_status st = upload_params(first, count);
    if(st == KGMT_OK) st = set_active(n_active);
    if(st == KGMT_OK) st = init_slots(first, count, d_inits, d_goals);
    if(st == KGMT_OK) st = schedule();
    return st;
}

kgmt_status Engine::record_event(cudaEvent_t* out)
{
    if(prof_used_ >= prof_events_.size())
        {
            cudaEvent_t e;
            KGMT_CUDA(cudaEventCreate(&e), "cudaEventCreate");
            prof_events_.push_back(e);
        }
    cudaEvent_t e = prof_events_[prof_used_++];
    KGMT_CUDA(cudaEventRecord(e, stream_), "cudaEventRecord");
    if(out) *out = e;
    return KGMT_OK;
}

kgmt_status Engine::launch_iteration()
{
    const LaunchArgs a = args();
    // kernel kinds in the profile: 0 propagate (with the region scores), 2 append
    for(int k = 0; k < 3; k += 2)
        {
            if(profile_)
                {
                    kgmt_status st = record_event(nullptr);
                    if(st != KGMT_OK) return st;
                    prof_kind_.push_back(k);
                }
            if(k == 0) KGMT_CUDA(launch_propagate(a, (int)prop_block_, models_, grid_a_[models_], smem_boxes_, stream_), "k_propagate");
            else KGMT_CUDA(launch_append(a, grid_c_, stream_), "k_append");
            if(profile_)
                {
                    kgmt_status st = record_event(nullptr);
                    if(st != KGMT_OK) return st;
                }
        }
    launches_ += 2;
    return KGMT_OK;
}

void Engine::reset_counters()
{
    launches_ = 0;
    prof_used_ = 0;
    prof_kind_.clear();
    tail_iters_ = 0;
    // the two counters are adjacent: one memset
    if(d_tail_) cudaMemsetAsync(&d_tail_->fp32_ops, 0, 2 * sizeof(unsigned long long), stream_);
}

kgmt_status Engine::tail_counters(uint32_t* iterations, uint64_t* fp32_ops, uint64_t* samples)
{
    unsigned long long v[2] = {0, 0};
    KGMT_CUDA(cudaMemcpyAsync(v, &d_tail_->fp32_ops, sizeof(v), cudaMemcpyDeviceToHost, stream_), "download(tail)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    *iterations = tail_iters_;
    *fp32_ops = v[0];
    *samples = v[1];
    return KGMT_OK;
}

kgmt_status Engine::run_tail(bool* done, bool* declined_at_once)
{
    NvtxRange r("kgmt tail launch");
    if(profile_)
        {
            kgmt_status st = record_event(nullptr);
            if(st != KGMT_OK) return st;
            prof_kind_.push_back(1);
        }
    KGMT_CUDA(launch_tail(args(), d_tail_, models_, tail_grid_[models_], smem_boxes_, tail_max_samples_, d_running_ + 2, stream_), "k_tail");
    if(profile_)
        {
            kgmt_status st = record_event(nullptr);
            if(st != KGMT_OK) return st;
        }
    launches_ += 1;
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    volatile uint32_t* w = h_running_;
    tail_iters_ += w[2];
    *done = w[0] == 0u;
    *declined_at_once = w[3] != 0u && w[2] == 0u;
    return KGMT_OK;
}

kgmt_status Engine::kernel_times(float ms[3], uint32_t n[3])
{
    for(int k = 0; k < 3; ++k) ms[k] = 0.0f, n[k] = 0;
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    for(size_t i = 0; i < prof_kind_.size(); ++i)
        {
            float t = 0.0f;
            KGMT_CUDA(cudaEventElapsedTime(&t, prof_events_[2 * i], prof_events_[2 * i + 1]), "cudaEventElapsedTime");
            ms[prof_kind_[i]] += t;
            n[prof_kind_[i]] += 1;
        }
    return KGMT_OK;
}

kgmt_status Engine::build_graph()
{
    cudaGraph_t g = nullptr;
    KGMT_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    kgmt_status st = KGMT_OK;
    const uint64_t saved = launches_;
    for(uint32_t i = 0; i < iters_per_graph_ && st == KGMT_OK; ++i) st = launch_iteration();
    launches_ = saved;
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if(st != KGMT_OK)
        {
            if(g) cudaGraphDestroy(g);
            return st;
        }
    KGMT_CUDA(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    return cuda_status(e, "cudaGraphInstantiate");
}

kgmt_status Engine::launch_unit()
{
    NvtxRange r(use_graph_ && !profile_ ? "kgmt iterations (graph replay)" : "kgmt iterations (direct launches)");
    if(use_graph_ && !profile_)
        {
            if(!graph_)
                {
                    kgmt_status st = build_graph();
                    if(st != KGMT_OK) return st;
                }
            KGMT_CUDA(cudaGraphLaunch(graph_, stream_), "cudaGraphLaunch");
            launches_ += 2ull * iters_per_graph_;
        }
    else
        {
            for(uint32_t i = 0; i < iters_per_graph_; ++i)
                {
                    kgmt_status st = launch_iteration();
                    if(st != KGMT_OK) return st;
                }
        }
    iters_launched_ += iters_per_graph_;
    return KGMT_OK;
}

kgmt_status Engine::run_until_done(uint32_t max_iters)
{
    // Units are launched one ahead of the poll: after unit u-1 completes, the
    // running count the last schedule wrote (unit u-1's or a later one's) is
    // read from the mapped host word; nothing but the event record sits in
    // the stream between two graph replays.  Once at most kTailQueries
    // queries run, one persistent tail launch takes the iterations left (it
    // hands back to the units when an iteration outgrows it; after a launch
    // that could not take even one iteration, the next attempt waits twice as
    // many units).
    NvtxRange r("kgmt run until done");
    const uint32_t G = iters_per_graph_;
    const uint32_t max_units = (max_iters + G - 1) / G + 2;
    volatile uint32_t* running = h_running_;
    const bool tail = tail_on_ && tail_grid_[models_] > 0;
    uint32_t backoff = 1, wait_units = 0;
    if(tail && n_active_ <= (uint32_t)kTailQueries)
        {
            bool done = false, at_once = false;
            kgmt_status st = run_tail(&done, &at_once);
            if(st != KGMT_OK) return st;
            if(done) return KGMT_OK;
            if(at_once) wait_units = backoff, backoff *= 2;
        }
    for(uint32_t u = 0; u < max_units; ++u)
        {
            kgmt_status st = launch_unit();
            if(st != KGMT_OK) return st;
            KGMT_CUDA(cudaEventRecord(ev_[u & 1], stream_), "cudaEventRecord");
            if(u > 0)
                {
                    KGMT_CUDA(cudaEventSynchronize(ev_[(u - 1) & 1]), "cudaEventSynchronize");
                    const uint32_t n = *running;
                    if(n == 0) break;
                    if(wait_units > 0) --wait_units;
                    else if(tail && n <= (uint32_t)kTailQueries)
                        {
                            bool done = false, at_once = false;
                            st = run_tail(&done, &at_once);
                            if(st != KGMT_OK) return st;
                            if(done) break;
                            if(at_once) wait_units = backoff, backoff *= 2;
                        }
                }
        }
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return KGMT_OK;
}

kgmt_status Engine::run_iterations(uint32_t iters)
{
    for(uint32_t i = 0; i < iters; ++i)
        {
            kgmt_status st = launch_iteration();
            if(st != KGMT_OK) return st;
        }
    iters_launched_ += iters;
    return KGMT_OK;
}

kgmt_status Engine::launch_units(uint32_t units)
{
    for(uint32_t u = 0; u < units; ++u)
        {
            kgmt_status st = launch_unit();
            if(st != KGMT_OK) return st;
        }
    return KGMT_OK;
}

kgmt_status Engine::upload_params_async(uint32_t slot, const QueryParams* pinned)
{
    if(slot >= slots_)
        {
            set_error("upload_params_async: slot out of bounds");
            return KGMT_ERR_INVALID_ARG;
        }
    h_params_[slot] = *pinned;
    KGMT_CUDA(cudaMemcpyAsync(d_params_ + slot, pinned, sizeof(QueryParams), cudaMemcpyHostToDevice, stream_), "upload(params)");
    return KGMT_OK;
}

kgmt_status Engine::admit_slot_list(const uint32_t* pinned_slots, uint32_t count)
{
    if(count == 0) return KGMT_OK;
    if(count > slots_)
        {
            set_error("admit_slot_list: more slots than the engine holds");
            return KGMT_ERR_INVALID_ARG;
        }
    KGMT_CUDA(cudaMemcpyAsync(d_slot_list_, pinned_slots, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, stream_), "upload(slots)");
    KGMT_CUDA(launch_admit(args(), 0, count, stream_, d_slot_list_), "k_admit");
    launches_ += 2;
    return KGMT_OK;
}

kgmt_status Engine::enqueue_state_copy(uint32_t count, QueryState* pinned_states, uint32_t* pinned_error)
{
    if(count > slots_)
        {
            set_error("enqueue_state_copy: more slots than the engine holds");
            return KGMT_ERR_INVALID_ARG;
        }
    if(count)
        KGMT_CUDA(cudaMemcpyAsync(pinned_states, d_states_, sizeof(QueryState) * count, cudaMemcpyDeviceToHost, stream_), "download(states)");
    KGMT_CUDA(cudaMemcpyAsync(pinned_error, &d_sched_->error, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "download(error)");
    return KGMT_OK;
}

kgmt_status Engine::read_states(uint32_t first, uint32_t count, QueryState* out)
{
    if(count == 0) return KGMT_OK;
    KGMT_CUDA(cudaMemcpyAsync(out, d_states_ + first, sizeof(QueryState) * count, cudaMemcpyDeviceToHost, stream_), "download(states)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return KGMT_OK;
}

kgmt_status Engine::write_status(uint32_t slot, uint32_t status)
{
    KGMT_CUDA(cudaMemcpyAsync(&d_states_[slot].status, &status, sizeof(status), cudaMemcpyHostToDevice, stream_), "upload(status)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return KGMT_OK;
}

kgmt_status Engine::read_states_and_error(uint32_t first, uint32_t count, QueryState* out, uint32_t* err)
{
    // both copies land in pinned staging, so they are queued together and
    // waited for once (a pageable destination would wait for each copy)
    if(first + count > slots_)
        {
            set_error("read_states_and_error: slot range out of bounds");
            return KGMT_ERR_INVALID_ARG;
        }
    if(count)
        KGMT_CUDA(cudaMemcpyAsync(h_stage_states_, d_states_ + first, sizeof(QueryState) * count, cudaMemcpyDeviceToHost, stream_),
                  "download(states)");
    KGMT_CUDA(cudaMemcpyAsync(&h_running_[1], &d_sched_->error, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "download(error)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    if(count) std::memcpy(out, h_stage_states_, sizeof(QueryState) * count);
    *err = h_running_[1];
    return KGMT_OK;
}

kgmt_status Engine::extract_paths(uint32_t n_active)
{
    NvtxRange r("kgmt paths");
    KGMT_CUDA(launch_paths(args(), n_active, stream_), "k_paths");
    launches_ += 1;
    return KGMT_OK;
}

kgmt_status Engine::read_error(uint32_t* err)
{
    KGMT_CUDA(cudaMemcpyAsync(err, &d_sched_->error, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_), "download(error)");
    KGMT_CUDA(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    return KGMT_OK;
}

}  // namespace kgmt
