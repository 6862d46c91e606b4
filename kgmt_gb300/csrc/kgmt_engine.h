// kgmt_engine.h -- host runtime of the planning engine.
//
// The engine owns the device-resident descriptors of up to `slots` queries
// and replays the per-iteration kernel chain (optionally as a captured CUDA
// graph) until every admitted query has finished.  The host only polls one
// counter, one replay behind, so the GPU never waits on the CPU.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "kgmt_kernels.h"
#include "kgmt_types.h"

namespace kgmt {

void set_error(const std::string& msg);
kgmt_status cuda_status(cudaError_t e, const char* what);
// device (or managed) memory the GPU may read and write; false for host
// memory, unregistered pointers and NULL (allocates nothing)
bool is_device_pointer(const void* p);

// first-fit allocator over one device allocation
class DeviceArena {
   public:
    ~DeviceArena();
    kgmt_status reserve(size_t bytes);  // (re)allocates when empty and too small
    bool alloc(size_t bytes, size_t* offset);
    void release(size_t offset);
    void reset();
    char* base() const { return base_; }
    size_t capacity() const { return cap_; }
    size_t in_use() const { return used_bytes_; }

   private:
    char* base_ = nullptr;
    size_t cap_ = 0;
    size_t used_bytes_ = 0;
    std::map<size_t, size_t> free_;  // offset -> size
    std::map<size_t, size_t> used_;
};

struct QueryLayout {
    size_t tree, parent, cost, node_r1, rep_old, rep_new, us, up, ur1f;
    size_t counter, valid, score, marks, newmarks, tiles_old, tiles_slot, path, grid_meta, grid_start, grid_items, obstacles;
    size_t total;
    uint32_t tiles_per_chain;
    uint32_t grid_budget;
};

kgmt_status validate_config(const kgmt_config& c);
// buffers of one query with n_obstacles boxes; the boxes themselves are
// placed in the chunk only when inline_obstacles (batches share one region)
QueryLayout layout_of(const kgmt_config& c, uint32_t n_obstacles, bool inline_obstacles);
// derived constants in float exactly as the kernels expect them; buffers
// point into `base + chunk_offset`; obstacles at `obstacles` (device)
QueryParams make_params(const kgmt_config& c, const float* init, const float* goal, char* chunk, const QueryLayout& L, float4* obstacles,
                        uint32_t n_obstacles);
uint32_t sample_dim_of(int32_t model);
uint32_t ws_dims_of(int32_t model);
kgmt_result to_result(const QueryState& s, uint64_t ticket);

class Engine {
   public:
    ~Engine();
    kgmt_status init(uint32_t slots, cudaStream_t stream, uint32_t prop_block, uint32_t iters_per_graph, bool use_graph);
    uint32_t slots() const { return slots_; }
    cudaStream_t stream() const { return stream_; }
    QueryParams& host_params(uint32_t slot) { return h_params_[slot]; }
    LaunchArgs args() const;

    // uploads params of [first, first+count), initialises those slots and
    // recomputes the schedule; n_active = slots the kernels look at.  With
    // d_inits / d_goals (device rows of KGMT_MAX_SAMPLE_DIM floats) the start
    // and goal are taken from device memory instead of the host params.
    kgmt_status admit(uint32_t first, uint32_t count, uint32_t n_active, const float* d_inits = nullptr,
                      const float* d_goals = nullptr);
    // the pieces of admit, for callers that admit several slot ranges
    kgmt_status upload_params(uint32_t first, uint32_t count);
    kgmt_status init_slots(uint32_t first, uint32_t count, const float* d_inits = nullptr, const float* d_goals = nullptr);
    kgmt_status set_active(uint32_t n_active);
    kgmt_status schedule();
    // runs iterations until no query is running (or max_iters + slack)
    kgmt_status run_until_done(uint32_t max_iters);
    // runs exactly `iters` iterations (direct launches)
    kgmt_status run_iterations(uint32_t iters);
    // enqueues `units` units of iters_per_graph iterations (graph replays when
    // graphs are on); returns without waiting
    kgmt_status launch_units(uint32_t units);
    // served admission, all enqueued without waiting: the params of one slot
    // from pinned host memory; then the slots listed in pinned host memory
    // admitted by one launch (their raw boxes staged by it)
    kgmt_status upload_params_async(uint32_t slot, const QueryParams* pinned);
    kgmt_status admit_slot_list(const uint32_t* pinned_slots, uint32_t count);
    // enqueues copies of the states of slots [0, count) and of the error bits
    // into pinned host memory (readable after the stream reaches them)
    kgmt_status enqueue_state_copy(uint32_t count, QueryState* pinned_states, uint32_t* pinned_error);
    kgmt_status read_states(uint32_t first, uint32_t count, QueryState* out);
    // sets one slot's status on the device (between launches)
    kgmt_status write_status(uint32_t slot, uint32_t status);
    // states and the error bits in one wait
    kgmt_status read_states_and_error(uint32_t first, uint32_t count, QueryState* out, uint32_t* err);
    kgmt_status extract_paths(uint32_t n_active);
    kgmt_status read_error(uint32_t* err);
    kgmt_status set_prop_block(uint32_t block);
    uint32_t prop_block() const { return prop_block_; }
    // model mix of the admitted queries (bit 0 double integrator, bit 1
    // quadrotor, bit 2 Dubins airplane, bit 3 unicycle): picks the propagate
    // kernel variant (single-model variants, or the one for any mix); a
    // change drops the graph
    void set_models(int mask);
    // largest box count of the admitted queries: sizes the propagate kernel's
    // shared-memory box stage (a change drops the graph)
    void set_max_obstacles(uint32_t max_obs);
    static int model_bit(int32_t model)
    {
        return model == KGMT_MODEL_QUADROTOR ? 2 : model == KGMT_MODEL_DUBINS_AIRPLANE ? 4 : model == KGMT_MODEL_UNICYCLE ? 8 : 1;
    }
    // the propagate variant a model mask runs on
    static int variant_of(int mask) { return (mask == 1 || mask == 2 || mask == 4 || mask == 8) ? mask : 15; }
    uint32_t iterations_launched() const { return iters_launched_; }

    // per-kernel CUDA-event timing (direct launches instead of the graph)
    void set_profile(bool on) { profile_ = on; }
    void reset_counters();
    void add_launches(uint64_t n) { launches_ += n; }
    uint64_t launches() const { return launches_; }
    // sums the event pairs recorded since reset_counters (call after a sync)
    // kinds: 0 propagate, 1 tail launch, 2 append
    kgmt_status kernel_times(float ms[3], uint32_t n[3]);
    // the persistent tail launch (kgmt_tail.cuh) for the last few running
    // queries in run_until_done; on by default, KGMT_TAIL=0 turns it off
    void set_tail(bool on) { tail_on_ = on; }
    // iterations and algorithmic FP32 operations of the tail launches since
    // reset_counters (call after a sync)
    kgmt_status tail_counters(uint32_t* iterations, uint64_t* fp32_ops, uint64_t* samples);

   private:
    kgmt_status launch_iteration();
    // one tail launch after what is queued, waited for; *done: nothing runs any more
    kgmt_status run_tail(bool* done, bool* declined_at_once);
    kgmt_status record_event(cudaEvent_t* out);
    kgmt_status launch_unit();
    kgmt_status build_graph();

    uint32_t slots_ = 0;
    cudaStream_t stream_ = nullptr;
    bool own_stream_ = false;
    uint32_t prop_block_ = 256;
    uint32_t iters_per_graph_ = 4;
    bool use_graph_ = true;
    int grid_a_[16] = {};           // propagate grid per variant
    int grid_c_ = 0;
    int models_ = 15;               // propagate variant (Engine::variant_of)
    uint32_t smem_boxes_ = kSmemObstacles;  // boxes staged in shared memory per propagate block
    QueryParams* d_params_ = nullptr;
    QueryState* d_states_ = nullptr;
    Sched* d_sched_ = nullptr;
    uint32_t* d_tile_a_ = nullptr;
    uint32_t* d_tile_c_ = nullptr;
    uint32_t* d_tile_old_ = nullptr;
    uint32_t* d_slot_list_ = nullptr;  // [slots] slots of a served admission
    uint32_t* h_running_ = nullptr;  // mapped pinned host words: [0] Sched::host_running, [1] error readback,
                                     // [2] tail iterations, [3] tail stopped for size
    QueryState* h_stage_states_ = nullptr;  // pinned staging for state readbacks
    uint32_t* d_running_ = nullptr;  // its device address
    cudaEvent_t ev_[2] = {nullptr, nullptr};
    cudaGraphExec_t graph_ = nullptr;
    std::vector<QueryParams> h_params_;
    uint32_t iters_launched_ = 0;
    uint64_t launches_ = 0;
    bool profile_ = false;
    bool tail_on_ = true;
    TailScratch* d_tail_ = nullptr;
    int tail_grid_[16] = {};          // tail launch grid per propagate variant (0: unavailable)
    uint32_t tail_max_samples_ = 0;   // largest iteration the tail launch takes
    uint32_t n_active_ = 0;           // slots the kernels look at
    uint32_t tail_iters_ = 0;
    std::vector<cudaEvent_t> prof_events_;  // pool, pairs (start, stop)
    std::vector<int> prof_kind_;            // kernel of each pair
    size_t prof_used_ = 0;
};

}  // namespace kgmt
