// kgmt_noalloc.cu -- kgmt_plan_noalloc: one planning query that allocates no
// memory at all.
//
// For callers that cannot call cudaMalloc: code running under a memory
// manager that owns every device byte (a fixed pool carved out at start-up,
// a real-time loop that must not hit the allocator), plug-in hosts that
// forbid allocation after initialisation.  The planner's working memory --
// engine descriptors, tree, frontier lists, unexplored samples, region
// tables, look-back words, path rows -- lives in the file-scope device array
// g_noalloc_scratch below, which every GPU that loads this library holds until
// the process exits.  The caller passes the obstacles and the output buffers.
//
// Rules of use:
//  * the first KGMT_NOALLOC_RESERVED_BYTES of the array hold the engine
//    descriptors; a query whose working memory (kgmt_query_bytes()) exceeds
//    the rest is rejected with KGMT_ERR_INVALID_ARG;
//  * every call on a device shares the one array, and it keeps the contents
//    of the last call: the entry point clears what must start at zero.  Calls
//    that overlap on the GPU (two host threads, or two streams) race on the
//    array and corrupt each other;
//  * the first call on a device, with that device current, looks up the
//    array's device address (cudaGetSymbolAddress); the address is kept per
//    CUDA context, so a context created anew (after cudaDeviceReset) is set
//    up again by its first call.  Make that first call before any stream
//    capture begins;
//  * every call waits for its stream before it returns (the iteration count
//    is read back between launches); no CUDA graph, event or stream is
//    created.
#include <cuda.h>

#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "kgmt_engine.h"

namespace kgmt {

constexpr size_t kNoAllocScratchBytes = KGMT_NOALLOC_SCRATCH_BYTES;
constexpr size_t kNoAllocReservedBytes = KGMT_NOALLOC_RESERVED_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// host-side cache of the array's device address, one entry per CUDA context
// (keyed on the context's unique id, which a recreated context never reuses)
static std::vector<std::pair<unsigned long long, unsigned char*>> g_scratch_addr;
static std::mutex g_scratch_mu;

// unique id of the calling thread's current context, through the driver entry
// points the runtime hands out (no link against the driver library); false
// when unavailable, and the address is then looked up on every call
static bool current_context_id(unsigned long long* id)
{
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
           q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f;
        f = nullptr;
        if(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
           q == cudaDriverEntryPointSuccess)
            get_id = (GetId)f;
        cudaGetLastError();
    });
    if(!get_current || !get_id) return false;
    CUcontext ctx = nullptr;
    if(get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

static kgmt_status scratch_address(unsigned char** out)
{
    int dev = 0;
    kgmt_status st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if(st != KGMT_OK) return st;
    // makes the device's primary context current on this thread (no allocation)
    st = cuda_status(cudaSetDevice(dev), "cudaSetDevice");
    if(st != KGMT_OK) return st;
    unsigned long long id = 0;
    const bool keyed = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if(keyed)
        for(const auto& e : g_scratch_addr)
            if(e.first == id)
                {
                    *out = e.second;
                    return KGMT_OK;
                }
    void* p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    if(st != KGMT_OK) return st;
    if(keyed) g_scratch_addr.emplace_back(id, (unsigned char*)p);
    *out = (unsigned char*)p;
    return KGMT_OK;
}

static size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace kgmt

using namespace kgmt;

#define NA_CHECK(expr)                      \
    do {                                    \
        kgmt_status st_ = (expr);           \
        if(st_ != KGMT_OK) return st_;      \
    } while(0)

extern "C" kgmt_status kgmt_plan_noalloc(const kgmt_config* cfg, const float* h_initial, const float* h_goal, const float* d_obstacles,
                                         uint32_t n_obstacles, float* d_samples, int32_t* d_parents, float* d_costs, uint32_t max_nodes,
                                         float* d_path, uint32_t max_path_rows, kgmt_result* result, void* stream)
{
    if(!cfg || !h_initial || !h_goal || !result)
        {
            set_error("kgmt_plan_noalloc: NULL argument");
            return KGMT_ERR_INVALID_ARG;
        }
    if(n_obstacles > 0 && !d_obstacles)
        {
            set_error("kgmt_plan_noalloc: obstacles pointer is NULL");
            return KGMT_ERR_INVALID_ARG;
        }
    NA_CHECK(validate_config(*cfg));
    int dev_count = 0;
    if(cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
        {
            cudaGetLastError();
            set_error("no CUDA device");
            return KGMT_ERR_NO_DEVICE;
        }
    // every pointer the kernels or the device-to-device copies touch must be
    // device memory: a host pointer would be read or written by the GPU
    // (cudaPointerGetAttributes allocates nothing)
    const struct {
        const void* p;
        const char* what;
    } dev_ptrs[] = {{n_obstacles ? d_obstacles : nullptr, "obstacles"}, {d_samples, "d_samples"}, {d_parents, "d_parents"},
                    {d_costs, "d_costs"}, {d_path, "d_path"}};
    for(const auto& d : dev_ptrs)
        if(d.p && !is_device_pointer(d.p))
            {
                set_error(std::string("kgmt_plan_noalloc: ") + d.what + " must be a device pointer");
                return KGMT_ERR_INVALID_ARG;
            }
    // working memory: engine descriptors in the reserved head, then the query chunk
    const size_t off_params = 0;
    const size_t off_state = round256(off_params + sizeof(QueryParams));
    const size_t off_sched = round256(off_state + sizeof(QueryState));
    const size_t off_tiles = round256(off_sched + sizeof(Sched));
    const size_t off_chunk = kNoAllocReservedBytes;
    static_assert(((sizeof(QueryParams) + 255) / 256 + (sizeof(QueryState) + 255) / 256 + (sizeof(Sched) + 255) / 256 + 1) * 256 <=
                    kNoAllocReservedBytes,
                  "the engine descriptors fit the reserved head of the scratch array");
    const QueryLayout L = layout_of(*cfg, n_obstacles, true);
    if(L.total > kNoAllocScratchBytes - off_chunk)
        {
            set_error("kgmt_plan_noalloc: the query needs " + std::to_string(L.total) + " bytes of working memory (kgmt_query_bytes); the static scratch holds " +
                      std::to_string(kNoAllocScratchBytes - off_chunk) + " for a query (reduce tree_capacity, or use kgmt_plan)");
            return KGMT_ERR_INVALID_ARG;
        }
    unsigned char* base = nullptr;
    NA_CHECK(scratch_address(&base));
    cudaStream_t s = (cudaStream_t)stream;

    QueryParams* d_params = (QueryParams*)(base + off_params);
    QueryState* d_state = (QueryState*)(base + off_state);
    Sched* d_sched = (Sched*)(base + off_sched);
    uint32_t* d_tiles = (uint32_t*)(base + off_tiles);
    LaunchArgs a{d_params, d_state, d_sched, d_tiles, d_tiles + 2, d_tiles + 4};

    const uint32_t block = 256;
    int dev = 0, sms = 0;
    NA_CHECK(cuda_status(cudaGetDevice(&dev), "cudaGetDevice"));
    NA_CHECK(cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
    const int models = Engine::variant_of(Engine::model_bit(cfg->model));
    const int grid_a = sms * propagate_blocks_per_sm((int)block, models);
    const int grid_c = sms * append_blocks_per_sm();

    // the array keeps the previous call's contents: reset what starts at zero
    const QueryParams params = make_params(*cfg, h_initial, h_goal, (char*)(base + off_chunk), L, nullptr, n_obstacles);
    Sched sched;
    std::memset(&sched, 0, sizeof(sched));
    sched.n_slots = 1;
    sched.prop_tile = block;
    sched.prop_block = block;
    sched.pair_samples = 2u * (uint32_t)grid_a * block;
    sched.n_sms = (uint32_t)sms;
    sched.old_tile = kTileOld;
    NA_CHECK(cuda_status(cudaMemcpyAsync(d_params, &params, sizeof(params), cudaMemcpyHostToDevice, s), "upload(params)"));
    NA_CHECK(cuda_status(cudaMemcpyAsync(d_sched, &sched, sizeof(sched), cudaMemcpyHostToDevice, s), "upload(sched)"));
    NA_CHECK(cuda_status(cudaMemsetAsync(d_state, 0xFF, sizeof(QueryState), s), "memset(state)"));
    NA_CHECK(cuda_status(cudaMemsetAsync(d_tiles, 0, 5 * sizeof(uint32_t), s), "memset(tiles)"));
    // params and sched live on this host stack frame: finish the copies first
    NA_CHECK(cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    NA_CHECK(cuda_status(launch_stage_obstacles(d_obstacles, params.obstacles, n_obstacles, (int)ws_dims_of(cfg->model), s), "stage obstacles"));
    NA_CHECK(cuda_status(launch_admit(a, 0, 1, s), "k_admit"));
    NA_CHECK(cuda_status(launch_schedule(a, s), "k_schedule"));

    // iterations until the query stops; poll the running count every 4
    uint32_t running = 1;
    for(uint32_t it = 0; it < cfg->max_iterations + 8 && running; it += 4)
        {
            for(int k = 0; k < 4; ++k)
                {
                    NA_CHECK(cuda_status(launch_propagate(a, (int)block, models, grid_a, smem_boxes_for(n_obstacles), s), "k_propagate"));
                    NA_CHECK(cuda_status(launch_append(a, grid_c, s), "k_append"));
                }
            NA_CHECK(cuda_status(cudaMemcpyAsync(&running, &d_sched->running, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "poll"));
            NA_CHECK(cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
        }
    NA_CHECK(cuda_status(launch_paths(a, 1, s), "k_paths"));
    QueryState state;
    uint32_t err = 0;
    NA_CHECK(cuda_status(cudaMemcpyAsync(&state, d_state, sizeof(state), cudaMemcpyDeviceToHost, s), "download(state)"));
    NA_CHECK(cuda_status(cudaMemcpyAsync(&err, &d_sched->error, sizeof(err), cudaMemcpyDeviceToHost, s), "download(error)"));
    NA_CHECK(cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    if(err != 0)
        {
            set_error("kgmt_plan_noalloc: a device-side wait gave up (error bits " + std::to_string(err) + ")");
            return KGMT_ERR_TIMEOUT;
        }
    if(bounds_error_take() != 0)
        {
            set_error("kgmt_plan_noalloc: an index check failed (bounds-checked build)");
            return KGMT_ERR_INTERNAL;
        }
    // outputs into the caller's buffers
    const uint32_t n = state.tree_size < max_nodes ? state.tree_size : max_nodes;
    const size_t D = params.sample_dim;
    if(d_samples && n)
        NA_CHECK(cuda_status(cudaMemcpyAsync(d_samples, params.tree, n * D * 4, cudaMemcpyDeviceToDevice, s), "copy tree"));
    if(d_parents && n)
        NA_CHECK(cuda_status(cudaMemcpyAsync(d_parents, params.parent, n * 4ull, cudaMemcpyDeviceToDevice, s), "copy parents"));
    if(d_costs && n) NA_CHECK(cuda_status(cudaMemcpyAsync(d_costs, params.cost, n * 4ull, cudaMemcpyDeviceToDevice, s), "copy costs"));
    const uint32_t rows = state.path_len < max_path_rows ? state.path_len : max_path_rows;
    if(d_path && rows)
        NA_CHECK(cuda_status(cudaMemcpyAsync(d_path, params.path, (size_t)rows * D * 4, cudaMemcpyDeviceToDevice, s), "copy path"));
    NA_CHECK(cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    *result = to_result(state, 0);
    return KGMT_OK;
}
