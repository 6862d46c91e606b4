// kgmt_iter.cuh -- device building blocks of one planning iteration: PTX
// helpers (mbarrier, bulk copy), block scans, the device-side schedule, the
// per-sample propagate steps and the propagate tile, region scores and the
// per-query finaliser.  The kernels in kgmt_kernels.cu are built from them.
#pragma once
#include <climits>
#include <cstdint>
#include <type_traits>

#include "kgmt_device.cuh"
#include "kgmt_kernels.h"

namespace kgmt {

// ---------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
    return ok != 0;
}

// bulk global -> shared copy through the TMA engine; bytes % 16 == 0, both
// addresses 16-byte aligned
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// the last-one-in count of a tile or query: a release add at GPU scope
// (everything this thread wrote, and what the block wrote before the last
// __syncthreads, is visible to whoever reads the count afterwards and
// fences) -- lighter than a full fence followed by a relaxed add
__device__ __forceinline__ uint32_t atomic_add_release(uint32_t* p, uint32_t v)
{
    uint32_t old;
    asm volatile("atom.add.release.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// programmatic dependent launch: the kernel that follows in the stream may
// be scheduled once every block of this one has called pdl_trigger (or
// exited); pdl_wait blocks until the kernel before this one has completed
// and its memory is visible (immediately when launched without the attribute)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// KGMT_CHECK_BOUNDS builds (libkgmt_checked.so) test the kernels' scattered
// indices against their buffers: a failed test records kErrBounds in
// g_bounds_error and the access is skipped -- no trap, no fault -- and the
// host reports KGMT_ERR_INTERNAL.  Other builds compile the tests away.
// (Only kgmt_kernels.cu includes this header: the word is defined once.)
#ifdef KGMT_CHECK_BOUNDS
__device__ uint32_t g_bounds_error;
__device__ __forceinline__ bool bound_ok(bool c)
{
    if(!c) atomicOr(&g_bounds_error, kErrBounds);
    return c;
}
#define KGMT_BOUND(c) bound_ok(c)
#else
#define KGMT_BOUND(c) true
#endif

__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p)
{
    return *(const volatile unsigned long long*)p;
}

__device__ __forceinline__ void st_volatile_u64(unsigned long long* p, unsigned long long v)
{
    *(volatile unsigned long long*)p = v;
}

// Tile bases of up to kBaseCache slots are copied to shared memory once per
// block, so finding a tile's query is a binary search in shared memory
// instead of ~log2(slots) dependent global loads.
constexpr int kBaseCache = 2048;

struct BaseCache {
    const uint32_t* base;  // shared copy, or the global array when too many slots
    int n;
};

__device__ __forceinline__ BaseCache cache_bases(const uint32_t* __restrict__ g, int n, uint32_t* s)
{
    if(n + 1 > kBaseCache) return {g, n};
    for(int i = threadIdx.x; i <= n; i += blockDim.x) s[i] = __ldcg(g + i);
    __syncthreads();
    return {s, n};
}

// last slot q with base[q] <= t (base is an exclusive prefix over n slots,
// base[n] = total, t < total)
__device__ __forceinline__ int find_slot(const uint32_t* __restrict__ base, int n, uint32_t t)
{
    int lo = 0, hi = n;
    while(lo < hi)
        {
            int mid = (lo + hi + 1) >> 1;
            if(base[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
    return lo;
}

// block-wide exclusive scan of one uint32 per thread; returns the exclusive
// prefix, *total the block sum.  scratch: >= 33 words of shared memory.
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* scratch, uint32_t* total)
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if(lane >= o) x += y;
        }
    if(lane == 31) scratch[warp] = x;
    __syncthreads();
    if(warp == 0)
        {
            uint32_t w = lane < NW ? scratch[lane] : 0u;
            uint32_t z = w;
#pragma unroll
            for(int o = 1; o < 32; o <<= 1)
                {
                    uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                    if(lane >= o) z += y;
                }
            if(lane < NW) scratch[lane] = z - w;
            if(lane == NW - 1) scratch[32] = z;
        }
    __syncthreads();
    uint32_t excl = scratch[warp] + x - v;
    *total = scratch[32];
    __syncthreads();
    return excl;
}

// block-wide exclusive scan of three uint32 per thread at once; returns the
// exclusive prefixes, *total the block sums.  scratch: >= 33 entries.
template <int NT>
__device__ __forceinline__ uint3 block_exclusive_scan3(uint3 v, uint3* scratch, uint3* total)
{
    constexpr int NW = NT / 32;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint3 x = v;
#pragma unroll
    for(int o = 1; o < 32; o <<= 1)
        {
            const uint32_t a = __shfl_up_sync(full, x.x, o), b = __shfl_up_sync(full, x.y, o), c = __shfl_up_sync(full, x.z, o);
            if(lane >= o) x.x += a, x.y += b, x.z += c;
        }
    if(lane == 31) scratch[warp] = x;
    __syncthreads();
    if(warp == 0)
        {
            const uint3 w = lane < NW ? scratch[lane] : make_uint3(0u, 0u, 0u);
            uint3 z = w;
#pragma unroll
            for(int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t a = __shfl_up_sync(full, z.x, o), b = __shfl_up_sync(full, z.y, o), c = __shfl_up_sync(full, z.z, o);
                    if(lane >= o) z.x += a, z.y += b, z.z += c;
                }
            if(lane < NW) scratch[lane] = make_uint3(z.x - w.x, z.y - w.y, z.z - w.z);
            if(lane == NW - 1) scratch[32] = z;
        }
    __syncthreads();
    const uint3 e = scratch[warp];
    *total = scratch[32];
    __syncthreads();
    return make_uint3(e.x + x.x - v.x, e.y + x.y - v.y, e.z + x.z - v.z);
}

// ---------------------------------------------------------------------------
// schedule of the next iteration, computed by one block (the last query to
// finalise, or the admission path): tiles per slot, prefix bases, running
// count, and this iteration's tile sizes.  All threads of the calling block
// must enter.
// ---------------------------------------------------------------------------
// TOTALS: the finalisers of this iteration accumulated the running queries'
// samples and tree sizes in Sched::next_samples / next_tree (else a first
// pass over the slots sums them)
template <int NT = kAppendThreads, bool TOTALS = false>
__device__ void compute_schedule(const QueryParams* __restrict__ P, const QueryState* __restrict__ S, Sched* sched, uint32_t* tile_a_base,
                                 uint32_t* tile_c_base, uint32_t* tile_c_old)
{
    __shared__ uint3 s_scan[33];
    const int n = (int)sched->n_slots;
    const uint32_t block = sched->prop_block;
    const uint32_t pair_samples = sched->pair_samples;
    const uint32_t sms = sched->n_sms;
    // samples per propagate tile: pairs per thread for large iterations; for
    // small ones the smallest power of two from 32 up to the block that keeps
    // the tiles within one per SM, so each tile's warps have an SM to
    // themselves (a tile's time is its slowest sample's)
    auto tile_for = [&](uint32_t total) -> uint32_t {
        if(total >= pair_samples) return kPropPer * block;
        if(sms == 0) return block;
        uint32_t t = 32u;
        while(t < block && (total + t - 1) / t > sms) t <<= 1;
        return t;
    };
    // old nodes per re-activation tile: small tiles while the old nodes of
    // all running queries fill fewer tiles than there are SMs, large ones
    // while they fill many waves of large tiles (each tile's fixed latency --
    // loads, scan, look-back -- spread over more nodes)
    auto old_tile_for = [&](uint32_t tree_total) -> uint32_t {
        if(sms != 0 && tree_total <= sms * (uint32_t)kTileOld) return (uint32_t)kTileOldSmall;
        if(sms != 0 && (unsigned long long)tree_total >= (unsigned long long)kOldLargeWaves * sms * (uint32_t)kTileOldLarge)
            return (uint32_t)kTileOldLarge;
        return (uint32_t)kTileOld;
    };
    // a slot's samples and tree size if it runs (three independent loads:
    // other blocks finalised these states in this kernel, so past L1)
    auto load = [&](int q, uint32_t& ns, uint32_t& tree) -> uint32_t {
        ns = tree = 0u;
        if(q >= n) return 0u;
        const uint32_t st = __ldcg(&S[q].status);
        const uint32_t a = __ldcg(&S[q].n_samples), b = __ldcg(&S[q].tree_size);
        if(st != KGMT_QUERY_RUNNING) return 0u;
        ns = a, tree = b;
        return 1u;
    };
    // totals only steer the tile sizes (thresholds below 2^22): clamped so
    // that no sum can wrap
    constexpr uint32_t kClamp = 1u << 22;
    auto publish = [&](uint32_t tiles_a, uint32_t tiles_c, uint32_t running, uint32_t prop_tile, uint32_t old_tile) {
        tile_a_base[n] = tiles_a;
        tile_c_base[n] = tiles_c;
        sched->tiles_a = tiles_a;
        sched->tiles_c = tiles_c;
        sched->running = running;
        sched->ticket_a = 0;
        sched->prop_tile = prop_tile;
        sched->old_tile = old_tile;
        sched->next_samples = 0ull;
        sched->next_tree = 0ull;
        if(running) sched->iterations += 1;
        if(sched->host_running) *(volatile uint32_t*)sched->host_running = running;
    };
    if(n <= 32)
        {
            // up to 32 slots: one warp, shuffle scans, no block barriers but the last
            if(threadIdx.x < 32)
                {
                    const unsigned full = 0xffffffffu;
                    const int q = (int)threadIdx.x;
                    uint32_t ns, tree;
                    const uint32_t run = load(q, ns, tree);
                    const uint32_t tot_s = __reduce_add_sync(full, ns < kClamp ? ns : kClamp);
                    const uint32_t tot_t = __reduce_add_sync(full, tree < kClamp ? tree : kClamp);
                    const uint32_t prop_tile = tile_for(tot_s), old_tile = old_tile_for(tot_t);
                    uint32_t ta = 0, tc = 0, told = 0;
                    if(run)
                        {
                            // tile sizes are powers of two
                            ta = (ns + prop_tile - 1) >> (__ffs(prop_tile) - 1);
                            told = (tree + old_tile - 1) >> (__ffs(old_tile) - 1);
                            tc = told + (ns + kTileC - 1) / kTileC;
                        }
                    uint32_t ia = ta, ic = tc, ir = run;
#pragma unroll
                    for(int o = 1; o < 32; o <<= 1)
                        {
                            const uint32_t ya = __shfl_up_sync(full, ia, o);
                            const uint32_t yc = __shfl_up_sync(full, ic, o);
                            const uint32_t yr = __shfl_up_sync(full, ir, o);
                            if(q >= o) ia += ya, ic += yc, ir += yr;
                        }
                    if(q < n)
                        {
                            tile_a_base[q] = ia - ta;
                            tile_c_base[q] = ic - tc;
                            tile_c_old[q] = told;
                        }
                    if(q == 31) publish(ia, ic, ir, prop_tile, old_tile);
                }
            __syncthreads();
            return;
        }
    // pass 1: the running queries' samples and tree sizes, for the tile sizes
    // (a block of slots or fewer keeps its loads in registers for pass 2)
    uint32_t ns0 = 0, tree0 = 0, run0 = 0;
    uint3 tot = make_uint3(0u, 0u, 0u);
    if(TOTALS)
        {
            const unsigned long long a = __ldcg(&sched->next_samples), b = __ldcg(&sched->next_tree);
            tot.x = a < kClamp ? (uint32_t)a : kClamp;
            tot.y = b < kClamp ? (uint32_t)b : kClamp;
            if(threadIdx.x < n) run0 = load((int)threadIdx.x, ns0, tree0);
        }
    else
        {
            uint3 part = make_uint3(0u, 0u, 0u);
            for(int q = threadIdx.x; q < n; q += NT)
                {
                    uint32_t ns, tree;
                    const uint32_t run = load(q, ns, tree);
                    if(q == (int)threadIdx.x) ns0 = ns, tree0 = tree, run0 = run;
                    part.x = min(part.x + min(ns, kClamp), kClamp);
                    part.y = min(part.y + min(tree, kClamp), kClamp);
                }
            block_exclusive_scan3<NT>(part, s_scan, &tot);
        }
    const uint32_t prop_tile = tile_for(tot.x), old_tile = old_tile_for(tot.y);
    const int sh_a = __ffs(prop_tile) - 1, sh_o = __ffs(old_tile) - 1;  // tile sizes are powers of two
    // pass 2: tiles per slot and their exclusive prefixes
    uint3 carry = make_uint3(0u, 0u, 0u);
    for(int base = 0; base < n; base += NT)
        {
            const int q = base + (int)threadIdx.x;
            uint32_t ns = ns0, tree = tree0, run = run0;
            if(base > 0) run = load(q, ns, tree);
            uint32_t ta = 0, tc = 0, told = 0;
            if(run)
                {
                    ta = (ns + prop_tile - 1) >> sh_a;
                    told = (tree + old_tile - 1) >> sh_o;
                    tc = told + (ns + kTileC - 1) / kTileC;
                }
            uint3 sum;
            const uint3 e = block_exclusive_scan3<NT>(make_uint3(ta, tc, run), s_scan, &sum);
            if(q < n)
                {
                    tile_a_base[q] = carry.x + e.x;
                    tile_c_base[q] = carry.y + e.y;
                    tile_c_old[q] = told;
                }
            carry.x += sum.x, carry.y += sum.y, carry.z += sum.z;
        }
    if(threadIdx.x == 0) publish(carry.x, carry.y, carry.z, prop_tile, old_tile);
    __syncthreads();
}

// frontier entries R, samples per entry and samples of the next iteration
// (KGMT.cu:183-201 with the capacity rule made safe)
__device__ __forceinline__ void plan_samples_vals(uint32_t capacity, uint32_t samples_per_node, uint32_t tree_size, uint32_t R, uint32_t* spe_out,
                                                  uint32_t* n_out)
{
    const uint32_t free_slots = capacity - tree_size;
    uint32_t spe = 0, ruse = R;
    if(R > 0)
        {
            spe = free_slots / R;
            if(spe > samples_per_node) spe = samples_per_node;
            if(spe == 0)
                {
                    spe = 1;
                    ruse = free_slots;
                }
        }
    *spe_out = spe;
    *n_out = ruse * spe;
}

__device__ __forceinline__ void plan_samples(const QueryParams& P, QueryState& st)
{
    plan_samples_vals(P.capacity, P.samples_per_node, st.tree_size, st.n_react + st.w_new, &st.spe, &st.n_samples);
}

// ---------------------------------------------------------------------------
// propagate (+ the region scores of each query, computed by the block that
// finishes the query's last propagate tile)
// ---------------------------------------------------------------------------
struct PropCtx {
    uint32_t itr, spe, n_react, n_samples;
};

constexpr int kSortBins = 32;  // step-count bins of the in-tile sort (last bin: dead lanes)

struct PropShared {
    uint32_t acc;                // accepted samples of the tile
    uint32_t steps;              // RK4 steps of the tile
    uint32_t tests;              // box tests of the tile
    uint32_t next_run;           // runs of the sorted tile handed to warps so far
};

// sample rows of a model
// SAMPLE_DIM and the number of control draws (the step draw follows them,
// then the accept draw)
template <int MODEL>
struct ModelDims {
    static constexpr int D = MODEL == KGMT_MODEL_QUADROTOR ? 17 : MODEL == KGMT_MODEL_UNICYCLE ? 7 : 10;
    static constexpr int NC = MODEL == KGMT_MODEL_QUADROTOR ? 4 : 3;
};

// model bits of the MODELS mask a propagate variant is compiled for
constexpr int kBitDI = 1, kBitQuad = 2, kBitDubins = 4, kBitUnicycle = 8, kAllModels = 15;

// calls f(std::integral_constant<int, model>) for the query's model, among
// the models the variant was compiled for (a single-model variant needs no test)
template <int MODELS, typename F>
__device__ __forceinline__ void with_model(int model, F&& f)
{
    if constexpr((MODELS & kBitDI) != 0)
        if(MODELS == kBitDI || model == KGMT_MODEL_DOUBLE_INTEGRATOR) f(std::integral_constant<int, KGMT_MODEL_DOUBLE_INTEGRATOR>{});
    if constexpr((MODELS & kBitQuad) != 0)
        if(MODELS == kBitQuad || model == KGMT_MODEL_QUADROTOR) f(std::integral_constant<int, KGMT_MODEL_QUADROTOR>{});
    if constexpr((MODELS & kBitDubins) != 0)
        if(MODELS == kBitDubins || model == KGMT_MODEL_DUBINS_AIRPLANE) f(std::integral_constant<int, KGMT_MODEL_DUBINS_AIRPLANE>{});
    if constexpr((MODELS & kBitUnicycle) != 0)
        if(MODELS == kBitUnicycle || model == KGMT_MODEL_UNICYCLE) f(std::integral_constant<int, KGMT_MODEL_UNICYCLE>{});
}

template <int MODEL>
__device__ __forceinline__ bool propagate_model(const QueryParams& p, const GridView& grid, const float* x0, const float* u, const float4* obs,
                                                uint32_t n_obs, float* x1, PropCount& cnt)
{
    if constexpr(MODEL == KGMT_MODEL_QUADROTOR) return propagate_quad(p, grid, x0, u, obs, n_obs, x1, cnt);
    else if constexpr(MODEL == KGMT_MODEL_DUBINS_AIRPLANE) return propagate_dubins(p, grid, x0, u, obs, n_obs, x1, cnt);
    else if constexpr(MODEL == KGMT_MODEL_UNICYCLE) return propagate_unicycle(p, grid, x0, u, obs, n_obs, x1, cnt);
    else return propagate_di(p, grid, x0, u, obs, n_obs, x1, cnt);
}

// rows of D floats: with D even every row starts 8-byte aligned (row
// buffers are 256-byte aligned), so they move as float2 pairs.  COHERENT:
// the row may have been written earlier in the same launch by another block
// (the persistent tail kernel), so it is read through L2 instead of the
// read-only path, which is only valid for data no one writes during the launch.
template <int D, bool COHERENT = false>
__device__ __forceinline__ void load_row_ro(const float* __restrict__ src, float* r)
{
    if constexpr(D % 2 == 0)
        {
#pragma unroll
            for(int c = 0; c < D / 2; ++c)
                {
                    const float2 v = COHERENT ? __ldcg((const float2*)src + c) : __ldg((const float2*)src + c);
                    r[2 * c] = v.x, r[2 * c + 1] = v.y;
                }
        }
    else
        {
#pragma unroll
            for(int c = 0; c < D; ++c) r[c] = COHERENT ? __ldcg(src + c) : __ldg(src + c);
        }
}

template <int D>
__device__ __forceinline__ void store_row(float* dst, const float* r)
{
    if constexpr(D % 2 == 0)
        {
#pragma unroll
            for(int c = 0; c < D / 2; ++c) ((float2*)dst)[c] = make_float2(r[2 * c], r[2 * c + 1]);
        }
    else
        {
#pragma unroll
            for(int c = 0; c < D; ++c) dst[c] = r[c];
        }
}

// A sample's eight uniforms come from two Philox blocks, (s, itr, 0, 0) and
// (s, itr, 0, 1): controls first, then the step draw, then the accept draw.
// The block holding the step draw ("key block": the first for three
// controls, the second for four) is drawn once, when the tile is sorted by
// step count, and handed to the thread that propagates the sample.
template <int MODEL>
__device__ __forceinline__ U4 sample_key_block(const QueryParams& p, const PropCtx& c, uint32_t s)
{
    const uint32_t k0 = (uint32_t)p.seed, k1 = (uint32_t)(p.seed >> 32);
    return philox4x32_10(s, c.itr, 0u, ModelDims<MODEL>::NC == 4 ? 1u : 0u, k0, k1);
}

// RK4 steps of the sample whose key block is kb, for ordering the samples of
// a tile so that a warp's lanes loop about equally long
template <int MODEL>
__device__ __forceinline__ int sample_steps(const QueryParams& p, const U4& kb)
{
    return draw_steps(p, u01(ModelDims<MODEL>::NC == 4 ? kb.x : kb.w));
}

// gather the parent row and draw the sample's uniforms (no obstacle access,
// so it runs while the tile's boxes are still in flight); kb: its key block
template <int MODEL, bool COHERENT = false>
__device__ __forceinline__ uint32_t prepare_sample(const QueryParams& p, const PropCtx& c, uint32_t s, const U4& kb, float* x0, float* u)
{
    constexpr int D = ModelDims<MODEL>::D;
    const uint32_t e = s / c.spe;
    uint32_t par = e < c.n_react ? (KGMT_BOUND(e < p.capacity) ? p.rep_old[e] : 0u)
                                 : (KGMT_BOUND(e - c.n_react < p.capacity) ? p.rep_new[e - c.n_react] : 0u);
    if(!KGMT_BOUND(par < p.capacity)) par = 0u;
    load_row_ro<D, COHERENT>(p.tree + (size_t)par * D, x0);
    const uint32_t k0 = (uint32_t)p.seed, k1 = (uint32_t)(p.seed >> 32);
    constexpr bool four = ModelDims<MODEL>::NC == 4;
    const U4 other = philox4x32_10(s, c.itr, 0u, four ? 0u : 1u, k0, k1);
    const U4& a = four ? other : kb;
    const U4& b = four ? kb : other;
    u[0] = u01(a.x), u[1] = u01(a.y), u[2] = u01(a.z), u[3] = u01(a.w);
    u[4] = u01(b.x), u[5] = u01(b.y), u[6] = u01(b.z), u[7] = u01(b.w);
    return par;
}

template <int MODEL>
__device__ __forceinline__ void finish_sample(const QueryParams& p, const GridView& grid, const float4* obs, uint32_t n_obs, uint32_t s,
                                              bool live, uint32_t par, const float* x0, const float* u, PropShared* sh)
{
    constexpr int D = ModelDims<MODEL>::D;
    constexpr int NC = ModelDims<MODEL>::NC;
    const unsigned full = 0xffffffffu;
    int r1 = -1;
    uint64_t bit = 0ull;
    PropCount cnt;
    bool ok = false, acc = false;
    if(live)
        {
            float x1[D];
            ok = propagate_model<MODEL>(p, grid, x0, u, obs, n_obs, x1, cnt);
            const CellIds cid = cell_ids(p, x1);
            r1 = cid.r1;
            bit = 1ull << cid.r2;
            if(!KGMT_BOUND((uint32_t)r1 < p.regions && s < p.capacity)) live = ok = false;
            if(ok)
                {
                    const uint64_t marks = p.marks[r1];
                    const float score = p.score[r1];
                    const bool fresh = (marks & bit) == 0ull;
                    acc = (u[NC + 1] < score) || fresh;
                }
            // only a sample that joins the tree is read again (by the append
            // kernel): its row and parent; every sample's region and accept
            // flag, in one word (region ids are below 2^31)
            if(acc)
                {
                    store_row<D>(p.us + (size_t)s * D, x1);
                    p.up[s] = (int32_t)par;
                }
            if(live) p.ur1f[s] = (uint32_t)r1 | (acc ? 0x80000000u : 0u);
        }
    // histogram updates (KGMT.cu:250-253): counter over all samples, valid
    // count and the fine-cell bit over the valid ones; one fire-and-forget L2
    // atomic per sample (aggregating a warp's equal regions first with
    // match.any cost more than it saved: the batch ran 2.5 % slower); tile
    // totals in shared memory
    if(live) atomicAdd(&p.counter[r1], 1);
    if(ok)
        {
            atomicAdd(&p.valid[r1], 1);
            atomicOr((unsigned long long*)&p.newmarks[r1], (unsigned long long)bit);
        }
    const unsigned acc_mask = __ballot_sync(full, acc);
    const unsigned warp_steps = __reduce_add_sync(full, (unsigned)cnt.steps);
    const unsigned warp_tests = __reduce_add_sync(full, cnt.tests);
    if((threadIdx.x & 31) == 0)
        {
            if(acc_mask) atomicAdd(&sh->acc, (unsigned)__popc(acc_mask));
            if(warp_steps) atomicAdd(&sh->steps, warp_steps);
            if(warp_tests) atomicAdd(&sh->tests, warp_tests);
        }
}

// One propagate tile of `tile` samples of one query: tile <= NT (a power of
// two) gives thread i < tile sample lt * tile + i; tile = kPropPer x NT gives
// thread i samples (2 lt + h) * NT + i, h = 0, 1.  A counting sort of the tile
// by step count (dead lanes last), then the sorted tile in runs of 32
// consecutive samples, one sample a lane: a warp takes the longest run left
// whenever it is free (a shared counter), so the warps of a block finish the
// tile together however early their samples end.  `wait` runs once per
// thread, after its first run has gathered its parents and draws (the boxes'
// bulk copy may be in flight until then).  Block-uniform call.  COHERENT:
// parent rows may have been appended by other blocks earlier in the same
// launch (see load_row_ro).
template <int NT, int MODELS, bool COHERENT = false, typename Wait>
__device__ __forceinline__ void propagate_tile(const QueryParams& sp, const PropCtx& sc, uint32_t lt, uint32_t tile, uint32_t smem_boxes, PropShared* sh,
                                               uint32_t* s_hist, uint32_t* s_perm, uint4* s_key, const float4* s_obs, const uint16_t* s_gstart,
                                               const uint16_t* s_gitems, const uint32_t* s_gmeta, Wait&& wait)
{
    const int model = sp.model;
    const int per = tile > (uint32_t)NT ? kPropPer : 1;
    {
        uint32_t s0[kPropPer], rank[kPropPer];
        int key[kPropPer];
        U4 kb[kPropPer];
        if(threadIdx.x < kSortBins) s_hist[threadIdx.x] = 0;
#pragma unroll
        for(int h = 0; h < kPropPer; ++h)
            {
                // with one sample per thread the second key is a dead lane
                if(per == kPropPer) s0[h] = (lt * kPropPer + h) * NT + threadIdx.x;
                else s0[h] = (h == 0 && threadIdx.x < tile) ? lt * tile + threadIdx.x : 0xFFFFFFFFu;
                key[h] = kSortBins - 1;
                kb[h] = U4{0u, 0u, 0u, 0u};
                if(s0[h] < sc.n_samples)
                    {
                        int k = 1;
                        with_model<MODELS>(model, [&](auto m) {
                            kb[h] = sample_key_block<decltype(m)::value>(sp, sc, s0[h]);
                            k = sample_steps<decltype(m)::value>(sp, kb[h]);
                        });
                        key[h] = k < kSortBins - 1 ? k : kSortBins - 2;
                    }
            }
        __syncthreads();
#pragma unroll
        for(int h = 0; h < kPropPer; ++h) rank[h] = atomicAdd(&s_hist[key[h]], 1u);
        __syncthreads();
        if(threadIdx.x < 32)
            {
                // exclusive scan of the bins (kSortBins <= 32)
                const uint32_t v = threadIdx.x < kSortBins ? s_hist[threadIdx.x] : 0u;
                uint32_t x = v;
#pragma unroll
                for(int o = 1; o < 32; o <<= 1)
                    {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                        if(threadIdx.x >= (unsigned)o) x += y;
                    }
                if(threadIdx.x < kSortBins) s_hist[threadIdx.x] = x - v;
            }
        __syncthreads();
#pragma unroll
        for(int h = 0; h < kPropPer; ++h)
            {
                const uint32_t pos = s_hist[key[h]] + rank[h];
                s_perm[pos] = s0[h];
                s_key[pos] = make_uint4(kb[h].x, kb[h].y, kb[h].z, kb[h].w);
            }
        __syncthreads();
    }
    const float4* obs = sp.n_obstacles <= smem_boxes ? s_obs : sp.obstacles;
    // live samples come first in the sorted order: the dead bin's start
    const uint32_t n_live = s_hist[kSortBins - 1];
    const uint32_t n_runs = (n_live + 31u) / 32u;
    const unsigned full = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31u;
    bool waited = false;
    for(;;)
        {
            uint32_t run = 0;
            if(lane == 0) run = atomicAdd(&sh->next_run, 1u);
            run = __shfl_sync(full, run, 0);
            if(run >= n_runs) break;
            // longest runs first
            const uint32_t slot = (n_runs - 1u - run) * 32u + lane;
            const uint32_t s = slot < n_live ? s_perm[slot] : 0xFFFFFFFFu;
            const bool live = s < sc.n_samples;
            float x0[KGMT_MAX_SAMPLE_DIM], u[8];
            uint32_t par = 0;
            if(live)
                {
                    const uint4 k4 = s_key[slot];
                    const U4 kb1{k4.x, k4.y, k4.z, k4.w};
                    with_model<MODELS>(model, [&](auto m) { par = prepare_sample<decltype(m)::value, COHERENT>(sp, sc, s, kb1, x0, u); });
                }
            if(!waited)
                {
                    wait();
                    waited = true;
                }
            const GridView grid{(sp.grid_meta != nullptr && s_gmeta[1] == 1u) ? s_gstart : nullptr, s_gitems, sp.grid_items};
            with_model<MODELS>(model, [&](auto m) { finish_sample<decltype(m)::value>(sp, grid, obs, sp.n_obstacles, s, live, par, x0, u, sh); });
        }
    // a thread that got no run still follows the copy's phase
    if(!waited) wait();
}

// Samples [s0, s0 + n) of one query, one per thread (n <= NT), in index
// order -- no sort: with one such range per block the time of a launch is its
// slowest warp's, which ordering the samples inside a block cannot shorten.
// Parent rows are read coherently (they may have been appended by other
// blocks in the same launch).  `wait` runs once, after the parents and draws
// are gathered.  Block-uniform call.
template <int NT, int MODELS, typename Wait>
__device__ __forceinline__ void propagate_range(const QueryParams& sp, const PropCtx& sc, uint32_t s0, uint32_t n, uint32_t smem_boxes,
                                                PropShared* sh, const float4* s_obs, const uint16_t* s_gstart, const uint16_t* s_gitems,
                                                const uint32_t* s_gmeta, Wait&& wait)
{
    const int model = sp.model;
    const uint32_t s = s0 + threadIdx.x;
    const bool live = threadIdx.x < n && s < sc.n_samples;
    float x0[KGMT_MAX_SAMPLE_DIM], u[8];
    uint32_t par = 0;
    if(live)
        with_model<MODELS>(model, [&](auto m) {
            const U4 kb = sample_key_block<decltype(m)::value>(sp, sc, s);
            par = prepare_sample<decltype(m)::value, true>(sp, sc, s, kb, x0, u);
        });
    wait();
    const float4* obs = sp.n_obstacles <= smem_boxes ? s_obs : sp.obstacles;
    const GridView grid{(sp.grid_meta != nullptr && s_gmeta[1] == 1u) ? s_gstart : nullptr, s_gitems, sp.grid_items};
    with_model<MODELS>(model, [&](auto m) { finish_sample<decltype(m)::value>(sp, grid, obs, sp.n_obstacles, s, live, par, x0, u, sh); });
}

// Graph::updateVertices (Graph.cu:311-358) for one query, by one block: all
// regions scored, lane l of kScoreLanes sums regions l, l+256, ... in order,
// then a halving tree over the lanes.  Histograms and marks were updated by
// other blocks' atomics in this kernel: read past L1.
// The fields of QueryParams the scores use, held in registers.
struct ScoreParams
{
    int32_t* counter;
    int32_t* valid;
    float* score;
    uint64_t* marks;
    uint64_t* newmarks;
    uint32_t regions, fine_cells;
    float epsilon, cell_volume;
};

template <int NT>
__device__ void update_scores(const ScoreParams& p, QueryState& st, float* lanes)
{
    const float F = (float)p.fine_cells;
    constexpr int U = 4;  // regions whose loads are issued together
    // the thread's first U regions keep their raw score in registers for the
    // normalisation pass (no re-read of what it just wrote)
    float kept[U];
    for(int l = threadIdx.x; l < kScoreLanes; l += NT)
        {
            float acc = 0.0f;
            for(uint32_t r0 = (uint32_t)l; r0 < p.regions; r0 += U * kScoreLanes)
                {
                    const bool first = l == (int)threadIdx.x && r0 == (uint32_t)l;
                    uint64_t m[U];
                    int32_t nv[U], n[U];
#pragma unroll
                    for(int k = 0; k < U; ++k)
                        {
                            const uint32_t r = r0 + k * kScoreLanes;
                            if(r < p.regions)
                                {
                                    m[k] = __ldcg(&p.marks[r]) | __ldcg(&p.newmarks[r]);
                                    nv[k] = __ldcg(&p.valid[r]);
                                    n[k] = __ldcg(&p.counter[r]);
                                }
                        }
                    // regions in increasing order: the lane's sum keeps its fixed order
#pragma unroll
                    for(int k = 0; k < U; ++k)
                        {
                            const uint32_t r = r0 + k * kScoreLanes;
                            if(r >= p.regions) break;
                            p.marks[r] = m[k];
                            p.newmarks[r] = 0ull;
                            float raw = 0.0f;    // adds nothing to the total
                            float keep = -1.0f;  // marks "no valid sample" for the normalisation pass
                            if(nv[k] > 0)
                                {
                                    const float cov = (float)__popcll(m[k]) / F;
                                    const float a = p.epsilon + (float)nv[k];
                                    const float b = a + (float)(n[k] - nv[k]);
                                    const float fv = (a / b) * p.cell_volume;
                                    const float f2 = fv * fv;
                                    const float f4 = f2 * f2;
                                    const float nf = (float)n[k];
                                    const float den = (1.0f + cov) * (1.0f + nf * nf);
                                    raw = f4 / den;
                                    keep = raw;
                                }
                            p.score[r] = keep;
                            if(first) kept[k] = keep;
                            acc = acc + raw;
                        }
                }
            lanes[l] = acc;
        }
    __syncthreads();
    static_assert(kScoreLanes >= 64, "the last five halving levels run in one warp");
    for(int stride = kScoreLanes / 2; stride >= 32; stride >>= 1)
        {
            for(int l = threadIdx.x; l < stride; l += NT) lanes[l] = lanes[l] + lanes[l + stride];
            __syncthreads();
        }
    if(threadIdx.x < 32)
        {
            // strides 16 .. 1 in registers: lane l < stride adds lane l + stride,
            // the same additions in the same order as the levels above
            float v = lanes[threadIdx.x];
#pragma unroll
            for(int stride = 16; stride >= 1; stride >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, stride);
            if(threadIdx.x == 0) lanes[0] = v;
        }
    __syncthreads();
    const float total = lanes[0];
    // raw score (-1 for regions without valid samples) -> normalised score;
    // past the registers each lane re-reads only what it wrote itself
    auto norm = [&](float raw) { return raw < 0.0f ? 1.0f : (total > 0.0f ? p.epsilon + raw / total : p.epsilon); };
    for(int l = threadIdx.x; l < kScoreLanes; l += NT)
        {
            uint32_t r = (uint32_t)l;
            if(l == (int)threadIdx.x)
                {
#pragma unroll
                    for(int k = 0; k < U; ++k, r += kScoreLanes)
                        if(r < p.regions) p.score[r] = norm(kept[k]);
                }
            for(; r < p.regions; r += kScoreLanes) p.score[r] = norm(p.score[r]);
        }
    if(threadIdx.x == 0) st.score_total = total;
}

// MODELS: bit 0 double integrator present, bit 1 quadrotor present; the
// launch picks the variant for the admitted mix, so a single-model batch
// pays for one model's registers only
// ---------------------------------------------------------------------------
// append / re-activation / frontier build
// ---------------------------------------------------------------------------
__device__ inline void finalize_query(const QueryParams& p, QueryState& st, Sched* sched)
{
    // runs on one thread.  Every input is loaded in one round (the totals
    // were accumulated by other blocks' atomics, so past L1), then the new
    // state is computed in registers and stored.
    const uint32_t acc_total = __ldcg(&st.acc_total), n_next = __ldcg(&st.n_next);
    const int32_t goal_cand = __ldcg(&st.goal_cand);
    const uint32_t react_total = __ldcg(&st.react_total), w_total = __ldcg(&st.w_total);
    const uint32_t tree0 = __ldcg(&st.tree_size), drawn = __ldcg(&st.samples_drawn), ns = __ldcg(&st.n_samples);
    const uint32_t itr = __ldcg(&st.itr);
    const uint32_t max_it = p.max_iterations, cap = p.capacity, spn = p.samples_per_node;
    if(acc_total != n_next) atomicOr(&sched->error, kErrAppendMismatch);
    const uint32_t tree = tree0 + acc_total;
    uint32_t status = KGMT_QUERY_RUNNING;
    if(goal_cand != INT_MAX) status = KGMT_QUERY_SUCCESS;
    else if(itr >= max_it) status = KGMT_QUERY_ITER_LIMIT;
    else if(tree >= cap) status = KGMT_QUERY_CAPACITY;
    st.tree_size = tree;
    st.samples_drawn = drawn + ns;
    // the next frontier's list lengths (kept for a finished query too: the
    // traced plan reports its last frontier)
    st.n_react = react_total;
    st.w_new = w_total;
    // per-iteration accumulators start from zero next iteration
    st.tiles_done = 0;
    st.prop_done = 0;
    st.react_total = 0;
    st.acc_total = 0;
    st.w_total = 0;
    st.goal_cand = INT_MAX;
    if(status != KGMT_QUERY_RUNNING)
        {
            st.status = status;
            if(status == KGMT_QUERY_SUCCESS) st.goal_index = goal_cand;
            st.t_end = globaltimer();
            return;
        }
    st.itr = itr + 1;
    st.n_next = 0;
    uint32_t spe, n_samples;
    plan_samples_vals(cap, spn, tree, react_total + w_total, &spe, &n_samples);
    st.spe = spe;
    st.n_samples = n_samples;
    // the next schedule's totals (it sizes the tiles from them)
    atomicAdd(&sched->next_samples, (unsigned long long)n_samples);
    atomicAdd(&sched->next_tree, (unsigned long long)tree);
}

// Copies one sample row (written by the propagate kernel, read-only here)
// into the tree and returns its goal distance.  The row is read into
// registers before the first store: the two buffers might alias as far as
// the compiler can tell, so interleaved loads would each wait for the
// previous store's turn.
template <int D, bool COHERENT = false>
__device__ __forceinline__ float append_row_d(const QueryParams& p, const float* src, float* dst)
{
    float r[D];
    load_row_ro<D, COHERENT>(src, r);
    store_row<D>(dst, r);
    return goal_distance(p, r);
}

template <bool COHERENT = false>
__device__ __forceinline__ float append_row(const QueryParams& p, const float* src, float* dst, int D)
{
    switch(D)
        {
            case 7: return append_row_d<7, COHERENT>(p, src, dst);
            case 17: return append_row_d<17, COHERENT>(p, src, dst);
            default: return append_row_d<10, COHERENT>(p, src, dst);
        }
}

// KGMT.cu:387-388
__device__ __forceinline__ float f_accept_vals(const QueryParams& p, uint32_t tree_size, uint32_t n_next, uint32_t itr)
{
    const float ta = 1.0f - (float)(tree_size + n_next) / (float)p.capacity;
    const float ie = (float)itr * p.epsilon;
    const double t = (double)ta;
    const double t5 = ((t * t) * (t * t)) * t;
    return (float)((double)ie * t5);
}

__device__ __forceinline__ float f_accept_of(const QueryParams& p, const QueryState& st)
{
    return f_accept_vals(p, st.tree_size, st.n_next, st.itr);
}


}  // namespace kgmt
