// kgmt_kernels.cu -- the per-iteration kernel chain of the KGMT planning loop.
//
// One iteration of every running query (reference: KGMT::plan loop body,
// src/planners/KGMT.cu:84-95) is two launches with fixed shapes, so the
// chain can be captured once in a CUDA graph and replayed:
//
//   k_propagate  KGMT::propagateFrontier + propagateFrontier_kernel1/2
//                (KGMT.cu:167-299): one thread per sample, persistent blocks
//                taking propagate tiles from a ticket counter, obstacles of
//                the tile's query staged in shared memory by a bulk (TMA)
//                copy, warp-aggregated atomics into the region histograms.
//                The block that finishes a query's last propagate tile
//                then runs Graph::updateVertices (Graph.cu:207-358) for that
//                query: region scores summed in a fixed order.
//   k_append     KGMT::updateFrontier + updateFrontier_kernel
//                (KGMT.cu:305-403) and the next iteration's frontier
//                compaction / repeat expansion (KGMT.cu:167-181,
//                Planner.cu:52-79): ordered stream compaction with
//                decoupled look-back gives every accepted sample its tree
//                index (an order-preserving "atomic append") and every
//                re-activated node its frontier slot; the last tile of a
//                query finalises it, the last query computes the schedule of
//                the next iteration on the device.
//
// Frontier representation: instead of frontier flags over the whole tree and
// two scans per iteration (KGMT.cu:170-181), the frontier of the next
// iteration is built directly as two index lists -- re-activated old nodes
// (repeat 1) followed by the nodes appended this iteration (repeat 15 or 1) --
// which is the order the reference's scan over node indices produces.
#include <cstdint>
#include <climits>
#include <type_traits>

#include "kgmt_iter.cuh"
#include "kgmt_tail.cuh"

namespace kgmt {

// ---------------------------------------------------------------------------
// decoupled look-back over one chain of tiles of one query.  Word layout:
// bits 62-63 status (0 empty, 1 aggregate, 2 inclusive prefix), bits 0-61 the
// value (the chains pack their counts so that sums never carry into the
// status bits).  Tiles are taken in ticket order, so every predecessor is
// held by a resident block; waits are bounded all the same.
// ---------------------------------------------------------------------------
constexpr unsigned long long kStAgg = 1ull << 62;
constexpr unsigned long long kStIncl = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

// Called by one full warp; lane i inspects predecessor lt-1-i, 32 at a time,
// until the nearest inclusive prefix; every nearer predecessor must have
// published at least its aggregate.  Returns the exclusive prefix on all lanes.
// After `limit` polls without progress it records kErrLookbackTimeout in
// *error and returns (the host reports KGMT_ERR_TIMEOUT).
__device__ unsigned long long lookback_warp(unsigned long long* tiles, int lt, uint32_t* error, uint32_t limit = kSpinLimit)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned long long prefix = 0;
    int base = lt - 1;
    uint32_t spins = 0;
    while(base >= 0)
        {
            const int j = base - lane;
            const unsigned long long w = j >= 0 ? ld_volatile_u64(&tiles[j]) : kStIncl;  // before tile 0: inclusive 0
            const unsigned st = (unsigned)(w >> 62);
            const unsigned incl = __ballot_sync(full, st == 2u);
            const unsigned not_ready = __ballot_sync(full, st == 0u);
            const int stop = incl ? __ffs(incl) - 1 : 31;  // nearest inclusive lane (or the whole window)
            const unsigned upto = stop == 31 ? full : ((2u << stop) - 1u);
            if(not_ready & upto)
                {
                    if(++spins > limit)
                        {
                            if(lane == 0) atomicOr(error, kErrLookbackTimeout);
                            return prefix;
                        }
                    __nanosleep(32);
                    continue;
                }
            unsigned long long v = lane <= stop ? (w & kValMask) : 0ull;
#pragma unroll
            for(int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(full, v, o);
            prefix += v;
            if(incl) break;
            base -= 32;
        }
    return prefix;
}

// Tile lt of a chain with block aggregate `agg`: publishes the aggregate,
// resolves the exclusive prefix (warp 0), publishes the inclusive prefix and
// leaves the exclusive prefix in *s_prefix.  Block-uniform call; the caller
// synchronises before reading *s_prefix.
__device__ __forceinline__ void publish_and_lookback(unsigned long long* tiles, uint32_t lt, unsigned long long agg,
                                                     unsigned long long* s_prefix, uint32_t* error)
{
    if(threadIdx.x >= 32) return;
    if(lt == 0)
        {
            if(threadIdx.x == 0)
                {
                    st_volatile_u64(&tiles[0], kStIncl | agg);
                    *s_prefix = 0;
                }
            return;
        }
    if(threadIdx.x == 0) st_volatile_u64(&tiles[lt], kStAgg | agg);
    __syncwarp();
    const unsigned long long prefix = lookback_warp(tiles, (int)lt, error);
    if(threadIdx.x == 0)
        {
            st_volatile_u64(&tiles[lt], kStIncl | (prefix + agg));
            *s_prefix = prefix;
        }
}

// Failure-detection self-test: the look-back wait of tile 1 of a chain whose
// tile 0 never publishes (a word nothing sets), with a short poll limit; it
// must give up, record the timeout and return.  One warp.
__global__ void k_selftest_wait(unsigned long long* tiles, uint32_t* error, uint32_t polls)
{
    lookback_warp(tiles, 1, error, polls);
}

uint32_t bounds_error_take()
{
#ifdef KGMT_CHECK_BOUNDS
    uint32_t v = 0, z = 0;
    if(cudaMemcpyFromSymbol(&v, g_bounds_error, sizeof(v)) != cudaSuccess) return kErrBounds;
    cudaMemcpyToSymbol(g_bounds_error, &z, sizeof(z));
    return v;
#else
    return 0u;
#endif
}

cudaError_t launch_selftest_wait(unsigned long long* tiles, uint32_t* error, uint32_t polls, cudaStream_t s)
{
    k_selftest_wait<<<1, 32, 0, s>>>(tiles, error, polls);
    return cudaGetLastError();
}

// rows of 2W floats (min corner, max corner; W = 3, or 2 for the planar
// model, whose z extents are then 0 and never tested) -> float4 pairs
__device__ __forceinline__ void stage_box(const float* r, int w, float4* dst)
{
    if(w == 2)
        {
            dst[0] = make_float4(r[0], r[1], 0.0f, 0.0f);
            dst[1] = make_float4(r[2], r[3], 0.0f, 0.0f);
        }
    else
        {
            dst[0] = make_float4(r[0], r[1], r[2], 0.0f);
            dst[1] = make_float4(r[3], r[4], r[5], 0.0f);
        }
}

// ---------------------------------------------------------------------------
// admission: root node, cleared region tables, first frontier (root x5); the
// slots are [first, first + count), or slots[0 .. count) when a list is given
// ---------------------------------------------------------------------------
__global__ void k_admit(const QueryParams* __restrict__ P, QueryState* S, uint32_t first, uint32_t count, const uint32_t* __restrict__ slots)
{
    if(blockIdx.x >= count) return;
    const uint32_t q = slots ? slots[blockIdx.x] : first + blockIdx.x;
    const QueryParams& p = P[q];
    if(p.raw_obstacles)
        for(uint32_t o = threadIdx.x; o < p.n_obstacles; o += blockDim.x)
            stage_box(p.raw_obstacles + (size_t)o * 2 * p.raw_w, p.raw_w, p.obstacles + 2 * o);
    for(uint32_t r = threadIdx.x; r < p.regions; r += blockDim.x)
        {
            p.counter[r] = 0;
            p.valid[r] = 0;
            p.score[r] = 0.0f;
            p.marks[r] = 0ull;
            p.newmarks[r] = 0ull;
        }
    for(uint32_t i = threadIdx.x; i < p.tiles_per_chain; i += blockDim.x)
        {
            p.tiles_old[i] = 0ull;
            p.tiles_slot[i] = 0ull;
        }
    for(uint32_t j = threadIdx.x; j < p.sample_dim; j += blockDim.x) p.tree[j] = p.init[j];
    if(threadIdx.x < kRootRepeat) p.rep_new[threadIdx.x] = 0u;
    if(threadIdx.x == 0)
        {
            p.parent[0] = -1;
            p.cost[0] = 0.0f;
            p.node_r1[0] = region_of(p, p.init);
            QueryState st = {};
            st.status = KGMT_QUERY_RUNNING;
            st.itr = 1;
            st.tree_size = 1;
            st.n_react = 0;
            st.w_new = kRootRepeat;
            st.goal_cand = INT_MAX;
            st.goal_index = -1;
            st.steps = 0;
            st.tests = 0;
            st.t_start = globaltimer();
            plan_samples(p, st);
            S[q] = st;
        }
}

// ---------------------------------------------------------------------------
// obstacle grid of one query per block: count boxes per cell, scan, fill.
// A box is listed in every cell of [cell(min), cell(max)] per axis (ordered,
// so an inverted box is still covered).  NaN coordinates, more boxes than
// 16-bit indices hold, or more entries than the budget leave the grid marked
// unusable and the propagate kernel tests every box.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_build_grid(const QueryParams* __restrict__ P, uint32_t first, uint32_t count,
                                                    const uint32_t* __restrict__ slots)
{
    __shared__ uint32_t cnt[kGridCells];
    __shared__ uint32_t scratch[34];
    __shared__ int s_bad;
    if(blockIdx.x >= count) return;
    const QueryParams& p = P[slots ? slots[blockIdx.x] : first + blockIdx.x];
    if(p.grid_start == nullptr) return;
    const uint32_t n = p.n_obstacles;
    for(uint32_t i = threadIdx.x; i < kGridCells; i += blockDim.x) cnt[i] = 0;
    if(threadIdx.x == 0) s_bad = n > kMaxObstacles ? 1 : 0;
    __syncthreads();
    const int G = (int)p.grid_dim;
    for(uint32_t o = threadIdx.x; o < n && !s_bad; o += blockDim.x)
        {
            const float4 a = p.obstacles[2 * o], b = p.obstacles[2 * o + 1];
            if(isnan(a.x) || isnan(a.y) || isnan(a.z) || isnan(b.x) || isnan(b.y) || isnan(b.z))
                {
                    s_bad = 1;
                    break;
                }
            const int x0 = grid_cell(p, fminf(a.x, b.x)), x1 = grid_cell(p, fmaxf(a.x, b.x));
            const int y0 = grid_cell(p, fminf(a.y, b.y)), y1 = grid_cell(p, fmaxf(a.y, b.y));
            const int z0 = p.planar ? 0 : grid_cell(p, fminf(a.z, b.z)), z1 = p.planar ? 0 : grid_cell(p, fmaxf(a.z, b.z));
            for(int cx = x0; cx <= x1; ++cx)
                for(int cy = y0; cy <= y1; ++cy)
                    for(int cz = z0; cz <= z1; ++cz) atomicAdd(&cnt[(cx * G + cy) * G + cz], 1u);
        }
    __syncthreads();
    // exclusive scan: thread t owns cells [16 t, 16 t + 16)
    constexpr int PER = kGridCells / 256;
    uint32_t local = 0;
    if(threadIdx.x < 256)
        for(int i = 0; i < PER; ++i) local += cnt[threadIdx.x * PER + i];
    uint32_t total;
    uint32_t run = block_exclusive_scan<256>(local, scratch, &total);
    for(int i = 0; i < PER; ++i)
        {
            const uint32_t c = threadIdx.x * PER + i;
            const uint32_t k = cnt[c];
            p.grid_start[c] = (uint16_t)run;  // meaningful only when usable (total <= 65535)
            cnt[c] = run;  // becomes the fill cursor
            run += k;
        }
    const bool usable = !s_bad && total <= p.grid_budget && total <= kMaxGridItems;
    if(threadIdx.x == 0)
        {
            p.grid_start[kGridCells] = (uint16_t)total;
            p.grid_meta[0] = total;
            p.grid_meta[1] = usable ? 1u : 0u;
        }
    __syncthreads();
    if(!usable) return;
    for(uint32_t o = threadIdx.x; o < n; o += blockDim.x)
        {
            const float4 a = p.obstacles[2 * o], b = p.obstacles[2 * o + 1];
            const int x0 = grid_cell(p, fminf(a.x, b.x)), x1 = grid_cell(p, fmaxf(a.x, b.x));
            const int y0 = grid_cell(p, fminf(a.y, b.y)), y1 = grid_cell(p, fmaxf(a.y, b.y));
            const int z0 = p.planar ? 0 : grid_cell(p, fminf(a.z, b.z)), z1 = p.planar ? 0 : grid_cell(p, fmaxf(a.z, b.z));
            for(int cx = x0; cx <= x1; ++cx)
                for(int cy = y0; cy <= y1; ++cy)
                    for(int cz = z0; cz <= z1; ++cz)
                        {
                            const uint32_t pos = atomicAdd(&cnt[(cx * G + cy) * G + cz], 1u);
                            p.grid_items[pos] = (uint16_t)o;
                        }
        }
}

__global__ void k_schedule(const QueryParams* __restrict__ P, const QueryState* __restrict__ S, Sched* sched, uint32_t* tile_a_base,
                           uint32_t* tile_c_base, uint32_t* tile_c_old)
{
    compute_schedule(P, S, sched, tile_a_base, tile_c_base, tile_c_old);
}

template <int NT, int MODELS>
__global__ void __launch_bounds__(NT, (MODELS == kBitDI ? 1024 : 512) / NT) k_propagate(const QueryParams* __restrict__ P, QueryState* S, Sched* sched,
                                                  const uint32_t* __restrict__ tile_base, uint32_t smem_boxes)
{
    // dynamic shared memory: grid starts | grid items | grid meta | boxes
    // (smem_boxes of them; a query with more reads its boxes from global memory)
    extern __shared__ float4 s_dyn[];
    uint16_t* s_gstart = (uint16_t*)s_dyn;
    uint16_t* s_gitems = (uint16_t*)((char*)s_dyn + kSmemStartBytes);
    uint32_t* s_gmeta = (uint32_t*)((char*)s_dyn + kSmemStartBytes + kSmemItemBytes);
    float4* s_obs = (float4*)((char*)s_dyn + kSmemGridBytes);
    __shared__ uint32_t s_copy;
    __shared__ alignas(8) uint64_t bar;
    __shared__ QueryParams s_p;
    __shared__ PropCtx s_c;
    __shared__ PropShared s_sh;
    __shared__ float s_lanes[kScoreLanes];
    __shared__ uint32_t s_base[kBaseCache];
    __shared__ uint32_t s_hist[kSortBins];
    __shared__ uint32_t s_perm[kPropPer * NT];
    __shared__ uint4 s_key[kPropPer * NT];  // key Philox block of each sorted sample
    __shared__ int s_tile, s_q, s_last;
    // everything here depends on the append kernel before this one (its
    // schedule, frontier and tree); once that is complete the append kernel
    // after this one may be scheduled into the SMs this launch leaves free
    pdl_wait();
    pdl_trigger();
    if(blockIdx.x == 0 && threadIdx.x == 0)
        {
            // counters of the append kernel that follows this one
            sched->ticket_c = 0;
            sched->finalized = 0;
        }
    const uint32_t total = sched->tiles_a;
    const int n_slots = (int)sched->n_slots;
    // samples per tile this iteration (the schedule sized the tiles)
    const uint32_t tile = sched->prop_tile;
    if(blockIdx.x >= total) return;
    if(threadIdx.x == 0)
        {
            mbar_init(&bar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    const BaseCache bases = cache_bases(tile_base, n_slots, s_base);
    int cur_q = -1;
    uint32_t phase = 0;
    uint32_t t = blockIdx.x;  // first tile static, then tickets
    uint32_t t_next = 0;      // ticket taken while the current tile runs (thread 0)
    for(;;)
        {
            if(threadIdx.x == 0)
                {
                    s_tile = (int)t;
                    s_q = t < total ? find_slot(bases.base, bases.n, t) : -1;
                    s_sh.acc = 0, s_sh.steps = 0, s_sh.tests = 0, s_sh.next_run = 0;
                    s_last = 0;
                    if(t < total) t_next = gridDim.x + atomicAdd(&sched->ticket_a, 1u);
                }
            __syncthreads();
            t = (uint32_t)s_tile;
            if(t >= total) break;
            const int q = s_q;
            bool wait_obs = false;
            if(q != cur_q)
                {
                    // stage the query's parameters; its boxes go by bulk copy
                    const uint32_t* src = (const uint32_t*)&P[q];
                    uint32_t* dst = (uint32_t*)&s_p;
                    for(int i = threadIdx.x; i < (int)(sizeof(QueryParams) / 4); i += NT) dst[i] = src[i];
                    if(threadIdx.x == 0)
                        {
                            const QueryState& st = S[q];
                            s_c.itr = st.itr;
                            s_c.spe = st.spe;
                            s_c.n_react = st.n_react;
                            s_c.n_samples = st.n_samples;
                            // boxes, grid meta, grid starts and the first grid
                            // items: one mbarrier transaction of bulk copies
                            const QueryParams& gp = P[q];
                            const uint32_t n_obs = gp.n_obstacles;
                            const bool obs_s = n_obs > 0 && n_obs <= smem_boxes;
                            const bool grid = gp.grid_meta != nullptr;
                            const uint32_t bytes = (obs_s ? n_obs * 32u : 0u) + (grid ? 16u + kSmemStartBytes + kSmemItemBytes : 0u);
                            s_copy = bytes;
                            if(bytes)
                                {
                                    fence_proxy_async_smem();
                                    mbar_expect_tx(&bar, bytes);
                                    if(obs_s) bulk_copy_g2s(s_obs, gp.obstacles, n_obs * 32u, &bar);
                                    if(grid)
                                        {
                                            bulk_copy_g2s(s_gmeta, gp.grid_meta, 16u, &bar);
                                            bulk_copy_g2s(s_gstart, gp.grid_start, kSmemStartBytes, &bar);
                                            bulk_copy_g2s(s_gitems, gp.grid_items, kSmemItemBytes, &bar);
                                        }
                                }
                        }
                    __syncthreads();
                    wait_obs = s_copy != 0;
                    cur_q = q;
                }
            const uint32_t lt = t - bases.base[q];
            propagate_tile<NT, MODELS>(s_p, s_c, lt, tile, smem_boxes, &s_sh, s_hist, s_perm, s_key, s_obs, s_gstart, s_gitems, s_gmeta, [&] {
                if(!wait_obs) return;
                uint32_t spins = 0;
                while(!mbar_try_wait(&bar, phase))
                    if(++spins > kSpinLimit)
                        {
                            if(threadIdx.x == 0) atomicOr(&sched->error, kErrCopyTimeout);
                            break;
                        }
                phase ^= 1u;
            });
            __syncthreads();
            if(threadIdx.x == 0)
                {
                    QueryState& st = S[q];
                    if(s_sh.acc) atomicAdd(&st.n_next, s_sh.acc);
                    if(s_sh.steps) atomicAdd(&st.steps, (unsigned long long)s_sh.steps);
                    if(s_sh.tests) atomicAdd(&st.tests, (unsigned long long)s_sh.tests);
                    const uint32_t n_tiles = bases.base[q + 1] - bases.base[q];
                    if(atomic_add_release(&st.prop_done, 1u) == n_tiles - 1) s_last = 1;
                    t = t_next;
                    s_tile = (int)t;
                }
            __syncthreads();
            if(s_last)
                {
                    __threadfence();
                    const ScoreParams sp{s_p.counter, s_p.valid, s_p.score, s_p.marks, s_p.newmarks, s_p.regions, s_p.fine_cells, s_p.epsilon, s_p.cell_volume};
                    update_scores<NT>(sp, S[q], s_lanes);
                }
            t = (uint32_t)s_tile;
            __syncthreads();
        }
}

// eight blocks per SM (32 registers; the kernel waits on loads, scans and
// look-back, so more tiles in flight hide more latency: the mixed batch
// +4 %, the double-integrator batch unchanged)
__global__ void __launch_bounds__(kAppendThreads, 8) k_append(const QueryParams* __restrict__ P, QueryState* S, Sched* sched,
                                                           uint32_t* tile_a_base, uint32_t* tile_c_base, uint32_t* tile_c_old)
{
    __shared__ uint32_t scratch[34];
    __shared__ int s_tile, s_q, s_glob, s_fin;
    __shared__ unsigned long long s_prefix;
    __shared__ float s_fa;
    __shared__ uint32_t s_cbase[kBaseCache];
    __shared__ uint32_t s_cold[kBaseCache];
    const uint32_t total = sched->tiles_c;
    const int n_slots = (int)sched->n_slots;
    const uint32_t old_tile = sched->old_tile;
    if(blockIdx.x >= total) return;
    // this iteration's tile bases (the schedule rewrites the global arrays only
    // after every tile is done)
    const BaseCache cbase = cache_bases(tile_c_base, n_slots, s_cbase);
    const BaseCache cold = cache_bases(tile_c_old, n_slots - 1, s_cold);
    // the schedule and tile bases above come from the append kernel before
    // the propagate kernel this one follows (complete before that propagate
    // kernel let this one start); the propagate kernel's own results are
    // read only from here on
    pdl_wait();
    pdl_trigger();
    // First tile static, then tickets, taken only when the block is free: a
    // ticket taken ahead would hold a tile that its successors' look-back
    // waits for behind the block's current tile.
    uint32_t next = blockIdx.x;
    for(;;)
        {
            if(threadIdx.x == 0)
                {
                    const uint32_t t = next;
                    s_tile = (int)t;
                    s_q = t < total ? find_slot(cbase.base, cbase.n, t) : -1;
                    s_glob = 0;
                    s_fin = 0;
                    if(t < total) s_fa = f_accept_of(P[s_q], S[s_q]);
                }
            __syncthreads();
            const uint32_t t = (uint32_t)s_tile;
            if(t >= total) break;
            const int q = s_q;
            const QueryParams& p = P[q];
            QueryState& st = S[q];
            const uint32_t lt = t - cbase.base[q];
            const uint32_t n_old = cold.base[q];
            const uint32_t itr = st.itr;
            const uint32_t tree_size = st.tree_size;
            if(lt < n_old)
                {
                    // ---- re-activation of old nodes (KGMT.cu:364-377) ----
                    // old_tile / kAppendThreads consecutive nodes a thread (4,
                    // 16 or 32), in rounds of at most kOldPer
                    const uint32_t per_t = old_tile / kAppendThreads;
                    const uint32_t i0 = lt * old_tile + threadIdx.x * per_t;
                    const float fa = s_fa;
                    const uint32_t k0 = (uint32_t)p.seed, k1 = (uint32_t)(p.seed >> 32);
                    uint32_t flags = 0, cnt = 0;
                    static_assert(kOldPer % 4 == 0 && kTileOldLarge / kAppendThreads <= 32, "re-activation: 4-node loads, one flag bit per node");
                    // one round: kOldPer nodes from i0 + r0 -- their regions
                    // four at a time (i0 + r0 is a multiple of 4: the 16-byte
                    // loads are aligned), then the region scores
                    auto round = [&](uint32_t r0) {
                        int32_t reg[kOldPer];
#pragma unroll
                        for(int g = 0; g < kOldPer; g += 4)
                            {
                                const uint32_t ib = i0 + r0 + g;
                                if(r0 + g >= per_t) reg[g] = reg[g + 1] = reg[g + 2] = reg[g + 3] = 0;
                                else if(ib + 3 < tree_size)
                                    {
                                        const int4 v = *(const int4*)(p.node_r1 + ib);
                                        reg[g] = v.x, reg[g + 1] = v.y, reg[g + 2] = v.z, reg[g + 3] = v.w;
                                    }
                                else
                                    {
#pragma unroll
                                        for(int j = 0; j < 4; ++j) reg[g + j] = ib + j < tree_size ? p.node_r1[ib + j] : 0;
                                    }
                            }
#pragma unroll
                        for(int j = 0; j < kOldPer; ++j)
                            {
                                const uint32_t i = i0 + r0 + j;
                                if(r0 + j < per_t && i < tree_size)
                                    {
                                        const U4 r = philox4x32_10(i, itr, 1u, 0u, k0, k1);
                                        const float ur = u01(r.x);
                                        if(ur <= p.score[reg[j]] + fa)
                                            {
                                                flags |= 1u << (r0 + j);
                                                ++cnt;
                                            }
                                    }
                            }
                    };
                    round(0u);
                    if(per_t > (uint32_t)kOldPer) round((uint32_t)kOldPer);
                    uint32_t agg;
                    const uint32_t excl = block_exclusive_scan<kAppendThreads>(cnt, scratch, &agg);
                    publish_and_lookback(p.tiles_old, lt, agg, &s_prefix, &sched->error);
                    if(threadIdx.x == 0) atomicAdd(&st.react_total, agg);
                    __syncthreads();
                    uint32_t pos = (uint32_t)s_prefix + excl;
                    for(uint32_t m = flags; m; m &= m - 1u)
                        {
                            if(KGMT_BOUND(pos < p.capacity)) p.rep_old[pos] = i0 + (uint32_t)(__ffs((int)m) - 1);
                            ++pos;
                        }
                }
            else
                {
                    // ---- ordered append of accepted samples (KGMT.cu:317-362) ----
                    // kAppendPer consecutive samples a thread: their
                    // region-and-flag words four at a time (s0 is a multiple
                    // of 4: 16-byte loads), then the accepted samples' valid
                    // counts -- two round trips; only the flag bits are kept
                    // past the scan (the scatter reads the word again)
                    const uint32_t lts = lt - n_old;
                    const uint32_t s0 = lts * kTileC + threadIdx.x * kAppendPer;
                    const uint32_t ns = st.n_samples;
                    static_assert(kAppendPer % 4 == 0 && kAppendPer <= 32, "16-byte loads of four words, one flag bit per sample");
                    static_assert(kTileC * kRepeatSparse < 65536, "a tile's repeat count fits the scan's low 16 bits");
                    uint32_t rf[kAppendPer];
#pragma unroll
                    for(int g = 0; g < kAppendPer; g += 4)
                        {
                            const uint32_t sb = s0 + g;
                            if(sb + 3 < ns)
                                {
                                    const uint4 v = *(const uint4*)(p.ur1f + sb);
                                    rf[g] = v.x, rf[g + 1] = v.y, rf[g + 2] = v.z, rf[g + 3] = v.w;
                                }
                            else
                                {
#pragma unroll
                                    for(int j = 0; j < 4; ++j) rf[g + j] = sb + j < ns ? p.ur1f[sb + j] : 0u;
                                }
                        }
                    uint32_t acc_bits = 0, sparse_bits = 0, ca = 0, cw = 0;
#pragma unroll
                    for(int j = 0; j < kAppendPer; ++j)
                        if(rf[j] >> 31)
                            {
                                const bool sparse = p.valid[rf[j] & 0x7FFFFFFFu] < kSparseValidLimit;
                                acc_bits |= 1u << j;
                                sparse_bits |= sparse ? 1u << j : 0u;
                                ++ca;
                                cw += sparse ? kRepeatSparse : kRepeatDense;
                            }
                    uint32_t agg;
                    const uint32_t excl = block_exclusive_scan<kAppendThreads>((ca << 16) | cw, scratch, &agg);
                    const uint32_t agg_a = agg >> 16, agg_w = agg & 0xffffu;
                    const unsigned long long val = ((unsigned long long)agg_a << 32) | agg_w;
                    publish_and_lookback(p.tiles_slot, lts, val, &s_prefix, &sched->error);
                    if(threadIdx.x == 0)
                        {
                            atomicAdd(&st.acc_total, agg_a);
                            atomicAdd(&st.w_total, agg_w);
                        }
                    __syncthreads();
                    const unsigned long long pre = s_prefix;
                    uint32_t ia = tree_size + (uint32_t)(pre >> 32) + (excl >> 16);
                    uint32_t iw = (uint32_t)(pre & 0xffffffffull) + (excl & 0xffffu);
                    const int D = (int)p.sample_dim;
                    for(uint32_t m = acc_bits; m; m &= m - 1u)
                        {
                            const int j = __ffs((int)m) - 1;
                            const uint32_t s = s0 + (uint32_t)j;
                            const uint32_t idx = ia++;
                            const uint32_t w = ((sparse_bits >> j) & 1u) ? kRepeatSparse : kRepeatDense;
                            if(!KGMT_BOUND(idx < p.capacity && s < p.capacity))
                                {
                                    iw += w;
                                    continue;
                                }
                            // everything the sample needs is loaded before its
                            // first store (one round trip, not one per field)
                            const int32_t par = __ldg(p.up + s), r1 = (int32_t)(__ldg(p.ur1f + s) & 0x7FFFFFFFu);
                            const float dist = append_row(p, p.us + (size_t)s * D, p.tree + (size_t)idx * D, D);
                            p.parent[idx] = par;
                            p.cost[idx] = dist;
                            p.node_r1[idx] = r1;
                            for(uint32_t r = 0; r < w; ++r, ++iw)
                                if(iw < p.capacity) p.rep_new[iw] = idx;
                            if(dist < p.goal_radius) atomicMin(&st.goal_cand, (int)idx);
                        }
                }
            // ---- tile done; the last tile of the query finalises it ----
            __syncthreads();
            if(threadIdx.x == 0)
                {
                    const uint32_t n_tiles = cbase.base[q + 1] - cbase.base[q];
                    const uint32_t done = atomic_add_release(&st.tiles_done, 1u);
                    // the block is free now: its next ticket, in flight with the count
                    next = gridDim.x + atomicAdd(&sched->ticket_c, 1u);
                    if(done == n_tiles - 1) s_fin = 1;
                }
            __syncthreads();
            if(s_fin)
                {
                    // every tile of this query is done: thread 0 finalises it
                    // and counts it finalised while the other threads clear
                    // its look-back words for the next iteration (nothing in
                    // this kernel reads them again, and the next append
                    // launch sees the stores: no fence on the path)
                    if(threadIdx.x == 0)
                        {
                            __threadfence();
                            st.f_accept = s_fa;
                            finalize_query(p, st, sched);
                            const uint32_t running = sched->running;
                            if(running == 1u)
                                {
                                    // the only running query: its finaliser is
                                    // the last, and no other block's results
                                    // are left to acquire (2: no block fence)
                                    __threadfence();
                                    s_glob = 2;
                                }
                            else if(atomic_add_release(&sched->finalized, 1u) == running - 1u) s_glob = 1;
                        }
                    const uint32_t n_tiles = cbase.base[q + 1] - cbase.base[q];
                    for(uint32_t i = threadIdx.x; i < n_old; i += kAppendThreads) p.tiles_old[i] = 0ull;
                    for(uint32_t i = threadIdx.x; i < n_tiles - n_old; i += kAppendThreads) p.tiles_slot[i] = 0ull;
                    __syncthreads();
                }
            if(s_glob)
                {
                    if(s_glob == 1) __threadfence();
                    compute_schedule<kAppendThreads, true>(P, S, sched, tile_a_base, tile_c_base, tile_c_old);
                }
            __syncthreads();
        }
}

// ---------------------------------------------------------------------------
// goal -> root path walk for finished queries (KGMT.cu:344-360)
// ---------------------------------------------------------------------------
__global__ void k_paths(const QueryParams* __restrict__ P, QueryState* S, uint32_t n)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if(q >= n) return;
    QueryState& st = S[q];
    if(st.status != KGMT_QUERY_SUCCESS || st.path_len != 0) return;
    const QueryParams& p = P[q];
    const uint32_t D = p.sample_dim;
    const uint32_t max_rows = p.max_iterations + 2;
    int32_t i = st.goal_index;
    uint32_t len = 0;
    while(i >= 0 && len < max_rows)
        {
            const float* src = p.tree + (size_t)i * D;
            float* dst = p.path + (size_t)len * D;
            for(uint32_t c = 0; c < D; ++c) dst[c] = src[c];
            ++len;
            i = p.parent[i];
        }
    st.goal_cost = p.cost[st.goal_index];
    st.path_len = len;
}

// ---------------------------------------------------------------------------
// obstacles: [n][6] rows (min xyz, max xyz) -> [n][2] float4 in the arena
// ---------------------------------------------------------------------------
__global__ void k_stage_obstacles(const float* __restrict__ src, float4* dst, uint32_t n, int w)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    stage_box(src + (size_t)i * 2 * w, w, dst + 2 * i);
}

// ---------------------------------------------------------------------------
// function-level propagation with explicit uniforms
// ---------------------------------------------------------------------------
__global__ void k_propagate_samples(const QueryParams p, const float* __restrict__ x0, const float* __restrict__ uni,
                                    const float* __restrict__ obs_rows, uint32_t n_obs, uint32_t n, float* x1, uint8_t* valid,
                                    int32_t* r1, int32_t* r2)
{
    extern __shared__ float4 s_obs[];
    const int w = p.planar ? 2 : 3;
    for(uint32_t i = threadIdx.x; i < n_obs; i += blockDim.x) stage_box(obs_rows + (size_t)i * 2 * w, w, s_obs + 2 * i);
    __syncthreads();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if(s >= n) return;
    const int D = (int)p.sample_dim;
    float a[kMaxSampleDim], b[kMaxSampleDim], u[8];
    for(int j = 0; j < D; ++j) a[j] = x0[(size_t)s * D + j];
    for(int j = 0; j < 8; ++j) u[j] = uni[(size_t)s * 8 + j];
    PropCount cnt;
    const GridView none{nullptr, nullptr, nullptr};
    bool ok = false;
    with_model<kAllModels>(p.model, [&](auto m) { ok = propagate_model<decltype(m)::value>(p, none, a, u, s_obs, n_obs, b, cnt); });
    for(int j = 0; j < D; ++j) x1[(size_t)s * D + j] = b[j];
    valid[s] = ok ? 1 : 0;
    const CellIds c = cell_ids(p, b);
    if(r1) r1[s] = c.r1;
    if(r2) r2[s] = c.r2;
}

// ---------------------------------------------------------------------------
// host-side launch wrappers
// ---------------------------------------------------------------------------
// launch as a programmatic dependent of the kernel before it in the stream
// (the kernel body waits for that one with pdl_wait)
static cudaLaunchConfig_t dependent_config(int grid, int block, size_t smem, cudaStream_t s, cudaLaunchAttribute* attr)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid, 1, 1);
    cfg.blockDim = dim3((unsigned)block, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <int NT, int MODELS>
static cudaError_t launch_propagate_t(const LaunchArgs& a, int grid, uint32_t boxes, cudaStream_t s)
{
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = dependent_config(grid, NT, prop_smem_bytes(boxes), s, attr);
    return cudaLaunchKernelEx(&cfg, k_propagate<NT, MODELS>, a.params, a.states, a.sched, (const uint32_t*)a.tile_a_base, boxes);
}

template <int NT>
static cudaError_t launch_propagate_m(const LaunchArgs& a, int models, int grid, uint32_t boxes, cudaStream_t s)
{
    switch(models)
        {
            case kBitDI: return launch_propagate_t<NT, kBitDI>(a, grid, boxes, s);
            case kBitQuad: return launch_propagate_t<NT, kBitQuad>(a, grid, boxes, s);
            case kBitDubins: return launch_propagate_t<NT, kBitDubins>(a, grid, boxes, s);
            case kBitUnicycle: return launch_propagate_t<NT, kBitUnicycle>(a, grid, boxes, s);
            default: return launch_propagate_t<NT, kAllModels>(a, grid, boxes, s);
        }
}

cudaError_t launch_propagate(const LaunchArgs& a, int block, int models, int grid, uint32_t smem_boxes, cudaStream_t s)
{
    const uint32_t boxes = smem_boxes < kSmemBoxesMin ? kSmemBoxesMin : smem_boxes > (uint32_t)kSmemObstacles ? (uint32_t)kSmemObstacles : smem_boxes;
    switch(block)
        {
            case 128: return launch_propagate_m<128>(a, models, grid, boxes, s);
            case 512: return launch_propagate_m<512>(a, models, grid, boxes, s);
            default: return launch_propagate_m<256>(a, models, grid, boxes, s);
        }
}

// blocks of one variant per SM; also lets the variant take its dynamic
// shared memory on top of more than 48 KB in total (the launch wrappers run
// after this has been called for the variant)
template <int NT, int MODELS>
static int occupancy_t()
{
    int n = 0;
    const size_t smem = kPropSmemBytes;
    if(cudaFuncSetAttribute(k_propagate<NT, MODELS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        {
            cudaGetLastError();
            return 0;
        }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_propagate<NT, MODELS>, NT, smem);
    return n;
}

template <int NT>
static int occupancy_m(int models)
{
    switch(models)
        {
            case kBitDI: return occupancy_t<NT, kBitDI>();
            case kBitQuad: return occupancy_t<NT, kBitQuad>();
            case kBitDubins: return occupancy_t<NT, kBitDubins>();
            case kBitUnicycle: return occupancy_t<NT, kBitUnicycle>();
            default: return occupancy_t<NT, kAllModels>();
        }
}

int propagate_blocks_per_sm(int block, int models)
{
    int n = 0;
    switch(block)
        {
            case 128: n = occupancy_m<128>(models); break;
            case 512: n = occupancy_m<512>(models); break;
            default: n = occupancy_m<256>(models); break;
        }
    return n > 0 ? n : 1;
}

int append_blocks_per_sm()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_append, kAppendThreads, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_append(const LaunchArgs& a, int grid, cudaStream_t s)
{
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = dependent_config(grid, kAppendThreads, 0, s, attr);
    return cudaLaunchKernelEx(&cfg, k_append, a.params, a.states, a.sched, a.tile_a_base, a.tile_c_base, a.tile_c_old);
}

cudaError_t launch_admit(const LaunchArgs& a, uint32_t first, uint32_t count, cudaStream_t s, const uint32_t* slots)
{
    if(count == 0) return cudaSuccess;
    k_admit<<<count, 256, 0, s>>>(a.params, a.states, first, count, slots);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return e;
    k_build_grid<<<count, 256, 0, s>>>(a.params, first, count, slots);
    return cudaGetLastError();
}

cudaError_t launch_schedule(const LaunchArgs& a, cudaStream_t s)
{
    k_schedule<<<1, kAppendThreads, 0, s>>>(a.params, a.states, a.sched, a.tile_a_base, a.tile_c_base, a.tile_c_old);
    return cudaGetLastError();
}

cudaError_t launch_paths(const LaunchArgs& a, uint32_t n, cudaStream_t s)
{
    if(n == 0) return cudaSuccess;
    k_paths<<<(n + 127) / 128, 128, 0, s>>>(a.params, a.states, n);
    return cudaGetLastError();
}

cudaError_t launch_stage_obstacles(const float* src, float4* dst, uint32_t n, int ws_dims, cudaStream_t s)
{
    if(n == 0) return cudaSuccess;
    k_stage_obstacles<<<(n + 255) / 256, 256, 0, s>>>(src, dst, n, ws_dims == 2 ? 2 : 3);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// persistent tail launch
// ---------------------------------------------------------------------------
size_t tail_scratch_bytes() { return sizeof(TailScratch); }

template <int MODELS>
static int tail_occupancy_t()
{
    int n = 0;
    if(cudaFuncSetAttribute(k_tail<MODELS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPropSmemBytes) != cudaSuccess)
        {
            cudaGetLastError();
            return 0;
        }
    if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tail<MODELS>, kTailThreads, kPropSmemBytes) != cudaSuccess)
        {
            cudaGetLastError();
            return 0;
        }
    return n;
}

int tail_blocks_per_sm(int models)
{
    switch(models)
        {
            case kBitDI: return tail_occupancy_t<kBitDI>();
            case kBitQuad: return tail_occupancy_t<kBitQuad>();
            case kBitDubins: return tail_occupancy_t<kBitDubins>();
            case kBitUnicycle: return tail_occupancy_t<kBitUnicycle>();
            default: return tail_occupancy_t<kAllModels>();
        }
}

template <int MODELS>
static cudaError_t launch_tail_t(const LaunchArgs& a, TailScratch* ts, int grid, uint32_t boxes, uint32_t max_samples, uint32_t* host_words,
                                 cudaStream_t s)
{
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid, 1, 1);
    cfg.blockDim = dim3((unsigned)kTailThreads, 1, 1);
    cfg.dynamicSmemBytes = prop_smem_bytes(boxes);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_tail<MODELS>, a.params, a.states, a.sched, ts, a.tile_a_base, a.tile_c_base, a.tile_c_old, boxes,
                              max_samples, host_words);
}

cudaError_t launch_tail(const LaunchArgs& a, TailScratch* ts, int models, int grid, uint32_t smem_boxes, uint32_t max_samples,
                        uint32_t* host_words, cudaStream_t s)
{
    if(grid < 2 * kTailQueries || grid > kTailMaxBlocks) return cudaErrorInvalidValue;
    const uint32_t boxes = smem_boxes < kSmemBoxesMin ? kSmemBoxesMin : smem_boxes > (uint32_t)kSmemObstacles ? (uint32_t)kSmemObstacles : smem_boxes;
    // the barrier counter starts each launch at zero
    cudaError_t e = cudaMemsetAsync(&ts->bar, 0, sizeof(uint32_t), s);
    if(e != cudaSuccess) return e;
    switch(models)
        {
            case kBitDI: return launch_tail_t<kBitDI>(a, ts, grid, boxes, max_samples, host_words, s);
            case kBitQuad: return launch_tail_t<kBitQuad>(a, ts, grid, boxes, max_samples, host_words, s);
            case kBitDubins: return launch_tail_t<kBitDubins>(a, ts, grid, boxes, max_samples, host_words, s);
            case kBitUnicycle: return launch_tail_t<kBitUnicycle>(a, ts, grid, boxes, max_samples, host_words, s);
            default: return launch_tail_t<kAllModels>(a, ts, grid, boxes, max_samples, host_words, s);
        }
}

cudaError_t launch_propagate_samples(const QueryParams& p, const float* x0, const float* u, const float* obs, uint32_t n_obs, uint32_t n,
                                     float* x1, uint8_t* valid, int32_t* r1, int32_t* r2, cudaStream_t s)
{
    if(n == 0) return cudaSuccess;
    const size_t smem = (size_t)n_obs * 2 * sizeof(float4);
    if(smem > 48 * 1024)
        {
            cudaError_t e = cudaFuncSetAttribute(k_propagate_samples, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if(e != cudaSuccess) return e;
        }
    k_propagate_samples<<<(n + 127) / 128, 128, smem, s>>>(p, x0, u, obs, n_obs, n, x1, valid, r1, r2);
    return cudaGetLastError();
}

}  // namespace kgmt
