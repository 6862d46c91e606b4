// kgmt_tail.cuh -- whole planning iterations in one persistent launch for the
// last few running queries.
//
// Once at most kTailQueries queries are still running (the straggler tail of a
// batch, or a single-query plan), an iteration of the two-kernel chain is a
// few thousand samples and a tree or two of old nodes: its time is latency --
// launches, the schedule round trip, the look-back hand-overs of the ordered
// append.  k_tail runs those iterations back to back inside one cooperative
// launch of one block per SM, with four grid-wide barriers per iteration
// instead of launches:
//
//   P1  propagate every running query's samples: the running queries split
//       the blocks into contiguous ranges (a block keeps its query and its
//       staged boxes until a query finishes), a query's samples spread
//       evenly over its blocks, one per thread, the same per-sample code as
//       k_propagate                                              -- barrier --
//   P2  region scores, one block per query (Graph.cu:207-358), while the other
//       blocks count each chunk's accepted samples and their repeat weights
//                                                               -- barrier --
//   P3  re-activation draws of the old nodes, counted per chunk (KGMT.cu:364-377)
//                                                               -- barrier --
//   P4  ordered scatter: each block adds up the counts of the chunks before
//       its own and writes its re-activated nodes, appended tree rows and
//       repeat entries in index order (KGMT.cu:305-403)         -- barrier --
//   P5  every block finalises every query from the totals it read in P4 (the
//       same values in every block, so no further barrier), block 0 writes
//       the state back.
//
// The per-iteration values that several blocks accumulate or read back
// (accepted samples, goal candidates) sit in two copies by iteration parity,
// so a block that is still reading one iteration's copy never sees the next
// iteration's reset.  Every wait is bounded (kErrBarrierTimeout, reported as
// KGMT_ERR_TIMEOUT).  The launch stops before an iteration larger than
// `max_samples` and leaves the state exactly as the two-kernel chain expects
// it (it recomputes the schedule), so the host can go on with that chain.
#pragma once
#include <climits>
#include <cstdint>

#include "kgmt_iter.cuh"

namespace kgmt {

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// All blocks of the cooperative launch meet here.  Thread 0 of each block
// publishes the block's writes (fence, then the arrival add) and waits for
// every arrival of this round; after the block barrier every thread acquires
// the counter, so its later loads see the other blocks' writes.  The counter
// only grows within a launch: round r completes at r * gridDim.x arrivals.
// Returns false when the wait gave up (kErrBarrierTimeout recorded).
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t& target, uint32_t* error)
{
    __shared__ int s_ok;
    __syncthreads();
    target += gridDim.x;
    if(threadIdx.x == 0)
        {
            __threadfence();
            atomicAdd(bar, 1u);
            int ok = 1;
            uint32_t spins = 0;
            while(ld_acquire_u32(bar) < target)
                {
                    if(++spins > kSpinLimit)
                        {
                            atomicOr(error, kErrBarrierTimeout);
                            ok = 0;
                            break;
                        }
                    __nanosleep(32);
                }
            s_ok = ok;
        }
    __syncthreads();
    (void)ld_acquire_u32(bar);
    return s_ok != 0;
}

// sums of K values over the block (every thread gets the totals)
template <int NT, int K>
__device__ __forceinline__ void block_sum(uint32_t (&v)[K], uint32_t (*scratch)[K])
{
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for(int k = 0; k < K; ++k) v[k] = __reduce_add_sync(0xffffffffu, v[k]);
    if(lane == 0)
#pragma unroll
        for(int k = 0; k < K; ++k) scratch[warp][k] = v[k];
    __syncthreads();
#pragma unroll
    for(int k = 0; k < K; ++k)
        {
            uint32_t t = 0;
#pragma unroll
            for(int w = 0; w < NW; ++w) t += scratch[w][k];
            v[k] = t;
        }
    __syncthreads();
}

// contiguous chunk `c` of `parts` over [0, n) (chunk sizes a multiple of 4),
// and the thread's contiguous share of it: items [*lo, *hi)
template <int NT>
__device__ __forceinline__ void thread_items(uint32_t n, uint32_t parts, uint32_t c, uint32_t* lo, uint32_t* hi)
{
    uint32_t cs = (n + parts - 1) / parts;
    cs = (cs + 3u) & ~3u;
    const uint32_t c0 = min(n, c * cs), c1 = min(n, c0 + cs);
    const uint32_t k = (cs + NT - 1) / NT;
    *lo = min(c1, c0 + threadIdx.x * k);
    *hi = min(c1, *lo + k);
}

// replicated per-query loop state (every block holds the same copy)
struct TailQuery {
    int slot;
    uint32_t status, itr, tree, n_react, w_new, spe, n_samples, drawn;
    uint32_t react_total, acc_total, w_total, n_next;
    float fa;
};

// re-activation draw of old node i (KGMT.cu:371-373)
__device__ __forceinline__ bool reactivated(const QueryParams& p, uint32_t i, uint32_t itr, float fa)
{
    const U4 r = philox4x32_10(i, itr, 1u, 0u, (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
    return u01(r.x) <= __ldcg(p.score + __ldcg(p.node_r1 + i)) + fa;
}

template <int MODELS>
__global__ void __launch_bounds__(kTailThreads, 1) k_tail(const QueryParams* __restrict__ P, QueryState* S, Sched* sched, TailScratch* ts,
                                                         uint32_t* tile_a_base, uint32_t* tile_c_base, uint32_t* tile_c_old,
                                                         uint32_t smem_boxes, uint32_t max_samples, uint32_t* host_words)
{
    constexpr int NT = kTailThreads;
    extern __shared__ float4 s_dyn[];
    uint16_t* s_gstart = (uint16_t*)s_dyn;
    uint16_t* s_gitems = (uint16_t*)((char*)s_dyn + kSmemStartBytes);
    uint32_t* s_gmeta = (uint32_t*)((char*)s_dyn + kSmemStartBytes + kSmemItemBytes);
    float4* s_obs = (float4*)((char*)s_dyn + kSmemGridBytes);
    __shared__ uint32_t s_copy;
    __shared__ alignas(8) uint64_t mbar;
    __shared__ QueryParams s_p;
    __shared__ PropCtx s_c;
    __shared__ PropShared s_sh;
    __shared__ float s_lanes[kScoreLanes];
    __shared__ uint32_t s_scan[34];
    __shared__ uint32_t s_sum[NT / 32][6];
    __shared__ TailQuery tq[kTailQueries];
    __shared__ uint32_t s_acc[kTailQueries];
    const uint32_t G = gridDim.x, b = blockIdx.x;
    uint32_t target = 0;

    // ---- the running queries, in slot order (the same in every block) ----
    if(threadIdx.x == 0)
        {
            mbar_init(&mbar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    const uint32_t n_slots = __ldcg(&sched->n_slots);
    uint32_t count = 0;
    for(uint32_t base = 0; base < n_slots; base += NT)
        {
            const uint32_t i = base + threadIdx.x;
            const uint32_t run = (i < n_slots && __ldcg(&S[i].status) == KGMT_QUERY_RUNNING) ? 1u : 0u;
            uint32_t tot;
            const uint32_t pos = count + block_exclusive_scan<NT>(run, s_scan, &tot);
            if(run && pos < (uint32_t)kTailQueries) tq[pos].slot = (int)i;
            count += tot;
        }
    if(count == 0 || count > (uint32_t)kTailQueries)
        {
            // nothing for this launch: the chain's state is untouched
            if(b == 0 && threadIdx.x == 0)
                {
                    ts->iterations = 0;
                    ts->declined = count > 0 ? 1u : 0u;
                    if(host_words)
                        {
                            *(volatile uint32_t*)&host_words[0] = 0u;
                            *(volatile uint32_t*)&host_words[1] = count > 0 ? 1u : 0u;
                        }
                }
            return;
        }
    const int nq = (int)count;
    __syncthreads();
    if((int)threadIdx.x < nq)
        {
            TailQuery& Q = tq[threadIdx.x];
            const QueryState& st = S[Q.slot];
            Q.status = __ldcg(&st.status);
            Q.itr = __ldcg(&st.itr);
            Q.tree = __ldcg(&st.tree_size);
            Q.n_react = __ldcg(&st.n_react);
            Q.w_new = __ldcg(&st.w_new);
            Q.spe = __ldcg(&st.spe);
            Q.n_samples = __ldcg(&st.n_samples);
            Q.drawn = __ldcg(&st.samples_drawn);
        }
    if(b == 0 && threadIdx.x < 2 * kTailQueries)
        {
            (&ts->n_next[0][0])[threadIdx.x] = 0u;
            (&ts->goal[0][0])[threadIdx.x] = ~0u;
        }
    if(!grid_barrier(&ts->bar, target, &sched->error)) return;

    uint32_t par = 0, iters = 0;
    uint32_t declined = 0;
    int cur_slot = -1;
    uint32_t phase = 0;
    for(;;)
        {
            // ---- the iteration's size; the running queries split the blocks
            // into contiguous ranges (a block keeps its query and its staged
            // boxes until a query finishes) ----
            uint32_t tot = 0;
            int nr = 0, rq[kTailQueries];
#pragma unroll
            for(int q = 0; q < kTailQueries; ++q)
                if(q < nq && tq[q].status == KGMT_QUERY_RUNNING) tot += tq[q].n_samples, rq[nr++] = q;
            if(nr == 0) break;
            if(tot > max_samples)
                {
                    declined = 1;
                    break;
                }
            if(threadIdx.x < kTailQueries) s_acc[threadIdx.x] = 0u;
            __syncthreads();

            // ---- P1: propagate (KGMT.cu:218-299), the query's samples spread
            // evenly over its blocks, one per thread ----
            {
                const int qi = (int)((b * (uint32_t)nr) / G);
                const uint32_t bq0 = ((uint32_t)qi * G + nr - 1) / nr, bq1 = ((uint32_t)(qi + 1) * G + nr - 1) / nr;
                const int q = rq[qi];
                const uint32_t ns = tq[q].n_samples, nb = bq1 - bq0;
                uint32_t share = (ns + nb - 1) / nb;
                share = (share + 31u) & ~31u;
                const uint32_t lo = min(ns, (b - bq0) * share), hi = min(ns, lo + share);
                if(lo < hi)
                    {
                        const int slot = tq[q].slot;
                        bool wait_obs = false;
                        if(slot != cur_slot)
                            {
                                const uint32_t* src = (const uint32_t*)&P[slot];
                                uint32_t* dst = (uint32_t*)&s_p;
                                for(int i = threadIdx.x; i < (int)(sizeof(QueryParams) / 4); i += NT) dst[i] = src[i];
                                if(threadIdx.x == 0)
                                    {
                                        const QueryParams& gp = P[slot];
                                        const uint32_t n_obs = gp.n_obstacles;
                                        const bool obs_s = n_obs > 0 && n_obs <= smem_boxes;
                                        const bool grid = gp.grid_meta != nullptr;
                                        const uint32_t bytes = (obs_s ? n_obs * 32u : 0u) + (grid ? 16u + kSmemStartBytes + kSmemItemBytes : 0u);
                                        s_copy = bytes;
                                        if(bytes)
                                            {
                                                fence_proxy_async_smem();
                                                mbar_expect_tx(&mbar, bytes);
                                                if(obs_s) bulk_copy_g2s(s_obs, gp.obstacles, n_obs * 32u, &mbar);
                                                if(grid)
                                                    {
                                                        bulk_copy_g2s(s_gmeta, gp.grid_meta, 16u, &mbar);
                                                        bulk_copy_g2s(s_gstart, gp.grid_start, kSmemStartBytes, &mbar);
                                                        bulk_copy_g2s(s_gitems, gp.grid_items, kSmemItemBytes, &mbar);
                                                    }
                                            }
                                    }
                                __syncthreads();
                                wait_obs = s_copy != 0;
                                cur_slot = slot;
                            }
                        if(threadIdx.x == 0)
                            {
                                s_c.itr = tq[q].itr;
                                s_c.spe = tq[q].spe;
                                s_c.n_react = tq[q].n_react;
                                s_c.n_samples = ns;
                                s_sh.acc = 0, s_sh.steps = 0, s_sh.tests = 0, s_sh.next_run = 0;
                            }
                        __syncthreads();
                        for(uint32_t r0 = lo; r0 < hi; r0 += NT)
                            propagate_range<NT, MODELS>(s_p, s_c, r0, min((uint32_t)NT, hi - r0), smem_boxes, &s_sh, s_obs, s_gstart, s_gitems,
                                                        s_gmeta, [&] {
                                                            // the staged boxes: waited for once, before their first use
                                                            if(!wait_obs) return;
                                                            wait_obs = false;
                                                            uint32_t spins = 0;
                                                            while(!mbar_try_wait(&mbar, phase))
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
                                s_acc[q] += s_sh.acc;
                                QueryState& st = S[slot];
                                if(s_sh.steps) atomicAdd(&st.steps, (unsigned long long)s_sh.steps);
                                if(s_sh.tests) atomicAdd(&st.tests, (unsigned long long)s_sh.tests);
                                const unsigned long long lookup = s_p.n_obstacles ? kOpsPerGridLookup : 0u;
                                const unsigned long long ops = (unsigned long long)s_sh.steps * (ops_per_step(s_p.model) + lookup) +
                                                               (unsigned long long)s_sh.tests * kOpsPerObstacleTest;
                                if(ops) atomicAdd(&ts->fp32_ops, ops);
                                atomicAdd(&ts->samples, (unsigned long long)(hi - lo));
                            }
                        __syncthreads();
                    }
            }
            if((int)threadIdx.x < nq && s_acc[threadIdx.x]) atomicAdd(&ts->n_next[par][threadIdx.x], s_acc[threadIdx.x]);
            if(!grid_barrier(&ts->bar, target, &sched->error)) return;

            // ---- P2: region scores (blocks 0..nq-1); accepted samples and
            // their repeat weights per chunk (the other blocks).  A thread
            // with at most 32 items keeps their flags for P4: bit i of abits
            // accepted, of wbits a sparse region (repeat 15) ----
            uint32_t abits[kTailQueries], wbits[kTailQueries], obits[kTailQueries];
            if((int)b < nq)
                {
                    if(tq[b].status == KGMT_QUERY_RUNNING)
                        {
                            const QueryParams& gp = P[tq[b].slot];
                            const ScoreParams sp{gp.counter, gp.valid, gp.score, gp.marks, gp.newmarks, gp.regions, gp.fine_cells, gp.epsilon,
                                                 gp.cell_volume};
                            update_scores<NT>(sp, S[tq[b].slot], s_lanes);
                        }
                }
            else
#pragma unroll
                for(int q = 0; q < kTailQueries; ++q)
                    {
                        abits[q] = wbits[q] = 0u;
                        if(q >= nq || tq[q].status != KGMT_QUERY_RUNNING) continue;
                        const QueryParams& gp = P[tq[q].slot];
                        uint32_t lo, hi;
                        thread_items<NT>(tq[q].n_samples, G - nq, b - nq, &lo, &hi);
                        uint32_t v[2] = {0u, 0u};
                        for(uint32_t s = lo; s < hi; ++s)
                            {
                                const uint32_t rf = __ldcg(gp.ur1f + s);
                                if(rf >> 31)
                                    {
                                        const bool sparse = __ldcg(gp.valid + (rf & 0x7FFFFFFFu)) < kSparseValidLimit;
                                        v[0] += 1u;
                                        v[1] += sparse ? kRepeatSparse : kRepeatDense;
                                        if(s - lo < 32u)
                                            {
                                                abits[q] |= 1u << (s - lo);
                                                wbits[q] |= sparse ? 1u << (s - lo) : 0u;
                                            }
                                    }
                            }
                        block_sum<NT, 2>(v, (uint32_t(*)[2])s_sum);
                        if(threadIdx.x == 0)
                            {
                                ts->acc_cnt[q][b - nq] = v[0];
                                ts->rep_cnt[q][b - nq] = v[1];
                            }
                    }
            if(b == 0 && threadIdx.x < kTailQueries)
                {
                    // the other parity's copies start the next iteration from
                    // zero (every block read them before this iteration began)
                    ts->n_next[par ^ 1u][threadIdx.x] = 0u;
                    ts->goal[par ^ 1u][threadIdx.x] = ~0u;
                }
            if(!grid_barrier(&ts->bar, target, &sched->error)) return;

            // ---- P3: re-activation draws of the old nodes, counted per chunk
            // (bit i of obits: item i re-activated, for threads of <= 32 items) ----
            if((int)threadIdx.x < nq)
                {
                    TailQuery& Q = tq[threadIdx.x];
                    if(Q.status == KGMT_QUERY_RUNNING)
                        {
                            Q.n_next = __ldcg(&ts->n_next[par][threadIdx.x]);
                            Q.fa = f_accept_vals(P[Q.slot], Q.tree, Q.n_next, Q.itr);
                        }
                }
            __syncthreads();
#pragma unroll
            for(int q = 0; q < kTailQueries; ++q)
                {
                    obits[q] = 0u;
                    if(q >= nq || tq[q].status != KGMT_QUERY_RUNNING) continue;
                    const QueryParams& gp = P[tq[q].slot];
                    uint32_t lo, hi;
                    thread_items<NT>(tq[q].tree, G, b, &lo, &hi);
                    uint32_t v[1] = {0u};
                    for(uint32_t i = lo; i < hi; ++i)
                        if(reactivated(gp, i, tq[q].itr, tq[q].fa))
                            {
                                v[0] += 1u;
                                if(i - lo < 32u) obits[q] |= 1u << (i - lo);
                            }
                    block_sum<NT, 1>(v, (uint32_t(*)[1])s_sum);
                    if(threadIdx.x == 0) ts->old_cnt[q][b] = v[0];
                }
            if(!grid_barrier(&ts->bar, target, &sched->error)) return;

            // ---- P4: ordered scatter of re-activated nodes and appended samples ----
#pragma unroll
            for(int q = 0; q < kTailQueries; ++q)
                {
                    if(q >= nq || tq[q].status != KGMT_QUERY_RUNNING) continue;
                    const QueryParams& gp = P[tq[q].slot];
                    // the chunks before this block's, and all of them
                    uint32_t v[6] = {0u, 0u, 0u, 0u, 0u, 0u};
                    for(uint32_t j = threadIdx.x; j < G; j += NT)
                        {
                            const uint32_t o = __ldcg(&ts->old_cnt[q][j]);
                            v[0] += j < b ? o : 0u;
                            v[1] += o;
                            if(j < G - nq)
                                {
                                    const uint32_t a = __ldcg(&ts->acc_cnt[q][j]), w = __ldcg(&ts->rep_cnt[q][j]);
                                    v[2] += j + nq < b ? a : 0u;
                                    v[3] += a;
                                    v[4] += j + nq < b ? w : 0u;
                                    v[5] += w;
                                }
                        }
                    block_sum<NT, 6>(v, s_sum);
                    const uint32_t cap = gp.capacity, itr = tq[q].itr, tree = tq[q].tree;
                    // re-activated old nodes in index order (KGMT.cu:364-377)
                    {
                        uint32_t lo, hi;
                        thread_items<NT>(tree, G, b, &lo, &hi);
                        const bool kept = hi - lo <= 32u;
                        uint32_t n = 0;
                        if(kept) n = __popc(obits[q]);
                        else
                            for(uint32_t i = lo; i < hi; ++i) n += reactivated(gp, i, itr, tq[q].fa) ? 1u : 0u;
                        uint32_t tot;
                        uint32_t pos = v[0] + block_exclusive_scan<NT>(n, s_scan, &tot);
                        if(kept)
                            for(uint32_t m = obits[q]; m; m &= m - 1u)
                                {
                                    if(KGMT_BOUND(pos < cap)) gp.rep_old[pos] = lo + (uint32_t)(__ffs(m) - 1);
                                    ++pos;
                                }
                        else if(n)
                            for(uint32_t i = lo; i < hi; ++i)
                                if(reactivated(gp, i, itr, tq[q].fa))
                                    {
                                        if(KGMT_BOUND(pos < cap)) gp.rep_old[pos] = i;
                                        ++pos;
                                    }
                    }
                    // accepted samples appended in slot order (KGMT.cu:317-362)
                    if(b >= (uint32_t)nq)
                        {
                            uint32_t lo, hi;
                            thread_items<NT>(tq[q].n_samples, G - nq, b - nq, &lo, &hi);
                            const bool kept = hi - lo <= 32u;
                            uint32_t ca = 0, cw = 0;
                            if(kept)
                                {
                                    ca = __popc(abits[q]);
                                    const uint32_t sp = __popc(abits[q] & wbits[q]);
                                    cw = sp * kRepeatSparse + (ca - sp) * kRepeatDense;
                                }
                            else
                                for(uint32_t s = lo; s < hi; ++s)
                                    {
                                        const uint32_t rf = __ldcg(gp.ur1f + s);
                                        if(rf >> 31)
                                            {
                                                ca += 1u;
                                                cw += __ldcg(gp.valid + (rf & 0x7FFFFFFFu)) < kSparseValidLimit ? kRepeatSparse : kRepeatDense;
                                            }
                                    }
                            uint3 tot3;
                            const uint3 ex = block_exclusive_scan3<NT>(make_uint3(ca, cw, 0u), (uint3*)s_lanes, &tot3);
                            uint32_t ia = tree + v[2] + ex.x, iw = v[4] + ex.y;
                            const int D = (int)gp.sample_dim;
                            if(ca)
                                for(uint32_t s = lo; s < hi; ++s)
                                    {
                                        uint32_t w;
                                        if(kept)
                                            {
                                                if(!((abits[q] >> (s - lo)) & 1u)) continue;
                                                w = ((wbits[q] >> (s - lo)) & 1u) ? kRepeatSparse : kRepeatDense;
                                            }
                                        else
                                            {
                                                const uint32_t rf = __ldcg(gp.ur1f + s);
                                                if(!(rf >> 31)) continue;
                                                w = __ldcg(gp.valid + (rf & 0x7FFFFFFFu)) < kSparseValidLimit ? kRepeatSparse : kRepeatDense;
                                            }
                                        const uint32_t idx = ia++;
                                        if(!KGMT_BOUND(idx < cap && s < cap))
                                            {
                                                iw += w;
                                                continue;
                                            }
                                        // region, parent and row: independent loads, one round trip
                                        const int32_t r1 = (int32_t)(__ldcg(gp.ur1f + s) & 0x7FFFFFFFu);
                                        const int32_t parent = __ldcg(gp.up + s);
                                        const float dist = append_row<true>(gp, gp.us + (size_t)s * D, gp.tree + (size_t)idx * D, D);
                                        gp.parent[idx] = parent;
                                        gp.cost[idx] = dist;
                                        gp.node_r1[idx] = r1;
                                        for(uint32_t r = 0; r < w; ++r, ++iw)
                                            if(iw < cap) gp.rep_new[iw] = idx;
                                        if(dist < gp.goal_radius) atomicMin(&ts->goal[par][q], idx);
                                    }
                        }
                    if(threadIdx.x == 0)
                        {
                            tq[q].react_total = v[1];
                            tq[q].acc_total = v[3];
                            tq[q].w_total = v[5];
                            if(b == 0 && v[3] != tq[q].n_next) atomicOr(&sched->error, kErrAppendMismatch);
                        }
                    __syncthreads();
                }
            if(!grid_barrier(&ts->bar, target, &sched->error)) return;

            // ---- P5: finalise (KGMT.cu:88-95, 380-403); every block computes
            // the same state, block 0 writes it back ----
            if((int)threadIdx.x < nq)
                {
                    TailQuery& Q = tq[threadIdx.x];
                    if(Q.status == KGMT_QUERY_RUNNING)
                        {
                            const QueryParams& gp = P[Q.slot];
                            const uint32_t goal = __ldcg(&ts->goal[par][threadIdx.x]);
                            const uint32_t tree = Q.tree + Q.acc_total;
                            uint32_t status = KGMT_QUERY_RUNNING;
                            if(goal != ~0u) status = KGMT_QUERY_SUCCESS;
                            else if(Q.itr >= gp.max_iterations) status = KGMT_QUERY_ITER_LIMIT;
                            else if(tree >= gp.capacity) status = KGMT_QUERY_CAPACITY;
                            Q.drawn += Q.n_samples;
                            Q.tree = tree;
                            Q.n_react = Q.react_total;
                            Q.w_new = Q.w_total;
                            QueryState& st = S[Q.slot];
                            if(b == 0)
                                {
                                    st.tree_size = tree;
                                    st.samples_drawn = Q.drawn;
                                    st.n_react = Q.n_react;
                                    st.w_new = Q.w_new;
                                    st.f_accept = Q.fa;
                                }
                            if(status != KGMT_QUERY_RUNNING)
                                {
                                    Q.status = status;
                                    if(b == 0)
                                        {
                                            if(status == KGMT_QUERY_SUCCESS) st.goal_index = (int32_t)goal;
                                            st.t_end = globaltimer();
                                            st.status = status;
                                        }
                                }
                            else
                                {
                                    Q.itr += 1;
                                    plan_samples_vals(gp.capacity, gp.samples_per_node, tree, Q.n_react + Q.w_new, &Q.spe, &Q.n_samples);
                                    if(b == 0)
                                        {
                                            st.itr = Q.itr;
                                            st.spe = Q.spe;
                                            st.n_samples = Q.n_samples;
                                        }
                                }
                        }
                }
            __syncthreads();
            par ^= 1u;
            ++iters;
        }

    // ---- hand the state back: the two-kernel chain's schedule of what is left ----
    if(b == 0)
        {
            if(threadIdx.x == 0)
                {
                    ts->iterations = iters;
                    ts->declined = declined;
                    atomicAdd(&sched->iterations, iters);
                    if(host_words)
                        {
                            *(volatile uint32_t*)&host_words[0] = iters;
                            *(volatile uint32_t*)&host_words[1] = declined;
                        }
                }
            __syncthreads();
            compute_schedule<NT, false>(P, S, sched, tile_a_base, tile_c_base, tile_c_old);
        }
}

}  // namespace kgmt
