// kgmt_types.h -- device-resident descriptors of the planning engine.
//
// One engine runs any number of independent queries ("slots").  Per slot:
//   QueryParams  immutable after admission: config values pre-derived in
//                float, and the device pointers of the slot's buffers
//   QueryState   mutable loop state (iteration, tree size, frontier sizes)
// and one Sched per engine: the device-computed schedule of the next
// iteration (tiles per slot, tickets), so the host never reads sizes back.
#pragma once
#include <cstdint>

#include "../../include/kgmt.h"

namespace kgmt {

constexpr int kMaxSampleDim = KGMT_MAX_SAMPLE_DIM;
constexpr int kScoreLanes = 256;        // fixed summation shape of the score total
constexpr int kTileC = 1024;            // samples per append tile
constexpr int kAppendThreads = 256;     // threads per append block
constexpr int kAppendPer = kTileC / kAppendThreads;  // samples per append thread
// old nodes per re-activation tile: larger than an append tile, so the fixed
// latency of a tile (loads, scan, look-back, hand-over) covers more nodes;
// small tiles (4 nodes a thread) while all running queries' old nodes fill
// fewer large tiles than there are SMs, so few trees still spread out
constexpr int kTileOld = 4096;
constexpr int kTileOldSmall = 1024;
constexpr int kTileOldLarge = 8192;
constexpr int kOldPer = kTileOld / kAppendThreads;  // old nodes per thread and round, at most
// iterations whose running trees hold at least this many large tiles per SM
// use large re-activation tiles (two rounds of kOldPer nodes a thread)
constexpr uint32_t kOldLargeWaves = 8;
// samples per propagate thread and tile in iterations with enough samples to
// fill the resident threads twice: a tile of kPropPer * NT samples is sorted
// by step count and run 32 consecutive samples at a time, the longest first,
// by whichever warp of the block is free, so the warps finish together.
// Smaller iterations keep one sample per thread (more tiles in parallel, a
// shorter chain per thread).
constexpr int kPropPer = 2;
constexpr int kRootRepeat = 5;          // KGMT.cu:67
constexpr int kRepeatSparse = 15;       // KGMT.cu:336-337
constexpr int kRepeatDense = 1;         // KGMT.cu:338-339
constexpr int kSparseValidLimit = 10;   // KGMT.cu:336
constexpr int kSmemObstacles = 512;     // boxes staged in shared memory per block
constexpr uint32_t kSpinLimit = 1u << 22;  // polls before a device-side wait gives up

constexpr uint32_t kSlotEmpty = 0xFFFFFFFFu;  // QueryState::status of a never-admitted slot

// persistent tail launch (kgmt_tail.cuh): at most this many running queries,
// one block of kTailThreads per SM, at most kTailMaxBlocks blocks
constexpr int kTailQueries = 4;
constexpr int kTailThreads = 256;
constexpr int kTailMaxBlocks = 1024;

// static FP32 lane-operation counts per RK4 step, from the code in
// kgmt_device.cuh (a multiply, add, fused multiply-add, divide or compare is
// one; the quadrotor's portable sine/cosine counted as the operations it is
// made of: 4 ode evaluations of ~140, stage and update combinations, checks)
constexpr uint32_t kOpsPerStepDI = 81;
constexpr uint32_t kOpsPerStepQuad = 662;
// Dubins airplane: 4 portable sine/cosine pairs (~26 each: reduction, two
// polynomials, quadrant selection), 4 attitude offsets, 12 stage products,
// 23 for the three position sums, 3 updates, 10 compares
constexpr uint32_t kOpsPerStepDubins = 148;
// unicycle: one sine/cosine pair, 14 for the Euler update, 4 compares
constexpr uint32_t kOpsPerStepUnicycle = 44;
__host__ __device__ constexpr uint32_t ops_per_step(int32_t model)
{
    return model == KGMT_MODEL_QUADROTOR ? kOpsPerStepQuad
         : model == KGMT_MODEL_DUBINS_AIRPLANE ? kOpsPerStepDubins
         : model == KGMT_MODEL_UNICYCLE ? kOpsPerStepUnicycle : kOpsPerStepDI;
}
constexpr uint32_t kOpsPerObstacleTest = 6;
constexpr uint32_t kOpsPerGridLookup = 24;  // six cell coordinates of the step box

constexpr uint32_t kGridDim = 16;           // obstacle grid cells per axis
constexpr uint32_t kGridCells = kGridDim * kGridDim * kGridDim;
constexpr uint32_t kGridMaxVisit = 8;       // cells a step box may visit before falling back to all boxes
constexpr uint32_t kMaxObstacles = 65535;   // grid items are 16-bit box indices
constexpr uint32_t kMaxGridItems = 65535;   // grid starts are 16-bit
constexpr uint32_t kSmemGridItems = 4096;   // grid items staged in shared memory per block
// dynamic shared memory of k_propagate: grid starts, grid items, grid meta,
// then the boxes -- as many as the launch's box capacity, a power of two
// from kSmemBoxesMin to kSmemObstacles sized to the admitted queries (what
// shared memory the boxes leave unused stays L1 cache)
constexpr uint32_t kSmemStartBytes = ((kGridCells + 1) * 2 + 15) / 16 * 16;
constexpr uint32_t kSmemItemBytes = kSmemGridItems * 2;
constexpr uint32_t kSmemGridBytes = kSmemStartBytes + kSmemItemBytes + 16;
constexpr uint32_t kSmemBoxesMin = 64;
constexpr uint32_t kPropSmemBytes = kSmemGridBytes + kSmemObstacles * 32;  // the largest launch
__host__ __device__ constexpr uint32_t prop_smem_bytes(uint32_t boxes) { return kSmemGridBytes + boxes * 32; }
// box capacity for queries of at most max_obs boxes
inline uint32_t smem_boxes_for(uint32_t max_obs)
{
    uint32_t c = kSmemBoxesMin;
    while(c < max_obs && c < (uint32_t)kSmemObstacles) c <<= 1;
    return c;
}

// error bits in Sched::error
constexpr uint32_t kErrLookbackTimeout = 1u;
constexpr uint32_t kErrCopyTimeout = 2u;
constexpr uint32_t kErrBounds = 4u;  // an index check of a KGMT_CHECK_BOUNDS build failed
constexpr uint32_t kErrAppendMismatch = 8u;  // appended samples != accepted samples
constexpr uint32_t kErrBarrierTimeout = 16u;  // a grid-wide barrier of the tail launch gave up

struct QueryParams {
    int32_t model;
    int32_t di_rule;
    uint32_t capacity;
    uint32_t samples_per_node;
    uint32_t max_iterations;
    uint32_t min_steps, max_steps;
    uint32_t sample_dim;
    float step_span;  // (float)(max_steps - min_steps + 1)
    float step_size, half_step, sixth_step;
    float goal_radius, epsilon;
    float ws_min, ws_max, ws_range, cell_size, cell_volume;
    float inv_range, inv_cell;     // exact reciprocals when the sizes are powers of two
    int32_t range_pow2, cell_pow2; // 1: divide by multiplying with the reciprocal (same IEEE result)
    uint32_t coarse_len, fine_len, regions, fine_cells;
    float v_min, v_max;
    float u_min[4], u_span[4];
    int32_t planar;                // 1: 2-D workspace (unicycle), z of every position = ws_min
    float pitch_min, pitch_max;    // Dubins airplane
    float wheelbase;               // unicycle
    float nu, mu, gravity, mass_inv;
    float iix, iiy, iiz;  // 1 / I
    float jx, jy, jz;     // (Iy - Iz) / Ix, (Iz - Ix) / Iy, (Ix - Iy) / Iz
    uint64_t seed;
    float goal[3];
    float init[kMaxSampleDim];
    uint32_t n_obstacles;
    uint32_t tiles_per_chain;  // capacity of each tile-state chain
    // buffers (device pointers into the engine arena)
    float* tree;          // [capacity][sample_dim]   d_treeSamples_
    int32_t* parent;      // [capacity]               d_treeSamplesParentIdxs_
    float* cost;          // [capacity]               d_treeSampleCosts_
    int32_t* node_r1;     // [capacity] coarse region of each node
    uint32_t* rep_old;    // [capacity] re-activated nodes (repeat 1 each)
    uint32_t* rep_new;    // [capacity] new nodes, each repeated 15 or 1 times
    float* us;            // [capacity][sample_dim] unexplored samples
    int32_t* up;          // [capacity] parent of each sample
    uint32_t* ur1f;       // [capacity] region of each sample; top bit: the sample joins the tree
    int32_t* counter;     // [regions] samples per region          (d_counterArray_)
    int32_t* valid;       // [regions] valid samples per region    (d_validCounterArray_)
    float* score;         // [regions]                              (d_vertexScoreArray_)
    uint64_t* marks;      // [regions] fine cells visited, one bit per cell (d_activeSubVertices_)
    uint64_t* newmarks;   // [regions] cells first visited this iteration
    float4* obstacles;    // [n_obstacles][2] (min.xyz, -), (max.xyz, -)
    unsigned long long* tiles_old;   // [tiles_per_chain] look-back words, re-activation chain
    unsigned long long* tiles_slot;  // [tiles_per_chain] look-back words, append chain
    float* path;          // [max_iterations + 2][sample_dim] goal -> root rows
    // uniform grid over the workspace listing the boxes that touch each cell
    // (built on the device at admission); lets a step box test only the boxes
    // of the cells it overlaps
    uint32_t grid_dim;       // cells per axis
    float grid_scale;        // grid_dim / workspace size
    uint32_t grid_budget;    // capacity of grid_items (<= 65535)
    uint32_t* grid_meta;     // [4]: [0] items in use, [1] 1 = usable
    // boxes as rows of 2 * raw_w floats (min corner, max corner) in device
    // memory, staged into `obstacles` by the admission kernel (served queries;
    // null when staged beforehand)
    const float* raw_obstacles;
    int32_t raw_w;
    uint16_t* grid_start;    // [grid_dim^3 + 1] CSR starts (16-bit: at most 65535 items)
    uint16_t* grid_items;    // [grid_budget] box indices, cell by cell
};

struct QueryState {
    uint32_t status;      // KGMT_QUERY_*
    uint32_t itr;         // iteration being run (1-based), h_itr_
    uint32_t tree_size;   // h_treeSize_
    uint32_t n_react;     // rep_old length
    uint32_t w_new;       // rep_new length (sum of repeats)
    uint32_t spe;         // samples per frontier entry this iteration
    uint32_t n_samples;   // samples this iteration
    uint32_t n_next;      // accepted samples (atomic, propagate)
    int32_t goal_cand;    // smallest new tree index in the goal ball (atomicMin)
    int32_t goal_index;
    uint32_t tiles_done;  // append/re-activation tiles finished this iteration
    uint32_t prop_done;   // propagate tiles finished this iteration
    uint32_t react_total; // atomics of the append kernel
    uint32_t acc_total;
    uint32_t w_total;
    float f_accept;
    float score_total;
    uint32_t samples_drawn;
    uint32_t path_len;
    float goal_cost;      // the goal node's cost (set with the path)
    unsigned long long t_start;  // %globaltimer at admission (ns)
    unsigned long long t_end;
    unsigned long long steps;    // RK4 steps executed over all samples
    unsigned long long tests;    // step-box x box tests performed
};

struct Sched {
    uint32_t n_slots;
    uint32_t running;
    uint32_t tiles_a;     // propagate tiles this iteration
    uint32_t tiles_c;     // append / re-activation tiles this iteration
    uint32_t ticket_a;
    uint32_t ticket_c;
    uint32_t finalized;
    uint32_t error;
    uint32_t iterations;  // engine iterations launched with work
    uint32_t prop_tile;   // samples per propagate tile this iteration: 32..prop_block (a power of two), or kPropPer x prop_block
    uint32_t prop_block;  // propagate block size
    uint32_t pair_samples;  // iterations with at least this many samples use kPropPer samples per thread
    uint32_t n_sms;         // SMs of the device: smaller iterations use smaller tiles, about one per SM
    uint32_t old_tile;      // old nodes per re-activation tile this iteration: kTileOld or kTileOldSmall
    // samples and tree nodes of the queries still running, summed by this
    // iteration's finalisers for the schedule of the next one
    unsigned long long next_samples;
    unsigned long long next_tree;
    // mapped pinned host word that mirrors `running` (or null): the host polls
    // it without a copy in the stream between graph replays
    uint32_t* host_running;
};

// device-side scratch of the persistent tail launch (kgmt_tail.cuh), one per engine
struct TailScratch {
    uint32_t bar;         // grid-barrier arrivals of the running launch (zeroed before it)
    uint32_t iterations;  // iterations the last launch ran
    uint32_t declined;    // 1: the last launch stopped before an iteration larger than it takes
    uint32_t pad;
    unsigned long long fp32_ops;  // algorithmic FP32 operations of the tail's propagation (host-zeroed)
    unsigned long long samples;   // samples the tail propagated (host-zeroed)
    uint32_t n_next[2][kTailQueries];                 // accepted samples per query, by iteration parity
    uint32_t goal[2][kTailQueries];                   // smallest new goal-ball index per query (~0u: none)
    uint32_t old_cnt[kTailQueries][kTailMaxBlocks];   // re-activated nodes of each block's chunk
    uint32_t acc_cnt[kTailQueries][kTailMaxBlocks];   // accepted samples of each block's chunk
    uint32_t rep_cnt[kTailQueries][kTailMaxBlocks];   // frontier entries (repeats) of each block's chunk
};

}  // namespace kgmt
