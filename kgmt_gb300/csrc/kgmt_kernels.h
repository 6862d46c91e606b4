// kgmt_kernels.h -- host-side launch wrappers of the kernel chain.
#pragma once
#include <cuda_runtime.h>

#include "kgmt_types.h"

namespace kgmt {

struct LaunchArgs {
    const QueryParams* params;
    QueryState* states;
    Sched* sched;
    uint32_t* tile_a_base;  // [slots + 1]
    uint32_t* tile_c_base;  // [slots + 1]
    uint32_t* tile_c_old;   // [slots]
};

// admits slots [first, first + count), or slots[0 .. count) (device memory) when given
cudaError_t launch_admit(const LaunchArgs& a, uint32_t first, uint32_t count, cudaStream_t s, const uint32_t* slots = nullptr);
cudaError_t launch_schedule(const LaunchArgs& a, cudaStream_t s);
// models: bit 0 double integrator, bit 1 quadrotor (the mix the launch may meet)
// smem_boxes: boxes a block stages in shared memory (the largest query of the
// launch, rounded by smem_boxes_for); more are read from global memory
cudaError_t launch_propagate(const LaunchArgs& a, int block, int models, int grid, uint32_t smem_boxes, cudaStream_t s);
cudaError_t launch_append(const LaunchArgs& a, int grid, cudaStream_t s);
cudaError_t launch_paths(const LaunchArgs& a, uint32_t n, cudaStream_t s);
// src: rows of 2 * ws_dims floats (min corner, max corner)
cudaError_t launch_stage_obstacles(const float* src, float4* dst, uint32_t n, int ws_dims, cudaStream_t s);
// KGMT_CHECK_BOUNDS builds: the index-check error bits since the last call
// (then cleared); always 0 in other builds
uint32_t bounds_error_take();
// one warp waiting on a look-back word nothing sets, for at most `polls` polls
cudaError_t launch_selftest_wait(unsigned long long* tiles, uint32_t* error, uint32_t polls, cudaStream_t s);
cudaError_t launch_propagate_samples(const QueryParams& p, const float* x0, const float* u, const float* obs, uint32_t n_obs, uint32_t n,
                                     float* x1, uint8_t* valid, int32_t* r1, int32_t* r2, cudaStream_t s);
int propagate_blocks_per_sm(int block, int models);
int append_blocks_per_sm();

// persistent tail launch (kgmt_tail.cuh): whole iterations for at most
// kTailQueries running queries in one cooperative launch of `grid` blocks;
// stops before an iteration of more than max_samples samples.  host_words
// (mapped, or null): [0] iterations run, [1] 1 if it stopped for size.
size_t tail_scratch_bytes();
// blocks of the tail kernel one SM holds (0: it cannot run)
int tail_blocks_per_sm(int models);
cudaError_t launch_tail(const LaunchArgs& a, TailScratch* ts, int models, int grid, uint32_t smem_boxes, uint32_t max_samples,
                        uint32_t* host_words, cudaStream_t s);

}  // namespace kgmt
