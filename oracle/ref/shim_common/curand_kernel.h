/* Host stand-in for curand_kernel.h used only when the reference's device
 * functions are compiled on the CPU to produce golden vectors: each
 * curand_uniform() call returns the next value of a caller-supplied list, so
 * the reference consumes exactly the uniforms the oracle and the CUDA planner
 * draw from Philox. */
#pragma once
struct curandState {
    const float* u;
    int i;
};
typedef struct curandState curandState;
static inline float curand_uniform(curandState* s) { return s->u[s->i++]; }
