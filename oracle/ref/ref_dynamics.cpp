/* Golden-vector harness: exposes the reference's own propagation and
 * collision functions (src/statePropagator/statePropagator.cu,
 * src/collisionCheck/collisionCheck.cu), compiled for the host by
 * oracle/ref/Makefile, through a C ABI.  The uniforms every curand_uniform()
 * call returns are passed in by the caller (shim_common/curand_kernel.h). */
#include "statePropagator/statePropagator.cuh"

extern "C" int ref_model(void) { return MODEL; }
extern "C" int ref_sample_dim(void) { return SAMPLE_DIM; }

/* statePropagator.cu:4-8 dispatch -> model function; returns the verdict */
extern "C" int ref_propagate(const float* x0, const float* u, const float* obstacles, int n_obs, float* x1)
{
    curandState st;
    st.u = u;
    st.i = 0;
    float a[SAMPLE_DIM];
    for(int i = 0; i < SAMPLE_DIM; ++i) a[i] = x0[i];
    return propagateAndCheck(a, x1, &st, const_cast<float*>(obstacles), n_obs) ? 1 : 0;
}

/* collisionCheck.cu:49-61 for one segment, box built as in
 * statePropagator.cu:121-133 */
extern "C" int ref_motion_valid(const float* p0, const float* p1, const float* obstacles, int n_obs)
{
    float a[W_DIM], b[W_DIM], bbMin[W_DIM], bbMax[W_DIM];
    for(int d = 0; d < W_DIM; ++d)
        {
            a[d] = p0[d];
            b[d] = p1[d];
            if(a[d] > b[d]) bbMin[d] = b[d], bbMax[d] = a[d];
            else bbMin[d] = a[d], bbMax[d] = b[d];
        }
    return isMotionValid(a, b, bbMin, bbMax, const_cast<float*>(obstacles), n_obs) ? 1 : 0;
}
