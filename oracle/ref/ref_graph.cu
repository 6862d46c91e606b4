/* Golden-vector harness: the reference's host-callable getRegion
 * (src/graphs/Graph.cu:99-153) through a C ABI.  Runs on the CPU; no kernel is
 * launched. */
#include "graphs/Graph.cuh"

extern "C" int ref_get_region(const float* x)
{
    float c[SAMPLE_DIM];
    for(int i = 0; i < SAMPLE_DIM; ++i) c[i] = x[i];
    return getRegion(c);
}
extern "C" int ref_num_r1(void) { return NUM_R1_REGIONS; }
