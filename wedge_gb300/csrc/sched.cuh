// The scheduler network: 16 features -> 64 -> 64 -> 3 (ReLU, FP32), whose
// outputs are predicted log2 costs (microseconds) of the three pull strategies
// (dense, Wedge, source-filtered) of the next iteration.  This file holds the
// blob layout and the forward pass one thread block runs for one sample; the
// engine evaluates it on the device after every pull (decide_kernel), and the
// training kernels in sched.cu run the same arithmetic in the same order.
// The network has no counterpart in the reference; its fallback, the plain
// fixed-threshold rule, is the reference's (execution_bfs.c:132,141).
#pragma once

#include "wedge_cuda.h"

namespace wedge {

constexpr int NF = WEDGE_SCHED_FEATURES;
constexpr int NH = WEDGE_SCHED_HIDDEN;
constexpr int NO = WEDGE_SCHED_OUTPUTS;
constexpr int OFF_MU = 0;
constexpr int OFF_SD = NF;
constexpr int OFF_LO = 2 * NF;
constexpr int OFF_HI = 3 * NF;
constexpr int OFF_W1 = WEDGE_SCHED_PARAM_OFFSET; /* [NH][NF] */
constexpr int OFF_B1 = OFF_W1 + NH * NF;
constexpr int OFF_W2 = OFF_B1 + NH; /* [NH][NH] */
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH; /* [NO][NH] */
constexpr int OFF_B3 = OFF_W3 + NO * NH;
constexpr int OFF_MARGIN = OFF_B3 + NO;
static_assert(OFF_W1 == 4 * NF, "statistics precede the parameters");
static_assert(OFF_MARGIN - OFF_W1 == WEDGE_SCHED_PARAMS, "parameter count");
static_assert(OFF_MARGIN + 1 == WEDGE_SCHED_BLOB, "blob size");

// Forward pass of one sample by the threads of a block (blockDim.x >= NH).
// raw[NF]: features (shared memory); xs[NF], h1[NH], h2[NH], out[NO]: shared
// scratch.  Every sum runs in index order with explicit fused multiply-adds,
// as in the training kernels.  Ends with the outputs visible to the block.
__device__ __forceinline__ void sched_forward_block(const float* __restrict__ net, const float* raw, float* xs,
                                                    float* h1, float* h2, float* out)
{
    const int t = threadIdx.x;
    if (t < NF)
        xs[t] = (raw[t] - net[OFF_MU + t]) / net[OFF_SD + t];
    __syncthreads();
    if (t < NH) {
        float a = net[OFF_B1 + t];
        for (int i = 0; i < NF; ++i)
            a = __fmaf_rn(net[OFF_W1 + t * NF + i], xs[i], a);
        h1[t] = fmaxf(a, 0.0f);
    }
    __syncthreads();
    if (t < NH) {
        float a = net[OFF_B2 + t];
        for (int j = 0; j < NH; ++j)
            a = __fmaf_rn(net[OFF_W2 + t * NH + j], h1[j], a);
        h2[t] = fmaxf(a, 0.0f);
    }
    __syncthreads();
    if (t < NO) {
        float a = net[OFF_B3 + t];
        for (int k = 0; k < NH; ++k)
            a = __fmaf_rn(net[OFF_W3 + t * NH + k], h2[k], a);
        out[t] = a;
    }
    __syncthreads();
}

}  // namespace wedge
