// mph_solver.cuh - device-side scalar bookkeeping of the CR solve.
//
// Dot products are reduced deterministically: every block writes its partial
// sum, and the last block to finish (atomic ticket) adds the partials in block
// order and stores the scalar.  The solver's scalars (rr0, rr, rho, ...) and
// its flags (converged, iteration count) live in device memory, so an
// iteration never waits for the host; the host polls the flags every few
// iterations.
#pragma once

#include "mph_device.cuh"

namespace mph {

// scalar slots (double)
enum {
    kSRR0 = 0, kSRR = 1, kSRS0 = 2, kSRS = 3, kSRho = 4, kSRhop = 5, kSQU = 6, kSBB = 7,
    kSOuterRes = 8, kSOuterRes0 = 9, kSScalarCount = 16
};
// int flag slots
enum { kFlagDone = 0, kFlagIter = 1, kFlagCap = 2, kFlagBad = 3, kFlagCounter = 4, kFlagCount = 8 };

constexpr int kReduceBlocks = 1216;   // 152 SMs x 8 blocks: bound on the partials count
constexpr int kReduceThreads = 256;

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double ws[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) ws[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? ws[threadIdx.x] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;   // valid in thread 0
}

// Store this block's partial; the last block reduces all partials in block
// order into *out.  Every thread of every block must call it.
__device__ __forceinline__ void reduce_finalize(double v, double* __restrict__ partials, unsigned* __restrict__ counter,
                                                double* __restrict__ out)
{
    __shared__ bool last;
    const double bs = block_sum(v);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += ((volatile double*)partials)[b];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        *out = s;
        *counter = 0u;
    }
}

void vcycle_fp64(mph_case* c, const double* q, double* u, double* dot_out);
void vcycle_mixed(mph_case* c, const float* q, float* u, double* dot_out);

}  // namespace mph
