// k_resid_noalloc.cu - residual norms of a solved system, with no device
// allocation by the call.
//
// mph_residual_noalloc reports ||b - A x||^2 and ||b||^2 of the system that a
// case's last solve worked on (A, b and the solution x stay resident after
// mph_stage_solve).  The arithmetic is that of the mixed solver's residual
// kernel k_resid64 (same rows per block, same summation order), but the
// reduction's block partials and its ticket live in one fixed file-scope
// device array instead of buffers sized for the case, and the residual vector
// itself is not stored.
//
// Callers this is for: a multi-case server that admits cases until device
// memory is committed has no room for a per-call buffer, so an allocation
// can fail exactly when the check is wanted (for instance right after another
// case ran out of memory); and cudaFree waits for the whole device, so a
// per-call buffer would stall the streams of every other resident case.
//
// When the array exists: this file is its own CUDA module, and with CUDA's
// default lazy module loading a module (with its __device__ arrays) is loaded
// on a device only when something in it is first used there.  So
// noalloc_prepare, called by mph_case_create on the case's device before the
// case allocates anything, looks up the array's address (which loads the
// module and reserves the array) and loads the kernel code; every later check
// on that device then needs no device memory at all, and no check has to
// come before a stream capture.
//
// Limits and rules:
//   - at most kNoAllocMaxBlocks blocks of 128 rows, i.e. 2,097,152 fluid
//     particles; larger cases are rejected with MPH_ERR_CAPACITY;
//   - one array per device serves every case: calls that overlap on the GPU
//     (other streams, other host threads) race on it and must be serialised
//     by the caller;
//   - the address is cached per device for the life of the process: the
//     check must not be used across a cudaDeviceReset (or any reset of the
//     device's primary context), which frees the array.
#include <mutex>

#include "mph_internal.h"
#include "mph_solver.cuh"

namespace mph {
namespace {

constexpr int kNoAllocRows = 128;                 // rows per block, as k_resid64
constexpr int kNoAllocMaxBlocks = 16384;          // 2,097,152 rows
constexpr int kNoAllocTail = 32;                  // results [2] + ticket, in doubles
constexpr int kMaxDevices = 64;

// [0, B): block partials of (r,r); [B, 2B): of (b,b); then the two results
// and the ticket counter.  262,400 bytes.
static __device__ __align__(256) double g_resid_scratch[2 * kNoAllocMaxBlocks + kNoAllocTail];

std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};

template <int D>
__global__ void __launch_bounds__(kNoAllocRows) k_resid_norms(int Nf, const int* __restrict__ nfc,
                                                              const long long* __restrict__ sptr,
                                                              const int* __restrict__ acol, const double* __restrict__ aval,
                                                              const double* __restrict__ x, const double* __restrict__ b,
                                                              double* __restrict__ scratch)
{
    constexpr int DD = D * D;
    double* part_rr = scratch;
    double* part_bb = scratch + kNoAllocMaxBlocks;
    double* result = scratch + 2 * kNoAllocMaxBlocks;
    unsigned* ticket = (unsigned*)(result + 2);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0, accb = 0.0;
    if (i < Nf) {
        const int lane = i & 31;
        const long long base = sptr[i >> 5];
        const int* cp = acol + base + lane;
        const double* vp = aval + base * DD + lane;
        double y[3] = {0.0, 0.0, 0.0};
        const int n = nfc[i];
#pragma unroll 2
        for (int k = 0; k < n; ++k) {
            const int col = cp[(long long)k * 32];
            double xv[3];
#pragma unroll
            for (int s = 0; s < D; ++s) xv[s] = x[(size_t)col * D + s];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) y[r] += vp[((long long)k * DD + r * D + s) * 32] * xv[s];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const double bk = b[(size_t)i * D + r];
            const double v = bk - y[r];
            acc += v * v;
            accb += bk * bk;
        }
    }
    // block sums, then the last block (ticket) adds the partials in block order
    __shared__ bool last;
    const double s_rr = block_sum(acc);
    const double s_bb = block_sum(accb);
    if (threadIdx.x == 0) {
        part_rr[blockIdx.x] = s_rr;
        part_bb[blockIdx.x] = s_bb;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t_rr = 0.0, t_bb = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
        t_rr += ((volatile double*)part_rr)[k];
        t_bb += ((volatile double*)part_bb)[k];
    }
    t_rr = block_sum(t_rr);
    t_bb = block_sum(t_bb);
    if (threadIdx.x == 0) {
        result[0] = t_rr;
        result[1] = t_bb;
    }
}

// Device address of the scratch array for device `dev` (which is current);
// looked up once per device (first case creation on it).
int scratch_for_device(int dev, double** out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail(MPH_ERR_CAPACITY, "device ordinal beyond the allocation-free residual's table");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_resid_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_resid_scratch)");
        g_scratch_ptr[dev] = (double*)p;
    }
    *out = g_scratch_ptr[dev];
    return MPH_OK;
}

int residual_noalloc(mph_case* c, double* out)
{
    if (!c || !out) return fail(MPH_ERR_ARG, "null argument");
    const int Nf = c->dp.Nf;
    const long long blocks = ((long long)Nf + kNoAllocRows - 1) / kNoAllocRows;
    if (blocks > kNoAllocMaxBlocks)
        return fail(MPH_ERR_CAPACITY, "allocation-free residual: " + std::to_string(Nf) + " fluid particles exceed its limit of " +
                                          std::to_string((long long)kNoAllocMaxBlocks * kNoAllocRows));
    if (c->stage != 7) return fail(MPH_ERR_STATE, "allocation-free residual: call it after mph_stage_solve, before the step ends");
    if (c->step_factored)
        return fail(MPH_ERR_STATE, "allocation-free residual: this step has no FP64 blocks (mixed form with the factored "
                                   "operator; set option \"factored\" to 0)");
    int prev = 0;
    MPH_CUDA(cudaGetDevice(&prev));
    if (prev != c->device) MPH_CUDA(cudaSetDevice(c->device));
    double* scratch = nullptr;
    int st = scratch_for_device(c->device, &scratch);
    if (st == MPH_OK) {
        double* result = scratch + 2 * kNoAllocMaxBlocks;
        cudaError_t e = cudaMemsetAsync(result, 0, kNoAllocTail * sizeof(double), c->stream);   // results and ticket start at 0
        if (e == cudaSuccess && blocks > 0) {
            const DeviceState& d = c->d;
            if (c->dim == 2)
                k_resid_norms<2><<<(unsigned)blocks, kNoAllocRows, 0, c->stream>>>(Nf, d.nfc, d.sptr, d.acol, d.aval, d.x, d.bvec, scratch);
            else
                k_resid_norms<3><<<(unsigned)blocks, kNoAllocRows, 0, c->stream>>>(Nf, d.nfc, d.sptr, d.acol, d.aval, d.x, d.bvec, scratch);
            MPH_COUNT_LAUNCH();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, result, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_check(e, "allocation-free residual");
    }
    if (prev != c->device) cudaSetDevice(prev);
    return st;
}

}  // namespace

// Called by case creation with the case's device current, before the case
// allocates: resolves the array's address and loads both kernel variants, so
// the module's memory is taken while memory is still free.
int noalloc_prepare(int dev)
{
    double* p = nullptr;
    MPH_TRY(scratch_for_device(dev, &p));
    cudaFuncAttributes a;
    MPH_CUDA(cudaFuncGetAttributes(&a, k_resid_norms<2>));
    MPH_CUDA(cudaFuncGetAttributes(&a, k_resid_norms<3>));
    return MPH_OK;
}

}  // namespace mph

extern "C" int mph_residual_noalloc(mph_case* c, double* out)
{
    try {
        return mph::residual_noalloc(c, out);
    } catch (...) {
        return mph::fail(MPH_ERR_STATE, "allocation-free residual: unexpected exception");
    }
}
