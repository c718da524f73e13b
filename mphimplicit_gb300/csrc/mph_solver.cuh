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
enum { kFlagDone = 0, kFlagIter = 1, kFlagCap = 2, kFlagBad = 3, kFlagCounter = 4, kFlagOuter = 5, kFlagCount = 8 };

constexpr int kReduceBlocks = 1216;   // 152 SMs x 8 blocks: bound on the partials count
constexpr int kGraphChunk = 8;        // CR iterations per captured graph chunk (FP64 form; the mixed form's option "chunk")
constexpr int kMaxGraphChunk = 32;
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

// A block's sum of per-thread FP32 values: FP32 within each warp (five more
// roundings of terms that are FP32 sums already), FP64 across the warps.  An
// FP64 shuffle tree in every warp took a visible share of the short CR
// kernels: FP64 issues at a small fraction of the FP32 rate on this part.
__device__ __forceinline__ double block_sum(float v)
{
    __shared__ double wsf[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) wsf[wid] = (double)v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double d = (threadIdx.x < nw) ? wsf[threadIdx.x] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    }
    return d;   // valid in thread 0
}

// Store this block's partial; the last block reduces all partials in block
// order into *out.  Every thread of every block must call it.  lb / nb: the
// block's index and the block count of its reduction (a launch's own, or one
// case's share of a launch over several cases).
// T: double, or float for per-thread FP32 sums (FP32 warp stage)
template <typename T>
__device__ __forceinline__ void reduce_finalize(T v, double* __restrict__ partials, unsigned* __restrict__ counter,
                                                double* __restrict__ out, int lb, int nb)
{
    __shared__ bool last;
    const double bs = block_sum(v);
    if (threadIdx.x == 0) {
        partials[lb] = bs;
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == (unsigned)nb - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += ((volatile double*)partials)[b];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        *out = s;
        *counter = 0u;
    }
}
template <typename T>
__device__ __forceinline__ void reduce_finalize(T v, double* __restrict__ partials, unsigned* __restrict__ counter,
                                                double* __restrict__ out)
{
    reduce_finalize(v, partials, counter, out, (int)blockIdx.x, (int)gridDim.x);
}

// As reduce_finalize; the last block also advances the device iteration
// counter *it (every block read it before taking its ticket).  Returns true
// in thread 0 of the last block, after the stores.
template <typename T>
__device__ __forceinline__ bool reduce_finalize_step(T v, double* __restrict__ partials, unsigned* __restrict__ counter,
                                                     double* __restrict__ out, int* __restrict__ it, int lb, int nb)
{
    __shared__ bool last;
    const double bs = block_sum(v);
    if (threadIdx.x == 0) {
        partials[lb] = bs;
        __threadfence();
        const unsigned ticket = atomicAdd(counter, 1u);
        last = (ticket == (unsigned)nb - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += ((volatile double*)partials)[b];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        *out = s;
        *counter = 0u;
        *it = *it + 1;
    }
    return threadIdx.x == 0;
}
template <typename T>
__device__ __forceinline__ bool reduce_finalize_step(T v, double* __restrict__ partials, unsigned* __restrict__ counter,
                                                     double* __restrict__ out, int* __restrict__ it)
{
    return reduce_finalize_step(v, partials, counter, out, it, (int)blockIdx.x, (int)gridDim.x);
}

// The case of launch block b: the last case whose first block is <= b (b0:
// ncases + 1 block starts; a case without blocks is never found).
__device__ __forceinline__ int batch_case_of(const int* __restrict__ b0, int ncases, int b)
{
    int lo = 0, hi = ncases - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b0[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Capture `body` (a fixed launch sequence on c->stream) into a CUDA graph and
// update or instantiate *exec with it; the graph is later launched on
// c->stream.  The capture records on the case's own side stream (c->stream
// may be the legacy stream, which cannot be captured): c->stream points
// there while `body` runs.  Returns the number of kernel launches the
// sequence contains in *launches.
//
// Every argument of the captured launches derives from the case's device
// buffers, parameters, level geometry and the given scalars, so a hash of
// those identifies the graph: when it matches the one *exec was made from,
// the capture is skipped (*launches is kept from that capture).
inline unsigned long long fnv1a(unsigned long long h, const void* p, size_t n)
{
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t k = 0; k < n; ++k) h = (h ^ b[k]) * 1099511628211ull;
    return h;
}

// (The slot total of a step changes every step but is no argument of a
// captured kernel, which read the slices through their pointers: it is left
// out so that a case's graphs are replayed from step to step.)
inline unsigned long long graph_signature(const mph_case* c, double tol, int cap)
{
    unsigned long long h = 1469598103934665603ull;
    // the particle arrays swap with their alternates every step and no
    // captured kernel reads them
    DeviceState d = c->d;
    d.pos = d.vel = d.force = d.pos_alt = d.vel_alt = nullptr;
    d.pos32 = nullptr;
    d.id = d.id_alt = d.type_alt = d.type = nullptr;
    d.vprev = d.vprev_alt = nullptr;
    h = fnv1a(h, &d, sizeof(d));
    h = fnv1a(h, &c->dp, sizeof(c->dp));
    if (!c->lv.empty()) h = fnv1a(h, c->lv.data(), c->lv.size() * sizeof(c->lv[0]));
    const long long misc[] = {c->depth, c->nslices, c->precision, c->step_factored, c->step_pairs, c->loc_smem, c->loc_ct_smem, c->prof.on, c->mixed_extra_sweeps, c->dense_level, c->pair_block, c->ct_block, c->chunk, c->mg_pre, c->mg_post, c->mg_depth, c->mg_coarsest, c->pair_recompute, c->pair_pack, c->pair_fuse, c->split_apply, c->fork_stream != nullptr, c->loc_cap,
                              cap, c->mg_rows_total, c->mg_cof_total};
    h = fnv1a(h, misc, sizeof(misc));
    h = fnv1a(h, &tol, sizeof(tol));
    return h;
}

template <typename F>
int capture_graph(mph_case* c, cudaGraphExec_t* exec, unsigned long long* sig_slot, unsigned long long sig, F&& body,
                  long long* launches)
{
    if (*exec && *sig_slot == sig) return MPH_OK;   // same graph as the last capture
    if (!c->cap_stream) MPH_CUDA(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    const long long l0 = t_launch_count;
    cudaGraph_t graph = nullptr;
    MPH_CUDA(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    cudaStream_t saved = c->stream;
    c->stream = c->cap_stream;
    body();
    c->stream = saved;
    const cudaError_t ec = cudaStreamEndCapture(c->cap_stream, &graph);
    *launches = t_launch_count - l0;
    t_launch_count = l0;
    g_launch_count -= *launches;
    if (ec != cudaSuccess) return cuda_check(ec, "cudaStreamEndCapture");
    bool ok = false;
    if (*exec) {
        cudaGraphExecUpdateResultInfo info;
        ok = cudaGraphExecUpdate(*exec, graph, &info) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            cudaGraphExecDestroy(*exec);
            *exec = nullptr;
        }
    }
    if (!ok) {
        const cudaError_t ei = cudaGraphInstantiate(exec, graph, 0);
        if (ei != cudaSuccess) {
            cudaGraphDestroy(graph);
            return cuda_check(ei, "cudaGraphInstantiate");
        }
    }
    cudaGraphDestroy(graph);
    *sig_slot = sig;
    return MPH_OK;
}

void vcycle_fp64(mph_case* c, const double* q, double* u, double* dot_out);
void vcycle_mixed(mph_case* c, const float* q, float* u, double* dot_out);

}  // namespace mph
