// k_mixed.cu - mixed-precision solve of the step's system: FP32 conjugate
// residual preconditioned by point Jacobi (option mg_depth -1, the default)
// or the FP32 V-cycle, with the FP64 residual replacing the recursive one at
// every refinement step.
//
//   x = v* - F/m dt ; r = b - A x                 (FP64, as the reference)
//   r32 = r / ||r_0|| ; s = M r32                  (one scale for the whole solve)
//   CR iterations in FP32 (FP64 dot products) until (r32, r32) has dropped by
//   tol_inner^2 since the last replacement; then
//       x += ||r_0|| z ; r = b - A x ; rr = (r,r)  (FP64)
//       stop if rr/rr0 < tol_outer^2 (rr0 = (b,b)), else replace r32, s = M r32
//       and go on with the same search directions and iteration count
//   v = x
//
// FP64 on the device is confined to the outer residual b - A x, the solution
// update and the dot products / norms, which also carry both convergence
// tests.  The CR recurrences are the reference's (main.cpp:4344-4377).  The
// default outer tolerance is the reference's ||r||/||b|| < 1e-6;
// mph_case_set_solver tightens it (e.g. 1e-10).
#include <algorithm>

#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

bool mixed_available() { return true; }

__host__ __device__ __forceinline__ int rho32_slot(int it) { return 20 + (it & 1); }
enum { kSIn0 = 16, kSIn = 17, kSQU32 = 18, kSTol2 = 23, kSScale = 24 };   // kSTol2: this phase's inner target
constexpr int kDeviceLoopMax = 100000;   // bound on the device-driven solve's inner iterations
constexpr int kVcycleEvents = 2 * kMaxGraphChunk;   // gev: operator pairs first, then preconditioner pairs

template <int D, int MODE, typename V>
__global__ void __launch_bounds__(128) k_spmv32(int Nf, const int* __restrict__ nfc, const long long* __restrict__ sptr,
                                                const int* __restrict__ acol, const float* __restrict__ aval,
                                                const V* __restrict__ xin, V* __restrict__ yout,
                                                double* __restrict__ scal, int* __restrict__ flags, int cap,
                                                double* __restrict__ partials, unsigned* __restrict__ counter)
{
    constexpr int DD = D * D;
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    const double tol2 = scal[kSTol2];
    const double rr0 = scal[kSIn0];
    const double rr = it == 0 ? rr0 : scal[kSIn];   // the inner solve starts from z = 0: r_in = r32
    const bool bad = !(rr == rr);
    if (it >= cap || rr / rr0 < tol2 || bad) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            flags[kFlagDone] = 1;
            if (bad) flags[kFlagBad] = 1;
        }
        return;
    }
    double* out = scal + rho32_slot(it);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (i < Nf) {
        const int lane = i & 31;
        const long long base = sptr[i >> 5];
        const int* cp = acol + base + lane;
        const float* vp = aval + base * DD + lane;
        float y[3] = {0.f, 0.f, 0.f};
        const int n = nfc[i];
#pragma unroll 4
        for (int k = 0; k < n; ++k) {
            // the blocks stream through once (evict-first), leaving L1 to the x gathers
            const int col = __ldcs(cp + (long long)k * 32);
            float xv[3];
#pragma unroll
            for (int s = 0; s < D; ++s) xv[s] = (float)xin[(size_t)col * D + s];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) y[r] += __ldcs(vp + ((long long)k * DD + r * D + s) * 32) * xv[s];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const size_t k = (size_t)i * D + r;
            yout[k] = (V)y[r];
            acc += (double)xin[k] * (double)y[r];
        }
    }
    (void)MODE;
    reduce_finalize(acc, partials, counter, out);
}

template <typename V>
__global__ void k_pq32(int n, const V* __restrict__ s, const V* __restrict__ y, V* __restrict__ p,
                       V* __restrict__ q, const double* __restrict__ scal, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    if (it == 0) {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            p[k] = s[k];
            q[k] = y[k];
        }
        return;
    }
    const V beta = (V)(scal[rho32_slot(it)] / scal[rho32_slot(it - 1)]);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        p[k] = beta * p[k] + s[k];
        q[k] = beta * q[k] + y[k];
    }
}

// The same update fused with the point-Jacobi preconditioner of the mixed
// form: u = D^-1 q and (q, u) -> kSQU32 in the same pass.
template <typename V>
__device__ __forceinline__ void pq_jacobi32_body(int lb, int nb, int n, const V* __restrict__ s, const V* __restrict__ y, V* __restrict__ p, V* __restrict__ q,
                              const V* __restrict__ invD, V* __restrict__ u, double* __restrict__ scal,
                              const int* __restrict__ flags, double* __restrict__ partials, unsigned* __restrict__ counter)
{
    // the flags and beta once a block, by one thread: an FP64 quotient in
    // every warp took a large share of this short kernel (FP64 issues at a
    // small fraction of the FP32 rate on this part)
    __shared__ int it_s;
    __shared__ V beta_s;
    if (threadIdx.x == 0) {
        const int it0 = flags[kFlagDone] ? -1 : flags[kFlagIter];
        if (it0 > 0) beta_s = (V)(scal[rho32_slot(it0)] / scal[rho32_slot(it0 - 1)]);
        it_s = it0;
    }
    __syncthreads();
    const int it = it_s;
    if (it < 0) return;   // the solve is done (block-uniform)
    const V beta = it == 0 ? (V)0 : beta_s;
    // a thread's few terms (q u = q^2 / d >= 0) and a warp's threads in FP32, the warps in FP64
    float acc = 0.f;
    for (int k = lb * blockDim.x + threadIdx.x; k < n; k += nb * blockDim.x) {
        const V pk = it == 0 ? s[k] : beta * p[k] + s[k];
        const V qk = it == 0 ? y[k] : beta * q[k] + y[k];
        p[k] = pk;
        q[k] = qk;
        const V uk = invD[k] * qk;
        u[k] = uk;
        acc += qk * uk;
    }
    reduce_finalize(acc, partials, counter, scal + kSQU32, lb, nb);
}

template <typename V>
__global__ void k_pq_jacobi32(int n, const V* __restrict__ s, const V* __restrict__ y, V* __restrict__ p, V* __restrict__ q,
                              const V* __restrict__ invD, V* __restrict__ u, double* __restrict__ scal,
                              const int* __restrict__ flags, double* __restrict__ partials, unsigned* __restrict__ counter)
{
    pq_jacobi32_body<V>((int)blockIdx.x, (int)gridDim.x, n, s, y, p, q, invD, u, scal, flags, partials, counter);
}

// z += alpha p, r -= alpha q, s -= alpha u, (r,r) -> kSIn; the last block
// then advances the iteration counter flags[kFlagIter].
// In the device-driven solve (use_cond) the last block also applies the
// next iteration's stop test (the one the operator kernels apply when an
// iteration begins) and sets the inner loop's condition; an iteration that
// found the solve done at its start clears it.
// COND (the device-driven solve only): the variant that sets the loop's
// condition; the host-driven solve's variant holds no device graph call (a
// kernel with one is not profiled by ncu).
template <typename V, bool COND>
__device__ __forceinline__ void xrs32_body(int lb, int nb, int n, V* __restrict__ z, V* __restrict__ r, V* __restrict__ s,
                        const V* __restrict__ p, const V* __restrict__ q, const V* __restrict__ u,
                        double* __restrict__ scal, int* __restrict__ flags, double* __restrict__ partials,
                        unsigned* __restrict__ counter, int cap = 0, int use_cond = 0, cudaGraphConditionalHandle cond = 0)
{
    __shared__ int go_s;   // the flags and alpha once a block, as in pq_jacobi32_body
    __shared__ V alpha_s;
    if (threadIdx.x == 0) {
        const int go = !flags[kFlagDone];
        if (go) alpha_s = (V)(scal[rho32_slot(flags[kFlagIter])] / scal[kSQU32]);
        go_s = go;
    }
    __syncthreads();
    if (!go_s) {   // block-uniform
        if constexpr (COND)
            if (use_cond && lb == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
        return;
    }
    const V alpha = alpha_s;
    float acc = 0.f;   // a thread's few squares and a warp's threads in FP32, the warps in FP64
    for (int k = lb * blockDim.x + threadIdx.x; k < n; k += nb * blockDim.x) {
        z[k] += alpha * p[k];
        const V rk = r[k] - alpha * q[k];
        r[k] = rk;
        s[k] -= alpha * u[k];
        acc += rk * rk;
    }
    const bool last = reduce_finalize_step(acc, partials, counter, scal + kSIn, flags + kFlagIter, lb, nb);
    if constexpr (COND) {
        if (use_cond && last) {
            const int it1 = flags[kFlagIter];
            const double rr = scal[kSIn], rr0 = scal[kSIn0];
            const bool bad = !(rr == rr);
            const bool stop = it1 >= cap || rr / rr0 < scal[kSTol2] || bad;
            if (stop) {
                flags[kFlagDone] = 1;
                if (bad) flags[kFlagBad] = 1;
            }
            cudaGraphSetConditional(cond, stop ? 0u : 1u);
        }
    }
}

template <typename V, bool COND>
__global__ void k_xrs32(int n, V* __restrict__ z, V* __restrict__ r, V* __restrict__ s,
                        const V* __restrict__ p, const V* __restrict__ q, const V* __restrict__ u,
                        double* __restrict__ scal, int* __restrict__ flags, double* __restrict__ partials,
                        unsigned* __restrict__ counter, int cap = 0, int use_cond = 0, cudaGraphConditionalHandle cond = 0)
{
    xrs32_body<V, COND>((int)blockIdx.x, (int)gridDim.x, n, z, r, s, p, q, u, scal, flags, partials, counter, cap, use_cond, cond);
}

// r32 = r * inv_scale, z = 0, and the inner reference norm (r32, r32) -> kSIn0
template <typename V>
__global__ void k_to32(int n, const double* __restrict__ r, V* __restrict__ r32, V* __restrict__ z,
                       double inv_scale, double* __restrict__ scal, double* __restrict__ partials,
                       unsigned* __restrict__ counter, const double* __restrict__ scale_src = nullptr)
{
    const double sc = scale_src ? 1.0 / *scale_src : inv_scale;   // the device-driven solve keeps the scale on the device
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const V v = (V)(r[k] * sc);
        r32[k] = v;
        z[k] = V(0);
        acc += (double)v * (double)v;
    }
    reduce_finalize(acc, partials, counter, scal + kSIn0);
}

// Inner target of the next phase: reduce the recursive residual by tol_in,
// but no further than half of what the outer test still asks for
// (rr / rr0 -> tol_out^2), so the last phase does not overshoot.
__global__ void k_phase_tol(double* __restrict__ scal, double tol_in2, double tol_out2)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double need = 0.25 * tol_out2 * scal[kSRR0] / scal[kSRR];
        scal[kSTol2] = need > tol_in2 ? need : tol_in2;
        scal[kSIn] = scal[kSIn0];
    }
}

// x += scale z  (FP64 update)
template <typename V>
__global__ void k_refine(int n, double* __restrict__ x, const V* __restrict__ z, double scale,
                         const double* __restrict__ scale_src = nullptr, const int* __restrict__ flags = nullptr)
{
    if (flags && flags[kFlagBad]) return;   // the device-driven solve: a phase that met a NaN ends the solve
    const double sc = scale_src ? *scale_src : scale;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) x[k] += sc * (double)z[k];
}

// ---- the device-driven solve: control kernels --------------------------------------
// Before every refinement phase (and once before the first): stop when the
// FP64 residual meets the outer tolerance, is zero or NaN, the refinement
// steps reach max_outer, a phase met a NaN, or the iterations reached their
// cap (after the first phase) - the tests of the host-driven loop - and set
// the outer loop's condition.
__global__ void k_outer_check(double* __restrict__ scal, int* __restrict__ flags, double tol_out2, int max_outer, int cap,
                              cudaGraphConditionalHandle cond)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double rr = scal[kSRR], rr0 = scal[kSRR0];
    const int outer = flags[kFlagOuter];
    const bool nan = !(rr == rr);
    if (nan) flags[kFlagBad] = 1;
    const bool stop = nan || flags[kFlagBad] || rr / rr0 < tol_out2 || outer >= max_outer || rr == 0.0 ||
                      (outer > 0 && flags[kFlagIter] >= cap);
    cudaGraphSetConditional(cond, stop ? 0u : 1u);
}

// Start of a refinement phase: the scale of the FP32 vectors (first phase:
// the initial FP64 residual norm), the done flag cleared (later phases), the
// phase count, and the inner loop's condition set.
__global__ void k_phase_begin(double* __restrict__ scal, int* __restrict__ flags, cudaGraphConditionalHandle inner)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int outer = flags[kFlagOuter];
    if (outer == 0) scal[kSScale] = sqrt(scal[kSRR]);
    else flags[kFlagDone] = 0;
    flags[kFlagOuter] = outer + 1;
    cudaGraphSetConditional(inner, 1u);
}

// r = b - A x in FP64 (the outer residual), (r,r) -> scal[kSRR]
template <int D>
__global__ void __launch_bounds__(128) k_resid64(int Nf, const int* __restrict__ nfc, const long long* __restrict__ sptr,
                                                 const int* __restrict__ acol, const double* __restrict__ aval,
                                                 const double* __restrict__ x, const double* __restrict__ b,
                                                 double* __restrict__ r, double* __restrict__ partials,
                                                 unsigned* __restrict__ counter, double* __restrict__ out)
{
    constexpr int DD = D * D;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
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
            for (int rr = 0; rr < D; ++rr)
#pragma unroll
                for (int s = 0; s < D; ++s) y[rr] += vp[((long long)k * DD + rr * D + s) * 32] * xv[s];
        }
#pragma unroll
        for (int rr = 0; rr < D; ++rr) {
            const size_t k = (size_t)i * D + rr;
            const double v = b[k] - y[rr];
            r[k] = v;
            acc += v * v;
        }
    }
    reduce_finalize(acc, partials, counter, out);
}

template <typename TI, typename TO>
__global__ void k_convert(long long n, const TI* __restrict__ a, TO* __restrict__ b)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        b[k] = (TO)a[k];
}

template <int D>
__global__ void k_store_velocity_m(int Nf, const double* __restrict__ x, double* __restrict__ vel)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Nf * D) return;
    vel[(size_t)(k / D) * (D == 2 ? 2 : 4) + k % D] = x[k];
}

// x0 = v* - F/m dt (= v_n, the reference's start, main.cpp:4299-4308) and
// (b, b) -> *out.  With a history (option "extrapolate", `have` previous
// start velocities in vprev: v_{n-1} at [0, nvs), v_{n-2} at [nvs, 2 nvs)),
// x0 extrapolates the start velocities of the last steps: linearly,
// 2 v_n - v_{n-1}, or quadratically, 3 v_n - 3 v_{n-1} + v_{n-2} (order =
// min(have, maximum order)); the history then shifts by one step.
template <int D>
__global__ void k_x0(int Nf, const int* __restrict__ type, const double* __restrict__ vel, const double* __restrict__ force,
                     const double* __restrict__ b, double* __restrict__ x, DevParams P, double* __restrict__ vprev, size_t nvs,
                     int have, int keep, double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out)
{
    double acc = 0.0;
    const int n = Nf * D;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / D, r = k % D;
        const double m = P.density[type[i]] * P.vol;
        const int VSD = D == 2 ? 2 : 4;
        const size_t a = (size_t)i * VSD + r;
        const double vn = vel[a] - force[a] / m * P.dt;
        double x0 = vn;
        if (vprev) {
            const double v1 = have >= 1 ? vprev[a] : 0.0;
            if (have >= 2) x0 = 3.0 * vn - 3.0 * v1 + vprev[nvs + a];
            else if (have == 1) x0 = 2.0 * vn - v1;
            if (keep >= 2) vprev[nvs + a] = v1;
            vprev[a] = vn;
        }
        x[k] = x0;
        acc += b[k] * b[k];
    }
    reduce_finalize(acc, partials, counter, out);
}

// ---- host side ---------------------------------------------------------------------
static int grow_f(float** p, long long* cap, long long need)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 256;
    MPH_CUDA(cudaMalloc((void**)p, (size_t)n * sizeof(float)));
    *cap = n;
    return MPH_OK;
}

// FP32 copies of the multigrid levels and of D^-1 (after the FP64 build)
int mixed_prepare(mph_case* c)
{
    DeviceState& d = c->d;
    if (c->split_apply && !c->fork_stream) {   // the split operator's side stream (created outside any capture)
        MPH_CUDA(cudaStreamCreateWithFlags(&c->fork_stream, cudaStreamNonBlocking));
        MPH_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        MPH_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    }
    if (mixed_jacobi(c)) {   // point Jacobi: the FP32 D^-1 only
        const long long nv = (long long)c->dp.Nf * c->dim;
        if (!d.v32) MPH_CUDA(cudaMalloc((void**)&d.v32, (size_t)nv * 8 * sizeof(float)));
        c->dense_level = -1;
        { k_convert<double, float><<<grid_for(nv, 256), 256, 0, c->stream>>>(nv, d.invDiag, d.v32 + 7 * nv); MPH_COUNT_LAUNCH(); }
        return MPH_OK;
    }
    MPH_TRY(grow_f(&d.mg_cof32, &d.cap_mg_cof32, c->mg_cof_total));
    if (c->mg_rows_total > d.cap_mg_vec32) {
        for (float** b : {&d.mg_invd32, &d.mg_q32, &d.mg_s32, &d.mg_r32, &d.mg_res32}) {
            if (*b) cudaFree(*b);
            *b = nullptr;
        }
        const long long n = c->mg_rows_total + c->mg_rows_total / 8 + 256;
        for (float** b : {&d.mg_invd32, &d.mg_q32, &d.mg_s32, &d.mg_r32, &d.mg_res32}) MPH_CUDA(cudaMalloc((void**)b, n * sizeof(float)));
        d.cap_mg_vec32 = n;
    }
    const long long nv = (long long)c->dp.Nf * c->dim;
    if (!d.v32) {
        MPH_CUDA(cudaMalloc((void**)&d.v32, (size_t)nv * 8 * sizeof(float)));
    }
    cudaStream_t st = c->stream;
    { k_convert<double, float><<<grid_for(c->mg_cof_total, 256), 256, 0, st>>>(c->mg_cof_total, d.mg_cof, d.mg_cof32); MPH_COUNT_LAUNCH(); }
    { k_convert<double, float><<<grid_for(c->mg_rows_total, 256), 256, 0, st>>>(c->mg_rows_total, d.mg_invd, d.mg_invd32); MPH_COUNT_LAUNCH(); }
    { k_convert<double, float><<<grid_for(nv, 256), 256, 0, st>>>(nv, d.invDiag, d.v32 + 7 * nv); MPH_COUNT_LAUNCH(); }
    return mixed_dense_coarse(c);
}

void vcycle_mixed(mph_case* c, const float* q, float* u, double* dot_out);

// p = beta p + s, q = beta q + y and u = M q with (q, u): the point-Jacobi
// mixed form in one kernel, else the update and the V-cycle
static void pq_precond(mph_case* c, cudaStream_t st, int n, unsigned rb, const float* s32, const float* y32, float* p32,
                       float* q32, float* u32)
{
    DeviceState& d = c->d;
    double* scal = d.scal;
    const int* flags = d.flags;
    if (mixed_jacobi(c)) {
        const float* invD = d.v32 + 7 * (size_t)c->dp.Nf * c->dim;
        { k_pq_jacobi32<float><<<rb, kReduceThreads, 0, st>>>(n, s32, y32, p32, q32, invD, u32, scal, flags, d.partials,
                                                              (unsigned*)(d.flags + kFlagCounter)); MPH_COUNT_LAUNCH(); }
        return;
    }
    { k_pq32<float><<<rb, kReduceThreads, 0, st>>>(n, s32, y32, p32, q32, scal, flags); MPH_COUNT_LAUNCH(); }
    vcycle_mixed(c, q32, u32, scal + kSQU32);
}

static void fill_mixed_stats(mph_case* c, int total_inner, int outer, const double* hs, bool bad, double tol_out2)
{
    c->stats.iterations = total_inner;
    c->stats.rr0 = hs[kSRR0];
    c->stats.rr = hs[kSRR];
    c->stats.rs0 = 0.0;
    c->stats.rs = 0.0;
    c->stats.outer_iterations = outer;
    c->stats.inner_form = c->step_pairs ? 2 : 1;
    c->stats.inner_local_blocks = c->step_pairs ? c->loc_blocks[0] : 0;
    c->stats.inner_gather_blocks = c->step_pairs ? c->loc_blocks[1] : 0;
    c->stats.inner_local_cols = c->step_pairs ? c->loc_cols : 0;
    c->stats.inner_ct_local_blocks = c->step_pairs ? c->loc_ct_blocks : 0;
    c->stats.status = bad ? MPH_ERR_NAN : (hs[kSRR] / hs[kSRR0] < tol_out2 || hs[kSRR] == 0.0 ? MPH_OK : MPH_ERR_NOT_CONVERGED);
}

// A while node on the capturing stream `st` (after its current dependencies),
// its body graph returned; the stream then continues after the node.
static int add_while_node(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraph_t* body)
{
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    MPH_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    MPH_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
    *body = p.conditional.phGraph_out[0];
    MPH_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return MPH_OK;
}

// The device-driven mixed solve: the whole solve (start value, FP64
// residual, refinement phases, FP32 CR iterations, velocity) as one CUDA
// graph whose two loops are conditional while nodes, so a solve is one graph
// launch and one read of its results instead of a host poll every few
// iterations and at every phase.  The same kernels in the same order as the
// host-driven solve (same bits); iterations stop where that solve's
// kernels would have found it done, and the inner loop is bounded by
// kDeviceLoopMax iterations, the outer by max_outer phases.
template <int D>
static int device_solve(mph_case* c, double* hs, int* hflags)
{
    using V = float;
    DeviceState& d = c->d;
    const int Nf = c->dp.Nf;
    const int n = Nf * D;
    double* scal = d.scal;
    int* flags = d.flags;
    unsigned* counter = (unsigned*)(flags + kFlagCounter);
    double* part = d.partials;
    const int rb = std::min<int>(grid_for(n, kReduceThreads), kReduceBlocks);
    const unsigned gs = grid_for(Nf, 128);
    V* vec = d.v32;
    V *r32 = vec, *z32 = vec + (size_t)n, *s32 = vec + 2 * (size_t)n, *y32 = vec + 3 * (size_t)n;
    V *p32 = vec + 4 * (size_t)n, *q32 = vec + 5 * (size_t)n, *u32 = vec + 6 * (size_t)n;
    const double tol_out2 = c->tol_outer * c->tol_outer;
    const double tol_in2 = c->tol_inner * c->tol_inner;
    const int cap = n;
    const int loop_cap = std::min(cap, kDeviceLoopMax);
    const size_t nvs = (size_t)c->dp.N * (D == 2 ? 2 : 4);
    double* vprev = c->extrapolate ? d.vprev : nullptr;
    const int have = std::min(c->prev_valid, c->extrapolate);
    unsigned long long sig = graph_signature(c, tol_in2, cap);
    // unlike the chunk graphs this one reads the particle arrays, which swap
    // with their alternates every step: two graphs serve the two parities
    const long long extra[] = {have, c->max_outer, (long long)(vprev != nullptr), (long long)(uintptr_t)d.vel,
                               (long long)(uintptr_t)d.force, (long long)(uintptr_t)d.type, (long long)(uintptr_t)d.vprev};
    sig = fnv1a(sig, extra, sizeof(extra));
    sig = fnv1a(sig, &tol_out2, sizeof(tol_out2));
    int slot = -1;
    for (int k = 0; k < 2; ++k)
        if (c->sx_exec[k] && c->sx_sig[k] == sig) slot = k;
    if (slot < 0) {
        slot = c->sx_next;   // replace the older of the two
        c->sx_next ^= 1;
        if (c->sx_exec[slot]) {
            cudaGraphExecDestroy(c->sx_exec[slot]);
            c->sx_exec[slot] = nullptr;
        }
        for (cudaStream_t* sp : {&c->cap_stream, &c->cap_stream2, &c->cap_stream3})
            if (!*sp) MPH_CUDA(cudaStreamCreateWithFlags(sp, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        MPH_CUDA(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h_out;
        MPH_CUDA(cudaGraphConditionalHandleCreate(&h_out, g, 0u, 0u));
        const long long l0 = t_launch_count;
        cudaStream_t saved = c->stream;
        int st_ = MPH_OK;
        auto fail_capture = [&](int e) { st_ = e; };
        auto residual = [&]() {
            if (c->step_factored) {
                launch_resid_factored(c, d.x, d.r, scal + kSRR);
            } else {
                k_resid64<D><<<gs, 128, 0, c->stream>>>(Nf, d.nfc, d.sptr, d.acol, d.aval, d.x, d.bvec, d.r, part, counter,
                                                        scal + kSRR);
                MPH_COUNT_LAUNCH();
            }
        };
        // top: start value and first residual, the outer loop, the velocity
        cudaStream_t s1 = c->cap_stream, s2 = c->cap_stream2, s3 = c->cap_stream3;
        MPH_CUDA(cudaStreamBeginCaptureToGraph(s1, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        c->stream = s1;
        cudaMemsetAsync(scal, 0, 32 * sizeof(double), s1);
        cudaMemsetAsync(flags, 0, kFlagCount * sizeof(int), s1);
        { k_x0<D><<<rb, kReduceThreads, 0, s1>>>(Nf, d.type, d.vel, d.force, d.bvec, d.x, c->dp, vprev, nvs, have, c->extrapolate,
                                                 part, counter, scal + kSRR0); MPH_COUNT_LAUNCH(); }
        residual();
        { k_outer_check<<<1, 32, 0, s1>>>(scal, flags, tol_out2, c->max_outer, cap, h_out); MPH_COUNT_LAUNCH(); }
        cudaGraph_t body_out = nullptr;
        int e = add_while_node(s1, h_out, &body_out);
        if (e != MPH_OK) fail_capture(e);
        // outer body: one refinement phase
        cudaGraphConditionalHandle h_in;
        if (st_ == MPH_OK && cudaGraphConditionalHandleCreate(&h_in, body_out, 0u, 0u) != cudaSuccess)
            fail_capture(fail(MPH_ERR_CUDA, "cudaGraphConditionalHandleCreate"));
        if (st_ == MPH_OK && cudaStreamBeginCaptureToGraph(s2, body_out, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            fail_capture(fail(MPH_ERR_CUDA, "capture of the refinement phase"));
        const long long l_phase0 = t_launch_count;
        long long l_iter = 0;
        if (st_ == MPH_OK) {
            c->stream = s2;
            { k_phase_begin<<<1, 32, 0, s2>>>(scal, flags, h_in); MPH_COUNT_LAUNCH(); }
            { k_to32<V><<<rb, kReduceThreads, 0, s2>>>(n, d.r, r32, z32, 1.0, scal, part, counter, scal + kSScale); MPH_COUNT_LAUNCH(); }
            { k_phase_tol<<<1, 32, 0, s2>>>(scal, tol_in2, tol_out2); MPH_COUNT_LAUNCH(); }
            vcycle_mixed(c, r32, s32, scal + kSQU32);   // s = M r
            cudaGraph_t body_in = nullptr;
            e = add_while_node(s2, h_in, &body_in);
            if (e != MPH_OK) fail_capture(e);
            // inner body: one FP32 CR iteration
            if (st_ == MPH_OK && cudaStreamBeginCaptureToGraph(s3, body_in, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                fail_capture(fail(MPH_ERR_CUDA, "capture of the CR iteration"));
            if (st_ == MPH_OK) {
                c->stream = s3;
                const long long li0 = t_launch_count;
                if (c->step_pairs) {
                    launch_apply32(c, s32, y32, cap);
                } else {
                    k_spmv32<D, 1, V><<<gs, 128, 0, s3>>>(Nf, d.nfc, d.sptr, d.acol, d.aval32, s32, y32, scal, flags, cap, part, counter);
                    MPH_COUNT_LAUNCH();
                }
                pq_precond(c, s3, n, rb, s32, y32, p32, q32, u32);
                { k_xrs32<V, true><<<rb, kReduceThreads, 0, s3>>>(n, z32, r32, s32, p32, q32, u32, scal, flags, part, counter, loop_cap,
                                                             1, h_in); MPH_COUNT_LAUNCH(); }
                l_iter = t_launch_count - li0;
                cudaGraph_t gi = nullptr;
                if (cudaStreamEndCapture(s3, &gi) != cudaSuccess) fail_capture(fail(MPH_ERR_CUDA, "end of the CR iteration capture"));
            }
            c->stream = s2;
            { k_refine<V><<<rb, kReduceThreads, 0, s2>>>(n, d.x, z32, 1.0, scal + kSScale, flags); MPH_COUNT_LAUNCH(); }
            residual();
            { k_outer_check<<<1, 32, 0, s2>>>(scal, flags, tol_out2, c->max_outer, cap, h_out); MPH_COUNT_LAUNCH(); }
            cudaGraph_t go = nullptr;
            if (cudaStreamEndCapture(s2, &go) != cudaSuccess) fail_capture(fail(MPH_ERR_CUDA, "end of the phase capture"));
        }
        const long long l_phase = t_launch_count - l_phase0 - l_iter;
        c->stream = s1;
        { k_store_velocity_m<D><<<grid_for(n, 256), 256, 0, s1>>>(Nf, d.x, d.vel); MPH_COUNT_LAUNCH(); }
        cudaGraph_t gt = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s1, &gt);
        c->stream = saved;
        const long long l_all = t_launch_count - l0;
        c->sx_launches[slot][0] = l_all - l_phase - l_iter;   // kernels of the graph's top level, of a phase, of an iteration
        c->sx_launches[slot][1] = l_phase;
        c->sx_launches[slot][2] = l_iter;
        t_launch_count = l0;
        g_launch_count -= l_all;
        if (st_ == MPH_OK && ec != cudaSuccess) st_ = cuda_check(ec, "end of the solve capture");
        if (st_ == MPH_OK) {
            const cudaError_t ei = cudaGraphInstantiate(&c->sx_exec[slot], g, 0);
            if (ei != cudaSuccess) st_ = cuda_check(ei, "cudaGraphInstantiate (solve)");
        }
        cudaGraphDestroy(g);
        if (st_ != MPH_OK) {
            cudaGetLastError();
            c->sx_exec[slot] = nullptr;
            return st_;
        }
        c->sx_sig[slot] = sig;
    }
    c->prev_valid = vprev ? std::min(c->prev_valid + 1, c->extrapolate) : 0;
    MPH_CUDA(cudaGraphLaunch(c->sx_exec[slot], c->stream));
    MPH_CUDA(cudaMemcpyAsync(hs, scal, 32 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(hflags, flags, kFlagCount * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    // the kernels that ran: the top level once, a phase's per refinement
    // phase, an iteration's per CR iteration
    g_launch_count += c->sx_launches[slot][0] + (long long)hflags[kFlagOuter] * c->sx_launches[slot][1] +
                      (long long)hflags[kFlagIter] * c->sx_launches[slot][2];
    return MPH_OK;
}

// The host side of one mixed solve in the parts the single-case solve and
// the batched solve share: the start (start value, FP64 residual), the test
// before each refinement phase and the phase's first kernels, the update and
// FP64 residual after its CR iterations, and the end (velocity, statistics).
// One FP32 CR run; at every refinement step the FP64 residual replaces the
// recursive FP32 one (and s = M r is recomputed), while the search
// directions p, q and the iteration count carry on, so the Krylov space is
// not thrown away.  All FP32 vectors share one scale, fixed at the start.
template <int D>
struct MixedRun {
    using V = float;
    mph_case* c = nullptr;
    int Nf = 0, n = 0, rb = 0, cap = 0;
    unsigned gs = 0;
    double* scal = nullptr;
    double* part = nullptr;
    int* flags = nullptr;
    unsigned* counter = nullptr;
    V *r32 = nullptr, *z32 = nullptr, *s32 = nullptr, *y32 = nullptr, *p32 = nullptr, *q32 = nullptr, *u32 = nullptr;
    double tol_out2 = 0.0, tol_in2 = 0.0, scale = 1.0;
    int outer = 0;
    long long launched = 0;           // CR iterations launched (the runaway bound)
    int host_flags[kFlagCount] = {};
    double hs[32] = {};
    bool bad = false;

    void init(mph_case* c_)
    {
        c = c_;
        DeviceState& d = c->d;
        Nf = c->dp.Nf;
        n = Nf * D;
        scal = d.scal;
        flags = d.flags;
        counter = (unsigned*)(flags + kFlagCounter);
        part = d.partials;
        rb = std::min<int>(grid_for(n, kReduceThreads), kReduceBlocks);
        gs = grid_for(Nf, 128);
        V* vec = d.v32;
        r32 = vec;
        z32 = vec + (size_t)n;
        s32 = vec + 2 * (size_t)n;
        y32 = vec + 3 * (size_t)n;
        p32 = vec + 4 * (size_t)n;
        q32 = vec + 5 * (size_t)n;
        u32 = vec + 6 * (size_t)n;
        tol_out2 = c->tol_outer * c->tol_outer;
        tol_in2 = c->tol_inner * c->tol_inner;
        cap = n;
    }

    // FP64 residual: from the assembled FP64 blocks, or in factored form
    void residual()
    {
        DeviceState& d = c->d;
        if (c->step_factored) {
            launch_resid_factored(c, d.x, d.r, scal + kSRR);
        } else {
            k_resid64<D><<<gs, 128, 0, c->stream>>>(Nf, d.nfc, d.sptr, d.acol, d.aval, d.x, d.bvec, d.r, part, counter, scal + kSRR);
            MPH_COUNT_LAUNCH();
        }
    }

    int start()
    {
        DeviceState& d = c->d;
        cudaStream_t st = c->stream;
        MPH_CUDA(cudaMemsetAsync(scal, 0, 32 * sizeof(double), st));
        MPH_CUDA(cudaMemsetAsync(flags, 0, kFlagCount * sizeof(int), st));
        const size_t nvs = (size_t)c->dp.N * (D == 2 ? 2 : 4);
        if (c->extrapolate && !d.vprev) {
            MPH_CUDA(cudaMalloc((void**)&d.vprev, 2 * nvs * sizeof(double)));
            MPH_CUDA(cudaMalloc((void**)&d.vprev_alt, 2 * nvs * sizeof(double)));
            c->prev_valid = 0;
        }
        double* vprev = c->extrapolate ? d.vprev : nullptr;
        const int have = std::min(c->prev_valid, c->extrapolate);
        { k_x0<D><<<rb, kReduceThreads, 0, st>>>(Nf, d.type, d.vel, d.force, d.bvec, d.x, c->dp, vprev, nvs, have, c->extrapolate,
                                                 part, counter, scal + kSRR0); MPH_COUNT_LAUNCH(); }
        c->prev_valid = vprev ? std::min(c->prev_valid + 1, c->extrapolate) : 0;
        residual();
        return MPH_OK;
    }

    // The test before a refinement phase (reads the solve's state: syncs the
    // case stream).  *go: a phase follows, its first kernels launched.
    int phase(bool* go)
    {
        *go = false;
        cudaStream_t st = c->stream;
        MPH_CUDA(cudaMemcpyAsync(hs, scal, sizeof(hs), cudaMemcpyDeviceToHost, st));
        MPH_CUDA(cudaMemcpyAsync(host_flags, flags, sizeof(host_flags), cudaMemcpyDeviceToHost, st));
        MPH_CUDA(cudaStreamSynchronize(st));
        if (!(hs[kSRR] == hs[kSRR])) {
            bad = true;
            return MPH_OK;
        }
        if (hs[kSRR] / hs[kSRR0] < tol_out2 || outer >= c->max_outer || hs[kSRR] == 0.0) return MPH_OK;
        if (outer > 0 && host_flags[kFlagIter] >= cap) return MPH_OK;
        if (outer == 0) scale = std::sqrt(hs[kSRR]);
        else MPH_CUDA(cudaMemsetAsync(flags + kFlagDone, 0, sizeof(int), st));
        ++outer;
        { k_to32<V><<<rb, kReduceThreads, 0, st>>>(n, c->d.r, r32, z32, 1.0 / scale, scal, part, counter); MPH_COUNT_LAUNCH(); }
        { k_phase_tol<<<1, 32, 0, st>>>(scal, tol_in2, tol_out2); MPH_COUNT_LAUNCH(); }
        vcycle_mixed(c, r32, s32, scal + kSQU32);   // s = M r
        *go = true;
        return MPH_OK;
    }

    // After a phase's CR iterations (host_flags read after them): a bad
    // solve stops; else x += scale z and the FP64 residual.
    int refine(bool* go)
    {
        *go = false;
        if (host_flags[kFlagBad]) {
            bad = true;
            return MPH_OK;
        }
        { k_refine<V><<<rb, kReduceThreads, 0, c->stream>>>(n, c->d.x, z32, scale); MPH_COUNT_LAUNCH(); }
        residual();
        *go = true;
        return MPH_OK;
    }

    int finish()
    {
        cudaStream_t st = c->stream;
        const int total_inner = host_flags[kFlagIter];
        { k_store_velocity_m<D><<<grid_for(n, 256), 256, 0, st>>>(Nf, c->d.x, c->d.vel); MPH_COUNT_LAUNCH(); }
        MPH_CUDA(cudaMemcpyAsync(hs, scal, sizeof(hs), cudaMemcpyDeviceToHost, st));
        MPH_CUDA(cudaStreamSynchronize(st));
        fill_mixed_stats(c, total_inner, outer, hs, bad, tol_out2);
        return MPH_OK;
    }
};

template <int D>
static int mixed_solve_t(mph_case* c)
{
    using V = float;
    MPH_TRY(mixed_prepare(c));
    if (c->device_loop && c->use_graphs && !c->prof.on) {
        if (c->extrapolate && !c->d.vprev) {
            const size_t nvs0 = (size_t)c->dp.N * (D == 2 ? 2 : 4);
            MPH_CUDA(cudaMalloc((void**)&c->d.vprev, 2 * nvs0 * sizeof(double)));
            MPH_CUDA(cudaMalloc((void**)&c->d.vprev_alt, 2 * nvs0 * sizeof(double)));
            c->prev_valid = 0;
        }
        double hs[32];
        int hf[kFlagCount];
        MPH_TRY(device_solve<D>(c, hs, hf));
        const bool bad = hf[kFlagBad] != 0 || !(hs[kSRR] == hs[kSRR]);
        const double tol_out2 = c->tol_outer * c->tol_outer;
        fill_mixed_stats(c, hf[kFlagIter], hf[kFlagOuter], hs, bad, tol_out2);
        return MPH_OK;
    }
    DeviceState& d = c->d;
    MixedRun<D> run;
    run.init(c);
    MPH_TRY(run.start());
    const int Nf = run.Nf, n = run.n, rb = run.rb, cap = run.cap;
    const unsigned gs = run.gs;
    double* scal = run.scal;
    int* flags = run.flags;
    unsigned* counter = run.counter;
    double* part = run.part;
    V *r32 = run.r32, *z32 = run.z32, *s32 = run.s32, *y32 = run.y32, *p32 = run.p32, *q32 = run.q32, *u32 = run.u32;
    (void)r32;
    int* host_flags = run.host_flags;
    // One FP32 CR iteration; its index lives in flags[kFlagIter] (it runs on
    // across refinement steps), so one launch sequence serves every iteration
    // and replays as a graph.  Iterations after a stop return at once.
    auto iteration = [&, c](cudaEvent_t* e, cudaEvent_t ev_end, cudaEvent_t ev_v0 = nullptr, cudaEvent_t ev_v1 = nullptr) {
        cudaStream_t st = c->stream;   // the capture stream while a graph is recorded
        if (c->step_pairs) {
            launch_apply32(c, s32, y32, cap);   // FP32 pair terms, no assembled blocks
        } else {
            k_spmv32<D, 1, V><<<gs, 128, 0, st>>>(Nf, d.nfc, d.sptr, d.acol, d.aval32, s32, y32, scal, flags, cap, part,
                                                  counter);
            MPH_COUNT_LAUNCH();
        }
        if (ev_end) cudaEventRecordWithFlags(ev_end, st, cudaEventRecordExternal);   // profiled graph: the operator's end
        else if (e) prof_begin(c, 0, &e[1]);
        if (mixed_jacobi(c)) {   // profiled graph: the update fused with the preconditioner
            if (ev_v0) cudaEventRecordWithFlags(ev_v0, st, cudaEventRecordExternal);
            pq_precond(c, st, n, rb, s32, y32, p32, q32, u32);
            if (ev_v1) cudaEventRecordWithFlags(ev_v1, st, cudaEventRecordExternal);
        } else {
            { k_pq32<V><<<rb, kReduceThreads, 0, st>>>(n, s32, y32, p32, q32, scal, flags); MPH_COUNT_LAUNCH(); }
            if (ev_v0) cudaEventRecordWithFlags(ev_v0, st, cudaEventRecordExternal);   // profiled graph: the V-cycle
            vcycle_mixed(c, q32, u32, scal + kSQU32);
            if (ev_v1) cudaEventRecordWithFlags(ev_v1, st, cudaEventRecordExternal);
        }
        { k_xrs32<V, false><<<rb, kReduceThreads, 0, st>>>(n, z32, r32, s32, p32, q32, u32, scal, flags, part, counter); MPH_COUNT_LAUNCH(); }
    };
    const int chunk = c->chunk;
    const bool graphs = c->use_graphs;
    // with profiling on, the captured chunk records a fixed event pair around
    // every iteration's operator; the pairs of the iterations that ran are
    // read after each chunk
    const bool gprof = graphs && c->prof.on;
    if (gprof && !c->gev[0])
        for (int k = 0; k < 4 * kMaxGraphChunk; ++k) MPH_CUDA(cudaEventCreate(&c->gev[k]));
    if (graphs) {
        MPH_TRY(capture_graph(c, &c->mx_exec, &c->mx_sig, graph_signature(c, run.tol_in2, cap), [&] {
            for (int k = 0; k < chunk; ++k) {
                if (gprof) cudaEventRecordWithFlags(c->gev[2 * k], c->stream, cudaEventRecordExternal);   // a record node
                iteration(nullptr, gprof ? c->gev[2 * k + 1] : nullptr, gprof ? c->gev[kVcycleEvents + 2 * k] : nullptr,
                          gprof ? c->gev[kVcycleEvents + 2 * k + 1] : nullptr);
            }
        }, &c->mx_launches));
    }
    const long long chunk_launches = c->mx_launches;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> timed;
    for (;;) {
        bool go = false;
        MPH_TRY(run.phase(&go));
        if (!go) break;
        cudaStream_t st = c->stream;
        bool done = false;
        while (!done) {
            const int it_before = host_flags[kFlagIter];
            if (graphs) {
                MPH_CUDA(cudaGraphLaunch(c->mx_exec, st));
                g_launch_count += chunk_launches;
                run.launched += chunk;
            } else {
                for (int k = 0; k < chunk; ++k, ++run.launched) {
                    cudaEvent_t e[2] = {nullptr, nullptr};
                    const bool pon = prof_begin(c, 0, &e[0]) != 0;
                    iteration(pon ? e : nullptr, nullptr);
                    if (pon) timed.push_back({(int)run.launched, {e[0], e[1]}});
                }
            }
            MPH_CUDA(cudaMemcpyAsync(host_flags, flags, sizeof(run.host_flags), cudaMemcpyDeviceToHost, st));
            MPH_CUDA(cudaStreamSynchronize(st));
            if (gprof) {   // the operators of the iterations this chunk ran
                const int ran = std::min(chunk, std::max(0, host_flags[kFlagIter] - it_before));
                for (int k = 0; k < ran; ++k) {
                    float ms = 0.f;
                    MPH_CUDA(cudaEventElapsedTime(&ms, c->gev[2 * k], c->gev[2 * k + 1]));
                    c->prof.kern_ms[0] += ms;
                    c->prof.kern_n[0] += 1;
                    MPH_CUDA(cudaEventElapsedTime(&ms, c->gev[kVcycleEvents + 2 * k], c->gev[kVcycleEvents + 2 * k + 1]));
                    c->prof.kern_ms[1] += ms;
                    c->prof.kern_n[1] += 1;
                }
            }
            done = host_flags[kFlagDone] != 0 || run.launched > cap + chunk;
        }
        MPH_TRY(run.refine(&go));
        if (!go) break;
    }
    const int total_inner = host_flags[kFlagIter];
    for (auto& t : timed) {   // keep the SpMV launches of iterations that ran
        if (t.first < total_inner) {
            c->prof.pending.push_back({0, t.second});
        } else {
            c->prof.pool.push_back(t.second.first);
            c->prof.pool.push_back(t.second.second);
        }
    }
    return run.finish();
}

// ---- the batched solve ---------------------------------------------------------------
// The cases of mph_batch_step that run the point-Jacobi mixed form on the pair
// path solve together: each case's start, phase tests, updates and FP64
// residuals are its own (MixedRun, on its stream), while the CR iterations of
// a refinement phase are four launches over all the cases still iterating
// (each block runs the single-case kernel body on its case, with the
// single-case block decomposition), so a case's bits are those it gets alone.
__global__ void k_batch_pq32(const BatchCase* __restrict__ cs, const int* __restrict__ b0, int nc)
{
    const int c = batch_case_of(b0, nc, (int)blockIdx.x);
    const BatchCase& B = cs[c];
    pq_jacobi32_body<float>((int)blockIdx.x - b0[c], B.el_nb, B.n, B.s32, B.y32, B.p32, B.q32, B.invD, B.u32, B.scal, B.flags,
                            B.partials, B.counter);
}

__global__ void k_batch_xrs32(const BatchCase* __restrict__ cs, const int* __restrict__ b0, int nc)
{
    const int c = batch_case_of(b0, nc, (int)blockIdx.x);
    const BatchCase& B = cs[c];
    xrs32_body<float, false>((int)blockIdx.x - b0[c], B.el_nb, B.n, B.z32, B.r32, B.s32, B.p32, B.q32, B.u32, B.scal, B.flags,
                             B.partials, B.counter);
}

// the cases' solver flags, gathered for one read
__global__ void k_batch_flags(const BatchCase* __restrict__ cs, int nc, int* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nc * kFlagCount) out[t] = cs[t / kFlagCount].flags[t % kFlagCount];
}

void launch_batch_iteration(const BatchCase* cs, const int* b0, int nc, int dim, bool pack, int pair_block, int ct_block,
                            int vp_smem, int ct_smem, const int* nblocks, cudaStream_t st)
{
    launch_batch_operator(cs, b0, b0 + (nc + 1), nc, dim, pack, pair_block, ct_block, vp_smem, ct_smem, nblocks[0], nblocks[1], st);
    if (nblocks[2] > 0) {
        { k_batch_pq32<<<nblocks[2], kReduceThreads, 0, st>>>(cs, b0 + 2 * (nc + 1), nc); MPH_COUNT_LAUNCH(); }
        { k_batch_xrs32<<<nblocks[2], kReduceThreads, 0, st>>>(cs, b0 + 2 * (nc + 1), nc); MPH_COUNT_LAUNCH(); }
    }
}

bool batch_solve_eligible(const mph_case* c)
{
    return c->batch_solve && c->precision == MPH_PRECISION_MIXED && c->stage == 6 && c->step_pairs && mixed_jacobi(c) &&
           !c->pair_recompute && !c->split_apply && !c->device_loop && !c->prof.on && c->dp.Nf > 0 && c->nslices > 0;
}

// The batched solve's device table, flag buffers, stream and events, per
// host thread (one batch at a time per thread).
struct BatchBuffers {
    BatchCase* tab = nullptr;
    int* b0 = nullptr;
    int* flags = nullptr;
    int* hflags = nullptr;
    int cap = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<cudaEvent_t> evs;
    int ensure(int nc)
    {
        if (!st) {
            MPH_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            MPH_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        }
        while ((int)evs.size() < nc) {
            cudaEvent_t e = nullptr;
            MPH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            evs.push_back(e);
        }
        if (nc <= cap) return MPH_OK;
        if (tab) cudaFree(tab);
        if (b0) cudaFree(b0);
        if (flags) cudaFree(flags);
        if (hflags) cudaFreeHost(hflags);
        tab = nullptr;
        b0 = flags = hflags = nullptr;
        cap = 0;
        MPH_CUDA(cudaMalloc((void**)&tab, (size_t)nc * sizeof(BatchCase)));
        MPH_CUDA(cudaMalloc((void**)&b0, (size_t)3 * (nc + 1) * sizeof(int)));
        MPH_CUDA(cudaMalloc((void**)&flags, (size_t)nc * kFlagCount * sizeof(int)));
        MPH_CUDA(cudaMallocHost((void**)&hflags, (size_t)nc * kFlagCount * sizeof(int)));
        cap = nc;
        return MPH_OK;
    }
};
static thread_local BatchBuffers t_batch;

using ParFor = std::function<void(int, const std::function<int(int)>&)>;

template <int D>
static int batched_solve_t(std::vector<mph_case*>& cs, bool pack, int pair_block, int ct_block, const ParFor& par)
{
    const int nc = (int)cs.size();
    BatchBuffers& tb = t_batch;
    MPH_TRY(tb.ensure(nc));
    std::vector<MixedRun<D>> runs(nc);
    std::vector<int> st(nc, MPH_OK);
    auto each = [&](const std::function<int(int)>& f) {   // f on every case, in parallel; the first failure
        par(nc, [&](int k) { return st[k] = f(k); });
        for (int k = 0; k < nc; ++k)
            if (st[k] != MPH_OK) return st[k];
        return (int)MPH_OK;
    };
    int chunk = 1;
    MPH_TRY(each([&](int k) {
        MPH_TRY(mixed_prepare(cs[k]));
        runs[k].init(cs[k]);
        return runs[k].start();
    }));
    for (int k = 0; k < nc; ++k) chunk = std::max(chunk, cs[k]->chunk);
    std::vector<BatchCase> tab(nc);
    int vp_smem = 0, ct_smem = 0;
    for (int k = 0; k < nc; ++k) {
        mph_case* c = cs[k];
        DeviceState& d = c->d;
        MixedRun<D>& R = runs[k];
        BatchCase& B = tab[k];
        B.N = c->dp.N;
        B.Nf = c->dp.Nf;
        B.n = R.n;
        B.cap = R.cap;
        B.ct_loc = c->loc_ct_smem != 0;
        B.vp_loc = c->loc_smem != 0;
        B.ct_nb = (int)grid_for(c->dp.N, ct_block);
        B.vp_nb = (int)grid_for(c->dp.Nf, pair_block);
        B.el_nb = R.rb;
        B.ctsptr = d.ctsptr;
        B.ct_cnt = d.ct_cnt;
        B.ctsval = (const float4*)d.ctsval;
        B.tct32 = d.tct32;
        B.ctuniq = d.ctuniq;
        B.ctucount = d.ctucount;
        B.nfc = d.nfc;
        B.sptr = d.sptr;
        B.acol = d.acol;
        B.grec16 = d.grec16;
        B.grec32 = d.grec32;
        B.lcol16 = d.lcol16;
        B.pscale = d.pscale;
        B.sdiag32 = d.sdiag32;
        B.ncp = d.ncp;
        B.psptr = d.psptr;
        B.psval = (const float4*)d.psval;
        B.uniq = d.uniq;
        B.ucount = d.ucount;
        B.s32 = R.s32;
        B.y32 = R.y32;
        B.p32 = R.p32;
        B.q32 = R.q32;
        B.u32 = R.u32;
        B.z32 = R.z32;
        B.r32 = R.r32;
        B.invD = d.v32 + 7 * (size_t)R.n;
        B.scal = R.scal;
        B.flags = R.flags;
        B.partials = R.part;
        B.counter = R.counter;
        vp_smem = std::max(vp_smem, c->loc_smem);
        ct_smem = std::max(ct_smem, c->loc_ct_smem);
    }
    MPH_CUDA(cudaMemcpyAsync(tb.tab, tab.data(), (size_t)nc * sizeof(BatchCase), cudaMemcpyHostToDevice, tb.st));
    std::vector<char> active(nc, 1);
    std::vector<int> b0(3 * (nc + 1));
    for (;;) {
        MPH_TRY(each([&](int k) {
            if (!active[k]) return (int)MPH_OK;
            bool go = false;
            MPH_TRY(runs[k].phase(&go));
            if (!go) active[k] = 0;
            return (int)MPH_OK;
        }));
        int nact = 0;
        for (int k = 0; k < nc; ++k) nact += active[k] ? 1 : 0;
        if (nact == 0) break;
        // this phase's block starts: the cases still iterating, the others none
        int nb[3] = {0, 0, 0};
        for (int k = 0; k < nc; ++k) {
            b0[k] = nb[0];
            b0[(nc + 1) + k] = nb[1];
            b0[2 * (nc + 1) + k] = nb[2];
            if (active[k]) {
                nb[0] += tab[k].ct_nb;
                nb[1] += tab[k].vp_nb;
                nb[2] += tab[k].el_nb;
            }
        }
        b0[nc] = nb[0];
        b0[2 * nc + 1] = nb[1];
        b0[3 * nc + 2] = nb[2];
        // the batch stream after the active cases' phase kernels
        for (int k = 0; k < nc; ++k) {
            if (!active[k]) continue;
            MPH_CUDA(cudaEventRecord(tb.evs[k], cs[k]->stream));
            MPH_CUDA(cudaStreamWaitEvent(tb.st, tb.evs[k], 0));
        }
        MPH_CUDA(cudaMemcpyAsync(tb.b0, b0.data(), b0.size() * sizeof(int), cudaMemcpyHostToDevice, tb.st));
        bool all = false;
        while (!all) {
            for (int it = 0; it < chunk; ++it)
                launch_batch_iteration(tb.tab, tb.b0, nc, D, pack, pair_block, ct_block, vp_smem, ct_smem, nb, tb.st);
            { k_batch_flags<<<grid_for((long long)nc * kFlagCount, 256), 256, 0, tb.st>>>(tb.tab, nc, tb.flags); MPH_COUNT_LAUNCH(); }
            MPH_CUDA(cudaMemcpyAsync(tb.hflags, tb.flags, (size_t)nc * kFlagCount * sizeof(int), cudaMemcpyDeviceToHost, tb.st));
            MPH_CUDA(cudaStreamSynchronize(tb.st));
            all = true;
            for (int k = 0; k < nc; ++k) {
                if (!active[k]) continue;
                std::copy(tb.hflags + (size_t)k * kFlagCount, tb.hflags + (size_t)(k + 1) * kFlagCount, runs[k].host_flags);
                runs[k].launched += chunk;
                if (!(runs[k].host_flags[kFlagDone] != 0 || runs[k].launched > runs[k].cap + chunk)) all = false;
            }
        }
        // the cases' streams after the batch's iterations: updates and FP64 residuals
        MPH_CUDA(cudaEventRecord(tb.ev, tb.st));
        MPH_TRY(each([&](int k) {
            if (!active[k]) return (int)MPH_OK;
            MPH_CUDA(cudaStreamWaitEvent(cs[k]->stream, tb.ev, 0));
            bool go = false;
            MPH_TRY(runs[k].refine(&go));
            if (!go) active[k] = 0;
            return (int)MPH_OK;
        }));
    }
    return each([&](int k) {
        MPH_TRY(runs[k].finish());
        MPH_CUDA(cudaGetLastError());
        cs[k]->stage = 7;
        return (int)MPH_OK;
    });
}

// Solve the eligible cases of a batch together, in groups of one dimension,
// record format and block widths (the cases' stage must be 6).
int batched_mixed_solve(std::vector<mph_case*>& cases, const ParFor& par)
{
    std::vector<char> taken(cases.size(), 0);
    for (size_t a = 0; a < cases.size(); ++a) {
        if (taken[a]) continue;
        mph_case* c0 = cases[a];
        std::vector<mph_case*> g;
        for (size_t b = a; b < cases.size(); ++b) {
            mph_case* c = cases[b];
            if (taken[b] || c->dim != c0->dim || c->pair_pack != c0->pair_pack || c->pair_block != c0->pair_block ||
                c->ct_block != c0->ct_block)
                continue;
            taken[b] = 1;
            g.push_back(c);
        }
        if (c0->dim == 2) MPH_TRY(batched_solve_t<2>(g, c0->pair_pack, c0->pair_block, c0->ct_block, par));
        else MPH_TRY(batched_solve_t<3>(g, c0->pair_pack, c0->pair_block, c0->ct_block, par));
    }
    return MPH_OK;
}

int run_mixed_solve(mph_case* c)
{
    return c->dim == 2 ? mixed_solve_t<2>(c) : mixed_solve_t<3>(c);
}

}  // namespace mph
