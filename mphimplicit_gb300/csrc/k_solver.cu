// k_solver.cu - preconditioned conjugate residual solve
// (solveWithConjugatedGradient, main.cpp:4270-4421; the reference names it
// conjugate gradient but runs the CR recurrences).
//
//   x0 = v* - F/m dt ; s = M b ; rs0 = (b,s) ; rr0 = (b,b) ; r = b - A x ; s = M r
//   loop: rr = (r,r); stop if rr/rr0 < 1e-12
//         y = A s ; rho = (s,y)
//         first: p = s, q = y (= A p)    else: p = s + beta p, q = y + beta q
//         u = M q ; alpha = rho / (q,u)
//         x += alpha p ; r -= alpha q ; s -= alpha u
//   v = x
//
// Kernels per iteration: sliced-ELL block SpMV with the (s,y) dot and the
// convergence test; p/q update; the V-cycle (its last kernel forms (q,u));
// x/r/s update with the (r,r) dot.  All scalars stay on the device.
#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

__host__ __device__ __forceinline__ int rho_slot(int it) { return kSRho + 8 + (it & 1); }   // two alternating slots

template <int D>
__global__ void k_cr_init(int Nf, const int* __restrict__ type, const double* __restrict__ vel, const double* __restrict__ force,
                          const double* __restrict__ b, double* __restrict__ x, double density0, double density1, double vol,
                          double dt, double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out)
{
    double acc = 0.0;
    const int n = Nf * D;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / D, r = k % D;
        const int t = type[i];
        const double m = (t == 0 ? density0 : density1) * vol;
        const int VSD = D == 2 ? 2 : 4;
        x[k] = vel[(size_t)i * VSD + r] - force[(size_t)i * VSD + r] / m * dt;
        const double bk = b[k];
        acc += bk * bk;
    }
    reduce_finalize(acc, partials, counter, out);
}

// MODE 0: r = b - A x with (r,r) -> out.   MODE 1: y = A s with (s,y) ->
// the rho slot of iteration it = flags[kFlagIter], after the convergence test
// of that iteration, rr/rr0 < tol2 (out is unused).  The reference's test is
// rr/rr0 < 1e-12 (main.cpp:4346), i.e. tol2 = (1e-6)^2.
template <int D, int MODE>
__global__ void __launch_bounds__(128) k_spmv(int Nf, const int* __restrict__ nfc, const long long* __restrict__ sptr,
                                              const int* __restrict__ acol, const double* __restrict__ aval,
                                              const double* __restrict__ xin, const double* __restrict__ b,
                                              double* __restrict__ yout, double* __restrict__ scal, int* __restrict__ flags,
                                              int cap, double tol2, double* __restrict__ partials,
                                              unsigned* __restrict__ counter, double* __restrict__ out)
{
    constexpr int DD = D * D;
    if (MODE == 1) {
        if (flags[kFlagDone]) return;
        const int it = flags[kFlagIter];
        const double rr = scal[kSRR], rr0 = scal[kSRR0];
        const bool bad = !(rr == rr);   // NaN residual
        if (it >= cap || rr / rr0 < tol2 || bad) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                flags[kFlagDone] = 1;
                if (bad) flags[kFlagBad] = 1;
            }
            return;
        }
        out = scal + rho_slot(it);
    }
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
            for (int s = 0; s < D; ++s) xv[s] = xin[(size_t)col * D + s];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) y[r] += vp[((long long)k * DD + r * D + s) * 32] * xv[s];
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const size_t k = (size_t)i * D + r;
            if (MODE == 0) {
                const double rv = b[k] - y[r];
                yout[k] = rv;
                acc += rv * rv;
            } else {
                yout[k] = y[r];
                acc += xin[k] * y[r];
            }
        }
    }
    reduce_finalize(acc, partials, counter, out);
}

__global__ void k_update_pq(int n, const double* __restrict__ s, const double* __restrict__ y, double* __restrict__ p,
                            double* __restrict__ q, const double* __restrict__ scal, const int* __restrict__ flags)
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
    const double beta = scal[rho_slot(it)] / scal[rho_slot(it - 1)];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        p[k] = beta * p[k] + s[k];
        q[k] = beta * q[k] + y[k];
    }
}

// x += alpha p, r -= alpha q, s -= alpha u, (r,r) -> rr; the last block then
// advances the iteration counter flags[kFlagIter].
__global__ void k_update_xrs(int n, double* __restrict__ x, double* __restrict__ r, double* __restrict__ s,
                             const double* __restrict__ p, const double* __restrict__ q, const double* __restrict__ u,
                             double* __restrict__ scal, int* __restrict__ flags, double* __restrict__ partials,
                             unsigned* __restrict__ counter)
{
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    const double alpha = scal[rho_slot(it)] / scal[kSQU];
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        x[k] += alpha * p[k];
        const double rk = r[k] - alpha * q[k];
        r[k] = rk;
        s[k] -= alpha * u[k];
        acc += rk * rk;
    }
    reduce_finalize_step(acc, partials, counter, scal + kSRR, flags + kFlagIter);
}

__global__ void k_dot(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ partials,
                      unsigned* __restrict__ counter, double* __restrict__ out)
{
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) acc += a[k] * b[k];
    reduce_finalize(acc, partials, counter, out);
}

template <int D>
__global__ void k_store_velocity(int Nf, const double* __restrict__ x, double* __restrict__ vel)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Nf * D) return;
    const int i = k / D, r = k % D;
    vel[(size_t)i * (D == 2 ? 2 : 4) + r] = x[k];
}

template <int D>
static int cr_solve_t(mph_case* c)
{
    const int Nf = c->dp.Nf;
    const int n = Nf * D;
    cudaStream_t st = c->stream;
    double* scal = c->d.scal;
    int* flags = c->d.flags;
    unsigned* counter = (unsigned*)(flags + kFlagCounter);
    double* part = c->d.partials;
    const int rb = std::min<int>(grid_for(n, kReduceThreads), kReduceBlocks);
    const unsigned gs = grid_for(Nf, 128);
    // stop test ||r||/||b|| < tol_outer on squared norms (1e-6 by default, the
    // reference's constant; mph_case_set_solver tightens it)
    const double tol2 = c->tol_outer == 1.0e-6 ? 1.0e-12 : c->tol_outer * c->tol_outer;
    MPH_CUDA(cudaMemsetAsync(flags, 0, kFlagCount * sizeof(int), st));
    MPH_CUDA(cudaMemsetAsync(scal, 0, 32 * sizeof(double), st));

    { k_cr_init<D><<<rb, kReduceThreads, 0, st>>>(Nf, c->d.type, c->d.vel, c->d.force, c->d.bvec, c->d.x, c->dp.density[0],
                                                c->dp.density[1], c->dp.vol, c->dp.dt, part, counter, scal + kSRR0); MPH_COUNT_LAUNCH(); }
    vcycle_fp64(c, c->d.bvec, c->d.s, scal + kSRS0);
    { k_spmv<D, 0><<<gs, 128, 0, st>>>(Nf, c->d.nfc, c->d.sptr, c->d.acol, c->d.aval, c->d.x, c->d.bvec, c->d.r, scal, flags, 0,
                                     tol2, part, counter, scal + kSRR); MPH_COUNT_LAUNCH(); }
    vcycle_fp64(c, c->d.r, c->d.s, scal + kSQU);

    // One CR iteration; the iteration index lives in flags[kFlagIter], so the
    // same launch sequence serves every iteration (and can be replayed as a
    // graph).  Iterations after convergence return at once.
    const int cap = n;   // the reference iterates at most N = D*Nf times
    auto iteration = [&, c](cudaEvent_t* e) {
        cudaStream_t st = c->stream;   // the capture stream while a graph is recorded
        { k_spmv<D, 1><<<gs, 128, 0, st>>>(Nf, c->d.nfc, c->d.sptr, c->d.acol, c->d.aval, c->d.s, nullptr, c->d.y, scal, flags,
                                         cap, tol2, part, counter, nullptr); MPH_COUNT_LAUNCH(); }
        if (e) prof_begin(c, 0, &e[1]);
        { k_update_pq<<<rb, kReduceThreads, 0, st>>>(n, c->d.s, c->d.y, c->d.p, c->d.q, scal, flags); MPH_COUNT_LAUNCH(); }
        if (e) prof_begin(c, 1, &e[2]);
        vcycle_fp64(c, c->d.q, c->d.u, scal + kSQU);
        if (e) prof_begin(c, 1, &e[3]);
        { k_update_xrs<<<rb, kReduceThreads, 0, st>>>(n, c->d.x, c->d.r, c->d.s, c->d.p, c->d.q, c->d.u, scal, flags, part,
                                                    counter); MPH_COUNT_LAUNCH(); }
    };
    const int chunk = 8;
    int host_flags[kFlagCount];
    int it = 0;   // iterations launched
    bool done = false;
    // (iteration | class bit, events) of timed SpMV / V-cycle launches; only
    // launches of iterations that ran are kept (later ones return at once)
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> timed;
    const bool graphs = c->use_graphs && !c->prof.on;
    if (graphs) {
        MPH_TRY(capture_graph(c, &c->cr_exec, &c->cr_sig, graph_signature(c, tol2, cap), [&] {
            for (int k = 0; k < chunk; ++k) iteration(nullptr);
        }, &c->cr_launches));
    }
    const long long chunk_launches = c->cr_launches;
    while (!done) {
        if (graphs) {
            MPH_CUDA(cudaGraphLaunch(c->cr_exec, st));
            g_launch_count += chunk_launches;
            it += chunk;
        } else {
            const int m = std::min(chunk, cap + 1 - it);
            for (int k = 0; k < m; ++k, ++it) {
                cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
                const bool pon = prof_begin(c, 0, &e[0]) != 0;
                iteration(pon ? e : nullptr);
                if (pon) {
                    timed.push_back({it, {e[0], e[1]}});
                    timed.push_back({it | (1 << 30), {e[2], e[3]}});
                }
            }
        }
        MPH_CUDA(cudaMemcpyAsync(host_flags, flags, sizeof(host_flags), cudaMemcpyDeviceToHost, st));
        MPH_CUDA(cudaStreamSynchronize(st));
        done = host_flags[kFlagDone] != 0 || it > cap;
    }
    { k_dot<<<rb, kReduceThreads, 0, st>>>(n, c->d.r, c->d.s, part, counter, scal + kSRS); MPH_COUNT_LAUNCH(); }
    { k_store_velocity<D><<<grid_for(n, 256), 256, 0, st>>>(Nf, c->d.x, c->d.vel); MPH_COUNT_LAUNCH(); }
    double hs[8];
    MPH_CUDA(cudaMemcpyAsync(hs, scal, sizeof(hs), cudaMemcpyDeviceToHost, st));
    MPH_CUDA(cudaMemcpyAsync(host_flags, flags, sizeof(host_flags), cudaMemcpyDeviceToHost, st));
    MPH_CUDA(cudaStreamSynchronize(st));
    c->stats.iterations = host_flags[kFlagDone] ? host_flags[kFlagIter] : cap;
    c->stats.rr0 = hs[kSRR0];
    c->stats.rr = hs[kSRR];
    c->stats.rs0 = hs[kSRS0];
    c->stats.rs = hs[kSRS];
    c->stats.inner_form = 0;
    c->stats.inner_local_blocks = c->stats.inner_gather_blocks = 0;
    c->stats.inner_local_cols = 0;
    c->stats.inner_ct_local_blocks = c->stats.inner_reserved = 0;
    c->stats.status = host_flags[kFlagBad] ? MPH_ERR_NAN : (host_flags[kFlagDone] && host_flags[kFlagIter] < cap ? MPH_OK : MPH_ERR_NOT_CONVERGED);
    for (auto& t : timed) {
        const int iter = t.first & ((1 << 30) - 1);
        const int cls = (t.first >> 30) & 1;
        if (iter < c->stats.iterations) {
            c->prof.pending.push_back({cls, t.second});
        } else {
            c->prof.pool.push_back(t.second.first);
            c->prof.pool.push_back(t.second.second);
        }
    }
    return MPH_OK;
}

int run_cr_solve(mph_case* c)
{
    if (c->precision == MPH_PRECISION_MIXED) return run_mixed_solve(c);
    return c->dim == 2 ? cr_solve_t<2>(c) : cr_solve_t<3>(c);
}


}  // namespace mph
