// k_assemble.cu - the implicit system of one step.
//
//   k_slice_width   : sliced-ELL slice widths (longest fluid row of each
//                     32-row slice); the row pointers come from the device scan
//   k_matrix_c      : calculateMatrixC (main.cpp:2462-2507): D coefficients per
//                     P-neighbour, stored aligned with the P-list
//   k_vector_p      : the source vector p (main.cpp:2509-2549)
//   k_matrix_a      : calculateMatrixA (main.cpp:2251-2335) + multiplyMatrixC
//                     (main.cpp:2574-2642) in one pass per fluid row: viscous
//                     and inertia blocks, wall velocities into b, b -= C p and
//                     the C Lambda C^T merge-join of the two sorted P-lists,
//                     written once into the sliced-ELL block layout.  The same
//                     pass sums each row's blocks per neighbour cell of the
//                     level-0 multigrid grid (part[]), so the Galerkin level-0
//                     matrix (main.cpp:3336-3411) never re-reads A.
#include "mph_device.cuh"

namespace mph {

__global__ void k_slice_width(int Nf, const int* __restrict__ nfc, int* __restrict__ width32, int pad = 1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int v = i < Nf ? nfc[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    v = (v + pad - 1) / pad * pad;
    if ((threadIdx.x & 31) == 0 && i < ((Nf + 31) / 32) * 32) width32[i >> 5] = 32 * v;
}

__global__ void k_max_int(const int* __restrict__ v, int n, int* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int m = i < n ? v[i] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

template <int D>
__global__ void __launch_bounds__(128) k_matrix_c(DevParams P, const double* __restrict__ pos, const int* __restrict__ ncp,
                                                  const long long* __restrict__ nptrP, const int* __restrict__ nindP,
                                                  double* __restrict__ cval)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.Nf) return;
    double xi[3];
    load_vec<D>(pos, i, xi);
    const double rP2 = P.rP * P.rP;
    const long long b = nptrP[i];
    const int n = ncp[i];
    double self[3] = {0, 0, 0};
    int selfk = 0;
    for (int a = 0; a < n; ++a) {
        const int j = nindP[b + a];
        double cv[3] = {0, 0, 0};
        if (j == i) {
            selfk = a;
        } else {
            double xj[3], q[3];
            load_vec<D>(pos, j, xj);
            sep_vec<D>(P, xj, xi, q);
            const double r2 = norm2_exact<D>(q);
            if (r2_pos_below(r2, rP2)) {
                const double inv = rsqrt(r2);
                const double wd = -P.kfp * (P.m2h_rp * (1.0 - (r2 * inv) * P.inv_rp));
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    cv[r] = (q[r] * inv) * wd;
                    self[r] += cv[r];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < D; ++r) cval[(b + a) * D + r] = cv[r];
    }
#pragma unroll
    for (int r = 0; r < D; ++r) cval[(b + selfk) * D + r] = self[r];
}

template <int D>
__global__ void __launch_bounds__(128) k_vector_p(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                  const double* __restrict__ vel, const double* __restrict__ vsp,
                                                  const int* __restrict__ ncp, const long long* __restrict__ nptrP,
                                                  const int* __restrict__ nindP, double* __restrict__ pvec)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const int ti = type[i];
    const double v0 = vsp[i];
    double p = 0.0;
    if (v0 > 0.0) p = P.bulk[ti] * v0;   // Kappa is 0 where VolStrainP < 0 (main.cpp:1704-1735)
    const bool wi = is_wall(ti);
    const double lam = P.lambda[ti];
    double xi[3], vi[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(vel, i, vi);
    const double rP2 = P.rP * P.rP;
    double sum = 0.0;
    const long long b = nptrP[i];
    for (int a = 0; a < ncp[i]; ++a) {
        const int j = nindP[b + a];
        if (j == i) continue;
        const bool wj = is_wall(type[j]);
        if (!wi && !wj) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (!r2_pos_below(r2, rP2)) continue;
        const double inv = rsqrt(r2);
        const double wd = -P.kfp * (P.m2h_rp * (1.0 - (r2 * inv) * P.inv_rp));
        double vj[3];
        if (wj) load_vec<D>(vel, j, vj);
#pragma unroll
        for (int s = 0; s < D; ++s) {
            const double e = q[s] * inv;
            if (wi) sum += lam * (e * wd) * vi[s];
            if (wj) sum += lam * (-e * wd) * vj[s];
        }
    }
    pvec[i] = p + sum;
}


template <int D>
__device__ __forceinline__ void flush_part(double* __restrict__ prow, int slot, const double (&acc)[D][D], bool add)
{
    double* dst = prow + (size_t)slot * D * D;
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int s = 0; s < D; ++s) dst[r * D + s] = add ? dst[r * D + s] + acc[r][s] : acc[r][s];
}

template <int D>
__global__ void __launch_bounds__(128) k_matrix_a(DevParams P, Level0Map M, const int* __restrict__ only_cells,
                                                  const int* __restrict__ type,
                                                  const int* __restrict__ key, const double* __restrict__ pos,
                                                  const double* __restrict__ vel, const double* __restrict__ force,
                                                  const int* __restrict__ nc, const int* __restrict__ nfc,
                                                  const long long* __restrict__ nptr, const int* __restrict__ nind,
                                                  const int* __restrict__ ncp, const long long* __restrict__ nptrP,
                                                  const int* __restrict__ nindP, const double* __restrict__ cval,
                                                  const double* __restrict__ pvec, const long long* __restrict__ sptr,
                                                  int* __restrict__ acol, double* __restrict__ aval,
                                                  float* __restrict__ aval32, double* __restrict__ bvec, double* __restrict__ invDiag,
                                                  int* __restrict__ selfk_out, double* __restrict__ part)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.Nf) return;
    if (only_cells && !only_cells[key[i]]) return;   // row assembled by the cell-block kernel
    constexpr int DD = D * D;
    const int lane = i & 31;
    const long long sbase = sptr[i >> 5];
    int* colp = acol + sbase + lane;
    double* valp = aval ? aval + sbase * DD + lane : nullptr;   // null when the FP64 operator is factored
    float* valp32 = aval32 ? aval32 + sbase * DD + lane : nullptr;   // mixed form: FP32 copy

    const int ti = type[i];
    double xi[3], vi[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(vel, i, vi);
    const double rV2 = P.rV * P.rV;

    // this row's P-list and C rows (used by every merge-join of the row)
    const long long pbi = nptrP[i];
    const int npi = ncp[i];
    const int* Pi = nindP + pbi;
    const double* Ci = cval + pbi * D;

    // level-0 stencil bookkeeping
    int gi[3];
    {
        int ic[3];
        key_coords(P, key[i], ic);
#pragma unroll
        for (int d = 0; d < 3; ++d) gi[d] = ic[d] - M.mn[d];
    }
    double* prow = part + (size_t)i * M.S * DD;
    if (M.folded) {
        for (int t = 0; t < M.S * DD; ++t) prow[t] = 0.0;
    }
    unsigned long long touched = 0ull;
    int run_slot = -1;
    double run[D][D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int s = 0; s < D; ++s) run[r][s] = 0.0;

    double selfc[D][D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int s = 0; s < D; ++s) selfc[r][s] = 0.0;
    double sumvec[3] = {0, 0, 0};
    int self = 0;

    const long long nb = nptr[i];
    const int n = nc[i];
    const int nf = nfc[i];
    for (int k = 0; k < n; ++k) {
        const int j = nind[nb + k];
        if (j == i) { self = k; continue; }
        double V[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) V[r][s] = 0.0;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        const bool fluid = k < nf;
        if (r2_pos_below(r2, rV2)) {
            // one reciprocal square root per pair (FP64 divide and sqrt are
            // slow on this part); -dw/dr = -kf (-2/h) (1 - r/h)
            const double inv = rsqrt(r2);
            const double dij = r2 * inv;
            const double wd = -P.kfv * (P.m2h_rv * (1.0 - dij * P.inv_rv));
            const double muij = P.muij[ti][type[j]];
            double e[3];
#pragma unroll
            for (int d = 0; d < D; ++d) e[d] = q[d] * inv;
            const double f = P.visc * muij * wd * inv;
            double vj[3];
            if (!fluid) load_vec<D>(vel, j, vj);
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) {
                    const double coef = f * e[s] * e[r];
                    selfc[r][s] += coef;
                    V[r][s] = coef;
                    if (!fluid) sumvec[r] += coef * vj[s];
                }
        }
        if (!fluid) continue;
        // C Lambda C^T for the pair (i, j): merge-join of the sorted P-lists
        double cc[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) cc[r][s] = 0.0;
        {
            const long long pbj = nptrP[j];
            const int npj = ncp[j];
            const int* Pj = nindP + pbj;
            const double* Cj = cval + pbj * D;
            int a = 0, b = 0;
            int ka = a < npi ? Pi[a] : 0, kb = b < npj ? Pj[b] : 0;
            while (a < npi && b < npj) {
                if (ka == kb) {
                    const double lam = P.lambda[type[ka]];
                    double ci[3], cj[3];
#pragma unroll
                    for (int r = 0; r < D; ++r) { ci[r] = Ci[(long long)a * D + r] * lam; cj[r] = Cj[(long long)b * D + r]; }
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int s = 0; s < D; ++s) cc[r][s] += ci[r] * cj[s];
                    ++a; ++b;
                    ka = a < npi ? Pi[a] : 0;
                    kb = b < npj ? Pj[b] : 0;
                } else if (ka < kb) {
                    ++a;
                    ka = a < npi ? Pi[a] : 0;
                } else {
                    ++b;
                    kb = b < npj ? Pj[b] : 0;
                }
            }
        }
        double blk[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) blk[r][s] = -V[r][s] + cc[r][s];
        colp[(long long)k * 32] = j;
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) {
                if (aval) valp[((long long)k * DD + r * D + s) * 32] = blk[r][s];
                if (valp32) valp32[((long long)k * DD + r * D + s) * 32] = (float)blk[r][s];
            }
        // per-cell partial sums of the row (runs of equal stencil slot)
        const int slot = stencil_slot<D>(P, M, gi, key[j]);
        if (slot != run_slot) {
            if (run_slot >= 0) {
                flush_part<D>(prow, run_slot, run, M.folded != 0);
                touched |= 1ull << run_slot;
            }
            run_slot = slot;
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) run[r][s] = blk[r][s];
        } else {
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) run[r][s] += blk[r][s];
        }
    }
    if (run_slot >= 0) {
        flush_part<D>(prow, run_slot, run, M.folded != 0);
        touched |= 1ull << run_slot;
    }
    // self block: viscous sum, inertia, C Lambda C^T(i, i)
    const double inert = P.inert64[ti];   // (rho vol) / vol / dt, formed on the host
    {
        double cc[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) cc[r][s] = 0.0;
        for (int a = 0; a < npi; ++a) {
            const double lam = P.lambda[type[Pi[a]]];
            double ci[3];
#pragma unroll
            for (int r = 0; r < D; ++r) ci[r] = Ci[(long long)a * D + r];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) cc[r][s] += ci[r] * lam * ci[s];
        }
        double blk[D][D];
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) blk[r][s] = (selfc[r][s] + (r == s ? inert : 0.0)) + cc[r][s];
        colp[(long long)self * 32] = i;
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) {
                if (aval) valp[((long long)self * DD + r * D + s) * 32] = blk[r][s];
                if (valp32) valp32[((long long)self * DD + r * D + s) * 32] = (float)blk[r][s];
            }
#pragma unroll
        for (int r = 0; r < D; ++r) invDiag[(size_t)i * D + r] = blk[r][r] != 0.0 ? 1.0 / blk[r][r] : 0.0;
        selfk_out[i] = self;
        // the own cell's slot received this row's other blocks already
        const int cslot = stencil_slot<D>(P, M, gi, key[i]);
        if (M.folded || (touched >> cslot) & 1ull) {
            double* dst = prow + (size_t)cslot * DD;
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) dst[r * D + s] += blk[r][s];
        } else {
            flush_part<D>(prow, cslot, blk, false);
        }
        touched |= 1ull << cslot;
    }
    if (!M.folded) {
        for (int t = 0; t < M.S; ++t) {
            if ((touched >> t) & 1ull) continue;
            double* dst = prow + (size_t)t * DD;
#pragma unroll
            for (int r = 0; r < DD; ++r) dst[r] = 0.0;
        }
    }
    // right-hand side: wall terms, inertia, then b -= C p
    double bv[3];
#pragma unroll
    for (int r = 0; r < D; ++r) bv[r] = sumvec[r] + inert * vi[r];
    for (int a = 0; a < npi; ++a) {
        const double pj = pvec[Pi[a]];
#pragma unroll
        for (int r = 0; r < D; ++r) bv[r] -= Ci[(long long)a * D + r] * pj;
    }
#pragma unroll
    for (int r = 0; r < D; ++r) bvec[(size_t)i * D + r] = bv[r];
}

// ---- launcher ---------------------------------------------------------------
static int ensure(void** p, long long* cap, long long need, size_t elem)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 1024;
    cudaError_t e = cudaMalloc(p, (size_t)n * elem);
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc(assembly)");
    *cap = n;
    return MPH_OK;
}

// Slice pointers of a sliced layout of 32-row slices over per-row counts:
// width[s] = 32 x the longest row of slice s, ptr = its exclusive scan, and
// the slot total on the host.
int launch_slice_ptr(mph_case* c, int rows, const int* counts, int* width, long long* ptr, long long* total)
{
    const int ns = (rows + 31) / 32;
    { k_slice_width<<<grid_for((long long)ns * 32, 256), 256, 0, c->stream>>>(rows, counts, width); MPH_COUNT_LAUNCH(); }
    MPH_TRY(launch_scan_i32_to_i64(c, width, ptr, ns));
    MPH_CUDA(cudaMemcpyAsync(total, ptr + ns, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    return MPH_OK;
}

int launch_assemble(mph_case* c)
{
    const DevParams& P = c->dp;
    const int Nf = P.Nf;
    const int D = c->dim;
    // slice pointers
    c->nslices = (Nf + 31) / 32;
    // the fluid rows' slices padded to a multiple of 4 slots (zero padding
    // records): the pair-term operator then loops over whole slices in steps
    // of four without per-slot bounds tests
    { k_slice_width<<<grid_for((long long)c->nslices * 32, 256), 256, 0, c->stream>>>(Nf, c->d.nfc, c->d.swidth, 4); MPH_COUNT_LAUNCH(); }
    MPH_CUDA(cudaMemsetAsync(c->d.dmax, 0, sizeof(int), c->stream));
    { k_max_int<<<grid_for(c->nslices, 256), 256, 0, c->stream>>>(c->d.swidth, c->nslices, c->d.dmax); MPH_COUNT_LAUNCH(); }
    MPH_TRY(launch_scan_i32_to_i64(c, c->d.swidth, c->d.sptr, c->nslices));
    long long h_slots = 0;
    int h_width = 0;
    MPH_CUDA(cudaMemcpyAsync(&h_slots, c->d.sptr + c->nslices, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(&h_width, c->d.dmax, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    const int kmax_rows = h_width / 32;   // longest fluid row
    c->nslots = h_slots;
    // the form of this step's system decides which block arrays exist: FP64
    // blocks unless the FP64 operator is factored, FP32 blocks for the mixed
    // form unless its inner operator runs on the pair terms
    c->step_factored = factored_applies(c);
    c->step_pairs = c->step_factored && !c->inner_blocks && c->visc_nonneg;
    {
        long long cap = c->d.cap_slots;
        void* p = c->d.acol;
        MPH_TRY(ensure(&p, &cap, h_slots, sizeof(int)));
        c->d.acol = (int*)p;
        c->d.cap_slots = cap;
        const bool need64 = !c->step_factored, need32 = c->precision == MPH_PRECISION_MIXED && !c->step_pairs;
        if (need64 && cap > c->d.cap_aval) {
            if (c->d.aval) cudaFree(c->d.aval);
            c->d.aval = nullptr;
            c->d.cap_aval = 0;
            MPH_CUDA(cudaMalloc(&c->d.aval, (size_t)cap * D * D * sizeof(double)));
            c->d.cap_aval = cap;
        }
        if (need32 && cap > c->d.cap_aval32) {
            if (c->d.aval32) cudaFree(c->d.aval32);
            c->d.aval32 = nullptr;
            c->d.cap_aval32 = 0;
            MPH_CUDA(cudaMalloc(&c->d.aval32, (size_t)cap * D * D * sizeof(float)));
            c->d.cap_aval32 = cap;
        }
        if (!need64 && c->d.aval) {   // a form change (option) since the last step: release what is unused
            cudaFree(c->d.aval);
            c->d.aval = nullptr;
            c->d.cap_aval = 0;
        }
        if (!need32 && c->d.aval32) {
            cudaFree(c->d.aval32);
            c->d.aval32 = nullptr;
            c->d.cap_aval32 = 0;
        }
    }
    // C values for the fluid rows (aligned with the P-list)
    long long h_cn = 0;
    MPH_CUDA(cudaMemcpyAsync(&h_cn, c->d.nptrP + Nf, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    {
        void* p = c->d.cval;
        MPH_TRY(ensure(&p, &c->d.cap_cval, h_cn * D, sizeof(double)));
        c->d.cval = (double*)p;
    }
    const unsigned gf = grid_for(Nf, 128);
    const unsigned ga = grid_for(P.N, 128);
    Level0Map M{};
    const mph::LevelGeom& g0 = c->lv[0];
    M.S = 1;
    M.folded = 0;
    for (int d = 0; d < 3; ++d) {
        M.mn[d] = g0.mn[d];
        M.cnt[d] = g0.cnt[d];
        M.st[d] = g0.st[d];
        M.S *= g0.st[d];
        if (d < D && g0.cnt[d] < 3) M.folded = 1;
    }
    if (D == 2) {
        { k_matrix_c<2><<<gf, 128, 0, c->stream>>>(P, c->d.pos, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.cval); MPH_COUNT_LAUNCH(); }
        { k_vector_p<2><<<ga, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.vsp, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.pvec); MPH_COUNT_LAUNCH(); }
    } else {
        { k_matrix_c<3><<<gf, 128, 0, c->stream>>>(P, c->d.pos, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.cval); MPH_COUNT_LAUNCH(); }
        { k_vector_p<3><<<ga, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.vsp, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.pvec); MPH_COUNT_LAUNCH(); }
    }
    // A: the cell-block kernel where it applies; the per-row kernel for the
    // rows of cells it flags (or for every row when it does not apply)
    cudaEvent_t pe = nullptr;
    const int pon = prof_begin(c, 2, &pe);
    bool cells = false;
    c->ct_ready = false;
    c->level0_done = false;
    if (c->step_factored) {
        // mixed form: FP64 pair terms and b, transposed P-lists (the factored
        // FP64 operator), then FP32 blocks only
        MPH_TRY(build_ct(c));
        if (c->step_pairs) MPH_TRY(launch_ct_slices(c));
        MPH_TRY(launch_pair_terms(c));
    }
    // the pair path of the point-Jacobi mixed form has all it needs (b and
    // D^-1 from k_pair_terms): no level-0 stencils, no per-row kernel
    const bool skip_rows = c->step_pairs && mixed_jacobi(c);
    if (c->cell_assembly && !skip_rows) {
        if (c->step_pairs) MPH_TRY(launch_part_pairs(c, M, &cells));   // no blocks: level-0 stencils and D^-1 only
        else MPH_TRY(launch_assemble_cells(c, kmax_rows, c->step_factored, &cells));
    }
    const int* only = cells ? c->d.cell_flags : nullptr;
    if (skip_rows) {
        if (c->step_pairs) MPH_TRY(launch_pairs_to_slices(c));
        if (pon) prof_end(c, 2, pe);
        return MPH_OK;
    }
    float* a32 = c->precision == MPH_PRECISION_MIXED ? c->d.aval32 : nullptr;   // null on the pair path
    if (D == 2) {
        { k_matrix_a<2><<<gf, 128, 0, c->stream>>>(P, M, only, c->d.type, c->d.key, c->d.pos, c->d.vel, c->d.force, c->d.nc, c->d.nfc,
                                                 c->d.nptr, c->d.nind, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.cval, c->d.pvec, c->d.sptr,
                                                 c->d.acol, c->d.aval, a32, c->d.bvec, c->d.invDiag, c->d.selfk, c->d.part); MPH_COUNT_LAUNCH(); }
    } else {
        { k_matrix_a<3><<<gf, 128, 0, c->stream>>>(P, M, only, c->d.type, c->d.key, c->d.pos, c->d.vel, c->d.force, c->d.nc, c->d.nfc,
                                                 c->d.nptr, c->d.nind, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.cval, c->d.pvec, c->d.sptr,
                                                 c->d.acol, c->d.aval, a32, c->d.bvec, c->d.invDiag, c->d.selfk, c->d.part); MPH_COUNT_LAUNCH(); }
    }
    if (c->step_pairs) MPH_TRY(launch_pairs_to_slices(c));
    if (pon) prof_end(c, 2, pe);
    return MPH_OK;
}

}  // namespace mph
