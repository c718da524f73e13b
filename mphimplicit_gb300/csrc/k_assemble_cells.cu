// k_assemble_cells.cu - block assembly of A, one thread block per cell.
//
// The same matrix as k_matrix_a (calculateMatrixA main.cpp:2251-2335 plus
// multiplyMatrixC main.cpp:2574-2642), organised for the GPU:
//
//  * C Lambda C^T is gathered column by column instead of by pairwise
//    merge-joins: for every P-neighbour k of row i the contribution
//    (C_ik Lambda_k) (x) C_jk goes to block (i, j) for every fluid row j whose
//    P-list contains k.  Those rows come from the transpose of the fluid
//    P-lists (built exactly, then sorted by row), so each row takes about
//    |P|^2 updates instead of |N|*2|P| merge steps.
//  * The neighbours of every row of a cell are a subsequence of the fluid
//    particles of the cell's 3^D neighbour cells, in the same order.  Each
//    row keeps a bitmask over that candidate set; the slot of j in row i is
//    a popcount prefix, O(1).
//  * One warp per row accumulates the row's blocks in shared memory (each
//    update of one column touches distinct slots, so the warp needs no
//    atomics and the summation order is fixed), then writes the sliced-ELL
//    blocks, b, D^-1 and the level-0 partial stencils.
// Cells whose candidate set or rows exceed the shared-memory budget, and
// grids with fewer than 3 cells along an axis (where the cell walk visits a
// cell twice), are assembled by k_matrix_a instead.
#include <type_traits>

#include "mph_device.cuh"

namespace mph {

// ---- exact transpose of the fluid rows' P-lists ------------------------------
__global__ void k_ct_count(int Nf, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
                           const int* __restrict__ nindP, int* __restrict__ cnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nf) return;
    const long long b = nptrP[i];
    for (int a = 0; a < ncp[i]; ++a) atomicAdd(&cnt[nindP[b + a]], 1);
}

// column entries in arrival order: row j, column k and the entry's P-list slot
__global__ void k_ct_fill(int Nf, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
                          const int* __restrict__ nindP, const long long* __restrict__ ctptr, int* __restrict__ cur,
                          int3* __restrict__ tmp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nf) return;
    const long long b = nptrP[i];
    for (int a = 0; a < ncp[i]; ++a) {
        const int k = nindP[b + a];
        const long long e = ctptr[k] + atomicAdd(&cur[k], 1);
        tmp[e] = make_int3(i, k, (int)(b + a));
    }
}

// every entry finds its place in its column (rows ascending: its rank among
// the column's rows, which are distinct) and copies its C values there
template <int D>
__global__ void k_ct_place(long long total, const long long* __restrict__ ctptr, const int3* __restrict__ tmp,
                           const double* __restrict__ cval, int* __restrict__ ct_j, double* __restrict__ ct_v)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int3 t = tmp[e];
    const long long e0 = ctptr[t.y], e1 = ctptr[t.y + 1];
    int rank = 0;
    for (long long f = e0; f < e1; ++f) rank += tmp[f].x < t.x;
    const long long d = e0 + rank;
    ct_j[d] = t.x;
#pragma unroll
    for (int r = 0; r < D; ++r) ct_v[d * D + r] = cval[(long long)t.z * D + r];
}

__global__ void k_to_f32(long long n, const double* __restrict__ a, float* __restrict__ b)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = (float)a[k];
}

// ---- the cell-block assembly ------------------------------------------------------
struct CellMap {
    int mn[3], cnt[3], st[3];
    int S;
};

constexpr int kAsmWarps = 4;

// MIX = false: the FP64 blocks (and their FP32 copy when aval32 is given), b
// and D^-1.  MIX = true (mixed form with the factored FP64 operator): FP32
// arithmetic throughout, the viscous blocks from the FP32 pair terms pe32
// (e, f), only the FP32 blocks, D^-1 and the level-0 stencils are written
// (b comes from k_pair_terms).
template <int D, bool MIX>
__global__ void __launch_bounds__(kAsmWarps * 32)
k_assemble_cells(DevParams P, CellMap M, int rx, int ry, int rz, int mwords, int kmax, const int* __restrict__ type,
                 const int* __restrict__ bucket, const double* __restrict__ pos, const double* __restrict__ vel,
                 const int* __restrict__ nc, const int* __restrict__ nfc, const long long* __restrict__ nptr,
                 const int* __restrict__ nind, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
                 const int* __restrict__ nindP, const double* __restrict__ cval, const double* __restrict__ pvec,
                 const long long* __restrict__ ctptr, const int* __restrict__ ct_j, const double* __restrict__ ct_v,
                 const long long* __restrict__ sptr, int* __restrict__ acol, double* __restrict__ aval,
                 float* __restrict__ aval32, double* __restrict__ bvec, double* __restrict__ invDiag,
                 int* __restrict__ selfk_out, double* __restrict__ part, int* __restrict__ overflow,
                 const float4* __restrict__ pe32, const float* __restrict__ ct_v32, const float* __restrict__ cval32,
                 float* __restrict__ arow32)
{
    using T = typename std::conditional<MIX, float, double>::type;
    constexpr int DD = D * D;
    const int c = blockIdx.x;
    const int r0 = bucket[c], r1 = bucket[c + 1];
    if (r0 == r1) return;
    __shared__ int wb0[27], wb1[27], woff[28], wslot[27];
    __shared__ int nwalk;
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* acc = reinterpret_cast<T*>(reinterpret_cast<char*>(smem) +
                                  (size_t)warp * ((size_t)kmax * DD * sizeof(T) + (size_t)mwords * 8));
    unsigned* mask = reinterpret_cast<unsigned*>(acc + (size_t)kmax * DD);
    int* wpre = reinterpret_cast<int*>(mask + mwords);

    if (threadIdx.x == 0) {
        // the cell walk of the neighbour search (ascending cell index per axis)
        int ic[3];
        key_coords(P, c, ic);
        const int range[3] = {rx, ry, rz};
        int lo[3], n[3], cells[3][3];
        for (int d = 0; d < 3; ++d) {
            n[d] = 2 * range[d] + 1;
            for (int j = 0; j < n[d]; ++j) cells[d][j] = wrapc(ic[d] - range[d] + j, P.cc[d]);
            const int b = 2 * range[d] - (ic[d] + range[d]) % P.cc[d];
            lo[d] = b > 0 ? b : 0;
        }
        int s = 0, off = 0;
        for (int jx = lo[0]; jx < lo[0] + n[0]; ++jx)
            for (int jy = lo[1]; jy < lo[1] + n[1]; ++jy)
                for (int jz = lo[2]; jz < lo[2] + n[2]; ++jz) {
                    const int cx = cells[0][jx % n[0]], cy = cells[1][jy % n[1]], cz = cells[2][jz % n[2]];
                    const int jc = cell_id(P, cx, cy, cz);
                    wb0[s] = bucket[jc];
                    wb1[s] = bucket[jc + 1];
                    woff[s] = off;
                    off += wb1[s] - wb0[s];
                    const int jcc[3] = {cx, cy, cz};
                    int o[3];
                    for (int d = 0; d < 3; ++d) o[d] = ((jcc[d] - M.mn[d]) - (ic[d] - M.mn[d]) + 1 + M.cnt[d]) % M.cnt[d];
                    wslot[s] = M.st[2] * M.st[1] * o[0] + M.st[2] * o[1] + o[2];
                    ++s;
                }
        woff[s] = off;
        nwalk = s;
        if (off > mwords * 32) overflow[c] = 1;
    }
    __syncthreads();
    if (woff[nwalk] > mwords * 32) return;
    const int nw = nwalk;
    const int mc = woff[nw];
    auto local_of = [&](int j) -> int {   // candidate index of particle j, or -1
        int lo = 0, hi = nw - 1;
        while (lo < hi) {                  // largest s with wb0[s] <= j
            const int mid = (lo + hi + 1) >> 1;
            if (wb0[mid] <= j) lo = mid; else hi = mid - 1;
        }
        if (j < wb0[lo] || j >= wb1[lo]) return -1;
        return woff[lo] + (j - wb0[lo]);
    };
    auto rank_of = [&](int x) -> int {     // set bits below candidate index x
        const int w = x >> 5, b = x & 31;
        return wpre[w] + __popc(mask[w] & ((1u << b) - 1u));
    };
    const double rV2 = P.rV * P.rV;

    for (int i = r0 + warp; i < r1; i += kAsmWarps) {
        const int n = nc[i], nf = nfc[i];
        if (nf > kmax) {
            if (lane == 0) overflow[c] = 1;
            continue;
        }
        const long long nb = nptr[i];
        // 1. membership mask of the row's fluid neighbours, and its word prefix
        for (int w = lane; w < mwords; w += 32) mask[w] = 0u;
        __syncwarp();
        for (int k = lane; k < nf; k += 32) {
            const int l = local_of(nind[nb + k]);
            atomicOr(&mask[l >> 5], 1u << (l & 31));
        }
        __syncwarp();
        {
            const int per = (mwords + 31) / 32;
            int s = 0;
            for (int w = lane * per; w < min(mwords, (lane + 1) * per); ++w) s += __popc(mask[w]);
            int incl = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            int run = incl - s;
            for (int w = lane * per; w < min(mwords, (lane + 1) * per); ++w) {
                wpre[w] = run;
                run += __popc(mask[w]);
            }
        }
        for (int t = lane; t < nf * DD; t += 32) acc[t] = T(0);
        __syncwarp();
        // 2. viscous blocks (main.cpp:2261-2304)
        const int ti = type[i];
        double xi[3], vi[3];
        if (!MIX) {
            load_vec<D>(pos, i, xi);
            load_vec<D>(vel, i, vi);
        }
        T selfc[DD];
        double sumv[3] = {0, 0, 0};
#pragma unroll
        for (int t = 0; t < DD; ++t) selfc[t] = T(0);
        int myself = -1;
        for (int k = lane; k < n; k += 32) {
            const int j = nind[nb + k];
            if (j == i) { myself = k; continue; }
            if (MIX) {
                const float4 pt = pe32[nb + k];
                const float e[3] = {pt.x, pt.y, pt.z};
                const bool fluid = k < nf;
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int s = 0; s < D; ++s) {
                        const float coef = pt.w * e[s] * e[r];
                        selfc[r * D + s] += coef;
                        if (fluid) acc[k * DD + r * D + s] = -coef;
                    }
                continue;
            }
            double xj[3], q[3];
            load_vec<D>(pos, j, xj);
            sep_vec<D>(P, xj, xi, q);
            const double r2 = norm2_exact<D>(q);
            if (!r2_pos_below(r2, rV2)) continue;
            const double inv = rsqrt(r2);
            const double wd = -P.kfv * (P.m2h_rv * (1.0 - (r2 * inv) * P.inv_rv));
            const double f = P.visc * P.muij[ti][type[j]] * wd * inv;
            double e[3];
#pragma unroll
            for (int d = 0; d < D; ++d) e[d] = q[d] * inv;
            const bool fluid = k < nf;
            double vj[3];
            if (!fluid) load_vec<D>(vel, j, vj);
            // the block f e (x) e is symmetric: the upper triangle is formed once
            // (f e_r first, then times e_s) and mirrored
            double fe[3];
#pragma unroll
            for (int r = 0; r < D; ++r) fe[r] = f * e[r];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = r; s < D; ++s) {
                    const double coef = fe[r] * e[s];
                    selfc[r * D + s] += (T)coef;
                    if (fluid) {
                        acc[k * DD + r * D + s] = (T)-coef;
                        if (s != r) acc[k * DD + s * D + r] = (T)-coef;
                    } else {
                        sumv[r] += coef * vj[s];
                        if (s != r) sumv[s] += coef * vj[r];
                    }
                }
        }
        // warp sums of the upper triangle, mirrored (the FP32 form sums all entries)
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int s = 0; s < D; ++s) {
                if (!MIX && s < r) continue;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) selfc[r * D + s] += __shfl_xor_sync(0xffffffffu, selfc[r * D + s], o);
            }
        if (!MIX) {
#pragma unroll
            for (int r = 1; r < D; ++r)
#pragma unroll
                for (int s = 0; s < r; ++s) selfc[r * D + s] = selfc[s * D + r];
        }
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sumv[r] += __shfl_xor_sync(0xffffffffu, sumv[r], o);
        const int self = __reduce_max_sync(0xffffffffu, myself);
        // inertia density/dt as the reference forms it, (rho*vol)/vol/dt,
        // formed once on the host (its FP32 rounding for the FP32 form)
        const T inert = MIX ? (T)P.inert32[ti] : (T)P.inert64[ti];
        __syncwarp();
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int s = 0; s < D; ++s) acc[self * DD + r * D + s] = selfc[r * D + s] + (r == s ? (T)inert : T(0));
        }
        __syncwarp();
        // sliced-ELL write-out of the row's blocks (the FP32 form writes them
        // only when its inner SpMV uses them)
        auto write_blocks = [&]() {
            if (MIX) {   // row-contiguous, coalesced; k_rows_to_slices builds the sliced layout
                float* dst = arow32 + nb * DD;
                for (int t = lane; t < nf * DD; t += 32) dst[t] = (float)acc[t];
                __syncwarp();
                return;
            }
            const long long sb = sptr[i >> 5];
            const int ln = i & 31;
            for (int t = lane; t < nf * DD; t += 32) {
                const int k = t / DD, rs = t - k * DD;
                const long long at = sb * DD + ((long long)k * DD + rs) * 32 + ln;
                if (MIX) {
                    aval32[at] = (float)acc[t];
                } else {
                    aval[at] = (double)acc[t];
                    if (aval32) aval32[at] = (float)acc[t];
                }
            }
            for (int k = lane; k < nf; k += 32) acol[sb + (long long)k * 32 + ln] = nind[nb + k];
            __syncwarp();
        };
        // 3. C Lambda C^T, one P-neighbour column at a time (main.cpp:2590-2641)
        const long long pb = nptrP[i];
        const int np = ncp[i];
        for (int a = 0; a < np; ++a) {
            const int k = nindP[pb + a];
            T ga[3];
            if (MIX) {
                const float lam = P.lambda32[type[k]];
#pragma unroll
                for (int r = 0; r < D; ++r) ga[r] = cval32[(pb + a) * D + r] * lam;
            } else {
                const double lam = P.lambda[type[k]];
#pragma unroll
                for (int r = 0; r < D; ++r) ga[r] = (T)(cval[(pb + a) * D + r] * lam);
            }
            const long long e0 = ctptr[k], e1 = ctptr[k + 1];
            for (long long e = e0 + lane; e < e1; e += 32) {
                const int l = local_of(ct_j[e]);
                if (l < 0 || !((mask[l >> 5] >> (l & 31)) & 1u)) continue;
                const int slot = rank_of(l);
                T cj[3];
                if (MIX) {
#pragma unroll
                    for (int s = 0; s < D; ++s) cj[s] = (T)ct_v32[e * D + s];
                } else {
#pragma unroll
                    for (int s = 0; s < D; ++s) cj[s] = (T)ct_v[e * D + s];
                }
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int s = 0; s < D; ++s) acc[slot * DD + r * D + s] += ga[r] * cj[s];
            }
            __syncwarp();
        }
        // 4. b: wall terms + inertia - C p (main.cpp:2318-2333, 2574-2584)
        double cp[3] = {0, 0, 0};
        for (int a = lane; a < (MIX ? 0 : np); a += 32) {
            const double pk = pvec[nindP[pb + a]];
#pragma unroll
            for (int r = 0; r < D; ++r) cp[r] += cval[(pb + a) * D + r] * pk;
        }
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) cp[r] += __shfl_xor_sync(0xffffffffu, cp[r], o);
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < D; ++r) {
                if (!MIX) bvec[(size_t)i * D + r] = (sumv[r] + (double)inert * vi[r]) - cp[r];
                const T dg = acc[self * DD + r * D + r];
                invDiag[(size_t)i * D + r] = (double)(dg != T(0) ? T(1) / dg : T(0));
            }
            selfk_out[i] = self;
        }
        // 5. level-0 partial stencils: the row's blocks summed per neighbour cell
        for (int t = lane; t < nw * DD; t += 32) {
            const int s = t / DD, rs = t % DD;
            const int k0 = rank_of(woff[s]);
            const int k1 = woff[s + 1] >= mc ? nf : rank_of(woff[s + 1]);
            T sum = T(0);
            for (int k = k0; k < k1; ++k) sum += acc[k * DD + rs];
            part[((size_t)i * M.S + wslot[s]) * DD + rs] = (double)sum;
        }
        // 6. sliced-ELL write-out of the full blocks
        if (!(MIX && !aval32)) write_blocks();
        __syncwarp();
    }
}

// ---- row-contiguous FP32 blocks -> sliced ELL --------------------------------------
// One block per slice of 32 rows: chunks of kRtsK block columns of the 32 rows
// are read row by row (coalesced) into shared memory and written in the
// sliced layout (coalesced), together with the block columns from the
// neighbour lists; padding slots are written as zeros so every sector is
// written whole.
constexpr int kRtsK = 16;

template <int D>
__global__ void __launch_bounds__(256) k_rows_to_slices(int Nf, const long long* __restrict__ sptr, const int* __restrict__ nfc, const long long* __restrict__ nptr,
                                                        const int* __restrict__ nind, const float* __restrict__ arow32,
                                                        int* __restrict__ acol, float* __restrict__ aval32)
{
    constexpr int DD = D * D;
    constexpr int W = kRtsK * DD + 1;          // odd row stride: no bank conflicts
    __shared__ float tile[32 * W];
    __shared__ int ctile[32 * (kRtsK + 1)];
    __shared__ int rn[32];
    __shared__ long long rb[32];
    const int sl = blockIdx.x;
    const int r0 = sl * 32;
    if (threadIdx.x < 32) {
        const int i = r0 + threadIdx.x;
        rn[threadIdx.x] = i < Nf ? nfc[i] : 0;
        rb[threadIdx.x] = i < Nf ? nptr[i] : 0;
    }
    __syncthreads();
    const long long sb = sptr[sl];
    const int w = (int)((sptr[sl + 1] - sb) / 32);   // block columns of the slice (its slots / 32 rows)
    for (int k0 = 0; k0 < w; k0 += kRtsK) {
        const int kc = min(kRtsK, w - k0);
        for (int t = threadIdx.x; t < 32 * kRtsK * DD; t += blockDim.x) {
            const int r = t / (kRtsK * DD), e = t % (kRtsK * DD);
            const int k = k0 + e / DD;
            tile[r * W + e] = (e < kc * DD && k < rn[r]) ? arow32[(rb[r] + k0) * DD + e] : 0.f;
        }
        for (int t = threadIdx.x; t < 32 * kRtsK; t += blockDim.x) {
            const int r = t / kRtsK, e = t % kRtsK;
            ctile[r * (kRtsK + 1) + e] = (e < kc && k0 + e < rn[r]) ? nind[rb[r] + k0 + e] : 0;
        }
        __syncthreads();
        for (int o = threadIdx.x; o < kc * DD * 32; o += blockDim.x) {
            const int ln = o & 31, ec = o >> 5;                    // ec = k_local*DD + comp
            aval32[sb * DD + (long long)k0 * DD * 32 + o] = tile[ln * W + ec];
        }
        for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
            const int ln = o & 31, kl = o >> 5;
            acol[sb + (long long)(k0 + kl) * 32 + ln] = ctile[ln * (kRtsK + 1) + kl];
        }
        __syncthreads();
    }
}

// ---- launcher ---------------------------------------------------------------------
static int grow_bytes(void** p, long long* cap, long long need)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 1024;
    MPH_CUDA(cudaMalloc(p, (size_t)n));
    *cap = n;
    return MPH_OK;
}

// Transpose of the fluid rows' P-lists: for every particle k, the fluid rows
// j whose P-list holds k, in ascending j, with C_jk.  Built once per step.
int build_ct(mph_case* c)
{
    if (c->ct_ready) return MPH_OK;
    const DevParams& P = c->dp;
    const int D = c->dim;
    DeviceState& dv = c->d;
    const int N = P.N, Nf = P.Nf;
    MPH_TRY(grow_bytes((void**)&dv.ct_cnt, &dv.cap_ct_cnt, (long long)2 * (N + 1) * sizeof(int)));
    MPH_TRY(grow_bytes((void**)&dv.ct_ptr, &dv.cap_ct_ptr, (long long)(N + 1) * sizeof(long long)));
    long long tot = 0;
    MPH_CUDA(cudaMemcpyAsync(&tot, dv.nptrP + Nf, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemsetAsync(dv.ct_cnt, 0, (size_t)2 * (N + 1) * sizeof(int), c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    MPH_TRY(grow_bytes((void**)&dv.ct_j, &dv.cap_ct_j, tot * (long long)sizeof(int)));
    MPH_TRY(grow_bytes((void**)&dv.ct_v, &dv.cap_ct_v, tot * D * (long long)sizeof(double)));
    MPH_TRY(grow_bytes((void**)&dv.ct_tmp, &dv.cap_ct_tmp, tot * (long long)sizeof(int3)));
    int* cnt = dv.ct_cnt;
    int* cur = dv.ct_cnt + (N + 1);
    const unsigned gf = grid_for(Nf, 256);
    { k_ct_count<<<gf, 256, 0, c->stream>>>(Nf, dv.ncp, dv.nptrP, dv.nindP, cnt); MPH_COUNT_LAUNCH(); }
    MPH_TRY(launch_scan_i32_to_i64(c, cnt, dv.ct_ptr, N));
    { k_ct_fill<<<gf, 256, 0, c->stream>>>(Nf, dv.ncp, dv.nptrP, dv.nindP, dv.ct_ptr, cur, (int3*)dv.ct_tmp); MPH_COUNT_LAUNCH(); }
    if (D == 2) {
        { k_ct_place<2><<<grid_for(tot, 256), 256, 0, c->stream>>>(tot, dv.ct_ptr, (const int3*)dv.ct_tmp, dv.cval, dv.ct_j, dv.ct_v); MPH_COUNT_LAUNCH(); }
    } else {
        { k_ct_place<3><<<grid_for(tot, 256), 256, 0, c->stream>>>(tot, dv.ct_ptr, (const int3*)dv.ct_tmp, dv.cval, dv.ct_j, dv.ct_v); MPH_COUNT_LAUNCH(); }
    }
    if (c->step_factored) {   // FP32 copy for the FP32 cell-block kernel
        MPH_TRY(grow_bytes((void**)&dv.ct_v32, &dv.cap_ct_v32, tot * D * (long long)sizeof(float)));
        { k_to_f32<<<grid_for(tot * D, 256), 256, 0, c->stream>>>(tot * D, dv.ct_v, dv.ct_v32); MPH_COUNT_LAUNCH(); }
    }
    c->ct_ready = true;
    return MPH_OK;
}

// Runs the cell-block kernel (FP32 form when `mix`); returns MPH_OK with
// *done = false when the case needs k_matrix_a for all rows, and leaves
// per-cell overflow flags in c->d.cell_flags otherwise.
int launch_assemble_cells(mph_case* c, int kmax_rows, bool mix, bool* done)
{
    *done = false;
    const DevParams& P = c->dp;
    const int D = c->dim;
    const LevelGeom& g0 = c->lv[0];
    for (int d = 0; d < D; ++d)
        if (P.cc[d] < 3 || g0.cnt[d] < 3) return MPH_OK;   // walk visits a cell twice: per-row kernel
    const int kmax = (kmax_rows + 7) & ~7;
    const int mwords = 64;                                 // up to 2048 candidates per cell
    const size_t smem = (size_t)kAsmWarps * ((size_t)kmax * D * D * (mix ? 4 : 8) + (size_t)mwords * 8);
    if (smem > 200 * 1024) return MPH_OK;
    DeviceState& dv = c->d;
    MPH_TRY(grow_bytes((void**)&dv.cell_flags, &dv.cap_cell_flags, (long long)(P.T + 1) * sizeof(int)));
    MPH_CUDA(cudaMemsetAsync(dv.cell_flags, 0, (size_t)(P.T + 1) * sizeof(int), c->stream));
    MPH_TRY(build_ct(c));
    CellMap M{};
    M.S = 1;
    for (int d = 0; d < 3; ++d) {
        M.mn[d] = g0.mn[d];
        M.cnt[d] = g0.cnt[d];
        M.st[d] = g0.st[d];
        M.S *= g0.st[d];
    }
    int r[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) r[d] = (int)std::ceil(P.maxR / P.cw[d]);
    // FP32 blocks: the mixed form's copy, except when its inner operator runs
    // on the sliced pair terms
    float* a32 = c->precision == MPH_PRECISION_MIXED && !c->step_pairs ? dv.aval32 : nullptr;
    if (mix && a32) {   // FP32 blocks go through the row-contiguous buffer
        long long slots = 0;
        MPH_CUDA(cudaMemcpyAsync(&slots, dv.nptr + P.Nf, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
        MPH_CUDA(cudaStreamSynchronize(c->stream));
        MPH_TRY(grow_bytes((void**)&dv.arow32, &dv.cap_arow32, slots * D * D * (long long)sizeof(float)));
    }
    // the attribute is per function and device, shared by the cases (and the
    // host threads of a batch or a server): always the device's opt-in limit
    // less the kernel's static shared memory
    int optin = 0;
    MPH_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    auto go = [&](auto kern) {
        cudaFuncAttributes fa;
        cudaFuncGetAttributes(&fa, kern);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
        kern<<<P.T, kAsmWarps * 32, smem, c->stream>>>(
            P, M, r[0], r[1], r[2], mwords, kmax, dv.type, dv.bucket, dv.pos, dv.vel, dv.nc, dv.nfc, dv.nptr, dv.nind, dv.ncp,
            dv.nptrP, dv.nindP, dv.cval, dv.pvec, dv.ct_ptr, dv.ct_j, dv.ct_v, dv.sptr, dv.acol, dv.aval, a32, dv.bvec,
            dv.invDiag, dv.selfk, dv.part, dv.cell_flags, dv.pe32, dv.ct_v32, dv.cval32, dv.arow32);
        MPH_COUNT_LAUNCH();
    };
    if (D == 2) {
        if (mix) go(k_assemble_cells<2, true>); else go(k_assemble_cells<2, false>);
    } else {
        if (mix) go(k_assemble_cells<3, true>); else go(k_assemble_cells<3, false>);
    }
    if (mix && a32) {
        if (D == 2) {
            k_rows_to_slices<2><<<c->nslices, 256, 0, c->stream>>>(P.Nf, dv.sptr, dv.nfc, dv.nptr, dv.nind, dv.arow32,
                                                                   dv.acol, a32);
        } else {
            k_rows_to_slices<3><<<c->nslices, 256, 0, c->stream>>>(P.Nf, dv.sptr, dv.nfc, dv.nptr, dv.nind, dv.arow32,
                                                                   dv.acol, a32);
        }
        MPH_COUNT_LAUNCH();
    }
    *done = true;
    return MPH_OK;
}

}  // namespace mph
