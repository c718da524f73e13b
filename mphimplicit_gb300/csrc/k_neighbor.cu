// k_neighbor.cu - neighbour lists (calculateNeighbor, main.cpp:1382-1667)
// and the device scan used for every CSR row pointer.
//
// One thread per particle walks the 3^D neighbour cells in the reference's
// order (ascending cell index along each axis, fluid cells first, then wall
// cells), so the lists come out in the reference's order.  Candidates are
// first classified with FP32 positions; a pair whose FP32 squared distance
// lies inside a conservative band around MaxRadius^2 or RadiusP^2 is decided
// by the reference's exact FP64 expression.  The band is derived from the
// coordinate magnitudes at case creation (or the FP32 step is disabled).
#include "mph_device.cuh"

namespace mph {

struct Walk {
    int lo[3], n[3], cells[3][3];
};

__device__ __forceinline__ void make_walk(const DevParams& P, const int* range, int k, Walk& w)
{
    int ic[3];
    key_coords(P, k, ic);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        w.n[d] = 2 * range[d] + 1;
        for (int j = 0; j < w.n[d]; ++j) w.cells[d][j] = wrapc(ic[d] - range[d] + j, P.cc[d]);
        const int b = 2 * range[d] - (ic[d] + range[d]) % P.cc[d];
        w.lo[d] = b > 0 ? b : 0;
    }
}

// classification of candidate j for particle i: bit0 = within MaxRadius,
// bit1 = within RadiusP
template <int D>
__device__ __forceinline__ int classify(const DevParams& P, const double* xi, const float* xi32, const double* __restrict__ pos,
                                        const float* __restrict__ pos32, int j)
{
    if (!P.exact_only) {
        float d2;
        if (D == 2) {
            const float2 pj = reinterpret_cast<const float2*>(pos32)[j];
            float a = pj.x - xi32[0], b = pj.y - xi32[1];
            a = a > P.hw32[0] ? a - P.w32[0] : (a < -P.hw32[0] ? a + P.w32[0] : a);
            b = b > P.hw32[1] ? b - P.w32[1] : (b < -P.hw32[1] ? b + P.w32[1] : b);
            d2 = a * a + b * b;
        } else {
            const float4 pj = reinterpret_cast<const float4*>(pos32)[j];
            float a = pj.x - xi32[0], b = pj.y - xi32[1], e = pj.z - xi32[2];
            a = a > P.hw32[0] ? a - P.w32[0] : (a < -P.hw32[0] ? a + P.w32[0] : a);
            b = b > P.hw32[1] ? b - P.w32[1] : (b < -P.hw32[1] ? b + P.w32[1] : b);
            e = e > P.hw32[2] ? e - P.w32[2] : (e < -P.hw32[2] ? e + P.w32[2] : e);
            d2 = a * a + b * b + e * e;
        }
        if (d2 > P.maxR2_hi) return 0;
        const bool inM = d2 < P.maxR2_lo;
        const bool inP = d2 < P.rP2_lo;
        const bool outP = d2 > P.rP2_hi;
        if (inM && (inP || outP)) return 1 | (inP ? 2 : 0);
    }
    double xj[3], q[3];
    load_vec<D>(pos, j, xj);
    sep_vec<D>(P, xj, xi, q);
    const double r2 = norm2_exact<D>(q);
    if (!(r2 <= P.maxR2)) return 0;
    return 1 | (r2 <= P.rP2 ? 2 : 0);
}

template <int D>
__device__ __forceinline__ void load_xi32(const float* __restrict__ pos32, int i, float* x)
{
    if (D == 2) {
        const float2 t = reinterpret_cast<const float2*>(pos32)[i];
        x[0] = t.x; x[1] = t.y;
    } else {
        const float4 t = reinterpret_cast<const float4*>(pos32)[i];
        x[0] = t.x; x[1] = t.y; x[2] = t.z;
    }
}

// The list of particle i by one thread (count pass: nc, nfc, ncp; FILL:
// nind, nindP at nptr, nptrP).
template <int D, bool FILL>
__device__ void neighbors_one(const DevParams& P, int rx, int ry, int rz, int wB, int wE,
                              const int* __restrict__ key, const int* __restrict__ bucket,
                              const double* __restrict__ pos, const float* __restrict__ pos32,
                              int* __restrict__ nc, int* __restrict__ nfc, int* __restrict__ ncp,
                              const long long* __restrict__ nptr, const long long* __restrict__ nptrP,
                              int* __restrict__ nind, int* __restrict__ nindP, int i)
{
    const int range[3] = {rx, ry, rz};
    Walk w;
    make_walk(P, range, key[i], w);
    double xi[3];
    float xi32[3];
    load_vec<D>(pos, i, xi);
    load_xi32<D>(pos32, i, xi32);
    long long o = 0, op = 0;
    if (FILL) { o = nptr[i]; op = nptrP[i]; }
    int n = 0, np = 0;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            const int nn = FILL ? nc[i] : n;
            if (wB <= i && i < wE && nn == 0) break;   // wall particle without fluid neighbours
        }
        const int boff = pass == 0 ? 0 : P.T;
        for (int jx = w.lo[0]; jx < w.lo[0] + w.n[0]; ++jx)
            for (int jy = w.lo[1]; jy < w.lo[1] + w.n[1]; ++jy)
                for (int jz = w.lo[2]; jz < w.lo[2] + w.n[2]; ++jz) {
                    const int jc = cell_id(P, w.cells[0][jx % w.n[0]], w.cells[1][jy % w.n[1]], w.cells[2][jz % w.n[2]]);
                    const int j0 = bucket[boff + jc], j1 = bucket[boff + jc + 1];
                    for (int j = j0; j < j1; ++j) {
                        const int cl = classify<D>(P, xi, xi32, pos, pos32, j);
                        if (cl & 1) {
                            if (FILL) nind[o++] = j;
                            ++n;
                            if (cl & 2) {
                                if (FILL) nindP[op++] = j;
                                ++np;
                            }
                        }
                    }
                }
        if (pass == 0 && !FILL) nfc[i] = n;
    }
    if (!FILL) { nc[i] = n; ncp[i] = np; }
}

template <int D, bool FILL>
__global__ void __launch_bounds__(128) k_neighbors(DevParams P, int rx, int ry, int rz, int wB, int wE,
                                                   const int* __restrict__ key, const int* __restrict__ bucket,
                                                   const double* __restrict__ pos, const float* __restrict__ pos32,
                                                   int* __restrict__ nc, int* __restrict__ nfc, int* __restrict__ ncp,
                                                   const long long* __restrict__ nptr, const long long* __restrict__ nptrP,
                                                   int* __restrict__ nind, int* __restrict__ nindP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    neighbors_one<D, FILL>(P, rx, ry, rz, wB, wE, key, bucket, pos, pos32, nc, nfc, ncp, nptr, nptrP, nind, nindP, i);
}

// ---- one block per cell bucket -------------------------------------------------
// The particles of one bucket (the fluid or the wall particles of one cell)
// share their walk: the block stages the candidates of each pass (fluid
// buckets, then wall buckets of the 3^D cells, in the walk's order) in shared
// memory once, and a warp takes one particle at a time, its lanes on 32
// consecutive candidates; ballots keep the list order, so a list is the same
// as the per-thread walk's, written with coalesced stores.  A walk that does
// not wrap around the periodic grid (and a grid of at least 2 range + 3 cells
// on every axis) needs no minimum-image correction in FP32.  A bucket with
// more than kNbMaxP particles, a pass with more than kNbCap candidates, a walk
// of more than 27 cells or the exact-only mode runs the per-thread walk.
constexpr int kNbThreads = 256;
constexpr int kNbCap = 1536;
constexpr int kNbMaxP = 256;

// The FP32 squared distance of a staged candidate (the minimum image only
// for a walk that wraps), as classify computes it.
template <int D>
__device__ __forceinline__ float d2_staged(const DevParams& P, bool wrap, const float* xi32, const float4 pj)
{
    float a = pj.x - xi32[0], b = pj.y - xi32[1];
    if (D == 2) {
        if (wrap) {
            a = a > P.hw32[0] ? a - P.w32[0] : (a < -P.hw32[0] ? a + P.w32[0] : a);
            b = b > P.hw32[1] ? b - P.w32[1] : (b < -P.hw32[1] ? b + P.w32[1] : b);
        }
        return a * a + b * b;
    }
    float e = pj.z - xi32[2];
    if (wrap) {
        a = a > P.hw32[0] ? a - P.w32[0] : (a < -P.hw32[0] ? a + P.w32[0] : a);
        b = b > P.hw32[1] ? b - P.w32[1] : (b < -P.hw32[1] ? b + P.w32[1] : b);
        e = e > P.hw32[2] ? e - P.w32[2] : (e < -P.hw32[2] ? e + P.w32[2] : e);
    }
    return a * a + b * b + e * e;
}

// The reference's FP64 decision for a pair inside the FP32 band.
template <int D>
__device__ __forceinline__ int classify_exact(const DevParams& P, const double* __restrict__ pos, int i, int j)
{
    double xi[3], xj[3], q[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(pos, j, xj);
    sep_vec<D>(P, xj, xi, q);
    const double r2 = norm2_exact<D>(q);
    if (!(r2 <= P.maxR2)) return 0;
    return 1 | (r2 <= P.rP2 ? 2 : 0);
}

template <int D, bool FILL>
__global__ void __launch_bounds__(kNbThreads) k_neighbors_cells(DevParams P, int rx, int ry, int rz, int wB, int wE,
                                                                const int* __restrict__ key, const int* __restrict__ bucket,
                                                                const double* __restrict__ pos, const float* __restrict__ pos32,
                                                                int* __restrict__ nc, int* __restrict__ nfc, int* __restrict__ ncp,
                                                                const long long* __restrict__ nptr, const long long* __restrict__ nptrP,
                                                                int* __restrict__ nind, int* __restrict__ nindP)
{
    __shared__ float4 spos[kNbCap];
    __shared__ int sj[kNbCap];
    __shared__ int coff[2][28];
    __shared__ int cbeg[2][27];
    __shared__ int sn0[kNbMaxP], snp0[kNbMaxP];
    const int u = blockIdx.x;   // bucket = sort key: cell u (fluid) or u - T (wall)
    const int r0 = bucket[u], r1 = bucket[u + 1];
    if (r0 >= r1) return;
    const int tid = threadIdx.x, lane = tid & 31, wl = tid >> 5, nw = blockDim.x >> 5;
    const unsigned full = 0xffffffffu;
    const int range[3] = {rx, ry, rz};
    Walk w;
    make_walk(P, range, u, w);
    const int ncell = w.n[0] * w.n[1] * w.n[2];
    bool wrap = false;
    {
        int ic[3];
        key_coords(P, u, ic);
        for (int d = 0; d < D; ++d) {
            const int c = wrapc(ic[d], P.cc[d]);
            wrap = wrap || c - range[d] < 0 || c + range[d] >= P.cc[d] || P.cc[d] < 2 * range[d] + 3;
        }
    }
    bool slow = ncell > 27 || r1 - r0 > kNbMaxP;
    if (!slow) {
        if (tid < 64) {   // warp 0: the fluid buckets of the walk's cells, warp 1: the wall buckets
            const int pass = tid >> 5;
            int beg = 0, cnt = 0;
            if (lane < ncell) {
                const int a = lane / (w.n[1] * w.n[2]), b = (lane / w.n[2]) % w.n[1], z = lane % w.n[2];
                const int jx = w.lo[0] + a, jy = w.lo[1] + b, jz = w.lo[2] + z;
                const int jc = cell_id(P, w.cells[0][jx % w.n[0]], w.cells[1][jy % w.n[1]], w.cells[2][jz % w.n[2]]);
                beg = bucket[pass * P.T + jc];
                cnt = bucket[pass * P.T + jc + 1] - beg;
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane < ncell) {
                cbeg[pass][lane] = beg;
                coff[pass][lane + 1] = incl;
            }
            if (lane == 0) coff[pass][0] = 0;
        }
        __syncthreads();
        slow = coff[0][ncell] > kNbCap || coff[1][ncell] > kNbCap;
    }
    if (slow) {   // the same for every thread of the block
        for (int i = r0 + tid; i < r1; i += blockDim.x)
            neighbors_one<D, FILL>(P, rx, ry, rz, wB, wE, key, bucket, pos, pos32, nc, nfc, ncp, nptr, nptrP, nind, nindP, i);
        return;
    }
    for (int pass = 0; pass < 2; ++pass) {
        const int F = coff[pass][ncell];
        // candidates F.. up to a multiple of 32: far away, never neighbours
        for (int k = F + tid; k < ((F + 31) & ~31); k += blockDim.x) {
            spos[k] = make_float4(1e18f, 1e18f, 1e18f, 0.f);
            sj[k] = -1;
        }
        for (int t = wl; t < ncell; t += nw) {
            const int beg = cbeg[pass][t], off = coff[pass][t], cnt = coff[pass][t + 1] - off;
            for (int k = lane; k < cnt; k += 32) {
                const int j = beg + k;
                float4 pj;
                if (D == 2) {
                    const float2 q = reinterpret_cast<const float2*>(pos32)[j];
                    pj = make_float4(q.x, q.y, 0.f, 0.f);
                } else {
                    pj = reinterpret_cast<const float4*>(pos32)[j];
                }
                spos[off + k] = pj;
                sj[off + k] = j;
            }
        }
        __syncthreads();
        for (int pi = wl; pi < r1 - r0; pi += nw) {
            const int i = r0 + pi;
            int n = 0, np = 0;
            if (pass == 1) {
                n = sn0[pi];
                np = snp0[pi];
                if (wB <= i && i < wE && n == 0) {   // wall particle without fluid neighbours
                    if (!FILL && lane == 0) { nc[i] = 0; ncp[i] = 0; }
                    continue;
                }
            }
            int* outM = nullptr;
            int* outP = nullptr;
            if (FILL) { outM = nind + nptr[i]; outP = nindP + nptrP[i]; }
            float xi32[3] = {0.f, 0.f, 0.f};
            load_xi32<D>(pos32, i, xi32);
            const unsigned lt = (1u << lane) - 1u;
            for (int c0 = 0; c0 < F; c0 += 32) {
                const int c = c0 + lane;
                // FP32 first: far (> the band above MaxRadius^2), or inside
                // MaxRadius and clear of the RadiusP band; the rest exactly
                const float d2 = d2_staged<D>(P, wrap, xi32, spos[c]);
                const bool inM = d2 < P.maxR2_lo, inP = d2 < P.rP2_lo;
                const bool sure = d2 > P.maxR2_hi || (inM && (inP || d2 > P.rP2_hi));
                bool m = sure && inM, pp = sure && inP;
                if (__any_sync(full, !sure)) {
                    if (!sure) {
                        const int cl = classify_exact<D>(P, pos, i, sj[c]);
                        m = cl & 1;
                        pp = (cl & 2) != 0;
                    }
                }
                const unsigned bm = __ballot_sync(full, m), bp = __ballot_sync(full, pp);
                if (FILL) {
                    if (bm) {
                        const int j = sj[c];
                        if (m) outM[n + __popc(bm & lt)] = j;
                        if (pp) outP[np + __popc(bp & lt)] = j;
                    }
                }
                n += __popc(bm);
                np += __popc(bp);
            }
            if (lane == 0) {
                if (pass == 0) {
                    sn0[pi] = n;
                    snp0[pi] = np;
                    if (!FILL) nfc[i] = n;
                } else if (!FILL) {
                    nc[i] = n;
                    ncp[i] = np;
                }
            }
        }
        __syncthreads();   // the staged candidates are replaced; sn0 is read by the same warp
    }
}

// ---- scan: out[0] = 0, out[k+1] = in[0] + ... + in[k] (int32 -> int64) ----
constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

__device__ __forceinline__ long long warp_incl_scan(long long v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ __forceinline__ long long block_excl_scan(long long v, long long* total)
{
    __shared__ long long wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long incl = warp_incl_scan(v);
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        long long s = lane < kScanThreads / 32 ? wsum[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < kScanThreads / 32) wsum[lane] = s;
    }
    __syncthreads();
    const long long base = wid == 0 ? 0 : wsum[wid - 1];
    *total = wsum[kScanThreads / 32 - 1];
    __syncthreads();
    return base + incl - v;
}

__global__ void k_scan_reduce(const int* __restrict__ in, int n, long long* __restrict__ bsum)
{
    const long long b0 = (long long)blockIdx.x * kScanChunk;
    long long s = 0;
    for (int k = 0; k < kScanPer; ++k) {
        const long long idx = b0 + (long long)threadIdx.x * kScanPer + k;
        if (idx < n) s += in[idx];
    }
    long long tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// exclusive scan of the block sums by a single block (any count)
__global__ void k_scan_blocks(long long* __restrict__ bsum, int nb)
{
    long long carry = 0;
    for (int base = 0; base < nb; base += kScanThreads) {
        const int k = base + threadIdx.x;
        const long long v = k < nb ? bsum[k] : 0;
        long long tot;
        const long long ex = block_excl_scan(v, &tot);
        if (k < nb) bsum[k] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void k_scan_apply(const int* __restrict__ in, int n, const long long* __restrict__ bsum, long long* __restrict__ out)
{
    const long long b0 = (long long)blockIdx.x * kScanChunk;
    long long v[kScanPer];
    long long s = 0;
    for (int k = 0; k < kScanPer; ++k) {
        const long long idx = b0 + (long long)threadIdx.x * kScanPer + k;
        v[k] = idx < n ? in[idx] : 0;
        s += v[k];
    }
    long long tot;
    long long run = block_excl_scan(s, &tot) + bsum[blockIdx.x];
    if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = 0;
    for (int k = 0; k < kScanPer; ++k) {
        const long long idx = b0 + (long long)threadIdx.x * kScanPer + k;
        run += v[k];
        if (idx < n) out[idx + 1] = run;
    }
}

int launch_scan_i32_to_i64(mph_case* c, const int* in, long long* out, int n)
{
    const int nb = (n + kScanChunk - 1) / kScanChunk;
    const size_t need = (size_t)(nb + 1) * sizeof(long long);
    if (need > c->d.scan_tmp_bytes) {
        if (c->d.scan_tmp) cudaFree(c->d.scan_tmp);
        c->d.scan_tmp = nullptr;
        c->d.scan_tmp_bytes = 0;
        MPH_CUDA(cudaMalloc(&c->d.scan_tmp, need * 2));
        c->d.scan_tmp_bytes = need * 2;
    }
    long long* bsum = (long long*)c->d.scan_tmp;
    if (n == 0) {
        MPH_CUDA(cudaMemsetAsync(out, 0, sizeof(long long), c->stream));
        return MPH_OK;
    }
    { k_scan_reduce<<<nb, kScanThreads, 0, c->stream>>>(in, n, bsum); MPH_COUNT_LAUNCH(); }
    { k_scan_blocks<<<1, kScanThreads, 0, c->stream>>>(bsum, nb); MPH_COUNT_LAUNCH(); }
    { k_scan_apply<<<nb, kScanThreads, 0, c->stream>>>(in, n, bsum, out); MPH_COUNT_LAUNCH(); }
    return MPH_OK;
}

static void neighbor_ranges(const mph_case* c, int* r)
{
    for (int d = 0; d < 3; ++d) r[d] = 0;
    for (int d = 0; d < c->dim; ++d) {
        // (int)ceil(MaxRadius/CellWidth) as the reference (main.cpp:1393-1399)
        double q = c->dp.maxR / c->dp.cw[d];
        r[d] = (int)std::ceil(q);
    }
}

// one block per bucket (2 T of them), or the per-thread walk in the exact-only mode
template <bool FILL>
static void launch_neighbors_cells(mph_case* c, const int* r)
{
    const unsigned g = (unsigned)(2 * c->dp.T);
    DeviceState& d = c->d;
    if (c->dim == 2)
        k_neighbors_cells<2, FILL><<<g, kNbThreads, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, d.key, d.bucket, d.pos, d.pos32,
                                                                    d.nc, d.nfc, d.ncp, d.nptr, d.nptrP, d.nind, d.nindP);
    else
        k_neighbors_cells<3, FILL><<<g, kNbThreads, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, d.key, d.bucket, d.pos, d.pos32,
                                                                    d.nc, d.nfc, d.ncp, d.nptr, d.nptrP, d.nind, d.nindP);
    MPH_COUNT_LAUNCH();
}

void launch_neighbor_count(mph_case* c)
{
    int r[3];
    neighbor_ranges(c, r);
    if (!c->dp.exact_only && c->dp.T > 0) {
        launch_neighbors_cells<false>(c, r);
        return;
    }
    const unsigned g = grid_for(c->dp.N, 128);
    if (c->dim == 2)
        { k_neighbors<2, false><<<g, 128, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, c->d.key, c->d.bucket, c->d.pos,
                                                       c->d.pos32, c->d.nc, c->d.nfc, c->d.ncp, nullptr, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
    else
        { k_neighbors<3, false><<<g, 128, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, c->d.key, c->d.bucket, c->d.pos,
                                                       c->d.pos32, c->d.nc, c->d.nfc, c->d.ncp, nullptr, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
}

void launch_neighbor_fill(mph_case* c)
{
    int r[3];
    neighbor_ranges(c, r);
    if (!c->dp.exact_only && c->dp.T > 0) {
        launch_neighbors_cells<true>(c, r);
        return;
    }
    const unsigned g = grid_for(c->dp.N, 128);
    if (c->dim == 2)
        { k_neighbors<2, true><<<g, 128, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, c->d.key, c->d.bucket, c->d.pos,
                                                      c->d.pos32, c->d.nc, c->d.nfc, c->d.ncp, c->d.nptr, c->d.nptrP, c->d.nind, c->d.nindP); MPH_COUNT_LAUNCH(); }
    else
        { k_neighbors<3, true><<<g, 128, 0, c->stream>>>(c->dp, r[0], r[1], r[2], c->wB, c->wE, c->d.key, c->d.bucket, c->d.pos,
                                                      c->d.pos32, c->d.nc, c->d.nfc, c->d.ncp, c->d.nptr, c->d.nptrP, c->d.nind, c->d.nindP); MPH_COUNT_LAUNCH(); }
}

}  // namespace mph
