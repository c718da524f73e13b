// k_particles.cu - particle motion and the cell list.
//
//   step_begin      : calculateConvection / calculateWall /
//                     calculatePeriodicBoundary / resetForce
//                     (main.cpp:1678, 2089, 4741, 1690), one pass per particle
//   cell keys       : main.cpp:1171-1186
//   bitonic network : the reference's compare-exchange network
//                     (main.cpp:1190-1211), stage by stage, with every stage
//                     whose partner distance is inside a 4096-key tile run in
//                     shared memory; it reproduces the reference's permutation
//                     (the network is not stable, so a stable sort would not)
//   bucket ranges   : main.cpp:1213-1311 as one boundary scatter
//   permute         : main.cpp:1316-1378 as one SoA gather (+ the FP32
//                     position copy used by the neighbour pre-classification)
#include "mph_device.cuh"

namespace mph {

struct WallMotion {
    double c[4][3], v[4][3], w[4][3], R[4][3][3];
};

template <int D>
__global__ void k_step_begin(DevParams P, WallMotion W, double* __restrict__ pos, double* __restrict__ vel,
                             double* __restrict__ force, int fB, int fE, int wB, int wE,
                             const int* __restrict__ type)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    double x[3], v[3];
    load_vec<D>(pos, i, x);
    load_vec<D>(vel, i, v);
    if (i >= fB && i < fE) {                                   // calculateConvection
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = DADD(x[d], DMUL(v[d], P.dt));
    } else if (i >= wB && i < wE) {                            // calculateWall
        const int t = type[i];
        double r[3];
#pragma unroll
        for (int d = 0; d < D; ++d) r[d] = DSUB(x[d], W.c[t][d]);
        const double (&R)[3][3] = W.R[t];
        const double* w = W.w[t];
        if (D == 3) {
            // rotated in place, component by component (main.cpp:2108-2110)
            r[0] = DADD(DADD(DMUL(R[0][0], r[0]), DMUL(R[0][1], r[1])), DMUL(R[0][2], r[2]));
            r[1] = DADD(DADD(DMUL(R[1][0], r[0]), DMUL(R[1][1], r[1])), DMUL(R[1][2], r[2]));
            r[2] = DADD(DADD(DMUL(R[2][0], r[0]), DMUL(R[2][1], r[1])), DMUL(R[2][2], r[2]));
            v[0] = DADD(DSUB(DMUL(w[1], r[2]), DMUL(w[2], r[1])), W.v[t][0]);
            v[1] = DADD(DSUB(DMUL(w[2], r[0]), DMUL(w[0], r[2])), W.v[t][1]);
            v[2] = DADD(DSUB(DMUL(w[0], r[1]), DMUL(w[1], r[0])), W.v[t][2]);
        } else {
            // 2D cases rotate about z only (checked at case creation), so the
            // z terms of the reference's expressions are exact zeros
            r[0] = DADD(DMUL(R[0][0], r[0]), DMUL(R[0][1], r[1]));
            r[1] = DADD(DMUL(R[1][0], r[0]), DMUL(R[1][1], r[1]));
            v[0] = DADD(-DMUL(w[2], r[1]), W.v[t][0]);
            v[1] = DADD(DMUL(w[2], r[0]), W.v[t][1]);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = DADD(DADD(r[d], W.c[t][d]), DMUL(W.v[t][d], P.dt));
        store_vec<D>(vel, i, v);
    }
#pragma unroll
    for (int d = 0; d < D; ++d) x[d] = DADD(mod_exact(DSUB(x[d], P.dmin[d]), P.dw[d]), P.dmin[d]);
    store_vec<D>(pos, i, x);
    const double z[3] = {0.0, 0.0, 0.0};
    store_vec<D>(force, i, z);
}

template <int D>
__global__ void k_cell_keys(DevParams P, const double* __restrict__ pos, const int* __restrict__ type,
                            int* __restrict__ key, int* __restrict__ perm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.nPow) return;
    if (i < P.N) {
        double x[3];
        load_vec<D>(pos, i, x);
        int c[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < D; ++d) c[d] = ((int)floor(DDIV(DSUB(x[d], P.dmin[d]), P.cw[d]))) % P.cc[d];
        key[i] = cell_id(P, c[0], c[1], c[2]) + (is_wall(type[i]) ? P.T : 0);
        perm[i] = i;
    } else {
        key[i] = 2 * P.T;
        perm[i] = P.N;
    }
}

// ---- bitonic network -------------------------------------------------------
constexpr int kTile = 4096;
constexpr int kTileThreads = 1024;

__device__ __forceinline__ void cmp_swap(int* key, int* perm, int i, int j, bool asc)
{
    const int ki = key[i], kj = key[j];
    if ((ki > kj) == asc) {
        key[i] = kj; key[j] = ki;
        const int pi = perm[i];
        perm[i] = perm[j]; perm[j] = pi;
    }
}

__global__ void k_bitonic_global(int* __restrict__ key, int* __restrict__ perm, int half, int m, int dist)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= half) return;
    const int low = t & (dist - 1);
    const int i = ((t - low) << 1) | low;
    cmp_swap(key, perm, i, i | dist, ((i >> m) & 2) == 0);
}

// All stages (m, dist) with m in [m0, m1] and dist <= dmax (< tile) on one
// tile in shared memory.  For m == m0 only dist <= dmax run; later m run all
// their dist < tile (m1 <= log2(tile)-1 when m0 < log2(tile)).
__global__ void k_bitonic_tile(int* __restrict__ key, int* __restrict__ perm, int tile, int m0, int m1, int dmax)
{
    __shared__ int sk[kTile];
    __shared__ int sp[kTile];
    const int base = blockIdx.x * tile;
    for (int t = threadIdx.x; t < tile; t += blockDim.x) {
        sk[t] = key[base + t];
        sp[t] = perm[base + t];
    }
    __syncthreads();
    for (int m = m0; m <= m1; ++m) {
        const int dstart = (m == m0) ? dmax : (1 << m);
        for (int dist = dstart; dist >= 1; dist >>= 1) {
            for (int t = threadIdx.x; t < tile / 2; t += blockDim.x) {
                const int low = t & (dist - 1);
                const int li = ((t - low) << 1) | low;
                const int gi = base + li;
                cmp_swap(sk, sp, li, li | dist, ((gi >> m) & 2) == 0);
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < tile; t += blockDim.x) {
        key[base + t] = sk[t];
        perm[base + t] = sp[t];
    }
}

// ---- counting sort (option cell_sort 1) ------------------------------------
// The production cell sort: the keys are cell indices in [0, 2T), so one
// counting pass sorts them.  A warp-aggregated histogram (lanes with equal
// keys, found with __match_any_sync, add their count once), the bucket
// offsets from the device scan (warp-level inclusive scans within a block),
// a warp-aggregated scatter, and last each bucket ordered by the particles'
// previous positions, so the permutation does not depend on the order in
// which the scatter's atomics were served: a stable sort.  Unlike the
// reference's bitonic network (main.cpp:1190-1211, not stable) it gives a
// different order inside a cell; cell ranges and per-cell particle sets are
// the same.
__global__ void k_count_keys(int N, const int* __restrict__ key, int* __restrict__ cnt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = i < N;
    const int k = valid ? key[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    if (valid && lane == __ffs(peers) - 1) atomicAdd(cnt + k, __popc(peers));
}

__global__ void k_scatter_keys(int N, const int* __restrict__ key, const long long* __restrict__ off, int* __restrict__ cursor,
                               int* __restrict__ perm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = i < N;
    const int k = valid ? key[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (valid && lane == leader) base = atomicAdd(cursor + k, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (valid) perm[off[k] + base + __popc(peers & ((1u << lane) - 1u))] = i;
}

// thread per bucket: its particles ordered by previous position (insertion
// sort: a bucket is one cell's fluid or wall particles), the sorted keys and
// the bucket starts
__global__ void k_bucket_order(int nb, const long long* __restrict__ off, int* __restrict__ key, int* __restrict__ perm,
                               int* __restrict__ bucket)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const long long s = off[b], e = off[b + 1];
    for (long long j = s + 1; j < e; ++j) {
        const int v = perm[j];
        long long k = j - 1;
        while (k >= s && perm[k] > v) {
            perm[k + 1] = perm[k];
            --k;
        }
        perm[k + 1] = v;
    }
    for (long long j = s; j < e; ++j) key[j] = b;
    bucket[b] = (int)s;
    if (b == nb - 1) bucket[nb] = (int)e;
}

// ---- bucket starts, permutation -------------------------------------------
// bucket[b] = first sorted position whose key >= b, b in [0, 2T]
__global__ void k_bucket_starts(const int* __restrict__ key, int N, int T, int* __restrict__ bucket)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > N) return;
    const int lo = (i == 0) ? 0 : key[i - 1] + 1;
    const int hi = (i == N) ? 2 * T : key[i];
    for (int b = lo; b <= hi; ++b) bucket[b] = i;
}

template <int D>
__global__ void k_permute(int N, const int* __restrict__ perm, const int* __restrict__ id, const int* __restrict__ type,
                          const double* __restrict__ pos, const double* __restrict__ vel, int* __restrict__ id2,
                          int* __restrict__ type2, double* __restrict__ pos2, double* __restrict__ vel2,
                          float* __restrict__ pos32, float* __restrict__ poslo32, float4* __restrict__ pt2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int s = perm[i];
    id2[i] = id[s];
    type2[i] = type[s];
    double x[3], v[3];
    load_vec<D>(pos, s, x);
    load_vec<D>(vel, s, v);
    store_vec<D>(pos2, i, x);
    store_vec<D>(vel2, i, v);
    float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d) {
        h[d] = (float)x[d];
        l[d] = (float)(x[d] - (double)h[d]);   // exact difference, rounded once
    }
    if (D == 2) {
        reinterpret_cast<float2*>(pos32)[i] = make_float2(h[0], h[1]);
        reinterpret_cast<float2*>(poslo32)[i] = make_float2(l[0], l[1]);
        pt2[i] = make_float4(h[0], h[1], 0.f, __int_as_float(type[s]));
    } else {
        // w: the type bits (read with the position by the pair-term operator)
        reinterpret_cast<float4*>(pos32)[i] = make_float4(h[0], h[1], h[2], __int_as_float(type[s]));
        reinterpret_cast<float4*>(poslo32)[i] = make_float4(l[0], l[1], l[2], 0.f);
    }
}

// the previous step's start velocity follows the particles through the sort
template <int D>
__global__ void k_permute_vec(int N, const int* __restrict__ perm, const double* __restrict__ v, double* __restrict__ v2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double a[3];
    load_vec<D>(v, perm[i], a);
    store_vec<D>(v2, i, a);
}

__global__ void k_fluid_bbox(const int* __restrict__ bucket, DevParams P, int* __restrict__ bbox)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.T) return;
    if (bucket[c + 1] - bucket[c] > 0) {
        const int p[3] = {(c / (P.cc[1] * P.cc[2])) % P.cc[0], (c / P.cc[2]) % P.cc[1], c % P.cc[2]};
        for (int d = 0; d < 3; ++d) {
            atomicMin(&bbox[d], p[d]);
            atomicMax(&bbox[3 + d], p[d]);
        }
    }
}

// ---- launchers -------------------------------------------------------------
void launch_step_begin(mph_case* c)
{
    WallMotion W;
    for (int t = 0; t < 4; ++t)
        for (int a = 0; a < 3; ++a) {
            W.c[t][a] = c->wallC[t][a];
            W.v[t][a] = c->wallV[t][a];
            W.w[t][a] = c->wallW[t][a];
            for (int b = 0; b < 3; ++b) W.R[t][a][b] = c->wallR[t][a][b];
        }
    const unsigned g = grid_for(c->dp.N, 256);
    if (c->dim == 2)
        { k_step_begin<2><<<g, 256, 0, c->stream>>>(c->dp, W, c->d.pos, c->d.vel, c->d.force, c->fB, c->fE, c->wB, c->wE, c->d.type); MPH_COUNT_LAUNCH(); }
    else
        { k_step_begin<3><<<g, 256, 0, c->stream>>>(c->dp, W, c->d.pos, c->d.vel, c->d.force, c->fB, c->fE, c->wB, c->wE, c->d.type); MPH_COUNT_LAUNCH(); }
}

void launch_cell_keys(mph_case* c)
{
    const unsigned g = grid_for(c->dp.nPow, 256);
    if (c->dim == 2) { k_cell_keys<2><<<g, 256, 0, c->stream>>>(c->dp, c->d.pos, c->d.type, c->d.key, c->d.perm); MPH_COUNT_LAUNCH(); }
    else { k_cell_keys<3><<<g, 256, 0, c->stream>>>(c->dp, c->d.pos, c->d.type, c->d.key, c->d.perm); MPH_COUNT_LAUNCH(); }
}

void launch_bitonic_sort(mph_case* c)
{
    const int n = c->dp.nPow, k = c->dp.powExp;
    if (k == 0) return;
    const int tile = n < kTile ? n : kTile;
    int tileExp = 0;
    while ((1 << tileExp) < tile) ++tileExp;
    const int ntiles = n / tile;
    // every stage of m < tileExp stays inside a tile
    { k_bitonic_tile<<<ntiles, kTileThreads, 0, c->stream>>>(c->d.key, c->d.perm, tile, 0, (k < tileExp ? k : tileExp) - 1, 1); MPH_COUNT_LAUNCH(); }
    for (int m = tileExp; m < k; ++m) {
        for (int s = 0; s <= m; ++s) {
            const int dist = 1 << (m - s);
            if (dist < tile) {
                { k_bitonic_tile<<<ntiles, kTileThreads, 0, c->stream>>>(c->d.key, c->d.perm, tile, m, m, dist); MPH_COUNT_LAUNCH(); }
                break;
            }
            { k_bitonic_global<<<grid_for(n / 2, 256), 256, 0, c->stream>>>(c->d.key, c->d.perm, n / 2, m, dist); MPH_COUNT_LAUNCH(); }
        }
    }
}

int launch_counting_sort(mph_case* c)
{
    const int N = c->dp.N, nb = 2 * c->dp.T;
    DeviceState& d = c->d;
    if (!d.sort_cnt) {
        MPH_CUDA(cudaMalloc((void**)&d.sort_cnt, (size_t)(nb + 1) * sizeof(int)));
        MPH_CUDA(cudaMalloc((void**)&d.sort_off, (size_t)(nb + 1) * sizeof(long long)));
    }
    const unsigned g = grid_for(N, 256);
    MPH_CUDA(cudaMemsetAsync(d.sort_cnt, 0, (size_t)(nb + 1) * sizeof(int), c->stream));
    { k_count_keys<<<g, 256, 0, c->stream>>>(N, d.key, d.sort_cnt); MPH_COUNT_LAUNCH(); }
    MPH_TRY(launch_scan_i32_to_i64(c, d.sort_cnt, d.sort_off, nb));
    MPH_CUDA(cudaMemsetAsync(d.sort_cnt, 0, (size_t)(nb + 1) * sizeof(int), c->stream));
    { k_scatter_keys<<<g, 256, 0, c->stream>>>(N, d.key, d.sort_off, d.sort_cnt, d.perm); MPH_COUNT_LAUNCH(); }
    { k_bucket_order<<<grid_for(nb, 128), 128, 0, c->stream>>>(nb, d.sort_off, d.key, d.perm, d.bucket); MPH_COUNT_LAUNCH(); }
    return MPH_OK;
}

void launch_cell_ranges_and_permute(mph_case* c)
{
    const int N = c->dp.N;
    if (!c->cell_sort)   // the counting sort wrote the bucket starts already
        { k_bucket_starts<<<grid_for(N + 1, 256), 256, 0, c->stream>>>(c->d.key, N, c->dp.T, c->d.bucket); MPH_COUNT_LAUNCH(); }
    const unsigned g = grid_for(N, 256);
    if (c->dim == 2)
        { k_permute<2><<<g, 256, 0, c->stream>>>(N, c->d.perm, c->d.id, c->d.type, c->d.pos, c->d.vel, c->d.id_alt,
                                                c->d.type_alt, c->d.pos_alt, c->d.vel_alt, c->d.pos32,
                                                c->d.poslo32, c->d.pt32); MPH_COUNT_LAUNCH(); }
    else
        { k_permute<3><<<g, 256, 0, c->stream>>>(N, c->d.perm, c->d.id, c->d.type, c->d.pos, c->d.vel, c->d.id_alt,
                                                c->d.type_alt, c->d.pos_alt, c->d.vel_alt, c->d.pos32,
                                                c->d.poslo32, nullptr); MPH_COUNT_LAUNCH(); }
    std::swap(c->d.id, c->d.id_alt);
    std::swap(c->d.type, c->d.type_alt);
    std::swap(c->d.pos, c->d.pos_alt);
    std::swap(c->d.vel, c->d.vel_alt);
    if (c->prev_valid && c->d.vprev) {
        const size_t nvs = (size_t)N * vs_of(c->dim);
        for (int h = 0; h < c->prev_valid; ++h) {
            if (c->dim == 2) { k_permute_vec<2><<<g, 256, 0, c->stream>>>(N, c->d.perm, c->d.vprev + h * nvs, c->d.vprev_alt + h * nvs); MPH_COUNT_LAUNCH(); }
            else { k_permute_vec<3><<<g, 256, 0, c->stream>>>(N, c->d.perm, c->d.vprev + h * nvs, c->d.vprev_alt + h * nvs); MPH_COUNT_LAUNCH(); }
        }
        std::swap(c->d.vprev, c->d.vprev_alt);
    }
}

void launch_fluid_bbox(mph_case* c)
{
    { k_fluid_bbox<<<grid_for(c->dp.T, 256), 256, 0, c->stream>>>(c->d.bucket, c->dp, c->d.bbox); MPH_COUNT_LAUNCH(); }
}

}  // namespace mph
