// k_multigrid.cu - cell-aggregation multigrid (main.cpp:2647-3546, 4122-4266).
//
// Level L is the fluid-cell bounding box of the neighbour grid coarsened L
// times by 2 (calculateMultiGridDepth, main.cpp:2777-2859).  Restriction (sum
// of the 2^D children), prolongation (injection) and the particle<->grid
// transfers (P2G sum, G2P injection) are index maps computed on the fly; only
// the level matrices are stored, as 3^D-cell block stencils with the
// reference's periodic wrap on the grid index.  A level's stencil is stored
// entry-major: value (entry e, row) at e*rows + row, so the threads of a
// warp (consecutive rows) read consecutive words.
//
// Build:  level 0 = per-cell sums of the per-row partial stencils written by
//         the assembly pass; level L = the reference's re-binning of level
//         L-1's stencil rows onto the parent cells (same summation order);
//         invD = 2 / sum |a_row| (calculateMultiGridInvDiagA, main.cpp:3510).
// V-cycle: levels with many rows run as grid-wide kernels: one fused Jacobi
//         kernel per smoothing sweep (S_new = S + invD (Q - A S)), a residual
//         kernel before each restriction, and the restriction (child sums).
//         Every level from the first one with at most kCtaRows rows down to
//         the coarsest and back runs inside one cluster of kClusterCtas
//         1024-thread blocks (one per SM), its sweeps separated by cluster
//         barriers, so the small levels cost one launch and read their
//         stencils through the L2 ports of eight SMs.
//         The last kernel adds G2P S_0 to D^-1 q and forms the (q, u) dot.
//         The mixed form's FP32 sweeps on grid-wide levels run three threads
//         a row (k_mg_sweep3), one stencil plane each.
#include <cooperative_groups.h>
#include <mutex>
#include <type_traits>

#include "mph_device.cuh"

#include "mph_solver.cuh"

namespace cg = cooperative_groups;

namespace mph {

#ifndef MPH_CTA_ROWS
#define MPH_CTA_ROWS 8192
#endif
#ifndef MPH_CLUSTER_CTAS
#define MPH_CLUSTER_CTAS 8
#endif
constexpr int kCtaRows = MPH_CTA_ROWS;
constexpr int kCtaThreads = 1024;
constexpr int kClusterCtas = MPH_CLUSTER_CTAS;   // above 8: a non-portable cluster size
constexpr int kDenseRows = 224;   // dense coarse level of the mixed form: n x n floats in one block's shared memory

struct LevelK {
    int mn[3], mx[3], cnt[3], st[3];
    int rows, width;   // width = D * st0*st1*st2
};

static LevelK level_k(const mph_case* c, int L)
{
    const LevelGeom& g = c->lv[L];
    LevelK k{};
    for (int d = 0; d < 3; ++d) {
        k.mn[d] = g.mn[d]; k.mx[d] = g.mx[d]; k.cnt[d] = g.cnt[d]; k.st[d] = g.st[d];
    }
    k.rows = g.rows;
    k.width = c->dim * g.st[0] * g.st[1] * g.st[2];
    return k;
}

__device__ __forceinline__ void grid_coords(const LevelK& L, int g, int* p)
{
    p[0] = (g / (L.cnt[1] * L.cnt[2])) % L.cnt[0];
    p[1] = (g / L.cnt[2]) % L.cnt[1];
    p[2] = g % L.cnt[2];
}
__device__ __forceinline__ int grid_index(const LevelK& L, int x, int y, int z)
{
    return (L.cnt[1] * L.cnt[2]) * x + L.cnt[2] * y + z;
}
// column grid cell of stencil slot (ix,iy,iz) of cell p (periodic on the grid)
__device__ __forceinline__ int stencil_col(const LevelK& L, const int* p, int ix, int iy, int iz)
{
    return grid_index(L, (p[0] + ix - 1 + L.cnt[0]) % L.cnt[0], (p[1] + iy - 1 + L.cnt[1]) % L.cnt[1],
                      (p[2] + iz - 1 + L.cnt[2]) % L.cnt[2]);
}
// children range of coarse cell p of level L inside the finer level S_
__device__ __forceinline__ void child_range(const LevelK& S_, const LevelK& L, const int* p, int* fm, int* fM)
{
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int lc = p[d] + L.mn[d];
        fm[d] = S_.mn[d] > 2 * lc ? 1 : 0;
        fM[d] = S_.mx[d] < 2 * (lc + 1) ? 1 : 0;
    }
}

// ---- build -------------------------------------------------------------------
template <int D>
__global__ void k_mg_level0(DevParams P, LevelK L, const int* __restrict__ bucket, const double* __restrict__ part,
                            double* __restrict__ cofT, const int* __restrict__ only_cells)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)L.rows * L.width) return;
    const int e = (int)(t / L.rows), row = (int)(t % L.rows);
    const int g = row / D, rD = row % D;
    const int slot = e / D, sD = e % D;
    const int S = L.st[0] * L.st[1] * L.st[2];
    int p[3];
    grid_coords(L, g, p);
    const int cx = p[0] + L.mn[0], cy = p[1] + L.mn[1], cz = p[2] + L.mn[2];
    double sum = 0.0;
    if (cx < P.cc[0] && cy < P.cc[1] && cz < P.cc[2]) {
        const int ic = cell_id(P, cx, cy, cz);
        if (only_cells && !only_cells[ic]) return;   // written by the assembly
        for (int i = bucket[ic]; i < bucket[ic + 1]; ++i) sum += part[((size_t)i * S + slot) * D * D + rD * D + sD];
    } else if (only_cells) {
        return;
    }
    cofT[t] = sum;
}

template <int D>
__global__ void k_mg_coarse(LevelK S_, LevelK L, const double* __restrict__ cofS, double* __restrict__ cofL)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)L.rows * L.width) return;
    const int e = (int)(t / L.rows), rowL = (int)(t % L.rows);
    const int g = rowL / D, rD = rowL % D;
    const int oslot = e / D, sD = e % D;
    int p[3], fm[3], fM[3];
    grid_coords(L, g, p);
    child_range(S_, L, p, fm, fM);
    double sum = 0.0;
    for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
        for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
            for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                const int sg = grid_index(S_, 2 * (p[0] + L.mn[0]) + dx - S_.mn[0], 2 * (p[1] + L.mn[1]) + dy - S_.mn[1],
                                          2 * (p[2] + L.mn[2]) + dz - S_.mn[2]);
                const int rowS = sg * D + rD;
                int sp[3];
                grid_coords(S_, sg, sp);
                int fe = 0;
                for (int ix = 0; ix < S_.st[0]; ++ix)
                    for (int iy = 0; iy < S_.st[1]; ++iy)
                        for (int iz = 0; iz < S_.st[2]; ++iz, ++fe) {
                            const int jf[3] = {(sp[0] + ix - 1 + S_.cnt[0]) % S_.cnt[0], (sp[1] + iy - 1 + S_.cnt[1]) % S_.cnt[1],
                                               (sp[2] + iz - 1 + S_.cnt[2]) % S_.cnt[2]};
                            int o[3];
#pragma unroll
                            for (int d = 0; d < 3; ++d) {
                                const int jl = (jf[d] + S_.mn[d]) / 2 - L.mn[d];
                                o[d] = (jl - p[d] + 1 + L.cnt[d]) % L.cnt[d];
                            }
                            if (L.st[2] * L.st[1] * o[0] + L.st[2] * o[1] + o[2] != oslot) continue;
                            sum += cofS[(size_t)(fe * D + sD) * S_.rows + rowS];
                        }
            }
    cofL[t] = sum;
}

__global__ void k_mg_invd(int rows, int width, const double* __restrict__ cofT, double* __restrict__ invd)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    double s = 0.0;
    for (int k = 0; k < width; ++k) s += fabs(cofT[(size_t)k * rows + row]);
    invd[row] = s != 0.0 ? 2.0 / s : 0.0;
}

// only_cells (cell flags by key, or null for every cell): the level-0 rows of
// those cells only, the others having been written by the assembly
void launch_mg_level0(mph_case* c, const int* only_cells)
{
    const LevelK L = level_k(c, 0);
    const long long n = (long long)L.rows * L.width;
    double* cof = c->d.mg_cof + c->lv[0].off_cof;
    if (c->dim == 2) { k_mg_level0<2><<<grid_for(n, 256), 256, 0, c->stream>>>(c->dp, L, c->d.bucket, c->d.part, cof, only_cells); MPH_COUNT_LAUNCH(); }
    else { k_mg_level0<3><<<grid_for(n, 256), 256, 0, c->stream>>>(c->dp, L, c->d.bucket, c->d.part, cof, only_cells); MPH_COUNT_LAUNCH(); }
}

void launch_mg_coarse(mph_case* c, int lvl)
{
    const LevelK S_ = level_k(c, lvl - 1), L = level_k(c, lvl);
    const long long n = (long long)L.rows * L.width;
    const double* cofS = c->d.mg_cof + c->lv[lvl - 1].off_cof;
    double* cofL = c->d.mg_cof + c->lv[lvl].off_cof;
    if (c->dim == 2) { k_mg_coarse<2><<<grid_for(n, 256), 256, 0, c->stream>>>(S_, L, cofS, cofL); MPH_COUNT_LAUNCH(); }
    else { k_mg_coarse<3><<<grid_for(n, 256), 256, 0, c->stream>>>(S_, L, cofS, cofL); MPH_COUNT_LAUNCH(); }
}

void launch_mg_invd(mph_case* c)
{
    for (int l = 0; l < c->depth; ++l) {
        const LevelK L = level_k(c, l);
        { k_mg_invd<<<grid_for(L.rows, 256), 256, 0, c->stream>>>(L.rows, L.width, c->d.mg_cof + c->lv[l].off_cof,
                                                               c->d.mg_invd + c->lv[l].off_vec); MPH_COUNT_LAUNCH(); }
    }
}

// ---- V-cycle row operations ------------------------------------------------------
// Q - A S for one row (the reference's csrmv with alpha = -1, beta = 1).
// UNROLL (the cluster kernel of the small levels, where a few SMs run each
// sweep and every row's loads wait in line): with the full 3^D stencil the
// loops are unrolled below the outer axis, so a row's coefficient and S loads
// are issued a stencil plane at a time instead of one latency per stencil
// cell (fully unrolled, the kernel spills), and the wrapped column
// coordinates are formed once per axis; the summation order is the same.
// The grid-wide levels keep the plain loop (measured faster there).
template <int D, typename T, bool UNROLL = false>
__device__ __forceinline__ T row_residual(const LevelK& L, const T* __restrict__ cofT, const T* __restrict__ Q,
                                          const T* __restrict__ S, int row)
{
    const int g = row / D;
    int p[3];
    grid_coords(L, g, p);
    T sum = 0;
    constexpr int SZ = D == 3 ? 3 : 1;
    if (UNROLL && L.st[0] == 3 && L.st[1] == 3 && L.st[2] == SZ) {
        int ys[3], zs[SZ];
#pragma unroll
        for (int k = 0; k < 3; ++k) ys[k] = ((p[1] + k - 1 + L.cnt[1]) % L.cnt[1]) * L.cnt[2];
#pragma unroll
        for (int k = 0; k < SZ; ++k) zs[k] = (p[2] + k - 1 + L.cnt[2]) % L.cnt[2];
#pragma unroll 1
        for (int ix = 0; ix < 3; ++ix) {
            const int xw = ((p[0] + ix - 1 + L.cnt[0]) % L.cnt[0]) * (L.cnt[1] * L.cnt[2]);
            const T* cx = cofT + (size_t)ix * (3 * SZ * D) * L.rows + row;
#pragma unroll
            for (int iy = 0; iy < 3; ++iy)
#pragma unroll
                for (int iz = 0; iz < SZ; ++iz) {
                    const int jg = xw + ys[iy] + zs[iz];
#pragma unroll
                    for (int sD = 0; sD < D; ++sD)
                        sum += (-cx[(size_t)((iy * SZ + iz) * D + sD) * L.rows]) * S[jg * D + sD];
                }
        }
        return Q[row] + sum;
    }
    int e = 0;
    for (int ix = 0; ix < L.st[0]; ++ix)
        for (int iy = 0; iy < L.st[1]; ++iy)
            for (int iz = 0; iz < L.st[2]; ++iz) {
                const int jg = stencil_col(L, p, ix, iy, iz);
#pragma unroll
                for (int sD = 0; sD < D; ++sD, ++e) sum += (-cofT[(size_t)e * L.rows + row]) * S[jg * D + sD];
            }
    return Q[row] + sum;
}

// sum of the children's residuals (the restriction R, main.cpp:3154-3174)
template <int D, typename T>
__device__ __forceinline__ T row_restrict(const LevelK& S_, const LevelK& L, const T* __restrict__ RS, int row)
{
    const int g = row / D, rD = row % D;
    int p[3], fm[3], fM[3];
    grid_coords(L, g, p);
    child_range(S_, L, p, fm, fM);
    T sum = 0;
    for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
        for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
            for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                const int sg = grid_index(S_, 2 * (p[0] + L.mn[0]) + dx - S_.mn[0], 2 * (p[1] + L.mn[1]) + dy - S_.mn[1],
                                          2 * (p[2] + L.mn[2]) + dz - S_.mn[2]);
                sum += RS[sg * D + rD];
            }
    return sum;
}

// parent row of fine row `row` (the prolongation P, main.cpp:3216-3240)
template <int D>
__device__ __forceinline__ int row_parent(const LevelK& S_, const LevelK& L, int row)
{
    const int g = row / D, rD = row % D;
    int p[3];
    grid_coords(S_, g, p);
    return grid_index(L, (p[0] + S_.mn[0]) / 2 - L.mn[0], (p[1] + S_.mn[1]) / 2 - L.mn[1], (p[2] + S_.mn[2]) / 2 - L.mn[2]) * D + rD;
}

// ---- grid-wide V-cycle kernels ------------------------------------------------------
template <int D, typename T>
__global__ void k_mg_jacobi(LevelK L, const T* __restrict__ cofT, const T* __restrict__ invd, const T* __restrict__ Q,
                            const T* __restrict__ Sin, T* __restrict__ Sout, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    const T r = row_residual<D, T>(L, cofT, Q, Sin, row);
    Sout[row] = Sin[row] + invd[row] * r;
}

template <int D, typename T>
__global__ void k_mg_residual(LevelK L, const T* __restrict__ cofT, const T* __restrict__ Q, const T* __restrict__ S,
                              T* __restrict__ R, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    R[row] = row_residual<D, T>(L, cofT, Q, S, row);
}

// FP32 sweeps of the mixed form's V-cycle on levels with the full 3^D
// stencil: three threads per row, one stencil plane (fixed first coordinate)
// each, summed in plane order (10 rows a warp, lanes 30 and 31 idle).  A
// row's stencil is then three short load chains instead of one of 3^D
// cells, with three times the threads in flight.  RESID: R = Q - A S; else
// S_out = S + invD (Q - A S).  Warp gw of nw walks the rows 10 at a time.
template <int D>
__device__ __forceinline__ float plane_part(const LevelK& L, const float* __restrict__ cofT, const float* __restrict__ Sin, int row,
                                            int ix)
{
    constexpr int SZ = D == 3 ? 3 : 1;
    int p[3];
    grid_coords(L, row / D, p);
    const int xw = ((p[0] + ix - 1 + L.cnt[0]) % L.cnt[0]) * (L.cnt[1] * L.cnt[2]);
    int ys[3], zs[SZ];
#pragma unroll
    for (int k = 0; k < 3; ++k) ys[k] = ((p[1] + k - 1 + L.cnt[1]) % L.cnt[1]) * L.cnt[2];
#pragma unroll
    for (int k = 0; k < SZ; ++k) zs[k] = (p[2] + k - 1 + L.cnt[2]) % L.cnt[2];
    const float* cx = cofT + (size_t)ix * (3 * SZ * D) * L.rows + row;
    float part = 0.f;
#pragma unroll
    for (int iy = 0; iy < 3; ++iy)
#pragma unroll
        for (int iz = 0; iz < SZ; ++iz) {
            const int jg = xw + ys[iy] + zs[iz];
#pragma unroll
            for (int sD = 0; sD < D; ++sD) part += (-cx[(size_t)((iy * SZ + iz) * D + sD) * L.rows]) * Sin[jg * D + sD];
        }
    return part;
}

template <int D, bool RESID>
__device__ __forceinline__ void sweep3_rows(const LevelK& L, const float* __restrict__ cofT, const float* __restrict__ invd,
                                            const float* __restrict__ Q, const float* __restrict__ Sin, float* __restrict__ out,
                                            int gw, int nw)
{
    const int lane = threadIdx.x & 31;
    const int rw = lane / 3, ix = lane - 3 * rw;
    const int b = min(3 * rw, 29);
    for (int base = gw * 10; base < L.rows; base += nw * 10) {
        const int row = base + rw;
        const bool valid = lane < 30 && row < L.rows;
        const float part = valid ? plane_part<D>(L, cofT, Sin, row, ix) : 0.f;
        const float p0 = __shfl_sync(0xffffffffu, part, b);
        const float p1 = __shfl_sync(0xffffffffu, part, b + 1);
        const float p2 = __shfl_sync(0xffffffffu, part, b + 2);
        if (valid && ix == 0) {
            const float r = Q[row] + ((p0 + p1) + p2);
            if (RESID) out[row] = r;
            else out[row] = Sin[row] + invd[row] * r;
        }
    }
}

__host__ __device__ inline bool full_stencil(const LevelK& L, int D)
{
    return L.st[0] == 3 && L.st[1] == 3 && L.st[2] == (D == 3 ? 3 : 1);
}

// one warp of 10 rows per launch slot (the grid covers the level once)
template <int D, bool RESID>
__global__ void k_mg_sweep3(LevelK L, const float* __restrict__ cofT, const float* __restrict__ invd, const float* __restrict__ Q,
                            const float* __restrict__ Sin, float* __restrict__ out, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int rw = lane / 3, ix = lane - 3 * rw;
    const int row = warp * 10 + rw;
    const bool valid = lane < 30 && row < L.rows;
    float part = 0.f;
    if (valid) part = plane_part<D>(L, cofT, Sin, row, ix);
    const int b = min(3 * rw, 29);
    const float p0 = __shfl_sync(0xffffffffu, part, b);
    const float p1 = __shfl_sync(0xffffffffu, part, b + 1);
    const float p2 = __shfl_sync(0xffffffffu, part, b + 2);
    if (valid && ix == 0) {
        const float r = Q[row] + ((p0 + p1) + p2);
        if (RESID) out[row] = r;
        else out[row] = Sin[row] + invd[row] * r;
    }
}

// Q_L = R r_{L-1};  S_L = invD_L Q_L (the first smoothing update from S = 0)
template <int D, typename T>
__global__ void k_mg_restrict(LevelK S_, LevelK L, const T* __restrict__ RS, const T* __restrict__ invdL, T* __restrict__ QL,
                              T* __restrict__ SL, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    const T q = row_restrict<D, T>(S_, L, RS, row);
    QL[row] = q;
    SL[row] = invdL[row] * q;
}

template <int D, typename T>
__global__ void k_mg_prolong(LevelK S_, LevelK L, const T* __restrict__ SL, T* __restrict__ SS, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= S_.rows) return;
    SS[row] = SS[row] + SL[row_parent<D>(S_, L, row)];
}

// Q_0 = P2G q (sum over the fluid particles of each cell); S_0 = invD_0 Q_0
template <int D, typename T, typename TQ>
__global__ void k_mg_p2g(DevParams P, LevelK L, const int* __restrict__ bucket, const TQ* __restrict__ q,
                         const T* __restrict__ invd, T* __restrict__ Q, T* __restrict__ S, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    const int g = row / D, rD = row % D;
    int p[3];
    grid_coords(L, g, p);
    const int ic = cell_id(P, p[0] + L.mn[0], p[1] + L.mn[1], p[2] + L.mn[2]);
    T sum = 0;
    for (int i = bucket[ic]; i < bucket[ic + 1]; ++i) sum += (T)q[(size_t)i * D + rD];
    Q[row] = sum;
    S[row] = invd[row] * sum;
}

// u = D^-1 q + G2P S_0, with the (q, u) dot product
template <int D, typename T, typename TQ>
__global__ void k_mg_g2p_dot(DevParams P, LevelK L, const int* __restrict__ key, const TQ* __restrict__ invDiag,
                             const TQ* __restrict__ q, const T* __restrict__ S0, TQ* __restrict__ u,
                             double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out,
                             const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    double acc = 0.0;
    // a thread per particle: its level-0 cell is decoded from the key once
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.Nf; i += gridDim.x * blockDim.x) {
        int cc3[3];
        key_coords(P, key[i], cc3);
        const int g = grid_index(L, cc3[0] - L.mn[0], cc3[1] - L.mn[1], cc3[2] - L.mn[2]);
#pragma unroll
        for (int rD = 0; rD < D; ++rD) {
            const size_t k = (size_t)i * D + rD;
            const TQ qk = q[k];
            const TQ v = invDiag[k] * qk + (TQ)S0[g * D + rD];
            u[k] = v;
            acc += (double)qk * (double)v;
        }
    }
    reduce_finalize(acc, partials, counter, out);
}

// u = D^-1 q with the (q, u) dot: the preconditioner without grid levels
// (mixed form, option mg_depth -1)
template <typename TQ>
__global__ void k_jacobi_dot(long long n, const TQ* __restrict__ invDiag, const TQ* __restrict__ q, TQ* __restrict__ u,
                             double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out,
                             const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    double acc = 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const TQ qk = q[k];
        const TQ v = invDiag[k] * qk;
        u[k] = v;
        acc += (double)qk * (double)v;
    }
    reduce_finalize(acc, partials, counter, out);
}

// ---- the small levels in one block ------------------------------------------------
template <typename T>
struct CoarseArgs {
    int first, depth;                 // levels first..depth-1 run here; first >= 1
    LevelK L[kMaxLevels];
    const T* cof[kMaxLevels];
    const T* invd[kMaxLevels];
    T* Q[kMaxLevels];
    T* Sa[kMaxLevels];
    T* Sb[kMaxLevels];
    T* R[kMaxLevels];                 // R[first-1] holds the finer level's residual
    T* Sfine;                         // current S of level first-1 (receives the prolongation)
    int pre, post;                    // smoothing sweeps of the levels below level 0 (the reference: 2 and 3)
    int dense;                        // >= 0: this level (one block's size) is solved exactly with dinv
    const T* dinv;                    // its dense inverse, n x n (symmetric)
};

// Dense inverse of one coarse level's matrix (mixed form, FP32), one block:
// the level's stencil rows into an n x n matrix in shared memory (a thread a
// row, its entries in stencil order, so the duplicated columns of a wrapped
// axis add up in a fixed order), then Gauss-Jordan elimination in place
// without pivoting, which is stable for the symmetric positive definite
// Galerkin level matrices.  n <= kDenseRows.
template <int D>
__global__ void __launch_bounds__(1024) k_mg_dense_inv(LevelK L, const float* __restrict__ cofT, float* __restrict__ inv)
{
    extern __shared__ float dn_smem[];
    const int n = L.rows;
    float* a = dn_smem;          // n x n, row-major
    float* colk = dn_smem + n * n;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) a[t] = 0.f;
    __syncthreads();
    for (int row = threadIdx.x; row < n; row += blockDim.x) {
        int p[3];
        grid_coords(L, row / D, p);
        int e = 0;
        for (int ix = 0; ix < L.st[0]; ++ix)
            for (int iy = 0; iy < L.st[1]; ++iy)
                for (int iz = 0; iz < L.st[2]; ++iz) {
                    const int jg = stencil_col(L, p, ix, iy, iz);
                    for (int sD = 0; sD < D; ++sD, ++e) a[(size_t)row * n + jg * D + sD] += cofT[(size_t)e * n + row];
                }
    }
    __syncthreads();
    // elimination: warp w takes rows w, w + 32, ..., lane l columns l, l + 32, ...
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int k = 0; k < n; ++k) {
        // a cell without fluid particles has a zero row and column: it stays
        // zero in the inverse (the pseudo-inverse on the occupied cells)
        const float akk = a[(size_t)k * n + k];
        const float pk = akk != 0.f ? 1.f / akk : 0.f;
        for (int i = threadIdx.x; i < n; i += blockDim.x) colk[i] = i == k ? 0.f : a[(size_t)i * n + k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) a[(size_t)k * n + j] = (j == k ? 1.f : a[(size_t)k * n + j]) * pk;
        __syncthreads();
        const float* ak = a + (size_t)k * n;
        for (int i = wid; i < n; i += nw) {
            if (i == k) continue;
            const float ci = colk[i];
            float* ai = a + (size_t)i * n;
            for (int j = lane; j < n; j += 32) ai[j] = (j == k ? 0.f : ai[j]) - ci * ak[j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) inv[t] = a[t];
}

template <int D, typename T>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kCtaThreads)
k_mg_small_levels(CoarseArgs<T> A, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;   // the same for every block of the cluster
    cg::cluster_group cluster = cg::this_cluster();
    const int tid = (int)cluster.block_rank() * blockDim.x + threadIdx.x;
    const int nth = (int)(blockDim.x * cluster.num_blocks());
    T* cur[kMaxLevels];
    T* oth[kMaxLevels];
    for (int l = A.first; l < A.depth; ++l) { cur[l] = A.Sa[l]; oth[l] = A.Sb[l]; }
    // levels from `narrow` on have at most one row per thread of a block:
    // block 0 runs them alone, with block barriers instead of cluster ones
    int narrow = A.depth;
    for (int l = A.first; l < A.depth; ++l)
        if (A.L[l].rows <= (int)blockDim.x) { narrow = l; break; }
    auto csync = [&]() { cluster.sync(); };
    auto bsync = [&]() { __syncthreads(); };
    // one smoothing sweep of level l over rows t0, t0 + nt, ...
    auto jacobi = [&](int l, int t0, int nt, auto sync) {
        const LevelK& L = A.L[l];
        if constexpr (std::is_same<T, float>::value) {
            if (full_stencil(L, D)) {   // three threads a row (t0, nt: multiples of 32)
                sweep3_rows<D, false>(L, A.cof[l], A.invd[l], A.Q[l], cur[l], oth[l], t0 >> 5, nt >> 5);
                sync();
                T* t = cur[l]; cur[l] = oth[l]; oth[l] = t;
                return;
            }
        }
        for (int row = t0; row < L.rows; row += nt) {
            const T r = row_residual<D, T, true>(L, A.cof[l], A.Q[l], cur[l], row);
            oth[l][row] = cur[l][row] + A.invd[l][row] * r;
        }
        sync();
        T* t = cur[l]; cur[l] = oth[l]; oth[l] = t;
    };
    // restriction into level l, pre-smoothing (3 updates, the coarsest 5), residual
    auto down = [&](int l, int t0, int nt, auto sync) {
        const LevelK& L = A.L[l];
        for (int row = t0; row < L.rows; row += nt) {
            const T q = row_restrict<D, T>(A.L[l - 1], L, A.R[l - 1], row);
            A.Q[l][row] = q;
            cur[l][row] = A.invd[l][row] * q;
        }
        sync();
        const int sweeps = (l == A.depth - 1) ? 4 : A.pre;
        for (int k = 0; k < sweeps; ++k) jacobi(l, t0, nt, sync);
        if (l < A.depth - 1) {
            bool done3 = false;
            if constexpr (std::is_same<T, float>::value) {
                if (full_stencil(L, D)) {
                    sweep3_rows<D, true>(L, A.cof[l], nullptr, A.Q[l], cur[l], A.R[l], t0 >> 5, nt >> 5);
                    done3 = true;
                }
            }
            if (!done3)
                for (int row = t0; row < L.rows; row += nt) A.R[l][row] = row_residual<D, T, true>(L, A.cof[l], A.Q[l], cur[l], row);
            sync();
        }
    };
    // prolongation of level l into level l-1 (S_{l-1} += P S_l)
    auto prolong = [&](int l, int t0, int nt) {
        const LevelK& S_ = A.L[l - 1];
        for (int row = t0; row < S_.rows; row += nt) cur[l - 1][row] = cur[l - 1][row] + cur[l][row_parent<D>(S_, A.L[l], row)];
    };
    // restriction into the dense level and its exact solve S = A^-1 Q (the
    // inverse is symmetric: column `row` read across the threads)
    auto dense_solve = [&](int l, int t0, int nt, auto sync) {
        const LevelK& L = A.L[l];
        for (int row = t0; row < L.rows; row += nt) A.Q[l][row] = row_restrict<D, T>(A.L[l - 1], L, A.R[l - 1], row);
        sync();
        for (int row = t0; row < L.rows; row += nt) {
            T v = 0;
            for (int c = 0; c < L.rows; ++c) v += A.dinv[(size_t)c * L.rows + row] * A.Q[l][c];
            cur[l][row] = v;
        }
        sync();
    };
    for (int l = A.first; l < narrow; ++l) down(l, tid, nth, csync);
    if (cluster.block_rank() == 0 && narrow < A.depth) {
        const int t0 = threadIdx.x, nt = blockDim.x;
        // levels narrow .. bottom-1 smoothed; the dense level (if any) solved exactly
        const int bottom = A.dense >= 0 ? A.dense : A.depth;
        for (int l = narrow; l < bottom; ++l) down(l, t0, nt, bsync);
        if (A.dense >= 0) dense_solve(A.dense, t0, nt, bsync);
        for (int l = bottom < A.depth ? bottom : A.depth - 1; l > narrow; --l) {
            prolong(l, t0, nt);
            bsync();
            for (int k = 0; k < A.post; ++k) jacobi(l - 1, t0, nt, bsync);   // post-smoothing (3 updates in the reference)
        }
        if (narrow > A.first) {
            prolong(narrow, t0, nt);
        } else {   // every small level is narrow: block 0 also prolongates into the finer level
            const LevelK& S_ = A.L[A.first - 1];
            for (int row = t0; row < S_.rows; row += nt)
                A.Sfine[row] = A.Sfine[row] + cur[A.first][row_parent<D>(S_, A.L[A.first], row)];
        }
    }
    if (narrow == A.first) return;   // done by block 0 (whose pointer swaps the others do not know)
    csync();
    for (int l = min(narrow, A.depth - 1); l > A.first; --l) {
        if (l < narrow) {
            prolong(l, tid, nth);
            csync();
        }
        for (int k = 0; k < A.post; ++k) jacobi(l - 1, tid, nth, csync);
    }
    // prolongation into the finer, grid-wide level
    const LevelK& S_ = A.L[A.first - 1];
    for (int row = tid; row < S_.rows; row += nth)
        A.Sfine[row] = A.Sfine[row] + cur[A.first][row_parent<D>(S_, A.L[A.first], row)];
}

// ---- host-side V-cycle -----------------------------------------------------------
template <int D, typename T, typename TQ>
static void vcycle_t(mph_case* c, const TQ* q, TQ* u, const TQ* invDiag, const T* cof, const T* invd, T* Qp, T* Sa, T* Sb,
                     T* Rp, double* dot_out, int extra0 = 0)
{
    // sweeps of the levels below level 0: the reference's 2 and 3, or the
    // mixed form's options mg_pre / mg_post; the mixed form's option mg_depth
    // (>= 2) cuts the cycle after that many levels (the last one coarsest)
    const bool mixed = std::is_same<T, float>::value;
    if (mixed && c->mg_depth < 0) {   // no grid levels: point Jacobi on the particles
        const long long n = (long long)c->dp.Nf * D;
        const int blocks = std::min<int>(grid_for(n, 256), kReduceBlocks);
        { k_jacobi_dot<TQ><<<blocks, 256, 0, c->stream>>>(n, invDiag, q, u, c->d.partials, (unsigned*)(c->d.flags + kFlagCounter),
                                                         dot_out, c->d.flags); MPH_COUNT_LAUNCH(); }
        return;
    }
    const int depth = mixed && c->mg_depth >= 1 ? std::min(c->depth, c->mg_depth) : c->depth;
    const int coarsest = mixed ? c->mg_coarsest : 4;   // sweeps of the coarsest grid-wide level
    cudaStream_t st = c->stream;
    const int* flags = c->d.flags;
    const int pre = mixed ? c->mg_pre : 2, post = mixed ? c->mg_post : 3;
    LevelK L[kMaxLevels];
    for (int l = 0; l < depth; ++l) L[l] = level_k(c, l);
    auto ov = [&](int l) { return c->lv[l].off_vec; };
    auto oc = [&](int l) { return c->lv[l].off_cof; };
    T* cur[kMaxLevels];
    T* oth[kMaxLevels];
    for (int l = 0; l < depth; ++l) { cur[l] = Sa + ov(l); oth[l] = Sb + ov(l); }
    // first level handled by the single-block kernel (>= 1), or depth if none
    int first = depth;
    for (int l = 1; l < depth; ++l)
        if (L[l].rows <= kCtaRows) { first = l; break; }
    // FP32 levels with the full stencil: the three-threads-a-row sweep
    auto split = [&](int l) { return std::is_same<T, float>::value && full_stencil(L[l], D); };
    auto grid3 = [&](int l) { return (unsigned)((L[l].rows + 39) / 40); };   // 4 warps of 10 rows a block
    auto jacobi = [&](int l) {
        if constexpr (std::is_same<T, float>::value) {
            if (split(l)) {
                { k_mg_sweep3<D, false><<<grid3(l), 128, 0, st>>>(L[l], cof + oc(l), invd + ov(l), Qp + ov(l), cur[l], oth[l], flags); MPH_COUNT_LAUNCH(); }
                T* t = cur[l]; cur[l] = oth[l]; oth[l] = t;
                return;
            }
        }
        { k_mg_jacobi<D, T><<<grid_for(L[l].rows, 128), 128, 0, st>>>(L[l], cof + oc(l), invd + ov(l), Qp + ov(l), cur[l], oth[l],
                                                                       flags); MPH_COUNT_LAUNCH(); }
        T* t = cur[l]; cur[l] = oth[l]; oth[l] = t;
    };
    auto residual = [&](int l) {
        if constexpr (std::is_same<T, float>::value) {
            if (split(l)) {
                { k_mg_sweep3<D, true><<<grid3(l), 128, 0, st>>>(L[l], cof + oc(l), nullptr, Qp + ov(l), cur[l], Rp + ov(l), flags); MPH_COUNT_LAUNCH(); }
                return;
            }
        }
        { k_mg_residual<D, T><<<grid_for(L[l].rows, 128), 128, 0, st>>>(L[l], cof + oc(l), Qp + ov(l), cur[l], Rp + ov(l), flags); MPH_COUNT_LAUNCH(); }
    };
    // down, grid-wide levels
    { k_mg_p2g<D, T, TQ><<<grid_for(L[0].rows, 128), 128, 0, st>>>(c->dp, L[0], c->d.bucket, q, invd + ov(0), Qp + ov(0),
                                                                   cur[0], flags); MPH_COUNT_LAUNCH(); }
    for (int k = 0; k < 1 + extra0; ++k) jacobi(0);      // level 0: 2 updates (+ extra0)
    for (int l = 1; l < first; ++l) {
        residual(l - 1);
        { k_mg_restrict<D, T><<<grid_for(L[l].rows, 128), 128, 0, st>>>(L[l - 1], L[l], Rp + ov(l - 1), invd + ov(l), Qp + ov(l),
                                                                        cur[l], flags); MPH_COUNT_LAUNCH(); }
        const int sweeps = (l == depth - 1) ? coarsest : pre;   // coarsest: 4 sweeps + one more update
        for (int k = 0; k < sweeps; ++k) jacobi(l);
    }
    if (first < depth) {
        residual(first - 1);
        CoarseArgs<T> A;
        A.first = first;
        A.depth = depth;
        for (int l = 0; l < depth; ++l) {
            A.L[l] = L[l];
            A.cof[l] = cof + oc(l);
            A.invd[l] = invd + ov(l);
            A.Q[l] = Qp + ov(l);
            A.Sa[l] = Sa + ov(l);
            A.Sb[l] = Sb + ov(l);
            A.R[l] = Rp + ov(l);
        }
        A.Sfine = cur[first - 1];
        A.pre = pre;
        A.post = post;
        A.dense = -1;
        A.dinv = nullptr;
        if constexpr (std::is_same<T, float>::value) {
            if (c->dense_level >= first && c->dense_level < depth) {
                A.dense = c->dense_level;
                A.dinv = c->d.mg_dinv32;
            }
        }
        if (kClusterCtas > 8) {
            static std::once_flag once;
            std::call_once(once, [] {
                cudaFuncSetAttribute(k_mg_small_levels<D, T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            });
        }
        { k_mg_small_levels<D, T><<<kClusterCtas, kCtaThreads, 0, st>>>(A, flags); MPH_COUNT_LAUNCH(); }
    }
    // up, grid-wide levels: the block kernel already prolongated into level
    // first-1; without it the coarsest level is prolongated here
    auto prolong = [&](int l) {   // S_{l-1} += P S_l
        { k_mg_prolong<D, T><<<grid_for(L[l - 1].rows, 128), 128, 0, st>>>(L[l - 1], L[l], cur[l], cur[l - 1], flags); MPH_COUNT_LAUNCH(); }
    };
    int top = first - 1;
    if (first == depth && depth > 1) {
        prolong(depth - 1);
        top = depth - 2;
    }
    for (int l = top; l >= 1; --l) {
        for (int k = 0; k < post; ++k) jacobi(l);
        prolong(l);
    }
    for (int k = 0; k < 2 + extra0; ++k) jacobi(0);      // level 0 post-smoothing
    const int blocks = std::min<int>(grid_for(c->dp.Nf, 256), kReduceBlocks);
    { k_mg_g2p_dot<D, T, TQ><<<blocks, 256, 0, st>>>(c->dp, L[0], c->d.key, invDiag, q, cur[0], u, c->d.partials,
                                                     (unsigned*)(c->d.flags + kFlagCounter), dot_out, flags); MPH_COUNT_LAUNCH(); }
}

// The mixed form's exact coarse solve: the first level handled by one block
// of the small-level kernel (at most kCtaThreads rows) that also has at most
// kDenseRows rows is solved with its dense FP32 inverse, built each step
// after the level stencils, instead of the reference's smoothing of it and
// the levels below (c->dense_level = -1: none, the reference's V-cycle).
int mixed_dense_coarse(mph_case* c)
{
    c->dense_level = -1;
    if (!c->dense_coarse || c->mg_depth < 0) return MPH_OK;
    const int depth = c->mg_depth >= 1 ? std::min(c->depth, c->mg_depth) : c->depth;   // the cycle's levels
    int first = depth;
    for (int l = 1; l < depth; ++l)
        if (c->lv[l].rows <= kCtaRows) { first = l; break; }
    int lev = -1;
    for (int l = first; l < depth; ++l)
        if (c->lv[l].rows <= kDenseRows) { lev = l; break; }
    if (lev < 0) return MPH_OK;
    const int n = c->lv[lev].rows;
    if ((long long)n * n > c->d.cap_mg_dinv32) {
        if (c->d.mg_dinv32) cudaFree(c->d.mg_dinv32);
        c->d.mg_dinv32 = nullptr;
        c->d.cap_mg_dinv32 = 0;
        MPH_CUDA(cudaMalloc((void**)&c->d.mg_dinv32, (size_t)kDenseRows * kDenseRows * sizeof(float)));
        c->d.cap_mg_dinv32 = (long long)kDenseRows * kDenseRows;
    }
    const int smem = (n * n + n) * (int)sizeof(float);
    // the attribute is per function and device, shared by every case (and
    // by the host threads of a batch or a server): always the largest size
    const int smax = (kDenseRows * kDenseRows + kDenseRows) * (int)sizeof(float);
    const LevelK L = level_k(c, lev);
    const float* cof = c->d.mg_cof32 + c->lv[lev].off_cof;
    if (c->dim == 2) {
        MPH_CUDA(cudaFuncSetAttribute(k_mg_dense_inv<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
        { k_mg_dense_inv<2><<<1, 1024, smem, c->stream>>>(L, cof, c->d.mg_dinv32); MPH_COUNT_LAUNCH(); }
    } else {
        MPH_CUDA(cudaFuncSetAttribute(k_mg_dense_inv<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
        { k_mg_dense_inv<3><<<1, 1024, smem, c->stream>>>(L, cof, c->d.mg_dinv32); MPH_COUNT_LAUNCH(); }
    }
    MPH_CUDA(cudaGetLastError());
    c->dense_level = lev;
    return MPH_OK;
}

// FP32 V-cycle of the mixed form: the FP32 copies of the level stencils and
// of D^-1 (prepared after the FP64 build), FP32 level vectors, FP64 (q,u) dot
void vcycle_mixed(mph_case* c, const float* q, float* u, double* dot_out)
{
    DeviceState& d = c->d;
    const float* invDiag32 = d.v32 + 7 * (size_t)c->dp.Nf * c->dim;
    if (c->dim == 2)
        vcycle_t<2, float, float>(c, q, u, invDiag32, d.mg_cof32, d.mg_invd32, d.mg_q32, d.mg_s32, d.mg_r32, d.mg_res32, dot_out,
                                  c->mixed_extra_sweeps);
    else
        vcycle_t<3, float, float>(c, q, u, invDiag32, d.mg_cof32, d.mg_invd32, d.mg_q32, d.mg_s32, d.mg_r32, d.mg_res32, dot_out,
                                  c->mixed_extra_sweeps);
}

void vcycle_fp64(mph_case* c, const double* q, double* u, double* dot_out)
{
    DeviceState& d = c->d;
    if (c->dim == 2)
        vcycle_t<2, double, double>(c, q, u, d.invDiag, d.mg_cof, d.mg_invd, d.mg_q, d.mg_s, d.mg_r, d.mg_res, dot_out);
    else
        vcycle_t<3, double, double>(c, q, u, d.invDiag, d.mg_cof, d.mg_invd, d.mg_q, d.mg_s, d.mg_r, d.mg_res, dot_out);
}

}  // namespace mph
