// k_multigrid.cu - cell-aggregation multigrid (main.cpp:2647-3546, 4122-4266).
//
// Level L is the fluid-cell bounding box of the neighbour grid coarsened L
// times by 2 (calculateMultiGridDepth, main.cpp:2777-2859).  Restriction (sum
// of the 2^D children), prolongation (injection) and the particle<->grid
// transfers (P2G sum, G2P injection) are index maps computed on the fly; only
// the level matrices are stored, as dense 3^D-cell block stencils with the
// reference's periodic wrap on the grid index.
//
// Build:  level 0 = per-cell sums of the per-row partial stencils written by
//         the assembly pass; level L = the reference's re-binning of level
//         L-1's stencil rows onto the parent cells (same summation order);
//         invD = 2 / sum |a_row| (calculateMultiGridInvDiagA, main.cpp:3510).
// V-cycle: one fused Jacobi kernel per smoothing sweep
//         (S_new = S + invD (Q - A S)); the fine residual is recomputed inside
//         the restriction kernel; the last kernel adds G2P S_0 to D^-1 q and
//         forms the (q, u) partial dot product.
#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

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

// ---- build -------------------------------------------------------------------
template <int D>
__global__ void k_mg_level0(DevParams P, LevelK L, const int* __restrict__ bucket, const double* __restrict__ part,
                            double* __restrict__ cof)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)L.rows * L.width) return;
    const int row = (int)(t / L.width), e = (int)(t % L.width);
    const int g = row / D, rD = row % D;
    const int slot = e / D, sD = e % D;
    const int S = L.st[0] * L.st[1] * L.st[2];
    int p[3];
    grid_coords(L, g, p);
    const int cx = p[0] + L.mn[0], cy = p[1] + L.mn[1], cz = p[2] + L.mn[2];
    double sum = 0.0;
    if (cx < P.cc[0] && cy < P.cc[1] && cz < P.cc[2]) {
        const int ic = cell_id(P, cx, cy, cz);
        for (int i = bucket[ic]; i < bucket[ic + 1]; ++i) sum += part[((size_t)i * S + slot) * D * D + rD * D + sD];
    }
    cof[t] = sum;
}

template <int D>
__global__ void k_mg_coarse(LevelK S_, LevelK L, const double* __restrict__ cofS, double* __restrict__ cofL)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)L.rows * L.width) return;
    const int rowL = (int)(t / L.width), e = (int)(t % L.width);
    const int g = rowL / D, rD = rowL % D;
    const int oslot = e / D, sD = e % D;
    int p[3];
    grid_coords(L, g, p);
    int fm[3], fM[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int lc = p[d] + L.mn[d];
        fm[d] = S_.mn[d] > 2 * lc ? 1 : 0;
        fM[d] = S_.mx[d] < 2 * (lc + 1) ? 1 : 0;
    }
    double sum = 0.0;
    for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
        for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
            for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                const int sg = grid_index(S_, 2 * (p[0] + L.mn[0]) + dx - S_.mn[0], 2 * (p[1] + L.mn[1]) + dy - S_.mn[1],
                                          2 * (p[2] + L.mn[2]) + dz - S_.mn[2]);
                int sp[3];
                grid_coords(S_, sg, sp);
                const double* in = cofS + (size_t)(sg * D + rD) * S_.width;
                for (int ix = 0; ix < S_.st[0]; ++ix)
                    for (int iy = 0; iy < S_.st[1]; ++iy)
                        for (int iz = 0; iz < S_.st[2]; ++iz) {
                            const int jf[3] = {(sp[0] + ix - 1 + S_.cnt[0]) % S_.cnt[0], (sp[1] + iy - 1 + S_.cnt[1]) % S_.cnt[1],
                                               (sp[2] + iz - 1 + S_.cnt[2]) % S_.cnt[2]};
                            int o[3];
#pragma unroll
                            for (int d = 0; d < 3; ++d) {
                                const int jl = (jf[d] + S_.mn[d]) / 2 - L.mn[d];
                                o[d] = (jl - p[d] + 1 + L.cnt[d]) % L.cnt[d];
                            }
                            if (L.st[2] * L.st[1] * o[0] + L.st[2] * o[1] + o[2] != oslot) continue;
                            sum += in[D * (S_.st[2] * S_.st[1] * ix + S_.st[2] * iy + iz) + sD];
                        }
            }
    cofL[t] = sum;
}

__global__ void k_mg_invd(int rows, int width, const double* __restrict__ cof, double* __restrict__ invd)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    double s = 0.0;
    for (int k = 0; k < width; ++k) s += fabs(cof[(size_t)row * width + k]);
    invd[row] = s != 0.0 ? 2.0 / s : 0.0;
}

void launch_mg_level0(mph_case* c)
{
    const LevelK L = level_k(c, 0);
    const long long n = (long long)L.rows * L.width;
    double* cof = c->d.mg_cof + c->lv[0].off_cof;
    if (c->dim == 2) { k_mg_level0<2><<<grid_for(n, 256), 256, 0, c->stream>>>(c->dp, L, c->d.bucket, c->d.part, cof); MPH_COUNT_LAUNCH(); }
    else { k_mg_level0<3><<<grid_for(n, 256), 256, 0, c->stream>>>(c->dp, L, c->d.bucket, c->d.part, cof); MPH_COUNT_LAUNCH(); }
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

// ---- V-cycle kernels -----------------------------------------------------------
template <int D, typename T>
__device__ __forceinline__ T level_residual(const LevelK& L, const T* __restrict__ cof, const T* __restrict__ Q,
                                            const T* __restrict__ S, int row)
{
    const int g = row / D;
    int p[3];
    grid_coords(L, g, p);
    const T* a = cof + (size_t)row * L.width;
    T sum = 0;
    int e = 0;
    for (int ix = 0; ix < L.st[0]; ++ix)
        for (int iy = 0; iy < L.st[1]; ++iy)
            for (int iz = 0; iz < L.st[2]; ++iz) {
                const int jg = stencil_col(L, p, ix, iy, iz);
#pragma unroll
                for (int sD = 0; sD < D; ++sD, ++e) sum += (-a[e]) * S[jg * D + sD];
            }
    return Q[row] + sum;
}

// S_out = S_in + invD (Q - A S_in)
template <int D, typename T>
__global__ void k_mg_jacobi(LevelK L, const T* __restrict__ cof, const T* __restrict__ invd, const T* __restrict__ Q,
                            const T* __restrict__ Sin, T* __restrict__ Sout, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    const T r = level_residual<D, T>(L, cof, Q, Sin, row);
    Sout[row] = Sin[row] + invd[row] * r;
}

// Q_L = R (Q_S - A_S S_S) over the children; S_L = invD_L Q_L
template <int D, typename T>
__global__ void k_mg_restrict(LevelK S_, LevelK L, const T* __restrict__ cofS, const T* __restrict__ QS,
                              const T* __restrict__ SS, const T* __restrict__ invdL, T* __restrict__ QL,
                              T* __restrict__ SL, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= L.rows) return;
    const int g = row / D, rD = row % D;
    int p[3];
    grid_coords(L, g, p);
    int fm[3], fM[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int lc = p[d] + L.mn[d];
        fm[d] = S_.mn[d] > 2 * lc ? 1 : 0;
        fM[d] = S_.mx[d] < 2 * (lc + 1) ? 1 : 0;
    }
    T sum = 0;
    for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
        for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
            for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                const int sg = grid_index(S_, 2 * (p[0] + L.mn[0]) + dx - S_.mn[0], 2 * (p[1] + L.mn[1]) + dy - S_.mn[1],
                                          2 * (p[2] + L.mn[2]) + dz - S_.mn[2]);
                sum += level_residual<D, T>(S_, cofS, QS, SS, sg * D + rD);
            }
    QL[row] = sum;
    SL[row] = invdL[row] * sum;
}

// S_S += P S_L (injection from the parent cell)
template <int D, typename T>
__global__ void k_mg_prolong(LevelK S_, LevelK L, const T* __restrict__ SL, T* __restrict__ SS, const int* __restrict__ flags)
{
    if (flags[kFlagDone]) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= S_.rows) return;
    const int g = row / D, rD = row % D;
    int p[3];
    grid_coords(S_, g, p);
    const int lg = grid_index(L, (p[0] + S_.mn[0]) / 2 - L.mn[0], (p[1] + S_.mn[1]) / 2 - L.mn[1], (p[2] + S_.mn[2]) / 2 - L.mn[2]);
    SS[row] = SS[row] + SL[lg * D + rD];
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
    const int n = P.Nf * D;
    double acc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k / D, rD = k % D;
        int cc3[3];
        key_coords(P, key[i], cc3);
        const int g = grid_index(L, cc3[0] - L.mn[0], cc3[1] - L.mn[1], cc3[2] - L.mn[2]);
        const TQ qk = q[k];
        const TQ v = invDiag[k] * qk + (TQ)S0[g * D + rD];
        u[k] = v;
        acc += (double)qk * (double)v;
    }
    reduce_finalize(acc, partials, counter, out);
}

// ---- host-side V-cycle -----------------------------------------------------------
template <int D, typename T, typename TQ>
static void vcycle_t(mph_case* c, const TQ* q, TQ* u, const TQ* invDiag, const T* cof, const T* invd, T* Qp, T* Sa, T* Sb,
                     double* dot_out)
{
    const int depth = c->depth;
    cudaStream_t st = c->stream;
    const int* flags = c->d.flags;
    std::vector<LevelK> L(depth);
    for (int l = 0; l < depth; ++l) L[l] = level_k(c, l);
    auto off_v = [&](int l) { return c->lv[l].off_vec; };
    auto off_c = [&](int l) { return c->lv[l].off_cof; };
    // current S buffer of each level (ping-pong between Sa and Sb)
    std::vector<T*> cur(depth), oth(depth);
    for (int l = 0; l < depth; ++l) { cur[l] = Sa + off_v(l); oth[l] = Sb + off_v(l); }
    auto jacobi = [&](int l) {
        { k_mg_jacobi<D, T><<<grid_for(L[l].rows, 128), 128, 0, st>>>(L[l], cof + off_c(l), invd + off_v(l), Qp + off_v(l),
                                                                     cur[l], oth[l], flags); MPH_COUNT_LAUNCH(); }
        std::swap(cur[l], oth[l]);
    };
    // pre-smoothing, going down
    { k_mg_p2g<D, T, TQ><<<grid_for(L[0].rows, 128), 128, 0, st>>>(c->dp, L[0], c->d.bucket, q, invd + off_v(0), Qp + off_v(0),
                                                                 cur[0], flags); MPH_COUNT_LAUNCH(); }
    jacobi(0);                                   // 2 sweeps on level 0
    for (int l = 1; l < depth; ++l) {
        { k_mg_restrict<D, T><<<grid_for(L[l].rows, 128), 128, 0, st>>>(L[l - 1], L[l], cof + off_c(l - 1), Qp + off_v(l - 1),
                                                                       cur[l - 1], invd + off_v(l), Qp + off_v(l), cur[l], flags); MPH_COUNT_LAUNCH(); }
        const int sweeps = (l == depth - 1) ? 5 : 3;   // coarsest: 4 sweeps + one more update
        for (int k = 1; k < sweeps; ++k) jacobi(l);
    }
    // post-smoothing, going up
    for (int l = depth - 1; l >= 1; --l) {
        { k_mg_prolong<D, T><<<grid_for(L[l - 1].rows, 128), 128, 0, st>>>(L[l - 1], L[l], cur[l], cur[l - 1], flags); MPH_COUNT_LAUNCH(); }
        const int sweeps = (l - 1 == 0) ? 2 : 3;
        for (int k = 0; k < sweeps; ++k) jacobi(l - 1);
    }
    const int n = c->dp.Nf * D;
    const int blocks = std::min<int>(grid_for(n, 256), kReduceBlocks);
    { k_mg_g2p_dot<D, T, TQ><<<blocks, 256, 0, st>>>(c->dp, L[0], c->d.key, invDiag, q, cur[0], u, c->d.partials,
                                                   (unsigned*)(c->d.flags + kFlagCounter), dot_out, flags); MPH_COUNT_LAUNCH(); }
}

void vcycle_fp64(mph_case* c, const double* q, double* u, double* dot_out)
{
    if (c->dim == 2)
        vcycle_t<2, double, double>(c, q, u, c->d.invDiag, c->d.mg_cof, c->d.mg_invd, c->d.mg_q, c->d.mg_s, c->d.mg_r, dot_out);
    else
        vcycle_t<3, double, double>(c, q, u, c->d.invDiag, c->d.mg_cof, c->d.mg_invd, c->d.mg_q, c->d.mg_s, c->d.mg_r, dot_out);
}

}  // namespace mph
