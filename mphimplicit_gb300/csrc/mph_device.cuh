// mph_device.cuh - device helpers shared by the kernels.
//
// Exact arithmetic: the cell keys, neighbour decisions, particle motion and
// the particle-number densities are computed with explicitly rounded
// operations (__dadd_rn, __dmul_rn, ...), which the compiler never contracts
// into FMAs.  They reproduce the reference's FP64 expressions operation by
// operation, so sort permutations and neighbour lists match it bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "mph_internal.h"

namespace mph {

#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn
#define DDIV __ddiv_rn

__host__ __device__ inline int vs_of(int dim) { return dim == 2 ? 2 : 4; }

template <int D> struct VS { static constexpr int v = D == 2 ? 2 : 4; };

// Mod(x, w) = x - w*floor(x/w) (reference macro, main.cpp:79), each operation
// rounded as in the reference.
__device__ __forceinline__ double mod_exact(double x, double w)
{
    return DSUB(x, DMUL(w, floor(DDIV(x, w))));
}

// Minimum-image component x_j - x_i: Mod(xj - xi + W/2, W) - W/2.  For
// 0 <= t < wsafe (wsafe = 0.75 W) floor(t/W) is 0 and Mod(t, W) == t exactly,
// so the division is skipped.  The range test compares bit patterns on the
// integer pipe (FP64 issues at a small fraction of the FP32 rate on this
// part): non-negative doubles order as their bit patterns; -0 (never formed
// here: hw > 0) and NaN of either sign take the exact path, which returns the
// same.
__device__ __forceinline__ double sep_exact(double xj, double xi, double hw, double w, double wsafe)
{
    const double t = DADD(DSUB(xj, xi), hw);
    const long long tb = __double_as_longlong(t);
    const double m = (tb >= 0 && tb < __double_as_longlong(wsafe)) ? t : mod_exact(t, w);
    return DSUB(m, hw);
}

// Radius tests of a squared distance r2 from norm2_exact (+0, positive, or
// NaN; never -0) against R2 > 0, by bit patterns as in sep_exact: the same
// outcome as the FP64 forms named, NaN included.
__device__ __forceinline__ bool r2_within(double r2, double R2)       // R2 - r2 >= 0
{
    const long long b = __double_as_longlong(r2);
    return b >= 0 && b <= __double_as_longlong(R2);
}
__device__ __forceinline__ bool r2_pos_below(double r2, double R2)    // r2 != 0 && R2 - r2 > 0
{
    const long long b = __double_as_longlong(r2);
    return b > 0 && b < __double_as_longlong(R2);
}

template <int D>
__device__ __forceinline__ double norm2_exact(const double* q)
{
    double s = DADD(DMUL(q[0], q[0]), DMUL(q[1], q[1]));
    if (D == 3) s = DADD(s, DMUL(q[2], q[2]));
    return s;
}

template <int D>
__device__ __forceinline__ void load_vec(const double* __restrict__ a, int i, double* v)
{
    if (D == 2) {
        const double2 t = reinterpret_cast<const double2*>(a)[i];
        v[0] = t.x; v[1] = t.y;
    } else {
        const double2 t0 = reinterpret_cast<const double2*>(a)[2 * i];
        const double2 t1 = reinterpret_cast<const double2*>(a)[2 * i + 1];
        v[0] = t0.x; v[1] = t0.y; v[2] = t1.x;
    }
}
// FP32 [N][VS] record (float2 in 2-D, float4 in 3-D)
template <int D>
__device__ __forceinline__ void load_f32(const float* __restrict__ a, int i, float* v)
{
    if (D == 2) {
        const float2 t = reinterpret_cast<const float2*>(a)[i];
        v[0] = t.x; v[1] = t.y; v[2] = 0.f;
    } else {
        const float4 t = reinterpret_cast<const float4*>(a)[i];
        v[0] = t.x; v[1] = t.y; v[2] = t.z;
    }
}
template <int D>
__device__ __forceinline__ void store_vec(double* a, int i, const double* v)
{
    if (D == 2) {
        reinterpret_cast<double2*>(a)[i] = make_double2(v[0], v[1]);
    } else {
        reinterpret_cast<double2*>(a)[2 * i] = make_double2(v[0], v[1]);
        reinterpret_cast<double2*>(a)[2 * i + 1] = make_double2(v[2], 0.0);
    }
}

template <int D>
__device__ __forceinline__ void sep_vec(const DevParams& P, const double* xj, const double* xi, double* q)
{
#pragma unroll
    for (int d = 0; d < D; ++d) q[d] = sep_exact(xj[d], xi[d], P.hw[d], P.dw[d], P.wsafe[d]);
}

// Weight functions (main.cpp:236-307) with the reference's evaluation order.
__device__ __forceinline__ double w_a(double kf, double r, double h)
{
    const double q = DDIV(r, h);
    const double oq = DSUB(1.0, q);
    return DMUL(DMUL(DMUL(kf, q), oq), oq);
}
__device__ __forceinline__ double dw_a(double kf, double r, double h)
{
    const double q = DDIV(r, h);
    return DMUL(DMUL(DMUL(kf, DSUB(1.0, q)), DSUB(1.0, DMUL(3.0, q))), DDIV(1.0, h));
}
__device__ __forceinline__ double w_quad(double kf, double r, double h)
{
    const double oq = DSUB(1.0, DDIV(r, h));
    return DMUL(kf, DMUL(oq, oq));
}
__device__ __forceinline__ double dw_quad(double kf, double r, double h)
{
    return DMUL(kf, DMUL(DDIV(-2.0, h), DSUB(1.0, DDIV(r, h))));
}

// The warp sums of D per-lane FP64 values by reduce-scatter: the same pairs,
// each added once, as the xor butterfly `v += shfl_xor(v, o)` for o = 16 ... 1
// (FP64 addition commutes, so every partial sum has the butterfly's bits),
// with 6 FP64 adds a lane in 3-D (5 in 2-D) instead of 15 (10): FP64 issues
// at a small fraction of the FP32 rate on this part.  Lane l returns the sum
// of component min(l >> 3, 2) in 3-D, l >> 4 in 2-D.
template <int D>
__device__ __forceinline__ double warp_sum_scatter(const double* v, int lane)
{
    const unsigned full = 0xffffffffu;
    const bool hi = (lane & 16) != 0;
    if (D == 2) {
        double a = hi ? v[1] : v[0];
        a += __shfl_xor_sync(full, hi ? v[0] : v[1], 16);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) a += __shfl_xor_sync(full, a, o);
        return a;
    }
    // lanes 0-15 keep components 0 and 1, lanes 16-31 component 2 (twice)
    double a0 = hi ? v[2] : v[0];
    double a1 = hi ? v[2] : v[1];
    a0 += __shfl_xor_sync(full, hi ? v[0] : v[2], 16);
    a1 += __shfl_xor_sync(full, hi ? v[1] : v[2], 16);
    // lanes 0-7 component 0, 8-15 component 1, 16-31 component 2
    const bool b8 = (lane & 8) != 0;
    double a = b8 ? a1 : a0;
    a += __shfl_xor_sync(full, b8 ? a0 : a1, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) a += __shfl_xor_sync(full, a, o);
    return a;
}

// The same for N (a power of two up to 32) values a lane: at the step of
// offset o, lanes with bit o set keep the upper half of their values and the
// others the lower half, each adding the partner's copy of the half it keeps
// (N - 1 adds, then plain butterfly steps: 16 adds for N = 16 against 80).
// Lane l returns the warp sum of value l >> (5 - log2 N).
template <int N>
__device__ __forceinline__ double warp_reduce_scatter(double (&v)[N], int lane)
{
    constexpr int L = N == 2 ? 1 : N == 4 ? 2 : N == 8 ? 3 : N == 16 ? 4 : 5;
    static_assert((1 << L) == N, "N must be a power of two, at most 32");
#pragma unroll
    for (int s = 0; s < L; ++s) {
        const int o = 16 >> s;
        const bool up = (lane & o) != 0;
        const int h = (N >> s) / 2;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const double keep = up ? v[h + k] : v[k];
            const double send = up ? v[k] : v[h + k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    double a = v[0];
#pragma unroll
    for (int o = 16 >> L; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
}

__device__ __forceinline__ bool is_wall(int t) { return t >= 2 && t < 4; }
__device__ __forceinline__ bool is_fluid(int t) { return t >= 0 && t < 2; }

__device__ __forceinline__ int wrapc(int i, int n) { return (i % n + n) % n; }
__device__ __forceinline__ int cell_id(const DevParams& P, int x, int y, int z)
{
    return wrapc(x, P.cc[0]) * P.cc[1] * P.cc[2] + wrapc(y, P.cc[1]) * P.cc[2] + wrapc(z, P.cc[2]);
}
// cell coordinates decoded from a sort key as the reference does (main.cpp:1410-1412)
__device__ __forceinline__ void key_coords(const DevParams& P, int k, int* c)
{
    c[0] = (k / (P.cc[1] * P.cc[2])) % P.T;
    c[1] = (k / P.cc[2]) % P.cc[1];
    c[2] = k % P.cc[2];
}

// The level-0 multigrid grid (the fluid-cell bounding box of the neighbour
// grid) as the assembly sees it: a row's partial stencil has one D x D block
// per neighbour cell slot (st0*st1*st2 slots, periodic on the grid index).
struct Level0Map {
    int mn[3], cnt[3], st[3];
    int S;          // st0*st1*st2
    int folded;     // 1 if some active axis has fewer than 3 grid cells
};

// slot of the cell of key keyj in the stencil of the cell at grid coords gi
template <int D>
__device__ __forceinline__ int stencil_slot(const DevParams& P, const Level0Map& M, const int* gi, int keyj)
{
    int jc[3];
    key_coords(P, keyj, jc);
    int o[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) o[d] = ((jc[d] - M.mn[d]) - gi[d] + 1 + M.cnt[d]) % M.cnt[d];
    return M.st[2] * M.st[1] * o[0] + M.st[2] * o[1] + o[2];
}

inline unsigned grid_for(long long n, int block)
{
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return (unsigned)g;
}

}  // namespace mph
