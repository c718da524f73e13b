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
// so the division is skipped.
__device__ __forceinline__ double sep_exact(double xj, double xi, double hw, double w, double wsafe)
{
    const double t = DADD(DSUB(xj, xi), hw);
    const double m = (t >= 0.0 && t < wsafe) ? t : mod_exact(t, w);
    return DSUB(m, hw);
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
