// k_factored.cu - the FP64 operator of the mixed form, applied in factored
// form instead of from assembled FP64 blocks.
//
// A = inertia + V + C Lambda C^T (calculateMatrixA main.cpp:2251-2335,
// multiplyMatrixC main.cpp:2574-2642).  Its viscous blocks are rank one:
// block (i,j) = -f_ij e_ij (x) e_ij for a fluid neighbour j, and the diagonal
// block adds f_ij e_ij (x) e_ij over every neighbour (fluid and wall), so
//
//   (V x)_i = sum_{j fluid} f e (e . (x_i - x_j)) + sum_{j wall} f e (e . x_i).
//
// The C Lambda C^T part is C (Lambda (C^T x)): t_k = sum over the fluid rows j
// whose P-list holds k of C_jk . x_j (the transposed P-lists), then
// sum_k C_ik lambda_k t_k.  In exact arithmetic this equals the assembled A
// whenever 2 RadiusP < MaxRadius (every pair with a common P-neighbour is then
// in the neighbour list, where the reference adds the product); the engine
// uses this form only then.
//
// k_pair_terms stores (e, f) per neighbour slot of every fluid row in FP32
// (used by the FP32 blocks and by the viscous part of the FP64 residual) and b
// in FP64; for the FP32 inner operator without blocks also the wall part of
// the FP32 viscous diagonal block, the FP32 inertia and the lambda-scaled C
// values.  No FP64 arithmetic is done per slot (the separation comes from
// two-float positions), against the nine-entry FP64 block and its
// accumulation of the assembled form; in the residual only inertia and
// C Lambda C^T (about 20 P-slots a row) are FP64.
#include <cuda_fp16.h>
#include <algorithm>
#include <atomic>
#include <climits>
#include <mutex>

#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

constexpr int kPairWarps = 8;
// warps per block of k_pair_terms (consecutive rows of a block share L1 for
// their position gathers)
#ifndef MPH_PT_WARPS
#define MPH_PT_WARPS 16
#endif
constexpr int kPtWarps = MPH_PT_WARPS;

// Tuning of the inner operator's viscous loop: slots unrolled per step and
// the minimum resident blocks of k_visc_pen32 (register cap).
#ifndef MPH_PAIR_UNROLL
#define MPH_PAIR_UNROLL 4
#endif
#ifndef MPH_PAIR_MINB
#define MPH_PAIR_MINB 1
#endif
// largest threads per block of k_visc_pen32 and k_resid_pairs (rows of a
// block share L1 for their x gathers); a case runs them with its option
// "pair_block" (128, 256 or this, the default)
#ifndef MPH_PAIR_BLOCK
#define MPH_PAIR_BLOCK 512
#endif
// largest threads per block of k_ct_apply32 (option "ct_block": 128 or this,
// the default)
#ifndef MPH_CT_BLOCK
#define MPH_CT_BLOCK 256
#endif
// Block-local neighbour columns of the inner operator: the fluid neighbours
// of a block of MPH_PAIR_BLOCK rows, sorted and deduplicated, at most kUMax
// of them (their x then fits the block's shared memory), found through a
// bitmap of an index window of at most kWinWords * 32 particles (2^18: two
// planes of neighbour cells of a 10^6-particle fluid body fit).
constexpr int kUMax = 8192;
constexpr int kLtsK = 32;   // slots of a row a slicing chunk takes
constexpr int kWinWords = 1 << 13;
constexpr int kPairUnroll = MPH_PAIR_UNROLL;
// the fluid slices are padded to a multiple of 4 slots (k_slice_width), which
// the operator's whole-slice loop steps through kPairUnroll at a time
static_assert(4 % kPairUnroll == 0, "the slice padding must be a multiple of the unroll");
// floats a staged s takes in shared memory in 3-D (3: packed, the default;
// 4: one 16-byte load, measured slower for the wider bank-conflict pattern)
#ifndef MPH_XS3
#define MPH_XS3 3
#endif
constexpr int kXs3 = MPH_XS3;


// (e, f) of every neighbour slot of the fluid rows in FP32, and b
// (main.cpp:2261-2304 for e, f; 2318-2333 and 2574-2584 for b).  The
// separation is the difference of the two-float positions (pos32, poslo32),
// within about one FP32 ulp of the FP64 difference (the exact minimum image
// of the neighbour search is evaluated only for periodic images); the rest
// of the viscous term is FP32: it is about nu dt / l0^2 (~1e-3) of the
// inertia term, so its FP32 rounding moves A x by ~1e-10 of |b| (the host
// keeps the factored form off when that bound would reach 1e-2 of the outer
// tolerance).  Inertia and C p stay FP64.
// (e, f) of the pair (i, j) in FP32, as every pair-term kernel evaluates it
// (one function, so that they agree bit for bit): x_j - x_i from the
// two-float positions (the high parts of nearby positions subtract with one
// FP32 rounding at most, so q is within about one FP32 ulp of the FP64
// difference, with no FP64 arithmetic); the exact minimum image only when a
// component is not well inside a quarter of the domain width (a periodic
// image, which also sets *wrap).  e = q / |q|, f = visc mu_ij w'(|q|) / |q|
// within RadiusV, else 0 (main.cpp:2261-2289).
template <int D>
__device__ __forceinline__ void pair_ef(const DevParams& P, int i, int j, int ti, const float* hi, const float* li,
                                        const int* __restrict__ type, const double* __restrict__ pos,
                                        const float* __restrict__ pos32, const float* __restrict__ poslo32,
                                        int* __restrict__ wrap, float* e, float& f)
{
    if (j != i) {
        float hj[3], lj[3];
        int tj;
        if (D == 3) {   // the high part's w holds the type bits (k_permute)
            const float4 h4 = reinterpret_cast<const float4*>(pos32)[j];
            hj[0] = h4.x; hj[1] = h4.y; hj[2] = h4.z;
            tj = __float_as_int(h4.w);
        } else {
            load_f32<D>(pos32, j, hj);
            tj = type[j];
        }
        load_f32<D>(poslo32, j, lj);
        float q32[3] = {0.f, 0.f, 0.f};
        bool inner = true;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            q32[d] = (hj[d] - hi[d]) + (lj[d] - li[d]);
            inner = inner && fabsf(q32[d]) < 0.48f * P.hw32[d];
        }
        if (!inner) {
            *wrap = 1;   // the recomputing inner operator then takes the minimum image
            double xi[3], xj[3], q[3];
            load_vec<D>(pos, i, xi);
            load_vec<D>(pos, j, xj);
            sep_vec<D>(P, xj, xi, q);
#pragma unroll
            for (int d = 0; d < D; ++d) q32[d] = (float)q[d];
        }
        const float r2 = q32[0] * q32[0] + q32[1] * q32[1] + q32[2] * q32[2];
        if (r2 != 0.f && P.rV2_32 - r2 > 0.f) {
            const float inv = rsqrtf(r2);
            const float wd = P.wdA32 * (1.f - (r2 * inv) * P.inv_rv32);
            f = P.vm32[ti][tj] * wd * inv;
#pragma unroll
            for (int d = 0; d < D; ++d) e[d] = q32[d] * inv;
        }
    }
}

// The end of a fluid row in the pair-term kernels, from its warp's per-lane
// partial sums: b_i = - C p + inertia v in FP64 (the lanes' sums by
// reduce-scatter; lane 8 r in 3-D, 16 r in 2-D, writes component r) and, with
// dinv, the inverse diagonal of A from FP32 sums (the mixed form's
// point-Jacobi preconditioner; lane r writes component r).
template <int D>
__device__ __forceinline__ void pair_row_end(const DevParams& P, int i, int ti, int lane, const double* sumv,
                                             const double* vi, float* tvd, float* dpd, double* __restrict__ bvec,
                                             double* __restrict__ dinv)
{
    const double sr = warp_sum_scatter<D>(sumv, lane);
    constexpr int kStep = D == 3 ? 8 : 16;
    const int r = lane / kStep;
    if (lane % kStep == 0 && r < D) {
        const double vr = r == 0 ? vi[0] : (r == 1 || D == 2 ? vi[1] : vi[2]);
        bvec[(size_t)i * D + r] = sr + P.inert64[ti] * vr;   // inertia as the assembly forms it
    }
    if (dinv) {
#pragma unroll
        for (int c = 0; c < D; ++c)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                tvd[c] += __shfl_xor_sync(0xffffffffu, tvd[c], o);
                dpd[c] += __shfl_xor_sync(0xffffffffu, dpd[c], o);
            }
        if (lane < D) {
            const float tv = lane == 0 ? tvd[0] : (lane == 1 ? tvd[1] : tvd[2]);
            const float dp = lane == 0 ? dpd[0] : (lane == 1 ? dpd[1] : dpd[2]);
            const float dg = P.inert32[ti] + tv + dp;
            dinv[(size_t)i * D + lane] = (double)(dg != 0.f ? 1.f / dg : 0.f);
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kPtWarps * 32)
k_pair_terms(DevParams P, const int* __restrict__ type, const double* __restrict__ pos, const float* __restrict__ pos32,
             const float* __restrict__ poslo32, const double* __restrict__ vel,
             const int* __restrict__ nc, const long long* __restrict__ nptr, const int* __restrict__ nind,
             const int* __restrict__ nfc, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
             const int* __restrict__ nindP, const double* __restrict__ cval, const double* __restrict__ pvec,
             float4* __restrict__ pe32, double* __restrict__ bvec, float* __restrict__ cvl32, unsigned* __restrict__ gmax,
             int* __restrict__ wrap, double* __restrict__ dinv)
{
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = wid; i < P.Nf; i += nwarps) {
        const int ti = type[i];
        const long long nb = nptr[i];
        const int n = nc[i], nf = nfc[i];
        double vi[3];
        load_vec<D>(vel, i, vi);
        float hi[3], li[3];
        load_f32<D>(pos32, i, hi);
        load_f32<D>(poslo32, i, li);
        float lm = 0.f;                                  // largest |g| component of the fluid slots
        float tvd[3] = {0.f, 0.f, 0.f}, dpd[3] = {0.f, 0.f, 0.f};   // dinv: viscous and C Lambda C^T diagonals
        for (int k = lane; k < n; k += 32) {
            const int j = nind[nb + k];
            float e[3] = {0.f, 0.f, 0.f};
            float f = 0.f;
            pair_ef<D>(P, i, j, ti, hi, li, type, pos, pos32, poslo32, wrap, e, f);
            pe32[nb + k] = make_float4(e[0], e[1], e[2], f);
            if (dinv) {
#pragma unroll
                for (int d = 0; d < D; ++d) tvd[d] += f * e[d] * e[d];
            }
            if (k < nf) lm = fmaxf(lm, sqrtf(f) * fmaxf(fabsf(e[0]), fmaxf(fabsf(e[1]), fabsf(e[2]))));
        }
        if (gmax) {   // the slice's largest |g| component, for the FP16 scale (f >= 0: bits order as values)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) lm = fmaxf(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            if (lane == 0) atomicMax(gmax + (i >> 5), __float_as_uint(lm));
        }
        // - C p over the row's P-neighbours (FP64); the wall velocities
        // follow in k_wall_terms64
        double sumv[3] = {0.0, 0.0, 0.0};
        const long long pb = nptrP[i];
        const int np = ncp[i];
        for (int a = lane; a < np; a += 32) {
            const int k = nindP[pb + a];
            const double pk = pvec[k];
#pragma unroll
            for (int r = 0; r < D; ++r) sumv[r] -= cval[(pb + a) * D + r] * pk;
            if (cvl32) {   // lambda_k C_ik for the FP32 inner operator
                const double lam = P.lambda[type[k]];
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    const float cl = (float)(cval[(pb + a) * D + r] * lam);
                    cvl32[(pb + a) * D + r] = cl;
                    dpd[r] += cl * (float)cval[(pb + a) * D + r];
                }
            }
        }
        pair_row_end<D>(P, i, ti, lane, sumv, vi, tvd, dpd, bvec, dinv);
    }
}

// k_pair_terms and the slicing of its fluid pair terms in one pass, for the
// point-Jacobi mixed form (which reads the pair terms only in the sliced
// layouts): a block of 32 warps per slice of 32 fluid rows, warp w on row w.
// Chunks of 32 fluid slots go through a shared-memory tile into the sliced
// FP32 g (pes32) and columns; the slice's largest |g| component then sets
// its scale and a second sweep over the slice (L2) writes the packed (or
// FP16) slot records.  The wall slots add to the diagonal only; b, lambda C
// and D^-1 as in k_pair_terms.  The same pair_ef and the same expressions as
// k_pair_terms and k_list_to_slices, so the outputs are theirs bit for bit.
template <int D, bool PACK>
__global__ void __launch_bounds__(1024)
k_pair_slices(DevParams P, const int* __restrict__ type, const double* __restrict__ pos, const float* __restrict__ pos32,
              const float* __restrict__ poslo32, const double* __restrict__ vel,
              const int* __restrict__ nc, const long long* __restrict__ nptr, const int* __restrict__ nind,
              const int* __restrict__ nfc, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
              const int* __restrict__ nindP, const double* __restrict__ cval, const double* __restrict__ pvec,
              const long long* __restrict__ sptr, int* __restrict__ scol, float* __restrict__ sval,
              unsigned* __restrict__ sval32, unsigned short* __restrict__ sval16, float* __restrict__ sscale,
              double* __restrict__ bvec, float* __restrict__ cvl32, int* __restrict__ wrap, double* __restrict__ dinv)
{
    constexpr int W = kLtsK * D + 1;   // odd row stride: no bank conflicts
    __shared__ float tile[32 * W];
    __shared__ int ctile[32 * (kLtsK + 1)];
    __shared__ float smax[32];
    const int sl = blockIdx.x, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = sl * 32 + w;
    const bool row = i < P.Nf;
    const long long sb = sptr[sl];
    const int width = (int)((sptr[sl + 1] - sb) / 32);
    int ti = 0, n = 0, nf = 0;
    long long nb = 0;
    float hi[3] = {0.f, 0.f, 0.f}, li[3] = {0.f, 0.f, 0.f};
    if (row) {
        ti = type[i];
        nb = nptr[i];
        n = nc[i];
        nf = nfc[i];
        load_f32<D>(pos32, i, hi);
        load_f32<D>(poslo32, i, li);
    }
    float lm = 0.f;
    float tvd[3] = {0.f, 0.f, 0.f}, dpd[3] = {0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < width; k0 += kLtsK) {   // fluid slots (the slice's width is theirs, padded)
        const int k = k0 + lane;
        float g[3] = {0.f, 0.f, 0.f};
        int col = 0;
        if (row && k < nf) {
            const int j = nind[nb + k];
            float e[3] = {0.f, 0.f, 0.f};
            float f = 0.f;
            pair_ef<D>(P, i, j, ti, hi, li, type, pos, pos32, poslo32, wrap, e, f);
#pragma unroll
            for (int d = 0; d < D; ++d) tvd[d] += f * e[d] * e[d];
            const float sf = sqrtf(f);
#pragma unroll
            for (int d = 0; d < D; ++d) g[d] = sf * e[d];
            lm = fmaxf(lm, sqrtf(f) * fmaxf(fabsf(e[0]), fmaxf(fabsf(e[1]), fabsf(e[2]))));
            col = j;
        }
#pragma unroll
        for (int d = 0; d < D; ++d) tile[w * W + lane * D + d] = g[d];
        ctile[w * (kLtsK + 1) + lane] = col;
        __syncthreads();
        const int kc = min(kLtsK, width - k0);
        for (int o = threadIdx.x; o < kc * D * 32; o += blockDim.x) {
            const int ln = o & 31, ec = o >> 5;   // ec = k_local * D + component
            sval[sb * D + (long long)k0 * D * 32 + o] = tile[ln * W + ec];
        }
        for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
            const int ln = o & 31, kl = o >> 5;
            scol[sb + (long long)(k0 + kl) * 32 + ln] = ctile[ln * (kLtsK + 1) + kl];
        }
        __syncthreads();
    }
    if (row)   // the wall slots: the viscous diagonal only
        for (int k = nf + lane; k < n; k += 32) {
            float e[3] = {0.f, 0.f, 0.f};
            float f = 0.f;
            pair_ef<D>(P, i, nind[nb + k], ti, hi, li, type, pos, pos32, poslo32, wrap, e, f);
#pragma unroll
            for (int d = 0; d < D; ++d) tvd[d] += f * e[d] * e[d];
        }
    // the slice's scale: its largest |g| component maps to 1023 (packed) or 2^15 (FP16)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lm = fmaxf(lm, __shfl_xor_sync(0xffffffffu, lm, o));
    if (lane == 0) smax[w] = lm;
    __syncthreads();
    float m = 0.f;
    for (int q = 0; q < 32; ++q) m = fmaxf(m, smax[q]);
    const float sigma = m / (PACK ? 1023.f : 32768.f);
    const float inv16 = m > 0.f ? 1.f / sigma : 0.f;
    if (threadIdx.x == 0) sscale[sl] = sigma;
    // the slot records from the sliced g just written (this block's, in L2)
    for (int o = threadIdx.x; o < width * 32; o += blockDim.x) {
        const int ln = o & 31, k = o >> 5;
        float gd[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) gd[d] = sval[sb * D + ((long long)k * D + d) * 32 + ln];
        if (PACK) {
            int q[3] = {0, 0, 0};
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const int lim = d == 2 ? 511 : 1023;
                const float v = gd[d] * inv16 * (d == 2 ? 0.5f : 1.f);
                q[d] = max(-lim, min(lim, __float2int_rn(v)));
            }
            sval32[sb + (long long)k * 32 + ln] =
                ((unsigned)q[0] & 0x7ffu) | (((unsigned)q[1] & 0x7ffu) << 11) | (((unsigned)q[2] & 0x3ffu) << 22);
        } else {
            unsigned h[3] = {0u, 0u, 0u};
#pragma unroll
            for (int d = 0; d < D; ++d) h[d] = __half_as_ushort(__float2half_rn(gd[d] * inv16));
            reinterpret_cast<uint2*>(sval16)[sb + (long long)k * 32 + ln] = make_uint2(h[0] | (h[1] << 16), h[2]);
        }
    }
    if (!row) return;   // warp-uniform
    // b = - C p + inertia v (FP64), lambda C for the inner operator, and the
    // C Lambda C^T diagonal, as k_pair_terms
    double vi[3];
    load_vec<D>(vel, i, vi);
    double sumv[3] = {0.0, 0.0, 0.0};
    const long long pb = nptrP[i];
    const int np = ncp[i];
    for (int a = lane; a < np; a += 32) {
        const int k = nindP[pb + a];
        const double pk = pvec[k];
#pragma unroll
        for (int r = 0; r < D; ++r) sumv[r] -= cval[(pb + a) * D + r] * pk;
        const double lam = P.lambda[type[k]];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const float cl = (float)(cval[(pb + a) * D + r] * lam);
            cvl32[(pb + a) * D + r] = cl;
            dpd[r] += cl * (float)cval[(pb + a) * D + r];
        }
    }
    pair_row_end<D>(P, i, ti, lane, sumv, vi, tvd, dpd, bvec, dinv);
}

// The wall neighbours of every fluid row in FP64 (after k_pair_terms), a
// warp per row: their viscous terms from the exact minimum image as the
// assembly of A (main.cpp:2274-2303), summed in FP64 into the wall part of
// the row's viscous diagonal block (sdiag64; an FP32 copy with the FP32
// inertia in sdiag32 for the inner operator) and, with the wall velocities,
// into b (main.cpp:2298-2300).  Wall slots are a few percent of a large
// case's slots, so FP64 costs little here and keeps the wall part of the
// outer residual and of b free of FP32 rounding.
template <int D>
__global__ void __launch_bounds__(256) k_wall_terms64(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                      const double* __restrict__ vel, const int* __restrict__ nc,
                                                      const int* __restrict__ nfc, const long long* __restrict__ nptr,
                                                      const int* __restrict__ nind, double* __restrict__ bvec,
                                                      float* __restrict__ sdiag32, double* __restrict__ sdiag64)
{
    // a warp per fluid row, its lanes over the row's wall slots; the lane
    // sums meet in a fixed shuffle tree (deterministic)
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= P.Nf) return;
    const int ti = type[i];
    const int n = nc[i], nf = nfc[i];
    double sd[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // xx xy xz yy yz zz
    double sw[3] = {0.0, 0.0, 0.0};
    // this lane's warp sum after the reduce-scatter: value lane >> 1 of
    // (sd[0..5], sw[0..2]); zero for a row without wall slots
    double val = 0.0;
    if (n > nf) {
        const long long nb = nptr[i];
        const double rV2 = P.rV * P.rV;
        double xi[3];
        load_vec<D>(pos, i, xi);
        for (int k = nf + lane; k < n; k += 32) {
            const int j = nind[nb + k];
            if (j == i) continue;
            double xj[3], q[3];
            load_vec<D>(pos, j, xj);
            sep_vec<D>(P, xj, xi, q);
            const double r2 = norm2_exact<D>(q);
            if (!r2_pos_below(r2, rV2)) continue;
            const double inv = rsqrt(r2);
            const double wd = -P.kfv * (P.m2h_rv * (1.0 - (r2 * inv) * P.inv_rv));
            const double f = P.visc * P.muij[ti][type[j]] * wd * inv;
            double e[3] = {0.0, 0.0, 0.0}, vj[3];
#pragma unroll
            for (int d = 0; d < D; ++d) e[d] = q[d] * inv;
            load_vec<D>(vel, j, vj);
            double ev = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) ev += e[d] * vj[d];
#pragma unroll
            for (int r = 0; r < D; ++r) sw[r] += f * e[r] * ev;
            sd[0] += f * e[0] * e[0];
            sd[1] += f * e[0] * e[1];
            sd[2] += f * e[0] * e[2];
            sd[3] += f * e[1] * e[1];
            sd[4] += f * e[1] * e[2];
            sd[5] += f * e[2] * e[2];
        }
        // the butterfly's sums (the same bits) with 16 FP64 adds a lane, not 45
        double v[16] = {sd[0], sd[1], sd[2], sd[3], sd[4], sd[5], sw[0], sw[1], sw[2],
                        0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        val = warp_reduce_scatter<16>(v, lane);
        const int t = lane >> 1;
        if ((lane & 1) == 0 && t >= 6 && t < 6 + D) bvec[(size_t)i * D + (t - 6)] += val;
    }
    if (sdiag32) {   // lane 2 t writes component t: one FP32 conversion a lane
        const int t = lane >> 1;
        if ((lane & 1) == 0 && t < 6) {
            sdiag32[(size_t)i * 8 + t] = (float)val;
            sdiag64[(size_t)i * 8 + t] = val;
        }
        if (lane == 1) sdiag32[(size_t)i * 8 + 6] = P.inert32[ti];
        if (lane == 3) sdiag32[(size_t)i * 8 + 7] = 0.f;
    }
}

__global__ void k_cval_f32(long long n, const double* __restrict__ a, float* __restrict__ b)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) b[k] = (float)a[k];
}

// t_k = sum over the transposed P-list of k of C_jk . x_j (every particle k)
template <int D>
__global__ void k_ct_apply(int N, DevParams P, const int* __restrict__ type, const long long* __restrict__ ctptr,
                           const int* __restrict__ ct_j, const double* __restrict__ ct_v, const double* __restrict__ x,
                           double* __restrict__ t)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    double s = 0.0;
    const long long e1 = ctptr[k + 1];
    for (long long e = ctptr[k]; e < e1; ++e) {
        const int j = ct_j[e];
#pragma unroll
        for (int d = 0; d < D; ++d) s += ct_v[e * D + d] * x[(size_t)j * D + d];
    }
    t[k] = P.lambda[type[k]] * s;   // lambda_k t_k, as the residuals use it
}

// r = b - A x in factored form, (r, r) -> *out (deterministic reduction):
// inertia and C Lambda t (t = C^T x) in FP64, the viscous pair terms in FP32
// on the FP32 copy x32 of x.
template <int D>
__global__ void __launch_bounds__(kPairWarps * 32)
k_resid_factored(DevParams P, const int* __restrict__ type, const int* __restrict__ nc, const int* __restrict__ nfc,
                 const long long* __restrict__ nptr, const int* __restrict__ nind, const float4* __restrict__ pe32,
                 const int* __restrict__ ncp, const long long* __restrict__ nptrP, const int* __restrict__ nindP,
                 const double* __restrict__ cval, const double* __restrict__ t, const double* __restrict__ x,
                 const float* __restrict__ x32, const double* __restrict__ b, double* __restrict__ r,
                 double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    double acc_rr = 0.0;
    for (int i = wid; i < P.Nf; i += nwarps) {
        float xi[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) xi[d] = x32[(size_t)i * D + d];
        float yv[3] = {0.f, 0.f, 0.f};
        const long long nb = nptr[i];
        const int n = nc[i], nf = nfc[i];
        for (int k = lane; k < n; k += 32) {
            const float4 p = pe32[nb + k];
            float dx[3] = {xi[0], xi[1], xi[2]};
            if (k < nf) {
                const int j = nind[nb + k];
#pragma unroll
                for (int d = 0; d < D; ++d) dx[d] -= x32[(size_t)j * D + d];
            }
            const float ed = p.x * dx[0] + p.y * dx[1] + (D == 3 ? p.z * dx[2] : 0.f);
            const float sc = p.w * ed;
            yv[0] += sc * p.x;
            yv[1] += sc * p.y;
            if (D == 3) yv[2] += sc * p.z;
        }
        double y[3] = {(double)yv[0], (double)yv[1], (double)yv[2]};
        const long long pb = nptrP[i];
        const int np = ncp[i];
        for (int a = lane; a < np; a += 32) {
            const int k = nindP[pb + a];
            const double lt = t[k];   // lambda_k t_k
#pragma unroll
            for (int d = 0; d < D; ++d) y[d] += cval[(pb + a) * D + d] * lt;
        }
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) y[d] += __shfl_xor_sync(0xffffffffu, y[d], o);
        if (lane == 0) {
            const double inert = P.inert64[type[i]];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const size_t k = (size_t)i * D + d;
                const double rv = b[k] - (inert * x[k] + y[d]);
                r[k] = rv;
                acc_rr += rv * rv;
            }
        }
    }
    reduce_finalize(acc_rr, partials, counter, out);
}

// ---- FP32 inner operator of the mixed form, without assembled blocks --------------
// The inner CR's y = A32 s from the FP32 pair terms in two launches, both one
// thread per row over sliced lists (entry e of row i at slice base + e*32 +
// lane, its D values at slice base * D + (e*D + d)*32 + lane: coalesced):
//   k_ct_apply32   t = C^T s per particle over the transposed P-lists, after
//                  the iteration's convergence test;
//   k_visc_pen32   y_i = (inertia + sum_{wall j} f e (x) e) s_i
//                        + sum_{fluid j} g (g . (s_i - s_j)) + sum_k lambda_k C_ik t_k
//                  with g = sqrt(f) e (f >= 0, so a fluid pair's terms
//                  f e (x) e are g (x) g), read from the packed slot records
//                  (11/11/10-bit fixed point of the slice's scale and a
//                  2-byte index: 6 bytes a slot, against 36 for an FP32
//                  block; option pair_pack 0: FP16, 8 bytes) — the viscous
//                  part is a few 1e-3 of the operator, so the 2^-11
//                  rounding of g moves the inner operator by ~1e-5 of itself;
//                  the FP64 outer residual takes the FP32 g.  (s, y) goes
//                  into the iteration's rho slot.  The pairs act on
//                  differences s_i - s_j, so the viscous sum has no
//                  cancellation between a large diagonal and its row.
// Same recurrences and flags as k_spmv32.
constexpr int kSIn0 = 16, kSIn = 17, kSTol2 = 23;
__device__ __forceinline__ int rho32_slot_f(int it) { return 20 + (it & 1); }

// A transposed slot is one 16-byte record: C (D floats, zero-padded) and the
// fluid row's column.  LOC: a block of MPH_CT_BLOCK particles whose lists
// hold ucount[b] >= 0 distinct fluid rows stages their s in shared memory;
// its records carry each row's rank among them in place of the column.
template <int D, bool LOC>
__device__ __forceinline__ void ct_apply32_body(int lb, int N, const long long* __restrict__ ctsptr, const int* __restrict__ ctcnt,
                                                    const float4* __restrict__ ctrec, const float* __restrict__ x, float* __restrict__ t,
                                                    const double* __restrict__ scal, int* __restrict__ flags, int cap,
                                                    const int* __restrict__ uniq, const int* __restrict__ ucount)
{
    extern __shared__ float xs_ct[];   // LOC: s of the lists' fluid rows by rank, a float4 (3-D) or float2 (2-D) each
    constexpr int XS = D == 3 ? kXs3 : 2;
    // the flags and the stop test once a block, by one thread (the test's FP64
    // quotient in every warp took a large share of the kernel's issue: FP64
    // runs at a small fraction of the FP32 rate on this part)
    __shared__ int go_s;
    if (threadIdx.x == 0) {   // the five loads issued together
        const int done = flags[kFlagDone], it = flags[kFlagIter];
        const double tol2 = scal[kSTol2], rr0 = scal[kSIn0], rrn = scal[kSIn];
        int go = !done;
        if (go) {
            const double rr = it == 0 ? rr0 : rrn;
            const bool bad = !(rr == rr);
            if (it >= cap || rr / rr0 < tol2 || bad) {
                go = 0;
                if (lb == 0) {
                    flags[kFlagDone] = 1;
                    if (bad) flags[kFlagBad] = 1;
                }
            }
        }
        go_s = go;
    }
    __syncthreads();
    if (!go_s) return;   // block-uniform
    const int k = lb * blockDim.x + threadIdx.x;
    int U = -1;
    if (LOC) {   // block-uniform
        U = ucount[lb];
        if (U >= 0) {
            const int* ul = uniq + (size_t)lb * kUMax;
#pragma unroll 4
            for (int a = threadIdx.x; a < U; a += blockDim.x) {
                const int j = ul[a];
#pragma unroll
                for (int d = 0; d < D; ++d) xs_ct[a * XS + d] = x[(size_t)j * D + d];
            }
            __syncthreads();
        }
    }
    if (k >= N) return;
    const int lane = k & 31;
    const float4* rp = ctrec + ctsptr[k >> 5] + lane;
    float s = 0.f;
    const int n = ctcnt[k];
    if (LOC && U >= 0) {   // by rank from shared memory
#pragma unroll 4
        for (int e = 0; e < n; ++e) {
            const float4 r = __ldcs(rp + (long long)e * 32);
            float xj[3];
            if (D == 3) {
                if (kXs3 == 4) {
                    const float4 v = reinterpret_cast<const float4*>(xs_ct)[__float_as_int(r.w)];
                    xj[0] = v.x; xj[1] = v.y; xj[2] = v.z;
                } else {
                    const float* v = xs_ct + (size_t)__float_as_int(r.w) * 3;
                    xj[0] = v[0]; xj[1] = v[1]; xj[2] = v[2];
                }
            } else {
                const float2 v = reinterpret_cast<const float2*>(xs_ct)[__float_as_int(r.w)];
                xj[0] = v.x; xj[1] = v.y; xj[2] = 0.f;
            }
            s += r.x * xj[0];
            s += r.y * xj[1];
            if (D == 3) s += r.z * xj[2];
        }
    } else {   // by column
#pragma unroll 4
        for (int e = 0; e < n; ++e) {
            const float4 r = __ldcs(rp + (long long)e * 32);
            const float* xj = x + (size_t)__float_as_int(r.w) * D;
            s += r.x * xj[0];
            s += r.y * xj[1];
            if (D == 3) s += r.z * xj[2];
        }
    }
    t[k] = s;
}

template <int D, bool LOC>
__global__ void __launch_bounds__(MPH_CT_BLOCK) k_ct_apply32(int N, const long long* __restrict__ ctsptr, const int* __restrict__ ctcnt,
                                                    const float4* __restrict__ ctrec, const float* __restrict__ x, float* __restrict__ t,
                                                    const double* __restrict__ scal, int* __restrict__ flags, int cap,
                                                    const int* __restrict__ uniq, const int* __restrict__ ucount)
{
    ct_apply32_body<D, LOC>((int)blockIdx.x, N, ctsptr, ctcnt, ctrec, x, t, scal, flags, cap, uniq, ucount);
}

// C Lambda t over the row's P-neighbours: 16-byte records (lambda C, column)
template <int D>
__device__ __forceinline__ void p_part32(int i, int lane, const int* __restrict__ ncp, const long long* __restrict__ psptr,
                                         const float4* __restrict__ psrec, const float* __restrict__ t, float* yv)
{
    const float4* rp = psrec + psptr[i >> 5] + lane;
    const int np = ncp[i];
#pragma unroll 4
    for (int a = 0; a < np; ++a) {
        const float4 r = __ldcs(rp + (long long)a * 32);
        const float tk = t[__float_as_int(r.w)];
        yv[0] += r.x * tk;
        yv[1] += r.y * tk;
        if (D == 3) yv[2] += r.z * tk;
    }
}

// Slot records of the inner operator's viscous pairs, in the slot order of
// the sliced layout.  FP16 form (8 bytes a slot): g = sqrt(f) e in FP16,
// scaled per slice, in the first D halves and the neighbour's block-local
// index in the fourth.  Packed form (option pair_pack, 6 bytes a slot): g in
// one 32-bit word as signed fixed point in units of the slice's scale
// (bits 0-10 x, 11-21 y, 22-31 z in units of twice the scale: relative
// rounding about 2^-11 of the slice's largest component) and the block-local
// index in a separate 2-byte stream.  A record is carried as a uint2: the
// FP16 record, or (g word, index).
template <bool PACK, bool LOC>
__device__ __forceinline__ uint2 load_slot(const uint2* __restrict__ r16, const unsigned* __restrict__ r32,
                                           const unsigned short* __restrict__ l16, long long e)
{
    if (PACK) return make_uint2(__ldcs(r32 + e), LOC ? (unsigned)__ldcs(l16 + e) : 0u);
    return __ldcs(r16 + e);
}

// g in units of the slice's scale, and the block-local index
template <int D, bool PACK>
__device__ __forceinline__ int decode_slot(uint2 r, float* g)
{
    if (PACK) {
        g[0] = (float)(((int)(r.x << 21)) >> 21);
        g[1] = (float)(((int)(r.x << 10)) >> 21);
        g[2] = D == 3 ? 2.f * (float)(((int)r.x) >> 22) : 0.f;
        return (int)r.y;
    }
    g[0] = __half2float(__ushort_as_half((unsigned short)(r.x & 0xffffu)));
    g[1] = __half2float(__ushort_as_half((unsigned short)(r.x >> 16)));
    g[2] = D == 3 ? __half2float(__ushort_as_half((unsigned short)(r.y & 0xffffu))) : 0.f;
    return (int)(r.y >> 16);
}

// The viscous part of row i in FP32 from the slot records:
// yv = S_wall x_i + sum_{fluid j} g (g . (x_i - x_j)).  LOC: the neighbour's
// x from the block's shared-memory copy by its block-local index, else
// gathered by column.  The record stream is software-pipelined: the next
// kPairUnroll records (and columns) are loaded while the current ones are
// applied; pre holds the first ones, loaded by the caller.
template <int D, bool PACK, bool LOC>
__device__ __forceinline__ void visc_row32(int i, int lane, const float* xi, const float* __restrict__ sdiag,
                                           const int* __restrict__ nfc, const long long* __restrict__ sptr,
                                           const int* __restrict__ acol, const uint2* __restrict__ r16,
                                           const unsigned* __restrict__ r32, const unsigned short* __restrict__ l16,
                                           const float* __restrict__ pscale, const float* __restrict__ x, float* yv,
                                           const float* xs, const uint2* pre)
{
    const float4 s0 = *reinterpret_cast<const float4*>(sdiag + (size_t)i * 8);
    const float4 s1 = *reinterpret_cast<const float4*>(sdiag + (size_t)i * 8 + 4);
    yv[0] = s0.x * xi[0] + s0.y * xi[1] + s0.z * xi[2];
    yv[1] = s0.y * xi[0] + s0.w * xi[1] + s1.x * xi[2];
    yv[2] = s0.z * xi[0] + s1.x * xi[1] + s1.y * xi[2];
    // whole slices (a multiple of R slots; padding records are zero and
    // point at column 0 / rank 0, so they add exact zeros): no per-slot tests
    const long long sb = sptr[i >> 5];
    const int w = (int)((sptr[(i >> 5) + 1] - sb) >> 5);
    const long long base = sb + lane;
    const int* cp = acol + base;
    float ys[3] = {0.f, 0.f, 0.f};
    constexpr int R = kPairUnroll;
    uint2 cur[R];
    int ccur[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
        cur[u] = pre[u];
        ccur[u] = (!LOC && u < w) ? __ldcs(cp + (long long)u * 32) : 0;
    }
    for (int k0 = 0; k0 < w; k0 += R) {
        uint2 nxt[R];
        int cnxt[R];
        if (k0 + R < w) {   // warp-uniform
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const long long e = base + (long long)(k0 + R + u) * 32;
                nxt[u] = load_slot<PACK, LOC>(r16, r32, l16, e);
                cnxt[u] = !LOC ? __ldcs(cp + (e - base)) : 0;
            }
        } else {
#pragma unroll
            for (int u = 0; u < R; ++u) {
                nxt[u] = make_uint2(0u, 0u);
                cnxt[u] = 0;
            }
        }
#pragma unroll
        for (int u = 0; u < R; ++u) {
            float g[3];
            const int lj = decode_slot<D, PACK>(cur[u], g);
            float xj[3];
            if (LOC) {   // staged s: a float4 (3-D) or float2 (2-D) per neighbour
                if (D == 3) {
                    if (kXs3 == 4) {
                        const float4 v = reinterpret_cast<const float4*>(xs)[lj];
                        xj[0] = v.x; xj[1] = v.y; xj[2] = v.z;
                    } else {
                        const float* v = xs + (size_t)lj * 3;
                        xj[0] = v[0]; xj[1] = v[1]; xj[2] = v[2];
                    }
                } else {
                    const float2 v = reinterpret_cast<const float2*>(xs)[lj];
                    xj[0] = v.x; xj[1] = v.y; xj[2] = 0.f;
                }
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d) xj[d] = x[(size_t)ccur[u] * D + d];
            }
            float gx = 0.f;
#pragma unroll
            for (int d = 0; d < D; ++d) gx += g[d] * (xi[d] - xj[d]);
#pragma unroll
            for (int d = 0; d < D; ++d) ys[d] += gx * g[d];
        }
#pragma unroll
        for (int u = 0; u < R; ++u) {
            cur[u] = nxt[u];
            ccur[u] = cnxt[u];
        }
    }
    const float s2 = pscale[i >> 5] * pscale[i >> 5];
#pragma unroll
    for (int d = 0; d < 3; ++d) yv[d] += ys[d] * s2;
}

// PPART false: the viscous pairs and the diagonal only, y written without
// the dot; k_ppart32 adds lambda C t and forms the dot (the split operator,
// whose transposed apply runs beside this kernel)
template <int D, bool LOC, bool PACK, bool PPART>
__device__ __forceinline__ void visc_pen32_body(int lb, int nb, int Nf, const int* __restrict__ nfc, const long long* __restrict__ sptr, const int* __restrict__ acol,
             const unsigned short* __restrict__ grec, const unsigned* __restrict__ grec32, const unsigned short* __restrict__ lcol,
             const float* __restrict__ pscale, const float* __restrict__ sdiag,
             const int* __restrict__ ncp, const long long* __restrict__ psptr, const float4* __restrict__ psrec,
             const float* __restrict__ t, const float* __restrict__ x, float* __restrict__ y, double* __restrict__ scal,
             const int* __restrict__ flags, double* __restrict__ partials, unsigned* __restrict__ counter,
             const int* __restrict__ uniq, const int* __restrict__ ucount)
{
    // LOC: s of the block's distinct fluid neighbours by block-local index,
    // a float4 (3-D) or float2 (2-D) each
    extern __shared__ float xs_loc[];
    constexpr int XS = D == 3 ? kXs3 : 2;
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    const int i = lb * blockDim.x + threadIdx.x;
    const uint2* r16 = reinterpret_cast<const uint2*>(grec);
    uint2 pre[kPairUnroll];   // the row's first slot records, in flight while s is staged
    {
        const long long s0 = i < Nf ? sptr[i >> 5] : 0;
        const int w0 = i < Nf ? (int)((sptr[(i >> 5) + 1] - s0) >> 5) : 0;
#pragma unroll
        for (int u = 0; u < kPairUnroll; ++u)
            pre[u] = u < w0 ? load_slot<PACK, LOC>(r16, grec32, lcol, s0 + (i & 31) + (long long)u * 32) : make_uint2(0u, 0u);
    }
    int U = -1;
    if (LOC) {   // stage s of the block's distinct neighbours once (block-uniform)
        U = ucount[lb];
        if (U >= 0) {
            const int* ul = uniq + (size_t)lb * kUMax;
#pragma unroll 4
            for (int k = threadIdx.x; k < U; k += blockDim.x) {
                const int j = ul[k];
#pragma unroll
                for (int d = 0; d < D; ++d) xs_loc[k * XS + d] = x[(size_t)j * D + d];
            }
            __syncthreads();
        }
    }
    float acc = 0.f;
    if (i < Nf) {
        const int lane = i & 31;
        float xi[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) xi[d] = x[(size_t)i * D + d];
        float yv[3];
        if (LOC && U >= 0)
            visc_row32<D, PACK, true>(i, lane, xi, sdiag, nfc, sptr, acol, r16, grec32, lcol, pscale, x, yv, xs_loc, pre);
        else
            visc_row32<D, PACK, false>(i, lane, xi, sdiag, nfc, sptr, acol, r16, grec32, lcol, pscale, x, yv, nullptr, pre);
        const float in32 = sdiag[(size_t)i * 8 + 6];
#pragma unroll
        for (int d = 0; d < D; ++d) yv[d] += in32 * xi[d];
        if (PPART) p_part32<D>(i, lane, ncp, psptr, psrec, t, yv);
        float dot = 0.f;   // the row's D terms and a warp's rows in FP32, the warps in FP64
#pragma unroll
        for (int d = 0; d < D; ++d) {
            y[(size_t)i * D + d] = yv[d];
            dot += xi[d] * yv[d];
        }
        acc = dot;
    }
    if (PPART) reduce_finalize(acc, partials, counter, scal + rho32_slot_f(it), lb, nb);
}

template <int D, bool LOC, bool PACK, bool PPART>
__global__ void __launch_bounds__(MPH_PAIR_BLOCK, 2)   // two 512-row blocks an SM
k_visc_pen32(int Nf, const int* __restrict__ nfc, const long long* __restrict__ sptr, const int* __restrict__ acol,
             const unsigned short* __restrict__ grec, const unsigned* __restrict__ grec32, const unsigned short* __restrict__ lcol,
             const float* __restrict__ pscale, const float* __restrict__ sdiag,
             const int* __restrict__ ncp, const long long* __restrict__ psptr, const float4* __restrict__ psrec,
             const float* __restrict__ t, const float* __restrict__ x, float* __restrict__ y, double* __restrict__ scal,
             const int* __restrict__ flags, double* __restrict__ partials, unsigned* __restrict__ counter,
             const int* __restrict__ uniq, const int* __restrict__ ucount)
{
    visc_pen32_body<D, LOC, PACK, PPART>((int)blockIdx.x, (int)gridDim.x, Nf, nfc, sptr, acol, grec, grec32, lcol, pscale, sdiag, ncp,
                                         psptr, psrec, t, x, y, scal, flags, partials, counter, uniq, ucount);
}

// The second half of the split operator: y_i += sum_k lambda_k C_ik t_k, then
// (s, y) into the iteration's rho slot (after the transposed apply and the
// viscous kernel; the same arithmetic as the fused kernel's P-part)
template <int D>
__global__ void __launch_bounds__(256) k_ppart32(int Nf, const int* __restrict__ ncp, const long long* __restrict__ psptr,
                                                 const float4* __restrict__ psrec, const float* __restrict__ t,
                                                 const float* __restrict__ x, float* __restrict__ y, double* __restrict__ scal,
                                                 const int* __restrict__ flags, double* __restrict__ partials,
                                                 unsigned* __restrict__ counter)
{
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.f;
    if (i < Nf) {
        float yv[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) yv[d] = y[(size_t)i * D + d];
        p_part32<D>(i, i & 31, ncp, psptr, psrec, t, yv);
        float dot = 0.f;   // the row's D terms and a warp's rows in FP32, the warps in FP64
#pragma unroll
        for (int d = 0; d < D; ++d) {
            y[(size_t)i * D + d] = yv[d];
            dot += x[(size_t)i * D + d] * yv[d];
        }
        acc = dot;
    }
    reduce_finalize(acc, partials, counter, scal + rho32_slot_f(it));
}

// The pair-term operator with its pair terms evaluated per slot (option
// pair_recompute, the default): a fluid slot reads only its neighbour's
// block-local index (2 bytes) or, in a row block that gathers by column, its
// column; the neighbour's FP32 position and type (pt32) and its s come from
// the block's shared-memory copy, or by column.  Per pair, as k_pair_terms:
// q = p_j - p_i from the high parts of the two-float positions,
// w = -dwvdr(|q|, RadiusV) (main.cpp:301, 2276) and f = visc mu_ij w / |q|
// (main.cpp:2285-2289), and the term g (g . (s_i - s_j)) with g = sqrt(f) e
// is f / |q|^2 q (q . (s_i - s_j)).  q_ji = -q_ij exactly, so the operator is
// exactly symmetric; its pair coefficients carry the FP32 rounding of the
// separation (about 1e-5 of it at the closest pairs of a unit-sized domain)
// instead of the FP16 storage of the slot records (2^-11).  WRAP: the minimum
// image of each separation, as the neighbour search (only when a pair of the
// step is a periodic image).
template <int D, bool LOC, bool WRAP>
__device__ __forceinline__ void visc_rc_loop(const DevParams& P, int n, const unsigned short* __restrict__ lp,
                                             const int* __restrict__ cp, const float4* pts, const float* xs,
                                             const float* pi, const float* xi, float vm0, float vm1, float* ys)
{
#pragma unroll (kPairUnroll)
    for (int k = 0; k < n; ++k) {
        const int j = LOC ? (int)__ldcs(lp + (long long)k * 32) : __ldcs(cp + (long long)k * 32);
        const float4 pj = pts[j];
        const float* xj = xs + (size_t)j * D;
        float q[3] = {pj.x - pi[0], pj.y - pi[1], D == 3 ? pj.z - pi[2] : 0.f};
        if (WRAP) {
#pragma unroll
            for (int d = 0; d < D; ++d)
                q[d] = q[d] > P.hw32[d] ? q[d] - P.w32[d] : (q[d] < -P.hw32[d] ? q[d] + P.w32[d] : q[d]);
        }
        const float r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        const bool in = r2 > 0.f && r2 < P.rV2_32;
        const float inv = rsqrtf(in ? r2 : 1.f);
        const float wd = P.wdA32 * (1.f - (r2 * inv) * P.inv_rv32);
        const float vm = __float_as_int(pj.w) == 1 ? vm1 : vm0;   // fluid types 0 and 1
        const float cf = in ? vm * wd * (inv * inv * inv) : 0.f;
        float dot = 0.f;
#pragma unroll
        for (int d = 0; d < D; ++d) dot += q[d] * (xi[d] - xj[d]);
        const float cd = cf * dot;
#pragma unroll
        for (int d = 0; d < D; ++d) ys[d] += cd * q[d];
    }
}

template <int D, bool LOC>
__global__ void __launch_bounds__(MPH_PAIR_BLOCK, MPH_PAIR_MINB)
k_visc_rc32(DevParams P, int Nf, const float4* __restrict__ pt32, const int* __restrict__ nfc, const long long* __restrict__ sptr,
            const int* __restrict__ acol, const unsigned short* __restrict__ lcol, const float* __restrict__ sdiag,
            const int* __restrict__ ncp, const long long* __restrict__ psptr, const float4* __restrict__ psrec,
            const float* __restrict__ t, const float* __restrict__ x, float* __restrict__ y, double* __restrict__ scal,
            const int* __restrict__ flags, double* __restrict__ partials, unsigned* __restrict__ counter,
            const int* __restrict__ uniq, const int* __restrict__ ucount, int ucap, const int* __restrict__ wrap)
{
    // LOC: the position and type of the block's distinct fluid neighbours
    // (ucap records), then their s, by block-local index
    extern __shared__ float4 rc_smem[];
    if (flags[kFlagDone]) return;
    const int it = flags[kFlagIter];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float4* ps = rc_smem;
    float* xs = reinterpret_cast<float*>(rc_smem + ucap);
    int U = -1;
    if (LOC) {   // block-uniform
        U = ucount[blockIdx.x];
        if (U >= 0) {
            const int* ul = uniq + (size_t)blockIdx.x * kUMax;
#pragma unroll 4
            for (int k = threadIdx.x; k < U; k += blockDim.x) {
                const int j = ul[k];
                ps[k] = pt32[j];
#pragma unroll
                for (int d = 0; d < D; ++d) xs[k * D + d] = x[(size_t)j * D + d];
            }
            __syncthreads();
        }
    }
    const bool wr = *wrap != 0;
    float acc = 0.f;
    if (i < Nf) {
        const int lane = i & 31;
        float xi[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) xi[d] = x[(size_t)i * D + d];
        const float4 p4 = pt32[i];
        const float pi[3] = {p4.x, p4.y, p4.z};
        const int ti = __float_as_int(p4.w);
        const float vm0 = P.vm32[ti][0], vm1 = P.vm32[ti][1];
        // wall part of the viscous diagonal block and the inertia
        const float4 s0 = *reinterpret_cast<const float4*>(sdiag + (size_t)i * 8);
        const float4 s1 = *reinterpret_cast<const float4*>(sdiag + (size_t)i * 8 + 4);
        float yv[3];
        yv[0] = s0.x * xi[0] + s0.y * xi[1] + s0.z * xi[2];
        yv[1] = s0.y * xi[0] + s0.w * xi[1] + s1.x * xi[2];
        yv[2] = s0.z * xi[0] + s1.x * xi[1] + s1.y * xi[2];
        const float in32 = s1.z;
#pragma unroll
        for (int d = 0; d < D; ++d) yv[d] += in32 * xi[d];
        const long long base = sptr[i >> 5] + lane;
        const int n = nfc[i];
        float ys[3] = {0.f, 0.f, 0.f};
        if (LOC && U >= 0) {
            if (wr) visc_rc_loop<D, true, true>(P, n, lcol + base, nullptr, ps, xs, pi, xi, vm0, vm1, ys);
            else visc_rc_loop<D, true, false>(P, n, lcol + base, nullptr, ps, xs, pi, xi, vm0, vm1, ys);
        } else {
            if (wr) visc_rc_loop<D, false, true>(P, n, nullptr, acol + base, pt32, x, pi, xi, vm0, vm1, ys);
            else visc_rc_loop<D, false, false>(P, n, nullptr, acol + base, pt32, x, pi, xi, vm0, vm1, ys);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) yv[d] += ys[d];
        {   // C Lambda t over the row's P-neighbours: 16-byte records (lambda C, column)
            const float4* rp = psrec + psptr[i >> 5] + lane;
            const int np = ncp[i];
#pragma unroll 4
            for (int a = 0; a < np; ++a) {
                const float4 r = __ldcs(rp + (long long)a * 32);
                const float tk = t[__float_as_int(r.w)];
                yv[0] += r.x * tk;
                yv[1] += r.y * tk;
                if (D == 3) yv[2] += r.z * tk;
            }
        }
        float dot = 0.f;   // the row's D terms and a warp's rows in FP32, the warps in FP64
#pragma unroll
        for (int d = 0; d < D; ++d) {
            y[(size_t)i * D + d] = yv[d];
            dot += xi[d] * yv[d];
        }
        acc = dot;
    }
    reduce_finalize(acc, partials, counter, scal + rho32_slot_f(it));
}

// Rows of a CSR list (count, row pointer, column, D FP32 values an entry) ->
// the sliced layout, one CTA per slice of 32 rows: chunks of kLtsK entries of
// the 32 rows are read row by row (coalesced) into shared memory and written
// slice-wise (coalesced), padding slots as zeros.  PAIRS: the values are the
// pair terms (e, f), stored as g = sqrt(f) e in FP32 and, for the inner
// operator, in FP16 scaled per slice (g / sigma, sigma = the slice's largest
// |g| component / 2^15: relative rounding 2^-11, no overflow) into the first
// D halves of the slot records (4 halves a slot).

template <int D, bool PAIRS>
__global__ void __launch_bounds__(256) k_list_to_slices(int rows, const long long* __restrict__ sptr, const int* __restrict__ cnt,
                                                        const long long* __restrict__ rptr, const int* __restrict__ cols,
                                                        const float4* __restrict__ pe32, const float* __restrict__ v32,
                                                        int* __restrict__ scol, float* __restrict__ sval,
                                                        unsigned short* __restrict__ sval16, float* __restrict__ sscale,
                                                        unsigned* __restrict__ sval32)
{
    constexpr int W = kLtsK * D + 1;   // odd row stride: no bank conflicts
    __shared__ float tile[32 * W];
    __shared__ int ctile[32 * (kLtsK + 1)];
    __shared__ int rn[32];
    __shared__ long long rb[32];
    const int sl = blockIdx.x;
    if (threadIdx.x < 32) {
        const int i = sl * 32 + threadIdx.x;
        rn[threadIdx.x] = i < rows ? cnt[i] : 0;
        rb[threadIdx.x] = i < rows ? rptr[i] : 0;
    }
    __syncthreads();
    const long long sb = sptr[sl];
    const int w = (int)((sptr[sl + 1] - sb) / 32);   // entries per row of the slice
    float inv16 = 0.f;
    if (PAIRS && (sval16 || sval32)) {
        // the slice's largest |g| component (from k_pair_terms, as bits) maps
        // to 2^15 (FP16 records) or to 1023 (packed records)
        const float m = __uint_as_float(reinterpret_cast<const unsigned*>(sscale)[sl]);
        const float sigma = m / (sval32 ? 1023.f : 32768.f);
        inv16 = m > 0.f ? 1.f / sigma : 0.f;
        __syncthreads();   // every thread has read the maximum before it is replaced by the scale
        if (threadIdx.x == 0) sscale[sl] = sigma;
    }
    for (int k0 = 0; k0 < w; k0 += kLtsK) {
        const int kc = min(kLtsK, w - k0);
        for (int t = threadIdx.x; t < 32 * kLtsK; t += blockDim.x) {
            const int r = t / kLtsK, kl = t % kLtsK;
            float v[3] = {0.f, 0.f, 0.f};
            int col = 0;
            if (kl < kc && k0 + kl < rn[r]) {
                const long long e = rb[r] + k0 + kl;
                col = cols[e];
                if (PAIRS) {
                    const float4 pv = pe32[e];
                    const float sf = sqrtf(pv.w);
                    v[0] = sf * pv.x;
                    v[1] = sf * pv.y;
                    v[2] = sf * pv.z;
                } else {
#pragma unroll
                    for (int d = 0; d < D; ++d) v[d] = v32[e * D + d];
                }
            }
#pragma unroll
            for (int d = 0; d < D; ++d) tile[r * W + kl * D + d] = v[d];
            ctile[r * (kLtsK + 1) + kl] = col;
        }
        __syncthreads();
        if (PAIRS) {
            for (int o = threadIdx.x; o < kc * D * 32; o += blockDim.x) {
                const int ln = o & 31, ec = o >> 5;   // ec = k_local * D + component
                sval[sb * D + (long long)k0 * D * 32 + o] = tile[ln * W + ec];
            }
        } else {   // 16-byte records: D values (zero-padded), the column
            for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
                const int ln = o & 31, kl = o >> 5;
                const float* v = tile + ln * W + kl * D;
                reinterpret_cast<float4*>(sval)[sb + (long long)(k0 + kl) * 32 + ln] =
                    make_float4(v[0], v[1], D == 3 ? v[2] : 0.f, __int_as_float(ctile[ln * (kLtsK + 1) + kl]));
            }
        }
        if (PAIRS && sval32) {   // packed g words (the indices are a separate stream)
            for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
                const int ln = o & 31, kl = o >> 5;
                int q[3] = {0, 0, 0};
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const int lim = d == 2 ? 511 : 1023;
                    const float v = tile[ln * W + kl * D + d] * inv16 * (d == 2 ? 0.5f : 1.f);
                    q[d] = max(-lim, min(lim, __float2int_rn(v)));
                }
                sval32[sb + (long long)(k0 + kl) * 32 + ln] =
                    ((unsigned)q[0] & 0x7ffu) | (((unsigned)q[1] & 0x7ffu) << 11) | (((unsigned)q[2] & 0x3ffu) << 22);
            }
        }
        if (PAIRS && sval16) {   // whole slot records (the index half is written later)
            for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
                const int ln = o & 31, kl = o >> 5;
                unsigned h[3] = {0u, 0u, 0u};
#pragma unroll
                for (int d = 0; d < D; ++d) h[d] = __half_as_ushort(__float2half_rn(tile[ln * W + kl * D + d] * inv16));
                reinterpret_cast<uint2*>(sval16)[sb + (long long)(k0 + kl) * 32 + ln] = make_uint2(h[0] | (h[1] << 16), h[2]);
            }
        }
        if (PAIRS)
            for (int o = threadIdx.x; o < kc * 32; o += blockDim.x) {
                const int ln = o & 31, kl = o >> 5;
                scol[sb + (long long)(k0 + kl) * 32 + ln] = ctile[ln * (kLtsK + 1) + kl];
            }
        __syncthreads();
    }
}

// The viscous part of row i of A x for the FP64 outer residual on the pair
// path.  The wall part of the diagonal block (FP64 sums of FP64 wall-slot
// terms) multiplies x_i in FP64; the fluid pairs g (g . (x_i - x_j)) take the
// FP32 g of the sliced pair terms and the difference of the two-float x
// (hi + lo, x to about 2^-48 relative), so x enters the viscous part without
// FP32 rounding: only the pair coefficients are FP32, which bounds the
// operator's perturbation by about 1e-7 of its viscous part.  The pair terms
// are summed in FP32 per row (they are differences, small against the row's
// inertia) and added in FP64.
template <int D>
__device__ __forceinline__ void visc_row_resid(int i, int lane, const double* __restrict__ sdiag64,
                                               const int* __restrict__ nfc, const long long* __restrict__ sptr,
                                               const int* __restrict__ acol, const float* __restrict__ pes,
                                               const float* __restrict__ xh, const float* __restrict__ xl,
                                               const double* __restrict__ x, double* y)
{
    double xi[3] = {0.0, 0.0, 0.0};
    float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d) {
        xi[d] = x[(size_t)i * D + d];
        hi[d] = xh[(size_t)i * D + d];
        lo[d] = xl[(size_t)i * D + d];
    }
    const double2* sp = reinterpret_cast<const double2*>(sdiag64 + (size_t)i * 8);
    const double2 a = sp[0], b = sp[1], e = sp[2];   // (xx, xy), (xz, yy), (yz, zz)
    y[0] = a.x * xi[0] + a.y * xi[1] + b.x * xi[2];
    y[1] = a.y * xi[0] + b.y * xi[1] + e.x * xi[2];
    y[2] = b.x * xi[0] + e.x * xi[1] + e.y * xi[2];
    const long long base = sptr[i >> 5];
    const int* cp = acol + base + lane;
    const long long vo = base * D + lane;
    const int n = nfc[i];
    float ys[3] = {0.f, 0.f, 0.f};
#pragma unroll 4
    for (int k = 0; k < n; ++k) {
        float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) g[d] = __ldcs(pes + vo + ((long long)k * D + d) * 32);
        const size_t j = (size_t)__ldcs(cp + (long long)k * 32) * D;
        float gx = 0.f;
#pragma unroll
        for (int d = 0; d < D; ++d) gx += g[d] * ((hi[d] - xh[j + d]) + (lo[d] - xl[j + d]));
#pragma unroll
        for (int d = 0; d < D; ++d) ys[d] += gx * g[d];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) y[d] += (double)ys[d];
}

// x in two floats: hi = FP32 rounding of x, lo = FP32 rounding of x - hi
__global__ void k_split_f32(long long n, const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double v = x[k];
    const float h = (float)v;
    hi[k] = h;
    lo[k] = (float)(v - (double)h);
}

// r = b - A x on the pair-term path, one thread per row: the viscous part as
// visc_row_resid, inertia and C Lambda t (t = C^T x) in FP64; (r, r) -> *out.
template <int D>
__global__ void __launch_bounds__(MPH_PAIR_BLOCK)
k_resid_pairs(DevParams P, int Nf, const int* __restrict__ type, const int* __restrict__ nfc, const long long* __restrict__ sptr,
              const int* __restrict__ acol, const float* __restrict__ pes, const double* __restrict__ sdiag64,
              const int* __restrict__ ncp, const long long* __restrict__ nptrP, const int* __restrict__ nindP,
              const double* __restrict__ cval, const double* __restrict__ t, const double* __restrict__ x,
              const float* __restrict__ x32, const double* __restrict__ b, double* __restrict__ r,
              double* __restrict__ partials, unsigned* __restrict__ counter, double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (i < Nf) {
        double y[3];
        visc_row_resid<D>(i, i & 31, sdiag64, nfc, sptr, acol, pes, x32, x32 + (size_t)Nf * D, x, y);
        const long long pb = nptrP[i];
        const int np = ncp[i];
        for (int a = 0; a < np; ++a) {
            const int k = nindP[pb + a];
            const double lt = t[k];   // lambda_k t_k
#pragma unroll
            for (int d = 0; d < D; ++d) y[d] += cval[(pb + a) * D + d] * lt;
        }
        const double inert = P.inert64[type[i]];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const size_t k = (size_t)i * D + d;
            const double rv = b[k] - (inert * x[k] + y[d]);
            r[k] = rv;
            acc += rv * rv;
        }
    }
    reduce_finalize(acc, partials, counter, out);
}

template <int D, bool PACK, bool PPART>
static void visc_pen_launch(mph_case* c, unsigned gv, const float* x, float* y, unsigned* counter)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    if (c->loc_smem)
        k_visc_pen32<D, true, PACK, PPART><<<gv, c->pair_block, c->loc_smem, c->stream>>>(P.Nf, d.nfc, d.sptr, d.acol, d.grec16, d.grec32,
            d.lcol16, d.pscale, d.sdiag32, d.ncp, d.psptr, (const float4*)d.psval, d.tct32, x, y, d.scal, d.flags, d.partials, counter,
            d.uniq, d.ucount);
    else
        k_visc_pen32<D, false, PACK, PPART><<<gv, c->pair_block, 0, c->stream>>>(P.Nf, d.nfc, d.sptr, d.acol, d.grec16, d.grec32,
            d.lcol16, d.pscale, d.sdiag32, d.ncp, d.psptr, (const float4*)d.psval, d.tct32, x, y, d.scal, d.flags, d.partials, counter,
            nullptr, nullptr);
    MPH_COUNT_LAUNCH();
}

template <int D>
static void ct_launch(mph_case* c, cudaStream_t st, const float* x, int cap)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    const unsigned gt = grid_for(P.N, c->ct_block);
    if (c->loc_ct_smem)
        k_ct_apply32<D, true><<<gt, c->ct_block, c->loc_ct_smem, st>>>(P.N, d.ctsptr, d.ct_cnt, (const float4*)d.ctsval, x, d.tct32,
                                                                      d.scal, d.flags, cap, d.ctuniq, d.ctucount);
    else
        k_ct_apply32<D, false><<<gt, c->ct_block, 0, st>>>(P.N, d.ctsptr, d.ct_cnt, (const float4*)d.ctsval, x, d.tct32, d.scal,
                                                          d.flags, cap, nullptr, nullptr);
    MPH_COUNT_LAUNCH();
}

// The inner operator y = A32 x (and (x, y) into the iteration's rho slot).
// Split form (option split_apply, off by default; the packed and FP16
// records): the transposed apply t = C^T x runs on a side stream beside the
// viscous kernel, which does not read t; k_ppart32 then adds lambda C t.  In
// a captured graph the fork and the join are graph edges.  Measured slower
// on the config-1 workload (0.409 against 0.404 ms an application): the
// viscous kernel keeps every SM busy, so the two do not overlap, and the
// third kernel costs more than the fork saves.
template <int D>
static void apply32(mph_case* c, const float* x, float* y, int cap)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    unsigned* counter = (unsigned*)(d.flags + kFlagCounter);
    const unsigned gv = grid_for(P.Nf, c->pair_block);
    if (c->split_apply && !c->pair_recompute && c->fork_stream) {
        cudaEventRecord(c->ev_fork, c->stream);
        cudaStreamWaitEvent(c->fork_stream, c->ev_fork, 0);
        ct_launch<D>(c, c->fork_stream, x, cap);
        cudaEventRecord(c->ev_join, c->fork_stream);
        if (c->pair_pack) visc_pen_launch<D, true, false>(c, gv, x, y, counter);
        else visc_pen_launch<D, false, false>(c, gv, x, y, counter);
        cudaStreamWaitEvent(c->stream, c->ev_join, 0);
        { k_ppart32<D><<<grid_for(P.Nf, 256), 256, 0, c->stream>>>(P.Nf, d.ncp, d.psptr, (const float4*)d.psval, d.tct32, x, y, d.scal,
                                                                   d.flags, d.partials, counter); MPH_COUNT_LAUNCH(); }
        return;
    }
    ct_launch<D>(c, c->stream, x, cap);
    if (c->pair_recompute) {
        if (c->loc_smem)
            k_visc_rc32<D, true><<<gv, c->pair_block, c->loc_smem, c->stream>>>(P, P.Nf, d.pt32, d.nfc, d.sptr, d.acol, d.lcol16,
                d.sdiag32, d.ncp, d.psptr, (const float4*)d.psval, d.tct32, x, y, d.scal, d.flags, d.partials, counter, d.uniq,
                d.ucount, c->loc_cap, d.wrap32);
        else
            k_visc_rc32<D, false><<<gv, c->pair_block, 0, c->stream>>>(P, P.Nf, d.pt32, d.nfc, d.sptr, d.acol, nullptr,
                d.sdiag32, d.ncp, d.psptr, (const float4*)d.psval, d.tct32, x, y, d.scal, d.flags, d.partials, counter, nullptr,
                nullptr, 0, d.wrap32);
        MPH_COUNT_LAUNCH();
    } else if (c->pair_pack)
        visc_pen_launch<D, true, true>(c, gv, x, y, counter);
    else
        visc_pen_launch<D, false, true>(c, gv, x, y, counter);
}

void launch_apply32(mph_case* c, const float* x, float* y, int cap)
{
    if (c->dim == 2) apply32<2>(c, x, y, cap);
    else apply32<3>(c, x, y, cap);
}

// ---- the operator over the cases of a batch ------------------------------------------
template <int D>
__global__ void __launch_bounds__(MPH_CT_BLOCK) k_batch_ct32(const BatchCase* __restrict__ cs, const int* __restrict__ b0, int nc)
{
    const int c = batch_case_of(b0, nc, (int)blockIdx.x);
    const BatchCase& B = cs[c];
    const int lb = (int)blockIdx.x - b0[c];
    if (B.ct_loc)
        ct_apply32_body<D, true>(lb, B.N, B.ctsptr, B.ct_cnt, B.ctsval, B.s32, B.tct32, B.scal, B.flags, B.cap, B.ctuniq, B.ctucount);
    else
        ct_apply32_body<D, false>(lb, B.N, B.ctsptr, B.ct_cnt, B.ctsval, B.s32, B.tct32, B.scal, B.flags, B.cap, nullptr, nullptr);
}

template <int D, bool PACK>
__global__ void __launch_bounds__(MPH_PAIR_BLOCK, 2) k_batch_visc32(const BatchCase* __restrict__ cs, const int* __restrict__ b0, int nc)
{
    const int c = batch_case_of(b0, nc, (int)blockIdx.x);
    const BatchCase& B = cs[c];
    const int lb = (int)blockIdx.x - b0[c];
    if (B.vp_loc)
        visc_pen32_body<D, true, PACK, true>(lb, B.vp_nb, B.Nf, B.nfc, B.sptr, B.acol, B.grec16, B.grec32, B.lcol16, B.pscale, B.sdiag32,
                                             B.ncp, B.psptr, B.psval, B.tct32, B.s32, B.y32, B.scal, B.flags, B.partials, B.counter,
                                             B.uniq, B.ucount);
    else
        visc_pen32_body<D, false, PACK, true>(lb, B.vp_nb, B.Nf, B.nfc, B.sptr, B.acol, B.grec16, B.grec32, B.lcol16, B.pscale,
                                              B.sdiag32, B.ncp, B.psptr, B.psval, B.tct32, B.s32, B.y32, B.scal, B.flags, B.partials,
                                              B.counter, nullptr, nullptr);
}

// the transposed apply and the viscous kernel of one batched CR iteration
// (ct_b0 / vp_b0: their block starts; shared memory: the batch's largest)
void launch_batch_operator(const BatchCase* cs, const int* ct_b0, const int* vp_b0, int nc, int dim, bool pack, int pair_block,
                           int ct_block, int vp_smem, int ct_smem, int ct_blocks, int vp_blocks, cudaStream_t st)
{
    static std::once_flag once;
    std::call_once(once, [] {   // fixed maxima (host threads of other batches would race on per-launch values)
        cudaFuncSetAttribute(k_batch_ct32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float));
        cudaFuncSetAttribute(k_batch_ct32<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float));
        cudaFuncSetAttribute(k_batch_visc32<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float));
        cudaFuncSetAttribute(k_batch_visc32<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float));
        cudaFuncSetAttribute(k_batch_visc32<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float));
        cudaFuncSetAttribute(k_batch_visc32<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float));
    });
    if (ct_blocks > 0) {
        if (dim == 2) k_batch_ct32<2><<<ct_blocks, ct_block, ct_smem, st>>>(cs, ct_b0, nc);
        else k_batch_ct32<3><<<ct_blocks, ct_block, ct_smem, st>>>(cs, ct_b0, nc);
        MPH_COUNT_LAUNCH();
    }
    if (vp_blocks > 0) {
        if (dim == 2) {
            if (pack) k_batch_visc32<2, true><<<vp_blocks, pair_block, vp_smem, st>>>(cs, vp_b0, nc);
            else k_batch_visc32<2, false><<<vp_blocks, pair_block, vp_smem, st>>>(cs, vp_b0, nc);
        } else {
            if (pack) k_batch_visc32<3, true><<<vp_blocks, pair_block, vp_smem, st>>>(cs, vp_b0, nc);
            else k_batch_visc32<3, false><<<vp_blocks, pair_block, vp_smem, st>>>(cs, vp_b0, nc);
        }
        MPH_COUNT_LAUNCH();
    }
}

// ---- level-0 multigrid stencils and D^-1 on the pair-term path --------------------
// The Galerkin level-0 matrix (calculateMultiGridCsrA, main.cpp:3245) sums
// the blocks of A of a cell's fluid rows per neighbour cell.  Without
// assembled blocks, row i contributes:
//  - viscous: a fluid neighbour j gives -f e (x) e to the slot of its cell,
//    and every neighbour (fluid or wall) f e (x) e to the row's own slot,
//    with the inertia;
//  - C Lambda C^T: row i's blocks sum, over its P-neighbours k, to
//    lambda_k C_ik (x) W_k(c), where W_k(c) is the sum of C_jk over the
//    transposed P-list of k inside cell c.  Every such j is a neighbour of i
//    (2 RadiusP < MaxRadius, the condition of the factored form) and the
//    cells are at least MaxRadius wide, so W_k has at most 2^D cells.
// Both kernels sum in a fixed order (no atomics), so the result is the same
// bits on every run.  A row whose neighbour list is not grouped into at most
// 3^D cells, or one of whose P-neighbours has more than kWBins cells, flags its
// cell; the per-row FP64 kernel then assembles that cell's rows and
// k_mg_level0 that cell's level-0 rows.
constexpr int kWBins = 8;
static_assert(kWBins * 3 <= 32, "one lane per bin and row component");

// Neighbour-grid cell coordinates packed 10 bits an axis (grids of at most
// 1024 cells an axis), so the stencil slot of one cell seen from another is
// a few integer operations instead of the divisions of key_coords.
__global__ void k_pack_cells(int N, DevParams P, const int* __restrict__ key, int* __restrict__ ccell)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    int c[3];
    key_coords(P, key[i], c);
    ccell[i] = c[0] | (c[1] << 10) | (c[2] << 20);
}

// stencil_slot for packed cell coordinates: the same slot, ((cj - ci) + 1)
// modulo the level-0 grid on every axis
__device__ __forceinline__ int slot_packed(const Level0Map& M, int pi, int pj)
{
    int o[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int v = ((pj >> (10 * d)) & 1023) - ((pi >> (10 * d)) & 1023) + 1;
        if ((unsigned)v >= (unsigned)min(3, M.cnt[d])) v = ((v % M.cnt[d]) + M.cnt[d]) % M.cnt[d];   // wrapped (rare)
        o[d] = v;
    }
    return M.st[2] * M.st[1] * o[0] + M.st[2] * o[1] + o[2];
}

// W_k: (packed cell, sum of C_jk over the rows j of that cell) for every particle
template <int D>
__global__ void __launch_bounds__(256) k_ct_cells(int N, const long long* __restrict__ ctptr, const int* __restrict__ ct_j,
                                                  const float* __restrict__ ct_v32, const int* __restrict__ ccell,
                                                  int* __restrict__ wkey, float* __restrict__ wval)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int bk[kWBins];
    float bw[kWBins][3];
#pragma unroll
    for (int b = 0; b < kWBins; ++b) {
        bk[b] = -1;
        bw[b][0] = bw[b][1] = bw[b][2] = 0.f;
    }
    bool over = false;
    const long long e1 = ctptr[k + 1];
    for (long long e = ctptr[k]; e < e1; ++e) {
        const int kj = ccell[ct_j[e]];
        float cv[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < D; ++d) cv[d] = ct_v32[e * D + d];
        bool placed = false;
#pragma unroll
        for (int b = 0; b < kWBins; ++b) {   // bins fill in order: a match comes before the first free bin
            if (!placed && (bk[b] == kj || bk[b] < 0)) {
                bk[b] = kj;
#pragma unroll
                for (int d = 0; d < 3; ++d) bw[b][d] += cv[d];
                placed = true;
            }
        }
        over = over || !placed;
    }
#pragma unroll
    for (int b = 0; b < kWBins; ++b) {
        wkey[(size_t)k * kWBins + b] = (over && b == 0) ? -2 : bk[b];
#pragma unroll
        for (int d = 0; d < 3; ++d) wval[((size_t)k * kWBins + b) * 3 + d] = bw[b][d];
    }
}

// The level-0 stencil rows (FP64 store of FP32 sums) and invDiag, one warp
// per level-0 cell: its fluid rows in order, each row's blocks accumulated
// into the cell's stencil in shared memory, written entry-major as
// k_mg_level0 writes it (zeros for a cell without fluid).  Global
// loads are issued ahead of the ordered accumulation: the cell keys of the
// next 32 neighbours while a chunk is scanned for runs, and the W_k bins of
// up to 32 P-neighbours at once into a per-warp stage.
constexpr int kPartStage = 16;   // P-neighbours staged at a time
static_assert(kPartStage * kWBins % 32 == 0 && kPartStage * 3 <= 64, "whole staging rounds");

template <int D>
__global__ void __launch_bounds__(kPairWarps * 32, 4)
k_part_pairs(DevParams P, Level0Map M, const int* __restrict__ key, const int* __restrict__ ccell, const int* __restrict__ type,
             const int* __restrict__ nc,
             const int* __restrict__ nfc, const long long* __restrict__ nptr, const int* __restrict__ nind,
             const float4* __restrict__ pe32, const int* __restrict__ ncp, const long long* __restrict__ nptrP,
             const int* __restrict__ nindP, const float* __restrict__ cval32, const float* __restrict__ cvl32,
             const int* __restrict__ wkey, const float* __restrict__ wval, const int* __restrict__ bucket,
             double* __restrict__ cof0, double* __restrict__ invDiag, int* __restrict__ cell_flags)
{
    constexpr int DD = D * D;
    constexpr int SMAX = D == 3 ? 27 : 9;
    __shared__ float sacc[kPairWarps][SMAX * DD];
    __shared__ int srun[kPairWarps][SMAX + 1];
    __shared__ int srkey[kPairWarps][SMAX];
    __shared__ int sslot[kPairWarps][kPartStage * kWBins];
    __shared__ float sval[kPairWarps][kPartStage * kWBins * 3];
    __shared__ float scl[kPairWarps][kPartStage * 3];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    float* acc = sacc[wl];
    int* run = srun[wl];
    int* rkey = srkey[wl];
    int* stslot = sslot[wl];
    float* stval = sval[wl];
    float* stcl = scl[wl];
    const unsigned full = 0xffffffffu;
    const int cells0 = M.cnt[0] * M.cnt[1] * M.cnt[2];
    const int rows0 = D * cells0;
    for (int g0 = wid; g0 < cells0; g0 += nwarps) {   // one level-0 cell: its fluid rows in order
        for (int t = lane; t < SMAX * DD; t += 32) acc[t] = 0.f;
        const int cx = g0 / (M.cnt[1] * M.cnt[2]) + M.mn[0], cy = (g0 / M.cnt[2]) % M.cnt[1] + M.mn[1], cz = g0 % M.cnt[2] + M.mn[2];
        const bool ingrid = cx < P.cc[0] && cy < P.cc[1] && cz < P.cc[2];
        const int icell = ingrid ? cell_id(P, cx, cy, cz) : 0;
        const int r0 = ingrid ? bucket[icell] : 0, r1 = ingrid ? bucket[icell + 1] : 0;
        bool cellbad = false;
        __syncwarp();
        for (int i = r0; i < r1; ++i) {
            const int pi = ccell[i];
            const long long nb = nptr[i];
            const int n = nc[i], nf = nfc[i];
            // runs of equal cell in the fluid part of the neighbour list
            int nrun = 0, last = -1;
            for (int c0 = 0; c0 < nf; c0 += 128) {   // four chunks of 32 slots, their loads issued together
                int kc[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = c0 + 32 * u + lane;
                    kc[u] = k < nf ? nind[nb + k] : -1;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) kc[u] = kc[u] >= 0 ? ccell[kc[u]] : -1;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = c0 + 32 * u + lane;
                    const int kj = kc[u];
                    int kp = __shfl_up_sync(full, kj, 1);
                    if (lane == 0) kp = last;
                    last = __shfl_sync(full, kj, 31);
                    const bool start = k < nf && kj != kp;
                    const unsigned bal = __ballot_sync(full, start);
                    const int at = nrun + __popc(bal & ((1u << lane) - 1u));
                    if (start && at < SMAX) {
                        run[at] = k;
                        rkey[at] = kj;
                    }
                    nrun += __popc(bal);
                }
            }
            bool bad = nrun > SMAX;
            if (lane == 0) run[min(nrun, SMAX)] = nf;
            __syncwarp();
            // viscous: lane r sums run r in list order; every term also enters the own slot
            float tv[DD];
#pragma unroll
            for (int t = 0; t < DD; ++t) tv[t] = 0.f;
            if (!bad && lane < nrun) {
                const int k0 = run[lane], k1 = run[lane + 1];
                float rsum[DD];
#pragma unroll
                for (int t = 0; t < DD; ++t) rsum[t] = 0.f;
#pragma unroll 4
                for (int k = k0; k < k1; ++k) {
                    const float4 pv = pe32[nb + k];
                    const float e[3] = {pv.x, pv.y, pv.z};
#pragma unroll
                    for (int r = 0; r < D; ++r)
#pragma unroll
                        for (int c = 0; c < D; ++c) rsum[r * D + c] += pv.w * e[r] * e[c];
                }
                const int slot = slot_packed(M, pi, rkey[lane]);
#pragma unroll
                for (int t = 0; t < DD; ++t) {
                    acc[slot * DD + t] -= rsum[t];
                    tv[t] = rsum[t];
                }
            }
            for (int k = nf + lane; k < n; k += 32) {   // wall neighbours: own slot only
                const float4 pv = pe32[nb + k];
                const float e[3] = {pv.x, pv.y, pv.z};
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int c = 0; c < D; ++c) tv[r * D + c] += pv.w * e[r] * e[c];
            }
            // lambda_k C_ik[r]^2 for the diagonal of the own block
            const long long pb = nptrP[i];
            const int np = ncp[i];
            float dp[3] = {0.f, 0.f, 0.f};
            for (int a = lane; a < np; a += 32) {
#pragma unroll
                for (int r = 0; r < D; ++r) dp[r] += cvl32[(pb + a) * D + r] * cval32[(pb + a) * D + r];
            }
#pragma unroll
            for (int t = 0; t < DD; ++t)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) tv[t] += __shfl_xor_sync(full, tv[t], o);
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) dp[r] += __shfl_xor_sync(full, dp[r], o);
            __syncwarp();
            const int si = slot_packed(M, pi, pi);
            const float in32 = P.inert32[type[i]];
            if (lane == 0 && !bad) {
#pragma unroll
                for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int c = 0; c < D; ++c) acc[si * DD + r * D + c] += tv[r * D + c] + (r == c ? in32 : 0.f);
            }
            __syncwarp();
            // C Lambda C^T: P-neighbours in order; the bins of one W_k are distinct cells
            for (int a0 = 0; a0 < np && !bad; a0 += kPartStage) {
                const int na = min(kPartStage, np - a0);
                bool over = false;
                // stage the bins (slot, W) of na P-neighbours, kPer a lane: all
                // loads of one level of the index chain issued together
                constexpr int kPer = kPartStage * kWBins / 32;
                int kk[kPer], wk[kPer];
                float wv[kPer][3];
#pragma unroll
                for (int u = 0; u < kPer; ++u) {
                    const int q = (lane + 32 * u) / kWBins;
                    kk[u] = q < na ? nindP[pb + a0 + q] : -1;
                }
#pragma unroll
                for (int u = 0; u < kPer; ++u) wk[u] = kk[u] >= 0 ? wkey[(size_t)kk[u] * kWBins + (lane + 32 * u) % kWBins] : -1;
#pragma unroll
                for (int u = 0; u < kPer; ++u)
#pragma unroll
                    for (int d = 0; d < 3; ++d)
                        wv[u][d] = wk[u] >= 0 ? wval[((size_t)kk[u] * kWBins + (lane + 32 * u) % kWBins) * 3 + d] : 0.f;
                float cl[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int t = lane + 32 * u;
                    cl[u] = t < na * 3 && t % 3 < D ? cvl32[(pb + a0 + t / 3) * D + t % 3] : 0.f;
                }
#pragma unroll
                for (int u = 0; u < kPer; ++u) {
                    const int t = lane + 32 * u;
                    if (wk[u] == -2) over = true;
                    stslot[t] = wk[u] >= 0 ? slot_packed(M, pi, wk[u]) : -1;
#pragma unroll
                    for (int d = 0; d < 3; ++d) stval[t * 3 + d] = wv[u][d];
                }
#pragma unroll
                for (int u = 0; u < 2; ++u)
                    if (lane + 32 * u < kPartStage * 3) stcl[lane + 32 * u] = cl[u];
                bad = __any_sync(full, over) || bad;
                __syncwarp();
                if (bad) break;
                for (int q = 0; q < na; ++q) {   // lane (bin, row component): a block row of one bin
                    if (lane < kWBins * D) {
                        const int b = lane / D, r = lane - b * D;
                        const int slot = stslot[q * kWBins + b];
                        if (slot >= 0) {
                            const float cr = stcl[q * 3 + r];
                            const float* w = stval + (q * kWBins + b) * 3;
                            float* a = acc + slot * DD + r * D;
#pragma unroll
                            for (int c2 = 0; c2 < D; ++c2) a[c2] += cr * w[c2];
                        }
                    }
                    __syncwarp();
                }
            }
            if (bad) {
                cellbad = true;
                break;
            }
            if (lane == 0) {
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    const float dg = in32 + tv[r * D + r] + dp[r];
                    invDiag[(size_t)i * D + r] = (double)(dg != 0.f ? 1.f / dg : 0.f);
                }
            }
            __syncwarp();
        }
        if (cellbad) {   // the per-row kernel assembles this cell's rows, k_mg_level0 its level-0 rows
            if (lane == 0) cell_flags[icell] = 1;
            __syncwarp();
            continue;
        }
        // the cell's level-0 rows (entry-major: entry e = slot * D + column component)
        for (int t = lane; t < SMAX * DD; t += 32) {
            const int slot = t / DD, rs = t - slot * DD;
            cof0[(size_t)(slot * D + rs % D) * rows0 + (size_t)g0 * D + rs / D] = (double)acc[t];
        }
        __syncwarp();
    }
}

// Block-local columns of a sliced list: for block b of blockDim rows (thread
// = row), the sorted distinct columns uniq[b][0..U) (slot e's column at
// acol[e * IS + IO]) and, per slot e, the column's rank among them at
// out16[e * OS + OO]: the fourth half of the fluid slot records, or the
// column word of the transposed P-list records itself (each slot's column
// is read before its rank replaces it, by the same thread).  A bitmap over the block's index
// window [lo, hi] marks the neighbours; word ranks come from a block scan of
// the word popcounts.  ucount[b] = U, or -1 when the window is wider than
// kWinWords * 32 or U > kUMax (the operator then gathers by column).
template <int IS, int IO, typename OutT, int OS, int OO>
__global__ void __launch_bounds__(MPH_PAIR_BLOCK) k_local_cols(int Nf, const long long* __restrict__ sptr, const int* __restrict__ nfc,
                                                             const int* acol, OutT* out16, int* __restrict__ uniq,
                                                             int* __restrict__ ucount)
{
    extern __shared__ unsigned lc_smem[];
    unsigned* bm = lc_smem;                       // kWinWords bitmap words
    unsigned* rank = lc_smem + kWinWords;         // kWinWords exclusive word ranks
    __shared__ int red[2][32];
    __shared__ unsigned wsum[32];
    const int tid = threadIdx.x, lane = tid & 31, wl = tid >> 5, nwl = blockDim.x >> 5;
    const int i = blockIdx.x * blockDim.x + tid;
    const bool row = i < Nf;
    const long long base = row ? sptr[i >> 5] + (i & 31) : 0;
    const int n = row ? nfc[i] : 0;
    // window of the block's columns
    int lo = INT_MAX, hi = -1;
    for (int k = 0; k < n; ++k) {
        const int col = acol[(base + (long long)k * 32) * IS + IO];
        lo = min(lo, col);
        hi = max(hi, col);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) { red[0][wl] = lo; red[1][wl] = hi; }
    __syncthreads();
    lo = INT_MAX;
    hi = -1;
    for (int w = 0; w < nwl; ++w) { lo = min(lo, red[0][w]); hi = max(hi, red[1][w]); }
    if (hi < 0) {   // no fluid neighbours in the block
        if (tid == 0) {
            ucount[blockIdx.x] = 0;
            atomicAdd(ucount + gridDim.x + 1, 1);
        }
        return;
    }
    const long long span = (long long)hi - lo + 1;
    if (span > (long long)kWinWords * 32) {
        if (tid == 0) ucount[blockIdx.x] = -1;
        return;
    }
    const int nw = (int)((span + 31) >> 5);
    for (int w = tid; w < nw; w += blockDim.x) bm[w] = 0u;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        const int off = acol[(base + (long long)k * 32) * IS + IO] - lo;
        atomicOr(&bm[off >> 5], 1u << (off & 31));
    }
    __syncthreads();
    // exclusive ranks of the words: thread chunks, then a block scan of the chunk sums
    const int per = (nw + blockDim.x - 1) / blockDim.x;
    const int w0 = min(nw, tid * per), w1 = min(nw, w0 + per);
    unsigned cs = 0;
    for (int w = w0; w < w1; ++w) cs += __popc(bm[w]);
    unsigned inc = cs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[wl] = inc;
    __syncthreads();
    unsigned woff = 0, total = 0;
    for (int w = 0; w < nwl; ++w) {
        if (w < wl) woff += wsum[w];
        total += wsum[w];
    }
    unsigned r = woff + inc - cs;
    for (int w = w0; w < w1; ++w) {
        rank[w] = r;
        r += __popc(bm[w]);
    }
    __syncthreads();
    const int U = (int)total;
    if (U > kUMax) {
        if (tid == 0) ucount[blockIdx.x] = -1;
        return;
    }
    for (int k = 0; k < n; ++k) {
        const long long e = base + (long long)k * 32;
        const int off = acol[e * IS + IO] - lo;
        const unsigned word = bm[off >> 5];
        out16[e * OS + OO] = (OutT)(rank[off >> 5] + __popc(word & ((1u << (off & 31)) - 1u)));
    }
    if (row) {   // the slice's padding slots (zero records) point at rank 0
        const int w = (int)((sptr[(i >> 5) + 1] - sptr[i >> 5]) >> 5);
        for (int k = n; k < w; ++k) out16[(base + (long long)k * 32) * OS + OO] = (OutT)0;
    }
    int* ul = uniq + (size_t)blockIdx.x * kUMax;
    for (int w = w0; w < w1; ++w) {
        unsigned word = bm[w];
        unsigned rr = rank[w];
        while (word) {
            const int b = __ffs(word) - 1;
            ul[rr++] = lo + w * 32 + b;
            word &= word - 1u;
        }
    }
    if (tid == 0) {   // after the blocks: the largest count, the staged blocks and their columns
        ucount[blockIdx.x] = U;
        atomicMax(ucount + gridDim.x, U);
        atomicAdd(ucount + gridDim.x + 1, 1);
        atomicAdd((unsigned*)ucount + gridDim.x + 2, (unsigned)U);
    }
}

// ---- host side ---------------------------------------------------------------------
static int grow_f(float** p, long long* cap, long long need)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 1024;
    MPH_CUDA(cudaMalloc((void**)p, (size_t)n * sizeof(float)));
    *cap = n;
    return MPH_OK;
}
static int grow_i(int** p, long long* cap, long long need)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 1024;
    MPH_CUDA(cudaMalloc((void**)p, (size_t)n * sizeof(int)));
    *cap = n;
    return MPH_OK;
}

static int grow_pairs(mph_case* c, long long slots)
{
    DeviceState& d = c->d;
    if (slots <= d.cap_pairs) return MPH_OK;
    if (d.pe32) cudaFree(d.pe32);
    d.pe32 = nullptr;
    d.cap_pairs = 0;
    const long long n = slots + slots / 8 + 1024;
    MPH_CUDA(cudaMalloc((void**)&d.pe32, (size_t)n * sizeof(float4)));
    d.cap_pairs = n;
    return MPH_OK;
}

// The sliced pair-term arrays of this step's form, allocated before the
// kernels that write them: FP32 g, the packed records and the block-local
// indices, or the FP16 records, and the slices' scales.
static int ensure_pair_records(mph_case* c)
{
    DeviceState& d = c->d;
    const int D = c->dim;
    MPH_TRY(grow_f(&d.pes32, &d.cap_pes32, c->nslots * D));
    const bool lrec = c->pair_recompute || c->pair_pack;   // records without the index half
    if (c->pair_pack && !c->pair_recompute && c->nslots > d.cap_grec32) {   // packed g, a word a slot
        if (d.grec32) cudaFree(d.grec32);
        d.grec32 = nullptr;
        d.cap_grec32 = 0;
        const long long n = c->nslots + c->nslots / 8 + 1024;
        MPH_CUDA(cudaMalloc((void**)&d.grec32, (size_t)n * sizeof(unsigned)));
        d.cap_grec32 = n;
    }
    if (lrec) {   // block-local indices, a half a slot
        if (c->nslots > d.cap_lcol16) {
            if (d.lcol16) cudaFree(d.lcol16);
            d.lcol16 = nullptr;
            d.cap_lcol16 = 0;
            const long long n = c->nslots + c->nslots / 8 + 1024;
            MPH_CUDA(cudaMalloc((void**)&d.lcol16, (size_t)n * sizeof(unsigned short)));
            d.cap_lcol16 = n;
        }
    } else if (c->nslots * 4 > d.cap_grec16) {   // slot records, 4 halves a slot
        if (d.grec16) cudaFree(d.grec16);
        d.grec16 = nullptr;
        d.cap_grec16 = 0;
        const long long n = c->nslots * 4 + c->nslots / 2 + 1024;
        MPH_CUDA(cudaMalloc((void**)&d.grec16, (size_t)n * sizeof(unsigned short)));
        d.cap_grec16 = n;
    }
    if (!d.pscale) MPH_CUDA(cudaMalloc((void**)&d.pscale, (size_t)(c->nslices + 1) * sizeof(float)));
    return MPH_OK;
}

// Option pair_fuse: k_pair_slices writes the sliced pair terms itself (no
// pair-term list in between: 16 bytes a neighbour slot less device memory,
// 3.7 GB on the config-1 workload) where nothing else reads that list, the
// point-Jacobi mixed form on the pair path with slot records.  Off by
// default: measured slower (assembly 9.6 against 8.2 ms on the config-1
// workload; a block of 32 warps per slice with a barrier per chunk hides
// the neighbours' position gathers worse than k_pair_terms' grid-stride
// warps).
static bool pair_fused(const mph_case* c) { return c->pair_fuse && c->step_pairs && mixed_jacobi(c) && !c->pair_recompute; }

// The factored operator equals the assembled one when 2 RadiusP < MaxRadius;
// its FP32 viscous part is accurate enough while FP32 rounding of that part
// (about 1e-7 of it, the part being visc_ratio of the inertia) stays below
// 1e-2 of the outer tolerance.
// The factored form holds its viscous pair coefficients in FP32, which moves
// A by about 1e-7 of its viscous part (visc_ratio of the inertia): it is used
// while that stays two orders under the 1e-6 velocity accuracy of the mixed
// form.  The pair path's residual (FP64 wall terms, two-float x) carries no
// other FP32 rounding, so it also serves outer tolerances below that bound
// (refinement to 1e-10); the warp-per-row residual of the FP32-block path
// rounds x to FP32 and is kept to tolerances above it.
bool factored_applies(const mph_case* c)
{
    if (!(c->precision == MPH_PRECISION_MIXED && c->factored && 2.0 * c->dp.rP < c->dp.maxR)) return false;
    const double pert = 1.0e-7 * c->visc_ratio;
    if (!(pert < 1.0e-8)) return false;
    const bool pair_path = !c->inner_blocks && c->visc_nonneg;
    return pair_path || pert < 1.0e-2 * c->tol_outer;
}

template <int D>
static void pair_slices_launch(mph_case* c)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    if (c->nslices == 0) return;
    if (c->pair_pack)
        k_pair_slices<D, true><<<c->nslices, 1024, 0, c->stream>>>(P, d.type, d.pos, d.pos32, d.poslo32, d.vel, d.nc, d.nptr, d.nind,
            d.nfc, d.ncp, d.nptrP, d.nindP, d.cval, d.pvec, d.sptr, d.acol, d.pes32, d.grec32, nullptr, d.pscale, d.bvec, d.cvl32,
            d.wrap32, d.invDiag);
    else
        k_pair_slices<D, false><<<c->nslices, 1024, 0, c->stream>>>(P, d.type, d.pos, d.pos32, d.poslo32, d.vel, d.nc, d.nptr, d.nind,
            d.nfc, d.ncp, d.nptrP, d.nindP, d.cval, d.pvec, d.sptr, d.acol, d.pes32, nullptr, d.grec16, d.pscale, d.bvec, d.cvl32,
            d.wrap32, d.invDiag);
    MPH_COUNT_LAUNCH();
}

int launch_pair_terms(mph_case* c)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    const bool fused = pair_fused(c);
    if (!fused) {   // the pair-term list, a record per neighbour slot
        long long slots = 0;
        MPH_CUDA(cudaMemcpyAsync(&slots, d.nptr + P.Nf, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
        MPH_CUDA(cudaStreamSynchronize(c->stream));
        MPH_TRY(grow_pairs(c, slots));
    }
    if (!d.tct) MPH_CUDA(cudaMalloc((void**)&d.tct, (size_t)(P.N + 1) * sizeof(double)));
    // FP32 copy of x and, after it, the FP32 remainders x - hi (two-float x
    // of the pair-path residual)
    if (!d.x32) MPH_CUDA(cudaMalloc((void**)&d.x32, (size_t)P.Nf * c->dim * 2 * sizeof(float)));
    if (!d.tct32) MPH_CUDA(cudaMalloc((void**)&d.tct32, (size_t)(P.N + 1) * sizeof(float)));
    long long ncv = 0;   // C values of the fluid rows, FP32 copy for the inner operator
    MPH_CUDA(cudaMemcpyAsync(&ncv, d.nptrP + P.Nf, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    ncv *= c->dim;
    if (ncv > d.cap_cval32) {
        if (d.cval32) cudaFree(d.cval32);
        d.cval32 = nullptr;
        d.cap_cval32 = 0;
        MPH_CUDA(cudaMalloc((void**)&d.cval32, (size_t)(ncv + ncv / 8 + 1024) * sizeof(float)));
        d.cap_cval32 = ncv + ncv / 8 + 1024;
    }
    { k_cval_f32<<<grid_for(ncv, 256), 256, 0, c->stream>>>(ncv, d.cval, d.cval32); MPH_COUNT_LAUNCH(); }
    float* sdiag = nullptr;
    double* sdiag64 = nullptr;
    float* cvl = nullptr;
    unsigned* gmax = nullptr;
    if (c->step_pairs) {   // FP32 inner operator on the pair terms
        if (!d.sdiag32) MPH_CUDA(cudaMalloc((void**)&d.sdiag32, (size_t)P.Nf * 8 * sizeof(float)));
        if (!d.sdiag64) MPH_CUDA(cudaMalloc((void**)&d.sdiag64, (size_t)P.Nf * 8 * sizeof(double)));
        sdiag64 = d.sdiag64;
        MPH_TRY(grow_f(&d.cvl32, &d.cap_cvl32, ncv));
        sdiag = d.sdiag32;
        cvl = d.cvl32;
        if (!d.pscale) MPH_CUDA(cudaMalloc((void**)&d.pscale, (size_t)((P.Nf + 31) / 32 + 1) * sizeof(float)));
        if (!fused) {
            MPH_CUDA(cudaMemsetAsync(d.pscale, 0, (size_t)((P.Nf + 31) / 32 + 1) * sizeof(float), c->stream));
            if (!c->pair_recompute)
                gmax = reinterpret_cast<unsigned*>(d.pscale);   // slice maxima, turned into scales by the slicing
        }
    }
    MPH_CUDA(cudaMemsetAsync(d.wrap32, 0, sizeof(int), c->stream));
    if (fused && c->nslices) MPH_TRY(ensure_pair_records(c));
    // the mixed form without grid levels takes D^-1 from here (no level-0 pass)
    double* dinv = c->step_pairs && mixed_jacobi(c) ? d.invDiag : nullptr;
    const unsigned g = std::min<long long>(((long long)P.Nf + kPtWarps - 1) / kPtWarps, 152LL * 128 / kPtWarps);
    const unsigned gw = grid_for((long long)P.Nf * 32, 256);
    if (c->dim == 2) {
        if (fused) pair_slices_launch<2>(c);
        else { k_pair_terms<2><<<g, kPtWarps * 32, 0, c->stream>>>(P, d.type, d.pos, d.pos32, d.poslo32, d.vel, d.nc, d.nptr, d.nind, d.nfc, d.ncp, d.nptrP,
                                                                    d.nindP, d.cval, d.pvec, d.pe32, d.bvec, cvl, gmax, d.wrap32, dinv); MPH_COUNT_LAUNCH(); }
        { k_wall_terms64<2><<<gw, 256, 0, c->stream>>>(P, d.type, d.pos, d.vel, d.nc, d.nfc, d.nptr, d.nind, d.bvec, sdiag, sdiag64); MPH_COUNT_LAUNCH(); }
    } else {
        if (fused) pair_slices_launch<3>(c);
        else { k_pair_terms<3><<<g, kPtWarps * 32, 0, c->stream>>>(P, d.type, d.pos, d.pos32, d.poslo32, d.vel, d.nc, d.nptr, d.nind, d.nfc, d.ncp, d.nptrP,
                                                                    d.nindP, d.cval, d.pvec, d.pe32, d.bvec, cvl, gmax, d.wrap32, dinv); MPH_COUNT_LAUNCH(); }
        { k_wall_terms64<3><<<gw, 256, 0, c->stream>>>(P, d.type, d.pos, d.vel, d.nc, d.nfc, d.nptr, d.nind, d.bvec, sdiag, sdiag64); MPH_COUNT_LAUNCH(); }
    }
    return MPH_OK;
}

// The sliced pair terms g = sqrt(f) e with the block columns, and the sliced
// lambda-scaled P-lists, of the fluid rows (after k_pair_terms).
// Block-local columns of one sliced list (rows in blocks of `block`), their
// counts and statistics after the blocks (read back with the other lists').
template <int IS, int IO, typename OutT, int OS, int OO>
static int local_cols(mph_case* c, int rows, int block, const long long* sptr, const int* cnt, const int* cols,
                      OutT* out16, int** uniq, long long* cap_uniq, int** ucount, long long* cap_ucount)
{
    const long long nb = grid_for(rows, block);
    MPH_TRY(grow_i(uniq, cap_uniq, nb * kUMax));
    MPH_TRY(grow_i(ucount, cap_ucount, nb + 3));
    const size_t smem = 2 * kWinWords * sizeof(unsigned);
    MPH_CUDA(cudaFuncSetAttribute(k_local_cols<IS, IO, OutT, OS, OO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MPH_CUDA(cudaMemsetAsync(*ucount + nb, 0, 3 * sizeof(int), c->stream));
    k_local_cols<IS, IO, OutT, OS, OO><<<(unsigned)nb, block, smem, c->stream>>>(rows, sptr, cnt, cols, out16, *uniq, *ucount);
    MPH_COUNT_LAUNCH();
    return MPH_OK;
}

// Dynamic shared memory the staging k_visc_rc32 may take: kUMax records (a
// float4 and D floats each), within the device's opt-in limit less the
// kernel's static shared memory.  The attribute is set to this fixed value
// (a per-launch value would race between host threads of batched cases).
static int rc_smem_max(int D)
{
    static std::atomic<int> cached[4];
    if (const int v = cached[D].load()) return v;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (D == 2) cudaFuncGetAttributes(&fa, k_visc_rc32<2, true>);
    else cudaFuncGetAttributes(&fa, k_visc_rc32<3, true>);
    const int want = kUMax * ((int)sizeof(float4) + D * (int)sizeof(float));
    const int v = std::max(0, std::min(want, optin - (int)fa.sharedSizeBytes));
    cached[D].store(v);
    return v;
}

// a step's count rounded up so that small changes keep the captured graphs
static int round_cols(int umax) { return umax > 0 ? (umax + 511) / 512 * 512 : 0; }

// Block-local columns of the inner operator's lists (after the slicing):
// the fluid neighbours of each 512-row block (their s, staged by
// k_visc_pen32) and the fluid rows of the transposed P-lists of each block of
// k_ct_apply32 (their s).  The largest counts set the operators' shared
// memory (0: gather by column).  Staging t for the P-lists the same way
// measured no faster.
static int launch_local_cols(mph_case* c)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    c->loc_smem = c->loc_ct_smem = 0;
    c->loc_blocks[0] = c->loc_blocks[1] = 0;
    c->loc_ct_blocks = 0;
    c->loc_cols = 0;
    if (P.Nf == 0 || !c->inner_local) return MPH_OK;
    const int D = c->dim;
    const long long nb = grid_for(P.Nf, c->pair_block), nbc = grid_for(P.N, c->ct_block);
    if (c->pair_recompute || c->pair_pack)
        MPH_TRY((local_cols<1, 0, unsigned short, 1, 0>(c, P.Nf, c->pair_block, d.sptr, d.nfc, d.acol, d.lcol16, &d.uniq, &d.cap_uniq,
                                                        &d.ucount, &d.cap_ucount)));
    else
        MPH_TRY((local_cols<1, 0, unsigned short, 4, 3>(c, P.Nf, c->pair_block, d.sptr, d.nfc, d.acol, d.grec16, &d.uniq, &d.cap_uniq,
                                                        &d.ucount, &d.cap_ucount)));
    int* ctw = reinterpret_cast<int*>(d.ctsval);   // the column words of the transposed records
    MPH_TRY((local_cols<4, 3, int, 4, 3>(c, P.N, c->ct_block, d.ctsptr, d.ct_cnt, ctw, ctw, &d.ctuniq, &d.cap_ctuniq, &d.ctucount,
                                         &d.cap_ctucount)));
    int h[2][3] = {};
    MPH_CUDA(cudaMemcpyAsync(h[0], d.ucount + nb, sizeof(h[0]), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(h[1], d.ctucount + nbc, sizeof(h[1]), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    const int xcap = round_cols(h[0][0]), ctcap = round_cols(h[1][0]);
    c->loc_blocks[0] = xcap ? h[0][1] : 0;
    c->loc_blocks[1] = (int)nb - c->loc_blocks[0];
    c->loc_cols = xcap ? (long long)(unsigned)h[0][2] : 0;
    c->loc_ct_blocks = ctcap ? h[1][1] : 0;
    c->loc_cap = xcap;
    const int xs = D == 3 ? kXs3 : 2;   // floats a staged s (float4 / float2)
    c->loc_smem = xcap * (c->pair_recompute ? (int)sizeof(float4) + D * (int)sizeof(float) : xs * (int)sizeof(float));
    c->loc_ct_smem = ctcap * xs * (int)sizeof(float);
    if (c->pair_recompute && c->loc_smem > rc_smem_max(D)) {   // a block's records do not fit: every block gathers
        c->loc_smem = 0;
        c->loc_blocks[1] += c->loc_blocks[0];
        c->loc_blocks[0] = 0;
        c->loc_cols = 0;
    }
    if (D == 2) {
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<2, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<2, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<2, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<2, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_rc32<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, rc_smem_max(2)));
        MPH_CUDA(cudaFuncSetAttribute(k_ct_apply32<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 2 * (int)sizeof(float)));
    } else {
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<3, true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<3, true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<3, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_pen32<3, true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float)));
        MPH_CUDA(cudaFuncSetAttribute(k_visc_rc32<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, rc_smem_max(3)));
        MPH_CUDA(cudaFuncSetAttribute(k_ct_apply32<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUMax * 4 * (int)sizeof(float)));
    }
    return MPH_OK;
}

int launch_pairs_to_slices(mph_case* c)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    const int D = c->dim;
    if (c->nslices == 0) return MPH_OK;
    MPH_TRY(ensure_pair_records(c));
    const bool lrec = c->pair_recompute || c->pair_pack;   // records without the index half
    if (!d.psptr) {
        MPH_CUDA(cudaMalloc((void**)&d.psptr, (size_t)(c->nslices + 1) * sizeof(long long)));
        MPH_CUDA(cudaMalloc((void**)&d.pswidth, (size_t)(c->nslices + 1) * sizeof(int)));
    }
    long long pslots = 0;
    MPH_TRY(launch_slice_ptr(c, P.Nf, d.ncp, d.pswidth, d.psptr, &pslots));
    MPH_TRY(grow_f(&d.psval, &d.cap_psval, pslots * 4));   // 16-byte records
    unsigned short* rec16 = lrec ? nullptr : d.grec16;
    unsigned* rec32 = c->pair_pack && !c->pair_recompute ? d.grec32 : nullptr;
    if (D == 2) {
        if (!pair_fused(c))
            { k_list_to_slices<2, true><<<c->nslices, 256, 0, c->stream>>>(P.Nf, d.sptr, d.nfc, d.nptr, d.nind, d.pe32, nullptr, d.acol,
                                                                          d.pes32, rec16, d.pscale, rec32); MPH_COUNT_LAUNCH(); }
        { k_list_to_slices<2, false><<<c->nslices, 256, 0, c->stream>>>(P.Nf, d.psptr, d.ncp, d.nptrP, d.nindP, nullptr, d.cvl32,
                                                                       nullptr, d.psval, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
    } else {
        if (!pair_fused(c))
            { k_list_to_slices<3, true><<<c->nslices, 256, 0, c->stream>>>(P.Nf, d.sptr, d.nfc, d.nptr, d.nind, d.pe32, nullptr, d.acol,
                                                                          d.pes32, rec16, d.pscale, rec32); MPH_COUNT_LAUNCH(); }
        { k_list_to_slices<3, false><<<c->nslices, 256, 0, c->stream>>>(P.Nf, d.psptr, d.ncp, d.nptrP, d.nindP, nullptr, d.cvl32,
                                                                       nullptr, d.psval, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
    }
    return launch_local_cols(c);
}

// The transposed P-lists (C in FP32) of every particle in the sliced layout
// (after build_ct).
int launch_ct_slices(mph_case* c)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    const int D = c->dim;
    const int ns = (P.N + 31) / 32;
    if (ns == 0) return MPH_OK;
    if (!d.ctsptr) {
        MPH_CUDA(cudaMalloc((void**)&d.ctsptr, (size_t)(ns + 1) * sizeof(long long)));
        MPH_CUDA(cudaMalloc((void**)&d.ctswidth, (size_t)(ns + 1) * sizeof(int)));
    }
    long long slots = 0;
    MPH_TRY(launch_slice_ptr(c, P.N, d.ct_cnt, d.ctswidth, d.ctsptr, &slots));
    MPH_TRY(grow_f(&d.ctsval, &d.cap_ctsval, slots * 4));   // 16-byte records
    if (D == 2) {
        { k_list_to_slices<2, false><<<ns, 256, 0, c->stream>>>(P.N, d.ctsptr, d.ct_cnt, d.ct_ptr, d.ct_j, nullptr, d.ct_v32, nullptr,
                                                               d.ctsval, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
    } else {
        { k_list_to_slices<3, false><<<ns, 256, 0, c->stream>>>(P.N, d.ctsptr, d.ct_cnt, d.ct_ptr, d.ct_j, nullptr, d.ct_v32, nullptr,
                                                               d.ctsval, nullptr, nullptr, nullptr); MPH_COUNT_LAUNCH(); }
    }
    return MPH_OK;
}

void launch_resid_factored(mph_case* c, const double* x, double* r, double* out)
{
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    unsigned* counter = (unsigned*)(d.flags + kFlagCounter);
    const unsigned gt = grid_for(P.N, 256);
    const unsigned g = std::min<long long>(((long long)P.Nf + kPairWarps - 1) / kPairWarps, kReduceBlocks);
    const long long nv = (long long)P.Nf * c->dim;
    if (c->step_pairs) {
        { k_split_f32<<<grid_for(nv, 256), 256, 0, c->stream>>>(nv, x, d.x32, d.x32 + nv); MPH_COUNT_LAUNCH(); }
        const unsigned gr = grid_for(P.Nf, c->pair_block);
        if (c->dim == 2) {
            { k_ct_apply<2><<<gt, 256, 0, c->stream>>>(P.N, P, d.type, d.ct_ptr, d.ct_j, d.ct_v, x, d.tct); MPH_COUNT_LAUNCH(); }
            { k_resid_pairs<2><<<gr, c->pair_block, 0, c->stream>>>(P, P.Nf, d.type, d.nfc, d.sptr, d.acol, d.pes32, d.sdiag64, d.ncp, d.nptrP,
                                                          d.nindP, d.cval, d.tct, x, d.x32, d.bvec, r, d.partials, counter, out); MPH_COUNT_LAUNCH(); }
        } else {
            { k_ct_apply<3><<<gt, 256, 0, c->stream>>>(P.N, P, d.type, d.ct_ptr, d.ct_j, d.ct_v, x, d.tct); MPH_COUNT_LAUNCH(); }
            { k_resid_pairs<3><<<gr, c->pair_block, 0, c->stream>>>(P, P.Nf, d.type, d.nfc, d.sptr, d.acol, d.pes32, d.sdiag64, d.ncp, d.nptrP,
                                                          d.nindP, d.cval, d.tct, x, d.x32, d.bvec, r, d.partials, counter, out); MPH_COUNT_LAUNCH(); }
        }
        return;
    }
    { k_cval_f32<<<grid_for(nv, 256), 256, 0, c->stream>>>(nv, x, d.x32); MPH_COUNT_LAUNCH(); }
    if (c->dim == 2) {
        { k_ct_apply<2><<<gt, 256, 0, c->stream>>>(P.N, P, d.type, d.ct_ptr, d.ct_j, d.ct_v, x, d.tct); MPH_COUNT_LAUNCH(); }
        { k_resid_factored<2><<<g, kPairWarps * 32, 0, c->stream>>>(P, d.type, d.nc, d.nfc, d.nptr, d.nind, d.pe32, d.ncp, d.nptrP,
                                                                   d.nindP, d.cval, d.tct, x, d.x32, d.bvec, r, d.partials, counter,
                                                                   out); MPH_COUNT_LAUNCH(); }
    } else {
        { k_ct_apply<3><<<gt, 256, 0, c->stream>>>(P.N, P, d.type, d.ct_ptr, d.ct_j, d.ct_v, x, d.tct); MPH_COUNT_LAUNCH(); }
        { k_resid_factored<3><<<g, kPairWarps * 32, 0, c->stream>>>(P, d.type, d.nc, d.nfc, d.nptr, d.nind, d.pe32, d.ncp, d.nptrP,
                                                                   d.nindP, d.cval, d.tct, x, d.x32, d.bvec, r, d.partials, counter,
                                                                   out); MPH_COUNT_LAUNCH(); }
    }
}

// Level-0 partial stencils and D^-1 on the pair-term path (instead of the
// cell-block kernel).  *done = false when the grids are too small for it
// (an axis with fewer than 3 cells): the per-row kernel then assembles every
// row; otherwise per-cell fallback flags are left in c->d.cell_flags.
int launch_part_pairs(mph_case* c, const Level0Map& M, bool* done)
{
    *done = false;
    DeviceState& d = c->d;
    const DevParams& P = c->dp;
    const int D = c->dim;
    for (int a = 0; a < D; ++a)
        if (P.cc[a] < 3 || M.cnt[a] < 3 || P.cc[a] > 1024) return MPH_OK;
    if (!d.wkey) {
        MPH_CUDA(cudaMalloc((void**)&d.ccell, (size_t)P.N * sizeof(int)));
        MPH_CUDA(cudaMalloc((void**)&d.wkey, (size_t)P.N * kWBins * sizeof(int)));
        MPH_CUDA(cudaMalloc((void**)&d.wval, (size_t)P.N * kWBins * 3 * sizeof(float)));
    }
    const long long fbytes = (long long)(P.T + 1) * sizeof(int);   // capacity kept in bytes
    if (fbytes > d.cap_cell_flags) {
        if (d.cell_flags) cudaFree(d.cell_flags);
        d.cell_flags = nullptr;
        d.cap_cell_flags = 0;
        MPH_CUDA(cudaMalloc((void**)&d.cell_flags, (size_t)(fbytes + fbytes / 8 + 1024)));
        d.cap_cell_flags = fbytes + fbytes / 8 + 1024;
    }
    MPH_CUDA(cudaMemsetAsync(d.cell_flags, 0, (size_t)(P.T + 1) * sizeof(int), c->stream));
    MPH_TRY(ensure_mg_cof(c));
    double* cof0 = d.mg_cof + c->lv[0].off_cof;
    const long long cells0 = (long long)M.cnt[0] * M.cnt[1] * M.cnt[2];
    const unsigned g = std::min<long long>((cells0 + kPairWarps - 1) / kPairWarps, 152LL * 16);
    { k_pack_cells<<<grid_for(P.N, 256), 256, 0, c->stream>>>(P.N, P, d.key, d.ccell); MPH_COUNT_LAUNCH(); }
    if (D == 2) {
        { k_ct_cells<2><<<grid_for(P.N, 256), 256, 0, c->stream>>>(P.N, d.ct_ptr, d.ct_j, d.ct_v32, d.ccell, d.wkey, d.wval); MPH_COUNT_LAUNCH(); }
        { k_part_pairs<2><<<g, kPairWarps * 32, 0, c->stream>>>(P, M, d.key, d.ccell, d.type, d.nc, d.nfc, d.nptr, d.nind, d.pe32, d.ncp, d.nptrP,
                                                               d.nindP, d.cval32, d.cvl32, d.wkey, d.wval, d.bucket, cof0, d.invDiag,
                                                               d.cell_flags); MPH_COUNT_LAUNCH(); }
    } else {
        { k_ct_cells<3><<<grid_for(P.N, 256), 256, 0, c->stream>>>(P.N, d.ct_ptr, d.ct_j, d.ct_v32, d.ccell, d.wkey, d.wval); MPH_COUNT_LAUNCH(); }
        { k_part_pairs<3><<<g, kPairWarps * 32, 0, c->stream>>>(P, M, d.key, d.ccell, d.type, d.nc, d.nfc, d.nptr, d.nind, d.pe32, d.ncp, d.nptrP,
                                                               d.nindP, d.cval32, d.cvl32, d.wkey, d.wval, d.bucket, cof0, d.invDiag,
                                                               d.cell_flags); MPH_COUNT_LAUNCH(); }
    }
    c->level0_done = true;
    *done = true;
    return MPH_OK;
}

}  // namespace mph
