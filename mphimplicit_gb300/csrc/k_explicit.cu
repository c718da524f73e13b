// k_explicit.cu - explicit particle physics and output-step fields.
//
//   k_density       : calculateDensityA + calculateGravityCenter +
//                     calculateDensityP (main.cpp:1737, 1767, 1903) in one
//                     neighbour pass; every sum keeps the reference's order
//   k_pressure_a_*  : calculatePressureA (main.cpp:1801)
//   k_diffuse       : calculateDiffuseInterface (main.cpp:1851)
//   k_accelerate    : calculatePhysicalCoefficients' mass (main.cpp:1710),
//                     calculateGravity and calculateAcceleration
//                     (main.cpp:2065, 2076)
//   k_div_pressure, k_output_forces : calculateDivergenceP,
//                     calculatePressureP, calculateViscosityV and
//                     calculateVirialStressAtParticle (main.cpp:1932-2063,
//                     4494-4738), output steps only
// When every surface-tension coefficient CofA is zero the pressure-A and
// diffuse-interface forces are exact zeros and their passes are skipped.
#include "mph_device.cuh"

namespace mph {

template <int D>
__global__ void __launch_bounds__(128) k_density(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                 const int* __restrict__ nc, const long long* __restrict__ nptr,
                                                 const int* __restrict__ nind, double* __restrict__ densA,
                                                 double* __restrict__ gcen, double* __restrict__ vsp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const int ti = type[i];
    double xi[3];
    load_vec<D>(pos, i, xi);
    const double rA2 = DMUL(P.rA, P.rA), rG2 = DMUL(P.rG, P.rG), rP2 = DMUL(P.rP, P.rP);
    double sa = 0.0, sp = 0.0, sg[3] = {0.0, 0.0, 0.0};
    const long long b = nptr[i];
    const int n = nc[i];
    for (int k = 0; k < n; ++k) {
        const int j = nind[b + k];
        if (j == i) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        const double ratio = P.ratio[ti][type[j]];
        const bool inA = rA2 - r2 >= 0, inG = rG2 - r2 >= 0, inP = rP2 - r2 >= 0;
        if (!(inA || inG || inP)) continue;
        const double r = __dsqrt_rn(r2);
        if (inA) sa = DADD(sa, DMUL(ratio, w_a(P.kfa, r, P.rA)));
        if (inG) {
            const double w = DMUL(ratio, w_quad(P.kfg, r, P.rG));
#pragma unroll
            for (int d = 0; d < D; ++d) sg[d] = DADD(sg[d], DMUL(DDIV(DMUL(q[d], w), P.R2g), P.rG));
        }
        if (inP) sp = DADD(sp, w_quad(P.kfp, r, P.rP));
    }
    densA[i] = sa;
    store_vec<D>(gcen, i, sg);
    vsp[i] = DSUB(sp, P.N0p);
}

__global__ void k_pressure_a(DevParams P, const int* __restrict__ type, const double* __restrict__ densA, double* __restrict__ presA)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const double a = densA[i];
    presA[i] = (P.N0a <= a) ? 0.0 : DDIV(DMUL(P.cofA[type[i]], DSUB(a, P.N0a)), P.l0);
}

template <int D>
__global__ void __launch_bounds__(128) k_surface_forces(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                        const int* __restrict__ nc, const long long* __restrict__ nptr,
                                                        const int* __restrict__ nind, const double* __restrict__ presA,
                                                        const double* __restrict__ gcen, double* __restrict__ force)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const int ti = type[i];
    double xi[3], gi[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(gcen, i, gi);
    const double rA2 = P.rA * P.rA, rG2 = P.rG * P.rG;
    const double ai = P.cofA[ti] * P.cofK * P.cofK, aj = ai;   // both from i's type (main.cpp:1857, 1863)
    const double pa_i = presA[i];
    double fa[3] = {0, 0, 0}, fd[3] = {0, 0, 0};
    const long long b = nptr[i];
    const int n = nc[i];
    const double sc = P.rG * (P.vol / P.l0);
    for (int k = 0; k < n; ++k) {
        const int j = nind[b + k];
        if (j == i) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (r2 == 0.0) continue;
        const int tj = type[j];
        const double rij = P.ratio[ti][tj], rji = P.ratio[tj][ti];
        const double r = sqrt(r2);
        double e[3];
#pragma unroll
        for (int d = 0; d < D; ++d) e[d] = q[d] / r;
        if (rA2 - r2 > 0) {                                    // pressure A force
            const double dwa = dw_a(P.kfa, r, P.rA);
            const double s = pa_i * (rij * dwa) + presA[j] * (rji * dwa);
#pragma unroll
            for (int d = 0; d < D; ++d) fa[d] += s * e[d] * P.vol;
        }
        if (rG2 - r2 > 0) {                                    // diffuse-interface force
            double gj[3];
            load_vec<D>(gcen, j, gj);
            const double wg = w_quad(P.kfg, r, P.rG);
            const double wij = rij * wg, wji = rji * wg;
#pragma unroll
            for (int d = 0; d < D; ++d) fd[d] -= (aj * gj[d] * wji - ai * gi[d] * wij) / P.R2g * sc;
            const double dwg = dw_quad(P.kfg, r, P.rG);
            const double dwij = rij * dwg, dwji = rji * dwg;
            double gr = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) gr += (aj * gj[d] * dwji - ai * gi[d] * dwij) * q[d];
#pragma unroll
            for (int d = 0; d < D; ++d) fd[d] -= gr * e[d] / P.R2g * sc;
        }
    }
    double f[3];
    load_vec<D>(force, i, f);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = (f[d] + fa[d]) + fd[d];
    store_vec<D>(force, i, f);
}

template <int D>
__global__ void k_accelerate(DevParams P, int fB, int fE, const int* __restrict__ type, double* __restrict__ force,
                             double* __restrict__ vel)
{
    const int i = fB + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= fE) return;
    const double m = DMUL(P.density[type[i]], P.vol);
    double f[3], v[3];
    load_vec<D>(force, i, f);
    load_vec<D>(vel, i, v);
#pragma unroll
    for (int d = 0; d < D; ++d) {
        f[d] = DADD(f[d], DMUL(m, P.gravity[d]));
        v[d] = DADD(v[d], DMUL(DDIV(f[d], m), P.dt));
    }
    store_vec<D>(force, i, f);
    store_vec<D>(vel, i, v);
}

// ---- output-step fields ----------------------------------------------------
template <int D>
__global__ void __launch_bounds__(128) k_div_pressure(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                      const double* __restrict__ vel, const int* __restrict__ nc,
                                                      const long long* __restrict__ nptr, const int* __restrict__ nind,
                                                      const double* __restrict__ vsp, double* __restrict__ divP,
                                                      double* __restrict__ presP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    double xi[3], vi[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(vel, i, vi);
    const double rP2 = P.rP * P.rP;
    double sum = 0.0;
    const long long b = nptr[i];
    for (int k = 0; k < nc[i]; ++k) {
        const int j = nind[b + k];
        if (j == i) continue;
        double xj[3], q[3], vj[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (r2 == 0.0) continue;
        if (rP2 - r2 >= 0) {
            const double r = sqrt(r2);
            const double dw = dw_quad(P.kfp, r, P.rP);
            load_vec<D>(vel, j, vj);
#pragma unroll
            for (int d = 0; d < D; ++d) sum -= (vj[d] - vi[d]) * (q[d] / r) * dw;
        }
    }
    divP[i] = sum;
    const int t = type[i];
    const double kap = vsp[i] < 0.0 ? 0.0 : P.bulk[t];
    double p = -P.lambda[t] * sum;
    if (vsp[i] > 0.0) p += kap * vsp[i];
    presP[i] = p;
}

template <int D>
__global__ void __launch_bounds__(128) k_output_forces(DevParams P, const int* __restrict__ type, const double* __restrict__ pos,
                                                       const double* __restrict__ vel, const int* __restrict__ nc,
                                                       const int* __restrict__ ncp, const long long* __restrict__ nptr,
                                                       const long long* __restrict__ nptrP, const int* __restrict__ nind,
                                                       const int* __restrict__ nindP, const double* __restrict__ presP,
                                                       const double* __restrict__ presA, const double* __restrict__ gcen,
                                                       double* __restrict__ force, double* __restrict__ virS,
                                                       double* __restrict__ virP)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const int ti = type[i];
    double xi[3], vi[3], gi[3];
    load_vec<D>(pos, i, xi);
    load_vec<D>(vel, i, vi);
    load_vec<D>(gcen, i, gi);
    const double pi = presP[i], pa = presA[i];
    const double mui = P.mu[ti];
    const double rA2 = P.rA * P.rA, rG2 = P.rG * P.rG, rP2 = P.rP * P.rP, rV2 = P.rV * P.rV;
    const double a = P.cofA[ti] * P.cofK * P.cofK;
    double fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0};
    double sP[3][3] = {}, sA[3][3] = {}, sV[3][3] = {}, sD[3][3] = {};
    const long long b = nptr[i];
    for (int k = 0; k < nc[i]; ++k) {
        const int j = nind[b + k];
        if (j == i) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (r2 == 0.0) continue;
        const int tj = type[j];
        const double r = sqrt(r2);
        double e[3];
#pragma unroll
        for (int d = 0; d < D; ++d) e[d] = q[d] / r;
        if (rP2 - r2 > 0) {        // pressure P force (calculatePressureP)
            const double dw = dw_quad(P.kfp, r, P.rP);
#pragma unroll
            for (int d = 0; d < D; ++d) fp[d] += (pi + presP[j]) * (dw * q[d] / r) * P.vol;
        }
        if (rV2 - r2 > 0) {        // viscosity force and its virial
            const double dw = -dw_quad(P.kfv, r, P.rV);
            double vj[3];
            load_vec<D>(vel, j, vj);
            double ue = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) ue += (vj[d] - vi[d]) * e[d];
            const double muj = P.mu[tj];
            const double muij = 2.0 * (mui * muj) / (mui + muj);
            double fij[3];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                fij[d] = P.visc * muij * ue * e[d] * dw / r * P.vol;
                fv[d] += fij[d];
            }
#pragma unroll
            for (int aa = 0; aa < D; ++aa)
#pragma unroll
                for (int bb = 0; bb < D; ++bb) sV[aa][bb] += 0.5 * fij[aa] * q[bb] / P.vol;
        }
        if (rA2 - r2 > 0) {        // pressure A virial
            const double dw = P.ratio[ti][tj] * dw_a(P.kfa, r, P.rA);
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {
                const double fij = pa * (dw * q[aa] / r) * P.vol;
#pragma unroll
                for (int bb = 0; bb < D; ++bb) sA[aa][bb] += fij * q[bb] / P.vol;
            }
        }
        if (rG2 - r2 > 0) {        // diffuse-interface virial (both terms)
            const double ratio = P.ratio[ti][tj];
            const double w = ratio * w_quad(P.kfg, r, P.rG);
            const double dw = ratio * dw_quad(P.kfg, r, P.rG);
            double gr = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) gr += (-gi[d]) * q[d];
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {
                const double f1 = -a * (-gi[aa]) * w / P.R2g * P.rG * (P.vol / P.l0);
                const double f2 = -a * gr * (dw * q[aa] / r) / P.R2g * P.rG * (P.vol / P.l0);
#pragma unroll
                for (int bb = 0; bb < D; ++bb) sD[aa][bb] += f1 * q[bb] / P.vol + f2 * q[bb] / P.vol;
            }
        }
    }
    // pressure P virial over the P list (main.cpp:4512-4555)
    for (int k = 0; k < ncp[i]; ++k) {
        const int j = nindP[nptrP[i] + k];
        if (j == i) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (r2 == 0.0) continue;
        if (rP2 - r2 > 0) {
            const double r = sqrt(r2);
            const double dw = dw_quad(P.kfp, r, P.rP);
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {
                const double fij = pi * (dw * q[aa] / r) * P.vol;
#pragma unroll
                for (int bb = 0; bb < D; ++bb) sP[aa][bb] += fij * q[bb] / P.vol;
            }
        }
    }
    double f[3];
    load_vec<D>(force, i, f);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = (f[d] + fp[d]) + fv[d];
    store_vec<D>(force, i, f);
    double tr = 0.0;
#pragma unroll
    for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
            double v = 0.0;
            if (aa < D && bb < D) v = ((sP[aa][bb] + sA[aa][bb]) + sV[aa][bb]) + sD[aa][bb];
            virS[9 * (size_t)i + 3 * aa + bb] = v;
            if (aa == bb) tr += v;
        }
    virP[i] = -1.0 / (double)D * tr;
}

// calculateDensityP alone over the P-list.  The P-list holds exactly the
// pairs with r^2 <= RadiusP^2, in the full list's order, so the sum is
// bit-identical to the full-list pass.
template <int D>
__global__ void __launch_bounds__(128) k_density_p(DevParams P, const double* __restrict__ pos, const int* __restrict__ ncp,
                                                   const long long* __restrict__ nptrP, const int* __restrict__ nindP,
                                                   double* __restrict__ vsp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    double xi[3];
    load_vec<D>(pos, i, xi);
    const double rP2 = DMUL(P.rP, P.rP);
    double sp = 0.0;
    const long long b = nptrP[i];
    const int n = ncp[i];
    for (int k = 0; k < n; ++k) {
        const int j = nindP[b + k];
        if (j == i) continue;
        double xj[3], q[3];
        load_vec<D>(pos, j, xj);
        sep_vec<D>(P, xj, xi, q);
        const double r2 = norm2_exact<D>(q);
        if (r2_within(r2, rP2)) sp = DADD(sp, w_quad(P.kfp, __dsqrt_rn(r2), P.rP));
    }
    vsp[i] = DSUB(sp, P.N0p);
}

// The full density pass (DensityA, GravityCenter, DensityP) and PressureA.
void launch_density_full(mph_case* c)
{
    const DevParams& P = c->dp;
    const unsigned g = grid_for(P.N, 128);
    if (c->dim == 2)
        { k_density<2><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.nc, c->d.nptr, c->d.nind, c->d.densA, c->d.gcen, c->d.vsp); MPH_COUNT_LAUNCH(); }
    else
        { k_density<3><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.nc, c->d.nptr, c->d.nind, c->d.densA, c->d.gcen, c->d.vsp); MPH_COUNT_LAUNCH(); }
    { k_pressure_a<<<grid_for(P.N, 256), 256, 0, c->stream>>>(P, c->d.type, c->d.densA, c->d.presA); MPH_COUNT_LAUNCH(); }
    c->densa_valid = true;
}

// DensityA, GravityCenter and PressureA only act through the surface-tension
// coefficients CofA.  With every CofA zero they are dead in the step, so the
// step computes DensityP alone; they are computed from the same positions and
// lists when a reader (export, output fields) asks for them.
void ensure_density_a(mph_case* c)
{
    if (!c->densa_valid) launch_density_full(c);
}

void launch_explicit(mph_case* c)
{
    const DevParams& P = c->dp;
    const unsigned g = grid_for(P.N, 128);
    if (P.surface) {
        launch_density_full(c);
    } else {
        if (c->dim == 2)
            { k_density_p<2><<<g, 128, 0, c->stream>>>(P, c->d.pos, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.vsp); MPH_COUNT_LAUNCH(); }
        else
            { k_density_p<3><<<g, 128, 0, c->stream>>>(P, c->d.pos, c->d.ncp, c->d.nptrP, c->d.nindP, c->d.vsp); MPH_COUNT_LAUNCH(); }
        c->densa_valid = false;
    }
    if (P.surface) {
        if (c->dim == 2)
            { k_surface_forces<2><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.nc, c->d.nptr, c->d.nind, c->d.presA, c->d.gcen, c->d.force); MPH_COUNT_LAUNCH(); }
        else
            { k_surface_forces<3><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.nc, c->d.nptr, c->d.nind, c->d.presA, c->d.gcen, c->d.force); MPH_COUNT_LAUNCH(); }
    }
    const int nf = c->fE - c->fB;
    if (nf > 0) {
        if (c->dim == 2)
            { k_accelerate<2><<<grid_for(nf, 256), 256, 0, c->stream>>>(P, c->fB, c->fE, c->d.type, c->d.force, c->d.vel); MPH_COUNT_LAUNCH(); }
        else
            { k_accelerate<3><<<grid_for(nf, 256), 256, 0, c->stream>>>(P, c->fB, c->fE, c->d.type, c->d.force, c->d.vel); MPH_COUNT_LAUNCH(); }
    }
}

// the density pass alone: the initial pass of main() (main.cpp:371-373)
void launch_explicit_density_only(mph_case* c)
{
    launch_density_full(c);
}

void launch_output_fields(mph_case* c)
{
    ensure_density_a(c);
    const DevParams& P = c->dp;
    const unsigned g = grid_for(P.N, 128);
    if (c->dim == 2) {
        { k_div_pressure<2><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.nc, c->d.nptr, c->d.nind, c->d.vsp, c->d.divP, c->d.presP); MPH_COUNT_LAUNCH(); }
        { k_output_forces<2><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.nc, c->d.ncp, c->d.nptr, c->d.nptrP, c->d.nind,
                                                     c->d.nindP, c->d.presP, c->d.presA, c->d.gcen, c->d.force, c->d.virS, c->d.virP); MPH_COUNT_LAUNCH(); }
    } else {
        { k_div_pressure<3><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.nc, c->d.nptr, c->d.nind, c->d.vsp, c->d.divP, c->d.presP); MPH_COUNT_LAUNCH(); }
        { k_output_forces<3><<<g, 128, 0, c->stream>>>(P, c->d.type, c->d.pos, c->d.vel, c->d.nc, c->d.ncp, c->d.nptr, c->d.nptrP, c->d.nind,
                                                     c->d.nindP, c->d.presP, c->d.presA, c->d.gcen, c->d.force, c->d.virS, c->d.virP); MPH_COUNT_LAUNCH(); }
    }
}

}  // namespace mph
