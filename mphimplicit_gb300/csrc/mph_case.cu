// mph_case.cu - case lifetime and the stage drivers of one time step.
//
// Host-side replacements of readGridFile's allocations and the
// initializeWeight / initializeFluid / initializeWall / initializeDomain
// set-up (main.cpp:565-1162), and the step sequence of main.cpp:386-474.
// The host code of this file is compiled without floating-point contraction so
// the derived constants (kernel normalisations, lattice sums N0a/N0p, wall
// rotations, cell widths) equal the reference's bit for bit on every host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

static thread_local std::string g_error;
std::atomic<long long> g_launch_count{0};
thread_local long long t_launch_count = 0;

// ---- profiling (CUDA events on the case stream) ------------------------------
static cudaEvent_t take_event(mph_case* c)
{
    cudaEvent_t e;
    if (!c->prof.pool.empty()) {
        e = c->prof.pool.back();
        c->prof.pool.pop_back();
    } else {
        cudaEventCreate(&e);
    }
    return e;
}

int prof_begin(mph_case* c, int k, cudaEvent_t* e0)
{
    (void)k;
    if (!c->prof.on) return 0;
    *e0 = take_event(c);
    cudaEventRecord(*e0, c->stream);
    return 1;
}

void prof_end(mph_case* c, int k, cudaEvent_t e0)
{
    if (!c->prof.on) return;
    cudaEvent_t e1 = take_event(c);
    cudaEventRecord(e1, c->stream);
    c->prof.pending.push_back({k, {e0, e1}});
}

int prof_collect(mph_case* c)
{
    if (c->prof.pending.empty()) return MPH_OK;
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& p : c->prof.pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        c->prof.kern_ms[p.first] += ms;
        c->prof.kern_n[p.first] += 1;
        c->prof.pool.push_back(p.second.first);
        c->prof.pool.push_back(p.second.second);
    }
    c->prof.pending.clear();
    return MPH_OK;
}

int fail(int status, const std::string& msg)
{
    g_error = msg;
    return status;
}
int cuda_check(cudaError_t e, const char* what)
{
    g_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? MPH_ERR_NOMEM : MPH_ERR_CUDA;
}
const char* last_error() { return g_error.c_str(); }

template <typename T>
static int dalloc(mph_case* c, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc");
    c->allocations.push_back((void*)*p);
    return MPH_OK;
}

// ---- parameter derivation (main.cpp:886-1111) --------------------------------
static double kfac(bool two_d, double Sw, double h) { return two_d ? (1.0 / Sw) / (h * h) : (1.0 / Sw) / (h * h * h); }

static int derive(mph_case* c, const mph_particles* parts)
{
    const bool two_d = c->dim == 2;
    const mph_params& p = c->prm;
    DevParams& P = c->dp;
    std::memset(&P, 0, sizeof(P));
    P.dim = c->dim;
    P.N = parts->count;
    P.l0 = parts->spacing;
    P.dt = p.dt;
    P.vol = two_d ? P.l0 * P.l0 : P.l0 * P.l0 * P.l0;
    const double l0 = P.l0;
    P.rA = p.radius_ratio_a * l0;
    P.rG = p.radius_ratio_a * l0;   // RadiusRatioG = RadiusRatioA (main.cpp:888)
    P.rP = p.radius_ratio_p * l0;
    P.rV = p.radius_ratio_v * l0;
    if (two_d) {
        c->Swa = 1.0 / 2.0 * 2.0 / 15.0 * M_PI / l0 / l0;
        c->Swg = 1.0 / 2.0 * 1.0 / 3.0 * M_PI / l0 / l0;
        P.R2g = 1.0 / 2.0 * 1.0 / 30.0 * M_PI * P.rG * P.rG / l0 / l0 / c->Swg;
    } else {
        c->Swa = 1.0 / 3.0 * 1.0 / 5.0 * M_PI / l0 / l0 / l0;
        c->Swg = 1.0 / 3.0 * 2.0 / 5.0 * M_PI / l0 / l0 / l0;
        P.R2g = 1.0 / 3.0 * 4.0 / 105.0 * M_PI * P.rG * P.rG / l0 / l0 / l0 / c->Swg;
    }
    c->Swp = c->Swg;
    c->Swv = c->Swg;
    P.kfa = kfac(two_d, c->Swa, P.rA);
    P.kfg = kfac(two_d, c->Swg, P.rG);
    P.kfp = kfac(two_d, c->Swp, P.rP);
    P.kfv = kfac(two_d, c->Swv, P.rV);
    // lattice sums (main.cpp:911-980), same loop and expression order
    auto lattice = [&](double radius, bool a) {
        const int range = (int)std::ceil(radius / l0);
        const int rz = two_d ? 0 : range;
        double sum = 0.0;
        for (int ix = -range; ix <= range; ++ix)
            for (int iy = -range; iy <= range; ++iy)
                for (int iz = -rz; iz <= rz; ++iz) {
                    if (ix == 0 && iy == 0 && iz == 0) continue;
                    const double x = l0 * (double)ix, y = l0 * (double)iy, z = l0 * (double)iz;
                    const double r2 = x * x + y * y + z * z;
                    if (r2 <= radius * radius) {
                        const double r = std::sqrt(r2);
                        const double q = r / radius;
                        if (a) sum += kfac(two_d, c->Swa, radius) * q * (1.0 - q) * (1.0 - q);
                        else sum += kfac(two_d, c->Swp, radius) * ((1.0 - q) * (1.0 - q));
                    }
                }
        return sum;
    };
    P.N0a = lattice(P.rA, true);
    P.N0p = lattice(P.rP, false);
    double integN, integX;
    if (two_d) { P.cofK = 0.350778153; integN = 0.024679383; integX = 0.226126699; }
    else       { P.cofK = 0.326976006; integN = 0.021425779; integX = 0.233977488; }
    P.surface = 0;
    for (int t = 0; t < kTypeCount; ++t) {
        P.cofA[t] = p.surface_tension[t] / ((P.rG / l0) * (integN + P.cofK * P.cofK * integX));
        if (P.cofA[t] != 0.0) P.surface = 1;
        P.density[t] = p.density[t];
        P.bulk[t] = p.bulk_modulus[t];
        P.lambda[t] = p.bulk_viscosity[t];
        P.mu[t] = p.shear_viscosity[t];
        for (int u = 0; u < kTypeCount; ++u) P.ratio[t][u] = p.interaction_ratio[t][u];
    }
    for (int d = 0; d < 3; ++d) P.gravity[d] = p.gravity[d];
    P.visc = two_d ? 8.0 : 10.0;
    P.inv_rv = 1.0 / P.rV;
    P.m2h_rv = -2.0 / P.rV;
    P.inv_rp = 1.0 / P.rP;
    P.m2h_rp = -2.0 / P.rP;
    for (int t = 0; t < kTypeCount; ++t)
        for (int u = 0; u < kTypeCount; ++u)
            P.muij[t][u] = 2.0 * (P.mu[t] * P.mu[u]) / (P.mu[t] + P.mu[u]);
    for (int t = 0; t < kTypeCount; ++t) {
        // IEEE products and quotients, no contraction: the kernels' FP64
        // inertia to the bit, without two divisions a row on the device
        P.inert64[t] = P.density[t] * P.vol / P.vol / P.dt;
        P.inert32[t] = (float)(P.density[t] * P.vol / P.vol / P.dt);
        P.lambda32[t] = (float)P.lambda[t];
        for (int u = 0; u < kTypeCount; ++u) P.vm32[t][u] = (float)(P.visc * P.muij[t][u]);
    }
    P.wdA32 = (float)(-P.kfv * P.m2h_rv);
    // the pair terms of the FP32 inner operator are stored as sqrt(f) e, which
    // needs f >= 0 for every pair of types
    c->visc_nonneg = P.wdA32 >= 0.f;
    for (int t = 0; t < kTypeCount; ++t)
        for (int u = 0; u < kTypeCount; ++u)
            if (!(P.vm32[t][u] >= 0.f)) c->visc_nonneg = false;
    P.inv_rv32 = (float)P.inv_rv;
    P.rV2_32 = (float)(P.rV * P.rV);
    // size of the viscous part of a row of A against its inertia rho/dt: the
    // sum of the pair coefficients f over the lattice within RadiusV (largest
    // viscosity, smallest density), with a factor 4 for compressed packings
    {
        double mu_max = 0.0, rho_min = 1.0e300;
        for (int t = 0; t < kTypeCount; ++t) {
            mu_max = std::max(mu_max, std::fabs(P.mu[t]));
            if (P.density[t] > 0.0) rho_min = std::min(rho_min, P.density[t]);
        }
        const int range = (int)std::ceil(P.rV / l0);
        const int rz = two_d ? 0 : range;
        double fsum = 0.0;
        for (int ix = -range; ix <= range; ++ix)
            for (int iy = -range; iy <= range; ++iy)
                for (int iz = -rz; iz <= rz; ++iz) {
                    if (ix == 0 && iy == 0 && iz == 0) continue;
                    const double r = l0 * std::sqrt((double)(ix * ix + iy * iy + iz * iz));
                    if (r < P.rV) fsum += P.visc * mu_max * P.kfv * (2.0 / P.rV) * (1.0 - r / P.rV) / r;
                }
        c->visc_ratio = 4.0 * fsum / (rho_min / P.dt);
    }
    // walls (initializeWall main.cpp:1023-1062; theta = |omega|^2 as written there)
    for (int t = 0; t < 4; ++t)
        for (int d = 0; d < 3; ++d) {
            c->wallC[t][d] = p.wall_center[t][d];
            c->wallV[t][d] = p.wall_velocity[t][d];
            c->wallW[t][d] = p.wall_omega[t][d];
        }
    for (int t = 2; t < 4; ++t) {
        const double* w = c->wallW[t];
        const double theta = std::fabs(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        double nrm[3] = {0, 0, 0};
        if (theta != 0.0)
            for (int d = 0; d < 3; ++d) nrm[d] = w[d] / theta;
        const double s = std::sin(theta * P.dt / 2.0), co = std::cos(theta * P.dt / 2.0);
        const double q0 = nrm[0] * s, q1 = nrm[1] * s, q2 = nrm[2] * s, q3 = co;
        double (&R)[3][3] = c->wallR[t];
        R[0][0] = q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3;
        R[0][1] = 2.0 * (q0 * q1 - q2 * q3);
        R[0][2] = 2.0 * (q0 * q2 + q1 * q3);
        R[1][0] = 2.0 * (q0 * q1 + q2 * q3);
        R[1][1] = -q0 * q0 + q1 * q1 - q2 * q2 + q3 * q3;
        R[1][2] = 2.0 * (q1 * q2 - q0 * q3);
        R[2][0] = 2.0 * (q0 * q2 - q1 * q3);
        R[2][1] = 2.0 * (q1 * q2 + q0 * q3);
        R[2][2] = -q0 * q0 - q1 * q1 + q2 * q2 + q3 * q3;
    }
    // domain and cells (initializeDomain main.cpp:1064-1096)
    P.maxR = 0.0;
    P.maxR = std::max(P.maxR, P.rA);
    P.maxR = std::max(P.maxR, 2.0 * P.rP);
    P.maxR = std::max(P.maxR, P.rV);
    double dmax[3];
    for (int d = 0; d < 3; ++d) {
        P.dmin[d] = parts->domain_min[d];
        dmax[d] = parts->domain_max[d];
        c->prm_domain_min[d] = parts->domain_min[d];
        c->prm_domain_max[d] = parts->domain_max[d];
        P.dw[d] = dmax[d] - P.dmin[d];
        P.hw[d] = 0.5 * P.dw[d];
        P.wsafe[d] = 0.75 * P.dw[d];
    }
    double cnt[3];
    cnt[0] = std::floor((dmax[0] - P.dmin[0]) / P.maxR);
    cnt[1] = std::floor((dmax[1] - P.dmin[1]) / P.maxR);
    cnt[2] = two_d ? 1.0 : std::floor((dmax[2] - P.dmin[2]) / P.maxR);
    for (int d = 0; d < 3; ++d) {
        if (!(cnt[d] >= 1.0) || cnt[d] > 1.0e9) return fail(MPH_ERR_INPUT, "domain narrower than MaxRadius along an axis");
        P.cc[d] = (int)cnt[d];
    }
    const double tot = cnt[0] * cnt[1] * cnt[2];
    if (tot > 1.0e9) return fail(MPH_ERR_INPUT, "too many background cells");
    P.T = (int)tot;
    for (int d = 0; d < 3; ++d) P.cw[d] = P.dw[d] / P.cc[d];
    for (int d = 0; d < c->dim; ++d) {
        const int range = (int)std::ceil(P.maxR / P.cw[d]);
        if (2 * range + 1 > 3)   // assert at main.cpp:1402-1404
            return fail(MPH_ERR_INPUT, "neighbour cell range exceeds one cell (reference assertion)");
    }
    P.maxR2 = P.maxR * P.maxR;
    P.rP2 = P.rP * P.rP;
    // sort size: smallest power of two above N (main.cpp:640-645)
    P.powExp = 0;
    while ((P.N >> P.powExp) != 0) ++P.powExp;
    P.nPow = 1 << P.powExp;
    // FP32 pre-classification band: worst-case FP32 error of a squared
    // separation, from the largest coordinate magnitude, with a 16x margin
    double mag = 0.0;
    for (int d = 0; d < c->dim; ++d) mag = std::max({mag, std::fabs(P.dmin[d]), std::fabs(dmax[d]), P.dw[d]});
    const double ulp = std::ldexp(1.0, (int)std::ceil(std::log2(std::max(mag, 1e-300))) - 23);
    const double e = 4.0 * ulp;                       // per-component separation error bound
    auto band = [&](double R2) { return 16.0 * (c->dim * (2.0 * std::sqrt(R2) * e + e * e) + R2 * 1.0e-6); };
    const double bM = band(P.maxR2), bP = band(P.rP2);
    P.maxR2_lo = (float)(P.maxR2 - bM);
    P.maxR2_hi = (float)(P.maxR2 + bM);
    P.rP2_lo = (float)(P.rP2 - bP);
    P.rP2_hi = (float)(P.rP2 + bP);
    P.exact_only = (bM > 0.25 * P.maxR2 || bP > 0.25 * P.rP2) ? 1 : 0;
    for (int d = 0; d < c->dim; ++d)
        if (P.cc[d] < 3) P.exact_only = 1;   // FP32 wrap would be ambiguous
    for (int d = 0; d < 3; ++d) {
        P.w32[d] = (float)P.dw[d];
        P.hw32[d] = (float)P.hw[d];
    }
    return MPH_OK;
}

static int validate(const mph_params* prm, const mph_particles* parts, int dim)
{
    if (!prm || !parts || !parts->type || !parts->pos || !parts->vel) return fail(MPH_ERR_ARG, "null argument");
    if (dim != 2 && dim != 3) return fail(MPH_ERR_ARG, "dim must be 2 or 3");
    if (parts->count < 1) return fail(MPH_ERR_INPUT, "no particles");
    if (!(parts->spacing > 0.0)) return fail(MPH_ERR_INPUT, "particle spacing must be positive");
    if (!(prm->dt > 0.0)) return fail(MPH_ERR_INPUT, "Dt must be positive");
    int nf = 0;
    for (int i = 0; i < parts->count; ++i) {
        const int t = parts->type[i];
        if (t < 0 || t > 3) return fail(MPH_ERR_INPUT, "particle type outside 0..3");
        nf += t < 2;
        for (int d = 0; d < 3; ++d)
            if (!std::isfinite(parts->pos[3 * i + d]) || !std::isfinite(parts->vel[3 * i + d]))
                return fail(MPH_ERR_INPUT, "non-finite particle position or velocity");
    }
    if (nf < 1) return fail(MPH_ERR_INPUT, "no fluid particles");
    if (dim == 2) {
        const double z0 = parts->pos[2];
        for (int i = 0; i < parts->count; ++i) {
            if (parts->pos[3 * i + 2] != z0) return fail(MPH_ERR_INPUT, "2D case with particles on different z planes");
            if (parts->vel[3 * i + 2] != 0.0) return fail(MPH_ERR_INPUT, "2D case with a z velocity");
        }
        if (prm->gravity[2] != 0.0) return fail(MPH_ERR_INPUT, "2D case with z gravity");
        for (int t = 2; t < 4; ++t)
            if (prm->wall_velocity[t][2] != 0.0 || prm->wall_omega[t][0] != 0.0 || prm->wall_omega[t][1] != 0.0)
                return fail(MPH_ERR_INPUT, "2D case with out-of-plane wall motion");
    }
    return MPH_OK;
}

int case_alloc_particles(mph_case* c)
{
    const DevParams& P = c->dp;
    const int VSn = vs_of(c->dim);
    const size_t N = P.N;
    DeviceState& d = c->d;
    MPH_TRY(dalloc(c, &d.pos, N * VSn));
    MPH_TRY(dalloc(c, &d.vel, N * VSn));
    MPH_TRY(dalloc(c, &d.force, N * VSn));
    MPH_TRY(dalloc(c, &d.pos_alt, N * VSn));
    MPH_TRY(dalloc(c, &d.vel_alt, N * VSn));
    MPH_TRY(dalloc(c, &d.pos32, N * VSn));
    MPH_TRY(dalloc(c, &d.poslo32, N * VSn));
    if (c->dim == 2) MPH_TRY(dalloc(c, &d.pt32, N));
    else d.pt32 = reinterpret_cast<float4*>(d.pos32);   // its w holds the type bits
    MPH_TRY(dalloc(c, &d.wrap32, 1));
    MPH_TRY(dalloc(c, &d.type, N));
    MPH_TRY(dalloc(c, &d.id, N));
    MPH_TRY(dalloc(c, &d.type_alt, N));
    MPH_TRY(dalloc(c, &d.id_alt, N));
    MPH_TRY(dalloc(c, &d.densA, N));
    MPH_TRY(dalloc(c, &d.gcen, N * VSn));
    MPH_TRY(dalloc(c, &d.presA, N));
    MPH_TRY(dalloc(c, &d.vsp, N));
    MPH_TRY(dalloc(c, &d.divP, N));
    MPH_TRY(dalloc(c, &d.presP, N));
    MPH_TRY(dalloc(c, &d.virP, N));
    MPH_TRY(dalloc(c, &d.virS, N * 9));
    MPH_TRY(dalloc(c, &d.key, (size_t)P.nPow));
    MPH_TRY(dalloc(c, &d.perm, (size_t)P.nPow));
    MPH_TRY(dalloc(c, &d.bucket, (size_t)2 * P.T + 2));
    MPH_TRY(dalloc(c, &d.nc, N));
    MPH_TRY(dalloc(c, &d.nfc, N + 32));
    MPH_TRY(dalloc(c, &d.ncp, N));
    MPH_TRY(dalloc(c, &d.nptr, N + 1));
    MPH_TRY(dalloc(c, &d.nptrP, N + 1));
    const size_t Nf = P.Nf, n = Nf * c->dim;
    const int nsl = (int)((Nf + 31) / 32);
    MPH_TRY(dalloc(c, &d.sptr, (size_t)nsl + 1));
    MPH_TRY(dalloc(c, &d.swidth, (size_t)nsl + 1));
    MPH_TRY(dalloc(c, &d.bvec, n));
    MPH_TRY(dalloc(c, &d.invDiag, n));
    MPH_TRY(dalloc(c, &d.selfk, Nf));
    MPH_TRY(dalloc(c, &d.pvec, N));
    const int S = c->dim == 2 ? 9 : 27;
    MPH_TRY(dalloc(c, &d.part, Nf * S * c->dim * c->dim));
    MPH_TRY(dalloc(c, &d.x, n));
    MPH_TRY(dalloc(c, &d.r, n));
    MPH_TRY(dalloc(c, &d.s, n));
    MPH_TRY(dalloc(c, &d.y, n));
    MPH_TRY(dalloc(c, &d.p, n));
    MPH_TRY(dalloc(c, &d.q, n));
    MPH_TRY(dalloc(c, &d.u, n));
    MPH_TRY(dalloc(c, &d.partials, (size_t)std::max<size_t>(kReduceBlocks, Nf / 32 + 64)));
    MPH_TRY(dalloc(c, &d.scal, 32));
    MPH_TRY(dalloc(c, &d.flags, kFlagCount));
    MPH_TRY(dalloc(c, &d.bbox, 8));
    MPH_TRY(dalloc(c, &d.totals, 8));
    MPH_TRY(dalloc(c, &d.dmax, 4));
    MPH_CUDA(cudaMemsetAsync(d.flags, 0, kFlagCount * sizeof(int), c->stream));
    return MPH_OK;
}

static int upload_particles(mph_case* c, const mph_particles* parts)
{
    const int N = parts->count;
    const int VSn = vs_of(c->dim);
    std::vector<double> pos((size_t)N * VSn, 0.0), vel((size_t)N * VSn, 0.0);
    std::vector<int> id(N);
    for (int i = 0; i < N; ++i) {
        for (int d = 0; d < c->dim; ++d) {
            pos[(size_t)i * VSn + d] = parts->pos[3 * i + d];
            vel[(size_t)i * VSn + d] = parts->vel[3 * i + d];
        }
        id[i] = parts->id ? parts->id[i] : i;
    }
    MPH_CUDA(cudaMemcpyAsync(c->d.pos, pos.data(), pos.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemcpyAsync(c->d.vel, vel.data(), vel.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemcpyAsync(c->d.type, parts->type, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemcpyAsync(c->d.id, id.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemsetAsync(c->d.force, 0, (size_t)N * VSn * sizeof(double), c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    // the plane of a 2D case (z is not simulated; the reference keeps it fixed)
    c->z_plane = c->dim == 2 ? parts->pos[2] : 0.0;
    return MPH_OK;
}

// ---- multigrid geometry (calculateMultiGridDepth main.cpp:2777-2850) --------
static int mg_geometry(mph_case* c)
{
    const int* mn = c->bbox;       // min x,y,z
    const int* mx = c->bbox + 3;   // max x,y,z
    double maxCount = 0.0;
    for (int d = 0; d < 3; ++d)
        if ((mx[d] - mn[d]) > maxCount) maxCount = (mx[d] - mn[d] + 1);
    int p = 0;
    while ((1 << p) <= maxCount) ++p;
    c->depth = p;
    if (c->depth < 2) return fail(MPH_ERR_INPUT, "fluid spans fewer than two neighbour cells: multigrid depth < 2 (the reference requires 2)");
    if (c->depth > kMaxLevels) return fail(MPH_ERR_INPUT, "multigrid too deep");
    c->lv.assign(c->depth, LevelGeom());
    long vec = 0, cof = 0;
    for (int L = 0; L < c->depth; ++L) {
        LevelGeom& g = c->lv[L];
        g.cells = 1;
        int S = 1;
        for (int d = 0; d < 3; ++d) {
            g.mn[d] = mn[d] >> L;
            g.mx[d] = (mx[d] >> L) + 1;
            g.cnt[d] = g.mx[d] - g.mn[d];
            g.st[d] = std::min(3, g.cnt[d]);
            g.cells *= g.cnt[d];
            S *= g.st[d];
        }
        g.rows = c->dim * g.cells;
        g.off_vec = vec;
        g.off_cof = cof;
        vec += g.rows;
        cof += (long)g.rows * c->dim * S;
    }
    c->mg_rows_total = vec;
    c->mg_cof_total = cof;
    return MPH_OK;
}

static int grow(void** p, long long* cap, long long need, size_t elem)
{
    if (need <= *cap) return MPH_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const long long n = need + need / 8 + 256;
    cudaError_t e = cudaMalloc(p, (size_t)n * elem);
    if (e != cudaSuccess) return cuda_check(e, "cudaMalloc(grow)");
    *cap = n;
    return MPH_OK;
}

// ---- stages --------------------------------------------------------------------
int stage_step_begin(mph_case* c)
{
    launch_step_begin(c);
    c->densa_valid = false;
    // WallCenter += WallVelocity*Dt after the particles moved (main.cpp:2123-2127)
    for (int t = 2; t < 4; ++t)
        for (int d = 0; d < 3; ++d) c->wallC[t][d] += c->wallV[t][d] * c->dp.dt;
    MPH_CUDA(cudaGetLastError());
    c->stage = 1;
    return MPH_OK;
}

int stage_cellsort(mph_case* c)
{
    launch_cell_keys(c);
    if (c->cell_sort) MPH_TRY(launch_counting_sort(c));
    else launch_bitonic_sort(c);
    launch_cell_ranges_and_permute(c);
    const int init[8] = {c->dp.cc[0], c->dp.cc[1], c->dp.cc[2], 0, 0, 0, 0, 0};
    MPH_CUDA(cudaMemcpyAsync(c->d.bbox, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
    launch_fluid_bbox(c);
    int hb[8];
    int ends[2];
    MPH_CUDA(cudaMemcpyAsync(hb, c->d.bbox, sizeof(hb), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(&ends[0], c->d.bucket + c->dp.T, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(&ends[1], c->d.bucket + 2 * c->dp.T, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    MPH_CUDA(cudaGetLastError());
    c->fB = 0;
    c->fE = ends[0];
    c->wB = ends[0];
    c->wE = ends[1];
    if (c->fE != c->dp.Nf) return fail(MPH_ERR_STATE, "fluid count changed in the cell sort");
    for (int k = 0; k < 6; ++k) c->bbox[k] = hb[k];
    MPH_TRY(mg_geometry(c));
    c->stage = 2;
    return MPH_OK;
}

int stage_neighbors(mph_case* c)
{
    const int N = c->dp.N;
    cudaEvent_t pe = nullptr;
    int pon = prof_begin(c, 3, &pe);
    launch_neighbor_count(c);
    if (pon) prof_end(c, 3, pe);
    MPH_TRY(launch_scan_i32_to_i64(c, c->d.nc, c->d.nptr, N));
    MPH_TRY(launch_scan_i32_to_i64(c, c->d.ncp, c->d.nptrP, N));
    long long tot[2];
    MPH_CUDA(cudaMemcpyAsync(&tot[0], c->d.nptr + N, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaMemcpyAsync(&tot[1], c->d.nptrP + N, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    c->nnb = tot[0];
    c->nnbP = tot[1];
    void* p = c->d.nind;
    MPH_TRY(grow(&p, &c->d.cap_nind, tot[0], sizeof(int)));
    c->d.nind = (int*)p;
    p = c->d.nindP;
    MPH_TRY(grow(&p, &c->d.cap_nindP, tot[1], sizeof(int)));
    c->d.nindP = (int*)p;
    pon = prof_begin(c, 3, &pe);
    launch_neighbor_fill(c);
    if (pon) prof_end(c, 3, pe);
    MPH_CUDA(cudaGetLastError());
    c->stage = 3;
    return MPH_OK;
}

int stage_explicit(mph_case* c)
{
    launch_explicit(c);
    MPH_CUDA(cudaGetLastError());
    c->stage = 4;
    return MPH_OK;
}

int stage_assemble(mph_case* c)
{
    if (c->stage < 4) return fail(MPH_ERR_STATE, "assemble before the explicit stage");
    MPH_TRY(launch_assemble(c));
    MPH_CUDA(cudaGetLastError());
    c->stage = 5;
    return MPH_OK;
}

int ensure_mg_cof(mph_case* c)
{
    void* p = c->d.mg_cof;
    MPH_TRY(grow(&p, &c->d.cap_mg_cof, c->mg_cof_total, sizeof(double)));
    c->d.mg_cof = (double*)p;
    return MPH_OK;
}

int stage_mg_build(mph_case* c)
{
    if (c->stage < 5) return fail(MPH_ERR_STATE, "multigrid build before assembly");
    if (mixed_jacobi(c)) {   // no multigrid levels in the point-Jacobi mixed form
        c->stage = 6;
        return MPH_OK;
    }
    MPH_TRY(ensure_mg_cof(c));
    if (c->mg_rows_total > c->d.cap_mg_vec) {
        for (double** b : {&c->d.mg_invd, &c->d.mg_q, &c->d.mg_s, &c->d.mg_r, &c->d.mg_res}) {
            if (*b) cudaFree(*b);
            *b = nullptr;
        }
        const long long n = c->mg_rows_total + c->mg_rows_total / 8 + 256;
        for (double** b : {&c->d.mg_invd, &c->d.mg_q, &c->d.mg_s, &c->d.mg_r, &c->d.mg_res}) MPH_CUDA(cudaMalloc((void**)b, n * sizeof(double)));
        c->d.cap_mg_vec = n;
    }
    // the pair path wrote the level-0 stencils already, except for the cells
    // it flagged for the per-row kernel
    launch_mg_level0(c, c->level0_done ? c->d.cell_flags : nullptr);
    for (int L = 1; L < c->depth; ++L) launch_mg_coarse(c, L);
    launch_mg_invd(c);
    MPH_CUDA(cudaGetLastError());
    c->stage = 6;
    return MPH_OK;
}

int stage_solve(mph_case* c)
{
    if (c->stage < 6) return fail(MPH_ERR_STATE, "solve before the multigrid build");
    MPH_TRY(run_cr_solve(c));
    MPH_CUDA(cudaGetLastError());
    c->stage = 7;
    return MPH_OK;
}

int stage_step_end(mph_case* c)
{
    c->time += c->dp.dt;
    c->stage = 0;
    return MPH_OK;
}

int stage_output_fields(mph_case* c)
{
    if (c->stage < 3 && c->stage != 0) return fail(MPH_ERR_STATE, "output fields need neighbour lists");
    launch_output_fields(c);
    MPH_CUDA(cudaGetLastError());
    c->have_output = true;
    return MPH_OK;
}

// ---- create / destroy ---------------------------------------------------------
// Whether a mixed-form case created from these inputs with the default
// options steps on the pair-term path (no assembled blocks): the parameter
// derivation of case creation, without device work.
bool pair_path_expected(const mph_params* prm, const mph_particles* parts, int dim)
{
    mph_case c;
    c.dim = dim;
    c.precision = MPH_PRECISION_MIXED;
    c.prm = *prm;
    if (derive(&c, parts) != MPH_OK) return false;
    return factored_applies(&c) && c.inner_blocks == false && c.visc_nonneg;
}

int case_create(const mph_params* prm, const mph_particles* parts, int dim, int precision, void* stream, mph_case** out)
{
    if (!out) return fail(MPH_ERR_ARG, "null output handle");
    *out = nullptr;
    MPH_TRY(validate(prm, parts, dim));
    if (precision != MPH_PRECISION_FP64 && precision != MPH_PRECISION_MIXED) return fail(MPH_ERR_ARG, "unknown precision");
    if (precision == MPH_PRECISION_MIXED && !mixed_available()) return fail(MPH_ERR_ARG, "mixed precision is not available in this build");
    mph_case* c = new mph_case();
    c->dim = dim;
    c->precision = precision;
    c->stream = (cudaStream_t)stream;
    c->prm = *prm;
    cudaGetDevice(&c->device);
    // the allocation-free residual check's fixed array is reserved on this
    // device before the case takes its memory
    int st = noalloc_prepare(c->device);
    if (st == MPH_OK) st = derive(c, parts);
    if (st == MPH_OK) {
        int nf = 0;
        for (int i = 0; i < parts->count; ++i) nf += parts->type[i] < 2;
        c->dp.Nf = nf;
        c->time = parts->time;
        st = case_alloc_particles(c);
    }
    if (st == MPH_OK) st = upload_particles(c, parts);
    // the initial pass of main() (main.cpp:369-373)
    if (st == MPH_OK) st = stage_cellsort(c);
    if (st == MPH_OK) st = stage_neighbors(c);
    if (st == MPH_OK) {
        launch_explicit_density_only(c);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_check(e, "initial pass");
    }
    c->stage = 0;
    if (st != MPH_OK) {
        case_destroy(c);
        return st;
    }
    *out = c;
    return MPH_OK;
}

int case_destroy(mph_case* c)
{
    if (!c) return MPH_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    else cudaDeviceSynchronize();
    if (c->cr_exec) cudaGraphExecDestroy(c->cr_exec);
    if (c->mx_exec) cudaGraphExecDestroy(c->mx_exec);
    for (cudaGraphExec_t e : c->sx_exec)
        if (e) cudaGraphExecDestroy(e);
    if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
    if (c->cap_stream2) cudaStreamDestroy(c->cap_stream2);
    if (c->cap_stream3) cudaStreamDestroy(c->cap_stream3);
    for (cudaEvent_t e : c->gev)
        if (e) cudaEventDestroy(e);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->fork_stream) cudaStreamDestroy(c->fork_stream);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    for (void* p : c->allocations) cudaFree(p);
    DeviceState& d = c->d;
    for (void* p : {(void*)d.nind, (void*)d.nindP, (void*)d.acol, (void*)d.aval, (void*)d.aval32, (void*)d.cval,
                    (void*)d.mg_cof, (void*)d.mg_invd, (void*)d.mg_q, (void*)d.mg_s, (void*)d.mg_r, (void*)d.mg_res, (void*)d.mg_cof32,
                    (void*)d.mg_q32, (void*)d.mg_s32, (void*)d.mg_r32, (void*)d.mg_res32, (void*)d.v32,
                    (void*)d.ct_cnt, (void*)d.ct_ptr, (void*)d.ct_j, (void*)d.ct_v, (void*)d.cell_flags, d.ct_tmp,
                    (void*)d.mg_invd32, (void*)d.mg_dinv32, (void*)d.pe32, (void*)d.tct, (void*)d.x32, (void*)d.arow32, (void*)d.ct_v32, (void*)d.cval32,
                    (void*)d.tct32, (void*)d.pes32, (void*)d.sdiag32, (void*)d.sdiag64, (void*)d.cvl32, (void*)d.psptr, (void*)d.ctsptr,
                    (void*)d.pswidth, (void*)d.ctswidth, (void*)d.pscol, (void*)d.ctscol, (void*)d.psval, (void*)d.ctsval,
                    (void*)d.grec16, (void*)d.grec32, (void*)d.pscale, (void*)d.lcol16, (void*)d.uniq, (void*)d.ucount,
                    (void*)d.ctuniq, (void*)d.ctucount, (void*)d.wkey, (void*)d.wval, (void*)d.ccell,
                    (void*)d.io3, (void*)d.vprev, (void*)d.vprev_alt, (void*)d.sort_cnt, (void*)d.sort_off, d.scan_tmp})
        if (p) cudaFree(p);
    for (auto& p : c->prof.pending) {
        cudaEventDestroy(p.second.first);
        cudaEventDestroy(p.second.second);
    }
    for (cudaEvent_t e : c->prof.pool) cudaEventDestroy(e);
    delete c;
    return MPH_OK;
}

int case_step(mph_case* c, int nsteps)
{
    int last = MPH_OK;
    for (int s = 0; s < nsteps; ++s) {
        cudaEvent_t ev[8];
        int ne = 0;
        auto mark = [&]() {
            if (!c->prof.on) return;
            ev[ne] = take_event(c);
            cudaEventRecord(ev[ne], c->stream);
            ++ne;
        };
        mark();
        MPH_TRY(stage_step_begin(c));
        mark();
        MPH_TRY(stage_cellsort(c));
        mark();
        MPH_TRY(stage_neighbors(c));
        mark();
        MPH_TRY(stage_explicit(c));
        mark();
        MPH_TRY(stage_assemble(c));
        mark();
        MPH_TRY(stage_mg_build(c));
        mark();
        MPH_TRY(stage_solve(c));
        mark();
        MPH_TRY(stage_step_end(c));
        if (c->prof.on) {
            MPH_CUDA(cudaStreamSynchronize(c->stream));
            for (int k = 0; k + 1 < ne; ++k) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
                c->prof.stage_ms[k] += ms;
            }
            for (int k = 0; k < ne; ++k) c->prof.pool.push_back(ev[k]);
            MPH_TRY(prof_collect(c));
        }
        if (c->stats.status != MPH_OK) last = c->stats.status;
    }
    return last;
}

int case_profile(mph_case* c, int enable)
{
    MPH_TRY(prof_collect(c));
    c->prof.on = enable != 0;
    for (double& v : c->prof.stage_ms) v = 0.0;
    for (double& v : c->prof.kern_ms) v = 0.0;
    for (long long& v : c->prof.kern_n) v = 0;
    return MPH_OK;
}

int case_profile_read(mph_case* c, double* out, int n)
{
    MPH_TRY(prof_collect(c));
    std::vector<double> v;
    for (int k = 0; k < 7; ++k) v.push_back(c->prof.stage_ms[k]);
    for (int k = 0; k < kProfKernels; ++k) v.push_back(c->prof.kern_ms[k]);
    for (int k = 0; k < kProfKernels; ++k) v.push_back((double)c->prof.kern_n[k]);
    v.push_back((double)c->nslots);
    v.push_back((double)c->nnb);
    v.push_back((double)c->nnbP);
    for (int k = 0; k < n && k < (int)v.size(); ++k) out[k] = v[k];
    return (int)v.size();
}

}  // namespace mph
