// mph_oracle.cpp - CPU oracle of the MPH-I implicit time step.
//
// TEST INFRASTRUCTURE ONLY: a restatement of the reference algorithm
// (MphImplicit source/main.cpp) in plain C++, used as the checker of the GPU
// engine and as the CPU baseline.  The shipped library never links it.
//
// Every stage cites the reference function it follows.  Floating-point
// expressions keep the reference's operation order (and the build uses
// -ffp-contract=off), so with one thread the results are bit-identical to the
// reference's OpenMP build run with one thread.  Vectors are stored with three
// components and matrix blocks as 3x3 also in 2D, as in the reference (DIM is
// always 3 there, main.cpp:49); 2D differs only in constants.
#include "mph_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int D = 3;             // storage components (reference DIM)
constexpr int kFluidEnd = 2;     // types [0,2) fluid, [2,4) wall (main.cpp:52-56)
constexpr int kWallBegin = 2;
constexpr int kWallEnd = 4;

inline bool is_wall(int t) { return kWallBegin <= t && t < kWallEnd; }
inline bool is_fluid(int t) { return 0 <= t && t < kFluidEnd; }

struct Level {
    int mn[3], mx[3], cnt[3];
    int cells, rows, width, st[3];     // st = stencil extent min(3, cnt)
    std::vector<double> cof;           // [rows][width]
    std::vector<double> invd;          // [rows]
    std::vector<double> q, s, r;       // V-cycle vectors [rows]
};

struct Case {
    bool two_d = false;
    mph_params prm{};
    double time = 0, dt = 0, l0 = 0, vol = 0;
    double dmin[3]{}, dmax[3]{}, dw[3]{};
    int N = 0, nPow = 0, powExp = 0;
    double rA = 0, rG = 0, rP = 0, rV = 0, maxR = 0;
    double Swa = 1, Swg = 1, Swp = 1, Swv = 1, N0a = 1, N0p = 1, R2g = 1, cofK = 0, cofA[4]{};
    double wallC[4][3]{}, wallV[4][3]{}, wallW[4][3]{}, wallR[4][3][3]{};
    int cc[3]{}, T = 0;
    double cw[3]{};
    int fB = 0, fE = 0, wB = 0, wE = 0;

    std::vector<int> id, type;
    std::vector<double> pos, vel, force, mass, kappa, lambda, mu;
    std::vector<double> densA, gcen, presA, vsp, divP, presP, virP, virS;
    std::vector<int> key, perm, cfb, cfe, cwb, cwe;
    std::vector<int> nc, nfc, ncp, nind, nindP;
    std::vector<long> nptr, nptrP;
    std::vector<long> aptr, cptr;
    std::vector<int> aind, cind;
    std::vector<double> aval, bvec, cval, pvec, invDiag;
    int depth = 0;
    std::vector<Level> lv;
    int iters = 0;
    double rr0 = 0, rr = 0, rs0 = 0, rs = 0;
    double tol2 = 1.0e-12;   // CR stop test rr/rr0 < tol2 (main.cpp:4346 has the constant 1e-12)
    std::vector<double> tmpd;
};

// ---- weight functions (main.cpp:236-307) ------------------------------------
// The reference writes e.g. `1.0/Swa * 1.0/(h*h) * (r/h)*...`, evaluated left
// to right: ((1/Sw)*1)/(h^DIM) first, then the polynomial factors.
inline double kfac(const Case& c, double Sw, double h)
{
    return c.two_d ? (1.0 / Sw) / (h * h) : (1.0 / Sw) / (h * h * h);
}
inline double w_a(const Case& c, double r, double h)
{
    const double q = r / h;
    return kfac(c, c.Swa, h) * q * (1.0 - q) * (1.0 - q);
}
inline double dw_a(const Case& c, double r, double h)
{
    const double q = r / h;
    return kfac(c, c.Swa, h) * (1.0 - q) * (1.0 - 3.0 * q) * (1.0 / h);
}
inline double w_quad(const Case& c, double Sw, double r, double h)   // wg, wp, wv
{
    const double q = r / h;
    return kfac(c, Sw, h) * ((1.0 - q) * (1.0 - q));
}
inline double dw_quad(const Case& c, double Sw, double r, double h)  // dwgdr, dwpdr, dwvdr
{
    const double q = r / h;
    return kfac(c, Sw, h) * (-2.0 / h * (1.0 - q));
}

// minimum-image separation x_j - x_i (the Mod(...) expression used in every
// pair loop, e.g. main.cpp:1452)
inline double fmodw(double x, double w) { return x - w * std::floor(x / w); }
inline void sep(const Case& c, int i, int j, double q[3])
{
    for (int d = 0; d < D; ++d) {
        const double hw = 0.5 * c.dw[d];
        q[d] = fmodw(c.pos[3 * j + d] - c.pos[3 * i + d] + hw, c.dw[d]) - hw;
    }
}
inline double norm2(const double q[3]) { return q[0] * q[0] + q[1] * q[1] + q[2] * q[2]; }

// ---- initialisation (main.cpp:886-1162) -----------------------------------
void init_weights(Case& c)
{
    c.rA = c.prm.radius_ratio_a * c.l0;
    c.rG = c.prm.radius_ratio_a * c.l0;   // RadiusRatioG = RadiusRatioA (main.cpp:888)
    c.rP = c.prm.radius_ratio_p * c.l0;
    c.rV = c.prm.radius_ratio_v * c.l0;
    const double l0 = c.l0;
    if (c.two_d) {
        c.Swa = 1.0 / 2.0 * 2.0 / 15.0 * M_PI / l0 / l0;
        c.Swg = 1.0 / 2.0 * 1.0 / 3.0 * M_PI / l0 / l0;
        c.Swp = c.Swg;
        c.Swv = c.Swg;
        c.R2g = 1.0 / 2.0 * 1.0 / 30.0 * M_PI * c.rG * c.rG / l0 / l0 / c.Swg;
    } else {
        c.Swa = 1.0 / 3.0 * 1.0 / 5.0 * M_PI / l0 / l0 / l0;
        c.Swg = 1.0 / 3.0 * 2.0 / 5.0 * M_PI / l0 / l0 / l0;
        c.Swp = c.Swg;
        c.Swv = c.Swg;
        c.R2g = 1.0 / 3.0 * 4.0 / 105.0 * M_PI * c.rG * c.rG / l0 / l0 / l0 / c.Swg;
    }
    // lattice sums N0a, N0p (main.cpp:911-980)
    auto lattice_sum = [&](double radius, bool use_a) {
        const int range = (int)std::ceil(radius / l0);
        const int rz = c.two_d ? 0 : range;
        double sum = 0.0;
        for (int ix = -range; ix <= range; ++ix)
            for (int iy = -range; iy <= range; ++iy)
                for (int iz = -rz; iz <= rz; ++iz) {
                    if (ix == 0 && iy == 0 && iz == 0) continue;
                    const double x = l0 * (double)ix, y = l0 * (double)iy, z = l0 * (double)iz;
                    const double r2 = x * x + y * y + z * z;
                    if (r2 <= radius * radius) {
                        const double r = std::sqrt(r2);
                        sum += use_a ? w_a(c, r, radius) : w_quad(c, c.Swp, r, radius);
                    }
                }
        return sum;
    };
    c.N0a = lattice_sum(c.rA, true);
    c.N0p = lattice_sum(c.rP, false);
}

void init_fluid(Case& c)   // main.cpp:988-1021
{
    for (int i = 0; i < c.N; ++i) {
        const int t = c.type[i];
        c.mass[i] = c.prm.density[t] * c.vol;
        c.kappa[i] = c.prm.bulk_modulus[t];
        c.lambda[i] = c.prm.bulk_viscosity[t];
        c.mu[i] = c.prm.shear_viscosity[t];
    }
    double integN, integX;
    if (c.two_d) { c.cofK = 0.350778153; integN = 0.024679383; integX = 0.226126699; }
    else         { c.cofK = 0.326976006; integN = 0.021425779; integX = 0.233977488; }
    for (int t = 0; t < 4; ++t)
        c.cofA[t] = c.prm.surface_tension[t] / ((c.rG / c.l0) * (integN + c.cofK * c.cofK * integX));
}

void init_wall(Case& c)    // main.cpp:1023-1062 (theta = |omega|^2 as written there)
{
    for (int t = kWallBegin; t < kWallEnd; ++t) {
        const double* w = c.wallW[t];
        const double theta = std::fabs(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        double n[3] = {0.0, 0.0, 0.0};
        if (theta != 0.0)
            for (int d = 0; d < 3; ++d) n[d] = w[d] / theta;
        const double s = std::sin(theta * c.dt / 2.0), co = std::cos(theta * c.dt / 2.0);
        const double q0 = n[0] * s, q1 = n[1] * s, q2 = n[2] * s, q3 = co;
        double (&R)[3][3] = c.wallR[t];
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
}

void init_domain(Case& c)  // main.cpp:1064-1111
{
    c.maxR = 0.0;
    c.maxR = std::max(c.maxR, c.rA);
    c.maxR = std::max(c.maxR, 2.0 * c.rP);
    c.maxR = std::max(c.maxR, c.rV);
    for (int d = 0; d < 3; ++d) c.dw[d] = c.dmax[d] - c.dmin[d];
    double cnt[3];
    cnt[0] = std::floor((c.dmax[0] - c.dmin[0]) / c.maxR);
    cnt[1] = std::floor((c.dmax[1] - c.dmin[1]) / c.maxR);
    cnt[2] = c.two_d ? 1.0 : std::floor((c.dmax[2] - c.dmin[2]) / c.maxR);
    for (int d = 0; d < 3; ++d) c.cc[d] = (int)cnt[d];
    c.T = (int)(cnt[0] * cnt[1] * cnt[2]);
    for (int d = 0; d < 3; ++d) c.cw[d] = c.dw[d] / c.cc[d];
    c.cfb.assign(c.T, 0); c.cfe.assign(c.T, 0); c.cwb.assign(c.T, 0); c.cwe.assign(c.T, 0);
    c.powExp = 0;
    while ((c.N >> c.powExp) != 0) ++c.powExp;
    c.nPow = 1 << c.powExp;
    c.key.assign(c.nPow, 0);
    c.perm.assign(c.nPow, 0);
}

inline int wrapc(int i, int n) { return (i % n + n) % n; }
inline int cell_id(const Case& c, int x, int y, int z)
{
    return wrapc(x, c.cc[0]) * c.cc[1] * c.cc[2] + wrapc(y, c.cc[1]) * c.cc[2] + wrapc(z, c.cc[2]);
}

// ---- cell list: key, bitonic network, ranges, permutation (main.cpp:1164-1379)
void cellsort(Case& c)
{
    const int N = c.N, T = c.T;
#pragma omp parallel for
    for (int i = 0; i < c.nPow; ++i) {
        if (i < N) {
            int ic[3];
            for (int d = 0; d < 3; ++d)
                ic[d] = ((int)std::floor((c.pos[3 * i + d] - c.dmin[d]) / c.cw[d])) % c.cc[d];
            c.key[i] = cell_id(c, ic[0], ic[1], ic[2]) + (is_wall(c.type[i]) ? T : 0);
            c.perm[i] = i;
        } else {
            c.key[i] = 2 * T;
            c.perm[i] = N;
        }
    }
    // the reference's bitonic compare-exchange network, stage by stage
    for (int m = 0; m < c.powExp; ++m) {
        for (int s = 0; s <= m; ++s) {
            const int dist = 1 << (m - s);
#pragma omp parallel for
            for (int i = 0; i < c.nPow; ++i) {
                if (i & dist) continue;
                const bool ascending = ((i >> m) & 2) == 0;
                const int j = i | dist;
                if ((c.key[i] > c.key[j]) == ascending) {
                    std::swap(c.key[i], c.key[j]);
                    std::swap(c.perm[i], c.perm[j]);
                }
            }
        }
    }
    // per-cell counts from key boundaries, then inclusive prefix sums over the
    // fluid cells followed by the wall cells (main.cpp:1214-1300)
    std::vector<long> cnt(2 * (size_t)T, 0);
    for (int i = 0; i < N; ++i) {
        const int k = c.key[i];
        if (k < 2 * T) cnt[k]++;
    }
    long run = 0;
    std::vector<long> incl(2 * (size_t)T);
    for (int k = 0; k < 2 * T; ++k) { run += cnt[k]; incl[k] = run; }
    for (int ic = 0; ic < T; ++ic) {
        c.cfb[ic] = ic == 0 ? 0 : (int)incl[ic - 1];
        c.cfe[ic] = (int)incl[ic];
        c.cwb[ic] = (int)incl[ic - 1 + T];
        c.cwe[ic] = (int)incl[ic + T];
    }
    c.fB = c.cfb[0];
    c.fE = c.cfe[T - 1];
    c.wB = c.cwb[0];
    c.wE = c.cwe[T - 1];
    // gather the particle state into cell order (main.cpp:1316-1378)
    std::vector<int> ti(N);
    std::vector<double> td(3 * (size_t)N);
    for (int i = 0; i < N; ++i) ti[i] = c.id[c.perm[i]];
    c.id.swap(ti);
    for (int i = 0; i < N; ++i) ti[i] = c.type[c.perm[i]];
    c.type.swap(ti);
    for (int i = 0; i < N; ++i) for (int d = 0; d < 3; ++d) td[3 * i + d] = c.pos[3 * c.perm[i] + d];
    c.pos.swap(td);
    for (int i = 0; i < N; ++i) for (int d = 0; d < 3; ++d) td[3 * i + d] = c.vel[3 * c.perm[i] + d];
    c.vel.swap(td);
}

// ---- neighbour lists (main.cpp:1382-1667) ----------------------------------
// Cells are visited in ascending index order along each axis (the rotated
// start jXmin of the reference), fluid cells first, then wall cells, so every
// list is ascending within its fluid part and within its wall part.
struct CellWalk {
    int n[3], lo[3], cells[3][3];
};
inline void cell_walk(const Case& c, int i, int range[3], CellWalk& w)
{
    const int k = c.key[i];
    const int ic[3] = {(k / (c.cc[1] * c.cc[2])) % c.T, (k / c.cc[2]) % c.cc[1], k % c.cc[2]};
    for (int d = 0; d < 3; ++d) {
        w.n[d] = 2 * range[d] + 1;
        for (int j = 0; j < w.n[d]; ++j) w.cells[d][j] = wrapc(ic[d] - range[d] + j, c.cc[d]);
        const int b = 2 * range[d] - (ic[d] + range[d]) % c.cc[d];
        w.lo[d] = b > 0 ? b : 0;
    }
}
template <class F>
inline void visit_cells(const Case& c, const CellWalk& w, F&& f)
{
    for (int jx = w.lo[0]; jx < w.lo[0] + w.n[0]; ++jx)
        for (int jy = w.lo[1]; jy < w.lo[1] + w.n[1]; ++jy)
            for (int jz = w.lo[2]; jz < w.lo[2] + w.n[2]; ++jz)
                f(cell_id(c, w.cells[0][jx % w.n[0]], w.cells[1][jy % w.n[1]], w.cells[2][jz % w.n[2]]));
}

void neighbors(Case& c)
{
    const int N = c.N;
    int range[3] = {(int)std::ceil(c.maxR / c.cw[0]), (int)std::ceil(c.maxR / c.cw[1]),
                    c.two_d ? 0 : (int)std::ceil(c.maxR / c.cw[2])};
    c.nc.assign(N, 0); c.nfc.assign(N, 0); c.ncp.assign(N, 0);
    const double R2 = c.maxR * c.maxR, P2 = c.rP * c.rP;
    // count pass
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
        CellWalk w;
        cell_walk(c, i, range, w);
        int n = 0, nf = 0, np = 0;
        visit_cells(c, w, [&](int jc) {
            for (int j = c.cfb[jc]; j < c.cfe[jc]; ++j) {
                double q[3];
                sep(c, i, j, q);
                const double r2 = norm2(q);
                if (r2 <= R2) { ++n; ++nf; if (r2 <= P2) ++np; }
            }
        });
        if (!(c.wB <= i && i < c.wE && n == 0)) {
            visit_cells(c, w, [&](int jc) {
                for (int j = c.cwb[jc]; j < c.cwe[jc]; ++j) {
                    double q[3];
                    sep(c, i, j, q);
                    const double r2 = norm2(q);
                    if (r2 <= R2) { ++n; if (r2 <= P2) ++np; }
                }
            });
        }
        c.nc[i] = n; c.nfc[i] = nf; c.ncp[i] = np;
    }
    c.nptr.assign(N + 1, 0);
    c.nptrP.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) { c.nptr[i + 1] = c.nptr[i] + c.nc[i]; c.nptrP[i + 1] = c.nptrP[i] + c.ncp[i]; }
    c.nind.assign(c.nptr[N], 0);
    c.nindP.assign(c.nptrP[N], 0);
    // fill pass
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
        CellWalk w;
        cell_walk(c, i, range, w);
        long o = c.nptr[i], op = c.nptrP[i];
        auto take = [&](int j) {
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 <= R2) { c.nind[o++] = j; if (r2 <= P2) c.nindP[op++] = j; }
        };
        visit_cells(c, w, [&](int jc) { for (int j = c.cfb[jc]; j < c.cfe[jc]; ++j) take(j); });
        if (!(c.wB <= i && i < c.wE && c.nc[i] == 0))
            visit_cells(c, w, [&](int jc) { for (int j = c.cwb[jc]; j < c.cwe[jc]; ++j) take(j); });
    }
}

// ---- explicit physics (main.cpp:1678-2128, 4741-4752) ---------------------
void step_begin(Case& c)
{
    const double dt = c.dt;
    for (int i = c.fB; i < c.fE; ++i)        // calculateConvection
        for (int d = 0; d < 3; ++d) c.pos[3 * i + d] += c.vel[3 * i + d] * dt;
    for (int i = c.wB; i < c.wE; ++i)        // calculateWall
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] = 0.0;
    for (int i = c.wB; i < c.wE; ++i) {
        const int t = c.type[i];
        const double (&R)[3][3] = c.wallR[t];
        const double* w = c.wallW[t];
        double r[3] = {c.pos[3 * i] - c.wallC[t][0], c.pos[3 * i + 1] - c.wallC[t][1], c.pos[3 * i + 2] - c.wallC[t][2]};
        // rotated in place, component by component, as the reference does
        r[0] = R[0][0] * r[0] + R[0][1] * r[1] + R[0][2] * r[2];
        r[1] = R[1][0] * r[0] + R[1][1] * r[1] + R[1][2] * r[2];
        r[2] = R[2][0] * r[0] + R[2][1] * r[1] + R[2][2] * r[2];
        c.vel[3 * i + 0] = w[1] * r[2] - w[2] * r[1] + c.wallV[t][0];
        c.vel[3 * i + 1] = w[2] * r[0] - w[0] * r[2] + c.wallV[t][1];
        c.vel[3 * i + 2] = w[0] * r[1] - w[1] * r[0] + c.wallV[t][2];
        for (int d = 0; d < 3; ++d) c.pos[3 * i + d] = r[d] + c.wallC[t][d] + c.wallV[t][d] * dt;
    }
    for (int t = kWallBegin; t < kWallEnd; ++t)
        for (int d = 0; d < 3; ++d) c.wallC[t][d] += c.wallV[t][d] * dt;
    for (int i = 0; i < c.N; ++i)            // calculatePeriodicBoundary
        for (int d = 0; d < 3; ++d)
            c.pos[3 * i + d] = fmodw(c.pos[3 * i + d] - c.dmin[d], c.dw[d]) + c.dmin[d];
    std::fill(c.force.begin(), c.force.end(), 0.0);   // resetForce
}

void density_a(Case& c)        // calculateDensityA main.cpp:1737
{
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        double sum = 0.0;
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            const double ratio = c.prm.interaction_ratio[c.type[i]][c.type[j]];
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (c.rA * c.rA - r2 >= 0) sum += ratio * w_a(c, std::sqrt(r2), c.rA);
        }
        c.densA[i] = sum;
    }
}

void gravity_center(Case& c)   // calculateGravityCenter main.cpp:1767
{
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        double s[3] = {0.0, 0.0, 0.0};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            const double ratio = c.prm.interaction_ratio[c.type[i]][c.type[j]];
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (c.rG * c.rG - r2 >= 0) {
                const double w = ratio * w_quad(c, c.Swg, std::sqrt(r2), c.rG);
                for (int d = 0; d < 3; ++d) s[d] += q[d] * w / c.R2g * c.rG;
            }
        }
        for (int d = 0; d < 3; ++d) c.gcen[3 * i + d] = s[d];
    }
}

void density_p(Case& c)        // calculateDensityP main.cpp:1903
{
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        double sum = 0.0;
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (c.rP * c.rP - r2 >= 0) sum += w_quad(c, c.Swp, std::sqrt(r2), c.rP);
        }
        c.vsp[i] = sum - c.N0p;
    }
}

void coefficients(Case& c)     // calculatePhysicalCoefficients main.cpp:1704
{
    for (int i = 0; i < c.N; ++i) {
        const int t = c.type[i];
        c.mass[i] = c.prm.density[t] * c.vol;
        c.kappa[i] = c.vsp[i] < 0.0 ? 0.0 : c.prm.bulk_modulus[t];
        c.lambda[i] = c.prm.bulk_viscosity[t];
        c.mu[i] = c.prm.shear_viscosity[t];
    }
}

void pressure_a(Case& c)       // calculatePressureA main.cpp:1801
{
    for (int i = 0; i < c.N; ++i) {
        c.presA[i] = c.cofA[c.type[i]] * (c.densA[i] - c.N0a) / c.l0;
        if (c.N0a <= c.densA[i]) c.presA[i] = 0.0;
    }
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        double f[3] = {0.0, 0.0, 0.0};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            const double rij_ = c.prm.interaction_ratio[c.type[i]][c.type[j]];
            const double rji_ = c.prm.interaction_ratio[c.type[j]][c.type[i]];
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rA * c.rA - r2 > 0) {
                const double r = std::sqrt(r2);
                const double dwij = rij_ * dw_a(c, r, c.rA);
                const double dwji = rji_ * dw_a(c, r, c.rA);
                const double e[3] = {q[0] / r, q[1] / r, q[2] / r};
                for (int d = 0; d < 3; ++d) f[d] += (c.presA[i] * dwij + c.presA[j] * dwji) * e[d] * c.vol;
            }
        }
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] += f[d];
    }
}

void diffuse_interface(Case& c)   // calculateDiffuseInterface main.cpp:1851
{
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        // both coefficients use particle i's type, as in the reference (main.cpp:1857, 1863)
        const double ai = c.cofA[c.type[i]] * (c.cofK) * (c.cofK);
        const double aj = ai;
        double f[3] = {0.0, 0.0, 0.0};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            const double rij_ = c.prm.interaction_ratio[c.type[i]][c.type[j]];
            const double rji_ = c.prm.interaction_ratio[c.type[j]][c.type[i]];
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rG * c.rG - r2 > 0) {
                const double r = std::sqrt(r2);
                const double wij = rij_ * w_quad(c, c.Swg, r, c.rG);
                const double wji = rji_ * w_quad(c, c.Swg, r, c.rG);
                const double* gi = &c.gcen[3 * i];
                const double* gj = &c.gcen[3 * j];
                for (int d = 0; d < 3; ++d)
                    f[d] -= (aj * gj[d] * wji - ai * gi[d] * wij) / c.R2g * c.rG * (c.vol / c.l0);
                const double dwij = rij_ * dw_quad(c, c.Swg, r, c.rG);
                const double dwji = rji_ * dw_quad(c, c.Swg, r, c.rG);
                const double e[3] = {q[0] / r, q[1] / r, q[2] / r};
                double gr = 0.0;
                for (int d = 0; d < 3; ++d) gr += (aj * gj[d] * dwji - ai * gi[d] * dwij) * q[d];
                for (int d = 0; d < 3; ++d) f[d] -= (gr)*e[d] / c.R2g * c.rG * (c.vol / c.l0);
            }
        }
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] += f[d];
    }
}

void explicit_stage(Case& c)   // main.cpp:413-430
{
    density_a(c);
    gravity_center(c);
    density_p(c);
    coefficients(c);
    pressure_a(c);
    diffuse_interface(c);
    for (int i = c.fB; i < c.fE; ++i)          // calculateGravity main.cpp:2065
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] += c.mass[i] * c.prm.gravity[d];
    for (int i = c.fB; i < c.fE; ++i)          // calculateAcceleration main.cpp:2076
        for (int d = 0; d < 3; ++d) c.vel[3 * i + d] += c.force[3 * i + d] / c.mass[i] * c.dt;
}

// ---- implicit system (main.cpp:2137-2643) ---------------------------------
void assemble(Case& c)
{
    const int nf = c.fE - c.fB;
    const long rows = (long)D * nf;
    // pattern of A: DIM x DIM block per (fluid i, fluid neighbour j)
    c.aptr.assign(rows + 1, 0);
    for (int i = 0; i < nf; ++i)
        for (int r = 0; r < D; ++r) c.aptr[D * i + r + 1] = (long)D * c.nfc[i];
    for (long k = 0; k < rows; ++k) c.aptr[k + 1] += c.aptr[k];
    c.aind.assign(c.aptr[rows], 0);
    c.aval.assign(c.aptr[rows], 0.0);
    c.bvec.assign(rows, 0.0);
#pragma omp parallel for
    for (int i = 0; i < nf; ++i)
        for (int jn = 0; jn < c.nfc[i]; ++jn) {
            const int j = c.nind[c.nptr[i] + jn];
            for (int r = 0; r < D; ++r)
                for (int s = 0; s < D; ++s) c.aind[c.aptr[D * i + r] + D * jn + s] = D * j + s;
        }
    const double visc = c.two_d ? 8.0 : 10.0;
    // viscous + inertia terms (calculateMatrixA main.cpp:2251-2335)
#pragma omp parallel for
    for (int i = c.fB; i < c.fE; ++i) {
        int self = 0;
        double selfCof[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double sumvec[3] = {0, 0, 0};
        for (int jn = 0; jn < c.nc[i]; ++jn) {
            const int j = c.nind[c.nptr[i] + jn];
            if (i == j) { self = jn; continue; }
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rV * c.rV - r2 > 0) {
                const double dij = std::sqrt(r2);
                const double wd = -dw_quad(c, c.Swv, dij, c.rV);
                const double e[3] = {q[0] / dij, q[1] / dij, q[2] / dij};
                const double muij = 2.0 * (c.mu[i] * c.mu[j]) / (c.mu[i] + c.mu[j]);
                for (int r = 0; r < D; ++r)
                    for (int s = 0; s < D; ++s) {
                        const double coef = +visc * muij * e[s] * e[r] * wd / dij;
                        selfCof[r][s] += coef;
                        if (is_fluid(c.type[j])) c.aval[c.aptr[D * i + r] + D * jn + s] = -coef;
                        else if (is_wall(c.type[j])) sumvec[r] += coef * c.vel[3 * j + s];
                    }
            }
        }
        for (int r = 0; r < D; ++r)
            for (int s = 0; s < D; ++s) c.aval[c.aptr[D * i + r] + D * self + s] = selfCof[r][s];
        for (int r = 0; r < D; ++r) c.bvec[D * i + r] += sumvec[r];
        for (int d = 0; d < D; ++d) {
            const double coef = c.mass[i] / c.vol / c.dt;
            c.aval[c.aptr[D * i + d] + D * self + d] += coef;
            c.bvec[D * i + d] += coef * c.vel[3 * i + d];
        }
    }
    // C and source p (calculateMatrixC main.cpp:2354-2551)
    c.cptr.assign(rows + 1, 0);
    for (int i = 0; i < nf; ++i)
        for (int r = 0; r < D; ++r) c.cptr[D * i + r + 1] = c.ncp[i];
    for (long k = 0; k < rows; ++k) c.cptr[k + 1] += c.cptr[k];
    c.cind.assign(c.cptr[rows], 0);
    c.cval.assign(c.cptr[rows], 0.0);
    c.pvec.assign(c.N, 0.0);
#pragma omp parallel for
    for (int i = 0; i < nf; ++i) {
        int self = 0;
        double selfCof[3] = {0, 0, 0};
        for (int jn = 0; jn < c.ncp[i]; ++jn) {
            const int j = c.nindP[c.nptrP[i] + jn];
            for (int r = 0; r < D; ++r) c.cind[c.cptr[D * i + r] + jn] = j;
            if (i == j) { self = jn; continue; }
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rP * c.rP - r2 > 0) {
                const double dij = std::sqrt(r2);
                const double e[3] = {q[0] / dij, q[1] / dij, q[2] / dij};
                const double wd = -dw_quad(c, c.Swp, dij, c.rP);
                for (int r = 0; r < D; ++r) {
                    const double coef = e[r] * wd;
                    selfCof[r] += coef;
                    c.cval[c.cptr[D * i + r] + jn] = coef;
                }
            }
        }
        for (int r = 0; r < D; ++r) c.cval[c.cptr[D * i + r] + self] = selfCof[r];
    }
#pragma omp parallel for
    for (int i = 0; i < c.N; ++i) {
        double p = 0.0;
        if (c.vsp[i] > 0.0) p = c.kappa[i] * c.vsp[i];
        double sum = 0.0;
        for (int jn = 0; jn < c.ncp[i]; ++jn) {
            const int j = c.nindP[c.nptrP[i] + jn];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rP * c.rP - r2 > 0) {
                const double dij = std::sqrt(r2);
                const double e[3] = {q[0] / dij, q[1] / dij, q[2] / dij};
                const double wd = -dw_quad(c, c.Swp, dij, c.rP);
                for (int s = 0; s < D; ++s) {
                    if (is_wall(c.type[i])) sum += c.lambda[i] * (+e[s] * wd) * c.vel[3 * i + s];
                    if (is_wall(c.type[j])) sum += c.lambda[i] * (-e[s] * wd) * c.vel[3 * j + s];
                }
            }
        }
        c.pvec[i] = p + sum;
    }
    // b -= C p ; A += C Lambda C^T (multiplyMatrixC main.cpp:2562-2643)
#pragma omp parallel for
    for (long row = 0; row < rows; ++row)
        for (long k = c.cptr[row]; k < c.cptr[row + 1]; ++k) c.bvec[row] -= c.cval[k] * c.pvec[c.cind[k]];
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < nf; ++i) {
        for (int jn = 0; jn < c.nfc[i]; ++jn) {
            const int j = c.nind[c.nptr[i] + jn];
            double sum[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            int a = 0, b = 0;
            const int* li = &c.nindP[c.nptrP[i]];
            const int* lj = &c.nindP[c.nptrP[j]];
            while (a < c.ncp[i] && b < c.ncp[j]) {
                if (li[a] == lj[b]) {
                    const int k = li[a];
                    for (int r = 0; r < D; ++r)
                        for (int s = 0; s < D; ++s)
                            sum[r][s] += c.cval[c.cptr[D * i + r] + a] * c.lambda[k] * c.cval[c.cptr[D * j + s] + b];
                    ++a; ++b;
                } else if (li[a] < lj[b]) {
                    ++a;
                } else {
                    ++b;
                }
            }
            for (int r = 0; r < D; ++r)
                for (int s = 0; s < D; ++s) c.aval[c.aptr[D * i + r] + D * jn + s] += sum[r][s];
        }
    }
}

// ---- multigrid hierarchy (main.cpp:2761-3546) ------------------------------
inline int grid_id(const int cnt[3], int x, int y, int z) { return (cnt[1] * cnt[2]) * x + cnt[2] * y + z; }

void mg_build(Case& c)
{
    // depth from the fluid-cell bounding box (calculateMultiGridDepth main.cpp:2777)
    int mx[3] = {0, 0, 0}, mn[3] = {c.cc[0], c.cc[1], c.cc[2]};
    for (int ic = 0; ic < c.T; ++ic) {
        if (c.cfe[ic] - c.cfb[ic] > 0) {
            const int p[3] = {(ic / (c.cc[1] * c.cc[2])) % c.cc[0], (ic / c.cc[2]) % c.cc[1], ic % c.cc[2]};
            for (int d = 0; d < 3; ++d) { mx[d] = std::max(mx[d], p[d]); mn[d] = std::min(mn[d], p[d]); }
        }
    }
    double maxCount = 0.0;
    for (int d = 0; d < 3; ++d)   // reproduces the reference's update rule (main.cpp:2804-2813)
        if ((mx[d] - mn[d]) > maxCount) maxCount = (mx[d] - mn[d] + 1);
    int p = 0;
    while ((1 << p) <= maxCount) ++p;
    c.depth = p;
    c.lv.assign(c.depth, Level());
    for (int L = 0; L < c.depth; ++L) {
        Level& l = c.lv[L];
        l.cells = 1;
        for (int d = 0; d < 3; ++d) {
            l.mn[d] = mn[d] >> L;
            l.mx[d] = (mx[d] >> L) + 1;
            l.cnt[d] = l.mx[d] - l.mn[d];
            l.st[d] = std::min(3, l.cnt[d]);
            l.cells *= l.cnt[d];
        }
        l.rows = D * l.cells;
        l.width = D * l.st[0] * l.st[1] * l.st[2];
        l.cof.assign((size_t)l.rows * l.width, 0.0);
        l.invd.assign(l.rows, 0.0);
        l.q.assign(l.rows, 0.0); l.s.assign(l.rows, 0.0); l.r.assign(l.rows, 0.0);
    }
    if (c.depth < 2) return;   // the reference indexes level depth-2 unconditionally
    const int nf = c.fE - c.fB;
    // particle diagonal inverse (calculateInvDiagA main.cpp:3045)
    c.invDiag.assign((size_t)D * nf, 0.0);
#pragma omp parallel for
    for (long row = 0; row < (long)D * nf; ++row)
        for (long k = c.aptr[row]; k < c.aptr[row + 1]; ++k)
            if (c.aind[k] == row && c.aval[k] != 0.0) c.invDiag[row] = 1.0 / c.aval[k];
    // level 0: Galerkin sum of the particle rows of every cell (main.cpp:3336-3411)
    {
        Level& l = c.lv[0];
#pragma omp parallel for
        for (int rowG = 0; rowG < l.rows; ++rowG) {
            const int g = rowG / D, rD = rowG % D;
            const int gp[3] = {(g / (l.cnt[1] * l.cnt[2])) % l.cnt[0], (g / l.cnt[2]) % l.cnt[1], g % l.cnt[2]};
            double* out = &l.cof[(size_t)rowG * l.width];
            const int cx = gp[0] + l.mn[0], cy = gp[1] + l.mn[1], cz = gp[2] + l.mn[2];
            if (!(cx < c.cc[0] && cy < c.cc[1] && cz < c.cc[2])) continue;
            const int ic = cell_id(c, cx, cy, cz);
            for (int i = c.cfb[ic]; i < c.cfe[ic]; ++i) {
                const long row = (long)D * i + rD;
                for (long k = c.aptr[row]; k < c.aptr[row + 1]; ++k) {
                    const int col = c.aind[k], j = col / D, sD = col % D;
                    const int kj = c.key[j];
                    const int jc[3] = {(kj / (c.cc[1] * c.cc[2])) % c.T, (kj / c.cc[2]) % c.cc[1], kj % c.cc[2]};
                    int o[3];
                    for (int d = 0; d < 3; ++d) o[d] = ((jc[d] - l.mn[d]) - gp[d] + 1 + l.cnt[d]) % l.cnt[d];
                    out[D * (l.st[2] * l.st[1] * o[0] + l.st[2] * o[1] + o[2]) + sD] += c.aval[k];
                }
            }
        }
    }
    // coarser levels: restriction (sum of the 2^DIM children) of the finer
    // level's stencil rows, re-binned by parent cell (main.cpp:3414-3507)
    for (int L = 1; L < c.depth; ++L) {
        const Level& s = c.lv[L - 1];
        Level& l = c.lv[L];
#pragma omp parallel for
        for (int rowL = 0; rowL < l.rows; ++rowL) {
            const int g = rowL / D, rD = rowL % D;
            const int gp[3] = {(g / (l.cnt[1] * l.cnt[2])) % l.cnt[0], (g / l.cnt[2]) % l.cnt[1], g % l.cnt[2]};
            double* out = &l.cof[(size_t)rowL * l.width];
            int fm[3], fM[3];
            for (int d = 0; d < 3; ++d) {
                const int lc = gp[d] + l.mn[d];
                fm[d] = s.mn[d] > 2 * lc ? 1 : 0;
                fM[d] = s.mx[d] < 2 * (lc + 1) ? 1 : 0;
            }
            for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
                for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
                    for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                        const int sg = grid_id(s.cnt, 2 * (gp[0] + l.mn[0]) + dx - s.mn[0],
                                               2 * (gp[1] + l.mn[1]) + dy - s.mn[1],
                                               2 * (gp[2] + l.mn[2]) + dz - s.mn[2]);
                        const int rowS = D * sg + rD;
                        const int sgp[3] = {(sg / (s.cnt[1] * s.cnt[2])) % s.cnt[0], (sg / s.cnt[2]) % s.cnt[1], sg % s.cnt[2]};
                        const double* in = &s.cof[(size_t)rowS * s.width];
                        for (int ix = 0; ix < s.st[0]; ++ix)
                            for (int iy = 0; iy < s.st[1]; ++iy)
                                for (int iz = 0; iz < s.st[2]; ++iz)
                                    for (int sD = 0; sD < D; ++sD) {
                                        // fine column cell: periodic stencil neighbour of sg
                                        const int jf[3] = {(sgp[0] + ix - 1 + s.cnt[0]) % s.cnt[0],
                                                           (sgp[1] + iy - 1 + s.cnt[1]) % s.cnt[1],
                                                           (sgp[2] + iz - 1 + s.cnt[2]) % s.cnt[2]};
                                        int o[3];
                                        for (int d = 0; d < 3; ++d) {
                                            const int jl = (jf[d] + s.mn[d]) / 2 - l.mn[d];
                                            o[d] = (jl - gp[d] + 1 + l.cnt[d]) % l.cnt[d];
                                        }
                                        out[D * (l.st[2] * l.st[1] * o[0] + l.st[2] * o[1] + o[2]) + sD] +=
                                            in[D * (s.st[2] * s.st[1] * ix + s.st[2] * iy + iz) + sD];
                                    }
                    }
        }
    }
    // damped l1-Jacobi inverse diagonals (calculateMultiGridInvDiagA main.cpp:3510)
    for (int L = 0; L < c.depth; ++L) {
        Level& l = c.lv[L];
        for (int row = 0; row < l.rows; ++row) {
            double sum = 0.0;
            for (int k = 0; k < l.width; ++k) sum += std::fabs(l.cof[(size_t)row * l.width + k]);
            l.invd[row] = sum != 0.0 ? 2.0 / sum : 0.0;
        }
    }
}

// ---- V-cycle and conjugate residual (main.cpp:4015-4421) -------------------
// y = Q - A_L S  (the reference's csrmv with alpha=-1, beta=1)
void level_residual(const Level& l, const std::vector<double>& S, std::vector<double>& R)
{
#pragma omp parallel for
    for (int row = 0; row < l.rows; ++row) {
        const int g = row / D;
        const int gp[3] = {(g / (l.cnt[1] * l.cnt[2])) % l.cnt[0], (g / l.cnt[2]) % l.cnt[1], g % l.cnt[2]};
        const double* a = &l.cof[(size_t)row * l.width];
        double sum = 0.0;
        for (int ix = 0; ix < l.st[0]; ++ix)
            for (int iy = 0; iy < l.st[1]; ++iy)
                for (int iz = 0; iz < l.st[2]; ++iz) {
                    const int jg = grid_id(l.cnt, (gp[0] + ix - 1 + l.cnt[0]) % l.cnt[0],
                                           (gp[1] + iy - 1 + l.cnt[1]) % l.cnt[1],
                                           (gp[2] + iz - 1 + l.cnt[2]) % l.cnt[2]);
                    for (int sD = 0; sD < D; ++sD)
                        sum += (-1.0 * a[D * (l.st[2] * l.st[1] * ix + l.st[2] * iy + iz) + sD]) * S[D * jg + sD];
                }
        R[row] = l.q[row] + sum;
    }
}
void level_smooth_update(const Level& l, std::vector<double>& S, const std::vector<double>& R)
{
    for (int row = 0; row < l.rows; ++row) S[row] = S[row] + (1.0 * l.invd[row]) * R[row];
}
// restriction Q_L = R (R_{L-1}) in the reference's child order (main.cpp:3154-3174)
void restrict_to(const Level& s, Level& l)
{
    for (int row = 0; row < l.rows; ++row) {
        const int g = row / D, rD = row % D;
        const int gp[3] = {(g / (l.cnt[1] * l.cnt[2])) % l.cnt[0], (g / l.cnt[2]) % l.cnt[1], g % l.cnt[2]};
        int fm[3], fM[3];
        for (int d = 0; d < 3; ++d) {
            const int lc = gp[d] + l.mn[d];
            fm[d] = s.mn[d] > 2 * lc ? 1 : 0;
            fM[d] = s.mx[d] < 2 * (lc + 1) ? 1 : 0;
        }
        double sum = 0.0;
        for (int dx = fm[0]; dx < 2 - fM[0]; ++dx)
            for (int dy = fm[1]; dy < 2 - fM[1]; ++dy)
                for (int dz = fm[2]; dz < 2 - fM[2]; ++dz) {
                    const int sg = grid_id(s.cnt, 2 * (gp[0] + l.mn[0]) + dx - s.mn[0], 2 * (gp[1] + l.mn[1]) + dy - s.mn[1],
                                           2 * (gp[2] + l.mn[2]) + dz - s.mn[2]);
                    sum += (1.0 * 1.0) * s.r[D * sg + rD];
                }
        l.q[row] = 0.0 * l.q[row] + sum;
    }
}
// S_{L-1} += P S_L (injection to the children, main.cpp:3216-3240)
void prolong_to(const Level& l, Level& s)
{
    for (int row = 0; row < s.rows; ++row) {
        const int g = row / D, rD = row % D;
        const int gp[3] = {(g / (s.cnt[1] * s.cnt[2])) % s.cnt[0], (g / s.cnt[2]) % s.cnt[1], g % s.cnt[2]};
        const int lg = grid_id(l.cnt, (gp[0] + s.mn[0]) / 2 - l.mn[0], (gp[1] + s.mn[1]) / 2 - l.mn[1],
                               (gp[2] + s.mn[2]) / 2 - l.mn[2]);
        s.s[row] = s.s[row] + (1.0 * 1.0) * l.s[D * lg + rD];
    }
}

// u = M q (preconditionWithMultiGrid main.cpp:4122-4266)
void precondition(Case& c, const double* q, double* u)
{
    const int nf = c.fE - c.fB;
    const long n = (long)D * nf;
    for (long k = 0; k < n; ++k) u[k] = 0.0 * u[k] + (1.0 * c.invDiag[k]) * q[k];
    const int depth = c.depth;
    // level 0: Q0 = P2G q, then 2 smoothing sweeps
    {
        Level& l = c.lv[0];
        for (int row = 0; row < l.rows; ++row) {
            const int g = row / D, rD = row % D;
            const int gp[3] = {(g / (l.cnt[1] * l.cnt[2])) % l.cnt[0], (g / l.cnt[2]) % l.cnt[1], g % l.cnt[2]};
            const int ic = cell_id(c, gp[0] + l.mn[0], gp[1] + l.mn[1], gp[2] + l.mn[2]);
            double sum = 0.0;
            for (int i = c.cfb[ic]; i < c.cfe[ic]; ++i) sum += (1.0 * 1.0) * q[D * i + rD];
            l.q[row] = 0.0 * l.q[row] + sum;
        }
        std::fill(l.s.begin(), l.s.end(), 0.0);
        l.r = l.q;
        for (int it = 0; it < 2; ++it) { level_smooth_update(l, l.s, l.r); level_residual(l, l.s, l.r); }
    }
    for (int L = 1; L < depth - 1; ++L) {
        Level& l = c.lv[L];
        restrict_to(c.lv[L - 1], l);
        std::fill(l.s.begin(), l.s.end(), 0.0);
        l.r = l.q;
        for (int it = 0; it < 3; ++it) { level_smooth_update(l, l.s, l.r); level_residual(l, l.s, l.r); }
    }
    {
        Level& l = c.lv[depth - 1];
        restrict_to(c.lv[depth - 2], l);
        std::fill(l.s.begin(), l.s.end(), 0.0);
        l.r = l.q;
        for (int it = 0; it < 4; ++it) { level_smooth_update(l, l.s, l.r); level_residual(l, l.s, l.r); }
        level_smooth_update(l, l.s, l.r);
        prolong_to(l, c.lv[depth - 2]);
    }
    for (int L = depth - 2; L > 0; --L) {
        Level& l = c.lv[L];
        for (int it = 0; it < 3; ++it) { level_residual(l, l.s, l.r); level_smooth_update(l, l.s, l.r); }
        prolong_to(l, c.lv[L - 1]);
    }
    {
        Level& l = c.lv[0];
        for (int it = 0; it < 2; ++it) { level_residual(l, l.s, l.r); level_smooth_update(l, l.s, l.r); }
        // u += G2P S0 (injection from the particle's cell)
        for (int i = 0; i < nf; ++i) {
            const int k = c.key[i];
            const int cp[3] = {(k / (c.cc[1] * c.cc[2])) % c.cc[0], (k / c.cc[2]) % c.cc[1], k % c.cc[2]};
            const int g = grid_id(l.cnt, cp[0] - l.mn[0], cp[1] - l.mn[1], cp[2] - l.mn[2]);
            for (int rD = 0; rD < D; ++rD) u[D * i + rD] = u[D * i + rD] + (1.0 * 1.0) * l.s[D * g + rD];
        }
    }
}

double dot(long n, const double* x, const double* y)
{
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (long k = 0; k < n; ++k) sum += x[k] * y[k];
    return sum;
}
void spmv_a(const Case& c, double alpha, const double* x, double beta, double* y)
{
    const long n = (long)D * (c.fE - c.fB);
#pragma omp parallel for
    for (long row = 0; row < n; ++row) {
        double sum = 0.0;
        for (long k = c.aptr[row]; k < c.aptr[row + 1]; ++k) sum += alpha * c.aval[k] * x[c.aind[k]];
        y[row] *= beta;
        y[row] += sum;
    }
}

int solve(Case& c)   // solveWithConjugatedGradient main.cpp:4270-4421
{
    const int nf = c.fE - c.fB;
    const long n = (long)D * nf;
    std::vector<double> x(n), r(n), s(n), y(n), p(n), q(n), u(n);
    for (int i = 0; i < nf; ++i)
        for (int d = 0; d < D; ++d) x[D * i + d] = c.vel[3 * i + d] - c.force[3 * i + d] / c.mass[i] * c.dt;
    const double* b = c.bvec.data();
    if (c.depth < 2) return -1;
    precondition(c, b, s.data());
    c.rs0 = dot(n, b, s.data());
    c.rr0 = dot(n, b, b);
    for (long k = 0; k < n; ++k) r[k] = b[k];
    spmv_a(c, -1.0, x.data(), 1.0, r.data());
    precondition(c, r.data(), s.data());
    double rho = 1.0, rhop = 0.0;
    int it;
    for (it = 0; it < n; ++it) {
        c.rr = dot(n, r.data(), r.data());
        if (c.rr / c.rr0 < c.tol2) break;
        spmv_a(c, 1.0, s.data(), 0.0, y.data());
        rho = dot(n, s.data(), y.data());
        if (it == 0) {
            p = s;
            spmv_a(c, 1.0, p.data(), 0.0, q.data());
        } else {
            const double beta = rho / rhop;
            for (long k = 0; k < n; ++k) { p[k] *= beta; p[k] += 1.0 * s[k]; }
            for (long k = 0; k < n; ++k) { q[k] *= beta; q[k] += 1.0 * y[k]; }
        }
        precondition(c, q.data(), u.data());
        const double alpha = rho / dot(n, q.data(), u.data());
        for (long k = 0; k < n; ++k) x[k] += alpha * p[k];
        for (long k = 0; k < n; ++k) r[k] += -alpha * q[k];
        for (long k = 0; k < n; ++k) s[k] += -alpha * u[k];
        rhop = rho;
    }
    c.rr = dot(n, r.data(), r.data());
    c.rs = dot(n, r.data(), s.data());
    c.iters = it;
    for (int i = 0; i < nf; ++i)
        for (int d = 0; d < D; ++d) c.vel[3 * i + d] = x[D * i + d];
    return it;
}

// ---- output-step fields (main.cpp:1932-2063, 4494-4738) --------------------
void output_fields(Case& c)
{
    const int N = c.N;
    const double visc = c.two_d ? 8.0 : 10.0;
    for (int i = 0; i < N; ++i) {   // calculateDivergenceP
        double sum = 0.0;
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rP * c.rP - r2 >= 0) {
                const double r = std::sqrt(r2);
                const double dw = dw_quad(c, c.Swp, r, c.rP);
                const double e[3] = {q[0] / r, q[1] / r, q[2] / r};
                for (int d = 0; d < 3; ++d) sum -= (c.vel[3 * j + d] - c.vel[3 * i + d]) * e[d] * dw;
            }
        }
        c.divP[i] = sum;
    }
    for (int i = 0; i < N; ++i) {   // calculatePressureP
        c.presP[i] = -c.lambda[i] * c.divP[i];
        if (c.vsp[i] > 0.0) c.presP[i] += c.kappa[i] * c.vsp[i];
    }
    for (int i = 0; i < N; ++i) {
        double f[3] = {0, 0, 0};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rP * c.rP - r2 > 0) {
                const double r = std::sqrt(r2);
                const double dw = dw_quad(c, c.Swp, r, c.rP);
                const double g[3] = {dw * q[0] / r, dw * q[1] / r, dw * q[2] / r};
                for (int d = 0; d < 3; ++d) f[d] += (c.presP[i] + c.presP[j]) * g[d] * c.vol;
            }
        }
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] += f[d];
    }
    for (int i = 0; i < N; ++i) {   // calculateViscosityV
        double f[3] = {0, 0, 0};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rV * c.rV - r2 > 0) {
                const double r = std::sqrt(r2);
                const double dw = -dw_quad(c, c.Swv, r, c.rV);
                const double e[3] = {q[0] / r, q[1] / r, q[2] / r};
                const double u[3] = {c.vel[3 * j] - c.vel[3 * i], c.vel[3 * j + 1] - c.vel[3 * i + 1], c.vel[3 * j + 2] - c.vel[3 * i + 2]};
                const double muij = 2.0 * (c.mu[i] * c.mu[j]) / (c.mu[i] + c.mu[j]);
                for (int d = 0; d < 3; ++d)
                    f[d] += visc * muij * (u[0] * e[0] + u[1] * e[1] + u[2] * e[2]) * e[d] * dw / r * c.vol;
            }
        }
        for (int d = 0; d < 3; ++d) c.force[3 * i + d] += f[d];
    }
    // calculateVirialStressAtParticle main.cpp:4494-4738
    for (int i = 0; i < N; ++i) {
        double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int jn = 0; jn < c.ncp[i]; ++jn) {   // pressure P part over the P list
            const int j = c.nindP[c.nptrP[i] + jn];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rP * c.rP - r2 > 0) {
                const double r = std::sqrt(r2);
                const double dw = dw_quad(c, c.Swp, r, c.rP);
                const double g[3] = {dw * q[0] / r, dw * q[1] / r, dw * q[2] / r};
                double fij[3];
                for (int d = 0; d < 3; ++d) fij[d] = (c.presP[i]) * g[d] * c.vol;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) st[a][b] += 1.0 * fij[a] * q[b] / c.vol;
            }
        }
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) c.virS[9 * i + 3 * a + b] = 0.0 + st[a][b];
    }
    for (int i = 0; i < N; ++i) {   // pressure A part
        double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rA * c.rA - r2 > 0) {
                const double ratio = c.prm.interaction_ratio[c.type[i]][c.type[j]];
                const double r = std::sqrt(r2);
                const double dw = ratio * dw_a(c, r, c.rA);
                const double g[3] = {dw * q[0] / r, dw * q[1] / r, dw * q[2] / r};
                double fij[3];
                for (int d = 0; d < 3; ++d) fij[d] = (c.presA[i]) * g[d] * c.vol;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) st[a][b] += 1.0 * fij[a] * q[b] / c.vol;
            }
        }
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) c.virS[9 * i + 3 * a + b] += st[a][b];
    }
    for (int i = 0; i < N; ++i) {   // viscosity part
        double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rV * c.rV - r2 > 0) {
                const double r = std::sqrt(r2);
                const double dw = -dw_quad(c, c.Swv, r, c.rV);
                const double e[3] = {q[0] / r, q[1] / r, q[2] / r};
                const double v[3] = {c.vel[3 * j] - c.vel[3 * i], c.vel[3 * j + 1] - c.vel[3 * i + 1], c.vel[3 * j + 2] - c.vel[3 * i + 2]};
                const double muij = 2.0 * (c.mu[i] * c.mu[j]) / (c.mu[i] + c.mu[j]);
                double fij[3];
                for (int d = 0; d < 3; ++d)
                    fij[d] = visc * muij * (v[0] * e[0] + v[1] * e[1] + v[2] * e[2]) * e[d] * dw / r * c.vol;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) st[a][b] += 0.5 * fij[a] * q[b] / c.vol;
            }
        }
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) c.virS[9 * i + 3 * a + b] += st[a][b];
    }
    for (int i = 0; i < N; ++i) {   // diffuse-interface parts
        double st[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (long k = c.nptr[i]; k < c.nptr[i + 1]; ++k) {
            const int j = c.nind[k];
            if (i == j) continue;
            double q[3];
            sep(c, i, j, q);
            const double r2 = norm2(q);
            if (r2 == 0.0) continue;
            if (c.rG * c.rG - r2 > 0) {
                const double a = c.cofA[c.type[i]] * (c.cofK) * (c.cofK);
                const double ratio = c.prm.interaction_ratio[c.type[i]][c.type[j]];
                const double r = std::sqrt(r2);
                const double w = ratio * w_quad(c, c.Swg, r, c.rG);
                double fij[3];
                for (int d = 0; d < 3; ++d) fij[d] = -a * (-c.gcen[3 * i + d]) * w / c.R2g * c.rG * (c.vol / c.l0);
                for (int aa = 0; aa < 3; ++aa)
                    for (int b = 0; b < 3; ++b) st[aa][b] += 1.0 * fij[aa] * q[b] / c.vol;
            }
            if (c.rG * c.rG - r2 > 0.0) {
                const double a = c.cofA[c.type[i]] * (c.cofK) * (c.cofK);
                const double ratio = c.prm.interaction_ratio[c.type[i]][c.type[j]];
                const double r = std::sqrt(r2);
                const double dw = ratio * dw_quad(c, c.Swg, r, c.rG);
                const double g[3] = {dw * q[0] / r, dw * q[1] / r, dw * q[2] / r};
                double gr = 0.0;
                for (int d = 0; d < 3; ++d) gr += (-c.gcen[3 * i + d]) * q[d];
                double fij[3];
                for (int d = 0; d < 3; ++d) fij[d] = -a * (gr)*g[d] / c.R2g * c.rG * (c.vol / c.l0);
                for (int aa = 0; aa < 3; ++aa)
                    for (int b = 0; b < 3; ++b) st[aa][b] += 1.0 * fij[aa] * q[b] / c.vol;
            }
        }
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) c.virS[9 * i + 3 * a + b] += st[a][b];
    }
    for (int i = 0; i < N; ++i) {
        const double* s = &c.virS[9 * i];
        c.virP[i] = c.two_d ? -1.0 / 2.0 * (s[0] + s[4]) : -1.0 / 3.0 * (s[0] + s[4] + s[8]);
    }
}

void load_particles(Case& c, const mph_particles* p)
{
    c.N = p->count;
    c.time = p->time;
    c.l0 = p->spacing;
    for (int d = 0; d < 3; ++d) { c.dmin[d] = p->domain_min[d]; c.dmax[d] = p->domain_max[d]; }
    c.vol = c.two_d ? c.l0 * c.l0 : c.l0 * c.l0 * c.l0;
    c.type.assign(p->type, p->type + c.N);
    c.pos.assign(p->pos, p->pos + 3 * (size_t)c.N);
    c.vel.assign(p->vel, p->vel + 3 * (size_t)c.N);
    c.id.resize(c.N);
    for (int i = 0; i < c.N; ++i) c.id[i] = p->id ? p->id[i] : i;
    const size_t n = c.N;
    c.force.assign(3 * n, 0.0);
    c.mass.assign(n, 0.0); c.kappa.assign(n, 0.0); c.lambda.assign(n, 0.0); c.mu.assign(n, 0.0);
    c.densA.assign(n, 0.0); c.gcen.assign(3 * n, 0.0); c.presA.assign(n, 0.0); c.vsp.assign(n, 0.0);
    c.divP.assign(n, 0.0); c.presP.assign(n, 0.0); c.virP.assign(n, 0.0); c.virS.assign(9 * n, 0.0);
}

}  // namespace

struct mpho_case { Case c; };

extern "C" {

mpho_case* mpho_create(const mph_params* prm, const mph_particles* parts, int dim)
{
    if (!prm || !parts || (dim != 2 && dim != 3)) return nullptr;
    mpho_case* h = new mpho_case();
    Case& c = h->c;
    c.two_d = dim == 2;
    c.prm = *prm;
    c.dt = prm->dt;
    std::memcpy(c.wallC, prm->wall_center, sizeof c.wallC);
    std::memcpy(c.wallV, prm->wall_velocity, sizeof c.wallV);
    std::memcpy(c.wallW, prm->wall_omega, sizeof c.wallW);
    load_particles(c, parts);
    init_weights(c);
    init_fluid(c);
    init_wall(c);
    init_domain(c);
    return h;
}

void mpho_destroy(mpho_case* h) { delete h; }

void mpho_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

void mpho_init(mpho_case* h)
{
    Case& c = h->c;
    cellsort(c);
    neighbors(c);
    density_a(c);
    gravity_center(c);
    density_p(c);
}
void mpho_step_begin(mpho_case* h) { step_begin(h->c); }
void mpho_cellsort(mpho_case* h) { cellsort(h->c); }
void mpho_neighbors(mpho_case* h) { neighbors(h->c); }
void mpho_explicit(mpho_case* h) { explicit_stage(h->c); }
void mpho_assemble(mpho_case* h) { assemble(h->c); }
void mpho_mg_build(mpho_case* h) { mg_build(h->c); }
int mpho_solve(mpho_case* h) { return solve(h->c); }
void mpho_step_end(mpho_case* h) { h->c.time += h->c.dt; }
void mpho_output_fields(mpho_case* h) { output_fields(h->c); }

int mpho_step(mpho_case* h, int nsteps)
{
    int last = 0;
    for (int s = 0; s < nsteps; ++s) {
        mpho_step_begin(h);
        mpho_cellsort(h);
        mpho_neighbors(h);
        mpho_explicit(h);
        mpho_assemble(h);
        mpho_mg_build(h);
        last = mpho_solve(h);
        mpho_step_end(h);
        if (last < 0) return last;
    }
    return last;
}

static const char* kNames =
    "Time,Dt,ParticleCount,FluidParticleBegin,FluidParticleEnd,WallParticleBegin,WallParticleEnd,"
    "TotalCellCount,CellCount0,CellCount1,CellCount2,PowerParticleCount,NeighborIndCount,NeighborIndCountP,"
    "NonzeroCountA,NonzeroCountC,MultiGridDepth,MaxRadius,RadiusA,RadiusG,RadiusP,RadiusV,N0a,N0p,R2g,"
    "Swa,Swg,Swp,Swv,CofK,ParticleVolume,ParticleSpacing";
const char* mpho_scalar_names(void) { return kNames; }

int mpho_scalars(mpho_case* h, double* out)
{
    const Case& c = h->c;
    const double v[] = {c.time, c.dt, (double)c.N, (double)c.fB, (double)c.fE, (double)c.wB, (double)c.wE,
                        (double)c.T, (double)c.cc[0], (double)c.cc[1], (double)c.cc[2], (double)c.nPow,
                        (double)c.nind.size(), (double)c.nindP.size(), (double)c.aval.size(), (double)c.cval.size(),
                        (double)c.depth, c.maxR, c.rA, c.rG, c.rP, c.rV, c.N0a, c.N0p, c.R2g,
                        c.Swa, c.Swg, c.Swp, c.Swv, c.cofK, c.vol, c.l0};
    const int n = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}

void mpho_set_tolerance(mpho_case* h, double rel)
{
    h->c.tol2 = rel == 1.0e-6 ? 1.0e-12 : rel * rel;
}

int mpho_solve_stats(mpho_case* h, double* out5)
{
    const Case& c = h->c;
    out5[0] = c.iters; out5[1] = c.rr0; out5[2] = c.rr; out5[3] = c.rs0; out5[4] = c.rs;
    return 0;
}

long mpho_array(mpho_case* h, const char* name, void** ptr, int* kind)
{
    Case& c = h->c;
#define ARR(nm, vec, k) if (std::strcmp(name, nm) == 0) { *ptr = (void*)vec.data(); *kind = k; return (long)vec.size(); }
    ARR("Property", c.type, 0)
    ARR("ParticleIndex", c.id, 0)
    ARR("Position", c.pos, 2)
    ARR("Velocity", c.vel, 2)
    ARR("Force", c.force, 2)
    ARR("Mass", c.mass, 2)
    ARR("Kappa", c.kappa, 2)
    ARR("Lambda", c.lambda, 2)
    ARR("Mu", c.mu, 2)
    ARR("DensityA", c.densA, 2)
    ARR("GravityCenter", c.gcen, 2)
    ARR("PressureA", c.presA, 2)
    ARR("VolStrainP", c.vsp, 2)
    ARR("DivergenceP", c.divP, 2)
    ARR("PressureP", c.presP, 2)
    ARR("VirialPressureAtParticle", c.virP, 2)
    ARR("VirialStressAtParticle", c.virS, 2)
    ARR("CellIndex", c.key, 0)
    ARR("CellParticle", c.perm, 0)
    ARR("CellFluidParticleBegin", c.cfb, 0)
    ARR("CellFluidParticleEnd", c.cfe, 0)
    ARR("CellWallParticleBegin", c.cwb, 0)
    ARR("CellWallParticleEnd", c.cwe, 0)
    ARR("NeighborCount", c.nc, 0)
    ARR("NeighborFluidCount", c.nfc, 0)
    ARR("NeighborCountP", c.ncp, 0)
    ARR("NeighborPtr", c.nptr, 1)
    ARR("NeighborPtrP", c.nptrP, 1)
    ARR("NeighborInd", c.nind, 0)
    ARR("NeighborIndP", c.nindP, 0)
    ARR("CsrPtrA", c.aptr, 1)
    ARR("CsrIndA", c.aind, 0)
    ARR("CsrCofA", c.aval, 2)
    ARR("VectorB", c.bvec, 2)
    ARR("CsrPtrC", c.cptr, 1)
    ARR("CsrIndC", c.cind, 0)
    ARR("CsrCofC", c.cval, 2)
    ARR("VectorP", c.pvec, 2)
    ARR("InvDiagA", c.invDiag, 2)
#undef ARR
    if (std::strcmp(name, "WallCenter") == 0) { *ptr = (void*)&c.wallC[0][0]; *kind = 2; return 12; }
    if (std::strcmp(name, "WallRotation") == 0) { *ptr = (void*)&c.wallR[0][0][0]; *kind = 2; return 36; }
    return -1;
}

int mpho_mg_level_geom(mpho_case* h, int level, int* out9)
{
    const Case& c = h->c;
    if (level < 0 || level >= c.depth) return -1;
    for (int d = 0; d < 3; ++d) {
        out9[d] = c.lv[level].mn[d];
        out9[3 + d] = c.lv[level].mx[d];
        out9[6 + d] = c.lv[level].cnt[d];
    }
    return 0;
}

int mpho_mg_level_matrix(mpho_case* h, int level, double** cof, double** invd, int* rows, int* width)
{
    Case& c = h->c;
    if (level < 0 || level >= c.depth) return -1;
    *cof = c.lv[level].cof.data();
    *invd = c.lv[level].invd.data();
    *rows = c.lv[level].rows;
    *width = c.lv[level].width;
    return 0;
}

void mpho_set_state(mpho_case* h, const mph_particles* p, const double* wall_center)
{
    Case& c = h->c;
    const int N = c.N;
    if (p->count != N) return;
    c.time = p->time;
    c.type.assign(p->type, p->type + N);
    c.pos.assign(p->pos, p->pos + 3 * (size_t)N);
    c.vel.assign(p->vel, p->vel + 3 * (size_t)N);
    for (int i = 0; i < N; ++i) c.id[i] = p->id ? p->id[i] : i;
    if (wall_center) std::memcpy(c.wallC, wall_center, sizeof c.wallC);
    // recompute the fluid / wall ranges the next step_begin relies on
    // (they hold the previous sort's result in the reference)
    int nfl = 0;
    for (int i = 0; i < N; ++i) nfl += !is_wall(c.type[i]);
    c.fB = 0; c.fE = nfl; c.wB = nfl; c.wE = N;
}

}  // extern "C"
