// mph_export.cu - host copies of the device state in the reference's layout
// (test and output support): named arrays, scalars, per-particle fields, and
// replacing the particle state of a case.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mph_device.cuh"
#include "mph_solver.cuh"

namespace mph {

template <typename T>
static int d2h(mph_case* c, std::vector<T>& h, const T* d, size_t n)
{
    h.resize(n);
    if (n == 0) return MPH_OK;
    MPH_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    return MPH_OK;
}

// [N][VS] device vectors -> [N][3] host vectors (2D: z = plane / 0)
static int vec3(mph_case* c, const double* d, std::vector<double>& out, double zfill)
{
    const int N = c->dp.N, VSn = vs_of(c->dim);
    std::vector<double> h;
    MPH_TRY(d2h(c, h, d, (size_t)N * VSn));
    out.assign((size_t)N * 3, 0.0);
    for (int i = 0; i < N; ++i) {
        for (int k = 0; k < c->dim; ++k) out[3 * (size_t)i + k] = h[(size_t)i * VSn + k];
        if (c->dim == 2) out[3 * (size_t)i + 2] = zfill;
    }
    return MPH_OK;
}

struct Out {
    int kind = 2;
    std::vector<int> i32;
    std::vector<long long> i64;
    std::vector<double> f64;
    long count() const { return kind == 0 ? (long)i32.size() : kind == 1 ? (long)i64.size() : (long)f64.size(); }
    const void* data() const { return kind == 0 ? (const void*)i32.data() : kind == 1 ? (const void*)i64.data() : (const void*)f64.data(); }
};

static int build_export(mph_case* c, const std::string& name, Out& o)
{
    const int N = c->dp.N, Nf = c->dp.Nf, D = c->dim, T = c->dp.T;
    DeviceState& d = c->d;
    auto i32 = [&](const int* p, size_t n) { o.kind = 0; return d2h(c, o.i32, p, n); };
    auto i64 = [&](const long long* p, size_t n) { o.kind = 1; return d2h(c, o.i64, p, n); };
    auto f64 = [&](const double* p, size_t n) { o.kind = 2; return d2h(c, o.f64, p, n); };
    if (name == "DensityA" || name == "GravityCenter" || name == "PressureA") {
        if (c->stage == 1 || c->stage == 2) return fail(MPH_ERR_STATE, name + " needs this step's neighbour lists");
        ensure_density_a(c);
        MPH_CUDA(cudaGetLastError());
    }
    if (name == "Position") { o.kind = 2; return vec3(c, d.pos, o.f64, c->z_plane); }
    if (name == "Velocity") { o.kind = 2; return vec3(c, d.vel, o.f64, 0.0); }
    if (name == "Force") { o.kind = 2; return vec3(c, d.force, o.f64, 0.0); }
    if (name == "GravityCenter") { o.kind = 2; return vec3(c, d.gcen, o.f64, 0.0); }
    if (name == "Property") return i32(d.type, N);
    if (name == "ParticleIndex") return i32(d.id, N);
    if (name == "CellIndex") return i32(d.key, c->dp.nPow);
    if (name == "CellParticle") return i32(d.perm, c->dp.nPow);
    if (name == "NeighborCount") return i32(d.nc, N);
    if (name == "NeighborFluidCount") return i32(d.nfc, N);
    if (name == "NeighborCountP") return i32(d.ncp, N);
    if (name == "NeighborPtr") return i64(d.nptr, (size_t)N + 1);
    if (name == "NeighborPtrP") return i64(d.nptrP, (size_t)N + 1);
    if (name == "NeighborInd") return i32(d.nind, c->nnb);
    if (name == "NeighborIndP") return i32(d.nindP, c->nnbP);
    if (name == "DensityA") return f64(d.densA, N);
    if (name == "VolStrainP") return f64(d.vsp, N);
    if (name == "PressureA") return f64(d.presA, N);
    if (name == "DivergenceP") return f64(d.divP, N);
    if (name == "PressureP") return f64(d.presP, N);
    if (name == "VirialPressureAtParticle") return f64(d.virP, N);
    if (name == "VirialStressAtParticle") return f64(d.virS, (size_t)N * 9);
    if (name == "VectorP") return f64(d.pvec, N);
    if (name == "VectorB") return f64(d.bvec, (size_t)Nf * D);
    if (name == "InvDiagA") return f64(d.invDiag, (size_t)Nf * D);
    if (name == "CellFluidParticleBegin" || name == "CellFluidParticleEnd" || name == "CellWallParticleBegin" ||
        name == "CellWallParticleEnd") {
        std::vector<int> b;
        MPH_TRY(d2h(c, b, d.bucket, (size_t)2 * T + 1));
        o.kind = 0;
        o.i32.resize(T);
        const int off = (name.find("Wall") != std::string::npos) ? T : 0;
        const int end = (name.find("End") != std::string::npos) ? 1 : 0;
        for (int k = 0; k < T; ++k) o.i32[k] = b[off + k + end];
        return MPH_OK;
    }
    if (name == "Mass" || name == "Kappa" || name == "Lambda" || name == "Mu") {
        std::vector<int> t;
        std::vector<double> v;
        MPH_TRY(d2h(c, t, d.type, N));
        MPH_TRY(d2h(c, v, d.vsp, N));
        o.kind = 2;
        o.f64.resize(N);
        for (int i = 0; i < N; ++i) {
            const int ty = t[i];
            if (name == "Mass") o.f64[i] = c->dp.density[ty] * c->dp.vol;
            else if (name == "Kappa") o.f64[i] = v[i] < 0.0 ? 0.0 : c->dp.bulk[ty];
            else if (name == "Lambda") o.f64[i] = c->dp.lambda[ty];
            else o.f64[i] = c->dp.mu[ty];
        }
        return MPH_OK;
    }
    if (name == "CsrCofA" && c->step_pairs)
        return fail(MPH_ERR_STATE, name + ": this step assembled no blocks (mixed form, factored operator; "
                                          "set option \"inner_blocks\" to 1 to keep FP32 blocks)");
    if (name == "CsrPtrA" || name == "CsrIndA" || name == "CsrCofA") {
        // sliced ELL -> CSR with rows D*i+r and entries (k, s), as the reference
        std::vector<int> nfc, acol;
        std::vector<long long> sptr;
        std::vector<double> aval;
        MPH_TRY(d2h(c, nfc, d.nfc, Nf));
        MPH_TRY(d2h(c, sptr, d.sptr, (size_t)c->nslices + 1));
        MPH_TRY(d2h(c, acol, d.acol, (size_t)c->nslots));
        if (name == "CsrCofA" && c->step_factored) {
            // mixed form with the factored FP64 operator: only FP32 blocks exist
            std::vector<float> a32;
            MPH_TRY(d2h(c, a32, d.aval32, (size_t)c->nslots * D * D));
            aval.assign(a32.begin(), a32.end());
        } else if (name == "CsrCofA") {
            MPH_TRY(d2h(c, aval, d.aval, (size_t)c->nslots * D * D));
        }
        long long nnz = 0;
        for (int i = 0; i < Nf; ++i) nnz += (long long)D * D * nfc[i];
        if (name == "CsrPtrA") {
            o.kind = 1;
            o.i64.assign((size_t)Nf * D + 1, 0);
            for (int i = 0; i < Nf; ++i)
                for (int r = 0; r < D; ++r) o.i64[(size_t)i * D + r + 1] = o.i64[(size_t)i * D + r] + (long long)D * nfc[i];
            return MPH_OK;
        }
        o.kind = name == "CsrIndA" ? 0 : 2;
        if (o.kind == 0) o.i32.resize(nnz); else o.f64.resize(nnz);
        long long w = 0;
        for (int i = 0; i < Nf; ++i) {
            const long long base = sptr[i >> 5];
            const int lane = i & 31;
            for (int r = 0; r < D; ++r)
                for (int k = 0; k < nfc[i]; ++k)
                    for (int s = 0; s < D; ++s, ++w) {
                        if (o.kind == 0) o.i32[w] = D * acol[base + (long long)k * 32 + lane] + s;
                        else o.f64[w] = aval[base * D * D + ((long long)k * D * D + r * D + s) * 32 + lane];
                    }
        }
        return MPH_OK;
    }
    if (name == "CsrPtrC" || name == "CsrIndC" || name == "CsrCofC") {
        std::vector<int> ncp, indP;
        std::vector<long long> ptrP;
        std::vector<double> cval;
        MPH_TRY(d2h(c, ncp, d.ncp, N));
        MPH_TRY(d2h(c, ptrP, d.nptrP, (size_t)N + 1));
        MPH_TRY(d2h(c, indP, d.nindP, (size_t)c->nnbP));
        if (name == "CsrCofC") MPH_TRY(d2h(c, cval, d.cval, (size_t)ptrP[Nf] * D));
        if (name == "CsrPtrC") {
            o.kind = 1;
            o.i64.assign((size_t)Nf * D + 1, 0);
            for (int i = 0; i < Nf; ++i)
                for (int r = 0; r < D; ++r) o.i64[(size_t)i * D + r + 1] = o.i64[(size_t)i * D + r] + ncp[i];
            return MPH_OK;
        }
        o.kind = name == "CsrIndC" ? 0 : 2;
        for (int i = 0; i < Nf; ++i)
            for (int r = 0; r < D; ++r)
                for (int a = 0; a < ncp[i]; ++a) {
                    if (o.kind == 0) o.i32.push_back(indP[ptrP[i] + a]);
                    else o.f64.push_back(cval[(ptrP[i] + a) * D + r]);
                }
        return MPH_OK;
    }
    const size_t colon = name.find(':');
    if (colon != std::string::npos) {
        const std::string base = name.substr(0, colon);
        const int L = std::atoi(name.c_str() + colon + 1);
        if (L < 0 || L >= c->depth) return fail(MPH_ERR_ARG, "no such multigrid level");
        if (mixed_jacobi(c)) return fail(MPH_ERR_STATE, "the point-Jacobi mixed form builds no multigrid levels");
        const LevelGeom& g = c->lv[L];
        if (base == "MultiGridCsrCofA") {
            // stored entry-major; returned row-major like the reference's CSR rows
            const size_t width = (size_t)D * g.st[0] * g.st[1] * g.st[2];
            std::vector<double> t;
            MPH_TRY(d2h(c, t, d.mg_cof + g.off_cof, (size_t)g.rows * width));
            o.kind = 2;
            o.f64.resize(t.size());
            for (size_t row = 0; row < (size_t)g.rows; ++row)
                for (size_t e = 0; e < width; ++e) o.f64[row * width + e] = t[e * g.rows + row];
            return MPH_OK;
        }
        if (base == "MultiGridInvDiagA") return f64(d.mg_invd + g.off_vec, (size_t)g.rows);
        if (base == "MultiGridGeom") {
            o.kind = 0;
            o.i32.clear();
            for (int k = 0; k < 3; ++k) o.i32.push_back(g.mn[k]);
            for (int k = 0; k < 3; ++k) o.i32.push_back(g.mx[k]);
            for (int k = 0; k < 3; ++k) o.i32.push_back(g.cnt[k]);
            return MPH_OK;
        }
    }
    if (name == "WallCenter") {
        o.kind = 2;
        o.f64.assign(&c->wallC[0][0], &c->wallC[0][0] + 12);
        return MPH_OK;
    }
    return fail(MPH_ERR_ARG, "unknown array name: " + name);
}

int case_export(mph_case* c, const char* name, void* dst, long* count, int* kind)
{
    if (!c || !name) return fail(MPH_ERR_ARG, "null argument");
    Out o;
    MPH_TRY(build_export(c, name, o));
    if (count) *count = o.count();
    if (kind) *kind = o.kind;
    if (dst) {
        const size_t es = o.kind == 0 ? 4 : 8;
        std::memcpy(dst, o.data(), (size_t)o.count() * es);
    }
    return MPH_OK;
}

static const char* kNames =
    "Time,Dt,ParticleCount,FluidParticleBegin,FluidParticleEnd,WallParticleBegin,WallParticleEnd,"
    "TotalCellCount,CellCount0,CellCount1,CellCount2,PowerParticleCount,NeighborIndCount,NeighborIndCountP,"
    "NonzeroCountA,NonzeroCountC,MultiGridDepth,MaxRadius,RadiusA,RadiusG,RadiusP,RadiusV,N0a,N0p,R2g,"
    "Swa,Swg,Swp,Swv,CofK,ParticleVolume,ParticleSpacing";
const char* scalar_names() { return kNames; }

int case_scalars(mph_case* c, double* out, int n)
{
    if (!c || !out) return fail(MPH_ERR_ARG, "null argument");
    const DevParams& P = c->dp;
    long long nnzA = 0, nnzC = 0;
    {
        std::vector<int> nfc, ncp;
        if (c->stage >= 3 || c->stage == 0) {
            MPH_TRY(d2h(c, nfc, c->d.nfc, P.Nf));
            MPH_TRY(d2h(c, ncp, c->d.ncp, P.Nf));
            for (int i = 0; i < P.Nf; ++i) { nnzA += (long long)c->dim * c->dim * nfc[i]; nnzC += (long long)c->dim * ncp[i]; }
        }
    }
    const double v[] = {c->time, P.dt, (double)P.N, (double)c->fB, (double)c->fE, (double)c->wB, (double)c->wE,
                        (double)P.T, (double)P.cc[0], (double)P.cc[1], (double)P.cc[2], (double)P.nPow,
                        (double)c->nnb, (double)c->nnbP, (double)nnzA, (double)nnzC, (double)c->depth,
                        P.maxR, P.rA, P.rG, P.rP, P.rV, P.N0a, P.N0p, P.R2g, c->Swa, c->Swg, c->Swp, c->Swv,
                        P.cofK, P.vol, P.l0};
    const int m = (int)(sizeof(v) / sizeof(v[0]));
    for (int k = 0; k < m && k < n; ++k) out[k] = v[k];
    return MPH_OK;
}

// ---- host-layout particle records: N x 3 doubles <-> the device's N x VS ----------
template <int D>
__global__ void k_pack3(int N, const double* __restrict__ src, double zfill, double* __restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double v[3];
    load_vec<D>(src, i, v);
    dst[3 * (size_t)i] = v[0];
    dst[3 * (size_t)i + 1] = v[1];
    dst[3 * (size_t)i + 2] = D == 3 ? v[2] : zfill;
}

template <int D>
__global__ void k_unpack3(int N, const double* __restrict__ src, double* __restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double v[3] = {src[3 * (size_t)i], src[3 * (size_t)i + 1], D == 3 ? src[3 * (size_t)i + 2] : 0.0};
    store_vec<D>(dst, i, v);
}

__global__ void k_iota(int N, int* __restrict__ a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) a[i] = i;
}

static int ensure_io3(mph_case* c)
{
    if (!c->d.io3) MPH_CUDA(cudaMalloc((void**)&c->d.io3, (size_t)c->dp.N * 6 * sizeof(double)));
    return MPH_OK;
}

// stage the N x 3 host layout of a device vector array in io3 slot `slot`
static void pack3(mph_case* c, const double* src, double zfill, int slot)
{
    const int N = c->dp.N;
    double* dst = c->d.io3 + (size_t)slot * N * 3;
    if (c->dim == 2) { k_pack3<2><<<grid_for(N, 256), 256, 0, c->stream>>>(N, src, zfill, dst); MPH_COUNT_LAUNCH(); }
    else { k_pack3<3><<<grid_for(N, 256), 256, 0, c->stream>>>(N, src, zfill, dst); MPH_COUNT_LAUNCH(); }
}

// The fields go straight from device memory to the caller's buffers: the
// per-particle arrays by one copy each, the vector arrays after a kernel puts
// them in the N x 3 host layout (a pinned caller buffer takes the copies at
// link speed).  Fields that need the output-step computations go through
// build_export.
int case_get_fields(mph_case* c, mph_fields* f)
{
    if (!c || !f) return fail(MPH_ERR_ARG, "null argument");
    const int N = c->dp.N;
    DeviceState& d = c->d;
    MPH_TRY(ensure_io3(c));
    const size_t b3 = (size_t)N * 3 * sizeof(double);
    if (f->id) MPH_CUDA(cudaMemcpyAsync(f->id, d.id, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (f->type) MPH_CUDA(cudaMemcpyAsync(f->type, d.type, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (f->neighbor_count) MPH_CUDA(cudaMemcpyAsync(f->neighbor_count, d.nc, (size_t)N * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    if (f->pos) {
        pack3(c, d.pos, c->z_plane, 0);
        MPH_CUDA(cudaMemcpyAsync(f->pos, d.io3, b3, cudaMemcpyDeviceToHost, c->stream));
    }
    if (f->vel) {
        pack3(c, d.vel, 0.0, 1);
        MPH_CUDA(cudaMemcpyAsync(f->vel, d.io3 + (size_t)N * 3, b3, cudaMemcpyDeviceToHost, c->stream));
    }
    if (f->force) {
        MPH_CUDA(cudaStreamSynchronize(c->stream));   // slot 0 is free again
        pack3(c, d.force, 0.0, 0);
        MPH_CUDA(cudaMemcpyAsync(f->force, d.io3, b3, cudaMemcpyDeviceToHost, c->stream));
    }
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    Out o;
    auto take_i = [&](const char* nm, int* dst) -> int {
        if (!dst) return MPH_OK;
        MPH_TRY(build_export(c, nm, o));
        std::memcpy(dst, o.i32.data(), (size_t)N * sizeof(int));
        return MPH_OK;
    };
    auto take_d = [&](const char* nm, double* dst, size_t n) -> int {
        if (!dst) return MPH_OK;
        MPH_TRY(build_export(c, nm, o));
        std::memcpy(dst, o.f64.data(), n * sizeof(double));
        return MPH_OK;
    };
    (void)take_i;
    MPH_TRY(take_d("VolStrainP", f->vol_strain_p, N));
    MPH_TRY(take_d("DivergenceP", f->divergence_p, N));
    MPH_TRY(take_d("PressureP", f->pressure_p, N));
    MPH_TRY(take_d("VirialPressureAtParticle", f->virial_p, N));
    return MPH_OK;
}

int case_set_state(mph_case* c, const mph_particles* parts, const double* wall_center)
{
    if (!c || !parts || !parts->type || !parts->pos || !parts->vel) return fail(MPH_ERR_ARG, "null argument");
    const int N = c->dp.N;
    if (parts->count != N) return fail(MPH_ERR_ARG, "particle count differs from the case");
    int nf = 0;
    bool wall_seen = false;
    for (int i = 0; i < N; ++i) {
        const int t = parts->type[i];
        if (t < 0 || t > 3) return fail(MPH_ERR_INPUT, "particle type outside 0..3");
        if (t < 2) {
            if (wall_seen) return fail(MPH_ERR_INPUT, "state must list fluid particles before wall particles");
            ++nf;
        } else {
            wall_seen = true;
        }
    }
    if (nf != c->dp.Nf) return fail(MPH_ERR_INPUT, "fluid particle count differs from the case");
    // the caller's N x 3 arrays go to device staging as they are (a pinned
    // caller buffer copies at link speed); a kernel lays them out as N x VS
    MPH_TRY(ensure_io3(c));
    DeviceState& d = c->d;
    const size_t b3 = (size_t)N * 3 * sizeof(double);
    MPH_CUDA(cudaMemcpyAsync(d.io3, parts->pos, b3, cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemcpyAsync(d.io3 + (size_t)N * 3, parts->vel, b3, cudaMemcpyHostToDevice, c->stream));
    MPH_CUDA(cudaMemcpyAsync(d.type, parts->type, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    if (parts->id) MPH_CUDA(cudaMemcpyAsync(d.id, parts->id, (size_t)N * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    else { k_iota<<<grid_for(N, 256), 256, 0, c->stream>>>(N, d.id); MPH_COUNT_LAUNCH(); }
    const unsigned g = grid_for(N, 256);
    if (c->dim == 2) {
        { k_unpack3<2><<<g, 256, 0, c->stream>>>(N, d.io3, d.pos); MPH_COUNT_LAUNCH(); }
        { k_unpack3<2><<<g, 256, 0, c->stream>>>(N, d.io3 + (size_t)N * 3, d.vel); MPH_COUNT_LAUNCH(); }
    } else {
        { k_unpack3<3><<<g, 256, 0, c->stream>>>(N, d.io3, d.pos); MPH_COUNT_LAUNCH(); }
        { k_unpack3<3><<<g, 256, 0, c->stream>>>(N, d.io3 + (size_t)N * 3, d.vel); MPH_COUNT_LAUNCH(); }
    }
    MPH_CUDA(cudaStreamSynchronize(c->stream));
    if (wall_center) std::memcpy(&c->wallC[0][0], wall_center, sizeof(c->wallC));
    c->time = parts->time;
    c->densa_valid = false;
    // a state from outside has no velocity history, unless the caller
    // declares (option keep_history) that it continues this case's own
    // trajectory in the case's particle order
    if (!c->keep_history) c->prev_valid = 0;
    c->fB = 0;
    c->fE = nf;
    c->wB = nf;
    c->wE = N;
    c->stage = 0;
    return MPH_OK;
}

}  // namespace mph
