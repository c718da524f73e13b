// mph_io.cpp - the reference's file formats.
//
//   .data : keyword lines (readDataFile, main.cpp:523-563); unknown lines are
//           ignored as in the reference
//   .grid : "Time" / "N l0 xmin xmax ymin ymax zmin zmax" / N particle lines
//           "type x y z vx vy vz" (readGridFile, main.cpp:565-669).  A file
//           with fewer particle lines than announced is an error here (the
//           reference silently stops reading, main.cpp:663)
//   .prof : the .grid format with %e fields (writeProfFile, main.cpp:696-720)
//   .vtk  : legacy ASCII unstructured grid with the reference's point data
//           (writeVtkFile, main.cpp:722-883)
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mph_internal.h"

namespace mph {

int read_data(const char* path, mph_params* o)
{
    if (!path || !o) return fail(MPH_ERR_ARG, "null argument");
    FILE* fp = std::fopen(path, "r");
    if (!fp) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    std::memset(o, 0, sizeof(*o));
    o->dt = 1.0e100;   // the reference's initial value (main.cpp:75)
    char buf[1024];
    while (std::fgets(buf, sizeof buf, fp)) {
        if (buf[0] == '#') continue;
        double* ir = nullptr;
        if (std::sscanf(buf, " Dt %lf", &o->dt) == 1) continue;
        if (std::sscanf(buf, " OutputInterval %lf", &o->output_interval) == 1) continue;
        if (std::sscanf(buf, " VtkOutputInterval %lf", &o->vtk_output_interval) == 1) continue;
        if (std::sscanf(buf, " EndTime %lf", &o->end_time) == 1) continue;
        if (std::sscanf(buf, " RadiusRatioA %lf", &o->radius_ratio_a) == 1) continue;
        if (std::sscanf(buf, " RadiusRatioP %lf", &o->radius_ratio_p) == 1) continue;
        if (std::sscanf(buf, " RadiusRatioV %lf", &o->radius_ratio_v) == 1) continue;
        struct Row { const char* fmt; double* dst; } rows[] = {
            {" Density %lf %lf %lf %lf", o->density},
            {" BulkModulus %lf %lf %lf %lf", o->bulk_modulus},
            {" BulkViscosity %lf %lf %lf %lf", o->bulk_viscosity},
            {" ShearViscosity %lf %lf %lf %lf", o->shear_viscosity},
            {" SurfaceTension %lf %lf %lf %lf", o->surface_tension},
            {" InteractionRatio(Type0) %lf %lf %lf %lf", o->interaction_ratio[0]},
            {" InteractionRatio(Type1) %lf %lf %lf %lf", o->interaction_ratio[1]},
            {" InteractionRatio(Type2) %lf %lf %lf %lf", o->interaction_ratio[2]},
            {" InteractionRatio(Type3) %lf %lf %lf %lf", o->interaction_ratio[3]},
        };
        bool done = false;
        for (const Row& r : rows) {
            double v[4];
            if (std::sscanf(buf, r.fmt, &v[0], &v[1], &v[2], &v[3]) == 4) {
                std::memcpy(r.dst, v, sizeof v);
                done = true;
                break;
            }
        }
        if (done) continue;
        double g[3];
        if (std::sscanf(buf, " Gravity %lf %lf %lf", &g[0], &g[1], &g[2]) == 3) {
            std::memcpy(o->gravity, g, sizeof g);
            continue;
        }
        for (int t = 2; t < 4; ++t) {
            double w[9];
            const char* fmt = t == 2 ? " Wall2  Center %lf %lf %lf Velocity %lf %lf %lf Omega %lf %lf %lf"
                                     : " Wall3  Center %lf %lf %lf Velocity %lf %lf %lf Omega %lf %lf %lf";
            if (std::sscanf(buf, fmt, &w[0], &w[1], &w[2], &w[3], &w[4], &w[5], &w[6], &w[7], &w[8]) == 9) {
                for (int d = 0; d < 3; ++d) {
                    o->wall_center[t][d] = w[d];
                    o->wall_velocity[t][d] = w[3 + d];
                    o->wall_omega[t][d] = w[6 + d];
                }
                done = true;
                break;
            }
        }
        (void)ir;
    }
    std::fclose(fp);
    return MPH_OK;
}

int read_grid(const char* path, mph_particles* o)
{
    if (!path || !o) return fail(MPH_ERR_ARG, "null argument");
    FILE* fp = std::fopen(path, "r");
    if (!fp) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    char buf[1024];
    double time = 0.0;
    int n = 0;
    double l0 = 0, dm[6] = {0, 0, 0, 0, 0, 0};
    if (!std::fgets(buf, sizeof buf, fp) || std::sscanf(buf, "%lf", &time) != 1) {
        std::fclose(fp);
        return fail(MPH_ERR_IO, "grid file: missing time line");
    }
    if (!std::fgets(buf, sizeof buf, fp) ||
        std::sscanf(buf, "%d %lf %lf %lf %lf %lf %lf %lf", &n, &l0, &dm[0], &dm[1], &dm[2], &dm[3], &dm[4], &dm[5]) != 8) {
        std::fclose(fp);
        return fail(MPH_ERR_IO, "grid file: malformed header line");
    }
    if (n < 0) {
        std::fclose(fp);
        return fail(MPH_ERR_IO, "grid file: negative particle count");
    }
    const bool want = o->type && o->pos && o->vel;
    if (want && o->count < n) {
        std::fclose(fp);
        return fail(MPH_ERR_ARG, "grid file: output buffers too small");
    }
    o->count = n;
    o->time = time;
    o->spacing = l0;
    o->domain_min[0] = dm[0]; o->domain_max[0] = dm[1];
    o->domain_min[1] = dm[2]; o->domain_max[1] = dm[3];
    o->domain_min[2] = dm[4]; o->domain_max[2] = dm[5];
    if (want) {
        for (int i = 0; i < n; ++i) {
            int t;
            double v[6];
            if (!std::fgets(buf, sizeof buf, fp) ||
                std::sscanf(buf, "%d %lf %lf %lf %lf %lf %lf", &t, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]) != 7) {
                std::fclose(fp);
                return fail(MPH_ERR_IO, "grid file: fewer particle lines than announced");
            }
            o->type[i] = t;
            for (int d = 0; d < 3; ++d) {
                o->pos[3 * i + d] = v[d];
                o->vel[3 * i + d] = v[3 + d];
            }
            if (o->id) o->id[i] = i;
        }
    }
    std::fclose(fp);
    return MPH_OK;
}

int write_prof(const char* path, const mph_particles* p)
{
    if (!path || !p) return fail(MPH_ERR_ARG, "null argument");
    FILE* fp = std::fopen(path, "w");
    if (!fp) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(fp, "%e\n", p->time);
    std::fprintf(fp, "%d %e %e %e %e %e %e %e\n", p->count, p->spacing, p->domain_min[0], p->domain_max[0], p->domain_min[1],
                 p->domain_max[1], p->domain_min[2], p->domain_max[2]);
    for (int i = 0; i < p->count; ++i)
        std::fprintf(fp, "%d %e %e %e  %e %e %e\n", p->type[i], p->pos[3 * i], p->pos[3 * i + 1], p->pos[3 * i + 2],
                     p->vel[3 * i], p->vel[3 * i + 1], p->vel[3 * i + 2]);
    std::fclose(fp);
    return MPH_OK;
}

int case_write_prof(mph_case* c, const char* path)
{
    const int N = c->dp.N;
    std::vector<int> type(N);
    std::vector<double> pos((size_t)N * 3), vel((size_t)N * 3);
    mph_fields f{};
    f.type = type.data();
    f.pos = pos.data();
    f.vel = vel.data();
    MPH_TRY(case_get_fields(c, &f));
    mph_particles p{};
    p.count = N;
    p.time = c->time;
    p.spacing = c->dp.l0;
    for (int d = 0; d < 3; ++d) {
        p.domain_min[d] = c->dp.dmin[d];
        p.domain_max[d] = c->dp.dmin[d] + c->dp.dw[d];
    }
    p.type = type.data();
    p.pos = pos.data();
    p.vel = vel.data();
    return write_prof(path, &p);
}

int case_write_vtk(mph_case* c, const char* path)
{
    const int N = c->dp.N;
    std::vector<int> type(N), nbc(N);
    std::vector<double> pos((size_t)N * 3), vel((size_t)N * 3), force((size_t)N * 3), vsp(N), divp(N), presp(N), virp(N);
    mph_fields f{};
    f.type = type.data();
    f.pos = pos.data();
    f.vel = vel.data();
    f.force = force.data();
    f.vol_strain_p = vsp.data();
    f.divergence_p = divp.data();
    f.pressure_p = presp.data();
    f.virial_p = virp.data();
    f.neighbor_count = nbc.data();
    MPH_TRY(case_get_fields(c, &f));
    FILE* fp = std::fopen(path, "w");
    if (!fp) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    std::fprintf(fp, "# vtk DataFile Version 2.0\n");
    std::fprintf(fp, "Unstructured Grid Example\n");
    std::fprintf(fp, "ASCII\n");
    std::fprintf(fp, "DATASET UNSTRUCTURED_GRID\n");
    std::fprintf(fp, "POINTS %d float\n", N);
    for (int i = 0; i < N; ++i) std::fprintf(fp, "%e %e %e\n", (float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2]);
    std::fprintf(fp, "CELLS %d %d\n", N, 2 * N);
    for (int i = 0; i < N; ++i) std::fprintf(fp, "1 %d ", i);
    std::fprintf(fp, "\n");
    std::fprintf(fp, "CELL_TYPES %d\n", N);
    for (int i = 0; i < N; ++i) std::fprintf(fp, "1 ");
    std::fprintf(fp, "\n");
    std::fprintf(fp, "\n");
    std::fprintf(fp, "POINT_DATA %d\n", N);
    std::fprintf(fp, "SCALARS label float 1\n");
    std::fprintf(fp, "LOOKUP_TABLE default\n");
    for (int i = 0; i < N; ++i) std::fprintf(fp, "%d\n", type[i]);
    std::fprintf(fp, "\n");
    const struct { const char* name; const std::vector<double>* v; } scal[] = {
        {"VolStrainP", &vsp}, {"DivergenceP", &divp}, {"PressureP", &presp}, {"VirialPressureAtParticle", &virp}};
    for (const auto& s : scal) {
        std::fprintf(fp, "SCALARS %s float 1\n", s.name);
        std::fprintf(fp, "LOOKUP_TABLE default\n");
        for (int i = 0; i < N; ++i) std::fprintf(fp, "%e\n", (float)(*s.v)[i]);
        std::fprintf(fp, "\n");
    }
    std::fprintf(fp, "SCALARS neighbor float 1\n");
    std::fprintf(fp, "LOOKUP_TABLE default\n");
    for (int i = 0; i < N; ++i) std::fprintf(fp, "%d\n", nbc[i]);
    std::fprintf(fp, "\n");
    std::fprintf(fp, "VECTORS velocity float\n");
    for (int i = 0; i < N; ++i) std::fprintf(fp, "%e %e %e\n", (float)vel[3 * i], (float)vel[3 * i + 1], (float)vel[3 * i + 2]);
    std::fprintf(fp, "\n");
    std::fprintf(fp, "VECTORS force float\n");
    for (int i = 0; i < N; ++i) std::fprintf(fp, "%e %e %e\n", (float)force[3 * i], (float)force[3 * i + 1], (float)force[3 * i + 2]);
    std::fprintf(fp, "\n");
    std::fclose(fp);
    return MPH_OK;
}

// ---- full-precision checkpoint sidecar ------------------------------------------
// The .prof frame keeps 7 significant digits (main.cpp:696-720); restarting a
// run from it changes the result.  The sidecar keeps the state in binary:
//   "MPHCKPT1", int32 count, double time, double spacing, double min[3],
//   double max[3], double wall_center[4][3], int32 id[count], int32
//   type[count], double pos[count][3], double vel[count][3]
// (host byte order; both build hosts are little-endian).  A case restored
// from it in the stored particle order continues bit for bit.
static const char kCkptMagic[8] = {'M', 'P', 'H', 'C', 'K', 'P', 'T', '1'};

int write_checkpoint(const char* path, const mph_particles* p, const double* wall_center)
{
    if (!path || !p || !p->type || !p->pos || !p->vel || p->count < 0) return fail(MPH_ERR_ARG, "null argument");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    const int n = p->count;
    std::vector<int> id(n);
    for (int i = 0; i < n; ++i) id[i] = p->id ? p->id[i] : i;
    double wc[12] = {0};
    if (wall_center) std::memcpy(wc, wall_center, sizeof(wc));
    bool ok = std::fwrite(kCkptMagic, 1, 8, f) == 8;
    ok = ok && std::fwrite(&n, sizeof(int), 1, f) == 1;
    ok = ok && std::fwrite(&p->time, sizeof(double), 1, f) == 1;
    ok = ok && std::fwrite(&p->spacing, sizeof(double), 1, f) == 1;
    ok = ok && std::fwrite(p->domain_min, sizeof(double), 3, f) == 3;
    ok = ok && std::fwrite(p->domain_max, sizeof(double), 3, f) == 3;
    ok = ok && std::fwrite(wc, sizeof(double), 12, f) == 12;
    ok = ok && std::fwrite(id.data(), sizeof(int), (size_t)n, f) == (size_t)n;
    ok = ok && std::fwrite(p->type, sizeof(int), (size_t)n, f) == (size_t)n;
    ok = ok && std::fwrite(p->pos, sizeof(double), (size_t)n * 3, f) == (size_t)n * 3;
    ok = ok && std::fwrite(p->vel, sizeof(double), (size_t)n * 3, f) == (size_t)n * 3;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MPH_OK : fail(MPH_ERR_IO, std::string("write failed: ") + path);
}

int read_checkpoint(const char* path, mph_particles* p, double* wall_center)
{
    if (!path || !p) return fail(MPH_ERR_ARG, "null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(MPH_ERR_IO, std::string("cannot open ") + path);
    char magic[8];
    int n = -1;
    double wc[12];
    mph_particles h = *p;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCkptMagic, 8) == 0;
    ok = ok && std::fread(&n, sizeof(int), 1, f) == 1 && n >= 0;
    ok = ok && std::fread(&h.time, sizeof(double), 1, f) == 1;
    ok = ok && std::fread(&h.spacing, sizeof(double), 1, f) == 1;
    ok = ok && std::fread(h.domain_min, sizeof(double), 3, f) == 3;
    ok = ok && std::fread(h.domain_max, sizeof(double), 3, f) == 3;
    ok = ok && std::fread(wc, sizeof(double), 12, f) == 12;
    if (!ok) {
        std::fclose(f);
        return fail(MPH_ERR_IO, std::string("not a checkpoint file: ") + path);
    }
    h.count = n;
    if (!p->type || !p->pos || !p->vel) {   // first call: the count only
        std::fclose(f);
        *p = h;
        p->type = nullptr;
        p->pos = p->vel = nullptr;
        p->id = nullptr;
        return MPH_OK;
    }
    if (p->count < n) {
        std::fclose(f);
        return fail(MPH_ERR_ARG, "buffers smaller than the checkpoint's particle count");
    }
    std::vector<int> id(n);
    ok = std::fread(id.data(), sizeof(int), (size_t)n, f) == (size_t)n;
    ok = ok && std::fread(p->type, sizeof(int), (size_t)n, f) == (size_t)n;
    ok = ok && std::fread(p->pos, sizeof(double), (size_t)n * 3, f) == (size_t)n * 3;
    ok = ok && std::fread(p->vel, sizeof(double), (size_t)n * 3, f) == (size_t)n * 3;
    std::fclose(f);
    if (!ok) return fail(MPH_ERR_IO, std::string("checkpoint file is short: ") + path);
    if (p->id) std::memcpy(p->id, id.data(), (size_t)n * sizeof(int));
    int* type = p->type;
    double *pos = p->pos, *vel = p->vel;
    int* pid = p->id;
    *p = h;
    p->type = type;
    p->pos = pos;
    p->vel = vel;
    p->id = pid;
    if (wall_center) std::memcpy(wall_center, wc, sizeof(wc));
    return MPH_OK;
}

int case_checkpoint(mph_case* c, const char* path)
{
    if (!c || !path) return fail(MPH_ERR_ARG, "null argument");
    const int n = c->dp.N;
    std::vector<int> id(n), type(n);
    std::vector<double> pos((size_t)n * 3), vel((size_t)n * 3);
    mph_fields f{};
    f.id = id.data();
    f.type = type.data();
    f.pos = pos.data();
    f.vel = vel.data();
    MPH_TRY(case_get_fields(c, &f));
    mph_particles p{};
    p.count = n;
    p.time = c->time;
    p.spacing = c->dp.l0;
    for (int d = 0; d < 3; ++d) {
        p.domain_min[d] = c->prm_domain_min[d];
        p.domain_max[d] = c->prm_domain_max[d];
    }
    p.type = type.data();
    p.pos = pos.data();
    p.vel = vel.data();
    p.id = id.data();
    return write_checkpoint(path, &p, &c->wallC[0][0]);
}

}  // namespace mph
