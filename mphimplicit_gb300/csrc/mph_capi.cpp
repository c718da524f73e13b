// mph_capi.cpp - the extern "C" boundary (include/mph_gb300.h).  Every entry
// point catches C++ exceptions and turns them into status codes.
#include <exception>
#include <new>
#include <string>

#include "mph_internal.h"

namespace mph {
int read_data(const char* path, mph_params* o);
int read_grid(const char* path, mph_particles* o);
int write_prof(const char* path, const mph_particles* p);
int case_write_prof(mph_case* c, const char* path);
int case_write_vtk(mph_case* c, const char* path);
int write_checkpoint(const char* path, const mph_particles* p, const double* wall_center);
int read_checkpoint(const char* path, mph_particles* p, double* wall_center);
int case_checkpoint(mph_case* c, const char* path);
}  // namespace mph

#define GUARD(expr)                                                              \
    try {                                                                        \
        return (expr);                                                           \
    } catch (const std::bad_alloc&) {                                            \
        return mph::fail(MPH_ERR_NOMEM, "host allocation failed");               \
    } catch (const std::exception& e) {                                          \
        return mph::fail(MPH_ERR_STATE, e.what());                               \
    } catch (...) {                                                              \
        return mph::fail(MPH_ERR_STATE, "unknown exception");                    \
    }

#define NEED(c) if (!(c)) return mph::fail(MPH_ERR_ARG, "null case handle")

extern "C" {

int mph_read_data(const char* path, mph_params* out) { GUARD(mph::read_data(path, out)) }
int mph_read_grid(const char* path, mph_particles* out) { GUARD(mph::read_grid(path, out)) }
int mph_write_prof(const char* path, const mph_particles* parts) { GUARD(mph::write_prof(path, parts)) }
int mph_case_write_vtk(mph_case* c, const char* path) { NEED(c); GUARD(mph::case_write_vtk(c, path)) }
int mph_case_write_prof(mph_case* c, const char* path) { NEED(c); GUARD(mph::case_write_prof(c, path)) }
int mph_write_checkpoint(const char* path, const mph_particles* parts, const double* wall_center)
{
    GUARD(mph::write_checkpoint(path, parts, wall_center))
}
int mph_read_checkpoint(const char* path, mph_particles* out, double* wall_center)
{
    GUARD(mph::read_checkpoint(path, out, wall_center))
}
int mph_case_checkpoint(mph_case* c, const char* path) { NEED(c); GUARD(mph::case_checkpoint(c, path)) }

int mph_case_create(const mph_params* prm, const mph_particles* parts, int dim, int precision, void* stream, mph_case** out)
{
    GUARD(mph::case_create(prm, parts, dim, precision, stream, out))
}
int mph_case_destroy(mph_case* c) { GUARD(mph::case_destroy(c)) }
int mph_case_set_stream(mph_case* c, void* stream)
{
    NEED(c);
    c->stream = (cudaStream_t)stream;
    return MPH_OK;
}

int mph_step(mph_case* c, int nsteps)
{
    NEED(c);
    if (nsteps < 0) return mph::fail(MPH_ERR_ARG, "negative step count");
    GUARD(mph::case_step(c, nsteps))
}

int mph_batch_step(mph_case** cases, int ncases, int nsteps) { GUARD(mph::batch_step(cases, ncases, nsteps, 0)) }
int mph_batch_step_workers(mph_case** cases, int ncases, int nsteps, int workers)
{
    GUARD(mph::batch_step(cases, ncases, nsteps, workers))
}
int mph_case_footprint(const mph_params* prm, const mph_particles* parts, int dim, int precision, long long* bytes)
{
    GUARD(mph::case_footprint(prm, parts, dim, precision, bytes))
}
int mph_server_create(long long budget_bytes, int workers, int device, mph_server** out)
{
    GUARD(mph::server_create(budget_bytes, workers, device, out))
}
int mph_server_submit(mph_server* s, const mph_params* prm, const mph_particles* parts, int dim, int precision, int steps,
                      const mph_fields* out, float* step_ms, long long* ticket)
{
    GUARD(mph::server_submit(s, prm, parts, dim, precision, steps, out, step_ms, ticket))
}
int mph_server_poll(mph_server* s, mph_server_result* out, int max, int wait_ms, int* count)
{
    GUARD(mph::server_poll(s, out, max, wait_ms, count))
}
int mph_server_stats_get(mph_server* s, mph_server_stats* out) { GUARD(mph::server_stats(s, out)) }
int mph_server_destroy(mph_server* s) { GUARD(mph::server_destroy(s)) }
int mph_server_set_solver(mph_server* s, double outer_rel_residual, double inner_rel_residual, int max_outer)
{
    GUARD(mph::server_set_solver(s, outer_rel_residual, inner_rel_residual, max_outer))
}
int mph_server_set_option(mph_server* s, const char* name, double value) { GUARD(mph::server_set_option(s, name, value)) }

int mph_case_set_solver(mph_case* c, double outer_rel_residual, double inner_rel_residual, int max_outer)
{
    NEED(c);
    if (!(outer_rel_residual > 0.0) || !(inner_rel_residual > 0.0) || inner_rel_residual >= 1.0 || max_outer < 1)
        return mph::fail(MPH_ERR_ARG, "solver tolerances must be positive (inner < 1) and max_outer >= 1");
    c->tol_outer = outer_rel_residual;
    c->tol_inner = inner_rel_residual;
    c->max_outer = max_outer;
    return MPH_OK;
}

int mph_case_set_option(mph_case* c, const char* name, double value)
{
    NEED(c);
    if (!name) return mph::fail(MPH_ERR_ARG, "null option name");
    if (std::string(name) == "cell_assembly") {
        c->cell_assembly = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "extrapolate") {
        if (c->precision != MPH_PRECISION_MIXED && value != 0.0)
            return mph::fail(MPH_ERR_ARG, "option extrapolate: mixed form only (the FP64 form starts from v_n as the reference)");
        if (!(value == 0.0 || value == 1.0 || value == 2.0))
            return mph::fail(MPH_ERR_ARG, "option extrapolate: 0 (the reference's start), 1 (linear) or 2 (quadratic)");
        c->extrapolate = (int)value;
        c->prev_valid = 0;
        return MPH_OK;
    }
    if (std::string(name) == "dense_coarse") {
        c->dense_coarse = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "cell_sort") {
        if (!(value == 0.0 || value == 1.0)) return mph::fail(MPH_ERR_ARG, "option cell_sort: 0 (bitonic network) or 1 (counting sort)");
        c->cell_sort = (int)value;
        return MPH_OK;
    }
    if (std::string(name) == "device_loop") {
        c->device_loop = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "pair_block" || std::string(name) == "ct_block" || std::string(name) == "chunk") {
        const int v = (int)value;
        const std::string n(name);
        const bool ok = (double)v == value &&
                        (n == "pair_block" ? (v == 128 || v == 256 || v == 512)
                                           : n == "ct_block" ? (v == 128 || v == 256) : (v == 4 || v == 8 || v == 16 || v == 32));
        if (!ok) return mph::fail(MPH_ERR_ARG, "option " + n + ": pair_block 128/256/512, ct_block 128/256, chunk 4/8/16/32");
        (n == "pair_block" ? c->pair_block : n == "ct_block" ? c->ct_block : c->chunk) = v;
        return MPH_OK;
    }
    if (std::string(name) == "keep_history") {
        c->keep_history = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "mg_pre" || std::string(name) == "mg_post") {
        const int v = (int)value;
        if ((double)v != value || v < 1 || v > 4) return mph::fail(MPH_ERR_ARG, "options mg_pre / mg_post: 1 .. 4 sweeps");
        (std::string(name) == "mg_pre" ? c->mg_pre : c->mg_post) = v;
        return MPH_OK;
    }
    if (std::string(name) == "graphs") {
        c->use_graphs = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "factored") {
        c->factored = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "inner_blocks") {
        c->inner_blocks = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "inner_local") {
        c->inner_local = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "pair_recompute") {
        c->pair_recompute = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "mg_depth") {
        const int v = (int)value;
        if ((double)v != value || v < -1 || v > 24)
            return mph::fail(MPH_ERR_ARG, "option mg_depth: 0 (every level), 1 .. 24 levels, or -1 (no grid levels)");
        c->mg_depth = v;
        return MPH_OK;
    }
    if (std::string(name) == "mg_coarsest") {
        const int v = (int)value;
        if ((double)v != value || v < 1 || v > 8) return mph::fail(MPH_ERR_ARG, "option mg_coarsest: 1 .. 8 sweeps");
        c->mg_coarsest = v;
        return MPH_OK;
    }
    if (std::string(name) == "batch_solve") {
        c->batch_solve = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "pair_fuse") {
        c->pair_fuse = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "split_apply") {
        c->split_apply = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "pair_pack") {
        c->pair_pack = value != 0.0;
        return MPH_OK;
    }
    if (std::string(name) == "mixed_extra_sweeps") {
        if (!(value >= 0.0 && value <= 8.0)) return mph::fail(MPH_ERR_ARG, "mixed_extra_sweeps must be 0..8");
        c->mixed_extra_sweeps = (int)value;
        return MPH_OK;
    }
    return mph::fail(MPH_ERR_ARG, std::string("unknown option: ") + name);
}

int mph_case_count(mph_case* c, int* count, int* fluid_count)
{
    NEED(c);
    if (count) *count = c->dp.N;
    if (fluid_count) *fluid_count = c->dp.Nf;
    return MPH_OK;
}
int mph_case_time(mph_case* c, double* time)
{
    NEED(c);
    if (time) *time = c->time;
    return MPH_OK;
}
int mph_get_fields(mph_case* c, mph_fields* out) { NEED(c); GUARD(mph::case_get_fields(c, out)) }
int mph_get_solve_stats(mph_case* c, mph_solve_stats* out)
{
    NEED(c);
    if (!out) return mph::fail(MPH_ERR_ARG, "null output");
    *out = c->stats;
    return MPH_OK;
}

int mph_stage_step_begin(mph_case* c) { NEED(c); GUARD(mph::stage_step_begin(c)) }
int mph_stage_cellsort(mph_case* c) { NEED(c); GUARD(mph::stage_cellsort(c)) }
int mph_stage_neighbors(mph_case* c) { NEED(c); GUARD(mph::stage_neighbors(c)) }
int mph_stage_explicit(mph_case* c) { NEED(c); GUARD(mph::stage_explicit(c)) }
int mph_stage_assemble(mph_case* c) { NEED(c); GUARD(mph::stage_assemble(c)) }
int mph_stage_mg_build(mph_case* c) { NEED(c); GUARD(mph::stage_mg_build(c)) }
int mph_stage_solve(mph_case* c) { NEED(c); GUARD(mph::stage_solve(c)) }
int mph_stage_step_end(mph_case* c) { NEED(c); GUARD(mph::stage_step_end(c)) }
int mph_stage_output_fields(mph_case* c) { NEED(c); GUARD(mph::stage_output_fields(c)) }

int mph_case_set_state(mph_case* c, const mph_particles* parts, const double* wall_center)
{
    NEED(c);
    GUARD(mph::case_set_state(c, parts, wall_center))
}
int mph_export(mph_case* c, const char* name, void* dst, long* count, int* kind)
{
    NEED(c);
    GUARD(mph::case_export(c, name, dst, count, kind))
}
int mph_scalars(mph_case* c, double* out, int n) { NEED(c); GUARD(mph::case_scalars(c, out, n)) }
const char* mph_scalar_names(void) { return mph::scalar_names(); }
int mph_case_profile(mph_case* c, int enable) { NEED(c); GUARD(mph::case_profile(c, enable)) }
int mph_case_profile_read(mph_case* c, double* out, int n)
{
    NEED(c);
    if (!out) return mph::fail(MPH_ERR_ARG, "null output");
    GUARD(mph::case_profile_read(c, out, n))
}
long long mph_launch_count(void) { return mph::g_launch_count; }
const char* mph_last_error(void) { return mph::last_error(); }
const char* mph_version(void) { return "mph_gb300 0.1 (sm_103a)"; }

}  // extern "C"
