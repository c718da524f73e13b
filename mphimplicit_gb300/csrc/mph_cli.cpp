// mph_cli.cpp - command-line drop-in for the reference executable.
//
//   mph_gb300 [-2|-3] <data> <grid> <prof%03d> <vtk%03d> <log> [nthreads]
//
// Same arguments and defaults as MphImplicit / MphImplicit_3d
// (main.cpp:313-330, 58-62; the 2D/3D choice is a flag instead of a build
// target, default 3D), same time loop and output cadence (main.cpp:381-474):
// a .prof frame whenever Time passes OutputNext, a .vtk frame (with the
// output-step fields) whenever it passes VtkOutputNext, and the CR log line
// "iter, rr0, rr, rs0, rs" after every solve.  nthreads is accepted and
// ignored (the work runs on the GPU).
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/mph_gb300.h"

static FILE* g_log = nullptr;

static void logf(const char* fmt, ...)
{
    va_list a, b;
    va_start(a, fmt);
    va_copy(b, a);
    if (g_log) std::vfprintf(g_log, fmt, a);
    std::vfprintf(stderr, fmt, b);
    va_end(a);
    va_end(b);
}

static int check(int st, const char* what)
{
    if (st != MPH_OK && st != MPH_ERR_NOT_CONVERGED) {
        logf("error in %s: %s\n", what, mph_last_error());
        std::exit(1);
    }
    return st;
}

int main(int argc, char** argv)
{
    int dim = 3;
    int a0 = 1;
    if (argc > 1 && (std::strcmp(argv[1], "-2") == 0 || std::strcmp(argv[1], "-3") == 0)) {
        dim = argv[1][1] - '0';
        a0 = 2;
    }
    const char* data = argc > a0 ? argv[a0] : "sample.data";
    const char* grid = argc > a0 + 1 ? argv[a0 + 1] : "sample.grid";
    const char* prof = argc > a0 + 2 ? argv[a0 + 2] : "sample%03d.prof";
    const char* vtk = argc > a0 + 3 ? argv[a0 + 3] : "sample%03d.vtk";
    const char* logn = argc > a0 + 4 ? argv[a0 + 4] : "sample.log";
    g_log = std::fopen(logn, "w");
    {
        time_t t = time(nullptr);
        logf("start reading files at %s\n", ctime(&t));
    }
    mph_params prm;
    check(mph_read_data(data, &prm), "reading the data file");
    mph_particles parts{};
    check(mph_read_grid(grid, &parts), "reading the grid file");
    std::vector<int> type(parts.count);
    std::vector<double> pos(3 * (size_t)parts.count), vel(3 * (size_t)parts.count);
    parts.type = type.data();
    parts.pos = pos.data();
    parts.vel = vel.data();
    check(mph_read_grid(grid, &parts), "reading the grid file");
    mph_case* c = nullptr;
    check(mph_case_create(&prm, &parts, dim, MPH_PRECISION_FP64, nullptr, &c), "creating the case");
    check(mph_case_write_vtk(c, "output.vtk"), "writing output.vtk");
    {
        time_t t = time(nullptr);
        logf("start main roop at %s\n", ctime(&t));
    }
    double Time = parts.time;
    const double Dt = prm.dt;
    int iStep = (int)(Time / Dt);
    double OutputNext = Time, VtkOutputNext = Time;
    const clock_t c0 = clock();
    while (Time < prm.end_time + 1.0e-5 * Dt) {
        if (Time + 1.0e-5 * Dt >= OutputNext) {
            char fn[1024];
            std::snprintf(fn, sizeof fn, prof, iStep);
            check(mph_case_write_prof(c, fn), "writing a prof file");
            logf("@ Prof Output Time : %e\n", Time);
            OutputNext += prm.output_interval;
        }
        check(mph_stage_step_begin(c), "step");
        check(mph_stage_cellsort(c), "cell sort");
        check(mph_stage_neighbors(c), "neighbour search");
        check(mph_stage_explicit(c), "explicit stage");
        check(mph_stage_assemble(c), "assembly");
        check(mph_stage_mg_build(c), "multigrid build");
        check(mph_stage_solve(c), "solve");
        mph_solve_stats st;
        mph_get_solve_stats(c, &st);
        logf("iter,=%d, rr0=,%e, rr=,%e, rs0=,%e, rs=,%e\n", st.iterations, st.rr0, st.rr, st.rs0, st.rs);
        if (Time + 1.0e-5 * Dt >= VtkOutputNext) {
            check(mph_stage_output_fields(c), "output fields");
            char fn[1024];
            std::snprintf(fn, sizeof fn, vtk, iStep);
            check(mph_case_write_vtk(c, fn), "writing a vtk file");
            logf("@ Vtk Output Time : %e\n", Time);
            VtkOutputNext += prm.vtk_output_interval;
        }
        check(mph_stage_step_end(c), "step end");
        Time += Dt;
        ++iStep;
    }
    {
        time_t t = time(nullptr);
        logf("end main roop at %s\n", ctime(&t));
        logf("total:                   %lf [CPU sec]\n", (double)(clock() - c0) / CLOCKS_PER_SEC);
    }
    mph_case_destroy(c);
    if (g_log) std::fclose(g_log);
    return 0;
}
