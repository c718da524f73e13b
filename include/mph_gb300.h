/*
 * mph_gb300.h - C ABI of the GB300 MPH-I time-step engine.
 *
 * The reference solver (MphImplicit, source/main.cpp) has no library API: its
 * boundary is the executable `MphImplicit <data> <grid> <prof%03d> <vtk%03d>
 * <log> <nthreads>` (main.cpp:313-330) plus the .data/.grid/.prof/.vtk files,
 * and every stage is a `static void f(void)` acting on file-static globals.
 * This header is the drop-in replacement for that path: each entry point below
 * names the reference function(s) it replaces.
 *
 * Conventions
 *   - Every function returns an int status (MPH_OK == 0, or an MPH_ERR_* code).
 *     No C++ exception crosses this boundary.
 *   - Host arrays are plain pointers; particle vectors are [count][3] doubles
 *     in the reference's layout (main.cpp:86-88), also for 2D cases.
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy stream).
 *   - A case handle is not thread safe; distinct handles are independent.
 *   - Particle order: like the reference, a case keeps its particles sorted by
 *     cell (main.cpp:1316-1378); mph_get_fields returns that order together with
 *     each particle's id (its index in the input).
 */
#ifndef MPH_GB300_H
#define MPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MPH_OK = 0,
    MPH_ERR_ARG = 1,          /* bad argument / null pointer                      */
    MPH_ERR_IO = 2,           /* file cannot be opened or is malformed            */
    MPH_ERR_INPUT = 3,        /* input violates a reference assumption            */
    MPH_ERR_CUDA = 4,         /* CUDA runtime error (message via mph_last_error) */
    MPH_ERR_NOMEM = 5,        /* device allocation failed                          */
    MPH_ERR_CAPACITY = 6,     /* a size bound was exceeded                         */
    MPH_ERR_NOT_CONVERGED = 7,/* CR reached its iteration cap                      */
    MPH_ERR_NAN = 8,          /* non-finite value detected in the solve            */
    MPH_ERR_STATE = 9         /* call out of order (e.g. stage before its inputs)  */
};

enum { MPH_TYPE_COUNT = 4 };  /* particle types 0,1 fluid; 2,3 wall (main.cpp:52-56) */

/* Keyword parameters of a .data file (main.cpp:523-563). */
typedef struct mph_params {
    double dt;
    double output_interval;
    double vtk_output_interval;
    double end_time;
    double radius_ratio_a;
    double radius_ratio_p;
    double radius_ratio_v;
    double density[MPH_TYPE_COUNT];
    double bulk_modulus[MPH_TYPE_COUNT];
    double bulk_viscosity[MPH_TYPE_COUNT];
    double shear_viscosity[MPH_TYPE_COUNT];
    double surface_tension[MPH_TYPE_COUNT];
    double interaction_ratio[MPH_TYPE_COUNT][MPH_TYPE_COUNT];
    double gravity[3];
    double wall_center[MPH_TYPE_COUNT][3];   /* rows 2,3 used */
    double wall_velocity[MPH_TYPE_COUNT][3];
    double wall_omega[MPH_TYPE_COUNT][3];
} mph_params;

/* Particle set of a .grid file (main.cpp:565-669). */
typedef struct mph_particles {
    int count;
    double time;
    double spacing;
    double domain_min[3];
    double domain_max[3];
    int* type;        /* [count]                              */
    double* pos;      /* [count][3]                           */
    double* vel;      /* [count][3]                           */
    int* id;          /* [count] particle ids, may be NULL    */
} mph_particles;

/* Per-particle fields returned by mph_get_fields (host buffers, [count] or
 * [count][3]).  Any pointer may be NULL to skip that field. */
typedef struct mph_fields {
    int* id;
    int* type;
    double* pos;
    double* vel;
    double* force;          /* Force (main.cpp:88)                       */
    double* vol_strain_p;   /* VolStrainP (main.cpp:147)                 */
    double* divergence_p;   /* DivergenceP, output steps only            */
    double* pressure_p;     /* PressureP, output steps only              */
    double* virial_p;       /* VirialPressureAtParticle, output steps    */
    int* neighbor_count;    /* NeighborCount                             */
} mph_fields;

/* Solve statistics of the last step (the reference logs the same numbers,
 * main.cpp:4381). */
typedef struct mph_solve_stats {
    int iterations;          /* CR iterations (mixed form: inner FP32 iterations, summed) */
    double rr0, rr, rs0, rs;
    int status;
    int outer_iterations;    /* mixed form: FP64 refinement steps (0 for the FP64 form) */
    int inner_form;          /* operator of the CR iterations: 0 FP64 blocks, 1 FP32 blocks,
                                2 FP32 pair terms (mixed form, factored, option inner_blocks 0) */
    int inner_local_blocks;  /* inner_form 2: row blocks (512 fluid rows) whose neighbours' values are
                                staged in shared memory, and the rest, which gather by column */
    int inner_gather_blocks;
    long long inner_local_cols;  /* distinct neighbour columns summed over the staged row blocks */
    int inner_ct_local_blocks;   /* particle blocks (256) of the transposed P-list apply staging s */
    int inner_reserved;          /* 0 */
} mph_solve_stats;

typedef struct mph_case mph_case;

/* Solver precision of a case. */
enum {
    MPH_PRECISION_FP64 = 0,   /* plain FP64 form: the reference algorithm as is    */
    MPH_PRECISION_MIXED = 1   /* FP32 inner CR + V-cycle, FP64 outer refinement      */
};

/* ---- files (replace readDataFile main.cpp:523, readGridFile main.cpp:565,
 *      writeProfFile main.cpp:696, writeVtkFile main.cpp:722) ---- */
int mph_read_data(const char* path, mph_params* out);
/* First call with buffers NULL to get the count; then with type/pos/vel set. */
int mph_read_grid(const char* path, mph_particles* out);
int mph_write_prof(const char* path, const mph_particles* parts);
int mph_case_write_vtk(mph_case* c, const char* path);
int mph_case_write_prof(mph_case* c, const char* path);

/* Full-precision checkpoint sidecar beside the .prof frames (which keep 7
 * digits, main.cpp:696-720): count, time, spacing, domain, the wall centres
 * (main.cpp:2123-2127) and per particle id, type, position and velocity in
 * binary.  mph_case_checkpoint stores a case in its current particle order;
 * a case created from the file (ids included) and given its order, wall
 * centres and time with mph_case_set_state continues bit for bit.
 * mph_read_checkpoint works like mph_read_grid: first call with NULL buffers
 * for the count; wall_center receives 4x3 doubles. */
int mph_write_checkpoint(const char* path, const mph_particles* parts, const double* wall_center);
int mph_read_checkpoint(const char* path, mph_particles* out, double* wall_center);
int mph_case_checkpoint(mph_case* c, const char* path);

/* ---- case lifetime ----
 * mph_case_create replaces readGridFile's allocation + initializeWeight /
 * initializeFluid / initializeWall / initializeDomain and the initial
 * calculateCellParticle / calculateNeighbor / density pass of main()
 * (main.cpp:347-375).  dim is 2 (the -D TWO_DIMENSIONAL build) or 3. */
int mph_case_create(const mph_params* prm, const mph_particles* parts, int dim,
                    int precision, void* stream, mph_case** out);
int mph_case_destroy(mph_case* c);
int mph_case_set_stream(mph_case* c, void* stream);

/* One or more full time steps (the body of main.cpp:386-474, without the
 * file output).  Returns MPH_ERR_NOT_CONVERGED if a solve hit its cap. */
int mph_step(mph_case* c, int nsteps);
/* ---- batching and serving (no counterpart in the reference, which runs one
 * case per process) ----
 * mph_batch_step advances independent cases concurrently: host worker
 * threads (one case at a time each) drive the cases' steps, every case on its
 * own stream (a case on the legacy stream gets a private non-blocking stream
 * for the call), so the kernels of different cases overlap on the device.
 * Returns when every case has taken nsteps steps; a case computes the same
 * bits alone or in a batch.  A case must not appear twice.  workers <= 0:
 * min(ncases, 2 x host threads, 64). */
int mph_batch_step(mph_case** cases, int ncases, int nsteps);
int mph_batch_step_workers(mph_case** cases, int ncases, int nsteps, int workers);

/* Upper bound of the device memory of one case (bytes): the admission unit
 * of the serving loop. */
int mph_case_footprint(const mph_params* prm, const mph_particles* parts, int dim, int precision,
                       long long* bytes);

/* Serving loop on the current device: submitted cases wait in arrival order
 * until their footprint fits the budget, are then created on their own
 * stream, kept resident and stepped round-robin by `workers` host threads
 * together with every other admitted case (continuous batching); a finished
 * case copies its fields to the caller's buffers (given at submit, kept valid
 * until the result is polled), frees its memory and admits the next. */
typedef struct mph_server mph_server;
typedef struct mph_server_result {
    long long ticket;
    int status;              /* MPH_OK, MPH_ERR_NOT_CONVERGED (a solve hit its cap), or the error */
    int steps;               /* steps completed */
    int particles;
    int pad;
    double submit_s, admit_s, done_s;   /* seconds since mph_server_create */
    long long footprint_bytes;
    char error[128];
} mph_server_result;
typedef struct mph_server_stats {
    long long budget_bytes, used_bytes;
    int pending, active, finished, pad;
    long long steps;
    double particle_steps, elapsed_s;
} mph_server_stats;
/* device: the CUDA device the server's cases live on (< 0: the current one);
 * one server per device makes the replicas of a multi-GPU node (host-side
 * assignment, no collective: serving.ReplicaDispatcher). */
int mph_server_create(long long budget_bytes, int workers, int device, mph_server** out);
/* out: fields to fill at completion (NULL: none); step_ms: `steps` floats
 * receiving each step's host-measured latency (NULL: none). */
int mph_server_submit(mph_server* s, const mph_params* prm, const mph_particles* parts, int dim, int precision,
                      int steps, const mph_fields* out, float* step_ms, long long* ticket);
/* Completed requests (up to max), waiting up to wait_ms for the first. */
int mph_server_poll(mph_server* s, mph_server_result* out, int max, int wait_ms, int* count);
int mph_server_stats_get(mph_server* s, mph_server_stats* out);
int mph_server_destroy(mph_server* s);
/* Solver tolerances (as mph_case_set_solver) and engine options (as
 * mph_case_set_option; the mixed form's own options skip FP64 cases) for the
 * cases of requests submitted from now on; each case gets them when it is
 * created.  An invalid option fails that request with the option's error.
 * Option "extrapolate" adds its velocity history to the admission footprint. */
int mph_server_set_solver(mph_server* s, double outer_rel_residual, double inner_rel_residual, int max_outer);
int mph_server_set_option(mph_server* s, const char* name, double value);

/* Solver tolerances.  outer_rel_residual: stop when ||b - A x|| / ||b|| is
 * below it (the reference stops at 1e-6: rr/rr0 < 1e-12, main.cpp:4346; this
 * is the default of both forms).  In the FP64 form it replaces only that
 * constant of the CR stop test (e.g. 1e-12 for a reference solution of a
 * tighter mixed solve).  Mixed form only: inner_rel_residual (relative
 * reduction of each FP32 inner solve, default 1e-3) and max_outer (refinement
 * steps, default 50; the FP64 form ignores both).  No counterpart in the
 * reference, whose tolerance is a constant. */
int mph_case_set_solver(mph_case* c, double outer_rel_residual, double inner_rel_residual, int max_outer);

/* Engine options (no counterpart in the reference):
 *   "cell_assembly" 1 (default) / 0: assemble A with the cell-block kernel
 *   where it applies, or with the per-row kernel only (same matrix).
 *   "graphs" 1 (default) / 0: replay the solver's iteration chunks as CUDA
 *   graphs, or launch every kernel directly (same arithmetic).  The chunks
 *   are recorded on a private side stream of the case and launched on the
 *   case stream.  A step waits on the host for its solver flags, so mph_step
 *   must not be called while the case stream is being captured.
 *   "factored" 1 (default) / 0: mixed form only.  1: where 2 RadiusP <
 *   MaxRadius, the FP64 operator of the outer residual is applied in factored
 *   form (viscous pair terms + C Lambda C^T through the transposed P-lists)
 *   and only FP32 blocks are assembled; CsrCofA then exports the FP32 blocks.
 *   0: FP64 blocks are assembled and copied to FP32.
 *   "mixed_extra_sweeps" 0 (default) .. 8: mixed form only, extra level-0
 *   smoothing sweeps before and after the rest of its V-cycle.
 *   "inner_blocks" 0 (default) / 1: factored mixed form only.  0: the inner
 *   FP32 operator runs on the sliced FP32 pair terms and P-lists and no
 *   blocks are written (CsrCofA export then fails with MPH_ERR_STATE; the
 *   block columns CsrIndA still export).  1: FP32 blocks are assembled and
 *   the inner SpMV runs on them.
 *   "inner_local" 1 (default) / 0: pair-term inner operator only.  1: each
 *   block of rows (particles, for the transposed P-lists) whose distinct
 *   neighbours fit stages their s in shared memory; 0: every block gathers s
 *   by column.  Both give the same bits. */
int mph_case_set_option(mph_case* c, const char* name, double value);
/* More options (no counterpart in the reference):
 *   "extrapolate" 0 (default) / 1 / 2: mixed form only.  The CR start value:
 *   the reference's v_n (main.cpp:4299-4308), or the linear / quadratic
 *   extrapolation of the start velocities of the last steps (the history
 *   follows the particles through the sort; mph_case_set_state clears it).
 *   "dense_coarse" 1 (default) / 0: mixed form only.  Solve the V-cycle's
 *   first one-block coarse level of at most 224 rows exactly with its dense
 *   FP32 inverse (built each step), or smooth it as the reference does.
 *   "cell_sort" 0 (default) / 1: the reference's bitonic network (the
 *   reference's particle order, bit for bit) or a counting sort of the cell
 *   keys (stable: inside a cell the previous order; same cell ranges).
 *   "mg_pre", "mg_post" 1 .. 4 (default 1 and 1): mixed form only.  Jacobi
 *   sweeps of the V-cycle's levels below level 0 before and after their
 *   coarse correction (the reference: 2 and 3, main.cpp:4189, 4238; the FP64
 *   form keeps those).
 *   "pair_block" 128 / 256 / 512 (default), "ct_block" 128 / 256 (default),
 *   "chunk" 4 / 8 (default) / 16 / 32: mixed form's launch shapes (block
 *   widths of the pair-term operator and of the transposed apply, CR
 *   iterations per captured graph chunk); mphimplicit_gb300/autotune.py
 *   chooses them by measurement.
 *   "keep_history" 0 (default) / 1: with 1, mph_case_set_state keeps the
 *   extrapolation history: the caller declares that the state continues this
 *   case's own steps in the case's particle order (e.g. the state it read back
 *   with mph_get_fields); the start value only changes the iteration count.
 *   "device_loop" 0 (default) / 1: mixed form with graphs.  1 runs the whole
 *   solve as one CUDA graph whose refinement and CR loops are device-side
 *   conditional while nodes (no host poll; same bits); not with profiling.
 *   "mg_depth" -1 (default) / 0 / 1 .. 24: mixed form only.  The inner CR's
 *   preconditioner: -1 point Jacobi (D^-1 from the pair terms; no multigrid
 *   levels are built, so their export fails with MPH_ERR_STATE), 0 the
 *   reference's V-cycle over every level (preconditionWithMultiGrid,
 *   main.cpp:4122), k the V-cycle cut after its first k levels.
 *   "mg_coarsest" 1 .. 8 (default 4): mixed form only, sweeps of a coarsest
 *   level run grid-wide (the reference's 4, main.cpp:4216).
 *   "pair_pack" 1 (default) / 0: pair-term inner operator only.  Slot records
 *   of 6 bytes (g as 11/11/10-bit fixed point of its slice's scale, and a
 *   2-byte block-local index) or 8 bytes (g in FP16 and the index).
 *   "pair_recompute" 0 (default) / 1: pair-term inner operator only; 1
 *   evaluates g per slot from the staged FP32 positions (2 bytes a slot).
 *   "batch_solve" 0 (default) / 1: in mph_batch_step, the point-Jacobi
 *   mixed cases on the pair path solve together: each refinement phase's CR
 *   iterations are one launch per kernel over all of them (a block runs its
 *   case's single-case kernel body with that case's block decomposition, so
 *   every case keeps the bits of its own solve); the stages before the solve
 *   then run for all cases before any solve starts.
 *   "pair_fuse" 0 (default) / 1: point-Jacobi mixed form on the pair path;
 *   1 writes the sliced pair terms in one kernel without the per-slot
 *   pair-term list (16 bytes a neighbour slot less device memory; slower).
 *   "split_apply" 0 (default) / 1: pair-term inner operator only; 1 runs the
 *   transposed apply on a side stream beside the viscous kernel and adds
 *   lambda C t in a third kernel.  The forms of these three options reach
 *   solutions within the refinement tolerance of each other (their inner
 *   operators differ in rounding or summation order only). */

int mph_case_count(mph_case* c, int* count, int* fluid_count);
int mph_case_time(mph_case* c, double* time);
int mph_get_fields(mph_case* c, mph_fields* out);
int mph_get_solve_stats(mph_case* c, mph_solve_stats* out);

/* ---- stage entry points (parity tests), in step order ----
 * step_begin  : calculateConvection, calculateWall, calculatePeriodicBoundary,
 *               resetForce (main.cpp:1678, 2089, 4741, 1690)
 * cellsort    : calculateCellParticle (main.cpp:1164)
 * neighbors   : calculateNeighbor (main.cpp:1382)
 * explicit    : calculateDensityA .. calculateAcceleration (main.cpp:413-430)
 * assemble    : calculateMatrixA, calculateMatrixC, multiplyMatrixC
 *               (main.cpp:2137, 2354, 2562)
 * mg_build    : calculateMultiGridMatrix (main.cpp:2761)
 * solve       : solveWithConjugatedGradient (main.cpp:4270)
 * step_end    : Time += Dt and the wall-centre update (main.cpp:470, 2123)
 * output_fields: calculateDivergenceP, calculatePressureP,
 *               calculateViscosityV, calculateVirialStressAtParticle
 *               (main.cpp:454-457) */
int mph_stage_step_begin(mph_case* c);
int mph_stage_cellsort(mph_case* c);
int mph_stage_neighbors(mph_case* c);
int mph_stage_explicit(mph_case* c);
int mph_stage_assemble(mph_case* c);
int mph_stage_mg_build(mph_case* c);
int mph_stage_solve(mph_case* c);
int mph_stage_step_end(mph_case* c);
int mph_stage_output_fields(mph_case* c);

/* Replace the particle state of a case (positions, velocities, types, ids in
 * the given order) and the wall centres / time, e.g. to continue from a state
 * produced elsewhere.  wall_center may be NULL. */
int mph_case_set_state(mph_case* c, const mph_particles* parts, const double* wall_center /*[4][3]*/);

/* Named device arrays copied to host in the reference's layout, for tests.
 * kind: 0 int32, 1 int64, 2 double.  With dst == NULL only *count and *kind
 * are returned.  Names follow the reference globals (e.g. "CellIndex",
 * "NeighborInd", "CsrCofA", "VectorB", "MultiGridCsrCofA:<level>"). */
int mph_export(mph_case* c, const char* name, void* dst, long* count, int* kind);
/* Scalars: fills out[] (capacity n) in the order of mph_scalar_names(). */
int mph_scalars(mph_case* c, double* out, int n);
const char* mph_scalar_names(void);

/* Measurement support (no counterpart in the reference, which times its
 * phases with clock(), main.cpp:310-311 and 480-491).
 * mph_case_profile: enable (1) / disable (0) CUDA-event timing on the case
 * stream and reset the accumulators.
 * mph_case_profile_read: fills out[] with the accumulated milliseconds of the
 * stages step_begin, cellsort, neighbors, explicit, assemble, mg_build, solve
 * (7 values), then the milliseconds and launch counts of the kernel classes
 * SpMV, V-cycle, A assembly, neighbour search (4 + 4 values), then the
 * sliced-ELL slot count, the neighbour and P-neighbour list lengths of the
 * last step.  Returns the number of values available. */
int mph_case_profile(mph_case* c, int enable);
int mph_case_profile_read(mph_case* c, double* out, int n);
/* Number of kernel launches this library has issued since it was loaded. */
long long mph_launch_count(void);

const char* mph_last_error(void);
const char* mph_version(void);

/* Residual norms of the solved system, with no device allocation by the call
 * (no counterpart in the reference).  out[0] = ||b - A x||^2 and out[1] =
 * ||b||^2 (host memory) for the system of the last mph_stage_solve; valid
 * between that stage and mph_stage_step_end, else MPH_ERR_STATE (also when
 * the step assembled no FP64 blocks: mixed form, option "factored").  Its scratch
 * is one fixed per-device array of 262,400 bytes, so it serves cases of at
 * most 2,097,152 fluid particles (larger: MPH_ERR_CAPACITY).  The first
 * mph_case_create on a device reserves that array and looks up its address
 * (before the case takes its own memory), so the check itself needs no device
 * memory.  Calls that overlap on the GPU share the array and race: serialise
 * them.  The address is kept for the life of the process: do not use the
 * check across a reset of the device (cudaDeviceReset).  For servers whose
 * device memory is fully committed to resident cases, where a per-call
 * allocation could fail and a free would stall every stream. */
int mph_residual_noalloc(mph_case* c, double* out);

#ifdef __cplusplus
}
#endif
#endif /* MPH_GB300_H */
