/*
 * mph_oracle.h - CPU oracle of the MPH-I time step (TEST INFRASTRUCTURE).
 *
 * A plain C++ restatement of the reference algorithm (MphImplicit
 * source/main.cpp), used only by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py as the checker and the CPU
 * baseline.  The shipped library never links or calls it.
 *
 * Storage follows the reference: 3 components per vector and 3x3 blocks even
 * for 2D cases (the reference keeps DIM=3 in its 2D build, main.cpp:49).
 */
#ifndef MPH_ORACLE_H
#define MPH_ORACLE_H
#include "../include/mph_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpho_case mpho_case;

mpho_case* mpho_create(const mph_params* prm, const mph_particles* parts, int dim);
void mpho_destroy(mpho_case* c);
void mpho_set_threads(int n);

/* stages, reference order (main.cpp:386-474) */
void mpho_init(mpho_case* c);          /* main.cpp:369-375 initial pass        */
void mpho_step_begin(mpho_case* c);    /* convection, wall, periodic, reset     */
void mpho_cellsort(mpho_case* c);
void mpho_neighbors(mpho_case* c);
void mpho_explicit(mpho_case* c);
void mpho_assemble(mpho_case* c);      /* A, C, b, p, b-=Cp, A+=C Lambda C^T    */
void mpho_mg_build(mpho_case* c);
int  mpho_solve(mpho_case* c);         /* returns CR iteration count            */
void mpho_step_end(mpho_case* c);
void mpho_output_fields(mpho_case* c);
int  mpho_step(mpho_case* c, int nsteps);
/* CR stop test ||r||/||b|| < rel (the reference's constant, main.cpp:4346, is
 * rel = 1e-6, i.e. rr/rr0 < 1e-12; only that constant changes). */
void mpho_set_tolerance(mpho_case* c, double rel);

/* Named arrays (same names and layouts as the reference globals). */
long mpho_array(mpho_case* c, const char* name, void** ptr, int* kind);
int  mpho_scalars(mpho_case* c, double* out);
const char* mpho_scalar_names(void);
int  mpho_solve_stats(mpho_case* c, double* out5);   /* iter, rr0, rr, rs0, rs */
int  mpho_mg_level_geom(mpho_case* c, int level, int* out9);
int  mpho_mg_level_matrix(mpho_case* c, int level, double** cof, double** invd, int* rows, int* width);
/* Replace particle state (sorted-order arrays) and wall centres. */
void mpho_set_state(mpho_case* c, const mph_particles* parts, const double* wall_center);

#ifdef __cplusplus
}
#endif
#endif
