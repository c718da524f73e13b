// Reference harness: test infrastructure only.
//
// This translation unit is compiled by oracle/Makefile against the UNMODIFIED
// reference solver sources (MphImplicit source/main.cpp, log.cpp, errorfunc.cpp)
// found in the reference checkout given by REF_DIR.  It renames the reference's
// main() and exposes the reference's own static stage functions one by one, so
// that fixture scripts can run one time step stage by stage and read the
// reference's global state after each stage.  Nothing in the shipped library
// links or calls this file; its output (oracle/_ref/*.so) is never committed.
//
// Stage order follows the reference time loop, source/main.cpp:386-474.

#define main mph_reference_main
#include "main.cpp"
#undef main
#undef malloc
#undef fopen

#include <cstring>

extern "C" {

// Initialisation exactly as main() does it (source/main.cpp:331-375), minus the
// "output.vtk" write.  ParticleIndex is never initialised by the reference
// (main.cpp:586); it is seeded here with the file order so particles carry ids.
int ref_init(const char* data, const char* grid, const char* logpath)
{
    log_open(logpath);
    readDataFile((char*)data);
    readGridFile((char*)grid);
    for (int i = 0; i < ParticleCount; ++i) ParticleIndex[i] = i;
    initializeWeight();
    initializeFluid();
    initializeWall();
    initializeDomain();
    calculateCellParticle();
    calculateNeighbor();
    calculateDensityA();
    calculateGravityCenter();
    calculateDensityP();
    freeNeighbor();
    OutputNext = Time;
    VtkOutputNext = Time;
    fflush(NULL);
    return ParticleCount;
}

// main.cpp:398-404
void ref_step_begin(void) { calculateConvection(); calculateWall(); calculatePeriodicBoundary(); resetForce(); }
// main.cpp:408
void ref_cellsort(void) { calculateCellParticle(); }
// main.cpp:409
void ref_neighbor(void) { calculateNeighbor(); }
// main.cpp:413-430
void ref_explicit(void)
{
    calculateDensityA(); calculateGravityCenter(); calculateDensityP();
    calculatePhysicalCoefficients(); calculatePressureA(); calculateDiffuseInterface();
    calculateGravity(); calculateAcceleration();
}
// main.cpp:435-438 (matrix C is kept alive until ref_free_c so it can be read)
void ref_assemble_ac(void) { calculateMatrixA(); calculateMatrixC(); }
void ref_multiply_c(void) { multiplyMatrixC(); }
void ref_free_c(void) { freeMatrixC(); }
// main.cpp:442
void ref_mg_build(void) { calculateMultiGridMatrix(); }
// main.cpp:445
void ref_solve(void) { solveWithConjugatedGradient(); fflush(NULL); }
// main.cpp:454-457
void ref_output_fields(void) { calculateDivergenceP(); calculatePressureP(); calculateViscosityV(); calculateVirialStressAtParticle(); }
// main.cpp:447-471
void ref_step_end(void) { freeMultiGridMatrix(); freeMatrixA(); freeNeighbor(); Time += Dt; }
void ref_free_mg(void) { freeMultiGridMatrix(); }
void ref_free_a(void) { freeMatrixA(); }
void ref_free_neighbor(void) { freeNeighbor(); }
void ref_advance_time(void) { Time += Dt; }

void ref_write_vtk(const char* path) { writeVtkFile((char*)path); }
void ref_write_prof(const char* path) { writeProfFile((char*)path); }

// Scalars of the reference state, in a fixed order documented by ref_scalar_names.
static const char* kScalarNames =
    "Time,Dt,ParticleCount,FluidParticleBegin,FluidParticleEnd,WallParticleBegin,WallParticleEnd,"
    "TotalCellCount,CellCount0,CellCount1,CellCount2,PowerParticleCount,NeighborIndCount,NeighborIndCountP,"
    "NonzeroCountA,NonzeroCountC,MultiGridDepth,MaxRadius,RadiusA,RadiusG,RadiusP,RadiusV,N0a,N0p,R2g,"
    "Swa,Swg,Swp,Swv,CofK,ParticleVolume,ParticleSpacing";
const char* ref_scalar_names(void) { return kScalarNames; }
int ref_scalars(double* out)
{
    const double v[] = {
        Time, Dt, (double)ParticleCount, (double)FluidParticleBegin, (double)FluidParticleEnd,
        (double)WallParticleBegin, (double)WallParticleEnd, (double)TotalCellCount,
        (double)CellCount[0], (double)CellCount[1], (double)CellCount[2], (double)PowerParticleCount,
        (double)NeighborIndCount, (double)NeighborIndCountP, (double)NonzeroCountA, (double)NonzeroCountC,
        (double)MultiGridDepth, MaxRadius, RadiusA, RadiusG, RadiusP, RadiusV, N0a, N0p, R2g,
        Swa, Swg, Swp, Swv, CofK, ParticleVolume, ParticleSpacing};
    const int n = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n; ++i) out[i] = v[i];
    return n;
}

// Named array access.  kind: 0=int32, 1=int64, 2=double.  Returns element count
// (or -1 for an unknown name).  Sizes follow the allocations in the reference.
long ref_array(const char* name, void** ptr, int* kind)
{
    const long N = ParticleCount;
    const long Nf3 = (long)DIM * (FluidParticleEnd - FluidParticleBegin);
#define ARR(nm, p, k, n) if (strcmp(name, nm) == 0) { *ptr = (void*)(p); *kind = (k); return (long)(n); }
    ARR("Property", Property, 0, N)
    ARR("ParticleIndex", ParticleIndex, 0, N)
    ARR("Position", Position, 2, N * DIM)
    ARR("Velocity", Velocity, 2, N * DIM)
    ARR("Force", Force, 2, N * DIM)
    ARR("Mass", Mass, 2, N)
    ARR("Kappa", Kappa, 2, N)
    ARR("Lambda", Lambda, 2, N)
    ARR("Mu", Mu, 2, N)
    ARR("DensityA", DensityA, 2, N)
    ARR("GravityCenter", GravityCenter, 2, N * DIM)
    ARR("PressureA", PressureA, 2, N)
    ARR("VolStrainP", VolStrainP, 2, N)
    ARR("DivergenceP", DivergenceP, 2, N)
    ARR("PressureP", PressureP, 2, N)
    ARR("VirialPressureAtParticle", VirialPressureAtParticle, 2, N)
    ARR("VirialStressAtParticle", VirialStressAtParticle, 2, N * DIM * DIM)
    ARR("CellIndex", CellIndex, 0, PowerParticleCount)
    ARR("CellParticle", CellParticle, 0, PowerParticleCount)
    ARR("CellFluidParticleBegin", CellFluidParticleBegin, 0, TotalCellCount)
    ARR("CellFluidParticleEnd", CellFluidParticleEnd, 0, TotalCellCount)
    ARR("CellWallParticleBegin", CellWallParticleBegin, 0, TotalCellCount)
    ARR("CellWallParticleEnd", CellWallParticleEnd, 0, TotalCellCount)
    ARR("NeighborCount", NeighborCount, 0, N)
    ARR("NeighborFluidCount", NeighborFluidCount, 0, N)
    ARR("NeighborCountP", NeighborCountP, 0, N)
    ARR("NeighborPtr", NeighborPtr, 1, N + 1)
    ARR("NeighborPtrP", NeighborPtrP, 1, N + 1)
    ARR("NeighborInd", NeighborInd, 0, NeighborIndCount)
    ARR("NeighborIndP", NeighborIndP, 0, NeighborIndCountP)
    ARR("CsrPtrA", CsrPtrA, 1, Nf3 + 1)
    ARR("CsrIndA", CsrIndA, 0, NonzeroCountA)
    ARR("CsrCofA", CsrCofA, 2, NonzeroCountA)
    ARR("VectorB", VectorB, 2, Nf3)
    ARR("CsrPtrC", CsrPtrC, 1, Nf3 + 1)
    ARR("CsrIndC", CsrIndC, 0, NonzeroCountC)
    ARR("CsrCofC", CsrCofC, 2, NonzeroCountC)
    ARR("VectorP", VectorP, 2, N)
    ARR("InvDiagA", InvDiagA, 2, Nf3)
    ARR("WallCenter", WallCenter, 2, WALL_END * DIM)
    ARR("WallRotation", WallRotation, 2, WALL_END * DIM * DIM)
#undef ARR
    return -1;
}

// Multigrid level geometry: min[3], max[3], count[3] of level `level`.
int ref_mg_level_geom(int level, int* out9)
{
    if (level < 0 || level >= MultiGridDepth) return -1;
    for (int d = 0; d < DIM; ++d) {
        out9[d] = MultiGridCellMin[level][d];
        out9[3 + d] = MultiGridCellMax[level][d];
        out9[6 + d] = MultiGridCount[level][d];
    }
    return 0;
}

// Multigrid level matrix (CSR view into the reference arrays) and its inverse
// diagonal: rows = DIM*cells of the level.
int ref_mg_level_matrix(int level, int** ptr, int** ind, double** cof, double** invd, int* rows)
{
    if (level < 0 || level >= MultiGridDepth) return -1;
    const int slot = MultiGridDepth - level - 1;
    const int offPtr = MultiGridOffset[slot] * OneGridSizeCsrPtrA + slot;
    const int offInd = MultiGridOffset[slot] * OneGridSizeCsrIndA;
    const int offInv = MultiGridOffset[slot] * OneGridSizeInvDiagA;
    *ptr = &MultiGridCsrPtrA[offPtr];
    *ind = &MultiGridCsrIndA[offInd];
    *cof = &MultiGridCsrCofA[offInd];
    *invd = &MultiGridInvDiagA[offInv];
    *rows = DIM * MultiGridCount[level][0] * MultiGridCount[level][1] * MultiGridCount[level][2];
    return 0;
}

}  // extern "C"
