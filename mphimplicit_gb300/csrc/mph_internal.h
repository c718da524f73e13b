// mph_internal.h - internal types of the GB300 MPH-I engine.
//
// Device data layout (DIM = D in {2,3}; particles in cell order, fluid first):
//   positions / velocities / forces : double[N][VS], VS = 2 (2D) or 4 (3D,
//                                      padded so one particle is one 32-byte sector)
//   pos32                           : float[N][VS] copy used only to pre-classify
//                                      neighbour candidates (exact FP64 decides
//                                      every pair near a radius)
//   poslo32                         : float[N][VS], x - pos32 rounded to FP32:
//                                      (pos32, poslo32) is a two-float position
//                                      for the FP32 pair terms of the mixed form
//   neighbour lists                 : CSR, int64 row pointers, int32 columns,
//                                      as the reference (main.cpp:92-97)
//   matrix A                        : sliced ELL of DxD blocks, 32 block rows per
//                                      slice, slice width = longest row; inside a
//                                      slice value (k, comp, lane) sits at
//                                      base + (k*D*D + comp)*32 + lane, so a warp
//                                      (one lane per row) reads 256 contiguous bytes
//   matrix C                        : per fluid particle, D values per P-neighbour,
//                                      aligned with the P-list (row-contiguous)
//   multigrid level L               : dense 3^D-cell block stencil per grid cell,
//                                      entry-major: row = cell*D + r, entry
//                                      e = slot*D + s, value at e*rows + row.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <string>
#include <functional>
#include <vector>

#include "../../include/mph_gb300.h"

namespace mph {

constexpr int kTypeCount = 4;
constexpr int kSliceRows = 32;         // rows per sliced-ELL slice (one warp)
constexpr int kMaxLevels = 24;

// Parameters every kernel reads, passed by value.
struct DevParams {
    int dim;
    int N, Nf, nPow, powExp;
    int cc[3], T;
    double dmin[3], dw[3], hw[3], wsafe[3];   // wsafe: Mod fast-path bound
    double cw[3];
    double l0, vol, dt;
    double rA, rG, rP, rV, maxR;
    double maxR2, rP2;
    double kfa, kfg, kfp, kfv;                 // (1/Sw)/h^dim per kernel
    double N0a, N0p, R2g, cofK;
    double cofA[kTypeCount];
    double density[kTypeCount], bulk[kTypeCount], lambda[kTypeCount], mu[kTypeCount];
    double ratio[kTypeCount][kTypeCount];
    double gravity[3];
    double visc;                               // 8 (2D) or 10 (3D)
    double inv_rv, m2h_rv, inv_rp, m2h_rp;     // 1/h and -2/h of the V and P kernels (assembly)
    double muij[kTypeCount][kTypeCount];       // harmonic mean 2 mu_i mu_j / (mu_i + mu_j)
    double inert64[kTypeCount];                // density * vol / vol / dt in that order (the reference's inertia), once
    float maxR2_lo, maxR2_hi, rP2_lo, rP2_hi;  // FP32 pre-classification band
    float w32[3], hw32[3];
    float inert32[kTypeCount];                 // FP32 density/dt and bulk viscosity (mixed-form kernels)
    float lambda32[kTypeCount];
    float vm32[kTypeCount][kTypeCount];        // FP32 visc * muij, -kfv * m2h_rv, 1/h, rV^2 (pair terms)
    float wdA32, inv_rv32, rV2_32;
    int exact_only;                            // 1: skip the FP32 pre-classification
    int surface;                               // 1 if any CofA != 0
};

struct LevelGeom {
    int mn[3], mx[3], cnt[3], st[3];
    int cells, rows;      // rows = D*cells
    long off_vec;         // offset into the level vector pool (rows)
    long off_cof;         // offset into the level coefficient pool
};

// Device buffers of one case.
struct DeviceState {
    // particles
    double *pos = nullptr, *vel = nullptr, *force = nullptr;
    double *pos_alt = nullptr, *vel_alt = nullptr;
    float* pos32 = nullptr;
    float* poslo32 = nullptr;
    int *type = nullptr, *id = nullptr, *type_alt = nullptr, *id_alt = nullptr;
    double *densA = nullptr, *gcen = nullptr, *presA = nullptr, *vsp = nullptr;
    double *divP = nullptr, *presP = nullptr, *virP = nullptr, *virS = nullptr;
    // cell list
    int *key = nullptr, *perm = nullptr, *bucket = nullptr;   // bucket: [2T+1] starts
    int* sort_cnt = nullptr;            // counting sort: bucket counts, then write cursors [2T+1]
    long long* sort_off = nullptr;      // counting sort: bucket offsets [2T+1]
    // neighbours
    int *nc = nullptr, *nfc = nullptr, *ncp = nullptr;
    long long *nptr = nullptr, *nptrP = nullptr;
    int *nind = nullptr, *nindP = nullptr;
    long long cap_nind = 0, cap_nindP = 0;
    // matrix A (sliced ELL)
    long long *sptr = nullptr;     // [nslices+1], block slots
    int* swidth = nullptr;         // [nslices]
    int* acol = nullptr;           // [slots]
    double* aval = nullptr;        // [slots*D*D]
    float* aval32 = nullptr;       // mixed precision copy
    long long cap_slots = 0, cap_aval = 0, cap_aval32 = 0;
    double *bvec = nullptr, *invDiag = nullptr;
    int* selfk = nullptr;          // position of the self block in each row
    // matrix C and source p
    double *cval = nullptr, *pvec = nullptr;
    long long cap_cval = 0;
    // level-0 partial stencils per fluid row: [Nf][S][D*D]
    double* part = nullptr;
    // transpose of the fluid P-lists (cell-block assembly) and per-cell
    // fallback flags; capacities in bytes
    int* ct_cnt = nullptr;
    long long* ct_ptr = nullptr;
    int* ct_j = nullptr;
    double* ct_v = nullptr;
    int* cell_flags = nullptr;
    int* dmax = nullptr;
    void* ct_tmp = nullptr;         // (row, column, P-slot) per entry before placement
    long long cap_ct_cnt = 0, cap_ct_ptr = 0, cap_ct_j = 0, cap_ct_v = 0, cap_cell_flags = 0, cap_ct_tmp = 0;
    // mixed form, factored FP64 operator: (e, f) per neighbour slot of the
    // fluid rows in FP32, t = C^T x per particle, FP32 copy of x
    float4* pe32 = nullptr;
    long long cap_pairs = 0;
    double* tct = nullptr;
    float* x32 = nullptr;
    float* ct_v32 = nullptr;        // FP32 copy of ct_v
    long long cap_ct_v32 = 0;
    float* arow32 = nullptr;        // FP32 blocks, row-contiguous at neighbour-list offsets (before slicing)
    long long cap_arow32 = 0;
    float* cval32 = nullptr;        // FP32 copy of the fluid rows' C values
    long long cap_cval32 = 0;
    float* tct32 = nullptr;         // t = C^T x of the FP32 inner operator
    // FP32 inner operator on pair terms: g = sqrt(f) e per fluid slot in the
    // sliced (k, component, lane) layout, the FP32 diagonal block (inertia +
    // sum f e (x) e, 6 entries a row), C scaled by lambda of its P-neighbour
    // (aligned with the P-lists), and the P-lists (lambda-scaled C) and
    // transposed P-lists (C) in sliced layouts: slice pointers, widths,
    // columns, D FP32 values a slot
    float* pes32 = nullptr;
    long long cap_pes32 = 0;
    unsigned short* grec16 = nullptr;  // inner operator slot records: g in FP16 scaled per slice (D halves), block-local index (4th)
    long long cap_grec16 = 0;
    float* pscale = nullptr;           // per slice: g = FP16 g * pscale
    unsigned* grec32 = nullptr;        // option pair_pack: g per fluid slot, packed fixed point (sliced layout)
    long long cap_grec32 = 0;
    unsigned short* lcol16 = nullptr;  // options pair_pack, pair_recompute: block-local index per fluid slot (sliced layout)
    long long cap_lcol16 = 0;
    int* wrap32 = nullptr;             // set when a pair of this step's fluid rows is a periodic image
    float4* pt32 = nullptr;            // FP32 position (high part) and type bits per particle (3D: pos32 itself)
    // block-local neighbour columns of the inner operator (per block its
    // distinct neighbours, kUMax a block, and their count or -1; their
    // maximum, the staged blocks and their columns after the blocks)
    int* uniq = nullptr;
    long long cap_uniq = 0;
    int* ucount = nullptr;
    long long cap_ucount = 0;
    // the same for the transposed P-lists of k_ct_apply32's particle blocks
    // (the rank replaces the column in the slot's record)
    int* ctuniq = nullptr;
    long long cap_ctuniq = 0;
    int* ctucount = nullptr;
    long long cap_ctucount = 0;
    int* ccell = nullptr;              // packed cell coordinates of every particle (pair path)
    double* io3 = nullptr;             // host-layout staging, 2 x N x 3 doubles (state upload, field download)
    double *vprev = nullptr, *vprev_alt = nullptr;   // mixed form, option "extrapolate": start velocities of the two previous
                                                     // steps (2 x N x VS: v_{n-1}, then v_{n-2})
    int* wkey = nullptr;               // per particle k, kWBins cells of its transposed P-list and
    float* wval = nullptr;             // the sums of C_jk over each (level-0 stencils of the pair path)
    float* sdiag32 = nullptr;
    double* sdiag64 = nullptr;         // FP64 wall part of the viscous diagonal block per fluid row (8 doubles: 6 used)
    float* cvl32 = nullptr;
    long long cap_cvl32 = 0;
    long long *psptr = nullptr, *ctsptr = nullptr;
    int *pswidth = nullptr, *ctswidth = nullptr;
    int *pscol = nullptr, *ctscol = nullptr;   // (unused: the columns live in the records)
    float *psval = nullptr, *ctsval = nullptr; // 16-byte slot records: D values (zero-padded), the column
    long long cap_pscol = 0, cap_psval = 0, cap_ctscol = 0, cap_ctsval = 0;
    // multigrid
    double *mg_cof = nullptr, *mg_invd = nullptr;
    double *mg_q = nullptr, *mg_s = nullptr, *mg_r = nullptr, *mg_res = nullptr;   // Q, S ping-pong pair, residual
    float *mg_cof32 = nullptr, *mg_invd32 = nullptr;
    float* mg_dinv32 = nullptr;     // mixed form: dense inverse of the exactly solved coarse level
    long long cap_mg_dinv32 = 0;
    float *mg_q32 = nullptr, *mg_s32 = nullptr, *mg_r32 = nullptr, *mg_res32 = nullptr;
    float* v32 = nullptr;           // mixed form: 7 FP32 CR vectors + FP32 D^-1, each D*Nf
    long long cap_mg_cof = 0, cap_mg_vec = 0, cap_mg_cof32 = 0, cap_mg_vec32 = 0;
    // solver vectors [D*Nf]
    double *x = nullptr, *r = nullptr, *s = nullptr, *y = nullptr, *p = nullptr, *q = nullptr, *u = nullptr;
    double* partials = nullptr;     // block partial sums for reductions
    double* scal = nullptr;         // solver scalars on device
    int* flags = nullptr;           // device status flags
    // misc
    int* bbox = nullptr;            // fluid-cell bounding box (6 ints)
    long long* totals = nullptr;    // scan totals read back by the host
    void* scan_tmp = nullptr;
    size_t scan_tmp_bytes = 0;
};

// Kernel launches issued by this library (host-side count, all threads), and
// the calling thread's own count (used to count the launches of a capture).
extern std::atomic<long long> g_launch_count;
extern thread_local long long t_launch_count;
#define MPH_COUNT_LAUNCH() (++::mph::g_launch_count, ++::mph::t_launch_count)

// Optional CUDA-event timing on the case stream: per stage and per launch of
// the hot kernels.
enum { kProfStages = 8, kProfKernels = 4 };                 // kernels: spmv, vcycle, assemble_a, neighbors
struct Profile {
    bool on = false;
    double stage_ms[kProfStages] = {};
    double kern_ms[kProfKernels] = {};
    long long kern_n[kProfKernels] = {};
    std::vector<cudaEvent_t> pool;                           // free events
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
};

}  // namespace mph

// Opaque handle of the C ABI.
struct mph_case {
    int dim = 3;
    int precision = MPH_PRECISION_FP64;
    cudaStream_t stream = nullptr;
    int device = 0;
    mph_params prm{};
    mph::DevParams dp{};
    double time = 0.0;
    double z_plane = 0.0;               // z of every particle of a 2D case
    double prm_domain_min[3]{}, prm_domain_max[3]{};   // the .grid header's domain
    double wallC[4][3]{}, wallV[4][3]{}, wallW[4][3]{}, wallR[4][3][3]{};
    double Swa = 1, Swg = 1, Swp = 1, Swv = 1;
    int fB = 0, fE = 0, wB = 0, wE = 0;
    long long nnb = 0, nnbP = 0;        // neighbour list totals of the current step
    int nslices = 0;
    long long nslots = 0;
    int depth = 0;
    std::vector<mph::LevelGeom> lv;
    long mg_rows_total = 0, mg_cof_total = 0;
    int bbox[6]{};
    // stage bookkeeping
    int stage = 0;                      // last completed stage
    bool have_output = false;
    bool densa_valid = false;           // DensityA / GravityCenter / PressureA hold this step's values
    mph_solve_stats stats{};
    int iter_cap = 0;
    double tol_outer = 1.0e-6;          // ||b - A x|| / ||b|| stop (the reference's rr/rr0 < 1e-12)
    double visc_ratio = 0.0;            // bound of |viscous part| / |inertia| of A (host estimate)
    double tol_inner = 1.0e-3;          // mixed form: inner relative reduction
    int max_outer = 50;                 // mixed form: refinement steps
    bool cell_assembly = true;          // cell-block assembly kernel (else per-row kernel only)
    bool factored = true;               // mixed form: FP64 operator in factored form where it applies
    bool inner_blocks = false;          // factored form: inner FP32 SpMV on assembled blocks (else sliced pair terms)
    bool inner_local = true;            // pair-term operator: stage neighbours' s in shared memory where a block fits
    bool pair_recompute = false;        // pair-term operator: evaluate g from the FP32 positions per slot (else slot records)
    bool pair_pack = true;              // pair-term operator: 6-byte slot records (packed g, 2-byte index; else FP16, 8 bytes)
    bool pair_fuse = false;             // point-Jacobi pair path: pair terms written sliced by one kernel (no pair-term list)
    bool batch_solve = false;           // in mph_batch_step: the CR iterations launched over the batch's cases together
                                        // (measured slower on the 512-case ensemble: the step-wide barriers cost more
                                        // than the launches saved)
    bool split_apply = false;           // pair-term operator: transposed apply beside the viscous kernel (fork / join;
                                        // measured slower: the viscous kernel fills every SM)
    cudaStream_t fork_stream = nullptr; // its side stream and events
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int pair_block = 512;               // threads a block of the pair-term operator (and its row blocks)
    int ct_block = 256;                 // threads a block of the transposed P-list apply (and its particle blocks)
    int chunk = 8;                      // mixed form: CR iterations per captured graph chunk
    int cell_sort = 0;                  // 0: the reference's bitonic network (bit-exact order); 1: counting sort
    int mg_pre = 1, mg_post = 1;        // mixed form: sweeps of the V-cycle's levels below level 0 (the reference's: 2 and 3)
    int mg_depth = -1;                  // mixed form: -1 point Jacobi (no multigrid), 0 every level, k >= 1 the first k
    int mg_coarsest = 4;                // mixed form: sweeps of a coarsest level run grid-wide (the reference's 4)
    bool dense_coarse = true;           // mixed form: solve the first one-block coarse level of <= 224 rows exactly
    int dense_level = -1;               // this step's exactly solved level (-1: none)
    int extrapolate = 0;                // mixed form: CR start from the last 1 + extrapolate start velocities
                                        // (1: 2 v_n - v_{n-1}; 2: 3 v_n - 3 v_{n-1} + v_{n-2}; 0: the reference's v_n)
    int prev_valid = 0;                 // start velocities of previous steps held in vprev (current particle order)
    bool keep_history = false;          // mph_case_set_state keeps vprev (the state continues this case's steps)
    int mixed_extra_sweeps = 0;         // mixed form: extra level-0 smoothing sweeps before and after
    bool step_factored = false;         // this step's system uses the factored form
    bool step_pairs = false;            // this step's FP32 inner operator runs on the sliced pair terms
    cudaEvent_t gev[128] = {};          // event pairs of a profiled CR graph chunk (operators, then V-cycles)
    bool level0_done = false;           // this step's level-0 multigrid stencils were written by the assembly
    int loc_smem = 0;                   // shared memory of k_visc_pen32's staged s (0: gathers by column)
    int loc_cap = 0;                    // staged neighbours a block of the pair-term operator has room for
    int loc_ct_smem = 0;                // shared memory of k_ct_apply32's staged s (0: gathers by column)
    int loc_blocks[2] = {};             // row blocks staged / gathering by column
    int loc_ct_blocks = 0;              // particle blocks of k_ct_apply32 staging s
    long long loc_cols = 0;             // distinct neighbour columns over the staged blocks
    bool visc_nonneg = true;            // every viscous pair coefficient f is >= 0
    bool ct_ready = false;              // transposed P-lists built for this step
    bool use_graphs = true;             // replay CR iteration chunks as CUDA graphs
    cudaGraphExec_t cr_exec = nullptr;  // FP64 CR chunk
    cudaGraphExec_t mx_exec = nullptr;  // mixed form: FP32 inner CR chunk
    cudaStream_t cap_stream = nullptr;  // side stream the chunks are captured on
    cudaStream_t cap_stream2 = nullptr, cap_stream3 = nullptr;   // the device-driven solve's loop bodies are captured on
    bool device_loop = false;           // mixed form with graphs: the whole solve as one graph with device-side loops
    cudaGraphExec_t sx_exec[2] = {};    // the device-driven mixed solve (one graph per parity of the swapped arrays)
    unsigned long long sx_sig[2] = {};
    int sx_next = 0;
    long long sx_launches[2][3] = {};   // their kernels: top level, per refinement phase, per CR iteration
    unsigned long long cr_sig = 0, mx_sig = 0;   // signatures the two graphs were captured from
    long long cr_launches = 0, mx_launches = 0;  // kernel launches in one replay of each
    cudaStream_t own_stream = nullptr;  // private stream for batched steps of a legacy-stream case
    mph::DeviceState d;
    std::vector<void*> allocations;
    mph::Profile prof;
};

namespace mph {

// error helper: set the thread-local message and return the status
int fail(int status, const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

#define MPH_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return ::mph::cuda_check(e_, #call); \
    } while (0)

#define MPH_TRY(call)                  \
    do {                               \
        int s_ = (call);               \
        if (s_ != MPH_OK) return s_;   \
    } while (0)

// host-side case API (mph_case.cu)
int case_create(const mph_params* prm, const mph_particles* parts, int dim, int precision, void* stream, mph_case** out);
int case_destroy(mph_case* c);
int case_step(mph_case* c, int nsteps);
const char* last_error();
int case_export(mph_case* c, const char* name, void* dst, long* count, int* kind);
int case_scalars(mph_case* c, double* out, int n);
const char* scalar_names();
int case_get_fields(mph_case* c, mph_fields* out);
int case_set_state(mph_case* c, const mph_particles* parts, const double* wall_center);
int case_profile(mph_case* c, int enable);
// batching and serving (mph_batch.cpp)
int batch_step(mph_case** cases, int ncases, int nsteps, int workers);
int case_footprint(const mph_params* prm, const mph_particles* parts, int dim, int precision, long long* bytes);
int server_create(long long budget, int workers, int device, mph_server** out);
int server_submit(mph_server* s, const mph_params* prm, const mph_particles* parts, int dim, int precision, int steps,
                  const mph_fields* out, float* step_ms, long long* ticket);
int server_poll(mph_server* s, mph_server_result* out, int max, int wait_ms, int* count);
int server_set_solver(mph_server* s, double outer, double inner, int max_outer);
int server_set_option(mph_server* s, const char* name, double value);
int server_stats(mph_server* s, mph_server_stats* out);
int server_destroy(mph_server* s);
int case_profile_read(mph_case* c, double* out, int n);

// profiling helpers (mph_case.cu): bracket a launch sequence of kernel class k
int prof_begin(mph_case* c, int k, cudaEvent_t* e0);
void prof_end(mph_case* c, int k, cudaEvent_t e0);
int prof_collect(mph_case* c);

// host-side stages (mph_case.cu)
int case_alloc_particles(mph_case* c);
int stage_step_begin(mph_case* c);
int stage_cellsort(mph_case* c);
int stage_neighbors(mph_case* c);
int stage_explicit(mph_case* c);
int stage_assemble(mph_case* c);
int stage_mg_build(mph_case* c);
int stage_solve(mph_case* c);
int stage_step_end(mph_case* c);
int stage_output_fields(mph_case* c);

// kernel launchers (k_*.cu)
void launch_step_begin(mph_case* c);
void launch_cell_keys(mph_case* c);
void launch_bitonic_sort(mph_case* c);
int launch_counting_sort(mph_case* c);
void launch_cell_ranges_and_permute(mph_case* c);
void launch_fluid_bbox(mph_case* c);
void launch_neighbor_count(mph_case* c);
int launch_scan_i32_to_i64(mph_case* c, const int* in, long long* out, int n);
int launch_slice_ptr(mph_case* c, int rows, const int* counts, int* width, long long* ptr, long long* total);
void launch_neighbor_fill(mph_case* c);
void launch_explicit(mph_case* c);
void launch_explicit_density_only(mph_case* c);
void launch_density_full(mph_case* c);
void ensure_density_a(mph_case* c);
void launch_output_fields(mph_case* c);
int launch_assemble(mph_case* c);
int launch_assemble_cells(mph_case* c, int kmax_rows, bool mix, bool* done);
int build_ct(mph_case* c);
bool factored_applies(const mph_case* c);
// One case of a CR iteration launched over several cases (the batched
// solve): the case's arrays and its share of each launch.  A block finds its
// case from the launches' block starts and runs the single-case kernel body
// with its block index inside the case, so each case's arithmetic, and its
// reductions' order, are the single-case launch's.
struct BatchCase {
    int N, Nf, n, cap;                 // particles, fluid rows, vector length, iteration cap
    int ct_loc, vp_loc;                // the case's blocks stage s (shared memory of the transposed / viscous kernel)
    int ct_nb, vp_nb, el_nb;           // the case's block counts: transposed apply, viscous kernel, vector kernels
    const long long* ctsptr; const int* ct_cnt; const float4* ctsval; float* tct32; const int* ctuniq; const int* ctucount;
    const int* nfc; const long long* sptr; const int* acol; const unsigned short* grec16; const unsigned* grec32;
    const unsigned short* lcol16; const float* pscale; const float* sdiag32; const int* ncp; const long long* psptr;
    const float4* psval; const int* uniq; const int* ucount;
    float *s32, *y32, *p32, *q32, *u32, *z32, *r32;
    const float* invD;
    double* scal; int* flags; double* partials; unsigned* counter;
};
// one FP32 CR iteration over the cases of a batch (all in the point-Jacobi
// mixed form on the pair path, one dimension, one record format and one
// pair / transposed block width): four launches on `st`; b0 holds the three
// launches' block starts per case (3 x (ncases + 1) ints, device)
void launch_batch_iteration(const BatchCase* cases_dev, const int* b0_dev, int ncases, int dim, bool pack, int pair_block,
                            int ct_block, int vp_smem, int ct_smem, const int* nblocks, cudaStream_t st);
void launch_batch_operator(const BatchCase* cs, const int* ct_b0, const int* vp_b0, int nc, int dim, bool pack, int pair_block,
                           int ct_block, int vp_smem, int ct_smem, int ct_blocks, int vp_blocks, cudaStream_t st);
// par(n, f): run f(0) .. f(n-1) (the batch's host worker pool); the per-case
// host parts of the batched solve (phase tests, updates) run through it
int batched_mixed_solve(std::vector<mph_case*>& cases, const std::function<void(int, const std::function<int(int)>&)>& par);
bool batch_solve_eligible(const mph_case* c);

// the mixed form preconditioned by point Jacobi (option mg_depth -1): no
// multigrid levels are built or used
inline bool mixed_jacobi(const mph_case* c) { return c->precision == MPH_PRECISION_MIXED && c->mg_depth < 0; }
bool pair_path_expected(const mph_params* prm, const mph_particles* parts, int dim);
int launch_pair_terms(mph_case* c);
void launch_resid_factored(mph_case* c, const double* x, double* r, double* out);
void launch_apply32(mph_case* c, const float* x, float* y, int cap);
int launch_pairs_to_slices(mph_case* c);
int launch_ct_slices(mph_case* c);
int launch_part_pairs(mph_case* c, const struct Level0Map& M, bool* done);
void launch_mg_level0(mph_case* c, const int* only_cells);
int ensure_mg_cof(mph_case* c);
void launch_mg_coarse(mph_case* c, int L);
void launch_mg_invd(mph_case* c);
int run_cr_solve(mph_case* c);
int noalloc_prepare(int dev);   // k_resid_noalloc.cu: reserve the allocation-free check's array on this device
int run_mixed_solve(mph_case* c);
int mixed_dense_coarse(mph_case* c);   // k_multigrid.cu: this step's dense coarse level of the mixed V-cycle
bool mixed_available();

}  // namespace mph
