// mph_batch.cpp - concurrent stepping of independent cases and the serving
// loop that admits cases by device-memory footprint.
//
// The reference runs one case per process (main.cpp:313-474); batching and
// serving have no counterpart there.  The unit of work is one time step of
// one case.  A step has host decisions in it (buffer sizes from the
// neighbour totals, the CR stopping test), so every case is driven by a host
// worker thread, each case on its own non-blocking stream: while one case's
// worker waits on its stream, the kernels of the other cases run beside it.
// No state is shared between cases, so a case computes bit for bit the same
// result alone or in a batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "mph_internal.h"

namespace mph {

// ---- device-memory footprint bound ------------------------------------------------
// Upper bound of a case's device memory: per-particle vectors, the neighbour
// lists, A (FP64 blocks, plus the FP32 copy in the mixed form), C, the
// transposed P-lists, the level-0 stencils and the solver vectors.  The
// neighbour counts are the lattice counts of the radii, with 25% room for
// compression and 10% for sliced-ELL padding.
static long long lattice_count(int dim, double ratio)
{
    const int r = (int)std::ceil(ratio);
    long long n = 0;
    for (int x = -r; x <= r; ++x)
        for (int y = -r; y <= r; ++y)
            for (int z = (dim == 2 ? 0 : -r); z <= (dim == 2 ? 0 : r); ++z)
                if ((double)(x * x + y * y + z * z) <= ratio * ratio) ++n;
    return n;
}

int case_footprint(const mph_params* prm, const mph_particles* parts, int dim, int precision, long long* bytes)
{
    if (!prm || !parts || !bytes) return fail(MPH_ERR_ARG, "null argument");
    if (dim != 2 && dim != 3) return fail(MPH_ERR_ARG, "dim must be 2 or 3");
    if (parts->count < 0 || (parts->count > 0 && !parts->type)) return fail(MPH_ERR_ARG, "bad particle set");
    const long long N = parts->count;
    long long Nf = 0;
    for (long long i = 0; i < N; ++i) Nf += parts->type[i] < 2;
    const double rmax = std::max(prm->radius_ratio_a, std::max(prm->radius_ratio_p, prm->radius_ratio_v));
    const double nb = 1.25 * (double)lattice_count(dim, rmax);
    const double np = 1.25 * (double)lattice_count(dim, prm->radius_ratio_p);
    const double D = dim, DD = dim * dim, S = dim == 2 ? 9.0 : 27.0;
    double b = 0.0;
    b += (double)N * 400.0;                                   // particle vectors, keys, sort scratch
    b += (double)N * (nb + np) * 4.0 + (double)N * 32.0;      // neighbour lists and row pointers
    const double blocks = 1.10 * (double)Nf * nb;             // block slots of A, with slice padding
    b += blocks * 4.0;                                        // block columns
    if (precision == MPH_PRECISION_MIXED && pair_path_expected(prm, parts, dim)) {
        // default options, factored operator, inner operator on pair terms:
        // no blocks; pair terms, their sliced FP32 / FP16 copies, sliced
        // P-lists and transposed P-lists, level-0 cell bins
        b += (double)Nf * nb * 16.0 + blocks * (D * 4.0 + 8.0);
        b += (double)Nf * np * (D * 4.0 + 4.0) * 2.2 + (double)N * (8.0 * 16.0 + 8.0) + (double)Nf * 32.0;
        b += (double)Nf * 17.0 * 4.0;                         // block-local neighbour columns
        b += (double)N * 33.0 * 4.0 + (double)Nf * np * 2.0;   // the same for the transposed P-lists (blocks of 256)
    } else {
        b += blocks * DD * 8.0;                               // FP64 blocks
        if (precision == MPH_PRECISION_MIXED) {
            b += 2.0 * blocks * DD * 4.0;                     // FP32 blocks, sliced and row-contiguous
            b += (double)Nf * nb * 16.0;                      // FP32 pair terms
        }
    }
    b += (double)Nf * np * (D * 8.0) * 2.0;                   // C and its transpose values
    b += (double)Nf * np * 4.0 * 2.0 + (double)N * 24.0;      // transpose indices and pointers
    b += (double)Nf * S * DD * 8.0;                           // level-0 stencils
    b += (double)Nf * D * 8.0 * 10.0;                         // solver vectors, b, D^-1
    if (precision == MPH_PRECISION_MIXED) b += (double)Nf * D * 4.0 * 8.0;
    b += (double)Nf * D * 8.0 * 6.0;                          // multigrid levels (<= level 0 size each)
    *bytes = (long long)(b * 1.05) + (64ll << 20);
    return MPH_OK;
}

// ---- batched stepping -------------------------------------------------------------
static int default_workers(int n)
{
    const unsigned hw = std::thread::hardware_concurrency();
    return std::max(1, std::min(n, (int)std::min<unsigned>(hw ? 2 * hw : 16, 64)));
}

int batch_step(mph_case** cases, int ncases, int nsteps, int workers)
{
    if (!cases || ncases < 0 || nsteps < 0) return fail(MPH_ERR_ARG, "bad case list");
    std::set<mph_case*> seen;
    for (int k = 0; k < ncases; ++k) {
        if (!cases[k]) return fail(MPH_ERR_ARG, "null case handle in batch");
        if (!seen.insert(cases[k]).second) return fail(MPH_ERR_ARG, "a case appears twice in the batch");
    }
    if (ncases == 0 || nsteps == 0) return MPH_OK;
    // cases on the legacy stream get a private non-blocking stream for the call
    MPH_CUDA(cudaStreamSynchronize(nullptr));
    std::vector<char> borrowed(ncases, 0);
    for (int k = 0; k < ncases; ++k) {
        mph_case* c = cases[k];
        if (c->stream) continue;
        if (!c->own_stream) MPH_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
        c->stream = c->own_stream;
        borrowed[k] = 1;
    }
    const int nw = workers > 0 ? std::min(workers, ncases) : default_workers(ncases);
    std::vector<int> status(ncases, MPH_OK);
    std::vector<std::string> msg(ncases);
    // run f(k) for every case k on the worker pool (a case's failure is kept,
    // and the case skipped afterwards)
    auto parallel = [&](auto&& f) {
        std::atomic<int> next{0};
        auto work = [&]() {
            int k;
            while ((k = next.fetch_add(1)) < ncases) {
                if (status[k] != MPH_OK) continue;
                mph_case* c = cases[k];
                cudaSetDevice(c->device);
                int st;
                try {
                    st = f(k);
                } catch (...) {
                    st = fail(MPH_ERR_STATE, "exception in a batched step");
                }
                status[k] = st;
                if (st != MPH_OK) msg[k] = last_error();
            }
        };
        std::vector<std::thread> pool;
        for (int w = 1; w < nw; ++w) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
    };
    bool batched = false;   // some case may solve in the batched solve (option batch_solve, mixed form)
    for (int k = 0; k < ncases; ++k)
        if (cases[k]->batch_solve && cases[k]->precision == MPH_PRECISION_MIXED && !cases[k]->prof.on) batched = true;
    if (!batched) {
        parallel([&](int k) -> int { return case_step(cases[k], nsteps); });
    } else {
        // step by step: the stages before the solve on the worker pool; the
        // eligible cases' solve batched on this thread (the CR iterations of
        // every case in one launch per kernel), the others' on the pool; the
        // step's end for all
        std::vector<int> last(ncases, MPH_OK);
        for (int s = 0; s < nsteps; ++s) {
            parallel([&](int k) -> int {
                mph_case* c = cases[k];
                MPH_TRY(stage_step_begin(c));
                MPH_TRY(stage_cellsort(c));
                MPH_TRY(stage_neighbors(c));
                MPH_TRY(stage_explicit(c));
                MPH_TRY(stage_assemble(c));
                return stage_mg_build(c);
            });
            std::vector<mph_case*> group;
            std::vector<int> group_k;
            for (int k = 0; k < ncases; ++k)
                if (status[k] == MPH_OK && batch_solve_eligible(cases[k])) {
                    group.push_back(cases[k]);
                    group_k.push_back(k);
                }
            if (!group.empty()) {
                cudaSetDevice(group[0]->device);
                const int dev = group[0]->device;
                // the per-case host parts on the worker pool
                auto par = [&](int n, const std::function<int(int)>& f) {
                    std::atomic<int> next{0};
                    auto work = [&]() {
                        cudaSetDevice(dev);
                        int k;
                        while ((k = next.fetch_add(1)) < n) f(k);
                    };
                    std::vector<std::thread> pool;
                    for (int w = 1; w < std::min(nw, n); ++w) pool.emplace_back(work);
                    work();
                    for (auto& t : pool) t.join();
                };
                const int st = batched_mixed_solve(group, par);
                if (st != MPH_OK)
                    for (int k : group_k) {
                        status[k] = st;
                        msg[k] = last_error();
                    }
            }
            parallel([&](int k) -> int {
                mph_case* c = cases[k];
                if (c->stage == 6) MPH_TRY(stage_solve(c));   // not in the batched solve
                MPH_TRY(stage_step_end(c));
                if (c->stats.status != MPH_OK) last[k] = c->stats.status;
                return MPH_OK;
            });
        }
        for (int k = 0; k < ncases; ++k)
            if (status[k] == MPH_OK && last[k] != MPH_OK) {
                status[k] = last[k];
                msg[k] = "the solve did not converge";
            }
    }
    for (int k = 0; k < ncases; ++k)
        if (borrowed[k]) cases[k]->stream = nullptr;
    int last = MPH_OK;
    for (int k = 0; k < ncases; ++k) {
        if (status[k] == MPH_OK) continue;
        if (status[k] != MPH_ERR_NOT_CONVERGED) return fail(status[k], "case " + std::to_string(k) + ": " + msg[k]);
        last = fail(status[k], "case " + std::to_string(k) + ": " + msg[k]);
    }
    return last;
}

}  // namespace mph

// ---- serving loop -----------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long long ticket = 0;
    mph_params prm{};
    int dim = 3, precision = MPH_PRECISION_FP64, steps = 0;
    std::vector<int> type;
    std::vector<double> pos, vel;
    mph_particles parts{};
    mph_fields out{};          // caller's host buffers, filled at completion
    float* step_ms = nullptr;  // caller's buffer of `steps` floats, or null
    long long footprint = 0;
    mph_case* c = nullptr;
    cudaStream_t stream = nullptr;
    int done_steps = 0;
    int status = MPH_OK;
    std::string error;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::vector<float> times;
    bool solver_set = false;   // the server's settings at submission
    double tol_outer = 1.0e-6, tol_inner = 1.0e-3;
    int max_outer = 50;
    std::vector<std::pair<std::string, double>> options;
};

}  // namespace

struct mph_server {
    int device = 0;
    long long budget = 0, used = 0;
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    bool stopping = false;
    std::deque<Request*> pending;   // submitted, waiting for memory (FIFO)
    std::deque<Request*> ready;     // admitted, waiting for a worker (round robin)
    std::deque<Request*> finished;  // completed, not yet polled
    int running = 0;                // requests a worker holds right now
    long long next_ticket = 1;
    long long steps_done = 0;
    // solver settings and options of the cases created from now on
    bool solver_set = false;
    double tol_outer = 1.0e-6, tol_inner = 1.0e-3;
    int max_outer = 50;
    std::vector<std::pair<std::string, double>> options;
    double particle_steps = 0.0;
    Clock::time_point t0 = Clock::now();
    std::vector<std::thread> workers;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    // admit waiting requests in arrival order while the budget allows (mu held)
    void admit()
    {
        while (!pending.empty() && used + pending.front()->footprint <= budget) {
            Request* r = pending.front();
            pending.pop_front();
            used += r->footprint;
            r->t_admit = now();
            ready.push_back(r);
            work_cv.notify_one();
        }
    }

    void finish(Request* r)
    {
        if (r->c) mph::case_destroy(r->c);
        r->c = nullptr;
        if (r->stream) cudaStreamDestroy(r->stream);
        r->stream = nullptr;
        std::lock_guard<std::mutex> lk(mu);
        used -= r->footprint;
        r->t_done = now();
        --running;
        finished.push_back(r);
        admit();
        done_cv.notify_all();
    }

    void worker()
    {
        cudaSetDevice(device);
        for (;;) {
            Request* r;
            {
                std::unique_lock<std::mutex> lk(mu);
                work_cv.wait(lk, [&] { return stopping || !ready.empty(); });
                if (stopping) return;
                r = ready.front();
                ready.pop_front();
                ++running;
            }
            int st = MPH_OK;
            try {
                if (!r->c) {
                    cudaError_t e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
                    st = e == cudaSuccess ? mph::case_create(&r->prm, &r->parts, r->dim, r->precision, r->stream, &r->c)
                                          : mph::cuda_check(e, "cudaStreamCreateWithFlags");
                    // the server's solver settings and options, as they were at submission
                    if (st == MPH_OK && r->solver_set)
                        st = mph_case_set_solver(r->c, r->tol_outer, r->tol_inner, r->max_outer);
                    for (size_t k = 0; st == MPH_OK && k < r->options.size(); ++k)
                        st = mph_case_set_option(r->c, r->options[k].first.c_str(), r->options[k].second);
                }
                if (st == MPH_OK) {
                    const auto a = Clock::now();
                    st = mph::case_step(r->c, 1);
                    const float ms = std::chrono::duration<float, std::milli>(Clock::now() - a).count();
                    if (st == MPH_OK || st == MPH_ERR_NOT_CONVERGED) {
                        if (r->step_ms) r->step_ms[r->done_steps] = ms;
                        ++r->done_steps;
                        if (st == MPH_ERR_NOT_CONVERGED) r->status = st;
                        st = MPH_OK;
                        std::lock_guard<std::mutex> lk(mu);
                        ++steps_done;
                        particle_steps += (double)r->parts.count;
                    }
                }
                if (st == MPH_OK && r->done_steps == r->steps) st = mph::case_get_fields(r->c, &r->out);
            } catch (...) {
                st = mph::fail(MPH_ERR_STATE, "exception in a served step");
            }
            if (st != MPH_OK) {
                r->status = st;
                r->error = mph::last_error();
                finish(r);
            } else if (r->done_steps == r->steps) {
                finish(r);
            } else {
                std::lock_guard<std::mutex> lk(mu);
                --running;
                ready.push_back(r);
                work_cv.notify_one();
            }
        }
    }
};

namespace mph {

int server_create(long long budget, int workers, int device, mph_server** out)
{
    if (!out || budget <= 0) return fail(MPH_ERR_ARG, "server needs an output handle and a positive budget");
    *out = nullptr;
    auto* s = new mph_server();
    if (device >= 0) s->device = device;
    else cudaGetDevice(&s->device);
    s->budget = budget;
    const int nw = workers > 0 ? workers : 16;
    for (int w = 0; w < nw; ++w) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return MPH_OK;
}

int server_submit(mph_server* s, const mph_params* prm, const mph_particles* parts, int dim, int precision, int steps,
                  const mph_fields* out, float* step_ms, long long* ticket)
{
    if (!s || !prm || !parts || !ticket) return fail(MPH_ERR_ARG, "null argument");
    if (steps < 1) return fail(MPH_ERR_ARG, "a request needs at least one step");
    if (parts->count < 1 || !parts->type || !parts->pos || !parts->vel) return fail(MPH_ERR_ARG, "bad particle set");
    long long fp = 0;
    MPH_TRY(case_footprint(prm, parts, dim, precision, &fp));
    auto* r = new Request();
    r->prm = *prm;
    r->dim = dim;
    r->precision = precision;
    r->steps = steps;
    const size_t n = (size_t)parts->count;
    r->type.assign(parts->type, parts->type + n);
    r->pos.assign(parts->pos, parts->pos + 3 * n);
    r->vel.assign(parts->vel, parts->vel + 3 * n);
    r->parts = *parts;
    r->parts.type = r->type.data();
    r->parts.pos = r->pos.data();
    r->parts.vel = r->vel.data();
    if (out) r->out = *out;
    r->step_ms = step_ms;
    std::lock_guard<std::mutex> lk(s->mu);
    r->solver_set = s->solver_set;
    r->tol_outer = s->tol_outer;
    r->tol_inner = s->tol_inner;
    r->max_outer = s->max_outer;
    if (precision == MPH_PRECISION_MIXED) {
        r->options = s->options;
        for (auto& o : r->options)   // the start-velocity history of option extrapolate: 2 x 2 vectors of N x VS doubles
            if (o.first == "extrapolate" && o.second > 0.0) fp += 4LL * parts->count * (dim == 2 ? 2 : 4) * 8;
    } else {
        for (auto& o : s->options)   // options of the mixed form do not apply to FP64 cases
            if (o.first != "extrapolate" && o.first != "dense_coarse" && o.first != "factored" && o.first != "inner_blocks" &&
                o.first != "inner_local" && o.first != "mixed_extra_sweeps")
                r->options.push_back(o);
    }
    if (fp > s->budget) {
        delete r;
        return fail(MPH_ERR_CAPACITY, "case footprint " + std::to_string(fp) + " B exceeds the server budget");
    }
    r->footprint = fp;
    r->ticket = s->next_ticket++;
    r->t_submit = s->now();
    s->pending.push_back(r);
    s->admit();
    *ticket = r->ticket;
    return MPH_OK;
}

int server_set_solver(mph_server* s, double outer, double inner, int max_outer)
{
    if (!s) return fail(MPH_ERR_ARG, "null server");
    if (!(outer > 0.0) || !(inner > 0.0) || inner >= 1.0 || max_outer < 1)
        return fail(MPH_ERR_ARG, "solver tolerances must be positive (inner < 1) and max_outer >= 1");
    std::lock_guard<std::mutex> lk(s->mu);
    s->solver_set = true;
    s->tol_outer = outer;
    s->tol_inner = inner;
    s->max_outer = max_outer;
    return MPH_OK;
}

int server_set_option(mph_server* s, const char* name, double value)
{
    if (!s || !name) return fail(MPH_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& o : s->options)
        if (o.first == name) {
            o.second = value;
            return MPH_OK;
        }
    s->options.push_back({name, value});
    return MPH_OK;
}

int server_poll(mph_server* s, mph_server_result* out, int max, int wait_ms, int* count)
{
    if (!s || !count || (max > 0 && !out)) return fail(MPH_ERR_ARG, "null argument");
    *count = 0;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->finished.empty() && wait_ms > 0)
        s->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->finished.empty(); });
    int k = 0;
    while (k < max && !s->finished.empty()) {
        Request* r = s->finished.front();
        s->finished.pop_front();
        mph_server_result& o = out[k++];
        std::memset(&o, 0, sizeof(o));
        o.ticket = r->ticket;
        o.status = r->status;
        o.steps = r->done_steps;
        o.particles = r->parts.count;
        o.submit_s = r->t_submit;
        o.admit_s = r->t_admit;
        o.done_s = r->t_done;
        o.footprint_bytes = r->footprint;
        std::strncpy(o.error, r->error.c_str(), sizeof(o.error) - 1);
        delete r;
    }
    *count = k;
    return MPH_OK;
}

int server_stats(mph_server* s, mph_server_stats* out)
{
    if (!s || !out) return fail(MPH_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    out->budget_bytes = s->budget;
    out->used_bytes = s->used;
    out->pending = (int)s->pending.size();
    out->active = (int)s->ready.size() + s->running;
    out->finished = (int)s->finished.size();
    out->steps = s->steps_done;
    out->particle_steps = s->particle_steps;
    out->elapsed_s = s->now();
    return MPH_OK;
}

int server_destroy(mph_server* s)
{
    if (!s) return MPH_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->work_cv.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto* q : {&s->pending, &s->ready, &s->finished})
        for (Request* r : *q) {
            if (r->c) case_destroy(r->c);
            if (r->stream) cudaStreamDestroy(r->stream);
            delete r;
        }
    delete s;
    return MPH_OK;
}

}  // namespace mph
