// lbm2d_serve.cpp -- a serving loop for many concurrent solves on one GPU.
//
// Requests (grid, geometry, Reynolds number, step budget, storage) arrive at
// any time through lbm2d_server_submit.
//   * Set-up threads admit queued requests in arrival order while the
//     device-memory footprint of the live solves stays within the budget and
//     a slot is free, and build each case the way the reference's drivers do
//     (mask, bounce-back geometry and its records, tau from Re, LES when
//     tau < 0.55, thermal set-up, initial state on the device).  Several
//     requests are set up at once, on the host cores, while the GPU steps
//     the others.
//   * The stepping thread adds the solves that are ready to the batch and
//     advances every active solve together: one lbm2d_batch_step of
//     steps_per_tick steps per tick (one packed launch per step per storage
//     group, CUDA-graph replay); each solve carries its remaining budget into
//     the batch and sits out the launches after it is spent, so every solve
//     stops exactly at its budget without shortening the tick;
//   * it then retires finished solves (non-finite check, drag/lift read back,
//     memory freed) and records arrival, admission and completion times.
//
// Resident mode (LBM2D_SERVE_RESIDENT) replaces the ticks with the device
// loop of lbm2d_resident.cu: the set-up threads also prepare each solve's
// table entry (its step parameters, work units and force reduction); the
// stepping thread copies it into a free slot of the device table and raises
// the slot's join word in mapped memory, and the loop admits the solve at its
// next step boundary, steps it with the others and retires it at its budget
// by writing the steps it took to the slot's done word, which the stepping
// thread polls.  The loop relaunches itself only when it ends (no active
// solve, a new kind of solve, or a bounded number of iterations).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "lbm2d_runtime.h"

using namespace lbm2d;

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Caller-supplied state of a request (lbm2d_server_submit_state): an initial
// population field copied at submission, and the caller's buffers that
// receive the final populations when the request retires.
struct StateIO {
    std::shared_ptr<std::vector<double>> f_init;
    double* f_out = nullptr;
    double* g_out = nullptr;
};

struct Pending {
    long long id;
    lbm2d_request req;
    double t_submit;
    StateIO io;
};

struct Active {
    long long id;
    lbm2d_request req;
    lbm2d_solver* h = nullptr;
    long long left = 0;
    double t_submit = 0, t_admit = 0;
    size_t footprint = 0;
    double tau = 0.0, u_bc = 0.0;
    StateIO io;
    std::shared_ptr<ResEntry> entry;  // resident mode: the solve's table entry
    bool in_batch = false;            // tick mode: chosen for the current tick
};

// Tick mode, shortest remaining first: each tick steps the active solves
// with the fewest remaining steps, as many as it takes to reach this many
// lattice nodes; the others wait out of the batch.  Per-solve arithmetic
// does not depend on the company a step keeps, so the results are those of
// any other order.  On the 200-request serving mix (FP16): 8 Mi nodes gave
// p50 / p99 1.51 / 10.1 s at 61.9 GLUPS, 16 Mi 1.72 / 9.38 s at 66.2, 32 Mi
// 2.58 / 9.05 s at 68.6, every solve each tick 3.02 / 8.96 s at 69.2.
constexpr long long kSaturateNodes = 16LL << 20;

size_t footprint_bytes(const lbm2d_request& r) {
    const size_t n = (size_t)r.nx * r.ny;
    const size_t es = r.storage == LBM2D_STORE_FP64 ? 8 : (r.storage == LBM2D_STORE_FP32 ? 4 : 2);
    const int sets = r.geometry == LBM2D_GEOM_HEATED_CAVITY ? 2 : 1;
    // populations (2 buffers) + FP64 staging + flags + boundary records (generous)
    return sets * (2 * 9 * n * es + 72 * n) + 4 * n + 256 * (size_t)(2 * (r.nx + r.ny)) + (1 << 20);
}

}  // namespace

struct lbm2d_server {
    int device = 0;
    bool resident = false;
    size_t budget = 0;
    int max_active = 0;
    int steps_per_tick = 0;
    bool fifo = false;  // tick mode: every active solve in every tick
    lbm2d_batch* batch = nullptr;
    std::thread worker;
    std::vector<std::thread> setup_threads;
    // guarded by mu: queue, ready, results, used, live, counters, stop
    std::mutex mu;
    std::condition_variable cv;        // results, ready solves, stop
    std::condition_variable cv_setup;  // queued requests, freed memory, stop
    std::deque<Pending> queue;
    std::deque<Active> ready;          // set up, waiting to join the batch
    std::vector<lbm2d_result> results;
    size_t used = 0;
    int live = 0;  // being set up + ready + active
    long long next_id = 0, submitted = 0, finished = 0;
    bool stop = false;
    double setup_s = 0.0;
    // stepping thread only
    std::vector<Active> active;
    double busy_s = 0.0;
    long long lattice_updates = 0;
    long long ticks = 0, member_ticks = 0;
    double gpu_s = 0.0;  // device time of the ticks (CUDA events on the batch stream)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // resident mode (stepping thread): the device loop, its streams, the
    // solve in each table slot and the slot's state (0 free, 1 entry written,
    // join not yet raised, 2 joined), the combos in use
    ResLoop* loop = nullptr;
    cudaStream_t loop_stream = nullptr, copy_stream = nullptr;
    ResEntry* h_entry = nullptr;  // pinned staging of one entry
    std::vector<Active> slot;
    std::vector<int> slot_state;
    unsigned mask_used = 0, mask_running = 0;
    bool running = false;
    // stepping-thread time split: step call (prepare + enqueue), wait for the
    // device, retirement, joining ready solves
    double call_s = 0.0, wait_s = 0.0, retire_s = 0.0, join_s = 0.0;
};

namespace {

// Resident mode: the solve's step parameters at both parities (the batched
// kernels' launch shape, 32x4), its kind, work units, force reduction and
// budget, as lbm2d_batch_step would launch it.
int prepare_entry(Active& a) {
    lbm2d_solver* h = a.h;
    h->bx = 32;
    h->by = 4;
    h->in_batch = true;
    h->resident = true;
    KParams p;
    int rc = rt::prepare_steps(h, a.tau, a.u_bc, p, true);
    if (rc) return rc;
    const bool paired = h->slot_kind == rt::KERNEL_PAIR;
    if (h->thermal && paired) return LBM2D_ERR_INVALID;  // the loop has no paired thermal kernel
    auto e = std::make_shared<ResEntry>();
    std::memset(e.get(), 0, sizeof(ResEntry));
    const int kind = h->thermal ? 2 : (paired ? 0 : 1);
    e->combo = 3 * h->storage + kind;
    const int gy = (h->ny + h->by - 1) / h->by;
    long long units = ((long long)(p.ftiles > 0 ? p.ftiles : (long long)p.gx * gy) + kBatchTiles - 1) / kBatchTiles;
    if (kind == 0 && p.nbpairs > 0) units += (p.nbpairs + p.bchunk - 1) / p.bchunk;
    e->units = (int)units;
    e->p[0] = p;
    e->p[1] = p;
    e->p[1].fin = p.fout;
    e->p[1].fout = const_cast<void*>(p.fin);
    e->p[1].gin = p.gout;
    e->p[1].gout = const_cast<void*>(p.gin);
    e->p[1].seed_in = p.seed_out;
    e->p[1].seed_out = const_cast<uint32_t*>(p.seed_in);
    if (h->nslots > 0) e->job = {h->d_partials, h->nslots, h->hist_cap, h->d_hist, h->d_counter, h->d_last, nullptr};
    e->left = (int)std::min<long long>(std::max(a.left, 0LL), 0x7FFFFFFF);
    // settled solids are skipped from the solve's third step since its last
    // re-collision on (never with the heated cavity's per-step passes)
    e->settle_after = h->hook == 1 ? -1 : (int)std::max<long long>(0, 2 - h->steps_since_collide);
    a.entry = e;
    return LBM2D_OK;
}

// Build one solve the way the reference's drivers do.
int setup_request(lbm2d_server* s, Active& a) {
    const lbm2d_request& r = a.req;
    const int nx = r.nx, ny = r.ny;
    const double u = r.u > 0 ? r.u : 0.1;
    int case_type = LBM2D_CASE_CAVITY;
    double L = nx, tau = 0.0;
    std::vector<uint8_t> mask((size_t)nx * ny, 0);
    double bcx = 0, bcy = 0, br = 0;
    bool thermal = false;
    switch (r.geometry) {
        case LBM2D_GEOM_CAVITY:  // src/cavity.cpp:27-29, :72
            case_type = LBM2D_CASE_CAVITY;
            lbm2d_mask_walls(nx, ny, mask.data());
            L = nx;
            break;
        case LBM2D_GEOM_STEP: {  // src/step.cpp:37-45, :89-104
            case_type = LBM2D_CASE_STEP;
            const int hs = ny / 3, hin = ny - 1 - hs;
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x)
                    if (y == 0 || y == ny - 1 || (x < nx / 4 && y < hs)) mask[(size_t)y * nx + x] = 1;
            L = 2.0 * hin;
            break;
        }
        case LBM2D_GEOM_CYLINDER:  // D = NY/5, src/main.cpp:32-36, :55-58
            case_type = LBM2D_CASE_CYLINDER;
            br = ny / 10;
            bcx = nx / 4;
            bcy = ny / 2 + 1;
            lbm2d_mask_cylinder(nx, ny, mask.data(), (int)bcx, (int)bcy, (int)br);
            L = ny / 5.0;
            break;
        case LBM2D_GEOM_SIDE_BY_SIDE: {  // two cylinders D = H/5 at S/D = param, src/side_by_side_cylinders.cpp:50-62
            case_type = LBM2D_CASE_SIDE_BY_SIDE;
            const int rad = ny / 10, D = 2 * rad;
            const double sd = r.param > 0 ? r.param : 3.0;
            const int spacing = (int)(sd * D), cx = nx / 4;
            const int cy1 = ny / 2 - spacing / 2, cy2 = cy1 + spacing;
            lbm2d_mask_cylinder(nx, ny, mask.data(), cx, cy1, rad);
            lbm2d_mask_cylinder(nx, ny, mask.data(), cx, cy2, rad);
            bcx = cx;
            bcy = cy2;
            br = rad;
            L = D;
            break;
        }
        case LBM2D_GEOM_HEATED_CAVITY:  // src/thermal_cavity.cpp:57-115 (tau 0.8)
            case_type = LBM2D_CASE_CYLINDER;
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x)
                    if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) mask[(size_t)y * nx + x] = 1;
            thermal = true;
            tau = 0.8;
            break;
        default:
            return LBM2D_ERR_INVALID;
    }
    const double re = r.re > 0 ? r.re : 100.0;
    if (!thermal) tau = 0.5 + 3.0 * (u * L / re);
    const int les = tau < 0.55 ? 1 : 0;  // the drivers' auto-LES (e.g. src/main.cpp:174-182)
    lbm2d_config cfg{nx, ny, case_type, LBM2D_MRT, les, 0.12, r.storage, s->device};
    int rc = lbm2d_create(&cfg, &a.h);
    if (rc) return rc;
    if ((rc = lbm2d_set_mask(a.h, mask.data()))) return rc;
    if (br > 0 && (rc = lbm2d_set_bb_cylinder(a.h, bcx, bcy, br))) return rc;
    double u_init = 0.0, u_bc = u;
    if (thermal) {
        const double Pr = 0.71, Th = 1.5, Tc = 0.5, Lc = ny;
        const double nu = (tau - 0.5) / 3.0, alpha = nu / Pr;
        const double ra = r.param > 0 ? r.param : 1e4;
        const double gb = ra * nu * alpha / ((Th - Tc) * Lc * Lc * Lc);
        const double beta = 0.001;
        if ((rc = lbm2d_set_thermal(a.h, 1, 1.0, alpha, 1.0 / (0.5 + 3.0 * alpha), beta, -gb / beta))) return rc;
        if ((rc = lbm2d_set_thermal_hook(a.h, LBM2D_HOOK_HEATED_CAVITY, Th, Tc))) return rc;
        u_bc = 0.0;
    } else if (case_type == LBM2D_CASE_CYLINDER || case_type == LBM2D_CASE_SIDE_BY_SIDE) {
        u_init = u;  // uniform inflow initial state
    }
    if ((rc = lbm2d_init_equilibrium(a.h, 1.0, u_init, 0.0, 1.0))) return rc;
    if (a.io.f_init && (rc = lbm2d_upload_f(a.h, a.io.f_init->data()))) return rc;
    a.io.f_init.reset();  // the copy is on the device now
    lbm2d_info info;  // builds and uploads the geometry here, off the stepping thread
    if ((rc = lbm2d_get_info(a.h, &info))) return rc;
    a.tau = tau;
    a.u_bc = u_bc;
    if (s->resident && (rc = prepare_entry(a))) return rc;
    if ((rc = lbm2d_synchronize(a.h))) return rc;
    return LBM2D_OK;
}

void record(lbm2d_server* s, const Active& a, int status) {
    lbm2d_result res{};
    res.id = a.id;
    res.status = status;
    res.t_submit = a.t_submit;
    res.t_admit = a.t_admit;
    res.t_done = now_s();
    res.steps = 0;  // the steps the solver actually took
    if (a.h) {
        lbm2d_info info{};
        if (lbm2d_get_info(a.h, &info) == LBM2D_OK) res.steps = info.steps_done;
    }
    res.nodes = (long long)a.req.nx * a.req.ny;
    if (a.h && status == LBM2D_OK) lbm2d_force_sums(a.h, &res.fx, &res.fy);
    std::lock_guard<std::mutex> lock(s->mu);
    s->results.push_back(res);
    ++s->finished;
    s->cv.notify_all();
}

// Free a solve that is in no batch and give its memory back to admission.
// A request that asked for its final state gets it first (a solve that was
// stepped, diverged or not), so the buffers are filled when the result shows.
void release(lbm2d_server* s, const Active& a, int status) {
    if (a.h && (status == LBM2D_OK || status == LBM2D_ERR_NAN)) {
        if (a.io.f_out) lbm2d_download_f(a.h, a.io.f_out);
        if (a.io.g_out && a.req.geometry == LBM2D_GEOM_HEATED_CAVITY) lbm2d_download_g(a.h, a.io.g_out);
    }
    record(s, a, status);
    if (a.h) lbm2d_destroy(a.h);
    std::lock_guard<std::mutex> lock(s->mu);
    s->used -= a.footprint;
    --s->live;
    s->cv_setup.notify_all();
}

void retire(lbm2d_server* s, size_t k, int status) {
    Active a = s->active[k];
    if (a.h && a.in_batch) lbm2d_batch_remove(s->batch, a.h);
    s->active.erase(s->active.begin() + k);
    release(s, a, status);
}

// Set-up thread: take queued requests in arrival order while the budget
// allows, build them, hand them to the stepping thread.
void setup_loop(lbm2d_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        Active a;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_setup.wait(lock, [&] {
                if (s->stop) return true;
                if (s->queue.empty() || s->live >= s->max_active) return false;
                const size_t fp = footprint_bytes(s->queue.front().req);
                return s->used + fp <= s->budget || s->live == 0;  // one solve always fits
            });
            if (s->stop) return;
            const Pending p = s->queue.front();
            s->queue.pop_front();
            a.id = p.id;
            a.req = p.req;
            a.left = p.req.steps;
            a.t_submit = p.t_submit;
            a.io = p.io;
            a.t_admit = now_s();
            a.footprint = footprint_bytes(p.req);
            s->used += a.footprint;
            ++s->live;
        }
        const double t0 = now_s();
        const int rc = setup_request(s, a);
        const double dt = now_s() - t0;
        if (rc) {
            release(s, a, rc);
            std::lock_guard<std::mutex> lock(s->mu);
            s->setup_s += dt;
            continue;
        }
        std::lock_guard<std::mutex> lock(s->mu);
        s->setup_s += dt;
        s->ready.push_back(a);
        s->cv.notify_all();
    }
}

// Move the solves that are set up to the active list (stepping thread);
// choose_tick puts them into the batch.
void join_ready(lbm2d_server* s) {
    std::deque<Active> r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        r.swap(s->ready);
    }
    for (auto& a : r) s->active.push_back(a);
}

// The solves the next tick steps (all of them in FIFO mode; else the
// fewest remaining steps first, up to kSaturateNodes nodes), moved into and
// out of the batch, with their budgets.  Returns the number chosen.
size_t choose_tick(lbm2d_server* s) {
    std::vector<size_t> order(s->active.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    if (!s->fifo)
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            const Active &x = s->active[a], &y = s->active[b];
            if (x.left != y.left) return x.left < y.left;
            return (long long)x.req.nx * x.req.ny < (long long)y.req.nx * y.req.ny;
        });
    std::vector<char> want(s->active.size(), 0);
    long long nodes = 0;
    size_t chosen = 0;
    for (size_t i : order) {
        if (!s->fifo && chosen > 0 && nodes >= kSaturateNodes) break;
        want[i] = 1;
        nodes += (long long)s->active[i].req.nx * s->active[i].req.ny;
        ++chosen;
    }
    for (size_t i = s->active.size(); i-- > 0;) {
        Active& a = s->active[i];
        if (!want[i] && a.in_batch) {
            lbm2d_batch_remove(s->batch, a.h);
            a.in_batch = false;
        } else if (want[i]) {
            int rc = LBM2D_OK;
            if (!a.in_batch) {
                rc = lbm2d_batch_add(s->batch, a.h, a.tau, a.u_bc);
                a.in_batch = rc == LBM2D_OK;
            }
            if (!rc) rc = lbm2d_batch_set_budget(s->batch, a.h, a.left);
            if (rc) {
                retire(s, i, rc);
                --chosen;
            }
        }
    }
    return chosen;
}

void worker_loop(lbm2d_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        join_ready(s);
        if (s->active.empty()) {
            std::unique_lock<std::mutex> lock(s->mu);
            if (s->stop) return;
            s->cv.wait(lock, [&] { return s->stop || !s->ready.empty(); });
            if (s->stop) return;
            continue;
        }
        // the solves of this tick; solves joining below wait for the next one
        const double tc = now_s();
        const size_t n_tick = choose_tick(s);
        s->join_s += now_s() - tc;
        if (n_tick == 0) continue;
        // every solve carries its own budget into the batch, so a tick can be
        // long: a solve whose budget runs out mid-tick sits out the rest
        long long k = 0;
        for (auto& a : s->active)
            if (a.in_batch) k = std::max(k, a.left);
        k = std::min<long long>(k, s->steps_per_tick);
        const size_t n_active = s->active.size();
        const double t0 = now_s();
        cudaStream_t bs = static_cast<cudaStream_t>(lbm2d_batch_stream(s->batch));
        if (s->ev0) cudaEventRecord(s->ev0, bs);
        int rc = lbm2d_batch_step(s->batch, (int)k);
        if (s->ev1) cudaEventRecord(s->ev1, bs);
        const double t1 = now_s();
        join_ready(s);  // adding members only edits the host-side member list
        const double t2 = now_s();
        // wait for the tick only: a diverged solve must not fail the others;
        // each solve's own non-finite flag is read when it retires
        if (!rc && cudaStreamSynchronize(bs) != cudaSuccess) rc = LBM2D_ERR_CUDA;
        const double t3 = now_s();
        s->call_s += t1 - t0;
        s->join_s += t2 - t1;
        s->wait_s += t3 - t2;
        float ms = 0.0f;
        if (!rc && s->ev0 && cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) s->gpu_s += 1e-3 * ms;
        ++s->ticks;
        s->member_ticks += (long long)n_tick;
        s->busy_s += now_s() - t0;
        for (size_t i = 0; i < n_active; ++i) {
            Active& a = s->active[i];
            if (!a.in_batch) continue;
            const long long taken = std::min(a.left, k);
            a.left -= taken;
            s->lattice_updates += taken * (long long)a.req.nx * a.req.ny;
        }
        const double t4 = now_s();
        for (size_t i = n_active; i-- > 0;) {
            Active& a = s->active[i];
            if (a.in_batch && (a.left <= 0 || rc)) {
                int st = rc;
                if (!st && a.h) st = lbm2d_synchronize(a.h);  // non-finite density -> LBM2D_ERR_NAN
                retire(s, i, st);
            }
        }
        s->retire_s += now_s() - t4;
    }
}

// ---------------------------------------------------------------- resident
// Retire the solves the loop has finished (their done word holds the steps
// they took + 1).  Returns whether any was.
bool res_retire_done(lbm2d_server* s) {
    volatile ResMailbox* mb = res_mailbox(s->loop);
    bool any = false;
    for (size_t k = 0; k < s->slot.size(); ++k) {
        if (s->slot_state[k] != 2) continue;
        const long long d = mb->done[k];
        if (d == 0) continue;
        mb->done[k] = 0;
        mb->join[k] = 0;
        Active a = s->slot[k];
        s->slot[k] = Active();
        s->slot_state[k] = 0;
        const long long taken = d - 1;
        rt::advance(a.h, taken);
        if (taken > 0) a.h->u_last = a.u_bc;  // the boundary velocity the state was stepped with
        s->lattice_updates += taken * (long long)a.req.nx * a.req.ny;
        ++s->member_ticks;
        const double t0 = now_s();
        // the solve's own non-finite flag: LBM2D_ERR_NAN
        release(s, a, taken < a.left ? LBM2D_ERR_STATE : lbm2d_synchronize(a.h));
        s->retire_s += now_s() - t0;
        any = true;
    }
    return any;
}

// Put the solves that are set up into free table slots.  A slot's join word
// is raised now when the running loop has its kind, else at the next launch
// (the running loop is asked to end so that it is rebuilt with it).
bool res_join_ready(lbm2d_server* s) {
    std::deque<Active> r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        r.swap(s->ready);
    }
    if (r.empty()) return false;
    volatile ResMailbox* mb = res_mailbox(s->loop);
    ResEntry* table = res_table(s->loop);
    const double t0 = now_s();
    for (auto& a : r) {
        size_t k = 0;
        while (k < s->slot.size() && s->slot_state[k] != 0) ++k;
        if (k == s->slot.size()) {  // admission keeps the live solves within the slots
            release(s, a, LBM2D_ERR_STATE);
            continue;
        }
        *s->h_entry = *a.entry;
        a.entry.reset();
        if (cudaMemcpyAsync(table + k, s->h_entry, sizeof(ResEntry), cudaMemcpyHostToDevice, s->copy_stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(s->copy_stream) != cudaSuccess) {
            release(s, a, LBM2D_ERR_CUDA);
            continue;
        }
        const unsigned bit = 1u << s->h_entry->combo;
        s->mask_used |= bit;
        s->slot[k] = a;
        mb->done[k] = 0;
        if (s->running && (s->mask_running & bit)) {
            std::atomic_thread_fence(std::memory_order_seq_cst);
            mb->join[k] = 1;
            std::atomic_thread_fence(std::memory_order_seq_cst);
            mb->join_gen = mb->join_gen + 1;
            s->slot_state[k] = 2;
        } else {
            s->slot_state[k] = 1;
            if (s->running) mb->stop = 1;
        }
    }
    s->join_s += now_s() - t0;
    return true;
}

void resident_loop(lbm2d_server* s) {
    cudaSetDevice(s->device);
    volatile ResMailbox* mb = res_mailbox(s->loop);
    const int max_iters = s->steps_per_tick;
    double t_launch = 0.0;
    for (;;) {
        bool did = res_retire_done(s);
        if (s->running && cudaEventQuery(s->ev1) != cudaErrorNotReady) {
            s->running = false;
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) s->gpu_s += 1e-3 * ms;
            s->busy_s += now_s() - t_launch;
            did = res_retire_done(s) || did;
        }
        bool stop;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            stop = s->stop;
        }
        if (stop) {
            if (s->running) {
                mb->stop = 1;
                cudaStreamSynchronize(s->loop_stream);
                s->running = false;
                res_retire_done(s);
            }
            return;
        }
        did = res_join_ready(s) || did;
        if (!s->running) {
            bool any = false;
            for (int st : s->slot_state) any = any || st != 0;
            if (any) {
                mb->stop = 0;
                for (size_t k = 0; k < s->slot.size(); ++k)
                    if (s->slot_state[k] == 1) {
                        mb->join[k] = 1;
                        s->slot_state[k] = 2;
                    }
                std::atomic_thread_fence(std::memory_order_seq_cst);
                mb->join_gen = mb->join_gen + 1;
                std::atomic_thread_fence(std::memory_order_seq_cst);
                const double t0 = now_s();
                cudaEventRecord(s->ev0, s->loop_stream);
                const int e = res_launch(s->loop, s->mask_used, max_iters, s->loop_stream);
                cudaEventRecord(s->ev1, s->loop_stream);
                s->call_s += now_s() - t0;
                if (e) {
                    // nothing runs: fail the solves waiting in the table
                    for (size_t k = 0; k < s->slot.size(); ++k)
                        if (s->slot_state[k] != 0) {
                            Active a = s->slot[k];
                            s->slot[k] = Active();
                            s->slot_state[k] = 0;
                            mb->join[k] = 0;
                            release(s, a, LBM2D_ERR_CUDA);
                        }
                    continue;
                }
                s->mask_running = s->mask_used;
                s->running = true;
                t_launch = t0;
                ++s->ticks;
                did = true;
            }
        }
        if (!did) {
            // nothing changed: wait a little for a set-up solve or the device
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait_for(lock, std::chrono::microseconds(s->running ? 50 : 2000),
                           [&] { return s->stop || !s->ready.empty(); });
        }
    }
}

}  // namespace

extern "C" {

int lbm2d_server_create_ex(int device, double budget_bytes, int max_active, int steps_per_tick, int flags,
                           lbm2d_server** out) {
    if (!out || max_active < 1 || steps_per_tick < 1) return LBM2D_ERR_INVALID;
    const bool resident = (flags & LBM2D_SERVE_RESIDENT) != 0;
    const bool fifo = (flags & LBM2D_SERVE_FIFO) != 0;
    if (resident && max_active > kResMaxSlots) return LBM2D_ERR_INVALID;
    auto* s = new lbm2d_server();
    s->device = device;
    s->resident = resident;
    s->fifo = fifo;
    s->budget = budget_bytes > 0 ? (size_t)budget_bytes : (size_t)64 << 30;
    s->max_active = max_active;
    s->steps_per_tick = steps_per_tick;
    int rc = lbm2d_batch_create(device, &s->batch);
    // narrow blocks: a serving mix holds many small grids, and a block that
    // overhangs a grid's right edge idles its overhanging threads
    if (!rc) rc = lbm2d_batch_set_block(s->batch, 32, 4);
    if (!rc && resident) {
        if (res_create(device, max_active, 32, 4, &s->loop) != 0 ||
            cudaStreamCreateWithFlags(&s->loop_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaMallocHost(&s->h_entry, sizeof(ResEntry)) != cudaSuccess)
            rc = LBM2D_ERR_CUDA;
        s->slot.assign((size_t)max_active, Active());
        s->slot_state.assign((size_t)max_active, 0);
    }
    if (rc) {
        if (s->loop) res_destroy(s->loop);
        if (s->loop_stream) cudaStreamDestroy(s->loop_stream);
        if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
        if (s->h_entry) cudaFreeHost(s->h_entry);
        if (s->batch) lbm2d_batch_destroy(s->batch);
        delete s;
        return rc;
    }
    cudaSetDevice(device);
    if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) s->ev0 = s->ev1 = nullptr;
    if (resident && !s->ev0) {
        lbm2d_server_destroy(s);
        return LBM2D_ERR_CUDA;
    }
    s->worker = std::thread(resident ? resident_loop : worker_loop, s);
    const unsigned hw = std::thread::hardware_concurrency();
    const int n_setup = (int)std::max(1u, std::min(hw > 2 ? hw - 2 : 1u, 6u));
    for (int k = 0; k < n_setup; ++k) s->setup_threads.emplace_back(setup_loop, s);
    *out = s;
    return LBM2D_OK;
}

int lbm2d_server_create(int device, double budget_bytes, int max_active, int steps_per_tick, lbm2d_server** out) {
    return lbm2d_server_create_ex(device, budget_bytes, max_active, steps_per_tick, 0, out);
}

int lbm2d_server_submit_state(lbm2d_server* s, const lbm2d_request* r, const double* f_init, double* f_out,
                              double* g_out, long long* id) {
    if (!s || !r || r->nx < 3 || r->ny < 3 || r->steps < 0) return LBM2D_ERR_INVALID;
    StateIO io;
    if (f_init) {
        const size_t n9 = (size_t)r->nx * r->ny * 9;
        io.f_init = std::make_shared<std::vector<double>>(f_init, f_init + n9);
    }
    io.f_out = f_out;
    io.g_out = g_out;
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return LBM2D_ERR_STATE;
    Pending p{s->next_id++, *r, now_s(), io};
    s->queue.push_back(p);
    ++s->submitted;
    if (id) *id = p.id;
    s->cv_setup.notify_all();
    return LBM2D_OK;
}

int lbm2d_server_submit(lbm2d_server* s, const lbm2d_request* r, long long* id) {
    return lbm2d_server_submit_state(s, r, nullptr, nullptr, nullptr, id);
}

int lbm2d_server_wait(lbm2d_server* s, long long n_finished, double timeout_s) {
    if (!s) return LBM2D_ERR_INVALID;
    std::unique_lock<std::mutex> lock(s->mu);
    const bool ok = s->cv.wait_for(lock, std::chrono::duration<double>(timeout_s),
                                   [&] { return s->finished >= n_finished; });
    return ok ? LBM2D_OK : LBM2D_ERR_TIMEOUT;
}

int lbm2d_server_results(lbm2d_server* s, lbm2d_result* out, int capacity, int* count) {
    if (!s || !count) return LBM2D_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    const int n = (int)s->results.size();
    for (int k = 0; k < std::min(n, capacity); ++k) out[k] = s->results[k];
    *count = n;
    return LBM2D_OK;
}

int lbm2d_server_stats(lbm2d_server* s, lbm2d_server_stats_t* st) {
    if (!s || !st) return LBM2D_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    st->submitted = s->submitted;
    st->finished = s->finished;
    st->queued = (long long)s->queue.size();
    st->active = (long long)s->live;
    st->setup_s = s->setup_s;
    st->gpu_s = s->gpu_s;
    st->call_s = s->call_s;
    st->wait_s = s->wait_s;
    st->retire_s = s->retire_s;
    st->join_s = s->join_s;
    st->busy_s = s->busy_s;
    st->lattice_updates = s->lattice_updates;
    st->device_bytes_in_use = (double)s->used;
    st->ticks = s->ticks;
    st->member_ticks = s->member_ticks;
    return LBM2D_OK;
}

int lbm2d_server_destroy(lbm2d_server* s) {
    if (!s) return LBM2D_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->queue.clear();
        s->cv.notify_all();
        s->cv_setup.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto& t : s->setup_threads)
        if (t.joinable()) t.join();
    for (size_t k = s->active.size(); k-- > 0;) retire(s, k, LBM2D_ERR_STATE);
    if (s->resident) {
        // solves still in the table (the loop has ended), then the ready ones
        for (size_t k = 0; k < s->slot.size(); ++k)
            if (s->slot_state[k] != 0) {
                Active a = s->slot[k];
                s->slot_state[k] = 0;
                release(s, a, LBM2D_ERR_STATE);
            }
        std::deque<Active> r;
        r.swap(s->ready);
        for (auto& a : r) release(s, a, LBM2D_ERR_STATE);
    } else {
        join_ready(s);  // set up but never stepped
    }
    for (size_t k = s->active.size(); k-- > 0;) retire(s, k, LBM2D_ERR_STATE);
    if (s->loop) res_destroy(s->loop);
    if (s->loop_stream) cudaStreamDestroy(s->loop_stream);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->h_entry) cudaFreeHost(s->h_entry);
    lbm2d_batch_destroy(s->batch);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
    return LBM2D_OK;
}

}  // extern "C"
