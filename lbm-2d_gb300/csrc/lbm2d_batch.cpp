// lbm2d_batch.cpp -- many independent solves in one launch, CUDA-graph
// replay, and the launch-shape autotuner.
//
// A batch owns a stream.  Each call of lbm2d_batch_step
//   1. prepares every member on its own stream (re-collision after a
//      parameter change, geometry and force-slot upload, prologue) and makes
//      the batch stream wait for it,
//   2. writes the kernel parameters of the next two steps of every member
//      (ping-pong parity 0 and 1) and the tile-to-instance table (first
//      launch block of every member) into device arrays,
//   3. launches, per (storage, thermal) group, one tile-pipelined kernel
//      over every member's tiles (FP64 members: one batch_step_kernel over
//      their blocks), followed by one batched force reduction, replaying step
//      pairs from a captured CUDA graph,
//   4. advances every member's state and orders the members' streams after
//      the batch stream.
#include <algorithm>
#include <chrono>
#include <map>
#include <tuple>

#include "lbm2d_runtime.h"

using namespace lbm2d;
using namespace lbm2d::rt;

namespace {
struct Member {
    lbm2d_solver* h;
    double tau, u;
    long long budget = -1;  // steps the member may still take (-1: unlimited)
};

struct Group {
    int storage = 0, thermal = 0;
    // KERNEL_TILES / KERNEL_SCALAR / KERNEL_PAIR (batched launches) or
    // KERNEL_ROWS (solo launches)
    int kind = 0;
    // KERNEL_TILES: global tile -> member, first global tile of each member,
    // and the persistent grid
    int* d_tile_member = nullptr;
    int* d_tile_start = nullptr;
    int ntiles = 0, grid = 0;
    std::vector<KParams> host;  // KERNEL_ROWS: each member's parameters of the call's first step
    std::vector<int> members;  // indices into lbm2d_batch::members
    int nblocks = 0;
    int njobs = 0;
    KParams* d_params[2] = {nullptr, nullptr};
    int2* d_block_map = nullptr;  // per launch block: (member, block index within the member)
    size_t cap_blocks = 0;
    std::vector<int2> h_block_map;  // the map last uploaded
    ReduceJob* d_jobs[2] = {nullptr, nullptr};  // per launch parity
    int* d_left = nullptr;  // step budgets: [0, m) read by parity-0 launches, [m, 2m) by parity 1
    size_t cap_members = 0;
};
}  // namespace

struct lbm2d_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    unsigned int* d_status = nullptr;  // bit 1: a tile-pipeline wait ran out
    cudaEvent_t ev = nullptr;
    // groups after the first run on side streams forked from the batch
    // stream at every step and joined back before the next
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev_join;
    std::vector<Member> members;
    std::vector<Group> groups;
    bool layout_dirty = true;
    int bx = 32, by = 4;  // one-warp-wide blocks (64 nodes for the paired kernel)
    // host staging (pinned) for parameters and budgets
    KParams* h_params = nullptr;
    size_t h_params_cap = 0;
    int* h_left = nullptr;
    size_t h_left_cap = 0;
    // captured step pair
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    long long launches = 0;
    std::string err;
};

namespace {

int bfail(lbm2d_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

#define BCK(expr, what)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (expr);                                                                 \
        if (e_ != cudaSuccess) return bfail(b, LBM2D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void free_groups(lbm2d_batch* b) {
    // stream-ordered: members join and leave a running serving loop without a
    // device-wide synchronization
    for (auto& g : b->groups) {
        cudaFreeAsync(g.d_params[0], b->stream);
        cudaFreeAsync(g.d_params[1], b->stream);
        if (g.d_block_map) cudaFreeAsync(g.d_block_map, b->stream);
        cudaFreeAsync(g.d_jobs[0], b->stream);
        cudaFreeAsync(g.d_jobs[1], b->stream);
        cudaFreeAsync(g.d_left, b->stream);
        if (g.d_tile_member) cudaFreeAsync(g.d_tile_member, b->stream);
        if (g.d_tile_start) cudaFreeAsync(g.d_tile_start, b->stream);
    }
    b->groups.clear();
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_valid = false;
}

int member_index(lbm2d_batch* b, lbm2d_solver* h) {
    for (size_t k = 0; k < b->members.size(); ++k)
        if (b->members[k].h == h) return (int)k;
    return -1;
}

// (Re)build the groups and their device arrays.
int build_layout(lbm2d_batch* b) {
    if (!b->layout_dirty) return LBM2D_OK;
    free_groups(b);
    std::map<std::tuple<int, int, int>, int> gi;
    for (size_t k = 0; k < b->members.size(); ++k) {
        lbm2d_solver* h = b->members[k].h;
        const auto key = std::make_tuple(h->storage, h->thermal ? 1 : 0, kernel_kind(h, true));
        auto it = gi.find(key);
        if (it == gi.end()) {
            gi[key] = (int)b->groups.size();
            Group g;
            g.storage = std::get<0>(key);
            g.thermal = std::get<1>(key);
            g.kind = std::get<2>(key);
            b->groups.push_back(g);
            it = gi.find(key);
        }
        b->groups[it->second].members.push_back((int)k);
    }
    for (auto& g : b->groups) {
        const size_t m = g.members.size();
        BCK(cudaMallocAsync(&g.d_params[0], m * sizeof(KParams), b->stream), "batch params");
        BCK(cudaMallocAsync(&g.d_params[1], m * sizeof(KParams), b->stream), "batch params");
        BCK(cudaMallocAsync(&g.d_jobs[0], m * sizeof(ReduceJob), b->stream), "batch jobs");
        BCK(cudaMallocAsync(&g.d_jobs[1], m * sizeof(ReduceJob), b->stream), "batch jobs");
        BCK(cudaMallocAsync(&g.d_left, 2 * m * sizeof(int), b->stream), "batch budgets");
        g.cap_members = m;
        if (g.kind == KERNEL_TILES) {
            // the tile table: member k owns global tiles [start[k], start[k+1])
            const int tw = tiles_width();
            std::vector<int> start(m + 1, 0), owner;
            for (size_t k = 0; k < m; ++k) {
                const long long nt = ((long long)b->members[g.members[k]].h->N + tw - 1) / tw;
                if ((long long)start[k] + nt > 0x7FFFFFFF) return bfail(b, LBM2D_ERR_INVALID, "batch: too many tiles");
                start[k + 1] = start[k] + (int)nt;
                owner.insert(owner.end(), (size_t)nt, (int)k);
            }
            g.ntiles = start[m];
            g.grid = tiles_grid(g.storage, g.thermal != 0, g.ntiles, b->device);
            if (g.grid <= 0) return bfail(b, LBM2D_ERR_CUDA, "tile pipeline: no launch configuration");
            BCK(cudaMallocAsync(&g.d_tile_member, owner.size() * sizeof(int), b->stream), "tile table");
            BCK(cudaMallocAsync(&g.d_tile_start, start.size() * sizeof(int), b->stream), "tile table");
            BCK(cudaMemcpyAsync(g.d_tile_member, owner.data(), owner.size() * sizeof(int), cudaMemcpyHostToDevice,
                                b->stream),
                "tile table");
            BCK(cudaMemcpyAsync(g.d_tile_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice,
                                b->stream),
                "tile table");
            BCK(cudaStreamSynchronize(b->stream), "tile table");  // the host vectors go out of scope
        }
    }
    b->layout_dirty = false;
    return LBM2D_OK;
}

int ensure_host_params(lbm2d_batch* b, size_t n) {
    if (n > b->h_params_cap) {
        if (b->h_params) cudaFreeHost(b->h_params);
        b->h_params = nullptr;
        BCK(cudaMallocHost(&b->h_params, n * sizeof(KParams)), "pinned params");
        b->h_params_cap = n;
    }
    if (n > b->h_left_cap) {
        if (b->h_left) cudaFreeHost(b->h_left);
        b->h_left = nullptr;
        BCK(cudaMallocHost(&b->h_left, n * sizeof(int)), "pinned budgets");
        b->h_left_cap = n;
    }
    return LBM2D_OK;
}

// Steps 1-2 of the file comment; fills every group's device arrays.
int prepare(lbm2d_batch* b) {
    int rc;
    if ((rc = build_layout(b))) return rc;
    size_t total = 0;
    for (auto& g : b->groups) total += 2 * g.members.size();
    if ((rc = ensure_host_params(b, std::max<size_t>(total, 1)))) return rc;
    size_t off = 0;
    for (auto& g : b->groups) {
        const size_t m = g.members.size();
        KParams* p0 = b->h_params + off;
        KParams* p1 = p0 + m;
        int* left = b->h_left + off;
        std::vector<int> start(m + 1, 0), reg(m, 0);
        std::vector<ReduceJob> jobs[2];
        for (size_t k = 0; k < m; ++k) {
            Member& mem = b->members[g.members[k]];
            lbm2d_solver* h = mem.h;
            if ((rc = check_handle(h))) return bfail(b, rc, std::string("member: ") + h->err);
            if (h->bx != b->bx || h->by != b->by) {
                h->bx = b->bx;
                h->by = b->by;
            }
            KParams p;
            const long long l0 = h->launches;
            if ((rc = prepare_steps(h, mem.tau, mem.u, p, true))) return bfail(b, rc, std::string("member: ") + h->err);
            const bool budgeted = mem.budget >= 0;
            left[k] = (int)std::min<long long>(std::max(mem.budget, 0LL), 0x7FFFFFFF);
            if (budgeted) {
                p.left_in = g.d_left + k;
                p.left_out = g.d_left + m + k;
            }
            p0[k] = p;
            p1[k] = p;
            p1[k].fin = p.fout;
            p1[k].fout = const_cast<void*>(p.fin);
            p1[k].gin = p.gout;
            p1[k].gout = const_cast<void*>(p.gin);
            p1[k].seed_in = p.seed_out;
            p1[k].seed_out = const_cast<uint32_t*>(p.seed_in);
            p1[k].left_in = p.left_out;
            p1[k].left_out = const_cast<int*>(p.left_in);
            // order the batch stream after the member's own preparation (a
            // prologue on the member's stream); nothing to order otherwise,
            // the member's stream already waits for the batch's last step
            if (h->launches != l0) {
                BCK(cudaEventRecord(b->ev, h->stream), "event");
                BCK(cudaStreamWaitEvent(b->stream, b->ev, 0), "wait");
            }
            const int gy = (h->ny + b->by - 1) / b->by;
            // tile blocks, then the member's boundary blocks (nbpairs set only
            // when its slots are laid out for them)
            const int nbb = p.nbpairs > 0 ? (p.nbpairs + p.bchunk - 1) / p.bchunk : 0;
            reg[k] = ((p.ftiles > 0 ? p.ftiles : p.gx * gy) + kBatchTiles - 1) / kBatchTiles;
            start[k + 1] = start[k] + reg[k] + nbb;
            if (h->nslots > 0) {
                jobs[0].push_back({h->d_partials, h->nslots, h->hist_cap, h->d_hist, h->d_counter, h->d_last,
                                   budgeted ? g.d_left + k : nullptr});
                jobs[1].push_back({h->d_partials, h->nslots, h->hist_cap, h->d_hist, h->d_counter, h->d_last,
                                   budgeted ? g.d_left + m + k : nullptr});
            }
        }
        if (g.kind == KERNEL_ROWS) {
            g.host.assign(p0, p0 + m);
            g.nblocks = 0;
            g.njobs = 0;
            off += 2 * m;
            continue;
        }
        g.nblocks = start[m];
        g.njobs = (int)jobs[0].size();
        BCK(cudaMemcpyAsync(g.d_params[0], p0, m * sizeof(KParams), cudaMemcpyHostToDevice, b->stream), "params");
        BCK(cudaMemcpyAsync(g.d_params[1], p1, m * sizeof(KParams), cudaMemcpyHostToDevice, b->stream), "params");
        // budgets at the start of the call, read by the first (parity-0) launch
        BCK(cudaMemcpyAsync(g.d_left, left, m * sizeof(int), cudaMemcpyHostToDevice, b->stream), "budgets");
        // the block map (rebuilt only when the member sizes or the shape change)
        std::vector<int2> map((size_t)g.nblocks);
        // (member, tile block index), or (member, -(i + 1)) for boundary block i
        for (size_t k = 0; k < m; ++k)
            for (int q = start[k]; q < start[k + 1]; ++q) {
                const int local = q - start[k];
                map[(size_t)q] = make_int2((int)k, local < reg[k] ? local : -(local - reg[k] + 1));
            }
        if (map.size() != g.h_block_map.size() ||
            !std::equal(map.begin(), map.end(), g.h_block_map.begin(),
                        [](const int2& a, const int2& c) { return a.x == c.x && a.y == c.y; })) {
            if (map.size() != g.h_block_map.size()) b->graph_valid = false;  // the grid size changed
            if (map.size() > g.cap_blocks) {
                if (g.d_block_map) cudaFreeAsync(g.d_block_map, b->stream);
                g.d_block_map = nullptr;
                BCK(cudaMallocAsync(&g.d_block_map, std::max<size_t>(map.size(), 1) * sizeof(int2), b->stream),
                    "batch block map");
                g.cap_blocks = map.size();
                b->graph_valid = false;  // captured launches name the old buffer
            }
            if (!map.empty())
                BCK(cudaMemcpyAsync(g.d_block_map, map.data(), map.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                    b->stream),
                    "batch block map");
            g.h_block_map.swap(map);
        }
        for (int par = 0; par < 2; ++par)
            if (!jobs[par].empty())
                BCK(cudaMemcpyAsync(g.d_jobs[par], jobs[par].data(), jobs[par].size() * sizeof(ReduceJob),
                                    cudaMemcpyHostToDevice, b->stream),
                    "jobs");
        off += 2 * m;
    }
    // the staging buffers may be rewritten by the next call: wait for the copies
    BCK(cudaStreamSynchronize(b->stream), "params sync");
    return LBM2D_OK;
}

// One step of every batched group.  The groups' members are independent, so
// the groups run concurrently: the first on the batch stream, each other one
// on a side stream forked from it and joined back (a paired and a one-node
// group overlap: 16 + 16 FP16 cylinders 512x256 / 511x256, 104-118 against
// 98 us per step).
// Side streams and join events for every batched group but the first
// (created outside any stream capture).
int ensure_side(lbm2d_batch* b) {
    size_t n = 0;
    for (auto& g : b->groups)
        if (g.kind != KERNEL_ROWS) ++n;
    while (b->side.size() + 1 < n) {
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        BCK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "side stream");
        b->side.push_back(s);
        BCK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "join event");
        b->ev_join.push_back(e);
    }
    return LBM2D_OK;
}

int launch_one(lbm2d_batch* b, int parity) {
    std::vector<Group*> gs;
    for (auto& g : b->groups)
        if (g.kind != KERNEL_ROWS) gs.push_back(&g);  // solo members are launched by lbm2d_batch_step
    const size_t nside = gs.empty() ? 0 : gs.size() - 1;
    if (b->side.size() < nside) return bfail(b, LBM2D_ERR_STATE, "batch side streams missing");
    if (nside > 0) BCK(cudaEventRecord(b->ev_fork, b->stream), "fork");
    for (size_t i = 0; i < gs.size(); ++i) {
        Group& g = *gs[i];
        cudaStream_t s = i == 0 ? b->stream : b->side[i - 1];
        if (i > 0) BCK(cudaStreamWaitEvent(s, b->ev_fork, 0), "fork wait");
        int e = g.kind == KERNEL_TILES
                    ? launch_tiles_batch(g.storage, g.thermal != 0, g.d_params[parity], g.d_tile_member,
                                         g.d_tile_start, g.ntiles, g.grid, b->d_status, s)
                    : launch_batch_step(g.storage, g.d_params[parity], g.d_block_map, g.nblocks, g.thermal, b->bx,
                                        b->by, s, g.kind == KERNEL_PAIR ? 1 : 0);
        ++b->launches;
        if (e) return bfail(b, LBM2D_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString((cudaError_t)e));
        if (g.njobs > 0) {
            e = launch_batch_force_reduce(g.d_jobs[parity], g.njobs, s);
            ++b->launches;
            if (e) return bfail(b, LBM2D_ERR_CUDA, std::string("batch reduce: ") + cudaGetErrorString((cudaError_t)e));
        }
        if (i > 0) {
            BCK(cudaEventRecord(b->ev_join[i - 1], s), "join");
            BCK(cudaStreamWaitEvent(b->stream, b->ev_join[i - 1], 0), "join wait");
        }
    }
    return LBM2D_OK;
}

int capture_pair(lbm2d_batch* b) {
    if (b->graph_valid) return LBM2D_OK;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaGraph_t g = nullptr;
    int rs = ensure_side(b);
    if (rs) return rs;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const long long l0 = b->launches;
    int rc = launch_one(b, 0);
    if (!rc) rc = launch_one(b, 1);
    b->launches = l0;  // captured launches are counted when replayed
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return bfail(b, LBM2D_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, LBM2D_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    b->graph_valid = true;
    return LBM2D_OK;
}

long long launches_per_step(const lbm2d_batch* b) {
    long long n = 0;
    for (auto& g : b->groups)
        if (g.kind != KERNEL_ROWS) n += 1 + (g.njobs > 0 ? 1 : 0);
    return n;
}

}  // namespace

extern "C" {

int lbm2d_batch_create(int device, lbm2d_batch** out) {
    if (!out) return LBM2D_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return LBM2D_ERR_NO_DEVICE;
    }
    auto* b = new lbm2d_batch();
    b->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&b->d_status, 16) != cudaSuccess || cudaMemset(b->d_status, 0, 16) != cudaSuccess) {
        delete b;
        return LBM2D_ERR_CUDA;
    }
    *out = b;
    return LBM2D_OK;
}

int lbm2d_batch_destroy(lbm2d_batch* b) {
    if (!b) return LBM2D_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    free_groups(b);
    cudaStreamSynchronize(b->stream);
    if (b->h_params) cudaFreeHost(b->h_params);
    if (b->h_left) cudaFreeHost(b->h_left);
    cudaEventDestroy(b->ev);
    cudaEventDestroy(b->ev_fork);
    for (cudaStream_t s : b->side) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->ev_join) cudaEventDestroy(e);
    cudaStreamDestroy(b->stream);
    cudaFree(b->d_status);
    delete b;
    return LBM2D_OK;
}

const char* lbm2d_batch_last_error(const lbm2d_batch* b) { return b ? b->err.c_str() : ""; }

int lbm2d_batch_add(lbm2d_batch* b, lbm2d_solver* h, double tau, double u) {
    if (!b || !h) return LBM2D_ERR_INVALID;
    if (h->device != b->device) return bfail(b, LBM2D_ERR_INVALID, "member lives on another device");
    if (!(tau > 0.0)) return bfail(b, LBM2D_ERR_INVALID, "tau must be positive");
    if (member_index(b, h) >= 0) return bfail(b, LBM2D_ERR_INVALID, "already a member");
    if (ibm_active(h)) return bfail(b, LBM2D_ERR_INVALID, "a solver with an immersed boundary steps alone");
    b->members.push_back({h, tau, u});
    h->in_batch = true;
    b->layout_dirty = true;
    return LBM2D_OK;
}

int lbm2d_batch_remove(lbm2d_batch* b, lbm2d_solver* h) {
    if (!b || !h) return LBM2D_ERR_INVALID;
    const int k = member_index(b, h);
    if (k < 0) return bfail(b, LBM2D_ERR_INVALID, "not a member");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);  // no batched work may still touch h
    b->members.erase(b->members.begin() + k);
    h->in_batch = false;
    b->layout_dirty = true;
    return LBM2D_OK;
}

int lbm2d_batch_set_params(lbm2d_batch* b, lbm2d_solver* h, double tau, double u) {
    if (!b || !h) return LBM2D_ERR_INVALID;
    const int k = member_index(b, h);
    if (k < 0) return bfail(b, LBM2D_ERR_INVALID, "not a member");
    if (!(tau > 0.0)) return bfail(b, LBM2D_ERR_INVALID, "tau must be positive");
    b->members[k].tau = tau;
    b->members[k].u = u;
    return LBM2D_OK;
}

int lbm2d_batch_set_budget(lbm2d_batch* b, lbm2d_solver* h, long long steps) {
    if (!b || !h) return LBM2D_ERR_INVALID;
    const int k = member_index(b, h);
    if (k < 0) return bfail(b, LBM2D_ERR_INVALID, "not a member");
    if (steps > 0x7FFFFFFF) return bfail(b, LBM2D_ERR_INVALID, "budget above 2^31 - 1 steps");
    b->members[k].budget = steps < 0 ? -1 : steps;
    return LBM2D_OK;
}

long long lbm2d_batch_budget(lbm2d_batch* b, lbm2d_solver* h) {
    if (!b || !h) return -1;
    const int k = member_index(b, h);
    return k < 0 ? -1 : b->members[k].budget;
}

int lbm2d_batch_size(lbm2d_batch* b) { return b ? (int)b->members.size() : 0; }

int lbm2d_batch_step(lbm2d_batch* b, int nsteps) {
    if (!b || nsteps < 0) return LBM2D_ERR_INVALID;
    if (nsteps == 0 || b->members.empty()) return LBM2D_OK;
    if (cudaSetDevice(b->device) != cudaSuccess) return LBM2D_ERR_CUDA;
    const bool relayout = b->layout_dirty;
    int rc = prepare(b);
    if (rc) return rc;
    if (relayout) b->graph_valid = false;
    // solo members (the row pipeline fills the GPU for each of them): their
    // steps are launched one after another on the batch stream; members are
    // independent, so they need no ordering against the batched launches
    for (auto& g : b->groups) {
        if (g.kind != KERNEL_ROWS) continue;
        for (size_t k = 0; k < g.members.size(); ++k) {
            const Member& mem = b->members[g.members[k]];
            lbm2d_solver* h = mem.h;
            const long long taken = mem.budget >= 0 ? std::min<long long>(mem.budget, nsteps) : nsteps;
            KParams p = g.host[k];
            for (long long st = 0; st < taken; ++st) {
                const int c = h->cur ^ (int)(st & 1);
                p.fin = h->P[c];
                p.fout = h->P[c ^ 1];
                p.gin = h->G[c];
                p.gout = h->G[c ^ 1];
                p.seed_in = h->d_seed + c;
                p.seed_out = h->d_seed + (c ^ 1);
                p.skip_settled_solids = (h->steps_since_collide + st >= 2 && h->hook != 1) ? 1 : 0;
                int e = launch_rows(h->storage, p, h->slot_grid, b->stream);
                ++b->launches;
                if (e) return bfail(b, LBM2D_ERR_CUDA, std::string("solo step: ") + cudaGetErrorString((cudaError_t)e));
                if (h->nslots > 0) {
                    e = launch_force_reduce(h->d_partials, h->nslots, h->d_hist, h->hist_cap, h->d_counter, h->d_last,
                                            b->stream);
                    ++b->launches;
                    if (e) return bfail(b, LBM2D_ERR_CUDA, std::string("solo reduce: ") + cudaGetErrorString((cudaError_t)e));
                }
            }
        }
    }
    if (launches_per_step(b) > 0) {
        const int pairs = nsteps / 2;
        if (pairs > 0) {
            if ((rc = capture_pair(b))) return rc;
            for (int k = 0; k < pairs; ++k) {
                BCK(cudaGraphLaunch(b->graph, b->stream), "graph launch");
                b->launches += 2 * launches_per_step(b);
            }
        }
        if (nsteps & 1) {
            if ((rc = ensure_side(b))) return rc;
            if ((rc = launch_one(b, 0))) return rc;
        }
    }
    for (auto& m : b->members) {
        lbm2d_solver* h = m.h;
        long long taken = nsteps;
        if (m.budget >= 0) {
            taken = std::min<long long>(m.budget, nsteps);
            m.budget -= taken;
        }
        h->cur ^= (int)(taken & 1);
        h->steps_since_collide += taken;
        h->steps_done += taken;
        if (taken > 0) h->u_last = m.u;
    }
    BCK(cudaEventRecord(b->ev, b->stream), "event");
    for (auto& m : b->members) BCK(cudaStreamWaitEvent(m.h->stream, b->ev, 0), "member wait");
    return LBM2D_OK;
}

int lbm2d_batch_synchronize(lbm2d_batch* b) {
    if (!b) return LBM2D_ERR_INVALID;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->stream), "batch sync");
    unsigned int status = 0;
    BCK(cudaMemcpy(&status, b->d_status, sizeof(status), cudaMemcpyDeviceToHost), "batch status");
    if (status) {
        cudaMemset(b->d_status, 0, sizeof(status));
        return bfail(b, LBM2D_ERR_TIMEOUT, "a batched tile-pipeline wait exceeded its limit");
    }
    for (auto& m : b->members) {
        int rc = lbm2d_synchronize(m.h);
        if (rc) return bfail(b, rc, std::string("member: ") + m.h->err);
    }
    return LBM2D_OK;
}

int lbm2d_batch_set_block(lbm2d_batch* b, int bx, int by) {
    if (!b) return LBM2D_ERR_INVALID;
    if (bx == 0 && by == 0) {  // the default: narrow blocks for mixes of small grids
        bx = 32;
        by = 4;
    }
    if (bx <= 0 || by <= 0 || bx * by > 512 || (bx * by) % 32 != 0)
        return bfail(b, LBM2D_ERR_INVALID, "block must have a multiple of 32 threads, at most 512");
    if (bx != b->bx || by != b->by) {
        b->bx = bx;
        b->by = by;
        b->layout_dirty = true;
    }
    return LBM2D_OK;
}

void* lbm2d_batch_stream(lbm2d_batch* b) { return b ? (void*)b->stream : nullptr; }
long long lbm2d_batch_launch_count(lbm2d_batch* b) { return b ? b->launches : 0; }

}  // extern "C"

// ---------------------------------------------------------------- autotuner
namespace {
const int kShapes[][2] = {{32, 4}, {32, 8}, {64, 2}, {64, 4}, {128, 1}, {128, 2}, {128, 4}, {256, 1}, {256, 2},
                          {512, 1}, {32, 16}, {64, 8}};

// Save a member's state (rebuild S into staging) so tuning steps can be undone.
int save_state(lbm2d_solver* h, unsigned long long& counter) {
    int rc;
    if ((rc = materialize(h))) return rc;
    // the handle's stream is non-blocking: read the counter on it, after its work
    if (cudaMemcpyAsync(&counter, h->d_counter, sizeof(counter), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return LBM2D_ERR_CUDA;
    return LBM2D_OK;
}

int restore_state(lbm2d_solver* h, unsigned long long counter, long long steps_done) {
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return LBM2D_ERR_CUDA;
    h->staged = true;  // staging still holds the saved S; the next step re-collides it
    h->steps_done = steps_done;
    if (cudaMemcpyAsync(h->d_counter, &counter, sizeof(counter), cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return LBM2D_ERR_CUDA;
    return LBM2D_OK;
}
}  // namespace

extern "C" {

int lbm2d_autotune(lbm2d_solver* h, int steps, double tau, double u, int* best_bx, int* best_by) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (steps < 1) steps = 1;
    unsigned long long counter = 0;
    const long long done = h->steps_done;
    if ((rc = save_state(h, counter))) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // Candidates: the row pipeline (when the solver would run it), then every
    // block shape of the paired (or scalar) kernel.
    const int v0 = h->variant;
    // the persistent kernels (row or tile pipeline) are one candidate; the
    // block shapes are candidates of the paired (or one-node) kernel
    const int kind0 = kernel_kind(h);
    const bool rows = kind0 == KERNEL_ROWS || kind0 == KERNEL_TILES;
    const int shape_variant = rows ? (use_pair(h) ? 2 : 1) : v0;
    float best = 1e30f;
    int bbx = h->bx, bby = h->by, bvar = v0;
    const int n_cand = (int)(sizeof(kShapes) / sizeof(kShapes[0])) + (rows ? 1 : 0);
    for (int c = 0; c < n_cand; ++c) {
        const bool is_rows = rows && c == 0;
        const int* s = is_rows ? nullptr : kShapes[c - (rows ? 1 : 0)];
        if (s && s[0] > 2 * h->nx && s[0] > 32) continue;
        h->variant = is_rows ? 0 : shape_variant;
        if (s) {
            h->bx = s[0];
            h->by = s[1];
        }
        h->staged = true;
        if ((rc = lbm2d_step(h, tau, u, 2))) break;  // prologue + warm-up
        cudaEventRecord(e0, h->stream);
        if ((rc = lbm2d_step(h, tau, u, steps))) break;
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bvar = h->variant;
            if (s) {
                bbx = s[0];
                bby = s[1];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->variant = bvar;
    h->bx = bbx;
    h->by = bby;
    const int rc2 = restore_state(h, counter, done);
    if (rc) return rc;
    if (rc2) return rc2;
    const bool rows_best = rows && bvar == 0;
    if (best_bx) *best_bx = rows_best ? 0 : bbx;
    if (best_by) *best_by = rows_best ? 0 : bby;
    return LBM2D_OK;
}

int lbm2d_batch_autotune(lbm2d_batch* b, int steps, int* best_bx, int* best_by) {
    if (!b) return LBM2D_ERR_INVALID;
    if (b->members.empty()) return LBM2D_OK;
    if (steps < 1) steps = 1;
    cudaSetDevice(b->device);
    std::vector<unsigned long long> counters(b->members.size());
    std::vector<long long> done(b->members.size()), budgets(b->members.size());
    int rc;
    for (size_t k = 0; k < b->members.size(); ++k) {
        done[k] = b->members[k].h->steps_done;
        budgets[k] = b->members[k].budget;
        b->members[k].budget = -1;  // tuning steps are not the members' own
        if ((rc = save_state(b->members[k].h, counters[k]))) return bfail(b, rc, "autotune save");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bbx = b->bx, bby = b->by;
    rc = LBM2D_OK;
    for (auto& s : kShapes) {
        if ((rc = lbm2d_batch_set_block(b, s[0], s[1]))) break;
        for (auto& m : b->members) m.h->staged = true;
        if ((rc = lbm2d_batch_step(b, 2))) break;
        cudaEventRecord(e0, b->stream);
        if ((rc = lbm2d_batch_step(b, steps))) break;
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bbx = s[0];
            bby = s[1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    lbm2d_batch_set_block(b, bbx, bby);
    for (size_t k = 0; k < b->members.size(); ++k) {
        const int r2 = restore_state(b->members[k].h, counters[k], done[k]);
        if (!rc && r2) rc = r2;
        b->members[k].budget = budgets[k];
    }
    if (rc) return rc;
    if (best_bx) *best_bx = bbx;
    if (best_by) *best_by = bby;
    return LBM2D_OK;
}

}  // extern "C"
