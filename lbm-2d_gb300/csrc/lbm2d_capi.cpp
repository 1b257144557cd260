// lbm2d_capi.cpp -- the C-ABI (include/lbm2d.h) over the CUDA kernels.
//
// The handle keeps the device state in one of two forms:
//   STAGED    the reference's state S (post-stream, post-boundary) as FP64
//             AoS in device staging buffers -- right after an upload;
//   COLLIDED  the post-collision populations of S in the storage precision,
//             SoA -- what the step kernel consumes and produces.
// A step call collides a STAGED state first (prologue kernel) with the
// call's own collision parameters, so results match execute_time_step
// (src/lbm.hpp:293-582) even when tau, the body force or the thermal
// parameters change between calls: a change of those parameters, of the
// geometry or of the case first rebuilds S from the stored populations
// (readback kernel) and re-collides it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "lbm2d_runtime.h"

using namespace lbm2d;

namespace {
thread_local std::string g_global_err;
}  // namespace

namespace lbm2d {
namespace rt {

int fail(lbm2d_solver* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

int cuda_fail(lbm2d_solver* h, cudaError_t e, const char* what) {
    return fail(h, e == cudaErrorMemoryAllocation ? LBM2D_ERR_OOM : LBM2D_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr, what)                                  \
    do {                                                \
        cudaError_t e_ = (expr);                        \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
    } while (0)

// Device buffers come from the stream-ordered allocator on the handle's
// stream: creating and destroying solves (the serving loop does it for every
// request) then neither synchronizes the device nor stalls other streams.
// Mapped pinned (fx, fy) pairs of the solvers, cut from chunks that live as
// long as the process: freeing pinned memory waits for the whole device, so
// a solver destroyed while other work runs (a serving loop retiring a solve
// while its device loop steps the others) would stall on it.
struct PinnedPairs {
    std::mutex mu;
    std::vector<double*> free_slots;
};
PinnedPairs& pinned_pairs() {
    static PinnedPairs* p = new PinnedPairs();  // never destroyed: solvers may outlive static destructors
    return *p;
}
int pinned_pair_get(double** host, double** dev) {
    PinnedPairs& P = pinned_pairs();
    std::lock_guard<std::mutex> lock(P.mu);
    if (P.free_slots.empty()) {
        constexpr int kChunk = 4096;
        double* c = nullptr;
        if (cudaHostAlloc(&c, kChunk * 2 * sizeof(double), cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess)
            return 1;
        for (int i = kChunk; i-- > 0;) P.free_slots.push_back(c + 2 * i);
    }
    double* h = P.free_slots.back();
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) return 1;
    P.free_slots.pop_back();
    *host = h;
    *dev = static_cast<double*>(d);
    return 0;
}
void pinned_pair_put(double* host) {
    PinnedPairs& P = pinned_pairs();
    std::lock_guard<std::mutex> lock(P.mu);
    P.free_slots.push_back(host);
}

template <class T>
int dalloc(lbm2d_solver* h, T** p, size_t bytes) {
    if (*p) return LBM2D_OK;
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, bytes ? bytes : 16, h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaMallocAsync");
    *p = static_cast<T*>(q);
    h->device_bytes += bytes;
    return LBM2D_OK;
}

template <class T>
void dfree(lbm2d_solver* h, T** p) {
    if (*p) cudaFreeAsync(*p, h->stream);
    *p = nullptr;
}

int bc_kind(int case_type) {
    if (case_type == CASE_CAVITY) return BC_LID;
    if (case_type == CASE_STEP) return BC_STEP;
    if (case_type == CASE_RIBS || case_type == CASE_HILLS) return BC_NONE;
    return BC_INFLOW;
}

CollideParams collide_params(const lbm2d_solver* h, double tau) {
    CollideParams c;
    c.collision = h->collision;
    c.tau = tau;
    const double s = 1.0 / tau;  // MRTParams::from_tau, src/lbm_types.hpp:72-76
    c.s_shear = (s < 0.5) ? 0.5 : ((s > 1.99) ? 1.99 : s);
    c.s_bulk = 1.2;
    c.s_normal = 1.0;
    c.cs_sq = h->use_les ? h->cs * h->cs : 0.0;
    c.les = (h->collision == 0 && c.cs_sq > 0.0 && tau > 0.0) ? 1 : 0;
    c.nu = (tau - 0.5) / 3.0;
    c.Fscale = (h->body_force != 0.0) ? (1.0 - 1.0 / (2.0 * tau)) * 3.0 * h->body_force : 0.0;
    c.thermal = h->thermal ? 1 : 0;
    if (h->thermal) {
        c.omega_k = h->omega_k;
        c.beta = h->beta;
        c.g_buoy = h->g_buoy;
        c.T_ref = h->T_ref;
    }
    return c;
}

// Flat tiles of a batched paired member: ceil(N / 2) pairs, bx*by per tile.
int flat_tiles(const lbm2d_solver* h) {
    const long long pairs = ((long long)h->N + 1) / 2, B = (long long)h->bx * h->by;
    return (int)((pairs + B - 1) / B);
}

KParams base_params(const lbm2d_solver* h) {
    KParams p;
    std::memset(&p, 0, sizeof(p));
    p.nx = h->nx;
    p.ny = h->ny;
    p.N = (long long)h->N;
    p.flags = h->d_flags;
    p.rec_info = h->d_rec_info;
    p.rec_force = h->d_rec_force;
    p.rec_wd = h->d_rec_wd;
    p.rec_q = h->d_rec_q;
    p.rec_uw = h->d_rec_uw;
    p.interp_classic = h->bb.use_mei ? 0 : 1;
    p.moving_wall = h->bb.has_moving_wall ? 1 : 0;
    p.bc_kind = bc_kind(h->case_type);
    p.thermal = h->thermal ? 1 : 0;
    p.hook_kind = h->thermal ? h->hook : 0;
    p.hook_a = h->hook_a;
    p.hook_b = h->hook_b;
    p.pd.hook_a = h->hook_a;
    p.pd.hook_b = h->hook_b;
    p.pf.hook_a = float(h->hook_a);
    p.pf.hook_b = float(h->hook_b);
    p.pd.T_ref = h->T_ref;
    p.pf.T_ref = float(h->T_ref);
    p.nan_flag = h->d_nan;
    p.consumer_wait = h->consumer_wait;
    p.inv_nx = 1.0f / float(h->nx);
    if (h->slot_kind == KERNEL_ROWS || h->slot_bpass) {
        p.bpairs = h->d_bpairs;
        p.nbpairs = h->nbpairs;
        p.bchunk = h->bchunk;
    }
    if (h->slot_bpass) p.ftiles = flat_tiles(h);
    p.pair = use_pair(h) ? 1 : 0;
    const int nbw = h->bx * (p.pair ? 2 : 1);  // node width of a block
    p.gx = (h->nx + nbw - 1) / nbw;
    const bool shifted = h->storage != ST_FP64;  // FP32/FP16/BF16 store deviations
    for (int j = 0; j < 9; ++j) {
        p.shf[j] = shifted ? float(W[j]) : 0.0f;
        p.shg[j] = shifted ? float(W[j] * h->T_ref) : 0.0f;
    }
    return p;
}

template <class R>
void fill_phys(Phys<R>& q, const CollideParams& c) {
    q.s_shear = R(c.s_shear);
    q.s_bulk = R(c.s_bulk);
    q.s_normal = R(c.s_normal);
    q.tau = R(c.tau);
    q.inv_tau = R(1.0 / c.tau);
    q.cs_sq = R(c.cs_sq);
    q.cs = R(std::sqrt(c.cs_sq));
    q.nu = R(c.nu);
    q.inv_nu = c.nu > 0.0 ? R(1.0 / c.nu) : R(0);
    q.Fscale = R(c.Fscale);
    q.omega_k = R(c.omega_k);
    q.beta = R(c.beta);
    q.g_buoy = R(c.g_buoy);
    q.T_ref = R(c.T_ref);
}

void set_u_bc(KParams& p, double u) {
    p.u_bc = u;
    p.pd.u_bc = u;
    p.pf.u_bc = float(u);
}

void apply_collide(KParams& p, const CollideParams& c) {
    fill_phys(p.pd, c);
    fill_phys(p.pf, c);
    p.collide = 1;
    p.collision = c.collision;
    p.s_shear = c.s_shear;
    p.s_bulk = c.s_bulk;
    p.s_normal = c.s_normal;
    p.tau = c.tau;
    p.cs_sq = c.cs_sq;
    p.nu = c.nu;
    p.Fscale = c.Fscale;
    p.les = c.les;
    p.omega_k = c.omega_k;
    p.beta = c.beta;
    p.g_buoy = c.g_buoy;
    p.T_ref = c.T_ref;
}

int ensure_populations(lbm2d_solver* h) {
    // 64 bytes of tail padding: the tile pipeline copies whole 16-byte granules
    const size_t bytes = h->N * 9 * elem_size(h->storage) + 64;
    int rc;
    if ((rc = dalloc(h, &h->P[0], bytes))) return rc;
    if ((rc = dalloc(h, &h->P[1], bytes))) return rc;
    if (h->thermal) {
        if ((rc = dalloc(h, &h->G[0], bytes))) return rc;
        if ((rc = dalloc(h, &h->G[1], bytes))) return rc;
    }
    return LBM2D_OK;
}

// Fill staging with the constructor defaults (f = 0, g = 1; src/lbm_types.hpp:211-216).
int ensure_stage(lbm2d_solver* h, bool want_g) {
    int rc;
    const size_t bytes = h->N * 9 * sizeof(double);
    if (!h->d_stage_f) {
        if ((rc = dalloc(h, &h->d_stage_f, bytes))) return rc;
        CK(cudaMemsetAsync(h->d_stage_f, 0, bytes, h->stream), "memset");
    }
    if (want_g && !h->d_stage_g) {
        if ((rc = dalloc(h, &h->d_stage_g, bytes))) return rc;
        std::vector<double> ones(std::min<size_t>(h->N * 9, size_t(1) << 20), 1.0);
        for (size_t off = 0; off < h->N * 9; off += ones.size()) {
            const size_t cnt = std::min(ones.size(), h->N * 9 - off);
            CK(cudaMemcpyAsync(h->d_stage_g + off, ones.data(), cnt * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream),
               "fill g");
            CK(cudaStreamSynchronize(h->stream), "sync");
        }
    }
    return LBM2D_OK;
}

int upload_geometry(lbm2d_solver* h) {
    if (!h->geom_dirty) return LBM2D_OK;
    GeometryInput in;
    in.nx = h->nx;
    in.ny = h->ny;
    in.case_type = h->case_type;
    in.thermal = h->thermal;
    in.les = h->use_les && h->collision == 0 && h->cs * h->cs > 0.0;
    in.mask = h->mask.data();
    in.bb = &h->bb;
    std::string err;
    if (!build_geometry(in, h->geo, err)) return fail(h, LBM2D_ERR_INVALID, err);
    dfree(h, &h->d_rec_info);
    dfree(h, &h->d_rec_force);
    dfree(h, &h->d_rec_wd);
    dfree(h, &h->d_rec_q);
    dfree(h, &h->d_rec_uw);
    dfree(h, &h->d_block_slot);
    dfree(h, &h->d_partials);
    dfree(h, &h->d_bpairs);
    h->nbpairs = h->bchunk = 0;
    h->nslots = 0;
    h->slot_bx = h->slot_by = 0;
    int rc;
    if ((rc = dalloc(h, &h->d_flags, h->N * sizeof(uint32_t) + 64))) return rc;  // granule padding
    CK(cudaMemcpyAsync(h->d_flags, h->geo.flags.data(), h->N * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream),
       "flags H2D");
    const size_t nr = h->geo.rec_info.size();
    if ((rc = dalloc(h, &h->d_rec_info, nr * 4 + 16))) return rc;
    if ((rc = dalloc(h, &h->d_rec_force, nr * 4 + 16))) return rc;
    if ((rc = dalloc(h, &h->d_rec_wd, nr * 8 + 16))) return rc;
    if ((rc = dalloc(h, &h->d_rec_q, nr * 72 + 16))) return rc;
    if ((rc = dalloc(h, &h->d_rec_uw, nr * 144 + 16))) return rc;
    if (nr) {
        CK(cudaMemcpyAsync(h->d_rec_info, h->geo.rec_info.data(), nr * 4, cudaMemcpyHostToDevice, h->stream), "H2D");
        CK(cudaMemcpyAsync(h->d_rec_force, h->geo.rec_force.data(), nr * 4, cudaMemcpyHostToDevice, h->stream), "H2D");
        CK(cudaMemcpyAsync(h->d_rec_wd, h->geo.rec_wd.data(), nr * 8, cudaMemcpyHostToDevice, h->stream), "H2D");
        CK(cudaMemcpyAsync(h->d_rec_q, h->geo.rec_q.data(), nr * 72, cudaMemcpyHostToDevice, h->stream), "H2D");
        CK(cudaMemcpyAsync(h->d_rec_uw, h->geo.rec_uw.data(), nr * 144, cudaMemcpyHostToDevice, h->stream), "H2D");
    }
    CK(cudaStreamSynchronize(h->stream), "geometry upload");
    h->geom_dirty = false;
    return LBM2D_OK;
}

// The paired thermal form (step_pair_kernel<T, true>) measured slower than the
// one-node kernel on heated cavities (2048^2 FP32: 25.7 against 30.2 GLUPS;
// 124 registers a thread): thermal solves pair only on request (variant 2).
bool use_pair(const lbm2d_solver* h) {
    return h->variant != 1 && (h->nx % 2 == 0) && h->storage != ST_FP64 && (!h->thermal || h->variant == 2);
}

// The kernel a step of h runs.  batch: stepped by a batch (or the resident
// serving loop), whose paired kernel walks flat pairs (2k, 2k + 1) of the
// node index, so any width pairs there; a plain step of the same solver runs
// the single-solve kernels.
int kernel_kind(const lbm2d_solver* h, bool batch) {
    const bool tiles_ok = h->storage != ST_FP64;
    if (h->variant == 3 && tiles_ok) return KERNEL_TILES;
    if (h->variant == 0 && tiles_ok) {
        if (rows_eligible(h->storage, h->nx, h->ny, h->thermal) && !(batch && h->resident) &&
            (!batch || (long long)h->N >= kBatchSoloNodes))
            return KERNEL_ROWS;
    }
    // flat pairs: any width (a lattice with an odd node count stores its
    // odd planes' pairs as two single-node stores, and its last node alone)
    const bool flat = batch && !h->thermal && h->storage != ST_FP64 && h->variant != 1;
    if (!use_pair(h) && !flat) return KERNEL_SCALAR;
    return KERNEL_PAIR;
}

int kernel_kind(const lbm2d_solver* h) { return kernel_kind(h, false); }

// Per-warp force slots of the kernel that will run.  Scalar / paired
// kernels: one table entry per launch block (blocks without a force node get
// -1).  Row pipeline: one entry per persistent CTA, marking the CTAs whose
// tiles (tile t goes to CTA t mod grid) hold a force node.
// The node pairs (x even, x + 1) that hold a boundary node (every boundary
// node has a record), first node's index, ascending.
// flat: the pairs (2k, 2k + 1) of the node index instead.
void boundary_pair_list(const lbm2d_solver* h, std::vector<int>& out, bool flat) {
    out.clear();
    out.reserve(h->geo.rec_node.size());
    for (int32_t id : h->geo.rec_node) out.push_back(flat ? (id & ~1) : id - (id % h->nx) % 2);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
}

int ensure_slots(lbm2d_solver* h, bool batch) {
    const int kind = kernel_kind(h, batch);
    // a batch member on the paired kernel: flat pair tiles, and its boundary
    // pairs in boundary blocks appended after them
    const bool bpass = kind == KERNEL_PAIR && batch && !h->thermal;
    int grid = 0;
    const long long ntiles = ((long long)h->N + tiles_width() - 1) / tiles_width();
    if (kind == KERNEL_ROWS) {
        grid = rows_grid(h->storage, h->nx, h->ny, h->device);
        if (grid <= 0) return fail(h, LBM2D_ERR_CUDA, "row pipeline: no launch configuration");
    } else if (kind == KERNEL_TILES) {
        grid = tiles_grid(h->storage, h->thermal, ntiles, h->device);
        if (grid <= 0) return fail(h, LBM2D_ERR_CUDA, "tile pipeline: no launch configuration");
    }
    const bool persistent = kind == KERNEL_ROWS || kind == KERNEL_TILES;
    if (h->slot_kind == kind && h->d_block_slot && h->slot_bpass == bpass &&
        (persistent ? h->slot_grid == grid : (h->slot_bx == h->bx && h->slot_by == h->by)))
        return LBM2D_OK;
    std::vector<int> slots, bpairs;
    int red_blocks = 0, bchunk = 0;
    if (kind == KERNEL_TILES) {
        // one entry per tile of W consecutive nodes: the first of the tile's
        // per-warp slots, -1 for a tile without force nodes; then one entry
        // per CTA of a single-instance launch (CTA c runs the contiguous tiles
        // [c*chunk, (c+1)*chunk), chunk = ceil(T / grid)): 1 when it holds
        // force tiles, the CTAs the fused second stage counts
        const int tw = tiles_width(), warps = tiles_warps();
        const long long chunk = (ntiles + grid - 1) / grid;
        slots.assign((size_t)ntiles + (size_t)grid, -1);
        for (size_t r = 0; r < h->geo.rec_force.size(); ++r)
            if (h->geo.rec_force[r]) slots[(size_t)(h->geo.rec_node[r] / tw)] = 0;
        int k = 0;
        for (size_t t = 0; t < (size_t)ntiles; ++t)
            if (slots[t] == 0) {
                slots[t] = k;
                k += warps;
                slots[(size_t)ntiles + (size_t)((long long)t / chunk)] = 1;
            }
        for (int c = 0; c < grid; ++c) red_blocks += slots[(size_t)ntiles + c] > 0 ? 1 : 0;
        h->nslots = k;
    } else if (kind == KERNEL_ROWS && rows_boundary_pass(h->storage)) {
        // Every boundary node has a record.  The pairs (x even, x + 1) that
        // hold one are rebuilt by a CTA before its tiles, CTA c taking the
        // contiguous chunk [c*bchunk, (c+1)*bchunk) of the ascending list;
        // force nodes are boundary nodes, so a CTA holds force slots when
        // its chunk has a pair with a force record.
        const int warps = rows_warps_per_block();
        boundary_pair_list(h, bpairs, false);
        bchunk = bpairs.empty() ? 0 : (int)((bpairs.size() + (size_t)grid - 1) / (size_t)grid);
        slots.assign((size_t)grid, -1);
        for (size_t r = 0; r < h->geo.rec_force.size(); ++r) {
            if (!h->geo.rec_force[r]) continue;
            const int id = h->geo.rec_node[r];
            const size_t i = (size_t)(std::lower_bound(bpairs.begin(), bpairs.end(), id - (id % h->nx) % 2) -
                                      bpairs.begin());
            slots[i / (size_t)bchunk] = 0;
        }
        int k = 0;
        for (auto& s : slots)
            if (s == 0) {
                s = k;
                k += warps;
            }
        h->nslots = k;
    } else if (kind == KERNEL_ROWS) {
        // boundary pairs inline: tile t (row-major over tpr tiles per row)
        // runs on CTA t mod grid
        const int tw = rows_tile_width(), tpr = (h->nx + tw - 1) / tw, warps = rows_warps_per_block();
        slots.assign((size_t)grid, -1);
        for (size_t r = 0; r < h->geo.rec_force.size(); ++r) {
            if (!h->geo.rec_force[r]) continue;
            const int id = h->geo.rec_node[r];
            const long long t = (long long)(id / h->nx) * tpr + (id % h->nx) / tw;
            slots[(size_t)(t % grid)] = 0;
        }
        int k = 0;
        for (auto& s : slots)
            if (s == 0) {
                s = k;
                k += warps;
            }
        h->nslots = k;
    } else if (bpass) {
        // ntiles flat tiles of B = bx*by pairs own no slots; boundary block
        // i (pairs [i*B, (i+1)*B), one per thread) owns one per warp when it
        // holds a force pair, at block_slot[ntiles + i]
        const int B = h->bx * h->by, warps = (B + 31) / 32;
        boundary_pair_list(h, bpairs, true);
        bchunk = B;
        const size_t ntl = (size_t)flat_tiles(h), nbb = (bpairs.size() + (size_t)B - 1) / (size_t)B;
        slots.assign(ntl + nbb, -1);
        for (size_t r = 0; r < h->geo.rec_force.size(); ++r) {
            if (!h->geo.rec_force[r]) continue;
            const int id = h->geo.rec_node[r];
            const size_t i = (size_t)(std::lower_bound(bpairs.begin(), bpairs.end(), id & ~1) - bpairs.begin());
            slots[ntl + i / (size_t)B] = 0;
        }
        int k = 0;
        for (auto& s : slots)
            if (s == 0) {
                s = k;
                k += warps;
            }
        h->nslots = k;
    } else {
        h->nslots = force_block_slots(h->geo, h->nx, h->ny, h->bx * (kind == KERNEL_PAIR ? 2 : 1), h->by,
                                      h->bx * h->by, slots);  // per-warp slots
    }
    dfree(h, &h->d_block_slot);
    dfree(h, &h->d_partials);
    dfree(h, &h->d_bpairs);
    h->nbpairs = h->bchunk = 0;
    int rc;
    if (!bpairs.empty()) {
        if ((rc = dalloc(h, &h->d_bpairs, bpairs.size() * sizeof(int)))) return rc;
        CK(cudaMemcpyAsync(h->d_bpairs, bpairs.data(), bpairs.size() * sizeof(int), cudaMemcpyHostToDevice,
                           h->stream),
           "boundary pairs H2D");
        h->nbpairs = (int)bpairs.size();
        h->bchunk = bchunk;
    }
    if ((rc = dalloc(h, &h->d_block_slot, slots.size() * sizeof(int)))) return rc;
    if ((rc = dalloc(h, &h->d_partials, (size_t)std::max(h->nslots, 1) * 2 * sizeof(double)))) return rc;
    CK(cudaMemcpyAsync(h->d_block_slot, slots.data(), slots.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream),
       "slots H2D");
    // arrival count of the fused second stage (blocks holding slots)
    h->red_blocks = red_blocks;
    if (kind != KERNEL_TILES)
        for (int s : slots)
            if (s >= 0) ++h->red_blocks;
    if (!h->d_red_done) {
        if ((rc = dalloc(h, &h->d_red_done, sizeof(unsigned int)))) return rc;
        CK(cudaMemsetAsync(h->d_red_done, 0, sizeof(unsigned int), h->stream), "reduction count");
    }
    CK(cudaStreamSynchronize(h->stream), "slots");
    h->slot_bx = h->bx;
    h->slot_by = h->by;
    h->slot_kind = kind;
    h->slot_grid = grid;
    h->slot_bpass = bpass;
    return LBM2D_OK;
}

// Parameters of a kernel that rebuilds the reference state S_n of the last
// step: S_n is pulled from the post-collision populations of the step BEFORE
// it (the other ping-pong buffer), with the boundary velocity of step n.
KParams rebuild_params(const lbm2d_solver* h) {
    KParams p = base_params(h);
    p.fin = h->P[h->cur ^ 1];
    p.gin = h->G[h->cur ^ 1];
    set_u_bc(p, h->u_last);
    ibm_state_params(h, p);
    return p;
}

// COLLIDED -> STAGED: rebuild the reference state S from the stored populations.
int materialize(lbm2d_solver* h) {
    if (h->staged) return LBM2D_OK;
    int rc;
    if ((rc = ensure_stage(h, h->thermal))) return rc;
    if (h->steps_since_collide > 0) {
        KParams p = rebuild_params(h);
        ROut o;
        std::memset(&o, 0, sizeof(o));
        o.f_aos = h->d_stage_f;
        o.g_aos = h->thermal ? h->d_stage_g : nullptr;
        int e = launch_readback(h->storage, p, o, h->stream);
        ++h->launches;
        if (e) return cuda_fail(h, (cudaError_t)e, "readback");
    }  // else: no step since the prologue, staging still holds S
    h->staged = true;
    h->stage_f_valid = true;
    if (h->thermal) h->stage_g_valid = true;
    return LBM2D_OK;
}

// Any change of geometry / case / thermal switch while COLLIDED must first
// rebuild S with the settings that produced the stored populations.
int before_setting_change(lbm2d_solver* h) {
    if (h->staged) return LBM2D_OK;
    if (h->geom_dirty) {
        // geometry already changed under a collided state cannot happen: every
        // setter calls this function first.
        return fail(h, LBM2D_ERR_STATE, "internal: dirty geometry under collided state");
    }
    return materialize(h);
}

int prologue(lbm2d_solver* h, const CollideParams& c) {
    int rc;
    if ((rc = ensure_populations(h))) return rc;
    if ((rc = ensure_stage(h, h->thermal))) return rc;
    KParams p = base_params(h);
    apply_collide(p, c);
    p.fout = h->P[h->cur];
    p.gout = h->G[h->cur];
    // rounding-noise seed of the prologue; the steps after it continue from
    // seed_host + 1 (written to the seed word of the current buffer)
    p.seed_host = (uint32_t)h->steps_done ^ 0xA511E9B3u;
    p.seed_out = h->d_seed + h->cur;
    int e = launch_prologue(h->storage, p, h->d_stage_f, h->thermal ? h->d_stage_g : nullptr, h->stream);
    ++h->launches;
    if (e) return cuda_fail(h, (cudaError_t)e, "prologue");
    // immersed boundary: the force of the first step comes from the staged state
    if ((rc = ibm_from_stage(h, p))) return rc;
    h->staged = false;
    h->cp_of_P = c;
    h->steps_since_collide = 0;
    return LBM2D_OK;
}

int check_handle(lbm2d_solver* h) {
    if (!h) return LBM2D_ERR_INVALID;
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
    return LBM2D_OK;
}

// Prepare a handle for steps with (tau, u): re-collide on parameter change,
// push geometry, force slots and the prologue, then fill the kernel
// parameters of the next step.
int prepare_steps(lbm2d_solver* h, double tau, double u_inflow, KParams& p, bool batch) {
    int rc;
    if (!(tau > 0.0)) return fail(h, LBM2D_ERR_INVALID, "tau must be positive");
    const CollideParams c = collide_params(h, tau);
    if (!h->staged && !(c == h->cp_of_P)) {
        if ((rc = materialize(h))) return rc;
    }
    if ((rc = upload_geometry(h))) return rc;
    if ((rc = ensure_slots(h, batch))) return rc;
    // set-up of the allocation-free entry point on this device (once); a
    // failure here is reported by that entry point, not by this step
    noalloc_bind_device(h->device);
    if (h->staged) {
        if ((rc = prologue(h, c))) return rc;
    }
    p = base_params(h);
    apply_collide(p, c);
    set_u_bc(p, u_inflow);
    p.block_slot = h->nslots > 0 ? h->d_block_slot : nullptr;
    p.partials = h->d_partials;
    p.fin = h->P[h->cur];
    p.fout = h->P[h->cur ^ 1];
    p.gin = h->G[h->cur];
    p.gout = h->G[h->cur ^ 1];
    p.seed_in = h->d_seed + h->cur;
    p.seed_out = h->d_seed + (h->cur ^ 1);
    p.skip_settled_solids = (h->steps_since_collide >= 2 && h->hook != 1) ? 1 : 0;
    return LBM2D_OK;
}

}  // namespace rt
}  // namespace lbm2d

using namespace lbm2d::rt;

extern "C" {

const char* lbm2d_last_error(const lbm2d_solver* h) { return h ? h->err.c_str() : g_global_err.c_str(); }
const char* lbm2d_global_error(void) { return g_global_err.c_str(); }

int lbm2d_create(const lbm2d_config* cfg, lbm2d_solver** out) {
    if (!cfg || !out) {
        g_global_err = "null argument";
        return LBM2D_ERR_INVALID;
    }
    *out = nullptr;
    if (cfg->nx < 3 || cfg->ny < 3 || (long long)cfg->nx * cfg->ny >= (1LL << 32)) {
        g_global_err = "grid must be at least 3x3 and hold fewer than 2^32 nodes";
        return LBM2D_ERR_INVALID;
    }
    if (cfg->storage < 0 || cfg->storage > 3 || cfg->collision < 0 || cfg->collision > 1 || cfg->case_type < 0 ||
        cfg->case_type > 13) {
        g_global_err = "invalid storage, collision or case";
        return LBM2D_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        g_global_err = "no CUDA device";
        return LBM2D_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) {
        g_global_err = "device ordinal out of range";
        return LBM2D_ERR_INVALID;
    }
    auto* h = new (std::nothrow) lbm2d_solver();
    if (!h) {
        g_global_err = "host allocation failed";
        return LBM2D_ERR_OOM;
    }
    h->device = cfg->device;
    h->nx = cfg->nx;
    h->ny = cfg->ny;
    h->N = (size_t)cfg->nx * cfg->ny;
    h->case_type = cfg->case_type;
    h->collision = cfg->collision;
    h->use_les = cfg->use_les;
    h->cs = cfg->cs;
    h->storage = cfg->storage;
    h->mask.assign(h->N, 0);
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        // keep freed solver memory in the device's pool for the next solver
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, h->device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    int rc = LBM2D_OK;
    if (e != cudaSuccess) {
        g_global_err = std::string("stream: ") + cudaGetErrorString(e);
        delete h;
        return LBM2D_ERR_CUDA;
    }
    if (!rc) rc = dalloc(h, &h->d_nan, 16);
    if (!rc) rc = dalloc(h, &h->d_seed, 16);
    if (!rc) rc = dalloc(h, &h->d_counter, 16);
    // The last step's drag/lift lives in mapped pinned memory: the kernel that
    // records it writes straight to the host, so a read needs no copy.
    if (!rc && pinned_pair_get(&h->h_last, &h->d_last)) rc = fail(h, LBM2D_ERR_CUDA, "mapped force buffer");
    if (!rc) h->h_last[0] = h->h_last[1] = 0.0;
    if (!rc) rc = dalloc(h, &h->d_hist, (size_t)h->hist_cap * 2 * sizeof(double));
    if (!rc) rc = ensure_stage(h, false);
    if (!rc) rc = ensure_populations(h);
    if (!rc) {
        cudaMemsetAsync(h->d_nan, 0, 16, h->stream);
        cudaMemsetAsync(h->d_seed, 0, 16, h->stream);
        cudaMemsetAsync(h->d_counter, 0, 16, h->stream);
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) rc = LBM2D_ERR_CUDA;
    }
    if (rc) {
        g_global_err = h->err;
        lbm2d_destroy(h);
        return rc;
    }
    *out = h;
    return LBM2D_OK;
}

int lbm2d_destroy(lbm2d_solver* h) {
    if (!h) return LBM2D_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->pair_graph) cudaGraphExecDestroy(h->pair_graph);
    ibm_release(h);
    void* bufs[] = {h->P[0], h->P[1], h->G[0], h->G[1], h->d_flags, h->d_rec_info, h->d_rec_force,
                    h->d_rec_wd, h->d_rec_q, h->d_rec_uw, h->d_partials, h->d_block_slot, h->d_bpairs, h->d_hist,
                    h->d_counter, h->d_nan, h->d_seed, h->d_stage_f, h->d_stage_g, h->d_fx, h->d_fy,
                    h->d_diag, h->d_prev_uv, h->d_red_done};
    for (void* b : bufs)
        if (b) cudaFreeAsync(b, h->stream);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (cudaEvent_t ev : h->ev_pool) cudaEventDestroy(ev);
    if (h->h_last) pinned_pair_put(h->h_last);  // d_last is its device alias
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LBM2D_OK;
}

int lbm2d_set_case(lbm2d_solver* h, int case_type, int collision, int use_les, double cs) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (case_type < 0 || case_type > 13 || collision < 0 || collision > 1)
        return fail(h, LBM2D_ERR_INVALID, "invalid case or collision");
    if (case_type == h->case_type && collision == h->collision && use_les == h->use_les && cs == h->cs)
        return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->case_type = case_type;
    h->collision = collision;
    h->use_les = use_les;
    h->cs = cs;
    h->geom_dirty = true;
    return LBM2D_OK;
}

int lbm2d_set_mask(lbm2d_solver* h, const uint8_t* obstacle) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!obstacle) return fail(h, LBM2D_ERR_INVALID, "null mask");
    bool same = true;
    for (size_t k = 0; k < h->N && same; ++k) same = (obstacle[k] != 0) == (h->mask[k] != 0);
    if (same && !h->geom_dirty) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    for (size_t k = 0; k < h->N; ++k) h->mask[k] = obstacle[k] ? 1 : 0;
    h->geom_dirty = true;
    return LBM2D_OK;
}

int lbm2d_set_bb_cylinder(lbm2d_solver* h, double cx, double cy, double radius) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (h->bb.cx == cx && h->bb.cy == cy && h->bb.radius == radius) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->bb.cx = cx;
    h->bb.cy = cy;
    h->bb.radius = radius;
    h->geom_dirty = true;
    return LBM2D_OK;
}

int lbm2d_set_bb_polygon(lbm2d_solver* h, const double* xy, int n) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (n < 0 || (n > 0 && !xy)) return fail(h, LBM2D_ERR_INVALID, "bad polygon");
    std::vector<double> poly(xy, xy + 2 * (size_t)n);
    if (h->bb.is_polygon == (n > 0) && h->bb.poly == poly) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->bb.poly = poly;
    h->bb.is_polygon = n > 0;
    h->geom_dirty = true;
    return LBM2D_OK;
}

int lbm2d_set_moving_wall(lbm2d_solver* h, int on, double omega, double rcx, double rcy) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (h->bb.has_moving_wall == (on != 0) && h->bb.omega == omega && h->bb.rot_cx == rcx && h->bb.rot_cy == rcy)
        return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->bb.has_moving_wall = on != 0;
    h->bb.omega = omega;
    h->bb.rot_cx = rcx;
    h->bb.rot_cy = rcy;
    h->geom_dirty = true;
    return LBM2D_OK;
}

int lbm2d_set_mei(lbm2d_solver* h, int on) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (h->bb.use_mei == (on != 0)) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->bb.use_mei = on != 0;
    return LBM2D_OK;
}

int lbm2d_set_body_force(lbm2d_solver* h, double fx) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    h->body_force = fx;  // takes effect through the collision parameters of the next step
    return LBM2D_OK;
}

int lbm2d_set_thermal(lbm2d_solver* h, int use, double T_ref, double alpha, double omega_k, double beta,
                      double g_buoyancy) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    const bool on = use != 0;
    if (on && ibm_active(h))
        return fail(h, LBM2D_ERR_INVALID, "the thermal DDF is not available with an immersed boundary");
    if (on != h->thermal || (on && T_ref != h->T_ref)) {
        if ((rc = before_setting_change(h))) return rc;
        if (on && (rc = ensure_stage(h, true))) return rc;
        h->geom_dirty = true;
    }
    h->thermal = on;
    h->T_ref = T_ref;
    h->alpha = alpha;
    h->omega_k = omega_k;
    h->beta = beta;
    h->g_buoy = g_buoyancy;
    if (on && (rc = ensure_populations(h))) return rc;
    return LBM2D_OK;
}

int lbm2d_set_thermal_hook(lbm2d_solver* h, int kind, double Ta, double Tb) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (kind < 0 || kind > 2) return fail(h, LBM2D_ERR_INVALID, "unknown thermal hook");
    if (kind == h->hook && Ta == h->hook_a && Tb == h->hook_b) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;
    h->hook = kind;
    h->hook_a = Ta;
    h->hook_b = Tb;
    return LBM2D_OK;
}

static int upload_common(lbm2d_solver* h, const double* src, bool is_g, cudaMemcpyKind kind) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!src) return fail(h, LBM2D_ERR_INVALID, "null populations");
    // the upload replaces one population set; the other one (g for an f
    // upload of a thermal solver, f for a g upload) is rebuilt first when the
    // stored populations are the newer state -- a non-thermal f upload
    // replaces everything and rebuilds nothing
    if (!h->staged && (h->thermal || is_g)) {
        if ((rc = materialize(h))) return rc;
    } else {
        h->staged = true;
    }
    if ((rc = ensure_stage(h, h->thermal || is_g))) return rc;
    double* dst = is_g ? h->d_stage_g : h->d_stage_f;
    CK(cudaMemcpyAsync(dst, src, h->N * 9 * sizeof(double), kind, h->stream), "upload");
    if (kind == cudaMemcpyHostToDevice) CK(cudaStreamSynchronize(h->stream), "upload");
    (is_g ? h->stage_g_valid : h->stage_f_valid) = true;
    h->staged = true;
    CK(cudaMemsetAsync(h->d_counter, 0, 8, h->stream), "reset history");
    h->steps_done = 0;
    return LBM2D_OK;
}

int lbm2d_upload_f(lbm2d_solver* h, const double* f) { return upload_common(h, f, false, cudaMemcpyHostToDevice); }
int lbm2d_upload_g(lbm2d_solver* h, const double* g) { return upload_common(h, g, true, cudaMemcpyHostToDevice); }
int lbm2d_upload_f_device(lbm2d_solver* h, const double* d_f) {
    return upload_common(h, d_f, false, cudaMemcpyDeviceToDevice);
}

int lbm2d_init_equilibrium(lbm2d_solver* h, double rho, double u, double v, double T) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if ((rc = materialize(h))) return rc;
    if ((rc = ensure_stage(h, true))) return rc;
    const int e = launch_fill_equilibrium(h->d_stage_f, h->d_stage_g, (long long)h->N, rho, u, v, T, h->stream);
    ++h->launches;
    if (e) return cuda_fail(h, (cudaError_t)e, "fill equilibrium");
    h->staged = true;
    h->stage_f_valid = h->stage_g_valid = true;
    CK(cudaMemsetAsync(h->d_counter, 0, 8, h->stream), "reset history");
    h->steps_done = 0;
    return LBM2D_OK;
}

}  // extern "C"

namespace lbm2d {
namespace rt {

// Launch one step from buffer h->cur (step kernel, force reduction,
// immersed-boundary forcing); host state is not advanced.  The per-warp
// force partials go to p.partials (the handle's buffer, or the fixed scratch
// of the allocation-free entry point).  With profiling events, e0 / e1
// bracket the step kernel alone.
int launch_one_step(lbm2d_solver* h, KParams& p, cudaEvent_t e0, cudaEvent_t e1) {
    p.fin = h->P[h->cur];
    p.fout = h->P[h->cur ^ 1];
    p.gin = h->G[h->cur];
    p.gout = h->G[h->cur ^ 1];
    p.seed_in = h->d_seed + h->cur;
    p.seed_out = h->d_seed + (h->cur ^ 1);
    p.skip_settled_solids = (h->steps_since_collide >= 2 && h->hook != 1) ? 1 : 0;
    // the drag/lift second stage runs in the step launch's last force block
    // when every block has the 128 threads it needs (the row pipeline has 256
    // consumers); otherwise in its own launch
    const bool fused = h->nslots > 0 && h->red_blocks > 0 &&
                       (h->slot_kind == KERNEL_ROWS || h->slot_kind == KERNEL_TILES || h->bx * h->by >= 128);
    p.red_done = fused ? h->d_red_done : nullptr;
    p.red_hist = h->d_hist;
    p.red_counter = h->d_counter;
    p.red_last = h->d_last;
    p.red_blocks = h->red_blocks;
    p.red_nslots = h->nslots;
    p.red_cap = h->hist_cap;
    if (e0) CK(cudaEventRecord(e0, h->stream), "event");
    int e = h->slot_kind == KERNEL_ROWS    ? launch_rows(h->storage, p, h->slot_grid, h->stream)
            : h->slot_kind == KERNEL_TILES ? launch_tiles_single(h->storage, p, h->slot_grid, h->stream)
                                           : launch_step(h->storage, p, h->bx, h->by, h->stream);
    if (e1) CK(cudaEventRecord(e1, h->stream), "event");
    ++h->launches;
    if (e) return cuda_fail(h, (cudaError_t)e, "step kernel");
    if (h->nslots > 0 && !fused) {
        e = launch_force_reduce(p.partials, h->nslots, h->d_hist, h->hist_cap, h->d_counter, h->d_last, h->stream);
        ++h->launches;
        if (e) return cuda_fail(h, (cudaError_t)e, "force reduce");
    }
    return ibm_after_step(h, p);
}

void advance(lbm2d_solver* h, long long n) {
    if (n & 1) {
        h->cur ^= 1;
        if (ibm_active(h)) h->ibm_next ^= 1;
    }
    h->steps_since_collide += n;
    h->steps_done += n;
}

namespace {

// Everything a captured step pair depends on: the parameters of its first
// step, the launch shape and the buffers passed outside the parameters.
std::vector<unsigned char> pair_key(lbm2d_solver* h, const KParams& p0) {
    KParams p = p0;
    p.fin = h->P[h->cur];
    p.fout = h->P[h->cur ^ 1];
    p.gin = h->G[h->cur];
    p.gout = h->G[h->cur ^ 1];
    p.seed_in = h->d_seed + h->cur;
    p.seed_out = h->d_seed + (h->cur ^ 1);
    p.skip_settled_solids = (h->hook != 1) ? 1 : 0;
    const long long extra[] = {h->slot_kind, h->slot_grid, h->bx, h->by, h->storage, h->cur, h->ibm_next,
                               h->nslots, h->hist_cap, h->ibm_np, h->ibm_nb,
                               (long long)(uintptr_t)h->d_hist, (long long)(uintptr_t)h->d_counter,
                               (long long)(uintptr_t)h->d_last, (long long)(uintptr_t)h->d_ibm_buf,
                               (long long)(uintptr_t)h->d_ibm_band, (long long)(uintptr_t)h->d_ibm_tab};
    std::vector<unsigned char> k(sizeof(p) + sizeof(extra) + sizeof(IbmParams));
    std::memcpy(k.data(), &p, sizeof(p));
    std::memcpy(k.data() + sizeof(p), extra, sizeof(extra));
    std::memcpy(k.data() + sizeof(p) + sizeof(extra), &h->ibm_q, sizeof(IbmParams));  // table offsets, dt, u_wall
    return k;
}

// Capture two consecutive steps from the current buffers into a graph.
int capture_pair(lbm2d_solver* h, const KParams& p0, std::vector<unsigned char>&& key) {
    if (h->pair_graph) cudaGraphExecDestroy(h->pair_graph);
    h->pair_graph = nullptr;
    h->pair_key.clear();
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const long long l0 = h->launches;
    const int cur0 = h->cur, next0 = h->ibm_next;
    const long long ssc = h->steps_since_collide, sd = h->steps_done;
    KParams p = p0;
    int rc = launch_one_step(h, p);
    if (!rc) {
        advance(h, 1);
        rc = launch_one_step(h, p);
    }
    h->cur = cur0;
    h->ibm_next = next0;
    h->steps_since_collide = ssc;
    h->steps_done = sd;
    const long long per_pair = h->launches - l0;
    h->launches = l0;  // counted when replayed
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "end capture");
    const cudaError_t ei = cudaGraphInstantiate(&h->pair_graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return cuda_fail(h, ei, "instantiate");
    h->pair_key = std::move(key);
    h->pair_launches = per_pair;
    return LBM2D_OK;
}

}  // namespace
}  // namespace rt
}  // namespace lbm2d

extern "C" {

// Steps run one launch sequence each until the per-step parameters are
// stable (two steps after the last collision), then whole step pairs replay
// a captured CUDA graph: one graph launch instead of 2-10 kernel launches per
// pair, which is what bounds small grids.  The graph is kept while the
// parameters, the launch shape and the buffers stay the same.
int lbm2d_step(lbm2d_solver* h, double tau, double u_inflow, int nsteps) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (nsteps < 0) return fail(h, LBM2D_ERR_INVALID, "negative step count");
    if (nsteps == 0) return LBM2D_OK;
    KParams p;
    if ((rc = prepare_steps(h, tau, u_inflow, p))) return rc;
    int k = 0;
    while (k < nsteps) {
        const int left = nsteps - k;
        if (!h->profiling && left >= 2 && h->steps_since_collide >= 2) {
            std::vector<unsigned char> key = pair_key(h, p);
            const bool have = h->pair_graph && key == h->pair_key;
            if (!have && k >= 2 && left >= 4) {
                if ((rc = capture_pair(h, p, std::move(key)))) return rc;
            }
            if (h->pair_graph && (have || k >= 2) && pair_key(h, p) == h->pair_key) {
                const int pairs = left / 2;
                for (int i = 0; i < pairs; ++i) CK(cudaGraphLaunch(h->pair_graph, h->stream), "graph launch");
                h->launches += h->pair_launches * pairs;
                advance(h, 2LL * pairs);
                k += 2 * pairs;
                continue;
            }
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (h->profiling) {
            if (h->ev_used + 2 > h->ev_pool.size()) {
                for (int k2 = 0; k2 < 64; ++k2) {
                    cudaEvent_t ev;
                    CK(cudaEventCreate(&ev), "event");
                    h->ev_pool.push_back(ev);
                }
            }
            e0 = h->ev_pool[h->ev_used++];
            e1 = h->ev_pool[h->ev_used++];
        }
        if ((rc = launch_one_step(h, p, e0, e1))) return rc;
        advance(h, 1);
        ++k;
    }
    h->u_last = u_inflow;
    return LBM2D_OK;
}

int lbm2d_synchronize(lbm2d_solver* h) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    CK(cudaStreamSynchronize(h->stream), "synchronize");
    unsigned int flag = 0;
    CK(cudaMemcpy(&flag, h->d_nan, sizeof(flag), cudaMemcpyDeviceToHost), "nan flag");
    if (flag) {
        cudaMemset(h->d_nan, 0, sizeof(flag));
        if (flag & 2u) return fail(h, LBM2D_ERR_TIMEOUT, "a step kernel's pipeline wait exceeded its limit");
        return fail(h, LBM2D_ERR_NAN, "a non-finite or zero density was produced");
    }
    return LBM2D_OK;
}

int lbm2d_force_sums(lbm2d_solver* h, double* fx, double* fy) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    // the recording kernel wrote the sums into mapped host memory: once the
    // stream has drained they are here, with no copy
    CK(cudaStreamSynchronize(h->stream), "force sync");
    if (fx) *fx = h->h_last[0];
    if (fy) *fy = h->h_last[1];
    return LBM2D_OK;
}

int lbm2d_force_history(lbm2d_solver* h, double* fx, double* fy, int n, int* n_recorded) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, h->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream), "counter");
    CK(cudaStreamSynchronize(h->stream), "sync");
    const long long rec = std::min<long long>((long long)cnt, h->hist_cap);
    if (n_recorded) *n_recorded = (int)cnt;
    const long long m = std::min<long long>(rec, n);
    if (m > 0) {
        std::vector<double> buf((size_t)m * 2);
        CK(cudaMemcpy(buf.data(), h->d_hist, buf.size() * sizeof(double), cudaMemcpyDeviceToHost), "hist");
        for (long long k = 0; k < m; ++k) {
            if (fx) fx[k] = buf[2 * k];
            if (fy) fy[k] = buf[2 * k + 1];
        }
    }
    return LBM2D_OK;
}

int lbm2d_force_history_reset(lbm2d_solver* h) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    CK(cudaMemsetAsync(h->d_counter, 0, 8, h->stream), "reset");
    return LBM2D_OK;
}

int lbm2d_download_f(lbm2d_solver* h, double* f) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!f) return fail(h, LBM2D_ERR_INVALID, "null output");
    if ((rc = ensure_stage(h, h->thermal))) return rc;
    if (!h->staged) {
        // rebuild S into staging, keep the collided populations as the live state
        if ((rc = materialize(h))) return rc;
        h->staged = false;
    }
    CK(cudaMemcpyAsync(f, h->d_stage_f, h->N * 9 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H f");
    CK(cudaStreamSynchronize(h->stream), "D2H f");
    return LBM2D_OK;
}

int lbm2d_download_f_device(lbm2d_solver* h, double* d_f) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!d_f) return fail(h, LBM2D_ERR_INVALID, "null output");
    if ((rc = ensure_stage(h, h->thermal))) return rc;
    if (!h->staged) {
        if ((rc = materialize(h))) return rc;
        h->staged = false;
    }
    CK(cudaMemcpyAsync(d_f, h->d_stage_f, h->N * 9 * sizeof(double), cudaMemcpyDeviceToDevice, h->stream), "D2D");
    return LBM2D_OK;
}

int lbm2d_download_g(lbm2d_solver* h, double* g) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!g) return fail(h, LBM2D_ERR_INVALID, "null output");
    if ((rc = ensure_stage(h, true))) return rc;
    if (!h->staged && h->thermal) {
        if ((rc = materialize(h))) return rc;
        h->staged = false;
    }
    CK(cudaMemcpyAsync(g, h->d_stage_g, h->N * 9 * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H g");
    CK(cudaStreamSynchronize(h->stream), "D2H g");
    return LBM2D_OK;
}

int lbm2d_download_force_field(lbm2d_solver* h, double* fx, double* fy) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!fx || !fy) return fail(h, LBM2D_ERR_INVALID, "null output");
    if (h->staged || h->steps_since_collide == 0) {
        // no step since the upload: the reference's fields are still the zeros
        // of LBMCapabilities::reset_forces (or the previous step's values,
        // which this handle does not keep across uploads)
        std::fill(fx, fx + h->N, 0.0);
        std::fill(fy, fy + h->N, 0.0);
        return LBM2D_OK;
    }
    if ((rc = dalloc(h, &h->d_fx, h->N * sizeof(double)))) return rc;
    if ((rc = dalloc(h, &h->d_fy, h->N * sizeof(double)))) return rc;
    KParams p = rebuild_params(h);
    ROut o;
    std::memset(&o, 0, sizeof(o));
    o.fx = h->d_fx;
    o.fy = h->d_fy;
    int e = launch_readback(h->storage, p, o, h->stream);
    ++h->launches;
    if (e) return cuda_fail(h, (cudaError_t)e, "force field");
    CK(cudaMemcpyAsync(fx, h->d_fx, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H fx");
    CK(cudaMemcpyAsync(fy, h->d_fy, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "D2H fy");
    CK(cudaStreamSynchronize(h->stream), "D2H force");
    return LBM2D_OK;
}

int lbm2d_download_macros(lbm2d_solver* h, double* rho, double* u, double* v, double* T) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (h->staged || h->steps_since_collide == 0) return fail(h, LBM2D_ERR_STATE, "no step since the last upload");
    double* bufs[4] = {nullptr, nullptr, nullptr, nullptr};
    double* outs[4] = {rho, u, v, (h->thermal ? T : nullptr)};
    for (int k = 0; k < 4; ++k) {
        if (!outs[k]) continue;
        if (cudaMallocAsync(&bufs[k], h->N * sizeof(double), h->stream) != cudaSuccess) {
            for (int j = 0; j < k; ++j)
                if (bufs[j]) cudaFreeAsync(bufs[j], h->stream);
            return fail(h, LBM2D_ERR_OOM, "macros buffer");
        }
    }
    KParams p = rebuild_params(h);
    ROut o;
    std::memset(&o, 0, sizeof(o));
    o.rho = bufs[0];
    o.u = bufs[1];
    o.v = bufs[2];
    o.T = bufs[3];
    int e = launch_readback(h->storage, p, o, h->stream);
    ++h->launches;
    int ret = LBM2D_OK;
    if (e) ret = cuda_fail(h, (cudaError_t)e, "macros");
    for (int k = 0; k < 4 && !ret; ++k)
        if (bufs[k]) {
            cudaError_t ce = cudaMemcpyAsync(outs[k], bufs[k], h->N * sizeof(double), cudaMemcpyDeviceToHost,
                                             h->stream);
            if (ce != cudaSuccess) ret = cuda_fail(h, ce, "D2H macros");
        }
    for (int k = 0; k < 4; ++k)
        if (bufs[k]) cudaFreeAsync(bufs[k], h->stream);
    cudaStreamSynchronize(h->stream);
    return ret;
}

int lbm2d_frame_fields(lbm2d_solver* h, int ds, int sanitize, double T_wall, double* rho, double* u, double* v,
                       double* vel, double* omega, double* T, uint8_t* obstacle) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (ds < 1) return fail(h, LBM2D_ERR_INVALID, "frame downsampling factor must be >= 1");
    if (h->staged || h->steps_since_collide == 0) return fail(h, LBM2D_ERR_STATE, "no step since the last upload");
    const int nxd = (h->nx + ds - 1) / ds, nyd = (h->ny + ds - 1) / ds;
    const size_t nd = (size_t)nxd * nyd;
    // one scratch block: six FP64 fields, then the obstacle bytes
    char* buf = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&buf), nd * (6 * sizeof(double) + 1), h->stream) != cudaSuccess)
        return fail(h, LBM2D_ERR_OOM, "frame buffer");
    double* d = reinterpret_cast<double*>(buf);
    FOut o;
    o.rho = d;
    o.u = d + nd;
    o.v = d + 2 * nd;
    o.vel = d + 3 * nd;
    o.omega = d + 4 * nd;
    o.T = d + 5 * nd;
    o.obstacle = reinterpret_cast<uint8_t*>(d + 6 * nd);
    o.T_wall = T_wall;
    o.ds = ds;
    o.nxd = nxd;
    o.nyd = nyd;
    o.sanitize = sanitize ? 1 : 0;
    KParams p = rebuild_params(h);
    const int e = launch_frame(h->storage, p, o, h->stream);
    h->launches += 2;
    int ret = e ? cuda_fail(h, (cudaError_t)e, "frame fields") : LBM2D_OK;
    const double* srcs[6] = {o.rho, o.u, o.v, o.vel, o.omega, o.T};
    double* outs[6] = {rho, u, v, vel, omega, T};
    for (int k = 0; k < 6 && !ret; ++k)
        if (outs[k]) {
            const cudaError_t ce =
                cudaMemcpyAsync(outs[k], srcs[k], nd * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
            if (ce != cudaSuccess) ret = cuda_fail(h, ce, "D2H frame");
        }
    if (!ret && obstacle) {
        const cudaError_t ce = cudaMemcpyAsync(obstacle, o.obstacle, nd, cudaMemcpyDeviceToHost, h->stream);
        if (ce != cudaSuccess) ret = cuda_fail(h, ce, "D2H frame obstacle");
    }
    cudaFreeAsync(buf, h->stream);
    const cudaError_t se = cudaStreamSynchronize(h->stream);
    if (!ret && se != cudaSuccess) ret = cuda_fail(h, se, "frame fields");
    return ret;
}

int lbm2d_diagnostics(lbm2d_solver* h, double* mass, double* mom_x, double* mom_y, double* residual) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (h->staged || h->steps_since_collide == 0) return fail(h, LBM2D_ERR_STATE, "no step since the last upload");
    if ((rc = dalloc(h, &h->d_diag, 5 * sizeof(double)))) return rc;
    if ((rc = dalloc(h, &h->d_prev_uv, h->N * 2 * sizeof(float)))) return rc;
    CK(cudaMemsetAsync(h->d_diag, 0, 5 * sizeof(double), h->stream), "diag reset");
    KParams p = rebuild_params(h);
    const int e = launch_diagnostics(h->storage, p, h->d_diag, h->d_prev_uv, h->have_prev_uv ? 1 : 0, h->stream);
    ++h->launches;
    if (e) return cuda_fail(h, (cudaError_t)e, "diagnostics");
    double acc[5];
    CK(cudaMemcpyAsync(acc, h->d_diag, sizeof(acc), cudaMemcpyDeviceToHost, h->stream), "diag D2H");
    CK(cudaStreamSynchronize(h->stream), "diag sync");
    if (mass) *mass = acc[0];
    if (mom_x) *mom_x = acc[1];
    if (mom_y) *mom_y = acc[2];
    if (residual) *residual = h->have_prev_uv && acc[4] > 0.0 ? std::sqrt(acc[3] / acc[4]) : NAN;
    h->have_prev_uv = true;
    return LBM2D_OK;
}

int lbm2d_download_wall_dist(lbm2d_solver* h, double* wd) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!wd) return fail(h, LBM2D_ERR_INVALID, "null output");
    std::vector<double> d;
    wall_distance(h->nx, h->ny, h->mask.data(), d);
    std::copy(d.begin(), d.end(), wd);
    return LBM2D_OK;
}

int lbm2d_get_info(lbm2d_solver* h, lbm2d_info* info) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (!info) return fail(h, LBM2D_ERR_INVALID, "null output");
    if ((rc = upload_geometry(h))) return rc;
    info->nx = h->nx;
    info->ny = h->ny;
    info->storage = h->storage;
    info->bytes_per_update = 2.0 * 9.0 * (double)elem_size(h->storage) * (h->thermal ? 2.0 : 1.0);
    info->device_bytes = h->device_bytes;
    info->n_boundary_nodes = (int)h->geo.rec_info.size();
    info->n_force_nodes = h->geo.n_force_nodes;
    info->steps_done = h->steps_done;
    info->block_x = h->bx;
    info->block_y = h->by;
    info->kernel = kernel_kind(h, h->in_batch);  // a batch member: the kernel its batch steps it with
    return LBM2D_OK;
}

int lbm2d_set_block(lbm2d_solver* h, int bx, int by) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (bx == 0 && by == 0) {
        bx = 128;
        by = 2;
    }
    if (bx <= 0 || by <= 0 || bx * by > 512 || (bx * by) % 32 != 0)
        return fail(h, LBM2D_ERR_INVALID, "block must have a multiple of 32 threads, at most 512");
    h->bx = bx;
    h->by = by;
    return LBM2D_OK;
}

int lbm2d_set_profiling(lbm2d_solver* h, int on) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    h->profiling = on != 0;
    return LBM2D_OK;
}

int lbm2d_profile(lbm2d_solver* h, double* ms, long long* n) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    CK(cudaStreamSynchronize(h->stream), "profile sync");
    double total = 0.0;
    for (size_t k = 0; k + 1 < h->ev_used; k += 2) {
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, h->ev_pool[k], h->ev_pool[k + 1]), "elapsed");
        total += t;
    }
    if (ms) *ms = total;
    if (n) *n = (long long)(h->ev_used / 2);
    h->ev_used = 0;
    return LBM2D_OK;
}

int lbm2d_set_wait_limit(lbm2d_solver* h, long long cycles) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    h->consumer_wait = cycles;
    return LBM2D_OK;
}

int lbm2d_set_kernel_variant(lbm2d_solver* h, int variant) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (variant < 0 || variant > 3) return fail(h, LBM2D_ERR_INVALID, "unknown kernel variant");
    if (variant == h->variant) return LBM2D_OK;
    if ((rc = before_setting_change(h))) return rc;  // the stored state stays valid; rebuild for safety
    h->variant = variant;
    return LBM2D_OK;
}

void* lbm2d_stream(lbm2d_solver* h) { return h ? (void*)h->stream : nullptr; }
long long lbm2d_launch_count(lbm2d_solver* h) { return h ? h->launches : 0; }

}  // extern "C"
