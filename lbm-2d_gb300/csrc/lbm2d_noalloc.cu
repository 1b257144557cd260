// lbm2d_noalloc.cu -- a step entry point that allocates nothing.
//
// Some callers must not allocate device memory once they are running:
//   * real-time and co-simulation loops that budget every step: cudaMalloc
//     and cudaFree can synchronize the whole device and take milliseconds,
//     which breaks a fixed per-step deadline;
//   * processes whose device-memory footprint is fixed when they start (a
//     serving process admitted by memory budget, or an application whose
//     device memory is handed out by its own allocator), where a later
//     allocation can fail or exceed the budget that admitted them.
// lbm2d_step_noalloc advances a solver that an earlier lbm2d_step has already
// set up, and takes the scratch space of the force reduction -- per-warp
// partial sums -- from a fixed array compiled into this library instead of
// the handle's own buffer.  It calls no allocating routine of any kind.
#include <mutex>

#include "lbm2d_runtime.h"

using namespace lbm2d;
using namespace lbm2d::rt;

namespace {

// Largest number of per-warp force slots the fixed scratch can hold: two
// doubles per slot, 2 MiB in total.  A 4096 x 4096 channel with 64
// obstacles at the default launch shape needs about 40 000 slots.
constexpr int kNoAllocMaxSlots = 1 << 17;

// Every GPU that loads this library holds this array until the process exits.
static __device__ __align__(256) double g_noalloc_partials[2 * kNoAllocMaxSlots];

constexpr int kMaxDevices = 64;
double* g_scratch[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device, looked up once
// per device (with that device current) on the first call made for it.
int scratch_address(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return LBM2D_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_partials);
        if (e != cudaSuccess || !ptr) return LBM2D_ERR_CUDA;
        g_scratch[device] = static_cast<double*>(ptr);
    }
    *out = g_scratch[device];
    return LBM2D_OK;
}

}  // namespace

extern "C" int lbm2d_step_noalloc(lbm2d_solver* h, double tau, double u_inflow, int nsteps) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (nsteps < 0) return fail(h, LBM2D_ERR_INVALID, "negative step count");
    if (nsteps == 0) return LBM2D_OK;
    if (!(tau > 0.0)) return fail(h, LBM2D_ERR_INVALID, "tau must be positive");
    // Everything the step needs must already exist: a prior lbm2d_step with the
    // same tau and settings has uploaded the geometry, collided the state and
    // built the force-slot table for the current launch shape.
    const CollideParams c = collide_params(h, tau);
    const int kind = kernel_kind(h);
    if (h->staged || h->geom_dirty || !(c == h->cp_of_P) || h->slot_kind != kind || !h->d_block_slot ||
        (kind != KERNEL_ROWS && (h->slot_bx != h->bx || h->slot_by != h->by)))
        return fail(h, LBM2D_ERR_STATE,
                    "lbm2d_step_noalloc needs a solver prepared by lbm2d_step with the same tau and settings");
    if (h->nslots > kNoAllocMaxSlots)
        return fail(h, LBM2D_ERR_INVALID,
                    "force reduction needs " + std::to_string(h->nslots) + " slots; lbm2d_step_noalloc holds at most " +
                        std::to_string(kNoAllocMaxSlots));
    double* scratch = nullptr;
    if ((rc = scratch_address(h->device, &scratch)))
        return fail(h, rc, "cudaGetSymbolAddress of the fixed scratch array failed");

    KParams p = base_params(h);
    apply_collide(p, c);
    set_u_bc(p, u_inflow);
    p.block_slot = h->nslots > 0 ? h->d_block_slot : nullptr;
    // Every slot in [0, nslots) is written by exactly one warp before the
    // reduction reads it, so the shared array needs no clearing between calls.
    p.partials = scratch;
    for (int k = 0; k < nsteps; ++k) {
        p.fin = h->P[h->cur];
        p.fout = h->P[h->cur ^ 1];
        p.gin = h->G[h->cur];
        p.gout = h->G[h->cur ^ 1];
        p.seed_in = h->d_seed + h->cur;
        p.seed_out = h->d_seed + (h->cur ^ 1);
        p.skip_settled_solids = (h->steps_since_collide >= 2 && h->hook != 1) ? 1 : 0;
        int e = kind == KERNEL_ROWS ? launch_rows(h->storage, p, h->slot_grid, h->stream)
                                    : launch_step(h->storage, p, h->bx, h->by, h->stream);
        ++h->launches;
        if (e) return cuda_fail(h, (cudaError_t)e, "step kernel");
        if (h->nslots > 0) {
            e = launch_force_reduce(scratch, h->nslots, h->d_hist, h->hist_cap, h->d_counter, h->d_last, h->stream);
            ++h->launches;
            if (e) return cuda_fail(h, (cudaError_t)e, "force reduce");
        }
        // immersed boundary: launches only, its buffers exist since lbm2d_set_ibm
        if ((rc = ibm_after_step(h, p))) return rc;
        h->cur ^= 1;
        if (ibm_active(h)) h->ibm_next ^= 1;
        ++h->steps_since_collide;
        ++h->steps_done;
    }
    h->u_last = u_inflow;
    return LBM2D_OK;
}
