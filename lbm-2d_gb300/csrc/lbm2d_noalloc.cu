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
// the handle's own buffer.  It calls no allocating routine of any kind and
// launches exactly the kernels lbm2d_step launches (step kernel with its
// fused force reduction, immersed-boundary kernels), so its first call loads
// no kernel that the preparing lbm2d_step did not load already.
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

// Device address of the scratch array on `device`, or null before
// noalloc_bind_device has resolved it there.
double* scratch_of(int device) {
    if (device < 0 || device >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    return g_scratch[device];
}

}  // namespace

namespace lbm2d {
namespace rt {

// Looks the array's device address up once per device, with that device
// current (the caller has made it current).  lbm2d_step calls this while it
// prepares a solver, so the lookup -- which loads this file's module, and
// with it the array, on a device that runs lazily loaded modules -- happens
// on the path that allocates anyway, never inside lbm2d_step_noalloc.
int noalloc_bind_device(int device) {
    if (device < 0 || device >= kMaxDevices) return LBM2D_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_partials);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return LBM2D_ERR_CUDA;
        }
        g_scratch[device] = static_cast<double*>(ptr);
    }
    return LBM2D_OK;
}

}  // namespace rt
}  // namespace lbm2d

extern "C" int lbm2d_step_noalloc(lbm2d_solver* h, double tau, double u_inflow, int nsteps) {
    int rc;
    if ((rc = check_handle(h))) return rc;
    if (nsteps < 0) return fail(h, LBM2D_ERR_INVALID, "negative step count");
    if (nsteps == 0) return LBM2D_OK;
    if (!(tau > 0.0)) return fail(h, LBM2D_ERR_INVALID, "tau must be positive");
    if (h->profiling)  // the event pool may have to grow: that is the regular path's job
        return fail(h, LBM2D_ERR_STATE, "lbm2d_step_noalloc does not record profiling events; switch profiling off");
    // Everything the step needs must already exist: a prior lbm2d_step with the
    // same tau and settings has uploaded the geometry, collided the state,
    // built the force-slot table for the current launch shape and looked the
    // scratch array up on this device.
    const CollideParams c = collide_params(h, tau);
    const int kind = kernel_kind(h);
    double* scratch = scratch_of(h->device);
    if (h->staged || h->geom_dirty || !(c == h->cp_of_P) || h->slot_kind != kind || !h->d_block_slot ||
        (kind != KERNEL_ROWS && kind != KERNEL_TILES && (h->slot_bx != h->bx || h->slot_by != h->by)) || !scratch)
        return fail(h, LBM2D_ERR_STATE,
                    "lbm2d_step_noalloc needs a solver prepared by lbm2d_step with the same tau and settings");
    if (h->nslots > kNoAllocMaxSlots)
        return fail(h, LBM2D_ERR_INVALID,
                    "force reduction needs " + std::to_string(h->nslots) + " slots; lbm2d_step_noalloc holds at most " +
                        std::to_string(kNoAllocMaxSlots));

    KParams p = base_params(h);
    apply_collide(p, c);
    set_u_bc(p, u_inflow);
    p.block_slot = h->nslots > 0 ? h->d_block_slot : nullptr;
    // Every slot in [0, nslots) is written by exactly one warp before the
    // reduction reads it, so the shared array needs no clearing between calls.
    p.partials = scratch;
    for (int k = 0; k < nsteps; ++k) {
        if ((rc = launch_one_step(h, p))) return rc;
        advance(h, 1);
    }
    h->u_last = u_inflow;
    return LBM2D_OK;
}
