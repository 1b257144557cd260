// lbm2d_runtime.h -- the solver handle and its state machine (host runtime),
// shared by the single-instance C-ABI (lbm2d_capi.cpp) and the batched /
// serving layer (lbm2d_batch.cpp).  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm2d.h"
#include "lbm2d_geometry.h"
#include "lbm2d_internal.h"

namespace lbm2d {
namespace rt {

inline constexpr double W[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                         1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
inline constexpr int CASE_CAVITY = 1, CASE_STEP = 2, CASE_RIBS = 3, CASE_HILLS = 9;

inline size_t elem_size(int storage) {
    switch (storage) {
        case ST_FP32: return 4;
        case ST_FP16:
        case ST_BF16: return 2;
        case ST_FP64: return 8;
    }
    return 0;
}

struct CollideParams {
    int collision = 0, les = 0, thermal = 0;
    double s_shear = 0, s_bulk = 0, s_normal = 0, tau = 0, cs_sq = 0, nu = 0, Fscale = 0;
    double omega_k = 0, beta = 0, g_buoy = 0, T_ref = 0;
    bool operator==(const CollideParams& o) const {
        return collision == o.collision && les == o.les && thermal == o.thermal && s_shear == o.s_shear &&
               s_bulk == o.s_bulk && s_normal == o.s_normal && tau == o.tau && cs_sq == o.cs_sq && nu == o.nu &&
               Fscale == o.Fscale && omega_k == o.omega_k && beta == o.beta && g_buoy == o.g_buoy &&
               T_ref == o.T_ref;
    }
};

}  // namespace rt
}  // namespace lbm2d

struct lbm2d_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    int nx = 0, ny = 0;
    size_t N = 0;
    int case_type = 0, collision = 0, use_les = 0, storage = 0;
    double cs = 0.12;
    std::vector<uint8_t> mask;
    lbm2d::BBGeometry bb;
    double body_force = 0.0;
    bool thermal = false;
    double T_ref = 1.0, alpha = 0.1666666667, omega_k = 1.0, beta = 0.0, g_buoy = 0.0;
    int hook = 0;
    double hook_a = 0.0, hook_b = 0.0;

    // device buffers
    void* P[2] = {nullptr, nullptr};
    void* G[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t* d_flags = nullptr;
    uint32_t* d_rec_info = nullptr;
    uint32_t* d_rec_force = nullptr;
    double* d_rec_wd = nullptr;
    double* d_rec_q = nullptr;
    double* d_rec_uw = nullptr;
    double* d_partials = nullptr;
    int* d_block_slot = nullptr;
    int* d_bpairs = nullptr;  // row pipeline: boundary pairs (KParams::bpairs)
    int nbpairs = 0, bchunk = 0;
    bool slot_bpass = false;  // slots laid out for a batch member's boundary blocks
    unsigned int* d_red_done = nullptr;  // arrivals of the fused force reduction
    int red_blocks = 0;                  // blocks (CTAs) that hold force slots
    int nslots = 0, slot_bx = 0, slot_by = 0, slot_kind = -1, slot_grid = 0;
    double* d_hist = nullptr;
    int hist_cap = 1 << 18;
    unsigned long long* d_counter = nullptr;
    double* d_last = nullptr;  // device alias of h_last
    double* h_last = nullptr;  // last (Fx, Fy): mapped pinned memory the kernels write
    unsigned int* d_nan = nullptr;
    uint32_t* d_seed = nullptr;  // rounding-noise seed words, one per population buffer
    double* d_stage_f = nullptr;
    double* d_stage_g = nullptr;
    double* d_fx = nullptr;
    double* d_diag = nullptr;    // 5 FP64 accumulators
    float* d_prev_uv = nullptr;  // velocity field of the last residual check
    bool have_prev_uv = false;
    double* d_fy = nullptr;
    size_t device_bytes = 0;

    lbm2d::GeometryTables geo;
    bool geom_dirty = true;
    bool staged = true;  // STAGED (true) or COLLIDED (false)
    bool stage_f_valid = false, stage_g_valid = false;  // staging holds S (else defaults)
    lbm2d::rt::CollideParams cp_of_P;
    double u_last = 0.0;
    long long steps_since_collide = 0;
    long long steps_done = 0;
    long long launches = 0;
    int bx = 128, by = 2;
    // 0: fastest kernel the configuration allows (row pipeline; else
    // paired, flat pairs in a batch; else one node per thread, the thermal
    // DDF's), 1: one node per thread, 2: paired nodes, 3: the tile pipeline
    int variant = 0;
    bool in_batch = false;  // a batch member is stepped by the batched kernels
    bool resident = false;  // a member of the resident serving loop (never the row pipeline)
    bool profiling = false;
    long long consumer_wait = 0;  // row pipeline's consumer wait limit in cycles (0: default)
    // immersed boundary (lbm2d_set_ibm); ibm_np == 0: none.  F and the
    // Lagrangian values are double-buffered: slot ibm_next holds the force
    // for the next step, slot ibm_next ^ 1 the force the current state
    // carries (and the point values that produced it).
    int ibm_np = 0, ibm_nb = 0, ibm_next = 0;
    double ibm_dt = 1.0, ibm_uwx = 0.0, ibm_uwy = 0.0;
    int* d_ibm_band = nullptr;    // per node: band index, -1 outside the band
    char* d_ibm_tab = nullptr;    // band nodes, spread and interpolation lists
    double* d_ibm_buf = nullptr;  // uv[2nb], F[2][2nb], lag[2][4np]
    lbm2d::IbmParams ibm_q{};     // table pointers; uv; F_out / lag set per launch
    // multi-step calls replay a captured pair of steps (see lbm2d_step)
    cudaGraphExec_t pair_graph = nullptr;
    std::vector<unsigned char> pair_key;
    long long pair_launches = 0;
    std::vector<cudaEvent_t> ev_pool;  // even/odd = start/stop
    size_t ev_used = 0;
    std::string err;
};


namespace lbm2d {
namespace rt {

int fail(lbm2d_solver* h, int code, const std::string& msg);
int cuda_fail(lbm2d_solver* h, cudaError_t e, const char* what);
int bc_kind(int case_type);
CollideParams collide_params(const lbm2d_solver* h, double tau);
KParams base_params(const lbm2d_solver* h);
void set_u_bc(KParams& p, double u);
void apply_collide(KParams& p, const CollideParams& c);
int ensure_populations(lbm2d_solver* h);
int ensure_stage(lbm2d_solver* h, bool want_g);
int upload_geometry(lbm2d_solver* h);
int ensure_slots(lbm2d_solver* h, bool batch = false);
KParams rebuild_params(const lbm2d_solver* h);
int materialize(lbm2d_solver* h);
int before_setting_change(lbm2d_solver* h);
int prologue(lbm2d_solver* h, const CollideParams& c);
int check_handle(lbm2d_solver* h);
// Immersed boundary (lbm2d_ibm.cpp).  ibm_after_step runs after each step
// kernel (p: that step's parameters; the caller then flips ibm_next with
// cur); ibm_from_stage after a prologue
// computes the first force from the staged state; ibm_state_params adds the
// forcing the current state carries to rebuild parameters.
inline bool ibm_active(const lbm2d_solver* h) { return h->ibm_np > 0; }
int ibm_after_step(lbm2d_solver* h, const KParams& p);
int ibm_from_stage(lbm2d_solver* h, const KParams& p);
void ibm_state_params(const lbm2d_solver* h, KParams& p);
void ibm_release(lbm2d_solver* h);
// Two x-neighbours per thread (packed FP32x2 collision) when nx is even and
// the storage is FP32/FP16/BF16 (for the thermal DDF only with variant 2).
bool use_pair(const lbm2d_solver* h);
// Step kernel of the next step: KERNEL_SCALAR, KERNEL_PAIR, KERNEL_ROWS
// (the bulk-copy row pipeline) or KERNEL_TILES (the bulk-copy tile pipeline:
// any nx, the thermal DDF, batches; kernel variant 3 only -- on the measured
// workloads the other kernels were faster).  Batch members run the batched
// paired / one-node kernels, except members of at least kBatchSoloNodes nodes
// that qualify for the row pipeline: those fill the GPU alone and get their
// own row-pipeline launches inside the batch's step.
enum KernelKind : int { KERNEL_SCALAR = 0, KERNEL_PAIR = 1, KERNEL_ROWS = 2, KERNEL_TILES = 3 };
constexpr long long kBatchSoloNodes = 1LL << 21;
int kernel_kind(const lbm2d_solver* h);              // a plain step's kernel
int kernel_kind(const lbm2d_solver* h, bool batch);  // batch: stepped by a batch or the resident loop
// Bring a handle to the COLLIDED state for steps with (tau, u) and fill the
// kernel parameters of the next step (fin = current buffer); returns status.
int prepare_steps(lbm2d_solver* h, double tau, double u_inflow, KParams& p, bool batch = false);
// Launch one step from buffer h->cur (step kernel with its force reduction
// into p.partials, immersed-boundary kernels); advance() then moves the host
// state on by n steps.  e0 / e1 (optional) bracket the step kernel.
int launch_one_step(lbm2d_solver* h, KParams& p, cudaEvent_t e0 = nullptr, cudaEvent_t e1 = nullptr);
void advance(lbm2d_solver* h, long long n);
// Device address of the allocation-free entry point's fixed scratch array on
// h's device, looked up once per device while a solver is being prepared
// (lbm2d_noalloc.cu); lbm2d_step calls it so that the first allocation-free
// call needs no lookup.
int noalloc_bind_device(int device);

}  // namespace rt
}  // namespace lbm2d
