// lbm2d_internal.h -- types shared by the CUDA kernels and the host runtime.
//
// Device data layout (one solver instance)
//   populations : structure-of-arrays, 9 planes of nx*ny elements each,
//                 plane j holds direction j for node y*nx + x.  Two buffers
//                 (ping-pong).  What is stored is the POST-COLLISION state of
//                 the last step: the step kernel pulls from it, rebuilds the
//                 reference's post-stream/post-boundary state in registers,
//                 collides, and writes the next post-collision state.
//   flags       : one uint32 per node
//                   bit 0      solid
//                   bit 1      boundary node (has a boundary record)
//                   boundary node: bits 2..31 = record index
//                   other fluid node: the LES wall distance as FP32 bits
//                              (an integer below 2^21, or 1e9 for "no
//                              obstacle"; its two low mantissa bits are 0)
//   records     : per boundary node: slot types, thermal bounce mask, force
//                 mask, wall distance, and per-slot q / wall velocity for
//                 interpolated links.
#pragma once
#include <vector_types.h>

#include <cstddef>
#include <cstdint>

namespace lbm2d {

constexpr uint32_t FLAG_SOLID = 1u;
constexpr uint32_t FLAG_BOUNDARY = 2u;
constexpr uint32_t MAX_RECORDS = 0x3FFFFFFFu;

// Slot types (2 bits per pull slot j) in rec_info bits 0..17.
constexpr uint32_t SLOT_REGULAR = 0;  // pull from the neighbour (wrapped)
constexpr uint32_t SLOT_SIMPLE_BB = 1;  // own post-collision value of bb(j)
constexpr uint32_t SLOT_INTERP = 2;  // interpolated bounce-back (Mei or Bouzidi)
constexpr uint32_t SLOT_ZERO = 3;  // no source (x outside the domain)
// rec_info bits 18..26: thermal slot j bounces (adiabatic) instead of pulling.
constexpr int REC_GBB_SHIFT = 18;

// Boundary-condition families of execute_time_step (src/lbm.hpp:531-540).
enum BcKind : int { BC_NONE = 0, BC_LID = 1, BC_INFLOW = 2, BC_STEP = 3 };

enum Storage : int { ST_FP32 = 0, ST_FP16 = 1, ST_BF16 = 2, ST_FP64 = 3 };

// Physical parameters of one step, held in both compute precisions so the
// FP32 kernels never convert from double at run time.
template <class R>
struct Phys {
    R s_shear, s_bulk, s_normal, tau, inv_tau, cs_sq, cs, inv_nu, nu, Fscale;
    R omega_k, beta, g_buoy, T_ref;
    R u_bc, hook_a, hook_b;
};

struct KParams {
    int nx, ny;
    long long N;  // nx*ny
    // populations
    const void* fin;
    void* fout;
    const void* gin;
    void* gout;
    // geometry
    const uint32_t* flags;
    const uint32_t* rec_info;
    const uint32_t* rec_force;  // force slot mask per record (bits 0..8)
    const double* rec_wd;
    const double* rec_q;   // [rec*9 + j]
    const double* rec_uw;  // [(rec*9 + j)*2 + {0,1}]
    int interp_classic;    // 1: classic Bouzidi (+Ladd), 0: Mei
    int moving_wall;
    // boundary conditions of THIS step
    int bc_kind;
    double u_bc;
    // collision parameters (for the collision that ends the step)
    int collide;  // 0: rebuild state only (readback)
    int collision;  // 0 MRT, 1 BGK
    double s_shear, s_bulk, s_normal, tau, cs_sq, nu, Fscale;
    int les;
    int thermal;
    double omega_k, beta, g_buoy, T_ref;
    int hook_kind;
    double hook_a, hook_b;
    // storage shifts (FP16/BF16 store f - w*rho0, g - w*T_ref)
    float shf[9], shg[9];
    Phys<float> pf;
    Phys<double> pd;
    // force reduction: blocks holding force nodes own (threads/32) consecutive
    // per-warp slots starting at block_slot[block] (-1: no force node)
    const int* block_slot;
    double* partials;       // [slot*2 + {0,1}]
    unsigned int* nan_flag;
    // solid nodes whose state can no longer change may skip their stores
    int skip_settled_solids;
    int gx;    // width of the instance's block grid (batched launches)
    int pair;  // 1: two x-neighbours per thread (nx even, non-thermal, not FP64)
    // stochastic-rounding seed of FP16/BF16 stores: a step reads *seed_in and
    // hands seed + 1 to the next step through *seed_out; a prologue (seed_in
    // null) uses seed_host
    const uint32_t* seed_in;
    uint32_t* seed_out;
    uint32_t seed_host;
    // batched launches only: remaining step budget of the instance (null:
    // unlimited); read from left_in, decremented into left_out
    const int* left_in;
    int* left_out;
    // immersed boundary (state rebuilds only; null in step launches): band
    // index of each node (-1 outside the band) and the grid force (fx, fy)
    // per band node whose forcing the current state carries
    const int* ibm_band;
    const double* ibm_F;
    // drag/lift second stage fused into a single-instance step launch (null:
    // a separate reduction launch).  The blocks that hold force slots count
    // themselves in red_done; the last to arrive sums every slot in the fixed
    // order of sum_slots128, records the sums and resets the count.
    unsigned int* red_done;
    double* red_hist;
    unsigned long long* red_counter;
    double* red_last;
    int red_blocks, red_nslots, red_cap, red_pad;
    // limit, in SM cycles, of the staging pipelines' consumer-side waits on
    // their staged tiles (0: the default of about one second); the producer's
    // own waits keep the default.  Negative: failure-path test -- the
    // producer stages nothing and every consumer wait runs out after
    // -consumer_wait cycles.
    long long consumer_wait;
    // tile pipeline (lbm2d_tiles.cu): 1 / nx for the node coordinates of a
    // flat tile, and the per-tile force-slot table is block_slot
    float inv_nx;
    // row pipeline: the node pairs (x even, x + 1) holding a boundary node,
    // first node's index, ascending; CTA c rebuilds pairs [c*bchunk,
    // (c+1)*bchunk) from device memory before its tiles, which skip them
    int nbpairs;
    const int* bpairs;
    int bchunk;
    // batched paired kernel: tiles of (threads per block) flat node pairs
    // (2k, 2k + 1) of the node index, any width; 0: 2-D tiles of row pairs
    int ftiles;
};
static_assert(sizeof(KParams) % 16 == 0, "KParams is staged with 16-byte copies");

// Readback outputs (any may be null).
struct ROut {
    double* f_aos;
    double* g_aos;
    double *rho, *u, *v, *T;
    double *fx, *fy;
};

// Downsampled frame fields: the point (i, j) of an nxd x nyd grid is node
// (i*ds, j*ds); arrays are row-major, nxd wide.  All pointers are device
// arrays of nxd*nyd entries and must be set.
struct FOut {
    double *rho, *u, *v, *vel, *omega, *T;
    uint8_t* obstacle;
    double T_wall;  // temperature reported at solid points
    int ds, nxd, nyd;
    int sanitize;  // 1: the JSON writers' NaN / zero-density replacements
};

// Immersed-boundary tables and buffers of one solver (device pointers).
// Band nodes: every node in the support of some Lagrangian point's delta
// kernel.  Spread lists (per band node, points in increasing order) and
// interpolation lists (per point, stencil nodes in the reference's y-major
// order) carry the host-computed kernel weights.
struct IbmParams {
    int nb, np;
    const uint32_t* band_node;
    const int* sp_start;
    const int* sp_pt;
    const double* sp_w;
    const int* ip_start;
    const int* ip_band;
    const double* ip_w;
    double* uv;             // [2*nb] band velocities of the latest state
    double* F;              // [2*nb] grid force the latest state carries
    const double* lag_in;   // [4*np] U, V, FX, FY whose forces the step applies
    double* lag_out;        // [4*np] the same from the new state (next step)
    double dt, uwx, uwy;
};

// One instance's second-stage force reduction in a batched launch.
struct ReduceJob {
    const double* partials;
    int nslots, cap;
    double* hist;
    unsigned long long* counter;
    double* last;
    const int* left;  // the step's budget word (null: unlimited); <= 0 means no step was taken
};

// Launchers (lbm2d_kernels.cu).  All return a cudaError_t as int.
int launch_step(int storage, const KParams& p, int bx, int by, void* stream);
int launch_readback(int storage, const KParams& p, const ROut& o, void* stream);
// Immersed boundary, after each step kernel (p: that step's parameters, fin
// its input buffer): per band node, the grid force from q.lag_in, the forced
// state, its velocity and its collision into p.fout; then per point the new
// velocity and force into q.lag_out.
int launch_ibm_after_step(int storage, const KParams& p, const IbmParams& q, void* stream);
// Band velocities of the staged FP64 AoS state (and a zero pending force),
// then the points' velocities and forces into q.lag_out, before the first
// step from it.
int launch_ibm_from_stage(int storage, const KParams& p, const IbmParams& q, const double* aos, void* stream);
// Frame fields of the post-stream state (two launches: point fields, then
// the vorticity stencil over them).
int launch_frame(int storage, const KParams& p, const FOut& o, void* stream);
// Collide an FP64 AoS state S (device) into the stored post-collision state.
int launch_prologue(int storage, const KParams& p, const double* f_aos, const double* g_aos, void* stream);
// Step several instances at once: inst[] holds one KParams per instance and
// block_map[b] (device memory, nblocks entries) the instance of launch block
// b and b's index among that instance's blocks.  A launch block walks
// kBatchTiles consecutive blocks (tiles) of its instance's block grid, so an
// instance with gx*gy tiles owns ceil(gx*gy / kBatchTiles) launch blocks.
constexpr int kBatchTiles = 4;
int launch_batch_step(int storage, const KParams* inst, const int2* block_map, int nblocks, int thermal, int bx,
                      int by, void* stream, int pair);
int launch_batch_force_reduce(const ReduceJob* jobs, int njobs, void* stream);

// Resident serving loop (lbm2d_resident.cu): a CUDA graph whose WHILE node
// steps every member of a device table once per iteration, with a scheduler
// kernel that admits and retires members at every step boundary through a
// mailbox in mapped host memory.  A member's kind ("combo") is its storage
// and kernel: combo = 3 * storage + {0 paired, 1 one node, 2 one node thermal}.
constexpr int kResCombos = 12;
constexpr int kResMaxSlots = 1024;  // one scheduler thread per slot
struct ResEntry {
    KParams p[2];      // the member's step parameters at parity 0 and 1 (p[1]: buffers and seeds swapped)
    ReduceJob job;     // its per-step force reduction (job.nslots == 0: none)
    int combo;         // kernel of the member
    int units;         // work units of one step (launch blocks of the batched kernels)
    int left;          // step budget
    int settle_after;  // steps after which its settled solids are no longer stored (-1: never)
};
// Host <-> device words, in mapped pinned memory.  join[k]: the host writes 1
// once entry k is in the table; the scheduler answers 2 when it admits it.
// done[k]: the scheduler writes the steps taken + 1 when member k retires
// (its last step and force reduction complete); the host clears it when it
// reuses the slot.  join_gen: the host increments it after raising join
// words, so the scheduler reads the join words only when it changed.  stop:
// the host asks the loop to end at the next step boundary.
struct ResMailbox {
    int join[kResMaxSlots];
    long long done[kResMaxSlots];
    int stop;
    int join_gen;
};
struct ResLoop;
int res_create(int device, int cap, int bx, int by, ResLoop** out);
void res_destroy(ResLoop* r);
ResEntry* res_table(ResLoop* r);          // device array of cap entries
volatile ResMailbox* res_mailbox(ResLoop* r);  // host view
// Launch the loop on stream s (graph rebuilt first when the set of combos in
// use changed); it ends by itself when no member is active, after
// max_iters iterations, or at the host's stop word.
int res_launch(ResLoop* r, unsigned combo_mask, int max_iters, void* stream);
// acc[0..4] += mass, x/y momentum, sum |u - u_prev|^2, sum |u|^2 (FP64).
int launch_diagnostics(int storage, const KParams& p, double* acc, float* prev_uv, int have_prev, void* stream);
int launch_fill_equilibrium(double* fa, double* ga, long long N, double rho, double u, double v, double T,
                            void* stream);
int launch_force_reduce(const double* partials, int nslots, double* hist, int hist_cap,
                        unsigned long long* counter, double* last, void* stream);

// Tile-pipelined step (lbm2d_tiles.cu): the lattice of each instance is cut
// into flat tiles of tiles_width() consecutive nodes (row-major, any nx), whose
// nine (thermal: eighteen) source windows, flags and -- in a batch -- the
// instance's parameters are staged by bulk copies; a persistent grid walks
// the tiles of one instance (single) or of many (tile_member[t] = instance of
// global tile t, tile_start[k] = its first global tile).  The force slots of
// an instance are per tile: block_slot[tile] = first of tiles_warps() slots.
int tiles_width();
int tiles_warps();
int tiles_grid(int storage, bool thermal, long long ntiles, int device);  // 0 on error
int launch_tiles_single(int storage, const KParams& p, int grid, void* stream);
int launch_tiles_batch(int storage, bool thermal, const KParams* inst, const int* tile_member, const int* tile_start,
                       int ntiles, int grid, unsigned int* status, void* stream);

// Row-pipelined step (lbm2d_rows.cu): persistent grid of `grid` CTAs, each
// walking row tiles of rows_tile_width() nodes; p.block_slot has one entry
// per CTA (first of rows_warps_per_block() per-warp force slots, or -1).
bool rows_eligible(int storage, int nx, int ny, bool thermal);
// whether the row pipeline of this storage rebuilds the boundary pairs in a
// pass of their own (KParams::bpairs) rather than inline in its tiles
bool rows_boundary_pass(int storage);
int rows_tile_width();
int rows_warps_per_block();
int rows_grid(int storage, int nx, int ny, int device);  // 0 on error
int launch_rows(int storage, const KParams& p, int grid, void* stream);

}  // namespace lbm2d
