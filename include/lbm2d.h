/*
 * lbm2d.h -- C-ABI of the GB300 (sm_103a) D2Q9 lattice-Boltzmann step.
 *
 * This is the drop-in boundary.  The lbm-2d reference exposes its solver as a
 * header-only C++ API: process-global knobs (src/lbm_types.hpp:15-32), a state
 * struct LBMCapabilities (src/lbm_types.hpp:187-224) and free functions in
 * src/lbm.hpp.  Each entry point below replaces one piece of that interface;
 * the comment names the reference declaration it stands in for.  The C++
 * headers in lbm-2d_gb300/dropin/ (lbm.hpp, lbm_types.hpp, thermal.hpp,
 * geometry.hpp) re-create the reference's names on top of these calls, so the
 * reference's case drivers compile unchanged against them.
 *
 * Conventions
 *   - Every call returns an int status (LBM2D_OK = 0).  lbm2d_last_error()
 *     gives a message for the last failing call on a handle, and
 *     lbm2d_global_error() for a failed lbm2d_create().
 *   - Host arrays are plain pointers with the reference's layouts:
 *     populations FP64 array-of-structures f[node*9 + i], node = y*nx + x,
 *     direction order of src/lbm_types.hpp:41-42; per-node fields FP64 or u8.
 *   - A handle owns its device buffers and one CUDA stream; it is not
 *     thread-safe.  Work is asynchronous on that stream; calls that return
 *     host data synchronize it.
 *   - State semantics follow execute_time_step (src/lbm.hpp:293-582): the
 *     state a caller uploads and downloads is the post-stream, post-boundary
 *     state the reference keeps in LBMCapabilities::f between steps.
 */
#ifndef LBM2D_H
#define LBM2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes */
#define LBM2D_OK 0
#define LBM2D_ERR_INVALID 1   /* bad argument or configuration */
#define LBM2D_ERR_OOM 2       /* device allocation failed */
#define LBM2D_ERR_CUDA 3      /* CUDA runtime error */
#define LBM2D_ERR_NAN 4       /* a non-finite density was produced */
#define LBM2D_ERR_STATE 5     /* call out of order (e.g. no state uploaded) */
#define LBM2D_ERR_NO_DEVICE 6 /* no usable CUDA device */
#define LBM2D_ERR_TIMEOUT 7   /* a bounded device wait ran out */

/* ---- case types: numbering of CaseType, src/lbm_types.hpp:20-23 */
#define LBM2D_CASE_CYLINDER 0
#define LBM2D_CASE_CAVITY 1
#define LBM2D_CASE_STEP 2
#define LBM2D_CASE_RIBS 3
#define LBM2D_CASE_URBAN_CANYON 4
#define LBM2D_CASE_DOWNWASH 5
#define LBM2D_CASE_SQUARE_CYLINDER 6
#define LBM2D_CASE_FLAT_PLATE 7
#define LBM2D_CASE_SPORTS_BALL 8
#define LBM2D_CASE_PERIODIC_HILLS 9
#define LBM2D_CASE_CYLINDER_NEAR_WALL 10
#define LBM2D_CASE_SIDE_BY_SIDE 11
#define LBM2D_CASE_ROTATING_CYLINDER 12
#define LBM2D_CASE_ORIFICE_PLATE 13

/* ---- collision operators: CollisionType, src/lbm_types.hpp:26 */
#define LBM2D_MRT 0
#define LBM2D_BGK 1

/* ---- population storage on the device (the collision always runs in FP32,
 *      or in FP64 for LBM2D_STORE_FP64).  FP16/BF16 store the shifted
 *      deviation f_i - w_i*rho0 (rho0 = 1), and g_i - w_i*T_ref for thermal. */
#define LBM2D_STORE_FP32 0
#define LBM2D_STORE_FP16 1
#define LBM2D_STORE_BF16 2
#define LBM2D_STORE_FP64 3

/* ---- device-side thermal boundary passes (the drivers' post-step loops) */
#define LBM2D_HOOK_NONE 0
#define LBM2D_HOOK_HEATED_CAVITY 1   /* src/thermal_cavity.cpp:168-204 */
#define LBM2D_HOOK_HEATED_SOLIDS 2   /* src/heated_cylinder.cpp:156-164 */

typedef struct lbm2d_config {
    int nx, ny;      /* NX, NY globals (src/lbm_types.hpp:15-16) */
    int case_type;   /* g_case (src/lbm_types.hpp:28) */
    int collision;   /* g_collision (src/lbm_types.hpp:27) */
    int use_les;     /* g_use_les (src/lbm_types.hpp:31) */
    double cs;       /* g_cs (src/lbm_types.hpp:32) */
    int storage;     /* LBM2D_STORE_* */
    int device;      /* CUDA device ordinal */
} lbm2d_config;

typedef struct lbm2d_info {
    int nx, ny, storage;
    double bytes_per_update;   /* algorithmic population bytes per lattice update */
    size_t device_bytes;       /* device memory held by the handle */
    int n_boundary_nodes;      /* nodes with a boundary record */
    int n_force_nodes;         /* nodes with momentum-exchange links */
    long long steps_done;      /* steps executed since the last upload */
    int block_x, block_y;      /* launch shape of the step kernel */
    int kernel;                /* LBM2D_KERNEL_* the next lbm2d_step runs */
} lbm2d_info;

#define LBM2D_KERNEL_SCALAR 0  /* one node per thread */
#define LBM2D_KERNEL_PAIR 1    /* two x-neighbours per thread, packed FP32x2 */
#define LBM2D_KERNEL_ROWS 2    /* row tiles staged by bulk copies, persistent grid */
#define LBM2D_KERNEL_TILES 3   /* flat tiles of consecutive nodes staged by bulk copies (any nx, thermal, batches) */

typedef struct lbm2d_solver lbm2d_solver;

/* Construct a solver: replaces `LBMCapabilities()` (src/lbm_types.hpp:209-218)
 * together with the globals it reads (src/lbm_types.hpp:15-32).  The initial
 * state matches the constructor: f = 0, g = 1, no obstacles. */
int lbm2d_create(const lbm2d_config *cfg, lbm2d_solver **out);
/* Release the handle and its device memory (LBMCapabilities destructor). */
int lbm2d_destroy(lbm2d_solver *h);
const char *lbm2d_last_error(const lbm2d_solver *h);
const char *lbm2d_global_error(void);

/* Re-select case/collision/LES: the globals g_case, g_collision, g_use_les,
 * g_cs read by execute_time_step (src/lbm.hpp:300-302, :408, :531-543). */
int lbm2d_set_case(lbm2d_solver *h, int case_type, int collision, int use_les, double cs);

/* Solid mask, one byte per node: LBMCapabilities::obstacle
 * (src/lbm_types.hpp:190), as written by place_walls / place_cylinder /
 * place_polygon (src/lbm.hpp:79-87, :931-964) or by drivers directly. */
int lbm2d_set_mask(lbm2d_solver *h, const uint8_t *obstacle);

/* Interpolated bounce-back geometry: LBMCapabilities::bb_geom
 * (BounceBackGeometry, src/lbm_types.hpp:90-182).  A cylinder with radius > 0
 * or a polygon with >= 1 vertex makes bb_geom "valid" (:102); radius 0 and
 * n = 0 clear it.  The polygon replaces any circle, as in the reference. */
int lbm2d_set_bb_cylinder(lbm2d_solver *h, double cx, double cy, double radius);
int lbm2d_set_bb_polygon(lbm2d_solver *h, const double *xy, int n_vertices);
/* BounceBackGeometry::has_moving_wall/omega/rot_cx/rot_cy (src/lbm_types.hpp:98-100). */
int lbm2d_set_moving_wall(lbm2d_solver *h, int on, double omega, double rot_cx, double rot_cy);
/* BounceBackGeometry::use_mei_bb (src/lbm_types.hpp:181): 1 = Mei/Filippova-
 * Hanel (default), 0 = classic Bouzidi with the Ladd wall term (src/lbm.hpp:257-285). */
int lbm2d_set_mei(lbm2d_solver *h, int on);

/* LBMCapabilities::body_force_x (src/lbm_types.hpp:207). */
int lbm2d_set_body_force(lbm2d_solver *h, double fx);
/* Thermal DDF knobs: LBMCapabilities::use_thermal, T_ref, alpha, omega_k,
 * beta, g_buoyancy (src/lbm_types.hpp:196-201). */
int lbm2d_set_thermal(lbm2d_solver *h, int use, double T_ref, double alpha, double omega_k,
                      double beta, double g_buoyancy);
/* Device-side version of a driver's post-step thermal loop (LBM2D_HOOK_*):
 * HEATED_CAVITY(Ta = hot, Tb = cold) as src/thermal_cavity.cpp:168-204,
 * HEATED_SOLIDS(Ta = wall temperature) as src/heated_cylinder.cpp:156-164.
 * Applied to the state after every step, exactly where the drivers apply it. */
int lbm2d_set_thermal_hook(lbm2d_solver *h, int kind, double Ta, double Tb);

/* Populations, FP64 AoS [nx*ny*9]: writes LBMCapabilities::f / g_thermal
 * (src/lbm_types.hpp:188, :194) as the drivers do before their loop. */
int lbm2d_upload_f(lbm2d_solver *h, const double *f);
int lbm2d_upload_g(lbm2d_solver *h, const double *g);

/* Uniform equilibrium state on the device, without a host transfer: the
 * drivers' initialisation loops, f_i = compute_equilibrium(i, rho, u, v)
 * (src/lbm_types.hpp:269-273) and g_i = thermal_equilibrium(i, T, u, v)
 * (src/thermal.hpp:25-30) at every node, e.g. src/cavity.cpp:79-84,
 * src/thermal_cavity.cpp:118-129. */
int lbm2d_init_equilibrium(lbm2d_solver *h, double rho, double u, double v, double T);

/* One or more calls of execute_time_step(sys, tau, u_inflow)
 * (src/lbm.hpp:293-582).  Asynchronous. */
int lbm2d_step(lbm2d_solver *h, double tau, double u_inflow, int nsteps);

/* Sum over nodes of fx_body / fy_body after the last step -- the driver's
 * per-step reduction (src/main.cpp:106-110) of the momentum-exchange force
 * (src/lbm.hpp:543-581).  FP64, synchronizes. */
int lbm2d_force_sums(lbm2d_solver *h, double *fx_total, double *fy_total);
/* Per-step force sums recorded on the device since the last upload or
 * lbm2d_force_history_reset(): copies min(n, recorded) pairs, returns the
 * number of recorded steps in *n_recorded. */
int lbm2d_force_history(lbm2d_solver *h, double *fx, double *fy, int n, int *n_recorded);
int lbm2d_force_history_reset(lbm2d_solver *h);

/* Read back LBMCapabilities::f / g_thermal (FP64 AoS), fx_body / fy_body
 * (FP64, per node), wall_dist (src/lbm_types.hpp:191) and the macroscopic
 * fields of compute_macros / compute_temperature (src/lbm_types.hpp:278-288,
 * src/thermal.hpp:55-60).  Any output pointer of download_macros may be NULL. */
int lbm2d_download_f(lbm2d_solver *h, double *f);
int lbm2d_download_g(lbm2d_solver *h, double *g);
int lbm2d_download_force_field(lbm2d_solver *h, double *fx_body, double *fy_body);
int lbm2d_download_macros(lbm2d_solver *h, double *rho, double *u, double *v, double *T);
int lbm2d_download_wall_dist(lbm2d_solver *h, double *wall_dist);

/* Fields of the reference's frame writers, computed on the device from the
 * state of the last step: save_json_frame (src/lbm.hpp:588-701),
 * save_json_frame_thermal (:707-817) and save_vtk_frame (:860-926).  Point
 * (i, j) of the nxd x nyd output grid, nxd = ceil(nx / ds), nyd =
 * ceil(ny / ds), is node (i*ds, j*ds); outputs are row-major, nxd wide.
 * rho, u, v follow compute_macros in the reference's FP64 operation order,
 * vel = sqrt(u*u + v*v), omega is the writers' downsampled central
 * difference dv/dx - du/dy (one-sided at the grid edges), T the sum of g
 * (zero without the thermal DDF).  obstacle is 1 at solid points, where
 * rho, u, v, vel and omega are 0 and T is T_wall.  sanitize = 1 applies the
 * JSON writers' replacements (rho < 1e-12 or NaN -> rho 1, u = v = 0; NaN
 * u, v, vel -> 0; NaN T -> 1); sanitize = 0 reports raw values, as the VTK
 * writer prints them.  Only nxd*nyd values per field cross to the host.  Any
 * output may be NULL.  Errors: LBM2D_ERR_INVALID for ds < 1,
 * LBM2D_ERR_STATE before the first step after an upload.  Not in the
 * reference (its writers loop over the host state). */
int lbm2d_frame_fields(lbm2d_solver *h, int ds, int sanitize, double T_wall, double *rho, double *u, double *v,
                       double *vel, double *omega, double *T, uint8_t *obstacle);

/* Immersed-boundary direct forcing (src/ibm.hpp) applied around every step
 * as the airfoil driver's loop does it (src/airfoil_ibm.cpp:121-176): the
 * velocity at each Lagrangian point (X[p], Y[p]) is interpolated with the
 * 4-point cosine delta from the fluid nodes of its 5x5 stencil, the no-slip
 * force (u_wall - U) / dt is spread back to the grid in point order, and
 * after the step every fluid node gets f_i += w_i (3 c_i.F + 9 (c_i.0)(c_i.F)).
 * The points are fixed until the next call; npts = 0 removes the boundary.
 * The momentum-exchange force (fx_body) still comes from the state before
 * the forcing, as in the reference; downloads of f, macros and frames see the
 * forced state.  Not with the thermal DDF or inside a batch
 * (LBM2D_ERR_INVALID).  The reference's driver loop has no library entry
 * point; this call replaces it. */
int lbm2d_set_ibm(lbm2d_solver *h, const double *X, const double *Y, int npts, double dt, double u_wall_x,
                  double u_wall_y);
/* The Lagrangian velocities U, V and forces FX, FY (ImmersedBoundary::points
 * and the driver's fx_lag / fy_lag, src/ibm.hpp:27-34, 139-149) that produced
 * the forcing of the last step.  Any output may be NULL. */
int lbm2d_ibm_lagrangian(lbm2d_solver *h, double *U, double *V, double *FX, double *FY);

/* FP64 reductions over the fluid nodes of the current state: total mass
 * (the quantity of the reference's conservation test, src/lbm_test.cpp:
 * 173-198), x/y momentum, and the steady-state residual
 * ||u - u_prev|| / ||u|| against the velocity field of the previous call
 * (NaN on the first call) -- the field-level counterpart of the reference's
 * check_convergence (src/lbm.hpp:93-104).  Any output may be NULL. */
int lbm2d_diagnostics(lbm2d_solver *h, double *mass, double *mom_x, double *mom_y, double *residual);

/* Wait for the handle's stream; reports LBM2D_ERR_NAN if any step since the
 * last check produced a non-finite density. */
int lbm2d_synchronize(lbm2d_solver *h);
int lbm2d_get_info(lbm2d_solver *h, lbm2d_info *info);
/* Launch shape of the step kernel (threads per block = bx*by, a multiple of
 * 32, at most 1024).  0,0 restores the tuned default. */
int lbm2d_set_block(lbm2d_solver *h, int bx, int by);
/* Step-kernel variant.  0 (default): the fastest kernel the configuration
 * allows -- the row pipeline (non-thermal FP32 with nx a multiple of 4, or
 * FP16/BF16 with nx a multiple of 8; in a batch only members of at least
 * 2^21 nodes), else two nodes per thread with packed FP32x2 arithmetic
 * (non-thermal, nx even; in a batch or the resident serving loop: flat
 * node pairs, any nx with an even node count), else one node per thread
 * (the thermal DDF: six 256-thread blocks per SM).  1: one node per
 * thread.  2: two x-neighbours per thread where nx is even (thermal
 * included).  3: the tile pipeline (FP32/FP16/BF16).  Same results to
 * rounding; lbm2d_get_info reports the kernel in use (for a batch member,
 * the kernel its batch steps it with; a plain lbm2d_step of a member runs
 * the single-solve kernels). */
int lbm2d_set_kernel_variant(lbm2d_solver *h, int variant);
/* Limit, in SM cycles, of the staging pipelines' (row and tile kernels)
 * consumer-side waits for their staged tiles (0, the default: about one
 * second).  A wait that runs out makes the kernel stop early and the next
 * lbm2d_synchronize report LBM2D_ERR_TIMEOUT, with the context still usable.
 * A negative value is the failure-path test: the producer stages nothing, so
 * every consumer wait runs out after -cycles cycles.  The producer's own
 * waits keep the default.  No counterpart in the reference. */
int lbm2d_set_wait_limit(lbm2d_solver *h, long long cycles);
/* The CUDA stream the handle launches on (cudaStream_t as void*). */
void *lbm2d_stream(lbm2d_solver *h);
/* Count of kernel launches made by this handle since creation. */
long long lbm2d_launch_count(lbm2d_solver *h);

/* Kernel timing: while on, the handle records a CUDA event pair around every
 * step-kernel launch on its stream; lbm2d_profile synchronizes, returns the
 * summed step-kernel time in milliseconds and the number of timed launches,
 * and clears the record. */
int lbm2d_set_profiling(lbm2d_solver *h, int on);
int lbm2d_profile(lbm2d_solver *h, double *step_kernel_ms, long long *n_launches);

/* Step without any allocation, for callers that may not allocate device
 * memory once running: real-time or co-simulation loops with a per-step
 * deadline (cudaMalloc/cudaFree can synchronize the device and take
 * milliseconds) and processes whose device footprint is fixed at start-up.
 * No counterpart in the reference.  The solver must have been prepared by a
 * prior lbm2d_step with the same tau and settings (else LBM2D_ERR_STATE);
 * the force-reduction scratch is a fixed 2 MiB array inside the library
 * (at most 131072 per-warp force slots, else LBM2D_ERR_INVALID), held on
 * every GPU that loads the library until the process exits.  The preparing
 * lbm2d_step looks the array's address up on its device (once per device,
 * cudaGetSymbolAddress), so the first lbm2d_step_noalloc call needs no set-up
 * of its own; it launches the same kernels as lbm2d_step.  It refuses to run
 * while profiling is on (LBM2D_ERR_STATE).  All callers share the array:
 * calls that overlap on the GPU (e.g. two solvers on different streams) race
 * and corrupt each other's drag/lift; serialize them on one stream. */
int lbm2d_step_noalloc(lbm2d_solver *h, double tau, double u_inflow, int nsteps);

/* Device-resident variants for callers that keep populations on the GPU:
 * pointers to device memory, same FP64 AoS layout, stream-ordered on the
 * handle's stream (no host synchronization). */
int lbm2d_upload_f_device(lbm2d_solver *h, const double *d_f);
int lbm2d_download_f_device(lbm2d_solver *h, double *d_f);


/* ---- batching: many independent solves in one launch.
 * The reference steps one LBMCapabilities per process (its globals allow no
 * more); these entry points have no counterpart there.  A batch steps every
 * member with one packed launch per storage/thermal group: a
 * tile-to-instance table maps each launch block to (member, block of that
 * member's grid).  Repeated step pairs are replayed from a captured CUDA
 * graph.  Members keep their own state, geometry, forces and history; their
 * own streams are ordered after the batch's work, so lbm2d_download_* on a
 * member sees the batched steps. */
typedef struct lbm2d_batch lbm2d_batch;
int lbm2d_batch_create(int device, lbm2d_batch **out);
int lbm2d_batch_destroy(lbm2d_batch *b);
const char *lbm2d_batch_last_error(const lbm2d_batch *b);
/* Add / remove a member; (tau, u_inflow) are the arguments of its
 * execute_time_step calls while in the batch. */
int lbm2d_batch_add(lbm2d_batch *b, lbm2d_solver *h, double tau, double u_inflow);
int lbm2d_batch_remove(lbm2d_batch *b, lbm2d_solver *h);
int lbm2d_batch_set_params(lbm2d_batch *b, lbm2d_solver *h, double tau, double u_inflow);
/* Step budget of a member: it takes at most `steps` more steps and then sits
 * out the batch's launches (its state is left after its last step, so
 * members with different budgets can share one long lbm2d_batch_step call).
 * -1 (the default) means unlimited. */
int lbm2d_batch_set_budget(lbm2d_batch *b, lbm2d_solver *h, long long steps);
/* Remaining budget of a member (-1: unlimited or not a member). */
long long lbm2d_batch_budget(lbm2d_batch *b, lbm2d_solver *h);
int lbm2d_batch_size(lbm2d_batch *b);
/* Step every member nsteps times (asynchronous on the batch stream). */
int lbm2d_batch_step(lbm2d_batch *b, int nsteps);
int lbm2d_batch_synchronize(lbm2d_batch *b);
/* Launch shape shared by the members (multiple of 32 threads, <= 512). */
int lbm2d_batch_set_block(lbm2d_batch *b, int bx, int by);
void *lbm2d_batch_stream(lbm2d_batch *b);
long long lbm2d_batch_launch_count(lbm2d_batch *b);

/* ---- serving loop: requests of different grid sizes, geometries, Reynolds
 * numbers and step budgets arrive at any time; set-up threads admit them by
 * device-memory footprint and build them on the host cores, a stepping
 * thread steps all active solves together through a batch (one packed
 * launch per step per storage group) and retires each one exactly at its
 * budget.  No counterpart in the reference (one solve per process there). */
#define LBM2D_GEOM_CAVITY 0        /* lid-driven cavity, src/cavity.cpp */
#define LBM2D_GEOM_STEP 1          /* backward-facing step h = NY/3, src/step.cpp */
#define LBM2D_GEOM_CYLINDER 2      /* cylinder D = NY/5, src/main.cpp */
#define LBM2D_GEOM_SIDE_BY_SIDE 3  /* two cylinders D = NY/5, S/D = param */
#define LBM2D_GEOM_HEATED_CAVITY 4 /* differentially heated cavity, Ra = param, src/thermal_cavity.cpp */

typedef struct lbm2d_request {
    int nx, ny;
    int geometry;   /* LBM2D_GEOM_* */
    double re;      /* Reynolds number (tau = 0.5 + 3 u L / Re; LES when tau < 0.55) */
    double param;   /* S/D for side-by-side cylinders, Ra for the heated cavity */
    double u;       /* lid / inlet velocity (default 0.1) */
    int steps;      /* step budget */
    int storage;    /* LBM2D_STORE_* */
} lbm2d_request;

typedef struct lbm2d_result {
    long long id;
    int status;                     /* LBM2D_OK, LBM2D_ERR_NAN, ... */
    double t_submit, t_admit, t_done; /* seconds, steady clock */
    long long steps, nodes;
    double fx, fy;                  /* final drag / lift sums */
} lbm2d_result;

typedef struct lbm2d_server_stats_t {
    long long submitted, finished, queued, active;
    double busy_s;                  /* wall time the worker spent stepping */
    long long lattice_updates;
    double device_bytes_in_use;
    long long ticks;        /* batched step calls made */
    long long member_ticks; /* sum over ticks of the solves in the tick */
    double setup_s;         /* host time spent building requests (all set-up threads) */
    double gpu_s;           /* time from the start to the end of each tick's batched step on the device */
    double call_s, wait_s, retire_s, join_s; /* stepping thread: step calls, device waits, retirements, joins */
} lbm2d_server_stats_t;

typedef struct lbm2d_server lbm2d_server;
int lbm2d_server_create(int device, double budget_bytes, int max_active, int steps_per_tick, lbm2d_server **out);
/* flags of lbm2d_server_create_ex.  LBM2D_SERVE_RESIDENT: the solves are
 * stepped by a device-resident loop (a CUDA graph WHILE loop over a device
 * table of solves): a solve joins at the next step boundary after it is set
 * up and retires at its budget with no host round trip between steps;
 * steps_per_tick bounds the iterations of one launch of the loop (it
 * relaunches while solves are active).  max_active <= 1024.  Without it:
 * ticks of steps_per_tick batched steps (lbm2d_server_create). */
#define LBM2D_SERVE_RESIDENT 1
/* LBM2D_SERVE_FIFO: every tick steps every active solve.  Without it a tick
 * steps the solves with the fewest remaining steps first, as many as make
 * 16 Mi lattice nodes, and the others wait: the same final states, a median
 * time to solution about half as long, 4% less aggregate throughput. */
#define LBM2D_SERVE_FIFO 2
int lbm2d_server_create_ex(int device, double budget_bytes, int max_active, int steps_per_tick, int flags,
                           lbm2d_server **out);
int lbm2d_server_submit(lbm2d_server *s, const lbm2d_request *r, long long *id);
/* lbm2d_server_submit with caller state: f_init (may be NULL) is the
 * request's initial population field, FP64 AoS [nx*ny*9], copied before the
 * call returns and uploaded in place of the geometry's equilibrium start;
 * f_out / g_out (may be NULL; g_out only for LBM2D_GEOM_HEATED_CAVITY)
 * receive the final populations / temperature populations when the request
 * retires (also when it diverged), before its result is reported -- the
 * buffers must stay valid until then.  No counterpart in the reference. */
int lbm2d_server_submit_state(lbm2d_server *s, const lbm2d_request *r, const double *f_init, double *f_out,
                              double *g_out, long long *id);
/* Block until at least n_finished requests are done (or timeout). */
int lbm2d_server_wait(lbm2d_server *s, long long n_finished, double timeout_s);
int lbm2d_server_results(lbm2d_server *s, lbm2d_result *out, int capacity, int *count);
int lbm2d_server_stats(lbm2d_server *s, lbm2d_server_stats_t *stats);
int lbm2d_server_destroy(lbm2d_server *s);

/* ---- launch-shape autotuner: times `steps` steps for each candidate (the
 * row pipeline when the solver would run it, then each block shape of the
 * paired or one-node kernel; the state is saved before and restored after),
 * keeps the fastest and returns its block shape -- (0, 0) when the row
 * pipeline won; otherwise the solver is left on that shape with kernel
 * variant 2 (or its own variant).  The batch form tunes the shared shape of
 * the batched kernels.  No counterpart in the reference. */
int lbm2d_autotune(lbm2d_solver *h, int steps, double tau, double u_inflow, int *best_bx, int *best_by);
int lbm2d_batch_autotune(lbm2d_batch *b, int steps, int *best_bx, int *best_by);

/* ---- host services (no device needed): the reference's set-up arithmetic,
 *      shared by the C++ drop-in headers and the Python binding so masks and
 *      link lists are bit-exact with the reference. */

/* compute_equilibrium, src/lbm_types.hpp:269-273 */
double lbm2d_equilibrium(int i, double rho, double u, double v);
/* place_walls on a mask [nx*ny], src/lbm.hpp:79-87 */
int lbm2d_mask_walls(int nx, int ny, uint8_t *mask);
/* place_cylinder's mask rule sqrt(dx^2+dy^2) < r, src/lbm.hpp:931-944 */
int lbm2d_mask_cylinder(int nx, int ny, uint8_t *mask, int cx, int cy, int radius);
/* place_polygon's mask rule (point_in_polygon per node), src/lbm.hpp:951-964 */
int lbm2d_mask_polygon(int nx, int ny, uint8_t *mask, const double *xy, int n_vertices);
/* point_in_polygon, src/geometry.hpp:120-134 */
int lbm2d_point_in_polygon(double px, double py, const double *xy, int n_vertices);
/* naca_coords, src/geometry.hpp:17-90: writes 2n-1 points (x,y pairs) into
 * out (capacity 2*(2n-1) doubles), returns the point count. */
int lbm2d_naca_coords(int series, int n, double *out);
/* transform_points, src/geometry.hpp:95-114 (in place) */
int lbm2d_transform_points(double *xy, int n, double cx, double cy, double scale, double angle_deg);
/* compute_wall_distance's result, src/lbm_types.hpp:231-264 */
int lbm2d_wall_distance(int nx, int ny, const uint8_t *mask, double *wall_dist);
/* Lagrangian points of ImmersedBoundary::build_from_polygon (src/ibm.hpp:
 * 42-69): max(8, perimeter / spacing) points spaced uniformly in the
 * polygon's vertex parameter.  Writes at most cap points to X, Y (either may
 * be NULL to query the count); returns the point count. */
int lbm2d_ibm_points_from_polygon(const double *xy, int n, double spacing, double *X, double *Y, int cap);

/* Statistics of a drag/lift series as the reference's post-processing
 * computes them (scripts/extract_forces.py:91-121 and :137-158): means of
 * v1 (Cd or Fx) and v2 (Cl or Fy) after skipping the first 20% of samples
 * (none if that is fewer than 10), the standard deviation of v2, and the
 * shedding frequency from upward crossings of the mean of v2 after a 40%
 * (at least 50 samples) transient: crossings / (2 * duration * dt); st is
 * NaN when the script reports None (fewer than 200 samples, fewer than 100
 * after the skip, or fewer than 2 crossings). */
typedef struct lbm2d_force_stats_t {
    double mean_v1, mean_v2, std_v2, st;
    int n_skip;
} lbm2d_force_stats_t;
int lbm2d_force_stats(const double *v1, const double *v2, int n, double dt, lbm2d_force_stats_t *out);

/* Geometry of the interpolated bounce-back (BounceBackGeometry,
 * src/lbm_types.hpp:90-182) for the host link query below. */
typedef struct lbm2d_bb_geometry {
    double cx, cy, radius;
    const double *poly; /* x,y pairs, may be NULL */
    int n_poly;
    int has_moving_wall;
    double omega, rot_cx, rot_cy;
} lbm2d_bb_geometry;

/* Every bounce-back link of a mask as the reference's streaming treats it
 * (src/lbm.hpp:408-484): node index, link direction i (node -> solid or
 * outside), kind (1 = simple bounce-back, 2 = interpolated, 3 = no source),
 * q and wall velocity of interpolated links (src/lbm_types.hpp:106-176) and
 * whether the force pass counts the link (src/lbm.hpp:543-581).  Returns the
 * total link count in *count; arrays receive at most `capacity` entries. */
int lbm2d_boundary_links(int nx, int ny, int case_type, const uint8_t *mask, const lbm2d_bb_geometry *geom,
                         int capacity, int32_t *node, int8_t *dir, int8_t *kind, double *q, double *uwx,
                         double *uwy, int8_t *counts_force, int *count);

#ifdef __cplusplus
}
#endif
#endif /* LBM2D_H */
