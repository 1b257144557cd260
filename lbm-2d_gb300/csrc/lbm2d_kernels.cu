// lbm2d_kernels.cu -- sm_103a kernels of the D2Q9 lattice-Boltzmann step.
//
// One fused, bandwidth-bound pull kernel per time step.  For node m it
//   1. pulls the post-collision populations of the previous step from the
//      9 neighbour positions (SoA planes, coalesced 32-bit/16-bit loads),
//   2. rebuilds the reference's post-stream state: bounce-back, interpolated
//      bounce-back (Mei / Filippova-Hanel or classic Bouzidi with the Ladd
//      wall term) and the "no source" slots, from a per-node boundary record,
//   3. applies the boundary conditions of execute_time_step (lid, Zou/He
//      inlet, parabolic step inlet, zero-gradient outlet) and, if enabled,
//      a driver's post-step thermal pass,
//   4. accumulates the momentum-exchange force of its links (FP64),
//   5. collides (MRT d'Humieres or BGK, Smagorinsky/Van Driest LES, body
//      force, thermal DDF with Boussinesq/Guo buoyancy) in FP32 (FP64 for the
//      FP64 storage variant) and writes the next post-collision state.
// Items 1-3 are the reference's steps streaming -> swap -> boundary
// conditions (src/lbm.hpp:400-540); item 4 is its force pass (:543-581) and
// item 5 is the collision that opens the next call (:300-397).  Storing the
// post-collision state makes the writes aligned and lets the force come from
// registers; the readback kernel rebuilds the reference's state on demand
// with the same device functions.
//
// No tensor cores: the step is a stencil with ~2-3 flop per byte.
#include "lbm2d_device.cuh"

namespace lbm2d {
namespace {

template <class T, bool TH>
__global__ void __launch_bounds__(512) step_pair_kernel(const KParams p) {
    step_pair_block<T, TH>(p, blockIdx.x, blockIdx.y, gridDim.x);
}

template <class T, bool TH>
__global__ void __launch_bounds__(512) step_kernel(const KParams p) {
    step_block<T, TH>(p, blockIdx.x, blockIdx.y, gridDim.x);
}

// The thermal one-node step in blocks of at most 256 threads with a register
// cap that lets MINB of them share an SM: more warps, so more of the 18
// population loads a node makes in flight per SM.  Six blocks (40 registers,
// a few bytes spilled) against the uncapped kernel's four (64 registers) on
// the heated cavity: FP32 4096^2 38.7 against 35.4 GLUPS (0.82 against 0.75
// of the measured copy bandwidth at 144 B per update), 2048^2 32.1 against
// 29.9; FP16 +8-10%.
template <class T, int MINB>
__global__ void __launch_bounds__(256, MINB) step_th_kernel(const KParams p) {
    step_block<T, true>(p, blockIdx.x, blockIdx.y, gridDim.x);
}

// Many independent instances in one launch (the tile-to-instance table):
// instance k owns a contiguous range of launch blocks and walks its own block
// grid (gx = p.gx blocks wide).  block_map[b] = (k, b's index within k), one
// 8-byte load that every thread of the block makes (a broadcast); the block
// then stages that instance's parameters in shared memory.  An instance with
// a step budget (left_in set) whose budget is spent does nothing; otherwise
// its first block hands the decremented budget to the next launch through
// left_out (the two budget words swap roles between launches, so no launch
// reads a word it writes).  Returns false when the block has nothing to do.
__device__ __forceinline__ bool batch_block_begin(const KParams* __restrict__ inst, const int2* __restrict__ block_map,
                                                  KParams& sp, int& local) {
    __shared__ int s_left;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int2 km = __ldg(block_map + blockIdx.x);
    const int k = km.x;
    local = km.y;
    {
        const int* src = reinterpret_cast<const int*>(inst + k);
        int* dst = reinterpret_cast<int*>(&sp);
        const int nw = (int)(sizeof(KParams) / sizeof(int));
        for (int w = tid; w < nw; w += blockDim.x * blockDim.y) dst[w] = src[w];
    }
    if (tid == 0) {
        const int* li = inst[k].left_in;
        const int L = li ? *li : 1;
        if (li && local == 0) *inst[k].left_out = L > 0 ? L - 1 : 0;
        s_left = L;
    }
    __syncthreads();
    return s_left > 0;
}

template <class T, bool TH>
__global__ void __launch_bounds__(512) batch_step_kernel(const KParams* __restrict__ inst,
                                                         const int2* __restrict__ block_map) {
    __shared__ KParams sp;
    int local;
    if (!batch_block_begin(inst, block_map, sp, local)) return;
    const int tiles = sp.gx * ((sp.ny + (int)blockDim.y - 1) / (int)blockDim.y);
    for (int t = local * kBatchTiles; t < min(tiles, (local + 1) * kBatchTiles); ++t)
        step_block<T, TH>(sp, t % sp.gx, t / sp.gx, sp.gx);
}

// The thermal batch members' one-node step, five blocks per SM (48
// registers).  Taken for the 16-bit forms only: on the C4 thermal members
// FP16 35.5 against 31.0 GLUPS, while FP32 spills more than it gains (28.5
// against 30.3).
template <class T, int MINB>
__global__ void __launch_bounds__(256, MINB) batch_step_th_kernel(const KParams* __restrict__ inst,
                                                                 const int2* __restrict__ block_map) {
    __shared__ KParams sp;
    int local;
    if (!batch_block_begin(inst, block_map, sp, local)) return;
    const int tiles = sp.gx * ((sp.ny + (int)blockDim.y - 1) / (int)blockDim.y);
    for (int t = local * kBatchTiles; t < min(tiles, (local + 1) * kBatchTiles); ++t)
        step_block<T, true>(sp, t % sp.gx, t / sp.gx, sp.gx);
}

// Capped at 64 registers (2 x 512 threads per SM): the batched kernel waits
// on its pulls, and the extra resident warps hide more of that latency than
// the few spilled values cost (C4 batch +1.6% FP32, +3% FP16).
template <class T>
__global__ void __launch_bounds__(512, 2) batch_step_pair_kernel(const KParams* __restrict__ inst,
                                                              const int2* __restrict__ block_map) {
    __shared__ KParams sp;
    int local;
    if (!batch_block_begin(inst, block_map, sp, local)) return;
    // a member on this kernel always has flat tiles and its boundary pairs
    // in its boundary blocks (none when it has no boundary node)
    const int tiles = sp.ftiles;
    if (local < 0) {  // boundary block -(local + 1)
        pair_boundary_block<T>(sp, -(local + 1), tiles);
        return;
    }
    for (int t = local * kBatchTiles; t < min(tiles, (local + 1) * kBatchTiles); ++t) step_flat_pair_block<T>(sp, t);
}

// The thermal form: twice the populations, so no register cap.
template <class T>
__global__ void __launch_bounds__(512) batch_step_pair_th_kernel(const KParams* __restrict__ inst,
                                                               const int2* __restrict__ block_map) {
    __shared__ KParams sp;
    int local;
    if (!batch_block_begin(inst, block_map, sp, local)) return;
    const int tiles = sp.gx * ((sp.ny + (int)blockDim.y - 1) / (int)blockDim.y);
    for (int t = local * kBatchTiles; t < min(tiles, (local + 1) * kBatchTiles); ++t)
        step_pair_block<T, true>(sp, t % sp.gx, t / sp.gx, sp.gx);
}

// Post-stream state of node (x, y) in FP64 as the step rebuilds it (before
// any immersed-boundary forcing): stored deviations are widened before the
// shift is added back, so the FP64 value is exact.
template <class T, bool TH>
__device__ __forceinline__ void state_raw_fp64(const KParams& p, int x, int y, uint32_t fl, double f[9],
                                               double g[9]) {
    if constexpr (std::is_same<T, double>::value) {
        build_state<T, TH>(p, x, y, fl, f, g);
    } else {
        float d[9], e[9];
        build_dev<T, TH>(p, x, y, fl, d, e);
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = double(d[j]) + double(p.shf[j]);
        if (TH) {
#pragma unroll
            for (int j = 0; j < 9; ++j) g[j] = double(e[j]) + double(p.shg[j]);
        }
    }
}

// Explicit forcing of a fluid node by the immersed boundary's grid force
// (src/airfoil_ibm.cpp:158-176): f_i += w_i (3 c_i.F + 9 (c_i.0)(c_i.F)),
// each operation rounded on its own in the reference's order (c_i.0 is the
// integer zero of the driver's "u ~ 0" approximation).
__device__ __forceinline__ void ibm_force_node(double f[9], double fx, double fy) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double cxd = double(CXf(i)), cyd = double(CYf(i));
        const double edotu = 0.0;
        const double Fdot = __dadd_rn(__dmul_rn(cxd, fx), __dmul_rn(cyd, fy));
        const double t = __dadd_rn(__dmul_rn(3.0, Fdot), __dmul_rn(__dmul_rn(9.0, edotu), Fdot));
        f[i] = __dadd_rn(f[i], __dmul_rn(wgt(i), t));
    }
}

// The immersed boundary's forcing carried by the current state, if any.
__device__ __forceinline__ void ibm_apply(const KParams& p, size_t n, uint32_t fl, double f[9]) {
    if (p.ibm_band && !(fl & FLAG_SOLID)) {
        const int b = p.ibm_band[n];
        if (b >= 0) ibm_force_node(f, p.ibm_F[2 * b], p.ibm_F[2 * b + 1]);
    }
}

// The reference's state S_n of node (x, y) in FP64: the rebuilt post-stream
// state plus the immersed-boundary forcing applied after the step.
template <class T, bool TH>
__device__ __forceinline__ void state_fp64(const KParams& p, int x, int y, uint32_t fl, double f[9], double g[9]) {
    state_raw_fp64<T, TH>(p, x, y, fl, f, g);
    if (!TH) ibm_apply(p, (size_t)y * p.nx + x, fl, f);
}

template <class T, bool TH>
__global__ void readback_kernel(const KParams p, const ROut o) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const size_t n = (size_t)y * p.nx + x;
    const uint32_t fl = p.flags[n];
    double f[9], g[9];  // the reference's post-stream state in FP64
    state_raw_fp64<T, TH>(p, x, y, fl, f, g);
    // momentum exchange from the state before the immersed-boundary forcing
    // (the reference's force pass ends its step; the driver forces after it)
    double fxn = 0.0, fyn = 0.0;
    if (o.fx && !(fl & FLAG_SOLID) && (fl & FLAG_BOUNDARY)) {
        const uint32_t fm = p.rec_force[fl >> 2];
        for (int i = 0; i < 9; ++i) {  // reference accumulation order (src/lbm.hpp:550-577)
            const int j = BBf(i);
            if (fm & (1u << j)) {
                fxn += double(CXf(i)) * 2.0 * double(f[j]);
                fyn += double(CYf(i)) * 2.0 * double(f[j]);
            }
        }
    }
    if (!TH) ibm_apply(p, n, fl, f);
    if (o.f_aos)
        for (int j = 0; j < 9; ++j) o.f_aos[n * 9 + j] = f[j];
    if (TH && o.g_aos)
        for (int j = 0; j < 9; ++j) o.g_aos[n * 9 + j] = g[j];
    if (o.rho || o.u || o.v) {
        const double* fd = f;
        double rho, u, v;
        macros(fd, rho, u, v);
        if (o.rho) o.rho[n] = rho;
        if (o.u) o.u[n] = u;
        if (o.v) o.v[n] = v;
    }
    if (TH && o.T) {
        double T = 0.0;
        for (int j = 0; j < 9; ++j) T += double(g[j]);
        o.T[n] = T;
    }
    if (o.fx) {
        o.fx[n] = fxn;
        o.fy[n] = fyn;
    }
}

// compute_macros (src/lbm_types.hpp:278-288) in the reference's FP64
// operation order: sequential sums in slot order, u = mx / rho, every
// operation rounded on its own.
__device__ __forceinline__ void macros_ref(const double f[9], double& rho, double& u, double& v) {
    double r = 0.0, mx = 0.0, my = 0.0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        r = __dadd_rn(r, f[q]);
        mx = __dadd_rn(mx, __dmul_rn(f[q], double(CXf(q))));
        my = __dadd_rn(my, __dmul_rn(f[q], double(CYf(q))));
    }
    rho = r;
    u = __ddiv_rn(mx, r);
    v = __ddiv_rn(my, r);
}

// ----------------------------------------------------------------- immersed boundary
// The airfoil driver's loop (src/airfoil_ibm.cpp:121-176) around the step:
// velocity at the Lagrangian points from the fluid nodes of their delta
// stencils, no-slip force (U_wall - U) / dt, spread to the grid, step, then
// explicit forcing of the fluid nodes.  On the device the forcing is folded
// into the stored state.  After the step kernel, a launch over the band (the
// nodes in some point's stencil) spreads the points' forces to each band
// node, forces the rebuilt node, records its velocity and collides it again
// over the step kernel's value; a launch over the points then interpolates
// the new velocities and forms the forces of the next step.  Nodes outside
// the band carry no force and keep the step kernel's result.  The
// momentum-exchange force of the step kernel comes from the unforced state,
// as the reference computes it inside its step.  FP64 storage keeps the
// reference's FP64 operations and order (R = double); the other storages
// compute in FP32 with the same order.

// Band node b after the step kernel: its grid force (the points' forces
// q.lag_in times the kernel weights, summed in point order from zero,
// src/ibm.hpp:72-103), the reference's state after the step with that
// forcing, its velocity, and its collision into p.fout.
template <class T>
__global__ void ibm_band_kernel(const KParams p, const IbmParams q) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= q.nb) return;
    using R = typename std::conditional<std::is_same<T, double>::value, double, float>::type;
    const uint32_t n = q.band_node[b];
    const int y = (int)(n / (uint32_t)p.nx), x = (int)(n - (uint32_t)y * (uint32_t)p.nx);
    const uint32_t fl = p.flags[n];
    R ax = R(0), ay = R(0);
    const int k0 = q.sp_start[b], k1 = q.sp_start[b + 1];
#pragma unroll 4
    for (int k = k0; k < k1; ++k) {
        const int pt = q.sp_pt[k];
        const R w = R(q.sp_w[k]);
        if constexpr (std::is_same<R, double>::value) {
            ax = __dadd_rn(ax, __dmul_rn(q.lag_in[2 * q.np + pt], w));
            ay = __dadd_rn(ay, __dmul_rn(q.lag_in[3 * q.np + pt], w));
        } else {
            ax = fmaf(float(q.lag_in[2 * q.np + pt]), w, ax);
            ay = fmaf(float(q.lag_in[3 * q.np + pt]), w, ay);
        }
    }
    const double Fx = double(ax), Fy = double(ay);
    q.F[2 * b] = Fx;  // the forcing the new state carries (readbacks add it)
    q.F[2 * b + 1] = Fy;
    if (fl & FLAG_SOLID) {
        q.uv[2 * b] = 0.0;
        q.uv[2 * b + 1] = 0.0;
        return;
    }
    T* __restrict__ Fo = static_cast<T*>(p.fout);
    const size_t N = (size_t)p.N;
    if constexpr (std::is_same<T, double>::value) {
        double f[9], g[9];
        state_raw_fp64<T, false>(p, x, y, fl, f, g);
        ibm_force_node(f, Fx, Fy);
        double rho, u, v;
        macros_ref(f, rho, u, v);
        q.uv[2 * b] = u;
        q.uv[2 * b + 1] = v;
        collide<double, false>(p, fl, f, g);
#pragma unroll
        for (int j = 0; j < 9; ++j) Fo[j * N + n] = f[j];
    } else {
        // on deviations, as the step kernels: the forcing adds w_i 3 c_i.F
        float d[9], e[9];
        build_dev<T, false>(p, x, y, fl, d, e);
        const float fx = float(Fx), fy = float(Fy);
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j] = fmaf(float(wgt(j)) * 3.0f, float(CXf(j)) * fx + float(CYf(j)) * fy, d[j]);
        const float drho = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
        const float mx = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
        const float my = (d[2] - d[4]) + (d[5] + d[6]) - (d[7] + d[8]);
        const float inv = 1.0f / (1.0f + drho);
        q.uv[2 * b] = double(mx * inv);
        q.uv[2 * b + 1] = double(my * inv);
        collide_dev<false>(p, fl, d, e);
        uint32_t rb[9] = {};
        if constexpr (Pop<T>::kRounds) rand9(seed_key(*p.seed_out ^ 0x2545F491u) + n, rb);
#pragma unroll
        for (int j = 0; j < 9; ++j) Pop<T>::std_(Fo + j * N, n, d[j], rb[j]);
    }
}

// Band velocities of a freshly staged FP64 AoS state; the staged state
// carries no pending forcing.
__global__ void ibm_stage_uv_kernel(const KParams p, const IbmParams q, const double* __restrict__ aos) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= q.nb) return;
    const uint32_t n = q.band_node[b];
    double u = 0.0, v = 0.0;
    if (!(p.flags[n] & FLAG_SOLID)) {
        double f[9], rho;
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = aos[(size_t)n * 9 + j];
        macros_ref(f, rho, u, v);
    }
    q.uv[2 * b] = u;
    q.uv[2 * b + 1] = v;
    q.F[2 * b] = 0.0;
    q.F[2 * b + 1] = 0.0;
}

// Point pt: velocity from the band velocities in the driver's y-major
// stencil order (src/airfoil_ibm.cpp:124-147) and the no-slip force
// (src/ibm.hpp:139-149) into q.lag_out = [U | V | FX | FY].  Solid stencil
// nodes, which the reference skips, hold a zero velocity; adding +0 leaves
// every partial sum unchanged bit for bit (a sum that starts at +0 under
// round-to-nearest is never -0).
// One warp per point: lane k loads stencil entry k (a stencil has at most
// 5 x 5 = 25 entries) and forms its products in parallel; lane 0 then adds
// them in stencil order, so the sum is the reference's sequential one.
template <class R>
__global__ void ibm_interp_kernel(const IbmParams q) {
    const int pt = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (pt >= q.np) return;  // whole warps exit together
    const int k0 = q.ip_start[pt], cnt = q.ip_start[pt + 1] - k0;
    R pu = R(0), pv = R(0);
    if (lane < cnt) {
        const int b = q.ip_band[k0 + lane];
        const R w = R(q.ip_w[k0 + lane]);
        if constexpr (std::is_same<R, double>::value) {
            pu = __dmul_rn(q.uv[2 * b], w);
            pv = __dmul_rn(q.uv[2 * b + 1], w);
        } else {
            pu = float(q.uv[2 * b]) * w;
            pv = float(q.uv[2 * b + 1]) * w;
        }
    }
    R U = R(0), V = R(0);
    for (int k = 0; k < cnt; ++k) {
        const R a = __shfl_sync(0xffffffffu, pu, k), c = __shfl_sync(0xffffffffu, pv, k);
        if constexpr (std::is_same<R, double>::value) {
            U = __dadd_rn(U, a);
            V = __dadd_rn(V, c);
        } else {
            U = __fadd_rn(U, a);
            V = __fadd_rn(V, c);
        }
    }
    if (lane == 0) {
        q.lag_out[pt] = double(U);
        q.lag_out[q.np + pt] = double(V);
        q.lag_out[2 * q.np + pt] = __ddiv_rn(__dsub_rn(q.uwx, double(U)), q.dt);
        q.lag_out[3 * q.np + pt] = __ddiv_rn(__dsub_rn(q.uwy, double(V)), q.dt);
    }
}

// Fields of the reference's frame writers at one downsampled point
// (src/lbm.hpp:609-630 and :728-754 for JSON frames, :860-910 for VTK):
// compute_macros in the reference's order (sequential sums in slot order,
// u = mx / rho; src/lbm_types.hpp:278-288), the temperature as the plain sum
// of g (src/thermal.hpp:55-60) and the speed sqrt(u*u + v*v).  Every
// operation is an explicitly rounded FP64 operation, so nothing is fused and
// the results equal the host writers' on the same state.  With `sanitize`
// the JSON writers' replacements apply: rho < 1e-12 or NaN -> (1, 0, 0),
// NaN u, v, speed -> 0, NaN T -> 1.  Solid points report zeros (T = T_wall).
template <class T, bool TH>
__global__ void frame_kernel(const KParams p, const FOut o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= o.nxd || j >= o.nyd) return;
    const int x = i * o.ds, y = j * o.ds;
    const size_t n = (size_t)y * p.nx + x;
    const size_t k = (size_t)j * o.nxd + i;
    const uint32_t fl = p.flags[n];
    const bool solid = (fl & FLAG_SOLID) != 0;
    double rho = 0.0, u = 0.0, v = 0.0, vel = 0.0, Tn = o.T_wall;
    if (!solid) {
        double f[9], g[9];
        state_fp64<T, TH>(p, x, y, fl, f, g);
        macros_ref(f, rho, u, v);
        Tn = 0.0;
        if (TH) {
#pragma unroll
            for (int q = 0; q < 9; ++q) Tn = __dadd_rn(Tn, g[q]);
        }
        if (o.sanitize) {
            if (rho < 1e-12 || isnan(rho)) {
                rho = 1.0;
                u = 0.0;
                v = 0.0;
            }
            if (isnan(u)) u = 0.0;
            if (isnan(v)) v = 0.0;
            if (TH && isnan(Tn)) Tn = 1.0;
        }
        vel = __dsqrt_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)));
        if (o.sanitize && isnan(vel)) vel = 0.0;
    }
    o.rho[k] = rho;
    o.u[k] = u;
    o.v[k] = v;
    o.vel[k] = vel;
    o.T[k] = Tn;
    o.obstacle[k] = solid ? 1 : 0;
}

// Vorticity dv/dx - du/dy on the downsampled grid with one-sided
// differences at its edges (src/lbm.hpp:632-653); zero at solid points.
__global__ void frame_omega_kernel(const FOut o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= o.nxd || j >= o.nyd) return;
    const int k = j * o.nxd + i;
    double om = 0.0;
    if (!o.obstacle[k]) {
        const int il = max(0, i - 1), ir = min(o.nxd - 1, i + 1);
        const int jd = max(0, j - 1), ju = min(o.nyd - 1, j + 1);
        const double dvdx = __ddiv_rn(__dsub_rn(o.v[j * o.nxd + ir], o.v[j * o.nxd + il]),
                                      __dmul_rn(2.0, double((ir - il) * o.ds)));
        const double dudy = __ddiv_rn(__dsub_rn(o.u[ju * o.nxd + i], o.u[jd * o.nxd + i]),
                                      __dmul_rn(2.0, double((ju - jd) * o.ds)));
        om = __dsub_rn(dvdx, dudy);
    }
    o.omega[k] = om;
}

template <class T, bool TH>
__global__ void prologue_kernel(const KParams p, const double* __restrict__ fa, const double* __restrict__ ga) {
    using R = typename Pop<T>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const size_t n = (size_t)y * p.nx + x;
    const uint32_t fl = p.flags[n];
    T* Fo = static_cast<T*>(p.fout);
    T* Go = static_cast<T*>(p.gout);
    const size_t N = (size_t)p.N;
    R f[9], g[9];
    if constexpr (std::is_same<T, double>::value) {
        for (int j = 0; j < 9; ++j) f[j] = fa[n * 9 + j];
        if (TH)
            for (int j = 0; j < 9; ++j) g[j] = ga[n * 9 + j];
        if (!(fl & FLAG_SOLID)) collide<R, TH>(p, fl, f, g);
        for (int j = 0; j < 9; ++j) Fo[j * N + n] = f[j];
        if (TH)
            for (int j = 0; j < 9; ++j) Go[j * N + n] = g[j];
    } else {
        // deviations taken in FP64, then collided in the FP32 deviation form
        for (int j = 0; j < 9; ++j) f[j] = float(fa[n * 9 + j] - double(p.shf[j]));
        if (TH)
            for (int j = 0; j < 9; ++j) g[j] = float(ga[n * 9 + j] - double(p.shg[j]));
        if (!(fl & FLAG_SOLID)) collide_dev<TH>(p, fl, f, g);
        uint32_t rb[9] = {};
        const uint32_t skey = seed_key(p.seed_host);
        if constexpr (Pop<T>::kRounds) rand9(skey + (uint32_t)n, rb);
        for (int j = 0; j < 9; ++j) Pop<T>::std_(Fo + j * N, n, f[j], rb[j]);
        if (TH) {
            if constexpr (Pop<T>::kRounds) rand9((skey + (uint32_t)n) ^ 0x6A09E667u, rb);
            for (int j = 0; j < 9; ++j) Pop<T>::std_(Go + j * N, n, g[j], rb[j]);
        }
    }
    pass_seed(p, p.seed_host, x == 0 && y == 0);
}

// Uniform equilibrium state written into the FP64 AoS staging buffers, as
// the drivers' initialisation loops do (every node, solids included).
__global__ void fill_equilibrium_kernel(double* __restrict__ fa, double* __restrict__ ga, long long N, double rho,
                                        double u, double v, double T) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const double ed = double(CXf(i)) * u + double(CYf(i)) * v;
        const double usq = u * u + v * v;
        const double poly = 1.0 + 3.0 * ed + 4.5 * ed * ed - 1.5 * usq;
        fa[n * 9 + i] = wgt(i) * rho * poly;
        if (ga) ga[n * 9 + i] = wgt(i) * T * poly;
    }
}

// FP64 diagnostics over the fluid nodes of the rebuilt reference state:
// total mass, momentum, and the squared velocity change against (and update
// of) the previous velocity field kept in prev_uv (2 floats per node).
template <class T, bool TH>
__global__ void diagnostics_kernel(const KParams p, double* __restrict__ acc, float* __restrict__ prev_uv,
                                   int have_prev) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    double m = 0.0, jx = 0.0, jy = 0.0, du2 = 0.0, u2 = 0.0;
    if (x < p.nx && y < p.ny) {
        const size_t n = (size_t)y * p.nx + x;
        const uint32_t fl = p.flags[n];
        if (!(fl & FLAG_SOLID)) {
            double f[9], g[9];
            state_fp64<T, TH>(p, x, y, fl, f, g);
            double rho = 0.0, mx = 0.0, my = 0.0;
            for (int j = 0; j < 9; ++j) {
                rho += double(f[j]);
                mx += double(f[j]) * CXf(j);
                my += double(f[j]) * CYf(j);
            }
            m = rho;
            jx = mx;
            jy = my;
            const float u = float(mx / rho), v = float(my / rho);
            if (have_prev) {
                const double a = double(u) - prev_uv[2 * n], b = double(v) - prev_uv[2 * n + 1];
                du2 = a * a + b * b;
            }
            u2 = double(u) * u + double(v) * v;
            prev_uv[2 * n] = u;
            prev_uv[2 * n + 1] = v;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, o);
        jx += __shfl_down_sync(0xffffffffu, jx, o);
        jy += __shfl_down_sync(0xffffffffu, jy, o);
        du2 += __shfl_down_sync(0xffffffffu, du2, o);
        u2 += __shfl_down_sync(0xffffffffu, u2, o);
    }
    if (((threadIdx.y * blockDim.x + threadIdx.x) & 31) == 0) {
        atomicAdd(acc + 0, m);
        atomicAdd(acc + 1, jx);
        atomicAdd(acc + 2, jy);
        atomicAdd(acc + 3, du2);
        atomicAdd(acc + 4, u2);
    }
}

// Prologue of a paired solver: the same packed collision as step_pair_block,
// so a re-collided state (parameter change, autotuner restore) rounds exactly
// as the steps do.
template <class T, bool TH>
__global__ void prologue_pair_kernel(const KParams p, const double* __restrict__ fa, const double* __restrict__ ga) {
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x0 >= p.nx || y >= p.ny) return;
    const size_t n0 = (size_t)y * p.nx + x0;
    const uint32_t fla = p.flags[n0], flb = p.flags[n0 + 1];
    const bool oka = !(fla & FLAG_SOLID), okb = !(flb & FLAG_SOLID);
    F2 f[9], g[9];
    const double S = Pop<T>::kS;
    for (int j = 0; j < 9; ++j)
        f[j] = mk2(float((fa[n0 * 9 + j] - double(p.shf[j])) * S), float((fa[(n0 + 1) * 9 + j] - double(p.shf[j])) * S));
    if (TH)
        for (int j = 0; j < 9; ++j)
            g[j] = mk2(float((ga[n0 * 9 + j] - double(p.shg[j])) * S),
                       float((ga[(n0 + 1) * 9 + j] - double(p.shg[j])) * S));
    if (oka || okb) {
        collide_pair_dev<T>(p, fla, flb, oka, okb, f);
        if (TH) thermal_pair_dev<T>(p, oka, okb, f, g);
    }
    T* Fo = static_cast<T*>(p.fout);
    const size_t N = (size_t)p.N;
    uint32_t rb[9] = {};
    const uint32_t key = seed_key(p.seed_host) + (uint32_t)n0;
    if constexpr (Pop<T>::kRounds) rand9(key, rb);
    for (int j = 0; j < 9; ++j) PairStore<T>::st(Fo + j * N, n0, f[j].v.x, f[j].v.y, rb[j]);
    if (TH) {
        T* Go = static_cast<T*>(p.gout);
        if constexpr (Pop<T>::kRounds) rand9(key ^ 0x6A09E667u, rb);
        for (int j = 0; j < 9; ++j) PairStore<T>::st(Go + j * N, n0, g[j].v.x, g[j].v.y, rb[j]);
    }
    pass_seed(p, p.seed_host, x0 == 0 && y == 0);
}

// Deterministic second stage of the force reduction: one block sums the
// per-block partials in a fixed order and appends (fx, fy) to the history.
// Launched with 128 threads: the same fixed-order sum as the fused form, so
// both give the same bits for the same partials.
__global__ void force_reduce_kernel(const double* __restrict__ part, int nslots, double* hist, int cap,
                                    unsigned long long* counter, double* last) {
    __shared__ double w8[8];
    double a, b;
    sum_slots128(part, nslots, threadIdx.x, w8, [] { __syncthreads(); }, a, b);
    if (threadIdx.x == 0) record_forces(hist, cap, counter, last, a, b);
}

// Force reduction of several instances: block b reduces job b.
__global__ void batch_force_reduce_kernel(const ReduceJob* __restrict__ jobs) {
    const ReduceJob j = jobs[blockIdx.x];
    if (j.left && *j.left <= 0) return;  // the instance's budget was spent: no step, no history entry
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < j.nslots; k += blockDim.x) {
        a += j.partials[2 * k];
        b += j.partials[2 * k + 1];
    }
    block_reduce2(a, b);
    if (threadIdx.x == 0) {
        const unsigned long long k = *j.counter;
        if (k < (unsigned long long)j.cap) {
            j.hist[2 * k] = a;
            j.hist[2 * k + 1] = b;
        }
        j.last[0] = a;
        j.last[1] = b;
        *j.counter = k + 1;
    }
}

template <class T>
int launch_batch_t(const KParams* inst, const int2* block_map, int nblocks, int thermal, int bx, int by,
                   cudaStream_t s, int pair) {
    if (nblocks <= 0) return 0;
    dim3 blk(bx, by);
    if (pair) {
        if constexpr (!std::is_same<T, double>::value) {
            if (thermal)
                batch_step_pair_th_kernel<T><<<nblocks, blk, 0, s>>>(inst, block_map);
            else
                batch_step_pair_kernel<T><<<nblocks, blk, 0, s>>>(inst, block_map);
            return (int)cudaGetLastError();
        }
        return (int)cudaErrorInvalidValue;
    }
    if constexpr (sizeof(T) == 2) {
        if (thermal && bx * by <= 256) {
            batch_step_th_kernel<T, 5><<<nblocks, blk, 0, s>>>(inst, block_map);
            return (int)cudaGetLastError();
        }
    }
    if (thermal)
        batch_step_kernel<T, true><<<nblocks, blk, 0, s>>>(inst, block_map);
    else
        batch_step_kernel<T, false><<<nblocks, blk, 0, s>>>(inst, block_map);
    return (int)cudaGetLastError();
}

template <class T>
int launch_step_t(const KParams& p, int bx, int by, cudaStream_t s) {
    if (p.pair) {
        if constexpr (!std::is_same<T, double>::value) {
            dim3 blk(bx, by), grd((p.nx / 2 + bx - 1) / bx, (p.ny + by - 1) / by);
            if (p.thermal)
                step_pair_kernel<T, true><<<grd, blk, 0, s>>>(p);
            else
                step_pair_kernel<T, false><<<grd, blk, 0, s>>>(p);
            return (int)cudaGetLastError();
        }
        return (int)cudaErrorInvalidValue;
    }
    dim3 blk(bx, by), grd((p.nx + bx - 1) / bx, (p.ny + by - 1) / by);
    if constexpr (!std::is_same<T, double>::value) {
        if (p.thermal && bx * by <= 256) {
            step_th_kernel<T, 6><<<grd, blk, 0, s>>>(p);
            return (int)cudaGetLastError();
        }
    }
    if (p.thermal)
        step_kernel<T, true><<<grd, blk, 0, s>>>(p);
    else
        step_kernel<T, false><<<grd, blk, 0, s>>>(p);
    return (int)cudaGetLastError();
}

template <class T>
int launch_readback_t(const KParams& p, const ROut& o, cudaStream_t s) {
    dim3 blk(128, 2), grd((p.nx + 127) / 128, (p.ny + 1) / 2);
    if (p.thermal)
        readback_kernel<T, true><<<grd, blk, 0, s>>>(p, o);
    else
        readback_kernel<T, false><<<grd, blk, 0, s>>>(p, o);
    return (int)cudaGetLastError();
}

template <class T>
int launch_frame_t(const KParams& p, const FOut& o, cudaStream_t s) {
    dim3 blk(64, 4), grd((o.nxd + 63) / 64, (o.nyd + 3) / 4);
    if (p.thermal)
        frame_kernel<T, true><<<grd, blk, 0, s>>>(p, o);
    else
        frame_kernel<T, false><<<grd, blk, 0, s>>>(p, o);
    frame_omega_kernel<<<grd, blk, 0, s>>>(o);
    return (int)cudaGetLastError();
}

template <class T>
int launch_prologue_t(const KParams& p, const double* fa, const double* ga, cudaStream_t s) {
    if (p.pair) {
        if constexpr (!std::is_same<T, double>::value) {
            dim3 blk(128, 2), grd((p.nx / 2 + 127) / 128, (p.ny + 1) / 2);
            if (p.thermal)
                prologue_pair_kernel<T, true><<<grd, blk, 0, s>>>(p, fa, ga);
            else
                prologue_pair_kernel<T, false><<<grd, blk, 0, s>>>(p, fa, nullptr);
            return (int)cudaGetLastError();
        }
        return (int)cudaErrorInvalidValue;
    }
    dim3 blk(128, 2), grd((p.nx + 127) / 128, (p.ny + 1) / 2);
    if (p.thermal)
        prologue_kernel<T, true><<<grd, blk, 0, s>>>(p, fa, ga);
    else
        prologue_kernel<T, false><<<grd, blk, 0, s>>>(p, fa, ga);
    return (int)cudaGetLastError();
}

}  // namespace

int launch_step(int storage, const KParams& p, int bx, int by, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_step_t<float>(p, bx, by, s);
        case ST_FP16: return launch_step_t<__half>(p, bx, by, s);
        case ST_BF16: return launch_step_t<__nv_bfloat16>(p, bx, by, s);
        case ST_FP64: return launch_step_t<double>(p, bx, by, s);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_readback(int storage, const KParams& p, const ROut& o, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_readback_t<float>(p, o, s);
        case ST_FP16: return launch_readback_t<__half>(p, o, s);
        case ST_BF16: return launch_readback_t<__nv_bfloat16>(p, o, s);
        case ST_FP64: return launch_readback_t<double>(p, o, s);
    }
    return (int)cudaErrorInvalidValue;
}

// The band and point kernels are short chains of dependent loads and
// arithmetic over a few thousand threads: one-warp blocks spread them over as
// many SMs as possible.
constexpr int kIbmBlock = 32;

template <class T>
int launch_ibm_band_t(const KParams& p, const IbmParams& q, cudaStream_t s) {
    using R = typename std::conditional<std::is_same<T, double>::value, double, float>::type;
    if (q.nb > 0) ibm_band_kernel<T><<<(q.nb + kIbmBlock - 1) / kIbmBlock, kIbmBlock, 0, s>>>(p, q);
    if (q.np > 0) ibm_interp_kernel<R><<<(q.np + 3) / 4, 128, 0, s>>>(q);  // a warp per point
    return (int)cudaGetLastError();
}

int launch_ibm_after_step(int storage, const KParams& p, const IbmParams& q, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_ibm_band_t<float>(p, q, s);
        case ST_FP16: return launch_ibm_band_t<__half>(p, q, s);
        case ST_BF16: return launch_ibm_band_t<__nv_bfloat16>(p, q, s);
        case ST_FP64: return launch_ibm_band_t<double>(p, q, s);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_ibm_from_stage(int storage, const KParams& p, const IbmParams& q, const double* aos, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (q.nb > 0) ibm_stage_uv_kernel<<<(q.nb + kIbmBlock - 1) / kIbmBlock, kIbmBlock, 0, s>>>(p, q, aos);
    if (q.np > 0) {
        const int g = (q.np + 3) / 4;  // a warp per point
        if (storage == ST_FP64)
            ibm_interp_kernel<double><<<g, 128, 0, s>>>(q);
        else
            ibm_interp_kernel<float><<<g, 128, 0, s>>>(q);
    }
    return (int)cudaGetLastError();
}

int launch_frame(int storage, const KParams& p, const FOut& o, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_frame_t<float>(p, o, s);
        case ST_FP16: return launch_frame_t<__half>(p, o, s);
        case ST_BF16: return launch_frame_t<__nv_bfloat16>(p, o, s);
        case ST_FP64: return launch_frame_t<double>(p, o, s);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_prologue(int storage, const KParams& p, const double* fa, const double* ga, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_prologue_t<float>(p, fa, ga, s);
        case ST_FP16: return launch_prologue_t<__half>(p, fa, ga, s);
        case ST_BF16: return launch_prologue_t<__nv_bfloat16>(p, fa, ga, s);
        case ST_FP64: return launch_prologue_t<double>(p, fa, ga, s);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_batch_step(int storage, const KParams* inst, const int2* block_map, int nblocks, int thermal, int bx,
                      int by, void* stream, int pair) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_batch_t<float>(inst, block_map, nblocks, thermal, bx, by, s, pair);
        case ST_FP16: return launch_batch_t<__half>(inst, block_map, nblocks, thermal, bx, by, s, pair);
        case ST_BF16: return launch_batch_t<__nv_bfloat16>(inst, block_map, nblocks, thermal, bx, by, s, pair);
        case ST_FP64: return launch_batch_t<double>(inst, block_map, nblocks, thermal, bx, by, s, pair);
    }
    return (int)cudaErrorInvalidValue;
}

int launch_batch_force_reduce(const ReduceJob* jobs, int njobs, void* stream) {
    if (njobs <= 0) return 0;
    batch_force_reduce_kernel<<<njobs, 256, 0, static_cast<cudaStream_t>(stream)>>>(jobs);
    return (int)cudaGetLastError();
}

int launch_diagnostics(int storage, const KParams& p, double* acc, float* prev_uv, int have_prev, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dim3 blk(128, 2), grd((p.nx + 127) / 128, (p.ny + 1) / 2);
#define LBM2D_DIAG(T)                                                                        \
    do {                                                                                     \
        if (p.thermal)                                                                       \
            diagnostics_kernel<T, true><<<grd, blk, 0, s>>>(p, acc, prev_uv, have_prev);     \
        else                                                                                 \
            diagnostics_kernel<T, false><<<grd, blk, 0, s>>>(p, acc, prev_uv, have_prev);    \
    } while (0)
    switch (storage) {
        case ST_FP32: LBM2D_DIAG(float); break;
        case ST_FP16: LBM2D_DIAG(__half); break;
        case ST_BF16: LBM2D_DIAG(__nv_bfloat16); break;
        case ST_FP64: LBM2D_DIAG(double); break;
        default: return (int)cudaErrorInvalidValue;
    }
#undef LBM2D_DIAG
    return (int)cudaGetLastError();
}

int launch_fill_equilibrium(double* fa, double* ga, long long N, double rho, double u, double v, double T,
                            void* stream) {
    const int bs = 256;
    fill_equilibrium_kernel<<<(unsigned)((N + bs - 1) / bs), bs, 0, static_cast<cudaStream_t>(stream)>>>(fa, ga, N, rho,
                                                                                                   u, v, T);
    return (int)cudaGetLastError();
}

int launch_force_reduce(const double* partials, int nslots, double* hist, int cap, unsigned long long* counter,
                        double* last, void* stream) {
    force_reduce_kernel<<<1, 128, 0, static_cast<cudaStream_t>(stream)>>>(partials, nslots, hist, cap, counter,
                                                                           last);
    return (int)cudaGetLastError();
}

}  // namespace lbm2d
