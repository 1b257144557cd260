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
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "lbm2d_internal.h"

namespace lbm2d {
namespace {

// D2Q9 lattice, direction order of src/lbm_types.hpp:41-55.
__host__ __device__ constexpr int CXf(int i) { return (i == 1 || i == 5 || i == 8) ? 1 : ((i == 3 || i == 6 || i == 7) ? -1 : 0); }
__host__ __device__ constexpr int CYf(int i) { return (i == 2 || i == 5 || i == 6) ? 1 : ((i == 4 || i == 7 || i == 8) ? -1 : 0); }
__host__ __device__ constexpr int BBf(int i) { return i == 0 ? 0 : (i < 5 ? ((i + 1) % 4 + 1) : ((i - 5 + 2) % 4 + 5)); }
static_assert(BBf(1) == 3 && BBf(2) == 4 && BBf(3) == 1 && BBf(4) == 2, "bounce-back map");
static_assert(BBf(5) == 7 && BBf(6) == 8 && BBf(7) == 5 && BBf(8) == 6, "bounce-back map");
__host__ __device__ constexpr double wgt(int i) { return i == 0 ? 4.0 / 9.0 : (i < 5 ? 1.0 / 9.0 : 1.0 / 36.0); }

// ----------------------------------------------------------------- storage formats
template <class T>
struct Pop;
template <>
struct Pop<float> {
    using R = float;
    static __device__ __forceinline__ R ld(const float* __restrict__ p, size_t i, float) { return __ldg(p + i); }
    static __device__ __forceinline__ void st(float* __restrict__ p, size_t i, R v, float) { p[i] = v; }
};
template <>
struct Pop<double> {
    using R = double;
    static __device__ __forceinline__ R ld(const double* __restrict__ p, size_t i, float) { return __ldg(p + i); }
    static __device__ __forceinline__ void st(double* __restrict__ p, size_t i, R v, float) { p[i] = v; }
};
template <>
struct Pop<__half> {
    using R = float;
    static __device__ __forceinline__ R ld(const __half* __restrict__ p, size_t i, float sh) {
        return __half2float(__ldg(p + i)) + sh;
    }
    static __device__ __forceinline__ void st(__half* __restrict__ p, size_t i, R v, float sh) {
        p[i] = __float2half_rn(v - sh);
    }
};
template <>
struct Pop<__nv_bfloat16> {
    using R = float;
    static __device__ __forceinline__ R ld(const __nv_bfloat16* __restrict__ p, size_t i, float sh) {
        return __bfloat162float(__ldg(p + i)) + sh;
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* __restrict__ p, size_t i, R v, float sh) {
        p[i] = __float2bfloat16_rn(v - sh);
    }
};

// Parameters in the compute precision.
template <class R>
__device__ __forceinline__ const Phys<R>& phys(const KParams& p);
template <>
__device__ __forceinline__ const Phys<float>& phys<float>(const KParams& p) { return p.pf; }
template <>
__device__ __forceinline__ const Phys<double>& phys<double>(const KParams& p) { return p.pd; }

// Reciprocal / square root / exponential: hardware approximations (a few
// ulp) in the FP32 path, IEEE in the FP64 path.
template <class R>
struct Fm;
template <>
struct Fm<float> {
    static __device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
    static __device__ __forceinline__ float sqrt(float x) { return x > 0.0f ? x * rsqrtf(x) : 0.0f; }
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
};
template <>
struct Fm<double> {
    static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
};

// ----------------------------------------------------------------- lattice math
// compute_equilibrium, src/lbm_types.hpp:269-273
template <class R>
__device__ __forceinline__ R feq(int i, R rho, R u, R v) {
    R ed = R(CXf(i)) * u + R(CYf(i)) * v;
    R usq = u * u + v * v;
    return R(wgt(i)) * rho * (R(1) + R(3) * ed + R(4.5) * ed * ed - R(1.5) * usq);
}

// compute_macros, src/lbm_types.hpp:278-288
template <class R>
__device__ __forceinline__ void macros(const R f[9], R& rho, R& u, R& v) {
    rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
    R mx = (f[1] - f[3]) + (f[5] - f[6]) + (f[8] - f[7]);
    R my = (f[2] - f[4]) + (f[5] + f[6]) - (f[7] + f[8]);
    const R inv = Fm<R>::rcp(rho);
    u = mx * inv;
    v = my * inv;
}

template <class R>
__device__ __forceinline__ R clamp_rate(R s) { return s < R(0.5) ? R(0.5) : (s > R(1.99) ? R(1.99) : s); }

// ----------------------------------------------------------------- pull + rebuild
template <class T>
__device__ __forceinline__ void pull(const KParams& p, const T* __restrict__ P, const float* sh, int x, int y,
                                     typename Pop<T>::R f[9]) {
    const unsigned nx = (unsigned)p.nx, ny = (unsigned)p.ny;
    const size_t N = (size_t)p.N;
    const unsigned ux = (unsigned)x, uy = (unsigned)y;
    const unsigned xm = ux == 0 ? nx - 1 : ux - 1, xp = ux == nx - 1 ? 0 : ux + 1;
    const unsigned ym = uy == 0 ? ny - 1 : uy - 1, yp = uy == ny - 1 ? 0 : uy + 1;
    const unsigned r0 = uy * nx, rm = ym * nx, rp = yp * nx;  // nx*ny < 2^32 (checked at create)
    // slot j pulls from (x - cx_j, y - cy_j), wrapped; records override the
    // slots whose source is solid or outside the domain.
    f[0] = Pop<T>::ld(P, r0 + ux, sh[0]);
    f[1] = Pop<T>::ld(P + N, r0 + xm, sh[1]);
    f[2] = Pop<T>::ld(P + 2 * N, rm + ux, sh[2]);
    f[3] = Pop<T>::ld(P + 3 * N, r0 + xp, sh[3]);
    f[4] = Pop<T>::ld(P + 4 * N, rp + ux, sh[4]);
    f[5] = Pop<T>::ld(P + 5 * N, rm + xm, sh[5]);
    f[6] = Pop<T>::ld(P + 6 * N, rm + xp, sh[6]);
    f[7] = Pop<T>::ld(P + 7 * N, rp + xp, sh[7]);
    f[8] = Pop<T>::ld(P + 8 * N, rp + xm, sh[8]);
}

// Rebuild the non-regular f slots of a boundary node from its record
// (streaming bounce-back src/lbm.hpp:418-428, :449-452, :470-480 and
// apply_bouzidi_bb :226-288).
template <class T>
__device__ __forceinline__ void fix_f(const KParams& p, const T* __restrict__ P, int x, int y, uint32_t rec,
                                   typename Pop<T>::R f[9]) {
    using R = typename Pop<T>::R;
    const uint32_t types = p.rec_info[rec] & 0x3FFFFu;
    if (types == 0) return;
    const size_t N = (size_t)p.N;
    const size_t n = (size_t)y * p.nx + x;
    R own[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) own[j] = Pop<T>::ld(P + j * N, n, p.shf[j]);
    R rho, u, v;
    macros(own, rho, u, v);
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const uint32_t t = (types >> (2 * j)) & 3u;
        if (t == SLOT_SIMPLE_BB) {
            f[j] = own[BBf(j)];
        } else if (t == SLOT_ZERO) {
            f[j] = R(0);
        } else if (t == SLOT_INTERP) {
            const int i = BBf(j);  // the reference's link direction (node -> solid)
            const R q = R(p.rec_q[(size_t)rec * 9 + j]);
            R uwx = R(0), uwy = R(0);
            if (p.moving_wall) {
                uwx = R(p.rec_uw[((size_t)rec * 9 + j) * 2]);
                uwy = R(p.rec_uw[((size_t)rec * 9 + j) * 2 + 1]);
            }
            const R ed = R(CXf(i)) * uwx + R(CYf(i)) * uwy;
            R fbb;
            if (!p.interp_classic) {
                // Mei (1999) / Filippova-Hanel (1998), src/lbm.hpp:234-256
                fbb = q * feq<R>(i, rho, uwx, uwy) + (R(1) - q) * own[i] +
                      (R(2) * q - R(1)) * R(wgt(i)) * rho * ed * R(3);
            } else {
                // classic Bouzidi (2001), src/lbm.hpp:257-273, + Ladd :276-285
                if (q < R(0.5)) {
                    const int sx = x - CXf(i), sy = y - CYf(i);
                    R fsrc = own[i];
                    if (sx >= 0 && sx < p.nx && sy >= 0 && sy < p.ny)
                        fsrc = Pop<T>::ld(P + i * N, (size_t)sy * p.nx + sx, p.shf[i]);
                    fbb = R(2) * q * own[i] + (R(1) - R(2) * q) * fsrc;
                } else {
                    const R inv2q = R(1) / (R(2) * q);
                    fbb = inv2q * own[i] + (R(1) - inv2q) * own[j];
                }
                if (p.moving_wall) fbb -= R(2) * R(wgt(i)) * rho * ed * R(3);
            }
            f[j] = fbb;
        }
    }
}

template <class T>
__device__ __forceinline__ void fix_g(const KParams& p, const T* __restrict__ G, int x, int y, uint32_t rec,
                                   typename Pop<T>::R g[9]) {
    using R = typename Pop<T>::R;
    const uint32_t m = (p.rec_info[rec] >> REC_GBB_SHIFT) & 0x1FFu;
    if (m == 0) return;
    const size_t N = (size_t)p.N;
    const size_t n = (size_t)y * p.nx + x;
    R own[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) own[j] = Pop<T>::ld(G + j * N, n, p.shg[j]);
#pragma unroll
    for (int j = 0; j < 9; ++j)
        if (m & (1u << j)) g[j] = own[BBf(j)];  // adiabatic bounce-back, src/lbm.hpp:512-520
}

// Zou/He velocity inlet on one node, src/lbm.hpp:21-34 / :40-58
template <class R>
__device__ __forceinline__ void zou_he(R f[9], R uin) {
    R rho = (f[0] + f[2] + f[4] + R(2) * (f[3] + f[6] + f[7])) / (R(1) - uin);
    f[1] = f[3] + R(2.0 / 3.0) * rho * uin;
    f[5] = f[7] + R(1.0 / 6.0) * rho * uin;
    f[8] = f[6] + R(1.0 / 6.0) * rho * uin;
}

// The reference's state after streaming, boundary conditions and (optionally)
// a driver thermal pass, for node (x, y).  f/g hold it on return.
template <class T, bool TH>
__device__ __forceinline__ void build_state(const KParams& p, int x, int y, uint32_t fl, typename Pop<T>::R f[9],
                                            typename Pop<T>::R g[9]) {
    using R = typename Pop<T>::R;
    const T* __restrict__ Pf = static_cast<const T*>(p.fin);
    const bool outflow_col = (p.bc_kind == BC_INFLOW || p.bc_kind == BC_STEP) && x == p.nx - 1;
    // zero-gradient outlet: column NX-1 takes NX-2's post-stream state (src/lbm.hpp:63-73)
    const int sx = outflow_col ? x - 1 : x;
    const uint32_t sfl = outflow_col ? __ldg(p.flags + (size_t)y * p.nx + sx) : fl;
    if (sfl & FLAG_SOLID) {
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = R(0);
    } else {
        pull<T>(p, Pf, p.shf, sx, y, f);
        if (sfl & FLAG_BOUNDARY) fix_f<T>(p, Pf, sx, y, sfl >> 2, f);
    }
    if (TH) {
        const T* __restrict__ Pg = static_cast<const T*>(p.gin);
        if (fl & FLAG_SOLID) {
#pragma unroll
            for (int j = 0; j < 9; ++j) g[j] = R(0);
        } else {
            pull<T>(p, Pg, p.shg, x, y, g);
            if (fl & FLAG_BOUNDARY) fix_g<T>(p, Pg, x, y, fl >> 2, g);
        }
    }
    // boundary conditions, src/lbm.hpp:531-540
    if (p.bc_kind == BC_LID) {
        if (y == p.ny - 1) {  // enforce_lid :110-120 (corner nodes included)
            R rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8];
            const R ul = phys<R>(p).u_bc;
#pragma unroll
            for (int i = 0; i < 9; ++i) f[i] = feq<R>(i, rho, ul, R(0));
        }
    } else if (p.bc_kind == BC_INFLOW) {
        if (x == 0) zou_he<R>(f, phys<R>(p).u_bc);
    } else if (p.bc_kind == BC_STEP) {
        const int hs = p.ny / 3;
        if (x == 0 && y >= hs && !(fl & FLAG_SOLID)) {
            const R yy = R(y - hs), h = R(p.ny - 1 - hs);
            zou_he<R>(f, phys<R>(p).u_bc * R(4) * yy * (h - yy) / (h * h));
        }
    }
    if (TH && p.hook_kind == 1) {
        // src/thermal_cavity.cpp:168-204: Dirichlet columns, then adiabatic rows
        if ((x == 1 || x == p.nx - 2) && y >= 1 && y <= p.ny - 2) {
            const R Tw = x == p.nx - 2 ? phys<R>(p).hook_b : phys<R>(p).hook_a;
            R rho, u, v;
            macros(f, rho, u, v);
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = feq<R>(i, Tw, u, v);
        }
        if ((y == 1 || y == p.ny - 2) && x >= 1 && x <= p.nx - 2) {
            g[1] = g[3];
            g[2] = g[4];
            g[5] = g[7];
            g[6] = g[8];
        }
    } else if (TH && p.hook_kind == 2) {
        if (fl & FLAG_SOLID) {  // src/heated_cylinder.cpp:156-164
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = R(wgt(i)) * phys<R>(p).hook_a;
        }
    }
}

template <class R>
__device__ __forceinline__ R wall_distance(const KParams& p, uint32_t fl) {
    if (fl & FLAG_BOUNDARY) return R(p.rec_wd[fl >> 2]);
    const uint32_t d = fl >> 2;
    if (d == WD_UNREACHED) return R(1e9);
    if (d < (1u << 23)) return R(__uint_as_float(0x4B000000u | d) - 8388608.0f);  // exact integer
    return R(d);
}

// Collision of one fluid node: src/lbm.hpp:300-354 (mrt_collide :128-218,
// LES :158-182 with y+ :317-325, body force :327-331) and the thermal
// collision with Boussinesq/Guo forcing :357-397 (src/thermal.hpp:25-52).
template <class R, bool TH>
__device__ __forceinline__ void collide(const KParams& p, uint32_t fl, R f[9], R g[9]) {
    const Phys<R>& q = phys<R>(p);
    R rho, u, v;
    macros(f, rho, u, v);
    if (!(rho == rho) || rho == R(0)) atomicOr(p.nan_flag, 1u);
    if (p.collision == 0) {
        const R f0 = f[0], f1 = f[1], f2 = f[2], f3 = f[3], f4 = f[4];
        const R f5 = f[5], f6 = f[6], f7 = f[7], f8 = f[8];
        const R sd = f5 + f6 + f7 + f8, sa = f1 + f2 + f3 + f4;
        R me = R(-4) * f0 - sa + R(2) * sd;
        R meps = R(4) * f0 - R(2) * sa + sd;
        R mpxx = f1 - f2 + f3 - f4;
        R mpxy = f5 - f6 + f7 - f8;
        const R jx = rho * u, jy = rho * v;
        const R usq = u * u + v * v;
        const R e_eq = R(-2) * rho + R(3) * rho * usq;
        const R eps_eq = rho - R(3) * rho * usq;
        const R pxx_eq = rho * (u * u - v * v);
        const R pxy_eq = rho * u * v;
        R s_eff = q.s_shear;
        if (p.les) {
            // Smagorinsky with Van Driest damping (src/lbm.hpp:158-182, y+ :317-325);
            // the damped branch always applies when y+ > 0
            R csq = q.cs_sq;
            if (q.nu > R(0)) {
                const R wd = wall_distance<R>(p, fl);
                const R yp = wd * Fm<R>::sqrt(usq + R(1e-12)) * q.inv_nu;
                if (yp > R(0)) {
                    const R cd = q.cs * (R(1) - Fm<R>::exp(-yp * R(1.0 / 26.0)));
                    csq = cd * cd;
                }
            }
            const R a = mpxx - pxx_eq, b = mpxy - pxy_eq;
            const R Q = Fm<R>::sqrt(R(2) * (a * a + b * b));
            const R A = R(4.5) * csq * Q * Fm<R>::rcp(rho);
            const R te2 = q.tau + Fm<R>::sqrt(q.tau * q.tau + R(4) * A);  // 2 * tau_eff
            s_eff = clamp_rate<R>(R(2) * Fm<R>::rcp(te2));
        }
        me -= q.s_bulk * (me - e_eq);
        meps -= q.s_bulk * (meps - eps_eq);
        // MRTParams::from_tau fixes s_normal = 1 (src/lbm_types.hpp:75): the
        // energy-flux moments relax exactly to their equilibrium -j
        const R mqx = -jx, mqy = -jy;
        mpxx -= s_eff * (mpxx - pxx_eq);
        mpxy -= s_eff * (mpxy - pxy_eq);
        // closed-form inverse transform (src/lbm.hpp:193-217), common terms shared
        const R a0 = R(1.0 / 9.0) * rho;
        const R ax = a0 - R(1.0 / 36.0) * me - R(1.0 / 18.0) * meps;  // axial base
        const R ad = a0 + R(1.0 / 18.0) * me + R(1.0 / 36.0) * meps;  // diagonal base
        const R hx = R(1.0 / 6.0) * (jx - mqx);
        const R hy = R(1.0 / 6.0) * (jy - mqy);
        const R dx = R(1.0 / 6.0) * jx + R(1.0 / 12.0) * mqx;
        const R dy = R(1.0 / 6.0) * jy + R(1.0 / 12.0) * mqy;
        const R px = R(0.25) * mpxx, py = R(0.25) * mpxy;
        f[0] = a0 - R(1.0 / 9.0) * me + R(1.0 / 9.0) * meps;
        f[1] = ax + hx + px;
        f[2] = ax + hy - px;
        f[3] = ax - hx + px;
        f[4] = ax - hy - px;
        f[5] = ad + dx + dy + py;
        f[6] = ad - dx + dy - py;
        f[7] = ad - dx - dy + py;
        f[8] = ad + dx - dy - py;
    } else {
        const R it = q.inv_tau;
#pragma unroll
        for (int i = 0; i < 9; ++i) f[i] -= it * (f[i] - feq<R>(i, rho, u, v));
    }
    if (q.Fscale != R(0)) {
        const R F = q.Fscale;
        const R fa = R(1.0 / 9.0) * F, fd = R(1.0 / 36.0) * F;
        f[1] += fa;
        f[3] -= fa;
        f[5] += fd;
        f[6] -= fd;
        f[7] -= fd;
        f[8] += fd;
    }
    if (TH) {
        R rho2, u2, v2;
        macros(f, rho2, u2, v2);
        const R T = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7] + g[8];
        const R om = q.omega_k;
#pragma unroll
        for (int i = 0; i < 9; ++i) g[i] -= om * (g[i] - feq<R>(i, T, u2, v2));
        if (q.beta > R(0) && q.g_buoy != R(0)) {
            const R fyb = -q.beta * (T - q.T_ref) * q.g_buoy;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const R eu = R(CXf(i)) * u2 + R(CYf(i)) * v2;
                const R Fd = R(CYf(i)) * fyb;
                f[i] += R(wgt(i)) * (R(3) * Fd + R(9) * eu * Fd);
            }
        }
    }
}

__device__ __forceinline__ void block_reduce2(double& a, double& b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __shared__ double sa[32], sb[32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    if ((tid & 31) == 0) {
        sa[tid >> 5] = a;
        sb[tid >> 5] = b;
    }
    __syncthreads();
    if (tid < 32) {
        a = tid < nw ? sa[tid] : 0.0;
        b = tid < nw ? sb[tid] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
}

// ----------------------------------------------------------------- kernels
// One step of the block (bxi, byi) of an instance whose block grid is gx wide.
template <class T, bool TH>
__device__ __forceinline__ void step_block(const KParams& p, int bxi, int byi, int gx) {
    using R = typename Pop<T>::R;
    const int x = bxi * blockDim.x + threadIdx.x;
    const int y = byi * blockDim.y + threadIdx.y;
    R fxs = R(0), fys = R(0);
    if (x < p.nx && y < p.ny) {
        const unsigned n = (unsigned)y * (unsigned)p.nx + (unsigned)x;
        const uint32_t fl = __ldg(p.flags + n);
        R f[9], g[9];
        build_state<T, TH>(p, x, y, fl, f, g);
        if (!(fl & FLAG_SOLID)) {
            if (fl & FLAG_BOUNDARY) {
                // momentum exchange of this node's links (src/lbm.hpp:565-577)
                const uint32_t fm = p.rec_force[fl >> 2];
#pragma unroll
                for (int j = 1; j < 9; ++j)
                    if (fm & (1u << j)) {
                        fxs -= R(CXf(j)) * R(2) * f[j];
                        fys -= R(CYf(j)) * R(2) * f[j];
                    }
            }
            collide<R, TH>(p, fl, f, g);
        }
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        const size_t N = (size_t)p.N;
        if (!((fl & FLAG_SOLID) && p.skip_settled_solids && x > 0 && x < p.nx - 1 && y < p.ny - 1)) {
#pragma unroll
            for (int j = 0; j < 9; ++j) Pop<T>::st(Fo + j * N, n, f[j], p.shf[j]);
            if (TH) {
                T* __restrict__ Go = static_cast<T*>(p.gout);
#pragma unroll
                for (int j = 0; j < 9; ++j) Pop<T>::st(Go + j * N, n, g[j], p.shg[j]);
            }
        }
    }
    if (p.block_slot) {
        const int base = p.block_slot[byi * gx + bxi];
        if (base >= 0) {  // uniform per block; no barrier: one slot per warp
            // Warp sum in the compute precision (FP32 per-node terms carry FP32
            // rounding already; the FP64 variant stays FP64), only in warps that
            // hold a force node; the cross-warp sum is FP64.
            R a = fxs, b = fys;
            if (__any_sync(0xffffffffu, a != R(0) || b != R(0))) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    a += __shfl_down_sync(0xffffffffu, a, o);
                    b += __shfl_down_sync(0xffffffffu, b, o);
                }
            }
            const int tid = threadIdx.y * blockDim.x + threadIdx.x;
            if ((tid & 31) == 0) {
                const int slot = base + (tid >> 5);
                p.partials[2 * slot] = double(a);
                p.partials[2 * slot + 1] = double(b);
            }
        }
    }
}

// ----------------------------------------------------------------- paired nodes
// A thread owns two x-neighbours (x0, x0+1) with x0 even (nx even).  The
// reference state of each node is rebuilt with the same per-node functions
// as above; the collision runs on both nodes at once with Blackwell's packed
// FP32x2 arithmetic (one FFMA2/FADD2/FMUL2 per operation pair) and the
// populations are written as 8-byte (FP32) or 4-byte (FP16/BF16) pairs.
struct F2 {
    float2 v;
};
__device__ __forceinline__ F2 mk2(float a, float b) { return {make_float2(a, b)}; }
__device__ __forceinline__ F2 sp2(float s) { return {make_float2(s, s)}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return {__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)}; }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 rcp2(F2 a) { return mk2(__fdividef(1.0f, a.v.x), __fdividef(1.0f, a.v.y)); }
__device__ __forceinline__ F2 sqrt2(F2 a) { return mk2(Fm<float>::sqrt(a.v.x), Fm<float>::sqrt(a.v.y)); }

// Same operator as collide<float, false> on two nodes; lane k is collided
// only when fluid_k (a solid lane keeps its value).
__device__ __forceinline__ void collide_pair(const KParams& p, uint32_t fla, uint32_t flb, bool fa_ok, bool fb_ok,
                                             F2 f[9]) {
    const Phys<float>& q = p.pf;
    const F2 rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
    const F2 mx = (f[1] - f[3]) + (f[5] - f[6]) + (f[8] - f[7]);
    const F2 my = (f[2] - f[4]) + (f[5] + f[6]) - (f[7] + f[8]);
    const F2 inv = rcp2(rho);
    const F2 u = mx * inv, v = my * inv;
    if ((fa_ok && (!(rho.v.x == rho.v.x) || rho.v.x == 0.0f)) || (fb_ok && (!(rho.v.y == rho.v.y) || rho.v.y == 0.0f)))
        atomicOr(p.nan_flag, 1u);
    F2 o[9];
    if (p.collision == 0) {
        const F2 sd = (f[5] + f[6]) + (f[7] + f[8]), sa = (f[1] + f[2]) + (f[3] + f[4]);
        F2 me = fma2(sp2(2.0f), sd, fma2(sp2(-4.0f), f[0], sp2(0.0f) - sa));
        F2 meps = fma2(sp2(4.0f), f[0], sd - sp2(2.0f) * sa);
        F2 mpxx = (f[1] - f[2]) + (f[3] - f[4]);
        F2 mpxy = (f[5] - f[6]) + (f[7] - f[8]);
        const F2 jx = rho * u, jy = rho * v;
        const F2 usq = fma2(u, u, v * v);
        const F2 r3u = sp2(3.0f) * rho * usq;
        const F2 e_eq = fma2(sp2(-2.0f), rho, r3u);
        const F2 eps_eq = rho - r3u;
        const F2 pxx_eq = rho * (u * u - v * v);
        const F2 pxy_eq = jx * v;
        F2 s_eff = sp2(q.s_shear);
        if (p.les) {
            F2 csq = sp2(q.cs_sq);
            if (q.nu > 0.0f) {
                const F2 wd = mk2(wall_distance<float>(p, fla), wall_distance<float>(p, flb));
                const F2 yp = wd * sqrt2(usq + sp2(1e-12f)) * sp2(q.inv_nu);
                const float dxa = yp.v.x > 0.0f ? q.cs * (1.0f - __expf(-yp.v.x * (1.0f / 26.0f))) : 0.0f;
                const float dxb = yp.v.y > 0.0f ? q.cs * (1.0f - __expf(-yp.v.y * (1.0f / 26.0f))) : 0.0f;
                csq = mk2(yp.v.x > 0.0f ? dxa * dxa : q.cs_sq, yp.v.y > 0.0f ? dxb * dxb : q.cs_sq);
            }
            const F2 a = mpxx - pxx_eq, b = mpxy - pxy_eq;
            const F2 Q = sqrt2(sp2(2.0f) * fma2(a, a, b * b));
            const F2 A = sp2(4.5f) * csq * Q * inv;
            const F2 te2 = sp2(q.tau) + sqrt2(fma2(sp2(q.tau), sp2(q.tau), sp2(4.0f) * A));
            const F2 s2 = sp2(2.0f) * rcp2(te2);
            s_eff = mk2(clamp_rate<float>(s2.v.x), clamp_rate<float>(s2.v.y));
        }
        const F2 sb = sp2(q.s_bulk);
        me = me - sb * (me - e_eq);
        meps = meps - sb * (meps - eps_eq);
        mpxx = mpxx - s_eff * (mpxx - pxx_eq);
        mpxy = mpxy - s_eff * (mpxy - pxy_eq);
        // s_normal = 1: the energy-flux moments relax to -j (see collide)
        const F2 a0 = sp2(1.0f / 9.0f) * rho;
        const F2 ax = a0 - sp2(1.0f / 36.0f) * me - sp2(1.0f / 18.0f) * meps;
        const F2 ad = fma2(sp2(1.0f / 18.0f), me, fma2(sp2(1.0f / 36.0f), meps, a0));
        const F2 hx = sp2(1.0f / 3.0f) * jx, hy = sp2(1.0f / 3.0f) * jy;  // (j - q)/6 with q = -j
        const F2 dx = sp2(1.0f / 12.0f) * jx, dy = sp2(1.0f / 12.0f) * jy;  // j/6 + q/12 with q = -j
        const F2 px = sp2(0.25f) * mpxx, py = sp2(0.25f) * mpxy;
        o[0] = a0 - sp2(1.0f / 9.0f) * (me - meps);
        o[1] = ax + hx + px;
        o[2] = ax + hy - px;
        o[3] = ax - hx + px;
        o[4] = ax - hy - px;
        o[5] = ad + dx + dy + py;
        o[6] = ad - dx + dy - py;
        o[7] = ad - dx - dy + py;
        o[8] = ad + dx - dy - py;
    } else {
        const F2 it = sp2(q.inv_tau), usq = fma2(u, u, v * v);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const F2 ed = sp2(float(CXf(i))) * u + sp2(float(CYf(i))) * v;
            const F2 poly = fma2(sp2(4.5f) * ed, ed, fma2(sp2(3.0f), ed, sp2(1.0f))) - sp2(1.5f) * usq;
            const F2 fe = sp2(float(wgt(i))) * rho * poly;
            o[i] = f[i] - it * (f[i] - fe);
        }
    }
    if (q.Fscale != 0.0f) {
        const F2 fa = sp2((1.0f / 9.0f) * q.Fscale), fd = sp2((1.0f / 36.0f) * q.Fscale);
        o[1] = o[1] + fa;
        o[3] = o[3] - fa;
        o[5] = o[5] + fd;
        o[6] = o[6] - fd;
        o[7] = o[7] - fd;
        o[8] = o[8] + fd;
    }
#pragma unroll
    for (int j = 0; j < 9; ++j) f[j] = mk2(fa_ok ? o[j].v.x : f[j].v.x, fb_ok ? o[j].v.y : f[j].v.y);
}

template <class T>
struct PairStore;
template <>
struct PairStore<float> {
    static __device__ __forceinline__ void st(float* p, size_t i, float a, float b, float) {
        *reinterpret_cast<float2*>(p + i) = make_float2(a, b);
    }
};
template <>
struct PairStore<__half> {
    static __device__ __forceinline__ void st(__half* p, size_t i, float a, float b, float sh) {
        *reinterpret_cast<__half2*>(p + i) = __floats2half2_rn(a - sh, b - sh);
    }
};
template <>
struct PairStore<__nv_bfloat16> {
    static __device__ __forceinline__ void st(__nv_bfloat16* p, size_t i, float a, float b, float sh) {
        *reinterpret_cast<__nv_bfloat162*>(p + i) = __floats2bfloat162_rn(a - sh, b - sh);
    }
};

// One step of the paired block (bxi, byi) of an instance whose paired block
// grid is gx wide (non-thermal, FP32/FP16/BF16 storage, nx even).
template <class T>
__device__ __forceinline__ void step_pair_block(const KParams& p, int bxi, int byi, int gx) {
    const int x0 = 2 * (bxi * blockDim.x + threadIdx.x);
    const int y = byi * blockDim.y + threadIdx.y;
    float fxs = 0.0f, fys = 0.0f;
    if (x0 < p.nx && y < p.ny) {
        const unsigned n0 = (unsigned)y * (unsigned)p.nx + (unsigned)x0;
        const uint2 fl = __ldg(reinterpret_cast<const uint2*>(p.flags + n0));
        float fa[9], fb[9], ga[9], gb[9];
        build_state<T, false>(p, x0, y, fl.x, fa, ga);
        build_state<T, false>(p, x0 + 1, y, fl.y, fb, gb);
        const bool oka = !(fl.x & FLAG_SOLID), okb = !(fl.y & FLAG_SOLID);
        if ((fl.x | fl.y) & FLAG_BOUNDARY) {
            // momentum exchange of the nodes' links (src/lbm.hpp:565-577)
            const uint32_t ma = (oka && (fl.x & FLAG_BOUNDARY)) ? p.rec_force[fl.x >> 2] : 0u;
            const uint32_t mb = (okb && (fl.y & FLAG_BOUNDARY)) ? p.rec_force[fl.y >> 2] : 0u;
#pragma unroll
            for (int j = 1; j < 9; ++j) {
                if (ma & (1u << j)) {
                    fxs -= float(CXf(j)) * 2.0f * fa[j];
                    fys -= float(CYf(j)) * 2.0f * fa[j];
                }
                if (mb & (1u << j)) {
                    fxs -= float(CXf(j)) * 2.0f * fb[j];
                    fys -= float(CYf(j)) * 2.0f * fb[j];
                }
            }
        }
        if (oka || okb) {
            F2 f[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) f[j] = mk2(fa[j], fb[j]);
            collide_pair(p, fl.x, fl.y, oka, okb, f);
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                fa[j] = f[j].v.x;
                fb[j] = f[j].v.y;
            }
        }
        const bool settled = p.skip_settled_solids && y < p.ny - 1;
        const bool skip_a = !oka && settled && x0 > 0;
        const bool skip_b = !okb && settled && x0 + 1 < p.nx - 1;
        if (!(skip_a && skip_b)) {
            T* __restrict__ Fo = static_cast<T*>(p.fout);
            const size_t N = (size_t)p.N;
#pragma unroll
            for (int j = 0; j < 9; ++j) PairStore<T>::st(Fo + j * N, n0, fa[j], fb[j], p.shf[j]);
        }
    }
    if (p.block_slot) {
        const int base = p.block_slot[byi * gx + bxi];
        if (base >= 0) {
            float a = fxs, b = fys;
            if (__any_sync(0xffffffffu, a != 0.0f || b != 0.0f)) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    a += __shfl_down_sync(0xffffffffu, a, o);
                    b += __shfl_down_sync(0xffffffffu, b, o);
                }
            }
            const int tid = threadIdx.y * blockDim.x + threadIdx.x;
            if ((tid & 31) == 0) {
                const int slot = base + (tid >> 5);
                p.partials[2 * slot] = double(a);
                p.partials[2 * slot + 1] = double(b);
            }
        }
    }
}

template <class T>
__global__ void __launch_bounds__(512) step_pair_kernel(const KParams p) {
    step_pair_block<T>(p, blockIdx.x, blockIdx.y, gridDim.x);
}

template <class T, bool TH>
__global__ void __launch_bounds__(512) step_kernel(const KParams p) {
    step_block<T, TH>(p, blockIdx.x, blockIdx.y, gridDim.x);
}

// Many independent instances in one launch (the tile-to-instance table):
// instance k owns the launch blocks [block_start[k], block_start[k+1]) and
// walks its own block grid (gx = p.gx blocks wide).  The block finds its
// instance by binary search and stages that instance's parameters in shared
// memory once.
template <class T, bool TH>
__global__ void __launch_bounds__(512) batch_step_kernel(const KParams* __restrict__ inst,
                                                         const int* __restrict__ block_start, int ninst) {
    __shared__ KParams sp;
    __shared__ int s_inst;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int b = blockIdx.x;
    if (tid == 0) {
        int lo = 0, hi = ninst - 1;  // last k with block_start[k] <= b
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (block_start[mid] <= b)
                lo = mid;
            else
                hi = mid - 1;
        }
        s_inst = lo;
    }
    __syncthreads();
    const int k = s_inst;
    {
        const int* src = reinterpret_cast<const int*>(inst + k);
        int* dst = reinterpret_cast<int*>(&sp);
        const int nw = (int)(sizeof(KParams) / sizeof(int));
        for (int w = tid; w < nw; w += blockDim.x * blockDim.y) dst[w] = src[w];
    }
    __syncthreads();
    const int local = b - block_start[k];
    step_block<T, TH>(sp, local % sp.gx, local / sp.gx, sp.gx);
}

template <class T>
__global__ void __launch_bounds__(512) batch_step_pair_kernel(const KParams* __restrict__ inst,
                                                              const int* __restrict__ block_start, int ninst) {
    __shared__ KParams sp;
    __shared__ int s_inst;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int b = blockIdx.x;
    if (tid == 0) {
        int lo = 0, hi = ninst - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (block_start[mid] <= b)
                lo = mid;
            else
                hi = mid - 1;
        }
        s_inst = lo;
    }
    __syncthreads();
    const int k = s_inst;
    {
        const int* src = reinterpret_cast<const int*>(inst + k);
        int* dst = reinterpret_cast<int*>(&sp);
        const int nw = (int)(sizeof(KParams) / sizeof(int));
        for (int w = tid; w < nw; w += blockDim.x * blockDim.y) dst[w] = src[w];
    }
    __syncthreads();
    const int local = b - block_start[k];
    step_pair_block<T>(sp, local % sp.gx, local / sp.gx, sp.gx);
}

template <class T, bool TH>
__global__ void readback_kernel(const KParams p, const ROut o) {
    using R = typename Pop<T>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const size_t n = (size_t)y * p.nx + x;
    const uint32_t fl = p.flags[n];
    R f[9], g[9];
    build_state<T, TH>(p, x, y, fl, f, g);
    if (o.f_aos)
        for (int j = 0; j < 9; ++j) o.f_aos[n * 9 + j] = double(f[j]);
    if (TH && o.g_aos)
        for (int j = 0; j < 9; ++j) o.g_aos[n * 9 + j] = double(g[j]);
    if (o.rho || o.u || o.v) {
        double fd[9];
        for (int j = 0; j < 9; ++j) fd[j] = double(f[j]);
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
        double fx = 0.0, fy = 0.0;
        if (!(fl & FLAG_SOLID) && (fl & FLAG_BOUNDARY)) {
            const uint32_t fm = p.rec_force[fl >> 2];
            for (int i = 0; i < 9; ++i) {  // reference accumulation order (src/lbm.hpp:550-577)
                const int j = BBf(i);
                if (fm & (1u << j)) {
                    fx += double(CXf(i)) * 2.0 * double(f[j]);
                    fy += double(CYf(i)) * 2.0 * double(f[j]);
                }
            }
        }
        o.fx[n] = fx;
        o.fy[n] = fy;
    }
}

template <class T, bool TH>
__global__ void prologue_kernel(const KParams p, const double* __restrict__ fa, const double* __restrict__ ga) {
    using R = typename Pop<T>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.nx || y >= p.ny) return;
    const size_t n = (size_t)y * p.nx + x;
    const uint32_t fl = p.flags[n];
    R f[9], g[9];
    for (int j = 0; j < 9; ++j) f[j] = R(fa[n * 9 + j]);
    if (TH)
        for (int j = 0; j < 9; ++j) g[j] = R(ga[n * 9 + j]);
    if (!(fl & FLAG_SOLID)) collide<R, TH>(p, fl, f, g);
    T* Fo = static_cast<T*>(p.fout);
    const size_t N = (size_t)p.N;
    for (int j = 0; j < 9; ++j) Pop<T>::st(Fo + j * N, n, f[j], p.shf[j]);
    if (TH) {
        T* Go = static_cast<T*>(p.gout);
        for (int j = 0; j < 9; ++j) Pop<T>::st(Go + j * N, n, g[j], p.shg[j]);
    }
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
    using R = typename Pop<T>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    double m = 0.0, jx = 0.0, jy = 0.0, du2 = 0.0, u2 = 0.0;
    if (x < p.nx && y < p.ny) {
        const size_t n = (size_t)y * p.nx + x;
        const uint32_t fl = p.flags[n];
        if (!(fl & FLAG_SOLID)) {
            R f[9], g[9];
            build_state<T, TH>(p, x, y, fl, f, g);
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
template <class T>
__global__ void prologue_pair_kernel(const KParams p, const double* __restrict__ fa) {
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x0 >= p.nx || y >= p.ny) return;
    const size_t n0 = (size_t)y * p.nx + x0;
    const uint32_t fla = p.flags[n0], flb = p.flags[n0 + 1];
    const bool oka = !(fla & FLAG_SOLID), okb = !(flb & FLAG_SOLID);
    F2 f[9];
    for (int j = 0; j < 9; ++j) f[j] = mk2(float(fa[n0 * 9 + j]), float(fa[(n0 + 1) * 9 + j]));
    if (oka || okb) collide_pair(p, fla, flb, oka, okb, f);
    T* Fo = static_cast<T*>(p.fout);
    const size_t N = (size_t)p.N;
    for (int j = 0; j < 9; ++j) PairStore<T>::st(Fo + j * N, n0, f[j].v.x, f[j].v.y, p.shf[j]);
}

// Deterministic second stage of the force reduction: one block sums the
// per-block partials in a fixed order and appends (fx, fy) to the history.
__global__ void force_reduce_kernel(const double* __restrict__ part, int nslots, double* hist, int cap,
                                    unsigned long long* counter, double* last) {
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nslots; k += blockDim.x) {
        a += part[2 * k];
        b += part[2 * k + 1];
    }
    block_reduce2(a, b);
    if (threadIdx.x == 0) {
        const unsigned long long k = *counter;
        if (k < (unsigned long long)cap) {
            hist[2 * k] = a;
            hist[2 * k + 1] = b;
        }
        last[0] = a;
        last[1] = b;
        *counter = k + 1;
    }
}

// Force reduction of several instances: block b reduces job b.
__global__ void batch_force_reduce_kernel(const ReduceJob* __restrict__ jobs) {
    const ReduceJob j = jobs[blockIdx.x];
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
int launch_batch_t(const KParams* inst, const int* block_start, int ninst, int nblocks, int thermal, int bx, int by,
                   cudaStream_t s, int pair) {
    if (nblocks <= 0 || ninst <= 0) return 0;
    dim3 blk(bx, by);
    if (pair) {
        if constexpr (!std::is_same<T, double>::value) {
            batch_step_pair_kernel<T><<<nblocks, blk, 0, s>>>(inst, block_start, ninst);
            return (int)cudaGetLastError();
        }
        return (int)cudaErrorInvalidValue;
    }
    if (thermal)
        batch_step_kernel<T, true><<<nblocks, blk, 0, s>>>(inst, block_start, ninst);
    else
        batch_step_kernel<T, false><<<nblocks, blk, 0, s>>>(inst, block_start, ninst);
    return (int)cudaGetLastError();
}

template <class T>
int launch_step_t(const KParams& p, int bx, int by, cudaStream_t s) {
    if (p.pair) {
        if constexpr (!std::is_same<T, double>::value) {
            dim3 blk(bx, by), grd((p.nx / 2 + bx - 1) / bx, (p.ny + by - 1) / by);
            step_pair_kernel<T><<<grd, blk, 0, s>>>(p);
            return (int)cudaGetLastError();
        }
        return (int)cudaErrorInvalidValue;
    }
    dim3 blk(bx, by), grd((p.nx + bx - 1) / bx, (p.ny + by - 1) / by);
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
int launch_prologue_t(const KParams& p, const double* fa, const double* ga, cudaStream_t s) {
    if (p.pair) {
        if constexpr (!std::is_same<T, double>::value) {
            dim3 blk(128, 2), grd((p.nx / 2 + 127) / 128, (p.ny + 1) / 2);
            prologue_pair_kernel<T><<<grd, blk, 0, s>>>(p, fa);
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

int launch_batch_step(int storage, const KParams* inst, const int* block_start, int ninst, int nblocks, int thermal,
                      int bx, int by, void* stream, int pair) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_batch_t<float>(inst, block_start, ninst, nblocks, thermal, bx, by, s, pair);
        case ST_FP16: return launch_batch_t<__half>(inst, block_start, ninst, nblocks, thermal, bx, by, s, pair);
        case ST_BF16: return launch_batch_t<__nv_bfloat16>(inst, block_start, ninst, nblocks, thermal, bx, by, s, pair);
        case ST_FP64: return launch_batch_t<double>(inst, block_start, ninst, nblocks, thermal, bx, by, s, pair);
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
    force_reduce_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(partials, nslots, hist, cap, counter,
                                                                           last);
    return (int)cudaGetLastError();
}

}  // namespace lbm2d
