// lbm2d_device.cuh -- device functions shared by the step kernels: storage
// formats, lattice math, the pull + rebuild of the reference's post-stream
// state, the MRT/BGK/LES/thermal collision (one node, and two nodes at once
// in packed FP32x2 arithmetic) and the per-block step bodies.
#pragma once
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
// FP32/FP16/BF16 hold shifted deviations d = f - w_i*rho0 (g - w_i*T_ref),
// FP64 holds f itself.  FP16 stores d * 2^12 so that small deviations stay
// clear of the FP16 subnormal range (|d| < 16 fits).  Both are written with STOCHASTIC rounding
// (Blackwell cvt.rs, one 32-bit random word per two values): round-to-nearest
// makes the same rounding error at every node of a near-uniform flow on
// every step, which drifts the conserved moments linearly in time; rounding
// up with probability equal to the discarded fraction leaves the stored
// value unbiased, so the errors stay a zero-mean random walk.
constexpr float kF16Scale = 4096.0f;
constexpr float kF16InvScale = 1.0f / 4096.0f;

// Two FP32 values -> packed FP16x2 / BF16x2 (lo = a, hi = b), rounded
// stochastically with the random bits rb.
__device__ __forceinline__ uint32_t cvt_rs_f16x2(float a, float b, uint32_t rb) {
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(b), "f"(a), "r"(rb));
    return d;
}
__device__ __forceinline__ uint32_t cvt_rs_bf16x2(float a, float b, uint32_t rb) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(b), "f"(a), "r"(rb));
    return d;
}

// ldd/std move the stored DEVIATION (the FP32 compute path works on
// deviations); ld/st move the full population f = deviation + sh (FP64
// stores f itself, sh = 0).
template <class T>
struct Pop;
template <>
struct Pop<float> {
    using R = float;
    static constexpr bool kRounds = false;
    static constexpr float kS = 1.0f, kInvS = 1.0f;  // stored value = deviation * kS
    static __device__ __forceinline__ float ldr(const float* __restrict__ p, size_t i) { return __ldg(p + i); }
    static __device__ __forceinline__ float ldd(const float* __restrict__ p, size_t i) { return __ldg(p + i); }
    static __device__ __forceinline__ void std_(float* __restrict__ p, size_t i, float d, uint32_t) { p[i] = d; }
    static __device__ __forceinline__ R ld(const float* __restrict__ p, size_t i, float sh) { return __ldg(p + i) + sh; }
    static __device__ __forceinline__ void st(float* __restrict__ p, size_t i, R v, float sh, uint32_t) {
        p[i] = v - sh;
    }
};
template <>
struct Pop<double> {
    using R = double;
    static constexpr bool kRounds = false;
    static __device__ __forceinline__ R ld(const double* __restrict__ p, size_t i, float) { return __ldg(p + i); }
    static __device__ __forceinline__ void st(double* __restrict__ p, size_t i, R v, float, uint32_t) { p[i] = v; }
};
template <>
struct Pop<__half> {
    using R = float;
    static constexpr bool kRounds = true;
    static constexpr float kS = kF16Scale, kInvS = kF16InvScale;
    static __device__ __forceinline__ float ldr(const __half* __restrict__ p, size_t i) {
        return __half2float(__ldg(p + i));
    }
    static __device__ __forceinline__ float ldd(const __half* __restrict__ p, size_t i) {
        return __half2float(__ldg(p + i)) * kF16InvScale;
    }
    static __device__ __forceinline__ void std_(__half* __restrict__ p, size_t i, float d, uint32_t rb) {
        const float x = d * kF16Scale;
        p[i] = __ushort_as_half((unsigned short)(cvt_rs_f16x2(x, x, rb) & 0xFFFFu));
    }
    static __device__ __forceinline__ R ld(const __half* __restrict__ p, size_t i, float sh) {
        return fmaf(__half2float(__ldg(p + i)), kF16InvScale, sh);
    }
    static __device__ __forceinline__ void st(__half* __restrict__ p, size_t i, R v, float sh, uint32_t rb) {
        std_(p, i, v - sh, rb);
    }
};
template <>
struct Pop<__nv_bfloat16> {
    using R = float;
    static constexpr bool kRounds = true;
    static constexpr float kS = 1.0f, kInvS = 1.0f;
    static __device__ __forceinline__ float ldr(const __nv_bfloat16* __restrict__ p, size_t i) {
        return __bfloat162float(__ldg(p + i));
    }
    static __device__ __forceinline__ float ldd(const __nv_bfloat16* __restrict__ p, size_t i) {
        return __bfloat162float(__ldg(p + i));
    }
    static __device__ __forceinline__ void std_(__nv_bfloat16* __restrict__ p, size_t i, float d, uint32_t rb) {
        p[i] = __ushort_as_bfloat16((unsigned short)(cvt_rs_bf16x2(d, d, rb) & 0xFFFFu));
    }
    static __device__ __forceinline__ R ld(const __nv_bfloat16* __restrict__ p, size_t i, float sh) {
        return __bfloat162float(__ldg(p + i)) + sh;
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* __restrict__ p, size_t i, R v, float sh, uint32_t rb) {
        std_(p, i, v - sh, rb);
    }
};

// ----------------------------------------------------------------- rounding noise
// Random words for stochastic rounding: the lowbias32 integer hash (C.
// Wellons, 2018) of a per-node key, times nine distinct odd constants.
// Multiplication by an odd constant is a bijection of the 32-bit words, so
// every word is exactly uniform, which is all unbiased rounding needs.  The
// key is node + seed * golden-ratio constant, the seed advancing by one per
// step through the solver's seed words (see seed_of).
__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ void rand9(uint32_t key, uint32_t r[9]) {
    const uint32_t h = lowbias32(key);
    r[0] = h;
    r[1] = h * 0x9E3779B1u;
    r[2] = h * 0x85EBCA77u;
    r[3] = h * 0xC2B2AE3Du;
    r[4] = h * 0x27D4EB2Fu;
    r[5] = h * 0x165667B1u;
    r[6] = h * 0xD3A2646Du;
    r[7] = h * 0xFD7046C5u;
    r[8] = h * 0xB55A4F09u;
}

// Seed of this launch's rounding noise, and the hand-over to the next launch:
// a step kernel reads seed_in and its first thread writes seed_in + 1 to
// seed_out (the solver's two seed words swap roles every step like the
// population buffers, so no launch reads a word that it writes).  A
// prologue has no seed_in and uses seed_host.
__device__ __forceinline__ uint32_t seed_of(const KParams& p) {
    return p.seed_in ? __ldg(p.seed_in) : p.seed_host;
}
__device__ __forceinline__ void pass_seed(const KParams& p, uint32_t s, bool first_thread) {
    if (first_thread && p.seed_out) *p.seed_out = s + 1u;
}
__device__ __forceinline__ uint32_t seed_key(uint32_t s) { return s * 0x9E3779B1u; }

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
// Where a rebuild reads the stored (post-collision) populations: plane j of
// node idx as a full population (the storage shift added back), and the flags
// of node idx.  GlobalSrc reads device memory; the tile pipeline supplies a
// source that serves the staged windows from shared memory.
template <class T>
struct GlobalSrc {
    const T* __restrict__ P;
    size_t N;
    const float* sh;
    const uint32_t* __restrict__ flags;
    __device__ __forceinline__ typename Pop<T>::R ld(int j, unsigned idx) const {
        return Pop<T>::ld(P + (size_t)j * N, idx, sh[j]);
    }
    __device__ __forceinline__ uint32_t flag(unsigned idx) const { return __ldg(flags + idx); }
};

template <class T>
__device__ __forceinline__ GlobalSrc<T> gsrc_f(const KParams& p) {
    return {static_cast<const T*>(p.fin), (size_t)p.N, p.shf, p.flags};
}
template <class T>
__device__ __forceinline__ GlobalSrc<T> gsrc_g(const KParams& p) {
    return {static_cast<const T*>(p.gin), (size_t)p.N, p.shg, p.flags};
}

template <class S, class R>
__device__ __forceinline__ void pull_src(const KParams& p, const S& src, int x, int y, R f[9]) {
    const unsigned nx = (unsigned)p.nx, ny = (unsigned)p.ny;
    const unsigned ux = (unsigned)x, uy = (unsigned)y;
    const unsigned xm = ux == 0 ? nx - 1 : ux - 1, xp = ux == nx - 1 ? 0 : ux + 1;
    const unsigned ym = uy == 0 ? ny - 1 : uy - 1, yp = uy == ny - 1 ? 0 : uy + 1;
    const unsigned r0 = uy * nx, rm = ym * nx, rp = yp * nx;  // nx*ny < 2^32 (checked at create)
    // slot j pulls from (x - cx_j, y - cy_j), wrapped; records override the
    // slots whose source is solid or outside the domain.
    f[0] = src.ld(0, r0 + ux);
    f[1] = src.ld(1, r0 + xm);
    f[2] = src.ld(2, rm + ux);
    f[3] = src.ld(3, r0 + xp);
    f[4] = src.ld(4, rp + ux);
    f[5] = src.ld(5, rm + xm);
    f[6] = src.ld(6, rm + xp);
    f[7] = src.ld(7, rp + xp);
    f[8] = src.ld(8, rp + xm);
}

template <class T>
__device__ __forceinline__ void pull(const KParams& p, const T* __restrict__ P, const float* sh, int x, int y,
                                     typename Pop<T>::R f[9]) {
    pull_src(p, GlobalSrc<T>{P, (size_t)p.N, sh, p.flags}, x, y, f);
}

// Rebuild the non-regular f slots of a boundary node from its record
// (streaming bounce-back src/lbm.hpp:418-428, :449-452, :470-480 and
// apply_bouzidi_bb :226-288).  With LAZY, the node's own stored values are
// read only when a slot bounces back (simple or interpolated): a record with
// "no source" slots alone (inlet and outlet columns) needs none of them.
template <class T, bool LAZY = false, class S>
__device__ __forceinline__ void fix_f_src(const KParams& p, const S& src, int x, int y, uint32_t rec,
                                          typename Pop<T>::R f[9]) {
    using R = typename Pop<T>::R;
    const uint32_t types = p.rec_info[rec] & 0x3FFFFu;
    if (types == 0) return;
    const unsigned n = (unsigned)y * (unsigned)p.nx + (unsigned)x;
    R own[9];
    R rho = R(0), u = R(0), v = R(0);
    if constexpr (LAZY) {
        // bit 0 of each 2-bit code: SIMPLE_BB (01) or ZERO (11); bit 1: INTERP (10) or ZERO
        const uint32_t lo = types & 0x15555u, hi = (types >> 1) & 0x15555u;
        if (lo == hi) {  // "no source" slots only
#pragma unroll
            for (int j = 0; j < 9; ++j)
                if (((types >> (2 * j)) & 3u) == SLOT_ZERO) f[j] = R(0);
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < 9; ++j) own[j] = src.ld(j, n);
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
                        fsrc = src.ld(i, (unsigned)sy * (unsigned)p.nx + (unsigned)sx);
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
__device__ __forceinline__ void fix_f(const KParams& p, const T* __restrict__ P, int x, int y, uint32_t rec,
                                      typename Pop<T>::R f[9]) {
    fix_f_src<T>(p, GlobalSrc<T>{P, (size_t)p.N, p.shf, p.flags}, x, y, rec, f);
}

template <class T, class S>
__device__ __forceinline__ void fix_g_src(const KParams& p, const S& src, int x, int y, uint32_t rec,
                                          typename Pop<T>::R g[9]) {
    using R = typename Pop<T>::R;
    const uint32_t m = (p.rec_info[rec] >> REC_GBB_SHIFT) & 0x1FFu;
    if (m == 0) return;
    const unsigned n = (unsigned)y * (unsigned)p.nx + (unsigned)x;
    R own[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) own[j] = src.ld(j, n);
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

// Boundary conditions of execute_time_step on node (x, y) after streaming,
// src/lbm.hpp:531-540.
template <class R>
__device__ __forceinline__ void apply_bc(const KParams& p, int x, int y, uint32_t fl, R f[9]) {
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
}

// The reference's state after streaming, boundary conditions and (optionally)
// a driver thermal pass, for node (x, y), reading the stored populations
// through sf (f) and sg (g).  f/g hold it on return.
template <class T, bool TH, bool LAZY = false, class SF, class SG>
__device__ __forceinline__ void build_state_src(const KParams& p, const SF& sf, const SG& sg, int x, int y,
                                                uint32_t fl, typename Pop<T>::R f[9], typename Pop<T>::R g[9]) {
    using R = typename Pop<T>::R;
    const bool outflow_col = (p.bc_kind == BC_INFLOW || p.bc_kind == BC_STEP) && x == p.nx - 1;
    // zero-gradient outlet: column NX-1 takes NX-2's post-stream state (src/lbm.hpp:63-73)
    const int sx = outflow_col ? x - 1 : x;
    const uint32_t sfl = outflow_col ? sf.flag((unsigned)y * (unsigned)p.nx + (unsigned)sx) : fl;
    if (sfl & FLAG_SOLID) {
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = R(0);
    } else {
        pull_src(p, sf, sx, y, f);
        if (sfl & FLAG_BOUNDARY) fix_f_src<T, LAZY>(p, sf, sx, y, sfl >> 2, f);
    }
    if (TH) {
        if (fl & FLAG_SOLID) {
#pragma unroll
            for (int j = 0; j < 9; ++j) g[j] = R(0);
        } else {
            pull_src(p, sg, x, y, g);
            if (fl & FLAG_BOUNDARY) fix_g_src<T>(p, sg, x, y, fl >> 2, g);
        }
    }
    apply_bc<R>(p, x, y, fl, f);
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

template <class T, bool TH>
__device__ __forceinline__ void build_state(const KParams& p, int x, int y, uint32_t fl, typename Pop<T>::R f[9],
                                            typename Pop<T>::R g[9]) {
    build_state_src<T, TH>(p, gsrc_f<T>(p), gsrc_g<T>(p), x, y, fl, f, g);
}

// LES wall distance of a fluid node: a boundary node's record holds it; any
// other fluid node's flags are its FP32 bit pattern (bits 0-1 zero).
template <class R>
__device__ __forceinline__ R wall_distance(const KParams& p, uint32_t fl) {
    if (fl & FLAG_BOUNDARY) return R(p.rec_wd[fl >> 2]);
    return R(__uint_as_float(fl));
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

// ----------------------------------------------------------------- deviation form
// The FP32 compute path (FP32/FP16/BF16 storage) keeps every population as
// its deviation d_i = f_i - w_i (g: e_i = g_i - w_i*T_ref) in registers.  A
// deviation is ~10x smaller than f_i, so its FP32 rounding is ~10x finer;
// the density enters as drho = sum d_i, the momentum as the exact moment
// sum c_i d_i (never rebuilt as rho * (m / rho) through an approximate
// reciprocal, which would break momentum conservation by ~1e-7 per step),
// and the body force is folded into the momentum terms of the inverse
// transform before the final rounding instead of being added to the rounded
// populations, where an increment below half an ulp of f_i vanishes.  In
// exact arithmetic every step below equals the full-population step.
//
// Nodes whose post-stream state is more than the plain pull (solid,
// boundary record, a boundary-condition row or column, a thermal hook) are
// rebuilt through build_state on full populations and converted back.
// Boundary-condition rows and columns carry a (possibly empty) boundary
// record (the geometry builder gives them one), so the flags alone mark
// every node of a non-thermal step that needs more than the plain pull.
template <bool TH>
__device__ __forceinline__ bool special_node(const KParams& p, int x, int y, uint32_t fl) {
    if (fl & (FLAG_SOLID | FLAG_BOUNDARY)) return true;
    if (TH && p.hook_kind == 1 && (x == 1 || x == p.nx - 2 || y == 1 || y == p.ny - 2)) return true;
    return false;
}

template <class T>
__device__ __forceinline__ void pull_dev(const KParams& p, const T* __restrict__ P, int x, int y, float d[9]) {
    const unsigned nx = (unsigned)p.nx, ny = (unsigned)p.ny;
    const size_t N = (size_t)p.N;
    const unsigned ux = (unsigned)x, uy = (unsigned)y;
    const unsigned xm = ux == 0 ? nx - 1 : ux - 1, xp = ux == nx - 1 ? 0 : ux + 1;
    const unsigned ym = uy == 0 ? ny - 1 : uy - 1, yp = uy == ny - 1 ? 0 : uy + 1;
    const unsigned r0 = uy * nx, rm = ym * nx, rp = yp * nx;
    d[0] = Pop<T>::ldd(P, r0 + ux);
    d[1] = Pop<T>::ldd(P + N, r0 + xm);
    d[2] = Pop<T>::ldd(P + 2 * N, rm + ux);
    d[3] = Pop<T>::ldd(P + 3 * N, r0 + xp);
    d[4] = Pop<T>::ldd(P + 4 * N, rp + ux);
    d[5] = Pop<T>::ldd(P + 5 * N, rm + xm);
    d[6] = Pop<T>::ldd(P + 6 * N, rm + xp);
    d[7] = Pop<T>::ldd(P + 7 * N, rp + xp);
    d[8] = Pop<T>::ldd(P + 8 * N, rp + xm);
}

// Post-stream state of node (x, y) as deviations; returns true for a special
// node (built on full populations).
template <class T, bool TH>
__device__ __forceinline__ bool build_dev(const KParams& p, int x, int y, uint32_t fl, float d[9], float e[9]) {
    if (!special_node<TH>(p, x, y, fl)) {
        pull_dev<T>(p, static_cast<const T*>(p.fin), x, y, d);
        if (TH) pull_dev<T>(p, static_cast<const T*>(p.gin), x, y, e);
        return false;
    }
    float f[9], g[9];
    build_state<T, TH>(p, x, y, fl, f, g);
#pragma unroll
    for (int j = 0; j < 9; ++j) d[j] = f[j] - p.shf[j];
    if (TH) {
#pragma unroll
        for (int j = 0; j < 9; ++j) e[j] = g[j] - p.shg[j];
    }
    return true;
}

// The paired kernels work in STORAGE units, deviation * kS (FP16: 2^12), so
// loads and stores need no scaling; the scale enters once per node through
// rho and u.
template <class T>
__device__ __forceinline__ void pull_raw(const KParams& p, const T* __restrict__ P, int x, int y, float d[9]) {
    const unsigned nx = (unsigned)p.nx, ny = (unsigned)p.ny;
    const size_t N = (size_t)p.N;
    const unsigned ux = (unsigned)x, uy = (unsigned)y;
    const unsigned xm = ux == 0 ? nx - 1 : ux - 1, xp = ux == nx - 1 ? 0 : ux + 1;
    const unsigned ym = uy == 0 ? ny - 1 : uy - 1, yp = uy == ny - 1 ? 0 : uy + 1;
    const unsigned r0 = uy * nx, rm = ym * nx, rp = yp * nx;
    d[0] = Pop<T>::ldr(P, r0 + ux);
    d[1] = Pop<T>::ldr(P + N, r0 + xm);
    d[2] = Pop<T>::ldr(P + 2 * N, rm + ux);
    d[3] = Pop<T>::ldr(P + 3 * N, r0 + xp);
    d[4] = Pop<T>::ldr(P + 4 * N, rp + ux);
    d[5] = Pop<T>::ldr(P + 5 * N, rm + xm);
    d[6] = Pop<T>::ldr(P + 6 * N, rm + xp);
    d[7] = Pop<T>::ldr(P + 7 * N, rp + xp);
    d[8] = Pop<T>::ldr(P + 8 * N, rp + xm);
}

// build_dev<T, false> in storage units.
template <class T>
__device__ __forceinline__ bool build_dev_s(const KParams& p, int x, int y, uint32_t fl, float d[9]) {
    if (!special_node<false>(p, x, y, fl)) {
        pull_raw<T>(p, static_cast<const T*>(p.fin), x, y, d);
        return false;
    }
    float f[9], g[9];
    build_state<T, false>(p, x, y, fl, f, g);
#pragma unroll
    for (int j = 0; j < 9; ++j) d[j] = (f[j] - p.shf[j]) * Pop<T>::kS;
    return true;
}

// Collision of one fluid node on deviations (same operator as collide<R, TH>).
template <bool TH>
__device__ __forceinline__ void collide_dev(const KParams& p, uint32_t fl, float d[9], float e[9]) {
    const Phys<float>& q = p.pf;
    const float drho = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
    const float mx = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
    const float my = (d[2] - d[4]) + (d[5] + d[6]) - (d[7] + d[8]);
    const float rho = 1.0f + drho;
    if (!(rho == rho) || rho == 0.0f) atomicOr(p.nan_flag, 1u);
    const float inv = Fm<float>::rcp(rho);
    const float u = mx * inv, v = my * inv;
    const float F = q.Fscale;
    if (p.collision == 0) {
        const float sd = (d[5] + d[6]) + (d[7] + d[8]), sa = (d[1] + d[2]) + (d[3] + d[4]);
        float me = fmaf(2.0f, sd, fmaf(-4.0f, d[0], -sa));   // e + 2
        float meps = fmaf(4.0f, d[0], fmaf(-2.0f, sa, sd));  // eps - 1
        float mpxx = (d[1] - d[2]) + (d[3] - d[4]);
        float mpxy = (d[5] - d[6]) + (d[7] - d[8]);
        const float r3u = 3.0f * fmaf(mx, u, my * v);  // 3 rho |u|^2
        const float e_eq = fmaf(-2.0f, drho, r3u);     // e_eq + 2
        const float eps_eq = drho - r3u;               // eps_eq - 1
        const float pxx_eq = fmaf(mx, u, -(my * v));   // rho (u^2 - v^2)
        const float pxy_eq = mx * v;                   // rho u v
        float s_eff = q.s_shear;
        if (p.les) {
            float csq = q.cs_sq;
            if (q.nu > 0.0f) {
                const float wd = wall_distance<float>(p, fl);
                const float yp = wd * Fm<float>::sqrt(fmaf(u, u, v * v) + 1e-12f) * q.inv_nu;
                if (yp > 0.0f) {
                    const float cd = q.cs * (1.0f - Fm<float>::exp(-yp * (1.0f / 26.0f)));
                    csq = cd * cd;
                }
            }
            const float a = mpxx - pxx_eq, b = mpxy - pxy_eq;
            const float Q = Fm<float>::sqrt(2.0f * fmaf(a, a, b * b));
            const float A = 4.5f * csq * Q * inv;
            const float te2 = q.tau + Fm<float>::sqrt(fmaf(q.tau, q.tau, 4.0f * A));
            s_eff = clamp_rate<float>(2.0f * Fm<float>::rcp(te2));
        }
        me -= q.s_bulk * (me - e_eq);
        meps -= q.s_bulk * (meps - eps_eq);
        mpxx -= s_eff * (mpxx - pxx_eq);
        mpxy -= s_eff * (mpxy - pxy_eq);
        // inverse transform with s_normal = 1 (q = -j) and the body force
        // w_i c_xi F folded into the x momentum terms
        const float a0 = (1.0f / 9.0f) * drho;
        const float ax = a0 - (1.0f / 36.0f) * me - (1.0f / 18.0f) * meps;
        const float ad = fmaf(1.0f / 18.0f, me, fmaf(1.0f / 36.0f, meps, a0));
        const float hx = fmaf(1.0f / 3.0f, mx, (1.0f / 9.0f) * F), hy = (1.0f / 3.0f) * my;
        const float dx = fmaf(1.0f / 12.0f, mx, (1.0f / 36.0f) * F), dy = (1.0f / 12.0f) * my;
        const float px = 0.25f * mpxx, py = 0.25f * mpxy;
        d[0] = a0 - (1.0f / 9.0f) * (me - meps);
        d[1] = ax + hx + px;
        d[2] = ax + hy - px;
        d[3] = ax - hx + px;
        d[4] = ax - hy - px;
        d[5] = ad + dx + dy + py;
        d[6] = ad - dx + dy - py;
        d[7] = ad - dx - dy + py;
        d[8] = ad + dx - dy - py;
    } else {
        // BGK: f_eq - w = w (drho + 3 c.j + rho (4.5 (c.u)^2 - 1.5 |u|^2))
        const float it = q.inv_tau, usq = fmaf(u, u, v * v);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float cj = float(CXf(i)) * mx + float(CYf(i)) * my;
            const float ed = float(CXf(i)) * u + float(CYf(i)) * v;
            const float fe = float(wgt(i)) * (fmaf(3.0f, cj, drho) + rho * fmaf(4.5f * ed, ed, -1.5f * usq));
            d[i] -= it * (d[i] - fe);
        }
        if (F != 0.0f) {
            const float fa = (1.0f / 9.0f) * F, fd = (1.0f / 36.0f) * F;
            d[1] += fa;
            d[3] -= fa;
            d[5] += fd;
            d[6] -= fd;
            d[7] -= fd;
            d[8] += fd;
        }
    }
    if (TH) {
        // thermal DDF on deviations: T = T_ref + dT, u from the post-collision f
        const float drho2 = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
        const float mx2 = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
        const float my2 = (d[2] - d[4]) + (d[5] + d[6]) - (d[7] + d[8]);
        const float inv2 = Fm<float>::rcp(1.0f + drho2);
        const float u2 = mx2 * inv2, v2 = my2 * inv2, usq2 = fmaf(u2, u2, v2 * v2);
        const float dT = ((e[0] + e[1]) + (e[2] + e[3])) + ((e[4] + e[5]) + (e[6] + e[7])) + e[8];
        const float T = q.T_ref + dT;
        const float om = q.omega_k;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float ed = float(CXf(i)) * u2 + float(CYf(i)) * v2;
            const float ge = float(wgt(i)) * fmaf(T, fmaf(4.5f * ed, ed, fmaf(3.0f, ed, -1.5f * usq2)), dT);
            e[i] -= om * (e[i] - ge);
        }
        if (q.beta > 0.0f && q.g_buoy != 0.0f) {
            const float fyb = -q.beta * dT * q.g_buoy;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const float eu = float(CXf(i)) * u2 + float(CYf(i)) * v2;
                const float Fd = float(CYf(i)) * fyb;
                d[i] += float(wgt(i)) * (3.0f * Fd + 9.0f * eu * Fd);
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

// Second stage of the drag/lift reduction in a fixed order that does not
// depend on the reducing block's shape: 128 lanes, lane t adds slots t,
// t + 128, ... in order; each of the four warps folds its lanes with the same
// shuffle tree; the four warp sums are added in warp order.  Every thread of
// the calling group calls it (threads 0..127 add), `sync` is the group's
// barrier, and the sums land in thread 0.  Partials are read through L2:
// other blocks of the same launch may have written them.
template <class Sync>
__device__ __forceinline__ void sum_slots128(const double* part, int nslots, int t, double* w8, Sync sync, double& a,
                                             double& b) {
    a = 0.0;
    b = 0.0;
    if (t < 128) {
        for (int k = t; k < nslots; k += 128) {
            a += __ldcg(part + 2 * k);
            b += __ldcg(part + 2 * k + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if ((t & 31) == 0) {
            w8[2 * (t >> 5)] = a;
            w8[2 * (t >> 5) + 1] = b;
        }
    }
    sync();
    if (t == 0) {
        a = ((w8[0] + w8[2]) + w8[4]) + w8[6];
        b = ((w8[1] + w8[3]) + w8[5]) + w8[7];
    }
}

// One step's sums appended to the force history (while it has room) and kept
// as the last pair.
__device__ __forceinline__ void record_forces(double* hist, int cap, unsigned long long* counter, double* last,
                                              double a, double b) {
    const unsigned long long k = *counter;
    if (k < (unsigned long long)cap) {
        hist[2 * k] = a;
        hist[2 * k + 1] = b;
    }
    last[0] = a;
    last[1] = b;
    *counter = k + 1;
}

// The fused second stage, for a block that has written its force partials:
// every thread of the block (or of the consumer group, `sync` being its
// barrier, at least 128 threads) calls it after its writes.  The writes are
// made visible device-wide before the block counts itself; the last block to
// count sums all slots and resets the count for the next launch.  No thread
// waits on another block.
template <class Sync>
__device__ __forceinline__ void fused_force_finish(const KParams& p, int tid, Sync sync) {
    __shared__ unsigned int s_last;
    __shared__ double s_w8[8];
    __threadfence();
    sync();
    if (tid == 0) s_last = atomicAdd(p.red_done, 1u) == (unsigned int)(p.red_blocks - 1) ? 1u : 0u;
    sync();
    if (s_last) {
        __threadfence();
        double a, b;
        sum_slots128(p.partials, p.red_nslots, tid, s_w8, sync, a, b);
        if (tid == 0) {
            record_forces(p.red_hist, p.red_cap, p.red_counter, p.red_last, a, b);
            *p.red_done = 0u;
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
    uint32_t skey = 0;
    if constexpr (Pop<T>::kRounds) {
        const uint32_t s = seed_of(p);
        skey = seed_key(s);
        pass_seed(p, s, bxi == 0 && byi == 0 && threadIdx.x == 0 && threadIdx.y == 0);
    }
    double fxs = 0.0, fys = 0.0;  // momentum exchange, summed in FP64 across nodes
    if (x < p.nx && y < p.ny) {
        const unsigned n = (unsigned)y * (unsigned)p.nx + (unsigned)x;
        const uint32_t fl = __ldg(p.flags + n);
        R f[9], g[9];  // FP64: populations; FP32 compute: deviations
        if constexpr (std::is_same<T, double>::value)
            build_state<T, TH>(p, x, y, fl, f, g);
        else
            build_dev<T, TH>(p, x, y, fl, f, g);
        if (!(fl & FLAG_SOLID)) {
            if (fl & FLAG_BOUNDARY) {
                // momentum exchange of this node's links (src/lbm.hpp:565-577):
                // the node's terms 2 f in the compute precision, FP64 across nodes
                const uint32_t fm = p.rec_force[fl >> 2];
                R fxn = R(0), fyn = R(0);
#pragma unroll
                for (int j = 1; j < 9; ++j)
                    if (fm & (1u << j)) {
                        const R fj = f[j] + R(p.shf[j]);
                        fxn -= R(CXf(j)) * R(2) * fj;
                        fyn -= R(CYf(j)) * R(2) * fj;
                    }
                fxs = double(fxn);
                fys = double(fyn);
            }
            if constexpr (std::is_same<T, double>::value)
                collide<R, TH>(p, fl, f, g);
            else
                collide_dev<TH>(p, fl, f, g);
        }
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        const size_t N = (size_t)p.N;
        if (!((fl & FLAG_SOLID) && p.skip_settled_solids && x > 0 && x < p.nx - 1 && y < p.ny - 1)) {
            if constexpr (std::is_same<T, double>::value) {
#pragma unroll
                for (int j = 0; j < 9; ++j) Fo[j * N + n] = f[j];
                if (TH) {
                    T* __restrict__ Go = static_cast<T*>(p.gout);
#pragma unroll
                    for (int j = 0; j < 9; ++j) Go[j * N + n] = g[j];
                }
            } else {
                uint32_t rb[9] = {};
                if constexpr (Pop<T>::kRounds) rand9(skey + n, rb);
#pragma unroll
                for (int j = 0; j < 9; ++j) Pop<T>::std_(Fo + j * N, n, f[j], rb[j]);
                if (TH) {
                    T* __restrict__ Go = static_cast<T*>(p.gout);
                    if constexpr (Pop<T>::kRounds) rand9((skey + n) ^ 0x6A09E667u, rb);
#pragma unroll
                    for (int j = 0; j < 9; ++j) Pop<T>::std_(Go + j * N, n, g[j], rb[j]);
                }
            }
        }
    }
    if (p.block_slot) {
        const int base = p.block_slot[byi * gx + bxi];
        if (base >= 0) {  // uniform per block; no barrier: one slot per warp
            // FP64 warp sum, only in warps that hold a force node; the
            // cross-warp sum is FP64 as well.
            double a = fxs, b = fys;
            if (__any_sync(0xffffffffu, a != 0.0 || b != 0.0)) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    a += __shfl_down_sync(0xffffffffu, a, o);
                    b += __shfl_down_sync(0xffffffffu, b, o);
                }
            }
            const int tid = threadIdx.y * blockDim.x + threadIdx.x;
            if ((tid & 31) == 0) {
                const int slot = base + (tid >> 5);
                p.partials[2 * slot] = a;
                p.partials[2 * slot + 1] = b;
            }
            if (p.red_done) fused_force_finish(p, tid, [] { __syncthreads(); });
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
// square root of a strictly positive argument (no zero guard)
__device__ __forceinline__ F2 sqrt2_pos(F2 a) { return a * mk2(rsqrtf(a.v.x), rsqrtf(a.v.y)); }

// collide_dev<false> on two nodes at once (FP32x2), in storage units
// (deviation * kS); lane k is collided only when ok_k (a solid lane keeps the
// solid state, f = 0).
// KC / KL fix the collision (0 MRT, 1 BGK) and LES (0/1) at compile time;
// -1 reads them from the parameters.
template <class T, int KC = -1, int KL = -1>
__device__ __forceinline__ void collide_pair_dev(const KParams& p, uint32_t fla, uint32_t flb, bool fa_ok,
                                                 bool fb_ok, F2 d[9]) {
    constexpr float S = Pop<T>::kS, iS = Pop<T>::kInvS;
    const bool mrt = KC >= 0 ? KC == 0 : p.collision == 0;
    const bool les = KL >= 0 ? KL == 1 : p.les != 0;
    const Phys<float>& q = p.pf;
    const F2 drho = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
    const F2 mx = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
    const F2 my = (d[2] - d[4]) + (d[5] + d[6]) - (d[7] + d[8]);
    const F2 rho = fma2(drho, sp2(iS), sp2(1.0f));
    const F2 inv = rcp2(rho);
    const F2 k = S == 1.0f ? inv : inv * sp2(iS);  // 1 / (rho * S)
    const F2 u = mx * k, v = my * k;
    // a non-finite or zero density in a collided lane: the product of the two
    // lanes' densities (1 for a solid lane) is NaN or zero
    if (!(fabsf((fa_ok ? rho.v.x : 1.0f) * (fb_ok ? rho.v.y : 1.0f)) > 0.0f)) atomicOr(p.nan_flag, 1u);
    const float F = q.Fscale * S;
    F2 o[9];
    if (mrt) {
        const F2 sd = (d[5] + d[6]) + (d[7] + d[8]), sa = (d[1] + d[2]) + (d[3] + d[4]);
        F2 me = fma2(sp2(2.0f), sd, fma2(sp2(-4.0f), d[0], sp2(0.0f) - sa));  // (e + 2) S
        F2 meps = fma2(sp2(4.0f), d[0], fma2(sp2(-2.0f), sa, sd));            // (eps - 1) S
        F2 mpxx = (d[1] - d[2]) + (d[3] - d[4]);
        F2 mpxy = (d[5] - d[6]) + (d[7] - d[8]);
        const F2 r3u = sp2(3.0f) * fma2(mx, u, my * v);
        const F2 e_eq = fma2(sp2(-2.0f), drho, r3u);
        const F2 eps_eq = drho - r3u;
        const F2 pxx_eq = fma2(mx, u, sp2(0.0f) - my * v);
        const F2 pxy_eq = mx * v;
        F2 s_eff = sp2(q.s_shear);
        if (les) {
            F2 csq = sp2(q.cs_sq);
            if (q.nu > 0.0f) {
                // y+ > 0 at every collided node (its wall distance is >= 1),
                // so the Van Driest branch always applies
                const F2 wd = mk2(wall_distance<float>(p, fla), wall_distance<float>(p, flb));
                const F2 yp = wd * sqrt2_pos(fma2(u, u, v * v) + sp2(1e-12f)) * sp2(q.inv_nu);
                const F2 cd = sp2(q.cs) - sp2(q.cs) * mk2(__expf(yp.v.x * (-1.0f / 26.0f)), __expf(yp.v.y * (-1.0f / 26.0f)));
                csq = cd * cd;
            }
            const F2 a = mpxx - pxx_eq, b = mpxy - pxy_eq;
            // Q * S; the 1e-30 (far below any nonzero 2|Pi_neq|^2 in FP32)
            // keeps the argument positive, so no zero guard is needed
            const F2 Q = sqrt2_pos(fma2(sp2(2.0f), fma2(a, a, b * b), sp2(1e-30f)));
            const F2 A = sp2(4.5f) * csq * Q * k;
            const F2 te2 = sp2(q.tau) + sqrt2_pos(fma2(sp2(q.tau), sp2(q.tau), sp2(4.0f) * A));
            const F2 s2 = sp2(2.0f) * rcp2(te2);
            s_eff = mk2(clamp_rate<float>(s2.v.x), clamp_rate<float>(s2.v.y));
        }
        const F2 sb = sp2(q.s_bulk);
        me = me - sb * (me - e_eq);
        meps = meps - sb * (meps - eps_eq);
        mpxx = mpxx - s_eff * (mpxx - pxx_eq);
        mpxy = mpxy - s_eff * (mpxy - pxy_eq);
        const F2 a0 = sp2(1.0f / 9.0f) * drho;
        const F2 ax = a0 - sp2(1.0f / 36.0f) * me - sp2(1.0f / 18.0f) * meps;
        const F2 ad = fma2(sp2(1.0f / 18.0f), me, fma2(sp2(1.0f / 36.0f), meps, a0));
        const F2 hx = fma2(sp2(1.0f / 3.0f), mx, sp2((1.0f / 9.0f) * F)), hy = sp2(1.0f / 3.0f) * my;
        const F2 dx = fma2(sp2(1.0f / 12.0f), mx, sp2((1.0f / 36.0f) * F)), dy = sp2(1.0f / 12.0f) * my;
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
        const F2 rhoS = drho + sp2(S);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const F2 cj = sp2(float(CXf(i))) * mx + sp2(float(CYf(i))) * my;
            const F2 ed = sp2(float(CXf(i))) * u + sp2(float(CYf(i))) * v;
            const F2 fe = sp2(float(wgt(i))) * (fma2(sp2(3.0f), cj, drho) +
                                                 rhoS * fma2(sp2(4.5f) * ed, ed, sp2(-1.5f) * usq));
            o[i] = d[i] - it * (d[i] - fe);
        }
        if (F != 0.0f) {
            const F2 fa = sp2((1.0f / 9.0f) * F), fd = sp2((1.0f / 36.0f) * F);
            o[1] = o[1] + fa;
            o[3] = o[3] - fa;
            o[5] = o[5] + fd;
            o[6] = o[6] - fd;
            o[7] = o[7] - fd;
            o[8] = o[8] + fd;
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        // keep a solid lane's input (measured faster for FP32 than the branch)
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j] = mk2(fa_ok ? o[j].v.x : d[j].v.x, fb_ok ? o[j].v.y : d[j].v.y);
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j] = o[j];
        if (!fa_ok) {  // solid lane: f = 0
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j].v.x = -p.shf[j] * S;
        }
        if (!fb_ok) {
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j].v.y = -p.shf[j] * S;
        }
    }
}

// The thermal double distribution of two nodes at once (FP32x2), in storage
// units: collide_dev<true>'s thermal part (src/lbm.hpp:357-397,
// src/thermal.hpp:25-52) after collide_pair_dev has collided f.  u comes from
// the post-collision f (d); g relaxes with omega_k toward w T (1 + 3 c.u +
// 4.5 (c.u)^2 - 1.5 u^2) on deviations e = g - w T_ref; the Boussinesq force
// (0, -beta (T - T_ref) g_y) is added to f as w (3 c.F + 9 (c.u)(c.F)).  A
// lane that is not collided (solid) keeps its input.
template <class T>
__device__ __forceinline__ void thermal_pair_dev(const KParams& p, bool fa_ok, bool fb_ok, F2 d[9], F2 e[9]) {
    constexpr float S = Pop<T>::kS, iS = Pop<T>::kInvS;
    const Phys<float>& q = p.pf;
    const F2 drho = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
    const F2 mx = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
    const F2 my = (d[2] - d[4]) + (d[5] + d[6]) - (d[7] + d[8]);
    const F2 k = rcp2(drho + sp2(S));  // 1 / (rho * S)
    const F2 u = mx * k, v = my * k, usq = fma2(u, u, v * v);
    const F2 dTS = ((e[0] + e[1]) + (e[2] + e[3])) + ((e[4] + e[5]) + (e[6] + e[7])) + e[8];
    const F2 dT = dTS * sp2(iS);
    const F2 TS = fma2(dT, sp2(S), sp2(q.T_ref * S));  // T * S
    const F2 om = sp2(q.omega_k);
    F2 o[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const F2 ed = sp2(float(CXf(i))) * u + sp2(float(CYf(i))) * v;
        const F2 poly = fma2(sp2(4.5f) * ed, ed, fma2(sp2(3.0f), ed, sp2(-1.5f) * usq));
        const F2 geS = sp2(float(wgt(i))) * fma2(TS, poly, dTS);
        o[i] = e[i] - om * (e[i] - geS);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) e[i] = mk2(fa_ok ? o[i].v.x : e[i].v.x, fb_ok ? o[i].v.y : e[i].v.y);
    if (q.beta > 0.0f && q.g_buoy != 0.0f) {
        const F2 fyb = sp2(-q.beta * q.g_buoy) * dT;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            if (CYf(i) == 0) continue;
            const F2 eu = sp2(float(CXf(i))) * u + sp2(float(CYf(i))) * v;
            const F2 Fd = sp2(float(CYf(i))) * fyb;
            const F2 inc = sp2(float(wgt(i)) * S) * fma2(sp2(9.0f) * eu, Fd, sp2(3.0f) * Fd);
            d[i] = mk2(fa_ok ? d[i].v.x + inc.v.x : d[i].v.x, fb_ok ? d[i].v.y + inc.v.y : d[i].v.y);
        }
    }
}

// build_dev_s<T> for the thermal DDF: f and g deviations in storage units.
template <class T>
__device__ __forceinline__ void build_dev_s_th(const KParams& p, int x, int y, uint32_t fl, float d[9], float e[9]) {
    if (!special_node<true>(p, x, y, fl)) {
        pull_raw<T>(p, static_cast<const T*>(p.fin), x, y, d);
        pull_raw<T>(p, static_cast<const T*>(p.gin), x, y, e);
        return;
    }
    float f[9], g[9];
    build_state<T, true>(p, x, y, fl, f, g);
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        d[j] = (f[j] - p.shf[j]) * Pop<T>::kS;
        e[j] = (g[j] - p.shg[j]) * Pop<T>::kS;
    }
}

template <class T>
struct PairStore;
// Two x-neighbours (index i even) in storage units as one 8-byte / 4-byte store.
template <>
struct PairStore<float> {
    // streaming store: the next step reads the populations back from DRAM
    // anyway (the lattice is far larger than L2); measured +0.5-1.7% for FP32
    static __device__ __forceinline__ void st(float* p, size_t i, float a, float b, uint32_t) {
        __stcs(reinterpret_cast<float2*>(p + i), make_float2(a, b));
    }
    // one node (the last of a lattice with an odd node count)
    static __device__ __forceinline__ void st1(float* p, size_t i, float a, uint32_t) { __stcs(p + i, a); }
    // the pair's values as two single-node stores (i odd: no pair alignment)
    static __device__ __forceinline__ void st_split(float* p, size_t i, float a, float b, uint32_t) {
        __stcs(p + i, a);
        __stcs(p + i + 1, b);
    }
};
template <>
struct PairStore<__half> {
    static __device__ __forceinline__ void st(__half* p, size_t i, float a, float b, uint32_t rb) {
        *reinterpret_cast<uint32_t*>(p + i) = cvt_rs_f16x2(a, b, rb);
    }
    static __device__ __forceinline__ void st1(__half* p, size_t i, float a, uint32_t rb) {
        p[i] = __ushort_as_half((unsigned short)(cvt_rs_f16x2(a, a, rb) & 0xFFFFu));
    }
    // the bits st would store, as two 2-byte stores (i odd)
    static __device__ __forceinline__ void st_split(__half* p, size_t i, float a, float b, uint32_t rb) {
        const uint32_t w = cvt_rs_f16x2(a, b, rb);
        p[i] = __ushort_as_half((unsigned short)(w & 0xFFFFu));
        p[i + 1] = __ushort_as_half((unsigned short)(w >> 16));
    }
};
template <>
struct PairStore<__nv_bfloat16> {
    static __device__ __forceinline__ void st(__nv_bfloat16* p, size_t i, float a, float b, uint32_t rb) {
        *reinterpret_cast<uint32_t*>(p + i) = cvt_rs_bf16x2(a, b, rb);
    }
    static __device__ __forceinline__ void st1(__nv_bfloat16* p, size_t i, float a, uint32_t rb) {
        p[i] = __ushort_as_bfloat16((unsigned short)(cvt_rs_bf16x2(a, a, rb) & 0xFFFFu));
    }
    static __device__ __forceinline__ void st_split(__nv_bfloat16* p, size_t i, float a, float b, uint32_t rb) {
        const uint32_t w = cvt_rs_bf16x2(a, b, rb);
        p[i] = __ushort_as_bfloat16((unsigned short)(w & 0xFFFFu));
        p[i + 1] = __ushort_as_bfloat16((unsigned short)(w >> 16));
    }
};

// One step of the node pair a = (xa, ya), b = (xb, yb), stored at node
// indices n0 and n0 + 1, n0 even: two x-neighbours of a row (b = a + x), or
// a flat pair of the node index, which may end one row and start the next
// (FP32/FP16/BF16 storage; TH: with the thermal double distribution, collided
// by thermal_pair_dev): pull with the rebuild of special nodes, momentum
// exchange (the pair's link terms summed in FP32, node a then b, returned in
// fxs/fys), collision and stores.  PLAIN: the pair holds no boundary node
// (those are stepped by a boundary block), so a solid lane (f = 0) is its
// only special case and the pulls need no rebuild.  has_b false: n0 is the
// last node of a lattice with an odd node count (b is absent: the caller
// marks it solid, and only a is stored).
template <class T, bool TH, bool PLAIN>
__device__ __forceinline__ void pair_step(const KParams& p, unsigned n0, int xa, int ya, int xb, int yb, bool has_b,
                                          uint32_t skey, uint2 fl, double& fxs, double& fys) {
    constexpr float iS = Pop<T>::kInvS;
    float fa[9], fb[9];  // deviations in storage units
    float ea[TH ? 9 : 1], eb[TH ? 9 : 1];  // thermal deviations (TH)
    const bool oka = !(fl.x & FLAG_SOLID), okb = !(fl.y & FLAG_SOLID);
    if constexpr (PLAIN) {
        const T* __restrict__ P = static_cast<const T*>(p.fin);
        pull_raw<T>(p, P, xa, ya, fa);
        if (has_b) pull_raw<T>(p, P, xb, yb, fb);
        constexpr float S = Pop<T>::kS;
        if (!oka) {
#pragma unroll
            for (int j = 0; j < 9; ++j) fa[j] = -p.shf[j] * S;
        }
        if (!okb) {
#pragma unroll
            for (int j = 0; j < 9; ++j) fb[j] = -p.shf[j] * S;
        }
    } else if constexpr (TH) {
        build_dev_s_th<T>(p, xa, ya, fl.x, fa, ea);
        build_dev_s_th<T>(p, xb, yb, fl.y, fb, eb);
    } else {
        build_dev_s<T>(p, xa, ya, fl.x, fa);
        if (has_b) {
            build_dev_s<T>(p, xb, yb, fl.y, fb);
        } else {
#pragma unroll
            for (int j = 0; j < 9; ++j) fb[j] = -p.shf[j] * Pop<T>::kS;
        }
    }
    if (!PLAIN && ((fl.x | fl.y) & FLAG_BOUNDARY)) {
        // momentum exchange of the nodes' links (src/lbm.hpp:565-577)
        const uint32_t ma = (oka && (fl.x & FLAG_BOUNDARY)) ? p.rec_force[fl.x >> 2] : 0u;
        const uint32_t mb = (okb && (fl.y & FLAG_BOUNDARY)) ? p.rec_force[fl.y >> 2] : 0u;
        // the pair's link terms in FP32, node x0 then x0 + 1
        float fxp = 0.0f, fyp = 0.0f;
#pragma unroll
        for (int j = 1; j < 9; ++j)
            if (ma & (1u << j)) {
                const float f = fmaf(fa[j], iS, p.shf[j]);
                fxp -= float(CXf(j)) * 2.0f * f;
                fyp -= float(CYf(j)) * 2.0f * f;
            }
#pragma unroll
        for (int j = 1; j < 9; ++j)
            if (mb & (1u << j)) {
                const float f = fmaf(fb[j], iS, p.shf[j]);
                fxp -= float(CXf(j)) * 2.0f * f;
                fyp -= float(CYf(j)) * 2.0f * f;
            }
        fxs = double(fxp);
        fys = double(fyp);
    }
    if (oka || okb) {
        F2 f[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = mk2(fa[j], fb[j]);
        collide_pair_dev<T>(p, fl.x, fl.y, oka, okb, f);
        if constexpr (TH) {
            F2 g[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) g[j] = mk2(ea[j], eb[j]);
            thermal_pair_dev<T>(p, oka, okb, f, g);
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                ea[j] = g[j].v.x;
                eb[j] = g[j].v.y;
            }
        }
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            fa[j] = f[j].v.x;
            fb[j] = f[j].v.y;
        }
    }
    // a solid node's state never changes once settled (the heated
    // cavity's Dirichlet passes rewrite node states every step)
    const bool skip_a = !oka && p.skip_settled_solids && ya < p.ny - 1 && xa > 0;
    const bool skip_b = !has_b || (!okb && p.skip_settled_solids && yb < p.ny - 1 && xb < p.nx - 1);
    if (!(skip_a && skip_b)) {
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        const size_t N = (size_t)p.N;
        uint32_t rb[9] = {};
        if constexpr (Pop<T>::kRounds) rand9(skey + n0, rb);
        // n0 is even, so element j*N + n0 is odd -- a pair store there
        // misaligned -- exactly in the odd planes of a lattice with an odd
        // node count (flat pairs of an odd width and height): two
        // single-node stores of the same values there
        const bool split_odd = (N & 1) != 0;
        if (has_b) {
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                if (split_odd && (j & 1))
                    PairStore<T>::st_split(Fo + j * N, n0, fa[j], fb[j], rb[j]);
                else
                    PairStore<T>::st(Fo + j * N, n0, fa[j], fb[j], rb[j]);
            }
        } else {
#pragma unroll
            for (int j = 0; j < 9; ++j) PairStore<T>::st1(Fo + j * N, n0, fa[j], rb[j]);
        }
        if constexpr (TH) {
            T* __restrict__ Go = static_cast<T*>(p.gout);
            if constexpr (Pop<T>::kRounds) rand9((skey + n0) ^ 0x6A09E667u, rb);
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                if (split_odd && (j & 1))
                    PairStore<T>::st_split(Go + j * N, n0, ea[j], eb[j], rb[j]);
                else
                    PairStore<T>::st(Go + j * N, n0, ea[j], eb[j], rb[j]);
            }
        }
    }
}

// The block's per-warp force partials: FP64 warp sums into the slots that
// block_slot[idx] opens (none when -1), then the fused second stage.
__device__ __forceinline__ void pair_block_slots(const KParams& p, int idx, double fxs, double fys) {
    if (p.block_slot) {
        const int base = p.block_slot[idx];
        if (base >= 0) {
            double a = fxs, b = fys;  // FP64 warp sum
            if (__any_sync(0xffffffffu, a != 0.0 || b != 0.0)) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    a += __shfl_down_sync(0xffffffffu, a, o);
                    b += __shfl_down_sync(0xffffffffu, b, o);
                }
            }
            const int tid = threadIdx.y * blockDim.x + threadIdx.x;
            if ((tid & 31) == 0) {
                const int slot = base + (tid >> 5);
                p.partials[2 * slot] = a;
                p.partials[2 * slot + 1] = b;
            }
            if (p.red_done) fused_force_finish(p, tid, [] { __syncthreads(); });
        }
    }
}

__device__ __forceinline__ uint32_t pair_seed_key(const KParams& p, bool first) {
    const uint32_t s = seed_of(p);
    pass_seed(p, s, first);
    return seed_key(s);
}

// One step of the paired block (bxi, byi) of an instance whose paired block
// grid is gx wide.  PLAIN: the instance's boundary pairs are stepped by its
// boundary blocks (pair_boundary_block); this block skips them.
template <class T, bool TH = false, bool PLAIN = false>
__device__ __forceinline__ void step_pair_block(const KParams& p, int bxi, int byi, int gx) {
    const int x0 = 2 * (bxi * blockDim.x + threadIdx.x);
    const int y = byi * blockDim.y + threadIdx.y;
    uint32_t skey = 0;
    if constexpr (Pop<T>::kRounds)
        skey = pair_seed_key(p, bxi == 0 && byi == 0 && threadIdx.x == 0 && threadIdx.y == 0);
    double fxs = 0.0, fys = 0.0;  // momentum exchange, FP64 across node pairs
    if (x0 < p.nx && y < p.ny) {
        const unsigned n0 = (unsigned)y * (unsigned)p.nx + (unsigned)x0;
        const uint2 fl = __ldg(reinterpret_cast<const uint2*>(p.flags + n0));
        if (!PLAIN || !((fl.x | fl.y) & FLAG_BOUNDARY))
            pair_step<T, TH, PLAIN>(p, n0, x0, y, x0 + 1, y, true, skey, fl, fxs, fys);
    }
    if (!PLAIN) pair_block_slots(p, byi * gx + bxi, fxs, fys);
}

// The nodes of the flat pair (n0, n0 + 1), n0 even: coordinates, flags and
// whether n0 + 1 exists.  The flags' second word past the last node is
// padding; an absent node is marked solid.
__device__ __forceinline__ void flat_pair(const KParams& p, unsigned n0, int& xa, int& ya, int& xb, int& yb,
                                          bool& has_b, uint2& fl) {
    ya = (int)(n0 / (unsigned)p.nx);
    xa = (int)n0 - ya * p.nx;
    xb = xa + 1;
    yb = ya;
    if (xb == p.nx) {
        xb = 0;
        ++yb;
    }
    has_b = (long long)n0 + 1 < p.N;
    fl = __ldg(reinterpret_cast<const uint2*>(p.flags + n0));
    if (!has_b) fl.y = FLAG_SOLID;
}

// Flat tile t of a batched paired instance: its pairs [t*B, (t+1)*B), B the
// block's threads, one pair (2k, 2k + 1) of the node index per thread, so
// any width pairs (pair_step splits the stores a pair would misalign).  The instance's boundary pairs are stepped by its
// boundary blocks (pair_boundary_block); this tile skips them.
template <class T>
__device__ __forceinline__ void step_flat_pair_block(const KParams& p, int t) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const long long q = (long long)t * (blockDim.x * blockDim.y) + tid;
    uint32_t skey = 0;
    if constexpr (Pop<T>::kRounds) skey = pair_seed_key(p, t == 0 && tid == 0);
    if (2 * q < p.N) {
        const unsigned n0 = (unsigned)(2 * q);
        int xa, ya, xb, yb;
        bool has_b;
        uint2 fl;
        flat_pair(p, n0, xa, ya, xb, yb, has_b, fl);
        if (!((fl.x | fl.y) & FLAG_BOUNDARY)) {
            double fxs = 0.0, fys = 0.0;
            pair_step<T, false, true>(p, n0, xa, ya, xb, yb, has_b, skey, fl, fxs, fys);
        }
    }
}

// Boundary block i of an instance: its boundary pairs [i*B, (i+1)*B), B the
// block's threads, one flat pair per thread (bpairs, ascending); the force
// slots of boundary block i are block_slot[ntiles + i], ntiles its flat
// tiles.
template <class T>
__device__ __forceinline__ void pair_boundary_block(const KParams& p, int i, int ntiles) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int j = i * (int)(blockDim.x * blockDim.y) + tid;
    uint32_t skey = 0;
    if constexpr (Pop<T>::kRounds) skey = pair_seed_key(p, false);
    double fxs = 0.0, fys = 0.0;
    if (j < p.nbpairs) {
        const unsigned n0 = (unsigned)p.bpairs[j];  // a flat pair
        int xa, ya, xb, yb;
        bool has_b;
        uint2 fl;
        flat_pair(p, n0, xa, ya, xb, yb, has_b, fl);
        pair_step<T, false, false>(p, n0, xa, ya, xb, yb, has_b, skey, fl, fxs, fys);
    }
    pair_block_slots(p, ntiles + i, fxs, fys);
}

}  // namespace
}  // namespace lbm2d
