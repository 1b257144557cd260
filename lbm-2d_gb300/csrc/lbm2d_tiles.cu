// lbm2d_tiles.cu -- the tile-pipelined step kernel (sm_103a): any grid width,
// the thermal double distribution, and many instances in one launch.
//
// The same step as the row pipeline (pull, rebuild, force, collision, store)
// with a different unit of work:
//
//   * a tile is W = 448 CONSECUTIVE nodes of an instance in row-major order
//     (it may span several short rows or part of a long one).  In that order
//     the pull source of direction j is node n - cy_j*nx - cx_j, so the
//     sources of a whole tile are one contiguous window per direction.  The
//     producer warp brings each window, rounded out to 16-byte
//     granules (the window's first element sits `lead` elements into the
//     staged row), the tile's flags and -- in a batch -- the instance's
//     parameters into a shared-memory stage with cp.async.bulk copies that
//     complete on the stage's mbarrier; the producer warp's lanes compute and
//     issue one copy each.  No alignment of nx is needed;
//   * nodes on the lattice border (x = 0, nx-1 or y = 0, ny-1), whose
//     periodic sources lie outside the window, and nodes that need more than
//     the plain pull (solid, boundary record, a thermal hook row or column)
//     are rebuilt from global memory with the per-node functions every step
//     kernel shares;
//   * a persistent grid walks the tiles of one instance, or of all instances
//     of a batch (tile_member[t] names the instance), each CTA a contiguous
//     chunk of ceil(T / G) tiles.  The producer skips the tiles of an
//     instance whose step budget is spent and ends the ring with a marker
//     stage;
//   * consumers: 7 warps.  Non-thermal: each lane owns two consecutive
//     nodes, collided with the packed FP32x2 collision (collide_pair_dev) and
//     stored as pairs (the paired kernels' rounding noise).  Thermal: each
//     lane owns nodes tid and tid + W/2, collided one at a time
//     (collide_dev<true>) with the one-node kernel's per-node noise;
//   * momentum exchange: FP64 per lane in shared memory, an FP64 warp sum per
//     tile into the instance's per-tile slots (fixed order, so the same
//     instance gives the same bits alone or in any mix); a single instance
//     fuses the second stage into its last force CTA.
// Every wait is bounded (about one second); a wait that runs out sets bit 1
// of the status word and the CTA leaves after draining its copies.
#include <algorithm>
#include <atomic>

#include "lbm2d_pipeline.cuh"

namespace lbm2d {
namespace {

// 7 consumer warps + the producer warp, two CTAs per SM: 16 warps per SM,
// four per SM sub-partition, which leaves each thread 128 registers of the
// sub-partition's 16K -- the collision plus the tile bookkeeping without
// spills
constexpr int kTWarps = 7;
constexpr int kTThreads = 32 * (kTWarps + 1);
constexpr int kTW = 2 * 32 * kTWarps;  // nodes per tile

template <class T, bool TH>
struct TilesCfg {
    static constexpr int ES = (int)sizeof(T);
    static constexpr int EPG = 16 / ES;         // elements per 16-byte granule
    static constexpr int WIN = kTW + 2 * EPG;   // staged elements per window (lead + W + 2 rounded up)
    static constexpr int ROWB = WIN * ES;
    static constexpr int NWIN = TH ? 18 : 9;
    static constexpr int FLAGS_OFF = NWIN * ROWB;
    static constexpr int PAR_OFF = FLAGS_OFF + kTW * 4;
    static constexpr int HDR_OFF = PAR_OFF + (int)sizeof(KParams);
    static constexpr int STAGE_BYTES = (HDR_OFF + 32 + 127) / 128 * 128;
    // two CTAs per SM with a ring of about 85 KB each: the deeper, the more
    // bytes in flight per SM
    static constexpr int STAGES = TH ? (ES == 4 ? 2 : 4) : (ES == 4 ? 4 : 7);
    static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
    static constexpr int ACC_OFF = BAR_OFF + 2 * STAGES * 8;
    static constexpr int SMEM = ACC_OFF + 32 * kTWarps * 16;
    static_assert(ROWB % 16 == 0 && FLAGS_OFF % 16 == 0 && PAR_OFF % 16 == 0, "bulk-copy alignment");
    static_assert(sizeof(KParams) % 16 == 0, "parameter copy size");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

// Stage header, written by the producer before it arrives on the stage:
// instance (-1: end of the ring), first node, its (x, y), rounding seed,
// tile index within the instance, the nine window leads (3 bits each) and the
// tile's first force slot (-1: none).
struct TileHdr {
    int k, n0, x0, y0;
    uint32_t seed;
    int tile, leads, slot;
};
static_assert(sizeof(TileHdr) == 32, "header size");

// Window j of a tile starting at node n0: global element g = j*N + n0 -
// cy_j*nx - 1 (the source of the tile's first node for cx = +1), rounded down
// to a granule: the staged row starts at a = g - lead.
__device__ __forceinline__ long long win_start(long long N, int nx, int n0, int j, int epg, int& lead) {
    const long long g = (long long)j * N + n0 - (long long)CYf(j) * nx - 1;
    const long long a = g >= 0 ? (g / epg) * epg : -((-g + epg - 1) / epg) * epg;
    lead = (int)(g - a);
    return a;
}

// Parameters a consumer reads for the tile: the instance's own copy in the
// stage (batch) or the kernel parameter (single instance).
template <bool SINGLE>
__device__ __forceinline__ const KParams& tile_params(const KParams& single, const unsigned char* stage,
                                                      int par_off) {
    if constexpr (SINGLE) return single;
    else return *reinterpret_cast<const KParams*>(stage + par_off);
}

// ----------------------------------------------------------------- producer
// The producer warp stages one tile at a time, its lanes in parallel: lane w
// < NWIN computes and issues the copy of window w (f windows, then g), lane
// NWIN the flags copy and lane NWIN + 1 (batch) the parameter copy; a warp sum
// gives the bytes lane 0 announces on the stage's mbarrier before any copy is
// issued.  Per-instance bookkeeping (tile range, budget, seed) is done by all
// lanes alike when the instance changes; the tile's force slot is loaded ahead
// of the stage wait, so no dependent global load sits on the per-tile path.
template <class T, bool TH, bool SINGLE>
__device__ __forceinline__ void tiles_produce(const KParams& single, const KParams* __restrict__ inst,
                                              const int* __restrict__ tile_member, const int* __restrict__ tile_start,
                                              int ntiles, unsigned char* smem, uint32_t sbase, uint32_t full0,
                                              uint32_t empty0, unsigned int* status) {
    using C = TilesCfg<T, TH>;
    const int lane = threadIdx.x & 31;
    int issued = 0;
    bool ok = true;
    // a contiguous chunk of tiles per CTA: consecutive tiles mostly belong to
    // the same instance (its parameters, budget and seed are looked up once
    // per instance, not per tile) and share halo rows in L2
    const int chunk = (ntiles + (int)gridDim.x - 1) / (int)gridDim.x;
    const int t_end = min(ntiles, ((int)blockIdx.x + 1) * chunk);
    int k = -1, k_first = 0, k_next = 0, L = 1;
    uint32_t seed = 0;
    // instance bookkeeping when tile t starts a new instance: its step budget
    // (an instance whose budget is spent takes no step) and rounding seed; the
    // CTA holding its first tile hands the decremented budget and the seed on
    auto begin_instance = [&](const KParams& g0, int t) {
        L = g0.left_in ? *g0.left_in : 1;
        seed = g0.seed_in ? *g0.seed_in : g0.seed_host;
        __syncwarp();
        if (t == k_first && lane == 0) {
            if (g0.left_in) *g0.left_out = L > 0 ? L - 1 : 0;
            if (L > 0 && g0.seed_out) *g0.seed_out = seed + 1u;
        }
    };
    // stage tile tl of instance gp; false when a wait ran out
    auto stage_tile = [&](const KParams& gp, int tl) -> bool {
        // loads that do not depend on the stage, ahead of the wait
        const int slot = (lane == 0 && gp.block_slot) ? __ldg(gp.block_slot + tl) : -1;
        const int s = issued % C::STAGES, n = issued / C::STAGES;
        if (n > 0 && !__all_sync(0xffffffffu, mbar_wait(empty0 + 8 * s, (uint32_t)((n - 1) & 1)))) return false;
        const uint32_t st = sbase + (uint32_t)(s * C::STAGE_BYTES);
        const uint32_t bar = full0 + 8 * s;
        const long long N = gp.N;
        const int nx = gp.nx;
        const int n0 = tl * kTW;
        // this lane's copy
        const void* src = nullptr;
        uint32_t dst = 0, nb = 0;
        int lead = 0;
        if (lane < C::NWIN) {
            const int set = lane / 9, j = lane - 9 * set;
            const T* P = static_cast<const T*>(set ? gp.gin : gp.fin);
            const long long a = win_start(N, nx, n0, j, C::EPG, lead);
            const long long gend = (9 * N + C::EPG - 1) / C::EPG * C::EPG;  // buffers are padded to it
            const long long cs = max(a, 0LL), ce = min(a + C::WIN, gend);
            if (ce > cs) {
                src = P + cs;
                dst = st + (uint32_t)(lane * C::ROWB) + (uint32_t)((cs - a) * C::ES);
                nb = (uint32_t)((ce - cs) * C::ES);
            }
        } else if (lane == C::NWIN) {
            src = gp.flags + n0;
            dst = st + C::FLAGS_OFF;
            nb = (uint32_t)(((min((long long)kTW, N - n0) * 4) + 15) / 16 * 16);
        } else if (!SINGLE && lane == C::NWIN + 1) {
            src = &gp;
            dst = st + C::PAR_OFF;
            nb = (uint32_t)sizeof(KParams);
        }
        uint32_t bytes = nb;
        int leads = lane < 9 ? lead << (3 * lane) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
            leads |= __shfl_xor_sync(0xffffffffu, leads, o);
        }
        if (lane == 0) {
            TileHdr* h = reinterpret_cast<TileHdr*>(smem + s * C::STAGE_BYTES + C::HDR_OFF);
            h->k = k;
            h->n0 = n0;
            h->x0 = n0 % nx;
            h->y0 = n0 / nx;
            h->seed = seed;
            h->tile = tl;
            h->leads = leads;
            h->slot = slot;
            mbar_expect_tx(bar, bytes);  // release: the header is visible with the stage
        }
        __syncwarp();
        if (nb) bulk_g2s(dst, src, nb, bar);
        ++issued;
        return true;
    };
    for (int t = (int)blockIdx.x * chunk; t < t_end; ++t) {
        if constexpr (SINGLE) {
            // the kernel parameter is used in place (never through its address)
            if (k < 0) {
                k = 0;
                begin_instance(single, t);
            }
            if (L <= 0) continue;
            if (!stage_tile(single, t)) {
                ok = false;
                break;
            }
        } else {
            if (t >= k_next) {
                k = __ldg(tile_member + t);
                k_first = __ldg(tile_start + k);
                k_next = __ldg(tile_start + k + 1);
                begin_instance(inst[k], t);
            }
            if (L <= 0) continue;
            if (!stage_tile(inst[k], t - k_first)) {
                ok = false;
                break;
            }
        }
    }
    if (lane != 0) return;
    // end marker: a stage whose header says k = -1, completed by a plain arrival
    if (ok) {
        const int s = issued % C::STAGES, n = issued / C::STAGES;
        if (n > 0 && !mbar_wait(empty0 + 8 * s, (uint32_t)((n - 1) & 1))) {
            ok = false;
        } else {
            reinterpret_cast<TileHdr*>(smem + s * C::STAGE_BYTES + C::HDR_OFF)->k = -1;
            mbar_arrive(full0 + 8 * s);
        }
    }
    // every issued copy completes before the CTA may exit (the stage of tile
    // issued - STAGES, if any, was refilled or consumed already)
    bool drained = true;
    for (int i = max(issued - C::STAGES + 1, 0); i < issued; ++i)
        drained = mbar_wait(full0 + 8 * (i % C::STAGES), (uint32_t)((i / C::STAGES) & 1)) && drained;
    if (!ok || !drained) atomicOr(status, 2u);
}

// ----------------------------------------------------------------- consumer
// Node coordinates of local node i of a tile whose first node is (x0, y0):
// a = x0 + i < nx + W, so a single-precision quotient estimate is off by at
// most one.
__device__ __forceinline__ void tile_xy(int x0, int y0, int i, int nx, float inv_nx, int& x, int& y) {
    const int a = x0 + i;
    int q = (int)(__int2float_rn(a) * inv_nx);
    int r = a - q * nx;
    if (r < 0) {
        --q;
        r += nx;
    } else if (r >= nx) {
        ++q;
        r -= nx;
    }
    x = r;
    y = y0 + q;
}

__device__ __forceinline__ bool border(const KParams& p, int x, int y) {
    return x == 0 || x == p.nx - 1 || y == 0 || y == p.ny - 1;
}

// Staged value of direction j (window w) for local node i, storage units.
template <class T, bool TH>
__device__ __forceinline__ float staged(const unsigned char* stage, int w, int lead, int i, int cx) {
    using C = TilesCfg<T, TH>;
    const T* r = reinterpret_cast<const T*>(stage + w * C::ROWB);
    if constexpr (std::is_same<T, float>::value) return r[lead + i + 1 - cx];
    else if constexpr (std::is_same<T, __half>::value) return __half2float(r[lead + i + 1 - cx]);
    else return __bfloat162float(r[lead + i + 1 - cx]);
}

// Stored populations of the tile's sources for the rebuild functions: the
// staged window of direction j when it holds node idx of plane j, else device
// memory.  Window j starts at global element j*N + n0 - cy_j*nx - 1 - lead_j,
// so node idx of plane j sits at offset lead_j + 1 + idx - n0 + cy_j*nx; an
// offset inside the window is an element the producer copied.  Values are
// converted exactly as Pop<T> converts them from device memory.
template <class T, bool TH>
struct TileSrc {
    const unsigned char* stage;
    int w0;  // first window of this population set (0: f, 9: g)
    long long n0;
    int leads, nx;
    const T* __restrict__ P;
    size_t N;
    const float* sh;
    const uint32_t* __restrict__ gflags;
    __device__ __forceinline__ float raw(int j, unsigned idx) const {
        using C = TilesCfg<T, TH>;
        const int lead = (leads >> (3 * j)) & 7;
        const long long o = (long long)lead + 1 + (long long)idx - n0 + (long long)CYf(j) * nx;
        if (o >= 0 && o < C::WIN) {
            const T v = reinterpret_cast<const T*>(stage + (w0 + j) * C::ROWB)[o];
            if constexpr (std::is_same<T, float>::value) return v;
            else if constexpr (std::is_same<T, __half>::value) return __half2float(v);
            else return __bfloat162float(v);
        }
        return Pop<T>::ldr(P + (size_t)j * N, idx);
    }
    // full population (shift added back), as Pop<T>::ld
    __device__ __forceinline__ float ld(int j, unsigned idx) const {
        if constexpr (std::is_same<T, __half>::value) return fmaf(raw(j, idx), kF16InvScale, sh[j]);
        else return raw(j, idx) + sh[j];
    }
    // deviation, as Pop<T>::ldd
    __device__ __forceinline__ float ldd(int j, unsigned idx) const {
        if constexpr (std::is_same<T, __half>::value) return raw(j, idx) * kF16InvScale;
        else return raw(j, idx);
    }
    __device__ __forceinline__ uint32_t flag(unsigned idx) const {
        using C = TilesCfg<T, TH>;
        const long long o = (long long)idx - n0;
        if (o >= 0 && o < kTW) return reinterpret_cast<const uint32_t*>(stage + C::FLAGS_OFF)[o];
        return __ldg(gflags + idx);
    }
};

template <class T, bool TH>
__device__ __forceinline__ TileSrc<T, TH> tile_src(const KParams& p, const unsigned char* stage, const TileHdr& h,
                                                   bool g) {
    return {stage, g ? 9 : 0, (long long)h.n0, h.leads, p.nx, static_cast<const T*>(g ? p.gin : p.fin),
            (size_t)p.N, g ? p.shg : p.shf, p.flags};
}

// Raw (storage-unit) or deviation pulls of node (x, y) through a tile source,
// with the periodic wrap: the pull_raw / pull_dev of the other kernels.
template <class S>
__device__ __forceinline__ void pull_via(const KParams& p, const S& src, int x, int y, float d[9], bool dev) {
    const unsigned nx = (unsigned)p.nx, ny = (unsigned)p.ny;
    const unsigned ux = (unsigned)x, uy = (unsigned)y;
    const unsigned xm = ux == 0 ? nx - 1 : ux - 1, xp = ux == nx - 1 ? 0 : ux + 1;
    const unsigned ym = uy == 0 ? ny - 1 : uy - 1, yp = uy == ny - 1 ? 0 : uy + 1;
    const unsigned r0 = uy * nx, rm = ym * nx, rp = yp * nx;
    const unsigned idx[9] = {r0 + ux, r0 + xm, rm + ux, r0 + xp, rp + ux, rm + xm, rm + xp, rp + xp, rp + xm};
#pragma unroll
    for (int j = 0; j < 9; ++j) d[j] = dev ? src.ldd(j, idx[j]) : src.raw(j, idx[j]);
}

// Two x-neighbours in storage units stored as a pair, or as two elements
// (element j*N + n odd for odd N and odd j) with the same rounding bits.
template <class T>
__device__ __forceinline__ void store_two(T* __restrict__ base, size_t n, float a, float b, uint32_t rb, bool pair,
                                          bool vb) {
    if (pair && vb) {
        PairStore<T>::st(base, n, a, b, rb);
        return;
    }
    if constexpr (std::is_same<T, float>::value) {
        base[n] = a;
        if (vb) base[n + 1] = b;
    } else {
        const uint32_t w = std::is_same<T, __half>::value ? cvt_rs_f16x2(a, b, rb) : cvt_rs_bf16x2(a, b, rb);
        reinterpret_cast<unsigned short*>(base)[n] = (unsigned short)(w & 0xFFFFu);
        if (vb) reinterpret_cast<unsigned short*>(base)[n + 1] = (unsigned short)(w >> 16);
    }
}

// Momentum exchange of one fluid boundary node (src/lbm.hpp:565-577) from
// its post-stream full populations f: the link terms 2 f (exact in FP32) are
// summed in FP32 into (fx, fy), a node pair's sum, which the caller adds to
// the lane's FP64 accumulator -- the accumulation every pair kernel uses.
__device__ __forceinline__ void link_terms(const KParams& p, uint32_t fl, const float f[9], float& fx, float& fy) {
    const uint32_t m = p.rec_force[fl >> 2];
#pragma unroll
    for (int j = 1; j < 9; ++j)
        if (m & (1u << j)) {
            fx -= float(CXf(j)) * 2.0f * f[j];
            fy -= float(CYf(j)) * 2.0f * f[j];
        }
}

// Non-thermal: nodes i, i+1 of the tile (pair), as consume_pair of the row
// pipeline with window pulls.
template <class T>
__device__ __forceinline__ void tile_pair(const KParams& p, const unsigned char* stage, const TileHdr& h, int i,
                                          uint32_t skey, double2* acc) {
    using C = TilesCfg<T, false>;
    const long long N = p.N;
    const unsigned na = (unsigned)h.n0 + (unsigned)i;
    const bool vb = (long long)na + 1 < N;
    int xa, ya, xb, yb;
    tile_xy(h.x0, h.y0, i, p.nx, p.inv_nx, xa, ya);
    xb = xa + 1;
    yb = ya;
    if (xb == p.nx) {
        xb = 0;
        ++yb;
    }
    const uint32_t* sfl = reinterpret_cast<const uint32_t*>(stage + C::FLAGS_OFF);
    const uint32_t fla = sfl[i];
    const uint32_t flb = vb ? sfl[i + 1] : FLAG_SOLID;
    const bool oka = !(fla & FLAG_SOLID), okb = vb && !(flb & FLAG_SOLID);
    const bool sa = border(p, xa, ya) || special_node<false>(p, xa, ya, fla);
    const bool sb = vb && (border(p, xb, yb) || special_node<false>(p, xb, yb, flb));
    // solid nodes whose state can no longer change skip their stores; decided
    // here so that no coordinate stays live across the collision
    const bool settled = p.skip_settled_solids != 0;
    const bool skip = (!oka && settled && xa > 0 && xa < p.nx - 1 && ya < p.ny - 1) &&
                      (!vb || (!okb && settled && xb > 0 && xb < p.nx - 1 && yb < p.ny - 1));
    float da[9], db[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const int lead = (h.leads >> (3 * j)) & 7;
        da[j] = staged<T, false>(stage, j, lead, i, CXf(j));
        db[j] = staged<T, false>(stage, j, lead, i + 1, CXf(j));
    }
    if (sa || sb) {
        // rebuild through the staged windows (device memory only for
        // sources outside them): build_dev_s of the other kernels, one node
        // at a time through a single copy of the (large) rebuild code
        const TileSrc<T, false> src = tile_src<T, false>(p, stage, h, false);
        float fxs = 0.0f, fys = 0.0f;  // the pair's link terms, node a then node b
#pragma unroll 1
        for (int k = 0; k < 2; ++k) {
            if (!(k ? sb : sa)) continue;
            const int xk = k ? xb : xa, yk = k ? yb : ya;
            const uint32_t flk = k ? flb : fla;
            float d[9];
            if (special_node<false>(p, xk, yk, flk)) {
                float f[9], g[9];
                build_state_src<T, false, true>(p, src, src, xk, yk, flk, f, g);
                if (h.slot >= 0 && !(flk & FLAG_SOLID) && (flk & FLAG_BOUNDARY)) link_terms(p, flk, f, fxs, fys);
#pragma unroll
                for (int j = 0; j < 9; ++j) d[j] = (f[j] - p.shf[j]) * Pop<T>::kS;
            } else {
                pull_via(p, src, xk, yk, d, false);
            }
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                if (k) db[j] = d[j];
                else da[j] = d[j];
            }
        }
        if (fxs != 0.0f || fys != 0.0f) {  // FP64 across the lane's node pairs
            acc->x += double(fxs);
            acc->y += double(fys);
        }
    }
    if (oka || okb) {
        F2 f[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = mk2(da[j], db[j]);
        collide_pair_dev<T>(p, fla, flb, oka, okb, f);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            da[j] = f[j].v.x;
            db[j] = f[j].v.y;
        }
    }  // solid nodes hold the solid state from build_dev_s
    if (!skip) {
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        uint32_t rb[9] = {};
        if constexpr (Pop<T>::kRounds) rand9(skey + na, rb);
        const bool even_n = (N & 1) == 0;
#pragma unroll
        for (int j = 0; j < 9; ++j)
            store_two<T>(Fo + (size_t)j * (size_t)N, na, da[j], db[j], rb[j], even_n || (j & 1) == 0, vb);
    }
}

// Thermal: one node of the tile (local index i), as step_block<T, true>.
template <class T>
__device__ __forceinline__ void tile_node_th(const KParams& p, const unsigned char* stage, const TileHdr& h, int i,
                                             uint32_t skey, double2* acc) {
    using C = TilesCfg<T, true>;
    constexpr float iS = Pop<T>::kInvS;
    const long long N = p.N;
    const unsigned n = (unsigned)h.n0 + (unsigned)i;
    int x, y;
    tile_xy(h.x0, h.y0, i, p.nx, p.inv_nx, x, y);
    const uint32_t fl = reinterpret_cast<const uint32_t*>(stage + C::FLAGS_OFF)[i];
    float d[9], e[9];  // deviations
    if (special_node<true>(p, x, y, fl)) {
        // build_dev<T, true> through the staged windows
        const TileSrc<T, true> sf = tile_src<T, true>(p, stage, h, false), sg = tile_src<T, true>(p, stage, h, true);
        float f[9], g[9];
        build_state_src<T, true, true>(p, sf, sg, x, y, fl, f, g);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            d[j] = f[j] - p.shf[j];
            e[j] = g[j] - p.shg[j];
        }
    } else if (border(p, x, y)) {
        pull_via(p, tile_src<T, true>(p, stage, h, false), x, y, d, true);
        pull_via(p, tile_src<T, true>(p, stage, h, true), x, y, e, true);
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const int lead = (h.leads >> (3 * j)) & 7;
            d[j] = staged<T, true>(stage, j, lead, i, CXf(j)) * iS;
            e[j] = staged<T, true>(stage, 9 + j, lead, i, CXf(j)) * iS;
        }
    }
    const bool ok = !(fl & FLAG_SOLID);
    if (ok) {
        if (h.slot >= 0 && (fl & FLAG_BOUNDARY)) {
            // the node's link terms in FP32, then FP64 (as the one-node kernel)
            float f[9], fx = 0.0f, fy = 0.0f;
#pragma unroll
            for (int j = 0; j < 9; ++j) f[j] = d[j] + p.shf[j];
            link_terms(p, fl, f, fx, fy);
            acc->x += double(fx);
            acc->y += double(fy);
        }
        collide_dev<true>(p, fl, d, e);
    }
    if (!(!ok && p.skip_settled_solids && x > 0 && x < p.nx - 1 && y < p.ny - 1)) {
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        T* __restrict__ Go = static_cast<T*>(p.gout);
        uint32_t rb[9] = {};
        if constexpr (Pop<T>::kRounds) rand9(skey + n, rb);
#pragma unroll
        for (int j = 0; j < 9; ++j) Pop<T>::std_(Fo + (size_t)j * (size_t)N, n, d[j], rb[j]);
        if constexpr (Pop<T>::kRounds) rand9((skey + n) ^ 0x6A09E667u, rb);
#pragma unroll
        for (int j = 0; j < 9; ++j) Pop<T>::std_(Go + (size_t)j * (size_t)N, n, e[j], rb[j]);
    }
}

template <class T, bool TH, bool SINGLE>
__device__ __forceinline__ void tiles_consume(const KParams& single, unsigned char* smem, uint32_t full0, uint32_t empty0,
                              unsigned int* status) {
    using C = TilesCfg<T, TH>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tid = threadIdx.x;  // consumer thread 0..255
    double2* acc = reinterpret_cast<double2*>(smem + C::ACC_OFF);
    const long long cw = single.consumer_wait;
    const long long wait_limit = cw != 0 ? (cw > 0 ? cw : -cw) : kWaitCycles;
    int s = 0;
    uint32_t phase = 0;
    for (;;) {
        if (!__all_sync(0xffffffffu, mbar_wait(full0 + 8 * s, phase, wait_limit))) {
            if (lane == 0) atomicOr(status, 2u);
            break;
        }
        const unsigned char* stage = smem + s * C::STAGE_BYTES;
        const TileHdr& h = *reinterpret_cast<const TileHdr*>(stage + C::HDR_OFF);  // read in place: no registers
        if (h.k < 0) break;
        const KParams& p = tile_params<SINGLE>(single, stage, C::PAR_OFF);
        const uint32_t skey = Pop<T>::kRounds ? seed_key(h.seed) : 0u;
        if (h.slot >= 0) acc[tid] = make_double2(0.0, 0.0);
        if constexpr (TH) {
            // one node at a time: lanes take consecutive nodes (tid, then
            // tid + W/2), so staged reads and stores are unit-stride; one
            // copy of the node code
#pragma unroll 1
            for (int i = tid; i < kTW; i += kTW / 2)
                if ((long long)h.n0 + i < p.N) tile_node_th<T>(p, stage, h, i, skey, acc + tid);
        } else {
            const int i = 2 * tid;
            if ((long long)h.n0 + i < p.N) tile_pair<T>(p, stage, h, i, skey, acc + tid);
        }
        if (h.slot >= 0) {
            // FP64 warp sum of the tile's link terms into its per-warp slot
            double a = acc[tid].x, b = acc[tid].y;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a += __shfl_down_sync(0xffffffffu, a, o);
                b += __shfl_down_sync(0xffffffffu, b, o);
            }
            if (lane == 0) {
                p.partials[2 * (h.slot + warp)] = a;
                p.partials[2 * (h.slot + warp) + 1] = b;
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8 * s);
        if (++s == C::STAGES) {
            s = 0;
            phase ^= 1u;
        }
    }
    if constexpr (SINGLE) {
        // the drag/lift second stage in the last CTA holding force tiles: the
        // host marks those CTAs (tile t runs on CTA t / ceil(T / grid)) after the
        // per-tile entries of the slot table, so every marked CTA counts
        // itself even when one of its waits ran out
        const int ntiles = (int)((single.N + kTW - 1) / kTW);
        if (single.red_done && single.block_slot && __ldg(single.block_slot + ntiles + blockIdx.x) > 0)
            fused_force_finish(single, tid, [] { asm volatile("bar.sync 1, %0;" ::"n"(32 * kTWarps) : "memory"); });
    }
}

template <class T, bool TH, bool SINGLE>
__global__ void __launch_bounds__(kTThreads, 2)
    step_tiles_kernel(const KParams single, const KParams* __restrict__ inst,
                      const int* __restrict__ tile_member, const int* __restrict__ tile_start, int ntiles,
                      unsigned int* status) {
    using C = TilesCfg<T, TH>;
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t sbase = smem_u32(smem);
    const uint32_t full0 = sbase + C::BAR_OFF, empty0 = full0 + 8 * C::STAGES;
    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, kTWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned int* st = SINGLE ? single.nan_flag : status;
    if ((threadIdx.x >> 5) == kTWarps) {
        // (a negative consumer_wait is the failure-path test: nothing is staged)
        if (single.consumer_wait >= 0)
            tiles_produce<T, TH, SINGLE>(single, inst, tile_member, tile_start, ntiles, smem, sbase, full0, empty0,
                                         st);
        return;
    }
    tiles_consume<T, TH, SINGLE>(single, smem, full0, empty0, st);
}

template <class T, bool TH, bool SINGLE>
int tiles_set_smem(int dev) {
    static std::atomic<unsigned long long> done{0};
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return 0;
    const cudaError_t e = cudaFuncSetAttribute(step_tiles_kernel<T, TH, SINGLE>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, TilesCfg<T, TH>::SMEM);
    if (e != cudaSuccess) return (int)e;
    done.fetch_or(bit);
    return 0;
}

template <class T, bool TH>
int tiles_per_sm(int dev) {
    static int cached[2] = {-1, -1};
    if (cached[TH] < 0) {
        int b0 = 0, b1 = 0;
        if (tiles_set_smem<T, TH, true>(dev) || tiles_set_smem<T, TH, false>(dev)) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, step_tiles_kernel<T, TH, true>, kTThreads,
                                                          TilesCfg<T, TH>::SMEM) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, step_tiles_kernel<T, TH, false>, kTThreads,
                                                          TilesCfg<T, TH>::SMEM) != cudaSuccess)
            return 0;
        cached[TH] = std::min(b0, b1);
    }
    return cached[TH];
}

template <class T, bool TH>
int tiles_grid_t(long long ntiles, int dev) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    const int per = tiles_per_sm<T, TH>(dev);
    if (per <= 0) return 0;
    return (int)std::max<long long>(1, std::min<long long>(ntiles, (long long)sms * per));
}

template <class T, bool TH, bool SINGLE>
int launch_tiles_t(const KParams& p, const KParams* inst, const int* tm, const int* ts, int ntiles, int grid,
                   unsigned int* status, cudaStream_t s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (const int r = tiles_set_smem<T, TH, SINGLE>(dev)) return r;
    if (grid <= 0) return (int)cudaErrorInvalidConfiguration;
    step_tiles_kernel<T, TH, SINGLE><<<grid, kTThreads, TilesCfg<T, TH>::SMEM, s>>>(p, inst, tm, ts, ntiles, status);
    return (int)cudaGetLastError();
}

}  // namespace

int tiles_width() { return kTW; }
int tiles_warps() { return kTWarps; }

int tiles_grid(int storage, bool thermal, long long ntiles, int device) {
    switch (storage) {
        case ST_FP32: return thermal ? tiles_grid_t<float, true>(ntiles, device) : tiles_grid_t<float, false>(ntiles, device);
        case ST_FP16: return thermal ? tiles_grid_t<__half, true>(ntiles, device) : tiles_grid_t<__half, false>(ntiles, device);
        case ST_BF16:
            return thermal ? tiles_grid_t<__nv_bfloat16, true>(ntiles, device)
                           : tiles_grid_t<__nv_bfloat16, false>(ntiles, device);
    }
    return 0;
}

int launch_tiles_single(int storage, const KParams& p, int grid, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nt = (int)((p.N + kTW - 1) / kTW);
    const bool th = p.thermal != 0;
#define LBM2D_TILES1(T)                                                                               \
    return th ? launch_tiles_t<T, true, true>(p, nullptr, nullptr, nullptr, nt, grid, nullptr, s) \
              : launch_tiles_t<T, false, true>(p, nullptr, nullptr, nullptr, nt, grid, nullptr, s)
    switch (storage) {
        case ST_FP32: LBM2D_TILES1(float);
        case ST_FP16: LBM2D_TILES1(__half);
        case ST_BF16: LBM2D_TILES1(__nv_bfloat16);
    }
#undef LBM2D_TILES1
    return (int)cudaErrorInvalidValue;
}

int launch_tiles_batch(int storage, bool thermal, const KParams* inst, const int* tile_member, const int* tile_start,
                       int ntiles, int grid, unsigned int* status, void* stream) {
    if (ntiles <= 0) return 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    KParams none;
    memset(&none, 0, sizeof(none));
#define LBM2D_TILESB(T)                                                                                         \
    return thermal ? launch_tiles_t<T, true, false>(none, inst, tile_member, tile_start, ntiles, grid, status, s) \
                   : launch_tiles_t<T, false, false>(none, inst, tile_member, tile_start, ntiles, grid, status, s)
    switch (storage) {
        case ST_FP32: LBM2D_TILESB(float);
        case ST_FP16: LBM2D_TILESB(__half);
        case ST_BF16: LBM2D_TILESB(__nv_bfloat16);
    }
#undef LBM2D_TILESB
    return (int)cudaErrorInvalidValue;
}

}  // namespace lbm2d
