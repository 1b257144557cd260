// lbm2d_rows.cu -- the row-pipelined step kernel (sm_103a).
//
// The same step as step_pair_kernel (pull, rebuild, force, packed FP32x2
// collision, store), with the pulls served from shared memory that the
// Blackwell bulk-copy engine fills ahead of the computation:
//
//   * work unit = a row tile: W = 512 consecutive nodes of one lattice row
//     (nx a multiple of 4 for FP32, 8 for FP16/BF16, so every row starts on
//     a 16-byte boundary).  The 9 source rows of a tile (direction j reads
//     row y - cy_j, x range [x0 - PAD, x0 + W + PAD)) and the tile's flags
//     are brought in by 10 cp.async.bulk copies (plus 16-byte copies for the
//     periodic x wrap at the row ends), completing on an mbarrier;
//   * a persistent grid (a multiple of the SM count) walks the tiles; each
//     CTA keeps S tiles in flight in a ring of shared-memory stages;
//   * warp 8 is the producer (one elected lane issues the copies), warps 0-7
//     consume: each lane owns two x-neighbours of the tile.
// The copies move the source bytes with no load instructions, so the
// consumer warps spend their issue slots on the collision and the stores,
// and the bytes in flight per SM no longer depend on how many warps happen
// to be waiting on loads.
//
// Every wait is bounded: after kWaitCycles SM cycles a waiting thread sets
// bit 1 of the solver's status word (the host reports a pipeline timeout)
// and leaves its loop; the producer waits, again bounded, for the copies it
// issued before it exits.  No wait can time out in a correct launch: the
// copies of a tile complete in microseconds.
#include <algorithm>
#include <atomic>

#include "lbm2d_pipeline.cuh"

namespace lbm2d {
namespace {

constexpr int kConsumerWarps = 8;
constexpr int kThreads = 32 * (kConsumerWarps + 1);
constexpr int kTileW = 2 * 32 * kConsumerWarps;  // nodes per row tile

template <class T>
struct RowsCfg {
    static constexpr int ES = (int)sizeof(T);
    static constexpr int PAD = 16 / ES;  // halo rounded to the 16-byte copy granule
    static constexpr int SW = kTileW + 2 * PAD;  // elements per staged row
    static constexpr int ROW_BYTES = SW * ES;
    static constexpr int FLAGS_OFF = 9 * ROW_BYTES;
    static constexpr int STAGE_BYTES = ((FLAGS_OFF + kTileW * 4) + 127) / 128 * 128;
    // FP32 moves twice the bytes per node: 2 CTAs per SM with deeper
    // registers and a 3-tile ring (measured faster than 4 or 5 tiles in
    // flight); the 16-bit forms are latency-bound on the arithmetic: 3 CTAs
    // with a 6-tile ring (70 KB each, 210 KB per SM; measured +0.6% on the
    // 4096^2 channel and +4% on 2048^2 against a 4-tile ring)
    static constexpr int STAGES = ES == 4 ? 3 : 6;
    static constexpr int MIN_BLOCKS = ES == 4 ? 2 : 3;
    static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
    // FP64 momentum-exchange sums, one (fx, fy) pair per consumer lane
    static constexpr int ACC_OFF = BAR_OFF + 2 * STAGES * 8;
    static constexpr int SMEM = ACC_OFF + 32 * kConsumerWarps * 16;
    static_assert(ROW_BYTES % 16 == 0 && FLAGS_OFF % 16 == 0, "bulk-copy alignment");
};

// ----------------------------------------------------------------- producer
// Bytes the copies of the tile starting at x0 complete on its mbarrier.
template <class T>
__device__ __forceinline__ uint32_t tile_bytes(const KParams& p, int x0) {
    using C = RowsCfg<T>;
    const int xs = max(x0 - C::PAD, 0), xe = min(x0 + kTileW + C::PAD, p.nx);
    uint32_t b = 9u * (uint32_t)((xe - xs) * C::ES);
    if (x0 == 0) b += 3u * 16u;                  // x = -1 of the three cx = +1 rows
    if (x0 + kTileW >= p.nx) b += 3u * 16u;      // x = nx of the three cx = -1 rows
    b += (uint32_t)((min(x0 + kTileW, p.nx) - x0) * 4);  // flags
    return b;
}

// Issue the copies of the tile (x0, y) into the stage at shared address st.
template <class T>
__device__ __forceinline__ void issue_tile(const KParams& p, int x0, int y, uint32_t st, uint32_t bar) {
    using C = RowsCfg<T>;
    const T* __restrict__ P = static_cast<const T*>(p.fin);
    const size_t N = (size_t)p.N;
    const int nx = p.nx, ny = p.ny;
    const int xs = max(x0 - C::PAD, 0), xe = min(x0 + kTileW + C::PAD, nx);
    const uint32_t dst_off = (uint32_t)((xs - (x0 - C::PAD)) * C::ES);
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        int ys = y - CYf(j);
        ys = ys < 0 ? ys + ny : (ys >= ny ? ys - ny : ys);
        const T* row = P + j * N + (size_t)ys * nx;
        const uint32_t rdst = st + (uint32_t)(j * C::ROW_BYTES);
        bulk_g2s(rdst + dst_off, row + xs, (uint32_t)((xe - xs) * C::ES), bar);
        if (CXf(j) == 1 && x0 == 0)  // periodic x: x = -1 is x = nx - 1
            bulk_g2s(rdst, row + (nx - C::PAD), 16u, bar);
        if (CXf(j) == -1 && x0 + kTileW >= nx)  // x = nx is x = 0
            bulk_g2s(rdst + (uint32_t)((nx - x0 + C::PAD) * C::ES), row, 16u, bar);
    }
    const int fe = min(x0 + kTileW, nx);
    bulk_g2s(st + C::FLAGS_OFF, p.flags + (size_t)y * nx + x0, (uint32_t)((fe - x0) * 4), bar);
}

// ----------------------------------------------------------------- consumer
// Elements e, e+1 of a staged row, in storage units (deviation * kS).
template <class T>
struct SmemPair;
template <>
struct SmemPair<float> {
    static __device__ __forceinline__ void aligned(const float* r, int e, float& a, float& b) {
        const float2 v = *reinterpret_cast<const float2*>(r + e);
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void any(const float* r, int e, float& a, float& b) {
        a = r[e];
        b = r[e + 1];
    }
};
template <>
struct SmemPair<__half> {
    static __device__ __forceinline__ void aligned(const __half* r, int e, float& a, float& b) {
        const float2 v = __half22float2(*reinterpret_cast<const __half2*>(r + e));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void any(const __half* r, int e, float& a, float& b) {
        a = __half2float(r[e]);
        b = __half2float(r[e + 1]);
    }
};
template <>
struct SmemPair<__nv_bfloat16> {
    static __device__ __forceinline__ void aligned(const __nv_bfloat16* r, int e, float& a, float& b) {
        const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(r + e));
        a = v.x;
        b = v.y;
    }
    static __device__ __forceinline__ void any(const __nv_bfloat16* r, int e, float& a, float& b) {
        a = __bfloat162float(r[e]);
        b = __bfloat162float(r[e + 1]);
    }
};

// Nodes (x, x+1) from their pulled values da, db (storage units, deviation
// * kS): the reference's post-stream state (bounce-back records, outflow
// column, boundary conditions), the momentum-exchange force, the collision
// and the stores -- the body of step_pair_block on deviations.  BND: the
// pair holds a boundary node and is rebuilt in full, reading device memory;
// otherwise its only special lanes are solid ones (f = 0).  The link terms of
// the two nodes (each 2 f, exact in FP32) are summed into (fxs, fys); the
// caller adds that pair sum to the lane's FP64 running sum.
template <class T, int KC, int KL, bool BND>
__device__ __forceinline__ void pair_body(const KParams& p, uint2 fl, int x, int y, float da[9], float db[9],
                                          uint32_t skey, float& fxs, float& fys) {
    const bool oka = !(fl.x & FLAG_SOLID), okb = !(fl.y & FLAG_SOLID);
    if constexpr (BND) {
        const bool sa = special_node<false>(p, x, y, fl.x), sb = special_node<false>(p, x + 1, y, fl.y);
        if (sa || sb) {
            // full populations for the special node(s)
            const T* __restrict__ Pf = static_cast<const T*>(p.fin);
            constexpr float S = Pop<T>::kS, iS = Pop<T>::kInvS;
            float fa[9], fb[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                fa[j] = fmaf(da[j], iS, p.shf[j]);
                fb[j] = fmaf(db[j], iS, p.shf[j]);
            }
            if (fl.x & FLAG_SOLID) {
#pragma unroll
                for (int j = 0; j < 9; ++j) fa[j] = 0.0f;
            } else if (fl.x & FLAG_BOUNDARY) {
                fix_f<T>(p, Pf, x, y, fl.x >> 2, fa);
            }
            // zero-gradient outlet: column NX-1 takes NX-2's post-stream state
            // (src/lbm.hpp:63-73); x + 1 == nx - 1 means x == nx - 2
            if ((p.bc_kind == BC_INFLOW || p.bc_kind == BC_STEP) && x + 1 == p.nx - 1) {
#pragma unroll
                for (int j = 0; j < 9; ++j) fb[j] = fa[j];
            } else if (fl.y & FLAG_SOLID) {
#pragma unroll
                for (int j = 0; j < 9; ++j) fb[j] = 0.0f;
            } else if (fl.y & FLAG_BOUNDARY) {
                fix_f<T>(p, Pf, x + 1, y, fl.y >> 2, fb);
            }
            apply_bc<float>(p, x, y, fl.x, fa);
            apply_bc<float>(p, x + 1, y, fl.y, fb);
            if ((fl.x | fl.y) & FLAG_BOUNDARY) {
                // momentum exchange of the nodes' links (src/lbm.hpp:565-577),
                // accumulated in FP64 (each term 2 f exact in FP64)
                const uint32_t ma = (oka && (fl.x & FLAG_BOUNDARY)) ? p.rec_force[fl.x >> 2] : 0u;
                const uint32_t mb = (okb && (fl.y & FLAG_BOUNDARY)) ? p.rec_force[fl.y >> 2] : 0u;
                // node x's links, then node x+1's (the order every pair kernel uses)
#pragma unroll
                for (int j = 1; j < 9; ++j)
                    if (ma & (1u << j)) {
                        fxs -= float(CXf(j)) * 2.0f * fa[j];
                        fys -= float(CYf(j)) * 2.0f * fa[j];
                    }
#pragma unroll
                for (int j = 1; j < 9; ++j)
                    if (mb & (1u << j)) {
                        fxs -= float(CXf(j)) * 2.0f * fb[j];
                        fys -= float(CYf(j)) * 2.0f * fb[j];
                    }
            }
            // back to deviations; a regular neighbour keeps its exact deviations
            if (sa) {
#pragma unroll
                for (int j = 0; j < 9; ++j) da[j] = (fa[j] - p.shf[j]) * S;
            }
            if (sb) {
#pragma unroll
                for (int j = 0; j < 9; ++j) db[j] = (fb[j] - p.shf[j]) * S;
            }
        }
    } else {
        constexpr float S = Pop<T>::kS;
        if (!oka) {
#pragma unroll
            for (int j = 0; j < 9; ++j) da[j] = -p.shf[j] * S;
        }
        if (!okb) {
#pragma unroll
            for (int j = 0; j < 9; ++j) db[j] = -p.shf[j] * S;
        }
    }
    if (oka || okb) {
        F2 f[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) f[j] = mk2(da[j], db[j]);
        collide_pair_dev<T, KC, KL>(p, fl.x, fl.y, oka, okb, f);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            da[j] = f[j].v.x;
            db[j] = f[j].v.y;
        }
    }
    const bool settled = p.skip_settled_solids && y < p.ny - 1;
    const bool skip_a = !oka && settled && x > 0;
    const bool skip_b = !okb && settled && x + 1 < p.nx - 1;
    if (!(skip_a && skip_b)) {
        T* __restrict__ Fo = static_cast<T*>(p.fout);
        const size_t N = (size_t)p.N;
        const size_t n0 = (size_t)y * p.nx + x;
        uint32_t rb[9] = {};
        if constexpr (Pop<T>::kRounds) rand9(skey + (uint32_t)n0, rb);
#pragma unroll
        for (int j = 0; j < 9; ++j) PairStore<T>::st(Fo + j * N, n0, da[j], db[j], rb[j]);
    }
}

// The 16-bit forms, bound by their instructions, leave the pairs that hold a
// boundary node to a boundary pass at the start of each CTA (boundary_pairs):
// inline, a warp with one boundary node runs the rebuild with all its lanes
// waiting (4096^2 LES channel, FP16: 112.0 against 107.5 GLUPS).  FP32,
// bound by HBM, keeps them inline: there the pass delays the CTA's first
// tiles, which the ring cannot absorb (75.7 against 77.0 GLUPS).
template <class T>
constexpr bool kBoundaryPass = sizeof(T) == 2;

// Nodes (x, x+1) of the tile staged at `stage` (x0 its first node), pulled
// from shared memory.  A settled solid pair needs no store.
template <class T, int KC, int KL>
__device__ __forceinline__ void consume_pair(const KParams& p, const unsigned char* stage, int x0, int x, int y,
                                             uint32_t skey, float& fxs, float& fys) {
    using C = RowsCfg<T>;
    const uint2 fl = *reinterpret_cast<const uint2*>(stage + C::FLAGS_OFF + (x - x0) * 4);
    if (kBoundaryPass<T> && ((fl.x | fl.y) & FLAG_BOUNDARY)) return;
    if ((fl.x & fl.y & FLAG_SOLID) && p.skip_settled_solids && y < p.ny - 1 && x > 0 && x + 1 < p.nx - 1) return;
    const int e0 = (x - x0) + C::PAD;
    float da[9], db[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const T* r = reinterpret_cast<const T*>(stage + j * C::ROW_BYTES);
        if (CXf(j) == 0)
            SmemPair<T>::aligned(r, e0, da[j], db[j]);
        else
            SmemPair<T>::any(r, e0 - CXf(j), da[j], db[j]);
    }
    pair_body<T, KC, KL, !kBoundaryPass<T>>(p, fl, x, y, da, db, skey, fxs, fys);
}

// The boundary pass: this CTA's chunk of the boundary pairs, one pair per
// consumer lane, pulled from device memory (the previous step's stored
// populations, which no tile of this launch writes) and rebuilt in full.
// Run before the CTA's first tile, so its device-memory latency overlaps
// the producer's filling of the ring.
template <class T, int KC, int KL>
__device__ __forceinline__ void boundary_pairs(const KParams& p, uint32_t skey, double2* acc) {
    const int b0 = (int)blockIdx.x * p.bchunk, b1 = min(b0 + p.bchunk, p.nbpairs);
    const T* __restrict__ P = static_cast<const T*>(p.fin);
    for (int i = b0 + (int)threadIdx.x; i < b1; i += 32 * kConsumerWarps) {
        const int n0 = p.bpairs[i];
        const int y = (int)((unsigned)n0 / (unsigned)p.nx), x = n0 - y * p.nx;
        const uint2 fl = make_uint2(p.flags[n0], p.flags[n0 + 1]);
        float da[9], db[9];
        pull_raw<T>(p, P, x, y, da);
        pull_raw<T>(p, P, x + 1, y, db);
        float fxs = 0.0f, fys = 0.0f;
        pair_body<T, KC, KL, true>(p, fl, x, y, da, db, skey, fxs, fys);
        if (fxs != 0.0f || fys != 0.0f) {
            acc[threadIdx.x].x += double(fxs);
            acc[threadIdx.x].y += double(fys);
        }
    }
}

// KC: 0 MRT, 1 BGK; KL: LES on/off (MRT only); -1: read from the parameters.
template <class T, int KC, int KL>
__global__ void __launch_bounds__(kThreads, RowsCfg<T>::MIN_BLOCKS) step_rows_kernel(const KParams p) {
    using C = RowsCfg<T>;
    extern __shared__ __align__(128) unsigned char smem[];
    const uint32_t sbase = smem_u32(smem);
    const uint32_t full0 = sbase + C::BAR_OFF, empty0 = full0 + 8 * C::STAGES;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tpr = (p.nx + kTileW - 1) / kTileW;
    // tile t = y * tpr + seg, walked t = blockIdx.x, blockIdx.x + G, ... with
    // (y, seg) advanced incrementally
    const int G = (int)gridDim.x, dy = G / tpr, dseg = G - dy * tpr;
    const int y_first = (int)blockIdx.x / tpr, seg_first = (int)blockIdx.x - y_first * tpr;
    double2* acc = reinterpret_cast<double2*>(smem + C::ACC_OFF);
    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, kConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < 32 * kConsumerWarps) acc[threadIdx.x] = make_double2(0.0, 0.0);
    __syncthreads();

    if (warp == kConsumerWarps) {  // producer
        if (lane != 0) return;
        if (p.consumer_wait < 0) return;  // failure-path test: nothing is staged, every consumer wait runs out
        int k = 0;  // tiles issued
        bool ok = true;
        int y = y_first, seg = seg_first;
        for (; y < p.ny; ++k) {
            const int s = k % C::STAGES, n = k / C::STAGES;
            if (n > 0 && !mbar_wait(empty0 + 8 * s, (uint32_t)((n - 1) & 1))) {
                ok = false;
                break;
            }
            const int x0 = seg * kTileW;
            const uint32_t bar = full0 + 8 * s;
            mbar_expect_tx(bar, tile_bytes<T>(p, x0));
            issue_tile<T>(p, x0, y, sbase + (uint32_t)(s * C::STAGE_BYTES), bar);
            seg += dseg;
            y += dy;
            if (seg >= tpr) {
                seg -= tpr;
                ++y;
            }
        }
        // every issued copy completes before the CTA may exit
        bool drained = true;
        for (int i = max(k - C::STAGES, 0); i < k; ++i)
            drained = mbar_wait(full0 + 8 * (i % C::STAGES), (uint32_t)((i / C::STAGES) & 1)) && drained;
        if (!ok || !drained) atomicOr(p.nan_flag, 2u);
        return;
    }

    // consumers
    uint32_t skey = 0;
    if constexpr (Pop<T>::kRounds) {
        const uint32_t s = seed_of(p);
        skey = seed_key(s);
        pass_seed(p, s, blockIdx.x == 0 && threadIdx.x == 0);
    }
    if constexpr (kBoundaryPass<T>)
        if (p.nbpairs > 0) boundary_pairs<T, KC, KL>(p, skey, acc);
    const bool force = p.block_slot != nullptr;
    const long long wait_limit = p.consumer_wait != 0 ? (p.consumer_wait > 0 ? p.consumer_wait : -p.consumer_wait)
                                                      : kWaitCycles;
    int y = y_first, seg = seg_first, s = 0;
    uint32_t phase = 0;
    while (y < p.ny) {
        // the whole warp leaves together when a wait runs out; the producer
        // then runs out on the stage it would refill, drains its copies and
        // the CTA ends
        if (!__all_sync(0xffffffffu, mbar_wait(full0 + 8 * s, phase, wait_limit))) {
            if (lane == 0) atomicOr(p.nan_flag, 2u);
            break;
        }
        const int x0 = seg * kTileW;
        const int x = x0 + 2 * (warp * 32 + lane);
        float fxs = 0.0f, fys = 0.0f;
        if (x < p.nx) consume_pair<T, KC, KL>(p, smem + s * C::STAGE_BYTES, x0, x, y, skey, fxs, fys);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty0 + 8 * s);
        if (fxs != 0.0f || fys != 0.0f) {  // the lane's FP64 running sum over its node pairs
            acc[threadIdx.x].x += double(fxs);
            acc[threadIdx.x].y += double(fys);
        }
        if (++s == C::STAGES) {
            s = 0;
            phase ^= 1u;
        }
        seg += dseg;
        y += dy;
        if (seg >= tpr) {
            seg -= tpr;
            ++y;
        }
    }
    if (force) {
        const int base = p.block_slot[blockIdx.x];  // uniform per CTA
        if (base >= 0) {
            // FP64 warp sum of the lanes' accumulators (fixed shuffle tree)
            double a = acc[threadIdx.x].x, b = acc[threadIdx.x].y;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a += __shfl_down_sync(0xffffffffu, a, o);
                b += __shfl_down_sync(0xffffffffu, b, o);
            }
            if (lane == 0) {
                p.partials[2 * (base + warp)] = a;
                p.partials[2 * (base + warp) + 1] = b;
            }
            // the producer warp has left: the consumers' own named barrier
            if (p.red_done)
                fused_force_finish(p, warp * 32 + lane, [] { asm volatile("bar.sync 1, 256;" ::: "memory"); });
        }
    }
}

template <class T, int KC, int KL>
int rows_blocks_per_sm() {
    static int cached = -1;
    if (cached < 0) {
        int b = 0;
        if (cudaFuncSetAttribute(step_rows_kernel<T, KC, KL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 RowsCfg<T>::SMEM) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, step_rows_kernel<T, KC, KL>, kThreads,
                                                          RowsCfg<T>::SMEM) != cudaSuccess)
            return 0;
        cached = b;
    }
    return cached;
}

// FP32 runs one kernel with the collision mode read at run time; the 16-bit
// forms, which are bound by their arithmetic, get one kernel per mode
// (fewer branches and registers in the hot loop).  Both choices were the
// faster ones measured on the 4096^2 channel.
template <class T>
constexpr bool kPerMode = !std::is_same<T, float>::value;

// Smallest resident-CTA count over the kernel's variants, so one grid (and
// one force-slot table) serves every collision mode.
template <class T>
int rows_grid_t(int nx, int ny, int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    int per = 0;
    if constexpr (kPerMode<T>)
        per = std::min({rows_blocks_per_sm<T, 0, 0>(), rows_blocks_per_sm<T, 0, 1>(), rows_blocks_per_sm<T, 1, 0>()});
    else
        per = rows_blocks_per_sm<T, -1, -1>();
    if (per <= 0) return 0;
    const long long tiles = (long long)((nx + kTileW - 1) / kTileW) * ny;
    return (int)std::min<long long>(tiles, (long long)sms * per);
}

template <class T, int KC, int KL>
int launch_rows_v(const KParams& p, int grid, cudaStream_t s) {
    // the shared-memory opt-in is per device: set it once for each
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(done.load() & bit)) {
        e = cudaFuncSetAttribute(step_rows_kernel<T, KC, KL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 RowsCfg<T>::SMEM);
        if (e != cudaSuccess) return (int)e;
        done.fetch_or(bit);
    }
    step_rows_kernel<T, KC, KL><<<grid, kThreads, RowsCfg<T>::SMEM, s>>>(p);
    return (int)cudaGetLastError();
}

template <class T>
int launch_rows_t(const KParams& p, int grid, cudaStream_t s) {
    if (grid <= 0) return (int)cudaErrorInvalidConfiguration;
    if constexpr (!kPerMode<T>) {
        return launch_rows_v<T, -1, -1>(p, grid, s);
    } else {
        if (p.collision != 0) return launch_rows_v<T, 1, 0>(p, grid, s);
        return p.les ? launch_rows_v<T, 0, 1>(p, grid, s) : launch_rows_v<T, 0, 0>(p, grid, s);
    }
}

}  // namespace

// Every staged row must start on a 16-byte boundary: nx a multiple of 4
// (FP32) or 8 (FP16/BF16).
bool rows_boundary_pass(int storage) { return storage == ST_FP16 || storage == ST_BF16; }

bool rows_eligible(int storage, int nx, int ny, bool thermal) {
    const int q = storage == ST_FP32 ? 4 : 8;
    return !thermal && (storage == ST_FP32 || storage == ST_FP16 || storage == ST_BF16) && nx % q == 0 && nx >= 16 &&
           ny >= 2;
}

int rows_tile_width() { return kTileW; }

int rows_warps_per_block() { return kConsumerWarps; }

int rows_grid(int storage, int nx, int ny, int device) {
    switch (storage) {
        case ST_FP32: return rows_grid_t<float>(nx, ny, device);
        case ST_FP16: return rows_grid_t<__half>(nx, ny, device);
        case ST_BF16: return rows_grid_t<__nv_bfloat16>(nx, ny, device);
    }
    return 0;
}

int launch_rows(int storage, const KParams& p, int grid, void* stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (storage) {
        case ST_FP32: return launch_rows_t<float>(p, grid, s);
        case ST_FP16: return launch_rows_t<__half>(p, grid, s);
        case ST_BF16: return launch_rows_t<__nv_bfloat16>(p, grid, s);
    }
    return (int)cudaErrorInvalidValue;
}

}  // namespace lbm2d
