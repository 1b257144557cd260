// lbm2d_resident.cu -- the resident serving loop.
//
// Every member of a serving table is stepped once per iteration of a CUDA
// graph WHILE loop, and members join and retire at every step boundary, with
// no host round trip between steps:
//
//   pre-launch schedule  ->  while (cond) { S0 -> T0 -> S1 -> T1 }
//
//   * S_b: one step kernel per member kind in use ("combo": storage x
//     paired / one-node / one-node thermal), a fixed grid whose blocks take
//     the work units of the members listed in list buffer b from a counter.
//     A unit is one launch block of the batched kernels (kBatchTiles tiles
//     of a member, or one boundary block of a paired member), so a member's
//     step is computed exactly as lbm2d_batch_step computes it.
//   * T_b: the tail.  Blocks 1.. reduce the force partials of the members
//     stepped from buffer b (same order and width as the batched reduction);
//     block 0 schedules the next iteration into buffer 1 - b: it admits the
//     members the host has announced in the mailbox (mapped host memory),
//     retires the members whose budget is spent once their last reduction is
//     complete (writing the steps they took to the mailbox), lists the
//     others per combo with their units, flips their parities and sets the
//     loop condition.
//
// The body holds two iterations so that no kernel reads a word the same
// kernel writes: T0 lists into buffer 1 while its reducers read buffer 0.
// A tail that ends the loop empties the other buffer, so the rest of the
// body does nothing.  The loop ends when no member is active, at the host's
// stop word, or after a bounded number of iterations; nothing in it waits
// on another block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "lbm2d_device.cuh"

namespace lbm2d {

namespace {

constexpr int kTailThreads = 256;
constexpr int kSlotsPerThread = kResMaxSlots / kTailThreads;  // 4

// Device-side state of a loop, passed by value to its kernels.
struct ResDev {
    ResEntry* table;        // [cap]
    ResMailbox* mb;         // device alias of the mapped mailbox
    int* state;             // [cap] 0 free, 1 active
    int* parity;            // [cap] parity of the member's next step
    int* taken;             // [cap] steps taken since it joined
    long long* last_it;     // [cap] iteration of its last step (-1: none)
    int* count;             // [2][kResCombos] members listed per combo
    int* start;             // [2][kResCombos][cap + 1] first unit of each listed member
    const KParams** params; // [2][kResCombos][cap] the listed members' step parameters
    ReduceJob* jobs;        // [2][cap]
    int* ctr;               // [2][kResCombos] units taken by the step kernels
    int* njobs;             // [2]
    long long* it;          // [0] last committed iteration, [1] iterations of this launch, [2] halted,
                            // [3] the join_gen last acted on
    int cap;
    int max_iters;
    unsigned combo_mask;  // combos with a step kernel in the graph
    cudaGraphConditionalHandle cond;
};

__device__ __forceinline__ int ld_vol(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
// acquire load at system scope: the host's writes before it are visible after it
__device__ __forceinline__ int ld_acquire_sys(const int* p) {
    int v;
    asm volatile("ld.acquire.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Exclusive block scan of a 64-bit value (kTailThreads threads); total in *tot.
__device__ __forceinline__ long long block_scan64(long long v, long long* tot) {
    __shared__ long long s_w[kTailThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    long long base = 0, all = 0;
#pragma unroll
    for (int i = 0; i < kTailThreads / 32; ++i) {
        if (i < w) base += s_w[i];
        all += s_w[i];
    }
    __syncthreads();  // s_w is reused by the next scan
    *tot = all;
    return base + x - v;
}

// Schedule the iteration whose lists go to buffer b.  pre: at the start of a
// launch (every earlier kernel is complete).
__device__ void res_schedule(const ResDev& d, int b, bool pre) {
    __shared__ int s_active, s_njobs, s_joins;
    __shared__ long long s_last, s_cont;
    const int t = threadIdx.x;
    if (t == 0) {
        s_active = 0;
        s_njobs = 0;
        // one read of mapped memory per step unless the host announced joins
        const int gen = ld_acquire_sys(&d.mb->join_gen);
        s_joins = gen != (int)d.it[3];
        d.it[3] = gen;
        if (pre) {
            d.it[1] = 0;
            d.it[2] = 0;
        } else {
            d.it[1] += 1;  // the iteration that just ran
        }
        s_last = d.it[0];
    }
    __syncthreads();
    const long long last = s_last, g = last + 1;
    // pass 1: admissions, retirements, who steps next (slots t*R .. t*R+R-1)
    int combo[kSlotsPerThread], units[kSlotsPerThread];
    bool listed[kSlotsPerThread];
#pragma unroll
    for (int r = 0; r < kSlotsPerThread; ++r) {
        const int k = t * kSlotsPerThread + r;
        combo[r] = -1;
        units[r] = 0;
        listed[r] = false;
        if (k >= d.cap) continue;
        int st = d.state[k];
        if (st == 0 && s_joins && ld_vol(&d.mb->join[k]) == 1) {
            // the host wrote the entry (copy complete) before the join word
            st = 1;
            d.state[k] = 1;
            d.parity[k] = 0;
            d.taken[k] = 0;
            d.last_it[k] = -1;
            *reinterpret_cast<volatile int*>(&d.mb->join[k]) = 2;
        }
        if (st != 1) continue;
        const ResEntry* e = d.table + k;
        const int left = __ldcg(&e->left) - d.taken[k];
        if (left <= 0) {
            // spent: retire once its last step's reduction is complete (it
            // was not stepped in the iteration whose tail this is)
            if (pre || d.last_it[k] < last) {
                d.state[k] = 0;
                __threadfence();
                *reinterpret_cast<volatile long long*>(&d.mb->done[k]) = (long long)d.taken[k] + 1;
                __threadfence_system();
                continue;
            }
        } else {
            combo[r] = __ldcg(&e->combo);
            units[r] = __ldcg(&e->units);
            // a kind this graph has no kernel for waits (the host relaunches
            // the loop with it)
            listed[r] = (d.combo_mask >> combo[r]) & 1u;
        }
        atomicAdd(&s_active, 1);
    }
    __syncthreads();
    if (t == 0) {
        const bool stop = ld_vol(&d.mb->stop) != 0;
        const bool cont = s_active > 0 && !stop && (pre || d.it[1] < d.max_iters);
        s_cont = cont ? 1 : 0;
        if (cont) d.it[0] = g;
        else d.it[2] = 1;  // halted: the rest of this body does nothing
        cudaGraphSetConditional(d.cond, cont ? 1u : 0u);
    }
    __syncthreads();
    const bool cont = s_cont != 0;
    // pass 2: per-combo lists in slot order (empty when the loop ends)
    const int cap = d.cap;
    if (t < kResCombos) d.ctr[b * kResCombos + t] = 0;
    for (int c = 0; c < kResCombos; ++c) {
        if (!(d.combo_mask & (1u << c))) continue;  // no kernel reads its list
        long long v = 0;
#pragma unroll
        for (int r = 0; r < kSlotsPerThread; ++r)
            if (cont && listed[r] && combo[r] == c) v += (1LL << 32) | (long long)units[r];
        long long tot;
        long long ex = block_scan64(v, &tot);
        if (tot == 0) {
            if (t == 0) d.count[b * kResCombos + c] = 0;
            continue;
        }
        int* st = d.start + (size_t)(b * kResCombos + c) * (cap + 1);
        const KParams** pp = d.params + (size_t)(b * kResCombos + c) * cap;
#pragma unroll
        for (int r = 0; r < kSlotsPerThread; ++r) {
            if (!(cont && listed[r] && combo[r] == c)) continue;
            const int k = t * kSlotsPerThread + r;
            const int pos = (int)(ex >> 32);
            st[pos] = (int)(ex & 0xFFFFFFFFLL);
            pp[pos] = &d.table[k].p[d.parity[k]];
            ex += (1LL << 32) | (long long)units[r];
        }
        if (t == 0) {
            d.count[b * kResCombos + c] = (int)(tot >> 32);
            st[tot >> 32] = (int)(tot & 0xFFFFFFFFLL);
        }
    }
    // force reductions of the listed members, and their step bookkeeping
#pragma unroll
    for (int r = 0; r < kSlotsPerThread; ++r) {
        if (!(cont && listed[r])) continue;
        const int k = t * kSlotsPerThread + r;
        ResEntry* e = d.table + k;
        if (e->job.nslots > 0) {
            const int j = atomicAdd(&s_njobs, 1);
            ReduceJob job = e->job;
            job.left = nullptr;
            d.jobs[(size_t)b * cap + j] = job;
        }
        // a settled solid's state no longer changes: stop storing it
        if (e->settle_after >= 0 && d.taken[k] >= e->settle_after && !e->p[d.parity[k]].skip_settled_solids) {
            e->p[0].skip_settled_solids = 1;
            e->p[1].skip_settled_solids = 1;
        }
        d.taken[k] += 1;
        d.parity[k] ^= 1;
        d.last_it[k] = g;
    }
    __syncthreads();
    if (t == 0) d.njobs[b] = s_njobs;
}

__global__ void __launch_bounds__(kTailThreads) res_pre_kernel(ResDev d) { res_schedule(d, 0, true); }

// The tail after the step kernels of buffer b.
__global__ void __launch_bounds__(kTailThreads) res_tail_kernel(ResDev d, int b) {
    if (blockIdx.x == 0) {
        if (d.it[2] == 0) res_schedule(d, 1 - b, false);
        return;
    }
    // the same sums, in the same order, as batch_force_reduce_kernel
    const int nj = d.njobs[b];
    for (int q = (int)blockIdx.x - 1; q < nj; q += (int)gridDim.x - 1) {
        const ReduceJob j = d.jobs[(size_t)b * d.cap + q];
        double a = 0.0, c = 0.0;
        for (int k = threadIdx.x; k < j.nslots; k += blockDim.x) {
            a += j.partials[2 * k];
            c += j.partials[2 * k + 1];
        }
        block_reduce2(a, c);
        if (threadIdx.x == 0) {
            const unsigned long long n = *j.counter;
            if (n < (unsigned long long)j.cap) {
                j.hist[2 * n] = a;
                j.hist[2 * n + 1] = c;
            }
            j.last[0] = a;
            j.last[1] = c;
            *j.counter = n + 1;
        }
        __syncthreads();  // block_reduce2's shared words are reused by the next job
    }
}

// One combo's step: the fixed grid walks the units of the members listed in
// buffer b, one unit per block at a time.  KIND 0: paired (tile blocks, then
// the member's boundary blocks); 1: one node per thread; 2: one node per
// thread with the thermal DDF.
// Launch bounds: the register budgets of the batched kernels
// (batch_step_pair_kernel 64, batch_step_th_kernel for the 16-bit thermal
// forms 48; batch_step_kernel's one-node forms need at most 80 and keep 6
// blocks of 128 threads per SM), so the unit loop's own state does not cost
// occupancy.
template <class T, int KIND>
constexpr int kResMaxThreads = (KIND == 2 && sizeof(T) == 2) ? 256 : (KIND == 0 ? 128 : 128);
template <class T, int KIND>
constexpr int kResMinBlocks = KIND == 0 ? 6 : ((KIND == 2 && sizeof(T) == 2) ? 5 : (KIND == 1 ? 6 : 1));

template <class T, int KIND>
__global__ void __launch_bounds__(kResMaxThreads<T, KIND>, kResMinBlocks<T, KIND>)
    res_step_kernel(ResDev d, int b, int c) {
    __shared__ __align__(16) KParams sp[2];
    __shared__ int s_st[kResMaxSlots + 1];
    __shared__ int s_next, s_next_m, s_next_buf;  // the block's next unit, its member and buffer
    __shared__ int s_staged[2];                    // the member whose parameters sp[k] holds
    const int n = d.count[b * kResCombos + c];
    if (n == 0) return;
    const int* st = d.start + (size_t)(b * kResCombos + c) * (d.cap + 1);
    const int total = st[n];
    // block k starts with unit k; a block without one has nothing to do
    if ((int)blockIdx.x >= total) return;
    const int first = min((int)gridDim.x, total);  // units handed out by block index
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    const int warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i <= n; i += nt) s_st[i] = st[i];
    const KParams* const* pp = d.params + (size_t)(b * kResCombos + c) * d.cap;
    int* ctr = d.ctr + b * kResCombos + c;
    auto member_of = [&](int u) {  // last member whose first unit is <= u
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_st[mid] <= u) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    };
    constexpr int kChunks = (int)(sizeof(KParams) / 16);
    auto stage = [&](int m, int buf) {  // warp 0: 16-byte asynchronous copies
        for (int k = lane; k < kChunks; k += 32) {
            const uint32_t dst = (uint32_t)__cvta_generic_to_shared(reinterpret_cast<char*>(&sp[buf]) + 16 * k);
            const char* src = reinterpret_cast<const char*>(pp[m]) + 16 * k;
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    __syncthreads();  // s_st
    if (warp == 0) {
        const int m0 = member_of((int)blockIdx.x);
        stage(m0, 0);
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (lane == 0) {
            s_next = (int)blockIdx.x;
            s_next_m = m0;
            s_next_buf = 0;
            s_staged[0] = m0;
            s_staged[1] = -1;
        }
    }
    __syncthreads();
    // Units are taken one at a time from the combo's counter, as the block
    // scheduler hands out launch blocks: warp 0 takes the next one when the
    // current unit starts its last tile and stages that member's parameters
    // in the other buffer meanwhile, so a block never holds a unit another
    // block could have started.
    int cb = 0;
    auto take_next = [&]() {
        if (warp != 0) return;
        int un = 0;
        if (lane == 0) un = first + atomicAdd(ctr, 1);
        un = __shfl_sync(0xffffffffu, un, 0);
        int mn = -1, nb = cb;
        if (un < total) {
            mn = member_of(un);
            if (mn != s_staged[cb]) {
                nb = cb ^ 1;
                if (mn != s_staged[nb]) stage(mn, nb);
            }
        }
        __syncwarp();
        if (lane == 0) {
            s_next = un;
            s_next_m = mn;
            s_next_buf = nb;
            if (mn >= 0) s_staged[nb] = mn;
        }
    };
    for (;;) {
        const int u = s_next;
        if (u >= total) break;
        const int m = s_next_m;
        cb = s_next_buf;
        __syncthreads();  // every thread has read the shared words take_next rewrites
        const KParams& p = sp[cb];
        const int local = u - s_st[m];
        if constexpr (KIND == 0) {
            if constexpr (!std::is_same<T, double>::value) {
                // flat tiles, then the member's boundary blocks (its
                // boundary pairs: none when it has no boundary node)
                const int tiles = p.ftiles;
                const int reg = (tiles + kBatchTiles - 1) / kBatchTiles;
                if (local >= reg) {
                    take_next();
                    pair_boundary_block<T>(p, local - reg, tiles);
                } else {
                    const int t1 = min(tiles, (local + 1) * kBatchTiles);
                    for (int t = local * kBatchTiles; t < t1; ++t) {
                        if (t == t1 - 1) take_next();
                        step_flat_pair_block<T>(p, t);
                    }
                }
            } else {
                take_next();  // never launched: FP64 is not paired
            }
        } else {
            const int tiles = p.gx * ((p.ny + (int)blockDim.y - 1) / (int)blockDim.y);
            const int t1 = min(tiles, (local + 1) * kBatchTiles);
            for (int t = local * kBatchTiles; t < t1; ++t) {
                if (t == t1 - 1) take_next();
                step_block<T, KIND == 2>(p, t % p.gx, t / p.gx, p.gx);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();  // the next unit's id and parameters are in place
    }
}

using StepFn = void (*)(ResDev, int, int);

// The step kernel of a combo (null: no such kernel -- FP64 is never paired).
StepFn step_fn(int combo) {
    const int st = combo / 3, kind = combo % 3;
#define LBM2D_RES_FN(T)                                  \
    return kind == 0 ? (std::is_same<T, double>::value ? nullptr : (StepFn)res_step_kernel<T, 0>) \
                     : (kind == 1 ? (StepFn)res_step_kernel<T, 1> : (StepFn)res_step_kernel<T, 2>)
    switch (st) {
        case ST_FP32: LBM2D_RES_FN(float);
        case ST_FP16: LBM2D_RES_FN(__half);
        case ST_BF16: LBM2D_RES_FN(__nv_bfloat16);
        case ST_FP64: LBM2D_RES_FN(double);
    }
#undef LBM2D_RES_FN
    return nullptr;
}

}  // namespace

struct ResLoop {
    int device = 0, cap = 0, bx = 32, by = 4, sms = 0;
    ResDev d{};
    ResMailbox* mb_host = nullptr;
    void* dev_block = nullptr;  // every device array of d, one allocation
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned built_mask = 0;
    int built_iters = -1;
};

namespace {

int build_graph(ResLoop* r, unsigned mask, int max_iters) {
    if (r->exec) cudaGraphExecDestroy(r->exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    r->exec = nullptr;
    r->graph = nullptr;
    cudaError_t e = cudaGraphCreate(&r->graph, 0);
    if (e != cudaSuccess) return (int)e;
    // each launch starts with the condition at 0; the pre-launch schedule
    // sets it
    e = cudaGraphConditionalHandleCreate(&r->d.cond, r->graph, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return (int)e;
    r->d.max_iters = max_iters;
    r->d.combo_mask = mask;
    ResDev d = r->d;
    int zero = 0, one = 1;
    void* pre_args[] = {&d};
    cudaKernelNodeParams kp{};
    kp.func = (void*)res_pre_kernel;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(kTailThreads);
    kp.kernelParams = pre_args;
    cudaGraphNode_t pre;
    if ((e = cudaGraphAddKernelNode(&pre, r->graph, nullptr, 0, &kp)) != cudaSuccess) return (int)e;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = r->d.cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t loop;
    if ((e = cudaGraphAddNode(&loop, r->graph, &pre, nullptr, 1, &cp)) != cudaSuccess) return (int)e;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    // tail grid: block 0 schedules, the others reduce (at most one job each
    // per pass)
    const int tail_blocks = 1 + std::min(r->cap, 2 * r->sms);
    std::vector<cudaGraphNode_t> prev;
    int combos[kResCombos];
    for (int b = 0; b < 2; ++b) {
        std::vector<cudaGraphNode_t> steps;
        for (int c = 0; c < kResCombos; ++c) {
            if (!(mask & (1u << c))) continue;
            StepFn fn = step_fn(c);
            if (!fn) continue;
            int per = 0;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, r->bx * r->by, 0)) != cudaSuccess)
                return (int)e;
            combos[c] = c;
            void* args[] = {&d, b == 0 ? &zero : &one, &combos[c]};
            cudaKernelNodeParams sk{};
            sk.func = (void*)fn;
            sk.gridDim = dim3((unsigned)std::max(1, per * r->sms));
            sk.blockDim = dim3(r->bx, r->by);
            sk.kernelParams = args;
            cudaGraphNode_t n;
            if ((e = cudaGraphAddKernelNode(&n, body, prev.data(), prev.size(), &sk)) != cudaSuccess) return (int)e;
            steps.push_back(n);
        }
        void* targs[] = {&d, b == 0 ? &zero : &one};
        cudaKernelNodeParams tk{};
        tk.func = (void*)res_tail_kernel;
        tk.gridDim = dim3((unsigned)tail_blocks);
        tk.blockDim = dim3(kTailThreads);
        tk.kernelParams = targs;
        const std::vector<cudaGraphNode_t>& deps = steps.empty() ? prev : steps;
        cudaGraphNode_t tn;
        if ((e = cudaGraphAddKernelNode(&tn, body, deps.data(), deps.size(), &tk)) != cudaSuccess) return (int)e;
        prev.assign(1, tn);
    }
    if ((e = cudaGraphInstantiate(&r->exec, r->graph, 0)) != cudaSuccess) return (int)e;
    r->built_mask = mask;
    r->built_iters = max_iters;
    return 0;
}

}  // namespace

int res_create(int device, int cap, int bx, int by, ResLoop** out) {
    if (cap < 1 || cap > kResMaxSlots || bx * by > 512 || (bx * by) % 32) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    auto* r = new ResLoop();
    r->device = device;
    r->cap = cap;
    r->bx = bx;
    r->by = by;
    cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, device);
    if (r->sms <= 0) r->sms = 1;
    if ((e = cudaHostAlloc(&r->mb_host, sizeof(ResMailbox), cudaHostAllocMapped | cudaHostAllocPortable)) !=
        cudaSuccess) {
        delete r;
        return (int)e;
    }
    std::memset(r->mb_host, 0, sizeof(ResMailbox));
    void* mb_dev = nullptr;
    if ((e = cudaHostGetDevicePointer(&mb_dev, r->mb_host, 0)) != cudaSuccess) {
        cudaFreeHost(r->mb_host);
        delete r;
        return (int)e;
    }
    // one device block for every array, each at a 256-byte boundary
    const size_t C = (size_t)cap;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) / 256 * 256;
        return o;
    };
    const size_t o_table = take(C * sizeof(ResEntry)), o_state = take(C * 4), o_par = take(C * 4),
                 o_taken = take(C * 4), o_last = take(C * 8), o_count = take(2 * kResCombos * 4),
                 o_start = take(2 * kResCombos * (C + 1) * 4), o_params = take(2 * kResCombos * C * sizeof(void*)),
                 o_jobs = take(2 * C * sizeof(ReduceJob)), o_njobs = take(2 * 4), o_it = take(4 * 8),
                 o_ctr = take(2 * kResCombos * 4);
    if ((e = cudaMalloc(&r->dev_block, off)) != cudaSuccess || (e = cudaMemset(r->dev_block, 0, off)) != cudaSuccess) {
        if (r->dev_block) cudaFree(r->dev_block);
        cudaFreeHost(r->mb_host);
        delete r;
        return (int)e;
    }
    char* base = static_cast<char*>(r->dev_block);
    ResDev& d = r->d;
    d.table = reinterpret_cast<ResEntry*>(base + o_table);
    d.mb = static_cast<ResMailbox*>(mb_dev);
    d.state = reinterpret_cast<int*>(base + o_state);
    d.parity = reinterpret_cast<int*>(base + o_par);
    d.taken = reinterpret_cast<int*>(base + o_taken);
    d.last_it = reinterpret_cast<long long*>(base + o_last);
    d.count = reinterpret_cast<int*>(base + o_count);
    d.start = reinterpret_cast<int*>(base + o_start);
    d.params = reinterpret_cast<const KParams**>(base + o_params);
    d.jobs = reinterpret_cast<ReduceJob*>(base + o_jobs);
    d.njobs = reinterpret_cast<int*>(base + o_njobs);
    d.it = reinterpret_cast<long long*>(base + o_it);
    d.ctr = reinterpret_cast<int*>(base + o_ctr);
    d.cap = cap;
    *out = r;
    return 0;
}

void res_destroy(ResLoop* r) {
    if (!r) return;
    cudaSetDevice(r->device);
    if (r->exec) cudaGraphExecDestroy(r->exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    if (r->dev_block) cudaFree(r->dev_block);
    if (r->mb_host) cudaFreeHost(r->mb_host);
    delete r;
}

ResEntry* res_table(ResLoop* r) { return r->d.table; }
volatile ResMailbox* res_mailbox(ResLoop* r) { return r->mb_host; }

int res_launch(ResLoop* r, unsigned combo_mask, int max_iters, void* stream) {
    if (max_iters < 1) return (int)cudaErrorInvalidValue;
    if (!r->exec || combo_mask != r->built_mask || max_iters != r->built_iters) {
        const int e = build_graph(r, combo_mask, max_iters);
        if (e) return e;
    }
    return (int)cudaGraphLaunch(r->exec, static_cast<cudaStream_t>(stream));
}

}  // namespace lbm2d
