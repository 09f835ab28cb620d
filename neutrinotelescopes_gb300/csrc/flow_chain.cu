// flow_chain.cu -- a chain of up to four dense layers in one kernel, for the
// conditioner MLP of the arrival-time flow (the forward pass
// X -> H1 -> H2 -> H3 -> P, and the backward chain of activation gradients
// dP -> dZ3 -> dZ2 -> dZ1).
//
// Stage s computes D_s = A_s W_s^T (+ bias, ReLU or a ReLU mask) with A_0
// the input tile (TMA from global memory) and A_s, s > 0, the previous
// stage's output, which never goes through global memory: its epilogue
// writes it as BF16 into shared memory in the 128-byte-swizzled K-major
// layout that the tensor cores read as the next A operand.  Only the outputs
// the caller asks for go to global memory (row-major BF16 by TMA store from
// that same on-chip tile, row-major FP32, the BF16 transpose, column sums).
// Design for sm_103a:
//   * a cluster of two CTAs per 128-row tile; CTA q of the pair computes
//     output columns [q n/2, (q+1) n/2) of every stage (its half of W_s
//     streamed by TMA) and writes its half of the stage's activations into
//     its own shared memory, and bulk copies (cp.async.bulk across the
//     cluster, one per 64-column slice as soon as it is written) push that
//     half into the partner's, completing on the partner's mbarrier, which
//     releases its next stage.  Two activation
//     buffers alternate between the stages, so a stage's writes never meet
//     the partner's reads of the previous stage;
//   * 256 threads (8 warps) per CTA; thread 0 issues the TMA loads and the
//     tcgen05.mma (cta_group::1, kind::f16, M = 128, N = n/2 <= 128, FP32
//     accumulator of 128 lanes x n/2 columns in TMEM); the weights stream
//     through a ring of three 64-wide K slices, refilled as slices are
//     consumed and, once a stage's MMAs are done, with the next stage's
//     slices while the epilogue runs;
//   * epilogue: warp w reads TMEM lanes 32 (w mod 4) (one row per lane),
//     32 columns per tcgen05.ld, column chunks alternating between w < 4 and
//     w >= 4, in two passes of 64 columns; ReLU masks are loaded before the
//     accumulator is complete; each pass's transposed output (two buffers)
//     and a last stage's FP32 output (128-byte-swizzled 32-column tiles in
//     the free activation buffer) are assembled in shared memory and written
//     by TMA stores;
//   * every wait on an mbarrier gives up after a bounded time and sets the
//     error word; a CTA whose wait gave up skips its remaining work but still
//     arrives on every barrier the partner waits for, and both CTAs meet at
//     one cluster barrier before either exits, so no CTA touches the shared
//     memory of a CTA that has finished.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "ntp_internal.h"
#include "tc_ptx.cuh"

namespace ntp {

namespace {

using namespace tc;

constexpr int kRows = 128;     // rows of a tile (UMMA M)
constexpr int kThreads = 256;  // 8 warps
constexpr int kRing = 3;       // weight slices in flight
constexpr int kMaxN = 256;     // columns of a stage (both CTAs)
constexpr int kMaxHalf = kMaxN / 2;
constexpr int kActSlices = kMaxN / kBK;
constexpr uint32_t kTmemCols = kMaxHalf;

struct ChainSmem {
    // activations of the tile: two buffers of four 64-column slices (the A
    // operand of the current stage and the output of the current stage)
    alignas(1024) __nv_bfloat16 act[2][kActSlices][kRows * kBK];  // 128 KB
    alignas(1024) __nv_bfloat16 w[kRing][kMaxHalf * kBK];         // weight slices, 48 KB
    alignas(1024) __nv_bfloat16 tr[2][kBK * kRows];               // transposed pass outputs, [column][row], 32 KB
    float bias[kMaxChainStages][kMaxHalf];
    uint64_t full[kRing];
    uint64_t empty[kRing];
    uint64_t a_full;
    uint64_t done;
    // per activation buffer: this CTA's half written and the partner's half
    // copied in (one barrier per buffer, so that the copies of consecutive
    // stages complete on different barriers)
    uint64_t act_ready[2];
    uint32_t tmem;
    int abort;
};

// byte offset of the 16-byte chunk c of row r in a 128-row x 64-column BF16
// slice with the 128-byte swizzle (8-row groups of 1024 bytes, chunk index
// XOR row mod 8), the layout TMA reads and writes with
// CU_TENSOR_MAP_SWIZZLE_128B
__device__ __forceinline__ uint32_t sw128_offset(int r, int c) {
    return static_cast<uint32_t>(r * 128 + ((c ^ (r & 7)) << 4));
}

// ReLU mask from the BF16 bit pattern: (bits - 1) < 0x7F80 holds for the
// positive values, from the smallest subnormal up to +inf
__device__ __forceinline__ bool bf16_positive(uint32_t bits16) { return bits16 - 1u < 0x7F80u; }

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// the address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t peer_addr(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

// bytes from this CTA's shared memory to the same-sized region of another
// CTA of the cluster (addresses from mapa), completing on that CTA's mbarrier
__device__ __forceinline__ void bulk_copy_to_peer(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst),
                 "r"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Bounded wait with cluster-scope acquire (the barrier is arrived on from the
// partner CTA); false after limit_ns.
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, unsigned long long limit_ns) {
    const uint32_t a = smem_u32(bar);
    const unsigned long long t0 = global_ns();
    for (unsigned i = 0;; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
            "selp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > limit_ns) return false;
    }
}

// 2-D TMA load delivered to the same shared-memory offset (data and
// mbarrier) of every CTA of the pair
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
        " [%0], [%1, {%3, %4}], [%2], %5;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "h"(static_cast<uint16_t>(3))
        : "memory");
}

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(smem_u32(src)), "r"(x), "r"(y)
                 : "memory");
}

struct ChainMaps {
    CUtensorMap a;                   // input tile, 128 rows x 64 columns per box
    CUtensorMap w[kMaxChainStages];  // a stage's weights, n/2 rows x 64 columns per box
    CUtensorMap c[kMaxChainStages];  // a stage's row-major BF16 output, 128 rows x 64 columns per box
    CUtensorMap ct[kMaxChainStages]; // a stage's transposed output, 64 columns x 128 rows per box
    CUtensorMap c32[kMaxChainStages];  // a stage's row-major FP32 output, 128 rows x 32 columns per box
};

__global__ void __launch_bounds__(kThreads, 1)
    chain_kernel(const __grid_constant__ ChainMaps maps, const ChainSpec spec, int* __restrict__ error,
                 unsigned long long wait_ns, int withhold_first) {
    extern __shared__ unsigned char smem_raw[];
    ChainSmem* s = reinterpret_cast<ChainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quad = warp & 3, half = warp >> 2;
    const uint32_t q = cluster_rank();  // this CTA's half of the columns
    const uint32_t partner = q ^ 1u;
    const int m0 = (blockIdx.x >> 1) * kRows;  // the pair's tile
    const int S = spec.n_stages;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s->tmem)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < kRing; ++i) {
            mbar_init(&s->full[i], 1);
            mbar_init(&s->empty[i], 1);
        }
        mbar_init(&s->a_full, 1);
        mbar_init(&s->done, 1);
        mbar_init(&s->act_ready[0], 1);  // this CTA's arrival, with the partner's bytes as transactions
        mbar_init(&s->act_ready[1], 1);
        s->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // the partner's barriers are initialised before anything arrives on them
    cluster_sync_all();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s->tmem;

    // the K slices of all stages in one sequence g = 0 .. total-1
    int first[kMaxChainStages + 1];
    int total = 0;
    for (int st = 0; st < S; ++st) {
        first[st] = total;
        total += spec.st[st].k / kBK;
    }
    first[S] = total;
    auto stage_of = [&](int g) {
        int st = 0;
        while (st + 1 < S && g >= first[st + 1]) ++st;
        return st;
    };
    int issued[kRing] = {}, landed[kRing] = {};  // loads per ring slot (thread 0)
    int next_load = 0;                            // next slice to load (thread 0)
    bool a_pending = false;
    auto load_slice = [&](int g) {
        const int r = g % kRing, st = stage_of(g);
        const int nq = spec.st[st].n / 2;
        mbar_expect_tx(&s->full[r], static_cast<uint32_t>(nq) * kBK * sizeof(__nv_bfloat16));
        tma_load_2d(s->w[r], &maps.w[st], &s->full[r], (g - first[st]) * kBK, static_cast<int>(q) * nq);
        ++issued[r];
        next_load = g + 1;
    };
    // the first weight slices, before the wait for the previous kernel when
    // the caller says they were written before it started
    if (threadIdx.x == 0 && spec.weights_ready)
        for (int g = 0; g < kRing && g < total; ++g) load_slice(g);
    // programmatic dependent launch: inputs (and otherwise the weights) and
    // biases are read only after the previous kernel of the stream has
    // completed
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (threadIdx.x == 0) {
        const int ka = spec.st[0].k / kBK;
        // the pair's input tile: each CTA loads every other 64-column slice
        // into both CTAs (multicast); each CTA's barrier expects all of it.
        // Failure-detection test: this CTA's slices are not loaded, so its
        // barrier (and the partner's) never completes and the first wait
        // runs out
        mbar_expect_tx(&s->a_full, static_cast<uint32_t>(ka) * kRows * kBK * sizeof(__nv_bfloat16));
        a_pending = true;
        if (!withhold_first)
            for (int j = static_cast<int>(q); j < ka; j += 2) tma_load_2d_pair(s->act[0][j], &maps.a, &s->a_full, j * kBK, m0);
        if (!spec.weights_ready)
            for (int g = 0; g < kRing && g < total; ++g) load_slice(g);
    }
    for (int st = 0; st < S; ++st) {
        const int nq = spec.st[st].n / 2;
        for (int i = threadIdx.x; i < nq; i += kThreads)
            s->bias[st][i] = spec.st[st].bias ? spec.st[st].bias[static_cast<int>(q) * nq + i] : 0.0f;
    }
    __syncthreads();

    bool ok = true;  // thread 0: every wait so far completed
    for (int st = 0; st < S; ++st) {
        const ChainStage& cs = spec.st[st];
        const int nq = cs.n / 2;
        const int cb = st & 1, nb = cb ^ 1;  // A operand / output buffers
        if (threadIdx.x == 0) {
            if (st == 0) {
                ok = mbar_wait(&s->a_full, 0, wait_ns);
                if (ok) a_pending = false;
            } else {
                // every phase is waited for in order, also after a failed
                // wait, so that no copy into this CTA is in flight at its end
                // buffer cb was filled by the transition out of stage st - 1,
                // the ((st - 1) / 2)-th on this buffer's barrier
                ok = mbar_wait_cluster(&s->act_ready[cb], ((st - 1) >> 1) & 1, wait_ns) && ok;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            const uint32_t idesc = instr_desc_bf16(kRows, nq);
            for (int g = first[st]; ok && g < first[st + 1]; ++g) {
                const int r = g % kRing;
                ok = mbar_wait(&s->full[r], (g / kRing) & 1, wait_ns);
                if (!ok) break;
                ++landed[r];
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int j = g - first[st];
#pragma unroll
                for (int kk = 0; kk < kBK / kUK; ++kk) {
                    const uint64_t ad = smem_desc_sw128(s->act[cb][j]) + static_cast<uint64_t>((kk * kUK * 2) >> 4);
                    const uint64_t bd = smem_desc_sw128(s->w[r]) + static_cast<uint64_t>((kk * kUK * 2) >> 4);
                    umma_bf16(tmem, ad, bd, idesc, (j > 0 || kk > 0) ? 1u : 0u);
                }
                umma_commit(&s->empty[r]);
                // refill the slot of the previous slice once its MMAs have read it
                const int prev = g - 1;
                if (prev >= 0 && prev + kRing < total && prev + kRing >= next_load) {
                    const int pr = prev % kRing;
                    ok = mbar_wait(&s->empty[pr], (prev / kRing) & 1, wait_ns);
                    if (!ok) break;
                    load_slice(prev + kRing);
                }
            }
            // the TMA stores of the previous stage have read the transposed
            // tile and the activations before this stage's epilogue (which
            // starts once done flips) writes them again
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            // done flips once the MMAs issued so far have completed (also
            // after a failed wait, so that the other threads' wait ends)
            umma_commit(&s->done);
            if (!ok) s->abort = 1;
        }
        __syncwarp();
        if (st == S - 1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

        // this thread's row and column chunks: row quad * 32 + lane, chunks
        // c0 = 32 half, 32 half + 64 of the CTA's nq columns
        const int r = quad * 32 + lane;
        const int row = m0 + r;
        const bool row_in = row < spec.m;
        // the ReLU masks of the thread's chunks, loaded while the MMAs run
        uint4 mk[2][4];
        if (cs.mask && row_in) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int c0 = 32 * half + 64 * i;
                if (c0 < nq) {
                    const uint4* mrow = reinterpret_cast<const uint4*>(
                        cs.mask + static_cast<size_t>(row) * cs.ldm + static_cast<int>(q) * nq + c0);
#pragma unroll
                    for (int e = 0; e < 4; ++e) mk[i][e] = __ldg(mrow + e);
                }
            }
        }
        // warp-uniform: tcgen05.ld below is .sync.aligned, and lanes whose
        // bounded waits end on either side of the limit must not split a warp
        const bool have = __all_sync(0xffffffffu, mbar_wait(&s->done, st & 1, wait_ns));
        if (!have) {
            if (lane == 0) atomicExch(error, 2);
            s->abort = 1;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // every slice of this stage has been consumed: load the next ones
        // into the freed slots while the epilogue runs
        if (threadIdx.x == 0 && have && ok)
            while (next_load < total && next_load < first[st + 1] + kRing) load_slice(next_load);
        const bool to_peer = st + 1 < S;                 // the next stage reads this output
        const bool to_act = to_peer || cs.c != nullptr;  // and the TMA store of c reads it
        // two passes of 64 columns (pass i: column chunks 32 half + 64 i);
        // after each, thread 0 sends the pass's activation slice to the
        // partner and stores the pass's row-major and transposed tiles
        const int ql = static_cast<int>(q) * nq;  // first column of this CTA's half
        // both passes' accumulator columns loaded at once, one wait
        uint32_t acc[2][32];
        if (have) {
            const uint32_t lanes = static_cast<uint32_t>(quad * 32) << 16;
            tmem_ld32_async(tmem + lanes + static_cast<uint32_t>(32 * half), acc[0]);
            if (32 * half + 64 < nq) tmem_ld32_async(tmem + lanes + static_cast<uint32_t>(32 * half + 64), acc[1]);
            tmem_wait_ld(acc[0]);
            tmem_regs_ready(acc[1]);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int c0 = 32 * half + 64 * i;  // column within this CTA's half
            if (i == 1 && 64 >= nq) break;  // CTA-uniform: a single pass
            if (have && c0 < nq) {
                const int col = ql + c0;
                float v[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(acc[i][j]);
                if (cs.bias) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] += s->bias[st][c0 + j];
                }
                if (cs.relu) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j], 0.0f);
                }
                if (cs.mask && row_in) {
#pragma unroll
                    for (int e4 = 0; e4 < 4; ++e4) {
                        const uint32_t wd[4] = {mk[i][e4].x, mk[i][e4].y, mk[i][e4].z, mk[i][e4].w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            if (!bf16_positive(wd[e] & 0xFFFFu)) v[e4 * 8 + 2 * e] = 0.0f;
                            if (!bf16_positive(wd[e] >> 16)) v[e4 * 8 + 2 * e + 1] = 0.0f;
                        }
                    }
                }
                if (!row_in) {  // rows beyond the matrix take no part in stores and column sums
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] = 0.0f;
                }
                uint32_t pk[16];  // the 32 values as BF16 pairs
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
                    pk[e] = *reinterpret_cast<const uint32_t*>(&h2);
                }
                if (to_act) {
                    unsigned char* base = reinterpret_cast<unsigned char*>(s->act[nb][col / kBK]);
                    const int cq = (col % kBK) / 8;
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        *reinterpret_cast<uint4*>(base + sw128_offset(r, cq + e)) =
                            make_uint4(pk[4 * e], pk[4 * e + 1], pk[4 * e + 2], pk[4 * e + 3]);
                }
                if (cs.c32) {  // 32-column FP32 tile c0 / 32 in the free activation buffer
                    unsigned char* tile = reinterpret_cast<unsigned char*>(s->act[nb][0]) + (c0 / 32) * (kRows * 128);
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        *reinterpret_cast<float4*>(tile + sw128_offset(r, e)) =
                            make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
                }
                if (cs.ct) {  // lanes hold consecutive rows: 64 contiguous bytes per column
                    unsigned short* tr = reinterpret_cast<unsigned short*>(s->tr[i]) + (c0 & (kBK - 1)) * kRows + r;
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        tr[(2 * e) * kRows] = static_cast<unsigned short>(pk[e] & 0xFFFFu);
                        tr[(2 * e + 1) * kRows] = static_cast<unsigned short>(pk[e] >> 16);
                    }
                }
                if (cs.colsum) {
                    // transpose-reduce: after the five halving steps lane l
                    // holds the warp's sum of column col + l
#pragma unroll
                    for (int o = 16; o >= 1; o >>= 1) {
                        const bool upper = (lane & o) != 0;
#pragma unroll
                        for (int k = 0; k < o; ++k) {
                            const float send = upper ? v[k] : v[k + o];
                            const float keep = upper ? v[k + o] : v[k];
                            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                        }
                    }
                    atomicAdd(cs.colsum + col + lane, v[0]);
                }
            }
            // the pass's activations and transposed tile (generic-proxy
            // stores) become visible to the bulk copy and the TMA stores, and
            // (last pass) the accumulator reads complete before the next
            // stage's MMAs
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (threadIdx.x == 0) {
                const int sl = (ql + 64 * i) / kBK;  // the pass's activation slice
                if (to_peer) {
                    // first the partner's copy (it gates the partner's next
                    // stage), also after a failed wait: the partner's wait
                    // must not be the one that runs out
                    const uint32_t src = smem_u32(s->act[nb][sl]);
                    bulk_copy_to_peer(peer_addr(src, partner), src, kRows * kBK * sizeof(__nv_bfloat16),
                                      peer_addr(smem_u32(&s->act_ready[nb]), partner));
                }
                const bool st_ok = have && !s->abort;  // abort: a wait of some warp gave up
                if (cs.c && st_ok) tma_store_2d(&maps.c[st], s->act[nb][sl], sl * kBK, m0);
                if (cs.ct && st_ok) tma_store_2d(&maps.ct[st], s->tr[i], m0, ql + 64 * i);
                if (cs.c32 && st_ok)
                    for (int j = 2 * i; j < 2 * i + 2 && 32 * j < nq; ++j)
                        tma_store_2d(&maps.c32[st], reinterpret_cast<unsigned char*>(s->act[nb][0]) + j * (kRows * 128),
                                     ql + 32 * j, m0);
                if ((cs.c || cs.ct || cs.c32) && st_ok) asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
        }
        if (threadIdx.x == 0 && to_peer) {
            // this CTA's arrival, expecting the partner's half of the stage
            const uint32_t bytes = static_cast<uint32_t>(nq) * kRows * sizeof(__nv_bfloat16);
            asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                             smem_u32(&s->act_ready[nb])),
                         "r"(bytes)
                         : "memory");
        }
    }
    if (threadIdx.x == 0) {
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        if (!ok || s->abort) {
            atomicExch(error, 1);
            // let copies still in flight land before the CTA's shared memory goes away
            if (a_pending) (void)mbar_wait(&s->a_full, 0, wait_ns);
            for (int r = 0; r < kRing; ++r)
                while (landed[r] < issued[r] && mbar_wait(&s->full[r], landed[r] & 1, wait_ns)) ++landed[r];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    // neither CTA of the pair leaves while the other may still write into its
    // shared memory or arrive on its barrier
    cluster_sync_all();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

constexpr size_t kSmemBytes = sizeof(ChainSmem) + 1024;

cudaError_t configure() {
    static std::atomic<unsigned long long> configured{0};  // one bit per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        e = cudaFuncSetAttribute(chain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kSmemBytes));
        if (e != cudaSuccess) return e;
        configured.fetch_or(bit);
    }
    return cudaSuccess;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

cudaError_t layer_chain_prepare() { return configure(); }

// Runs the chain described by spec on the rows of A [m x k_0] (BF16, leading
// dimension lda); w[s] is stage s's weight matrix [n_s x k_s] (BF16,
// row-major, K contiguous).  Shapes: k_0 and every n_s a multiple of 64 in
// [64, 256] (a multiple of 128 for a stage with the row-major BF16 output
// c or ct or whose output the next stage reads), k_s = n_{s-1}; A, the weights and
// every output 16-byte aligned with row strides that keep the rows so.
cudaError_t layer_chain(const void* a, int lda, const void* const* w, const ChainSpec& spec, int* error,
                        cudaStream_t stream) {
    const int S = spec.n_stages;
    if (S < 1 || S > kMaxChainStages || spec.m <= 0 || !a || !aligned16(a) || lda % 8) return cudaErrorInvalidValue;
    for (int st = 0; st < S; ++st) {
        const ChainStage& c = spec.st[st];
        if (c.n < 64 || c.n > kMaxN || c.n % 64 || c.k < 64 || c.k > kMaxN || c.k % kBK) return cudaErrorInvalidValue;
        if (st > 0 && c.k != spec.st[st - 1].n) return cudaErrorInvalidValue;
        if (st == 0 && c.k > lda) return cudaErrorInvalidValue;
        if (!w[st] || !aligned16(w[st])) return cudaErrorInvalidValue;
        // a stage whose output the next stage reads, or with the row-major
        // output, splits into two halves of whole 64-column slices
        if ((st + 1 < S || c.c || c.ct) && c.n % 128) return cudaErrorInvalidValue;
        // the FP32 output is staged in the activation buffer the stage would write
        if (c.c32 && (st + 1 < S || c.c)) return cudaErrorInvalidValue;
        if ((c.c && (!aligned16(c.c) || c.ldc % 8 || c.ldc < c.n)) ||
            (c.c32 && (!aligned16(c.c32) || c.ldc32 % 4 || c.ldc32 < c.n)) ||
            (c.mask && (!aligned16(c.mask) || c.ldm % 8 || c.ldm < c.n)) ||
            (c.ct && (!aligned16(c.ct) || c.ldct % 8 || c.ldct < spec.m)))
            return cudaErrorInvalidValue;
    }
    cudaError_t e = configure();
    if (e != cudaSuccess) return e;
    ChainMaps maps;
    if (!tensor_map_bf16(&maps.a, a, spec.m, spec.st[0].k, lda, kRows)) return cudaErrorInvalidValue;
    for (int st = 0; st < kMaxChainStages; ++st) {
        const int src = st < S ? st : 0;
        const ChainStage& c = spec.st[src];
        if (!tensor_map_bf16(&maps.w[st], w[src], c.n, c.k, c.k, c.n / 2)) return cudaErrorInvalidValue;
        // the row-major output map (a copy of the input map where unused)
        if (st < S && c.c) {
            if (!tensor_map_bf16(&maps.c[st], c.c, spec.m, c.n, c.ldc, kRows)) return cudaErrorInvalidValue;
        } else {
            maps.c[st] = maps.a;
        }
        if (st < S && c.ct) {
            if (!tensor_map_bf16_plain(&maps.ct[st], c.ct, c.n, spec.m, c.ldct, kRows, kBK))
                return cudaErrorInvalidValue;
        } else {
            maps.ct[st] = maps.a;
        }
        if (st < S && c.c32) {
            if (!tensor_map_f32_sw128(&maps.c32[st], c.c32, spec.m, c.n, c.ldc32, kRows)) return cudaErrorInvalidValue;
        } else {
            maps.c32[st] = maps.a;
        }
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(2 * ((spec.m + kRows - 1) / kRows));
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kSmemBytes;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = pdl_enabled();
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cudaLaunchKernelEx(&cfg, chain_kernel, maps, spec, error, wait_limit_ns(), withhold_first());
}

}  // namespace ntp
