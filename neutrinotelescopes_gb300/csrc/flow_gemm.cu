// flow_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05) for
// the conditioner MLP of the arrival-time flow.
//
// C[M x N] = A[M x K] * B[N x K]^T (+ bias[N], optional ReLU), A and B
// row-major with K contiguous (K-major), FP32 accumulation in tensor memory.
//   * one CTA per 128 x BN output tile (BN = 64, 128 or 256, the widest that
//     still gives every SM a CTA), 128 threads (4 warps); split-K over
//     blockIdx.z for the weight gradients, whose K is the batch;
//   * operands staged in shared memory by TMA (cp.async.bulk.tensor) in the
//     128-byte-swizzled layout, 3-4 pipeline stages of 64-wide K slices;
//   * one elected thread issues tcgen05.mma (cta_group::1, kind::f16, BF16
//     inputs, FP32 accumulator of 128 lanes x BN columns in TMEM) and
//     tcgen05.commit signals the stage free / the accumulator complete;
//   * the epilogue: each warp reads its 32 TMEM lanes (one row per lane) 32
//     columns at a time with tcgen05.ld, adds the bias, applies ReLU or a
//     ReLU mask read as 16-byte vectors, stores FP32 / BF16 or reduces FP32
//     (split-K) with 16-byte vector operations along the row, writes the
//     BF16 transpose (one contiguous run per column) and reduces column sums
//     across the warp by a five-step transpose-reduce (31 shuffles for 32
//     columns) with one atomic per column.
// Every wait on an mbarrier gives up after a bounded number of polls, sets
// the error word and skips to the TMEM release, so a fault in the pipeline
// returns a status instead of hanging the GPU.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "ntp_internal.h"
#include "tc_ptx.cuh"

namespace ntp {

namespace {

using namespace tc;

constexpr int kBM = 128;   // rows of a tile (UMMA M)
constexpr int kThreads = 128;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // by default a wait gives up after 2 s

// failure-detection controls (ntp_gemm_set_wait_limit), read at each launch
std::atomic<unsigned long long> g_wait_limit_ns{kWaitLimitNs};
std::atomic<int> g_withhold_first{0};
// programmatic dependent launch of the GEMMs (NTP_GEMM_PDL=0 in the
// environment turns it off)
std::atomic<int> g_pdl{[] {
    const char* e = std::getenv("NTP_GEMM_PDL");
    return (e && e[0] == '0') ? 0 : 1;
}()};

// pipeline depth: 4 stages (3 for the widest tile), within 227 KB of shared memory
template <int BN>
constexpr int stages_for() { return BN >= 256 ? 3 : 4; }

template <int BN>
struct Smem {
    static constexpr int kStages = stages_for<BN>();
    alignas(1024) __nv_bfloat16 a[kStages][kBM * kBK];
    alignas(1024) __nv_bfloat16 b[kStages][BN * kBK];
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t done;
    uint32_t tmem;
};

// One 128 x BN output tile over K slices [kt0, kt1) (the whole CTA).
// out_kind: 0 = FP32 store, 1 = BF16 store, 2 = FP32 atomic add (split-K);
// the bias is added by the first K split only (first_split).
template <int BN>
__device__ __forceinline__ void gemm_tile(const CUtensorMap& map_a, const CUtensorMap& map_b, int M, int N, int m0,
                                          int n0, int kt0, int kt1, bool first_split, const GemmEpilogue& ep,
                                          int vec_ok, int* __restrict__ error, unsigned long long wait_ns,
                                          int withhold_first) {
    extern __shared__ unsigned char smem_raw[];
    Smem<BN>* s = reinterpret_cast<Smem<BN>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr int kStages = Smem<BN>::kStages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr uint32_t kCols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s->tmem)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) {
            mbar_init(&s->full[i], 1);
            mbar_init(&s->empty[i], 1);
        }
        mbar_init(&s->done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s->tmem;
    bool ok = true;
    // Programmatic dependent launch: the set-up above (tensor memory,
    // barriers) may overlap the previous kernel of the stream; its outputs
    // are read only after this wait, which returns once that kernel has
    // completed and its writes are visible (a no-op without the launch
    // attribute).
    asm volatile("griddepcontrol.wait;" ::: "memory");

    if (threadIdx.x == 0 && kt1 > kt0) {
        constexpr uint32_t kStageBytes = (kBM + BN) * kBK * sizeof(__nv_bfloat16);
        const uint32_t idesc = instr_desc_bf16(kBM, BN);
        const int nk = kt1 - kt0;
        int issued[kStages] = {}, landed[kStages] = {};  // TMA pairs per stage
        for (int i = 0; i < kStages && i < nk; ++i) {
            // failure-detection test: the first stage's copies are not issued,
            // so its barrier is a flag that nothing completes and the first
            // wait runs out (nothing else is skipped; outputs are undefined)
            if (i == 0 && withhold_first) continue;
            mbar_expect_tx(&s->full[i], kStageBytes);
            tma_load_2d(s->a[i], &map_a, &s->full[i], (kt0 + i) * kBK, m0);
            tma_load_2d(s->b[i], &map_b, &s->full[i], (kt0 + i) * kBK, n0);
            ++issued[i];
        }
        for (int i = 0; i < nk && ok; ++i) {
            const int st = i % kStages;
            ok = mbar_wait(&s->full[st], (i / kStages) & 1, wait_ns);
            if (!ok) break;
            ++landed[st];
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < kBK / kUK; ++kk) {
                const uint64_t ad = smem_desc_sw128(s->a[st]) + static_cast<uint64_t>((kk * kUK * 2) >> 4);
                const uint64_t bd = smem_desc_sw128(s->b[st]) + static_cast<uint64_t>((kk * kUK * 2) >> 4);
                umma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            }
            umma_commit(&s->empty[st]);
            // refill the stage of the previous slice once its MMAs have read it
            const int prev = i - 1;
            if (prev >= 0 && prev + kStages < nk) {
                const int ps = prev % kStages;
                ok = mbar_wait(&s->empty[ps], (prev / kStages) & 1, wait_ns);
                if (!ok) break;
                mbar_expect_tx(&s->full[ps], kStageBytes);
                tma_load_2d(s->a[ps], &map_a, &s->full[ps], (kt0 + prev + kStages) * kBK, m0);
                tma_load_2d(s->b[ps], &map_b, &s->full[ps], (kt0 + prev + kStages) * kBK, n0);
                ++issued[ps];
            }
        }
        umma_commit(&s->done);
        if (!ok) {
            atomicExch(error, 1);
            // let copies still in flight land before the CTA's shared memory goes away
            for (int st = 0; st < kStages; ++st)
                while (landed[st] < issued[st] && mbar_wait(&s->full[st], landed[st] & 1, wait_ns)) ++landed[st];
        }
    }
    __syncwarp();
    // the next kernel of the stream may start its own set-up now; it reads
    // this kernel's outputs only after its griddepcontrol.wait, i.e. after
    // this grid has completed
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // the accumulator is complete when `done` flips (a thread that timed out
    // above still committed, so this wait ends once its MMAs drain)
    // warp-uniform: tcgen05.ld below is .sync.aligned, and lanes whose
    // bounded waits end on either side of the limit must not split a warp
    const bool have = __all_sync(0xffffffffu, (kt1 > kt0) && mbar_wait(&s->done, 0, wait_ns));
    if (kt1 > kt0 && !have && lane == 0) atomicExch(error, 2);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (have) {
        const int row = m0 + warp * 32 + lane;
        const bool row_in = row < M;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            const int colb = n0 + c0;
            if (colb >= N) break;  // the same for every thread of the CTA
            float v[32];
            tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0), v);
            const bool full = colb + 32 <= N;
            if (ep.bias && first_split) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (full || colb + j < N) v[j] += __ldg(ep.bias + colb + j);
            }
            if (ep.relu) {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j], 0.0f);
            }
            if (ep.mask && row_in) {
                const __nv_bfloat16* mrow = ep.mask + static_cast<size_t>(row) * ep.ldm + colb;
                if (full && vec_ok) {  // 64 contiguous bytes of the lane's row
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint4 m4 = __ldg(reinterpret_cast<const uint4*>(mrow) + q);
                        const uint32_t w[4] = {m4.x, m4.y, m4.z, m4.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            // (bits - 1) < 0x7F80: positive, from the smallest subnormal up to +inf
                            const uint32_t lo = w[e] & 0xFFFFu, hi = w[e] >> 16;
                            if (!(lo - 1u < 0x7F80u)) v[q * 8 + 2 * e] = 0.0f;
                            if (!(hi - 1u < 0x7F80u)) v[q * 8 + 2 * e + 1] = 0.0f;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (colb + j < N && !(__bfloat162float(mrow[j]) > 0.0f)) v[j] = 0.0f;
                }
            }
            // values outside the matrix take no part in stores and column sums
            if (!row_in) {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = 0.0f;
            } else if (!full) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (colb + j >= N) v[j] = 0.0f;
            }
            if (ep.c && row_in) {
                const size_t o = static_cast<size_t>(row) * ep.ldc + colb;
                if (full && vec_ok) {  // 16-byte vector stores / reductions along the lane's row
                    if (ep.out_kind == 0) {
                        float4* d = reinterpret_cast<float4*>(static_cast<float*>(ep.c) + o);
#pragma unroll
                        for (int q = 0; q < 8; ++q) d[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    } else if (ep.out_kind == 1) {
                        uint4* d = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(ep.c) + o);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            uint32_t w[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const __nv_bfloat162 h = __floats2bfloat162_rn(v[q * 8 + 2 * e], v[q * 8 + 2 * e + 1]);
                                w[e] = *reinterpret_cast<const uint32_t*>(&h);
                            }
                            d[q] = make_uint4(w[0], w[1], w[2], w[3]);
                        }
                    } else {
                        float4* d = reinterpret_cast<float4*>(static_cast<float*>(ep.c) + o);
#pragma unroll
                        for (int q = 0; q < 8; ++q)
                            atomicAdd(d + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        if (colb + j >= N) continue;
                        if (ep.out_kind == 0) static_cast<float*>(ep.c)[o + j] = v[j];
                        else if (ep.out_kind == 1) static_cast<__nv_bfloat16*>(ep.c)[o + j] = __float2bfloat16(v[j]);
                        else atomicAdd(static_cast<float*>(ep.c) + o + j, v[j]);
                    }
                }
            }
            if (ep.ct && row_in) {  // lanes hold consecutive rows: each store is one contiguous 64-byte run
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (full || colb + j < N) ep.ct[static_cast<size_t>(colb + j) * ep.ldct + row] = __float2bfloat16(v[j]);
            }
            if (ep.colsum) {
                // transpose-reduce: after the five halving steps lane l holds the warp's sum of column l
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
                if (colb + lane < N) atomicAdd(ep.colsum + colb + lane, v[0]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// C = A B^T: grid (tiles of M, tiles of N, K splits)
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_bf16_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int M,
                     int N, int k_tiles_per_split, int k_tiles_total, const GemmEpilogue ep, int vec_ok,
                     int* __restrict__ error, unsigned long long wait_ns, int withhold_first) {
    const int kt0 = blockIdx.z * k_tiles_per_split;
    gemm_tile<BN>(map_a, map_b, M, N, blockIdx.x * kBM, blockIdx.y * BN, kt0,
                  min(kt0 + k_tiles_per_split, k_tiles_total), blockIdx.z == 0, ep, vec_ok, error, wait_ns,
                  withhold_first);
}

// Several independent products in one launch: CTA b belongs to problem p
// with cta_begin[p] <= b < cta_begin[p + 1], which it splits into (K split,
// N tile, M tile) with the M tile fastest.
struct GroupMaps {
    CUtensorMap a[kMaxGemmGroup];
    CUtensorMap b[kMaxGemmGroup];
};
struct GroupDesc {
    int n;
    int cta_begin[kMaxGemmGroup + 1];
    int tiles_m[kMaxGemmGroup], tiles_n[kMaxGemmGroup];
    int per[kMaxGemmGroup], k_tiles[kMaxGemmGroup];
    int M[kMaxGemmGroup], N[kMaxGemmGroup];
    int vec_ok[kMaxGemmGroup];
    GemmEpilogue ep[kMaxGemmGroup];
};

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    gemm_group_kernel(const __grid_constant__ GroupMaps maps, const __grid_constant__ GroupDesc g,
                      int* __restrict__ error, unsigned long long wait_ns, int withhold_first) {
    const int cta = static_cast<int>(blockIdx.x);
    int p = 0;
    while (p + 1 < g.n && cta >= g.cta_begin[p + 1]) ++p;
    const int local = cta - g.cta_begin[p];
    const int tiles = g.tiles_m[p] * g.tiles_n[p];
    const int split = local / tiles, t = local % tiles;
    const int kt0 = split * g.per[p];
    gemm_tile<BN>(maps.a[p], maps.b[p], g.M[p], g.N[p], (t % g.tiles_m[p]) * kBM, (t / g.tiles_m[p]) * BN, kt0,
                  min(kt0 + g.per[p], g.k_tiles[p]), split == 0, g.ep[p], g.vec_ok[p], error, wait_ns,
                  withhold_first);
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    });
    return fn;
}

// Tensor map of a row-major bf16 matrix [rows x cols] (leading dimension ld
// elements) read in boxes of box_rows x 64 with 128-byte swizzle; rows and
// columns beyond the matrix read as zero.
bool make_map(CUtensorMap* map, const void* base, int rows, int cols, int ld, int box_rows) {
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Sets the dynamic shared-memory limit of the BN variant once per device.
template <int BN>
cudaError_t configure_bn() {
    static std::atomic<unsigned long long> configured{0};  // one bit per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        e = cudaFuncSetAttribute(gemm_bf16_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(Smem<BN>) + 1024));
        if (e != cudaSuccess) return e;
        configured.fetch_or(bit);
    }
    return cudaSuccess;
}

template <int BN>
cudaError_t launch_bn(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int splits, int k_tiles,
                      const GemmEpilogue& ep, int vec_ok, int* error, cudaStream_t st) {
    const size_t smem = sizeof(Smem<BN>) + 1024;
    cudaError_t e = configure_bn<BN>();
    if (e != cudaSuccess) return e;
    const int per = (k_tiles + splits - 1) / splits;
    dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN, (k_tiles + per - 1) / per);
    // launched with programmatic stream serialisation: the kernel's prologue
    // overlaps the tail of the previous kernel on the stream (see the
    // griddepcontrol instructions in the kernel)
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = g_pdl.load();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, gemm_bf16_kernel<BN>, ma, mb, M, N, per, k_tiles, ep, vec_ok, error,
                              g_wait_limit_ns.load(), g_withhold_first.load());
}

int sm_count() {
    static std::atomic<int> cached{0};
    int n = cached.load();
    if (n == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        cached.store(n);
    }
    return n;
}

}  // namespace

namespace tc {
bool tensor_map_bf16(CUtensorMap* map, const void* base, int rows, int cols, int ld, int box_rows) {
    return make_map(map, base, rows, cols, ld, box_rows);
}
bool tensor_map_bf16_plain(CUtensorMap* map, const void* base, int rows, int cols, int ld, int box_cols,
                           int box_rows) {
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_cols), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
bool tensor_map_f32_sw128(CUtensorMap* map, const void* base, int rows, int cols, int ld, int box_rows) {
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 4};
    const cuuint32_t box[2] = {32, static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
int device_sm_count() { return sm_count(); }
unsigned long long wait_limit_ns() { return g_wait_limit_ns.load(); }
int withhold_first() { return g_withhold_first.load(); }
int pdl_enabled() { return g_pdl.load(); }
}  // namespace tc

// C = A * B^T on the tensor cores with the epilogue ep; see the file comment.
// lda / ldb in elements; A's and B's rows must start on 16-byte boundaries
// (lda, ldb multiples of 8) and K a multiple of 64.  splits > 1 splits K
// across CTAs and allows only the atomic FP32 output (out_kind 2); splits = 0
// chooses the split for about two CTAs per SM.
cudaError_t gemm_bf16_ep(const void* A, int lda, const void* B, int ldb, int M, int N, int K, const GemmEpilogue& ep,
                         int splits, int* error, cudaStream_t st) {
    if (M <= 0 || N <= 0 || K <= 0 || K % kBK || lda % 8 || ldb % 8 || splits < 0 ||
        (splits != 1 && (ep.out_kind != 2 || ep.ct || ep.mask || ep.colsum || ep.relu)) ||
        (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15))
        return cudaErrorInvalidValue;
    const int k_tiles = K / kBK;
    const int tiles_m = (M + kBM - 1) / kBM;
    const int sms = sm_count();
    // widest tile that still gives every SM a CTA (the GEMMs here are small), at most what N needs
    auto ctas = [&](int bn, int sp) { return static_cast<long long>(tiles_m) * ((N + bn - 1) / bn) * sp; };
    const int sp1 = splits == 0 ? 1 : splits;
    int bn = 64;
    for (int cand : {256, 128}) {
        if (cand < 2 * N && ctas(cand, sp1) >= sms) {
            bn = cand;
            break;
        }
    }
    if (splits == 0) {  // split K to about two CTAs per SM, at least 4 K slices each
        const long long t = ctas(bn, 1);
        long long sp = (2ll * sms + t - 1) / t;
        sp = std::min<long long>(sp, std::max(1, k_tiles / 4));
        splits = static_cast<int>(std::max<long long>(1, sp));
    }
    splits = splits > k_tiles ? k_tiles : splits;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda, kBM) || !make_map(&mb, B, N, K, ldb, bn)) return cudaErrorInvalidValue;
    // 16-byte vector access along a row of C and of the mask
    const size_t esz = ep.out_kind == 1 ? 2 : 4;
    int vec_ok = 1;
    if (ep.c && ((reinterpret_cast<uintptr_t>(ep.c) & 15) || (static_cast<size_t>(ep.ldc) * esz) % 16)) vec_ok = 0;
    if (ep.mask && ((reinterpret_cast<uintptr_t>(ep.mask) & 15) || ep.ldm % 8)) vec_ok = 0;
    if (bn == 64) return launch_bn<64>(ma, mb, M, N, splits, k_tiles, ep, vec_ok, error, st);
    if (bn == 128) return launch_bn<128>(ma, mb, M, N, splits, k_tiles, ep, vec_ok, error, st);
    return launch_bn<256>(ma, mb, M, N, splits, k_tiles, ep, vec_ok, error, st);
}

cudaError_t configure_group() {
    static std::atomic<unsigned long long> configured{0};  // one bit per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(configured.load() & bit)) {
        e = cudaFuncSetAttribute(gemm_group_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sizeof(Smem<64>) + 1024));
        if (e != cudaSuccess) return e;
        configured.fetch_or(bit);
    }
    return cudaSuccess;
}

// Up to kMaxGemmGroup independent products C_p = A_p B_p^T in one launch
// (64-column tiles); each problem is split along K so that the launch has
// about two CTAs per SM, which needs the atomic FP32 output (out_kind 2)
// wherever a split happens.  Shapes and alignment as in gemm_bf16_ep.
cudaError_t gemm_bf16_group(const GemmProblem* pr, int n, int* error, cudaStream_t st) {
    if (n < 1 || n > kMaxGemmGroup) return cudaErrorInvalidValue;
    long long tiles_total = 0;
    for (int p = 0; p < n; ++p) {
        const GemmProblem& q = pr[p];
        if (q.M <= 0 || q.N <= 0 || q.K <= 0 || q.K % kBK || q.lda % 8 || q.ldb % 8 ||
            (reinterpret_cast<uintptr_t>(q.a) & 15) || (reinterpret_cast<uintptr_t>(q.b) & 15))
            return cudaErrorInvalidValue;
        tiles_total += static_cast<long long>((q.M + kBM - 1) / kBM) * ((q.N + 63) / 64);
    }
    cudaError_t e = configure_group();
    if (e != cudaSuccess) return e;
    GroupMaps maps;
    GroupDesc g{};
    g.n = n;
    const long long want = (2ll * sm_count() + tiles_total - 1) / tiles_total;
    int cta = 0;
    for (int p = 0; p < n; ++p) {
        const GemmProblem& q = pr[p];
        const int k_tiles = q.K / kBK;
        const bool atomic_out = q.ep.out_kind == 2 && !q.ep.ct && !q.ep.mask && !q.ep.colsum && !q.ep.relu;
        long long sp = atomic_out ? std::min<long long>(want, std::max(1, k_tiles / 4)) : 1;
        sp = std::max<long long>(1, sp);
        const int per = static_cast<int>((k_tiles + sp - 1) / sp);
        const int splits = (k_tiles + per - 1) / per;
        g.cta_begin[p] = cta;
        g.tiles_m[p] = (q.M + kBM - 1) / kBM;
        g.tiles_n[p] = (q.N + 63) / 64;
        g.per[p] = per;
        g.k_tiles[p] = k_tiles;
        g.M[p] = q.M;
        g.N[p] = q.N;
        g.ep[p] = q.ep;
        const size_t esz = q.ep.out_kind == 1 ? 2 : 4;
        g.vec_ok[p] = !((q.ep.c && ((reinterpret_cast<uintptr_t>(q.ep.c) & 15) || (static_cast<size_t>(q.ep.ldc) * esz) % 16)) ||
                        (q.ep.mask && ((reinterpret_cast<uintptr_t>(q.ep.mask) & 15) || q.ep.ldm % 8)));
        if (!make_map(&maps.a[p], q.a, q.M, q.K, q.lda, kBM) || !make_map(&maps.b[p], q.b, q.N, q.K, q.ldb, 64))
            return cudaErrorInvalidValue;
        cta += g.tiles_m[p] * g.tiles_n[p] * splits;
    }
    g.cta_begin[n] = cta;
    for (int p = n; p < kMaxGemmGroup; ++p) {
        maps.a[p] = maps.a[0];
        maps.b[p] = maps.b[0];
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cta);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = sizeof(Smem<64>) + 1024;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = g_pdl.load();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, gemm_group_kernel<64>, maps, g, error, g_wait_limit_ns.load(),
                              g_withhold_first.load());
}

cudaError_t gemm_prepare() {
    cudaError_t e = configure_group();
    if (e == cudaSuccess) e = configure_bn<64>();
    if (e == cudaSuccess) e = configure_bn<128>();
    if (e == cudaSuccess) e = configure_bn<256>();
    if (e == cudaSuccess) (void)sm_count();
    if (e == cudaSuccess && !encode_fn()) e = cudaErrorNotSupported;  // the CUDA driver API's tensor-map encoder
    return e;
}

cudaError_t gemm_bf16(const void* A, int lda, const void* B, int ldb, void* C, int ldc, int M, int N, int K,
                      const float* bias, int relu, int out_kind, int splits, int* error, cudaStream_t st) {
    GemmEpilogue ep{};
    ep.c = C;
    ep.ldc = ldc;
    ep.out_kind = out_kind;
    ep.bias = bias;
    ep.relu = relu;
    return gemm_bf16_ep(A, lda, B, ldb, M, N, K, ep, splits, error, st);
}

}  // namespace ntp

extern "C" ntp_status ntp_gemm_bf16(const void* A, int32_t lda, const void* B, int32_t ldb, void* C, int32_t ldc,
                                    int32_t M, int32_t N, int32_t K, const float* bias, int32_t relu,
                                    int32_t out_kind, int32_t splits, void* stream) {
    if (!A || !B || !C || out_kind < 0 || out_kind > 2) return NTP_ERR_INVALID;
    static int* d_err = nullptr;  // error word of the GEMM pipeline (one per process)
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (!d_err && cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) return NTP_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) return NTP_ERR_CUDA;
    const cudaError_t e = ntp::gemm_bf16(A, lda, B, ldb, C, ldc, M, N, K, bias, relu, out_kind, splits, d_err, st);
    if (e == cudaErrorInvalidValue) return NTP_ERR_INVALID;
    if (e != cudaSuccess) return NTP_ERR_CUDA;
    int h = 0;
    if (cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return NTP_ERR_CUDA;
    return h ? NTP_ERR_TIMEOUT : NTP_OK;
}

extern "C" ntp_status ntp_gemm_set_wait_limit(uint64_t wait_limit_ns, int32_t withhold_first_copy) {
    ntp::g_wait_limit_ns.store(wait_limit_ns ? wait_limit_ns : ntp::kWaitLimitNs);
    ntp::g_withhold_first.store(withhold_first_copy ? 1 : 0);
    return NTP_OK;
}
