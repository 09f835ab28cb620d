// ntp_internal.h -- shared declarations between the C ABI layer and the
// kernels of libntp.so.  Not part of the public interface.
#pragma once

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/ntp.h"

namespace ntp {

constexpr int kPropBlock = 256;      // threads per block of the propagation kernel
constexpr int kMaxSmemTargets = 8192;  // targets staged in shared memory (20 B each)
// with column culling, targets are staged only while the kernel's shared
// memory stays within this budget (four blocks per SM, room left for L1)
constexpr size_t kSmemStageBudget = 32 * 1024;
constexpr int kMaxSmemColumns = 2048;  // columns staged in shared memory (32 B each)
constexpr int kMaxSmemGridInts = 16384; // grid offsets + items staged in shared memory (4 B each)
constexpr int kGridMinColumns = 9;      // below this many columns every column is tested

// A vertical column of targets sharing (x, y): the unit of the geometric
// culling.  Members are target indices sorted by z.
struct Column {
    float cx, cy;  // axis
    float r_cull;  // largest member radius plus a rounding margin
    float z0;      // z of the lowest member
    float dz;      // uniform member spacing, 0 if not uniform
    int first;     // offset of the members in the member list
    int count;
    float z_last;  // z of the highest member
};
static_assert(sizeof(Column) == 32, "Column is 32 bytes");

// Everything one launch of the propagation kernel reads.
struct PropParams {
    const ntp_source* sources;            // device
    const unsigned long long* prefix;     // device, n_src + 1 exclusive photon offsets
    int n_src;
    unsigned long long total;             // photons over all sources

    const float4* targets;                // device, (x, y, z, r^2)
    const uint32_t* target_ids;           // device, module_id per target
    int n_targets;
    int targets_in_smem;                  // stage targets (and ids, column members) in shared memory
    int columns_in_smem;                  // stage the columns (and the cell grid) in shared memory

    const Column* columns;                // device; nullptr = scan every target
    const int* members;                   // device, target indices grouped by column
    int n_columns;

    // 2-D grid over the column axes (used when cell_start != nullptr): cell
    // (ix, iy) lists the columns whose culling disk, widened by a margin,
    // overlaps it; a step walks the cells its horizontal projection crosses.
    const int* cell_start;                // device, nx * ny + 1 offsets into cell_items
    const int* cell_items;                // device, column indices
    int grid_nx, grid_ny, n_cell_items;
    float grid_x0, grid_y0, grid_h, grid_inv_h;
    // Lattice mode (grid_lattice != 0): every cell holds at most one column,
    // sitting at the cell's centre (strings on a regular lattice); a step
    // then tests the lattice points near its line directly instead of
    // walking every cell it crosses.  lat_rcull2: the largest r_cull^2.
    int grid_lattice;
    float lat_rcull2;

    const float4* medium;                 // device, per knot (n, v_group, l_scatter, 0)
    int n_medium;
    float wl_min;
    float medium_scale;                   // (n_medium - 1) / (wl_max - wl_min)

    int spec_kind;
    int n_spec;
    const float* spec_knots;              // device
    float spec_p0, spec_p1;

    float hg_g;
    float rayleigh_fraction;
    // the Rayleigh branch as an integer test on the Philox word w:
    // u01(w) < rayleigh_fraction exactly when w <= rayleigh_wmax (and
    // rayleigh_on); set by set_rayleigh
    uint32_t rayleigh_wmax;
    int rayleigh_on;
    int max_steps;
    int hit_policy;
    int exact_pole;
    uint2 key;
    // Philox round keys: rk[2r], rk[2r + 1] = key + r (0x9E3779B9, 0xBB67AE85)
    // for rounds r = 0..9, precomputed on the host so that each round reads
    // them as kernel-parameter operands (set by set_key)
    uint32_t rk[20];

    // Philox stream word per source (nullptr: the source index).  The serving
    // loop passes event ids, so an event draws the same photons whatever
    // batch it is simulated in.
    const uint32_t* src_stream;

    // Per-source output (serving): when src_hit_count != nullptr, hits of
    // source s go to hits[src_hit_base[o] + k] for k < src_hit_cap[o], with
    // src_hit_count[o] counting every hit (exact even past the cap), where
    // o = src_out[s] (nullptr: o = s).  Several sources of a launch, or of
    // successive launches, may share one output slot: the serving loop
    // splits an event into photon chunks that all write to the event's slot.
    unsigned long long* src_hit_count;
    const unsigned long long* src_hit_base;
    const unsigned long long* src_hit_cap;
    const uint32_t* src_out;
    // First photon index of each source entry within its Philox stream
    // (nullptr: 0): a chunk [a, b) of an event draws exactly the photons a
    // .. b-1 that the whole event draws.
    const unsigned long long* src_photon_offset;

    ntp_hit* hits;                        // device
    unsigned long long capacity;
    unsigned long long* counters;         // device: [0] photons claimed, [1] hits, [2] photons done, [3] photon-steps
    unsigned long long chunk;             // photons a warp claims at once
    int refill_min;                       // idle lanes a warp gathers before it initialises new photons
};

// The Philox key of a launch (low and high 32 bits of the seed) and its
// round keys.
inline void set_key(PropParams& p, uint64_t seed) {
    p.key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    for (uint32_t r = 0; r < 10; ++r) {
        p.rk[2 * r] = p.key.x + r * 0x9E3779B9u;
        p.rk[2 * r + 1] = p.key.y + r * 0xBB67AE85u;
    }
}

// The phase-function mixture: u01(w) = (m + 1/2) 2^-23 with m = w >> 9 is
// below f for the first T = ceil(f 2^23 - 1/2) values of m (clamped to [0,
// 2^23]), i.e. for w <= 512 T - 1.
inline void set_rayleigh(PropParams& p, float f) {
    p.rayleigh_fraction = f;
    double t = std::ceil(static_cast<double>(f) * 8388608.0 - 0.5);
    t = t < 0.0 ? 0.0 : (t > 8388608.0 ? 8388608.0 : t);
    const uint64_t T = static_cast<uint64_t>(t);
    p.rayleigh_on = T > 0 ? 1 : 0;
    p.rayleigh_wmax = T > 0 ? static_cast<uint32_t>(T * 512u - 1u) : 0u;
}

size_t prop_smem_bytes(const PropParams& p);

// What the propagation kernel stages in shared memory.  Without columns a
// step tests every target: targets staged when they fit at all.  With
// column culling a step reads the columns (and the cell grid) every time
// and a target only when it is a candidate: columns staged, targets only
// while the total stays within kSmemStageBudget (more would cost blocks per
// SM; cached global loads serve the rare candidate tests).
inline void choose_staging(PropParams& p) {
    p.columns_in_smem = p.columns ? 1 : 0;
    p.targets_in_smem = p.n_targets <= kMaxSmemTargets ? 1 : 0;
    if (p.columns && p.targets_in_smem && prop_smem_bytes(p) > kSmemStageBudget) p.targets_in_smem = 0;
}
cudaError_t launch_propagate(const PropParams& p, int grid, cudaStream_t stream);
cudaError_t propagate_occupancy(const PropParams& p, int* blocks_per_sm);
// the kernel launch_propagate uses (for CUDA-graph kernel-node updates)
const void* propagate_kernel_fn();

// Checks shared by ntp_set_medium / ntp_set_spectrum and the context-free
// ntp_propagate_noalloc: nullptr when the descriptor is valid, else the
// reason.  need_absorption: also check the absorption table (unused by the
// propagation kernel itself).
const char* check_medium(const ntp_medium_desc* m, bool need_absorption);
const char* check_spectrum(const ntp_spectrum_desc* s);

// The error slot of context-free calls (ntp_create, ntp_propagate_noalloc),
// one per host thread; ntp_last_error(NULL) returns it.
void set_free_error(const char* msg);
const char* free_error();

// Medium / spectrum / target part of the kernel parameters from a context
// whose tables are set (ntp_abi.cu); returns false if a table is missing.
bool fill_world_params(const ntp_ctx* ctx, PropParams& p);
int ctx_device(const ntp_ctx* ctx);
int ctx_num_sms(const ntp_ctx* ctx);
void set_ctx_error(ntp_ctx* ctx, const char* msg);

// Hit post-processing (make_hits / weights / time residual).
struct HitTargetTable {
    const uint2* sorted_ids;   // (module_id, target index), ascending module_id
    int n_targets;
    const float4* targets;     // (x, y, z, r^2)
    const float* radius;       // float radius per target
    const int* kind;           // ntp_target_kind per target
    const int* n_pmts;
    const int* pmt_offset;
    const double* opening;     // PMT opening angle (rad) per target
    const double* area_acc;    // area acceptance per target
};

cudaError_t launch_make_hits(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                             const double* pmt_axes, int32_t* pmt_id, cudaStream_t stream);
cudaError_t launch_total_weight(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                                const float* abs_wl, const float* abs_len, int n_abs,
                                const double* acc_wl, const double* acc, int n_acc,
                                double* area_acc, double* wl_acc, double* abs_weight,
                                double* total, cudaStream_t stream);
cudaError_t launch_pmt_summary(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n, const double* axes,
                               const float* abs_wl, const float* abs_len, int n_abs, const double* acc_wl,
                               const double* acc, int n_acc, const double* tgeo, int use_tres, int max_pmts,
                               int n_bins, double t_min, double t_max, double* wsum, double* count, double* hist,
                               cudaStream_t stream);
// Epilogue of the tensor-core GEMM: value = acc (+ bias[col]) (ReLU) (zeroed
// where mask[row][col] <= 0); stored to c (FP32 / BF16 / FP32 atomic add),
// to ct transposed (BF16, ct[col * ldct + row]) and summed per column into
// colsum (FP32 atomics); every output pointer may be NULL.
struct GemmEpilogue {
    void* c;
    int ldc;
    int out_kind;                // 0 FP32, 1 BF16, 2 FP32 atomic add
    const float* bias;
    int relu;
    __nv_bfloat16* ct;
    int ldct;
    const __nv_bfloat16* mask;
    int ldm;
    float* colsum;
};
cudaError_t gemm_bf16_ep(const void* A, int lda, const void* B, int ldb, int M, int N, int K, const GemmEpilogue& ep,
                         int splits, int* error, cudaStream_t st);
// Sets the GEMM kernels' function attributes (before a stream capture).
cudaError_t gemm_prepare();
// Independent products C_p = A_p B_p^T (each as in gemm_bf16_ep) in one
// launch, split along K to about two CTAs per SM where the epilogue is the
// atomic FP32 output alone (flow_gemm.cu).
constexpr int kMaxGemmGroup = 4;
struct GemmProblem {
    const void* a;
    int lda;
    const void* b;
    int ldb;
    int M, N, K;
    GemmEpilogue ep;
};
cudaError_t gemm_bf16_group(const GemmProblem* problems, int n, int* error, cudaStream_t st);

// C = A * B^T, BF16 operands (K-major), FP32 accumulation on the tensor cores
// (flow_gemm.cu).  out_kind: 0 = FP32, 1 = BF16, 2 = FP32 atomic add.
cudaError_t gemm_bf16(const void* A, int lda, const void* B, int ldb, void* C, int ldc, int M, int N, int K,
                      const float* bias, int relu, int out_kind, int splits, int* error, cudaStream_t st);

// One stage of a layer chain (flow_chain.cu): D = A W^T with n output and k
// input columns, value = D (+ bias[col]) (ReLU) (zeroed where
// mask[row][col] <= 0), stored as BF16 row-major to c, FP32 row-major to c32,
// BF16 transposed to ct (ct[col * ldct + row]) and summed per column into
// colsum (FP32 atomics); every output pointer may be NULL.  The value also
// becomes the next stage's A (BF16, on chip).
constexpr int kMaxChainStages = 4;
struct ChainStage {
    int n, k;
    const float* bias;
    int relu;
    const __nv_bfloat16* mask;
    int ldm;
    __nv_bfloat16* c;
    int ldc;
    float* c32;
    int ldc32;
    __nv_bfloat16* ct;
    int ldct;
    float* colsum;
};
struct ChainSpec {
    int n_stages;
    int m;  // rows
    // nonzero: the weights were written before the previous kernel of the
    // stream started, so the first slices may be loaded before the wait for
    // that kernel (programmatic dependent launch)
    int weights_ready;
    ChainStage st[kMaxChainStages];
};
cudaError_t layer_chain(const void* a, int lda, const void* const* w, const ChainSpec& spec, int* error,
                        cudaStream_t stream);
// Sets the chain kernel's function attributes (before a stream capture).
cudaError_t layer_chain_prepare();

// training-table generator passes (tables.cu)
cudaError_t launch_table_count(const ntp_hit* hits, unsigned long long n, const double* w, const double* scale,
                               int n_sims, int R, int P, float3 center, const float* axes, float cos_open,
                               double* wsum, double* w2sum, unsigned long long* npos, unsigned long long* nall,
                               cudaStream_t st);
cudaError_t launch_table_bucket(const ntp_hit* hits, unsigned long long n, const double* w, const double* scale,
                                int n_sims, int R, int P, float3 center, const float* axes, float cos_open, uint2 key,
                                const unsigned long long* start, unsigned long long* fill, unsigned long long* order,
                                unsigned long long* okey, cudaStream_t st);
cudaError_t launch_table_tres(const ntp_hit* hits, unsigned long long n, const double* tgeo, int n_sims, double* tres,
                              cudaStream_t st);
cudaError_t launch_table_rows(unsigned long long n_hit_rows, const int32_t* og, const double* ot,
                              unsigned long long n_zero, const int32_t* zero_groups, const unsigned long long* ndraw,
                              const float* gcond, float* cond, float* tres, float* nhits, int32_t* has_time,
                              int32_t* row_group, cudaStream_t st);

// flow conditions of (event, module, PMT) triples (surrogate.cu); events are
// packed as {position[3], direction[3], log10 E, id (u32)} (event_in_size bytes)
size_t event_in_size();
cudaError_t launch_event_conditions_count(const void* events, int n_events, const float4* tg, const int* kind,
                                          const int* npmt, int n_targets, float d_min, float d_max,
                                          unsigned long long* ev_rows, int* ev_close, cudaStream_t st);
cudaError_t launch_event_conditions_fill(const void* events, int n_events, const float4* tg, const float* radius,
                                         const int* kind, const int* npmt, const int* pmt_off, const float* axes,
                                         int n_targets, float d_min, float d_max, float tgeo_scale,
                                         const unsigned long long* ev_first, unsigned long long* ev_fill, float* cond,
                                         unsigned long long* ckey, float* ctgeo, int32_t* cev, int32_t* ctgt,
                                         int32_t* cpmt, cudaStream_t st);

// resample_simulation passes (resample.cu)
cudaError_t launch_resample_group(const ntp_hit* hits, unsigned long long n, const int32_t* pmt, const double* w,
                                  const uint2* sorted_ids, int n_targets, int max_pmts, int32_t* group, double* wsum,
                                  unsigned long long* npos, unsigned long long* nall, cudaStream_t st);
cudaError_t launch_resample_draw(int n_groups, const double* wsum, const unsigned long long* npos, double downsample,
                                 uint2 key, unsigned long long* nsel, cudaStream_t st);
cudaError_t launch_resample_bucket(const ntp_hit* hits, unsigned long long n, const int32_t* group, const double* w,
                                   uint2 key, const unsigned long long* start, unsigned long long* fill,
                                   unsigned long long* order, unsigned long long* okey, cudaStream_t st);
cudaError_t launch_resample_select(int n_groups, const ntp_hit* hits, const double* tval,
                                   const unsigned long long* start, const unsigned long long* nall,
                                   const unsigned long long* nsel, const unsigned long long* out_start,
                                   const unsigned long long* order, const unsigned long long* okey, int32_t* out_group,
                                   double* out_time, unsigned long long* out_hit, cudaStream_t st);
cudaError_t launch_time_residual(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                                 const double* tgeo, double* tres, cudaStream_t stream);

}  // namespace ntp
