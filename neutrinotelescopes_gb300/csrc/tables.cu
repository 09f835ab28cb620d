// tables.cu -- the flow's training-table generator on the device.
//
// Restates run_sim of scripts/photon_tables.jl:52-170 (chrhck/NeutrinoTelescopes)
// for many simulations at once: every simulation is one source of a single
// propagation launch around one multi-PMT module; each of its hits is
// weighted (calc_total_weight!, times a per-simulation factor: the
// oversampling correction, photons of the source / photons simulated), then
// for R random module orientations
// assigned to the PMT whose cone contains it (make_hits_from_photons with a
// rotated module, detection.jl:72-104) and resampled per (simulation,
// orientation, PMT) as resample_simulation does (pmt_frontend/pipeline.jl:
// 86-116), with the count N = Poisson(sum(w) * downsample) not capped by the
// simulated hits, and min(N, max_rows_per_group, ESS/4 + 1) hits drawn
// without replacement with probability proportional to w, where ESS =
// (sum w)^2 / sum w^2 is the group's effective sample size (the cap on rows
// is create_pmt_table's limit of 200, extended_cascade_model.jl:298-311).
// The ESS cap keeps the drawn times a weighted sample: with weights scaled up
// (fewer photons simulated than the source emits) N can reach the number of
// simulated hits, and a draw of nearly all hits would ignore their weights.
// A drawn hit becomes one row (condition of its group, time residual, N).
//
// A hit can fall into a PMT of several orientations, so the unit of the
// grouping is a (hit, orientation) pair.  The PMT test uses FP32 dot products
// against cos(opening angle) rather than the reference's FP64 acos of the
// clamped dot product: the same rule up to rounding at the cone's edge.
// Selection keys: Efraimidis-Spirakis log(u)/w with u from Philox4x32-10
// keyed by the pair (photon identity, orientation), so rows do not depend on
// the order of the hits; counts use the Poisson stream of resample.cu.
#include <cuda_runtime.h>

#include "ntp_device.cuh"
#include "ntp_internal.h"

namespace ntp {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kDrawTableKey = 0x54424C00u;  // "TBL" + orientation in the low byte(s)

__device__ __forceinline__ unsigned long long ordered_key(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// First PMT (0-based) of orientation r of simulation s whose cone contains the
// unit direction (ux, uy, uz) from the module centre; -1 for none.
__device__ __forceinline__ int table_pmt(const float* __restrict__ axes, int s, int r, int R, int P, float ux,
                                         float uy, float uz, float cos_open) {
    const float* a = axes + (static_cast<size_t>(s) * R + r) * P * 3;
    for (int j = 0; j < P; ++j) {
        const float dp = ux * __ldg(a + 3 * j) + uy * __ldg(a + 3 * j + 1) + uz * __ldg(a + 3 * j + 2);
        if (dp > cos_open) return j;
    }
    return -1;
}

struct HitDir {
    int s;
    float ux, uy, uz;
};

__device__ __forceinline__ HitDir hit_dir(const ntp_hit* hits, unsigned long long i, float3 c) {
    const float4 pos = __ldg(reinterpret_cast<const float4*>(hits + i));
    const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
    const float rx = pos.x - c.x, ry = pos.y - c.y, rz = pos.z - c.z;
    const float inv = rsqrtf(rx * rx + ry * ry + rz * rz);
    return HitDir{static_cast<int>(ids.y), rx * inv, ry * inv, rz * inv};
}

__global__ void count_kernel(const ntp_hit* __restrict__ hits, unsigned long long n, const double* __restrict__ w,
                             const double* __restrict__ scale, int n_sims, int R, int P, float3 c,
                             const float* __restrict__ axes, float cos_open, double* __restrict__ wsum,
                             double* __restrict__ w2sum, unsigned long long* __restrict__ npos,
                             unsigned long long* __restrict__ nall) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const HitDir h = hit_dir(hits, i, c);
        if (h.s < 0 || h.s >= n_sims) continue;
        const double wi = w[i] * __ldg(scale + h.s);
        for (int r = 0; r < R; ++r) {
            const int j = table_pmt(axes, h.s, r, R, P, h.ux, h.uy, h.uz, cos_open);
            if (j < 0) continue;
            const size_t g = (static_cast<size_t>(h.s) * R + r) * P + j;
            atomicAdd(wsum + g, wi);
            atomicAdd(w2sum + g, wi * wi);
            atomicAdd(nall + g, 1ull);
            if (wi > 0.0) atomicAdd(npos + g, 1ull);
        }
    }
}

__global__ void bucket_kernel(const ntp_hit* __restrict__ hits, unsigned long long n, const double* __restrict__ w,
                              const double* __restrict__ scale, int n_sims, int R, int P, float3 c,
                              const float* __restrict__ axes, float cos_open, uint2 key,
                              const unsigned long long* __restrict__ start,
                              unsigned long long* __restrict__ fill, unsigned long long* __restrict__ order,
                              unsigned long long* __restrict__ okey) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const HitDir h = hit_dir(hits, i, c);
        if (h.s < 0 || h.s >= n_sims) continue;
        const double wi = w[i] * __ldg(scale + h.s);
        const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
        for (int r = 0; r < R; ++r) {
            const int j = table_pmt(axes, h.s, r, R, P, h.ux, h.uy, h.uz, cos_open);
            if (j < 0) continue;
            const size_t g = (static_cast<size_t>(h.s) * R + r) * P + j;
            const unsigned long long pos = start[g] + atomicAdd(fill + g, 1ull);
            order[pos] = i;
            if (wi > 0.0) {
                const uint4 u = philox4x32_10(make_uint4(kDrawTableKey + static_cast<uint32_t>(r), ids.z, ids.w, ids.y),
                                              key);
                okey[pos] = ordered_key(log(u01_53(u.x, u.y)) / wi);
            } else {
                okey[pos] = 0ull;  // never drawn; real keys map to >= 1
            }
        }
    }
}

__global__ void tres_kernel(const ntp_hit* __restrict__ hits, unsigned long long n, const double* __restrict__ tgeo,
                            int n_sims, double* __restrict__ tres) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float t = __ldg(reinterpret_cast<const float*>(hits + i) + 3);
        const int s = static_cast<int>(__ldg(reinterpret_cast<const uint32_t*>(hits + i) + 13));
        tres[i] = (s >= 0 && s < n_sims) ? static_cast<double>(t) - __ldg(tgeo + s)
                                         : __longlong_as_double(0x7ff8000000000000LL);
    }
}

// rows [0, n_hit_rows) from the selection (group, time residual); rows
// [n_hit_rows, n_hit_rows + n_zero) count-only rows of groups without hits
__global__ void rows_kernel(unsigned long long n_hit_rows, const int32_t* __restrict__ og,
                            const double* __restrict__ ot, unsigned long long n_zero,
                            const int32_t* __restrict__ zero_groups, const unsigned long long* __restrict__ ndraw,
                            const float* __restrict__ gcond, float* __restrict__ cond, float* __restrict__ tres,
                            float* __restrict__ nhits, int32_t* __restrict__ has_time, int32_t* __restrict__ row_group) {
    const unsigned long long total = n_hit_rows + n_zero;
    for (unsigned long long q = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; q < total;
         q += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const bool hit = q < n_hit_rows;
        const int g = hit ? og[q] : zero_groups[q - n_hit_rows];
#pragma unroll
        for (int k = 0; k < 5; ++k) cond[q * 5 + k] = __ldg(gcond + static_cast<size_t>(g) * 5 + k);
        tres[q] = hit ? static_cast<float>(ot[q]) : 0.0f;
        nhits[q] = static_cast<float>(ndraw[g]);
        has_time[q] = hit ? 1 : 0;
        if (row_group) row_group[q] = g;
    }
}

int grid_for(unsigned long long n) {
    unsigned long long g = (n + kBlock - 1) / kBlock;
    return static_cast<int>(g < 1 ? 1 : (g > 65535ull * 8 ? 65535ull * 8 : g));
}

}  // namespace

cudaError_t launch_table_count(const ntp_hit* hits, unsigned long long n, const double* w, const double* scale,
                               int n_sims, int R, int P, float3 center, const float* axes, float cos_open,
                               double* wsum, double* w2sum, unsigned long long* npos, unsigned long long* nall,
                               cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    count_kernel<<<grid_for(n), kBlock, 0, st>>>(hits, n, w, scale, n_sims, R, P, center, axes, cos_open, wsum, w2sum,
                                                 npos, nall);
    return cudaGetLastError();
}

cudaError_t launch_table_bucket(const ntp_hit* hits, unsigned long long n, const double* w, const double* scale,
                                int n_sims, int R, int P, float3 center, const float* axes, float cos_open, uint2 key,
                                const unsigned long long* start, unsigned long long* fill, unsigned long long* order,
                                unsigned long long* okey, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    bucket_kernel<<<grid_for(n), kBlock, 0, st>>>(hits, n, w, scale, n_sims, R, P, center, axes, cos_open, key, start, fill,
                                                  order, okey);
    return cudaGetLastError();
}

cudaError_t launch_table_tres(const ntp_hit* hits, unsigned long long n, const double* tgeo, int n_sims, double* tres,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    tres_kernel<<<grid_for(n), kBlock, 0, st>>>(hits, n, tgeo, n_sims, tres);
    return cudaGetLastError();
}

cudaError_t launch_table_rows(unsigned long long n_hit_rows, const int32_t* og, const double* ot,
                              unsigned long long n_zero, const int32_t* zero_groups, const unsigned long long* ndraw,
                              const float* gcond, float* cond, float* tres, float* nhits, int32_t* has_time,
                              int32_t* row_group, cudaStream_t st) {
    if (n_hit_rows + n_zero == 0) return cudaSuccess;
    rows_kernel<<<grid_for(n_hit_rows + n_zero), kBlock, 0, st>>>(n_hit_rows, og, ot, n_zero, zero_groups, ndraw,
                                                                  gcond, cond, tres, nhits, has_time, row_group);
    return cudaGetLastError();
}

}  // namespace ntp
