// resample.cu -- resample_simulation on the device.
//
// Restates pmt_frontend/pipeline.jl:86-116 of chrhck/NeutrinoTelescopes for
// hits grouped by (module, PMT): per group, N = min(Poisson(sum(w) *
// downsample), #hits with w > 0), then N hits drawn without replacement with
// probabilities proportional to w.  The weighted draw without replacement is
// done with exponential keys (Efraimidis and Spirakis, 2006): the N hits with
// the largest log(u)/w are distributed as successive weighted sampling.  u
// comes from Philox4x32-10 keyed by the hit's photon identity (source,
// photon) and the Poisson count from a Philox stream keyed by the group, so
// the result does not depend on the order of the hits.  Poisson variates: by
// inversion below a mean of 30, above by the transformed rejection of
// Hormann (1993, "PTRS"), at most kPoissonAttempts tries.
//
// Passes: (1) group of every hit, weight sums and positive-weight counts
// (FP64 atomics); (2) one thread per group draws N; (3) hits bucketed by
// group (counting sort); (4) one block per group finds the N-th largest key by
// bisection over its order-preserving 64-bit image and writes the selected
// hits to the group's output range.
#include <cuda_runtime.h>

#include <cmath>

#include "ntp_device.cuh"
#include "ntp_internal.h"

namespace ntp {

namespace {

constexpr int kBlock = 256;
constexpr uint32_t kDrawResampleKey = 0x52534B59u;  // "RSKY": per-hit key stream

__device__ __forceinline__ unsigned long long ordered(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double hit_key(const ntp_hit* hits, unsigned long long i, double w, uint2 key) {
    const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
    const uint4 r = philox4x32_10(make_uint4(kDrawResampleKey, ids.z, ids.w, ids.y), key);
    return log(u01_53(r.x, r.y)) / w;
}

__global__ void group_kernel(const ntp_hit* __restrict__ hits, unsigned long long n, const int32_t* __restrict__ pmt,
                             const double* __restrict__ w, const uint2* __restrict__ sorted_ids, int n_targets,
                             int max_pmts, int32_t* __restrict__ group, double* __restrict__ wsum,
                             unsigned long long* __restrict__ npos, unsigned long long* __restrict__ nall) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const uint32_t id = __ldg(reinterpret_cast<const uint32_t*>(hits + i) + 12);
        int lo = 0, hi = n_targets - 1, k = -1;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const uint2 e = __ldg(sorted_ids + mid);
            if (e.x == id) { k = static_cast<int>(e.y); break; }
            if (e.x < id) lo = mid + 1;
            else hi = mid - 1;
        }
        const int j = pmt[i];
        int g = -1;
        if (k >= 0 && j > 0 && j <= max_pmts) {
            g = k * max_pmts + (j - 1);
            atomicAdd(wsum + g, w[i]);
            atomicAdd(nall + g, 1ull);
            if (w[i] > 0.0) atomicAdd(npos + g, 1ull);
        }
        group[i] = g;
    }
}

__global__ void draw_kernel(int n_groups, const double* __restrict__ wsum, const unsigned long long* __restrict__ npos,
                            double downsample, uint2 key, unsigned long long* __restrict__ nsel) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_groups) return;
    const double k = poisson_draw(wsum[g] * downsample, key, static_cast<uint32_t>(g), 0u);
    const unsigned long long m = npos[g];
    nsel[g] = k < static_cast<double>(m) ? static_cast<unsigned long long>(k) : m;
}

// Buckets the hits by group and stores each hit's key image next to it
// (0 for hits with w <= 0, which are never drawn; real keys map to >= 1).
__global__ void bucket_kernel(const ntp_hit* __restrict__ hits, unsigned long long n, const int32_t* __restrict__ group,
                              const double* __restrict__ w, uint2 key, const unsigned long long* __restrict__ start,
                              unsigned long long* __restrict__ fill, unsigned long long* __restrict__ order,
                              unsigned long long* __restrict__ okey) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const int g = group[i];
        if (g < 0) continue;
        const unsigned long long pos = start[g] + atomicAdd(fill + g, 1ull);
        const double wi = w[i];
        order[pos] = i;
        okey[pos] = wi > 0.0 ? ordered(hit_key(hits, i, wi, key)) : 0ull;
    }
}

// One block per group: the N-th largest key by bisection on its 64-bit image,
// then every hit with a larger key (and ties up to N) goes to the output.
__global__ void select_kernel(const ntp_hit* __restrict__ hits, const double* __restrict__ tval,
                              const unsigned long long* __restrict__ start, const unsigned long long* __restrict__ nall,
                              const unsigned long long* __restrict__ nsel, const unsigned long long* __restrict__ out_start,
                              const unsigned long long* __restrict__ order, const unsigned long long* __restrict__ okey,
                              int32_t* __restrict__ out_group, double* __restrict__ out_time,
                              unsigned long long* __restrict__ out_hit) {
    const int g = blockIdx.x;
    const unsigned long long want = nsel[g];
    if (want == 0) return;
    const unsigned long long s0 = start[g], m = nall[g], o0 = out_start[g];
    __shared__ unsigned long long s_count;
    __shared__ unsigned long long s_fill;
    // largest T >= 1 with #{key >= T} >= want (T = 1 always qualifies)
    unsigned long long lo = 1, hi = ~0ull;
    for (int it = 0; it < 64 && lo < hi; ++it) {
        const unsigned long long mid = lo + (hi - lo) / 2 + 1;
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        unsigned long long c = 0;
        for (unsigned long long q = threadIdx.x; q < m; q += blockDim.x) c += okey[s0 + q] >= mid ? 1ull : 0ull;
        atomicAdd(&s_count, c);
        __syncthreads();
        if (s_count >= want) lo = mid;
        else hi = mid - 1;
        __syncthreads();
    }
    if (threadIdx.x == 0) s_fill = 0;
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass) {  // strictly above the threshold first, then ties
        for (unsigned long long q = threadIdx.x; q < m; q += blockDim.x) {
            const unsigned long long kb = okey[s0 + q];
            if (pass == 0 ? kb > lo : kb == lo) {
                const unsigned long long slot = atomicAdd(&s_fill, 1ull);
                if (slot < want) {
                    const unsigned long long i = order[s0 + q];
                    out_group[o0 + slot] = g;
                    out_time[o0 + slot] =
                        tval ? tval[i] : static_cast<double>(__ldg(reinterpret_cast<const float*>(hits + i) + 3));
                    out_hit[o0 + slot] = i;
                }
            }
        }
        __syncthreads();
    }
}

int grid_for(unsigned long long n) {
    unsigned long long g = (n + kBlock - 1) / kBlock;
    return static_cast<int>(g < 1 ? 1 : (g > 65535ull * 8 ? 65535ull * 8 : g));
}

}  // namespace

cudaError_t launch_resample_group(const ntp_hit* hits, unsigned long long n, const int32_t* pmt, const double* w,
                                  const uint2* sorted_ids, int n_targets, int max_pmts, int32_t* group, double* wsum,
                                  unsigned long long* npos, unsigned long long* nall, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    group_kernel<<<grid_for(n), kBlock, 0, st>>>(hits, n, pmt, w, sorted_ids, n_targets, max_pmts, group, wsum, npos,
                                                 nall);
    return cudaGetLastError();
}

cudaError_t launch_resample_draw(int n_groups, const double* wsum, const unsigned long long* npos, double downsample,
                                 uint2 key, unsigned long long* nsel, cudaStream_t st) {
    if (n_groups == 0) return cudaSuccess;
    draw_kernel<<<(n_groups + kBlock - 1) / kBlock, kBlock, 0, st>>>(n_groups, wsum, npos, downsample, key, nsel);
    return cudaGetLastError();
}

cudaError_t launch_resample_bucket(const ntp_hit* hits, unsigned long long n, const int32_t* group, const double* w,
                                   uint2 key, const unsigned long long* start, unsigned long long* fill,
                                   unsigned long long* order, unsigned long long* okey, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    bucket_kernel<<<grid_for(n), kBlock, 0, st>>>(hits, n, group, w, key, start, fill, order, okey);
    return cudaGetLastError();
}

cudaError_t launch_resample_select(int n_groups, const ntp_hit* hits, const double* tval,
                                   const unsigned long long* start, const unsigned long long* nall,
                                   const unsigned long long* nsel, const unsigned long long* out_start,
                                   const unsigned long long* order, const unsigned long long* okey, int32_t* out_group,
                                   double* out_time, unsigned long long* out_hit, cudaStream_t st) {
    if (n_groups == 0) return cudaSuccess;
    select_kernel<<<n_groups, kBlock, 0, st>>>(hits, tval, start, nall, nsel, out_start, order, okey, out_group,
                                               out_time, out_hit);
    return cudaGetLastError();
}

}  // namespace ntp
