// hits.cu -- per-hit post-processing on the device.
//
// Replaces the host DataFrame passes of chrhck/NeutrinoTelescopes:
//   make_hits_from_photons / check_pmt_hit  photon_prop_cuda.jl:884-904, detection.jl:72-104
//   calc_total_weight!                     photon_prop_cuda.jl:850-882, detection.jl:139-163
//   calc_time_residual!                    photon_prop_cuda.jl:906-924
// The reference evaluates these in double precision where its types promote to
// Float64 (hit position minus module centre, PMT axes, acceptance table, the
// weight product, tgeo); the kernels do the same, so PMT indices match the
// reference's rule exactly on identical hits.  They are memory-bound
// streaming passes over the 64-byte hit records.
#include <cuda_runtime.h>

#include "ntp_device.cuh"
#include "ntp_internal.h"

namespace ntp {

namespace {

constexpr int kHitBlock = 256;

__device__ __forceinline__ int find_target(const uint2* __restrict__ sorted, int n, uint32_t id) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const uint2 e = __ldg(sorted + mid);
        if (e.x == id) return static_cast<int>(e.y);
        if (e.x < id) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// check_pmt_hit, detection.jl:72-104 (and :86 for a DetectionSphere): the
// 1-based PMT whose opening cone contains the hit position, 0 for none.
__device__ __forceinline__ int pmt_of_hit(const HitTargetTable& t, int k, const float4 pos,
                                          const double* __restrict__ axes) {
    if (__ldg(t.kind + k) == NTP_TARGET_SPHERE) return 1;
    const float4 c = __ldg(t.targets + k);
    double rx = static_cast<double>(pos.x) - static_cast<double>(c.x);
    double ry = static_cast<double>(pos.y) - static_cast<double>(c.y);
    double rz = static_cast<double>(pos.z) - static_cast<double>(c.z);
    const double nr = sqrt(rx * rx + ry * ry + rz * rz);
    rx /= nr;
    ry /= nr;
    rz /= nr;
    const double opening = __ldg(t.opening + k);
    const int off = __ldg(t.pmt_offset + k), np = __ldg(t.n_pmts + k);
    for (int j = 0; j < np; ++j) {
        const double* a = axes + 3 * (off + j);
        double dp = rx * __ldg(a) + ry * __ldg(a + 1) + rz * __ldg(a + 2);
        dp = fmin(fmax(dp, -1.0), 1.0);
        if (acos(dp) < opening) return j + 1;
    }
    return 0;
}

__global__ void make_hits_kernel(const HitTargetTable t, const ntp_hit* __restrict__ hits,
                                 unsigned long long n, const double* __restrict__ axes,
                                 int32_t* __restrict__ pmt_id) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float4 pos = __ldg(reinterpret_cast<const float4*>(hits + i));
        const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
        const int k = find_target(t.sorted_ids, t.n_targets, ids.x);
        pmt_id[i] = k >= 0 ? pmt_of_hit(t, k, pos, axes) : 0;
    }
}

// fast_linear_interp, utils.jl:24-53, on ascending knots (float or double).
template <typename T>
__device__ __forceinline__ T fast_linear_interp(T x, const T* __restrict__ xs, const T* __restrict__ ys, int n) {
    const T lower = xs[0], upper = xs[n - 1];
    x = x < lower ? lower : (x > upper ? upper : x);
    if (x == lower) return ys[0];
    if (x == upper) return ys[n - 1];
    int lo = 0, hi = n - 1;  // first index with xs[i] >= x lies in (lo, hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (xs[mid] < x) lo = mid;
        else hi = mid;
    }
    const T step = xs[hi] - xs[lo];
    const T along = (x - xs[lo]) / step;
    return ys[lo] + (ys[hi] - ys[lo]) * along;
}

__global__ void total_weight_kernel(const HitTargetTable t, const ntp_hit* __restrict__ hits,
                                    unsigned long long n, const float* __restrict__ abs_wl,
                                    const float* __restrict__ abs_len, int n_abs,
                                    const double* __restrict__ acc_wl, const double* __restrict__ acc,
                                    int n_acc, double* area_acc, double* wl_acc, double* abs_weight,
                                    double* total) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float4 dirwl = __ldg(reinterpret_cast<const float4*>(hits + i) + 1);
        const float4 idir_dist = __ldg(reinterpret_cast<const float4*>(hits + i) + 2);
        const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
        const int k = find_target(t.sorted_ids, t.n_targets, ids.x);
        const double aa = k >= 0 ? __ldg(t.area_acc + k) : 0.0;
        const float wl = dirwl.w;
        // absorption_length on Float32 knots (medium.jl:399-404), exp in float
        const float al = fast_linear_interp<float>(wl, abs_wl, abs_len, n_abs);
        const double aw = static_cast<double>(expf(-idir_dist.w / al));
        const double wa = fast_linear_interp<double>(static_cast<double>(wl), acc_wl, acc, n_acc);
        if (area_acc) area_acc[i] = aa;
        if (wl_acc) wl_acc[i] = wa;
        if (abs_weight) abs_weight[i] = aw;
        if (total) total[i] = aa * wa * aw;
    }
}

// Per-hit total weight of calc_total_weight! (photon_prop_cuda.jl:850-882).
__device__ __forceinline__ double hit_weight(double area_acc, float wl, float dist, const float* __restrict__ abs_wl,
                                             const float* __restrict__ abs_len, int n_abs,
                                             const double* __restrict__ acc_wl, const double* __restrict__ acc,
                                             int n_acc) {
    const float al = fast_linear_interp<float>(wl, abs_wl, abs_len, n_abs);
    const double aw = static_cast<double>(expf(-dist / al));
    const double wa = fast_linear_interp<double>(static_cast<double>(wl), acc_wl, acc, n_acc);
    return area_acc * wa * aw;
}

// One pass over the hits: PMT assignment, weight and time (hit time or time
// residual) of every hit, accumulated in double precision per (target, PMT):
// weight sum, hit count and a weighted time histogram.
__global__ void pmt_summary_kernel(const HitTargetTable t, const ntp_hit* __restrict__ hits, unsigned long long n,
                                   const double* __restrict__ axes, const float* __restrict__ abs_wl,
                                   const float* __restrict__ abs_len, int n_abs, const double* __restrict__ acc_wl,
                                   const double* __restrict__ acc, int n_acc, const double* __restrict__ tgeo,
                                   int use_tres, int max_pmts, int n_bins, double t_min, double inv_bin,
                                   double* __restrict__ wsum, double* __restrict__ count, double* __restrict__ hist) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float4 pos = __ldg(reinterpret_cast<const float4*>(hits + i));
        const float4 dirwl = __ldg(reinterpret_cast<const float4*>(hits + i) + 1);
        const float4 idir_dist = __ldg(reinterpret_cast<const float4*>(hits + i) + 2);
        const uint4 ids = __ldg(reinterpret_cast<const uint4*>(hits + i) + 3);
        const int k = find_target(t.sorted_ids, t.n_targets, ids.x);
        if (k < 0) continue;
        const int j = pmt_of_hit(t, k, pos, axes);
        if (j <= 0 || j > max_pmts) continue;
        const double w = hit_weight(__ldg(t.area_acc + k), dirwl.w, idir_dist.w, abs_wl, abs_len, n_abs, acc_wl, acc,
                                    n_acc);
        const size_t slot = static_cast<size_t>(k) * max_pmts + (j - 1);
        atomicAdd(wsum + slot, w);
        atomicAdd(count + slot, 1.0);
        if (n_bins > 0) {
            const double tv = use_tres ? static_cast<double>(pos.w) - __ldg(tgeo + k) : static_cast<double>(pos.w);
            const double b = floor((tv - t_min) * inv_bin);
            if (b >= 0.0 && b < static_cast<double>(n_bins)) atomicAdd(hist + slot * n_bins + static_cast<int>(b), w);
        }
    }
}

__global__ void time_residual_kernel(const HitTargetTable t, const ntp_hit* __restrict__ hits,
                                     unsigned long long n, const double* __restrict__ tgeo,
                                     double* __restrict__ tres) {
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const float time = __ldg(reinterpret_cast<const float*>(hits + i) + 3);
        const uint32_t id = __ldg(reinterpret_cast<const uint32_t*>(hits + i) + 12);
        const int k = find_target(t.sorted_ids, t.n_targets, id);
        tres[i] = k >= 0 ? static_cast<double>(time) - __ldg(tgeo + k) : __longlong_as_double(0x7ff8000000000000LL);
    }
}

int grid_for(unsigned long long n) {
    unsigned long long g = (n + kHitBlock - 1) / kHitBlock;
    return static_cast<int>(g < 1 ? 1 : (g > 65535ull * 8 ? 65535ull * 8 : g));
}

}  // namespace

cudaError_t launch_make_hits(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                             const double* pmt_axes, int32_t* pmt_id, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    make_hits_kernel<<<grid_for(n), kHitBlock, 0, stream>>>(t, hits, n, pmt_axes, pmt_id);
    return cudaGetLastError();
}

cudaError_t launch_total_weight(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                                const float* abs_wl, const float* abs_len, int n_abs,
                                const double* acc_wl, const double* acc, int n_acc,
                                double* area_acc, double* wl_acc, double* abs_weight,
                                double* total, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    total_weight_kernel<<<grid_for(n), kHitBlock, 0, stream>>>(t, hits, n, abs_wl, abs_len, n_abs, acc_wl,
                                                               acc, n_acc, area_acc, wl_acc, abs_weight,
                                                               total);
    return cudaGetLastError();
}

cudaError_t launch_pmt_summary(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n, const double* axes,
                               const float* abs_wl, const float* abs_len, int n_abs, const double* acc_wl,
                               const double* acc, int n_acc, const double* tgeo, int use_tres, int max_pmts,
                               int n_bins, double t_min, double t_max, double* wsum, double* count, double* hist,
                               cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const double inv_bin = n_bins > 0 ? static_cast<double>(n_bins) / (t_max - t_min) : 0.0;
    pmt_summary_kernel<<<grid_for(n), kHitBlock, 0, stream>>>(t, hits, n, axes, abs_wl, abs_len, n_abs, acc_wl, acc,
                                                              n_acc, tgeo, use_tres, max_pmts, n_bins, t_min, inv_bin,
                                                              wsum, count, hist);
    return cudaGetLastError();
}

cudaError_t launch_time_residual(const HitTargetTable& t, const ntp_hit* hits, unsigned long long n,
                                 const double* tgeo, double* tres, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    time_residual_kernel<<<grid_for(n), kHitBlock, 0, stream>>>(t, hits, n, tgeo, tres);
    return cudaGetLastError();
}

}  // namespace ntp
