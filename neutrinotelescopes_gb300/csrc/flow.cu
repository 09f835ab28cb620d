// flow.cu -- the arrival-time surrogate: a conditional rational-quadratic-
// spline flow with a Poisson count head, trained and evaluated on the GPU.
//
// Model (RQNormFlow, src/surrogate_models/extended_cascade_model.jl:53-125 and
// rq_spline_flow.jl:127-418 of chrhck/NeutrinoTelescopes): a conditioner
// network maps the condition c (5 features, zero-padded to 64) through three
// ReLU layers of 256 to the flow parameters: for each of L spline layers
// 3K+1 raw values (K = 10 or 12 bins) (K bin widths, K bin heights, K+1 knot slopes, constrained
// as constrain_spline_params, :170-206), then shift, raw scale (scale =
// 100 sigmoid(raw), :396-418) and the log expected hit count
// (extended_cascade_model.jl:119-121).  The output width L(3K+1)+3 is padded
// to a multiple of 64 with rows that stay zero.  The density of a time
// residual y: x = g_0(g_1(... g_{L-1}(y))) with g_l the inverse spline of
// layer l (inv_rqs_univariate, :334-389, linear outside [t_min, t_max]), and
// log p(y) = log N(x; shift, scale) + the sum of the inverse log-determinants.
// L = 1 is the reference's model.  Loss (log_likelihood_with_poisson,
// extended_cascade_model.jl:132-139): per sample -(n log lambda - lambda -
// lgamma(n + 1)) for its label's hit count n, plus -log p(y) when the sample
// carries a time; the mean over the batch.  The reference's dropout is not
// applied.
//
// The GEMMs of the network run on the tensor cores (flow_gemm.cu) with BF16
// weights / activations and FP32 accumulation; master weights, Adam moments
// and the spline head are FP32.  The head's gradient: the in-bin inverse
// spline in forward-mode dual numbers over its 7 inputs (y, bin x0, width,
// y0, height, two knot slopes), chained analytically through the softmax /
// cumulative-sum / softplus parametrisation, and in reverse mode across the
// spline layers and the base normal.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <type_traits>
#include <vector>

#include "ntp_device.cuh"
#include "ntp_internal.h"
#include "tc_ptx.cuh"

namespace ntp {

namespace {

constexpr int kCond = 5;
constexpr int kDerived = 4;    // derived input columns of NTP_FLOW_INPUT_DERIVED
constexpr int kIn = 64;        // padded input width (one K slice of the GEMM)
constexpr float kHalfLog200 = 2.6491586832740182f;  // ln(200) / 2
constexpr float kCherenkovCos = 0.74074074f;         // 1 / 1.35
constexpr float kPi = 3.14159265358979f;
constexpr int kMaxLayers = 5;
constexpr float kMinBin = 1e-4f, kMinSlope = 1e-4f;
constexpr float kLog2Pi = 1.8378770664093453f;
constexpr float kSlopeOffset = 0.5411666523385311f;  // log(exp(1 - 1e-4) - 1), rq_spline_flow.jl:152

// K bins per spline layer: 3K+1 raw parameters; per layer 3(K+1) knot values
__host__ __device__ constexpr int n_outputs(int L, int K) { return L * (3 * K + 1) + 3; }
__host__ __device__ constexpr int n_outputs_padded(int L, int K) { return (n_outputs(L, K) + 63) / 64 * 64; }
__host__ __device__ constexpr int knot_row(int L, int K) { return L * 3 * (K + 1) + 3; }

// ---------------------------------------------------------------- dual numbers
template <int N>
struct Dual {
    float v;
    float g[N];
};
template <int N>
__device__ __forceinline__ Dual<N> dvar(float v, int i) {
    Dual<N> r;
    r.v = v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = (j == i) ? 1.0f : 0.0f;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dconst(float v) {
    Dual<N> r;
    r.v = v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = 0.0f;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = a.g[j] + b.g[j];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = a.g[j] - b.g[j];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = a.g[j] * b.v + a.v * b.g[j];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    const float inv = 1.0f / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = (a.g[j] - r.v * b.g[j]) * inv;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(float s, const Dual<N>& a) {
    Dual<N> r;
    r.v = s * a.v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = s * a.g[j];
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dlog(const Dual<N>& a) {
    Dual<N> r;
    r.v = logf(a.v);
    const float inv = 1.0f / a.v;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = a.g[j] * inv;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<N> dsqrt(const Dual<N>& a) {
    Dual<N> r;
    r.v = sqrtf(a.v);
    // the derivative of safe_quadratic_root's sqrt, held at zero where the
    // discriminant is within FP32 rounding of zero (it is positive in exact
    // arithmetic, rq_spline_flow.jl:215-244)
    const float h = r.v > 1e-18f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int j = 0; j < N; ++j) r.g[j] = a.g[j] * h;
    return r;
}
// clamp to [0, 1]: outside the interval the value is constant
template <int N>
__device__ __forceinline__ Dual<N> dclamp01(const Dual<N>& a) {
    if (a.v < 0.0f) return dconst<N>(0.0f);
    if (a.v > 1.0f) return dconst<N>(1.0f);
    return a;
}

// ------------------------------------------------------------------- splines
template <int K>
struct Knots {
    float xp[K + 1], yp[K + 1], d[K + 1];
    float sw[K], sh[K];  // softmax of the raw widths / heights
    float sig[K + 1];        // derivative of each slope by its raw value
};

__device__ __forceinline__ float softplus(float t) { return t > 20.0f ? t : log1pf(expf(t)); }

// constrain_spline_params, rq_spline_flow.jl:170-206 (with _normalize_bin_sizes
// :127-136 and _normalize_knot_slopes :146-154)
template <int K>
__device__ __forceinline__ void constrain(const float* __restrict__ p, float r0, float r1, Knots<K>& kn) {
    const float span = (r1 - r0) - K * kMinBin;
    float mw = p[0], mh = p[K];
#pragma unroll
    for (int i = 1; i < K; ++i) {
        mw = fmaxf(mw, p[i]);
        mh = fmaxf(mh, p[K + i]);
    }
    float zw = 0.0f, zh = 0.0f;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        kn.sw[i] = expf(p[i] - mw);
        kn.sh[i] = expf(p[K + i] - mh);
        zw += kn.sw[i];
        zh += kn.sh[i];
    }
    const float izw = 1.0f / zw, izh = 1.0f / zh;
    float cx = r0, cy = r0;
    kn.xp[0] = r0;
    kn.yp[0] = r0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        kn.sw[i] *= izw;
        kn.sh[i] *= izh;
        cx += kMinBin + span * kn.sw[i];
        cy += kMinBin + span * kn.sh[i];
        kn.xp[i + 1] = cx;
        kn.yp[i + 1] = cy;
    }
    kn.xp[K] = r1;
    kn.yp[K] = r1;
    // The FP32 running sum can reach the pinned last knot when the last bins
    // are at the minimum width (11 roundings of up to half an ulp near r1
    // exceed kMinBin): keep the knots strictly increasing (the reference sums
    // in Float64, where this cannot happen)
#pragma unroll
    for (int i = K - 1; i >= 1; --i) {
        kn.xp[i] = fminf(kn.xp[i], nextafterf(kn.xp[i + 1], -INFINITY));
        kn.yp[i] = fminf(kn.yp[i], nextafterf(kn.yp[i + 1], -INFINITY));
    }
#pragma unroll
    for (int i = 0; i <= K; ++i) {
        const float t = p[2 * K + i] + kSlopeOffset;
        kn.d[i] = softplus(t) + kMinSlope;
        kn.sig[i] = 1.0f / (1.0f + expf(-t));
    }
}

// the bin k with yp[k] <= y < yp[k+1] (y strictly inside the range)
template <int K>
__device__ __forceinline__ int find_bin(const float* yp, float y) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < K; ++i) k += (y >= yp[i]) ? 1 : 0;
    return k;
}

// safe_quadratic_root, rq_spline_flow.jl:215-244
__device__ __forceinline__ Dual<7> quad_root(const Dual<7>& a, const Dual<7>& b, const Dual<7>& c) {
    const Dual<7> disc = b * b - 4.0f * (a * c);
    const Dual<7> sq = disc.v > 0.0f ? dsqrt(disc) : dconst<7>(0.0f);
    if (b.v >= 0.0f) return (2.0f * c) / (dconst<7>(0.0f) - b - sq);
    return (dconst<7>(0.0f) - b + sq) / (2.0f * a);
}

// Inverse spline on one bin (inv_rqs_univariate, rq_spline_flow.jl:358-381)
// with derivatives by u = (y, x0, w, y0, h, d0, d1).
__device__ __forceinline__ void inv_bin_dual(float yv, float x0v, float wv, float y0v, float hv, float d0v, float d1v,
                                             Dual<7>& x, Dual<7>& logdet) {
    using D = Dual<7>;
    const D y = dvar<7>(yv, 0), x0 = dvar<7>(x0v, 1), w = dvar<7>(wv, 2), y0 = dvar<7>(y0v, 3);
    const D h = dvar<7>(hv, 4), d0 = dvar<7>(d0v, 5), d1 = dvar<7>(d1v, 6);
    const D s = h / w;
    const D ww = dclamp01((y - y0) / h);
    const D st = d1 + d0 - 2.0f * s;
    const D c = dconst<7>(0.0f) - s * ww;
    const D b = d0 - st * ww;
    const D a = s - b;
    const D z = dclamp01(quad_root(a, b, c));
    x = w * z + x0;
    const D sq_z = z * z, z1mz = z - sq_z;
    const D omz = dconst<7>(1.0f) - z;
    const D den = s + st * z1mz;
    logdet = dconst<7>(0.0f) - 2.0f * dlog(s) - dlog(d1 * sq_z + 2.0f * (s * z1mz) + d0 * (omz * omz)) +
             2.0f * dlog(den);
}

__device__ __forceinline__ void inv_bin(float y, float x0, float w, float y0, float h, float d0, float d1, float& x,
                                        float& logdet) {
    const float s = h / w;
    const float ww = fminf(fmaxf((y - y0) / h, 0.0f), 1.0f);
    const float st = d1 + d0 - 2.0f * s;
    const float c = -s * ww, b = d0 - st * ww, a = s - b;
    const float disc = b * b - 4.0f * a * c;
    const float sq = disc > 0.0f ? sqrtf(disc) : 0.0f;
    float z = b >= 0.0f ? (2.0f * c) / (-b - sq) : (-b + sq) / (2.0f * a);
    z = fminf(fmaxf(z, 0.0f), 1.0f);
    x = w * z + x0;
    const float z1mz = z - z * z, omz = 1.0f - z;
    const float den = s + st * z1mz;
    logdet = -2.0f * logf(s) - logf(d1 * z * z + 2.0f * s * z1mz + d0 * omz * omz) + 2.0f * logf(den);
}

// inv_rqs_univariate on constrained knots: x and the log-determinant
template <int K>
__device__ __forceinline__ void inv_spline(const float* xp, const float* yp, const float* d, float y, float& x,
                                           float& logdet) {
    if (y <= yp[0]) {
        x = (y - yp[0]) / d[0] + xp[0];
        logdet = -logf(d[0]);
    } else if (y >= yp[K]) {
        x = (y - yp[K]) / d[K] + xp[K];
        logdet = -logf(d[K]);
    } else {
        const int k = find_bin<K>(yp, y);
        inv_bin(y, xp[k], xp[k + 1] - xp[k], yp[k], yp[k + 1] - yp[k], d[k], d[k + 1], x, logdet);
    }
}

// The same inverse for inference: hardware reciprocal / logarithm
// (__fdividef, __logf, relative error ~1e-6) and the three logarithms of the
// log-determinant folded into one, log(den^2 / (s^2 q)).
__device__ __forceinline__ void inv_bin_fast(float y, float x0, float w, float y0, float h, float d0, float d1,
                                             float& x, float& logdet) {
    const float s = __fdividef(h, w);
    const float ww = fminf(fmaxf(__fdividef(y - y0, h), 0.0f), 1.0f);
    const float st = d1 + d0 - 2.0f * s;
    const float c = -s * ww, b = d0 - st * ww, a = s - b;
    const float disc = b * b - 4.0f * a * c;
    const float sq = disc > 0.0f ? sqrtf(disc) : 0.0f;
    float z = b >= 0.0f ? __fdividef(2.0f * c, -b - sq) : __fdividef(-b + sq, 2.0f * a);
    z = fminf(fmaxf(z, 0.0f), 1.0f);
    x = w * z + x0;
    const float z1mz = z - z * z, omz = 1.0f - z;
    const float den = s + st * z1mz;
    const float q = d1 * z * z + 2.0f * s * z1mz + d0 * omz * omz;
    logdet = __logf(__fdividef(den * den, s * s * q));
}

template <int K>
__device__ __forceinline__ void inv_spline_fast(const float* xp, const float* yp, const float* d, float y, float& x,
                                                float& logdet) {
    if (y <= yp[0]) {
        x = __fdividef(y - yp[0], d[0]) + xp[0];
        logdet = -__logf(d[0]);
    } else if (y >= yp[K]) {
        x = __fdividef(y - yp[K], d[K]) + xp[K];
        logdet = -__logf(d[K]);
    } else {
        const int k = find_bin<K>(yp, y);
        inv_bin_fast(y, xp[k], xp[k + 1] - xp[k], yp[k], yp[k + 1] - yp[k], d[k], d[k + 1], x, logdet);
    }
}

// FP32 range guards of the head (the reference computes in Float64): the log
// expectation is used within [-30, 30] (expected counts 1e-13 to 1e13) and
// the raw scale within [-20, 20] (scale >= 2e-7 ns); outside, the value is
// held and the gradient is zero
// the standardised residual of the base normal is held within +-1e6 (a
// log-density below -5e11) so that the loss and its gradient stay finite
constexpr float kMaxU = 1e6f;
__device__ __forceinline__ float clamp_le(float x) { return fminf(fmaxf(x, -30.0f), 30.0f); }
__device__ __forceinline__ float clamp_scale(float x) { return fminf(fmaxf(x, -20.0f), 20.0f); }

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    return x;
}

// ------------------------------------------------------------------- kernels
// Input column j of a condition row f[0..4] (the normalised features: log
// distance over 1-200 m, cos theta of the source direction, cos theta of the
// PMT axis, azimuth, log10 E).  With derived columns (input mode
// NTP_FLOW_INPUT_DERIVED) four more follow, functions of the features that a
// count model otherwise has to build from them: the distance in units of
// 100 m, the source direction's cosine offset from the Cherenkov cosine
// 1 / 1.35 and its square, and sin(theta_pmt) cos(phi).
__device__ __forceinline__ float input_column(const float* __restrict__ f, int j, int mode) {
    if (j < kCond) return f[j];
    if (mode != NTP_FLOW_INPUT_DERIVED || j >= kCond + kDerived) return 0.0f;
    switch (j - kCond) {
    case 0: return expf((f[0] + 1.0f) * kHalfLog200) * 0.01f;
    case 1: return f[1] + kCherenkovCos;
    case 2: { const float c = f[1] + kCherenkovCos; return c * c; }
    default: return sqrtf(fmaxf(1.0f - f[2] * f[2], 0.0f)) * cosf(kPi * (f[3] + 1.0f));
    }
}

// cond [n x 5] FP32 -> X [n x 64] BF16 (zero padded) and X^T [64 x n];
// rows >= n_valid are zero.  Thread (b, g) writes columns 8g .. 8g + 7 of
// row b, with b fastest across threads: the transposed stores of a warp are
// contiguous, the row stores one 16-byte vector each.
__global__ void pack_kernel(const float* __restrict__ cond, int n_valid, int n, int mode,
                            __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ xt) {
    // programmatic dependent launch: reads follow the previous kernel
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * (kIn / 8)) return;
    const int b = i % n, g = i / n;
    const float* f = cond + static_cast<size_t>(b) * kCond;
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int j = 8 * g + 2 * e;
        const __nv_bfloat162 h = __floats2bfloat162_rn(b < n_valid ? input_column(f, j, mode) : 0.0f,
                                                       b < n_valid ? input_column(f, j + 1, mode) : 0.0f);
        w[e] = *reinterpret_cast<const uint32_t*>(&h);
        xt[static_cast<size_t>(j) * n + b] = h.x;
        xt[static_cast<size_t>(j + 1) * n + b] = h.y;
    }
    *reinterpret_cast<uint4*>(x + static_cast<size_t>(b) * kIn + 8 * g) = make_uint4(w[0], w[1], w[2], w[3]);
}

// Shared-memory layout of the head kernel for L layers of K bins and a
// block of 32 samples (one warp per layer), in floats.
__host__ __device__ constexpr int head_smem_floats(int L, int K, int ldp) {
    return L * 32 * (3 * (K + 1) + 2 * K + (K + 1))  // knots x, y, slope; softmax widths, heights; slope derivative
           + L * 32 * 2                               // layer input y, bin (or tail) index
           + L * 32 * 14                              // dx/du, dlogdet/du for u = (y, x0, w, y0, h, d0, d1)
           + L * 32 * 7                               // adjoint dL/du
           + 32 * 4                                   // per sample: dL/dx innermost, shift, scale, log expectation
           + L * 32 + 32                              // per layer and sample: squared gradient norm; clip factor
           + 32 * (ldp + 2) / 2                       // the block's rows of dL/dP in BF16 (padded stride)
           + 32 * (ldp + 1);                          // the block's rows of P (padded stride)
}

// Loss and gradient of the head.  P [B x ldp] FP32.  A block takes 32
// samples; warp w handles spline layer w of all of them where the work is
// independent across layers, warp 0 runs the two short chains through the
// layers:
//   P1 (all warps)  constrain_spline_params of the warp's layer -> shared memory
//   P2 (warp 0)     inverse splines, layer L-1 first: each layer's input y and
//                   bin; base normal; Poisson count term; loss
//   P3 (all warps)  the in-bin inverse spline of the warp's layer as dual numbers:
//                   d x / d u and d logdet / d u (linear tails in closed form)
//   P4 (warp 0)     reverse chain: dL/du of every layer from dL/dx of the innermost
//   P5 (all warps)  dL/du -> dL/draw through softmax / cumulative sum / softplus;
//                   the sample's row of dL/dP scaled to an L2 norm of at most
//                   clip / B; warp 0 adds shift, scale, log expectation and
//                   the padding
// The block's 32 rows of P are first copied to shared memory with coalesced
// 16-byte loads (a row stride of ldp + 1 words keeps each lane's reads of
// its own row in its own bank).
// Outputs: dL/dP as BF16 row-major dp [B x ldp] (rows staged in shared memory)
// and transposed dpt [ldp x B]; optionally FP32 row-major gf; the output
// layer's bias gradient into gbias (per warp a transpose-reduce of 32 columns
// and one atomic per column); the batch-mean loss into *loss.
template <int K>
__global__ void __launch_bounds__(32 * kMaxLayers) head_grad_kernel(
    const float* __restrict__ P, int ldp, int L, const float* __restrict__ y, const float* __restrict__ nhits,
    const int* __restrict__ has_y, int B, float r0, float r1, float clip, float count_w,
    const float* __restrict__ count_w_rows, __nv_bfloat16* __restrict__ dp,
    __nv_bfloat16* __restrict__ dpt, float* __restrict__ gf, float* __restrict__ gbias, double* __restrict__ loss) {
    constexpr int NP = 3 * K + 1, NK = K + 1, KN = 3 * NK + 2 * K + NK;
    extern __shared__ float sm[];
    // programmatic dependent launch: reads follow the previous kernel; the
    // next kernel's blocks may take SMs as this kernel's blocks finish
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = L * 32;
    float* s_kn = sm;                          // [L][32][KN]
    float* s_y = s_kn + S * KN;                // [L][32]
    int* s_bin = reinterpret_cast<int*>(s_y + S);  // [L][32]: bin, -1 low tail, K high tail
    float* s_d = s_y + 2 * S;                  // [L][32][14]
    float* s_g = s_d + S * 14;                 // [L][32][7]
    float* s_s = s_g + S * 7;                  // [32][4]
    float* s_n2 = s_s + 32 * 4;                // [L][32]
    float* s_f = s_n2 + S;                     // [32]
    // [32][ldp + 2]: the row stride of 97 words puts the lanes' stores to one
    // column in 32 different banks
    const int lds = ldp + 2;
    uint16_t* s_dp = reinterpret_cast<uint16_t*>(s_f + 32);
    const int ldsp = ldp + 1;
    float* s_p = reinterpret_cast<float*>(s_dp) + 16 * lds;  // [32][ldp + 1]
    const int b = blockIdx.x * 32 + lane;
    const bool act = b < B;
    // the sample's inputs, loaded before the rows of P arrive (warp 0's
    // chains use the time, the hit count and the count weight)
    const bool timed = act && has_y[b];
    const float y_b = (warp == 0 && timed) ? y[b] : 0.0f;
    const float n_b = (warp == 0 && act) ? nhits[b] : 0.0f;
    const float cwr_b = (warp == 0 && act && count_w_rows) ? count_w_rows[b] : 1.0f;
    // warp w copies rows w, w + L, ..., four rows at a time (all loads in
    // flight before the stores); lane c the row's 16-byte columns c, c + 32
    // (ldp <= 256: at most two per lane)
    for (int r0 = warp; r0 < 32; r0 += 4 * L) {
        float4 v[4][2];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = r0 + u * L, rb = blockIdx.x * 32 + r;
            const float4* src = reinterpret_cast<const float4*>(P + static_cast<size_t>(rb) * ldp);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                v[u][h] = (r < 32 && rb < B && c < ldp / 4) ? __ldg(src + c) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int r = r0 + u * L;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = lane + 32 * h;
                if (r < 32 && c < ldp / 4) {
                    float* d = s_p + r * ldsp + 4 * c;
                    d[0] = v[u][h].x;
                    d[1] = v[u][h].y;
                    d[2] = v[u][h].z;
                    d[3] = v[u][h].w;
                }
            }
        }
    }
    __syncthreads();
    const float* p = s_p + lane * ldsp;
    const int li = warp;
    const int slot = li * 32 + lane;
    const int o_shift = L * NP, o_scale = o_shift + 1, o_le = o_shift + 2;
    const float inv_b = 1.0f / static_cast<float>(B);
    float l_loss = 0.0f;  // warp 0: the sample's loss, summed at the end

    // P1
    {
        Knots<K> kn;
        constrain<K>(p + li * NP, r0, r1, kn);
        float* q = s_kn + slot * KN;
#pragma unroll
        for (int i = 0; i < NK; ++i) {
            q[i] = kn.xp[i];
            q[NK + i] = kn.yp[i];
            q[2 * NK + i] = kn.d[i];
            q[3 * NK + 2 * K + i] = kn.sig[i];
        }
#pragma unroll
        for (int i = 0; i < K; ++i) {
            q[3 * NK + i] = kn.sw[i];
            q[3 * NK + K + i] = kn.sh[i];
        }
    }
    __syncthreads();
    // P2
    if (warp == 0) {
        float l = 0.0f;
        const float le_raw = p[o_le], n = n_b;
        const float le = clamp_le(le_raw);
        const float lam = expf(le);
        const float cw = act ? (count_w_rows ? count_w * cwr_b : count_w) : 0.0f;
        if (act && cw != 0.0f) l -= cw * (n * le - lam - lgammaf(n + 1.0f));
        float a = 0.0f, g_shift = 0.0f, g_scale = 0.0f;
        if (timed) {
            float cur = y_b, ldsum = 0.0f;
            for (int k = L - 1; k >= 0; --k) {
                const float* q = s_kn + (k * 32 + lane) * KN;
                s_y[k * 32 + lane] = cur;
                s_bin[k * 32 + lane] = cur <= q[NK] ? -1 : (cur >= q[NK + K] ? K : find_bin<K>(q + NK, cur));
                // the chain with the hardware reciprocal and logarithm
                // (relative error ~1e-6; the gradient's dual numbers below
                // are exact to FP32)
                float x, ld;
                inv_spline_fast<K>(q, q + NK, q + 2 * NK, cur, x, ld);
                cur = x;
                ldsum += ld;
            }
            const float rs = p[o_scale];
            const float sg = 1.0f / (1.0f + expf(-clamp_scale(rs)));
            const float scale = 100.0f * sg;
            const float u_raw = (cur - p[o_shift]) / scale;
            const float u = fminf(fmaxf(u_raw, -kMaxU), kMaxU);
            l -= -logf(scale) - 0.5f * (kLog2Pi + u * u) + ldsum;
            a = u / scale * inv_b;
            g_shift = -u / scale * inv_b;
            g_scale = rs == clamp_scale(rs) ? (1.0f - u * u) / scale * 100.0f * sg * (1.0f - sg) * inv_b : 0.0f;
        }
        s_s[lane * 4 + 0] = a;
        s_s[lane * 4 + 1] = g_shift;
        s_s[lane * 4 + 2] = g_scale;
        s_s[lane * 4 + 3] = act && le_raw == le ? cw * (lam - n) * inv_b : 0.0f;
        l_loss = l;
    }
    __syncthreads();
    // P3
    if (timed) {
        const float* q = s_kn + slot * KN;
        const float yv = s_y[slot];
        const int k = s_bin[slot];
        float* d = s_d + slot * 14;
#pragma unroll
        for (int j = 0; j < 14; ++j) d[j] = 0.0f;
        if (k < 0 || k >= K) {  // x = (y - e)/d_e + e, logdet = -log d_e
            const int e = k < 0 ? 0 : K;
            const float de = q[2 * NK + e];
            d[0] = 1.0f / de;                           // dx/dy
            d[5] = -(yv - q[NK + e]) / (de * de);       // dx/dd_e
            d[7 + 5] = -1.0f / de;                      // dlogdet/dd_e
        } else {
            Dual<7> x, ld;
            inv_bin_dual(yv, q[k], q[k + 1] - q[k], q[NK + k], q[NK + k + 1] - q[NK + k], q[2 * NK + k],
                         q[2 * NK + k + 1], x, ld);
#pragma unroll
            for (int j = 0; j < 7; ++j) {
                d[j] = x.g[j];
                d[7 + j] = ld.g[j];
            }
        }
    }
    __syncthreads();
    // P4
    if (warp == 0 && timed) {
        float a = s_s[lane * 4];
        for (int k = 0; k < L; ++k) {
            const float* d = s_d + (k * 32 + lane) * 14;
            float* g = s_g + (k * 32 + lane) * 7;
#pragma unroll
            for (int j = 0; j < 7; ++j) g[j] = a * d[j] - inv_b * d[7 + j];
            a = g[0];
        }
    }
    __syncthreads();
    // P5
    // stores of column col (not its bias-gradient sum)
    auto store_col = [&](int col, float v) {
        if (act) {
            s_dp[lane * lds + col] = __bfloat16_as_ushort(__float2bfloat16(v));
            dpt[static_cast<size_t>(col) * B + b] = __float2bfloat16(v);
            if (gf) gf[static_cast<size_t>(b) * ldp + col] = v;
        }
    };
    // the bias gradient of column col: the warp's sum, one atomic
    auto sum_col = [&](int col, float v) {
        const float sum = warp_sum(act ? v : 0.0f);
        if (lane == 0 && sum != 0.0f) atomicAdd(gbias + col, sum);
    };
    float g[NP];
    {
#pragma unroll
        for (int i = 0; i < NP; ++i) g[i] = 0.0f;
        if (timed) {
            const float* q = s_kn + slot * KN;
            const float* gu = s_g + slot * 7;
            const int k = s_bin[slot];
            const float* sig = q + 3 * NK + 2 * K;
            if (k < 0 || k >= K) {
                const int e = k < 0 ? 0 : K;
                g[2 * K + e] = gu[5] * sig[e];
            } else {
                // x0 = r0 + sum_{i<k} wd_i, w = wd_k with wd = kMinBin + span * softmax(raw);
                // the last knot pinned to r1 equals the cumulative sum exactly
                const float span = (r1 - r0) - K * kMinBin;
                const float* sw = q + 3 * NK;
                const float* sh = sw + K;
                float dot_w = 0.0f, dot_h = 0.0f;
#pragma unroll
                for (int i = 0; i < K; ++i) {
                    dot_w += sw[i] * (i < k ? gu[1] : (i == k ? gu[2] : 0.0f));
                    dot_h += sh[i] * (i < k ? gu[3] : (i == k ? gu[4] : 0.0f));
                }
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    g[j] = span * sw[j] * ((j < k ? gu[1] : (j == k ? gu[2] : 0.0f)) - dot_w);
                    g[K + j] = span * sh[j] * ((j < k ? gu[3] : (j == k ? gu[4] : 0.0f)) - dot_h);
                }
#pragma unroll
                for (int j = 0; j <= K; ++j)
                    g[2 * K + j] = ((j == k ? gu[5] : 0.0f) + (j == k + 1 ? gu[6] : 0.0f)) * sig[j];
            }
        }
    }
    // per-sample clip of dL/dP to an L2 norm of clip / B: one extreme sample
    // cannot overflow the FP32 / BF16 backward GEMMs
    {
        float n2 = 0.0f;
#pragma unroll
        for (int i = 0; i < NP; ++i) n2 += g[i] * g[i];
        s_n2[slot] = n2;
    }
    __syncthreads();
    if (warp == 0) {
        float n2 = s_s[lane * 4 + 1] * s_s[lane * 4 + 1] + s_s[lane * 4 + 2] * s_s[lane * 4 + 2] +
                   s_s[lane * 4 + 3] * s_s[lane * 4 + 3];
        for (int k = 0; k < L; ++k) n2 += s_n2[k * 32 + lane];
        const float lim = clip * inv_b;
        s_f[lane] = (clip > 0.0f && n2 > lim * lim) ? lim * rsqrtf(n2) : 1.0f;
    }
    __syncthreads();
    const float fs = s_f[lane];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        g[i] *= fs;
        store_col(li * NP + i, g[i]);
    }
    if (gbias) {
        // the layer's first 32 columns by a transpose-reduce (after the five
        // halving steps lane l holds the warp's sum of column l; 31 shuffles
        // and one atomic instruction instead of 32 warp sums), the rest by
        // warp sums
        float v[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) v[k] = (act && k < NP) ? g[k < NP ? k : 0] : 0.0f;
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
        if (lane < NP && v[0] != 0.0f) atomicAdd(gbias + li * NP + lane, v[0]);
#pragma unroll
        for (int i = 32; i < NP; ++i) sum_col(li * NP + i, g[i]);
    }
    if (warp == 0) {
        const float tail[3] = {s_s[lane * 4 + 1] * fs, s_s[lane * 4 + 2] * fs, s_s[lane * 4 + 3] * fs};
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            store_col(o_shift + e, tail[e]);
            if (gbias) sum_col(o_shift + e, tail[e]);
        }
        if (act)
            for (int col = o_le + 1; col < ldp; ++col) {
                s_dp[lane * lds + col] = 0;
                dpt[static_cast<size_t>(col) * B + b] = __float2bfloat16(0.0f);
                if (gf) gf[static_cast<size_t>(b) * ldp + col] = 0.0f;
            }
    }
    __syncthreads();
    // the block's rows of dp: 32 rows of ldp BF16 values, 4 bytes at a time
    // (warp w rows w, w + L, ...; lane c words c, c + 32, ...)
    for (int r = warp; r < 32; r += L) {
        const int rb = blockIdx.x * 32 + r;
        if (rb >= B) break;
        uint32_t* dst = reinterpret_cast<uint32_t*>(dp + static_cast<size_t>(rb) * ldp);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(s_dp + r * lds);
#pragma unroll 3
        for (int c = lane; c < ldp / 2; c += 32) dst[c] = src[c];
    }
    // the batch-mean loss, off the path of the gradient phases
    if (warp == 0) {
        const float l = warp_sum(l_loss);
        if (lane == 0 && l != 0.0f) atomicAdd(loss, static_cast<double>(l) / B);
    }
}

// Sets *flag if any of the n gradient values is not finite.
__global__ void nonfinite_kernel(const float* __restrict__ g, long long n, int* __restrict__ flag) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    bool bad = false;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        bad |= !isfinite(g[i]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicExch(flag, 1);
}

// The parameter blocks of the flat vector: offsets (blocks + 1 entries) and,
// for weight matrices, the BF16 copy and its transpose [cols x rows].
struct ParamBlocks {
    int n;
    long long off[9];
    int rows[8], cols[8];
    __nv_bfloat16* wb[8];
    __nv_bfloat16* wt[8];
};

// Adam (Flux's: bias-corrected moments) over the whole flat FP32 vector in
// one launch; refreshes the BF16 weight copies and their transposes.  The
// step size and the step count are read from device memory, so a captured
// training step replays with the current values.  step_dev[0] is the step
// count, step_dev[1] the blocks finished: the last block to finish counts
// the step, after every block has read the count.
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, const ParamBlocks pb, const float* __restrict__ lr_dev,
                            float b1, float b2, float eps, int* __restrict__ step_dev,
                            const int* __restrict__ skip) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (*skip) return;  // a non-finite gradient: the step is skipped (and not counted)
    const float t = static_cast<float>(*reinterpret_cast<volatile int*>(step_dev) + 1);
    const float c1 = 1.0f - powf(b1, t), c2 = 1.0f - powf(b2, t);
    const float lr = *lr_dev;
    const long long total = pb.off[pb.n];
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        int k = 0;
        while (k + 1 < pb.n && i >= pb.off[k + 1]) ++k;
        if (pb.wb[k]) {
            const long long j = i - pb.off[k];
            const __nv_bfloat16 h = __float2bfloat16(wi);
            pb.wb[k][j] = h;
            pb.wt[k][(j % pb.cols[k]) * pb.rows[k] + j / pb.cols[k]] = h;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(step_dev + 1, 1) == static_cast<int>(gridDim.x) - 1) {
            step_dev[1] = 0;
            atomicAdd(step_dev, 1);
        }
    }
}

// The batch sources of a multi-step call whose rows are on the device, read
// by the step's kernels from device memory so that one captured step serves
// every batch: step i reads rows [i B, (i + 1) B); the step's last kernel
// records its loss and skip flag and advances i.
struct StepIO {
    const float* cond;
    const float* tres;
    const float* nhits;
    const int* has_time;
    const float* count_w;  // may be null
    double* loss_hist;
    int* skip_hist;
    int step;
};

// the step's rows into the staging buffers the step's kernels read
__global__ void stage_kernel(const StepIO* __restrict__ io, int B, float* __restrict__ cond, float* __restrict__ y,
                             float* __restrict__ nh, int* __restrict__ hy, float* __restrict__ cw) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const long long o = static_cast<long long>(io->step) * B;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * kCond; i += stride) cond[i] = io->cond[o * kCond + i];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += stride) {
        y[i] = io->tres[o + i];
        nh[i] = io->nhits[o + i];
        hy[i] = io->has_time[o + i];
        if (io->count_w) cw[i] = io->count_w[o + i];
    }
}

// the step's loss (and skip flag) into the call's history; the next step
// reads the next rows
__global__ void step_end_kernel(StepIO* __restrict__ io, const double* __restrict__ loss,
                                const int* __restrict__ skip, int update) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    io->loss_hist[io->step] = *loss;
    if (update) io->skip_hist[io->step] = *skip;
    io->step += 1;
}

__global__ void to_bf16_kernel(const float* __restrict__ w, int n, int cols, int rows,
                               __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    wb[i] = __float2bfloat16(w[i]);
    wt[static_cast<size_t>(i % cols) * rows + i / cols] = __float2bfloat16(w[i]);
}

// Per condition: the constrained knots of every layer, then shift, scale and
// log expectation.  Row of knot_row(L, K) floats.
template <int K>
__global__ void knots_kernel(const float* __restrict__ P, int ldp, int L, int n, float r0, float r1,
                             float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float* p = P + static_cast<size_t>(c) * ldp;
    float* o = out + static_cast<size_t>(c) * knot_row(L, K);
    for (int li = 0; li < L; ++li) {
        Knots<K> kn;
        constrain<K>(p + li * (3 * K + 1), r0, r1, kn);
        float* q = o + li * (3 * (K + 1));
        for (int i = 0; i <= K; ++i) {
            q[i] = kn.xp[i];
            q[K + 1 + i] = kn.yp[i];
            q[2 * (K + 1) + i] = kn.d[i];
        }
    }
    o[L * (3 * (K + 1))] = p[L * (3 * K + 1)];
    o[L * (3 * (K + 1)) + 1] = 100.0f / (1.0f + expf(-clamp_scale(p[L * (3 * K + 1) + 1])));
    o[L * (3 * (K + 1)) + 2] = clamp_le(p[L * (3 * K + 1) + 2]);
}

// The log expectation column of the conditioner's raw outputs, with the
// knot tables' clamp (the count-only query: no spline knots are built).
__global__ void log_expec_kernel(const float* __restrict__ P, int ldp, int col, int n, float* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r] = clamp_le(P[static_cast<size_t>(r) * ldp + col]);
}

// log p(t | condition) for (condition index, time) tuples
template <int K>
__global__ void logpdf_kernel(const float* __restrict__ knots, int L, int n_cond, const int* __restrict__ cidx,
                              const float* __restrict__ t, unsigned long long n, float* __restrict__ out) {
    const int row = knot_row(L, K);
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        const int c = __ldg(cidx + i);
        if (c < 0 || c >= n_cond) {
            out[i] = __int_as_float(0x7fc00000);  // NaN for an index outside the conditions
            continue;
        }
        const float* o = knots + static_cast<size_t>(c) * row;
        float cur = __ldg(t + i), ldsum = 0.0f;
        for (int li = L - 1; li >= 0; --li) {
            const float* xp = o + li * (3 * (K + 1));
            float x, ld;
            inv_spline_fast<K>(xp, xp + K + 1, xp + 2 * (K + 1), cur, x, ld);
            cur = x;
            ldsum += ld;
        }
        const float scale = o[L * (3 * (K + 1)) + 1];
        const float u = (cur - o[L * (3 * (K + 1))]) * __fdividef(1.0f, scale);
        out[i] = -__logf(scale) - 0.5f * (kLog2Pi + u * u) + ldsum;
    }
}

// log p(t_j | condition c) on a time grid shared by all conditions: out[c *
// n_times + j].  One block per condition (grid-stride), its knot row staged in
// shared memory; the threads sweep the grid.
template <int K>
__global__ void logpdf_grid_kernel(const float* __restrict__ knots, int L, int n_cond,
                                   const float* __restrict__ times, int n_times, float* __restrict__ out) {
    extern __shared__ float s_row[];
    const int row = knot_row(L, K);
    for (int c = blockIdx.x; c < n_cond; c += gridDim.x) {
        __syncthreads();
        for (int i = threadIdx.x; i < row; i += blockDim.x) s_row[i] = knots[static_cast<size_t>(c) * row + i];
        __syncthreads();
        const float shift = s_row[L * 3 * (K + 1)], scale = s_row[L * 3 * (K + 1) + 1];
        const float inv_scale = __fdividef(1.0f, scale), log_scale = __logf(scale);
        for (int j = threadIdx.x; j < n_times; j += blockDim.x) {
            float cur = __ldg(times + j), ldsum = 0.0f;
            for (int li = L - 1; li >= 0; --li) {
                const float* xp = s_row + li * 3 * (K + 1);
                float x, ld;
                inv_spline_fast<K>(xp, xp + K + 1, xp + 2 * (K + 1), cur, x, ld);
                cur = x;
                ldsum += ld;
            }
            const float u = (cur - shift) * inv_scale;
            out[static_cast<size_t>(c) * n_times + j] = -log_scale - 0.5f * (kLog2Pi + u * u) + ldsum;
        }
    }
}

// sum of the mixture weights: w[c], or exp(log expectation) of the knot rows
// when w is NULL; one block
__global__ void mixture_total_kernel(const float* __restrict__ knots, int L, int K, int n_cond,
                                     const float* __restrict__ w, double* __restrict__ total) {
    __shared__ double part[32];
    double acc = 0.0;
    for (int c = threadIdx.x; c < n_cond; c += blockDim.x)
        acc += w ? static_cast<double>(w[c])
                 : exp(static_cast<double>(knots[static_cast<size_t>(c) * knot_row(L, K) + L * 3 * (K + 1) + 2]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) *total = acc;
    }
}

// The pooled CDF of a mixture of conditions at times t_j:
//   F(t_j) = sum_c w_c Phi(u_c(t_j - off_c)) / sum_c w_c,
// Phi of the base-normal residual being each condition's CDF (the splines
// and the affine map are increasing bijections).  A block takes blockDim.x
// consecutive times, one per thread, and walks the conditions in tiles whose
// knot rows (and weights, offsets) are staged in shared memory.
constexpr int kMixTile = 32;
template <int K>
__global__ void mixture_cdf_kernel(const float* __restrict__ knots, int L, int n_cond, const float* __restrict__ w,
                                   const float* __restrict__ off, const float* __restrict__ t, unsigned long long n,
                                   const double* __restrict__ total, double* __restrict__ out) {
    extern __shared__ float s_tile[];
    const int row = knot_row(L, K);
    float* s_w = s_tile + kMixTile * row;
    float* s_off = s_w + kMixTile;
    const unsigned long long j = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    const float tj = j < n ? __ldg(t + j) : 0.0f;
    double acc = 0.0;
    for (int c0 = 0; c0 < n_cond; c0 += kMixTile) {
        const int m = min(kMixTile, n_cond - c0);
        __syncthreads();
        for (int i = threadIdx.x; i < m * row; i += blockDim.x) s_tile[i] = knots[static_cast<size_t>(c0) * row + i];
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const float le = knots[static_cast<size_t>(c0 + i) * row + L * 3 * (K + 1) + 2];
            s_w[i] = w ? w[c0 + i] : expf(le);
            s_off[i] = off ? off[c0 + i] : 0.0f;
        }
        __syncthreads();
        if (j < n) {
            for (int c = 0; c < m; ++c) {
                const float* o = s_tile + c * row;
                float cur = tj - s_off[c];
                for (int li = L - 1; li >= 0; --li) {
                    const float* xp = o + li * 3 * (K + 1);
                    float x, ld;
                    inv_spline_fast<K>(xp, xp + K + 1, xp + 2 * (K + 1), cur, x, ld);
                    cur = x;
                }
                const float u = (cur - o[L * 3 * (K + 1)]) * __fdividef(1.0f, o[L * 3 * (K + 1) + 1]);
                acc += static_cast<double>(s_w[c]) * static_cast<double>(normcdff(u));
            }
        }
    }
    if (j < n) {
        const double tot = *total;
        out[j] = tot > 0.0 ? acc / tot : 0.0;
    }
}

// ------------------------------------------------------------ sampling
// rqs_univariate (rq_spline_flow.jl:262-324) on constrained knots: the
// forward spline, linear outside the range
template <int K>
__device__ __forceinline__ float fwd_spline(const float* xp, const float* yp, const float* d, float x) {
    if (x <= xp[0]) return (x - xp[0]) * d[0] + yp[0];
    if (x >= xp[K]) return (x - xp[K]) * d[K] + yp[K];
    const int k = find_bin<K>(xp, x);
    const float w = xp[k + 1] - xp[k], h = yp[k + 1] - yp[k], s = h / w;
    const float z = fminf(fmaxf((x - xp[k]) / w, 0.0f), 1.0f);
    const float z1mz = z - z * z;
    const float num = h * (s * z * z + d[k] * z1mz);
    const float den = s + (d[k + 1] + d[k] - 2.0f * s) * z1mz;
    return yp[k] + num / den;
}

constexpr uint32_t kDrawSample = 0x534D504Cu;  // "SMPL": time draws of the surrogate

// Expected count exp(log expectation) -> Poisson count per condition, from the
// stream of the condition's 64-bit key.
__global__ void sample_count_kernel(const float* __restrict__ knots, int L, int K, int n,
                                    const unsigned long long* __restrict__ ckey, uint2 key,
                                    unsigned long long* __restrict__ counts) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const float le = knots[static_cast<size_t>(c) * knot_row(L, K) + L * 3 * (K + 1) + 2];
    const unsigned long long k = ckey[c];
    counts[c] = static_cast<unsigned long long>(
        poisson_draw(exp(static_cast<double>(le)), key, static_cast<uint32_t>(k), static_cast<uint32_t>(k >> 32)));
}

// Exclusive scan of n counts: per block of 1024 an in-block scan, the block
// totals scanned by one block, then added (n <= 1024 * 1024).
__global__ void scan_block_kernel(const unsigned long long* __restrict__ in, int n,
                                  unsigned long long* __restrict__ out, unsigned long long* __restrict__ block_sum) {
    __shared__ unsigned long long s[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const unsigned long long v = i < n ? in[i] : 0ull;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const unsigned long long t = threadIdx.x >= off ? s[threadIdx.x - off] : 0ull;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == 1023) block_sum[blockIdx.x] = s[1023];
}

__global__ void scan_add_kernel(unsigned long long* __restrict__ out, int n, const unsigned long long* __restrict__ block_off,
                                unsigned long long* __restrict__ total, int n_blocks) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += block_off[blockIdx.x];
    if (i == 0) *total = block_off[n_blocks];
}

// One thread per drawn hit: its condition by binary search on the offsets,
// x ~ Normal(shift, scale) (Box-Muller on the stream of the condition's key
// and the draw index), then the forward splines of layers 0 .. L-1.
template <int K>
__global__ void sample_draw_kernel(const float* __restrict__ knots, int L, int n,
                                   const unsigned long long* __restrict__ ckey, uint2 key,
                                   const unsigned long long* __restrict__ offsets, unsigned long long total,
                                   int32_t* __restrict__ hit_cond, float* __restrict__ hit_time) {
    const int row = knot_row(L, K);
    for (unsigned long long h = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; h < total;
         h += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        int lo = 0, hi = n - 1;  // last condition with offsets[c] <= h
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (offsets[mid] <= h) lo = mid;
            else hi = mid - 1;
        }
        const int c = lo;
        const unsigned long long j = h - offsets[c];
        const unsigned long long k = ckey[c];
        const uint4 r = philox4x32_10(make_uint4(kDrawSample ^ static_cast<uint32_t>(j >> 32), static_cast<uint32_t>(j),
                                                 static_cast<uint32_t>(k), static_cast<uint32_t>(k >> 32)),
                                      key);
        const float u1 = u01(r.x), u2 = u01(r.y);
        const float z = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
        const float* o = knots + static_cast<size_t>(c) * row;
        float y = o[L * 3 * (K + 1)] + o[L * 3 * (K + 1) + 1] * z;
        for (int li = 0; li < L; ++li) {
            const float* xp = o + li * 3 * (K + 1);
            y = fwd_spline<K>(xp, xp + K + 1, xp + 2 * (K + 1), y);
        }
        hit_cond[h] = c;
        hit_time[h] = y;
    }
}

int blocks_for(long long n, int t = 256) { return static_cast<int>((n + t - 1) / t); }

}  // namespace
}  // namespace ntp

// ======================================================================= host
namespace {

using bf16 = __nv_bfloat16;

struct Block {  // one parameter block of the flat FP32 vector
    int rows, cols;
    size_t off;
};

}  // namespace

struct ntp_flow {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // weight-gradient GEMMs, alongside the activation-gradient chain
    cudaEvent_t ev[5] = {};
    int cap = 0;  // batch capacity (multiple of 128)
    int L = 1, K = 12, n_out = 0, n_pad = 0;
    int in_mode = NTP_FLOW_INPUT_FEATURES;  // input columns: the features, or with the derived ones
    float r0 = -20.0f, r1 = 1500.0f;
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float clip = 1e3f;  // per-sample bound on |dL/dP| times the batch size (0 = none)
    float count_w = 1.0f;  // weight of the Poisson count term (1 = log_likelihood_with_poisson)
    long long step = 0;
    std::string err;
    Block blk[8];  // W1 b1 W2 b2 W3 b3 W4 b4
    size_t n_params = 0;
    float *theta = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    bf16 *wb[4] = {}, *wt[4] = {};
    // activations of one batch
    bf16 *x = nullptr, *xt = nullptr, *h[3] = {}, *ht[3] = {}, *dz[3] = {}, *dzt[3] = {};
    bf16 *dp = nullptr, *dpt = nullptr;
    float* P = nullptr;
    float *cond = nullptr, *y = nullptr, *nh = nullptr;
    int* hy = nullptr;
    float* cw = nullptr;  // per-row weights of the count term
    double* loss = nullptr;
    int* gemm_err = nullptr;
    int* skip = nullptr;     // set when a step's gradient is not finite
    ntp::StepIO* io = nullptr;  // the batch sources of a multi-step call on the device
    long long skipped = 0;   // steps skipped for that reason
    int* step_dev = nullptr;  // Adam's step count on the device, and its finished-block counter
    float* lr_dev = nullptr;  // Adam's step size on the device
    // the training step captured as a CUDA graph (per batch size and update flag)
    bool use_graph = true;
    // the conditioner's forward pass and the backward chain of activation
    // gradients as one fused kernel each (NTP_FLOW_CHAIN=0: one GEMM per layer)
    bool use_chain = true;
    cudaGraphExec_t gexec = nullptr;
    int g_B = 0, g_update = -1, g_rows_w = -1, g_dev = -1;
    // per-step losses and skip flags of a multi-step call (grown on demand)
    double* loss_hist = nullptr;
    int* skip_hist = nullptr;
    int hist_cap = 0;
    // inference
    float* knots = nullptr;
    size_t knots_cap = 0;
    // sampling scratch (keys, counts, offsets, scan sums; grown on demand) and
    // the state of a sample that overflowed its buffers (resumable)
    unsigned long long* samp = nullptr;
    size_t samp_cap = 0;
    int samp_n = 0;  // conditions of the pending sample, 0 = none
    uint2 samp_key{};
    unsigned long long samp_total = 0;
};

namespace {

constexpr int kHid = 256, kIn = 64, kCond = 5;

ntp_status ferr(ntp_flow* f, cudaError_t e, const char* what) {
    f->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorInvalidValue ? NTP_ERR_INVALID : (e == cudaErrorMemoryAllocation ? NTP_ERR_NOMEM : NTP_ERR_CUDA);
}

#define F_CUDA(f, call)                                     \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return ferr((f), e_, #call); \
    } while (0)

#define F_OK(expr)                          \
    do {                                    \
        const ntp_status s_ = (expr);       \
        if (s_ != NTP_OK) return s_;        \
    } while (0)

// calls fn with the bin count as a compile-time constant (10 or 12)
template <typename Fn>
void with_bins(int K, Fn&& fn) {
    if (K == 10) fn(std::integral_constant<int, 10>{});
    else fn(std::integral_constant<int, 12>{});
}

// Launch with programmatic stream serialisation (the kernel waits for the
// previous kernel of the stream with griddepcontrol.wait before it reads)
template <typename... Exp, typename... Act>
cudaError_t launch_dep(void (*kernel)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Act&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = ntp::tc::pdl_enabled();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Act>(args)...);
}

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1));
}

ntp_status gemm(ntp_flow* f, const bf16* A, int lda, const bf16* B, int ldb, int M, int N, int K,
                const ntp::GemmEpilogue& ep, int splits = 1, cudaStream_t st = nullptr) {
    F_CUDA(f, ntp::gemm_bf16_ep(A, lda, B, ldb, M, N, K, ep, splits, f->gemm_err, st ? st : f->stream));
    return NTP_OK;
}

// P = conditioner(X) for n rows (X packed, n a multiple of 128); for
// training also the transposed activations the weight gradients read
ntp_status forward(ntp_flow* f, int n, bool keep_transposed) {
    if (f->use_chain) {
        // X -> H1 -> H2 -> H3 -> P in one kernel per 128-row tile; for
        // training the activations (the backward pass's ReLU masks) and their
        // transposes (the weight gradients' operands) go to global memory too
        ntp::ChainSpec cs{};
        cs.n_stages = 4;
        cs.m = n;
        cs.weights_ready = 1;  // written by Adam or a parameter upload, before the pack kernel
        for (int l = 0; l < 3; ++l) {
            ntp::ChainStage& s = cs.st[l];
            s.n = kHid;
            s.k = l == 0 ? kIn : kHid;
            s.bias = f->theta + f->blk[2 * l + 1].off;
            s.relu = 1;
            s.c = keep_transposed ? f->h[l] : nullptr;
            s.ldc = kHid;
            s.ct = keep_transposed ? f->ht[l] : nullptr;
            s.ldct = n;
        }
        ntp::ChainStage& o = cs.st[3];
        o.n = f->n_pad;
        o.k = kHid;
        o.bias = f->theta + f->blk[7].off;
        o.c32 = f->P;
        o.ldc32 = f->n_pad;
        const void* w[4] = {f->wb[0], f->wb[1], f->wb[2], f->wb[3]};
        F_CUDA(f, ntp::layer_chain(f->x, kIn, w, cs, f->gemm_err, f->stream));
        return NTP_OK;
    }
    ntp::GemmEpilogue e{};
    e.out_kind = 1;
    e.relu = 1;
    e.ldc = kHid;
    e.ldct = n;
    const bf16* in = f->x;
    int k_in = kIn;
    for (int l = 0; l < 3; ++l) {
        e.c = f->h[l];
        e.ct = keep_transposed ? f->ht[l] : nullptr;
        e.bias = f->theta + f->blk[2 * l + 1].off;
        F_OK(gemm(f, in, k_in, f->wb[l], k_in, n, kHid, k_in, e));
        in = f->h[l];
        k_in = kHid;
    }
    ntp::GemmEpilogue o{};
    o.c = f->P;
    o.ldc = f->n_pad;
    o.out_kind = 0;
    o.bias = f->theta + f->blk[7].off;
    return gemm(f, f->h[2], kHid, f->wb[3], kHid, n, f->n_pad, kHid, o);
}

// conditions (host or device, n_valid rows) -> packed X with n rows
ntp_status pack(ntp_flow* f, const float* cond, int n_valid, int n, int on_device) {
    const float* dc = cond;
    if (!on_device) {
        F_CUDA(f, cudaMemcpyAsync(f->cond, cond, sizeof(float) * kCond * n_valid, cudaMemcpyHostToDevice, f->stream));
        dc = f->cond;
    }
    F_CUDA(f, launch_dep(ntp::pack_kernel, dim3(ntp::blocks_for(static_cast<long long>(n) * (kIn / 8))), dim3(256), 0,
                         f->stream, dc, n_valid, n, f->in_mode, f->x, f->xt));
    return NTP_OK;
}

ntp_status check_gemm(ntp_flow* f) {
    int herr = 0;
    F_CUDA(f, cudaMemcpyAsync(&herr, f->gemm_err, sizeof(int), cudaMemcpyDeviceToHost, f->stream));
    F_CUDA(f, cudaStreamSynchronize(f->stream));
    if (herr) {
        f->err = "tensor-core pipeline wait timed out";
        return NTP_ERR_TIMEOUT;
    }
    return NTP_OK;
}

// the head kernel on f->P for B samples (32 per block, one warp per layer)
ntp_status launch_head(ntp_flow* f, const float* y, const float* nh, const int* hy, const float* cwr, int B, float* gf,
                       float* gbias) {
    const size_t smem = sizeof(float) * ntp::head_smem_floats(f->L, f->K, f->n_pad);
    cudaError_t e = cudaSuccess;
    with_bins(f->K, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        e = cudaStreamIsCapturing(f->stream, &cs);
        if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone)  // set before a capture by prepare_kernels
            e = cudaFuncSetAttribute(ntp::head_grad_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem));
        if (e == cudaSuccess) {
            e = launch_dep(ntp::head_grad_kernel<K>, dim3((B + 31) / 32), dim3(32 * f->L), smem, f->stream, f->P,
                           f->n_pad, f->L, y, nh, hy, B, f->r0, f->r1, f->clip, f->count_w, cwr, f->dp, f->dpt, gf,
                           gbias, f->loss);
        }
    });
    if (e != cudaSuccess) return ferr(f, e, "head kernel");
    return NTP_OK;
}

void free_all(ntp_flow* f) {
    void* ps[] = {f->theta, f->m, f->v, f->grad, f->x, f->xt, f->dp, f->dpt, f->P, f->cond, f->y, f->nh, f->hy,
                  f->loss, f->gemm_err, f->skip, f->io, f->step_dev, f->lr_dev, f->knots, f->loss_hist, f->skip_hist, f->cw,
                  f->samp};
    for (void* p : ps)
        if (p) cudaFree(p);
    for (int l = 0; l < 4; ++l) {
        if (f->wb[l]) cudaFree(f->wb[l]);
        if (f->wt[l]) cudaFree(f->wt[l]);
    }
    for (int l = 0; l < 3; ++l) {
        if (f->h[l]) cudaFree(f->h[l]);
        if (f->ht[l]) cudaFree(f->ht[l]);
        if (f->dz[l]) cudaFree(f->dz[l]);
        if (f->dzt[l]) cudaFree(f->dzt[l]);
    }
}

// Every device operation of one training step on the staged batch (f->cond,
// f->y, f->nh, f->hy): no host synchronisation, so it can be captured.
// (dev_io: the batch is staged from the sources in f->io by the step's
// first kernel and the step's loss and skip flag recorded by its last; the
// memsets come first, so that every kernel follows a kernel and takes the
// programmatic dependent launch.)
ntp_status record_step(ntp_flow* f, int B, bool update, bool rows_w, bool dev_io) {
    cudaStream_t st = f->stream;
    F_CUDA(f, cudaMemsetAsync(f->gemm_err, 0, sizeof(int), st));
    F_CUDA(f, cudaMemsetAsync(f->loss, 0, sizeof(double), st));
    F_CUDA(f, cudaMemsetAsync(f->grad, 0, sizeof(float) * f->n_params, st));
    if (update) F_CUDA(f, cudaMemsetAsync(f->skip, 0, sizeof(int), st));
    if (dev_io)
        F_CUDA(f, launch_dep(ntp::stage_kernel, dim3(ntp::blocks_for(static_cast<long long>(B) * kCond)), dim3(256), 0,
                             st, f->io, B, f->cond, f->y, f->nh, f->hy, f->cw));
    F_OK(pack(f, f->cond, B, B, 1));
    F_OK(forward(f, B, true));
    float* g = f->grad;
    auto gw = [&](int l) { return g + f->blk[2 * l].off; };
    auto gb = [&](int l) { return g + f->blk[2 * l + 1].off; };
    F_OK(launch_head(f, f->y, f->nh, f->hy, rows_w ? f->cw : nullptr, B, nullptr, gb(3)));
    cudaStream_t s2 = f->stream2;
    if (f->use_chain) {
        // dP -> dZ3 -> dZ2 -> dZ1 in one kernel per 128-row tile: each stage
        // masked by its layer's activations, its transpose and column sums
        // (the bias gradient) to global memory; then the four weight
        // gradients dW_l = dZ_l^T X_l (dW4 = dP^T H3) in one grouped launch
        ntp::ChainSpec cs{};
        cs.n_stages = 3;
        cs.m = B;
        cs.weights_ready = 1;  // written by Adam or a parameter upload, before this step's kernels
        for (int i = 0; i < 3; ++i) {
            const int l = 2 - i;
            ntp::ChainStage& s = cs.st[i];
            s.n = kHid;
            s.k = i == 0 ? f->n_pad : kHid;
            s.mask = f->h[l];
            s.ldm = kHid;
            s.ct = f->dzt[l];
            s.ldct = B;
            s.colsum = gb(l);
        }
        const void* w[3] = {f->wt[3], f->wt[2], f->wt[1]};
        F_CUDA(f, ntp::layer_chain(f->dp, f->n_pad, w, cs, f->gemm_err, st));
        ntp::GemmProblem pr[4] = {};
        for (int l = 3; l >= 0; --l) {
            ntp::GemmProblem& q = pr[3 - l];
            q.a = l == 3 ? f->dpt : f->dzt[l];
            q.lda = B;
            q.b = l == 0 ? f->xt : f->ht[l - 1];
            q.ldb = B;
            q.M = l == 3 ? f->n_pad : kHid;
            q.N = l == 0 ? kIn : kHid;
            q.K = B;
            q.ep.out_kind = 2;
            q.ep.c = gw(l);
            q.ep.ldc = q.N;
        }
        F_CUDA(f, ntp::gemm_bf16_group(pr, 4, f->gemm_err, st));
    } else {
        // The weight gradients dW_l = dZ_l^T X_l run on stream2 beside the
        // chain of activation gradients dZ_{l-1} = (dZ_l W_l) * mask on the
        // main stream; events order each dW_l after its dZ_l and join the
        // two before Adam.
        F_CUDA(f, cudaEventRecord(f->ev[0], st));
        F_CUDA(f, cudaStreamWaitEvent(s2, f->ev[0], 0));
        ntp::GemmEpilogue ew{};  // output layer: dW4 = dP^T H3
        ew.out_kind = 2;
        ew.ldc = kHid;
        ew.c = gw(3);
        F_OK(gemm(f, f->dpt, B, f->ht[2], B, f->n_pad, kHid, B, ew, 0, s2));
    }
    const bf16* dnext = f->dp;
    int k_next = f->n_pad;
    for (int l = 2; !f->use_chain && l >= 0; --l) {
        // dZ_l = (dZ_{l+1} W_{l+1}) masked by H_l > 0, its transpose, and its
        // column sums (the bias gradient of layer l)
        ntp::GemmEpilogue ed{};
        ed.c = f->dz[l];
        ed.ldc = kHid;
        ed.out_kind = 1;
        ed.ct = f->dzt[l];
        ed.ldct = B;
        ed.mask = f->h[l];
        ed.ldm = kHid;
        ed.colsum = gb(l);
        F_OK(gemm(f, dnext, k_next, f->wt[l + 1], k_next, B, kHid, k_next, ed));
        F_CUDA(f, cudaEventRecord(f->ev[3 - l], st));
        F_CUDA(f, cudaStreamWaitEvent(s2, f->ev[3 - l], 0));
        // dW_l = dZ_l^T X_l with X_l = H_{l-1} or the packed input
        ntp::GemmEpilogue eg{};
        eg.out_kind = 2;
        eg.c = gw(l);
        eg.ldc = l == 0 ? kIn : kHid;
        const bf16* xt = l == 0 ? f->xt : f->ht[l - 1];
        F_OK(gemm(f, f->dzt[l], B, xt, B, kHid, l == 0 ? kIn : kHid, B, eg, 0, s2));
        dnext = f->dz[l];
        k_next = kHid;
    }
    if (!f->use_chain) {
        F_CUDA(f, cudaEventRecord(f->ev[4], s2));
        F_CUDA(f, cudaStreamWaitEvent(st, f->ev[4], 0));
    }
    if (update) {
        ntp::ParamBlocks pb{};
        pb.n = 8;
        for (int i = 0; i < 8; ++i) {
            pb.off[i] = static_cast<long long>(f->blk[i].off);
            pb.rows[i] = f->blk[i].rows;
            pb.cols[i] = f->blk[i].cols;
            pb.wb[i] = (i % 2) == 0 ? f->wb[i / 2] : nullptr;
            pb.wt[i] = (i % 2) == 0 ? f->wt[i / 2] : nullptr;
        }
        pb.off[8] = static_cast<long long>(f->n_params);
        const int grid = static_cast<int>(std::min<size_t>((f->n_params + 255) / 256, 152 * 8));
        F_CUDA(f, launch_dep(ntp::nonfinite_kernel, dim3(grid), dim3(256), 0, st, g, static_cast<long long>(f->n_params),
                             f->skip));
        F_CUDA(f, launch_dep(ntp::adam_kernel, dim3(grid), dim3(256), 0, st, f->theta, f->m, f->v, g, pb, f->lr_dev,
                             f->b1, f->b2, f->eps, f->step_dev, f->skip));
    }
    if (dev_io)
        F_CUDA(f, launch_dep(ntp::step_end_kernel, dim3(1), dim3(1), 0, st, f->io, f->loss, f->skip,
                             update ? 1 : 0));
    return NTP_OK;
}

// Function attributes the step's kernels need, set before a capture.
cudaError_t prepare_kernels(ntp_flow* f) {
    cudaError_t e = ntp::gemm_prepare();
    if (e == cudaSuccess) e = ntp::layer_chain_prepare();
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(float) * ntp::head_smem_floats(f->L, f->K, f->n_pad);
    with_bins(f->K, [&](auto kc) {
        e = cudaFuncSetAttribute(ntp::head_grad_kernel<decltype(kc)::value>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    });
    return e;
}

}  // namespace

extern "C" {

ntp_status ntp_flow_create(int32_t device, const ntp_flow_config* cfg, ntp_flow** out) {
    if (!cfg || !out) return NTP_ERR_INVALID;
    *out = nullptr;
    if (cfg->batch_capacity < 128 || cfg->batch_capacity % 128 || cfg->n_layers < 1 ||
        (cfg->n_bins != 10 && cfg->n_bins != 12) ||
        cfg->n_layers > ntp::kMaxLayers || !(cfg->t_max > cfg->t_min) || !(cfg->lr > 0.0f) ||
        !(cfg->beta1 >= 0.0f && cfg->beta1 < 1.0f) || !(cfg->beta2 >= 0.0f && cfg->beta2 < 1.0f) ||
        !(cfg->eps > 0.0f) || !(cfg->grad_clip >= 0.0f) || !(cfg->count_weight >= 0.0f) ||
        (cfg->input_columns != NTP_FLOW_INPUT_FEATURES && cfg->input_columns != NTP_FLOW_INPUT_DERIVED))
        return NTP_ERR_INVALID;
    ntp_flow* f = new ntp_flow();
    f->device = device;
    f->in_mode = cfg->input_columns;
    f->cap = cfg->batch_capacity;
    f->L = cfg->n_layers;
    f->K = cfg->n_bins;
    f->n_out = ntp::n_outputs(f->L, f->K);
    f->n_pad = ntp::n_outputs_padded(f->L, f->K);
    f->r0 = cfg->t_min;
    f->r1 = cfg->t_max;
    f->lr = cfg->lr;
    f->b1 = cfg->beta1;
    f->b2 = cfg->beta2;
    f->eps = cfg->eps;
    f->clip = cfg->grad_clip;
    {
        const char* eg = std::getenv("NTP_FLOW_GRAPH");
        f->use_graph = !(eg && eg[0] == '0');
        const char* ec = std::getenv("NTP_FLOW_CHAIN");
        f->use_chain = !(ec && ec[0] == '0');
    }
    f->count_w = cfg->count_weight;
    const int dims[4][2] = {{kHid, kIn}, {kHid, kHid}, {kHid, kHid}, {f->n_pad, kHid}};
    size_t off = 0;
    for (int l = 0; l < 4; ++l) {
        f->blk[2 * l] = Block{dims[l][0], dims[l][1], off};
        off += static_cast<size_t>(dims[l][0]) * dims[l][1];
        f->blk[2 * l + 1] = Block{1, dims[l][0], off};
        off += dims[l][0];
    }
    f->n_params = off;
    auto fail = [&](cudaError_t e) {
        if (f->stream) cudaStreamDestroy(f->stream);
        if (f->stream2) cudaStreamDestroy(f->stream2);
        for (cudaEvent_t ev : f->ev)
            if (ev) cudaEventDestroy(ev);
        free_all(f);
        delete f;
        return e == cudaErrorMemoryAllocation ? NTP_ERR_NOMEM : NTP_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return fail(e);
    if ((e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
    if ((e = cudaStreamCreateWithFlags(&f->stream2, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
    for (cudaEvent_t& ev : f->ev)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
    const size_t B = f->cap;
    if ((e = dalloc(&f->theta, off)) || (e = dalloc(&f->m, off)) || (e = dalloc(&f->v, off)) ||
        (e = dalloc(&f->grad, off)))
        return fail(e);
    for (int l = 0; l < 4; ++l) {
        const size_t n = static_cast<size_t>(dims[l][0]) * dims[l][1];
        if ((e = dalloc(&f->wb[l], n)) || (e = dalloc(&f->wt[l], n))) return fail(e);
    }
    if ((e = dalloc(&f->x, B * kIn)) || (e = dalloc(&f->xt, B * kIn))) return fail(e);
    for (int l = 0; l < 3; ++l)
        if ((e = dalloc(&f->h[l], B * kHid)) || (e = dalloc(&f->ht[l], B * kHid)) ||
            (e = dalloc(&f->dz[l], B * kHid)) || (e = dalloc(&f->dzt[l], B * kHid)))
            return fail(e);
    const size_t np = static_cast<size_t>(f->n_pad);
    if ((e = dalloc(&f->dp, B * np)) || (e = dalloc(&f->dpt, B * np)) || (e = dalloc(&f->P, B * np)) ||
        (e = dalloc(&f->cond, B * kCond)) || (e = dalloc(&f->y, B)) || (e = dalloc(&f->nh, B)) ||
        (e = dalloc(&f->hy, B)) || (e = dalloc(&f->cw, B)) || (e = dalloc(&f->loss, 1)) || (e = dalloc(&f->gemm_err, 1)) ||
        (e = dalloc(&f->skip, 1)) || (e = dalloc(&f->io, 1)) || (e = dalloc(&f->step_dev, 2)) || (e = dalloc(&f->lr_dev, 1)))
        return fail(e);
    // He-uniform weights (seeded); zero biases, zero padding input columns of
    // W1 and zero padding rows of W4; the output layer scaled by 0.1
    std::vector<float> th(off, 0.0f);
    std::mt19937_64 rng(cfg->seed);
    for (int l = 0; l < 4; ++l) {
        const Block& b = f->blk[2 * l];
        const int n_in = kCond + (f->in_mode == NTP_FLOW_INPUT_DERIVED ? ntp::kDerived : 0);
        const int fan_in = l == 0 ? n_in : b.cols;
        const float lim = std::sqrt(6.0f / fan_in) * (l == 3 ? 0.1f : 1.0f);
        std::uniform_real_distribution<float> u(-lim, lim);
        for (int r = 0; r < b.rows; ++r)
            for (int c = 0; c < b.cols; ++c) {
                const bool pad = (l == 0 && c >= n_in) || (l == 3 && r >= f->n_out);
                const float val = u(rng);
                th[b.off + static_cast<size_t>(r) * b.cols + c] = pad ? 0.0f : val;
            }
    }
    const ntp_status s = ntp_flow_set_params(f, th.data(), off);
    if (s != NTP_OK) {
        ntp_flow_destroy(f);
        return s;
    }
    *out = f;
    return NTP_OK;
}

void ntp_flow_destroy(ntp_flow* f) {
    if (!f) return;
    cudaSetDevice(f->device);
    if (f->stream) cudaStreamSynchronize(f->stream);
    if (f->gexec) cudaGraphExecDestroy(f->gexec);
    if (f->stream2) cudaStreamSynchronize(f->stream2);
    free_all(f);
    for (cudaEvent_t ev : f->ev)
        if (ev) cudaEventDestroy(ev);
    if (f->stream2) cudaStreamDestroy(f->stream2);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
}

const char* ntp_flow_last_error(const ntp_flow* f) { return f ? f->err.c_str() : "null flow"; }

ntp_status ntp_flow_get_layout(const ntp_flow* f, uint64_t* n_params, int32_t* n_outputs, int32_t* n_outputs_padded) {
    if (!f) return NTP_ERR_INVALID;
    if (n_params) *n_params = f->n_params;
    if (n_outputs) *n_outputs = f->n_out;
    if (n_outputs_padded) *n_outputs_padded = f->n_pad;
    return NTP_OK;
}

ntp_status ntp_flow_set_params(ntp_flow* f, const float* host, uint64_t n) {
    if (!f || !host || n != f->n_params) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    F_CUDA(f, cudaMemcpyAsync(f->theta, host, sizeof(float) * n, cudaMemcpyHostToDevice, f->stream));
    for (int l = 0; l < 4; ++l) {
        const Block& b = f->blk[2 * l];
        const int cnt = b.rows * b.cols;
        ntp::to_bf16_kernel<<<ntp::blocks_for(cnt), 256, 0, f->stream>>>(f->theta + b.off, cnt, b.cols, b.rows,
                                                                         f->wb[l], f->wt[l]);
        F_CUDA(f, cudaGetLastError());
    }
    F_CUDA(f, cudaMemsetAsync(f->m, 0, sizeof(float) * n, f->stream));
    F_CUDA(f, cudaMemsetAsync(f->v, 0, sizeof(float) * n, f->stream));
    F_CUDA(f, cudaMemsetAsync(f->grad, 0, sizeof(float) * n, f->stream));
    F_CUDA(f, cudaMemsetAsync(f->step_dev, 0, 2 * sizeof(int), f->stream));
    F_CUDA(f, cudaMemcpyAsync(f->lr_dev, &f->lr, sizeof(float), cudaMemcpyHostToDevice, f->stream));
    F_CUDA(f, cudaStreamSynchronize(f->stream));
    f->step = 0;
    return NTP_OK;
}

ntp_status ntp_flow_set_lr(ntp_flow* f, float lr) {
    if (!f || !(lr > 0.0f)) return NTP_ERR_INVALID;
    f->lr = lr;
    F_CUDA(f, cudaSetDevice(f->device));
    F_CUDA(f, cudaMemcpyAsync(f->lr_dev, &f->lr, sizeof(float), cudaMemcpyHostToDevice, f->stream));
    F_CUDA(f, cudaStreamSynchronize(f->stream));
    return NTP_OK;
}

ntp_status ntp_flow_get_params(ntp_flow* f, float* host, uint64_t n, int32_t which) {
    if (!f || !host || n != f->n_params || which < 0 || which > 3) return NTP_ERR_INVALID;
    const float* src = which == 0 ? f->theta : which == 1 ? f->grad : which == 2 ? f->m : f->v;
    F_CUDA(f, cudaSetDevice(f->device));
    F_CUDA(f, cudaMemcpyAsync(host, src, sizeof(float) * n, cudaMemcpyDeviceToHost, f->stream));
    F_CUDA(f, cudaStreamSynchronize(f->stream));
    return NTP_OK;
}

ntp_status ntp_flow_train_step(ntp_flow* f, const float* cond, const float* tres, const float* nhits,
                               const int32_t* has_time, int32_t B, int32_t on_device, int32_t update,
                               double* loss_out) {
    return ntp_flow_train_steps(f, cond, tres, nhits, has_time, nullptr, B, 1, on_device, update, loss_out);
}

ntp_status ntp_flow_train_steps(ntp_flow* f, const float* cond, const float* tres, const float* nhits,
                                const int32_t* has_time, const float* count_weight, int32_t B, int32_t n_steps,
                                int32_t on_device, int32_t update, double* losses) {
    if (!f || !cond || !tres || !nhits || !has_time || n_steps < 1) return NTP_ERR_INVALID;
    if (B < 128 || B > f->cap || B % 128) {
        f->err = "ntp_flow_train_step: the batch must be a multiple of 128 up to the capacity";
        return NTP_ERR_INVALID;
    }
    F_CUDA(f, cudaSetDevice(f->device));
    cudaStream_t st = f->stream;
    // per-step loss and skip flag, gathered on the device and read once
    if (f->hist_cap < n_steps) {
        if (f->loss_hist) cudaFree(f->loss_hist);
        if (f->skip_hist) cudaFree(f->skip_hist);
        f->loss_hist = nullptr;
        f->skip_hist = nullptr;
        f->hist_cap = 0;
        F_CUDA(f, dalloc(&f->loss_hist, static_cast<size_t>(n_steps)));
        F_CUDA(f, dalloc(&f->skip_hist, static_cast<size_t>(n_steps)));
        f->hist_cap = n_steps;
    }
    double* d_loss = f->loss_hist;
    int* d_skip = f->skip_hist;
    const bool rows_w = count_weight != nullptr;
    const bool dev_io = on_device != 0;
    F_CUDA(f, cudaMemsetAsync(d_skip, 0, sizeof(int) * n_steps, st));
    if (dev_io) {
        // the sources once; each step stages its own rows and records its loss
        ntp::StepIO io{cond, tres, nhits, has_time, count_weight, d_loss, d_skip, 0};
        F_CUDA(f, cudaMemcpyAsync(f->io, &io, sizeof(io), cudaMemcpyHostToDevice, st));
    }
    for (int i = 0; i < n_steps; ++i) {
        const size_t o = static_cast<size_t>(i) * B;
        if (!dev_io) {
            // the batch into the staging buffers the step reads
            F_CUDA(f, cudaMemcpyAsync(f->cond, cond + o * kCond, sizeof(float) * kCond * B, cudaMemcpyHostToDevice, st));
            F_CUDA(f, cudaMemcpyAsync(f->y, tres + o, sizeof(float) * B, cudaMemcpyHostToDevice, st));
            F_CUDA(f, cudaMemcpyAsync(f->nh, nhits + o, sizeof(float) * B, cudaMemcpyHostToDevice, st));
            F_CUDA(f, cudaMemcpyAsync(f->hy, has_time + o, sizeof(int) * B, cudaMemcpyHostToDevice, st));
            if (rows_w)
                F_CUDA(f, cudaMemcpyAsync(f->cw, count_weight + o, sizeof(float) * B, cudaMemcpyHostToDevice, st));
        }
        if (f->use_graph) {
            if (!f->gexec || f->g_B != B || f->g_update != update || f->g_rows_w != static_cast<int>(rows_w) ||
                f->g_dev != static_cast<int>(dev_io)) {
                if (f->gexec) cudaGraphExecDestroy(f->gexec);
                f->gexec = nullptr;
                F_CUDA(f, prepare_kernels(f));
                F_CUDA(f, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                const ntp_status rs = record_step(f, B, update != 0, rows_w, dev_io);
                cudaGraph_t graph = nullptr;
                const cudaError_t ec = cudaStreamEndCapture(st, &graph);
                if (rs != NTP_OK || ec != cudaSuccess) {
                    if (graph) cudaGraphDestroy(graph);
                    if (rs != NTP_OK) return rs;
                    return ferr(f, ec, "ntp_flow_train_step: capture");
                }
                const cudaError_t ei = cudaGraphInstantiate(&f->gexec, graph, 0);
                cudaGraphDestroy(graph);
                if (ei != cudaSuccess) {
                    f->gexec = nullptr;
                    return ferr(f, ei, "ntp_flow_train_step: instantiate");
                }
                f->g_B = B;
                f->g_update = update;
                f->g_rows_w = static_cast<int>(rows_w);
                f->g_dev = static_cast<int>(dev_io);
            }
            F_CUDA(f, cudaGraphLaunch(f->gexec, st));
        } else {
            F_OK(record_step(f, B, update != 0, rows_w, dev_io));
        }
        if (!dev_io) {
            F_CUDA(f, cudaMemcpyAsync(d_loss + i, f->loss, sizeof(double), cudaMemcpyDeviceToDevice, st));
            if (update) F_CUDA(f, cudaMemcpyAsync(d_skip + i, f->skip, sizeof(int), cudaMemcpyDeviceToDevice, st));
        }
    }
    std::vector<double> hl(n_steps);
    std::vector<int> hs(n_steps);
    F_CUDA(f, cudaMemcpyAsync(hl.data(), d_loss, sizeof(double) * n_steps, cudaMemcpyDeviceToHost, st));
    F_CUDA(f, cudaMemcpyAsync(hs.data(), d_skip, sizeof(int) * n_steps, cudaMemcpyDeviceToHost, st));
    F_OK(check_gemm(f));
    for (int i = 0; i < n_steps; ++i) {
        if (update) {
            if (hs[i]) {
                ++f->skipped;
                hl[i] = std::numeric_limits<double>::quiet_NaN();
            } else {
                ++f->step;
            }
        }
        if (losses) losses[i] = hl[i];
    }
    return NTP_OK;
}

ntp_status ntp_flow_forward(ntp_flow* f, const float* cond, int32_t n, float* params_out) {
    if (!f || !cond || !params_out || n <= 0) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    cudaStream_t st = f->stream;
    F_CUDA(f, cudaMemsetAsync(f->gemm_err, 0, sizeof(int), st));
    for (int c0 = 0; c0 < n; c0 += f->cap) {
        const int m = std::min(f->cap, n - c0);
        const int mp = (m + 127) / 128 * 128;
        F_OK(pack(f, cond + static_cast<size_t>(c0) * kCond, m, mp, 0));
        F_OK(forward(f, mp, false));
        F_CUDA(f, cudaMemcpy2DAsync(params_out + static_cast<size_t>(c0) * f->n_out, sizeof(float) * f->n_out, f->P,
                                    sizeof(float) * f->n_pad, sizeof(float) * f->n_out, m, cudaMemcpyDeviceToHost,
                                    st));
    }
    return check_gemm(f);
}

ntp_status ntp_flow_head(ntp_flow* f, const float* params, const float* tres, const float* nhits,
                         const int32_t* has_time, const float* count_weight, int32_t B, double* loss_out,
                         float* grad_out) {
    if (!f || !params || !tres || !nhits || !has_time || B <= 0 || B > f->cap) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    cudaStream_t st = f->stream;
    float* gf = nullptr;
    F_CUDA(f, dalloc(&gf, static_cast<size_t>(B) * f->n_pad));
    auto run = [&]() -> ntp_status {
        F_CUDA(f, cudaMemcpy2DAsync(f->P, sizeof(float) * f->n_pad, params, sizeof(float) * f->n_out,
                                    sizeof(float) * f->n_out, B, cudaMemcpyHostToDevice, st));
        F_CUDA(f, cudaMemcpyAsync(f->y, tres, sizeof(float) * B, cudaMemcpyHostToDevice, st));
        F_CUDA(f, cudaMemcpyAsync(f->nh, nhits, sizeof(float) * B, cudaMemcpyHostToDevice, st));
        F_CUDA(f, cudaMemcpyAsync(f->hy, has_time, sizeof(int) * B, cudaMemcpyHostToDevice, st));
        if (count_weight)
            F_CUDA(f, cudaMemcpyAsync(f->cw, count_weight, sizeof(float) * B, cudaMemcpyHostToDevice, st));
        F_CUDA(f, cudaMemsetAsync(f->loss, 0, sizeof(double), st));
        F_OK(launch_head(f, f->y, f->nh, f->hy, count_weight ? f->cw : nullptr, B, gf, nullptr));
        F_CUDA(f, cudaGetLastError());
        double hl = 0.0;
        F_CUDA(f, cudaMemcpyAsync(&hl, f->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (grad_out)
            F_CUDA(f, cudaMemcpy2DAsync(grad_out, sizeof(float) * f->n_out, gf, sizeof(float) * f->n_pad,
                                        sizeof(float) * f->n_out, B, cudaMemcpyDeviceToHost, st));
        F_CUDA(f, cudaStreamSynchronize(st));
        if (loss_out) *loss_out = hl;
        return NTP_OK;
    };
    const ntp_status s = run();
    cudaFree(gf);
    return s;
}

ntp_status ntp_flow_evaluate(ntp_flow* f, const float* cond, int32_t n_cond, const int32_t* cond_index,
                             const float* times, uint64_t n_tuples, float* logpdf, float* log_expec,
                             int32_t on_device) {
    if (!f || !cond || n_cond <= 0) return NTP_ERR_INVALID;
    if (n_tuples > 0 && (!cond_index || !times || !logpdf)) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    f->samp_n = 0;  // the knots are rewritten: no pending sample
    cudaStream_t st = f->stream;
    const int row = ntp::knot_row(f->L, f->K);
    const size_t need = static_cast<size_t>(n_cond) * row;
    if (need > f->knots_cap) {
        if (f->knots) cudaFree(f->knots);
        f->knots = nullptr;
        f->knots_cap = 0;
        F_CUDA(f, dalloc(&f->knots, need));
        f->knots_cap = need;
    }
    F_CUDA(f, cudaMemsetAsync(f->gemm_err, 0, sizeof(int), st));
    // the conditioner in chunks of the batch capacity, then the knots
    for (int c0 = 0; c0 < n_cond; c0 += f->cap) {
        const int m = std::min(f->cap, n_cond - c0);
        const int mp = (m + 127) / 128 * 128;
        F_OK(pack(f, cond + static_cast<size_t>(c0) * kCond, m, mp, on_device));
        F_OK(forward(f, mp, false));
        with_bins(f->K, [&](auto kc) {
            ntp::knots_kernel<decltype(kc)::value><<<ntp::blocks_for(m, 128), 128, 0, st>>>(
                f->P, f->n_pad, f->L, m, f->r0, f->r1, f->knots + static_cast<size_t>(c0) * row);
        });
        F_CUDA(f, cudaGetLastError());
    }
    if (log_expec) {
        F_CUDA(f, cudaMemcpy2DAsync(log_expec, sizeof(float), f->knots + row - 1, sizeof(float) * row, sizeof(float),
                                    n_cond, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    }
    if (n_tuples > 0) {
        const int grid = static_cast<int>(std::min<unsigned long long>((n_tuples + 255) / 256, 152ull * 16));
        if (on_device) {
            with_bins(f->K, [&](auto kc) {
                ntp::logpdf_kernel<decltype(kc)::value>
                    <<<grid, 256, 0, st>>>(f->knots, f->L, n_cond, cond_index, times, n_tuples, logpdf);
            });
            F_CUDA(f, cudaGetLastError());
        } else {
            void* tmp = nullptr;
            F_CUDA(f, cudaMalloc(&tmp, n_tuples * (sizeof(int) + 2 * sizeof(float))));
            int* di = static_cast<int*>(tmp);
            float* dt = reinterpret_cast<float*>(di + n_tuples);
            float* dout = dt + n_tuples;
            cudaError_t e = cudaMemcpyAsync(di, cond_index, sizeof(int) * n_tuples, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dt, times, sizeof(float) * n_tuples, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                with_bins(f->K, [&](auto kc) {
                    ntp::logpdf_kernel<decltype(kc)::value>
                        <<<grid, 256, 0, st>>>(f->knots, f->L, n_cond, di, dt, n_tuples, dout);
                });
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(logpdf, dout, sizeof(float) * n_tuples, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            cudaFree(tmp);
            if (e != cudaSuccess) return ferr(f, e, "ntp_flow_evaluate");
        }
    }
    return check_gemm(f);
}


namespace {

// Draws the hits of the counts and offsets in f->samp (keys | counts |
// offsets) for the knots in f->knots.
ntp_status sample_draw(ntp_flow* f, int n_cond, uint2 key, unsigned long long total, int32_t* hit_cond,
                       float* hit_time, int32_t on_device) {
    cudaStream_t st = f->stream;
    const size_t n = static_cast<size_t>(n_cond);
    const unsigned long long* d_key = f->samp;
    const unsigned long long* d_off = f->samp + 2 * n;
    int32_t* d_hc = hit_cond;
    float* d_ht = hit_time;
    void* stage = nullptr;
    if (!on_device) {
        F_CUDA(f, cudaMalloc(&stage, 8 * total));
        d_hc = static_cast<int32_t*>(stage);
        d_ht = reinterpret_cast<float*>(static_cast<int32_t*>(stage) + total);
    }
    const int grid = static_cast<int>(std::min<unsigned long long>((total + 255) / 256, 152ull * 32));
    cudaError_t e = cudaSuccess;
    with_bins(f->K, [&](auto kc) {
        ntp::sample_draw_kernel<decltype(kc)::value>
            <<<grid, 256, 0, st>>>(f->knots, f->L, n_cond, d_key, key, d_off, total, d_hc, d_ht);
        e = cudaGetLastError();
    });
    if (e == cudaSuccess && !on_device) {
        e = cudaMemcpyAsync(hit_cond, d_hc, 4 * total, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hit_time, d_ht, 4 * total, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (stage) cudaFree(stage);
    if (e != cudaSuccess) return ferr(f, e, "ntp_flow_sample");
    return NTP_OK;
}

}  // namespace

ntp_status ntp_flow_sample(ntp_flow* f, const float* cond, int32_t n_cond, const uint64_t* cond_key, uint64_t seed,
                           uint64_t* counts, int32_t* hit_cond, float* hit_time, uint64_t capacity, uint64_t* n_hits,
                           int32_t on_device) {
    return ntp_flow_sample_expec(f, cond, n_cond, cond_key, seed, nullptr, counts, hit_cond, hit_time, capacity,
                                 n_hits, on_device);
}

ntp_status ntp_flow_sample_expec(ntp_flow* f, const float* cond, int32_t n_cond, const uint64_t* cond_key,
                                 uint64_t seed, const float* log_expec, uint64_t* counts, int32_t* hit_cond,
                                 float* hit_time, uint64_t capacity, uint64_t* n_hits, int32_t on_device) {
    if (n_hits) *n_hits = 0;
    if (!f || !cond || !cond_key || n_cond <= 0) return NTP_ERR_INVALID;
    if (n_cond > (1 << 20)) {
        f->err = "ntp_flow_sample: at most 1048576 conditions per call";
        return NTP_ERR_INVALID;
    }
    F_CUDA(f, cudaSetDevice(f->device));
    cudaStream_t st = f->stream;
    // knots of every condition (the inference pass of ntp_flow_evaluate)
    F_OK(ntp_flow_evaluate(f, cond, n_cond, nullptr, nullptr, 0, nullptr, nullptr, on_device));
    if (log_expec) {  // the counts' expectations from the caller: into each knot row's last slot
        const int row = ntp::knot_row(f->L, f->K);
        F_CUDA(f, cudaMemcpy2DAsync(f->knots + row - 1, sizeof(float) * row, log_expec, sizeof(float), sizeof(float),
                                    n_cond, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    }
    const int nb = (n_cond + 1023) / 1024;
    // scratch: keys u64[n] | counts u64[n] | offsets u64[n] | block sums u64[nb + 1] x 2 | total
    const size_t n = static_cast<size_t>(n_cond);
    const size_t need = 3 * n + 2 * (static_cast<size_t>(nb) + 1) + 1;
    if (need > f->samp_cap) {
        if (f->samp) cudaFree(f->samp);
        f->samp = nullptr;
        f->samp_cap = 0;
        F_CUDA(f, dalloc(&f->samp, need));
        f->samp_cap = need;
    }
    unsigned long long* d_key = f->samp;
    unsigned long long* d_cnt = f->samp + n;
    unsigned long long* d_off = f->samp + 2 * n;
    unsigned long long* d_bs = f->samp + 3 * n;
    unsigned long long* d_bo = d_bs + nb + 1;
    unsigned long long* d_tot = d_bo + nb + 1;
    F_CUDA(f, cudaMemcpyAsync(d_key, cond_key, 8 * n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              st));
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    ntp::sample_count_kernel<<<ntp::blocks_for(n_cond), 256, 0, st>>>(f->knots, f->L, f->K, n_cond, d_key, key,
                                                                      d_cnt);
    F_CUDA(f, cudaGetLastError());
    ntp::scan_block_kernel<<<nb, 1024, 0, st>>>(d_cnt, n_cond, d_off, d_bs);
    ntp::scan_block_kernel<<<1, 1024, 0, st>>>(d_bs, nb, d_bo, d_bs + nb);  // nb <= 1024
    F_CUDA(f, cudaMemcpyAsync(d_bo + nb, d_bs + nb, 8, cudaMemcpyDeviceToDevice, st));
    ntp::scan_add_kernel<<<nb, 1024, 0, st>>>(d_off, n_cond, d_bo, d_tot, nb);
    F_CUDA(f, cudaGetLastError());
    unsigned long long total = 0;
    F_CUDA(f, cudaMemcpyAsync(&total, d_tot, 8, cudaMemcpyDeviceToHost, st));
    if (counts)
        F_CUDA(f, cudaMemcpyAsync(counts, d_cnt, 8 * n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                  st));
    F_CUDA(f, cudaStreamSynchronize(st));
    if (n_hits) *n_hits = total;
    if (total > capacity) {
        f->samp_n = n_cond;  // resumable: knots, keys and offsets stay
        f->samp_key = key;
        f->samp_total = total;
        f->err = "ntp_flow_sample: capacity " + std::to_string(capacity) + " below " + std::to_string(total);
        return NTP_ERR_OVERFLOW;
    }
    if (total == 0) return NTP_OK;
    if (!hit_cond || !hit_time) return NTP_ERR_INVALID;
    return sample_draw(f, n_cond, key, total, hit_cond, hit_time, on_device);
}

ntp_status ntp_flow_sample_resume(ntp_flow* f, int32_t* hit_cond, float* hit_time, uint64_t capacity,
                                  uint64_t* n_hits, int32_t on_device) {
    if (n_hits) *n_hits = 0;
    if (!f) return NTP_ERR_INVALID;
    if (f->samp_n == 0) {
        f->err = "ntp_flow_sample_resume: no pending sample";
        return NTP_ERR_NOT_READY;
    }
    if (n_hits) *n_hits = f->samp_total;
    if (f->samp_total > capacity) {
        f->err = "ntp_flow_sample_resume: capacity " + std::to_string(capacity) + " below " +
                 std::to_string(f->samp_total);
        return NTP_ERR_OVERFLOW;
    }
    if (!hit_cond || !hit_time) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    const int n = f->samp_n;
    f->samp_n = 0;
    return sample_draw(f, n, f->samp_key, f->samp_total, hit_cond, hit_time, on_device);
}

ntp_status ntp_flow_log_expectation(ntp_flow* f, const float* cond, int32_t n_cond, float* log_expec,
                                    int32_t on_device) {
    if (!f || !cond || !log_expec || n_cond <= 0) return NTP_ERR_INVALID;
    F_CUDA(f, cudaSetDevice(f->device));
    cudaStream_t st = f->stream;
    F_CUDA(f, cudaMemsetAsync(f->gemm_err, 0, sizeof(int), st));
    float* dout = log_expec;
    void* stage = nullptr;
    if (!on_device) {
        F_CUDA(f, cudaMalloc(&stage, sizeof(float) * static_cast<size_t>(n_cond)));
        dout = static_cast<float*>(stage);
    }
    const int col = f->L * (3 * f->K + 1) + 2;
    ntp_status status = NTP_OK;
    for (int c0 = 0; c0 < n_cond && status == NTP_OK; c0 += f->cap) {
        const int m = std::min(f->cap, n_cond - c0);
        const int mp = (m + 127) / 128 * 128;
        status = pack(f, cond + static_cast<size_t>(c0) * kCond, m, mp, on_device);
        if (status == NTP_OK) status = forward(f, mp, false);
        if (status == NTP_OK) {
            ntp::log_expec_kernel<<<ntp::blocks_for(m), 256, 0, st>>>(f->P, f->n_pad, col, m, dout + c0);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) status = ferr(f, e, "ntp_flow_log_expectation");
        }
    }
    if (status == NTP_OK && stage) {
        const cudaError_t e = cudaMemcpyAsync(log_expec, stage, sizeof(float) * n_cond, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) status = ferr(f, e, "ntp_flow_log_expectation");
    }
    if (stage) {
        cudaStreamSynchronize(st);
        cudaFree(stage);
    }
    if (status != NTP_OK) return status;
    return check_gemm(f);
}

ntp_status ntp_flow_evaluate_grid(ntp_flow* f, const float* cond, int32_t n_cond, const float* times, int32_t n_times,
                                  float* logpdf, float* log_expec, int32_t on_device) {
    if (!f || !cond || n_cond <= 0 || n_times <= 0 || !times || !logpdf) return NTP_ERR_INVALID;
    F_OK(ntp_flow_evaluate(f, cond, n_cond, nullptr, nullptr, 0, nullptr, log_expec, on_device));
    cudaStream_t st = f->stream;
    const size_t n_out = static_cast<size_t>(n_cond) * n_times;
    const float* d_t = times;
    float* d_out = logpdf;
    void* stage = nullptr;
    if (!on_device) {
        F_CUDA(f, cudaMalloc(&stage, sizeof(float) * (n_times + n_out)));
        d_t = static_cast<float*>(stage);
        d_out = static_cast<float*>(stage) + n_times;
    }
    auto run = [&]() -> ntp_status {
        if (!on_device)
            F_CUDA(f, cudaMemcpyAsync(const_cast<float*>(d_t), times, sizeof(float) * n_times, cudaMemcpyHostToDevice,
                                      st));
        const int row = ntp::knot_row(f->L, f->K);
        const int grid = std::min(n_cond, 152 * 16);
        cudaError_t e = cudaSuccess;
        with_bins(f->K, [&](auto kc) {
            ntp::logpdf_grid_kernel<decltype(kc)::value>
                <<<grid, 256, sizeof(float) * row, st>>>(f->knots, f->L, n_cond, d_t, n_times, d_out);
            e = cudaGetLastError();
        });
        if (e != cudaSuccess) return ferr(f, e, "ntp_flow_evaluate_grid");
        if (!on_device) F_CUDA(f, cudaMemcpyAsync(logpdf, d_out, sizeof(float) * n_out, cudaMemcpyDeviceToHost, st));
        F_CUDA(f, cudaStreamSynchronize(st));
        return NTP_OK;
    };
    const ntp_status s2 = run();
    if (stage) cudaFree(stage);
    return s2;
}

ntp_status ntp_flow_mixture_cdf(ntp_flow* f, const float* cond, int32_t n_cond, const float* weight,
                                const float* offset, const float* times, uint64_t n_times, double* cdf,
                                int32_t on_device) {
    if (!f || !cond || n_cond <= 0) return NTP_ERR_INVALID;
    if (n_times > 0 && (!times || !cdf)) return NTP_ERR_INVALID;
    F_OK(ntp_flow_evaluate(f, cond, n_cond, nullptr, nullptr, 0, nullptr, nullptr, on_device));
    if (n_times == 0) return NTP_OK;
    cudaStream_t st = f->stream;
    // device copies of host inputs, the output and the weight total
    const size_t nc = static_cast<size_t>(n_cond);
    const size_t bytes = sizeof(double) * (1 + (on_device ? 0 : n_times)) +
                         (on_device ? 0 : sizeof(float) * (n_times + (weight ? nc : 0) + (offset ? nc : 0)));
    void* stage = nullptr;
    F_CUDA(f, cudaMalloc(&stage, bytes));
    double* d_total = static_cast<double*>(stage);
    double* d_out = on_device ? cdf : d_total + 1;
    float* fl = reinterpret_cast<float*>(on_device ? d_total + 1 : d_out + n_times);
    const float* d_t = times;
    const float* d_w = weight;
    const float* d_off = offset;
    auto run = [&]() -> ntp_status {
        if (!on_device) {
            F_CUDA(f, cudaMemcpyAsync(fl, times, sizeof(float) * n_times, cudaMemcpyHostToDevice, st));
            d_t = fl;
            float* nxt = fl + n_times;
            if (weight) {
                F_CUDA(f, cudaMemcpyAsync(nxt, weight, sizeof(float) * nc, cudaMemcpyHostToDevice, st));
                d_w = nxt;
                nxt += nc;
            }
            if (offset) {
                F_CUDA(f, cudaMemcpyAsync(nxt, offset, sizeof(float) * nc, cudaMemcpyHostToDevice, st));
                d_off = nxt;
            }
        }
        const int row = ntp::knot_row(f->L, f->K);
        const size_t smem = sizeof(float) * (ntp::kMixTile * (row + 2));
        const unsigned long long blocks = (n_times + 255) / 256;
        if (blocks > 0x7fffffffull) {
            f->err = "ntp_flow_mixture_cdf: too many times";
            return NTP_ERR_INVALID;
        }
        cudaError_t e = cudaSuccess;
        with_bins(f->K, [&](auto kc) {
            constexpr int K = decltype(kc)::value;
            ntp::mixture_total_kernel<<<1, 1024, 0, st>>>(f->knots, f->L, K, n_cond, d_w, d_total);
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(ntp::mixture_cdf_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
            if (e == cudaSuccess) {
                ntp::mixture_cdf_kernel<K><<<static_cast<unsigned>(blocks), 256, smem, st>>>(
                    f->knots, f->L, n_cond, d_w, d_off, d_t, n_times, d_total, d_out);
                e = cudaGetLastError();
            }
        });
        if (e != cudaSuccess) return ferr(f, e, "ntp_flow_mixture_cdf");
        if (!on_device) F_CUDA(f, cudaMemcpyAsync(cdf, d_out, sizeof(double) * n_times, cudaMemcpyDeviceToHost, st));
        F_CUDA(f, cudaStreamSynchronize(st));
        return NTP_OK;
    };
    const ntp_status s2 = run();
    cudaFree(stage);
    return s2;
}

}  // extern "C"
