// surrogate.cu -- flow conditions of (event, module, PMT) triples.
//
// For each event (a cascade: position, direction, log10 E) and each
// multi-PMT module of the context within [d_min, d_max] of it, one row per
// PMT with the condition features of the flow (the same mapping as the
// training tables: 2 ln(d)/ln(200) - 1, v.u, a.u, phi/pi - 1, (log10 E - 4)/2
// with u the unit vector module -> source, v the source direction, a the PMT
// axis and phi the angle around u from the projection of v to that of a), a
// 64-bit stream key (event id, module, PMT) for the sampler, and the
// geometric time (|source - module| - R) n800 / c that turns a time residual
// into a time (calc_time_residual!, photon_prop_cuda.jl:906-924).  Modules are
// upright (PMT axes straight from the coordinate table).  Rows are grouped
// by event; modules closer than d_min are counted per event (outside the
// flow's domain).
#include <cuda_runtime.h>

#include "ntp_device.cuh"
#include "ntp_internal.h"

namespace ntp {

namespace {

constexpr int kBlock = 256;

struct EventIn {
    float px, py, pz, dx, dy, dz, log10e;
    uint32_t id;
};

__global__ void count_kernel(const EventIn* __restrict__ ev, int n_events, const float4* __restrict__ tg,
                             const int* __restrict__ kind, const int* __restrict__ npmt, int n_targets, float d_min,
                             float d_max, unsigned long long* __restrict__ ev_rows, int* __restrict__ ev_close) {
    const long long total = static_cast<long long>(n_events) * n_targets;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int e = static_cast<int>(i / n_targets), k = static_cast<int>(i % n_targets);
        if (kind[k] != NTP_TARGET_MULTI_PMT) continue;
        const float4 c = tg[k];
        const float rx = ev[e].px - c.x, ry = ev[e].py - c.y, rz = ev[e].pz - c.z;
        const float d = sqrtf(rx * rx + ry * ry + rz * rz);
        if (d < d_min) atomicAdd(ev_close + e, 1);
        else if (d <= d_max) atomicAdd(ev_rows + e, static_cast<unsigned long long>(npmt[k]));
    }
}

__global__ void fill_kernel(const EventIn* __restrict__ ev, int n_events, const float4* __restrict__ tg,
                            const float* __restrict__ radius, const int* __restrict__ kind, const int* __restrict__ npmt,
                            const int* __restrict__ pmt_off, const float* __restrict__ axes, int n_targets, float d_min,
                            float d_max, float tgeo_scale, const unsigned long long* __restrict__ ev_first,
                            unsigned long long* __restrict__ ev_fill, float* __restrict__ cond,
                            unsigned long long* __restrict__ ckey, float* __restrict__ ctgeo, int32_t* __restrict__ cev,
                            int32_t* __restrict__ ctgt, int32_t* __restrict__ cpmt) {
    const long long total = static_cast<long long>(n_events) * n_targets;
    const float inv_ln200 = 1.0f / logf(200.0f);
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int e = static_cast<int>(i / n_targets), k = static_cast<int>(i % n_targets);
        if (kind[k] != NTP_TARGET_MULTI_PMT) continue;
        const float4 c = tg[k];
        const EventIn E = ev[e];
        const float rx = E.px - c.x, ry = E.py - c.y, rz = E.pz - c.z;
        const float d = sqrtf(rx * rx + ry * ry + rz * rz);
        if (d < d_min || d > d_max) continue;
        const int np = npmt[k], off = pmt_off[k];
        const unsigned long long base = ev_first[e] + atomicAdd(ev_fill + e, static_cast<unsigned long long>(np));
        const float ux = rx / d, uy = ry / d, uz = rz / d;
        const float vu = E.dx * ux + E.dy * uy + E.dz * uz;
        const float e1x = E.dx - vu * ux, e1y = E.dy - vu * uy, e1z = E.dz - vu * uz;
        const float f0 = 2.0f * logf(d) * inv_ln200 - 1.0f, f4 = (E.log10e - 4.0f) * 0.5f;
        const float tgeo = (d - radius[k]) * tgeo_scale;
        for (int j = 0; j < np; ++j) {
            const float* a = axes + 3 * (off + j);
            const float au = a[0] * ux + a[1] * uy + a[2] * uz;
            const float e2x = a[0] - au * ux, e2y = a[1] - au * uy, e2z = a[2] - au * uz;
            const float cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
            float phi = atan2f(cx * ux + cy * uy + cz * uz, e1x * e2x + e1y * e2y + e1z * e2z);
            if (phi < 0.0f) phi += 6.283185307179586f;
            const unsigned long long r = base + j;
            float* f = cond + 5 * r;
            f[0] = f0;
            f[1] = vu;
            f[2] = au;
            f[3] = phi * 0.3183098861837907f - 1.0f;
            f[4] = f4;
            ckey[r] = (static_cast<unsigned long long>(E.id) << 32) | (static_cast<unsigned long long>(k) << 8) |
                      static_cast<unsigned long long>(j);
            if (ctgeo) ctgeo[r] = tgeo;
            if (cev) cev[r] = e;
            if (ctgt) ctgt[r] = k;
            if (cpmt) cpmt[r] = j + 1;
        }
    }
}

int grid_for(long long n) {
    long long g = (n + kBlock - 1) / kBlock;
    return static_cast<int>(g < 1 ? 1 : (g > 65535ll * 8 ? 65535ll * 8 : g));
}

}  // namespace

cudaError_t launch_event_conditions_count(const void* events, int n_events, const float4* tg, const int* kind,
                                          const int* npmt, int n_targets, float d_min, float d_max,
                                          unsigned long long* ev_rows, int* ev_close, cudaStream_t st) {
    count_kernel<<<grid_for(static_cast<long long>(n_events) * n_targets), kBlock, 0, st>>>(
        static_cast<const EventIn*>(events), n_events, tg, kind, npmt, n_targets, d_min, d_max, ev_rows, ev_close);
    return cudaGetLastError();
}

cudaError_t launch_event_conditions_fill(const void* events, int n_events, const float4* tg, const float* radius,
                                         const int* kind, const int* npmt, const int* pmt_off, const float* axes,
                                         int n_targets, float d_min, float d_max, float tgeo_scale,
                                         const unsigned long long* ev_first, unsigned long long* ev_fill, float* cond,
                                         unsigned long long* ckey, float* ctgeo, int32_t* cev, int32_t* ctgt,
                                         int32_t* cpmt, cudaStream_t st) {
    fill_kernel<<<grid_for(static_cast<long long>(n_events) * n_targets), kBlock, 0, st>>>(
        static_cast<const EventIn*>(events), n_events, tg, radius, kind, npmt, pmt_off, axes, n_targets, d_min, d_max,
        tgeo_scale, ev_first, ev_fill, cond, ckey, ctgeo, cev, ctgt, cpmt);
    return cudaGetLastError();
}

size_t event_in_size() { return sizeof(EventIn); }

}  // namespace ntp
