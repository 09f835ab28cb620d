// noalloc.cu -- ntp_propagate_noalloc: photon propagation without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Some programs that embed this library own all device memory themselves: an
// online trigger or data-acquisition process that reserves its device memory
// at start-up and must not allocate while taking data (cudaMalloc
// synchronises the device and can fail once memory is fragmented), or a host
// framework whose buffers come from its own pool or arena allocator.  Such a
// caller can hand over the hit buffer it already owns, but cannot let the
// library obtain more device memory.  This entry point therefore keeps the
// kernel's scratch memory -- the photon / hit counters, the source table and
// its prefix sums, the interleaved medium table, the spectrum knots and the
// target table -- in one file-scope __device__ array of fixed size, and
// allocates nothing: no context, no stream, no cudaMalloc / cudaFree, no host
// heap (the host-side packing uses fixed stack buffers).
//
// Limits (scratch of kScratchBytes = 256 KiB, held by every GPU that loads
// the library until the process exits): at most kMaxSources sources,
// kMaxTargets targets, NTP_MAX_MEDIUM_KNOTS medium knots and
// NTP_MAX_SPECTRUM_KNOTS spectrum knots.  Larger inputs are rejected with
// NTP_ERR_INVALID.  Targets are tested one by one at every step (no column
// culling or grid walk), which gives the same hits as ntp_propagate but costs
// a sphere test per target and step: on a string of 20 modules this is a few
// per cent, on thousands of modules many times ntp_propagate's time.
//
// The scratch is shared by every call on a device and keeps the last call's
// contents; each call rewrites all of it that the kernel reads and zeroes the
// counters first.  Calls that overlap on the GPU (different host threads or
// different streams) race on the scratch and must be serialised by the caller.
// The first call on a device looks up the scratch's device address there
// (cudaGetSymbolAddress); that first call should come before any stream
// capture on that device.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "ntp_internal.h"

namespace {

constexpr size_t kScratchBytes = 256 * 1024;
constexpr int kMaxSources = 1024;
constexpr int kMaxTargets = 4096;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffCounters = 0;  // 4 x u64
constexpr size_t kOffSources = 256;
constexpr size_t kOffPrefix = align256(kOffSources + sizeof(ntp_source) * kMaxSources);
constexpr size_t kOffMedium = align256(kOffPrefix + sizeof(unsigned long long) * (kMaxSources + 1));
constexpr size_t kOffSpectrum = align256(kOffMedium + sizeof(float4) * NTP_MAX_MEDIUM_KNOTS);
constexpr size_t kOffTargets = align256(kOffSpectrum + sizeof(float) * NTP_MAX_SPECTRUM_KNOTS);
constexpr size_t kOffIds = align256(kOffTargets + sizeof(float4) * kMaxTargets);
constexpr size_t kEnd = kOffIds + sizeof(uint32_t) * kMaxTargets;
static_assert(kEnd <= kScratchBytes, "scratch layout exceeds the scratch array");

// The scratch.  Host code never uses this name as an address: it is a
// host-side stand-in for the device symbol; the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

unsigned char* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// the error slot of context-free calls on this thread (ntp_last_error(NULL))
thread_local char g_err[256];

ntp_status fail(ntp_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return st;
}

#define NA_CUDA(call)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) return fail(NTP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

}  // namespace

namespace ntp {

void set_free_error(const char* msg) { std::snprintf(g_err, sizeof(g_err), "%s", msg ? msg : ""); }
const char* free_error() { return g_err; }

}  // namespace ntp

extern "C" ntp_status ntp_propagate_noalloc(const ntp_medium_desc* m, const ntp_spectrum_desc* sp,
                                             const ntp_target* targets, int32_t n_targets,
                                             const ntp_source* sources, int32_t n_sources, uint64_t seed,
                                             const ntp_prop_opts* opts, ntp_hit* hits, uint64_t capacity,
                                             uint64_t* n_hits, uint64_t* n_photons_simulated) {
    g_err[0] = '\0';
    if (n_hits) *n_hits = 0;
    if (n_photons_simulated) *n_photons_simulated = 0;
    if (const char* why = ntp::check_medium(m, false)) return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: %s", why);
    if (const char* why = ntp::check_spectrum(sp)) return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: %s", why);
    if (n_sources < 0 || n_sources > kMaxSources || (n_sources > 0 && !sources))
        return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: n_sources must be in [0, %d]", kMaxSources);
    if (n_targets < 0 || n_targets > kMaxTargets || (n_targets > 0 && !targets))
        return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: n_targets must be in [0, %d]", kMaxTargets);
    int spec_n = 0;
    float p0 = 0.0f, p1 = 0.0f;
    switch (sp->kind) {
    case NTP_SPEC_MONOCHROMATIC:
        p0 = sp->wavelength;
        break;
    case NTP_SPEC_TABLE_LINEAR:
    case NTP_SPEC_TABLE_TEXTURE:
        spec_n = sp->n_knots;
        break;
    default:  // NTP_SPEC_INV_SQUARE
        p0 = 1.0f / sp->wl_min;
        p1 = 1.0f / sp->wl_min - 1.0f / sp->wl_max;
        break;
    }
    ntp_prop_opts o{15, NTP_HIT_FIRST_IN_LIST, 0, 0, nullptr};
    if (opts) o = *opts;
    if (o.max_steps < 1 || o.max_steps > (1 << 24) ||
        (o.hit_policy != NTP_HIT_FIRST_IN_LIST && o.hit_policy != NTP_HIT_NEAREST))
        return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: bad options");
    if (capacity > 0 && (!hits || (reinterpret_cast<uintptr_t>(hits) & 15u)))
        return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: hits must be a 16-byte aligned device pointer");
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: device index too large");
    if (capacity > 0) {
        cudaPointerAttributes attr{};
        if (cudaPointerGetAttributes(&attr, hits) != cudaSuccess ||
            (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: hits is not device memory");
        }
        // the kernel runs on the current device: a buffer on another GPU would
        // be written through peer memory
        if (attr.type == cudaMemoryTypeDevice && attr.device != dev)
            return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: hits is on device %d, the current device is %d",
                        attr.device, dev);
    }
    unsigned long long prefix[kMaxSources + 1];
    prefix[0] = 0;
    for (int i = 0; i < n_sources; ++i) {
        const ntp_source& s = sources[i];
        if (s.kind < NTP_SRC_POINT_ISOTROPIC || s.kind > NTP_SRC_CHERENKOV_TRACK)
            return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: source %d has an unknown kind", i);
        if (s.kind == NTP_SRC_EXTENDED_CHERENKOV && s.photons > 0 &&
            (!(s.long_a > 1.0f) || !(s.long_b > 0.0f) || !(s.long_lrad > 0.0f)))
            return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: extended source %d needs long_a > 1, long_b > 0, "
                        "long_lrad > 0", i);
        if (prefix[i] + s.photons < prefix[i]) return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: photon count overflows");
        prefix[i + 1] = prefix[i] + s.photons;
    }
    for (int i = 0; i < n_targets; ++i)
        if (!(targets[i].radius > 0.0f) || !finite3(targets[i].position))
            return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: target %d has a bad position or radius", i);
    const unsigned long long total = prefix[n_sources];
    if (total == 0) return NTP_OK;

    // one-time set-up per device: the scratch's device address
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void* ptr = nullptr;
            NA_CUDA(cudaGetSymbolAddress(&ptr, g_scratch));
            g_scratch_ptr[dev] = static_cast<unsigned char*>(ptr);
        }
        base = g_scratch_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(o.stream);

    // inputs into the scratch (pageable copies; fixed host buffers only)
    unsigned long long* d_counters = reinterpret_cast<unsigned long long*>(base + kOffCounters);
    NA_CUDA(cudaMemsetAsync(d_counters, 0, 4 * sizeof(unsigned long long), st));
    NA_CUDA(cudaMemcpyAsync(base + kOffSources, sources, sizeof(ntp_source) * n_sources, cudaMemcpyHostToDevice, st));
    NA_CUDA(cudaMemcpyAsync(base + kOffPrefix, prefix, sizeof(unsigned long long) * (n_sources + 1),
                            cudaMemcpyHostToDevice, st));
    float4 buf[256];
    for (int i0 = 0; i0 < m->n_knots; i0 += 256) {
        const int n = m->n_knots - i0 < 256 ? m->n_knots - i0 : 256;
        for (int k = 0; k < n; ++k) {
            const int i = i0 + k;
            buf[k] = make_float4(m->ref_index[i], m->group_velocity[i], m->scattering_length[i], 0.0f);
        }
        NA_CUDA(cudaMemcpyAsync(base + kOffMedium + sizeof(float4) * i0, buf, sizeof(float4) * n,
                                cudaMemcpyHostToDevice, st));
    }
    if (spec_n > 0)
        NA_CUDA(cudaMemcpyAsync(base + kOffSpectrum, sp->icdf_knots, sizeof(float) * spec_n, cudaMemcpyHostToDevice, st));
    uint32_t ids[256];
    for (int i0 = 0; i0 < n_targets; i0 += 256) {
        const int n = n_targets - i0 < 256 ? n_targets - i0 : 256;
        for (int k = 0; k < n; ++k) {
            const ntp_target& t = targets[i0 + k];
            buf[k] = make_float4(t.position[0], t.position[1], t.position[2], t.radius * t.radius);
            ids[k] = t.module_id;
        }
        NA_CUDA(cudaMemcpyAsync(base + kOffTargets + sizeof(float4) * i0, buf, sizeof(float4) * n,
                                cudaMemcpyHostToDevice, st));
        NA_CUDA(cudaMemcpyAsync(base + kOffIds + sizeof(uint32_t) * i0, ids, sizeof(uint32_t) * n,
                                cudaMemcpyHostToDevice, st));
    }

    ntp::PropParams p{};
    p.sources = reinterpret_cast<const ntp_source*>(base + kOffSources);
    p.prefix = reinterpret_cast<const unsigned long long*>(base + kOffPrefix);
    p.n_src = n_sources;
    p.total = total;
    p.targets = reinterpret_cast<const float4*>(base + kOffTargets);
    p.target_ids = reinterpret_cast<const uint32_t*>(base + kOffIds);
    p.n_targets = n_targets;
    p.targets_in_smem = 1;
    p.columns_in_smem = 0;
    p.columns = nullptr;
    p.members = nullptr;
    p.n_columns = 0;
    p.cell_start = nullptr;
    p.cell_items = nullptr;
    p.medium = reinterpret_cast<const float4*>(base + kOffMedium);
    p.n_medium = m->n_knots;
    p.wl_min = m->wl_min;
    p.medium_scale = static_cast<float>(m->n_knots - 1) / (m->wl_max - m->wl_min);
    p.spec_kind = sp->kind;
    p.n_spec = spec_n;
    p.spec_knots = reinterpret_cast<const float*>(base + kOffSpectrum);
    p.spec_p0 = p0;
    p.spec_p1 = p1;
    p.hg_g = m->hg_g;
    ntp::set_rayleigh(p, m->rayleigh_fraction);
    p.max_steps = o.max_steps;
    p.hit_policy = o.hit_policy;
    p.exact_pole = (o.flags & NTP_FLAG_EXACT_POLE_ROTATION) ? 1 : 0;
    ntp::set_key(p, seed);
    p.hits = hits;
    p.capacity = capacity;
    p.counters = d_counters;
    p.refill_min = 8;

    int per_sm = 0, n_sms = 0;
    NA_CUDA(cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev));
    NA_CUDA(ntp::propagate_occupancy(p, &per_sm));
    if (per_sm < 1) return fail(NTP_ERR_INVALID, "ntp_propagate_noalloc: kernel does not fit on an SM");
    const int grid = per_sm * n_sms;
    const unsigned long long warps = static_cast<unsigned long long>(grid) * (ntp::kPropBlock / 32);
    unsigned long long chunk = total / (warps * 8);
    chunk = chunk < 32 ? 32 : (chunk > 4096 ? 4096 : chunk);
    p.chunk = (chunk + 31) / 32 * 32;
    NA_CUDA(ntp::launch_propagate(p, grid, st));

    unsigned long long counters[4];
    NA_CUDA(cudaMemcpyAsync(counters, d_counters, sizeof(counters), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    if (n_hits) *n_hits = counters[1];
    if (n_photons_simulated) *n_photons_simulated = counters[2];
    if (counters[1] > capacity)
        return fail(NTP_ERR_OVERFLOW, "ntp_propagate_noalloc: hit buffer overflow (%llu hits, capacity %llu)",
                    counters[1], static_cast<unsigned long long>(capacity));
    return NTP_OK;
}
