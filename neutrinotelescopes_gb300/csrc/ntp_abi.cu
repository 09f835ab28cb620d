// ntp_abi.cu -- the extern "C" entry points of libntp.so (declared in
// include/ntp.h).  Owns the per-context device state: medium / spectrum /
// target tables (uploaded once by the ntp_set_* calls, like the arguments
// of PhotonPropSetup, photon_prop_cuda.jl:34-45), the launch scratch
// (photon / hit counters) and grow-only staging buffers for host-memory calls.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ntp_internal.h"

struct ntp_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    // medium
    bool have_medium = false;
    int n_med = 0;
    float wl_min = 0, wl_max = 0, hg_g = 0, f_ray = 0;
    float4* d_med = nullptr;
    int n_abs = 0;
    float* d_abs_wl = nullptr;
    float* d_abs_len = nullptr;

    // spectrum
    bool have_spec = false;
    int spec_kind = 0, n_spec = 0;
    float spec_p0 = 0, spec_p1 = 0;
    float* d_spec = nullptr;

    // targets
    bool have_targets = false;
    int n_tgt = 0;
    std::vector<ntp_target> targets;
    std::vector<float> pmt_coords;  // (theta, phi) pairs
    float4* d_tgt = nullptr;
    uint32_t* d_tgt_id = nullptr;
    uint2* d_sorted = nullptr;
    float* d_radius = nullptr;
    int* d_kind = nullptr;
    int* d_npmt = nullptr;
    int* d_pmtoff = nullptr;
    double* d_opening = nullptr;
    double* d_area = nullptr;
    ntp::Column* d_cols = nullptr;  // vertical columns of targets (culling)
    int* d_members = nullptr;
    int n_cols = 0;
    int* d_cell_start = nullptr;    // 2-D grid over the columns
    int* d_cell_items = nullptr;
    int grid_nx = 0, grid_ny = 0, n_cell_items = 0;
    float grid_x0 = 0, grid_y0 = 0, grid_h = 0;
    int grid_lattice = 0;     // every cell holds at most its centred column
    float lat_rcull2 = 0.0f;  // the largest r_cull^2
    double* d_axes = nullptr;  // PMT axes for the current orientation
    double* d_tgeo = nullptr;  // per-target tgeo for time residuals

    // wavelength acceptance
    int n_acc = 0;
    double* d_acc_wl = nullptr;
    double* d_acc = nullptr;

    // launch scratch
    unsigned long long* d_counters = nullptr;  // 4 words
    unsigned long long* h_counters = nullptr;  // pinned
    ntp_source* d_src = nullptr;
    size_t src_cap = 0;
    unsigned long long* d_prefix = nullptr;
    size_t prefix_cap = 0;

    ntp_run_stats stats{};

    // staging for host-buffer calls
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    void* d_stage2 = nullptr;
    size_t stage2_bytes = 0;
    void* d_scratch = nullptr;  // resampling work arrays
    size_t scratch_bytes = 0;
};

namespace {

#define NTP_CUDA(ctx, call)                                                                   \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
            return NTP_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

ntp_status invalid(ntp_ctx* ctx, const std::string& msg) {
    ctx->err = msg;
    return NTP_ERR_INVALID;
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

template <typename T>
cudaError_t dupload(T*& d, const T* h, size_t n, cudaStream_t s) {
    dfree(d);
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d), sizeof(T) * n);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

// Grow-only device buffer: reallocates (by at least 1.5x) when too small.
cudaError_t ensure(void*& d, size_t& cap, size_t bytes) {
    if (d && bytes <= cap) return cudaSuccess;
    const size_t want = std::max(bytes, cap + cap / 2);
    if (d) cudaFree(d);
    d = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&d, want);
    if (e == cudaSuccess) cap = want;
    return e;
}

bool finite(float x) { return std::isfinite(x); }

cudaStream_t pick_stream(ntp_ctx* ctx, void* s) { return s ? static_cast<cudaStream_t>(s) : ctx->stream; }

}  // namespace

namespace ntp {

bool fill_world_params(const ntp_ctx* ctx, PropParams& p) {
    if (!ctx->have_medium || !ctx->have_spec || !ctx->have_targets) return false;
    p.targets = ctx->d_tgt;
    p.target_ids = ctx->d_tgt_id;
    p.n_targets = ctx->n_tgt;
    p.columns = ctx->n_cols > 0 ? ctx->d_cols : nullptr;
    p.members = ctx->d_members;
    p.n_columns = ctx->n_cols;
    p.cell_start = p.columns ? ctx->d_cell_start : nullptr;
    p.cell_items = ctx->d_cell_items;
    p.grid_nx = ctx->grid_nx;
    p.grid_ny = ctx->grid_ny;
    p.n_cell_items = ctx->n_cell_items;
    p.grid_x0 = ctx->grid_x0;
    p.grid_y0 = ctx->grid_y0;
    p.grid_h = ctx->grid_h;
    p.grid_inv_h = ctx->grid_h > 0 ? 1.0f / ctx->grid_h : 0.0f;
    p.grid_lattice = ctx->grid_lattice;
    p.lat_rcull2 = ctx->lat_rcull2;
    p.medium = ctx->d_med;
    p.n_medium = ctx->n_med;
    p.wl_min = ctx->wl_min;
    p.medium_scale = static_cast<float>(ctx->n_med - 1) / (ctx->wl_max - ctx->wl_min);
    p.spec_kind = ctx->spec_kind;
    p.n_spec = ctx->n_spec;
    p.spec_knots = ctx->d_spec;
    p.spec_p0 = ctx->spec_p0;
    p.spec_p1 = ctx->spec_p1;
    p.hg_g = ctx->hg_g;
    ntp::set_rayleigh(p, ctx->f_ray);
    ntp::choose_staging(p);
    return true;
}

int ctx_device(const ntp_ctx* ctx) { return ctx->device; }
int ctx_num_sms(const ntp_ctx* ctx) { return ctx->num_sms; }
void set_ctx_error(ntp_ctx* ctx, const char* msg) { ctx->err = msg; }

}  // namespace ntp

namespace {

ntp::HitTargetTable hit_table(const ntp_ctx* ctx) {
    ntp::HitTargetTable t;
    t.sorted_ids = ctx->d_sorted;
    t.n_targets = ctx->n_tgt;
    t.targets = ctx->d_tgt;
    t.radius = ctx->d_radius;
    t.kind = ctx->d_kind;
    t.n_pmts = ctx->d_npmt;
    t.pmt_offset = ctx->d_pmtoff;
    t.opening = ctx->d_opening;
    t.area_acc = ctx->d_area;
    return t;
}

}  // namespace

namespace ntp {

const char* check_medium(const ntp_medium_desc* m, bool need_absorption) {
    if (!m) return "medium is NULL";
    if (m->n_knots < 2 || m->n_knots > NTP_MAX_MEDIUM_KNOTS) return "n_knots must be in [2, NTP_MAX_MEDIUM_KNOTS]";
    if (!m->ref_index || !m->group_velocity || !m->scattering_length) return "a medium table is NULL";
    if (!(m->wl_max > m->wl_min) || !finite(m->wl_min) || !finite(m->wl_max)) return "need wl_max > wl_min";
    if (!finite(m->hg_g) || !(m->hg_g > -1.0f && m->hg_g < 1.0f)) return "hg_g must lie in (-1, 1)";
    if (!(m->rayleigh_fraction >= 0.0f && m->rayleigh_fraction <= 1.0f)) return "rayleigh_fraction must lie in [0, 1]";
    for (int i = 0; i < m->n_knots; ++i) {
        const float n = m->ref_index[i], vg = m->group_velocity[i], ls = m->scattering_length[i];
        if (!(n > 1.0f) || !(vg > 0.0f) || !(ls > 0.0f) || !finite(n) || !finite(vg) || !finite(ls))
            return "need n > 1, group velocity > 0, scattering length > 0 (finite) at every knot";
    }
    if (!need_absorption) return nullptr;
    if (m->n_abs_knots < 2 || m->n_abs_knots > NTP_MAX_ABS_KNOTS || !m->abs_wavelength || !m->abs_length)
        return "absorption table needs 2..NTP_MAX_ABS_KNOTS knots";
    for (int i = 0; i < m->n_abs_knots; ++i) {
        if (i && !(m->abs_wavelength[i] > m->abs_wavelength[i - 1])) return "absorption wavelengths must ascend";
        if (!(m->abs_length[i] > 0.0f)) return "absorption length must be > 0";
    }
    return nullptr;
}

const char* check_spectrum(const ntp_spectrum_desc* s) {
    if (!s) return "spectrum is NULL";
    switch (s->kind) {
    case NTP_SPEC_MONOCHROMATIC:
        return s->wavelength > 0.0f && finite(s->wavelength) ? nullptr : "wavelength must be > 0";
    case NTP_SPEC_TABLE_LINEAR:
    case NTP_SPEC_TABLE_TEXTURE:
        if (s->n_knots < 2 || s->n_knots > NTP_MAX_SPECTRUM_KNOTS || !s->icdf_knots)
            return "table needs 2..NTP_MAX_SPECTRUM_KNOTS knots";
        for (int i = 0; i < s->n_knots; ++i)
            if (!(s->icdf_knots[i] > 0.0f) || !finite(s->icdf_knots[i])) return "knots must be finite wavelengths > 0";
        return nullptr;
    case NTP_SPEC_INV_SQUARE:
        return s->wl_min > 0.0f && s->wl_max > s->wl_min && finite(s->wl_max) ? nullptr : "need 0 < wl_min < wl_max";
    default:
        return "unknown kind";
    }
}

}  // namespace ntp

extern "C" {

int ntp_abi_version(void) { return NTP_ABI_VERSION; }

ntp_status ntp_create(int device, ntp_ctx** out) {
    ntp::set_free_error("");
    if (!out) return NTP_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        ntp::set_free_error(e != cudaSuccess ? (std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e)).c_str()
                                             : "device index out of range");
        return e != cudaSuccess ? NTP_ERR_CUDA : NTP_ERR_INVALID;
    }
    ntp_ctx* ctx = new ntp_ctx();
    ctx->device = device;
    auto fail = [&](cudaError_t err, const char* what) {
        ntp::set_free_error((std::string(what) + ": " + cudaGetErrorString(err)).c_str());
        ntp_destroy(ctx);
        return NTP_ERR_CUDA;
    };
    if ((e = cudaSetDevice(device)) != cudaSuccess) return fail(e, "cudaSetDevice");
    if ((e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
        return fail(e, "cudaDeviceGetAttribute");
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(e, "cudaStreamCreate");
    if ((e = cudaMalloc(&ctx->d_counters, 4 * sizeof(unsigned long long))) != cudaSuccess)
        return fail(e, "cudaMalloc");
    if ((e = cudaMallocHost(&ctx->h_counters, 4 * sizeof(unsigned long long))) != cudaSuccess)
        return fail(e, "cudaMallocHost");
    *out = ctx;
    return NTP_OK;
}

void ntp_destroy(ntp_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    dfree(ctx->d_med);
    dfree(ctx->d_abs_wl);
    dfree(ctx->d_abs_len);
    dfree(ctx->d_spec);
    dfree(ctx->d_tgt);
    dfree(ctx->d_tgt_id);
    dfree(ctx->d_sorted);
    dfree(ctx->d_radius);
    dfree(ctx->d_kind);
    dfree(ctx->d_npmt);
    dfree(ctx->d_pmtoff);
    dfree(ctx->d_opening);
    dfree(ctx->d_area);
    dfree(ctx->d_axes);
    dfree(ctx->d_tgeo);
    dfree(ctx->d_cols);
    dfree(ctx->d_members);
    dfree(ctx->d_cell_start);
    dfree(ctx->d_cell_items);
    dfree(ctx->d_acc_wl);
    dfree(ctx->d_acc);
    dfree(ctx->d_counters);
    dfree(ctx->d_src);
    dfree(ctx->d_prefix);
    if (ctx->d_stage) cudaFree(ctx->d_stage);
    if (ctx->d_stage2) cudaFree(ctx->d_stage2);
    if (ctx->d_scratch) cudaFree(ctx->d_scratch);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* ntp_last_error(const ntp_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    return ntp::free_error();
}

ntp_status ntp_set_medium(ntp_ctx* ctx, const ntp_medium_desc* m) {
    if (!ctx) return NTP_ERR_INVALID;
    if (const char* why = ntp::check_medium(m, true)) return invalid(ctx, std::string("ntp_set_medium: ") + why);
    std::vector<float4> tab(m->n_knots);
    for (int i = 0; i < m->n_knots; ++i)
        tab[i] = make_float4(m->ref_index[i], m->group_velocity[i], m->scattering_length[i], 0.0f);
    cudaSetDevice(ctx->device);
    NTP_CUDA(ctx, dupload(ctx->d_med, tab.data(), tab.size(), ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_abs_wl, m->abs_wavelength, m->n_abs_knots, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_abs_len, m->abs_length, m->n_abs_knots, ctx->stream));
    ctx->n_med = m->n_knots;
    ctx->wl_min = m->wl_min;
    ctx->wl_max = m->wl_max;
    ctx->n_abs = m->n_abs_knots;
    ctx->hg_g = m->hg_g;
    ctx->f_ray = m->rayleigh_fraction;
    ctx->have_medium = true;
    return NTP_OK;
}

ntp_status ntp_set_spectrum(ntp_ctx* ctx, const ntp_spectrum_desc* s) {
    if (!ctx) return NTP_ERR_INVALID;
    if (const char* why = ntp::check_spectrum(s)) return invalid(ctx, std::string("ntp_set_spectrum: ") + why);
    cudaSetDevice(ctx->device);
    switch (s->kind) {
    case NTP_SPEC_MONOCHROMATIC:
        dfree(ctx->d_spec);
        ctx->n_spec = 0;
        ctx->spec_p0 = s->wavelength;
        ctx->spec_p1 = 0;
        break;
    case NTP_SPEC_TABLE_LINEAR:
    case NTP_SPEC_TABLE_TEXTURE:
        NTP_CUDA(ctx, dupload(ctx->d_spec, s->icdf_knots, s->n_knots, ctx->stream));
        ctx->n_spec = s->n_knots;
        break;
    default:  // NTP_SPEC_INV_SQUARE
        dfree(ctx->d_spec);
        ctx->n_spec = 0;
        ctx->spec_p0 = 1.0f / s->wl_min;
        ctx->spec_p1 = 1.0f / s->wl_min - 1.0f / s->wl_max;
        break;
    }
    ctx->spec_kind = s->kind;
    ctx->have_spec = true;
    return NTP_OK;
}

ntp_status ntp_set_targets(ntp_ctx* ctx, const ntp_target* t, int32_t n, const float* pmt_coords,
                           int32_t n_pmt_coords) {
    if (!ctx) return NTP_ERR_INVALID;
    if (n < 0 || (n > 0 && !t)) return invalid(ctx, "ntp_set_targets: bad target array");
    if (n_pmt_coords < 0 || (n_pmt_coords > 0 && !pmt_coords))
        return invalid(ctx, "ntp_set_targets: bad PMT coordinate table");
    std::vector<float4> tg(n);
    std::vector<uint32_t> ids(n);
    std::vector<uint2> sorted(n);
    std::vector<float> radius(n);
    std::vector<int> kind(n), npmt(n), off(n);
    std::vector<double> opening(n), area(n);
    for (int i = 0; i < n; ++i) {
        const ntp_target& x = t[i];
        if (!(x.radius > 0.0f) || !finite(x.radius) || !finite(x.position[0]) || !finite(x.position[1]) ||
            !finite(x.position[2]))
            return invalid(ctx, "ntp_set_targets: target " + std::to_string(i) + " has a bad position or radius");
        if (x.kind != NTP_TARGET_SPHERE && x.kind != NTP_TARGET_MULTI_PMT)
            return invalid(ctx, "ntp_set_targets: unknown target kind");
        if (x.kind == NTP_TARGET_MULTI_PMT &&
            (x.n_pmts < 0 || x.pmt_offset < 0 || static_cast<long long>(x.pmt_offset) + x.n_pmts > n_pmt_coords))
            return invalid(ctx, "ntp_set_targets: PMT layout outside the coordinate table");
        tg[i] = make_float4(x.position[0], x.position[1], x.position[2], x.radius * x.radius);
        ids[i] = x.module_id;
        sorted[i] = make_uint2(x.module_id, static_cast<unsigned>(i));
        radius[i] = x.radius;
        kind[i] = x.kind;
        npmt[i] = x.kind == NTP_TARGET_MULTI_PMT ? x.n_pmts : 0;
        off[i] = x.kind == NTP_TARGET_MULTI_PMT ? x.pmt_offset : 0;
        // check_pmt_hit, detection.jl:94-95: opening angle in Float32
        const float pmt_radius = std::sqrt(x.pmt_area / static_cast<float>(M_PI));
        opening[i] = static_cast<double>(std::asin(pmt_radius / x.radius));
        // area_acceptance, detection.jl:139-146
        if (x.kind == NTP_TARGET_SPHERE) {
            const float total_pmt_area = static_cast<float>(x.n_pmts) * x.pmt_area;
            const float r2 = x.radius * x.radius;
            area[i] = static_cast<double>(total_pmt_area) / (4.0 * M_PI * static_cast<double>(r2));
        } else {
            area[i] = 1.0;
        }
    }
    std::sort(sorted.begin(), sorted.end(), [](uint2 a, uint2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); });
    for (int i = 1; i < n; ++i)
        if (sorted[i].x == sorted[i - 1].x)
            return invalid(ctx, "ntp_set_targets: duplicate module_id " + std::to_string(sorted[i].x));
    // vertical columns: targets with the same (x, y), sorted by z
    std::vector<ntp::Column> cols;
    std::vector<int> members;
    {
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int a, int b) {
            const ntp_target &A = t[a], &B = t[b];
            if (A.position[0] != B.position[0]) return A.position[0] < B.position[0];
            if (A.position[1] != B.position[1]) return A.position[1] < B.position[1];
            if (A.position[2] != B.position[2]) return A.position[2] < B.position[2];
            return a < b;
        });
        for (int i = 0; i < n;) {
            int j = i;
            while (j < n && t[order[j]].position[0] == t[order[i]].position[0] &&
                   t[order[j]].position[1] == t[order[i]].position[1])
                ++j;
            ntp::Column c{};
            c.cx = t[order[i]].position[0];
            c.cy = t[order[i]].position[1];
            c.first = static_cast<int>(members.size());
            c.count = j - i;
            c.z0 = t[order[i]].position[2];
            c.z_last = t[order[j - 1]].position[2];
            float rmax = 0.0f;
            for (int k = i; k < j; ++k) {
                rmax = std::max(rmax, t[order[k]].radius);
                members.push_back(order[k]);
            }
            c.r_cull = rmax * (1.0f + 1e-6f) + 0.02f;
            c.dz = 0.0f;
            if (c.count > 1) {
                const double step = (static_cast<double>(c.z_last) - c.z0) / (c.count - 1);
                bool uniform = step > 0;
                for (int k = i + 1; k < j && uniform; ++k) {
                    const double want = c.z0 + step * (k - i);
                    uniform = std::fabs(t[order[k]].position[2] - want) <= 1e-5 * std::max(1.0, std::fabs(want));
                }
                if (uniform) c.dz = static_cast<float>(step);
            }
            cols.push_back(c);
            i = j;
        }
    }
    const bool use_cols = n >= 4 && 2 * static_cast<int>(cols.size()) <= n && static_cast<int>(cols.size()) <= ntp::kMaxSmemColumns;
    cudaSetDevice(ctx->device);
    dfree(ctx->d_cols);
    dfree(ctx->d_members);
    ctx->n_cols = 0;
    dfree(ctx->d_cell_start);
    dfree(ctx->d_cell_items);
    ctx->grid_nx = ctx->grid_ny = ctx->n_cell_items = 0;
    ctx->grid_lattice = 0;
    if (use_cols) {
        NTP_CUDA(ctx, dupload(ctx->d_cols, cols.data(), cols.size(), ctx->stream));
        NTP_CUDA(ctx, dupload(ctx->d_members, members.data(), members.size(), ctx->stream));
        ctx->n_cols = static_cast<int>(cols.size());
    }
    if (use_cols && static_cast<int>(cols.size()) >= ntp::kGridMinColumns) {
        // cells of side h over the axes' bounding box; each column goes into
        // every cell its culling disk, widened by 0.5 m, overlaps
        const float margin = 0.5f;
        double x0 = 1e30, y0 = 1e30, x1 = -1e30, y1 = -1e30, rmax = 0;
        for (const auto& c : cols) {
            x0 = std::min(x0, static_cast<double>(c.cx));
            x1 = std::max(x1, static_cast<double>(c.cx));
            y0 = std::min(y0, static_cast<double>(c.cy));
            y1 = std::max(y1, static_cast<double>(c.cy));
            rmax = std::max(rmax, static_cast<double>(c.r_cull));
        }
        // cell side: the median distance from a column to its nearest
        // neighbour (about one column per cell), grid shifted so that a
        // regular lattice of strings sits at cell centres
        std::vector<double> nn(cols.size(), 1e30);
        for (size_t a = 0; a < cols.size(); ++a)
            for (size_t b = 0; b < cols.size(); ++b)
                if (a != b) {
                    const double dx = cols[a].cx - cols[b].cx, dy = cols[a].cy - cols[b].cy;
                    nn[a] = std::min(nn[a], std::sqrt(dx * dx + dy * dy));
                }
        std::nth_element(nn.begin(), nn.begin() + nn.size() / 2, nn.end());
        double h = std::max(nn[nn.size() / 2], 2.0 * (rmax + margin));
        x0 -= h / 2; y0 -= h / 2; x1 += h / 2; y1 += h / 2;
        int nx = static_cast<int>(std::ceil((x1 - x0) / h)), ny = static_cast<int>(std::ceil((y1 - y0) / h));
        while (static_cast<long long>(nx) * ny > 65536) {
            h *= 1.5;
            nx = static_cast<int>(std::ceil((x1 - x0) / h));
            ny = static_cast<int>(std::ceil((y1 - y0) / h));
        }
        std::vector<std::vector<int>> cells(static_cast<size_t>(nx) * ny);
        for (int ci = 0; ci < static_cast<int>(cols.size()); ++ci) {
            const double r = cols[ci].r_cull + margin;
            const int ax = std::max(0, static_cast<int>(std::floor((cols[ci].cx - r - x0) / h)));
            const int bx = std::min(nx - 1, static_cast<int>(std::floor((cols[ci].cx + r - x0) / h)));
            const int ay = std::max(0, static_cast<int>(std::floor((cols[ci].cy - r - y0) / h)));
            const int by = std::min(ny - 1, static_cast<int>(std::floor((cols[ci].cy + r - y0) / h)));
            for (int iy = ay; iy <= by; ++iy)
                for (int ix = ax; ix <= bx; ++ix) cells[static_cast<size_t>(iy) * nx + ix].push_back(ci);
        }
        std::vector<int> start(cells.size() + 1, 0), items;
        for (size_t c = 0; c < cells.size(); ++c) {
            start[c] = static_cast<int>(items.size());
            items.insert(items.end(), cells[c].begin(), cells[c].end());
        }
        start[cells.size()] = static_cast<int>(items.size());
        NTP_CUDA(ctx, dupload(ctx->d_cell_start, start.data(), start.size(), ctx->stream));
        NTP_CUDA(ctx, dupload(ctx->d_cell_items, items.data(), items.size(), ctx->stream));
        ctx->grid_nx = nx;
        ctx->grid_ny = ny;
        ctx->n_cell_items = static_cast<int>(items.size());
        ctx->grid_x0 = static_cast<float>(x0);
        ctx->grid_y0 = static_cast<float>(y0);
        ctx->grid_h = static_cast<float>(h);
        // lattice mode: each cell lists at most one column, each column is
        // listed once, at the centre of its cell (within 1e-4 of the side)
        bool lattice = items.size() == cols.size();
        float rc2 = 0.0f;
        for (size_t c = 0; c < cells.size() && lattice; ++c) {
            if (cells[c].size() > 1) lattice = false;
            if (cells[c].size() == 1) {
                const ntp::Column& col = cols[cells[c][0]];
                const double cx = x0 + (static_cast<double>(c % nx) + 0.5) * h;
                const double cy = y0 + (static_cast<double>(c / nx) + 0.5) * h;
                if (std::fabs(col.cx - cx) > 1e-4 * h || std::fabs(col.cy - cy) > 1e-4 * h) lattice = false;
                rc2 = std::max(rc2, col.r_cull * col.r_cull);
            }
        }
        ctx->grid_lattice = lattice ? 1 : 0;
        ctx->lat_rcull2 = rc2;
    }
    NTP_CUDA(ctx, dupload(ctx->d_tgt, tg.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_tgt_id, ids.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_sorted, sorted.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_radius, radius.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_kind, kind.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_npmt, npmt.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_pmtoff, off.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_opening, opening.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_area, area.data(), n, ctx->stream));
    dfree(ctx->d_axes);
    dfree(ctx->d_tgeo);
    if (n_pmt_coords > 0) {
        NTP_CUDA(ctx, cudaMalloc(&ctx->d_axes, sizeof(double) * 3 * n_pmt_coords));
    }
    if (n > 0) {
        NTP_CUDA(ctx, cudaMalloc(&ctx->d_tgeo, sizeof(double) * n));
    }
    ctx->targets.assign(t, t + n);
    ctx->pmt_coords.assign(pmt_coords, pmt_coords + 2 * static_cast<size_t>(n_pmt_coords));
    ctx->n_tgt = n;
    ctx->have_targets = true;
    return NTP_OK;
}

ntp_status ntp_set_wavelength_acceptance(ntp_ctx* ctx, const double* wl, const double* acc, int32_t n) {
    if (!ctx) return NTP_ERR_INVALID;
    if (n < 2 || !wl || !acc) return invalid(ctx, "ntp_set_wavelength_acceptance: need >= 2 knots");
    std::vector<double> x(n), y(n);
    for (int i = 0; i < n; ++i) {
        if (i && !(wl[i] > wl[i - 1])) return invalid(ctx, "ntp_set_wavelength_acceptance: wavelengths must ascend");
        x[i] = wl[i];
        y[i] = acc[i];
    }
    cudaSetDevice(ctx->device);
    NTP_CUDA(ctx, dupload(ctx->d_acc_wl, x.data(), n, ctx->stream));
    NTP_CUDA(ctx, dupload(ctx->d_acc, y.data(), n, ctx->stream));
    ctx->n_acc = n;
    return NTP_OK;
}

ntp_status ntp_propagate(ntp_ctx* ctx, const ntp_source* sources, int32_t n_sources, uint64_t seed,
                         const ntp_prop_opts* opts, ntp_hit* hits, uint64_t capacity, int32_t hits_on_device,
                         uint64_t* n_hits, uint64_t* n_photons_simulated) {
    if (!ctx) return NTP_ERR_INVALID;
    if (!ctx->have_medium || !ctx->have_spec || !ctx->have_targets) {
        ctx->err = "ntp_propagate: medium, spectrum and targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (n_sources < 0 || (n_sources > 0 && !sources)) return invalid(ctx, "ntp_propagate: bad source array");
    if (capacity > 0 && !hits) return invalid(ctx, "ntp_propagate: hits is NULL with capacity > 0");
    ntp_prop_opts o{15, NTP_HIT_FIRST_IN_LIST, 0, 0, nullptr};
    if (opts) o = *opts;
    if (o.max_steps < 1 || o.max_steps > (1 << 24)) return invalid(ctx, "ntp_propagate: max_steps out of range");
    if (o.hit_policy != NTP_HIT_FIRST_IN_LIST && o.hit_policy != NTP_HIT_NEAREST)
        return invalid(ctx, "ntp_propagate: unknown hit_policy");
    if (hits_on_device && (reinterpret_cast<uintptr_t>(hits) & 15u))
        return invalid(ctx, "ntp_propagate: device hit buffer must be 16-byte aligned");

    std::vector<unsigned long long> prefix(static_cast<size_t>(n_sources) + 1, 0);
    for (int i = 0; i < n_sources; ++i) {
        const ntp_source& s = sources[i];
        if (s.kind < NTP_SRC_POINT_ISOTROPIC || s.kind > NTP_SRC_CHERENKOV_TRACK)
            return invalid(ctx, "ntp_propagate: source " + std::to_string(i) + " has an unknown kind");
        if (s.kind == NTP_SRC_EXTENDED_CHERENKOV && s.photons > 0 &&
            (!(s.long_a > 1.0f) || !(s.long_b > 0.0f) || !(s.long_lrad > 0.0f)))
            return invalid(ctx, "ntp_propagate: extended source needs long_a > 1, long_b > 0, long_lrad > 0");
        if (prefix[i] + s.photons < prefix[i]) return invalid(ctx, "ntp_propagate: photon count overflows");
        prefix[i + 1] = prefix[i] + s.photons;
    }
    const unsigned long long total = prefix.back();
    if (n_hits) *n_hits = 0;
    if (n_photons_simulated) *n_photons_simulated = 0;
    if (total == 0) return NTP_OK;

    cudaSetDevice(ctx->device);
    cudaStream_t st = hits_on_device ? pick_stream(ctx, o.stream) : ctx->stream;
    void* src_buf = ctx->d_src;
    NTP_CUDA(ctx, ensure(src_buf, ctx->src_cap, sizeof(ntp_source) * n_sources));
    ctx->d_src = static_cast<ntp_source*>(src_buf);
    void* pre_buf = ctx->d_prefix;
    NTP_CUDA(ctx, ensure(pre_buf, ctx->prefix_cap, sizeof(unsigned long long) * prefix.size()));
    ctx->d_prefix = static_cast<unsigned long long*>(pre_buf);
    NTP_CUDA(ctx, cudaMemcpyAsync(ctx->d_src, sources, sizeof(ntp_source) * n_sources, cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(ctx->d_prefix, prefix.data(), sizeof(unsigned long long) * prefix.size(),
                                  cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), st));

    ntp_hit* d_hits = hits;
    if (!hits_on_device) {
        NTP_CUDA(ctx, ensure(ctx->d_stage, ctx->stage_bytes, sizeof(ntp_hit) * std::max<uint64_t>(capacity, 1)));
        d_hits = static_cast<ntp_hit*>(ctx->d_stage);
    }

    ntp::PropParams p{};
    p.sources = ctx->d_src;
    p.prefix = ctx->d_prefix;
    p.n_src = n_sources;
    p.total = total;
    ntp::fill_world_params(ctx, p);
    if (o.flags & NTP_FLAG_PLAIN_SCAN) {
        p.columns = nullptr;
        p.cell_start = nullptr;
        ntp::choose_staging(p);
    }
    p.max_steps = o.max_steps;
    p.hit_policy = o.hit_policy;
    p.exact_pole = (o.flags & NTP_FLAG_EXACT_POLE_ROTATION) ? 1 : 0;
    ntp::set_key(p, seed);
    p.hits = d_hits;
    p.capacity = capacity;
    p.counters = ctx->d_counters;

    int per_sm = 0;
    NTP_CUDA(ctx, ntp::propagate_occupancy(p, &per_sm));
    if (per_sm < 1) {
        ctx->err = "ntp_propagate: kernel does not fit on an SM (too many targets or knots)";
        return NTP_ERR_INVALID;
    }
    const int grid = per_sm * ctx->num_sms;
    const unsigned long long warps = static_cast<unsigned long long>(grid) * (ntp::kPropBlock / 32);
    unsigned long long chunk = total / (warps * 8);
    chunk = std::max<unsigned long long>(32, std::min<unsigned long long>(4096, chunk));
    p.chunk = (chunk + 31) / 32 * 32;
    p.refill_min = 8;
    if (const char* env = std::getenv("NTP_REFILL_MIN")) p.refill_min = std::max(1, std::min(32, std::atoi(env)));

    NTP_CUDA(ctx, ntp::launch_propagate(p, grid, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, 4 * sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    const unsigned long long nh = ctx->h_counters[1];
    if (!hits_on_device && nh > 0 && capacity > 0) {
        const unsigned long long ncopy = std::min<unsigned long long>(nh, capacity);
        NTP_CUDA(ctx, cudaMemcpyAsync(hits, d_hits, sizeof(ntp_hit) * ncopy, cudaMemcpyDeviceToHost, st));
        NTP_CUDA(ctx, cudaStreamSynchronize(st));
    }
    if (n_hits) *n_hits = nh;
    if (n_photons_simulated) *n_photons_simulated = ctx->h_counters[2];
    ctx->stats.photons = ctx->h_counters[2];
    ctx->stats.hits = nh;
    ctx->stats.photon_steps = ctx->h_counters[3];
    ctx->stats.grid = grid;
    ctx->stats.block = ntp::kPropBlock;
    ctx->stats.chunk = p.chunk;
    if (nh > capacity) {
        ctx->err = "ntp_propagate: hit buffer overflow (" + std::to_string(nh) + " hits, capacity " +
                   std::to_string(capacity) + ")";
        return NTP_ERR_OVERFLOW;
    }
    return NTP_OK;
}

ntp_status ntp_get_run_stats(const ntp_ctx* ctx, ntp_run_stats* out) {
    if (!ctx || !out) return NTP_ERR_INVALID;
    *out = ctx->stats;
    return NTP_OK;
}

static ntp_status stage_hits(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, int on_device, cudaStream_t st,
                             const ntp_hit** d_hits) {
    if (on_device) {
        *d_hits = hits;
        return NTP_OK;
    }
    NTP_CUDA(ctx, ensure(ctx->d_stage, ctx->stage_bytes, sizeof(ntp_hit) * n));
    NTP_CUDA(ctx, cudaMemcpyAsync(ctx->d_stage, hits, sizeof(ntp_hit) * n, cudaMemcpyHostToDevice, st));
    *d_hits = static_cast<const ntp_hit*>(ctx->d_stage);
    return NTP_OK;
}

// PMT axes for an orientation: orientation * sph_to_cart(theta, phi), the
// spherical step in float as the coordinates are Float32 (detection.jl:60-70).
static ntp_status upload_axes(ntp_ctx* ctx, const double orientation[9], cudaStream_t st) {
    const int npc = static_cast<int>(ctx->pmt_coords.size() / 2);
    if (npc == 0) return NTP_OK;
    std::vector<double> axes(3 * static_cast<size_t>(npc));
    for (int j = 0; j < npc; ++j) {
        const float th = ctx->pmt_coords[2 * j], ph = ctx->pmt_coords[2 * j + 1];
        const float s_t = sinf(th), c_t = cosf(th), s_p = sinf(ph), c_p = cosf(ph);
        const double v[3] = {static_cast<double>(c_p * s_t), static_cast<double>(s_p * s_t), static_cast<double>(c_t)};
        for (int r = 0; r < 3; ++r)
            axes[3 * j + r] = orientation[3 * r] * v[0] + orientation[3 * r + 1] * v[1] + orientation[3 * r + 2] * v[2];
    }
    NTP_CUDA(ctx, cudaMemcpyAsync(ctx->d_axes, axes.data(), sizeof(double) * axes.size(), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

// tgeo per target, photon_prop_cuda.jl:913-914
static ntp_status upload_tgeo(ntp_ctx* ctx, const float src[3], float n800, cudaStream_t st) {
    std::vector<double> tgeo(ctx->n_tgt);
    const double c_vac = 0.299792458;
    for (int k = 0; k < ctx->n_tgt; ++k) {
        const ntp_target& t = ctx->targets[k];
        const float dx = src[0] - t.position[0], dy = src[1] - t.position[1], dz = src[2] - t.position[2];
        const float distance = std::sqrt(dx * dx + dy * dy + dz * dz);
        tgeo[k] = static_cast<double>(distance - t.radius) / (c_vac / static_cast<double>(n800));
    }
    if (!tgeo.empty())
        NTP_CUDA(ctx, cudaMemcpyAsync(ctx->d_tgeo, tgeo.data(), sizeof(double) * tgeo.size(), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

ntp_status ntp_make_hits(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, const double orientation[9],
                         int32_t* pmt_id, int32_t on_device, void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (!ctx->have_targets) {
        ctx->err = "ntp_make_hits: targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (n == 0) return NTP_OK;
    if (!hits || !pmt_id || !orientation) return invalid(ctx, "ntp_make_hits: NULL argument");
    cudaSetDevice(ctx->device);
    cudaStream_t st = on_device ? pick_stream(ctx, stream) : ctx->stream;
    ntp_status sa = upload_axes(ctx, orientation, st);
    if (sa != NTP_OK) return sa;
    const ntp_hit* d_hits = nullptr;
    ntp_status s = stage_hits(ctx, hits, n, on_device, st, &d_hits);
    if (s != NTP_OK) return s;
    int32_t* d_out = pmt_id;
    if (!on_device) {
        NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, sizeof(int32_t) * n));
        d_out = static_cast<int32_t*>(ctx->d_stage2);
    }
    NTP_CUDA(ctx, ntp::launch_make_hits(hit_table(ctx), d_hits, n, ctx->d_axes, d_out, st));
    if (!on_device) {
        NTP_CUDA(ctx, cudaMemcpyAsync(pmt_id, d_out, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    }
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

ntp_status ntp_calc_total_weight(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, double* area_acc, double* wl_acc,
                                 double* abs_weight, double* total, int32_t on_device, void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (!ctx->have_targets || !ctx->have_medium || ctx->n_acc < 2) {
        ctx->err = "ntp_calc_total_weight: targets, medium and wavelength acceptance must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (n == 0) return NTP_OK;
    if (!hits) return invalid(ctx, "ntp_calc_total_weight: hits is NULL");
    cudaSetDevice(ctx->device);
    cudaStream_t st = on_device ? pick_stream(ctx, stream) : ctx->stream;
    const ntp_hit* d_hits = nullptr;
    ntp_status s = stage_hits(ctx, hits, n, on_device, st, &d_hits);
    if (s != NTP_OK) return s;
    double* outs[4] = {area_acc, wl_acc, abs_weight, total};
    double* d_outs[4] = {area_acc, wl_acc, abs_weight, total};
    if (!on_device) {
        NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, 4 * sizeof(double) * n));
        for (int k = 0; k < 4; ++k) d_outs[k] = outs[k] ? static_cast<double*>(ctx->d_stage2) + k * n : nullptr;
    }
    NTP_CUDA(ctx, ntp::launch_total_weight(hit_table(ctx), d_hits, n, ctx->d_abs_wl, ctx->d_abs_len, ctx->n_abs,
                                           ctx->d_acc_wl, ctx->d_acc, ctx->n_acc, d_outs[0], d_outs[1],
                                           d_outs[2], d_outs[3], st));
    if (!on_device)
        for (int k = 0; k < 4; ++k)
            if (outs[k])
                NTP_CUDA(ctx, cudaMemcpyAsync(outs[k], d_outs[k], sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

ntp_status ntp_pmt_summary(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, const double orientation[9],
                           const ntp_summary_spec* spec, double* wsum, double* count, double* hist,
                           int32_t on_device, void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (!ctx->have_targets || !ctx->have_medium || ctx->n_acc < 2) {
        ctx->err = "ntp_pmt_summary: targets, medium and wavelength acceptance must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (!spec || !orientation) return invalid(ctx, "ntp_pmt_summary: NULL argument");
    int need = 1;
    for (const auto& t : ctx->targets) need = std::max(need, t.kind == NTP_TARGET_MULTI_PMT ? t.n_pmts : 1);
    if (spec->max_pmts < need) return invalid(ctx, "ntp_pmt_summary: max_pmts is below a target's PMT count");
    if (spec->n_bins < 0 || (spec->n_bins > 0 && (!hist || !(spec->t_max > spec->t_min))))
        return invalid(ctx, "ntp_pmt_summary: need t_max > t_min and time_hist when n_bins > 0");
    if (spec->use_time_residual && !(spec->n800 > 0.0f)) return invalid(ctx, "ntp_pmt_summary: n800 must be > 0");
    if (n > 0 && !hits) return invalid(ctx, "ntp_pmt_summary: hits is NULL");
    cudaSetDevice(ctx->device);
    cudaStream_t st = on_device ? pick_stream(ctx, stream) : ctx->stream;
    const size_t slots = static_cast<size_t>(ctx->n_tgt) * spec->max_pmts;
    const size_t nb = static_cast<size_t>(spec->n_bins);
    double* outs[3] = {wsum, count, hist};
    const size_t sizes[3] = {slots, slots, slots * nb};
    double* d_outs[3] = {wsum, count, hist};
    if (!on_device) {
        NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, sizeof(double) * (sizes[0] + sizes[1] + sizes[2] + 1)));
        double* base = static_cast<double*>(ctx->d_stage2);
        d_outs[0] = base;
        d_outs[1] = base + sizes[0];
        d_outs[2] = base + sizes[0] + sizes[1];
    }
    // outputs not wanted by the caller still receive the sums (scratch)
    for (int k = 0; k < 3; ++k)
        if (sizes[k] && d_outs[k]) NTP_CUDA(ctx, cudaMemsetAsync(d_outs[k], 0, sizeof(double) * sizes[k], st));
    if (n > 0) {
        ntp_status s0 = upload_axes(ctx, orientation, st);
        if (s0 != NTP_OK) return s0;
        if (spec->use_time_residual) {
            s0 = upload_tgeo(ctx, spec->source_position, spec->n800, st);
            if (s0 != NTP_OK) return s0;
        }
        const ntp_hit* d_hits = nullptr;
        s0 = stage_hits(ctx, hits, n, on_device, st, &d_hits);
        if (s0 != NTP_OK) return s0;
        if (!d_outs[0] || !d_outs[1]) {  // device call with NULL outputs: give them scratch
            NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, sizeof(double) * 2 * slots));
            double* base = static_cast<double*>(ctx->d_stage2);
            if (!d_outs[0]) { d_outs[0] = base; NTP_CUDA(ctx, cudaMemsetAsync(base, 0, sizeof(double) * slots, st)); }
            if (!d_outs[1]) { d_outs[1] = base + slots; NTP_CUDA(ctx, cudaMemsetAsync(base + slots, 0, sizeof(double) * slots, st)); }
        }
        NTP_CUDA(ctx, ntp::launch_pmt_summary(hit_table(ctx), d_hits, n, ctx->d_axes, ctx->d_abs_wl, ctx->d_abs_len,
                                              ctx->n_abs, ctx->d_acc_wl, ctx->d_acc, ctx->n_acc, ctx->d_tgeo,
                                              spec->use_time_residual, spec->max_pmts, spec->n_bins, spec->t_min,
                                              spec->t_max, d_outs[0], d_outs[1], d_outs[2], st));
    }
    if (!on_device)
        for (int k = 0; k < 3; ++k)
            if (outs[k] && sizes[k])
                NTP_CUDA(ctx, cudaMemcpyAsync(outs[k], d_outs[k], sizeof(double) * sizes[k], cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

ntp_status ntp_resample(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, const int32_t* pmt_id, const double* weight,
                        const double* time, int32_t max_pmts, double downsample, uint64_t seed, int32_t* out_group,
                        double* out_time, uint64_t* out_hit, uint64_t capacity, uint64_t* n_out, int32_t on_device,
                        void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (n_out) *n_out = 0;
    if (!ctx->have_targets) {
        ctx->err = "ntp_resample: targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (max_pmts < 1 || !(downsample >= 0.0)) return invalid(ctx, "ntp_resample: need max_pmts >= 1, downsample >= 0");
    if (n > 0 && (!hits || !pmt_id || !weight)) return invalid(ctx, "ntp_resample: NULL input");
    const long long G = static_cast<long long>(ctx->n_tgt) * max_pmts;
    if (G > (1ll << 26)) return invalid(ctx, "ntp_resample: too many (module, PMT) groups");
    if (n == 0 || G == 0) return NTP_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t st = on_device ? pick_stream(ctx, stream) : ctx->stream;
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    // inputs on the device
    const ntp_hit* d_hits = nullptr;
    ntp_status s0 = stage_hits(ctx, hits, n, on_device, st, &d_hits);
    if (s0 != NTP_OK) return s0;
    // scratch: group i32[n] | order u64[n] | okey u64[n] | pmt i32[n] | w f64[n] | t f64[n] |
    //          wsum f64[G] | npos, nall, nsel, fill u64[G] | start, out_start u64[G+1]
    const size_t nn = n, g = static_cast<size_t>(G);
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_group = take(4 * nn), o_order = take(8 * nn), o_okey = take(8 * nn);
    const size_t o_pmt = on_device ? 0 : take(4 * nn), o_w = on_device ? 0 : take(8 * nn);
    const size_t o_t = (on_device || !time) ? 0 : take(8 * nn);
    const size_t o_wsum = take(8 * g), o_npos = take(8 * g), o_nall = take(8 * g), o_nsel = take(8 * g);
    const size_t o_fill = take(8 * g), o_start = take(8 * (g + 1)), o_ostart = take(8 * (g + 1));
    NTP_CUDA(ctx, ensure(ctx->d_scratch, ctx->scratch_bytes, off));
    unsigned char* sc = static_cast<unsigned char*>(ctx->d_scratch);
    const int32_t* d_pmt = pmt_id;
    const double* d_w = weight;
    const double* d_t = time;
    if (!on_device) {
        NTP_CUDA(ctx, cudaMemcpyAsync(sc + o_pmt, pmt_id, 4 * nn, cudaMemcpyHostToDevice, st));
        NTP_CUDA(ctx, cudaMemcpyAsync(sc + o_w, weight, 8 * nn, cudaMemcpyHostToDevice, st));
        d_pmt = reinterpret_cast<const int32_t*>(sc + o_pmt);
        d_w = reinterpret_cast<const double*>(sc + o_w);
        if (time) {
            NTP_CUDA(ctx, cudaMemcpyAsync(sc + o_t, time, 8 * nn, cudaMemcpyHostToDevice, st));
            d_t = reinterpret_cast<const double*>(sc + o_t);
        }
    }
    auto u64p = [&](size_t o) { return reinterpret_cast<unsigned long long*>(sc + o); };
    int32_t* d_group = reinterpret_cast<int32_t*>(sc + o_group);
    double* d_wsum = reinterpret_cast<double*>(sc + o_wsum);
    NTP_CUDA(ctx, cudaMemsetAsync(sc + o_wsum, 0, o_start - o_wsum, st));  // wsum, npos, nall, nsel, fill
    NTP_CUDA(ctx, ntp::launch_resample_group(d_hits, n, d_pmt, d_w, ctx->d_sorted, ctx->n_tgt, max_pmts, d_group,
                                             d_wsum, u64p(o_npos), u64p(o_nall), st));
    NTP_CUDA(ctx, ntp::launch_resample_draw(static_cast<int>(G), d_wsum, u64p(o_npos), downsample, key,
                                            u64p(o_nsel), st));
    // bucket offsets and output offsets (prefix sums on the host)
    std::vector<unsigned long long> nall(g), nsel(g), start(g + 1), ostart(g + 1);
    NTP_CUDA(ctx, cudaMemcpyAsync(nall.data(), u64p(o_nall), 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(nsel.data(), u64p(o_nsel), 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    start[0] = ostart[0] = 0;
    for (size_t i = 0; i < g; ++i) {
        start[i + 1] = start[i] + nall[i];
        ostart[i + 1] = ostart[i] + nsel[i];
    }
    const unsigned long long total = ostart[g];
    if (n_out) *n_out = total;
    if (total > capacity) {
        ctx->err = "ntp_resample: output capacity " + std::to_string(capacity) + " below " + std::to_string(total);
        return NTP_ERR_OVERFLOW;
    }
    if (total == 0) return NTP_OK;
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_start), start.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_ostart), ostart.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, ntp::launch_resample_bucket(d_hits, n, d_group, d_w, key, u64p(o_start), u64p(o_fill),
                                              u64p(o_order), u64p(o_okey), st));
    // outputs (staged for host buffers)
    int32_t* d_og = out_group;
    double* d_ot = out_time;
    unsigned long long* d_oh = reinterpret_cast<unsigned long long*>(out_hit);
    if (!on_device || !out_group || !out_time || !out_hit) {
        NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, 24 * total));
        unsigned char* b = static_cast<unsigned char*>(ctx->d_stage2);
        if (!on_device || !d_og) d_og = reinterpret_cast<int32_t*>(b);
        if (!on_device || !d_ot) d_ot = reinterpret_cast<double*>(b + 8 * total);
        if (!on_device || !d_oh) d_oh = reinterpret_cast<unsigned long long*>(b + 16 * total);
    }
    NTP_CUDA(ctx, ntp::launch_resample_select(static_cast<int>(G), d_hits, d_t, u64p(o_start), u64p(o_nall),
                                              u64p(o_nsel), u64p(o_ostart), u64p(o_order), u64p(o_okey), d_og, d_ot,
                                              d_oh, st));
    if (!on_device) {
        if (out_group) NTP_CUDA(ctx, cudaMemcpyAsync(out_group, d_og, 4 * total, cudaMemcpyDeviceToHost, st));
        if (out_time) NTP_CUDA(ctx, cudaMemcpyAsync(out_time, d_ot, 8 * total, cudaMemcpyDeviceToHost, st));
        if (out_hit) NTP_CUDA(ctx, cudaMemcpyAsync(out_hit, d_oh, 8 * total, cudaMemcpyDeviceToHost, st));
    }
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

ntp_status ntp_calc_time_residual(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, const float src[3], float n800,
                                  double* tres, int32_t on_device, void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (!ctx->have_targets) {
        ctx->err = "ntp_calc_time_residual: targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (n == 0) return NTP_OK;
    if (!hits || !tres || !src) return invalid(ctx, "ntp_calc_time_residual: NULL argument");
    if (!(n800 > 0.0f)) return invalid(ctx, "ntp_calc_time_residual: n800 must be > 0");
    cudaSetDevice(ctx->device);
    cudaStream_t st = on_device ? pick_stream(ctx, stream) : ctx->stream;
    ntp_status sg = upload_tgeo(ctx, src, n800, st);
    if (sg != NTP_OK) return sg;
    const ntp_hit* d_hits = nullptr;
    ntp_status s = stage_hits(ctx, hits, n, on_device, st, &d_hits);
    if (s != NTP_OK) return s;
    double* d_out = tres;
    if (!on_device) {
        NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, sizeof(double) * n));
        d_out = static_cast<double*>(ctx->d_stage2);
    }
    NTP_CUDA(ctx, ntp::launch_time_residual(hit_table(ctx), d_hits, n, ctx->d_tgeo, d_out, st));
    if (!on_device) NTP_CUDA(ctx, cudaMemcpyAsync(tres, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}


ntp_status ntp_make_table(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n, const double* weight,
                          const ntp_source* sims, const float* sim_log10_energy, const double* sim_weight_scale,
                          const double* orientations, const ntp_table_spec* spec, float* cond, float* tres,
                          float* nhits, int32_t* has_time, int32_t* row_group, uint64_t capacity, uint64_t* n_rows,
                          float* group_cond, double* group_expec, uint64_t* group_count, uint64_t* group_hits,
                          void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (n_rows) *n_rows = 0;
    if (!ctx->have_targets) {
        ctx->err = "ntp_make_table: targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (!spec || !sims || !sim_log10_energy || !orientations) return invalid(ctx, "ntp_make_table: NULL argument");
    if (ctx->n_tgt != 1 || ctx->targets[0].kind != NTP_TARGET_MULTI_PMT || ctx->targets[0].n_pmts < 1)
        return invalid(ctx, "ntp_make_table: the context must hold exactly one MULTI_PMT module");
    if (spec->n_sims < 1 || spec->n_orientations < 1 || spec->max_rows_per_group < 1 || !(spec->downsample >= 0.0) ||
        !(spec->n800 > 0.0f))
        return invalid(ctx, "ntp_make_table: need n_sims, n_orientations, max_rows_per_group >= 1, downsample >= 0, "
                            "n800 > 0");
    if (n > 0 && (!hits || !weight)) return invalid(ctx, "ntp_make_table: NULL hits or weights");
    const ntp_target& mod = ctx->targets[0];
    const int S = spec->n_sims, R = spec->n_orientations, P = mod.n_pmts;
    const long long G = static_cast<long long>(S) * R * P;
    if (G > (1ll << 26)) return invalid(ctx, "ntp_make_table: too many (simulation, orientation, PMT) groups");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick_stream(ctx, stream);
    const uint2 key = make_uint2(static_cast<uint32_t>(spec->seed), static_cast<uint32_t>(spec->seed >> 32));
    const size_t g = static_cast<size_t>(G);

    // host: PMT axes per (simulation, orientation), group features, tgeo per simulation
    std::vector<float> axes(3 * g), gcond(5 * g);
    std::vector<double> tgeo(S);
    std::vector<double> pm(3 * static_cast<size_t>(P));
    for (int j = 0; j < P; ++j) {  // module-frame axes as in ntp_make_hits
        const float th = ctx->pmt_coords[2 * (mod.pmt_offset + j)], ph = ctx->pmt_coords[2 * (mod.pmt_offset + j) + 1];
        const float s_t = sinf(th), c_t = cosf(th), s_p = sinf(ph), c_p = cosf(ph);
        pm[3 * j] = static_cast<double>(c_p * s_t);
        pm[3 * j + 1] = static_cast<double>(s_p * s_t);
        pm[3 * j + 2] = static_cast<double>(c_t);
    }
    const double c_vac = 0.299792458, two_pi = 6.283185307179586;
    for (int si = 0; si < S; ++si) {
        const ntp_source& src = sims[si];
        double u[3] = {static_cast<double>(src.position[0]) - mod.position[0],
                       static_cast<double>(src.position[1]) - mod.position[1],
                       static_cast<double>(src.position[2]) - mod.position[2]};
        const double d = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (!(d > 0.0)) return invalid(ctx, "ntp_make_table: a simulation's source sits at the module centre");
        for (double& x : u) x /= d;
        {  // calc_time_residual!: (|src - module| - R) / (c / n800), with the Float32 distance
            const float dx = src.position[0] - mod.position[0], dy = src.position[1] - mod.position[1],
                        dz = src.position[2] - mod.position[2];
            const float df = std::sqrt(dx * dx + dy * dy + dz * dz);
            tgeo[si] = static_cast<double>(df - mod.radius) / (c_vac / static_cast<double>(spec->n800));
        }
        const double v[3] = {src.direction[0], src.direction[1], src.direction[2]};
        const double vu = v[0] * u[0] + v[1] * u[1] + v[2] * u[2];
        const double e1[3] = {v[0] - vu * u[0], v[1] - vu * u[1], v[2] - vu * u[2]};
        for (int r = 0; r < R; ++r) {
            const double* O = orientations + (static_cast<size_t>(si) * R + r) * 9;
            for (int j = 0; j < P; ++j) {
                const size_t gi = (static_cast<size_t>(si) * R + r) * P + j;
                double a[3];
                for (int k = 0; k < 3; ++k) a[k] = O[3 * k] * pm[3 * j] + O[3 * k + 1] * pm[3 * j + 1] + O[3 * k + 2] * pm[3 * j + 2];
                for (int k = 0; k < 3; ++k) axes[3 * gi + k] = static_cast<float>(a[k]);
                const double au = a[0] * u[0] + a[1] * u[1] + a[2] * u[2];
                const double e2[3] = {a[0] - au * u[0], a[1] - au * u[1], a[2] - au * u[2]};
                const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                      e1[0] * e2[1] - e1[1] * e2[0]};
                double phi = std::atan2(cr[0] * u[0] + cr[1] * u[1] + cr[2] * u[2],
                                        e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]);
                if (phi < 0.0) phi += two_pi;
                float* f = &gcond[5 * gi];
                f[0] = static_cast<float>(2.0 * std::log(d) / std::log(200.0) - 1.0);
                f[1] = static_cast<float>(vu);
                f[2] = static_cast<float>(au);
                f[3] = static_cast<float>(phi / M_PI - 1.0);
                f[4] = static_cast<float>((static_cast<double>(sim_log10_energy[si]) - 4.0) / 2.0);
            }
        }
    }
    const float cos_open = static_cast<float>(std::cos(std::asin(std::sqrt(mod.pmt_area / static_cast<float>(M_PI)) /
                                                                 mod.radius)));
    const float3 center = make_float3(mod.position[0], mod.position[1], mod.position[2]);

    // phase 1 scratch: axes f32[3G] | gcond f32[5G] | tgeo f64[S] | tres f64[n] | wsum f64[G] |
    //                  npos, nall, nsel, fill u64[G] | start, ostart, want u64[G+1]
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_axes = take(4 * 3 * g), o_gcond = take(4 * 5 * g), o_tgeo = take(8 * S), o_tres = take(8 * n);
    const size_t o_scale = take(8 * S);
    const size_t o_wsum = take(8 * g), o_w2 = take(8 * g), o_npos = take(8 * g), o_nall = take(8 * g);
    const size_t o_nsel = take(8 * g), o_fill = take(8 * g), o_start = take(8 * (g + 1));
    const size_t o_ostart = take(8 * (g + 1)), o_want = take(8 * (g + 1));
    NTP_CUDA(ctx, ensure(ctx->d_scratch, ctx->scratch_bytes, off));
    unsigned char* sc = static_cast<unsigned char*>(ctx->d_scratch);
    auto u64p = [&](size_t o) { return reinterpret_cast<unsigned long long*>(sc + o); };
    float* d_axes = reinterpret_cast<float*>(sc + o_axes);
    float* d_gcond = reinterpret_cast<float*>(sc + o_gcond);
    double* d_tgeo = reinterpret_cast<double*>(sc + o_tgeo);
    double* d_tres = reinterpret_cast<double*>(sc + o_tres);
    double* d_wsum = reinterpret_cast<double*>(sc + o_wsum);
    NTP_CUDA(ctx, cudaMemcpyAsync(d_axes, axes.data(), 4 * 3 * g, cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(d_gcond, gcond.data(), 4 * 5 * g, cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(d_tgeo, tgeo.data(), 8 * S, cudaMemcpyHostToDevice, st));
    std::vector<double> scale(S, 1.0);
    if (sim_weight_scale) scale.assign(sim_weight_scale, sim_weight_scale + S);
    double* d_scale = reinterpret_cast<double*>(sc + o_scale);
    NTP_CUDA(ctx, cudaMemcpyAsync(d_scale, scale.data(), 8 * S, cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemsetAsync(sc + o_wsum, 0, o_start - o_wsum, st));  // wsum, w2, npos, nall, nsel, fill
    double* d_w2 = reinterpret_cast<double*>(sc + o_w2);
    NTP_CUDA(ctx, ntp::launch_table_count(hits, n, weight, d_scale, S, R, P, center, d_axes, cos_open, d_wsum, d_w2,
                                          u64p(o_npos), u64p(o_nall), st));
    // the group count N = Poisson(sum(w) * downsample), not capped by the simulated hits (the
    // oversampling factor may be below 1); the no-cap bound goes through the draw's cap argument
    NTP_CUDA(ctx, cudaMemsetAsync(u64p(o_want), 0xFF, 8 * (g + 1), st));
    NTP_CUDA(ctx, ntp::launch_resample_draw(static_cast<int>(G), d_wsum, u64p(o_want), spec->downsample, key,
                                            u64p(o_nsel), st));
    std::vector<unsigned long long> nall(g), npos(g), nsel(g), start(g + 1), ostart(g + 1), want(g + 1, 0);
    NTP_CUDA(ctx, cudaMemcpyAsync(npos.data(), u64p(o_npos), 8 * g, cudaMemcpyDeviceToHost, st));
    std::vector<double> wsum(g), w2(g);
    NTP_CUDA(ctx, cudaMemcpyAsync(nall.data(), u64p(o_nall), 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(nsel.data(), u64p(o_nsel), 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(wsum.data(), d_wsum, 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(w2.data(), d_w2, 8 * g, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    std::vector<int32_t> zero;
    start[0] = ostart[0] = 0;
    const unsigned long long cap_rows = static_cast<unsigned long long>(spec->max_rows_per_group);
    for (size_t i = 0; i < g; ++i) {
        start[i + 1] = start[i] + nall[i];
        // rows: at most max_rows_per_group and a quarter of the effective sample size
        const double ess = w2[i] > 0.0 ? wsum[i] * wsum[i] / w2[i] : 0.0;
        const unsigned long long ess_cap = static_cast<unsigned long long>(ess / 4.0) + 1ull;
        want[i] = std::min(std::min(std::min(nsel[i], cap_rows), npos[i]), ess_cap);
        ostart[i + 1] = ostart[i] + want[i];
        if (nsel[i] == 0 && spec->zero_rows) zero.push_back(static_cast<int32_t>(i));
    }
    const unsigned long long pairs = start[g], hit_rows = ostart[g], total = hit_rows + zero.size();
    if (n_rows) *n_rows = total;
    if (total > capacity) {
        ctx->err = "ntp_make_table: capacity " + std::to_string(capacity) + " below " + std::to_string(total) + " rows";
        return NTP_ERR_OVERFLOW;
    }
    if (total > 0 && (!cond || !tres || !nhits || !has_time)) return invalid(ctx, "ntp_make_table: NULL output");
    // phase 2 scratch: order, okey u64[pairs] | og i32[rows] | ot f64[rows] | oh u64[rows] | zero i32[nz]
    size_t off2 = 0;
    auto take2 = [&](size_t bytes) { size_t o = off2; off2 += (bytes + 255) / 256 * 256; return o; };
    const size_t o_order = take2(8 * pairs), o_okey = take2(8 * pairs), o_og = take2(4 * hit_rows);
    const size_t o_ot = take2(8 * hit_rows), o_oh = take2(8 * hit_rows), o_zero = take2(4 * zero.size());
    NTP_CUDA(ctx, ensure(ctx->d_stage2, ctx->stage2_bytes, off2));
    unsigned char* s2 = static_cast<unsigned char*>(ctx->d_stage2);
    auto u64q = [&](size_t o) { return reinterpret_cast<unsigned long long*>(s2 + o); };
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_start), start.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_ostart), ostart.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_want), want.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st));
    if (!zero.empty())
        NTP_CUDA(ctx, cudaMemcpyAsync(s2 + o_zero, zero.data(), 4 * zero.size(), cudaMemcpyHostToDevice, st));
    if (pairs > 0) {
        NTP_CUDA(ctx, ntp::launch_table_bucket(hits, n, weight, d_scale, S, R, P, center, d_axes, cos_open, key, u64p(o_start),
                                               u64p(o_fill), u64q(o_order), u64q(o_okey), st));
        NTP_CUDA(ctx, ntp::launch_table_tres(hits, n, d_tgeo, S, d_tres, st));
        NTP_CUDA(ctx, ntp::launch_resample_select(static_cast<int>(G), hits, d_tres, u64p(o_start), u64p(o_nall),
                                                  u64p(o_want), u64p(o_ostart), u64q(o_order), u64q(o_okey),
                                                  reinterpret_cast<int32_t*>(s2 + o_og),
                                                  reinterpret_cast<double*>(s2 + o_ot), u64q(o_oh), st));
    }
    NTP_CUDA(ctx, ntp::launch_table_rows(hit_rows, reinterpret_cast<const int32_t*>(s2 + o_og),
                                         reinterpret_cast<const double*>(s2 + o_ot), zero.size(),
                                         reinterpret_cast<const int32_t*>(s2 + o_zero), u64p(o_nsel), d_gcond, cond,
                                         tres, nhits, has_time, row_group, st));
    if (group_cond) NTP_CUDA(ctx, cudaMemcpyAsync(group_cond, d_gcond, 4 * 5 * g, cudaMemcpyDeviceToDevice, st));
    if (group_count) NTP_CUDA(ctx, cudaMemcpyAsync(group_count, u64p(o_nsel), 8 * g, cudaMemcpyDeviceToDevice, st));
    if (group_hits) NTP_CUDA(ctx, cudaMemcpyAsync(group_hits, u64p(o_npos), 8 * g, cudaMemcpyDeviceToDevice, st));
    if (group_expec) {
        for (double& w : wsum) w *= spec->downsample;
        NTP_CUDA(ctx, cudaMemcpyAsync(group_expec, wsum.data(), 8 * g, cudaMemcpyHostToDevice, st));
    }
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}


ntp_status ntp_event_conditions(ntp_ctx* ctx, const ntp_source* events, const float* log10_energy,
                                const uint32_t* event_id, int32_t n_events, float d_min, float d_max, float n800,
                                float* cond, uint64_t* cond_key, float* cond_tgeo, int32_t* cond_event,
                                int32_t* cond_target, int32_t* cond_pmt, uint64_t capacity, uint64_t* n_cond,
                                uint64_t* event_first, int32_t* event_close, void* stream) {
    if (!ctx) return NTP_ERR_INVALID;
    if (n_cond) *n_cond = 0;
    if (!ctx->have_targets) {
        ctx->err = "ntp_event_conditions: targets must be set first";
        return NTP_ERR_NOT_READY;
    }
    if (n_events <= 0 || !events || !log10_energy || !(d_max >= d_min) || !(n800 > 0.0f))
        return invalid(ctx, "ntp_event_conditions: need events, energies, d_max >= d_min, n800 > 0");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick_stream(ctx, stream);
    const size_t ne = static_cast<size_t>(n_events);
    // host: packed events and the PMT axes of upright modules
    struct EventIn {
        float px, py, pz, dx, dy, dz, log10e;
        uint32_t id;
    };
    static_assert(sizeof(EventIn) == 32, "event record");
    if (ntp::event_in_size() != sizeof(EventIn)) return invalid(ctx, "ntp_event_conditions: event layout");
    std::vector<EventIn> ev(ne);
    for (size_t e = 0; e < ne; ++e) {
        const ntp_source& s = events[e];
        ev[e] = EventIn{s.position[0], s.position[1], s.position[2], s.direction[0], s.direction[1], s.direction[2],
                        log10_energy[e], event_id ? event_id[e] : static_cast<uint32_t>(e)};
    }
    const size_t npc = ctx->pmt_coords.size() / 2;
    std::vector<float> axes(3 * std::max<size_t>(npc, 1), 0.0f);
    for (size_t j = 0; j < npc; ++j) {
        const float th = ctx->pmt_coords[2 * j], ph = ctx->pmt_coords[2 * j + 1];
        axes[3 * j] = std::cos(ph) * std::sin(th);
        axes[3 * j + 1] = std::sin(ph) * std::sin(th);
        axes[3 * j + 2] = std::cos(th);
    }
    // scratch: events | axes | rows u64[ne] | fill u64[ne] | first u64[ne+1] | close i32[ne]
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_ev = take(sizeof(EventIn) * ne), o_ax = take(4 * axes.size()), o_rows = take(8 * ne);
    const size_t o_fill = take(8 * ne), o_first = take(8 * (ne + 1)), o_close = take(4 * ne);
    NTP_CUDA(ctx, ensure(ctx->d_scratch, ctx->scratch_bytes, off));
    unsigned char* sc = static_cast<unsigned char*>(ctx->d_scratch);
    auto u64p = [&](size_t o) { return reinterpret_cast<unsigned long long*>(sc + o); };
    NTP_CUDA(ctx, cudaMemcpyAsync(sc + o_ev, ev.data(), sizeof(EventIn) * ne, cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(sc + o_ax, axes.data(), 4 * axes.size(), cudaMemcpyHostToDevice, st));
    NTP_CUDA(ctx, cudaMemsetAsync(sc + o_rows, 0, o_first - o_rows, st));  // rows, fill
    NTP_CUDA(ctx, cudaMemsetAsync(sc + o_close, 0, 4 * ne, st));
    NTP_CUDA(ctx, ntp::launch_event_conditions_count(sc + o_ev, n_events, ctx->d_tgt, ctx->d_kind, ctx->d_npmt,
                                                     ctx->n_tgt, d_min, d_max, u64p(o_rows),
                                                     reinterpret_cast<int*>(sc + o_close), st));
    std::vector<unsigned long long> rows(ne), first(ne + 1);
    std::vector<int32_t> close(ne);
    NTP_CUDA(ctx, cudaMemcpyAsync(rows.data(), u64p(o_rows), 8 * ne, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaMemcpyAsync(close.data(), sc + o_close, 4 * ne, cudaMemcpyDeviceToHost, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    first[0] = 0;
    for (size_t e = 0; e < ne; ++e) first[e + 1] = first[e] + rows[e];
    if (event_first) std::copy(first.begin(), first.end(), event_first);
    if (event_close) std::copy(close.begin(), close.end(), event_close);
    const unsigned long long total = first[ne];
    if (n_cond) *n_cond = total;
    if (total > capacity) {
        ctx->err = "ntp_event_conditions: capacity " + std::to_string(capacity) + " below " + std::to_string(total);
        return NTP_ERR_OVERFLOW;
    }
    if (total == 0) return NTP_OK;
    if (!cond || !cond_key) return invalid(ctx, "ntp_event_conditions: NULL output");
    NTP_CUDA(ctx, cudaMemcpyAsync(u64p(o_first), first.data(), 8 * (ne + 1), cudaMemcpyHostToDevice, st));
    const float tgeo_scale = n800 / 0.299792458f;
    NTP_CUDA(ctx, ntp::launch_event_conditions_fill(sc + o_ev, n_events, ctx->d_tgt, ctx->d_radius, ctx->d_kind,
                                                    ctx->d_npmt, ctx->d_pmtoff, reinterpret_cast<float*>(sc + o_ax),
                                                    ctx->n_tgt, d_min, d_max, tgeo_scale, u64p(o_first), u64p(o_fill),
                                                    cond, reinterpret_cast<unsigned long long*>(cond_key), cond_tgeo,
                                                    cond_event, cond_target, cond_pmt, st));
    NTP_CUDA(ctx, cudaStreamSynchronize(st));
    return NTP_OK;
}

}  // extern "C"
