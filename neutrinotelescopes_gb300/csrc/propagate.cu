// propagate.cu -- the photon propagation kernel.
//
// Replaces cuda_propagate_photons! (chrhck/NeutrinoTelescopes,
// src/photon_propagation/photon_prop_cuda.jl:402-506) and its launch loop
// (:726-759).  Design for sm_103a:
//   * persistent grid (a multiple of the SM count); each warp claims chunks of
//     photon indices from a global counter and keeps its 32 lanes busy: a lane
//     whose photon ended (hit or step cap) takes the next index of the chunk
//     before the next step, so lanes never idle behind a long photon;
//   * all randoms come from Philox4x32-10 in registers, one block per step,
//     keyed by (draw, photon, source) so any photon can be replayed;
//   * medium table, spectrum knots and targets sit in shared memory;
//   * hits are written through one atomic per warp (ballot + popc) into an
//     array of 64-byte records with 16-byte vector stores; the hit counter
//     keeps counting past the capacity so the caller learns the exact size.
#include <cstdlib>

#include <cuda_runtime.h>

#include "ntp_device.cuh"
#include "ntp_internal.h"

namespace ntp {

namespace {

struct Photon {
    V3 pos, dir, init_dir;
    float time, wl, dist, sca_len_ln2, inv_vg;  // sca_len_ln2: scattering length times ln 2
    uint32_t src;
    uint32_t pk_lo, pk_hi;  // photon index within its source
    int step;
    int slot;               // index of the source in this launch
};

__device__ __forceinline__ int source_of(const unsigned long long* prefix, int n_src,
                                         unsigned long long gid) {
    int lo = 0, hi = n_src - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= gid) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// rand_gamma(shape, scale), utils.jl:267-294 (Marsaglia-Tsang, shape > 1),
// the normal from Box-Muller on Philox words; at most kGammaAttempts tries.
__device__ __forceinline__ float rand_gamma(float shape, float scale, uint4 ctr, const uint32_t (&rk)[20]) {
    const float d = shape - (1.0f / 3.0f);
    const float c = rsqrtf(9.0f * d);
    for (int k = 0; k < kGammaAttempts; ++k) {
        ctr.x = kDrawGamma0 + static_cast<uint32_t>(k);
        const uint4 r = philox4x32_10_rk(ctr, rk);
        float s, cs;
        sincos_2pi(u01(r.y), &s, &cs);
        const float x = fast_sqrt(-2.0f * __logf(u01(r.x))) * cs;
        float v = fmaf(c, x, 1.0f);
        if (v <= 0.0f) continue;
        v = v * v * v;
        const float u = u01(r.z);
        const float xsq = x * x;
        // the squeeze 1 - (1 + 0.0331 x^4) is never above u (utils.jl:286)
        if (__logf(u) < 0.5f * xsq + d * (1.0f - v + __logf(v))) return d * v * scale;
    }
    return d * scale;
}

// check_intersection(::Spherical, ...), photon_prop_cuda.jl:233-271: the
// segment pos + t dir, 0 < t < step, enters the sphere (x, y, z, r^2) at t = d.
// check_intersection(::Spherical), photon_prop_cuda.jl:233-271: with
// a = dir . (p - c) the segment enters the sphere at d = -a - sqrt(b),
// b = r^2 - |(p - c) - a dir|^2 (the squared distance of the line from the
// centre, subtracted from r^2).  The reference evaluates b as
// a^2 + r^2 - |p - c|^2: mathematically the same, but in single precision
// that difference of two numbers of order |p - c|^2 loses the r^2 it is
// compared with once the centre is a few hundred metres away, and a
// direction whose norm is 1 - e (rounding of the rotations) shifts it by
// -2 e a^2, a bias of the hit rate on distant modules.  The perpendicular
// vector form keeps b accurate to the rounding of r^2 at any distance and
// is insensitive to the norm to first order.
__device__ __forceinline__ bool sphere_hit(const float4 T, const V3 pos, const V3 dir, float step, float& d) {
    const float dx = pos.x - T.x, dy = pos.y - T.y, dz = pos.z - T.z;
    const float a = dir.x * dx + dir.y * dy + dir.z * dz;
    const float qx = fmaf(-a, dir.x, dx), qy = fmaf(-a, dir.y, dy), qz = fmaf(-a, dir.z, dz);
    const float b = T.w - (qx * qx + qy * qy + qz * qz);
    if (b >= 0.0f) {
        d = -a - fast_sqrt(b);
        return d > 0.0f && d < step;
    }
    return false;
}

// Per-step quantities of the column tests.
struct SegmentView {
    V3 pos, dir;
    float step;
    float dd;       // dir.x^2 + dir.y^2
    float slack2;   // rounding envelope of the float sphere test, grows as step^2
};

__device__ __forceinline__ SegmentView make_segment(const V3 pos, const V3 dir, float step) {
    return SegmentView{pos, dir, step, dir.x * dir.x + dir.y * dir.y, 4e-7f * step * step};
}

// Tests the members of one vertical column that the segment can reach.  The
// culling is conservative: the horizontal distance of the segment from the
// column axis is compared with r_cull^2 plus the rounding envelope of the
// single-precision sphere test, and the z range is padded by r_cull and one
// member; every member it keeps goes through the same sphere_hit as the plain
// scan.  Among the hits it keeps the first in target-list order (or the
// nearest), as the plain scan does.  The cheapest test comes first: the
// distance of the column axis from the infinite line.
__device__ __forceinline__ void column_candidates(const Column& C, const int* __restrict__ mem,
                                                  const float4* __restrict__ tg, const SegmentView& sg,
                                                  int policy, int& hit_t, float& hit_d) {
    const V3 pos = sg.pos, dir = sg.dir;
    const float step = sg.step, dd = sg.dd;
    const float px = pos.x - C.cx, py = pos.y - C.cy;
    const float rc2 = fmaf(C.r_cull, C.r_cull, sg.slack2);
    float t0 = 0.0f, t1 = step;
    if (dd > 1e-12f) {
        const float cr = px * dir.y - py * dir.x;  // perpendicular distance * sqrt(dd)
        if (cr * cr > rc2 * dd) return;            // the line passes wide of the axis
        const float pd = -(px * dir.x + py * dir.y);  // closest approach at ts = pd / dd
        bool far = false;
        if (pd <= 0.0f) {
            far = px * px + py * py > rc2;
        } else if (pd >= step * dd) {
            const float ex = fmaf(step, dir.x, px), ey = fmaf(step, dir.y, py);
            far = ex * ex + ey * ey > rc2;
        }
        if (far) return;
        const float inv_dd = rcp_ftz(dd);  // dd > 1e-12
        const float ts = pd * inv_dd;
        const float h = fast_sqrt((rc2 - cr * cr * inv_dd) * inv_dd);
        t0 = fmaxf(ts - h, 0.0f);
        t1 = fminf(ts + h, step);
    } else if (px * px + py * py > rc2) {
        return;
    }
    const float za = fmaf(t0, dir.z, pos.z), zb = fmaf(t1, dir.z, pos.z);
    const float zlo = fminf(za, zb) - C.r_cull, zhi = fmaxf(za, zb) + C.r_cull;
    if (zhi < C.z0 - C.r_cull || zlo > C.z_last + C.r_cull) return;
    int k0 = 0, k1 = C.count - 1;
    if (C.dz > 0.0f) {
        const float inv = rcp_ftz(C.dz);
        k0 = max(k0, static_cast<int>(floorf(fmaxf((zlo - C.z0) * inv, -1.0f))) - 1);
        k1 = min(k1, static_cast<int>(ceilf(fminf((zhi - C.z0) * inv, static_cast<float>(C.count)))) + 1);
    }
    for (int k = k0; k <= k1; ++k) {
        const int t = mem[C.first + k];
        const float4 T = tg[t];
        if (C.dz <= 0.0f && (T.z < zlo - 1.0f || T.z > zhi + 1.0f)) continue;
        float d;
        if (sphere_hit(T, pos, dir, step, d)) {
            if (policy == NTP_HIT_NEAREST ? d < hit_d : (hit_t < 0 || t < hit_t)) {
                hit_d = d;
                hit_t = t;
            }
        }
    }
}

// Walks the cells of the column grid that the horizontal projection of the
// segment pos + t dir, 0 <= t <= step, crosses (Amanatides-Woo), testing the
// columns listed in each.  A column listed in several visited cells is
// tested more than once, which does not change the result.  The walk is
// bounded by nx + ny + 2 cells.
__device__ __forceinline__ void grid_candidates(const PropParams& p, const int* __restrict__ cstart,
                                                const int* __restrict__ citems, const Column* __restrict__ cols,
                                                const int* __restrict__ mem, const float4* __restrict__ tg,
                                                const SegmentView& sg, int& hit_t, float& hit_d) {
    const V3 pos = sg.pos, dir = sg.dir;
    const float step = sg.step;
    const float h = p.grid_h, inv_h = p.grid_inv_h;
    const float x1 = p.grid_x0 + h * static_cast<float>(p.grid_nx);
    const float y1 = p.grid_y0 + h * static_cast<float>(p.grid_ny);
    // reciprocal direction components (0 components never cross a cell wall)
    const float inf = __int_as_float(0x7f800000);
    const float rx = dir.x != 0.0f ? fast_rcp(dir.x) : inf, ry = dir.y != 0.0f ? fast_rcp(dir.y) : inf;
    // clip the segment to the grid box
    float t_in = 0.0f, t_out = step;
    if (dir.x != 0.0f) {
        const float ta = (p.grid_x0 - pos.x) * rx, tb = (x1 - pos.x) * rx;
        t_in = fmaxf(t_in, fminf(ta, tb));
        t_out = fminf(t_out, fmaxf(ta, tb));
    } else if (pos.x < p.grid_x0 || pos.x > x1) {
        return;
    }
    if (dir.y != 0.0f) {
        const float ta = (p.grid_y0 - pos.y) * ry, tb = (y1 - pos.y) * ry;
        t_in = fmaxf(t_in, fminf(ta, tb));
        t_out = fminf(t_out, fmaxf(ta, tb));
    } else if (pos.y < p.grid_y0 || pos.y > y1) {
        return;
    }
    if (!(t_in <= t_out)) return;
    const float sx = fmaf(t_in, dir.x, pos.x), sy = fmaf(t_in, dir.y, pos.y);
    int ix = min(max(static_cast<int>(floorf((sx - p.grid_x0) * inv_h)), 0), p.grid_nx - 1);
    int iy = min(max(static_cast<int>(floorf((sy - p.grid_y0) * inv_h)), 0), p.grid_ny - 1);
    const int stx = dir.x > 0.0f ? 1 : -1, sty = dir.y > 0.0f ? 1 : -1;
    float tmx = dir.x != 0.0f ? (p.grid_x0 + h * static_cast<float>(ix + (dir.x > 0.0f)) - pos.x) * rx : inf;
    float tmy = dir.y != 0.0f ? (p.grid_y0 + h * static_cast<float>(iy + (dir.y > 0.0f)) - pos.y) * ry : inf;
    const float tdx = h * fabsf(rx), tdy = h * fabsf(ry);
    for (int guard = p.grid_nx + p.grid_ny + 2; guard > 0; --guard) {
        const int c = iy * p.grid_nx + ix;
        for (int k = cstart[c]; k < cstart[c + 1]; ++k)
            column_candidates(cols[citems[k]], mem, tg, sg, p.hit_policy, hit_t, hit_d);
        if (tmx < tmy) {
            if (tmx > t_out) break;
            ix += stx;
            if (ix < 0 || ix >= p.grid_nx) break;
            tmx += tdx;
        } else {
            if (tmy > t_out) break;
            iy += sty;
            if (iy < 0 || iy >= p.grid_ny) break;
            tmy += tdy;
        }
    }
}

// The lattice form of grid_candidates (grid_lattice): the columns sit at the
// cell centres (i + 1/2, j + 1/2) h of a regular lattice, at most one per
// cell.  In lattice units (u, v) along the step's major horizontal axis u,
// a column within R of the segment has |u - u(segment)| <= R / h and lies
// within R of the line, i.e. |v_col - v_line(u_col)| <= R / (h cos phi) <=
// sqrt(2) R / h (cos phi >= 1/sqrt 2 on the major axis).  With R^2 the
// largest r_cull^2 plus the single-precision envelope of the step (as in
// column_candidates) and a 1e-3 margin for the rounding of u and v, the
// points kept include every column column_candidates could accept; each
// goes through column_candidates, so the hits equal the plain scan's.  A
// step costs one short loop over the lattice rows its u range spans
// (usually one to four), with no cell-crossing bookkeeping.
__device__ __forceinline__ void lattice_candidates(const PropParams& p, const int* __restrict__ cstart,
                                                   const int* __restrict__ citems, const Column* __restrict__ cols,
                                                   const int* __restrict__ mem, const float4* __restrict__ tg,
                                                   const SegmentView& sg, int& hit_t, float& hit_d) {
    const float inv_h = p.grid_inv_h;
    const float ua = (sg.pos.x - p.grid_x0) * inv_h - 0.5f, va = (sg.pos.y - p.grid_y0) * inv_h - 0.5f;
    const float du = sg.dir.x * sg.step * inv_h, dv = sg.dir.y * sg.step * inv_h;
    const float delta = fast_sqrt(2.0f * (p.lat_rcull2 + sg.slack2)) * inv_h + 1e-3f;
    const bool u_major = fabsf(du) >= fabsf(dv);
    // major axis a (extent n_a), minor axis b (extent n_b)
    const float a0 = u_major ? ua : va, b0 = u_major ? va : ua;
    const float da = u_major ? du : dv, db = u_major ? dv : du;
    const int n_a = u_major ? p.grid_nx : p.grid_ny, n_b = u_major ? p.grid_ny : p.grid_nx;
    const float slope = da != 0.0f ? db / da : 0.0f;  // |slope| <= 1
    const int a_lo = max(0, static_cast<int>(ceilf(fminf(a0, a0 + da) - delta)));
    const int a_hi = min(n_a - 1, static_cast<int>(floorf(fmaxf(a0, a0 + da) + delta)));
    for (int ia = a_lo; ia <= a_hi; ++ia) {
        const float b = fmaf(static_cast<float>(ia) - a0, slope, b0);
        const int b_lo = max(0, static_cast<int>(ceilf(b - delta)));
        const int b_hi = min(n_b - 1, static_cast<int>(floorf(b + delta)));
        for (int ib = b_lo; ib <= b_hi; ++ib) {
            const int c = u_major ? ib * p.grid_nx + ia : ia * p.grid_nx + ib;
            if (cstart[c + 1] > cstart[c])
                column_candidates(cols[citems[cstart[c]]], mem, tg, sg, p.hit_policy, hit_t, hit_d);
        }
    }
}

// initialize_photon_state methods, photon_prop_cuda.jl:133-200 and
// sample_cherenkov_direction :107-125.
__device__ __forceinline__ void init_photon(Photon& ph, const ntp_source* __restrict__ sources,
                                         const PropParams& p, const SpectrumView& spec,
                                         const float4* medium, unsigned long long gid, int s) {
    const ntp_source* src = sources + s;
    const unsigned long long pk =
        gid - __ldg(p.prefix + s) + (p.src_photon_offset ? __ldg(p.src_photon_offset + s) : 0ull);
    ph.src = p.src_stream ? __ldg(p.src_stream + s) : static_cast<uint32_t>(s);
    ph.slot = p.src_out ? static_cast<int>(__ldg(p.src_out + s)) : s;
    ph.pk_lo = static_cast<uint32_t>(pk);
    ph.pk_hi = static_cast<uint32_t>(pk >> 32);
    const uint4 base = make_uint4(kDrawInitA, ph.pk_lo, ph.pk_hi, ph.src);
    const uint4 A = philox4x32_10_rk(base, p.rk);

    const int kind = __ldg(&src->kind);
    ph.wl = sample_wavelength(spec, u01(A.x));
    ph.pos = V3{__ldg(&src->position[0]), __ldg(&src->position[1]), __ldg(&src->position[2])};
    ph.time = __ldg(&src->time);
    const V3 sdir{__ldg(&src->direction[0]), __ldg(&src->direction[1]), __ldg(&src->direction[2])};
    const float4 med = interp_table(medium, p.n_medium, p.wl_min, p.medium_scale, ph.wl);
    bool cherenkov = false;

    switch (kind) {
    case NTP_SRC_POINT_ISOTROPIC:
    case NTP_SRC_POINT_TIME_RANGE: {  // initialize_direction_isotropic :100-104
        const float u = u01(A.z);     // cos = 2u - 1, 1 - cos = 2(1 - u)
        ph.dir = dir_from_omc(2.0f * (1.0f - u), u01(A.y));  // sin = sqrt(omc (2 - omc)) = 2 sqrt(u (1 - u))
        if (kind == NTP_SRC_POINT_TIME_RANGE) {
            const float t1 = __ldg(&src->time_end);
            ph.time = ph.time + u01(A.w) * (t1 - ph.time);
        }
        break;
    }
    case NTP_SRC_AXICONE: {  // :148-156
        float st, ct, sp, cp;
        sincosf(__ldg(&src->angle), &st, &ct);
        sincos_2pi(u01(A.y), &sp, &cp);
        ph.dir = rot_from_ez(sdir, V3{cp * st, sp * st, ct}, p.exact_pole);
        break;
    }
    case NTP_SRC_PENCIL:  // :158-161
        ph.dir = sdir;
        break;
    case NTP_SRC_EXTENDED_CHERENKOV: {  // :164-176
        const float b = __ldg(&src->long_b);
        const float long_pos =
            rand_gamma(__ldg(&src->long_a), __frcp_rn(b), base, p.rk) * __ldg(&src->long_lrad);
        ph.pos = V3{fmaf(long_pos, sdir.x, ph.pos.x), fmaf(long_pos, sdir.y, ph.pos.y),
                    fmaf(long_pos, sdir.z, ph.pos.z)};
        ph.time = fmaf(long_pos, kInvCVac, ph.time);
        cherenkov = true;
        break;
    }
    case NTP_SRC_CHERENKOV_TRACK: {  // :190-200, direction as :178-188
        const float along = u01(A.w) * __ldg(&src->length);
        ph.pos = V3{fmaf(along, sdir.x, ph.pos.x), fmaf(along, sdir.y, ph.pos.y),
                    fmaf(along, sdir.z, ph.pos.z)};
        ph.time = fmaf(along, kInvCVac, ph.time);
        cherenkov = true;
        break;
    }
    default:  // NTP_SRC_POINT_CHERENKOV :178-188
        cherenkov = true;
        break;
    }
    if (cherenkov) {
        // photon on the Cherenkov cone cos = 1/n(lambda) (medium.jl:309-311)
        const float cos_c = fast_rcp(med.x);
        float sp, cp;
        sincos_2pi(u01(A.y), &sp, &cp);
        const float sin_c = fast_sqrt(fmaf(-cos_c, cos_c, 1.0f));
        V3 d{cp * sin_c, sp * sin_c, cos_c};
        // track smearing, sample_cherenkov_track_direction utils.jl:249-260:
        // 1 - cos = (-log(1 - u I)/b)^(1/a), a = 0.39, b = 2.61
        const uint4 B = philox4x32_10_rk(make_uint4(kDrawInitB, ph.pk_lo, ph.pk_hi, ph.src), p.rk);
        const float I = 0.96729171f;  // 1 - exp(-2.61 * 2^0.39)
        const float base = -log1pf(-u01(B.x) * I) * (1.0f / 2.61f);
        // base >= ~2e-8 (u01 >= 2^-24): base^(1/0.39) stays normal
        const float omc = fminf(fast_exp2(log2_ftz(base) * (1.0f / 0.39f)), 2.0f);
        const V3 track = dir_from_omc(omc, u01(B.y));
        d = rot_from_ez(track, d, p.exact_pole);
        ph.dir = rot_from_ez(sdir, d, p.exact_pole);
    }
    ph.init_dir = ph.dir;
    ph.dist = 0.0f;
    ph.sca_len_ln2 = med.z * 0.6931471805599453f;
    ph.inv_vg = fast_rcp(med.y);
    ph.step = 0;
}

template <int kMinBlocks>
__global__ void __launch_bounds__(kPropBlock, kMinBlocks) propagate_kernel(const PropParams p) {
    // shared memory: medium knots | targets | columns | module ids | members |
    // cell grid | spectrum knots (targets, ids and members when
    // targets_in_smem; columns and the grid when columns_in_smem)
    extern __shared__ float4 smem[];
    const int nt_s = p.targets_in_smem ? p.n_targets : 0;
    const int nc_s = p.columns_in_smem && p.columns ? p.n_columns : 0;
    const int nm_s = nt_s && nc_s ? p.n_targets : 0;
    float4* s_med = smem;
    float4* s_tgt = s_med + p.n_medium;
    Column* s_col = reinterpret_cast<Column*>(s_tgt + nt_s);
    uint32_t* s_tid = reinterpret_cast<uint32_t*>(s_col + nc_s);
    int* s_mem = reinterpret_cast<int*>(s_tid + nt_s);
    const bool grid_s = nc_s && p.cell_start && (p.grid_nx * p.grid_ny + 1 + p.n_cell_items) <= kMaxSmemGridInts;
    const int ng_s = grid_s ? p.grid_nx * p.grid_ny + 1 : 0;
    int* s_cstart = s_mem + nm_s;
    int* s_citems = s_cstart + ng_s;
    float* s_spec = reinterpret_cast<float*>(s_citems + (grid_s ? p.n_cell_items : 0));

    for (int i = threadIdx.x; i < p.n_medium; i += blockDim.x) s_med[i] = p.medium[i];
    for (int i = threadIdx.x; i < p.n_spec; i += blockDim.x) s_spec[i] = p.spec_knots[i];
    for (int i = threadIdx.x; i < nt_s; i += blockDim.x) {
        s_tgt[i] = p.targets[i];
        s_tid[i] = p.target_ids[i];
    }
    for (int i = threadIdx.x; i < nc_s; i += blockDim.x) s_col[i] = p.columns[i];
    for (int i = threadIdx.x; i < nm_s; i += blockDim.x) s_mem[i] = p.members[i];
    if (grid_s) {
        for (int i = threadIdx.x; i < ng_s; i += blockDim.x) s_cstart[i] = p.cell_start[i];
        for (int i = threadIdx.x; i < p.n_cell_items; i += blockDim.x) s_citems[i] = p.cell_items[i];
    }
    __syncthreads();
    const int* cstart = grid_s ? s_cstart : p.cell_start;
    const int* citems = grid_s ? s_citems : p.cell_items;
    const float4* tg = nt_s ? s_tgt : p.targets;
    const uint32_t* tid = nt_s ? s_tid : p.target_ids;
    const Column* cols = p.columns ? (nc_s ? s_col : p.columns) : nullptr;
    const int* mem = nm_s ? s_mem : p.members;

    SpectrumView spec{p.spec_kind, p.n_spec, s_spec, p.spec_p0, p.spec_p1};
    const float g = p.hg_g, one_m_g = 1.0f - g, one_m_g2 = fmaf(-g, g, 1.0f);
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    unsigned long long c_next = 0, c_end = 0;  // warp-uniform chunk of photon indices
    bool exhausted = false;
    bool active = false;
    unsigned long long done = 0, steps = 0;
    Photon ph;

    for (;;) {
        // refill idle lanes in batches of at least refill_min (or when every
        // lane is idle), so the divergent initialisation runs for many lanes
        // at once instead of for one or two in almost every iteration
        // (no lane idle, the common case, costs one vote and one branch)
        const unsigned idle = __ballot_sync(kFull, !active);
        if (idle) {
            bool refilled = false;  // warp-uniform
            if (!exhausted && (idle == kFull || __popc(idle) >= p.refill_min)) {
                unsigned long long avail = c_end - c_next;
                if (avail == 0) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(p.counters, p.chunk);
                    base = __shfl_sync(kFull, base, 0);
                    if (base >= p.total) {
                        exhausted = true;
                    } else {
                        c_next = base;
                        c_end = min(base + p.chunk, p.total);
                        avail = c_end - c_next;
                    }
                }
                if (avail) {
                    const unsigned long long take = min(static_cast<unsigned long long>(__popc(idle)), avail);
                    const unsigned rank = __popc(idle & lt_mask);
                    if (!active && rank < take) {
                        const unsigned long long gid = c_next + rank;
                        init_photon(ph, p.sources, p, spec, s_med, gid, source_of(p.prefix, p.n_src, gid));
                        active = true;
                    }
                    c_next += take;
                    refilled = true;
                }
            }
            if (idle == kFull && !refilled) break;  // every lane idle and no photon left
        }

        bool hit = false;
        int hit_t = -1;
        if (active) {
            const uint4 r = philox4x32_10_rk(
                make_uint4(kDrawStep0 + static_cast<uint32_t>(ph.step), ph.pk_lo, ph.pk_hi, ph.src), p.rk);
            // -ln(u) lambda_sca as -log2(u) (lambda_sca ln 2)
            const float step = -log2_ftz(u01(r.x)) * ph.sca_len_ln2;

            // check_intersection over the targets, photon_prop_cuda.jl:233-271, :460-468
            float hit_d = step;
            if (cols) {
                const SegmentView sg = make_segment(ph.pos, ph.dir, step);
                if (cstart) {
                    if (p.grid_lattice)
                        lattice_candidates(p, cstart, citems, cols, mem, tg, sg, hit_t, hit_d);
                    else
                        grid_candidates(p, cstart, citems, cols, mem, tg, sg, hit_t, hit_d);
                } else {
                    for (int c = 0; c < p.n_columns; ++c)
                        column_candidates(cols[c], mem, tg, sg, p.hit_policy, hit_t, hit_d);
                }
            } else {
                for (int t = 0; t < p.n_targets; ++t) {
                    float d;
                    if (sphere_hit(tg[t], ph.pos, ph.dir, step, d)) {
                        if (p.hit_policy == NTP_HIT_NEAREST) {
                            if (d < hit_d) { hit_d = d; hit_t = t; }
                        } else {
                            hit_d = d;
                            hit_t = t;
                            break;
                        }
                    }
                }
            }
            const float move = hit_t >= 0 ? hit_d : step;
            ph.pos = V3{fmaf(ph.dir.x, move, ph.pos.x), fmaf(ph.dir.y, move, ph.pos.y),
                        fmaf(ph.dir.z, move, ph.pos.z)};
            ph.dist += move;
            ph.time = fmaf(move, ph.inv_vg, ph.time);
            if (hit_t >= 0) {
                hit = true;
            } else {
                // update_direction, photon_prop_cuda.jl:204-222, phase function
                // mixture Rayleigh / Henyey-Greenstein.  Both cosines are
                // computed and one selected, so lanes of a warp do not diverge.
                const float eta = u01(r.y);
                float omc = hg_one_minus_cos(g, one_m_g, one_m_g2, eta);
                if (p.rayleigh_on) {
                    const float omr = 1.0f - rayleigh_cos(eta);
                    omc = r.w <= p.rayleigh_wmax ? omr : omc;  // u01(r.w) < rayleigh_fraction
                }
                ph.dir = rot_from_ez(ph.dir, dir_from_omc(omc, u01(r.z)), p.exact_pole);
                if (++ph.step >= p.max_steps) {
                    active = false;
                    ++done;
                    steps += static_cast<unsigned>(ph.step);
                }
            }
        }

        if (hit) {
            // one atomic for the lanes of this warp that hit in this step (per
            // source in the per-source output mode)
            const unsigned act = __activemask();
            const unsigned hm = p.src_hit_count ? __match_any_sync(act, ph.slot) : act;
            const int leader = __ffs(hm) - 1;
            unsigned long long base = 0;
            if (static_cast<int>(lane) == leader) {
                const unsigned long long n = static_cast<unsigned long long>(__popc(hm));
                if (p.src_hit_count) {
                    base = atomicAdd(p.src_hit_count + ph.slot, n);
                    atomicAdd(p.counters + 1, n);
                } else {
                    base = atomicAdd(p.counters + 1, n);
                }
            }
            base = __shfl_sync(hm, base, leader);
            unsigned long long slot = base + __popc(hm & lt_mask);
            bool room = slot < p.capacity;
            if (p.src_hit_count) {
                room = slot < __ldg(p.src_hit_cap + ph.slot);
                slot += __ldg(p.src_hit_base + ph.slot);
            }
            if (room) {
                float4* o = reinterpret_cast<float4*>(p.hits + slot);
                __stcs(o + 0, make_float4(ph.pos.x, ph.pos.y, ph.pos.z, ph.time));
                __stcs(o + 1, make_float4(ph.dir.x, ph.dir.y, ph.dir.z, ph.wl));
                __stcs(o + 2, make_float4(ph.init_dir.x, ph.init_dir.y, ph.init_dir.z, ph.dist));
                __stcs(reinterpret_cast<uint4*>(o + 3),
                       make_uint4(tid[hit_t], p.src_stream ? ph.src : static_cast<uint32_t>(ph.slot), ph.pk_lo, ph.pk_hi));
            }
            active = false;
            ++done;
            steps += static_cast<unsigned>(ph.step) + 1u;
        }
    }

    // photons finished and photon-steps taken: one atomic per warp each
    for (int off = 16; off > 0; off >>= 1) {
        done += __shfl_down_sync(kFull, done, off);
        steps += __shfl_down_sync(kFull, steps, off);
    }
    if (lane == 0 && done) atomicAdd(p.counters + 2, done);
    if (lane == 0 && steps) atomicAdd(p.counters + 3, steps);
}

}  // namespace

size_t prop_smem_bytes(const PropParams& p) {
    size_t b = sizeof(float4) * static_cast<size_t>(p.n_medium);
    const bool nt = p.targets_in_smem != 0, nc = p.columns_in_smem && p.columns;
    if (nt) b += (sizeof(float4) + sizeof(uint32_t)) * static_cast<size_t>(p.n_targets);
    if (nc) {
        b += sizeof(Column) * static_cast<size_t>(p.n_columns);
        if (nt) b += sizeof(int) * static_cast<size_t>(p.n_targets);  // members
        const long long g = p.cell_start ? static_cast<long long>(p.grid_nx) * p.grid_ny + 1 + p.n_cell_items : 0;
        if (p.cell_start && g <= kMaxSmemGridInts) b += sizeof(int) * static_cast<size_t>(g);
    }
    b += sizeof(float) * static_cast<size_t>(p.n_spec);
    return b;
}

// Register budget of the propagation kernel: 4 blocks of 256 threads per SM
// (<= 64 registers; measured 5.7% faster on GB300 than 3 blocks, the kernel
// being bound by dependency latency), or 3 (<= 85 registers) when
// NTP_PROP_OCCUPANCY=3.
static bool use_four_blocks() {
    const char* e = std::getenv("NTP_PROP_OCCUPANCY");
    return !(e && e[0] == '3');
}

template <int B>
static cudaError_t occupancy_of(const PropParams& p, int* blocks_per_sm) {
    const size_t smem = prop_smem_bytes(p);
    cudaError_t e = cudaFuncSetAttribute(propagate_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, propagate_kernel<B>, kPropBlock, smem);
}

cudaError_t propagate_occupancy(const PropParams& p, int* blocks_per_sm) {
    return use_four_blocks() ? occupancy_of<4>(p, blocks_per_sm) : occupancy_of<3>(p, blocks_per_sm);
}

const void* propagate_kernel_fn() {
    return use_four_blocks() ? reinterpret_cast<const void*>(&propagate_kernel<4>)
                             : reinterpret_cast<const void*>(&propagate_kernel<3>);
}

cudaError_t launch_propagate(const PropParams& p, int grid, cudaStream_t stream) {
    const size_t smem = prop_smem_bytes(p);
    if (use_four_blocks()) propagate_kernel<4><<<grid, kPropBlock, smem, stream>>>(p);
    else propagate_kernel<3><<<grid, kPropBlock, smem, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace ntp
