/*
 * ntp_oracle.c -- CPU oracle of the photon-propagation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates the reference algorithm of
 * chrhck/NeutrinoTelescopes (Julia + CUDA.jl) in plain C so that the CUDA
 * library can be checked against it.  Only tests, the smoke check and the CPU
 * baseline leg of the benchmark load it; nothing in the product links it.
 *
 * Parity status: the reference cannot run in this environment (its path is
 * CUDA.jl device code and no Julia toolchain is present).  The geometric and
 * numerical helpers are pinned by the reference's own known-answer tests
 * (test/runtests.jl:60-83, :89-118, :121-130, :132-158), Philox4x32-10 by its
 * published known-answer vectors, and the medium functions by values derived
 * from the formulas in medium.jl.  The random stream itself is unpinned: the
 * reference draws from CUDA.jl's device RNG, which is replaced here and in the
 * library by a counter-based Philox4x32-10 stream (counter = draw, photon,
 * source; key = seed), shared by the oracle and the kernel.
 *
 * Build: oracle/Makefile -> oracle/libntp_oracle.so
 */
#include <math.h>
#include <stdint.h>
#include <tgmath.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ntp.h"

#define NTPO_PI 3.14159265358979323846
#define NTPO_C_VAC 0.299792458          /* m/ns, SpeedOfLightInVacuum */
#define NTPO_FINE_STRUCTURE 7.2973525693e-3  /* CODATA2018 */

/* Philox block indices (the "draw" word of the counter); the same layout is
   used by the CUDA kernel. */
#define NTPO_DRAW_INIT_A 0u
#define NTPO_DRAW_INIT_B 1u
#define NTPO_DRAW_GAMMA0 2u
#define NTPO_GAMMA_ATTEMPTS 32
#define NTPO_DRAW_STEP0 64u

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of two
   32x32->64 multiplies with Weyl key increments. */
void ntpo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0;
        uint32_t y1 = (uint32_t)p1;
        uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
        uint32_t y3 = (uint32_t)p0;
        x0 = y0; x1 = y1; x2 = y2; x3 = y3;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* A 32-bit word to a uniform in the open interval (0, 1): the top 23 bits
   plus one half, times 2^-23.  Exactly representable in float and double. */
double ntpo_u01_f64(uint32_t w) { return ((double)(w >> 9) + 0.5) * (1.0 / 8388608.0); }

/* Candidate lookup for large detectors (the statistical checks on a string
   grid), used only when asked for.  Target centres are bucketed on a 2-D
   (x, y) grid.  A step segment that enters a sphere passes within one radius
   of its centre, so the centre lies in the segment's bounding box widened by
   that radius; the cells this box overlaps therefore hold every target the
   literal scan of photon_prop_cuda.jl:460-468 can report.  Those candidates
   go through the same check_intersection and the lowest list index (first
   in list order) or the smallest distance (nearest) wins, which is what the
   scan returns: the lookup only skips targets that cannot be hit.  The
   widening adds 5 cm to the largest radius to cover float rounding of the
   segment end points. */
typedef struct {
    int nx, ny;
    double x0, y0, inv_h;
    double margin;
    int* start; /* nx * ny + 1 offsets into items */
    int* items; /* target indices, ascending within a cell */
} ntpo_bins;

static int ntpo_clampi(long long v, int hi) { return v < 0 ? 0 : (v > hi ? hi : (int)v); }

static void ntpo_bins_build(ntpo_bins* b, const ntp_target* tg, int n_tg) {
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300, rmax = 0.0;
    for (int t = 0; t < n_tg; ++t) {
        double x = tg[t].position[0], y = tg[t].position[1];
        if (x < xmin) xmin = x;
        if (x > xmax) xmax = x;
        if (y < ymin) ymin = y;
        if (y > ymax) ymax = y;
        if (tg[t].radius > rmax) rmax = tg[t].radius;
    }
    double extent = (xmax - xmin) > (ymax - ymin) ? (xmax - xmin) : (ymax - ymin);
    double cells = n_tg / 16.0 > 1.0 ? n_tg / 16.0 : 1.0;
    double h = extent / sqrt(cells);
    if (h < 4.0 * rmax) h = 4.0 * rmax;
    if (h < 1.0) h = 1.0;
    b->x0 = xmin;
    b->y0 = ymin;
    b->inv_h = 1.0 / h;
    b->nx = (int)((xmax - xmin) / h) + 1;
    b->ny = (int)((ymax - ymin) / h) + 1;
    b->margin = rmax + 0.05;
    int nc = b->nx * b->ny;
    b->start = (int*)calloc((size_t)nc + 1, sizeof(int));
    b->items = (int*)malloc(sizeof(int) * (size_t)(n_tg ? n_tg : 1));
    int* cell = (int*)malloc(sizeof(int) * (size_t)(n_tg ? n_tg : 1));
    for (int t = 0; t < n_tg; ++t) {
        int ix = ntpo_clampi((long long)floor((tg[t].position[0] - b->x0) * b->inv_h), b->nx - 1);
        int iy = ntpo_clampi((long long)floor((tg[t].position[1] - b->y0) * b->inv_h), b->ny - 1);
        cell[t] = iy * b->nx + ix;
        b->start[cell[t] + 1]++;
    }
    for (int c = 0; c < nc; ++c) b->start[c + 1] += b->start[c];
    int* fill = (int*)calloc((size_t)nc, sizeof(int));
    for (int t = 0; t < n_tg; ++t) b->items[b->start[cell[t]] + fill[cell[t]]++] = t;
    free(fill);
    free(cell);
}

static void ntpo_bins_free(ntpo_bins* b) {
    free(b->start);
    free(b->items);
}

/* ------------------------------------------------------------------------
 * The step law, in double and in float. */
#define REAL double
#define F(name) name##_f64
#include "steplaw.inc"
#undef REAL
#undef F
#define REAL float
#define F(name) name##_f32
#include "steplaw.inc"
#undef REAL
#undef F

static int ntpo_source_of(const uint64_t* prefix, int n_src, uint64_t gid) {
    int lo = 0, hi = n_src - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (prefix[mid] <= gid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

/* Simulates photons with global index [gid_begin, gid_end) over the sources
   concatenated in order (double precision); writes hits in increasing global
   index.  Returns the number of hits, which may exceed cap (then only the
   first cap are written). */
static uint64_t ntpo_f64_run(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                             const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg, uint64_t seed,
                             const ntp_prop_opts* o, uint64_t gid_begin, uint64_t gid_end, ntp_hit* out,
                             uint64_t cap, int binned) {
    uint64_t* prefix = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n_src + 1));
    prefix[0] = 0;
    for (int i = 0; i < n_src; ++i) prefix[i + 1] = prefix[i] + src[i].photons;
    ntpo_bins bins;
    if (n_tg == 0) binned = 0;
    if (binned) ntpo_bins_build(&bins, tg, n_tg);
    uint64_t n = 0;
    for (uint64_t gid = gid_begin; gid < gid_end && gid < prefix[n_src]; ++gid) {
        int s = ntpo_source_of(prefix, n_src, gid);
        ntp_hit h;
        if (propagate_one_f64(&src[s], (uint32_t)s, gid - prefix[s], m, sp, tg, n_tg, seed, o,
                              binned ? &bins : NULL, &h)) {
            if (n < cap) out[n] = h;
            ++n;
        }
    }
    if (binned) ntpo_bins_free(&bins);
    free(prefix);
    return n;
}

uint64_t ntpo_propagate_f64(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                            const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg,
                            uint64_t seed, const ntp_prop_opts* o, uint64_t gid_begin,
                            uint64_t gid_end, ntp_hit* out, uint64_t cap) {
    return ntpo_f64_run(src, n_src, m, sp, tg, n_tg, seed, o, gid_begin, gid_end, out, cap, 0);
}

/* The same with the bucket-grid candidate lookup (ntpo_bins): the same hits
   as the scan over every target, for detectors of thousands of modules. */
uint64_t ntpo_propagate_f64_binned(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                                   const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg,
                                   uint64_t seed, const ntp_prop_opts* o, uint64_t gid_begin,
                                   uint64_t gid_end, ntp_hit* out, uint64_t cap) {
    return ntpo_f64_run(src, n_src, m, sp, tg, n_tg, seed, o, gid_begin, gid_end, out, cap, 1);
}

static uint64_t ntpo_f32_run(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                             const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg, uint64_t seed,
                             const ntp_prop_opts* o, uint64_t gid_begin, uint64_t gid_end, ntp_hit* out,
                             uint64_t cap, int n_threads, int binned) {
    uint64_t* prefix = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(n_src + 1));
    prefix[0] = 0;
    for (int i = 0; i < n_src; ++i) prefix[i + 1] = prefix[i] + src[i].photons;
    if (gid_end > prefix[n_src]) gid_end = prefix[n_src];
    ntpo_bins bins;
    if (n_tg == 0) binned = 0;
    if (binned) ntpo_bins_build(&bins, tg, n_tg);
    const ntpo_bins* bp = binned ? &bins : NULL;
    uint64_t n = 0;
    long long b = (long long)gid_begin, e = (long long)gid_end;
#pragma omp parallel for schedule(dynamic, 4096) num_threads(n_threads > 0 ? n_threads : 1)
    for (long long gid = b; gid < e; ++gid) {
        int s = ntpo_source_of(prefix, n_src, (uint64_t)gid);
        ntp_hit h;
        if (propagate_one_f32(&src[s], (uint32_t)s, (uint64_t)gid - prefix[s], m, sp, tg, n_tg,
                              seed, o, bp, &h)) {
            uint64_t slot;
#pragma omp atomic capture
            slot = n++;
            if (slot < cap) out[slot] = h;
        }
    }
    if (binned) ntpo_bins_free(&bins);
    free(prefix);
    return n;
}

/* Single-precision mirror over photons [gid_begin, gid_end) with OpenMP
   threads; used as the timed CPU baseline.  Returns the hit count; hits are
   written (unordered) up to cap. */
uint64_t ntpo_propagate_f32(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                            const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg,
                            uint64_t seed, const ntp_prop_opts* o, uint64_t gid_begin,
                            uint64_t gid_end, ntp_hit* out, uint64_t cap, int n_threads) {
    return ntpo_f32_run(src, n_src, m, sp, tg, n_tg, seed, o, gid_begin, gid_end, out, cap, n_threads, 0);
}

/* The same with the bucket-grid candidate lookup (ntpo_bins) in place of the
   scan over every target: the same hits, for detectors of thousands of
   modules. */
uint64_t ntpo_propagate_f32_binned(const ntp_source* src, int n_src, const ntp_medium_desc* m,
                                   const ntp_spectrum_desc* sp, const ntp_target* tg, int n_tg,
                                   uint64_t seed, const ntp_prop_opts* o, uint64_t gid_begin,
                                   uint64_t gid_end, ntp_hit* out, uint64_t cap, int n_threads) {
    return ntpo_f32_run(src, n_src, m, sp, tg, n_tg, seed, o, gid_begin, gid_end, out, cap, n_threads, 1);
}

/* ------------------------------------------------------------------------
 * Hit post-processing, photon_prop_cuda.jl:850-924 and detection.jl:60-163. */

/* PMT axes of MultiPMTDetector under `orientation` (get_pmt_positions,
   detection.jl:60-70): orientation * sph_to_cart(theta, phi) with the
   spherical-to-Cartesian step in single precision, as the coordinates are
   Float32 there, and the product in double. */
void ntpo_pmt_axes(const double R[9], const float* theta_phi, int n, double* axes) {
    for (int j = 0; j < n; ++j) {
        float th = theta_phi[2 * j], ph = theta_phi[2 * j + 1];
        float st = sinf(th), ct = cosf(th), s_p = sinf(ph), c_p = cosf(ph);
        double v[3] = {(double)(c_p * st), (double)(s_p * st), (double)ct};
        for (int r = 0; r < 3; ++r)
            axes[3 * j + r] = R[3 * r + 0] * v[0] + R[3 * r + 1] * v[1] + R[3 * r + 2] * v[2];
    }
}

/* check_pmt_hit for a batch of hits (detection.jl:72-104): 1-based PMT index
   or 0.  Targets are looked up by module_id. */
void ntpo_make_hits(const ntp_hit* hits, uint64_t n, const ntp_target* tg, int n_tg,
                    const float* pmt_coords, const double R[9], int32_t* pmt_id) {
    for (uint64_t i = 0; i < n; ++i) {
        const ntp_target* t = NULL;
        for (int k = 0; k < n_tg; ++k)
            if (tg[k].module_id == hits[i].module_id) { t = &tg[k]; break; }
        if (!t) { pmt_id[i] = 0; continue; }
        if (t->kind == NTP_TARGET_SPHERE) { pmt_id[i] = 1; continue; }
        float pmt_radius = sqrtf(t->pmt_area / (float)NTPO_PI);
        double opening = (double)asinf(pmt_radius / t->radius);
        double rel[3];
        for (int r = 0; r < 3; ++r) rel[r] = (double)hits[i].position[r] - (double)t->position[r];
        double nr = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2]);
        for (int r = 0; r < 3; ++r) rel[r] /= nr;
        double axes[3 * 64];
        int np = t->n_pmts > 64 ? 64 : t->n_pmts;
        ntpo_pmt_axes(R, pmt_coords + 2 * t->pmt_offset, np, axes);
        int id = 0;
        for (int j = 0; j < np; ++j) {
            double dp = rel[0] * axes[3 * j] + rel[1] * axes[3 * j + 1] + rel[2] * axes[3 * j + 2];
            if (dp < -1.0) dp = -1.0;
            if (dp > 1.0) dp = 1.0;
            if (acos(dp) < opening) { id = j + 1; break; }
        }
        pmt_id[i] = id;
    }
}

/* calc_total_weight!, photon_prop_cuda.jl:850-882.  Absorption follows
   fast_linear_interp on Float32 knots (medium.jl:399-404); the acceptance
   table is a linear interpolation on double knots (detection.jl:148-163). */
void ntpo_total_weight(const ntp_hit* hits, uint64_t n, const ntp_target* tg, int n_tg,
                       const float* abs_wl, const float* abs_len, int n_abs,
                       const double* acc_wl, const double* acc, int n_acc,
                       double* area_acc, double* wl_acc, double* abs_weight, double* total) {
    float* xs = (float*)malloc(sizeof(float) * (size_t)n_abs);
    float* ys = (float*)malloc(sizeof(float) * (size_t)n_abs);
    memcpy(xs, abs_wl, sizeof(float) * (size_t)n_abs);
    memcpy(ys, abs_len, sizeof(float) * (size_t)n_abs);
    for (uint64_t i = 0; i < n; ++i) {
        const ntp_target* t = NULL;
        for (int k = 0; k < n_tg; ++k)
            if (tg[k].module_id == hits[i].module_id) { t = &tg[k]; break; }
        double aa = 0.0;
        if (t) {
            if (t->kind == NTP_TARGET_SPHERE) {
                float total_pmt_area = (float)t->n_pmts * t->pmt_area;
                float r2 = t->radius * t->radius;
                aa = (double)total_pmt_area / (4.0 * NTPO_PI * (double)r2);
            } else {
                aa = 1.0;
            }
        }
        float wl = hits[i].wavelength;
        float al = fast_linear_interp_f32(wl, xs, ys, n_abs);
        double aw = (double)expf(-hits[i].dist_travelled / al);
        double wa = fast_linear_interp_f64((double)wl, acc_wl, acc, n_acc);
        if (area_acc) area_acc[i] = aa;
        if (wl_acc) wl_acc[i] = wa;
        if (abs_weight) abs_weight[i] = aw;
        if (total) total[i] = aa * wa * aw;
    }
    free(xs);
    free(ys);
}

/* calc_time_residual!, photon_prop_cuda.jl:906-924 */
void ntpo_time_residual(const ntp_hit* hits, uint64_t n, const ntp_target* tg, int n_tg,
                        const float src_pos[3], float n800, double* tres) {
    for (uint64_t i = 0; i < n; ++i) {
        const ntp_target* t = NULL;
        for (int k = 0; k < n_tg; ++k)
            if (tg[k].module_id == hits[i].module_id) { t = &tg[k]; break; }
        if (!t) { tres[i] = (double)NAN; continue; }
        float dx = src_pos[0] - t->position[0], dy = src_pos[1] - t->position[1],
              dz = src_pos[2] - t->position[2];
        float distance = sqrtf(dx * dx + dy * dy + dz * dz);
        double tgeo = (double)(distance - t->radius) / (NTPO_C_VAC / (double)n800);
        tres[i] = (double)hits[i].time - tgeo;
    }
}

/* ------------------------------------------------------------------------
 * Known-answer helpers (test/runtests.jl) and medium formulas (medium.jl). */

int ntpo_check_intersection(const double c[3], double radius, const double pos[3],
                            const double dir[3], double step, double* d) {
    vec3_f64 p = {pos[0], pos[1], pos[2]}, u = {dir[0], dir[1], dir[2]};
    return check_intersection_f64(c[0], c[1], c[2], radius, p, u, step, d);
}

int ntpo_check_intersection_f32(const float c[3], float radius, const float pos[3],
                                const float dir[3], float step, float* d) {
    vec3_f32 p = {pos[0], pos[1], pos[2]}, u = {dir[0], dir[1], dir[2]};
    return check_intersection_f32(c[0], c[1], c[2], radius, p, u, step, d);
}

void ntpo_rot_from_ez(const double a[3], const double v[3], int exact_pole, double out[3]) {
    vec3_f64 r = rot_from_ez_f64((vec3_f64){a[0], a[1], a[2]}, (vec3_f64){v[0], v[1], v[2]}, exact_pole);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ntpo_rot_to_ez(const double a[3], const double v[3], double out[3]) {
    vec3_f64 r = rot_to_ez_f64((vec3_f64){a[0], a[1], a[2]}, (vec3_f64){v[0], v[1], v[2]});
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

void ntpo_sph_to_cart(double theta, double phi, double out[3]) {
    vec3_f64 r = sph_to_cart_f64(theta, phi);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

/* cart_to_sph, utils.jl:118-133 */
void ntpo_cart_to_sph(const double v[3], double* theta, double* phi) {
    double x = v[0], y = v[1], z = v[2];
    if (z == 1) { *theta = 0; *phi = 0; return; }
    if (z == -1) { *theta = NTPO_PI; *phi = 0; return; }
    *theta = acos(z);
    if (x == 0 && y > 0) *phi = NTPO_PI / 2;
    else if (x == 0 && y < 0) *phi = -NTPO_PI / 2;
    else *phi = atan2(y, x);
}

/* calc_rot_matrix + apply_rot, utils.jl:173-197: rotation taking a to b
   (Rodrigues form I + [c]x + [c]x^2 (1 - a.b)/|c|^2, c = a x b), applied to v
   and normalised. */
void ntpo_apply_rot(const double a[3], const double b[3], const double v[3], double out[3]) {
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (!(a[0] == b[0] && a[1] == b[1] && a[2] == b[2])) {
        double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double S[9] = {0, -c[2], c[1], c[2], 0, -c[0], -c[1], c[0], 0};
        double S2[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 3; ++k) s += S[3 * i + k] * S[3 * k + j];
                S2[3 * i + j] = s;
            }
        double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        double nc2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        for (int i = 0; i < 9; ++i) R[i] += S[i] + S2[i] * (1 - ab) / nc2;
    }
    double r[3];
    for (int i = 0; i < 3; ++i) r[i] = R[3 * i] * v[0] + R[3 * i + 1] * v[1] + R[3 * i + 2] * v[2];
    double nr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (int i = 0; i < 3; ++i) out[i] = r[i] / nr;
}

/* 10-point Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on
   P_10), for integrate_gauss_quad, utils.jl:17 and :91-103. */
static void ntpo_gl10(double x[10], double w[10]) {
    const int n = 10;
    for (int i = 0; i < n; ++i) {
        double z = cos(NTPO_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) break;
        }
        x[i] = -z;
        w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

double ntpo_integrate_gauss_quad(double (*f)(double, void*), void* ctx, double a, double b) {
    double x[10], w[10];
    ntpo_gl10(x, w);
    double half = (b - a) / 2, mid = (a + b) / 2, s = 0;
    for (int i = 0; i < 10; ++i) s += w[i] * f(half * x[i] + mid, ctx) * half;
    return s;
}

void ntpo_gauss_legendre_10(double* x, double* w) { ntpo_gl10(x, w); }

/* _calc_quan_fry_params, medium.jl:174-205 */
void ntpo_quan_fry_params(double salinity, double temperature, double pressure, double out[4]) {
    double n0 = 1.31405, n1 = 1.45e-5, n2 = 1.779e-4, n3 = 1.05e-6, n4 = 1.6e-8, n5 = 2.02e-6,
           n6 = 15.868, n7 = 0.01155, n8 = 0.00423, n9 = 4382, n10 = 1.1455e6;
    out[0] = n0 + (n2 - n3 * temperature + n4 * temperature * temperature) * salinity -
             n5 * temperature * temperature + n1 * pressure;
    out[1] = n6 + n7 * salinity - n8 * temperature;
    out[2] = -n9;
    out[3] = n10;
}

/* refractive_index_fry, medium.jl:234-244 */
double ntpo_refractive_index_fry(double wl, const double p[4]) {
    double x = 1.0 / wl, x2 = x * x;
    return fma(x, p[1], p[0]) + fma(x2, p[2], x2 * x * p[3]);
}

/* dispersion_fry, medium.jl:293-298, including the unpacking of the first
   three of the four parameters into (a2, a3, a4). */
double ntpo_dispersion_fry(double wl, const double p[4]) {
    double a2 = p[0], a3 = p[1], a4 = p[2];
    double x = 1.0 / wl;
    return (a2 + 2.0 * x * a3 + 3.0 * x * x * a4) * -1.0 / (wl * wl);
}

/* group_velocity, medium.jl:313-318 (lambda_0 = n * lambda as written) */
double ntpo_group_velocity(double wl, const double p[4]) {
    double n = ntpo_refractive_index_fry(wl, p);
    double l0 = n * wl;
    return NTPO_C_VAC / (n - l0 * ntpo_dispersion_fry(wl, p));
}

/* _sca_len_part_conc, medium.jl:331-347 */
double ntpo_scattering_length(double wl, double vol_small, double vol_large) {
    double x = 550.0 / wl;
    double c = 0.0017 * pow(x, 4.3) + 1.34 * vol_small * pow(x, 1.7) + 0.312 * vol_large * pow(x, 0.3);
    return 1.0 / c;
}

/* DIPPR105, medium.jl:46-48 (temperature in K) */
double ntpo_dippr105(double temperature) {
    double A = 0.14395, B = 0.0112, C = 649.727, D = 0.05107;
    return A / pow(B, 1 + pow(1 - temperature / C, D));
}

/* frank_tamm, spectrum.jl:32-34, and frank_tamm_norm, :42-45, for the
   Quan-Fry refractive index */
typedef struct { const double* p; } ntpo_ft_ctx;
static double ntpo_ft_integrand(double wl, void* c) {
    double n = ntpo_refractive_index_fry(wl, ((ntpo_ft_ctx*)c)->p);
    return 2 * NTPO_PI * NTPO_FINE_STRUCTURE / (wl * wl) * (1 - 1 / (n * n));
}
double ntpo_frank_tamm_norm(double wl_lo, double wl_hi, const double p[4]) {
    ntpo_ft_ctx c = {p};
    return ntpo_integrate_gauss_quad(ntpo_ft_integrand, &c, wl_lo, wl_hi) * 1e9;
}

/* Wavelength samples of the first n photons of a source (for spectrum
   tests): the same draw the propagation uses. */
void ntpo_sample_wavelengths(const ntp_spectrum_desc* sp, uint64_t seed, uint32_t src_index,
                             uint64_t n, double* out) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t c[4] = {NTPO_DRAW_INIT_A, (uint32_t)i, (uint32_t)(i >> 32), src_index}, A[4];
        ntpo_philox4x32_10(c, key, A);
        out[i] = sample_wavelength_f64(sp, A[0]);
    }
}

/* Gamma variates as drawn for photon i of an extended source (tests). */
void ntpo_sample_gamma(float shape, float scale, uint64_t seed, uint32_t src_index, uint64_t n,
                       double* out) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t base[4] = {0, (uint32_t)i, (uint32_t)(i >> 32), src_index};
        out[i] = rand_gamma_f64((double)shape, (double)scale, base, key);
    }
}

/* Scattering cosines for tests of the phase functions. */
double ntpo_hg_costheta(double g, double eta) { return hg_costheta_f64(g, eta); }
double ntpo_rayleigh_costheta(double u) { return rayleigh_costheta_f64(u); }

/* ------------------------------------------------------------------------
 * resample_simulation, pmt_frontend/pipeline.jl:86-116 (per_pmt = true),
 * with the random draws of the device version: Poisson counts from the
 * Philox stream of each (module, PMT) group (inversion below a mean of 30,
 * Hormann's PTRS above), and the weighted draw without replacement as the N
 * largest exponential keys log(u)/w (Efraimidis-Spirakis), u from the Philox
 * stream of each hit's (source, photon). */
#define NTPO_DRAW_RESAMPLE_KEY 0x52534B59u
#define NTPO_DRAW_POISSON 0x504F4953u

static double ntpo_u01_53(uint32_t a, uint32_t b) {
    uint64_t m = ((uint64_t)a << 21) ^ (b >> 11);
    return ((double)(m & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
}

static uint64_t ntpo_ordered(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

double ntpo_poisson(double lam, uint64_t seed, uint32_t group) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)}, r[4];
    if (!(lam > 0.0)) return 0.0;
    if (lam < 30.0) {
        uint32_t c[4] = {NTPO_DRAW_POISSON, group, 0u, 0u};
        ntpo_philox4x32_10(c, key, r);
        double u = ntpo_u01_53(r[0], r[1]), p = exp(-lam), F = p, k = 0.0;
        while (u > F && k < 1000.0) {
            k += 1.0;
            p *= lam / k;
            F += p;
        }
        return k;
    }
    double slam = sqrt(lam), loglam = log(lam);
    double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
    double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int t = 0; t < 64; ++t) {
        uint32_t c[4] = {NTPO_DRAW_POISSON, group, (uint32_t)t + 1u, 0u};
        ntpo_philox4x32_10(c, key, r);
        double U = ntpo_u01_53(r[0], r[1]) - 0.5, V = ntpo_u01_53(r[2], r[3]);
        double us = 0.5 - fabs(U);
        double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= vr) return k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
    }
    return floor(lam + 0.5);
}

typedef struct { uint64_t key, hit; } ntpo_keyed;
static int ntpo_desc(const void* a, const void* b) {
    uint64_t x = ((const ntpo_keyed*)a)->key, y = ((const ntpo_keyed*)b)->key;
    return x < y ? 1 : (x > y ? -1 : 0);
}

/* Returns the number of drawn hits; writes (group, time, hit index) grouped by
   increasing group, each group by decreasing key, up to cap. */
uint64_t ntpo_resample(const ntp_hit* hits, uint64_t n, const int32_t* pmt, const double* w, const double* tval,
                       const ntp_target* tg, int n_tg, int max_pmts, double downsample, uint64_t seed,
                       int32_t* out_group, double* out_time, uint64_t* out_hit, uint64_t cap) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    size_t G = (size_t)n_tg * (size_t)max_pmts;
    int32_t* grp = (int32_t*)malloc(sizeof(int32_t) * (n ? n : 1));
    double* wsum = (double*)calloc(G ? G : 1, sizeof(double));
    uint64_t* npos = (uint64_t*)calloc(G ? G : 1, sizeof(uint64_t));
    for (uint64_t i = 0; i < n; ++i) {
        int k = -1;
        for (int t = 0; t < n_tg; ++t)
            if (tg[t].module_id == hits[i].module_id) { k = t; break; }
        grp[i] = -1;
        if (k >= 0 && pmt[i] > 0 && pmt[i] <= max_pmts) {
            grp[i] = k * max_pmts + pmt[i] - 1;
            wsum[grp[i]] += w[i];
            if (w[i] > 0.0) npos[grp[i]]++;
        }
    }
    uint64_t total = 0;
    ntpo_keyed* buf = (ntpo_keyed*)malloc(sizeof(ntpo_keyed) * (n ? n : 1));
    for (size_t g = 0; g < G; ++g) {
        double kk = ntpo_poisson(wsum[g] * downsample, seed, (uint32_t)g);
        uint64_t want = kk < (double)npos[g] ? (uint64_t)kk : npos[g];
        if (!want) continue;
        uint64_t m = 0;
        for (uint64_t i = 0; i < n; ++i) {
            if (grp[i] != (int32_t)g || !(w[i] > 0.0)) continue;
            uint32_t c[4] = {NTPO_DRAW_RESAMPLE_KEY, (uint32_t)hits[i].photon_index,
                             (uint32_t)(hits[i].photon_index >> 32), hits[i].source_index}, r[4];
            ntpo_philox4x32_10(c, key, r);
            buf[m].key = ntpo_ordered(log(ntpo_u01_53(r[0], r[1])) / w[i]);
            buf[m].hit = i;
            ++m;
        }
        qsort(buf, m, sizeof(ntpo_keyed), ntpo_desc);
        for (uint64_t q = 0; q < want; ++q, ++total) {
            if (total < cap) {
                uint64_t i = buf[q].hit;
                if (out_group) out_group[total] = (int32_t)g;
                if (out_time) out_time[total] = tval ? tval[i] : (double)hits[i].time;
                if (out_hit) out_hit[total] = i;
            }
        }
    }
    free(buf);
    free(grp);
    free(wsum);
    free(npos);
    return total;
}
