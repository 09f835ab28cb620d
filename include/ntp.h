/*
 * ntp.h -- C ABI of the GB300-native photon-propagation library (libntp.so).
 *
 * The library replaces the photon-propagation hot path of NeutrinoTelescopes
 * (Julia + CUDA.jl).  Every entry point below names the reference function it
 * stands in for.  All structs are plain old data with fixed sizes, all
 * buffers are raw pointers plus element counts, and every call returns an
 * ntp_status.  A context is used by one host thread at a time (or is
 * synchronised by the caller).
 *
 * Units follow the reference: metres, nanoseconds, nanometres, radians.
 */
#ifndef NTP_H
#define NTP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NTP_ABI_VERSION 2

typedef enum ntp_status {
    NTP_OK = 0,
    NTP_ERR_INVALID = 1,   /* bad argument: null pointer, size out of range, unknown kind   */
    NTP_ERR_OVERFLOW = 2,  /* hit buffer too small: hits truncated, returned counts exact   */
    NTP_ERR_CUDA = 3,      /* CUDA runtime error; text in ntp_last_error()                 */
    NTP_ERR_NOT_READY = 4, /* medium, spectrum or targets not set on the context           */
    NTP_ERR_TIMEOUT = 5,   /* a bounded wait gave up                                        */
    NTP_ERR_NOMEM = 6      /* device allocation failed or an HBM budget would be exceeded   */
} ntp_status;

/* ------------------------------------------------------------------ sources
 * Photon emitters, src/photon_propagation/lightyield.jl:421-530.  One record
 * type carries every emitter kind; fields a kind does not use are ignored.   */
enum ntp_source_kind {
    NTP_SRC_POINT_ISOTROPIC = 0,    /* PointlikeIsotropicEmitter   lightyield.jl:436-440 */
    NTP_SRC_POINT_TIME_RANGE = 1,   /* PointlikeTimeRangeEmitter   lightyield.jl:449-453 */
    NTP_SRC_AXICONE = 2,            /* AxiconeEmitter              lightyield.jl:421-427 */
    NTP_SRC_PENCIL = 3,             /* PencilEmitter               lightyield.jl:429-434 */
    NTP_SRC_EXTENDED_CHERENKOV = 4, /* ExtendedCherenkovEmitter    lightyield.jl:463-481 */
    NTP_SRC_POINT_CHERENKOV = 5,    /* PointlikeCherenkovEmitter   lightyield.jl:491-509 */
    NTP_SRC_CHERENKOV_TRACK = 6     /* CherenkovTrackEmitter       lightyield.jl:519-530 */
};

typedef struct ntp_source {  /* 64 bytes */
    float position[3];
    float time;          /* emission time (ns); start of the range for TIME_RANGE       */
    float direction[3];  /* unit vector (AXICONE, PENCIL, Cherenkov kinds)               */
    float angle;         /* AXICONE opening angle (rad)                                  */
    uint64_t photons;    /* number of photons to emit                                    */
    int32_t kind;        /* enum ntp_source_kind                                         */
    float time_end;      /* TIME_RANGE end of the range (ns)                             */
    float long_a;        /* EXTENDED_CHERENKOV: gamma shape a of the longitudinal profile */
    float long_b;        /* EXTENDED_CHERENKOV: gamma rate b                              */
    float long_lrad;     /* EXTENDED_CHERENKOV: radiation length (m)                      */
    float length;        /* CHERENKOV_TRACK: track length (m)                             */
} ntp_source;

/* ------------------------------------------------------------------ targets
 * Optical modules, src/photon_propagation/detection.jl:29-46.               */
enum ntp_target_kind {
    NTP_TARGET_SPHERE = 0,    /* DetectionSphere   detection.jl:29-36 */
    NTP_TARGET_MULTI_PMT = 1  /* MultiPMTDetector  detection.jl:39-46 */
};

typedef struct ntp_target {  /* 48 bytes */
    float position[3];
    float radius;
    uint32_t module_id;   /* written into every hit on this module                     */
    int32_t kind;         /* enum ntp_target_kind                                      */
    float pmt_area;       /* m^2                                                       */
    int32_t n_pmts;       /* SPHERE: PMT count (area acceptance); MULTI_PMT: PMTs in layout */
    int32_t pmt_offset;   /* MULTI_PMT: first (theta, phi) pair in the PMT coordinate table */
    int32_t reserved[3];
} ntp_target;

/* --------------------------------------------------------------------- hits
 * One photon that reached a module, PhotonHit photon_prop_cuda.jl:391-399,
 * plus the photon's identity so that a run can be replayed and photons can be
 * assigned to their sources.  64 bytes, 16-byte aligned, stored as an array. */
typedef struct ntp_hit {
    float position[3];
    float time;
    float direction[3];          /* direction at the hit                        */
    float wavelength;
    float initial_direction[3];  /* direction at emission                       */
    float dist_travelled;
    uint32_t module_id;
    uint32_t source_index;       /* index of the source in the ntp_propagate call */
    uint64_t photon_index;       /* index of the photon within its source        */
} ntp_hit;

/* ------------------------------------------------------------------- medium
 * Water optics, src/photon_propagation/medium.jl.  The per-photon quantities
 * are tabulated by the caller on a uniform wavelength grid (the caller
 * evaluates its own refractive_index / group_velocity / scattering_length at
 * the knots); absorption is a per-hit weight on its own, possibly non-uniform,
 * knots, as in medium.jl:392-414.                                            */
typedef struct ntp_medium_desc {
    int32_t n_knots;               /* >= 2, <= NTP_MAX_MEDIUM_KNOTS                         */
    float wl_min;                  /* nm, first knot                                        */
    float wl_max;                  /* nm, last knot                                         */
    const float* ref_index;        /* phase refractive index n(lambda), medium.jl:234-244   */
    const float* group_velocity;   /* m/ns, medium.jl:313-318                               */
    const float* scattering_length;/* m, medium.jl:331-370                                  */
    int32_t n_abs_knots;           /* >= 2, <= NTP_MAX_ABS_KNOTS                             */
    const float* abs_wavelength;   /* nm, ascending                                         */
    const float* abs_length;       /* m, medium.jl:392-414                                  */
    float hg_g;                    /* Henyey-Greenstein mean cosine, photon_prop_cuda.jl:70-77 */
    float rayleigh_fraction;       /* share of Rayleigh scatters, 0 for the reference medium */
} ntp_medium_desc;

#define NTP_MAX_MEDIUM_KNOTS 2048
#define NTP_MAX_ABS_KNOTS 1024

/* ----------------------------------------------------------------- spectrum
 * Wavelength sampling, src/photon_propagation/spectrum.jl:89-108 and
 * photon_prop_cuda.jl:128-130.                                               */
enum ntp_spectrum_kind {
    NTP_SPEC_MONOCHROMATIC = 0,  /* Monochromatic spectrum.jl:21-23                          */
    NTP_SPEC_TABLE_LINEAR = 1,   /* inverse-CDF knots at u = k/(n-1), linear interpolation   */
    NTP_SPEC_TABLE_TEXTURE = 2,  /* inverse-CDF knots read like the reference's 1-D texture:
                                    normalised coordinate u*n-0.5, clamp, linear filter with
                                    an 8-bit fraction (spectrum.jl:102-103)                  */
    NTP_SPEC_INV_SQUARE = 3      /* dN/dlambda ~ 1/lambda^2 on [wl_min, wl_max], exact inverse */
};

typedef struct ntp_spectrum_desc {
    int32_t kind;              /* enum ntp_spectrum_kind                         */
    int32_t n_knots;           /* TABLE kinds: >= 2, <= NTP_MAX_SPECTRUM_KNOTS    */
    const float* icdf_knots;   /* TABLE kinds: wavelength (nm) at each knot      */
    float wl_min;              /* INV_SQUARE range (nm)                           */
    float wl_max;
    float wavelength;          /* MONOCHROMATIC wavelength (nm)                   */
} ntp_spectrum_desc;

#define NTP_MAX_SPECTRUM_KNOTS 4096

/* ---------------------------------------------------------- propagation opts */
enum ntp_hit_policy {
    NTP_HIT_FIRST_IN_LIST = 0,  /* first intersecting target in list order wins, photon_prop_cuda.jl:460-468 */
    NTP_HIT_NEAREST = 1         /* nearest intersecting target wins                                       */
};

enum ntp_prop_flags {
    /* rot_from_ez_fast (utils.jl:228-243) maps v to (v1, copysign(v2,a3), copysign(v3,a3))
       when |a3| == 1.  By default that is reproduced; this flag applies the true rotation. */
    NTP_FLAG_EXACT_POLE_ROTATION = 1,
    /* Test every target at every step (the reference's linear scan,
       photon_prop_cuda.jl:460-468) instead of culling by vertical columns;
       the hits are the same either way. */
    NTP_FLAG_PLAIN_SCAN = 2
};

typedef struct ntp_prop_opts {
    int32_t max_steps;   /* scatter steps per photon, photon_prop_cuda.jl:449 uses 15 */
    int32_t hit_policy;  /* enum ntp_hit_policy                                       */
    int32_t flags;       /* enum ntp_prop_flags                                       */
    int32_t reserved;
    void* stream;        /* cudaStream_t for device-buffer calls; NULL = context stream */
} ntp_prop_opts;

/* -------------------------------------------------------------------- calls */
typedef struct ntp_ctx ntp_ctx;

/* ABI version compiled into the library (NTP_ABI_VERSION). */
int ntp_abi_version(void);

/* Creates a context on CUDA device `device`.  Replaces the implicit CUDA.jl
   device state used by run_photon_prop_no_local_cache, photon_prop_cuda.jl:726-759. */
ntp_status ntp_create(int device, ntp_ctx** out);
void ntp_destroy(ntp_ctx* ctx);

/* Text of the last error on this context ("" if none).  With ctx == NULL,
   the last error of a context-free call (ntp_create, ntp_propagate_noalloc)
   on the calling thread; each such call clears it first. */
const char* ntp_last_error(const ntp_ctx* ctx);

/* Medium of PhotonPropSetup (photon_prop_cuda.jl:34-39): copies the tables to
   the device. */
ntp_status ntp_set_medium(ntp_ctx* ctx, const ntp_medium_desc* medium);

/* Spectrum of PhotonPropSetup; replaces the CuTexture built by
   CherenkovSpectrum, spectrum.jl:97-106. */
ntp_status ntp_set_spectrum(ntp_ctx* ctx, const ntp_spectrum_desc* spectrum);

/* Targets of PhotonPropSetup (CuVector(targets), photon_prop_cuda.jl:740),
   with the (theta, phi) PMT coordinate table of MultiPMTDetector
   (pmt_coords holds n_pmt_coords pairs; may be NULL if no MULTI_PMT target). */
ntp_status ntp_set_targets(ntp_ctx* ctx, const ntp_target* targets, int32_t n_targets,
                           const float* pmt_coords, int32_t n_pmt_coords);

/* propagate_photons(setup), photon_prop_cuda.jl:804-817 with the kernel
   cuda_propagate_photons!, :402-506.  Simulates every photon of every source
   and appends hits to `hits` (capacity records).  hits_on_device != 0: `hits`
   is a device pointer and the call is asynchronous on opts->stream except for
   the final count read; otherwise `hits` is host memory.  On return
   *n_hits is the exact number of hits (it may exceed capacity: then
   NTP_ERR_OVERFLOW, and the first `capacity` slots are filled) and
   *n_photons_simulated the number of photons stepped.  Photon k of source s
   draws its random numbers from the Philox4x32-10 counter (draw, k, s) under
   key `seed`, so a rerun with the same arguments yields the same set of hits. */
ntp_status ntp_propagate(ntp_ctx* ctx, const ntp_source* sources, int32_t n_sources,
                         uint64_t seed, const ntp_prop_opts* opts,
                         ntp_hit* hits, uint64_t capacity, int32_t hits_on_device,
                         uint64_t* n_hits, uint64_t* n_photons_simulated);

/* ntp_propagate without any allocation.  This entry point has no counterpart
   in the reference.  It is for callers that cannot call cudaMalloc: a data-
   taking or trigger process that reserves its device memory at start-up and
   must not allocate afterwards (cudaMalloc synchronises the device and can
   fail on fragmented memory), or a host framework whose device buffers all
   come from its own pool.  Such a caller owns the output hit buffer (device
   memory, 16-byte aligned) and passes the inputs as host descriptors, as for
   ntp_set_medium / ntp_set_spectrum / ntp_set_targets / ntp_propagate; no
   context is needed.  The kernel's scratch (counters, source table and prefix
   sums, medium, spectrum and target tables) lives in a fixed 256 KiB device
   array inside the library, so the call allocates nothing.  Limits: at most
   1024 sources, 4096 targets, NTP_MAX_MEDIUM_KNOTS medium knots and
   NTP_MAX_SPECTRUM_KNOTS spectrum knots; more is rejected with
   NTP_ERR_INVALID, as are tables that ntp_set_medium / ntp_set_spectrum
   reject and a hit buffer on another device than the current one.  Every
   target is tested at every step (no column culling or grid walk): the same
   hits as ntp_propagate, at a cost that grows with the number of targets
   (a few per cent on a 20-module string, many times ntp_propagate's time on
   thousands of modules).  The scratch is shared by all calls on a device: calls
   that overlap on the GPU race and must be serialised by the caller.  The
   first call on a device looks up the scratch address on that device (the
   current device); make that first call before any stream capture.  Uses
   opts->stream (NULL = the legacy default stream) and returns once the hit
   count is known; the error text is ntp_last_error(NULL). */
ntp_status ntp_propagate_noalloc(const ntp_medium_desc* medium, const ntp_spectrum_desc* spectrum,
                                 const ntp_target* targets, int32_t n_targets,
                                 const ntp_source* sources, int32_t n_sources, uint64_t seed,
                                 const ntp_prop_opts* opts, ntp_hit* hits, uint64_t capacity,
                                 uint64_t* n_hits, uint64_t* n_photons_simulated);

/* Counters of the last ntp_propagate on this context (no reference
   counterpart beyond n_ph_sim of photon_prop_cuda.jl:758). */
typedef struct ntp_run_stats {
    uint64_t photons;        /* photons simulated                                  */
    uint64_t hits;           /* hits found (may exceed the buffer capacity)         */
    uint64_t photon_steps;   /* scatter segments stepped over all photons          */
    int32_t grid;            /* blocks launched                                    */
    int32_t block;           /* threads per block                                  */
    uint64_t chunk;          /* photons a warp claims at once                      */
} ntp_run_stats;

ntp_status ntp_get_run_stats(const ntp_ctx* ctx, ntp_run_stats* out);

/* make_hits_from_photons, photon_prop_cuda.jl:884-904 with check_pmt_hit,
   detection.jl:88-104: for each hit the 1-based index of the PMT whose
   opening cone contains the hit position, 0 for none.  `orientation` is a
   row-major 3x3 rotation applied to every module's PMT axes.  A hit on a
   SPHERE target gets PMT 1 (detection.jl:86).  buffers_on_device selects
   device or host pointers for hits and pmt_id. */
ntp_status ntp_make_hits(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits,
                         const double orientation[9], int32_t* pmt_id,
                         int32_t buffers_on_device, void* stream);

/* calc_total_weight!, photon_prop_cuda.jl:850-882: per hit the area
   acceptance (detection.jl:139-146), the PMT wavelength acceptance
   (detection.jl:148-163, table set by ntp_set_wavelength_acceptance) and the
   absorption weight exp(-dist/abs_length(lambda)).  Any output pointer may be
   NULL.  total_weight = area_acc * wl_acc * abs_weight. */
ntp_status ntp_calc_total_weight(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits,
                                 double* area_acc, double* wl_acc, double* abs_weight,
                                 double* total_weight, int32_t buffers_on_device, void* stream);

/* Wavelength acceptance table of one PMT (assets/PMTAcc.csv in the
   reference, detection.jl:161-163): n ascending knots, linear interpolation. */
ntp_status ntp_set_wavelength_acceptance(ntp_ctx* ctx, const double* wavelength,
                                         const double* acceptance, int32_t n);

/* calc_time_residual!, photon_prop_cuda.jl:906-924: tres = time - tgeo(module),
   tgeo = (|source_position - module_position| - radius) / (c_vac / n800),
   n800 = refractive index at 800 nm. */
ntp_status ntp_calc_time_residual(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits,
                                  const float source_position[3], float n800,
                                  double* tres, int32_t buffers_on_device, void* stream);

/* Per-PMT reduction of a hit set in double precision (no single reference
   counterpart: it fuses make_hits_from_photons, calc_total_weight! and
   calc_time_residual!, photon_prop_cuda.jl:850-924, with the per-(module,
   PMT) grouping of pmt_frontend/pipeline.jl:104-116).  For every hit on a
   PMT: weight_sum[k][j] += total weight, hit_count[k][j] += 1 and, with
   n_bins > 0, time_hist[k][j][bin] += total weight, where k is the target's
   index in ntp_set_targets, j the 0-based PMT and the binned time either the
   hit time or the time residual.  Outputs are zeroed first; any may be NULL
   except that time_hist is needed when n_bins > 0. */
typedef struct ntp_summary_spec {
    int32_t max_pmts;          /* PMT slots per target; >= every target's PMT count       */
    int32_t n_bins;            /* time-histogram bins over [t_min, t_max), 0 for none     */
    float t_min;               /* ns                                                      */
    float t_max;
    int32_t use_time_residual; /* 1: bin time - tgeo(module) as calc_time_residual!        */
    float source_position[3];  /* for the time residual                                   */
    float n800;                /* refractive index at 800 nm, for the time residual       */
} ntp_summary_spec;

ntp_status ntp_pmt_summary(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits, const double orientation[9],
                           const ntp_summary_spec* spec, double* weight_sum, double* hit_count, double* time_hist,
                           int32_t buffers_on_device, void* stream);

/* resample_simulation (pmt_frontend/pipeline.jl:86-116) with per_pmt = true:
   hits grouped by (module, PMT) with pmt_id from ntp_make_hits (0 = none) and
   weight from ntp_calc_total_weight; per group N = min(Poisson(sum(weight) *
   downsample), number of hits with weight > 0), then N hits drawn without
   replacement with probability proportional to weight.  Outputs, grouped by
   group g = target_index * max_pmts + pmt_id - 1 in increasing g: out_group,
   out_time (the input time, or the hit time when time is NULL) and out_hit
   (index of the drawn hit); any output may be NULL.  The random draws are
   keyed by seed and by each hit's (source_index, photon_index), so the
   result does not depend on the order of the hits.  *n_out receives the
   total; above capacity nothing is written and NTP_ERR_OVERFLOW returned. */
ntp_status ntp_resample(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits, const int32_t* pmt_id,
                        const double* weight, const double* time, int32_t max_pmts, double downsample,
                        uint64_t seed, int32_t* out_group, double* out_time, uint64_t* out_hit,
                        uint64_t capacity, uint64_t* n_out, int32_t buffers_on_device, void* stream);

/* --------------------------------------------------- flow training tables
 * run_sim of scripts/photon_tables.jl:52-170 for many simulations at once.
 * The context holds exactly one MULTI_PMT target (the module); the hits of
 * one propagation launch over n_sims sources (source_index = simulation) and
 * their weights (ntp_calc_total_weight) are on the device; sim_weight_scale
 * (host, per simulation, may be NULL = 1) multiplies the weights: photons of
 * the source over photons simulated (the reference's oversampling
 * correction, photon_tables.jl:110).  For each
 * simulation s and each of n_orientations module orientations r
 * (orientations[(s * R + r) * 9 ..], row-major, PMT axes rotated as
 * ntp_make_hits does), every hit is assigned to the PMT whose cone contains
 * it (FP32 dot product against cos of the opening angle) and each (s, r,
 * PMT) group is resampled as ntp_resample does, except that the group count
 * N = Poisson(sum(w) * downsample) is not capped by the number of simulated
 * hits (with weights scaled up, fewer photons than the source's may have
 * been simulated); min(N, #hits with w > 0, max_rows_per_group) hits are
 * drawn without replacement (see the cap below), each a row: cond[5] (the group's condition
 * features), tres (hit time minus (|source - module| - R) n800 / c,
 * calc_time_residual!), nhits = N, has_time = 1, row_group (may be NULL) =
 * the group's index.  With zero_rows a group with N = 0 gives one row with
 * has_time = 0, nhits = 0.  The rows drawn from a group are also capped at a
 * quarter of its effective sample size (sum w)^2 / sum w^2 plus one, so that
 * they stay a weighted sample when N approaches the simulated hits.  Condition features of a group
 * (u = unit vector module -> source, a = PMT axis, v = source direction):
 * 2 ln(d)/ln(200) - 1, v.u, a.u, phi/pi - 1 with phi in [0, 2 pi) the angle
 * from the projection of v to that of a on the plane normal to u (around u),
 * (log10 E - 4)/2.  Outputs are device buffers; the group outputs (n_sims * R
 * * n_pmts entries: features, expected count sum(w) * downsample, drawn
 * count, simulated hits with w > 0) may be NULL.  *n_rows receives the row count; above capacity
 * nothing is written and NTP_ERR_OVERFLOW returned. */
typedef struct ntp_table_spec {
    int32_t n_sims;             /* simulations = sources of the propagation launch          */
    int32_t n_orientations;     /* R module orientations per simulation (n_resample)          */
    int32_t max_rows_per_group; /* rows kept per (simulation, orientation, PMT), e.g. 200      */
    int32_t zero_rows;          /* 1: a count-only row for a group that draws no hit          */
    double downsample;          /* resample_simulation's downsample                           */
    float n800;                 /* refractive index of the time residual                      */
    int32_t reserved;
    uint64_t seed;              /* Philox key of the counts and the draws                     */
} ntp_table_spec;

ntp_status ntp_make_table(ntp_ctx* ctx, const ntp_hit* hits, uint64_t n_hits, const double* weight,
                          const ntp_source* sims, const float* sim_log10_energy, const double* sim_weight_scale,
                          const double* orientations, const ntp_table_spec* spec, float* cond, float* tres,
                          float* nhits, int32_t* has_time, int32_t* row_group, uint64_t capacity, uint64_t* n_rows,
                          float* group_cond, double* group_expec, uint64_t* group_count, uint64_t* group_hits,
                          void* stream);

/* Flow conditions of every (event, module, PMT) with the module within
   [d_min, d_max] of the event's vertex (the surrogate's domain): events are
   cascades (position, direction of each ntp_source; log10_energy per event;
   event_id may be NULL = the index).  Per row: cond[5] (the features of
   ntp_make_table), cond_key = event_id << 32 | target_index << 8 | pmt
   (the sampler's stream key), cond_tgeo = (|vertex - module| - R) n800 / c
   (time = time residual + tgeo + event time), and the event index, target
   index and 1-based PMT (these three may be NULL).  Modules are upright.
   Rows are grouped by event: event_first (host, n_events + 1) are the
   offsets; event_close (host, may be NULL) counts the modules closer than
   d_min (outside the domain) per event.  Outputs device buffers; *n_cond
   receives the total, above capacity nothing is written and
   NTP_ERR_OVERFLOW returned.  No reference counterpart (the reference builds
   flow inputs on the host, extended_cascade_model.jl:367-437). */
ntp_status ntp_event_conditions(ntp_ctx* ctx, const ntp_source* events, const float* log10_energy,
                                const uint32_t* event_id, int32_t n_events, float d_min, float d_max, float n800,
                                float* cond, uint64_t* cond_key, float* cond_tgeo, int32_t* cond_event,
                                int32_t* cond_target, int32_t* cond_pmt, uint64_t capacity, uint64_t* n_cond,
                                uint64_t* event_first, int32_t* event_close, void* stream);

/* ------------------------------------------------------------ tensor cores
 * C = A * B^T with BF16 A [M x K] and B [N x K] (row-major, K contiguous,
 * device pointers, 16-byte aligned rows: lda, ldb multiples of 8, K a
 * multiple of 64), FP32 accumulation on the tensor cores (tcgen05 + TMA),
 * plus bias[N] (FP32, may be NULL) and optional ReLU.  out_kind 0 stores
 * FP32, 1 stores BF16, 2 adds FP32 atomically (with splits > 1 the K range is
 * split across CTAs; C must be zeroed first).  The GEMM of the flow's
 * conditioner network (no reference counterpart: the reference uses
 * Flux Dense layers, extended_cascade_model.jl:53-101). */
ntp_status ntp_gemm_bf16(const void* A, int32_t lda, const void* B, int32_t ldb, void* C, int32_t ldc, int32_t M,
                         int32_t N, int32_t K, const float* bias, int32_t relu, int32_t out_kind, int32_t splits,
                         void* stream);

/* Failure detection of the tensor-core GEMM (no reference counterpart; the
 * reference's only device check, the @cuassert of photon_prop_cuda.jl:484,
 * kills the context).  Every mbarrier wait of the GEMM pipeline gives up after
 * wait_limit_ns of the GPU's global timer (0 = the default, 2 s), sets an
 * error word, lets its copies in flight land, frees its tensor memory and
 * returns; ntp_gemm_bf16 (and the flow calls built on it) then return
 * NTP_ERR_TIMEOUT and the context stays usable.  The same limit and switch
 * govern the flow's fused layer-chain kernel (its first wait is for its
 * input tile) and the grouped weight-gradient GEMM.  withhold_first_copy != 0
 * makes the following launches leave out the first pipeline stage's copies
 * (the chain: its input tile), so that the first wait has nothing to
 * complete and runs out: this is how the timeout path is tested (outputs are
 * undefined while it is set).  Process-wide; applies to launches made after
 * the call.  NTP_GEMM_PDL=0 in the environment turns off the programmatic
 * dependent launch of these kernels and of the flow's other kernels. */
ntp_status ntp_gemm_set_wait_limit(uint64_t wait_limit_ns, int32_t withhold_first_copy);

/* --------------------------------------------------------- arrival-time flow
 * The per-module arrival-time surrogate: RQNormFlow with a log-expectation
 * head (src/surrogate_models/extended_cascade_model.jl:53-139, with the
 * spline of rq_spline_flow.jl:170-418), trained and evaluated on the GPU.
 * Conditioner: 5 condition features -> 3 ReLU layers of 256 -> per spline
 * layer 3K+1 raw values (K bins on [t_min, t_max]), then shift, raw scale and
 * log expectation; n_layers stacked inverse splines (1 = the reference's
 * model).  Weights BF16 on the tensor cores with FP32 accumulation, FP32
 * master weights and Adam (Flux's defaults).  Parameters form one flat FP32
 * vector: W1 [256 x 64] (only the first 5 input columns used, 9 with
 * derived columns), b1 [256],
 * W2 [256 x 256], b2, W3 [256 x 256], b3, W4 [n_outputs_padded x 256], b4;
 * rows of W4 beyond n_outputs stay zero. */
typedef struct ntp_flow ntp_flow;

typedef struct ntp_flow_config {
    int32_t batch_capacity; /* most samples per training step / conditions per pass; multiple of 128 */
    int32_t n_layers;       /* spline layers, 1..5                                           */
    int32_t n_bins;         /* K, bins per spline: 10 (the reference's default) or 12        */
    float t_min, t_max;     /* spline range (ns); linear tails outside                        */
    float lr, beta1, beta2, eps; /* Adam                                                      */
    float grad_clip;        /* per-sample bound on |dL/draw outputs| x batch (0 = none), e.g. 1e3 */
    float count_weight;     /* weight of the Poisson count term in the loss (1 = the reference's)  */
    uint64_t seed;          /* weight initialisation                                           */
    int32_t input_columns;  /* enum ntp_flow_input                                              */
    int32_t reserved;
} ntp_flow_config;

/* Input columns of the conditioner.  FEATURES: the 5 condition features.
   DERIVED: the features and four functions of them, computed on the device
   when the conditions are packed -- the distance / 100 m, the source
   direction's cosine minus the Cherenkov cosine 1/1.35 and its square, and
   sin(theta_pmt) cos(phi); a count-only model (hit expectations, trained
   without time rows) learns the steep count function much better with them,
   while they hurt the time shapes of a joint model. */
enum ntp_flow_input {
    NTP_FLOW_INPUT_FEATURES = 0,
    NTP_FLOW_INPUT_DERIVED = 1
};

ntp_status ntp_flow_create(int32_t device, const ntp_flow_config* config, ntp_flow** out);
void ntp_flow_destroy(ntp_flow* flow);
const char* ntp_flow_last_error(const ntp_flow* flow);
ntp_status ntp_flow_get_layout(const ntp_flow* flow, uint64_t* n_params, int32_t* n_outputs,
                               int32_t* n_outputs_padded);
/* Replaces the weights (host FP32, n = n_params) and resets Adam. */
ntp_status ntp_flow_set_lr(ntp_flow* flow, float lr);
ntp_status ntp_flow_set_params(ntp_flow* flow, const float* host, uint64_t n);
/* which: 0 weights, 1 gradient of the last training step, 2 / 3 Adam moments. */
ntp_status ntp_flow_get_params(ntp_flow* flow, float* host, uint64_t n, int32_t which);
/* One step of train_model! (extended_cascade_model.jl:237-295) on a batch of
   B samples (a multiple of 128): cond [B x 5], time residual tres [B],
   label hit count nhits [B], has_time [B] (0: the sample adds only the count
   term).  update = 0 computes loss and gradient without an Adam step.  All
   inputs on the host, or on the device when on_device != 0.  A step whose
   gradient is not finite (an FP32 overflow) is skipped: the weights and Adam
   state stay as they were and *loss is NaN. */
ntp_status ntp_flow_train_step(ntp_flow* flow, const float* cond, const float* tres, const float* nhits,
                               const int32_t* has_time, int32_t B, int32_t on_device, int32_t update,
                               double* loss);
/* n_steps training steps on consecutive batches of B rows (rows i*B ..
   (i+1)*B - 1 form step i), one synchronisation for all of them; losses
   (host, n_steps, may be NULL) receives each step's loss (NaN for a skipped
   step).  count_weight (may be NULL = 1 for every row) multiplies each row's
   Poisson count term: -(sum logpdf + sum c_i Poisson(n_i; exp(le_i))) / B;
   with c = 1 / (rows of the PMT) every PMT's count enters once (the
   reference's tables repeat it on each of the PMT's rows); with c = the
   PMT's simulated photons per emitted photon over its rows and nhits = its
   MC expectation, every PMT pulls in proportion to the hits simulated for
   it (the information-weighted count term).  nhits need not be an
   integer.  The training
   step itself is captured once as a CUDA graph and replayed
   (NTP_FLOW_GRAPH=0 in the environment runs it eagerly). */
ntp_status ntp_flow_train_steps(ntp_flow* flow, const float* cond, const float* tres, const float* nhits,
                                const int32_t* has_time, const float* count_weight, int32_t B, int32_t n_steps,
                                int32_t on_device, int32_t update, double* losses);
/* The conditioner's raw outputs for n conditions (host): params_out [n x n_outputs]. */
ntp_status ntp_flow_forward(ntp_flow* flow, const float* cond, int32_t n, float* params_out);
/* The loss and its gradient by the raw outputs, for given raw outputs
   params [B x n_outputs] (host buffers; B <= batch_capacity; count_weight
   as in ntp_flow_train_steps, may be NULL). */
ntp_status ntp_flow_head(ntp_flow* flow, const float* params, const float* tres, const float* nhits,
                         const int32_t* has_time, const float* count_weight, int32_t B, double* loss,
                         float* grad_out);
/* The model call (extended_cascade_model.jl:110-125): log p(t | cond) for
   n_tuples (condition index, time) pairs, and per condition the log
   expectation (log_expec may be NULL).  An index outside [0, n_cond) gives NaN. */
ntp_status ntp_flow_evaluate(ntp_flow* flow, const float* cond, int32_t n_cond, const int32_t* cond_index,
                             const float* times, uint64_t n_tuples, float* logpdf, float* log_expec,
                             int32_t on_device);
/* Only the log expectation of each condition (the count head, clamped as in
   ntp_flow_evaluate), without building spline knots: the count model's query
   in the hybrid simulator.  Leaves a pending ntp_flow_sample resumable.
   Host, or device buffers with on_device. */
ntp_status ntp_flow_log_expectation(ntp_flow* flow, const float* cond, int32_t n_cond, float* log_expec,
                                    int32_t on_device);
/* The model call on a time grid shared by the conditions, as the reference
   evaluates a module's density (`model(repeat(times), repeat(input))` on a
   111-point grid, extended_cascade_model.jl:416-437 and the scripts):
   logpdf[c * n_times + j] = log p(times[j] | cond[c]); log_expec as in
   ntp_flow_evaluate (may be NULL).  Host, or device buffers with on_device. */
ntp_status ntp_flow_evaluate_grid(ntp_flow* flow, const float* cond, int32_t n_cond, const float* times,
                                  int32_t n_times, float* logpdf, float* log_expec, int32_t on_device);
/* The pooled arrival-time CDF of a mixture of conditions:
   cdf[j] = sum_c w_c F(times[j] - offset[c] | cond[c]) / sum_c w_c, with F
   the flow's CDF (the base normal's CDF of the inverse-transformed time: the
   splines and the affine map are increasing bijections) and w_c = weight[c],
   or the condition's expected count exp(log expectation) when weight is
   NULL; offset may be NULL (0).  With the conditions of one event's PMTs and
   their geometric times as offsets this is the event's predicted hit-time
   CDF, the reference of a one-sample Kolmogorov-Smirnov test of Monte Carlo
   hits.  No reference counterpart.  Host, or device buffers with on_device;
   cdf in FP64. */
ntp_status ntp_flow_mixture_cdf(ntp_flow* flow, const float* cond, int32_t n_cond, const float* weight,
                                const float* offset, const float* times, uint64_t n_times, double* cdf,
                                int32_t on_device);

/* Sampling from the surrogate (the hits a PMT sees, as the MC would give
   them after resample_simulation): per condition c a count N_c ~
   Poisson(exp(log expectation)), then N_c times drawn from the flow (a
   normal draw through the forward splines, rqs_univariate,
   rq_spline_flow.jl:262-324).  Draws come from Philox streams keyed by seed
   and cond_key[c], so a condition's hits do not depend on the other
   conditions of the call.  Outputs grouped by condition in increasing c:
   hit_cond (the condition index) and hit_time; counts (may be NULL) per
   condition.  *n_hits receives the total; above capacity no hit is written
   (counts are) and NTP_ERR_OVERFLOW returned: the counts and offsets of
   the call are kept, and ntp_flow_sample_resume draws its hits into larger
   buffers without repeating the conditioner pass.  n_cond <= 1048576.  All
   buffers on the host, or on the device when on_device != 0.  No reference
   counterpart: the reference only evaluates the density. */
ntp_status ntp_flow_sample(ntp_flow* flow, const float* cond, int32_t n_cond, const uint64_t* cond_key, uint64_t seed,
                           uint64_t* counts, int32_t* hit_cond, float* hit_time, uint64_t capacity, uint64_t* n_hits,
                           int32_t on_device);
/* ntp_flow_sample with the counts drawn from the given log expectations
   (log_expec [n_cond], host or device as the other buffers; NULL = the
   flow's own count head) instead of this flow's: the hybrid simulator takes
   a PMT's expected hits from a separate count model and its arrival times
   from this flow.  A later ntp_flow_sample_resume draws the same hits. */
ntp_status ntp_flow_sample_expec(ntp_flow* flow, const float* cond, int32_t n_cond, const uint64_t* cond_key,
                                 uint64_t seed, const float* log_expec, uint64_t* counts, int32_t* hit_cond,
                                 float* hit_time, uint64_t capacity, uint64_t* n_hits, int32_t on_device);
/* The hits of the last ntp_flow_sample call that returned NTP_ERR_OVERFLOW,
   into buffers of at least its *n_hits entries (the same hits that call
   would have written).  Any other call on the flow in between discards the
   pending sample (NTP_ERR_NOT_READY). */
ntp_status ntp_flow_sample_resume(ntp_flow* flow, int32_t* hit_cond, float* hit_time, uint64_t capacity,
                                  uint64_t* n_hits, int32_t on_device);

/* ------------------------------------------------------------------ serving
 * Continuous-batching event server (no reference counterpart; the reference
 * runs one propagate_photons per event, photon_prop_cuda.jl:804-817).  Each
 * event is one source; its photons draw from the Philox stream of its
 * event_id, so an event's hits do not depend on which events share its batch.
 * Hits stay on the device in an arena of hbm_budget_bytes: an event is
 * admitted (FIFO) when a batch slot is free and its hit reservation fits in
 * the arena, and keeps its hits there until ntp_server_release.  Admitted
 * events are packed into one propagation launch per batch (a CUDA graph
 * replayed with new parameters); two batch slots on two streams let a new
 * batch start while the previous one drains.  With chunk_photons > 0 an
 * event enters a batch with at most that many of its photons (a chunk: the
 * photon indices a .. b-1 of its stream, written to the event's own arena
 * range) and goes back to the head of the queue for its next chunk (events
 * keep their arrival order), so a batch stays short and events that arrive
 * meanwhile join the next one instead of waiting behind a large event; an
 * event has at most one chunk in flight.  An event whose hits exceed its reservation is re-run whole with
 * the exact size (same hits).  The server uses the medium, spectrum and
 * targets of its context, which must not change while the server exists. */
typedef struct ntp_server ntp_server;

typedef struct ntp_server_config {
    uint64_t hbm_budget_bytes;      /* hit arena size (64 bytes per hit)                     */
    uint64_t seed;                  /* Philox key of every event                             */
    int32_t max_events_per_batch;   /* <= 65536                                              */
    int32_t max_steps;              /* scatter steps per photon (15 in the reference)        */
    int32_t hit_policy;             /* enum ntp_hit_policy                                   */
    int32_t flags;                  /* enum ntp_prop_flags                                   */
    double reserve_hits_per_photon; /* initial hit reservation per photon                    */
    uint64_t min_reserve_hits;      /* smallest reservation of an event                      */
    uint64_t max_batch_photons;     /* photons per batch before it is closed                 */
    uint64_t chunk_photons;         /* an event's photons per batch (0 = the whole event)     */
} ntp_server_config;

typedef struct ntp_event_result {
    uint32_t event_id;
    int32_t status;         /* NTP_OK, or NTP_ERR_NOMEM if the event can never fit the arena */
    uint64_t n_hits;
    uint64_t n_photons;
    const ntp_hit* hits;    /* device pointer into the arena, valid until ntp_server_release */
    double t_submit;        /* seconds on the server's clock                                */
    double t_launch;        /* launch of the batch that produced the hits                   */
    double t_done;          /* completion observed by ntp_server_poll                       */
    int32_t reruns;         /* re-runs after a reservation overflow                         */
    int32_t batch_events;   /* events in that batch                                          */
} ntp_event_result;

typedef struct ntp_server_stats {
    uint64_t queued, running, completed, released;
    uint64_t batches, photons;
    uint64_t arena_hits, arena_reserved_hits;
    double clock;           /* the server's clock now (seconds)                             */
} ntp_server_stats;

ntp_status ntp_server_create(ntp_ctx* ctx, const ntp_server_config* config, ntp_server** out);
void ntp_server_destroy(ntp_server* server);
/* Queues one event (stamped with the submit time). */
ntp_status ntp_server_submit(ntp_server* server, uint32_t event_id, const ntp_source* source);
/* Advances the loop (collects finished batches, admits queued events, launches
   batches) and returns up to max finished events in out, waiting up to
   timeout_us for one if none is ready.  Returns the number written, or -1
   on a CUDA error (text in ntp_last_error of the server's context). */
int32_t ntp_server_poll(ntp_server* server, ntp_event_result* out, int32_t max, int32_t timeout_us);
/* Copies up to max of a finished event's hits from the arena into host
   memory; *n receives the event's hit count. */
ntp_status ntp_server_copy_hits(ntp_server* server, uint32_t event_id, ntp_hit* host_dst, uint64_t max,
                                uint64_t* n);
/* Frees an event's hits in the arena. */
ntp_status ntp_server_release(ntp_server* server, uint32_t event_id);
ntp_status ntp_server_get_stats(const ntp_server* server, ntp_server_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* NTP_H */
