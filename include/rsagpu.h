/*
 * rsagpu.h -- C ABI of the GB300 sampler (bias-free maximal Poisson-sphere
 * sampling by random sequential addition with voxel subdivision).
 *
 * Plain C types only: opaque handles, pointers to host buffers and sizes.
 * Every function returns RSAGPU_OK (0) or a negative status; the text of the
 * last error of the calling thread is returned by rsagpu_last_error().
 *
 * Each entry point names the reference interface it replaces
 * (MarcJos/RSA_MPI, file:line).  The reference is header-only C++; its Python
 * binding (Interface_python/Interface.cxx) is replaced by the ctypes module
 * rsa_mpi_gb300.rsa_mpi_py, and its C++ facade by include/rsa_gpu/user_interface.hxx.
 *
 * Threading: one CUDA stream per algo handle.  Calls on one handle are not
 * thread-safe; calls on different handles are.  All device memory of a
 * domain lives on the GPU that was current when the domain was created.
 */
#ifndef RSAGPU_H
#define RSAGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSAGPU_MAX_DIM 7

/* status codes */
#define RSAGPU_OK 0
#define RSAGPU_ERR_ARG (-1)          /* invalid argument (std::runtime_error in the reference) */
#define RSAGPU_ERR_CUDA (-2)         /* CUDA runtime failure (allocation, launch) */
#define RSAGPU_ERR_NO_PROGRESS (-3)  /* a device loop hit its iteration cap */
#define RSAGPU_ERR_STATE (-4)        /* call out of order (e.g. refine before begin) */
#define RSAGPU_ERR_INVARIANT (-5)    /* a device check failed (two centres in one cell, ...) */
#define RSAGPU_ERR_PIVOT (-6)        /* count-cap pivot search failed (the reference throws here) */
#define RSAGPU_ERR_CAPACITY (-7)     /* a size limit of this build was exceeded */

typedef struct rsagpu_domain rsagpu_domain;
typedef struct rsagpu_radgen rsagpu_radgen;
typedef struct rsagpu_algo rsagpu_algo;

const char* rsagpu_last_error(void);
/* Library version string. */
const char* rsagpu_version(void);
/* Number of CUDA kernels this process launched through the library (for accounting). */
uint64_t rsagpu_kernel_launches(void);

/* ---- domain: replaces ::rsa_domain<DIM> / user_interface::rsa_domain<DIM>
 *      (include/rsa_domain.hxx:18-94, include/user_interface.hxx:13-53).
 * The periodic box [inf, sup]; rad_max bounds the radius of every sphere placed in it
 * (the reference's cell size / ghost width, rsa_domain.ixx:6-28). */
int rsagpu_domain_create(int dim, const double* inf, const double* sup, double rad_max,
                         rsagpu_domain** out);
int rsagpu_domain_destroy(rsagpu_domain* dom);
/* get_total_volume (rsa_domain.ixx:164-168) */
int rsagpu_domain_total_volume(const rsagpu_domain* dom, double* out);
/* compute_total_volume_of_spheres (rsa_domain.ixx:170-175) */
int rsagpu_domain_spheres_volume(rsagpu_domain* dom, double* out);
/* number of spheres placed (rsa_grid::get_number_of_spheres_fast, rsa_grid.hxx:64) */
int rsagpu_domain_count(rsagpu_domain* dom, uint64_t* out);
/* extract_spheres (rsa_grid.ixx:88-98): copies at most cap spheres into caller buffers
 * (centers: cap*dim doubles, row major; radii: cap; phases: cap; any may be NULL) in cell order,
 * and writes the number of spheres to *n_out.  Buffers in pinned host memory that the device addresses at
 * the same pointer (cudaHostAlloc's, with unified addressing) are written by the device directly; others
 * through a device copy.  The call returns when the buffers hold the spheres. */
int rsagpu_domain_extract(rsagpu_domain* dom, double* centers, double* radii, int* phases,
                          uint64_t cap, uint64_t* n_out);
/* operator_check_cell validators (operator_check_cell.ixx:8-78, rsa_data_storage.ixx:216-243):
 * number of overlapping pairs (exact FP64, periodic images) and of spheres stored in a cell that
 * does not contain their centre. */
int rsagpu_domain_check(rsagpu_domain* dom, uint64_t* overlapping_pairs, uint64_t* misplaced);

/* ---- radius generator: replaces sac_de_billes::RadiusGenerator<DIM>
 *      (include/radius_generator.hxx:46-105, radius_generator.ixx:9-86). */
/* (radius, count, phase) classes; placed by nonincreasing radius. */
int rsagpu_radgen_create_counts(int dim, const double* radii, const uint64_t* counts,
                                const int* phases, int n_classes, double exclusion_distance,
                                rsagpu_radgen** out);
/* (radius, volume fraction, phase) classes: count = uint64(volume * phi / v_D(r)). */
int rsagpu_radgen_create_fractions(int dim, const double* radii, const double* fractions,
                                   const int* phases, int n_classes, double volume,
                                   double exclusion_distance, rsagpu_radgen** out);
/* Continuous radius law: each dart's radius is r_min + (r_max - r_min) x, x uniform in [0, 1), and
 * count spheres are wanted (10^16: run to maximality).  Replaces sac_de_billes::RadiusGenerator<DIM>(
 * min_radius, max_radius, &RandomRadiusGenerator(transform, phase), nb_spheres, 0) with the uniform transform
 * (radius_generator.ixx:39-48, radius_generator.hxx:12-38, test/test_random_radius_generator.cpp:13-29). */
int rsagpu_radgen_create_uniform(int dim, double r_min, double r_max, uint64_t count, int phase,
                                 rsagpu_radgen** out);
/* Continuous radius law with any transform: knots[j] = transform(j / (n_knots - 1)), j = 0 .. n_knots - 1
 * (2 to 2^20 positive radii); each dart's radius is the transform interpolated linearly at its x, uniform in
 * [0, 1), kept within [min knots, max knots].  Replaces sac_de_billes::RadiusGenerator<DIM>(min_radius,
 * max_radius, &RandomRadiusGenerator(transform, phase), nb_spheres, 0) for an arbitrary std::function
 * transform (radius_generator.hxx:12-38, radius_generator.ixx:39-48), which the C++ facade tabulates. */
int rsagpu_radgen_create_table(int dim, const double* knots, int n_knots, uint64_t count, int phase,
                               rsagpu_radgen** out);
int rsagpu_radgen_destroy(rsagpu_radgen* rg);
int rsagpu_radgen_max_radius(const rsagpu_radgen* rg, double* out);
int rsagpu_radgen_min_radius(const rsagpu_radgen* rg, double* out);

/* ---- algorithm: replaces algorithm::rsa_algo<DIM> / user_interface::rsa_algo<DIM>
 *      (include/operator_algorithm.hxx:18-109, include/user_interface.hxx:85-110).
 * The algo keeps a reference to the domain (which must outlive it) and a copy of the
 * radius generator.  Creating it clears the spheres of the domain (operator_algorithm.ixx:15-30). */
int rsagpu_algo_create(rsagpu_domain* dom, const rsagpu_radgen* rg, int nbshots,
                       rsagpu_algo** out);
int rsagpu_algo_destroy(rsagpu_algo* algo);

/* precision form */
#define RSAGPU_FORM_FP64 0        /* every decision in FP64 */
#define RSAGPU_FORM_FP32_GUARD 1  /* FP32 decisions outside a guard band, FP64 inside it */
/* schedule of darts and subdivisions */
#define RSAGPU_SCHEDULE_HEURISTIC 0 /* darts per round from the voxel count, refine on miss rate */
#define RSAGPU_SCHEDULE_LEARNED 1   /* MLP decides when to refine (heuristic as fallback) */
#define RSAGPU_SCHEDULE_REFERENCE 2 /* the reference's round sizes: Poisson(min(nbshots, 0.01 V)) */
int rsagpu_algo_set_form(rsagpu_algo* algo, int form, int schedule);
/* No counterpart in the reference.  With on = 1 the FP32 form's 3D mask pass hands each surviving voxel's
 * nearby spheres to its children, which then test those and the spheres placed since instead of walking
 * their whole neighbourhood.  Off (the default) walks every neighbourhood.  The decisions are the same
 * either way. */
int rsagpu_algo_set_inherit(rsagpu_algo* algo, int on);
/* count cap of a round that would exceed the class count */
#define RSAGPU_CAP_REFERENCE 0    /* retain_only_first_elements pivot rule (operator_algorithm.ixx:475-519) */
#define RSAGPU_CAP_EXACT 1        /* exactly the remaining count, smallest priorities first */
int rsagpu_algo_set_cap_rule(rsagpu_algo* algo, int rule);
/* darts per round of the heuristic schedule = clamp(factor * voxels, min_darts, max_darts),
 * refinement when the round's miss rate exceeds miss_threshold (<= 0: the reference's rule,
 * operator_algorithm.ixx:344-351). */
int rsagpu_algo_set_schedule_params(rsagpu_algo* algo, double factor, uint64_t min_darts,
                                    uint64_t max_darts, double miss_threshold);
/* Learned schedule: weights of the 16-64-64-2 MLP (bf16 bit patterns, row major W1[64][16], b1[64],
 * W2[64][64], b2[64], W3[2][64], b3[2]; 16*64+64+64*64+64+2*64+2 = 5378 values). */
int rsagpu_algo_set_mlp(rsagpu_algo* algo, const uint16_t* weights_bf16, uint64_t n);

/* proceed(seed) (operator_algorithm.ixx:225-236, user_interface.hxx:101): runs rounds until no
 * voxel is left (certified maximal) or the class list is exhausted. */
int rsagpu_algo_proceed(rsagpu_algo* algo, uint64_t seed);
/* reset_radius_generator (operator_algorithm.ixx:238-250): keeps the placed spheres; the new
 * generator's largest radius may not exceed the current one. */
int rsagpu_algo_reset_radgen(rsagpu_algo* algo, const rsagpu_radgen* rg);

/* Per-round trace of the last proceed(): for each round the voxels before it, darts, accepted
 * spheres, refinement flag (1) and voxel level; returns the number of rounds in *n_out. */
int rsagpu_algo_trace(rsagpu_algo* algo, uint64_t* voxels, uint64_t* darts, uint64_t* accepted,
                      uint8_t* refined, int32_t* level, uint64_t cap, uint64_t* n_out);
/* Statistics of the last proceed(): rounds, refinements, darts, settle iterations, guard-band
 * retests, device milliseconds per kernel family (darts, probe, settle, commit, refine), and the count
 * cap's passes and classification steps (reference rule). */
typedef struct {
    uint64_t rounds, refinements, darts, accepted, settle_iterations, retests, peak_voxels;
    uint64_t bytes_darts, bytes_probe, bytes_settle, bytes_commit, bytes_refine;
    double ms_darts, ms_probe, ms_settle, ms_commit, ms_refine, ms_total;
    int32_t final_level, maximal;
    uint64_t cap_passes, cap_steps;
} rsagpu_stats;
int rsagpu_algo_stats(rsagpu_algo* algo, rsagpu_stats* out);
/* Per launch of the refinement's mask kernel in the last proceed(): device milliseconds (CUDA events
 * on the algo's stream around the launch) and algorithmic bytes (parent coordinates, stencil occupancy
 * bits up to the grid size, visited spheres up to the spheres placed, child masks). */
int rsagpu_algo_kernel_profile(rsagpu_algo* algo, double* ms, double* bytes, double* voxels, uint64_t cap,
                               uint64_t* n_out);
/* Learned schedule training data: after each pass the schedule's decision is flipped with probability
 * epsilon (host RNG seeded with seed).  0 = off (default). */
int rsagpu_algo_set_exploration(rsagpu_algo* algo, double epsilon, uint64_t seed);
/* Per round of the last proceed(): the 16 state features the schedule saw, whether it refined, and the
 * host wall time of the pass and of the refinement that followed. */
int rsagpu_algo_trace_features(rsagpu_algo* algo, float* features, uint8_t* refined, double* pass_ms,
                               double* refine_ms, uint64_t cap, uint64_t* n_out);
/* Turns per-kernel CUDA-event timing on (1) or off (0, default). */
int rsagpu_algo_set_timing(rsagpu_algo* algo, int on);

/* ---- replay seam (operator_algorithm.ixx:534-566 generate_spheres with injected candidate
 * generators; list_of_voxels.ixx:30-100).  Used to prove decision parity with the FP64 oracle. */
/* Builds the level-0 voxel list (list_of_voxels.ixx:11-28) and resets the round state. */
int rsagpu_algo_begin(rsagpu_algo* algo);
/* Decides n candidates (host arrays) against the placed spheres and among themselves, as one round
 * of generate_spheres; keys are priorities (smaller first, equal keys do not block each other).
 * accepted_out[i] = 1 for accepted candidates, *n_new = their number. */
int rsagpu_algo_replay_round(rsagpu_algo* algo, uint64_t n, const double* pos, const uint64_t* key,
                             const double* rad, const int* phase, uint64_t max_new,
                             int may_outreach, uint8_t* accepted_out, uint64_t* n_new);
/* Class bookkeeping and the miss-rate rule after a round (operator_algorithm.ixx:140-162);
 * *refined = 1 if the voxels were culled and subdivided, *done = 1 if no class is left. */
int rsagpu_algo_end_round(rsagpu_algo* algo, uint64_t n_shots, uint64_t n_new, int* refined,
                          int* done);
/* remove_covered + subdivide_uncovered, unconditionally (operator_algorithm.ixx:190-206). */
int rsagpu_algo_refine(rsagpu_algo* algo);
/* Current voxel list: count, level and length; coords (count*dim int64) may be NULL. */
int rsagpu_algo_voxels(rsagpu_algo* algo, int64_t* coords, uint64_t cap, uint64_t* count,
                       int32_t* level, double* length);
/* Draws one round of darts with the product's Philox stream (round r of seed) and copies the
 * candidates to host buffers (for checking the dart kernel); *n = number drawn. */
int rsagpu_algo_draw_darts(rsagpu_algo* algo, uint64_t seed, uint64_t round, uint64_t n,
                           double* pos, uint64_t* key, uint64_t* voxel_index);

/* ---- batched instances ----
 * No counterpart in the reference, which runs one domain per process (rsa_algo::proceed_voxel,
 * operator_algorithm.ixx:85-188).  Runs n independent one-radius instances to certified maximality:
 * instance i is the box [0, sup[0..dim-1]] with spheres of one radius and the Philox key seed.  It places
 * exactly the spheres of its own single-instance run: rsagpu_domain_create([0], sup, radius),
 * rsagpu_radgen_create_fractions({radius}, {1.0}, {0}, 1, box volume, 0), rsagpu_algo_create(.., 6000),
 * rsagpu_algo_set_form(form, RSAGPU_SCHEDULE_HEURISTIC) with the default schedule, rsagpu_algo_proceed(seed).
 * The instances of one dimension advance together, one launch sequence per round over every unfinished
 * instance, in waves whose estimated device memory fits max_bytes (0 = 60% of the free memory).  With
 * autotune != 0 the block shapes of the probe, collect, settle and voxel-mask kernels are chosen by timing
 * (outputs never depend on them).  Outputs per instance (each pointer may be NULL): counts_out = spheres;
 * checksums_out = sum mod 2^64 over its spheres of h, where h starts at 0x9E3779B97F4A7C15 and for each
 * coordinate x_d in order becomes mix64(h ^ bits(x_d)) (mix64 = splitmix64's output function:
 * z ^= z >> 30; z *= 0xbf58476d1ce4e5b9; z ^= z >> 27; z *= 0x94d049bb133111eb; z ^= z >> 31);
 * seconds_out = time from the call's start until the instance was certified maximal. */
typedef struct {
    int dim;
    double sup[RSAGPU_MAX_DIM];  /* box [0, sup] */
    double radius;               /* the one radius */
    uint64_t seed;               /* Philox key of the instance's darts */
} rsagpu_instance_desc;
typedef struct {
    double seconds;              /* wall time of the call */
    uint64_t waves, rounds, darts, retests, peak_voxels, launches, budget_bytes;
    int32_t block[RSAGPU_MAX_DIM + 1][4]; /* threads per block chosen per dimension for probe, collect,
                                             settle, voxel mask (0 = not tuned) */
} rsagpu_batch_stats;
int rsagpu_batch_run(const rsagpu_instance_desc* inst, int n, int form, uint64_t max_bytes, int autotune,
                     uint64_t* counts_out, uint64_t* checksums_out, double* seconds_out,
                     rsagpu_batch_stats* stats_out);

/* ---- learned schedule: MLP kernels (16-64-64-2, bf16 weights, fp32 accumulate) ---- */
/* forward: x[n][16] (fp32) -> y[n][2] (fp32), weights as rsagpu_algo_set_mlp */
int rsagpu_mlp_forward(const uint16_t* weights_bf16, const float* x, uint64_t n, float* y);
/* one training step of mean squared error on (x, target): returns the loss and the gradient of every
 * weight (fp32, same layout), and applies SGD with learning rate lr to the master fp32 weights
 * (in/out), refreshing weights_bf16. */
int rsagpu_mlp_train_step(float* master_weights, uint16_t* weights_bf16, const float* x,
                          const float* target, uint64_t n, float lr, float* loss_out,
                          float* grad_out);

/* ---- conflict resolution that allocates nothing ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc: code running inside
 * another framework's memory pool or under its allocator, a real-time loop whose device memory is
 * fixed up front, or a library that must not touch the device heap.  The caller passes device
 * buffers: d_pos (n*dim doubles, row major, every centre within [inf, sup]), d_key (n priorities,
 * smaller first, ties broken by the index), d_rad (n radii, none above r_max; a radius above it or a
 * centre outside the box is found on the device and refused with RSAGPU_ERR_ARG, with d_accepted left
 * unwritten) and d_accepted (n bytes, written 1 for an accepted
 * candidate, 0 otherwise).  The result is the same-round decision of the sampler: the sequential
 * greedy in priority order on the periodic box [inf, sup] (inf and sup are host arrays), with no
 * placed spheres.  Every temporary lives in one static device array of the library, sized for at most
 * RSAGPU_NOALLOC_MAX_CANDIDATES candidates (about 10.5 MB, held by every GPU that loads the library
 * until the process exits); larger batches are refused with RSAGPU_ERR_CAPACITY.  The first call on a
 * device looks up the array's device address with that device current (cudaGetSymbolAddress) and
 * keeps it for the life of the process, so a cudaDeviceReset between calls is not supported; make
 * that first call before any stream capture.  Every call shares the one array and it keeps the last
 * call's contents: calls that overlap on the GPU race and give wrong results.  Work runs on `stream`
 * (a cudaStream_t, NULL = the default stream); the call synchronises `stream` and returns when the
 * output is written. */
#define RSAGPU_NOALLOC_MAX_CANDIDATES (1u << 18)
int rsagpu_resolve_batch_noalloc(int dim, const double* inf, const double* sup, double r_max,
                                 const double* d_pos, const uint64_t* d_key, const double* d_rad,
                                 uint64_t n, uint8_t* d_accepted, void* stream);

#ifdef __cplusplus
}
#endif
#endif
