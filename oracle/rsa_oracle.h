/*
 * rsa_oracle: CPU restatement of the reference sampler's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library, and only as the
 * checker or the CPU baseline; the GPU library never links or calls it.
 *
 * What it restates (MarcJos/RSA_MPI, file:line):
 *   - the round loop of rsa_algo::proceed_voxel       include/operator_algorithm.ixx:85-188
 *   - Poisson shot count / intensity / miss-rate rule  include/operator_algorithm.ixx:208-223, 344-351
 *   - candidate generation (centres, priorities)       include/list_of_voxels.ixx:107-129,
 *                                                      include/operator_algorithm.ixx:373-381, 568-582
 *   - decisions of generate_spheres / add_to_sample    include/operator_algorithm.ixx:383-443, 534-566,
 *     as the sequential greedy in priority order       include/operator_cells_and_data_storage.ixx:5-143
 *   - remove_covered / subdivide_uncovered             include/list_of_voxels.ixx:30-100, 225-318
 *   - RadiusGenerator class bookkeeping                include/radius_generator.ixx:9-86
 *   - the random stream of law::create_random_generator include/rsa_random.hxx:8-42: std::mt19937,
 *     std::seed_seq, and the libstdc++ (GCC 13) algorithms behind uniform_int_distribution<int>,
 *     uniform_real_distribution<double> and poisson_distribution<int>.
 *
 * Parity pin: fed the same seed, a full run reproduces the reference's sphere
 * set bit for bit (tests/golden/, made by oracle/_ref/ref_rsa).
 */
#ifndef RSA_ORACLE_H
#define RSA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_DIM 7

typedef struct rsa_oracle rsa_oracle;

/* Class list (r, count, phase), sorted and adjusted like RadiusGenerator(vector<tuple<double,uint64_t,int>>, excl)
 * (radius_generator.ixx:9-28).  domain_rad is the rsa_domain radius (cell size / ghost width). */
rsa_oracle* ora_create(int dim, const double* inf, const double* sup, double domain_rad,
    int n_classes, const double* radii, const uint64_t* counts, const int* phases,
    double exclusion_distance, int nbshots);
void ora_destroy(rsa_oracle* o);

/* A continuous radius law: radius = r_min + (r_max - r_min) x per dart, x ~ U[0, 1), <count> spheres wanted
 * (RadiusGenerator with a RandomRadiusGenerator, radius_generator.ixx:39-48, radius_generator.hxx:12-38). */
rsa_oracle* ora_create_uniform(int dim, const double* inf, const double* sup, double r_min, double r_max,
    uint64_t count, int phase, int nbshots);
/* the uniform law's transform replaced by one tabulated at x = j / (n - 1) (the radius generator's r_min and
 * r_max must be the knots' range) */
int ora_set_radius_table(rsa_oracle* o, const double* knots, int n);

/* rsa_algo::reset_radius_generator (operator_algorithm.ixx:238-250): new classes, same spheres; r_max stays the
 * larger one.  Returns -2 for a larger maximal radius (the reference throws). */
int ora_reset_classes(rsa_oracle* o, int n_classes, const double* radii, const uint64_t* counts,
    const int* phases, double exclusion_distance);

/* uint64(volume * phi / v_D(r)) as compute_desired_radius_nb_phase (radius_generator.ixx:71-86). */
uint64_t ora_count_from_fraction(int dim, double r, double phi, double volume);
/* v_D(r) as sphereTools::volumeSphere (auxiliary/Geometry/Sphere.ixx:30-57). */
double ora_volume_sphere(int dim, double r);

/* ---- full run with the reference's random stream ---- */
int ora_proceed(rsa_oracle* o, uint64_t seed);

/* ---- lockstep interface (the replay seam) ---- */
/* Builds the level-0 voxel list and seeds mt19937 with seed_seq{0, seed}. */
int ora_begin(rsa_oracle* o, uint64_t seed);
/* Draws one round with the reference's stream.  Returns 0 = round drawn (n may be 0),
 * 1 = no voxel left (certified maximal), 2 = no class left.  Candidates are readable through
 * ora_cand_* until the next call. */
int ora_gen_round(rsa_oracle* o, uint64_t* n_out, uint64_t* max_new, int* may_outreach);
const double* ora_cand_pos(const rsa_oracle* o);     /* n*dim, row major */
const uint64_t* ora_cand_key(const rsa_oracle* o);   /* priority (31-bit) */
const double* ora_cand_rad(const rsa_oracle* o);
const int* ora_cand_phase(const rsa_oracle* o);
/* Decides a batch of candidates against the validated set and among themselves, inserts the
 * accepted ones.  accepted_out[i] = 1 if candidate i is accepted.  Candidates are ordered by
 * (key, index): equal keys are broken by the candidate index (the reference's detection sees
 * strictly smaller priorities only, operator_cells_and_data_storage.ixx:39, and so accepts both
 * of two overlapping equal-priority candidates). */
int ora_apply_round(rsa_oracle* o, uint64_t n, const double* pos, const uint64_t* key,
    const double* rad, const int* phase, uint64_t max_new, int may_outreach,
    uint8_t* accepted_out, uint64_t* n_new);
/* Class bookkeeping + miss rate + voxel update of one round.  refined_out = 1 when the voxels
 * were culled and subdivided.  Returns 1 if the class list is exhausted. */
int ora_end_round(rsa_oracle* o, uint64_t n_shots, uint64_t n_new, int* refined_out);
/* remove_covered then subdivide_uncovered, unconditionally. */
int ora_refine(rsa_oracle* o);

uint64_t ora_voxel_count(const rsa_oracle* o);
/* coords: count*dim int64; len: dim doubles (current voxel length) */
int ora_voxel_export(const rsa_oracle* o, int64_t* coords, double* len);
int ora_voxel_level(const rsa_oracle* o);

uint64_t ora_sphere_count(const rsa_oracle* o);
int ora_sphere_export(const rsa_oracle* o, double* pos, double* rad, int* phase);
/* inserts already-validated spheres (no checks) */
int ora_sphere_import(rsa_oracle* o, uint64_t n, const double* pos, const double* rad, const int* phase);

/* Per-round trace of the last run: voxels before the round, shots, new spheres, refined flag. */
uint64_t ora_trace_len(const rsa_oracle* o);
int ora_trace_export(const rsa_oracle* o, uint64_t* voxels, uint64_t* shots, uint64_t* news, uint8_t* refined);

double ora_min_radius(const rsa_oracle* o);
double ora_max_radius(const rsa_oracle* o);

/* Count cap of a round that would exceed the class count: 0 (default) = the reference's
 * retain_only_first_elements pivot rule, which can keep fewer than the count; 1 = exactly the
 * smallest-priority count. */
void ora_set_cap_exact(rsa_oracle* o, int exact);
/* median_of_medians::find_pivot_for_first_elements restated; -1 where the reference throws. */
int ora_ref_pivot(const uint64_t* values, int64_t n, int64_t n_first, double* pivot_out);

/* ---- checkers ---- */
/* Number of pairs i<j with dist2(i, periodic image of j) < (r_i + r_j)^2, exact FP64, images by
 * per-coordinate x_j +/- L as the reference's ghost copies (rsa_ghost_area.ixx:22-30). */
uint64_t ora_count_overlaps(int dim, const double* inf, const double* sup, uint64_t n,
    const double* pos, const double* rad);
/* Certifies maximality: builds the level-0 voxel list for (r_max + r_min) and refines it until
 * empty or max_levels is reached.  Returns the voxels left (0 = maximal). */
uint64_t ora_uncovered_after_refinement(int dim, const double* inf, const double* sup,
    uint64_t n, const double* pos, const double* rad, double r_max, double r_min, int max_levels);

/* ---- raw RNG restatement, for tests ---- */
typedef struct { uint32_t x[624]; int i; } ora_mt19937;
void ora_mt_seed_seq(ora_mt19937* g, const uint32_t* seeds, int n_seeds);
uint32_t ora_mt_next(ora_mt19937* g);
double ora_canonical(ora_mt19937* g);
uint32_t ora_uniform_int(ora_mt19937* g, uint32_t lo, uint32_t hi);
int ora_poisson(ora_mt19937* g, double mean);

/* ---- Philox-4x32-10 restatement (Salmon et al., SC'11) for checking the GPU dart stream ---- */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
