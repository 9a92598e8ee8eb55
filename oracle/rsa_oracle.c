/*
 * rsa_oracle.c -- CPU restatement of the reference sampler's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see rsa_oracle.h).  Written for clarity, not speed:
 * every FP64 expression follows the operation order of the reference source
 * line it cites, and the file must be compiled with -ffp-contract=off so that
 * no multiply-add is fused.
 */
#include "rsa_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ===================================================================== */
/* Random stream                                                         */
/* ===================================================================== */

/* std::seed_seq::generate ([rand.util.seedseq]) into 624 words, then
 * mersenne_twister_engine::seed(seq) ([rand.eng.mers]). */
void ora_mt_seed_seq(ora_mt19937* g, const uint32_t* v, int s) {
    const int n = 624;
    uint32_t* b = g->x;
    for (int i = 0; i < n; i++) b[i] = 0x8b8b8b8bu;
    const int t = 11; /* n >= 623 */
    const int p = (n - t) / 2;
    const int q = p + t;
    const int m = (s + 1 > n) ? s + 1 : n;
#define ORA_T(x) ((x) ^ ((x) >> 27))
    for (int k = 0; k < m; k++) {
        uint32_t a = b[k % n] ^ b[(k + p) % n] ^ b[(k - 1 + n) % n];
        uint32_t r1 = 1664525u * ORA_T(a);
        uint32_t r2;
        if (k == 0) r2 = r1 + (uint32_t)s;
        else if (k <= s) r2 = r1 + (uint32_t)(k % n) + v[k - 1];
        else r2 = r1 + (uint32_t)(k % n);
        b[(k + p) % n] += r1;
        b[(k + q) % n] += r2;
        b[k % n] = r2;
    }
    for (int k = m; k < m + n; k++) {
        uint32_t a = b[k % n] + b[(k + p) % n] + b[(k - 1 + n) % n];
        uint32_t r3 = 1566083941u * ORA_T(a);
        uint32_t r4 = r3 - (uint32_t)(k % n);
        b[(k + p) % n] ^= r3;
        b[(k + q) % n] ^= r4;
        b[k % n] = r4;
    }
#undef ORA_T
    /* all-zero guard of the engine's seed(seq) */
    int zero = (b[0] & 0x80000000u) == 0;
    for (int i = 1; i < n && zero; i++) zero = (b[i] == 0);
    if (zero) b[0] = 0x80000000u;
    g->i = n;
}

static void ora_mt_twist(ora_mt19937* g) {
    const int n = 624, m = 397;
    for (int i = 0; i < n; i++) {
        uint32_t y = (g->x[i] & 0x80000000u) | (g->x[(i + 1) % n] & 0x7fffffffu);
        g->x[i] = g->x[(i + m) % n] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->i = 0;
}

uint32_t ora_mt_next(ora_mt19937* g) {
    if (g->i >= 624) ora_mt_twist(g);
    uint32_t y = g->x[g->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* generate_canonical<double, 53> for a 32-bit engine: two draws,
 * sum = g1 + g2 * 2^32 rounded to double, divided by 2^64, clamped below 1. */
double ora_canonical(ora_mt19937* g) {
    double sum = 0.0, tmp = 1.0;
    for (int k = 0; k < 2; k++) {
        sum += (double)ora_mt_next(g) * tmp;
        tmp *= 4294967296.0;
    }
    double r = sum / tmp;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

/* uniform_int_distribution<int>(lo, hi) of libstdc++ (GCC >= 11) for a 32-bit engine:
 * Lemire's nearly divisionless method (ACM TOMACS 29(1), 2019). */
uint32_t ora_uniform_int(ora_mt19937* g, uint32_t lo, uint32_t hi) {
    uint32_t range = hi - lo + 1u;
    if (range == 0u) return lo + ora_mt_next(g); /* full 32-bit range */
    uint64_t product = (uint64_t)ora_mt_next(g) * (uint64_t)range;
    uint32_t low = (uint32_t)product;
    if (low < range) {
        uint32_t threshold = (uint32_t)(-range) % range;
        while (low < threshold) {
            product = (uint64_t)ora_mt_next(g) * (uint64_t)range;
            low = (uint32_t)product;
        }
    }
    return lo + (uint32_t)(product >> 32);
}

/* normal_distribution<double>: Marsaglia polar method, second value cached in *saved. */
static double ora_normal(ora_mt19937* g, int* has_saved, double* saved) {
    if (*has_saved) {
        *has_saved = 0;
        return *saved;
    }
    double x, y, r2;
    do {
        x = 2.0 * ora_canonical(g) - 1.0;
        y = 2.0 * ora_canonical(g) - 1.0;
        r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double mult = sqrt(-2 * log(r2) / r2);
    *saved = x * mult;
    *has_saved = 1;
    return y * mult;
}

/* poisson_distribution<int>: for mean >= 12 the rejection method of Devroye,
 * "Non-Uniform Random Variate Generation" (1986), p. 511, in the form libstdc++
 * (GCC 13) uses; below 12 the multiplicative method with threshold exp(-mean). */
int ora_poisson(ora_mt19937* g, double mean) {
    if (mean >= 12) {
        const double pi_4 = (double)0.7853981633974483096156608458198757L;
        const double m = floor(mean);
        const double lm_thr = log(mean);
        const double lfm = lgamma(m + 1);
        const double sm = sqrt(m);
        const double dx = sqrt(2 * m * log(32 * m / pi_4));
        const double d = round(fmax(6.0, fmin(m, dx)));
        const double cx = 2 * m + d;
        const double scx = sqrt(cx / 2);
        const double one_cx = 1 / cx;
        const double c2b = sqrt(pi_4 * cx) * exp(one_cx);
        const double cb = 2 * cx * exp(-d * one_cx * (1 + d / 2)) / d;

        const double naf = (1 - DBL_EPSILON) / 2;
        const double thr = (double)INT_MAX + naf;
        const double spi_2 = (double)1.2533141373155002512078826424055226L;
        const double c1 = sm * spi_2;
        const double c2 = c2b + c1;
        const double c3 = c2 + 1;
        const double c4 = c3 + 1;
        const double r178 = (double)0.0128205128205128205128205128205128L;
        const double e178 = (double)1.0129030479320018583185514777512983L;
        const double c5 = c4 + e178;
        const double c = cb + c5;
        const double two_cx = 2 * (2 * m + d);

        int has_saved = 0;
        double saved = 0.0;
        double x = 0.0;
        int reject = 1;
        do {
            const double u = c * ora_canonical(g);
            const double e = -log(1.0 - ora_canonical(g));
            double w = 0.0;
            if (u <= c1) {
                const double nrm = ora_normal(g, &has_saved, &saved);
                const double y = -fabs(nrm) * sm - 1;
                x = floor(y);
                w = -nrm * nrm / 2;
                if (x < -m) continue;
            } else if (u <= c2) {
                const double nrm = ora_normal(g, &has_saved, &saved);
                const double y = 1 + fabs(nrm) * scx;
                x = ceil(y);
                w = y * (2 - y) * one_cx;
                if (x > d) continue;
            } else if (u <= c3) {
                x = -1;
            } else if (u <= c4) {
                x = 0;
            } else if (u <= c5) {
                x = 1;
                w = r178;
            } else {
                const double v = -log(1.0 - ora_canonical(g));
                const double y = d + v * two_cx / d;
                x = ceil(y);
                w = -d * one_cx * (1 + y / 2);
            }
            reject = (w - e - x * lm_thr > lfm - lgamma(x + m + 1));
            reject |= (x + m >= thr);
        } while (reject);
        return (int)(x + m + naf);
    } else {
        const double lm_thr = exp(-mean);
        int x = 0;
        double prod = 1.0;
        do {
            prod *= ora_canonical(g);
            x += 1;
        } while (prod > lm_thr);
        return x - 1;
    }
}

/* ===================================================================== */
/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)                     */
/* ===================================================================== */
void ora_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ===================================================================== */
/* Geometry helpers                                                      */
/* ===================================================================== */

/* puissance<N>(x) = puissance<N/2>(x) * puissance<N - N/2>(x)  (auxiliary/AuxiFunctions.ixx:35-44) */
static double ora_pow_int(double x, int e) {
    if (e == 0) return 1;
    if (e == 1) return x;
    int e1 = e / 2;
    return ora_pow_int(x, e1) * ora_pow_int(x, e - e1);
}

/* volumeUnitSphere (auxiliary/Geometry/Sphere.ixx:30-44) */
static double ora_volume_unit_sphere(int D) {
    const double pi = (double)3.1415926535897932384626433832795029L;
    double mult = 1;
    if (D % 2 == 0) {
        for (int k = 0; k <= D / 2 - 1; k++) mult *= (2 * pi) / (D - 2 * k);
    } else {
        mult = 1. / pi;
        for (int k = 0; k <= (D - 1) / 2; k++) mult *= (2 * pi) / (D - 2 * k);
    }
    return mult;
}

double ora_volume_sphere(int dim, double r) { return ora_volume_unit_sphere(dim) * ora_pow_int(r, dim); }

uint64_t ora_count_from_fraction(int dim, double r, double phi, double volume) {
    return (uint64_t)(volume * phi / ora_volume_sphere(dim, r));
}

/* is_there_collision (operator_cells_and_data_storage.ixx:5-14): sum_d (a-b)^2 < (r1+r2)^2 */
static int ora_collide(int D, double r1, const double* a, double r2, const double* b) {
    double dist2 = 0;
    for (int d = 0; d < D; d++) {
        const double dr = a[d] - b[d];
        dist2 += dr * dr;
    }
    const double rr = r1 + r2;
    return dist2 < rr * rr;
}

/* TabCorner order (auxiliary/Path.ixx:86-103) for D = 2, 3; for D >= 4 the reference's generic
 * branch (Path.ixx:105-114) writes out of bounds and never sets dimension 0, so the oracle uses
 * the complete table with bit d of the corner index as the offset along dimension d. */
static int ora_corner(int D, int i, int d) {
    static const int t2[4][2] = { {0, 0}, {1, 1}, {0, 1}, {1, 0} };
    static const int t3[8][3] = { {0, 0, 0}, {1, 1, 1}, {0, 0, 1}, {1, 1, 0},
                                  {0, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 0, 0} };
    if (D == 2) return t2[i][d];
    if (D == 3) return t3[i][d];
    return (i >> d) & 1;
}

/* ===================================================================== */
/* Sphere storage with a periodic cell list                              */
/* ===================================================================== */

typedef struct {
    int D;
    double inf[ORA_MAX_DIM], L[ORA_MAX_DIM];
    int n[ORA_MAX_DIM];
    double c[ORA_MAX_DIM];
    int64_t ncells;
    int64_t* head; /* per cell, -1 = empty */
    /* spheres */
    uint64_t count, cap;
    double* pos;
    double* rad;
    int* phase;
    uint64_t* key;
    int64_t* next;
} ora_store;

static void store_init(ora_store* s, int D, const double* inf, const double* L, double search) {
    memset(s, 0, sizeof(*s));
    s->D = D;
    s->ncells = 1;
    for (int d = 0; d < D; d++) {
        s->inf[d] = inf[d];
        s->L[d] = L[d];
        int n = (int)(L[d] / search);
        if (n < 1) n = 1;
        if (n > 4096) n = 4096;
        s->n[d] = n;
        s->c[d] = L[d] / n;
        s->ncells *= n;
    }
    s->head = (int64_t*)malloc(sizeof(int64_t) * s->ncells);
    for (int64_t i = 0; i < s->ncells; i++) s->head[i] = -1;
}

/* an empty store with the same cells as *like */
static void store_init_like(ora_store* s, const ora_store* like) {
    memset(s, 0, sizeof(*s));
    s->D = like->D;
    s->ncells = like->ncells;
    for (int d = 0; d < like->D; d++) {
        s->inf[d] = like->inf[d];
        s->L[d] = like->L[d];
        s->n[d] = like->n[d];
        s->c[d] = like->c[d];
    }
    s->head = (int64_t*)malloc(sizeof(int64_t) * s->ncells);
    for (int64_t i = 0; i < s->ncells; i++) s->head[i] = -1;
}

static void store_free(ora_store* s) {
    free(s->head); free(s->pos); free(s->rad); free(s->phase); free(s->key); free(s->next);
    memset(s, 0, sizeof(*s));
}

static void store_cell_coords(const ora_store* s, const double* x, int* cc) {
    for (int d = 0; d < s->D; d++) {
        int k = (int)floor((x[d] - s->inf[d]) / s->c[d]);
        if (k < 0) k = 0;
        if (k >= s->n[d]) k = s->n[d] - 1;
        cc[d] = k;
    }
}

static int64_t store_cell_index(const ora_store* s, const int* cc) {
    int64_t idx = 0;
    for (int d = s->D - 1; d >= 0; d--) idx = idx * s->n[d] + cc[d];
    return idx;
}

static void store_add(ora_store* s, const double* x, double r, int ph, uint64_t key) {
    if (s->count == s->cap) {
        uint64_t nc = s->cap ? s->cap * 2 : 1024;
        s->pos = (double*)realloc(s->pos, sizeof(double) * nc * s->D);
        s->rad = (double*)realloc(s->rad, sizeof(double) * nc);
        s->phase = (int*)realloc(s->phase, sizeof(int) * nc);
        s->key = (uint64_t*)realloc(s->key, sizeof(uint64_t) * nc);
        s->next = (int64_t*)realloc(s->next, sizeof(int64_t) * nc);
        s->cap = nc;
    }
    uint64_t i = s->count++;
    memcpy(s->pos + i * s->D, x, sizeof(double) * s->D);
    s->rad[i] = r;
    s->phase[i] = ph;
    s->key[i] = key;
    int cc[ORA_MAX_DIM];
    store_cell_coords(s, x, cc);
    int64_t cell = store_cell_index(s, cc);
    s->next[i] = s->head[cell];
    s->head[cell] = (int64_t)i;
}

/* Visits every sphere of the 3^D cells around the cell of x, with its periodic image: the
 * image coordinate is x_s + (+/-L) for a wrapped dimension, as the ghost copies of the
 * reference (rsa_ghost_area.ixx:22-30, rsa_domain.ixx:160-186).  The callback returns
 * nonzero to stop. */
typedef int (*ora_visit_fn)(void* ctx, uint64_t id, const double* image);

static int store_visit(const ora_store* s, const double* x, ora_visit_fn fn, void* ctx) {
    const int D = s->D;
    int cc[ORA_MAX_DIM];
    store_cell_coords(s, x, cc);
    int total = 1;
    for (int d = 0; d < D; d++) total *= 3;
    for (int t = 0; t < total; t++) {
        int nc[ORA_MAX_DIM];
        double shift[ORA_MAX_DIM];
        int tt = t;
        for (int d = 0; d < D; d++) {
            int o = tt % 3 - 1;
            tt /= 3;
            int k = cc[d] + o;
            shift[d] = 0.0;
            if (k < 0) { k += s->n[d]; shift[d] = -s->L[d]; }
            else if (k >= s->n[d]) { k -= s->n[d]; shift[d] = s->L[d]; }
            nc[d] = k;
        }
        int64_t cell = store_cell_index(s, nc);
        for (int64_t i = s->head[cell]; i >= 0; i = s->next[i]) {
            double img[ORA_MAX_DIM];
            const double* p = s->pos + (uint64_t)i * D;
            for (int d = 0; d < D; d++) img[d] = (shift[d] != 0.0) ? p[d] + shift[d] : p[d];
            if (fn(ctx, (uint64_t)i, img)) return 1;
        }
    }
    return 0;
}

/* ===================================================================== */
/* Oracle state                                                          */
/* ===================================================================== */

struct rsa_oracle {
    int D;
    double inf[ORA_MAX_DIM], sup[ORA_MAX_DIM], L[ORA_MAX_DIM];
    double domain_rad;
    int nbshots;
    /* radius classes, sorted by nonincreasing radius */
    int k;
    double* cls_r;
    uint64_t* cls_n;
    int* cls_phase;
    int cls_idx;
    double r_max, r_min;
    /* validated spheres */
    ora_store st;
    /* voxel list */
    int64_t* vox;
    uint64_t nvox, capvox;
    double vlen[ORA_MAX_DIM];
    int vlevel;
    /* rng */
    ora_mt19937 g;
    /* current round candidates */
    uint64_t ncand, capcand;
    double* cpos;
    uint64_t* ckey;
    double* crad;
    int* cphase;
    /* trace */
    uint64_t ntrace, captrace;
    uint64_t* tr_vox;
    uint64_t* tr_shots;
    uint64_t* tr_new;
    uint8_t* tr_ref;
    uint64_t last_round_vox;
    int cap_exact;
    /* continuous radius law: radius = r_min + (r_max - r_min) x, x ~ U[0, 1) */
    int uniform_radius;
    double* rtab; /* a tabulated transform (knots at x = j / (ntab - 1)), or NULL: r_min + (r_max - r_min) x */
    int ntab;
    int uniform_phase;
};

rsa_oracle* ora_create(int dim, const double* inf, const double* sup, double domain_rad,
    int n_classes, const double* radii, const uint64_t* counts, const int* phases,
    double exclusion_distance, int nbshots) {
    if (dim < 1 || dim > ORA_MAX_DIM || n_classes < 1) return NULL;
    rsa_oracle* o = (rsa_oracle*)calloc(1, sizeof(rsa_oracle));
    o->D = dim;
    for (int d = 0; d < dim; d++) {
        o->inf[d] = inf[d];
        o->sup[d] = sup[d];
        o->L[d] = sup[d] - inf[d];
    }
    o->domain_rad = domain_rad;
    o->nbshots = nbshots;
    o->k = n_classes;
    o->cls_r = (double*)malloc(sizeof(double) * n_classes);
    o->cls_n = (uint64_t*)malloc(sizeof(uint64_t) * n_classes);
    o->cls_phase = (int*)malloc(sizeof(int) * n_classes);
    /* std::sort by descending radius (radius_generator.ixx:17-20); a stable insertion sort gives the
     * same order as long as radii are distinct. */
    for (int i = 0; i < n_classes; i++) {
        o->cls_r[i] = radii[i];
        o->cls_n[i] = counts[i];
        o->cls_phase[i] = phases[i];
    }
    for (int i = 1; i < n_classes; i++) {
        for (int j = i; j > 0 && o->cls_r[j] > o->cls_r[j - 1]; j--) {
            double tr = o->cls_r[j]; o->cls_r[j] = o->cls_r[j - 1]; o->cls_r[j - 1] = tr;
            uint64_t tn = o->cls_n[j]; o->cls_n[j] = o->cls_n[j - 1]; o->cls_n[j - 1] = tn;
            int tp = o->cls_phase[j]; o->cls_phase[j] = o->cls_phase[j - 1]; o->cls_phase[j - 1] = tp;
        }
    }
    /* exclusion distance added to entry 0, once per class (radius_generator.ixx:23-25) */
    for (int i = 0; i < n_classes; i++) o->cls_r[0] += 0.5 * exclusion_distance;
    o->r_max = o->cls_r[0];
    o->r_min = o->cls_r[n_classes - 1];
    o->cls_idx = 0;
    double search = 2 * (o->r_max > domain_rad ? o->r_max : domain_rad);
    store_init(&o->st, dim, o->inf, o->L, search);
    return o;
}

/* RadiusGenerator(min_radius, max_radius, &RandomRadiusGenerator(transform, phase), nb_spheres, 0)
 * (radius_generator.ixx:39-48, radius_generator.hxx:12-38) with transform x -> r_min + (r_max - r_min) x:
 * one entry (radius 0, nb_spheres, phase 0) in the class list, explicit r_min and r_max, every dart's
 * radius drawn after the priorities (generate_candidates, operator_algorithm.ixx:568-582). */
/* A transform given by its values at x = j / (ntab - 1), interpolated linearly at x and kept within
 * [r_min, r_max] (the knots' range): the tabulated form of an arbitrary RandomRadiusGenerator transform
 * (radius_generator.hxx:12-38), with the same arithmetic as the GPU darts. */
static double ora_table_radius(const rsa_oracle* o, double x) {
    const double t = x * (double)(o->ntab - 1);
    int j = (int)t;
    if (j > o->ntab - 2) j = o->ntab - 2;
    const double f = t - (double)j;
    const double a = o->rtab[j], b = o->rtab[j + 1];
    const double v = a + f * (b - a);
    const double hi = o->r_min + (o->r_max - o->r_min);
    return v < o->r_min ? o->r_min : (v > hi ? hi : v);
}

int ora_set_radius_table(rsa_oracle* o, const double* knots, int n) {
    if (!o->uniform_radius || n < 2) return -1;
    free(o->rtab);
    o->rtab = (double*)malloc(sizeof(double) * n);
    memcpy(o->rtab, knots, sizeof(double) * n);
    o->ntab = n;
    return 0;
}

rsa_oracle* ora_create_uniform(int dim, const double* inf, const double* sup, double r_min, double r_max,
    uint64_t count, int phase, int nbshots) {
    const double r0 = 0.;
    const int ph0 = 0;
    rsa_oracle* o = ora_create(dim, inf, sup, r_max, 1, &r0, &count, &ph0, 0., nbshots);
    if (!o) return NULL;
    o->r_min = r_min;
    o->r_max = r_max;
    o->uniform_radius = 1;
    o->uniform_phase = phase;
    store_free(&o->st);
    store_init(&o->st, dim, o->inf, o->L, 2 * r_max);
    return o;
}

/* rsa_algo::reset_radius_generator (operator_algorithm.ixx:238-250): a new class list on the same domain and
 * spheres; the algorithm's r_max stays the larger of the two (m_r_max), which the next voxel lattice uses. */
int ora_reset_classes(rsa_oracle* o, int n_classes, const double* radii, const uint64_t* counts,
    const int* phases, double exclusion_distance) {
    if (!o || n_classes < 1) return -1;
    double* r = (double*)malloc(sizeof(double) * n_classes);
    uint64_t* n = (uint64_t*)malloc(sizeof(uint64_t) * n_classes);
    int* ph = (int*)malloc(sizeof(int) * n_classes);
    for (int i = 0; i < n_classes; i++) {
        r[i] = radii[i];
        n[i] = counts[i];
        ph[i] = phases[i];
    }
    for (int i = 1; i < n_classes; i++) {
        for (int j = i; j > 0 && r[j] > r[j - 1]; j--) {
            double tr = r[j]; r[j] = r[j - 1]; r[j - 1] = tr;
            uint64_t tn = n[j]; n[j] = n[j - 1]; n[j - 1] = tn;
            int tp = ph[j]; ph[j] = ph[j - 1]; ph[j - 1] = tp;
        }
    }
    for (int i = 0; i < n_classes; i++) r[0] += 0.5 * exclusion_distance;
    if (r[0] > o->r_max) {
        free(r); free(n); free(ph);
        return -2; /* runtime_error("Incorrect maximal radius") */
    }
    free(o->cls_r); free(o->cls_n); free(o->cls_phase);
    o->cls_r = r;
    o->cls_n = n;
    o->cls_phase = ph;
    o->k = n_classes;
    o->cls_idx = 0;
    o->r_min = r[n_classes - 1];
    o->uniform_radius = 0;
    return 0;
}

void ora_destroy(rsa_oracle* o) {
    if (!o) return;
    store_free(&o->st);
    free(o->cls_r); free(o->cls_n); free(o->cls_phase);
    free(o->vox);
    free(o->cpos); free(o->ckey); free(o->crad); free(o->cphase);
    free(o->tr_vox); free(o->tr_shots); free(o->tr_new); free(o->tr_ref);
    free(o->rtab);
    free(o);
}

double ora_min_radius(const rsa_oracle* o) { return o->r_min; }
double ora_max_radius(const rsa_oracle* o) { return o->r_max; }

/* ---- voxel list (list_of_voxels.ixx) ---- */

static void vox_reserve(rsa_oracle* o, uint64_t n) {
    if (n <= o->capvox) return;
    uint64_t nc = o->capvox ? o->capvox : 1024;
    while (nc < n) nc *= 2;
    o->vox = (int64_t*)realloc(o->vox, sizeof(int64_t) * nc * o->D);
    o->capvox = nc;
}

/* ctor + compute_nb_vox / compute_voxel_length (list_of_voxels.ixx:11-28, 192-211);
 * getAllIndices enumerates with dimension 0 fastest (auxiliary/Loops.ixx:45-54). */
static void vox_build(rsa_oracle* o, double max_diagonal) {
    const int D = o->D;
    int64_t nb[ORA_MAX_DIM];
    uint64_t total = 1;
    for (int d = 0; d < D; d++) {
        nb[d] = 1 + (int)(sqrt((double)D) * o->L[d] / max_diagonal);
        o->vlen[d] = o->L[d] / (double)nb[d];
        total *= (uint64_t)nb[d];
    }
    vox_reserve(o, total);
    int64_t idx[ORA_MAX_DIM] = { 0 };
    for (uint64_t v = 0; v < total; v++) {
        for (int d = 0; d < D; d++) o->vox[v * D + d] = idx[d];
        for (int d = 0; d < D; d++) {
            if (++idx[d] < nb[d]) break;
            idx[d] = 0;
        }
    }
    o->nvox = total;
    o->vlevel = 0;
}

/* is_in_sphere (list_of_voxels.ixx:225-238): every corner within (r_s + r_min) */
static int vox_corners_in(int D, const double* len, const double* delta, double rs, double rmin) {
    /* Corner i's squared distance is the rounded sum, in dimension order, of (c_d - delta_d)^2 with c_d = 0
     * or len_d.  Round-to-nearest addition is monotone, so the largest of the 2^D corner sums is the rounded
     * sum of the per-dimension larger squares: one sum decides every corner, bit for bit. */
    const double R = rs + rmin;
    const double R2 = R * R;
    double dist2 = 0.;
    for (int d = 0; d < D; d++) {
        const double t0 = 0.0 - delta[d];
        const double t1 = len[d] - delta[d];
        const double s0 = t0 * t0, s1 = t1 * t1;
        dist2 += s0 > s1 ? s0 : s1;
    }
    return !(dist2 > R2);
}

static void vox_origin(const rsa_oracle* o, const int64_t* coord, const double* len, double* orig) {
    for (int d = 0; d < o->D; d++) orig[d] = o->inf[d] + (double)coord[d] * len[d];
}

/* The validated spheres by cell with one layer of ghost cells, as the reference's rsa_grid holds them
 * (rsa_grid.ixx, ghost copies rsa_ghost_area.ixx:22-30): each cell of the padded grid lists, contiguously,
 * the spheres of the real cell it maps to with the periodic shift of that ghost position applied.  Built
 * once per refinement, during which the spheres do not change; the voxel passes then read the 3^D cells
 * around a point at fixed index offsets.  The (sphere, image) pairs are those store_visit yields. */
typedef struct {
    int D;
    int np[ORA_MAX_DIM];      /* padded cells per dimension (n + 2) */
    int64_t* start;           /* padded cells + 1 */
    uint64_t* ids;
    double* img;              /* D doubles per entry: the image coordinates */
    int64_t off[2187];        /* the 3^D neighbour offsets in the padded grid (3^7 at most) */
    int noff;
} ora_csr;

static void csr_build(ora_csr* c, const ora_store* s) {
    const int D = s->D;
    c->D = D;
    int64_t npc = 1;
    for (int d = 0; d < D; d++) {
        c->np[d] = s->n[d] + 2;
        npc *= c->np[d];
    }
    c->start = (int64_t*)calloc((size_t)npc + 1, sizeof(int64_t));
    /* counts: the real cell of each padded cell */
    int pc[ORA_MAX_DIM] = { 0 };
    for (int64_t p = 0; p < npc; p++) {
        int rc[ORA_MAX_DIM];
        for (int d = 0; d < D; d++) {
            int k = pc[d] - 1;
            if (k < 0) k += s->n[d];
            else if (k >= s->n[d]) k -= s->n[d];
            rc[d] = k;
        }
        int64_t cnt = 0;
        for (int64_t i = s->head[store_cell_index(s, rc)]; i >= 0; i = s->next[i]) cnt++;
        c->start[p + 1] = c->start[p] + cnt;
        for (int d = 0; d < D && ++pc[d] == c->np[d]; d++) pc[d] = 0;
    }
    const int64_t total = c->start[npc];
    c->ids = (uint64_t*)malloc(sizeof(uint64_t) * (total ? total : 1));
    c->img = (double*)malloc(sizeof(double) * (total ? total : 1) * D);
    for (int d = 0; d < D; d++) pc[d] = 0;
    for (int64_t p = 0; p < npc; p++) {
        int rc[ORA_MAX_DIM];
        double sh[ORA_MAX_DIM];
        for (int d = 0; d < D; d++) {
            int k = pc[d] - 1;
            sh[d] = 0.0;
            if (k < 0) { k += s->n[d]; sh[d] = -s->L[d]; }
            else if (k >= s->n[d]) { k -= s->n[d]; sh[d] = s->L[d]; }
            rc[d] = k;
        }
        int64_t k = c->start[p];
        for (int64_t i = s->head[store_cell_index(s, rc)]; i >= 0; i = s->next[i], k++) {
            c->ids[k] = (uint64_t)i;
            for (int d = 0; d < D; d++) {
                const double x = s->pos[(size_t)i * D + d];
                c->img[(size_t)k * D + d] = sh[d] != 0.0 ? x + sh[d] : x;
            }
        }
        for (int d = 0; d < D && ++pc[d] == c->np[d]; d++) pc[d] = 0;
    }
    /* neighbour offsets */
    int od[ORA_MAX_DIM] = { 0 };
    c->noff = 0;
    for (;;) {
        int64_t o = 0;
        for (int d = D - 1; d >= 0; d--) o = o * c->np[d] + (od[d] - 1);
        c->off[c->noff++] = o;
        int d = 0;
        while (d < D && ++od[d] == 3) od[d++] = 0;
        if (d == D) break;
    }
}

static void csr_free(ora_csr* c) {
    free(c->start);
    free(c->ids);
    free(c->img);
}

/* the padded cell of the point x (its real cell plus one in every dimension) */
static int64_t csr_cell(const ora_csr* c, const ora_store* s, const double* x) {
    int cc[ORA_MAX_DIM];
    store_cell_coords(s, x, cc);
    int64_t idx = 0;
    for (int d = c->D - 1; d >= 0; d--) idx = idx * c->np[d] + (cc[d] + 1);
    return idx;
}

/* remove_covered (list_of_voxels.ixx:30-54), including the swap-remove order. */
static void vox_remove_covered(rsa_oracle* o) {
    const int D = o->D;
    uint64_t n = o->nvox;
    uint8_t* cov = (uint8_t*)malloc(n ? n : 1);
    ora_csr csr;
    csr_build(&csr, &o->st);
    for (uint64_t v = 0; v < n; v++) {
        double orig[ORA_MAX_DIM], centre[ORA_MAX_DIM];
        vox_origin(o, o->vox + v * D, o->vlen, orig);
        for (int d = 0; d < D; d++) centre[d] = orig[d] + 0.5 * o->vlen[d];
        /* is_covered (list_of_voxels.ixx:240-257): the spheres of the 3^D cells around the centre's */
        const int64_t base = csr_cell(&csr, &o->st, centre);
        int found = 0;
        for (int t = 0; t < csr.noff && !found; t++) {
            const int64_t cell = base + csr.off[t];
            for (int64_t k = csr.start[cell]; k < csr.start[cell + 1]; k++) {
                double delta[ORA_MAX_DIM];
                for (int d = 0; d < D; d++) delta[d] = csr.img[(size_t)k * D + d] - orig[d];
                if (vox_corners_in(D, o->vlen, delta, o->st.rad[csr.ids[k]], o->r_min)) {
                    found = 1;
                    break;
                }
            }
        }
        cov[v] = (uint8_t)found;
    }
    csr_free(&csr);
    uint64_t size = n;
    for (int64_t v = 0; v < (int64_t)size; v++) {
        if (cov[v]) {
            memcpy(o->vox + v * D, o->vox + (size - 1) * D, sizeof(int64_t) * D);
            cov[v] = cov[size - 1];
            v--;
            size--;
        }
    }
    o->nvox = size;
    free(cov);
}

typedef struct {
    const rsa_oracle* o;
    const double* centre;
    uint64_t* ids;
    double* imgs;
    int n, cap;
} pre_ctx;

static int pre_visit(void* vctx, uint64_t id, const double* img) {
    pre_ctx* c = (pre_ctx*)vctx;
    const int D = c->o->D;
    /* get_list_of_spheres (list_of_voxels.ixx:283-307): dist2(centre) < (r_s + r_min)^2 */
    double dist2 = 0.;
    for (int d = 0; d < D; d++) {
        const double t = img[d] - c->centre[d];
        dist2 += t * t;
    }
    const double R = c->o->st.rad[id] + c->o->r_min;
    if (dist2 < R * R) {
        if (c->n == c->cap) {
            c->cap = c->cap ? 2 * c->cap : 64;
            c->ids = (uint64_t*)realloc(c->ids, sizeof(uint64_t) * c->cap);
            c->imgs = (double*)realloc(c->imgs, sizeof(double) * c->cap * D);
        }
        c->ids[c->n] = id;
        memcpy(c->imgs + (size_t)c->n * D, img, sizeof(double) * D);
        c->n++;
    }
    return 0;
}

/* subdivide_uncovered (list_of_voxels.ixx:56-100): children in TabCorner order. */
static void vox_subdivide(rsa_oracle* o) {
    const int D = o->D;
    if (o->nvox == 0) return;
    double nlen[ORA_MAX_DIM];
    for (int d = 0; d < D; d++) nlen[d] = 0.5 * o->vlen[d];
    const int nc = 1 << D;
    uint64_t cap = o->nvox * nc;
    int64_t* out = (int64_t*)malloc(sizeof(int64_t) * (cap ? cap : 1) * D);
    if (!out) abort(); /* the oracle is for cases that fit in host memory */
    uint64_t k = 0;
    pre_ctx pc = { o, NULL, NULL, NULL, 0, 0 };
    ora_csr csr;
    csr_build(&csr, &o->st);
    for (uint64_t v = 0; v < o->nvox; v++) {
        const int64_t* pcoord = o->vox + v * D;
        double centre[ORA_MAX_DIM];
        /* center(i) = origin + (coord + 0.5) * len (list_of_voxels.ixx:154-160) */
        for (int d = 0; d < D; d++) centre[d] = o->inf[d] + ((double)pcoord[d] + 0.5) * o->vlen[d];
        pc.centre = centre;
        pc.n = 0;
        {
            const int64_t base = csr_cell(&csr, &o->st, centre);
            for (int t = 0; t < csr.noff; t++) {
                const int64_t cell = base + csr.off[t];
                for (int64_t k = csr.start[cell]; k < csr.start[cell + 1]; k++)
                    pre_visit(&pc, csr.ids[k], csr.img + (size_t)k * D);
            }
        }
        for (int i = 0; i < nc; i++) {
            int64_t cc[ORA_MAX_DIM];
            double orig[ORA_MAX_DIM];
            for (int d = 0; d < D; d++) {
                cc[d] = 2 * pcoord[d] + ora_corner(D, i, d);
                orig[d] = o->inf[d] + (double)cc[d] * nlen[d];
            }
            int covered = 0;
            for (int s = 0; s < pc.n && !covered; s++) {
                double delta[ORA_MAX_DIM];
                for (int d = 0; d < D; d++) delta[d] = pc.imgs[(size_t)s * D + d] - orig[d];
                covered = vox_corners_in(D, nlen, delta, o->st.rad[pc.ids[s]], o->r_min);
            }
            if (!covered) {
                memcpy(out + k * D, cc, sizeof(int64_t) * D);
                k++;
            }
        }
    }
    csr_free(&csr);
    free(pc.ids);
    free(pc.imgs);
    free(o->vox);
    o->vox = out;
    o->capvox = cap ? cap : 1;
    o->nvox = k;
    for (int d = 0; d < D; d++) o->vlen[d] = nlen[d];
    o->vlevel++;
}

int ora_refine(rsa_oracle* o) {
    vox_remove_covered(o);
    vox_subdivide(o);
    return 0;
}

uint64_t ora_voxel_count(const rsa_oracle* o) { return o->nvox; }
int ora_voxel_level(const rsa_oracle* o) { return o->vlevel; }
int ora_voxel_export(const rsa_oracle* o, int64_t* coords, double* len) {
    if (coords) memcpy(coords, o->vox, sizeof(int64_t) * o->nvox * o->D);
    if (len) memcpy(len, o->vlen, sizeof(double) * o->D);
    return 0;
}

/* ---- spheres ---- */
uint64_t ora_sphere_count(const rsa_oracle* o) { return o->st.count; }
int ora_sphere_export(const rsa_oracle* o, double* pos, double* rad, int* phase) {
    if (pos) memcpy(pos, o->st.pos, sizeof(double) * o->st.count * o->D);
    if (rad) memcpy(rad, o->st.rad, sizeof(double) * o->st.count);
    if (phase) memcpy(phase, o->st.phase, sizeof(int) * o->st.count);
    return 0;
}
int ora_sphere_import(rsa_oracle* o, uint64_t n, const double* pos, const double* rad, const int* phase) {
    for (uint64_t i = 0; i < n; i++) store_add(&o->st, pos + i * o->D, rad[i], phase ? phase[i] : 0, 0);
    return 0;
}

/* ---- one round of decisions ---- */

typedef struct {
    int D;
    const double* x;
    double r;
    const double* rads;
    const uint64_t* keys;
    uint64_t key;
    int use_key;
    int hit;
} hit_ctx;

static int hit_visit(void* vctx, uint64_t id, const double* img) {
    hit_ctx* c = (hit_ctx*)vctx;
    if (c->use_key && !(c->keys[id] < c->key)) return 0;
    if (ora_collide(c->D, c->r, c->x, c->rads[id], img)) {
        c->hit = 1;
        return 1;
    }
    return 0;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* number of e in sorted[] with !(pivot < e) under std::less<uint64_t>, the pivot converted to
 * uint64_t first (median_of_medians.ixx:168-178: upper_bound with the caller's order). */
static int64_t pivot_count(const uint64_t* sorted, int64_t n, double pivot) {
    uint64_t pv = (uint64_t)pivot;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (pv < sorted[mid]) hi = mid; else lo = mid + 1;
    }
    return lo;
}

/* median_of_medians::find_pivot_for_first_elements with one rank (median_of_medians.ixx:8-123,
 * find_pivot :128-157).  Returns 0 and the pivot, or -1 where the reference throws. */
int ora_ref_pivot(const uint64_t* values, int64_t n, int64_t n_first, double* pivot_out) {
    if (n_first > n || n_first <= 0 || n == 0) return -1;
    double pct = n_first / (1. * n);
    uint64_t* v = (uint64_t*)malloc(sizeof(uint64_t) * n);
    memcpy(v, values, sizeof(uint64_t) * n);
    qsort(v, n, sizeof(uint64_t), cmp_u64);
    int64_t piv = (int64_t)(n * pct) - 1;
    int64_t mn = piv, mx = piv + 1;
    if (fabs(n * pct - 1 - piv) < 1e-8) mn -= 1;
    if (mn < 0) mn = 0;
    if (fabs(n * pct - 1 - piv - 1) < 1e-8) mx += 1;
    if (mx > n - 1) mx = n - 1;
    double cand[2] = { (double)v[mn] - DBL_EPSILON, (double)v[mx] + DBL_EPSILON };
    /* std::sort of the candidates with std::less<uint64_t> */
    if ((uint64_t)cand[1] < (uint64_t)cand[0]) { double t = cand[0]; cand[0] = cand[1]; cand[1] = t; }
    /* upper_bound(cands, n_first, [](n, c){ return n <= count(c); }) */
    int p = 2;
    for (int i = 0; i < 2; i++) {
        if (n_first <= pivot_count(v, n, cand[i])) { p = i; break; }
    }
    if (p == 2) { free(v); return -1; }
    double pmax = cand[p];
    double pivot = pmax;
    int64_t below = pivot_count(v, n, pivot);
    if (below != n_first) {
        if (p == 0) { free(v); return -1; }
        double pmin = cand[p - 1];
        double step = pmax - pmin;
        double add = 0.5 * step;
        for (int j = 0; j < 20; j++) {
            pivot = pmin + add;
            below = pivot_count(v, n, pivot);
            if (below == n_first) break;
            if (below > n_first) add = 0.5 * fabs(add);
            if (below < n_first) add = -0.5 * fabs(add);
        }
    }
    free(v);
    *pivot_out = pivot;
    return 0;
}

static const uint64_t* g_sort_keys;
static int cmp_key_idx(const void* a, const void* b) {
    uint64_t ia = *(const uint64_t*)a, ib = *(const uint64_t*)b;
    uint64_t ka = g_sort_keys[ia], kb = g_sort_keys[ib];
    if (ka != kb) return ka < kb ? -1 : 1;
    return ia < ib ? -1 : (ia > ib ? 1 : 0);
}

typedef struct {
    int D;
    const double* x;
    double r;
    const double* pos;
    const double* rads;
    const uint64_t* keys;
    uint64_t key;
    const uint64_t* ids; /* store slot -> candidate index */
    const int8_t* status;
    uint64_t self;
    int blocked_real_u, blocked_conflict;
} pass_ctx;

enum { ST_NONE = 0, ST_U = 1, ST_C = 2, ST_S = 3 };

static int pass_visit(void* vctx, uint64_t slot, const double* img) {
    pass_ctx* c = (pass_ctx*)vctx;
    const uint64_t other = c->ids[slot];
    if (!(c->keys[slot] < c->key || (c->keys[slot] == c->key && other < c->self))) return 0;
    if (!ora_collide(c->D, c->r, c->x, c->rads[slot], img)) return 0;
    int wrapped = 0;
    for (int d = 0; d < c->D; d++) wrapped |= (img[d] != c->pos[slot * c->D + d]);
    if (wrapped) { c->blocked_conflict = 1; return 0; } /* ghost copy: Undecided during the pass */
    int8_t st = c->status[c->ids[slot]];
    if (st == ST_C) c->blocked_conflict = 1;
    else if (st == ST_U) c->blocked_real_u = 1;
    return 0;
}

/* One find_solve_conflicts pass (operator_cells_and_data_storage.ixx:79-143) over the set und[]
 * (sorted by key): a candidate with no lower-priority non-Skip collider stays Undecided; one with a
 * collider that is a periodic image (ghost copy, always Undecided during the pass) or Conflict
 * becomes Conflict; otherwise Skip.  Where a candidate has both kinds of colliders the reference
 * takes the first one in its cell-scan order; this restatement lets Conflict win. */
static void pass_classify(const rsa_oracle* o, const uint64_t* und, uint64_t nu, const double* pos,
    const uint64_t* key, const double* rad, int8_t* status) {
    const int D = o->D;
    ora_store tmp;
    store_init_like(&tmp, &o->st);
    uint64_t* ids = (uint64_t*)malloc(sizeof(uint64_t) * (nu ? nu : 1));
    for (uint64_t t = 0; t < nu; t++) {
        store_add(&tmp, pos + und[t] * D, rad[und[t]], 0, key[und[t]]);
        ids[t] = und[t];
    }
    for (uint64_t t = 0; t < nu; t++) {
        uint64_t i = und[t];
        pass_ctx c = { D, pos + i * D, rad[i], tmp.pos, tmp.rad, tmp.key, key[i], ids, status, i, 0, 0 };
        store_visit(&tmp, pos + i * D, pass_visit, &c);
        status[i] = c.blocked_conflict ? ST_C : (c.blocked_real_u ? ST_S : ST_U);
    }
    free(ids);
    store_free(&tmp);
}

/* The add_to_sample loop of a round that may reach the class count (may_outreach,
 * operator_algorithm.ixx:383-443): each pass compares its Undecided count with the class count
 * given to the round (the count is passed by value, so every pass sees the original one); above
 * it, retain_only_first_elements keeps the priorities under the pivot and drops the rest; at or
 * below it, the Undecided are validated and the Conflict ones go to the next pass, unless the
 * count is reached exactly.  Returns -1 where the reference throws. */
static int apply_capped(rsa_oracle* o, uint64_t n, const double* pos, const uint64_t* key,
    const double* rad, const int* phase, uint64_t max_new, const uint8_t* alive0,
    uint8_t* accepted_out, uint64_t* n_new) {
    const int D = o->D;
    int8_t* status = (int8_t*)calloc(n ? n : 1, 1);
    uint64_t* und = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    uint64_t nu = 0;
    for (uint64_t i = 0; i < n; i++) if (alive0[i]) und[nu++] = i;
    g_sort_keys = key;
    qsort(und, nu, sizeof(uint64_t), cmp_key_idx);
    uint64_t total = 0;
    int rc = 0;
    for (int pass = 0; pass < 1000 && nu > 0; pass++) {
        for (uint64_t t = 0; t < nu; t++) status[und[t]] = ST_NONE;
        pass_classify(o, und, nu, pos, key, rad, status);
        uint64_t nU = 0;
        for (uint64_t t = 0; t < nu; t++) nU += (status[und[t]] == ST_U);
        if (nU > max_new) {
            uint64_t* pk = (uint64_t*)malloc(sizeof(uint64_t) * nU);
            uint64_t k = 0;
            for (uint64_t t = 0; t < nu; t++) if (status[und[t]] == ST_U) pk[k++] = key[und[t]];
            double pivot = 0;
            if (ora_ref_pivot(pk, (int64_t)nU, (int64_t)max_new, &pivot) != 0) rc = -1;
            free(pk);
            if (rc == 0) {
                for (uint64_t t = 0; t < nu; t++) {
                    uint64_t i = und[t];
                    if (status[i] == ST_U && !((double)key[i] > pivot)) {
                        accepted_out[i] = 1;
                        store_add(&o->st, pos + i * D, rad[i], phase[i], key[i]);
                        total++;
                    }
                }
            }
            break;
        }
        for (uint64_t t = 0; t < nu; t++) {
            uint64_t i = und[t];
            if (status[i] == ST_U) {
                accepted_out[i] = 1;
                store_add(&o->st, pos + i * D, rad[i], phase[i], key[i]);
            }
        }
        total += nU;
        if (max_new - nU == 0) break;
        /* next pass: the Conflict ones, minus those now hitting a validated sphere */
        uint64_t k = 0;
        for (uint64_t t = 0; t < nu; t++) {
            uint64_t i = und[t];
            if (status[i] != ST_C) continue;
            hit_ctx c = { D, pos + i * D, rad[i], o->st.rad, NULL, 0, 0, 0 };
            store_visit(&o->st, pos + i * D, hit_visit, &c);
            if (!c.hit) und[k++] = i;
        }
        nu = k;
    }
    *n_new = total;
    free(status);
    free(und);
    return rc;
}

/* Decisions of generate_spheres (operator_algorithm.ixx:534-566): a candidate is accepted iff
 * it overlaps no validated sphere (remove_collisions_with_validated_spheres,
 * operator_cells_and_data_storage.ixx:54-76) and no accepted candidate that precedes it in
 * (priority, candidate index) order (find_solve_conflicts + the add_to_sample loop, :79-143 and
 * operator_algorithm.ixx:383-443).  The reference's detection sees strictly smaller priorities
 * only (:39), so it accepts two overlapping candidates of equal priority; the index breaks
 * that tie instead.  When the round may exceed the class count
 * (may_outreach), only the max_new accepted candidates of smallest priority are kept
 * (retain_only_first_elements, operator_algorithm.ixx:475-519). */
int ora_apply_round(rsa_oracle* o, uint64_t n, const double* pos, const uint64_t* key,
    const double* rad, const int* phase, uint64_t max_new, int may_outreach,
    uint8_t* accepted_out, uint64_t* n_new) {
    const int D = o->D;
    uint8_t* alive = (uint8_t*)malloc(n ? n : 1);
    for (uint64_t i = 0; i < n; i++) {
        hit_ctx c = { D, pos + i * D, rad[i], o->st.rad, NULL, 0, 0, 0 };
        store_visit(&o->st, pos + i * D, hit_visit, &c);
        alive[i] = (uint8_t)!c.hit;
    }
    if (may_outreach && !o->cap_exact) {
        for (uint64_t i = 0; i < n; i++) accepted_out[i] = 0;
        int rc = apply_capped(o, n, pos, key, rad, phase, max_new, alive, accepted_out, n_new);
        free(alive);
        return rc;
    }
    uint64_t* order = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    for (uint64_t i = 0; i < n; i++) order[i] = i;
    g_sort_keys = key;
    qsort(order, n, sizeof(uint64_t), cmp_key_idx);
    /* accepted candidates in a scratch store, in priority order */
    ora_store acc; /* same cells as the main store */
    store_init_like(&acc, &o->st);
    uint64_t* acc_ids = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    uint64_t nacc = 0;
    for (uint64_t t = 0; t < n; t++) {
        uint64_t i = order[t];
        if (!alive[i]) continue;
        /* every candidate in acc precedes i in (key, index) order, so any overlap blocks i */
        hit_ctx c = { D, pos + i * D, rad[i], acc.rad, acc.key, key[i], 0, 0 };
        store_visit(&acc, pos + i * D, hit_visit, &c);
        if (!c.hit) {
            store_add(&acc, pos + i * D, rad[i], phase[i], key[i]);
            acc_ids[nacc++] = i;
        }
    }
    for (uint64_t i = 0; i < n; i++) accepted_out[i] = 0;
    int rc = 0;
    /* exact cap (ora_set_cap_exact): the max_new smallest priorities; acc_ids is in (key, index) order */
    if (may_outreach && nacc > max_new) nacc = max_new;
    for (uint64_t t = 0; t < nacc; t++) {
        uint64_t i = acc_ids[t];
        accepted_out[i] = 1;
    }
    /* insert in candidate order */
    for (uint64_t i = 0; i < n; i++)
        if (accepted_out[i]) store_add(&o->st, pos + i * D, rad[i], phase[i], key[i]);
    *n_new = nacc;
    store_free(&acc);
    free(acc_ids);
    free(order);
    free(alive);
    return rc;
}

/* ---- round loop (operator_algorithm.ixx:85-188) ---- */

static double ora_miss_threshold(int D) {
    /* magical_default_miss_rate (operator_algorithm.ixx:344-351) */
    if (D <= 3) return 0.95;
    return 1 - 0.05 * ora_pow_int(0.1, D - 3);
}

int ora_begin(rsa_oracle* o, uint64_t seed) {
    /* law::create_random_generator: seed_seq{rank = 0, seed} (rsa_random.hxx:37-42) */
    uint32_t sv[2] = { 0u, (uint32_t)seed };
    ora_mt_seed_seq(&o->g, sv, 2);
    vox_build(o, o->r_max + o->r_min);
    o->ntrace = 0;
    return 0;
}

static void cand_reserve(rsa_oracle* o, uint64_t n) {
    if (n <= o->capcand) return;
    uint64_t nc = o->capcand ? o->capcand : 1024;
    while (nc < n) nc *= 2;
    o->cpos = (double*)realloc(o->cpos, sizeof(double) * nc * o->D);
    o->ckey = (uint64_t*)realloc(o->ckey, sizeof(uint64_t) * nc);
    o->crad = (double*)realloc(o->crad, sizeof(double) * nc);
    o->cphase = (int*)realloc(o->cphase, sizeof(int) * nc);
    o->capcand = nc;
}

int ora_gen_round(rsa_oracle* o, uint64_t* n_out, uint64_t* max_new, int* may_outreach) {
    const int D = o->D;
    *n_out = 0;
    if (o->cls_idx >= o->k) return 2;
    /* compute_intensity_poisson takes an int (operator_algorithm.ixx:220-223) */
    const double intensity = 0.01 * (double)(int)o->nvox;
    const double maxI = intensity;
    o->last_round_vox = o->nvox;
    if (o->nvox == 0) return 1;
    double mult = (double)o->nbshots / maxI;
    if (mult > 1) mult = 1.;
    int nb = ora_poisson(&o->g, mult * intensity);
    uint64_t n = (uint64_t)nb;
    *max_new = o->cls_n[o->cls_idx];
    *may_outreach = (n >= o->cls_n[o->cls_idx]);
    cand_reserve(o, n);
    /* pick_points (list_of_voxels.ixx:107-129): voxel ~ U{0..V-1}, then D coordinates */
    for (uint64_t i = 0; i < n; i++) {
        uint32_t v = ora_uniform_int(&o->g, 0u, (uint32_t)(o->nvox - 1));
        const int64_t* c = o->vox + (uint64_t)v * D;
        for (int d = 0; d < D; d++) {
            const double orig = o->inf[d] + (double)c[d] * o->vlen[d];
            o->cpos[i * D + d] = orig + o->vlen[d] * ora_canonical(&o->g);
        }
    }
    /* generate_priority<int> (operator_algorithm.ixx:373-381) */
    for (uint64_t i = 0; i < n; i++) o->ckey[i] = ora_uniform_int(&o->g, 0u, (uint32_t)INT_MAX);
    if (o->uniform_radius) {
        /* RandomRadiusGenerator::operator() (radius_generator.hxx:27-34): law::uniform<double>(0, 1) */
        for (uint64_t i = 0; i < n; i++) {
            const double x = ora_canonical(&o->g);
            o->crad[i] = o->rtab ? ora_table_radius(o, x) : o->r_min + (o->r_max - o->r_min) * x;
            o->cphase[i] = o->uniform_phase;
        }
    } else {
        for (uint64_t i = 0; i < n; i++) {
            o->crad[i] = o->cls_r[o->cls_idx];
            o->cphase[i] = o->cls_phase[o->cls_idx];
        }
    }
    o->ncand = n;
    *n_out = n;
    return 0;
}

const double* ora_cand_pos(const rsa_oracle* o) { return o->cpos; }
const uint64_t* ora_cand_key(const rsa_oracle* o) { return o->ckey; }
const double* ora_cand_rad(const rsa_oracle* o) { return o->crad; }
const int* ora_cand_phase(const rsa_oracle* o) { return o->cphase; }

static void trace_push(rsa_oracle* o, uint64_t vox, uint64_t shots, uint64_t news, int refined) {
    if (o->ntrace == o->captrace) {
        uint64_t nc = o->captrace ? 2 * o->captrace : 256;
        o->tr_vox = (uint64_t*)realloc(o->tr_vox, sizeof(uint64_t) * nc);
        o->tr_shots = (uint64_t*)realloc(o->tr_shots, sizeof(uint64_t) * nc);
        o->tr_new = (uint64_t*)realloc(o->tr_new, sizeof(uint64_t) * nc);
        o->tr_ref = (uint8_t*)realloc(o->tr_ref, nc);
        o->captrace = nc;
    }
    o->tr_vox[o->ntrace] = vox;
    o->tr_shots[o->ntrace] = shots;
    o->tr_new[o->ntrace] = news;
    o->tr_ref[o->ntrace] = (uint8_t)refined;
    o->ntrace++;
}

int ora_end_round(rsa_oracle* o, uint64_t n_shots, uint64_t n_new, int* refined_out) {
    /* RadiusGenerator::update_placed (radius_generator.ixx:62-68), uint64 arithmetic */
    o->cls_n[o->cls_idx] = o->cls_n[o->cls_idx] - n_new;
    if (o->cls_n[o->cls_idx] == 0) o->cls_idx++;
    int should_continue = o->cls_idx < o->k;
    uint64_t nb_miss = n_shots - n_new;
    double miss_rate = (double)nb_miss / (0.000001 + (double)n_shots);
    int refined = 0;
    if (miss_rate > ora_miss_threshold(o->D)) {
        ora_refine(o);
        refined = 1;
    }
    trace_push(o, o->last_round_vox, n_shots, n_new, refined);
    if (refined_out) *refined_out = refined;
    return should_continue ? 0 : 1;
}

int ora_proceed(rsa_oracle* o, uint64_t seed) {
    ora_begin(o, seed);
    uint8_t* acc = NULL;
    uint64_t acccap = 0;
    for (;;) {
        uint64_t n, max_new;
        int may;
        int st = ora_gen_round(o, &n, &max_new, &may);
        if (st != 0) break;
        if (n == 0) continue;
        if (n > acccap) {
            acc = (uint8_t*)realloc(acc, n);
            acccap = n;
        }
        uint64_t n_new = 0;
        if (ora_apply_round(o, n, o->cpos, o->ckey, o->crad, o->cphase, max_new, may, acc, &n_new) != 0) {
            free(acc);
            return -1; /* the reference throws runtime_error("Unexpected ...") here */
        }
        int refined;
        if (ora_end_round(o, n, n_new, &refined)) break;
    }
    free(acc);
    return 0;
}

uint64_t ora_trace_len(const rsa_oracle* o) { return o->ntrace; }
void ora_set_cap_exact(rsa_oracle* o, int exact) { o->cap_exact = exact; }
int ora_trace_export(const rsa_oracle* o, uint64_t* voxels, uint64_t* shots, uint64_t* news, uint8_t* refined) {
    for (uint64_t i = 0; i < o->ntrace; i++) {
        if (voxels) voxels[i] = o->tr_vox[i];
        if (shots) shots[i] = o->tr_shots[i];
        if (news) news[i] = o->tr_new[i];
        if (refined) refined[i] = o->tr_ref[i];
    }
    return 0;
}

/* ===================================================================== */
/* Checkers                                                              */
/* ===================================================================== */

typedef struct {
    int D;
    uint64_t self;
    const double* x;
    double r;
    const double* rads;
    uint64_t count;
} ovl_ctx;

static int ovl_visit(void* vctx, uint64_t id, const double* img) {
    ovl_ctx* c = (ovl_ctx*)vctx;
    if (id <= c->self) return 0; /* each unordered pair once */
    if (ora_collide(c->D, c->r, c->x, c->rads[id], img)) c->count++;
    return 0;
}

uint64_t ora_count_overlaps(int dim, const double* inf, const double* sup, uint64_t n,
    const double* pos, const double* rad) {
    double L[ORA_MAX_DIM], rmax = 0;
    for (int d = 0; d < dim; d++) L[d] = sup[d] - inf[d];
    for (uint64_t i = 0; i < n; i++) if (rad[i] > rmax) rmax = rad[i];
    ora_store s;
    store_init(&s, dim, inf, L, 2 * rmax > 0 ? 2 * rmax : 1.0);
    for (uint64_t i = 0; i < n; i++) store_add(&s, pos + i * dim, rad[i], 0, 0);
    uint64_t total = 0;
    for (uint64_t i = 0; i < n; i++) {
        ovl_ctx c = { dim, i, pos + i * dim, rad[i], s.rad, 0 };
        store_visit(&s, pos + i * dim, ovl_visit, &c);
        total += c.count;
    }
    store_free(&s);
    return total;
}

uint64_t ora_uncovered_after_refinement(int dim, const double* inf, const double* sup,
    uint64_t n, const double* pos, const double* rad, double r_max, double r_min, int max_levels) {
    double r = r_max;
    uint64_t one = 1;
    int ph = 0;
    rsa_oracle* o = ora_create(dim, inf, sup, r_max, 1, &r, &one, &ph, 0.0, 1);
    o->r_min = r_min;
    ora_sphere_import(o, n, pos, rad, NULL);
    vox_build(o, r_max + r_min);
    for (int l = 0; l < max_levels && o->nvox > 0 && o->nvox < 20000000ull; l++) ora_refine(o);
    if (o->nvox > 0) vox_remove_covered(o);
    uint64_t left = o->nvox;
    ora_destroy(o);
    return left;
}
