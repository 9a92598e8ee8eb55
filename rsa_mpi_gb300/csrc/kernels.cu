// kernels.cu -- the sampler's kernels for one space dimension, compiled with -DRSA_DIM=D.
//
// One round (generate_spheres, operator_algorithm.ixx:534-566) is
//   k_darts -> k_probe -> k_collect -> k_settle x iterations -> [count cap] -> k_commit
// and one refinement (update_covered_voxels, :190-206) is
//   k_refine_mask -> scan of block counts -> k_refine_write.
#include <cfloat>
#include <vector>

#include "rsa_device.cuh"
#include "rsa_ops.h"

#ifndef RSA_DIM
#error "compile with -DRSA_DIM=<dimension>"
#endif

namespace rsagpu {
namespace {

constexpr int D = RSA_DIM;
constexpr int CHILDREN = 1 << D;
constexpr int MASK_WORDS = (CHILDREN + 31) / 32;
constexpr int K_PRE = 12;  // prefilter spheres kept per parent voxel (more: re-read from the grid)

// Child order of subdivide_uncovered: TabCorner (auxiliary/Path.ixx:86-103) for D = 2, 3; for D >= 4
// bit d of the child index is the offset along dimension d (the reference's generic table,
// Path.ixx:105-114, writes out of bounds and never sets dimension 0).
// Corner-table position of the child with offset bit d = (j >> d) & 1: the inverse of child_bits.
__device__ __forceinline__ int corner_of_child(int j) {
    if (D == 2) {
        const int tab = 0 | (3 << 2) | (2 << 4) | (1 << 6);
        return (tab >> (2 * j)) & 3;
    } else if (D == 3) {
        const uint32_t tab = 0u | (7u << 3) | (4u << 6) | (3u << 9) | (2u << 12) | (5u << 15) | (6u << 18) | (1u << 21);
        return (tab >> (3 * j)) & 7;
    } else {
        return j;
    }
}

__device__ __forceinline__ int corner_bit(int t, int d) {
    if (D == 2) {
        const int tab = 0b01101100;  // (0,0) (1,1) (0,1) (1,0): bit (2t + d)
        return (tab >> (2 * t + d)) & 1;
    } else if (D == 3) {
        // (0,0,0) (1,1,1) (0,0,1) (1,1,0) (0,1,0) (1,0,1) (0,1,1) (1,0,0)
        const uint32_t tab = (0u) | (7u << 3) | (4u << 6) | (3u << 9) | (2u << 12) | (5u << 15) | (6u << 18) | (1u << 21);
        return (tab >> (3 * t + d)) & 1;
    } else {
        return (t >> d) & 1;
    }
}

__host__ __device__ inline Grid<D> make_grid(const GridArgs& a) {
    Grid<D> g;
    g.ncells = a.ncells;
    for (int d = 0; d < D; d++) {
        g.n[d] = a.n[d];
        g.inv_c[d] = a.inv_c[d];
    }
    g.occ = a.occ;
    g.pos = a.pos;
    g.rad = a.rad;
    g.phase = a.phase;
    g.stencil = a.stencil;
    g.S = a.S;
    g.rows = a.rows;
    g.R = a.R;
    g.rows_r2 = a.rows_r2;
    g.c0f = (float)(1.0 / a.inv_c[0]);
    g.inv_c0f = (float)a.inv_c[0];
    g.rmax = a.rmax;
    g.off = a.off;
    g.radf = a.radf;
    for (int d = 0; d < D; d++) {
        g.c[d] = a.c[d];
        g.cf[d] = a.cf[d];
    }
    g.guard = a.guard;
    g.mono = a.mono;
    g.bocc = a.bocc;
    for (int d = 0; d < D; d++) {
        g.nb[d] = a.nb[d];
        g.inv_cf[d] = (float)a.inv_c[d];
    }
    g.rmono = a.rmono;
    g.rmonof = (float)a.rmono;
    g.rmaxf = (float)a.rmax;
    g.bnew = a.bnew;
    return g;
}

__host__ __device__ inline Geo<D> make_geo(const GridArgs& a) {
    Geo<D> g;
    for (int d = 0; d < D; d++) {
        g.inf[d] = a.inf[d];
        g.L[d] = a.L[d];
    }
    return g;
}

inline unsigned nblocks(uint64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// ------------------------------------------------------------------------------------------------
// level-0 voxel list: the lattice of getAllIndices (auxiliary/Loops.ixx:45-69) in 2x..x2 block order
// (block_order_coords); the list order is free (the reference's own order only matters to its own darts)
// ------------------------------------------------------------------------------------------------
struct NVox {
    int64_t n[D];
};

// Coordinates of entry v of the lattice n[0] x .. x n[D-1] listed block by block: blocks of 2 voxels per
// dimension (1 at an odd upper edge) in lattice order, dimension 0 fastest, and the voxels of a block
// dimension 0 fastest.  Any 8 consecutive entries of a 3D list form one 2x2x2 block, the group of the
// cooperative level-0 mask pass (k_refine_mask32c).  (A full Morton order costs some 80 64-bit products per
// voxel here, and the deeper levels, whose children are written next to their parent in either order,
// measured no faster with it.)
__device__ __forceinline__ void block_order_coords(uint64_t v, const int64_t* n, int64_t* out) {
    uint64_t thick[D], blk[D], rem = v;
#pragma unroll
    for (int d = D - 1; d >= 0; d--) {
        uint64_t t = 1, q = 1;
#pragma unroll
        for (int e = d + 1; e < D; e++) t *= thick[e];
#pragma unroll
        for (int e = 0; e < d; e++) q *= (uint64_t)n[e];
        const uint64_t unit = 2 * t * q;  // entries of a slab two voxels thick along d
        const uint64_t sl = rem / unit;
        blk[d] = sl;
        thick[d] = 2 * sl + 2 <= (uint64_t)n[d] ? 2 : 1;
        rem -= sl * unit;
    }
#pragma unroll
    for (int d = 0; d < D; d++) {
        out[d] = (int64_t)(2 * blk[d] + rem % thick[d]);
        rem /= thick[d];
    }
}

__global__ void k_vox_init(int64_t* vox, uint64_t V, NVox nv) {
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    block_order_coords(v, nv.n, vox + v * D);
}

// ------------------------------------------------------------------------------------------------
// darts: voxel ~ U{0..V-1}, x_d = (inf_d + coord_d len_d) + len_d u_d (pick_points,
// list_of_voxels.ixx:107-129), priority = 32 random bits (generate_priority, operator_algorithm.ixx:373-381)
// ------------------------------------------------------------------------------------------------
struct DartParams {
    uint32_t n;
    uint64_t V;
    const int64_t* vox;
    double len[D];
    double inf[D];
    uint32_t seed_lo, seed_hi, round_lo, round_hi;
    double radius;
    int32_t phase;
    int32_t rand_radius;  // continuous radius law: radius = r_lo + r_span x (dart_radius)
    double r_lo, r_span;
    const double* rtab;   // or a tabulated transform (ntab >= 2 knots), radii clamped to [r_lo, r_lo + r_span]
    int32_t ntab;
    double* pos;
    uint64_t* key;
    double* rad;
    int32_t* cphase;
    uint8_t* state;
    uint64_t* vidx_out;
    // FP32 form: the candidate's cell and FP32 offsets from a fixed-point map, the exact position deferred
    int32_t* kc;
    float* off;
    int64_t* cell;
    uint64_t rho_frac[D];  // level-0 voxel length / cell edge (voxel_cell_ratio)
    uint32_t rho_int[D];
    int32_t level;         // voxel level (fixed-point shift)
    int32_t ncell[D];      // cells per dimension
    float cf[D];           // cell edge rounded to float
    // binned order (optional): slot t holds dart perm[t]; perm lists the darts bin by bin, bin b =
    // (vbase + voxel) >> bin_shift, so that neighbouring threads of the probe hold neighbouring darts
    uint32_t* bin_hist;
    const uint64_t* bin_off;
    int32_t bin_shift;
    uint64_t vbase;        // first voxel of this list in the binned index space
    uint32_t* perm;
    uint32_t* err;         // error bits (ERR_DART_SLOT)
};

// radius of dart i: the class radius, or under a continuous law r_lo + r_span x with x the 53-bit uniform of
// the dart's own Philox call in a separate counter space (call word 0x80000000), as the reference's transform
// x -> r_min + (r_max - r_min) x (radius_generator.hxx:27-34)
// With a tabulated transform T (knots T(j / (n - 1)), j = 0 .. n - 1: any law the reference's
// RandomRadiusGenerator takes as a function of x, radius_generator.hxx:12-38) the radius is T interpolated
// linearly at x, kept within the knots' range.
__device__ __forceinline__ double dart_radius(const DartParams& p, uint32_t i) {
    if (!p.rand_radius) return p.radius;
    const uint4 r = philox4x32_10(make_uint4(i, p.round_lo, p.round_hi, 0x80000000u), make_uint2(p.seed_lo, p.seed_hi));
    const uint64_t bits = ((((uint64_t)r.x) << 32) | r.y) >> 11;
    const double x = (double)bits * 0x1.0p-53;
    if (p.ntab >= 2) {
        const double t = __dmul_rn(x, (double)(p.ntab - 1));
        int32_t j = (int32_t)t;
        j = j > p.ntab - 2 ? p.ntab - 2 : j;
        const double f = __dsub_rn(t, (double)j);
        const double a = p.rtab[j], b = p.rtab[j + 1];
        const double v = __dadd_rn(a, __dmul_rn(f, __dsub_rn(b, a)));
        const double hi = __dadd_rn(p.r_lo, p.r_span);
        return v < p.r_lo ? p.r_lo : (v > hi ? hi : v);
    }
    return __dadd_rn(p.r_lo, __dmul_rn(p.r_span, x));
}

// voxel drawn by dart i (the first Philox call's words 0 and 1)
__device__ __forceinline__ uint64_t dart_voxel(const DartParams& p, uint32_t i) {
    const uint4 r = philox4x32_10(make_uint4(i, p.round_lo, p.round_hi, 0u), make_uint2(p.seed_lo, p.seed_hi));
    return __umul64hi(((uint64_t)r.x << 32) | r.y, p.V);
}

// places dart i (index t in perm's index space) in its bin: perm[bin_off[b] + rank] = t.  A full bin (which
// the histogram pass rules out) raises ERR_DART_SLOT and places nothing.
__device__ __forceinline__ void place_dart(const DartParams& p, uint32_t i, uint32_t t) {
    const uint64_t b = (p.vbase + dart_voxel(p, i)) >> p.bin_shift;
    const uint32_t left = atomicSub(p.bin_hist + b, 1u);
    if (left == 0u) {
        atomicOr(p.err, (uint32_t)ERR_DART_SLOT);
        return;
    }
    p.perm[p.bin_off[b] + (left - 1u)] = t;
}

// Philox words of dart i: [0, 1] voxel draw, [2 + 2d, 3 + 2d] coordinate d, [2 + 2D] priority
template <int CALLS>
__device__ __forceinline__ void dart_words(const DartParams& p, uint32_t i, uint32_t* w) {
    const uint2 k = make_uint2(p.seed_lo, p.seed_hi);
#pragma unroll
    for (int c = 0; c < CALLS; c++) {
        const uint4 r = philox4x32_10(make_uint4(i, p.round_lo, p.round_hi, (uint32_t)c), k);
        w[4 * c + 0] = r.x;
        w[4 * c + 1] = r.y;
        w[4 * c + 2] = r.z;
        w[4 * c + 3] = r.w;
    }
}

// FP32 form of a dart: the same voxel, coordinates and priority as dart_body, but the FP64 position is not
// formed (that is 7 FP64 instructions per coordinate, each costing 64 FP32 ones on this GPU).  Instead:
//  * cell and FP32 offset from the exact dart y = (cc + u) len / c in fixed point (fixed_cell: integer part =
//    cell, fraction = offset; error below 2^-31 cell edges, far inside the guard band);
//  * the inputs of the exact position kept for later: the voxel index in cell[o] and the 53 random bits of
//    each coordinate in pos[o] (lazy_position forms the FP64 position for the candidates that need it).
__device__ __forceinline__ void dart32_body(const DartParams& p, uint32_t i, uint64_t o) {
    constexpr int WORDS = 2 + 2 * D + 1;
    constexpr int CALLS = (WORDS + 3) / 4;
    uint32_t w[CALLS * 4];
    dart_words<CALLS>(p, i, w);
    const uint64_t r64 = ((uint64_t)w[0] << 32) | w[1];
    const uint64_t v = __umul64hi(r64, p.V);
    p.cell[o] = (int64_t)v;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const uint64_t bits = (((uint64_t)w[2 + 2 * d] << 32) | w[3 + 2 * d]) >> 11;  // 53 bits
        p.pos[o * D + d] = __longlong_as_double((long long)bits);
        int64_t kd;
        uint32_t fr;
        fixed_cell((uint64_t)p.vox[v * D + d], bits, p.rho_int[d], p.rho_frac[d], p.level, kd, fr);
        if (kd >= p.ncell[d]) kd -= p.ncell[d];
        kd = kd < p.ncell[d] ? kd : p.ncell[d] - 1;
        p.kc[o * D + d] = (int32_t)kd;
        p.off[o * D + d] = __fmul_rn(__fmul_rn(u32_to_float(fr), 0x1p-32f), p.cf[d]);
    }
    p.key[o] = ((uint64_t)w[2 + 2 * D] << 32) | i;
    p.rad[o] = dart_radius(p, i);
    p.cphase[o] = p.phase;
    p.state[o] = ST_UNDECIDED;
}

// Dart i of the round (counter (i, round, call) under the run's key), written to candidate slot o.
__device__ __forceinline__ void dart_body(const DartParams& p, uint32_t i, uint64_t o) {
    constexpr int WORDS = 2 + 2 * D + 1;
    constexpr int CALLS = (WORDS + 3) / 4;
    uint32_t w[CALLS * 4];
    dart_words<CALLS>(p, i, w);
    const uint64_t r64 = ((uint64_t)w[0] << 32) | w[1];
    const uint64_t v = __umul64hi(r64, p.V);
    if (p.vidx_out) p.vidx_out[o] = v;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const uint64_t bits = (((uint64_t)w[2 + 2 * d] << 32) | w[3 + 2 * d]) >> 11;  // 53 bits
        const double u = (double)bits * 0x1.0p-53;
        const double orig = __dadd_rn(p.inf[d], __dmul_rn((double)p.vox[v * D + d], p.len[d]));
        p.pos[o * D + d] = __dadd_rn(orig, __dmul_rn(p.len[d], u));
    }
    p.key[o] = ((uint64_t)w[2 + 2 * D] << 32) | i;
    p.rad[o] = dart_radius(p, i);
    p.cphase[o] = p.phase;
    p.state[o] = ST_UNDECIDED;
}

// slot t of the round: dart perm[t] in the binned order, else dart t
__global__ void k_darts(DartParams p) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    dart_body(p, p.perm ? p.perm[t] % p.n : t, t);
}

__global__ void k_darts32(DartParams p) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.n) return;
    dart32_body(p, p.perm ? p.perm[t] % p.n : t, t);
}

// binned order: histogram of the darts' bins, then (after a scan) the permutation
__global__ void k_dart_bins(DartParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    atomicAdd(p.bin_hist + ((p.vbase + dart_voxel(p, i)) >> p.bin_shift), 1u);
}

__global__ void k_dart_perm(DartParams p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    place_dart(p, i, i);
}

// The exact FP64 position of lazy candidate i, by dart_body's own expression (list_of_voxels.ixx:107-129).
// The empty volatile asm keeps the FP64 work where it is called (the guard band, the survivors).
__device__ __forceinline__ void lazy_position(const Geo<D>& geo, const CandArgs& c, uint32_t i, double* x) {
    uint64_t v = (uint64_t)c.cell[i];
    asm volatile("" : "+l"(v));
#pragma unroll
    for (int d = 0; d < D; d++) {
        const uint64_t bits = (uint64_t)__double_as_longlong(c.pos[(uint64_t)i * D + d]);
        const double u = (double)bits * 0x1.0p-53;
        const double orig = __dadd_rn(geo.inf[d], __dmul_rn((double)c.lvox[v * D + d], c.llen[d]));
        x[d] = __dadd_rn(orig, __dmul_rn(c.llen[d], u));
    }
}

// ------------------------------------------------------------------------------------------------
// probe: a candidate overlapping a placed sphere (or its periodic image) is dead
// (remove_collisions_with_validated_spheres, operator_cells_and_data_storage.ixx:54-76); the
// others are linked into the candidate cell lists and appended to the alive list.
// ------------------------------------------------------------------------------------------------
// Probe of undecided candidate i; returns true when it stays alive (linked into the cell lists).  OWN_FIRST
// (FP32 form, one radius class) walks the dart's own brick first: 97 % of the darts die, most at a near sphere.
template <bool F32, bool OWN_FIRST = false>
__device__ __forceinline__ bool probe_body(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i,
                                           uint32_t& rt) {
    const double r = c.rad[i];
    int32_t k[D];
    double x[D];
    auto fp64_cell = [&]() {
        // cell and FP32 offsets of an exact FP64 position, as the placed spheres' are formed (k_commit)
        cell_of<D>(g, geo, x, k);
        if (F32) {
#pragma unroll
            for (int d = 0; d < D; d++) {
                const double base = __dadd_rn(geo.inf[d], __dmul_rn((double)k[d], g.c[d]));
                c.off[(uint64_t)i * D + d] = __double2float_rn(__dsub_rn(x[d], base));
                c.kc[(uint64_t)i * D + d] = k[d];
            }
        }
    };
    bool hit;
    if constexpr (!F32) {
#pragma unroll
        for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
        cell_of<D>(g, geo, x, k);
        hit = visit_placed<D>(g, geo, k, nullptr, search_r2(r, g.rmax), [&](int64_t, const double* img, double rs) {
            return collide64<D>(r, x, rs, img);
        });
    } else {
        // FP32 screen: certain outside the guard band, FP64 retest inside it.  A lazy candidate (FP32 darts)
        // has its cell and offsets already and forms its FP64 position only when a retest or survival needs it.
        const bool lazy = c.lazy != 0;
        if (!lazy) {
#pragma unroll
            for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
            fp64_cell();
        }
        bool have_x = !lazy;
        float offq[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            k[d] = c.kc[(uint64_t)i * D + d];
            offq[d] = c.off[(uint64_t)i * D + d];
        }
        float rf = __double2float_rn(r);
        asm volatile("" : "+f"(rf));  // not rematerialised in the loop below: the conversion runs on the FP64 pipe
        hit = visit_placed_fo<D, OWN_FIRST>(g, k, offq, search_r2f(rf, g.rmaxf), [&](int64_t idx, const int32_t* o, const int8_t* q) {
            const float rs = g.mono ? g.rmonof : g.radf[idx];
            const float R = __fadd_rn(rf, rs);
            const float R2 = __fmul_rn(R, R);
            float dlt[D];
            model_delta<D>(g.cf, o, g.off + idx * D, offq, dlt);
            const float d2 = sumsq32<D>(dlt);
            if (d2 < __fsub_rn(R2, g.guard)) return true;
            if (d2 > __fadd_rn(R2, g.guard)) return false;
            rt++;
            if (!have_x) {
                lazy_position(geo, c, i, x);
                have_x = true;
            }
            double p[D], img[D];
#pragma unroll
            for (int d = 0; d < D; d++) p[d] = g.pos[idx * D + d];
            image_of<D>(geo, p, q, img);
            return collide64<D>(r, x, g.mono ? g.rmono : g.rad[idx], img);
        });
        if (!hit && lazy) {
            // a survivor: its exact position, and its cell and offsets from it, for the rest of the round
            if (!have_x) lazy_position(geo, c, i, x);
#pragma unroll
            for (int d = 0; d < D; d++) c.pos[(uint64_t)i * D + d] = x[d];
            fp64_cell();
        }
    }
    if (hit) {
        c.state[i] = ST_DEAD;
        return false;
    }
    if (F32) c.radf[i] = __double2float_rn(r);
    const int64_t idx = cell_index<D>(g, k);
    c.cell[i] = idx;
    c.next[i] = atomicExch(c.head + idx, (int32_t)i);
    atomicOr(c.cocc + (idx >> 5), 1u << (idx & 31));
    return true;
}

template <bool F32, bool OWN_FIRST = false>
__global__ void k_probe(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t rt = 0;
    const bool alive = i < c.n && c.state[i] == ST_UNDECIDED && probe_body<F32, OWN_FIRST>(g, geo, c, i, rt);
    const uint32_t slot = warp_append(&c.counters[0], alive);
    if (alive) c.alive[slot] = i;
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// Reach of a candidate-candidate search: the round's largest candidate radius when the host gives it, else the
// grid's largest radius.
__device__ __forceinline__ double cand_rmax(const Grid<D>& g, const CandArgs& c) {
    return c.rcmaxf > 0.f ? c.rcmax : g.rmax;
}
__device__ __forceinline__ float cand_rmaxf(const Grid<D>& g, const CandArgs& c) {
    return c.rcmaxf > 0.f ? c.rcmaxf : g.rmaxf;
}

// Visits the same-round candidates in the stencil around cell k (linked lists head/next): f(j, img, q), img the
// image of candidate j seen through the periodic shift q (q = 0: its own position).
template <class F>
__device__ __forceinline__ void visit_candidates(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c,
                                                 const int32_t* k, const float* qo, float R2q, F&& f) {
    walk_rows<D>(g.n, g.rows, g.R, g.rows_r2, g.cf, g.inv_c0f, R2q, k, qo, [&](int64_t base, int32_t lo, int32_t hi, const int8_t* q, const int8_t*) {
        for (int32_t x = lo; x <= hi; x += 32) {
            const int len = hi - x + 1 < 32 ? hi - x + 1 : 32;
            uint32_t bits = occ_bits(c.cocc, base + x, len);  // cells holding a candidate of this round
            while (bits) {
                const int jj = __ffs(bits) - 1;
                bits &= bits - 1;
                for (int32_t j = c.head[base + x + jj]; j >= 0; j = c.next[j]) {
                    double p[D], img[D];
#pragma unroll
                    for (int d = 0; d < D; d++) p[d] = c.pos[(uint64_t)j * D + d];
                    image_of<D>(geo, p, q, img);
                    if (f(j, img, q)) return true;
                }
            }
        }
        return false;
    });
}

// Same walk with the integer cell offset o of each candidate (FP32 screen); f(j, o, q).
template <class F>
__device__ __forceinline__ void visit_candidates_o(const Grid<D>& g, const CandArgs& c, const int32_t* k, const float* qo,
                                                   float R2q, F&& f) {
    walk_rows<D>(g.n, g.rows, g.R, g.rows_r2, g.cf, g.inv_c0f, R2q, k, qo, [&](int64_t base, int32_t lo, int32_t hi, const int8_t* q, const int8_t* row) {
        int32_t o[D];
#pragma unroll
        for (int d = 1; d < D; d++) o[d] = row[1 + d];
        const int32_t shift0 = (q[0] < 0 ? -g.n[0] : (q[0] > 0 ? g.n[0] : 0)) - k[0];
        for (int32_t x = lo; x <= hi; x += 32) {
            const int len = hi - x + 1 < 32 ? hi - x + 1 : 32;
            uint32_t bits = occ_bits(c.cocc, base + x, len);
            while (bits) {
                const int jj = __ffs(bits) - 1;
                bits &= bits - 1;
                o[0] = x + jj + shift0;
                for (int32_t j = c.head[base + x + jj]; j >= 0; j = c.next[j])
                    if (f(j, o, q)) return true;
            }
        }
        return false;
    });
}

// Screened overlap test of candidate i (FP32 data offq, rf; FP64 data x, r) with candidate j seen at
// cell offset o and image shift q: certain outside the guard band, FP64 retest inside it.
__device__ __forceinline__ bool cand_collide32(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, const double* x,
                                               double r, const float* offq, float rf, int32_t j, const int32_t* o,
                                               const int8_t* q, uint32_t& rt) {
    const float R = __fadd_rn(rf, c.radf[j]);
    const float R2 = __fmul_rn(R, R);
    float dlt[D];
    model_delta<D>(g.cf, o, c.off + (uint64_t)j * D, offq, dlt);
    const float d2 = sumsq32<D>(dlt);
    if (d2 < __fsub_rn(R2, g.guard)) return true;
    if (d2 > __fadd_rn(R2, g.guard)) return false;
    rt++;
    double p[D], img[D];
#pragma unroll
    for (int d = 0; d < D; d++) p[d] = c.pos[(uint64_t)j * D + d];
    image_of<D>(geo, p, q, img);
    return collide64<D>(r, x, c.rad[j], img);
}

// candidate order: priority key, then candidate index (a strict total order; the reference's
// detection compares priorities only, so two overlapping equal-priority candidates both pass there)
__device__ __forceinline__ bool precedes(uint64_t kj, int32_t j, uint64_t ki, uint32_t i) {
    return kj < ki || (kj == ki && (uint32_t)j < i);
}

__device__ __forceinline__ uint8_t load_state(const uint8_t* s, int32_t j) {
    return *((volatile const uint8_t*)(s + j));
}

// ------------------------------------------------------------------------------------------------
// settle: the accepted set is the sequential greedy in ascending key (find_solve_conflicts and the
// add_to_sample loop, operator_cells_and_data_storage.ixx:79-143, operator_algorithm.ixx:383-443):
// a candidate is accepted iff no accepted candidate that precedes it (key, then index) overlaps it.  Computed as
// a monotone fixpoint: collect stores each candidate's strictly-lower overlapping candidates (seen
// from the candidate itself, i.e. against their periodic image); settle iterations then accept a
// candidate whose blockers are all rejected and reject one with an accepted blocker.  The smallest
// undecided key always settles, so each iteration makes progress.
// ------------------------------------------------------------------------------------------------
// Collects the overlapping candidates that precede alive candidate i; returns true when it stays undecided.
template <bool F32>
__device__ __forceinline__ bool collect_body(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i,
                                             uint32_t& rt) {
    {
        double x[D];
#pragma unroll
        for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
        const double r = c.rad[i];
        const uint64_t key = c.key[i];
        int nb = 0;
        // a collider seen through the periodic boundary is stored with BLK_WRAP set (the count cap's pass
        // structure treats it as the reference's ghost copy)
        auto record = [&](int32_t j, const int8_t* q) {
            if (nb < NB) c.blk[(uint64_t)i * NB + nb] = wrapped<D>(q) ? (int32_t)((uint32_t)j | BLK_WRAP) : j;
            nb++;
        };
        if constexpr (!F32) {
            int32_t k[D];
            cell_of<D>(g, geo, x, k);
            visit_candidates(g, geo, c, k, nullptr, search_r2(r, cand_rmax(g, c)), [&](int32_t j, const double* img, const int8_t* q) {
                if (!precedes(c.key[j], j, key, i)) return false;
                if (collide64<D>(r, x, c.rad[j], img)) record(j, q);
                return false;
            });
        } else {
            int32_t k[D];
            float offq[D];
#pragma unroll
            for (int d = 0; d < D; d++) {
                k[d] = c.kc[(uint64_t)i * D + d];
                offq[d] = c.off[(uint64_t)i * D + d];
            }
            float rf = __double2float_rn(r);
        asm volatile("" : "+f"(rf));  // not rematerialised in the loop below: the conversion runs on the FP64 pipe
            visit_candidates_o(g, c, k, offq, search_r2f(rf, cand_rmaxf(g, c)), [&](int32_t j, const int32_t* o, const int8_t* q) {
                if (!precedes(c.key[j], j, key, i)) return false;
                if (cand_collide32(g, geo, c, x, r, offq, rf, j, o, q, rt)) record(j, q);
                return false;
            });
        }
        if (nb == 0) {
            c.state[i] = ST_ACCEPTED;
            c.nblk[i] = 0;  // read again by the count cap's passes
            return false;
        }
        c.nblk[i] = nb > NB ? (uint8_t)NB_OVERFLOW : (uint8_t)nb;
        return true;
    }
}

template <bool F32>
__global__ void k_collect(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    uint32_t rt = 0;
    const bool undecided = t < nalive && collect_body<F32>(g, geo, c, c.alive[t], rt);
    const uint32_t mask = __ballot_sync(0xffffffffu, undecided);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[0], (uint32_t)__popc(mask));
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// One settle step of alive candidate i; returns true when it is still undecided.
template <bool F32>
__device__ __forceinline__ bool settle_body(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i,
                                            uint32_t& rt) {
    bool still = false;
    {
        {
            if (load_state(c.state, i) == ST_UNDECIDED) {
                bool any_acc = false, all_rej = true;
                const uint8_t nb = c.nblk[i];
                auto tally_blocker = [&](int32_t j) {
                    const uint8_t s = load_state(c.state, j);
                    any_acc |= (s == ST_ACCEPTED);
                    all_rej &= (s == ST_REJECTED);
                };
                if (nb != NB_OVERFLOW) {
                    for (int b = 0; b < nb; b++) tally_blocker(blk_index(c.blk[(uint64_t)i * NB + b]));
                } else {
                    double x[D];
#pragma unroll
                    for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
                    const double r = c.rad[i];
                    const uint64_t key = c.key[i];
                    if constexpr (!F32) {
                        int32_t k[D];
                        cell_of<D>(g, geo, x, k);
                        visit_candidates(g, geo, c, k, nullptr, search_r2(r, cand_rmax(g, c)), [&](int32_t j, const double* img, const int8_t*) {
                            if (!precedes(c.key[j], j, key, i)) return false;
                            if (collide64<D>(r, x, c.rad[j], img)) tally_blocker(j);
                            return any_acc;
                        });
                    } else {
                        int32_t k[D];
                        float offq[D];
#pragma unroll
                        for (int d = 0; d < D; d++) {
                            k[d] = c.kc[(uint64_t)i * D + d];
                            offq[d] = c.off[(uint64_t)i * D + d];
                        }
                        float rf = __double2float_rn(r);
        asm volatile("" : "+f"(rf));  // not rematerialised in the loop below: the conversion runs on the FP64 pipe
                        visit_candidates_o(g, c, k, offq, search_r2f(rf, cand_rmaxf(g, c)), [&](int32_t j, const int32_t* o, const int8_t* q) {
                            if (!precedes(c.key[j], j, key, i)) return false;
                            if (cand_collide32(g, geo, c, x, r, offq, rf, j, o, q, rt)) tally_blocker(j);
                            return any_acc;
                        });
                    }
                }
                if (any_acc) c.state[i] = ST_REJECTED;
                else if (all_rej) c.state[i] = ST_ACCEPTED;
                else still = true;
            }
        }
    }
    return still;
}

template <bool F32>
__global__ void k_settle(Grid<D> g, Geo<D> geo, CandArgs c, int it) {
    if (c.und[it - 1] == 0) return;
    const uint32_t nalive = c.counters[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (nalive + stride - 1) / stride;  // same trip count for every lane
    uint32_t rt = 0;
    for (uint32_t rr = 0; rr < rounds; rr++) {
        const uint32_t t = t0 + rr * stride;
        const bool still = t < nalive && settle_body<F32>(g, geo, c, c.alive[t], rt);
        const uint32_t mask = __ballot_sync(0xffffffffu, still);
        if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[it], (uint32_t)__popc(mask));
    }
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// keys of the accepted candidates, for the count cap (retain_only_first_elements)
__global__ void k_gather_accepted(CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    bool acc = false;
    uint32_t i = 0;
    if (t < nalive) {
        i = c.alive[t];
        acc = c.state[i] == ST_ACCEPTED;
    }
    const uint32_t slot = warp_append(&c.counters[3], acc);
    if (acc) c.gather[slot] = c.key[i];
}

// drops accepted candidates beyond the cap: priority (key >> 32) > pivot (reference rule) or
// key > key_cut (exact rule)
__global__ void k_cut_accepted(CandArgs c, int use_pivot, double pivot, uint64_t key_cut) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    if (t >= nalive) return;
    const uint32_t i = c.alive[t];
    if (c.state[i] != ST_ACCEPTED) return;
    const uint64_t key = c.key[i];
    const bool drop = use_pivot ? ((double)(key >> 32) > pivot) : (key > key_cut);
    if (drop) c.state[i] = ST_REJECTED;
}

// ------------------------------------------------------------------------------------------------
// Count cap under the reference rule: the pass structure of add_to_sample (operator_algorithm.ixx:383-443)
// over find_solve_conflicts (operator_cells_and_data_storage.ixx:79-143).  A pass classifies its candidates
// in key order.  A candidate is Conflict when a preceding colliding candidate of the pass is seen through the
// periodic boundary (the reference's ghost copy, which stays Undecided during a pass) or is itself Conflict;
// else Skip when one is Undecided; else Undecided.  Where a candidate has colliders of both kinds the
// reference takes the first in its cell-scan order; here Conflict wins.  Each classification depends only on
// preceding candidates, so it is a monotone fixpoint like settle: the smallest unclassified key always
// classifies.  The host then compares the pass's Undecided count with the cap (retain_only_first_elements
// with the pivot, or validation and the next pass of the Conflict ones).
// ------------------------------------------------------------------------------------------------
// Visits the preceding colliders of alive candidate i, stored by collect or, after an overflow, walked again:
// f(j, wrapped) returns true to stop.
template <bool F32, class F>
__device__ __forceinline__ void visit_colliders(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i,
                                                uint32_t& rt, F&& f) {
    const uint8_t nb = c.nblk[i];
    if (nb != NB_OVERFLOW) {
        for (int b = 0; b < nb; b++) {
            const int32_t e = c.blk[(uint64_t)i * NB + b];
            if (f(blk_index(e), blk_wrapped(e))) return;
        }
        return;
    }
    double x[D];
#pragma unroll
    for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
    const double r = c.rad[i];
    const uint64_t key = c.key[i];
    if constexpr (!F32) {
        int32_t k[D];
        cell_of<D>(g, geo, x, k);
        visit_candidates(g, geo, c, k, nullptr, search_r2(r, cand_rmax(g, c)), [&](int32_t j, const double* img, const int8_t* q) {
            if (!precedes(c.key[j], j, key, i)) return false;
            return collide64<D>(r, x, c.rad[j], img) && f(j, wrapped<D>(q));
        });
    } else {
        int32_t k[D];
        float offq[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            k[d] = c.kc[(uint64_t)i * D + d];
            offq[d] = c.off[(uint64_t)i * D + d];
        }
        float rf = __double2float_rn(r);
        asm volatile("" : "+f"(rf));
        visit_candidates_o(g, c, k, offq, search_r2f(rf, cand_rmaxf(g, c)), [&](int32_t j, const int32_t* o, const int8_t* q) {
            if (!precedes(c.key[j], j, key, i)) return false;
            return cand_collide32(g, geo, c, x, r, offq, rf, j, o, q, rt) && f(j, wrapped<D>(q));
        });
    }
}

// the candidates of the first pass: every alive candidate (the greedy settle's states are replaced)
__global__ void k_pass_begin(CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    const bool in = t < nalive;
    if (in) c.state[c.alive[t]] = ST_UNDECIDED;
    const uint32_t mask = __ballot_sync(0xffffffffu, in);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[0], (uint32_t)__popc(mask));
}

// The classification.  A candidate is Conflict iff a chain of colliders of the pass, each preceding the next,
// leads to it from a collision through the periodic boundary: Conflict never depends on the Undecided / Skip
// outcome.  So the Conflict set is found first, as a breadth-first search: the sources are the candidates with
// a preceding collider of the pass seen through the boundary (k_pass_sources), and each Conflict candidate marks
// the later candidates of the pass that collide with it (k_pass_push, over the round's candidate lists).  The
// candidates left are not Conflict, and their preceding colliders of the pass are neither Conflict nor seen
// through the boundary, so the rest is the greedy on them (pass_body): Skip as soon as a preceding collider is
// Undecided (the pass's accepted), Undecided once all are Skip.
//
// Frontiers of the search: c.gather's memory as two arrays of candidate indices, counts in counters[5 + f].
__device__ __forceinline__ uint32_t* frontier(const CandArgs& c, int f) {
    return reinterpret_cast<uint32_t*>(c.gather) + (uint64_t)f * c.n;
}

// Claims candidate i for the Conflict set (its state byte UNDECIDED -> ST_PASS_C, by a CAS on the word holding
// it); true for the one thread that changed it.
__device__ __forceinline__ bool claim_conflict(const CandArgs& c, uint32_t i) {
    uint32_t* w = reinterpret_cast<uint32_t*>(c.state + (i & ~3u));
    const int sh = 8 * (int)(i & 3u);
    uint32_t old = *((volatile uint32_t*)w);
    while (((old >> sh) & 0xffu) == ST_UNDECIDED) {
        const uint32_t nw = (old & ~(0xffu << sh)) | ((uint32_t)ST_PASS_C << sh);
        const uint32_t prev = atomicCAS(w, old, nw);
        if (prev == old) return true;
        old = prev;
    }
    return false;
}

template <bool F32>
__global__ void k_pass_sources(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    bool src = false;
    uint32_t i = 0, rt = 0;
    if (t < nalive) {
        i = c.alive[t];
        const uint8_t nb = c.nblk[i];
        if (c.state[i] == ST_UNDECIDED && nb != 0) {
            if (nb != NB_OVERFLOW) {
                for (int b = 0; b < nb && !src; b++) {
                    const int32_t e = c.blk[(uint64_t)i * NB + b];
                    if (blk_wrapped(e)) src = c.state[blk_index(e)] == ST_UNDECIDED;  // in the pass
                }
            } else {
                visit_colliders<F32>(g, geo, c, i, rt, [&](int32_t j, bool wrap) {
                    src |= wrap && c.state[j] == ST_UNDECIDED;
                    return src;
                });
            }
        }
    }
    // mark after every source test of the pass has read the states it needs: sources only by the ones read
    // here, so a separate loop writes
    const uint32_t slot = warp_append(&c.counters[5], src);
    if (src) frontier(c, 0)[slot] = i;
}

// marks the sources found (their states stay UNDECIDED while the sources are searched)
__global__ void k_pass_mark(CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < c.counters[5]) c.state[frontier(c, 0)[t]] = ST_PASS_C;
}

// One level of the search: every Conflict candidate of frontier `from` marks the later candidates of the pass
// that collide with it and puts them in frontier 1 - from.
template <bool F32>
__global__ void k_pass_push(Grid<D> g, Geo<D> geo, CandArgs c, int from) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nf = c.counters[5 + from];
    if (t >= nf) return;
    const uint32_t j = frontier(c, from)[t];
    uint32_t* out = frontier(c, 1 - from);
    uint32_t* cnt = &c.counters[5 + (1 - from)];
    double x[D];
#pragma unroll
    for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)j * D + d];
    const double r = c.rad[j];
    const uint64_t key = c.key[j];
    uint32_t rt = 0;
    auto mark = [&](int32_t i) {
        if (claim_conflict(c, (uint32_t)i)) out[atomicAdd(cnt, 1u)] = (uint32_t)i;
    };
    if constexpr (!F32) {
        int32_t k[D];
        cell_of<D>(g, geo, x, k);
        visit_candidates(g, geo, c, k, nullptr, search_r2(r, cand_rmax(g, c)), [&](int32_t i, const double* img, const int8_t*) {
            if (!precedes(key, (int32_t)j, c.key[i], (uint32_t)i)) return false;
            if (load_state(c.state, i) != ST_UNDECIDED) return false;
            if (collide64<D>(r, x, c.rad[i], img)) mark(i);
            return false;
        });
    } else {
        int32_t k[D];
        float offq[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            k[d] = c.kc[(uint64_t)j * D + d];
            offq[d] = c.off[(uint64_t)j * D + d];
        }
        float rf = __double2float_rn(r);
        asm volatile("" : "+f"(rf));
        visit_candidates_o(g, c, k, offq, search_r2f(rf, cand_rmaxf(g, c)), [&](int32_t i, const int32_t* o, const int8_t* q) {
            if (!precedes(key, (int32_t)j, c.key[i], (uint32_t)i)) return false;
            if (load_state(c.state, i) != ST_UNDECIDED) return false;
            if (cand_collide32(g, geo, c, x, r, offq, rf, i, o, q, rt)) mark(i);
            return false;
        });
    }
    if (F32 && rt) atomicAdd(&c.counters[4], rt);
}

// One greedy step of a candidate of the pass that is not Conflict; returns true when it is still undecided.
template <bool F32>
__device__ __forceinline__ bool pass_body(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i,
                                          uint32_t& rt) {
    if (load_state(c.state, i) != ST_UNDECIDED) return false;
    bool any_u = false, pending = false;
    visit_colliders<F32>(g, geo, c, i, rt, [&](int32_t j, bool) {
        const uint8_t s = load_state(c.state, j);
        any_u |= s == ST_PASS_U;
        pending |= s == ST_UNDECIDED;
        return any_u;
    });
    if (any_u) c.state[i] = ST_PASS_S;
    else if (pending) return true;
    else c.state[i] = ST_PASS_U;
    return false;
}

template <bool F32>
__global__ void k_pass_step(Grid<D> g, Geo<D> geo, CandArgs c, int it) {
    if (c.und[it - 1] == 0) return;
    const uint32_t nalive = c.counters[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (nalive + stride - 1) / stride;  // same trip count for every lane
    uint32_t rt = 0;
    for (uint32_t rr = 0; rr < rounds; rr++) {
        const uint32_t t = t0 + rr * stride;
        const bool still = t < nalive && pass_body<F32>(g, geo, c, c.alive[t], rt);
        const uint32_t mask = __ballot_sync(0xffffffffu, still);
        if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[it], (uint32_t)__popc(mask));
    }
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// keys of the pass's Undecided candidates (counters[3] = their number)
__global__ void k_pass_gather(CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    bool u = false;
    uint32_t i = 0;
    if (t < nalive) {
        i = c.alive[t];
        u = c.state[i] == ST_PASS_U;
    }
    const uint32_t slot = warp_append(&c.counters[3], u);
    if (u) c.gather[slot] = c.key[i];
}

// End of a pass.  PASS_VALIDATE: Undecided -> accepted, Skip -> rejected, Conflict kept for the next pass
// (update_sphere_tags).  PASS_PIVOT: Undecided with priority <= pivot -> accepted, every other candidate not
// accepted -> rejected (retain_only_first_elements).  PASS_END: every candidate not accepted -> rejected.
constexpr int PASS_VALIDATE = CAP_PASS_VALIDATE, PASS_PIVOT = CAP_PASS_PIVOT;
__global__ void k_pass_close(CandArgs c, int mode, double pivot) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    if (t >= nalive) return;
    const uint32_t i = c.alive[t];
    const uint8_t s = c.state[i];
    if (s == ST_ACCEPTED) return;
    uint8_t ns = ST_REJECTED;
    if (mode == PASS_VALIDATE) {
        if (s == ST_PASS_U) ns = ST_ACCEPTED;
        else if (s == ST_PASS_C) ns = ST_PASS_C;
    } else if (mode == PASS_PIVOT) {
        if (s == ST_PASS_U && !((double)(c.key[i] >> 32) > pivot)) ns = ST_ACCEPTED;
    }
    if (ns != s) c.state[i] = ns;
}

// The next pass: the Conflict candidates that collide with no candidate validated so far.  A validated
// candidate that collides with a Conflict one always precedes it (a later one would have seen the Conflict
// candidate, or its ghost copy, and been Conflict itself), so the preceding colliders are enough.
template <bool F32>
__global__ void k_pass_next(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    bool in = false;
    uint32_t rt = 0;
    if (t < nalive) {
        const uint32_t i = c.alive[t];
        if (c.state[i] == ST_PASS_C) {
            bool hit = false;
            visit_colliders<F32>(g, geo, c, i, rt, [&](int32_t j, bool) {
                hit |= c.state[j] == ST_ACCEPTED;
                return hit;
            });
            c.state[i] = hit ? ST_REJECTED : ST_UNDECIDED;
            in = !hit;
        }
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, in);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[0], (uint32_t)__popc(mask));
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// commit: accepted candidates become placed spheres; the candidate lists are cleared.
// Commit of alive candidate i; returns true when it was accepted (and is now a placed sphere).
__device__ __forceinline__ bool commit_body(const Grid<D>& g, const Geo<D>& geo, const CandArgs& c, uint32_t i) {
    bool acc = false;
    {
        const int64_t idx = c.cell[i];
        c.head[idx] = -1;
        atomicAnd(c.cocc + (idx >> 5), ~(1u << (idx & 31)));
        if (c.state[i] == ST_ACCEPTED) {
            acc = true;
            const uint32_t bit = 1u << (idx & 31);
            const uint32_t old = atomicOr(g.occ + (idx >> 5), bit);
            if (old & bit) atomicOr(&c.counters[2], (uint32_t)ERR_DOUBLE_OCCUPANCY);
            int64_t rem = idx;
            int64_t bidx = 0, bmul = 1;
            int bbit = 0;
            constexpr int SB = brick_bits<D>();
#pragma unroll
            for (int d = 0; d < D; d++) {
                const int32_t kd = (int32_t)(rem % g.n[d]);
                rem /= g.n[d];
                if (D == 2 || D == 3) {
                    bidx += (kd >> SB) * bmul;
                    bmul *= g.nb[d];
                    bbit += (kd & ((1 << SB) - 1)) << (SB * d);
                }
                const double x = c.pos[(uint64_t)i * D + d];
                g.pos[idx * D + d] = x;
                // FP32 screening offset from the cell's corner (guard-band form)
                const double base = __dadd_rn(geo.inf[d], __dmul_rn((double)kd, g.c[d]));
                if (g.off) ((float*)g.off)[idx * D + d] = __double2float_rn(__dsub_rn(x, base));
            }
            if ((D == 2 || D == 3) && g.bocc) atomicOr((unsigned long long*)g.bocc + bidx, 1ull << bbit);
            if (D == 3 && g.bnew) atomicOr(g.bnew + bidx, 1ull << bbit);
            // a one-radius grid without per-cell radius or phase arrays (batched instances) skips them
            if (g.rad) g.rad[idx] = c.rad[i];
            if (g.radf) ((float*)g.radf)[idx] = __double2float_rn(c.rad[i]);
            if (g.phase) g.phase[idx] = c.phase[i];
        }
    }
    return acc;
}

__global__ void k_commit(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    const bool acc = t < nalive && commit_body(g, geo, c, c.alive[t]);
    const uint32_t mask = __ballot_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.counters[1], (uint32_t)__popc(mask));
}

// ------------------------------------------------------------------------------------------------
// refinement: remove_covered + subdivide_uncovered (list_of_voxels.ixx:30-100).  A parent is
// dropped when one sphere's exclusion ball (r_s + r_min) holds all its corners; otherwise each child
// is kept unless a sphere of the parent's prefilter list (dist^2(parent centre) < (r_s + r_min)^2,
// get_list_of_spheres :283-307) holds all the child's corners.  Output order: parents in list order,
// children in corner-table order (stable compaction).
// ------------------------------------------------------------------------------------------------
struct RefineParams {
    uint64_t V;
    const int64_t* vin;
    int64_t* vout;
    uint64_t vout_cap;
    double len[D];
    double nlen[D];
    double inf[D];
    double rmin;
    uint32_t* masks;
    uint32_t* warp_counts;
    const uint64_t* warp_offsets;
    uint32_t* err;
    uint32_t* survivors;
    unsigned long long* visits;
    unsigned long long* retests;
    float lenf[D];
    float nlenf[D];
    float rminf;
    uint64_t rho_frac[D];  // level-0 voxel length / cell edge: 64-bit fraction and integer part
    uint32_t rho_int[D];
    int32_t level;         // parent level (fixed-point shift)
    // sphere lists handed from voxels to their children (RefineArgs)
    int32_t record, inherit;
    float hdiagf;
    const uint32_t* lin;
    const uint8_t* nin;
    const uint32_t* parent;
    uint32_t* lout;
    uint8_t* nout;
    uint32_t* parent_out;
    uint64_t div0, div1;
};

// child index with bit d = offset along dimension d, for the child at position t of the corner table
__device__ __forceinline__ int child_bits(int t) {
    int j = 0;
#pragma unroll
    for (int d = 0; d < D; d++) j |= corner_bit(t, d) << d;
    return j;
}

// Squared corner terms of one sphere for the two child origins along each dimension: origin t = 0 is the
// parent's origin (2c nlen = c len exactly) and origin t = 1 is the parent's centre ((2c+1) nlen =
// (c + 0.5) len exactly), so delta_t = img - origin_t are the parent's own differences.  sq[d][t] =
// max over the child's two corners along d of the rounded square, and the child's rounded corner sum is
// accumulated over d in order, as the reference's corner loop does.
__device__ __forceinline__ uint32_t children_covered(const double* dl0, const double* dl1, const double* nlen,
                                                     uint64_t R2b) {
    constexpr int NC = CHILDREN <= 32 ? CHILDREN : 32;  // the wide variant serves D >= 6
    constexpr int DD = CHILDREN <= 32 ? D : 5;
    double acc[NC];
    {
        const double a0 = maxabs(dl0[0], __dsub_rn(nlen[0], dl0[0]));
        const double a1 = maxabs(dl1[0], __dsub_rn(nlen[0], dl1[0]));
        acc[0] = __dmul_rn(a0, a0);
        acc[1] = __dmul_rn(a1, a1);
    }
#pragma unroll
    for (int d = 1; d < DD; d++) {
        const double a0 = maxabs(dl0[d], __dsub_rn(nlen[d], dl0[d]));
        const double a1 = maxabs(dl1[d], __dsub_rn(nlen[d], dl1[d]));
        const double s0 = __dmul_rn(a0, a0), s1 = __dmul_rn(a1, a1);
#pragma unroll
        for (int j = (1 << d) - 1; j >= 0; j--) {
            acc[j | (1 << d)] = __dadd_rn(acc[j], s1);
            acc[j] = __dadd_rn(acc[j], s0);
        }
    }
    uint32_t cov = 0;  // bit t (corner-table order) set when the child is covered
#pragma unroll
    for (int t = 0; t < NC; t++) cov |= (dbits(acc[child_bits(t)]) <= R2b ? 1u : 0u) << t;
    return cov;
}

__device__ __forceinline__ void children_covered_wide(const double* dl0, const double* dl1, const double* nlen,
                                                      uint64_t R2b, uint32_t* cov) {
    // D >= 6: 2^D children, same arithmetic as children_covered, one child at a time
    for (int t = 0; t < CHILDREN; t++) {
        const int j = child_bits(t);
        double acc = 0.0;
        for (int d = 0; d < D; d++) {
            const double* dl = ((j >> d) & 1) ? dl1 : dl0;
            const double a = maxabs(dl[d], __dsub_rn(nlen[d], dl[d]));
            const double sq = __dmul_rn(a, a);
            acc = d == 0 ? sq : __dadd_rn(acc, sq);
        }
        if (dbits(acc) <= R2b) cov[t >> 5] |= 1u << (t & 31);
    }
}

constexpr uint64_t FAR_MARGIN_ULPS = 1ull << 13;  // relative 2^-39, far above the rounding of a distance

// Child mask of the parent voxel with coordinates cc (mask[] zeroed by the caller); returns true when
// remove_covered keeps the parent.
__device__ __forceinline__ bool refine_mask64_body(const Grid<D>& g, const Geo<D>& geo, const RefineParams& p,
                                                   const int64_t* cc, uint32_t* mask, uint32_t& visits) {
    bool survived = false;
    {
        double orig[D], centre[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            orig[d] = __dadd_rn(p.inf[d], __dmul_rn((double)cc[d], p.len[d]));
            // center(i) = origin + (coord + 0.5) * len (list_of_voxels.ixx:154-160)
            centre[d] = __dadd_rn(p.inf[d], __dmul_rn(__dadd_rn((double)cc[d], 0.5), p.len[d]));
        }
        int32_t k[D];
        float qo[D];  // the walk's query point: the voxel centre (every sphere that matters is within r_max + r_min of it)
        cell_of_q<D>(g, geo, centre, k, qo);
        double pre0[K_PRE][D], pre1[K_PRE][D];
        uint64_t preR2[K_PRE];
        int npre = 0;
        bool overflow = false;
        const float R2q = search_r2f(p.rminf, g.rmaxf);
        const bool covered = visit_placed<D>(g, geo, k, qo, R2q, [&](int64_t, const double* img, double rs) {
            visits++;
            const double R = __dadd_rn(rs, p.rmin);
            const uint64_t R2b = dbits(__dmul_rn(R, R));
            // distance to the parent's centre: the prefilter of get_list_of_spheres (:283-307)
            double dl1[D], s = 0.0;
#pragma unroll
            for (int d = 0; d < D; d++) {
                dl1[d] = __dsub_rn(img[d], centre[d]);
                const double sq = __dmul_rn(dl1[d], dl1[d]);
                s = d == 0 ? sq : __dadd_rn(s, sq);
            }
            const uint64_t sb = dbits(s);
            // A sphere that holds every corner holds the centre too: past R^2 (1 + 2^-39) it can neither
            // cover the parent nor enter the prefilter list.
            if (sb > R2b + FAR_MARGIN_ULPS) return false;
            // is_in_sphere over the parent's corners (remove_covered, :30-54)
            double dl0[D], m = 0.0;
#pragma unroll
            for (int d = 0; d < D; d++) {
                dl0[d] = __dsub_rn(img[d], orig[d]);
                const double a = maxabs(dl0[d], __dsub_rn(p.len[d], dl0[d]));
                const double sq = __dmul_rn(a, a);
                m = d == 0 ? sq : __dadd_rn(m, sq);
            }
            if (dbits(m) <= R2b) return true;  // the parent is covered
            if (sb < R2b) {
                if (npre < K_PRE) {
#pragma unroll
                    for (int d = 0; d < D; d++) {
                        pre0[npre][d] = dl0[d];
                        pre1[npre][d] = dl1[d];
                    }
                    preR2[npre] = R2b;
                    npre++;
                } else {
                    overflow = true;
                }
            }
            return false;
        });
        if (!covered) {
            survived = true;
            uint32_t cov[MASK_WORDS];
#pragma unroll
            for (int w = 0; w < MASK_WORDS; w++) cov[w] = 0;
            for (int s = 0; s < npre; s++) {
                if constexpr (CHILDREN <= 32) cov[0] |= children_covered(pre0[s], pre1[s], p.nlen, preR2[s]);
                else children_covered_wide(pre0[s], pre1[s], p.nlen, preR2[s], cov);
            }
            if (overflow) {
                atomicOr(p.err, (uint32_t)ERR_PREFILTER_OVERFLOW);
                // the list was full: test every prefilter sphere again, straight from the grid
                cov[0] = 0;
                for (int w = 1; w < MASK_WORDS; w++) cov[w] = 0;
                visit_placed<D>(g, geo, k, qo, R2q, [&](int64_t, const double* img, double rs) {
                    const double R = __dadd_rn(rs, p.rmin);
                    const uint64_t R2b = dbits(__dmul_rn(R, R));
                    double dl0[D], dl1[D], s = 0.0;
#pragma unroll
                    for (int d = 0; d < D; d++) {
                        dl1[d] = __dsub_rn(img[d], centre[d]);
                        const double sq = __dmul_rn(dl1[d], dl1[d]);
                        s = d == 0 ? sq : __dadd_rn(s, sq);
                        dl0[d] = __dsub_rn(img[d], orig[d]);
                    }
                    if (!(dbits(s) < R2b)) return false;
                    if constexpr (CHILDREN <= 32) cov[0] |= children_covered(dl0, dl1, p.nlen, R2b);
                    else children_covered_wide(dl0, dl1, p.nlen, R2b, cov);
                    return false;
                });
            }
#pragma unroll
            for (int w = 0; w < MASK_WORDS; w++) {
                const int bits_here = CHILDREN - 32 * w < 32 ? CHILDREN - 32 * w : 32;
                const uint32_t all = bits_here >= 32 ? 0xffffffffu : ((1u << bits_here) - 1u);
                mask[w] = ~cov[w] & all;
            }
        }
    }
    return survived;
}

__global__ void __launch_bounds__(REFINE_BLOCK) k_refine_mask(Grid<D> g, Geo<D> geo, RefineParams p) {
    const uint64_t v = (uint64_t)blockIdx.x * REFINE_BLOCK + threadIdx.x;
    uint32_t mask[MASK_WORDS];
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) mask[w] = 0;
    bool survived = false;
    uint32_t visits = 0;
    if (v < p.V) {
        int64_t cc[D];
#pragma unroll
        for (int d = 0; d < D; d++) cc[d] = p.vin[v * D + d];
        survived = refine_mask64_body(g, geo, p, cc, mask, visits);
#pragma unroll
        for (int w = 0; w < MASK_WORDS; w++) p.masks[v * MASK_WORDS + w] = mask[w];
    }
    // per-warp child counts (no block barrier: warps that finish early leave)
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) cnt += __popc(mask[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    const uint32_t alive = __ballot_sync(0xffffffffu, survived);
    uint32_t wv = visits;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wv += __shfl_xor_sync(0xffffffffu, wv, o);
    if ((threadIdx.x & 31) == 0) {
        const uint64_t warp = v >> 5;
        if (warp * 32 < p.V) p.warp_counts[warp] = cnt;
        if (alive) atomicAdd(p.survivors, (uint32_t)__popc(alive));
        if (wv) atomicAdd(p.visits, (unsigned long long)wv);
    }
}

// FP32 form of k_refine_mask: the same decisions, screened in FP32 against the guard band.  Per voxel the
// origin, centre and their offsets from the centre's cell corner are computed in FP64 (O(D) work);
// each (voxel, sphere) test is FP32 unless it falls inside the guard band, where it is redone in FP64
// exactly as the FP64 kernel does.
// The voxel centre in cell edges, y = (cc + 1/2) len / c, in fixed point (fixed_cell): its integer part is the
// cell k, its fraction the centre's offset relc from the cell's corner; relo is the voxel origin's offset.
// Integer instructions only; the FP64 pipe of this GPU runs at 1/64 of the FP32 rate.  The error (below 2^-31
// cell edges) is far inside the guard band, and only the screen uses these values.
__device__ __forceinline__ void voxel_query32(const Grid<D>& g, const RefineParams& p, const int64_t* cc, int32_t* k,
                                              float* relc, float* relo) {
#pragma unroll
    for (int d = 0; d < D; d++) {
        int64_t kd;
        uint32_t fb;
        fixed_cell((uint64_t)cc[d], 1ull << 52, p.rho_int[d], p.rho_frac[d], p.level, kd, fb);
        if (kd >= g.n[d]) kd -= g.n[d];  // the top face rounds onto the periodic image of cell 0
        k[d] = (int32_t)(kd < g.n[d] ? kd : g.n[d] - 1);
        relc[d] = __fmul_rn(__fmul_rn(u32_to_float(fb), 0x1p-32f), g.cf[d]);
        relo[d] = __fsub_rn(relc[d], __fmul_rn(0.5f, p.lenf[d]));
    }
}

// Exact FP64 quantities of the guard band for the voxel cc.  The empty volatile asm pins them inside the
// guard-band branches: loop-invariant, they would otherwise be hoisted onto the common path, where FP64
// instructions cost 64 FP32 ones on this GPU.
struct Exact64 {
    const Grid<D>& g;
    const Geo<D>& geo;
    const RefineParams& p;
    const int64_t* cc;
    // the voxel's origin and centre (list_of_voxels.ixx:154-160)
    __device__ __forceinline__ void corners(double* orig, double* centre) const {
#pragma unroll
        for (int d = 0; d < D; d++) {
            int64_t cv = cc[d];
            asm volatile("" : "+l"(cv));
            orig[d] = __dadd_rn(p.inf[d], __dmul_rn((double)cv, p.len[d]));
            centre[d] = __dadd_rn(p.inf[d], __dmul_rn(__dadd_rn((double)cv, 0.5), p.len[d]));
        }
    }
    // image of sphere idx (shift q) minus the voxel's origin and centre
    __device__ __forceinline__ void deltas(int64_t idx, const int8_t* q, double* dl0, double* dl1) const {
        double pp[D], img[D], orig[D], centre[D];
#pragma unroll
        for (int d = 0; d < D; d++) pp[d] = g.pos[idx * D + d];
        image_of<D>(geo, pp, q, img);
        corners(orig, centre);
#pragma unroll
        for (int d = 0; d < D; d++) {
            dl0[d] = __dsub_rn(img[d], orig[d]);
            dl1[d] = __dsub_rn(img[d], centre[d]);
        }
    }
    // bits of (r_s + r_min)^2
    __device__ __forceinline__ uint64_t R2b(int64_t idx) const {
        double rs = g.mono ? g.rmono : g.rad[idx];
        asm volatile("" : "+d"(rs));
        const double R = __dadd_rn(rs, p.rmin);
        return dbits(__dmul_rn(R, R));
    }
};

enum : int { PAIR_NONE = 0, PAIR_COVERS = 1, PAIR_PRE = 2 };

// One (voxel, sphere) pair of the FP32 form: the sphere at cell offset o (offsets offs from its cell corner,
// radius rs) against the voxel's centre and corners.  Returns PAIR_COVERS when the sphere holds every corner
// (remove_covered, list_of_voxels.ixx:30-54), PAIR_PRE when it enters the prefilter list of the children
// (get_list_of_spheres, :283-307), PAIR_NONE otherwise; d0, d1 receive the FP32 model deltas from the
// voxel's origin and centre.  Decided in FP32 outside the guard band, in FP64 inside it (sphere idx, image
// shift q), exactly as the FP64 kernel decides.
template <class Locate>
__device__ __forceinline__ int pair32(const Grid<D>& g, const RefineParams& p, const Exact64& ex, const int32_t* o,
                                      const float* offs, float rs, const float* relc, const float* relo, float* d0,
                                      float* d1, Locate&& locate, uint32_t& rt) {
    const float R = __fadd_rn(rs, p.rminf);
    const float R2 = __fmul_rn(R, R);
    const float lo = __fsub_rn(R2, g.guard), hi = __fadd_rn(R2, g.guard);
    model_delta<D>(g.cf, o, offs, relc, d1);
    const float s1 = sumsq32<D>(d1);
    if (s1 > hi) return PAIR_NONE;  // far: covers nothing, not in the prefilter list
    model_delta<D>(g.cf, o, offs, relo, d0);
    float m = 0.f;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const float a = fmaxf(fabsf(d0[d]), fabsf(__fsub_rn(p.lenf[d], d0[d])));
        m = __fadd_rn(m, __fmul_rn(a, a));
    }
    if (m < lo) return PAIR_COVERS;
    bool in_pre = s1 < lo;
    if (m <= hi || (!in_pre && s1 <= hi)) {
        // guard band: redo this pair in FP64, as the FP64 kernel does
        rt++;
        int64_t idx;
        int8_t q[D];
        locate(idx, q);
        double dl0[D], dl1[D];
        ex.deltas(idx, q, dl0, dl1);
        const uint64_t R2b = ex.R2b(idx);
        double mm = 0.0, ss = 0.0;
#pragma unroll
        for (int d = 0; d < D; d++) {
            const double a = maxabs(dl0[d], __dsub_rn(p.len[d], dl0[d]));
            const double sq = __dmul_rn(a, a);
            mm = d == 0 ? sq : __dadd_rn(mm, sq);
            const double s2 = __dmul_rn(dl1[d], dl1[d]);
            ss = d == 0 ? s2 : __dadd_rn(ss, s2);
        }
        if (dbits(mm) <= R2b) return PAIR_COVERS;
        in_pre = dbits(ss) < R2b;
    }
    return in_pre ? PAIR_PRE : PAIR_NONE;
}

// Children of one prefilter sphere (FP32 deltas d0, d1 from the parent's origin and centre, radius rs): the
// bits of the children it covers.  Any child inside the guard band -> this sphere in FP64 (sphere idx,
// image shift q), as children_covered.
template <class Locate>
__device__ __forceinline__ void children32(const Grid<D>& g, const RefineParams& p, const Exact64& ex,
                                           const float* d0, const float* d1, float rs, Locate&& locate,
                                           uint32_t* c32, uint32_t& rt) {
    const float R = __fadd_rn(rs, p.rminf);
    const float R2 = __fmul_rn(R, R);
    const float lo = __fsub_rn(R2, g.guard), hi = __fadd_rn(R2, g.guard);
    bool band = false;
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) c32[w] = 0;
    if constexpr (CHILDREN <= 16) {
        // the children's corner sums as a tree over the dimensions, in dimension order (the association of the
        // per-child loop below, bit for bit): two squared terms per dimension instead of one per child (D <= 4:
        // the 2^D partial sums stay in registers)
        float acc[CHILDREN];
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float a0 = fmaxf(fabsf(d0[d]), fabsf(__fsub_rn(p.nlenf[d], d0[d])));
            const float a1 = fmaxf(fabsf(d1[d]), fabsf(__fsub_rn(p.nlenf[d], d1[d])));
            const float s0 = __fmul_rn(a0, a0), s1 = __fmul_rn(a1, a1);
            if (d == 0) {
                acc[0] = __fadd_rn(0.f, s0);
                acc[1] = __fadd_rn(0.f, s1);
            } else {
#pragma unroll
                for (int j = (1 << d) - 1; j >= 0; j--) {
                    acc[j | (1 << d)] = __fadd_rn(acc[j], s1);
                    acc[j] = __fadd_rn(acc[j], s0);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < CHILDREN; t++) {
            const float x = acc[child_bits(t)];
            if (x < lo) c32[0] |= 1u << t;
            else if (x <= hi) band = true;
        }
    } else {
        for (int t = 0; t < CHILDREN; t++) {
            const int jb = child_bits(t);
            float acc = 0.f;
#pragma unroll
            for (int d = 0; d < D; d++) {
                const float dd = ((jb >> d) & 1) ? d1[d] : d0[d];
                const float a = fmaxf(fabsf(dd), fabsf(__fsub_rn(p.nlenf[d], dd)));
                acc = __fadd_rn(acc, __fmul_rn(a, a));
            }
            if (acc < lo) c32[t >> 5] |= 1u << (t & 31);
            else if (acc <= hi) band = true;
        }
    }
    if (band) {
        rt++;
        int64_t idx;
        int8_t q[D];
        locate(idx, q);
        double dl0[D], dl1[D];
        ex.deltas(idx, q, dl0, dl1);
        const uint64_t R2b = ex.R2b(idx);
        if constexpr (CHILDREN <= 32) c32[0] = children_covered(dl0, dl1, p.nlen, R2b);
        else {
#pragma unroll
            for (int w = 0; w < MASK_WORDS; w++) c32[w] = 0;
            children_covered_wide(dl0, dl1, p.nlen, R2b, c32);
        }
    }
}

__device__ __forceinline__ bool refine_mask32_body(const Grid<D>& g, const Geo<D>& geo, const RefineParams& p,
                                                   const int64_t* cc, uint32_t* mask, uint32_t& visits, uint32_t& rt) {
    bool survived = false;
    {
        float relo[D], relc[D];
        int32_t k[D];
        voxel_query32(g, p, cc, k, relc, relo);
        const Exact64 ex{g, geo, p, cc};
        float pre0[K_PRE][D], pre1[K_PRE][D], prers[K_PRE];
        int64_t preidx[K_PRE];
        uint32_t preq[K_PRE];  // 2 bits per dimension: image shift + 1
        int npre = 0;
        bool overflow = false;
        const float R2q = search_r2f(p.rminf, g.rmaxf);
        const bool covered = visit_placed_fo<D>(g, k, relc, R2q, [&](int64_t idx, const int32_t* o, const int8_t* q) {
            visits++;
            const float rs = g.mono ? g.rmonof : g.radf[idx];
            float d0[D], d1[D];
            const int r = pair32(g, p, ex, o, g.off + idx * D, rs, relc, relo, d0, d1,
                                 [&](int64_t& i2, int8_t* q2) {
                                     i2 = idx;
#pragma unroll
                                     for (int d = 0; d < D; d++) q2[d] = q[d];
                                 }, rt);
            if (r == PAIR_COVERS) return true;  // the parent is covered
            if (r == PAIR_PRE) {
                if (npre < K_PRE) {
#pragma unroll
                    for (int d = 0; d < D; d++) {
                        pre0[npre][d] = d0[d];
                        pre1[npre][d] = d1[d];
                    }
                    prers[npre] = rs;
                    preidx[npre] = idx;
                    uint32_t qq = 0;
#pragma unroll
                    for (int d = 0; d < D; d++) qq |= (uint32_t)(q[d] + 1) << (2 * d);
                    preq[npre] = qq;
                    npre++;
                } else {
                    overflow = true;
                }
            }
            return false;
        });
        if (!covered) {
            survived = true;
            uint32_t cov[MASK_WORDS];
#pragma unroll
            for (int w = 0; w < MASK_WORDS; w++) cov[w] = 0;
            for (int sidx = 0; sidx < npre; sidx++) {
                // children of this sphere in FP32; any child inside the guard band -> this sphere in FP64
                int8_t q[D];
#pragma unroll
                for (int d = 0; d < D; d++) q[d] = (int8_t)((preq[sidx] >> (2 * d)) & 3u) - 1;
                uint32_t c32[MASK_WORDS];
                children32(g, p, ex, pre0[sidx], pre1[sidx], prers[sidx],
                           [&](int64_t& i2, int8_t* q2) {
                               i2 = preidx[sidx];
#pragma unroll
                               for (int d = 0; d < D; d++) q2[d] = q[d];
                           }, c32, rt);
#pragma unroll
                for (int w = 0; w < MASK_WORDS; w++) cov[w] |= c32[w];
            }
            if (overflow) {
                atomicOr(p.err, (uint32_t)ERR_PREFILTER_OVERFLOW);
                // the list was full: every prefilter sphere again, in FP64, straight from the grid
#pragma unroll
                for (int w = 0; w < MASK_WORDS; w++) cov[w] = 0;
                double orig[D], centre[D];
                ex.corners(orig, centre);
                visit_placed<D>(g, geo, k, relc, R2q, [&](int64_t idx, const double* img, double rs) {
                    const double R = __dadd_rn(rs, p.rmin);
                    const uint64_t R2b = dbits(__dmul_rn(R, R));
                    double dl0[D], dl1[D], ss = 0.0;
#pragma unroll
                    for (int d = 0; d < D; d++) {
                        dl1[d] = __dsub_rn(img[d], centre[d]);
                        const double sq = __dmul_rn(dl1[d], dl1[d]);
                        ss = d == 0 ? sq : __dadd_rn(ss, sq);
                        dl0[d] = __dsub_rn(img[d], orig[d]);
                    }
                    if (!(dbits(ss) < R2b)) return false;
                    if constexpr (CHILDREN <= 32) cov[0] |= children_covered(dl0, dl1, p.nlen, R2b);
                    else children_covered_wide(dl0, dl1, p.nlen, R2b, cov);
                    return false;
                });
            }
#pragma unroll
            for (int w = 0; w < MASK_WORDS; w++) {
                const int bits_here = CHILDREN - 32 * w < 32 ? CHILDREN - 32 * w : 32;
                const uint32_t all = bits_here >= 32 ? 0xffffffffu : ((1u << bits_here) - 1u);
                mask[w] = ~cov[w] & all;
            }
        }
    }
    return survived;
}

__global__ void __launch_bounds__(REFINE_BLOCK) k_refine_mask32(Grid<D> g, Geo<D> geo, RefineParams p) {
    const uint64_t v = (uint64_t)blockIdx.x * REFINE_BLOCK + threadIdx.x;
    uint32_t mask[MASK_WORDS];
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) mask[w] = 0;
    bool survived = false;
    uint32_t visits = 0, rt = 0;
    if (v < p.V) {
        int64_t cc[D];
#pragma unroll
        for (int d = 0; d < D; d++) cc[d] = p.vin[v * D + d];
        survived = refine_mask32_body(g, geo, p, cc, mask, visits, rt);
#pragma unroll
        for (int w = 0; w < MASK_WORDS; w++) p.masks[v * MASK_WORDS + w] = mask[w];
    }
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) cnt += __popc(mask[w]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    const uint32_t alive = __ballot_sync(0xffffffffu, survived);
    uint32_t wv = visits, wr = rt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        wv += __shfl_xor_sync(0xffffffffu, wv, o);
        wr += __shfl_xor_sync(0xffffffffu, wr, o);
    }
    if ((threadIdx.x & 31) == 0) {
        const uint64_t warp = v >> 5;
        if (warp * 32 < p.V) p.warp_counts[warp] = cnt;
        if (alive) atomicAdd(p.survivors, (uint32_t)__popc(alive));
        if (wv) atomicAdd(p.visits, (unsigned long long)wv);
        if (wr) atomicAdd(p.retests, (unsigned long long)wr);
    }
}

// ------------------------------------------------------------------------------------------------
// Cooperative FP32 mask pass.  Groups of COOP_G consecutive voxels of the list (siblings, or neighbours in
// the block order of the level-0 list) gather the occupied cells around their common box of cells once, into
// shared memory, and every lane tests its own voxel against that list in step with the others: no per-lane
// stencil walk with its divergent row loops.  A group whose voxels lie too far apart (union wider than one
// occupancy window, more rows than COOP_ROWS_MAX or more than COOP_CAND spheres) takes the per-lane walk
// (refine_mask32_body).  The decisions are those of k_refine_mask32: the group's list holds every sphere
// within reach of each of its voxels' centres, the per-pair tests are the same functions (pair32,
// children32), and the results (covered, prefilter set, child masks) do not depend on the visiting order.
// ------------------------------------------------------------------------------------------------
constexpr int COOP_G = 8;
constexpr int COOP_CAND = 64;
constexpr int COOP_BLOCK = 128;
constexpr int COOP_ROWS_MAX = 1024;

// Padding (in 4-byte words) that brings a list of `words` words to `target` modulo 32 banks.
constexpr int list_pad(int words, int target) {
    return ((target - words % 32) % 32 + 32) % 32 == 0 ? 32 : ((target - words % 32) % 32 + 32) % 32;
}

// A group's sphere list in shared memory.  The groups of a warp read the same slot of their own lists in
// step: the padding puts consecutive lists BANK_STEP banks apart, free of bank conflicts.
template <int CAND, int BANK_STEP>
struct SphereList {
    float off[D][CAND];  // the sphere's offsets from its cell corner
    float rs[CAND];      // its radius
    int16_t t[D][CAND];  // its image's cell: base + t (unwrapped)
    float pad[list_pad(D * CAND + CAND + D * CAND / 2, BANK_STEP)];
};
using CoopList = SphereList<COOP_CAND, 8>;  // four 8-lane groups per warp
static_assert((sizeof(CoopList) / 4) % 32 == 8, "CoopList bank spacing");

// Row t[1..D-1] of the group's union: the wrapped linear base of its cells (times n_0) and the dimension-0
// range [t0lo, t0hi] within reach of the box [kmin, kmax] of the group's cells (false: the row is out of
// reach).  sqrt.approx and the reciprocal cell edge stand for the exact operations: the search radius
// carries a 1e-4 margin, far above their error.
__device__ __forceinline__ bool coop_row(const Grid<D>& g, const int32_t* t, const int32_t* kb, const int32_t* kmin,
                                         const int32_t* kmax, const int32_t* w, float R2q, int64_t& base,
                                         int32_t& t0lo, int32_t& t0hi) {
    float rest = 0.f;
#pragma unroll
    for (int d = 1; d < D; d++) {
        const int32_t u = kb[d] + t[d];
        const int32_t gap = u < kmin[d] ? kmin[d] - u - 1 : (u > kmax[d] ? u - kmax[d] - 1 : 0);
        const float gf = __fmul_rn(small_i2f(gap), g.cf[d]);
        rest = __fadd_rn(rest, __fmul_rn(gf, gf));
    }
    if (rest > R2q) return false;
    base = 0;
#pragma unroll
    for (int d = D - 1; d >= 1; d--) {
        int32_t kk = kb[d] + t[d];
        kk = kk < 0 ? kk + g.n[d] : (kk >= g.n[d] ? kk - g.n[d] : kk);
        base = base * g.n[d] + kk;
    }
    base *= g.n[0];
    const int32_t mx = 1 + small_floor(__fmul_rn(sqrt_approx(__fsub_rn(R2q, rest)), g.inv_c0f));
    const int32_t m0 = kmin[0] - kb[0];
    t0lo = max(0, m0 - mx);
    t0hi = min(w[0] - 1, m0 + (kmax[0] - kmin[0]) + mx);
    return t0lo <= t0hi;
}

// Occupancy bits of cells t0lo..t0hi of a row (at most 32 cells, wrapped along dimension 0 in up to two
// pieces): bit i = cell t0lo + i.
__device__ __forceinline__ uint32_t coop_row_bits(const Grid<D>& g, int64_t base, int32_t kb0, int32_t t0lo,
                                                  int32_t t0hi) {
    const int32_t n0 = g.n[0];
    uint32_t bits = 0;
    int32_t t = t0lo;
    while (t <= t0hi) {
        const int32_t u = kb0 + t;
        const int32_t x = u < 0 ? u + n0 : (u >= n0 ? u - n0 : u);
        // cells of this piece: up to the wrap point or the end of the range
        const int32_t piece_end = u < 0 ? min(t0hi, -1 - kb0) : (u >= n0 ? t0hi : min(t0hi, n0 - 1 - kb0));
        const int32_t len = piece_end - t + 1;
        bits |= occ_bits(g.occ, base + x, len) << (t - t0lo);
        t += len;
    }
    return bits;
}

// The voxel cc (cell k, offsets relc / relo) against a group's list (slots 0..total-1, cells base + t):
// remove_covered over the list, then the children of the prefilter spheres, as refine_mask32_body does
// over its walk.  Fills mask; returns true when the voxel survives.
template <class List>
__device__ __forceinline__ bool list_test(const Grid<D>& g, const Geo<D>& geo, const RefineParams& p, const List& L,
                                          uint32_t total, const int32_t* base, const int32_t* k, const float* relc,
                                          const float* relo, const int64_t* cc, uint32_t* mask, uint32_t& rt) {
    const Exact64 ex{g, geo, p, cc};
    // the sphere of slot j: linear index and image shift, for the guard band only
    auto sphere_of = [&](uint32_t j, int64_t& idx, int8_t* q) {
        idx = 0;
#pragma unroll
        for (int d = D - 1; d >= 0; d--) {
            const int32_t u = base[d] + (int32_t)L.t[d][j];
            q[d] = u < 0 ? -1 : (u >= g.n[d] ? 1 : 0);
            idx = idx * g.n[d] + (u - (int32_t)q[d] * g.n[d]);
        }
    };
    int32_t ob[D];  // cell offset of slot t = 0 from this voxel's cell
#pragma unroll
    for (int d = 0; d < D; d++) ob[d] = base[d] - k[d];
    uint64_t pre = 0;
    for (uint32_t j = 0; j < total; j++) {
        int32_t o[D];
        float offs[D], d0[D], d1[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            o[d] = ob[d] + (int32_t)L.t[d][j];
            offs[d] = L.off[d][j];
        }
        const int r = pair32(g, p, ex, o, offs, L.rs[j], relc, relo, d0, d1,
                             [&](int64_t& idx, int8_t* q) { sphere_of(j, idx, q); }, rt);
        if (r == PAIR_COVERS) return false;
        if (r == PAIR_PRE) pre |= 1ull << j;
    }
    uint32_t cov[MASK_WORDS];
#pragma unroll
    for (int w2 = 0; w2 < MASK_WORDS; w2++) cov[w2] = 0;
    while (pre) {
        const uint32_t j = (uint32_t)(__ffsll((long long)pre) - 1);
        pre &= pre - 1;
        int32_t o[D];
        float offs[D], d0[D], d1[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            o[d] = ob[d] + (int32_t)L.t[d][j];
            offs[d] = L.off[d][j];
        }
        model_delta<D>(g.cf, o, offs, relc, d1);
        model_delta<D>(g.cf, o, offs, relo, d0);
        uint32_t c32[MASK_WORDS];
        children32(g, p, ex, d0, d1, L.rs[j], [&](int64_t& idx, int8_t* q) { sphere_of(j, idx, q); }, c32, rt);
#pragma unroll
        for (int w2 = 0; w2 < MASK_WORDS; w2++) cov[w2] |= c32[w2];
    }
#pragma unroll
    for (int w2 = 0; w2 < MASK_WORDS; w2++) {
        const int bits_here = CHILDREN - 32 * w2 < 32 ? CHILDREN - 32 * w2 : 32;
        const uint32_t all = bits_here >= 32 ? 0xffffffffu : ((1u << bits_here) - 1u);
        mask[w2] = ~cov[w2] & all;
    }
    return true;
}

// Writes the voxel's child mask and the warp's child count, survivors, visits and retests (all lanes).
__device__ __forceinline__ void mask_epilogue(const RefineParams& p, uint64_t v, bool active, const uint32_t* mask,
                                              bool survived, uint32_t visits, uint32_t rt) {
    if (active) {
#pragma unroll
        for (int w2 = 0; w2 < MASK_WORDS; w2++) p.masks[v * MASK_WORDS + w2] = mask[w2];
    }
    uint32_t cntc = 0;
#pragma unroll
    for (int w2 = 0; w2 < MASK_WORDS; w2++) cntc += __popc(mask[w2]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cntc += __shfl_xor_sync(0xffffffffu, cntc, o);
    const uint32_t alive = __ballot_sync(0xffffffffu, survived);
    uint32_t wv = visits, wr = rt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        wv += __shfl_xor_sync(0xffffffffu, wv, o);
        wr += __shfl_xor_sync(0xffffffffu, wr, o);
    }
    if ((threadIdx.x & 31) == 0) {
        const uint64_t warp = v >> 5;
        if (warp * 32 < p.V) p.warp_counts[warp] = cntc;
        if (alive) atomicAdd(p.survivors, (uint32_t)__popc(alive));
        if (wv) atomicAdd(p.visits, (unsigned long long)wv);
        if (wr) atomicAdd(p.retests, (unsigned long long)wr);
    }
}

__global__ void __launch_bounds__(COOP_BLOCK) k_refine_mask32c(Grid<D> g, Geo<D> geo, RefineParams p) {
    __shared__ CoopList lists[COOP_BLOCK / COOP_G];
    const uint64_t v = (uint64_t)blockIdx.x * COOP_BLOCK + threadIdx.x;
    const int gl = threadIdx.x & (COOP_G - 1);
    CoopList& L = lists[threadIdx.x / COOP_G];
    const bool active = v < p.V;
    int64_t cc[D];
    int32_t k[D];
    float relc[D], relo[D];
#pragma unroll
    for (int d = 0; d < D; d++) {
        cc[d] = active ? p.vin[v * D + d] : 0;
        k[d] = 0;
        relc[d] = relo[d] = 0.f;
    }
    if (active) voxel_query32(g, p, cc, k, relc, relo);
    // the group's box of cells and its union of reach
    const float R2q = search_r2f(p.rminf, g.rmaxf);
    const float sq = __fsqrt_rn(R2q);
    int32_t kmin[D], kmax[D], kb[D], w[D];
    bool ok = true;
    int64_t rows = 1;
#pragma unroll
    for (int d = 0; d < D; d++) {
        int32_t lo = active ? k[d] : 0x7fffffff, hi = active ? k[d] : -1;
#pragma unroll
        for (int o = 1; o < COOP_G; o <<= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        kmin[d] = lo;
        kmax[d] = hi;
        const int32_t m = 1 + (int32_t)floorf(__fdiv_rn(sq, g.cf[d]));
        ok = ok && hi >= 0 && (int64_t)(hi - lo) + 1 + 2 * (int64_t)m <= (int64_t)g.n[d];
        w[d] = ok ? hi - lo + 1 + 2 * m : 1;
        kb[d] = lo - m;
        if (d >= 1 && rows <= COOP_ROWS_MAX) rows *= w[d];  // saturates above the limit
    }
    ok = ok && w[0] <= 32 && rows <= COOP_ROWS_MAX;
    // One pass over the union's rows, COOP_G rows per step (lane gl takes row step * COOP_G + gl, its
    // coordinates t[1..D-1] advanced by COOP_G in mixed radix w, dimension 1 fastest): occupied cells ->
    // the group's list, in row order, slots from a scan within the group.  Past COOP_CAND the group only
    // counts, and falls back to the per-lane walk.
    const uint32_t gmask = 0xffu << (threadIdx.x & 31 & ~(COOP_G - 1));
    uint32_t total = 0;
    if (ok) {
        int32_t t[D];
        t[0] = 0;
        {
            int32_t r = gl;
#pragma unroll
            for (int d = 1; d < D; d++) {
                int32_t q = 0;
                while (r >= w[d]) {
                    r -= w[d];
                    q++;
                }
                t[d] = r;
                r = q;
            }
        }
        const int steps = ((int)rows + COOP_G - 1) / COOP_G;
        for (int st = 0; st < steps; st++) {
            const bool has_row = st * COOP_G + gl < (int)rows;
            int64_t base = 0;
            int32_t t0lo = 0, t0hi = -1;
            uint32_t bits = 0;
            if (has_row && coop_row(g, t, kb, kmin, kmax, w, R2q, base, t0lo, t0hi))
                bits = coop_row_bits(g, base, kb[0], t0lo, t0hi);
            const uint32_t c = __popc(bits);
            uint32_t incl = c;
#pragma unroll
            for (int o = 1; o < COOP_G; o <<= 1) {
                const uint32_t y = __shfl_up_sync(gmask, incl, o, COOP_G);
                if (gl >= o) incl += y;
            }
            uint32_t slot = total + incl - c;
            total += __shfl_sync(gmask, incl, COOP_G - 1, COOP_G);
            while (bits) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                if (slot < COOP_CAND) {
                    const int32_t t0 = t0lo + j;
                    const int32_t u = kb[0] + t0;
                    const int64_t idx = base + (u < 0 ? u + g.n[0] : (u >= g.n[0] ? u - g.n[0] : u));
#pragma unroll
                    for (int d = 0; d < D; d++) L.off[d][slot] = g.off[idx * D + d];
                    L.rs[slot] = g.mono ? g.rmonof : g.radf[idx];
                    L.t[0][slot] = (int16_t)t0;
#pragma unroll
                    for (int d = 1; d < D; d++) L.t[d][slot] = (int16_t)t[d];
                }
                slot++;
            }
            // next row of this lane: t[1..] + COOP_G in mixed radix
            if (D > 1) {
                t[1] += COOP_G;
#pragma unroll
                for (int d = 1; d < D - 1; d++) {
                    while (t[d] >= w[d]) {
                        t[d] -= w[d];
                        t[d + 1]++;
                    }
                }
            }
        }
    }
    ok = ok && total <= COOP_CAND;
    __syncwarp();
    uint32_t mask[MASK_WORDS];
#pragma unroll
    for (int w2 = 0; w2 < MASK_WORDS; w2++) mask[w2] = 0;
    bool survived = false;
    uint32_t visits = 0, rt = 0;
    if (ok && active) {
        if (gl == 0) visits = total;
        survived = list_test(g, geo, p, L, total, kb, k, relc, relo, cc, mask, rt);
    } else if (active) {
        survived = refine_mask32_body(g, geo, p, cc, mask, visits, rt);
    }
    mask_epilogue(p, v, active, mask, survived, visits, rt);
}

// ------------------------------------------------------------------------------------------------
// Warp-queue FP32 mask pass (3D grids with a brick map, levels >= 1).  In the per-lane walk each lane loops
// over its own occupied cells and its own prefilter spheres, loops of very different lengths: 10 of 32 lanes
// were active per instruction.  Here each lane puts its (voxel, occupied cell) pairs of 8 brick slots into a
// queue in shared memory, and the 32 lanes of the warp test the queued pairs together (pair32): coverage as a
// bit per voxel, prefilter spheres into a list per voxel.  The children of the uncovered voxels' prefilter
// spheres are tested the same way (children32), the child masks ORed per voxel.  The set of pairs each voxel
// gets is the set its own brick walk visits, and covering, the prefilter set and the child masks do not depend
// on the order of the tests: the decisions are those of k_refine_mask32.  A voxel whose neighbourhood wraps
// around the box, spans 3 bricks in a dimension, or has more than Q_PRE prefilter spheres takes the per-lane
// walk.
// ------------------------------------------------------------------------------------------------
constexpr int Q_WARPS = 4;
constexpr int Q_BLOCK = 32 * Q_WARPS;
constexpr int Q_CAP = 160;  // queued (voxel, cell) pairs per warp
constexpr int Q_PRE = 16;   // prefilter spheres kept per voxel
constexpr int Q_TOUCH = 8;  // recording passes: spheres kept per voxel that reach into it but are not prefilter
constexpr int QD2 = D > 2 ? 2 : 0;  // the third dimension's index (this kernel runs for D = 3 only)

template <bool LISTS>
struct WarpQueue {
    float relc[D][32], relo[D][32];
    // one queued pair per word: cell index (bits 0-31), cell offsets + 128 (8 bits each, from bit 32), owner
    // lane (bits 56-63)
    unsigned long long q[Q_CAP];
    uint32_t pcell[32][Q_PRE];
    int8_t po[32][Q_PRE][D];
    uint32_t tcell[LISTS ? 32 : 1][Q_TOUCH];  // recording passes only
    uint32_t ntouch[32];
    uint32_t npre[32];
    uint32_t pref[32];  // inclusive prefix of the children phase's per-lane counts
    uint32_t cov[32];
    uint32_t covered;   // bit per lane: voxel covered
    uint32_t over;      // bit per lane: prefilter list overflow
};

// Whether the sphere at cell offset o (offsets offs, radius rs) reaches into the voxel with origin offset relo:
// the squared distance from its centre to the voxel's nearest point below (r_s + r_min)^2, screened in FP32 with
// twice the guard band to spare (a sphere it keeps in error only costs a test).
__device__ __forceinline__ bool reaches32(const Grid<D>& g, const RefineParams& p, const int32_t* o,
                                          const float* offs, float rs, const float* relo) {
    float d0[D];
    model_delta<D>(g.cf, o, offs, relo, d0);
    const float R = __fadd_rn(rs, p.rminf);
    const float hi = __fadd_rn(__fmul_rn(R, R), __fmul_rn(2.f, g.guard));
    float m = 0.f;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const float t = d0[d] < 0.f ? -d0[d] : fmaxf(__fsub_rn(d0[d], p.lenf[d]), 0.f);
        m = __fadd_rn(m, __fmul_rn(t, t));
    }
    return m <= hi;
}

// Coordinates of cell idx of a 3D grid: two divisions by multiplies with ceil(2^64 / n) (exact for idx < 2^32,
// n < 2^32, n >= 2).
__device__ __forceinline__ void cell_coords(const Grid<D>& g, const RefineParams& p, uint32_t idx, int32_t* c) {
    const uint32_t t = (uint32_t)__umul64hi((unsigned long long)idx, p.div0);
    c[0] = (int32_t)(idx - t * (uint32_t)g.n[0]);
    const uint32_t z = (uint32_t)__umul64hi((unsigned long long)t, p.div1);
    c[1] = (int32_t)(t - z * (uint32_t)g.n[1]);
    c[QD2] = (int32_t)z;
}

// The warp-queue pass for the 32 voxels of a warp, all lanes together (every lane calls it, active or not,
// with the same grid): fills mask, returns true when this lane's voxel survives.  vin and vbase locate the
// warp's voxels (their coordinates are reloaded for the guard band's retests).
// Recording passes (p.record) reach r_s + r_min beyond the voxel's half diagonal and store, per surviving
// voxel, its prefilter spheres and the other spheres that reach into it (RefineArgs).  Inheriting passes
// (p.inherit) test a voxel against its parent's stored spheres and walk only the bricks of the spheres placed
// since (g.bnew): a sphere that reaches into a voxel reaches into its parent, so it is in the parent's list
// or new.  The decisions are those of the full walk.
template <bool LISTS>
__device__ __forceinline__ bool mask32q_warp(const Grid<D>& g, const Geo<D>& geo, const RefineParams& p,
                                             WarpQueue<LISTS>& Q, const int64_t* vin, uint64_t vbase, bool active,
                                             const int64_t* cc_in, uint32_t* mask, uint32_t& visits, uint32_t& rt) {
    const int lane = threadIdx.x & 31;
    int64_t cc[D];
    int32_t k[D], lo[D], hi[D];
    float relc[D], relo[D];
#pragma unroll
    for (int d = 0; d < D; d++) {
        cc[d] = cc_in[d];
        k[d] = lo[d] = hi[d] = 0;
        relc[d] = relo[d] = 0.f;
    }
    if (active) voxel_query32(g, p, cc, k, relc, relo);
    float R2q = search_r2f(p.rminf, g.rmaxf);
    if (LISTS && p.record) {
        const float sr = __fadd_ru(__fadd_ru(p.rminf, g.rmaxf), p.hdiagf);
        R2q = __fmul_ru(__fmul_ru(sr, sr), 1.0001f);
    }
    bool mine = active && brick_reach<D>(g, k, relc, R2q, lo, hi);
#pragma unroll
    for (int d = 0; d < D; d++) mine = mine && (hi[d] >> 2) - (lo[d] >> 2) <= 1;
    // an inherited list: the parent's spheres, then the bricks of the spheres placed since its pass
    uint32_t ninh = 0, lbase = 0;
    bool inh = false;
    if (LISTS && p.inherit && mine) {
        const uint32_t par = p.parent[vbase + lane];
        const uint8_t cnt = p.nin[par];
        if (cnt != LIST_NONE) {
            inh = true;
            ninh = cnt;
            lbase = par * (uint32_t)LIST_K;
        }
    }
    const unsigned long long* bmap = inh ? g.bnew : g.bocc;
#pragma unroll
    for (int d = 0; d < D; d++) {
        Q.relc[d][lane] = relc[d];
        Q.relo[d][lane] = relo[d];
    }
    Q.npre[lane] = 0;
    Q.ntouch[lane] = 0;
    Q.cov[lane] = 0;
    if (lane == 0) {
        Q.covered = 0;
        Q.over = 0;
    }
    __syncwarp();
    // the voxel of lane `own`, for the guard band's FP64 retests (loaded only there)
    int64_t occ[D];
    const Exact64 ex{g, geo, p, occ};
    auto test_pair = [&](int own, uint32_t idx, const int32_t* o) {
        float oc[D], oo[D], offs[D], d0[D], d1[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            oc[d] = Q.relc[d][own];
            oo[d] = Q.relo[d][own];
            offs[d] = g.off[(uint64_t)idx * D + d];
        }
        const float rs = g.mono ? g.rmonof : g.radf[idx];
        const int r = pair32(g, p, ex, o, offs, rs, oc, oo, d0, d1,
                             [&](int64_t& i2, int8_t* q2) {
                                 i2 = idx;
#pragma unroll
                                 for (int d = 0; d < D; d++) {
                                     q2[d] = 0;
                                     occ[d] = vin[(vbase + own) * D + d];
                                 }
                             }, rt);
        if (r == PAIR_COVERS) {
            atomicOr(&Q.covered, 1u << own);
        } else if (r == PAIR_PRE) {
            const uint32_t sl = atomicAdd(&Q.npre[own], 1u);
            if (sl < Q_PRE) {
                Q.pcell[own][sl] = idx;
#pragma unroll
                for (int d = 0; d < D; d++) Q.po[own][sl][d] = (int8_t)o[d];
            } else {
                atomicOr(&Q.over, 1u << own);
            }
        } else if (LISTS && p.record && reaches32(g, p, o, offs, rs, oo)) {
            // not a prefilter sphere of this voxel, but one of a descendant's, or its cover
            const uint32_t sl = atomicAdd(&Q.ntouch[own], 1u);
            if (sl < Q_TOUCH) Q.tcell[own][sl] = idx;
        }
    };
    uint32_t fill = 0;  // warp-uniform
    auto flush = [&]() {
        for (uint32_t e = lane; e < fill; e += 32) {
            const unsigned long long w = Q.q[e];
            const int own = (int)(w >> 56);
            if ((*(volatile uint32_t*)&Q.covered >> own) & 1u) continue;
            int32_t o[D];
#pragma unroll
            for (int d = 0; d < D; d++) o[d] = (int32_t)((w >> (32 + 8 * d)) & 0xffu) - 128;
            visits++;
            test_pair(own, (uint32_t)w, o);
        }
        __syncwarp();
        fill = 0;
    };
    // inherited pairs: each lane's parent list, one entry per lane per step
    if (LISTS && p.inherit) {
        uint32_t mx = ninh;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        for (uint32_t j = 0; j < mx; j++) {
            const bool has = j < ninh;
            const uint32_t bal = __ballot_sync(0xffffffffu, has);
            if (fill + 32 > Q_CAP) flush();
            if (has) {
                const uint32_t idx = p.lin[lbase + j];
                int32_t c[D];
                cell_coords(g, p, idx, c);
                const uint32_t offs = (uint32_t)(c[0] - k[0] + 128) | ((uint32_t)(c[1] - k[1] + 128) << 8) |
                                      ((uint32_t)(c[QD2] - k[QD2] + 128) << 16) | ((uint32_t)lane << 24);
                Q.q[fill + __popc(bal & ((1u << lane) - 1u))] = (unsigned long long)idx | ((unsigned long long)offs << 32);
            }
            fill += __popc(bal);
            __syncwarp();
        }
    }
    // visit phase: the (up to) 2 x 2 x 2 bricks of each voxel's range
    for (int sl = 0; sl < 8; sl++) {
        unsigned long long bits = 0;
        int32_t b[D];
        if (mine) {
            b[0] = (lo[0] >> 2) + (sl & 1);
            b[1] = (lo[1] >> 2) + ((sl >> 1) & 1);
            b[QD2] = (lo[QD2] >> 2) + (sl >> 2);
            if (b[0] <= (hi[0] >> 2) && b[1] <= (hi[1] >> 2) && b[QD2] <= (hi[QD2] >> 2)) {
                const uint32_t xm = brick_span<2>(lo[0], hi[0], b[0]);
                const uint32_t ym = brick_span<2>(lo[1], hi[1], b[1]);
                const uint32_t zm = brick_span<2>(lo[QD2], hi[QD2], b[QD2]);
                const unsigned long long mask = brick_mask3(xm, ym, zm);
                bits = __ldg(bmap + (b[0] + (int64_t)g.nb[0] * (b[1] + (int64_t)g.nb[1] * b[QD2]))) & mask;
                if ((Q.covered >> lane) & 1u) bits = 0;  // covered already: no more pairs
            }
        }
        const uint32_t c = __popcll(bits);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
        if (fill + tot > Q_CAP) flush();
        if (tot <= Q_CAP) {
            uint32_t pos = fill + incl - c;
            while (bits) {
                const int j = __ffsll((long long)bits) - 1;
                bits &= bits - 1;
                const int32_t c0 = (b[0] << 2) + (j & 3), c1 = (b[1] << 2) + ((j >> 2) & 3), c2 = (b[QD2] << 2) + (j >> 4);
                const uint32_t cell = (uint32_t)(c0 + g.n[0] * (c1 + g.n[1] * c2));
                const uint32_t offs = (uint32_t)(c0 - k[0] + 128) | ((uint32_t)(c1 - k[1] + 128) << 8) |
                                      ((uint32_t)(c2 - k[QD2] + 128) << 16) | ((uint32_t)lane << 24);
                Q.q[pos] = (unsigned long long)cell | ((unsigned long long)offs << 32);
                pos++;
            }
            fill += tot;
            __syncwarp();
        } else {
            // more pairs than the queue holds: this slot lane by lane
            while (bits) {
                const int j = __ffsll((long long)bits) - 1;
                bits &= bits - 1;
                const int32_t c0 = (b[0] << 2) + (j & 3), c1 = (b[1] << 2) + ((j >> 2) & 3), c2 = (b[QD2] << 2) + (j >> 4);
                int32_t o[D];
                o[0] = c0 - k[0];
                o[1] = c1 - k[1];
                o[QD2] = c2 - k[QD2];
                visits++;
                test_pair(lane, (uint32_t)(c0 + g.n[0] * (c1 + g.n[1] * c2)), o);
            }
            __syncwarp();
        }
    }
    flush();
    // children phase: the (voxel, prefilter sphere) pairs of the uncovered voxels, over the warp
    const uint32_t covered = Q.covered, over = Q.over;
    const bool live = mine && !((covered >> lane) & 1u) && !((over >> lane) & 1u);
    const uint32_t cnt = live ? min(Q.npre[lane], (uint32_t)Q_PRE) : 0u;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    Q.pref[lane] = incl;
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (uint32_t e = lane; e < total; e += 32) {
        int own = 0;  // the lane whose inclusive prefix first exceeds e
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
            if (Q.pref[own + step - 1] <= e) own += step;
        const uint32_t sl = e - (own ? Q.pref[own - 1] : 0u);
        const uint32_t idx = Q.pcell[own][sl];
        int32_t o[D];
        float oc[D], oo[D], offs[D], d0[D], d1[D];
#pragma unroll
        for (int d = 0; d < D; d++) {
            o[d] = Q.po[own][sl][d];
            oc[d] = Q.relc[d][own];
            oo[d] = Q.relo[d][own];
            offs[d] = g.off[(uint64_t)idx * D + d];
        }
        model_delta<D>(g.cf, o, offs, oc, d1);
        model_delta<D>(g.cf, o, offs, oo, d0);
        uint32_t c32[MASK_WORDS];
        children32(g, p, ex, d0, d1, g.mono ? g.rmonof : g.radf[idx],
                   [&](int64_t& i2, int8_t* q2) {
                       i2 = idx;
#pragma unroll
                       for (int d = 0; d < D; d++) {
                           q2[d] = 0;
                           occ[d] = vin[(vbase + own) * D + d];
                       }
                   }, c32, rt);
        atomicOr(&Q.cov[own], c32[0]);
    }
    __syncwarp();
    if (LISTS && p.record && active) {
        // this voxel's list for its children: its prefilter spheres and the others that reach into it
        const uint64_t v = vbase + lane;
        uint8_t n = LIST_NONE;
        if (live) {
            const uint32_t np = Q.npre[lane], nt = Q.ntouch[lane];
            if (nt <= (uint32_t)Q_TOUCH && np + nt <= (uint32_t)LIST_K) {
                for (uint32_t j = 0; j < np; j++) p.lout[v * LIST_K + j] = Q.pcell[lane][j];
                for (uint32_t j = 0; j < nt; j++) p.lout[v * LIST_K + np + j] = Q.tcell[lane][j];
                n = (uint8_t)(np + nt);
            }
        }
        p.nout[v] = n;
    }
#pragma unroll
    for (int w2 = 0; w2 < MASK_WORDS; w2++) mask[w2] = 0;
    bool survived = false;
    if (live) {
        survived = true;
        const uint32_t all = CHILDREN >= 32 ? 0xffffffffu : ((1u << CHILDREN) - 1u);
        mask[0] = ~Q.cov[lane] & all;
    } else if (active && !(mine && ((covered >> lane) & 1u))) {
        // outside the brick walk's reach, or a prefilter list overflow: the per-lane walk
        survived = refine_mask32_body(g, geo, p, cc, mask, visits, rt);
    }
    __syncwarp();
    return survived;
}

template <bool LISTS>
__global__ void __launch_bounds__(Q_BLOCK) k_refine_mask32q(Grid<D> g, Geo<D> geo, RefineParams p) {
    __shared__ WarpQueue<LISTS> wq[Q_WARPS];
    const uint64_t v = (uint64_t)blockIdx.x * Q_BLOCK + threadIdx.x;
    const bool active = v < p.V;
    int64_t cc[D];
#pragma unroll
    for (int d = 0; d < D; d++) cc[d] = active ? p.vin[v * D + d] : 0;
    uint32_t mask[MASK_WORDS], visits = 0, rt = 0;
    const bool survived = mask32q_warp<LISTS>(g, geo, p, wq[threadIdx.x >> 5], p.vin, v - (threadIdx.x & 31), active, cc,
                                       mask, visits, rt);
    mask_epilogue(p, v, active, mask, survived, visits, rt);
}


__global__ void __launch_bounds__(REFINE_BLOCK) k_refine_write(RefineParams p) {
    const uint64_t v = (uint64_t)blockIdx.x * REFINE_BLOCK + threadIdx.x;
    uint32_t mask[MASK_WORDS];
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) {
        mask[w] = v < p.V ? p.masks[v * MASK_WORDS + w] : 0u;
        cnt += __popc(mask[w]);
    }
    const int lane = threadIdx.x & 31;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (v >= p.V || cnt == 0) return;
    uint64_t o = p.warp_offsets[v >> 5] + (incl - cnt);
    if (o + cnt > p.vout_cap) {
        atomicOr(p.err, (uint32_t)ERR_WRITE_BOUNDS);
        return;
    }
    int64_t cc[D];
#pragma unroll
    for (int d = 0; d < D; d++) cc[d] = p.vin[v * D + d];
    // children in Morton order (bit d of j = offset along d): a 2x..x2 block, as the level-0 blocks
    for (int j = 0; j < CHILDREN; j++) {
        const int t = corner_of_child(j);
        if (!((mask[t >> 5] >> (t & 31)) & 1u)) continue;
#pragma unroll
        for (int d = 0; d < D; d++) p.vout[o * D + d] = 2 * cc[d] + ((j >> d) & 1);
        if (p.parent_out) p.parent_out[o] = (uint32_t)v;
        o++;
    }
}

// regrid: spheres put back into a rebuilt grid enter it as accepted candidates (k_commit); their cells
__global__ void k_locate(Grid<D> g, Geo<D> geo, CandArgs c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double x[D];
#pragma unroll
    for (int d = 0; d < D; d++) x[d] = c.pos[(uint64_t)i * D + d];
    int32_t k[D];
    cell_of<D>(g, geo, x, k);
    c.cell[i] = cell_index<D>(g, k);
    c.state[i] = ST_ACCEPTED;
    c.alive[i] = i;
}

// ------------------------------------------------------------------------------------------------
// validators (operator_check_cell.ixx:8-78, rsa_data_storage.ixx:216-243) and reductions
// ------------------------------------------------------------------------------------------------
__global__ void k_check(Grid<D> g, Geo<D> geo, unsigned long long* overlaps, unsigned long long* misplaced) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.ncells || !occupied(g.occ, idx)) return;
    double x[D];
#pragma unroll
    for (int d = 0; d < D; d++) x[d] = g.pos[idx * D + d];
    const double r = g.rad[idx];
    int32_t k[D];
    cell_of<D>(g, geo, x, k);
    if (cell_index<D>(g, k) != idx) atomicAdd(misplaced, 1ull);
    // stencil around the cell the sphere is stored in
    int32_t kc[D];
    int64_t rem = idx;
#pragma unroll
    for (int d = 0; d < D; d++) {
        kc[d] = (int32_t)(rem % g.n[d]);
        rem /= g.n[d];
    }
    unsigned long long cnt = 0;
    visit_placed<D>(g, geo, kc, nullptr, search_r2(r, g.rmax), [&](int64_t j, const double* img, double rs) {
        if (j > idx && collide64<D>(r, x, rs, img)) cnt++;
        return false;
    });
    if (cnt) atomicAdd(overlaps, cnt);
}

__global__ void k_volume_partials(Grid<D> g, double unit, double* partials) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < g.ncells;
         idx += (int64_t)gridDim.x * blockDim.x) {
        if (!occupied(g.occ, idx)) continue;
        const double r = g.rad[idx];
        // volumeSphere = mult * puissance<D>(R) (auxiliary/Geometry/Sphere.ixx:46-57)
        double pw;
        if (D == 2) pw = __dmul_rn(r, r);
        else if (D == 3) pw = __dmul_rn(r, __dmul_rn(r, r));
        else if (D == 4) { const double s = __dmul_rn(r, r); pw = __dmul_rn(s, s); }
        else if (D == 5) { const double s = __dmul_rn(r, r); pw = __dmul_rn(s, __dmul_rn(r, s)); }
        else if (D == 6) { const double s = __dmul_rn(r, __dmul_rn(r, r)); pw = __dmul_rn(s, s); }
        else { const double s = __dmul_rn(r, __dmul_rn(r, r)); const double t = __dmul_rn(__dmul_rn(r, r), __dmul_rn(r, r)); pw = __dmul_rn(s, t); }
        acc += __dmul_rn(unit, pw);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(OCC_BLOCK) k_extract_write(Grid<D> g, const uint64_t* block_offsets, double* pos,
                                                           double* rad, int32_t* phase) {
    const int64_t nwords = (g.ncells + 31) / 32;
    const int64_t w = (int64_t)blockIdx.x * OCC_BLOCK + threadIdx.x;
    const uint32_t bits = w < nwords ? g.occ[w] : 0u;
    const uint32_t local = block_exclusive_scan<OCC_BLOCK>((uint32_t)__popc(bits), nullptr);
    uint64_t o = block_offsets[blockIdx.x] + local;
    uint32_t b = bits;
    while (b) {
        const int j = __ffs(b) - 1;
        b &= b - 1;
        const int64_t idx = w * 32 + j;
        if (pos) {
#pragma unroll
            for (int d = 0; d < D; d++) pos[o * D + d] = g.pos[idx * D + d];
        }
        if (rad) rad[o] = g.rad[idx];
        if (phase) phase[o] = g.phase[idx];
        o++;
    }
}

// The same output as k_extract_write, each warp's spheres written as contiguous runs: the warp's occupied cells
// (its 32 words, in order) are handed out one per lane (owner lane by binary search over the warp's inclusive
// counts, the cell by the rank of its bit), then every array is stored lane after lane.  For outputs in pinned host
// memory, which the kernel writes across the chip-to-host link: whole lines instead of one short run per thread.
__global__ void __launch_bounds__(OCC_BLOCK) k_extract_direct(Grid<D> g, const uint64_t* block_offsets, double* pos,
                                                            double* rad, int32_t* phase) {
    constexpr uint32_t FULL = 0xffffffffu;
    const int64_t nwords = (g.ncells + 31) / 32;
    const int64_t w = (int64_t)blockIdx.x * OCC_BLOCK + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const uint32_t bits = w < nwords ? g.occ[w] : 0u;
    const uint32_t c = (uint32_t)__popc(bits);
    const uint32_t local = block_exclusive_scan<OCC_BLOCK>(c, nullptr);
    const uint64_t wbase = block_offsets[blockIdx.x] + __shfl_sync(FULL, local, 0);  // the warp's first output
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    for (uint32_t e0 = 0; e0 < total; e0 += 32) {
        const uint32_t e = e0 + lane;
        const uint32_t n = total - e0 < 32 ? total - e0 : 32;  // spheres in this step (warp-uniform)
        int own = 0;  // the lane whose inclusive count first exceeds e
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t v = __shfl_sync(FULL, incl, own + step - 1);
            if (v <= e) own += step;
        }
        own = own < 31 ? own : 31;
        const uint32_t ob = __shfl_sync(FULL, bits, own), oc = __shfl_sync(FULL, c, own);
        const uint32_t oi = __shfl_sync(FULL, incl, own);
        const uint32_t rank = e - (oi - oc);
        int64_t idx = 0;
        if (e < total) idx = ((int64_t)blockIdx.x * OCC_BLOCK + (threadIdx.x & ~31u) + own) * 32 + (__fns(ob, 0, (int)rank + 1));
        if (pos) {
            // n spheres x D coordinates, stored lane after lane
            for (uint32_t k = lane; k < ((n * D + 31u) & ~31u); k += 32) {
                const uint32_t sph = k / D, d = k - sph * D;
                const int64_t src = __shfl_sync(FULL, idx, (int)(sph < 32 ? sph : 31));
                if (k < n * D) pos[(wbase + e0) * D + k] = g.pos[src * D + d];
            }
        }
        if (e < total) {
            if (rad) rad[wbase + e] = g.rad[idx];
            if (phase) phase[wbase + e] = g.phase[idx];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// host launchers
// ------------------------------------------------------------------------------------------------
void op_vox_init(int64_t* vox, uint64_t V, const int64_t* nvox, cudaStream_t s) {
    NVox nv;
    for (int d = 0; d < D; d++) nv.n[d] = nvox[d];
    if (V == 0) return;
    k_vox_init<<<nblocks(V, 256), 256, 0, s>>>(vox, V, nv);
    count_launch();
}

void op_darts(const GridArgs& ga, const CandArgs& c, const DartArgs& a, cudaStream_t s) {
    DartParams p{};
    p.n = a.n;
    p.V = a.V;
    p.vox = a.vox;
    for (int d = 0; d < D; d++) {
        p.len[d] = a.len[d];
        p.inf[d] = ga.inf[d];
    }
    p.seed_lo = (uint32_t)a.seed;
    p.seed_hi = (uint32_t)(a.seed >> 32);
    p.round_lo = (uint32_t)a.round;
    p.round_hi = (uint32_t)(a.round >> 32);
    p.radius = a.radius;
    p.phase = a.phase;
    p.rand_radius = a.rand_radius;
    p.r_lo = a.r_lo;
    p.r_span = a.r_span;
    p.rtab = a.rtab;
    p.ntab = a.ntab;
    p.pos = c.pos;
    p.key = c.key;
    p.rad = c.rad;
    p.cphase = c.phase;
    p.state = c.state;
    p.vidx_out = a.vidx_out;
    p.perm = a.perm;
    if (a.n == 0) return;
    k_darts<<<nblocks(a.n, 256), 256, 0, s>>>(p);
    count_launch();
}

// pass 1 (histogram) when a.bin_off is null, else pass 2 (the permutation a.perm)
void op_dart_bins(const CandArgs& c, const DartArgs& a, cudaStream_t s) {
    DartParams p{};
    p.n = a.n;
    p.V = a.V;
    p.seed_lo = (uint32_t)a.seed;
    p.seed_hi = (uint32_t)(a.seed >> 32);
    p.round_lo = (uint32_t)a.round;
    p.round_hi = (uint32_t)(a.round >> 32);
    p.bin_hist = a.bin_hist;
    p.bin_off = a.bin_off;
    p.bin_shift = a.bin_shift;
    p.vbase = 0;
    p.perm = a.perm;
    p.err = c.counters + 2;
    if (a.n == 0 || !a.bin_hist) return;
    if (!a.bin_off) k_dart_bins<<<nblocks(a.n, 256), 256, 0, s>>>(p);
    else k_dart_perm<<<nblocks(a.n, 256), 256, 0, s>>>(p);
    count_launch();
}

void op_darts32(const GridArgs& ga, const CandArgs& c, const DartArgs& a, cudaStream_t s) {
    DartParams p{};
    p.n = a.n;
    p.V = a.V;
    p.vox = a.vox;
    for (int d = 0; d < D; d++) {
        p.len[d] = a.len[d];
        p.inf[d] = ga.inf[d];
        p.rho_frac[d] = a.rho_frac[d];
        p.rho_int[d] = a.rho_int[d];
        p.ncell[d] = ga.n[d];
        p.cf[d] = ga.cf[d];
    }
    p.seed_lo = (uint32_t)a.seed;
    p.seed_hi = (uint32_t)(a.seed >> 32);
    p.round_lo = (uint32_t)a.round;
    p.round_hi = (uint32_t)(a.round >> 32);
    p.radius = a.radius;
    p.phase = a.phase;
    p.rand_radius = a.rand_radius;
    p.r_lo = a.r_lo;
    p.r_span = a.r_span;
    p.rtab = a.rtab;
    p.ntab = a.ntab;
    p.pos = c.pos;
    p.key = c.key;
    p.rad = c.rad;
    p.cphase = c.phase;
    p.state = c.state;
    p.vidx_out = nullptr;
    p.kc = c.kc;
    p.off = c.off;
    p.cell = c.cell;
    p.level = a.level;
    p.perm = a.perm;
    if (a.n == 0) return;
    k_darts32<<<nblocks(a.n, 256), 256, 0, s>>>(p);
    count_launch();
}

void op_probe(const GridArgs& ga, const CandArgs& c, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32 && ga.mono) k_probe<true, true><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    else if (f32) k_probe<true><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    else k_probe<false><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    count_launch();
}

void op_collect(const GridArgs& ga, const CandArgs& c, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32) k_collect<true><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    else k_collect<false><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    count_launch();
}

void op_settle(const GridArgs& ga, const CandArgs& c, int it, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    // grid-stride over the alive list (its length is on the device): 8 blocks per SM at most
    const unsigned nb = nblocks(c.n, 256) < 152u * 8u ? nblocks(c.n, 256) : 152u * 8u;
    if (f32) k_settle<true><<<nb, 256, 0, s>>>(make_grid(ga), make_geo(ga), c, it);
    else k_settle<false><<<nb, 256, 0, s>>>(make_grid(ga), make_geo(ga), c, it);
    count_launch();
}

void op_gather_accepted(const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_gather_accepted<<<nblocks(c.n, 256), 256, 0, s>>>(c);
    count_launch();
}

void op_cut_accepted(const CandArgs& c, int use_pivot, double pivot, uint64_t key_cut, cudaStream_t s) {
    if (c.n == 0) return;
    k_cut_accepted<<<nblocks(c.n, 256), 256, 0, s>>>(c, use_pivot, pivot, key_cut);
    count_launch();
}

void op_pass_begin(const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_pass_begin<<<nblocks(c.n, 256), 256, 0, s>>>(c);
    count_launch();
}

void op_pass_step(const GridArgs& ga, const CandArgs& c, int it, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    const unsigned nb = nblocks(c.n, 256) < 152u * 8u ? nblocks(c.n, 256) : 152u * 8u;
    if (f32) k_pass_step<true><<<nb, 256, 0, s>>>(make_grid(ga), make_geo(ga), c, it);
    else k_pass_step<false><<<nb, 256, 0, s>>>(make_grid(ga), make_geo(ga), c, it);
    count_launch();
}

void op_pass_sources(const GridArgs& ga, const CandArgs& c, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32) k_pass_sources<true><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    else k_pass_sources<false><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    k_pass_mark<<<nblocks(c.n, 256), 256, 0, s>>>(c);
    count_launch(2);
}

void op_pass_push(const GridArgs& ga, const CandArgs& c, int from, uint32_t nf, int f32, cudaStream_t s) {
    if (nf == 0) return;
    if (f32) k_pass_push<true><<<nblocks(nf, 128), 128, 0, s>>>(make_grid(ga), make_geo(ga), c, from);
    else k_pass_push<false><<<nblocks(nf, 128), 128, 0, s>>>(make_grid(ga), make_geo(ga), c, from);
    count_launch();
}

void op_pass_gather(const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_pass_gather<<<nblocks(c.n, 256), 256, 0, s>>>(c);
    count_launch();
}

void op_pass_close(const CandArgs& c, int mode, double pivot, cudaStream_t s) {
    if (c.n == 0) return;
    k_pass_close<<<nblocks(c.n, 256), 256, 0, s>>>(c, mode, pivot);
    count_launch();
}

void op_pass_next(const GridArgs& ga, const CandArgs& c, int f32, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32) k_pass_next<true><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    else k_pass_next<false><<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    count_launch();
}

void op_commit(const GridArgs& ga, const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_commit<<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    count_launch();
}

RefineParams make_refine(const GridArgs& ga, const RefineArgs& a) {
    RefineParams p;
    p.V = a.V;
    p.vin = a.vin;
    p.vout = a.vout;
    p.vout_cap = a.vout_cap;
    for (int d = 0; d < D; d++) {
        p.len[d] = a.len[d];
        p.nlen[d] = a.nlen[d];
        p.inf[d] = ga.inf[d];
    }
    p.rmin = a.rmin;
    p.masks = a.masks;
    p.warp_counts = a.warp_counts;
    p.warp_offsets = a.warp_offsets;
    p.err = a.err;
    p.survivors = a.survivors;
    p.visits = a.visits;
    p.retests = a.retests;
    for (int d = 0; d < D; d++) {
        p.lenf[d] = (float)a.len[d];
        p.nlenf[d] = (float)a.nlen[d];
        p.rho_frac[d] = a.rho_frac[d];
        p.rho_int[d] = a.rho_int[d];
    }
    p.level = a.level;
    p.rminf = (float)a.rmin;
    p.record = a.record;
    p.inherit = a.inherit;
    p.hdiagf = a.hdiagf;
    p.lin = a.lin;
    p.nin = a.nin;
    p.parent = a.parent;
    p.lout = a.lout;
    p.nout = a.nout;
    p.parent_out = a.parent_out;
    p.div0 = a.div0;
    p.div1 = a.div1;
    return p;
}

void op_refine_mask(const GridArgs& ga, const RefineArgs& a, int f32, cudaStream_t s) {
    if (a.V == 0) return;
    // Level 0 (one voxel per cell, 2x2x2 blocks in the list): 8-lane groups over their box of cells.  Deeper
    // levels of 3D grids with a brick map: the warp queue of (voxel, cell) pairs.  Else the per-lane walk.
    if (f32 && a.level == 0) {
        k_refine_mask32c<<<nblocks(a.V, COOP_BLOCK), COOP_BLOCK, 0, s>>>(make_grid(ga), make_geo(ga), make_refine(ga, a));
    } else if (f32 && D == 3 && ga.bocc && ga.ncells < (1ll << 32)) {
        if (a.record)
            k_refine_mask32q<true><<<nblocks(a.V, Q_BLOCK), Q_BLOCK, 0, s>>>(make_grid(ga), make_geo(ga), make_refine(ga, a));
        else
            k_refine_mask32q<false><<<nblocks(a.V, Q_BLOCK), Q_BLOCK, 0, s>>>(make_grid(ga), make_geo(ga), make_refine(ga, a));
    } else if (f32) {
        k_refine_mask32<<<nblocks(a.V, REFINE_BLOCK), REFINE_BLOCK, 0, s>>>(make_grid(ga), make_geo(ga), make_refine(ga, a));
    }
    else
        k_refine_mask<<<nblocks(a.V, REFINE_BLOCK), REFINE_BLOCK, 0, s>>>(make_grid(ga), make_geo(ga), make_refine(ga, a));
    count_launch();
}

void op_refine_write(const RefineArgs& a, cudaStream_t s) {
    if (a.V == 0) return;
    GridArgs none{};  // the write pass needs no geometry
    k_refine_write<<<nblocks(a.V, REFINE_BLOCK), REFINE_BLOCK, 0, s>>>(make_refine(none, a));
    count_launch();
}

void op_locate(const GridArgs& ga, const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_locate<<<nblocks(c.n, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), c);
    count_launch();
}

void op_check(const GridArgs& ga, unsigned long long* overlaps, unsigned long long* misplaced, cudaStream_t s) {
    k_check<<<nblocks(ga.ncells, 256), 256, 0, s>>>(make_grid(ga), make_geo(ga), overlaps, misplaced);
    count_launch();
}

void op_volume_partials(const GridArgs& ga, double unit, double* partials, int nb, cudaStream_t s) {
    k_volume_partials<<<nb, 256, 0, s>>>(make_grid(ga), unit, partials);
    count_launch();
}

void op_extract_write(const GridArgs& ga, const uint64_t* block_offsets, double* pos, double* rad, int32_t* phase,
                      cudaStream_t s) {
    const int64_t nwords = (ga.ncells + 31) / 32;
    k_extract_write<<<nblocks(nwords, OCC_BLOCK), OCC_BLOCK, 0, s>>>(make_grid(ga), block_offsets, pos, rad, phase);
    count_launch();
}

void op_extract_direct(const GridArgs& ga, const uint64_t* block_offsets, double* pos, double* rad, int32_t* phase,
                       cudaStream_t s) {
    const int64_t nwords = (ga.ncells + 31) / 32;
    k_extract_direct<<<nblocks(nwords, OCC_BLOCK), OCC_BLOCK, 0, s>>>(make_grid(ga), block_offsets, pos, rad, phase);
    count_launch();
}

#include "kernels_batch.cuh"

const DimOps kOps = {
    D,
    op_vox_init,
    op_darts,
    op_darts32,
    op_dart_bins,
    op_probe,
    op_collect,
    op_settle,
    op_gather_accepted,
    op_cut_accepted,
    op_commit,
    op_refine_mask,
    op_refine_write,
    op_check,
    op_volume_partials,
    op_extract_write,
    op_locate,
    CHILDREN,
    MASK_WORDS,
    op_batch_table_bytes,
    op_batch_table_fill,
    op_b_vox_init,
    op_b_darts,
    op_b_dart_bins,
    op_b_probe,
    op_b_collect,
    op_b_settle,
    op_b_commit,
    op_b_refine_mask,
    op_b_refine_offsets,
    op_b_refine_write,
    op_b_results,
    op_pass_begin,
    op_pass_step,
    op_pass_gather,
    op_pass_close,
    op_pass_next,
    op_pass_sources,
    op_pass_push,
    op_extract_direct,
};

}  // namespace

#define RSA_CAT2(a, b) a##b
#define RSA_CAT(a, b) RSA_CAT2(a, b)
const DimOps* RSA_CAT(dim_ops_, RSA_DIM)() { return &kOps; }

}  // namespace rsagpu
