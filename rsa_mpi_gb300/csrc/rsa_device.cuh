// rsa_device.cuh -- device code of the GB300 sampler, templated on the space dimension D.
//
// Data layout in HBM (one sampler instance):
//   sphere grid  : cells of edge c_d = L_d / n_d with c * sqrt(D) < 2 r_min, so that a cell holds at
//                  most one accepted centre.  occ = 1 bit per cell (10 MB for 434^3 cells, L2
//                  resident); pos = D doubles per cell, rad = 1 double per cell, phase = int32 per
//                  cell (all indexed by the cell, so the cell index IS the sphere id).
//   voxel list   : AoS int64[V][D] integer coordinates at the current level, one length per level.
//   candidates   : SoA per round (pos, key, rad, phase, cell, state, next) + a per-cell list head.
//
// Every FP64 decision uses __dadd_rn / __dsub_rn / __dmul_rn in the operation order of the
// reference line it restates, so nothing is contracted into an FMA and every comparison rounds as
// the reference's does (is_there_collision operator_cells_and_data_storage.ixx:5-14,
// is_in_sphere list_of_voxels.ixx:225-238, get_list_of_spheres :283-307, pick_points :107-129).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rsagpu {

enum : uint8_t { ST_DEAD = 0, ST_UNDECIDED = 1, ST_ACCEPTED = 2, ST_REJECTED = 3 };

// error bits written by kernels
enum : uint32_t {
    ERR_DOUBLE_OCCUPANCY = 1u,   // two accepted centres in one cell
    ERR_BLOCKER_OVERFLOW = 2u,   // (informational) a candidate had more than NB lower colliders
    ERR_PREFILTER_OVERFLOW = 4u, // (informational) a parent voxel had more than K prefilter spheres
    ERR_WRITE_BOUNDS = 8u,       // a refinement output offset beyond the output buffer (write skipped)
    ERR_DART_SLOT = 16u,         // a dart found its bin of the binned order full (dart skipped)
};

constexpr int NB = 24;     // stored lower-priority colliders per candidate (more: rescan)
constexpr int NB_OVERFLOW = 255;
// a stored collider seen through the periodic boundary (candidate indices stay below 2^31)
constexpr uint32_t BLK_WRAP = 0x80000000u;

__host__ __device__ __forceinline__ int32_t blk_index(int32_t e) { return (int32_t)((uint32_t)e & ~BLK_WRAP); }
__host__ __device__ __forceinline__ bool blk_wrapped(int32_t e) { return ((uint32_t)e & BLK_WRAP) != 0; }

// image shift q of a stencil walk: the neighbour is seen through the periodic boundary
template <int D>
__device__ __forceinline__ bool wrapped(const int8_t* q) {
    bool w = false;
#pragma unroll
    for (int d = 0; d < D; d++) w |= q[d] != 0;
    return w;
}

// count-cap passes (find_solve_conflicts with the Undecided / Conflict / Skip tags of one pass): states of the
// candidates of the current pass next to ST_UNDECIDED (in the pass, not classified yet)
enum : uint8_t { ST_PASS_U = 4, ST_PASS_C = 5, ST_PASS_S = 6 };

template <int D>
struct Geo {
    double inf[D];
    double L[D];
};

template <int D>
struct Grid {
    int64_t ncells;
    int32_t n[D];
    double inv_c[D];
    uint32_t* occ;
    double* pos;
    double* rad;
    int32_t* phase;
    const int8_t* stencil;  // S offsets of D int8
    int S;
    // the same stencil as rows along dimension 0: row r = {xlo, xhi, o_1, ..., o_{D-1}} (D+1 int8)
    const int8_t* rows;
    int R;
    const float* rows_r2;  // per row: squared distance to its nearest cell along dimensions 1..D-1 (rows sorted by it)
    float c0f;             // cell edge along dimension 0
    float inv_c0f;         // its inverse
    double rmax;           // largest radius the grid holds
    float rmaxf;           // the same, rounded to float (search radii carry a margin far above that rounding)
    // FP32 screening representation of the placed centres (guard-band form): off = centre minus the
    // corner of its cell, rounded to float; radf = radius rounded to float
    const float* off;
    const float* radf;
    double c[D];    // cell edge
    float cf[D];    // cell edge rounded to float
    float guard;    // bound on |FP32 model - FP64 value| of any squared distance the kernels compare
    int mono;       // one radius for every sphere
    const unsigned long long* bocc;  // 2D / 3D: occupancy by bricks of 64 cells (8x8, 4x4x4), or null
    int32_t nb[D];                   // bricks per dimension
    float inv_cf[D];                 // inverse cell edges
    double rmono;
    float rmonof;
    unsigned long long* bnew;        // bricks of the spheres placed since the last mask pass, or null
};

// ---------------------------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3", SC'11)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = c.x * 0xD2511F53u, hi0 = __umulhi(c.x, 0xD2511F53u);
        const uint32_t lo1 = c.z * 0xCD9E8D57u, hi1 = __umulhi(c.z, 0xCD9E8D57u);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// ---------------------------------------------------------------------------------------------
// geometry, exact FP64
// ---------------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ bool collide64(double r1, const double* a, double r2, const double* b) {
    double dist2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const double dr = __dsub_rn(a[d], b[d]);
        dist2 = __dadd_rn(dist2, __dmul_rn(dr, dr));
    }
    const double rr = __dadd_rn(r1, r2);
    return dist2 < __dmul_rn(rr, rr);
}

// max over the 2^D corners {orig + t * len, t in {0,1}^D} of the reference's rounded corner distance
// sum_d (corner_d - delta_d)^2 with delta = img - orig.  Round-to-nearest addition is monotone in each
// operand, so the largest rounded sum is the rounded sum of the per-dimension largest terms: one
// evaluation equals the reference's 2^D-corner loop bit for bit.
template <int D>
__device__ __forceinline__ double maxcorner_dist2(const double* img, const double* orig, const double* len) {
    double dist2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const double delta = __dsub_rn(img[d], orig[d]);
        const double t0 = __dsub_rn(0.0, delta);
        const double t1 = __dsub_rn(len[d], delta);
        const double s0 = __dmul_rn(t0, t0), s1 = __dmul_rn(t1, t1);
        dist2 = __dadd_rn(dist2, s0 > s1 ? s0 : s1);
    }
    return dist2;
}

template <int D>
__device__ __forceinline__ double dist2_64(const double* a, const double* b) {
    double dist2 = 0.0;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const double t = __dsub_rn(a[d], b[d]);
        dist2 = __dadd_rn(dist2, __dmul_rn(t, t));
    }
    return dist2;
}

template <int D>
__device__ __forceinline__ void cell_of(const Grid<D>& g, const Geo<D>& geo, const double* x, int32_t* k) {
#pragma unroll
    for (int d = 0; d < D; d++) {
        int32_t kk = (int32_t)floor(__dmul_rn(__dsub_rn(x[d], geo.inf[d]), g.inv_c[d]));
        kk = kk < 0 ? 0 : (kk >= g.n[d] ? g.n[d] - 1 : kk);
        k[d] = kk;
    }
}

template <int D>
__device__ __forceinline__ int64_t cell_index(const Grid<D>& g, const int32_t* k) {
    int64_t idx = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; d--) idx = idx * g.n[d] + k[d];
    return idx;
}

// Wrapped stencil cell s around cell k: linear index and per-dimension image shift q in {-1,0,1}.
template <int D>
__device__ __forceinline__ int64_t stencil_cell(const Grid<D>& g, const int32_t* k, int s, int8_t* q) {
    int64_t idx = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; d--) {
        int32_t kk = k[d] + (int32_t)g.stencil[s * D + d];
        int8_t qq = 0;
        if (kk < 0) { kk += g.n[d]; qq = -1; }
        else if (kk >= g.n[d]) { kk -= g.n[d]; qq = 1; }
        q[d] = qq;
        idx = idx * g.n[d] + kk;
    }
    return idx;
}

// image of a stored centre: x + q L per wrapped dimension (the reference's ghost copy x + (+-L),
// rsa_ghost_area.ixx:22-30)
template <int D>
__device__ __forceinline__ void image_of(const Geo<D>& geo, const double* p, const int8_t* q, double* img) {
#pragma unroll
    for (int d = 0; d < D; d++) img[d] = q[d] == 0 ? p[d] : __dadd_rn(p[d], q[d] > 0 ? geo.L[d] : -geo.L[d]);
}

__device__ __forceinline__ bool occupied(const uint32_t* occ, int64_t idx) {
    return (__ldg(occ + (idx >> 5)) >> (idx & 31)) & 1u;
}

// len (<= 32) occupancy bits of consecutive cells starting at linear index lin; the bitmap carries one
// padding word so that the two-word window never reads past it.
__device__ __forceinline__ uint32_t occ_bits(const uint32_t* occ, int64_t lin, int len) {
    const int64_t w = lin >> 5;
    const int sh = (int)(lin & 31);
    const uint64_t win = ((uint64_t)__ldg(occ + w + 1) << 32) | (uint64_t)__ldg(occ + w);
    const uint32_t bits = (uint32_t)(win >> sh);
    return len >= 32 ? bits : (bits & ((1u << len) - 1u));
}

// Exact int <-> float conversions of small integers by FP32 adds of 1.5 * 2^23 (the float whose mantissa
// unit is 1): the FMA pipe runs them at the full FP32 rate, while this GPU executes the conversion
// instructions on its FP64 pipe, at 1/64 of that rate.
__device__ __forceinline__ float small_i2f(int32_t i) {  // |i| < 2^22
    return __fsub_rn(__int_as_float(0x4B400000 + i), 12582912.0f);
}
__device__ __forceinline__ int32_t small_floor(float x) {  // floor(x), |x| < 2^22
    return __float_as_int(__fadd_rd(x, 12582912.0f)) - 0x4B400000;
}
// __uint2float_rn without a conversion instruction: the two 16-bit halves are exact floats, and the one
// rounding of their sum is the rounding of x to nearest
__device__ __forceinline__ float u32_to_float(uint32_t x) {
    return __fadd_rn(__fmul_rn(small_i2f((int32_t)(x >> 16)), 65536.0f), small_i2f((int32_t)(x & 0xffffu)));
}

__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Walks the stencil row by row: for each row, the wrapped cell coordinates of dimensions 1..D-1 and up to
// three contiguous segments along dimension 0 (left wrap, inside, right wrap).  g(base, lo, hi, q, row) is
// called per segment [lo, hi] with the image shifts q; it returns true to stop.  With query offsets qo, only
// cells whose nearest point lies within sqrt(R2q) of the query point are walked: the query is cell k at offset
// qo from its corner (FP32), each row is cut by the point's distance to it along dimensions 1..D-1, and its
// dimension-0 range by the remaining distance.  R2q carries a 1e-4 margin, far above the float error of these
// bounds.  Without (qo null) the rows are cut by the distance from the query's whole cell: the lanes of a warp
// then walk the same cells in step, which the FP64 candidate kernels need (on this GPU a divergent FP64
// instruction costs 16 SM cycles whatever the number of lanes it serves).
template <int D, class G>
__device__ __forceinline__ bool walk_rows(const int32_t* n, const int8_t* rows, int R, const float* rows_r2,
                                          const float* cf, float inv_c0, float R2q, const int32_t* k, const float* qo,
                                          G&& g) {
    for (int r = 0; r < R; r++) {
        // rows in order of their nearest cell-to-cell distance: none after the first one beyond R2q
        if (rows_r2[r] > R2q) break;
        // the row's D + 1 bytes in one load where they make a whole aligned word (D = 3, 7)
        int8_t row[D + 1];
        if constexpr (D + 1 == 4) {
            const uint32_t wd = __ldg((const unsigned int*)(rows + r * 4));
#pragma unroll
            for (int j = 0; j < 4; j++) row[j] = (int8_t)(wd >> (8 * j));
        } else if constexpr (D + 1 == 8) {
            const uint2 wd = __ldg((const uint2*)(rows + r * 8));
#pragma unroll
            for (int j = 0; j < 8; j++) row[j] = (int8_t)((j < 4 ? wd.x : wd.y) >> (8 * (j & 3)));
        } else {
#pragma unroll
            for (int j = 0; j <= D; j++) row[j] = rows[r * (D + 1) + j];
        }
        int32_t olo, ohi;
        if (qo) {
            float rest = 0.f;
#pragma unroll
            for (int d = 1; d < D; d++) {
                const int32_t o = row[1 + d];
                const float gap = o > 0 ? __fsub_rn(__fmul_rn(small_i2f(o), cf[d]), qo[d])
                                        : (o < 0 ? __fsub_rn(qo[d], __fmul_rn(small_i2f(o + 1), cf[d])) : 0.f);
                rest = __fadd_rn(rest, __fmul_rn(gap, gap));
            }
            if (rest > R2q) continue;
            // dimension 0: offset o > 0 is within reach iff o c0 - q0 <= s, o < 0 iff q0 - (o + 1) c0 <= s
            const float sr = sqrt_approx(__fsub_rn(R2q, rest));
            const int32_t up = small_floor(__fmul_rn(__fadd_rn(sr, qo[0]), inv_c0));
            const int32_t dn = -1 - small_floor(__fmul_rn(__fsub_rn(sr, qo[0]), inv_c0));
            olo = max((int32_t)row[0], min(dn, 0));
            ohi = min((int32_t)row[1], max(up, 0));
        } else {
            // cell-based range: |o_0| <= 1 + sqrt(R2q - row distance) / c0, as the largest j with
            // j^2 c0^2 <= R2q - rest (no square root, no division), up to the row's own extent
            const float avail = R2q - rows_r2[r], c0sq = cf[0] * cf[0];
            const int32_t ext = 1 + max(-(int32_t)row[0], (int32_t)row[1]);
            int32_t o0max = 1;
            while (o0max < ext && __fmul_rn(small_i2f(o0max * o0max), c0sq) <= avail) o0max++;
            olo = max((int32_t)row[0], -o0max);
            ohi = min((int32_t)row[1], o0max);
        }
        int8_t q[D];
        int64_t base = 0;
#pragma unroll
        for (int d = D - 1; d >= 1; d--) {
            int32_t kk = k[d] + (int32_t)row[1 + d];
            int8_t qq = 0;
            if (kk < 0) { kk += n[d]; qq = -1; }
            else if (kk >= n[d]) { kk -= n[d]; qq = 1; }
            q[d] = qq;
            base = base * n[d] + kk;
        }
        base *= n[0];
        const int32_t a = k[0] + olo, b = k[0] + ohi;
        if (a < 0) {
            q[0] = -1;
            if (g(base, a + n[0], (b < 0 ? b : -1) + n[0], q, row)) return true;
        }
        {
            const int32_t lo = a > 0 ? a : 0, hi = b < n[0] - 1 ? b : n[0] - 1;
            q[0] = 0;
            if (lo <= hi && g(base, lo, hi, q, row)) return true;
        }
        if (b >= n[0]) {
            q[0] = 1;
            if (g(base, (a > n[0] ? a : n[0]) - n[0], b - n[0], q, row)) return true;
        }
    }
    return false;
}

// cell_of and the walk's query offsets together: the offset is the fraction of the cell coordinate that
// cell_of already forms, times the cell edge (two more FP64-pipe instructions per dimension)
template <int D>
__device__ __forceinline__ void cell_of_q(const Grid<D>& g, const Geo<D>& geo, const double* x, int32_t* k, float* qo) {
#pragma unroll
    for (int d = 0; d < D; d++) {
        const double y = __dmul_rn(__dsub_rn(x[d], geo.inf[d]), g.inv_c[d]);
        const double fl = floor(y);
        int32_t kk = (int32_t)fl;
        kk = kk < 0 ? 0 : (kk >= g.n[d] ? g.n[d] - 1 : kk);
        k[d] = kk;
        qo[d] = __fmul_rn(__double2float_rn(__dsub_rn(y, (double)kk)), g.cf[d]);
    }
}

// Visits the placed spheres in the stencil around cell k; f(idx, img, r) returns true to stop.
template <int D, class F>
__device__ __forceinline__ bool visit_placed(const Grid<D>& g, const Geo<D>& geo, const int32_t* k, const float* qo,
                                             float R2q, F&& f) {
    return walk_rows<D>(g.n, g.rows, g.R, g.rows_r2, g.cf, g.inv_c0f, R2q, k, qo, [&](int64_t base, int32_t lo, int32_t hi, const int8_t* q, const int8_t*) {
        for (int32_t x = lo; x <= hi; x += 32) {
            const int len = hi - x + 1 < 32 ? hi - x + 1 : 32;
            uint32_t bits = occ_bits(g.occ, base + x, len);
            while (bits) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                const int64_t idx = base + x + j;
                double p[D], img[D];
#pragma unroll
                for (int d = 0; d < D; d++) p[d] = g.pos[idx * D + d];
                image_of<D>(geo, p, q, img);
                if (f(idx, img, g.mono ? g.rmono : g.rad[idx])) return true;
            }
        }
        return false;
    });
}

// Visits the placed spheres in the stencil around cell k with their integer cell offset o (the periodic
// shift folded in: o = cell of the image - k); f(idx, o, q) returns true to stop.
template <int D, class F>
__device__ __forceinline__ bool visit_placed_o(const Grid<D>& g, const int32_t* k, const float* qo, float R2q, F&& f) {
    return walk_rows<D>(g.n, g.rows, g.R, g.rows_r2, g.cf, g.inv_c0f, R2q, k, qo, [&](int64_t base, int32_t lo, int32_t hi, const int8_t* q, const int8_t* row) {
        int32_t o[D];
#pragma unroll
        for (int d = 1; d < D; d++) o[d] = row[1 + d];
        const int32_t shift0 = (q[0] < 0 ? -g.n[0] : (q[0] > 0 ? g.n[0] : 0)) - k[0];
        for (int32_t x = lo; x <= hi; x += 32) {
            const int len = hi - x + 1 < 32 ? hi - x + 1 : 32;
            uint32_t bits = occ_bits(g.occ, base + x, len);
            while (bits) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                o[0] = x + j + shift0;
                if (f(base + x + j, o, q)) return true;
            }
        }
        return false;
    });
}

// Brick walk (2D and 3D grids with a brick map): the placed spheres in the cells within reach of the query, read
// as bricks of 64 occupancy bits (8x8 cells in 2D, 4x4x4 in 3D; brick_bits per side), 1 to 3 bricks per
// dimension, instead of stencil rows.  Cell-box based (a superset of the point-trimmed walk); only for
// neighbourhoods that do not wrap around the periodic box (brick_reach returns false otherwise, and the caller
// walks the rows).  f(idx, o) returns true to stop.
template <int D>
__host__ __device__ constexpr int brick_bits() { return D == 2 ? 3 : 2; }

// The cells [lo_d, hi_d] within reach sqrt(R2q) of the query: cell k at offset qo from its corner (the
// reach along +d is the distance to the cell's upper face plus whole cells, along -d to its lower face), or
// of any point of cell k when qo is null.  The 1e-4 margin of R2q covers the float error of these bounds.
template <int D>
__device__ __forceinline__ bool brick_reach(const Grid<D>& g, const int32_t* k, const float* qo, float R2q,
                                            int32_t* lo, int32_t* hi) {
    if ((D != 2 && D != 3) || !g.bocc) return false;
    const float s = sqrt_approx(R2q);
    bool ok = true;
#pragma unroll
    for (int d = 0; d < D; d++) {
        const float up = qo ? __fsub_rn(s, __fsub_rn(g.cf[d], qo[d])) : s;  // beyond the upper face
        const float dn = qo ? __fsub_rn(s, qo[d]) : s;                      // beyond the lower face
        hi[d] = k[d] + (up < 0.f ? 0 : 1 + small_floor(__fmul_rn(up, g.inv_cf[d])));
        lo[d] = k[d] - (dn < 0.f ? 0 : 1 + small_floor(__fmul_rn(dn, g.inv_cf[d])));
        ok = ok && lo[d] >= 0 && hi[d] < g.n[d];
    }
    return ok;
}

// Cell mask of a 4x4x4 brick (bit x + 4y + 16z) from its per-dimension spans xm, ym, zm (4 bits each): the x
// span placed in the selected rows by one multiply (xm < 16 against bits 4 apart: no carries), then the row
// plane copied into the selected z planes.
__device__ __forceinline__ unsigned long long brick_mask3(uint32_t xm, uint32_t ym, uint32_t zm) {
    const uint32_t ys = (ym & 1u) | ((ym & 2u) << 3) | ((ym & 4u) << 6) | ((ym & 8u) << 9);
    const uint32_t plane = xm * ys;
    const uint32_t p2 = plane | (plane << 16);
    const uint32_t lo = p2 & (((0u - (zm & 1u)) & 0xFFFFu) | ((0u - ((zm >> 1) & 1u)) & 0xFFFF0000u));
    const uint32_t hi = p2 & (((0u - ((zm >> 2) & 1u)) & 0xFFFFu) | ((0u - ((zm >> 3) & 1u)) & 0xFFFF0000u));
    return ((unsigned long long)hi << 32) | lo;
}

// bits of cells [lo, hi] within brick b of a side of 2^SB cells
template <int SB>
__device__ __forceinline__ uint32_t brick_span(int32_t lo, int32_t hi, int32_t b) {
    const int32_t a = max(lo, b << SB) - (b << SB), e = min(hi, (b << SB) + (1 << SB) - 1) - (b << SB);
    return ((2u << e) - 1u) & ~((1u << a) - 1u);
}

// the brick visited at step a of the ascending walk a = b0, b0 + 1, ...: brick a itself, or (OWN_FIRST) brick
// `own` first, then the others ascending
template <bool OWN_FIRST>
__device__ __forceinline__ int32_t brick_at(int32_t b0, int32_t own, int32_t a) {
    if (!OWN_FIRST) return a;
    if (a == b0) return own;
    return a - 1 < own ? a - 1 : a;
}

template <int D, bool OWN_FIRST = false, class F>
__device__ __forceinline__ bool visit_bricks(const Grid<D>& g, const int32_t* k, const int32_t* lo, const int32_t* hi,
                                             F&& f) {
    static_assert(D == 2 || D == 3, "bricks of 8x8 or 4x4x4 cells");
    constexpr int SB = brick_bits<D>(), SIDE = 1 << SB;
    constexpr int Z = D == 3 ? 2 : 0;
    const int32_t lo2 = D == 3 ? lo[Z] : 0, hi2 = D == 3 ? hi[Z] : 0;
    for (int32_t az = lo2 >> SB; az <= (hi2 >> SB); az++) {
        const int32_t bz = brick_at<OWN_FIRST>(lo2 >> SB, D == 3 ? k[Z] >> SB : 0, az);
        const uint32_t zm = D == 3 ? brick_span<SB>(lo2, hi2, bz) : 1u;
        for (int32_t ay = lo[1] >> SB; ay <= (hi[1] >> SB); ay++) {
            const int32_t by = brick_at<OWN_FIRST>(lo[1] >> SB, k[1] >> SB, ay);
            const uint32_t ym = brick_span<SB>(lo[1], hi[1], by);
            for (int32_t ax = lo[0] >> SB; ax <= (hi[0] >> SB); ax++) {
                const int32_t bx = brick_at<OWN_FIRST>(lo[0] >> SB, k[0] >> SB, ax);
                const uint32_t xm = brick_span<SB>(lo[0], hi[0], bx);
                unsigned long long mask;
                if constexpr (D == 3) {
                    mask = brick_mask3(xm, ym, zm);
                } else {
                    mask = 0;
#pragma unroll
                    for (int y = 0; y < SIDE; y++)
                        if ((ym >> y) & 1u) mask |= (unsigned long long)xm << (SIDE * y);
                }
                const int64_t word = bx + (int64_t)g.nb[0] * (by + (D == 3 ? (int64_t)g.nb[1] * bz : 0));
                unsigned long long bits = __ldg(g.bocc + word) & mask;
                while (bits) {
                    const int j = __ffsll((long long)bits) - 1;
                    bits &= bits - 1;
                    int32_t c[D], o[D];
                    c[0] = (bx << SB) + (j & (SIDE - 1));
                    c[1] = (by << SB) + ((j >> SB) & (SIDE - 1));
                    if (D == 3) c[D == 3 ? 2 : 0] = (bz << SB) + (j >> (2 * SB));
                    int64_t idx = 0;
#pragma unroll
                    for (int d = D - 1; d >= 0; d--) {
                        o[d] = c[d] - k[d];
                        idx = idx * g.n[d] + c[d];
                    }
                    if (f(idx, o)) return true;
                }
            }
        }
    }
    return false;
}

// visit_placed_o by bricks where they apply, else by rows; OWN_FIRST visits the query's own brick first in each
// dimension (a walk that stops at its first hit meets the near spheres sooner)
template <int D, bool OWN_FIRST = false, class F>
__device__ __forceinline__ bool visit_placed_fo(const Grid<D>& g, const int32_t* k, const float* qo, float R2q, F&& f) {
    if constexpr (D == 2 || D == 3) {
        int32_t lo[D], hi[D];
        if (brick_reach<D>(g, k, qo, R2q, lo, hi)) {
            const int8_t q0[D] = {};
            return visit_bricks<D, OWN_FIRST>(g, k, lo, hi,
                                              [&](int64_t idx, const int32_t* o) { return f(idx, o, q0); });
        }
    }
    return visit_placed_o<D>(g, k, qo, R2q, f);
}

// FP32 model of (image of a stored centre) - (query point): o c + (off_s - off_q), with o the integer
// cell offset; its error against the FP64 difference is bounded by the guard band of the grid.
template <int D>
__device__ __forceinline__ void model_delta(const float* cf, const int32_t* o, const float* off_s, const float* off_q,
                                            float* dlt) {
#pragma unroll
    for (int d = 0; d < D; d++) dlt[d] = __fadd_rn(__fmul_rn(small_i2f(o[d]), cf[d]), __fsub_rn(off_s[d], off_q[d]));
}

template <int D>
__device__ __forceinline__ float sumsq32(const float* v) {
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < D; d++) s = __fadd_rn(s, __fmul_rn(v[d], v[d]));
    return s;
}

// Fixed-point cell map of the FP32 form: y = (a + bits 2^-53) (ri + rf 2^-64) 2^-shift for integers a >= 0,
// bits < 2^53 and 0 <= shift < 64.  k = floor(y); frac32 = the top 32 bits of y's fraction.  Integer
// instructions only; exact but for the truncation of rf (below a 2^-64 cell edge per unit of a 2^-shift).
__device__ __forceinline__ void fixed_cell(uint64_t a, uint64_t bits, uint32_t ri, uint64_t rf, int shift, int64_t& k,
                                           uint32_t& frac32) {
    const uint64_t lo1 = a * rf, hi1 = __umul64hi(a, rf);
    const uint64_t iu = bits * (uint64_t)ri;                 // u ri in 2^-53 units
    const uint64_t f2 = (iu & ((1ull << 53) - 1)) << 11;     // its fraction, 2^-64 units
    const uint64_t f3 = __umul64hi(bits << 11, rf);          // u rf, 2^-64 units
    uint64_t lo = lo1 + f2;
    uint64_t carry = lo < f2 ? 1u : 0u;
    lo += f3;
    carry += lo < f3 ? 1u : 0u;
    const uint64_t ip = a * (uint64_t)ri + hi1 + (iu >> 53) + carry;
    if (shift == 0) {
        k = (int64_t)ip;
        frac32 = (uint32_t)(lo >> 32);
    } else {
        k = (int64_t)(ip >> shift);
        frac32 = (uint32_t)(((lo >> shift) | (ip << (64 - shift))) >> 32);
    }
}

// squared search radius (r_query + r_max)^2 with a margin, as float
__device__ __forceinline__ float search_r2(double rq, double rmax) {
    const float s = (float)(rq + rmax);
    return s * s * 1.0001f;
}
// the same from float radii, rounded up: no FP64 instruction (the 1e-4 margin is far above the radii's rounding)
__device__ __forceinline__ float search_r2f(float rq, float rmax) {
    const float s = __fadd_ru(rq, rmax);
    return __fmul_ru(__fmul_ru(s, s), 1.0001f);
}

// Bit patterns of non-negative doubles order like the values: integer max / compare on the ALU
// instead of the FP64 pipe.
__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double maxabs(double a, double b) {
    const uint64_t ua = dbits(a) & 0x7fffffffffffffffull, ub = dbits(b) & 0x7fffffffffffffffull;
    return __longlong_as_double((long long)(ua > ub ? ua : ub));
}

// ---------------------------------------------------------------------------------------------
// warp / block helpers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const uint32_t mask = __activemask();
    const uint32_t ballot = __ballot_sync(mask, pred);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader && ballot) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(ballot & ((1u << lane) - 1u));
}

template <int BLOCK>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[BLOCK / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < BLOCK / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < BLOCK / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    const uint32_t warp_prefix = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[BLOCK / 32 - 1];
    const uint32_t r = warp_prefix + x - v;
    __syncthreads();
    return r;
}

}  // namespace rsagpu
