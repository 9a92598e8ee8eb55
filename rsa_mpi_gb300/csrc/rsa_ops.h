// rsa_ops.h -- host-side launch interface of the per-dimension kernel sets.
// kernels.cu is compiled once per dimension D (-DRSA_DIM=D) and exports dim_ops_D(); the host driver
// (rsagpu.cu) picks the table for the instance's dimension.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace rsagpu {

constexpr int MAX_D = 7;

struct GridArgs {
    int64_t ncells;
    int32_t n[MAX_D];
    double inv_c[MAX_D];
    double inf[MAX_D];
    double L[MAX_D];
    uint32_t* occ;
    double* pos;
    double* rad;
    int32_t* phase;
    const int8_t* stencil;
    int S;
    const int8_t* rows;  // stencil rows along dimension 0: {xlo, xhi, o_1, ..., o_{D-1}}
    int R;
    const float* rows_r2;  // per row: squared nearest distance along dimensions 1..D-1 (rows sorted by it)
    double rmax;           // largest radius the grid holds
    float* off;          // FP32 screening offsets (D floats per cell)
    float* radf;         // radii rounded to float
    double c[MAX_D];     // cell edge
    float cf[MAX_D];     // cell edge rounded to float
    float guard;         // guard band of the FP32 screen (absolute, on squared distances)
    int mono;            // one radius class
    double rmono;
    unsigned long long* bocc;  // 3D: occupancy by 4x4x4 bricks of cells (bit x + 4 y + 16 z), or null
    int32_t nb[MAX_D];         // bricks per dimension
    // 3D single-instance grids: the same bricks for the spheres placed since the last mask pass (the mask pass
    // of voxels with an inherited sphere list walks only these), or null
    unsigned long long* bnew = nullptr;
};

struct CandArgs {
    uint32_t n;         // candidates in the round
    double* pos;        // n * D
    uint64_t* key;      // priority key (smaller first)
    double* rad;
    int32_t* phase;
    int64_t* cell;      // sphere-grid cell of the candidate
    uint8_t* state;     // ST_*
    int32_t* next;      // linked list of candidates per cell
    int32_t* head;      // per grid cell, -1 = no candidate
    uint32_t* cocc;     // 1 bit per grid cell: holds a candidate of this round (one padding word)
    uint32_t* alive;    // candidates that survived the probe
    uint32_t* counters; // [0] = alive, [1] = accepted, [2] = error bits, [3] = gathered, [4] = FP64 retests
    float* off;         // FP32 screening offsets of the candidates (guard-band form)
    float* radf;        // their radii in FP32, written by the probe for the candidates it keeps (guard-band form)
    int32_t* kc;        // cell coordinates of the candidates (guard-band form)
    int32_t* blk;       // NB lower-priority colliders per candidate
    uint8_t* nblk;
    uint32_t* und;      // undecided count after each settle iteration (und[0] after collect)
    uint64_t* gather;   // keys of accepted candidates (count cap)
    // the largest candidate radius of the round (0: the grid's rmax): it bounds the candidate-candidate search
    // of collect and settle, which otherwise reaches for the grid's largest placed radius
    double rcmax;
    float rcmaxf;
    // lazy candidates (FP32-form darts): until the probe forms the exact position, cell holds the dart's
    // voxel and pos its 53 random bits per coordinate; lvox and llen are that round's voxel list and length
    int32_t lazy;
    const int64_t* lvox;
    double llen[MAX_D];
};

struct DartArgs {
    uint32_t n;
    uint64_t V;
    const int64_t* vox;
    double len[MAX_D];
    uint64_t seed;
    uint64_t round;
    double radius;
    int32_t phase;
    uint64_t* vidx_out;  // optional: chosen voxel per dart
    int32_t rand_radius;  // continuous radius law: radius = r_lo + r_span x, x from the dart's own Philox draw
    double r_lo, r_span;
    // or, with ntab >= 2, the transform tabulated at x = j / (ntab - 1) (device array), interpolated linearly
    const double* rtab;
    int32_t ntab;
    uint64_t rho_frac[MAX_D];  // FP32-form darts: level-0 voxel length / cell edge (voxel_cell_ratio)
    uint32_t rho_int[MAX_D];
    int32_t level;             // voxel level (the fixed-point shift)
    // binned order (optional): slot t of the round holds dart perm[t]; DimOps::dart_bins builds perm, the darts
    // of each bin of 2^bin_shift consecutive voxels together
    uint32_t* bin_hist;        // per bin: dart count (pass 1; consumed by pass 2)
    const uint64_t* bin_off;   // per bin: first slot (exclusive scan of the counts; null in pass 1)
    int32_t bin_shift;
    uint32_t* perm;            // n dart indices
};

struct RefineArgs {
    uint64_t V;
    const int64_t* vin;
    int64_t* vout;
    uint64_t vout_cap;   // voxels vout holds
    double len[MAX_D];   // parent length
    double nlen[MAX_D];  // child length = 0.5 * parent
    double rmin;
    uint32_t* masks;     // W words per parent
    uint32_t* warp_counts;     // children kept per warp of 32 parents
    uint64_t* warp_offsets;    // exclusive scan of warp_counts
    uint32_t* err;
    uint32_t* survivors;  // parents not covered (remove_covered keeps them)
    unsigned long long* visits;  // occupied stencil cells visited by the mask pass
    unsigned long long* retests; // (voxel, sphere) pairs redone in FP64 (guard-band form)
    uint64_t rho_frac[MAX_D];    // level-0 voxel length / cell edge in fixed point (voxel_cell_ratio)
    uint32_t rho_int[MAX_D];
    int32_t level;               // parent level (the fixed-point shift)
    // Sphere lists handed from a voxel to its children (3D FP32 mask pass at levels >= 1).  A recording pass
    // stores, for every surviving voxel, the cells of the spheres that reach into the voxel (centre within
    // r_s + r_min of some point of it): every sphere that can cover a descendant or enter its prefilter list,
    // among those placed so far.  An inheriting pass then tests each voxel against its parent's list plus
    // the spheres placed since (GridArgs::bnew) instead of walking the whole neighbourhood.
    int32_t record;              // store this pass's lists (lout, nout)
    int32_t inherit;             // read the parents' lists (lin, nin, parent)
    float hdiagf;                // half diagonal of this pass's voxels, rounded up (the reach of a recording walk)
    const uint32_t* lin;         // LIST_K cell indices per voxel of the previous pass
    const uint8_t* nin;          // their counts (LIST_NONE: no list, walk the whole neighbourhood)
    const uint32_t* parent;      // index of each voxel's parent in the previous pass
    uint32_t* lout;              // this pass's lists, LIST_K per voxel
    uint8_t* nout;
    uint32_t* parent_out;        // k_refine_write: the parent of each child written (or null)
    uint64_t div0, div1;         // ceil(2^64 / n_0), ceil(2^64 / n_1): cell index -> coordinates
};

constexpr int LIST_K = 16;           // cells in one voxel's sphere list
constexpr uint8_t LIST_NONE = 0xFF;  // no list: the voxel's children walk their whole neighbourhood

// The FP32 form maps a point of a voxel at level `level` to cells in 64-bit fixed point:
// y = (coordinate + u) * rho0 * 2^-level cell edges, rho0 = len0 / c (level-0 voxel length over cell edge; the
// voxel length halves exactly per level), held as an integer part and a 64-bit fraction with the double's full
// precision.  len is the current length; returns false when y * 2^level could leave 64 bits.
inline bool voxel_cell_ratio(double len, int level, double c, int32_t n, uint32_t* rho_int, uint64_t* rho_frac) {
    const double rho = std::ldexp(len, level) / c;
    const double ip = std::floor(rho);
    *rho_int = (uint32_t)ip;
    *rho_frac = (uint64_t)std::ldexp(rho - ip, 64);  // rho - ip <= 1 - 2^-53: below 2^64
    return std::ldexp((double)n * (ip + 1), level + 1) < 9.0e18;
}

// ------------------------------------------------------------------------------------------------
// batched instances: many independent one-radius instances of one dimension share every launch.
// Each instance owns a segment of the wave's arrays (cells, voxels, darts); a thread finds the
// instance of its element by binary search over the segment offsets.
// ------------------------------------------------------------------------------------------------
struct BatchInstance {   // host description of one instance of a wave
    GridArgs g;          // its grid (mono = 1); pointers into the wave's arrays
    int32_t* head;       // its candidate lists and candidate occupancy bits
    uint32_t* cocc;
    uint64_t seed;       // Philox key of its darts
    int64_t nvox0[MAX_D];  // level-0 voxels per dimension
};

struct BatchRound {      // per instance, per round
    uint64_t vbase;      // first voxel of its segment
    uint64_t V;          // voxels in its segment
    double len[MAX_D];   // voxel length at its level
    double nlen[MAX_D];  // child length = 0.5 * len
    uint64_t rho_frac[MAX_D];  // level-0 voxel length / cell edge (voxel_cell_ratio)
    uint32_t rho_int[MAX_D];
    int32_t level;             // its voxel level
    int32_t refine;      // subdivide its voxels after this round's pass
};

struct BatchArgs {
    uint32_t M;                // instances in the wave
    const void* table;         // per-dimension instance table (DimOps::batch_table_fill)
    const BatchRound* rnd;     // M entries
    const uint64_t* dart_off;  // M + 1: the darts of instance s are [dart_off[s], dart_off[s + 1])
    const uint64_t* vox_off;   // M + 1: its voxels
    const uint64_t* word_off;  // M + 1: its occupancy words (32 cells each)
    const int64_t* vox;        // the wave's voxel list (D coordinates per voxel)
    uint32_t* cinst;           // instance of each candidate
    uint32_t* acc;             // spheres accepted per instance in the current round
    uint32_t* alive_inst;      // candidates per instance that survived the probe in the current round
    uint64_t round;            // round index (the Philox counter's round words)
    uint32_t* bin_hist;        // binned dart order over the wave's voxel list (see DartArgs), or null
    const uint64_t* bin_off;   // null in pass 1
    int32_t bin_shift;
    uint32_t* perm;            // slot t holds global dart perm[t]
    uint64_t ndarts;           // darts of the round, all instances
    uint64_t V;                // voxels, all instances
    uint64_t nwords;           // occupancy words, all instances
    const uint32_t* occ;       // the wave's occupancy bits and centres (results pass)
    const double* pos;
};

struct DimOps {
    int D;
    void (*vox_init)(int64_t* vox, uint64_t V, const int64_t* nvox, cudaStream_t s);
    void (*darts)(const GridArgs& g, const CandArgs& c, const DartArgs& a, cudaStream_t s);
    void (*darts32)(const GridArgs& g, const CandArgs& c, const DartArgs& a, cudaStream_t s);  // lazy candidates
    void (*dart_bins)(const CandArgs& c, const DartArgs& a, cudaStream_t s);  // binned order: pass 1 or 2
    void (*probe)(const GridArgs& g, const CandArgs& c, int f32, cudaStream_t s);
    void (*collect)(const GridArgs& g, const CandArgs& c, int f32, cudaStream_t s);
    void (*settle)(const GridArgs& g, const CandArgs& c, int iteration, int f32, cudaStream_t s);
    void (*gather_accepted)(const CandArgs& c, cudaStream_t s);
    void (*cut_accepted)(const CandArgs& c, int use_pivot, double pivot, uint64_t key_cut, cudaStream_t s);
    void (*commit)(const GridArgs& g, const CandArgs& c, cudaStream_t s);
    void (*refine_mask)(const GridArgs& g, const RefineArgs& a, int f32, cudaStream_t s);
    void (*refine_write)(const RefineArgs& a, cudaStream_t s);
    void (*check)(const GridArgs& g, unsigned long long* overlaps, unsigned long long* misplaced, cudaStream_t s);
    void (*volume_partials)(const GridArgs& g, double unit_volume, double* partials, int nblocks, cudaStream_t s);
    void (*extract_write)(const GridArgs& g, const uint64_t* block_offsets, double* pos, double* rad,
                          int32_t* phase, cudaStream_t s);
    // regrid: cell of each of c.n spheres in c.pos, state ACCEPTED, alive list 0..n-1 (then commit)
    void (*locate)(const GridArgs& g, const CandArgs& c, cudaStream_t s);
    int children;      // 2^D
    int mask_words;    // 32-bit words of child mask per voxel
    // batched instances (block = threads per block, from the autotuner)
    uint64_t (*batch_table_bytes)(uint32_t M);
    // copies the instance table to the device (synchronous); returns a cudaError_t
    int (*batch_table_fill)(const BatchInstance* inst, uint32_t M, void* d_table, cudaStream_t s);
    void (*b_vox_init)(const BatchArgs& b, int64_t* vox, cudaStream_t s);
    void (*b_darts)(const BatchArgs& b, const CandArgs& c, int f32, cudaStream_t s);  // f32: lazy candidates
    void (*b_dart_bins)(const BatchArgs& b, const CandArgs& c, cudaStream_t s);  // pass 1 or 2 (as dart_bins)
    void (*b_probe)(const BatchArgs& b, const CandArgs& c, int f32, int block, cudaStream_t s);
    void (*b_collect)(const BatchArgs& b, const CandArgs& c, int f32, int block, cudaStream_t s);
    void (*b_settle)(const BatchArgs& b, const CandArgs& c, int iteration, int f32, int block, cudaStream_t s);
    void (*b_commit)(const BatchArgs& b, const CandArgs& c, cudaStream_t s);
    void (*b_refine_mask)(const BatchArgs& b, const RefineArgs& a, int f32, int block, cudaStream_t s);
    void (*b_refine_offsets)(const BatchArgs& b, const RefineArgs& a, uint64_t* new_off, cudaStream_t s);
    void (*b_refine_write)(const BatchArgs& b, const RefineArgs& a, cudaStream_t s);
    void (*b_results)(const BatchArgs& b, unsigned long long* counts, unsigned long long* sums, cudaStream_t s);
    // count cap under the reference rule (the pass structure of find_solve_conflicts): the first pass's
    // candidates, one greedy step on the candidates that are not Conflict, the keys of the pass's Undecided
    // candidates (counters[3]), the end of a pass (mode PASS_VALIDATE / PASS_PIVOT / PASS_END), the next pass's
    // candidates (und[0]), the Conflict sources (frontier 0, count in counters[5]), and one level of the Conflict
    // search (frontier `from` of nf candidates -> frontier 1 - from, count in counters[6 - from])
    void (*pass_begin)(const CandArgs& c, cudaStream_t s);
    void (*pass_step)(const GridArgs& g, const CandArgs& c, int iteration, int f32, cudaStream_t s);
    void (*pass_gather)(const CandArgs& c, cudaStream_t s);
    void (*pass_close)(const CandArgs& c, int mode, double pivot, cudaStream_t s);
    void (*pass_next)(const GridArgs& g, const CandArgs& c, int f32, cudaStream_t s);
    void (*pass_sources)(const GridArgs& g, const CandArgs& c, int f32, cudaStream_t s);
    void (*pass_push)(const GridArgs& g, const CandArgs& c, int from, uint32_t nf, int f32, cudaStream_t s);
    // extract_write into outputs the kernels can store to directly (pinned host memory): each warp writes its
    // spheres as contiguous runs of the output arrays
    void (*extract_direct)(const GridArgs& g, const uint64_t* block_offsets, double* pos, double* rad,
                           int32_t* phase, cudaStream_t s);
};

// modes of DimOps::pass_close
constexpr int CAP_PASS_VALIDATE = 0, CAP_PASS_PIVOT = 1, CAP_PASS_END = 2;

const DimOps* dim_ops(int D);

// dimension-independent kernels (kernels_common.cu)
void launch_scan_blocks(const uint32_t* counts, uint64_t* offsets, uint64_t n, uint64_t* total, cudaStream_t s);
void launch_occ_block_counts(const uint32_t* occ, int64_t nwords, uint32_t* counts, cudaStream_t s);
// 65536-bin histogram (zeroed first) of the 16-bit digit (key >> S >> dshift) & 0xFFFF over the keys with
// (key >> S) >> pshift == prefix (pshift = 64: all keys)
void launch_key_digit_hist(const uint64_t* keys, uint64_t n, int S, int dshift, int pshift, uint64_t prefix,
                           uint32_t* hist, cudaStream_t s);
uint64_t kernel_launch_count();
void count_launch(int n = 1);
// text returned by rsagpu_last_error() for the calling thread
void set_last_error(const char* msg);
// learned schedule: y[0..1] = MLP(features[0..15]) on stream s (mlp.cu)
int mlp_decide(const uint16_t* d_weights, const float* d_features, float* d_out, cudaStream_t s);

constexpr int REFINE_BLOCK = 256;
constexpr int OCC_BLOCK = 256;  // words per extract block

}  // namespace rsagpu
