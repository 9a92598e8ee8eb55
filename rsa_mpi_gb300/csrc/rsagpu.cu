// rsagpu.cu -- host driver and C ABI of the GB300 sampler (include/rsagpu.h).
//
// The round loop restates rsa_algo::proceed_voxel (operator_algorithm.ixx:85-188) with device-resident
// state: the whole periodic domain lives in one device cell grid, so the reference's MPI ghost exchange
// (operator_ghost, rsa_ghost_area, rsa_buffer) becomes periodic index wrap inside the kernels and its
// Allreduce counters become device counters read once per round.
#include <algorithm>
#include <chrono>
#include <map>
#include <cmath>
#include <random>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rsagpu.h"
#include "rsa_device.cuh"
#include "rsa_ops.h"
#include "host_common.h"

using namespace rsagpu;
using namespace rsagpu::host;

namespace {
thread_local std::string g_err;  // text of rsagpu_last_error() for the calling thread

// magical_default_miss_rate (operator_algorithm.ixx:344-351)
double reference_miss_threshold(int D) { return D <= 3 ? 0.95 : 1 - 0.05 * pow_int(0.1, D - 3); }

struct TraceRow {
    uint64_t voxels, darts, accepted;
    uint8_t refined;
    int32_t level;
    float features[16];  // state seen by the schedule after the round's pass
    double pass_ms;      // host wall time of the pass (darts to commit)
    double refine_ms;    // host wall time of the refinement that followed (0 if none)
};

constexpr int NFEAT = 16;

constexpr int MAX_SETTLE = 4096;
constexpr int COUNTERS = 8;
// pinned mirror of the counters: COUNTERS + und[MAX_SETTLE + 1], then a copy of the settle's und[] kept for the
// round's statistics (read with the commit's counters, not in a synchronisation of its own)
constexpr int H_COUNTERS = COUNTERS + 2 * (MAX_SETTLE + 1);
constexpr int H_SETTLE = COUNTERS + MAX_SETTLE + 1;

}  // namespace

// ------------------------------------------------------------------------------------------------
// handles
// ------------------------------------------------------------------------------------------------
struct rsagpu_radgen {
    int dim = 0;
    std::vector<double> r;
    std::vector<uint64_t> n;
    std::vector<int> phase;
    double excl = 0;
    int idx = 0;
    // continuous radius law (RandomRadiusGenerator with x -> r_min + (r_max - r_min) x): one entry
    // (radius 0, count, phase 0) in the class list, every dart's radius drawn (radius_generator.ixx:39-48)
    bool uniform = false;
    double u_rmin = 0, u_rmax = 0;
    std::vector<double> table;  // a tabulated transform (knots at x = j / (n - 1)); empty: r_min + (r_max - r_min) x
    int u_phase = 0;
    double rmax() const { return uniform ? u_rmax : r.front(); }
    double rmin() const { return uniform ? u_rmin : r.back(); }
};

struct SphereGrid {
    bool ready = false;
    double rmin = 0, rmax = 0;
    GridArgs a{};
    std::vector<int8_t> stencil;
    std::vector<int8_t> rows;
    int8_t* d_stencil = nullptr;
    int8_t* d_rows = nullptr;
    float* d_rows_r2 = nullptr;
    int32_t* head = nullptr;
    uint32_t* cocc = nullptr;  // candidate occupancy bits of the current round
    uint64_t nbricks = 0;      // words of a.bocc (and of a.bnew)
    void release() {
        dfree(cocc);
        dfree(a.bnew);
        dfree(d_rows);
        dfree(d_rows_r2);
        dfree(a.off);
        dfree(a.radf);
        dfree(a.occ);
        dfree(a.bocc);
        dfree(a.pos);
        dfree(a.rad);
        dfree(a.phase);
        dfree(d_stencil);
        dfree(head);
        ready = false;
    }
};

struct rsagpu_domain {
    int dim = 0;
    int device = 0;
    double inf[MAX_D]{}, sup[MAX_D]{}, L[MAX_D]{};
    double rad_max = 0;
    SphereGrid grid;
    cudaStream_t stream = nullptr;
    ~rsagpu_domain() { grid.release(); }
};

struct CandBuffers {
    uint64_t cap = 0;
    CandArgs a{};
    uint64_t* vidx = nullptr;
    void release() {
        dfree(a.pos);
        dfree(a.key);
        dfree(a.rad);
        dfree(a.phase);
        dfree(a.cell);
        dfree(a.state);
        dfree(a.next);
        dfree(a.alive);
        dfree(a.counters);
        dfree(a.blk);
        dfree(a.nblk);
        dfree(a.gather);
        dfree(a.off);
        dfree(a.radf);
        dfree(a.kc);
        dfree(vidx);
        cap = 0;
    }
};

struct rsagpu_algo {
    rsagpu_domain* dom = nullptr;
    rsagpu_radgen rg;
    int nbshots = 6000;
    double rmax_algo = 0;  // m_r_max: the largest r_max of the radius generators so far
    double cand_rmax = 0;  // the largest candidate radius of the current round (0: unknown, the grid's rmax)
    // a learned-schedule input: the cells of a grid for the smallest radius of the generators so far
    double feat_rmin = 0;
    int64_t feat_ncells = 0;
    const DimOps* ops = nullptr;
    cudaStream_t stream = nullptr;
    // voxels
    int64_t* vox[2] = {nullptr, nullptr};
    uint64_t vox_cap[2] = {0, 0};
    int cur = 0;
    uint64_t V = 0;
    int level = 0;
    int64_t nvox0[MAX_D]{};
    double len[MAX_D]{};
    uint32_t* bin_hist = nullptr;  // binned dart order: per-bin counts and first slots, the permutation
    uint64_t* bin_off = nullptr;
    uint64_t bins_cap = 0;
    uint32_t* perm = nullptr;
    uint64_t perm_cap = 0;
    uint32_t* masks = nullptr;
    uint64_t masks_cap = 0;
    uint32_t* block_counts = nullptr;
    uint64_t* block_offsets = nullptr;
    uint64_t blocks_cap = 0;
    uint32_t* d_err = nullptr;
    unsigned long long* d_visits = nullptr;
    uint32_t* d_sel_hist = nullptr;  // digit histogram of the count cap's radix selection
    // sphere lists handed from voxels to their children (3D FP32 mask pass, RefineArgs): lists and counts of the
    // voxels of vox[i], the parent of each voxel of vox[i]
    uint32_t* lists[2] = {nullptr, nullptr};
    uint8_t* lcount[2] = {nullptr, nullptr};
    uint32_t* parents[2] = {nullptr, nullptr};
    uint64_t lists_cap[2] = {0, 0}, parents_cap[2] = {0, 0};
    bool inherit_lists = false;  // rsagpu_algo_set_inherit (measured slower on config 2, so off by default)
    double* d_table = nullptr;  // the radius generator's tabulated transform on the device, or null
    uint8_t* greedy_state = nullptr;  // count cap: the settle's states, kept across the passes
    uint64_t greedy_cap = 0;
    bool lists_ready = false;   // the last mask pass stored lists for the current voxels' parents
    uint64_t placed = 0;              // spheres in the grid
    std::vector<double> mask_ms, mask_bytes, mask_voxels;  // per refine_mask launch
    // candidates
    CandBuffers cand;
    uint32_t* h_counters = nullptr;  // pinned mirror: COUNTERS + MAX_SETTLE + 1
    // schedule
    int form = RSAGPU_FORM_FP64, schedule = RSAGPU_SCHEDULE_HEURISTIC, cap_rule = RSAGPU_CAP_REFERENCE;
    // heuristic defaults tuned on config 2 (a sweep of factor x threshold): a quarter dart per voxel per pass,
    // refine when 99% of the darts miss
    double factor = kDefaultFactor, miss_thr = kDefaultMissThreshold;
    uint64_t min_darts = kDefaultMinDarts, max_darts = kDefaultMaxDarts;
    std::vector<uint16_t> mlp;
    uint16_t* d_mlp = nullptr;      // the weights on the device
    float* d_feat = nullptr;        // features in, two outputs out
    double explore_eps = 0.0;       // probability of taking the other action (training data)
    std::mt19937_64 explore_rng{0};
    // learned-schedule state
    int passes_at_level = 0;
    double prev_miss = 1.0;
    // hit ratio (greedy accepted / darts) of the last round and the class it was drawn for (class_darts)
    double class_hit = 0.0;
    int class_hit_idx = -1;
    double alive_ratio = 1.0;  // survivors of the probe / darts, last round (alive_darts)
    uint64_t level_start_V = 0, prev_level_start_V = 0;
    // state
    bool begun = false;
    bool heads_dirty = false;  // a round stopped before its commit cleared the candidate lists
    bool lazy = false;         // the candidates in the buffers came from the FP32-form darts
    uint64_t seed = 0, round = 0;
    std::vector<TraceRow> trace;
    rsagpu_stats stats{};
    bool timing = false;
    cudaEvent_t ev[12]{};  // [8], [9] bracket the refine_mask launch
    ~rsagpu_algo() {
        cand.release();
        dfree(vox[0]);
        dfree(vox[1]);
        dfree(bin_hist);
        dfree(bin_off);
        dfree(perm);
        dfree(masks);
        dfree(block_counts);
        dfree(block_offsets);
        dfree(d_table);
        dfree(greedy_state);
        for (int i = 0; i < 2; i++) {
            dfree(lists[i]);
            dfree(lcount[i]);
            dfree(parents[i]);
        }
        dfree(d_err);
        dfree(d_visits);
        dfree(d_sel_hist);
        dfree(d_mlp);
        dfree(d_feat);
        if (h_counters) cudaFreeHost(h_counters);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace rsagpu {
namespace host {

// ------------------------------------------------------------------------------------------------
// sphere grid plan: cells of edge c with c sqrt(D) < 2 r_min (at most one accepted centre per cell) and
// a stencil of every cell within 2 r_max (the largest centre distance any decision looks at).
// ------------------------------------------------------------------------------------------------
GridPlan plan_grid(int D, const double* inf, const double* L, double rmin, double rmax) {
    GridPlan P;
    GridArgs& a = P.a;
    int64_t ncells = 1;
    double c[MAX_D];
    for (int d = 0; d < D; d++) {
        int n = 1 + (int)(std::sqrt((double)D) * L[d] / (2 * rmin));
        while (L[d] / n * std::sqrt((double)D) >= 2 * rmin * (1 - 1e-9)) n++;
        a.n[d] = n;
        c[d] = L[d] / n;
        a.inv_c[d] = 1.0 / c[d];
        a.inf[d] = inf[d];
        a.L[d] = L[d];
        ncells *= n;
        if (ncells > (int64_t)1 << 40) raise(RSAGPU_ERR_CAPACITY, "cell grid too large");
    }
    a.ncells = ncells;
    for (int d = 0; d < D; d++) {
        a.c[d] = c[d];
        a.cf[d] = (float)c[d];
    }
    const double R = 2 * rmax;
    int w[MAX_D];
    for (int d = 0; d < D; d++) {
        w[d] = (int)std::floor(R / c[d]) + 1;
        if (w[d] > a.n[d])
            raise(RSAGPU_ERR_ARG, "box too small for radius %g: %d cells along dimension %d", rmax, a.n[d], d);
        if (w[d] > 127) raise(RSAGPU_ERR_CAPACITY, "radius ratio too large for the stencil");
    }
    // offsets o with sum_d (max(0, |o_d| - 1) c_d)^2 <= R^2, sorted by |o|^2 (own cell first)
    std::vector<std::vector<int8_t>> offs;
    std::vector<int> o(D);
    for (int d = 0; d < D; d++) o[d] = -w[d];
    while (true) {
        double lb = 0;
        for (int d = 0; d < D; d++) {
            double t = std::max(0, std::abs(o[d]) - 1) * c[d];
            lb += t * t;
        }
        if (lb <= R * R * (1 + 1e-9)) {
            std::vector<int8_t> v;
            v.reserve(D);
            for (int d = 0; d < D; d++) v.push_back((int8_t)o[d]);
            offs.push_back(v);
        }
        int d = 0;
        for (; d < D; d++) {
            if (++o[d] <= w[d]) break;
            o[d] = -w[d];
        }
        if (d == D) break;
    }
    std::stable_sort(offs.begin(), offs.end(), [](const std::vector<int8_t>& x, const std::vector<int8_t>& y) {
        int nx = 0, ny = 0;
        for (size_t d = 0; d < x.size(); d++) {
            nx += x[d] * x[d];
            ny += y[d] * y[d];
        }
        return nx < ny;
    });
    for (auto& v : offs) P.stencil.insert(P.stencil.end(), v.begin(), v.end());
    a.S = (int)offs.size();
    // the same offsets as rows along dimension 0: for each (o_1..o_{D-1}) the contiguous range of o_0
    // (the bound is monotone in |o_0|), rows ordered by their nearest distance
    {
        std::vector<std::vector<int8_t>> rows;  // {xlo, xhi, o_1..o_{D-1}}
        for (auto& v : offs) {
            bool found = false;
            for (auto& r : rows) {
                bool same = true;
                for (int d = 1; d < D; d++) same &= (r[1 + d] == v[d]);
                if (same) {
                    r[0] = std::min<int8_t>(r[0], v[0]);
                    r[1] = std::max<int8_t>(r[1], v[0]);
                    found = true;
                    break;
                }
            }
            if (!found) {
                std::vector<int8_t> r(D + 1);
                r[0] = r[1] = v[0];
                for (int d = 1; d < D; d++) r[1 + d] = v[d];
                rows.push_back(r);
            }
        }
        auto rest2 = [&](const std::vector<int8_t>& r) {
            double s2 = 0;
            for (int d = 1; d < D; d++) {
                const double t = std::max(0, std::abs((int)r[1 + d]) - 1) * c[d];
                s2 += t * t;
            }
            return s2;
        };
        std::stable_sort(rows.begin(), rows.end(), [&](const std::vector<int8_t>& x, const std::vector<int8_t>& y) {
            return rest2(x) < rest2(y);
        });
        for (auto& r : rows) {
            P.rows.insert(P.rows.end(), r.begin(), r.end());
            P.rows_r2.push_back((float)(rest2(r) * (1 - 1e-6)));  // rounded down: never drops a needed row
        }
        a.R = (int)rows.size();
        a.rmax = rmax;
    }
    {
        // Guard band of the FP32 screen: a bound, with a factor 4 to spare, on |FP32 model - FP64 value| of
        // every squared distance the kernels compare.  Per dimension the model o c_f + (off_s - off_q)
        // errs by at most E (float rounding of c, of the offsets, of the product and of the two sums, and of
        // a voxel length); every difference is below A; the squares and the D-term sum add (D+1) roundings of
        // a quantity below D A^2; the threshold (r_s + r_q)^2 in float adds 8 ulps of (2 r_max)^2.  The voxel
        // offsets of the mask pass come from a fixed-point cell map (error below 2^-31 c) and two more float
        // roundings (the centre's offset, then the origin's = centre's - len / 2): u (4 c + 2 len) more; the
        // FP32-form darts' offsets come from the same kind of map and are covered by the same term.
        const double u = std::ldexp(1.0, -24);
        double cmax = 0;
        int wmax = 0;
        for (int d = 0; d < D; d++) {
            cmax = std::max(cmax, c[d]);
            wmax = std::max(wmax, w[d]);
        }
        const double lmax = (rmax + rmin) / std::sqrt((double)D);  // level-0 voxel length bound
        const double E = u * cmax * (4 * wmax + 8) + u * lmax + u * (4 * cmax + 2 * lmax);
        const double Amax = (wmax + 1) * cmax + lmax;
        const double G = 4 * (D * E * (2 * Amax + E) + (D + 1) * u * D * Amax * Amax + 8 * u * (2 * rmax) * (2 * rmax));
        a.guard = (float)G;
    }
    return P;
}

}  // namespace host
}  // namespace rsagpu

namespace {

void set_device(const rsagpu_domain* d) { CK(cudaSetDevice(d->device)); }

// the radius generator's tabulated transform, copied to the device (or released)
void upload_table(rsagpu_algo* A);

// a continuous radius law draws each dart's radius: r_min + (r_max - r_min) x, the span rounded first as in
// the transform of the reference's RandomRadiusGenerator
void set_dart_radius_law(const rsagpu_radgen& rg, const double* d_table, DartArgs* da) {
    da->rand_radius = rg.uniform ? 1 : 0;
    if (rg.uniform) {
        da->r_lo = rg.u_rmin;
        da->r_span = rg.u_rmax - rg.u_rmin;
        da->phase = rg.u_phase;
        da->rtab = d_table;
        da->ntab = d_table ? (int32_t)rg.table.size() : 0;
    }
}

// ------------------------------------------------------------------------------------------------
// sphere grid: cells of edge c with c sqrt(D) < 2 r_min (at most one accepted centre per cell) and
// a stencil of every cell within 2 r_max (the largest centre distance any decision looks at).
// ------------------------------------------------------------------------------------------------
void build_grid(rsagpu_domain* dom, double rmin, double rmax) {
    const int D = dom->dim;
    SphereGrid& G = dom->grid;
    G.release();
    G.rmin = rmin;
    G.rmax = rmax;
    GridPlan plan = plan_grid(D, dom->inf, dom->L, rmin, rmax);
    GridArgs& a = G.a;
    a = plan.a;
    const int64_t ncells = a.ncells;
    G.stencil = plan.stencil;
    G.rows = plan.rows;
    G.d_stencil = dalloc<int8_t>(G.stencil.size());
    CK(cudaMemcpy(G.d_stencil, G.stencil.data(), G.stencil.size(), cudaMemcpyHostToDevice));
    a.stencil = G.d_stencil;
    G.d_rows = dalloc<int8_t>(G.rows.size());
    CK(cudaMemcpy(G.d_rows, G.rows.data(), G.rows.size(), cudaMemcpyHostToDevice));
    a.rows = G.d_rows;
    G.d_rows_r2 = dalloc<float>(plan.rows_r2.size());
    CK(cudaMemcpy(G.d_rows_r2, plan.rows_r2.data(), plan.rows_r2.size() * sizeof(float), cudaMemcpyHostToDevice));
    a.rows_r2 = G.d_rows_r2;
    // one padding word: the two-word window of occ_bits reads up to word nwords
    const int64_t nwords = (ncells + 31) / 32 + 1;
    a.occ = dalloc<uint32_t>(nwords);
    a.pos = dalloc<double>((uint64_t)ncells * D);
    a.rad = dalloc<double>(ncells);
    a.off = dalloc<float>((uint64_t)ncells * D);
    a.radf = dalloc<float>(ncells);
    a.phase = dalloc<int32_t>(ncells);
    G.head = dalloc<int32_t>(ncells);
    G.cocc = dalloc<uint32_t>(nwords);
    CK(cudaMemset(a.occ, 0, nwords * sizeof(uint32_t)));
    a.bocc = nullptr;
    a.bnew = nullptr;
    G.nbricks = 0;
    if (D == 2 || D == 3) {
        // the same occupancy by bricks of 64 cells (8x8, 4x4x4), for the brick walks
        const int side = D == 2 ? 8 : 4;
        uint64_t nbricks = 1;
        for (int d = 0; d < D; d++) {
            a.nb[d] = (a.n[d] + side - 1) / side;
            nbricks *= (uint64_t)a.nb[d];
        }
        a.bocc = dalloc<unsigned long long>(nbricks);
        CK(cudaMemset(a.bocc, 0, nbricks * sizeof(unsigned long long)));
        G.nbricks = nbricks;
        if (D == 3) {
            // the spheres placed since the last mask pass, for the sphere lists handed to the children
            a.bnew = dalloc<unsigned long long>(nbricks);
            CK(cudaMemset(a.bnew, 0, nbricks * sizeof(unsigned long long)));
        }
    }
    CK(cudaMemset(G.cocc, 0, nwords * sizeof(uint32_t)));
    CK(cudaMemset(G.head, 0xFF, ncells * sizeof(int32_t)));
    G.ready = true;
}

void ensure_cand(rsagpu_algo* A, uint64_t n) {
    CandBuffers& C = A->cand;
    const int D = A->dom->dim;
    if (!C.a.counters) {
        C.a.counters = dalloc<uint32_t>(COUNTERS + MAX_SETTLE + 1);
        A->h_counters = nullptr;
        CK(cudaMallocHost(&A->h_counters, H_COUNTERS * sizeof(uint32_t)));
    }
    if (n <= C.cap) return;
    uint32_t* keep = C.a.counters;
    C.a.counters = nullptr;
    const uint64_t grown = C.cap + C.cap / 2;  // geometric growth: few reallocations in a run of growing rounds
    C.release();
    C.a.counters = keep;
    const uint64_t cap = std::max<uint64_t>({n, 1024, std::min<uint64_t>(grown, 0x7fffffffull)});
    if (cap > 0x7fffffffull) raise(RSAGPU_ERR_CAPACITY, "more than 2^31 candidates in one round");
    C.a.pos = dalloc<double>(cap * D);
    C.a.key = dalloc<uint64_t>(cap);
    C.a.rad = dalloc<double>(cap);
    C.a.phase = dalloc<int32_t>(cap);
    C.a.cell = dalloc<int64_t>(cap);
    C.a.state = dalloc<uint8_t>((cap + 3) & ~3ull);  // whole 32-bit words (the count cap's CAS on them)
    C.a.next = dalloc<int32_t>(cap);
    C.a.alive = dalloc<uint32_t>(cap);
    C.a.blk = dalloc<int32_t>(cap * NB);
    C.a.nblk = dalloc<uint8_t>(cap);
    C.a.gather = dalloc<uint64_t>(cap);
    C.a.off = dalloc<float>(cap * D);
    C.a.radf = dalloc<float>(cap);
    C.a.kc = dalloc<int32_t>(cap * D);
    C.vidx = dalloc<uint64_t>(cap);
    C.cap = cap;
}

CandArgs cand_args(rsagpu_algo* A, uint32_t n) {
    CandArgs c = A->cand.a;
    c.n = n;
    c.head = A->dom->grid.head;
    c.cocc = A->dom->grid.cocc;
    c.und = c.counters + COUNTERS;
    c.lazy = A->lazy ? 1 : 0;
    c.lvox = A->vox[A->cur];
    for (int d = 0; d < A->dom->dim; d++) c.llen[d] = A->len[d];
    // bounded by the grid's rmax, as the search was before (its stencil rows reach no further)
    const double rg = A->dom->grid.a.rmax;
    const double rc = A->cand_rmax > 0 && A->cand_rmax < rg ? A->cand_rmax : rg;
    c.rcmax = rc;
    c.rcmaxf = (float)rc;
    return c;
}

// Rebuilds the domain's grid for a smaller minimal radius with the placed spheres kept: they are extracted on
// the device, the grid is rebuilt (cells for rmin, stencil for rmax), and they re-enter it as accepted
// candidates through the commit kernel.  Spheres of radius >= rmin are more than 2 rmin apart, so each
// new cell still holds at most one of them (checked by the commit kernel).
void regrid(rsagpu_algo* A, double rmin, double rmax) {
    rsagpu_domain* dom = A->dom;
    const GridArgs old = dom->grid.a;
    const int64_t nwords = (old.ncells + 31) / 32;
    const uint64_t nb = (nwords + OCC_BLOCK - 1) / OCC_BLOCK;
    uint32_t* counts = dalloc<uint32_t>(nb);
    uint64_t* offs = dalloc<uint64_t>(nb + 1);
    launch_occ_block_counts(old.occ, nwords, counts, dom->stream);
    launch_scan_blocks(counts, offs, nb, nullptr, dom->stream);
    uint64_t total = 0;
    CK(cudaMemcpyAsync(&total, offs + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, dom->stream));
    CK(cudaStreamSynchronize(dom->stream));
    ensure_cand(A, total);
    CandArgs c = cand_args(A, (uint32_t)total);
    c.lazy = 0;
    if (total) A->ops->extract_write(old, offs, c.pos, c.rad, c.phase, dom->stream);
    CK(cudaStreamSynchronize(dom->stream));
    dfree(counts);
    dfree(offs);
    build_grid(dom, rmin, rmax);
    dom->grid.a.mono = 0;
    dom->grid.a.rmono = 0;
    A->heads_dirty = false;
    A->lists_ready = false;  // the stored lists name cells of the old grid
    if (total == 0) return;
    c.head = dom->grid.head;  // the new grid's candidate lists (the old ones were released)
    c.cocc = dom->grid.cocc;
    CK(cudaMemsetAsync(c.counters, 0, (COUNTERS + MAX_SETTLE + 1) * sizeof(uint32_t), A->stream));
    A->ops->locate(dom->grid.a, c, A->stream);
    const uint32_t n32 = (uint32_t)total;
    CK(cudaMemcpyAsync(c.counters, &n32, sizeof(uint32_t), cudaMemcpyHostToDevice, A->stream));
    A->ops->commit(dom->grid.a, c, A->stream);
    CK(cudaMemcpyAsync(A->h_counters, c.counters, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaStreamSynchronize(A->stream));
    if (A->h_counters[2] & ERR_DOUBLE_OCCUPANCY) raise(RSAGPU_ERR_INVARIANT, "regrid: two centres in one cell");
    if (A->h_counters[1] != total) raise(RSAGPU_ERR_INVARIANT, "regrid: %u of %llu spheres put back",
                                         A->h_counters[1], (unsigned long long)total);
}

// Staged grid of a generator of several radius classes (largest first): the cells are sized for the smallest
// radius placed so far or drawn in the current class, not for the generator's smallest, so that the rounds of
// the large classes walk few cells; the grid is rebuilt with the spheres kept (regrid) when a smaller class
// begins.  Every decision is exact, so the cell size changes no result.
double stage_radius(const rsagpu_radgen& rg) {
    if (rg.uniform) return rg.u_rmin;
    const int last = std::min<int>(rg.idx, (int)rg.r.size() - 1);
    double r = rg.r[0];
    for (int j = 1; j <= last; j++) r = std::min(r, rg.r[j]);
    return r;
}

void stage_grid(rsagpu_algo* A) {
    const double want = stage_radius(A->rg);
    if (want < A->dom->grid.rmin) regrid(A, want, A->dom->grid.rmax);
}

// Voxel list `which` holds at least n voxels (and `reserve`, when it has to grow).
void ensure_vox(rsagpu_algo* A, int which, uint64_t n, uint64_t reserve = 0) {
    const int D = A->dom->dim;
    if (n <= A->vox_cap[which]) return;
    uint64_t cap = std::max<uint64_t>({n, reserve, A->vox_cap[which] + A->vox_cap[which] / 2});
    dfree(A->vox[which]);
    A->vox[which] = dalloc<int64_t>(cap * D);
    A->vox_cap[which] = cap;
}

void ensure_refine_buffers(rsagpu_algo* A, uint64_t V) {
    const uint64_t words = V * A->ops->mask_words;
    if (words > A->masks_cap) {
        dfree(A->masks);
        A->masks_cap = std::max<uint64_t>(words, A->masks_cap + A->masks_cap / 2);
        A->masks = dalloc<uint32_t>(A->masks_cap);
    }
    const uint64_t blocks = (V + 31) / 32 + 1;  // warp counts of the refinement
    const uint64_t oblocks = ((uint64_t)((A->dom->grid.a.ncells + 31) / 32) + OCC_BLOCK - 1) / OCC_BLOCK + 1;
    const uint64_t need = std::max(blocks, oblocks);
    if (need > A->blocks_cap) {
        dfree(A->block_counts);
        dfree(A->block_offsets);
        A->blocks_cap = std::max<uint64_t>(need, A->blocks_cap + A->blocks_cap / 2);
        A->block_counts = dalloc<uint32_t>(A->blocks_cap);
        A->block_offsets = dalloc<uint64_t>(A->blocks_cap + 1);
    }
}

void begin(rsagpu_algo* A) {
    const int D = A->dom->dim;
    A->class_hit_idx = -1;  // no hit ratio yet for the classes of this proceed
    A->alive_ratio = 1.0;   // the first round: every dart may survive
    // list_of_voxels(origin, L, r_max + r_min): n_d = 1 + int(sqrt(D) L_d / diag), len_d = L_d / n_d
    // (list_of_voxels.ixx:11-28, 192-211)
    // the algorithm's r_max is the largest over its radius generators (m_r_max, operator_algorithm.ixx:89-90,
    // 246): after a reset to smaller radii the lattice still uses the first one
    const double diag = A->rmax_algo + A->rg.rmin();
    uint64_t V = 1;
    for (int d = 0; d < D; d++) {
        A->nvox0[d] = 1 + (int)(std::sqrt((double)D) * A->dom->L[d] / diag);
        A->len[d] = A->dom->L[d] / (double)A->nvox0[d];
        V *= (uint64_t)A->nvox0[d];
    }
    // twice the lattice: the list refilled at the second refinement (whose voxels outnumber the lattice's in 3D,
    // 1.5x at r = 0.002) then fits without a reallocation inside the run.  Growing it there cost a fresh mapping
    // of about 3 GB (2.5 ms with the GPU idle), as the memory pool had split the block of the previous run's size.
    // Lattices whose doubled list would pass 16 GB get no headroom.
    const bool headroom = (double)V * (double)D * sizeof(int64_t) * 2.0 <= 16e9;
    ensure_vox(A, 0, V, headroom ? 2 * V : V);
    // the candidate buffers of the run's rounds at once: rounds grow from the survivor-bounded first ones to the
    // voxel-based size of the first refinements (about 0.37 darts per lattice voxel at config 2), and every growth
    // reallocates 15 arrays, at the risk of a fresh mapping with the GPU idle
    if (A->schedule != RSAGPU_SCHEDULE_REFERENCE) {
        const double want = std::min(2.0 * A->factor * (double)V, (double)A->max_darts);
        if (want * 256.0 <= 16e9) ensure_cand(A, (uint64_t)want);
    }
    A->cur = 0;
    A->V = V;
    A->level = 0;
    A->lists_ready = false;
    A->ops->vox_init(A->vox[0], V, A->nvox0, A->stream);
    A->begun = true;
    A->round = 0;
    A->trace.clear();
    A->stats = rsagpu_stats{};
    A->stats.peak_voxels = V;
    A->mask_ms.clear();
    A->mask_bytes.clear();
    A->mask_voxels.clear();
    A->passes_at_level = 0;
    A->prev_miss = 1.0;
    A->level_start_V = V;
    A->prev_level_start_V = 0;
}

// remove_covered + subdivide_uncovered (list_of_voxels.ixx:30-100)
void check_write_bounds(uint32_t err) {
    if (err & ERR_WRITE_BOUNDS) raise(RSAGPU_ERR_INVARIANT, "refinement offsets beyond the output list");
}

void refine(rsagpu_algo* A) {
    const int D = A->dom->dim;
    if (A->V == 0) return;
    for (int d = 0; d < D; d++)
        if ((double)A->nvox0[d] * std::ldexp(1.0, A->level + 1) > 4.0e18)
            raise(RSAGPU_ERR_CAPACITY, "voxel coordinates overflow int64 at level %d", A->level + 1);
    ensure_refine_buffers(A, A->V);
    RefineArgs r{};
    r.V = A->V;
    r.vin = A->vox[A->cur];
    for (int d = 0; d < D; d++) {
        r.len[d] = A->len[d];
        r.nlen[d] = 0.5 * A->len[d];
        if (!voxel_cell_ratio(A->len[d], A->level, A->dom->grid.a.c[d], A->dom->grid.a.n[d], &r.rho_int[d],
                              &r.rho_frac[d]))
            raise(RSAGPU_ERR_CAPACITY, "level %d too deep for the fixed-point cell map", A->level);
    }
    r.level = A->level;
    r.rmin = A->rg.rmin();
    r.masks = A->masks;
    r.warp_counts = A->block_counts;
    r.warp_offsets = A->block_offsets;
    r.err = A->d_err;
    r.survivors = A->d_err + 1;
    r.visits = A->d_visits;
    r.retests = A->d_visits + 1;
    CK(cudaMemsetAsync(r.survivors, 0, sizeof(uint32_t), A->stream));
    CK(cudaMemsetAsync(r.visits, 0, 2 * sizeof(unsigned long long), A->stream));
    // sphere lists handed to the children: the warp-queue pass of 3D FP32 grids at levels >= 1 (op_refine_mask)
    const SphereGrid& G = A->dom->grid;
    const bool qpath = A->form == RSAGPU_FORM_FP32_GUARD && D == 3 && G.a.bocc && G.a.bnew &&
                       G.a.ncells < (1ll << 32) && A->level >= 1;
    const bool record = qpath && A->inherit_lists && A->V * LIST_K < (1ull << 32) && G.a.n[0] >= 2 && G.a.n[1] >= 2;
    const bool inherit = record && A->lists_ready;
    if (record) {
        const int c = A->cur;
        if (A->V * LIST_K > A->lists_cap[c]) {
            dfree(A->lists[c]);
            dfree(A->lcount[c]);
            A->lists_cap[c] = std::max<uint64_t>(A->V * LIST_K, A->lists_cap[c] + A->lists_cap[c] / 2);
            A->lists[c] = dalloc<uint32_t>(A->lists_cap[c]);
            A->lcount[c] = dalloc<uint8_t>(A->lists_cap[c] / LIST_K + 1);
        }
        r.record = 1;
        r.lout = A->lists[c];
        r.nout = A->lcount[c];
        double h = 0;
        for (int d = 0; d < D; d++) h += A->len[d] * A->len[d];
        r.hdiagf = (float)(0.5 * std::sqrt(h) * (1 + 1e-5));
        r.div0 = UINT64_MAX / (uint64_t)G.a.n[0] + 1;
        r.div1 = UINT64_MAX / (uint64_t)G.a.n[1] + 1;
        if (inherit) {
            r.inherit = 1;
            r.lin = A->lists[1 - c];
            r.nin = A->lcount[1 - c];
            r.parent = A->parents[c];
        }
    }
    const uint64_t nb = (A->V + 31) / 32;  // warps
    CK(cudaEventRecord(A->ev[8], A->stream));
    A->ops->refine_mask(A->dom->grid.a, r, A->form == RSAGPU_FORM_FP32_GUARD, A->stream);
    CK(cudaEventRecord(A->ev[9], A->stream));
    // the next pass's new spheres are those placed from now on
    if (G.a.bnew) CK(cudaMemsetAsync(G.a.bnew, 0, G.nbricks * sizeof(unsigned long long), A->stream));
    A->lists_ready = false;
    launch_scan_blocks(A->block_counts, A->block_offsets, nb, nullptr, A->stream);
    uint64_t total = 0;
    uint32_t err_surv[2] = {0, 0};  // error bits (of this mask pass and of the earlier write passes), survivors
    unsigned long long visits = 0, retests = 0;
    CK(cudaMemcpyAsync(&retests, r.retests, sizeof(unsigned long long), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaMemcpyAsync(&total, A->block_offsets + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaMemcpyAsync(err_surv, r.err, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaMemcpyAsync(&visits, r.visits, sizeof(unsigned long long), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaStreamSynchronize(A->stream));
    check_write_bounds(err_surv[0]);
    const uint32_t survivors = err_surv[1];
    A->stats.retests += retests;
    {
        // the mask pass of this launch: its device time and algorithmic bytes (each logical element once:
        // parent coordinates, stencil occupancy bits up to the grid size, visited spheres up to the
        // spheres placed, the child masks)
        float ms = 0;
        cudaEventElapsedTime(&ms, A->ev[8], A->ev[9]);
        const GridArgs& g = A->dom->grid.a;
        const double bits = std::min<double>((double)A->V * g.S, (double)g.ncells);
        const double sph = std::min<double>((double)visits, (double)A->placed);
        // bytes per visited sphere: FP64 centre + radius, or FP32 offsets (+ FP32 radius unless one class)
        const double per_sphere = A->form == RSAGPU_FORM_FP32_GUARD ? 4.0 * D + (g.mono ? 0 : 4) : 8.0 * D + (g.mono ? 0 : 8);
        A->mask_ms.push_back(ms);
        A->mask_voxels.push_back((double)A->V);
        A->mask_bytes.push_back((double)A->V * 8 * D + bits / 8 + sph * per_sphere + (double)A->V * 4 * A->ops->mask_words);
    }
    if (survivors == 0) {
        // remove_covered emptied the list: subdivide_uncovered returns before halving the length
        // (list_of_voxels.ixx:58)
        A->V = 0;
        A->stats.refinements++;
        return;
    }
    const int other = 1 - A->cur;
    ensure_vox(A, other, total);
    r.vout = A->vox[other];
    r.vout_cap = total;
    if (record) {
        if (total > A->parents_cap[other]) {
            dfree(A->parents[other]);
            A->parents_cap[other] = std::max<uint64_t>(total, A->parents_cap[other] + A->parents_cap[other] / 2);
            A->parents[other] = dalloc<uint32_t>(A->parents_cap[other]);
        }
        r.parent_out = A->parents[other];
    }
    // its bound check (ERR_WRITE_BOUNDS in the error word) is read with the next readback of the error word: the
    // next refinement's, or the end of proceed (a write past the list is skipped, never made)
    A->ops->refine_write(r, A->stream);
    A->cur = other;
    A->V = total;
    A->level++;
    A->lists_ready = record;
    for (int d = 0; d < D; d++) A->len[d] = r.nlen[d];
    A->stats.refinements++;
    A->stats.peak_voxels = std::max(A->stats.peak_voxels, total);
}

// Order statistics and rank counts of v = key >> S over keys on the device, by radix selection with 16-bit
// digit histograms (each a pass over the keys and a 256 KB copy, cached per digit prefix).
struct DeviceSelect {
    const uint64_t* keys;
    uint64_t n;
    int S, L;  // value shift, 16-bit digits per value
    uint32_t* d_hist;
    cudaStream_t st;
    std::map<std::pair<int, uint64_t>, std::vector<uint64_t>> cum;  // (level, prefix) -> inclusive prefix sums
    const std::vector<uint64_t>& hist(int level, uint64_t prefix) {
        auto it = cum.find({level, prefix});
        if (it != cum.end()) return it->second;
        const int dshift = 16 * (L - 1 - level);
        const int pshift = level == 0 ? 64 : 16 * (L - level);
        launch_key_digit_hist(keys, n, S, dshift, pshift, prefix, d_hist, st);
        std::vector<uint32_t> h(65536);
        CK(cudaMemcpyAsync(h.data(), d_hist, 65536 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<uint64_t> c(65536);
        uint64_t run = 0;
        for (int d = 0; d < 65536; d++) c[d] = (run += h[d]);
        return cum.emplace(std::make_pair(level, prefix), std::move(c)).first->second;
    }
    // the rank-th smallest value (0-based)
    uint64_t at(uint64_t rank) {
        uint64_t prefix = 0;
        for (int level = 0; level < L; level++) {
            const std::vector<uint64_t>& c = hist(level, prefix);
            const int d = (int)(std::upper_bound(c.begin(), c.end(), rank) - c.begin());
            if (d > 0) rank -= c[d - 1];
            prefix = (prefix << 16) | (uint64_t)d;
        }
        return prefix;
    }
    // the number of values <= t
    uint64_t count_le(uint64_t t) {
        if (L < 4 && (t >> (16 * L)) != 0) return n;
        uint64_t total = 0, prefix = 0;
        for (int level = 0; level < L; level++) {
            const int d = (int)((t >> (16 * (L - 1 - level))) & 0xFFFFu);
            const std::vector<uint64_t>& c = hist(level, prefix);
            if (d > 0) total += c[d - 1];
            if (level == L - 1) total += c[d] - (d > 0 ? c[d - 1] : 0);
            prefix = (prefix << 16) | (uint64_t)d;
        }
        return total;
    }
};

// median_of_medians::find_pivot_for_first_elements with one rank (median_of_medians.ixx:8-157): the pivot
// retain_only_first_elements compares priorities with, from the priorities' order statistics (at) and rank
// counts (count_le of the integer part of a pivot; upper_bound over the sorted priorities in the reference).
// Returns false where the reference throws.
template <class At, class CountLe>
bool reference_pivot(int64_t n, int64_t n_first, At&& at, CountLe&& count_le, double* out) {
    if (n_first > n || n_first <= 0 || n == 0) return false;
    auto pivot_count = [&](double pivot) { return count_le((uint64_t)pivot); };
    const double pct = n_first / (1. * n);
    int64_t piv = (int64_t)(n * pct) - 1;
    int64_t mn = piv, mx = piv + 1;
    if (std::fabs(n * pct - 1 - piv) < 1e-8) mn -= 1;
    if (mn < 0) mn = 0;
    if (std::fabs(n * pct - 1 - piv - 1) < 1e-8) mx += 1;
    if (mx > n - 1) mx = n - 1;
    double cand[2] = {(double)at(mn) - 2.220446049250313e-16, (double)at(mx) + 2.220446049250313e-16};
    if ((uint64_t)cand[1] < (uint64_t)cand[0]) std::swap(cand[0], cand[1]);
    int p = 2;
    for (int i = 0; i < 2; i++)
        if ((uint64_t)n_first <= pivot_count(cand[i])) {
            p = i;
            break;
        }
    if (p == 2) return false;
    double pmax = cand[p], pivot = pmax;
    uint64_t below = pivot_count(pivot);
    if (below != (uint64_t)n_first) {
        if (p == 0) return false;
        const double pmin = cand[p - 1];
        double add = 0.5 * (pmax - pmin);
        for (int j = 0; j < 20; j++) {
            pivot = pmin + add;
            below = pivot_count(pivot);
            if (below == (uint64_t)n_first) break;
            if (below > (uint64_t)n_first) add = 0.5 * std::fabs(add);
            if (below < (uint64_t)n_first) add = -0.5 * std::fabs(add);
        }
    }
    *out = pivot;
    return true;
}

constexpr int MAX_CAP_PASSES = 1000;

// The count cap under the reference rule, on the device: the passes of add_to_sample (operator_algorithm.ixx:
// 383-443).  Each pass classifies its candidates (DimOps::pass_step, find_solve_conflicts) and compares its
// Undecided count with the class count given to the round; the count is passed by value, so every pass sees
// the same one.  Above it, retain_only_first_elements (:475-519) keeps the Undecided priorities up to the pivot
// (median_of_medians.ixx:8-157) and the round ends.  Else the pass is validated (update_sphere_tags), the round
// ends when the count is met exactly, and the Conflict candidates that hit no validated one make the next
// pass.  Without a collision through the periodic boundary the first pass is the greedy set.
//
// The Undecided sets of successive passes are disjoint parts of the greedy set (whose size `greedy` the settle
// found), and without a cut their union is the greedy set.  So once the greedy candidates not yet validated are
// fewer than the count, no later pass can reach the count: every later pass is validated in full and the round
// keeps the greedy set.  The passes stop there, and the greedy states saved before the first pass are restored.
void reference_cap_passes(rsagpu_algo* A, const CandArgs& c, uint64_t max_new, uint64_t greedy, int f32) {
    const DimOps* ops = A->ops;
    const GridArgs& g = A->dom->grid.a;
    uint32_t* h = A->h_counters;
    if (c.n > A->greedy_cap) {
        dfree(A->greedy_state);
        A->greedy_cap = std::max<uint64_t>(c.n, A->greedy_cap + A->greedy_cap / 2);
        A->greedy_state = dalloc<uint8_t>(A->greedy_cap);
    }
    CK(cudaMemcpyAsync(A->greedy_state, c.state, c.n, cudaMemcpyDeviceToDevice, A->stream));
    uint64_t validated = 0;
    CK(cudaMemsetAsync(c.und, 0, (MAX_SETTLE + 1) * sizeof(uint32_t), A->stream));
    ops->pass_begin(c, A->stream);
    for (int pass = 0;; pass++) {
        if (pass >= MAX_CAP_PASSES) raise(RSAGPU_ERR_NO_PROGRESS, "count cap: more than %d passes", MAX_CAP_PASSES);
        A->stats.cap_passes++;
        CK(cudaMemcpyAsync(h + COUNTERS, c.und, sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
        CK(cudaStreamSynchronize(A->stream));
        if (h[COUNTERS] == 0) break;  // no candidate left in the pass
        // the Conflict set: its sources, then the search level by level (frontiers in counters[5], [6])
        CK(cudaMemsetAsync(c.counters + 5, 0, 2 * sizeof(uint32_t), A->stream));
        ops->pass_sources(g, c, f32, A->stream);
        for (int level = 0, from = 0;; level++, from = 1 - from) {
            if (level > MAX_SETTLE)
                raise(RSAGPU_ERR_NO_PROGRESS, "count-cap Conflict search did not end in %d levels", MAX_SETTLE);
            CK(cudaMemcpyAsync(h + 5 + from, c.counters + 5 + from, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               A->stream));
            CK(cudaStreamSynchronize(A->stream));
            const uint32_t nf = h[5 + from];
            if (nf == 0) break;
            CK(cudaMemsetAsync(c.counters + 5 + (1 - from), 0, sizeof(uint32_t), A->stream));
            ops->pass_push(g, c, from, nf, f32, A->stream);
            A->stats.cap_steps++;
        }
        // the greedy on the candidates that are not Conflict, until all are classified
        CK(cudaMemsetAsync(c.und, 0, (MAX_SETTLE + 1) * sizeof(uint32_t), A->stream));
        CK(cudaMemsetAsync(c.und, 0x01, sizeof(uint32_t), A->stream));  // nonzero: the first step runs
        int it = 1;
        while (true) {
            for (int b = 0; b < 4; b++, it++) {
                if (it > MAX_SETTLE)
                    raise(RSAGPU_ERR_NO_PROGRESS, "count-cap pass did not converge in %d iterations", MAX_SETTLE);
                ops->pass_step(g, c, it, f32, A->stream);
                A->stats.cap_steps++;
            }
            CK(cudaMemcpyAsync(h + COUNTERS + it - 1, c.und + it - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               A->stream));
            CK(cudaStreamSynchronize(A->stream));
            if (h[COUNTERS + it - 1] == 0) break;
        }
        CK(cudaMemsetAsync(c.counters + 3, 0, sizeof(uint32_t), A->stream));
        ops->pass_gather(c, A->stream);
        CK(cudaMemcpyAsync(h + 3, c.counters + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
        CK(cudaStreamSynchronize(A->stream));
        const uint64_t nu = h[3];
        if (nu > max_new) {
            DeviceSelect sel{c.gather, nu, 32, 2, A->d_sel_hist, A->stream, {}};
            double pivot = 0;
            if (!reference_pivot((int64_t)nu, (int64_t)max_new, [&](int64_t r) { return sel.at((uint64_t)r); },
                                 [&](uint64_t t) { return sel.count_le(t); }, &pivot))
                raise(RSAGPU_ERR_PIVOT, "count-cap pivot search failed (%llu undecided, cap %llu)",
                      (unsigned long long)nu, (unsigned long long)max_new);
            ops->pass_close(c, CAP_PASS_PIVOT, pivot, A->stream);
            return;
        }
        ops->pass_close(c, CAP_PASS_VALIDATE, 0.0, A->stream);
        if (nu == max_new) break;
        validated += nu;
        if (validated + max_new > greedy) {
            // every later pass is validated in full: the round keeps the greedy set
            CK(cudaMemcpyAsync(c.state, A->greedy_state, c.n, cudaMemcpyDeviceToDevice, A->stream));
            return;
        }
        CK(cudaMemsetAsync(c.und, 0, (MAX_SETTLE + 1) * sizeof(uint32_t), A->stream));
        ops->pass_next(g, c, f32, A->stream);
    }
    ops->pass_close(c, CAP_PASS_END, 0.0, A->stream);
}

void ev_record(rsagpu_algo* A, int i) {
    if (A->timing) CK(cudaEventRecord(A->ev[i], A->stream));
}
float ev_ms(rsagpu_algo* A, int a, int b) {
    float ms = 0;
    if (A->timing) cudaEventElapsedTime(&ms, A->ev[a], A->ev[b]);
    return ms;
}

// One round on candidates already in the buffers (state = UNDECIDED): probe, settle, cap, commit.
// Returns the number accepted.
uint64_t decide_round(rsagpu_algo* A, uint32_t n, uint64_t max_new, bool may_outreach, bool keep_state,
                      uint64_t* n_greedy = nullptr) {
    rsagpu_domain* dom = A->dom;
    const GridArgs& g = dom->grid.a;
    if (A->heads_dirty) {
        // stale list heads would link this round's candidates to indices of an unfinished round
        CK(cudaMemsetAsync(dom->grid.head, 0xFF, g.ncells * sizeof(int32_t), A->stream));
        CK(cudaMemsetAsync(dom->grid.cocc, 0, ((g.ncells + 31) / 32 + 1) * sizeof(uint32_t), A->stream));
        A->heads_dirty = false;
    }
    A->heads_dirty = true;
    CandArgs c = cand_args(A, n);
    const DimOps* ops = A->ops;
    const int f32 = A->form == RSAGPU_FORM_FP32_GUARD;
    ev_record(A, 2);
    ops->probe(g, c, f32, A->stream);
    ev_record(A, 3);
    ops->collect(g, c, f32, A->stream);
    ev_record(A, 10);
    if (A->timing) {
        CK(cudaEventSynchronize(A->ev[10]));
        A->stats.ms_probe += ev_ms(A, 2, 3);
        A->stats.ms_settle += ev_ms(A, 3, 10);  // collect
    }
    int it = 1;
    const int batch = 4;
    while (true) {
        ev_record(A, 10);
        for (int b = 0; b < batch; b++, it++) {
            if (it > MAX_SETTLE) raise(RSAGPU_ERR_NO_PROGRESS, "settle did not converge in %d iterations", MAX_SETTLE);
            ops->settle(g, c, it, f32, A->stream);
        }
        ev_record(A, 11);
        CK(cudaMemcpyAsync(A->h_counters + COUNTERS + it - 1, c.und + it - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           A->stream));
        CK(cudaStreamSynchronize(A->stream));
        if (A->timing) A->stats.ms_settle += ev_ms(A, 10, 11);
        if (A->h_counters[COUNTERS + it - 1] == 0) break;
    }
    // settle iterations actually needed (the first zero counter): counted after the commit's readback
    CK(cudaMemcpyAsync(A->h_counters + H_SETTLE, c.und, sizeof(uint32_t) * it, cudaMemcpyDeviceToHost, A->stream));
    ev_record(A, 4);
    uint64_t greedy = 0;
    if (may_outreach) {
        ops->gather_accepted(c, A->stream);
        CK(cudaMemcpyAsync(A->h_counters + 3, c.counters + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
        CK(cudaStreamSynchronize(A->stream));
        const uint64_t nacc = A->h_counters[3];
        greedy = nacc;
        if (nacc > max_new) {
            // the cap's order statistics by radix selection on the device (no copy or sort of the keys)
            if (!A->d_sel_hist) A->d_sel_hist = dalloc<uint32_t>(65536);
            if (A->cap_rule == RSAGPU_CAP_EXACT) {
                if (max_new > 0) {
                    DeviceSelect sel{c.gather, nacc, 0, 4, A->d_sel_hist, A->stream, {}};
                    ops->cut_accepted(c, 0, 0.0, sel.at(max_new - 1), A->stream);
                } else {
                    ops->cut_accepted(c, 1, -1.0, 0, A->stream);
                }
            } else {
                reference_cap_passes(A, c, max_new, nacc, f32);
            }
        }
    }
    ops->commit(g, c, A->stream);
    A->heads_dirty = false;
    ev_record(A, 5);
    CK(cudaMemcpyAsync(A->h_counters, c.counters, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaStreamSynchronize(A->stream));
    int used = 0;
    while (used < it && A->h_counters[H_SETTLE + used] != 0) used++;
    A->stats.settle_iterations += used;
    A->stats.retests += A->h_counters[4];
    if (n_greedy) *n_greedy = may_outreach ? greedy : A->h_counters[1];
    if (A->h_counters[2] & ERR_DOUBLE_OCCUPANCY)
        raise(RSAGPU_ERR_INVARIANT, "two accepted centres in one grid cell");
    if (A->h_counters[2] & ERR_DART_SLOT) raise(RSAGPU_ERR_INVARIANT, "binned dart order: a bin overflowed");
    (void)keep_state;
    A->placed += A->h_counters[1];
    if (A->timing) A->stats.ms_commit += ev_ms(A, 4, 5);
    return A->h_counters[1];
}

void reset_counters(rsagpu_algo* A) {
    CK(cudaMemsetAsync(A->cand.a.counters, 0, (COUNTERS + MAX_SETTLE + 1) * sizeof(uint32_t), A->stream));
}

// RadiusGenerator::update_placed (radius_generator.ixx:62-68) + the miss-rate rule (operator_algorithm.ixx:
// 140-162, 190-206).  Returns true when no class is left.
int mlp_decide_host(rsagpu_algo* A, const float* feat, bool* refine);

// saturate: a round that placed more spheres than its class still wanted ends the class (the product loop).  The
// reference subtracts in size_t (update_placed), so such an overshoot, which its count-cap pivot can leave, wraps
// the count and the class never ends: its radius is thrown until no voxel is left and the later classes are never
// drawn.  The replay seam keeps that arithmetic (saturate = false).
bool end_round(rsagpu_algo* A, uint64_t n_shots, uint64_t n_new, bool* refined, double thr, uint64_t n_hits,
               TraceRow* row = nullptr, bool saturate = false) {
    rsagpu_radgen& rg = A->rg;
    if (rg.idx < (int)rg.n.size()) {
        rg.n[rg.idx] = saturate && n_new > rg.n[rg.idx] ? 0 : rg.n[rg.idx] - n_new;
        if (rg.n[rg.idx] == 0) {
            rg.idx++;
            if (rg.idx < (int)rg.n.size()) stage_grid(A);
        }
    }
    const bool done = rg.idx >= (int)rg.n.size();
    const double miss = miss_rate(n_shots, n_hits);
    *refined = false;
    bool do_refine = miss > thr;
    if (row) {
        // state features of the learned schedule (documented in rsa_mpi_gb300/schedule.py)
        const int D = A->dom->dim;
        const GridArgs& g = A->dom->grid.a;
        double vol = 1;
        for (int d = 0; d < D; d++) vol *= A->dom->L[d];
        const double r = A->rg.r[std::min<int>(rg.idx, (int)rg.r.size() - 1)];
        uint64_t V0 = 1;
        for (int d = 0; d < D; d++) V0 *= (uint64_t)A->nvox0[d];
        float* f = row->features;
        f[0] = (float)(std::log2((double)A->V + 1) / 32);
        f[1] = (float)A->level / 32;
        f[2] = (float)miss;
        f[3] = (float)(A->passes_at_level > 0 ? A->prev_miss : miss);
        f[4] = (float)std::min(A->passes_at_level, 16) / 16;
        f[5] = (float)(std::log2((double)n_shots + 1) / 32);
        f[6] = (float)(std::log2((double)n_hits + 1) / 32);
        f[7] = (float)(std::log2((double)A->placed + 1) / 32);
        f[8] = (float)(A->placed * ball_volume(D, r) / vol);
        f[9] = (float)D / 8;
        f[10] = (float)(std::log2((double)A->V / (double)A->feat_ncells + 1e-9) / 32);
        f[11] = (float)((double)n_hits / ((double)A->V + 1));
        f[12] = (float)(std::log2((double)V0) / 32);
        f[13] = (float)(A->prev_level_start_V > 0
                            ? (double)A->level_start_V / ((double)A->prev_level_start_V * (double)(1u << D))
                            : 1.0);
        f[14] = miss > thr ? 1.f : 0.f;
        f[15] = 1.f;
        if (A->schedule == RSAGPU_SCHEDULE_LEARNED && !A->mlp.empty()) {
            bool r_mlp = do_refine;
            if (mlp_decide_host(A, f, &r_mlp) == RSAGPU_OK) do_refine = r_mlp;  // else: heuristic fallback
        }
        if (A->explore_eps > 0) {
            std::uniform_real_distribution<double> U(0, 1);
            if (U(A->explore_rng) < A->explore_eps) do_refine = !do_refine;
        }
        if (A->schedule == RSAGPU_SCHEDULE_LEARNED || A->explore_eps > 0) {
            // guard rails neither the network nor exploration may cross: subdividing while more than a tenth
            // of the darts still land multiplies the voxels by nearly 2^D per level (little of them is
            // covered yet); a pass that places nothing must subdivide (or nothing changes)
            if (miss < 0.9) do_refine = false;
            if (miss > 0.999 || A->passes_at_level >= 32) do_refine = true;
        }
        A->prev_miss = miss;
        A->passes_at_level++;
    }
    if (do_refine && A->V > 0) {
        ev_record(A, 6);
        refine(A);
        ev_record(A, 7);
        if (A->timing) {
            CK(cudaEventSynchronize(A->ev[7]));
            A->stats.ms_refine += ev_ms(A, 6, 7);
        }
        *refined = true;
        A->prev_level_start_V = A->level_start_V;
        A->level_start_V = A->V;
        A->passes_at_level = 0;
    }
    return done;
}

int mlp_decide_host(rsagpu_algo* A, const float* feat, bool* refine) {
    if (!A->d_mlp) {
        A->d_mlp = (uint16_t*)dalloc<uint16_t>(A->mlp.size());
        A->d_feat = dalloc<float>(NFEAT + 2);
        CK(cudaMemcpy(A->d_mlp, A->mlp.data(), A->mlp.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpyAsync(A->d_feat, feat, NFEAT * sizeof(float), cudaMemcpyHostToDevice, A->stream));
    const int rc = mlp_decide(A->d_mlp, A->d_feat, A->d_feat + NFEAT, A->stream);
    if (rc != RSAGPU_OK) return rc;
    float y[2];
    CK(cudaMemcpyAsync(y, A->d_feat + NFEAT, 2 * sizeof(float), cudaMemcpyDeviceToHost, A->stream));
    CK(cudaStreamSynchronize(A->stream));
    if (!std::isfinite(y[0]) || !std::isfinite(y[1])) return RSAGPU_ERR_STATE;
    *refine = y[1] < y[0];  // smaller predicted remaining time
    return RSAGPU_OK;
}

double threshold(const rsagpu_algo* A) {
    return A->miss_thr > 0 ? A->miss_thr : reference_miss_threshold(A->dom->dim);
}

uint64_t darts_for(const rsagpu_algo* A) {
    const double V = (double)A->V;
    if (A->schedule == RSAGPU_SCHEDULE_REFERENCE) {
        // E[shots] of compute_nb_shots_voxel (operator_algorithm.ixx:208-223)
        const double I = 0.01 * V;
        const double m = std::min(1.0, A->nbshots / I);
        return std::max<uint64_t>(1, (uint64_t)std::llround(m * I));
    }
    return heuristic_darts(A->factor, A->min_darts, A->max_darts, A->V);
}

void proceed(rsagpu_algo* A, uint64_t seed) {
    rsagpu_domain* dom = A->dom;
    const int D = dom->dim;
    // proceed_voxel builds a fresh level-0 voxel list on every call; placed spheres are kept
    // (operator_algorithm.ixx:89-90, 238-250)
    begin(A);
    A->seed = seed;
    cudaEvent_t t0, t1;
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    CK(cudaEventRecord(t0, A->stream));
    const double thr = threshold(A);
    while (true) {
        if (A->V == 0) {
            A->stats.maximal = 1;
            break;
        }
        if (A->rg.idx >= (int)A->rg.n.size()) break;
        const uint64_t remaining = A->rg.n[A->rg.idx];
        uint64_t C = darts_for(A);
        // no more than 16x the spheres still wanted of this class
        if (A->schedule != RSAGPU_SCHEDULE_REFERENCE) {
            C = cap_darts(C, remaining, A->min_darts);
            C = class_darts(C, remaining, A->min_darts, A->class_hit_idx == A->rg.idx ? A->class_hit : 0.0);
            C = alive_darts(C, A->V, A->alive_ratio);
        }
        const bool may = C >= remaining;
        ensure_cand(A, C);
        reset_counters(A);
        DartArgs da{};
        da.n = (uint32_t)C;
        da.V = A->V;
        da.vox = A->vox[A->cur];
        for (int d = 0; d < D; d++) da.len[d] = A->len[d];
        da.seed = seed;
        da.round = A->round++;
        da.radius = A->rg.r[A->rg.idx];
        set_dart_radius_law(A->rg, A->d_table, &da);
        da.phase = A->rg.phase[A->rg.idx];
        A->cand_rmax = A->rg.uniform ? A->rg.u_rmax : da.radius;  // every dart of the round has this radius or less
        const auto tp0 = std::chrono::steady_clock::now();
        ev_record(A, 0);
        CandArgs c = cand_args(A, (uint32_t)C);
        {
            // binned order: slot t of the round holds dart perm[t], the darts of each voxel region together
            da.bin_shift = dart_bin_shift(A->V, C);
            const uint64_t nbins = ((A->V - 1) >> da.bin_shift) + 1;
            if (nbins > A->bins_cap) {
                dfree(A->bin_hist);
                dfree(A->bin_off);
                A->bins_cap = std::max<uint64_t>(nbins, A->bins_cap + A->bins_cap / 2);
                A->bin_hist = dalloc<uint32_t>(A->bins_cap);
                A->bin_off = dalloc<uint64_t>(A->bins_cap + 1);
            }
            if (C > A->perm_cap) {
                dfree(A->perm);
                A->perm_cap = std::max<uint64_t>(C, A->perm_cap + A->perm_cap / 2);
                A->perm = dalloc<uint32_t>(A->perm_cap);
            }
            CK(cudaMemsetAsync(A->bin_hist, 0, nbins * sizeof(uint32_t), A->stream));
            da.bin_hist = A->bin_hist;
            da.perm = A->perm;
            A->ops->dart_bins(c, da, A->stream);  // histogram
            launch_scan_blocks(A->bin_hist, A->bin_off, nbins, nullptr, A->stream);
            da.bin_off = A->bin_off;
            A->ops->dart_bins(c, da, A->stream);  // permutation
        }
        if (A->form == RSAGPU_FORM_FP32_GUARD) {
            // FP32 form: lazy candidates (cell and offsets in fixed point, the FP64 position formed in the
            // probe for the candidates that need it)
            for (int d = 0; d < D; d++)
                if (!voxel_cell_ratio(A->len[d], A->level, dom->grid.a.c[d], dom->grid.a.n[d], &da.rho_int[d],
                                      &da.rho_frac[d]))
                    raise(RSAGPU_ERR_CAPACITY, "level %d too deep for the fixed-point cell map", A->level);
            da.level = A->level;
            A->ops->darts32(dom->grid.a, c, da, A->stream);
            A->lazy = true;
        } else {
            A->ops->darts(dom->grid.a, c, da, A->stream);
            A->lazy = false;
        }
        ev_record(A, 1);
        uint64_t n_hits = 0;
        const uint64_t n_new = decide_round(A, (uint32_t)C, remaining, may, false, &n_hits);
        A->class_hit = (double)n_hits / (double)C;
        A->class_hit_idx = A->rg.idx;
        A->alive_ratio = (double)A->h_counters[0] / (double)C;
        if (A->timing) A->stats.ms_darts += ev_ms(A, 0, 1);
        TraceRow row{};
        row.voxels = A->V;
        row.darts = C;
        row.accepted = n_new;
        row.level = A->level;
        const auto tp1 = std::chrono::steady_clock::now();
        bool refined = false;
        // the miss rate of the geometry: darts the count cap dropped are not misses (with 10^7-dart rounds the
        // cap would otherwise read as a miss rate near 1 and refine every round)
        const bool done = end_round(A, C, n_new, &refined, thr, n_hits, &row, true);
        CK(cudaStreamSynchronize(A->stream));
        const auto tp2 = std::chrono::steady_clock::now();
        row.pass_ms = std::chrono::duration<double, std::milli>(tp1 - tp0).count();
        row.refine_ms = std::chrono::duration<double, std::milli>(tp2 - tp1).count();
        row.refined = refined;
        A->trace.push_back(row);
        A->stats.rounds++;
        A->stats.darts += C;
        A->stats.accepted += n_new;
        if (done) break;
    }
    CK(cudaEventRecord(t1, A->stream));
    CK(cudaEventSynchronize(t1));
    if (A->d_err) {
        uint32_t err = 0;
        CK(cudaMemcpy(&err, A->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        check_write_bounds(err);
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    A->stats.ms_total += ms;
    A->stats.final_level = A->level;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
}

void upload_table(rsagpu_algo* A) {
    dfree(A->d_table);
    A->d_table = nullptr;
    const std::vector<double>& t = A->rg.table;
    if (t.empty()) return;
    A->d_table = dalloc<double>(t.size());
    CK(cudaMemcpy(A->d_table, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
}

uint64_t count_spheres(rsagpu_domain* dom, rsagpu_algo* helper_none) {
    (void)helper_none;
    const GridArgs& g = dom->grid.a;
    if (!dom->grid.ready) return 0;
    const int64_t nwords = (g.ncells + 31) / 32;
    const uint64_t nb = (nwords + OCC_BLOCK - 1) / OCC_BLOCK;
    uint32_t* counts = dalloc<uint32_t>(nb);
    uint64_t* offs = dalloc<uint64_t>(nb + 1);
    launch_occ_block_counts(g.occ, nwords, counts, dom->stream);
    launch_scan_blocks(counts, offs, nb, nullptr, dom->stream);
    uint64_t total = 0;
    CK(cudaMemcpyAsync(&total, offs + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, dom->stream));
    CK(cudaStreamSynchronize(dom->stream));
    dfree(counts);
    dfree(offs);
    return total;
}

rsagpu_radgen* make_radgen(int dim, const double* r, const uint64_t* n, const int* ph, int k, double excl) {
    if (dim < 2 || dim > MAX_D) raise(RSAGPU_ERR_ARG, "dimension %d not supported (2..%d)", dim, MAX_D);
    if (k <= 0) raise(RSAGPU_ERR_ARG, "Empty radius generator!");
    // the exclusion distance widens the first radius (below); a negative one could put it under the next
    // class's radius, and the grid and the one-radius shortcut take the radii in descending order
    if (!(excl >= 0)) raise(RSAGPU_ERR_ARG, "exclusion distance must be non-negative");
    auto* rg = new rsagpu_radgen();
    rg->dim = dim;
    std::vector<int> order(k);
    for (int i = 0; i < k; i++) order[i] = i;
    // descending radius (radius_generator.ixx:17-20)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return r[a] > r[b]; });
    for (int i : order) {
        if (!(r[i] > 0)) {
            delete rg;
            raise(RSAGPU_ERR_ARG, "radius must be positive");
        }
        rg->r.push_back(r[i]);
        rg->n.push_back(n[i]);
        rg->phase.push_back(ph ? ph[i] : 0);
    }
    // exclusion distance added to entry 0 once per class (radius_generator.ixx:23-25)
    for (int i = 0; i < k; i++) rg->r[0] += 0.5 * excl;
    rg->excl = excl;
    return rg;
}

}  // namespace

namespace rsagpu {
void set_last_error(const char* msg) { g_err = msg ? msg : ""; }
}  // namespace rsagpu

// ================================================================================================
// C ABI
// ================================================================================================
extern "C" {

const char* rsagpu_last_error(void) { return g_err.c_str(); }
const char* rsagpu_version(void) { return "rsagpu 0.1 (sm_103a)"; }
uint64_t rsagpu_kernel_launches(void) { return kernel_launch_count(); }

int rsagpu_domain_create(int dim, const double* inf, const double* sup, double rad_max, rsagpu_domain** out) {
    return guarded([&] {
        if (!out || !inf || !sup) raise(RSAGPU_ERR_ARG, "null argument");
        if (dim < 2 || dim > MAX_D) raise(RSAGPU_ERR_ARG, "dimension %d not supported (2..%d)", dim, MAX_D);
        if (!(rad_max > 0)) raise(RSAGPU_ERR_ARG, "rad_max must be positive");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            raise(RSAGPU_ERR_CUDA, "no CUDA device");
        }
        auto* d = new rsagpu_domain();
        d->dim = dim;
        cudaGetDevice(&d->device);
        for (int i = 0; i < dim; i++) {
            d->inf[i] = inf[i];
            d->sup[i] = sup[i];
            d->L[i] = sup[i] - inf[i];
            // rsa_grid_traversal::define / check_sufficiently_large (rsa_grid_traversal.ixx:20-23,
            // rsa_domain.ixx:135-143)
            if (!(d->L[i] >= 2 * rad_max)) {
                delete d;
                raise(RSAGPU_ERR_ARG, "Too small domain wrt ghost layer");
            }
        }
        d->rad_max = rad_max;
        CK(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking));
        *out = d;
    });
}

int rsagpu_domain_destroy(rsagpu_domain* dom) {
    return guarded([&] {
        if (!dom) return;
        set_device(dom);
        if (dom->stream) cudaStreamDestroy(dom->stream);
        delete dom;
    });
}

int rsagpu_domain_total_volume(const rsagpu_domain* dom, double* out) {
    return guarded([&] {
        if (!dom || !out) raise(RSAGPU_ERR_ARG, "null argument");
        double v = 1;
        for (int d = 0; d < dom->dim; d++) v *= dom->L[d];
        *out = v;
    });
}

int rsagpu_domain_count(rsagpu_domain* dom, uint64_t* out) {
    return guarded([&] {
        if (!dom || !out) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(dom);
        *out = count_spheres(dom, nullptr);
    });
}

int rsagpu_domain_spheres_volume(rsagpu_domain* dom, double* out) {
    return guarded([&] {
        if (!dom || !out) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(dom);
        *out = 0;
        if (!dom->grid.ready) return;
        const int nb = 1024;
        double* partials = dalloc<double>(nb);
        dim_ops(dom->dim)->volume_partials(dom->grid.a, unit_ball_volume(dom->dim), partials, nb, dom->stream);
        std::vector<double> h(nb);
        CK(cudaMemcpyAsync(h.data(), partials, nb * sizeof(double), cudaMemcpyDeviceToHost, dom->stream));
        CK(cudaStreamSynchronize(dom->stream));
        dfree(partials);
        double s = 0;
        for (double x : h) s += x;
        *out = s;
    });
}

int rsagpu_domain_extract(rsagpu_domain* dom, double* centers, double* radii, int* phases, uint64_t cap,
                          uint64_t* n_out) {
    return guarded([&] {
        if (!dom || !n_out) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(dom);
        *n_out = 0;
        if (!dom->grid.ready) return;
        const GridArgs& g = dom->grid.a;
        const int D = dom->dim;
        const int64_t nwords = (g.ncells + 31) / 32;
        const uint64_t nb = (nwords + OCC_BLOCK - 1) / OCC_BLOCK;
        uint32_t* counts = dalloc<uint32_t>(nb);
        uint64_t* offs = dalloc<uint64_t>(nb + 1);
        launch_occ_block_counts(g.occ, nwords, counts, dom->stream);
        launch_scan_blocks(counts, offs, nb, nullptr, dom->stream);
        uint64_t total = 0;
        CK(cudaMemcpyAsync(&total, offs + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, dom->stream));
        CK(cudaStreamSynchronize(dom->stream));
        *n_out = total;
        if (cap < total || (!centers && !radii && !phases)) {
            dfree(counts);
            dfree(offs);
            return;
        }
        // outputs in pinned host memory that the device can store to at the same address: written there directly
        // (no device staging, no copies)
        auto mapped = [](const void* p) {
            if (!p) return true;
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            return at.type == cudaMemoryTypeHost && at.devicePointer == p;
        };
        if (mapped(centers) && mapped(radii) && mapped(phases)) {
            dim_ops(D)->extract_direct(g, offs, centers, radii, phases, dom->stream);
            CK(cudaStreamSynchronize(dom->stream));
            dfree(counts);
            dfree(offs);
            return;
        }
        double* dp = centers ? dalloc<double>(total * D) : nullptr;
        double* dr = radii ? dalloc<double>(total) : nullptr;
        int32_t* dph = phases ? dalloc<int32_t>(total) : nullptr;
        dim_ops(D)->extract_write(g, offs, dp, dr, dph, dom->stream);
        if (centers) CK(cudaMemcpyAsync(centers, dp, total * D * sizeof(double), cudaMemcpyDeviceToHost, dom->stream));
        if (radii) CK(cudaMemcpyAsync(radii, dr, total * sizeof(double), cudaMemcpyDeviceToHost, dom->stream));
        if (phases) CK(cudaMemcpyAsync(phases, dph, total * sizeof(int32_t), cudaMemcpyDeviceToHost, dom->stream));
        CK(cudaStreamSynchronize(dom->stream));
        dfree(dp);
        dfree(dr);
        dfree(dph);
        dfree(counts);
        dfree(offs);
    });
}

int rsagpu_domain_check(rsagpu_domain* dom, uint64_t* overlapping_pairs, uint64_t* misplaced) {
    return guarded([&] {
        if (!dom) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(dom);
        uint64_t h[2] = {0, 0};
        if (dom->grid.ready) {
            unsigned long long* d = dalloc<unsigned long long>(2);
            CK(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), dom->stream));
            dim_ops(dom->dim)->check(dom->grid.a, d, d + 1, dom->stream);
            CK(cudaMemcpyAsync(h, d, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, dom->stream));
            CK(cudaStreamSynchronize(dom->stream));
            dfree(d);
        }
        if (overlapping_pairs) *overlapping_pairs = h[0];
        if (misplaced) *misplaced = h[1];
    });
}

int rsagpu_radgen_create_counts(int dim, const double* radii, const uint64_t* counts, const int* phases,
                                int n_classes, double exclusion_distance, rsagpu_radgen** out) {
    return guarded([&] {
        if (!out || !radii || !counts) raise(RSAGPU_ERR_ARG, "null argument");
        *out = make_radgen(dim, radii, counts, phases, n_classes, exclusion_distance);
    });
}

int rsagpu_radgen_create_fractions(int dim, const double* radii, const double* fractions, const int* phases,
                                   int n_classes, double volume, double exclusion_distance, rsagpu_radgen** out) {
    return guarded([&] {
        if (!out || !radii || !fractions) raise(RSAGPU_ERR_ARG, "null argument");
        if (n_classes <= 0) raise(RSAGPU_ERR_ARG, "Empty radius generator!");
        std::vector<uint64_t> n(n_classes);
        // compute_desired_radius_nb_phase (radius_generator.ixx:71-86)
        for (int i = 0; i < n_classes; i++) n[i] = (uint64_t)(volume * fractions[i] / ball_volume(dim, radii[i]));
        *out = make_radgen(dim, radii, n.data(), phases, n_classes, exclusion_distance);
    });
}

int rsagpu_radgen_create_uniform(int dim, double r_min, double r_max, uint64_t count, int phase,
                                 rsagpu_radgen** out) {
    return guarded([&] {
        if (!out) raise(RSAGPU_ERR_ARG, "null argument");
        if (!(r_min > 0) || !(r_max >= r_min)) raise(RSAGPU_ERR_ARG, "need 0 < r_min <= r_max");
        if (dim < 2 || dim > MAX_D) raise(RSAGPU_ERR_ARG, "dimension %d not supported (2..%d)", dim, MAX_D);
        auto* rg = new rsagpu_radgen();
        rg->dim = dim;
        rg->r.push_back(0.0);
        rg->n.push_back(count);
        rg->phase.push_back(0);
        rg->uniform = true;
        rg->u_rmin = r_min;
        rg->u_rmax = r_max;
        rg->u_phase = phase;
        *out = rg;
    });
}

int rsagpu_radgen_create_table(int dim, const double* knots, int n_knots, uint64_t count, int phase,
                               rsagpu_radgen** out) {
    return guarded([&] {
        if (!out || !knots) raise(RSAGPU_ERR_ARG, "null argument");
        if (dim < 2 || dim > MAX_D) raise(RSAGPU_ERR_ARG, "dimension %d not supported (2..%d)", dim, MAX_D);
        if (n_knots < 2 || n_knots > (1 << 20)) raise(RSAGPU_ERR_ARG, "need 2 to 2^20 knots, got %d", n_knots);
        double lo = knots[0], hi = knots[0];
        for (int j = 0; j < n_knots; j++) {
            if (!(knots[j] > 0) || !std::isfinite(knots[j])) raise(RSAGPU_ERR_ARG, "radius must be positive");
            lo = std::min(lo, knots[j]);
            hi = std::max(hi, knots[j]);
        }
        auto* rg = new rsagpu_radgen();
        rg->dim = dim;
        rg->r.push_back(0.0);
        rg->n.push_back(count);
        rg->phase.push_back(0);
        rg->uniform = true;
        rg->u_rmin = lo;
        rg->u_rmax = hi;
        rg->u_phase = phase;
        rg->table.assign(knots, knots + n_knots);
        *out = rg;
    });
}

int rsagpu_radgen_destroy(rsagpu_radgen* rg) {
    delete rg;
    return RSAGPU_OK;
}

int rsagpu_radgen_max_radius(const rsagpu_radgen* rg, double* out) {
    if (!rg || !out) return fail(RSAGPU_ERR_ARG, "null argument");
    *out = rg->rmax();
    return RSAGPU_OK;
}

int rsagpu_radgen_min_radius(const rsagpu_radgen* rg, double* out) {
    if (!rg || !out) return fail(RSAGPU_ERR_ARG, "null argument");
    *out = rg->rmin();
    return RSAGPU_OK;
}

int rsagpu_algo_create(rsagpu_domain* dom, const rsagpu_radgen* rg, int nbshots, rsagpu_algo** out) {
    return guarded([&] {
        if (!dom || !rg || !out) raise(RSAGPU_ERR_ARG, "null argument");
        if (rg->dim != dom->dim) raise(RSAGPU_ERR_ARG, "radius generator and domain dimensions differ");
        // operator_algorithm.ixx:27-29
        if (rg->rmax() > dom->rad_max)
            raise(RSAGPU_ERR_ARG,
                  "Impossible to have the maximal radius of radius generator larger than domain implicit radius");
        set_device(dom);
        auto* A = new rsagpu_algo();
        try {
            A->dom = dom;
            A->rg = *rg;
            A->rg.idx = 0;
            A->nbshots = nbshots;
            A->rmax_algo = rg->rmax();
            A->ops = dim_ops(dom->dim);
            if (!A->ops) raise(RSAGPU_ERR_ARG, "dimension not built");
            CK(cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
            for (auto& e : A->ev) CK(cudaEventCreate(&e));
            A->d_err = dalloc<uint32_t>(2);
            CK(cudaMemset(A->d_err, 0, 2 * sizeof(uint32_t)));
            A->d_visits = dalloc<unsigned long long>(2);
            // the algo rebuilds the domain's grid and drops its spheres (operator_algorithm.ixx:25-26); the
            // grid of the first class (stage_grid), which holds one radius only
            const double rmax = std::max(rg->rmax(), 0.0);
            A->feat_rmin = rg->rmin();
            A->feat_ncells = plan_grid(dom->dim, dom->inf, dom->L, A->feat_rmin, rmax).a.ncells;
            build_grid(dom, stage_radius(A->rg), rmax);
            dom->grid.a.mono = !rg->uniform;
            dom->grid.a.rmono = rg->r.front();
            A->placed = 0;
            ensure_cand(A, 1024);
            upload_table(A);
        } catch (...) {
            delete A;
            throw;
        }
        *out = A;
    });
}

int rsagpu_algo_destroy(rsagpu_algo* algo) {
    return guarded([&] {
        if (!algo) return;
        set_device(algo->dom);
        delete algo;
    });
}

int rsagpu_algo_set_form(rsagpu_algo* algo, int form, int schedule) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (form != RSAGPU_FORM_FP64 && form != RSAGPU_FORM_FP32_GUARD) raise(RSAGPU_ERR_ARG, "unknown form %d", form);
        if (schedule < 0 || schedule > RSAGPU_SCHEDULE_REFERENCE) raise(RSAGPU_ERR_ARG, "unknown schedule %d", schedule);
        algo->form = form;
        algo->schedule = schedule;
    });
}

int rsagpu_algo_set_inherit(rsagpu_algo* algo, int on) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        algo->inherit_lists = on != 0;
        if (!on) algo->lists_ready = false;
    });
}

int rsagpu_algo_set_cap_rule(rsagpu_algo* algo, int rule) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (rule != RSAGPU_CAP_REFERENCE && rule != RSAGPU_CAP_EXACT) raise(RSAGPU_ERR_ARG, "unknown cap rule");
        algo->cap_rule = rule;
    });
}

int rsagpu_algo_set_schedule_params(rsagpu_algo* algo, double factor, uint64_t min_darts, uint64_t max_darts,
                                    double miss_threshold) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (!(factor > 0) || min_darts == 0 || max_darts < min_darts || max_darts > 0x7fffffffull)
            raise(RSAGPU_ERR_ARG, "invalid schedule parameters");
        algo->factor = factor;
        algo->min_darts = min_darts;
        algo->max_darts = max_darts;
        algo->miss_thr = miss_threshold;
    });
}

int rsagpu_algo_set_mlp(rsagpu_algo* algo, const uint16_t* w, uint64_t n) {
    return guarded([&] {
        if (!algo || !w) raise(RSAGPU_ERR_ARG, "null argument");
        if (n != 5378) raise(RSAGPU_ERR_ARG, "expected 5378 weights, got %llu", (unsigned long long)n);
        algo->mlp.assign(w, w + n);
        dfree(algo->d_mlp);
        dfree(algo->d_feat);
    });
}

int rsagpu_algo_kernel_profile(rsagpu_algo* algo, double* ms, double* bytes, double* voxels, uint64_t cap,
                               uint64_t* n_out) {
    if (!algo || !n_out) return fail(RSAGPU_ERR_ARG, "null argument");
    *n_out = algo->mask_ms.size();
    for (uint64_t i = 0; i < std::min<uint64_t>(cap, algo->mask_ms.size()); i++) {
        if (ms) ms[i] = algo->mask_ms[i];
        if (bytes) bytes[i] = algo->mask_bytes[i];
        if (voxels) voxels[i] = algo->mask_voxels[i];
    }
    return RSAGPU_OK;
}

int rsagpu_algo_set_exploration(rsagpu_algo* algo, double epsilon, uint64_t seed) {
    if (!algo || !(epsilon >= 0 && epsilon <= 1)) return fail(RSAGPU_ERR_ARG, "invalid exploration");
    algo->explore_eps = epsilon;
    algo->explore_rng.seed(seed);
    return RSAGPU_OK;
}

int rsagpu_algo_trace_features(rsagpu_algo* algo, float* features, uint8_t* refined, double* pass_ms,
                               double* refine_ms, uint64_t cap, uint64_t* n_out) {
    if (!algo || !n_out) return fail(RSAGPU_ERR_ARG, "null argument");
    *n_out = algo->trace.size();
    const uint64_t n = std::min<uint64_t>(cap, algo->trace.size());
    for (uint64_t i = 0; i < n; i++) {
        const TraceRow& t = algo->trace[i];
        if (features)
            for (int k = 0; k < NFEAT; k++) features[i * NFEAT + k] = t.features[k];
        if (refined) refined[i] = t.refined;
        if (pass_ms) pass_ms[i] = t.pass_ms;
        if (refine_ms) refine_ms[i] = t.refine_ms;
    }
    return RSAGPU_OK;
}

int rsagpu_algo_set_timing(rsagpu_algo* algo, int on) {
    if (!algo) return fail(RSAGPU_ERR_ARG, "null argument");
    algo->timing = on != 0;
    return RSAGPU_OK;
}

int rsagpu_algo_proceed(rsagpu_algo* algo, uint64_t seed) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(algo->dom);
        proceed(algo, seed);
    });
}

int rsagpu_algo_reset_radgen(rsagpu_algo* algo, const rsagpu_radgen* rg) {
    return guarded([&] {
        if (!algo || !rg) raise(RSAGPU_ERR_ARG, "null argument");
        // operator_algorithm.ixx:238-250
        if (algo->rg.rmax() < rg->rmax()) raise(RSAGPU_ERR_ARG, "Incorrect maximal radius");
        set_device(algo->dom);
        algo->rmax_algo = std::max(algo->rmax_algo, rg->rmax());
        algo->rg = *rg;
        algo->rg.idx = 0;
        upload_table(algo);
        // a smaller radius needs smaller cells (one centre per cell): regrid, keeping the spheres
        stage_grid(algo);
        if (rg->rmin() < algo->feat_rmin) {
            algo->feat_rmin = rg->rmin();
            algo->feat_ncells =
                plan_grid(algo->dom->dim, algo->dom->inf, algo->dom->L, algo->feat_rmin, algo->dom->grid.rmax).a.ncells;
        }
        algo->begun = false;
        // spheres of the previous generator keep their radii: the grid's one-radius shortcut holds only if
        // the new generator has the same single radius
        GridArgs& ga = algo->dom->grid.a;
        ga.mono = ga.mono && rg->r.size() == 1 && !rg->uniform && rg->r.front() == ga.rmono;
    });
}

int rsagpu_algo_trace(rsagpu_algo* algo, uint64_t* voxels, uint64_t* darts, uint64_t* accepted, uint8_t* refined,
                      int32_t* level, uint64_t cap, uint64_t* n_out) {
    if (!algo || !n_out) return fail(RSAGPU_ERR_ARG, "null argument");
    *n_out = algo->trace.size();
    const uint64_t n = std::min<uint64_t>(cap, algo->trace.size());
    for (uint64_t i = 0; i < n; i++) {
        const TraceRow& t = algo->trace[i];
        if (voxels) voxels[i] = t.voxels;
        if (darts) darts[i] = t.darts;
        if (accepted) accepted[i] = t.accepted;
        if (refined) refined[i] = t.refined;
        if (level) level[i] = t.level;
    }
    return RSAGPU_OK;
}

int rsagpu_algo_stats(rsagpu_algo* algo, rsagpu_stats* out) {
    if (!algo || !out) return fail(RSAGPU_ERR_ARG, "null argument");
    *out = algo->stats;
    return RSAGPU_OK;
}

int rsagpu_algo_begin(rsagpu_algo* algo) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        set_device(algo->dom);
        begin(algo);
        CK(cudaStreamSynchronize(algo->stream));
    });
}

int rsagpu_algo_replay_round(rsagpu_algo* algo, uint64_t n, const double* pos, const uint64_t* key, const double* rad,
                             const int* phase, uint64_t max_new, int may_outreach, uint8_t* accepted_out,
                             uint64_t* n_new) {
    return guarded([&] {
        if (!algo || !n_new || (n > 0 && (!pos || !key || !rad || !accepted_out)))
            raise(RSAGPU_ERR_ARG, "null argument");
        if (n > 0x7fffffffull) raise(RSAGPU_ERR_CAPACITY, "too many candidates");
        set_device(algo->dom);
        const int D = algo->dom->dim;
        ensure_cand(algo, n);
        reset_counters(algo);
        *n_new = 0;
        if (n == 0) return;
        CandArgs c = cand_args(algo, (uint32_t)n);
        CK(cudaMemcpyAsync(c.pos, pos, n * D * sizeof(double), cudaMemcpyHostToDevice, algo->stream));
        CK(cudaMemcpyAsync(c.key, key, n * sizeof(uint64_t), cudaMemcpyHostToDevice, algo->stream));
        CK(cudaMemcpyAsync(c.rad, rad, n * sizeof(double), cudaMemcpyHostToDevice, algo->stream));
        if (phase) CK(cudaMemcpyAsync(c.phase, phase, n * sizeof(int32_t), cudaMemcpyHostToDevice, algo->stream));
        else CK(cudaMemsetAsync(c.phase, 0, n * sizeof(int32_t), algo->stream));
        CK(cudaMemsetAsync(c.state, ST_UNDECIDED, n, algo->stream));
        algo->lazy = false;  // exact positions given
        double rc = 0;
        for (uint64_t i = 0; i < n; i++) rc = std::max(rc, rad[i]);
        algo->cand_rmax = rc;
        c = cand_args(algo, (uint32_t)n);
        *n_new = decide_round(algo, (uint32_t)n, max_new, may_outreach != 0, true);
        std::vector<uint8_t> st(n);
        CK(cudaMemcpyAsync(st.data(), c.state, n, cudaMemcpyDeviceToHost, algo->stream));
        CK(cudaStreamSynchronize(algo->stream));
        for (uint64_t i = 0; i < n; i++) accepted_out[i] = st[i] == ST_ACCEPTED;
    });
}

int rsagpu_algo_end_round(rsagpu_algo* algo, uint64_t n_shots, uint64_t n_new, int* refined, int* done) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (!algo->begun) raise(RSAGPU_ERR_STATE, "end_round before begin");
        set_device(algo->dom);
        bool r = false;
        const bool dn = end_round(algo, n_shots, n_new, &r, reference_miss_threshold(algo->dom->dim), n_new);
        CK(cudaStreamSynchronize(algo->stream));
        if (r) {
            uint32_t err = 0;
            CK(cudaMemcpy(&err, algo->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            check_write_bounds(err);
        }
        if (refined) *refined = r;
        if (done) *done = dn;
    });
}

int rsagpu_algo_refine(rsagpu_algo* algo) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (!algo->begun) raise(RSAGPU_ERR_STATE, "refine before begin");
        set_device(algo->dom);
        refine(algo);
        CK(cudaStreamSynchronize(algo->stream));
        uint32_t err = 0;
        CK(cudaMemcpy(&err, algo->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        check_write_bounds(err);
    });
}

int rsagpu_algo_voxels(rsagpu_algo* algo, int64_t* coords, uint64_t cap, uint64_t* count, int32_t* level,
                       double* length) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (!algo->begun) raise(RSAGPU_ERR_STATE, "voxels before begin");
        set_device(algo->dom);
        const int D = algo->dom->dim;
        if (count) *count = algo->V;
        if (level) *level = algo->level;
        if (length)
            for (int d = 0; d < D; d++) length[d] = algo->len[d];
        if (coords && cap >= algo->V && algo->V > 0) {
            CK(cudaMemcpyAsync(coords, algo->vox[algo->cur], algo->V * D * sizeof(int64_t), cudaMemcpyDeviceToHost,
                               algo->stream));
            CK(cudaStreamSynchronize(algo->stream));
        }
    });
}

int rsagpu_algo_draw_darts(rsagpu_algo* algo, uint64_t seed, uint64_t round, uint64_t n, double* pos, uint64_t* key,
                           uint64_t* voxel_index) {
    return guarded([&] {
        if (!algo) raise(RSAGPU_ERR_ARG, "null argument");
        if (!algo->begun) raise(RSAGPU_ERR_STATE, "draw before begin");
        if (algo->V == 0) raise(RSAGPU_ERR_STATE, "Impossible to draw centers in no voxels");
        if (n > 0x7fffffffull) raise(RSAGPU_ERR_CAPACITY, "too many darts");
        set_device(algo->dom);
        const int D = algo->dom->dim;
        ensure_cand(algo, n);
        if (n == 0) return;
        DartArgs da{};
        da.n = (uint32_t)n;
        da.V = algo->V;
        da.vox = algo->vox[algo->cur];
        for (int d = 0; d < D; d++) da.len[d] = algo->len[d];
        da.seed = seed;
        da.round = round;
        da.radius = algo->rg.r[std::min<int>(algo->rg.idx, (int)algo->rg.r.size() - 1)];
        set_dart_radius_law(algo->rg, algo->d_table, &da);
        da.phase = 0;
        da.vidx_out = algo->cand.vidx;
        CandArgs c = cand_args(algo, (uint32_t)n);
        algo->ops->darts(algo->dom->grid.a, c, da, algo->stream);
        algo->lazy = false;
        if (pos) CK(cudaMemcpyAsync(pos, c.pos, n * D * sizeof(double), cudaMemcpyDeviceToHost, algo->stream));
        if (key) CK(cudaMemcpyAsync(key, c.key, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, algo->stream));
        if (voxel_index)
            CK(cudaMemcpyAsync(voxel_index, algo->cand.vidx, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, algo->stream));
        CK(cudaStreamSynchronize(algo->stream));
    });
}

}  // extern "C"
