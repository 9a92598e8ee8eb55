// batch.cu -- rsagpu_batch_run: many independent one-radius instances, each run to certified maximality.
//
// The reference runs one domain per process (rsa_algo::proceed_voxel, operator_algorithm.ixx:85-188);
// thousands of small domains would each pay a full round of launches per pass.  Here the instances of
// one dimension advance together: a round is one launch sequence over the darts, candidates and voxels
// of every unfinished instance of a wave, and the waves are sized to a device-memory budget.  Each
// instance keeps its own sphere grid, voxel list, Philox key, round counter and schedule state, so it
// places exactly the spheres of its single-instance run (a domain [0, sup], one radius class of volume
// fraction 1, rsagpu_algo_proceed(seed), the default schedule, the same form).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/rsagpu.h"
#include "host_common.h"
#include "rsa_device.cuh"
#include "rsa_ops.h"

using namespace rsagpu;
using namespace rsagpu::host;

namespace {

constexpr int B_COUNTERS = 8;  // [0] alive, [1] accepted, [2] error bits, [3] unused, [4] FP64 retests
constexpr int B_MAX_SETTLE = 4096;
constexpr double PEAK_VOXELS_PER_LEVEL0 = 2.5;  // measured peak / level-0 voxels is 1.4 to 2.4 in 3D

using Clock = std::chrono::steady_clock;

struct Inst {
    int user = 0;  // index in the caller's array
    int D = 0;
    double L[MAX_D]{};
    double r = 0;
    uint64_t seed = 0;
    GridPlan plan;
    uint64_t cells = 0;  // ncells rounded up to 32
    int64_t nvox0[MAX_D]{};
    uint64_t V0 = 0;
    uint64_t target = 0;  // spheres wanted: volume fraction 1 (never reached, so the count cap never binds)
    double est_bytes = 0;
    // run state
    uint64_t V = 0, remaining = 0, placed = 0, C = 0;
    double alive_ratio = 1.0;  // survivors of the probe / darts in the instance's last round (alive_darts)
    int level = 0;
    double len[MAX_D]{};
    bool refine = false;
    bool done = false;
    double t_done = 0;
    uint64_t count = 0, checksum = 0;
};

// device buffers of one wave; freed when it goes out of scope
struct Wave {
    uint32_t* occ = nullptr;
    unsigned long long* bocc = nullptr;  // 2D / 3D: brick occupancy of every instance
    double* pos = nullptr;
    float* off = nullptr;
    int32_t* head = nullptr;
    uint32_t* cocc = nullptr;
    int8_t* rows = nullptr;
    float* rows_r2 = nullptr;
    void* table = nullptr;
    BatchRound* rnd = nullptr;
    uint64_t* dart_off = nullptr;
    uint64_t* vox_off = nullptr;
    uint64_t* new_off = nullptr;
    uint64_t* word_off = nullptr;
    uint32_t* acc = nullptr;
    uint32_t* alive_inst = nullptr;
    unsigned long long* counts = nullptr;
    unsigned long long* sums = nullptr;
    int64_t* vox[2] = {nullptr, nullptr};
    uint64_t vox_cap[2] = {0, 0};
    uint32_t* masks = nullptr;
    uint64_t masks_cap = 0;
    uint32_t* bin_hist = nullptr;  // binned dart order
    uint64_t* bin_off = nullptr;
    uint64_t bins_cap = 0;
    uint32_t* warp_counts = nullptr;
    uint64_t* warp_offsets = nullptr;
    uint64_t warps_cap = 0;
    uint32_t* err = nullptr;  // [0] refine error bits, [1] survivors
    unsigned long long* visits = nullptr;  // [0] visits, [1] retests
    // candidates
    CandArgs c{};
    uint32_t* cinst = nullptr;
    uint32_t* perm = nullptr;  // binned dart order
    uint64_t cand_cap = 0;
    ~Wave() {
        dfree(occ);
        dfree(bocc);
        dfree(pos);
        dfree(off);
        dfree(head);
        dfree(cocc);
        dfree(rows);
        dfree(rows_r2);
        dfree(table);
        dfree(rnd);
        dfree(dart_off);
        dfree(vox_off);
        dfree(new_off);
        dfree(word_off);
        dfree(acc);
        dfree(alive_inst);
        dfree(counts);
        dfree(sums);
        dfree(vox[0]);
        dfree(vox[1]);
        dfree(masks);
        dfree(bin_hist);
        dfree(bin_off);
        dfree(warp_counts);
        dfree(warp_offsets);
        dfree(err);
        dfree(visits);
        free_cand();
        dfree(c.counters);
    }
    void free_cand() {
        dfree(c.pos);
        dfree(c.key);
        dfree(c.rad);
        dfree(c.phase);
        dfree(c.cell);
        dfree(c.state);
        dfree(c.next);
        dfree(c.alive);
        dfree(c.off);
        dfree(c.radf);
        dfree(c.kc);
        dfree(c.blk);
        dfree(c.nblk);
        dfree(cinst);
        dfree(perm);
        cand_cap = 0;
    }
};

// per-candidate bytes of the round buffers
double cand_bytes(int D, bool f32) {
    return 8.0 * D + 8 + 8 + 4 + 8 + 1 + 4 + 4 + 4.0 * NB + 1 + 4 + (f32 ? 8.0 * D : 0.0);
}

void ensure_cand(Wave& W, int D, bool f32, uint64_t n) {
    if (n <= W.cand_cap) return;
    W.free_cand();
    const uint64_t cap = std::max<uint64_t>(n + n / 4, 4096);
    if (cap > 0x7fffffffull) raise(RSAGPU_ERR_CAPACITY, "more than 2^31 darts in one round of a wave");
    W.c.pos = dalloc<double>(cap * D);
    W.c.key = dalloc<uint64_t>(cap);
    W.c.rad = dalloc<double>(cap);
    W.c.phase = dalloc<int32_t>(cap);
    W.c.cell = dalloc<int64_t>(cap);
    W.c.state = dalloc<uint8_t>(cap);
    W.c.next = dalloc<int32_t>(cap);
    W.c.alive = dalloc<uint32_t>(cap);
    if (f32) {
        W.c.off = dalloc<float>(cap * D);
        W.c.radf = dalloc<float>(cap);
        W.c.kc = dalloc<int32_t>(cap * D);
    }
    W.c.blk = dalloc<int32_t>(cap * NB);
    W.c.nblk = dalloc<uint8_t>(cap);
    W.cinst = dalloc<uint32_t>(cap);
    W.perm = dalloc<uint32_t>(cap);
    W.cand_cap = cap;
}

void ensure_vox(Wave& W, int D, int which, uint64_t n) {
    if (n <= W.vox_cap[which]) return;
    const uint64_t cap = std::max<uint64_t>(n, W.vox_cap[which] + W.vox_cap[which] / 2);
    dfree(W.vox[which]);
    W.vox[which] = dalloc<int64_t>(cap * D);
    W.vox_cap[which] = cap;
}

void ensure_refine(Wave& W, int mask_words, uint64_t V) {
    if (V * mask_words > W.masks_cap) {
        dfree(W.masks);
        W.masks_cap = std::max<uint64_t>(V * mask_words, W.masks_cap + W.masks_cap / 2);
        W.masks = dalloc<uint32_t>(W.masks_cap);
    }
    const uint64_t warps = (V + 31) / 32 + 1;
    if (warps > W.warps_cap) {
        dfree(W.warp_counts);
        dfree(W.warp_offsets);
        W.warps_cap = std::max<uint64_t>(warps, W.warps_cap + W.warps_cap / 2);
        W.warp_counts = dalloc<uint32_t>(W.warps_cap);
        W.warp_offsets = dalloc<uint64_t>(W.warps_cap + 1);
    }
}

// ------------------------------------------------------------------------------------------------
// block-shape autotuner.  probe, collect and settle rotate through the candidate shapes over the first
// rounds in a palindromic order (so the cost drift from round to round cancels to first order) and
// keep the cheapest time per item; the voxel mask pass, which is a pure function of its inputs, is run
// once per shape on the first subdivision and keeps the fastest.  Outputs never depend on the shape.
// ------------------------------------------------------------------------------------------------
struct Tuner {
    static constexpr int NS = 3;
    static constexpr int shapes[NS] = {128, 256, 512};
    static constexpr int SEQ = 6;
    static constexpr int seq[SEQ] = {0, 1, 2, 2, 1, 0};
    bool enabled = true;
    int best[4] = {-1, -1, -1, -1};  // probe, collect, settle, refine mask
    double cost[4][NS] = {};
    int step[3] = {0, 0, 0};
    int pick(int k) const {
        if (!enabled) return 256;
        if (best[k] >= 0) return shapes[best[k]];
        return shapes[seq[step[k]]];
    }
    void record(int k, double ms, double items) {
        if (!enabled || best[k] >= 0 || items <= 0) return;
        cost[k][seq[step[k]]] += ms / items;
        if (++step[k] == SEQ) best[k] = (int)(std::min_element(cost[k], cost[k] + NS) - cost[k]);
    }
};
constexpr int Tuner::shapes[Tuner::NS];
constexpr int Tuner::seq[Tuner::SEQ];

struct Events {
    cudaEvent_t e[8]{};
    Events() {
        for (auto& x : e) CK(cudaEventCreate(&x));
    }
    ~Events() {
        for (auto& x : e)
            if (x) cudaEventDestroy(x);
    }
    float ms(int a, int b) const {
        float t = 0;
        cudaEventElapsedTime(&t, e[a], e[b]);
        return t;
    }
};

struct RunStats {
    uint64_t rounds = 0, darts = 0, retests = 0, settle_iterations = 0, peak_voxels = 0;
};

// Runs one wave (instances of one dimension) to maximality.
void run_wave(int D, const DimOps* ops, std::vector<Inst*>& I, bool f32, Tuner& tuner, cudaStream_t st,
              Clock::time_point t0, RunStats& rs) {
    const uint32_t M = (uint32_t)I.size();
    Wave W;
    Events ev;
    // layout of the cell arrays and stencil rows
    std::vector<uint64_t> word_off(M + 1, 0), vox_off(M + 1, 0);
    std::vector<uint64_t> rows_base(M), r2_base(M), brick_off(M + 1, 0);
    uint64_t rows_total = 0, r2_total = 0;
    const bool bricks = D == 2 || D == 3;
    const int side = D == 2 ? 8 : 4;  // bricks of 64 cells, as the single-instance grids
    for (uint32_t s = 0; s < M; s++) {
        uint64_t nbr = 1;
        for (int d = 0; d < D && bricks; d++) nbr *= (uint64_t)((I[s]->plan.a.n[d] + side - 1) / side);
        brick_off[s + 1] = brick_off[s] + (bricks ? nbr : 0);
        word_off[s + 1] = word_off[s] + I[s]->cells / 32;
        vox_off[s + 1] = vox_off[s] + I[s]->V0;
        rows_base[s] = rows_total;
        r2_base[s] = r2_total;
        rows_total += I[s]->plan.rows.size();
        r2_total += I[s]->plan.rows_r2.size();
    }
    const uint64_t nwords = word_off[M];
    const uint64_t ncells = nwords * 32;
    W.occ = dalloc<uint32_t>(nwords + 1);  // + the padding word of occ_bits' two-word window
    W.cocc = dalloc<uint32_t>(nwords + 1);
    W.pos = dalloc<double>(ncells * D);
    if (f32) W.off = dalloc<float>(ncells * D);
    W.head = dalloc<int32_t>(ncells);
    CK(cudaMemsetAsync(W.occ, 0, (nwords + 1) * sizeof(uint32_t), st));
    if (bricks) {
        W.bocc = dalloc<unsigned long long>(brick_off[M]);
        CK(cudaMemsetAsync(W.bocc, 0, brick_off[M] * sizeof(unsigned long long), st));
    }
    CK(cudaMemsetAsync(W.cocc, 0, (nwords + 1) * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(W.head, 0xFF, ncells * sizeof(int32_t), st));
    {
        std::vector<int8_t> rows(rows_total);
        std::vector<float> r2(r2_total);
        for (uint32_t s = 0; s < M; s++) {
            std::copy(I[s]->plan.rows.begin(), I[s]->plan.rows.end(), rows.begin() + rows_base[s]);
            std::copy(I[s]->plan.rows_r2.begin(), I[s]->plan.rows_r2.end(), r2.begin() + r2_base[s]);
        }
        W.rows = dalloc<int8_t>(rows_total);
        W.rows_r2 = dalloc<float>(r2_total);
        CK(cudaMemcpy(W.rows, rows.data(), rows_total, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(W.rows_r2, r2.data(), r2_total * sizeof(float), cudaMemcpyHostToDevice));
    }
    std::vector<BatchInstance> tab(M);
    for (uint32_t s = 0; s < M; s++) {
        BatchInstance& b = tab[s];
        b.g = I[s]->plan.a;
        const uint64_t cell0 = word_off[s] * 32;
        b.g.occ = W.occ + word_off[s];
        b.g.pos = W.pos + cell0 * D;
        b.g.rad = nullptr;  // one radius: no per-cell radius, FP32 radius or phase arrays
        b.g.radf = nullptr;
        b.g.phase = nullptr;
        b.g.off = f32 ? W.off + cell0 * D : nullptr;
        b.g.stencil = nullptr;
        b.g.rows = W.rows + rows_base[s];
        b.g.rows_r2 = W.rows_r2 + r2_base[s];
        b.g.mono = 1;
        b.g.rmono = I[s]->r;
        b.g.bocc = bricks ? W.bocc + brick_off[s] : nullptr;
        for (int d = 0; d < D && bricks; d++) b.g.nb[d] = (I[s]->plan.a.n[d] + side - 1) / side;
        b.head = W.head + cell0;
        b.cocc = W.cocc + word_off[s];
        b.seed = I[s]->seed;
        for (int d = 0; d < D; d++) b.nvox0[d] = I[s]->nvox0[d];
    }
    W.table = dalloc<char>(ops->batch_table_bytes(M));
    {
        const int e = ops->batch_table_fill(tab.data(), M, W.table, st);
        if (e != 0) raise(RSAGPU_ERR_CUDA, "instance table copy failed: %s", cudaGetErrorString((cudaError_t)e));
    }
    W.rnd = dalloc<BatchRound>(M);
    W.dart_off = dalloc<uint64_t>(M + 1);
    W.vox_off = dalloc<uint64_t>(M + 1);
    W.new_off = dalloc<uint64_t>(M + 1);
    W.word_off = dalloc<uint64_t>(M + 1);
    W.acc = dalloc<uint32_t>(M);
    W.alive_inst = dalloc<uint32_t>(M);
    W.counts = dalloc<unsigned long long>(M);
    W.sums = dalloc<unsigned long long>(M);
    W.err = dalloc<uint32_t>(2);
    W.visits = dalloc<unsigned long long>(2);
    W.c.counters = dalloc<uint32_t>(B_COUNTERS + B_MAX_SETTLE + 1);
    CK(cudaMemcpy(W.vox_off, vox_off.data(), (M + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(W.word_off, word_off.data(), (M + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CK(cudaMemset(W.err, 0, 2 * sizeof(uint32_t)));

    BatchArgs b{};
    b.M = M;
    b.table = W.table;
    b.rnd = W.rnd;
    b.dart_off = W.dart_off;
    b.vox_off = W.vox_off;
    b.word_off = W.word_off;
    b.cinst = nullptr;
    b.acc = W.acc;
    b.alive_inst = W.alive_inst;
    b.nwords = nwords;
    b.occ = W.occ;
    b.pos = W.pos;
    // level-0 voxels (list_of_voxels.ixx:11-28), one segment per instance
    int cur = 0;
    uint64_t Vtot = vox_off[M];
    ensure_vox(W, D, 0, Vtot);
    b.V = Vtot;
    ops->b_vox_init(b, W.vox[0], st);
    rs.peak_voxels = std::max(rs.peak_voxels, Vtot);

    std::vector<BatchRound> rnd(M);
    std::vector<uint64_t> dart_off(M + 1);
    uint32_t* h_acc = nullptr;
    uint32_t* h_cnt = nullptr;
    uint64_t* h_off = nullptr;
    CK(cudaMallocHost(&h_acc, 2 * (size_t)M * sizeof(uint32_t)));  // accepted, then survivors, per instance
    uint32_t* h_alive = h_acc + M;
    struct HostFree {
        void* p;
        ~HostFree() {
            if (p) cudaFreeHost(p);
        }
    } f1{h_acc};
    CK(cudaMallocHost(&h_cnt, (B_COUNTERS + B_MAX_SETTLE + 1) * sizeof(uint32_t)));
    HostFree f2{h_cnt};
    CK(cudaMallocHost(&h_off, (M + 1) * sizeof(uint64_t)));
    HostFree f3{h_off};
    const int f = f32 ? 1 : 0;

    for (uint64_t round = 0;; round++) {
        // schedule of every unfinished instance (the single-instance proceed loop)
        bool any = false;
        for (uint32_t s = 0; s < M; s++) {
            Inst& x = *I[s];
            x.C = 0;
            x.refine = false;
            if (x.done) continue;
            any = true;
            x.C = cap_darts(heuristic_darts(kDefaultFactor, kDefaultMinDarts, kDefaultMaxDarts, x.V), x.remaining,
                            kDefaultMinDarts);
            x.C = alive_darts(x.C, x.V, x.alive_ratio);
        }
        if (!any) break;
        dart_off[0] = 0;
        for (uint32_t s = 0; s < M; s++) {
            Inst& x = *I[s];
            dart_off[s + 1] = dart_off[s] + x.C;
            rnd[s].vbase = vox_off[s];
            rnd[s].V = x.V;
            for (int d = 0; d < D; d++) {
                rnd[s].len[d] = x.len[d];
                rnd[s].nlen[d] = 0.5 * x.len[d];
                if (!voxel_cell_ratio(x.len[d], x.level, x.plan.a.c[d], x.plan.a.n[d], &rnd[s].rho_int[d],
                                      &rnd[s].rho_frac[d]))
                    raise(RSAGPU_ERR_CAPACITY, "instance %d: level %d too deep for the fixed-point cell map", x.user,
                          x.level);
            }
            rnd[s].level = x.level;
            rnd[s].refine = 0;
        }
        const uint64_t ndarts = dart_off[M];
        ensure_cand(W, D, f32, ndarts);
        CK(cudaMemcpyAsync(W.rnd, rnd.data(), M * sizeof(BatchRound), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(W.dart_off, dart_off.data(), (M + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(W.c.counters, 0, (B_COUNTERS + B_MAX_SETTLE + 1) * sizeof(uint32_t), st));
        CK(cudaMemsetAsync(W.acc, 0, M * sizeof(uint32_t), st));
        CK(cudaMemsetAsync(W.alive_inst, 0, M * sizeof(uint32_t), st));
        CandArgs c = W.c;
        c.n = (uint32_t)ndarts;
        c.head = nullptr;  // per instance, from the table
        c.cocc = nullptr;
        c.und = c.counters + B_COUNTERS;
        c.gather = nullptr;
        b.cinst = W.cinst;
        b.round = round;
        b.ndarts = ndarts;
        b.vox = W.vox[cur];
        b.V = Vtot;
        c.lazy = f32 ? 1 : 0;  // FP32 form: lazy candidates (positions formed in the probe when needed)
        {
            // binned order over the wave's voxel list: the darts are written grouped by voxel region
            b.bin_shift = dart_bin_shift(Vtot, ndarts);
            const uint64_t nbins = ((Vtot - 1) >> b.bin_shift) + 1;
            if (nbins > W.bins_cap) {
                dfree(W.bin_hist);
                dfree(W.bin_off);
                W.bins_cap = std::max<uint64_t>(nbins, W.bins_cap + W.bins_cap / 2);
                W.bin_hist = dalloc<uint32_t>(W.bins_cap);
                W.bin_off = dalloc<uint64_t>(W.bins_cap + 1);
            }
            CK(cudaMemsetAsync(W.bin_hist, 0, nbins * sizeof(uint32_t), st));
            b.bin_hist = W.bin_hist;
            b.bin_off = nullptr;
            b.perm = W.perm;
            ops->b_dart_bins(b, c, st);  // histogram
            launch_scan_blocks(W.bin_hist, W.bin_off, nbins, nullptr, st);
            b.bin_off = W.bin_off;
            ops->b_dart_bins(b, c, st);  // permutation
        }
        ops->b_darts(b, c, f, st);
        const int bp = tuner.pick(0), bc = tuner.pick(1), bs = tuner.pick(2);
        CK(cudaEventRecord(ev.e[0], st));
        ops->b_probe(b, c, f, bp, st);
        CK(cudaEventRecord(ev.e[1], st));
        ops->b_collect(b, c, f, bc, st);
        CK(cudaEventRecord(ev.e[2], st));
        // settle to the fixpoint (each iteration returns at once when the last one left nothing undecided)
        int it = 1;
        while (true) {
            for (int k = 0; k < 4; k++, it++) {
                if (it > B_MAX_SETTLE)
                    raise(RSAGPU_ERR_NO_PROGRESS, "settle did not converge in %d iterations", B_MAX_SETTLE);
                ops->b_settle(b, c, it, f, bs, st);
            }
            CK(cudaMemcpyAsync(h_cnt + B_COUNTERS + it - 1, c.und + it - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               st));
            CK(cudaStreamSynchronize(st));
            if (h_cnt[B_COUNTERS + it - 1] == 0) break;
        }
        CK(cudaEventRecord(ev.e[3], st));
        ops->b_commit(b, c, st);
        CK(cudaMemcpyAsync(h_cnt, c.counters, B_COUNTERS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(h_acc, W.acc, M * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(h_alive, W.alive_inst, M * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (h_cnt[2] & ERR_DOUBLE_OCCUPANCY) raise(RSAGPU_ERR_INVARIANT, "two accepted centres in one grid cell");
        if (h_cnt[2] & ERR_DART_SLOT) raise(RSAGPU_ERR_INVARIANT, "binned dart order: a bin overflowed");
        {
            const double alive = (double)h_cnt[0];
            tuner.record(0, ev.ms(0, 1), (double)ndarts);
            tuner.record(1, ev.ms(1, 2), alive);
            tuner.record(2, ev.ms(2, 3), alive);
        }
        rs.rounds++;
        rs.darts += ndarts;
        rs.retests += h_cnt[4];
        // end of round per instance (RadiusGenerator::update_placed and the miss-rate rule)
        bool any_refine = false;
        for (uint32_t s = 0; s < M; s++) {
            Inst& x = *I[s];
            if (x.done) continue;
            const uint64_t a = h_acc[s];
            x.alive_ratio = x.C ? (double)h_alive[s] / (double)x.C : 1.0;
            if (a > x.remaining)
                raise(RSAGPU_ERR_STATE, "instance %d: the count cap binds (batched instances target fraction 1)",
                      x.user);
            x.remaining -= a;
            x.placed += a;
            if (miss_rate(x.C, a) > kDefaultMissThreshold && x.V > 0) {
                for (int d = 0; d < D; d++)
                    if ((double)x.nvox0[d] * std::ldexp(1.0, x.level + 1) > 4.0e18)
                        raise(RSAGPU_ERR_CAPACITY, "instance %d: voxel coordinates overflow int64 at level %d",
                              x.user, x.level + 1);
                x.refine = true;
                rnd[s].refine = 1;
                any_refine = true;
            }
        }
        if (any_refine) {
            CK(cudaMemcpyAsync(W.rnd, rnd.data(), M * sizeof(BatchRound), cudaMemcpyHostToDevice, st));
            ensure_refine(W, ops->mask_words, Vtot);
            RefineArgs ra{};
            ra.V = Vtot;
            ra.vin = W.vox[cur];
            ra.masks = W.masks;
            ra.warp_counts = W.warp_counts;
            ra.warp_offsets = W.warp_offsets;
            ra.err = W.err;
            ra.survivors = W.err + 1;
            ra.visits = W.visits;
            ra.retests = W.visits + 1;
            if (tuner.enabled && tuner.best[3] < 0) {
                // the mask pass is a pure function of its inputs: time each shape on the same data
                float best_ms = 0;
                for (int k = 0; k < Tuner::NS; k++) {
                    CK(cudaEventRecord(ev.e[4], st));
                    ops->b_refine_mask(b, ra, f, Tuner::shapes[k], st);
                    CK(cudaEventRecord(ev.e[5], st));
                    CK(cudaEventSynchronize(ev.e[5]));
                    const float ms = ev.ms(4, 5);
                    if (k == 0 || ms < best_ms) {
                        best_ms = ms;
                        tuner.best[3] = k;
                    }
                }
            }
            CK(cudaMemsetAsync(W.visits, 0, 2 * sizeof(unsigned long long), st));
            ops->b_refine_mask(b, ra, f, tuner.enabled ? Tuner::shapes[tuner.best[3]] : 256, st);
            const uint64_t nwarps = (Vtot + 31) / 32;
            launch_scan_blocks(W.warp_counts, W.warp_offsets, nwarps, nullptr, st);
            ops->b_refine_offsets(b, ra, W.new_off, st);
            unsigned long long rt = 0;
            CK(cudaMemcpyAsync(h_off, W.new_off, (M + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(&rt, W.visits + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            rs.retests += rt;
            const uint64_t total = h_off[M];
            const int other = 1 - cur;
            ensure_vox(W, D, other, total);
            ra.vout = W.vox[other];
            ra.vout_cap = total;
            ops->b_refine_write(b, ra, st);
            {
                uint32_t err = 0;
                CK(cudaMemcpyAsync(&err, W.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                if (err & ERR_WRITE_BOUNDS) raise(RSAGPU_ERR_INVARIANT, "refinement offsets beyond the output list");
            }
            cur = other;
            Vtot = total;
            std::swap(W.vox_off, W.new_off);
            b.vox_off = W.vox_off;
            for (uint32_t s = 0; s <= M; s++) vox_off[s] = h_off[s];
            for (uint32_t s = 0; s < M; s++) {
                Inst& x = *I[s];
                x.V = vox_off[s + 1] - vox_off[s];
                if (x.refine && x.V > 0) {
                    x.level++;
                    for (int d = 0; d < D; d++) x.len[d] = 0.5 * x.len[d];
                }
            }
            rs.peak_voxels = std::max(rs.peak_voxels, Vtot);
        }
        const double now = std::chrono::duration<double>(Clock::now() - t0).count();
        for (uint32_t s = 0; s < M; s++) {
            Inst& x = *I[s];
            if (!x.done && x.V == 0) {
                x.done = true;
                x.t_done = now;
            }
        }
    }
    // per-instance results
    CK(cudaMemsetAsync(W.counts, 0, M * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(W.sums, 0, M * sizeof(unsigned long long), st));
    ops->b_results(b, W.counts, W.sums, st);
    std::vector<unsigned long long> cnt(M), sum(M);
    CK(cudaMemcpyAsync(cnt.data(), W.counts, M * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(sum.data(), W.sums, M * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (uint32_t s = 0; s < M; s++) {
        I[s]->count = cnt[s];
        I[s]->checksum = sum[s];
        if (cnt[s] != I[s]->placed)
            raise(RSAGPU_ERR_INVARIANT, "instance %d: %llu spheres in the grid, %llu accepted", I[s]->user,
                  (unsigned long long)cnt[s], (unsigned long long)I[s]->placed);
    }
}

}  // namespace

extern "C" {

int rsagpu_batch_run(const rsagpu_instance_desc* inst, int n, int form, uint64_t max_bytes, int autotune,
                     uint64_t* counts_out, uint64_t* checksums_out, double* seconds_out,
                     rsagpu_batch_stats* stats_out) {
    return guarded([&] {
        if (n < 0 || (n > 0 && !inst)) raise(RSAGPU_ERR_ARG, "null instance array");
        if (form != RSAGPU_FORM_FP64 && form != RSAGPU_FORM_FP32_GUARD) raise(RSAGPU_ERR_ARG, "unknown form %d", form);
        const auto t0 = Clock::now();
        const uint64_t launches0 = kernel_launch_count();
        const bool f32 = form == RSAGPU_FORM_FP32_GUARD;
        std::vector<Inst> all(n);
        for (int i = 0; i < n; i++) {
            Inst& x = all[i];
            const rsagpu_instance_desc& d = inst[i];
            if (d.dim < 2 || d.dim > MAX_D) raise(RSAGPU_ERR_ARG, "instance %d: dimension %d not supported", i, d.dim);
            if (!(d.radius > 0)) raise(RSAGPU_ERR_ARG, "instance %d: radius must be positive", i);
            x.user = i;
            x.D = d.dim;
            x.r = d.radius;
            x.seed = d.seed;
            double vol = 1;
            const double zero[MAX_D] = {};
            for (int k = 0; k < d.dim; k++) {
                x.L[k] = d.sup[k];
                if (!(x.L[k] >= 2 * d.radius))
                    raise(RSAGPU_ERR_ARG, "instance %d: box side %g below twice the radius", i, x.L[k]);
                vol *= x.L[k];
            }
            x.plan = plan_grid(d.dim, zero, x.L, d.radius, d.radius);
            x.cells = ((uint64_t)x.plan.a.ncells + 31) / 32 * 32;
            // list_of_voxels(origin, L, r_max + r_min) (list_of_voxels.ixx:11-28, 192-211)
            const double diag = d.radius + d.radius;
            x.V0 = 1;
            for (int k = 0; k < d.dim; k++) {
                x.nvox0[k] = 1 + (int)(std::sqrt((double)d.dim) * x.L[k] / diag);
                x.len[k] = x.L[k] / (double)x.nvox0[k];
                x.V0 *= (uint64_t)x.nvox0[k];
            }
            // compute_desired_radius_nb_phase with volume fraction 1 (radius_generator.ixx:71-86)
            x.target = (uint64_t)(vol * 1.0 / ball_volume(d.dim, d.radius));
            x.remaining = x.target;
            x.alive_ratio = 1.0;
            x.V = x.V0;
            const int D = d.dim;
            const double Vpeak = PEAK_VOXELS_PER_LEVEL0 * (double)x.V0;
            const double mw = (double)(((1 << D) + 31) / 32);
            x.est_bytes = (double)x.cells * (8.0 * D + (f32 ? 4.0 * D : 0.0) + 4 + 0.25) +
                          Vpeak * (16.0 * D + 4 * mw + 0.25) +
                          std::max(kDefaultFactor * Vpeak, (double)kDefaultMinDarts) * cand_bytes(D, f32);
        }
        int device = 0;
        CK(cudaGetDevice(&device));
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        // memory the device's pool holds but no allocation uses (freed by earlier runs of this process) is free
        // to the allocations too, though cudaMemGetInfo counts it as used
        uint64_t pool_reserved = 0, pool_used = 0;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &pool_reserved);
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &pool_used);
        }
        cudaGetLastError();
        const double pool_free = pool_reserved > pool_used ? (double)(pool_reserved - pool_used) : 0.0;
        const double budget = max_bytes ? (double)max_bytes : 0.6 * ((double)free_b + pool_free);
        cudaStream_t st = nullptr;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } sg{st};
        RunStats rs;
        uint64_t waves = 0;
        Tuner tuners[MAX_D + 1];
        for (auto& t : tuners) t.enabled = autotune != 0;
        for (int D = 2; D <= MAX_D; D++) {
            std::vector<Inst*> group;
            for (auto& x : all)
                if (x.D == D) group.push_back(&x);
            if (group.empty()) continue;
            const DimOps* ops = dim_ops(D);
            if (!ops) raise(RSAGPU_ERR_ARG, "dimension %d not built", D);
            // largest first; a wave takes instances while the estimate fits the budget
            std::stable_sort(group.begin(), group.end(), [](const Inst* a, const Inst* b) { return a->est_bytes > b->est_bytes; });
            size_t k = 0;
            while (k < group.size()) {
                std::vector<Inst*> wave;
                double bytes = 0;
                while (k < group.size() && (wave.empty() || bytes + group[k]->est_bytes <= budget) &&
                       wave.size() < 65536) {
                    bytes += group[k]->est_bytes;
                    wave.push_back(group[k++]);
                }
                // instances in caller order inside the wave
                std::sort(wave.begin(), wave.end(), [](const Inst* a, const Inst* b) { return a->user < b->user; });
                run_wave(D, ops, wave, f32, tuners[D], st, t0, rs);
                waves++;
            }
        }
        const double secs = std::chrono::duration<double>(Clock::now() - t0).count();
        for (int i = 0; i < n; i++) {
            if (counts_out) counts_out[i] = all[i].count;
            if (checksums_out) checksums_out[i] = all[i].checksum;
            if (seconds_out) seconds_out[i] = all[i].t_done;
        }
        if (stats_out) {
            rsagpu_batch_stats S{};
            S.seconds = secs;
            S.waves = waves;
            S.rounds = rs.rounds;
            S.darts = rs.darts;
            S.retests = rs.retests;
            S.peak_voxels = rs.peak_voxels;
            S.launches = kernel_launch_count() - launches0;
            S.budget_bytes = (uint64_t)budget;
            for (int D = 2; D <= MAX_D; D++) {
                const Tuner& t = tuners[D];
                for (int k = 0; k < 4; k++)
                    if (t.best[k] >= 0) S.block[D][k] = Tuner::shapes[t.best[k]];
            }
            *stats_out = S;
        }
    });
}

}  // extern "C"
