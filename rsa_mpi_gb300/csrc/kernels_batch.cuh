// kernels_batch.cuh -- the batched kernels: every launch covers all unfinished instances of a wave.
//
// Included by kernels.cu inside its per-dimension namespace.  The work per dart, candidate or voxel is the
// single-instance kernels' own device body (dart_body, probe_body, collect_body, settle_body, commit_body,
// refine_mask64_body / refine_mask32_body), applied with the grid of the element's instance, so each
// instance makes exactly the decisions of its single-instance run.  The instance of a dart or voxel is
// found by binary search over the wave's segment offsets; a candidate carries it in cinst.

struct BInst {
    Grid<D> g;
    Geo<D> geo;
    int32_t* head;
    uint32_t* cocc;
    uint32_t seed_lo, seed_hi;
    int64_t nvox0[D];
};

// segment s with off[s] <= x < off[s + 1], given off[0] = 0 <= x < off[M] (empty segments are passed over)
__device__ __forceinline__ uint32_t segment_of(const uint64_t* off, uint32_t M, uint64_t x) {
    uint32_t lo = 0, hi = M;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ CandArgs with_lists(const CandArgs& c, const BInst& I) {
    CandArgs ci = c;
    ci.head = I.head;
    ci.cocc = I.cocc;
    return ci;
}

// level-0 voxels of every instance, in block order within each segment (as k_vox_init)
__global__ void k_b_vox_init(BatchArgs b, int64_t* vox) {
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= b.V) return;
    const BInst* tab = (const BInst*)b.table;
    const uint32_t s = segment_of(b.vox_off, b.M, v);
    int64_t n[D];
#pragma unroll
    for (int d = 0; d < D; d++) n[d] = tab[s].nvox0[d];
    block_order_coords(v - b.vox_off[s], n, vox + v * D);
}

// Slot t of the round holds global dart g = perm[t] (or t): dart (g - dart_off[s]) of instance s, under the
// instance's key (F32: a lazy candidate).
template <bool F32>
__global__ void __launch_bounds__(256) k_b_darts(BatchArgs b, CandArgs c) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.ndarts) return;
    const uint64_t gi = b.perm ? (uint64_t)b.perm[t] % b.ndarts : t;
    const BInst* tab = (const BInst*)b.table;
    const uint32_t s = segment_of(b.dart_off, b.M, gi);
    const BInst& I = tab[s];
    const BatchRound& R = b.rnd[s];
    DartParams p{};
    p.n = 0;
    p.V = R.V;
    p.vox = b.vox + R.vbase * D;
#pragma unroll
    for (int d = 0; d < D; d++) {
        p.len[d] = R.len[d];
        p.inf[d] = I.geo.inf[d];
    }
    p.seed_lo = I.seed_lo;
    p.seed_hi = I.seed_hi;
    p.round_lo = (uint32_t)b.round;
    p.round_hi = (uint32_t)(b.round >> 32);
    p.radius = I.g.rmono;
    p.phase = 0;
    p.pos = c.pos;
    p.key = c.key;
    p.rad = c.rad;
    p.cphase = c.phase;
    p.state = c.state;
    p.vidx_out = nullptr;
    const uint32_t i = (uint32_t)(gi - b.dart_off[s]);
    if constexpr (F32) {
        p.kc = c.kc;
        p.off = c.off;
        p.cell = c.cell;
#pragma unroll
        for (int d = 0; d < D; d++) {
            p.rho_frac[d] = R.rho_frac[d];
            p.rho_int[d] = R.rho_int[d];
            p.ncell[d] = I.g.n[d];
            p.cf[d] = I.g.cf[d];
        }
        p.level = R.level;
        dart32_body(p, i, t);
    } else {
        dart_body(p, i, t);
    }
    b.cinst[t] = s;
}

// binned dart order over the wave's voxel list: pass 1 (histogram) without bin_off, else pass 2 (perm)
__global__ void __launch_bounds__(256) k_b_dart_bins(BatchArgs b, CandArgs c) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.ndarts) return;
    const BInst* tab = (const BInst*)b.table;
    const uint32_t s = segment_of(b.dart_off, b.M, t);
    const BatchRound& R = b.rnd[s];
    DartParams p{};
    p.V = R.V;
    p.seed_lo = tab[s].seed_lo;
    p.seed_hi = tab[s].seed_hi;
    p.round_lo = (uint32_t)b.round;
    p.round_hi = (uint32_t)(b.round >> 32);
    p.vbase = R.vbase;
    p.bin_hist = b.bin_hist;
    p.bin_off = b.bin_off;
    p.bin_shift = b.bin_shift;
    p.perm = b.perm;
    p.err = c.counters + 2;
    const uint32_t i = (uint32_t)(t - b.dart_off[s]);
    if (!b.bin_off) atomicAdd(b.bin_hist + ((R.vbase + dart_voxel(p, i)) >> b.bin_shift), 1u);
    else place_dart(p, i, (uint32_t)t);
}

// the candidate arguments seen by one candidate of instance s: its cell lists, and for a lazy candidate
// the voxel segment and length its exact position comes from
__device__ __forceinline__ CandArgs with_instance(const CandArgs& c, const BatchArgs& b, const BInst& I, uint32_t s) {
    CandArgs ci = with_lists(c, I);
    if (c.lazy) {
        const BatchRound& R = b.rnd[s];
        ci.lvox = b.vox + R.vbase * D;
#pragma unroll
        for (int d = 0; d < D; d++) ci.llen[d] = R.len[d];
    }
    return ci;
}

template <bool F32>
__global__ void __launch_bounds__(512, 2) k_b_probe(BatchArgs b, CandArgs c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t rt = 0;
    bool alive = false;
    uint32_t s = 0xffffffffu;
    if (i < c.n && c.state[i] == ST_UNDECIDED) {
        s = b.cinst[i];
        const BInst& I = ((const BInst*)b.table)[s];
        const Grid<D>& g = I.g;
        const Geo<D>& geo = I.geo;
        alive = probe_body<F32, F32>(g, geo, with_instance(c, b, I, s), i, rt);  // one radius per instance
    }
    const uint32_t slot = warp_append(&c.counters[0], alive);
    if (alive) c.alive[slot] = i;
    // survivors per instance (the next round's size, alive_darts): one atomic per instance present in the warp
    const uint32_t peers = __match_any_sync(0xffffffffu, alive ? s : 0xffffffffu);
    if (alive && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&b.alive_inst[s], (uint32_t)__popc(peers));
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

template <bool F32>
__global__ void __launch_bounds__(512, 2) k_b_collect(BatchArgs b, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    uint32_t rt = 0;
    bool undecided = false;
    if (t < nalive) {
        const uint32_t i = c.alive[t];
        const BInst& I = ((const BInst*)b.table)[b.cinst[i]];
        const Grid<D>& g = I.g;
        const Geo<D>& geo = I.geo;
        undecided = collect_body<F32>(g, geo, with_lists(c, I), i, rt);
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, undecided);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[0], (uint32_t)__popc(mask));
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

template <bool F32>
__global__ void __launch_bounds__(512, 2) k_b_settle(BatchArgs b, CandArgs c, int it) {
    if (c.und[it - 1] == 0) return;
    const uint32_t nalive = c.counters[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rounds = (nalive + stride - 1) / stride;  // same trip count for every lane
    uint32_t rt = 0;
    for (uint32_t rr = 0; rr < rounds; rr++) {
        const uint32_t t = t0 + rr * stride;
        bool still = false;
        if (t < nalive) {
            const uint32_t i = c.alive[t];
            const BInst& I = ((const BInst*)b.table)[b.cinst[i]];
            const Grid<D>& g = I.g;
            const Geo<D>& geo = I.geo;
            still = settle_body<F32>(g, geo, with_lists(c, I), i, rt);
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, still);
        if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.und[it], (uint32_t)__popc(mask));
    }
    if (F32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rt += __shfl_xor_sync(0xffffffffu, rt, o);
        if ((threadIdx.x & 31) == 0 && rt) atomicAdd(&c.counters[4], rt);
    }
}

// commit, with the accepted count of each instance (one atomic per instance present in the warp)
__global__ void __launch_bounds__(256) k_b_commit(BatchArgs b, CandArgs c) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nalive = c.counters[0];
    bool acc = false;
    uint32_t s = 0xffffffffu;
    if (t < nalive) {
        const uint32_t i = c.alive[t];
        s = b.cinst[i];
        const BInst& I = ((const BInst*)b.table)[s];
        const Grid<D>& g = I.g;
        const Geo<D>& geo = I.geo;
        acc = commit_body(g, geo, with_lists(c, I), i);
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&c.counters[1], (uint32_t)__popc(mask));
    const uint32_t peers = __match_any_sync(0xffffffffu, acc ? s : 0xffffffffu);
    if (acc && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&b.acc[s], (uint32_t)__popc(peers));
}

// Child masks of every voxel of the wave: an instance that refines this round gets the single-instance
// masks; the voxels of the others pass through unchanged (one output each).
template <bool F32>
__global__ void __launch_bounds__(512, 2) k_b_refine_mask(BatchArgs b, RefineArgs a) {
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t mask[MASK_WORDS];
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) mask[w] = 0;
    bool survived = false;
    uint32_t visits = 0, rt = 0;
    if (v < b.V) {
        const uint32_t s = segment_of(b.vox_off, b.M, v);
        const BatchRound& R = b.rnd[s];
        if (!R.refine) {
            mask[0] = 1u;
        } else {
            const BInst& I = ((const BInst*)b.table)[s];
            const Grid<D>& g = I.g;
            const Geo<D>& geo = I.geo;
            RefineParams p;
            p.V = 0;
            p.vin = nullptr;
            p.vout = nullptr;
#pragma unroll
            for (int d = 0; d < D; d++) {
                p.len[d] = R.len[d];
                p.nlen[d] = R.nlen[d];
                p.inf[d] = geo.inf[d];
                p.lenf[d] = (float)R.len[d];
                p.nlenf[d] = (float)R.nlen[d];
                p.rho_frac[d] = R.rho_frac[d];
                p.rho_int[d] = R.rho_int[d];
            }
            p.level = R.level;
            p.rmin = g.rmono;
            p.rminf = (float)g.rmono;
            p.masks = nullptr;
            p.warp_counts = nullptr;
            p.warp_offsets = nullptr;
            p.err = a.err;
            p.survivors = nullptr;
            p.visits = nullptr;
            p.retests = nullptr;
            int64_t cc[D];
#pragma unroll
            for (int d = 0; d < D; d++) cc[d] = a.vin[v * D + d];
            if constexpr (F32) survived = refine_mask32_body(g, geo, p, cc, mask, visits, rt);
            else survived = refine_mask64_body(g, geo, p, cc, mask, visits);
        }
#pragma unroll
        for (int w = 0; w < MASK_WORDS; w++) a.masks[v * MASK_WORDS + w] = mask[w];
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
        if (warp * 32 < b.V) a.warp_counts[warp] = cnt;
        if (alive) atomicAdd(a.survivors, (uint32_t)__popc(alive));
        if (wv) atomicAdd(a.visits, (unsigned long long)wv);
        if (wr) atomicAdd(a.retests, (unsigned long long)wr);
    }
}

// new_off[s] = first output voxel of instance s (s = 0..M): the warp's offset plus the children of the
// voxels before vox_off[s] in its warp
__global__ void k_b_refine_offsets(BatchArgs b, RefineArgs a, uint64_t* new_off) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > b.M) return;
    const uint64_t v0 = b.vox_off[s];
    if (v0 >= b.V) {
        new_off[s] = a.warp_offsets[(b.V + 31) / 32];  // the total
        return;
    }
    const uint64_t w = v0 >> 5;
    uint64_t o = a.warp_offsets[w];
    for (uint64_t u = w * 32; u < v0; u++)
        for (int k = 0; k < MASK_WORDS; k++) o += __popc(a.masks[u * MASK_WORDS + k]);
    new_off[s] = o;
}

__global__ void __launch_bounds__(256) k_b_refine_write(BatchArgs b, RefineArgs a) {
    const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t mask[MASK_WORDS];
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < MASK_WORDS; w++) {
        mask[w] = v < b.V ? a.masks[v * MASK_WORDS + w] : 0u;
        cnt += __popc(mask[w]);
    }
    const int lane = threadIdx.x & 31;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (v >= b.V || cnt == 0) return;
    uint64_t o = a.warp_offsets[v >> 5] + (incl - cnt);
    if (o + cnt > a.vout_cap) {
        atomicOr(a.err, (uint32_t)ERR_WRITE_BOUNDS);
        return;
    }
    int64_t cc[D];
#pragma unroll
    for (int d = 0; d < D; d++) cc[d] = a.vin[v * D + d];
    if (!b.rnd[segment_of(b.vox_off, b.M, v)].refine) {
#pragma unroll
        for (int d = 0; d < D; d++) a.vout[o * D + d] = cc[d];
        return;
    }
    for (int j = 0; j < CHILDREN; j++) {  // as k_refine_write
        const int t = corner_of_child(j);
        if (!((mask[t >> 5] >> (t & 31)) & 1u)) continue;
#pragma unroll
        for (int d = 0; d < D; d++) a.vout[o * D + d] = 2 * cc[d] + ((j >> d) & 1);
        o++;
    }
}

// splitmix64's output function (Steele, Lea, Flood, OOPSLA 2014): a bijective 64-bit mix
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xbf58476d1ce4e5b9ull;
    z ^= z >> 27;
    z *= 0x94d049bb133111ebull;
    z ^= z >> 31;
    return z;
}

// Per instance: the sphere count and an order-free checksum, the sum mod 2^64 over its spheres of
// h = mix64(... mix64(mix64(0x9E3779B97F4A7C15 ^ bits(x_0)) ^ bits(x_1)) ... ^ bits(x_{D-1})).
__global__ void __launch_bounds__(256) k_b_results(BatchArgs b, unsigned long long* counts, unsigned long long* sums) {
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t s = 0xffffffffu;
    uint32_t cnt = 0;
    uint64_t h = 0;
    if (w < b.nwords) {
        s = segment_of(b.word_off, b.M, w);
        uint32_t bits = b.occ[w];
        cnt = __popc(bits);
        while (bits) {
            const int j = __ffs(bits) - 1;
            bits &= bits - 1;
            const uint64_t idx = w * 32 + j;
            uint64_t z = 0x9E3779B97F4A7C15ull;
#pragma unroll
            for (int d = 0; d < D; d++) z = mix64(z ^ (uint64_t)__double_as_longlong(b.pos[idx * D + d]));
            h += z;
        }
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, s);
    if (peers == 0xffffffffu) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            h += __shfl_xor_sync(0xffffffffu, h, o);
        }
        if ((threadIdx.x & 31) == 0 && s != 0xffffffffu && cnt) {
            atomicAdd(counts + s, (unsigned long long)cnt);
            atomicAdd(sums + s, (unsigned long long)h);
        }
    } else if (s != 0xffffffffu && cnt) {
        atomicAdd(counts + s, (unsigned long long)cnt);
        atomicAdd(sums + s, (unsigned long long)h);
    }
}

// ------------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------------
uint64_t op_batch_table_bytes(uint32_t M) { return (uint64_t)M * sizeof(BInst); }

int op_batch_table_fill(const BatchInstance* inst, uint32_t M, void* d_table, cudaStream_t s) {
    std::vector<BInst> h(M);
    for (uint32_t i = 0; i < M; i++) {
        h[i].g = make_grid(inst[i].g);
        h[i].geo = make_geo(inst[i].g);
        h[i].head = inst[i].head;
        h[i].cocc = inst[i].cocc;
        h[i].seed_lo = (uint32_t)inst[i].seed;
        h[i].seed_hi = (uint32_t)(inst[i].seed >> 32);
        for (int d = 0; d < D; d++) h[i].nvox0[d] = inst[i].nvox0[d];
    }
    cudaError_t e = cudaMemcpyAsync(d_table, h.data(), (size_t)M * sizeof(BInst), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return (int)e;
}

void op_b_vox_init(const BatchArgs& b, int64_t* vox, cudaStream_t s) {
    if (b.V == 0) return;
    k_b_vox_init<<<nblocks(b.V, 256), 256, 0, s>>>(b, vox);
    count_launch();
}

void op_b_darts(const BatchArgs& b, const CandArgs& c, int f32, cudaStream_t s) {
    if (b.ndarts == 0) return;
    if (f32) k_b_darts<true><<<nblocks(b.ndarts, 256), 256, 0, s>>>(b, c);
    else k_b_darts<false><<<nblocks(b.ndarts, 256), 256, 0, s>>>(b, c);
    count_launch();
}

void op_b_dart_bins(const BatchArgs& b, const CandArgs& c, cudaStream_t s) {
    if (b.ndarts == 0 || !b.bin_hist) return;
    k_b_dart_bins<<<nblocks(b.ndarts, 256), 256, 0, s>>>(b, c);
    count_launch();
}

void op_b_probe(const BatchArgs& b, const CandArgs& c, int f32, int block, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32) k_b_probe<true><<<nblocks(c.n, block), block, 0, s>>>(b, c);
    else k_b_probe<false><<<nblocks(c.n, block), block, 0, s>>>(b, c);
    count_launch();
}

void op_b_collect(const BatchArgs& b, const CandArgs& c, int f32, int block, cudaStream_t s) {
    if (c.n == 0) return;
    if (f32) k_b_collect<true><<<nblocks(c.n, block), block, 0, s>>>(b, c);
    else k_b_collect<false><<<nblocks(c.n, block), block, 0, s>>>(b, c);
    count_launch();
}

void op_b_settle(const BatchArgs& b, const CandArgs& c, int it, int f32, int block, cudaStream_t s) {
    if (c.n == 0) return;
    // grid-stride over the alive list: at most 2048 resident threads per SM on 152 SMs
    const unsigned cap = 152u * (2048u / (unsigned)block);
    const unsigned nb = nblocks(c.n, block) < cap ? nblocks(c.n, block) : cap;
    if (f32) k_b_settle<true><<<nb, block, 0, s>>>(b, c, it);
    else k_b_settle<false><<<nb, block, 0, s>>>(b, c, it);
    count_launch();
}

void op_b_commit(const BatchArgs& b, const CandArgs& c, cudaStream_t s) {
    if (c.n == 0) return;
    k_b_commit<<<nblocks(c.n, 256), 256, 0, s>>>(b, c);
    count_launch();
}

void op_b_refine_mask(const BatchArgs& b, const RefineArgs& a, int f32, int block, cudaStream_t s) {
    if (b.V == 0) return;
    if (f32) k_b_refine_mask<true><<<nblocks(b.V, block), block, 0, s>>>(b, a);
    else k_b_refine_mask<false><<<nblocks(b.V, block), block, 0, s>>>(b, a);
    count_launch();
}

void op_b_refine_offsets(const BatchArgs& b, const RefineArgs& a, uint64_t* new_off, cudaStream_t s) {
    k_b_refine_offsets<<<nblocks((uint64_t)b.M + 1, 256), 256, 0, s>>>(b, a, new_off);
    count_launch();
}

void op_b_refine_write(const BatchArgs& b, const RefineArgs& a, cudaStream_t s) {
    if (b.V == 0) return;
    k_b_refine_write<<<nblocks(b.V, 256), 256, 0, s>>>(b, a);
    count_launch();
}

void op_b_results(const BatchArgs& b, unsigned long long* counts, unsigned long long* sums, cudaStream_t s) {
    if (b.nwords == 0) return;
    k_b_results<<<nblocks(b.nwords, 256), 256, 0, s>>>(b, counts, sums);
    count_launch();
}
