// kernels_common.cu -- dimension-independent kernels: scans of per-block counts.
#include <atomic>

#include "rsa_device.cuh"
#include "rsa_ops.h"

namespace rsagpu {

namespace {
std::atomic<uint64_t> g_launches{0};

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;                            // counts per thread
constexpr uint64_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // counts per block

// Exclusive scan of n uint32 counts into uint64 offsets (total in offsets[n]) in three passes over tiles of
// SCAN_TILE counts: the tile sums are parked in the first offset slot of each tile (which the last pass
// overwrites), scanned by one block, then every tile is scanned from its base.
__device__ __forceinline__ uint32_t load_items(const uint32_t* counts, uint64_t n, uint64_t i0, uint32_t* v) {
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = i0 + k < n ? counts[i0 + k] : 0u;
        sum += v[k];
    }
    return sum;
}

// exclusive scan over the block's SCAN_THREADS threads; *total (if given) = the block's sum, for every thread
__device__ __forceinline__ uint64_t block_scan64(uint64_t x, uint64_t* total) {
    __shared__ uint64_t warp_sums[SCAN_THREADS / 32];
    __shared__ uint64_t block_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = warp_sums[lane];
        uint64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31) block_total = wi;
    }
    __syncthreads();
    const uint64_t r = warp_sums[warp] + incl - x;
    if (total) *total = block_total;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_sums(const uint32_t* counts, uint64_t* offsets, uint64_t n) {
    const uint64_t i0 = blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint64_t s = load_items(counts, n, i0, v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ uint64_t ws[SCAN_THREADS / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint64_t t = ws[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) offsets[blockIdx.x * SCAN_TILE] = t;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_bases(uint64_t* offsets, uint64_t n, uint64_t tiles) {
    __shared__ uint64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint64_t b = 0; b < tiles; b += SCAN_THREADS) {
        const uint64_t t = b + threadIdx.x;
        const uint64_t x = t < tiles ? offsets[t * SCAN_TILE] : 0;
        uint64_t chunk;
        const uint64_t ex = block_scan64(x, &chunk);
        if (t < tiles) offsets[t * SCAN_TILE] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += chunk;
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[n] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const uint32_t* counts, uint64_t* offsets, uint64_t n) {
    __shared__ uint64_t base;
    if (threadIdx.x == 0) base = offsets[blockIdx.x * SCAN_TILE];
    __syncthreads();
    const uint64_t i0 = blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    const uint32_t s = load_items(counts, n, i0, v);
    uint64_t run = base + block_scan64(s, nullptr);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (i0 + k < n) offsets[i0 + k] = run;
        run += v[k];
    }
}

// 16-bit digit histogram of v = key >> S over the keys whose digits above it equal prefix (radix select):
// the digit is (v >> dshift) & 0xFFFF, the prefix (v >> pshift), pshift = 64 for the top digit (no prefix).
__global__ void k_key_digit_hist(const uint64_t* keys, uint64_t n, int S, int dshift, int pshift, uint64_t prefix,
                                 uint32_t* hist) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = keys[i] >> S;
        if (pshift >= 64 || (v >> pshift) == prefix) atomicAdd(hist + ((v >> dshift) & 0xFFFFu), 1u);
    }
}

__global__ void __launch_bounds__(OCC_BLOCK) k_occ_block_counts(const uint32_t* occ, int64_t nwords, uint32_t* counts) {
    const int64_t w = (int64_t)blockIdx.x * OCC_BLOCK + threadIdx.x;
    const uint32_t c = w < nwords ? (uint32_t)__popc(occ[w]) : 0u;
    uint32_t total;
    block_exclusive_scan<OCC_BLOCK>(c, &total);
    if (threadIdx.x == 0) counts[blockIdx.x] = total;
}
}  // namespace

void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
uint64_t kernel_launch_count() { return g_launches.load(); }

void launch_scan_blocks(const uint32_t* counts, uint64_t* offsets, uint64_t n, uint64_t* total, cudaStream_t s) {
    (void)total;
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles) k_scan_tile_sums<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(counts, offsets, n);
    k_scan_tile_bases<<<1, SCAN_THREADS, 0, s>>>(offsets, n, tiles);
    if (tiles) k_scan_tiles<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(counts, offsets, n);
    count_launch(tiles ? 3 : 1);
}

void launch_key_digit_hist(const uint64_t* keys, uint64_t n, int S, int dshift, int pshift, uint64_t prefix,
                           uint32_t* hist, cudaStream_t s) {
    cudaMemsetAsync(hist, 0, 65536 * sizeof(uint32_t), s);
    if (n == 0) return;
    const uint64_t nb = (n + 255) / 256;
    k_key_digit_hist<<<(unsigned)(nb < 152 * 16 ? nb : 152 * 16), 256, 0, s>>>(keys, n, S, dshift, pshift, prefix, hist);
    count_launch();
}

void launch_occ_block_counts(const uint32_t* occ, int64_t nwords, uint32_t* counts, cudaStream_t s) {
    const unsigned nb = (unsigned)((nwords + OCC_BLOCK - 1) / OCC_BLOCK);
    if (nb == 0) return;
    k_occ_block_counts<<<nb, OCC_BLOCK, 0, s>>>(occ, nwords, counts);
    count_launch();
}

const DimOps* dim_ops_2();
const DimOps* dim_ops_3();
const DimOps* dim_ops_4();
const DimOps* dim_ops_5();
const DimOps* dim_ops_6();
const DimOps* dim_ops_7();

const DimOps* dim_ops(int D) {
    switch (D) {
    case 2: return dim_ops_2();
    case 3: return dim_ops_3();
    case 4: return dim_ops_4();
    case 5: return dim_ops_5();
    case 6: return dim_ops_6();
    case 7: return dim_ops_7();
    default: return nullptr;
    }
}

}  // namespace rsagpu
