// kernels_common.cu -- dimension-independent kernels: scans of per-block counts.
#include <atomic>

#include "rsa_device.cuh"
#include "rsa_ops.h"

namespace rsagpu {

namespace {
std::atomic<uint64_t> g_launches{0};

constexpr int SCAN_THREADS = 1024;

// Exclusive scan of n uint32 counts into uint64 offsets with one block; total in offsets[n].
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_blocks(const uint32_t* counts, uint64_t* offsets, uint64_t n) {
    __shared__ uint64_t sh[SCAN_THREADS];
    const uint64_t chunk = (n + SCAN_THREADS - 1) / SCAN_THREADS;
    const uint64_t b = threadIdx.x * chunk;
    const uint64_t e = b + chunk < n ? b + chunk : n;
    uint64_t sum = 0;
    for (uint64_t i = b; i < e; i++) sum += counts[i];
    sh[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < SCAN_THREADS; o <<= 1) {
        uint64_t y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += y;
        __syncthreads();
    }
    uint64_t run = sh[threadIdx.x] - sum;
    for (uint64_t i = b; i < e; i++) {
        offsets[i] = run;
        run += counts[i];
    }
    if (threadIdx.x == SCAN_THREADS - 1) offsets[n] = sh[SCAN_THREADS - 1];
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
    k_scan_blocks<<<1, SCAN_THREADS, 0, s>>>(counts, offsets, n);
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
