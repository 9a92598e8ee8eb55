// noalloc.cu -- rsagpu_resolve_batch_noalloc: same-round conflict resolution of a candidate batch that
// allocates nothing.
//
// Callers that cannot call cudaMalloc (code running inside another framework's memory pool, a
// pre-allocated real-time loop, or a library that must not touch the device heap) pass device
// buffers for the inputs and the output; every temporary of the computation lives in one static
// device array of this file, g_noalloc_scratch, which each GPU that loads this library holds until
// the process exits.
#include <cstdint>
#include <mutex>

#include "../../include/rsagpu.h"
#include "rsa_device.cuh"
#include "rsa_ops.h"

namespace rsagpu {
namespace {

constexpr uint32_t NA_MAX_N = RSAGPU_NOALLOC_MAX_CANDIDATES;
constexpr uint32_t NA_BUCKETS = 1u << 18;  // hash buckets of the per-cell candidate lists
constexpr int NA_MAX_IT = 4096;            // settle iterations before RSAGPU_ERR_NO_PROGRESS

struct NoAllocScratch {
    int32_t head[NA_BUCKETS];
    int32_t next[NA_MAX_N];
    int32_t blk[(size_t)NA_MAX_N * NB];
    uint8_t state[NA_MAX_N];
    uint8_t nblk[NA_MAX_N];
    uint32_t und[NA_MAX_IT + 1];
    uint32_t err;  // NA_ERR_* bits of the current call
};

// input errors found on the device (the inputs live in device memory, so the host cannot check them)
enum : uint32_t { NA_ERR_RADIUS = 1u, NA_ERR_OUTSIDE = 2u };

// Device-side scratch.  In host code this name is only a host-side stand-in for the array: host code
// reaches the device address through cudaGetSymbolAddress (see scratch_on_current_device).
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

template <int D>
struct NaGeo {
    double inf[D], sup[D], L[D], inv_c[D];
    int32_t n[D];
    double r_max;
};

template <int D>
__device__ __forceinline__ void na_cell(const NaGeo<D>& g, const double* x, int32_t* k) {
#pragma unroll
    for (int d = 0; d < D; d++) {
        int32_t kk = (int32_t)floor(__dmul_rn(__dsub_rn(x[d], g.inf[d]), g.inv_c[d]));
        k[d] = kk < 0 ? 0 : (kk >= g.n[d] ? g.n[d] - 1 : kk);
    }
}

template <int D>
__device__ __forceinline__ uint32_t na_bucket(const NaGeo<D>& g, const int32_t* k) {
    uint64_t idx = 0;
#pragma unroll
    for (int d = D - 1; d >= 0; d--) idx = idx * (uint64_t)g.n[d] + (uint64_t)k[d];
    return (uint32_t)((idx * 0x9E3779B97F4A7C15ull) >> 46) & (NA_BUCKETS - 1);
}

// Visits the candidates of the 3^D cells around k (cells of edge >= 2 r_max), with the periodic image
// shift of each cell.  A bucket may also hold candidates of other cells; testing those against an
// image is still a test against a real periodic copy, so the decisions are unchanged.
template <int D, class F>
__device__ __forceinline__ void na_visit(const NaGeo<D>& g, const NoAllocScratch* S, const double* pos,
                                         const int32_t* k, F&& f) {
    int total = 1;
#pragma unroll
    for (int d = 0; d < D; d++) total *= 3;
    for (int t = 0; t < total; t++) {
        int32_t kk[D];
        int8_t q[D];
        int tt = t;
#pragma unroll
        for (int d = 0; d < D; d++) {
            int32_t v = k[d] + (tt % 3) - 1;
            tt /= 3;
            q[d] = 0;
            if (v < 0) { v += g.n[d]; q[d] = -1; }
            else if (v >= g.n[d]) { v -= g.n[d]; q[d] = 1; }
            kk[d] = v;
        }
        const uint32_t b = na_bucket<D>(g, kk);
        for (int32_t j = S->head[b]; j >= 0; j = S->next[j]) {
            double img[D];
#pragma unroll
            for (int d = 0; d < D; d++) {
                const double p = pos[(uint64_t)j * D + d];
                img[d] = q[d] == 0 ? p : __dadd_rn(p, q[d] > 0 ? g.L[d] : -g.L[d]);
            }
            if (f(j, img)) return;
        }
    }
}

__device__ __forceinline__ bool na_precedes(uint64_t kj, int32_t j, uint64_t ki, uint32_t i) {
    return kj < ki || (kj == ki && (uint32_t)j < i);
}

__global__ void k_na_clear() {
    NoAllocScratch* S = &g_noalloc_scratch;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < NA_BUCKETS; i += gridDim.x * blockDim.x) S->head[i] = -1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= (uint32_t)NA_MAX_IT; i += gridDim.x * blockDim.x)
        S->und[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) S->err = 0;
}

template <int D>
__global__ void k_na_link(NaGeo<D> g, const double* pos, const double* rad, uint32_t n) {
    NoAllocScratch* S = &g_noalloc_scratch;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[D];
#pragma unroll
    for (int d = 0; d < D; d++) x[d] = pos[(uint64_t)i * D + d];
    // the cells are sized for radii up to r_max and hold points of [inf, sup]: a larger radius or a point
    // outside the box would miss colliders, so the call reports it instead of deciding
    uint32_t err = rad[i] <= g.r_max ? 0u : NA_ERR_RADIUS;
#pragma unroll
    for (int d = 0; d < D; d++)
        if (!(x[d] >= g.inf[d] && x[d] <= g.sup[d])) err |= NA_ERR_OUTSIDE;
    if (err) atomicOr(&S->err, err);
    int32_t k[D];
    na_cell<D>(g, x, k);
    S->next[i] = atomicExch(S->head + na_bucket<D>(g, k), (int32_t)i);
    S->state[i] = ST_UNDECIDED;
}

template <int D>
__global__ void k_na_collect(NaGeo<D> g, const double* pos, const uint64_t* key, const double* rad, uint32_t n) {
    NoAllocScratch* S = &g_noalloc_scratch;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool undecided = false;
    if (i < n) {
        double x[D];
#pragma unroll
        for (int d = 0; d < D; d++) x[d] = pos[(uint64_t)i * D + d];
        const double r = rad[i];
        const uint64_t ki = key[i];
        int32_t k[D];
        na_cell<D>(g, x, k);
        int nb = 0;
        na_visit<D>(g, S, pos, k, [&](int32_t j, const double* img) {
            if (!na_precedes(key[j], j, ki, i)) return false;
            if (!collide64<D>(r, x, rad[j], img)) return false;
            if (nb < NB) S->blk[(uint64_t)i * NB + nb] = j;
            nb++;
            return false;
        });
        if (nb == 0) {
            S->state[i] = ST_ACCEPTED;
        } else {
            S->nblk[i] = nb > NB ? (uint8_t)NB_OVERFLOW : (uint8_t)nb;
            undecided = true;
        }
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, undecided);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&S->und[0], (uint32_t)__popc(mask));
}

template <int D>
__global__ void k_na_settle(NaGeo<D> g, const double* pos, const uint64_t* key, const double* rad, uint32_t n, int it) {
    NoAllocScratch* S = &g_noalloc_scratch;
    if (S->und[it - 1] == 0) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool still = false;
    if (i < n && *((volatile uint8_t*)(S->state + i)) == ST_UNDECIDED) {
        bool any_acc = false, all_rej = true;
        const uint8_t nb = S->nblk[i];
        if (nb != NB_OVERFLOW) {
            for (int b = 0; b < nb; b++) {
                const uint8_t s = *((volatile uint8_t*)(S->state + S->blk[(uint64_t)i * NB + b]));
                any_acc |= (s == ST_ACCEPTED);
                all_rej &= (s == ST_REJECTED);
            }
        } else {
            double x[D];
#pragma unroll
            for (int d = 0; d < D; d++) x[d] = pos[(uint64_t)i * D + d];
            const double r = rad[i];
            const uint64_t ki = key[i];
            int32_t k[D];
            na_cell<D>(g, x, k);
            na_visit<D>(g, S, pos, k, [&](int32_t j, const double* img) {
                if (!na_precedes(key[j], j, ki, i)) return false;
                if (!collide64<D>(r, x, rad[j], img)) return false;
                const uint8_t s = *((volatile uint8_t*)(S->state + j));
                any_acc |= (s == ST_ACCEPTED);
                all_rej &= (s == ST_REJECTED);
                return any_acc;
            });
        }
        if (any_acc) S->state[i] = ST_REJECTED;
        else if (all_rej) S->state[i] = ST_ACCEPTED;
        else still = true;
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, still);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(&S->und[it], (uint32_t)__popc(mask));
}

__global__ void k_na_output(uint8_t* accepted, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) accepted[i] = g_noalloc_scratch.state[i] == ST_ACCEPTED ? 1 : 0;
}

// Device address of g_noalloc_scratch on the current device, looked up once per device with that
// device current and kept for the life of the process.  A cudaDeviceReset (or any other teardown of the
// device's primary context) makes the kept address stale, so the entry point does not support it.
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
NoAllocScratch* g_na_ptr[NA_MAX_DEVICES] = {};

cudaError_t scratch_on_current_device(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_ptr[dev] = (NoAllocScratch*)p;
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

template <int D>
int run(const NaGeo<D>& g, const double* pos, const uint64_t* key, const double* rad, uint32_t n, uint8_t* accepted,
        cudaStream_t s, NoAllocScratch* S, const char** why) {
    const unsigned nb = (n + 255) / 256;
    k_na_clear<<<256, 256, 0, s>>>();
    k_na_link<D><<<nb, 256, 0, s>>>(g, pos, rad, n);
    count_launch(2);
    {
        uint32_t err = 0;
        cudaError_t e = cudaMemcpyAsync(&err, &S->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            *why = cudaGetErrorString(e);
            return RSAGPU_ERR_CUDA;
        }
        if (err & NA_ERR_RADIUS) {
            *why = "rsagpu_resolve_batch_noalloc: a radius above r_max";
            return RSAGPU_ERR_ARG;
        }
        if (err & NA_ERR_OUTSIDE) {
            *why = "rsagpu_resolve_batch_noalloc: a centre outside [inf, sup]";
            return RSAGPU_ERR_ARG;
        }
    }
    k_na_collect<D><<<nb, 256, 0, s>>>(g, pos, key, rad, n);
    count_launch();
    int it = 1;
    while (true) {
        for (int b = 0; b < 4; b++, it++) {
            if (it > NA_MAX_IT) {
                *why = "settle did not converge";
                return RSAGPU_ERR_NO_PROGRESS;
            }
            k_na_settle<D><<<nb, 256, 0, s>>>(g, pos, key, rad, n, it);
            count_launch();
        }
        uint32_t left = 0;
        cudaError_t e = cudaMemcpyAsync(&left, S->und + (it - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            *why = cudaGetErrorString(e);
            return RSAGPU_ERR_CUDA;
        }
        if (left == 0) break;
    }
    k_na_output<<<nb, 256, 0, s>>>(accepted, n);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        *why = cudaGetErrorString(e);
        return RSAGPU_ERR_CUDA;
    }
    return RSAGPU_OK;
}

template <int D>
int dispatch(const double* inf, const double* sup, double r_max, const double* pos, const uint64_t* key,
             const double* rad, uint32_t n, uint8_t* accepted, cudaStream_t s, NoAllocScratch* S, const char** why) {
    NaGeo<D> g;
    g.r_max = r_max;
    for (int d = 0; d < D; d++) {
        g.inf[d] = inf[d];
        g.sup[d] = sup[d];
        g.L[d] = sup[d] - inf[d];
        int32_t c = (int32_t)(g.L[d] / (2 * r_max));
        if (c < 1) c = 1;
        if (c > (1 << 20)) c = 1 << 20;
        g.n[d] = c;
        g.inv_c[d] = 1.0 / (g.L[d] / c);
    }
    return run<D>(g, pos, key, rad, n, accepted, s, S, why);
}

}  // namespace
}  // namespace rsagpu

extern "C" int rsagpu_resolve_batch_noalloc(int dim, const double* inf, const double* sup, double r_max,
                                            const double* d_pos, const uint64_t* d_key, const double* d_rad,
                                            uint64_t n, uint8_t* d_accepted, void* stream) {
    using namespace rsagpu;
    if (dim < 2 || dim > RSAGPU_MAX_DIM || !inf || !sup) {
        set_last_error("rsagpu_resolve_batch_noalloc: invalid dimension or box");
        return RSAGPU_ERR_ARG;
    }
    for (int d = 0; d < dim; d++)
        if (!(sup[d] > inf[d])) {
            set_last_error("rsagpu_resolve_batch_noalloc: empty box");
            return RSAGPU_ERR_ARG;
        }
    if (!(r_max > 0)) {
        set_last_error("rsagpu_resolve_batch_noalloc: r_max must be positive");
        return RSAGPU_ERR_ARG;
    }
    if (n > NA_MAX_N) {
        set_last_error("rsagpu_resolve_batch_noalloc: more candidates than RSAGPU_NOALLOC_MAX_CANDIDATES");
        return RSAGPU_ERR_CAPACITY;
    }
    if (n == 0) return RSAGPU_OK;
    if (!d_pos || !d_key || !d_rad || !d_accepted) {
        set_last_error("rsagpu_resolve_batch_noalloc: null device buffer");
        return RSAGPU_ERR_ARG;
    }
    NoAllocScratch* S = nullptr;
    cudaError_t e = scratch_on_current_device(&S);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(cudaGetErrorString(e));
        return RSAGPU_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const char* why = nullptr;
    int rc;
    const uint32_t m = (uint32_t)n;
    switch (dim) {
    case 2: rc = dispatch<2>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    case 3: rc = dispatch<3>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    case 4: rc = dispatch<4>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    case 5: rc = dispatch<5>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    case 6: rc = dispatch<6>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    default: rc = dispatch<7>(inf, sup, r_max, d_pos, d_key, d_rad, m, d_accepted, s, S, &why); break;
    }
    if (rc != RSAGPU_OK) set_last_error(why ? why : "rsagpu_resolve_batch_noalloc failed");
    return rc;
}
