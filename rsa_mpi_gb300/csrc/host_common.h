// host_common.h -- host-side helpers shared by the single-instance driver (rsagpu.cu) and the batched
// driver (batch.cu): error reporting, device allocation, ball volumes and the sphere-grid plan.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rsagpu.h"
#include "rsa_ops.h"

namespace rsagpu {
namespace host {

inline int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_last_error(buf);
    return code;
}

struct CudaError {
    int code;
};

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            ::rsagpu::host::fail(RSAGPU_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                 __FILE__, __LINE__);                                              \
            throw ::rsagpu::host::CudaError{RSAGPU_ERR_CUDA};                                      \
        }                                                                                          \
    } while (0)

struct Fail {
    int code;
};

[[noreturn]] inline void raise(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_last_error(buf);
    throw Fail{code};
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return RSAGPU_OK;
    } catch (const CudaError& e) {
        return e.code;
    } catch (const Fail& e) {
        return e.code;
    } catch (const std::bad_alloc&) {
        return fail(RSAGPU_ERR_CAPACITY, "host allocation failed");
    }
}

// Device memory comes from the current device's stream-ordered pool, which keeps freed memory for reuse
// (up to kPoolKeepBytes): a user's create / proceed / extract / destroy cycle then does not unmap and map
// gigabytes each time (cudaFree of the 3D r = 0.002 buffers took 13.6 ms of a 225 ms call).  The
// allocation is made on the legacy stream and waited for, and a free first waits for the device, as cudaMalloc
// and cudaFree do, so every caller keeps their synchronous semantics.
constexpr uint64_t kPoolKeepBytes = 128ull << 30;

inline void keep_pool_memory() {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = kPoolKeepBytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
}

template <class T>
T* dalloc(uint64_t n) {
    if (n == 0) n = 1;
    void* p = nullptr;
    keep_pool_memory();
    cudaError_t e = cudaMallocAsync(&p, n * sizeof(T), 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        raise(RSAGPU_ERR_CUDA, "device allocation of %llu bytes failed: %s", (unsigned long long)(n * sizeof(T)),
              cudaGetErrorString(e));
    }
    return (T*)p;
}

template <class T>
void dfree(T*& p) {
    if (p) {
        cudaDeviceSynchronize();  // no kernel in flight may still use p
        cudaFreeAsync(p, 0);
        cudaStreamSynchronize(0);
    }
    p = nullptr;
}

// v_D(r) as volumeSphere (auxiliary/Geometry/Sphere.ixx:30-57): mult * puissance<D>(r)
inline double pow_int(double x, int e) {
    if (e == 0) return 1;
    if (e == 1) return x;
    int e1 = e / 2;
    return pow_int(x, e1) * pow_int(x, e - e1);
}
inline double unit_ball_volume(int D) {
    const double pi = 3.14159265358979323846;
    double mult = 1;
    if (D % 2 == 0) {
        for (int k = 0; k <= D / 2 - 1; k++) mult *= (2 * pi) / (D - 2 * k);
    } else {
        mult = 1. / pi;
        for (int k = 0; k <= (D - 1) / 2; k++) mult *= (2 * pi) / (D - 2 * k);
    }
    return mult;
}
inline double ball_volume(int D, double r) { return unit_ball_volume(D) * pow_int(r, D); }

// The fixed (heuristic) schedule shared by both drivers: a pass throws factor * V darts (clamped to
// [min_darts, max_darts], and to 16x the spheres still wanted), and the voxels are subdivided after a
// pass in which more than miss_threshold of the darts missed.  Defaults tuned on the 3D r = 0.002 cube.
constexpr double kDefaultFactor = 0.25;
constexpr double kDefaultMissThreshold = 0.99;
constexpr uint64_t kDefaultMinDarts = 4096;
constexpr uint64_t kDefaultMaxDarts = 1ull << 26;

inline uint64_t heuristic_darts(double factor, uint64_t min_darts, uint64_t max_darts, uint64_t V) {
    double c = factor * (double)V;
    c = std::max(c, (double)min_darts);
    c = std::min(c, (double)max_darts);
    return (uint64_t)c;
}

inline uint64_t cap_darts(uint64_t C, uint64_t remaining, uint64_t min_darts) {
    const double cap = std::max(16.0 * (double)remaining, (double)min_darts);
    return (double)C > cap ? (uint64_t)cap : C;
}

// Darts of a round bounded by the survivors it can expect (single-instance and batched schedules alike): at most
// kAlivePerVoxel darts per voxel that survive the probe, at the survival ratio (alive / darts) of the previous round,
// or all of them for the first; never fewer than kAliveFloor.  Collect and settle work over the survivors and their
// same-round neighbours, so a round with many survivors per cell costs more per dart than two half rounds: the first
// round of config 2 (20.4 M darts into an empty box) took 16.7 ms, a tenth of the run.  The floor leaves small runs,
// where every extra round costs its launches and readbacks, as they were.
constexpr double kAlivePerVoxel = 1.0 / 16.0;
constexpr double kAliveFloor = (double)(1u << 20);
inline uint64_t alive_darts(uint64_t C, uint64_t V, double alive_ratio) {
    const double lim = std::max(kAliveFloor, kAlivePerVoxel * (double)V / std::max(alive_ratio, 1e-3));
    return (double)C > lim ? (uint64_t)lim : C;
}

// Darts of a round of a class that has a count (single-instance heuristic and learned schedules): about 1.25x the
// spheres still wanted at the hit ratio (greedy accepted / darts) of the class's previous round, or 4x the spheres
// still wanted for the class's first round.  A round past the count is cut by the count cap, so its extra darts
// are work thrown away (in a near-empty box nearly every dart survives the probe and enters the conflict
// resolution); a round short of it costs one more round.  Where the count is far off (a class given by a volume
// fraction the packing never reaches) the bound stays above the voxel-based round size.
inline uint64_t class_darts(uint64_t C, uint64_t remaining, uint64_t min_darts, double hit_ratio) {
    const double want = hit_ratio > 0 ? 1.25 * (double)remaining / std::max(hit_ratio, 1e-4) : 4.0 * (double)remaining;
    const double cap = std::max(want, (double)min_darts);
    return (double)C > cap ? (uint64_t)cap : C;
}

// miss rate of a pass (operator_algorithm.ixx:140-162): darts that placed no sphere
inline double miss_rate(uint64_t shots, uint64_t hits) {
    return (double)(shots - hits) / (0.000001 + (double)shots);
}

// Binned dart order: bins of 2^shift consecutive voxels, about 64 darts per bin (the voxel list is in spatial
// order, so a bin is a small region of the box and the probe's neighbouring threads share stencil cells).
inline int dart_bin_shift(uint64_t V, uint64_t darts) {
    int sh = 0;
    while (sh < 48 && (double)darts * std::ldexp(1.0, sh) < 64.0 * (double)V) sh++;
    return sh;
}

// Geometry of a sphere grid: the cell counts, the stencil, its rows and the FP32 guard band.  Both drivers
// build every grid through this one function, so a batched instance gets exactly the grid of its
// single-instance run.
struct GridPlan {
    GridArgs a{};  // geometry only; the device pointers are left null
    std::vector<int8_t> stencil;
    std::vector<int8_t> rows;
    std::vector<float> rows_r2;
};

GridPlan plan_grid(int D, const double* inf, const double* L, double rmin, double rmax);

}  // namespace host
}  // namespace rsagpu
