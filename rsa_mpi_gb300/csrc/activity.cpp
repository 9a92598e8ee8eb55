// activity.cpp -- GPU busy and idle time of the process over a span, from CUPTI activity records (kernels,
// memcpys, memsets of every stream).  Measurement support for bench.py --idle, built into
// rsa_mpi_gb300/_build/libactivity.so apart from the sampler library (which never loads it).
//
// rsa_activity_start() enables the records; rsa_activity_stop(out) flushes them and writes, over the records
// since the start: out[0] records, out[1] span (first start to last end, ns), out[2] busy (union of the
// records' intervals, ns), out[3] gaps between busy intervals, out[4] median gap (ns), out[5] 99th percentile
// gap (ns), out[6] largest gap (ns), out[7] sum of the gaps longer than 10 us (ns).  Returns 0, or the CUPTI
// error code of the call that failed.
#include <cupti.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <utility>
#include <vector>

namespace {

std::vector<std::pair<uint64_t, uint64_t>> g_spans;

void CUPTIAPI on_request(uint8_t** buffer, size_t* size, size_t* max_records) {
    *size = 16u << 20;
    *buffer = static_cast<uint8_t*>(std::aligned_alloc(8, *size));
    *max_records = 0;
}

void CUPTIAPI on_complete(CUcontext, uint32_t, uint8_t* buffer, size_t, size_t valid) {
    CUpti_Activity* rec = nullptr;
    while (cuptiActivityGetNextRecord(buffer, valid, &rec) == CUPTI_SUCCESS) {
        uint64_t s = 0, e = 0;
        if (rec->kind == CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL || rec->kind == CUPTI_ACTIVITY_KIND_KERNEL) {
            const auto* k = reinterpret_cast<const CUpti_ActivityKernel10*>(rec);
            s = k->start;
            e = k->end;
        } else if (rec->kind == CUPTI_ACTIVITY_KIND_MEMCPY) {
            const auto* m = reinterpret_cast<const CUpti_ActivityMemcpy6*>(rec);
            s = m->start;
            e = m->end;
        } else if (rec->kind == CUPTI_ACTIVITY_KIND_MEMSET) {
            const auto* m = reinterpret_cast<const CUpti_ActivityMemset4*>(rec);
            s = m->start;
            e = m->end;
        } else {
            continue;
        }
        g_spans.emplace_back(s, e);
    }
    std::free(buffer);
}

const CUpti_ActivityKind kKinds[] = {CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL, CUPTI_ACTIVITY_KIND_MEMCPY,
                                     CUPTI_ACTIVITY_KIND_MEMSET};

}  // namespace

extern "C" int rsa_activity_start() {
    g_spans.clear();
    CUptiResult r = cuptiActivityRegisterCallbacks(on_request, on_complete);
    if (r != CUPTI_SUCCESS) return (int)r;
    for (CUpti_ActivityKind k : kKinds) {
        r = cuptiActivityEnable(k);
        if (r != CUPTI_SUCCESS) return (int)r;
    }
    return 0;
}

extern "C" int rsa_activity_stop(double* out) {
    const CUptiResult r = cuptiActivityFlushAll(1);
    for (CUpti_ActivityKind k : kKinds) cuptiActivityDisable(k);
    std::sort(g_spans.begin(), g_spans.end());
    double busy = 0, long_gaps = 0;
    std::vector<double> gaps;
    uint64_t cs = 0, ce = 0;
    bool open = false;
    for (const auto& p : g_spans) {
        if (!open) {
            cs = p.first;
            ce = p.second;
            open = true;
        } else if (p.first > ce) {
            busy += (double)(ce - cs);
            const double g = (double)(p.first - ce);
            gaps.push_back(g);
            if (g > 10000.0) long_gaps += g;
            cs = p.first;
            ce = p.second;
        } else if (p.second > ce) {
            ce = p.second;
        }
    }
    if (open) busy += (double)(ce - cs);
    std::sort(gaps.begin(), gaps.end());
    out[0] = (double)g_spans.size();
    out[1] = g_spans.empty() ? 0.0 : (double)(ce - g_spans.front().first);
    out[2] = busy;
    out[3] = (double)gaps.size();
    out[4] = gaps.empty() ? 0.0 : gaps[gaps.size() / 2];
    out[5] = gaps.empty() ? 0.0 : gaps[(size_t)((double)gaps.size() * 0.99)];
    out[6] = gaps.empty() ? 0.0 : gaps.back();
    out[7] = long_gaps;
    return r == CUPTI_SUCCESS ? 0 : (int)r;
}
