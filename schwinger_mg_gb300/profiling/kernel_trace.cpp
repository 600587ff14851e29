// Per-kernel device-time totals from the CUPTI activity API (concurrent kernel
// records: start/end timestamps of every kernel the process launches, graph
// nodes included).  Used by the benchmark to attribute the time of one solve
// to its kernels without serialising them.
//
//   int smg_ktrace_start(void);              0 on success
//   int smg_ktrace_stop(const char* path);   writes "launches total_ns gridXxYxZ name" lines
//                                            (one line per kernel and grid shape)
#include <cupti.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

namespace {

struct Agg {
    unsigned long long n = 0, ns = 0;
};
std::mutex g_mu;
std::map<std::string, Agg> g_agg;
unsigned long long g_first = ~0ull, g_last = 0;

void CUPTIAPI buffer_requested(uint8_t** buf, size_t* size, size_t* max_records) {
    *size = 8u << 20;
    *buf = static_cast<uint8_t*>(std::aligned_alloc(8, *size));
    *max_records = 0;
}

void CUPTIAPI buffer_completed(CUcontext, uint32_t, uint8_t* buf, size_t, size_t valid) {
    CUpti_Activity* rec = nullptr;
    std::lock_guard<std::mutex> lock(g_mu);
    while (cuptiActivityGetNextRecord(buf, valid, &rec) == CUPTI_SUCCESS) {
        if (rec->kind != CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) continue;
        const auto* k = reinterpret_cast<const CUpti_ActivityKernel10*>(rec);
        char grid[64];
        std::snprintf(grid, sizeof grid, "%dx%dx%d ", k->gridX, k->gridY, k->gridZ);
        Agg& a = g_agg[std::string(grid) + (k->name ? k->name : "?")];
        a.n += 1;
        a.ns += k->end - k->start;
        if (k->start < g_first) g_first = k->start;
        if (k->end > g_last) g_last = k->end;
    }
    std::free(buf);
}

}  // namespace

extern "C" int smg_ktrace_start() {
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_agg.clear();
        g_first = ~0ull;
        g_last = 0;
    }
    if (cuptiActivityRegisterCallbacks(buffer_requested, buffer_completed) != CUPTI_SUCCESS) return 1;
    if (cuptiActivityEnable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL) != CUPTI_SUCCESS) return 2;
    return 0;
}

extern "C" int smg_ktrace_stop(const char* path) {
    cuptiActivityFlushAll(1);
    cuptiActivityDisable(CUPTI_ACTIVITY_KIND_CONCURRENT_KERNEL);
    cuptiActivityFlushAll(1);
    FILE* f = std::fopen(path, "w");
    if (!f) return 1;
    std::lock_guard<std::mutex> lock(g_mu);
    std::fprintf(f, "# span_ns %llu\n", g_last > g_first ? g_last - g_first : 0ull);
    for (const auto& kv : g_agg) std::fprintf(f, "%llu %llu %s\n", kv.second.n, kv.second.ns, kv.first.c_str());
    std::fclose(f);
    return 0;
}
