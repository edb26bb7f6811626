// Error reporting and version of the fdmgpu C ABI (include/fdmgpu.h).
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace fdmgpu {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int current_device() {
    int dev = 0;
    FDM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) FDM_FAIL(FDMGPU_EINVAL, "device ordinal %d out of range", dev);
    return dev;
}

// ---- launch accounting ---------------------------------------------------
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<int> g_profile{0};
struct ProfRecord {
    const char* name;
    cudaEvent_t e0, e1;
};
static std::mutex g_prof_mu;
static std::vector<ProfRecord> g_prof;
struct ProfSum {
    std::string name;
    long long count;
    double ms;
};
static std::vector<ProfSum> g_prof_sums;

LaunchTimer::LaunchTimer(const char* n, cudaStream_t s) : name(n), st(s) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!g_profile.load(std::memory_order_relaxed)) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    if (cudaEventCreate(&e0) != cudaSuccess) {
        e0 = nullptr;
        return;
    }
    cudaEventRecord(e0, st);
}

LaunchTimer::~LaunchTimer() {
    if (!e0) return;
    cudaEvent_t e1;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return;
    }
    cudaEventRecord(e1, st);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof.push_back({name, e0, e1});
}

}  // namespace fdmgpu

extern "C" {

unsigned long long fdmgpu_launch_count(void) { return fdmgpu::g_launches.load(); }

int fdmgpu_profile_enable(int on) {
    fdmgpu::g_profile.store(on ? 1 : 0);
    return FDMGPU_OK;
}

// Resolves every recorded launch (synchronising their events) into per-name
// totals; returns the number of distinct names.
int fdmgpu_profile_collect(int* nnames) {
    using namespace fdmgpu;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto& r : g_prof) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.e1) == cudaSuccess && cudaEventElapsedTime(&ms, r.e0, r.e1) == cudaSuccess) {
            bool found = false;
            for (auto& s : g_prof_sums)
                if (s.name == r.name) {
                    s.count++;
                    s.ms += ms;
                    found = true;
                }
            if (!found) g_prof_sums.push_back({r.name, 1, (double)ms});
        }
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    g_prof.clear();
    if (nnames) *nnames = (int)g_prof_sums.size();
    return FDMGPU_OK;
}

int fdmgpu_profile_entry(int i, char* name, int namelen, long long* count, double* total_ms) {
    using namespace fdmgpu;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (i < 0 || i >= (int)g_prof_sums.size()) {
        set_error("profile entry %d out of range", i);
        return FDMGPU_EINVAL;
    }
    if (name && namelen > 0) snprintf(name, namelen, "%s", g_prof_sums[i].name.c_str());
    if (count) *count = g_prof_sums[i].count;
    if (total_ms) *total_ms = g_prof_sums[i].ms;
    return FDMGPU_OK;
}

int fdmgpu_profile_reset(void) {
    using namespace fdmgpu;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto& r : g_prof) {
        cudaEventDestroy(r.e0);
        cudaEventDestroy(r.e1);
    }
    g_prof.clear();
    g_prof_sums.clear();
    return FDMGPU_OK;
}

const char* fdmgpu_last_error(void) { return fdmgpu::g_last_error; }

int fdmgpu_version(void) { return 100; }

}  // extern "C"
