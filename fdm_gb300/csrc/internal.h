// Internal host helpers of libfdmgpu.so: status propagation and error text.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/fdmgpu.h"

namespace fdmgpu {

void set_error(const char* fmt, ...);

// Error carried through the C++ layer; converted to a status at the ABI.
struct Error {
    int code;
};

#define FDM_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ::fdmgpu::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                                __LINE__);                                                    \
            throw ::fdmgpu::Error{e_ == cudaErrorMemoryAllocation ? FDMGPU_ENOMEM : FDMGPU_ECUDA}; \
        }                                                                                     \
    } while (0)

#define FDM_FAIL(code, ...)                 \
    do {                                    \
        ::fdmgpu::set_error(__VA_ARGS__);   \
        throw ::fdmgpu::Error{code};        \
    } while (0)

// Checks the launch just made (configuration errors only; asynchronous
// faults surface at the next synchronising call).
#define FDM_LAUNCH_CHECK() FDM_CUDA(cudaGetLastError())

// Counts every kernel launch of the library and, when profiling is on,
// brackets it with CUDA events on its stream (skipped while the stream is
// being captured into a graph).  Declared per launch site:
//     FDM_TIMED("k_name", stream);  kernel<<<...>>>(...);
struct LaunchTimer {
    const char* name;
    cudaStream_t st;
    cudaEvent_t e0 = nullptr;
    LaunchTimer(const char* name, cudaStream_t st);
    ~LaunchTimer();
};
#define FDM_TIMED(name, st) ::fdmgpu::LaunchTimer fdm_timer_(name, st)

// Largest device ordinal + 1 that per-device state is kept for.
constexpr int kMaxDevices = 64;

// The calling thread's current device, checked against kMaxDevices.
int current_device();

// A value computed once per device by the first caller on that device (with
// the device current), e.g. a kernel's launch attributes, which are
// per-device state, or a device property.  A failing initialiser throws and
// leaves the slot to be tried again by the next caller.
template <typename T>
struct PerDevice {
    std::once_flag once[kMaxDevices];
    T val[kMaxDevices] = {};
    template <typename F>
    const T& get(F&& init) {
        const int d = current_device();
        std::call_once(once[d], [&] { val[d] = init(); });
        return val[d];
    }
};

// Device buffer that grows on demand and frees itself.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void* get(size_t need) {
        if (need > bytes) {
            if (p) cudaFree(p);
            p = nullptr;
            bytes = 0;
            FDM_CUDA(cudaMalloc(&p, need));
            bytes = need;
        }
        return p;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
};

}  // namespace fdmgpu

// Runs body, converting exceptions to status codes.
#define FDM_API_BEGIN try {
#define FDM_API_END                                         \
    return FDMGPU_OK;                                       \
    }                                                       \
    catch (const ::fdmgpu::Error& e) { return e.code; }     \
    catch (const std::bad_alloc&) {                         \
        ::fdmgpu::set_error("host allocation failed");      \
        return FDMGPU_ENOMEM;                               \
    }                                                       \
    catch (...) {                                           \
        ::fdmgpu::set_error("unexpected internal error");   \
        return FDMGPU_EINVAL;                               \
    }
