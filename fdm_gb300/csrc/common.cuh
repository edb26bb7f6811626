// Shared helpers for the GB300 Poisson / NSCube kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fdmgpu {

template <typename T> struct vec2;
template <> struct vec2<float> { using type = float2; };
template <> struct vec2<double> { using type = double2; };
template <typename T> using vec2_t = typename vec2<T>::type;

template <typename T>
__device__ __forceinline__ vec2_t<T> cmul(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename T>
__device__ __forceinline__ vec2_t<T> cadd(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r; r.x = a.x + b.x; r.y = a.y + b.y; return r;
}
template <typename T>
__device__ __forceinline__ vec2_t<T> csub(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r; r.x = a.x - b.x; r.y = a.y - b.y; return r;
}
// multiply by -i
template <typename T>
__device__ __forceinline__ vec2_t<T> cmul_mi(vec2_t<T> a) {
    vec2_t<T> r; r.x = a.y; r.y = -a.x; return r;
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

__host__ __device__ inline int ilog2_exact(int n) {
    int q = 0;
    if (n < 1) return -1;
    while ((1 << q) < n) q++;
    return (1 << q) == n ? q : -1;
}

}  // namespace fdmgpu
