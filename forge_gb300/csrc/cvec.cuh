// Complex helpers templated on the real type (double2 / float2 storage).
#pragma once
#include <cuda_runtime.h>

namespace forge {

template <class T>
struct CV;
template <>
struct CV<double> {
    using type = double2;
};
template <>
struct CV<float> {
    using type = float2;
};

template <class V>
__host__ __device__ inline V vmake(decltype(V{}.x) r, decltype(V{}.x) i) {
    V v;
    v.x = r;
    v.y = i;
    return v;
}
template <class V>
__host__ __device__ inline V vadd(V a, V b) {
    return vmake<V>(a.x + b.x, a.y + b.y);
}
template <class V>
__host__ __device__ inline V vsub(V a, V b) {
    return vmake<V>(a.x - b.x, a.y - b.y);
}
template <class V>
__host__ __device__ inline V vmul(V a, V b) {
    return vmake<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <class V>
__host__ __device__ inline V vcjmul(V a, V b) {
    return vmake<V>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
// a * conj(b)
template <class V>
__host__ __device__ inline V vmulcj(V a, V b) {
    return vmake<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <class V>
__host__ __device__ inline V vconj(V a) {
    return vmake<V>(a.x, -a.y);
}
template <class V>
__host__ __device__ inline V vzero() {
    return vmake<V>(0, 0);
}

template <class V>
__device__ inline V warp_sum(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
__device__ inline double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline double warp_max_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace forge
