// Complex arithmetic and small shared helpers for the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace s1g {

template <typename R>
struct alignas(2 * sizeof(R)) cpx {
    R x, y;
};

using cf32 = cpx<float>;
using cf64 = cpx<double>;

template <typename R>
__host__ __device__ __forceinline__ cpx<R> mk(R a, R b) {
    cpx<R> c;
    c.x = a;
    c.y = b;
    return c;
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator+(cpx<R> a, cpx<R> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator-(cpx<R> a, cpx<R> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, cpx<R> b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename R>
__host__ __device__ __forceinline__ cpx<R> operator*(cpx<R> a, R s) { return mk(a.x * s, a.y * s); }
template <typename R>
__host__ __device__ __forceinline__ cpx<R> conj(cpx<R> a) { return mk(a.x, -a.y); }
template <typename R>
__host__ __device__ __forceinline__ R norm2(cpx<R> a) { return a.x * a.x + a.y * a.y; }
// multiply by +i (dir>0) or -i (dir<0)
template <typename R>
__host__ __device__ __forceinline__ cpx<R> mul_i(cpx<R> a, int dir) {
    return dir > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x);
}

template <typename To, typename From>
__host__ __device__ __forceinline__ cpx<To> cvt(cpx<From> a) { return mk((To)a.x, (To)a.y); }

#ifdef __CUDACC__
// read-only cached loads of complex values
__device__ __forceinline__ cpx<float> ldg(const cpx<float>* p) {
    float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return mk(v.x, v.y);
}
__device__ __forceinline__ cpx<double> ldg(const cpx<double>* p) {
    double2 v = __ldg(reinterpret_cast<const double2*>(p));
    return mk(v.x, v.y);
}
#endif

}  // namespace s1g
