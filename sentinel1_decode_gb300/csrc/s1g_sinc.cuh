// Warp-cooperative Hann-windowed sinc interpolation (sinc_interpolate,
// signal_processing.cpp:228-257), shared by the resampler s1g_sinc_interpolate
// and the sinc RCMC of the row pass.
#pragma once

#include <climits>

#include "s1g_kernels.h"

namespace s1g {

// The reference's truncated PI (structs.h).
constexpr double kSincPi = 3.14159265358979;

template <typename R>
__device__ __forceinline__ R sinc_weight(double x, int L);

template <>
__device__ __forceinline__ float sinc_weight<float>(double xd, int L) {
    const float x = (float)xd;
    const float s = x == 0.0f ? 1.0f : sinpif(x) / (3.14159265358979f * x);
    return s * (0.5f * (1.0f + cospif(x / (float)L)));
}
template <>
__device__ __forceinline__ double sinc_weight<double>(double x, int L) {
    const double s = x == 0.0 ? 1.0 : sin(kSincPi * x) / (kSincPi * x);
    return s * (0.5 * (1.0 + cos(kSincPi * x / L)));
}

template <typename R>
__device__ __forceinline__ cpx<R> shfl(cpx<R> v, int src) {
    return mk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Sample idx of a line, zero outside [0, n).
template <typename R>
__device__ __forceinline__ cpx<R> sample(const cpx<R>* line, int n, long long idx) {
    return (idx >= 0 && idx < n) ? line[idx] : mk((R)0, (R)0);
}

// One output per lane at position t (lanes with act false return 0 and only
// take part in the shuffles; every lane of the warp must call this).  When the
// taps of the warp's active lanes span fewer than 64 samples, each lane loads
// two samples of that window and the taps come from their owners by warp
// shuffles; otherwise they are read from the line directly.  Both paths add
// the same products in the same order (idx ascending).
template <typename R>
__device__ __forceinline__ cpx<R> sinc_warp(const cpx<R>* line, int n, double t, int L, bool act) {
    const int lane = threadIdx.x & 31;
    // positions far outside the line touch no sample; keep floor() in int range
    t = fmin(fmax(t, -1.0e9), 1.0e9);
    const int n0 = (int)floor(t);
    const int lo = __reduce_min_sync(0xffffffffu, act ? n0 - L : INT_MAX);
    const int hi = __reduce_max_sync(0xffffffffu, act ? n0 + L : INT_MIN);
    cpx<R> acc = mk((R)0, (R)0);
    if (hi - lo < 64) {
        const cpx<R> s0 = sample(line, n, (long long)lo + lane);
        const cpx<R> s1 = sample(line, n, (long long)lo + 32 + lane);
        for (int j = -L; j <= L; ++j) {
            const int idx = n0 + j;
            const int q = act ? idx - lo : 0;   // 0 <= q < 64 on active lanes
            const cpx<R> v0 = shfl(s0, q & 31);
            const cpx<R> v1 = shfl(s1, q & 31);
            if (act && idx >= 0 && idx < n) acc = acc + (q < 32 ? v0 : v1) * sinc_weight<R>(t - (double)idx, L);
        }
    } else if (act) {
        for (int j = -L; j <= L; ++j) {
            const int idx = n0 + j;
            if (idx < 0 || idx >= n) continue;
            acc = acc + line[idx] * sinc_weight<R>(t - (double)idx, L);
        }
    }
    return acc;
}

}  // namespace s1g
