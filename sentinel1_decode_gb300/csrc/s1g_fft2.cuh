// FP32 shared-memory FFT core of the fused kernels.
//
// Same in-place decimation-in-time / -frequency structure as s1g_fft.cuh
// (digit-reversed positions from FftDesc::perm), tuned for throughput:
//   * one twiddle-table load per butterfly (the base root), higher powers by
//     a depth-3 complex multiplication tree;
//   * shared-memory layout padded by one element per 32 (pad()), which
//     removes the 8- and 16-way bank conflicts of the short-span stages;
//   * butterfly index split (group, offset) with a float reciprocal and one
//     correction step instead of integer division.
// Accuracy: a few 1e-7 relative per transform.
#pragma once

#include "s1g_fft.cuh"

namespace s1g {

__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }
__host__ __device__ inline int padded_len(int n) { return n + (n >> 5) + 1; }

// t = g * ns + k with 0 <= k < ns (t < 2^24)
__device__ __forceinline__ void split_idx(int t, int ns, float inv_ns, int& g, int& k) {
    g = __float2int_rz((float)t * inv_ns);
    k = t - g * ns;
    if (k < 0) {
        --g;
        k += ns;
    } else if (k >= ns) {
        ++g;
        k -= ns;
    }
}

// exp(dir * 2 pi i * num / den), 0 <= num < den, argument reduced to [-pi, pi]
__device__ __forceinline__ cf32 root_fast(int num, int den, int dir) {
    float a = (float)num / (float)den;
    if (a > 0.5f) a -= 1.0f;
    float s, c;
    __sincosf(6.28318530717958648f * a, &s, &c);
    return mk(c, dir > 0 ? s : -s);
}

// w[r] = w1^r by a multiplication tree of depth <= 3 (keeps the rounding of
// the highest power within a few ulps).
template <int P>
__device__ __forceinline__ void powers(cf32 w1, cf32* w) {
    w[1] = w1;
    if (P > 2) w[2] = w1 * w1;
    if (P > 3) w[3] = w[2] * w1;
    if (P > 4) w[4] = w[2] * w[2];
    if (P > 5) w[5] = w[4] * w1;
    if (P > 6) w[6] = w[4] * w[2];
    if (P > 7) w[7] = w[4] * w[3];
}

// exp(dir 2 pi i k / span) from the FP64-accurate table of the transform
__device__ __forceinline__ cf32 root_tab(const cf32* tw, int k, int step, int dir) {
    const cf32 w = ldg(tw + k * step);
    return dir > 0 ? conj(w) : w;
}

template <int P>
__device__ __forceinline__ void dit2_stage(cf32* buf, int n, int Ns, int dir, const cf32* tw) {
    const int nb = n / P;
    const int span = Ns * P;
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * span + k;
        cf32 a[P];
        a[0] = buf[pad(base)];
        if (Ns > 1) {
            cf32 w[P];
            const int step = n / span;
#pragma unroll
            for (int r = 1; r < P; ++r) w[r] = root_tab(tw, r * k, step, dir);
#pragma unroll
            for (int r = 1; r < P; ++r) a[r] = buf[pad(base + r * Ns)] * w[r];
        } else {
#pragma unroll
            for (int r = 1; r < P; ++r) a[r] = buf[pad(base + r * Ns)];
        }
        Bfly<float, P>::run(a, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) buf[pad(base + s * Ns)] = a[s];
    }
}

template <int P>
__device__ __forceinline__ void dif2_stage(cf32* buf, int n, int Ns, int dir, const cf32* tw) {
    const int nb = n / P;
    const int span = Ns * P;
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * span + k;
        cf32 a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) a[r] = buf[pad(base + r * Ns)];
        Bfly<float, P>::run(a, dir);
        buf[pad(base)] = a[0];
        if (Ns > 1) {
            cf32 w[P];
            const int step = n / span;
#pragma unroll
            for (int r = 1; r < P; ++r) w[r] = root_tab(tw, r * k, step, dir);
#pragma unroll
            for (int s = 1; s < P; ++s) buf[pad(base + s * Ns)] = a[s] * w[s];
        } else {
#pragma unroll
            for (int s = 1; s < P; ++s) buf[pad(base + s * Ns)] = a[s];
        }
    }
}

// Input at pad(perm[j]) -> natural order output at pad(k).
__device__ __forceinline__ void fft2_dit(cf32* buf, const FftDesc<float>& d, int dir) {
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        switch (p) {
            case 2: dit2_stage<2>(buf, d.n, Ns, dir, d.tw); break;
            case 3: dit2_stage<3>(buf, d.n, Ns, dir, d.tw); break;
            case 4: dit2_stage<4>(buf, d.n, Ns, dir, d.tw); break;
            case 5: dit2_stage<5>(buf, d.n, Ns, dir, d.tw); break;
            case 7: dit2_stage<7>(buf, d.n, Ns, dir, d.tw); break;
            default: dit2_stage<8>(buf, d.n, Ns, dir, d.tw); break;
        }
        __syncthreads();
        Ns *= p;
    }
}

// Natural order input at pad(k) -> output at pad(perm[j]).
__device__ __forceinline__ void fft2_dif(cf32* buf, const FftDesc<float>& d, int dir) {
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        switch (p) {
            case 2: dif2_stage<2>(buf, d.n, Ns, dir, d.tw); break;
            case 3: dif2_stage<3>(buf, d.n, Ns, dir, d.tw); break;
            case 4: dif2_stage<4>(buf, d.n, Ns, dir, d.tw); break;
            case 5: dif2_stage<5>(buf, d.n, Ns, dir, d.tw); break;
            case 7: dif2_stage<7>(buf, d.n, Ns, dir, d.tw); break;
            default: dif2_stage<8>(buf, d.n, Ns, dir, d.tw); break;
        }
        __syncthreads();
    }
}

}  // namespace s1g
