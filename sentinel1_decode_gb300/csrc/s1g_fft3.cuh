// FP32 shared-memory FFT core with radix-16 stages and shared-memory
// twiddles.
//
// Same in-place structure as s1g_fft2.cuh (decimation in time from
// digit-reversed positions, decimation in frequency to digit-reversed
// positions, padded layout pad(i)), with two changes aimed at the counters of
// the earlier core (twiddle gathers from L2 on the critical path, five to six
// shared-memory passes for 10^4-point transforms):
//   * radix 16 for the power-of-two part (two radix-4 layers in registers
//     with constant inner twiddles), so an 8192-point transform takes 4
//     passes instead of 5;
//   * twiddles exp(-2 pi i e / n) from two small tables staged in shared
//     memory once per block: W[e] = HI[e >> 6] * LO[e & 63], with HI and LO
//     rounded from FP64 (error about 1.5 ulp; n/64 + 64 entries).
#pragma once

#include "s1g_fft2.cuh"

namespace s1g {

struct Fft3Desc {
    int n = 0;
    int nstages = 0;
    int8_t radix[kMaxStages] = {};
    const int* perm = nullptr;   // digit-reversed position of index j
    const cf32* tw = nullptr;    // [nhi] HI then [64] LO, exp(-2 pi i (64 q) / n) and exp(-2 pi i q / n)
};

__host__ __device__ inline int fft3_nhi(int n) { return (n + 63) / 64; }
// shared-memory floats (cf32 count) taken by the twiddle tables
__host__ __device__ inline int fft3_tw_len(int n) { return fft3_nhi(n) + 64; }

// Stage the twiddle tables into shared memory (all threads; caller syncs).
__device__ __forceinline__ void fft3_stage_tw(cf32* smtw, const Fft3Desc& d) {
    const int m = fft3_tw_len(d.n);
    for (int i = threadIdx.x; i < m; i += blockDim.x) smtw[i] = ldg(d.tw + i);
}

__device__ __forceinline__ cf32 tw3(const cf32* smtw, int nhi, int e, int dir) {
    const cf32 w = smtw[e >> 6] * smtw[nhi + (e & 63)];
    return dir > 0 ? conj(w) : w;
}

// 16-point butterfly: X[s] = sum_r a[r] W^{r s}, W = exp(dir 2 pi i / 16), as
// 4 x 4 (r = r0 + 4 r1, s = s0 + 4 s1) with inner twiddles W^{r0 s0}.
template <typename R>
struct Bfly<R, 16> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        const R c1 = (R)0.92387953251128675613, s1 = (R)0.38268343236508977173;
        const R h = (R)0.70710678118654752440;
        cpx<R> b[4][4];
#pragma unroll
        for (int r0 = 0; r0 < 4; ++r0) {
            cpx<R> v[4] = {a[r0], a[r0 + 4], a[r0 + 8], a[r0 + 12]};
            Bfly<R, 4>::run(v, dir);
#pragma unroll
            for (int s0 = 0; s0 < 4; ++s0) b[r0][s0] = v[s0];
        }
        // inner twiddles W^{r0 s0}: W^1 = c1 + dir i s1, W^2 = h (1 + dir i),
        // W^3 = s1 + dir i c1, W^4 = dir i, W^6 = h (-1 + dir i), W^9 = -c1 - dir i s1
        const R d = (R)dir;
        auto rot = [&](cpx<R> v, R c, R s) { return mk(c * v.x - d * s * v.y, c * v.y + d * s * v.x); };
        b[1][1] = rot(b[1][1], c1, s1);
        b[1][2] = rot(b[1][2], h, h);
        b[1][3] = rot(b[1][3], s1, c1);
        b[2][1] = rot(b[2][1], h, h);
        b[2][2] = mul_i(b[2][2], dir);
        b[2][3] = rot(b[2][3], -h, h);
        b[3][1] = rot(b[3][1], s1, c1);
        b[3][2] = rot(b[3][2], -h, h);
        b[3][3] = rot(b[3][3], -c1, -s1);
#pragma unroll
        for (int s0 = 0; s0 < 4; ++s0) {
            cpx<R> v[4] = {b[0][s0], b[1][s0], b[2][s0], b[3][s0]};
            Bfly<R, 4>::run(v, dir);
#pragma unroll
            for (int s1i = 0; s1i < 4; ++s1i) a[s0 + 4 * s1i] = v[s1i];
        }
    }
};

// a[r] *= W^(r e1) for r = 1..P-1 (W = exp(dir 2 pi i / n)).  Only the powers
// W^e1, W^2e1, W^4e1, W^8e1 below P come from the tables; the others are their
// products (at most three, ~6 ulp), which halves the shared-memory traffic of a
// radix-16 pass (twiddle loads were half of it).
template <int P>
__device__ __forceinline__ void apply_tw(cf32* a, const cf32* smtw, int nhi, int e1, int dir) {
    if (P == 16) {
        const cf32 w1 = tw3(smtw, nhi, e1, dir), w2 = tw3(smtw, nhi, 2 * e1, dir);
        const cf32 w4 = tw3(smtw, nhi, 4 * e1, dir), w8 = tw3(smtw, nhi, 8 * e1, dir);
        a[1] = a[1] * w1;
        a[2] = a[2] * w2;
        a[4] = a[4] * w4;
        a[8] = a[8] * w8;
        a[9] = a[9] * (w1 * w8);
        a[10] = a[10] * (w2 * w8);
        a[12] = a[12] * (w4 * w8);
        const cf32 w3 = w1 * w2;
        a[3] = a[3] * w3;
        a[11] = a[11] * (w3 * w8);
        const cf32 w5 = w1 * w4;
        a[5] = a[5] * w5;
        a[13] = a[13] * (w5 * w8);
        const cf32 w6 = w2 * w4;
        a[6] = a[6] * w6;
        a[14] = a[14] * (w6 * w8);
        const cf32 w7 = w3 * w4;
        a[7] = a[7] * w7;
        a[15] = a[15] * (w7 * w8);
    } else if (P == 8) {
        const cf32 w1 = tw3(smtw, nhi, e1, dir), w2 = tw3(smtw, nhi, 2 * e1, dir);
        const cf32 w4 = tw3(smtw, nhi, 4 * e1, dir);
        a[1] = a[1] * w1;
        a[2] = a[2] * w2;
        a[4] = a[4] * w4;
        const cf32 w3 = w1 * w2;
        a[3] = a[3] * w3;
        a[5] = a[5] * (w1 * w4);
        a[6] = a[6] * (w2 * w4);
        a[7] = a[7] * (w3 * w4);
    } else {
        // P = 3, 4, 5, 7: W^e1, W^2e1 (, W^4e1) from the tables, the rest products
        cf32 wp[3];
#pragma unroll
        for (int b = 0; b < 3; ++b)
            if ((1 << b) < P) wp[b] = tw3(smtw, nhi, e1 << b, dir);
#pragma unroll
        for (int r = 1; r < P; ++r) {
            cf32 w = mk(1.f, 0.f);
            bool first = true;
#pragma unroll
            for (int b = 0; b < 3; ++b)
                if (r & (1 << b)) {
                    w = first ? wp[b] : w * wp[b];
                    first = false;
                }
            a[r] = a[r] * w;
        }
    }
}

template <int P>
__device__ __forceinline__ void dit3_stage(cf32* buf, int n, int Ns, int dir, const cf32* smtw, int nhi) {
    const int nb = n / P;
    const int step = n / (Ns * P);
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * Ns * P + k;
        cf32 a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) a[r] = buf[pad(base + r * Ns)];
        if (Ns > 1) apply_tw<P>(a, smtw, nhi, k * step, dir);
        Bfly<float, P>::run(a, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) buf[pad(base + s * Ns)] = a[s];
    }
}

template <int P>
__device__ __forceinline__ void dif3_stage(cf32* buf, int n, int Ns, int dir, const cf32* smtw, int nhi) {
    const int nb = n / P;
    const int step = n / (Ns * P);
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * Ns * P + k;
        cf32 a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) a[r] = buf[pad(base + r * Ns)];
        Bfly<float, P>::run(a, dir);
        if (Ns > 1) apply_tw<P>(a, smtw, nhi, k * step, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) buf[pad(base + s * Ns)] = a[s];
    }
}

// Input at pad(perm[j]) -> natural order output at pad(k).  smtw holds the
// staged twiddle tables of d.
__device__ __forceinline__ void fft3_dit(cf32* buf, const Fft3Desc& d, int dir, const cf32* smtw) {
    const int nhi = fft3_nhi(d.n);
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        switch (p) {
            case 2: dit3_stage<2>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 3: dit3_stage<3>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 4: dit3_stage<4>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 5: dit3_stage<5>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 7: dit3_stage<7>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 8: dit3_stage<8>(buf, d.n, Ns, dir, smtw, nhi); break;
            default: dit3_stage<16>(buf, d.n, Ns, dir, smtw, nhi); break;
        }
        __syncthreads();
        Ns *= p;
    }
}

// Natural order input at pad(k) -> output at pad(perm[j]).
__device__ __forceinline__ void fft3_dif(cf32* buf, const Fft3Desc& d, int dir, const cf32* smtw) {
    const int nhi = fft3_nhi(d.n);
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        switch (p) {
            case 2: dif3_stage<2>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 3: dif3_stage<3>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 4: dif3_stage<4>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 5: dif3_stage<5>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 7: dif3_stage<7>(buf, d.n, Ns, dir, smtw, nhi); break;
            case 8: dif3_stage<8>(buf, d.n, Ns, dir, smtw, nhi); break;
            default: dif3_stage<16>(buf, d.n, Ns, dir, smtw, nhi); break;
        }
        __syncthreads();
    }
}

}  // namespace s1g
