// Compensated FP32 FFT in shared memory (device side).
//
// Each complex value is carried as an unevaluated sum h + e of two cf32: h is
// the ordinary FP32 result and e accumulates, in FP32, the rounding error of
// every operation that produced h.  Additions use TwoSum and products use
// TwoProd (fused multiply-add) to capture their rounding errors exactly; the
// error terms themselves are propagated to first order without
// renormalisation (the compensated Cooley-Tukey scheme of Jiang, Graillat,
// Hu, Luo & Rump, "Accurate complex multiplication and FFT in floating-point
// arithmetic", restated for float pairs).  The result h + e carries about
// 1e-13 relative error, against ~2e-7 for the plain FP32 core, at roughly
// six times the arithmetic.  Twiddles are exp(-2 pi i k/n) split into float
// pairs from FP64.
//
// Layout: two padded arrays H[pad(i)], E[pad(i)] (s1g_fft2.cuh padding).
// Radices 2, 3 and 4 only (transform lengths 2^a 3^b).  dit: input at
// pad(perm[j]), output natural; dif: natural input, output at pad(perm[j]).
#pragma once

#include "s1g_df.cuh"
#include "s1g_fft2.cuh"

namespace s1g {

struct CfftDesc {
    int n = 0;
    int nstages = 0;
    int8_t radix[kMaxStages] = {};
    const float4* tw = nullptr;  // {cos hi, -sin hi, cos lo, -sin lo} of exp(-2 pi i k / n)
    const int* perm = nullptr;
};

struct cc {
    float hx, hy, ex, ey;
};

__device__ __forceinline__ cc cc_make(cf32 h, cf32 e) { return cc{h.x, h.y, e.x, e.y}; }

__device__ __forceinline__ cc cc_add(const cc& a, const cc& b) {
    const df sx = two_sum(a.hx, b.hx);
    const df sy = two_sum(a.hy, b.hy);
    return cc{sx.hi, sy.hi, sx.lo + (a.ex + b.ex), sy.lo + (a.ey + b.ey)};
}

__device__ __forceinline__ cc cc_sub(const cc& a, const cc& b) {
    const df sx = two_sum(a.hx, -b.hx);
    const df sy = two_sum(a.hy, -b.hy);
    return cc{sx.hi, sy.hi, sx.lo + (a.ex - b.ex), sy.lo + (a.ey - b.ey)};
}

// times dir * i (exact)
__device__ __forceinline__ cc cc_mul_i(const cc& a, int dir) {
    return dir > 0 ? cc{-a.hy, a.hx, -a.ey, a.ex} : cc{a.hy, -a.hx, a.ey, -a.ex};
}

// times the float-pair complex w = (wx + wlx) + i (wy + wly)
__device__ __forceinline__ cc cc_mul(const cc& a, float wx, float wy, float wlx, float wly) {
    const df p1 = two_prod(a.hx, wx);
    const df p2 = two_prod(a.hy, wy);
    const df s = two_sum(p1.hi, -p2.hi);
    const float er = s.lo + (p1.lo - p2.lo) + (a.hx * wlx - a.hy * wly) + (a.ex * wx - a.ey * wy);
    const df q1 = two_prod(a.hx, wy);
    const df q2 = two_prod(a.hy, wx);
    const df t = two_sum(q1.hi, q2.hi);
    const float ei = t.lo + (q1.lo + q2.lo) + (a.hx * wly + a.hy * wlx) + (a.ex * wy + a.ey * wx);
    return cc{s.hi, t.hi, er, ei};
}

// twiddle exp(dir 2 pi i idx / n) from the table
__device__ __forceinline__ cc cc_twiddle(const cc& a, const float4* tw, int idx, int dir) {
    const float4 w = __ldg(tw + idx);
    return dir > 0 ? cc_mul(a, w.x, -w.y, w.z, -w.w) : cc_mul(a, w.x, w.y, w.z, w.w);
}

// times a real float pair (c + cl)
__device__ __forceinline__ cc cc_scale(const cc& a, float c, float cl) {
    const df px = two_prod(a.hx, c);
    const df py = two_prod(a.hy, c);
    return cc{px.hi, py.hi, px.lo + a.hx * cl + a.ex * c, py.lo + a.hy * cl + a.ey * c};
}

template <int P>
struct CBfly;

template <>
struct CBfly<2> {
    static __device__ __forceinline__ void run(cc* a, int) {
        const cc t = a[0];
        a[0] = cc_add(t, a[1]);
        a[1] = cc_sub(t, a[1]);
    }
};

template <>
struct CBfly<4> {
    static __device__ __forceinline__ void run(cc* a, int dir) {
        const cc t0 = cc_add(a[0], a[2]), t1 = cc_sub(a[0], a[2]);
        const cc t2 = cc_add(a[1], a[3]), t3 = cc_mul_i(cc_sub(a[1], a[3]), dir);
        a[0] = cc_add(t0, t2);
        a[2] = cc_sub(t0, t2);
        a[1] = cc_add(t1, t3);
        a[3] = cc_sub(t1, t3);
    }
};

template <>
struct CBfly<3> {
    // X1 = a0 - (a1 + a2)/2 + dir i (sqrt(3)/2) (a1 - a2), X2 the conjugate combination
    static __device__ __forceinline__ void run(cc* a, int dir) {
        const cc t = cc_add(a[1], a[2]);
        const cc d = cc_sub(a[1], a[2]);
        const cc x0 = cc_add(a[0], t);
        const cc half = cc{0.5f * t.hx, 0.5f * t.hy, 0.5f * t.ex, 0.5f * t.ey};
        const cc m = cc_sub(a[0], half);
        const cc r = cc_mul_i(cc_scale(d, 0.866025388240814209f, 1.55436250537377420e-08f), dir);
        a[0] = x0;
        a[1] = cc_add(m, r);
        a[2] = cc_sub(m, r);
    }
};

template <int P>
__device__ __forceinline__ void cdit_stage(cf32* H, cf32* E, const CfftDesc& d, int Ns, int dir) {
    const int n = d.n;
    const int nb = n / P;
    const int span = Ns * P;
    const int step = n / span;
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * span + k;
        cc a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const int i = pad(base + r * Ns);
            a[r] = cc_make(H[i], E[i]);
        }
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < P; ++r) a[r] = cc_twiddle(a[r], d.tw, r * k * step, dir);
        }
        CBfly<P>::run(a, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int i = pad(base + s * Ns);
            H[i] = mk(a[s].hx, a[s].hy);
            E[i] = mk(a[s].ex, a[s].ey);
        }
    }
}

template <int P>
__device__ __forceinline__ void cdif_stage(cf32* H, cf32* E, const CfftDesc& d, int Ns, int dir) {
    const int n = d.n;
    const int nb = n / P;
    const int span = Ns * P;
    const int step = n / span;
    const float inv = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        int g, k;
        split_idx(t, Ns, inv, g, k);
        const int base = g * span + k;
        cc a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const int i = pad(base + r * Ns);
            a[r] = cc_make(H[i], E[i]);
        }
        CBfly<P>::run(a, dir);
        if (Ns > 1) {
#pragma unroll
            for (int s = 1; s < P; ++s) a[s] = cc_twiddle(a[s], d.tw, s * k * step, dir);
        }
#pragma unroll
        for (int s = 0; s < P; ++s) {
            const int i = pad(base + s * Ns);
            H[i] = mk(a[s].hx, a[s].hy);
            E[i] = mk(a[s].ex, a[s].ey);
        }
    }
}

__device__ __forceinline__ void cfft_dit(cf32* H, cf32* E, const CfftDesc& d, int dir) {
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        if (p == 4) cdit_stage<4>(H, E, d, Ns, dir);
        else if (p == 3) cdit_stage<3>(H, E, d, Ns, dir);
        else cdit_stage<2>(H, E, d, Ns, dir);
        __syncthreads();
        Ns *= p;
    }
}

__device__ __forceinline__ void cfft_dif(cf32* H, cf32* E, const CfftDesc& d, int dir) {
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        if (p == 4) cdif_stage<4>(H, E, d, Ns, dir);
        else if (p == 3) cdif_stage<3>(H, E, d, Ns, dir);
        else cdif_stage<2>(H, E, d, Ns, dir);
        __syncthreads();
    }
}

}  // namespace s1g
