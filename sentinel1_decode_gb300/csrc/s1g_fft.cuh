// Shared-memory mixed-radix FFT building blocks (device side).
//
// In-place iterative Cooley-Tukey over a factor list of radices {2,3,4,5,7,8}:
//   * fft_dit: input must be stored at digit-reversed positions (perm[j]),
//     output comes out in natural order;
//   * fft_dif: natural-order input, output at digit-reversed positions.
// Using DIT for a forward transform and DIF for the following inverse lets a
// kernel go signal -> spectrum -> signal in one shared buffer with no
// permutation pass in between (the spectrum is in natural order for the
// pointwise filter).  Both are unnormalised; dir=-1 is exp(-2 pi i jk/n),
// dir=+1 is exp(+2 pi i jk/n).  All threads of the block must call them, and
// the caller synchronises after filling the buffer.
#pragma once

#include "s1g_complex.cuh"

namespace s1g {

constexpr int kMaxStages = 24;

template <typename R>
struct FftDesc {
    int n = 0;
    int nstages = 0;
    int8_t radix[kMaxStages] = {};
    const cpx<R>* tw = nullptr;  // tw[i] = exp(-2 pi i * i / n), i < n
    const int* perm = nullptr;   // digit-reversed position of index j, j < n
};

template <typename R>
__device__ __forceinline__ cpx<R> twid(const FftDesc<R>& d, int idx, int dir) {
    cpx<R> w = ldg(d.tw + idx);
    return dir > 0 ? conj(w) : w;
}

// ---------------------------------------------------------------- butterflies
template <typename R, int P>
struct Bfly;

template <typename R>
struct Bfly<R, 2> {
    static __device__ __forceinline__ void run(cpx<R>* a, int) {
        cpx<R> t = a[0];
        a[0] = t + a[1];
        a[1] = t - a[1];
    }
};

template <typename R>
struct Bfly<R, 4> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        cpx<R> t0 = a[0] + a[2], t1 = a[0] - a[2];
        cpx<R> t2 = a[1] + a[3], t3 = mul_i(a[1] - a[3], dir);
        a[0] = t0 + t2;
        a[2] = t0 - t2;
        a[1] = t1 + t3;
        a[3] = t1 - t3;
    }
};

template <typename R>
struct Bfly<R, 8> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        const R h = (R)0.70710678118654752440;
        cpx<R> e[4] = {a[0], a[2], a[4], a[6]};
        cpx<R> o[4] = {a[1], a[3], a[5], a[7]};
        Bfly<R, 4>::run(e, dir);
        Bfly<R, 4>::run(o, dir);
        // w8^1 = h(1 + dir i), w8^2 = dir i, w8^3 = h(-1 + dir i)
        cpx<R> o1 = mk(h * (o[1].x - dir * o[1].y), h * (o[1].y + dir * o[1].x));
        cpx<R> o2 = mul_i(o[2], dir);
        cpx<R> o3 = mk(h * (-o[3].x - dir * o[3].y), h * (-o[3].y + dir * o[3].x));
        a[0] = e[0] + o[0];
        a[4] = e[0] - o[0];
        a[1] = e[1] + o1;
        a[5] = e[1] - o1;
        a[2] = e[2] + o2;
        a[6] = e[2] - o2;
        a[3] = e[3] + o3;
        a[7] = e[3] - o3;
    }
};

template <typename R>
struct Bfly<R, 3> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        const R c = (R)-0.5, s = (R)0.86602540378443864676;
        cpx<R> sum = a[1] + a[2], dif = a[1] - a[2];
        cpx<R> m = a[0] + sum * c;
        cpx<R> r = mul_i(dif, dir) * s;
        a[0] = a[0] + sum;
        a[1] = m + r;
        a[2] = m - r;
    }
};

template <typename R>
struct Bfly<R, 5> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;
        const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;
        cpx<R> t1 = a[1] + a[4], t2 = a[2] + a[3], t3 = a[1] - a[4], t4 = a[2] - a[3];
        cpx<R> m1 = a[0] + t1 * c1 + t2 * c2;
        cpx<R> m2 = a[0] + t1 * c2 + t2 * c1;
        cpx<R> r1 = mul_i(t3 * s1 + t4 * s2, dir);
        cpx<R> r2 = mul_i(t3 * s2 - t4 * s1, dir);
        a[0] = a[0] + t1 + t2;
        a[1] = m1 + r1;
        a[4] = m1 - r1;
        a[2] = m2 + r2;
        a[3] = m2 - r2;
    }
};

template <typename R>
struct Bfly<R, 7> {
    static __device__ __forceinline__ void run(cpx<R>* a, int dir) {
        const R C[7] = {(R)1.0, (R)0.62348980185873353053, (R)-0.22252093395631440429,
                        (R)-0.90096886790241912624, (R)-0.90096886790241912624,
                        (R)-0.22252093395631440429, (R)0.62348980185873353053};
        const R S[7] = {(R)0.0, (R)0.78183148246802980871, (R)0.97492791218182360702,
                        (R)0.43388373911755812048, (R)-0.43388373911755812048,
                        (R)-0.97492791218182360702, (R)-0.78183148246802980871};
        cpx<R> t[4], u[4];
#pragma unroll
        for (int k = 1; k <= 3; ++k) {
            t[k] = a[k] + a[7 - k];
            u[k] = a[k] - a[7 - k];
        }
        cpx<R> out[7];
        out[0] = a[0] + t[1] + t[2] + t[3];
#pragma unroll
        for (int m = 1; m <= 6; ++m) {
            cpx<R> re = a[0], im = mk((R)0, (R)0);
#pragma unroll
            for (int k = 1; k <= 3; ++k) {
                const int q = (k * m) % 7;
                re = re + t[k] * C[q];
                im = im + u[k] * S[q];
            }
            out[m] = re + mul_i(im, dir);
        }
#pragma unroll
        for (int m = 0; m < 7; ++m) a[m] = out[m];
    }
};

// ---------------------------------------------------------------- stages
template <typename R, int P>
__device__ __forceinline__ void dit_stage(cpx<R>* buf, const FftDesc<R>& d, int Ns, int dir) {
    const int nb = d.n / P;
    const int span = Ns * P;
    const int twstep = d.n / span;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        const int k = t % Ns;
        const int base = (t / Ns) * span + k;
        cpx<R> a[P];
        a[0] = buf[base];
#pragma unroll
        for (int r = 1; r < P; ++r) a[r] = buf[base + r * Ns] * twid(d, r * k * twstep, dir);
        Bfly<R, P>::run(a, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) buf[base + s * Ns] = a[s];
    }
}

template <typename R, int P>
__device__ __forceinline__ void dif_stage(cpx<R>* buf, const FftDesc<R>& d, int Ns, int dir) {
    const int nb = d.n / P;
    const int span = Ns * P;
    const int twstep = d.n / span;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        const int k = t % Ns;
        const int base = (t / Ns) * span + k;
        cpx<R> a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) a[r] = buf[base + r * Ns];
        Bfly<R, P>::run(a, dir);
        buf[base] = a[0];
#pragma unroll
        for (int s = 1; s < P; ++s) buf[base + s * Ns] = a[s] * twid(d, s * k * twstep, dir);
    }
}

template <typename R>
__device__ __forceinline__ void dit_dispatch(cpx<R>* buf, const FftDesc<R>& d, int p, int Ns, int dir) {
    switch (p) {
        case 2: dit_stage<R, 2>(buf, d, Ns, dir); break;
        case 3: dit_stage<R, 3>(buf, d, Ns, dir); break;
        case 4: dit_stage<R, 4>(buf, d, Ns, dir); break;
        case 5: dit_stage<R, 5>(buf, d, Ns, dir); break;
        case 7: dit_stage<R, 7>(buf, d, Ns, dir); break;
        default: dit_stage<R, 8>(buf, d, Ns, dir); break;
    }
}

template <typename R>
__device__ __forceinline__ void dif_dispatch(cpx<R>* buf, const FftDesc<R>& d, int p, int Ns, int dir) {
    switch (p) {
        case 2: dif_stage<R, 2>(buf, d, Ns, dir); break;
        case 3: dif_stage<R, 3>(buf, d, Ns, dir); break;
        case 4: dif_stage<R, 4>(buf, d, Ns, dir); break;
        case 5: dif_stage<R, 5>(buf, d, Ns, dir); break;
        case 7: dif_stage<R, 7>(buf, d, Ns, dir); break;
        default: dif_stage<R, 8>(buf, d, Ns, dir); break;
    }
}

// Batched variants: nbatch transforms of length d.n stored back to back.
template <typename R, int P>
__device__ __forceinline__ void dit_stage_b(cpx<R>* buf, const FftDesc<R>& d, int Ns, int dir, int nbatch) {
    const int nb = d.n / P;
    const int span = Ns * P;
    const int twstep = d.n / span;
    for (int t = threadIdx.x; t < nb * nbatch; t += blockDim.x) {
        const int w = t / nb, tt = t - w * nb;
        const int k = tt % Ns;
        const int base = w * d.n + (tt / Ns) * span + k;
        cpx<R> a[P];
        a[0] = buf[base];
#pragma unroll
        for (int r = 1; r < P; ++r) a[r] = buf[base + r * Ns] * twid(d, r * k * twstep, dir);
        Bfly<R, P>::run(a, dir);
#pragma unroll
        for (int s = 0; s < P; ++s) buf[base + s * Ns] = a[s];
    }
}

template <typename R, int P>
__device__ __forceinline__ void dif_stage_b(cpx<R>* buf, const FftDesc<R>& d, int Ns, int dir, int nbatch) {
    const int nb = d.n / P;
    const int span = Ns * P;
    const int twstep = d.n / span;
    for (int t = threadIdx.x; t < nb * nbatch; t += blockDim.x) {
        const int w = t / nb, tt = t - w * nb;
        const int k = tt % Ns;
        const int base = w * d.n + (tt / Ns) * span + k;
        cpx<R> a[P];
#pragma unroll
        for (int r = 0; r < P; ++r) a[r] = buf[base + r * Ns];
        Bfly<R, P>::run(a, dir);
        buf[base] = a[0];
#pragma unroll
        for (int s = 1; s < P; ++s) buf[base + s * Ns] = a[s] * twid(d, s * k * twstep, dir);
    }
}

template <typename R>
__device__ void fft_dit_batched(cpx<R>* buf, const FftDesc<R>& d, int dir, int nbatch) {
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        switch (p) {
            case 2: dit_stage_b<R, 2>(buf, d, Ns, dir, nbatch); break;
            case 3: dit_stage_b<R, 3>(buf, d, Ns, dir, nbatch); break;
            case 4: dit_stage_b<R, 4>(buf, d, Ns, dir, nbatch); break;
            case 5: dit_stage_b<R, 5>(buf, d, Ns, dir, nbatch); break;
            case 7: dit_stage_b<R, 7>(buf, d, Ns, dir, nbatch); break;
            default: dit_stage_b<R, 8>(buf, d, Ns, dir, nbatch); break;
        }
        __syncthreads();
        Ns *= p;
    }
}

template <typename R>
__device__ void fft_dif_batched(cpx<R>* buf, const FftDesc<R>& d, int dir, int nbatch) {
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        switch (p) {
            case 2: dif_stage_b<R, 2>(buf, d, Ns, dir, nbatch); break;
            case 3: dif_stage_b<R, 3>(buf, d, Ns, dir, nbatch); break;
            case 4: dif_stage_b<R, 4>(buf, d, Ns, dir, nbatch); break;
            case 5: dif_stage_b<R, 5>(buf, d, Ns, dir, nbatch); break;
            case 7: dif_stage_b<R, 7>(buf, d, Ns, dir, nbatch); break;
            default: dif_stage_b<R, 8>(buf, d, Ns, dir, nbatch); break;
        }
        __syncthreads();
    }
}

// Input at perm[] positions -> natural-order output.
template <typename R>
__device__ void fft_dit(cpx<R>* buf, const FftDesc<R>& d, int dir) {
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        dit_dispatch(buf, d, p, Ns, dir);
        __syncthreads();
        Ns *= p;
    }
}

// Natural-order input -> output at perm[] positions.
template <typename R>
__device__ void fft_dif(cpx<R>* buf, const FftDesc<R>& d, int dir) {
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        dif_dispatch(buf, d, p, Ns, dir);
        __syncthreads();
    }
}

}  // namespace s1g
