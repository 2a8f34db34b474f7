// The ECCM notch of the FP32 pipelines in compensated FP32 arithmetic.
//
// eccm() (signal_processing.cpp:914-1004) zeroes the bins of 128-point
// short-time spectra whose central-difference gradient magnitude reaches the
// mitigation threshold.  Those are hard decisions, and the notched lines feed
// the Doppler-centroid estimate, whose sums turn ~2e-7 relative noise into
// SLC errors beyond 1e-4; the FP32 pipelines therefore need the notch to the
// accuracy of the FP64 one.  Here every sample is carried as h + e (two
// complex<float>, s1g_cfft.cuh: TwoSum / TwoProd error terms propagated to
// first order, ~1e-13 relative), taken from the FP64 decoded samples, so the
// gradient decisions are the FP64 path's (up to bins within ~1e-12 of the
// threshold) and the notched samples round to the same floats, at FP32
// arithmetic speed rather than FP64's.
//
// One block per flagged line (flags from k_eccm_detect_mixed below), windows
// of 128 samples at stride 64 in batches of kEccmBatch, forward transform
// from digit-reversed positions, gradient and decision in FP64 from h + e,
// zeroing, inverse transform back to digit-reversed positions, 1/128, and
// each sample written from the last window that covers it (later windows
// overwrite earlier ones).
#include <stdexcept>

#include "s1g_dcest.h"
#include "s1g_fft_engine.h"
#include "s1g_kernels.h"

namespace s1g {

namespace {

constexpr int kEccmFft = 128;
constexpr int kEccmBatch = 16;   // windows per pass

template <int P>
__device__ __forceinline__ void cdit_stage_b(cf32* H, cf32* E, const CfftDesc& d, int Ns, int dir, int nwin) {
    const int n = d.n;
    const int nb = n / P;
    const int span = Ns * P;
    const int step = n / span;
    for (int t = threadIdx.x; t < nwin * nb; t += blockDim.x) {
        const int w = t / nb, tt = t - w * nb;
        const int g = tt / Ns, k = tt - g * Ns;
        const int base = w * n + g * span + k;
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
__device__ __forceinline__ void cdif_stage_b(cf32* H, cf32* E, const CfftDesc& d, int Ns, int dir, int nwin) {
    const int n = d.n;
    const int nb = n / P;
    const int span = Ns * P;
    const int step = n / span;
    for (int t = threadIdx.x; t < nwin * nb; t += blockDim.x) {
        const int w = t / nb, tt = t - w * nb;
        const int g = tt / Ns, k = tt - g * Ns;
        const int base = w * n + g * span + k;
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

// digit-reversed input -> natural output (every window of the batch)
__device__ void cfft_dit_b(cf32* H, cf32* E, const CfftDesc& d, int dir, int nwin) {
    int Ns = 1;
    for (int st = 0; st < d.nstages; ++st) {
        const int p = d.radix[st];
        if (p == 4) cdit_stage_b<4>(H, E, d, Ns, dir, nwin);
        else if (p == 3) cdit_stage_b<3>(H, E, d, Ns, dir, nwin);
        else cdit_stage_b<2>(H, E, d, Ns, dir, nwin);
        __syncthreads();
        Ns *= p;
    }
}

// natural input -> digit-reversed output
__device__ void cfft_dif_b(cf32* H, cf32* E, const CfftDesc& d, int dir, int nwin) {
    int Ns = d.n;
    for (int st = d.nstages - 1; st >= 0; --st) {
        const int p = d.radix[st];
        Ns /= p;
        if (p == 4) cdif_stage_b<4>(H, E, d, Ns, dir, nwin);
        else if (p == 3) cdif_stage_b<3>(H, E, d, Ns, dir, nwin);
        else cdif_stage_b<2>(H, E, d, Ns, dir, nwin);
        __syncthreads();
    }
}

__device__ __forceinline__ double2 cc_value(const cf32* H, const cf32* E, int i) {
    return make_double2((double)H[i].x + (double)E[i].x, (double)H[i].y + (double)E[i].y);
}

}  // namespace

__global__ void __launch_bounds__(256) k_eccm_notch_cc(const cf64* __restrict__ in, long long ip, cf32* __restrict__ out,
                                                       long long op, int n_r, const int* __restrict__ flags,
                                                       double mit, CfftDesc d, int num_ffts) {
    __shared__ cf32 H[kEccmBatch * kEccmFft + (kEccmBatch * kEccmFft) / 32 + 1];
    __shared__ cf32 E[kEccmBatch * kEccmFft + (kEccmBatch * kEccmFft) / 32 + 1];
    __shared__ unsigned char zero[kEccmBatch * kEccmFft];
    const long long row = blockIdx.x;
    if (!flags[row]) return;
    const cf64* line = in + row * ip;
    cf32* o = out + row * op;
    for (int w0 = 0; w0 < num_ffts; w0 += kEccmBatch) {
        const int nw = min(kEccmBatch, num_ffts - w0);
        // windows of the original line, zero-filled past their (cut) end
        for (int t = threadIdx.x; t < nw * kEccmFft; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const int s = (w0 + w) * 64;
            int e = s + kEccmFft;
            if (e > n_r) e = n_r - 1;
            double vx = 0.0, vy = 0.0;
            if (s + q < e) {
                vx = line[s + q].x;
                vy = line[s + q].y;
            }
            const float hx = (float)vx, hy = (float)vy;
            const int i = pad(w * kEccmFft + __ldg(d.perm + q));
            H[i] = mk(hx, hy);
            E[i] = mk((float)(vx - (double)hx), (float)(vy - (double)hy));
        }
        __syncthreads();
        cfft_dit_b(H, E, d, -1, nw);
        // central-difference gradient along frequency (one-sided at the ends)
        for (int t = threadIdx.x; t < nw * kEccmFft; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const int b = w * kEccmFft;
            double2 gr;
            if (q != 0 && q != kEccmFft - 1) {
                const double2 a = cc_value(H, E, pad(b + q + 1)), c = cc_value(H, E, pad(b + q - 1));
                gr = make_double2((a.x - c.x) * 0.5, (a.y - c.y) * 0.5);
            } else if (q == 0) {
                const double2 a = cc_value(H, E, pad(b + 1)), c = cc_value(H, E, pad(b));
                gr = make_double2(a.x - c.x, a.y - c.y);
            } else {
                const double2 a = cc_value(H, E, pad(b + q)), c = cc_value(H, E, pad(b + q - 1));
                gr = make_double2(a.x - c.x, a.y - c.y);
            }
            zero[t] = (hypot(gr.x, gr.y) < mit) ? 0 : 1;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nw * kEccmFft; t += blockDim.x)
            if (zero[t]) {
                const int i = pad(t);
                H[i] = mk(0.f, 0.f);
                E[i] = mk(0.f, 0.f);
            }
        __syncthreads();
        cfft_dif_b(H, E, d, +1, nw);
        for (int t = threadIdx.x; t < nw * kEccmFft; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const int wi = w0 + w;
            const int s = wi * 64;
            int e = s + kEccmFft;
            if (e > n_r) e = n_r - 1;
            const int j = s + q;
            if (j >= e) continue;
            // owner of j: the later of the (at most two) windows covering it
            int owner = -1;
            for (int c = j / 64; c >= j / 64 - 1 && c >= 0; --c) {
                if (c >= num_ffts) continue;
                int ce = c * 64 + kEccmFft;
                if (ce > n_r) ce = n_r - 1;
                if (j < ce) {
                    owner = c;
                    break;
                }
            }
            if (owner != wi) continue;
            const double2 v = cc_value(H, E, pad(w * kEccmFft + __ldg(d.perm + q)));
            o[j] = mk((float)(v.x * (1.0 / 128.0)), (float)(v.y * (1.0 / 128.0)));
        }
        __syncthreads();
    }
}

// ---- line detection from an FP32 spectrum, FP64 where it is close
// A line is flagged when max_k |X_k| >= det.  From the FP32 spectrum of the
// line (FP32 samples and FFT: every |X_k| good to ~1e-6 of det whenever the
// maximum is near det) the decision is certain unless the maximum lies within
// kDetMargin (relative) of det; such a line is decided from the exact FP64
// DFT of its FP64 samples at the bins that could reach det (FP32 magnitude
// >= det (1 - kDetMargin)), one bin at a time by the whole block, stopping at
// the first bin that reaches det.
constexpr double kDetMargin = 1e-4;

__global__ void k_roots64(cf64* __restrict__ roots, int n) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        double sn, cs;
        sincospi(-2.0 * (double)m / (double)n, &sn, &cs);
        cf64 r;
        r.x = cs;
        r.y = sn;
        roots[m] = r;
    }
}

__device__ __forceinline__ double block_sum256(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < 8; ++w) t += red[w];
    return t;   // thread 0
}

__global__ void __launch_bounds__(256) k_eccm_detect_mixed(const cf32* __restrict__ X, long long xp, int n, double det,
                                                           const cf64* __restrict__ x64, long long p64,
                                                           const cf64* __restrict__ roots, int* __restrict__ flags) {
    __shared__ double red[256];
    __shared__ int cand[256];
    __shared__ int ncand, hit;
    const long long row = blockIdx.x;
    const cf32* Xr = X + row * xp;
    double mx = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) {
        const cf32 v = Xr[k];
        mx = fmax(mx, hypot((double)v.x, (double)v.y));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    mx = red[0];
    __syncthreads();
    if (mx < det * (1.0 - kDetMargin) || mx >= det * (1.0 + kDetMargin)) {
        if (threadIdx.x == 0) flags[row] = (mx < det) ? 0 : 1;
        return;
    }
    const cf64* line = x64 + row * p64;
    const double lo = det * (1.0 - kDetMargin);
    if (threadIdx.x == 0) hit = 0;
    for (int base = 0; base < n; base += 256) {
        if (threadIdx.x == 0) ncand = 0;
        __syncthreads();
        const int k = base + threadIdx.x;
        if (k < n) {
            const cf32 v = Xr[k];
            if (hypot((double)v.x, (double)v.y) >= lo) cand[atomicAdd(&ncand, 1)] = k;
        }
        __syncthreads();
        const int nc = ncand;
        for (int c = 0; c < nc; ++c) {
            const long long kk = cand[c];
            long long m = (kk * threadIdx.x) % n;
            const long long step = (kk * 256) % n;
            double re = 0.0, im = 0.0;
            for (int j = threadIdx.x; j < n; j += 256) {
                const cf64 v = line[j], w = roots[m];
                re = fma(v.x, w.x, fma(-v.y, w.y, re));
                im = fma(v.x, w.y, fma(v.y, w.x, im));
                m += step;
                if (m >= n) m -= n;
            }
            re = block_sum256(re, red);
            im = block_sum256(im, red + 8);
            if (threadIdx.x == 0 && !(hypot(re, im) < det)) hit = 1;
            __syncthreads();
            if (hit) break;
        }
        __syncthreads();
        if (hit) break;
    }
    if (threadIdx.x == 0) flags[row] = hit;
}

void eccm_detect_mixed(const cf32* X32, long long xp, int n, long long rows, double det, const cf64* x64,
                       long long p64, cf64* roots, int* flags, cudaStream_t st) {
    if (rows <= 0 || n <= 0) return;
    note_launch(), k_roots64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(roots, n);
    note_launch(), k_eccm_detect_mixed<<<(unsigned)rows, 256, 0, st>>>(X32, xp, n, det, x64, p64, roots, flags);
}

void eccm_notch_cc(const cf64* in, long long ip, cf32* out, long long op, int n_r, long long rows, const int* flags,
                   double mit, const CfftDesc& d128, cudaStream_t st) {
    if (d128.n != kEccmFft) throw std::runtime_error("eccm: the compensated transform must have 128 points");
    const int num_ffts = eccm_num_windows(n_r);
    if (rows > 0 && num_ffts > 0)
        note_launch(), k_eccm_notch_cc<<<(unsigned)rows, 256, 0, st>>>(in, ip, out, op, n_r, flags, mit, d128,
                                                                        num_ffts);
}

}  // namespace s1g
