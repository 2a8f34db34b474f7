// Fused FP32 kernels of the fast path.  Each stage of the reference's
// _range_compress / _azimuth_compress runs as one kernel that keeps its
// working line in shared memory:
//   k_rc_fused      range compression (pad, FFT, matched filter, IFFT, shift/crop)
//   k_fufr_fused    azimuth FFT + frequency unfolding,
//                   the two length-S DFTs done as band-limited chirp-z transforms
//   k_rowpass_fused range FFT, SRC, range IFFT, scaling, RCMC, azimuth filter
//   k_czt_rows      azimuth IFFT (length S, chirp-z) per range bin
//   k_tufr_fused    time unfolding + quadratic resampling + re-ramp: the band
//                   of the length-(T*S) DFT and its evaluation at the
//                   resampling stencils as two non-uniform FFTs on one grid
// The Doppler lag-1 sums come from s1g_dcest.cu.
// Phase arguments are formed in double-float (s1g_df.cuh); no FP64
// arithmetic runs per sample.
#include <cmath>
#include <map>
#include <mutex>
#include <stdexcept>

#include "s1g_fast.cuh"
#include "s1g_sinc.cuh"

namespace s1g {

__device__ __forceinline__ cf32 cexpf_fast(float th) {
    float s, c;
    __sincosf(th, &s, &c);
    return mk(c, s);
}

// exp(2 pi i num / den) for 0 <= num < den < 2^24: the fraction is reduced to
// (-1/2, 1/2] before the hardware sine/cosine (absolute error ~4e-7).
__device__ __forceinline__ cf32 cis_frac(long long num, long long den) {
    float f = (float)num / (float)den;
    if (f > 0.5f) f -= 1.0f;
    return cexpf_fast(6.28318530717958648f * f);
}

// Block size of the fused kernels: two 512-thread CTAs per SM when their
// shared memory fits (each SM holds 228 KB, 1 KB reserved per CTA), else one
// 1024-thread CTA.  Both variants are capped at 64 registers per thread (the
// time unfolding runs two 384-thread CTAs instead: kTufrThreads).
static inline bool two_per_sm(size_t smem) { return smem + 1024 <= 114 * 1024; }

template <class K>
static void allow_smem(K kernel, bool& done) {
    if (!done) {
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        done = true;
    }
}

// Stage the twiddle tables of d at smtw (all threads; caller syncs).
__device__ __forceinline__ void stage_tw(cf32* smtw, const Fft3Desc& d) { fft3_stage_tw(smtw, d); }

// CZT: X[k] = sum_{s<nin} x[s] exp(dir 2 pi i s k / P) (k < nout).
// czt_core leaves the convolution in buf (padded layout); czt_out(k) then
// reads X[k].  czt_run adds a store loop and a trailing barrier.  smtw holds
// the staged twiddle tables of c.dm.
template <class LoadF>
__device__ __forceinline__ void czt_core(cf32* buf, const CztDev& c, int dir, LoadF load, const cf32* smtw) {
    const int m = c.dm.n;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
        cf32 v = mk(0.f, 0.f);
        if (q < c.nin) {
            cf32 x = load(q);
            if (dir > 0) x = conj(x);
            v = x * ldg(c.chirp + q);
        }
        buf[pad(__ldg(c.dm.perm + q))] = v;
    }
    __syncthreads();
    fft3_dit(buf, c.dm, -1, smtw);
    for (int q = threadIdx.x; q < m; q += blockDim.x) buf[pad(q)] = buf[pad(q)] * ldg(c.kern + q);
    __syncthreads();
    fft3_dif(buf, c.dm, +1, smtw);
}

__device__ __forceinline__ cf32 czt_out(const cf32* buf, const CztDev& c, int dir, int k) {
    cf32 v = ldg(c.chirp + k) * buf[pad(__ldg(c.dm.perm + k))];
    return dir > 0 ? conj(v) : v;
}

template <class LoadF, class StoreF>
__device__ __forceinline__ void czt_run(cf32* buf, const CztDev& c, int dir, LoadF load, StoreF store,
                                        const cf32* smtw) {
    czt_core(buf, c, dir, load, smtw);
    for (int k = threadIdx.x; k < c.nout; k += blockDim.x) store(k, czt_out(buf, c, dir, k));
    __syncthreads();
}

// Row-wise CZT: out[row][k] = scale * X_row[k] (used for the azimuth IFFT of
// the time unfolding, length S, dir +1).
template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1)
    k_czt_rows(const cf32* __restrict__ in, long long ip, cf32* __restrict__ out, long long op, CztDev c, int dir,
               float scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cf32* smtw = reinterpret_cast<cf32*>(smem_raw);
    cf32* buf = smtw + fft3_tw_len(c.dm.n);
    stage_tw(smtw, c.dm);
    const cf32* x = in + (long long)blockIdx.x * ip;
    cf32* y = out + (long long)blockIdx.x * op;
    czt_core(buf, c, dir, [&](int q) { return x[q]; }, smtw);
    for (int k = threadIdx.x; k < c.nout; k += blockDim.x) y[k] = czt_out(buf, c, dir, k) * scale;
}

void czt_rows(const cf32* in, long long ip, cf32* out, long long op, long long rows, const CztDev& c, int dir,
              float scale, cudaStream_t st) {
    const size_t smem = sizeof(cf32) * ((size_t)fft3_tw_len(c.dm.n) + padded_len(c.dm.n));
    if (two_per_sm(smem)) {
        static bool a = false;
        allow_smem(k_czt_rows<512>, a);
        note_launch(), k_czt_rows<512><<<(unsigned)rows, 512, smem, st>>>(in, ip, out, op, c, dir, scale);
    } else {
        static bool a = false;
        allow_smem(k_czt_rows<1024>, a);
        note_launch(), k_czt_rows<1024><<<(unsigned)rows, 1024, smem, st>>>(in, ip, out, op, c, dir, scale);
    }
}

// ------------------------------------------------------------------ range compression
template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1)
    k_rc_fused(const cf32* __restrict__ raw, cf32* __restrict__ rc, int n_r, int h, Fft3Desc d,
               const cf32* __restrict__ ref) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = d.n;
    cf32* smtw = reinterpret_cast<cf32*>(smem_raw);
    cf32* buf = smtw + fft3_tw_len(M);
    stage_tw(smtw, d);
    const long long row = blockIdx.x;
    const cf32* x = raw + row * n_r;
    for (int q = threadIdx.x; q < M; q += blockDim.x) buf[pad(__ldg(d.perm + q))] = q < n_r ? x[q] : mk(0.f, 0.f);
    __syncthreads();
    fft3_dit(buf, d, -1, smtw);
    for (int k = threadIdx.x; k < M; k += blockDim.x) buf[pad(k)] = buf[pad(k)] * ldg(ref + k);
    __syncthreads();
    fft3_dif(buf, d, +1, smtw);
    cf32* y = rc + row * n_r;
    for (int k = threadIdx.x; k < n_r; k += blockDim.x) {
        int src = k - h;
        if (src < 0) src += M;
        y[k] = buf[pad(__ldg(d.perm + src))];
    }
}

void rc_fused(const cf32* raw, cf32* rc, int n_a, int n_r, int h, const Fft3Desc& d, const cf32* ref,
              cudaStream_t st) {
    const size_t smem = sizeof(cf32) * ((size_t)fft3_tw_len(d.n) + padded_len(d.n));
    if (two_per_sm(smem)) {
        static bool a = false;
        allow_smem(k_rc_fused<512>, a);
        note_launch(), k_rc_fused<512><<<n_a, 512, smem, st>>>(raw, rc, n_r, h, d, ref);
    } else {
        static bool a = false;
        allow_smem(k_rc_fused<1024>, a);
        note_launch(), k_rc_fused<1024><<<n_a, 1024, smem, st>>>(raw, rc, n_r, h, d, ref);
    }
}

// ------------------------------------------------------------------ frequency unfolding
// Shared memory: twiddles of the n_a transform, of cf.dm and of ci.dm, then
// the chirp-z buffer (padded mbig), X (padded n_a) and the band (bw).
struct FufrLayout {
    int tw_na, tw_f, tw_i, mbig;
    __host__ __device__ explicit FufrLayout(const FufrArgs& a) {
        const Fft3Desc& dn = a.na_smooth ? a.dna : a.cna.dm;
        tw_na = fft3_tw_len(dn.n);
        tw_f = fft3_tw_len(a.cf.dm.n);
        tw_i = fft3_tw_len(a.ci.dm.n);
        mbig = a.cf.dm.n > a.ci.dm.n ? a.cf.dm.n : a.ci.dm.n;
        if (!a.na_smooth && a.cna.dm.n > mbig) mbig = a.cna.dm.n;
    }
    __host__ __device__ size_t floats(const FufrArgs& a) const {
        return (size_t)tw_na + tw_f + tw_i + padded_len(mbig) + padded_len(a.n_a) + a.bw;
    }
};

template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1) k_fufr_fused(FufrArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const FufrLayout L(a);
    cf32* tw_na = reinterpret_cast<cf32*>(smem_raw);
    cf32* tw_f = tw_na + L.tw_na;
    cf32* tw_i = tw_f + L.tw_f;
    cf32* big = tw_i + L.tw_i;
    cf32* X = big + padded_len(L.mbig);   // n_a, natural order, padded layout
    cf32* band = X + padded_len(a.n_a);   // bw
    stage_tw(tw_na, a.na_smooth ? a.dna : a.cna.dm);
    stage_tw(tw_f, a.cf.dm);
    stage_tw(tw_i, a.ci.dm);
    const int j = blockIdx.x;
    const cf32* row = a.rcT + (long long)j * a.n_a;
    // azimuth FFT (length n_a) into X
    if (a.na_smooth) {
        for (int t = threadIdx.x; t < a.n_a; t += blockDim.x) X[pad(__ldg(a.dna.perm + t))] = row[t];
        __syncthreads();
        fft3_dit(X, a.dna, -1, tw_na);
    } else {
        __syncthreads();
        czt_run(big, a.cna, -1, [&](int q) { return row[q]; }, [&](int k, cf32 v) { X[pad(k)] = v; }, tw_na);
    }
    // tile (after the azimuth fftshift), deramp, band-limited forward DFT_S
    const int n_a = a.n_a;
    czt_run(
        big, a.cf, -1,
        [&](int s) {
            if (s >= a.tile_len) return mk(0.f, 0.f);
            int q = (s % n_a) - n_a / 2;
            if (q < 0) q += n_a;
            return X[pad(q)] * ldg(a.dfwd + s);
        },
        [&](int k, cf32 v) { band[k] = v; }, tw_f);
    // inverse DFT_S of the band moved to the front, re-ramp, 1/S
    cf32* out = a.out + (long long)j * a.S;
    czt_run(big, a.ci, +1, [&](int q) { return band[q]; },
            [&](int k, cf32 v) { out[k] = v * ldg(a.reramp + k); }, tw_i);
}

void fufr_fused(const FufrArgs& a, cudaStream_t st) {
    const size_t smem = sizeof(cf32) * FufrLayout(a).floats(a);
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("frequency unfolding: shared memory");
    if (two_per_sm(smem)) {
        static bool b = false;
        allow_smem(k_fufr_fused<512>, b);
        note_launch(), k_fufr_fused<512><<<a.n_r, 512, smem, st>>>(a);
    } else {
        static bool b = false;
        allow_smem(k_fufr_fused<1024>, b);
        note_launch(), k_fufr_fused<1024><<<a.n_r, 1024, smem, st>>>(a);
    }
}

// ------------------------------------------------------------------ Doppler fit (parallel DFT)
constexpr double kPIref = 3.14159265358979;

__global__ void k_dc_fit_fast(const cf64* part, int nchunk, DcFitArgs a, double* f_dc, df* f_dc_df) {
    __shared__ double fine[64];
    __shared__ double fval[64];
    __shared__ double mag2[512];
    __shared__ double fre[512], fim[512];
    __shared__ double poly[3];
    const int n = a.n_rng, nb = a.num_blocks;
    (void)part;
    (void)nchunk;
    // f_dc holds the wrapped per-bin estimates (k_dc_wrapped)
    const int bs = n / nb;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const int s = b * bs;
        const int e = (s + bs < n) ? s + bs : n - 1;
        double acc = 0.0;
        for (int j = s; j < e; ++j) acc += f_dc[j];
        fine[b] = acc / ((double)e - (double)s);
        double sn, cs;
        sincos((2.0 * kPIref) * fine[b] / a.prf, &sn, &cs);
        fval[b] = floor(hypot(cs, sn));
    }
    __syncthreads();
    const int m = nb * 8;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int j = 0; j < nb; ++j) {
            if (fval[j] == 0.0) continue;
            double ws, wc;
            sincospi(-2.0 * (double)((long long)j * k % m) / (double)m, &ws, &wc);
            re += fval[j] * wc;
            im += fval[j] * ws;
        }
        const double mg = hypot(re, im);
        mag2[k] = mg * mg;
        fre[k] = re;
        fim[k] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int bi = 0;
        for (int k = 1; k < m; ++k)
            if (mag2[k] > mag2[bi]) bi = k;
        const float dt = (float)(a.rt[1] - a.rt[0]);
        const double val = 1.0 / (m * (double)dt);
        const int N = (m - 1) / 2 + 1;
        const double v = bi < N ? bi * val : (bi - m) * val;
        const double aa = v / (double)dt;
        const double bb = atan2(fim[bi], fre[bi]) / (2.0 * kPIref);
        double un[64];
        for (int j = 0; j < nb; ++j) {
            double s1, c1, s2, c2;
            sincos((2.0 * kPIref) * fine[j] / a.prf, &s1, &c1);
            sincos(-1.0 * (aa * a.rt[j] + bb), &s2, &c2);
            const double pr = c1 * c2 - s1 * s2, pi_ = c1 * s2 + s1 * c2;
            un[j] = (aa * a.rt[j] + bb + atan2(pi_, pr) / (2.0 * kPIref)) * a.prf;
        }
        double Sx[5] = {0, 0, 0, 0, 0}, Sy[3] = {0, 0, 0};
        for (int i = 0; i < nb; ++i) {
            double xi = 1.0;
            for (int jj = 0; jj <= 4; ++jj) {
                if (jj <= 2) Sy[jj] += xi * un[i];
                Sx[jj] += xi;
                xi *= a.rt[i];
            }
        }
        double A[3][3] = {{Sx[0], Sx[1], Sx[2]}, {Sx[1], Sx[2], Sx[3]}, {Sx[2], Sx[3], Sx[4]}};
        double B[3] = {Sy[0], Sy[1], Sy[2]};
        for (int i = 0; i < 3; ++i) {
            for (int k = i + 1; k < 3; ++k)
                if (fabs(A[k][i]) > fabs(A[i][i])) {
                    for (int jj = 0; jj < 3; ++jj) {
                        const double t = A[i][jj];
                        A[i][jj] = A[k][jj];
                        A[k][jj] = t;
                    }
                    const double t = B[i];
                    B[i] = B[k];
                    B[k] = t;
                }
            for (int k = i + 1; k < 3; ++k) {
                const double f = A[k][i] / A[i][i];
                for (int jj = i; jj < 3; ++jj) A[k][jj] -= f * A[i][jj];
                B[k] -= f * B[i];
            }
        }
        double c[3];
        for (int i = 2; i >= 0; --i) {
            c[i] = B[i];
            for (int jj = i + 1; jj < 3; ++jj) c[i] -= A[i][jj] * c[jj];
            c[i] /= A[i][i];
        }
        poly[0] = c[0];
        poly[1] = c[1];
        poly[2] = c[2];
    }
    __syncthreads();
    const double step = (a.far - a.near) / (n - 1);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double t = (a.near + j * step) - a.near;
        const double v = (poly[0] + poly[1] * t + poly[2] * t * t);
        f_dc[j] = v;
        f_dc_df[j] = df_from(v);
    }
}

// Wrapped per-bin centroid -prf arg(sum) / (2 pi) (doppler.cpp:4-39), all bins in parallel.
__global__ void k_dc_wrapped(const cf64* __restrict__ part, int nchunk, int n, double prf, double* __restrict__ f_dc) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double sr = 0.0, si = 0.0;
    for (int c = 0; c < nchunk; ++c) {
        sr += part[(long long)c * n + j].x;
        si += part[(long long)c * n + j].y;
    }
    f_dc[j] = -prf * atan2(si, sr) / (2 * kPIref);
}

void dc_fit_fast(const cf64* part, int nchunk, const DcFitArgs& a, double* f_dc, df* f_dc_df, cudaStream_t st) {
    note_launch(), k_dc_wrapped<<<(a.n_rng + 127) / 128, 128, 0, st>>>(part, nchunk, a.n_rng, a.prf, f_dc);
    note_launch(), k_dc_fit_fast<<<1, 256, 0, st>>>(part, nchunk, a, f_dc, f_dc_df);
}

// ------------------------------------------------------------------ row pass


// SRC phase, image_formation.cpp:422-455: -pi f_r^2 / K_src with
// K_src = 2 v^2 f_c^3 D^2 / (c R F^2).
__device__ __forceinline__ float src_phase(const RowDf& r, const ColDf& c, df fdc, float lam2_4) {
    const float F = r.fa.hi + fdc.hi + (r.fa.lo + fdc.lo);
    const float vq = r.P.hi * ((r.A.hi - c.Q.hi) + (r.A.lo - c.Q.lo));
    const float F2 = F * F;
    const float D2 = 1.0f - lam2_4 * F2 / vq;
    return -c.csrc * F2 / (vq * D2);
}

// Scale, RCMC and azimuth filter factor (s1_decoder.cpp:643-676).
__device__ __forceinline__ cf32 post_factor(const RowDf& r, const ColDf& c, df fdc, df lam2_4, int tops) {
    const df F = df_add(r.fa, fdc);
    const df vq = df_mul(r.P, df_sub(r.A, c.Q));
    const df x = df_div(df_mul(lam2_4, df_mul(F, F)), vq);
    const df D = df_sqrt(df_sub(df_make(1.f, 0.f), x));
    const df omd = df_div(x, df_add_f(D, 1.0f));   // 1 - D
    const df th = df_add(df_neg(df_mul(c.k4r, omd)), df_mul(c.tau2pi, F));
    float theta = df_wrap(th);
    if (tops) theta -= c.crcmc * (omd.hi / D.hi);
    const cf32 f = cexpf_fast(theta) * c.az0;
    return f * (1.0f / c.rscale);
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1) k_rowpass_fused(RowArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Fft3Desc& dd = a.smooth ? a.d : a.cz.dm;
    cf32* smtw = reinterpret_cast<cf32*>(smem_raw);
    cf32* buf = smtw + fft3_tw_len(dd.n);
    stage_tw(smtw, dd);
    const int i = blockIdx.x;
    const RowDf rp = a.rows[i];
    cf32* row = a.data + (long long)i * a.n_r;
    const int n = a.n_r;
    const float l24 = a.lam2_4.hi;
    if (a.smooth) {
        if (a.tops) {
            for (int j = threadIdx.x; j < n; j += blockDim.x) buf[pad(__ldg(a.d.perm + j))] = row[j];
            __syncthreads();
            fft3_dit(buf, a.d, -1, smtw);
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                buf[pad(j)] = buf[pad(j)] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
        } else {
            // stripmap: the SRC phase is applied to the range-time samples
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                buf[pad(j)] = row[j] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
        }
        __syncthreads();
        fft3_dif(buf, a.d, +1, smtw);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const cf32 v = buf[pad(__ldg(a.d.perm + j))];
            row[j] = a.post ? v * post_factor(rp, a.cols[j], a.fdc[j], a.lam2_4, a.tops) : v;
        }
    } else {
        __syncthreads();
        if (a.tops) {
            czt_run(buf, a.cz, -1, [&](int q) { return row[q]; },
                    [&](int k, cf32 v) { row[k] = v * cexpf_fast(src_phase(rp, a.cols[k], a.fdc[k], l24)); },
                    smtw);
        } else {
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                row[j] = row[j] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
            __syncthreads();
        }
        czt_run(buf, a.cz, +1, [&](int q) { return row[q]; },
                [&](int k, cf32 v) {
                    row[k] = a.post ? v * post_factor(rp, a.cols[k], a.fdc[k], a.lam2_4, a.tops) : v;
                },
                smtw);
    }
}

void rowpass_fused(const RowArgs& a, cudaStream_t st) {
    const int m = a.smooth ? a.d.n : a.cz.dm.n;
    const size_t smem = sizeof(cf32) * ((size_t)fft3_tw_len(m) + padded_len(m));
    if (two_per_sm(smem)) {
        static bool b = false;
        allow_smem(k_rowpass_fused<512>, b);
        note_launch(), k_rowpass_fused<512><<<a.S, 512, smem, st>>>(a);
    } else {
        static bool b = false;
        allow_smem(k_rowpass_fused<1024>, b);
        note_launch(), k_rowpass_fused<1024><<<a.S, 1024, smem, st>>>(a);
    }
}

// Sinc RCMC: a warp forms 32 consecutive range bins of one azimuth row.  The
// migration of bin j is rmig_j (1 - D) / D samples (D of post_factor, a few
// samples at the band edges), so the 32 positions advance about one sample
// per lane and their taps come from two samples per lane by warp shuffles.
__global__ void __launch_bounds__(256) k_rcmc_sinc(RcmcArgs a) {
    const int lane = threadIdx.x & 31;
    const int wpr = (a.n_r + 31) / 32;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (long long)a.S * wpr) return;   // whole warps leave together
    const int i = (int)(gw / wpr);
    const int j = (int)(gw % wpr) * 32 + lane;
    const bool act = j < a.n_r;
    const RowDf rp = a.rows[i];
    const int jj = act ? j : a.n_r - 1;
    const ColDf c = a.cols[jj];
    const df fdc = a.fdc[jj];
    const df F = df_add(rp.fa, fdc);
    const df vq = df_mul(rp.P, df_sub(rp.A, c.Q));
    const df x = df_div(df_mul(a.lam2_4, df_mul(F, F)), vq);
    const df D = df_sqrt(df_sub(df_make(1.f, 0.f), x));
    const df omd = df_div(x, df_add_f(D, 1.0f));   // 1 - D
    const double t = (double)j + (double)(c.rmig * (omd.hi / D.hi));
    const cf32 v = sinc_warp<float>(a.in + (long long)i * a.n_r, a.n_r, t, a.L, act);
    if (act) a.out[(long long)i * a.n_r + j] = v * post_factor(rp, c, fdc, a.lam2_4, 0);
}

void rcmc_sinc(const RcmcArgs& a, cudaStream_t st) {
    const long long warps = (long long)a.S * ((a.n_r + 31) / 32);
    note_launch(), k_rcmc_sinc<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(a);
}

// ------------------------------------------------------------------ time unfolding

// Knot of the deramp / re-ramp phase: pi K_t and the deramp time -f_dc/K_a,
// as float pairs (one float4 per knot).
__device__ __forceinline__ void load_knot(const float4* KN, int i, df& pkt, df& dct) {
    const float4 v = KN[i];
    pkt = df_make(v.x, v.y);
    dct = df_make(v.z, v.w);
}

// Deramp (sgn -1) / re-ramp (sgn +1) phase of azimuth_time_ufr
// (image_formation.cpp:305-313, 365-373) at time tau between knots i and i+1
// (fraction al).  With t = dct + tau and K_a dct = -f_dc the reference's
//   -pi kt t^2 + 2 pi (kt + K_a) dct t
// equals -[pi kt (tau^2 - dct^2) + 2 pi f_dc (tau + dct)], evaluated here as
// -(tau + dct) [pi kt (tau - dct) + 2 pi f_dc].
__device__ __forceinline__ float tufr_phase(const float4* KN, int i, float al, df tau, int sgn, df tpf) {
    df p0, d0, p1, d1;
    load_knot(KN, i, p0, d0);
    load_knot(KN, i + 1, p1, d1);
    const df pkt = df_add_f(p0, ((p1.hi - p0.hi) + (p1.lo - p0.lo)) * al);
    const df dct = df_add_f(d0, ((d1.hi - d0.hi) + (d1.lo - d0.lo)) * al);
    const df a = df_add(tau, dct);
    const df b = df_sub(tau, dct);
    const df th = df_mul(a, df_add(df_mul(pkt, b), tpf));
    return sgn < 0 ? -df_wrap(th) : df_wrap(th);
}

// ---- deramp phase of a knot interval as a polynomial in the sample step
// Over the samples n = n_a + d of one knot interval iv (K_a resampled from
// knots iv, iv + 1, fraction al = al_a + d (S - 1) / (TS - 1)), pi K_t and
// -f_dc/K_a are linear in d and so is az_time, and the deramp argument
// th = (tau + dct) [pi kt (tau - dct) + 2 pi f_dc] (tufr_phase) is the cubic
//   th(d) = H0 + G1 d + G2 d^2 + (A1 C2 d^3, below 1e-8 rad over an interval)
// H0 and G1 in double-float, reduced to fractions of a turn in 32-bit fixed
// point; the phase -th / (2 pi) - n k_s / TS then wraps by integer overflow.
struct DerampPoly {
    unsigned int base, slope;   // -H0, -G1 in turns x 2^32 (mod 2^32)
    float curv;                 // -G2 in turns x 2^32
};

// frac(x / (2 pi)) x 2^32 (mod 2^32) of a double-float x (|x| < ~1e6)
__device__ __forceinline__ unsigned int turns_fx(df x, df i2p) {
    const df t = df_mul(x, i2p);
    const float k = rintf(t.hi);
    // |t.hi - k| <= 1/2: x 2^32 saturates only at exactly +2^31 (one unit off)
    return (unsigned int)__float2int_rn((t.hi - k) * 4294967296.0f) + (unsigned int)__float2int_rn(t.lo * 4294967296.0f);
}

// Double-float sum without the second error term (Hida-Li-Bailey's "sloppy"
// add): its error is below 2^-46 of the larger operand, the absolute
// accuracy the phases need, at half the operations of df_add.
__device__ __forceinline__ df df_add_abs(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ DerampPoly deramp_poly(const float4* KN, int iv, float al, df tau, df tpf, df dt, float gk,
                                                  df i2p) {
    df p0, d0, p1, d1;
    load_knot(KN, iv, p0, d0);
    load_knot(KN, iv + 1, p1, d1);
    const float dpk = (p1.hi - p0.hi) + (p1.lo - p0.lo);
    const float ddc = (d1.hi - d0.hi) + (d1.lo - d0.lo);
    const df P = df_add_f(p0, dpk * al);
    const df D = df_add_f(d0, ddc * al);
    const float Pd = dpk * gk, Dd = ddc * gk;   // per-sample steps of P and D
    const df A0 = df_add_abs(tau, D), B0 = df_add_abs(tau, df_neg(D));
    const df C0 = df_add_abs(df_mul(P, B0), tpf);
    const df H0 = df_mul(A0, C0);
    // th'(0) = A1 C0 + A0 C1 with A1 = dt + Dd, B1 = dt - Dd, C1 = P B1 + Pd B0:
    //   dt (C0 + A0 P) + Dd (C0 - A0 P) + A0 Pd B0
    // the first term (~1 rad per sample) in double-float, the others (~1e-3)
    // in float
    const df Q = df_mul(A0, P);
    const float small = fmaf(Dd, C0.hi - Q.hi, A0.hi * Pd * B0.hi);
    const df G1 = df_add_f(df_mul(dt, df_add_abs(C0, Q)), small);
    // th''(0) / 2 = A0 C2 + A1 C1 with C2 = Pd B1 (~1e-5 rad): float
    const float B1 = dt.hi - Dd, A1 = dt.hi + Dd;
    const float C1 = fmaf(P.hi, B1, Pd * B0.hi);
    const float G2 = fmaf(A0.hi, Pd * B1, A1 * C1);
    DerampPoly r;
    r.base = 0u - turns_fx(H0, i2p);
    r.slope = 0u - turns_fx(G1, i2p);
    r.curv = -G2 * 683565275.57643158f;   // 2^32 / (2 pi)
    return r;
}

// exp(i 2 pi (phase in turns)) at step d of the interval, band shift pm
__device__ __forceinline__ cf32 deramp_rot(const DerampPoly& p, int d, float d2, unsigned int pm) {
    const unsigned int ph = p.base + p.slope * (unsigned int)d + (unsigned int)__float2int_rn(p.curv * d2) - pm;
    float sn, cs;
    __sincosf((float)(int)ph * 1.46291807926715968e-9f, &sn, &cs);   // 2 pi / 2^32
    return mk(cs, sn);
}

__host__ __device__ __forceinline__ long long floor_div_ll(long long a, long long b) {
    return a >= 0 ? a / b : -((-a + b - 1) / b);
}
// Knot intervals of the TS-point deramp axis (K_a resampled S -> TS,
// linear_resample): sample u lies in interval floor(u (S - 1) / (TS - 1))
// (the last sample in interval S - 2), and interval iv starts at
// ceil(iv (TS - 1) / (S - 1)).  Both from float estimates (within one of the
// answer for TS < 2^24) corrected with exact integer products, which keeps
// 64-bit divisions off the sample path.
__device__ __forceinline__ int knot_of_near(int u, int S, long long TS, float gk) {
    int q = __float2int_rz((float)u * gk);
    const long long num = (long long)u * (S - 1);
    if ((long long)q * (TS - 1) > num) --q;
    else if ((long long)(q + 1) * (TS - 1) <= num) ++q;
    return min(q, S - 2);
}
__device__ __forceinline__ int knot_first_near(int iv, int S, long long TS, float rt) {
    const long long num = (long long)iv * (TS - 1);
    int n = __float2int_ru((float)iv * rt);
    if ((long long)n * (S - 1) < num) ++n;
    else if ((long long)(n - 1) * (S - 1) >= num) --n;
    return n;
}

// Shared memory: twiddles of the grid FFT, then one region that holds either
// the deramped samples of a spreading pass (ychunk, kTufrGroup range bins
// interleaved) or the grid (padded M) of one range bin's transforms.
struct TufrLayout {
    static constexpr int head = 8;   // the group's 2 pi f_dc (kTufrGroup double-floats)
    int tw, grid;
    // the region starts 16-byte aligned (it is read as float4)
    __host__ __device__ explicit TufrLayout(const TufrArgs& a)
        : tw((fft3_tw_len(a.dnu.n) + 1) & ~1), grid(padded_len(a.dnu.n)) {}
    __host__ __device__ size_t floats(const TufrArgs& a) const {
        return (size_t)head + tw + (size_t)(grid > a.ychunk ? grid : a.ychunk);
    }
};

// ex2.approx / sqrt.approx (relative error ~2^-22): the spreading weights
// need ~1e-6, far looser than the special-function paths would give.
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Smallest n with m2 n >= A, and largest n with m2 n <= B (m2 > 0), for
// A = a TS, B = b TS: the float estimate a TS / m2 (two exact float factors,
// |a|, TS < 2^24) is within one of the answer, the loops correct it with
// exact integer products.  No 64-bit conversions (FP64 pipe on this part).
__device__ __forceinline__ int first_at_or_above(int a, int TS, int m2, float inv_m2) {
    const long long A = (long long)a * TS;
    int n = (int)ceilf((float)a * (float)TS * inv_m2);
    while ((long long)m2 * n < A) ++n;
    while ((long long)m2 * (n - 1) >= A) --n;
    return n;
}
__device__ __forceinline__ int last_at_or_below(int b, int TS, int m2, float inv_m2) {
    const long long B = (long long)b * TS;
    int n = (int)floorf((float)b * (float)TS * inv_m2);
    while ((long long)m2 * n > B) --n;
    while ((long long)m2 * (n + 1) <= B) ++n;
    return n;
}

// Out-of-line grid transforms of k_tufr_fused: behind the call boundary the
// radix-16 stages get the 64 registers to themselves instead of sharing them
// with the kernel's loop state (which then spilled inside the stages).
__device__ __noinline__ void tufr_grid_fwd(cf32* buf, Fft3Desc d, const cf32* tw) { fft3_dif(buf, d, -1, tw); }
__device__ __noinline__ void tufr_grid_inv(cf32* buf, Fft3Desc d, const cf32* tw) { fft3_dit(buf, d, +1, tw); }

template <int NT>
__global__ void __launch_bounds__(NT, NT <= 512 ? 2 : 1) k_tufr_fused(TufrArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int R = kTufrGroup;
    static_assert(R == 2, "the staged samples are range-bin pairs (16 bytes per sample)");
    const TufrParams q = a.P->q;
    const int S = a.S;
    const int T = q.num_tiles;
    const int M = a.dnu.n;
    const int bw = q.end - q.start;
    const long long TS = (long long)T * S;
    // grid points per spreading pass: their samples (at most (L - 1 + W) TS / M + 1
    // per range bin) fit the staged chunk; two per thread of the block when possible
    const int cap = a.ychunk / R;
    const long long lmax = (T >= 1 ? ((long long)(cap - 2) * M) / TS : 0) - kNuW + 1;
    const int Lc = (int)(lmax >= 2 * NT ? (lmax / (2 * NT)) * (2 * NT) : lmax);   // two grid points per thread
    // outside the launch plan (tile count, band, chunk): flag, do nothing
    if (!q.ok || T < 1 || T > a.tmax || S < 8 || bw > a.bwmax || 4 * bw > 5 * M || lmax < 1 || TS >= (1LL << 24)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.status = 1;
        return;
    }
    const TufrLayout L(a);
    df* s_tpf = reinterpret_cast<df*>(smem_raw);
    cf32* tw = reinterpret_cast<cf32*>(smem_raw) + L.head;
    cf32* big = tw + L.tw;                 // grid of one range bin (padded M) ...
    cf32* ych = big;                       // ... or the staged samples of a pass, range-bin
                                           // pairs (16 bytes per sample)
    stage_tw(tw, a.dnu);
    const int K0 = bw / 2;
    const long long ks = q.start + K0;     // band centre bin
    // spreading kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)), z = 2 (x_n - l) / W
    const double sigma = (double)M / (double)bw;
    const float bl2 = (float)(0.97 * 3.141592653589793 * kNuW * (1.0 - 1.0 / (2.0 * sigma)) * 1.4426950408889634);
    const float zs = (float)(2.0 / ((double)kNuW * (double)TS));
    const int m2 = 2 * M;
    const float inv_m2 = 1.0f / (float)m2;
    // deramp: sample spacing of az_times (linspace over TS), knot-position
    // step per sample, 1 / (2 pi), and the band shift k_s / TS as a 64-bit
    // fraction of a turn (floor(2^64 (k_s mod TS) / TS))
    const df dt = df_from(q.focused_time / (double)(TS - 1));
    const float gk = (float)((double)(S - 1) / (double)(TS - 1));
    const df i2p = df_from(0.15915494309189533577);
    const float inv_s = 1.0f / (float)S;
    const float rt = (float)((double)(TS - 1) / (double)(S - 1));
    const double ft = q.focused_time;
    const double dtau = (ft / 2 - (-ft / 2)) / (double)(TS - 1);   // az_times = linspace(-ft/2, ft/2, TS)
    const df tau0 = df_from(-ft / 2), dtau_df = df_from(dtau);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long KS64;
    {
        const unsigned long long kk = (unsigned long long)(((ks % TS) + TS) % TS);
        const unsigned long long hi = (kk << 32) / (unsigned long long)TS;
        const unsigned long long rem = (kk << 32) - hi * (unsigned long long)TS;
        KS64 = (hi << 32) | ((rem << 32) / (unsigned long long)TS);
    }
    float4* KNg = reinterpret_cast<float4*>(a.KN) + (long long)blockIdx.x * R * S;
    cf32* Gg = a.G + (long long)blockIdx.x * R * M;
    for (int j0 = blockIdx.x * R; j0 < a.n_r; j0 += gridDim.x * R) {
        const int rc = min(R, a.n_r - j0);
        // 1. the azimuth IFFT (length S, 1/S, s1_decoder.cpp:682) ran in k_czt_rows
        // 2. knots: pi K_t and -f_dc/K_a at the S azimuth rows of each range bin
        for (int r = 0; r < rc; ++r) {
            const int j = j0 + r;
            const ColDf cj = a.cols[j];
            const df fdc = a.fdc[j];
            const df ilr = a.inv_lamR[j];
            float4* KN = KNg + (long long)r * S;
            for (int s = threadIdx.x; s < S; s += blockDim.x) {
                const RowDf rw = a.rows[s];
                const df F = df_add(rw.fa, fdc);
                const df vq = df_mul(rw.P, df_sub(rw.A, cj.Q));
                const df x = df_div(df_mul(a.lam2_4, df_mul(F, F)), vq);
                const df D = df_sqrt(df_sub(df_make(1.f, 0.f), x));
                const df D3 = df_mul(D, df_mul(D, D));
                const df u = df_neg(df_mul(df_mul(df_mul(df_make(2.f, 0.f), vq), D3), ilr));   // K_a = -2 v^2 D^3/(lambda R)
                const df kt = df_neg(df_div(df_mul(u, a.rate), df_sub(a.rate, u)));              // -K_a r / (r - K_a)
                const df dct = df_neg(df_div(fdc, u));                                          // -f_dc / K_a
                const df pkt = df_mul(a.pi_, kt);
                KN[s] = make_float4(pkt.hi, pkt.lo, dct.hi, dct.lo);
            }
            if (threadIdx.x == 0) s_tpf[r] = df_mul(a.two_pi_, fdc);
        }
        __syncthreads();
        // 3. band of the length-TS DFT (image_formation.cpp:315-333), type-1
        //    non-uniform FFT: spread y[n] exp(-2 pi i n k_s / TS), the deramped
        //    tiled line y[s + S t] = A[s] exp(-i deramp(s + S t)), onto the grid
        //    (grid point l gathers the samples within W/2 of x_n = n M / TS;
        //    n is taken modulo TS), in passes of Lc grid points, R range bins
        //    per pass sharing each kernel weight
        for (int l0 = 0; l0 < M; l0 += Lc) {
            const int l1 = min(M, l0 + Lc);
            const int nA = first_at_or_above(2 * l0 - kNuW, (int)TS, m2, inv_m2);
            const int nB = last_at_or_below(2 * (l1 - 1) + kNuW, (int)TS, m2, inv_m2);
            // Deramped samples of the pass.  The deramp phase is a cubic in
            // the sample step over each knot interval (the ~T consecutive
            // samples whose K_a comes from knots iv, iv + 1): a warp takes a
            // share of the samples, each lane anchors one interval in
            // double-float (deramp_poly), and the lanes then take the samples
            // in runs of 32 (coalesced loads and stores), fetching their
            // interval's anchor by shuffle and evaluating the phase in 32-bit
            // fixed-point turns; the band shift n k_s / TS in 64-bit fixed point.
            for (long long k = floor_div_ll(nA, TS); k <= floor_div_ll(nB, TS); ++k) {
                const int u0 = (int)max((long long)nA - k * TS, 0LL);
                const int u1 = (int)min((long long)nB - k * TS, TS - 1);
                const int posoff = (int)(k * TS - nA);   // staged position of sample u: u + posoff
                const int len = u1 - u0 + 1;
                const int wlo = u0 + (int)((long long)len * warp / (NT / 32));
                const int whi = u0 + (int)((long long)len * (warp + 1) / (NT / 32)) - 1;
                int nstart = wlo;
                int ivw = knot_of_near(wlo, S, TS, gk);
                const int ivlast = knot_of_near(whi, S, TS, gk);
                const cf32* in0 = a.in + (long long)j0 * S;
                const cf32* in1 = in0 + (rc > 1 ? S : 0);
                while (nstart <= whi) {   // warp-uniform: up to 32 intervals per round
                    const int ive = min(ivw + 31, ivlast);
                    const int nend = min(whi, ive == S - 2 ? (int)TS - 1 : knot_first_near(ive + 1, S, TS, rt) - 1);
                    // the first run's samples are loaded before the anchors
                    int n = min(nstart + lane, nend);
                    int si = n - S * __float2int_rz((float)n * inv_s);
                    if (si < 0) si += S;
                    else if (si >= S) si -= S;
                    cf32 v0 = in0[si], v1 = in1[si];
                    const int iv = ivw + lane;
                    int na = nstart;
                    DerampPoly p0 = {0u, 0u, 0.f}, p1 = {0u, 0u, 0.f};
                    if (iv <= ive) {
                        na = max(nstart, knot_first_near(iv, S, TS, rt));
                        // knot fraction and az_time of the anchor, as the
                        // reference's linear_resample and linspace give them
                        const float al = (float)(int)((long long)na * (S - 1) - (long long)iv * (TS - 1)) / (float)(TS - 1);
                        const df taua = df_add(tau0, df_mul_f(dtau_df, (float)na));
                        p0 = deramp_poly(KNg, iv, al, taua, s_tpf[0], dt, gk, i2p);
                        if (rc > 1) p1 = deramp_poly(KNg + S, iv, al, taua, s_tpf[1], dt, gk, i2p);
                    }
                    for (int n0 = nstart; n0 <= nend; n0 += 32) {
                        // next run's samples in flight while this one is evaluated
                        const int nn = min(n0 + 32 + lane, nend);
                        int sn = nn - S * __float2int_rz((float)nn * inv_s);
                        if (sn < 0) sn += S;
                        else if (sn >= S) sn -= S;
                        cf32 w0 = mk(0.f, 0.f), w1 = w0;
                        if (n0 + 32 <= nend) {
                            w0 = in0[sn];
                            w1 = in1[sn];
                        }
                        const int src = knot_of_near(n, S, TS, gk) - ivw;
                        const unsigned int b0 = __shfl_sync(0xffffffffu, p0.base, src);
                        const unsigned int s0 = __shfl_sync(0xffffffffu, p0.slope, src);
                        const float c0 = __shfl_sync(0xffffffffu, p0.curv, src);
                        const unsigned int b1 = __shfl_sync(0xffffffffu, p1.base, src);
                        const unsigned int s1 = __shfl_sync(0xffffffffu, p1.slope, src);
                        const float c1 = __shfl_sync(0xffffffffu, p1.curv, src);
                        const int d = n - __shfl_sync(0xffffffffu, na, src);
                        if (n0 + lane <= nend) {
                            const unsigned int pm = (unsigned int)(((unsigned long long)n * KS64) >> 32);
                            const float d2 = (float)(d * d);
                            const cf32 e0 = deramp_rot({b0, s0, c0}, d, d2, pm);
                            float4 o;
                            o.x = v0.x * e0.x - v0.y * e0.y;
                            o.y = v0.x * e0.y + v0.y * e0.x;
                            o.z = 0.f;
                            o.w = 0.f;
                            if (rc > 1) {
                                const cf32 e1 = deramp_rot({b1, s1, c1}, d, d2, pm);
                                o.z = v1.x * e1.x - v1.y * e1.y;
                                o.w = v1.x * e1.y + v1.y * e1.x;
                            }
                            reinterpret_cast<float4*>(ych)[n + posoff] = o;
                        }
                        n = nn;
                        v0 = w0;
                        v1 = w1;
                    }
                    nstart = nend + 1;
                    ivw = ive + 1;
                }
            }
            __syncthreads();
            // a thread takes two adjacent grid points and reads each sample of
            // their joint window once (16 bytes: both range bins); lanes'
            // windows start ~2 TS / M samples apart, so a quarter-warp's loads
            // fall in distinct bank quads
            const float4* y01 = reinterpret_cast<const float4*>(ych);
            for (int pi = threadIdx.x; 2 * pi < l1 - l0; pi += NT) {
                const int l = l0 + 2 * pi;
                const bool two = l + 1 < l1;
                const int lo = first_at_or_above(2 * l - kNuW, (int)TS, m2, inv_m2);
                const int hi = last_at_or_below(2 * (two ? l + 1 : l) + kNuW, (int)TS, m2, inv_m2);
                int num = (int)((long long)lo * M - (long long)l * TS);   // (x_n - l) TS, |.| <= W TS / 2 + TS
                const float4* p01 = y01 + (lo - nA);
                float4 aa = make_float4(0.f, 0.f, 0.f, 0.f), ab = aa;
                for (int n = 0; n <= hi - lo; ++n) {
                    const float za = (float)num * zs;
                    const float zb = (float)(num - (int)TS) * zs;
                    // outside the support (|z| >= 1) the weight is exp(-beta)
                    // (~4e-11 of the peak) instead of 0: a few window-edge samples
                    const float wa = ex2_approx(fmaf(bl2, sqrt_approx(fmaxf(fmaf(-za, za, 1.0f), 0.f)), -bl2));
                    const float wb = ex2_approx(fmaf(bl2, sqrt_approx(fmaxf(fmaf(-zb, zb, 1.0f), 0.f)), -bl2));
                    const float4 v = p01[n];
                    aa.x = fmaf(wa, v.x, aa.x);
                    aa.y = fmaf(wa, v.y, aa.y);
                    aa.z = fmaf(wa, v.z, aa.z);
                    aa.w = fmaf(wa, v.w, aa.w);
                    ab.x = fmaf(wb, v.x, ab.x);
                    ab.y = fmaf(wb, v.y, ab.y);
                    ab.z = fmaf(wb, v.z, ab.z);
                    ab.w = fmaf(wb, v.w, ab.w);
                    num += M;
                }
                Gg[l] = mk(aa.x, aa.y);
                if (rc > 1) Gg[M + l] = mk(aa.z, aa.w);
                if (two) {
                    Gg[l + 1] = mk(ab.x, ab.y);
                    if (rc > 1) Gg[M + l + 1] = mk(ab.z, ab.w);
                }
            }
            __syncthreads();
        }
        for (int r = 0; r < rc; ++r) {
            const float4* KN = KNg + (long long)r * S;
            const df tpf = s_tpf[r];
            for (int l = threadIdx.x; l < M; l += blockDim.x) big[pad(l)] = Gg[(long long)r * M + l];
            __syncthreads();
            // grid FFT (natural order in, digit-reversed out); bin p holds
            // Z[K0 + p] Phi(p / M) on the band
            tufr_grid_fwd(big, a.dnu, tw);
            // 4. band mask and both deconvolutions, then the inverse grid FFT of
            //    the type-2 evaluation (digit-reversed in, natural order out)
            for (int p = threadIdx.x; p < M; p += blockDim.x) {
                const int e = pad(__ldg(a.dnu.perm + p));
                big[e] = big[e] * __ldg(a.tab.band + p);
            }
            __syncthreads();
            tufr_grid_inv(big, a.dnu, tw);
            // 5. kNuTaps-tap interpolation (weights fold the Lagrange stencil, the
            //    centring phase and 1/TS), re-ramp (image_formation.cpp:355-378),
            //    store the cropped rows
            cf32* out = a.out + (long long)(j0 + r) * a.n_out;
            for (int p = threadIdx.x; p < a.n_out; p += blockDim.x) {
                int l = __ldg(a.tab.nu_l0 + p) % M;
                if (l < 0) l += M;
                const cf32* w = a.tab.nu_w + p;   // tap t at w[t n_out]: lanes read consecutive words
                cf32 acc = mk(0.f, 0.f);
#pragma unroll
                for (int t = 0; t < kNuTaps; ++t) {
                    acc = acc + big[pad(l)] * ldg(w + (long long)t * a.n_out);
                    if (++l == M) l = 0;
                }
                const float4 rr = __ldg(a.tab.rer + p);
                out[p] = acc * cexpf_fast(tufr_phase(KN, __float_as_int(rr.x), rr.y, df_make(rr.z, rr.w), +1, tpf));
            }
            __syncthreads();
        }
    }
}

// Exponential-of-semicircle kernel of width kNuW (support |t| < kNuW / 2, t in
// grid units) and its Fourier transform by Gauss-Legendre quadrature.
__device__ __forceinline__ double nu_kernel(double t, double beta) {
    const double z = 2.0 * t / kNuW;
    return fabs(z) < 1.0 ? exp(beta * (sqrt(1.0 - z * z) - 1.0)) : 0.0;
}

__device__ double nu_kernel_ft(double xi, double beta, const double* gx, const double* gw) {
    double acc = 0.0;
    for (int q = 0; q < kNuQuad; ++q) {
        const double t = 0.5 * kNuW * gx[q];
        acc += gw[q] * nu_kernel(t, beta) * cospi(2.0 * xi * t);
    }
    return 0.5 * kNuW * acc;
}

// Per-burst tables of the time unfolding (see TufrTables), one thread per entry.
__global__ void k_tufr_tables(const TufrDev* __restrict__ P, int S, int n_out, int s0, int M, TufrTables t) {
    const TufrParams q = P->q;
    const int T = q.num_tiles;
    if (!q.ok || T < 1) return;
    const long long TS = (long long)T * S;
    const double ft = q.focused_time;
    const int bw = q.end - q.start;
    const int K0 = bw / 2;
    // oversampling M / bw >= 1.25 and the kernel's beta for it
    const double sigma = (double)M / (double)bw;
    const double beta = 0.97 * 3.141592653589793 * kNuW * (1.0 - 1.0 / (2.0 * sigma));
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    // band mask / Phi(p / M)^2 at the grid bins (FFT order), Phi by the
    // Gauss-Legendre rule of nu_kernel_ft with the kernel values at the nodes
    // (which do not depend on the bin) formed once per block
    __shared__ double kq[kNuQuad], tq[kNuQuad];
    for (int q = threadIdx.x; q < kNuQuad; q += blockDim.x) {
        tq[q] = 0.5 * kNuW * t.gl_x[q];
        kq[q] = t.gl_w[q] * nu_kernel(tq[q], beta);
    }
    __syncthreads();
    for (long long p = tid; p < M; p += stride) {
        const bool in_band = p < bw - K0 || p >= M - K0;
        if (!in_band) {
            t.band[p] = 0.0f;
            continue;
        }
        const double xi = (double)(p < bw - K0 ? p : p - M) / (double)M;
        double acc = 0.0;
        for (int q = 0; q < kNuQuad; ++q) acc += kq[q] * cospi(2.0 * xi * tq[q]);
        const double inv_phi = 1.0 / (0.5 * kNuW * acc);
        t.band[p] = (float)(inv_phi * inv_phi);
    }
    for (long long p = tid; p < n_out; p += stride) {
        const long long qo = s0 + p;
        // quadratic resampling TS -> down: stencil n = i-1, i, i+1 (signal_processing.cpp:109-155)
        const long long num = qo * (TS - 1);
        long long i = num / (q.down - 1);
        double xi = (double)(num - i * (q.down - 1)) / (double)(q.down - 1);
        if (i > TS - 2) {
            xi += (double)(i - (TS - 2));
            i = TS - 2;
        }
        const double L[3] = {0.5 * xi * (xi - 1.0), -(xi + 1.0) * (xi - 1.0), 0.5 * (xi + 1.0) * xi};
        // grid positions x = M n / TS of the three stencil points (n modulo TS)
        double xs[3], ph_c[3], ph_s[3];
        for (int k = 0; k < 3; ++k) {
            const long long n = (((i - 1 + k) % TS) + TS) % TS;
            xs[k] = (double)M * (double)n / (double)TS;
            sincospi(2.0 * (double)(((long long)K0 * n) % TS) / (double)TS, &ph_s[k], &ph_c[k]);
        }
        const long long l0 = (long long)ceil(xs[0] - 0.5 * kNuW);
        t.nu_l0[p] = (int)l0;
        for (int jt = 0; jt < kNuTaps; ++jt) {
            double wr = 0.0, wi = 0.0;
            for (int k = 0; k < 3; ++k) {
                // a stencil point at the top of the TS period wraps to the grid's start
                double d = xs[k] - (double)(l0 + jt);
                if (d > 0.5 * M) d -= M;
                if (d < -0.5 * M) d += M;
                const double f = L[k] * nu_kernel(d, beta) / (double)TS;
                wr += f * ph_c[k];
                wi += f * ph_s[k];
            }
            t.nu_w[(long long)jt * n_out + p] = mk((float)wr, (float)wi);
        }
        // re-ramp: az_times = linspace(n_ref - ft/2, n_ref + ft/2, down); K_a resampled S -> down
        const long long nr = qo * (S - 1);
        int ir = (int)(nr / (q.down - 1));
        float alr = (float)(nr - (long long)ir * (q.down - 1)) / (float)(q.down - 1);
        if (ir >= S - 1) {
            ir = S - 2;
            alr = 1.0f;
        }
        const df taur = df_from((q.n_ref - ft / 2) + qo * (((q.n_ref + ft / 2) - (q.n_ref - ft / 2)) / (double)(q.down - 1)));
        t.rer[p] = make_float4(__int_as_float(ir), alr, taur.hi, taur.lo);
    }
}

void tufr_tables(const TufrArgs& a, cudaStream_t st) {
    const long long n = std::max<long long>((long long)a.tmax * a.S, a.dnu.n);
    const int grid = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    note_launch(), k_tufr_tables<<<grid, 256, 0, st>>>(a.P, a.S, a.n_out, a.s0, a.dnu.n, a.tab);
}

// Staged-sample region (kTufrGroup range bins interleaved): what is left of
// two CTAs' shared memory per SM after the head and twiddles, when that also
// holds the grid and at least 1024 samples per range bin (checked with the
// occupancy calculator), else of one CTA's.
template <class K>
static bool fits_two(K kernel, int threads, size_t smem) {
    static bool attr = false;
    allow_smem(kernel, attr);
    int nb = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) == cudaSuccess && nb >= 2;
}

// Two CTAs of 384 threads per SM (85 registers a thread; 512-thread CTAs at
// 64 registers spilled and ran 4 % slower), else one of 1024.
constexpr int kTufrThreads = 384;

static int tufr_chunk(const TufrArgs& a, bool& two) {
    TufrArgs b = a;
    b.ychunk = 0;
    const TufrLayout L(b);
    static std::mutex mu;
    static std::map<int, std::pair<int, bool>> memo;   // grid length -> (chunk, two per SM)
    std::lock_guard<std::mutex> lk(mu);
    auto it = memo.find(a.dnu.n);
    if (it != memo.end()) {
        two = it->second.second;
        return it->second.first;
    }
    const long long fixed = L.head + L.tw;
    long long cap = (114LL * 1024 - 1024) / (long long)sizeof(cf32) - fixed;
    cap -= cap % 16;
    two = false;
    for (; cap >= L.grid && cap >= 1024LL * kTufrGroup; cap -= 16)
        if (fits_two(k_tufr_fused<kTufrThreads>, kTufrThreads, sizeof(cf32) * (size_t)(fixed + cap))) {
            two = true;
            break;
        }
    if (!two) cap = (long long)kSmemBytes / (long long)sizeof(cf32) - fixed;
    if (cap < L.grid || cap < 512LL * kTufrGroup) throw std::runtime_error("time unfolding: shared memory");
    const int chunk = (int)(cap / 2 * 2);
    memo[a.dnu.n] = {chunk, two};
    return chunk;
}

int tufr_ctas_per_sm(const TufrArgs& a) {
    bool two = false;
    tufr_chunk(a, two);
    return two ? 2 : 1;
}

void tufr_fused(const TufrArgs& args, int grid, cudaStream_t st) {
    TufrArgs a = args;
    bool two = false;
    a.ychunk = tufr_chunk(a, two);
    const size_t smem = sizeof(cf32) * TufrLayout(a).floats(a);
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("time unfolding: shared memory");
    if (two) {
        static bool b = false;
        allow_smem(k_tufr_fused<kTufrThreads>, b);
        note_launch(), k_tufr_fused<kTufrThreads><<<grid, kTufrThreads, smem, st>>>(a);
    } else {
        static bool b = false;
        allow_smem(k_tufr_fused<1024>, b);
        note_launch(), k_tufr_fused<1024><<<grid, 1024, smem, st>>>(a);
    }
}

// Scalars of azimuth_time_ufr (tile count, band, output crop), FP64, one block.
// K_a is evaluated analytically (the reference's az_fm_rate table).
// K_a of azimuth row i at range bin j (get_effective_velocities and the
// s1_decoder.cpp:667-676 expression), FP64.
__device__ __forceinline__ double ka_at(const RowParam* rows, const double* slant, const double* f_dc, int i, int j) {
    const double wl = 299792458.0 / 5.405000454334350e+9;
    const RowParam rp = rows[i];
    const double R = slant[j];
    const double num = rp.re * rp.re + rp.h * rp.h - R * R;
    const double beta = num / (2 * rp.re * rp.h);
    const double vg = rp.re * rp.v * beta / rp.h;
    const double v = sqrt(rp.v * vg);
    const double fa = rp.fa + f_dc[j];
    const double D = sqrt(1 - ((wl * wl) * (fa * fa)) / (4 * v * v));
    return (-2 * (v * v) * (D * D * D)) / (wl * R);
}

// K_a along the first range bin, all azimuth rows in parallel.
__global__ void k_ka_row0(const RowParam* rows, const double* slant, const double* f_dc, int S, double* ka0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S) ka0[i] = ka_at(rows, slant, f_dc, i, 0);
}

__global__ void k_tufr_params_fast(const RowParam* rows, const double* slant, const double* f_dc, int S, int n_r,
                                   double rate, double T, double prf, double bd, int swath_number,
                                   const double* ka0, TufrDev* out) {
    __shared__ double part[256];
    // ordered blocked sum of K_a over the first range bin (contiguous runs per thread)
    const int per = (S + blockDim.x - 1) / blockDim.x;
    double acc = 0.0;
    for (int i = threadIdx.x * per; i < min(S, (int)(threadIdx.x + 1) * per); ++i) acc += ka0[i];
    part[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double partial = 0.0;
    for (int k = 0; k < (int)blockDim.x; ++k) partial += part[k];
    auto ka_at_ = [&](int i, int j) { return ka_at(rows, slant, f_dc, i, j); };
    TufrDev d;
    TufrParams& q = d.q;
    const int num_az = S, num_rng = n_r;
    const double num_replicas = fabs(rate * T / prf);
    q.bandwidth = (num_replicas * prf) - bd;
    q.ka_mean = fabs(partial) / num_az;
    double ft = T + ((q.bandwidth - (2 * bd)) / q.ka_mean);
    double ka_ref;
    if (num_az / 2 < num_rng && num_rng / 2 < num_az) ka_ref = ka_at_(num_rng / 2, num_az / 2);
    else ka_ref = ka_at_(num_az / 2, num_rng / 2);
    q.n_ref = f_dc[num_rng / 2] / ka_ref;
    ft *= (swath_number != 11) ? 0.9 : 1.05;
    q.focused_time = ft;
    const int pos = (int)ceil((q.n_ref + ft / 2) / T);
    const int neg = (int)floor((q.n_ref - ft / 2) / T);
    q.num_tiles = pos - neg;
    const int ext = swath_number == 11 ? (int)floor(bd * 1.15) : (int)floor(bd * 0.26);
    q.output_shape = (int)floor(prf * T);
    q.down = q.output_shape + ext;
    q.shape = q.num_tiles * num_az;
    const int mid = q.shape / 2;
    q.start = (int)(mid - q.bandwidth / 2);
    q.end = (int)(mid + q.bandwidth / 2);
    q.ok = (q.num_tiles >= 1 && q.num_tiles <= 64 && q.start >= 0 && q.end <= q.shape && q.down >= 3) ? 1 : 0;
    *out = d;
}

void tufr_params_fast(const RowParam* rows, const double* slant, const double* f_dc, int S, int n_r, double rate,
                      double T, double prf, double bd, int swath_number, double* ka0, TufrDev* out, cudaStream_t st) {
    note_launch(), k_ka_row0<<<(S + 127) / 128, 128, 0, st>>>(rows, slant, f_dc, S, ka0);
    note_launch(), k_tufr_params_fast<<<1, 256, 0, st>>>(rows, slant, f_dc, S, n_r, rate, T, prf, bd, swath_number,
                                                        ka0, out);
}

}  // namespace s1g
