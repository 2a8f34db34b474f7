// Fused FP32 kernels of the fast path.  Each stage of the reference's
// _range_compress / _azimuth_compress runs as one kernel that keeps its
// working line in shared memory:
//   k_rc_fused      range compression (pad, FFT, matched filter, IFFT, shift/crop)
//   k_fufr_fused    azimuth FFT + frequency unfolding,
//                   the two length-S DFTs done as band-limited chirp-z transforms
//   k_rowpass_fused range FFT, SRC, range IFFT, scaling, RCMC, azimuth filter
//   k_czt_rows      azimuth IFFT (length S, chirp-z) per range bin
//   k_tufr_fused    time unfolding + quadratic resampling + re-ramp, the
//                   length-(T*S) DFT split into T residue classes of length S
// The Doppler lag-1 sums come from s1g_dcest.cu.
// Phase arguments are formed in double-float (s1g_df.cuh); no FP64
// arithmetic runs per sample.
#include <cmath>
#include <stdexcept>

#include "s1g_fast.cuh"

namespace s1g {

__device__ __forceinline__ cf32 cexpf_fast(float th) {
    float s, c;
    __sincosf(th, &s, &c);
    return mk(c, s);
}

// CZT: X[k] = sum_{s<nin} x[s] exp(dir 2 pi i s k / P) (k < nout).
// czt_core leaves the convolution in buf (padded layout); czt_out(k) then
// reads X[k].  czt_run adds a store loop and a trailing barrier.
template <class LoadF>
__device__ __forceinline__ void czt_core(cf32* buf, const CztDev& c, int dir, LoadF load) {
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
    fft2_dit(buf, c.dm, -1);
    for (int q = threadIdx.x; q < m; q += blockDim.x) buf[pad(q)] = buf[pad(q)] * ldg(c.kern + q);
    __syncthreads();
    fft2_dif(buf, c.dm, +1);
}

__device__ __forceinline__ cf32 czt_out(const cf32* buf, const CztDev& c, int dir, int k) {
    cf32 v = ldg(c.chirp + k) * buf[pad(__ldg(c.dm.perm + k))];
    return dir > 0 ? conj(v) : v;
}

template <class LoadF, class StoreF>
__device__ __forceinline__ void czt_run(cf32* buf, const CztDev& c, int dir, LoadF load, StoreF store) {
    czt_core(buf, c, dir, load);
    for (int k = threadIdx.x; k < c.nout; k += blockDim.x) store(k, czt_out(buf, c, dir, k));
    __syncthreads();
}

// Row-wise CZT: out[row][k] = scale * X_row[k] (used for the azimuth IFFT of
// the time unfolding, length S, dir +1).
__global__ void __launch_bounds__(512) k_czt_rows(const cf32* __restrict__ in, long long ip, cf32* __restrict__ out,
                                                  long long op, CztDev c, int dir, float scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cf32* buf = reinterpret_cast<cf32*>(smem_raw);
    const cf32* x = in + (long long)blockIdx.x * ip;
    cf32* y = out + (long long)blockIdx.x * op;
    czt_core(buf, c, dir, [&](int q) { return x[q]; });
    for (int k = threadIdx.x; k < c.nout; k += blockDim.x) y[k] = czt_out(buf, c, dir, k) * scale;
}

void czt_rows(const cf32* in, long long ip, cf32* out, long long op, long long rows, const CztDev& c, int dir,
              float scale, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_czt_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        attr = true;
    }
    note_launch(), k_czt_rows<<<(unsigned)rows, 512, sizeof(cf32) * padded_len(c.dm.n), st>>>(in, ip, out, op, c, dir,
                                                                                              scale);
}

// ------------------------------------------------------------------ range compression
__global__ void __launch_bounds__(512) k_rc_fused(const cf32* __restrict__ raw, cf32* __restrict__ rc, int n_r,
                                                  int h, FftDesc<float> d, const cf32* __restrict__ ref) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cf32* buf = reinterpret_cast<cf32*>(smem_raw);
    const int M = d.n;
    const long long row = blockIdx.x;
    const cf32* x = raw + row * n_r;
    for (int q = threadIdx.x; q < M; q += blockDim.x) buf[pad(__ldg(d.perm + q))] = q < n_r ? x[q] : mk(0.f, 0.f);
    __syncthreads();
    fft2_dit(buf, d, -1);
    for (int k = threadIdx.x; k < M; k += blockDim.x) buf[pad(k)] = buf[pad(k)] * ldg(ref + k);
    __syncthreads();
    fft2_dif(buf, d, +1);
    cf32* y = rc + row * n_r;
    for (int k = threadIdx.x; k < n_r; k += blockDim.x) {
        int src = k - h;
        if (src < 0) src += M;
        y[k] = buf[pad(__ldg(d.perm + src))];
    }
}

void rc_fused(const cf32* raw, cf32* rc, int n_a, int n_r, int h, const FftDesc<float>& d, const cf32* ref,
              cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_rc_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        attr = true;
    }
    note_launch(), k_rc_fused<<<n_a, 512, sizeof(cf32) * padded_len(d.n), st>>>(raw, rc, n_r, h, d, ref);
}

// ------------------------------------------------------------------ frequency unfolding


__global__ void __launch_bounds__(512) k_fufr_fused(FufrArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int mbig = max(a.cf.dm.n, a.na_smooth ? 0 : a.cna.dm.n);
    cf32* big = reinterpret_cast<cf32*>(smem_raw);
    cf32* X = big + padded_len(mbig);   // n_a, natural order, padded layout
    cf32* band = X + padded_len(a.n_a); // bw
    const int j = blockIdx.x;
    const cf32* row = a.rcT + (long long)j * a.n_a;
    // azimuth FFT (length n_a) into X
    if (a.na_smooth) {
        for (int t = threadIdx.x; t < a.n_a; t += blockDim.x) X[pad(__ldg(a.dna.perm + t))] = row[t];
        __syncthreads();
        fft2_dit(X, a.dna, -1);
    } else {
        czt_run(big, a.cna, -1, [&](int q) { return row[q]; }, [&](int k, cf32 v) { X[pad(k)] = v; });
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
        [&](int k, cf32 v) { band[k] = v; });
    // inverse DFT_S of the band moved to the front, re-ramp, 1/S
    cf32* out = a.out + (long long)j * a.S;
    czt_run(big, a.ci, +1, [&](int q) { return band[q]; },
            [&](int k, cf32 v) { out[k] = v * ldg(a.reramp + k); });
}

void fufr_fused(const FufrArgs& a, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_fufr_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        attr = true;
    }
    const int mbig = std::max(a.cf.dm.n, a.na_smooth ? 0 : a.cna.dm.n);
    const size_t smem = sizeof(cf32) * ((size_t)padded_len(mbig) + padded_len(a.n_a) + a.bw);
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("frequency unfolding: shared memory");
    note_launch(), k_fufr_fused<<<a.n_r, 512, smem, st>>>(a);
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
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double sr = 0.0, si = 0.0;
        for (int c = 0; c < nchunk; ++c) {
            sr += part[(long long)c * n + j].x;
            si += part[(long long)c * n + j].y;
        }
        f_dc[j] = -a.prf * atan2(si, sr) / (2 * kPIref);
    }
    __syncthreads();
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

void dc_fit_fast(const cf64* part, int nchunk, const DcFitArgs& a, double* f_dc, df* f_dc_df, cudaStream_t st) {
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

__global__ void __launch_bounds__(512) k_rowpass_fused(RowArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cf32* buf = reinterpret_cast<cf32*>(smem_raw);
    const int i = blockIdx.x;
    const RowDf rp = a.rows[i];
    cf32* row = a.data + (long long)i * a.n_r;
    const int n = a.n_r;
    const float l24 = a.lam2_4.hi;
    if (a.smooth) {
        if (a.tops) {
            for (int j = threadIdx.x; j < n; j += blockDim.x) buf[pad(__ldg(a.d.perm + j))] = row[j];
            __syncthreads();
            fft2_dit(buf, a.d, -1);
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                buf[pad(j)] = buf[pad(j)] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
        } else {
            // stripmap: the SRC phase is applied to the range-time samples
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                buf[pad(j)] = row[j] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
        }
        __syncthreads();
        fft2_dif(buf, a.d, +1);
        for (int j = threadIdx.x; j < n; j += blockDim.x)
            row[j] = buf[pad(__ldg(a.d.perm + j))] * post_factor(rp, a.cols[j], a.fdc[j], a.lam2_4, a.tops);
    } else {
        if (a.tops) {
            czt_run(buf, a.cz, -1, [&](int q) { return row[q]; },
                    [&](int k, cf32 v) { row[k] = v * cexpf_fast(src_phase(rp, a.cols[k], a.fdc[k], l24)); });
        } else {
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                row[j] = row[j] * cexpf_fast(src_phase(rp, a.cols[j], a.fdc[j], l24));
            __syncthreads();
        }
        czt_run(buf, a.cz, +1, [&](int q) { return row[q]; },
                [&](int k, cf32 v) { row[k] = v * post_factor(rp, a.cols[k], a.fdc[k], a.lam2_4, a.tops); });
    }
}

void rowpass_fused(const RowArgs& a, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_rowpass_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                   "attr");
        attr = true;
    }
    const int m = a.smooth ? a.d.n : a.cz.dm.n;
    note_launch(), k_rowpass_fused<<<a.S, 512, sizeof(cf32) * padded_len(m), st>>>(a);
}

// ------------------------------------------------------------------ time unfolding


struct KnotDf {
    df kt, dct, u;
};

__device__ __forceinline__ KnotDf load_knot(const float* KN, int i) {
    const float4 a = *reinterpret_cast<const float4*>(KN + 8 * i);
    const float2 b = *reinterpret_cast<const float2*>(KN + 8 * i + 4);
    KnotDf k;
    k.kt = df_make(a.x, a.y);
    k.dct = df_make(a.z, a.w);
    k.u = df_make(b.x, b.y);
    return k;
}

// Deramp / re-ramp phase of azimuth_time_ufr (image_formation.cpp:305-313,
// 365-373) at a resampled position between knots i and i+1 (fraction al),
// time tau: sgn = -1 for the deramp, +1 for the re-ramp.
__device__ __forceinline__ float tufr_phase(const KnotDf& k0, const KnotDf& k1, float al, df tau, int sgn, df pi_,
                                            df two_pi_) {
    const df kt = df_add(k0.kt, df_mul_f(df_sub(k1.kt, k0.kt), al));
    const df dct = df_add(k0.dct, df_mul_f(df_sub(k1.dct, k0.dct), al));
    const df u = df_add(k0.u, df_mul_f(df_sub(k1.u, k0.u), al));
    const df t = df_add(dct, tau);
    const df th1 = df_mul(df_mul(pi_, kt), df_mul(t, t));
    const df th2 = df_mul(df_mul(df_mul(two_pi_, df_add(kt, u)), dct), t);
    const df th = sgn < 0 ? df_add(df_neg(th1), th2) : df_sub(th1, th2);
    return df_wrap(th);
}

__global__ void __launch_bounds__(512) k_tufr_fused(TufrArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TufrParams q = a.P->q;
    const int S = a.S;
    const int T = q.num_tiles;
    if (T > a.tmax || q.end - q.start > a.bwmax || !q.ok) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *a.status = 1;
        return;
    }
    const int mbig = max(a.cf.dm.n, a.ci.dm.n);
    cf32* big = reinterpret_cast<cf32*>(smem_raw);    // padded mbig
    cf32* acc = big + padded_len(mbig);                // n_out
    const long long TS = (long long)T * S;
    const int bw = q.end - q.start;
    cf32* V = a.V + (long long)blockIdx.x * a.tmax * S;
    cf32* ZB = a.ZB + (long long)blockIdx.x * a.bwmax;
    float* KN = a.KN + (long long)blockIdx.x * 8 * S;
    const double ft = q.focused_time;
    const df tau0 = df_from(-ft / 2);
    const df tstep = df_from((ft / 2 - (-ft / 2)) / (double)(TS - 1));
    const df tau0r = df_from(q.n_ref - ft / 2);
    const df tstepr = df_from(((q.n_ref + ft / 2) - (q.n_ref - ft / 2)) / (double)(q.down - 1));
    for (int j = blockIdx.x; j < a.n_r; j += gridDim.x) {
        // 1. the azimuth IFFT (length S, 1/S, s1_decoder.cpp:682) ran in k_czt_rows
        const cf32* A = a.in + (long long)j * S;
        const ColDf cj = a.cols[j];
        const df fdc = a.fdc[j];
        const df ilr = a.inv_lamR[j];
        // 2. K_a, kt and dct at the S knots of this range bin
        for (int s = threadIdx.x; s < S; s += blockDim.x) {
            const RowDf r = a.rows[s];
            const df F = df_add(r.fa, fdc);
            const df vq = df_mul(r.P, df_sub(r.A, cj.Q));
            const df x = df_div(df_mul(a.lam2_4, df_mul(F, F)), vq);
            const df D = df_sqrt(df_sub(df_make(1.f, 0.f), x));
            const df D3 = df_mul(D, df_mul(D, D));
            const df u = df_neg(df_mul(df_mul(df_mul(df_make(2.f, 0.f), vq), D3), ilr));   // -2 v^2 D^3/(lambda R)
            const df kt = df_neg(df_div(df_mul(u, a.rate), df_sub(a.rate, u)));              // -u r / (r - u)
            const df dct = df_neg(df_div(fdc, u));                                          // -f_dc / u
            *reinterpret_cast<float4*>(KN + 8 * s) = make_float4(kt.hi, kt.lo, dct.hi, dct.lo);
            *reinterpret_cast<float2*>(KN + 8 * s + 4) = make_float2(u.hi, u.lo);
        }
        __syncthreads();
        // 3. deramp the T tiles and split into residue classes r:
        //    v_r[s] = exp(-2 pi i s r / (T S)) sum_t y[s + S t] exp(-2 pi i t r / T)
        for (int s = threadIdx.x; s < S; s += blockDim.x) {
            const cf32 as = A[s];
            for (int r0 = 0; r0 < T; r0 += 8) {
                cf32 accr[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) accr[u] = mk(0.f, 0.f);
                for (int t = 0; t < T; ++t) {
                    const long long n = s + (long long)S * t;
                    const long long num = n * (S - 1);
                    int i = (int)(num / (TS - 1));
                    float al = (float)(num - (long long)i * (TS - 1)) / (float)(TS - 1);
                    if (i >= S - 1) {
                        i = S - 2;
                        al = 1.0f;
                    }
                    const KnotDf k0 = load_knot(KN, i), k1 = load_knot(KN, i + 1);
                    const df tau = df_add(tau0, df_mul_f(tstep, (float)n));
                    const cf32 y = as * cexpf_fast(tufr_phase(k0, k1, al, tau, -1, a.pi_, a.two_pi_));
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int r = r0 + u;
                        if (r < T) {
                            float sn, cs;
                            sincospif(-2.0f * (float)((t * r) % T) / (float)T, &sn, &cs);
                            accr[u] = accr[u] + y * mk(cs, sn);
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int r = r0 + u;
                    if (r < T) {
                        float sn, cs;
                        sincospif(-2.0f * (float)(((long long)s * r) % TS) / (float)TS, &sn, &cs);
                        V[(long long)r * S + s] = accr[u] * mk(cs, sn);
                    }
                }
            }
        }
        __syncthreads();
        // 4. forward residue CZTs: Z[T q + r] for the band [start, end)
        for (int r = 0; r < T; ++r) {
            const int q0 = a.P->q0[r];
            const int kc = a.P->kcount[r];
            const cf32* vr = V + (long long)r * S;
            czt_run(
                big, a.cf, -1,
                [&](int s) {
                    float sn, cs;
                    sincospif(-2.0f * (float)(((long long)s * q0) % S) / (float)S, &sn, &cs);
                    return vr[s] * mk(cs, sn);
                },
                [&](int k, cf32 v) {
                    if (k < kc) ZB[(long long)T * (q0 + k) + r - q.start] = v;
                });
        }
        for (int p = threadIdx.x; p < a.n_out; p += blockDim.x) acc[p] = mk(0.f, 0.f);
        __syncthreads();
        // 5. inverse residue CZTs and the 3-point Lagrange stencils of the
        //    quadratic resampling (signal_processing.cpp:109-155)
        for (int r = 0; r < T; ++r) {
            const int kin = (bw - r + T - 1) / T;
            czt_core(big, a.ci, +1, [&](int qq) { return qq < kin ? ZB[(long long)T * qq + r] : mk(0.f, 0.f); });
            for (int p = threadIdx.x; p < a.n_out; p += blockDim.x) {
                const long long qo = a.s0 + p;
                const long long num = qo * (TS - 1);
                int i = (int)(num / (q.down - 1));
                float xi = (float)(num - (long long)i * (q.down - 1)) / (float)(q.down - 1);
                if (i > TS - 2) {
                    xi += (float)(i - (TS - 2));
                    i = (int)(TS - 2);
                }
                const float L0 = 0.5f * xi * (xi - 1.0f);
                const float L1 = -(xi + 1.0f) * (xi - 1.0f);
                const float L2 = 0.5f * (xi + 1.0f) * xi;
                cf32 sum = mk(0.f, 0.f);
                const long long nk[3] = {i - 1, i, i + 1};
                const float Lk[3] = {L0, L1, L2};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const long long nn = nk[k];
                    float sn, cs;
                    sincospif(2.0f * (float)(((long long)r * nn) % TS) / (float)TS, &sn, &cs);
                    sum = sum + czt_out(big, a.ci, +1, (int)(nn % S)) * mk(cs, sn) * Lk[k];
                }
                acc[p] = acc[p] + sum;
            }
            __syncthreads();
        }
        // 6. re-ramp (image_formation.cpp:355-378) and store the cropped rows
        cf32* out = a.out + (long long)j * a.n_out;
        const float invTS = 1.0f / (float)TS;
        for (int p = threadIdx.x; p < a.n_out; p += blockDim.x) {
            const long long qo = a.s0 + p;
            const long long num = qo * (S - 1);
            int i = (int)(num / (q.down - 1));
            float al = (float)(num - (long long)i * (q.down - 1)) / (float)(q.down - 1);
            if (i >= S - 1) {
                i = S - 2;
                al = 1.0f;
            }
            const KnotDf k0 = load_knot(KN, i), k1 = load_knot(KN, i + 1);
            const df tau = df_add(tau0r, df_mul_f(tstepr, (float)qo));
            out[p] = acc[p] * invTS * cexpf_fast(tufr_phase(k0, k1, al, tau, +1, a.pi_, a.two_pi_));
        }
        __syncthreads();
    }
}

void tufr_fused(const TufrArgs& a, int grid, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_tufr_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        attr = true;
    }
    const int mbig = std::max(a.cf.dm.n, a.ci.dm.n);
    const size_t smem = sizeof(cf32) * ((size_t)padded_len(mbig) + a.n_out);
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("time unfolding: shared memory");
    note_launch(), k_tufr_fused<<<grid, 512, smem, st>>>(a);
}

// Scalars of azimuth_time_ufr plus the residue band layout, FP64, one block.
// K_a is evaluated analytically (the reference's az_fm_rate table).
__global__ void k_tufr_params_fast(const RowParam* rows, const double* slant, const double* f_dc, int S, int n_r,
                                   double rate, double T, double prf, double bd, int swath_number, TufrDev* out) {
    __shared__ double ka0[1024];
    __shared__ double partial;
    const double wl = 299792458.0 / 5.405000454334350e+9;
    auto ka_at = [&](int i, int j) {
        const RowParam rp = rows[i];
        const double R = slant[j];
        const double num = rp.re * rp.re + rp.h * rp.h - R * R;
        const double beta = num / (2 * rp.re * rp.h);
        const double vg = rp.re * rp.v * beta / rp.h;
        const double v = sqrt(rp.v * vg);
        const double fa = rp.fa + f_dc[j];
        const double D = sqrt(1 - ((wl * wl) * (fa * fa)) / (4 * v * v));
        return (-2 * (v * v) * (D * D * D)) / (wl * R);
    };
    if (threadIdx.x == 0) partial = 0.0;
    __syncthreads();
    // sequential sum in chunks of blockDim (keeps the reference's order)
    for (int base = 0; base < S; base += blockDim.x) {
        const int i = base + threadIdx.x;
        if (i < S) ka0[threadIdx.x] = ka_at(i, 0);
        __syncthreads();
        if (threadIdx.x == 0) {
            double acc = partial;
            for (int k = 0; k < (int)blockDim.x && base + k < S; ++k) acc += ka0[k];
            partial = acc;
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    TufrDev d;
    TufrParams& q = d.q;
    const int num_az = S, num_rng = n_r;
    const double num_replicas = fabs(rate * T / prf);
    q.bandwidth = (num_replicas * prf) - bd;
    q.ka_mean = fabs(partial) / num_az;
    double ft = T + ((q.bandwidth - (2 * bd)) / q.ka_mean);
    double ka_ref;
    if (num_az / 2 < num_rng && num_rng / 2 < num_az) ka_ref = ka_at(num_rng / 2, num_az / 2);
    else ka_ref = ka_at(num_az / 2, num_rng / 2);
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
    const int Tn = q.num_tiles;
    for (int r = 0; r < 64; ++r) {
        d.q0[r] = 0;
        d.kcount[r] = 0;
        if (q.ok && r < Tn) {
            const int q0 = q.start >= r ? (q.start - r + Tn - 1) / Tn : 0;
            const int q1 = (q.end - r + Tn - 1) / Tn;   // first q with T q + r >= end
            d.q0[r] = q0;
            d.kcount[r] = q1 > q0 ? q1 - q0 : 0;
        }
    }
    *out = d;
}

void tufr_params_fast(const RowParam* rows, const double* slant, const double* f_dc, int S, int n_r, double rate,
                      double T, double prf, double bd, int swath_number, TufrDev* out, cudaStream_t st) {
    note_launch(), k_tufr_params_fast<<<1, 256, 0, st>>>(rows, slant, f_dc, S, n_r, rate, T, prf, bd, swath_number,
                                                        out);
}

}  // namespace s1g
