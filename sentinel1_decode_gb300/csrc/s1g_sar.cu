// SAR stage kernels of the per-burst pipeline (range compression pieces,
// Doppler centroid, frequency/time-domain unfolding, the per-row SRC / RCMC /
// azimuth filter, ECCM).  Arithmetic follows the reference function named
// at each kernel; phases are generated in FP64 and wrapped before the
// complex exponential, so the FP32 instantiations only round the result.
#include <cmath>
#include <stdexcept>

#include "s1g_kernels.h"

namespace s1g {

// Constants of structs.h:23-34 (PI is truncated there; reproduced).
constexpr double kPI = 3.14159265358979;
constexpr double kC = 299792458.0;
constexpr double kCenterFreq = 5.405000454334350e+9;
constexpr double kWavelength = kC / kCenterFreq;

static inline int grid1(long long total, int threads = 256) {
    long long g = (total + threads - 1) / threads;
    return (int)std::max(1LL, std::min(g, 152LL * 32));
}

#define GRID_STRIDE(i, total) \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (total); i += (long long)gridDim.x * blockDim.x)

template <typename R>
__device__ __forceinline__ cpx<R> expi(double theta) {
    double s, c;
    sincos(theta, &s, &c);
    return mk((R)c, (R)s);
}

// ------------------------------------------------------------------ elementwise
template <typename R>
__global__ void k_pad_rows(const cpx<R>* in, long long ip, int n_in, cpx<R>* out, long long op, int n_out, long long rows) {
    GRID_STRIDE(i, rows * n_out) {
        const long long r = i / n_out;
        const int q = (int)(i % n_out);
        out[r * op + q] = q < n_in ? in[r * ip + q] : mk((R)0, (R)0);
    }
}
template <typename R>
void pad_rows(const cpx<R>* in, long long ip, int n_in, cpx<R>* out, long long op, int n_out, long long rows,
              cudaStream_t st) {
    note_launch(), k_pad_rows<R><<<grid1(rows * n_out), 256, 0, st>>>(in, ip, n_in, out, op, n_out, rows);
}

template <typename R>
__global__ void k_mul_rows_by_vec(cpx<R>* a, long long p, int n, long long rows, const cpx<R>* v) {
    GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int q = (int)(i % n);
        a[r * p + q] = a[r * p + q] * v[q];
    }
}
template <typename R>
void mul_rows_by_vec(cpx<R>* a, long long p, int n, long long rows, const cpx<R>* v, cudaStream_t st) {
    note_launch(), k_mul_rows_by_vec<R><<<grid1(rows * n), 256, 0, st>>>(a, p, n, rows, v);
}

// out[k] = in[(k - h) mod m]: the fftshift + crop of s1g_decoder.cpp:493-497
// expressed on the shorter correlation length m.
template <typename R>
__global__ void k_rc_crop(const cpx<R>* in, long long ip, int m, cpx<R>* out, long long op, int n_r, int h, long long rows) {
    GRID_STRIDE(i, rows * n_r) {
        const long long r = i / n_r;
        const int k = (int)(i % n_r);
        int src = k - h;
        if (src < 0) src += m;
        out[r * op + k] = in[r * ip + src];
    }
}
template <typename R>
void rc_crop(const cpx<R>* in, long long ip, int m, cpx<R>* out, long long op, int n_r, int h, long long rows,
             cudaStream_t st) {
    note_launch(), k_rc_crop<R><<<grid1(rows * n_r), 256, 0, st>>>(in, ip, m, out, op, n_r, h, rows);
}

// out[k] = in[(k - shift) mod n] (std::rotate right by shift)
template <typename R>
__global__ void k_roll_rows(const cpx<R>* in, long long ip, cpx<R>* out, long long op, int n, int shift, long long rows) {
    GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int k = (int)(i % n);
        int src = k - shift;
        if (src < 0) src += n;
        out[r * op + k] = in[r * ip + src];
    }
}
template <typename R>
void roll_rows(const cpx<R>* in, long long ip, cpx<R>* out, long long op, int n, int shift, long long rows,
               cudaStream_t st) {
    note_launch(), k_roll_rows<R><<<grid1(rows * n), 256, 0, st>>>(in, ip, out, op, n, shift, rows);
}

template <typename R>
__global__ void k_scale_mul_vec(cpx<R>* a, long long p, int n, long long rows, const cpx<R>* v, double scale) {
    GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int q = (int)(i % n);
        cpx<R> x = a[r * p + q] * (R)scale;
        a[r * p + q] = x * v[q];
    }
}
template <typename R>
void scale_mul_vec(cpx<R>* a, long long p, int n, long long rows, const cpx<R>* v, double scale, cudaStream_t st) {
    note_launch(), k_scale_mul_vec<R><<<grid1(rows * n), 256, 0, st>>>(a, p, n, rows, v, scale);
}

template <typename R>
__global__ void k_scale_rows(cpx<R>* a, long long p, int n, long long rows, double scale) {
    GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int q = (int)(i % n);
        a[r * p + q] = a[r * p + q] * (R)scale;
    }
}
template <typename R>
void scale_rows(cpx<R>* a, long long p, int n, long long rows, double scale, cudaStream_t st) {
    note_launch(), k_scale_rows<R><<<grid1(rows * n), 256, 0, st>>>(a, p, n, rows, scale);
}

template <typename R>
__global__ void k_band_select(const cpx<R>* Y, long long yp, cpx<R>* Z, long long zp, int n, int start, int len, long long rows) {
    GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int q = (int)(i % n);
        Z[r * zp + q] = q < len ? Y[r * yp + start + q] : mk((R)0, (R)0);
    }
}
template <typename R>
void band_select(const cpx<R>* Y, long long yp, cpx<R>* Z, long long zp, int n, int start, int len, long long rows,
                 cudaStream_t st) {
    note_launch(), k_band_select<R><<<grid1(rows * n), 256, 0, st>>>(Y, yp, Z, zp, n, start, len, rows);
}

template <typename To, typename Ti>
__global__ void k_convert_rows(const cpx<Ti>* in, long long ip, cpx<To>* out, long long op, int cols, int valid,
                               long long rows) {
    GRID_STRIDE(i, rows * cols) {
        const long long r = i / cols;
        const int c = (int)(i % cols);
        out[r * op + c] = c < valid ? mk((To)in[r * ip + c].x, (To)in[r * ip + c].y) : mk((To)0, (To)0);
    }
}
template <typename To, typename Ti>
void convert_rows(const cpx<Ti>* in, long long ip, cpx<To>* out, long long op, int cols, int valid, long long rows,
                  cudaStream_t st) {
    note_launch(), k_convert_rows<To, Ti><<<grid1(rows * cols), 256, 0, st>>>(in, ip, out, op, cols, valid, rows);
}

// ------------------------------------------------------------------ Doppler
// Lag-1 sums of the deramped range-compressed burst per range bin
// (dce_preconditioning + get_wrapped_estimates, doppler.cpp:4-39,119-143).
template <typename R>
__global__ void k_dc_sums(const cpx<R>* rc, long long p, int n_a, int n_r, const cpx<R>* d, cf64* sums) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_r) return;
    double sr = 0.0, si = 0.0;
    cpx<R> prev = rc[j] * d[0];
    for (int a = 0; a < n_a - 1; ++a) {
        const cpx<R> next = rc[(long long)(a + 1) * p + j] * d[a + 1];
        // cur * conj(next)
        sr += (double)prev.x * (double)next.x + (double)prev.y * (double)next.y;
        si += (double)prev.y * (double)next.x - (double)prev.x * (double)next.y;
        prev = next;
    }
    sums[j] = mk(sr, si);
}
template <typename R>
void dc_sums(const cpx<R>* rc, long long p, int n_a, int n_r, const cpx<R>* d, cf64* sums, cudaStream_t st) {
    note_launch(), k_dc_sums<R><<<(n_r + 127) / 128, 128, 0, st>>>(rc, p, n_a, n_r, d, sums);
}

// get_doppler_centroid after the sums: block means, get_unwrapped_estimates
// (doppler.cpp:42-95), polyfit (signal_processing.cpp:159-214), evaluation.
__global__ void k_dc_fit(const cf64* sums, DcFitArgs a, double* f_dc) {
    __shared__ double fine[64];
    __shared__ double poly[3];
    const int n = a.n_rng;
    const int nb = a.num_blocks;
    // wrapped estimates into f_dc (temporary)
    for (int j = threadIdx.x; j < n; j += blockDim.x)
        f_dc[j] = -a.prf * atan2(sums[j].y, sums[j].x) / (2 * kPI);
    __syncthreads();
    const int bs = n / nb;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const int s = b * bs;
        const int e = (s + bs < n) ? s + bs : n - 1;
        double acc = 0.0;
        for (int j = s; j < e; ++j) acc += f_dc[j];
        fine[b] = acc / ((double)e - (double)s);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int dense = 8;
        const int m = nb * dense;
        const float dt = (float)(a.rt[1] - a.rt[0]);
        // F = floor(|exp(2 pi i dc/prf)|) for the estimates, zero padded
        double best = -1.0;
        int bi = 0;
        double bre = 0.0, bim = 0.0;
        for (int k = 0; k < m; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < nb; ++j) {
                double s, c;
                sincos((2.0 * kPI) * fine[j] / a.prf, &s, &c);
                const double f = floor(hypot(c, s));
                if (f == 0.0) continue;
                double ws, wc;
                sincospi(-2.0 * (double)((long long)j * k % m) / (double)m, &ws, &wc);
                re += f * wc;
                im += f * ws;
            }
            const double mag = hypot(re, im);
            const double p2 = mag * mag;
            if (p2 > best) {
                best = p2;
                bi = k;
                bre = re;
                bim = im;
            }
        }
        const double val = 1.0 / (m * (double)dt);
        const int N = (m - 1) / 2 + 1;
        const double v = bi < N ? bi * val : (bi - m) * val;
        const double aa = v / (double)dt;
        const double bb = atan2(bim, bre) / (2.0 * kPI);
        double un[64];
        for (int j = 0; j < nb; ++j) {
            double s1, c1, s2, c2;
            sincos((2.0 * kPI) * fine[j] / a.prf, &s1, &c1);
            sincos(-1.0 * (aa * a.rt[j] + bb), &s2, &c2);
            const double pr = c1 * c2 - s1 * s2, pi_ = c1 * s2 + s1 * c2;
            const double res = atan2(pi_, pr) / (2.0 * kPI);
            un[j] = (aa * a.rt[j] + bb + res) * a.prf;
        }
        // polyfit, degree 2
        double Sx[5] = {0, 0, 0, 0, 0}, Sy[3] = {0, 0, 0};
        for (int i = 0; i < nb; ++i) {
            double xi = 1.0;
            for (int j = 0; j <= 4; ++j) {
                if (j <= 2) Sy[j] += xi * un[i];
                Sx[j] += xi;
                xi *= a.rt[i];
            }
        }
        double A[3][3] = {{Sx[0], Sx[1], Sx[2]}, {Sx[1], Sx[2], Sx[3]}, {Sx[2], Sx[3], Sx[4]}};
        double B[3] = {Sy[0], Sy[1], Sy[2]};
        for (int i = 0; i < 3; ++i) {
            for (int k = i + 1; k < 3; ++k) {
                if (fabs(A[k][i]) > fabs(A[i][i])) {
                    for (int j = 0; j < 3; ++j) {
                        const double t = A[i][j];
                        A[i][j] = A[k][j];
                        A[k][j] = t;
                    }
                    const double t = B[i];
                    B[i] = B[k];
                    B[k] = t;
                }
            }
            for (int k = i + 1; k < 3; ++k) {
                const double f = A[k][i] / A[i][i];
                for (int j = i; j < 3; ++j) A[k][j] -= f * A[i][j];
                B[k] -= f * B[i];
            }
        }
        double c[3];
        for (int i = 2; i >= 0; --i) {
            c[i] = B[i];
            for (int j = i + 1; j < 3; ++j) c[i] -= A[i][j] * c[j];
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
        f_dc[j] = (poly[0] + poly[1] * t + poly[2] * t * t);
    }
}
void dc_fit(const cf64* sums, const DcFitArgs& a, double* f_dc, cudaStream_t st) {
    note_launch(), k_dc_fit<<<1, 256, 0, st>>>(sums, a, f_dc);
}

// ------------------------------------------------------------------ frequency UFR
// y[k] = shifted_X[k mod n_a] * deramp[k] for k < tile_len (get_tiled_signal,
// image_formation.cpp:87-122, after the azimuth fftshift, :139-140).
template <typename R>
__global__ void k_fufr_prep(const cpx<R>* X, long long xp, int n_a, cpx<R>* y, long long yp, int S, int tile_len,
                            const cpx<R>* d, long long rows) {
    GRID_STRIDE(i, rows * S) {
        const long long r = i / S;
        const int k = (int)(i % S);
        cpx<R> v = mk((R)0, (R)0);
        if (k < tile_len) {
            int q = (k % n_a) - n_a / 2;
            if (q < 0) q += n_a;
            v = X[r * xp + q] * d[k];
        }
        y[r * yp + k] = v;
    }
}
template <typename R>
void fufr_prep(const cpx<R>* X, long long xp, int n_a, cpx<R>* y, long long yp, int S, int tile_len, const cpx<R>* d,
               long long rows, cudaStream_t st) {
    note_launch(), k_fufr_prep<R><<<grid1(rows * S), 256, 0, st>>>(X, xp, n_a, y, yp, S, tile_len, d, rows);
}

// ------------------------------------------------------------------ row pass
// effective velocity, image_formation.cpp:406-416
__device__ __forceinline__ double v_rel_of(const RowParam& rp, double R) {
    const double num = rp.re * rp.re + rp.h * rp.h - R * R;
    const double den = 2 * rp.re * rp.h;
    const double beta = num / den;
    const double vg = rp.re * rp.v * beta / rp.h;
    return sqrt(rp.v * vg);
}

// SRC filter, image_formation.cpp:422-455
template <typename R>
__global__ void k_src(cpx<R>* data, long long p, int S, int n_r, const RowParam* rows, const double* slant,
                      const double* rf, const double* f_dc, double c3) {
    GRID_STRIDE(i, (long long)S * n_r) {
        const int row = (int)(i / n_r), j = (int)(i % n_r);
        const RowParam rp = rows[row];
        const double Rj = slant[j];
        const double v = v_rel_of(rp, Rj);
        const double fa = rp.fa + f_dc[j];
        const double D = sqrt(1 - ((kWavelength * kWavelength) * (fa * fa)) / (4 * v * v));
        double k = 2.0 * (v * v) * c3 * (D * D);
        k /= (kC * Rj * (fa * fa));
        const double th = (-kPI) * (rf[j] * rf[j]) / k;
        cpx<R>& x = data[(long long)row * p + j];
        x = x * expi<R>(th);
    }
}
template <typename R>
void src_filter(cpx<R>* data, long long p, int S, int n_r, const RowParam* rows, const double* slant,
                const double* rf, const double* f_dc, double c3, cudaStream_t st) {
    note_launch(), k_src<R><<<grid1((long long)S * n_r), 256, 0, st>>>(data, p, S, n_r, rows, slant, rf, f_dc, c3);
}

// scale, RCMC phase and azimuth filter: s1g_decoder.cpp:643-676,
// image_formation.cpp:458-476
template <typename R>
__global__ void k_azf(cpx<R>* data, long long p, int S, int n_r, const RowParam* rows, const double* slant,
                      const double* rf, const double* f_dc, const double* tcorr, const double* rscale, int tops) {
    GRID_STRIDE(i, (long long)S * n_r) {
        const int row = (int)(i / n_r), j = (int)(i % n_r);
        const RowParam rp = rows[row];
        const double Rj = slant[j];
        const double v = v_rel_of(rp, Rj);
        const double fa = rp.fa + f_dc[j];
        const double D = sqrt(1 - ((kWavelength * kWavelength) * (fa * fa)) / (4 * v * v));
        cpx<R> x = data[(long long)row * p + j];
        // x /= sqrt(pow(ref/R, 3)) -- divisor precomputed per column
        x = mk((R)((double)x.x / rscale[j]), (R)((double)x.y / rscale[j]));
        double th = 0.0;
        if (tops) {
            const double shift = (Rj / D) - Rj;
            th = ((((-4.0) * kPI) * rf[j]) * shift) / kC;
            x = x * expi<R>(th);
        }
        const double ph_t = ((2.0 * kPI) * fa) * tcorr[j];
        const double ph_a = (((4.0 * kPI) * Rj) * D) / kWavelength;
        double sa, ca, st_, ct;
        sincos(ph_a, &sa, &ca);
        sincos(ph_t, &st_, &ct);
        const double fr = ca * ct - sa * st_, fi = ca * st_ + sa * ct;
        x = x * mk((R)fr, (R)fi);
        data[(long long)row * p + j] = x;
    }
}
template <typename R>
void az_filter(cpx<R>* data, long long p, int S, int n_r, const RowParam* rows, const double* slant, const double* rf,
               const double* f_dc, const double* tcorr, const double* rscale, int tops, cudaStream_t st) {
    note_launch(), k_azf<R><<<grid1((long long)S * n_r), 256, 0, st>>>(data, p, S, n_r, rows, slant, rf, f_dc, tcorr, rscale, tops);
}

// K_a = -2 v^2 D^3 / (lambda R) (s1g_decoder.cpp:671-672), stored [n_r][S]
__global__ void k_ka_table(double* kaT, long long p, int S, int n_r, const RowParam* rows, const double* slant,
                           const double* f_dc) {
    GRID_STRIDE(i, (long long)S * n_r) {
        const int j = (int)(i / S), row = (int)(i % S);
        const RowParam rp = rows[row];
        const double Rj = slant[j];
        const double v = v_rel_of(rp, Rj);
        const double fa = rp.fa + f_dc[j];
        const double D = sqrt(1 - ((kWavelength * kWavelength) * (fa * fa)) / (4 * v * v));
        kaT[(long long)j * p + row] = (-2 * (v * v) * (D * D * D)) / (kWavelength * Rj);
    }
}
void ka_table(double* kaT, long long p, int S, int n_r, const RowParam* rows, const double* slant, const double* f_dc,
              cudaStream_t st) {
    note_launch(), k_ka_table<<<grid1((long long)S * n_r), 256, 0, st>>>(kaT, p, S, n_r, rows, slant, f_dc);
}

// ------------------------------------------------------------------ time UFR
// Scalars of azimuth_time_ufr (image_formation.cpp:233-268).
__global__ void k_tufr_params(const double* kaT, long long p, int S, int n_r, const double* f_dc, double dc_rate,
                              double T, double prf, double bd, int swath_number, TufrParams* out) {
    if (threadIdx.x != 0) return;
    TufrParams q;
    const int num_az = S, num_rng = n_r;
    const double num_replicas = fabs(dc_rate * T / prf);
    q.bandwidth = (num_replicas * prf) - bd;
    double acc = 0.0;
    for (int i = 0; i < num_az; ++i) acc += kaT[i];
    q.ka_mean = fabs(acc) / num_az;
    double ft = T + ((q.bandwidth - (2 * bd)) / q.ka_mean);
    double ka_ref;
    if (num_az / 2 < num_rng && num_rng / 2 < num_az)
        ka_ref = kaT[(long long)(num_az / 2) * p + num_rng / 2];
    else  // the reference indexes outside its array here; use the intended element
        ka_ref = kaT[(long long)(num_rng / 2) * p + num_az / 2];
    q.n_ref = f_dc[num_rng / 2] / ka_ref;
    if (swath_number != 11) ft *= 0.9;
    else ft *= 1.05;
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
    q.ok = (q.num_tiles >= 1 && q.start >= 0 && q.end <= q.shape && q.down >= 3) ? 1 : 0;
    *out = q;
}
void tufr_params(const double* kaT, long long p, int S, int n_r, const double* f_dc, double dc_rate, double T,
                 double prf, double bd, int swath_number, TufrParams* out, cudaStream_t st) {
    note_launch(), k_tufr_params<<<1, 32, 0, st>>>(kaT, p, S, n_r, f_dc, dc_rate, T, prf, bd, swath_number, out);
}

// linear_resample(arr, n_out)[k] of signal_processing.cpp:32-67, arr = kaT row.
__device__ __forceinline__ double lin_resample_at(const double* arr, int n_in, int n_out, int k) {
    if (n_in == n_out) return arr[k];
    if (k == n_out - 1) return arr[n_in - 1];
    const double dx_in = 1.0 / (n_in - 1);
    const double dx_out = 1.0 / (n_out - 1);
    const double x = k * dx_out;
    int i = (int)(x / dx_in);
    if (i > n_in - 2) i = n_in - 2;
    if (i < n_in - 2 && (i + 1 + 1) * dx_in <= x) ++i;   // knot x1 = (i+1) dx_in must exceed x
    if (i > 0 && (i + 1) * dx_in <= x) ++i;
    while (i > 0 && x < i * dx_in) --i;
    const double x0 = i * dx_in, x1 = (i + 1) * dx_in;
    const double y0 = arr[i], y1 = arr[i + 1];
    return y0 + ((x - x0) * (y1 - y0) / (x1 - x0));
}

template <typename R>
__global__ void k_tufr_deramp(const cpx<R>* a, long long ap, int S, cpx<R>* y, long long yp, const double* kaT,
                              long long kp, const double* f_dc, int n_r, double dc_rate, int num_tiles, double ft) {
    const int shape = num_tiles * S;
    const double start = -ft / 2, end = ft / 2;
    const double step = (end - start) / (shape - 1);
    GRID_STRIDE(i, (long long)n_r * shape) {
        const int j = (int)(i / shape), k = (int)(i % shape);
        const double ka = lin_resample_at(kaT + (long long)j * kp, S, shape, k);
        const double kt = -ka * dc_rate / (dc_rate - ka);
        const double dct = -f_dc[j] / ka;
        const double t = dct + (start + k * step);
        const double th1 = ((-kPI) * kt) * (t * t);
        const double th2 = (((2.0 * kPI) * (kt + ka)) * dct) * t;
        y[(long long)j * yp + k] = a[(long long)j * ap + (k % S)] * expi<R>(th1 + th2);
    }
}
template <typename R>
void tufr_deramp(const cpx<R>* a, long long ap, int S, cpx<R>* y, long long yp, const double* kaT, long long kp,
                 const double* f_dc, int n_r, double dc_rate, int num_tiles, double ft, cudaStream_t st) {
    note_launch(), k_tufr_deramp<R><<<grid1((long long)n_r * num_tiles * S), 256, 0, st>>>(a, ap, S, y, yp, kaT, kp, f_dc, n_r,
                                                                            dc_rate, num_tiles, ft);
}

// quadratic_resample (signal_processing.cpp:109-155) + re-ramp
// (image_formation.cpp:355-378); z already carries the 1/shape of the IFFT.
template <typename R>
__global__ void k_tufr_resample(const cpx<R>* z, long long zp, int shape, cpx<R>* out, long long op, int down,
                                const double* kaT, long long kp, int S, const double* f_dc, int n_r, double dc_rate,
                                double n_ref, double ft) {
    const double dx_in = 1.0 / (shape - 1);
    const double dx_out = 1.0 / (down - 1);
    const double ts = n_ref - ft / 2, te = n_ref + ft / 2;
    const double tstep = (te - ts) / (down - 1);
    GRID_STRIDE(idx, (long long)n_r * down) {
        const int j = (int)(idx / down), q = (int)(idx % down);
        const double x = q * dx_out;
        int i = (int)(x / dx_in);
        if (i > shape - 2) i = shape - 2;
        const int i0 = i - 1 < 0 ? 0 : i - 1;
        const int i1 = i;
        const int i2 = i + 1 > shape - 1 ? shape - 1 : i + 1;
        const double x0 = i0 * dx_in, x1 = i1 * dx_in, x2 = i2 * dx_in;
        const double L0 = (x - x1) * (x - x2) / ((x0 - x1) * (x0 - x2));
        const double L1 = (x - x0) * (x - x2) / ((x1 - x0) * (x1 - x2));
        const double L2 = (x - x0) * (x - x1) / ((x2 - x0) * (x2 - x1));
        const cpx<R>* zr = z + (long long)j * zp;
        const cpx<R> y0 = zr[i0], y1 = zr[i1], y2 = zr[i2];
        const double vr = L0 * (double)y0.x + L1 * (double)y1.x + L2 * (double)y2.x;
        const double vi = L0 * (double)y0.y + L1 * (double)y1.y + L2 * (double)y2.y;
        const double ka = lin_resample_at(kaT + (long long)j * kp, S, down, q);
        const double kt = -ka * dc_rate / (dc_rate - ka);
        const double dct = -f_dc[j] / ka;
        const double t = dct + (ts + q * tstep);
        const double th1 = (kPI * kt) * (t * t);
        const double th2 = (((2.0 * kPI) * (kt + ka)) * dct) * t;
        double s, c;
        sincos(th1 - th2, &s, &c);
        out[(long long)j * op + q] = mk((R)(vr * c - vi * s), (R)(vr * s + vi * c));
    }
}
template <typename R>
void tufr_resample(const cpx<R>* z, long long zp, int shape, cpx<R>* out, long long op, int down, const double* kaT,
                   long long kp, int S, const double* f_dc, int n_r, double dc_rate, double n_ref, double ft,
                   cudaStream_t st) {
    note_launch(), k_tufr_resample<R><<<grid1((long long)n_r * down), 256, 0, st>>>(z, zp, shape, out, op, down, kaT, kp, S, f_dc,
                                                                     n_r, dc_rate, n_ref, ft);
}

// ------------------------------------------------------------------ ECCM
// eccm(), signal_processing.cpp:914-1004.  detect: max |FFT(line)| >= det.
template <typename R>
__global__ void k_eccm_detect(const cpx<R>* X, long long p, int n, double det, int* flags) {
    __shared__ double red[256];
    const long long row = blockIdx.x;
    double mx = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const cpx<R> v = X[row * p + k];
        mx = fmax(mx, hypot((double)v.x, (double)v.y));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) flags[row] = (red[0] < det) ? 0 : 1;
}
template <typename R>
void eccm_detect(const cpx<R>* X, long long p, int n, long long rows, double det, int* flags, cudaStream_t st) {
    if (rows > 0) note_launch(), k_eccm_detect<R><<<(unsigned)rows, 256, 0, st>>>(X, p, n, det, flags);
}

// Notch: windows of 128 at stride 64 from the original line (the last one
// cut at n_r-1), FFT, zero bins whose central-difference gradient magnitude
// reaches mit, IFFT (1/128), and every sample taken from the last window
// that covers it (later windows overwrite earlier ones).
template <typename R, int WB>
__global__ void k_eccm_notch(cpx<R>* data, long long p, int n_r, const int* flags, double mit, FftDesc<R> d,
                             unsigned char* mask_out, int num_ffts) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const long long row = blockIdx.x;
    if (!flags[row]) return;
    cpx<R>* line = reinterpret_cast<cpx<R>*>(smem_raw);
    cpx<R>* win = line + n_r;
    unsigned char* zero = reinterpret_cast<unsigned char*>(win + WB * 128);
    cpx<R>* g = data + row * p;
    for (int j = threadIdx.x; j < n_r; j += blockDim.x) line[j] = g[j];
    __syncthreads();
    for (int w0 = 0; w0 < num_ffts; w0 += WB) {
        const int nw = min(WB, num_ffts - w0);
        for (int t = threadIdx.x; t < nw * 128; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const int s = (w0 + w) * 64;
            int e = s + 128;
            if (e > n_r) e = n_r - 1;
            win[w * 128 + __ldg(d.perm + q)] = (s + q < e) ? line[s + q] : mk((R)0, (R)0);
        }
        __syncthreads();
        fft_dit_batched(win, d, -1, nw);
        for (int t = threadIdx.x; t < nw * 128; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const cpx<R>* S = win + w * 128;
            cpx<R> gr;
            if (q != 0 && q != 127) gr = (S[q + 1] - S[q - 1]) * (R)0.5;
            else if (q == 0) gr = S[1] - S[0];
            else gr = S[q] - S[q - 1];
            const unsigned char z = (hypot((double)gr.x, (double)gr.y) < mit) ? 0 : 1;
            zero[t] = z;
            if (mask_out) mask_out[(row * num_ffts + w0 + w) * 128 + q] = z;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nw * 128; t += blockDim.x)
            if (zero[t]) win[t] = mk((R)0, (R)0);
        __syncthreads();
        fft_dif_batched(win, d, +1, nw);
        for (int t = threadIdx.x; t < nw * 128; t += blockDim.x) {
            const int w = t >> 7, q = t & 127;
            const int wi = w0 + w;
            const int s = wi * 64;
            int e = s + 128;
            if (e > n_r) e = n_r - 1;
            const int j = s + q;
            if (j >= e) continue;
            // owner of j: the later of the (at most two) windows covering it
            int owner = -1;
            for (int c = j / 64; c >= j / 64 - 1 && c >= 0; --c) {
                if (c >= num_ffts) continue;
                int ce = c * 64 + 128;
                if (ce > n_r) ce = n_r - 1;
                if (j < ce) { owner = c; break; }
            }
            if (owner != wi) continue;
            const cpx<R> v = win[w * 128 + __ldg(d.perm + q)] * (R)(1.0 / 128.0);
            g[j] = v;
        }
        __syncthreads();
    }
}
template <typename R>
void eccm_notch(cpx<R>* data, long long p, int n_r, long long rows, const int* flags, double mit,
                const FftDesc<R>& d128, unsigned char* mask_out, cudaStream_t st) {
    const int num_ffts = eccm_num_windows(n_r);
    constexpr int WB = sizeof(R) == 4 ? 32 : 8;
    const size_t smem = sizeof(cpx<R>) * ((size_t)n_r + WB * 128) + WB * 128;
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_eccm_notch<R, WB>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                   "eccm attr");
        attr = true;
    }
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("eccm: line too long for shared memory");
    if (rows > 0)
        note_launch(), k_eccm_notch<R, WB><<<(unsigned)rows, 256, smem, st>>>(data, p, n_r, flags, mit, d128, mask_out, num_ffts);
}

// ------------------------------------------------------------------ instantiations
#define INST(R)                                                                                                   \
    template void pad_rows<R>(const cpx<R>*, long long, int, cpx<R>*, long long, int, long long, cudaStream_t);  \
    template void mul_rows_by_vec<R>(cpx<R>*, long long, int, long long, const cpx<R>*, cudaStream_t);             \
    template void rc_crop<R>(const cpx<R>*, long long, int, cpx<R>*, long long, int, int, long long, cudaStream_t); \
    template void roll_rows<R>(const cpx<R>*, long long, cpx<R>*, long long, int, int, long long, cudaStream_t);   \
    template void scale_mul_vec<R>(cpx<R>*, long long, int, long long, const cpx<R>*, double, cudaStream_t);       \
    template void scale_rows<R>(cpx<R>*, long long, int, long long, double, cudaStream_t);                         \
    template void band_select<R>(const cpx<R>*, long long, cpx<R>*, long long, int, int, int, long long,           \
                                 cudaStream_t);                                                                  \
    template void dc_sums<R>(const cpx<R>*, long long, int, int, const cpx<R>*, cf64*, cudaStream_t);              \
    template void fufr_prep<R>(const cpx<R>*, long long, int, cpx<R>*, long long, int, int, const cpx<R>*,         \
                               long long, cudaStream_t);                                                         \
    template void src_filter<R>(cpx<R>*, long long, int, int, const RowParam*, const double*, const double*,      \
                                const double*, double, cudaStream_t);                                            \
    template void az_filter<R>(cpx<R>*, long long, int, int, const RowParam*, const double*, const double*,       \
                               const double*, const double*, const double*, int, cudaStream_t);                  \
    template void tufr_deramp<R>(const cpx<R>*, long long, int, cpx<R>*, long long, const double*, long long,      \
                                 const double*, int, double, int, double, cudaStream_t);                         \
    template void tufr_resample<R>(const cpx<R>*, long long, int, cpx<R>*, long long, int, const double*,         \
                                   long long, int, const double*, int, double, double, double, cudaStream_t);    \
    template void eccm_detect<R>(const cpx<R>*, long long, int, long long, double, int*, cudaStream_t);            \
    template void eccm_notch<R>(cpx<R>*, long long, int, long long, const int*, double, const FftDesc<R>&,        \
                                unsigned char*, cudaStream_t);
INST(float)
INST(double)
template void convert_rows<float, float>(const cpx<float>*, long long, cpx<float>*, long long, int, int, long long, cudaStream_t);
template void convert_rows<double, float>(const cpx<float>*, long long, cpx<double>*, long long, int, int, long long, cudaStream_t);
template void convert_rows<float, double>(const cpx<double>*, long long, cpx<float>*, long long, int, int, long long, cudaStream_t);
template void convert_rows<double, double>(const cpx<double>*, long long, cpx<double>*, long long, int, int, long long, cudaStream_t);

}  // namespace s1g
