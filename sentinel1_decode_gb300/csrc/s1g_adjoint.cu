// Pointwise and reduction kernels of the differentiable azimuth chain
// (s1g_azimuth_adjoint / s1g_azimuth_focus; orchestration in s1g_api.cu).
// The reference has no gradients or autofocus: the chain is the
// range-Doppler azimuth processing of one range-compressed burst X[a][r],
//
//   U = X exp(-i phi_a)                       phase-error polynomial in azimuth time
//   V = FFT_az(U)                             per range bin
//   W[k] = IFFT_r(FFT_r(V[k]) exp(i beta_k f_r))          bulk RCMC, beta_k = 4 pi R_ref (1/D_k - 1)/c
//   Z[k][r] = W[k][r] exp(-i (4 pi/lambda) R_r (1 - D_k))  azimuth matched filter
//   Y = IFFT_az(Z),  L = -sum p ln p, p = |Y|^2 / sum |Y|^2
//
// and its adjoint carries G = dL/dRe + i dL/dIm back through the same
// transforms.  Phases are formed in FP64 (they reach ~10^3 rad) and reduced
// before the FP32 sine / cosine; reductions accumulate in FP64.
#include <algorithm>
#include <cmath>

#include "s1g_kernels.h"

namespace s1g {

#define ADJ_GRID_STRIDE(i, total) \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (total); i += (long long)gridDim.x * blockDim.x)

namespace {

template <typename R>
__device__ __forceinline__ cpx<R> cis_d(double ph);

template <>
__device__ __forceinline__ cpx<double> cis_d<double>(double ph) {
    double s, c;
    sincos(ph, &s, &c);
    return mk(c, s);
}

template <>
__device__ __forceinline__ cpx<float> cis_d<float>(double ph) {
    const double two_pi = 6.283185307179586476925;
    const float r = (float)(ph - two_pi * rint(ph / two_pi));
    float s, c;
    __sincosf(r, &s, &c);
    return mk(c, s);
}

template <typename R>
__device__ __forceinline__ cpx<R> cmul_(cpx<R> a, cpx<R> b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// FFT-order frequency of bin f of an n-point transform sampled at rate fs
__device__ __forceinline__ double fft_freq(int f, int n, double fs) {
    return (double)(f < (n + 1) / 2 ? f : f - n) * fs / (double)n;
}

}  // namespace

template <typename R>
__global__ void k_row_factor(cpx<R>* a, long long pitch, int cols, long long rows, const cpx<R>* __restrict__ f) {
    ADJ_GRID_STRIDE(i, rows * cols) {
        const long long r = i / cols;
        const int c = (int)(i % cols);
        a[r * pitch + c] = cmul_(a[r * pitch + c], f[r]);
    }
}

template <typename R>
__global__ void k_rcmc_phase(cpx<R>* a, int n, long long rows, const double* __restrict__ beta, double fs, int sign) {
    ADJ_GRID_STRIDE(i, rows * n) {
        const long long k = i / n;
        const int f = (int)(i % n);
        a[i] = cmul_(a[i], cis_d<R>((double)sign * beta[k] * fft_freq(f, n, fs)));
    }
}

template <typename R>
__global__ void k_az_filter(cpx<R>* a, int n_r, long long rows, const double* __restrict__ omd,
                            const double* __restrict__ slant, double c4pl, int sign) {
    ADJ_GRID_STRIDE(i, rows * n_r) {
        const long long k = i / n_r;
        const int r = (int)(i % n_r);
        a[i] = cmul_(a[i], cis_d<R>((double)sign * c4pl * slant[r] * omd[k]));
    }
}

// sums[0] += sum |y|^2, sums[1] += sum |y|^2 ln |y|^2
template <typename R>
__global__ void k_entropy_sums(const cpx<R>* __restrict__ y, long long n, double* sums) {
    double s = 0.0, t = 0.0;
    ADJ_GRID_STRIDE(i, n) {
        const double I = (double)y[i].x * y[i].x + (double)y[i].y * y[i].y;
        s += I;
        if (I > 0.0) t += I * log(I);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        t += __shfl_down_sync(0xffffffffu, t, o);
    }
    __shared__ double ws[32], wt[32];
    if ((threadIdx.x & 31) == 0) {
        ws[threadIdx.x >> 5] = s;
        wt[threadIdx.x >> 5] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            s += ws[w];
            t += wt[w];
        }
        atomicAdd(sums, s);
        atomicAdd(sums + 1, t);
    }
}

// G = 2 y dL/dI with L = -sum p ln p: dL/dI = -(ln I - ln S - H) / S,
// H = sum p ln p = T/S - ln S (S, T from k_entropy_sums)
template <typename R>
__global__ void k_entropy_grad(const cpx<R>* y, cpx<R>* g, long long n, const double* __restrict__ sums) {
    const double S = sums[0];
    const double lnS = log(S);
    const double H = sums[1] / S - lnS;
    ADJ_GRID_STRIDE(i, n) {
        const cpx<R> v = y[i];
        const double I = (double)v.x * v.x + (double)v.y * v.y;
        const double d = I > 0.0 ? -2.0 * (log(I) - lnS - H) / S : 0.0;
        g[i] = mk((R)(d * v.x), (R)(d * v.y));
    }
}

// out[row] = sum_c w_c Im(conj(a[row][c]) b[row][c]), w = 1 when colw is null
// (the value at w_c = fft_freq(c, cols, fs) when freq_fs > 0)
template <typename R>
__global__ void k_row_imdot(const cpx<R>* __restrict__ a, const cpx<R>* __restrict__ b, int cols,
                            const double* __restrict__ colw, double freq_fs, double* out) {
    const long long row = blockIdx.x;
    const cpx<R>* ar = a + row * cols;
    const cpx<R>* br = b + row * cols;
    double acc = 0.0;
    for (int c = threadIdx.x; c < cols; c += blockDim.x) {
        const double im = (double)ar[c].x * br[c].y - (double)ar[c].y * br[c].x;
        const double w = colw ? colw[c] : (freq_fs > 0.0 ? fft_freq(c, cols, freq_fs) : 1.0);
        acc += w * im;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double wa[32];
    if ((threadIdx.x & 31) == 0) wa[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) acc += wa[w];
        out[row] = acc;
    }
}

static int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 16)); }

template <typename R>
void row_factor(cpx<R>* a, long long pitch, int cols, long long rows, const cpx<R>* f, cudaStream_t st) {
    note_launch(), k_row_factor<R><<<grid_for(rows * cols), 256, 0, st>>>(a, pitch, cols, rows, f);
}
template <typename R>
void rcmc_phase(cpx<R>* a, int n, long long rows, const double* beta, double fs, int sign, cudaStream_t st) {
    note_launch(), k_rcmc_phase<R><<<grid_for(rows * n), 256, 0, st>>>(a, n, rows, beta, fs, sign);
}
template <typename R>
void az_filter(cpx<R>* a, int n_r, long long rows, const double* omd, const double* slant, double c4pl, int sign,
               cudaStream_t st) {
    note_launch(), k_az_filter<R><<<grid_for(rows * n_r), 256, 0, st>>>(a, n_r, rows, omd, slant, c4pl, sign);
}
template <typename R>
void entropy_sums(const cpx<R>* y, long long n, double* sums, cudaStream_t st) {
    check_cuda(cudaMemsetAsync(sums, 0, 2 * sizeof(double), st), "entropy reset");
    note_launch(), k_entropy_sums<R><<<grid_for(n), 256, 0, st>>>(y, n, sums);
}
template <typename R>
void entropy_grad(const cpx<R>* y, cpx<R>* g, long long n, const double* sums, cudaStream_t st) {
    note_launch(), k_entropy_grad<R><<<grid_for(n), 256, 0, st>>>(y, g, n, sums);
}
template <typename R>
void row_imdot(const cpx<R>* a, const cpx<R>* b, int cols, long long rows, const double* colw, double freq_fs,
               double* out, cudaStream_t st) {
    note_launch(), k_row_imdot<R><<<(unsigned)rows, 256, 0, st>>>(a, b, cols, colw, freq_fs, out);
}

// ------------------------------------------------------------------ TOPS chain
// The row pass factors of the TOPS chain (s1g_tops_adjoint) at azimuth row
// `row` and range bin j, with F = f_a + f_dc + offset (the offset already
// in fdc): their phase psi, d psi / dF and real scale.
//   stage 0, SRC (image_formation.cpp:422-455, k_src):
//     psi = -PI f_r^2 / K_src, K_src = 2 v^2 f_c^3 D^2 / (c R F^2)
//   stage 1, scale, RCMC phase and azimuth filter (s1_decoder.cpp:643-676,
//   image_formation.cpp:458-476, k_azf with tops):
//     scale = 1 / rscale, psi = -4 PI f_r (R / D - R) / c + 4 PI R D / lambda + 2 PI F tau
// D = sqrt(1 - lambda^2 F^2 / (4 v^2)), v the effective velocity of the row
// at range R (image_formation.cpp:406-416).
namespace {
constexpr double kTopsPI = 3.14159265358979;   // the reference's PI (structs.h)
constexpr double kTopsC = 299792458.0;
constexpr double kTopsFc = 5.405000454334350e+9;

__device__ __forceinline__ void tops_factor(const RowParam& rp, double Rj, double rf, double fa, double tc, double rs,
                                            int stage, double& psi, double& dpsi, double& scale) {
    const double lam = kTopsC / kTopsFc;
    const double num = rp.re * rp.re + rp.h * rp.h - Rj * Rj;
    const double beta = num / (2 * rp.re * rp.h);
    const double vg = rp.re * rp.v * beta / rp.h;
    const double v2 = rp.v * vg;                       // v^2
    const double D = sqrt(1 - ((lam * lam) * (fa * fa)) / (4 * v2));
    const double dD = -(lam * lam) * fa / (4 * v2 * D);
    if (stage == 0) {
        const double K = kTopsPI * (rf * rf) * kTopsC * Rj / (2.0 * v2 * (kTopsFc * kTopsFc * kTopsFc));
        psi = -K * (fa * fa) / (D * D);
        dpsi = -K * (2.0 * fa / (D * D) - 2.0 * fa * fa * dD / (D * D * D));
        scale = 1.0;
    } else {
        psi = (-4.0 * kTopsPI) * rf * ((Rj / D) - Rj) / kTopsC + (4.0 * kTopsPI) * Rj * D / lam +
              (2.0 * kTopsPI) * fa * tc;
        dpsi = 4.0 * kTopsPI * rf * Rj * dD / (kTopsC * D * D) + 4.0 * kTopsPI * Rj * dD / lam + 2.0 * kTopsPI * tc;
        scale = 1.0 / rs;
    }
}
}  // namespace

// g[row][j] *= scale exp(-i psi): the adjoint of the stage's factor
template <typename R>
__global__ void k_tops_factor_adj(cpx<R>* g, long long p, int S, int n_r, const RowParam* __restrict__ rows,
                                  TopsCols c, int stage) {
    ADJ_GRID_STRIDE(i, (long long)S * n_r) {
        const int row = (int)(i / n_r), j = (int)(i % n_r);
        double psi, dpsi, scale;
        tops_factor(rows[row], c.slant[j], c.rf[j], rows[row].fa + c.fdc[j], c.tcorr[j], c.rscale[j], stage, psi, dpsi,
                    scale);
        double sn, cs;
        sincos(psi, &sn, &cs);
        const cpx<R> v = g[(long long)row * p + j];
        const double re = (double)v.x * cs + (double)v.y * sn, im = (double)v.y * cs - (double)v.x * sn;
        g[(long long)row * p + j] = mk((R)(scale * re), (R)(scale * im));
    }
}

// out[row] = sum_j -Im(conj(G) V) d psi / dF: the derivative of the loss
// along F (so along the centroid offset) through the stage's factor, V its
// output and G the loss gradient there.
template <typename R>
__global__ void k_tops_dpsi(const cpx<R>* __restrict__ G, const cpx<R>* __restrict__ V, long long p, int n_r,
                            const RowParam* __restrict__ rows, TopsCols c, int stage, double* out) {
    const int row = blockIdx.x;
    const RowParam rp = rows[row];
    double acc = 0.0;
    for (int j = threadIdx.x; j < n_r; j += blockDim.x) {
        double psi, dpsi, scale;
        tops_factor(rp, c.slant[j], c.rf[j], rp.fa + c.fdc[j], c.tcorr[j], c.rscale[j], stage, psi, dpsi, scale);
        const cpx<R> a = G[(long long)row * p + j], b = V[(long long)row * p + j];
        acc -= dpsi * ((double)a.x * b.y - (double)a.y * b.x);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double wa[32];
    if ((threadIdx.x & 31) == 0) wa[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) acc += wa[w];
        out[row] = acc;
    }
}

// Adjoint of the band move of azimuth_frequency_ufr (bins [start, start+len)
// to the front, the rest zeroed): out[q] = in[q - start] on the band, else 0.
template <typename R>
__global__ void k_band_insert(const cpx<R>* in, long long ip, cpx<R>* out, long long op, int n, int start, int len,
                              long long rows) {
    ADJ_GRID_STRIDE(i, rows * n) {
        const long long r = i / n;
        const int q = (int)(i % n);
        out[r * op + q] = (q >= start && q < start + len) ? in[r * ip + (q - start)] : mk((R)0, (R)0);
    }
}

// Adjoint of the tiling + deramp of azimuth_frequency_ufr (k_fufr_prep:
// y[k] = X[(k mod n_a - n_a/2) mod n_a] d[k] for k < tile_len): every
// replica folded back onto its source bin, times conj(d).
template <typename R>
__global__ void k_ufr_fold(const cpx<R>* Gy, long long yp, int tile_len, const cpx<R>* d, cpx<R>* Gx, long long xp,
                           int n_a, long long rows) {
    ADJ_GRID_STRIDE(i, rows * n_a) {
        const long long r = i / n_a;
        const int q = (int)(i % n_a);
        const int k0 = (q + n_a / 2) % n_a;
        cpx<R> acc = mk((R)0, (R)0);
        for (int k = k0; k < tile_len; k += n_a) acc = acc + cmul_(Gy[r * yp + k], conj(d[k]));
        Gx[r * xp + q] = acc;
    }
}

template <typename R>
void tops_factor_adj(cpx<R>* g, long long p, int S, int n_r, const RowParam* rows, const TopsCols& c, int stage,
                     cudaStream_t st) {
    note_launch(), k_tops_factor_adj<R><<<grid_for((long long)S * n_r), 256, 0, st>>>(g, p, S, n_r, rows, c, stage);
}
template <typename R>
void tops_dpsi(const cpx<R>* G, const cpx<R>* V, long long p, int S, int n_r, const RowParam* rows, const TopsCols& c,
               int stage, double* out, cudaStream_t st) {
    note_launch(), k_tops_dpsi<R><<<(unsigned)S, 256, 0, st>>>(G, V, p, n_r, rows, c, stage, out);
}
template <typename R>
void band_insert(const cpx<R>* in, long long ip, cpx<R>* out, long long op, int n, int start, int len, long long rows,
                 cudaStream_t st) {
    note_launch(), k_band_insert<R><<<grid_for(rows * n), 256, 0, st>>>(in, ip, out, op, n, start, len, rows);
}
template <typename R>
void ufr_fold(const cpx<R>* Gy, long long yp, int tile_len, const cpx<R>* d, cpx<R>* Gx, long long xp, int n_a,
              long long rows, cudaStream_t st) {
    note_launch(), k_ufr_fold<R><<<grid_for(rows * n_a), 256, 0, st>>>(Gy, yp, tile_len, d, Gx, xp, n_a, rows);
}

#define S1G_ADJ_INST(R)                                                                                         \
    template void row_factor<R>(cpx<R>*, long long, int, long long, const cpx<R>*, cudaStream_t);              \
    template void rcmc_phase<R>(cpx<R>*, int, long long, const double*, double, int, cudaStream_t);            \
    template void az_filter<R>(cpx<R>*, int, long long, const double*, const double*, double, int, cudaStream_t); \
    template void entropy_sums<R>(const cpx<R>*, long long, double*, cudaStream_t);                            \
    template void entropy_grad<R>(const cpx<R>*, cpx<R>*, long long, const double*, cudaStream_t);             \
    template void row_imdot<R>(const cpx<R>*, const cpx<R>*, int, long long, const double*, double, double*,   \
                               cudaStream_t);                                                                   \
    template void tops_factor_adj<R>(cpx<R>*, long long, int, int, const RowParam*, const TopsCols&, int,       \
                                     cudaStream_t);                                                             \
    template void tops_dpsi<R>(const cpx<R>*, const cpx<R>*, long long, int, int, const RowParam*,              \
                               const TopsCols&, int, double*, cudaStream_t);                                    \
    template void band_insert<R>(const cpx<R>*, long long, cpx<R>*, long long, int, int, int, long long,        \
                                 cudaStream_t);                                                                 \
    template void ufr_fold<R>(const cpx<R>*, long long, int, const cpx<R>*, cpx<R>*, long long, int, long long,  \
                              cudaStream_t);
S1G_ADJ_INST(float)
S1G_ADJ_INST(double)

}  // namespace s1g
