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

#define S1G_ADJ_INST(R)                                                                                         \
    template void row_factor<R>(cpx<R>*, long long, int, long long, const cpx<R>*, cudaStream_t);              \
    template void rcmc_phase<R>(cpx<R>*, int, long long, const double*, double, int, cudaStream_t);            \
    template void az_filter<R>(cpx<R>*, int, long long, const double*, const double*, double, int, cudaStream_t); \
    template void entropy_sums<R>(const cpx<R>*, long long, double*, cudaStream_t);                            \
    template void entropy_grad<R>(const cpx<R>*, cpx<R>*, long long, const double*, cudaStream_t);             \
    template void row_imdot<R>(const cpx<R>*, const cpx<R>*, int, long long, const double*, double, double*,   \
                               cudaStream_t);
S1G_ADJ_INST(float)
S1G_ADJ_INST(double)

}  // namespace s1g
