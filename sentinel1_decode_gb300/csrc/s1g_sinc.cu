// Hann-windowed sinc interpolation of complex lines at fractional positions
// (sinc_interpolate, signal_processing.cpp:228-257):
//
//   out[r][k] = sum over idx = floor(t) - L .. floor(t) + L, 0 <= idx < n, of
//               in[r][idx] * sinc(t - idx) * hann(t - idx),  t = t[r][k],
//   sinc(x) = sin(PI x) / (PI x) (1 at x = 0),  hann(x) = 0.5 (1 + cos(PI x / L)).
//
// The raised cosine is not cut at |x| = L, so all 2L + 1 taps count, as in
// the reference.  A warp forms 32 consecutive outputs of one line.  When the
// taps of its 32 positions lie in a window of 64 samples (positions that
// advance about one sample per output, as a range-migration shift does), each
// lane loads two samples of the window once and every tap is fetched from the
// owning lane by warp shuffles; otherwise (scattered positions) the taps are
// read from global memory directly.  Both paths give the same sums in the
// same order.
//
// Used by the RCMC option of the row pass (S1G_RCMC_SINC) and exposed as a
// general resampler (s1g_sinc_interpolate).
#include <climits>
#include <cmath>

#include "s1g_kernels.h"
#include "s1g_sinc.cuh"
#include "s1g_sinc.h"

namespace s1g {

template <typename R>
__global__ void __launch_bounds__(256) k_sinc_interp(SincArgs<R> a) {
    const int lane = threadIdx.x & 31;
    const int wpr = (a.m + 31) / 32;   // warps per line
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (long long)a.rows * wpr) return;   // whole warps leave together
    const int r = (int)(gw / wpr);
    const int k = (int)(gw % wpr) * 32 + lane;
    const bool act = k < a.m;
    const cpx<R>* line = a.in + (long long)r * a.in_pitch;
    const double t = act ? a.t[(long long)r * a.t_pitch + k] : 0.0;
    const cpx<R> acc = sinc_warp<R>(line, a.n, t, a.L, act);
    if (act) a.out[(long long)r * a.out_pitch + k] = acc;
}

template <typename R>
void sinc_interp(const SincArgs<R>& a, cudaStream_t st) {
    if (a.rows <= 0 || a.m <= 0) return;
    const long long warps = (long long)a.rows * ((a.m + 31) / 32);
    const long long blocks = (warps * 32 + 255) / 256;
    note_launch(), k_sinc_interp<R><<<(unsigned)blocks, 256, 0, st>>>(a);
}

template void sinc_interp<float>(const SincArgs<float>&, cudaStream_t);
template void sinc_interp<double>(const SincArgs<double>&, cudaStream_t);

}  // namespace s1g

using namespace s1g;

extern "C" {

int s1g_sinc_interpolate(const void* d_in, int64_t rows, int64_t n, int64_t in_pitch, const double* d_t, int64_t m,
                         int64_t t_pitch, int half_width, void* d_out, int64_t out_pitch, int elem_type,
                         void* stream) {
    if (!d_in || !d_t || !d_out || rows < 0 || n < 0 || m < 0 || half_width < 1 || half_width > 16)
        return S1G_E_INVALID_ARGUMENT;
    if (in_pitch < n || out_pitch < m || t_pitch < 0 || (t_pitch > 0 && t_pitch < m)) return S1G_E_INVALID_ARGUMENT;
    if (rows > INT_MAX || n > INT_MAX / 2 || m > INT_MAX / 2) return S1G_E_INVALID_ARGUMENT;
    if ((rows * ((m + 31) / 32) * 32 + 255) / 256 > INT_MAX) return S1G_E_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (elem_type == S1G_CF32) {
        SincArgs<float> a{(const cf32*)d_in, in_pitch, (int)n, d_t, t_pitch, (int)m, half_width, (cf32*)d_out,
                          out_pitch, (int)rows};
        sinc_interp<float>(a, st);
    } else if (elem_type == S1G_CF64) {
        SincArgs<double> a{(const cf64*)d_in, in_pitch, (int)n, d_t, t_pitch, (int)m, half_width, (cf64*)d_out,
                           out_pitch, (int)rows};
        sinc_interp<double>(a, st);
    } else {
        return S1G_E_INVALID_ARGUMENT;
    }
    return cudaGetLastError() == cudaSuccess ? S1G_OK : S1G_E_CUDA;
}

}  // extern "C"
