// Parameter blocks of the fused FP32 kernels (s1g_fast.cu).
#pragma once

#include "s1g_df.cuh"
#include "s1g_fft3.cuh"
#include "s1g_kernels.h"

namespace s1g {

// Chirp-z transform X[k] = sum_{s<nin} x[s] exp(dir 2 pi i s k / period),
// k < nout, computed as a circular convolution of length m (7-smooth,
// m >= nin + nout - 1) in shared memory (Bluestein's identity).
struct CztDev {
    Fft3Desc dm;           // length m
    const cf32* chirp;     // w[n] = exp(-i pi n^2 / period), n < max(nin, nout)
    const cf32* kern;      // FFT_m of b[n] = conj(w[n]), n in (-nin, nout), scaled by 1/m
    int nin, nout;
};

// Per-row (azimuth line) parameters of the row pass / K_a, as float pairs.
struct RowDf {
    df fa;      // azimuth frequency of the row
    df P;       // v^2 / (2 h^2)
    df A;       // re^2 + h^2   (so v_rel^2 = P (A - R^2), image_formation.cpp:406-413)
};

// Per-range-bin constants.
struct ColDf {
    df Q;            // R^2
    df k4r;          // 4 pi R / lambda
    df tau2pi;       // 2 pi * timing correction (packet.cpp:322-342)
    cf32 az0;        // exp(i (4 pi R / lambda mod 2 pi))
    float rscale;    // sqrt((R_ref / R)^3)
    float csrc;      // pi f_r^2 c R / (2 f_c^3)   (SRC phase = -csrc F^2 / (v_rel^2 D^2))
    float crcmc;     // 4 pi f_r R / c             (RCMC phase = -crcmc (1-D)/D)
    float rmig;      // 2 R f_s / c                (range migration in samples = rmig (1-D)/D)
};

struct TufrDev {       // device-side time unfolding parameters (from k_tufr_params_fast)
    TufrParams q;
};

struct FufrArgs {
    const cf32* rcT;        // [n_r][n_a]
    int n_a, n_r;
    int na_smooth;
    Fft3Desc dna;           // n_a (smooth case)
    CztDev cna;             // n_a-point DFT (otherwise)
    CztDev cf, ci;          // band CZT forward (nin=S, nout=bw) and inverse (nin=bw, nout=S)
    const cf32* dfwd;       // deramp * exp(-2 pi i s start / S), S
    const cf32* reramp;     // re-ramp / S, S
    int S, tile_len, bw;
    cf32* out;              // [n_r][S]
};
struct RowArgs {
    cf32* data;              // [S][n_r], in place
    int S, n_r, tops;
    const RowDf* rows;
    const ColDf* cols;
    const df* fdc;
    int smooth;
    Fft3Desc d;              // n_r (smooth)
    CztDev cz;               // n_r-point DFT (non-smooth)
    df lam2_4;               // lambda^2 / 4
    int post;                // 1: multiply by the scale / RCMC / azimuth-filter factor; 0: store the range IFFT
};
// Range cell migration correction by sinc interpolation (the S1G_RCMC_SINC
// option of the TOPS row pass): every range line of the range-Doppler burst
// is resampled at j + rmig_j (1 - D) / D with a Hann-windowed sinc of 2L + 1
// taps, then multiplied by the scale and azimuth-filter factor (without the
// phase RCMC).
struct RcmcArgs {
    const cf32* in;          // [S][n_r], range IFFT output of the row pass
    cf32* out;               // [S][n_r]
    int S, n_r, L;
    const RowDf* rows;
    const ColDf* cols;
    const df* fdc;
    df lam2_4;
};
void rcmc_sinc(const RcmcArgs& a, cudaStream_t st);
// Time unfolding band: the length-TS DFT of the deramped, tiled azimuth line
// y[n] is needed only on the band [start, end) (bw bins, centred on
// K0 = bw/2), and its inverse only at three consecutive integers n per
// output row.  Both ends are non-uniform FFTs on one oversampled grid of
// M >= 1.25 bw points with an exponential-of-semicircle kernel phi of width
// kNuW:
//   type 1 (band):  y[n] exp(-2 pi i n k_s / TS) (k_s = start + K0) spread
//                   onto the grid at x_n = n M / TS, forward FFT; grid bin p
//                   is Z[K0 + p] Phi(p / M) for |p| < bw / 2;
//   type 2 (rows):  the band divided by Phi a second time (so the grid bins
//                   are scaled once by the band mask / Phi^2), inverse FFT,
//                   kNuTaps-tap interpolation per output row whose weights
//                   fold in the three Lagrange coefficients, the centring
//                   phase exp(2 pi i K0 n / TS) and 1/TS.
// Phi is the kernel's Fourier transform (Gauss-Legendre quadrature); each
// end has relative error ~1e-8 in FP64, below the FP32 FFT noise.
constexpr int kNuW = 13;
constexpr int kTufrGroup = 2;   // range bins spread together (one kernel weight for both lines)
constexpr int kNuTaps = kNuW + 2;
constexpr int kNuQuad = 128;   // Gauss-Legendre nodes of the kernel's Fourier transform

// Per-burst tables of the time unfolding that do not depend on the range bin
// (k_tufr_tables, from the device-side parameters):
//   band[p], p < M       band mask / Phi(p / M)^2 on the grid (p in FFT order)
//   nu_l0[p], p < n_out  first grid point of the interpolation window
//   nu_w[j][p]           interpolation weights (complex), tap-major
//   rer[p]               {knot index (int bits), fraction, tau hi, tau lo} of the re-ramp
//   gl_x, gl_w           Gauss-Legendre nodes and weights on [-1, 1] (kNuQuad)
struct TufrTables {
    float* band;
    int* nu_l0;
    cf32* nu_w;
    float4* rer;
    const double* gl_x;
    const double* gl_w;
};

struct TufrArgs {
    const cf32* in;          // [n_r][S], row pass output transposed
    int S, n_r;
    const TufrDev* P;
    Fft3Desc dnu;            // grid FFT of both non-uniform FFTs (length M)
    const RowDf* rows;       // S knots
    const ColDf* cols;
    const df* fdc;
    const df* inv_lamR;      // 1 / (lambda R), per range bin
    df lam2_4, rate, pi_, two_pi_;
    float* KN;               // per-CTA scratch: kTufrGroup * 4 * S (pi K_t and -f_dc/K_a as float pairs)
    cf32* G;                 // per-CTA scratch: kTufrGroup * M (spread grids)
    int tmax, bwmax;
    int ychunk;              // shared-memory samples of a spreading pass (all kTufrGroup range bins)
    cf32* out;               // [n_r][n_out]
    int n_out, s0;           // cropped output rows: [s0, s0 + n_out)
    int* status;             // set to 1 if the burst falls outside the launch plan
    TufrTables tab;
};

void rc_fused(const cf32* raw, cf32* rc, int n_a, int n_r, int h, const Fft3Desc& d, const cf32* ref,
              cudaStream_t st);
void fufr_fused(const FufrArgs& a, cudaStream_t st);
// Doppler centroid polynomial from nchunk partial lag-1 sums [nchunk][n_r]
void dc_fit_fast(const cf64* part, int nchunk, const DcFitArgs& a, double* f_dc, df* f_dc_df, cudaStream_t st);
void rowpass_fused(const RowArgs& a, cudaStream_t st);
// ka0: device scratch of S doubles
void tufr_params_fast(const RowParam* rows, const double* slant, const double* f_dc, int S, int n_r, double rate,
                      double T, double prf, double bd, int swath_number, double* ka0, TufrDev* out, cudaStream_t st);
// CTAs per SM the time-unfolding kernel runs with (its grid is this times the SM count)
int tufr_ctas_per_sm(const TufrArgs& a);
void tufr_fused(const TufrArgs& a, int grid, cudaStream_t st);
// Fill a.tab for the burst whose parameters are at a.P (tables sized for a.tmax tiles).
void tufr_tables(const TufrArgs& a, cudaStream_t st);
void czt_rows(const cf32* in, long long ip, cf32* out, long long op, long long rows, const CztDev& c, int dir,
              float scale, cudaStream_t st);

}  // namespace s1g
