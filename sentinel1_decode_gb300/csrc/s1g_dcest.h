// Doppler-centroid lag-1 sums from a compensated range compression
// (s1g_dcest.cu).
#pragma once

#include <memory>
#include <vector>

#include "s1g_cfft.cuh"

namespace s1g {

struct CfftPlan {
    CfftDesc d;
    std::vector<void*> owned;
    ~CfftPlan();
};

struct DcEstArgs {
    const cf32* raw;       // [n_a][n_r] decoded (and notched) echo lines
    int n_a, n_r;
    int M, h;              // circular length and output shift of the range correlation
    CfftDesc d;            // overlap-save block length B
    int U, nb;             // outputs per block, blocks per line
    const float4* H;       // B: conj(FFT_B(chirp)) * 2^-32 / (E B), float pairs {re, im, re lo, im lo}
    float4* rcd;           // [n_a][n_r] compressed lines * 2^-32, float pairs {re, im, re lo, im lo}
    const float4* g;       // n_a - 1: deramp_t conj(deramp_t+1), float pairs
    cf64* part;            // [nchunk][n_r] partial lag-1 sums
    int nchunk;
};

std::shared_ptr<CfftPlan> make_cfft_plan(int n);
// Overlap-save block B = 2^a 3^b (B >= L + 32, fits shared memory) of least
// cost for lines of n_r samples and a chirp of L samples.
bool choose_dc_block(int n_r, int L, int& B, int& U, int& nb);
void dc_lag1_sums(const DcEstArgs& a, cudaStream_t st);

// The ECCM notch of the FP32 pipelines in compensated FP32 arithmetic
// (s1g_eccm.cu): the lines with flags[row] set, read from the FP64 decoded
// samples `in`, notched (fft 128, stride 64, mitigation threshold mit) into
// the complex<float> rows of `out`; other rows of `out` are left as they are.
// d128: a 128-point compensated transform plan (make_cfft_plan(128)).
void eccm_notch_cc(const cf64* in, long long ip, cf32* out, long long op, int n_r, long long rows, const int* flags,
                   double mit, const CfftDesc& d128, cudaStream_t st);
// The ECCM line detection flags[row] = (max_k |FFT(line)_k| >= det) from the
// FP32 spectra X32 of the lines, with every line whose FP32 maximum lies
// within 1e-4 (relative) of det decided by the exact FP64 DFT of its FP64
// samples x64 at the bins that could reach det.  roots: n complex<double> of
// scratch (filled here with exp(-2 pi i m / n)).
void eccm_detect_mixed(const cf32* X32, long long xp, int n, long long rows, double det, const cf64* x64,
                       long long p64, cf64* roots, int* flags, cudaStream_t st);

}  // namespace s1g
