// Doppler-centroid estimator input of the FP32 path: the lag-1 azimuth sums
// of doppler.cpp:4-39,98-143 formed from a compensated (double-float
// accurate) range compression.
//
// The TOPS time unfolding turns the centroid into a deramp time -f_dc/K_a,
// and the burst SLC moves by ~7e-5 (relative L2) per 1e-5 Hz of centroid
// change.  Range-compressed lines carrying FP32 rounding noise (~2e-7) shift
// the centroid by up to ~1e-5 Hz on low-coherence scenes, so the sums are
// formed from a second range compression in compensated arithmetic
// (s1g_cfft.cuh) whose result is accurate to ~1e-13, as the reference's
// FP64 range compression is.
//
// The correlation out[k] = (1/E) sum_t x~[k - h + t] conj(c[t]) (x~ the
// zero-padded line indexed modulo M, s1_decoder.cpp:459-509 with the shift h
// of the fused FP32 kernel) is evaluated by overlap-save with blocks of B
// points: block b produces the U = B - L + 1 outputs [b U, b U + U).
#include <algorithm>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <vector>

#include "s1g_dcest.h"
#include "s1g_fft_engine.h"

namespace s1g {

__global__ void __launch_bounds__(512) k_rc_dc(DcEstArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int B = a.d.n;
    cf32* H = reinterpret_cast<cf32*>(smem_raw);
    cf32* E = H + padded_len(B);
    const int line = blockIdx.x / a.nb;
    const int b = blockIdx.x - line * a.nb;
    const long long k0 = (long long)b * a.U;
    const cf32* x = a.raw + (long long)line * a.n_r;
    for (int u = threadIdx.x; u < B; u += blockDim.x) {
        long long i = (k0 - a.h + u) % a.M;
        if (i < 0) i += a.M;
        const cf32 v = i < a.n_r ? x[i] : mk(0.f, 0.f);
        const int p = pad(__ldg(a.d.perm + u));
        H[p] = v;
        E[p] = mk(0.f, 0.f);
    }
    __syncthreads();
    cfft_dit(H, E, a.d, -1);
    for (int f = threadIdx.x; f < B; f += blockDim.x) {
        const int p = pad(f);
        const float4 w = __ldg(a.H + f);
        const cc v = cc_mul(cc_make(H[p], E[p]), w.x, w.y, w.z, w.w);
        H[p] = mk(v.hx, v.hy);
        E[p] = mk(v.ex, v.ey);
    }
    __syncthreads();
    cfft_dif(H, E, a.d, +1);
    float4* y = a.rcd + (long long)line * a.n_r;
    for (int u = threadIdx.x; u < a.U; u += blockDim.x) {
        const long long k = k0 + u;
        if (k >= a.n_r) break;
        const int p = pad(__ldg(a.d.perm + u));
        const df re = two_sum(H[p].x, E[p].x);
        const df im = two_sum(H[p].y, E[p].y);
        y[k] = make_float4(re.hi, im.hi, re.lo, im.lo);
    }
}

__device__ __forceinline__ void ld_pair(const float4& v, df& re, df& im) {
    re = df_make(v.x, v.z);
    im = df_make(v.y, v.w);
}

// part[c][j] = sum over the pairs t of chunk c of rc[t][j] conj(rc[t+1][j]) g[t]
__global__ void __launch_bounds__(128) k_dc_lag1(DcEstArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n_r) return;
    const int pairs = a.n_a - 1;
    const int per = (pairs + a.nchunk - 1) / a.nchunk;
    const int t0 = blockIdx.y * per;
    const int t1 = min(t0 + per, pairs);
    df sr = df_make(0.f, 0.f), si = df_make(0.f, 0.f);
    if (t0 < t1) {
        df xr, xi;
        ld_pair(a.rcd[(long long)t0 * a.n_r + j], xr, xi);
        for (int t = t0; t < t1; ++t) {
            df yr, yi;
            ld_pair(a.rcd[(long long)(t + 1) * a.n_r + j], yr, yi);
            const df pr = df_add(df_mul(xr, yr), df_mul(xi, yi));
            const df pi_ = df_sub(df_mul(xi, yr), df_mul(xr, yi));
            const float4 g = __ldg(a.g + t);
            const df gr = df_make(g.x, g.z), gi = df_make(g.y, g.w);
            sr = df_add(sr, df_sub(df_mul(pr, gr), df_mul(pi_, gi)));
            si = df_add(si, df_add(df_mul(pr, gi), df_mul(pi_, gr)));
            xr = yr;
            xi = yi;
        }
    }
    a.part[(long long)blockIdx.y * a.n_r + j] = mk(df_to_double(sr), df_to_double(si));
}

void dc_lag1_sums(const DcEstArgs& a, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_rc_dc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes), "attr");
        attr = true;
    }
    const size_t smem = 2 * sizeof(cf32) * (size_t)padded_len(a.d.n);
    if (smem > (size_t)kSmemBytes) throw std::runtime_error("Doppler estimator: shared memory");
    const long long blocks = (long long)a.n_a * a.nb;
    if (blocks > 0x7fffffffLL) throw std::runtime_error("Doppler estimator: grid");
    note_launch(), k_rc_dc<<<(unsigned)blocks, 512, smem, st>>>(a);
    dim3 grid((a.n_r + 127) / 128, a.nchunk);
    note_launch(), k_dc_lag1<<<grid, 128, 0, st>>>(a);
}

// ------------------------------------------------------------------ host tables
CfftPlan::~CfftPlan() {
    for (void* p : owned) cudaFree(p);
}

static bool only_23(int n) {
    while (n % 2 == 0) n /= 2;
    while (n % 3 == 0) n /= 3;
    return n == 1;
}

std::shared_ptr<CfftPlan> make_cfft_plan(int n) {
    if (n < 2 || !only_23(n)) throw std::runtime_error("compensated FFT: length must be 2^a 3^b");
    auto p = std::make_shared<CfftPlan>();
    std::vector<int> rad;
    int m = n, c2 = 0, c3 = 0;
    while (m % 2 == 0) { m /= 2; ++c2; }
    while (m % 3 == 0) { m /= 3; ++c3; }
    while (c2 >= 2) { rad.push_back(4); c2 -= 2; }
    if (c2) rad.push_back(2);
    for (int i = 0; i < c3; ++i) rad.push_back(3);
    if ((int)rad.size() > kMaxStages) throw std::runtime_error("compensated FFT: too many stages");
    CfftDesc& d = p->d;
    d.n = n;
    d.nstages = (int)rad.size();
    for (size_t i = 0; i < rad.size(); ++i) d.radix[i] = (int8_t)rad[i];
    std::vector<float4> tw(n);
    for (int i = 0; i < n; ++i) {
        const double ang = 2.0 * M_PI * ((double)i / (double)n);
        const df c = df_from(std::cos(ang)), s = df_from(-std::sin(ang));
        tw[i] = make_float4(c.hi, s.hi, c.lo, s.lo);
    }
    std::vector<int> perm(n);
    for (int j = 0; j < n; ++j) {
        int jj = j, size = n, pos = 0;
        for (int st = d.nstages - 1; st >= 0; --st) {
            const int r = jj % rad[st];
            jj /= rad[st];
            size /= rad[st];
            pos += r * size;
        }
        perm[j] = pos;
    }
    void *dt = nullptr, *dp = nullptr;
    check_cuda(cudaMalloc(&dt, sizeof(float4) * n), "cfft tw");
    p->owned.push_back(dt);
    check_cuda(cudaMalloc(&dp, sizeof(int) * n), "cfft perm");
    p->owned.push_back(dp);
    check_cuda(cudaMemcpy(dt, tw.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "cfft tw up");
    check_cuda(cudaMemcpy(dp, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "cfft perm up");
    d.tw = (const float4*)dt;
    d.perm = (const int*)dp;
    return p;
}

bool choose_dc_block(int n_r, int L, int& B, int& U, int& nb) {
    double best = 0;
    B = 0;
    for (int p3 = 1; p3 <= 27; p3 *= 3) {
        for (long long b = p3; b <= 1 << 16; b *= 2) {
            if (b < 64 || b < L + 32) continue;
            if (2 * sizeof(cf32) * (size_t)padded_len((int)b) > (size_t)kSmemBytes) continue;
            const int u = (int)b - L + 1;
            const int nbl = (n_r + u - 1) / u;
            const double cost = (double)nbl * (double)b * (std::log2((double)b) + 2.0);
            if (B == 0 || cost < best * 0.999 || (cost < best * 1.001 && b < B)) {
                best = cost;
                B = (int)b;
                U = u;
                nb = nbl;
            }
        }
    }
    return B != 0;
}

}  // namespace s1g
