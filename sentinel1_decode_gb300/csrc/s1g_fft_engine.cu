// Batched row-FFT engine: plans, kernels and launchers (see s1g_fft_engine.h).
#include "s1g_fft_engine.h"
#include "s1g_tma.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace s1g {

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(); }
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool is_smooth7(long long n) {
    if (n < 1) return false;
    for (int p : {2, 3, 5, 7})
        while (n % p == 0) n /= p;
    return n == 1;
}

long long next_smooth7(long long n) {
    if (n < 1) n = 1;
    while (!is_smooth7(n)) ++n;
    return n;
}

static void radices3_for(long long n, std::vector<int>& out) {
    int c2 = 0, c3 = 0, c5 = 0, c7 = 0;
    while (n % 2 == 0) { n /= 2; ++c2; }
    while (n % 3 == 0) { n /= 3; ++c3; }
    while (n % 5 == 0) { n /= 5; ++c5; }
    while (n % 7 == 0) { n /= 7; ++c7; }
    while (c2 >= 4) { out.push_back(16); c2 -= 4; }
    if (c2 == 3) out.push_back(8);
    if (c2 == 2) out.push_back(4);
    if (c2 == 1) out.push_back(2);
    for (int i = 0; i < c5; ++i) out.push_back(5);
    for (int i = 0; i < c3; ++i) out.push_back(3);
    for (int i = 0; i < c7; ++i) out.push_back(7);
}

int fft3_passes(long long n) {
    std::vector<int> r;
    radices3_for(n, r);
    return (int)r.size();
}

long long fast_len(long long minlen, long long cap) {
    long long best = -1;
    double bc = 0;
    const long long hi = std::max(minlen, (long long)(minlen * 1.25) + 1);
    for (long long m = std::max(1LL, minlen); m <= hi; ++m) {
        if (m > cap) break;
        if (!is_smooth7(m)) continue;
        const double c = (double)m * (double)fft3_passes(m);
        if (best < 0 || c < bc) {
            best = m;
            bc = c;
        }
    }
    if (best < 0) best = next_smooth7(minlen);
    return best;
}

DeviceArena::~DeviceArena() {
    if (ptr) cudaFree(ptr);
}

void* DeviceArena::get(size_t bytes) {
    if (bytes > size) {
        if (ptr) {
            cudaDeviceSynchronize();
            cudaFree(ptr);
        }
        ptr = nullptr;
        size = 0;
        check_cuda(cudaMalloc(&ptr, bytes), "scratch cudaMalloc");
        size = bytes;
    }
    return ptr;
}

// ------------------------------------------------------------------ kernels
constexpr int kFftThreads = 512;

template <typename R>
__global__ void __launch_bounds__(kFftThreads) k_fft_smem(const cpx<R>* __restrict__ in, long long in_pitch,
                                                         cpx<R>* __restrict__ out, long long out_pitch,
                                                         FftDesc<R> d, int dir) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<R>* buf = reinterpret_cast<cpx<R>*>(smem_raw);
    const long long row = blockIdx.x;
    const cpx<R>* x = in + row * in_pitch;
    for (int j = threadIdx.x; j < d.n; j += blockDim.x) buf[__ldg(d.perm + j)] = x[j];
    __syncthreads();
    fft_dit(buf, d, dir);
    cpx<R>* y = out + row * out_pitch;
    for (int k = threadIdx.x; k < d.n; k += blockDim.x) y[k] = buf[k];
}

template <typename R>
struct BlueArgs {
    int n;
    FftDesc<R> dm;          // length m
    const cpx<R>* chirp;    // n
    const cpx<R>* kern;     // m
};

template <typename R>
__global__ void __launch_bounds__(kFftThreads) k_fft_blue(const cpx<R>* __restrict__ in, long long in_pitch,
                                                         cpx<R>* __restrict__ out, long long out_pitch,
                                                         BlueArgs<R> b, int dir) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<R>* buf = reinterpret_cast<cpx<R>*>(smem_raw);
    const long long row = blockIdx.x;
    const cpx<R>* x = in + row * in_pitch;
    const int m = b.dm.n;
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
        cpx<R> v = mk((R)0, (R)0);
        if (q < b.n) {
            cpx<R> xv = x[q];
            if (dir > 0) xv = conj(xv);
            v = xv * ldg(b.chirp + q);
        }
        buf[__ldg(b.dm.perm + q)] = v;
    }
    __syncthreads();
    fft_dit(buf, b.dm, -1);
    for (int q = threadIdx.x; q < m; q += blockDim.x) buf[q] = buf[q] * ldg(b.kern + q);
    __syncthreads();
    fft_dif(buf, b.dm, +1);
    cpx<R>* y = out + row * out_pitch;
    for (int k = threadIdx.x; k < b.n; k += blockDim.x) {
        cpx<R> v = ldg(b.chirp + k) * buf[__ldg(b.dm.perm + k)];
        y[k] = dir > 0 ? conj(v) : v;
    }
}

// 32x32 tiled transpose of a batch of matrices.
template <typename R>
__global__ void k_transpose(const cpx<R>* __restrict__ in, long long irp, long long ibp, cpx<R>* __restrict__ out,
                            long long orp, long long obp, int rows, int cols) {
    __shared__ cpx<R> tile[32][33];
    const long long b = blockIdx.z;
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const cpx<R>* src = in + b * ibp;
    cpx<R>* dst = out + b * obp;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = src[(long long)r * irp + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[(long long)c * orp + r] = tile[threadIdx.x][i];
    }
}

// four-step twiddle: data [B][n2][n1], element (j2, k1) *= w_n^(dir j2 k1)
template <typename R>
__global__ void k_twiddle4(cpx<R>* __restrict__ a, long long total, int n1, int n2, const cpx<R>* __restrict__ tw,
                           int n, int dir) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k1 = (int)(i % n1);
        const int j2 = (int)((i / n1) % n2);
        const int idx = (int)(((long long)j2 * k1) % n);
        cpx<R> w = tw[idx];
        if (dir > 0) w = conj(w);
        a[i] = a[i] * w;
    }
}

template <typename R>
__global__ void k_blue_pre(const cpx<R>* __restrict__ in, long long in_pitch, cpx<R>* __restrict__ a, int n, int m,
                           long long batch, const cpx<R>* __restrict__ chirp, int dir) {
    const long long total = batch * m;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(i % m);
        const long long b = i / m;
        cpx<R> v = mk((R)0, (R)0);
        if (q < n) {
            cpx<R> xv = in[b * in_pitch + q];
            if (dir > 0) xv = conj(xv);
            v = xv * chirp[q];
        }
        a[i] = v;
    }
}

template <typename R>
__global__ void k_mul_rows(cpx<R>* __restrict__ a, long long total, int m, const cpx<R>* __restrict__ k) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
        a[i] = a[i] * k[i % m];
}

template <typename R>
__global__ void k_blue_post(const cpx<R>* __restrict__ a, int m, cpx<R>* __restrict__ out, long long out_pitch, int n,
                            long long batch, const cpx<R>* __restrict__ chirp, int dir) {
    const long long total = batch * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i % n);
        const long long b = i / n;
        cpx<R> v = chirp[k] * a[b * m + k];
        out[b * out_pitch + k] = dir > 0 ? conj(v) : v;
    }
}

template <typename R>
__global__ void k_cvt64(const cpx<double>* __restrict__ in, cpx<R>* __restrict__ out, long long n, double scale) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = mk((R)(in[i].x * scale), (R)(in[i].y * scale));
}

static int grid_for(long long total, int threads = 256) {
    long long g = (total + threads - 1) / threads;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (int)g;
}

// ------------------------------------------------------------------ plans
template <typename R>
FftPlan<R>::~FftPlan() {
    for (void* p : owned) cudaFree(p);
}

static void radices_for(int n, std::vector<int>& out) {
    int c2 = 0, c3 = 0, c5 = 0, c7 = 0;
    while (n % 2 == 0) { n /= 2; ++c2; }
    while (n % 3 == 0) { n /= 3; ++c3; }
    while (n % 5 == 0) { n /= 5; ++c5; }
    while (n % 7 == 0) { n /= 7; ++c7; }
    while (c2 >= 3) { out.push_back(8); c2 -= 3; }
    if (c2 == 2) out.push_back(4);
    if (c2 == 1) out.push_back(2);
    for (int i = 0; i < c5; ++i) out.push_back(5);
    for (int i = 0; i < c3; ++i) out.push_back(3);
    for (int i = 0; i < c7; ++i) out.push_back(7);
}

template <typename R>
static void* upload(FftPlan<R>& p, const void* host, size_t bytes) {
    void* d = nullptr;
    check_cuda(cudaMalloc(&d, bytes), "plan cudaMalloc");
    check_cuda(cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice), "plan upload");
    p.owned.push_back(d);
    return d;
}

// exp(-2 pi i num/den) in FP64 with the argument reduced exactly first.
static inline void unit_root(long long num, long long den, double& c, double& s) {
    num %= den;
    if (num < 0) num += den;
    const double a = 2.0 * M_PI * ((double)num / (double)den);
    c = std::cos(a);
    s = -std::sin(a);
}

template <typename R>
static void fill_desc(FftPlan<R>& p, FftDesc<R>& d, int n) {
    std::vector<int> rad;
    radices_for(n, rad);
    if ((int)rad.size() > kMaxStages) throw std::runtime_error("fft: too many stages");
    d.n = n;
    d.nstages = (int)rad.size();
    for (size_t i = 0; i < rad.size(); ++i) d.radix[i] = (int8_t)rad[i];
    std::vector<cpx<R>> tw(n);
    for (int i = 0; i < n; ++i) {
        double c, s;
        unit_root(i, n, c, s);
        tw[i] = mk((R)c, (R)s);
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
    d.tw = (const cpx<R>*)upload(p, tw.data(), sizeof(cpx<R>) * n);
    d.perm = (const int*)upload(p, perm.data(), sizeof(int) * n);
}

template <typename R>
static void set_smem_attr() {
    static bool done = false;
    if (!done) {
        check_cuda(cudaFuncSetAttribute(k_fft_smem<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                   "smem attr");
        check_cuda(cudaFuncSetAttribute(k_fft_blue<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                   "smem attr");
        done = true;
    }
}

static void split_four(int n, int cap, int& n1, int& n2) {
    int best = -1;
    for (int a = 2; a <= cap && a < n; ++a) {
        if (n % a) continue;
        const int b = n / a;
        if (b > cap) continue;
        if (best < 0 || std::abs(a - b) < std::abs(best - n / best)) best = a;
    }
    if (best < 0) throw std::runtime_error("fft: no four-step split for n=" + std::to_string(n));
    n1 = best;
    n2 = n / best;
}

FftEngine::FftEngine(cudaStream_t s) : stream(s) {
    set_smem_attr<float>();
    set_smem_attr<double>();
}
FftEngine::~FftEngine() = default;

template <typename R>
static std::map<int, std::shared_ptr<FftPlan<R>>>& plan_map(FftEngine& e);
template <>
std::map<int, std::shared_ptr<FftPlan<float>>>& plan_map<float>(FftEngine& e) { return e.plans32; }
template <>
std::map<int, std::shared_ptr<FftPlan<double>>>& plan_map<double>(FftEngine& e) { return e.plans64; }

template <typename R>
std::shared_ptr<FftPlan<R>> FftEngine::plan(int n) {
    auto& mp = plan_map<R>(*this);
    auto it = mp.find(n);
    if (it != mp.end()) return it->second;
    auto p = std::make_shared<FftPlan<R>>();
    p->n = n;
    const int cap = smem_capacity<R>();
    if (is_smooth7(n) && n <= cap) {
        p->kind = FFT_SMEM;
        fill_desc(*p, p->d, n);
    } else if (is_smooth7(n)) {
        p->kind = FFT_FOUR;
        split_four(n, cap, p->n1, p->n2);
        p->p1 = plan<R>(p->n1);
        p->p2 = plan<R>(p->n2);
        std::vector<cpx<R>> tw(n);
        for (int i = 0; i < n; ++i) {
            double c, s;
            unit_root(i, n, c, s);
            tw[i] = mk((R)c, (R)s);
        }
        p->tw4 = (cpx<R>*)upload(*p, tw.data(), sizeof(cpx<R>) * n);
    } else {
        const long long m = next_smooth7(2LL * n - 1);
        p->m = (int)m;
        if (m <= cap) {
            p->kind = FFT_BLUE;
            fill_desc(*p, p->d, (int)m);
        } else {
            p->kind = FFT_BLUE4;
            p->pm = plan<R>((int)m);
        }
        // chirp w[k] = exp(-i pi k^2/n) = exp(-2 pi i (k^2 mod 2n)/(2n))
        std::vector<cpx<R>> w(n);
        std::vector<cpx<double>> b((size_t)m, mk(0.0, 0.0));
        for (int k = 0; k < n; ++k) {
            double c, s;
            unit_root((long long)k * k % (2LL * n), 2LL * n, c, s);
            w[k] = mk((R)c, (R)s);
            b[k] = mk(c, -s);  // conj(w)
            if (k > 0) b[m - k] = mk(c, -s);
        }
        p->chirp = (cpx<R>*)upload(*p, w.data(), sizeof(cpx<R>) * n);
        // kernel spectrum computed in FP64 on the device, scaled by 1/m
        auto p64 = plan<double>((int)m);
        cpx<double>* d64 = nullptr;
        check_cuda(cudaMalloc(&d64, sizeof(cpx<double>) * m), "blue tmp");
        check_cuda(cudaMemcpy(d64, b.data(), sizeof(cpx<double>) * m, cudaMemcpyHostToDevice), "blue up");
        rows<double>(*p64, d64, m, d64, m, 1, -1);
        cpx<R>* kd = nullptr;
        check_cuda(cudaMalloc(&kd, sizeof(cpx<R>) * m), "blue kern");
        p->owned.push_back(kd);
        note_launch(), k_cvt64<R><<<grid_for(m), 256, 0, stream>>>(d64, kd, m, 1.0 / (double)m);
        check_cuda(cudaStreamSynchronize(stream), "blue kern sync");
        cudaFree(d64);
        p->kern = kd;
    }
    mp[n] = p;
    return p;
}

Fft3Plan::~Fft3Plan() {
    for (void* p : owned) cudaFree(p);
}

std::vector<int> default_radices3(long long n) {
    std::vector<int> r;
    radices3_for(n, r);
    return r;
}

std::shared_ptr<Fft3Plan> build_plan3(int n, const std::vector<int>& rad) {
    if (!is_smooth7(n) || n > smem_capacity<float>()) throw std::runtime_error("desc3: length not smooth/small");
    if ((int)rad.size() > kMaxStages) throw std::runtime_error("desc3: too many stages");
    long long prod = 1;
    for (int r : rad) prod *= r;
    if (prod != n) throw std::runtime_error("desc3: radices do not multiply to the length");
    auto p = std::make_shared<Fft3Plan>();
    Fft3Desc& d = p->d;
    d.n = n;
    d.nstages = (int)rad.size();
    for (size_t i = 0; i < rad.size(); ++i) d.radix[i] = (int8_t)rad[i];
    const int nhi = fft3_nhi(n);
    std::vector<cf32> tw(fft3_tw_len(n));
    for (int q = 0; q < nhi; ++q) {
        double c, s;
        unit_root(64LL * q, n, c, s);
        tw[q] = mk((float)c, (float)s);
    }
    for (int q = 0; q < 64; ++q) {
        double c, s;
        unit_root(q, n, c, s);
        tw[nhi + q] = mk((float)c, (float)s);
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
    check_cuda(cudaMalloc(&dt, sizeof(cf32) * tw.size()), "desc3 tw");
    p->owned.push_back(dt);
    check_cuda(cudaMalloc(&dp, sizeof(int) * n), "desc3 perm");
    p->owned.push_back(dp);
    check_cuda(cudaMemcpy(dt, tw.data(), sizeof(cf32) * tw.size(), cudaMemcpyHostToDevice), "desc3 tw up");
    check_cuda(cudaMemcpy(dp, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "desc3 perm up");
    d.tw = (const cf32*)dt;
    d.perm = (const int*)dp;
    return p;
}

Fft3Desc FftEngine::desc3(int n) {
    auto it = plans3.find(n);
    if (it != plans3.end()) return it->second->d;
    const std::vector<int> rad = tuned_radices(n, stream);
    auto p = build_plan3(n, rad);
    plans3[n] = p;
    return p->d;
}

long long FftEngine::tuned_len(long long minlen, long long cap) { return tuned_length(minlen, cap, stream); }

template <typename R>
FftDesc<R> FftEngine::smem_desc(int n) {
    auto p = plan<R>(n);
    if (p->kind != FFT_SMEM) throw std::runtime_error("smem_desc: length not smooth/small: " + std::to_string(n));
    return p->d;
}

template <typename R>
void transpose_batched(const cpx<R>* in, long long irp, long long ibp, cpx<R>* out, long long orp, long long obp,
                       int rows, int cols, long long batch, cudaStream_t s) {
    if constexpr (sizeof(R) == 4) {
        // single complex<float> matrices go through the TMA-staged corner turn
        if (batch == 1 && transpose_tma(in, irp, out, orp, rows, cols, s)) return;
    }
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, (unsigned)batch);
    note_launch(), k_transpose<R><<<grid, dim3(32, 8), 0, s>>>(in, irp, ibp, out, orp, obp, rows, cols);
}

template <typename R>
void FftEngine::rows(const FftPlan<R>& p, const cpx<R>* in, long long in_pitch, cpx<R>* out, long long out_pitch,
                     long long batch, int dir) {
    if (batch <= 0) return;
    const int n = p.n;
    switch (p.kind) {
        case FFT_SMEM: {
            for (long long b0 = 0; b0 < batch; b0 += 65535LL * 16) {
                const long long nb = std::min(batch - b0, 65535LL * 16);
                note_launch(), k_fft_smem<R><<<(unsigned)nb, kFftThreads, sizeof(cpx<R>) * n, stream>>>(
                    in + b0 * in_pitch, in_pitch, out + b0 * out_pitch, out_pitch, p.d, dir);
            }
            break;
        }
        case FFT_BLUE: {
            BlueArgs<R> a{n, p.d, p.chirp, p.kern};
            for (long long b0 = 0; b0 < batch; b0 += 65535LL * 16) {
                const long long nb = std::min(batch - b0, 65535LL * 16);
                note_launch(), k_fft_blue<R><<<(unsigned)nb, kFftThreads, sizeof(cpx<R>) * p.m, stream>>>(
                    in + b0 * in_pitch, in_pitch, out + b0 * out_pitch, out_pitch, a, dir);
            }
            break;
        }
        case FFT_FOUR: {
            const int n1 = p.n1, n2 = p.n2;
            const long long limit = (256LL << 20) / (long long)sizeof(cpx<R>);
            const long long chunk = std::max(1LL, std::min(batch, limit / n));
            cpx<R>* A = (cpx<R>*)scratch_a.get(sizeof(cpx<R>) * chunk * n);
            cpx<R>* B = (cpx<R>*)scratch_b.get(sizeof(cpx<R>) * chunk * n);
            for (long long b0 = 0; b0 < batch; b0 += chunk) {
                const long long nb = std::min(chunk, batch - b0);
                // [nb][n1][n2] -> A [nb][n2][n1]
                transpose_batched<R>(in + b0 * in_pitch, n2, in_pitch, A, n1, n, n1, n2, nb, stream);
                rows<R>(*p.p1, A, n1, A, n1, nb * n2, dir);
                note_launch(), k_twiddle4<R><<<grid_for(nb * n), 256, 0, stream>>>(A, nb * n, n1, n2, p.tw4, n, dir);
                // A [nb][n2][n1] -> B [nb][n1][n2]
                transpose_batched<R>(A, n1, n, B, n2, n, n2, n1, nb, stream);
                rows<R>(*p.p2, B, n2, B, n2, nb * n1, dir);
                // B [nb][n1(k1)][n2(k2)] -> out [nb][n2][n1]: index k1 + n1 k2
                transpose_batched<R>(B, n2, n, out + b0 * out_pitch, n1, out_pitch, n1, n2, nb, stream);
            }
            break;
        }
        case FFT_BLUE4: {
            const int m = p.m;
            const long long limit = (256LL << 20) / (long long)sizeof(cpx<R>);
            const long long chunk = std::max(1LL, std::min(batch, limit / m));
            // this level's buffer must not alias the four-step scratch (a, b)
            cpx<R>* A = (cpx<R>*)scratch_c.get(sizeof(cpx<R>) * chunk * m);
            for (long long b0 = 0; b0 < batch; b0 += chunk) {
                const long long nb = std::min(chunk, batch - b0);
                note_launch(), k_blue_pre<R><<<grid_for(nb * m), 256, 0, stream>>>(in + b0 * in_pitch, in_pitch, A, n, m, nb,
                                                                    p.chirp, dir);
                rows<R>(*p.pm, A, m, A, m, nb, -1);
                note_launch(), k_mul_rows<R><<<grid_for(nb * m), 256, 0, stream>>>(A, nb * m, m, p.kern);
                rows<R>(*p.pm, A, m, A, m, nb, +1);
                note_launch(), k_blue_post<R><<<grid_for(nb * n), 256, 0, stream>>>(A, m, out + b0 * out_pitch, out_pitch, n, nb,
                                                                     p.chirp, dir);
            }
            break;
        }
    }
    check_cuda(cudaGetLastError(), "fft launch");
}

template std::shared_ptr<FftPlan<float>> FftEngine::plan<float>(int);
template std::shared_ptr<FftPlan<double>> FftEngine::plan<double>(int);
template void FftEngine::rows<float>(const FftPlan<float>&, const cpx<float>*, long long, cpx<float>*, long long,
                                     long long, int);
template void FftEngine::rows<double>(const FftPlan<double>&, const cpx<double>*, long long, cpx<double>*, long long,
                                      long long, int);
template FftDesc<float> FftEngine::smem_desc<float>(int);
template FftDesc<double> FftEngine::smem_desc<double>(int);
template void transpose_batched<float>(const cpx<float>*, long long, long long, cpx<float>*, long long, long long,
                                       int, int, long long, cudaStream_t);
template void transpose_batched<double>(const cpx<double>*, long long, long long, cpx<double>*, long long,
                                        long long, int, int, long long, cudaStream_t);
template struct FftPlan<float>;
template struct FftPlan<double>;

}  // namespace s1g
