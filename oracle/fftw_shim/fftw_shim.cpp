// FP64 discrete Fourier transform behind the FFTW3 API used by the reference.
// TEST INFRASTRUCTURE ONLY (oracle build of the reference sources).
//
// Restates the DFT definition that FFTW computes (FFTW3 documentation,
// "What FFTW Really Computes"):
//     Y[k] = sum_{j<n} X[j] * exp(sign * 2*pi*i*j*k/n),  unnormalised.
// Algorithm: recursive mixed-radix Cooley-Tukey (decimation in time) over the
// prime factorisation of n; lengths whose largest prime factor exceeds 61 are
// computed with Bluestein's chirp-z identity on a power-of-two convolution.
// Twiddle tables are cached per (n, sign); fftw_execute is re-entrant, since
// the reference executes plans concurrently inside OpenMP loops.
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

namespace {

using cd = std::complex<double>;

struct Engine {
    int n = 0;
    int sign = -1;
    std::vector<int> factors;        // prime factors (4 first when possible)
    std::vector<cd> tw;              // tw[k] = exp(sign*2*pi*i*k/n)
    bool bluestein = false;
    int m = 0;                       // Bluestein convolution length (power of two)
    std::vector<cd> chirp;           // exp(sign*pi*i*k^2/n), k < n
    std::vector<cd> kernel_fft;      // FFT_m of conj-chirp kernel
    std::shared_ptr<Engine> fwd_m, inv_m;
};

std::mutex g_cache_mutex;
std::map<std::pair<int, int>, std::shared_ptr<Engine>> g_cache;

std::shared_ptr<Engine> get_engine(int n, int sign);

// exp(sign * 2*pi*i * num/den) with the argument reduced exactly first.
cd unit_root(long long num, long long den, int sign) {
    num %= den;
    if (num < 0) num += den;
    // reduce to the first octant-ish by symmetry for accuracy: use long double
    long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)num / (long double)den;
    return cd((double)cosl(a), (double)(sign * sinl(a)));
}

void factorize(int n, std::vector<int>& f) {
    while (n % 4 == 0) { f.push_back(4); n /= 4; }
    while (n % 2 == 0) { f.push_back(2); n /= 2; }
    for (int p = 3; (long long)p * p <= n; p += 2)
        while (n % p == 0) { f.push_back(p); n /= p; }
    if (n > 1) f.push_back(n);
}

// out[k*os] = sum_j in[j*is] w^{jk} for a length-len sub-transform.  tws is
// the twiddle stride (N/len) into the full table.
void rec(const Engine& e, const cd* in, ptrdiff_t is, cd* out, int len, size_t fi, int tws) {
    if (len == 1) { out[0] = in[0]; return; }
    const int p = e.factors[fi];
    const int mlen = len / p;
    for (int r = 0; r < p; ++r)
        rec(e, in + r * is, is * p, out + (ptrdiff_t)r * mlen, mlen, fi + 1, tws * p);
    const int N = e.n;
    std::vector<cd> t(p), y(p);
    for (int k = 0; k < mlen; ++k) {
        for (int r = 0; r < p; ++r) {
            long long idx = (long long)r * k * tws % N;
            t[r] = out[(ptrdiff_t)r * mlen + k] * e.tw[idx];
        }
        for (int s = 0; s < p; ++s) {
            cd acc = 0.0;
            for (int r = 0; r < p; ++r) {
                long long idx = (long long)((r * s) % p) * (N / p);
                acc += t[r] * e.tw[idx];
            }
            y[s] = acc;
        }
        for (int s = 0; s < p; ++s) out[(ptrdiff_t)s * mlen + k] = y[s];
    }
}

void run(const Engine& e, const cd* in, cd* out) {
    const int n = e.n;
    if (!e.bluestein) {
        std::vector<cd> src(in, in + n);
        rec(e, src.data(), 1, out, n, 0, 1);
        return;
    }
    // Bluestein: X[k] = c[k] * sum_j (x[j] c[j]) conj(c[k-j]),  c[k] = exp(sign*pi*i*k^2/n)
    const int m = e.m;
    std::vector<cd> a(m, 0.0), b(m);
    for (int j = 0; j < n; ++j) a[j] = in[j] * e.chirp[j];
    run(*e.fwd_m, a.data(), b.data());
    for (int k = 0; k < m; ++k) b[k] *= e.kernel_fft[k];
    run(*e.inv_m, b.data(), a.data());
    for (int k = 0; k < n; ++k) out[k] = a[k] * e.chirp[k] / (double)m;
}

std::shared_ptr<Engine> build_engine(int n, int sign) {
    auto e = std::make_shared<Engine>();
    e->n = n;
    e->sign = sign;
    std::vector<int> f;
    factorize(n, f);
    int maxp = 1;
    for (int p : f) maxp = std::max(maxp, p);
    if (maxp > 61) {
        e->bluestein = true;
        int m = 1;
        while (m < 2 * n - 1) m <<= 1;
        e->m = m;
        e->chirp.resize(n);
        for (int k = 0; k < n; ++k) {
            long long k2 = (long long)k * k % (2LL * n);
            e->chirp[k] = unit_root(k2, 2LL * n, sign);  // exp(sign*pi*i*k^2/n)
        }
        e->fwd_m = get_engine(m, -1);
        e->inv_m = get_engine(m, +1);
        std::vector<cd> kern(m, 0.0);
        for (int k = 0; k < n; ++k) kern[k] = std::conj(e->chirp[k]);
        for (int k = 1; k < n; ++k) kern[m - k] = std::conj(e->chirp[k]);
        e->kernel_fft.resize(m);
        run(*e->fwd_m, kern.data(), e->kernel_fft.data());
    } else {
        e->factors = f;
        e->tw.resize(n);
        for (int k = 0; k < n; ++k) e->tw[k] = unit_root(k, n, sign);
    }
    return e;
}

std::shared_ptr<Engine> get_engine(int n, int sign) {
    {
        std::lock_guard<std::mutex> lk(g_cache_mutex);
        auto it = g_cache.find({n, sign});
        if (it != g_cache.end()) return it->second;
    }
    auto e = build_engine(n, sign);
    std::lock_guard<std::mutex> lk(g_cache_mutex);
    g_cache[{n, sign}] = e;
    return e;
}

}  // namespace

struct fftw_plan_s {
    int rank;
    int n0, n1;
    cd* in;
    cd* out;
    std::shared_ptr<Engine> e0, e1;
};

extern "C" fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    auto* p = new fftw_plan_s;
    p->rank = 1;
    p->n0 = n;
    p->n1 = 1;
    p->in = reinterpret_cast<cd*>(in);
    p->out = reinterpret_cast<cd*>(out);
    p->e0 = get_engine(n, sign);
    return p;
}

extern "C" fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    auto* p = new fftw_plan_s;
    p->rank = 2;
    p->n0 = n0;
    p->n1 = n1;
    p->in = reinterpret_cast<cd*>(in);
    p->out = reinterpret_cast<cd*>(out);
    p->e0 = get_engine(n0, sign);
    p->e1 = get_engine(n1, sign);
    return p;
}

extern "C" void fftw_execute(const fftw_plan p) {
    if (p->rank == 1) {
        run(*p->e0, p->in, p->out);
        return;
    }
    const int n0 = p->n0, n1 = p->n1;
    std::vector<cd> tmp(p->in, p->in + (size_t)n0 * n1);
    for (int r = 0; r < n0; ++r) run(*p->e1, tmp.data() + (size_t)r * n1, tmp.data() + (size_t)r * n1);
    std::vector<cd> col(n0), colo(n0);
    for (int c = 0; c < n1; ++c) {
        for (int r = 0; r < n0; ++r) col[r] = tmp[(size_t)r * n1 + c];
        run(*p->e0, col.data(), colo.data());
        for (int r = 0; r < n0; ++r) p->out[(size_t)r * n1 + c] = colo[r];
    }
}

extern "C" void fftw_destroy_plan(fftw_plan p) { delete p; }
