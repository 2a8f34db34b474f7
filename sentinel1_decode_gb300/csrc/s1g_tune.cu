// Autotuner of the radix-16 shared-memory FFT core (s1g_fft3.cuh): for each
// transform length the fused kernels need, it times candidate radix orders
// (the stage sequence of the in-place DIT / DIF passes) and, where the
// length is free (chirp-z / Bluestein convolutions, zero-padded range lines,
// the non-uniform FFT grid), candidate 7-smooth lengths, on this GPU with
// the kernels' own launch shape (two 512-thread CTAs per SM when the buffer
// fits, else one 1024-thread CTA), and keeps the fastest.
//
// A measurement is a launch of one CTA slot per SM slot, each running a
// forward DIT and an inverse DIF transform twice on its shared-memory
// buffer; the minimum of three timed launches after one warm-up counts.
// Results persist in a text file so every process on a machine makes the
// same choices (the FP32 results depend on them at the rounding level):
//   R <n> <r1> <r2> ...        radix order of length n
//   L <minlen> <cap> <M>       length chosen for a request
// S1G_AUTOTUNE=0 turns tuning off (fast_len's length x passes model and the
// default radix order); S1G_FFT_TUNE_FILE names the file (default
// fft_tune.txt in the directory of this library).
#include <dlfcn.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <set>
#include <sstream>

#include "s1g_fft_engine.h"

namespace s1g {

template <int NT>
__global__ void __launch_bounds__(NT, NT == 512 ? 2 : 1) k_fft_tune(Fft3Desc d, int reps, float* sink) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cf32* tw = reinterpret_cast<cf32*>(smem_raw);
    cf32* buf = tw + fft3_tw_len(d.n);
    fft3_stage_tw(tw, d);
    for (int i = threadIdx.x; i < d.n; i += blockDim.x) buf[pad(i)] = mk((float)((i * 7 + blockIdx.x) & 15), 1.0f);
    __syncthreads();
    for (int r = 0; r < reps; ++r) {
        fft3_dit(buf, d, -1, tw);
        fft3_dif(buf, d, +1, tw);
    }
    if (threadIdx.x == 0) sink[blockIdx.x] = buf[0].x;
}

namespace {

struct Tuner {
    std::mutex mu;
    bool on = true;
    std::string path;
    std::map<int, std::vector<int>> rad;
    std::map<std::pair<long long, long long>, long long> len;
    int sms = 0;
    float* sink = nullptr;
    bool attr = false;

    Tuner() {
        const char* e = std::getenv("S1G_AUTOTUNE");
        on = !(e && std::string(e) == "0");
        const char* f = std::getenv("S1G_FFT_TUNE_FILE");
        if (f && *f) {
            path = f;
        } else {
            Dl_info info;
            if (dladdr(reinterpret_cast<void*>(&tuning_report), &info) && info.dli_fname) {
                std::string so = info.dli_fname;
                const size_t k = so.rfind('/');
                path = (k == std::string::npos ? std::string(".") : so.substr(0, k)) + "/fft_tune.txt";
            }
        }
    }

    // (re)read the file: another process may have tuned lengths since
    void load() {
        if (path.empty()) return;
        std::ifstream in(path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream is(line);
            std::string tag;
            is >> tag;
            if (tag == "R") {
                int n = 0, r = 0;
                std::vector<int> v;
                is >> n;
                long long prod = 1;
                while (is >> r) {
                    v.push_back(r);
                    prod *= r;
                }
                if (n > 0 && prod == n && !v.empty() && !rad.count(n)) rad[n] = v;
            } else if (tag == "L") {
                long long a = 0, c = 0, m = 0;
                if ((is >> a >> c >> m) && m >= a && m <= c && is_smooth7(m) && !len.count({a, c})) len[{a, c}] = m;
            }
        }
    }

    void save() {
        if (path.empty()) return;
        const std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
        {
            std::ofstream out(tmp);
            if (!out) return;
            for (const auto& kv : rad) {
                out << "R " << kv.first;
                for (int r : kv.second) out << " " << r;
                out << "\n";
            }
            for (const auto& kv : len) out << "L " << kv.first.first << " " << kv.first.second << " " << kv.second << "\n";
        }
        std::rename(tmp.c_str(), path.c_str());
    }

    static bool capturing(cudaStream_t st) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
    }

    // time of one launch (microseconds) of the forward + inverse pair, x2
    double time_plan(const Fft3Desc& d, cudaStream_t st) {
        if (!sms) {
            int dev = 0;
            check_cuda(cudaGetDevice(&dev), "tune device");
            check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "tune sms");
            check_cuda(cudaMalloc(&sink, sizeof(float) * 4096), "tune sink");
        }
        if (!attr) {
            check_cuda(cudaFuncSetAttribute(k_fft_tune<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                       "tune attr");
            check_cuda(cudaFuncSetAttribute(k_fft_tune<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes),
                       "tune attr");
            attr = true;
        }
        const size_t smem = sizeof(cf32) * ((size_t)fft3_tw_len(d.n) + padded_len(d.n));
        if (smem > (size_t)kSmemBytes) return 1e30;
        const bool two = smem + 1024 <= 114 * 1024;
        const int grid = std::min(sms * (two ? 2 : 1), 4096);
        cudaEvent_t e0, e1;
        check_cuda(cudaEventCreate(&e0), "tune event");
        check_cuda(cudaEventCreate(&e1), "tune event");
        double best = 1e30;
        for (int it = 0; it < 4; ++it) {
            check_cuda(cudaEventRecord(e0, st), "tune record");
            if (two) note_launch(), k_fft_tune<512><<<grid, 512, smem, st>>>(d, 2, sink);
            else note_launch(), k_fft_tune<1024><<<grid, 1024, smem, st>>>(d, 2, sink);
            check_cuda(cudaGetLastError(), "tune launch");
            check_cuda(cudaEventRecord(e1, st), "tune record");
            check_cuda(cudaEventSynchronize(e1), "tune sync");
            float ms = 0;
            check_cuda(cudaEventElapsedTime(&ms, e0, e1), "tune elapsed");
            if (it > 0) best = std::min(best, 1e3 * (double)ms);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return best;
    }

    static std::vector<std::vector<int>> candidates(int n) {
        const std::vector<int> base = default_radices3(n);
        std::set<std::vector<int>> seen;
        std::vector<std::vector<int>> out;
        auto add = [&](std::vector<int> v) {
            if (!v.empty() && (int)v.size() <= kMaxStages && seen.insert(v).second) out.push_back(v);
        };
        add(base);
        std::vector<int> p16, rem2, odd;
        for (int r : base) (r == 16 ? p16 : (r == 2 || r == 4 || r == 8) ? rem2 : odd).push_back(r);
        auto cat = [](std::initializer_list<const std::vector<int>*> parts) {
            std::vector<int> v;
            for (auto* p : parts) v.insert(v.end(), p->begin(), p->end());
            return v;
        };
        add(cat({&rem2, &p16, &odd}));   // short power-of-two stage first
        add(cat({&odd, &p16, &rem2}));   // odd radices first
        add(cat({&p16, &odd, &rem2}));   // odd radices before the short stage
        if (!p16.empty() && rem2.size() == 1 && (rem2[0] == 2 || rem2[0] == 4)) {
            // 16 x r -> 8 x 2r: same passes, different stage widths
            std::vector<int> a(p16.begin() + 1, p16.end());
            const std::vector<int> b = {8, 2 * rem2[0]};
            add(cat({&b, &a, &odd}));
            add(cat({&a, &odd, &b}));
        }
        return out;
    }

    std::vector<int> radices_locked(int n, cudaStream_t st) {
        auto it = rad.find(n);
        if (it != rad.end()) return it->second;
        load();
        it = rad.find(n);
        if (it != rad.end()) return it->second;
        if (!on || capturing(st)) return default_radices3(n);
        // the first candidate is the default order; another replaces it only
        // when it is more than 2 % faster
        std::vector<int> best;
        double bt = 1e30;
        for (const auto& c : candidates(n)) {
            auto plan = build_plan3(n, c);
            const double t = time_plan(plan->d, st);
            if (best.empty() || t < bt * 0.98) {
                bt = t;
                best = c;
            }
        }
        rad[n] = best;
        save();
        return best;
    }
};

Tuner& tuner() {
    static Tuner t;
    return t;
}

}  // namespace

std::vector<int> tuned_radices(int n, cudaStream_t st) {
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk(t.mu);
    return t.radices_locked(n, st);
}

long long tuned_length(long long minlen, long long cap, cudaStream_t st) {
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk(t.mu);
    const std::pair<long long, long long> key{minlen, cap};
    auto it = t.len.find(key);
    if (it != t.len.end()) return it->second;
    t.load();
    it = t.len.find(key);
    if (it != t.len.end()) return it->second;
    const long long model = fast_len(minlen, cap);
    if (!t.on || Tuner::capturing(st) || model > cap) return model;
    // candidates: the three cheapest 7-smooth lengths by length x passes
    std::vector<std::pair<double, long long>> c;
    const long long hi = std::max(minlen, (long long)(minlen * 1.25) + 1);
    for (long long m = std::max(1LL, minlen); m <= hi && m <= cap; ++m)
        if (is_smooth7(m)) c.push_back({(double)m * fft3_passes(m), m});
    std::sort(c.begin(), c.end());
    if (c.size() > 3) c.resize(3);
    long long best = model;
    double bt = 1e30;
    for (const auto& kv : c) {
        const long long m = kv.second;
        const std::vector<int> r = t.radices_locked((int)m, st);
        auto plan = build_plan3((int)m, r);
        const double us = t.time_plan(plan->d, st);
        if (us < bt * 0.98) {
            bt = us;
            best = m;
        }
    }
    t.len[key] = best;
    t.save();
    return best;
}

std::string tuning_report() {
    Tuner& t = tuner();
    std::lock_guard<std::mutex> lk(t.mu);
    std::ostringstream o;
    o << (t.on ? "on" : "off") << " radices";
    for (const auto& kv : t.rad) {
        o << " " << kv.first << ":";
        for (size_t i = 0; i < kv.second.size(); ++i) o << (i ? "." : "") << kv.second[i];
    }
    o << " lengths";
    for (const auto& kv : t.len) o << " " << kv.first.first << ">" << kv.second;
    return o.str();
}

}  // namespace s1g
