// Batched row-FFT engine of arbitrary length (host-side plans).
//
// Plan kinds, chosen by length n and precision:
//   SMEM      n is 7-smooth and fits one CTA's shared memory: one kernel, one
//             CTA per row, in-place DIT;
//   BLUE      n has a prime factor > 7: Bluestein chirp-z through a 7-smooth
//             convolution length m >= 2n-1 that fits shared memory;
//   FOUR      n is 7-smooth but too long: four-step (n = n1*n2) through global
//             memory with batched transposes;
//   BLUE4     Bluestein whose convolution length needs the four-step path.
// Every transform is unnormalised; dir=-1 forward, dir=+1 backward.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "s1g_fft.cuh"
#include "s1g_fft3.cuh"

namespace s1g {

enum FftKind { FFT_SMEM = 0, FFT_BLUE = 1, FFT_FOUR = 2, FFT_BLUE4 = 3 };

// Largest shared-memory buffer a CTA may use (bytes).
constexpr int kSmemBytes = 220 * 1024;

bool is_smooth7(long long n);
long long next_smooth7(long long n);
// Transform length >= minlen for the radix-16 core: the 7-smooth length in
// [minlen, 1.25 minlen] (and <= cap) of least length x passes.
long long fast_len(long long minlen, long long cap);
// Shared-memory passes of the radix-16 core for length n.
int fft3_passes(long long n);
template <typename R>
inline int smem_capacity() { return kSmemBytes / (int)sizeof(cpx<R>); }

// Device memory arena owned by a processing context: grow-only scratch.
struct DeviceArena {
    void* ptr = nullptr;
    size_t size = 0;
    ~DeviceArena();
    void* get(size_t bytes);
};

template <typename R>
struct FftPlan {
    int n = 0;
    FftKind kind = FFT_SMEM;
    FftDesc<R> d;                 // SMEM: length n; BLUE: length m
    int m = 0;                    // Bluestein convolution length
    cpx<R>* chirp = nullptr;      // w[k] = exp(-i pi k^2 / n), k < n
    cpx<R>* kern = nullptr;       // FFT_m of conj chirp, scaled by 1/m
    int n1 = 0, n2 = 0;           // four-step split (FOUR) of n, or of m (BLUE4)
    std::shared_ptr<FftPlan<R>> p1, p2, pm;   // sub-plans
    cpx<R>* tw4 = nullptr;        // four-step twiddle table, length n (or m)
    std::vector<void*> owned;     // device allocations
    ~FftPlan();
};

// Device tables of the radix-16 core for one length.
struct Fft3Plan {
    Fft3Desc d;
    std::vector<void*> owned;
    ~Fft3Plan();
};

// One per processing context (device + stream).
struct FftEngine {
    explicit FftEngine(cudaStream_t s);
    ~FftEngine();
    cudaStream_t stream;
    std::map<int, std::shared_ptr<FftPlan<float>>> plans32;
    std::map<int, std::shared_ptr<FftPlan<double>>> plans64;
    std::map<int, std::shared_ptr<Fft3Plan>> plans3;
    DeviceArena scratch_a, scratch_b, scratch_c;

    template <typename R>
    std::shared_ptr<FftPlan<R>> plan(int n);

    // out[b*out_pitch + k] = sum_j in[b*in_pitch + j] exp(dir 2 pi i jk/n).
    // in may equal out.  Works for any n >= 1.
    template <typename R>
    void rows(const FftPlan<R>& p, const cpx<R>* in, long long in_pitch, cpx<R>* out,
              long long out_pitch, long long batch, int dir);

    // Smooth descriptor for device-side fused kernels (throws if n is not
    // 7-smooth or does not fit shared memory).
    template <typename R>
    FftDesc<R> smem_desc(int n);

    // Radix-16 core descriptor (n 7-smooth, fits shared memory); the radix
    // order comes from the autotuner (s1g_tune.cu) when it is on.
    Fft3Desc desc3(int n);
    // Transform length >= minlen (<= cap) for the fused kernels: the
    // autotuner's pick among the cheapest 7-smooth candidates, or fast_len.
    long long tuned_len(long long minlen, long long cap);
};

// Radix-16 plans and their autotuner (s1g_tune.cu).
std::vector<int> default_radices3(long long n);
std::shared_ptr<Fft3Plan> build_plan3(int n, const std::vector<int>& radices);
// Radix order for length n: the fastest measured candidate when tuning is on
// (S1G_AUTOTUNE unset or not "0"), else default_radices3.  Measurements run
// on `st` (skipped while st is being captured) and persist in a text file
// (S1G_FFT_TUNE_FILE, default fft_tune.txt beside the library).
std::vector<int> tuned_radices(int n, cudaStream_t st);
long long tuned_length(long long minlen, long long cap, cudaStream_t st);
// "n:r1.r2..;..." of the radix orders and "minlen>M;..." of the lengths
// chosen so far in this process.
std::string tuning_report();

// batched transpose: in [B][rows][cols] (pitches in elements) -> out [B][cols][rows]
template <typename R>
void transpose_batched(const cpx<R>* in, long long in_row_pitch, long long in_batch_pitch, cpx<R>* out,
                       long long out_row_pitch, long long out_batch_pitch, int rows, int cols, long long batch,
                       cudaStream_t s);

void check_cuda(cudaError_t e, const char* what);

// Count of kernels this library has launched (reported by the benchmark).
void note_launch();
// Add n (may be negative) to the launch count (graph replays and captures).
void note_launches(long long n);
long long launch_count();

}  // namespace s1g
