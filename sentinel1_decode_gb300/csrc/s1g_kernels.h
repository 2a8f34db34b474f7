// Internal kernel launchers shared by the pipeline (not part of the C ABI).
#pragma once

#include <string>

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "../../include/s1g.h"
#include "s1g_fft_engine.h"

namespace s1g {

// ------------------------------------------------------------------ indexing
struct IndexScratch {
    long long* entry = nullptr;
    long long* exitp = nullptr;
    int* count = nullptr;
    int* base = nullptr;
    int* total = nullptr;
    int cap = 0;
    void reserve(int nchunks);
    void release();
    ~IndexScratch() { release(); }
};

// Index the space packets of a device-resident stream.  Writes up to
// max_packets offsets; if sync_count, returns the packet count (host sync).
int index_packets(const uint8_t* d_stream, long long n, long long* d_offsets, int max_packets, IndexScratch& sc,
                  cudaStream_t st, bool sync_count, int* h_count);
void gather_headers(const uint8_t* d_stream, long long n, const long long* d_off, int npk, uint8_t* d_hdr,
                    cudaStream_t st);

// ------------------------------------------------------------------ decode
struct DecodeTables {
    void* lut = nullptr;
    void init();
    ~DecodeTables();
};

struct DecodeScratch {
    uint8_t* sym = nullptr;
    uint8_t* brc = nullptr;
    uint8_t* thidx = nullptr;
    size_t sym_cap = 0, blk_cap = 0;
    void reserve(size_t sym_bytes, size_t blk_bytes);
    ~DecodeScratch();
};

// Symbol-row pitch (bytes) of one decoded channel: nq rounded up to 4.
__host__ __device__ inline int sym_pitch(int nq) { return (nq + 3) & ~3; }

// Short-time windows of the ECCM notch on a line of n_r samples (fft 128,
// stride 64): floor((n_r / 128) * (128 / 64)), signal_processing.cpp:918.
inline int eccm_num_windows(int n_r) { return (int)floor(((double)n_r / 128.0) * (128.0 / 64.0)); }

// One packet of a batched decode (any mix of bursts and row lengths): packet
// index, quads, byte offset of its 4 symbol rows in the symbol scratch, index
// of its first block code in the BRC/THIDX scratch, element offset of its
// output row.
struct DecodeJob {
    int pk;
    int nq;
    long long sym;
    long long blk;
    long long out;
};

template <typename R>
void decode_jobs(const uint8_t* d_stream, long long n, const long long* d_offsets, const DecodeJob* d_jobs, int njobs,
                 size_t sym_bytes, size_t blk_bytes, cpx<R>* out, int* d_status, DecodeScratch& sc,
                 const DecodeTables& tabs, cudaStream_t st);

// Scaled float image of n complex samples (CF32 or CF64 `elem`), mode
// S1G_SCALE_*; d_max: one device word for the max |x| of the norm modes.
void scale_image(const void* in, int elem, long long n, int mode, float* out, unsigned long long* d_max,
                 cudaStream_t st);
// Spectrogram of one echo line (FP64): [fft][windows] complex, and the number
// of windows for n samples.
int spectrogram_windows(int n, int fft, int stride);
void spectrogram(const cf64* line, int n, int fft, int stride, cf64* out, cudaStream_t st);
// BigTIFF float32 writer, bottom-up rows (host).
int write_bigtiff(const char* path, const float* img, long long rows, long long cols, std::string& err);

template <typename R>
void decode_burst(const uint8_t* d_stream, long long n, const long long* d_offsets, const int* d_pkidx, int p0,
                  int npk, int nq, cpx<R>* out, long long pitch, int* d_status, DecodeScratch& sc, const DecodeTables& tabs,
                  cudaStream_t st);

// Data formats A/B (bypass) and C (BAQ): rows of packets whose baq_mode is
// 0 or 3..5 (FDBAQ rows are skipped).  fields = 0: the reference's output;
// 1: every sample from its own bits.
template <typename R>
void decode_fixed_burst(const uint8_t* d_stream, long long n, const long long* d_offsets, const int* d_pkidx, int p0,
                        int npk, int nq, cpx<R>* out, long long pitch, int* d_status, int fields, cudaStream_t st);
template <typename R>
void decode_fixed_jobs(const uint8_t* d_stream, long long n, const long long* d_offsets, const DecodeJob* d_jobs,
                       int njobs, cpx<R>* out, int* d_status, int fields, cudaStream_t st);
// The reconstruction of jobs whose symbols decode_jobs just left in sc (the
// FP64 samples of an FP32-decoded batch, for the FP64 ECCM notch).
template <typename R>
void decode_jobs_values(const DecodeJob* d_jobs, int njobs, cpx<R>* out, int* d_status, const DecodeScratch& sc,
                        cudaStream_t st);

// Differentiable azimuth chain (s1g_adjoint.cu): row factors, bulk RCMC
// phase exp(i sign beta_k f_r), azimuth filter exp(i sign c4pl R_r omd_k),
// image entropy sums / gradient, per-row sum_c w_c Im(conj(a) b) (w = colw,
// or the FFT-order frequency of c at rate freq_fs when colw is null and
// freq_fs > 0, else 1).
template <typename R>
void row_factor(cpx<R>* a, long long pitch, int cols, long long rows, const cpx<R>* f, cudaStream_t st);
template <typename R>
void rcmc_phase(cpx<R>* a, int n, long long rows, const double* beta, double fs, int sign, cudaStream_t st);
template <typename R>
void az_filter(cpx<R>* a, int n_r, long long rows, const double* omd, const double* slant, double c4pl, int sign,
               cudaStream_t st);
template <typename R>
void entropy_sums(const cpx<R>* y, long long n, double* sums, cudaStream_t st);
template <typename R>
void entropy_grad(const cpx<R>* y, cpx<R>* g, long long n, const double* sums, cudaStream_t st);
template <typename R>
void row_imdot(const cpx<R>* a, const cpx<R>* b, int cols, long long rows, const double* colw, double freq_fs,
               double* out, cudaStream_t st);

// ------------------------------------------------------------------ SAR stages
// Per-row (azimuth line) parameters of the row pass, FP64.
struct RowParam {
    double fa;        // azimuth frequency of the row
    double re;        // local earth radius under the platform (image_formation.cpp:398-401)
    double h;         // platform distance from earth centre
    double v;         // platform speed
};

// TOPS differentiable chain (s1g_adjoint.cu): per-range-bin columns of the
// row pass factors (fdc includes the centroid offset), the adjoint of each
// factor, its derivative along the Doppler frequency, and the adjoints of
// the frequency unfolding's band move and tiling.
struct TopsCols {
    const double* slant;
    const double* rf;
    const double* fdc;
    const double* tcorr;
    const double* rscale;
};
template <typename R>
void tops_factor_adj(cpx<R>* g, long long p, int S, int n_r, const RowParam* rows, const TopsCols& c, int stage,
                     cudaStream_t st);
template <typename R>
void tops_dpsi(const cpx<R>* G, const cpx<R>* V, long long p, int S, int n_r, const RowParam* rows, const TopsCols& c,
               int stage, double* out, cudaStream_t st);
template <typename R>
void band_insert(const cpx<R>* in, long long ip, cpx<R>* out, long long op, int n, int start, int len, long long rows,
                 cudaStream_t st);
template <typename R>
void ufr_fold(const cpx<R>* Gy, long long yp, int tile_len, const cpx<R>* d, cpx<R>* Gx, long long xp, int n_a,
              long long rows, cudaStream_t st);

struct DcFitArgs {
    int n_rng;
    int num_blocks;
    double prf;
    double rt[64];     // block range times minus the first (get_slant_range_times(num_blocks))
    double near, far;  // slant range time span of the full range axis
};

struct TufrParams {     // time-domain unfolding parameters, computed on the device
    double ka_mean, n_ref, focused_time, bandwidth;
    int num_tiles, shape, start, end, output_shape, down, ok;
};

template <typename R>
void pad_rows(const cpx<R>* in, long long in_pitch, int n_in, cpx<R>* out, long long out_pitch, int n_out,
              long long rows, cudaStream_t st);
template <typename R>
void mul_rows_by_vec(cpx<R>* a, long long pitch, int n, long long rows, const cpx<R>* vec, cudaStream_t st);
template <typename R>
void rc_crop(const cpx<R>* in, long long in_pitch, int m, cpx<R>* out, long long out_pitch, int n_r, int h,
             long long rows, cudaStream_t st);
template <typename R>
void roll_rows(const cpx<R>* in, long long in_pitch, cpx<R>* out, long long out_pitch, int n, int shift,
               long long rows, cudaStream_t st);
template <typename R>
void dc_sums(const cpx<R>* rc, long long pitch, int n_a, int n_r, const cpx<R>* deramp, cf64* sums,
             cudaStream_t st);
void dc_fit(const cf64* sums, const DcFitArgs& a, double* f_dc, cudaStream_t st);
template <typename R>
void fufr_prep(const cpx<R>* X, long long xpitch, int n_a, cpx<R>* y, long long ypitch, int S, int tile_len,
               const cpx<R>* deramp, long long rows, cudaStream_t st);
template <typename R>
void band_select(const cpx<R>* Y, long long ypitch, cpx<R>* Z, long long zpitch, int n, int start, int len,
                 long long rows, cudaStream_t st);
template <typename R>
void scale_mul_vec(cpx<R>* a, long long pitch, int n, long long rows, const cpx<R>* vec, double scale,
                   cudaStream_t st);
template <typename R>
void scale_rows(cpx<R>* a, long long pitch, int n, long long rows, double scale, cudaStream_t st);
template <typename R>
void src_filter(cpx<R>* data, long long pitch, int S, int n_r, const RowParam* rows, const double* slant,
                const double* range_freq, const double* f_dc, double c3, cudaStream_t st);
template <typename R>
void az_filter(cpx<R>* data, long long pitch, int S, int n_r, const RowParam* rows, const double* slant,
               const double* range_freq, const double* f_dc, const double* tcorr, const double* rscale, int tops,
               cudaStream_t st);
void ka_table(double* kaT, long long pitch, int S, int n_r, const RowParam* rows, const double* slant,
              const double* f_dc, cudaStream_t st);
void tufr_params(const double* kaT, long long pitch, int S, int n_r, const double* f_dc, double dc_rate,
                 double burst_duration, double prf, double doppler_bandwidth, int swath_number, TufrParams* out,
                 cudaStream_t st);
template <typename R>
void tufr_deramp(const cpx<R>* a, long long apitch, int S, cpx<R>* y, long long ypitch, const double* kaT,
                 long long kpitch, const double* f_dc, int n_r, double dc_rate, int num_tiles, double focused_time,
                 cudaStream_t st);
template <typename R>
void tufr_resample(const cpx<R>* z, long long zpitch, int shape, cpx<R>* out, long long opitch, int down,
                   const double* kaT, long long kpitch, int S, const double* f_dc, int n_r, double dc_rate,
                   double n_ref, double focused_time, cudaStream_t st);
template <typename R>
void eccm_detect(const cpx<R>* X, long long pitch, int n, long long rows, double det, int* flags, cudaStream_t st);
template <typename R>
void eccm_notch(cpx<R>* data, long long pitch, int n_r, long long rows, const int* flags, double mit,
                const FftDesc<R>& d128, unsigned char* mask_out, cudaStream_t st);
template <typename To, typename Ti>
void convert_rows(const cpx<Ti>* in, long long in_pitch, cpx<To>* out, long long out_pitch, int cols, int valid_cols,
                  long long rows, cudaStream_t st);

}  // namespace s1g
