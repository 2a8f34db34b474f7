// Image output of the s1_write TIFF commands: the scaling modes of
// scale() (signal_processing.cpp:1031-1071, with norm_2d :366-400 and
// magnitude_2d :444-459) as a GPU epilogue on a device-resident product, and
// a BigTIFF float32 writer with the layout of _write_tif
// (image_write.cpp:3-25: one sample per pixel, IEEE float, min-is-black,
// rows written bottom-up).
//
// Modes (the reference computes in double and casts the result to float):
//   real, imag   the component
//   mag          |x|^2
//   norm         (|x| + 1e-12) / max|x|
//   norm_log     20 log10((|x| + 1e-12) / max|x|)
// max|x| is taken over the whole product (atomicMax on the bit pattern of
// the non-negative double).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "s1g_kernels.h"

namespace s1g {

template <typename R>
__global__ void k_abs_max(const cpx<R>* __restrict__ in, long long n, unsigned long long* __restrict__ maxbits) {
    double m = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cpx<R> v = in[i];
        m = fmax(m, hypot((double)v.x, (double)v.y));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ double wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, wm[w]);
        atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
    }
}

template <typename R>
__global__ void k_scale(const cpx<R>* __restrict__ in, long long n, int mode,
                        const unsigned long long* __restrict__ maxbits, float* __restrict__ out) {
    const double mx = maxbits ? __longlong_as_double((long long)*maxbits) : 1.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const cpx<R> v = in[i];
        float r;
        switch (mode) {
            case S1G_SCALE_REAL: r = (float)v.x; break;
            case S1G_SCALE_IMAG: r = (float)v.y; break;
            case S1G_SCALE_MAG: {
                const double a = hypot((double)v.x, (double)v.y);
                r = (float)(a * a);
                break;
            }
            case S1G_SCALE_NORM: r = (float)((hypot((double)v.x, (double)v.y) + 1e-12) / mx); break;
            default: r = (float)(20.0 * log10((hypot((double)v.x, (double)v.y) + 1e-12) / mx)); break;
        }
        out[i] = r;
    }
}

void scale_image(const void* in, int elem, long long n, int mode, float* out, unsigned long long* d_max,
                 cudaStream_t st) {
    const int threads = 256;
    const int grid = (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, 152 * 16));
    const bool norm = mode == S1G_SCALE_NORM || mode == S1G_SCALE_NORM_LOG;
    if (norm) {
        check_cuda(cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), st), "max reset");
        if (elem == S1G_CF32)
            note_launch(), k_abs_max<float><<<grid, threads, 0, st>>>((const cf32*)in, n, d_max);
        else
            note_launch(), k_abs_max<double><<<grid, threads, 0, st>>>((const cf64*)in, n, d_max);
    }
    if (elem == S1G_CF32)
        note_launch(), k_scale<float><<<grid, threads, 0, st>>>((const cf32*)in, n, mode, norm ? d_max : nullptr, out);
    else
        note_launch(), k_scale<double><<<grid, threads, 0, st>>>((const cf64*)in, n, mode, norm ? d_max : nullptr, out);
    check_cuda(cudaGetLastError(), "scale");
}

// ------------------------------------------------------------------ spectrogram
// spectrogram() of signal_processing.cpp:794-844 on one echo line: window i
// takes samples [i stride, i stride + fft) -- cut at n - 1 when that passes
// the end, as the reference does -- zero-padded to fft, times the Hann window
// 0.5 (1 - cos(2 pi j / (fft - 1))); forward DFT, fftshift, transpose:
// out[k'][i] = X_i[(k' + fft/2) mod fft].  FP64, direct DFT (fft is small).
__global__ void k_spectrogram(const cf64* __restrict__ line, int n, int fft, int stride, int nwin,
                              cf64* __restrict__ out) {
    const double kPI = 3.14159265358979;
    const long long total = (long long)fft * nwin;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int kp = (int)(e / nwin), i = (int)(e % nwin);
        const int k = (kp + fft / 2) % fft;
        const int start = i * stride;
        int end = start + fft;
        if (end > n) end = n - 1;
        double re = 0.0, im = 0.0;
        for (int j = 0; j < end - start; ++j) {
            const double w = 0.5 * (1.0 - cos(2.0 * kPI * (double)j / ((double)fft - 1)));
            const cf64 x = line[start + j];
            double sn, cs;
            sincospi(-2.0 * (double)(((long long)j * k) % fft) / (double)fft, &sn, &cs);
            re += w * (x.x * cs - x.y * sn);
            im += w * (x.x * sn + x.y * cs);
        }
        out[(long long)kp * nwin + i] = mk(re, im);
    }
}

int spectrogram_windows(int n, int fft, int stride) {
    return (int)std::floor(((double)n / (double)fft) * ((double)fft / (double)stride));
}

void spectrogram(const cf64* line, int n, int fft, int stride, cf64* out, cudaStream_t st) {
    const int nwin = spectrogram_windows(n, fft, stride);
    const long long total = (long long)fft * nwin;
    if (total <= 0) return;
    const int grid = (int)std::min<long long>((total + 255) / 256, 152 * 8);
    note_launch(), k_spectrogram<<<grid, 256, 0, st>>>(line, n, fft, stride, nwin, out);
    check_cuda(cudaGetLastError(), "spectrogram");
}

// ------------------------------------------------------------------ BigTIFF
namespace {

struct Entry {
    uint16_t tag, type;
    uint64_t count, value;   // value or offset (little-endian, left-justified)
};

void put16(std::vector<uint8_t>& b, uint16_t v) {
    b.push_back((uint8_t)v);
    b.push_back((uint8_t)(v >> 8));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i)));
}

}  // namespace

// Little-endian BigTIFF ("II", version 43), strips of about 8 KB (whole rows),
// image row 0 = data row rows-1 (the reference's bottom-up scanline loop).
int write_bigtiff(const char* path, const float* img, long long rows, long long cols, std::string& err) {
    if (!path || !img || rows <= 0 || cols <= 0) {
        err = "write_tiff: bad arguments";
        return S1G_E_INVALID_ARGUMENT;
    }
    FILE* f = fopen(path, "wb");
    if (!f) {
        err = std::string("Unable to open ") + path + " for writing.";
        return S1G_E_IO;
    }
    const uint64_t row_bytes = (uint64_t)cols * 4;
    const uint64_t rps = std::max<uint64_t>(1, 8192 / row_bytes);
    const uint64_t nstrips = ((uint64_t)rows + rps - 1) / rps;
    const uint64_t data_off = 16;
    const uint64_t data_bytes = row_bytes * (uint64_t)rows;
    std::vector<uint64_t> offs(nstrips), counts(nstrips);
    for (uint64_t s = 0; s < nstrips; ++s) {
        const uint64_t r0 = s * rps, r1 = std::min<uint64_t>((uint64_t)rows, r0 + rps);
        offs[s] = data_off + r0 * row_bytes;
        counts[s] = (r1 - r0) * row_bytes;
    }
    // IFD after the pixel data, then the strip arrays
    const uint64_t ifd_off = data_off + data_bytes + (data_bytes & 1);
    const int nent = 12;
    const uint64_t arrays_off = ifd_off + 8 + 20ull * nent + 8;
    const bool inl = nstrips == 1;
    std::vector<Entry> e = {
        {256, 16, 1, (uint64_t)cols},                                   // ImageWidth (LONG8)
        {257, 16, 1, (uint64_t)rows},                                   // ImageLength
        {258, 3, 1, 32},                                                // BitsPerSample
        {259, 3, 1, 1},                                                 // Compression: none
        {262, 3, 1, 1},                                                 // Photometric: min-is-black
        {273, 16, nstrips, inl ? offs[0] : arrays_off},                 // StripOffsets
        {274, 3, 1, 1},                                                 // Orientation: top-left
        {277, 3, 1, 1},                                                 // SamplesPerPixel
        {278, 16, 1, rps},                                              // RowsPerStrip
        {279, 16, nstrips, inl ? counts[0] : arrays_off + 8 * nstrips}, // StripByteCounts
        {284, 3, 1, 1},                                                 // PlanarConfig: contiguous
        {339, 3, 1, 3},                                                 // SampleFormat: IEEE float
    };
    std::vector<uint8_t> hdr;
    hdr.push_back('I');
    hdr.push_back('I');
    put16(hdr, 43);
    put16(hdr, 8);
    put16(hdr, 0);
    put64(hdr, ifd_off);
    bool ok = fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
    for (long long r = rows - 1; r >= 0 && ok; --r)
        ok = fwrite(img + r * cols, 4, (size_t)cols, f) == (size_t)cols;
    if (ok && (data_bytes & 1)) ok = fputc(0, f) != EOF;
    std::vector<uint8_t> ifd;
    put64(ifd, nent);
    for (const Entry& x : e) {
        put16(ifd, x.tag);
        put16(ifd, x.type);
        put64(ifd, x.count);
        put64(ifd, x.value);
    }
    put64(ifd, 0);
    if (!inl) {
        for (uint64_t v : offs) put64(ifd, v);
        for (uint64_t v : counts) put64(ifd, v);
    }
    if (ok) ok = fwrite(ifd.data(), 1, ifd.size(), f) == ifd.size();
    if (fclose(f) != 0) ok = false;
    if (!ok) {
        err = std::string("Failed to write ") + path;
        return S1G_E_IO;
    }
    return S1G_OK;
}

}  // namespace s1g
