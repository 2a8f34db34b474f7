// Header-only C++ facade over the s1g C ABI with the interface of the
// reference's S1_Decoder (s1_decoder.h:13-77), so that code written against
// sentinel1_decode compiles unchanged against this library:
//
//   S1_Decoder s1(path);
//   s1.apply_eccm(13000, 100);
//   CF_VEC_2D slc = s1.get_azimuth_compressed_burst("IW2", 0);
//
// Products come back by value as CF_VEC_2D (vector<vector<complex<double>>>),
// as in the reference.  Errors follow the reference: a swath or burst that is
// not in the data prints the reference's message and exits with status 1
// (s1_decoder.cpp:45-89) unless S1G_FACADE_THROW is defined, in which case
// std::out_of_range is thrown; decode errors throw std::runtime_error with
// the reference's message, bad arguments std::invalid_argument, unsupported
// modes std::domain_error.
//
// Additions beyond the reference's interface: set_precision() selects the GPU
// arithmetic ("fp32" fused path, the default; "fp64"; "fp32_plain"), and the
// *_cf32() calls return one contiguous complex<float> array (the layout that
// save_*_as_cf32 writes) without the CF_VEC_2D copy.
//
// Also provided: index_decoder / annotation_decoder / annotation_time_decoder
// (aux_decoding.cpp) for the product sidecars, and check_sidecars(), which
// cross-checks them against the packet stream.
//
// Link with libs1g.so.  Define S1G_NO_REFERENCE_TYPES when the reference's
// misc_types.h is also included.
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include <sys/types.h>

#include "s1g.h"

#ifndef S1G_NO_REFERENCE_TYPES
using cdouble = std::complex<double>;
using CF_VEC_1D = std::vector<cdouble>;
using CF_VEC_2D = std::vector<CF_VEC_1D>;
#endif

// State vectors parsed from the sub-commutated ancillary data, with the
// members of the reference's STATE_VECTORS (state_vectors.h:55-120):
// time, position (x, y, z), velocity (x, y, z), quaternion (x, y, z, w:
// scalar last), angular rate (x, y, z) and attitude (-pitch, -roll, yaw).
struct S1G_STATE_VECTORS {
    std::vector<double> times;
    std::vector<std::vector<double>> positions;
    std::vector<std::vector<double>> velocities;
    std::vector<std::vector<double>> quaternions;
    std::vector<std::vector<double>> angular_rates;
    std::vector<std::vector<double>> attitudes;
};

#ifndef S1G_NO_REFERENCE_TYPES
#include <unordered_map>
#define S1G_VEC_UNSORTEDMAP std::vector<std::unordered_map<std::string, u_int64_t>>

// index_decoder / annotation_decoder / annotation_time_decoder
// (aux_decoding.cpp:61-145) with the reference's results, including the
// extra record its read loop appends at the end of a file.  Throw
// std::runtime_error when the file cannot be opened.
inline S1G_VEC_UNSORTEDMAP index_decoder(const std::string& filename) {
    int64_t n = 0;
    if (s1g_read_index(filename.c_str(), nullptr, 0, &n, 1) != S1G_OK)
        throw std::runtime_error("Unable to open: " + filename);
    std::vector<s1g_index_record> r((size_t)n);
    s1g_read_index(filename.c_str(), r.data(), n, &n, 1);
    S1G_VEC_UNSORTEDMAP out;
    for (const auto& x : r)
        out.push_back({{"date_time", x.date_time}, {"time_delta", x.time_delta}, {"data_size", x.data_size},
                       {"unit_offset", x.unit_offset}, {"byte_offset", x.byte_offset},
                       {"variable_flag", x.variable_flag}, {"spare_data", x.spare_data}});
    return out;
}

inline S1G_VEC_UNSORTEDMAP annotation_decoder(const std::string& filename) {
    int64_t n = 0;
    if (s1g_read_annotation(filename.c_str(), nullptr, 0, &n, 1) != S1G_OK)
        throw std::runtime_error("Unable to open: " + filename);
    std::vector<s1g_annotation_record> r((size_t)n);
    s1g_read_annotation(filename.c_str(), r.data(), n, &n, 1);
    S1G_VEC_UNSORTEDMAP out;
    for (const auto& x : r)
        out.push_back({{"days_ul", x.days_ul}, {"milliseconds_ul", x.milliseconds_ul},
                       {"microseconds_ul", x.microseconds_ul}, {"days_dl", x.days_dl},
                       {"milliseconds_dl", x.milliseconds_dl}, {"microseconds_dl", x.microseconds_dl},
                       {"packet_length", x.packet_length}, {"num_transfer_frames", x.num_transfer_frames},
                       {"error_flag", x.error_flag}, {"bit_1_type", x.bit_1_type}, {"bit_2_type", x.bit_2_type},
                       {"bit_6_type", x.bit_6_type}, {"spare_field", x.spare_field}});
    return out;
}

inline std::vector<double> annotation_time_decoder(const std::string& filename) {
    int64_t n = 0;
    if (s1g_annotation_times(filename.c_str(), nullptr, 0, &n, 1) != S1G_OK)
        throw std::runtime_error("Unable to open: " + filename);
    std::vector<double> t((size_t)n);
    s1g_annotation_times(filename.c_str(), t.data(), n, &n, 1);
    return t;
}
#endif

// A product as one contiguous row-major complex<float> array.
struct S1G_CF32_PRODUCT {
    int64_t rows = 0, cols = 0;
    std::vector<std::complex<float>> data;
};

class S1_Decoder {
  public:
    S1_Decoder() = default;

    explicit S1_Decoder(const std::string& filename, int device = 0) : _filename(filename) {
        const int st = s1g_open_file(filename.c_str(), device, &_h);
        if (st == S1G_E_IO) throw std::runtime_error("Unable to open file: " + filename);
        check(st);
    }

    S1_Decoder(const S1_Decoder&) = delete;
    S1_Decoder& operator=(const S1_Decoder&) = delete;
    S1_Decoder(S1_Decoder&& o) noexcept : _filename(std::move(o._filename)), _h(o._h) { o._h = nullptr; }
    S1_Decoder& operator=(S1_Decoder&& o) noexcept {
        if (this != &o) {
            if (_h) s1g_close(_h);
            _filename = std::move(o._filename);
            _h = o._h;
            o._h = nullptr;
        }
        return *this;
    }
    ~S1_Decoder() {
        if (_h) s1g_close(_h);
    }

    // The reference's argument-less apply_eccm() enables the notch with
    // thresholds it never initialises; here the thresholds of an earlier
    // apply_eccm(det, mit) call are kept, and without one it is an error.
    void apply_eccm() {
        if (!_eccm_set) throw std::invalid_argument("apply_eccm(): thresholds were never set; use apply_eccm(det, mit)");
        check(s1g_apply_eccm(handle(), _det, _mit));
    }
    void apply_eccm(const int& detection_threshold, const int& mitigation_threshold) {
        _det = detection_threshold;
        _mit = mitigation_threshold;
        _eccm_set = true;
        check(s1g_apply_eccm(handle(), _det, _mit));
    }

    void set_precision(const std::string& precision) {
        int p = S1G_PREC_FP32;
        if (precision == "fp64") p = S1G_PREC_FP64;
        else if (precision == "fp32_plain") p = S1G_PREC_FP32_PLAIN;
        else if (precision != "fp32") throw std::invalid_argument("precision must be fp32, fp32_plain or fp64");
        check(s1g_set_precision(handle(), p));
    }

    [[nodiscard]] S1G_STATE_VECTORS get_state_vectors() {
        int count = 0;
        check(s1g_state_vectors(handle(), nullptr, 0, &count));
        std::vector<double> buf((size_t)count * 7);
        check(s1g_state_vectors(handle(), buf.data(), count, &count));
        std::vector<double> att((size_t)count * 10);
        check(s1g_attitudes(handle(), att.data(), count, &count));
        S1G_STATE_VECTORS sv;
        for (int i = 0; i < count; ++i) {
            const double* r = buf.data() + 7 * i;
            const double* a = att.data() + 10 * i;
            sv.times.push_back(r[0]);
            sv.positions.push_back({r[1], r[2], r[3]});
            sv.velocities.push_back({r[4], r[5], r[6]});
            sv.quaternions.push_back({a[0], a[1], a[2], a[3]});
            sv.angular_rates.push_back({a[4], a[5], a[6]});
            sv.attitudes.push_back({a[7], a[8], a[9]});
        }
        return sv;
    }

    // Data formats A/B/C: "reference" (default; the reference's samples) or
    // "fields" (each sample from its own bits), see s1g_set_abc_decode.
    void set_abc_decode(const std::string& mode) {
        if (mode != "reference" && mode != "fields") throw std::invalid_argument("mode must be reference or fields");
        check(s1g_set_abc_decode(handle(), mode == "fields" ? S1G_ABC_FIELDS : S1G_ABC_REFERENCE));
    }

    // Cross-check the product's index / annotation sidecars (either path may
    // be empty) against the packets the GPU indexer found; throws
    // std::runtime_error describing the first disagreement.
    s1g_sidecar_report check_sidecars(const std::string& index_path, const std::string& annotation_path) {
        s1g_sidecar_report rep;
        check(s1g_check_sidecars(handle(), index_path.empty() ? nullptr : index_path.c_str(),
                                 annotation_path.empty() ? nullptr : annotation_path.c_str(), &rep));
        return rep;
    }

    [[nodiscard]] CF_VEC_2D get_burst(const std::string& swath, const int& burst) {
        return burst_product(swath, burst, S1G_RAW);
    }
    [[nodiscard]] CF_VEC_2D get_swath(const std::string& swath) { return swath_product(swath, S1G_RAW); }

    [[nodiscard]] CF_VEC_2D get_range_compressed_burst(const std::string& swath, const int& burst,
                                                       const bool& range_doppler = false) {
        return burst_product(swath, burst, range_doppler ? S1G_RANGE_DOPPLER : S1G_RANGE_COMPRESSED);
    }
    [[nodiscard]] CF_VEC_2D get_range_compressed_swath(const std::string& swath, const bool& range_doppler = false) {
        return swath_product(swath, range_doppler ? S1G_RANGE_DOPPLER : S1G_RANGE_COMPRESSED);
    }

    [[nodiscard]] CF_VEC_2D get_azimuth_compressed_burst(const std::string& swath, const int& burst) {
        return burst_product(swath, burst, S1G_AZIMUTH_COMPRESSED);
    }
    [[nodiscard]] CF_VEC_2D get_azimuth_compressed_swath(const std::string& swath) {
        return swath_product(swath, S1G_AZIMUTH_COMPRESSED);
    }

    // Contiguous complex<float> products (level: S1G_RAW ... S1G_AZIMUTH_COMPRESSED).
    [[nodiscard]] S1G_CF32_PRODUCT get_burst_cf32(const std::string& swath, int burst, int level) {
        validate(swath, burst);
        S1G_CF32_PRODUCT p;
        check(s1g_burst_shape(handle(), swath.c_str(), burst, level, &p.rows, &p.cols));
        p.data.resize((size_t)(p.rows * p.cols));
        check(s1g_burst_product(handle(), swath.c_str(), burst, level, p.data.data(), p.rows, p.cols, S1G_CF32, 0));
        return p;
    }
    // The swath as the reference's save_swath_as_cf32 writes it
    // (image_write_main.cpp:302-315): every row as wide as the first row
    // (longer rows cut, shorter rows zero-filled, where the reference reads
    // past the end of the shorter row).
    [[nodiscard]] S1G_CF32_PRODUCT get_swath_cf32(const std::string& swath, int level) {
        validate(swath, 0);
        S1G_CF32_PRODUCT p;
        int64_t wide = 0;
        check(s1g_swath_shape(handle(), swath.c_str(), level, &p.rows, &wide));
        p.data.resize((size_t)(p.rows * wide));
        check(s1g_swath_product(handle(), swath.c_str(), level, p.data.data(), p.rows, wide, S1G_CF32, 0));
        const std::vector<int64_t> w = row_widths(swath, level);
        p.cols = w.empty() ? wide : w[0];
        if (p.cols != wide) {
            for (int64_t r = 0; r < p.rows; ++r)
                std::copy(p.data.begin() + r * wide, p.data.begin() + r * wide + std::min(p.cols, wide),
                          p.data.begin() + r * p.cols);
            p.data.resize((size_t)(p.rows * p.cols));
        }
        return p;
    }

    // Scaled float32 image of a product, formed and scaled on the GPU (the
    // data of s1_write's TIFF commands; scaling: real, imag, mag, norm,
    // norm_log).  burst < 0 selects the swath product.
    [[nodiscard]] std::vector<float> get_image(const std::string& swath, int burst, int level,
                                               const std::string& scaling, int64_t& rows, int64_t& cols) {
        int mode = -1;
        const char* names[] = {"real", "imag", "mag", "norm", "norm_log"};
        for (int i = 0; i < 5; ++i)
            if (scaling == names[i]) mode = i;
        if (mode < 0) throw std::invalid_argument(scaling + " is not a valid scaling mode.");
        validate(swath, burst < 0 ? 0 : burst);
        if (burst >= 0) check(s1g_burst_shape(handle(), swath.c_str(), burst, level, &rows, &cols));
        else check(s1g_swath_shape(handle(), swath.c_str(), level, &rows, &cols));
        std::vector<float> img((size_t)(rows * cols));
        if (burst >= 0)
            check(s1g_burst_image(handle(), swath.c_str(), burst, level, mode, img.data(), rows, cols, 0));
        else
            check(s1g_swath_image(handle(), swath.c_str(), level, mode, img.data(), rows, cols, 0));
        return img;
    }

    // Scaled image of spectrogram() of one echo line (signal_processing.cpp:
    // 794-844; s1_write uses fft_size 64, stride 32), on the GPU.
    [[nodiscard]] std::vector<float> get_spectrogram_image(const std::string& swath, int burst, int azimuth_line,
                                                           const std::string& scaling, int64_t& rows, int64_t& cols,
                                                           int fft_size = 64, int stride = 32) {
        int mode = -1;
        const char* names[] = {"real", "imag", "mag", "norm", "norm_log"};
        for (int i = 0; i < 5; ++i)
            if (scaling == names[i]) mode = i;
        if (mode < 0) throw std::invalid_argument(scaling + " is not a valid scaling mode.");
        validate(swath, burst);
        check(s1g_spectrogram_shape(handle(), swath.c_str(), burst, fft_size, stride, &rows, &cols));
        std::vector<float> img((size_t)(rows * cols));
        check(s1g_spectrogram_image(handle(), swath.c_str(), burst, azimuth_line, fft_size, stride, mode, img.data(),
                                    rows, cols, 0));
        return img;
    }

    // BigTIFF float32 file with the reference's layout (_write_tif).
    static void write_tiff(const std::string& path, const std::vector<float>& img, int64_t rows, int64_t cols) {
        if (s1g_write_tiff(path.c_str(), img.data(), rows, cols) != S1G_OK)
            throw std::runtime_error("Unable to write " + path);
    }

    s1g_decoder* handle() const {
        if (!_h) throw std::runtime_error("S1_Decoder: no file opened");
        return _h;
    }

  private:
    std::string _filename;
    s1g_decoder* _h = nullptr;
    int _det = 0, _mit = 0;
    bool _eccm_set = false;

    static CF_VEC_2D to_vec2d(const std::vector<std::complex<double>>& flat, int64_t rows, int64_t cols) {
        CF_VEC_2D out((size_t)rows);
        for (int64_t r = 0; r < rows; ++r) out[r].assign(flat.begin() + r * cols, flat.begin() + (r + 1) * cols);
        return out;
    }

    CF_VEC_2D burst_product(const std::string& swath, int burst, int level) {
        validate(swath, burst);
        int64_t rows = 0, cols = 0;
        check(s1g_burst_shape(handle(), swath.c_str(), burst, level, &rows, &cols));
        std::vector<std::complex<double>> flat((size_t)(rows * cols));
        check(s1g_burst_product(handle(), swath.c_str(), burst, level, flat.data(), rows, cols, S1G_CF64, 0));
        return to_vec2d(flat, rows, cols);
    }

    CF_VEC_2D swath_product(const std::string& swath, int level) {
        validate(swath, 0);
        int64_t rows = 0, cols = 0;
        check(s1g_swath_shape(handle(), swath.c_str(), level, &rows, &cols));
        std::vector<std::complex<double>> flat((size_t)(rows * cols));
        check(s1g_swath_product(handle(), swath.c_str(), level, flat.data(), rows, cols, S1G_CF64, 0));
        CF_VEC_2D out = to_vec2d(flat, rows, cols);
        // rows keep the reference's lengths (bursts / blocks of different widths)
        const std::vector<int64_t> w = row_widths(swath, level);
        for (size_t r = 0; r < out.size() && r < w.size(); ++r) out[r].resize((size_t)w[r]);
        return out;
    }

    std::vector<int64_t> row_widths(const std::string& swath, int level) {
        int64_t rows = 0;
        check(s1g_swath_row_widths(handle(), swath.c_str(), level, nullptr, 0, &rows));
        std::vector<int64_t> w((size_t)rows);
        check(s1g_swath_row_widths(handle(), swath.c_str(), level, w.data(), rows, &rows));
        return w;
    }

    // _validate_request (s1_decoder.cpp:45-89): messages and exit status of the reference.
    void validate(const std::string& swath, int burst) {
        int n = 0;
        const int st = s1g_num_bursts(handle(), swath.c_str(), &n);
        if (st == S1G_E_BAD_SWATH) {
            std::string names(4096, '\0');
            s1g_swath_names(handle(), &names[0], names.size());
            names.resize(names.find('\0'));
#ifdef S1G_FACADE_THROW
            throw std::out_of_range("The requested swath, " + swath + ", does not exist in the data.");
#else
            std::cout << "The requested swath, " << swath << ", does not exist in the data."
                      << " The available swaths are: " << std::endl;
            size_t pos = 0;
            while (pos < names.size()) {
                size_t e = names.find('\n', pos);
                if (e == std::string::npos) e = names.size();
                const std::string line = names.substr(pos, e - pos);
                if (!line.empty()) std::cout << line.substr(0, line.find(' ')) << std::endl;
                pos = e + 1;
            }
            std::exit(1);
#endif
        }
        check(st);
        if (burst && (burst < 0 || burst >= n)) {
#ifdef S1G_FACADE_THROW
            throw std::out_of_range("The requested burst, " + std::to_string(burst) + ", does not exist in the data.");
#else
            std::cout << "The requested burst, " << burst << ", does not exist in the data."
                      << " There are " << n << " bursts in swath " << swath << "." << std::endl;
            std::exit(1);
#endif
        }
    }

    void check(int st) const {
        if (st == S1G_OK) return;
        const std::string msg = _h ? s1g_last_error(_h) : std::string("s1g error ") + std::to_string(st);
        switch (st) {
            case S1G_E_INVALID_ARGUMENT:
            case S1G_E_BUFFER:
                throw std::invalid_argument(msg);
            case S1G_E_UNSUPPORTED:
                throw std::domain_error(msg);
            case S1G_E_BAD_SWATH:
            case S1G_E_BAD_BURST:
                throw std::out_of_range(msg);
            default:
                throw std::runtime_error(msg);
        }
    }
};
