// s1g_write: the commands of the reference's s1_write binary
// (image_write_main.cpp:1-393) on the GPU path, through the header-only
// S1_Decoder facade.
//
//   s1g_write burst [swath] [burst_num] [in_path] [out_path]
//   s1g_write swath [swath] [in_path] [out_path]
//   s1g_write range_compressed_burst | range_doppler_burst | azimuth_compressed_burst
//             [swath] [burst_num] [in_path] [out_path]
//   s1g_write range_compressed_swath | range_doppler_swath | azimuth_compressed_swath
//             [swath] [in_path] [out_path]
//   s1g_write azimuth_compressed_burst_eccm [swath] [burst_num] [det] [mit] [in_path] [out_path]
//   s1g_write azimuth_compressed_swath_eccm [swath] [det] [mit] [in_path] [out_path]
//   s1g_write save_burst_as_cf32 [swath] [burst_num] [processing_level] [in_path] [out_path]
//   s1g_write save_swath_as_cf32 [swath] [processing_level] [in_path] [out_path]
//   s1g_write spectrogram [swath] [burst_num] [azimuth_line] [in_path] [out_path]
//
// TIFF commands write a BigTIFF float32 image (bottom-up rows, as
// _write_tif, image_write.cpp:3-25) scaled by --real (default), --imag,
// --mag, --norm or --norm_log (scale(), signal_processing.cpp:1031-1071;
// with several flags the priority of parse_scaling_mode), the scaling done
// on the GPU.  cf32 commands write row-major
// complex<float> with no header.  processing_level: raw, range_compressed,
// range_doppler, azimuth_compressed (case-insensitive).  Extra options:
// --fp64 or --fp32_plain select the GPU arithmetic (default: the fused FP32
// path); --eccm DET MIT enables the RFI notch for the cf32 commands.
#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "s1_decoder_gb300.hpp"

namespace {

int level_of(std::string proc) {
    std::transform(proc.begin(), proc.end(), proc.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (proc == "raw") return S1G_RAW;
    if (proc == "range_compressed") return S1G_RANGE_COMPRESSED;
    if (proc == "range_doppler") return S1G_RANGE_DOPPLER;
    if (proc == "azimuth_compressed") return S1G_AZIMUTH_COMPRESSED;
    throw std::invalid_argument(
        "Invalid processing_level. Options are raw, range_compressed, range_doppler, or azimuth_compressed.");
}

void print_help() {
    const char* lines[] = {
        "burst [swath] [burst_num] [in_path] [out_path]",
        "swath [swath] [in_path] [out_path]",
        "range_compressed_burst [swath] [burst_num] [in_path] [out_path]",
        "range_compressed_swath [swath] [in_path] [out_path]",
        "range_doppler_burst [swath] [burst_num] [in_path] [out_path]",
        "range_doppler_swath [swath] [in_path] [out_path]",
        "azimuth_compressed_burst [swath] [burst_num] [in_path] [out_path]",
        "azimuth_compressed_swath [swath] [in_path] [out_path]",
        "azimuth_compressed_burst_eccm [swath] [burst_num] [detection_threshold] [mitigation_threshold] [in_path] "
        "[out_path]",
        "azimuth_compressed_swath_eccm [swath] [detection_threshold] [mitigation_threshold] [in_path] [out_path]",
        "save_burst_as_cf32 [swath] [burst_num] [processing_level] [in_path] [out_path]",
        "save_swath_as_cf32 [swath] [processing_level] [in_path] [out_path]",
        "spectrogram [swath] [burst_num] [azimuth_line] [in_path] [out_path]",
        "Scaling Options: [--norm_log|--norm|--mag|--real|--imag]",
        "Options: [--fp64|--fp32_plain] [--eccm detection_threshold mitigation_threshold]",
    };
    for (const char* l : lines) std::cout << l << std::endl;
}

// One TIFF command: product level, burst (-1 = swath) and optional ECCM.
int write_image(S1_Decoder& s1, const std::string& swath, int burst, int level, const std::string& scaling,
                const std::string& out_path) {
    int64_t rows = 0, cols = 0;
    const std::vector<float> img = s1.get_image(swath, burst, level, scaling, rows, cols);
    std::cout << "Num Rows: " << rows << std::endl;
    std::cout << "Num Cols: " << cols << std::endl;
    S1_Decoder::write_tiff(out_path, img, rows, cols);
    std::cout << "Image written to " << out_path << "." << std::endl;
    return 0;
}

int write_cf32(const S1G_CF32_PRODUCT& p, const std::string& out_path) {
    std::ofstream file(out_path, std::ios::binary);
    if (!file) {
        std::cerr << "Error: Unable to open file " << out_path << " for writing." << std::endl;
        return 0;
    }
    std::cout << "Num Rows: " << p.rows << std::endl;
    std::cout << "Num Cols: " << p.cols << std::endl;
    file.write(reinterpret_cast<const char*>(p.data.data()),
               (std::streamsize)(p.data.size() * sizeof(std::complex<float>)));
    file.close();
    if (!file) std::cerr << "Error: Failed to write to file " << out_path << "." << std::endl;
    else std::cout << "Data successfully saved to " << out_path << "." << std::endl;
    return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
    if (argc < 2) {
        std::cout << "Please enter a command:" << std::endl;
        print_help();
        return 1;
    }
    const std::string command = argv[1];
    std::vector<std::string> pos;
    std::string precision = "fp32";
    std::string scaling = "real";
    std::vector<std::string> flags;
    bool eccm = false;
    int det = 0, mit = 0;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--norm_log" || a == "--norm" || a == "--mag" || a == "--real" || a == "--imag") {
            flags.push_back(a.substr(2));
        } else if (a == "--fp64") precision = "fp64";
        else if (a == "--fp32_plain") precision = "fp32_plain";
        else if (a == "--fp32") precision = "fp32";
        else if (a == "--eccm" && i + 2 < argc) {
            eccm = true;
            det = std::stoi(argv[++i]);
            mit = std::stoi(argv[++i]);
        } else pos.push_back(a);
    }
    // parse_scaling_mode (cli.cpp:68-80): norm_log, norm, mag, real, imag in that priority; default real
    for (const char* m : {"imag", "real", "mag", "norm", "norm_log"})
        if (std::find(flags.begin(), flags.end(), m) != flags.end()) scaling = m;
    if (command == "help" || command == "--help" || command == "-h") {
        print_help();
        return 0;
    }
    try {
        if (command == "save_burst_as_cf32") {
            if (pos.size() != 5) {
                std::cout << "save_burst_as_cf32 expects [swath] [burst_num] [processing_level] [in_path] [out_path]"
                          << std::endl;
                return 1;
            }
            const int level = level_of(pos[2]);
            S1_Decoder s1(pos[3]);
            s1.set_precision(precision);
            if (eccm) s1.apply_eccm(det, mit);
            return write_cf32(s1.get_burst_cf32(pos[0], std::stoi(pos[1]), level), pos[4]);
        }
        if (command == "save_swath_as_cf32") {
            if (pos.size() != 4) {
                std::cout << "save_swath_as_cf32 expects [swath] [processing_level] [in_path] [out_path]" << std::endl;
                return 1;
            }
            const int level = level_of(pos[1]);
            S1_Decoder s1(pos[2]);
            s1.set_precision(precision);
            if (eccm) s1.apply_eccm(det, mit);
            return write_cf32(s1.get_swath_cf32(pos[0], level), pos[3]);
        }
        struct Cmd {
            const char* name;
            int level;
            bool burst, eccm;
        };
        const Cmd cmds[] = {
            {"burst", S1G_RAW, true, false},
            {"swath", S1G_RAW, false, false},
            {"range_compressed_burst", S1G_RANGE_COMPRESSED, true, false},
            {"range_compressed_swath", S1G_RANGE_COMPRESSED, false, false},
            {"range_doppler_burst", S1G_RANGE_DOPPLER, true, false},
            {"range_doppler_swath", S1G_RANGE_DOPPLER, false, false},
            {"azimuth_compressed_burst", S1G_AZIMUTH_COMPRESSED, true, false},
            {"azimuth_compressed_swath", S1G_AZIMUTH_COMPRESSED, false, false},
            {"azimuth_compressed_burst_eccm", S1G_AZIMUTH_COMPRESSED, true, true},
            {"azimuth_compressed_swath_eccm", S1G_AZIMUTH_COMPRESSED, false, true},
        };
        for (const Cmd& c : cmds) {
            if (command != c.name) continue;
            const size_t want = 3 + (c.burst ? 1 : 0) + (c.eccm ? 2 : 0);
            if (pos.size() != want) {
                std::cout << command << " expects " << want << " arguments (see help)" << std::endl;
                return 1;
            }
            size_t k = 0;
            const std::string swath = pos[k++];
            const int burst = c.burst ? std::stoi(pos[k++]) : -1;
            int d = 0, m = 0;
            if (c.eccm) {
                d = std::stoi(pos[k++]);
                m = std::stoi(pos[k++]);
            }
            const std::string in_path = pos[k++], out_path = pos[k++];
            S1_Decoder s1(in_path);
            s1.set_precision(precision);
            if (c.eccm) s1.apply_eccm(d, m);
            else if (eccm) s1.apply_eccm(det, mit);
            return write_image(s1, swath, burst, c.level, scaling, out_path);
        }
        if (command == "spectrogram") {
            // spectrogram [swath] [burst_num] [azimuth_line] [in_path] [out_path] (image_write.cpp:44-66)
            if (pos.size() != 5) {
                std::cout << "spectrogram expects [swath] [burst_num] [azimuth_line] [in_path] [out_path]" << std::endl;
                return 1;
            }
            S1_Decoder s1(pos[3]);
            s1.set_precision(precision);
            int64_t rows = 0, cols = 0;
            const std::vector<float> img =
                s1.get_spectrogram_image(pos[0], std::stoi(pos[1]), std::stoi(pos[2]), scaling, rows, cols);
            std::cout << "Num Rows: " << rows << std::endl;
            std::cout << "Num Cols: " << cols << std::endl;
            S1_Decoder::write_tiff(pos[4], img, rows, cols);
            std::cout << "Image written to " << pos[4] << "." << std::endl;
            return 0;
        }
        std::cout << command << " is not a valid command." << std::endl;
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "terminate called after throwing an instance of an exception" << std::endl;
        std::cerr << "  what():  " << e.what() << std::endl;
        return 134;
    }
}
