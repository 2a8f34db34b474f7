// s1g_write: the raw-output commands of the reference's s1_write binary
// (image_write_main.cpp:186-324, 328-393) on the GPU path, through the
// header-only S1_Decoder facade.
//
//   s1g_write save_burst_as_cf32 [swath] [burst_num] [processing_level] [in_path] [out_path]
//   s1g_write save_swath_as_cf32 [swath] [processing_level] [in_path] [out_path]
//
// processing_level: raw, range_compressed, range_doppler, azimuth_compressed
// (case-insensitive).  The output is the reference's file format: row-major
// complex<float> (re, im) with no header, and the same "Num Rows / Num Cols /
// Data successfully saved" console lines.  Options (anywhere after the
// command): --fp64 or --fp32_plain select the GPU arithmetic (default: the
// fused FP32 path); --eccm DET MIT enables the RFI notch first.
//
// The TIFF-writing commands of s1_write (burst, swath, *_compressed_*,
// spectrogram) print that they are not available in this build and exit 1.
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
        "save_burst_as_cf32 [swath] [burst_num] [processing_level] [in_path] [out_path]",
        "save_swath_as_cf32 [swath] [processing_level] [in_path] [out_path]",
        "Options: [--fp64|--fp32_plain] [--eccm detection_threshold mitigation_threshold]",
    };
    for (const char* l : lines) std::cout << l << std::endl;
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
    bool eccm = false;
    int det = 0, mit = 0;
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--fp64") precision = "fp64";
        else if (a == "--fp32_plain") precision = "fp32_plain";
        else if (a == "--fp32") precision = "fp32";
        else if (a == "--eccm" && i + 2 < argc) {
            eccm = true;
            det = std::stoi(argv[++i]);
            mit = std::stoi(argv[++i]);
        } else pos.push_back(a);
    }
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
        const char* tiff[] = {"burst", "swath", "spectrogram", "range_compressed_burst", "range_compressed_swath",
                              "range_doppler_burst", "range_doppler_swath", "azimuth_compressed_burst",
                              "azimuth_compressed_swath", "azimuth_compressed_burst_eccm",
                              "azimuth_compressed_swath_eccm"};
        for (const char* t : tiff)
            if (command == t) {
                std::cout << command << " writes a TIFF image, which this build does not provide; use "
                          << "save_burst_as_cf32 / save_swath_as_cf32." << std::endl;
                return 1;
            }
        std::cout << command << " is not a valid command." << std::endl;
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "terminate called after throwing an instance of an exception" << std::endl;
        std::cerr << "  what():  " << e.what() << std::endl;
        return 134;
    }
}
