// Driver around the reference's own S1_Decoder, compiled from the reference
// sources by oracle/Makefile.  TEST INFRASTRUCTURE ONLY: it produces the FP64
// golden products that pin the oracle restatement and the CUDA path.
//
// The cf32 write loop of image_write_main.cpp:232-245 is replaced by a raw
// FP64 dump (libtiff is absent, and the goldens keep full precision).
//
// usage:
//   ref_driver product <dat> <swath> <burst|-1> <raw|range_compressed|range_doppler|azimuth_compressed> <out> [det mit]
//   ref_driver headers <dat> <out.txt>
//   ref_driver state_vectors <dat> <out.txt>
//   ref_driver doppler <dat> <swath> <burst> <out.txt>
//   ref_driver bursts <dat> <swath>
//   ref_driver attitude <dat> <out.txt>        (STATE_VECTORS of print_state_vectors, all members)
//   ref_driver sidecars <index.dat> <annot.dat> <out.txt>
//   ref_driver eccm_raw <dat> <swath> <burst> <det> <mit> <out>
//        the decoded burst after the reference's own eccm() (fft 128, stride
//        64, as _range_compress calls it, s1_decoder.cpp:470-474)
//   ref_driver scale <dat> <swath> <burst> <level> <mode> <out>
//        scale(CF_VEC_2D, mode) of a burst product (the TIFF commands' data,
//        image_write.cpp:29-40): "S1GF" magic, int64 rows, int64 cols, floats
//   ref_driver spectrogram <dat> <swath> <burst> <line> <fft_size> <stride> <out>
//        spectrogram() of one decoded echo line (image_write.cpp:43-64)
//   ref_driver sinc <in.bin> <L> <out>
//        sinc_interpolate(signal, t, L) (signal_processing.cpp:238-257) at
//        every t: in.bin = int64 n, n complex<double>, int64 m, m doubles;
//        out = m complex<double>
// Output of `product`: "S1GR" magic, int64 rows, then per row int64 len and
// len complex<double> values (rows may be ragged for swath products).
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>

#include "aux_decoding.h"
#include "s1_decoder.h"

static void dump(const CF_VEC_2D& d, const std::string& path) {
    std::ofstream f(path, std::ios::binary);
    const char magic[4] = {'S', '1', 'G', 'R'};
    f.write(magic, 4);
    int64_t rows = (int64_t)d.size();
    f.write(reinterpret_cast<const char*>(&rows), 8);
    for (const auto& r : d) {
        int64_t len = (int64_t)r.size();
        f.write(reinterpret_cast<const char*>(&len), 8);
        f.write(reinterpret_cast<const char*>(r.data()), len * sizeof(std::complex<double>));
    }
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: see header" << std::endl;
        return 2;
    }
    std::string cmd = argv[1];
    std::cout << std::setprecision(17);
    if (cmd == "product") {
        std::string dat = argv[2], swath = argv[3];
        int burst = std::stoi(argv[4]);
        std::string level = argv[5], out = argv[6];
        auto t0 = std::chrono::steady_clock::now();
        S1_Decoder s1(dat);
        auto t1 = std::chrono::steady_clock::now();
        if (argc > 8) s1.apply_eccm(std::stoi(argv[7]), std::stoi(argv[8]));
        CF_VEC_2D data;
        if (burst >= 0) {
            if (level == "raw") data = s1.get_burst(swath, burst);
            else if (level == "range_compressed") data = s1.get_range_compressed_burst(swath, burst);
            else if (level == "range_doppler") data = s1.get_range_compressed_burst(swath, burst, true);
            else if (level == "azimuth_compressed") data = s1.get_azimuth_compressed_burst(swath, burst);
        } else {
            if (level == "raw") data = s1.get_swath(swath);
            else if (level == "range_compressed") data = s1.get_range_compressed_swath(swath);
            else if (level == "range_doppler") data = s1.get_range_compressed_swath(swath, true);
            else if (level == "azimuth_compressed") data = s1.get_azimuth_compressed_swath(swath);
        }
        auto t2 = std::chrono::steady_clock::now();
        dump(data, out);
        std::cerr << "TIMING open_s " << std::chrono::duration<double>(t1 - t0).count()
                  << " product_s " << std::chrono::duration<double>(t2 - t1).count() << std::endl;
        return 0;
    }
    if (cmd == "headers") {
        std::ifstream data = open_file(argv[2]);
        PACKET_VEC_1D packets = get_packets(data, 0);
        std::ofstream o(argv[3]);
        o << std::setprecision(17);
        for (auto& p : packets) {
            for (const auto& k : PRIMARY_HEADER_FIELDS) o << k << "=" << p.primary_header(k) << " ";
            for (const auto& k : SECONDARY_HEADER_FIELDS) o << k << "=" << p.secondary_header(k) << " ";
            o << "pri_us=" << p.get_pri() << " pulse_length_us=" << p.get_pulse_length()
              << " txprr=" << p.get_tx_ramp_rate() << " txpsf=" << p.get_start_frequency()
              << " swst_us=" << p.get_swst() << " swl_us=" << p.get_swl() << " rx_gain_db=" << p.get_rx_gain()
              << " time=" << p.get_time() << " swath=" << p.get_swath()
              << " replica_len=" << p.get_replica_chirp_length() << "\n";
        }
        return 0;
    }
    if (cmd == "state_vectors") {
        S1_Decoder s1(argv[2]);
        STATE_VECTORS sv = s1.get_state_vectors();
        std::ofstream o(argv[3]);
        o << std::setprecision(17);
        for (size_t i = 0; i < sv.times.size(); ++i) {
            o << sv.times[i];
            for (int c = 0; c < 3; ++c) o << " " << sv.positions[i][c];
            for (int c = 0; c < 3; ++c) o << " " << sv.velocities[i][c];
            o << "\n";
        }
        return 0;
    }
    if (cmd == "doppler") {
        std::string dat = argv[2], swath = argv[3];
        int burst = std::stoi(argv[4]);
        S1_Decoder s1(dat);
        STATE_VECTORS sv = s1.get_state_vectors();
        CF_VEC_2D rc = s1.get_range_compressed_burst(swath, burst);
        // Same packet list as S1_Decoder::get_azimuth_compressed_burst.
        PACKET_VEC_2D bursts = get_packets_in_bursts(dat, swath);
        PACKET_VEC_1D& pk = bursts[burst];
        D_VEC_1D v0 = sv.velocities[0];
        double v_norm = std::sqrt(std::pow(v0[0], 2.0) + std::pow(v0[1], 2.0) + std::pow(v0[2], 2.0));
        double prf = 1.0 / (pk[0].get_pri() * 1e-6);
        double T = double(pk.size()) / prf;
        double rate = get_doppler_centroid_rate(pk, v_norm);
        D_VEC_1D dc = get_doppler_centroid(rc, rate, T, pk[0], 30);
        std::ofstream o(argv[5]);
        o << std::setprecision(17) << "rate " << rate << "\n";
        for (double v : dc) o << v << "\n";
        return 0;
    }
    if (cmd == "attitude") {
        // print_main.cpp:17-23: the state vectors of every packet in the file
        PACKET_VEC_1D packets = get_packets(std::string(argv[2]), 0);
        STATE_VECTORS sv(packets);
        std::ofstream o(argv[3]);
        o << std::setprecision(17);
        for (size_t i = 0; i < sv.times.size(); ++i) {
            o << sv.times[i];
            for (double x : sv.positions[i]) o << " " << x;
            for (double x : sv.velocities[i]) o << " " << x;
            for (double x : sv.quaternions[i]) o << " " << x;
            for (double x : sv.angular_rates[i]) o << " " << x;
            for (double x : sv.attitudes[i]) o << " " << x;
            o << "\n";
        }
        return 0;
    }
    if (cmd == "sidecars") {
        // aux_decoding.cpp:61-145: every field of every record, then the
        // annotation times
        std::ofstream o(argv[4]);
        o << std::setprecision(17);
        const char* ik[] = {"date_time", "time_delta", "data_size", "unit_offset", "byte_offset", "variable_flag",
                            "spare_data"};
        for (auto& r : index_decoder(std::string(argv[2]))) {
            o << "index";
            for (const char* k : ik) o << " " << r[k];
            o << "\n";
        }
        const char* ak[] = {"days_ul", "milliseconds_ul", "microseconds_ul", "days_dl", "milliseconds_dl",
                            "microseconds_dl", "packet_length", "num_transfer_frames", "error_flag", "bit_1_type",
                            "bit_2_type", "bit_6_type", "spare_field"};
        for (auto& r : annotation_decoder(std::string(argv[3]))) {
            o << "annot";
            for (const char* k : ak) o << " " << r[k];
            o << "\n";
        }
        for (double t : annotation_time_decoder(std::string(argv[3]))) o << "time " << t << "\n";
        return 0;
    }
    if (cmd == "eccm_raw") {
        S1_Decoder s1(argv[2]);
        const int burst = std::stoi(argv[4]);
        CF_VEC_2D raw = s1.get_burst(argv[3], burst);
        PACKET_VEC_2D bursts = get_packets_in_bursts(argv[2], argv[3]);
        const char rx_pol = bursts[burst][0].get_rx_polarization();
        eccm(raw, 128, 64, std::stoi(argv[5]), std::stoi(argv[6]), rx_pol);
        dump(raw, argv[7]);
        return 0;
    }
    if (cmd == "scale") {
        std::string dat = argv[2], swath = argv[3], level = argv[5];
        const int burst = std::stoi(argv[4]);
        S1_Decoder s1(dat);
        CF_VEC_2D data;
        if (level == "raw") data = s1.get_burst(swath, burst);
        else if (level == "range_compressed") data = s1.get_range_compressed_burst(swath, burst);
        else if (level == "range_doppler") data = s1.get_range_compressed_burst(swath, burst, true);
        else data = s1.get_azimuth_compressed_burst(swath, burst);
        std::vector<float> img = scale(data, argv[6]);
        std::ofstream f(argv[7], std::ios::binary);
        const char magic[4] = {'S', '1', 'G', 'F'};
        f.write(magic, 4);
        int64_t rows = (int64_t)data.size(), cols = (int64_t)data[0].size();
        f.write(reinterpret_cast<const char*>(&rows), 8);
        f.write(reinterpret_cast<const char*>(&cols), 8);
        f.write(reinterpret_cast<const char*>(img.data()), (std::streamsize)(img.size() * sizeof(float)));
        return 0;
    }
    if (cmd == "spectrogram") {
        S1_Decoder s1(argv[2]);
        CF_VEC_2D burst = s1.get_burst(argv[3], std::stoi(argv[4]));
        CF_VEC_2D sg = spectrogram(burst[std::stoi(argv[5])], std::stoi(argv[6]), std::stoi(argv[7]));
        dump(sg, argv[8]);
        return 0;
    }
    if (cmd == "sinc") {
        std::ifstream f(argv[2], std::ios::binary);
        int64_t n = 0, m = 0;
        f.read(reinterpret_cast<char*>(&n), 8);
        CF_VEC_1D sig((size_t)n);
        f.read(reinterpret_cast<char*>(sig.data()), n * (std::streamsize)sizeof(std::complex<double>));
        f.read(reinterpret_cast<char*>(&m), 8);
        std::vector<double> t((size_t)m);
        f.read(reinterpret_cast<char*>(t.data()), m * (std::streamsize)sizeof(double));
        const int L = std::stoi(argv[3]);
        CF_VEC_2D out(1, CF_VEC_1D((size_t)m));
        for (int64_t i = 0; i < m; ++i) out[0][(size_t)i] = sinc_interpolate(sig, t[(size_t)i], L);
        dump(out, argv[4]);
        return 0;
    }
    if (cmd == "bursts") {
        PACKET_VEC_2D bursts = get_packets_in_bursts(argv[2], argv[3]);
        for (auto& b : bursts) std::cout << b.size() << " " << 2 * b[0].get_num_quads() << "\n";
        return 0;
    }
    std::cerr << "unknown command" << std::endl;
    return 2;
}
