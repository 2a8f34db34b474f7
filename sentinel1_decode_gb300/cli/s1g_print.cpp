// s1g_print: the commands of the reference's s1_print binary
// (print_main.cpp:50-158) over the C ABI, with the same arguments, argument
// checks (validate_args, cli.cpp:26-64) and printouts:
//
//   s1g_print packet_info [packet_index] [path]
//   s1g_print complex_samples [packet_index] [path]
//   s1g_print swath_names [path]
//   s1g_print index_records [path]
//   s1g_print annotation_record [record_index] [path]
//   s1g_print state_vectors [path]
//
// Packets are indexed and decoded on the GPU; the sidecar commands are host
// only.  swath_names prints swaths in the order they first occur (the
// reference prints an unordered_map, whose order is unspecified).  An
// exception the reference would leave uncaught (an index past the end)
// prints its message and exits with 134, like the reference's abort.
#include <complex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "s1g.h"

namespace {

const char* kHelp[] = {
    "packet_info [packet_index] [path]",
    "complex_samples [packet_index] [path]",
    "swath_names [path]",
    "index_records [path]",
    "annotation_record [record_index] [path]",
    "state_vectors [path]",
};

void print_help() {
    for (const char* l : kHelp) std::cout << l << std::endl;
}

// validate_args: every argument present, ints parse, paths open
void validate(const std::string& cmd, const std::vector<std::pair<const char*, const char*>>& spec, int argc,
              char** argv) {
    for (size_t k = 0; k < spec.size(); ++k) {
        const int i = 2 + (int)k;
        if (i >= argc) {
            std::cout << cmd << " is missing the following argument: " << spec[k].first << std::endl;
            std::exit(1);
        }
        bool ok = true;
        if (!strcmp(spec[k].second, "int")) {
            try {
                (void)std::stoi(argv[i]);
            } catch (...) {
                ok = false;
            }
        } else if (!strcmp(spec[k].second, "path")) {
            std::ifstream f(argv[i], std::ios::binary);
            ok = f.is_open();
        }
        if (!ok) {
            std::cout << argv[i] << " is not a valid " << spec[k].first;
            if (!strcmp(spec[k].second, "path")) std::cout << " or the file may not exist";
            std::cout << std::endl;
            std::exit(1);
        }
    }
}

struct Handle {
    s1g_decoder* h = nullptr;
    explicit Handle(const char* path) {
        const int rc = s1g_open_file(path, 0, &h);
        if (rc != S1G_OK) throw std::runtime_error(std::string("Unable to open ") + path);
    }
    ~Handle() {
        if (h) s1g_close(h);
    }
    void check(int rc) const {
        if (rc != S1G_OK) throw std::runtime_error(s1g_last_error(h));
    }
    int64_t packets() const {
        int64_t n = 0;
        check(s1g_num_packets(h, &n));
        return n;
    }
};

void packet_info(const char* path, int index) {
    Handle d(path);
    if (index < 0 || index >= d.packets()) throw std::out_of_range("Index is greater than the number of packets.");
    size_t need = 0;
    d.check(s1g_packet_info(d.h, index, nullptr, 0, &need));
    std::string buf(need, '\0');
    d.check(s1g_packet_info(d.h, index, &buf[0], need, &need));
    std::cout << buf.c_str();
}

void complex_samples(const char* path, int index) {
    Handle d(path);
    if (index < 0 || index >= d.packets()) throw std::out_of_range("Index is greater than the number of packets.");
    int64_t nq = 0;
    d.check(s1g_packet_field(d.h, index, "num_quadratures", &nq));
    std::vector<std::complex<double>> s((size_t)(2 * nq));
    d.check(s1g_packet_samples(d.h, index, s.data(), 2 * nq, S1G_CF64, 0));
    for (const auto& x : s) std::cout << x << std::endl;
}

void swath_names(const char* path) {
    Handle d(path);
    std::string buf(1 << 16, '\0');
    d.check(s1g_swath_names(d.h, &buf[0], buf.size()));
    // "NAME count" lines -> "NAME: count"
    std::string line;
    for (const char* c = buf.c_str();; ++c) {
        if (*c == '\n' || *c == 0) {
            const size_t sp = line.rfind(' ');
            if (sp != std::string::npos) std::cout << line.substr(0, sp) << ": " << line.substr(sp + 1) << std::endl;
            line.clear();
            if (*c == 0) break;
        } else {
            line += *c;
        }
    }
}

void index_records(const char* path) {
    int64_t n = 0;
    if (s1g_read_index(path, nullptr, 0, &n, 1) != S1G_OK) throw std::runtime_error(std::string("Unable to open ") + path);
    std::vector<s1g_index_record> r((size_t)n);
    s1g_read_index(path, r.data(), n, &n, 1);
    for (int64_t i = 0; i < n; ++i) {
        std::cout << "Index Record #" << i << ":" << std::endl;
        std::cout << "Date/Time: " << r[i].date_time << std::endl;
        std::cout << "Time Delta: " << r[i].time_delta << std::endl;
        std::cout << "Data Size: " << r[i].data_size << std::endl;
        std::cout << "Unit Offset: " << r[i].unit_offset << std::endl;
        std::cout << "Byte Offset: " << r[i].byte_offset << std::endl;
        std::cout << "Variable Flag: " << r[i].variable_flag << std::endl;
        std::cout << "Spare Data: " << r[i].spare_data << std::endl;
        std::cout << "---" << std::endl;
    }
}

void annotation_record(const char* path, int index) {
    int64_t n = 0;
    if (s1g_read_annotation(path, nullptr, 0, &n, 1) != S1G_OK)
        throw std::runtime_error(std::string("Unable to open ") + path);
    if (index < 0 || index >= n) throw std::out_of_range("Index is greater than the number of records.");
    std::vector<s1g_annotation_record> r((size_t)n);
    s1g_read_annotation(path, r.data(), n, &n, 1);
    const s1g_annotation_record& a = r[(size_t)index];
    std::cout << "Days Uplink: " << a.days_ul << std::endl;
    std::cout << "Milliseconds Uplink: " << a.milliseconds_ul << std::endl;
    std::cout << "Microseconds Uplink: " << a.microseconds_ul << std::endl;
    std::cout << "Days Downlink: " << a.days_dl << std::endl;
    std::cout << "Milliseconds Downlink: " << a.milliseconds_dl << std::endl;
    std::cout << "Microseconds Downlink: " << a.microseconds_dl << std::endl;
    std::cout << "Packet Length: " << a.packet_length << std::endl;
    std::cout << "Error Flag: " << a.error_flag << std::endl;
}

// STATE_VECTORS::print (state_vectors.cpp:86-124)
void state_vectors(const char* path) {
    Handle d(path);
    int n = 0;
    d.check(s1g_state_vectors(d.h, nullptr, 0, &n));
    std::vector<double> sv(7 * (size_t)n), at(10 * (size_t)n);
    d.check(s1g_state_vectors(d.h, sv.data(), n, &n));
    d.check(s1g_attitudes(d.h, at.data(), n, &n));
    const int hyphens = 210;
    std::cout << std::string(hyphens, '-') << std::endl;
    const char* cols[] = {"time", "position_x", "position_y", "position_z", "velocity_x", "velocity_y", "velocity_z",
                          "q0_quaternion", "q1_quaternion", "q2_quaternion", "q3_quaternion", "roll", "pitch", "yaw"};
    for (int c = 0; c < 14; ++c) std::cout << std::setw(15) << cols[c];
    std::cout << std::endl;
    std::cout << std::string(hyphens, '-') << std::endl;
    for (int i = 0; i < n; ++i) {
        std::cout << std::fixed << std::setprecision(4);
        for (int c = 0; c < 7; ++c) std::cout << std::setw(15) << sv[7 * (size_t)i + c];
        for (int c = 0; c < 4; ++c) std::cout << std::setw(15) << at[10 * (size_t)i + c];
        for (int c = 7; c < 10; ++c) std::cout << std::setw(15) << at[10 * (size_t)i + c];
        std::cout << std::endl;
    }
    std::cout << std::string(hyphens, '-') << std::endl;
}

}  // namespace

int main(int argc, char* argv[]) {
    if (argc < 2) {
        std::cout << "Please enter a command:" << std::endl;
        print_help();
        return 1;
    }
    const std::string cmd = argv[1];
    try {
        if (cmd == "packet_info") {
            validate(cmd, {{"packet_index", "int"}, {"path", "path"}}, argc, argv);
            packet_info(argv[3], std::stoi(argv[2]));
        } else if (cmd == "complex_samples") {
            validate(cmd, {{"packet_index", "int"}, {"path", "path"}}, argc, argv);
            complex_samples(argv[3], std::stoi(argv[2]));
        } else if (cmd == "swath_names") {
            validate(cmd, {{"path", "path"}}, argc, argv);
            swath_names(argv[2]);
        } else if (cmd == "index_records") {
            validate(cmd, {{"path", "path"}}, argc, argv);
            index_records(argv[2]);
        } else if (cmd == "annotation_record") {
            validate(cmd, {{"record_index", "int"}, {"path", "path"}}, argc, argv);
            annotation_record(argv[3], std::stoi(argv[2]));
        } else if (cmd == "state_vectors") {
            validate(cmd, {{"path", "path"}}, argc, argv);
            state_vectors(argv[2]);
        } else if (cmd == "help" || cmd == "--help" || cmd == "-h") {
            print_help();
        } else {
            std::cout << cmd << " is not a valid command." << std::endl;
        }
    } catch (const std::exception& e) {
        std::cerr << "terminate called after throwing an exception" << std::endl;
        std::cerr << "  what():  " << e.what() << std::endl;
        return 134;
    }
    return 0;
}
