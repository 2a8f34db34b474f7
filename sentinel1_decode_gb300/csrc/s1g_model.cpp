// Host-side packet model (see s1g_model.h).
#include "s1g_model.h"

#include <algorithm>
#include <cmath>
#include <set>
#include <stdexcept>

namespace s1g {

const char* const kFieldNames[F_COUNT] = {
    "packet_version_number", "packet_type", "secondary_header_flag", "process_id", "process_category",
    "sequence_flags", "packet_sequence_count", "packet_data_length",
    "coarse_time", "fine_time", "sync_marker", "data_take_id", "ecc_number", "na_1", "test_mode",
    "rx_channel_id", "instrument_configuration_id", "sc_data_word_index", "sc_data_word",
    "space_packet_count", "pri_count", "error_flag", "na_2", "baq_mode", "baq_block_length", "na_3",
    "range_decimation", "rx_gain", "tx_ramp_rate_sign", "tx_ramp_rate_mag", "pulse_start_frequency_sign",
    "pulse_start_frequency_mag", "pulse_length", "na_4", "rank", "pri", "swst", "swl", "ssb_flag",
    "polarisation", "temperature_compensation", "na_5", "elevation_beam_address", "na_6",
    "azimuth_beam_address", "calibration_mode", "na_7", "tx_pulse_number", "signal_type", "na_8", "swap",
    "swath_number", "num_quadratures", "na_9"};

const int kFieldBits[F_COUNT] = {3, 1, 1, 7, 4, 2, 14, 16,
                                 32, 16, 32, 32, 8, 1, 3, 4, 32, 8, 16, 32, 32, 1, 2, 5, 8, 8, 8, 8, 1, 15, 1,
                                 15, 24, 3, 5, 24, 24, 24, 1, 3, 2, 2, 4, 2, 10, 2, 1, 5, 4, 3, 1, 8, 16, 8};

// structs.h:21-38, 561-574 (PI truncated as in the reference)
static const double kPI = 3.14159265358979;
static const double kC = 299792458.0;
static const double kFRef = 37.53472224;
static const double kDeltaT = (320 / (8 * kFRef)) * 1e-6;
static const double kLatch = 1.439 * 1e-6;
static const double kRangeDec[12] = {112.6041667, 100.0925926, 0.000000000, 83.41049387, 66.72839509, 56.30208336,
                                     50.04629632, 25.02314816, 64.34523813, 46.91840280, 17.32371796, 54.59595962};

// Field i occupies kFieldBits[i] bits starting where field i-1 ended, MSB
// first (parse_packet_header, packet.cpp:829-846).  No field is wider than
// 32 bits, so each is the top bits of the big-endian 64-bit word at its
// first byte, shifted by the bit offset inside that byte.
void parse_header(const uint8_t* b, PacketHdr& h) {
    uint8_t buf[68 + 8] = {0};
    for (int i = 0; i < 68; ++i) buf[i] = b[i];
    int bit = 0;
    for (int i = 0; i < F_COUNT; ++i) {
        const int w = kFieldBits[i];
        const uint8_t* p = buf + (bit >> 3);
        uint64_t word = 0;
        for (int k = 0; k < 8; ++k) word = (word << 8) | p[k];
        h.f[i] = (int64_t)((word << (bit & 7)) >> (64 - w));
        bit += w;
    }
}

double PacketHdr::pri_us() const { return f[F_PRI] / kFRef; }
double PacketHdr::pulse_length_us() const { return f[F_PULSE_LEN] / kFRef; }
double PacketHdr::swst_us() const { return f[F_SWST] / kFRef; }
double PacketHdr::swl_us() const { return f[F_SWL] / kFRef; }
double PacketHdr::rx_gain_db() const { return -0.5 * f[F_RX_GAIN]; }
double PacketHdr::time() const { return (double)f[F_COARSE] + (1.0 / (double)f[F_FINE]); }
double PacketHdr::tx_ramp_rate() const {
    const int sign = f[F_TXPRR_SIGN] == 0 ? -1 : 1;
    const int mag = (int)f[F_TXPRR_MAG];
    return sign * mag * (std::pow(kFRef, 2) / 2097152);
}
double PacketHdr::start_frequency() const {
    const int sign = f[F_TXPSF_SIGN] == 0 ? -1 : 1;
    const int mag = (int)f[F_TXPSF_MAG];
    return (sign * mag * (kFRef / 16384)) + (tx_ramp_rate() / (4 * kFRef));
}
double PacketHdr::azimuth_beam_angle() const {
    static const std::vector<double> table = linspace(-0.018, 0.018, 1024);
    return table[(size_t)f[F_AZ_BEAM]];
}
double PacketHdr::range_sample_rate_mhz() const {
    const int rd = (int)f[F_RANGE_DEC];
    return (rd >= 0 && rd < 12) ? kRangeDec[rd] : 0.0;
}
int PacketHdr::replica_chirp_length() const { return (int)std::floor(range_sample_rate_mhz() * pulse_length_us()); }

std::string PacketHdr::swath() const {
    // structs.h:488-558
    static const std::map<int, std::string> m = {
        {0, "S1"}, {1, "S2"}, {2, "S3"}, {3, "S4"}, {4, "S5_N"}, {5, "S5_S"}, {6, "S6"}, {10, "IW1"}, {11, "IW2"},
        {12, "IW3"}, {20, "EW1"}, {21, "EW2"}, {22, "EW3"}, {23, "EW4"}, {24, "EW5"}, {25, "EW1_100MHz_CAL"},
        {26, "EW2_100MHz_CAL"}, {27, "EW3_100MHz_CAL"}, {28, "EW4_100MHz_CAL"}, {29, "EW5_100MHz_CAL"},
        {30, "WV1"}, {31, "WV2"}, {32, "WV1_100MHz_CAL"}, {33, "WV2_100MHz_CAL"}, {36, "S1_100MHz_CAL"},
        {37, "S2_100MHz_CAL"}, {38, "S3_100MHz_CAL"}, {39, "S4_100MHz_CAL"}, {40, "S5_100MHz_N_CAL"},
        {41, "S5_100MHz_S_CAL"}, {42, "S6_100MHz_CAL"}, {43, "IW1_100MHz_CAL"}, {44, "IW2_100MHz_CAL"},
        {45, "IW3_100MHz_CAL"}, {50, "S1_TXCAL"}, {51, "S2_TXCAL"}, {52, "S3_TXCAL"}, {53, "S4_TXCAL"},
        {54, "S5_N_TXCAL"}, {55, "S5_S_TXCAL"}, {56, "S6_TXCAL"}, {60, "IW1_TXCAL"}, {61, "IW2_TXCAL"},
        {62, "IW3_TXCAL"}, {70, "EW1_TXCAL"}, {71, "EW2_TXCAL"}, {72, "EW3_TXCAL"}, {73, "EW4_TXCAL"},
        {74, "EW5_TXCAL"}, {75, "EW1_100MHz_TXCAL"}, {76, "EW2_100MHz_TXCAL"}, {77, "EW3_100MHz_TXCAL"},
        {78, "EW4_100MHz_TXCAL"}, {79, "EW5_100MHz_TXCAL"}, {80, "WV1_TXCAL"}, {81, "WV2_TXCAL"},
        {82, "WV1_100MHz_TXCAL"}, {83, "WV2_100MHz_TXCAL"}, {86, "S1_100MHz_TXCAL"}, {87, "S2_100MHz_TXCAL"},
        {88, "S3_100MHz_TXCAL"}, {89, "S4_100MHz_TXCAL"}, {90, "S5_100MHz_N_TXCAL"}, {91, "S5_100MHz_S_TXCAL"},
        {92, "S6_100MHz_TXCAL"}, {93, "IW1_100MHz_TXCAL"}, {94, "IW2_100MHz_TXCAL"}, {95, "IW3_100MHz_TXCAL"}};
    auto it = m.find((int)f[F_SWATH]);
    return it == m.end() ? "UNKNOWN_" + std::to_string(f[F_SWATH]) : it->second;
}

// ------------------------------------------------------------------ header text
// The names L0Packet prints for header codes (packet.cpp:104-202,
// 264-274; sensor modes: the ECC table of structs.h:358-406).
char data_format(const PacketHdr& h) {
    const int baq = (int)h[F_BAQ_MODE];
    if (baq == 0) return h[F_TEST] % 3 == 0 ? 'A' : 'B';
    if (baq >= 3 && baq <= 5) return 'C';
    if (baq >= 12 && baq <= 14) return 'D';
    throw std::out_of_range("BAQ Mode is invalid.");
}

std::string baq_mode_name(const PacketHdr& h) {
    switch ((int)h[F_BAQ_MODE]) {
        case 0: return "bypass_mode";
        case 3: return "3_bit_mode";
        case 4: return "4_bit_mode";
        case 5: return "5_bit_mode";
        case 12: return "fdbaq_mode_0";
        case 13: return "fdbaq_mode_1";
        case 14: return "fdbaq_mode_2";
        default: return "n_a";
    }
}

std::string test_mode_name(const PacketHdr& h) {
    switch ((int)h[F_TEST]) {
        case 0: return "measurement_mode";
        case 1: case 3: return "n_a";
        case 4: case 5: return "contingency";
        case 6: return "test_mode_baq";
        case 7: return "test_mode_bypass";
        default: throw std::out_of_range("The test mode number is not in the range of valid values.");
    }
}

std::string sensor_mode_name(const PacketHdr& h) {
    static const char* const modes[] = {
        "contingency", "stripmap_1", "stripmap_2", "stripmap_3", "stripmap_4", "stripmap_5n", "stripmap_6",
        "contingency", "interferomatric_wide_swath", "wave_mode", "stripmap-5s", "stripmap_1_w_cal",
        "stripmap_2_w_cal", "stripmap_3_w_cal", "stripmap_4_w_cal", "rf_characterization_mode", "test_mode",
        "elevation_notch_s3", "azimuth_notch_s1", "azimuth_notch_s2", "azimuth_notch_s3", "azimuth_notch_s4",
        "azimuth_notch_s5n", "azimuth_notch_s5s", "azimuth_notch_s6", "stripmap_5n_wo_cal", "stripmap_5s_wo_cal",
        "stripmap_6_wo_cal", "contingency", "contingency", "contingency", "elevation_notch_s3_wo_cal",
        "extra_wide_swath", "azimuth_notch_s1_wo_cal", "azimuth_notch_s2_wo_cal", "azimuth_notch_s3_wo_cal",
        "contingency", "noise_characterization_s1", "noise_characterization_s2", "noise_characterization_s3",
        "noise_characterization_s4", "noise_characterization_s5n", "noise_characterization_s5s",
        "noise_characterization_s6", "noise_characterization_ew", "noise_characterization_iw",
        "noise_characterization_wave", "contingency"};
    const int64_t e = h[F_ECC];
    // the reference indexes its vector unchecked; codes past the table read
    // out of bounds there and are reported as "n_a" here
    return (e >= 0 && e < (int64_t)(sizeof(modes) / sizeof(modes[0]))) ? modes[e] : "n_a";
}

std::string signal_type_name(const PacketHdr& h) {
    switch ((int)h[F_SIG_TYPE]) {
        case 0: return "echo";
        case 1: return "noise";
        case 8: return "tx_cal";
        case 9: return "rx_cal";
        case 10: return "epdn_cal";
        case 11: return "ta_cal";
        case 12: return "apdn_cal";
        case 15: return "txh_cal_iso";
        default: return "n_a";
    }
}

char tx_polarization(const PacketHdr& h) {
    const int64_t c = h[F_POL];
    if (c >= 0 && c <= 3) return 'H';
    if (c >= 4 && c <= 7) return 'V';
    throw std::runtime_error("The polarization code is invalid.");
}

char rx_polarization(const PacketHdr& h) {
    switch ((int)h[F_RXCH]) {
        case 0: return 'V';
        case 1: return 'H';
        default: throw std::runtime_error("The rx_channel_id is invalid.");
    }
}

int num_baq_blocks(const PacketHdr& h) { return (int)std::ceil((2.0 * double(h.num_quads())) / 256.0); }

std::vector<double> linspace(double start, double end, int n) {
    // signal_processing.cpp:18-29
    std::vector<double> r(n);
    const double step = (end - start) / (n - 1);
    for (int i = 0; i < n; ++i) r[i] = start + i * step;
    return r;
}

// ------------------------------------------------------------------ state vectors
static double int_to_ieee754(uint64_t number, int is_double) {
    // decoding_utils.cpp:149-170
    const int ms = is_double ? 52 : 23;
    const uint64_t emask = is_double ? 0x7FF0000000000000ULL : 0x7f800000ULL;
    const int bias = is_double ? 1023 : 127;
    const int ss = is_double ? 63 : 31;
    const int sign = (number >> ss) & 0x01;
    const int exponent = (int)((number & emask) >> ms) - bias;
    int power = -1;
    double total = 0.0;
    for (int i = 0; i < ms; i++) {
        const int calc = (number >> (ms - i - 1)) & 0x01;
        total += calc * std::pow(2.0, power);
        power--;
    }
    return (sign ? -1 : 1) * std::pow(2.0, exponent) * (total + 1.0);
}

static double parse_time_stamp(uint64_t raw) {
    // state_vectors.cpp:5-16, including the mask it applies to the fine bits
    const unsigned coarse = (raw >> 24) & 0xffffffff;
    unsigned fine_raw = raw & 0xffffff;
    double fine = 0.0;
    for (int i = 23; i >= 0; i--) {
        fine += (fine_raw >> i) * std::pow(2, i - 24);
        fine_raw &= 1 << 8;
    }
    return double(coarse) + fine;
}

// The reference builds the EOCFI rotation matrix in float (e00..e22 and the
// matrix entries are float) and then takes sums and differences of those
// floats before widening to double; the float temporaries below keep those
// roundings.  This file is compiled without floating-point contraction.
void parse_attitude(const double qr[4], double qo[4], double att[3]) {
    const double w = qr[0], x = qr[1], y = qr[2], z = qr[3];
    // get_eocfi_rotation_matrix (state_vectors.cpp:280-300)
    const float e00 = (float)(x * x - y * y - z * z + w * w);
    const float e01 = (float)(2 * (x * y + z * w));
    const float e02 = (float)(2 * (x * z - y * w));
    const float e10 = (float)(2 * (x * y - z * w));
    const float e11 = (float)(-x * x + y * y - z * z + w * w);
    const float e12 = (float)(2 * (y * z + x * w));
    const float e20 = (float)(2 * (x * z + y * w));
    const float e21 = (float)(2 * (y * z - x * w));
    const float e22 = (float)(-x * x - y * y + z * z + w * w);
    const float R[3][3] = {{-e10, -e11, -e12}, {-e00, -e01, -e02}, {-e20, -e21, -e22}};
    // get_quaternions_from_rotation_matrix (state_vectors.cpp:203-240)
    double qw, qx, qy, qz;
    const float tr = R[0][0] + R[1][1] + R[2][2];
    const double trace = tr;
    if (trace > 0) {
        const double S = std::sqrt(trace + 1.0) * 2;
        qw = 0.25 * S;
        qx = (float)(R[2][1] - R[1][2]) / S;
        qy = (float)(R[0][2] - R[2][0]) / S;
        qz = (float)(R[1][0] - R[0][1]) / S;
    } else if ((R[0][0] > R[1][1]) && (R[0][0] > R[2][2])) {
        const double S = std::sqrt(1.0 + R[0][0] - R[1][1] - R[2][2]) * 2;
        qw = (float)(R[2][1] - R[1][2]) / S;
        qx = 0.25 * S;
        qy = (float)(R[0][1] + R[1][0]) / S;
        qz = (float)(R[0][2] + R[2][0]) / S;
    } else if (R[1][1] > R[2][2]) {
        const double S = std::sqrt(1.0 + R[1][1] - R[0][0] - R[2][2]) * 2;
        qw = (float)(R[0][2] - R[2][0]) / S;
        qx = (float)(R[0][1] + R[1][0]) / S;
        qy = 0.25 * S;
        qz = (float)(R[1][2] + R[2][1]) / S;
    } else {
        const double S = std::sqrt(1.0 + R[2][2] - R[0][0] - R[1][1]) * 2;
        qw = (float)(R[1][0] - R[0][1]) / S;
        qx = (float)(R[0][2] + R[2][0]) / S;
        qy = (float)(R[1][2] + R[2][1]) / S;
        qz = 0.25 * S;
    }
    // parse_quaternions: (w, -x, -y, -z); stored scalar last
    const double W = qw, X = -qx, Y = -qy, Z = -qz;
    qo[0] = X;
    qo[1] = Y;
    qo[2] = Z;
    qo[3] = W;
    // Quaternion::to_rotation_matrix / to_euler_angles (state_vectors.cpp:243-277)
    const double r1 = 2 * (X * Y + W * Z);
    const double r4 = 1 - 2 * (X * X + Z * Z);
    const double r5 = 2 * (Y * Z + W * X);
    const double r6 = 2 * (X * Z + W * Y);
    const double r7 = 2 * (Y * Z - W * X);
    const double r8 = 1 - 2 * (X * X + Y * Y);
    const double pitch = std::asin(-std::max(-1.0, std::min(1.0, r7)));
    double roll, yaw;
    if (std::abs(r7) < 1) {
        roll = std::atan2(r6, r8);
        yaw = std::atan2(r1, r4);
    } else {
        roll = std::atan2(r5, r4);
        yaw = 0.0;
    }
    att[0] = -pitch;
    att[1] = -roll;
    att[2] = yaw;
}

void StateVectors::build(const std::vector<PacketHdr>& pk) {
    // sub-commutated word index -> key (structs.h:622-688): 1-4 x, 5-8 y,
    // 9-12 z (double words), 13-14 vx, 15-16 vy, 17-18 vz, 23-30 q0..q3,
    // 31-36 omega x..z (float words), 37-40 data time stamp
    t.clear();
    p.clear();
    v.clear();
    q.clear();
    w.clear();
    att.clear();
    const int n = (int)pk.size();
    int start = 0;
    do {
        ++start;
        if (start >= n) return;
    } while (pk[start][F_SC_INDEX] != 1);
    enum { KX, KY, KZ, KVX, KVY, KVZ, KQ0, KQ1, KQ2, KQ3, KWX, KWY, KWZ, KT, KOTHER, NKEYS };
    uint64_t raw[NKEYS] = {0};
    auto key_of = [](int idx) {
        if (idx >= 1 && idx <= 12) return KX + (idx - 1) / 4;
        if (idx >= 13 && idx <= 18) return KVX + (idx - 13) / 2;
        if (idx >= 23 && idx <= 30) return KQ0 + (idx - 23) / 2;
        if (idx >= 31 && idx <= 36) return KWX + (idx - 31) / 2;
        if (idx >= 37 && idx <= 40) return (int)KT;
        return (int)KOTHER;
    };
    double last = 0.0;
    for (int i = start; i < n; ++i) {
        const int idx = (int)pk[i][F_SC_INDEX];
        if (idx == 1 && i != start) {
            const double tt = parse_time_stamp(raw[KT]);
            if (tt > last) {
                last = tt;
                t.push_back(tt);
                p.push_back({int_to_ieee754(raw[KX], 1), int_to_ieee754(raw[KY], 1), int_to_ieee754(raw[KZ], 1)});
                v.push_back({int_to_ieee754(raw[KVX], 0), int_to_ieee754(raw[KVY], 0), int_to_ieee754(raw[KVZ], 0)});
                w.push_back({int_to_ieee754(raw[KWX], 0), int_to_ieee754(raw[KWY], 0), int_to_ieee754(raw[KWZ], 0)});
                const double qr[4] = {int_to_ieee754(raw[KQ0], 0), int_to_ieee754(raw[KQ1], 0),
                                      int_to_ieee754(raw[KQ2], 0), int_to_ieee754(raw[KQ3], 0)};
                std::array<double, 4> qo;
                std::array<double, 3> a;
                parse_attitude(qr, qo.data(), a.data());
                q.push_back(qo);
                att.push_back(a);
            }
            for (auto& r : raw) r = 0;
        }
        const int k = key_of(idx);
        raw[k] = (raw[k] << 16) | (uint64_t)pk[i][F_SC_WORD];
    }
}

static double std_lerp(double a, double b, double t) {
    // libstdc++ std::lerp (state_vectors.cpp:149)
    if ((a <= 0 && b >= 0) || (a >= 0 && b <= 0)) return t * b + (1 - t) * a;
    if (t == 1) return b;
    const double x = a + t * (b - a);
    return (t > 1) == (b > a) ? (b < x ? x : b) : (x < b ? x : b);
}

void StateVectors::interpolate(double time, double pos[3], double vel[3]) const {
    const int n = (int)t.size();
    if (n == 0) {
        for (int c = 0; c < 3; ++c) pos[c] = vel[c] = 0.0;
        return;
    }
    if (time > t.back()) {
        for (int c = 0; c < 3; ++c) { pos[c] = p.back()[c]; vel[c] = v.back()[c]; }
        return;
    }
    if (time < t[0]) {
        for (int c = 0; c < 3; ++c) { pos[c] = p[0][c]; vel[c] = v[0][c]; }
        return;
    }
    int lo = 0, hi = n, a = 0, b = 0;
    while (true) {
        const int size = hi - lo;
        if (size == 1) { a = lo; b = hi < n ? hi : n - 1; break; }
        const int pivot = size / 2;
        const double tp = t[lo + pivot];
        if (tp == time) { a = b = lo; break; }
        if (tp > time) hi = lo + pivot;
        else lo = lo + pivot;
    }
    const double ta = t[a], tb = t[b];
    const double f = (time - ta) / (tb - ta);
    for (int c = 0; c < 3; ++c) {
        pos[c] = std_lerp(p[a][c], p[b][c], f);
        vel[c] = std_lerp(v[a][c], v[b][c], f);
    }
}

// ------------------------------------------------------------------ geometry
BurstGeom make_geom(const std::vector<PacketHdr>& hdr, const std::vector<int>& pk) {
    BurstGeom g;
    const PacketHdr& f = hdr[pk.front()];
    g.n_a = (int)pk.size();
    g.nq = f.num_quads();
    g.n_r = 2 * g.nq;
    g.swath_number = (int)f[F_SWATH];
    g.pri = f.pri_us() * 1e-6;
    g.prf = 1 / g.pri;
    g.T = double(g.n_a) / g.prf;
    g.fs = f.range_sample_rate_mhz() * 1e6;
    g.t0 = f.time();
    g.beam0 = f.azimuth_beam_angle();
    g.beam1 = hdr[pk.back()].azimuth_beam_angle();
    // packet.cpp:284-318
    {
        const double num_rng = 2 * g.nq;
        const double start_time = f.swst_us() * 1e-6;
        const double rank = (double)f[F_RANK];
        g.near = rank * g.pri + start_time + kDeltaT;
        g.far = g.near + (num_rng / g.fs);
        g.slant = linspace(g.near * kC / 2, g.far * kC / 2, g.n_r);
    }
    g.range_freq = linspace(-g.fs / 2, g.fs / 2, g.n_r);
    // packet.cpp:322-342
    {
        const double swst = f.swst_us() * 1e-6;
        const double rank = (double)f[F_RANK];
        const double dt = 1 / g.fs;
        g.tcorr.resize(g.n_r);
        for (int i = 0; i < g.n_r; i++)
            g.tcorr[i] = (swst + kLatch) + ((swst + (rank * g.pri) - ((double)i * dt)) / 2);
    }
    g.ref_range = g.slant[g.n_r / 2];
    g.rscale.resize(g.n_r);
    for (int j = 0; j < g.n_r; ++j) g.rscale[j] = std::sqrt(std::pow(g.ref_range / g.slant[j], 3.0));
    // replica chirp, packet.cpp:345-373
    const double txpsf = f.start_frequency();
    const double txprr = f.tx_ramp_rate();
    const double txpl = f.pulse_length_us();
    const double phi_1 = txpsf, phi_2 = txprr * 0.5;
    g.L = (int)std::floor(f.range_sample_rate_mhz() * txpl);
    if (g.L < 1) throw std::runtime_error("replica chirp length < 1");
    const std::vector<double> tt = linspace(0.0, txpl, g.L);
    g.chirp.resize(g.L);
    const int rep_len = g.n_r + 2 * g.L;
    double energy = 0.0;
    for (int i = 0; i < g.L; ++i) {
        const double t = tt[i];
        const double th = 2.0 * kPI * ((phi_1 * t) + phi_2 * (t * t));
        const double s = double(1.0 / g.L);
        const double re = s * std::cos(th), im = s * std::sin(th);
        g.chirp[i] = mk(re, im);
        // image_formation.cpp:7-14: sum |c|^2 * (|c|^2 / rep_len)
        const double a2 = std::pow(std::hypot(re, im), 2.0);
        energy += a2 * (a2 / (double)rep_len);
    }
    g.energy = energy;
    // the reference correlates at length rep_len with the chirp centred at
    // c0 and rotates by ceil(rep_len/2): out[k] = sum_t x[k + t - h] conj(c[t]) / E
    const int c0 = (rep_len - g.L) / 2;
    const int gsh = (g.L + (rep_len + 1) / 2 + c0) % rep_len;
    g.h = g.L - gsh;
    return g;
}

}  // namespace s1g
