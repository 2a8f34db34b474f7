// Host-side packet model: header fields, swath/burst segmentation, state
// vectors and per-burst geometry, following the reference's S1_Decoder
// constructor path (packet.cpp, state_vectors.cpp, s1_decoder.cpp:13-34).
#pragma once

#include <array>
#include <map>
#include <string>
#include <vector>

#include "s1g_complex.cuh"

namespace s1g {

// Header fields in parse order (structs.h:42-166): 8 primary then 46 secondary.
enum Field {
    F_VERSION = 0, F_TYPE, F_SEC_FLAG, F_PID, F_PCAT, F_SEQ_FLAGS, F_SEQ_COUNT, F_PDL,
    F_COARSE, F_FINE, F_SYNC, F_DTID, F_ECC, F_NA1, F_TEST, F_RXCH, F_ICID, F_SC_INDEX, F_SC_WORD,
    F_SPC, F_PRI_COUNT, F_ERR, F_NA2, F_BAQ_MODE, F_BAQ_BL, F_NA3, F_RANGE_DEC, F_RX_GAIN,
    F_TXPRR_SIGN, F_TXPRR_MAG, F_TXPSF_SIGN, F_TXPSF_MAG, F_PULSE_LEN, F_NA4, F_RANK, F_PRI, F_SWST,
    F_SWL, F_SSB, F_POL, F_TEMP, F_NA5, F_ELEV, F_NA6, F_AZ_BEAM, F_CAL_MODE, F_NA7, F_TXPN,
    F_SIG_TYPE, F_NA8, F_SWAP, F_SWATH, F_NQ, F_NA9, F_COUNT
};
extern const char* const kFieldNames[F_COUNT];
extern const int kFieldBits[F_COUNT];

struct PacketHdr {
    std::array<int64_t, F_COUNT> f;
    long long offset;
    int64_t operator[](int i) const { return f[i]; }
    // packet.cpp:15-100
    double pri_us() const;
    double pulse_length_us() const;
    double swst_us() const;
    double swl_us() const;
    double rx_gain_db() const;
    double time() const;
    double tx_ramp_rate() const;
    double start_frequency() const;
    double azimuth_beam_angle() const;
    double range_sample_rate_mhz() const;
    int num_quads() const { return (int)f[F_NQ]; }
    int replica_chirp_length() const;
    std::string swath() const;
};

void parse_header(const uint8_t* b68, PacketHdr& h);

struct StateVectors {
    std::vector<double> t;
    std::vector<std::array<double, 3>> p, v;
    // STATE_VECTORS members quaternions (x, y, z, w: scalar last),
    // angular_rates and attitudes (state_vectors.h:55-120)
    std::vector<std::array<double, 4>> q;
    std::vector<std::array<double, 3>> w, att;
    void build(const std::vector<PacketHdr>& pk);   // state_vectors.cpp:19-83
    void interpolate(double time, double pos[3], double vel[3]) const;   // state_vectors.cpp:127-200
};

// Per-burst geometry and tables computed in FP64 on the host.
struct BurstGeom {
    int n_a = 0, nq = 0, n_r = 0, L = 0, h = 0, m_rc = 0, swath_number = 0;
    double pri = 0, prf = 0, T = 0, fs = 0, t0 = 0;
    double near = 0, far = 0;           // slant range times of first/last range bin
    double energy = 0;                  // get_reference_function energy
    std::vector<cpx<double>> chirp;     // L replica samples (packet.cpp:345-373)
    std::vector<double> slant, range_freq, tcorr, rscale;
    double ref_range = 0;
    double beam0 = 0, beam1 = 0;        // azimuth beam angles of first/last packet
};

// The attitude of one sub-commutated quaternion (q0 scalar first):
// parse_quaternions, the EOCFI rotation and the Euler angles of
// state_vectors.cpp:203-320.  q_out = (x, y, z, w), att = (-pitch, -roll, yaw).
void parse_attitude(const double q_raw[4], double q_out[4], double att[3]);

// Text helpers of L0Packet (packet.cpp:104-202, packet.h:156)
char data_format(const PacketHdr& h);          // throws std::out_of_range on a bad BAQ mode
std::string baq_mode_name(const PacketHdr& h);
std::string test_mode_name(const PacketHdr& h);  // throws std::out_of_range
std::string sensor_mode_name(const PacketHdr& h);
std::string signal_type_name(const PacketHdr& h);
char tx_polarization(const PacketHdr& h);        // throws std::runtime_error
char rx_polarization(const PacketHdr& h);        // throws std::runtime_error
int num_baq_blocks(const PacketHdr& h);

BurstGeom make_geom(const std::vector<PacketHdr>& hdr, const std::vector<int>& pk);

std::vector<double> linspace(double a, double b, int n);

}  // namespace s1g
