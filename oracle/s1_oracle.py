"""FP64 CPU restatement of the reference's Level-0 -> SLC path.

TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
against (and, timed on the host cores, the CPU baseline of the benchmark).
It must never be imported by the shipped library; only tests/, bench.py's
CPU legs and __graft_entry__.smoke() use it.

Every function names the reference function (file:line, paths relative to
the reference project) whose arithmetic it follows, in FP64 and with the
same operation order where that matters.  The DFTs are numpy/scipy FFTs:
the reference's FFTW computes the plain DFT definition (unnormalised
forward exp(-2 pi i jk/n) and backward exp(+...)), which any correct FFT
restates.  The type-D packet decode is the C restatement in
fdbaq_oracle.c (bit-exact integer work), loaded through ctypes.

Parity: pinned against the reference's own sources compiled here with an
FFTW-API shim (oracle/Makefile); the committed golden fixtures in
tests/golden/ were produced that way (tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from typing import Dict, List, Optional, Tuple

import numpy as np

try:
    import scipy.fft as _sfft

    def _fft(x, axis=-1, workers=None):
        return _sfft.fft(x, axis=axis, workers=workers or _WORKERS)

    def _ifft_unnorm(x, axis=-1, workers=None):
        n = x.shape[axis]
        return _sfft.ifft(x, axis=axis, workers=workers or _WORKERS) * n
except ImportError:  # pragma: no cover
    def _fft(x, axis=-1, workers=None):
        return np.fft.fft(x, axis=axis)

    def _ifft_unnorm(x, axis=-1, workers=None):
        return np.fft.ifft(x, axis=axis) * x.shape[axis]

_WORKERS = int(os.environ.get("S1G_ORACLE_THREADS", os.cpu_count() or 1))

# ------------------------------------------------------------ constants
# structs.h:21-38
PI = 3.14159265358979
SPEED_OF_LIGHT = 299792458.0
SEMI_MAJOR = 6378137.0
SEMI_MINOR = 6356752.3142
CENTER_FREQ = 5.405000454334350e9
WAVELENGTH = SPEED_OF_LIGHT / CENTER_FREQ
F_REF = 37.53472224
DELTA_T_SUPPRESSED = (320 / (8 * F_REF)) * 1e-6
LATCH_TIME_OFFSET = 1.439 * 1e-6
# structs.h:561-574
RANGE_DECIMATION = [112.6041667, 100.0925926, 0.0, 83.41049387, 66.72839509, 56.30208336,
                    50.04629632, 25.02314816, 64.34523813, 46.91840280, 17.32371796, 54.59595962]
PRIMARY_HEADER = [("packet_version_number", 3), ("packet_type", 1), ("secondary_header_flag", 1),
                  ("process_id", 7), ("process_category", 4), ("sequence_flags", 2),
                  ("packet_sequence_count", 14), ("packet_data_length", 16)]
SECONDARY_HEADER = [
    ("coarse_time", 32), ("fine_time", 16), ("sync_marker", 32), ("data_take_id", 32),
    ("ecc_number", 8), ("na_1", 1), ("test_mode", 3), ("rx_channel_id", 4),
    ("instrument_configuration_id", 32), ("sc_data_word_index", 8), ("sc_data_word", 16),
    ("space_packet_count", 32), ("pri_count", 32), ("error_flag", 1), ("na_2", 2),
    ("baq_mode", 5), ("baq_block_length", 8), ("na_3", 8), ("range_decimation", 8),
    ("rx_gain", 8), ("tx_ramp_rate_sign", 1), ("tx_ramp_rate_mag", 15),
    ("pulse_start_frequency_sign", 1), ("pulse_start_frequency_mag", 15), ("pulse_length", 24),
    ("na_4", 3), ("rank", 5), ("pri", 24), ("swst", 24), ("swl", 24), ("ssb_flag", 1),
    ("polarisation", 3), ("temperature_compensation", 2), ("na_5", 2),
    ("elevation_beam_address", 4), ("na_6", 2), ("azimuth_beam_address", 10),
    ("calibration_mode", 2), ("na_7", 1), ("tx_pulse_number", 5), ("signal_type", 4),
    ("na_8", 3), ("swap", 1), ("swath_number", 8), ("num_quadratures", 16), ("na_9", 8)]
# structs.h:488-558 (echo and calibration swath numbers used here)
SWATH_NUM_TO_STRING = {0: "S1", 1: "S2", 2: "S3", 3: "S4", 4: "S5_N", 5: "S5_S", 6: "S6",
                       10: "IW1", 11: "IW2", 12: "IW3", 20: "EW1", 21: "EW2", 22: "EW3",
                       23: "EW4", 24: "EW5", 30: "WV1", 31: "WV2"}
STRIPMAP_SWATHS = {"S1", "S2", "S3", "S4", "S5", "S6", "S5_N", "S5_S"}
IW_SWATHS = {"IW1", "IW2", "IW3"}
ECHO_SWATHS = STRIPMAP_SWATHS | IW_SWATHS | {"EW1", "EW2", "EW3", "EW4", "EW5", "WV1", "WV2"}


# ------------------------------------------------------------ helpers
def linspace(start: float, end: float, n: int) -> np.ndarray:
    """signal_processing.cpp:18-29: start + i*step, step=(end-start)/(n-1)."""
    step = (end - start) / (n - 1)
    return start + np.arange(n, dtype=np.float64) * step


def fftshift_rows(x: np.ndarray, axis: int = -1) -> np.ndarray:
    """signal_processing.cpp:713-727: std::rotate by n/2 (right rotation)."""
    return np.roll(x, x.shape[axis] // 2, axis=axis)


def cexp_i(theta):
    """exp(i*theta) for a purely imaginary argument."""
    return np.cos(theta) + 1j * np.sin(theta)


def std_lerp(a: float, b: float, t: float) -> float:
    """libstdc++ std::lerp (C++20), used by state_vectors.cpp:149."""
    if (a <= 0 and b >= 0) or (a >= 0 and b <= 0):
        return t * b + (1 - t) * a
    if t == 1:
        return b
    x = a + t * (b - a)
    if (t > 1) == (b > a):
        return x if b < x else b
    return x if x < b else b


# ------------------------------------------------------------ packets
class Packet:
    """Header fields of one space packet plus the location of its user data
    (packet.h:142-167, packet.cpp:829-879)."""

    __slots__ = ("ph", "sh", "offset", "length", "index")

    def __init__(self, ph, sh, offset, length, index):
        self.ph, self.sh, self.offset, self.length, self.index = ph, sh, offset, length, index

    # packet.cpp:15-100
    @property
    def num_quads(self):
        return self.sh["num_quadratures"]

    def get_pri(self):
        return self.sh["pri"] / F_REF

    def get_pulse_length(self):
        return self.sh["pulse_length"] / F_REF

    def get_swst(self):
        return self.sh["swst"] / F_REF

    def get_time(self):
        return float(self.sh["coarse_time"]) + (1.0 / float(self.sh["fine_time"])) if self.sh["fine_time"] else math.inf

    def get_tx_ramp_rate(self):
        sign = -1 if self.sh["tx_ramp_rate_sign"] == 0 else 1
        return (sign * self.sh["tx_ramp_rate_mag"]) * (math.pow(F_REF, 2) / 2097152)

    def get_start_frequency(self):
        sign = -1 if self.sh["pulse_start_frequency_sign"] == 0 else 1
        return (sign * self.sh["pulse_start_frequency_mag"] * (F_REF / 16384)) + (self.get_tx_ramp_rate() / (4 * F_REF))

    def get_azimuth_beam_angle(self):
        return float(linspace(-0.018, 0.018, 1024)[self.sh["azimuth_beam_address"]])

    def get_range_sample_rate(self):
        return RANGE_DECIMATION[self.sh["range_decimation"]]

    def get_swath(self):
        return SWATH_NUM_TO_STRING.get(self.sh["swath_number"], "UNKNOWN_%d" % self.sh["swath_number"])

    def get_rx_polarization(self):
        return {0: "V", 1: "H"}[self.sh["rx_channel_id"]]

    def _delays(self):
        n = 2 * self.num_quads
        fs = self.get_range_sample_rate() * 1e6
        start_time = self.get_swst() * 1e-6
        pri = self.get_pri() * 1e-6
        rank = float(self.sh["rank"])
        near = rank * pri + start_time + DELTA_T_SUPPRESSED
        far = near + (float(n) / fs)
        return near, far

    def get_slant_ranges(self, n=0):  # packet.cpp:284-301
        if n <= 0:
            n = 2 * self.num_quads
        near, far = self._delays()
        return linspace(near * SPEED_OF_LIGHT / 2, far * SPEED_OF_LIGHT / 2, n)

    def get_slant_range_times(self, n=0):  # packet.cpp:304-318
        if n <= 0:
            n = 2 * self.num_quads
        near, far = self._delays()
        return linspace(near, far, n)

    def get_timing_corrections(self):  # packet.cpp:322-342
        n = 2 * self.num_quads
        fs = self.get_range_sample_rate() * 1e6
        swst = self.get_swst() * 1e-6
        rank = float(self.sh["rank"])
        pri = self.get_pri() * 1e-6
        dt = 1 / fs
        i = np.arange(n, dtype=np.float64)
        return (swst + LATCH_TIME_OFFSET) + ((swst + (rank * pri) - (i * dt)) / 2)

    def get_replica_chirp_length(self):  # packet.cpp:376-380
        return int(math.floor(RANGE_DECIMATION[self.sh["range_decimation"]] * self.get_pulse_length()))

    def get_replica_chirp(self):  # packet.cpp:345-373
        num_range = 2 * self.num_quads
        txpsf = self.get_start_frequency()
        txprr = self.get_tx_ramp_rate()
        txpl = self.get_pulse_length()
        phi_1 = txpsf
        phi_2 = txprr * 0.5
        L = int(math.floor(RANGE_DECIMATION[self.sh["range_decimation"]] * txpl))
        t = linspace(0.0, txpl, L)
        rep_len = num_range + 2 * L
        lo = (rep_len - L) // 2
        chirp = np.zeros(rep_len, dtype=np.complex128)
        theta = (2.0 * PI) * ((phi_1 * t) + phi_2 * (t * t))
        chirp[lo:lo + L] = (1.0 / L) * cexp_i(theta)
        return chirp


def _parse_fields(raw: bytes, spec) -> Dict[str, int]:
    """parse_packet_header, packet.cpp:829-846 (MSB-first bit fields)."""
    v = int.from_bytes(raw, "big")
    total = len(raw) * 8
    out = {}
    pos = 0
    for name, w in spec:
        out[name] = (v >> (total - pos - w)) & ((1 << w) - 1)
        pos += w
    return out


def get_packets(data: bytes) -> List[Packet]:
    """get_packets / get_next_packet, packet.cpp:850-917.  A truncated final
    packet is kept with its missing user bytes read as zero (read_bytes
    always sizes the buffer to the requested length)."""
    pkts = []
    off = 0
    n = len(data)
    idx = 0
    while off + 6 <= n:
        ph = _parse_fields(data[off:off + 6], PRIMARY_HEADER)
        sec = data[off + 6:off + 68]
        if len(sec) < 62:
            sec = sec + b"\0" * (62 - len(sec))
        sh = _parse_fields(sec, SECONDARY_HEADER)
        ulen = ph["packet_data_length"] + 1 - 62
        pkts.append(Packet(ph, sh, off + 68, ulen, idx))
        idx += 1
        off += 6 + 62 + ulen
        if off > n:
            break
    return pkts


def get_packets_in_bursts(packets: List[Packet], swath: str, get_cal_packets=False):
    """packet.cpp:1026-1076 (split when the azimuth beam address decreases or
    the PRI count jumps; bursts under 1000 packets dropped at a split)."""
    bursts, cur = [], []
    prev_az = 0
    prev_pri = 0
    num = len(packets)
    for i, p in enumerate(packets):
        if p.get_swath() == swath:
            if not get_cal_packets:
                az = p.sh["azimuth_beam_address"]
                pri_count = p.sh["pri_count"]
                if prev_az == 0:
                    prev_az = az
                    prev_pri = pri_count
                if az < prev_az or pri_count > prev_pri + 1:
                    if len(cur) >= 1000:
                        bursts.append(cur)
                    cur = []
                prev_pri = pri_count
                prev_az = az
            cur.append(p)
        if i == num - 1 and cur:
            bursts.append(cur)
    return bursts


# ------------------------------------------------------------ FDBAQ decode
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        here = os.path.dirname(os.path.abspath(__file__))
        so = os.path.join(here, "_build", "liboracle_fdbaq.so")
        if not os.path.exists(so):
            build_oracle()
        _LIB = ctypes.CDLL(so)
        _LIB.oracle_decode_batch.restype = None
    return _LIB


def build_oracle() -> str:
    """Compile fdbaq_oracle.c with gcc (host code, no GPU)."""
    here = os.path.dirname(os.path.abspath(__file__))
    os.makedirs(os.path.join(here, "_build"), exist_ok=True)
    so = os.path.join(here, "_build", "liboracle_fdbaq.so")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-o", so,
                           os.path.join(here, "fdbaq_oracle.c")])
    return so


def decode_packets(data: bytes, packets: List[Packet], threads: Optional[int] = None):
    """L0Packet::get_signal for each packet (packet.cpp:393-453, type D).
    Returns (rows: complex128 [P, 2*max_nq], status int32[P])."""
    lib = _lib()
    P = len(packets)
    nqs = np.array([p.num_quads for p in packets], dtype=np.int32)
    nqmax = int(nqs.max()) if P else 0
    out = np.zeros((P, 2 * nqmax), dtype=np.complex128)
    offs = np.array([p.offset for p in packets], dtype=np.int64)
    lens = np.array([p.length for p in packets], dtype=np.int64)
    buf = np.frombuffer(data, dtype=np.uint8)
    need = int((offs + lens).max()) if P else 0
    if need > buf.size:  # zero-extend a truncated final packet (read_bytes semantics)
        buf = np.concatenate([buf, np.zeros(need - buf.size, dtype=np.uint8)])
    status = np.zeros(P, dtype=np.int32)
    lib.oracle_decode_batch(
        buf.ctypes.data_as(ctypes.c_void_p), offs.ctypes.data_as(ctypes.c_void_p),
        lens.ctypes.data_as(ctypes.c_void_p), nqs.ctypes.data_as(ctypes.c_void_p),
        ctypes.c_int(P), out.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(4 * nqmax),
        status.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(threads or _WORKERS))
    return out, status


# ------------------------------------------------------------ data formats A, B, C
# BAQ rows of the reconstruction tables and the per-mode limits
# (structs.h:292-333; BAQ modes 3, 4, 5)
_BAQ_THIDX = {3: 3, 4: 7, 5: 15}
_BAQ_MCODE = {3: 3, 4: 5, 5: 10}
_BAQ_SIMPLE = [[3.00, 3.00, 3.12, 3.55], [7.00, 7.00, 7.00, 7.17, 7.40, 7.76],
               [15.00, 15.00, 15.00, 15.00, 15.00, 15.00, 15.44, 15.56, 16.11, 16.38, 16.65]]
_BAQ_NORM = [[0.2490, 0.7680, 1.3655, 2.1864],
             [0.1290, 0.3900, 0.6601, 0.9471, 1.2623, 1.6261, 2.0793, 2.7467],
             [0.0660, 0.1985, 0.3320, 0.4677, 0.6061, 0.7487, 0.8964, 1.0510, 1.2143, 1.3896, 1.5800,
              1.7914, 2.0329, 2.3234, 2.6971, 3.2692]]


def _bits(user: bytes, start: int, n: int) -> int:
    """read_n_bits (decoding_utils.cpp:95-134): n bits MSB first; reading past
    the user data raises like the reference's out_of_range."""
    end = start + n
    if (end + 7) // 8 > len(user):
        raise IndexError("Byte index exceeded data vector size.")
    v = int.from_bytes(user[start // 8:(end + 7) // 8], "big")
    return (v >> ((8 - end % 8) % 8)) & ((1 << n) - 1)


def _sf_table():
    from sentinel1_decode_gb300 import synth  # the THIDX -> sigma factor table restated there
    return synth.THIDX_TO_SF


def decode_fixed_packet(data: bytes, p: Packet, fields: bool = False) -> np.ndarray:
    """get_signal of a data-format A/B (bypass) or C (BAQ 3/4/5) packet,
    packet.cpp:404-453, 485-666.

    fields=False restates the reference exactly, including its containers:
    the codes of each channel are appended to vectors that were created with
    128 (H_CODE()) or num_codes (H_CODE(n)) zero entries and QUAD(key, n)
    holds n default blocks before the decoded ones, so the reference reads
    zero codes where the decoded ones were meant: for A/B, quad q takes the
    codes of quad q - 128 (zero for q < 128); for C every sample of block b is
    the reconstruction of code 0 with sign 0 at the block's THIDX.  The bits
    are still all read, so a packet too short raises as the reference does.
    fields=True decodes every sample from its own fields."""
    user = data[p.offset:p.offset + p.length]
    user = user + b"\0" * (p.length - len(user))
    nq = p.num_quads
    baq = p.sh["baq_mode"]
    out = np.zeros(2 * nq, np.complex128)
    if baq == 0:
        w = (10 * nq + 15) // 16 * 16
        codes = np.zeros((4, nq), np.float64)
        for c in range(4):
            for q in range(nq):
                v = _bits(user, c * w + 10 * q, 10)
                codes[c, q] = (-1.0 if v >> 9 else 1.0) * (v & 511)
        src = np.arange(nq) if fields else np.arange(nq) - 128
        ok = src >= 0
        vals = np.zeros((4, nq))
        vals[:, ok] = codes[:, src[ok]]
        out[0::2] = vals[0] + 1j * vals[2]
        out[1::2] = vals[1] + 1j * vals[3]
        return out
    if baq not in (3, 4, 5):
        raise ValueError("BAQ Mode is invalid.")
    M = baq
    nb = (2 * nq + 255) // 256
    lim, flag = _BAQ_THIDX[M], _BAQ_MCODE[M]
    sf = _sf_table()
    bit = 0
    chans = []
    thidx = []
    for c in range(4):
        signs, mcodes = [], []
        for b in range(nb):
            if c == 2:
                thidx.append(_bits(user, bit, 8))
                bit += 8
            cnt = nq - 128 * (nb - 1) if b == nb - 1 else 128
            for _ in range(cnt):
                signs.append(_bits(user, bit, 1))
                mcodes.append(_bits(user, bit + 1, M - 1))
                bit += M
        bit = (bit + 15) // 16 * 16
        chans.append((signs, mcodes))

    def sval(th, sg, m):
        if th <= lim:
            if m < flag:
                return (-1.0) ** sg * float(m)
            if m == flag:
                return (-1.0) ** sg * _BAQ_SIMPLE[M - 3][th]
            raise ValueError("Invalid m_code in s_value generation.")
        return (-1.0) ** sg * _BAQ_NORM[M - 3][m] * sf[th]

    vals = np.zeros((4, nq))
    for q in range(nq):
        th = thidx[q // 128]
        for c in range(4):
            vals[c, q] = sval(th, chans[c][0][q], chans[c][1][q]) if fields else sval(th, 0, 0)
    out[0::2] = vals[0] + 1j * vals[2]
    out[1::2] = vals[1] + 1j * vals[3]
    return out


# ------------------------------------------------------------ state vectors
def _int_to_ieee754(number: int, is_double: bool) -> float:
    """decoding_utils.cpp:149-170 (normal numbers only)."""
    ms = 52 if is_double else 23
    emask = 0x7FF0000000000000 if is_double else 0x7F800000
    bias = 1023 if is_double else 127
    ss = 63 if is_double else 31
    sign = (number >> ss) & 1
    exponent = ((number & emask) >> ms) - bias
    total = 0.0
    power = -1
    for i in range(ms):
        total += ((number >> (ms - i - 1)) & 1) * math.pow(2.0, power)
        power -= 1
    return (-1 if sign else 1) * math.pow(2.0, exponent) * (total + 1.0)


def _parse_time_stamp(raw: int) -> float:
    """state_vectors.cpp:5-16, including its mask of the fine bits."""
    coarse = (raw >> 24) & 0xFFFFFFFF
    fine_raw = raw & 0xFFFFFF
    fine = 0.0
    for i in range(23, -1, -1):
        fine += (fine_raw >> i) * math.pow(2, i - 24)
        fine_raw &= 1 << 8
    return float(coarse) + fine


_SC_KEY = ([("dummy", 0)] + [("px", k) for k in range(4)] + [("py", k) for k in range(4)]
           + [("pz", k) for k in range(4)] + [("vx", 0), ("vx", 1), ("vy", 0), ("vy", 1), ("vz", 0), ("vz", 1)]
           + [("pod", k) for k in range(4)] + [("q%d" % (k // 2), k % 2) for k in range(8)]
           + [("w%d" % (k // 2), k % 2) for k in range(6)] + [("t", k) for k in range(4)]
           + [("other%d" % k, 0) for k in range(24)])


def _subcomm_dicts(packets: List[Packet]):
    """build_data_word_dicts, state_vectors.cpp:19-57: the raw words of every
    complete sub-commutation cycle after the first index-1 packet past
    packet 0."""
    start = 0
    while True:
        start += 1
        if packets[start].sh["sc_data_word_index"] == 1:
            break
    raw: Dict[str, int] = {}
    dicts = []
    for i in range(start, len(packets)):
        idx = packets[i].sh["sc_data_word_index"]
        if idx == 1 and i != start:
            dicts.append(raw)
            raw = {}
        key = _SC_KEY[idx][0] if idx < len(_SC_KEY) else "other"
        raw[key] = ((raw.get(key, 0) << 16) | packets[i].sh["sc_data_word"]) & 0xFFFFFFFFFFFFFFFF
    return dicts


def state_vectors(packets: List[Packet]):
    """build_data_word_dicts + parse_subcomm_dicts, state_vectors.cpp:19-83.
    Returns (times, positions[n,3], velocities[n,3])."""
    full = state_vectors_full(packets)
    return full["times"], full["positions"], full["velocities"]


def parse_attitude(q_raw):
    """parse_quaternions -> (quaternion scalar last, attitude), following
    get_eocfi_rotation_matrix (float entries), get_quaternions_from_rotation_matrix
    (float sums, double division) and Quaternion::to_euler_angles,
    state_vectors.cpp:203-320."""
    f32 = np.float32
    w, x, y, z = (float(v) for v in q_raw)
    e00 = f32(x * x - y * y - z * z + w * w)
    e01 = f32(2 * (x * y + z * w))
    e02 = f32(2 * (x * z - y * w))
    e10 = f32(2 * (x * y - z * w))
    e11 = f32(-x * x + y * y - z * z + w * w)
    e12 = f32(2 * (y * z + x * w))
    e20 = f32(2 * (x * z + y * w))
    e21 = f32(2 * (y * z - x * w))
    e22 = f32(-x * x - y * y + z * z + w * w)
    R = [[-e10, -e11, -e12], [-e00, -e01, -e02], [-e20, -e21, -e22]]
    trace = float(R[0][0] + R[1][1] + R[2][2])          # float adds, then widened
    if trace > 0:
        S = math.sqrt(trace + 1.0) * 2
        qw, qx = 0.25 * S, float(R[2][1] - R[1][2]) / S
        qy, qz = float(R[0][2] - R[2][0]) / S, float(R[1][0] - R[0][1]) / S
    elif R[0][0] > R[1][1] and R[0][0] > R[2][2]:
        S = math.sqrt(1.0 + float(R[0][0]) - float(R[1][1]) - float(R[2][2])) * 2
        qw, qx = float(R[2][1] - R[1][2]) / S, 0.25 * S
        qy, qz = float(R[0][1] + R[1][0]) / S, float(R[0][2] + R[2][0]) / S
    elif R[1][1] > R[2][2]:
        S = math.sqrt(1.0 + float(R[1][1]) - float(R[0][0]) - float(R[2][2])) * 2
        qw, qx = float(R[0][2] - R[2][0]) / S, float(R[0][1] + R[1][0]) / S
        qy, qz = 0.25 * S, float(R[1][2] + R[2][1]) / S
    else:
        S = math.sqrt(1.0 + float(R[2][2]) - float(R[0][0]) - float(R[1][1])) * 2
        qw, qx = float(R[1][0] - R[0][1]) / S, float(R[0][2] + R[2][0]) / S
        qy, qz = float(R[1][2] + R[2][1]) / S, 0.25 * S
    W, X, Y, Z = qw, -qx, -qy, -qz
    r1 = 2 * (X * Y + W * Z)
    r4 = 1 - 2 * (X * X + Z * Z)
    r5 = 2 * (Y * Z + W * X)
    r6 = 2 * (X * Z + W * Y)
    r7 = 2 * (Y * Z - W * X)
    r8 = 1 - 2 * (X * X + Y * Y)
    pitch = math.asin(-max(-1.0, min(1.0, r7)))
    if abs(r7) < 1:
        roll, yaw = math.atan2(r6, r8), math.atan2(r1, r4)
    else:
        roll, yaw = math.atan2(r5, r4), 0.0
    return [X, Y, Z, W], [-pitch, -roll, yaw]


def state_vectors_full(packets: List[Packet]):
    """Every member of STATE_VECTORS (state_vectors.h:55-120,
    parse_subcomm_dicts state_vectors.cpp:60-83): times, positions,
    velocities, quaternions (scalar last), angular_rates, attitudes."""
    out = {k: [] for k in ("times", "positions", "velocities", "quaternions", "angular_rates", "attitudes")}
    last = 0.0
    for d in _subcomm_dicts(packets):
        t = _parse_time_stamp(d.get("t", 0))
        if t > last:
            last = t
            out["times"].append(t)
            out["positions"].append([_int_to_ieee754(d.get(k, 0), True) for k in ("px", "py", "pz")])
            out["velocities"].append([_int_to_ieee754(d.get(k, 0), False) for k in ("vx", "vy", "vz")])
            out["angular_rates"].append([_int_to_ieee754(d.get(k, 0), False) for k in ("w0", "w1", "w2")])
            q, a = parse_attitude([_int_to_ieee754(d.get(k, 0), False) for k in ("q0", "q1", "q2", "q3")])
            out["quaternions"].append(q)
            out["attitudes"].append(a)
    return {k: np.array(v) for k, v in out.items()}


def interpolate_state(times, pos, vel, t: float):
    """STATE_VECTORS::interpolate, state_vectors.cpp:127-200."""
    if t > times[-1]:
        return pos[-1].copy(), vel[-1].copy()
    if t < times[0]:
        return pos[0].copy(), vel[0].copy()
    lo, hi = 0, len(times)
    while True:
        size = hi - lo
        if size == 1:
            a_i, b_i = lo, hi
            break
        pivot = size // 2
        tp = times[lo + pivot]
        if tp == t:
            a_i = b_i = lo
            break
        if tp > t:
            hi = lo + pivot
        else:
            lo = lo + pivot
    a, b = times[a_i], times[b_i]
    tt = (t - a) / (b - a) if b != a else math.nan
    p = np.array([std_lerp(pos[a_i][c], pos[b_i][c], tt) for c in range(3)])
    v = np.array([std_lerp(vel[a_i][c], vel[b_i][c], tt) for c in range(3)])
    return p, v


# ------------------------------------------------------------ DSP
def get_reference_function(chirp: np.ndarray) -> np.ndarray:
    """image_formation.cpp:4-25."""
    norm = np.abs(chirp) ** 2
    norm = norm * (norm / float(norm.size))
    energy = float(np.sum(norm))
    return np.conj(_fft(chirp)) / energy


def eccm(signals: np.ndarray, det: float, mit: float, fft_size=128, stride=64, ties=None):
    """signal_processing.cpp:914-1004, rows modified in place.  Returns the
    per-row notch mask (bins zeroed) for inspection: [rows, num_ffts, fft].
    With `ties` (a relative width), also returns a same-shaped boolean array
    marking the bins whose gradient magnitude lies within ties * mit of the
    mitigation threshold: there an FFT of other rounding may decide either
    way."""
    rows, cols = signals.shape
    num_ffts = int(math.floor((float(cols) / float(fft_size)) * (float(fft_size) / float(stride))))
    masks = np.zeros((rows, num_ffts, fft_size), dtype=bool)
    near = np.zeros((rows, num_ffts, fft_size), dtype=bool) if ties is not None else None
    maxamp = np.abs(_fft(signals, axis=1)).max(axis=1)
    for r in np.nonzero(~(maxamp < det))[0]:
        sig = signals[r]
        spec = np.zeros((num_ffts, fft_size), dtype=np.complex128)
        for i in range(num_ffts):
            s = i * stride
            e = s + fft_size
            if e > cols:
                e = cols - 1
            spec[i, :e - s] = sig[s:e]
        spec = _fft(spec, axis=1)
        grad = np.empty_like(spec)
        grad[:, 1:-1] = (spec[:, 2:] - spec[:, :-2]) / 2.0
        grad[:, 0] = spec[:, 1] - spec[:, 0]
        grad[:, -1] = spec[:, -1] - spec[:, -2]
        zero = ~(np.abs(grad) < mit)
        masks[r] = zero
        if near is not None:
            near[r] = np.abs(np.abs(grad) - mit) <= ties * mit
        spec = np.where(zero, spec * 0.0, spec * 1.0)
        spec = _ifft_unnorm(spec, axis=1) * (1.0 / fft_size)
        for i in range(num_ffts):
            s = i * stride
            e = s + fft_size
            if e > cols:
                e = cols - 1
            sig[s:e] = spec[i, :e - s]
    return (masks, near) if near is not None else masks


def eccm_flags(signals: np.ndarray, det: float) -> np.ndarray:
    """The line detection of eccm() (signal_processing.cpp:926-932): a line
    is notched unless max |DFT(line)| < det."""
    return ~(np.abs(_fft(signals, axis=1)).max(axis=1) < det)


def scale(x: np.ndarray, mode: str) -> np.ndarray:
    """scale(CF_VEC_2D, mode), signal_processing.cpp:1031-1071, with
    norm_2d / magnitude_2d (:367-400, :444-460): float32 samples of
    real, imag, |x|^2 (pow(abs, 2)), (|x| + 1e-12) / max|x| and
    20 log10 of that.  norm_2d's maximum is the true maximum (the reference
    computes it in an OpenMP loop without a reduction, which races when more
    than one thread runs; its goldens are made single-threaded)."""
    if mode == "real":
        return x.real.astype(np.float32)
    if mode == "imag":
        return x.imag.astype(np.float32)
    a = np.abs(x)
    if mode == "mag":
        return (a ** 2.0).astype(np.float32)
    if mode in ("norm", "norm_log"):
        v = (a + 1e-12) / a.max()
        return (20.0 * np.log10(v) if mode == "norm_log" else v).astype(np.float32)
    raise ValueError(mode + " is not a valid scaling mode.")


def spectrogram(line: np.ndarray, fft_size: int = 64, stride: int = 32) -> np.ndarray:
    """spectrogram(), signal_processing.cpp:794-844: Hann windows
    0.5 (1 - cos(2 PI j / (fft_size - 1))) over windows at multiples of
    stride (a window ending past the line is cut at n - 1 and zero-filled),
    DFT, fftshift (rotate by fft_size / 2), transpose -> [fft_size, windows]."""
    n = line.size
    nwin = int(math.floor((float(n) / float(fft_size)) * (float(fft_size) / float(stride))))
    hann = 0.5 * (1.0 - np.cos(2.0 * PI * np.arange(fft_size, dtype=np.float64) / (float(fft_size) - 1)))
    spec = np.zeros((nwin, fft_size), np.complex128)
    for i in range(nwin):
        s = i * stride
        e = s + fft_size
        if e > n:
            e = n - 1
        spec[i, :e - s] = line[s:e]
    spec = _fft(spec * hann[None, :], axis=1)
    return np.ascontiguousarray(fftshift_rows(spec, axis=1).T)


def sinc_interpolate(signal: np.ndarray, t: np.ndarray, L: int = 8) -> np.ndarray:
    """sinc_interpolate(signal, t, L), signal_processing.cpp:228-257, at
    every position of t: sum over idx = floor(t) + k, k = -L..L, idx inside
    the signal, of signal[idx] * sinc(t - idx) * hann(t - idx), with
    sinc(x) = sin(PI x) / (PI x) (1 at x = 0) and hann(x) = 0.5 (1 +
    cos(PI x / L)) -- the raised cosine is not cut at |x| = L, so all 2L + 1
    taps count."""
    t = np.asarray(t, dtype=np.float64)
    n0 = np.floor(t).astype(np.int64)
    out = np.zeros(t.shape, np.complex128)
    for k in range(-L, L + 1):
        idx = n0 + k
        ok = (idx >= 0) & (idx < signal.size)
        x = t - idx
        with np.errstate(invalid="ignore", divide="ignore"):
            sc = np.where(x == 0.0, 1.0, np.sin(PI * x) / (PI * x))
        w = 0.5 * (1.0 + np.cos(PI * x / L))
        out = out + np.where(ok, signal[np.clip(idx, 0, signal.size - 1)] * sc * w, 0.0)
    return out


def range_compress(data: bytes, packets: List[Packet], do_azimuth_fft=False, eccm_thresholds=None,
                   return_mask=False):
    """S1_Decoder::_range_compress, s1_decoder.cpp:448-508 (do_ifft=true)."""
    raw, status = decode_packets(data, packets)
    if status.any():
        raise RuntimeError("decode error status %d" % int(status[status != 0][0]))
    n_r = 2 * packets[0].num_quads
    rc = raw[:, :n_r].copy()
    mask = None
    if eccm_thresholds is not None:
        mask = eccm(rc, float(eccm_thresholds[0]), float(eccm_thresholds[1]))
    L = packets[0].get_replica_chirp_length()
    M = n_r + 2 * L
    padded = np.zeros((rc.shape[0], M), dtype=np.complex128)
    padded[:, L:L + n_r] = rc
    spec = _fft(padded, axis=1)
    ref = get_reference_function(packets[0].get_replica_chirp())
    spec *= ref[None, :]
    out = _ifft_unnorm(spec, axis=1) * (1.0 / M)
    out = fftshift_rows(out, axis=1)[:, L:M - L]
    if do_azimuth_fft:
        out = fftshift_rows(_fft(out, axis=0), axis=0)
    out = np.ascontiguousarray(out)
    return (out, mask) if return_mask else out


def polyfit2(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """signal_processing.cpp:159-214 (normal equations + partial pivoting)."""
    Sx = [0.0] * 5
    Sy = [0.0] * 3
    for i in range(len(x)):
        xi = 1.0
        for j in range(5):
            if j <= 2:
                Sy[j] += xi * y[i]
            Sx[j] += xi
            xi *= x[i]
    A = [[Sx[0], Sx[1], Sx[2]], [Sx[1], Sx[2], Sx[3]], [Sx[2], Sx[3], Sx[4]]]
    b = [Sy[0], Sy[1], Sy[2]]
    for i in range(3):
        for k in range(i + 1, 3):
            if abs(A[k][i]) > abs(A[i][i]):
                A[i], A[k] = A[k], A[i]
                b[i], b[k] = b[k], b[i]
        for k in range(i + 1, 3):
            f = A[k][i] / A[i][i]
            for j in range(i, 3):
                A[k][j] -= f * A[i][j]
            b[k] -= f * b[i]
    c = [0.0] * 3
    for i in range(2, -1, -1):
        c[i] = b[i]
        for j in range(i + 1, 3):
            c[i] -= A[i][j] * c[j]
        c[i] /= A[i][i]
    return np.array(c)


def doppler_centroid_rate(packets: List[Packet], velocity: float) -> float:
    """doppler.cpp:224-232."""
    pri = packets[0].get_pri() * 1e-6
    a0 = packets[0].get_azimuth_beam_angle()
    a1 = packets[-1].get_azimuth_beam_angle()
    rate = (a1 - a0) / (pri * len(packets))
    return (-2 * velocity * rate) / WAVELENGTH


def wrapped_sums(rc: np.ndarray, rate: float) -> np.ndarray:
    """dce_preconditioning + the lag-1 sums of get_wrapped_estimates
    (doppler.cpp:4-39, 98-143) with the hard-coded 1.06 s duration."""
    n_az = rc.shape[0]
    t = linspace(0.0, 1.06, n_az)
    theta = (PI * rate) * np.power(t - (0.5 * 1.06), 2.0)
    deramp = cexp_i(theta)
    pre = rc * deramp[:, None]
    return np.sum(pre[:-1] * np.conj(pre[1:]), axis=0)


def doppler_centroid_from_sums(sums: np.ndarray, first: Packet, prf_unused=None, num_blocks=30):
    """get_doppler_centroid after the lag-1 sums (doppler.cpp:146-221), with
    get_unwrapped_estimates (doppler.cpp:42-95) and polyfit."""
    n_rng = sums.size
    prf = 1.0 / (first.get_pri() * 1e-6)
    wrapped = -prf * np.arctan2(sums.imag, sums.real) / (2 * PI)
    bs = n_rng // num_blocks
    fine = np.zeros(num_blocks)
    for b in range(num_blocks):
        s = b * bs
        e = s + bs if s + bs < n_rng else n_rng - 1
        fine[b] = float(np.sum(wrapped[s:e])) / (float(e) - float(s))
    rt = first.get_slant_range_times(num_blocks)
    rt = rt - rt[0]
    # get_unwrapped_estimates
    dense = 8
    dt = float(np.float32(rt[1] - rt[0]))
    F = np.zeros(num_blocks * dense, dtype=np.complex128)
    F[:num_blocks] = np.floor(np.abs(cexp_i((2.0 * PI) * fine / prf)))
    F = np.fft.fft(F)
    mag2 = np.abs(F) * np.abs(F)
    mi = int(np.argmax(mag2))
    n = num_blocks * dense
    val = 1.0 / (n * dt)
    N = (n - 1) // 2 + 1
    freqs = np.array([i * val if i < N else (i - n) * val for i in range(n)])
    v = freqs[mi]
    a = v / dt
    b = float(np.arctan2(F[mi].imag, F[mi].real)) / (2.0 * PI)
    r1 = cexp_i((2.0 * PI) * fine / prf)
    r2 = cexp_i(-1.0 * (a * rt + b))
    prod = r1 * r2
    res = np.arctan2(prod.imag, prod.real) / (2.0 * PI)
    unwrapped = (a * rt + b + res) * prf
    poly = polyfit2(rt, unwrapped)
    t = first.get_slant_range_times(n_rng)
    t = t - t[0]
    return poly[0] + poly[1] * t + poly[2] * t * t


def tiled(sig: np.ndarray, num_replicas: float, axis=0) -> np.ndarray:
    """get_tiled_signal, image_formation.cpp:87-122 (along `axis`).  Writes
    that would fall past the tiled length are dropped."""
    num_az = sig.shape[axis]
    shape = int(math.floor(num_replicas * num_az))
    offset = int(math.floor(num_replicas))
    out_shape = list(sig.shape)
    out_shape[axis] = shape
    out = np.zeros(out_shape, dtype=sig.dtype)
    sl = [slice(None)] * sig.ndim
    for i in range(offset):
        lo = i * num_az
        hi = min(lo + num_az, shape)
        if hi <= lo:
            break
        sl[axis] = slice(lo, hi)
        src = [slice(None)] * sig.ndim
        src[axis] = slice(0, hi - lo)
        out[tuple(sl)] = sig[tuple(src)]
    if math.floor(num_replicas) != num_replicas:
        ns = int(math.floor((num_replicas - math.floor(num_replicas)) * num_az))
        lo = offset * num_az
        hi = min(lo + ns, shape)
        if hi > lo:
            sl[axis] = slice(lo, hi)
            src = [slice(None)] * sig.ndim
            src[axis] = slice(0, hi - lo)
            out[tuple(sl)] = sig[tuple(src)]
    return out


def azimuth_frequency_ufr(rc: np.ndarray, dc_rate: float, burst_duration: float, prf: float,
                          doppler_bandwidth: float) -> np.ndarray:
    """image_formation.cpp:125-219.  rc: [N_a, N_r] -> [S, N_r]."""
    num_az = rc.shape[0]
    x = fftshift_rows(_fft(rc, axis=0), axis=0)
    num_replicas = abs(dc_rate * burst_duration / prf)
    bandwidth = num_replicas * prf / 2.0
    shape = int(math.floor(num_replicas * num_az))
    mid = shape // 2
    start = int(mid - (math.floor(doppler_bandwidth) / 2))
    end = int(mid + (math.floor(doppler_bandwidth) / 2))
    f = linspace(-bandwidth, bandwidth, shape)
    inv_rate = 1 / dc_rate
    y = tiled(x, num_replicas, axis=0)
    y *= cexp_i((-PI * inv_rate) * np.power(f, 2.0))[:, None]
    Y = _fft(y, axis=0)
    Z = np.zeros_like(Y)
    Z[:end - start] = Y[start:end]
    z = _ifft_unnorm(Z, axis=0) * (1.0 / shape)
    z *= cexp_i((PI * inv_rate) * np.power(f, 2.0))[:, None]
    return z


def effective_velocities(position, velocity, slant_ranges):
    """image_formation.cpp:391-419 (lat = z/x as written)."""
    lat = position[2] / position[0]
    num = math.pow(SEMI_MAJOR * SEMI_MAJOR * math.cos(lat), 2.0) + math.pow(SEMI_MINOR * SEMI_MINOR * math.sin(lat), 2.0)
    den = math.pow(SEMI_MAJOR * math.cos(lat), 2.0) + math.pow(SEMI_MINOR * math.sin(lat), 2.0)
    re = math.sqrt(num / den)
    h = math.sqrt(position[0] * position[0] + position[1] * position[1] + position[2] * position[2])
    beta = (re * re + h * h - slant_ranges * slant_ranges) / (2 * re * h)
    vg = re * velocity * beta / h
    return np.sqrt(velocity * vg)


def linear_resample(arr: np.ndarray, n_out: int) -> np.ndarray:
    """signal_processing.cpp:32-67 with its accumulated x grid.  Works on the
    last axis of a 2-D array (rows resampled independently)."""
    n_in = arr.shape[-1]
    if n_in == n_out:
        return arr.copy()
    dx_in = 1.0 / (n_in - 1)
    dx_out = 1.0 / (n_out - 1)
    steps = np.full(n_out, dx_out)
    steps[0] = 0.0
    x = np.add.accumulate(steps)
    x1 = (np.arange(n_in - 1) + 1) * dx_in
    seg = np.searchsorted(x1, x, side="right")
    valid = seg < n_in - 1
    segc = np.minimum(seg, n_in - 2)
    x0 = segc * dx_in
    x1s = (segc + 1) * dx_in
    y0 = arr[..., segc]
    y1 = arr[..., segc + 1]
    out = y0 + ((x - x0) * (y1 - y0) / (x1s - x0))
    out = np.where(valid, out, 0.0)
    out[..., n_out - 1] = arr[..., n_in - 1]
    return out


def quadratic_resample(arr: np.ndarray, n_out: int) -> np.ndarray:
    """signal_processing.cpp:109-155 on the last axis (3-point Lagrange)."""
    n_in = arr.shape[-1]
    if n_in == n_out:
        return arr.copy()
    dx_in = 1.0 / (n_in - 1)
    dx_out = 1.0 / (n_out - 1)
    x = np.arange(n_out) * dx_out
    i = np.minimum((x / dx_in).astype(np.int64), n_in - 2)
    i0 = np.maximum(i - 1, 0)
    i1 = i
    i2 = np.minimum(i + 1, n_in - 1)
    x0, x1, x2 = i0 * dx_in, i1 * dx_in, i2 * dx_in
    with np.errstate(divide="ignore", invalid="ignore"):
        L0 = (x - x1) * (x - x2) / ((x0 - x1) * (x0 - x2))
        L1 = (x - x0) * (x - x2) / ((x1 - x0) * (x1 - x2))
        L2 = (x - x0) * (x - x1) / ((x2 - x0) * (x2 - x1))
        return L0 * arr[..., i0] + L1 * arr[..., i1] + L2 * arr[..., i2]


def azimuth_time_ufr(az: np.ndarray, dc: np.ndarray, ka: np.ndarray, dc_rate: float, burst_duration: float,
                     prf: float, doppler_bandwidth: float, swath_number: int) -> np.ndarray:
    """image_formation.cpp:222-388.  az, ka: [S, N_r]."""
    azT = az.T  # [N_r, S]
    kaT = ka.T
    num_az = azT.shape[1]
    num_rng = azT.shape[0]
    num_replicas = abs(dc_rate * burst_duration / prf)
    bandwidth = (num_replicas * prf) - doppler_bandwidth
    ka_mean = abs(float(np.add.accumulate(kaT[0])[-1])) / num_az
    focused_time = burst_duration + ((bandwidth - (2 * doppler_bandwidth)) / ka_mean)
    if num_az // 2 < num_rng and num_rng // 2 < num_az:
        ka_ref = kaT[num_az // 2][num_rng // 2]
    else:  # the reference reads outside the array here; use the intended element
        ka_ref = kaT[num_rng // 2][num_az // 2]
    n_ref = dc[num_rng // 2] / ka_ref
    focused_time *= 0.9 if swath_number != 11 else 1.05
    pos = int(math.ceil((n_ref + focused_time / 2) / burst_duration))
    neg = int(math.floor((n_ref - focused_time / 2) / burst_duration))
    num_tiles = pos - neg
    ext = int(math.floor(doppler_bandwidth * 1.15)) if swath_number == 11 else int(math.floor(doppler_bandwidth * 0.26))
    output_shape = int(math.floor(prf * burst_duration))
    down = output_shape + ext
    shape = num_tiles * num_az
    mid = shape // 2
    start = int(mid - bandwidth / 2)
    end = int(mid + bandwidth / 2)
    az_times = linspace(-focused_time / 2, focused_time / 2, shape)
    az_times2 = linspace(n_ref - focused_time / 2, n_ref + focused_time / 2, down)
    out = np.empty((num_rng, down), dtype=np.complex128)
    chunk = max(1, int(2 ** 27 // max(shape, 1) // 16))   # ~128 MB per complex work array
    for r0 in range(0, num_rng, chunk):
        r1 = min(num_rng, r0 + chunk)
        kk = linear_resample(kaT[r0:r1], shape)
        y = np.tile(azT[r0:r1], (1, num_tiles))
        kt = -kk * dc_rate / (dc_rate - kk)
        dct = -dc[r0:r1, None] / kk
        t = dct + az_times[None, :]
        th1 = ((-PI) * kt) * np.power(t, 2.0)
        th2 = (((2.0 * PI) * (kt + kk)) * dct) * t
        y *= cexp_i(th1 + th2)
        del kk, kt, dct, t, th1, th2
        Y = _fft(y, axis=1)
        Z = np.zeros_like(Y)
        Z[:, :end - start] = Y[:, start:end]
        del Y, y
        z = _ifft_unnorm(Z, axis=1) * (1.0 / shape)
        del Z
        o = quadratic_resample(z, down)
        del z
        kk = linear_resample(kaT[r0:r1], down)
        kt = -kk * dc_rate / (dc_rate - kk)
        dct = -dc[r0:r1, None] / kk
        t = dct + az_times2[None, :]
        th1 = (PI * kt) * np.power(t, 2.0)
        th2 = (((2.0 * PI) * (kt + kk)) * dct) * t
        o *= cexp_i(th1 - th2)
        out[r0:r1] = o
    out = out.T
    mid = down // 2
    s = mid - (output_shape // 2)
    e = mid + (output_shape // 2)
    return np.ascontiguousarray(out[s:e]), dict(num_tiles=num_tiles, shape=shape, down=down,
                                                 n_ref=n_ref, focused_time=focused_time)


def azimuth_compress(data: bytes, packets: List[Packet], sv, tops_mode: bool, eccm_thresholds=None,
                     return_info=False, rcmc=("phase", 4)):
    """S1_Decoder::_azimuth_compress, s1_decoder.cpp:511-701.

    rcmc = ("sinc", L) replaces the reference's phase RCMC of the TOPS row
    pass by a shift of every range line to j + 2 R_j (1/D - 1) f_s / c
    samples with sinc_interpolate (half-width L), before the azimuth filter:
    the library's S1G_RCMC_SINC option, which has no reference counterpart."""
    times, poss, vels = sv
    first = packets[0]
    num_packets = len(packets)
    n_r = 2 * first.num_quads
    radar = range_compress(data, packets, do_azimuth_fft=not tops_mode, eccm_thresholds=eccm_thresholds)
    slant = first.get_slant_ranges()
    v0 = vels[0]
    swath_number = first.sh["swath_number"]
    v_norm = math.sqrt(math.pow(v0[0], 2.0) + math.pow(v0[1], 2.0) + math.pow(v0[2], 2.0))
    pri = first.get_pri() * 1e-6
    prf = 1 / pri
    T = float(num_packets) / prf
    bd = 675.0 if swath_number == 11 else 600.0
    t0 = first.get_time()
    time_delta = T / prf
    fs = first.get_range_sample_rate() * 1e6
    range_freqs = linspace(-fs / 2, fs / 2, n_r)
    dc = np.zeros(n_r)
    info = {}
    if tops_mode:
        dc_rate = doppler_centroid_rate(packets, v_norm)
        sums = wrapped_sums(radar, dc_rate)
        dc = doppler_centroid_from_sums(sums, first)
        radar = azimuth_frequency_ufr(radar, dc_rate, T, prf, bd)
        num_packets = radar.shape[0]
        time_delta /= float(num_packets) / float(len(packets))
        info.update(dc_rate=dc_rate, dc=dc, S=num_packets)
    S = num_packets
    positions = np.zeros((S, 3))
    vnorm = np.zeros(S)
    for i in range(S):
        p, v = interpolate_state(times, poss, vels, t0 + time_delta * i)
        positions[i] = p
        vnorm[i] = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    if tops_mode:
        nrep = abs(dc_rate * T / prf)
        az_freqs = linspace(-nrep * prf / 2, nrep * prf / 2, S)
    else:
        az_freqs = linspace(-prf / 2, prf / 2, S)
    tc = first.get_timing_corrections()
    ref_range = slant[n_r // 2]
    ka = np.zeros((S, n_r)) if tops_mode else None
    if tops_mode:
        radar = _fft(radar, axis=1)
    # per-row SRC / IFFT / scale / RCMC / azimuth filter (s1_decoder.cpp:616-677)
    veff = np.stack([effective_velocities(positions[i], vnorm[i], slant) for i in range(S)])
    fa = az_freqs[:, None] + dc[None, :]
    D = np.sqrt(1 - ((math.pow(WAVELENGTH, 2.0) * np.power(fa, 2.0)) / (4 * veff * veff)))
    with np.errstate(divide="ignore"):
        ksrc = 2.0 * np.power(veff, 2.0) * math.pow(CENTER_FREQ, 3.0) * np.power(D, 2.0)
        ksrc = ksrc / (SPEED_OF_LIGHT * slant[None, :] * np.power(fa, 2.0))
        radar *= cexp_i(((-PI) * np.power(range_freqs, 2.0))[None, :] / ksrc)
    radar = _ifft_unnorm(radar, axis=1)
    radar /= np.sqrt(np.power(ref_range / slant, 3.0))[None, :]
    if tops_mode and rcmc[0] == "sinc":
        mig = ((slant[None, :] / D) - slant[None, :]) * (2.0 * fs / SPEED_OF_LIGHT)
        pos = np.arange(n_r, dtype=np.float64)[None, :] + mig
        radar = np.stack([sinc_interpolate(radar[i], pos[i], rcmc[1]) for i in range(S)])
    elif tops_mode:
        shift = (slant[None, :] / D) - slant[None, :]
        radar *= cexp_i(((((-4.0) * PI) * range_freqs[None, :]) * shift) / SPEED_OF_LIGHT)
    tcorr = cexp_i(((2.0 * PI) * fa) * tc[None, :])
    azf = cexp_i((((4.0 * PI) * slant[None, :]) * D) / WAVELENGTH) * tcorr
    if tops_mode:
        ka[:] = (-2 * np.power(veff, 2.0) * np.power(D, 3.0)) / (WAVELENGTH * slant[None, :])
    radar *= azf
    del azf, tcorr, D, veff, fa
    radar = _ifft_unnorm(radar, axis=0) * (1.0 / S)
    if tops_mode:
        radar, tinfo = azimuth_time_ufr(radar, dc, ka, dc_rate, T, prf, bd, swath_number)
        info.update(tinfo)
    return (radar, info) if return_info else radar


# ------------------------------------------------------------ decoder facade
class S1Decoder:
    """Mirror of S1_Decoder (s1_decoder.h:13-77) over the restated functions."""

    def __init__(self, data: bytes):
        self.data = data
        self.packets = get_packets(data)
        counts: Dict[str, int] = {}
        for p in self.packets:
            counts[p.get_swath()] = counts.get(p.get_swath(), 0) + 1
        self.swath_counts = counts
        self.echo = {s: get_packets_in_bursts(self.packets, s) for s in counts if s in ECHO_SWATHS}
        self.sv = state_vectors(self.packets)
        self.eccm = None
        self.rcmc = ("phase", 4)

    def apply_eccm(self, det: int, mit: int):
        self.eccm = (det, mit)

    def get_burst(self, swath, burst):
        pk = self.echo[swath][burst]
        raw, status = decode_packets(self.data, pk)
        return raw[:, :2 * pk[0].num_quads]

    def get_range_compressed_burst(self, swath, burst, range_doppler=False):
        return range_compress(self.data, self.echo[swath][burst], range_doppler, self.eccm)

    def set_rcmc(self, mode: str, half_width: int = 4):
        self.rcmc = (mode, half_width)

    def get_azimuth_compressed_burst(self, swath, burst):
        return azimuth_compress(self.data, self.echo[swath][burst], self.sv, True, self.eccm, rcmc=self.rcmc)

    def get_azimuth_compressed_swath_sm(self, swath):
        pk = self.echo[swath][0]
        blocks = _azimuth_blocks(pk)
        if len(blocks) == 1:
            return azimuth_compress(self.data, blocks[0], self.sv, False, self.eccm)
        raise NotImplementedError("multi-block stripmap")

    def get_azimuth_compressed_swath_iw(self, swath):
        rows = []
        for pk in self.echo[swath]:
            if len(pk) < 1000:
                continue
            a = azimuth_compress(self.data, pk, self.sv, True, self.eccm)
            rows.extend(list(a))
            rows.extend([np.zeros(rows[0].size, dtype=np.complex128)] * 20)
        return rows


def _azimuth_blocks(packets: List[Packet]):
    """get_azimuth_blocks, image_formation.cpp:46-84 (split on NQ changes)."""
    blocks, cur = [], []
    prev = 2 * packets[0].num_quads
    for p in packets:
        size = 2 * p.num_quads
        if size != prev and cur:
            blocks.append(cur)
            cur = []
            prev = size
        cur.append(p)
    if cur:
        blocks.append(cur)
    return blocks


def read_ref_dump(path: str):
    """Read the reference driver's FP64 product dump (rows may be ragged)."""
    with open(path, "rb") as f:
        assert f.read(4) == b"S1GR"
        rows = int(np.frombuffer(f.read(8), dtype=np.int64)[0])
        out = []
        for _ in range(rows):
            n = int(np.frombuffer(f.read(8), dtype=np.int64)[0])
            out.append(np.frombuffer(f.read(16 * n), dtype=np.complex128))
    return out
