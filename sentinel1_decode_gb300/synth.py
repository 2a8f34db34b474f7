"""Seeded synthetic Sentinel-1 Level-0 generator.

Writes CCSDS space packets (6-byte primary + 62-byte secondary header + FDBAQ
user data) that the reference's packet reader accepts unchanged, so the
reference and this library can be run on identical inputs.  It inverts the
decoder's bit layout:

* header field widths: structs.h:42-115 (primary / secondary header tables);
* FDBAQ (baq_mode 12, data format D): channels IE, IO, QE, QO in that order,
  blocks of 128 quads, a 3-bit BRC before each IE block and an 8-bit THIDX
  before each QE block, every sample a sign bit then the BRC's Huffman code,
  each channel padded to a 16-bit word (packet.cpp:779-818, 468-473);
* reconstruction tables used to quantise (structs.h:295-354, packet.cpp:678-693);
* sub-commutated ancillary words carrying ECEF position/velocity and the
  data time stamp (structs.h:578-688, state_vectors.cpp:19-57);
* radar parameters as header fields (packet.cpp:29-100, 284-318).

The scene is point targets (range chirp at the target delay times an azimuth
phase history, TOPS-windowed for IW) over complex-Gaussian clutter, with
optional RFI (tones + a chirped interferer) and an azimuth phase error.
Nothing here is used by the processing path; it only makes inputs.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

# ---------------------------------------------------------------- constants
# Physical constants restated from structs.h:23-34 (PI is truncated there on
# purpose; the generator uses numpy's pi, only the decoder side must match).
SPEED_OF_LIGHT = 299792458.0
CENTER_FREQ = 5.405000454334350e9
WAVELENGTH = SPEED_OF_LIGHT / CENTER_FREQ
F_REF = 37.53472224  # MHz
DELTA_T_SUPPRESSED = (320 / (8 * F_REF)) * 1e-6
RANGE_DECIMATION_MHZ = {8: 64.34523813, 0: 112.6041667, 1: 100.0925926, 3: 83.41049387,
                        4: 66.72839509, 5: 56.30208336, 6: 50.04629632, 7: 25.02314816,
                        9: 46.91840280, 10: 17.32371796, 11: 54.59595962}

PRIMARY_WIDTHS = [3, 1, 1, 7, 4, 2, 14, 16]
SECONDARY_FIELDS = [
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
    ("na_8", 3), ("swap", 1), ("swath_number", 8), ("num_quadratures", 16), ("na_9", 8),
]
assert sum(w for _, w in SECONDARY_FIELDS) == 62 * 8
SYNC_MARKER = 0x352EF853

# FDBAQ Huffman code words (value, length) per BRC and m-code: the trees of
# the SAR SPPDU document as keyed in structs.h:170-227.
HUFFMAN = [
    [(0b0, 1), (0b10, 2), (0b110, 3), (0b111, 3)],
    [(0b0, 1), (0b10, 2), (0b110, 3), (0b1110, 4), (0b1111, 4)],
    [(0b0, 1), (0b10, 2), (0b110, 3), (0b1110, 4), (0b11110, 5), (0b111110, 6), (0b111111, 6)],
    [(0b00, 2), (0b01, 2), (0b10, 2), (0b110, 3), (0b1110, 4), (0b11110, 5), (0b111110, 6),
     (0b1111110, 7), (0b11111110, 8), (0b11111111, 8)],
    [(0b00, 2), (0b010, 3), (0b011, 3), (0b100, 3), (0b101, 3), (0b1100, 4), (0b1101, 4),
     (0b1110, 4), (0b11110, 5), (0b111110, 6), (0b11111100, 8), (0b11111101, 8),
     (0b111111100, 9), (0b111111101, 9), (0b111111110, 9), (0b111111111, 9)],
]
BRC_TO_THIDX = [3, 3, 5, 6, 8]
BRC_TO_M_CODE = [3, 4, 6, 9, 15]
SIMPLE_RECONSTRUCTION = np.array([
    [3.0000, 3.0000, 3.1600, 3.5300] + [0.0] * 13,
    [4.0000, 4.0000, 4.0800, 4.3700] + [0.0] * 13,
    [6.0000, 6.0000, 6.0000, 6.1500, 6.5000, 6.8800] + [0.0] * 11,
    [9.0000, 9.0000, 9.0000, 9.0000, 9.3600, 9.5000, 10.1000] + [0.0] * 10,
    [15.0000, 15.0000, 15.0000, 15.0000, 15.0000, 15.0000, 15.2200, 15.5000, 16.0600] + [0.0] * 8,
])
NORMALIZED_RECONSTRUCTION = np.array([
    [0.3637, 1.0915, 1.8208, 2.6406] + [0.0] * 12,
    [0.3042, 0.9127, 1.5216, 2.1313, 2.8426] + [0.0] * 11,
    [0.2305, 0.6916, 1.1528, 1.6140, 2.0754, 2.5369, 3.1191] + [0.0] * 9,
    [0.1702, 0.5107, 0.8511, 1.1916, 1.5321, 1.8726, 2.2131, 2.5536, 2.8942, 3.3744] + [0.0] * 6,
    [0.1130, 0.3389, 0.5649, 0.7908, 1.0167, 1.2428, 1.4687, 1.6947, 1.9206, 2.1466, 2.3725,
     2.5985, 2.8244, 3.0504, 3.2764, 3.6623],
])
# THIDX -> sigma factor (structs.h:338-354): 0.627/step up to 100, then 1.2545/step.
_SF = [0.00, 0.63, 1.25, 1.88, 2.51, 3.13, 3.76, 4.39, 5.01, 5.64, 6.27, 6.89, 7.52, 8.15, 8.77,
       9.40, 10.03, 10.65, 11.28, 11.91, 12.53, 13.16, 13.79, 14.41, 15.04, 15.67, 16.29, 16.92,
       17.55, 18.17, 18.80, 19.43, 20.06, 20.68, 21.31, 21.93, 22.56, 23.19, 23.81, 24.44, 25.06,
       25.69, 26.32, 26.94, 27.57, 28.20, 28.83, 29.45, 30.08, 30.71, 31.33, 31.96, 32.59, 33.21,
       33.84, 34.47, 35.09, 35.72, 36.35, 36.97, 37.60, 38.23, 38.85, 39.48, 40.11, 40.73, 41.36,
       41.99, 42.61, 43.24, 43.87, 44.49, 45.12, 45.75, 46.37, 47.00, 47.63, 48.25, 48.88, 49.51,
       50.13, 50.76, 51.39, 52.01, 52.64, 53.27, 53.89, 54.52, 55.15, 55.77, 56.40, 57.03, 57.65,
       58.28, 58.91, 59.54, 60.16, 60.79, 61.41, 62.04, 62.98, 64.24, 65.49, 66.74, 68.00, 69.25,
       70.50, 71.76, 73.01, 74.26, 75.52, 76.77, 78.02, 79.28, 80.53, 81.78, 83.04, 84.29, 85.54,
       86.80, 88.05, 89.30, 90.56, 91.81, 93.07, 94.32, 95.57, 96.83, 98.08, 99.33, 100.58,
       101.84, 103.09, 104.34, 105.60, 106.85, 108.10, 109.36, 110.61, 111.86, 113.11, 114.37,
       115.62, 116.87, 118.13, 119.38, 120.63, 121.89, 123.14, 124.39, 125.65, 126.90, 128.15,
       129.41, 130.66, 131.91, 133.17, 134.42, 135.67, 136.93, 138.18, 139.43, 140.69, 141.94,
       143.19, 144.45, 145.70, 146.95, 148.21, 149.46, 150.71, 151.97, 153.22, 154.47, 155.73,
       156.98, 158.23, 159.49, 160.74, 161.99, 163.25, 164.50, 165.75, 167.01, 168.26, 169.51,
       170.77, 172.02, 173.27, 174.53, 175.78, 177.03, 178.29, 179.54, 180.79, 182.05, 183.30,
       184.55, 185.81, 187.06, 188.31, 189.57, 190.82, 192.07, 193.33, 194.58, 195.83, 197.09,
       198.34, 199.59, 200.85, 202.10, 203.35, 204.61, 205.86, 207.11, 208.37, 209.62, 210.87,
       212.13, 213.38, 214.63, 215.89, 217.14, 218.39, 219.65, 220.90, 222.15, 223.41, 224.66,
       225.91, 227.17, 228.42, 229.67, 230.93, 232.18, 233.43, 234.69, 235.94, 237.19, 238.45,
       239.70, 240.95, 242.21, 243.46, 244.71, 245.97, 247.22, 248.47, 249.73, 250.98, 252.23,
       253.49, 254.74, 255.99, 255.99]
THIDX_TO_SF = np.array(_SF[:256])

SWATH_NUMBERS = {"S1": 0, "S2": 1, "S3": 2, "S4": 3, "S5_N": 4, "S5_S": 5, "S6": 6,
                 "IW1": 10, "IW2": 11, "IW3": 12}


# ------------------------------------------------------------ configuration
@dataclasses.dataclass
class RadarParams:
    """Physical radar parameters, realised as header fields (packet.cpp:29-100)."""
    prf_hz: float = 1717.0
    pulse_length_us: float = 40.0
    ramp_rate_mhz_per_us: float = 0.79
    range_decimation: int = 8
    slant_range_mid_m: float = 850e3
    velocity_mps: float = 7600.0

    def fields(self, num_quads: int) -> dict:
        pri = int(round(F_REF * 1e6 / self.prf_hz))
        pri_us = pri / F_REF
        pulse_length = int(round(self.pulse_length_us * F_REF))
        txpl = pulse_length / F_REF
        mag = int(round(abs(self.ramp_rate_mhz_per_us) * 2097152 / F_REF ** 2))
        txprr = mag * F_REF ** 2 / 2097152 * (1 if self.ramp_rate_mhz_per_us >= 0 else -1)
        # centred chirp: TXPSF = -B/2 (packet.cpp:74-80 adds txprr/(4 F_REF))
        start = -0.5 * txprr * txpl - txprr / (4 * F_REF)
        psf_mag = int(round(abs(start) * 16384 / F_REF))
        fs_hz = RANGE_DECIMATION_MHZ[self.range_decimation] * 1e6
        n_r = 2 * num_quads
        delay_mid = 2 * self.slant_range_mid_m / SPEED_OF_LIGHT
        delay_near = delay_mid - 0.5 * n_r / fs_hz
        rank = int((delay_near - DELTA_T_SUPPRESSED) // (pri_us * 1e-6))
        swst_s = delay_near - DELTA_T_SUPPRESSED - rank * pri_us * 1e-6
        swst = int(round(swst_s * 1e6 * F_REF))
        swl = int(round(n_r / fs_hz * 1e6 * F_REF))
        return dict(pri=pri, pulse_length=pulse_length,
                    tx_ramp_rate_sign=1 if self.ramp_rate_mhz_per_us >= 0 else 0,
                    tx_ramp_rate_mag=mag,
                    pulse_start_frequency_sign=0 if start < 0 else 1,
                    pulse_start_frequency_mag=psf_mag,
                    range_decimation=self.range_decimation, rank=rank, swst=swst, swl=swl)


def decoded_params(f: dict, num_quads: int) -> dict:
    """Header fields -> physical values exactly as packet.cpp:29-100,284-318."""
    txprr = (1 if f["tx_ramp_rate_sign"] else -1) * f["tx_ramp_rate_mag"] * (F_REF ** 2 / 2097152)
    txpsf = (1 if f["pulse_start_frequency_sign"] else -1) * f["pulse_start_frequency_mag"] * (
        F_REF / 16384) + txprr / (4 * F_REF)
    txpl = f["pulse_length"] / F_REF
    fs = RANGE_DECIMATION_MHZ[f["range_decimation"]]
    pri = f["pri"] / F_REF * 1e-6
    delay_near = f["rank"] * pri + f["swst"] / F_REF * 1e-6 + DELTA_T_SUPPRESSED
    return dict(txprr=txprr, txpsf=txpsf, txpl=txpl, fs_mhz=fs, pri=pri,
                delay_near=delay_near, replica_len=int(math.floor(fs * txpl)),
                n_r=2 * num_quads)


@dataclasses.dataclass
class BurstSpec:
    num_lines: int
    num_quads: int
    swath: str = "IW2"
    beam_start: int = 100        # azimuth beam address of the first line
    beam_sweep: int = 820        # total address change over the burst (IW); 0 = stripmap
    gap_lines: int = 300         # PRI-count gap before this burst
    num_targets: int = 50
    snr_db: float = 15.0
    rfi: bool = False
    phase_error: bool = False
    dc_offset_hz: float = 0.0
    baq_mode: int = 12           # 12 FDBAQ (format D); 0 bypass (A/B); 3, 4, 5 BAQ (C)
    test_mode: int = 0           # with baq_mode 0: test_mode % 3 == 0 -> format A, else B


@dataclasses.dataclass
class StreamSpec:
    bursts: List[BurstSpec]
    seed: int = 0
    radar: RadarParams = dataclasses.field(default_factory=RadarParams)
    polarisation: str = "VV"
    clutter_sigma: float = 6.0
    start_time: float = 1_000_000.3
    sv_cycle_step: Optional[float] = None   # if set, cycle c is stamped floor(start_time) + c * step (s)
    attitude: bool = False       # write a varying attitude quaternion and angular rates


# ---------------------------------------------------------------- bit packing
def _pack_fields(values: np.ndarray, widths: np.ndarray, offsets: np.ndarray, total_bits: int) -> np.ndarray:
    """Write each (value, width) MSB-first at its bit offset into a bit array."""
    bits = np.zeros(total_bits, dtype=np.uint8)
    values = values.astype(np.uint64)
    maxw = int(widths.max()) if widths.size else 0
    for b in range(maxw):
        sel = widths > b
        shift = (widths[sel] - 1 - b).astype(np.uint64)
        bits[offsets[sel] + b] = ((values[sel] >> shift) & np.uint64(1)).astype(np.uint8)
    return bits


def _huffman_tables():
    code = np.zeros((5, 16), dtype=np.int64)
    length = np.zeros((5, 16), dtype=np.int64)
    for brc, t in enumerate(HUFFMAN):
        for m, (c, l) in enumerate(t):
            code[brc, m] = c
            length[brc, m] = l
    return code, length


_HCODE, _HLEN = _huffman_tables()


def quantise_blocks(chan: np.ndarray, brc: np.ndarray, thidx: np.ndarray, nq: int, lines_per_pass: int = 16):
    """chan: (L, 4, NQ) real samples; brc/thidx: (L, nb).  Returns sign, mcode (L,4,NQ).
    Lines are quantised in passes of `lines_per_pass` (each line on its own,
    so the result does not depend on it; small passes keep the temporaries
    in cache)."""
    L = chan.shape[0]
    if L > lines_per_pass:
        sign = np.empty(chan.shape, dtype=np.uint8)
        mcode = np.empty(chan.shape, dtype=np.int64)
        for a in range(0, L, lines_per_pass):
            b = min(L, a + lines_per_pass)
            sign[a:b], mcode[a:b] = quantise_blocks(chan[a:b], brc[a:b], thidx[a:b], nq, lines_per_pass)
        return sign, mcode
    nb = brc.shape[1]
    blk = np.minimum(np.arange(nq) // 128, nb - 1)
    b_q = brc[:, blk][:, None, :]          # (L,1,NQ)
    t_q = thidx[:, blk][:, None, :]
    mag = np.abs(chan)
    sign = (chan < 0).astype(np.uint8)
    simple = t_q <= np.array(BRC_TO_THIDX)[b_q]
    flag = np.array(BRC_TO_M_CODE)[b_q]
    # simple branch: candidates 0..flag-1 (integers) and SIMPLE_RECONSTRUCTION at flag
    sr = SIMPLE_RECONSTRUCTION[b_q, np.minimum(t_q, 16)]
    m_simple = np.minimum(np.rint(mag), flag - 1)
    use_flag = np.abs(sr - mag) < np.abs(m_simple - mag)
    m_simple = np.where(use_flag, flag, m_simple)
    # normalized branch: nearest NRL*SF over m in [0, flag] (the first m of
    # the smallest error), evaluated per BRC on the samples that take it
    sf = np.broadcast_to(THIDX_TO_SF[t_q], chan.shape)
    bq = np.broadcast_to(b_q, chan.shape)
    best = np.zeros(chan.shape, dtype=np.int64)
    for b in range(5):
        sel = (bq == b) & ~simple
        if not sel.any():
            continue
        mg = mag[sel]
        sfs = sf[sel]
        bb = np.zeros(mg.shape, dtype=np.int64)
        be = np.full(mg.shape, np.inf)
        for m in range(BRC_TO_M_CODE[b] + 1):
            err = np.abs(NORMALIZED_RECONSTRUCTION[b, m] * sfs - mg)
            better = err < be
            bb = np.where(better, m, bb)
            be = np.where(better, err, be)
        best[sel] = bb
    mcode = np.where(simple, m_simple, best).astype(np.int64)
    sign = np.where(mcode == 0, sign & (chan < 0), sign).astype(np.uint8)
    return sign, mcode


def encode_user_data(lines: np.ndarray, rng: np.random.Generator, brc_mode: str = "uniform"):
    """FDBAQ-encode complex lines (L, N_r).  Returns (list of bytes, brc, thidx)."""
    L, n_r = lines.shape
    nq = n_r // 2
    nb = (2 * nq + 255) // 256   # packet.h:156 ceil(2 NQ / 256)
    chan = np.empty((L, 4, nq))
    chan[:, 0] = lines[:, 0::2].real   # IE
    chan[:, 1] = lines[:, 1::2].real   # IO
    chan[:, 2] = lines[:, 0::2].imag   # QE
    chan[:, 3] = lines[:, 1::2].imag   # QO
    brc = rng.integers(0, 5, size=(L, nb))
    # THIDX from block RMS: sigma factor nearest the RMS of the block's 4 channels
    blk = np.minimum(np.arange(nq) // 128, nb - 1)
    sq = np.zeros((L, nb))
    cnt = np.zeros(nb)
    np.add.at(sq.T, blk, (chan ** 2).sum(axis=1).T)
    np.add.at(cnt, blk, 4)
    rms = np.sqrt(sq / cnt)
    thidx = np.abs(THIDX_TO_SF[None, None, :] - rms[:, :, None]).argmin(axis=2)
    sign, mcode = quantise_blocks(chan, brc, thidx, nq)
    # per-sample bit lengths / code values
    b_q = brc[:, blk][:, None, :]
    clen = 1 + _HLEN[b_q, mcode]                         # (L,4,NQ)
    cval = (sign.astype(np.int64) << _HLEN[b_q, mcode]) | _HCODE[b_q, mcode]
    # block headers: IE gets 3-bit BRC, QE gets 8-bit THIDX before each block
    hdr_w = np.array([3, 0, 8, 0])
    # bit length of each channel: sum over blocks (hdr + codes)
    chan_bits = clen.sum(axis=2) + nb * hdr_w[None, :]
    chan_bits_padded = (chan_bits + 15) // 16 * 16
    pkt_bits = chan_bits_padded.sum(axis=1)             # (L,)
    pkt_start = np.concatenate([[0], np.cumsum(pkt_bits)[:-1]])
    chan_start = pkt_start[:, None] + np.concatenate(
        [np.zeros((L, 1), dtype=np.int64), np.cumsum(chan_bits_padded, axis=1)[:, :-1]], axis=1)
    # field stream per channel: for block b: [hdr], code_0..code_{n_b-1}
    # offset of sample q inside its channel = hdr_w*(blk(q)+1) + sum of clen of previous samples
    csum = np.cumsum(clen, axis=2) - clen
    samp_off = chan_start[:, :, None] + csum + hdr_w[None, :, None] * (blk[None, None, :] + 1)
    # header offsets: block b header sits after all samples of blocks < b
    first_q = np.arange(nb) * 128
    hdr_off = chan_start[:, :, None] + csum[:, :, first_q] + hdr_w[None, :, None] * np.arange(nb)[None, None, :]
    vals = [cval.ravel()]
    widths = [clen.ravel()]
    offs = [samp_off.ravel()]
    vals += [brc.ravel(), thidx.ravel()]
    widths += [np.full(L * nb, 3), np.full(L * nb, 8)]
    offs += [hdr_off[:, 0, :].ravel(), hdr_off[:, 2, :].ravel()]
    total = int(pkt_bits.sum())
    bits = _pack_fields(np.concatenate(vals), np.concatenate(widths), np.concatenate(offs), total)
    by = np.packbits(bits)
    starts = pkt_start // 8
    ends = (pkt_start + pkt_bits) // 8
    return [by[s:e].tobytes() for s, e in zip(starts, ends)], brc, thidx


# BAQ (data format C) tables: the "BAQ" rows of the reconstruction tables
# and the per-mode limits (structs.h:292-333, BAQ modes 3, 4, 5)
BAQ_MODE_TO_THIDX = {3: 3, 4: 7, 5: 15}
BAQ_MODE_TO_M_CODE = {3: 3, 4: 5, 5: 10}
BAQ_SIMPLE_RECONSTRUCTION = np.array([
    [3.00, 3.00, 3.12, 3.55] + [0.0] * 13,
    [7.00, 7.00, 7.00, 7.17, 7.40, 7.76] + [0.0] * 11,
    [15.00, 15.00, 15.00, 15.00, 15.00, 15.00, 15.44, 15.56, 16.11, 16.38, 16.65] + [0.0] * 6,
])
BAQ_NORMALIZED_RECONSTRUCTION = np.array([
    [0.2490, 0.7680, 1.3655, 2.1864] + [0.0] * 12,
    [0.1290, 0.3900, 0.6601, 0.9471, 1.2623, 1.6261, 2.0793, 2.7467] + [0.0] * 8,
    [0.0660, 0.1985, 0.3320, 0.4677, 0.6061, 0.7487, 0.8964, 1.0510, 1.2143, 1.3896, 1.5800, 1.7914,
     2.0329, 2.3234, 2.6971, 3.2692],
])


def _split_channels(lines: np.ndarray) -> np.ndarray:
    nq = lines.shape[1] // 2
    chan = np.empty((lines.shape[0], 4, nq))
    chan[:, 0] = lines[:, 0::2].real   # IE
    chan[:, 1] = lines[:, 1::2].real   # IO
    chan[:, 2] = lines[:, 0::2].imag   # QE
    chan[:, 3] = lines[:, 1::2].imag   # QO
    return chan


def _join_channels(v: np.ndarray) -> np.ndarray:
    L, _, nq = v.shape
    out = np.empty((L, 2 * nq), np.complex128)
    out[:, 0::2] = v[:, 0] + 1j * v[:, 2]
    out[:, 1::2] = v[:, 1] + 1j * v[:, 3]
    return out


def encode_fixed_user_data(lines: np.ndarray, baq_mode: int):
    """Encode complex lines (L, N_r) in a fixed-length format and return
    (list of user-data bytes, the decoded lines each sample's own fields give).

    baq_mode 0 (bypass, data formats A/B): every sample is a sign bit and a
    9-bit magnitude; each channel IE, IO, QE, QO holds N_q samples and is
    padded to a 16-bit word (packet.cpp:485-538).
    baq_mode 3/4/5 (BAQ, data format C): blocks of 128 quads, every sample a
    sign bit and a (baq_mode - 1)-bit code, an 8-bit THIDX before each QE
    block, 16-bit padding per channel; reconstruction of
    _get_s_values_type_c (packet.cpp:548-564) with the BAQ table rows."""
    L, n_r = lines.shape
    nq = n_r // 2
    chan = _split_channels(lines)
    mag = np.abs(chan)
    sign = (chan < 0).astype(np.int64)
    if baq_mode == 0:
        mcode = np.minimum(np.rint(mag), 511).astype(np.int64)
        sign = np.where(mcode == 0, 0, sign)
        value = np.where(sign == 1, -1.0, 1.0) * mcode
        code_w = 10
        nb, th_w, thidx = 0, 0, np.zeros((L, 0), np.int64)
    else:
        M = baq_mode
        lim, flag = BAQ_MODE_TO_THIDX[M], BAQ_MODE_TO_M_CODE[M]
        nb = (2 * nq + 255) // 256
        blk = np.minimum(np.arange(nq) // 128, nb - 1)
        sq = np.zeros((L, nb))
        cnt = np.zeros(nb)
        np.add.at(sq.T, blk, (chan ** 2).sum(axis=1).T)
        np.add.at(cnt, blk, 4)
        rms = np.sqrt(sq / cnt)
        thidx = np.abs(THIDX_TO_SF[None, None, :] - rms[:, :, None]).argmin(axis=2)
        t_q = thidx[:, blk][:, None, :]
        # simple branch (THIDX <= limit): integers below the flag, or the
        # flag code standing for SIMPLE_RECONSTRUCTION
        sr = BAQ_SIMPLE_RECONSTRUCTION[M - 3][np.minimum(t_q, 16)]
        m_s = np.minimum(np.rint(mag), flag - 1)
        m_s = np.where(np.abs(sr - mag) < np.abs(m_s - mag), flag, m_s).astype(np.int64)
        v_s = np.where(m_s == flag, sr, m_s)
        # normalized branch: nearest NRL * SF over every code
        lv = BAQ_NORMALIZED_RECONSTRUCTION[M - 3][: 1 << (M - 1)][None, None, None, :] * THIDX_TO_SF[t_q][..., None]
        m_n = np.abs(lv - mag[..., None]).argmin(axis=-1)
        v_n = np.take_along_axis(lv, m_n[..., None], axis=-1)[..., 0]
        simple = t_q <= lim
        mcode = np.where(simple, m_s, m_n)
        value = np.where(sign == 1, -1.0, 1.0) * np.where(simple, v_s, v_n)
        code_w = M
        th_w = 8
    # bit layout: per packet, channels in order, each padded to 16 bits
    ch_bits = np.array([nq * code_w + (nb * th_w if c == 2 else 0) for c in range(4)])
    ch_pad = (ch_bits + 15) // 16 * 16
    pkt_bits = int(ch_pad.sum())
    ch_start = np.concatenate([[0], np.cumsum(ch_pad)[:-1]])
    q = np.arange(nq)
    blkq = q // 128 if nb else np.zeros(nq, np.int64)
    samp_off = np.empty((4, nq), np.int64)
    for c in range(4):
        samp_off[c] = ch_start[c] + q * code_w + (th_w * (blkq + 1) if c == 2 else 0)
    vals = ((sign << (code_w - 1)) | mcode).reshape(L, -1)
    offs = (np.arange(L)[:, None] * pkt_bits + samp_off.ravel()[None, :])
    widths = np.full(vals.shape, code_w)
    if nb:
        th_off = ch_start[2] + np.arange(nb) * (th_w + 128 * code_w)
        vals = np.concatenate([vals, thidx], axis=1)
        offs = np.concatenate([offs, np.arange(L)[:, None] * pkt_bits + th_off[None, :]], axis=1)
        widths = np.concatenate([widths, np.full((L, nb), th_w)], axis=1)
    bits = _pack_fields(vals.ravel(), widths.ravel(), offs.ravel(), L * pkt_bits)
    by = np.packbits(bits)
    nbytes = pkt_bits // 8
    user = [by[i * nbytes:(i + 1) * nbytes].tobytes() for i in range(L)]
    return user, _join_channels(value)


def build_headers(fields: List[dict], user_lens: Sequence[int]) -> np.ndarray:
    """Pack primary+secondary headers for each packet. Returns (P, 68) uint8."""
    P = len(fields)
    prim_vals = np.zeros((P, 8), dtype=np.int64)
    prim_vals[:, 0] = 0      # version
    prim_vals[:, 1] = 0      # type
    prim_vals[:, 2] = 1      # secondary header flag
    prim_vals[:, 3] = 65     # process id
    prim_vals[:, 4] = 12     # category
    prim_vals[:, 5] = 3      # sequence flags
    prim_vals[:, 6] = [f.get("packet_sequence_count", i) & 0x3FFF for i, f in enumerate(fields)]
    prim_vals[:, 7] = [62 + n - 1 for n in user_lens]
    sec_vals = np.array([[f.get(name, 0) for name, _ in SECONDARY_FIELDS] for f in fields], dtype=np.int64)
    widths = np.array(PRIMARY_WIDTHS + [w for _, w in SECONDARY_FIELDS])
    offs_one = np.concatenate([[0], np.cumsum(widths)[:-1]])
    vals = np.concatenate([prim_vals, sec_vals], axis=1)
    offs = offs_one[None, :] + (np.arange(P) * 68 * 8)[:, None]
    bits = _pack_fields(vals.ravel(), np.tile(widths, P), offs.ravel(), P * 68 * 8)
    return np.packbits(bits).reshape(P, 68)


# ---------------------------------------------------------------- scene
def _f32_words(x: float) -> List[int]:
    u = int(np.array([x], dtype=">f4").view(">u4")[0])
    return [(u >> 16) & 0xFFFF, u & 0xFFFF]


def _f64_words(x: float) -> List[int]:
    u = int(np.array([x], dtype=">f8").view(">u8")[0])
    return [(u >> 48) & 0xFFFF, (u >> 32) & 0xFFFF, (u >> 16) & 0xFFFF, u & 0xFFFF]


def _orbit(velocity: float):
    p0 = np.array([6.0e6, 1.0e6, 3.6e6])
    d = np.cross(p0, np.array([0.3, -0.2, 1.0]))
    d = d / np.linalg.norm(d)
    return p0, velocity * d


def attitude_at(cycle: int):
    """A slowly varying platform attitude for sub-commutation cycle `cycle`:
    the scalar-first unit quaternion (w, x, y, z) of the roll/pitch/yaw
    rotation R_z(yaw) R_y(pitch) R_x(roll), and body angular rates (rad/s)."""
    roll = 0.012 + 0.004 * math.sin(0.7 * cycle)
    pitch = -0.031 + 0.003 * math.cos(0.4 * cycle)
    yaw = 0.047 + 0.0005 * cycle
    cr, sr = math.cos(roll / 2), math.sin(roll / 2)
    cp, sp = math.cos(pitch / 2), math.sin(pitch / 2)
    cy, sy = math.cos(yaw / 2), math.sin(yaw / 2)
    q = [cr * cp * cy + sr * sp * sy, sr * cp * cy - cr * sp * sy,
         cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy]
    omega = [1.1e-3 * math.cos(0.3 * cycle), -2.3e-4, 6.0e-5 * (1 + cycle % 3)]
    return q, omega


def subcomm_words(t_sv: float, p: np.ndarray, v: np.ndarray, q=None, omega=None) -> List[int]:
    """The 64 sub-commutated data words of one cycle (index 1..64).  The
    quaternion defaults to (1, 0, 0, 0) and the angular rates to zero words."""
    w = [0] * 65
    for axis in range(3):
        ws = _f64_words(float(p[axis]))
        for k in range(4):
            w[1 + 4 * axis + k] = ws[k]
    for axis in range(3):
        ws = _f32_words(float(v[axis]))
        w[13 + 2 * axis] = ws[0]
        w[14 + 2 * axis] = ws[1]
    # quaternion q0..q3 as float32 words at indices 23..30
    q = [1.0, 0.0, 0.0, 0.0] if q is None else q
    for k in range(4):
        ws = _f32_words(q[k])
        w[23 + 2 * k] = ws[0]
        w[24 + 2 * k] = ws[1]
    # angular rates omega_x, omega_y, omega_z as float32 words at 31..36
    if omega is not None:
        for k in range(3):
            ws = _f32_words(omega[k])
            w[31 + 2 * k] = ws[0]
            w[32 + 2 * k] = ws[1]
    coarse = int(math.floor(t_sv))
    fine = int(round((t_sv - coarse) * (1 << 24))) & 0xFFFFFF
    raw = (coarse << 24) | fine
    for k in range(4):
        w[37 + k] = (raw >> (48 - 16 * k)) & 0xFFFF
    return w[1:65]


def chirp_samples(dp: dict) -> np.ndarray:
    fs = dp["fs_mhz"]
    n = int(math.floor(fs * dp["txpl"]))
    t = np.arange(n) / fs  # us
    return np.exp(2j * np.pi * (dp["txpsf"] * t + 0.5 * dp["txprr"] * t * t))


def simulate_burst(spec: BurstSpec, rp: RadarParams, dp: dict, rng: np.random.Generator,
                   clutter_sigma: float, beam_addrs: np.ndarray) -> np.ndarray:
    """Complex echo lines (num_lines, 2*num_quads) in FP64."""
    L, n_r = spec.num_lines, 2 * spec.num_quads
    prf = 1.0 / dp["pri"]
    fs = dp["fs_mhz"] * 1e6
    echo = (rng.standard_normal((L, n_r)) + 1j * rng.standard_normal((L, n_r))) * (clutter_sigma / math.sqrt(2))
    eta = (np.arange(L) - L / 2) / prf
    # Doppler steering implied by the beam sweep (doppler.cpp:224-232 sign convention)
    psi = -0.018 + beam_addrs * (0.036 / 1023)
    k_psi = (psi[-1] - psi[0]) / (L / prf) if L > 1 else 0.0
    k_dc = -2 * rp.velocity_mps * k_psi / WAVELENGTH
    impulses = np.zeros((L, n_r), dtype=np.complex128)
    amp = clutter_sigma * 10 ** (spec.snr_db / 20)
    v_rel = rp.velocity_mps * 0.95
    chirp = chirp_samples(dp)
    n_ch = chirp.size
    for _ in range(spec.num_targets):
        r_bin = rng.uniform(0.05, 0.95) * n_r
        r0 = (dp["delay_near"] + r_bin / fs) * SPEED_OF_LIGHT / 2
        if spec.beam_sweep:
            eta_c = rng.uniform(-0.35, 0.35) * L / prf
            eta_k = eta_c + WAVELENGTH * r0 * k_dc * eta_c / (2 * v_rel ** 2) + spec.dc_offset_hz * WAVELENGTH * r0 / (2 * v_rel ** 2)
            width = 0.12 * L / prf
        else:
            eta_c = rng.uniform(-0.3, 0.3) * L / prf
            eta_k = eta_c
            width = 0.35 * L / prf
        rr = np.sqrt(r0 ** 2 + (v_rel * (eta - eta_k)) ** 2)
        w = np.exp(-0.5 * ((eta - eta_c) / width) ** 2)
        delay_bins = (2 * rr / SPEED_OF_LIGHT - dp["delay_near"]) * fs - n_ch // 2
        idx = np.rint(delay_bins).astype(np.int64)
        ok = (idx >= 0) & (idx < n_r) & (w > 1e-3)
        ph = np.exp(-4j * np.pi * rr / WAVELENGTH + 1j * rng.uniform(0, 2 * np.pi))
        impulses[np.nonzero(ok)[0], idx[ok]] += amp * w[ok] * ph[ok]
    # range chirp convolution (FFT, linear)
    nfft = 1 << int(math.ceil(math.log2(n_r + n_ch)))
    spec_c = np.fft.fft(chirp, nfft)
    conv = np.fft.ifft(np.fft.fft(impulses, nfft, axis=1) * spec_c[None, :], axis=1)[:, :n_r]
    echo += conv
    if spec.phase_error:
        x = np.linspace(-1.0, 1.0, L)
        echo *= np.exp(1j * (1.3 * np.pi * x ** 2 + 0.7 * np.pi * x ** 3))[:, None]
    if spec.rfi:
        hit = rng.random(L) < 0.3
        t = np.arange(n_r) / fs
        ntones = int(rng.integers(3, 9))
        for a in np.nonzero(hit)[0]:
            inr = 10 ** (rng.uniform(10, 30) / 20) * clutter_sigma
            sig = np.zeros(n_r, dtype=np.complex128)
            for _ in range(ntones):
                f0 = rng.uniform(-0.45, 0.45) * fs
                sig += np.exp(2j * np.pi * f0 * t + 1j * rng.uniform(0, 6.3))
            kr = rng.uniform(-2e12, 2e12)
            sig += np.exp(1j * np.pi * kr * (t - t.mean()) ** 2)
            echo[a] += inr / math.sqrt(ntones + 1) * sig
    return echo


def _beam_addresses(b: BurstSpec) -> np.ndarray:
    if b.beam_sweep:
        return np.rint(b.beam_start + np.arange(b.num_lines) * (b.beam_sweep / max(b.num_lines - 1, 1))).astype(int)
    return np.full(b.num_lines, b.beam_start, dtype=int)


def _burst_payload(args):
    """Simulate and FDBAQ-encode one burst (the expensive part), with its own
    seeded generator so bursts can be made in parallel processes."""
    spec, i, return_truth = args
    b = spec.bursts[i]
    rng = np.random.default_rng([spec.seed, i])
    hf = spec.radar.fields(b.num_quads)
    dp = decoded_params(hf, b.num_quads)
    lines = simulate_burst(b, spec.radar, dp, rng, spec.clutter_sigma, _beam_addresses(b))
    if b.baq_mode == 12:
        user, _, _ = encode_user_data(lines, rng)
        return user, (lines if return_truth else None)
    user, decoded = encode_fixed_user_data(lines, b.baq_mode)
    return user, (decoded if return_truth else None)


def generate(spec: StreamSpec, return_truth: bool = False, workers: int = 1):
    """Build a Level-0 byte stream for the bursts in `spec`.  Returns bytes
    (and, if asked, the per-burst FP64 echo lines before quantisation).
    workers > 1 simulates bursts in a process pool (spawned, so it is safe in
    a process that already uses CUDA); the output does not depend on it."""
    rp = spec.radar
    p0, v0 = _orbit(rp.velocity_mps)
    out_packets = []
    truth = []
    global_idx = 0
    pri_count = 100_000
    t = spec.start_time
    rx_channel = 0 if spec.polarisation[1] == "V" else 1
    pol_code = 4 if spec.polarisation[0] == "V" else 0
    jobs = [(spec, i, return_truth) for i in range(len(spec.bursts))]
    if workers > 1 and len(jobs) > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(workers, len(jobs))) as pool:
            payloads = pool.map(_burst_payload, jobs)
    else:
        payloads = [_burst_payload(j) for j in jobs]
    for bi, b in enumerate(spec.bursts):
        nq = b.num_quads
        hf = rp.fields(nq)
        dp = decoded_params(hf, nq)
        pri_s = dp["pri"]
        addrs = _beam_addresses(b)
        user, lines = payloads[bi]
        if return_truth:
            truth.append(lines)
        pri_count += b.gap_lines
        t += b.gap_lines * pri_s
        fields = []
        for a in range(b.num_lines):
            tt = t + a * pri_s
            coarse = int(math.floor(tt))
            fine = int((tt - coarse) * 65536) & 0xFFFF
            if fine == 0:
                fine = 1
            cyc = global_idx // 64
            t_cyc = spec.start_time + cyc * 64 * pri_s
            if spec.sv_cycle_step:
                t_sv = math.floor(spec.start_time) + cyc * spec.sv_cycle_step
            else:
                t_sv = math.floor(2 * t_cyc) / 2
            q, om = attitude_at(cyc) if spec.attitude else (None, None)
            words = subcomm_words(t_sv, p0 + v0 * (t_sv - spec.start_time), v0, q, om)
            f = dict(hf)
            f.update(coarse_time=coarse, fine_time=fine, sync_marker=SYNC_MARKER,
                     data_take_id=0x0D6D0C0, ecc_number=8 if b.swath.startswith("IW") else 1,
                     test_mode=b.test_mode, rx_channel_id=rx_channel, instrument_configuration_id=7,
                     sc_data_word_index=(global_idx % 64) + 1,
                     sc_data_word=words[global_idx % 64],
                     space_packet_count=global_idx, pri_count=pri_count + a, error_flag=0,
                     baq_mode=b.baq_mode, baq_block_length=31, rx_gain=8, ssb_flag=0,
                     polarisation=pol_code, temperature_compensation=3, elevation_beam_address=6,
                     azimuth_beam_address=int(addrs[a]), calibration_mode=0, tx_pulse_number=6,
                     signal_type=0, swap=1, swath_number=SWATH_NUMBERS[b.swath],
                     num_quadratures=nq, packet_sequence_count=global_idx)
            fields.append(f)
            global_idx += 1
        hdr = build_headers(fields, [len(u) for u in user])
        for a in range(b.num_lines):
            out_packets.append(hdr[a].tobytes())
            out_packets.append(user[a])
        pri_count += b.num_lines
        t += b.num_lines * pri_s
    data = b"".join(out_packets)
    return (data, truth) if return_truth else data


# -------------------------------------------------------- product sidecars
# A Level-0 product stores, beside each measurement .dat file, an annotation
# file (one 26-byte record per packet) and an index file (one 36-byte record
# per block of packets).  The field layouts are those the reference reads
# (aux_decoding.cpp:61-145); the values written here follow the meaning of
# the field names: packet_length = the packet's size in bytes, unit_offset /
# byte_offset = number / byte position of a block's first packet, data_size
# = the block's bytes, date_time / time_delta = IEEE doubles (block start
# time in days, block duration in seconds).
def packet_offsets(data: bytes) -> List[int]:
    """Start offset of every packet: a sequential walk over the primary
    headers (next = cur + 6 + packet_data_length + 1)."""
    offs, pos = [], 0
    while pos + 6 <= len(data):
        offs.append(pos)
        pos += 7 + ((data[pos + 4] << 8) | data[pos + 5])
    return offs


def _packet_time(data: bytes, off: int) -> float:
    coarse = int.from_bytes(data[off + 6:off + 10], "big")
    fine = int.from_bytes(data[off + 10:off + 12], "big")
    return coarse + fine / 65536.0


def annotation_sidecar(data: bytes, downlink_delay_s: float = 2.25) -> bytes:
    """One 26-byte annotation record per packet: sensing time (days,
    milliseconds, microseconds), downlink time, packet length, transfer
    frames, error flag and the bit fields, big-endian."""
    out = bytearray()
    offs = packet_offsets(data)
    ends = offs[1:] + [len(data)]
    for k, (o, e) in enumerate(zip(offs, ends)):
        rec = bytearray(26)
        for base, t in ((0, _packet_time(data, o)), (8, _packet_time(data, o) + downlink_delay_s)):
            days = int(t // 86400)
            ms = int((t - days * 86400) * 1000)
            us = int(round(((t - days * 86400) * 1000 - ms) * 1000)) % 1000
            rec[base:base + 2] = days.to_bytes(2, "big")
            rec[base + 2:base + 6] = ms.to_bytes(4, "big")
            rec[base + 6:base + 8] = us.to_bytes(2, "big")
        length = e - o
        rec[16:18] = (length & 0xFFFF).to_bytes(2, "big")
        rec[18:20] = (-(-length // 1908)).to_bytes(2, "big")
        rec[20] = 0
        # bit_1_type (1 bit) = 0, bit_2_type (2 bits) = k mod 4, bit_6_type (6 bits) = 2, spare 8 bits
        bits = ((k % 4) << 21) | (2 << 15)
        rec[21:24] = bits.to_bytes(3, "big")
        out += rec
    return bytes(out)


def index_sidecar(data: bytes, block_bytes: int = 64 * 1024) -> bytes:
    """One 36-byte index record per block of whole packets of about
    `block_bytes` bytes: date_time and time_delta (big-endian IEEE doubles),
    data_size, unit_offset, byte_offset, variable_flag, 3 spare bytes."""
    offs = packet_offsets(data)
    ends = offs[1:] + [len(data)]
    out = bytearray()
    k = 0
    while k < len(offs):
        j = k
        while j + 1 < len(offs) and ends[j] - offs[k] < block_bytes:
            j += 1
        t0, t1 = _packet_time(data, offs[k]), _packet_time(data, offs[j])
        rec = bytearray(36)
        rec[0:8] = np.array([t0 / 86400.0], dtype=">f8").tobytes()
        rec[8:16] = np.array([t1 - t0], dtype=">f8").tobytes()
        rec[16:20] = (ends[j] - offs[k]).to_bytes(4, "big")
        rec[20:24] = k.to_bytes(4, "big")
        rec[24:32] = offs[k].to_bytes(8, "big")
        rec[32] = 1
        out += rec
        k = j + 1
    return bytes(out)


# -------------------------------------------------------- named workloads
def config_spec(name: str, seed: int = 0, scale: float = 1.0) -> StreamSpec:
    """Named workloads: 'c1' stripmap 1024x2048, 'c2' IW burst 1500x12000,
    'c3' 9-burst IW swath (one polarisation stream), 'c4' C2 + RFI,
    'c5' C2 + azimuth phase error + Doppler-centroid offset.
    `scale` < 1 shrinks line and quad counts for quick tests (>= 1000 lines
    are kept for IW so bursts are not discarded)."""
    rng = np.random.default_rng(10_000 + seed)

    def nq(x):
        return max(64, int(round(x * scale)))

    if name == "c1":
        return StreamSpec([BurstSpec(num_lines=1024, num_quads=nq(1024), swath="S1", beam_start=512,
                                     beam_sweep=0, num_targets=5, snr_db=20.0)], seed=seed)
    if name in ("c2", "c4", "c5"):
        b = BurstSpec(num_lines=1500 if scale >= 1 else 1100, num_quads=nq(6000), swath="IW2",
                      num_targets=50, snr_db=15.0, rfi=(name == "c4"), phase_error=(name == "c5"),
                      dc_offset_hz=30.0 if name == "c5" else 0.0)
        return StreamSpec([b], seed=seed)
    if name == "c3":
        bursts = []
        for i in range(9):
            nl = int(rng.integers(1450, 1561)) if scale >= 1 else int(rng.integers(1050, 1150))
            nr = int(rng.integers(11800 // 2, 12500 // 2 + 1)) * 2
            bursts.append(BurstSpec(num_lines=nl, num_quads=nq(nr // 2), swath="IW2",
                                    num_targets=22, snr_db=15.0, gap_lines=250 + i))
        return StreamSpec(bursts, seed=seed)
    raise ValueError(name)
