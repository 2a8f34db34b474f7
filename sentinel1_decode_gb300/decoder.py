"""Python mirror of the reference's S1_Decoder (s1_decoder.h:13-77) over the
C ABI of include/s1g.h (libs1g.so, built in-tree by build.py).

Method names, argument meaning and error behaviour follow S1_Decoder:
products come back as 2-D numpy complex arrays (rows = azimuth lines), and
the reference's exceptions / exit(1) paths raise S1GError carrying the
library's status code.  There is no CPU fallback: if the CUDA library is
missing the constructor raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Union

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libs1g.so")

RAW, RANGE_COMPRESSED, RANGE_DOPPLER, AZIMUTH_COMPRESSED = 0, 1, 2, 3
CF32, CF64 = 0, 1
PREC_FP64, PREC_FP32, PREC_FP32_PLAIN = 0, 1, 2
# "fp32": fused FP32 kernels with double-float phases (default);
# "fp32_plain": FP32 per-stage kernels with FP64 phases; "fp64": FP64 throughout.
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "fp32_plain": PREC_FP32_PLAIN}
LEVELS = {"raw": RAW, "range_compressed": RANGE_COMPRESSED, "range_doppler": RANGE_DOPPLER,
          "azimuth_compressed": AZIMUTH_COMPRESSED}

# every entry point declared in include/s1g.h
EXPORTS = ["s1g_version", "s1g_open_file", "s1g_open_buffer", "s1g_close", "s1g_last_error", "s1g_set_precision",
           "s1g_apply_eccm", "s1g_num_packets", "s1g_swath_names", "s1g_num_bursts", "s1g_packet_field",
           "s1g_state_vectors", "s1g_burst_shape", "s1g_burst_product", "s1g_swath_shape", "s1g_swath_product",
           "s1g_burst_doppler", "s1g_process_swath_batch", "s1g_batch_output", "s1g_last_timing",
           "s1g_set_stage_timing", "s1g_launch_count", "s1g_decode_fdbaq_noalloc", "s1g_burst_unfold_shape",
           "s1g_set_batch_graph", "s1g_burst_image", "s1g_swath_image", "s1g_write_tiff",
           "s1g_spectrogram_shape", "s1g_spectrogram", "s1g_spectrogram_image", "s1g_attitudes",
           "s1g_packet_samples", "s1g_packet_offset", "s1g_ingest_stats", "s1g_read_index", "s1g_read_annotation",
           "s1g_annotation_times", "s1g_check_sidecars", "s1g_field_name", "s1g_packet_info",
           "s1g_set_abc_decode", "s1g_swath_row_widths", "s1g_azimuth_adjoint", "s1g_azimuth_focus",
           "s1g_tuning_report", "s1g_reload_buffer", "s1g_reload_file", "s1g_batch_host_outputs",
           "s1g_eccm_mask_shape", "s1g_eccm_mask", "s1g_burst_stage_flops", "s1g_set_batch_bursts",
           "s1g_set_rcmc", "s1g_sinc_interpolate", "s1g_transpose", "s1g_take_device_timeout",
           "s1g_tops_adjoint", "s1g_tops_focus"]



class IndexRecord(ctypes.Structure):
    """s1g_index_record: one 36-byte index record (index_decoder's fields)."""
    _fields_ = [("date_time", ctypes.c_uint64), ("time_delta", ctypes.c_uint64), ("data_size", ctypes.c_uint32),
                ("unit_offset", ctypes.c_uint32), ("byte_offset", ctypes.c_uint64),
                ("variable_flag", ctypes.c_uint32), ("spare_data", ctypes.c_uint32)]


class AnnotationRecord(ctypes.Structure):
    """s1g_annotation_record: one 26-byte annotation record (annotation_decoder's fields)."""
    _fields_ = [(n, ctypes.c_uint32) for n in (
        "days_ul", "milliseconds_ul", "microseconds_ul", "days_dl", "milliseconds_dl", "microseconds_dl",
        "packet_length", "num_transfer_frames", "error_flag", "bit_1_type", "bit_2_type", "bit_6_type",
        "spare_field")]


class SidecarReport(ctypes.Structure):
    """s1g_sidecar_report: the cross-check of the sidecars against the packets."""
    _fields_ = [(n, ctypes.c_int64) for n in (
        "packets", "index_records", "index_mismatches", "index_first_mismatch", "index_packets_covered",
        "annotation_records", "annotation_mismatches", "annotation_first_mismatch")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


# image scaling modes of the TIFF commands (s1_write --real/--imag/--mag/--norm/--norm_log)
SCALINGS = {"real": 0, "imag": 1, "mag": 2, "norm": 3, "norm_log": 4}


class S1GError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("s1g error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load_library(path: Optional[str] = None):
    """Load libs1g.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libs1g.so not built (%s); run sentinel1_decode_gb300.build.build()" % p)
    lib = ctypes.CDLL(p)
    vp, i64p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)
    lib.s1g_version.restype = ctypes.c_char_p
    lib.s1g_last_error.restype = ctypes.c_char_p
    lib.s1g_last_error.argtypes = [vp]
    lib.s1g_open_file.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)]
    lib.s1g_open_buffer.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(vp)]
    lib.s1g_close.argtypes = [vp]
    lib.s1g_reload_buffer.argtypes = [vp, ctypes.c_void_p, ctypes.c_size_t]
    lib.s1g_reload_file.argtypes = [vp, ctypes.c_char_p]
    lib.s1g_set_precision.argtypes = [vp, ctypes.c_int]
    lib.s1g_apply_eccm.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.s1g_set_abc_decode.argtypes = [vp, ctypes.c_int]
    lib.s1g_azimuth_adjoint.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp, vp,
                                        vp]
    lib.s1g_azimuth_focus.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp,
                                      ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    lib.s1g_tops_adjoint.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp, vp, vp]
    lib.s1g_tops_focus.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp,
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    lib.s1g_num_packets.argtypes = [vp, i64p]
    lib.s1g_swath_names.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.s1g_num_bursts.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
    lib.s1g_packet_field.argtypes = [vp, ctypes.c_int64, ctypes.c_char_p, i64p]
    lib.s1g_state_vectors.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.s1g_burst_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, i64p, i64p]
    lib.s1g_burst_unfold_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, i64p, i64p]
    lib.s1g_set_batch_graph.argtypes = [vp, ctypes.c_int]
    lib.s1g_batch_host_outputs.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    lib.s1g_burst_image.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int]
    lib.s1g_swath_image.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_int]
    lib.s1g_write_tiff.argtypes = [ctypes.c_char_p, vp, ctypes.c_int64, ctypes.c_int64]
    lib.s1g_spectrogram_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, i64p, i64p]
    lib.s1g_spectrogram.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                    ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    lib.s1g_spectrogram_image.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
    lib.s1g_burst_product.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int64,
                                      ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    lib.s1g_swath_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, i64p, i64p]
    lib.s1g_swath_row_widths.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int64, i64p]
    lib.s1g_swath_product.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int, ctypes.c_int]
    lib.s1g_burst_doppler.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double), ctypes.c_int64]
    lib.s1g_set_rcmc.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.s1g_transpose.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, vp, ctypes.c_int64,
                                  ctypes.c_int, vp]
    lib.s1g_take_device_timeout.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib.s1g_sinc_interpolate.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, vp, ctypes.c_int64,
                                         ctypes.c_int64, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int, vp]
    lib.s1g_set_batch_bursts.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.s1g_burst_stage_flops.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    lib.s1g_eccm_mask_shape.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, i64p, i64p]
    lib.s1g_eccm_mask.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
    lib.s1g_process_swath_batch.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_char_p, ctypes.c_int, i64p]
    lib.s1g_batch_output.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), i64p, i64p, i64p,
                                     ctypes.POINTER(ctypes.c_int)]
    lib.s1g_last_timing.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_char_p, ctypes.c_size_t]
    lib.s1g_set_stage_timing.argtypes = [vp, ctypes.c_int]
    lib.s1g_launch_count.argtypes = [i64p]
    lib.s1g_tuning_report.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.s1g_decode_fdbaq_noalloc.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int, vp,
                                             ctypes.c_int64, vp, vp]
    dp = ctypes.POINTER(ctypes.c_double)
    lib.s1g_attitudes.argtypes = [vp, dp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.s1g_packet_samples.argtypes = [vp, ctypes.c_int64, vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
    lib.s1g_packet_offset.argtypes = [vp, ctypes.c_int64, i64p]
    lib.s1g_field_name.argtypes = [ctypes.c_int]
    lib.s1g_field_name.restype = ctypes.c_char_p
    lib.s1g_packet_info.argtypes = [vp, ctypes.c_int64, ctypes.c_char_p, ctypes.c_size_t,
                                    ctypes.POINTER(ctypes.c_size_t)]
    lib.s1g_ingest_stats.argtypes = [vp, dp, i64p]
    lib.s1g_read_index.argtypes = [ctypes.c_char_p, vp, ctypes.c_int64, i64p, ctypes.c_int]
    lib.s1g_read_annotation.argtypes = [ctypes.c_char_p, vp, ctypes.c_int64, i64p, ctypes.c_int]
    lib.s1g_annotation_times.argtypes = [ctypes.c_char_p, vp, ctypes.c_int64, i64p, ctypes.c_int]
    lib.s1g_check_sidecars.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(SidecarReport)]
    if path is None:
        _lib = lib
    return lib


def launch_count() -> int:
    n = ctypes.c_int64()
    load_library().s1g_launch_count(ctypes.byref(n))
    return n.value


def tuning_report() -> str:
    """The FFT autotuner's choices so far in this process (s1g_tuning_report)."""
    buf = ctypes.create_string_buffer(1 << 16)
    load_library().s1g_tuning_report(buf, len(buf))
    return buf.value.decode()


def process_swath_batch(decoders, swath: str, level: int = AZIMUTH_COMPRESSED):
    """Process every burst of `swath` in each decoder (s1g_process_swath_batch).
    Returns (samples, device_ms)."""
    lib = load_library()
    arr = (ctypes.c_void_p * len(decoders))(*[d.handle for d in decoders])
    n = ctypes.c_int64()
    rc = lib.s1g_process_swath_batch(arr, len(decoders), swath.encode(), level, ctypes.byref(n))
    if rc != 0:
        raise S1GError(rc, lib.s1g_last_error(decoders[0].handle).decode(errors="replace"))
    return n.value, decoders[0].last_ms()


def batch_host_outputs(decoder, pointers):
    """Register page-locked host destinations (addresses, one per output burst
    of the batch, None to skip) for the following batch calls on `decoder`
    (s1g_batch_host_outputs); an empty list turns the copies off."""
    arr = (ctypes.c_void_p * max(len(pointers), 1))(*[p or None for p in pointers])
    rc = load_library().s1g_batch_host_outputs(decoder.handle, arr, len(pointers))
    if rc != 0:
        raise S1GError(rc, "batch_host_outputs failed")


def batch_outputs(decoder):
    """Device pointers of the last batch's products: list of
    (ptr, rows, cols, pitch_elems, elem_type)."""
    lib = load_library()
    out = []
    i = 0
    while True:
        p = ctypes.c_void_p()
        r, c, pt = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        t = ctypes.c_int()
        if lib.s1g_batch_output(decoder.handle, i, ctypes.byref(p), ctypes.byref(r), ctypes.byref(c),
                                ctypes.byref(pt), ctypes.byref(t)) != 0:
            break
        out.append((p.value, r.value, c.value, pt.value, t.value))
        i += 1
    return out


class S1Decoder:
    """S1_Decoder(filename) -- s1_decoder.h:50-55.  `source` is a path or the
    stream's bytes."""

    def __init__(self, source: Union[str, bytes, bytearray, memoryview], device: int = 0,
                 precision: str = "fp32"):
        self._lib = load_library()
        h = ctypes.c_void_p()
        if isinstance(source, str):
            rc = self._lib.s1g_open_file(source.encode(), device, ctypes.byref(h))
        else:
            b = bytes(source)
            rc = self._lib.s1g_open_buffer(b, len(b), device, ctypes.byref(h))
        if rc != 0:
            raise S1GError(rc, "open failed")
        self._h = h
        self.set_precision(precision)

    @classmethod
    def from_pointer(cls, ptr: int, nbytes: int, device: int = 0, precision: str = "fp32"):
        """Open from a host pointer (e.g. pinned memory) without a Python copy."""
        self = cls.__new__(cls)
        self._lib = load_library()
        h = ctypes.c_void_p()
        rc = self._lib.s1g_open_buffer(ctypes.cast(ctypes.c_void_p(ptr), ctypes.c_char_p), nbytes, device,
                                       ctypes.byref(h))
        if rc != 0:
            raise S1GError(rc, "open failed")
        self._h = h
        self.set_precision(precision)
        return self

    # -- lifetime
    def reload(self, source: Union[str, bytes, bytearray, memoryview]):
        """Replace the byte stream (s1g_reload_buffer / s1g_reload_file),
        keeping plans when the new stream has the same packet layout."""
        if isinstance(source, str):
            self._check(self._lib.s1g_reload_file(self._h, source.encode()))
        else:
            b = bytes(source)
            self._check(self._lib.s1g_reload_buffer(self._h, b, len(b)))

    def reload_from_pointer(self, ptr: int, nbytes: int):
        """Replace the byte stream from host or device memory at `ptr`."""
        self._check(self._lib.s1g_reload_buffer(self._h, ctypes.c_void_p(ptr), nbytes))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.s1g_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise S1GError(rc, self._lib.s1g_last_error(self._h).decode(errors="replace"))

    # -- configuration
    def set_precision(self, precision: str):
        if precision not in PRECISIONS:
            raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
        self._check(self._lib.s1g_set_precision(self._h, PRECISIONS[precision]))
        self.precision = precision

    def set_abc_decode(self, mode: str):
        """Data formats A/B/C: "reference" (default; the reference's samples,
        see s1g_set_abc_decode) or "fields" (each sample from its own bits)."""
        modes = {"reference": 0, "fields": 1}
        if mode not in modes:
            raise ValueError("mode must be 'reference' or 'fields'")
        self._check(self._lib.s1g_set_abc_decode(self._h, modes[mode]))

    def apply_eccm(self, detection_threshold: int, mitigation_threshold: int):
        """S1_Decoder::apply_eccm (s1_decoder.h:65)."""
        self._check(self._lib.s1g_apply_eccm(self._h, int(detection_threshold), int(mitigation_threshold)))

    # -- bookkeeping
    def num_packets(self) -> int:
        n = ctypes.c_int64()
        self._check(self._lib.s1g_num_packets(self._h, ctypes.byref(n)))
        return n.value

    def swath_counts(self) -> dict:
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._lib.s1g_swath_names(self._h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt = line.split()
            out[name] = int(cnt)
        return out

    def num_bursts(self, swath: str) -> int:
        n = ctypes.c_int()
        self._check(self._lib.s1g_num_bursts(self._h, swath.encode(), ctypes.byref(n)))
        return n.value

    def packet_field(self, packet: int, name: str) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.s1g_packet_field(self._h, packet, name.encode(), ctypes.byref(v)))
        return v.value

    def get_state_vectors(self) -> np.ndarray:
        """(n, 7) array of time, x, y, z, vx, vy, vz (STATE_VECTORS)."""
        cnt = ctypes.c_int()
        self._check(self._lib.s1g_state_vectors(self._h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 7))
        self._check(self._lib.s1g_state_vectors(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                cnt.value, ctypes.byref(cnt)))
        return out

    def get_attitudes(self) -> dict:
        """The attitude members of STATE_VECTORS (state_vectors.h:55-120),
        one row per state vector: quaternions (n, 4) scalar last,
        angular_rates (n, 3), attitudes (n, 3) = (-pitch, -roll, yaw)."""
        cnt = ctypes.c_int()
        self._check(self._lib.s1g_attitudes(self._h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 10))
        self._check(self._lib.s1g_attitudes(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            cnt.value, ctypes.byref(cnt)))
        return {"quaternions": out[:, 0:4], "angular_rates": out[:, 4:7], "attitudes": out[:, 7:10]}

    def azimuth_adjoint(self, swath: str, burst: int, theta, doppler_centroid: float = 0.0, grads: bool = True):
        """Image entropy of the differentiable azimuth chain (s1g_azimuth_adjoint)
        for the phase-error polynomial `theta` (coefficients of x^2, x^3, ...)
        and Doppler centroid; returns (loss, dloss/dtheta, dloss/dcentroid)."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).ravel())
        loss = ctypes.c_double()
        g = np.zeros(th.size)
        gf = ctypes.c_double()
        self._check(self._lib.s1g_azimuth_adjoint(
            self._h, swath.encode(), burst, th.ctypes.data if th.size else None, th.size, float(doppler_centroid),
            ctypes.byref(loss), g.ctypes.data if grads and th.size else None, ctypes.byref(gf) if grads else None))
        return loss.value, g, gf.value

    def azimuth_focus(self, swath: str, burst: int, theta, doppler_centroid: float = 0.0, dtype=np.complex64):
        """Focused image of the differentiable azimuth chain (s1g_azimuth_focus)."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).ravel())
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_burst_shape(self._h, swath.encode(), burst, RAW, ctypes.byref(r), ctypes.byref(c)))
        out = np.empty((r.value, c.value), dtype=dtype)
        self._check(self._lib.s1g_azimuth_focus(
            self._h, swath.encode(), burst, th.ctypes.data if th.size else None, th.size, float(doppler_centroid),
            out.ctypes.data, r.value, c.value, CF32 if out.dtype == np.complex64 else CF64, 0))
        return out

    def tops_adjoint(self, swath: str, burst: int, theta, centroid_offset: float = 0.0, grads: bool = True):
        """Image entropy of the differentiable TOPS chain (s1g_tops_adjoint) for
        the phase-error polynomial `theta` and an offset added to the burst's
        estimated Doppler centroid; returns (loss, dloss/dtheta, dloss/doffset)."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).ravel())
        loss = ctypes.c_double()
        g = np.zeros(th.size)
        gf = ctypes.c_double()
        self._check(self._lib.s1g_tops_adjoint(
            self._h, swath.encode(), burst, th.ctypes.data if th.size else None, th.size, float(centroid_offset),
            ctypes.byref(loss), g.ctypes.data if grads and th.size else None, ctypes.byref(gf) if grads else None))
        return loss.value, g, gf.value

    def tops_focus(self, swath: str, burst: int, theta, centroid_offset: float = 0.0, dtype=np.complex64):
        """Focused image of the differentiable TOPS chain (s1g_tops_focus):
        S unfolded azimuth rows x range samples."""
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).ravel())
        S, _ = self.unfold_shape(swath, burst)
        _, c = self.burst_shape(swath, burst)
        out = np.empty((S, c), dtype=dtype)
        self._check(self._lib.s1g_tops_focus(
            self._h, swath.encode(), burst, th.ctypes.data if th.size else None, th.size, float(centroid_offset),
            out.ctypes.data, S, c, CF32 if out.dtype == np.complex64 else CF64, 0))
        return out

    def packet_info(self, packet: int) -> str:
        """The s1_print packet_info text of one packet."""
        need = ctypes.c_size_t()
        self._check(self._lib.s1g_packet_info(self._h, packet, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self._check(self._lib.s1g_packet_info(self._h, packet, buf, need.value, ctypes.byref(need)))
        return buf.value.decode()

    def packet_offset(self, packet: int) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.s1g_packet_offset(self._h, packet, ctypes.byref(v)))
        return v.value

    def get_packet_samples(self, packet: int, dtype=np.complex128) -> np.ndarray:
        """Decoded samples of one packet (L0Packet::get_signal)."""
        n = 2 * self.packet_field(packet, "num_quadratures")
        out = np.zeros(n, dtype=dtype)
        self._check(self._lib.s1g_packet_samples(self._h, packet, out.ctypes.data_as(ctypes.c_void_p), n,
                                                 CF64 if out.dtype == np.complex128 else CF32, 0))
        return out

    def ingest_stats(self):
        """(ms, bytes) of the memory-mapped file ingest of the constructor."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        self._check(self._lib.s1g_ingest_stats(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def check_sidecars(self, index_path: Optional[str] = None, annotation_path: Optional[str] = None,
                       raise_on_mismatch: bool = True) -> dict:
        """Cross-check the product's index / annotation files against the
        packets the GPU indexer found (s1g_check_sidecars)."""
        rep = SidecarReport()
        rc = self._lib.s1g_check_sidecars(self._h, index_path.encode() if index_path else None,
                                          annotation_path.encode() if annotation_path else None, ctypes.byref(rep))
        if rc != 0 and (raise_on_mismatch or rc != -17):
            self._check(rc)
        out = rep.as_dict()
        out["ok"] = rc == 0
        return out

    # -- products
    def burst_shape(self, swath: str, burst: int, level: int = RAW):
        """(rows, cols) of a burst product (s1g_burst_shape)."""
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_burst_shape(self._h, swath.encode(), burst, level, ctypes.byref(r), ctypes.byref(c)))
        return r.value, c.value

    def _burst(self, swath: str, burst: int, level: int, dtype) -> np.ndarray:
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_burst_shape(self._h, swath.encode(), burst, level, ctypes.byref(r), ctypes.byref(c)))
        out = np.empty((r.value, c.value), dtype=dtype)
        t = CF32 if dtype == np.complex64 else CF64
        self._check(self._lib.s1g_burst_product(self._h, swath.encode(), burst, level, out.ctypes.data, r.value,
                                                c.value, t, 0))
        return out

    def _swath(self, swath: str, level: int, dtype) -> np.ndarray:
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_swath_shape(self._h, swath.encode(), level, ctypes.byref(r), ctypes.byref(c)))
        out = np.empty((r.value, c.value), dtype=dtype)
        t = CF32 if dtype == np.complex64 else CF64
        self._check(self._lib.s1g_swath_product(self._h, swath.encode(), level, out.ctypes.data, r.value, c.value,
                                                t, 0))
        return out

    def swath_row_widths(self, swath: str, level: int = RAW) -> np.ndarray:
        """Length of every row of a swath product as the reference's
        CF_VEC_2D has it (s1g_swath_row_widths); the arrays of the swath
        getters are as wide as the widest row, shorter rows zero-filled."""
        r = ctypes.c_int64()
        self._check(self._lib.s1g_swath_row_widths(self._h, swath.encode(), level, None, 0, ctypes.byref(r)))
        w = np.zeros(r.value, np.int64)
        self._check(self._lib.s1g_swath_row_widths(self._h, swath.encode(), level, w.ctypes.data, r.value,
                                                   ctypes.byref(r)))
        return w

    def get_burst(self, swath: str, burst: int, dtype=np.complex128):
        return self._burst(swath, burst, RAW, dtype)

    def get_swath(self, swath: str, dtype=np.complex128):
        return self._swath(swath, RAW, dtype)

    def get_range_compressed_burst(self, swath: str, burst: int, range_doppler: bool = False, dtype=np.complex128):
        return self._burst(swath, burst, RANGE_DOPPLER if range_doppler else RANGE_COMPRESSED, dtype)

    def get_range_compressed_swath(self, swath: str, range_doppler: bool = False, dtype=np.complex128):
        return self._swath(swath, RANGE_DOPPLER if range_doppler else RANGE_COMPRESSED, dtype)

    def get_azimuth_compressed_burst(self, swath: str, burst: int, dtype=np.complex128):
        return self._burst(swath, burst, AZIMUTH_COMPRESSED, dtype)

    def get_azimuth_compressed_swath(self, swath: str, dtype=np.complex128):
        return self._swath(swath, AZIMUTH_COMPRESSED, dtype)

    def get_burst_image(self, swath: str, burst: int, level: int = RAW, scaling: str = "real") -> np.ndarray:
        """Scaled float32 image of a burst product (the data of s1_write's
        TIFF commands), scaled on the GPU."""
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_burst_shape(self.handle, swath.encode(), burst, level, ctypes.byref(r), ctypes.byref(c)))
        out = np.empty((r.value, c.value), np.float32)
        self._check(self._lib.s1g_burst_image(self.handle, swath.encode(), burst, level, SCALINGS[scaling],
                                              out.ctypes.data_as(ctypes.c_void_p), r, c, 0))
        return out

    def get_spectrogram(self, swath: str, burst: int, azimuth_line: int, fft_size: int = 64, stride: int = 32,
                        scaling: str = None) -> np.ndarray:
        """spectrogram() of one echo line ([fft_size][windows], complex128),
        or its scaled float32 image when `scaling` is given."""
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_spectrogram_shape(self.handle, swath.encode(), burst, fft_size, stride,
                                                    ctypes.byref(r), ctypes.byref(c)))
        if scaling is None:
            out = np.empty((r.value, c.value), np.complex128)
            self._check(self._lib.s1g_spectrogram(self.handle, swath.encode(), burst, azimuth_line, fft_size, stride,
                                                  out.ctypes.data_as(ctypes.c_void_p), r, c, CF64, 0))
        else:
            out = np.empty((r.value, c.value), np.float32)
            self._check(self._lib.s1g_spectrogram_image(self.handle, swath.encode(), burst, azimuth_line, fft_size,
                                                        stride, SCALINGS[scaling],
                                                        out.ctypes.data_as(ctypes.c_void_p), r, c, 0))
        return out

    def get_swath_image(self, swath: str, level: int = RAW, scaling: str = "real") -> np.ndarray:
        r, c = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_swath_shape(self.handle, swath.encode(), level, ctypes.byref(r), ctypes.byref(c)))
        out = np.empty((r.value, c.value), np.float32)
        self._check(self._lib.s1g_swath_image(self.handle, swath.encode(), level, SCALINGS[scaling],
                                              out.ctypes.data_as(ctypes.c_void_p), r, c, 0))
        return out

    def set_rcmc(self, mode: str = "phase", half_width: int = 4):
        """Range cell migration correction of the TOPS chain (s1g_set_rcmc):
        "phase" (the reference's) or "sinc" (FP32 precision)."""
        self._check(self._lib.s1g_set_rcmc(self._h, {"phase": 0, "sinc": 1}[mode], int(half_width)))

    def set_batch_bursts(self, bursts=None):
        """Bursts this handle contributes to the following batch calls
        (s1g_set_batch_bursts); None = all."""
        if bursts is None:
            self._check(self._lib.s1g_set_batch_bursts(self._h, None, -1))
            return
        arr = (ctypes.c_int * max(len(bursts), 1))(*[int(b) for b in bursts])
        self._check(self._lib.s1g_set_batch_bursts(self._h, arr, len(bursts)))

    def set_batch_graph(self, on: bool):
        """CUDA-graph capture of process_swath_batch calls led by this handle."""
        self._check(self._lib.s1g_set_batch_graph(self.handle, 1 if on else 0))

    def unfold_shape(self, swath: str, burst: int):
        """(S, N_out): unfolded azimuth length of the TOPS chain (N_a for
        stripmap) and SLC rows of a burst (host-side)."""
        S, n = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_burst_unfold_shape(self.handle, swath.encode(), burst, ctypes.byref(S),
                                                     ctypes.byref(n)))
        return S.value, n.value

    def get_doppler(self, swath: str, burst: int):
        """(rate, per-range-bin centroid) of a burst (doppler.cpp:146-232)."""
        _, c = ctypes.c_int64(), ctypes.c_int64()
        r = ctypes.c_int64()
        self._check(self._lib.s1g_burst_shape(self._h, swath.encode(), burst, RAW, ctypes.byref(r), ctypes.byref(c)))
        dc = np.zeros(c.value)
        rate = ctypes.c_double()
        self._check(self._lib.s1g_burst_doppler(self._h, swath.encode(), burst, ctypes.byref(rate),
                                                dc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), c.value))
        return rate.value, dc

    def get_eccm_mask(self, swath: str, burst: int) -> np.ndarray:
        """The ECCM notch mask of a burst, [lines, windows, 128] bool: True
        where eccm() (signal_processing.cpp:914-1004) zeroes that bin of
        that short-time window.  Needs apply_eccm first."""
        r, w = ctypes.c_int64(), ctypes.c_int64()
        self._check(self._lib.s1g_eccm_mask_shape(self._h, swath.encode(), burst, ctypes.byref(r), ctypes.byref(w)))
        out = np.empty((r.value, w.value, 128), dtype=np.uint8)
        self._check(self._lib.s1g_eccm_mask(self._h, swath.encode(), burst, out.ctypes.data_as(ctypes.c_void_p),
                                            r.value, w.value, 0))
        return out.astype(bool)

    def stage_flops(self, swath: str, burst: int) -> dict:
        """{stage: nominal FP32 flops} of the fused FP32 path for one burst
        (s1g_burst_stage_flops)."""
        buf = ctypes.create_string_buffer(4096)
        self._check(self._lib.s1g_burst_stage_flops(self._h, swath.encode(), burst, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            k, v = line.split()
            out[k] = float(v)
        return out

    def set_stage_timing(self, on: bool):
        self._check(self._lib.s1g_set_stage_timing(self._h, 1 if on else 0))

    def stage_times(self) -> dict:
        """{stage: (total_ms, count)} accumulated while stage timing is on."""
        ms = ctypes.c_double()
        buf = ctypes.create_string_buffer(1 << 14)
        self._check(self._lib.s1g_last_timing(self._h, ctypes.byref(ms), buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, t, n = line.split()
            out[name] = (float(t), int(n))
        return out

    def last_ms(self) -> float:
        ms = ctypes.c_double()
        self._check(self._lib.s1g_last_timing(self._h, ctypes.byref(ms), None, 0))
        return ms.value

    @property
    def handle(self):
        return self._h


def write_tiff(path: str, image: np.ndarray) -> None:
    """BigTIFF float32 file of a 2-D image, rows written bottom-up like the
    reference's _write_tif (s1g_write_tiff; host only)."""
    img = np.ascontiguousarray(image, dtype=np.float32)
    lib = load_library()
    st = lib.s1g_write_tiff(path.encode(), img.ctypes.data_as(ctypes.c_void_p), img.shape[0], img.shape[1])
    if st != 0:
        raise S1GError(st, "write_tiff failed for %s" % path)


def sidecar_paths(dat_path: str):
    """The index and annotation files a Level-0 product keeps beside the
    measurement file `<name>.dat`: `<name>-index.dat`, `<name>-annot.dat`."""
    stem = dat_path[:-4] if dat_path.endswith(".dat") else dat_path
    return stem + "-index.dat", stem + "-annot.dat"


def _read_records(fn, rec_type, path: str, reference_tail: bool):
    lib = load_library()
    n = ctypes.c_int64()
    rc = fn(lib)(path.encode(), None, 0, ctypes.byref(n), int(reference_tail))
    if rc != 0:
        raise S1GError(rc, "Unable to open %s" % path)
    arr = (rec_type * max(n.value, 1))()
    rc = fn(lib)(path.encode(), ctypes.cast(arr, ctypes.c_void_p), n.value, ctypes.byref(n), int(reference_tail))
    if rc != 0:
        raise S1GError(rc, "Unable to read %s" % path)
    return [{k: getattr(arr[i], k) for k, _ in rec_type._fields_} for i in range(n.value)]


def read_index(path: str, reference_tail: bool = False):
    """Index records of a sidecar file as dicts (index_decoder,
    aux_decoding.cpp:61-83).  reference_tail adds the extra record the
    reference's read loop appends at the end of the file."""
    return _read_records(lambda lib: lib.s1g_read_index, IndexRecord, path, reference_tail)


def read_annotation(path: str, reference_tail: bool = False):
    """Annotation records as dicts (annotation_decoder, aux_decoding.cpp:93-118)."""
    return _read_records(lambda lib: lib.s1g_read_annotation, AnnotationRecord, path, reference_tail)


def annotation_times(path: str, reference_tail: bool = False) -> np.ndarray:
    """Sensing times of the annotation records (annotation_time_decoder,
    aux_decoding.cpp:121-145)."""
    lib = load_library()
    n = ctypes.c_int64()
    rc = lib.s1g_annotation_times(path.encode(), None, 0, ctypes.byref(n), int(reference_tail))
    if rc != 0:
        raise S1GError(rc, "Unable to open %s" % path)
    out = np.zeros(n.value)
    rc = lib.s1g_annotation_times(path.encode(), out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n),
                                  int(reference_tail))
    if rc != 0:
        raise S1GError(rc, "Unable to read %s" % path)
    return out
