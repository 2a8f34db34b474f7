/*
 * s1g: GB300-native Sentinel-1 Level-0 -> SLC hot path, C ABI.
 *
 * This is the drop-in boundary for the sentinel1_decode library's product
 * path.  The reference exposes that path only as the C++ class S1_Decoder
 * (s1_decoder.h:13-77); each entry point below replaces one of its members,
 * with plain pointers, sizes and integer status codes in place of C++
 * containers and exceptions:
 *
 *   s1g_open_file / s1g_open_buffer  <- S1_Decoder(const std::string&)      s1_decoder.h:50-55
 *   s1g_apply_eccm                   <- S1_Decoder::apply_eccm(int, int)     s1_decoder.h:65
 *   s1g_burst_product (S1G_RAW)      <- S1_Decoder::get_burst                s1_decoder.h:69
 *   s1g_burst_product (S1G_RANGE_COMPRESSED / S1G_RANGE_DOPPLER)
 *                                    <- S1_Decoder::get_range_compressed_burst s1_decoder.h:72
 *   s1g_burst_product (S1G_AZIMUTH_COMPRESSED)
 *                                    <- S1_Decoder::get_azimuth_compressed_burst s1_decoder.h:75
 *   s1g_swath_product                <- get_swath / get_range_compressed_swath /
 *                                       get_azimuth_compressed_swath        s1_decoder.h:70,73,76
 *   s1g_num_bursts, s1g_swath_names  <- the swath/burst bookkeeping of _set_packets and
 *                                       _validate_request                   s1_decoder.cpp:13-89
 *   s1g_state_vectors                <- S1_Decoder::get_state_vectors        s1_decoder.h:67
 *   s1g_attitudes                    <- STATE_VECTORS quaternions / angular_rates /
 *                                       attitudes                     state_vectors.h:55-120
 *   s1g_read_index / s1g_read_annotation / s1g_annotation_times
 *                                    <- index_decoder / annotation_decoder /
 *                                       annotation_time_decoder      aux_decoding.cpp:61-145
 *   s1g_packet_info                  <- s1_print packet_info               print_main.cpp:26-47
 *   s1g_packet_samples               <- L0Packet::get_signal (s1_print complex_samples)
 *                                                                    packet.cpp:404-453
 *
 * Products are written into caller-allocated buffers, row-major, complex
 * interleaved (re, im), as complex<float> (S1G_CF32, the layout that
 * s1_write's save_*_as_cf32 writes, image_write_main.cpp:238-245) or
 * complex<double> (S1G_CF64, the reference's in-memory type).  Buffers may be
 * host or device memory (out_on_device).  The shape of a product is queried
 * first with the *_shape calls.
 *
 * Errors: every call returns S1G_OK or a negative code; s1g_last_error()
 * gives the message.  A decoder handle is not thread-safe: use one handle per
 * host thread.  All GPU work of a handle runs on its own CUDA stream.
 */
#ifndef S1G_H
#define S1G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference's exceptions and exits) */
#define S1G_OK 0
#define S1G_E_INVALID_ARGUMENT (-1)   /* std::invalid_argument                          */
#define S1G_E_BAD_SWATH (-2)          /* _validate_request: swath not in data (exit 1) */
#define S1G_E_BAD_BURST (-3)          /* _validate_request: burst not in data (exit 1) */
#define S1G_E_IO (-4)                 /* open_file: "Unable to open"                    */
#define S1G_E_CUDA (-5)               /* CUDA runtime failure                           */
#define S1G_E_UNSUPPORTED (-6)        /* std::domain_error: swath mode not IW/SM         */
#define S1G_E_PACKET_LENGTH (-7)      /* packet length field inconsistent              */
#define S1G_E_READ_PAST_END (-8)      /* read_n_bits: bit read past the user data       */
#define S1G_E_BAD_BRC (-9)            /* "BRC value is invalid."                        */
#define S1G_E_HUFFMAN (-10)           /* "Max bit length exceeded in Huffman decoding." */
#define S1G_E_MCODE (-11)             /* "MCode is greater than the comparison flag."   */
#define S1G_E_RAGGED_BURST (-12)      /* packets of one burst differ in num_quadratures */
#define S1G_E_BAD_FORMAT (-13)        /* "BAQ Mode is invalid." (not 0, 3-5 or 12-14)    */
#define S1G_E_BUFFER (-14)            /* caller buffer shape does not match the product */
#define S1G_E_GEOMETRY (-15)          /* burst too short for azimuth processing          */
#define S1G_E_SCRATCH_LIMIT (-16)     /* request exceeds the fixed scratch of the allocation-free decode */
#define S1G_E_SIDECAR (-17)           /* index / annotation sidecar disagrees with the packet stream */
#define S1G_E_TIMEOUT (-18)           /* a bounded device wait ran out (TMA corner-turn tile load)       */

/* processing levels (s1_write save_*_as_cf32 processing_level strings) */
#define S1G_RAW 0
#define S1G_RANGE_COMPRESSED 1
#define S1G_RANGE_DOPPLER 2
#define S1G_AZIMUTH_COMPRESSED 3

/* output element types */
#define S1G_CF32 0
#define S1G_CF64 1

/* image scaling modes of the TIFF commands (s1_write --real/--imag/--mag/--norm/--norm_log) */
#define S1G_SCALE_REAL 0
#define S1G_SCALE_IMAG 1
#define S1G_SCALE_MAG 2
#define S1G_SCALE_NORM 3
#define S1G_SCALE_NORM_LOG 4

/* range cell migration correction of the TOPS row pass */
#define S1G_RCMC_PHASE 0  /* the reference's: exp(-4 pi i f_r (R/D - R) / c) on the range-time samples (default) */
#define S1G_RCMC_SINC 1   /* a shift of each range line by the migration 2 (R/D - R) f_s / c samples by
                             Hann-windowed sinc interpolation (2L + 1 taps), FP32 path only */

/* arithmetic precision of the GPU path */
#define S1G_PREC_FP64 0   /* plain FP64 everywhere (the reference's arithmetic)          */
#define S1G_PREC_FP32 1   /* fused FP32 kernels; double-float phases, FP64 fits (default)  */
#define S1G_PREC_FP32_PLAIN 2 /* FP32 per-stage kernels with FP64 phase arithmetic        */

typedef struct s1g_decoder s1g_decoder;

/* Version string of the library. */
const char* s1g_version(void);

/* Open a Level-0 .dat file / an in-memory byte stream.  The stream is copied
 * to the GPU, indexed there, and segmented into swaths and bursts exactly as
 * S1_Decoder's constructor does.  device: CUDA ordinal. */
int s1g_open_file(const char* path, int device, s1g_decoder** out);
int s1g_open_buffer(const uint8_t* bytes, size_t nbytes, int device, s1g_decoder** out);
int s1g_close(s1g_decoder* h);
/* Replace the handle's byte stream with a new one (host or device memory /
 * a file), as a fresh open would, but keep the handle's FFT plans and
 * device buffers.  Plans derived from the content -- per-burst tables,
 * batch decode jobs, the captured batch graph -- are kept when the new
 * stream's packet headers and layout are identical to the previous one's
 * (e.g. the next acquisition of a repeated geometry) and rebuilt otherwise. */
int s1g_reload_buffer(s1g_decoder* h, const uint8_t* bytes, size_t nbytes);
int s1g_reload_file(s1g_decoder* h, const char* path);
const char* s1g_last_error(const s1g_decoder* h);

int s1g_set_precision(s1g_decoder* h, int precision);

/* Decoding of the fixed-length data formats A/B (bypass, baq_mode 0) and C
 * (BAQ 3/4/5-bit).  S1G_ABC_REFERENCE (the default) gives the reference's
 * samples exactly: its decoders (packet.cpp:485-666) append the codes to
 * containers pre-filled with zero entries and then read the leading ones, so
 * in bypass packets quad q carries the codes of quad q - 128 (quads below 128
 * are zero), and in BAQ packets every sample of a 128-quad block is the
 * reconstruction of code 0 at the block's THIDX.  S1G_ABC_FIELDS decodes
 * every sample from its own sign and code bits with the same field layout
 * and reconstruction tables.  FDBAQ (format D) is not affected. */
#define S1G_ABC_REFERENCE 0
#define S1G_ABC_FIELDS 1
int s1g_set_abc_decode(s1g_decoder* h, int mode);
/* Range cell migration correction of the TOPS azimuth chain.  S1G_RCMC_PHASE
 * (default) is the reference's (apply_range_cell_migration_correction,
 * image_formation.cpp:458-476: a phase ramp applied to the range-time
 * samples, which moves no energy).  S1G_RCMC_SINC moves it: after the range
 * IFFT of the row pass every range-Doppler line is resampled at
 * j + 2 R_j (1 - D) / D f_s / c (the range at which a target of range bin j
 * appears at that azimuth frequency) with sinc_interpolate's Hann-windowed
 * sinc kernel of half-width half_width (signal_processing.cpp:228-257; 1..16,
 * 4 = 9 taps), then the scale and azimuth filter follow as before.  Products
 * then differ from the reference's by the migration; S1G_PREC_FP32 only
 * (other precisions return S1G_E_UNSUPPORTED for TOPS azimuth products).
 * No counterpart in the reference's product path (it defines
 * sinc_interpolate but does not call it). */
int s1g_set_rcmc(s1g_decoder* h, int mode, int half_width);
int s1g_apply_eccm(s1g_decoder* h, int detection_threshold, int mitigation_threshold);

/* Number of packets found in the stream, and the swath names present
 * (newline-separated "NAME count" lines, like s1_print swath_names). */
int s1g_num_packets(const s1g_decoder* h, int64_t* n);
int s1g_swath_names(const s1g_decoder* h, char* buf, size_t buflen);
int s1g_num_bursts(const s1g_decoder* h, const char* swath, int* n);

/* Per-packet header field by name (as parse_packet_header keys it, e.g.
 * "num_quadratures", "azimuth_beam_address"). */
int s1g_packet_field(const s1g_decoder* h, int64_t packet, const char* name, int64_t* value);

/* State vectors parsed from the sub-commutated ancillary words: up to cap
 * entries of (time, x, y, z, vx, vy, vz). */
int s1g_state_vectors(const s1g_decoder* h, double* out7, int cap, int* count);

/* The rest of each state vector, in the order of s1g_state_vectors: up to
 * cap entries of (qx, qy, qz, qw, omega_x, omega_y, omega_z, att0, att1,
 * att2) -- the quaternion scalar last and the attitude (-pitch, -roll, yaw)
 * exactly as STATE_VECTORS stores them (parse_quaternions and
 * to_euler_angles, state_vectors.cpp:203-320). */
int s1g_attitudes(const s1g_decoder* h, double* out10, int cap, int* count);

/* Name of header field i in parse order (the 8 primary then the 46
 * secondary fields of structs.h:42-166), NULL past the last. */
const char* s1g_field_name(int i);

/* The s1_print packet_info printout of one packet (primary and secondary
 * header fields, operating modes and pulse info, print_main.cpp:26-47 with
 * packet.cpp:204-261) as text.  *needed receives the size including the
 * terminating NUL; buf may be NULL to query it. */
int s1g_packet_info(s1g_decoder* h, int64_t packet, char* buf, size_t buflen, size_t* needed);

/* The decoded complex samples of one packet (2 * num_quadratures of them,
 * get_signal's order), decoded on the GPU; out_type S1G_CF32 or S1G_CF64. */
int s1g_packet_samples(s1g_decoder* h, int64_t packet, void* out, int64_t n, int out_type, int out_on_device);

/* Byte offset of a packet in the stream, as found by the GPU indexer. */
int s1g_packet_offset(const s1g_decoder* h, int64_t packet, int64_t* offset);

/* Host time (ms) and bytes of the last s1g_open_file ingest: the file is
 * memory-mapped and streamed to the device through pinned staging buffers. */
int s1g_ingest_stats(const s1g_decoder* h, double* ms, int64_t* bytes);

/* ---- product sidecars ----------------------------------------------------
 * A Level-0 product keeps beside each measurement file an index file (one
 * 36-byte record per block of packets) and an annotation file (one 26-byte
 * record per packet).  Field layouts and widths: index_decoder /
 * annotation_decoder, aux_decoding.cpp:61-118; the values are the raw
 * big-endian fields (date_time and time_delta are the 64 raw bits). */
typedef struct s1g_index_record {
    uint64_t date_time;
    uint64_t time_delta;
    uint32_t data_size;      /* bytes in the block */
    uint32_t unit_offset;    /* number of the block's first packet */
    uint64_t byte_offset;    /* byte position of the block's first packet */
    uint32_t variable_flag;
    uint32_t spare_data;
} s1g_index_record;

typedef struct s1g_annotation_record {
    uint32_t days_ul, milliseconds_ul, microseconds_ul;
    uint32_t days_dl, milliseconds_dl, microseconds_dl;
    uint32_t packet_length, num_transfer_frames, error_flag;
    uint32_t bit_1_type, bit_2_type, bit_6_type, spare_field;
} s1g_annotation_record;

/* Read every record of a sidecar file.  *count receives the number of
 * records; out may be NULL (or cap too small) to query it.  With
 * reference_tail = 1 the count also includes the extra record the
 * reference's read loop appends (aux_decoding.cpp:67,102: the bytes of a last
 * partial record, zero-padded, or an all-zero record when the file ends on a
 * record boundary); with 0 only the complete records are returned. */
int s1g_read_index(const char* path, s1g_index_record* out, int64_t cap, int64_t* count, int reference_tail);
int s1g_read_annotation(const char* path, s1g_annotation_record* out, int64_t cap, int64_t* count,
                        int reference_tail);
/* Sensing time of every annotation record in seconds, as
 * annotation_time_decoder computes it (aux_decoding.cpp:121-145):
 * days_ul * 86400 + milliseconds_ul * 1e-3 + 7300 * 86400.  The reference's
 * microseconds term reads a key that no record has, so it adds 0. */
int s1g_annotation_times(const char* path, double* out, int64_t cap, int64_t* count, int reference_tail);

/* Cross-check the sidecars of a product against the packets the GPU indexer
 * found in the opened stream.  Index records: unit_offset names an existing
 * packet, byte_offset equals that packet's offset, data_size equals the bytes
 * up to the next record's first packet (the end of the stream for the last).
 * Annotation records: one per packet, packet_length equal to the packet's
 * size in bytes.  Either path may be NULL to skip that file.  Returns S1G_OK
 * when everything agrees, S1G_E_SIDECAR (message in s1g_last_error) when
 * anything disagrees, S1G_E_IO when a file cannot be read. */
typedef struct s1g_sidecar_report {
    int64_t packets;               /* packets in the stream */
    int64_t index_records;         /* complete index records read */
    int64_t index_mismatches;      /* index records that disagree */
    int64_t index_first_mismatch;  /* first such record, -1 if none */
    int64_t index_packets_covered; /* packets inside the agreeing blocks */
    int64_t annotation_records;    /* complete annotation records read */
    int64_t annotation_mismatches; /* annotation records whose packet_length disagrees */
    int64_t annotation_first_mismatch;
} s1g_sidecar_report;
int s1g_check_sidecars(s1g_decoder* h, const char* index_path, const char* annotation_path, s1g_sidecar_report* rep);

/* ---- differentiable azimuth chain -----------------------------------------
 * No counterpart in the reference (it has no gradients or autofocus).  The
 * range-Doppler azimuth chain of one burst, recomputed from the byte stream
 * on each call (range compression included, nothing stored between calls):
 *   U = X exp(-i phi_a), phi_a = sum_j theta[j] x_a^(j+2), x_a = linspace(-1, 1, lines)
 *   V = FFT_az(U); bulk RCMC exp(i 4 pi f_r R_ref (1/D_k - 1)/c) in range frequency;
 *   azimuth filter exp(-i 4 pi R_r (1 - D_k)/lambda), D_k = sqrt(1 - lambda^2 f_k^2/(4 v^2)),
 *   f_k = (FFT bin frequency) + doppler_centroid;  Y = IFFT_az;
 *   loss = image entropy -sum p ln p, p = |Y|^2 / sum |Y|^2.
 * s1g_azimuth_adjoint returns the loss and (when the pointers are not NULL)
 * its gradient with respect to theta[0..ntheta) (ntheta <= 8) and to the
 * Doppler centroid, by a hand-written reverse-mode adjoint of the chain.
 * s1g_azimuth_focus writes the focused image Y (lines x range samples).  The
 * handle's precision selects FP64 or FP32 arithmetic (phases and gradient
 * sums stay FP64). */
int s1g_azimuth_adjoint(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                        double doppler_centroid, double* loss, double* grad_theta, double* grad_centroid);
int s1g_azimuth_focus(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                      double doppler_centroid, void* out, int64_t rows, int64_t cols, int out_type, int out_on_device);

/* ---- differentiable TOPS azimuth chain -------------------------------------
 * No counterpart in the reference.  The TOPS chain of one IW burst up to the
 * focused image before the time-domain unfolding (frequency unfolding,
 * range FFT, SRC, range IFFT, scale / RCMC / azimuth filter, azimuth IFFT:
 * s1_decoder.cpp:511-682 without azimuth_time_ufr, which only regrids the
 * focused burst), recomputed from the byte stream on each call:
 *   U = X exp(-i phi_a), phi_a = sum_j theta[j] x_a^(j+2), x_a = linspace(-1, 1, lines)
 *   F = f_a + f_dc(R) + centroid_offset  (f_dc the burst's estimated centroid)
 *   loss = image entropy of the focused S x range-samples image.
 * s1g_tops_adjoint returns the loss and (pointers not NULL) its gradient
 * with respect to theta[0..ntheta) (ntheta <= 8) and the centroid offset, by
 * a hand-written reverse-mode adjoint of every stage.  s1g_tops_focus writes
 * the focused image (rows = S of s1g_burst_unfold_shape, cols = range
 * samples).  IW swaths only (S1G_E_UNSUPPORTED otherwise); the handle's
 * precision selects FP64 or FP32 arithmetic (phases and sums in FP64). */
int s1g_tops_adjoint(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                     double centroid_offset, double* loss, double* grad_theta, double* grad_offset);
int s1g_tops_focus(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                   double centroid_offset, void* out, int64_t rows, int64_t cols, int out_type, int out_on_device);

/* Shape of a burst product (rows x cols). */
int s1g_burst_shape(s1g_decoder* h, const char* swath, int burst, int level, int64_t* rows, int64_t* cols);
/* Compute a burst product into out (rows*cols elements of out_type, row
 * pitch = cols; out_on_device: 1 if out is device memory).  The work runs on
 * the handle's stream and the call returns when out holds the result. */
int s1g_burst_product(s1g_decoder* h, const char* swath, int burst, int level, void* out, int64_t rows,
                      int64_t cols, int out_type, int out_on_device);

/* Swath products: rows of all bursts concatenated as the reference does
 * (IW azimuth products skip bursts of fewer than 1000 lines and append 20
 * zero rows after each).  Rows are cols wide, cols = width of the first row
 * (the width save_swath_as_cf32 writes, image_write_main.cpp:302-315); shorter
 * rows are zero-filled. */
int s1g_swath_shape(s1g_decoder* h, const char* swath, int level, int64_t* rows, int64_t* cols);
/* The length of every row of a swath product as the reference's CF_VEC_2D
 * has it: IW bursts keep their own widths (the zero rows after an azimuth
 * burst are as wide as the first row); a stripmap raw swath keeps each
 * azimuth block's width; processed multi-block stripmap rows are all as wide
 * as the widest block.  The buffers of s1g_swath_product are as wide as the
 * widest row, shorter rows zero-filled on the right.  widths may be NULL (or
 * cap < rows) to query *rows. */
int s1g_swath_row_widths(s1g_decoder* h, const char* swath, int level, int64_t* widths, int64_t cap, int64_t* rows);
int s1g_swath_product(s1g_decoder* h, const char* swath, int level, void* out, int64_t rows, int64_t cols,
                      int out_type, int out_on_device);

/* Scaled float32 images of a product (the s1_write TIFF commands' data,
 * scale() in signal_processing.cpp:1031-1071): the product is formed on the
 * GPU and scaled there (real, imag, |x|^2, (|x|+1e-12)/max|x|, or
 * 20 log10 of that), and rows x cols floats are written to out (host or
 * device).  Shapes as s1g_burst_shape / s1g_swath_shape. */
int s1g_burst_image(s1g_decoder* h, const char* swath, int burst, int level, int scaling, float* out, int64_t rows,
                    int64_t cols, int out_on_device);
int s1g_swath_image(s1g_decoder* h, const char* swath, int level, int scaling, float* out, int64_t rows,
                    int64_t cols, int out_on_device);
/* Spectrogram of one echo line of a burst's decoded data (spectrogram(),
 * signal_processing.cpp:794-844; s1_write uses fft_size 64, stride 32):
 * rows = fft_size, cols = floor((n/fft_size)(fft_size/stride)) windows, FP64.
 * The _image variant scales it on the GPU like s1g_burst_image. */
int s1g_spectrogram_shape(s1g_decoder* h, const char* swath, int burst, int fft_size, int stride, int64_t* rows,
                          int64_t* cols);
int s1g_spectrogram(s1g_decoder* h, const char* swath, int burst, int azimuth_line, int fft_size, int stride,
                    void* out, int64_t rows, int64_t cols, int out_type, int out_on_device);
int s1g_spectrogram_image(s1g_decoder* h, const char* swath, int burst, int azimuth_line, int fft_size, int stride,
                          int scaling, float* out, int64_t rows, int64_t cols, int out_on_device);
/* Write a rows x cols float32 host image as a BigTIFF file laid out like the
 * reference's _write_tif (image_write.cpp:3-25): one IEEE-float sample per
 * pixel, min-is-black, and data row rows-1 first (image row 0).  Host only. */
int s1g_write_tiff(const char* path, const float* image, int64_t rows, int64_t cols);

/* Azimuth geometry of a burst's SLC formation: S = the unfolded azimuth
 * length of the TOPS chain (floor(|k_dc T / prf| N_a), image_formation.cpp:
 * 125-160; N_a for stripmap) and the number of output rows.  Host-side only. */
int s1g_burst_unfold_shape(s1g_decoder* h, const char* swath, int burst, int64_t* S, int64_t* n_out);

/* The ECCM notch mask of a burst (eccm(), signal_processing.cpp:914-1004,
 * as _range_compress applies it with fft 128 and stride 64,
 * s1_decoder.cpp:470-474): rows x windows x 128 bytes, windows =
 * floor((n_r / 128) * (128 / 64)); byte [r][w][k] is 1 where bin k of
 * short-time window w of echo line r was zeroed (its central-difference
 * gradient magnitude reached the mitigation threshold) and 0 elsewhere,
 * including every bin of the lines the detection threshold passed over.
 * Uses the thresholds of s1g_apply_eccm (S1G_E_INVALID_ARGUMENT before it).
 * The decisions are taken in FP64 whatever the handle's precision, as every
 * pipeline takes them.  No counterpart returns the mask in the reference;
 * it is the set of bins its notch zeroes. */
int s1g_eccm_mask_shape(s1g_decoder* h, const char* swath, int burst, int64_t* rows, int64_t* windows);
int s1g_eccm_mask(s1g_decoder* h, const char* swath, int burst, uint8_t* out, int64_t rows, int64_t windows,
                  int out_on_device);

/* Hann-windowed sinc interpolation of complex lines at fractional sample
 * positions, on the GPU (sinc_interpolate, signal_processing.cpp:228-257,
 * applied at every position):
 *   out[r][k] = sum_{idx = floor(t) - L .. floor(t) + L, 0 <= idx < n}
 *               in[r][idx] sinc(t - idx) 0.5 (1 + cos(PI (t - idx) / L)),
 *   t = d_t[r * t_pitch + k]  (t_pitch 0: the same m positions for every line),
 * with 2L + 1 taps, L = half_width in 1..16 (L = 4: the 8-tap kernel with the
 * reference's centre tap).  d_in, d_t and d_out are device buffers (line
 * pitches in elements); elem_type S1G_CF32 (FP32 arithmetic) or S1G_CF64.
 * Work is queued on `stream` (a cudaStream_t or NULL); the call returns
 * without waiting. */
int s1g_sinc_interpolate(const void* d_in, int64_t rows, int64_t n, int64_t in_pitch, const double* d_t, int64_t m,
                         int64_t t_pitch, int half_width, void* d_out, int64_t out_pitch, int elem_type,
                         void* stream);

/* Corner turn of a complex matrix on the GPU (transpose,
 * signal_processing.cpp:463-479): d_out[c][r] = d_in[r][c] for rows x cols,
 * row pitches in elements, S1G_CF32 or S1G_CF64, d_in != d_out.  complex<float>
 * sources whose row pitch is even and base 16-byte aligned are staged through
 * shared memory by TMA tile loads (cp.async.bulk.tensor, 128 x 16 tiles);
 * others by a shared-memory tile transpose.  Queued on `stream`; returns
 * without waiting.  A TMA tile wait that ran out is reported by
 * s1g_take_device_timeout. */
int s1g_transpose(const void* d_in, int64_t rows, int64_t cols, int64_t in_pitch, void* d_out, int64_t out_pitch,
                  int elem_type, void* stream);
/* *flag = 1 if a bounded device wait (a TMA corner-turn tile load) ran out
 * since the last call, else 0; clears it.  Synchronous. */
int s1g_take_device_timeout(int* flag);

/* Doppler centroid rate and per-range-bin centroid of a burst's
 * range-compressed data (doppler.cpp:146-232); dc has cols entries. */
int s1g_burst_doppler(s1g_decoder* h, const char* swath, int burst, double* rate, double* dc, int64_t cols);

/* ---- batched processing (the benchmark's unit of work) --------------------
 * Process every burst of `swath` in each of n_streams decoders (e.g. the VV
 * and VH streams of one acquisition) to azimuth-compressed products in device
 * memory owned by the first handle, starting from the device-resident byte
 * streams (packet indexing included).  Returns the total number of input
 * echo samples processed (sum of lines x samples) in *samples.  The product
 * of burst b of stream s is then available through s1g_batch_output. */
int s1g_process_swath_batch(s1g_decoder** hs, int n_streams, const char* swath, int level, int64_t* samples);
int s1g_batch_output(s1g_decoder* h, int burst, const void** dev_ptr, int64_t* rows, int64_t* cols,
                     int64_t* pitch_elems, int* elem_type);
/* Restrict the bursts of h that the following batch calls process to
 * bursts[0..n) (indices into the swath's bursts; unknown indices select
 * nothing); n = -1 restores all bursts.  Used to split one swath's
 * (stream, burst) units across GPUs, one process per GPU: every rank opens
 * the same streams and processes only its share.  No counterpart in the
 * reference (which forms bursts one at a time, s1_decoder.cpp:315-346). */
int s1g_set_batch_bursts(s1g_decoder* h, const int* bursts, int n);
/* CUDA-graph batching (on by default): the first s1g_process_swath_batch call
 * for a given (handles, swath, level, settings) runs eagerly and sizes every
 * buffer; the second captures the whole enqueue sequence (both streams) into
 * one CUDA graph; later calls replay it.  Turning it off (or on) drops the
 * graph.  Stage timing (s1g_set_stage_timing) always runs eagerly. */
int s1g_set_batch_graph(s1g_decoder* h, int on);
/* Page-locked host destinations for the outputs of the following batch
 * calls on h (the first handle of the batch): host[k] receives burst k's
 * product (rows x pitch elements, as s1g_batch_output reports) by a copy that
 * starts as soon as that burst is formed, on a copy stream of the handle, so
 * the transfers overlap the later bursts' work; the batch call returns when
 * every copy has landed.  A null entry skips that burst; n = 0 turns the
 * copies off. */
int s1g_batch_host_outputs(s1g_decoder* h, void* const* host, int n);

/* Wall time (ms) of the last product / batch call measured with CUDA events
 * on the handle's stream, and (when stage timing is on) the accumulated
 * per-stage times as "name total_ms count" lines. */
int s1g_last_timing(const s1g_decoder* h, double* ms, char* stages, size_t stages_len);
/* Record CUDA events between pipeline stages (adds a little overhead);
 * switching it resets the accumulated stage times. */
int s1g_set_stage_timing(s1g_decoder* h, int on);
/* Choices of the FFT autotuner so far in this process: "on|off radices
 * n:r1.r2... lengths minlen>M ...".  The tuner times candidate radix orders
 * and 7-smooth transform lengths of the fused kernels' FFT core on this GPU
 * the first time a length is needed (S1G_AUTOTUNE=0 turns it off) and keeps
 * the choices in a file shared by the processes of a machine
 * (S1G_FFT_TUNE_FILE, default fft_tune.txt beside the library). */
int s1g_tuning_report(char* buf, size_t buflen);

/* Nominal FP32 arithmetic of the fused FP32 path per stage for one burst, as
 * "stage flops" lines (stage names as in s1g_last_timing): 5 N log2 N per
 * complex FFT of N points, a chirp-z transform as its two convolution FFTs
 * plus its pointwise products, the compensated Doppler transforms as plain
 * FFTs, the time unfolding's gather, grid FFTs and stencil.  A TOPS burst's
 * SLC is formed once for the tile count (line "tiles").  The handle must be
 * in S1G_PREC_FP32 precision.  No counterpart in
 * the reference; the benchmark divides these by the stage times for the
 * compute roofline. */
int s1g_burst_stage_flops(s1g_decoder* h, const char* swath, int burst, char* buf, size_t len);

/* Number of GPU kernels this library has launched since it was loaded. */
int s1g_launch_count(int64_t* n);

/* ---- allocation-free decode --------------------------------------------
 * No counterpart in the reference (whose decode allocates per packet).
 * For callers that must not allocate device memory while they run: a chain
 * whose GPU memory budget is fixed at start-up, or a program sharing the GPU
 * with latency-sensitive streams that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree imply.  The caller owns every buffer:
 *   d_stream   device copy of the Level-0 byte stream (nbytes)
 *   d_offsets  device int64 byte offsets of the npackets packets to decode
 *              (all type-D/FDBAQ with num_quadratures == num_quads)
 *   d_out      device complex<float> rows, row r at d_out + r*out_pitch
 *              elements, 2*num_quads samples each (get_signal's layout)
 *   d_status   device int32 per packet: 0 or one of the S1G_E_* decode codes
 *              (rows of failed packets are zero; an offset whose 68-byte
 *              header does not lie inside the nbytes of the stream gives
 *              S1G_E_PACKET_LENGTH without a read)
 * Work is queued on `stream` (a cudaStream_t, or NULL for the default
 * stream); the call returns without waiting.  Nothing is allocated: the
 * decoder's scratch is a fixed 16 MiB device array inside the library (held
 * by every GPU that loads it until exit).  num_quads is at most 65535 (the
 * width of the num_quadratures field; S1G_E_INVALID_ARGUMENT beyond), which
 * needs 262 KB of scratch per packet, so the array holds at least 64 packets
 * at a time and longer packet runs are decoded in chunks of that many (696
 * packets per chunk at num_quads 6000).  S1G_E_SCRATCH_LIMIT is returned if
 * one packet's scratch cannot fit.  The first call on each device, with that device
 * current, resolves the scratch address and copies the 10 KB Huffman table in
 * with a synchronous cudaMemcpyToSymbol; make that first call before any
 * stream capture.  All calls share the one scratch array: calls that can
 * overlap on the GPU (different streams without ordering between them) race
 * and corrupt each other's results; calls on one stream are safe.  Nothing
 * in the scratch has to start at zero: every byte read was written earlier in
 * the same call. */
int s1g_decode_fdbaq_noalloc(const uint8_t* d_stream, int64_t nbytes, const int64_t* d_offsets, int64_t npackets,
                             int num_quads, void* d_out, int64_t out_pitch, int32_t* d_status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* S1G_H */
