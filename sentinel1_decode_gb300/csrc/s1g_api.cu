// C ABI and per-burst pipeline orchestration (include/s1g.h).
//
// A decoder handle owns: the device copy of the byte stream, the packet
// offsets found by the GPU indexer, the host header mirror used for
// segmentation (the reference's S1_Decoder constructor path), an FFT engine,
// and grow-only device work buffers.  Each product call runs the stages of
// the reference's _range_compress / _azimuth_compress (s1_decoder.cpp:448-701)
// as GPU kernels on the handle's stream.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>

#include "s1g_kernels.h"
#include "s1g_dcest.h"
#include "s1g_fast.cuh"
#include "s1g_model.h"
#include "s1g_aux.h"
#include "s1g_tma.h"

namespace s1g {

constexpr double kPI_ = 3.14159265358979;
constexpr double kC_ = 299792458.0;
constexpr double kCF_ = 5.405000454334350e+9;
constexpr double kWL_ = kC_ / kCF_;

struct S1Error : std::runtime_error {
    int code;
    S1Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

struct Buf {
    void* p = nullptr;
    size_t n = 0;
    void* get(size_t bytes) {
        if (bytes > n) {
            if (p) cudaFree(p);
            p = nullptr;
            n = 0;
            check_cuda(cudaMalloc(&p, bytes), "work buffer cudaMalloc");
            n = bytes;
        }
        return p;
    }
    template <typename T>
    T* as(size_t count) { return (T*)get(sizeof(T) * count); }
    ~Buf() {
        if (p) cudaFree(p);
    }
};

struct Result {   // a product left in device memory
    const void* ptr = nullptr;
    long long rows = 0, cols = 0, pitch = 0;
    int elem = S1G_CF64;   // element type of ptr
    const int* status = nullptr;   // device status word of the time unfolding (TOPS FP32 path)
};

}  // namespace s1g

using namespace s1g;

struct s1g_decoder {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::unique_ptr<FftEngine> fft;
    uint8_t* d_stream = nullptr;
    long long nbytes = 0;
    long long* d_off = nullptr;
    int npk = 0;
    size_t stream_cap = 0;        // bytes allocated at d_stream
    long long off_cap = 0;        // offsets allocated at d_off
    uint64_t content_sig = 0;     // hash of the packet headers and offsets of the current stream
    uint64_t epoch = 0;           // bumped whenever content_sig changes (invalidates content-derived plans)
    std::vector<PacketHdr> hdr;
    std::vector<std::string> swath_order;
    std::map<std::string, int> swath_counts;
    std::map<std::string, std::vector<std::vector<int>>> bursts;
    StateVectors sv;
    bool use_eccm = false;
    int det = 0, mit = 0;
    int precision = S1G_PREC_FP32;
    int rcmc = S1G_RCMC_PHASE;    // range cell migration correction of the TOPS row pass
    int rcmc_L = 4;               // sinc half-width (S1G_RCMC_SINC)
    int abc_fields = 0;   // formats A/B/C: 0 = the reference's output, 1 = each sample from its own fields
    std::string err;
    IndexScratch isc;
    DecodeScratch dsc;
    DecodeTables tabs;
    Buf bA, bB, bC, bD, bE, bKa, bOut, bStage, bSmall, bRows, bCols, bStatus, bFlags, bRef, bTab, bPk;
    Buf bFdf, bKN, bTd, bTstat, bDc, bDcPart, bRawAll, bDecStatus, bBatchStatus;
    Buf bTuD, bTuG, bTuI, bTuW, bTuR, bKa0;   // time-unfolding per-burst tables
    Buf bImgIn, bImgOut, bImgMax;        // image epilogue
    Buf bJ0, bJ1, bJ2, bJ3, bJ4, bJ5, bJe, bJd;   // differentiable azimuth chains
    Buf bRawW;                               // decoded rows after the FP64 ECCM notch (FP32 paths)
    Buf bEccm, bEccmSt;                      // FP64 decode of the ECCM notch
    Buf bEccmRoots;                          // FP64 roots of unity of the ECCM detection
    Buf bRawAll64;                           // FP64 samples of a batch decode (ECCM)
    Buf bEccmMask;                           // s1g_eccm_mask output staging
    // fast-path caches: per-burst tables (keyed by first packet index) and
    // chirp-z transform tables (keyed by period, nin, nout)
    std::map<int, std::shared_ptr<struct FastBurst>> fast_bursts;
    std::map<std::tuple<int, int, int>, std::shared_ptr<struct CztTables>> czts;
    std::map<int, std::shared_ptr<s1g::CfftPlan>> cffts;   // compensated FFT plans by length
    std::map<std::string, std::shared_ptr<struct BatchDecode>> batch_decodes;   // by swath/level
    // every burst of a swath decoded in one launch pair for the per-burst
    // FP32 calls (built on the first such call, dropped when the stream
    // content or the A/B/C decode mode changes)
    std::map<std::string, std::shared_ptr<struct SwathDecode>> swath_decodes;
    int num_sms = 0;
    Result last;
    double last_ms = 0;
    std::string stage_text;
    bool stage_timing = false;
    double ingest_ms = 0;           // s1g_open_file: map + staged upload
    long long ingest_bytes = 0;
    // batched launch captured into a CUDA graph (s1g_process_swath_batch)
    bool use_graph = true;
    std::map<std::vector<int>, std::unique_ptr<Buf>> burst_idx;   // device packet lists of non-contiguous bursts
    std::unique_ptr<struct BatchGraph> graph;
    std::string graph_warm;
    std::vector<std::pair<std::string, cudaEvent_t>> marks;
    std::map<std::string, double> stage_ms;
    std::map<std::string, int> stage_n;
    void mark(const char* name) {
        if (!stage_timing) return;
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, stream);
        marks.push_back({name, e});
    }
    void close_marks() {
        if (marks.empty()) return;
        mark("end");
        cudaEventSynchronize(marks.back().second);
        for (size_t i = 0; i + 1 < marks.size(); ++i) {
            float ms = 0;
            cudaEventElapsedTime(&ms, marks[i].second, marks[i + 1].second);
            stage_ms[marks[i].first] += ms;
            stage_n[marks[i].first] += 1;
        }
        for (auto& m : marks) cudaEventDestroy(m.second);
        marks.clear();
    }
    // batch outputs (per burst of the last batch call)
    std::vector<std::unique_ptr<Buf>> batch_bufs;
    std::vector<Result> batch_out;
    // pinned host destinations of the batch outputs (s1g_batch_host_outputs),
    // filled by copies on copy_stream as each burst finishes
    std::vector<void*> batch_host;
    // bursts of this handle's swath that s1g_process_swath_batch processes
    // (s1g_set_batch_bursts; empty with batch_sel_on false = all)
    std::vector<int> batch_sel;
    bool batch_sel_on = false;
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> slot_done;
    ~s1g_decoder() {
        for (auto e : slot_done) cudaEventDestroy(e);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (d_stream) cudaFree(d_stream);
        if (d_off) cudaFree(d_off);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace s1g {

static bool is_iw(const std::string& s) { return s == "IW1" || s == "IW2" || s == "IW3"; }
static bool is_sm(const std::string& s) {
    return s == "S1" || s == "S2" || s == "S3" || s == "S4" || s == "S5" || s == "S6" || s == "S5_N" || s == "S5_S";
}
// Data format of a packet (_set_data_format, packet.cpp:264-274): D =
// FDBAQ (baq_mode 12..14), A/B = bypass (0), C = BAQ (3..5).
enum FormatKind { FMT_D, FMT_FIXED, FMT_INVALID };
static FormatKind format_kind(const PacketHdr& p) {
    const int64_t b = p[F_BAQ_MODE];
    if (b >= 12 && b <= 14) return FMT_D;
    if (b == 0 || (b >= 3 && b <= 5)) return FMT_FIXED;
    return FMT_INVALID;
}

static bool is_echo(const std::string& s) {
    return is_iw(s) || is_sm(s) || s == "EW1" || s == "EW2" || s == "EW3" || s == "EW4" || s == "EW5" || s == "WV1" ||
           s == "WV2";
}

// get_packets_in_bursts (packet.cpp:1026-1076)
static std::vector<std::vector<int>> split_bursts(const std::vector<PacketHdr>& hdr, const std::string& swath,
                                                  bool cal) {
    std::vector<std::vector<int>> bursts;
    std::vector<int> cur;
    long long prev_az = 0, prev_pri = 0;
    const int n = (int)hdr.size();
    for (int i = 0; i < n; ++i) {
        if (hdr[i].swath() == swath) {
            if (!cal) {
                const long long az = hdr[i][F_AZ_BEAM];
                const long long pc = hdr[i][F_PRI_COUNT];
                if (prev_az == 0) {
                    prev_az = az;
                    prev_pri = pc;
                }
                if (az < prev_az || pc > prev_pri + 1) {
                    if (cur.size() >= 1000) bursts.push_back(cur);
                    cur.clear();
                }
                prev_pri = pc;
                prev_az = az;
            }
            cur.push_back(i);
        }
        if (i == n - 1 && !cur.empty()) bursts.push_back(cur);
    }
    return bursts;
}

// Copy n bytes of pageable host memory (e.g. a memory-mapped file) to the
// device through two pinned staging buffers: host threads fill one buffer
// (touching the mapped pages, which reads the file) while the copy engine
// drains the other.
static void upload_staged(uint8_t* dst, const uint8_t* src, size_t n, cudaStream_t st) {
    const size_t chunk = (size_t)32 << 20;
    struct Staging {
        uint8_t* pin[2] = {nullptr, nullptr};
        cudaEvent_t done[2] = {nullptr, nullptr};
        ~Staging() {
            for (int b = 0; b < 2; ++b) {
                if (done[b]) cudaEventSynchronize(done[b]), cudaEventDestroy(done[b]);
                if (pin[b]) cudaFreeHost(pin[b]);
            }
        }
    } sg;
    for (int b = 0; b < 2; ++b) {
        check_cuda(cudaMallocHost(&sg.pin[b], std::min(chunk, std::max<size_t>(n, 1))), "staging alloc");
        check_cuda(cudaEventCreateWithFlags(&sg.done[b], cudaEventDisableTiming), "staging event");
    }
    const unsigned nthr = std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2));
    for (size_t off = 0, i = 0; off < n; off += chunk, ++i) {
        const int b = (int)(i & 1);
        const size_t len = std::min(chunk, n - off);
        if (i >= 2) check_cuda(cudaEventSynchronize(sg.done[b]), "staging wait");
        const size_t part = (len + nthr - 1) / nthr;
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nthr && t * part < len; ++t)
            th.emplace_back([&, t] { std::memcpy(sg.pin[b] + t * part, src + off + t * part, std::min(part, len - t * part)); });
        std::memcpy(sg.pin[b], src + off, std::min(part, len));
        for (auto& x : th) x.join();
        check_cuda(cudaMemcpyAsync(dst + off, sg.pin[b], len, cudaMemcpyHostToDevice, st), "stream upload");
        check_cuda(cudaEventRecord(sg.done[b], st), "staging record");
    }
    check_cuda(cudaStreamSynchronize(st), "stream upload sync");
}

// Load a byte stream into the handle: copy it to the device (reusing the
// allocation when it is large enough), index it on the GPU, parse the
// headers, segment swaths and bursts (S1_Decoder::_set_packets,
// s1_decoder.cpp:13-34), build the state vectors.  Plans derived from the
// content (per-burst tables, batch decode jobs, the captured batch graph)
// are kept only when the new stream's headers and packet layout hash to the
// same value as the previous stream's and no buffer moved.
static void ingest(s1g_decoder* h, const uint8_t* bytes, size_t n, bool staged) {
    const size_t need = std::max<size_t>(n, 1) + 64;
    bool moved = false;
    if (!h->d_stream || need > h->stream_cap) {
        if (h->d_stream) cudaFree(h->d_stream);
        h->d_stream = nullptr;
        h->stream_cap = 0;
        check_cuda(cudaMalloc(&h->d_stream, need), "stream alloc");
        h->stream_cap = need;
        moved = true;
    }
    h->nbytes = (long long)n;
    if (staged) {
        upload_staged(h->d_stream, bytes, n, h->stream);
    } else if (n) {
        // cudaMemcpyDefault: `bytes` may be host (pageable or pinned) or device memory
        check_cuda(cudaMemcpyAsync(h->d_stream, bytes, n, cudaMemcpyDefault, h->stream), "stream upload");
    }
    check_cuda(cudaMemsetAsync(h->d_stream + n, 0, 64, h->stream), "stream pad");
    // upper bound on packets: every packet is at least 7 bytes
    const int maxp = (int)std::min<long long>(h->nbytes / 7 + 1, 1LL << 30);
    if (!h->d_off || maxp > h->off_cap) {
        if (h->d_off) cudaFree(h->d_off);
        h->d_off = nullptr;
        h->off_cap = 0;
        check_cuda(cudaMalloc(&h->d_off, sizeof(long long) * (size_t)maxp), "offsets");
        h->off_cap = maxp;
        moved = true;
    }
    int count = 0;
    index_packets(h->d_stream, h->nbytes, h->d_off, maxp, h->isc, h->stream, true, &count);
    h->npk = count;
    std::vector<uint8_t> hh((size_t)count * 68);
    std::vector<long long> off(count);
    if (count > 0) {
        uint8_t* d_hdr = h->bSmall.as<uint8_t>((size_t)count * 68);
        gather_headers(h->d_stream, h->nbytes, h->d_off, count, d_hdr, h->stream);
        check_cuda(cudaMemcpyAsync(hh.data(), d_hdr, hh.size(), cudaMemcpyDeviceToHost, h->stream), "hdr down");
        check_cuda(cudaMemcpyAsync(off.data(), h->d_off, sizeof(long long) * count, cudaMemcpyDeviceToHost, h->stream),
                   "off down");
        check_cuda(cudaStreamSynchronize(h->stream), "open sync");
    }
    h->hdr.assign(count, PacketHdr());
    for (int i = 0; i < count; ++i) {
        parse_header(hh.data() + (size_t)i * 68, h->hdr[i]);
        h->hdr[i].offset = off[i];
    }
    h->swath_order.clear();
    h->swath_counts.clear();
    h->bursts.clear();
    for (const auto& p : h->hdr) {
        const std::string s = p.swath();
        if (!h->swath_counts.count(s)) h->swath_order.push_back(s);
        h->swath_counts[s]++;
    }
    for (const auto& s : h->swath_order) h->bursts[s] = split_bursts(h->hdr, s, !is_echo(s));
    h->sv = StateVectors();
    if (h->hdr.size() > 1) h->sv.build(h->hdr);
    // 64-bit multiply-xorshift hash over the stream size, the headers and
    // the packet offsets, eight bytes at a time
    uint64_t sig = 1469598103934665603ULL;
    auto mix = [&sig](const void* p, size_t k) {
        const uint8_t* b = (const uint8_t*)p;
        size_t i = 0;
        for (; i + 8 <= k; i += 8) {
            uint64_t w;
            memcpy(&w, b + i, 8);
            sig = (sig ^ w) * 0x9E3779B97F4A7C15ULL;
            sig ^= sig >> 29;
        }
        for (; i < k; ++i) sig = (sig ^ b[i]) * 1099511628211ULL;
    };
    mix(&h->nbytes, sizeof(h->nbytes));
    mix(hh.data(), hh.size());
    mix(off.data(), sizeof(long long) * off.size());
    if (moved || sig != h->content_sig || h->epoch == 0) {
        h->content_sig = sig;
        ++h->epoch;
        h->fast_bursts.clear();
        h->batch_decodes.clear();
        h->swath_decodes.clear();
        h->burst_idx.clear();
        h->graph.reset();
        h->graph_warm.clear();
    }
}

static void open_stream(s1g_decoder* h, const uint8_t* bytes, size_t n, bool staged = false) {
    check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
    check_cuda(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
    h->fft.reset(new FftEngine(h->stream));
    h->tabs.init();
    ingest(h, bytes, n, staged);
}

static const std::vector<int>& burst_packets(s1g_decoder* h, const std::string& swath, int burst) {
    // _validate_request, s1_decoder.cpp:45-89
    auto it = h->bursts.find(swath);
    if (it == h->bursts.end()) throw S1Error(S1G_E_BAD_SWATH, "The requested swath, " + swath + ", does not exist in the data.");
    if (burst < 0 || burst >= (int)it->second.size())
        throw S1Error(S1G_E_BAD_BURST, "The requested burst, " + std::to_string(burst) + ", does not exist in the data. There are " +
                                           std::to_string(it->second.size()) + " bursts in swath " + swath + ".");
    return it->second[burst];
}

// ------------------------------------------------------------------ per-burst pipeline
template <typename R>
struct Pipe {
    s1g_decoder* h;
    cudaStream_t st;
    FftEngine& fft;
    const std::vector<int>* cur_pk = nullptr;   // packets of the burst being processed
    explicit Pipe(s1g_decoder* hh) : h(hh), st(hh->stream), fft(*hh->fft) {}

    template <typename T>
    T* upload(Buf& b, const std::vector<T>& v) {
        T* d = b.as<T>(v.size());
        check_cuda(cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st), "upload");
        return d;
    }

    void fft_rows(int n, const cpx<R>* in, long long ip, cpx<R>* out, long long op, long long rows, int dir) {
        auto p = fft.plan<R>(n);
        fft.rows<R>(*p, in, ip, out, op, rows, dir);
    }

    // decode -> [n_a][n_r] in buffer A
    cpx<R>* decode(const std::vector<int>& pk, const BurstGeom& g) {
        const int npk = (int)pk.size();
        bool contiguous = true;
        for (size_t i = 1; i < pk.size(); ++i)
            if (pk[i] != pk[i - 1] + 1) contiguous = false;
        const int* d_idx = contiguous ? nullptr : upload(h->bPk, pk);
        bool any_d = false, any_fixed = false;
        for (int i : pk) {
            const FormatKind k = format_kind(h->hdr[i]);
            if (k == FMT_INVALID) throw S1Error(S1G_E_BAD_FORMAT, "packet " + std::to_string(i) + ": BAQ Mode is invalid.");
            (k == FMT_D ? any_d : any_fixed) = true;
        }
        cpx<R>* A = h->bA.as<cpx<R>>((size_t)npk * g.n_r);
        int* status = h->bStatus.as<int>(npk);
        if (any_d)
            decode_burst<R>(h->d_stream, h->nbytes, h->d_off, d_idx, pk.front(), npk, g.nq, A, g.n_r, status, h->dsc, h->tabs, st);
        if (any_fixed)
            decode_fixed_burst<R>(h->d_stream, h->nbytes, h->d_off, d_idx, pk.front(), npk, g.nq, A, g.n_r, status,
                                  h->abc_fields, st);
        std::vector<int> hs(npk);
        check_cuda(cudaMemcpyAsync(hs.data(), status, sizeof(int) * npk, cudaMemcpyDeviceToHost, st), "status");
        check_cuda(cudaStreamSynchronize(st), "decode sync");
        for (int i = 0; i < npk; ++i)
            if (hs[i]) {
                static const char* names[] = {"", "", "", "", "", "", "", "packet length", "bit read past end",
                                              "BRC value is invalid.", "Max bit length exceeded in Huffman decoding.",
                                              "MCode is greater than the comparison flag.", "ragged burst",
                                              "BAQ Mode is invalid."};
                const int c = hs[i];
                throw S1Error(c, std::string("packet ") + std::to_string(pk[i]) + ": " + (c >= -13 ? names[-c] : "decode error"));
            }
        return A;
    }

    // mask (optional): n_a x windows x 128 bytes, 1 where a bin was zeroed;
    // the rows the detector passes over are left untouched (zero them first)
    void eccm(cpx<R>* A, const BurstGeom& g, unsigned char* mask = nullptr) {
        const int n_a = g.n_a, n_r = g.n_r;
        cpx<R>* B = h->bB.as<cpx<R>>((size_t)n_a * n_r);
        fft_rows(n_r, A, n_r, B, n_r, n_a, -1);
        int* flags = h->bFlags.as<int>(n_a);
        eccm_detect<R>(B, n_r, n_r, n_a, (double)h->det, flags, st);
        const FftDesc<R> d128 = fft.smem_desc<R>(128);
        eccm_notch<R>(A, n_r, n_r, n_a, flags, (double)h->mit, d128, mask, st);
    }

    // The ECCM notch of the FP32 paths, run in FP64: its line detection and
    // bin mitigation are hard thresholds (signal_processing.cpp:914-1004), and
    // FP32 rounding flips the decisions of bins near them, which moves the
    // product by far more than rounding.  The burst's FP64 samples come from
    // pre64 when the batch decode reconstructed them from its own symbols
    // (notched in place there), else the burst is decoded again in FP64 (no
    // host synchronisation; the FP32 decode of the same packets reports any
    // decode error); the notched lines are written to `out` as complex<float>.
    void eccm_fp64(const std::vector<int>& pk, const BurstGeom& g, cf32* out, cf64* pre64 = nullptr) {
        if (pre64) {
            eccm_from64(pre64, g, out);
            return;
        }
        const int npk = (int)pk.size();
        bool contiguous = true;
        bool any_d = false, any_fixed = false;
        for (size_t i = 0; i < pk.size(); ++i) {
            if (i && pk[i] != pk[i - 1] + 1) contiguous = false;
            (format_kind(h->hdr[pk[i]]) == FMT_D ? any_d : any_fixed) = true;
        }
        // a packet list that stays in device memory: this runs inside captured batches
        const int* d_idx = nullptr;
        if (!contiguous) {
            std::unique_ptr<Buf>& b = h->burst_idx[pk];
            if (!b) {
                b = std::make_unique<Buf>();
                check_cuda(cudaMemcpy(b->as<int>(pk.size()), pk.data(), sizeof(int) * pk.size(), cudaMemcpyHostToDevice),
                           "burst index upload");
            }
            d_idx = (const int*)b->p;
        }
        cf64* a64 = h->bEccm.as<cf64>((size_t)npk * g.n_r);
        int* status = h->bEccmSt.as<int>(npk);
        if (any_d)
            decode_burst<double>(h->d_stream, h->nbytes, h->d_off, d_idx, pk.front(), npk, g.nq, a64, g.n_r, status,
                                 h->dsc, h->tabs, st);
        if (any_fixed)
            decode_fixed_burst<double>(h->d_stream, h->nbytes, h->d_off, d_idx, pk.front(), npk, g.nq, a64, g.n_r,
                                       status, h->abc_fields, st);
        eccm_from64(a64, g, out);
    }

    // Line detection (max |FFT(line)| >= det) from an FP32 FFT of the lines,
    // with the lines whose maximum lies within 1e-4 of det decided by FP64
    // DFT bins, then the notch of the flagged lines in compensated FP32 from
    // the FP64 samples (s1g_eccm.cu), written as complex<float>; the other
    // lines are the samples cast.
    void eccm_from64(const cf64* a64, const BurstGeom& g, cf32* out) {
        const int n_a = g.n_a, n_r = g.n_r;
        convert_rows<float, double>(a64, n_r, out, n_r, n_r, n_r, n_a, st);
        Pipe<float> p32(h);
        cf32* B = h->bB.as<cf32>((size_t)n_a * n_r);
        p32.fft_rows(n_r, out, n_r, B, n_r, n_a, -1);
        int* flags = h->bFlags.as<int>(n_a);
        eccm_detect_mixed(B, n_r, n_r, n_a, (double)h->det, a64, n_r, h->bEccmRoots.as<cf64>(n_r), flags, st);
        auto& cp = h->cffts[128];
        if (!cp) cp = make_cfft_plan(128);
        eccm_notch_cc(a64, n_r, out, n_r, n_r, n_a, flags, (double)h->mit, cp->d, st);
    }

    // _range_compress (s1_decoder.cpp:448-508) -> [n_a][n_r] in A
    cpx<R>* range_compress(cpx<R>* A, const BurstGeom& g, bool rd) {
        const int n_a = g.n_a, n_r = g.n_r;
        if (h->use_eccm) {
            if constexpr (sizeof(R) == 4) {
                if (cur_pk) eccm_fp64(*cur_pk, g, A);
                else eccm(A, g);
            } else {
                eccm(A, g);
            }
        }
        const int M = (int)next_smooth7((long long)n_r + g.L);
        // reference function at length M: conj(FFT_M(chirp at [0,L))) / (E * M)
        {
            std::vector<cpx<double>> c((size_t)M, mk(0.0, 0.0));
            for (int t = 0; t < g.L; ++t) c[t] = g.chirp[t];
            cf64* dc = (cf64*)h->bTab.get(sizeof(cf64) * M);
            check_cuda(cudaMemcpyAsync(dc, c.data(), sizeof(cf64) * M, cudaMemcpyHostToDevice, st), "chirp up");
            auto p64 = fft.plan<double>(M);
            fft.rows<double>(*p64, dc, M, dc, M, 1, -1);
            std::vector<cpx<double>> spec(M);
            check_cuda(cudaMemcpyAsync(spec.data(), dc, sizeof(cf64) * M, cudaMemcpyDeviceToHost, st), "chirp down");
            check_cuda(cudaStreamSynchronize(st), "ref sync");
            std::vector<cpx<R>> ref(M);
            const double s = 1.0 / (g.energy * (double)M);
            for (int k = 0; k < M; ++k) ref[k] = mk((R)(spec[k].x * s), (R)(-spec[k].y * s));
            upload(h->bRef, ref);
        }
        const cpx<R>* ref = (const cpx<R>*)h->bRef.p;
        cpx<R>* B = h->bB.as<cpx<R>>((size_t)n_a * M);
        pad_rows<R>(A, n_r, n_r, B, M, M, n_a, st);
        fft_rows(M, B, M, B, M, n_a, -1);
        mul_rows_by_vec<R>(B, M, M, n_a, ref, st);
        fft_rows(M, B, M, B, M, n_a, +1);
        rc_crop<R>(B, M, M, A, n_r, n_r, g.h, n_a, st);
        if (rd) {
            // transpose, azimuth FFT, fftshift, transpose (s1_decoder.cpp:499-505)
            cpx<R>* Bt = h->bB.as<cpx<R>>((size_t)n_a * n_r);
            cpx<R>* Ct = h->bC.as<cpx<R>>((size_t)n_a * n_r);
            transpose_batched<R>(A, n_r, 0, Bt, n_a, 0, n_a, n_r, 1, st);
            fft_rows(n_a, Bt, n_a, Bt, n_a, n_r, -1);
            roll_rows<R>(Bt, n_a, Ct, n_a, n_a, n_a / 2, n_r, st);
            transpose_batched<R>(Ct, n_a, 0, A, n_r, 0, n_r, n_a, 1, st);
        }
        return A;
    }

    std::vector<RowParam> row_params(const BurstGeom& g, int S, double time_delta, const std::vector<double>& az_freqs) {
        std::vector<RowParam> rp(S);
        for (int i = 0; i < S; ++i) {
            double pos[3], vel[3];
            h->sv.interpolate(g.t0 + time_delta * i, pos, vel);
            const double vn = std::sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
            // image_formation.cpp:398-402
            const double lat = pos[2] / pos[0];
            const double a = 6378137.0, b = 6356752.3142;
            const double num = std::pow(a * a * std::cos(lat), 2.0) + std::pow(b * b * std::sin(lat), 2.0);
            const double den = std::pow(a * std::cos(lat), 2.0) + std::pow(b * std::sin(lat), 2.0);
            rp[i].re = std::sqrt(num / den);
            rp[i].h = std::sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
            rp[i].v = vn;
            rp[i].fa = az_freqs[i];
        }
        return rp;
    }

    double v_norm0() const {
        if (h->sv.v.empty()) throw S1Error(S1G_E_GEOMETRY, "no state vectors in the data");
        const auto& v0 = h->sv.v[0];
        return std::sqrt(std::pow(v0[0], 2.0) + std::pow(v0[1], 2.0) + std::pow(v0[2], 2.0));
    }

    double dc_rate(const BurstGeom& g) const {
        // doppler.cpp:224-232
        const double rate = ((g.beam1 - g.beam0) / (g.pri * g.n_a));
        return (-2 * v_norm0() * rate) / kWL_;
    }

    // Doppler centroid (doppler.cpp:146-221) of the range-compressed burst
    double* doppler(const cpx<R>* rc, const BurstGeom& g, double rate) {
        const int n_a = g.n_a, n_r = g.n_r;
        std::vector<cpx<R>> d(n_a);
        const std::vector<double> t = linspace(0.0, 1.06, n_a);
        for (int a = 0; a < n_a; ++a) {
            const double th = kPI_ * rate * std::pow(t[a] - (0.5 * 1.06), 2.0);
            d[a] = mk((R)std::cos(th), (R)std::sin(th));
        }
        cpx<R>* dd = upload(h->bTab, d);
        cf64* sums = (cf64*)h->bSmall.get(sizeof(cf64) * n_r);
        dc_sums<R>(rc, n_r, n_a, n_r, dd, sums, st);
        DcFitArgs fa{};
        fa.n_rng = n_r;
        fa.num_blocks = 30;
        fa.prf = 1.0 / (g.pri);
        const std::vector<double> rt = linspace(g.near, g.far, 30);
        for (int b = 0; b < 30; ++b) fa.rt[b] = rt[b] - rt[0];
        fa.near = g.near;
        fa.far = g.far;
        double* fdc = h->bCols.as<double>(n_r);
        dc_fit(sums, fa, fdc, st);
        return fdc;
    }

    // _azimuth_compress (s1_decoder.cpp:511-701); returns the product
    Result azimuth(cpx<R>* A, const BurstGeom& g, bool tops) {
        const int n_r = g.n_r;
        int n_a = g.n_a;
        const double bd = g.swath_number == 11 ? 675 : 600;
        double time_delta = g.T / g.prf;
        double rate = 0.0;
        double* fdc = nullptr;
        int S = n_a;
        double nrep = 0.0;
        if (tops) {
            rate = dc_rate(g);
            h->mark("doppler");
            fdc = doppler(A, g, rate);
            h->mark("freq_unfold");
            // azimuth_frequency_ufr (image_formation.cpp:125-219)
            nrep = std::abs(rate * g.T / g.prf);
            const double bw = nrep * g.prf / 2.0;
            S = (int)std::floor(nrep * n_a);
            if (S < 4) throw S1Error(S1G_E_GEOMETRY, "azimuth frequency unfolding needs a beam sweep (no Doppler rate)");
            const int mid = S / 2;
            const int start = (int)(mid - (std::floor(bd) / 2));
            const int end = (int)(mid + (std::floor(bd) / 2));
            const int offset = (int)std::floor(nrep);
            int tile_len = offset * n_a;
            if (std::floor(nrep) != nrep) tile_len += (int)std::floor((nrep - std::floor(nrep)) * n_a);
            tile_len = std::min(tile_len, S);
            const std::vector<double> f = linspace(-bw, bw, S);
            std::vector<cpx<R>> der(S), rer(S);
            for (int k = 0; k < S; ++k) {
                const double th = -kPI_ * (1 / rate) * std::pow(f[k], 2.0);
                const double th2 = kPI_ * (1 / rate) * std::pow(f[k], 2.0);
                der[k] = mk((R)std::cos(th), (R)std::sin(th));
                rer[k] = mk((R)std::cos(th2), (R)std::sin(th2));
            }
            cpx<R>* dder = upload(h->bTab, der);
            cpx<R>* Bt = h->bB.as<cpx<R>>((size_t)n_r * std::max(n_a, S));
            cpx<R>* Ct = h->bC.as<cpx<R>>((size_t)n_r * S);
            transpose_batched<R>(A, n_r, 0, Bt, n_a, 0, n_a, n_r, 1, st);
            fft_rows(n_a, Bt, n_a, Bt, n_a, n_r, -1);
            fufr_prep<R>(Bt, n_a, n_a, Ct, S, S, tile_len, dder, n_r, st);
            fft_rows(S, Ct, S, Ct, S, n_r, -1);
            band_select<R>(Ct, S, Bt, S, S, start, end - start, n_r, st);
            fft_rows(S, Bt, S, Bt, S, n_r, +1);
            cpx<R>* drer = upload(h->bRef, rer);
            scale_mul_vec<R>(Bt, S, S, n_r, drer, 1.0 / S, st);
            A = h->bA.as<cpx<R>>((size_t)S * n_r);
            transpose_batched<R>(Bt, S, 0, A, n_r, 0, n_r, S, 1, st);
            time_delta /= double(S) / double(n_a);
        } else {
            std::vector<double> z(n_r, 0.0);
            fdc = h->bCols.as<double>(n_r);
            check_cuda(cudaMemcpyAsync(fdc, z.data(), sizeof(double) * n_r, cudaMemcpyHostToDevice, st), "dc0");
        }
        const std::vector<double> az_freqs =
            tops ? linspace(-nrep * g.prf / 2, nrep * g.prf / 2, S) : linspace(-g.prf / 2, g.prf / 2, S);
        const std::vector<RowParam> rp = row_params(g, S, time_delta, az_freqs);
        RowParam* drp = upload(h->bRows, rp);
        double* cols = h->bD.as<double>((size_t)4 * n_r);
        check_cuda(cudaMemcpyAsync(cols, g.slant.data(), sizeof(double) * n_r, cudaMemcpyHostToDevice, st), "cols");
        check_cuda(cudaMemcpyAsync(cols + n_r, g.range_freq.data(), sizeof(double) * n_r, cudaMemcpyHostToDevice, st), "cols");
        check_cuda(cudaMemcpyAsync(cols + 2 * n_r, g.tcorr.data(), sizeof(double) * n_r, cudaMemcpyHostToDevice, st), "cols");
        check_cuda(cudaMemcpyAsync(cols + 3 * n_r, g.rscale.data(), sizeof(double) * n_r, cudaMemcpyHostToDevice, st), "cols");
        const double* slant = cols;
        const double* rf = cols + n_r;
        const double* tcorr = cols + 2 * n_r;
        const double* rscale = cols + 3 * n_r;
        h->mark("row_pass");
        // row pass (s1_decoder.cpp:616-677)
        if (tops) fft_rows(n_r, A, n_r, A, n_r, S, -1);
        src_filter<R>(A, n_r, S, n_r, drp, slant, rf, fdc, std::pow(kCF_, 3.0), st);
        fft_rows(n_r, A, n_r, A, n_r, S, +1);
        az_filter<R>(A, n_r, S, n_r, drp, slant, rf, fdc, tcorr, rscale, tops ? 1 : 0, st);
        h->mark("azimuth_ifft");
        // azimuth IFFT with 1/S (s1_decoder.cpp:682)
        cpx<R>* Bt = h->bB.as<cpx<R>>((size_t)n_r * S);
        transpose_batched<R>(A, n_r, 0, Bt, S, 0, S, n_r, 1, st);
        fft_rows(S, Bt, S, Bt, S, n_r, +1);
        scale_rows<R>(Bt, S, S, n_r, 1.0 / S, st);
        if (!tops) {
            transpose_batched<R>(Bt, S, 0, A, n_r, 0, n_r, S, 1, st);
            Result r;
            r.ptr = A;
            r.rows = S;
            r.cols = n_r;
            r.pitch = n_r;
            r.elem = sizeof(R) == 4 ? S1G_CF32 : S1G_CF64;
            return r;
        }
        h->mark("time_unfold");
        // K_a table and azimuth_time_ufr (image_formation.cpp:222-388)
        double* kaT = h->bKa.as<double>((size_t)n_r * S);
        ka_table(kaT, S, S, n_r, drp, slant, fdc, st);
        TufrParams* dq = (TufrParams*)h->bSmall.get(sizeof(TufrParams));
        tufr_params(kaT, S, S, n_r, fdc, rate, g.T, g.prf, bd, g.swath_number, dq, st);
        TufrParams q;
        check_cuda(cudaMemcpyAsync(&q, dq, sizeof(q), cudaMemcpyDeviceToHost, st), "tufr down");
        check_cuda(cudaStreamSynchronize(st), "tufr sync");
        if (!q.ok) throw S1Error(S1G_E_GEOMETRY, "azimuth time unfolding parameters out of range");
        const int shape = q.shape, down = q.down;
        cpx<R>* C = h->bC.as<cpx<R>>((size_t)n_r * shape);
        cpx<R>* D = h->bD.as<cpx<R>>((size_t)n_r * shape);
        // bD held the column tables; they are no longer needed after the row pass
        tufr_deramp<R>(Bt, S, S, C, shape, kaT, S, fdc, n_r, rate, q.num_tiles, q.focused_time, st);
        fft_rows(shape, C, shape, C, shape, n_r, -1);
        band_select<R>(C, shape, D, shape, shape, q.start, q.end - q.start, n_r, st);
        fft_rows(shape, D, shape, D, shape, n_r, +1);
        scale_rows<R>(D, shape, shape, n_r, 1.0 / shape, st);
        cpx<R>* E = h->bE.as<cpx<R>>((size_t)n_r * down);
        tufr_resample<R>(D, shape, shape, E, down, down, kaT, S, S, fdc, n_r, rate, q.n_ref, q.focused_time, st);
        const int mid = down / 2;
        const int s0 = mid - (q.output_shape / 2);
        const int e0 = mid + (q.output_shape / 2);
        cpx<R>* O = h->bA.as<cpx<R>>((size_t)(e0 - s0) * n_r);
        transpose_batched<R>(E + s0, down, 0, O, n_r, 0, n_r, e0 - s0, 1, st);
        Result r;
        r.ptr = O;
        r.rows = e0 - s0;
        r.cols = n_r;
        r.pitch = n_r;
        r.elem = sizeof(R) == 4 ? S1G_CF32 : S1G_CF64;
        return r;
    }

    Result run(const std::vector<int>& pk, int level, bool tops) {
        if (h->rcmc != S1G_RCMC_PHASE && level == S1G_AZIMUTH_COMPRESSED && tops)
            throw S1Error(S1G_E_UNSUPPORTED, "sinc RCMC: only the FP32 precision (S1G_PREC_FP32) has it");
        const BurstGeom g = make_geom(h->hdr, pk);
        cur_pk = &pk;
        h->mark("decode");
        cpx<R>* A = decode(pk, g);
        h->mark("range_compress");
        Result r;
        r.elem = sizeof(R) == 4 ? S1G_CF32 : S1G_CF64;
        r.rows = g.n_a;
        r.cols = g.n_r;
        r.pitch = g.n_r;
        if (level == S1G_RAW) {
            r.ptr = A;
            return r;
        }
        if (level == S1G_RANGE_COMPRESSED || level == S1G_RANGE_DOPPLER) {
            r.ptr = range_compress(A, g, level == S1G_RANGE_DOPPLER);
            return r;
        }
        A = range_compress(A, g, !tops);
        return azimuth(A, g, tops);
    }
};

}  // namespace s1g

// ------------------------------------------------------------------ differentiable azimuth chain
// Forward model and reverse-mode adjoint of the range-Doppler azimuth chain
// of one burst (kernels and the model in s1g_adjoint.cu).  The
// range-compressed burst is recomputed from the byte stream on every call
// rather than kept.  Geometry in FP64 on the host: effective velocity at
// the burst centre and mid-swath range (the expression of
// get_effective_velocities, image_formation.cpp:391-419), wavelength,
// slant ranges of the range bins.
namespace s1g {

struct ChainResult {
    double loss = 0.0;
    std::vector<double> g_theta;
    double g_fc = 0.0;
    const void* image = nullptr;   // focused image [n_a][n_r] (when kept)
    long long rows = 0, cols = 0;
};

template <typename R>
static ChainResult azimuth_chain(s1g_decoder* h, const std::vector<int>& pk, const double* theta, int nt, double fc,
                                 bool grads, bool keep_image) {
    Pipe<R> p(h);
    cudaStream_t st = h->stream;
    const BurstGeom g = make_geom(h->hdr, pk);
    const int n_a = g.n_a, n_r = g.n_r;
    if (n_a < 2 || n_r < 2) throw S1Error(S1G_E_GEOMETRY, "burst too small for the azimuth chain");
    if (h->sv.t.empty()) throw S1Error(S1G_E_GEOMETRY, "no state vectors in the data");
    const long long N = (long long)n_a * n_r;
    p.cur_pk = &pk;
    const cpx<R>* X = p.range_compress(p.decode(pk, g), g, false);
    // geometry
    const double kPi = 3.141592653589793238463;
    double pos[3], vel[3];
    h->sv.interpolate(g.t0 + 0.5 * g.T, pos, vel);
    const double vn = std::sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    const double r_ref = g.slant[n_r / 2];
    double v_eff;
    {
        const double lat = pos[2] / pos[0];
        const double a = 6378137.0, b = 6356752.3142;
        const double num = std::pow(a * a * std::cos(lat), 2.0) + std::pow(b * b * std::sin(lat), 2.0);
        const double den = std::pow(a * std::cos(lat), 2.0) + std::pow(b * std::sin(lat), 2.0);
        const double re = std::sqrt(num / den);
        const double hh = std::sqrt(pos[0] * pos[0] + pos[1] * pos[1] + pos[2] * pos[2]);
        const double beta_g = (re * re + hh * hh - r_ref * r_ref) / (2 * re * hh);
        v_eff = std::sqrt(vn * (re * vn * beta_g / hh));
    }
    const double lam = kC_ / kCF_;
    const double c4pl = 4.0 * kPi / lam;
    std::vector<double> f(n_a), D(n_a), hostd((size_t)3 * n_a + n_r + 3 * n_a + 2, 0.0);
    double* beta = hostd.data();
    double* omd = beta + n_a;
    double* slant = omd + n_a;
    for (int k = 0; k < n_a; ++k) {
        const double nu = (double)(k < (n_a + 1) / 2 ? k : k - n_a) * g.prf / n_a;
        f[k] = nu + fc;
        const double x = lam * lam * f[k] * f[k] / (4.0 * v_eff * v_eff);
        if (!(x < 1.0)) throw S1Error(S1G_E_GEOMETRY, "azimuth frequency beyond the velocity limit");
        D[k] = std::sqrt(1.0 - x);
        omd[k] = x / (1.0 + D[k]);
        beta[k] = 4.0 * kPi * r_ref * (omd[k] / D[k]) / kC_;
    }
    for (int r = 0; r < n_r; ++r) slant[r] = g.slant[r];
    std::vector<double> xa(n_a);
    std::vector<cpx<R>> e(n_a);
    for (int a = 0; a < n_a; ++a) {
        xa[a] = -1.0 + 2.0 * a / (double)(n_a - 1);
        double ph = 0.0, xp = xa[a] * xa[a];
        for (int j = 0; j < nt; ++j, xp *= xa[a]) ph += theta[j] * xp;
        e[a] = mk((R)std::cos(-ph), (R)std::sin(-ph));
    }
    double* dd = (double*)h->bJd.get(sizeof(double) * hostd.size());
    check_cuda(cudaMemcpyAsync(dd, hostd.data(), sizeof(double) * (3 * n_a + n_r), cudaMemcpyHostToDevice, st),
               "chain geometry");
    const double* d_beta = dd;
    const double* d_omd = dd + n_a;
    const double* d_slant = dd + 2 * n_a;
    double* d_ak = dd + 2 * n_a + n_r;
    double* d_bk = d_ak + n_a;
    double* d_dphi = d_bk + n_a;
    double* d_sums = d_dphi + n_a;
    cpx<R>* d_e = p.upload(h->bJe, e);
    cpx<R>* U = h->bJ0.as<cpx<R>>((size_t)N);
    cpx<R>* T1 = h->bJ1.as<cpx<R>>((size_t)N);
    cpx<R>* QM = h->bJ2.as<cpx<R>>((size_t)N);
    cpx<R>* Z = h->bJ3.as<cpx<R>>((size_t)N);
    cpx<R>* T2 = h->bJ4.as<cpx<R>>((size_t)N);
    // forward
    check_cuda(cudaMemcpyAsync(U, X, sizeof(cpx<R>) * N, cudaMemcpyDeviceToDevice, st), "chain copy");
    row_factor<R>(U, n_r, n_r, n_a, d_e, st);
    transpose_batched<R>(U, n_r, 0, T1, n_a, 0, n_a, n_r, 1, st);
    p.fft_rows(n_a, T1, n_a, T1, n_a, n_r, -1);
    transpose_batched<R>(T1, n_a, 0, QM, n_r, 0, n_r, n_a, 1, st);
    p.fft_rows(n_r, QM, n_r, QM, n_r, n_a, -1);
    rcmc_phase<R>(QM, n_r, n_a, d_beta, g.fs, +1, st);
    p.fft_rows(n_r, QM, n_r, Z, n_r, n_a, +1);
    scale_rows<R>(Z, n_r, n_r, n_a, 1.0 / n_r, st);
    az_filter<R>(Z, n_r, n_a, d_omd, d_slant, c4pl, -1, st);
    transpose_batched<R>(Z, n_r, 0, T2, n_a, 0, n_a, n_r, 1, st);
    p.fft_rows(n_a, T2, n_a, T2, n_a, n_r, +1);
    scale_rows<R>(T2, n_a, n_a, n_r, 1.0 / n_a, st);
    entropy_sums<R>(T2, N, d_sums, st);
    double sums[2];
    check_cuda(cudaMemcpyAsync(sums, d_sums, sizeof(sums), cudaMemcpyDeviceToHost, st), "entropy down");
    check_cuda(cudaStreamSynchronize(st), "chain sync");
    ChainResult res;
    res.rows = n_a;
    res.cols = n_r;
    if (!(sums[0] > 0.0)) throw S1Error(S1G_E_GEOMETRY, "the focused burst is zero");
    res.loss = -(sums[1] / sums[0] - std::log(sums[0]));
    if (keep_image) {
        transpose_batched<R>(T2, n_a, 0, T1, n_r, 0, n_r, n_a, 1, st);
        res.image = T1;
    }
    if (!grads) return res;
    // adjoint
    entropy_grad<R>(T2, T2, N, d_sums, st);
    p.fft_rows(n_a, T2, n_a, T2, n_a, n_r, -1);
    scale_rows<R>(T2, n_a, n_a, n_r, 1.0 / n_a, st);
    transpose_batched<R>(T2, n_a, 0, T1, n_r, 0, n_r, n_a, 1, st);   // G_Z
    row_imdot<R>(T1, Z, n_r, n_a, d_slant, 0.0, d_ak, st);
    az_filter<R>(T1, n_r, n_a, d_omd, d_slant, c4pl, +1, st);         // G_W
    p.fft_rows(n_r, T1, n_r, T1, n_r, n_a, -1);                       // F
    row_imdot<R>(T1, QM, n_r, n_a, nullptr, g.fs, d_bk, st);
    rcmc_phase<R>(T1, n_r, n_a, d_beta, g.fs, -1, st);
    p.fft_rows(n_r, T1, n_r, T1, n_r, n_a, +1);
    scale_rows<R>(T1, n_r, n_r, n_a, 1.0 / n_r, st);                  // G_V
    transpose_batched<R>(T1, n_r, 0, T2, n_a, 0, n_a, n_r, 1, st);
    p.fft_rows(n_a, T2, n_a, T2, n_a, n_r, +1);                       // n_a IFFT_az
    transpose_batched<R>(T2, n_a, 0, T1, n_r, 0, n_r, n_a, 1, st);   // G_U
    row_imdot<R>(T1, U, n_r, n_a, nullptr, 0.0, d_dphi, st);
    std::vector<double> red((size_t)3 * n_a);
    check_cuda(cudaMemcpyAsync(red.data(), d_ak, sizeof(double) * red.size(), cudaMemcpyDeviceToHost, st),
               "chain gradient down");
    check_cuda(cudaStreamSynchronize(st), "chain gradient sync");
    const double* ak = red.data();
    const double* bk = ak + n_a;
    const double* dphi = bk + n_a;
    res.g_theta.assign(nt, 0.0);
    for (int a = 0; a < n_a; ++a) {
        double xp = xa[a] * xa[a];
        for (int j = 0; j < nt; ++j, xp *= xa[a]) res.g_theta[j] += dphi[a] * xp;
    }
    double gf = 0.0;
    for (int k = 0; k < n_a; ++k) {
        const double dLdD = -c4pl * ak[k] + (-bk[k] / n_r) * (-4.0 * kPi * r_ref / (kC_ * D[k] * D[k]));
        gf += dLdD * (-lam * lam * f[k] / (4.0 * v_eff * v_eff * D[k]));
    }
    res.g_fc = gf;
    return res;
}

// The TOPS azimuth chain of one IW burst up to the focused image before the
// time-domain unfolding (s1_decoder.cpp:511-682 without azimuth_time_ufr,
// which regrids the focused burst and does not change its focus), with a
// phase-error polynomial on the range-compressed lines and an offset added
// to the estimated Doppler centroid, the image entropy, and its gradient by
// a hand-written reverse-mode adjoint:
//   U = X exp(-i phi_a)                         phase-error polynomial
//   V = azimuth_frequency_ufr(U)                image_formation.cpp:125-219
//   A1 = SRC(FFT_r V)                           image_formation.cpp:422-455
//   Z = post(IFFT_r A1)                         scale, RCMC, azimuth filter (s1_decoder.cpp:643-676)
//   Y = IFFT_az(Z) / S,  L = -sum p ln p
// The frequency unfolding, the transforms and the SRC / post factors are the
// FP64 (or plain FP32) pipeline's own kernels; each adjoint is the opposite
// transform or the conjugate factor, the band move's adjoint re-inserts the
// band and the tiling's folds the replicas back.  The centroid offset enters
// every factor through F = f_a + f_dc + offset.
template <typename R>
static ChainResult tops_chain(s1g_decoder* h, const std::vector<int>& pk, const double* theta, int nt, double offset,
                              bool grads, bool keep_image) {
    Pipe<R> p(h);
    cudaStream_t st = h->stream;
    const BurstGeom g = make_geom(h->hdr, pk);
    const int n_a = g.n_a, n_r = g.n_r;
    if (n_a < 2 || n_r < 2) throw S1Error(S1G_E_GEOMETRY, "burst too small for the azimuth chain");
    if (h->sv.t.empty()) throw S1Error(S1G_E_GEOMETRY, "no state vectors in the data");
    p.cur_pk = &pk;
    cpx<R>* X = p.range_compress(p.decode(pk, g), g, false);
    const double rate = p.dc_rate(g);
    std::vector<double> fdc(n_r);
    check_cuda(cudaMemcpyAsync(fdc.data(), p.doppler(X, g, rate), sizeof(double) * n_r, cudaMemcpyDeviceToHost, st),
               "centroid down");
    check_cuda(cudaStreamSynchronize(st), "centroid sync");
    for (double& f : fdc) f += offset;
    // frequency-unfolding geometry (Pipe::azimuth)
    const double bd = g.swath_number == 11 ? 675 : 600;
    const double nrep = std::abs(rate * g.T / g.prf);
    const int S = (int)std::floor(nrep * n_a);
    if (S < 4) throw S1Error(S1G_E_GEOMETRY, "azimuth frequency unfolding needs a beam sweep (no Doppler rate)");
    const int mid = S / 2;
    const int start = (int)(mid - (std::floor(bd) / 2));
    const int end = (int)(mid + (std::floor(bd) / 2));
    const int offset_rep = (int)std::floor(nrep);
    int tile_len = offset_rep * n_a;
    if (std::floor(nrep) != nrep) tile_len += (int)std::floor((nrep - std::floor(nrep)) * n_a);
    tile_len = std::min(tile_len, S);
    const std::vector<double> f = linspace(-nrep * g.prf / 2.0, nrep * g.prf / 2.0, S);
    std::vector<cpx<R>> der(S), rer(S), rer_c(S);
    for (int k = 0; k < S; ++k) {
        const double th = -kPI_ * (1 / rate) * std::pow(f[k], 2.0);
        const double th2 = kPI_ * (1 / rate) * std::pow(f[k], 2.0);
        der[k] = mk((R)std::cos(th), (R)std::sin(th));
        rer[k] = mk((R)std::cos(th2), (R)std::sin(th2));
        rer_c[k] = mk((R)std::cos(th2), (R)(-std::sin(th2)));
    }
    const double time_delta = g.T / g.prf / (double(S) / double(n_a));
    const std::vector<RowParam> rp = p.row_params(g, S, time_delta, f);
    // device tables: [der | rer | conj rer] complex, then the per-range-bin
    // columns and the reductions in FP64
    std::vector<cpx<R>> vecs;
    vecs.reserve((size_t)3 * S + n_a);
    vecs.insert(vecs.end(), der.begin(), der.end());
    vecs.insert(vecs.end(), rer.begin(), rer.end());
    vecs.insert(vecs.end(), rer_c.begin(), rer_c.end());
    std::vector<double> xa(n_a);
    for (int a = 0; a < n_a; ++a) {
        xa[a] = -1.0 + 2.0 * a / (double)(n_a - 1);
        double ph = 0.0, xp = xa[a] * xa[a];
        for (int j = 0; j < nt; ++j, xp *= xa[a]) ph += theta[j] * xp;
        vecs.push_back(mk((R)std::cos(-ph), (R)std::sin(-ph)));
    }
    cpx<R>* dv = p.upload(h->bJe, vecs);
    const cpx<R>* d_der = dv;
    const cpx<R>* d_rer = dv + S;
    const cpx<R>* d_rerc = dv + 2 * S;
    const cpx<R>* d_e = dv + 3 * S;
    std::vector<double> cols((size_t)5 * n_r + 2 * S + n_a + 2, 0.0);
    for (int j = 0; j < n_r; ++j) {
        cols[j] = g.slant[j];
        cols[n_r + j] = g.range_freq[j];
        cols[2 * n_r + j] = fdc[j];
        cols[3 * n_r + j] = g.tcorr[j];
        cols[4 * n_r + j] = g.rscale[j];
    }
    double* dd = (double*)h->bJd.get(sizeof(double) * cols.size());
    check_cuda(cudaMemcpyAsync(dd, cols.data(), sizeof(double) * 5 * n_r, cudaMemcpyHostToDevice, st), "tops columns");
    TopsCols tc{dd, dd + n_r, dd + 2 * n_r, dd + 3 * n_r, dd + 4 * n_r};
    double* d_dz = dd + 5 * n_r;      // per azimuth row: centroid derivative through the post factor
    double* d_ds = d_dz + S;          // ... through SRC
    double* d_dphi = d_ds + S;        // per line: d L / d phi_a
    double* d_sums = d_dphi + n_a;    // entropy sums
    RowParam* drp = p.upload(h->bRows, rp);
    const long long NA = (long long)n_a * n_r, NS = (long long)S * n_r;
    const int wmax = std::max(n_a, S);
    cpx<R>* U = h->bJ0.as<cpx<R>>((size_t)NA);
    cpx<R>* T = h->bJ1.as<cpx<R>>((size_t)n_r * wmax);
    cpx<R>* C = h->bJ2.as<cpx<R>>((size_t)std::max(NS, NA));
    cpx<R>* A = h->bJ3.as<cpx<R>>((size_t)NS);
    cpx<R>* A1 = h->bJ4.as<cpx<R>>((size_t)NS);
    cpx<R>* YT = h->bJ5.as<cpx<R>>((size_t)NS);
    // forward
    check_cuda(cudaMemcpyAsync(U, X, sizeof(cpx<R>) * NA, cudaMemcpyDeviceToDevice, st), "chain copy");
    row_factor<R>(U, n_r, n_r, n_a, d_e, st);
    transpose_batched<R>(U, n_r, 0, T, n_a, 0, n_a, n_r, 1, st);
    p.fft_rows(n_a, T, n_a, T, n_a, n_r, -1);
    fufr_prep<R>(T, n_a, n_a, C, S, S, tile_len, d_der, n_r, st);
    p.fft_rows(S, C, S, C, S, n_r, -1);
    band_select<R>(C, S, T, S, S, start, end - start, n_r, st);
    p.fft_rows(S, T, S, T, S, n_r, +1);
    scale_mul_vec<R>(T, S, S, n_r, d_rer, 1.0 / S, st);
    transpose_batched<R>(T, S, 0, A, n_r, 0, n_r, S, 1, st);
    p.fft_rows(n_r, A, n_r, A, n_r, S, -1);
    src_filter<R>(A, n_r, S, n_r, drp, tc.slant, tc.rf, tc.fdc, std::pow(kCF_, 3.0), st);
    check_cuda(cudaMemcpyAsync(A1, A, sizeof(cpx<R>) * NS, cudaMemcpyDeviceToDevice, st), "chain keep");
    p.fft_rows(n_r, A, n_r, A, n_r, S, +1);
    az_filter<R>(A, n_r, S, n_r, drp, tc.slant, tc.rf, tc.fdc, tc.tcorr, tc.rscale, 1, st);
    transpose_batched<R>(A, n_r, 0, YT, S, 0, S, n_r, 1, st);
    p.fft_rows(S, YT, S, YT, S, n_r, +1);
    scale_rows<R>(YT, S, S, n_r, 1.0 / S, st);
    entropy_sums<R>(YT, NS, d_sums, st);
    double sums[2];
    check_cuda(cudaMemcpyAsync(sums, d_sums, sizeof(sums), cudaMemcpyDeviceToHost, st), "entropy down");
    check_cuda(cudaStreamSynchronize(st), "chain sync");
    ChainResult res;
    res.rows = S;
    res.cols = n_r;
    if (!(sums[0] > 0.0)) throw S1Error(S1G_E_GEOMETRY, "the focused burst is zero");
    res.loss = -(sums[1] / sums[0] - std::log(sums[0]));
    if (keep_image) {
        transpose_batched<R>(YT, S, 0, T, n_r, 0, n_r, S, 1, st);
        res.image = T;
    }
    if (!grads) return res;
    // adjoint
    entropy_grad<R>(YT, T, NS, d_sums, st);
    p.fft_rows(S, T, S, T, S, n_r, -1);
    scale_rows<R>(T, S, S, n_r, 1.0 / S, st);                        // G_Z^T
    transpose_batched<R>(T, S, 0, C, n_r, 0, n_r, S, 1, st);         // G_Z
    tops_dpsi<R>(C, A, n_r, S, n_r, drp, tc, 1, d_dz, st);
    tops_factor_adj<R>(C, n_r, S, n_r, drp, tc, 1, st);
    p.fft_rows(n_r, C, n_r, C, n_r, S, -1);                           // G_A1
    tops_dpsi<R>(C, A1, n_r, S, n_r, drp, tc, 0, d_ds, st);
    tops_factor_adj<R>(C, n_r, S, n_r, drp, tc, 0, st);
    p.fft_rows(n_r, C, n_r, C, n_r, S, +1);                           // G_V
    transpose_batched<R>(C, n_r, 0, T, S, 0, S, n_r, 1, st);
    scale_mul_vec<R>(T, S, S, n_r, d_rerc, 1.0 / S, st);
    p.fft_rows(S, T, S, T, S, n_r, -1);                               // band gradient
    band_insert<R>(T, S, YT, S, S, start, end - start, n_r, st);
    p.fft_rows(S, YT, S, YT, S, n_r, +1);                             // tiled-line gradient
    ufr_fold<R>(YT, S, tile_len, d_der, T, n_a, n_a, n_r, st);
    p.fft_rows(n_a, T, n_a, T, n_a, n_r, +1);                         // G_U^T
    transpose_batched<R>(T, n_a, 0, C, n_r, 0, n_r, n_a, 1, st);     // G_U
    row_imdot<R>(C, U, n_r, n_a, nullptr, 0.0, d_dphi, st);
    std::vector<double> red((size_t)2 * S + n_a);
    check_cuda(cudaMemcpyAsync(red.data(), d_dz, sizeof(double) * red.size(), cudaMemcpyDeviceToHost, st),
               "chain gradient down");
    check_cuda(cudaStreamSynchronize(st), "chain gradient sync");
    double go = 0.0;
    for (int i = 0; i < 2 * S; ++i) go += red[i];
    res.g_fc = go;
    const double* dphi = red.data() + 2 * S;
    res.g_theta.assign(nt, 0.0);
    for (int a = 0; a < n_a; ++a) {
        double xp = xa[a] * xa[a];
        for (int j = 0; j < nt; ++j, xp *= xa[a]) res.g_theta[j] += dphi[a] * xp;
    }
    return res;
}

}  // namespace s1g

// ------------------------------------------------------------------ fast FP32 path
struct CztTables {
    s1g::CztDev dev;
    std::vector<void*> owned;
    ~CztTables() {
        for (void* p : owned) cudaFree(p);
    }
};

struct FastBurst {          // per-burst tables of the fast path
    s1g::BurstGeom g;
    int M = 0;
    s1g::Fft3Desc dM;
    s1g::cf32* ref = nullptr;
    // TOPS azimuth
    double rate = 0, nrep = 0, time_delta = 0;
    int S = 0, start = 0, bw = 0, tile_len = 0;
    s1g::cf32 *dfwd = nullptr, *reramp = nullptr;
    // Doppler estimator: overlap-save block, its compensated FFT and filter,
    // and the lag-1 deramp products
    int dcB = 0, dcU = 0, dcNb = 0;
    s1g::CfftDesc dcDesc;
    float4 *dcH = nullptr, *dcG = nullptr;
    int na_smooth = 0, nr_smooth = 0;
    s1g::Fft3Desc dna, dnr;
    s1g::CztDev cna, cnr, cf, ci, cS;
    s1g::RowDf* rows_df = nullptr;
    s1g::RowParam* rows64 = nullptr;
    s1g::ColDf* cols = nullptr;
    s1g::df* inv_lamR = nullptr;
    double* slant = nullptr;
    s1g::df* zero_df = nullptr;
    // time-unfolding launch plan (bounds valid for any Doppler centroid; the
    // kernel reads the actual tile count and band from the device)
    int t_hi = 0, bw_max = 0, n_out = 0, s0 = 0;
    int m_nu = 0;                       // grid length of the band evaluation
    double *gl_x = nullptr, *gl_w = nullptr;   // Gauss-Legendre nodes (kNuQuad)
    std::vector<void*> owned;
    ~FastBurst() {
        for (void* p : owned) cudaFree(p);
    }
    template <typename T>
    T* up(const std::vector<T>& v, cudaStream_t st) {
        void* d = nullptr;
        s1g::check_cuda(cudaMalloc(&d, sizeof(T) * std::max<size_t>(v.size(), 1)), "fast table");
        owned.push_back(d);
        s1g::check_cuda(cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st), "fast up");
        s1g::check_cuda(cudaStreamSynchronize(st), "fast up sync");
        return (T*)d;
    }
};

namespace s1g {

static const double kPIref_ = 3.14159265358979;

// exp(sign i pi n^2 / P) with n^2 reduced modulo 2P first (exact)
static inline cpx<double> chirp_at(long long n, long long P, int sign) {
    const long long n2 = (n % (2 * P)) * (n % (2 * P)) % (2 * P);
    const double a = M_PI * (double)n2 / (double)P;
    return mk(std::cos(a), sign * std::sin(a));
}

// Longest transform a fused kernel holds: padded buffer plus twiddle tables
// within the shared-memory budget.
static int fused_cap() { return smem_capacity<float>() * 31 / 32 - 512; }

// Chirp-z tables for X[k] = sum_{s<nin} x[s] exp(-2 pi i s k / P), k < nout.
static CztDev get_czt(s1g_decoder* h, int P, int nin, int nout) {
    auto key = std::make_tuple(P, nin, nout);
    auto it = h->czts.find(key);
    if (it != h->czts.end()) return it->second->dev;
    auto t = std::make_shared<CztTables>();
    const int m = (int)h->fft->tuned_len((long long)nin + nout - 1, fused_cap());
    if (m > fused_cap()) throw S1Error(S1G_E_GEOMETRY, "chirp-z length " + std::to_string(m) + " too long");
    t->dev.dm = h->fft->desc3(m);
    t->dev.nin = nin;
    t->dev.nout = nout;
    const int nw = std::max(nin, nout);
    std::vector<cf32> w(nw);
    for (int k = 0; k < nw; ++k) {
        const cpx<double> c = chirp_at(k, P, -1);
        w[k] = mk((float)c.x, (float)c.y);
    }
    std::vector<cpx<double>> b((size_t)m, mk(0.0, 0.0));
    for (int q = 0; q < m; ++q) {
        const long long n = q < nout ? q : (long long)q - m;
        if (n > -(long long)nin) b[q] = chirp_at(n < 0 ? -n : n, P, +1);
    }
    void *dw = nullptr, *db = nullptr, *dk = nullptr;
    check_cuda(cudaMalloc(&dw, sizeof(cf32) * nw), "czt chirp");
    check_cuda(cudaMalloc(&db, sizeof(cpx<double>) * m), "czt tmp");
    check_cuda(cudaMalloc(&dk, sizeof(cf32) * m), "czt kern");
    t->owned = {dw, dk};
    check_cuda(cudaMemcpy(dw, w.data(), sizeof(cf32) * nw, cudaMemcpyHostToDevice), "czt up");
    check_cuda(cudaMemcpy(db, b.data(), sizeof(cpx<double>) * m, cudaMemcpyHostToDevice), "czt up");
    auto p64 = h->fft->plan<double>(m);
    h->fft->rows<double>(*p64, (cpx<double>*)db, m, (cpx<double>*)db, m, 1, -1);
    check_cuda(cudaStreamSynchronize(h->stream), "czt fft");
    std::vector<cpx<double>> B(m);
    check_cuda(cudaMemcpy(B.data(), db, sizeof(cpx<double>) * m, cudaMemcpyDeviceToHost), "czt down");
    cudaFree(db);
    std::vector<cf32> K(m);
    for (int q = 0; q < m; ++q) K[q] = mk((float)(B[q].x / m), (float)(B[q].y / m));
    check_cuda(cudaMemcpy(dk, K.data(), sizeof(cf32) * m, cudaMemcpyHostToDevice), "czt up");
    t->dev.chirp = (const cf32*)dw;
    t->dev.kern = (const cf32*)dk;
    h->czts[key] = t;
    return t->dev;
}

struct FastPipe {
    s1g_decoder* h;
    cudaStream_t st;
    FftEngine& fft;
    const cf32* predecoded = nullptr;   // burst already decoded (batched decode)
    cf64* predecoded64 = nullptr;       // ... and its FP64 samples (for the ECCM notch), or null
    cf32* final_out = nullptr;          // write the SLC here ([N_out][N_r]) instead of a work buffer
    int* tufr_status = nullptr;         // per-burst time-unfolding status slot
    explicit FastPipe(s1g_decoder* hh) : h(hh), st(hh->stream), fft(*hh->fft) {}

    // Bounds of the time-unfolding tile count, band and output crop from host
    // quantities (image_formation.cpp:222-288).  Only n_ref = f_dc[mid] /
    // K_a[mid][mid] and, through K_a, the focused time depend on the device
    // centroid: num_tiles = ceil(x + a) - floor(x - a) with a = focused/(2T)
    // lies in {ceil(2a), ceil(2a) + 1} for any x, and a moves by far less
    // than the 1e-3 margin used here.
    void plan_tufr(FastBurst& fb, const std::vector<RowParam>& rp, double bd) {
        const BurstGeom& g = fb.g;
        const double wl = kC_ / kCF_;
        const double R0 = g.slant[0];
        double acc = 0.0;
        for (int i = 0; i < fb.S; ++i) {
            const RowParam& r = rp[i];
            const double num = r.re * r.re + r.h * r.h - R0 * R0;
            const double beta = num / (2 * r.re * r.h);
            const double vg = r.re * r.v * beta / r.h;
            const double v = std::sqrt(r.v * vg);
            const double fa = r.fa;
            const double D = std::sqrt(1 - ((wl * wl) * (fa * fa)) / (4 * v * v));
            acc += (-2 * (v * v) * (D * D * D)) / (wl * R0);
        }
        const double ka_mean = std::fabs(acc) / fb.S;
        const double bandwidth = fb.nrep * g.prf - bd;
        double ft = g.T + ((bandwidth - 2 * bd) / ka_mean);
        ft *= (g.swath_number != 11) ? 0.9 : 1.05;
        const double a2 = ft / g.T;
        fb.t_hi = (int)std::ceil(a2 * (1 + 1e-3)) + 1;
        fb.bw_max = (int)std::floor(bandwidth) + 2;
        const int ext = g.swath_number == 11 ? (int)std::floor(bd * 1.15) : (int)std::floor(bd * 0.26);
        const int output_shape = (int)std::floor(g.prf * g.T);
        const int down = output_shape + ext;
        const int mid = down / 2;
        fb.s0 = mid - output_shape / 2;
        fb.n_out = (mid + output_shape / 2) - fb.s0;
        fb.m_nu = (int)h->fft->tuned_len((5LL * fb.bw_max + 3) / 4, fused_cap());
    }

    // Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on the
    // Legendre recurrence), for the Fourier transform of the band-evaluation kernel.
    static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
        x.assign(n, 0.0);
        w.assign(n, 0.0);
        for (int i = 0; i < (n + 1) / 2; ++i) {
            double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
            for (int it = 0; it < 100; ++it) {
                double p0 = 1.0, p1 = 0.0;
                for (int k = 1; k <= n; ++k) {
                    const double p2 = p1;
                    p1 = p0;
                    p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
                }
                dp = n * (z * p0 - p1) / (z * z - 1.0);
                const double dz = p0 / dp;
                z -= dz;
                if (std::fabs(dz) < 1e-16) break;
            }
            x[i] = -z;
            x[n - 1 - i] = z;
            w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
        }
    }

    std::shared_ptr<FastBurst> prepare(const std::vector<int>& pk, bool tops) {
        const int key = pk.front() * 2 + (tops ? 1 : 0);
        auto it = h->fast_bursts.find(key);
        if (it != h->fast_bursts.end()) return it->second;
        auto fb = std::make_shared<FastBurst>();
        fb->g = make_geom(h->hdr, pk);
        const BurstGeom& g = fb->g;
        // range compression: correlation length M and reference spectrum
        fb->M = (int)fft.tuned_len((long long)g.n_r + g.L, fused_cap());
        if (fb->M > fused_cap()) throw S1Error(S1G_E_GEOMETRY, "range line too long for the fused kernel");
        fb->dM = fft.desc3(fb->M);
        {
            Pipe<float> plain(h);
            const int M = fb->M;
            std::vector<cpx<double>> c((size_t)M, mk(0.0, 0.0));
            for (int t = 0; t < g.L; ++t) c[t] = g.chirp[t];
            cf64* dc = (cf64*)h->bTab.get(sizeof(cf64) * M);
            check_cuda(cudaMemcpyAsync(dc, c.data(), sizeof(cf64) * M, cudaMemcpyHostToDevice, st), "chirp up");
            auto p64 = fft.plan<double>(M);
            fft.rows<double>(*p64, dc, M, dc, M, 1, -1);
            std::vector<cpx<double>> spec(M);
            check_cuda(cudaMemcpyAsync(spec.data(), dc, sizeof(cf64) * M, cudaMemcpyDeviceToHost, st), "chirp down");
            check_cuda(cudaStreamSynchronize(st), "ref sync");
            std::vector<cf32> ref(M);
            const double s = 1.0 / (g.energy * (double)M);
            for (int k = 0; k < M; ++k) ref[k] = mk((float)(spec[k].x * s), (float)(-spec[k].y * s));
            fb->ref = fb->up(ref, st);
        }
        const int n_a = g.n_a, n_r = g.n_r;
        const double bd = g.swath_number == 11 ? 675 : 600;
        double time_delta = g.T / g.prf;
        int S = n_a;
        std::vector<double> az_freqs;
        if (tops) {
            Pipe<float> plain(h);
            fb->rate = plain.dc_rate(g);
            const double rate = fb->rate;
            fb->nrep = std::abs(rate * g.T / g.prf);
            const double bwh = fb->nrep * g.prf / 2.0;
            S = (int)std::floor(fb->nrep * n_a);
            if (S < 4) throw S1Error(S1G_E_GEOMETRY, "azimuth frequency unfolding needs a beam sweep (no Doppler rate)");
            const int mid = S / 2;
            fb->start = (int)(mid - (std::floor(bd) / 2));
            const int end = (int)(mid + (std::floor(bd) / 2));
            fb->bw = end - fb->start;
            const int offset = (int)std::floor(fb->nrep);
            int tl = offset * n_a;
            if (std::floor(fb->nrep) != fb->nrep) tl += (int)std::floor((fb->nrep - std::floor(fb->nrep)) * n_a);
            fb->tile_len = std::min(tl, S);
            // Doppler-estimate deramp (doppler.cpp:98-116, duration fixed at 1.06 s)
            // as the lag-1 products g_t = d_t conj(d_t+1), float pairs
            const std::vector<double> t = linspace(0.0, 1.06, n_a);
            std::vector<float4> gt(std::max(n_a - 1, 1));
            for (int a = 0; a + 1 < n_a; ++a) {
                const double th0 = kPIref_ * rate * std::pow(t[a] - (0.5 * 1.06), 2.0);
                const double th1 = kPIref_ * rate * std::pow(t[a + 1] - (0.5 * 1.06), 2.0);
                const double c0 = std::cos(th0), s0 = std::sin(th0), c1 = std::cos(th1), s1 = std::sin(th1);
                const df gr = df_from(c0 * c1 + s0 * s1), gi = df_from(s0 * c1 - c0 * s1);
                gt[a] = make_float4(gr.hi, gi.hi, gr.lo, gi.lo);
            }
            fb->dcG = fb->up(gt, st);
            // compensated overlap-save range compression for the lag-1 sums
            if (!choose_dc_block(n_r, g.L, fb->dcB, fb->dcU, fb->dcNb))
                throw S1Error(S1G_E_GEOMETRY, "chirp too long for the Doppler estimator");
            auto& cp = h->cffts[fb->dcB];
            if (!cp) cp = make_cfft_plan(fb->dcB);
            fb->dcDesc = cp->d;
            {
                const int B = fb->dcB;
                std::vector<cpx<double>> c((size_t)B, mk(0.0, 0.0));
                for (int k = 0; k < g.L; ++k) c[k] = g.chirp[k];
                cf64* dc = (cf64*)h->bTab.get(sizeof(cf64) * B);
                check_cuda(cudaMemcpyAsync(dc, c.data(), sizeof(cf64) * B, cudaMemcpyHostToDevice, st), "dc chirp up");
                auto pB = fft.plan<double>(B);
                fft.rows<double>(*pB, dc, B, dc, B, 1, -1);
                std::vector<cpx<double>> spec(B);
                check_cuda(cudaMemcpyAsync(spec.data(), dc, sizeof(cf64) * B, cudaMemcpyDeviceToHost, st), "dc down");
                check_cuda(cudaStreamSynchronize(st), "dc sync");
                const double sc = std::ldexp(1.0, -32) / (g.energy * (double)B);
                std::vector<float4> Hb(B);
                for (int k = 0; k < B; ++k) {
                    const df re = df_from(spec[k].x * sc), im = df_from(-spec[k].y * sc);
                    Hb[k] = make_float4(re.hi, im.hi, re.lo, im.lo);
                }
                fb->dcH = fb->up(Hb, st);
            }
            // unfolding deramp (with the band offset folded in) and re-ramp / S
            const std::vector<double> f = linspace(-bwh, bwh, S);
            std::vector<cf32> dfwd(S), rer(S);
            for (int k = 0; k < S; ++k) {
                const double th = -kPIref_ * (1 / rate) * std::pow(f[k], 2.0);
                const long long idx = ((long long)k * fb->start) % S;
                const double th2 = th - 2.0 * M_PI * (double)idx / (double)S;
                dfwd[k] = mk((float)std::cos(th2), (float)std::sin(th2));
                const double th3 = kPIref_ * (1 / rate) * std::pow(f[k], 2.0);
                rer[k] = mk((float)(std::cos(th3) / S), (float)(std::sin(th3) / S));
            }
            fb->dfwd = fb->up(dfwd, st);
            fb->reramp = fb->up(rer, st);
            fb->na_smooth = is_smooth7(n_a) && n_a <= fused_cap();
            if (fb->na_smooth) fb->dna = fft.desc3(n_a);
            else fb->cna = get_czt(h, n_a, n_a, n_a);
            fb->cf = get_czt(h, S, S, fb->bw);
            fb->ci = get_czt(h, S, fb->bw, S);
            fb->cS = get_czt(h, S, S, S);
            time_delta /= double(S) / double(n_a);
            az_freqs = linspace(-fb->nrep * g.prf / 2, fb->nrep * g.prf / 2, S);
        } else {
            az_freqs = linspace(-g.prf / 2, g.prf / 2, S);
        }
        fb->S = S;
        fb->time_delta = time_delta;
        // per-row and per-range-bin constants (FP64 on the host, stored as float pairs)
        Pipe<float> plain(h);
        const std::vector<RowParam> rp = plain.row_params(g, S, time_delta, az_freqs);
        std::vector<RowDf> rdf(S);
        for (int i = 0; i < S; ++i) {
            rdf[i].fa = df_from(rp[i].fa);
            rdf[i].P = df_from(rp[i].v * rp[i].v / (2.0 * rp[i].h * rp[i].h));
            rdf[i].A = df_from(rp[i].re * rp[i].re + rp[i].h * rp[i].h);
        }
        fb->rows_df = fb->up(rdf, st);
        fb->rows64 = fb->up(rp, st);
        if (tops) {
            plan_tufr(*fb, rp, g.swath_number == 11 ? 675 : 600);
            std::vector<double> gx, gw;
            gauss_legendre(kNuQuad, gx, gw);
            fb->gl_x = fb->up(gx, st);
            fb->gl_w = fb->up(gw, st);
        }
        std::vector<ColDf> cols(n_r);
        std::vector<df> ilr(n_r);
        const double wl = kC_ / kCF_;
        const double c3 = std::pow(kCF_, 3.0);
        for (int j = 0; j < n_r; ++j) {
            const double R = g.slant[j];
            const double k4r = ((4.0 * kPIref_) * R) / wl;
            cols[j].Q = df_from(R * R);
            cols[j].k4r = df_from(k4r);
            cols[j].tau2pi = df_from((2.0 * kPIref_) * g.tcorr[j]);
            const double a0 = std::fmod(k4r, 2.0 * M_PI);
            cols[j].az0 = mk((float)std::cos(a0), (float)std::sin(a0));
            cols[j].rscale = (float)g.rscale[j];
            const double fr = g.range_freq[j];
            cols[j].csrc = (float)(kPIref_ * fr * fr * kC_ * R / (2.0 * c3));
            cols[j].crcmc = (float)((4.0 * kPIref_) * fr * R / kC_);
            cols[j].rmig = (float)(2.0 * R * g.fs / kC_);
            ilr[j] = df_from(1.0 / (wl * R));
        }
        fb->cols = fb->up(cols, st);
        fb->inv_lamR = fb->up(ilr, st);
        fb->slant = fb->up(g.slant, st);
        fb->zero_df = fb->up(std::vector<df>(n_r, df_make(0.f, 0.f)), st);
        fb->nr_smooth = is_smooth7(n_r) && n_r <= fused_cap();
        if (fb->nr_smooth) fb->dnr = fft.desc3(n_r);
        else fb->cnr = get_czt(h, n_r, n_r, n_r);
        h->fast_bursts[key] = fb;
        return fb;
    }

    Result run(const std::vector<int>& pk, int level, bool tops) {
        const bool az = level == S1G_AZIMUTH_COMPRESSED;
        auto fbp = prepare(pk, az ? tops : false);
        const FastBurst& fb = *fbp;
        const BurstGeom& g = fb.g;
        const int n_a = g.n_a, n_r = g.n_r;
        Pipe<float> plain(h);
        h->mark("decode");
        cf32* raw = predecoded ? const_cast<cf32*>(predecoded) : plain.decode(pk, g);
        Result r;
        r.elem = S1G_CF32;
        r.rows = n_a;
        r.cols = n_r;
        r.pitch = n_r;
        if (level == S1G_RAW) {
            r.ptr = raw;
            return r;
        }
        h->mark("range_compress");
        if (h->use_eccm) {
            cf32* w = h->bRawW.as<cf32>((size_t)n_a * n_r);
            plain.eccm_fp64(pk, g, w, predecoded64);
            raw = w;
        }
        cf32* rc = h->bB.as<cf32>((size_t)n_a * n_r);
        rc_fused(raw, rc, n_a, n_r, g.h, fb.dM, fb.ref, st);
        const bool rd = (level == S1G_RANGE_DOPPLER) || (az && !tops);
        if (rd) {
            cf32* Bt = h->bC.as<cf32>((size_t)n_a * n_r);
            cf32* Ct = h->bD.as<cf32>((size_t)n_a * n_r);
            transpose_batched<float>(rc, n_r, 0, Bt, n_a, 0, n_a, n_r, 1, st);
            plain.fft_rows(n_a, Bt, n_a, Bt, n_a, n_r, -1);
            roll_rows<float>(Bt, n_a, Ct, n_a, n_a, n_a / 2, n_r, st);
            transpose_batched<float>(Ct, n_a, 0, rc, n_r, 0, n_r, n_a, 1, st);
        }
        if (!az) {
            r.ptr = rc;
            return r;
        }
        if (!tops) return stripmap(rc, fb, plain);
        return tops_chain(rc, raw, fb);
    }

    RowArgs row_args(cf32* data, const FastBurst& fb, int tops, const df* fdc) {
        RowArgs ra{};
        ra.data = data;
        ra.S = fb.S;
        ra.n_r = fb.g.n_r;
        ra.tops = tops;
        ra.rows = fb.rows_df;
        ra.cols = fb.cols;
        ra.fdc = fdc;
        ra.smooth = fb.nr_smooth;
        ra.d = fb.dnr;
        ra.cz = fb.cnr;
        const double wl = kC_ / kCF_;
        ra.lam2_4 = df_from(std::pow(wl, 2.0) / 4.0);
        ra.post = 1;
        return ra;
    }

    Result stripmap(cf32* rd, const FastBurst& fb, Pipe<float>& plain) {
        const int n_a = fb.g.n_a, n_r = fb.g.n_r;
        h->mark("row_pass");
        rowpass_fused(row_args(rd, fb, 0, fb.zero_df), st);
        h->mark("azimuth_ifft");
        cf32* Bt = h->bC.as<cf32>((size_t)n_a * n_r);
        transpose_batched<float>(rd, n_r, 0, Bt, n_a, 0, n_a, n_r, 1, st);
        plain.fft_rows(n_a, Bt, n_a, Bt, n_a, n_r, +1);
        scale_rows<float>(Bt, n_a, n_a, n_r, 1.0 / n_a, st);
        transpose_batched<float>(Bt, n_a, 0, rd, n_r, 0, n_r, n_a, 1, st);
        Result r;
        r.ptr = rd;
        r.rows = n_a;
        r.cols = n_r;
        r.pitch = n_r;
        r.elem = S1G_CF32;
        return r;
    }

    Result tops_chain(cf32* rc, const cf32* raw, const FastBurst& fb) {
        const BurstGeom& g = fb.g;
        const int n_a = g.n_a, n_r = g.n_r, S = fb.S;
        const double bd = g.swath_number == 11 ? 675 : 600;
        h->mark("doppler");
        const int nchunk = 8;
        DcEstArgs da{};
        da.raw = raw;
        da.n_a = n_a;
        da.n_r = n_r;
        da.M = fb.M;
        da.h = g.h;
        da.d = fb.dcDesc;
        da.U = fb.dcU;
        da.nb = fb.dcNb;
        da.H = fb.dcH;
        da.rcd = h->bDc.as<float4>((size_t)n_a * n_r);
        da.g = fb.dcG;
        da.part = h->bDcPart.as<cf64>((size_t)nchunk * n_r);
        da.nchunk = nchunk;
        dc_lag1_sums(da, st);
        h->mark("freq_unfold");
        cf32* rcT = h->bC.as<cf32>((size_t)n_a * n_r);
        transpose_batched<float>(rc, n_r, 0, rcT, n_a, 0, n_a, n_r, 1, st);
        cf32* ufrT = h->bD.as<cf32>((size_t)n_r * S);
        FufrArgs fa{};
        fa.rcT = rcT;
        fa.n_a = n_a;
        fa.n_r = n_r;
        fa.na_smooth = fb.na_smooth;
        fa.dna = fb.dna;
        fa.cna = fb.cna;
        fa.cf = fb.cf;
        fa.ci = fb.ci;
        fa.dfwd = fb.dfwd;
        fa.reramp = fb.reramp;
        fa.S = S;
        fa.tile_len = fb.tile_len;
        fa.bw = fb.bw;
        fa.out = ufrT;
        fufr_fused(fa, st);
        h->mark("doppler_fit");
        DcFitArgs dfa{};
        dfa.n_rng = n_r;
        dfa.num_blocks = 30;
        dfa.prf = 1.0 / g.pri;
        const std::vector<double> rt = linspace(g.near, g.far, 30);
        for (int b = 0; b < 30; ++b) dfa.rt[b] = rt[b] - rt[0];
        dfa.near = g.near;
        dfa.far = g.far;
        double* fdc = h->bCols.as<double>(n_r);
        df* fdc_df = h->bFdf.as<df>(n_r);
        dc_fit_fast(da.part, nchunk, dfa, fdc, fdc_df, st);
        h->mark("row_pass");
        cf32* ufr = h->bA.as<cf32>((size_t)S * n_r);
        transpose_batched<float>(ufrT, S, 0, ufr, n_r, 0, n_r, S, 1, st);
        if (h->rcmc == S1G_RCMC_SINC) {
            // the range IFFT as is, then the sinc migration shift with the
            // scale and azimuth-filter factor (no phase RCMC)
            RowArgs ra = row_args(ufr, fb, 1, fdc_df);
            ra.post = 0;
            rowpass_fused(ra, st);
            RcmcArgs rc{};
            rc.in = ufr;
            rc.out = h->bE.as<cf32>((size_t)S * n_r);
            rc.S = S;
            rc.n_r = n_r;
            rc.L = h->rcmc_L;
            rc.rows = fb.rows_df;
            rc.cols = fb.cols;
            rc.fdc = fdc_df;
            rc.lam2_4 = ra.lam2_4;
            rcmc_sinc(rc, st);
            ufr = rc.out;
        } else {
            rowpass_fused(row_args(ufr, fb, 1, fdc_df), st);
        }
        h->mark("time_unfold");
        cf32* ufrT2 = h->bD.as<cf32>((size_t)n_r * S);
        transpose_batched<float>(ufr, n_r, 0, ufrT2, S, 0, S, n_r, 1, st);
        TufrDev* dP = h->bTd.as<TufrDev>(1);
        tufr_params_fast(fb.rows64, fb.slant, fdc, S, n_r, fb.rate, g.T, g.prf, bd, g.swath_number,
                         h->bKa0.as<double>(S), dP, st);
        if (h->num_sms == 0) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
        }
        h->mark("azimuth_ifft");
        // azimuth IFFT (length S, 1/S) of every range bin, s1_decoder.cpp:682
        cf32* Aaz = h->bC.as<cf32>((size_t)n_r * S);
        czt_rows(ufrT2, S, Aaz, S, n_r, fb.cS, +1, 1.0f / (float)S, st);
        h->mark("time_unfold");
        // launch sized from the host plan; the kernel takes the tile count and
        // band from dP and flags (status) a burst outside the plan
        TufrArgs ta{};
        ta.in = Aaz;
        ta.S = S;
        ta.n_r = n_r;
        ta.P = dP;
        ta.dnu = fft.desc3(fb.m_nu);
        ta.rows = fb.rows_df;
        ta.cols = fb.cols;
        ta.fdc = fdc_df;
        ta.inv_lamR = fb.inv_lamR;
        const double wl = kC_ / kCF_;
        ta.lam2_4 = df_from(std::pow(wl, 2.0) / 4.0);
        ta.rate = df_from(fb.rate);
        ta.pi_ = df_from(kPIref_);
        ta.two_pi_ = df_from(2.0 * kPIref_);
        ta.tmax = fb.t_hi;
        ta.bwmax = fb.bw_max;
        ta.s0 = fb.s0;
        ta.n_out = fb.n_out;
        const int grid = std::max(1, h->num_sms * tufr_ctas_per_sm(ta));
        ta.KN = h->bKN.as<float>((size_t)grid * kTufrGroup * 4 * S);
        ta.G = h->bTuG.as<cf32>((size_t)grid * kTufrGroup * fb.m_nu);
        ta.tab.band = h->bTuD.as<float>((size_t)fb.m_nu);
        ta.tab.nu_l0 = h->bTuI.as<int>((size_t)ta.n_out);
        ta.tab.nu_w = h->bTuW.as<cf32>((size_t)ta.n_out * kNuTaps);
        ta.tab.rer = h->bTuR.as<float4>((size_t)ta.n_out);
        ta.tab.gl_x = fb.gl_x;
        ta.tab.gl_w = fb.gl_w;
        tufr_tables(ta, st);
        cf32* outT = h->bE.as<cf32>((size_t)n_r * ta.n_out);
        ta.out = outT;
        int* stat = tufr_status ? tufr_status : h->bTstat.as<int>(1);
        if (!tufr_status) check_cuda(cudaMemsetAsync(stat, 0, sizeof(int), st), "tstat");
        ta.status = stat;
        tufr_fused(ta, grid, st);
        h->mark("corner_turn");
        cf32* O = final_out ? final_out : h->bA.as<cf32>((size_t)ta.n_out * n_r);
        transpose_batched<float>(outT, ta.n_out, 0, O, n_r, 0, n_r, ta.n_out, 1, st);
        Result r;
        r.ptr = O;
        r.rows = ta.n_out;
        r.cols = n_r;
        r.pitch = n_r;
        r.elem = S1G_CF32;
        r.status = stat;
        return r;
    }
};

static const cf32* swath_cached_decode(s1g_decoder* h, const std::vector<int>& pk);

static Result compute_burst(s1g_decoder* h, const std::vector<int>& pk, int level, bool tops) {
    for (auto& m : h->marks) cudaEventDestroy(m.second);
    h->marks.clear();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, h->stream);
    Result r;
    if (h->precision == S1G_PREC_FP64) r = Pipe<double>(h).run(pk, level, tops);
    else if (h->precision == S1G_PREC_FP32_PLAIN) r = Pipe<float>(h).run(pk, level, tops);
    else {
        FastPipe fp(h);
        fp.predecoded = swath_cached_decode(h, pk);
        r = fp.run(pk, level, tops);
    }
    cudaEventRecord(e1, h->stream);
    check_cuda(cudaEventSynchronize(e1), "product");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    h->last_ms = ms;
    h->close_marks();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_cuda(cudaGetLastError(), "product kernels");
    if (tma_take_error() != 0) throw S1Error(S1G_E_TIMEOUT, "a TMA corner turn gave up waiting for its tile");
    if (r.status) {
        int st = 0;
        check_cuda(cudaMemcpy(&st, r.status, sizeof(int), cudaMemcpyDeviceToHost), "tufr status");
        if (st) throw S1Error(S1G_E_GEOMETRY, "azimuth time unfolding parameters out of range");
    }
    return r;
}

// Copy a device result into a caller buffer (rows x cols, zero-fill beyond valid_cols).
// Copy rows [row0, row0 + rows_to_copy) of a product into rows dst_row0..
// of a caller buffer of `cols` columns: the product's row starts at column
// col0 (columns before it are zero) and a row narrower than the rest of the
// buffer row is zero-filled on the right.
static void deliver(s1g_decoder* h, const Result& r, long long row0, void* out, long long cols, int out_type,
                    int on_device, long long rows_to_copy, long long dst_row0, long long col0 = 0) {
    const size_t esz = out_type == S1G_CF32 ? 8 : 16;
    void* dst = nullptr;
    void* stage = nullptr;
    if (on_device) {
        dst = (char*)out + (size_t)dst_row0 * cols * esz;
    } else {
        stage = h->bStage.get((size_t)rows_to_copy * cols * esz);
        dst = stage;
    }
    if (col0 > 0) check_cuda(cudaMemsetAsync(dst, 0, (size_t)rows_to_copy * cols * esz, h->stream), "left pad");
    char* d0 = (char*)dst + (size_t)col0 * esz;
    const int width = (int)(cols - col0);
    const int valid = (int)std::min<long long>(width, r.cols);
    if (r.elem == S1G_CF32) {
        const cf32* src = (const cf32*)r.ptr + row0 * r.pitch;
        if (out_type == S1G_CF32) convert_rows<float, float>(src, r.pitch, (cf32*)d0, cols, width, valid, rows_to_copy, h->stream);
        else convert_rows<double, float>(src, r.pitch, (cf64*)d0, cols, width, valid, rows_to_copy, h->stream);
    } else {
        const cf64* src = (const cf64*)r.ptr + row0 * r.pitch;
        if (out_type == S1G_CF32) convert_rows<float, double>(src, r.pitch, (cf32*)d0, cols, width, valid, rows_to_copy, h->stream);
        else convert_rows<double, double>(src, r.pitch, (cf64*)d0, cols, width, valid, rows_to_copy, h->stream);
    }
    if (!on_device)
        check_cuda(cudaMemcpyAsync((char*)out + (size_t)dst_row0 * cols * esz, stage, (size_t)rows_to_copy * cols * esz,
                                   cudaMemcpyDeviceToHost, h->stream),
                   "result download");
    check_cuda(cudaStreamSynchronize(h->stream), "deliver");
}

static bool tops_for(const std::string& swath) { return !is_sm(swath); }

}  // namespace s1g

// ------------------------------------------------------------------ C ABI
#define API_BEGIN(h)       \
    if (!(h)) return S1G_E_INVALID_ARGUMENT; \
    try {
#define API_END(h)                                   \
    }                                                \
    catch (const S1Error& e) {                       \
        (h)->err = e.what();                         \
        return e.code;                               \
    }                                                \
    catch (const std::exception& e) {                \
        (h)->err = e.what();                         \
        return S1G_E_CUDA;                           \
    }                                                \
    return S1G_OK;

extern "C" {

const char* s1g_version(void) { return "s1g 0.1 (sm_103a)"; }

int s1g_tuning_report(char* buf, size_t buflen) {
    if (!buf || !buflen) return S1G_E_INVALID_ARGUMENT;
    const std::string t = tuning_report();
    const size_t k = std::min(buflen - 1, t.size());
    memcpy(buf, t.data(), k);
    buf[k] = 0;
    return t.size() < buflen ? S1G_OK : S1G_E_BUFFER;
}

int s1g_open_buffer(const uint8_t* bytes, size_t nbytes, int device, s1g_decoder** out) {
    if (!out || (!bytes && nbytes)) return S1G_E_INVALID_ARGUMENT;
    auto* h = new s1g_decoder();
    h->device = device;
    try {
        open_stream(h, bytes, nbytes);
    } catch (const std::exception& e) {
        fprintf(stderr, "s1g_open: %s\n", e.what());
        delete h;
        *out = nullptr;
        return S1G_E_CUDA;
    }
    *out = h;
    return S1G_OK;
}

int s1g_open_file(const char* path, int device, s1g_decoder** out) {
    if (!path || !out) return S1G_E_INVALID_ARGUMENT;
    *out = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    // map the file read-only and stream it to the device; nothing of it is
    // copied into a host vector first
    const void* map = nullptr;
    size_t n = 0;
    if (!map_file(path, &map, &n)) return S1G_E_IO;
    auto* h = new s1g_decoder();
    h->device = device;
    int rc = S1G_OK;
    try {
        open_stream(h, (const uint8_t*)map, n, true);
    } catch (const std::exception& e) {
        fprintf(stderr, "s1g_open: %s\n", e.what());
        rc = S1G_E_CUDA;
    }
    unmap_file(map, n);
    if (rc != S1G_OK) {
        delete h;
        return rc;
    }
    h->ingest_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    h->ingest_bytes = (long long)n;
    *out = h;
    return S1G_OK;
}

int s1g_reload_buffer(s1g_decoder* h, const uint8_t* bytes, size_t nbytes) {
    API_BEGIN(h)
    if (!bytes && nbytes) return S1G_E_INVALID_ARGUMENT;
    check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
    ingest(h, bytes, nbytes, false);
    API_END(h)
}

int s1g_reload_file(s1g_decoder* h, const char* path) {
    API_BEGIN(h)
    if (!path) return S1G_E_INVALID_ARGUMENT;
    const auto t0 = std::chrono::steady_clock::now();
    const void* map = nullptr;
    size_t n = 0;
    if (!map_file(path, &map, &n)) throw S1Error(S1G_E_IO, std::string("Unable to open ") + path);
    try {
        check_cuda(cudaSetDevice(h->device), "cudaSetDevice");
        ingest(h, (const uint8_t*)map, n, true);
    } catch (...) {
        unmap_file(map, n);
        throw;
    }
    unmap_file(map, n);
    h->ingest_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    h->ingest_bytes = (long long)n;
    API_END(h)
}

int s1g_ingest_stats(const s1g_decoder* h, double* ms, int64_t* bytes) {
    if (!h) return S1G_E_INVALID_ARGUMENT;
    if (ms) *ms = h->ingest_ms;
    if (bytes) *bytes = h->ingest_bytes;
    return S1G_OK;
}

int s1g_close(s1g_decoder* h) {
    if (!h) return S1G_E_INVALID_ARGUMENT;
    delete h;
    return S1G_OK;
}

const char* s1g_last_error(const s1g_decoder* h) { return h ? h->err.c_str() : "null handle"; }

int s1g_set_precision(s1g_decoder* h, int precision) {
    if (!h || (precision != S1G_PREC_FP32 && precision != S1G_PREC_FP64 && precision != S1G_PREC_FP32_PLAIN))
        return S1G_E_INVALID_ARGUMENT;
    h->precision = precision;
    return S1G_OK;
}

int s1g_set_abc_decode(s1g_decoder* h, int mode) {
    if (!h || (mode != S1G_ABC_REFERENCE && mode != S1G_ABC_FIELDS)) return S1G_E_INVALID_ARGUMENT;
    const int f = mode == S1G_ABC_FIELDS;
    if (f != h->abc_fields) h->swath_decodes.clear();
    h->abc_fields = f;
    return S1G_OK;
}

int s1g_apply_eccm(s1g_decoder* h, int det, int mit) {
    if (!h) return S1G_E_INVALID_ARGUMENT;
    h->use_eccm = true;
    h->det = det;
    h->mit = mit;
    return S1G_OK;
}

int s1g_num_packets(const s1g_decoder* h, int64_t* n) {
    if (!h || !n) return S1G_E_INVALID_ARGUMENT;
    *n = h->npk;
    return S1G_OK;
}

int s1g_swath_names(const s1g_decoder* h, char* buf, size_t len) {
    if (!h || !buf || !len) return S1G_E_INVALID_ARGUMENT;
    std::ostringstream o;
    for (const auto& s : h->swath_order) o << s << " " << h->swath_counts.at(s) << "\n";
    const std::string t = o.str();
    if (t.size() + 1 > len) return S1G_E_BUFFER;
    memcpy(buf, t.c_str(), t.size() + 1);
    return S1G_OK;
}

int s1g_num_bursts(const s1g_decoder* h, const char* swath, int* n) {
    if (!h || !swath || !n) return S1G_E_INVALID_ARGUMENT;
    auto it = h->bursts.find(swath);
    if (it == h->bursts.end()) return S1G_E_BAD_SWATH;
    *n = (int)it->second.size();
    return S1G_OK;
}

int s1g_packet_field(const s1g_decoder* h, int64_t packet, const char* name, int64_t* value) {
    if (!h || !name || !value || packet < 0 || packet >= (int64_t)h->hdr.size()) return S1G_E_INVALID_ARGUMENT;
    for (int i = 0; i < F_COUNT; ++i)
        if (!strcmp(kFieldNames[i], name)) {
            *value = h->hdr[packet][i];
            return S1G_OK;
        }
    if (!strcmp(name, "offset")) {
        *value = h->hdr[packet].offset;
        return S1G_OK;
    }
    return S1G_E_INVALID_ARGUMENT;
}

int s1g_state_vectors(const s1g_decoder* h, double* out7, int cap, int* count) {
    if (!h || !count) return S1G_E_INVALID_ARGUMENT;
    const int n = (int)h->sv.t.size();
    *count = n;
    for (int i = 0; i < n && i < cap && out7; ++i) {
        out7[7 * i] = h->sv.t[i];
        for (int c = 0; c < 3; ++c) {
            out7[7 * i + 1 + c] = h->sv.p[i][c];
            out7[7 * i + 4 + c] = h->sv.v[i][c];
        }
    }
    return S1G_OK;
}

int s1g_attitudes(const s1g_decoder* h, double* out10, int cap, int* count) {
    if (!h || !count) return S1G_E_INVALID_ARGUMENT;
    const int n = (int)h->sv.t.size();
    *count = n;
    for (int i = 0; i < n && i < cap && out10; ++i) {
        double* o = out10 + 10 * i;
        for (int c = 0; c < 4; ++c) o[c] = h->sv.q[i][c];
        for (int c = 0; c < 3; ++c) o[4 + c] = h->sv.w[i][c];
        for (int c = 0; c < 3; ++c) o[7 + c] = h->sv.att[i][c];
    }
    return S1G_OK;
}

const char* s1g_field_name(int i) { return (i >= 0 && i < F_COUNT) ? kFieldNames[i] : nullptr; }

// The printout of L0Packet::print_primary_header, print_secondary_header,
// print_modes and print_pulse_info as s1_print packet_info shows it
// (print_main.cpp:26-47, packet.cpp:204-261).
int s1g_packet_info(s1g_decoder* h, int64_t packet, char* buf, size_t buflen, size_t* needed) {
    API_BEGIN(h)
    if (packet < 0 || packet >= (int64_t)h->hdr.size())
        throw S1Error(S1G_E_INVALID_ARGUMENT, "Index is greater than the number of packets.");
    const PacketHdr& p = h->hdr[packet];
    std::ostringstream o;
    o << "Primary Header:" << std::endl;
    for (int i = 0; i < F_COARSE; ++i) o << kFieldNames[i] << ": " << p[i] << std::endl;
    o << "\nSecondary Header: " << std::endl;
    for (int i = F_COARSE; i < F_COUNT; ++i)
        if (strncmp(kFieldNames[i], "na_", 3) != 0) o << kFieldNames[i] << ": " << p[i] << std::endl;
    o << "\nOperating Mode Info:" << std::endl;
    o << "Data Format: " << data_format(p) << std::endl;
    o << "BAQ Mode: " << baq_mode_name(p) << std::endl;
    o << "BAQ Block Length: " << 8 * (p[F_BAQ_BL] + 1) << std::endl;
    o << "Num BAQ Blocks: " << num_baq_blocks(p) << std::endl;
    o << "Test Mode: " << test_mode_name(p) << std::endl;
    o << "Sensor Mode: " << sensor_mode_name(p) << std::endl;
    o << "Signal Type: " << signal_type_name(p) << std::endl;
    o << "Error Status: " << (p[F_ERR] == 0 ? "nominal" : "ssb_corrupt") << std::endl;
    o << "\nPulse Info:" << std::endl;
    o << std::fixed << std::setprecision(8);
    o << "Time: " << p.time() << std::endl;
    o << "Swath: " << p.swath() << std::endl;
    o << "RX Polarization: " << rx_polarization(p) << std::endl;
    o << "TX Polarization: " << tx_polarization(p) << std::endl;
    o << "Pulse Length: " << p.pulse_length_us() << std::endl;
    o << "TX Ramp Rate (TXPRR): " << p.tx_ramp_rate() << std::endl;
    o << "Start Frequency (TXPSF): " << p.start_frequency() << std::endl;
    o << "PRI: " << p.pri_us() << std::endl;
    o << "SWL: " << p.swl_us() << std::endl;
    o << "SWST: " << p.swst_us() << std::endl;
    o << "RX Gain: " << p.rx_gain_db() << std::endl;
    o << "Range Decimation: " << (int)p[F_RANGE_DEC] << std::endl;
    o << "TX Pulse Number: " << (int)p[F_TXPN] << std::endl;
    const std::string t = o.str();
    if (needed) *needed = t.size() + 1;
    if (buf && buflen) {
        const size_t k = std::min(buflen - 1, t.size());
        memcpy(buf, t.data(), k);
        buf[k] = 0;
    }
    API_END(h)
}

static const int kMaxChainTerms = 8;

int s1g_azimuth_adjoint(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                        double doppler_centroid, double* loss, double* grad_theta, double* grad_centroid) {
    API_BEGIN(h)
    if (!swath || !loss || ntheta < 0 || ntheta > kMaxChainTerms || (ntheta && !theta)) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const bool grads = grad_theta || grad_centroid;
    const ChainResult r = h->precision == S1G_PREC_FP64
                              ? azimuth_chain<double>(h, pk, theta, ntheta, doppler_centroid, grads, false)
                              : azimuth_chain<float>(h, pk, theta, ntheta, doppler_centroid, grads, false);
    *loss = r.loss;
    if (grad_theta)
        for (int j = 0; j < ntheta; ++j) grad_theta[j] = r.g_theta[j];
    if (grad_centroid) *grad_centroid = r.g_fc;
    API_END(h)
}

int s1g_azimuth_focus(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                      double doppler_centroid, void* out, int64_t rows, int64_t cols, int out_type, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || ntheta < 0 || ntheta > kMaxChainTerms || (ntheta && !theta) ||
        (out_type != S1G_CF32 && out_type != S1G_CF64))
        return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    if (rows != g.n_a || cols != g.n_r) return S1G_E_BUFFER;
    const bool f64 = h->precision == S1G_PREC_FP64;
    const ChainResult c = f64 ? azimuth_chain<double>(h, pk, theta, ntheta, doppler_centroid, false, true)
                              : azimuth_chain<float>(h, pk, theta, ntheta, doppler_centroid, false, true);
    Result r;
    r.ptr = c.image;
    r.rows = c.rows;
    r.cols = c.cols;
    r.pitch = c.cols;
    r.elem = f64 ? S1G_CF64 : S1G_CF32;
    deliver(h, r, 0, out, cols, out_type, out_on_device, rows, 0);
    API_END(h)
}

int s1g_tops_adjoint(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                     double centroid_offset, double* loss, double* grad_theta, double* grad_offset) {
    API_BEGIN(h)
    if (!swath || !loss || ntheta < 0 || ntheta > kMaxChainTerms || (ntheta && !theta)) return S1G_E_INVALID_ARGUMENT;
    if (!is_iw(swath)) return S1G_E_UNSUPPORTED;
    const auto& pk = burst_packets(h, swath, burst);
    const bool grads = grad_theta || grad_offset;
    const ChainResult r = h->precision == S1G_PREC_FP64
                              ? tops_chain<double>(h, pk, theta, ntheta, centroid_offset, grads, false)
                              : tops_chain<float>(h, pk, theta, ntheta, centroid_offset, grads, false);
    *loss = r.loss;
    if (grad_theta)
        for (int j = 0; j < ntheta; ++j) grad_theta[j] = r.g_theta[j];
    if (grad_offset) *grad_offset = r.g_fc;
    API_END(h)
}

int s1g_tops_focus(s1g_decoder* h, const char* swath, int burst, const double* theta, int ntheta,
                   double centroid_offset, void* out, int64_t rows, int64_t cols, int out_type, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || ntheta < 0 || ntheta > kMaxChainTerms || (ntheta && !theta) ||
        (out_type != S1G_CF32 && out_type != S1G_CF64))
        return S1G_E_INVALID_ARGUMENT;
    if (!is_iw(swath)) return S1G_E_UNSUPPORTED;
    const auto& pk = burst_packets(h, swath, burst);
    const bool f64 = h->precision == S1G_PREC_FP64;
    const ChainResult c = f64 ? tops_chain<double>(h, pk, theta, ntheta, centroid_offset, false, true)
                              : tops_chain<float>(h, pk, theta, ntheta, centroid_offset, false, true);
    if (rows != c.rows || cols != c.cols) return S1G_E_BUFFER;
    Result r;
    r.ptr = c.image;
    r.rows = c.rows;
    r.cols = c.cols;
    r.pitch = c.cols;
    r.elem = f64 ? S1G_CF64 : S1G_CF32;
    deliver(h, r, 0, out, cols, out_type, out_on_device, rows, 0);
    API_END(h)
}

int s1g_packet_offset(const s1g_decoder* h, int64_t packet, int64_t* offset) {
    if (!h || !offset || packet < 0 || packet >= (int64_t)h->hdr.size()) return S1G_E_INVALID_ARGUMENT;
    *offset = h->hdr[packet].offset;
    return S1G_OK;
}

int s1g_packet_samples(s1g_decoder* h, int64_t packet, void* out, int64_t n, int out_type, int out_on_device) {
    API_BEGIN(h)
    if (!out || packet < 0 || packet >= (int64_t)h->hdr.size() || (out_type != S1G_CF32 && out_type != S1G_CF64))
        return S1G_E_INVALID_ARGUMENT;
    BurstGeom g;
    g.n_a = 1;
    g.nq = h->hdr[packet].num_quads();
    g.n_r = 2 * g.nq;
    if (n != g.n_r) throw S1Error(S1G_E_BUFFER, "expected " + std::to_string(g.n_r) + " samples");
    if (g.n_r == 0) return S1G_OK;
    Pipe<double> p(h);
    const cf64* d = p.decode({(int)packet}, g);
    std::vector<cf64> line((size_t)g.n_r);
    check_cuda(cudaMemcpyAsync(line.data(), d, sizeof(cf64) * g.n_r, cudaMemcpyDeviceToHost, h->stream), "samples");
    check_cuda(cudaStreamSynchronize(h->stream), "samples sync");
    const void* src = line.data();
    std::vector<cf32> line32;
    size_t bytes = sizeof(cf64) * g.n_r;
    if (out_type == S1G_CF32) {
        line32.resize(line.size());
        for (size_t i = 0; i < line.size(); ++i) line32[i] = mk((float)line[i].x, (float)line[i].y);
        src = line32.data();
        bytes = sizeof(cf32) * g.n_r;
    }
    if (out_on_device)
        check_cuda(cudaMemcpy(out, src, bytes, cudaMemcpyHostToDevice), "samples up");
    else
        std::memcpy(out, src, bytes);
    API_END(h)
}

int s1g_check_sidecars(s1g_decoder* h, const char* index_path, const char* annotation_path, s1g_sidecar_report* rep) {
    API_BEGIN(h)
    s1g_sidecar_report r;
    std::memset(&r, 0, sizeof(r));
    r.index_first_mismatch = r.annotation_first_mismatch = -1;
    const int64_t npk = (int64_t)h->hdr.size();
    r.packets = npk;
    // packet k spans [offset_k, offset_k + 7 + packet_data_length)
    auto pk_end = [&](int64_t k) { return (int64_t)h->hdr[k].offset + 7 + h->hdr[k][F_PDL]; };
    std::string msg;
    if (index_path) {
        std::vector<s1g_index_record> ix;
        if (!load_index(index_path, false, ix)) throw S1Error(S1G_E_IO, std::string("Unable to open ") + index_path);
        r.index_records = (int64_t)ix.size();
        for (size_t i = 0; i < ix.size(); ++i) {
            const int64_t u = ix[i].unit_offset;
            const int64_t next = i + 1 < ix.size() ? (int64_t)ix[i + 1].unit_offset : npk;
            bool ok = u < npk && next > u && next <= npk && (int64_t)ix[i].byte_offset == (int64_t)h->hdr[u].offset;
            if (ok) ok = (int64_t)ix[i].data_size == pk_end(next - 1) - (int64_t)h->hdr[u].offset;
            if (ok) {
                r.index_packets_covered += next - u;
            } else {
                if (r.index_first_mismatch < 0) r.index_first_mismatch = (int64_t)i;
                r.index_mismatches++;
            }
        }
        if (r.index_mismatches)
            msg += std::to_string(r.index_mismatches) + " index records disagree with the packet stream (first: record " +
                   std::to_string(r.index_first_mismatch) + "). ";
        else if (r.index_packets_covered != npk)
            msg += "index blocks cover " + std::to_string(r.index_packets_covered) + " of " + std::to_string(npk) +
                   " packets. ";
    }
    if (annotation_path) {
        std::vector<s1g_annotation_record> an;
        if (!load_annotation(annotation_path, false, an))
            throw S1Error(S1G_E_IO, std::string("Unable to open ") + annotation_path);
        r.annotation_records = (int64_t)an.size();
        const int64_t m = std::min<int64_t>((int64_t)an.size(), npk);
        for (int64_t k = 0; k < m; ++k)
            if ((int64_t)an[k].packet_length != ((7 + h->hdr[k][F_PDL]) & 0xFFFF)) {
                if (r.annotation_first_mismatch < 0) r.annotation_first_mismatch = k;
                r.annotation_mismatches++;
            }
        if ((int64_t)an.size() != npk)
            msg += std::to_string(an.size()) + " annotation records for " + std::to_string(npk) + " packets. ";
        if (r.annotation_mismatches)
            msg += std::to_string(r.annotation_mismatches) + " annotation packet lengths disagree (first: packet " +
                   std::to_string(r.annotation_first_mismatch) + "). ";
    }
    if (rep) *rep = r;
    if (!msg.empty()) throw S1Error(S1G_E_SIDECAR, msg.substr(0, msg.size() - 1));
    API_END(h)
}

static int level_ok(int level) { return level >= S1G_RAW && level <= S1G_AZIMUTH_COMPRESSED; }

int s1g_burst_shape(s1g_decoder* h, const char* swath, int burst, int level, int64_t* rows, int64_t* cols) {
    API_BEGIN(h)
    if (!swath || !rows || !cols || !level_ok(level)) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    *cols = g.n_r;
    *rows = g.n_a;
    if (level == S1G_AZIMUTH_COMPRESSED) {
        // get_azimuth_compressed_burst always runs the TOPS chain
        // (s1_decoder.cpp:296-304): rows = 2*floor(floor(prf*T)/2)
        const int os = (int)std::floor(g.prf * g.T);
        *rows = 2 * (os / 2);
    }
    API_END(h)
}

int s1g_burst_unfold_shape(s1g_decoder* h, const char* swath, int burst, int64_t* S, int64_t* n_out) {
    API_BEGIN(h)
    if (!swath || !S || !n_out) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    *S = g.n_a;
    if (tops_for(swath)) {
        // azimuth_frequency_ufr's tiled length (image_formation.cpp:125-160)
        const double rate = Pipe<float>(h).dc_rate(g);
        *S = (int64_t)std::floor(std::abs(rate * g.T / g.prf) * g.n_a);
    }
    const int os = (int)std::floor(g.prf * g.T);
    *n_out = 2 * (os / 2);
    API_END(h)
}

int s1g_burst_product(s1g_decoder* h, const char* swath, int burst, int level, void* out, int64_t rows, int64_t cols,
                      int out_type, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || !level_ok(level) || (out_type != S1G_CF32 && out_type != S1G_CF64))
        return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const Result r = compute_burst(h, pk, level, true);
    if (r.rows != rows || r.cols != cols) {
        h->err = "output buffer shape " + std::to_string(rows) + "x" + std::to_string(cols) + " != product " +
                 std::to_string(r.rows) + "x" + std::to_string(r.cols);
        return S1G_E_BUFFER;
    }
    h->last = r;
    deliver(h, r, 0, out, cols, out_type, out_on_device, rows, 0);
    API_END(h)
}

// Swath assembly (s1_decoder.cpp:136-417).
//   IW: the bursts in order; azimuth products skip bursts of < 1000 lines and
//       add 20 zero rows after each burst.
//   SM: burst 0 split into azimuth blocks wherever num_quadratures changes
//       (get_azimuth_blocks, image_formation.cpp:46-84).  Raw: the blocks'
//       lines in order.  Range / range-Doppler / azimuth products of more
//       than one block: each block processed on its own, its rows
//       left-padded with zeros to the widest block, and (azimuth only) 20
//       zero rows after every block; a single block is returned as is.
// The buffer is as wide as the widest row.  Where the reference returns
// rows of different lengths (IW bursts of different widths, SM raw blocks),
// the shorter rows are zero-filled on the right.
struct SwathPlanEntry {
    std::vector<int> pk;
    long long rows, cols;
    long long col0;       // left zero padding
    long long pad_rows;   // zero rows after the entry
};

static std::vector<std::vector<int>> azimuth_blocks(const std::vector<PacketHdr>& hdr, const std::vector<int>& pk) {
    std::vector<std::vector<int>> blocks;
    std::vector<int> cur;
    int prev = pk.empty() ? 0 : hdr[pk.front()].num_quads();
    for (int i : pk) {
        const int nq = hdr[i].num_quads();
        if (nq != prev && !cur.empty()) {
            blocks.push_back(cur);
            cur.clear();
            prev = nq;
        }
        cur.push_back(i);
    }
    if (!cur.empty()) blocks.push_back(cur);
    return blocks;
}

static std::vector<SwathPlanEntry> swath_plan(s1g_decoder* h, const std::string& swath, int level, long long& rows,
                                              long long& cols) {
    auto it = h->bursts.find(swath);
    if (it == h->bursts.end()) throw S1Error(S1G_E_BAD_SWATH, "The requested swath, " + swath + ", does not exist in the data.");
    if (!is_iw(swath) && !is_sm(swath))
        throw S1Error(S1G_E_UNSUPPORTED, swath + " is not a supported swath type. Only IW and SM imaging modes are supported.");
    std::vector<SwathPlanEntry> plan;
    const auto& bs = it->second;
    const bool az = level == S1G_AZIMUTH_COMPRESSED;
    if (is_iw(swath)) {
        for (int b = 0; b < (int)bs.size(); ++b) {
            if (az && bs[b].size() < 1000) continue;
            const BurstGeom g = make_geom(h->hdr, bs[b]);
            const long long r = az ? 2 * ((int)std::floor(g.prf * g.T) / 2) : g.n_a;
            plan.push_back({bs[b], r, g.n_r, 0, az ? 20 : 0});
        }
    } else if (!bs.empty()) {
        const auto blocks = azimuth_blocks(h->hdr, bs[0]);
        long long widest = 0;
        for (const auto& b : blocks) widest = std::max<long long>(widest, 2LL * h->hdr[b.front()].num_quads());
        const bool multi = blocks.size() > 1 && level != S1G_RAW;
        for (const auto& b : blocks) {
            const long long n_r = 2LL * h->hdr[b.front()].num_quads();
            plan.push_back({b, (long long)b.size(), n_r, multi ? widest - n_r : 0, multi && az ? 20 : 0});
        }
    }
    rows = 0;
    cols = 0;
    for (const auto& e : plan) {
        rows += e.rows + e.pad_rows;
        cols = std::max(cols, e.col0 + e.cols);
    }
    return plan;
}

int s1g_swath_shape(s1g_decoder* h, const char* swath, int level, int64_t* rows, int64_t* cols) {
    API_BEGIN(h)
    if (!swath || !rows || !cols || !level_ok(level)) return S1G_E_INVALID_ARGUMENT;
    long long r, c;
    swath_plan(h, swath, level, r, c);
    *rows = r;
    *cols = c;
    API_END(h)
}

int s1g_swath_row_widths(s1g_decoder* h, const char* swath, int level, int64_t* widths, int64_t cap, int64_t* rows) {
    API_BEGIN(h)
    if (!swath || !rows || !level_ok(level)) return S1G_E_INVALID_ARGUMENT;
    long long R, C;
    const auto plan = swath_plan(h, swath, level, R, C);
    *rows = R;
    if (widths && cap >= R) {
        long long r = 0, first = -1;
        for (const auto& e : plan) {
            const long long w = e.col0 + e.cols;
            if (first < 0) first = w;
            for (long long k = 0; k < e.rows; ++k) widths[r++] = w;
            // the zero rows are as wide as the swath's first row
            for (long long k = 0; k < e.pad_rows; ++k) widths[r++] = first;
        }
    }
    API_END(h)
}

int s1g_swath_product(s1g_decoder* h, const char* swath, int level, void* out, int64_t rows, int64_t cols, int out_type,
                      int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || !level_ok(level)) return S1G_E_INVALID_ARGUMENT;
    long long R, C;
    const auto plan = swath_plan(h, swath, level, R, C);
    if (R != rows || C != cols) return S1G_E_BUFFER;
    const size_t esz = out_type == S1G_CF32 ? 8 : 16;
    const bool tops = tops_for(swath);
    long long row = 0;
    for (const auto& e : plan) {
        const Result r = compute_burst(h, e.pk, level, tops);
        deliver(h, r, 0, out, cols, out_type, out_on_device, r.rows, row, e.col0);
        row += r.rows;
        if (e.pad_rows) {
            const size_t nb = (size_t)e.pad_rows * cols * esz;
            if (out_on_device) check_cuda(cudaMemset((char*)out + (size_t)row * cols * esz, 0, nb), "pad");
            else memset((char*)out + (size_t)row * cols * esz, 0, nb);
            row += e.pad_rows;
        }
    }
    API_END(h)
}

static bool scaling_ok(int m) { return m >= S1G_SCALE_REAL && m <= S1G_SCALE_NORM_LOG; }

// Form the product in a device buffer of the handle, scale it on the GPU,
// deliver the float image.
static int product_image(s1g_decoder* h, const char* swath, int burst, int level, int scaling, float* out,
                         int64_t rows, int64_t cols, int out_on_device) {
    const int elem = h->precision == S1G_PREC_FP64 ? S1G_CF64 : S1G_CF32;
    const size_t esz = elem == S1G_CF32 ? 8 : 16;
    void* prod = h->bImgIn.get((size_t)rows * cols * esz);
    const int st = burst >= 0 ? s1g_burst_product(h, swath, burst, level, prod, rows, cols, elem, 1)
                              : s1g_swath_product(h, swath, level, prod, rows, cols, elem, 1);
    if (st != S1G_OK) return st;
    float* img = out_on_device ? out : h->bImgOut.as<float>((size_t)rows * cols);
    unsigned long long* mx = h->bImgMax.as<unsigned long long>(1);
    scale_image(prod, elem, (long long)rows * cols, scaling, img, mx, h->stream);
    if (!out_on_device)
        check_cuda(cudaMemcpyAsync(out, img, sizeof(float) * (size_t)rows * cols, cudaMemcpyDeviceToHost, h->stream),
                   "image down");
    check_cuda(cudaStreamSynchronize(h->stream), "image sync");
    return S1G_OK;
}

int s1g_burst_image(s1g_decoder* h, const char* swath, int burst, int level, int scaling, float* out, int64_t rows,
                    int64_t cols, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || !level_ok(level) || !scaling_ok(scaling) || burst < 0) return S1G_E_INVALID_ARGUMENT;
    return product_image(h, swath, burst, level, scaling, out, rows, cols, out_on_device);
    API_END(h)
}

int s1g_swath_image(s1g_decoder* h, const char* swath, int level, int scaling, float* out, int64_t rows,
                    int64_t cols, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || !level_ok(level) || !scaling_ok(scaling)) return S1G_E_INVALID_ARGUMENT;
    return product_image(h, swath, -1, level, scaling, out, rows, cols, out_on_device);
    API_END(h)
}

int s1g_spectrogram_shape(s1g_decoder* h, const char* swath, int burst, int fft_size, int stride, int64_t* rows,
                          int64_t* cols) {
    API_BEGIN(h)
    if (!swath || !rows || !cols || fft_size < 2 || stride < 1) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    *rows = fft_size;
    *cols = spectrogram_windows(g.n_r, fft_size, stride);
    API_END(h)
}

// The complex spectrogram in a device buffer of the handle (FP64 decode of the burst).
static const cf64* spectrogram_dev(s1g_decoder* h, const char* swath, int burst, int line, int fft_size, int stride,
                                   int64_t rows, int64_t cols) {
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    if (rows != fft_size || cols != spectrogram_windows(g.n_r, fft_size, stride))
        throw S1Error(S1G_E_BUFFER, "spectrogram buffer shape does not match");
    if (line < 0 || line >= g.n_a)
        throw S1Error(S1G_E_INVALID_ARGUMENT, "Azimuth Line " + std::to_string(line) +
                                                  " is outside of the valid range of 0 to " + std::to_string(g.n_a));
    Pipe<double> p(h);
    const cf64* A = p.decode(pk, g);
    cf64* out = h->bImgIn.as<cf64>((size_t)rows * cols);
    spectrogram(A + (size_t)line * g.n_r, g.n_r, fft_size, stride, out, h->stream);
    return out;
}

int s1g_spectrogram(s1g_decoder* h, const char* swath, int burst, int azimuth_line, int fft_size, int stride,
                    void* out, int64_t rows, int64_t cols, int out_type, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || fft_size < 2 || stride < 1 || (out_type != S1G_CF32 && out_type != S1G_CF64))
        return S1G_E_INVALID_ARGUMENT;
    const cf64* sp = spectrogram_dev(h, swath, burst, azimuth_line, fft_size, stride, rows, cols);
    Result r;
    r.ptr = sp;
    r.rows = rows;
    r.cols = cols;
    r.pitch = cols;
    r.elem = S1G_CF64;
    deliver(h, r, 0, out, cols, out_type, out_on_device, rows, 0);
    API_END(h)
}

int s1g_spectrogram_image(s1g_decoder* h, const char* swath, int burst, int azimuth_line, int fft_size, int stride,
                          int scaling, float* out, int64_t rows, int64_t cols, int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out || fft_size < 2 || stride < 1 || !scaling_ok(scaling)) return S1G_E_INVALID_ARGUMENT;
    const cf64* sp = spectrogram_dev(h, swath, burst, azimuth_line, fft_size, stride, rows, cols);
    float* img = out_on_device ? out : h->bImgOut.as<float>((size_t)rows * cols);
    scale_image(sp, S1G_CF64, (long long)rows * cols, scaling, img, h->bImgMax.as<unsigned long long>(1), h->stream);
    if (!out_on_device)
        check_cuda(cudaMemcpyAsync(out, img, sizeof(float) * (size_t)rows * cols, cudaMemcpyDeviceToHost, h->stream),
                   "image down");
    check_cuda(cudaStreamSynchronize(h->stream), "image sync");
    API_END(h)
}

int s1g_write_tiff(const char* path, const float* image, int64_t rows, int64_t cols) {
    std::string err;
    const int st = write_bigtiff(path, image, rows, cols, err);
    if (st != S1G_OK) fprintf(stderr, "s1g_write_tiff: %s\n", err.c_str());
    return st;
}

int s1g_burst_doppler(s1g_decoder* h, const char* swath, int burst, double* rate, double* dc, int64_t cols) {
    API_BEGIN(h)
    if (!swath || !rate || !dc) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    if (cols != g.n_r) return S1G_E_BUFFER;
    auto run = [&](auto tag) {
        using R = decltype(tag);
        Pipe<R> p(h);
        p.cur_pk = &pk;
        cpx<R>* A = p.decode(pk, g);
        A = p.range_compress(A, g, false);
        *rate = p.dc_rate(g);
        double* f = p.doppler(A, g, *rate);
        check_cuda(cudaMemcpyAsync(dc, f, sizeof(double) * g.n_r, cudaMemcpyDeviceToHost, h->stream), "dc down");
        check_cuda(cudaStreamSynchronize(h->stream), "dc sync");
    };
    if (h->precision == S1G_PREC_FP64) run(double());
    else run(float());
    API_END(h)
}

int s1g_eccm_mask_shape(s1g_decoder* h, const char* swath, int burst, int64_t* rows, int64_t* windows) {
    API_BEGIN(h)
    if (!swath || !rows || !windows) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    *rows = g.n_a;
    *windows = eccm_num_windows(g.n_r);
    API_END(h)
}

int s1g_eccm_mask(s1g_decoder* h, const char* swath, int burst, uint8_t* out, int64_t rows, int64_t windows,
                  int out_on_device) {
    API_BEGIN(h)
    if (!swath || !out) return S1G_E_INVALID_ARGUMENT;
    if (!h->use_eccm) {
        h->err = "s1g_eccm_mask: no ECCM thresholds set (call s1g_apply_eccm first)";
        return S1G_E_INVALID_ARGUMENT;
    }
    const auto& pk = burst_packets(h, swath, burst);
    const BurstGeom g = make_geom(h->hdr, pk);
    const int nw = eccm_num_windows(g.n_r);
    if (rows != g.n_a || windows != nw) {
        h->err = "mask buffer shape " + std::to_string(rows) + "x" + std::to_string(windows) + " != " +
                 std::to_string(g.n_a) + "x" + std::to_string(nw);
        return S1G_E_BUFFER;
    }
    // every precision takes the notch decisions in FP64 (the FP32 paths run
    // the FP64 notch too), so the mask is the FP64 pipeline's
    Pipe<double> p(h);
    cf64* A = p.decode(pk, g);
    const size_t bytes = (size_t)g.n_a * nw * 128;
    unsigned char* m = h->bEccmMask.as<unsigned char>(bytes);
    check_cuda(cudaMemsetAsync(m, 0, bytes, h->stream), "mask clear");
    p.eccm(A, g, m);
    check_cuda(cudaMemcpyAsync(out, m, bytes, out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               h->stream), "mask down");
    check_cuda(cudaStreamSynchronize(h->stream), "mask sync");
    API_END(h)
}

// Nominal FP32 arithmetic of the fused FP32 path for one burst, per stage:
// 5 N log2 N flops per complex FFT of N points; a chirp-z transform as its
// two convolution FFTs of length m plus 3 complex multiplications per point
// (6 flops each); the compensated Doppler transforms counted as plain FFTs
// (a lower bound: compensated arithmetic costs several times more); the time
// unfolding's gather as 7 flops per (sample, grid point) pair and range bin
// (one complex multiply-add by a real weight plus half of the weight, shared
// by two range bins) over ~(W T S + M) pairs, its two grid FFTs and a
// 15-tap complex stencil per output row.
static double fft_flops(double n) { return n > 1 ? 5.0 * n * std::log2(n) : 0.0; }
static double czt_flops(const CztDev& c) { return 2.0 * fft_flops(c.dm.n) + 18.0 * c.dm.n; }

int s1g_burst_stage_flops(s1g_decoder* h, const char* swath, int burst, char* buf, size_t len) {
    API_BEGIN(h)
    if (!swath || !buf || len == 0 || h->precision != S1G_PREC_FP32) return S1G_E_INVALID_ARGUMENT;
    const auto& pk = burst_packets(h, swath, burst);
    const bool tops = tops_for(swath);
    FastPipe fp(h);
    auto fbp = fp.prepare(pk, tops);
    const FastBurst& fb = *fbp;
    const double n_a = fb.g.n_a, n_r = fb.g.n_r, S = fb.S;
    std::ostringstream o;
    o << "range_compress " << n_a * (2.0 * fft_flops(fb.M) + 6.0 * fb.M) << "\n";
    if (tops) {
        // the burst's SLC once, for the tile count the device chose
        compute_burst(h, pk, S1G_AZIMUTH_COMPRESSED, true);
        TufrDev q{};
        check_cuda(cudaMemcpy(&q, h->bTd.p, sizeof(q), cudaMemcpyDeviceToHost), "tile count");
        const double T = q.q.num_tiles, M = fb.m_nu, n_out = fb.n_out;
        o << "doppler " << (double)fb.dcNb * n_a * 2.0 * fft_flops(fb.dcB) << "\n";
        const double dna = fb.na_smooth ? fft_flops(n_a) : czt_flops(fb.cna);
        o << "freq_unfold " << n_r * (dna + czt_flops(fb.cf) + czt_flops(fb.ci) + 12.0 * S) << "\n";
        const double dnr = fb.nr_smooth ? 2.0 * fft_flops(n_r) : 2.0 * czt_flops(fb.cnr);
        o << "row_pass " << S * (dnr + 60.0 * n_r) << "\n";
        o << "azimuth_ifft " << n_r * czt_flops(fb.cS) << "\n";
        o << "time_unfold " << n_r * (7.0 * (kNuW * T * S + M) + 2.0 * fft_flops(M) + 6.0 * M +
                                      8.0 * kNuTaps * n_out) << "\n";
        o << "tiles " << T << "\n";
    } else {
        const double dnr = fb.nr_smooth ? 2.0 * fft_flops(n_r) : 2.0 * czt_flops(fb.cnr);
        o << "row_pass " << n_a * (dnr + 60.0 * n_r) << "\n";
        o << "azimuth_ifft " << n_r * 2.0 * fft_flops(n_a) << "\n";
    }
    const std::string t = o.str();
    if (t.size() + 1 > len) return S1G_E_BUFFER;
    std::memcpy(buf, t.c_str(), t.size() + 1);
    API_END(h)
}

// Messages of the per-packet decode status codes (the reference's exceptions).
static std::string decode_error_text(int c, int packet) {
    static const char* names[] = {"", "", "", "", "", "", "", "packet length", "bit read past end",
                                  "BRC value is invalid.", "Max bit length exceeded in Huffman decoding.",
                                  "MCode is greater than the comparison flag.", "ragged burst"};
    return std::string("packet ") + std::to_string(packet) + ": " + (c < 0 && c > -13 ? names[-c] : "decode error");
}

// Batched decode of every listed burst of one handle (one launch pair): the
// job table (one entry per packet) is built once per burst list and cached.
struct BatchDecode {
    std::vector<int> pk;                 // packet index per job (for messages)
    std::vector<long long> raw_off;      // element offset of each burst in the raw array
    long long raw_elems = 0;
    size_t sym_bytes = 0, blk_bytes = 0;
    DecodeJob* d_jobs = nullptr;
    int njobs = 0;
    bool any_d = false, any_fixed = false;
    ~BatchDecode() {
        if (d_jobs) cudaFree(d_jobs);
    }
};

static std::shared_ptr<BatchDecode> batch_decode_plan(s1g_decoder* h, const std::vector<const std::vector<int>*>& bl) {
    auto bd = std::make_shared<BatchDecode>();
    std::vector<DecodeJob> jobs;
    long long sym = 0, blk = 0, out = 0;
    for (const auto* pkp : bl) {
        const std::vector<int>& pk = *pkp;
        const int nq = h->hdr[pk.front()].num_quads();
        const int n_r = 2 * nq;
        const int nb = (2 * nq + 255) / 256;
        bd->raw_off.push_back(out);
        for (int i : pk) {
            const FormatKind k = format_kind(h->hdr[i]);
            if (k == FMT_INVALID) throw S1Error(S1G_E_BAD_FORMAT, "packet " + std::to_string(i) + ": BAQ Mode is invalid.");
            (k == FMT_D ? bd->any_d : bd->any_fixed) = true;
            DecodeJob j;
            j.pk = i;
            j.nq = nq;
            j.sym = sym;
            j.blk = blk;
            j.out = out;
            jobs.push_back(j);
            bd->pk.push_back(i);
            sym += 4LL * sym_pitch(nq);
            blk += nb;
            out += n_r;
        }
    }
    bd->raw_elems = out;
    bd->sym_bytes = (size_t)sym;
    bd->blk_bytes = (size_t)blk;
    bd->njobs = (int)jobs.size();
    check_cuda(cudaMalloc(&bd->d_jobs, sizeof(DecodeJob) * std::max<size_t>(jobs.size(), 1)), "decode jobs");
    check_cuda(cudaMemcpy(bd->d_jobs, jobs.data(), sizeof(DecodeJob) * jobs.size(), cudaMemcpyHostToDevice),
               "decode jobs up");
    return bd;
}

// Host-side record of one enqueued batch: what to check once it has run.
struct BatchRun {
    long long total = 0;
    size_t nslots = 0;
    std::vector<std::shared_ptr<BatchDecode>> dec;
    std::vector<int*> dec_status;
    int* tstat = nullptr;
};

// Per-burst FP32 calls decode the whole swath once: one thread per packet
// walks its bitstream, so a single burst (~1500 packets) occupies few SMs
// and waits on the walk's latency, while a swath's packets fill the GPU.
// A burst whose packets failed to decode is not served from the cache (its
// own decode reports the error as usual).
struct SwathDecode {
    std::shared_ptr<BatchDecode> plan;
    Buf raw;
    std::vector<int> status;                  // per job
    std::map<int, size_t> burst_of_first;     // first packet index -> burst
    std::vector<size_t> job0;                 // first job of each burst
};

extern "C++" {
namespace s1g {
static const cf32* swath_cached_decode(s1g_decoder* h, const std::vector<int>& pk) {
    if (pk.empty()) return nullptr;
    const std::string sw = h->hdr[pk.front()].swath();
    auto bit = h->bursts.find(sw);
    if (bit == h->bursts.end() || bit->second.size() < 2) return nullptr;
    auto& slot = h->swath_decodes[sw];
    if (!slot) {
        auto sd = std::make_shared<SwathDecode>();
        std::vector<const std::vector<int>*> lists;
        size_t j = 0;
        for (size_t k = 0; k < bit->second.size(); ++k) {
            lists.push_back(&bit->second[k]);
            sd->burst_of_first[bit->second[k].front()] = k;
            sd->job0.push_back(j);
            j += bit->second[k].size();
        }
        try {
            sd->plan = batch_decode_plan(h, lists);
        } catch (const S1Error&) {
            return nullptr;   // a format the decoder rejects: leave it to the burst's own decode
        }
        cf32* raw = sd->raw.as<cf32>((size_t)std::max<long long>(sd->plan->raw_elems, 1));
        int* st = h->bDecStatus.as<int>((size_t)std::max(sd->plan->njobs, 1));
        if (sd->plan->any_d)
            decode_jobs<float>(h->d_stream, h->nbytes, h->d_off, sd->plan->d_jobs, sd->plan->njobs,
                               sd->plan->sym_bytes, sd->plan->blk_bytes, raw, st, h->dsc, h->tabs, h->stream);
        if (sd->plan->any_fixed)
            decode_fixed_jobs<float>(h->d_stream, h->nbytes, h->d_off, sd->plan->d_jobs, sd->plan->njobs, raw, st,
                                     h->abc_fields, h->stream);
        sd->status.resize(sd->plan->njobs);
        check_cuda(cudaMemcpyAsync(sd->status.data(), st, sizeof(int) * sd->status.size(), cudaMemcpyDeviceToHost,
                                   h->stream),
                   "swath decode status");
        check_cuda(cudaStreamSynchronize(h->stream), "swath decode");
        slot = sd;
    }
    const SwathDecode& sd = *slot;
    auto it = sd.burst_of_first.find(pk.front());
    if (it == sd.burst_of_first.end()) return nullptr;
    const size_t k = it->second;
    if (bit->second[k] != pk) return nullptr;
    for (size_t i = 0; i < pk.size(); ++i)
        if (sd.status[sd.job0[k] + i]) return nullptr;
    return (const cf32*)sd.raw.p + sd.plan->raw_off[k];
}
}  // namespace s1g
}  // extern "C++"

// Enqueue a whole batch without host synchronisation: the other streams fork
// from h0's stream and join back into it at the end (so the batch can also be
// captured into a CUDA graph from h0's stream).
static void enqueue_batch(s1g_decoder** hs, int n_streams, const char* swath, int level, BatchRun& br) {
    s1g_decoder* h0 = hs[0];
    const bool tops = tops_for(swath);
    // the bursts each stream processes (IW azimuth products skip < 1000 lines)
    std::vector<std::vector<const std::vector<int>*>> lists(n_streams);
    for (int s = 0; s < n_streams; ++s) {
        auto it = hs[s]->bursts.find(swath);
        if (it == hs[s]->bursts.end()) throw S1Error(S1G_E_BAD_SWATH, std::string("swath ") + swath + " not in data");
        for (size_t k = 0; k < it->second.size(); ++k) {
            const auto& pk = it->second[k];
            if (level == S1G_AZIMUTH_COMPRESSED && is_iw(swath) && pk.size() < 1000) continue;
            if (hs[s]->batch_sel_on &&
                std::find(hs[s]->batch_sel.begin(), hs[s]->batch_sel.end(), (int)k) == hs[s]->batch_sel.end())
                continue;
            lists[s].push_back(&pk);
        }
    }
    cudaEvent_t fork;
    check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "fork event");
    check_cuda(cudaEventRecord(fork, h0->stream), "fork");
    for (int s = 1; s < n_streams; ++s) check_cuda(cudaStreamWaitEvent(hs[s]->stream, fork, 0), "fork wait");
    // per stream: re-index the device-resident byte stream (the first step of
    // the path), then decode all its bursts in one launch pair (fused FP32 path)
    br.dec.assign(n_streams, nullptr);
    br.dec_status.assign(n_streams, nullptr);
    std::vector<cf32*> raw_all(n_streams, nullptr);
    std::vector<cf64*> raw64_all(n_streams, nullptr);
    for (int s = 0; s < n_streams; ++s) {
        s1g_decoder* h = hs[s];
        h->mark("index");
        index_packets(h->d_stream, h->nbytes, h->d_off, h->npk, h->isc, h->stream, false, nullptr);
        if (h->precision != S1G_PREC_FP32 || lists[s].empty()) continue;
        h->mark("batch_decode");
        std::string key = std::string(swath) + "/" + std::to_string(level);
        if (h->batch_sel_on)
            for (int b : h->batch_sel) key += ":" + std::to_string(b);
        auto& bd = h->batch_decodes[key];
        if (!bd) bd = batch_decode_plan(h, lists[s]);
        br.dec[s] = bd;
        raw_all[s] = h->bRawAll.as<cf32>((size_t)bd->raw_elems);
        br.dec_status[s] = h->bDecStatus.as<int>((size_t)bd->njobs);
        if (bd->any_d)
            decode_jobs<float>(h->d_stream, h->nbytes, h->d_off, bd->d_jobs, bd->njobs, bd->sym_bytes, bd->blk_bytes,
                               raw_all[s], br.dec_status[s], h->dsc, h->tabs, h->stream);
        if (bd->any_fixed)
            decode_fixed_jobs<float>(h->d_stream, h->nbytes, h->d_off, bd->d_jobs, bd->njobs, raw_all[s],
                                     br.dec_status[s], h->abc_fields, h->stream);
        if (h->use_eccm) {
            // FP64 samples for the notch from the same symbols (no second bit walk)
            raw64_all[s] = h->bRawAll64.as<cf64>((size_t)bd->raw_elems);
            if (bd->any_d) decode_jobs_values<double>(bd->d_jobs, bd->njobs, raw64_all[s], br.dec_status[s], h->dsc,
                                                      h->stream);
            if (bd->any_fixed)
                decode_fixed_jobs<double>(h->d_stream, h->nbytes, h->d_off, bd->d_jobs, bd->njobs, raw64_all[s],
                                          br.dec_status[s], h->abc_fields, h->stream);
        }
    }
    // burst products, enqueued round-robin over the streams so that they overlap
    size_t nslots = 0;
    for (int s = 0; s < n_streams; ++s) nslots += lists[s].size();
    br.nslots = nslots;
    br.tstat = h0->bBatchStatus.as<int>(std::max<size_t>(nslots, 1));
    check_cuda(cudaMemsetAsync(br.tstat, 0, sizeof(int) * std::max<size_t>(nslots, 1), h0->stream), "batch status");
    cudaEvent_t ready;
    check_cuda(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), "ready event");
    check_cuda(cudaEventRecord(ready, h0->stream), "ready");
    for (int s = 1; s < n_streams; ++s) check_cuda(cudaStreamWaitEvent(hs[s]->stream, ready, 0), "ready wait");
    if (!h0->batch_host.empty()) check_cuda(cudaStreamWaitEvent(h0->copy_stream, ready, 0), "copy fork");
    std::vector<std::vector<size_t>> slot_of(n_streams);
    size_t slot = 0;
    for (int s = 0; s < n_streams; ++s)
        for (size_t k = 0; k < lists[s].size(); ++k) slot_of[s].push_back(slot++);
    for (size_t i = h0->batch_bufs.size(); i < nslots; ++i) h0->batch_bufs.emplace_back(new Buf());
    h0->batch_out.assign(nslots, Result());
    size_t kmax = 0;
    for (int s = 0; s < n_streams; ++s) kmax = std::max(kmax, lists[s].size());
    long long total = 0;
    for (size_t k = 0; k < kmax; ++k) {
        for (int s = 0; s < n_streams; ++s) {
            if (k >= lists[s].size()) continue;
            s1g_decoder* h = hs[s];
            const std::vector<int>& pk = *lists[s][k];
            const size_t sl = slot_of[s][k];
            Result r;
            if (h->precision == S1G_PREC_FP32) {
                FastPipe fp(h);
                fp.predecoded = raw_all[s] ? raw_all[s] + br.dec[s]->raw_off[k] : nullptr;
                fp.predecoded64 = raw64_all[s] ? raw64_all[s] + br.dec[s]->raw_off[k] : nullptr;
                fp.tufr_status = br.tstat + sl;
                if (level == S1G_AZIMUTH_COMPRESSED && tops) {
                    auto fb = fp.prepare(pk, true);
                    fp.final_out = (cf32*)h0->batch_bufs[sl]->get((size_t)fb->n_out * fb->g.n_r * sizeof(cf32));
                }
                r = fp.run(pk, level, tops);
            } else if (h->precision == S1G_PREC_FP64) {
                r = Pipe<double>(h).run(pk, level, tops);
            } else {
                r = Pipe<float>(h).run(pk, level, tops);
            }
            const size_t esz = r.elem == S1G_CF32 ? 8 : 16;
            void* dst = h0->batch_bufs[sl]->get((size_t)r.rows * r.pitch * esz);
            if (dst != r.ptr)
                check_cuda(cudaMemcpyAsync(dst, r.ptr, (size_t)r.rows * r.pitch * esz, cudaMemcpyDeviceToDevice,
                                           h->stream), "batch copy");
            Result c = r;
            c.ptr = dst;
            c.status = nullptr;
            h0->batch_out[sl] = c;
            if (sl < h0->batch_host.size() && h0->batch_host[sl]) {
                // copy this burst to its host destination on the copy stream
                // while the next bursts compute
                check_cuda(cudaEventRecord(h0->slot_done[sl], h->stream), "slot done");
                check_cuda(cudaStreamWaitEvent(h0->copy_stream, h0->slot_done[sl], 0), "copy wait");
                check_cuda(cudaMemcpyAsync(h0->batch_host[sl], dst, (size_t)r.rows * r.pitch * esz,
                                           cudaMemcpyDeviceToHost, h0->copy_stream),
                           "batch host copy");
            }
            total += (long long)pk.size() * 2 * h->hdr[pk.front()].num_quads();
        }
    }
    br.total = total;
    if (!h0->batch_host.empty()) {
        cudaEvent_t e;
        check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy join event");
        check_cuda(cudaEventRecord(e, h0->copy_stream), "copy join");
        check_cuda(cudaStreamWaitEvent(h0->stream, e, 0), "copy join wait");
        cudaEventDestroy(e);
    }
    // join back into h0's stream
    for (int s = 1; s < n_streams; ++s) {
        cudaEvent_t e;
        check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "join event");
        check_cuda(cudaEventRecord(e, hs[s]->stream), "join");
        check_cuda(cudaStreamWaitEvent(h0->stream, e, 0), "join wait");
        cudaEventDestroy(e);
    }
    cudaEventDestroy(fork);
    cudaEventDestroy(ready);
}

// Deferred checks once a batch has run: decode status per packet, time-unfolding status per burst.
static void check_batch(const BatchRun& br, int n_streams) {
    for (int s = 0; s < n_streams; ++s) {
        if (!br.dec[s]) continue;
        std::vector<int> st(br.dec[s]->njobs);
        check_cuda(cudaMemcpy(st.data(), br.dec_status[s], sizeof(int) * st.size(), cudaMemcpyDeviceToHost),
                   "decode status");
        for (size_t i = 0; i < st.size(); ++i)
            if (st[i]) throw S1Error(st[i], decode_error_text(st[i], br.dec[s]->pk[i]));
    }
    std::vector<int> ts(std::max<size_t>(br.nslots, 1));
    check_cuda(cudaMemcpy(ts.data(), br.tstat, sizeof(int) * ts.size(), cudaMemcpyDeviceToHost), "batch status");
    for (size_t i = 0; i < br.nslots; ++i)
        if (ts[i]) throw S1Error(S1G_E_GEOMETRY, "azimuth time unfolding parameters out of range");
    if (tma_take_error() != 0) throw S1Error(S1G_E_TIMEOUT, "a TMA corner turn gave up waiting for its tile");
}

// A batch captured into a CUDA graph (second call with the same handles,
// swath, level and settings; the first call runs eagerly and leaves every
// buffer and table at its final size).
struct BatchGraph {
    std::string key;
    cudaGraphExec_t exec = nullptr;
    BatchRun run;
    std::vector<Result> out;
    long long kernels = 0;
    ~BatchGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

static std::string batch_key(s1g_decoder** hs, int n, const char* swath, int level) {
    std::ostringstream o;
    o << swath << "/" << level;
    for (int s = 0; s < n; ++s)
        o << "/" << (const void*)hs[s] << ":" << hs[s]->precision << ":" << hs[s]->use_eccm << ":" << hs[s]->det << ":"
          << hs[s]->mit << ":" << hs[s]->abc_fields << ":" << hs[s]->epoch << ":" << hs[s]->rcmc << ":"
          << hs[s]->rcmc_L;
    for (int s = 0; s < n; ++s) {
        o << "/sel" << s << (hs[s]->batch_sel_on ? ":" : "-");
        for (int b : hs[s]->batch_sel) o << b << ",";
    }
    o << "/host";
    for (void* p : hs[0]->batch_host) o << ":" << p;
    return o.str();
}

int s1g_process_swath_batch(s1g_decoder** hs, int n_streams, const char* swath, int level, int64_t* samples) {
    if (!hs || n_streams < 1 || !hs[0] || !swath || !samples || !level_ok(level)) return S1G_E_INVALID_ARGUMENT;
    for (int s = 0; s < n_streams; ++s)
        if (!hs[s]) return S1G_E_INVALID_ARGUMENT;
    s1g_decoder* h0 = hs[0];
    try {
        bool timing = false;
        for (int s = 0; s < n_streams; ++s) {
            for (auto& m : hs[s]->marks) cudaEventDestroy(m.second);
            hs[s]->marks.clear();
            timing = timing || hs[s]->stage_timing;
        }
        for (int s = 0; s < n_streams; ++s)
            if (!hs[s]->bursts.count(swath)) return S1G_E_BAD_SWATH;
        const std::string key = batch_key(hs, n_streams, swath, level);
        // only the FP32 fused pipeline enqueues without host synchronisation
        // (the plain pipelines read the decode status back per burst)
        bool graph = h0->use_graph && !timing;
        for (int s = 0; s < n_streams; ++s)
            if (hs[s]->precision != S1G_PREC_FP32) graph = false;
        cudaEvent_t b0, b1;
        check_cuda(cudaEventCreate(&b0), "event");
        check_cuda(cudaEventCreate(&b1), "event");
        const BatchRun* run = nullptr;
        BatchRun eager;
        if (graph && h0->graph && h0->graph->key == key) {
            // replay
            check_cuda(cudaEventRecord(b0, h0->stream), "b0");
            check_cuda(cudaGraphLaunch(h0->graph->exec, h0->stream), "graph launch");
            check_cuda(cudaEventRecord(b1, h0->stream), "b1");
            note_launches(h0->graph->kernels);
            h0->batch_out = h0->graph->out;
            run = &h0->graph->run;
        } else if (graph && h0->graph_warm == key) {
            // capture the enqueue sequence, then launch it
            auto g = std::make_unique<BatchGraph>();
            g->key = key;
            const long long l0 = launch_count();
            check_cuda(cudaStreamBeginCapture(h0->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            cudaGraph_t cg = nullptr;
            try {
                enqueue_batch(hs, n_streams, swath, level, g->run);
            } catch (...) {
                cudaStreamEndCapture(h0->stream, &cg);
                if (cg) cudaGraphDestroy(cg);
                throw;
            }
            check_cuda(cudaStreamEndCapture(h0->stream, &cg), "end capture");
            g->kernels = launch_count() - l0;
            note_launches(-g->kernels);
            check_cuda(cudaGraphInstantiate(&g->exec, cg, 0), "graph instantiate");
            cudaGraphDestroy(cg);
            g->out = h0->batch_out;
            h0->graph = std::move(g);
            check_cuda(cudaEventRecord(b0, h0->stream), "b0");
            check_cuda(cudaGraphLaunch(h0->graph->exec, h0->stream), "graph launch");
            check_cuda(cudaEventRecord(b1, h0->stream), "b1");
            note_launches(h0->graph->kernels);
            run = &h0->graph->run;
        } else {
            check_cuda(cudaEventRecord(b0, h0->stream), "b0");
            enqueue_batch(hs, n_streams, swath, level, eager);
            check_cuda(cudaEventRecord(b1, h0->stream), "b1");
            run = &eager;
            if (graph) h0->graph_warm = key;
        }
        check_cuda(cudaEventSynchronize(b1), "batch end");
        float ms = 0;
        cudaEventElapsedTime(&ms, b0, b1);
        h0->last_ms = ms;
        cudaEventDestroy(b0);
        cudaEventDestroy(b1);
        for (int s = 0; s < n_streams; ++s) hs[s]->close_marks();
        check_cuda(cudaGetLastError(), "batch kernels");
        check_batch(*run, n_streams);
        *samples = run->total;
    } catch (const S1Error& e) {
        h0->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        h0->err = e.what();
        return S1G_E_CUDA;
    }
    return S1G_OK;
}

int s1g_batch_host_outputs(s1g_decoder* h, void* const* host, int n) {
    API_BEGIN(h)
    if (n < 0 || (n && !host)) return S1G_E_INVALID_ARGUMENT;
    for (int k = 0; k < n; ++k) {
        if (!host[k]) continue;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, host[k]) != cudaSuccess || at.type != cudaMemoryTypeHost) {
            cudaGetLastError();
            throw S1Error(S1G_E_INVALID_ARGUMENT, "batch host outputs must be page-locked host memory");
        }
    }
    if (n && !h->copy_stream)
        check_cuda(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "copy stream");
    for (int k = (int)h->slot_done.size(); k < n; ++k) {
        cudaEvent_t e;
        check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "slot event");
        h->slot_done.push_back(e);
    }
    h->batch_host.assign(host, host + n);
    API_END(h)
}

int s1g_set_rcmc(s1g_decoder* h, int mode, int half_width) {
    if (!h || (mode != S1G_RCMC_PHASE && mode != S1G_RCMC_SINC) || half_width < 1 || half_width > 16)
        return S1G_E_INVALID_ARGUMENT;
    h->rcmc = mode;
    h->rcmc_L = half_width;
    return S1G_OK;
}

int s1g_set_batch_bursts(s1g_decoder* h, const int* bursts, int n) {
    if (!h || (n > 0 && !bursts)) return S1G_E_INVALID_ARGUMENT;
    h->batch_sel.clear();
    h->batch_sel_on = n >= 0;
    for (int i = 0; i < n; ++i) {
        if (bursts[i] < 0) return S1G_E_INVALID_ARGUMENT;
        h->batch_sel.push_back(bursts[i]);
    }
    std::sort(h->batch_sel.begin(), h->batch_sel.end());
    h->batch_sel.erase(std::unique(h->batch_sel.begin(), h->batch_sel.end()), h->batch_sel.end());
    return S1G_OK;
}

int s1g_set_batch_graph(s1g_decoder* h, int on) {
    if (!h) return S1G_E_INVALID_ARGUMENT;
    h->use_graph = on != 0;
    h->graph.reset();
    h->graph_warm.clear();
    return S1G_OK;
}

int s1g_batch_output(s1g_decoder* h, int burst, const void** dev_ptr, int64_t* rows, int64_t* cols, int64_t* pitch,
                     int* elem_type) {
    if (!h || !dev_ptr || burst < 0 || burst >= (int)h->batch_out.size()) return S1G_E_INVALID_ARGUMENT;
    const Result& r = h->batch_out[burst];
    *dev_ptr = r.ptr;
    if (rows) *rows = r.rows;
    if (cols) *cols = r.cols;
    if (pitch) *pitch = r.pitch;
    if (elem_type) *elem_type = r.elem;
    return S1G_OK;
}

int s1g_last_timing(const s1g_decoder* h, double* ms, char* stages, size_t len) {
    if (!h || !ms) return S1G_E_INVALID_ARGUMENT;
    *ms = h->last_ms;
    if (stages && len) {
        std::ostringstream o;
        for (const auto& kv : h->stage_ms) o << kv.first << " " << kv.second << " " << h->stage_n.at(kv.first) << "\n";
        const std::string t = o.str();
        const size_t n = std::min(len - 1, t.size());
        memcpy(stages, t.data(), n);
        stages[n] = 0;
    }
    return S1G_OK;
}

int s1g_set_stage_timing(s1g_decoder* h, int on) {
    if (!h) return S1G_E_INVALID_ARGUMENT;
    h->stage_timing = on != 0;
    h->stage_ms.clear();
    h->stage_n.clear();
    return S1G_OK;
}

int s1g_launch_count(int64_t* n) {
    if (!n) return S1G_E_INVALID_ARGUMENT;
    *n = launch_count();
    return S1G_OK;
}

}  // extern "C"
