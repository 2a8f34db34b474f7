// Allocation-free FDBAQ decode entry point (s1g_decode_fdbaq_noalloc).
//
// Who needs it: callers that must not allocate device memory while they run
// -- a processing chain whose GPU memory budget is fixed when it starts (a
// ground-station or on-board style pipeline that reserves everything up
// front), or a host program that shares the device with latency-sensitive
// streams and cannot afford the device-wide synchronisation that cudaMalloc
// and cudaFree imply.  Such a caller allocates its inputs and outputs itself,
// once, and then decodes packets with this call, which allocates nothing.
//
// The decoder's working memory (one byte per decoded sample plus the
// per-block BRC / THIDX codes) lives in the file-scope array below, 16 MiB,
// which every GPU that loads the library keeps until the process exits.
// Longer inputs are decoded in chunks that fit it.  Host code may not use the
// array's name as a device address (it is only a host-side stand-in), so the
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, and passed to the kernels.
#include <cstring>
#include <mutex>
#include <string>

#include "s1g_kernels.h"

namespace s1g {

size_t huffman_lut_bytes();
void huffman_lut_fill(void* host_dst);
void decode_fp32_with_scratch(const uint8_t* d_stream, long long n, const long long* d_offsets, int p0, int npk,
                              int nq, cf32* out, long long pitch, int* d_status, uint8_t* sym, uint8_t* brc,
                              uint8_t* thidx, const void* d_lut, cudaStream_t st);

constexpr size_t kNoAllocScratchBytes = 16u << 20;   // 16 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];
static __device__ __align__(256) uint8_t g_noalloc_lut[5 * 2048 * 2];   // 11-bit windows x 5 BRCs, 2 bytes each

struct NoAllocDevice {
    bool ready = false;
    uint8_t* scratch = nullptr;
    uint8_t* lut = nullptr;
};
static NoAllocDevice g_dev[kMaxDevices];
static std::mutex g_setup_mutex;

// Once per device, with that device current: resolve the arrays' device
// addresses and copy the Huffman table in (a synchronous copy, no allocation).
static int setup_device(int dev, std::string& err) {
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    NoAllocDevice& d = g_dev[dev];
    if (d.ready) return S1G_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
        return S1G_E_CUDA;
    }
    d.scratch = (uint8_t*)p;
    e = cudaGetSymbolAddress(&p, g_noalloc_lut);
    if (e != cudaSuccess) {
        err = std::string("cudaGetSymbolAddress(lut): ") + cudaGetErrorString(e);
        return S1G_E_CUDA;
    }
    d.lut = (uint8_t*)p;
    if (huffman_lut_bytes() != sizeof(g_noalloc_lut)) {
        err = "Huffman table size mismatch";
        return S1G_E_CUDA;
    }
    uint8_t host[sizeof(g_noalloc_lut)];
    huffman_lut_fill(host);
    e = cudaMemcpyToSymbol(g_noalloc_lut, host, sizeof(host));
    if (e != cudaSuccess) {
        err = std::string("cudaMemcpyToSymbol(lut): ") + cudaGetErrorString(e);
        return S1G_E_CUDA;
    }
    d.ready = true;
    return S1G_OK;
}

}  // namespace s1g

using namespace s1g;

extern "C" {

int s1g_decode_fdbaq_noalloc(const uint8_t* d_stream, int64_t nbytes, const int64_t* d_offsets, int64_t npackets,
                             int num_quads, void* d_out, int64_t out_pitch, int32_t* d_status, void* stream) {
    if (!d_stream || !d_offsets || !d_out || !d_status || npackets < 0 || nbytes < 0) return S1G_E_INVALID_ARGUMENT;
    // num_quadratures is a 16-bit packet field
    if (num_quads <= 0 || num_quads > 65535 || out_pitch < 2LL * num_quads) return S1G_E_INVALID_ARGUMENT;
    const long long nb = (2LL * num_quads + 255) / 256;
    const long long per_packet = 4LL * ((num_quads + 3LL) & ~3LL) + 2 * nb;   // symbol rows + BRC + THIDX
    if (per_packet > (long long)kNoAllocScratchBytes) return S1G_E_SCRATCH_LIMIT;
    if (npackets == 0) return S1G_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return S1G_E_CUDA;
    std::string err;
    int rc = setup_device(dev, err);
    if (rc != S1G_OK) return rc;
    const NoAllocDevice& d = g_dev[dev];
    cudaStream_t st = (cudaStream_t)stream;
    // chunks of packets that fit the scratch array; stream order keeps the
    // chunks (and successive calls on one stream) from overlapping
    const long long chunk = std::min<long long>(npackets, (long long)kNoAllocScratchBytes / per_packet);
    for (long long p0 = 0; p0 < npackets; p0 += chunk) {
        const int n = (int)std::min(chunk, npackets - p0);
        uint8_t* sym = d.scratch;
        uint8_t* brc = sym + (size_t)n * 4 * sym_pitch(num_quads);
        uint8_t* th = brc + (size_t)n * nb;
        decode_fp32_with_scratch(d_stream, nbytes, (const long long*)d_offsets, (int)p0, n, num_quads,
                                 (cf32*)d_out + p0 * out_pitch, out_pitch, d_status + p0, sym, brc, th, d.lut, st);
    }
    return cudaGetLastError() == cudaSuccess ? S1G_OK : S1G_E_CUDA;
}

}  // extern "C"
