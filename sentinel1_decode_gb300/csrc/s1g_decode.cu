// Packet indexer and FDBAQ (type D) decoder kernels.
//
// Indexer: the space-packet chain is sequential (next = cur + 7 +
// packet_data_length, packet.cpp:850-879), so the stream is cut into chunks
// and one warp per chunk finds the first packet start in its chunk (ballot
// over the secondary-header sync marker 0x352EF853 at byte 12 of a packet)
// and walks the chain to the chunk end.  A single block then checks that
// every chunk's speculative entry equals the previous chunk's exit (re-walking
// sequentially only where it does not), and exclusive-scans the per-chunk
// packet counts.  A last pass writes every packet offset at its global index.
//
// Decoder: one thread per packet reproduces the bitstream walk of
// _set_quad_type_d / _get_h_code_type_d / huffman_decode (packet.cpp:755-818,
// decoding_utils.cpp:44-77) with a 16-entry value-keyed lookup per BRC held
// in shared memory and a 64-bit bit buffer, storing one byte (sign<<7|mcode)
// per sample; a second, coalesced kernel applies the reconstruction of
// _get_s_values_type_d (packet.cpp:678-693) and the IE/IO/QE/QO interleave of
// _get_signal_type_d (packet.cpp:696-752).  Errors become per-packet status
// codes instead of exceptions.
#include <cstring>

#include "s1g_kernels.h"

namespace s1g {

// ------------------------------------------------------------------ tables
__constant__ double c_simple[5][17] = {
    {3.0000, 3.0000, 3.1600, 3.5300},
    {4.0000, 4.0000, 4.0800, 4.3700},
    {6.0000, 6.0000, 6.0000, 6.1500, 6.5000, 6.8800},
    {9.0000, 9.0000, 9.0000, 9.0000, 9.3600, 9.5000, 10.1000},
    {15.0000, 15.0000, 15.0000, 15.0000, 15.0000, 15.0000, 15.2200, 15.5000, 16.0600},
};
__constant__ double c_norm[5][16] = {
    {0.3637, 1.0915, 1.8208, 2.6406},
    {0.3042, 0.9127, 1.5216, 2.1313, 2.8426},
    {0.2305, 0.6916, 1.1528, 1.6140, 2.0754, 2.5369, 3.1191},
    {0.1702, 0.5107, 0.8511, 1.1916, 1.5321, 1.8726, 2.2131, 2.5536, 2.8942, 3.3744},
    {0.1130, 0.3389, 0.5649, 0.7908, 1.0167, 1.2428, 1.4687, 1.6947, 1.9206, 2.1466, 2.3725,
     2.5985, 2.8244, 3.0504, 3.2764, 3.6623},
};
__constant__ double c_sf[256] = {
    0.00, 0.63, 1.25, 1.88, 2.51, 3.13, 3.76, 4.39, 5.01, 5.64, 6.27, 6.89, 7.52, 8.15, 8.77,
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
    253.49, 254.74, 255.99,
};
__constant__ int c_brc_thidx[5] = {3, 3, 5, 6, 8};
__constant__ int c_brc_mcode[5] = {3, 4, 6, 9, 15};

// Huffman lookup: for BRC b and an 11-bit window w (MSB = next bit: the
// sign, then the 10 bits the code can take), the value-keyed walk of
// huffman_decode is resolved into the symbol byte sign<<7 | mcode (low byte)
// and the bits the sample takes, 1 + code length (high byte; 0 = "Max bit
// length exceeded").  The table is built on the host by running that walk on
// every window.
typedef uint16_t HuffEntry;
constexpr int kHuffWindow = 2048;

// ------------------------------------------------------------------ indexer
constexpr uint32_t kSync = 0x352EF853u;

__device__ __forceinline__ bool is_packet_start(const uint8_t* s, long long n, long long p) {
    if (p + 68 > n) return false;
    const uint8_t b0 = s[p];
    if ((b0 >> 5) != 0) return false;          // packet version 0
    if (((b0 >> 3) & 1) != 1) return false;    // secondary header flag
    const uint32_t sync = ((uint32_t)s[p + 12] << 24) | ((uint32_t)s[p + 13] << 16) |
                          ((uint32_t)s[p + 14] << 8) | (uint32_t)s[p + 15];
    return sync == kSync;
}

__device__ __forceinline__ long long packet_next(const uint8_t* s, long long p) {
    const uint32_t pdl = ((uint32_t)s[p + 4] << 8) | s[p + 5];
    return p + 7 + (long long)pdl;
}

// One warp per chunk: entry = first position in [chunk begin, chunk end) that
// looks like a packet start (or -1); the walk from there counts chain
// positions p with p < chunk end and p + 6 <= n (the reference stops when a
// 6-byte primary header can no longer be read); exit = where the walk left.
__global__ void k_index_chunks(const uint8_t* __restrict__ s, long long n, long long chunk, int nchunks,
                               long long* __restrict__ entry, long long* __restrict__ exitp, int* __restrict__ count) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nchunks) return;
    const long long c0 = (long long)warp * chunk;
    const long long c1 = min(n, c0 + chunk);
    long long found = -1;
    for (long long base = c0; base < c1 && found < 0; base += 32) {
        const long long p = base + lane;
        const bool hit = p < c1 && is_packet_start(s, n, p);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (m) found = base + __ffs(m) - 1;
    }
    if (lane == 0) {
        int cnt = 0;
        long long p = found;
        if (found >= 0) {
            while (p < c1 && p + 6 <= n) {
                ++cnt;
                p = packet_next(s, p);
            }
        }
        entry[warp] = found;
        count[warp] = cnt;
        exitp[warp] = p;
    }
}

// Block-wide inclusive scan helpers (1024 threads, one value per thread).
__device__ int block_scan_max(int v, int* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        const int t = threadIdx.x >= off ? sh[threadIdx.x - off] : -1;
        __syncthreads();
        sh[threadIdx.x] = max(sh[threadIdx.x], t);
        __syncthreads();
    }
    return sh[threadIdx.x];
}

__device__ int block_scan_sum(int v, int* sh) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        const int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    return sh[threadIdx.x];
}

// Single block of 1024 threads.  The chain reaches chunk k at T_k = exit of
// the last non-empty chunk before k (0 for the first).  Chunk k is consistent
// if the chain skips it and its walk found nothing, or if its speculative
// entry is T_k.  If every chunk is consistent the per-chunk counts are the
// chain's; otherwise thread 0 re-walks the chain sequentially.
__global__ void k_index_fix(const uint8_t* __restrict__ s, long long n, long long chunk, int nchunks,
                            long long* __restrict__ entry, long long* __restrict__ exitp, int* __restrict__ count,
                            int* __restrict__ base, int* __restrict__ total) {
    __shared__ int sh[1024];
    __shared__ int bad;
    const int per = (nchunks + blockDim.x - 1) / blockDim.x;
    const int k0 = threadIdx.x * per;
    const int k1 = min(nchunks, k0 + per);
    if (threadIdx.x == 0) bad = 0;
    // last non-empty chunk index at or before each position (segment-local, then block scan)
    int last = -1;
    for (int k = k0; k < k1; ++k)
        if (count[k] > 0) last = k;
    const int incl = block_scan_max(last, sh);
    int prev = (threadIdx.x > 0) ? sh[threadIdx.x - 1] : -1;
    (void)incl;
    __syncthreads();
    for (int k = k0; k < k1; ++k) {
        const long long T = (prev < 0) ? 0 : exitp[prev];
        const long long c1 = min(n, (long long)k * chunk + chunk);
        const bool ok = (T >= c1) ? (count[k] == 0) : (entry[k] == T);
        if (!ok) atomicAdd(&bad, 1);
        if (count[k] > 0) prev = k;
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) {
            long long p = 0;
            int acc = 0;
            for (int k = 0; k < nchunks; ++k) {
                const long long c1 = min(n, (long long)k * chunk + chunk);
                entry[k] = p;
                int cnt = 0;
                while (p < c1 && p + 6 <= n) {
                    ++cnt;
                    p = packet_next(s, p);
                }
                count[k] = cnt;
                exitp[k] = p;
                base[k] = acc;
                acc += cnt;
            }
            *total = acc;
        }
        return;
    }
    int local = 0;
    for (int k = k0; k < k1; ++k) local += count[k];
    const int inc = block_scan_sum(local, sh);
    int acc = inc - local;
    for (int k = k0; k < k1; ++k) {
        base[k] = acc;
        acc += count[k];
    }
    if (threadIdx.x == blockDim.x - 1) *total = inc;
}

__global__ void k_index_write(const uint8_t* __restrict__ s, long long n, long long chunk, int nchunks,
                              const long long* __restrict__ entry, const int* __restrict__ count,
                              const int* __restrict__ base, long long* __restrict__ offsets, int max_out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    long long p = entry[k];
    for (int i = 0; i < count[k]; ++i) {
        const int idx = base[k] + i;
        if (idx < max_out) offsets[idx] = p;
        p = packet_next(s, p);
    }
}

int index_packets(const uint8_t* d_stream, long long n, long long* d_offsets, int max_packets, IndexScratch& sc,
                  cudaStream_t st, bool sync_count, int* h_count) {
    const long long chunk = 1 << 14;
    const int nchunks = (int)((n + chunk - 1) / chunk);
    if (nchunks <= 0) {
        // an empty stream holds no packets; launch nothing (the scratch
        // arrays, the count word included, are not allocated for 0 chunks)
        if (h_count) *h_count = 0;
        return 0;
    }
    sc.reserve(nchunks);
    const int threads = 256;
    const int warps_per_block = threads / 32;
    note_launch(), k_index_chunks<<<(nchunks + warps_per_block - 1) / warps_per_block, threads, 0, st>>>(
        d_stream, n, chunk, nchunks, sc.entry, sc.exitp, sc.count);
    note_launch(), k_index_fix<<<1, 1024, 0, st>>>(d_stream, n, chunk, nchunks, sc.entry, sc.exitp, sc.count, sc.base, sc.total);
    note_launch(), k_index_write<<<(nchunks + 127) / 128, 128, 0, st>>>(d_stream, n, chunk, nchunks, sc.entry, sc.count, sc.base,
                                                         d_offsets, max_packets);
    if (sync_count && h_count) {
        check_cuda(cudaMemcpyAsync(h_count, sc.total, sizeof(int), cudaMemcpyDeviceToHost, st), "index count");
        check_cuda(cudaStreamSynchronize(st), "index sync");
        return *h_count;
    }
    return -1;
}

void IndexScratch::reserve(int nchunks) {
    if (nchunks <= cap) return;
    release();
    check_cuda(cudaMalloc(&entry, sizeof(long long) * nchunks), "index scratch");
    check_cuda(cudaMalloc(&exitp, sizeof(long long) * nchunks), "index scratch");
    check_cuda(cudaMalloc(&count, sizeof(int) * nchunks), "index scratch");
    check_cuda(cudaMalloc(&base, sizeof(int) * nchunks), "index scratch");
    check_cuda(cudaMalloc(&total, sizeof(int)), "index scratch");
    cap = nchunks;
}

void IndexScratch::release() {
    if (entry) cudaFree(entry);
    if (exitp) cudaFree(exitp);
    if (count) cudaFree(count);
    if (base) cudaFree(base);
    if (total) cudaFree(total);
    entry = exitp = nullptr;
    count = base = total = nullptr;
    cap = 0;
}

// Gather the 68 header bytes of each packet (for host-side segmentation).
__global__ void k_gather_headers(const uint8_t* __restrict__ s, long long n, const long long* __restrict__ off,
                                 int npk, uint8_t* __restrict__ hdr) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)npk * 68) return;
    const int p = (int)(i / 68), b = (int)(i % 68);
    const long long at = off[p] + b;
    hdr[i] = at < n ? s[at] : 0;
}

void gather_headers(const uint8_t* d_stream, long long n, const long long* d_off, int npk, uint8_t* d_hdr,
                    cudaStream_t st) {
    const long long tot = (long long)npk * 68;
    if (tot == 0) return;
    note_launch(), k_gather_headers<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(d_stream, n, d_off, npk, d_hdr);
}

// ------------------------------------------------------------------ decoder
// Bit reader over one packet's user data: a 64-bit MSB-first buffer refilled
// with big-endian 32-bit words.  The data's aligned 32-bit words stream
// through an 8-slot ring in shared memory (one column per thread) by
// asynchronous copies (cp.async): a refill assembles the next word from the
// ring (funnel shift by the data's constant misalignment, byte swap) and
// starts the copy of the word six ahead, so a copy has five refills to land
// and no register ever waits on a global load.  Only aligned words that end
// inside the data are copied (the first may start up to 3 bytes before u,
// inside the packet header), and the words within 8 bytes of the end are
// assembled byte by byte, bytes beyond `avail` read as zero: nothing past the
// data is read, so a caller's unpadded buffer is safe.
constexpr int kDecodeThreads = 128;
constexpr int kRing = 8;

struct BitBuf {
    const uint8_t* u;
    int avail;
    int pos;                // byte position of the next word to enter buf
    uint64_t buf;           // unread bits, MSB first
    int nb;                 // number of valid bits in buf
    int sh;                 // misalignment of u, in bits
    int k;                  // aligned word holding byte pos (from wbase)
    const uint32_t* wbase;  // aligned word holding byte 0
    const uint32_t* ring;   // this thread's column: slot s at ring[s * kDecodeThreads]
};

__device__ __forceinline__ uint32_t load_be32(const uint8_t* u, long long pos, long long avail) {
    uint32_t v = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) v = (v << 8) | (pos + i < avail ? (uint32_t)u[pos + i] : 0u);
    return v;
}

// start the copy of aligned word kw into its ring slot (one commit group per
// word, empty past the end, so the group count stays one per word)
__device__ __forceinline__ void bb_copy(const BitBuf& b, int kw) {
    const uint32_t* g = b.wbase + kw;
    if (reinterpret_cast<const uint8_t*>(g + 1) <= b.u + b.avail) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(b.ring + (kw & (kRing - 1)) * kDecodeThreads);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(g) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ BitBuf bb_open(const uint8_t* u, int avail, const uint32_t* ring) {
    BitBuf b;
    b.u = u;
    b.avail = avail;
    b.pos = 0;
    b.buf = 0ull;
    b.nb = 0;
    b.sh = (int)((uintptr_t)u & 3) * 8;
    b.k = 0;
    b.wbase = reinterpret_cast<const uint32_t*>((uintptr_t)u & ~(uintptr_t)3);
    b.ring = ring;
#pragma unroll
    for (int kw = 0; kw < 6; ++kw) bb_copy(b, kw);
    return b;
}

// at least 32 unread bits in buf afterwards
__device__ __forceinline__ void bb_refill(BitBuf& b) {
    if (b.nb <= 32) {
        // words k and k + 1 are in: at most the four younger copies pending
        asm volatile("cp.async.wait_group 4;" ::: "memory");
        uint32_t nx;
        if (b.pos + 8 <= b.avail) {
            const uint32_t lo = b.ring[(b.k & (kRing - 1)) * kDecodeThreads];
            const uint32_t hi = b.ring[((b.k + 1) & (kRing - 1)) * kDecodeThreads];
            nx = __byte_perm(__funnelshift_r(lo, hi, b.sh), 0, 0x0123);
        } else {
            nx = load_be32(b.u, b.pos, b.avail);
        }
        b.buf |= (uint64_t)nx << (32 - b.nb);
        b.pos += 4;
        b.nb += 32;
        bb_copy(b, b.k + 6);   // into the slot of word k - 2, already consumed
        ++b.k;
    }
}
__device__ __forceinline__ uint32_t bb_top32(const BitBuf& b) { return (uint32_t)(b.buf >> 32); }
__device__ __forceinline__ void bb_skip(BitBuf& b, int k) {
    b.buf <<= k;
    b.nb -= k;
}

// Where packet j of a decode goes.  Job-table mode (jobs != nullptr): any mix
// of bursts and row lengths in one launch.  Uniform mode: packets p0 + j (or
// pk_idx[j]) of one burst, nq quads each, rows j * pitch.
struct DecodeSpec {
    const DecodeJob* jobs;
    int njobs;
    const int* pk_idx;
    int p0;
    int nq;
    long long pitch;
};

__device__ __forceinline__ DecodeJob job_at(const DecodeSpec& d, int j) {
    if (d.jobs) return d.jobs[j];
    DecodeJob o;
    o.pk = d.pk_idx ? d.pk_idx[j] : d.p0 + j;
    o.nq = d.nq;
    const int nb = (2 * d.nq + 255) / 256;
    o.sym = (long long)j * 4 * sym_pitch(d.nq);
    o.blk = (long long)j * nb;
    o.out = (long long)j * d.pitch;
    return o;
}

// Symbols: one byte per sample, sign<<7 | mcode; rows ch = IE, IO, QE, QO of
// sym_pitch(nq) bytes each at job.sym.  The walk reproduces _set_quad_type_d /
// _get_h_code_type_d / huffman_decode (packet.cpp:755-818,
// decoding_utils.cpp:44-77): per channel, blocks of 128 codes (IE blocks led
// by the 3-bit BRC, QE blocks by the 8-bit THIDX), then a 16-bit alignment.
__global__ void __launch_bounds__(kDecodeThreads) k_decode_symbols(const uint8_t* __restrict__ s, long long n,
                                                        const long long* __restrict__ offsets, DecodeSpec spec,
                                                        uint8_t* __restrict__ sym, uint8_t* __restrict__ brc_out,
                                                        uint8_t* __restrict__ thidx_out, int* __restrict__ status,
                                                        const HuffEntry* __restrict__ lut_g) {
    __shared__ HuffEntry lut[5 * kHuffWindow];
    __shared__ uint32_t ring[kRing * kDecodeThreads];
    for (int i = threadIdx.x; i < 5 * kHuffWindow; i += blockDim.x) lut[i] = lut_g[i];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= spec.njobs) return;
    const DecodeJob jb = job_at(spec, j);
    const int nq = jb.nq;
    const long long off = offsets[jb.pk];
    // the 68 header bytes must lie inside the stream before any is read
    // (offsets can come from the caller, not only from the indexer)
    if (off < 0 || off > n - 68) {
        status[j] = S1G_E_PACKET_LENGTH;
        return;
    }
    const uint8_t* hdr = s + off;
    const long long pdl = ((long long)hdr[4] << 8) | hdr[5];
    const long long ulen = pdl + 1 - 62;
    // bytes actually present (a truncated last packet reads as zeros)
    long long avail = n - (off + 68);
    if (avail > ulen) avail = ulen;
    if (avail < 0) avail = 0;
    const int pnq = (hdr[6 + 59] << 8) | hdr[6 + 60];
    int st = 0;
    if (ulen < 0) st = S1G_E_PACKET_LENGTH;
    else if (pnq != nq) st = S1G_E_RAGGED_BURST;
    const int nb = (2 * nq + 255) / 256;
    const int sp = sym_pitch(nq);
    uint8_t* my_sym = sym + jb.sym;
    uint8_t* my_brc = brc_out + jb.blk;
    uint8_t* my_th = thidx_out + jb.blk;
    BitBuf bb = bb_open(s + off + 68, (int)avail, ring + threadIdx.x);
    int bit = 0;                               // user data: below 65536 bytes
    const int ubits = (int)ulen * 8;
    for (int ch = 0; ch < 4 && !st; ++ch) {
        uint32_t* row = reinterpret_cast<uint32_t*>(my_sym + (long long)ch * sp);
        // the BRCs of channels IO, QE, QO come back from the IE walk's stores,
        // each read one block ahead of its use
        int brc_next = ch > 0 ? my_brc[0] : 0;
        for (int b = 0; b < nb && !st; ++b) {
            bb_refill(bb);
            int brc;
            if (ch == 0) {
                if (bit + 3 > ubits) { st = S1G_E_READ_PAST_END; break; }
                const uint32_t v = bb_top32(bb) >> 29;
                if (v > 4) { st = S1G_E_BAD_BRC; break; }
                my_brc[b] = (uint8_t)v;
                brc = (int)v;
                bb_skip(bb, 3);
                bit += 3;
            } else {
                brc = brc_next;
                brc_next = my_brc[min(b + 1, nb - 1)];
                if (ch == 2) {
                    if (bit + 8 > ubits) { st = S1G_E_READ_PAST_END; break; }
                    my_th[b] = (uint8_t)(bb_top32(bb) >> 24);
                    bb_skip(bb, 8);
                    bit += 8;
                }
            }
            const HuffEntry* L = lut + brc * kHuffWindow;
            const int cnt = (b == nb - 1) ? nq - 128 * (nb - 1) : 128;
            uint32_t pack = 0;
            int i = 0;
            if (bit + 11 * cnt <= ubits) {
                // every code of the block ends inside the user data: no
                // per-sample bounds checks, and an invalid code (0 bits) is
                // reported after the block.  Four samples per step with two
                // refills: after a refill at least 32 bits are buffered, two
                // samples take at most 22.
                uint32_t ok = 1;
                for (; i + 4 <= cnt; i += 4) {
                    bb_refill(bb);
                    const uint32_t e0 = L[bb_top32(bb) >> 21];
                    bb_skip(bb, (int)(e0 >> 8));
                    const uint32_t e1 = L[bb_top32(bb) >> 21];
                    bb_skip(bb, (int)(e1 >> 8));
                    bb_refill(bb);
                    const uint32_t e2 = L[bb_top32(bb) >> 21];
                    bb_skip(bb, (int)(e2 >> 8));
                    const uint32_t e3 = L[bb_top32(bb) >> 21];
                    bb_skip(bb, (int)(e3 >> 8));
                    ok &= (uint32_t)((e0 >> 8) != 0) & (uint32_t)((e1 >> 8) != 0) & (uint32_t)((e2 >> 8) != 0) &
                          (uint32_t)((e3 >> 8) != 0);
                    bit += (int)((e0 >> 8) + (e1 >> 8) + (e2 >> 8) + (e3 >> 8));
                    row[(128 * b + i) >> 2] = __byte_perm(__byte_perm(e0, e1, 0x0040), __byte_perm(e2, e3, 0x0040), 0x5410);
                }
                for (; i < cnt; ++i) {
                    bb_refill(bb);
                    const uint32_t e = L[bb_top32(bb) >> 21];
                    bb_skip(bb, (int)(e >> 8));
                    ok &= (uint32_t)((e >> 8) != 0);
                    bit += (int)(e >> 8);
                    pack |= (e & 0xffu) << (8 * (i & 3));
                }
                if (!ok) st = S1G_E_HUFFMAN;
            } else {
                for (; i < cnt; ++i) {
                    bb_refill(bb);
                    const uint32_t e = L[bb_top32(bb) >> 21];
                    const int k = (int)(e >> 8);
                    if (k == 0) { st = S1G_E_HUFFMAN; break; }
                    // the reference reads the code's bits one width at a time, all
                    // inside the user data (decoding_utils.cpp:107-119)
                    if (bit + k > ubits) { st = S1G_E_READ_PAST_END; break; }
                    pack |= (e & 0xffu) << (8 * (i & 3));
                    if ((i & 3) == 3) {
                        row[(128 * b + i) >> 2] = pack;
                        pack = 0;
                    }
                    bb_skip(bb, k);
                    bit += k;
                }
            }
            if (!st && (i & 3)) row[(128 * b + i) >> 2] = pack;   // tail word (row padded to 4 bytes)
        }
        const int r = (int)(bit & 15);
        if (r) {
            bb_refill(bb);
            bb_skip(bb, 16 - r);
            bit += 16 - r;
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");   // no copy outlives the walk
    status[j] = st;
}

// Reconstruction + interleave, one block per packet: out[2k] = IE_k + i QE_k,
// out[2k+1] = IO_k + i QO_k (_get_s_values_type_d / _get_signal_type_d,
// packet.cpp:678-752).  A packet that failed (here or in the symbol walk)
// gets a zero row.
template <typename R>
__global__ void __launch_bounds__(256) k_decode_values(const uint8_t* __restrict__ sym, const uint8_t* __restrict__ brc_g,
                                                       const uint8_t* __restrict__ th_g, DecodeSpec spec,
                                                       cpx<R>* __restrict__ out, int* __restrict__ status) {
    __shared__ int bad;
    const int j = blockIdx.x;
    const DecodeJob jb = job_at(spec, j);
    const int nq = jb.nq;
    const int sp = sym_pitch(nq);
    cpx<R>* row = out + jb.out;
    if (threadIdx.x == 0) bad = status[j];
    __syncthreads();
    if (bad == 0) {
        const uint8_t* sj = sym + jb.sym;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int b = q >> 7;
            const int brc = brc_g[jb.blk + b];
            const int th = th_g[jb.blk + b];
            double v[4];
            bool err = false;
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) {
                const uint8_t c = sj[(long long)ch * sp + q];
                const int m = c & 127;
                const double sg = (c >> 7) ? -1.0 : 1.0;
                if (th <= c_brc_thidx[brc]) {
                    const int flag = c_brc_mcode[brc];
                    if (m < flag) v[ch] = sg * (double)m;
                    else if (m == flag) v[ch] = sg * c_simple[brc][th];
                    else { v[ch] = 0.0; err = true; }
                } else {
                    v[ch] = sg * c_norm[brc][m] * c_sf[th];
                }
            }
            if (err) atomicExch(&bad, S1G_E_MCODE);
            row[2 * q] = mk((R)v[0], (R)v[2]);
            row[2 * q + 1] = mk((R)v[1], (R)v[3]);
        }
        __syncthreads();
        if (bad != 0 && threadIdx.x == 0) status[j] = bad;
    }
    if (bad != 0)
        for (int k = threadIdx.x; k < 2 * nq; k += blockDim.x) row[k] = mk((R)0, (R)0);
}

// ------------------------------------------------------------------ formats A, B, C
// Bypass (formats A/B, baq_mode 0) and BAQ (format C, baq_mode 3/4/5)
// packets have fixed-length fields, so every sample is found by arithmetic:
// one block per packet, one thread per quad.
//   A/B: channel c (IE, IO, QE, QO) at c * W, W = 10 nq rounded up to 16;
//        sample q = sign bit + 9-bit magnitude at 10 q (packet.cpp:519-538).
//   C:   sample = sign bit + (M-1)-bit code, M = baq_mode, in blocks of 128
//        quads; every QE block starts with an 8-bit THIDX; channels padded to
//        16 bits (packet.cpp:622-666); reconstruction _get_s_values_type_c
//        (packet.cpp:548-564) with the BAQ rows of the tables.
// With `fields` == 0 the output is the reference's: its decoders append the
// codes to containers that already hold zero entries (H_CODE() with 128,
// H_CODE(n) with n, QUAD(key, n) with n default blocks) and then read the
// leading entries, so for A/B quad q carries the codes of quad q - 128 (zero
// below 128) and for C every sample of a block is the reconstruction of
// sign 0, code 0 at that block's THIDX.  With `fields` == 1 every sample is
// decoded from its own bits.  Either way the packet must hold every bit the
// reference reads, else S1G_E_READ_PAST_END.  FDBAQ rows are left alone.
__constant__ double c_baq_simple[3][17] = {
    {3.00, 3.00, 3.12, 3.55},
    {7.00, 7.00, 7.00, 7.17, 7.40, 7.76},
    {15.00, 15.00, 15.00, 15.00, 15.00, 15.00, 15.44, 15.56, 16.11, 16.38, 16.65},
};
__constant__ double c_baq_norm[3][16] = {
    {0.2490, 0.7680, 1.3655, 2.1864},
    {0.1290, 0.3900, 0.6601, 0.9471, 1.2623, 1.6261, 2.0793, 2.7467},
    {0.0660, 0.1985, 0.3320, 0.4677, 0.6061, 0.7487, 0.8964, 1.0510, 1.2143, 1.3896, 1.5800, 1.7914, 2.0329,
     2.3234, 2.6971, 3.2692},
};
__constant__ int c_baq_thidx[3] = {3, 7, 15};
__constant__ int c_baq_mcode[3] = {3, 5, 10};

// n <= 25 bits at bit position `bit` of u (bytes at or past `avail` read as 0)
__device__ __forceinline__ uint32_t read_field(const uint8_t* u, long long avail, long long bit, int n) {
    const long long by = bit >> 3;
    uint32_t w = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) w = (w << 8) | (by + i < avail ? (uint32_t)u[by + i] : 0u);
    return (w << (bit & 7)) >> (32 - n);
}

__device__ __forceinline__ long long align16(long long b) { return (b + 15) & ~15LL; }

template <typename R>
__global__ void __launch_bounds__(256) k_decode_fixed(const uint8_t* __restrict__ s, long long n,
                                                      const long long* __restrict__ offsets, DecodeSpec spec,
                                                      cpx<R>* __restrict__ out, int* __restrict__ status, int fields) {
    __shared__ int bad;
    const int j = blockIdx.x;
    const DecodeJob jb = job_at(spec, j);
    const long long off = offsets[jb.pk];
    if (off < 0 || off > n - 68) {           // header outside the stream
        if (threadIdx.x == 0) status[j] = S1G_E_PACKET_LENGTH;
        for (int k = threadIdx.x; k < 2 * jb.nq; k += blockDim.x) out[jb.out + k] = mk((R)0, (R)0);
        return;
    }
    const uint8_t* hdr = s + off;
    const int baq = hdr[37] & 31;            // baq_mode: bits 299..303 of the header
    if (baq >= 12 && baq <= 14) return;      // FDBAQ: the type-D decoder's row
    const int nq = jb.nq;
    cpx<R>* row = out + jb.out;
    const long long pdl = ((long long)hdr[4] << 8) | hdr[5];
    const long long ulen = pdl + 1 - 62;
    long long avail = n - (off + 68);
    if (avail > ulen) avail = ulen;
    if (avail < 0) avail = 0;
    const int pnq = (hdr[6 + 59] << 8) | hdr[6 + 60];
    const int M = baq;
    const int nb = (2 * nq + 255) / 256;
    // bit offsets of the channels and the last bit the reference reads
    long long w = 0, cw = 0, qe = 0, need = 0;
    int st = 0;
    if (ulen < 0) st = S1G_E_PACKET_LENGTH;
    else if (pnq != nq) st = S1G_E_RAGGED_BURST;
    else if (baq == 0) {
        w = align16(10LL * nq);
        need = 3 * w + 10LL * nq;
    } else if (baq >= 3 && baq <= 5) {
        cw = align16((long long)M * nq);
        qe = align16(8LL * nb + (long long)M * nq);
        need = 2 * cw + qe + (long long)M * nq;
    } else {
        st = S1G_E_BAD_FORMAT;
    }
    if (!st && need > 8 * ulen) st = S1G_E_READ_PAST_END;
    if (threadIdx.x == 0) bad = st;
    __syncthreads();
    const uint8_t* u = hdr + 68;
    if (bad == 0) {
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            double v[4] = {0.0, 0.0, 0.0, 0.0};
            bool err = false;
            if (baq == 0) {
                const int src = fields ? q : q - 128;
                if (src >= 0) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint32_t x = read_field(u, avail, c * w + 10LL * src, 10);
                        v[c] = ((x >> 9) ? -1.0 : 1.0) * (double)(x & 511u);
                    }
                }
            } else {
                const int b = q >> 7;
                const int th = (int)read_field(u, avail, 2 * cw + (long long)b * (8 + 128 * M), 8);
                const int lim = c_baq_thidx[M - 3], flag = c_baq_mcode[M - 3];
                if (!fields) {
                    const double x = th <= lim ? 0.0 : c_baq_norm[M - 3][0] * c_sf[th];
                    v[0] = v[1] = v[2] = v[3] = x;
                } else {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const long long start = c == 0 ? 0 : c == 1 ? cw : c == 2 ? 2 * cw : 2 * cw + qe;
                        const long long pos = start + (c == 2 ? 8LL * (b + 1) : 0) + (long long)M * q;
                        const uint32_t x = read_field(u, avail, pos, M);
                        const double sg = (x >> (M - 1)) ? -1.0 : 1.0;
                        const int m = (int)(x & ((1u << (M - 1)) - 1));
                        if (th <= lim) {
                            if (m < flag) v[c] = sg * (double)m;
                            else if (m == flag) v[c] = sg * c_baq_simple[M - 3][th];
                            else err = true;
                        } else {
                            v[c] = sg * c_baq_norm[M - 3][m] * c_sf[th];
                        }
                    }
                }
            }
            if (err) atomicExch(&bad, S1G_E_MCODE);
            row[2 * q] = mk((R)v[0], (R)v[2]);
            row[2 * q + 1] = mk((R)v[1], (R)v[3]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) status[j] = bad;
    if (bad != 0)
        for (int k = threadIdx.x; k < 2 * nq; k += blockDim.x) row[k] = mk((R)0, (R)0);
}

static void build_lut(std::vector<HuffEntry>& lut) {
    // value-keyed maps of structs.h:170-227 (key value -> mcode) and the
    // start lengths of structs.h:170; the walk of decoding_utils.cpp:44-77
    static const int keys[5][16][2] = {
        {{0, 0}, {2, 1}, {6, 2}, {7, 3}},
        {{0, 0}, {2, 1}, {6, 2}, {14, 3}, {15, 4}},
        {{0, 0}, {2, 1}, {6, 2}, {14, 3}, {30, 4}, {62, 5}, {63, 6}},
        {{0, 0}, {1, 1}, {2, 2}, {6, 3}, {14, 4}, {30, 5}, {62, 6}, {126, 7}, {254, 8}, {255, 9}},
        {{0, 0}, {2, 1}, {3, 2}, {4, 3}, {5, 4}, {12, 5}, {13, 6}, {14, 7}, {30, 8}, {62, 9},
         {252, 10}, {253, 11}, {508, 12}, {509, 13}, {510, 14}, {511, 15}},
    };
    static const int nkeys[5] = {4, 5, 7, 10, 16};
    static const int start[5] = {1, 1, 1, 2, 2};
    lut.assign(5 * kHuffWindow, 0);
    for (int brc = 0; brc < 5; ++brc) {
        for (int w = 0; w < 1024; ++w) {
            auto bits = [&](int len) { return (w >> (10 - len)) & ((1 << len) - 1); };
            int len = start[brc];
            int mcode = 0, clen = 0;   // clen 0: no code within 10 bits
            if (brc == 4 && bits(2) == 0) {
                clen = 2;
            } else {
                if (brc == 4) len += 1;
                for (int i = 0; i < 10; ++i) {
                    const int v = bits(len);
                    int m = -1;
                    for (int k = 0; k < nkeys[brc]; ++k)
                        if (keys[brc][k][0] == v) m = keys[brc][k][1];
                    if (m >= 0) {
                        mcode = m;
                        clen = len;
                        break;
                    }
                    len += 1;
                    if (len > 10) break;
                }
            }
            for (int sign = 0; sign < 2; ++sign)
                lut[brc * kHuffWindow + (sign << 10) + w] =
                    clen ? (HuffEntry)(((1 + clen) << 8) | (sign << 7) | mcode) : (HuffEntry)0;
        }
    }
}

size_t huffman_lut_bytes() { return sizeof(HuffEntry) * 5 * kHuffWindow; }

void huffman_lut_fill(void* host_dst) {
    std::vector<HuffEntry> h;
    build_lut(h);
    memcpy(host_dst, h.data(), sizeof(HuffEntry) * h.size());
}

// Decode npk packets (offsets d_offsets[p0 .. p0+npk)) into FP32 rows using
// caller-supplied scratch (sym: npk*4*sym_pitch(nq) bytes, brc/thidx: npk*nb
// bytes) and a device copy of the Huffman table.  Used by the allocation-free
// entry point.
void decode_fp32_with_scratch(const uint8_t* d_stream, long long n, const long long* d_offsets, int p0, int npk,
                              int nq, cf32* out, long long pitch, int* d_status, uint8_t* sym, uint8_t* brc,
                              uint8_t* thidx, const void* d_lut, cudaStream_t st) {
    const DecodeSpec spec{nullptr, npk, nullptr, p0, nq, pitch};
    note_launch(), k_decode_symbols<<<(npk + kDecodeThreads - 1) / kDecodeThreads, kDecodeThreads, 0, st>>>(d_stream, n, d_offsets, spec, sym, brc, thidx,
                                                                     d_status, (const HuffEntry*)d_lut);
    note_launch(), k_decode_values<float><<<npk, 256, 0, st>>>(sym, brc, thidx, spec, out, d_status);
}

DecodeTables::~DecodeTables() {
    if (lut) cudaFree(lut);
}

void DecodeTables::init() {
    if (lut) return;
    std::vector<HuffEntry> h;
    build_lut(h);
    check_cuda(cudaMalloc(&lut, sizeof(HuffEntry) * h.size()), "lut");
    check_cuda(cudaMemcpy(lut, h.data(), sizeof(HuffEntry) * h.size(), cudaMemcpyHostToDevice), "lut up");
}

template <typename R>
void decode_burst(const uint8_t* d_stream, long long n, const long long* d_offsets, const int* d_pkidx, int p0,
                  int npk, int nq, cpx<R>* out, long long pitch, int* d_status, DecodeScratch& sc, const DecodeTables& tabs,
                  cudaStream_t st) {
    const int nb = (2 * nq + 255) / 256;
    sc.reserve((size_t)npk * 4 * sym_pitch(nq), (size_t)npk * nb);
    const DecodeSpec spec{nullptr, npk, d_pkidx, p0, nq, pitch};
    note_launch(), k_decode_symbols<<<(npk + kDecodeThreads - 1) / kDecodeThreads, kDecodeThreads, 0, st>>>(d_stream, n, d_offsets, spec, sc.sym, sc.brc,
                                                                     sc.thidx, d_status, (const HuffEntry*)tabs.lut);
    note_launch(), k_decode_values<R><<<npk, 256, 0, st>>>(sc.sym, sc.brc, sc.thidx, spec, out, d_status);
}

template <typename R>
void decode_jobs(const uint8_t* d_stream, long long n, const long long* d_offsets, const DecodeJob* d_jobs, int njobs,
                 size_t sym_bytes, size_t blk_bytes, cpx<R>* out, int* d_status, DecodeScratch& sc,
                 const DecodeTables& tabs, cudaStream_t st) {
    if (njobs <= 0) return;
    sc.reserve(sym_bytes, blk_bytes);
    const DecodeSpec spec{d_jobs, njobs, nullptr, 0, 0, 0};
    note_launch(), k_decode_symbols<<<(njobs + kDecodeThreads - 1) / kDecodeThreads, kDecodeThreads, 0, st>>>(d_stream, n, d_offsets, spec, sc.sym, sc.brc,
                                                                       sc.thidx, d_status, (const HuffEntry*)tabs.lut);
    note_launch(), k_decode_values<R><<<njobs, 256, 0, st>>>(sc.sym, sc.brc, sc.thidx, spec, out, d_status);
}

// The reconstruction (k_decode_values) of jobs whose symbols a decode_jobs
// call just left in sc: e.g. FP64 samples of packets decoded for FP32 output,
// without a second bit walk.  d_status must hold that walk's status.
template <typename R>
void decode_jobs_values(const DecodeJob* d_jobs, int njobs, cpx<R>* out, int* d_status, const DecodeScratch& sc,
                        cudaStream_t st) {
    if (njobs <= 0) return;
    const DecodeSpec spec{d_jobs, njobs, nullptr, 0, 0, 0};
    note_launch(), k_decode_values<R><<<njobs, 256, 0, st>>>(sc.sym, sc.brc, sc.thidx, spec, out, d_status);
}
template void decode_jobs_values<double>(const DecodeJob*, int, cpx<double>*, int*, const DecodeScratch&,
                                         cudaStream_t);

template <typename R>
void decode_fixed_burst(const uint8_t* d_stream, long long n, const long long* d_offsets, const int* d_pkidx, int p0,
                        int npk, int nq, cpx<R>* out, long long pitch, int* d_status, int fields, cudaStream_t st) {
    if (npk <= 0) return;
    const DecodeSpec spec{nullptr, npk, d_pkidx, p0, nq, pitch};
    note_launch(), k_decode_fixed<R><<<npk, 256, 0, st>>>(d_stream, n, d_offsets, spec, out, d_status, fields);
}

template <typename R>
void decode_fixed_jobs(const uint8_t* d_stream, long long n, const long long* d_offsets, const DecodeJob* d_jobs,
                       int njobs, cpx<R>* out, int* d_status, int fields, cudaStream_t st) {
    if (njobs <= 0) return;
    const DecodeSpec spec{d_jobs, njobs, nullptr, 0, 0, 0};
    note_launch(), k_decode_fixed<R><<<njobs, 256, 0, st>>>(d_stream, n, d_offsets, spec, out, d_status, fields);
}

template void decode_fixed_burst<float>(const uint8_t*, long long, const long long*, const int*, int, int, int,
                                        cpx<float>*, long long, int*, int, cudaStream_t);
template void decode_fixed_burst<double>(const uint8_t*, long long, const long long*, const int*, int, int, int,
                                         cpx<double>*, long long, int*, int, cudaStream_t);
template void decode_fixed_jobs<float>(const uint8_t*, long long, const long long*, const DecodeJob*, int,
                                       cpx<float>*, int*, int, cudaStream_t);
template void decode_fixed_jobs<double>(const uint8_t*, long long, const long long*, const DecodeJob*, int,
                                        cpx<double>*, int*, int, cudaStream_t);

void DecodeScratch::reserve(size_t sym_bytes, size_t blk_bytes) {
    if (sym_bytes > sym_cap) {
        if (sym) cudaFree(sym);
        check_cuda(cudaMalloc(&sym, sym_bytes), "decode scratch");
        sym_cap = sym_bytes;
    }
    if (blk_bytes > blk_cap) {
        if (brc) cudaFree(brc);
        if (thidx) cudaFree(thidx);
        check_cuda(cudaMalloc(&brc, blk_bytes), "decode scratch");
        check_cuda(cudaMalloc(&thidx, blk_bytes), "decode scratch");
        blk_cap = blk_bytes;
    }
}

DecodeScratch::~DecodeScratch() {
    if (sym) cudaFree(sym);
    if (brc) cudaFree(brc);
    if (thidx) cudaFree(thidx);
}

template void decode_burst<float>(const uint8_t*, long long, const long long*, const int*, int, int, int, cpx<float>*,
                                  long long, int*, DecodeScratch&, const DecodeTables&, cudaStream_t);
template void decode_burst<double>(const uint8_t*, long long, const long long*, const int*, int, int, int,
                                   cpx<double>*, long long, int*, DecodeScratch&, const DecodeTables&, cudaStream_t);
template void decode_jobs<float>(const uint8_t*, long long, const long long*, const DecodeJob*, int, size_t, size_t,
                                 cpx<float>*, int*, DecodeScratch&, const DecodeTables&, cudaStream_t);

}  // namespace s1g
