// Corner turns (matrix transposes of complex<float> bursts) staged through
// shared memory by the Tensor Memory Accelerator: the range <-> azimuth
// turns of the fused path (transpose, signal_processing.cpp:463-479, which
// the reference runs on vector<vector> rows).
//
// A tile is 128 source rows x 16 source columns (16 KB).  One thread issues
// cp.async.bulk.tensor.2d for it into shared memory with the 128-byte swizzle
// (16-byte chunk c of row r stored at chunk c ^ (r mod 8)), completing on an
// mbarrier; the block then writes the tile's 16 columns as 16 rows of the
// output, each warp storing 32 consecutive elements (256 bytes) at a time and
// reading them from shared memory with at most two-way bank conflicts.  Two
// tile buffers per block: the next-but-one tile is in flight while a tile is
// written out.  Blocks walk the tiles grid-stride (a persistent grid of a few
// blocks per SM).  Source rows of another pitch or alignment fall back to
// the shared-memory tile transpose of s1g_fft_engine.cu.
//
// Every mbarrier wait is bounded; a wait that runs out sets a device flag
// (read by tma_take_error), waits (bounded) for the copies the block has in
// flight and leaves the kernel.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <climits>
#include <cstdint>
#include <mutex>
#include <stdexcept>

#include "s1g_fft_engine.h"
#include "s1g_kernels.h"
#include "s1g_tma.h"

namespace s1g {

namespace {

constexpr int kTileCols = 16;                 // 16 x 8 bytes = the 128-byte swizzle span
constexpr int kTileRows = 128;
constexpr unsigned kTileBytes = kTileCols * kTileRows * 8;
constexpr long long kWaitLimit = 1LL << 22;   // polls of one mbarrier wait (far beyond a tile's load time)

__device__ int g_tma_error = 0;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Poll until the phase with this parity completes, at most kWaitLimit times.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (long long k = 0; k < kWaitLimit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace

__global__ void __launch_bounds__(256) k_transpose_tma(const __grid_constant__ CUtensorMap src, cf32* __restrict__ out,
                                                       long long op, int rows, int cols) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t bar[2];
    __shared__ int s_fail;
    // the 128-byte swizzle repeats every 1024 bytes: tile buffers 1024-aligned
    unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char* buf0 = base;
    unsigned char* buf1 = base + kTileBytes;
    const int ntx = (cols + kTileCols - 1) / kTileCols;
    const int nty = (rows + kTileRows - 1) / kTileRows;
    const long long total = (long long)ntx * nty;
    const long long g = gridDim.x;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // tile t into buffer b (one elected thread)
    auto issue = [&](long long t, int b) {
        const int tx = (int)(t % ntx), ty = (int)(t / ntx);
        mbar_expect_tx(&bar[b], kTileBytes);
        tma_load_2d(b ? buf1 : buf0, &src, tx * kTileCols, ty * kTileRows, &bar[b]);
    };
    int inflight = 0;   // loads issued and not yet waited for (thread 0's count)
    if (threadIdx.x == 0) {
        if (blockIdx.x < total) issue(blockIdx.x, 0), ++inflight;
        if (blockIdx.x + g < total) issue(blockIdx.x + g, 1), ++inflight;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int i = 0;
    for (long long t = blockIdx.x; t < total; t += g, ++i) {
        const int b = i & 1;
        const uint32_t parity = (uint32_t)(i >> 1) & 1u;
        if (!mbar_wait_bounded(&bar[b], parity)) atomicExch(&s_fail, 1);
        __syncthreads();
        if (s_fail) {
            if (threadIdx.x == 0) {
                atomicExch(&g_tma_error, 1);
                // the loads still in flight land before the block leaves
                // (bounded): the current tile's and, if issued, the next one's
                mbar_wait_bounded(&bar[b], parity);
                if (inflight > 1) mbar_wait_bounded(&bar[b ^ 1], ((uint32_t)(i + 1) >> 1) & 1u);
            }
            return;
        }
        if (threadIdx.x == 0) --inflight;
        const unsigned char* tile = b ? buf1 : buf0;
        const int c0 = (int)(t % ntx) * kTileCols, r0 = (int)(t / ntx) * kTileRows;
        // warp w writes output rows c0 + 2w, c0 + 2w + 1 (source columns)
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
            const int c = 2 * warp + cc;
            if (c0 + c >= cols) continue;
            cf32* orow = out + (long long)(c0 + c) * op + r0;
#pragma unroll
            for (int q = 0; q < kTileRows / 32; ++q) {
                const int r = 32 * q + lane;
                if (r0 + r >= rows) continue;
                const int off = r * 128 + ((((c >> 1) ^ (r & 7))) << 4) + ((c & 1) << 3);
                orow[r] = *reinterpret_cast<const cf32*>(tile + off);
            }
        }
        __syncthreads();   // the buffer is free again
        if (threadIdx.x == 0 && t + 2 * g < total) {
            // the generic-proxy reads above come before the async-proxy write
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(t + 2 * g, b);
            ++inflight;
        }
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

bool transpose_tma(const cf32* in, long long ip, cf32* out, long long op, int rows, int cols, cudaStream_t st) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
    // a tiled TMA copy needs a 16-byte aligned base and a row pitch that is a
    // multiple of 16 bytes (an even number of complex<float>)
    if (!enc || rows < 1 || cols < 1 || (reinterpret_cast<uintptr_t>(in) & 15) || (ip & 1) || ip < cols)
        return false;
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ip * 8};
    const cuuint32_t box[2] = {(cuuint32_t)kTileCols, (cuuint32_t)kTileRows};
    const cuuint32_t estr[2] = {1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<cf32*>(in), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long long tiles = (long long)((cols + kTileCols - 1) / kTileCols) * ((rows + kTileRows - 1) / kTileRows);
    const int grid = (int)std::min<long long>(tiles, 4LL * sms);
    const size_t smem = 2 * kTileBytes + 1024;
    static bool attr = false;
    if (!attr) {
        check_cuda(cudaFuncSetAttribute(k_transpose_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "tma transpose attr");
        attr = true;
    }
    note_launch(), k_transpose_tma<<<grid, 256, smem, st>>>(map, out, op, rows, cols);
    return true;
}

int tma_take_error() {
    int e = 0;
    if (cudaMemcpyFromSymbol(&e, g_tma_error, sizeof(int)) != cudaSuccess) return -1;
    if (e) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_tma_error, &zero, sizeof(int));
    }
    return e;
}

}  // namespace s1g

using namespace s1g;

extern "C" {

int s1g_transpose(const void* d_in, int64_t rows, int64_t cols, int64_t in_pitch, void* d_out, int64_t out_pitch,
                  int elem_type, void* stream) {
    if (!d_in || !d_out || d_in == d_out || rows < 0 || cols < 0 || in_pitch < cols || out_pitch < rows)
        return S1G_E_INVALID_ARGUMENT;
    if (rows > INT_MAX || cols > INT_MAX || (cols + 31) / 32 > INT_MAX || (rows + 31) / 32 > 65535)
        return S1G_E_INVALID_ARGUMENT;
    if (rows == 0 || cols == 0) return S1G_OK;
    cudaStream_t st = (cudaStream_t)stream;
    try {
        if (elem_type == S1G_CF32)
            transpose_batched<float>((const cf32*)d_in, in_pitch, 0, (cf32*)d_out, out_pitch, 0, (int)rows, (int)cols,
                                     1, st);
        else if (elem_type == S1G_CF64)
            transpose_batched<double>((const cf64*)d_in, in_pitch, 0, (cf64*)d_out, out_pitch, 0, (int)rows,
                                      (int)cols, 1, st);
        else
            return S1G_E_INVALID_ARGUMENT;
    } catch (const std::exception&) {
        return S1G_E_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? S1G_OK : S1G_E_CUDA;
}

int s1g_take_device_timeout(int* flag) {
    if (!flag) return S1G_E_INVALID_ARGUMENT;
    const int e = tma_take_error();
    if (e < 0) return S1G_E_CUDA;
    *flag = e;
    return S1G_OK;
}

}  // extern "C"
