// TMA-staged corner turns of complex<float> matrices (s1g_tma.cu).
#pragma once

#include "s1g_kernels.h"

namespace s1g {

// out[c][r] = in[r][c] (rows x cols, row pitches ip / op in elements) with
// tensor-memory-accelerator tile loads.  Returns false, launching nothing,
// where a tiled TMA copy cannot read the source (odd pitch, base not 16-byte
// aligned, no driver entry point); the caller then transposes another way.
bool transpose_tma(const cf32* in, long long ip, cf32* out, long long op, int rows, int cols, cudaStream_t st);

// 1 if a TMA corner turn gave up waiting for its tile since the last call
// (and clears the flag), 0 otherwise, -1 if the flag cannot be read.
// Synchronous: call it after the work has been waited for.
int tma_take_error();

}  // namespace s1g
