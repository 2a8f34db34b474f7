// Hann-windowed sinc interpolation of complex lines (s1g_sinc.cu).
#pragma once

#include "s1g_kernels.h"

namespace s1g {

template <typename R>
struct SincArgs {
    const cpx<R>* in;       // rows x in_pitch, n samples per line
    long long in_pitch;
    int n;
    const double* t;        // positions, rows x t_pitch (t_pitch 0: one set of m shared by all lines)
    long long t_pitch;
    int m;                  // outputs per line
    int L;                  // half-width (2L + 1 taps), 1..16
    cpx<R>* out;            // rows x out_pitch
    long long out_pitch;
    int rows;
};

template <typename R>
void sinc_interp(const SincArgs<R>& a, cudaStream_t st);

}  // namespace s1g
