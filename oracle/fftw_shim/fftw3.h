/*
 * FFTW-API shim for building the reference's own C++ sources as a CPU
 * oracle.  TEST INFRASTRUCTURE ONLY: nothing in the shipped library links it.
 *
 * FFTW3 is not installed in this image.  The reference uses exactly these
 * symbols (signal_processing.cpp:527-535,559-567,647-666,687-699,766-777 and
 * s1_decoder.cpp:593-594,621,641,679-680): fftw_complex, fftw_plan,
 * FFTW_FORWARD, FFTW_BACKWARD, FFTW_ESTIMATE, fftw_plan_dft_1d,
 * fftw_plan_dft_2d, fftw_execute and fftw_destroy_plan.  This header declares
 * them with FFTW's documented semantics: forward = unnormalised
 * sum x[j] exp(-2 pi i jk/n), backward = unnormalised exp(+...).
 * The transform itself is restated in fftw_shim.cpp (mixed radix + Bluestein,
 * FP64), so any length n is supported.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
