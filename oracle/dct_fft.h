/* ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Double-precision REDFT10 (DCT-II) and REDFT01 (DCT-III) of arbitrary length,
 * written from FFTW's published definitions (FFTW 3.3 manual, "Real even/odd
 * DFTs (cosine/sine transforms)"):
 *
 *   REDFT10: Y[k] = 2 * sum_{j=0}^{n-1} x[j] cos(pi (j + 1/2) k / n)
 *   REDFT01: Y[k] = x[0] + 2 * sum_{j=1}^{n-1} x[j] cos(pi j (k + 1/2) / n)
 *
 * Both are unnormalised; REDFT01(REDFT10(x)) = 2n x.  The reference calls them
 * through fftwf_plan_r2r_3d (ARD-simulator-190113/dct_volume.cpp:17,19,44,60).
 * FFTW itself is not installed (the reference ships it only as Windows DLLs),
 * so this file provides the transform for both the headless reference build
 * (via the fftw3.h shim in ref_build/) and the C oracle.
 *
 * Algorithm: Makhoul's reordering (J. Makhoul, "A fast cosine transform in
 * one and multiple dimensions", IEEE TASSP 28(1), 1980) maps a length-n DCT-II
 * onto one length-n complex DFT; the DCT-III is its transpose.  The complex
 * DFT is a recursive mixed-radix Cooley-Tukey FFT with radix-2/3/4/5
 * butterflies and a direct butterfly for any other prime factor.
 */
#ifndef ARD_ORACLE_DCT_FFT_H
#define ARD_ORACLE_DCT_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dctfft_plan dctfft_plan;

/* Plan for length n (n >= 1).  Thread-safe to execute concurrently. */
dctfft_plan* dctfft_make(int n);
void dctfft_free(dctfft_plan* p);
int dctfft_length(const dctfft_plan* p);

/* Scratch size (in doubles) that dctfft_redft10 / dctfft_redft01 need. */
int dctfft_scratch_doubles(const dctfft_plan* p);

/* In-place 1D transforms of x[0..n-1] (contiguous).  scratch must hold
 * dctfft_scratch_doubles(p) doubles. */
void dctfft_redft10(const dctfft_plan* p, double* x, double* scratch);
void dctfft_redft01(const dctfft_plan* p, double* x, double* scratch);

/* 3D transform of a [n0][n1][n2] row-major array (n2 fastest), all three axes
 * of the same kind (10 or 01), as fftw_plan_r2r_3d does.  in and out may alias.
 * Float I/O with double arithmetic. */
void dctfft_3d_float(int n0, int n1, int n2, int kind,
                     const float* in, float* out);
/* Same with double I/O. */
void dctfft_3d_double(int n0, int n1, int n2, int kind,
                      const double* in, double* out);

#ifdef __cplusplus
}
#endif
#endif
