/* ORACLE / TEST INFRASTRUCTURE ONLY.
 * FFTW-compatible declarations for the four FFTW names the reference uses
 * (ARD-simulator-190113/dct_volume.h:3, dct_volume.cpp:17,19,44,60).  FFTW is
 * not installed here; shim.cpp implements them with oracle/dct_fft.c
 * (REDFT10 / REDFT01 by their published definitions, double arithmetic). */
#pragma once

typedef struct ard_fftwf_plan_s* fftwf_plan;
typedef int fftw_r2r_kind;

#define FFTW_REDFT01 4
#define FFTW_REDFT10 5
#define FFTW_MEASURE (0U)

fftwf_plan fftwf_plan_r2r_3d(int n0, int n1, int n2, float* in, float* out,
                             fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                             fftw_r2r_kind kind2, unsigned flags);
void fftwf_execute(const fftwf_plan plan);
void fftwf_destroy_plan(fftwf_plan plan);
