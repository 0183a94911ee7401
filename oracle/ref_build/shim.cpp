/* ORACLE / TEST INFRASTRUCTURE ONLY.
 * Implementations behind the fftw3.h and utils_VkFFT.h stand-ins. */
#include "fftw3.h"
#include "utils_VkFFT.h"

#include <cstdlib>

#include "../dct_fft.h"

struct ard_fftwf_plan_s {
  int n0, n1, n2;
  int kind;
  float* in;
  float* out;
};

fftwf_plan fftwf_plan_r2r_3d(int n0, int n1, int n2, float* in, float* out,
                             fftw_r2r_kind kind0, fftw_r2r_kind kind1,
                             fftw_r2r_kind kind2, unsigned) {
  if (kind0 != kind1 || kind1 != kind2) std::abort();
  if (kind0 != FFTW_REDFT10 && kind0 != FFTW_REDFT01) std::abort();
  fftwf_plan p = (fftwf_plan)std::calloc(1, sizeof(ard_fftwf_plan_s));
  p->n0 = n0; p->n1 = n1; p->n2 = n2;
  p->kind = kind0 == FFTW_REDFT10 ? 10 : 1;
  p->in = in; p->out = out;
  return p;
}

void fftwf_execute(const fftwf_plan p) {
  dctfft_3d_float(p->n0, p->n1, p->n2, p->kind, p->in, p->out);
}

void fftwf_destroy_plan(fftwf_plan p) { std::free(p); }

VkFFT_DCT::VkFFT_DCT(VkGPU*, int dctType, int width, int height, int depth,
                     float* input, float* output)
    : m_dctType(dctType), m_width(width), m_height(height), m_depth(depth),
      m_input(input), m_output(output) {
  if (dctType != 2 && dctType != 3) std::abort();
}

VkFFT_DCT::~VkFFT_DCT() {}

VkFFTResult VkFFT_DCT::execute() {
  /* FFTW's plan dimension order: (depth, height, width), width fastest. */
  dctfft_3d_float(m_depth, m_height, m_width, m_dctType == 2 ? 10 : 1,
                  m_input, m_output);
  return 0;
}
