/* ORACLE / TEST INFRASTRUCTURE ONLY.
 * Replaces ARD-simulator-190113/utils_VkFFT.h for the headless build.  The
 * reference hard-wires the VkFFT path on (dct_volume.cpp:8), and Vulkan cannot
 * be brought up here, so VkFFT_DCT::execute runs the same 3D REDFT10 (type 2)
 * or REDFT01 (type 3) on the host that the FFTW path would
 * (utils_VkFFT.cpp:623-690 configures VkFFT for exactly those transforms,
 * unnormalised, size (width, height, depth) with x fastest). */
#pragma once
#include <cstdint>

typedef int VkFFTResult;

struct VkGPU {
  int unused;
};

class VkFFT_DCT {
 public:
  VkFFT_DCT(VkGPU* vkGPU, int dctType, int width, int height, int depth,
            float* input, float* output);
  ~VkFFT_DCT();
  VkFFTResult execute();

 private:
  int m_dctType;
  int m_width, m_height, m_depth;
  float* m_input;
  float* m_output;
};
