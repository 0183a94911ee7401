// Adjoint of the ARD time step (gradients of a recorder misfit).
#include <cuda_runtime.h>

#include <string>

#include "ard_engine.h"
#include "ard_gb300.h"

using namespace ard;

extern "C" int ard_adjoint(ard_ctx* c, int64_t, const float*, int32_t, float*, float*, float*) {
  if (!c) return ARD_ERR_INVALID;
  reinterpret_cast<Ctx*>(c)->err = "ard_adjoint: not available in this build";
  return ARD_ERR_STATE;
}

extern "C" int ard_read_initial_pressure_grad(ard_ctx* c, int32_t, int32_t, float*) {
  if (!c) return ARD_ERR_INVALID;
  reinterpret_cast<Ctx*>(c)->err = "ard_read_initial_pressure_grad: not available in this build";
  return ARD_ERR_STATE;
}
