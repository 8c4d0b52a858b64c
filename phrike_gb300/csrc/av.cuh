// Element-wise kernels of the 2D artificial-viscosity terms (av.cu).
#pragma once
#include <cuda_runtime.h>

#include "pass_common.cuh"

namespace ps {

struct AVFluxArgs {
  const float* q;    // sensor variable q (per solve stride ssQ)
  const float* qx;   // dx1 q
  const float* qy;   // dy1 q
  float* GX;         // dx1 U_c (4 fields per solve), scaled in place to w_c nu dx1 U_c
  float* GY;         // dy1 U_c
  long cells, ssS, ssG, ssQ;
  AVParams av;
};

cudaError_t launch_av_uy(const float* S, long cells, long ssS, int nsolve, float* Q, cudaStream_t s);
cudaError_t launch_av_flux(const AVFluxArgs& a, int nsolve, cudaStream_t s);
cudaError_t launch_av_sub(float* G, long ssG, const float* T, const float* T2, long ssT, long cells, int nsolve,
                          cudaStream_t s);

}  // namespace ps
