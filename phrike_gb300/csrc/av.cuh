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
// 2D MHD resistivity / viscosity: G[f0 .. f0+2] -= coef (T1 + T2) per solve
cudaError_t launch_mhd_diff_fold(float* G, long ssG, const float* T1, const float* T2, long ssT, long cells,
                                 int nsolve, int f0, float coef, cudaStream_t s);

}  // namespace ps
