// Element-wise kernels of the 2D artificial-viscosity terms
// (artificial_viscosity.py:270-403).  The host (ps_api.cu) evaluates
//   term_c = dx1(w_c nu dx1 U_c) + dy1(w_c nu dy1 U_c)
// with the pencil operator passes: gradients dx1 = D_x P_y and dy1 = P_x D_y
// of the stage input (and of the sensor variable), nu and the viscous fluxes
// here, then their x factors D_x and P_x, which are subtracted from the Euler
// x-pass outputs so that the y (last) pass evaluates Euler and viscous terms
// together by linearity.
#include <cuda_runtime.h>

#include "av.cuh"

namespace ps {

// q = u_y of a 2D state (the reference's 2D "pressure" sensor, see AVParams)
__global__ void k_av_uy(const float* __restrict__ S, long cells, long ssS, float* __restrict__ Q) {
  const long so = (long)blockIdx.y * ssS, qo = (long)blockIdx.y * cells;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x)
    Q[qo + i] = S[so + 2 * cells + i] / S[so + i];
}

// nu from (dx1 q, dy1 q, q); then GX_c <- w_c nu GX_c, GY_c <- w_c nu GY_c
__global__ void k_av_flux(AVFluxArgs a) {
  const long so = (long)blockIdx.y * a.ssS, go = (long)blockIdx.y * a.ssG, qo = (long)blockIdx.y * a.ssQ;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < a.cells; i += (long)gridDim.x * blockDim.x) {
    const float gx = a.qx[qo + i], gy = a.qy[qo + i];
    const float q = a.q[qo + i];
    const float nu = av_nu(a.av, sqrtf(gx * gx + gy * gy), q);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float wn = a.av.w[c] * nu;
      a.GX[go + c * a.cells + i] *= wn;
      a.GY[go + c * a.cells + i] *= wn;
    }
    (void)so;
  }
}

// G[solve][f] -= T[solve][f] for f < 4 (x factors of the viscous x fluxes)
// and G[solve][4 + f] -= T2[solve][f] (x factors of the viscous y fluxes)
__global__ void k_av_sub(float* __restrict__ G, long ssG, const float* __restrict__ T, const float* __restrict__ T2,
                         long ssT, long cells) {
  const long go = (long)blockIdx.y * ssG, to = (long)blockIdx.y * ssT;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < 4 * cells; i += (long)gridDim.x * blockDim.x) {
    G[go + i] -= T[to + i];
    G[go + 4 * cells + i] -= T2[to + i];
  }
}

// 2D MHD explicit diffusion (SpectralSolverMHD._compute_rhs, solver.py:942-954):
// G[solve][f0 + f] -= coef (T1 + T2)[solve][f], f < 3, with T1 = L_x X and
// T2 = (-k_y^2) P_x X, so that the last pass's P_y G carries
// coef (P_y L_x + L_y P_x) X = coef lap(X) (grid.py:1329-1338).
__global__ void k_mhd_diff_fold(float* __restrict__ G, long ssG, const float* __restrict__ T1,
                                const float* __restrict__ T2, long ssT, long cells, int f0, float coef) {
  const long go = (long)blockIdx.y * ssG + (long)f0 * cells, to = (long)blockIdx.y * ssT;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < 3 * cells; i += (long)gridDim.x * blockDim.x)
    G[go + i] -= coef * (T1[to + i] + T2[to + i]);
}

static int grid_x(long n, int nsolve) {
  const long want = (n + 255) / 256;
  const long cap = (2048 + nsolve - 1) / nsolve;
  return (int)(want < cap ? want : (cap > 0 ? cap : 1));
}

cudaError_t launch_av_uy(const float* S, long cells, long ssS, int nsolve, float* Q, cudaStream_t s) {
  k_av_uy<<<dim3(grid_x(cells, nsolve), nsolve), 256, 0, s>>>(S, cells, ssS, Q);
  return cudaGetLastError();
}

cudaError_t launch_av_flux(const AVFluxArgs& a, int nsolve, cudaStream_t s) {
  k_av_flux<<<dim3(grid_x(a.cells, nsolve), nsolve), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_av_sub(float* G, long ssG, const float* T, const float* T2, long ssT, long cells, int nsolve,
                          cudaStream_t s) {
  k_av_sub<<<dim3(grid_x(4 * cells, nsolve), nsolve), 256, 0, s>>>(G, ssG, T, T2, ssT, cells);
  return cudaGetLastError();
}

cudaError_t launch_mhd_diff_fold(float* G, long ssG, const float* T1, const float* T2, long ssT, long cells,
                                 int nsolve, int f0, float coef, cudaStream_t s) {
  k_mhd_diff_fold<<<dim3(grid_x(3 * cells, nsolve), nsolve), 256, 0, s>>>(G, ssG, T1, T2, ssT, cells, f0, coef);
  return cudaGetLastError();
}

}  // namespace ps
