// Launchers of the cell-wise kernels in reduce.cu.
#pragma once
#include <cuda_runtime.h>

namespace ps {
cudaError_t launch_eref_set(const float* E, float* eref, cudaStream_t s);
cudaError_t launch_energy_shift(float* E, long n, const float* eref, float sign, cudaStream_t s);
cudaError_t launch_speed(int nd, const float* U, long cells, float gamma, float* out, cudaStream_t s);
cudaError_t launch_conserved(int nd, const float* U, long cells, double gamma, double* out, cudaStream_t s);
cudaError_t launch_flux1d(const float* U, long n, float gamma, float* F, cudaStream_t s);
cudaError_t launch_cfl_dt(const float* speed, double cfl, double hmin, const double* t, double t_end, double* dt,
                          cudaStream_t s);
}  // namespace ps
