// Launchers of the cell-wise kernels in reduce.cu (all per solve of a batch;
// ss is the solve stride of U in elements).
#pragma once
#include <cuda_runtime.h>

namespace ps {
cudaError_t launch_fill_int(int* a, int n, int v, cudaStream_t s);
cudaError_t launch_eref_set(const float* E, long ss, int nsolve, float* eref, cudaStream_t s);
cudaError_t launch_energy_shift(float* E, long n, long ss, int nsolve, const float* eref, float sign,
                                cudaStream_t s);
// dt_cap > 0: a further upper bound on dt (parabolic CFL of explicit diffusion)
cudaError_t launch_step_control(const float* speed, double cfl, double hmin, const double* t, const double* tend,
                                int nsolve, double* dt, int* active, cudaStream_t s, double dt_cap = 0.0);
cudaError_t launch_step_advance(double* t, const double* dt, float* speed, const int* active, int* steps,
                                int nsolve, cudaStream_t s);
// eshift (nullable): per-solve energy offset of states stored as E - E_ref
cudaError_t launch_speed(int nd, const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                         cudaStream_t s, const float* eshift = nullptr);
cudaError_t launch_conserved(int nd, const float* U, long cells, long ss, int nsolve, double gamma, double* out,
                             cudaStream_t s);
cudaError_t launch_speed_mhd(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                             cudaStream_t s);
cudaError_t launch_speed_mhd1d(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                               cudaStream_t s);
cudaError_t launch_project_mhd1d(float* U, long n, long ss, int nsolve, const int* active, cudaStream_t s);
cudaError_t launch_conserved_mhd(const float* U, long cells, long ss, int nsolve, double gamma, double* out,
                                 cudaStream_t s);
cudaError_t launch_flux1d(const float* U, long n, long ss, int nsolve, float gamma, float* F, cudaStream_t s);
}  // namespace ps
