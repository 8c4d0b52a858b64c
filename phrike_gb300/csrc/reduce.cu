// Cell-wise kernels: CFL wave speed (max), conserved sums (float64), 1D flux,
// device-side CFL step size.
#include <cuda_runtime.h>

#include "pass_common.cuh"
#include "reduce.cuh"

namespace ps {

// Max wave speed with the reference's per-dimension rule
// (equations.py:89-98 1D |u|+a, 137-147 2D |u_x|+a, 199-211 3D max|u_i|+a).
template <int ND>
__global__ void k_speed(const float* __restrict__ U, long cells, float gamma, float* out) {
  __shared__ float red[32];
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i];
    const float rinv = 1.0f / rho;
    float kin = 0.0f, um = 0.0f;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const float v = U[(1 + d) * cells + i] * rinv;
      kin = fmaf(v, v, kin);
      if (d == 0 || ND == 3) um = fmaxf(um, fabsf(v));
    }
    const float p = (gamma - 1.0f) * (U[(ND + 1) * cells + i] - 0.5f * rho * kin);
    m = fmaxf(m, um + sqrtf(gamma * p / rho));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(out, m);
}

// Plain sums of rho, rho u_i and p/(gamma-1) + rho|u|^2/2 from primitives, in
// float64 (solver.py:372-377, 741-767, 1439-1468).
template <int ND>
__global__ void k_conserved(const float* __restrict__ U, long cells, double gamma, double* out) {
  constexpr int NC = ND + 2;
  __shared__ double red[NC][32];
  double s[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) s[c] = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const double rho = U[i];
    double kin = 0.0;
    double vel[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      vel[d] = (double)U[(1 + d) * cells + i] / rho;
      kin += vel[d] * vel[d];
    }
    const double p = (gamma - 1.0) * ((double)U[(ND + 1) * cells + i] - 0.5 * rho * kin);
    s[0] += rho;
#pragma unroll
    for (int d = 0; d < ND; ++d) s[1 + d] += rho * vel[d];
    s[NC - 1] += p / (gamma - 1.0) + 0.5 * rho * kin;
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    double v = s[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[c][w] = v;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double v = (l < nw) ? red[c][l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (l == 0) atomicAdd(out + c, v);
    }
  }
}

// 1D flux F = [rho u, rho u^2 + p, (E + p) u] (equations.py:67-86)
__global__ void k_flux1d(const float* __restrict__ U, long n, float gamma, float* __restrict__ F) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i], m = U[n + i], E = U[2 * n + i];
    const float u = m / rho;
    const float p = (gamma - 1.0f) * (E - 0.5f * rho * u * u);
    const float mom = rho * u;
    F[i] = mom;
    F[n + i] = mom * u + p;
    F[2 * n + i] = (E + p) * u;
  }
}

// dt = cfl * hmin / speed (1e-6 when speed <= 0), clipped to t_end - t
// (solver.py:235-240, 386-389).
__global__ void k_cfl_dt(const float* speed, double cfl, double hmin, const double* t, double t_end,
                         double* dt) {
  const double s = (double)(*speed);
  double d = (s <= 0.0) ? 1e-6 : cfl * hmin / s;
  if (t != nullptr) d = fmin(d, t_end - *t);
  *dt = d;
}

// E_ref of the energy-perturbation form: the energy of the first cell.
__global__ void k_eref_set(const float* E, float* eref) { *eref = E[0]; }

// E <- E + sign * E_ref (sign -1: to perturbation form, +1: back)
__global__ void k_energy_shift(float* E, long n, const float* eref, float sign) {
  const float s = sign * (*eref);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) E[i] += s;
}

cudaError_t launch_eref_set(const float* E, float* eref, cudaStream_t s) {
  k_eref_set<<<1, 1, 0, s>>>(E, eref);
  return cudaGetLastError();
}

cudaError_t launch_energy_shift(float* E, long n, const float* eref, float sign, cudaStream_t s) {
  const long want = (n + 255) / 256;
  const int blocks = (int)(want < 4096 ? want : 4096);
  k_energy_shift<<<blocks, 256, 0, s>>>(E, n, eref, sign);
  return cudaGetLastError();
}

cudaError_t launch_speed(int nd, const float* U, long cells, float gamma, float* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  const int blocks = (int)((cells + 255) / 256 < 1184 ? (cells + 255) / 256 : 1184);
  if (nd == 1) k_speed<1><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  else if (nd == 2) k_speed<2><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  else k_speed<3><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_conserved(int nd, const float* U, long cells, double gamma, double* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * (nd + 2), s);
  if (e != cudaSuccess) return e;
  const int blocks = (int)((cells + 255) / 256 < 1184 ? (cells + 255) / 256 : 1184);
  if (nd == 1) k_conserved<1><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  else if (nd == 2) k_conserved<2><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  else k_conserved<3><<<blocks, 256, 0, s>>>(U, cells, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_flux1d(const float* U, long n, float gamma, float* F, cudaStream_t s) {
  const int blocks = (int)((n + 255) / 256);
  k_flux1d<<<blocks, 256, 0, s>>>(U, n, gamma, F);
  return cudaGetLastError();
}

cudaError_t launch_cfl_dt(const float* speed, double cfl, double hmin, const double* t, double t_end, double* dt,
                          cudaStream_t s) {
  k_cfl_dt<<<1, 1, 0, s>>>(speed, cfl, hmin, t, t_end, dt);
  return cudaGetLastError();
}

}  // namespace ps
