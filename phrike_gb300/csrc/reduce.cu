// Cell-wise kernels: CFL wave speed (max), conserved sums (float64), 1D flux,
// device-side CFL step size.
#include <cuda_runtime.h>

#include "pass_common.cuh"
#include "reduce.cuh"

namespace ps {

// Max wave speed with the reference's per-dimension rule
// (equations.py:89-98 1D |u|+a, 137-147 2D |u_x|+a, 199-211 3D max|u_i|+a).
// eshift (nullable): per-solve constant added to the stored energy (states in
// energy-perturbation form store E - E_ref).
template <int ND>
__global__ void k_speed(const float* __restrict__ U, long cells, long ss, float gamma, const float* eshift,
                        float* out) {
  __shared__ float red[32];
  const float es = (eshift != nullptr) ? eshift[blockIdx.y] : 0.0f;
  U += (long)blockIdx.y * ss;
  out += blockIdx.y;
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
    const float p = (gamma - 1.0f) * ((U[(ND + 1) * cells + i] + es) - 0.5f * rho * kin);
    m = fmaxf(m, um + sqrtf(gamma * p / rho));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(out, m);
}

// Plain sums of rho, rho u_i and p/(gamma-1) + rho|u|^2/2 from primitives, in
// float64 (solver.py:372-377, 741-767, 1439-1468).
template <int ND>
__global__ void k_conserved(const float* __restrict__ U, long cells, long ss, double gamma, double* out) {
  constexpr int NC = ND + 2;
  __shared__ double red[NC][32];
  U += (long)blockIdx.y * ss;
  out += (long)blockIdx.y * NC;
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

// 2D ideal MHD: max(|ux|, |uy|) + sqrt(a^2 + b^2) (equations.py:874-887)
__global__ void k_speed_mhd(const float* __restrict__ U, long cells, long ss, float gamma, float* out) {
  __shared__ float red[32];
  U += (long)blockIdx.y * ss;
  out += blockIdx.y;
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i];
    const float ux = U[cells + i] / rho, uy = U[2 * cells + i] / rho, uz = U[3 * cells + i] / rho;
    const float bx = U[5 * cells + i], by = U[6 * cells + i], bz = U[7 * cells + i];
    const float b2 = bx * bx + by * by + bz * bz;
    const float p = (gamma - 1.0f) * (U[4 * cells + i] - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
    m = fmaxf(m, fmaxf(fabsf(ux), fabsf(uy)) + sqrtf(fmaxf(gamma * p / rho + b2 / rho, 0.0f)));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(out, m);
}

// 1D MHD CFL speed (MHDEquations1D.max_wave_speed, equations.py:735-750):
// |u_x| + c_f with the exact fast magnetosonic speed along x
__global__ void k_speed_mhd1d(const float* __restrict__ U, long cells, long ss, float gamma, float* out) {
  __shared__ float red[32];
  U += (long)blockIdx.y * ss;
  out += blockIdx.y;
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i];
    const float ux = U[cells + i] / rho, uy = U[2 * cells + i] / rho, uz = U[3 * cells + i] / rho;
    const float bx = U[5 * cells + i], by = U[6 * cells + i], bz = U[7 * cells + i];
    const float b2 = bx * bx + by * by + bz * bz;
    const float p = (gamma - 1.0f) * (U[4 * cells + i] - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
    const float a2 = gamma * p / rho, bb = b2 / rho, cax2 = bx * bx / rho;
    const float disc = fmaxf((a2 + bb) * (a2 + bb) - 4.0f * a2 * cax2, 0.0f);
    m = fmaxf(m, fabsf(ux) + sqrtf(0.5f * (a2 + bb + sqrtf(disc))));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(out, m);
}

// 1D projection (grid.py:554-567 with solver.py:966-986): Bx <- mean(Bx),
// E += (Bx_new^2 - Bx_old^2) / 2; one block per solve
__global__ void k_project_mhd1d(float* U, long n, long ss, const int* active) {
  __shared__ float red[32];
  if (active != nullptr && !active[blockIdx.x]) return;
  U += (long)blockIdx.x * ss;
  float sum = 0.0f;
  for (long i = threadIdx.x; i < n; i += blockDim.x) sum += U[5 * n + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  float tot = 0.0f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
  const float mean = tot / (float)n;
  for (long i = threadIdx.x; i < n; i += blockDim.x) {
    const float bo = U[5 * n + i];
    U[4 * n + i] += 0.5f * (mean * mean - bo * bo);
    U[5 * n + i] = mean;
  }
}

// 2D ideal MHD conserved sums in float64 (equations.py:889-907): mass,
// momentum x/y/z, energy rebuilt from primitives, magnetic energy, cross
// helicity (and a zero pad to 8 values)
__global__ void k_conserved_mhd(const float* __restrict__ U, long cells, long ss, double gamma, double* out) {
  __shared__ double red[7][32];
  U += (long)blockIdx.y * ss;
  out += (long)blockIdx.y * 8;
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const double rho = U[i];
    const double ux = U[cells + i] / rho, uy = U[2 * cells + i] / rho, uz = U[3 * cells + i] / rho;
    const double bx = U[5 * cells + i], by = U[6 * cells + i], bz = U[7 * cells + i];
    const double v2 = ux * ux + uy * uy + uz * uz, b2 = bx * bx + by * by + bz * bz;
    const double p = (gamma - 1.0) * ((double)U[4 * cells + i] - 0.5 * rho * v2 - 0.5 * b2);
    s[0] += rho;
    s[1] += rho * ux;
    s[2] += rho * uy;
    s[3] += rho * uz;
    s[4] += p / (gamma - 1.0) + 0.5 * rho * v2 + 0.5 * b2;
    s[5] += 0.5 * b2;
    s[6] += ux * bx + uy * by + uz * bz;
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < 7; ++c) {
    double v = s[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[c][w] = v;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < 7; ++c) {
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

// E_ref of the energy-perturbation form: the energy of each solve's first cell.
__global__ void k_eref_set(const float* E, long ss, int nsolve, float* eref) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsolve) eref[s] = E[(long)s * ss];
}

// E <- E + sign * E_ref[solve] (sign -1: to perturbation form, +1: back)
__global__ void k_energy_shift(float* E, long n, long ss, const float* eref, float sign) {
  const float s = sign * eref[blockIdx.y];
  E += (long)blockIdx.y * ss;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) E[i] += s;
}

// Per-solve CFL step control before a step (solver.py:386-389, 235-240):
// active = t < t_end - 1e-12; dt = active ? min(cfl h / speed, t_end - t) : 0.
__global__ void k_step_control(const float* speed, double cfl, double hmin, const double* t, const double* tend,
                               int nsolve, double* dt, int* active, double dt_cap) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsolve) return;
  const bool on = t[s] < tend[s] - 1e-12;
  const double sp = (double)speed[s];
  double d = (sp <= 0.0) ? 1e-6 : cfl * hmin / sp;
  if (sp > 0.0 && dt_cap > 0.0) d = fmin(d, dt_cap);  // parabolic limit of explicit diffusion
  d = fmin(d, tend[s] - t[s]);
  dt[s] = on ? d : 0.0;
  active[s] = on ? 1 : 0;
}

// After a step: t += dt, count the step of every solve that advanced, clear
// the speed maxima for the next step.
__global__ void k_step_advance(double* t, const double* dt, float* speed, const int* active, int* steps,
                               int nsolve) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsolve) return;
  t[s] += dt[s];
  if (active[s]) steps[s] += 1;
  speed[s] = 0.0f;
}

__global__ void k_fill_int(int* a, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

cudaError_t launch_fill_int(int* a, int n, int v, cudaStream_t s) {
  k_fill_int<<<(n + 127) / 128, 128, 0, s>>>(a, n, v);
  return cudaGetLastError();
}

cudaError_t launch_eref_set(const float* E, long ss, int nsolve, float* eref, cudaStream_t s) {
  k_eref_set<<<(nsolve + 127) / 128, 128, 0, s>>>(E, ss, nsolve, eref);
  return cudaGetLastError();
}

cudaError_t launch_energy_shift(float* E, long n, long ss, int nsolve, const float* eref, float sign,
                                cudaStream_t s) {
  const long want = (n + 255) / 256;
  const int blocks = (int)(want < 1024 ? want : 1024);
  k_energy_shift<<<dim3(blocks, nsolve), 256, 0, s>>>(E, n, ss, eref, sign);
  return cudaGetLastError();
}

cudaError_t launch_step_control(const float* speed, double cfl, double hmin, const double* t, const double* tend,
                                int nsolve, double* dt, int* active, cudaStream_t s, double dt_cap) {
  k_step_control<<<(nsolve + 127) / 128, 128, 0, s>>>(speed, cfl, hmin, t, tend, nsolve, dt, active, dt_cap);
  return cudaGetLastError();
}

cudaError_t launch_step_advance(double* t, const double* dt, float* speed, const int* active, int* steps,
                                int nsolve, cudaStream_t s) {
  k_step_advance<<<(nsolve + 127) / 128, 128, 0, s>>>(t, dt, speed, active, steps, nsolve);
  return cudaGetLastError();
}

static int reduce_blocks(long cells, int nsolve) {
  const long per = (1184 + nsolve - 1) / nsolve;  // about 1184 blocks in total
  const long want = (cells + 255) / 256;
  return (int)(want < per ? want : (per > 0 ? per : 1));
}

cudaError_t launch_speed(int nd, const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                         cudaStream_t s, const float* eshift) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * nsolve, s);
  if (e != cudaSuccess) return e;
  const dim3 grid(reduce_blocks(cells, nsolve), nsolve);
  if (nd == 1) k_speed<1><<<grid, 256, 0, s>>>(U, cells, ss, gamma, eshift, out);
  else if (nd == 2) k_speed<2><<<grid, 256, 0, s>>>(U, cells, ss, gamma, eshift, out);
  else k_speed<3><<<grid, 256, 0, s>>>(U, cells, ss, gamma, eshift, out);
  return cudaGetLastError();
}

cudaError_t launch_conserved(int nd, const float* U, long cells, long ss, int nsolve, double gamma, double* out,
                             cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * (nd + 2) * nsolve, s);
  if (e != cudaSuccess) return e;
  const dim3 grid(reduce_blocks(cells, nsolve), nsolve);
  if (nd == 1) k_conserved<1><<<grid, 256, 0, s>>>(U, cells, ss, gamma, out);
  else if (nd == 2) k_conserved<2><<<grid, 256, 0, s>>>(U, cells, ss, gamma, out);
  else k_conserved<3><<<grid, 256, 0, s>>>(U, cells, ss, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_flux1d(const float* U, long n, long ss, int nsolve, float gamma, float* F, cudaStream_t s) {
  const int blocks = (int)((n + 255) / 256);
  for (int q = 0; q < nsolve; ++q) {
    k_flux1d<<<blocks, 256, 0, s>>>(U + (long)q * ss, n, gamma, F + (long)q * 3 * n);
  }
  return cudaGetLastError();
}

}  // namespace ps

namespace ps {

cudaError_t launch_speed_mhd(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                             cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * nsolve, s);
  if (e != cudaSuccess) return e;
  k_speed_mhd<<<dim3(reduce_blocks(cells, nsolve), nsolve), 256, 0, s>>>(U, cells, ss, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_speed_mhd1d(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                               cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * nsolve, s);
  if (e != cudaSuccess) return e;
  k_speed_mhd1d<<<dim3(reduce_blocks(cells, nsolve), nsolve), 256, 0, s>>>(U, cells, ss, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_project_mhd1d(float* U, long n, long ss, int nsolve, const int* active, cudaStream_t s) {
  k_project_mhd1d<<<nsolve, 256, 0, s>>>(U, n, ss, active);
  return cudaGetLastError();
}

cudaError_t launch_conserved_mhd(const float* U, long cells, long ss, int nsolve, double gamma, double* out,
                                 cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * 8 * nsolve, s);
  if (e != cudaSuccess) return e;
  k_conserved_mhd<<<dim3(reduce_blocks(cells, nsolve), nsolve), 256, 0, s>>>(U, cells, ss, gamma, out);
  return cudaGetLastError();
}

}  // namespace ps
