// 3D ideal and resistive MHD (MHDEquations3D, SpectralSolverMHD3D:
// equations.py:911-1100, solver.py:840-1049, 1173-1174; Grid3D.project_solenoidal,
// grid.py:1649-1684).
//
// Right-hand side.  An elementwise flux kernel writes the three 8-component
// fluxes Fx, Fy, Fz; one-axis operator passes then form dx1 Fx = D_x P_y P_z Fx,
// dy1 Fy = P_x D_y P_z Fy and dz1 Fz = P_x P_y D_z Fz in place (the separable
// factorisation of the masked spectral derivatives); an elementwise update
// kernel sums them, adds eta lap B and nu lap(rho u) (lap = L_x P_y P_z +
// P_x L_y P_z + P_x P_y L_z on copies of the six fields) and applies the RK
// stage with the MHD clamp.
//
// Projection.  B_hat -= k (k . B_hat) / |k|^2 with the Nyquist planes zeroed is
// not separable, so it runs as a real 3D transform: x rows to half spectra
// (kx = 0..Nx/2), complex y pencils forward, complex z pencils forward +
// projection + inverse (all three components per thread), y pencils inverse,
// x rows back by Hermitian symmetry, with E updated at fixed thermal pressure.
#pragma once
#include <cuda_runtime.h>

#include "pass_common.cuh"

namespace ps {

struct Mhd3FluxArgs {
  const float* U;     // [nsolve][8][cells]
  float* F;           // [3][nsolve][8][cells]: Fx, Fy, Fz blocks
  float* dif;         // nullable: [3][nsolve][6][cells] copies of (rho u, B) for the Laplacians
  long cells;
  int nsolve;
  float gamma;
  float* speed;       // nullable: per-solve max(|ux|,|uy|,|uz|) + sqrt(a^2 + b^2)
  const int* active;  // nullable per-solve flags
};

struct Mhd3UpdateArgs {
  const float* F;     // the three blocks after the operator passes, or (rhs_in) the right-hand side
  int rhs_in;         // 1: F is one 8-field block holding the right-hand side itself (2D)
  const float* dif;   // nullable: the three Laplacian blocks
  float eta, nu;
  const float* Un;    // U^n
  float* acc;         // RK accumulator
  float* out;         // next stage input / new state / (stage < 0) the right-hand side
  long cells;
  int nsolve;
  int stage;          // -1: right-hand side only; 0..3 RK stage
  int rk2;
  const double* dt_dev;
  double dt;
  float gamma, rho_min, p_min;
  const int* active;
};

struct Proj3Args {
  float* B[3];        // Bx, By, Bz of solve 0; solve s at + s * ss
  float* E;           // nullable: E += (|B_new|^2 - |B_old|^2) / 2
  long ss;            // solve stride of B and E
  float2* H;          // half spectra [nsolve][3][nz][ny][hx]
  int nx, ny, nz, hx;
  int nsolve;
  AxisOps ax;         // tables of the transformed axis
  float k0x, k0y, k0z;  // 2 pi / L per axis
  const int* active;
};

cudaError_t launch_mhd3_flux(const Mhd3FluxArgs& a, cudaStream_t s);
cudaError_t launch_mhd3_update(const Mhd3UpdateArgs& a, cudaStream_t s);
cudaError_t launch_speed_mhd3(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                              cudaStream_t s);
// the five projection passes; n = the pencil length of the pass
cudaError_t launch_proj3_xf(int n, const Proj3Args& a, cudaStream_t s);
cudaError_t launch_proj3_y(int n, bool inverse, const Proj3Args& a, cudaStream_t s);
cudaError_t launch_proj3_z(int n, const Proj3Args& a, cudaStream_t s);
cudaError_t launch_proj3_xi(int n, const Proj3Args& a, cudaStream_t s);
bool mhd3_supported_n(int n);

}  // namespace ps
