// 1D Legendre-Gauss-Lobatto collocation (lgl1d.cu): whole-step kernel,
// matrix application along the nodes, boundary conditions.
#pragma once
#include <cuda_runtime.h>

namespace ps {

// Boundary codes per (side, variable), index side * 3 + var with sides
// (left, right) and variables (density, momentum, energy):
// 0 copy the neighbouring interior value, 1 set to zero, 2 leave unchanged.
struct Bc1D {
  int c[6];
};

struct Lgl1DArgs {
  float* U;              // [nsolve][3][n]
  long solve_stride;
  int n;
  const void* DT;        // D^T [n][n] (float or double)
  const void* FT;        // nodal filter transposed, null when the filter is off
  Bc1D bc;
  int nsteps;
  const double* dt_dev;
  double dt;
  const int* active;
  float gamma, rho_min, p_min;
  float gx;              // gravity along x
  int filter_interval;
  int step_counter0;
  double* t;             // CFL mode
  const double* tend;
  float cfl, hmin;
  int* steps_done;
  float* rhs_out;        // non-null: write rhs(U) only
  int rk2;
};

size_t lgl1d_smem(int n, bool fp64);
cudaError_t launch_lgl1d(const Lgl1DArgs& a, bool fp64, int nsolve, cudaStream_t s);
// out[f] = M in[f] for nf fields of n nodes per solve (MT = M^T; rowsum = the
// row sum of M, 0 for D and 1 for the filter)
cudaError_t launch_lgl1d_apply(const void* MT, bool fp64, const float* in, float* out, int n, int nf, int nsolve,
                               long ss, float rowsum, cudaStream_t s);
cudaError_t launch_transpose(const void* in, void* out, int n, bool fp64, cudaStream_t s);
cudaError_t launch_lgl1d_bc(float* U, int n, long ss, int nsolve, const Bc1D& bc, const int* active,
                            cudaStream_t s);

}  // namespace ps
