// Legendre-Gauss-Lobatto (LGL) collocation on an LGL x LGL grid: device
// construction of nodes, weights and differentiation matrices in float64,
// wall boundary conditions, and the two contraction kernels of an RK stage
// (x flux . D_x^T; D_y . y flux fused with the stage update).
#pragma once
#include <cuda_runtime.h>

namespace ps {

// C[z][m][n] = alpha * sum_k A[z][m][k] B[z][n][k] with strided operands:
//   A[m][k] = a[z*az + m*am + k*ak],  B[n][k] = b[z*bz + n*bn + k*bk],
//   C[m][n] = c[z*cz + m*cm + n*cn].
struct GemmArgs {
  const void* a;
  const void* b;
  float* c;
  int M, N, K, batch;
  long am, ak, az, bn, bk, bz, cm, cn, cz;
  float alpha;
  const int* active;  // nullable: batch entry z is skipped when active[z / zper] == 0
  int zper;
  // Pencil offset: 1 subtracts A[m][0] from row m of A, 2 subtracts B[n][0]
  // from row n of B, before the product (exact for a matrix that annihilates
  // constants, such as a differentiation matrix, and it keeps the rounding of
  // the operand relative to its variation, not its size); add_back adds the
  // subtracted value to the output (for a matrix that preserves constants,
  // such as the nodal filter).
  int offset;
  int add_back;
};

// Operand storage / arithmetic of the generic contraction
enum GemmKind {
  kGemmF32 = 0,     // float A, float B, float accumulate
  kGemmF32F64 = 1,  // float A, double B, double accumulate
  kGemmF64F32 = 2,  // double A, float B, double accumulate
  kGemmSplitAB = 3, // float A and B split into bf16 hi + lo on load, hi*hi + hi*lo + lo*hi in float
};

// One RK stage (or a bare right-hand side) of an LGL x LGL Euler solve.  All
// field buffers are [nsolve][4][ny][nx] float32 (solve stride ss); the energy
// slot holds E' = E - eref[solve] (energy-perturbation form).
struct LglStageArgs {
  const float* U;      // stage input (walls already applied)
  float* Gx;           // d/dx of the x flux (written by the x kernel)
  const void* Dx;      // [nx][nx]: float (modes 0 and 2) or double (mode 1)
  const void* Dy;      // [ny][ny]
  int nx, ny;
  long ss;
  float gamma;
  const float* eref;   // per solve
  const int* active;   // per solve (null: all active)
  int stage;           // -1: out = rhs; 0..3: RK4 stage
  const float* Un;     // U^n
  float* acc;          // RK accumulator
  float* out;          // rhs, next stage input or new state
  const double* dt_dev;  // per-solve step sizes (null: dt)
  double dt;
  float rho_min, p_min;  // 2D clamp floors
  int nsolve;
  float g[2];            // constant gravity (solver.py:453-464); gravity = 0: off
  int gravity;
  int rk2;               // midpoint RK2 coefficients (stages 0 and 3 only)
};

cudaError_t launch_lgl_build(int n, double length, double* x, double* w, double* D, float* D32, cudaStream_t s);
cudaError_t launch_lgl_filter_matrix(int n, double length, const double* x, const double* w, int p, double alpha,
                                     double* F, float* F32, cudaStream_t s);
cudaError_t launch_gemm(const GemmArgs& g, GemmKind kind, bool a_kcontig, bool b_kcontig, cudaStream_t s);

cudaError_t launch_lgl_bc(float* U, int nx, int ny, long ss, int nsolve, const int* active, cudaStream_t s);
// mode: 0 float32, 1 float64, 2 split bf16 (both operands split into bf16 hi + lo
// on load; hi*hi + hi*lo + lo*hi accumulated in float32)
cudaError_t launch_lgl_x(const LglStageArgs& a, int mode, cudaStream_t s);
cudaError_t launch_lgl_y(const LglStageArgs& a, int mode, cudaStream_t s);

}  // namespace ps
