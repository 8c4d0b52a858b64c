// Split-bf16 x3 contractions of the LGL x LGL path on tcgen05 tensor cores
// (lgl_tc.cu): operand splitting, flux planes, the batched TMA-fed MMA kernel
// and the elementwise stage update.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace ps {

// hi/lo bf16 planes [2][rows][pitch] of a float32 matrix [rows][n]
cudaError_t launch_split_matrix(const float* M, int rows, int n, int pitch, void* out, cudaStream_t s);

// x flux F_x[solve, c][j][k] -> fx planes [2][nsolve*4*ny][px]; y flux
// transposed F_y^T[solve, c][i][j] -> fyt planes [2][nsolve*4][nx][py]
struct FluxSplitArgs {
  const float* U;  // [nsolve][4][ny][nx], energy slot E' = E - eref
  void* fx;        // __nv_bfloat16 planes
  void* fyt;
  int nx, ny, px, py, nsolve;
  float gamma;
  const float* eref;
  const int* active;
};
cudaError_t launch_flux_split(const FluxSplitArgs& a, cudaStream_t s);

// C[z][m][n] = alpha * sum_k A[z or 0][m][k] B[z or 0][n][k] (split bf16 x3,
// float32 accumulate), A and B from 4-D split-plane tensor maps.
struct UmmaArgs {
  float* C;
  long ldc, cz;
  int M, N, K, batch;
  int a_batched, b_batched;
  int c_trans;        // 1: element (m, n) stored at C[z*cz + n*ldc + m] (lanes along contiguous memory)
  const int* active;  // nullable: batch entry z skipped when active[z / zper] == 0
  int zper;
  float alpha;
  int* status;        // PS_STATUS_TMA_TIMEOUT on a wait that ran out
};
// tensor map over split planes [2][batch][rows][pitch] with a 64 x box_rows box
int encode_split_map(CUtensorMap* m, const void* base, int nk, int rows, int batch, int pitch, int box_rows);
// N tile (64, 128, 176 or 256 columns) for an M x N x batch problem: the
// smallest whose grid fits in one wave of resident CTAs, else 256
int umma_n_tile(int M, int N, int batch);
cudaError_t launch_umma_x3(const CUtensorMap& mA, const CUtensorMap& mB, const UmmaArgs& g, int nt, cudaStream_t s);

// k = ksign (Gx + Gy) (LGL: ksign = -1; a Fourier right-hand side R passed
// as Gx with Gy null: ksign = 1); stage -1 writes k, stages 0..3 the RK4
// update and the 2D clamp
struct LglUpdateArgs {
  const float* Gx;
  const float* Gy;    // may be null
  float ksign;
  const float* Un;
  float* acc;
  float* out;
  long cells;
  int nsolve;
  int stage;
  const double* dt_dev;
  double dt;
  float gamma, rho_min, p_min;
  const float* eref;
  const int* active;
  const float* Uin;  // stage input (gravity source)
  float g[2];
  int gravity;
  int rk2;  // midpoint RK2 coefficients (stages 0 and 3 only)
};
cudaError_t launch_lgl_update(const LglUpdateArgs& a, cudaStream_t s);

}  // namespace ps
