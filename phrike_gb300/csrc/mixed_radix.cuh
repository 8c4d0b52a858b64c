// Mixed-radix pencil passes for Fourier axes of any 2^a 3^b 5^c length up to
// 4096 (mixed_radix.cu).  The reference builds every Fourier axis from
// np.fft.fftfreq(N) for any N (phrike/grid.py:47-63, 87-115); the
// register-resident pencil transforms of the other pass kernels are compiled
// for powers of two, and plans with any other axis length run on these
// kernels instead.
//
// A pencil lives in shared memory and is transformed in place by a Stockham
// autosort FFT with radix-4, -3, -5 and -2 stages (decimation in time: inputs
// strided by N/R, twiddle W_N^{k r N/(Ns R)}, outputs at (j - k) R + k + r Ns
// for butterfly j, k = j mod Ns, Ns the product of the earlier radices).
// Every thread reads all its butterfly inputs into registers, the block
// synchronises, then the outputs are written back: one buffer per pencil.
//
// The passes keep the contracts of the power-of-two passes (same buffers,
// field layouts, operator tables and stage arithmetic), so the step loops,
// adaptive stepping and the operator entry points run on either:
//   op    : out = op(in) along one axis, pairs of real fields packed into one
//           complex transform (op: P, D, L, raw second derivative, or the
//           complementary filter in - IFFT((1/N - P) FFT in))
//   x     : optional fused filter P_x of the state, CFL speed, flux of the
//           state, G = [D_x F^x, P_x F^y (, P_x F^z)]
//   y3    : 3D middle axis: AB = [P_y G + D_y H^y, P_y H^z]
//   last  : -(P a + D b) along the last axis, gravity, RK stage update,
//           2D clamp, the last axis of the end-of-step filter
//   line1d: 1D stage: -D F(U), gravity, RK stage update and the 1D clamp
#pragma once
#include <cuda_runtime.h>

#include "pass_common.cuh"

namespace ps {

constexpr int kMrMaxStages = 14;  // 4 bits each in MrAxis::rcode
constexpr int kMrMaxLen = 4096;
constexpr int kMrMaxPencils = 64;  // pencils per CTA
#ifndef MR_DIV
#define MR_DIV 12
#endif
#ifndef MR_LB
#define MR_LB 768
#endif
#ifndef MR_MINB
#define MR_MINB 1
#endif
constexpr int kMrDiv = MR_DIV;         // values a thread holds per stage: ntp = ceil(n / kMrDiv)
constexpr int kMrThreads = MR_LB;      // threads per CTA at most
constexpr int kMrMinBlocks = MR_MINB;  // resident CTAs per SM the register allocation allows

// One Fourier axis: factorisation, threads per pencil and device tables.
struct MrAxis {
  int n;                     // pencil length
  int nst;                   // Stockham stages
  unsigned long long rcode;  // radix of stage s in bits [4s, 4s + 4)
  int ntp;                   // threads per pencil, ceil(n / kMrDiv)
  const float2* tw;          // W_n^q = exp(-2 pi i q / n), q < n
  const float* P;            // m s / n
  const float* d;            // kphys m s / n, zero at the Nyquist index of even n
};

// Pencils of one axis inside one solve: element i of pencil j sits at
// (j / es) * es * n + (j % es) + i * es.
struct MrGeom {
  int n;
  long es;    // element stride along the pencil (1 for x, nx for y, nx*ny for z)
  long npen;  // pencils per field
  int pg;     // pencils per CTA
  int threads;
  int smem;   // dynamic shared memory bytes
};

struct MrOpArgs {
  const float* in;
  float* out;
  int nf;
  long fs;             // elements per field
  long ss_in, ss_out;  // solve strides
  MrAxis ax;
  MrGeom g;
  int deriv;  // 0 P, 1 D, 2 L, 3 raw second derivative (op_symbol)
  float scale, kunit;
  int complement;
  const int* active;
};

struct MrXArgs {
  const float* U;
  float* Uw;   // fused filter P_x of the state (null: none)
  float* out;  // [nsolve][ND*NC][cells]
  long fs, ssU, ssOut;
  MrAxis ax;
  MrGeom g;
  int nd;
  float gamma;
  float* speed;
  const float* eref;
  const int* active;
  int shift_in;
};

struct MrY3Args {
  const float* G;  // 15 fields per solve
  float* out;      // 10 fields per solve
  long fs, ssG, ssOut;
  MrAxis ax;
  MrGeom g;
  const int* active;
};

struct MrLastArgs {
  const float* AB;
  int fa0, fb0;
  long ssAB;
  float* acc;
  float* out;
  const float* Un;
  const float* Uin;
  long fs, ssAcc, ssOut, ssUn;
  MrAxis ax;
  MrGeom g;
  int nd;
  int stage;
  const double* dt_dev;
  double dt;
  float gamma, rho_min, p_min;
  const float* eref;
  int filter_last;
  int clamp;
  int rk2;
  int gravity;
  float grav[3];
  const int* active;
};

struct MrLineArgs {
  const float* in;  // stage input [nsolve][3][n]
  float* out;
  float* acc;       // increments of the stage sum
  const float* Un;
  long ss;
  MrAxis ax;
  MrGeom g;
  int stage;
  const double* dt_dev;
  double dt;
  float gamma, rho_min, p_min;
  const float* eref;
  float gx;
  int rk2;
  const int* active;
};

// Radices (4 first, then 3, 5, 2) of n; false when n has another prime factor.
bool mr_factor(int n, int* radix, int* nst);
// Threads per pencil and pencils per CTA for a kernel needing `extra` bytes
// of shared memory per pencil beside its two complex signal buffers.
MrGeom mr_geom(const MrAxis& ax, long es, long npen, int extra_per_pencil);

cudaError_t launch_mr_op(const MrOpArgs& a, int nsolve, cudaStream_t s);
cudaError_t launch_mr_x(const MrXArgs& a, int nsolve, cudaStream_t s);
cudaError_t launch_mr_y3(const MrY3Args& a, int nsolve, cudaStream_t s);
cudaError_t launch_mr_last(const MrLastArgs& a, int nsolve, cudaStream_t s);
cudaError_t launch_mr_line(const MrLineArgs& a, int nsolve, cudaStream_t s);

}  // namespace ps
