// LGL collocation kernels (declared in lgl.cuh).
//
// Node construction follows the published Newton iteration for LGL points as
// roots of q = L_{p+1} - L_{p-1}, q' = (2p+1) L_p, started from the asymptotic
// guess -cos((j + 1/4) pi / p - 3 / (8 p pi (j + 1/4))) (Kopriva, "Implementing
// Spectral Methods for PDEs", 2009, algorithms 24-25).  The differentiation
// matrix is the closed form D_ij = L_p(x_i) / (L_p(x_j) (x_i - x_j)) with the
// diagonal from the negative row sum.  The reference builds the same nodes
// from scipy's Jacobi(1,1) roots and D by a Vandermonde solve
// (phrike/basis/legendre.py:523-624, 694-729); the two agree to rounding.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "lgl.cuh"
#include "pass_common.cuh"

namespace ps {

// ---------------------------------------------------------------------------
// Construction (float64)
// ---------------------------------------------------------------------------

// q = L_{p+1}(x) - L_{p-1}(x), dq = q'(x) and L_p(x) by the three-term recurrence
__device__ void lgl_q_and_l(int p, double x, double& q, double& dq, double& Lp) {
  double lm2 = 1.0, lm1 = x, dm2 = 0.0, dm1 = 1.0;
  for (int k = 2; k <= p; ++k) {
    const double lk = ((2.0 * k - 1.0) / k) * x * lm1 - ((k - 1.0) / k) * lm2;
    const double dk = dm2 + (2.0 * k - 1.0) * lm1;
    lm2 = lm1;
    lm1 = lk;
    dm2 = dm1;
    dm1 = dk;
  }
  // lm1 = L_p, lm2 = L_{p-1}, dm1 = L'_p, dm2 = L'_{p-1}
  const double lp1 = ((2.0 * p + 1.0) / (p + 1.0)) * x * lm1 - (p / (p + 1.0)) * lm2;
  const double dp1 = dm2 + (2.0 * p + 1.0) * lm1;
  q = lp1 - lm2;
  dq = dp1 - dm2;
  Lp = lm1;
}

// Nodes xi_j ascending on [-1, 1], weights w_j = 2 / (p (p+1) L_p(xi_j)^2),
// physical nodes x_j = (xi_j + 1) L / 2.  Interior nodes come in +- pairs;
// each thread solves for the one in (-1, 0) and mirrors it.
__global__ void k_lgl_nodes(int n, double length, double* x, double* w) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int p = n - 1;
  double xi, Lp;
  if (j == 0 || j == p) {
    xi = (j == 0) ? -1.0 : 1.0;
    Lp = 1.0;  // |L_p(+-1)| = 1
  } else if (2 * j == p) {
    double q, dq;
    xi = 0.0;
    lgl_q_and_l(p, 0.0, q, dq, Lp);
  } else {
    const int jj = (j < p - j) ? j : p - j;
    const double pi = 3.14159265358979323846;
    double t = -cos((jj + 0.25) * pi / p - 3.0 / (8.0 * p * pi * (jj + 0.25)));
    double q = 0.0, dq = 1.0;
    for (int it = 0; it < 100; ++it) {
      lgl_q_and_l(p, t, q, dq, Lp);
      const double delta = -q / dq;
      t += delta;
      if (fabs(delta) <= 1e-15 * fabs(t)) break;
    }
    lgl_q_and_l(p, t, q, dq, Lp);
    xi = (j < p - j) ? t : -t;
  }
  if (x) x[j] = (xi + 1.0) * 0.5 * length;
  if (w) w[j] = 2.0 / (p * (p + 1.0) * Lp * Lp);
}

// D_x = (2/L) D_xi.  L_p alternates in sign along the LGL nodes, so
// L_p(xi_i) / L_p(xi_j) = (-1)^(j-i) sqrt(w_j / w_i).  One CTA per row.
__global__ void k_lgl_dmatrix(int n, double length, const double* __restrict__ x, const double* __restrict__ w,
                              double* D, float* D32) {
  const int i = blockIdx.x;
  const double scale = 2.0 / length;
  const double xi_i = 2.0 * x[i] / length - 1.0;
  double rowsum = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    if (j == i) continue;
    const double xi_j = 2.0 * x[j] / length - 1.0;
    const double ratio = (((j - i) & 1) ? -1.0 : 1.0) * sqrt(w[j] / w[i]);
    const double v = scale * ratio / (xi_i - xi_j);
    if (D) D[(long)i * n + j] = v;
    if (D32) D32[(long)i * n + j] = (float)v;
    rowsum += v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) rowsum += __shfl_xor_sync(0xffffffffu, rowsum, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = rowsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    if (D) D[(long)i * n + i] = -s;
    if (D32) D32[(long)i * n + i] = (float)(-s);
  }
}

// Nodal filter Fn = (V diag(sigma_k (2k+1)/2) V^T) diag(w) with V[j][k] =
// P_k(y_j) on the reference coordinate y = -xi (the reference orders y
// descending, which is this x order), sigma_k = exp(-alpha (k/(n-1))^p)
// (legendre.py:825-841).  One thread per entry.
__global__ void k_lgl_filter(int n, double length, const double* __restrict__ x, const double* __restrict__ w,
                             int pexp, double alpha, double* F, float* F32) {
  const int i = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double yi = 1.0 - 2.0 * x[i] / length, yj = 1.0 - 2.0 * x[j] / length;
  const double kmax = (n - 1 > 1) ? (double)(n - 1) : 1.0;
  double pi0 = 1.0, pi1 = yi, pj0 = 1.0, pj1 = yj;
  double s = 0.0;
  for (int k = 0; k < n; ++k) {
    double Pik, Pjk;
    if (k == 0) {
      Pik = Pjk = 1.0;
    } else if (k == 1) {
      Pik = yi;
      Pjk = yj;
    } else {
      Pik = ((2.0 * k - 1.0) * yi * pi1 - (k - 1.0) * pi0) / k;
      Pjk = ((2.0 * k - 1.0) * yj * pj1 - (k - 1.0) * pj0) / k;
      pi0 = pi1;
      pi1 = Pik;
      pj0 = pj1;
      pj1 = Pjk;
    }
    const double sig = exp(-alpha * pow(k / kmax, (double)pexp));
    s += Pik * sig * (2.0 * k + 1.0) * 0.5 * Pjk;
  }
  const double v = s * w[j];
  F[(long)i * n + j] = v;
  if (F32) F32[(long)i * n + j] = (float)v;
}

cudaError_t launch_lgl_build(int n, double length, double* x, double* w, double* D, float* D32, cudaStream_t s) {
  k_lgl_nodes<<<(n + 127) / 128, 128, 0, s>>>(n, length, x, w);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || (D == nullptr && D32 == nullptr)) return e;
  k_lgl_dmatrix<<<n, 256, 0, s>>>(n, length, x, w, D, D32);
  return cudaGetLastError();
}

cudaError_t launch_lgl_filter_matrix(int n, double length, const double* x, const double* w, int p, double alpha,
                                     double* F, float* F32, cudaStream_t s) {
  k_lgl_filter<<<dim3((n + 127) / 128, n), 128, 0, s>>>(n, length, x, w, p, alpha, F, F32);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Arithmetic modes of the contractions
// ---------------------------------------------------------------------------

// bf16 rounding of a float, returned as the float it represents
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// MODE 0: float; 1: double; 2: split bf16 (values kept as floats that are
// exactly representable in bf16, so the product of two of them is exact).
template <int MODE>
using compute_t = typename std::conditional<MODE == 1, double, float>::type;

// Stores operand value v into plane 0 (and its bf16 low part into plane 1).
template <int MODE, typename T>
__device__ __forceinline__ void split_store(T* hi, T* lo, T v) {
  if constexpr (MODE == 2) {
    const float h = bf16r(v);
    *hi = h;
    *lo = bf16r(v - h);
  } else {
    *hi = v;
  }
}

// acc += a * b in the mode's arithmetic; planes [0] = hi (or value), [1] = lo
template <int MODE, typename T>
__device__ __forceinline__ T mac(T acc, T ahi, T alo, T bhi, T blo) {
  if constexpr (MODE == 2) {
    acc = fmaf(ahi, bhi, acc);
    acc = fmaf(ahi, blo, acc);
    return fmaf(alo, bhi, acc);
  } else {
    return fma(ahi, bhi, acc);
  }
}

// 2D Euler flux along AXIS (0 = x, 1 = y) in energy-perturbation form: e is
// the stored E' = E - eref, p' = (gamma-1)(E' - rho|u|^2/2) = p - (gamma-1) eref,
// momentum flux with p' (a constant offset, annihilated by D), energy flux
// (E' + p' + gamma eref) u = (E + p) u (equations.py:322-359).
template <int AXIS, typename T>
__device__ __forceinline__ void euler_flux2(float r, float mx, float my, float e, T gm1, T geref, T (&f)[4]) {
  const T rho = r;
  const T ux = (T)mx / rho, uy = (T)my / rho;
  const T pp = gm1 * ((T)e - T(0.5) * rho * (ux * ux + uy * uy));
  const T un = (AXIS == 0) ? ux : uy;
  f[0] = rho * un;
  f[1] = rho * ux * un + ((AXIS == 0) ? pp : T(0));
  f[2] = rho * uy * un + ((AXIS == 1) ? pp : T(0));
  f[3] = ((T)e + pp + geref) * un;
}

// ---------------------------------------------------------------------------
// Stage kernels
// ---------------------------------------------------------------------------
constexpr int kLglBK = 16;

// Gx[c][j][i] = sum_k Fx_c(U[:, j, k]) Dx[i][k]: rows j (M), columns i (N),
// the x flux computed while its tile is staged.  Thread (tr, tc) owns rows
// tr + NTR*m and columns tc + NTC*q of the CTA tile.
template <int MODE, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_lgl_x(LglStageArgs a) {
  using T = compute_t<MODE>;
  constexpr int NTR = BM / TM, NTC = BN / TN, NT = NTR * NTC, BK = kLglBK, NS = (MODE == 2) ? 2 : 1;
  __shared__ T As[NS][4][BK][BM + 1];
  __shared__ T Bs[NS][BK][BN + 1];
  const int sol = blockIdx.z;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const int nx = a.nx, ny = a.ny;
  const long cells = (long)nx * ny;
  const float* __restrict__ U = a.U + (long)sol * a.ss;
  const T* __restrict__ D = static_cast<const T*>(a.Dx);
  const int j0 = blockIdx.y * BM, i0 = blockIdx.x * BN;
  const int tr = threadIdx.x / NTC, tc = threadIdx.x % NTC;
  const T gm1 = (T)a.gamma - T(1), geref = (T)a.gamma * (T)a.eref[sol];
  T acc[4][TM][TN];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int m = 0; m < TM; ++m)
#pragma unroll
      for (int q = 0; q < TN; ++q) acc[c][m][q] = T(0);
  for (int k0 = 0; k0 < nx; k0 += BK) {
    for (int idx = threadIdx.x; idx < BM * BK; idx += NT) {
      const int r = idx / BK, kk = idx % BK, j = j0 + r, k = k0 + kk;
      T f[4] = {T(0), T(0), T(0), T(0)};
      if (j < ny && k < nx) {
        const long o = (long)j * nx + k;
        euler_flux2<0, T>(U[o], U[cells + o], U[2 * cells + o], U[3 * cells + o], gm1, geref, f);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) split_store<MODE, T>(&As[0][c][kk][r], &As[NS - 1][c][kk][r], f[c]);
    }
    for (int idx = threadIdx.x; idx < BN * BK; idx += NT) {
      const int n = idx / BK, kk = idx % BK, i = i0 + n, k = k0 + kk;
      const T v = (i < nx && k < nx) ? D[(long)i * nx + k] : T(0);
      split_store<MODE, T>(&Bs[0][kk][n], &Bs[NS - 1][kk][n], v);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      T bh[TN], bl[TN];
#pragma unroll
      for (int q = 0; q < TN; ++q) {
        bh[q] = Bs[0][kk][tc + NTC * q];
        bl[q] = Bs[NS - 1][kk][tc + NTC * q];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int m = 0; m < TM; ++m) {
          const T ah = As[0][c][kk][tr + NTR * m], al = As[NS - 1][c][kk][tr + NTR * m];
#pragma unroll
          for (int q = 0; q < TN; ++q) acc[c][m][q] = mac<MODE, T>(acc[c][m][q], ah, al, bh[q], bl[q]);
        }
    }
    __syncthreads();
  }
  float* G = a.Gx + (long)sol * a.ss;
#pragma unroll
  for (int m = 0; m < TM; ++m) {
    const int j = j0 + tr + NTR * m;
    if (j >= ny) continue;
#pragma unroll
    for (int q = 0; q < TN; ++q) {
      const int i = i0 + tc + NTC * q;
      if (i >= nx) continue;
      const long o = (long)j * nx + i;
#pragma unroll
      for (int c = 0; c < 4; ++c) G[c * cells + o] = (float)acc[c][m][q];
    }
  }
}

// Gy[c][j][i] = sum_k Dy[j][k] Fy_c(U[:, k, i]) and the epilogue
// k = -(Gx + Gy): the bare right-hand side (stage -1) or the RK4 stage update
// with the 2D positivity clamp (solver.py:428-466, 623-648).
template <int MODE, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) k_lgl_y(LglStageArgs a) {
  using T = compute_t<MODE>;
  constexpr int NTR = BM / TM, NTC = BN / TN, NT = NTR * NTC, BK = kLglBK, NS = (MODE == 2) ? 2 : 1;
  __shared__ T As[NS][BK][BM + 1];
  __shared__ T Bs[NS][4][BK][BN + 1];
  const int sol = blockIdx.z;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const int nx = a.nx, ny = a.ny;
  const long cells = (long)nx * ny;
  const float* __restrict__ U = a.U + (long)sol * a.ss;
  const T* __restrict__ D = static_cast<const T*>(a.Dy);
  const int j0 = blockIdx.y * BM, i0 = blockIdx.x * BN;
  const int tr = threadIdx.x / NTC, tc = threadIdx.x % NTC;
  const T gm1 = (T)a.gamma - T(1), geref = (T)a.gamma * (T)a.eref[sol];
  T acc[4][TM][TN];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int m = 0; m < TM; ++m)
#pragma unroll
      for (int q = 0; q < TN; ++q) acc[c][m][q] = T(0);
  for (int k0 = 0; k0 < ny; k0 += BK) {
    for (int idx = threadIdx.x; idx < BM * BK; idx += NT) {
      const int r = idx / BK, kk = idx % BK, j = j0 + r, k = k0 + kk;
      const T v = (j < ny && k < ny) ? D[(long)j * ny + k] : T(0);
      split_store<MODE, T>(&As[0][kk][r], &As[NS - 1][kk][r], v);
    }
    for (int idx = threadIdx.x; idx < BN * BK; idx += NT) {
      const int kk = idx / BN, n = idx % BN, k = k0 + kk, i = i0 + n;
      T f[4] = {T(0), T(0), T(0), T(0)};
      if (k < ny && i < nx) {
        const long o = (long)k * nx + i;
        euler_flux2<1, T>(U[o], U[cells + o], U[2 * cells + o], U[3 * cells + o], gm1, geref, f);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) split_store<MODE, T>(&Bs[0][c][kk][n], &Bs[NS - 1][c][kk][n], f[c]);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      T ah[TM], al[TM];
#pragma unroll
      for (int m = 0; m < TM; ++m) {
        ah[m] = As[0][kk][tr + NTR * m];
        al[m] = As[NS - 1][kk][tr + NTR * m];
      }
#pragma unroll
      for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < TN; ++q) {
          const T bh = Bs[0][c][kk][tc + NTC * q], bl = Bs[NS - 1][c][kk][tc + NTC * q];
#pragma unroll
          for (int m = 0; m < TM; ++m) acc[c][m][q] = mac<MODE, T>(acc[c][m][q], ah[m], al[m], bh, bl);
        }
    }
    __syncthreads();
  }
  const long so = (long)sol * a.ss;
  const float* __restrict__ Gx = a.Gx + so;
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  const float pmin_shift = a.p_min - (a.gamma - 1.0f) * a.eref[sol];
#pragma unroll
  for (int m = 0; m < TM; ++m) {
    const int j = j0 + tr + NTR * m;
    if (j >= ny) continue;
#pragma unroll
    for (int q = 0; q < TN; ++q) {
      const int i = i0 + tc + NTC * q;
      if (i >= nx) continue;
      const long o = (long)j * nx + i;
      // the point's loads before its stores (a store between them would make
      // each component wait for the previous one's round trip to memory)
      float gx[4], un[4], ac[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long g = so + c * cells + o;
        gx[c] = Gx[c * cells + o];
        un[c] = (a.stage >= 0) ? a.Un[g] : 0.0f;
        ac[c] = (a.stage >= 1) ? a.acc[g] : 0.0f;
      }
      float grho = 0.0f, gmx = 0.0f, gmy = 0.0f;
      if (a.gravity) {
        grho = U[o];
        gmx = U[cells + o];
        gmy = U[2 * cells + o];
      }
      float k[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) k[c] = -(gx[c] + (float)acc[c][m][q]);
      if (a.gravity) {  // rho g on the momenta, g . m on the energy, from the stage input
        k[1] = fmaf(grho, a.g[0], k[1]);
        k[2] = fmaf(grho, a.g[1], k[2]);
        k[3] += a.g[0] * gmx + a.g[1] * gmy;
      }
      if (a.stage < 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) a.out[so + c * cells + o] = k[c];
        continue;
      }
      float u[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) u[c] = rk_update_incr(a.stage, rk, k[c], un[c], ac[c]);
      if (a.stage != 3) {
#pragma unroll
        for (int c = 0; c < 4; ++c) a.acc[so + c * cells + o] = ac[c];
      }
      clamp_state<2>(u, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
      for (int c = 0; c < 4; ++c) a.out[so + c * cells + o] = u[c];
    }
  }
}

// Large tiles when they already give about one CTA per SM, else small ones.
// Tile of the CUDA-core contractions: 32 x 64 outputs per 256-thread CTA
// once those fill four waves of the SMs, else 16 x 32 per 128 threads once
// those fill two, else 8 x 32 per 128 threads: one CTA per SM leaves the
// contraction latency-bound, and smaller tiles put more warps on each SM.
// Measured (one solve, ms per RK4 step, FP32 / FP64): 257^2 0.40 / 3.28 with
// the 16 x 32 tile, 0.35 / 2.21 with 8 x 32; 513^2 1.02 / 20.1 with 32 x 64,
// 0.82 / 12.6 with 16 x 32 (0.99 / 15.3 with 8 x 32).
static int tile_kind(int nx, int ny, int nsolve) {
  const long big = (long)((nx + 63) / 64) * ((ny + 31) / 32) * nsolve;
  const long small = (long)((nx + 31) / 32) * ((ny + 15) / 16) * nsolve;
  return big >= 4 * 148 ? 0 : (small >= 2 * 148 ? 1 : 2);
}

template <int MODE>
static cudaError_t lgl_x_mode(const LglStageArgs& a, cudaStream_t s) {
  const int k = tile_kind(a.nx, a.ny, a.nsolve);
  if (k == 0) {
    const dim3 grid((a.nx + 63) / 64, (a.ny + 31) / 32, a.nsolve);
    k_lgl_x<MODE, 32, 64, 2, 4><<<grid, 256, 0, s>>>(a);
  } else if (k == 1) {
    const dim3 grid((a.nx + 31) / 32, (a.ny + 15) / 16, a.nsolve);
    k_lgl_x<MODE, 16, 32, 2, 2><<<grid, 128, 0, s>>>(a);
  } else {
    const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, a.nsolve);
    k_lgl_x<MODE, 8, 32, 1, 2><<<grid, 128, 0, s>>>(a);
  }
  return cudaGetLastError();
}

template <int MODE>
static cudaError_t lgl_y_mode(const LglStageArgs& a, cudaStream_t s) {
  const int k = tile_kind(a.nx, a.ny, a.nsolve);
  if (k == 0) {
    const dim3 grid((a.nx + 63) / 64, (a.ny + 31) / 32, a.nsolve);
    k_lgl_y<MODE, 32, 64, 4, 2><<<grid, 256, 0, s>>>(a);
  } else if (k == 1) {
    const dim3 grid((a.nx + 31) / 32, (a.ny + 15) / 16, a.nsolve);
    k_lgl_y<MODE, 16, 32, 2, 2><<<grid, 128, 0, s>>>(a);
  } else {
    const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, a.nsolve);
    k_lgl_y<MODE, 8, 32, 1, 2><<<grid, 128, 0, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_lgl_x(const LglStageArgs& a, int mode, cudaStream_t s) {
  if (mode == 1) return lgl_x_mode<1>(a, s);
  if (mode == 2) return lgl_x_mode<2>(a, s);
  return lgl_x_mode<0>(a, s);
}

cudaError_t launch_lgl_y(const LglStageArgs& a, int mode, cudaStream_t s) {
  if (mode == 1) return lgl_y_mode<1>(a, s);
  if (mode == 2) return lgl_y_mode<2>(a, s);
  return lgl_y_mode<0>(a, s);
}

// ---------------------------------------------------------------------------
// Wall boundary conditions (grid.py:1004-1039, 1072-1154, bc "dirichlet"):
// left, right, top, bottom in that order; density, tangential momentum and
// energy copy the neighbouring line (Neumann), the normal momentum is 0.
// One CTA per solve: columns first, then rows (which read the columns'
// results at the corners).
// ---------------------------------------------------------------------------
__global__ void k_lgl_bc(float* U, int nx, int ny, long ss, const int* active) {
  const int sol = blockIdx.x;
  if (active != nullptr && active[sol] == 0) return;
  float* u = U + (long)sol * ss;
  const long cells = (long)nx * ny;
  // Each row's (column's) interior neighbours are loaded before its wall
  // values are stored: the walls never overwrite what they copy, and loads
  // issued behind possibly aliasing stores would each wait a round trip.
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    const long l = (long)j * nx, r = l + nx - 1;
    const float l0 = u[l + 1], l2 = u[2 * cells + l + 1], l3 = u[3 * cells + l + 1];
    const float r0 = u[r - 1], r2 = u[2 * cells + r - 1], r3 = u[3 * cells + r - 1];
    u[l] = l0;
    u[cells + l] = 0.0f;
    u[2 * cells + l] = l2;
    u[3 * cells + l] = l3;
    u[r] = r0;
    u[cells + r] = 0.0f;
    u[2 * cells + r] = r2;
    u[3 * cells + r] = r3;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const long t = (long)(ny - 1) * nx + i, b = i;
    const float t0 = u[t - nx], t1 = u[cells + t - nx], t3 = u[3 * cells + t - nx];
    const float b0 = u[b + nx], b1 = u[cells + b + nx], b3 = u[3 * cells + b + nx];
    u[t] = t0;
    u[cells + t] = t1;
    u[2 * cells + t] = 0.0f;
    u[3 * cells + t] = t3;
    u[b] = b0;
    u[cells + b] = b1;
    u[2 * cells + b] = 0.0f;
    u[3 * cells + b] = b3;
  }
}

cudaError_t launch_lgl_bc(float* U, int nx, int ny, long ss, int nsolve, const int* active, cudaStream_t s) {
  k_lgl_bc<<<nsolve, 512, 0, s>>>(U, nx, ny, ss, active);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Generic strided contraction (derivatives and filters of arbitrary fields):
// 64 x 64 output tile, k-tiles of 16, 256 threads with 4 x 4 outputs each
// (rows ty + 16 m, columns tx + 16 q).
// ---------------------------------------------------------------------------
template <typename TA, typename TB, typename TC, int MODE, bool AK, bool BK>
__global__ void __launch_bounds__(256) k_gemm(GemmArgs g) {
  constexpr int BMg = 64, BNg = 64, BKg = 16, NS = (MODE == 2) ? 2 : 1;
  __shared__ TC As[NS][BKg][BMg + 1];
  __shared__ TC Bs[NS][BKg][BNg + 1];
  if (g.active != nullptr && g.active[blockIdx.z / g.zper] == 0) return;
  const TA* __restrict__ A = static_cast<const TA*>(g.a) + blockIdx.z * g.az;
  const TB* __restrict__ Bm = static_cast<const TB*>(g.b) + blockIdx.z * g.bz;
  float* C = g.c + blockIdx.z * g.cz;
  const int m0 = blockIdx.y * BMg, n0 = blockIdx.x * BNg;
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  TC acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = TC(0);
  for (int k0 = 0; k0 < g.K; k0 += BKg) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + 256 * q;
      int r, c;
      if (AK) {
        r = idx / BKg;
        c = idx % BKg;
      } else {
        c = idx / BMg;
        r = idx % BMg;
      }
      const int m = m0 + r, k = k0 + c;
      TC va = TC(0);
      if (m < g.M && k < g.K) {
        va = (TC)A[m * g.am + k * g.ak];
        if (g.offset == 1) va -= (TC)A[m * g.am];
      }
      split_store<MODE, TC>(&As[0][c][r], &As[NS - 1][c][r], va);
      if (BK) {
        r = idx / BKg;
        c = idx % BKg;
      } else {
        c = idx / BNg;
        r = idx % BNg;
      }
      const int n = n0 + r, k2 = k0 + c;
      TC vb = TC(0);
      if (n < g.N && k2 < g.K) {
        vb = (TC)Bm[n * g.bn + k2 * g.bk];
        if (g.offset == 2) vb -= (TC)Bm[n * g.bn];
      }
      split_store<MODE, TC>(&Bs[0][c][r], &Bs[NS - 1][c][r], vb);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BKg; ++kk) {
      TC ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ah[i] = As[0][kk][ty + 16 * i];
        al[i] = As[NS - 1][kk][ty + 16 * i];
        bh[i] = Bs[0][kk][tx + 16 * i];
        bl[i] = Bs[NS - 1][kk][tx + 16 * i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = mac<MODE, TC>(acc[i][j], ah[i], al[i], bh[j], bl[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
    const TC base_a = (g.add_back && g.offset == 1) ? (TC)A[m * g.am] : TC(0);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      const TC base = (g.add_back && g.offset == 2) ? (TC)Bm[n * g.bn] : base_a;
      C[m * g.cm + n * g.cn] = (float)((TC)g.alpha * acc[i][j] + base);
    }
  }
}

template <typename TA, typename TB, typename TC, int MODE>
static cudaError_t gemm_t(const GemmArgs& g, bool ak, bool bk, cudaStream_t s) {
  const dim3 grid((g.N + 63) / 64, (g.M + 63) / 64, g.batch);
  if (ak && bk) k_gemm<TA, TB, TC, MODE, true, true><<<grid, 256, 0, s>>>(g);
  else if (ak) k_gemm<TA, TB, TC, MODE, true, false><<<grid, 256, 0, s>>>(g);
  else if (bk) k_gemm<TA, TB, TC, MODE, false, true><<<grid, 256, 0, s>>>(g);
  else k_gemm<TA, TB, TC, MODE, false, false><<<grid, 256, 0, s>>>(g);
  return cudaGetLastError();
}

cudaError_t launch_gemm(const GemmArgs& g, GemmKind kind, bool ak, bool bk, cudaStream_t s) {
  switch (kind) {
    case kGemmF32F64: return gemm_t<float, double, double, 1>(g, ak, bk, s);
    case kGemmF64F32: return gemm_t<double, float, double, 1>(g, ak, bk, s);
    case kGemmSplitAB: return gemm_t<float, float, float, 2>(g, ak, bk, s);
    default: return gemm_t<float, float, float, 0>(g, ak, bk, s);
  }
}

}  // namespace ps
