// Pencil pass kernels of the 2D (2.5D) ideal MHD right-hand side and of the
// Helmholtz (Leray) projection of the magnetic field.
//
// State: 8 components [rho, rho ux, rho uy, rho uz, E, Bx, By, Bz]
// (equations.py:770-810).  The right-hand side -(dx1 Fx + dy1 Fy) factors
// exactly like the Euler one (euler_passes.cuh): the x pass writes D_x Fx and
// P_x Fy (16 fields), the strided last pass evaluates -(P_y G + D_y H) and
// the RK4 stage update with the MHD clamp (passes_tma.cuh, PHYS = 1).
//
// The projection (grid.py:1297-1327) is not separable (it divides by
// kx^2 + ky^2), so it runs as a real 2D transform in three passes:
//   k_proj_xf   rows: FFT_x of Bx and By, half spectra kx = 0..Nx/2 stored
//   k_proj_y    columns kx: FFT_y, Nyquist row/column zeroed,
//               B_hat -= k (k . B_hat)/|k|^2, inverse FFT_y, 1/(Nx Ny)
//   k_proj_xi   rows: rebuild the full x spectra by Hermitian symmetry,
//               Bx + i By in one inverse FFT_x, and E updated with the
//               thermal pressure held fixed (solver.py:966-986):
//               E += (|B_new|^2 - |B_old|^2)/2.
#pragma once
#include "pass_common.cuh"

namespace ps {

// ---------------------------------------------------------------------------
// MHD clamp (solver.py:956-964): rho >= rho_min, p >= p_min, E rebuilt from
// the clamped primitives; B and the velocities are kept.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void clamp_mhd(float (&u)[8], float gamma, float rho_min, float p_min) {
  const float rho = u[0];
  const float ux = u[1] / rho, uy = u[2] / rho, uz = u[3] / rho;
  const float v2 = ux * ux + uy * uy + uz * uz;
  const float b2 = u[5] * u[5] + u[6] * u[6] + u[7] * u[7];
  const float p = (gamma - 1.0f) * (u[4] - 0.5f * rho * v2 - 0.5f * b2);
  if (rho >= rho_min && p >= p_min) return;  // no floor acts: the round trip is the identity
  const float rc = fmaxf(rho, rho_min);
  const float pc = fmaxf(p, p_min);
  u[0] = rc;
  u[1] = rc * ux;
  u[2] = rc * uy;
  u[3] = rc * uz;
  u[4] = pc / (gamma - 1.0f) + 0.5f * rc * v2 + 0.5f * b2;
}

// Flux component C along DIR (0 = x, 1 = y) from q = (rho, ux, uy, uz, E,
// Bx, By, Bz) (equations.py:812-872).
template <int DIR, int C>
__device__ __forceinline__ float mhd_flux(float rho, float ux, float uy, float uz, float E, float Bx, float By,
                                          float Bz, float g1) {
  const float b2 = Bx * Bx + By * By + Bz * Bz;
  const float p = g1 * (E - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
  const float ps = p + 0.5f * b2;
  const float un = (DIR == 0) ? ux : uy;
  const float Bn = (DIR == 0) ? Bx : By;
  const float mn = rho * un;
  if constexpr (C == 0) return mn;
  if constexpr (C == 1) return mn * ux + ((DIR == 0) ? ps : 0.0f) - Bn * Bx;
  if constexpr (C == 2) return mn * uy + ((DIR == 1) ? ps : 0.0f) - Bn * By;
  if constexpr (C == 3) return mn * uz - Bn * Bz;
  if constexpr (C == 4) return (E + ps) * un - Bn * (ux * Bx + uy * By + uz * Bz);
  if constexpr (C == 5) return (DIR == 0) ? 0.0f : uy * Bx - ux * By;
  if constexpr (C == 6) return (DIR == 1) ? 0.0f : ux * By - uy * Bx;
  return un * Bz - uz * Bn;  // C == 7
}

struct MhdXArgs {
  const float* U;     // [nsolve][8][rps][N]
  float* out;         // [nsolve][16][rps][N]: D_x Fx_c (c < 8), P_x Fy_c
  long fs;            // cells of one solve
  long ssU, ssOut;
  int rows, rps;      // x-pencil rows of all solves / of one solve
  AxisOps ax;
  float gamma;
  float* speed;       // nullable: per-solve max of max(|ux|,|uy|) + sqrt(a^2 + b^2)
  const int* active;  // nullable per-solve flags
};

template <int N, int T>
struct MhdXSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, false>::BUF];
  float red[32];
};

template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_xfirst_mhd(MhdXArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<MhdXSmem<N, T>*>(smem_raw);
  const int t = threadIdx.x % A;
  const int p = threadIdx.x / A;
  const int row = blockIdx.x * T + p;
  const int sol = (row < a.rows ? row : a.rows - 1) / a.rps;
  const bool valid = row < a.rows && (a.active == nullptr || a.active[sol] != 0);
  {
    const int r0 = blockIdx.x * T, r1 = min(r0 + T, a.rows) - 1;
    bool any = a.active == nullptr;
    for (int s2 = r0 / a.rps; !any && s2 <= r1 / a.rps; ++s2) any = a.active[s2] != 0;
    if (!any) return;
  }
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  const long rloc = (long)(row % a.rps) * N + t;
  const long rbase = (long)sol * a.ssU + rloc;
  const long obase = (long)sol * a.ssOut + rloc;
  const float g1 = a.gamma - 1.0f;
  // q = (rho, ux, uy, uz, E, Bx, By, Bz) at the thread's B points
  float q[8][B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    float u[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) u[c] = valid ? a.U[c * a.fs + rbase + A * n2] : ((c == 0) ? 1.0f : 0.0f);
    const float rinv = 1.0f / u[0];
    q[0][n2] = u[0];
    q[1][n2] = u[1] * rinv;
    q[2][n2] = u[2] * rinv;
    q[3][n2] = u[3] * rinv;
#pragma unroll
    for (int c = 4; c < 8; ++c) q[c][n2] = u[c];
  }
  if (a.speed != nullptr && blockIdx.y == 0) {
    float smax = 0.0f;
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = q[0][n2], ux = q[1][n2], uy = q[2][n2], uz = q[3][n2];
        const float b2 = q[5][n2] * q[5][n2] + q[6][n2] * q[6][n2] + q[7][n2] * q[7][n2];
        const float pr = g1 * (q[4][n2] - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
        const float fast = sqrtf(fmaxf(a.gamma * pr / rho + b2 / rho, 0.0f));
        smax = fmaxf(smax, fmaxf(fabsf(ux), fabsf(uy)) + fast);
      }
    }
    const int s0 = (blockIdx.x * T) / a.rps;
    const int s1 = (min(blockIdx.x * T + T, a.rows) - 1) / a.rps;
    if (s0 == s1) {
      const float m = block_max(smax, S.red);
      if (threadIdx.x == 0) atomic_max_nonneg(a.speed + s0, m);
    } else if (valid) {
      atomic_max_nonneg(a.speed + sol, smax);
    }
  }
  __syncthreads();
  // jobs 0..3: D_x on Fx pairs (2j, 2j+1); jobs 4..7: P_x on Fy pairs.  On
  // grids with few pencil tiles the jobs are split over gridDim.y equal
  // groups of CTAs (each group rebuilds the primitives of its rows), which
  // shortens the chain of transforms each CTA runs.
  const int jpg = (8 + (int)gridDim.y - 1) / (int)gridDim.y;
  const int j_lo = jpg * (int)blockIdx.y;
  const int j_hi = min(8, j_lo + jpg);
#pragma unroll 1
  for (int j = j_lo; j < j_hi; ++j) {
    float2 v[B];
    switch (j) {
#define PS_MHD_JOB(J)                                                                                      \
  case J: {                                                                                                \
    constexpr int dir = (J) < 4 ? 0 : 1;                                                                   \
    constexpr int c = 2 * ((J) % 4);                                                                       \
    _Pragma("unroll") for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(                                  \
        mhd_flux<dir, c>(q[0][n2], q[1][n2], q[2][n2], q[3][n2], q[4][n2], q[5][n2], q[6][n2], q[7][n2], g1), \
        mhd_flux<dir, c + 1>(q[0][n2], q[1][n2], q[2][n2], q[3][n2], q[4][n2], q[5][n2], q[6][n2], q[7][n2],  \
                             g1));                                                                         \
    break;                                                                                                 \
  }
      PS_MHD_JOB(0)
      PS_MHD_JOB(1)
      PS_MHD_JOB(2)
      PS_MHD_JOB(3)
      PS_MHD_JOB(4)
      PS_MHD_JOB(5)
      PS_MHD_JOB(6)
      PS_MHD_JOB(7)
#undef PS_MHD_JOB
      default:
        break;
    }
    pf.fwd(v);
    const bool deriv = j < 4;
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = pf.kidx(r);
      if (deriv) {
        const float dd = S.ax.d[k];
        v[r] = make_float2(-v[r].y * dd, v[r].x * dd);
      } else {
        const float s = S.ax.P[k];
        v[r].x *= s;
        v[r].y *= s;
      }
    }
    pf.inv(v);
    if (valid) {
      const int f0 = deriv ? 2 * j : 8 + 2 * (j - 4);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[f0 * a.fs + obase + A * n2] = v[n2].x;
        a.out[(f0 + 1) * a.fs + obase + A * n2] = v[n2].y;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Helmholtz projection passes
// ---------------------------------------------------------------------------
struct ProjArgs {
  float* Bx;          // field planes of solve 0; solve s at + s * ss
  float* By;
  float* E;           // nullable: energy updated with the thermal pressure held fixed
  long ss;            // solve stride of Bx / By / E (elements)
  float2* H;          // half spectra [nsolve][2][ny][hx]
  int nx, ny, hx;     // hx = nx / 2 + 1
  int nsolve;
  AxisOps ax;         // x tables (x passes) or y tables (y pass)
  float kx0, ky0;     // 2 pi / Lx, 2 pi / Ly
  const int* active;
};

// rows: FFT_x of Bx and By (separately, imaginary parts zero), half spectra out
template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj_xf(ProjArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<MhdXSmem<N, T>*>(smem_raw);
  const int t = threadIdx.x % A, p = threadIdx.x / A;
  const int rows = a.ny * a.nsolve;
  const int row = blockIdx.x * T + p;
  const int sol = (row < rows ? row : rows - 1) / a.ny;
  const int j = row % a.ny;
  const bool valid = row < rows && (a.active == nullptr || a.active[sol] != 0);
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  // Bx and By: both in each CTA, or one per CTA row of a two-row grid
#pragma unroll 1
  for (int f = (int)blockIdx.y; f < 2; f += (int)gridDim.y) {
    const float* src = ((f == 0) ? a.Bx : a.By) + (long)sol * a.ss + (long)j * N;
    float2 v[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(valid ? src[t + A * n2] : 0.0f, 0.0f);
    pf.fwd(v);
    if (valid) {
      float2* dst = a.H + (((long)sol * 2 + f) * a.ny + j) * a.hx;
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const int k = pf.kidx(r);
        if (k <= N / 2) dst[k] = v[r];
      }
    }
  }
}

// columns kx of the half spectra: FFT_y, projection, inverse FFT_y
template <int N, int T>
struct ProjYSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, true>::BUF];
};

template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj_y(ProjArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<ProjYSmem<N, T>*>(smem_raw);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int kx = blockIdx.x * T + p;
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const bool valid = kx < a.hx;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  float2* hx_ = a.H + ((long)sol * 2 + 0) * a.ny * a.hx + kx;
  float2* hy_ = a.H + ((long)sol * 2 + 1) * a.ny * a.hx + kx;
  float2 X[B], Y[B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    const long o = (long)(t + A * n2) * a.hx;
    X[n2] = valid ? hx_[o] : make_float2(0.0f, 0.0f);
    Y[n2] = valid ? hy_[o] : make_float2(0.0f, 0.0f);
  }
  pf.fwd(X);
  pf.fwd(Y);
  const float kxp = a.kx0 * (float)kx;
  const float scale = 1.0f / ((float)a.nx * (float)N);
  const bool nyq_x = (kx == a.nx / 2);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const int k = pf.kidx(r);
    if (nyq_x || k == N / 2) {
      X[r] = make_float2(0.0f, 0.0f);
      Y[r] = make_float2(0.0f, 0.0f);
      continue;
    }
    const float kyp = a.ky0 * (float)((k < N / 2) ? k : k - N);
    const float k2 = kxp * kxp + kyp * kyp;
    const float inv = (k2 == 0.0f) ? 1.0f : 1.0f / k2;
    const float cr = (kxp * X[r].x + kyp * Y[r].x) * inv;
    const float ci = (kxp * X[r].y + kyp * Y[r].y) * inv;
    X[r] = make_float2((X[r].x - kxp * cr) * scale, (X[r].y - kxp * ci) * scale);
    Y[r] = make_float2((Y[r].x - kyp * cr) * scale, (Y[r].y - kyp * ci) * scale);
  }
  pf.inv(X);
  pf.inv(Y);
  if (valid) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const long o = (long)(t + A * n2) * a.hx;
      hx_[o] = X[n2];
      hy_[o] = Y[n2];
    }
  }
}

// rows: full spectra by Hermitian symmetry, Bx + i By in one inverse FFT_x,
// write B and (optionally) the energy with the thermal pressure kept
template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj_xi(ProjArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<MhdXSmem<N, T>*>(smem_raw);
  const int t = threadIdx.x % A, p = threadIdx.x / A;
  const int rows = a.ny * a.nsolve;
  const int row = blockIdx.x * T + p;
  const int sol = (row < rows ? row : rows - 1) / a.ny;
  const int j = row % a.ny;
  const bool valid = row < rows && (a.active == nullptr || a.active[sol] != 0);
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const float2* hx_ = a.H + (((long)sol * 2 + 0) * a.ny + j) * a.hx;
  const float2* hy_ = a.H + (((long)sol * 2 + 1) * a.ny + j) * a.hx;
  float2 z[B];
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const int k = pf.kidx(r);
    float2 X = make_float2(0.0f, 0.0f), Y = make_float2(0.0f, 0.0f);
    if (valid) {
      if (k <= N / 2) {
        X = hx_[k];
        Y = hy_[k];
      } else {
        const float2 xc = hx_[N - k], yc = hy_[N - k];
        X = make_float2(xc.x, -xc.y);
        Y = make_float2(yc.x, -yc.y);
      }
    }
    z[r] = make_float2(X.x - Y.y, X.y + Y.x);  // X + i Y
  }
  pf.inv(z);
  if (valid) {
    float* bx = a.Bx + (long)sol * a.ss + (long)j * N;
    float* by = a.By + (long)sol * a.ss + (long)j * N;
    float* e = (a.E != nullptr) ? a.E + (long)sol * a.ss + (long)j * N : nullptr;
    if (e != nullptr) {  // every old B and E of the row loaded before the first store
      float ox[B], oy[B], oe[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const int i = t + A * n2;
        ox[n2] = bx[i];
        oy[n2] = by[i];
        oe[n2] = e[i];
      }
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2)
        e[t + A * n2] = oe[n2] + 0.5f * ((z[n2].x * z[n2].x + z[n2].y * z[n2].y) - (ox[n2] * ox[n2] + oy[n2] * oy[n2]));
    }
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const int i = t + A * n2;
      bx[i] = z[n2].x;
      by[i] = z[n2].y;
    }
  }
}

}  // namespace ps
