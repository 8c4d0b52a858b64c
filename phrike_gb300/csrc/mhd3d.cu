// 3D MHD kernels: flux, stage update, CFL speed and the five passes of the
// Helmholtz projection (see mhd3d.cuh).
#include <cuda_runtime.h>

#include "launch.cuh"
#include "mhd3d.cuh"
#include "mhd_passes.cuh"

namespace ps {
namespace {

constexpr int EW_THREADS = 256;

inline int ew_blocks(long cells) {
  const long b = (cells + EW_THREADS - 1) / EW_THREADS;
  return (int)(b < 4096 ? b : 4096);
}

// Fx, Fy, Fz of MHDEquations3D.flux (equations.py:946-1038)
__global__ void __launch_bounds__(EW_THREADS) k_mhd3_flux(Mhd3FluxArgs a) {
  __shared__ float red[32];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const long cells = a.cells;
  const float* U = a.U + (long)sol * 8 * cells;
  const float g1 = a.gamma - 1.0f;
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i], mx = U[cells + i], my = U[2 * cells + i], mz = U[3 * cells + i];
    const float ux = mx / rho, uy = my / rho, uz = mz / rho;
    const float E = U[4 * cells + i];
    const float bx = U[5 * cells + i], by = U[6 * cells + i], bz = U[7 * cells + i];
    const float b2 = bx * bx + by * by + bz * bz;
    const float p = g1 * (E - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
    const float ps = p + 0.5f * b2;
    const float ub = ux * bx + uy * by + uz * bz;
    const float u[3] = {ux, uy, uz}, b[3] = {bx, by, bz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float* F = a.F + ((long)d * a.nsolve + sol) * 8 * cells + i;
      const float un = u[d], bn = b[d], mn = rho * un;
      F[0] = mn;
      F[cells] = mn * ux + (d == 0 ? ps : 0.0f) - bn * bx;
      F[2 * cells] = mn * uy + (d == 1 ? ps : 0.0f) - bn * by;
      F[3 * cells] = mn * uz + (d == 2 ? ps : 0.0f) - bn * bz;
      F[4 * cells] = (E + ps) * un - bn * ub;
      F[5 * cells] = (d == 0) ? 0.0f : un * bx - ux * bn;
      F[6 * cells] = (d == 1) ? 0.0f : un * by - uy * bn;
      F[7 * cells] = (d == 2) ? 0.0f : un * bz - uz * bn;
    }
    if (a.dif != nullptr) {  // (rho u, B) for the three Laplacian terms
      const float x[6] = {mx, my, mz, bx, by, bz};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float* D = a.dif + ((long)d * a.nsolve + sol) * 6 * cells + i;
#pragma unroll
        for (int c = 0; c < 6; ++c) D[c * cells] = x[c];
      }
    }
    if (a.speed != nullptr) {  // equations.py:1040-1061
      const float um = fmaxf(fmaxf(fabsf(ux), fabsf(uy)), fabsf(uz));
      m = fmaxf(m, um + sqrtf(fmaxf(a.gamma * p / rho + b2 / rho, 0.0f)));
    }
  }
  if (a.speed != nullptr) {
    m = block_max(m, red);
    if (threadIdx.x == 0) atomic_max_nonneg(a.speed + sol, m);
  }
}

// k = -(dx1 Fx + dy1 Fy + dz1 Fz) + eta lap B + nu lap(rho u) (solver.py:932-954),
// or (rhs_in) the 2D right-hand side written by the unclamped last pass, then
// the RK stage with the MHD clamp (solver.py:956-964, 988-1006)
__global__ void __launch_bounds__(EW_THREADS) k_mhd3_update(Mhd3UpdateArgs a) {
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const long cells = a.cells;
  const long so = (long)sol * 8 * cells;
  const float* F0 = a.F + so;
  const float* F1 = a.rhs_in ? F0 : a.F + (long)a.nsolve * 8 * cells + so;
  const float* F2 = a.rhs_in ? F0 : a.F + (long)2 * a.nsolve * 8 * cells + so;
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    float k[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const long o = (long)c * cells + i;
      k[c] = a.rhs_in ? F0[o] : -(F0[o] + F1[o] + F2[o]);
    }
    if (a.dif != nullptr) {
      const long ds = (long)a.nsolve * 6 * cells;
      const float* D = a.dif + (long)sol * 6 * cells + i;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const long o = (long)c * cells;
        const float lap = D[o] + D[ds + o] + D[2 * ds + o];
        if (c < 3) k[1 + c] += a.nu * lap;
        else k[2 + c] += a.eta * lap;
      }
    }
    float* out = a.out + so + i;
    if (a.stage < 0) {
#pragma unroll
      for (int c = 0; c < 8; ++c) out[(long)c * cells] = k[c];
      continue;
    }
    const float* un = a.Un + so + i;
    float* acc = a.acc + so + i;
    // the cell's loads before its stores (a store between them would make
    // each component wait for the previous one's round trip to memory)
    float vu[8], va[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const long o = (long)c * cells;
      vu[c] = (a.stage != 3) ? un[o] : 0.0f;
      va[c] = (a.stage != 0) ? acc[o] : 0.0f;
    }
    float u[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if (a.stage == 3) {
        u[c] = fmaf(rk.wacc, k[c], va[c]);
      } else {
        va[c] = fmaf(rk.wacc, k[c], (a.stage == 0) ? vu[c] : va[c]);
        u[c] = fmaf(rk.wnext, k[c], vu[c]);
      }
    }
    if (a.stage != 3) {
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[(long)c * cells] = va[c];
    }
    clamp_mhd(u, a.gamma, a.rho_min, a.p_min);
#pragma unroll
    for (int c = 0; c < 8; ++c) out[(long)c * cells] = u[c];
  }
}

// CFL speed of MHDEquations3D.max_wave_speed (equations.py:1040-1061)
__global__ void __launch_bounds__(EW_THREADS) k_speed_mhd3(const float* __restrict__ U, long cells, long ss,
                                                          float gamma, float* out) {
  __shared__ float red[32];
  U += (long)blockIdx.y * ss;
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    const float rho = U[i];
    const float ux = U[cells + i] / rho, uy = U[2 * cells + i] / rho, uz = U[3 * cells + i] / rho;
    const float bx = U[5 * cells + i], by = U[6 * cells + i], bz = U[7 * cells + i];
    const float b2 = bx * bx + by * by + bz * bz;
    const float p = (gamma - 1.0f) * (U[4 * cells + i] - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
    m = fmaxf(m, fmaxf(fmaxf(fabsf(ux), fabsf(uy)), fabsf(uz)) + sqrtf(fmaxf(gamma * p / rho + b2 / rho, 0.0f)));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(out + blockIdx.y, m);
}

// ---- projection passes

// rows (sol, z, y): FFT_x of Bx, By, Bz, half spectra out
template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj3_xf(Proj3Args a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<MhdXSmem<N, T>*>(smem_raw);
  const int t = threadIdx.x % A, p = threadIdx.x / A;
  const int rps = a.ny * a.nz;
  const int rows = rps * a.nsolve;
  const int row = blockIdx.x * T + p;
  const int sol = (row < rows ? row : rows - 1) / rps;
  const int r = row % rps;
  const bool valid = row < rows && (a.active == nullptr || a.active[sol] != 0);
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
#pragma unroll 1
  for (int f = 0; f < 3; ++f) {
    const float* src = a.B[f] + (long)sol * a.ss + (long)r * N;
    float2 v[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(valid ? src[t + A * n2] : 0.0f, 0.0f);
    pf.fwd(v);
    if (valid) {
      float2* dst = a.H + (((long)sol * 3 + f) * rps + r) * a.hx;
#pragma unroll
      for (int q = 0; q < B; ++q) {
        const int k = pf.kidx(q);
        if (k <= N / 2) dst[k] = v[q];
      }
    }
  }
}

// complex y pencils of the half spectra (column kx, plane (sol, f, z)):
// forward (store in spectral order) or inverse (load in spectral order)
template <int N, int T, bool INV>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj3_y(Proj3Args a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<ProjYSmem<N, T>*>(smem_raw);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int kx = blockIdx.x * T + p;
  const int plane = blockIdx.y;  // (sol * 3 + f) * nz + z
  const int sol = plane / (3 * a.nz);
  if (a.active != nullptr && a.active[sol] == 0) return;
  const bool valid = kx < a.hx;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  float2* col = a.H + (long)plane * N * a.hx + kx;
  float2 v[B];
  if (!INV) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = valid ? col[(long)(t + A * n2) * a.hx] : make_float2(0.0f, 0.0f);
    pf.fwd(v);
    if (valid) {
#pragma unroll
      for (int q = 0; q < B; ++q) col[(long)pf.kidx(q) * a.hx] = v[q];
    }
  } else {
#pragma unroll
    for (int q = 0; q < B; ++q) v[q] = valid ? col[(long)pf.kidx(q) * a.hx] : make_float2(0.0f, 0.0f);
    pf.inv(v);
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) col[(long)(t + A * n2) * a.hx] = v[n2];
    }
  }
}

// complex z pencils at (ky, kx): forward, Nyquist planes zeroed,
// B_hat -= k (k . B_hat)/|k|^2, 1/(nx ny nz), inverse (grid.py:1649-1684)
template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj3_z(Proj3Args a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<ProjYSmem<N, T>*>(smem_raw);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int colid = blockIdx.x * T + p;  // ky * hx + kx
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const long plane = (long)a.ny * a.hx;
  const bool valid = colid < plane;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const long fstride = (long)N * plane;
  float2* c0 = a.H + (long)sol * 3 * fstride + colid;
  float2 X[B], Y[B], Z[B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    const long o = (long)(t + A * n2) * plane;
    X[n2] = valid ? c0[o] : make_float2(0.0f, 0.0f);
    Y[n2] = valid ? c0[fstride + o] : make_float2(0.0f, 0.0f);
    Z[n2] = valid ? c0[2 * fstride + o] : make_float2(0.0f, 0.0f);
  }
  pf.fwd(X);
  pf.fwd(Y);
  pf.fwd(Z);
  const int kyi = valid ? colid / a.hx : 0, kxi = valid ? colid % a.hx : 0;
  const float kxp = a.k0x * (float)kxi;
  const float kyp = a.k0y * (float)((kyi < a.ny / 2) ? kyi : kyi - a.ny);
  const bool nyq_xy = (kxi == a.nx / 2) || (kyi == a.ny / 2);
  const float scale = 1.0f / ((float)a.nx * (float)a.ny * (float)N);
#pragma unroll
  for (int q = 0; q < B; ++q) {
    const int k = pf.kidx(q);
    if (nyq_xy || k == N / 2) {
      X[q] = make_float2(0.0f, 0.0f);
      Y[q] = make_float2(0.0f, 0.0f);
      Z[q] = make_float2(0.0f, 0.0f);
      continue;
    }
    const float kzp = a.k0z * (float)((k < N / 2) ? k : k - N);
    const float k2 = kxp * kxp + kyp * kyp + kzp * kzp;
    const float inv = (k2 == 0.0f) ? 1.0f : 1.0f / k2;
    const float cr = (kxp * X[q].x + kyp * Y[q].x + kzp * Z[q].x) * inv;
    const float ci = (kxp * X[q].y + kyp * Y[q].y + kzp * Z[q].y) * inv;
    X[q] = make_float2((X[q].x - kxp * cr) * scale, (X[q].y - kxp * ci) * scale);
    Y[q] = make_float2((Y[q].x - kyp * cr) * scale, (Y[q].y - kyp * ci) * scale);
    Z[q] = make_float2((Z[q].x - kzp * cr) * scale, (Z[q].y - kzp * ci) * scale);
  }
  pf.inv(X);
  pf.inv(Y);
  pf.inv(Z);
  if (valid) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const long o = (long)(t + A * n2) * plane;
      c0[o] = X[n2];
      c0[fstride + o] = Y[n2];
      c0[2 * fstride + o] = Z[n2];
    }
  }
}

// rows: full x spectra by Hermitian symmetry, Bx + i By in one inverse FFT and
// Bz in another; B written back and E updated at fixed thermal pressure
template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T) k_proj3_xi(Proj3Args a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<MhdXSmem<N, T>*>(smem_raw);
  const int t = threadIdx.x % A, p = threadIdx.x / A;
  const int rps = a.ny * a.nz;
  const int rows = rps * a.nsolve;
  const int row = blockIdx.x * T + p;
  const int sol = (row < rows ? row : rows - 1) / rps;
  const int r = row % rps;
  const bool valid = row < rows && (a.active == nullptr || a.active[sol] != 0);
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const float2* h0 = a.H + (((long)sol * 3 + 0) * rps + r) * a.hx;
  const float2* h1 = h0 + (long)rps * a.hx;
  const float2* h2 = h1 + (long)rps * a.hx;
  float2 z[B], w[B];
#pragma unroll
  for (int q = 0; q < B; ++q) {
    const int k = pf.kidx(q);
    float2 X = make_float2(0.0f, 0.0f), Y = X, Z = X;
    if (valid) {
      if (k <= N / 2) {
        X = h0[k];
        Y = h1[k];
        Z = h2[k];
      } else {
        const float2 xc = h0[N - k], yc = h1[N - k], zc = h2[N - k];
        X = make_float2(xc.x, -xc.y);
        Y = make_float2(yc.x, -yc.y);
        Z = make_float2(zc.x, -zc.y);
      }
    }
    z[q] = make_float2(X.x - Y.y, X.y + Y.x);  // X + i Y
    w[q] = Z;
  }
  pf.inv(z);
  pf.inv(w);
  if (valid) {
    const long base = (long)sol * a.ss + (long)r * N;
    float* bx = a.B[0] + base;
    float* by = a.B[1] + base;
    float* bz = a.B[2] + base;
    float* e = (a.E != nullptr) ? a.E + base : nullptr;
    if (e != nullptr) {  // every old B and E of the row loaded before the first store
      float ox[B], oy[B], oz[B], oe[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const int i = t + A * n2;
        ox[n2] = bx[i];
        oy[n2] = by[i];
        oz[n2] = bz[i];
        oe[n2] = e[i];
      }
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2)
        e[t + A * n2] = oe[n2] + 0.5f * ((z[n2].x * z[n2].x + z[n2].y * z[n2].y + w[n2].x * w[n2].x) -
                                         (ox[n2] * ox[n2] + oy[n2] * oy[n2] + oz[n2] * oz[n2]));
    }
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const int i = t + A * n2;
      bx[i] = z[n2].x;
      by[i] = z[n2].y;
      bz[i] = w[n2].x;
    }
  }
}

template <typename F>
cudaError_t dispatch_n3(int n, F&& f) {
  switch (n) {
    case 8: return f(std::integral_constant<int, 8>{});
    case 16: return f(std::integral_constant<int, 16>{});
    case 32: return f(std::integral_constant<int, 32>{});
    case 64: return f(std::integral_constant<int, 64>{});
    case 128: return f(std::integral_constant<int, 128>{});
    case 256: return f(std::integral_constant<int, 256>{});
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool mhd3_supported_n(int n) { return n == 8 || n == 16 || n == 32 || n == 64 || n == 128 || n == 256; }

cudaError_t launch_mhd3_flux(const Mhd3FluxArgs& a, cudaStream_t s) {
  k_mhd3_flux<<<dim3(ew_blocks(a.cells), a.nsolve), EW_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mhd3_update(const Mhd3UpdateArgs& a, cudaStream_t s) {
  k_mhd3_update<<<dim3(ew_blocks(a.cells), a.nsolve), EW_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_speed_mhd3(const float* U, long cells, long ss, int nsolve, float gamma, float* out,
                              cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(float) * nsolve, s);
  if (e != cudaSuccess) return e;
  k_speed_mhd3<<<dim3(ew_blocks(cells), nsolve), EW_THREADS, 0, s>>>(U, cells, ss, gamma, out);
  return cudaGetLastError();
}

cudaError_t launch_proj3_xf(int n, const Proj3Args& a, cudaStream_t s) {
  return dispatch_n3(n, [&](auto nc) -> cudaError_t {
    constexpr int NN = decltype(nc)::value, T = Tile<NN>::TC;
    const size_t sm = sizeof(MhdXSmem<NN, T>);
    cudaError_t e = set_smem(k_proj3_xf<NN, T>, sm);
    if (e != cudaSuccess) return e;
    const int rows = a.ny * a.nz * a.nsolve;
    k_proj3_xf<NN, T><<<(rows + T - 1) / T, Shape<NN>::A * T, sm, s>>>(a);
    return cudaGetLastError();
  });
}

cudaError_t launch_proj3_y(int n, bool inverse, const Proj3Args& a, cudaStream_t s) {
  return dispatch_n3(n, [&](auto nc) -> cudaError_t {
    constexpr int NN = decltype(nc)::value, T = 16;
    const size_t sm = sizeof(ProjYSmem<NN, T>);
    const dim3 grid((a.hx + T - 1) / T, a.nsolve * 3 * a.nz);
    cudaError_t e;
    if (inverse) {
      if ((e = set_smem(k_proj3_y<NN, T, true>, sm)) != cudaSuccess) return e;
      k_proj3_y<NN, T, true><<<grid, Shape<NN>::A * T, sm, s>>>(a);
    } else {
      if ((e = set_smem(k_proj3_y<NN, T, false>, sm)) != cudaSuccess) return e;
      k_proj3_y<NN, T, false><<<grid, Shape<NN>::A * T, sm, s>>>(a);
    }
    return cudaGetLastError();
  });
}

cudaError_t launch_proj3_z(int n, const Proj3Args& a, cudaStream_t s) {
  return dispatch_n3(n, [&](auto nc) -> cudaError_t {
    constexpr int NN = decltype(nc)::value, T = 16;
    const size_t sm = sizeof(ProjYSmem<NN, T>);
    cudaError_t e = set_smem(k_proj3_z<NN, T>, sm);
    if (e != cudaSuccess) return e;
    const dim3 grid((a.ny * a.hx + T - 1) / T, a.nsolve);
    k_proj3_z<NN, T><<<grid, Shape<NN>::A * T, sm, s>>>(a);
    return cudaGetLastError();
  });
}

cudaError_t launch_proj3_xi(int n, const Proj3Args& a, cudaStream_t s) {
  return dispatch_n3(n, [&](auto nc) -> cudaError_t {
    constexpr int NN = decltype(nc)::value, T = Tile<NN>::TC;
    const size_t sm = sizeof(MhdXSmem<NN, T>);
    cudaError_t e = set_smem(k_proj3_xi<NN, T>, sm);
    if (e != cudaSuccess) return e;
    const int rows = a.ny * a.nz * a.nsolve;
    k_proj3_xi<NN, T><<<(rows + T - 1) / T, Shape<NN>::A * T, sm, s>>>(a);
    return cudaGetLastError();
  });
}

}  // namespace ps
