// 1D ideal / resistive MHD: whole RK steps in one launch, one CTA per solve.
//
// Follows MHDEquations1D (equations.py:659-767) and SpectralSolverMHD with
// dim 1 (solver.py:840-1049, 1165-1166):
//   k = -D_x F(U) + eta lap(B) + nu lap(rho u)   (F: the x flux, F_Bx = 0)
//   every stage: clamp (rho >= rho_min, p >= p_min, E rebuilt) and, with
//   project_each_substage, the 1D projection Bx <- mean(Bx) with the thermal
//   pressure held fixed (grid.py:554-567, solver.py:966-986);
//   after the step, at the filter cadence: the spectral filter, then the
//   projection.
// CFL: |u_x| + c_f with the exact fast magnetosonic speed along x
// (equations.py:735-750), capped by the parabolic limit of the diffusion.
// The states U^n, stage input, accumulator and slopes live in shared memory
// (U^n and the accumulator in a per-solve global scratch from 2048 points).
#pragma once
#include "mhd_passes.cuh"
#include "pass_common.cuh"

namespace ps {

struct Mhd1DArgs {
  float* U;              // [nsolve][8][N]
  long solve_stride;
  AxisOps ax;
  int nsteps;
  const double* dt_dev;  // per-solve step sizes (null: dt)
  double dt;
  const int* active;
  float gamma, rho_min, p_min;
  int filter_interval;
  int step_counter0;
  int project_stages;    // project B after every stage
  int clean;             // divergence cleaning on (else no projection at all)
  float eta, nu;         // resistivity, viscosity
  float kunit;           // 2 pi / Lx
  double* t;             // CFL mode: per-solve time (advanced), end time
  const double* tend;
  float cfl, dx;
  double dt_cap;         // parabolic limit of the diffusion (0: none)
  int* steps_done;
  float* scratch;        // N >= 2048: U^n and accumulator, [nsolve][16][N]
  float* rhs_out;        // non-null: write rhs(U) and return (ps_rhs)
  int rk2;
};

template <int N>
struct Mhd1DGlobal {
  static constexpr bool value = N >= 2048;
};

template <int N>
struct Mhd1DSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, 1, false>::BUF];
  float un[Mhd1DGlobal<N>::value ? 1 : 8 * N];
  float us[8 * N];
  float acc[Mhd1DGlobal<N>::value ? 1 : 8 * N];
  float kb[8 * N];
  float red[32];
};

// sum over the block, returned to every thread
__device__ __forceinline__ float block_sum(float v, float* red) {
  const int ww = warp_width();
  const unsigned mask = warp_mask();
  for (int o = 16; o > 0; o >>= 1)
    if (o < ww) v += __shfl_xor_sync(mask, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.0f;
  for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

template <int N>
__global__ void __launch_bounds__(Shape<N>::A) k_mhd1d(Mhd1DArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, 1, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<Mhd1DSmem<N>*>(smem_raw);
  const int t = threadIdx.x;
  const int sol = blockIdx.x;
  if (a.active != nullptr && a.active[sol] == 0) return;
  PF pf{0, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  float* U = a.U + (long)sol * a.solve_stride;
  float* const s_un = Mhd1DGlobal<N>::value ? a.scratch + (long)sol * 16 * N : S.un;
  float* const s_acc = Mhd1DGlobal<N>::value ? s_un + 8 * N : S.acc;
  auto sl = [&](int c, int n2) { return (c * B + n2) * A + t; };
  const float g1 = a.gamma - 1.0f;
#pragma unroll
  for (int c = 0; c < 8; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float v = U[c * N + t + A * n2];
      s_un[sl(c, n2)] = v;
      S.us[sl(c, n2)] = v;
    }
  __syncthreads();

  // Bx <- mean(Bx), E += (Bx_new^2 - Bx_old^2) / 2 on array q (1D projection)
  auto project = [&](float* q) {
    float sbx = 0.0f;
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) sbx += q[sl(5, n2)];
    const float mean = block_sum(sbx, S.red) * (1.0f / N);
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float bo = q[sl(5, n2)];
      q[sl(4, n2)] += 0.5f * (mean * mean - bo * bo);
      q[sl(5, n2)] = mean;
    }
  };
  // spectral filter (complementary form) of all 8 components of q, in place
  auto filter_all = [&](float* q) {
#pragma unroll 1
    for (int c = 0; c < 8; c += 2) {
      float2 w[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) w[n2] = make_float2(q[sl(c, n2)], q[sl(c + 1, n2)]);
      filter_pair1d<N>(pf, S.ax, w);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        q[sl(c, n2)] = w[n2].x;
        q[sl(c + 1, n2)] = w[n2].y;
      }
    }
  };
  // kb <- rhs(us): -D_x F for the flux pairs (0,1) (2,3) (4,6) (7,-), F_5 = 0,
  // then the diffusion terms on (1,2) (3,-) [nu] and (5,6) (7,-) [eta]
  auto rhs = [&]() {
#pragma unroll 1
    for (int j = 0; j < 4; ++j) {
      const int ca = (j == 2) ? 4 : (j == 3) ? 7 : 2 * j;
      const int cb = (j == 2) ? 6 : (j == 3) ? -1 : 2 * j + 1;
      float2 w[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = S.us[sl(0, n2)];
        const float ux = S.us[sl(1, n2)] / rho, uy = S.us[sl(2, n2)] / rho, uz = S.us[sl(3, n2)] / rho;
        const float E = S.us[sl(4, n2)], Bx = S.us[sl(5, n2)], By = S.us[sl(6, n2)], Bz = S.us[sl(7, n2)];
        float fa, fb = 0.0f;
        switch (j) {
          case 0:
            fa = mhd_flux<0, 0>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            fb = mhd_flux<0, 1>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            break;
          case 1:
            fa = mhd_flux<0, 2>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            fb = mhd_flux<0, 3>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            break;
          case 2:
            fa = mhd_flux<0, 4>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            fb = mhd_flux<0, 6>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            break;
          default:
            fa = mhd_flux<0, 7>(rho, ux, uy, uz, E, Bx, By, Bz, g1);
            break;
        }
        w[n2] = make_float2(fa, fb);
      }
      pf.fwd(w);
#pragma unroll
      for (int r = 0; r < B; ++r) w[r] = op_symbol<N>(w[r], pf.kidx(r), 1, -1.0f, a.kunit, S.ax.P, S.ax.d);
      pf.inv(w);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        S.kb[sl(ca, n2)] = w[n2].x;
        if (cb >= 0) S.kb[sl(cb, n2)] = w[n2].y;
      }
    }
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) S.kb[sl(5, n2)] = 0.0f;
    if (a.nu != 0.0f || a.eta != 0.0f) {
#pragma unroll 1
      for (int j = 0; j < 4; ++j) {
        const float coef = (j < 2) ? a.nu : a.eta;
        if (coef == 0.0f) continue;
        const int ca = (j == 0) ? 1 : (j == 1) ? 3 : (j == 2) ? 5 : 7;
        const int cb = (j == 0) ? 2 : (j == 2) ? 6 : -1;
        float2 w[B];
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) w[n2] = make_float2(S.us[sl(ca, n2)], cb >= 0 ? S.us[sl(cb, n2)] : 0.0f);
        pf.fwd(w);
#pragma unroll
        for (int r = 0; r < B; ++r) w[r] = op_symbol<N>(w[r], pf.kidx(r), 2, coef, a.kunit, S.ax.P, S.ax.d);
        pf.inv(w);
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          S.kb[sl(ca, n2)] += w[n2].x;
          if (cb >= 0) S.kb[sl(cb, n2)] += w[n2].y;
        }
      }
    }
  };

  if (a.rhs_out != nullptr) {  // rhs(U) only
    rhs();
    float* R = a.rhs_out + (long)sol * a.solve_stride;
#pragma unroll
    for (int c = 0; c < 8; ++c)
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) R[c * N + t + A * n2] = S.kb[sl(c, n2)];
    return;
  }

  float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  double tl = (a.t != nullptr) ? a.t[sol] : 0.0;
  const double te = (a.tend != nullptr) ? a.tend[sol] : 0.0;
  int taken = 0;
  const int cad0 = (a.steps_done != nullptr) ? a.steps_done[sol] : a.step_counter0;
#pragma unroll 1
  for (int step = 0; step < a.nsteps; ++step) {
    double dtd = dt;
    if (a.t != nullptr) {  // CFL step size from the current state (uniform across the CTA)
      if (tl >= te - 1e-12) break;
      float sm = 0.0f;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = s_un[sl(0, n2)];
        const float ux = s_un[sl(1, n2)] / rho, uy = s_un[sl(2, n2)] / rho, uz = s_un[sl(3, n2)] / rho;
        const float Bx = s_un[sl(5, n2)], By = s_un[sl(6, n2)], Bz = s_un[sl(7, n2)];
        const float b2 = Bx * Bx + By * By + Bz * Bz;
        const float p = g1 * (s_un[sl(4, n2)] - 0.5f * rho * (ux * ux + uy * uy + uz * uz) - 0.5f * b2);
        const float a2 = a.gamma * p / rho, bb = b2 / rho, cax2 = Bx * Bx / rho;
        const float disc = fmaxf((a2 + bb) * (a2 + bb) - 4.0f * a2 * cax2, 0.0f);
        sm = fmaxf(sm, fabsf(ux) + sqrtf(0.5f * (a2 + bb + sqrtf(disc))));
      }
      sm = block_max(sm, S.red);
      if (threadIdx.x == 0) S.red[0] = sm;
      __syncthreads();
      const double spd = (double)S.red[0];
      __syncthreads();
      dtd = (spd <= 0.0) ? 1e-6 : (double)a.cfl * (double)a.dx / spd;
      if (spd > 0.0 && a.dt_cap > 0.0) dtd = fmin(dtd, a.dt_cap);
      dtd = fmin(dtd, te - tl);
      dt = (float)dtd;
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      if (a.rk2 && (stage == 1 || stage == 2)) continue;
      const RKCoef rc = rk_coef(stage, dt, a.rk2);
      rhs();
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        float u[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const int s = sl(c, n2);
          u[c] = rk_update_incr(stage, rc, S.kb[s], s_un[s], s_acc[s]);
        }
        clamp_mhd(u, a.gamma, a.rho_min, a.p_min);
#pragma unroll
        for (int c = 0; c < 8; ++c) S.us[sl(c, n2)] = u[c];
      }
      if (a.clean && a.project_stages) project(S.us);
    }
    // end of step: at the cadence the filter, then the projection
    if (((cad0 + step) % a.filter_interval) == 0) {
      filter_all(S.us);
      if (a.clean) project(S.us);
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) s_un[sl(c, n2)] = S.us[sl(c, n2)];
    tl += dtd;
    ++taken;
  }
  if (threadIdx.x == 0) {
    if (a.t != nullptr) a.t[sol] = tl;
    if (a.steps_done != nullptr) a.steps_done[sol] += taken;
  }
#pragma unroll
  for (int c = 0; c < 8; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) U[c * N + t + A * n2] = s_un[sl(c, n2)];
}

}  // namespace ps
