// 1D Fourier Euler: whole RK4 steps in one launch, one CTA per solve.
//
// Follows SpectralSolver1D._fixed_step / _rk4_step / _compute_rhs
// (phrike/solver.py:62-132, 259-269):
//   k_i = -D_x F(U_i)               (flux equations.py:67-86, D = i k m s)
//   U_{i+1} = clamp(U + c_i dt k_i) (clamp solver.py:32-59, floors 1e-10/1e-12)
//   U_new = clamp(U + dt/6 (k1 + 2 k2 + 2 k3 + k4)), then the filter P_x is
//   applied inside the step and once more by the cadence counter.
// The three state tiles (U^n, stage input, accumulator) stay in shared
// memory for all nsteps, so a launch touches HBM only to load and store U.
// Energy is held in perturbation form E' = E - E_ref (E_ref = energy of the
// first cell at launch) and filters use the complementary form; both are
// exact rewrites that cut float32 rounding noise (see pass_common.cuh).
#pragma once
#include "adaptive.cuh"
#include "pass_common.cuh"

namespace ps {

struct Step1DArgs {
  float* U;           // [nsolve][3][N]
  long solve_stride;  // elements between solves
  AxisOps ax;
  int nsteps;
  const double* dt_dev;  // if non-null, per-solve step sizes dt_dev[solve]
  double dt;
  const int* active;     // per-solve flags (null: all active)
  float gamma;
  float rho_min, p_min;
  int filter_interval;
  int step_counter0;     // cadence counter value before the first step
  float gx;              // gravity along x (0 when disabled)
  // CFL mode (t != null): before each step dt = min(cfl dx / max(|u| + a),
  // t_end - t) per solve; a solve stops once t >= t_end - 1e-12 (solver.py:384-417)
  double* t;             // per-solve simulation time, advanced in place
  const double* tend;    // per-solve end time
  float cfl, dx;
  int* steps_done;       // per-solve count of steps taken (CFL mode; may be null)
  AVParams av;           // artificial viscosity (mode 0: off)
  float* scratch;        // N >= 4096: U^n and accumulator, [nsolve][6][N]
  int rk2;               // midpoint RK2: stages 0 and 3 with rk_coef
};

// N = 4096 keeps U^n and the accumulator in global scratch (6 fields per
// solve, L2-resident) so that the rest fits in one CTA's shared memory.
template <int N>
struct Step1DGlobal {
  static constexpr bool value = N >= 4096;
};

template <int N>
struct Step1DSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, 1, false>::BUF];
  float un[Step1DGlobal<N>::value ? 1 : 3 * N];
  float us[3 * N];
  float acc[Step1DGlobal<N>::value ? 1 : 3 * N];
  float red[32];
};

// w <- D w for a packed pair of real pencils (D = i k m s)
template <int N, typename PF>
__device__ __forceinline__ void deriv_pair(const PF& pf, const AxisSmem<N>& ax, float2 (&w)[Shape<N>::B]) {
  pf.fwd(w);
#pragma unroll
  for (int r = 0; r < Shape<N>::B; ++r) {
    const float dd = ax.d[pf.kidx(r)];
    w[r] = make_float2(-w[r].y * dd, w[r].x * dd);
  }
  pf.inv(w);
}

// w <- P w for a packed pair of real pencils, in the complementary form
// P w = w - IFFT((1/N - P) FFT w) that keeps the retained band exact
template <int N, typename PF>
__device__ __forceinline__ void filter_pair1d(const PF& pf, const AxisSmem<N>& ax, float2 (&w)[Shape<N>::B]) {
  constexpr int B = Shape<N>::B;
  float2 w0[B];
#pragma unroll
  for (int r = 0; r < B; ++r) w0[r] = w[r];
  pf.fwd(w);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const float q = (1.0f / N) - ax.P[pf.kidx(r)];
    w[r].x *= q;
    w[r].y *= q;
  }
  pf.inv(w);
#pragma unroll
  for (int r = 0; r < B; ++r) w[r] = make_float2(w0[r].x - w[r].x, w0[r].y - w[r].y);
}

// k = rhs(us) at this thread's points (private slots (c*B + n2)*A + t):
// -D_x F(us) (equations.py:67-86), plus the artificial-viscosity terms
// (artificial_viscosity.py:270-403) and the gravity source (solver.py:82-91).
// Returns (k0, k1) in w01 and k2 in w2.x; us holds E' = E - er.
template <int N, typename PF>
__device__ __forceinline__ void rhs1d(const PF& pf, const AxisSmem<N>& ax, const float* us, int t, float gamma,
                                      float er, const AVParams& av, float gx, float2 (&w01)[Shape<N>::B],
                                      float2 (&w2)[Shape<N>::B]) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  auto sl = [&](int c, int n2) { return (c * B + n2) * A + t; };
  const float g1 = gamma - 1.0f;
  const float href = gamma * er;
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    const float rho = us[sl(0, n2)], m = us[sl(1, n2)], E = us[sl(2, n2)];
    const float u = m / rho;
    const float p = g1 * (E - 0.5f * rho * u * u);  // p' (E holds E')
    const float mom = rho * u;
    w01[n2] = make_float2(mom, mom * u + p);
    w2[n2] = make_float2(((E + p) + href) * u, 0.0f);
  }
  // k = -i d FFT(F): multiply by -i d
  pf.fwd(w01);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const float dd = ax.d[pf.kidx(r)];
    w01[r] = make_float2(w01[r].y * dd, -w01[r].x * dd);
  }
  pf.inv(w01);
  pf.fwd(w2);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const float dd = ax.d[pf.kidx(r)];
    w2[r] = make_float2(w2[r].y * dd, -w2[r].x * dd);
  }
  pf.inv(w2);
  if (av.mode != 0) {
    // gradients of (q, U_0) and (U_1, U_2) packed in two transforms, nu per
    // point, then the divergence of the viscous fluxes w_c nu dU_c/dx
    float2 g0[B], g1v[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float rho = us[sl(0, n2)], m = us[sl(1, n2)], E = us[sl(2, n2)];
      const float u = m / rho;
      float q = rho;
      if (av.sensor == 1) q = g1 * (E - 0.5f * rho * u * u) + g1 * er;  // true pressure
      else if (av.sensor == 2) q = fabsf(u);
      g0[n2] = make_float2(q, rho);
      g1v[n2] = make_float2(m, E);
    }
    float qv[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) qv[n2] = g0[n2].x;
    deriv_pair<N>(pf, ax, g0);
    deriv_pair<N>(pf, ax, g1v);
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float nu = av_nu(av, fabsf(g0[n2].x), qv[n2]);
      g0[n2] = make_float2(av.w[0] * nu * g0[n2].y, av.w[1] * nu * g1v[n2].x);
      g1v[n2] = make_float2(av.w[2] * nu * g1v[n2].y, 0.0f);
    }
    deriv_pair<N>(pf, ax, g0);
    deriv_pair<N>(pf, ax, g1v);
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      w01[n2].x += g0[n2].x;
      w01[n2].y += g0[n2].y;
      w2[n2].x += g1v[n2].x;
    }
  }
  if (gx != 0.0f) {  // gravity source (solver.py:82-91)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float rho = us[sl(0, n2)];
      const float u = us[sl(1, n2)] / rho;
      w01[n2].y += rho * gx;
      w2[n2].x += rho * gx * u;
    }
  }
}

template <int N>
__global__ void __launch_bounds__(Shape<N>::A) k_step1d(Step1DArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, 1, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<Step1DSmem<N>*>(smem_raw);
  const int t = threadIdx.x;
  if (a.active != nullptr && a.active[blockIdx.x] == 0) return;
  PF pf{0, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  float* U = a.U + (long)blockIdx.x * a.solve_stride;
  float* const s_un = Step1DGlobal<N>::value ? a.scratch + (long)blockIdx.x * 6 * N : S.un;
  float* const s_acc = Step1DGlobal<N>::value ? s_un + 3 * N : S.acc;
  // private slots: (c*B + n2)*A + t  <-> position t + A*n2
  auto sl = [&](int c, int n2) { return (c * B + n2) * A + t; };
  const float er = U[2 * N];  // E_ref; U is written only after the last step
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float v = U[c * N + t + A * n2];
      if (c == 2) v -= er;
      s_un[sl(c, n2)] = v;
      S.us[sl(c, n2)] = v;
    }
  __syncthreads();
  float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[blockIdx.x] : (float)a.dt;
  const float g1 = a.gamma - 1.0f;
  double tl = (a.t != nullptr) ? a.t[blockIdx.x] : 0.0;
  const double te = (a.tend != nullptr) ? a.tend[blockIdx.x] : 0.0;
  int taken = 0;
  const int cad0 = (a.steps_done != nullptr) ? a.steps_done[blockIdx.x] : a.step_counter0;
  const float pmin_shift = a.p_min - g1 * er;
  auto filter_pair = [&](float2 (&w)[B]) { filter_pair1d<N>(pf, S.ax, w); };

#pragma unroll 1
  for (int step = 0; step < a.nsteps; ++step) {
    double dtd = dt;
    if (a.t != nullptr) {  // CFL step size from the current state (uniform across the CTA)
      if (tl >= te - 1e-12) break;
      float sm = 0.0f;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = s_un[sl(0, n2)];
        const float u = s_un[sl(1, n2)] / rho;
        const float pp = g1 * (s_un[sl(2, n2)] - 0.5f * rho * u * u) + g1 * er;  // true pressure
        sm = fmaxf(sm, fabsf(u) + sqrtf(a.gamma * pp / rho));
      }
      sm = block_max(sm, S.red);
      if (threadIdx.x == 0) S.red[0] = sm;
      __syncthreads();
      const double spd = (double)S.red[0];
      __syncthreads();
      dtd = (spd <= 0.0) ? 1e-6 : (double)a.cfl * (double)a.dx / spd;
      dtd = fmin(dtd, te - tl);
      dt = (float)dtd;
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      if (a.rk2 && (stage == 1 || stage == 2)) continue;
      const RKCoef rc = rk_coef(stage, dt, a.rk2);
      float2 w01[B], w2[B];
      rhs1d<N>(pf, S.ax, S.us, t, a.gamma, er, a.av, a.gx, w01, w2);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float k[3] = {w01[n2].x, w01[n2].y, w2[n2].x};
        float u3[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int s = sl(c, n2);
          u3[c] = rk_update_incr(stage, rc, k[c], s_un[s], s_acc[s]);
        }
        clamp_state<1>(u3, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
        for (int c = 0; c < 3; ++c) S.us[sl(c, n2)] = u3[c];
      }
    }
    // end of step: filter inside the RK step, then again by cadence
    const bool second = ((cad0 + step) % a.filter_interval) == 0;
    float2 w01[B], w2[B];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      w01[n2] = make_float2(S.us[sl(0, n2)], S.us[sl(1, n2)]);
      w2[n2] = make_float2(S.us[sl(2, n2)], 0.0f);
    }
    filter_pair(w01);
    filter_pair(w2);
    if (second) {
      filter_pair(w01);
      filter_pair(w2);
    }
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      const float v[3] = {w01[n2].x, w01[n2].y, w2[n2].x};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        s_un[sl(c, n2)] = v[c];
        S.us[sl(c, n2)] = v[c];
      }
    }
    tl += dtd;
    ++taken;
  }
  if (threadIdx.x == 0) {
    if (a.t != nullptr) a.t[blockIdx.x] = tl;
    if (a.steps_done != nullptr) a.steps_done[blockIdx.x] += taken;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) U[c * N + t + A * n2] = s_un[sl(c, n2)] + (c == 2 ? er : 0.0f);
}

// ---------------------------------------------------------------------------
// Adaptive embedded RK, whole attempt loops in one launch, one CTA per solve
// (the 1D adaptive run loop: solver.py:295-323, 338-422 with the stepper of
// adaptive.py:23-419).  The stage right-hand sides include artificial
// viscosity and gravity, as the 1D solver passes both; no clamp in the
// stages; an accepted attempt is filtered once (_apply_physical_filters).
// The stage slopes K_i live in a per-solve global scratch that stays in L2.
// ---------------------------------------------------------------------------
struct Ark1DArgs {
  float* U;            // [nsolve][3][N], updated in place
  long solve_stride;
  AxisOps ax;
  float gamma;
  AVParams av;
  float gx;
  int nattempts;
  ArkTableau tab;
  ArkCtrl ctrl;
  double* t;           // per solve: time, end time, proposed dt (in/out)
  const double* tend;
  double* dtp;
  const double* tout;  // nullable: pause once t + 1e-12 >= tout
  int* rej;            // consecutive rejections (in/out)
  int* counts;         // nullable [nsolve][2]: accepted, rejected attempts
  float* scratch;      // per solve: [U^n 3N when N >= 4096][stages][3N]
  long scratch_stride;
};

template <int N>
__global__ void __launch_bounds__(Shape<N>::A) k_ark1d(Ark1DArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, 1, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<Step1DSmem<N>*>(smem_raw);
  const int t = threadIdx.x;
  const int sol = blockIdx.x;
  PF pf{0, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  float* U = a.U + (long)sol * a.solve_stride;
  float* scr = a.scratch + (long)sol * a.scratch_stride;
  float* const s_un = Step1DGlobal<N>::value ? scr : S.un;
  float* const K = scr + (Step1DGlobal<N>::value ? 3 * N : 0);
  auto sl = [&](int c, int n2) { return (c * B + n2) * A + t; };
  const float er = U[2 * N];  // E_ref; U is written only at the end
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float v = U[c * N + t + A * n2];
      if (c == 2) v -= er;
      s_un[sl(c, n2)] = v;
    }
  __syncthreads();
  double tl = a.t[sol];
  const double te = a.tend[sol];
  const double to = (a.tout != nullptr) ? a.tout[sol] : 0.0;
  double dtp = a.dtp[sol];
  int rej = a.rej[sol];
  int nacc = 0, nrej = 0;
  const int ns = a.tab.stages;
  // uniform block-wide max: every thread gets the same value
  auto bmax = [&](float v) {
    v = block_max(v, S.red);
    if (threadIdx.x == 0) S.red[0] = v;
    __syncthreads();
    const float r = S.red[0];
    __syncthreads();
    return r;
  };

#pragma unroll 1
  for (int att = 0; att < a.nattempts; ++att) {
    if (!(tl < te - 1e-12) || (a.tout != nullptr && !(tl + 1e-12 < to))) break;
    const double dtd = fmin(dtp, te - tl);
    // solution scale max |U| with the true energy
    float sc = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) sc = fmaxf(sc, fabsf(s_un[sl(c, n2)] + (c == 2 ? er : 0.0f)));
    sc = bmax(sc);
#pragma unroll 1
    for (int i = 0; i < ns; ++i) {
      float cf[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) cf[j] = (j < i) ? (float)(dtd * a.tab.a[i][j]) : 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          const int s = sl(c, n2);
          float v = s_un[s];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (j < i && cf[j] != 0.0f) v = fmaf(cf[j], K[j * 3 * N + s], v);
          S.us[s] = v;
        }
      float2 w01[B], w2[B];
      rhs1d<N>(pf, S.ax, S.us, t, a.gamma, er, a.av, a.gx, w01, w2);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        K[i * 3 * N + sl(0, n2)] = w01[n2].x;
        K[i * 3 * N + sl(1, n2)] = w01[n2].y;
        K[i * 3 * N + sl(2, n2)] = w2[n2].x;
      }
    }
    // U_high and the error estimate |U_high - U_low| = dt |sum (bh - bl) K|
    float ch[8], ce[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      ch[j] = (j < ns) ? (float)(dtd * a.tab.bh[j]) : 0.0f;
      ce[j] = (j < ns) ? (float)(dtd * (a.tab.bh[j] - a.tab.bl[j])) : 0.0f;
    }
    float em = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const int s = sl(c, n2);
        float vh = s_un[s], ve = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j < ns && (ch[j] != 0.0f || ce[j] != 0.0f)) {
            const float k = K[j * 3 * N + s];
            vh = fmaf(ch[j], k, vh);
            ve = fmaf(ce[j], k, ve);
          }
        S.us[s] = vh;
        em = fmaxf(em, fabsf(ve));
      }
    em = bmax(em);
    // controller (adaptive.py:45-81) and the rejection counter (359-419)
    const double err = (double)em;
    const double tol = a.ctrl.atol + a.ctrl.rtol * (double)sc;
    bool accept = err <= tol;
    double dt_new;
    if (err > 0.0) {
      const double dt_opt = dtd * pow(tol / err, 1.0 / (double)a.tab.order) * a.ctrl.safety;
      dt_new = dtd * fmin(fmax(dt_opt / dtd, a.ctrl.minf), a.ctrl.maxf);
    } else {
      dt_new = dtd * a.ctrl.maxf;
    }
    if (!accept) {
      if (++rej >= a.ctrl.max_rej) {
        rej = 0;
        accept = true;
      }
    } else {
      rej = 0;
    }
    if (accept) {  // U <- filter(U_high)
      float2 w01[B], w2[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        w01[n2] = make_float2(S.us[sl(0, n2)], S.us[sl(1, n2)]);
        w2[n2] = make_float2(S.us[sl(2, n2)], 0.0f);
      }
      filter_pair1d<N>(pf, S.ax, w01);
      filter_pair1d<N>(pf, S.ax, w2);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        s_un[sl(0, n2)] = w01[n2].x;
        s_un[sl(1, n2)] = w01[n2].y;
        s_un[sl(2, n2)] = w2[n2].x;
      }
      tl += dtd;
      ++nacc;
    } else {
      ++nrej;
    }
    dtp = dt_new;
  }
  if (threadIdx.x == 0) {
    a.t[sol] = tl;
    a.dtp[sol] = dtp;
    a.rej[sol] = rej;
    if (a.counts != nullptr) {
      a.counts[2 * sol] += nacc;
      a.counts[2 * sol + 1] += nrej;
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) U[c * N + t + A * n2] = s_un[sl(c, n2)] + (c == 2 ? er : 0.0f);
}

}  // namespace ps
