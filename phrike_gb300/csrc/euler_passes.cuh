// Pencil pass kernels of the Fourier pseudo-spectral Euler right-hand side.
//
// The reference evaluates every derivative with a full N-D complex transform
// (phrike/grid.py:1226-1252, 1705-1721): d/dx_a f = Re IFFT(i k_a m s FFT f),
// with the dealias mask m and filter s separable products of one-axis tables
// (grid.py:87-141).  Because those tables are real and even in k, every factor
// maps real fields to real fields, so the N-D operator factors exactly into
// one-axis pencil operators:
//     dx1 = D_x P_y P_z,  dy1 = P_x D_y P_z,  dz1 = P_x P_y D_z,
// where P_a applies m s along axis a and D_a applies i k m s (Nyquist term
// zeroed: the reference's .real drops it).  The right-hand side
//     -(dx1 Fx + dy1 Fy + dz1 Fz)
// is then evaluated in one pencil pass per axis:
//     X pass: flux of U; G = D_x Fx, Hy = P_x Fy, Hz = P_x Fz
//     Y pass: A = P_y G + D_y Hy, B = P_y Hz              (3D only)
//     last  : rhs = -(P_z A + D_z B)  (3D)  or  -(P_y G + D_y Hy)  (2D)
// followed in the last pass by the RK4 stage update (plus the positivity clamp
// in 2D) and, after the final stage, the last axis of the end-of-step filter.
//
// Two real pencils are packed into one complex transform.  When the two
// packed signals need different operators (a with symbol P, b with symbol
// i d) and only their sum is wanted, the sum's spectrum is recovered from the
// packed spectrum Z as  C(k) = ((P+d) Z(k) + (P-d) conj Z(-k)) / 2.
#pragma once
#include "pass_common.cuh"

namespace ps {

// ---------------------------------------------------------------------------
// X pass (pencils along the contiguous axis): optional fused filter P_x of the
// incoming state, optional CFL speed, flux assembly, D_x / P_x.
// ---------------------------------------------------------------------------
struct XFirstArgs {
  const float* U;    // [NC][rows][N]
  float* Uw;         // if non-null: U after P_x is written here (fused filter)
  float* out;        // [ND*NC][rows][N]: D_x F^x (NC), P_x F^y (NC), P_x F^z (NC)
  long fs;           // elements per field
  int rows;          // rows of the x-pencils (Ny*Nz)
  AxisOps ax;
  float gamma;
  float* speed;      // if non-null: atomic max of the CFL wave speed
  const float* eref; // device scalar E_ref of the energy-perturbation form
  int shift_in;      // 1: U holds E (subtract E_ref on load); 0: U holds E'
};

template <int N, int T, int ND>
struct XFirstSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, false>::BUF];
  float tile[(ND + 2) * N * T];
  float red[32];
};

template <int N, int T, int ND>
__global__ void __launch_bounds__(Shape<N>::A * T) k_xfirst(XFirstArgs a) {
  constexpr int NC = ND + 2;
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, false>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<XFirstSmem<N, T, ND>*>(smem_raw);

  const int t = threadIdx.x % A;
  const int p = threadIdx.x / A;
  const int row = blockIdx.x * T + p;
  const bool valid = row < a.rows;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);

  // per-thread private slots of the tile: ((c*B + n2)*T + p)*A + t
  auto slot = [&](int c, int n2) -> float& { return S.tile[((c * B + n2) * T + p) * A + t]; };
  const long rbase = (long)row * N + t;
  const float er = *a.eref;
  const float eshift = a.shift_in ? er : 0.0f;
  const float pref = (a.gamma - 1.0f) * er;
  const float href = a.gamma * er;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float v = (c == 0) ? 1.0f : 0.0f;
      if (valid) v = a.U[c * a.fs + rbase + A * n2];  // may alias a.Uw: plain load
      if (c == NC - 1 && valid) v -= eshift;
      slot(c, n2) = v;
    }
  }
  __syncthreads();

  // flux component F^dir_c at this thread's points (branches outside the point loop)
  auto flux_vals = [&](int dir, int c, float (&o)[B]) {
    if (c == 0) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) o[n2] = slot(0, n2) * slot(1 + dir, n2);
    } else if (c == NC - 1) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = slot(0, n2), pr = slot(NC - 1, n2);
        float kin = 0.0f;
#pragma unroll
        for (int d = 0; d < ND; ++d) kin = fmaf(slot(1 + d, n2), slot(1 + d, n2), kin);
        const float Ep = pr / (a.gamma - 1.0f) + 0.5f * rho * kin;  // E' = E - E_ref
        o[n2] = ((Ep + pr) + href) * slot(1 + dir, n2);             // (E + p) u_dir
      }
    } else {
      const bool diag = (c - 1 == dir);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rv = slot(0, n2) * slot(1 + dir, n2) * slot(c, n2);
        o[n2] = diag ? rv + slot(NC - 1, n2) : rv;
      }
    }
  };

  // Jobs, one FFT body for all of them:
  //   [0, nfx)        complementary filter P_x of state pairs (fused end-of-step filter)
  //   then            D_x on F^x pairs, P_x on (F^y_c, F^z_c) [3D] or F^y pairs [2D]
  constexpr int nD = (NC + 1) / 2;
  constexpr int nP = (ND == 3) ? NC : NC / 2;
  const int nfx = (a.Uw != nullptr) ? (NC + 1) / 2 : 0;
  const int njobs = nfx + nD + nP;
#pragma unroll 1
  for (int j = 0; j < njobs; ++j) {
    if (j == nfx) {
      // conservative -> primitive (rho, u_1..u_ND, p') in place; CFL speed
      float smax = 0.0f;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = slot(0, n2);
        const float rinv = 1.0f / rho;
        float kin = 0.0f;
        float vel[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
          vel[d] = slot(1 + d, n2) * rinv;
          kin = fmaf(vel[d], vel[d], kin);
          slot(1 + d, n2) = vel[d];
        }
        const float pr = (a.gamma - 1.0f) * (slot(NC - 1, n2) - 0.5f * rho * kin);
        slot(NC - 1, n2) = pr;
        if (a.speed != nullptr && valid) {
          const float cs = sqrtf(a.gamma * (pr + pref) / rho);
          float um = fabsf(vel[0]);
          if (ND == 3) um = fmaxf(um, fmaxf(fabsf(vel[1]), fabsf(vel[ND - 1])));
          // 2D keeps |u_x| + a only (equations.py:137-147)
          smax = fmaxf(smax, um + cs);
        }
      }
      if (a.speed != nullptr) {
        const float m = block_max(smax, S.red);
        if (threadIdx.x == 0) atomic_max_nonneg(a.speed, m);
      }
    }
    int mode, fA, fB;  // mode 0: complementary filter, 1: D, 2: P
    float2 v[B];
    if (j < nfx) {
      const int c = 2 * j;
      mode = 0;
      fA = c;
      fB = (c + 1 < NC) ? c + 1 : -1;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(slot(fA, n2), fB >= 0 ? slot(fB, n2) : 0.0f);
    } else {
      const int jj = j - nfx;
      int dirA, cA, dirB, cB;
      if (jj < nD) {
        mode = 1;
        dirA = dirB = 0;
        cA = 2 * jj;
        cB = (cA + 1 < NC) ? cA + 1 : -1;
        fA = cA;
        fB = cB;
      } else {
        const int k = jj - nD;
        mode = 2;
        if (ND == 3) {
          dirA = 1, cA = k, dirB = 2, cB = k;
          fA = NC + k;
          fB = 2 * NC + k;
        } else {
          dirA = dirB = 1;
          cA = 2 * k;
          cB = 2 * k + 1;
          fA = NC + cA;
          fB = NC + cB;
        }
      }
      float oa[B], ob[B];
      flux_vals(dirA, cA, oa);
      if (cB >= 0) flux_vals(dirB, cB, ob);
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(oa[n2], cB >= 0 ? ob[n2] : 0.0f);
    }
    pf.fwd(v);
    if (mode == 1) {
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const float dd = S.ax.d[pf.kidx(r)];
        v[r] = make_float2(-v[r].y * dd, v[r].x * dd);
      }
    } else {
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const float P = S.ax.P[pf.kidx(r)];
        const float s = (mode == 0) ? (1.0f / N) - P : P;
        v[r].x *= s;
        v[r].y *= s;
      }
    }
    pf.inv(v);
    if (mode == 0) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float f0 = slot(fA, n2) - v[n2].x;
        slot(fA, n2) = f0;
        if (valid) a.Uw[fA * a.fs + rbase + A * n2] = f0;
        if (fB >= 0) {
          const float f1 = slot(fB, n2) - v[n2].y;
          slot(fB, n2) = f1;
          if (valid) a.Uw[fB * a.fs + rbase + A * n2] = f1;
        }
      }
    } else if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[fA * a.fs + rbase + A * n2] = v[n2].x;
        if (fB >= 0) a.out[fB * a.fs + rbase + A * n2] = v[n2].y;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Strided geometry: pencils along an axis of stride `as`, tiles of T adjacent
// x columns, `nouter` slabs of stride `os`.
// ---------------------------------------------------------------------------
struct StridedGeom {
  int ncol;   // Nx
  long as;    // axis stride (elements)
  long os;    // outer stride
  int nouter;
};

template <int N, int T, bool STRIDED = true>
struct StridedSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, STRIDED>::BUF];
};

// Load the packed pair (fa, fb) of this thread's positions into v.
template <int N>
__device__ __forceinline__ void load_pair(float2 (&v)[Shape<N>::B], const float* fa, const float* fb,
                                          long base, long step, bool valid) {
#pragma unroll
  for (int n2 = 0; n2 < Shape<N>::B; ++n2) {
    float x = 0.0f, y = 0.0f;
    if (valid) {
      x = fa[base + n2 * step];  // plain loads: in-place passes alias in and out
      if (fb) y = fb[base + n2 * step];
    }
    v[n2] = make_float2(x, y);
  }
}

// C(k) = ((P+d) Z(k) + (P-d) conj Z(-k)) / 2 : spectrum of P a + D b for z = a + i b
template <int N, int T>
__device__ __forceinline__ void combine_pd(float2 (&v)[Shape<N>::B], const Pencil<N, T, true>& pf,
                                           const AxisSmem<N>& ax, float sign) {
  constexpr int B = Shape<N>::B;
  float2 vn[B];
  pf.negk(v, vn);
#pragma unroll
  for (int r = 0; r < B; ++r) {
    const int k = pf.kidx(r);
    const float P = ax.P[k], d = ax.d[k];
    const float al = 0.5f * sign * (P + d), be = 0.5f * sign * (P - d);
    v[r] = make_float2(al * v[r].x + be * vn[r].x, al * v[r].y - be * vn[r].y);
  }
}

// ---------------------------------------------------------------------------
// 3D Y pass: A_c = P_y G_c + D_y Hy_c, B_c = P_y Hz_c.
// in: 15 fields [G(5), Hy(5), Hz(5)];  out: 10 fields [A(5), B(5)]
// ---------------------------------------------------------------------------
struct YMidArgs {
  const float* in;
  float* out;
  long fs;
  StridedGeom g;
  AxisOps ax;
};

template <int N, int T>
__global__ void __launch_bounds__(Shape<N>::A * T, (Shape<N>::A * T <= 256) ? 2 : 1) k_ymid3(YMidArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<StridedSmem<N, T>*>(smem_raw);
  const int p = threadIdx.x % T;
  const int t = threadIdx.x / T;
  const int col = blockIdx.x * T + p;
  const int outer = blockIdx.y;
  const bool valid = col < a.g.ncol;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const long base = (long)outer * a.g.os + col + (long)t * a.g.as;
  const long step = (long)A * a.g.as;

  auto store = [&](float* f, int n2, float v) {
    if (valid) f[base + n2 * step] = v;
  };
  // A outputs: pairs of combined spectra
#pragma unroll 1
  for (int c = 0; c < 5; c += 2) {
    float2 w[B];
    load_pair<N>(w, a.in + c * a.fs, a.in + (5 + c) * a.fs, base, step, valid);
    pf.fwd(w);
    combine_pd<N, T>(w, pf, S.ax, 1.0f);
    if (c + 1 < 5) {
      float2 w2[B];
      load_pair<N>(w2, a.in + (c + 1) * a.fs, a.in + (6 + c) * a.fs, base, step, valid);
      pf.fwd(w2);
      combine_pd<N, T>(w2, pf, S.ax, 1.0f);
#pragma unroll
      for (int r = 0; r < B; ++r) w[r] = make_float2(w[r].x - w2[r].y, w[r].y + w2[r].x);
    }
    pf.inv(w);
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      store(a.out + c * a.fs, n2, w[n2].x);
      if (c + 1 < 5) store(a.out + (c + 1) * a.fs, n2, w[n2].y);
    }
  }
  // B outputs: P_y on Hz pairs
#pragma unroll 1
  for (int c = 0; c < 5; c += 2) {
    float2 w[B];
    load_pair<N>(w, a.in + (10 + c) * a.fs, (c + 1 < 5) ? a.in + (11 + c) * a.fs : nullptr, base, step, valid);
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const float s = S.ax.P[pf.kidx(r)];
      w[r].x *= s;
      w[r].y *= s;
    }
    pf.inv(w);
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      store(a.out + (5 + c) * a.fs, n2, w[n2].x);
      if (c + 1 < 5) store(a.out + (6 + c) * a.fs, n2, w[n2].y);
    }
  }
}

// ---------------------------------------------------------------------------
// Last pass: rhs_c = -(P a_c + D b_c) along the pass axis, then
//   mode RHS   : write rhs
//   mode STAGE : RK4 stage update (clamp if enabled); after stage 3 the filter
//                P along this axis is applied to the new state when requested.
// ---------------------------------------------------------------------------
struct LastArgs {
  const float* a;      // a_c fields base (NC fields)
  const float* b;      // b_c fields base (NC fields)
  long fs;
  StridedGeom g;
  AxisOps ax;
  int stage;           // -1: rhs only; 0..3 RK4 stage
  const float* Un;     // state at the start of the step
  float* acc;          // RK accumulator
  float* out;          // rhs (stage -1), next stage input (0..2), new state (3)
  const double* dt_dev;
  double dt;
  float gamma;
  float rho_min, p_min;
  const float* eref;   // E_ref of the energy-perturbation form (clamp floor shift)
  int filter_last;     // stage 3: apply P along this axis to the new state
};

template <int N, int T, int ND, bool CLAMP>
__global__ void __launch_bounds__(Shape<N>::A * T, (Shape<N>::A * T <= 256) ? 2 : 1) k_last(LastArgs a) {
  constexpr int NC = ND + 2;
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<StridedSmem<N, T>*>(smem_raw);
  const int p = threadIdx.x % T;
  const int t = threadIdx.x / T;
  const int col = blockIdx.x * T + p;
  const int outer = blockIdx.y;
  const bool valid = col < a.g.ncol;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const long base = (long)outer * a.g.os + col + (long)t * a.g.as;
  const long step = (long)A * a.g.as;
  const float dt = (a.dt_dev != nullptr) ? (float)(*a.dt_dev) : (float)a.dt;
  const RKCoef rc = rk4_coef(a.stage < 0 ? 0 : a.stage, dt);

  // rhs for components (c, c+1) packed in one inverse transform
  auto rhs_pair = [&](int c, float2 (&w)[B]) {
    load_pair<N>(w, a.a + c * a.fs, a.b + c * a.fs, base, step, valid);
    pf.fwd(w);
    combine_pd<N, T>(w, pf, S.ax, -1.0f);
    if (c + 1 < NC) {
      float2 w2[B];
      load_pair<N>(w2, a.a + (c + 1) * a.fs, a.b + (c + 1) * a.fs, base, step, valid);
      pf.fwd(w2);
      combine_pd<N, T>(w2, pf, S.ax, -1.0f);
#pragma unroll
      for (int r = 0; r < B; ++r) w[r] = make_float2(w[r].x - w2[r].y, w[r].y + w2[r].x);
    }
    pf.inv(w);
  };
  auto filter_pair = [&](float2 (&w)[B]) {  // complementary form, see AxisOps
    float2 w0[B];
#pragma unroll
    for (int r = 0; r < B; ++r) w0[r] = w[r];
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const float q = (1.0f / N) - S.ax.P[pf.kidx(r)];
      w[r].x *= q;
      w[r].y *= q;
    }
    pf.inv(w);
#pragma unroll
    for (int r = 0; r < B; ++r) w[r] = make_float2(w0[r].x - w[r].x, w0[r].y - w[r].y);
  };
  auto addr = [&](int c, int n2) { return c * a.fs + base + n2 * step; };
  const float pmin_shift = a.p_min - (a.gamma - 1.0f) * (*a.eref);

  if (!CLAMP || a.stage < 0) {
    // components are independent: process pair by pair
#pragma unroll 1
    for (int c = 0; c < NC; c += 2) {
      float2 w[B];
      rhs_pair(c, w);
      const bool two = c + 1 < NC;
      if (a.stage < 0) {
        if (valid) {
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) {
            a.out[addr(c, n2)] = w[n2].x;
            if (two) a.out[addr(c + 1, n2)] = w[n2].y;
          }
        }
        continue;
      }
      // batch the epilogue loads (U^n, accumulator) before any store so the
      // DRAM latencies overlap instead of serialising behind the acc writes
      float un[2][B], ac[2][B];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          const bool live = valid && (q == 0 || two);
          un[q][n2] = (live && a.stage != 3) ? __ldg(a.Un + addr(c + q, n2)) : 0.0f;
          ac[q][n2] = (live && a.stage != 0) ? a.acc[addr(c + q, n2)] : 0.0f;
        }
      }
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float k[2] = {w[n2].x, w[n2].y};
        float res[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (a.stage == 3) {
            res[q] = fmaf(rc.wacc, k[q], ac[q][n2]);
          } else {
            const float base_acc = (a.stage == 0) ? un[q][n2] : ac[q][n2];
            ac[q][n2] = fmaf(rc.wacc, k[q], base_acc);
            res[q] = fmaf(rc.wnext, k[q], un[q][n2]);
          }
        }
        w[n2] = make_float2(res[0], res[1]);
      }
      if (valid && a.stage != 3) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (q == 1 && !two) break;
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) a.acc[addr(c + q, n2)] = ac[q][n2];
        }
      }
      if (a.stage == 3 && a.filter_last) filter_pair(w);
      if (valid) {
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          a.out[addr(c, n2)] = w[n2].x;
          if (two) a.out[addr(c + 1, n2)] = w[n2].y;
        }
      }
    }
    return;
  }

  if constexpr (CLAMP) {
  // clamped update: all components of a cell are needed together
  float2 kk[(NC + 1) / 2][B];
#pragma unroll
  for (int c = 0; c < NC; c += 2) rhs_pair(c, kk[c / 2]);
  constexpr int CH = 4;  // positions per batch of epilogue loads
#pragma unroll
  for (int n0 = 0; n0 < B; n0 += CH) {
    float un[CH][NC], ac[CH][NC];
#pragma unroll
    for (int j = 0; j < CH; ++j)
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        un[j][c] = (valid && a.stage != 3) ? __ldg(a.Un + addr(c, n0 + j)) : 0.0f;
        ac[j][c] = (valid && a.stage != 0) ? a.acc[addr(c, n0 + j)] : 0.0f;
      }
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int n2 = n0 + j;
      float u[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const float k = (c & 1) ? kk[c / 2][n2].y : kk[c / 2][n2].x;
        float res;
        if (a.stage == 3) {
          res = fmaf(rc.wacc, k, ac[j][c]);
        } else {
          const float base_acc = (a.stage == 0) ? un[j][c] : ac[j][c];
          ac[j][c] = fmaf(rc.wacc, k, base_acc);
          res = fmaf(rc.wnext, k, un[j][c]);
        }
        u[c] = valid ? res : ((c == 0) ? 1.0f : 0.0f);
      }
      clamp_state<ND>(u, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (c & 1) kk[c / 2][n2].y = u[c];
        else kk[c / 2][n2].x = u[c];
      }
    }
    if (valid && a.stage != 3) {
#pragma unroll
      for (int j = 0; j < CH; ++j)
#pragma unroll
        for (int c = 0; c < NC; ++c) a.acc[addr(c, n0 + j)] = ac[j][c];
    }
  }
#pragma unroll
  for (int c = 0; c < NC; c += 2) {
    if (a.stage == 3 && a.filter_last) filter_pair(kk[c / 2]);
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[addr(c, n2)] = kk[c / 2][n2].x;
        if (c + 1 < NC) a.out[addr(c + 1, n2)] = kk[c / 2][n2].y;
      }
    }
  }
  }
}

// ---------------------------------------------------------------------------
// Plain one-axis operator on nf fields (P or D), contiguous or strided.
// in and out may alias: each thread reads and writes only its own points.
// ---------------------------------------------------------------------------
struct OpArgs {
  const float* in;
  float* out;
  int nf;
  long fs;
  int rows;          // contiguous: number of rows
  StridedGeom g;     // strided geometry
  AxisOps ax;
  int deriv;         // 0: P, 1: D
  float scale;       // multiplies the symbol (e.g. -1 for a right-hand side)
  int complement;    // P only: out = in - IFFT((1/N - P) FFT in)  (exact, see AxisOps)
};

template <int N, int T, bool STRIDED>
__global__ void __launch_bounds__(Shape<N>::A * T) k_op(OpArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, STRIDED>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<StridedSmem<N, T, STRIDED>*>(smem_raw);
  int p, t;
  long base, step;
  bool valid;
  if constexpr (STRIDED) {
    p = threadIdx.x % T;
    t = threadIdx.x / T;
    const int col = blockIdx.x * T + p;
    valid = col < a.g.ncol;
    base = (long)blockIdx.y * a.g.os + col + (long)t * a.g.as;
    step = (long)A * a.g.as;
  } else {
    t = threadIdx.x % A;
    p = threadIdx.x / A;
    const int row = blockIdx.x * T + p;
    valid = row < a.rows;
    base = (long)row * N + t;
    step = A;
  }
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
#pragma unroll 1
  for (int c = 0; c < a.nf; c += 2) {
    const bool two = c + 1 < a.nf;
    float2 w[B], w0[B];
    load_pair<N>(w, a.in + c * a.fs, two ? a.in + (c + 1) * a.fs : nullptr, base, step, valid);
    const bool comp = a.complement && !a.deriv;
#pragma unroll
    for (int r = 0; r < B; ++r) w0[r] = w[r];
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = pf.kidx(r);
      if (a.deriv) {
        const float dd = a.scale * S.ax.d[k];
        w[r] = make_float2(-w[r].y * dd, w[r].x * dd);
      } else {
        const float s = comp ? (1.0f / N) - S.ax.P[k] : a.scale * S.ax.P[k];
        w[r].x *= s;
        w[r].y *= s;
      }
    }
    pf.inv(w);
    if (comp) {
#pragma unroll
      for (int r = 0; r < B; ++r) w[r] = make_float2(w0[r].x - w[r].x, w0[r].y - w[r].y);
    }
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[c * a.fs + base + n2 * step] = w[n2].x;
        if (two) a.out[(c + 1) * a.fs + base + n2 * step] = w[n2].y;
      }
    }
  }
}

}  // namespace ps
