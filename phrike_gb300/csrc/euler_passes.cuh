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
// Two real pencils are packed into one complex transform: P and i d are
// real-to-real operators, so they act on the real and imaginary halves of a
// packed pencil independently.  The strided passes (passes_tma.cuh) evaluate
// P a_c + D b_c for two components at once as
// IFFT(P FFT(a_c + i a_c') + i d FFT(b_c + i b_c')).
#pragma once
#include "pass_common.cuh"

namespace ps {

// ---------------------------------------------------------------------------
// X pass (pencils along the contiguous axis): optional fused filter P_x of the
// incoming state, optional CFL speed, flux assembly, D_x / P_x.
// ---------------------------------------------------------------------------
// Batches: every buffer is [nsolve][nfields][cells]; a solve's fields are
// contiguous and solves follow each other at the buffer's solve stride.
struct XFirstArgs {
  const float* U;    // [nsolve][NC][rows_per_solve][N]
  float* Uw;         // if non-null: U after P_x is written here (fused filter), same layout as U
  float* out;        // [nsolve][ND*NC][..]: D_x F^x (NC), P_x F^y (NC), P_x F^z (NC)
  long fs;           // elements per field (cells of one solve)
  long ssU, ssOut;   // solve strides of U / Uw and of out
  int rows;          // x-pencil rows of all solves
  int rps;           // rows per solve (Ny*Nz)
  AxisOps ax;
  float gamma;
  float* speed;      // if non-null: per-solve atomic max of the CFL wave speed
  const float* eref; // per-solve E_ref of the energy-perturbation form
  const int* active; // per-solve flags (null: all active); inactive solves are not written
  int shift_in;      // 1: U holds E (subtract E_ref on load); 0: U holds E'
};

template <int N, int T, int ND>
struct XFirstSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, false>::BUF];
  float red[32];
};

// The thread's B points of all NC components stay in registers (q[c][n2]);
// a switch over the job index gives every job compile-time register indices
// while a single FFT body serves all jobs (keeps the kernel's code small).
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
  const int sol = (row < a.rows ? row : a.rows - 1) / a.rps;
  const bool live = a.active == nullptr || a.active[sol] != 0;
  const bool valid = row < a.rows && live;
  {  // a CTA whose rows all belong to inactive solves has nothing to do
    const int r0 = blockIdx.x * T, r1 = min(r0 + T, a.rows) - 1;
    bool any = a.active == nullptr;
    for (int s2 = r0 / a.rps; !any && s2 <= r1 / a.rps; ++s2) any = a.active[s2] != 0;
    if (!any) return;
  }
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);

  const long rloc = (long)(row % a.rps) * N + t;
  const long rbase = (long)sol * a.ssU + rloc;    // U / Uw
  const long obase = (long)sol * a.ssOut + rloc;  // out
  const float er = a.eref[sol];
  const float eshift = a.shift_in ? er : 0.0f;
  const float pref = (a.gamma - 1.0f) * er;
  const float href = a.gamma * er;
  const float g1 = a.gamma - 1.0f;
  const float ig1 = 1.0f / g1;  // one division per thread instead of one per energy flux
  float q[NC][B];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float v = (c == 0) ? 1.0f : 0.0f;
      if (valid) v = a.U[c * a.fs + rbase + A * n2];  // may alias a.Uw: plain load
      if (c == NC - 1 && valid) v -= eshift;
      q[c][n2] = v;
    }
  }
  __syncthreads();

  // F^dir_c at point n2 from primitives q = (rho, u_1..u_ND, p')
  auto fx = [&](int dir, int c, int n2) -> float {
    const float rho = q[0][n2], ua = q[1 + dir][n2], pr = q[NC - 1][n2];
    if (c == 0) return rho * ua;
    if (c == NC - 1) {
      float kin = 0.0f;
#pragma unroll
      for (int d = 0; d < ND; ++d) kin = fmaf(q[1 + d][n2], q[1 + d][n2], kin);
      const float Ep = fmaf(pr, ig1, 0.5f * rho * kin);  // E' = E - E_ref
      return ((Ep + pr) + href) * ua;              // (E + p) u_dir
    }
    const float rv = rho * ua * q[c][n2];
    return (c - 1 == dir) ? rv + pr : rv;
  };
  auto fill = [&](float2 (&v)[B], int dA, int cA, int dB, int cB) {
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(fx(dA, cA, n2), cB >= 0 ? fx(dB, cB, n2) : 0.0f);
  };

  // jobs: [0, nfx) complementary filter P_x of state pairs (fused end-of-step
  // filter), then D_x on F^x pairs, then P_x on (F^y_c, F^z_c) [3D] or F^y pairs [2D]
  constexpr int nFX = (NC + 1) / 2;
  constexpr int nD = (NC + 1) / 2;
  constexpr int nP = (ND == 3) ? NC : NC / 2;
  const int nfx = (a.Uw != nullptr) ? nFX : 0;
  const int njobs = nfx + nD + nP;
#pragma unroll 1
  for (int j = 0; j < njobs; ++j) {
    if (j == nfx) {
      // conservative -> primitive (rho, u_1..u_ND, p') in registers; CFL speed
      float smax = 0.0f;
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const float rho = q[0][n2];
        const float rinv = 1.0f / rho;
        float kin = 0.0f;
        float vel[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
          vel[d] = q[1 + d][n2] * rinv;
          kin = fmaf(vel[d], vel[d], kin);
          q[1 + d][n2] = vel[d];
        }
        const float pr = g1 * (q[NC - 1][n2] - 0.5f * rho * kin);
        q[NC - 1][n2] = pr;
        if (a.speed != nullptr && valid) {
          const float cs = sqrtf(a.gamma * (pr + pref) * rinv);
          float um = fabsf(vel[0]);
          if (ND == 3) um = fmaxf(um, fmaxf(fabsf(vel[1]), fabsf(vel[ND - 1])));
          // 2D keeps |u_x| + a only (equations.py:137-147)
          smax = fmaxf(smax, um + cs);
        }
      }
      if (a.speed != nullptr) {
        const int s0 = (blockIdx.x * T) / a.rps;
        const int s1 = (min(blockIdx.x * T + T, a.rows) - 1) / a.rps;
        if (s0 == s1) {
          const float m = block_max(smax, S.red);
          if (threadIdx.x == 0) atomic_max_nonneg(a.speed + s0, m);
        } else if (valid) {  // rows of several small solves in one CTA
          atomic_max_nonneg(a.speed + sol, smax);
        }
      }
    }
    // job -> (mode, output fields); the switch fills v with constant register indices
    // job kind: 0.. filter pairs, 10.. D_x pairs, 20.. P_x jobs
    const int k = (j < nfx) ? j : (j - nfx < nD) ? 10 + (j - nfx) : 20 + (j - nfx - nD);
    int mode, fA, fB;  // mode 0: complementary filter, 1: D, 2: P
    float2 v[B];
    switch (k) {
#define PS_FX_CASE(K)                                                                                   \
  case K: {                                                                                             \
    constexpr int c = (2 * (K) < NC) ? 2 * (K) : 0;                                                     \
    constexpr int c1 = (c + 1 < NC) ? c + 1 : c;                                                        \
    mode = 0;                                                                                           \
    fA = c;                                                                                             \
    fB = (c + 1 < NC) ? c + 1 : -1;                                                                     \
    _Pragma("unroll") for (int n2 = 0; n2 < B; ++n2) v[n2] =                                            \
        make_float2(q[c][n2], (c + 1 < NC) ? q[c1][n2] : 0.0f);                                         \
    break;                                                                                              \
  }
      PS_FX_CASE(0)
      PS_FX_CASE(1)
      PS_FX_CASE(2)
#undef PS_FX_CASE
#define PS_D_CASE(K)                                                                                    \
  case 10 + (K): {                                                                                      \
    constexpr int c = (2 * (K) < NC) ? 2 * (K) : 0;                                                     \
    mode = 1;                                                                                           \
    fA = c;                                                                                             \
    fB = (c + 1 < NC) ? c + 1 : -1;                                                                     \
    fill(v, 0, c, 0, (c + 1 < NC) ? c + 1 : -1);                                                        \
    break;                                                                                              \
  }
      PS_D_CASE(0)
      PS_D_CASE(1)
      PS_D_CASE(2)
#undef PS_D_CASE
#define PS_P_CASE(K)                                                                                    \
  case 20 + (K): {                                                                                      \
    mode = 2;                                                                                           \
    if constexpr (ND == 3) {                                                                            \
      fA = NC + (K);                                                                                    \
      fB = 2 * NC + (K);                                                                                \
      fill(v, 1, (K), 2, (K));                                                                          \
    } else {                                                                                            \
      constexpr int c = (2 * (K) + 1 < NC) ? 2 * (K) : 0;                                               \
      fA = NC + c;                                                                                      \
      fB = NC + c + 1;                                                                                  \
      fill(v, 1, c, 1, c + 1);                                                                          \
    }                                                                                                   \
    break;                                                                                              \
  }
      PS_P_CASE(0)
      PS_P_CASE(1)
      PS_P_CASE(2)
      PS_P_CASE(3)
      PS_P_CASE(4)
#undef PS_P_CASE
      default:
        mode = 2;
        fA = fB = -1;
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) v[n2] = make_float2(0.0f, 0.0f);
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
        const float sc = (mode == 0) ? (1.0f / N) - P : P;
        v[r].x *= sc;
        v[r].y *= sc;
      }
    }
    pf.inv(v);
    if (mode == 0) {
      switch (k) {
#define PS_FX_BACK(K)                                                                                   \
  case K: {                                                                                             \
    constexpr int c = (2 * (K) < NC) ? 2 * (K) : 0;                                                     \
    constexpr int c1 = (c + 1 < NC) ? c + 1 : c;                                                        \
    _Pragma("unroll") for (int n2 = 0; n2 < B; ++n2) {                                                  \
      q[c][n2] -= v[n2].x;                                                                              \
      if (valid) a.Uw[c * a.fs + rbase + A * n2] = q[c][n2];                                            \
      if constexpr (c + 1 < NC) {                                                                       \
        q[c1][n2] -= v[n2].y;                                                                           \
        if (valid) a.Uw[c1 * a.fs + rbase + A * n2] = q[c1][n2];                                        \
      }                                                                                                 \
    }                                                                                                   \
    break;                                                                                              \
  }
        PS_FX_BACK(0)
        PS_FX_BACK(1)
        PS_FX_BACK(2)
#undef PS_FX_BACK
        default:
          break;
      }
    } else if (valid && fA >= 0) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[fA * a.fs + obase + A * n2] = v[n2].x;
        if (fB >= 0) a.out[fB * a.fs + obase + A * n2] = v[n2].y;
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

// ---------------------------------------------------------------------------
// Plain one-axis operator on nf fields (P or D), contiguous or strided.
// in and out may alias: each thread reads and writes only its own points.
// ---------------------------------------------------------------------------
struct OpArgs {
  const float* in;
  float* out;
  int nf;
  long fs;
  long ss;           // solve stride of in and out
  int rows;          // contiguous: rows of all solves
  int rps;           // rows per solve
  StridedGeom g;     // strided geometry
  AxisOps ax;
  int deriv;         // 0: P, 1: D, 2: L (Laplacian factor), 3: raw second derivative (op_symbol)
  float scale;       // multiplies the symbol (e.g. -1 for a right-hand side)
  int complement;    // P only: out = in - IFFT((1/N - P) FFT in)  (exact, see AxisOps)
  const int* active; // contiguous only, nullable: rows of inactive solves are left as they are
  float kunit;       // 2 pi / L of the axis (deriv 2, 3)
  long ss_in;        // contiguous only: solve stride of in (0: ss)
};

template <int N, int T, bool STRIDED>
__global__ void __launch_bounds__(Shape<N>::A * T) k_op(OpArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, STRIDED>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& S = *reinterpret_cast<StridedSmem<N, T, STRIDED>*>(smem_raw);
  int p, t;
  long base_in, base_out, step;
  bool valid;
  if constexpr (STRIDED) {
    p = threadIdx.x % T;
    t = threadIdx.x / T;
    const int col = blockIdx.x * T + p;
    valid = col < a.g.ncol;
    base_in = base_out = (long)blockIdx.y * a.g.os + col + (long)t * a.g.as;
    step = (long)A * a.g.as;
  } else {
    t = threadIdx.x % A;
    p = threadIdx.x / A;
    const int row = blockIdx.x * T + p;
    valid = row < a.rows;
    const int r = valid ? row : 0;
    if (a.active != nullptr && a.active[r / a.rps] == 0) valid = false;
    // in may be a field subset of a wider state (its own solve stride)
    const long loc = (long)(r % a.rps) * N + t;
    base_in = (long)(r / a.rps) * (a.ss_in ? a.ss_in : a.ss) + loc;
    base_out = (long)(r / a.rps) * a.ss + loc;
    step = A;
  }
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
#pragma unroll 1
  for (int c = 0; c < a.nf; c += 2) {
    const bool two = c + 1 < a.nf;
    float2 w[B], w0[B];
    load_pair<N>(w, a.in + c * a.fs, two ? a.in + (c + 1) * a.fs : nullptr, base_in, step, valid);
    const bool comp = a.complement && !a.deriv;
#pragma unroll
    for (int r = 0; r < B; ++r) w0[r] = w[r];
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = pf.kidx(r);
      if (comp) {
        const float s = (1.0f / N) - S.ax.P[k];
        w[r].x *= s;
        w[r].y *= s;
      } else {
        w[r] = op_symbol<N>(w[r], k, a.deriv, a.scale, a.kunit, S.ax.P, S.ax.d);
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
        a.out[c * a.fs + base_out + n2 * step] = w[n2].x;
        if (two) a.out[(c + 1) * a.fs + base_out + n2 * step] = w[n2].y;
      }
    }
  }
}

}  // namespace ps
