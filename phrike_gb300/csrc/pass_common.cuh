// Shared pieces of the pencil pass kernels: per-axis spectral tables staged in
// shared memory, tile shapes and small helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_pencil.cuh"

namespace ps {

// Per-axis device tables (built on the host in float64, stored as float).
//   P[k]  = mask(k) * sigma(k) / N                 projection / filter symbol
//   d[k]  = kphys(k) * mask(k) * sigma(k) / N      derivative symbol is i*d[k];
//           d = 0 at the Nyquist index (the reference keeps only the real part
//           of a full complex inverse transform, which drops that term)
//   twf   = W_N^{n1*k2}  laid out [k2][n1]   (forward twiddles)
//   twi   = W_N^{-n1*k2} laid out [n1][k2]   (inverse twiddles)
// Filters of the state are applied in complementary form,
//   P f = f - IFFT((1/N - P[k]) FFT f),
// which is exact and leaves the retained band untouched when m*s = 1 there
// (1/N - P[k] is then exactly 0), so a filter round trip adds no float32
// rounding noise to the modes it keeps.
struct AxisOps {
  const float* P;
  const float* d;
  const float2* twf;
  const float2* twi;
};

// Shared-memory copy of one axis' tables.
template <int N>
struct AxisSmem {
  float P[N];
  float d[N];
  float2 twf[N];
  float2 twi[N];
};

template <int N>
__device__ __forceinline__ void load_axis(AxisSmem<N>& s, const AxisOps& ax) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    s.P[i] = ax.P[i];
    s.d[i] = ax.d[i];
    s.twf[i] = ax.twf[i];
    s.twi[i] = ax.twi[i];
  }
}

// Pencils per CTA: contiguous passes (pencils along x) and strided passes
// (pencils along y or z, tiles of adjacent x columns).
template <int N> struct Tile;
template <> struct Tile<8> { static constexpr int TC = 64, TS = 16; };
template <> struct Tile<16> { static constexpr int TC = 32, TS = 16; };
template <> struct Tile<32> { static constexpr int TC = 32, TS = 16; };
template <> struct Tile<64> { static constexpr int TC = 16, TS = 16; };
template <> struct Tile<128> { static constexpr int TC = 16, TS = 16; };
template <> struct Tile<256> { static constexpr int TC = 8, TS = 16; };
template <> struct Tile<512> { static constexpr int TC = 4, TS = 16; };
template <> struct Tile<1024> { static constexpr int TC = 2, TS = 8; };
template <> struct Tile<2048> { static constexpr int TC = 1, TS = 1; };  // 1D plans only
template <> struct Tile<4096> { static constexpr int TC = 1, TS = 1; };

// Non-negative float max via integer compare (valid for x >= 0).
__device__ __forceinline__ void atomic_max_nonneg(float* addr, float x) {
  atomicMax(reinterpret_cast<int*>(addr), __float_as_int(x));
}

// Lanes of the first warp that exist (blocks of fewer than 32 threads are a
// power of two wide); shuffles stay within them.
__device__ __forceinline__ int warp_width() { return blockDim.x < 32 ? (int)blockDim.x : 32; }
__device__ __forceinline__ unsigned warp_mask() {
  return blockDim.x < 32 ? ((1u << blockDim.x) - 1u) : 0xffffffffu;
}

__device__ __forceinline__ float block_max(float v, float* red) {
  const int ww = warp_width();
  const unsigned mask = warp_mask();
  for (int o = 16; o > 0; o >>= 1)
    if (o < ww) v = fmaxf(v, __shfl_xor_sync(mask, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = (l < nw) ? red[l] : 0.0f;
    for (int o = 16; o > 0; o >>= 1)
      if (o < ww) v = fmaxf(v, __shfl_xor_sync(mask, v, o));
  }
  return v;  // valid in thread 0
}

// RK4 stage bookkeeping (classical RK4, low-storage accumulator form):
//   stage 0: acc  = U + dt/6 k;  next = U + dt/2 k
//   stage 1: acc += dt/3 k;      next = U + dt/2 k
//   stage 2: acc += dt/3 k;      next = U + dt k
//   stage 3: new  = acc + dt/6 k
struct RKCoef {
  float wacc;   // weight of k in the accumulator
  float wnext;  // weight of k in the next stage input
};
__device__ __forceinline__ RKCoef rk4_coef(int stage, float dt) {
  RKCoef c;
  c.wacc = (stage == 0 || stage == 3) ? dt * (1.0f / 6.0f) : dt * (1.0f / 3.0f);
  c.wnext = (stage == 2) ? dt : 0.5f * dt;
  return c;
}
// Midpoint RK2 (solver.py:96-105) on the same stage slots, stages 0 and 3
// only: stage 0: acc = U, next = U + dt/2 k1; stage 3: new = acc + dt k2.
__device__ __forceinline__ RKCoef rk_coef(int stage, float dt, int rk2) {
  if (!rk2) return rk4_coef(stage, dt);
  RKCoef c;
  c.wacc = (stage == 0) ? 0.0f : dt;
  c.wnext = 0.5f * dt;
  return c;
}

// One RK stage update of a state value with the accumulator in increment
// form: acc holds only sum_i w_i k_i, and U^n is added once, at the last
// stage (u = U^n + (acc + w_4 k_4)).  The sum is the same as RK4's
// U^n + sum_i w_i k_i; its float32 rounding is relative to the increments
// instead of to |U^n|.  Used where the accumulator lives in shared memory or
// where U^n is read at the last stage anyway (LGL, 1D kernels).
__device__ __forceinline__ float rk_update_incr(int stage, const RKCoef& rk, float k, float un, float& acc) {
  if (stage == 3) return un + fmaf(rk.wacc, k, acc);
  acc = (stage == 0) ? rk.wacc * k : fmaf(rk.wacc, k, acc);
  return fmaf(rk.wnext, k, un);
}

// Multiplier of the one-axis operators at spectral index k (tables hold
// m s / N and k m s / N):
//   deriv 0: P  = m s / N
//   deriv 1: D  = i k m s / N (Nyquist term zero)
//   deriv 2: L  = -k^2 m s / N, the one-axis factor of the spectral Laplacian
//            (grid.py:569-579, 1329-1338: -(kx^2 + ky^2) m s, Nyquist kept)
//   deriv 3: -k^2 / N, the second derivative without mask or filter (so that
//            P applied after it gives L exactly, Nyquist included)
// kunit = 2 pi / L of the axis; the result is scaled by `scale`.
template <int N>
__device__ __forceinline__ float2 op_symbol(float2 w, int k, int deriv, float scale, float kunit, const float* P,
                                           const float* d) {
  if (deriv == 1) {
    const float dd = scale * d[k];
    return make_float2(-w.y * dd, w.x * dd);
  }
  const float kk = (float)((k <= N / 2) ? k : k - N) * kunit;
  const float s = (deriv == 0) ? scale * P[k] : (deriv == 2) ? -kk * kk * scale * P[k] : -kk * kk * scale * (1.0f / N);
  return make_float2(w.x * s, w.y * s);
}

// Energy-perturbation form.  Inside the engine the energy slot of a state holds
// E' = E - E_ref for a per-run constant E_ref (the energy of the first cell
// when the run starts).  With p_ref = (gamma-1) E_ref the primitive pressure
// becomes p' = p - p_ref = (gamma-1)(E' - rho|u|^2/2), computed from small
// numbers, and every flux keeps its exact value:
//   momentum:  rho u_a u_b + delta_ab p'      (constant offset; each flux is
//              differentiated along its own axis, which annihilates constants)
//   energy:    (E' + p' + gamma E_ref) u_a  == (E + p) u_a
// In float32 this removes the rounding noise of |E| >> |p - <p>| at low Mach
// number from the pressure gradient.

// Conservative -> primitive -> floors -> conservative (the positivity clamp of
// the 1D/2D solvers) in energy-perturbation form: pmin_shift = p_min - p_ref.
// comps: NC = ND + 2, velocity components ND.
template <int ND>
__device__ __forceinline__ void clamp_state(float (&u)[ND + 2], float gamma, float rho_min, float pmin_shift) {
  const float rho = u[0];
  float vel[ND];
  float kin = 0.0f;
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    vel[a] = u[1 + a] / rho;
    kin = fmaf(vel[a], vel[a], kin);
  }
  const float p = (gamma - 1.0f) * (u[ND + 1] - 0.5f * rho * kin);
  // where no floor acts the reference's primitive -> conservative round trip
  // is the identity (to float64 rounding): keep the state as it is instead of
  // adding float32 rounding to E and the momenta
  if (rho >= rho_min && p >= pmin_shift) return;
  const float rc = fmaxf(rho, rho_min);
  const float pc = fmaxf(p, pmin_shift);
  u[0] = rc;
#pragma unroll
  for (int a = 0; a < ND; ++a) u[1 + a] = rc * vel[a];
  u[ND + 1] = pc / (gamma - 1.0f) + 0.5f * rc * kin;
}

// Artificial-viscosity parameters (artificial_viscosity.py:37-105, 193-235)
struct AVParams {
  int mode;      // 0 off, 1 sensor, 2 constant
  int sensor;    // 0 density, 1 pressure (2D: u_y), 2 |u|
  float nu_max, nu_const, s_ref, s_min, p, eps;
  float w[5];    // per-component weights
};

// Viscosity coefficient from |grad q| and q: the sensor
// s = clip(|grad q| / (|q| + eps) / s_ref, 0, 1) (s_ref > 0), then
// nu = nu_max ((s > s_min ? s : 0) / s_ref)^p; constant mode returns nu_const.
__device__ __forceinline__ float av_nu(const AVParams& av, float gradmag, float q) {
  if (av.mode == 2) return av.nu_const;
  float s = gradmag / (fabsf(q) + av.eps);
  if (av.s_ref > 0.0f) s = fminf(fmaxf(s / av.s_ref, 0.0f), 1.0f);
  float act = (s > av.s_min) ? s : 0.0f;
  if (av.s_ref > 0.0f) act = act / av.s_ref;
  return av.nu_max * powf(act, av.p);
}

}  // namespace ps
