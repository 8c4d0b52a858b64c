// Mixed-radix pencil passes (see mixed_radix.cuh for the pass contracts).
#include <cuda_runtime.h>

#include "mixed_radix.cuh"
#include "mr_fft.cuh"

namespace ps {
namespace {

using namespace mrfft;

// Operator symbol at spectral index k for a runtime length (op_symbol with n
// a kernel argument); the tables hold m s / n and kphys m s / n.
__device__ __forceinline__ float2 mr_symbol(float2 w, int k, int n, int deriv, float scale, float kunit,
                                            const float* P, const float* d) {
  if (deriv == 1) {
    const float dd = scale * __ldg(d + k);
    return make_float2(-w.y * dd, w.x * dd);
  }
  const float kk = (float)((2 * k <= n) ? k : k - n) * kunit;
  const float s = (deriv == 0)   ? scale * __ldg(P + k)
                  : (deriv == 2) ? -kk * kk * scale * __ldg(P + k)
                                 : -kk * kk * scale * (1.0f / n);
  return make_float2(w.x * s, w.y * s);
}

__device__ __forceinline__ float complement_factor(const MrAxis& ax, int k) { return (1.0f / ax.n) - __ldg(ax.P + k); }

// Solve-local offsets of element 0 of the CTA's pencils (-1: past the end).
__device__ __forceinline__ void mr_bases(const MrGeom& g, long* pb) {
  const long j0 = (long)blockIdx.x * g.pg;
  for (int q = threadIdx.x; q < g.pg; q += blockDim.x) {
    const long j = j0 + q;
    pb[q] = (j < g.npen) ? (j / g.es) * g.es * g.n + (j % g.es) : -1L;
  }
  __syncthreads();
}

// f(q, i, off) for every element i of every pencil q of the CTA; off is the
// solve-local offset (-1 for pencils past the end).  x pencils run i fastest,
// strided pencils q fastest, so that either way a warp reads adjacent words.
template <typename F>
__device__ __forceinline__ void mr_each(const MrGeom& g, const long* pb, F&& f) {
  const int tot = g.pg * g.n;
  const bool rows = g.es == 1;
  const float inv = 1.0f / (float)(rows ? g.n : g.pg);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    int q, i;
    if (rows) {
      q = qdiv(e, inv);
      i = e - q * g.n;
    } else {
      i = qdiv(e, inv);
      q = e - i * g.pg;
    }
    const long b = pb[q];
    f(q, i, b < 0 ? -1L : b + (long)i * g.es);
  }
}

// f(s, q, k, w&) for every spectral value of signals 0..nsig-1
template <typename F>
__device__ __forceinline__ void mr_spectra(float2* sig, const MrGeom& g, int nsig, F&& f) {
  const int n = g.n, pitch = n + 1;
  const int tot = nsig * g.pg * n;
  const float inv = 1.0f / (float)n;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int p2 = qdiv(e, inv), k = e - p2 * n;
    f(p2 / g.pg, k, sig[p2 * pitch + k]);
  }
}

// ---------------------------------------------------------------------------
// out = op(in) along one axis
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_mr_op(MrOpArgs a) {
  extern __shared__ __align__(16) float2 mr_sig[];
  __shared__ long pb[kMrMaxPencils];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  mr_bases(a.g, pb);
  const int pg = a.g.pg, n = a.g.n, pitch = n + 1;
  float2* tws = mr_sig + 2 * pg * pitch;  // twiddles W_n^q in shared memory
  for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = __ldg(a.ax.tw + i);
  MrAxis ax = a.ax;
  ax.tw = tws;
  const float* in = a.in + (long)sol * a.ss_in;
  float* out = a.out + (long)sol * a.ss_out;
  for (int f0 = 0; f0 < a.nf; f0 += 4) {
    const int nsig = (f0 + 2 < a.nf) ? 2 : 1;
    mr_each(a.g, pb, [&](int q, int i, long off) {
      for (int s = 0; s < nsig; ++s) {
        const int fa = f0 + 2 * s, fb = fa + 1;
        float2 v = make_float2(0.0f, 0.0f);
        if (off >= 0) {
          v.x = in[fa * a.fs + off];
          if (fb < a.nf) v.y = in[fb * a.fs + off];
        }
        mr_sig[(s * pg + q) * pitch + i] = v;
      }
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, false);
    mr_spectra(mr_sig, a.g, nsig, [&](int, int k, float2& w) {
      if (a.complement) w = cscale(w, complement_factor(a.ax, k));
      else w = mr_symbol(w, k, a.g.n, a.deriv, a.scale, a.kunit, a.ax.P, a.ax.d);
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long off) {
      if (off < 0) return;
      for (int s = 0; s < nsig; ++s) {
        const int fa = f0 + 2 * s, fb = fa + 1;
        const float2 w = mr_sig[(s * pg + q) * pitch + i];
        const long oa = fa * a.fs + off, ob = fb * a.fs + off;
        if (a.complement) {
          const float va = in[oa] - w.x;
          const float vb = (fb < a.nf) ? in[ob] - w.y : 0.0f;
          out[oa] = va;
          if (fb < a.nf) out[ob] = vb;
        } else {
          out[oa] = w.x;
          if (fb < a.nf) out[ob] = w.y;
        }
      }
    });
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// x pass: [fused filter P_x of the state], CFL speed, G = [D_x F^x, P_x F^y (, P_x F^z)]
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_mr_x(MrXArgs a) {
  constexpr int NC = ND + 2;
  constexpr int NPAIR = (NC + 1) / 2;
  extern __shared__ __align__(16) float2 mr_sig[];
  __shared__ long pb[kMrMaxPencils];
  __shared__ float red[32];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  mr_bases(a.g, pb);
  const int pg = a.g.pg, n = a.g.n, pitch = n + 1;
  float2* tws = mr_sig + 2 * pg * pitch;  // twiddles W_n^q in shared memory
  for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = __ldg(a.ax.tw + i);
  MrAxis ax = a.ax;
  ax.tw = tws;
  float* prim = reinterpret_cast<float*>(tws + n);  // [NC][pg][n]
  auto pv = [&](int c, int q, int i) -> float& { return prim[(c * pg + q) * n + i]; };
  const float er = a.eref[sol];
  const float eshift = a.shift_in ? er : 0.0f;
  const float g1 = a.gamma - 1.0f, ig1 = 1.0f / g1;
  const float pref = g1 * er, href = a.gamma * er;
  const float* U = a.U + (long)sol * a.ssU;
  mr_each(a.g, pb, [&](int q, int i, long off) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      float v = (c == 0) ? 1.0f : 0.0f;
      if (off >= 0) v = U[c * a.fs + off] - ((c == NC - 1) ? eshift : 0.0f);
      pv(c, q, i) = v;
    }
  });
  if (a.Uw != nullptr) {  // complementary filter P_x of the state, written to Uw
    float* Uw = a.Uw + (long)sol * a.ssU;
    for (int c0 = 0; c0 < NC; c0 += 4) {
      const int nsig = (c0 + 2 < NC) ? 2 : 1;
      __syncthreads();
      mr_each(a.g, pb, [&](int q, int i, long) {
        for (int s = 0; s < nsig; ++s) {
          const int ca = c0 + 2 * s, cb = ca + 1;
          mr_sig[(s * pg + q) * pitch + i] = make_float2(pv(ca, q, i), cb < NC ? pv(cb, q, i) : 0.0f);
        }
      });
      mr_fft(mr_sig, pitch, nsig * pg, ax, false);
      mr_spectra(mr_sig, a.g, nsig, [&](int, int k, float2& w) { w = cscale(w, complement_factor(a.ax, k)); });
      mr_fft(mr_sig, pitch, nsig * pg, ax, true);
      mr_each(a.g, pb, [&](int q, int i, long off) {
        for (int s = 0; s < nsig; ++s) {
          const int ca = c0 + 2 * s, cb = ca + 1;
          const float2 w = mr_sig[(s * pg + q) * pitch + i];
          const float va = pv(ca, q, i) - w.x;
          pv(ca, q, i) = va;
          if (off >= 0) Uw[ca * a.fs + off] = va + ((ca == NC - 1) ? eshift : 0.0f);
          if (cb < NC) {
            const float vb = pv(cb, q, i) - w.y;
            pv(cb, q, i) = vb;
            if (off >= 0) Uw[cb * a.fs + off] = vb + ((cb == NC - 1) ? eshift : 0.0f);
          }
        }
      });
    }
  }
  __syncthreads();
  // conservative -> primitive (rho, u_1..u_ND, p') in place; CFL speed
  float smax = 0.0f;
  mr_each(a.g, pb, [&](int q, int i, long off) {
    const float rho = pv(0, q, i);
    const float rinv = 1.0f / rho;
    float kin = 0.0f;
    float vel[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      vel[d] = pv(1 + d, q, i) * rinv;
      kin = fmaf(vel[d], vel[d], kin);
      pv(1 + d, q, i) = vel[d];
    }
    const float pr = g1 * (pv(NC - 1, q, i) - 0.5f * rho * kin);
    pv(NC - 1, q, i) = pr;
    if (a.speed != nullptr && off >= 0) {
      const float cs = sqrtf(a.gamma * (pr + pref) * rinv);
      float um = fabsf(vel[0]);
      if (ND == 3) um = fmaxf(um, fmaxf(fabsf(vel[1]), fabsf(vel[ND - 1])));
      smax = fmaxf(smax, um + cs);
    }
  });
  if (a.speed != nullptr) {
    const float m = block_max(smax, red);
    if (threadIdx.x == 0) atomic_max_nonneg(a.speed + sol, m);
  }
  __syncthreads();
  // F^dir_c from the primitives
  auto flux = [&](int dir, int c, int q, int i) -> float {
    const float rho = pv(0, q, i), ua = pv(1 + dir, q, i), pr = pv(NC - 1, q, i);
    if (c == 0) return rho * ua;
    if (c == NC - 1) {
      float kin = 0.0f;
#pragma unroll
      for (int d = 0; d < ND; ++d) kin = fmaf(pv(1 + d, q, i), pv(1 + d, q, i), kin);
      const float Ep = fmaf(pr, ig1, 0.5f * rho * kin);
      return ((Ep + pr) + href) * ua;
    }
    const float rv = rho * ua * pv(c, q, i);
    return (c - 1 == dir) ? rv + pr : rv;
  };
  float* out = a.out + (long)sol * a.ssOut;
  constexpr int NJOB = ND * NPAIR;  // job j: direction j / NPAIR, components 2 (j % NPAIR), +1
  for (int j0 = 0; j0 < NJOB; j0 += 2) {
    const int nsig = (j0 + 1 < NJOB) ? 2 : 1;
    __syncthreads();
    mr_each(a.g, pb, [&](int q, int i, long) {
      for (int s = 0; s < nsig; ++s) {
        const int j = j0 + s, dir = j / NPAIR, c = 2 * (j % NPAIR);
        mr_sig[(s * pg + q) * pitch + i] = make_float2(flux(dir, c, q, i), (c + 1 < NC) ? flux(dir, c + 1, q, i) : 0.0f);
      }
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, false);
    mr_spectra(mr_sig, a.g, nsig, [&](int s, int k, float2& w) {
      const int dir = (j0 + s) / NPAIR;
      w = mr_symbol(w, k, n, dir == 0 ? 1 : 0, 1.0f, 0.0f, a.ax.P, a.ax.d);
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long off) {
      if (off < 0) return;
      for (int s = 0; s < nsig; ++s) {
        const int j = j0 + s, dir = j / NPAIR, c = 2 * (j % NPAIR);
        const float2 w = mr_sig[(s * pg + q) * pitch + i];
        out[(dir * NC + c) * a.fs + off] = w.x;
        if (c + 1 < NC) out[(dir * NC + c + 1) * a.fs + off] = w.y;
      }
    });
  }
}

// ---------------------------------------------------------------------------
// 3D y pass: AB = [P_y G + D_y H^y (5), P_y H^z (5)]
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_mr_y3(MrY3Args a) {
  extern __shared__ __align__(16) float2 mr_sig[];
  __shared__ long pb[kMrMaxPencils];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  mr_bases(a.g, pb);
  const int pg = a.g.pg, n = a.g.n, pitch = n + 1;
  float2* tws = mr_sig + 2 * pg * pitch;  // twiddles W_n^q in shared memory
  for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = __ldg(a.ax.tw + i);
  MrAxis ax = a.ax;
  ax.tw = tws;
  const float* G = a.G + (long)sol * a.ssG;
  float* out = a.out + (long)sol * a.ssOut;
  // jobs 0..2: sums over component pairs (0,1), (2,3), (4); jobs 3..5: P_y H^z pairs
  for (int job = 0; job < 3; ++job) {
    const int c = 2 * job;
    const bool two = c + 1 < 5;
    __syncthreads();
    mr_each(a.g, pb, [&](int q, int i, long off) {
      float2 za = make_float2(0.0f, 0.0f), zb = za;
      if (off >= 0) {
        za.x = G[c * a.fs + off];
        zb.x = G[(5 + c) * a.fs + off];
        if (two) {
          za.y = G[(c + 1) * a.fs + off];
          zb.y = G[(6 + c) * a.fs + off];
        }
      }
      mr_sig[q * pitch + i] = za;
      mr_sig[(pg + q) * pitch + i] = zb;
    });
    mr_fft(mr_sig, pitch, 2 * pg, ax, false);
    mr_spectra(mr_sig, a.g, 1, [&](int, int k, float2& w) {
      const float2 z = mr_sig[(&w - mr_sig) + pg * pitch];
      const float P = __ldg(a.ax.P + k), d = __ldg(a.ax.d + k);
      w = make_float2(fmaf(P, w.x, -d * z.y), fmaf(P, w.y, d * z.x));
    });
    mr_fft(mr_sig, pitch, pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long off) {
      if (off < 0) return;
      const float2 w = mr_sig[q * pitch + i];
      out[c * a.fs + off] = w.x;
      if (two) out[(c + 1) * a.fs + off] = w.y;
    });
  }
  for (int c0 = 0; c0 < 5; c0 += 4) {  // H^z pairs (0,1),(2,3) then (4)
    const int nsig = (c0 + 2 < 5) ? 2 : 1;
    __syncthreads();
    mr_each(a.g, pb, [&](int q, int i, long off) {
      for (int s = 0; s < nsig; ++s) {
        const int ca = c0 + 2 * s, cb = ca + 1;
        float2 v = make_float2(0.0f, 0.0f);
        if (off >= 0) {
          v.x = G[(10 + ca) * a.fs + off];
          if (cb < 5) v.y = G[(10 + cb) * a.fs + off];
        }
        mr_sig[(s * pg + q) * pitch + i] = v;
      }
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, false);
    mr_spectra(mr_sig, a.g, nsig, [&](int, int k, float2& w) { w = cscale(w, __ldg(a.ax.P + k)); });
    mr_fft(mr_sig, pitch, nsig * pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long off) {
      if (off < 0) return;
      for (int s = 0; s < nsig; ++s) {
        const int ca = c0 + 2 * s, cb = ca + 1;
        const float2 w = mr_sig[(s * pg + q) * pitch + i];
        out[(5 + ca) * a.fs + off] = w.x;
        if (cb < 5) out[(5 + cb) * a.fs + off] = w.y;
      }
    });
  }
}

// ---------------------------------------------------------------------------
// last axis: rhs = -(P a + D b) (+ gravity), RK stage update, 2D clamp, the
// last factor of the end-of-step filter.  The accumulator is the plain RK4
// sum acc = U^n + sum w_i k_i, as in the power-of-two last pass.
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_mr_last(MrLastArgs a) {
  constexpr int NC = ND + 2;
  extern __shared__ __align__(16) float2 mr_sig[];
  __shared__ long pb[kMrMaxPencils];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  mr_bases(a.g, pb);
  const int pg = a.g.pg, n = a.g.n, pitch = n + 1;
  float2* tws = mr_sig + 2 * pg * pitch;  // twiddles W_n^q in shared memory
  for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = __ldg(a.ax.tw + i);
  MrAxis ax = a.ax;
  ax.tw = tws;
  float* rb = reinterpret_cast<float*>(tws + n);  // [NC][pg][n]
  auto rv = [&](int c, int q, int i) -> float& { return rb[(c * pg + q) * n + i]; };
  const float* AB = a.AB + (long)sol * a.ssAB;
  for (int c = 0; c < NC; c += 2) {
    const bool two = c + 1 < NC;
    __syncthreads();
    mr_each(a.g, pb, [&](int q, int i, long off) {
      float2 za = make_float2(0.0f, 0.0f), zb = za;
      if (off >= 0) {
        za.x = AB[(a.fa0 + c) * a.fs + off];
        zb.x = AB[(a.fb0 + c) * a.fs + off];
        if (two) {
          za.y = AB[(a.fa0 + c + 1) * a.fs + off];
          zb.y = AB[(a.fb0 + c + 1) * a.fs + off];
        }
      }
      mr_sig[q * pitch + i] = za;
      mr_sig[(pg + q) * pitch + i] = zb;
    });
    mr_fft(mr_sig, pitch, 2 * pg, ax, false);
    mr_spectra(mr_sig, a.g, 1, [&](int, int k, float2& w) {
      const float2 z = mr_sig[(&w - mr_sig) + pg * pitch];
      const float P = -__ldg(a.ax.P + k), d = -__ldg(a.ax.d + k);
      w = make_float2(fmaf(P, w.x, -d * z.y), fmaf(P, w.y, d * z.x));
    });
    mr_fft(mr_sig, pitch, pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long) {
      const float2 w = mr_sig[q * pitch + i];
      rv(c, q, i) = w.x;
      if (two) rv(c + 1, q, i) = w.y;
    });
  }
  __syncthreads();
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  const float pmin_shift = a.p_min - (a.gamma - 1.0f) * a.eref[sol];
  float* const acc_s = (a.acc != nullptr) ? a.acc + (long)sol * a.ssAcc : nullptr;
  float* const out_s = a.out + (long)sol * a.ssOut;
  const float* const un_s = a.Un + (long)sol * a.ssUn;
  const float* const uin = a.Uin + (long)sol * a.ssUn;
  const bool filt = a.stage == 3 && a.filter_last;
  mr_each(a.g, pb, [&](int q, int i, long off) {
    if (off < 0) return;
    float k[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) k[c] = rv(c, q, i);
    if (a.gravity) {  // rho g on the momenta, g . m on the energy
      const float rho = uin[off];
      float gm = 0.0f;
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        k[1 + d] = fmaf(rho, a.grav[d], k[1 + d]);
        gm = fmaf(a.grav[d], uin[off + (1 + d) * a.fs], gm);
      }
      k[NC - 1] += gm;
    }
    if (a.stage < 0) {
#pragma unroll
      for (int c = 0; c < NC; ++c) out_s[c * a.fs + off] = k[c];
      return;
    }
    // the point's loads before its stores: a store between them would make
    // each component wait for the previous one's round trip to memory
    float vu[NC], va[NC], u[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const long o = c * a.fs + off;
      vu[c] = (a.stage != 3) ? un_s[o] : 0.0f;
      va[c] = (a.stage != 0) ? acc_s[o] : 0.0f;
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (a.stage == 3) {
        u[c] = fmaf(rk.wacc, k[c], va[c]);
      } else {
        va[c] = fmaf(rk.wacc, k[c], (a.stage == 0) ? vu[c] : va[c]);
        u[c] = fmaf(rk.wnext, k[c], vu[c]);
      }
    }
    if (a.stage != 3) {
#pragma unroll
      for (int c = 0; c < NC; ++c) acc_s[c * a.fs + off] = va[c];
    }
    if (a.clamp) clamp_state<ND>(u, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (filt) rv(c, q, i) = u[c];
      else out_s[c * a.fs + off] = u[c];
    }
  });
  if (!filt) return;
  for (int c0 = 0; c0 < NC; c0 += 4) {
    const int nsig = (c0 + 2 < NC) ? 2 : 1;
    __syncthreads();
    mr_each(a.g, pb, [&](int q, int i, long) {
      for (int s = 0; s < nsig; ++s) {
        const int ca = c0 + 2 * s, cb = ca + 1;
        mr_sig[(s * pg + q) * pitch + i] = make_float2(rv(ca, q, i), cb < NC ? rv(cb, q, i) : 0.0f);
      }
    });
    mr_fft(mr_sig, pitch, nsig * pg, ax, false);
    mr_spectra(mr_sig, a.g, nsig, [&](int, int k, float2& w) { w = cscale(w, complement_factor(a.ax, k)); });
    mr_fft(mr_sig, pitch, nsig * pg, ax, true);
    mr_each(a.g, pb, [&](int q, int i, long off) {
      if (off < 0) return;
      for (int s = 0; s < nsig; ++s) {
        const int ca = c0 + 2 * s, cb = ca + 1;
        const float2 w = mr_sig[(s * pg + q) * pitch + i];
        out_s[ca * a.fs + off] = rv(ca, q, i) - w.x;
        if (cb < NC) out_s[cb * a.fs + off] = rv(cb, q, i) - w.y;
      }
    });
  }
}

// ---------------------------------------------------------------------------
// 1D stage: k = -D F(U) (+ gravity), increment-form RK update, 1D clamp.  One
// pencil per solve.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_mr_line(MrLineArgs a) {
  extern __shared__ __align__(16) float2 mr_sig[];
  __shared__ long pb[kMrMaxPencils];
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  mr_bases(a.g, pb);
  const int pg = 1, n = a.g.n, pitch = n + 1;
  float2* tws = mr_sig + 2 * pg * pitch;  // twiddles W_n^q in shared memory
  for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = __ldg(a.ax.tw + i);
  MrAxis ax = a.ax;
  ax.tw = tws;

  const float er = a.eref[sol];
  const float g1 = a.gamma - 1.0f, href = a.gamma * er;
  const float* in = a.in + (long)sol * a.ss;
  mr_each(a.g, pb, [&](int, int i, long) {
    const float rho = in[i], m = in[n + i], E = in[2 * n + i];
    const float u = m / rho;
    const float p = g1 * (E - 0.5f * rho * u * u);  // p' (E holds E')
    const float mom = rho * u;
    mr_sig[i] = make_float2(mom, mom * u + p);
    mr_sig[pitch + i] = make_float2(((E + p) + href) * u, 0.0f);
  });
  mr_fft(mr_sig, pitch, 2, ax, false);
  mr_spectra(mr_sig, a.g, 2, [&](int, int k, float2& w) {
    const float dd = __ldg(a.ax.d + k);
    w = make_float2(w.y * dd, -w.x * dd);
  });
  mr_fft(mr_sig, pitch, 2, ax, true);
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  const float pmin_shift = a.p_min - g1 * er;
  float* out = a.out + (long)sol * a.ss;
  float* acc = a.acc + (long)sol * a.ss;
  const float* un = a.Un + (long)sol * a.ss;
  mr_each(a.g, pb, [&](int, int i, long) {
    float k[3] = {mr_sig[i].x, mr_sig[i].y, mr_sig[pitch + i].x};
    if (a.gx != 0.0f) {  // gravity source (solver.py:82-91)
      const float rho = in[i];
      const float u = in[n + i] / rho;
      k[1] += rho * a.gx;
      k[2] += rho * a.gx * u;
    }
    if (a.stage < 0) {
#pragma unroll
      for (int c = 0; c < 3; ++c) out[c * n + i] = k[c];
      return;
    }
    float u3[3], vu[3], va[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {  // loads before stores
      vu[c] = un[c * n + i];
      va[c] = (a.stage == 0) ? 0.0f : acc[c * n + i];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) u3[c] = rk_update_incr(a.stage, rk, k[c], vu[c], va[c]);
    if (a.stage != 3) {
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c * n + i] = va[c];
    }
    clamp_state<1>(u3, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
    for (int c = 0; c < 3; ++c) out[c * n + i] = u3[c];
  });
}

cudaError_t launch_cfg(const void* fn, const MrGeom& g, int nsolve, void** args, cudaStream_t s) {
  if (g.smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, g.smem);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)((g.npen + g.pg - 1) / g.pg), (unsigned)nsolve);
  return cudaLaunchKernel(fn, grid, dim3(g.threads), args, (size_t)g.smem, s);
}

}  // namespace

bool mr_factor(int n, int* radix, int* nst) {
  int m = n, k = 0;
  const int order[4] = {4, 3, 5, 2};
  for (int r : order)
    while (m % r == 0 && k < kMrMaxStages) {
      radix[k++] = r;
      m /= r;
    }
  *nst = k;
  return m == 1 && n >= 2;
}

MrGeom mr_geom(const MrAxis& ax, long es, long npen, int extra_per_pencil) {
  MrGeom g{};
  g.n = ax.n;
  g.es = es;
  g.npen = npen;
  const int per = 2 * (ax.n + 1) * (int)sizeof(float2) + extra_per_pencil;
  const int budget = 100 * 1024;  // two or more CTAs per SM where the pencils allow it
  int pg = kMrThreads / (2 * ax.ntp);
  if (pg < 1) pg = 1;
  while (pg > 1 && pg * per + ax.n * (int)sizeof(float2) > budget) --pg;
  if (pg > kMrMaxPencils) pg = kMrMaxPencils;
  if (pg > npen) pg = (int)npen;
  if (pg < 1) pg = 1;
  g.pg = pg;
  const int t = 2 * pg * ax.ntp;
  g.threads = (t + 31) / 32 * 32;
  g.smem = pg * per + ax.n * (int)sizeof(float2);  // + the twiddle table
  return g;
}

cudaError_t launch_mr_op(const MrOpArgs& a, int nsolve, cudaStream_t s) {
  MrOpArgs c = a;
  void* args[] = {&c};
  return launch_cfg((const void*)k_mr_op, a.g, nsolve, args, s);
}

cudaError_t launch_mr_x(const MrXArgs& a, int nsolve, cudaStream_t s) {
  MrXArgs c = a;
  void* args[] = {&c};
  if (a.nd == 2) return launch_cfg((const void*)k_mr_x<2>, a.g, nsolve, args, s);
  if (a.nd == 3) return launch_cfg((const void*)k_mr_x<3>, a.g, nsolve, args, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_mr_y3(const MrY3Args& a, int nsolve, cudaStream_t s) {
  MrY3Args c = a;
  void* args[] = {&c};
  return launch_cfg((const void*)k_mr_y3, a.g, nsolve, args, s);
}

cudaError_t launch_mr_last(const MrLastArgs& a, int nsolve, cudaStream_t s) {
  MrLastArgs c = a;
  void* args[] = {&c};
  if (a.nd == 2) return launch_cfg((const void*)k_mr_last<2>, a.g, nsolve, args, s);
  if (a.nd == 3) return launch_cfg((const void*)k_mr_last<3>, a.g, nsolve, args, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_mr_line(const MrLineArgs& a, int nsolve, cudaStream_t s) {
  MrLineArgs c = a;
  void* args[] = {&c};
  return launch_cfg((const void*)k_mr_line, a.g, nsolve, args, s);
}

}  // namespace ps
