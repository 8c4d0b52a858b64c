// Spectral interpolation of Fourier fields at arbitrary points and the
// leap-frog advection of tracer particles (phrike/tracers.py:35-236 with
// phrike/grid.py:581-618, 1180-1222, 1520-1632).
//
// The reference evaluates  f(x) = Re( sum_k c_k F_k exp(i k.x) ) / N_total,
// F = FFT(f), c = dealias mask x filter (separable), k = 2 pi fftfreq(N)/L
// per axis (Nyquist at -N/2).  Substituting F gives a separable sum over the
// grid points,
//     f(x_p) = Re sum_j f_j  K_x(x_p - x_jx) K_y(y_p - y_jy) K_z(z_p - z_jz),
//     K_a(x_p - j L/N) = sum_q (c_q / N) exp(2 pi i k_q x_p / L) W_N^{q j},
// with W_N = exp(-2 pi i / N).  One CTA serves TPC tracers: it builds their
// per-axis weights K_a in shared memory (an N-point DFT of g_q = (c_q/N)
// exp(2 pi i k_q x_p / L) per axis and tracer, phases reduced in float64),
// then sweeps the field once, each warp over (row, segment) units with lanes
// along x (coalesced; a lane's points of a unit are loaded together), and
// accumulates Re(K_x K_y K_z f) for all its tracers.
// K_a is complex only through the unpaired Nyquist term (even N, dealias
// off); K_x's imaginary part is carried only then (NYQX).  Partial sums are
// float32 over TR_FLUSH units, then summed across the warp and added to
// float64 accumulators in shared memory.
//
// The velocity mode evaluates u_a = U[1+a] / U[0] on the fly (the primitive
// velocity of equations.primitive) and, with pos/prev given, advances the
// tracers by leap-frog (Euler on the first step) and wraps them into [0, L)
// with numpy's mod rule.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "plan.cuh"

namespace ps {
namespace {

constexpr int TR_THREADS = 256;
constexpr int TR_WARPS = TR_THREADS / 32;
constexpr int TR_FLUSH = 16;      // units summed in float32 before the float64 accumulators
constexpr int TR_MAXN = 8192;     // points per axis

struct TracerArgs {
  const float* f;      // field mode: nf fields of `cells` floats; velocity mode: the state U
  int velocity;        // 1: component a is U[1+a] / U[0]
  int nf;              // components evaluated (1..3)
  long cells;
  int nd;
  int n[3];            // points per axis, x contiguous; 1 beyond nd
  double len[3];
  const float* P[3];   // per-axis c_q / N in fftfreq order (the plan's projection tables)
  int np;
  double* pos;         // [nd][np] point coordinates
  double* prev;        // [nd][np] previous positions (advection mode) or null
  int first;           // 1: Euler step (first leap-frog step)
  double dt;
  float* out;          // [nf][np] values (evaluation mode) or null
};

// numpy's float mod for b > 0: result in [0, b), sign of b
__device__ __forceinline__ double np_mod(double a, double b) {
  double r = fmod(a, b);
  if (r != 0.0 && r < 0.0) r += b;
  if (r == 0.0) r = 0.0;  // +0
  return r;
}

template <int TPC, bool NYQX, int MX>
__global__ void __launch_bounds__(TR_THREADS) k_tracers(TracerArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n0 = a.n[0], n1 = a.n[1], n2 = a.n[2];
  const int nmax = max(n0, max(n1, n2));
  float2* W = reinterpret_cast<float2*>(smem_raw);        // [nmax]
  float2* G = W + nmax;                                    // [TPC][nmax]
  float2* Ky = G + TPC * nmax;                             // [TPC][n1]
  float2* Kz = Ky + TPC * n1;                              // [TPC][n2]
  float* Kx = reinterpret_cast<float*>(Kz + TPC * n2);     // [TPC][n0] (x2 when NYQX: re, im)
  double* red = reinterpret_cast<double*>(Kx + TPC * n0 * (NYQX ? 2 : 1) + 2);  // [TR_WARPS][TPC*3]
  red = reinterpret_cast<double*>((reinterpret_cast<unsigned long long>(red) + 7ull) & ~7ull);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p0 = blockIdx.x * TPC;
  const int ntr = min(TPC, a.np - p0);

  // ---- per-axis weights
  for (int ax = 0; ax < 3; ++ax) {
    const int N = a.n[ax];
    if (ax >= a.nd) {  // missing axes: K = 1
      for (int t = tid; t < TPC; t += blockDim.x) (ax == 1 ? Ky : Kz)[t] = make_float2(1.0f, 0.0f);
      continue;
    }
    for (int m = tid; m < N; m += blockDim.x) {
      float s, c;
      sincospif(2.0f * (float)m / (float)N, &s, &c);
      W[m] = make_float2(c, -s);
    }
    const double inv_len = 1.0 / a.len[ax];
    for (int idx = tid; idx < TPC * N; idx += blockDim.x) {
      const int t = idx / N, q = idx - t * N;
      float2 g = make_float2(0.0f, 0.0f);
      const float cq = a.P[ax][q];
      if (t < ntr && cq != 0.0f) {
        const int kq = (q <= (N - 1) / 2) ? q : q - N;
        double ph = (double)kq * (a.pos[(long)ax * a.np + p0 + t] * inv_len);
        ph -= floor(ph);  // turns in [0, 1)
        float s, c;
        sincospif((float)(2.0 * ph), &s, &c);
        g = make_float2(cq * c, cq * s);
      }
      G[t * nmax + q] = g;
    }
    __syncthreads();
    for (int idx = tid; idx < TPC * N; idx += blockDim.x) {
      const int t = idx / N, j = idx - t * N;
      const float2* gt = G + t * nmax;
      float re = 0.0f, im = 0.0f;
      int m = 0;  // (q * j) mod N
      for (int q = 0; q < N; ++q) {
        const float2 g = gt[q], w = W[m];
        re = fmaf(g.x, w.x, fmaf(-g.y, w.y, re));
        im = fmaf(g.x, w.y, fmaf(g.y, w.x, im));
        m += j;
        if (m >= N) m -= N;
      }
      if (ax == 0) {
        if (NYQX) {
          Kx[(t * n0 + j) * 2] = re;
          Kx[(t * n0 + j) * 2 + 1] = im;
        } else {
          Kx[t * n0 + j] = re;
        }
      } else {
        (ax == 1 ? Ky : Kz)[t * N + j] = make_float2(re, im);
      }
    }
    __syncthreads();
  }
  __syncthreads();  // the unit weights of missing axes

  // ---- the sweep over the field: each warp takes (row, segment) units of up
  // to 32 * MX points along x; lanes hold MX points each, loaded together
  const int rows = n1 * n2;
  const int ux = min(n0, 32 * MX);
  const int segs = (n0 + ux - 1) / ux;
  const int units = rows * segs;
  for (int i = tid; i < TR_WARPS * TPC * 3; i += blockDim.x) red[i] = 0.0;
  __syncthreads();
  float sf[TPC][3];
#pragma unroll
  for (int t = 0; t < TPC; ++t)
#pragma unroll
    for (int c = 0; c < 3; ++c) sf[t][c] = 0.0f;
  // float partials of TR_FLUSH units are summed across the warp's lanes and
  // added to the warp's float64 accumulators in shared memory
  auto flush = [&]() {
#pragma unroll
    for (int t = 0; t < TPC; ++t)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float v = sf[t][c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp * TPC * 3 + t * 3 + c] += (double)v;
        sf[t][c] = 0.0f;
      }
  };
  int since = 0;
  for (int u = warp; u < units; u += TR_WARPS) {
    const int row = (segs == 1) ? u : u / segs, seg = u - row * segs;
    const int jz = row / n1, jy = row - jz * n1;
    float v[MX][3];
    int jxs[MX];
#pragma unroll
    for (int m = 0; m < MX; ++m) {
      const int jx = seg * ux + 32 * m + lane;
      const bool ok = jx < n0 && 32 * m + lane < ux;
      jxs[m] = ok ? jx : -1;
      const long cell = (long)row * n0 + (ok ? jx : 0);
      if (a.velocity) {
        const float rinv = ok ? 1.0f / a.f[cell] : 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) v[m][c] = (ok && c < a.nf) ? a.f[(1 + c) * a.cells + cell] * rinv : 0.0f;
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) v[m][c] = (ok && c < a.nf) ? a.f[c * a.cells + cell] : 0.0f;
      }
    }
#pragma unroll
    for (int t = 0; t < TPC; ++t) {
      const float2 wy = Ky[t * n1 + jy], wz = Kz[t * n2 + jz];
      const float wr = wy.x * wz.x - wy.y * wz.y, wi = wy.x * wz.y + wy.y * wz.x;
      float pr[3] = {0.0f, 0.0f, 0.0f}, pi[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int m = 0; m < MX; ++m) {
        if (jxs[m] < 0) continue;
        if (NYQX) {
          const float kr = Kx[(t * n0 + jxs[m]) * 2], ki = Kx[(t * n0 + jxs[m]) * 2 + 1];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            pr[c] = fmaf(v[m][c], kr, pr[c]);
            pi[c] = fmaf(v[m][c], ki, pi[c]);
          }
        } else {
          const float kr = Kx[t * n0 + jxs[m]];
#pragma unroll
          for (int c = 0; c < 3; ++c) pr[c] = fmaf(v[m][c], kr, pr[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) sf[t][c] = fmaf(pr[c], wr, NYQX ? fmaf(-pi[c], wi, sf[t][c]) : sf[t][c]);
    }
    if (++since == TR_FLUSH) {
      since = 0;
      flush();
    }
  }
  flush();
  __syncthreads();
  if (tid < TPC * 3) {
    const int t = tid / 3, c = tid % 3;
    if (t < ntr && c < a.nf) {
      double v = 0.0;
      for (int w = 0; w < TR_WARPS; ++w) v += red[w * TPC * 3 + tid];
      const long p = p0 + t;
      if (a.out != nullptr) a.out[(long)c * a.np + p] = (float)v;
      if (a.prev != nullptr) {  // leap-frog (tracers.py:50-79, 103-148, 178-236)
        const long i = (long)c * a.np + p;
        const double x = a.pos[i];
        double xn;
        if (a.first) {
          a.prev[i] = x;
          xn = x + a.dt * v;
        } else {
          xn = a.prev[i] + 2.0 * a.dt * v;
          a.prev[i] = x;
        }
        a.pos[i] = np_mod(xn, a.len[c]);
      }
    }
  }
}

size_t tracer_smem(const TracerArgs& a, int tpc, bool nyqx) {
  const size_t nmax = (size_t)std::max(a.n[0], std::max(a.n[1], a.n[2]));
  size_t b = 8 * nmax + 8 * (size_t)tpc * nmax + 8 * (size_t)tpc * (a.n[1] + a.n[2]) +
             4 * (size_t)tpc * a.n[0] * (nyqx ? 2 : 1) + 8;
  b += 8 + 8 * (size_t)TR_WARPS * tpc * 3;
  return b;
}

template <int TPC, bool NYQX, int MX>
cudaError_t launch_tracers_t(const TracerArgs& a, cudaStream_t s) {
  const size_t sm = tracer_smem(a, TPC, NYQX);
  cudaError_t e =
      cudaFuncSetAttribute(k_tracers<TPC, NYQX, MX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int blocks = (a.np + TPC - 1) / TPC;
  k_tracers<TPC, NYQX, MX><<<blocks, TR_THREADS, sm, s>>>(a);
  return cudaGetLastError();
}

template <int TPC, bool NYQX>
cudaError_t launch_tracers_mx(const TracerArgs& a, cudaStream_t s) {
  const int mx = (std::min(a.n[0], 256) + 31) / 32;  // points per lane and unit
  if (mx <= 1) return launch_tracers_t<TPC, NYQX, 1>(a, s);
  if (mx <= 2) return launch_tracers_t<TPC, NYQX, 2>(a, s);
  if (mx <= 4) return launch_tracers_t<TPC, NYQX, 4>(a, s);
  return launch_tracers_t<TPC, NYQX, 8>(a, s);
}

// 16 tracers per CTA (4 with the Nyquist term of x) when their tables fit in
// 200 KB of shared memory, else 4, else 1
cudaError_t launch_tracers(const TracerArgs& a, bool nyqx, cudaStream_t s) {
  if (a.np <= 0) return cudaSuccess;
  const size_t cap = 200 * 1024;
  if (!nyqx && tracer_smem(a, 16, false) <= cap) return launch_tracers_mx<16, false>(a, s);
  if (tracer_smem(a, 4, nyqx) <= cap)
    return nyqx ? launch_tracers_mx<4, true>(a, s) : launch_tracers_mx<4, false>(a, s);
  return nyqx ? launch_tracers_mx<1, true>(a, s) : launch_tracers_mx<1, false>(a, s);
}

int tracer_args(ps_plan p, TracerArgs& a) {
  if (p == nullptr) return errorf(PS_ERR_INVALID, "null plan");
  if (p->lgl) return errorf(PS_ERR_UNSUPPORTED, "point evaluation needs a Fourier grid (tracers.py:50-52)");
  a.nd = p->nd;
  for (int ax = 0; ax < 3; ++ax) {
    a.n[ax] = (ax < p->nd) ? p->n[ax] : 1;
    a.len[ax] = (ax < p->nd) ? p->desc.length[ax] : 1.0;
    a.P[ax] = (ax < p->nd) ? p->P[ax] : nullptr;
    if (a.n[ax] > TR_MAXN) return errorf(PS_ERR_UNSUPPORTED, "point evaluation supports up to %d points per axis", TR_MAXN);
  }
  a.cells = p->cells;
  return PS_OK;
}

// Exact interpolant or NUFFT: the plan's choice; automatic picks NUFFT once
// points x cells exceeds 2^24 (the exact sweep's cost) where the grid allows it
int tracer_route(ps_plan p, int np, bool* nu) {
  const bool ok = nufft_supported(p);
  if (p->tracer_method == PS_TRACERS_NUFFT && !ok)
    return errorf(PS_ERR_UNSUPPORTED, "NUFFT point evaluation needs Fourier axes of 2^a 3^b 5^c points up to 2048");
  *nu = (p->tracer_method == PS_TRACERS_NUFFT) ||
        (p->tracer_method == PS_TRACERS_AUTO && ok && (double)np * (double)p->cells > 16777216.0);
  return PS_OK;
}

}  // namespace
}  // namespace ps

extern "C" {

int ps_tracer_method(ps_plan p, int method) {
  if (p == nullptr) return ps::errorf(PS_ERR_INVALID, "null plan");
  if (method < PS_TRACERS_AUTO || method > PS_TRACERS_NUFFT)
    return ps::errorf(PS_ERR_INVALID, "method must be PS_TRACERS_AUTO, PS_TRACERS_EXACT or PS_TRACERS_NUFFT");
  if (method == PS_TRACERS_NUFFT && !ps::nufft_supported(p))
    return ps::errorf(PS_ERR_UNSUPPORTED, "NUFFT point evaluation needs Fourier axes of 2^a 3^b 5^c points up to 2048");
  p->tracer_method = method;
  return PS_OK;
}

int ps_eval_points(ps_plan p, const float* f, int nf, const double* points, int npoints, float* out, void* stream) {
  ps::TracerArgs a{};
  int rc = ps::tracer_args(p, a);
  if (rc != PS_OK) return rc;
  if (nf < 1 || nf > 3) return ps::errorf(PS_ERR_INVALID, "nf must be 1..3 (got %d)", nf);
  if (npoints < 0 || (npoints > 0 && (f == nullptr || points == nullptr || out == nullptr)))
    return ps::errorf(PS_ERR_INVALID, "null buffer or negative point count");
  bool nu = false;
  if ((rc = ps::tracer_route(p, npoints, &nu)) != PS_OK) return rc;
  if (nu)
    return ps::nufft_points(p, f, nf, false, const_cast<double*>(points), nullptr, npoints, 0, 0.0, out,
                            (cudaStream_t)stream);
  a.f = f;
  a.velocity = 0;
  a.nf = nf;
  a.np = npoints;
  a.pos = const_cast<double*>(points);
  a.out = out;
  const bool nyqx = (a.n[0] % 2 == 0) && !p->desc.dealias;
  cudaError_t e = ps::launch_tracers(a, nyqx, (cudaStream_t)stream);
  if (e != cudaSuccess) return ps::errorf(PS_ERR_CUDA, "point evaluation: %s", cudaGetErrorString(e));
  return PS_OK;
}

int ps_tracers_step(ps_plan p, const float* U, double* pos, double* prev, int npoints, int first, double dt,
                    float* velocity_out, void* stream) {
  ps::TracerArgs a{};
  int rc = ps::tracer_args(p, a);
  if (rc != PS_OK) return rc;
  if (npoints < 0 || (npoints > 0 && (U == nullptr || pos == nullptr || prev == nullptr)))
    return ps::errorf(PS_ERR_INVALID, "null buffer or negative tracer count");
  bool nu = false;
  if ((rc = ps::tracer_route(p, npoints, &nu)) != PS_OK) return rc;
  if (nu)
    return ps::nufft_points(p, U, p->nd, true, pos, prev, npoints, first, dt, velocity_out, (cudaStream_t)stream);
  a.f = U;
  a.velocity = 1;
  a.nf = p->nd;
  a.np = npoints;
  a.pos = pos;
  a.prev = prev;
  a.first = first ? 1 : 0;
  a.dt = dt;
  a.out = velocity_out;
  const bool nyqx = (a.n[0] % 2 == 0) && !p->desc.dealias;
  cudaError_t e = ps::launch_tracers(a, nyqx, (cudaStream_t)stream);
  if (e != cudaSuccess) return ps::errorf(PS_ERR_CUDA, "tracer step: %s", cudaGetErrorString(e));
  return PS_OK;
}

}  // extern "C"
