// Point evaluation of Fourier fields through type-2 non-uniform FFT
// interpolation: the method of the reference's finufft branch
// (phrike/grid.py:611, 1214, 1555 call finufft's nufft{1,2,3}d2 with
// eps = 1e-6), here with the published "exponential of semicircle" kernel of
// FINUFFT (Barnett, Magland, af Klinteberg 2019):
//     psi(x) = exp(beta (sqrt(1 - z^2) - 1)),  z = 2 x / (w h),  |z| < 1,
// on an oversampled grid of M = 2N points per axis (spacing h = L / M),
// w = 8 points of support per axis, beta = 2.30 w.
//
// The exact interpolant is f(x) = Re sum_k c_k F_k exp(i k.x), c_k / N the
// plan's projection table and F = FFT(f).  With the separable kernel,
//     f(x) = Re sum_m g_m psi(x - x_m),
//     g_m  = sum_k (c_k F_k h / (N psi_hat(k))) exp(i k.x_m),
// which is exact up to the aliasing of psi_hat beyond the retained band
// (about 3e-8 per axis at w = 8).  g is built by one resampling pass per
// axis (FFT of the N-point pencil, factor c_k h / (N psi_hat(k)), spectrum
// placed into the M-point pencil, inverse FFT), complex throughout so that
// an unpaired Nyquist mode (dealias off, even N) keeps the reference's real
// part at the end; psi_hat is integrated on the host in float64 by
// Gauss-Legendre quadrature.  The interpolation then sums w^d kernel
// weights per point.  Cost O(N^d log N + points w^d) instead of the exact
// interpolant's O(N^d points).
#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "mr_fft.cuh"
#include "plan.cuh"

namespace ps {
namespace {

using namespace mrfft;

constexpr int kNuW = 8;             // kernel support in fine-grid points per axis
constexpr double kNuBetaPerW = 2.30;
constexpr int kNuMaxN = kMrMaxLen / 2;

struct NuResampleArgs {
  const float* fin;   // first pass: real fields, or the state in velocity mode
  const float2* cin;  // later passes: complex fields
  float2* out;        // intermediate passes: complex pencils
  float* out_re;      // last pass: the real part only (what the interpolation keeps)
  int velocity;       // first pass: field c is U[1 + c] / U[0]
  long fs_in, fs_out; // elements per field
  long es;            // element stride along the pencil (the same in input and output)
  long npen;          // pencils per field
  int n, m;           // input and output pencil lengths (m = 2 n)
  MrAxis axn, axm;
  const float* s;     // per-mode factor c_k h / (N psi_hat(k)), fftfreq order, n entries
  int pg;             // pencils per CTA
};

__global__ void __launch_bounds__(kMrThreads, kMrMinBlocks) k_nufft_resample(NuResampleArgs a) {
  extern __shared__ __align__(16) float2 nu_sig[];
  __shared__ long pin[kMrMaxPencils], pout[kMrMaxPencils];
  const int field = blockIdx.y;
  const int n = a.n, m = a.m, pg = a.pg, pitch = m + 1;
  float2* twn = nu_sig + pg * pitch;
  float2* twm = twn + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) twn[i] = __ldg(a.axn.tw + i);
  for (int i = threadIdx.x; i < m; i += blockDim.x) twm[i] = __ldg(a.axm.tw + i);
  MrAxis axn = a.axn, axm = a.axm;
  axn.tw = twn;
  axm.tw = twm;
  const long j0 = (long)blockIdx.x * pg;
  for (int q = threadIdx.x; q < pg; q += blockDim.x) {
    const long j = j0 + q;
    const bool ok = j < a.npen;
    pin[q] = ok ? (j / a.es) * a.es * n + (j % a.es) : -1L;
    pout[q] = ok ? (j / a.es) * a.es * m + (j % a.es) : -1L;
  }
  __syncthreads();
  const bool rows = a.es == 1;
  {  // load the N-point pencils
    const int tot = pg * n;
    const float inv = 1.0f / (float)(rows ? n : pg);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      int q, i;
      if (rows) {
        q = qdiv(e, inv);
        i = e - q * n;
      } else {
        i = qdiv(e, inv);
        q = e - i * pg;
      }
      float2 v = make_float2(0.0f, 0.0f);
      if (pin[q] >= 0) {
        const long o = pin[q] + (long)i * a.es;
        if (a.cin != nullptr) {
          v = a.cin[field * a.fs_in + o];
        } else if (a.velocity) {
          v.x = a.fin[(1 + field) * a.fs_in + o] / a.fin[o];
        } else {
          v.x = a.fin[field * a.fs_in + o];
        }
      }
      nu_sig[q * pitch + i] = v;
    }
  }
  mr_fft(nu_sig, pitch, pg, axn, false);
  // scale, and move the negative modes k = q - n to m + q - n; then clear the
  // new band between them
  const int P = (n + 1) / 2;  // modes 0 .. P-1 are k >= 0 (fftfreq order)
  {
    const int tot = pg * n;
    const float inv = 1.0f / (float)n;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int q = qdiv(e, inv), k = e - q * n;
      float2* b = nu_sig + q * pitch;
      const float f = __ldg(a.s + k);
      const float2 v = b[k];
      b[(k < P) ? k : m - n + k] = make_float2(v.x * f, v.y * f);
    }
  }
  __syncthreads();
  {
    const int band = m - n;  // cleared entries P .. P + m - n - 1
    const int tot = pg * band;
    const float inv = 1.0f / (float)band;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int q = qdiv(e, inv), k = e - q * band;
      nu_sig[q * pitch + P + k] = make_float2(0.0f, 0.0f);
    }
  }
  mr_fft(nu_sig, pitch, pg, axm, true);
  {  // store the M-point pencils
    const int tot = pg * m;
    const float inv = 1.0f / (float)(rows ? m : pg);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      int q, i;
      if (rows) {
        q = qdiv(e, inv);
        i = e - q * m;
      } else {
        i = qdiv(e, inv);
        q = e - i * pg;
      }
      if (pout[q] < 0) continue;
      const long o = field * a.fs_out + pout[q] + (long)i * a.es;
      if (a.out_re != nullptr) a.out_re[o] = nu_sig[q * pitch + i].x;
      else a.out[o] = nu_sig[q * pitch + i];
    }
  }
}

struct NuInterpArgs {
  const float* g;   // [nf][Mz][My][Mx], real part of the oversampled grid
  long fs;
  int nd, nf;
  int m[3];
  double len[3];
  float beta;
  int np;
  double* pos;   // [nd][np]
  double* prev;  // advection mode (leap-frog) or null
  int first;
  double dt;
  float* out;    // [nf][np] or null
};

__device__ __forceinline__ float es_kernel(float z, float beta) {
  const float t = fmaf(-z, z, 1.0f);
  return (t > 0.0f) ? expf(beta * (sqrtf(t) - 1.0f)) : 0.0f;
}

// numpy's float mod for b > 0: result in [0, b)
__device__ __forceinline__ double nu_mod(double a, double b) {
  double r = fmod(a, b);
  if (r < 0.0) r += b;
  if (r == 0.0) r = 0.0;
  return r;
}

template <int ND>
__global__ void __launch_bounds__(256) k_nufft_interp(NuInterpArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.np) return;
  float wt[3][kNuW];
  int ix[3][kNuW];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int i = 0; i < kNuW; ++i) {
      wt[d][i] = 1.0f;
      ix[d][i] = 0;
    }
    if (d >= ND) continue;
    const int M = a.m[d];
    const double t = a.pos[(long)d * a.np + p] * ((double)M / a.len[d]);  // fine-grid coordinate
    const double m0 = ceil(t - 0.5 * kNuW);
    long b = (long)m0 % M;
    if (b < 0) b += M;
#pragma unroll
    for (int i = 0; i < kNuW; ++i) {
      const float z = (float)((t - (m0 + i)) * (2.0 / kNuW));
      wt[d][i] = es_kernel(z, a.beta);
      long id = b + i;
      if (id >= M) id -= M;
      ix[d][i] = (int)id;
    }
  }
  for (int c = 0; c < a.nf; ++c) {
    const float* gc = a.g + (long)c * a.fs;
    float re = 0.0f;
#pragma unroll 1
    for (int iz = 0; iz < (ND == 3 ? kNuW : 1); ++iz) {
      // wt[2] / ix[2] entries selected without dynamic register indexing
      float wz = 1.0f;
      int jz = 0;
#pragma unroll
      for (int i = 0; i < kNuW; ++i)
        if (i == iz) {
          wz = wt[2][i];
          jz = ix[2][i];
        }
#pragma unroll
      for (int iy = 0; iy < (ND >= 2 ? kNuW : 1); ++iy) {
        const long row = ((long)jz * a.m[1] + ix[1][iy]) * a.m[0];
        float rr = 0.0f;
#pragma unroll
        for (int i = 0; i < kNuW; ++i) rr = fmaf(__ldg(gc + row + ix[0][i]), wt[0][i], rr);
        re = fmaf(rr, wz * wt[1][iy], re);
      }
    }
    // the real part, as the reference keeps
    if (a.out != nullptr) a.out[(long)c * a.np + p] = re;
    if (a.prev != nullptr) {  // leap-frog (tracers.py:50-79, 103-148, 178-236)
      const long i = (long)c * a.np + p;
      const double x = a.pos[i];
      double xn;
      if (a.first) {
        a.prev[i] = x;
        xn = x + a.dt * re;
      } else {
        xn = a.prev[i] + 2.0 * a.dt * re;
        a.prev[i] = x;
      }
      a.pos[i] = nu_mod(xn, a.len[c]);
    }
  }
}

int nfail(cudaError_t e, const char* what) { return errorf(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); }

#define NU_CU(expr, what)                          \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return nfail(_e, what); \
  } while (0)

// Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on P_n)
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-15) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// psi_hat(k) = int psi(x) exp(-i k x) dx = a int_{-1}^{1} es(t) cos(k a t) dt, a = w h / 2
double es_hat(double k, double a, double beta, const std::vector<double>& gx, const std::vector<double>& gw) {
  double s = 0.0;
  for (size_t i = 0; i < gx.size(); ++i) {
    const double t = gx[i];
    s += gw[i] * exp(beta * (sqrt(1.0 - t * t) - 1.0)) * cos(k * a * t);
  }
  return a * s;
}

MrAxis axis_tables(ps_plan p, int n, float2** tw, int* rc) {
  MrAxis ax{};
  int radix[kMrMaxStages];
  if (!mr_factor(n, radix, &ax.nst)) {
    *rc = errorf(PS_ERR_UNSUPPORTED, "NUFFT: length %d is not 5-smooth", n);
    return ax;
  }
  ax.n = n;
  for (int s = 0; s < ax.nst; ++s) ax.rcode |= (unsigned long long)radix[s] << (4 * s);
  ax.ntp = (n + kMrDiv - 1) / kMrDiv;
  std::vector<float2> h(n);
  for (int k = 0; k < n; ++k) {
    const double ang = -2.0 * M_PI * (double)k / n;
    h[k] = make_float2((float)cos(ang), (float)sin(ang));
  }
  if ((*rc = plan_alloc(p, tw, n)) != PS_OK) return ax;
  cudaError_t e = cudaMemcpy(*tw, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    *rc = nfail(e, "NUFFT tables");
    return ax;
  }
  ax.tw = *tw;
  *rc = PS_OK;
  return ax;
}

}  // namespace

bool nufft_supported(const ps_plan_s* p) {
  if (p->lgl) return false;
  for (int a = 0; a < p->nd; ++a)
    if (p->n[a] > kNuMaxN || !mr_axis_ok(p->n[a]) || !mr_axis_ok(2 * p->n[a])) return false;
  return true;
}

// Tables (lazily, on first use): per axis the FFT tables of N and 2N points
// and the factor c_k h / (N psi_hat(k)); three fields of the oversampled
// grid plus two intermediate buffers.
int nufft_setup(ps_plan p) {
  if (p->nu_ready) return PS_OK;
  if (!nufft_supported(p))
    return errorf(PS_ERR_UNSUPPORTED, "NUFFT interpolation needs Fourier axes of 2^a 3^b 5^c points up to %d", kNuMaxN);
  int rc;
  std::vector<double> gx, gw;
  gauss_legendre(100, gx, gw);
  const double beta = kNuBetaPerW * kNuW;
  for (int a = 0; a < p->nd; ++a) {
    const int N = p->n[a], M = 2 * N;
    float2* tw = nullptr;
    p->nu_axn[a] = axis_tables(p, N, &tw, &rc);
    if (rc != PS_OK) return rc;
    p->nu_axm[a] = axis_tables(p, M, &tw, &rc);
    if (rc != PS_OK) return rc;
    if (2 * p->nu_axm[a].ntp > kMrThreads) return errorf(PS_ERR_UNSUPPORTED, "NUFFT: axis %d too long", a);
    std::vector<float> P(N);
    NU_CU(cudaMemcpy(P.data(), p->P[a], sizeof(float) * N, cudaMemcpyDeviceToHost), "NUFFT tables");
    const double L = p->desc.length[a], h = L / M, half = 0.5 * kNuW * h;
    std::vector<float> s(N);
    for (int q = 0; q < N; ++q) {
      const int kq = (2 * q <= N - 1) ? q : q - N;
      const double k = 2.0 * M_PI * kq / L;
      s[q] = (float)((double)P[q] * h / es_hat(k, half, beta, gx, gw));
    }
    if ((rc = plan_alloc(p, &p->nu_s[a], N)) != PS_OK) return rc;
    NU_CU(cudaMemcpy(p->nu_s[a], s.data(), sizeof(float) * N, cudaMemcpyHostToDevice), "NUFFT tables");
  }
  const long fine = (1L << p->nd) * p->cells;  // every axis resampled
  const long t1 = 2L * p->cells;               // x resampled
  const long t2 = 4L * p->cells;               // x and y resampled (3D)
  if ((rc = plan_alloc(p, &p->nu_g, (size_t)3 * fine)) != PS_OK) return rc;
  if (p->nd >= 2 && (rc = plan_alloc(p, &p->nu_t1, (size_t)3 * t1)) != PS_OK) return rc;
  if (p->nd == 3 && (rc = plan_alloc(p, &p->nu_t2, (size_t)3 * t2)) != PS_OK) return rc;
  p->nu_ready = true;
  return PS_OK;
}

// f (nf real fields, or the velocity of the state U) at np points; with prev
// given, the leap-frog advection of the points (one solve: the first of a batch)
int nufft_points(ps_plan p, const float* f, int nf, bool velocity, double* pos, double* prev, int np, int first,
                 double dt, float* out, cudaStream_t s) {
  int rc;
  if ((rc = nufft_setup(p)) != PS_OK) return rc;
  if (np <= 0) return PS_OK;
  int ext[3] = {p->n[0], p->nd > 1 ? p->n[1] : 1, p->nd > 2 ? p->n[2] : 1};
  const float2* cin = nullptr;
  const float* fin = f;
  for (int a = 0; a < p->nd; ++a) {
    NuResampleArgs r{};
    long fs_in = (long)ext[0] * ext[1] * ext[2];
    long es = 1;
    for (int b = 0; b < a; ++b) es *= ext[b];
    const int N = p->n[a], M = 2 * N;
    r.fin = fin;
    r.cin = cin;
    r.velocity = (a == 0 && velocity) ? 1 : 0;
    r.fs_in = fs_in;
    r.npen = fs_in / N;
    ext[a] = M;
    r.fs_out = (long)ext[0] * ext[1] * ext[2];
    r.es = es;
    r.n = N;
    r.m = M;
    r.axn = p->nu_axn[a];
    r.axm = p->nu_axm[a];
    r.s = p->nu_s[a];
    const bool last = a == p->nd - 1;
    float2* dst = last ? nullptr : (a == 0) ? p->nu_t1 : p->nu_t2;
    r.out = dst;
    r.out_re = last ? p->nu_g : nullptr;
    const int per = (M + 1) * (int)sizeof(float2);
    int pg = kMrThreads / (2 * r.axm.ntp);
    if (pg < 1) pg = 1;
    if (pg > kMrMaxPencils) pg = kMrMaxPencils;
    while (pg > 1 && pg * per + (N + M) * (int)sizeof(float2) > 100 * 1024) --pg;
    if (pg > r.npen) pg = (int)r.npen;
    r.pg = pg;
    const int threads = (pg * r.axm.ntp + 31) / 32 * 32;
    const int smem = pg * per + (N + M) * (int)sizeof(float2);
    if (smem > 48 * 1024)
      NU_CU(cudaFuncSetAttribute(k_nufft_resample, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
            "NUFFT resample attribute");
    const dim3 grid((unsigned)((r.npen + pg - 1) / pg), (unsigned)nf);
    ProfScope prof(p, s, PS_KIND_OP, 4.0 * nf * (fs_in * (a == 0 ? 1 : 2) + 2 * r.fs_out));
    k_nufft_resample<<<grid, threads, smem, s>>>(r);
    NU_CU(cudaGetLastError(), "NUFFT resample");
    cin = dst;
    fin = nullptr;
  }
  NuInterpArgs ia{};
  ia.g = p->nu_g;
  ia.fs = (long)ext[0] * ext[1] * ext[2];
  ia.nd = p->nd;
  ia.nf = nf;
  for (int a = 0; a < 3; ++a) {
    ia.m[a] = ext[a];
    ia.len[a] = (a < p->nd) ? p->desc.length[a] : 1.0;
  }
  ia.beta = (float)(kNuBetaPerW * kNuW);
  ia.np = np;
  ia.pos = pos;
  ia.prev = prev;
  ia.first = first;
  ia.dt = dt;
  ia.out = out;
  const int blocks = (np + 255) / 256;
  if (p->nd == 1) k_nufft_interp<1><<<blocks, 256, 0, s>>>(ia);
  else if (p->nd == 2) k_nufft_interp<2><<<blocks, 256, 0, s>>>(ia);
  else k_nufft_interp<3><<<blocks, 256, 0, s>>>(ia);
  NU_CU(cudaGetLastError(), "NUFFT interpolation");
  return PS_OK;
}

}  // namespace ps
