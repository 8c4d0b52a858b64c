// Adaptive embedded Runge-Kutta: tableaux, controller and the cell-wise
// kernels of one attempt (the reference's adaptive.py:23-437 with the run
// loops of solver.py:338-422, 706-800, 1095-1160, 1395-1513).
//
// One attempt of a batch is a fixed launch sequence: begin (per-solve dt and
// live flags), scale (max |U|), for every stage a combination kernel and the
// plan's right-hand-side passes, final (U_high and the error), decide (the
// controller), then the solver's post-step operator on the accepted solves.
// Every decision stays on the device, so attempt loops need no host round
// trip and can be captured in CUDA graphs.
#include <cuda_runtime.h>

#include "adaptive.cuh"
#include "mhd_passes.cuh"
#include "pass_common.cuh"

namespace ps {

int ark_tableau(int method, ArkTableau* tab) {
  *tab = ArkTableau{};
  auto set_row = [&](int i, std::initializer_list<double> r) {
    int j = 0;
    for (double v : r) tab->a[i][j++] = v;
  };
  auto set_vec = [](double* d, std::initializer_list<double> r) {
    int j = 0;
    for (double v : r) d[j++] = v;
  };
  switch (method) {
    case 0:  // Bogacki-Shampine 3(2) (adaptive.py:136-187)
      tab->stages = 4;
      tab->order = 2;
      set_row(1, {1.0 / 2.0});
      set_row(2, {0.0, 3.0 / 4.0});
      set_row(3, {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0});
      set_vec(tab->bh, {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0, 0.0});
      set_vec(tab->bl, {7.0 / 24.0, 1.0 / 4.0, 1.0 / 3.0, 1.0 / 8.0});
      return 0;
    case 1:  // Dormand-Prince 5(4) (adaptive.py:190-238)
      tab->stages = 7;
      tab->order = 4;
      set_row(1, {1.0 / 5.0});
      set_row(2, {3.0 / 40.0, 9.0 / 40.0});
      set_row(3, {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0});
      set_row(4, {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0});
      set_row(5, {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0});
      set_row(6, {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0});
      set_vec(tab->bh, {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0.0});
      set_vec(tab->bl, {5179.0 / 57600.0, 0.0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                        187.0 / 2100.0, 1.0 / 40.0});
      return 0;
    case 2:  // the reference's simplified 8-stage "rk78" table (adaptive.py:241-292)
      tab->stages = 8;
      tab->order = 7;
      set_row(1, {1.0 / 6.0});
      set_row(2, {1.0 / 12.0, 1.0 / 4.0});
      set_row(3, {1.0 / 8.0, 0.0, 3.0 / 8.0});
      set_row(4, {13.0 / 72.0, 0.0, 0.0, 11.0 / 72.0});
      set_row(5, {5.0 / 24.0, 0.0, 0.0, 0.0, 5.0 / 24.0});
      set_row(6, {1.0 / 20.0, 0.0, 0.0, 0.0, 0.0, 1.0 / 20.0});
      set_row(7, {1.0 / 8.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0 / 8.0});
      set_vec(tab->bh, {1.0 / 8.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0 / 8.0, 0.0});
      set_vec(tab->bl, {1.0 / 9.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0 / 9.0, 1.0 / 9.0});
      return 0;
    default:
      return -1;
  }
}

namespace {

// run loop condition (solver.py:384) plus the optional output pause
__device__ __forceinline__ bool ark_on(double t, double tend, const double* tout, int s) {
  return t < tend - 1e-12 && (tout == nullptr || t + 1e-12 < tout[s]);
}

__global__ void k_ark_begin(ArkState st) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st.nsolve) return;
  const double t = st.t[s], te = st.tend[s];
  const bool on = ark_on(t, te, st.tout, s);
  st.live[s] = on ? 1 : 0;
  st.ok[s] = 0;
  st.err[s] = 0.0f;
  st.scale[s] = 0.0f;
  st.dt[s] = on ? fmin(st.dtp[s], te - t) : 0.0;  // dt = min(dt, t_end - t)
}

__global__ void k_ark_scale(const float* __restrict__ U, long n, long ss, long cells, int ecomp,
                            const float* eref, ArkState st) {
  __shared__ float red[32];
  const int sol = blockIdx.y;
  if (!st.live[sol]) return;
  U += (long)sol * ss;
  const float er = (eref != nullptr) ? eref[sol] : 0.0f;
  const long e0 = (long)ecomp * cells, e1 = e0 + cells;
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float v = U[i];
    if (i >= e0 && i < e1) v += er;
    m = fmaxf(m, fabsf(v));
  }
  m = block_max(m, red);
  if (threadIdx.x == 0) atomic_max_nonneg(st.scale + sol, m);
}

// float4 over n elements per solve (n and ss are multiples of 4)
__global__ void k_ark_stage(const float* __restrict__ U, const float* __restrict__ K, long kstride,
                            float* __restrict__ out, long n, long ss, ArkComb cmb, ArkState st) {
  const int sol = blockIdx.y;
  if (!st.live[sol]) return;
  const double dt = st.dt[sol];
  float c[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) c[j] = (j < cmb.m) ? (float)(dt * cmb.c[j]) : 0.0f;
  const long base = (long)sol * ss;
  const long n4 = n / 4;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    float4 v = reinterpret_cast<const float4*>(U + base)[i];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (j < cmb.m) {
        const float4 k = reinterpret_cast<const float4*>(K + cmb.idx[j] * kstride + base)[i];
        v.x = fmaf(c[j], k.x, v.x);
        v.y = fmaf(c[j], k.y, v.y);
        v.z = fmaf(c[j], k.z, v.z);
        v.w = fmaf(c[j], k.w, v.w);
      }
    }
    reinterpret_cast<float4*>(out + base)[i] = v;
  }
}

// high and diff share the index list (the union of nonzero high / diff weights)
__global__ void k_ark_final(const float* __restrict__ U, const float* __restrict__ K, long kstride,
                            float* __restrict__ W, long n, long ss, ArkComb high, ArkComb diff, ArkState st) {
  __shared__ float red[32];
  const int sol = blockIdx.y;
  if (!st.live[sol]) return;
  const double dt = st.dt[sol];
  float ch[8], ce[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    ch[j] = (j < high.m) ? (float)(dt * high.c[j]) : 0.0f;
    ce[j] = (j < high.m) ? (float)(dt * diff.c[j]) : 0.0f;
  }
  const long base = (long)sol * ss;
  const long n4 = n / 4;
  float em = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    float4 v = reinterpret_cast<const float4*>(U + base)[i];
    float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (j < high.m) {
        const float4 k = reinterpret_cast<const float4*>(K + high.idx[j] * kstride + base)[i];
        v.x = fmaf(ch[j], k.x, v.x);
        v.y = fmaf(ch[j], k.y, v.y);
        v.z = fmaf(ch[j], k.z, v.z);
        v.w = fmaf(ch[j], k.w, v.w);
        e.x = fmaf(ce[j], k.x, e.x);
        e.y = fmaf(ce[j], k.y, e.y);
        e.z = fmaf(ce[j], k.z, e.z);
        e.w = fmaf(ce[j], k.w, e.w);
      }
    }
    reinterpret_cast<float4*>(W + base)[i] = v;
    em = fmaxf(em, fmaxf(fmaxf(fabsf(e.x), fabsf(e.y)), fmaxf(fabsf(e.z), fabsf(e.w))));
  }
  em = block_max(em, red);
  if (threadIdx.x == 0) atomic_max_nonneg(st.err + sol, em);
}

__global__ void k_ark_decide(ArkState st, int order, ArkCtrl c) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st.nsolve || !st.live[s]) return;
  const double dt = st.dt[s];
  const double err = (double)st.err[s];
  const double tol = c.atol + c.rtol * (double)st.scale[s];
  bool accept = err <= tol;
  double dt_new;
  if (err > 0.0) {
    const double dt_opt = dt * pow(tol / err, 1.0 / (double)order) * c.safety;
    dt_new = dt * fmin(fmax(dt_opt / dt, c.minf), c.maxf);
  } else {
    dt_new = dt * c.maxf;
  }
  int r = st.rej[s];
  if (!accept) {
    r += 1;
    if (r >= c.max_rej) {  // forced acceptance after max_rejections in a row
      r = 0;
      accept = true;
    }
  } else {
    r = 0;
  }
  st.rej[s] = r;
  st.ok[s] = accept ? 1 : 0;
  if (accept) st.t[s] += dt;
  if (st.counts != nullptr) st.counts[2 * s + (accept ? 0 : 1)] += 1;
  st.dtp[s] = dt_new;
}

__global__ void k_ark_clamp_mhd(float* U, long cells, long ss, float gamma, float rho_min, float p_min,
                                const int* mask) {
  const int sol = blockIdx.y;
  if (mask != nullptr && !mask[sol]) return;
  U += (long)sol * ss;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cells; i += (long)gridDim.x * blockDim.x) {
    float u[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) u[c] = U[c * cells + i];
    clamp_mhd(u, gamma, rho_min, p_min);
#pragma unroll
    for (int c = 0; c < 8; ++c) U[c * cells + i] = u[c];
  }
}

int blocks_for(long n, int nsolve) {
  const long per = (2 * 1216 + nsolve - 1) / nsolve;  // about 16 blocks of 256 per SM in total
  const long want = (n + 255) / 256;
  long b = want < per ? want : per;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_ark_begin(const ArkState& st, cudaStream_t s) {
  k_ark_begin<<<(st.nsolve + 127) / 128, 128, 0, s>>>(st);
  return cudaGetLastError();
}

cudaError_t launch_ark_scale(const float* U, long n, long ss, long cells, int ecomp, const float* eref,
                             const ArkState& st, cudaStream_t s) {
  k_ark_scale<<<dim3(blocks_for(n, st.nsolve), st.nsolve), 256, 0, s>>>(U, n, ss, cells, ecomp, eref, st);
  return cudaGetLastError();
}

cudaError_t launch_ark_stage(const float* U, const float* K, long kstride, float* out, long n, long ss,
                             const ArkComb& cmb, const ArkState& st, cudaStream_t s) {
  k_ark_stage<<<dim3(blocks_for(n / 4, st.nsolve), st.nsolve), 256, 0, s>>>(U, K, kstride, out, n, ss, cmb, st);
  return cudaGetLastError();
}

cudaError_t launch_ark_final(const float* U, const float* K, long kstride, float* W, long n, long ss,
                             const ArkComb& high, const ArkComb& diff, const ArkState& st, cudaStream_t s) {
  k_ark_final<<<dim3(blocks_for(n / 4, st.nsolve), st.nsolve), 256, 0, s>>>(U, K, kstride, W, n, ss, high, diff,
                                                                            st);
  return cudaGetLastError();
}

cudaError_t launch_ark_decide(const ArkState& st, int order, const ArkCtrl& ctrl, cudaStream_t s) {
  k_ark_decide<<<(st.nsolve + 127) / 128, 128, 0, s>>>(st, order, ctrl);
  return cudaGetLastError();
}

cudaError_t launch_ark_clamp_mhd(float* U, long cells, long ss, int nsolve, float gamma, float rho_min,
                                 float p_min, const int* mask, cudaStream_t s) {
  k_ark_clamp_mhd<<<dim3(blocks_for(cells, nsolve), nsolve), 256, 0, s>>>(U, cells, ss, gamma, rho_min, p_min,
                                                                          mask);
  return cudaGetLastError();
}

}  // namespace ps
