// 1D Legendre-Gauss-Lobatto (LGL) collocation: whole RK steps of the Euler
// equations in one launch, one CTA per solve (one thread per node up to 1024) (SpectralSolver1D on a Grid1D
// with basis "legendre": solver.py:62-132, 259-269; grid.py:276-300,
// 620-735; basis/legendre.py:681-859).
//
// Per stage: the boundary conditions in place on the stage input (codes per
// boundary and variable: copy the neighbouring interior value, set to zero,
// or leave), the flux in shared memory, k = -D F with the differentiation
// matrix read column by column from L2 (D^T, coalesced across the CTA's
// threads), constant gravity, the RK update and the 1D positivity clamp.
// After the step: the nodal filter (if enabled) with the boundary conditions,
// inside the step and again at the filter cadence.  The energy slot holds
// E' = E - E_ref (the energy of the first node), an exact rewrite that keeps
// float32 rounding relative to the field's variation.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "lgl1d.cuh"
#include "pass_common.cuh"

namespace ps {

namespace {

__device__ __forceinline__ void bc_apply(float* u, int N, const int* codes, int i) {
  // codes[side * 3 + var]; thread i handles (side, var) = (i / 3, i % 3)
  if (i >= 6) return;
  const int side = i / 3, var = i % 3;
  const int c = codes[i];
  const int dst = side == 0 ? 0 : N - 1, src = side == 0 ? 1 : N - 2;
  if (c == 0) u[var * N + dst] = u[var * N + src];
  else if (c == 1) u[var * N + dst] = 0.0f;
}

// the three flux (or state) values of one node, one vector load per node
template <typename REAL>
struct alignas(4 * sizeof(REAL)) Node4 {
  REAL v0, v1, v2, pad;
};

template <typename REAL>
__global__ void __launch_bounds__(1024) k_lgl1d(Lgl1DArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int N = a.n;
  const int sol = blockIdx.x;
  if (a.active != nullptr && !a.active[sol]) return;
  Node4<REAL>* F = reinterpret_cast<Node4<REAL>*>(smem_raw);  // [N] nodes x (3 + pad)
  float* us = reinterpret_cast<float*>(F + N);           // [3][N]
  float* un = us + 3 * N;                                 // [3][N]
  float* acc = un + 3 * N;                                // [3][N]
  __shared__ float red[32];
  __shared__ int codes[6];
  const REAL* DT = static_cast<const REAL*>(a.DT);
  const REAL* FT = static_cast<const REAL*>(a.FT);
  float* U = a.U + (long)sol * a.solve_stride;
  if (threadIdx.x < 6) codes[threadIdx.x] = a.bc.c[threadIdx.x];
  const float er = U[2 * N];
  for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) {
    float v = U[i];
    if (i >= 2 * N) v -= er;
    un[i] = v;
    us[i] = v;
  }
  __syncthreads();
  const float g1 = a.gamma - 1.0f;
  const float href = a.gamma * er;
  const float pmin_shift = a.p_min - g1 * er;

  // k = -D F(us) (+ gravity) for the node i, after flux() and a barrier
  auto flux = [&]() {
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      const float rho = us[j], m = us[N + j], E = us[2 * N + j];
      const float u = m / rho;
      const float p = g1 * (E - 0.5f * rho * u * u);  // p' (E holds E')
      F[j] = Node4<REAL>{(REAL)m, (REAL)(m * u + p), (REAL)(((E + p) + href) * u), (REAL)0};
    }
  };
  // (D F)_i = sum_j D_ij (F_j - F_i): D annihilates constants, and the large
  // entries of D (near the diagonal at the ends, O(N^2)) then multiply small
  // differences, so the rounding of D and F stays relative to F's variation
  auto deriv = [&](int i, float (&k)[3]) {
    REAL s0 = 0, s1 = 0, s2 = 0;
    const Node4<REAL> fi = F[i];
#pragma unroll 4
    for (int j = 0; j < N; ++j) {
      const REAL d = DT[(long)j * N + i];
      const Node4<REAL> fj = F[j];
      s0 += d * (fj.v0 - fi.v0);
      s1 += d * (fj.v1 - fi.v1);
      s2 += d * (fj.v2 - fi.v2);
    }
    k[0] = -(float)s0;
    k[1] = -(float)s1;
    k[2] = -(float)s2;
    if (a.gx != 0.0f) {  // gravity source (solver.py:82-91)
      const float rho = us[i], u = us[N + i] / rho;
      k[1] += rho * a.gx;
      k[2] += rho * a.gx * u;
    }
  };
  // nodal filter of us (if enabled) and the boundary conditions; the filter
  // keeps constants (rows sum to 1), so it is summed as
  // u_i + sum_j F_ij (u_j - u_i) with rounding relative to the variation
  auto filter_bc = [&]() {
    if (FT != nullptr) {
      for (int i = threadIdx.x; i < N; i += blockDim.x)
        F[i] = Node4<REAL>{(REAL)us[i], (REAL)us[N + i], (REAL)us[2 * N + i], (REAL)0};
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        REAL s0 = 0, s1 = 0, s2 = 0;
        const Node4<REAL> fi = F[i];
#pragma unroll 4
        for (int j = 0; j < N; ++j) {
          const REAL f = FT[(long)j * N + i];
          const Node4<REAL> fj = F[j];
          s0 += f * (fj.v0 - fi.v0);
          s1 += f * (fj.v1 - fi.v1);
          s2 += f * (fj.v2 - fi.v2);
        }
        us[i] = (float)(fi.v0 + s0);
        us[N + i] = (float)(fi.v1 + s1);
        us[2 * N + i] = (float)(fi.v2 + s2);
      }
      __syncthreads();
    }
    bc_apply(us, N, codes, threadIdx.x);
    __syncthreads();
  };

  if (a.rhs_out != nullptr) {  // rhs only (the boundary conditions act on the copy in shared memory)
    bc_apply(us, N, codes, threadIdx.x);
    __syncthreads();
    flux();
    __syncthreads();
    float* R = a.rhs_out + (long)sol * a.solve_stride;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      float k[3];
      deriv(i, k);
      R[i] = k[0];
      R[N + i] = k[1];
      R[2 * N + i] = k[2];
    }
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
    if (a.t != nullptr) {  // CFL step size from the state as given (solver.py:235-240)
      if (tl >= te - 1e-12) break;
      float sm = 0.0f;
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float rho = un[i], u = un[N + i] / rho;
        const float pp = g1 * (un[2 * N + i] - 0.5f * rho * u * u) + g1 * er;
        sm = fmaxf(sm, fabsf(u) + sqrtf(a.gamma * pp / rho));
      }
      sm = block_max(sm, red);
      if (threadIdx.x == 0) red[0] = sm;
      __syncthreads();
      const double spd = (double)red[0];
      __syncthreads();
      dtd = (spd <= 0.0) ? 1e-6 : (double)a.cfl * (double)a.hmin / spd;
      dtd = fmin(dtd, te - tl);
      dt = (float)dtd;
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      if (a.rk2 && (stage == 1 || stage == 2)) continue;
      const RKCoef rc = rk_coef(stage, dt, a.rk2);
      // the boundary conditions act on the stage input (and so on U^n at stage 0)
      bc_apply(us, N, codes, threadIdx.x);
      __syncthreads();
      if (stage == 0) {
        for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) un[i] = us[i];
        __syncthreads();
      }
      flux();
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        float k[3];
        deriv(i, k);
        float u3[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int s = c * N + i;
          u3[c] = rk_update_incr(stage, rc, k[c], un[s], acc[s]);
        }
        clamp_state<1>(u3, a.gamma, a.rho_min, pmin_shift);
        us[i] = u3[0];
        us[N + i] = u3[1];
        us[2 * N + i] = u3[2];
      }
      __syncthreads();
    }
    filter_bc();  // inside the step (_rk4_step -> _apply_physical_filters)
    if (((cad0 + step) % a.filter_interval) == 0) filter_bc();  // cadence
    for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) un[i] = us[i];
    __syncthreads();
    tl += dtd;
    ++taken;
  }
  if (threadIdx.x == 0) {
    if (a.t != nullptr) a.t[sol] = tl;
    if (a.steps_done != nullptr) a.steps_done[sol] += taken;
  }
  for (int i = threadIdx.x; i < 3 * N; i += blockDim.x) U[i] = un[i] + (i >= 2 * N ? er : 0.0f);
}

// out[f][i] = sum_j M[i][j] in[f][j] for nf fields per solve (MT = M^T),
// summed as sum_j M[i][j] (in[f][j] - in[f][i]) + c in[f][i] with c the row
// sum of M (0 for D, 1 for the filter) so rounding follows the variation
template <typename REAL>
__global__ void k_lgl1d_apply(const REAL* MT, const float* in, float* out, int n, int nf, long ss, float rowsum) {
  const int f = blockIdx.y % nf, sol = blockIdx.y / nf;
  const float* x = in + (long)sol * ss + (long)f * n;
  float* y = out + (long)sol * ss + (long)f * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const REAL xi = (REAL)x[i];
    REAL s = 0;
    for (int j = 0; j < n; ++j) s += MT[(long)j * n + i] * ((REAL)x[j] - xi);
    y[i] = (float)(s + (REAL)rowsum * xi);
  }
}

template <typename REAL>
__global__ void k_transpose(const REAL* in, REAL* out, int n) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x) {
    const long i = e / n, j = e % n;
    out[j * n + i] = in[e];
  }
}

__global__ void k_lgl1d_bc(float* U, int n, long ss, Bc1D bc, const int* active) {
  if (active != nullptr && !active[blockIdx.x]) return;
  bc_apply(U + (long)blockIdx.x * ss, n, bc.c, threadIdx.x);
}

// ---------------------------------------------------------------------------
// Cluster form for 130..513 nodes (float32 contractions): a cluster of C CTAs
// per solve, CTA r owning rows [r R, r R + R) of D (R = ceil(n / C) <= 65)
// in its shared memory, so a stage reads no matrix from L2.  Every CTA keeps
// the whole stage state and computes the flux of every node (cheap); it
// evaluates k = -D F for its rows (one warp per row, lanes along the
// columns), updates those rows, and writes them into every CTA's copy of the
// state through distributed shared memory between two cluster barriers.
// The boundary conditions, the CFL speed and the time loop are evaluated
// identically in every CTA from identical data.  Same algorithm as k_lgl1d;
// the column sums are split across lanes, so the two forms agree to float32
// rounding rather than bit for bit (plans pick the form from n alone, so a
// solve gives the same bits alone and in a batch).
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;
constexpr int CL_THREADS = 256;
constexpr int CL_WARPS = CL_THREADS / 32;
constexpr int CL_ROWS = 65;

__host__ __device__ constexpr int cl_dl_floats(int n, int C) { return ((((n + C - 1) / C) * n + 3) / 4) * 4; }

template <int C>
__global__ void __launch_bounds__(CL_THREADS) k_lgl1d_cl(Lgl1DArgs a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int sol = blockIdx.x / C;
  if (a.active != nullptr && !a.active[sol]) return;  // the same for every CTA of the cluster
  const int N = a.n;
  const int R = (N + C - 1) / C;
  const int i0 = rank * R, nr = max(0, min(N, i0 + R) - i0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* Dl = reinterpret_cast<float*>(smem_raw);                          // [R][N] rows of D
  Node4<float>* F = reinterpret_cast<Node4<float>*>(Dl + cl_dl_floats(N, C));  // [N]
  float* us = reinterpret_cast<float*>(F + N);                             // [3][N] stage state
  float* un = us + 3 * N;                                                  // [3][N] U^n
  float* acc = un + 3 * N;                                                 // [3][R] own rows
  float* mine = acc + 3 * R;                                               // [3][R] own new rows
  float* kb = mine + 3 * R;                                                // [3][R] own k
  __shared__ float red[32];
  __shared__ int codes[6];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float* DT = static_cast<const float*>(a.DT);
  const float* FT = static_cast<const float*>(a.FT);
  float* U = a.U + (long)sol * a.solve_stride;
  if (tid < 6) codes[tid] = a.bc.c[tid];
  for (int idx = tid; idx < R * N; idx += CL_THREADS) {  // Dl[r][j] = D[i0 + r][j] = DT[j][i0 + r]
    const int j = idx / R, r = idx - j * R;
    Dl[r * N + j] = (r < nr) ? DT[(long)j * N + i0 + r] : 0.0f;
  }
  const float er = U[2 * N];
  for (int i = tid; i < 3 * N; i += CL_THREADS) {
    float v = U[i];
    if (i >= 2 * N) v -= er;
    un[i] = v;
    us[i] = v;
  }
  cluster.sync();  // every CTA has read the state before any CTA writes its rows back
  const float g1 = a.gamma - 1.0f;
  const float href = a.gamma * er;
  const float pmin_shift = a.p_min - g1 * er;

  auto flux = [&]() {
    for (int j = tid; j < N; j += CL_THREADS) {
      const float rho = us[j], m = us[N + j], E = us[2 * N + j];
      const float u = m / rho;
      const float p = g1 * (E - 0.5f * rho * u * u);
      F[j] = Node4<float>{m, m * u + p, ((E + p) + href) * u, 0.0f};
    }
  };
  // kb = -(D F)_i (+ gravity) for the own rows, summed as D_ij (F_j - F_i)
  auto own_rhs = [&]() {
    for (int r = warp; r < nr; r += CL_WARPS) {
      const int i = i0 + r;
      const Node4<float> fi = F[i];
      float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
      const float* drow = Dl + r * N;
      for (int j = lane; j < N; j += 32) {
        const float d = drow[j];
        const Node4<float> fj = F[j];
        s0 = fmaf(d, fj.v0 - fi.v0, s0);
        s1 = fmaf(d, fj.v1 - fi.v1, s1);
        s2 = fmaf(d, fj.v2 - fi.v2, s2);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      }
      if (lane == 0) {
        float k1 = -s1, k2 = -s2;
        if (a.gx != 0.0f) {  // gravity source (solver.py:82-91)
          const float rho = us[i], u = us[N + i] / rho;
          k1 += rho * a.gx;
          k2 += rho * a.gx * u;
        }
        kb[r] = -s0;
        kb[R + r] = k1;
        kb[2 * R + r] = k2;
      }
    }
  };
  // own new rows (mine) into every CTA's stage state
  auto exchange = [&]() {
    cluster.sync();  // every CTA has finished reading its stage state
    for (int idx = tid; idx < C * 3 * nr; idx += CL_THREADS) {
      const int q = idx / (3 * nr), rem = idx - q * 3 * nr, c = rem / nr, r = rem - c * nr;
      float* dst = cluster.map_shared_rank(us, q);
      dst[c * N + i0 + r] = mine[c * R + r];
    }
    cluster.sync();  // the new state is visible everywhere
  };
  auto filter_bc = [&]() {
    if (FT != nullptr) {  // own rows of F u, summed as u_i + F_ij (u_j - u_i)
      for (int r = tid; r < nr; r += CL_THREADS) {
        const int i = i0 + r;
        const float f0 = us[i], f1 = us[N + i], f2 = us[2 * N + i];
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (int j = 0; j < N; ++j) {
          const float f = FT[(long)j * N + i];
          s0 = fmaf(f, us[j] - f0, s0);
          s1 = fmaf(f, us[N + j] - f1, s1);
          s2 = fmaf(f, us[2 * N + j] - f2, s2);
        }
        mine[r] = f0 + s0;
        mine[R + r] = f1 + s1;
        mine[2 * R + r] = f2 + s2;
      }
      exchange();
    }
    bc_apply(us, N, codes, tid);
    __syncthreads();
  };

  if (a.rhs_out != nullptr) {  // rhs only
    bc_apply(us, N, codes, tid);
    __syncthreads();
    flux();
    __syncthreads();
    own_rhs();
    __syncthreads();
    float* Rh = a.rhs_out + (long)sol * a.solve_stride;
    for (int idx = tid; idx < 3 * nr; idx += CL_THREADS) {
      const int c = idx / nr, r = idx - c * nr;
      Rh[c * N + i0 + r] = kb[c * R + r];
    }
    cluster.sync();  // no CTA leaves while others may map its shared memory
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
    if (a.t != nullptr) {  // CFL step size from the state as given (identical in every CTA)
      if (tl >= te - 1e-12) break;
      float sm = 0.0f;
      for (int i = tid; i < N; i += CL_THREADS) {
        const float rho = un[i], u = un[N + i] / rho;
        const float pp = g1 * (un[2 * N + i] - 0.5f * rho * u * u) + g1 * er;
        sm = fmaxf(sm, fabsf(u) + sqrtf(a.gamma * pp / rho));
      }
      sm = block_max(sm, red);
      if (tid == 0) red[0] = sm;
      __syncthreads();
      const double spd = (double)red[0];
      __syncthreads();
      dtd = (spd <= 0.0) ? 1e-6 : (double)a.cfl * (double)a.hmin / spd;
      dtd = fmin(dtd, te - tl);
      dt = (float)dtd;
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      if (a.rk2 && (stage == 1 || stage == 2)) continue;
      const RKCoef rc = rk_coef(stage, dt, a.rk2);
      bc_apply(us, N, codes, tid);
      __syncthreads();
      if (stage == 0) {
        for (int i = tid; i < 3 * N; i += CL_THREADS) un[i] = us[i];
        __syncthreads();
      }
      flux();
      __syncthreads();
      own_rhs();
      __syncthreads();
      for (int r = tid; r < nr; r += CL_THREADS) {
        float u3[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int s = c * N + i0 + r;
          u3[c] = rk_update_incr(stage, rc, kb[c * R + r], un[s], acc[c * R + r]);
        }
        clamp_state<1>(u3, a.gamma, a.rho_min, pmin_shift);
        mine[r] = u3[0];
        mine[R + r] = u3[1];
        mine[2 * R + r] = u3[2];
      }
      exchange();
    }
    filter_bc();  // inside the step (_rk4_step -> _apply_physical_filters)
    if (((cad0 + step) % a.filter_interval) == 0) filter_bc();  // cadence
    for (int i = tid; i < 3 * N; i += CL_THREADS) un[i] = us[i];
    __syncthreads();
    tl += dtd;
    ++taken;
  }
  if (rank == 0 && tid == 0) {
    if (a.t != nullptr) a.t[sol] = tl;
    if (a.steps_done != nullptr) a.steps_done[sol] += taken;
  }
  for (int idx = tid; idx < 3 * nr; idx += CL_THREADS) {
    const int c = idx / nr, r = idx - c * nr;
    const int i = c * N + i0 + r;
    U[i] = un[i] + (c == 2 ? er : 0.0f);
  }
  cluster.sync();  // no CTA leaves while others may map its shared memory
}

size_t cl_smem(int n, int C) {
  const int R = (n + C - 1) / C;
  return sizeof(float) * (size_t)cl_dl_floats(n, C) + 16 * (size_t)n + sizeof(float) * (6 * (size_t)n + 9 * (size_t)R);
}

template <int C>
cudaError_t launch_lgl1d_cl(const Lgl1DArgs& a, int nsolve, cudaStream_t s) {
  const size_t sm = cl_smem(a.n, C);
  cudaError_t e = cudaFuncSetAttribute(k_lgl1d_cl<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nsolve * C));
  cfg.blockDim = dim3(CL_THREADS);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, k_lgl1d_cl<C>, &cfg) != cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return cudaErrorInvalidClusterSize;  // cannot be placed on this device: the caller falls back
  }
  return cudaLaunchKernelEx(&cfg, k_lgl1d_cl<C>, a);
}

}  // namespace

size_t lgl1d_smem(int n, bool fp64) { return (size_t)4 * n * (fp64 ? 8 : 4) + (size_t)9 * n * 4; }

// one thread per node up to 1024 (whole warps), so the contraction rows are
// spread evenly and the column loads of D^T have many warps in flight
static int lgl1d_threads(int n) { return n >= 1024 ? 1024 : ((n + 31) / 32) * 32; }

// clusters of 4 CTAs for 130..257 nodes and 8 for 258..513 (float32), from n alone
static int lgl1d_cluster(int n, bool fp64) { return (fp64 || n < 130 || n > 8 * CL_ROWS) ? 0 : (n <= 4 * CL_ROWS ? 4 : 8); }

cudaError_t launch_lgl1d(const Lgl1DArgs& a, bool fp64, int nsolve, cudaStream_t s) {
  const int C = lgl1d_cluster(a.n, fp64);
  if (C > 0) {
    const cudaError_t e = (C == 4) ? launch_lgl1d_cl<4>(a, nsolve, s) : launch_lgl1d_cl<8>(a, nsolve, s);
    if (e != cudaErrorInvalidClusterSize) return e;
    cudaGetLastError();  // clusters of this shape cannot be placed here: one CTA per solve
  }
  const size_t sm = lgl1d_smem(a.n, fp64);
  cudaError_t e;
  if (fp64) {
    if ((e = cudaFuncSetAttribute(k_lgl1d<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess)
      return e;
    k_lgl1d<double><<<nsolve, lgl1d_threads(a.n), sm, s>>>(a);
  } else {
    if ((e = cudaFuncSetAttribute(k_lgl1d<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess)
      return e;
    k_lgl1d<float><<<nsolve, lgl1d_threads(a.n), sm, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_lgl1d_apply(const void* MT, bool fp64, const float* in, float* out, int n, int nf, int nsolve,
                               long ss, float rowsum, cudaStream_t s) {
  const dim3 grid((n + 255) / 256, nf * nsolve);
  if (fp64) k_lgl1d_apply<double><<<grid, 256, 0, s>>>(static_cast<const double*>(MT), in, out, n, nf, ss, rowsum);
  else k_lgl1d_apply<float><<<grid, 256, 0, s>>>(static_cast<const float*>(MT), in, out, n, nf, ss, rowsum);
  return cudaGetLastError();
}

cudaError_t launch_transpose(const void* in, void* out, int n, bool fp64, cudaStream_t s) {
  const long total = (long)n * n;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  if (fp64) k_transpose<double><<<blocks, 256, 0, s>>>(static_cast<const double*>(in), static_cast<double*>(out), n);
  else k_transpose<float><<<blocks, 256, 0, s>>>(static_cast<const float*>(in), static_cast<float*>(out), n);
  return cudaGetLastError();
}

cudaError_t launch_lgl1d_bc(float* U, int n, long ss, int nsolve, const Bc1D& bc, const int* active,
                            cudaStream_t s) {
  k_lgl1d_bc<<<nsolve, 32, 0, s>>>(U, n, ss, bc, active);
  return cudaGetLastError();
}

}  // namespace ps
