// Split-bf16 x3 differentiation-matrix contractions of the LGL x LGL path on
// the 5th-generation tensor cores (declared in lgl_tc.cuh).
//
// A float32 operand v is split as hi = bf16(v), lo = bf16(v - hi); the
// product A B^T is taken as hi_A hi_B^T + hi_A lo_B^T + lo_A hi_B^T, each term
// a bf16 tcgen05 MMA accumulating in float32 in tensor memory (the lo*lo term,
// below 2^-16 of the product, is dropped).  Operands are stored as bf16
// planes [2 (hi, lo)][batch][rows][pitch], K contiguous, and loaded by TMA
// with the 128-byte swizzle into a ring of shared-memory stages.
//
// Per RK stage (solver.py:428-466, 623-648):
//   k_flux_split   walls already applied; x flux F_x[c][j][k] and the
//                  transposed y flux F_y^T[c][i][k] as hi/lo planes
//   k_umma_x3      Gx^T = D_x F_x^T (columns (solve, c, j) stacked) and
//                  Gy[c]^T = F_y[c]^T D_y^T per solve and component: the
//                  accumulator lanes run along x, the contiguous axis of the
//                  outputs, so the epilogue stores whole 128-byte lines
//   k_lgl_update   k = -(Gx + Gy), the RK4 stage update and the 2D clamp
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "lgl.cuh"
#include "lgl_tc.cuh"
#include "pass_common.cuh"
#include "tma.cuh"
#include "umma.cuh"

namespace ps {

namespace {

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

}  // namespace

// ---------------------------------------------------------------------------
// Split a float32 matrix [rows][n] into hi/lo planes [2][rows][pitch]
// ---------------------------------------------------------------------------
__global__ void k_split_matrix(const float* __restrict__ M, int rows, int n, int pitch, __nv_bfloat16* out) {
  const long total = (long)rows * n;
  const long plane = (long)rows * pitch;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long r = e / n, k = e % n;
    __nv_bfloat16 hi, lo;
    split_bf16(M[e], hi, lo);
    out[r * pitch + k] = hi;
    out[plane + r * pitch + k] = lo;
  }
}

cudaError_t launch_split_matrix(const float* M, int rows, int n, int pitch, void* out, cudaStream_t s) {
  k_split_matrix<<<256, 256, 0, s>>>(M, rows, n, pitch, static_cast<__nv_bfloat16*>(out));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Fluxes as split planes.  Tile of 32 x 32 cells (rows j, columns i) per CTA,
// 256 threads; the transposed y flux goes through shared memory.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_flux_split(FluxSplitArgs a) {
  __shared__ float fy[4][32][33];
  const int sol = blockIdx.z;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const int nx = a.nx, ny = a.ny;
  const long cells = (long)nx * ny;
  const float* __restrict__ U = a.U + (long)sol * 4 * cells;
  const int j0 = blockIdx.y * 32, i0 = blockIdx.x * 32;
  const float gm1 = a.gamma - 1.0f, geref = a.gamma * a.eref[sol];
  const long planeX = (long)a.nsolve * 4 * ny * a.px;  // hi -> lo offset of F_x
  const long planeY = (long)a.nsolve * 4 * nx * a.py;  // of F_y^T
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  __nv_bfloat16* const fxp = static_cast<__nv_bfloat16*>(a.fx);
  __nv_bfloat16* const fyp = static_cast<__nv_bfloat16*>(a.fyt);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int jj = ty + 8 * q, j = j0 + jj, i = i0 + tx;
    float f[4] = {0.f, 0.f, 0.f, 0.f}, g[4] = {0.f, 0.f, 0.f, 0.f};
    if (j < ny && i < nx) {
      const long o = (long)j * nx + i;
      const float rho = U[o], mx = U[cells + o], my = U[2 * cells + o], e = U[3 * cells + o];
      const float ux = mx / rho, uy = my / rho;
      const float pp = gm1 * (e - 0.5f * rho * (ux * ux + uy * uy));
      const float h = e + pp + geref;
      f[0] = rho * ux;
      f[1] = rho * ux * ux + pp;
      f[2] = rho * uy * ux;
      f[3] = h * ux;
      g[0] = rho * uy;
      g[1] = rho * ux * uy;
      g[2] = rho * uy * uy + pp;
      g[3] = h * uy;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long row = ((long)sol * 4 + c) * ny + j;
        __nv_bfloat16 hi, lo;
        split_bf16(f[c], hi, lo);
        fxp[row * a.px + i] = hi;
        fxp[planeX + row * a.px + i] = lo;
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) fy[c][jj][tx] = g[c];
  }
  __syncthreads();
  // F_y^T[sol, c][i][j]: rows i, contiguous j
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int ii = ty + 8 * q, i = i0 + ii, j = j0 + tx;
    if (i < nx && j < ny) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long row = ((long)sol * 4 + c) * nx + i;
        __nv_bfloat16 hi, lo;
        split_bf16(fy[c][tx][ii], hi, lo);
        fyp[row * a.py + j] = hi;
        fyp[planeY + row * a.py + j] = lo;
      }
    }
  }
}

cudaError_t launch_flux_split(const FluxSplitArgs& a, cudaStream_t s) {
  const dim3 grid((a.nx + 31) / 32, (a.ny + 31) / 32, a.nsolve);
  k_flux_split<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// C[z][m][n] = alpha * sum_k A[z_a][m][k] B[z_b][n][k] in split bf16 x3.
// One CTA per 128 x NT output tile, 128 threads: thread 0 issues the TMA
// loads, thread 32 the MMAs, all four warps drain TMEM in the epilogue.
// ---------------------------------------------------------------------------
template <int NT, int ST>
struct UmmaSmem {
  static constexpr int kABytes = 128 * 128;  // one plane of A: 128 rows x 128 B
  static constexpr int kBBytes = NT * 128;
  static constexpr int kStage = 2 * kABytes + 2 * kBBytes;
  static constexpr int kBytes = ST * kStage + 1024;  // + alignment slack
};

template <int NT>
struct TmemCols {
  static constexpr uint32_t value = NT <= 32 ? 32 : NT <= 64 ? 64 : NT <= 128 ? 128 : 256;
};

template <int NT, int ST>
__global__ void __launch_bounds__(128, 1) k_umma_x3(const __grid_constant__ CUtensorMap mA,
                                                   const __grid_constant__ CUtensorMap mB, UmmaArgs g) {
  static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
  using SM = UmmaSmem<NT, ST>;
  constexpr uint32_t COLS = TmemCols<NT>::value;
  extern __shared__ unsigned char umma_smem_raw[];
  __shared__ uint64_t full[ST], empty[ST], done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag, issued, consumed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int z = blockIdx.z;
  if (g.active != nullptr && g.active[z / g.zper] == 0) return;
  const uint32_t raw = smem_addr(umma_smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char* sbase = umma_smem_raw + (base - raw);
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * NT;
  const int nk = (g.K + 63) / 64;
  if (tid == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    fence_barrier_init();
    abort_flag = 0;
    issued = 0;
    consumed = 0;
  }
  __syncwarp();
  if (warp == 0) {  // whole warp, converged (.sync.aligned)
    tmem_alloc(&tmem_base, COLS);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  volatile int* vabort = &abort_flag;

  if (tid == 0) {
    // producer
    const int za = g.a_batched ? z : 0, zb = g.b_batched ? z : 0;
    int kb = 0;
    for (; kb < nk; ++kb) {
      const int s = kb % ST;
      if (kb >= ST) {
        const uint32_t par = ((kb / ST) - 1) & 1;
        bool ok = false;
        for (uint32_t i = 0; i < kMaxPolls && !ok; ++i) {
          ok = mbar_try_wait(&empty[s], par);
          if (!ok && *vabort) break;
        }
        if (!ok) {
          if (!*vabort) atomicOr(g.status, kStatusTmaTimeout);
          *vabort = 1;
          break;
        }
      }
      if (*vabort) break;
      unsigned char* st = sbase + s * SM::kStage;
      mbar_arrive_expect_tx(&full[s], SM::kStage);
      tma_load_4d(st, &mA, kb * 64, m0, za, 0, &full[s]);
      tma_load_4d(st + SM::kABytes, &mA, kb * 64, m0, za, 1, &full[s]);
      tma_load_4d(st + 2 * SM::kABytes, &mB, kb * 64, n0, zb, 0, &full[s]);
      tma_load_4d(st + 2 * SM::kABytes + SM::kBBytes, &mB, kb * 64, n0, zb, 1, &full[s]);
    }
    issued = kb;
  } else if (tid == 32) {
    // MMA issuer
    constexpr uint32_t idesc = bf16_idesc(128, NT);
    int kb = 0;
    for (; kb < nk; ++kb) {
      const int s = kb % ST;
      const uint32_t par = (kb / ST) & 1;
      bool ok = false;
      for (uint32_t i = 0; i < kMaxPolls && !ok; ++i) {
        ok = mbar_try_wait(&full[s], par);
        if (!ok && *vabort) break;
      }
      if (!ok) {
        if (!*vabort) atomicOr(g.status, kStatusTmaTimeout);
        *vabort = 1;
        break;
      }
      tc_fence_after();
      const uint32_t st = base + s * SM::kStage;
      const uint32_t ahi = st, alo = st + SM::kABytes;
      const uint32_t bhi = st + 2 * SM::kABytes, blo = bhi + SM::kBBytes;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t off = kk * 32;  // 16 bf16 along K
        const uint64_t dAh = sw128_kmajor_desc(ahi + off), dAl = sw128_kmajor_desc(alo + off);
        const uint64_t dBh = sw128_kmajor_desc(bhi + off), dBl = sw128_kmajor_desc(blo + off);
        umma_bf16(tmem, dAh, dBh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
        umma_bf16(tmem, dAh, dBl, idesc, 1u);
        umma_bf16(tmem, dAl, dBh, idesc, 1u);
      }
      umma_commit(&empty[s]);
    }
    consumed = kb;
    umma_commit(&done);
  }
  __syncwarp();
  // epilogue: every thread owns one accumulator row (TMEM lane)
  bool ok = false;
  for (uint32_t i = 0; i < kMaxPolls && !ok; ++i) ok = mbar_try_wait(&done, 0);
  if (!ok) atomicOr(g.status, kStatusTmaTimeout);
  tc_fence_after();
  const int all_ok = __syncthreads_and(ok ? 1 : 0);  // CTA-uniform: TMEM loads are warp-collective
  const bool valid = all_ok && (*vabort == 0);
  const int m = m0 + warp * 32 + lane;
  float* C = g.C + (long)z * g.cz;
  if (valid) {
#pragma unroll 1
    for (int c0 = 0; c0 < NT; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (m < g.M) {
        if (g.c_trans) {  // lanes (m) along contiguous memory: one 128-byte store per column
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int n = n0 + c0 + q;
            if (n < g.N) C[(long)n * g.ldc + m] = g.alpha * v[q];
          }
        } else {
          float* row = C + (long)m * g.ldc;
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int n = n0 + c0 + q;
            if (n < g.N) row[n] = g.alpha * v[q];
          }
        }
      }
    }
  }
  // drain loads that were issued but never consumed (abort path only)
  if (tid == 0) {
    for (int kb = consumed; kb < issued; ++kb) {
      const int s = kb % ST;
      const uint32_t par = (kb / ST) & 1;
      for (uint32_t i = 0; i < kMaxPolls; ++i)
        if (mbar_try_wait(&full[s], par)) break;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, COLS);
  }
}

// 4-D map over split planes [2][batch][rows][pitch] bf16 (dims innermost
// first: k (logical n_k), rows, batch, plane), box 64 x box_rows, 128-byte swizzle.
int encode_split_map(CUtensorMap* m, const void* base, int nk, int rows, int batch, int pitch, int box_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  if (!fn) return -1;
  const cuuint64_t dims[4] = {(cuuint64_t)nk, (cuuint64_t)rows, (cuuint64_t)batch, 2};
  const cuuint64_t row_b = (cuuint64_t)pitch * 2;
  const cuuint64_t strides[3] = {row_b, row_b * rows, row_b * rows * batch};
  const cuuint32_t box[4] = {64, (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return (r == CUDA_SUCCESS) ? 0 : (int)r;
}

template <int NT, int ST>
static cudaError_t umma_t(const CUtensorMap& mA, const CUtensorMap& mB, const UmmaArgs& g, cudaStream_t s) {
  constexpr int bytes = UmmaSmem<NT, ST>::kBytes;
  static bool configured = false;  // attribute set once per process (same value every time)
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_umma_x3<NT, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const dim3 grid((g.N + NT - 1) / NT, (g.M + 127) / 128, g.batch);
  k_umma_x3<NT, ST><<<grid, 128, bytes, s>>>(mA, mB, g);
  return cudaGetLastError();
}

// Resident CTAs per SM of each N tile (shared memory: NT = 64 runs 2 stages in
// 97 KB, two per SM; the others 150-200 KB, one per SM).  The smallest tile
// whose grid fits in one wave gives the most parallelism; a grid too large for
// one wave takes the widest tile (fewest re-reads of the A operand).
int umma_n_tile(int M, int N, int batch) {
  const long mt = (M + 127) / 128;
  const int cand[4] = {64, 128, 176, 256};
  const int per_sm[4] = {2, 1, 1, 1};
  for (int i = 0; i < 4; ++i)
    if (mt * ((N + cand[i] - 1) / cand[i]) * batch <= 148L * per_sm[i]) return cand[i];
  return 256;
}

cudaError_t launch_umma_x3(const CUtensorMap& mA, const CUtensorMap& mB, const UmmaArgs& g, int nt, cudaStream_t s) {
  switch (nt) {
    case 64: return umma_t<64, 2>(mA, mB, g, s);
    case 128: return umma_t<128, 3>(mA, mB, g, s);
    case 176: return umma_t<176, 2>(mA, mB, g, s);
    case 256: return umma_t<256, 2>(mA, mB, g, s);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// k = -(Gx + Gy), RK4 stage update and the 2D clamp, per cell (E' form)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_lgl_update(LglUpdateArgs a) {
  const int sol = blockIdx.y;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const long cells = a.cells;
  const long so = (long)sol * 4 * cells;
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  const float pmin_shift = a.p_min - (a.gamma - 1.0f) * a.eref[sol];
  for (long o = blockIdx.x * (long)blockDim.x + threadIdx.x; o < cells; o += (long)gridDim.x * blockDim.x) {
    // every load of the cell first, then the arithmetic, then the stores: a
    // store between loads (acc may alias nothing the compiler can prove) would
    // make each component wait for the previous one's round trip to memory
    float k[4], un[4], ac[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const long g = so + c * cells + o;
      k[c] = a.Gy != nullptr ? a.Gx[g] + a.Gy[g] : a.Gx[g];
      un[c] = (a.stage >= 0) ? a.Un[g] : 0.0f;
      ac[c] = (a.stage >= 1) ? a.acc[g] : 0.0f;
    }
    float grho = 0.0f, gmx = 0.0f, gmy = 0.0f;
    if (a.gravity) {
      grho = a.Uin[so + o];
      gmx = a.Uin[so + cells + o];
      gmy = a.Uin[so + 2 * cells + o];
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) k[c] = a.ksign * k[c];
    if (a.gravity) {  // rho g on the momenta, g . m on the energy (solver.py:453-464)
      k[1] = fmaf(grho, a.g[0], k[1]);
      k[2] = fmaf(grho, a.g[1], k[2]);
      k[3] += a.g[0] * gmx + a.g[1] * gmy;
    }
    if (a.stage < 0) {
#pragma unroll
      for (int c = 0; c < 4; ++c) a.out[so + c * cells + o] = k[c];
      continue;
    }
    float u[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) u[c] = rk_update_incr(a.stage, rk, k[c], un[c], ac[c]);
    if (a.stage != 3) {
#pragma unroll
      for (int c = 0; c < 4; ++c) a.acc[so + c * cells + o] = ac[c];
    }
    clamp_state<2>(u, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
    for (int c = 0; c < 4; ++c) a.out[so + c * cells + o] = u[c];
  }
}

cudaError_t launch_lgl_update(const LglUpdateArgs& a, cudaStream_t s) {
  const long want = (a.cells + 255) / 256;
  const int per = (int)((want < 1216 / a.nsolve + 1) ? want : 1216 / a.nsolve + 1);
  k_lgl_update<<<dim3(per > 0 ? per : 1, a.nsolve), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace ps
