// ps_rhs_static: the right-hand side of ps_rhs for small 2D/3D Fourier
// grids, computed without allocating any device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// evaluate a right-hand side -- code running inside a CUDA stream capture
// (allocation is not a capturable operation), solvers embedded in a host
// framework that owns every device allocation through its own pool, and
// real-time loops that forbid allocator calls after start-up.  ps_rhs needs a
// plan, and ps_plan_create allocates the spectral tables and the pass
// intermediates; this entry point takes the grid description by value and
// keeps everything it needs in one fixed-size array in device global memory.
//
// Scratch: g_rhs_static_scratch below (file-scope __device__ array, 256-byte
// aligned).  Every GPU that loads the library holds it until the process
// exits.  It is sized for grids of at most PS_RHS_STATIC_MAX_CELLS cells and
// pencils of at most 1024 points; larger grids are rejected.  All calls share
// the one array and it keeps the last call's contents: a call rebuilds the
// spectral tables and E_ref and overwrites every intermediate before reading
// it, so nothing has to start at zero.  Two calls whose kernels overlap on the
// GPU (different streams, or different host threads on one device) race on
// the array; order them on one stream.
//
// Device address: host code cannot pass g_rhs_static_scratch to a kernel
// directly (in host code the name is a host-side shadow, not a device
// address).  The first call on each device, with that device current, calls
// cudaGetSymbolAddress once and caches the result; that first call should
// therefore come before any stream capture.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <mutex>

#include "../../include/phrike_gb300.h"
#include "launch.cuh"
#include "reduce.cuh"

namespace ps {
int record_error(int code, const char* msg);
int encode_field_map(CUtensorMap* m, const float* base, const int n[3], int nf, int axis, int tcols = 0);
int validate_desc(const ps_plan_desc* d);
int tile_cols_2d(int nx, int ny, int nsolve, bool mhd);
}

namespace {

constexpr long kMaxCells = PS_RHS_STATIC_MAX_CELLS;
constexpr int kMaxN = 1024;
constexpr long kAxisFloats = 6L * kMaxN;       // P, d (N floats each), twf, twi (N float2 each)
constexpr long kTableFloats = 3 * kAxisFloats;  // three axes
constexpr long kErefOffset = kTableFloats;      // one float, padded to 256 bytes
constexpr long kGOffset = kErefOffset + 64;
constexpr long kABOffset = kGOffset + 15 * kMaxCells;
constexpr long kTotalFloats = kABOffset + 10 * kMaxCells;

__device__ __align__(256) float g_rhs_static_scratch[kTotalFloats];

std::mutex g_addr_mutex;
float* g_addr[64] = {nullptr};

int fail(int code, const char* msg) { return ps::record_error(code, msg); }

int fail_cuda(cudaError_t e, const char* what) {
  char msg[256];
  snprintf(msg, sizeof(msg), "ps_rhs_static: %s: %s", what, cudaGetErrorString(e));
  return ps::record_error(PS_ERR_CUDA, msg);
}

__host__ __device__ inline int threads_per_pencil(int N) {  // two-step pencils, N <= 256
  return (N == 8) ? 2 : (N == 16 || N == 32) ? 4 : (N == 64 || N == 128) ? 8 : 16;
}

// Spectral tables of one axis, built on the device in float64 (same
// definitions as the plan's host-built tables: 2/3 mask, exponential filter,
// 1/N folded in, Nyquist derivative term zeroed, twiddles of the pencil FFT:
// the two-step layout for N <= 256; for N > 256 the 256-point sub-pencil
// tables followed by the group twiddles W_N^{g j}).
__global__ void k_static_axis(int N, double L, int dealias, int fon, int fp, double falpha, float* P, float* d,
                              float2* twf, float2* twi) {
  const double kmax = N / 2;
  const int base = (N > 256) ? 256 : N;
  const int A = threads_per_pencil(base);
  const int B = base / A;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    const int kk = (k < N / 2) ? k : k - N;
    const double ak = fabs((double)kk);
    double m = (!dealias || ak <= (double)(N / 3)) ? 1.0 : 0.0;
    if (fon) m *= exp(-falpha * pow(ak / (kmax > 1.0 ? kmax : 1.0), (double)fp));
    P[k] = (float)(m / N);
    d[k] = (k == N / 2) ? 0.0f : (float)((2.0 * kk / L) * 3.14159265358979323846 * m / N);
    double sn, cs;
    if (k < base) {  // entry k = k2*A + n1 of the forward table, n1*B + k2 of the inverse
      const int k2 = k / A, n1 = k % A;
      sincospi(-2.0 * (double)((long)n1 * k2 % base) / base, &sn, &cs);
      twf[k2 * A + n1] = make_float2((float)cs, (float)sn);
      twi[n1 * B + k2] = make_float2((float)cs, (float)-sn);
    } else {  // group twiddles, k = 256 g + j
      const int g = k / 256, j = k % 256;
      sincospi(-2.0 * (double)((long)g * j % N) / N, &sn, &cs);
      twf[k] = make_float2((float)cs, (float)sn);
      twi[k] = make_float2((float)cs, (float)-sn);
    }
  }
}

}  // namespace

extern "C" int ps_rhs_static(const ps_plan_desc* desc, const float* U, float* rhs, void* stream) {
  if (!desc || !U || !rhs) return fail(PS_ERR_INVALID, "ps_rhs_static: null argument");
  if (desc->ndim != 2 && desc->ndim != 3)
    return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: only 2D and 3D grids are supported");
  if (desc->equations != PS_EQ_EULER) return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: Euler equations only");
  for (int a = 0; a < desc->ndim; ++a)
    if (desc->basis[a] != PS_BASIS_FOURIER) return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: Fourier basis only");
  if (desc->av_mode != PS_AV_OFF || desc->gravity[0] != 0.0 || desc->gravity[1] != 0.0 || desc->gravity[2] != 0.0)
    return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: no artificial viscosity or gravity terms");
  int rc = ps::validate_desc(desc);  // the checks ps_plan_create makes
  if (rc != PS_OK) return rc;
  for (int a = 0; a < desc->ndim; ++a)  // plans take any 5-smooth length; the static tables hold powers of two
    if (!ps::supported_n(desc->n[a]))
      return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: axis lengths are powers of two from 8 to 1024");
  long cells = 1;
  for (int a = 0; a < desc->ndim; ++a) cells *= desc->n[a];
  if (cells > kMaxCells) {
    char msg[200];
    snprintf(msg, sizeof(msg), "ps_rhs_static: grid of %ld cells exceeds the static scratch limit of %ld cells",
             cells, kMaxCells);
    return fail(PS_ERR_UNSUPPORTED, msg);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(PS_ERR_UNSUPPORTED, "ps_rhs_static: device ordinal out of range");
  float* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (g_addr[dev] == nullptr) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_rhs_static_scratch);
      if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress");
      g_addr[dev] = static_cast<float*>(ptr);
    }
    base = g_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nd = desc->ndim, nc = nd + 2;
  ps::AxisOps ax[3];
  for (int a = 0; a < nd; ++a) {
    const int N = desc->n[a];
    float* tab = base + a * kAxisFloats;
    float* P = tab;
    float* d = tab + kMaxN;
    float2* twf = reinterpret_cast<float2*>(tab + 2 * kMaxN);
    float2* twi = reinterpret_cast<float2*>(tab + 4 * kMaxN);
    k_static_axis<<<(N + 127) / 128, 128, 0, s>>>(N, desc->length[a], desc->dealias,
                                                  desc->filter_enabled, desc->filter_p, desc->filter_alpha, P, d,
                                                  twf, twi);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "table kernel");
    ax[a] = ps::AxisOps{P, d, twf, twi};
  }
  float* eref = base + kErefOffset;
  float* G = base + kGOffset;
  float* AB = base + kABOffset;
  const int nx = desc->n[0], ny = desc->n[1], nz = (nd == 3) ? desc->n[2] : 1;
  if ((e = ps::launch_eref_set(U + (long)(nc - 1) * cells, (long)nc * cells, 1, eref, s)) != cudaSuccess)
    return fail_cuda(e, "energy reference");

  ps::XFirstArgs xa{};
  xa.U = U;
  xa.Uw = nullptr;
  xa.out = G;
  xa.fs = cells;
  xa.ssU = (long)nc * cells;
  xa.ssOut = (long)nd * nc * cells;
  xa.rows = (int)(cells / nx);
  xa.rps = xa.rows;
  xa.active = nullptr;
  xa.ax = ax[0];
  xa.gamma = (float)desc->gamma;
  xa.speed = nullptr;
  xa.eref = eref;
  xa.shift_in = 1;
  e = ps::dispatch_n(nx, [&](auto n) { return ps::launch_xfirst<decltype(n)::value>(nd, xa, s); });
  if (e != cudaSuccess) return fail_cuda(e, "x pass");

  // tensor maps of the scratch intermediates and of U (host structs, no
  // allocation); 2D grids take the plan's tile width (the maps' box width)
  const int n3[3] = {nx, ny, nz};
  const int tc = (nd == 2) ? ps::tile_cols_2d(nx, ny, 1, false) : 0;
  CUtensorMap mG, mAB, mU;
  if ((rc = ps::encode_field_map(&mG, G, n3, (nd == 3) ? 15 : 8, 1, tc)) != PS_OK) return rc;
  if (nd == 3 && (rc = ps::encode_field_map(&mAB, AB, n3, 10, 2)) != PS_OK) return rc;
  if ((rc = ps::encode_field_map(&mU, U, n3, nc, (nd == 3) ? 2 : 1, tc)) != PS_OK) return rc;
  const ps::StridedGeom gy{nx, (long)nx, (long)nx * ny, nz};
  if (nd == 3) {
    ps::YMidTArgs ya{};
    ya.out = AB;
    ya.fs = cells;
    ya.ssOut = 10 * cells;
    ya.active = nullptr;
    ya.nsolve = 1;
    ya.g = gy;
    ya.ax = ax[1];
    ya.status = nullptr;
    e = ps::dispatch_n(ny, [&](auto n) { return ps::launch_ymid3_t<decltype(n)::value>(mG, ya, s); });
    if (e != cudaSuccess) return fail_cuda(e, "y pass");
  }
  ps::LastTArgs la{};
  if (nd == 3) {
    la.fa0 = 0;
    la.fb0 = 5;
    la.g = ps::StridedGeom{nx, (long)nx * ny, (long)nx, ny};
    la.axis = 2;
    la.ax = ax[2];
  } else {
    la.fa0 = 0;
    la.fb0 = nc;
    la.g = gy;
    la.axis = 1;
    la.ax = ax[1];
  }
  la.nfAB = (nd == 3) ? 10 : 2 * nc;
  la.acc = nullptr;
  la.out = rhs;
  la.fs = cells;
  la.ssAcc = la.ssOut = la.ssUn = (long)nc * cells;
  la.active = nullptr;
  la.nsolve = 1;
  la.stage = -1;
  la.Un = U;
  la.dt_dev = nullptr;
  la.dt = 0.0;
  la.gamma = (float)desc->gamma;
  la.rho_min = 1e-8f;
  la.p_min = 1e-10f;
  la.eref = eref;
  la.filter_last = 0;
  la.status = nullptr;
  la.tcols = tc;
  const int nlast = (nd == 3) ? nz : ny;
  // rhs mode reads no U^n or accumulator tiles; U's map fills those slots
  e = ps::dispatch_n(nlast, [&](auto n) {
    return ps::launch_last_t<decltype(n)::value>(nd, (nd == 3) ? mAB : mG, mU, mU, la, s);
  });
  if (e != cudaSuccess) return fail_cuda(e, "last pass");
  return PS_OK;
}
