// LGL x LGL plans: validation, device tables, the RK4 step loop (fixed dt or
// CFL), bare right-hand side, derivative and filter operators.
//
// One RK stage is three launches: the walls on the stage input (in place, as
// _compute_rhs_2d does, solver.py:428-466 with grid.py:1072-1154), the x
// kernel (x flux contracted with D_x) and the y kernel (y flux contracted
// with D_y, fused with the RK4 stage update and the 2D clamp).  After each
// step, at the filter cadence, the nodal filter (if enabled) and the walls
// are applied to the new state (solver.py:623-648).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "lgl.cuh"
#include "lgl_tc.cuh"
#include "lgl1d.cuh"
#include "plan.cuh"
#include "reduce.cuh"

namespace ps {
namespace {

int cfail(cudaError_t e, const char* what) { return errorf(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); }

#define LGL_CU(expr, what)                     \
  do {                                         \
    cudaError_t _e = (expr);                   \
    if (_e != cudaSuccess) return cfail(_e, what); \
  } while (0)

// arithmetic of the CUDA-core kernels (split bf16 for both bf16x3 modes)
int mode_of(const ps_plan_s* p) {
  return (p->gemm == PS_GEMM_FP64) ? 1 : (p->gemm == PS_GEMM_BF16X3 || p->gemm == PS_GEMM_BF16X3_SIMT) ? 2 : 0;
}
bool tensor_cores(const ps_plan_s* p) { return p->gemm == PS_GEMM_BF16X3; }

// axis index of the LGL tables: 0 = x (n[0]), 1 = y (n[1])
const void* dmat(const ps_plan_s* p, int a) {
  return (p->gemm == PS_GEMM_FP64) ? static_cast<const void*>(p->D64[a]) : static_cast<const void*>(p->D32[a]);
}
const void* fmat(const ps_plan_s* p, int a) {
  return (p->gemm == PS_GEMM_FP64) ? static_cast<const void*>(p->F64[a]) : static_cast<const void*>(p->F32[a]);
}

LglStageArgs stage_args(ps_plan p, const float* in, int stage, const float* Un, float* out, double dt,
                        const double* d_dt, const int* active) {
  LglStageArgs a{};
  a.U = in;
  a.Gx = p->G;
  a.Dx = dmat(p, 0);
  a.Dy = dmat(p, 1);
  a.nx = p->n[0];
  a.ny = p->n[1];
  a.ss = p->ss(4);
  a.gamma = (float)p->desc.gamma;
  a.eref = p->eref;
  a.active = active;
  a.stage = stage;
  a.Un = Un;
  a.acc = p->acc;
  a.out = out;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.rho_min = 1e-8f;  // 2D clamp floors (solver.py:489-490)
  a.p_min = 1e-10f;
  a.nsolve = p->nsolve;
  a.g[0] = (float)p->desc.gravity[0];
  a.g[1] = (float)p->desc.gravity[1];
  a.gravity = (p->desc.gravity[0] != 0.0 || p->desc.gravity[1] != 0.0) ? 1 : 0;
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  return a;
}

// bytes of one float32 field over all solves; the x kernel moves 8 fields
// (reads U, writes Gx), the y kernel 12..24 (reads U and Gx, plus U^n and the
// accumulator and their writes as the stage needs them)
double field_bytes(const ps_plan_s* p) { return 4.0 * p->cells * p->nsolve; }

// One stage on the tensor cores: split flux planes, the two split-bf16 x3
// contractions (x: all solves and components stacked as rows; y: one batch
// entry per solve and component), then the elementwise update.
int stage_tc(ps_plan p, const float* in, int st, const float* Un, float* out, double dt, const double* d_dt,
             const int* act, cudaStream_t s) {
  const int nx = p->n[0], ny = p->n[1];
  float* Gx = p->G;
  float* Gy = p->G + 4 * p->cells * p->nsolve;
  {
    FluxSplitArgs f{};
    f.U = in;
    f.fx = p->FX;
    f.fyt = p->FYT;
    f.nx = nx;
    f.ny = ny;
    f.px = p->pitch[0];
    f.py = p->pitch[1];
    f.nsolve = p->nsolve;
    f.gamma = (float)p->desc.gamma;
    f.eref = p->eref;
    f.active = act;
    ProfScope prof(p, s, PS_KIND_OP, (4.0 + 8.0) * field_bytes(p));
    LGL_CU(launch_flux_split(f, s), "LGL split fluxes");
  }
  {
    // Gx^T[i][(solve, c, j)] = sum_k D_x[i][k] F_x[(solve, c, j)][k]
    UmmaArgs g{};
    g.C = Gx;
    g.ldc = nx;
    g.cz = 0;
    g.M = nx;
    g.N = p->nsolve * 4 * ny;
    g.K = nx;
    g.batch = 1;
    g.c_trans = 1;
    g.alpha = 1.0f;
    g.zper = 1;
    g.status = p->status;
    ProfScope prof(p, s, PS_KIND_LGL_X, 8.0 * field_bytes(p));
    LGL_CU(launch_umma_x3(p->map_Dx, p->map_FX, g, p->nt_x, s), "LGL x contraction (tensor cores)");
  }
  {
    // Gy[solve, c]^T[i][j] = sum_k F_y^T[solve, c][i][k] D_y[j][k]
    UmmaArgs g{};
    g.C = Gy;
    g.ldc = nx;
    g.cz = p->cells;
    g.M = nx;
    g.N = ny;
    g.K = ny;
    g.batch = p->nsolve * 4;
    g.a_batched = 1;
    g.c_trans = 1;
    g.active = act;
    g.zper = 4;
    g.alpha = 1.0f;
    g.status = p->status;
    ProfScope prof(p, s, PS_KIND_LGL_Y, 8.0 * field_bytes(p));
    LGL_CU(launch_umma_x3(p->map_FYT, p->map_Dy, g, p->nt_y, s), "LGL y contraction (tensor cores)");
  }
  LglUpdateArgs u{};
  u.Gx = Gx;
  u.Gy = Gy;
  u.ksign = -1.0f;
  u.Un = Un;
  u.acc = p->acc;
  u.out = out;
  u.cells = p->cells;
  u.nsolve = p->nsolve;
  u.stage = st;
  u.dt_dev = d_dt;
  u.dt = dt;
  u.gamma = (float)p->desc.gamma;
  u.rho_min = 1e-8f;
  u.p_min = 1e-10f;
  u.eref = p->eref;
  u.active = act;
  u.Uin = in;
  u.g[0] = (float)p->desc.gravity[0];
  u.g[1] = (float)p->desc.gravity[1];
  u.gravity = (p->desc.gravity[0] != 0.0 || p->desc.gravity[1] != 0.0) ? 1 : 0;
  u.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  const double words = (st < 0) ? 12.0 : (st == 0) ? 20.0 : (st == 3) ? 20.0 : 24.0;
  ProfScope prof(p, s, PS_KIND_LAST, words * field_bytes(p));
  LGL_CU(launch_lgl_update(u, s), "LGL stage update");
  return PS_OK;
}

int stage(ps_plan p, float* in, int st, float* Un, float* out, double dt, const double* d_dt, const int* act,
          cudaStream_t s) {
  LGL_CU(launch_lgl_bc(in, p->n[0], p->n[1], p->ss(4), p->nsolve, act, s), "LGL walls");
  if (tensor_cores(p)) return stage_tc(p, in, st, Un, out, dt, d_dt, act, s);
  const LglStageArgs a = stage_args(p, in, st, Un, out, dt, d_dt, act);
  {
    ProfScope prof(p, s, PS_KIND_LGL_X, 8.0 * field_bytes(p));
    LGL_CU(launch_lgl_x(a, mode_of(p), s), "LGL x contraction");
  }
  {
    const double words = (st < 0) ? 12.0 : (st == 0) ? 20.0 : (st == 3) ? 20.0 : 24.0;
    ProfScope prof(p, s, PS_KIND_LGL_Y, words * field_bytes(p));
    LGL_CU(launch_lgl_y(a, mode_of(p), s), "LGL y contraction + stage update");
  }
  return PS_OK;
}

// out[z] = f[z] . M^T along x (M = D_x or F_x) or M . f[z] along y, for Z
// consecutive fields of `cells` each.  f and out must not alias.
int contract(ps_plan p, int axis, bool filter, const float* f, float* out, long Z, const int* act, int zper,
             cudaStream_t s) {
  const int nx = p->n[0], ny = p->n[1];
  const long cells = p->cells;
  GemmArgs g{};
  g.c = out;
  g.batch = (int)Z;
  g.alpha = 1.0f;
  g.active = act;
  g.zper = zper;
  const void* M = filter ? fmat(p, axis) : dmat(p, axis);
  GemmKind kind = kGemmF32;
  bool ak, bk;
  if (axis == 0) {
    g.a = f;
    g.b = M;
    g.M = ny;
    g.N = nx;
    g.K = nx;
    g.am = nx, g.ak = 1, g.az = cells;
    g.bn = nx, g.bk = 1, g.bz = 0;
    ak = true;
    bk = true;
    if (p->gemm == PS_GEMM_FP64) kind = kGemmF32F64;
  } else {
    g.a = M;
    g.b = f;
    g.M = ny;
    g.N = nx;
    g.K = ny;
    g.am = ny, g.ak = 1, g.az = 0;
    g.bn = 1, g.bk = nx, g.bz = cells;
    ak = true;
    bk = false;
    if (p->gemm == PS_GEMM_FP64) kind = kGemmF64F32;
  }
  g.cm = nx, g.cn = 1, g.cz = cells;
  // subtract each pencil's first value from the field operand (x pencils are
  // rows of A, y pencils rows of B); D annihilates it, the filter keeps it
  g.offset = (axis == 0) ? 1 : 2;
  g.add_back = filter ? 1 : 0;
  if (p->gemm == PS_GEMM_BF16X3 || p->gemm == PS_GEMM_BF16X3_SIMT) kind = kGemmSplitAB;
  for (long z0 = 0; z0 < Z; z0 += 65535) {  // grid.z limit
    GemmArgs gz = g;
    gz.batch = (int)((Z - z0 < 65535) ? Z - z0 : 65535);
    gz.a = (axis == 0) ? static_cast<const void*>(f + z0 * cells) : M;
    gz.b = (axis == 0) ? M : static_cast<const void*>(f + z0 * cells);
    gz.c = out + z0 * cells;
    if (act != nullptr && z0 != 0) return errorf(PS_ERR_INVALID, "internal: masked contraction over 65535 fields");
    LGL_CU(launch_gemm(gz, kind, ak, bk, s), "LGL contraction");
  }
  return PS_OK;
}

// nodal filter of the state, both axes, through the scratch G (4 nsolve fields)
int filter_state(ps_plan p, float* U, const int* act, cudaStream_t s) {
  int rc;
  const long Z = 4L * p->nsolve;
  ProfScope prof(p, s, PS_KIND_OP, 16.0 * 4.0 * p->cells * p->nsolve);
  if ((rc = contract(p, 0, true, U, p->G, Z, act, 4, s)) != PS_OK) return rc;
  return contract(p, 1, true, p->G, U, Z, act, 4, s);
}

}  // namespace

int lgl_validate(const ps_plan_desc* d) {
  if (d->ndim == 1) {  // Grid1D(basis="legendre") with SpectralSolver1D
    if (d->equations != PS_EQ_EULER) return errorf(PS_ERR_UNSUPPORTED, "1D Legendre grids carry the Euler equations");
    if (d->n[0] < 3 || d->n[0] > 2048) return errorf(PS_ERR_UNSUPPORTED, "1D LGL grids need 3..2048 nodes");
    if (!(d->length[0] > 0.0)) return errorf(PS_ERR_INVALID, "length must be positive");
    if (!(d->gamma > 1.0)) return errorf(PS_ERR_INVALID, "gamma must exceed 1");
    if (d->filter_interval < 1) return errorf(PS_ERR_INVALID, "filter_interval must be >= 1");
    if (d->av_mode != PS_AV_OFF)
      return errorf(PS_ERR_UNSUPPORTED, "artificial viscosity is not implemented for LGL grids");
    if (d->gemm_precision != PS_GEMM_FP32 && d->gemm_precision != PS_GEMM_FP64)
      return errorf(PS_ERR_UNSUPPORTED, "1D LGL contractions run in float32 or float64");
    for (int i = 0; i < 6; ++i)
      if (d->lgl_bc1d[i] < 0 || d->lgl_bc1d[i] > 2) return errorf(PS_ERR_INVALID, "boundary codes are 0, 1 or 2");
    return PS_OK;
  }
  if (d->ndim != 2) return errorf(PS_ERR_UNSUPPORTED, "the Legendre basis is supported on 1D and 2D grids only");
  if (d->basis[0] != PS_BASIS_LEGENDRE || d->basis[1] != PS_BASIS_LEGENDRE)
    return errorf(PS_ERR_UNSUPPORTED, "mixed Fourier x Legendre grids are not supported (LGL on both axes only)");
  if (d->equations != PS_EQ_EULER) return errorf(PS_ERR_UNSUPPORTED, "equation set %d not supported", d->equations);
  for (int a = 0; a < 2; ++a) {
    if (d->n[a] < 3 || d->n[a] > 4096)
      return errorf(PS_ERR_UNSUPPORTED, "axis %d: LGL grids need 3..4096 nodes (got %d)", a, d->n[a]);
    if (!(d->length[a] > 0.0)) return errorf(PS_ERR_INVALID, "axis %d: length must be positive", a);
  }
  if (!(d->gamma > 1.0)) return errorf(PS_ERR_INVALID, "gamma must exceed 1");
  if (d->filter_interval < 1) return errorf(PS_ERR_INVALID, "filter_interval must be >= 1");
  if (d->av_mode != PS_AV_OFF)
    return errorf(PS_ERR_UNSUPPORTED, "artificial viscosity is not implemented for LGL grids");
  if (d->gemm_precision < PS_GEMM_FP32 || d->gemm_precision > PS_GEMM_BF16X3_SIMT)
    return errorf(PS_ERR_INVALID,
                  "gemm_precision must be PS_GEMM_FP32, PS_GEMM_FP64, PS_GEMM_BF16X3 or PS_GEMM_BF16X3_SIMT");
  return PS_OK;
}

size_t lgl_scratch_bytes(const ps_plan_desc* d, int nsolve) {
  size_t b = 0;
  if (d->ndim == 1) {
    const size_t n = (size_t)d->n[0];
    return 16 * n + 20 * n * n + (d->filter_enabled ? 20 * n * n : 0);  // D, F (float64, float32, transposed)
  }
  for (int a = 0; a < 2; ++a) {
    const size_t n = (size_t)d->n[a];
    b += 16 * n + 12 * n * n;                 // nodes, weights, D in float64 and float32
    if (d->filter_enabled) b += 12 * n * n;  // filter matrices
  }
  if (d->gemm_precision == PS_GEMM_BF16X3) {
    const size_t nx = d->n[0], ny = d->n[1], px = (nx + 7) / 8 * 8, py = (ny + 7) / 8 * 8;
    b += 4 * (nx * px + ny * py);                             // split D planes
    b += 4 * 4 * (size_t)nsolve * (ny * px + nx * py);       // split flux planes
  }
  return b;
}

int lgl_setup(ps_plan p) {
  int rc;
  p->lgl = true;
  p->gemm = p->desc.gemm_precision;
  double hmin = 1e300;
  for (int a = 0; a < p->nd; ++a) {
    const int n = p->n[a];
    if ((rc = plan_alloc(p, &p->lgl_x[a], n)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &p->lgl_w[a], n)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &p->D64[a], (size_t)n * n)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &p->D32[a], (size_t)n * n)) != PS_OK) return rc;
    LGL_CU(launch_lgl_build(n, p->desc.length[a], p->lgl_x[a], p->lgl_w[a], p->D64[a], p->D32[a], 0),
           "LGL construction");
    if (p->desc.filter_enabled) {
      if ((rc = plan_alloc(p, &p->F64[a], (size_t)n * n)) != PS_OK) return rc;
      if ((rc = plan_alloc(p, &p->F32[a], (size_t)n * n)) != PS_OK) return rc;
      LGL_CU(launch_lgl_filter_matrix(n, p->desc.length[a], p->lgl_x[a], p->lgl_w[a], p->desc.filter_p,
                                      p->desc.filter_alpha, p->F64[a], p->F32[a], 0),
             "LGL filter matrix");
    }
    std::vector<double> x(n);
    LGL_CU(cudaMemcpy(x.data(), p->lgl_x[a], sizeof(double) * n, cudaMemcpyDeviceToHost), "LGL nodes read");
    for (int j = 0; j + 1 < n; ++j) hmin = fmin(hmin, x[j + 1] - x[j]);  // grid.py:826-832
  }
  p->lgl_hmin = hmin;
  if (p->nd == 1) {  // transposed matrices for the column-by-column contractions of k_lgl1d
    const int n = p->n[0];
    const bool fp64 = p->gemm == PS_GEMM_FP64;
    const size_t esz = fp64 ? sizeof(double) : sizeof(float);
    unsigned char* dt = nullptr;
    if ((rc = plan_alloc(p, &dt, esz * n * n)) != PS_OK) return rc;
    LGL_CU(launch_transpose(fp64 ? (const void*)p->D64[0] : (const void*)p->D32[0], dt, n, fp64, 0), "D transpose");
    p->lgl_DT = dt;
    if (p->desc.filter_enabled) {
      unsigned char* ft = nullptr;
      if ((rc = plan_alloc(p, &ft, esz * n * n)) != PS_OK) return rc;
      LGL_CU(launch_transpose(fp64 ? (const void*)p->F64[0] : (const void*)p->F32[0], ft, n, fp64, 0),
             "filter transpose");
      p->lgl_FT = ft;
    }
    LGL_CU(cudaDeviceSynchronize(), "1D LGL tables");
    return PS_OK;
  }
  if (p->gemm == PS_GEMM_BF16X3) {
    const int nx = p->n[0], ny = p->n[1];
    p->pitch[0] = (nx + 7) / 8 * 8;
    p->pitch[1] = (ny + 7) / 8 * 8;
    for (int a = 0; a < 2; ++a) {
      const int n = p->n[a];
      unsigned short* q = nullptr;  // bf16 storage
      if ((rc = plan_alloc(p, &q, 2 * (size_t)n * p->pitch[a])) != PS_OK) return rc;
      LGL_CU(cudaMemset(q, 0, sizeof(unsigned short) * 2 * (size_t)n * p->pitch[a]), "split D clear");
      LGL_CU(launch_split_matrix(p->D32[a], n, n, p->pitch[a], q, 0), "split D");
      p->Dsplit[a] = q;
    }
    unsigned short* fx = nullptr;
    unsigned short* fyt = nullptr;
    const size_t nfx = 2 * (size_t)p->nsolve * 4 * ny * p->pitch[0];
    const size_t nfy = 2 * (size_t)p->nsolve * 4 * nx * p->pitch[1];
    if ((rc = plan_alloc(p, &fx, nfx)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &fyt, nfy)) != PS_OK) return rc;
    LGL_CU(cudaMemset(fx, 0, sizeof(unsigned short) * nfx), "flux planes clear");
    LGL_CU(cudaMemset(fyt, 0, sizeof(unsigned short) * nfy), "flux planes clear");
    p->FX = fx;
    p->FYT = fyt;
    // A operands (128-row boxes): D_x and F_y^T; B operands (N-tile boxes): F_x and D_y
    p->nt_x = umma_n_tile(nx, p->nsolve * 4 * ny, 1);
    p->nt_y = umma_n_tile(nx, ny, p->nsolve * 4);
    const int nt = p->desc.umma_n_tile;
    if (nt != 0) {  // an explicit tile (autotuner)
      if (nt != 64 && nt != 128 && nt != 176 && nt != 256)
        return errorf(PS_ERR_INVALID, "umma_n_tile must be 0, 64, 128, 176 or 256 (got %d)", nt);
      p->nt_x = p->nt_y = nt;
    }
    int e = 0;
    if ((e = encode_split_map(&p->map_Dx, p->Dsplit[0], nx, nx, 1, p->pitch[0], 128)) != 0 ||
        (e = encode_split_map(&p->map_FX, p->FX, nx, p->nsolve * 4 * ny, 1, p->pitch[0], p->nt_x)) != 0 ||
        (e = encode_split_map(&p->map_FYT, p->FYT, ny, nx, p->nsolve * 4, p->pitch[1], 128)) != 0 ||
        (e = encode_split_map(&p->map_Dy, p->Dsplit[1], ny, ny, 1, p->pitch[1], p->nt_y)) != 0)
      return errorf(PS_ERR_CUDA, "tensor map encoding for the split contractions failed (%d)", e);
    LGL_CU(cudaDeviceSynchronize(), "split tables");
  }
  return PS_OK;
}

// 1D: whole steps (or the right-hand side) in k_lgl1d
int lgl1d_run(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
              float* rhs_out, cudaStream_t s) {
  Lgl1DArgs a{};
  a.U = U;
  a.solve_stride = p->ss(3);
  a.n = p->n[0];
  a.DT = p->lgl_DT;
  a.FT = p->lgl_FT;
  for (int i = 0; i < 6; ++i) a.bc.c[i] = p->desc.lgl_bc1d[i];
  a.nsteps = nsteps;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.gamma = (float)p->desc.gamma;
  a.rho_min = 1e-10f;  // 1D clamp floors (solver.py:32-59)
  a.p_min = 1e-12f;
  a.gx = (float)p->desc.gravity[0];
  a.filter_interval = p->desc.filter_interval;
  a.step_counter0 = (int)(p->step_counter % p->desc.filter_interval);
  a.t = d_t;
  a.tend = d_tend;
  a.cfl = (float)p->desc.cfl;
  a.hmin = (float)p->lgl_hmin;
  a.steps_done = (d_t != nullptr) ? p->steps_done : nullptr;
  a.rhs_out = rhs_out;
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  ProfScope prof(p, s, PS_KIND_STEP1D, 4.0 * p->cells * p->nsolve * 3 * 2);
  LGL_CU(launch_lgl1d(a, p->gemm == PS_GEMM_FP64, p->nsolve, s), "1D LGL kernel");
  if (rhs_out == nullptr && d_t == nullptr) p->step_counter += nsteps;
  return PS_OK;
}

// out = M f for nf fields (M^T given), through the 3-field scratch when in place
int lgl1d_apply(ps_plan p, const void* MT, float rowsum, const float* f, float* out, int nf, cudaStream_t s) {
  const bool fp64 = p->gemm == PS_GEMM_FP64;
  const int n = p->n[0];
  if (f != out) {
    LGL_CU(launch_lgl1d_apply(MT, fp64, f, out, n, nf, p->nsolve, (long)nf * n, rowsum, s), "1D LGL contraction");
    return PS_OK;
  }
  for (int f0 = 0; f0 < nf; ++f0) {  // field by field through F1 (one field of every solve)
    for (int z = 0; z < p->nsolve; ++z) {
      const float* src = f + ((long)z * nf + f0) * n;
      LGL_CU(launch_lgl1d_apply(MT, fp64, src, p->F1, n, 1, 1, n, rowsum, s), "1D LGL contraction");
      LGL_CU(cudaMemcpyAsync(out + ((long)z * nf + f0) * n, p->F1, sizeof(float) * n, cudaMemcpyDeviceToDevice, s),
             "contraction copy");
    }
  }
  return PS_OK;
}

int lgl_rhs(ps_plan p, const float* U, float* rhs, cudaStream_t s) {
  if (p->nd == 1) return lgl1d_run(p, const_cast<float*>(U), 0, 0.0, nullptr, nullptr, nullptr, rhs, s);
  // the reference applies the walls to U in place before the fluxes; here to
  // a copy, so U is left as given
  const size_t bytes = sizeof(float) * p->ss(4) * p->nsolve;
  LGL_CU(cudaMemcpyAsync(p->Us, U, bytes, cudaMemcpyDeviceToDevice, s), "state copy");
  float* E = p->Us + 3 * p->cells;
  LGL_CU(launch_eref_set(E, p->ss(4), p->nsolve, p->eref, s), "energy reference");
  LGL_CU(launch_energy_shift(E, p->cells, p->ss(4), p->nsolve, p->eref, -1.0f, s), "energy shift");
  return stage(p, p->Us, -1, nullptr, rhs, 0.0, nullptr, nullptr, s);
}

int lgl_steps(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
              cudaStream_t s) {
  int rc;
  if (p->nd == 1) return lgl1d_run(p, U, nsteps, dt, d_dt, d_t, d_tend, nullptr, s);
  const bool cfl = d_t != nullptr;
  const int* act = cfl ? p->active : nullptr;
  const double* dtp = cfl ? p->dt : d_dt;
  const long ssU = p->ss(4);
  float* E = U + 3 * p->cells;
  LGL_CU(launch_eref_set(E, ssU, p->nsolve, p->eref, s), "energy reference");
  LGL_CU(launch_energy_shift(E, p->cells, ssU, p->nsolve, p->eref, -1.0f, s), "energy shift");
  if (cfl) LGL_CU(launch_fill_int(p->active, p->nsolve, 1, s), "active reset");
  for (int it = 0; it < nsteps; ++it) {
    const bool due = (p->step_counter % p->desc.filter_interval) == 0;
    if (cfl) {
      // dt from the state as given, before the walls of the first stage
      // (solver.py:386-389 compute_dt, then step)
      LGL_CU(launch_speed(2, U, p->cells, ssU, p->nsolve, (float)p->desc.gamma, p->speed, s, p->eref),
             "wave speed");
      LGL_CU(launch_step_control(p->speed, p->desc.cfl, p->hmin(), d_t, d_tend, p->nsolve, p->dt, p->active, s),
             "step control");
    }
    // The CUDA-core y contraction reads its stage input along whole columns
    // while its epilogue writes the next stage input, so that stage's input
    // and output must differ: stages 1 and 2 alternate between Us and the
    // free upper half of G (the x contraction writes the lower half).  The
    // tensor-core path updates in a separate kernel after both contractions.
    float* const alt = tensor_cores(p) ? p->Us : p->G + 4 * p->cells * p->nsolve;
    for (int st = 0; st < 4; ++st) {
      if (p->desc.scheme == PS_SCHEME_RK2 && (st == 1 || st == 2)) continue;  // midpoint RK2
      float* in = (st == 0) ? U : (st == 2) ? alt : p->Us;
      float* out = (st == 1) ? alt : (st < 3) ? p->Us : U;
      if ((rc = stage(p, in, st, U, out, dt, dtp, act, s)) != PS_OK) return rc;
    }
    if (due) {
      if (p->desc.filter_enabled && (rc = filter_state(p, U, act, s)) != PS_OK) return rc;
      LGL_CU(launch_lgl_bc(U, p->n[0], p->n[1], ssU, p->nsolve, act, s), "LGL walls");
    }
    if (cfl) LGL_CU(launch_step_advance(d_t, p->dt, p->speed, p->active, p->steps_done, p->nsolve, s), "advance");
    p->step_counter += 1;
  }
  LGL_CU(launch_energy_shift(E, p->cells, ssU, p->nsolve, p->eref, 1.0f, s), "energy shift");
  return PS_OK;
}

int lgl_derivative(ps_plan p, int axis, const float* f, float* out, int nf, cudaStream_t s) {
  if (p->nd == 1) return lgl1d_apply(p, p->lgl_DT, 0.0f, f, out, nf, s);
  const long Z = (long)nf * p->nsolve;
  if (f != out) return contract(p, axis, false, f, out, Z, nullptr, 1, s);
  // in place: through the scratch G (8 nsolve fields) in chunks
  const long cap = 8L * p->nsolve;
  int rc;
  for (long z0 = 0; z0 < Z; z0 += cap) {
    const long zc = (Z - z0 < cap) ? Z - z0 : cap;
    if ((rc = contract(p, axis, false, f + z0 * p->cells, p->G, zc, nullptr, 1, s)) != PS_OK) return rc;
    LGL_CU(cudaMemcpyAsync(out + z0 * p->cells, p->G, sizeof(float) * zc * p->cells, cudaMemcpyDeviceToDevice, s),
           "derivative copy");
  }
  return PS_OK;
}

int lgl_filter(ps_plan p, const float* f, float* out, int nf, cudaStream_t s) {
  if (!p->desc.filter_enabled) {
    // the reference returns the input unchanged when the filter is off
    // (grid.py:1260-1267)
    if (f != out)
      LGL_CU(cudaMemcpyAsync(out, f, sizeof(float) * p->cells * nf * p->nsolve, cudaMemcpyDeviceToDevice, s),
             "filter copy");
    return PS_OK;
  }
  if (p->nd == 1) return lgl1d_apply(p, p->lgl_FT, 1.0f, f, out, nf, s);
  const long Z = (long)nf * p->nsolve;
  const long cap = 8L * p->nsolve;
  int rc;
  for (long z0 = 0; z0 < Z; z0 += cap) {
    const long zc = (Z - z0 < cap) ? Z - z0 : cap;
    if ((rc = contract(p, 0, true, f + z0 * p->cells, p->G, zc, nullptr, 1, s)) != PS_OK) return rc;
    if ((rc = contract(p, 1, true, p->G, out + z0 * p->cells, zc, nullptr, 1, s)) != PS_OK) return rc;
  }
  return PS_OK;
}

}  // namespace ps
