// C ABI of the step engine: plan construction (spectral tables, scratch) and
// the step / rhs / operator / reduction entry points declared in
// include/phrike_gb300.h.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/phrike_gb300.h"
#include "lgl_tc.cuh"
#include "adaptive.cuh"
#include "av.cuh"
#include "launch.cuh"
#include "lgl.cuh"
#include "lgl1d.cuh"
#include "mhd3d.cuh"
#include "plan.cuh"
#include "reduce.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char msg[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define PS_CU(expr, what)                      \
  do {                                         \
    cudaError_t _e = (expr);                   \
    if (_e != cudaSuccess) return cuda_fail(_e, what); \
  } while (0)

}  // namespace

namespace ps {
// Records `msg` as the thread's last error (read by ps_last_error) and
// returns `code`; for entry points implemented in other translation units.
int record_error(int code, const char* msg) {
  g_err = msg;
  return code;
}

int errorf(int code, const char* fmt, ...) {
  char msg[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  g_err = msg;
  return code;
}
}  // namespace ps

namespace {

using ps::ProfScope;

bool is_lgl(const ps_plan_desc* d) {
  for (int a = 0; a < d->ndim && a < 3; ++a)
    if (d->basis[a] == PS_BASIS_LEGENDRE) return true;
  return false;
}

// every axis has a length the power-of-two pencil kernels are compiled for
bool pow2_axes(const ps_plan_desc* d) {
  for (int a = 0; a < d->ndim && a < 3; ++a)
    if (d->ndim == 1 ? !ps::supported_n_1d(d->n[a]) : !ps::supported_n(d->n[a])) return false;
  return true;
}

// a Fourier grid with some other axis length: the mixed-radix passes
bool is_mr(const ps_plan_desc* d) { return !is_lgl(d) && !pow2_axes(d); }

// 2D Euler and 2D MHD on power-of-two grids from 256 rows: the last pass is
// split into the right-hand side and an elementwise stage update (the clamped
// last pass holds every component's right-hand side in registers and runs one
// CTA per SM at these lengths).  Chosen from the grid alone, so a solve gives
// the same bits alone and in a batch.  The MHD update repeats the clamped
// pass's stage arithmetic (accumulator form, then the clamp).
bool split2d_grid(const ps_plan_desc* d) {
  return d->ndim == 2 && (d->equations == PS_EQ_EULER || d->equations == PS_EQ_MHD) && !is_lgl(d) && !is_mr(d) &&
         d->n[1] >= 256;
}

// Fields of the split 2D right-hand side buffer.
int split2d_fields(const ps_plan_desc* d) { return d->equations == PS_EQ_MHD ? 8 : 4; }

// 3D Fourier Euler with gravity on power-of-two axes keeps a second stage
// input (plan.cuh Us2); the mixed-radix last pass reads every component of a
// point before writing it and needs none.
bool stage_buffer3d(const ps_plan_desc* d) {
  return d->ndim == 3 && d->equations == PS_EQ_EULER && !is_lgl(d) && !is_mr(d) &&
         (d->gravity[0] != 0.0 || d->gravity[1] != 0.0 || d->gravity[2] != 0.0);
}

int validate(const ps_plan_desc* d) {
  if (!d) return fail(PS_ERR_INVALID, "null descriptor");
  if (d->ndim < 1 || d->ndim > 3) return fail(PS_ERR_INVALID, "ndim must be 1, 2 or 3 (got %d)", d->ndim);
  if (d->scheme != PS_SCHEME_RK4 && d->scheme != PS_SCHEME_RK2)
    return fail(PS_ERR_INVALID, "scheme must be PS_SCHEME_RK4 or PS_SCHEME_RK2 (got %d)", d->scheme);
  if (is_lgl(d)) return ps::lgl_validate(d);
  if (d->equations == PS_EQ_MHD) {
    if (d->ndim == 3)
      for (int a = 0; a < 3; ++a)
        if (!ps::mhd3_supported_n(d->n[a]))
          return fail(PS_ERR_UNSUPPORTED, "3D MHD axis %d: N=%d not supported (powers of two 8..256)", a, d->n[a]);
    if (d->ndim == 1 && d->n[0] > 2048)
      return fail(PS_ERR_UNSUPPORTED, "1D MHD pencils are limited to 2048 points (got %d)", d->n[0]);
    if (!(d->mhd_resistivity >= 0.0) || !(d->mhd_viscosity >= 0.0) || !(d->mhd_cfl_diff > 0.0))
      return fail(PS_ERR_INVALID, "MHD resistivity and viscosity must be >= 0 and cfl_diff > 0");
    if (!(d->mhd_rho_min >= 0.0) || !(d->mhd_p_min >= 0.0))
      return fail(PS_ERR_INVALID, "MHD clamp floors must be non-negative");
  } else if (d->equations != PS_EQ_EULER) {
    return fail(PS_ERR_UNSUPPORTED, "equation set %d not supported", d->equations);
  }
  for (int a = 0; a < d->ndim; ++a) {
    if (d->basis[a] != PS_BASIS_FOURIER)
      return fail(PS_ERR_UNSUPPORTED, "axis %d: only the Fourier basis is supported by this plan type", a);
    const bool p2 = d->ndim == 1 ? ps::supported_n_1d(d->n[a]) : ps::supported_n(d->n[a]);
    if (!p2 && !ps::mr_axis_ok(d->n[a]))
      return fail(PS_ERR_UNSUPPORTED, "axis %d: N=%d not supported (2^a 3^b 5^c from 2 to 4096%s)", a, d->n[a],
                  d->ndim == 1 ? ", powers of two to 4096" : "");
    if (!(d->length[a] > 0.0)) return fail(PS_ERR_INVALID, "axis %d: length must be positive", a);
  }
  if (!(d->gamma > 1.0)) return fail(PS_ERR_INVALID, "gamma must exceed 1");
  if (d->filter_interval < 1) return fail(PS_ERR_INVALID, "filter_interval must be >= 1");
  if (is_mr(d)) {
    if (d->equations != PS_EQ_EULER)
      return fail(PS_ERR_UNSUPPORTED, "MHD plans need power-of-two axes (8..1024; 2048 in 1D)");
    if (d->av_mode != PS_AV_OFF)
      return fail(PS_ERR_UNSUPPORTED, "artificial viscosity needs power-of-two axes");
  }
  if (d->av_mode != PS_AV_OFF) {
    if (d->av_mode != PS_AV_SENSOR && d->av_mode != PS_AV_CONSTANT)
      return fail(PS_ERR_INVALID, "av_mode must be PS_AV_OFF, PS_AV_SENSOR or PS_AV_CONSTANT");
    if (d->ndim == 3 || d->equations != PS_EQ_EULER)
      return fail(PS_ERR_UNSUPPORTED,
                  "artificial viscosity is defined for 1D/2D Euler (the reference's 3D solver passes none)");
    if (d->av_sensor < PS_AV_Q_DENSITY || d->av_sensor > PS_AV_Q_SPEED)
      return fail(PS_ERR_INVALID, "av_sensor out of range");
    if (d->ndim == 2 && d->av_sensor == PS_AV_Q_SPEED)
      return fail(PS_ERR_UNSUPPORTED, "the 2D velocity-magnitude sensor is not supported");
  }
  return PS_OK;
}

ps::AVParams av_params(const ps_plan_desc* d) {
  ps::AVParams a{};
  a.mode = d->av_mode;
  a.sensor = d->av_sensor;
  a.nu_max = (float)d->av_nu_max;
  a.nu_const = (float)d->av_nu_constant;
  a.s_ref = (float)d->av_s_ref;
  a.s_min = (float)d->av_s_min;
  a.p = (float)d->av_p;
  a.eps = (float)d->av_epsilon;
  for (int c = 0; c < 5; ++c) a.w[c] = (float)d->av_weight[c];
  return a;
}

size_t scratch_fields(int nd, bool mhd = false) {
  // G + AB + acc + Us (+ 1D flux); MHD: G (16) + acc + Us + half spectra (~2);
  // 3D MHD: three 8-field flux blocks + acc + Us + 3 half spectra (~3)
  if (nd == 1) return 3;
  if (mhd && nd == 3) return 24 + 8 + 8 + 4;
  if (mhd) return 16 + 8 + 8 + 3;
  if (nd == 2) return 8 + 4 + 4;
  return 15 + 10 + 5 + 5;
}

// Spectral tables of one axis in float64, stored as float (grid.py:47-63 for
// the mask and filter; wavenumbers 2 pi fftfreq(N, L/N), grid.py:255-257).
void build_axis(int N, double L, int dealias, int fon, int fp, double falpha, std::vector<float>& P,
                std::vector<float>& d, std::vector<float2>& twf, std::vector<float2>& twi) {
  P.resize(N);
  d.resize(N);
  twf.resize(N);
  twi.resize(N);
  const double kmax = N / 2;  // max |fftfreq(N) * N| for even N
  for (int k = 0; k < N; ++k) {
    const int kk = (k < N / 2) ? k : k - N;  // fftfreq ordering, index N/2 -> -N/2
    const double ak = fabs((double)kk);
    double m = (!dealias || ak <= (double)(N / 3)) ? 1.0 : 0.0;
    if (fon) m *= exp(-falpha * pow(ak / (kmax > 1.0 ? kmax : 1.0), fp));
    P[k] = (float)(m / N);
    const double kphys = 2.0 * M_PI * kk / L;
    d[k] = (k == N / 2) ? 0.0f : (float)(kphys * m / N);
  }
  // pencil FFT twiddles (layouts of fft_pencil.cuh): N <= 256 two-step
  // pencils with A threads x B points; N > 256 groups of 256-point pencils
  const int base = (N > 256) ? 256 : N;
  const int A = (base == 8) ? 2 : (base == 16 || base == 32) ? 4 : (base == 64 || base == 128) ? 8 : 16;
  const int B = base / A;
  for (int k2 = 0; k2 < B; ++k2)
    for (int n1 = 0; n1 < A; ++n1) {
      const double ang = -2.0 * M_PI * (double)((long)n1 * k2 % base) / base;
      twf[k2 * A + n1] = make_float2((float)cos(ang), (float)sin(ang));
      twi[n1 * B + k2] = make_float2((float)cos(ang), (float)-sin(ang));
    }
  for (int g = 1; g < N / 256; ++g)  // group twiddles W_N^{g k}, k < 256
    for (int k = 0; k < 256; ++k) {
      const double ang = -2.0 * M_PI * (double)((long)g * k % N) / N;
      twf[256 * g + k] = make_float2((float)cos(ang), (float)sin(ang));
      twi[256 * g + k] = make_float2((float)cos(ang), (float)-sin(ang));
    }
}

template <typename Tp>
int dalloc(ps_plan p, Tp** ptr, size_t count) {
  return ps::plan_alloc(p, ptr, count);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// libcuda link needed).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

}  // namespace

namespace ps {
// Plan descriptor checks shared by ps_plan_create / ps_batch_create and the
// allocation-free ps_rhs_static.
int validate_desc(const ps_plan_desc* d) { return validate(d); }

// Columns per strided-pass tile of a 2D Fourier grid (nx, ny: points along x
// and y): the widest of 16, 8, 4 that still gives about two CTAs per SM
// (small grids get more, narrower CTAs).  2D Euler: the clamped last pass
// runs at ~168 registers with 128-thread CTAs (8 columns of 16-thread pencils
// at N <= 256) and three CTAs per SM; at 512 points 8 columns (256 threads,
// 230 registers, one CTA per SM) move whole 32-byte sectors and measured
// 12% faster than 4 on a batch of sixteen 512^2 solves (194 vs 220 us); 4
// columns from 1024 up.  The 8-component MHD last pass takes at most 8
// columns from 512 rows up.
int tile_cols_2d(int nx, int ny, int nsolve, bool mhd) {
  const int cap = mhd ? ((ny >= 1024) ? 8 : 16) : ((ny >= 1024) ? 4 : (ny >= 256) ? 8 : 16);
  int tc = 4;
  for (int T = cap; T >= 4; T /= 2) {
    if ((long)((nx + T - 1) / T) * nsolve >= 2L * 148) {
      tc = T;
      break;
    }
  }
  if (mhd && ny >= 512 && tc > 8) tc = 8;
  return tc;
}

// 4-D map over a [nf][Nz][Ny][Nx] float32 buffer (n = {Nx, Ny, Nz}) with the
// tile box of the TMA strided passes for pencils along `axis` (1 = y, 2 = z).
// Host-only: fills the 128-byte map, allocates nothing.
int encode_field_map(CUtensorMap* m, const float* base, const int n[3], int nf, int axis, int tcols) {
  auto fn = encode_fn();
  if (!fn) return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const int naxis = n[axis];
  const int T = (tcols > 0) ? tcols : (naxis >= 1024) ? 8 : 16;
  const cuuint32_t rows = (cuuint32_t)(naxis < 256 ? naxis : 256);
  const cuuint64_t cells = (cuuint64_t)n[0] * n[1] * n[2];
  const cuuint64_t dims[4] = {(cuuint64_t)n[0], (cuuint64_t)n[1], (cuuint64_t)n[2], (cuuint64_t)nf};
  const cuuint64_t strides[3] = {(cuuint64_t)n[0] * 4, (cuuint64_t)n[0] * n[1] * 4, cells * 4};
  const cuuint32_t box[4] = {(cuuint32_t)T, axis == 1 ? rows : 1u, axis == 2 ? rows : 1u, 1u};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PS_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return PS_OK;
}
}  // namespace ps

namespace {


// maps over the batch: a buffer of nsolve solves x nf fields is nsolve*nf fields
int make_map(CUtensorMap* m, const float* base, const ps_plan_s* p, int nf, int axis) {
  return ps::encode_field_map(m, base, p->n, p->nsolve * nf, axis, p->tcols);
}

// maps of the caller's state pointer (re-encoded when the pointer changes)
int state_maps(ps_plan p, const float* U) {
  if (U == p->map_U_ptr) return PS_OK;
  int rc;
  const int last_axis = (p->nd == 3) ? 2 : 1;
  if ((rc = make_map(&p->map_U_last, U, p, p->nc, last_axis)) != PS_OK) return rc;
  p->map_U_ptr = U;
  return PS_OK;
}

ps::StridedGeom geom_y(const ps_plan_s* p) {
  // pencils along y: axis stride Nx, outer slabs z (stride Nx*Ny)
  return ps::StridedGeom{p->n[0], (long)p->n[0], (long)p->n[0] * p->n[1], p->n[2]};
}
ps::StridedGeom geom_z(const ps_plan_s* p) {
  // pencils along z: axis stride Nx*Ny, outer rows y (stride Nx)
  return ps::StridedGeom{p->n[0], (long)p->n[0] * p->n[1], (long)p->n[0], p->n[1]};
}

// One-axis operator on nf fields per solve (P, D or complementary P), axis 0 = x.
// One-axis operator (deriv: 0 P, 1 D, 2 Laplacian factor L, 3 raw second derivative)
// on nf fields.  ss_in (axis 0 only): solve stride of `in` when it is a field
// subset of a wider state (0: the nf-field stride of `out`).
int apply_op(ps_plan p, int axis, const float* in, float* out, int nf, int deriv, float scale, cudaStream_t s,
             bool complement = false, const int* active = nullptr, long ss_in = 0) {
  ProfScope prof(p, s, PS_KIND_OP, 8.0 * nf * p->cells * p->nsolve);
  if (p->mr) return ps::mr_apply_op(p, axis, in, out, nf, deriv, scale, complement, active, ss_in, s);
  cudaError_t e;
  const float kunit = (float)(2.0 * M_PI / p->desc.length[axis]);
  if (axis != 0 && ss_in != 0) return fail(PS_ERR_INVALID, "field-subset input is supported along x only");
  if (axis == 0) {
    ps::OpArgs a{};
    a.kunit = kunit;
    a.ss_in = ss_in;
    a.active = active;
    a.in = in;
    a.out = out;
    a.nf = nf;
    a.fs = p->cells;
    a.ss = p->ss(nf);
    a.rows = p->rows() * p->nsolve;
    a.rps = p->rows();
    a.ax = p->ax(0);
    a.deriv = deriv;
    a.scale = scale;
    a.complement = complement ? 1 : 0;
    e = ps::dispatch_n_1d(p->n[0], [&](auto nc) { return ps::launch_op<decltype(nc)::value>(false, a, s); });
  } else {
    if (nf > 63) return fail(PS_ERR_INVALID, "at most 63 fields per operator call");
    CUtensorMap m;
    int rc = make_map(&m, in, p, nf, axis);
    if (rc != PS_OK) return rc;
    ps::OpTArgs a{};
    a.out = out;
    a.nf = nf;
    a.fs = p->cells;
    a.ss = p->ss(nf);
    a.active = active;
    a.nsolve = p->nsolve;
    a.g = (axis == 1) ? geom_y(p) : geom_z(p);
    a.axis = axis;
    a.ax = p->ax(axis);
    a.deriv = deriv;
    a.scale = scale;
    a.complement = complement ? 1 : 0;
    a.status = p->status;
    a.tcols = (p->nd == 2) ? p->tcols : 0;
    a.kunit = kunit;
    e = ps::dispatch_n(p->n[axis], [&](auto nc) { return ps::launch_op_t<decltype(nc)::value>(m, a, s); });
  }
  if (e != cudaSuccess) return cuda_fail(e, "operator pass");
  return PS_OK;
}

int xfirst(ps_plan p, const float* U, float* Uw, float* speed, cudaStream_t s, bool shift_in = false,
           const int* active = nullptr) {
  ps::XFirstArgs a{};
  a.U = U;
  a.Uw = Uw;
  a.out = p->G;
  a.fs = p->cells;
  a.ssU = p->ss(p->nc);
  a.ssOut = p->ss(p->nd * p->nc);
  a.rows = p->rows() * p->nsolve;
  a.rps = p->rows();
  a.ax = p->ax(0);
  a.gamma = (float)p->desc.gamma;
  a.speed = speed;
  a.eref = p->eref;
  a.active = active;
  a.shift_in = shift_in ? 1 : 0;
  ProfScope prof(p, s, PS_KIND_X,
                 4.0 * p->cells * p->nsolve * (p->nc * (Uw ? 2 : 1) + p->nd * p->nc));
  if (p->mr) return ps::mr_xfirst(p, U, Uw, speed, shift_in, active, s);
  cudaError_t e = ps::dispatch_n(p->n[0], [&](auto nc) {
    return ps::launch_xfirst<decltype(nc)::value>(p->nd, a, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "x pass");
  return PS_OK;
}

int ymid(ps_plan p, cudaStream_t s, const int* active) {
  ps::YMidTArgs a{};
  a.out = p->AB;
  a.fs = p->cells;
  a.ssOut = p->ss(10);
  a.nsolve = p->nsolve;
  a.g = geom_y(p);
  a.ax = p->ax(1);
  a.active = active;
  a.status = p->status;
  ProfScope prof(p, s, PS_KIND_Y, 4.0 * p->cells * p->nsolve * 25);
  if (p->mr) return ps::mr_ymid(p, active, s);
  cudaError_t e = ps::dispatch_n(p->n[1], [&](auto nc) {
    return ps::launch_ymid3_t<decltype(nc)::value>(p->map_G_y, a, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "y pass");
  return PS_OK;
}

int last(ps_plan p, int stage, const float* Un, float* out, double dt, const double* d_dt, bool filter_last,
         cudaStream_t s, const int* active, const float* stage_in = nullptr) {
  int rc;
  if (p->mr) {
    const int st_words = (stage < 0) ? 1 : (stage == 0) ? 3 : (stage == 3) ? 2 : 4;
    ProfScope prof(p, s, PS_KIND_LAST, 4.0 * p->cells * p->nsolve * p->nc * (2 + st_words));
    return ps::mr_last(p, stage, Un, out, dt, d_dt, filter_last, active, s);
  }
  if (p->split2d && stage >= 0 && p->mhd) {
    // 2D MHD from 256 rows: the right-hand side into R, then the RK stage and
    // the MHD clamp elementwise, in the clamped pass's accumulator form
    const float* in = (stage == 0) ? Un : p->Us;
    if ((rc = last(p, -1, in, p->R2, 0.0, nullptr, false, s, active)) != PS_OK) return rc;
    ps::Mhd3UpdateArgs u{};
    u.F = p->R2;
    u.rhs_in = 1;
    u.dif = nullptr;
    u.Un = Un;
    u.acc = p->acc;
    u.out = out;
    u.cells = p->cells;
    u.nsolve = p->nsolve;
    u.stage = stage;
    u.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
    u.dt_dev = d_dt;
    u.dt = dt;
    u.gamma = (float)p->desc.gamma;
    u.rho_min = (float)p->desc.mhd_rho_min;  // SpectralSolverMHD._clamp floors (solver.py:876-877)
    u.p_min = (float)p->desc.mhd_p_min;
    u.active = active;
    // words per cell: R, U^n (not at stage 3), acc read (from stage 1), acc write (to stage 2), output
    const double words = 8.0 * ((stage == 0) ? 4 : (stage == 3) ? 3 : 5);
    ProfScope prof(p, s, PS_KIND_LAST, words * 4.0 * p->cells * p->nsolve);
    PS_CU(ps::launch_mhd3_update(u, s), "MHD stage update");
    return PS_OK;
  }
  if (p->split2d && stage >= 0) {
    // 2D Euler from 256 rows: the right-hand side of the stage input (with
    // gravity) into R, the RK stage and the clamp elementwise (increment-form
    // accumulator), then the y factor of the end-of-step filter
    const float* in = (stage == 0) ? Un : p->Us;
    if ((rc = last(p, -1, in, p->R2, 0.0, nullptr, false, s, active)) != PS_OK) return rc;
    ps::LglUpdateArgs u{};
    u.Gx = p->R2;
    u.Gy = nullptr;
    u.ksign = 1.0f;
    u.Un = Un;
    u.acc = p->acc;
    u.out = out;
    u.cells = p->cells;
    u.nsolve = p->nsolve;
    u.stage = stage;
    u.dt_dev = d_dt;
    u.dt = dt;
    u.gamma = (float)p->desc.gamma;
    u.rho_min = 1e-8f;  // _positivity_clamp_2d floors (solver.py:467)
    u.p_min = 1e-10f;
    u.eref = p->eref;
    u.active = active;
    u.gravity = 0;  // already in R
    u.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
    {
      const double words = (stage == 0) ? 16.0 : 20.0;
      ProfScope prof(p, s, PS_KIND_LAST, words * 4.0 * p->cells * p->nsolve);
      PS_CU(ps::launch_lgl_update(u, s), "stage update");
    }
    if (stage == 3 && filter_last && (rc = apply_op(p, 1, out, out, p->nc, 0, 1.0f, s, true, active)) != PS_OK)
      return rc;
    return PS_OK;
  }
  if ((rc = state_maps(p, Un)) != PS_OK) return rc;
  ps::LastTArgs a{};
  const int nc = p->nc;
  const CUtensorMap* mAB;
  if (p->nd == 3) {
    a.fa0 = 0;
    a.fb0 = 5;
    a.nfAB = 10;
    a.g = geom_z(p);
    a.axis = 2;
    a.ax = p->ax(2);
    mAB = &p->map_AB_z;
  } else {
    a.fa0 = 0;
    a.fb0 = nc;
    a.nfAB = 2 * nc;
    a.g = geom_y(p);
    a.axis = 1;
    a.ax = p->ax(1);
    mAB = &p->map_G_y;
  }
  a.acc = p->acc;
  a.out = out;
  a.fs = p->cells;
  a.ssAcc = p->ss(nc);
  a.ssOut = p->ss(nc);
  a.ssUn = p->ss(nc);
  a.active = active;
  a.nsolve = p->nsolve;
  a.stage = stage;
  a.Un = Un;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.gamma = (float)p->desc.gamma;
  // the 2D kernel clamps (solver.py:467-513); the 3D solver has none (1220-1230)
  a.rho_min = 1e-8f;  // _positivity_clamp_2d floors (solver.py:467)
  a.p_min = 1e-10f;
  if (p->mhd) {  // SpectralSolverMHD._clamp floors from mhd_config (solver.py:876-877)
    a.rho_min = (float)p->desc.mhd_rho_min;
    a.p_min = (float)p->desc.mhd_p_min;
    a.mhd = 1;
  }
  a.eref = p->eref;
  a.filter_last = filter_last ? 1 : 0;
  a.status = p->status;
  a.tcols = (p->nd == 2) ? p->tcols : 0;
  // the stage input: U^n at stage 0 and for a bare rhs
  a.Uin = (stage_in != nullptr) ? stage_in : (stage <= 0) ? Un : p->Us;
  a.gravity = 0;
  for (int d = 0; d < p->nd && d < 3; ++d) {
    a.grav[d] = (float)p->desc.gravity[d];
    if (p->desc.gravity[d] != 0.0) a.gravity = 1;
  }
  if (p->mhd) a.gravity = 0;
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  a.rhs2d = (p->split2d && stage < 0) ? 1 : 0;
  if (a.rhs2d) {  // fewer column tiles than two per SM: split the component pairs over gridDim.z
    const long tiles = (long)((a.g.ncol + p->tcols - 1) / p->tcols) * a.g.nouter * p->nsolve;
    const int npair = (nc + 1) / 2;
    a.pair_groups = 1;
    while (a.pair_groups < npair && tiles * a.pair_groups < 2L * 148 && npair % (2 * a.pair_groups) == 0)
      a.pair_groups *= 2;
  }
  const int naxis = (p->nd == 3) ? p->n[2] : p->n[1];
  // words per cell: 2*nc inputs, plus U^n / acc reads and acc / output writes
  const int st_words = (stage < 0) ? 1 : (stage == 0) ? 3 : (stage == 3) ? 2 : 4;
  ProfScope prof(p, s, PS_KIND_LAST, 4.0 * p->cells * p->nsolve * nc * (2 + st_words));
  cudaError_t e = ps::dispatch_n(naxis, [&](auto nc2) {
    return ps::launch_last_t<decltype(nc2)::value>(p->nd, *mAB, p->map_U_last, p->map_acc, a, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "last pass");
  return PS_OK;
}

bool filter_due(ps_plan p, long counter) {
  if (p->nd == 3) return true;  // every step (solver.py:1336)
  return (counter % p->desc.filter_interval) == 0;
}

int step_1d(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
            cudaStream_t s) {
  if (p->mr) return ps::mr_steps_1d(p, U, nsteps, dt, d_dt, d_t, d_tend, s);
  ps::Step1DArgs a{};
  a.U = U;
  a.solve_stride = p->ss(3);
  a.ax = p->ax(0);
  a.nsteps = nsteps;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.active = nullptr;
  a.gamma = (float)p->desc.gamma;
  a.rho_min = 1e-10f;  // _positivity_clamp floors (solver.py:32)
  a.p_min = 1e-12f;
  a.filter_interval = p->desc.filter_interval;
  a.step_counter0 = (int)(p->step_counter % p->desc.filter_interval);
  a.gx = (float)p->desc.gravity[0];
  a.t = d_t;
  a.tend = d_tend;
  a.cfl = (float)p->desc.cfl;
  a.dx = (float)(p->desc.length[0] / p->n[0]);
  a.steps_done = (d_t != nullptr) ? p->steps_done : nullptr;
  a.av = p->av;
  a.scratch = p->acc;  // N >= 4096: U^n and accumulator in global scratch
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  ProfScope prof(p, s, PS_KIND_STEP1D, 2.0 * 4.0 * p->cells * 3 * p->nsolve);
  cudaError_t e = ps::dispatch_n_1d(p->n[0], [&](auto nc) {
    return ps::launch_step1d<decltype(nc)::value>(a, p->nsolve, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "1D step");
  if (d_t == nullptr) p->step_counter += nsteps;
  return PS_OK;
}

// 2D artificial viscosity, before the stage's x pass: gradients of the stage
// input S (and of the sensor variable), nu and the viscous fluxes, then their
// x factors into the av_buf fields TA (D_x of the x fluxes) and TB (P_x of the
// y fluxes), which av_apply subtracts from the Euler x-pass outputs.
int av_prepass(ps_plan p, const float* S, cudaStream_t s, const int* act) {
  int rc;
  const long c = p->cells * p->nsolve;
  float* TA = p->av_buf;
  float* TB = TA + 4 * c;
  float* GX = TB + 4 * c;
  float* GY = GX + 4 * c;
  float* Q = GY + 4 * c;
  float* QA = Q + c;
  float* QB = QA + c;
  float* QX = QB + c;
  float* QY = QX + c;
  if ((rc = apply_op(p, 0, S, TA, 4, 1, 1.0f, s, false, act)) != PS_OK) return rc;  // D_x U
  if ((rc = apply_op(p, 0, S, TB, 4, 0, 1.0f, s, false, act)) != PS_OK) return rc;  // P_x U
  if ((rc = apply_op(p, 1, TA, GX, 4, 0, 1.0f, s, false, act)) != PS_OK) return rc; // dx1 U
  if ((rc = apply_op(p, 1, TB, GY, 4, 1, 1.0f, s, false, act)) != PS_OK) return rc; // dy1 U
  ps::AVFluxArgs f{};
  f.GX = GX;
  f.GY = GY;
  f.cells = p->cells;
  f.ssG = p->ss(4);
  f.ssS = p->ss(4);
  f.av = p->av;
  if (p->av.mode == PS_AV_SENSOR && p->av.sensor == PS_AV_Q_PRESSURE) {
    PS_CU(ps::launch_av_uy(S, p->cells, p->ss(4), p->nsolve, Q, s), "AV sensor variable");
    if ((rc = apply_op(p, 0, Q, QA, 1, 1, 1.0f, s, false, act)) != PS_OK) return rc;
    if ((rc = apply_op(p, 0, Q, QB, 1, 0, 1.0f, s, false, act)) != PS_OK) return rc;
    if ((rc = apply_op(p, 1, QA, QX, 1, 0, 1.0f, s, false, act)) != PS_OK) return rc;
    if ((rc = apply_op(p, 1, QB, QY, 1, 1, 1.0f, s, false, act)) != PS_OK) return rc;
    f.q = Q;
    f.qx = QX;
    f.qy = QY;
    f.ssQ = p->cells;
  } else {  // density: q = rho, its gradients are the first fields of GX, GY
    f.q = S;
    f.qx = GX;
    f.qy = GY;
    f.ssQ = p->ss(4);
  }
  PS_CU(ps::launch_av_flux(f, p->nsolve, s), "AV fluxes");
  if ((rc = apply_op(p, 0, GX, TA, 4, 1, 1.0f, s, false, act)) != PS_OK) return rc;  // D_x (w nu dx1 U)
  if ((rc = apply_op(p, 0, GY, TB, 4, 0, 1.0f, s, false, act)) != PS_OK) return rc;  // P_x (w nu dy1 U)
  return PS_OK;
}

int av_apply(ps_plan p, cudaStream_t s) {
  const long c = p->cells * p->nsolve;
  PS_CU(ps::launch_av_sub(p->G, p->ss(8), p->av_buf, p->av_buf + 4 * c, p->ss(4), p->cells, p->nsolve, s),
        "AV terms");
  return PS_OK;
}

// nsteps RK4 steps for 2D/3D batches.  Fixed step: dt (or per-solve d_dt).
// CFL mode (d_t != null): per-solve dt from the fused x-pass speed, solves
// stop at their end time.  The x axis of the end-of-step filter of step i is
// fused into the first x pass of step i+1.
int steps_nd(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
             cudaStream_t s) {
  int rc;
  const bool cfl = d_t != nullptr;
  const int* act = cfl ? p->active : nullptr;
  const double* dtp = cfl ? p->dt : d_dt;
  bool pending_px = false;
  float* UE = U + (long)(p->nc - 1) * p->cells;
  const long ssU = p->ss(p->nc);
  PS_CU(ps::launch_eref_set(UE, ssU, p->nsolve, p->eref, s), "energy reference");
  PS_CU(ps::launch_energy_shift(UE, p->cells, ssU, p->nsolve, p->eref, -1.0f, s), "energy shift");
  if (cfl) {
    PS_CU(cudaMemsetAsync(p->speed, 0, sizeof(float) * p->nsolve, s), "speed reset");
    PS_CU(ps::launch_fill_int(p->active, p->nsolve, 1, s), "active reset");
  }
  for (int it = 0; it < nsteps; ++it) {
    const bool filt = filter_due(p, p->step_counter);
    for (int stage = 0; stage < 4; ++stage) {
      if (p->desc.scheme == PS_SCHEME_RK2 && (stage == 1 || stage == 2)) continue;  // midpoint RK2
      // stage inputs U, Us, Us, Us (3D with gravity: U, Us, Us2, Us)
      const float* src = (stage == 0) ? U : (stage == 2 && p->Us2 != nullptr) ? p->Us2 : p->Us;
      float* Uw = (stage == 0 && pending_px) ? U : nullptr;
      if (p->av_buf && (rc = av_prepass(p, src, s, act)) != PS_OK) return rc;
      if ((rc = xfirst(p, src, Uw, (cfl && stage == 0) ? p->speed : nullptr, s, false, act)) != PS_OK) return rc;
      if (p->av_buf && (rc = av_apply(p, s)) != PS_OK) return rc;
      if (cfl && stage == 0)
        PS_CU(ps::launch_step_control(p->speed, p->desc.cfl, p->hmin(), d_t, d_tend, p->nsolve, p->dt, p->active, s),
              "step control");
      if (p->nd == 3 && (rc = ymid(p, s, act)) != PS_OK) return rc;
      float* out = (stage == 1 && p->Us2 != nullptr) ? p->Us2 : (stage < 3) ? p->Us : U;
      if ((rc = last(p, stage, U, out, dt, dtp, filt && stage == 3, s, act, src)) != PS_OK) return rc;
    }
    pending_px = false;
    if (filt) {
      if (p->nd == 3 && (rc = apply_op(p, 1, U, U, p->nc, 0, 1.0f, s, true, act)) != PS_OK) return rc;
      if (p->av_buf) {
        // the viscosity pre-pass of the next step reads the state, so the
        // filter's x factor is applied now instead of in the next x pass
        if ((rc = apply_op(p, 0, U, U, p->nc, 0, 1.0f, s, true, act)) != PS_OK) return rc;
      } else {
        pending_px = true;
      }
    }
    if (cfl)
      PS_CU(ps::launch_step_advance(d_t, p->dt, p->speed, p->active, p->steps_done, p->nsolve, s), "step advance");
    p->step_counter += 1;
  }
  if (pending_px) {
    if (act != nullptr) {
      // solves that took the last step still owe the x factor of its filter
      if ((rc = xfirst(p, U, U, nullptr, s, false, act)) != PS_OK) return rc;
    } else if ((rc = apply_op(p, 0, U, U, p->nc, 0, 1.0f, s, true)) != PS_OK) {
      return rc;
    }
  }
  PS_CU(ps::launch_energy_shift(UE, p->cells, ssU, p->nsolve, p->eref, 1.0f, s), "energy shift");
  return PS_OK;
}

// ---------------------------------------------------------------------------
// 2D ideal MHD (SpectralSolverMHD, solver.py:840-1049)
// ---------------------------------------------------------------------------
int xfirst_mhd(ps_plan p, const float* U, float* speed, cudaStream_t s, const int* active) {
  ps::MhdXArgs a{};
  a.U = U;
  a.out = p->G;
  a.fs = p->cells;
  a.ssU = p->ss(8);
  a.ssOut = p->ss(16);
  a.rows = p->rows() * p->nsolve;
  a.rps = p->rows();
  a.ax = p->ax(0);
  a.gamma = (float)p->desc.gamma;
  a.speed = speed;
  a.active = active;
  ProfScope prof(p, s, PS_KIND_X, 4.0 * p->cells * p->nsolve * (8 + 16));
  cudaError_t e = ps::dispatch_n(p->n[0], [&](auto nc) { return ps::launch_xfirst_mhd<decltype(nc)::value>(a, s); });
  if (e != cudaSuccess) return cuda_fail(e, "MHD x pass");
  if (p->dif_buf == nullptr) return PS_OK;
  // explicit viscosity (momenta, fields 1-3) and resistivity (B, fields 5-7):
  // T1 = L_x X and T2 = (-k_y^2) P_x X, folded into G so that the last pass adds
  // coef lap(X) (SpectralSolverMHD._compute_rhs, solver.py:942-954)
  const double coef[2] = {p->desc.mhd_viscosity, p->desc.mhd_resistivity};
  const int f0[2] = {1, 5};
  const long c3 = 3 * p->cells * p->nsolve;
  int rc;
  for (int g = 0; g < 2; ++g) {
    if (coef[g] == 0.0) continue;
    float* T1 = p->dif_buf + 2 * g * c3;
    float* T2 = T1 + c3;
    const float* X = U + (long)f0[g] * p->cells;
    if ((rc = apply_op(p, 0, X, T1, 3, 2, 1.0f, s, false, active, p->ss(8))) != PS_OK) return rc;
    if ((rc = apply_op(p, 0, X, T2, 3, 0, 1.0f, s, false, active, p->ss(8))) != PS_OK) return rc;
    if ((rc = apply_op(p, 1, T2, T2, 3, 3, 1.0f, s, false, active)) != PS_OK) return rc;
    PS_CU(ps::launch_mhd_diff_fold(p->G, p->ss(16), T1, T2, p->ss(3), p->cells, p->nsolve, f0[g], (float)coef[g], s),
          "MHD diffusion");
  }
  return PS_OK;
}

// Helmholtz projection of (Bx, By) in place (solve stride ss); E (nullable)
// updated with the thermal pressure held fixed.
int project(ps_plan p, float* Bx, float* By, float* E, long ss, const int* active, cudaStream_t s) {
  ps::ProjArgs a{};
  a.Bx = Bx;
  a.By = By;
  a.E = E;
  a.ss = ss;
  a.H = p->H;
  a.nx = p->n[0];
  a.ny = p->n[1];
  a.hx = p->n[0] / 2 + 1;
  a.nsolve = p->nsolve;
  a.kx0 = (float)(2.0 * M_PI / p->desc.length[0]);
  a.ky0 = (float)(2.0 * M_PI / p->desc.length[1]);
  a.active = active;
  // bytes: read B (2), write 2 half spectra; read/write them; read B (+E), write B (+E)
  ProfScope prof(p, s, PS_KIND_OP, 4.0 * p->cells * p->nsolve * (2 + 2 + 4 + 2 + (E ? 4 : 2)));
  a.ax = p->ax(0);
  cudaError_t e = ps::dispatch_n(p->n[0], [&](auto nc) { return ps::launch_proj_xf<decltype(nc)::value>(a, s); });
  if (e != cudaSuccess) return cuda_fail(e, "projection x forward");
  a.ax = p->ax(1);
  e = ps::dispatch_n(p->n[1], [&](auto nc) { return ps::launch_proj_y<decltype(nc)::value>(a, s); });
  if (e != cudaSuccess) return cuda_fail(e, "projection y");
  a.ax = p->ax(0);
  e = ps::dispatch_n(p->n[0], [&](auto nc) { return ps::launch_proj_xi<decltype(nc)::value>(a, s); });
  if (e != cudaSuccess) return cuda_fail(e, "projection x inverse");
  return PS_OK;
}

// 3D Helmholtz projection of (Bx, By, Bz) in place (solve stride ss); E
// (nullable) updated at fixed thermal pressure (grid.py:1649-1684,
// solver.py:966-986)
int project3(ps_plan p, float* Bx, float* By, float* Bz, float* E, long ss, const int* active, cudaStream_t s) {
  ps::Proj3Args a{};
  a.B[0] = Bx;
  a.B[1] = By;
  a.B[2] = Bz;
  a.E = E;
  a.ss = ss;
  a.H = p->H;
  a.nx = p->n[0];
  a.ny = p->n[1];
  a.nz = p->n[2];
  a.hx = p->n[0] / 2 + 1;
  a.nsolve = p->nsolve;
  a.k0x = (float)(2.0 * M_PI / p->desc.length[0]);
  a.k0y = (float)(2.0 * M_PI / p->desc.length[1]);
  a.k0z = (float)(2.0 * M_PI / p->desc.length[2]);
  a.active = active;
  // bytes: read B (3), write/read/write/read/write/read the half spectra (~3 each), write B (+E)
  ProfScope prof(p, s, PS_KIND_OP, 4.0 * p->cells * p->nsolve * (3 + 6 * 3 + 3 + (E ? 2 : 0)));
  cudaError_t e;
  a.ax = p->ax(0);
  if ((e = ps::launch_proj3_xf(p->n[0], a, s)) != cudaSuccess) return cuda_fail(e, "3D projection x forward");
  a.ax = p->ax(1);
  if ((e = ps::launch_proj3_y(p->n[1], false, a, s)) != cudaSuccess) return cuda_fail(e, "3D projection y forward");
  a.ax = p->ax(2);
  if ((e = ps::launch_proj3_z(p->n[2], a, s)) != cudaSuccess) return cuda_fail(e, "3D projection z");
  a.ax = p->ax(1);
  if ((e = ps::launch_proj3_y(p->n[1], true, a, s)) != cudaSuccess) return cuda_fail(e, "3D projection y inverse");
  a.ax = p->ax(0);
  if ((e = ps::launch_proj3_xi(p->n[0], a, s)) != cudaSuccess) return cuda_fail(e, "3D projection x inverse");
  return PS_OK;
}

int project_state(ps_plan p, float* U, const int* active, cudaStream_t s) {
  if (!p->desc.mhd_divergence_clean) return PS_OK;  // divergence_clean "none"
  if (p->nd == 3)
    return project3(p, U + 5 * p->cells, U + 6 * p->cells, U + 7 * p->cells, U + 4 * p->cells, p->ss(8), active, s);
  if (p->nd == 1) {
    PS_CU(ps::launch_project_mhd1d(U, p->cells, p->ss(8), p->nsolve, active, s), "1D projection");
    return PS_OK;
  }
  return project(p, U + 5 * p->cells, U + 6 * p->cells, U + 4 * p->cells, p->ss(8), active, s);
}

// Fixed dt or CFL steps: every stage the x pass, the last pass with the MHD
// clamp and (project_each_substage) the projection; after a step, at the
// filter cadence, the spectral filter then the projection (solver.py:988-1049).
// 1D MHD: whole steps in k_mhd1d (rhs_out non-null: the right-hand side only)
int mhd1d(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
          float* rhs_out, cudaStream_t s) {
  ps::Mhd1DArgs a{};
  a.U = U;
  a.solve_stride = p->ss(8);
  a.ax = p->ax(0);
  a.nsteps = nsteps;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.gamma = (float)p->desc.gamma;
  a.rho_min = (float)p->desc.mhd_rho_min;
  a.p_min = (float)p->desc.mhd_p_min;
  a.filter_interval = p->desc.filter_interval;
  a.step_counter0 = (int)(p->step_counter % p->desc.filter_interval);
  a.project_stages = p->desc.mhd_project_substages;
  a.clean = p->desc.mhd_divergence_clean;
  a.eta = (float)p->desc.mhd_resistivity;
  a.nu = (float)p->desc.mhd_viscosity;
  a.kunit = (float)(2.0 * M_PI / p->desc.length[0]);
  a.t = d_t;
  a.tend = d_tend;
  a.cfl = (float)p->desc.cfl;
  a.dx = (float)(p->desc.length[0] / p->n[0]);
  a.dt_cap = p->dt_diff();
  a.steps_done = (d_t != nullptr) ? p->steps_done : nullptr;
  a.scratch = p->acc;
  a.rhs_out = rhs_out;
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  ProfScope prof(p, s, PS_KIND_STEP1D, 4.0 * p->cells * p->nsolve * 8 * 2);
  cudaError_t e = ps::dispatch_n_1d(p->n[0], [&](auto nn) { return ps::launch_mhd1d<decltype(nn)::value>(a, p->nsolve, s); });
  if (e != cudaSuccess) return cuda_fail(e, "1D MHD kernel");
  if (rhs_out == nullptr && d_t == nullptr) p->step_counter += nsteps;
  return PS_OK;
}

// 3D MHD stage: the flux kernel (with the CFL speed on request), the nine
// operator passes dx1 Fx, dy1 Fy, dz1 Fz (and the nine of the three
// Laplacian blocks with explicit diffusion), then the update kernel: stage
// < 0 writes the right-hand side to out, else the RK stage with the clamp.
// control: after the flux kernel, the device CFL step control (solver.py:1018-1034).
int mhd3_stage(ps_plan p, const float* src, int stage, const float* Un, float* out, double dt, const double* dtp,
               float* speed, bool control, double* d_t, const double* d_tend, cudaStream_t s, const int* act) {
  int rc;
  const bool dif = p->dif_buf != nullptr;
  ps::Mhd3FluxArgs f{};
  f.U = src;
  f.F = p->G;
  f.dif = dif ? p->dif_buf : nullptr;
  f.cells = p->cells;
  f.nsolve = p->nsolve;
  f.gamma = (float)p->desc.gamma;
  f.speed = speed;
  f.active = act;
  {
    ProfScope prof(p, s, PS_KIND_X, 4.0 * p->cells * p->nsolve * (8 + 24 + (dif ? 18 : 0)));
    PS_CU(ps::launch_mhd3_flux(f, s), "3D MHD flux");
  }
  if (control)
    PS_CU(ps::launch_step_control(p->speed, p->desc.cfl, p->hmin(), d_t, d_tend, p->nsolve, p->dt, p->active, s,
                                  p->dt_diff()),
          "step control");
  const long c = p->cells * p->nsolve;
  for (int d = 0; d < 3; ++d) {  // block d: the flux along axis d, D on axis d and P on the others
    float* F = p->G + (long)d * 8 * c;
    for (int ax = 0; ax < 3; ++ax)
      if ((rc = apply_op(p, ax, F, F, 8, ax == d ? 1 : 0, 1.0f, s, false, act)) != PS_OK) return rc;
  }
  if (dif)
    for (int d = 0; d < 3; ++d) {  // L on axis d (-k^2 m s, Nyquist kept) and P on the others
      float* D = p->dif_buf + (long)d * 6 * c;
      for (int ax = 0; ax < 3; ++ax)
        if ((rc = apply_op(p, ax, D, D, 6, ax == d ? 2 : 0, 1.0f, s, false, act)) != PS_OK) return rc;
    }
  ps::Mhd3UpdateArgs u{};
  u.F = p->G;
  u.dif = dif ? p->dif_buf : nullptr;
  u.eta = (float)p->desc.mhd_resistivity;
  u.nu = (float)p->desc.mhd_viscosity;
  u.Un = Un;
  u.acc = p->acc;
  u.out = out;
  u.cells = p->cells;
  u.nsolve = p->nsolve;
  u.stage = stage;
  u.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  u.dt_dev = dtp;
  u.dt = dt;
  u.gamma = (float)p->desc.gamma;
  u.rho_min = (float)p->desc.mhd_rho_min;
  u.p_min = (float)p->desc.mhd_p_min;
  u.active = act;
  ProfScope prof(p, s, PS_KIND_LAST, 4.0 * p->cells * p->nsolve * (24 + (dif ? 18 : 0) + (stage < 0 ? 8 : 32)));
  PS_CU(ps::launch_mhd3_update(u, s), "3D MHD update");
  return PS_OK;
}

int steps_mhd(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
              cudaStream_t s) {
  int rc;
  if (p->nd == 1) return mhd1d(p, U, nsteps, dt, d_dt, d_t, d_tend, nullptr, s);
  const bool cfl = d_t != nullptr;
  const int* act = cfl ? p->active : nullptr;
  const double* dtp = cfl ? p->dt : d_dt;
  if (cfl) {
    PS_CU(cudaMemsetAsync(p->speed, 0, sizeof(float) * p->nsolve, s), "speed reset");
    PS_CU(ps::launch_fill_int(p->active, p->nsolve, 1, s), "active reset");
  }
  for (int it = 0; it < nsteps; ++it) {
    const bool due = (p->step_counter % p->desc.filter_interval) == 0;
    for (int stage = 0; stage < 4; ++stage) {
      if (p->desc.scheme == PS_SCHEME_RK2 && (stage == 1 || stage == 2)) continue;  // midpoint RK2
      const float* src = (stage == 0) ? U : p->Us;
      float* out = (stage < 3) ? p->Us : U;
      if (p->nd == 3) {
        const bool ctl = cfl && stage == 0;
        if ((rc = mhd3_stage(p, src, stage, U, out, dt, dtp, ctl ? p->speed : nullptr, ctl, d_t, d_tend, s, act)) !=
            PS_OK)
          return rc;
        if (p->desc.mhd_project_substages && (rc = project_state(p, out, act, s)) != PS_OK) return rc;
        continue;
      }
      if ((rc = xfirst_mhd(p, src, (cfl && stage == 0) ? p->speed : nullptr, s, act)) != PS_OK) return rc;
      if (cfl && stage == 0)
        PS_CU(ps::launch_step_control(p->speed, p->desc.cfl, p->hmin(), d_t, d_tend, p->nsolve, p->dt, p->active, s,
                                      p->dt_diff()),
              "step control");
      if ((rc = last(p, stage, U, out, dt, dtp, false, s, act)) != PS_OK) return rc;
      if (p->desc.mhd_project_substages && (rc = project_state(p, out, act, s)) != PS_OK) return rc;
    }
    if (due) {
      for (int ax = 0; ax < p->nd; ++ax)
        if ((rc = apply_op(p, ax, U, U, 8, 0, 1.0f, s, true, act)) != PS_OK) return rc;
      if ((rc = project_state(p, U, act, s)) != PS_OK) return rc;
    }
    if (cfl)
      PS_CU(ps::launch_step_advance(d_t, p->dt, p->speed, p->active, p->steps_done, p->nsolve, s), "step advance");
    p->step_counter += 1;
  }
  return PS_OK;
}

// ---------------------------------------------------------------------------
// Adaptive embedded RK (adaptive.py:23-437 driven by the run loops of
// solver.py).  1D: whole attempt loops in k_ark1d.  2D/3D and MHD: one launch
// sequence per attempt, every decision on the device (adaptive.cu).
// ---------------------------------------------------------------------------
// stage-slope storage, grown on demand (the old buffer is released)
int ark_ensure(ps_plan p, size_t floats) {
  if (p->ark_cap >= floats) return PS_OK;
  if (p->ark_K != nullptr) {
    cudaFree(p->ark_K);
    for (auto it = p->allocations.begin(); it != p->allocations.end(); ++it)
      if (*it == p->ark_K) {
        p->allocations.erase(it);
        break;
      }
    p->ark_K = nullptr;
    p->ark_cap = 0;
  }
  const int rc = dalloc(p, &p->ark_K, floats);
  if (rc == PS_OK) p->ark_cap = floats;
  return rc;
}

// nonzero a[i][j], j < i
ps::ArkComb ark_row(const ps::ArkTableau& t, int i) {
  ps::ArkComb c{};
  for (int j = 0; j < i; ++j)
    if (t.a[i][j] != 0.0) {
      c.idx[c.m] = j;
      c.c[c.m++] = t.a[i][j];
    }
  return c;
}

// U_high weights and the error weights bh - bl over the union of their supports
void ark_final_combs(const ps::ArkTableau& t, ps::ArkComb* high, ps::ArkComb* diff) {
  *high = ps::ArkComb{};
  *diff = ps::ArkComb{};
  for (int j = 0; j < t.stages; ++j) {
    const double e = t.bh[j] - t.bl[j];
    if (t.bh[j] == 0.0 && e == 0.0) continue;
    high->idx[high->m] = j;
    diff->idx[diff->m] = j;
    high->c[high->m++] = t.bh[j];
    diff->c[diff->m++] = e;
  }
}

// k = rhs(src) of the adaptive stages: Euler flux divergence plus gravity (no
// artificial viscosity, as the 2D/3D reference passes none), or the ideal MHD
// flux divergence
int ark_rhs(ps_plan p, const float* src, float* k, const int* act, cudaStream_t s) {
  int rc;
  if (p->mhd && p->nd == 3) return mhd3_stage(p, src, -1, src, k, 0.0, nullptr, nullptr, false, nullptr, nullptr, s, act);
  if (p->mhd) {
    if ((rc = xfirst_mhd(p, src, nullptr, s, act)) != PS_OK) return rc;
  } else {
    if ((rc = xfirst(p, src, nullptr, nullptr, s, false, act)) != PS_OK) return rc;
    if (p->nd == 3 && (rc = ymid(p, s, act)) != PS_OK) return rc;
  }
  return last(p, -1, src, k, 0.0, nullptr, false, s, act);
}

int run_adaptive_nd(ps_plan p, float* U, int nattempts, const ps::ArkTableau& tab, const ps::ArkCtrl& ctrl,
                    double* d_t, const double* d_tend, double* d_dt, const double* d_tout, int* d_counts,
                    cudaStream_t s) {
  int rc;
  const int nc = p->nc;
  const long n = (long)nc * p->cells;
  const long ssU = p->ss(nc);
  const long kstride = ssU * p->nsolve;
  if ((rc = ark_ensure(p, (size_t)tab.stages * kstride)) != PS_OK) return rc;
  const bool eprime = !p->mhd;  // Euler states run in the energy-perturbation form
  float* UE = U + (long)(nc - 1) * p->cells;
  if (eprime) {
    PS_CU(ps::launch_eref_set(UE, ssU, p->nsolve, p->eref, s), "energy reference");
    PS_CU(ps::launch_energy_shift(UE, p->cells, ssU, p->nsolve, p->eref, -1.0f, s), "energy shift");
  }
  const ps::ArkState st{d_t, d_tend, d_dt, d_tout, p->dt, p->active, p->ark_ok, p->ark_rej,
                        p->ark_err, p->ark_scale, d_counts, p->nsolve};
  ps::ArkComb high, diff;
  ark_final_combs(tab, &high, &diff);
  for (int it = 0; it < nattempts; ++it) {
    PS_CU(ps::launch_ark_begin(st, s), "adaptive begin");
    PS_CU(ps::launch_ark_scale(U, n, ssU, p->cells, eprime ? nc - 1 : -1, eprime ? p->eref : nullptr, st, s),
          "adaptive scale");
    for (int i = 0; i < tab.stages; ++i) {
      const float* src = U;
      if (i > 0) {
        PS_CU(ps::launch_ark_stage(U, p->ark_K, kstride, p->Us, n, ssU, ark_row(tab, i), st, s), "adaptive stage");
        src = p->Us;
      }
      if ((rc = ark_rhs(p, src, p->ark_K + (long)i * kstride, p->active, s)) != PS_OK) return rc;
    }
    PS_CU(ps::launch_ark_final(U, p->ark_K, kstride, p->acc, n, ssU, high, diff, st, s), "adaptive final");
    PS_CU(ps::launch_ark_decide(st, tab.order, ctrl, s), "adaptive controller");
    // post-step operator of accepted attempts: U <- filter(U_high) (Euler,
    // solver.py:683-689, 1375-1380); MHD then clamps and projects (1077-1079)
    if ((rc = apply_op(p, 0, p->acc, U, nc, 0, 1.0f, s, true, p->ark_ok)) != PS_OK) return rc;
    for (int ax = 1; ax < p->nd; ++ax)
      if ((rc = apply_op(p, ax, U, U, nc, 0, 1.0f, s, true, p->ark_ok)) != PS_OK) return rc;
    if (p->mhd) {
      PS_CU(ps::launch_ark_clamp_mhd(U, p->cells, ssU, p->nsolve, (float)p->desc.gamma, (float)p->desc.mhd_rho_min,
                                     (float)p->desc.mhd_p_min, p->ark_ok, s),
            "MHD clamp");
      if ((rc = project_state(p, U, p->ark_ok, s)) != PS_OK) return rc;
    }
  }
  if (eprime) PS_CU(ps::launch_energy_shift(UE, p->cells, ssU, p->nsolve, p->eref, 1.0f, s), "energy shift");
  return PS_OK;
}

int run_adaptive_1d(ps_plan p, float* U, int nattempts, const ps::ArkTableau& tab, const ps::ArkCtrl& ctrl,
                    double* d_t, const double* d_tend, double* d_dt, const double* d_tout, int* d_counts,
                    cudaStream_t s) {
  const int N = p->n[0];
  const long per = (N >= 4096 ? 3L * N : 0L) + (long)tab.stages * 3 * N;
  int rc;
  if ((rc = ark_ensure(p, (size_t)per * p->nsolve)) != PS_OK) return rc;
  ps::Ark1DArgs a{};
  a.U = U;
  a.solve_stride = p->ss(3);
  a.ax = p->ax(0);
  a.gamma = (float)p->desc.gamma;
  a.av = p->av;
  a.gx = (float)p->desc.gravity[0];
  a.nattempts = nattempts;
  a.tab = tab;
  a.ctrl = ctrl;
  a.t = d_t;
  a.tend = d_tend;
  a.dtp = d_dt;
  a.tout = d_tout;
  a.rej = p->ark_rej;
  a.counts = d_counts;
  a.scratch = p->ark_K;
  a.scratch_stride = per;
  cudaError_t e = ps::dispatch_n_1d(N, [&](auto nn) { return ps::launch_ark1d<decltype(nn)::value>(a, p->nsolve, s); });
  if (e != cudaSuccess) return cuda_fail(e, "1D adaptive kernel");
  return PS_OK;
}

int create(const ps_plan_desc* d, int nsolve, ps_plan* out) {
  int rc = validate(d);
  if (rc != PS_OK) return rc;
  if (!out) return fail(PS_ERR_INVALID, "null output handle");
  if (nsolve < 1) return fail(PS_ERR_INVALID, "nsolve must be >= 1");
  ps_plan p = new ps_plan_s();
  p->desc = *d;
  p->nd = d->ndim;
  p->mhd = d->equations == PS_EQ_MHD;
  p->nc = p->mhd ? 8 : d->ndim + 2;
  p->nsolve = nsolve;
  p->cells = 1;
  for (int a = 0; a < p->nd; ++a) {
    p->n[a] = d->n[a];
    p->cells *= d->n[a];
  }
  if ((long)nsolve * p->nc > (1L << 30)) return fail(PS_ERR_INVALID, "batch too large");
  auto cleanup = [&](int code) {
    ps_plan_destroy(p);
    return code;
  };
  const bool lgl = is_lgl(d);
  const bool mr = is_mr(d);
  for (int a = 0; a < p->nd && !lgl && !mr; ++a) {
    std::vector<float> P, dd;
    std::vector<float2> twf, twi;
    build_axis(p->n[a], d->length[a], d->dealias, d->filter_enabled, d->filter_p, d->filter_alpha, P, dd, twf, twi);
    const int N = p->n[a];
    if ((rc = dalloc(p, &p->P[a], N)) != PS_OK) return cleanup(rc);
    if ((rc = dalloc(p, &p->d[a], N)) != PS_OK) return cleanup(rc);
    if ((rc = dalloc(p, &p->twf[a], N)) != PS_OK) return cleanup(rc);
    if ((rc = dalloc(p, &p->twi[a], N)) != PS_OK) return cleanup(rc);
    cudaError_t e;
    if ((e = cudaMemcpy(p->P[a], P.data(), N * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(p->d[a], dd.data(), N * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(p->twf[a], twf.data(), N * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(p->twi[a], twi.data(), N * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess)
      return cleanup(cuda_fail(e, "table upload"));
  }
  const long c = p->cells * nsolve;
  if (p->nd == 1) {
    if ((rc = dalloc(p, &p->F1, 3 * c)) != PS_OK) return cleanup(rc);
    if (mr && ((rc = dalloc(p, &p->acc, 3 * c)) != PS_OK || (rc = dalloc(p, &p->Us, 3 * c)) != PS_OK))
      return cleanup(rc);
    if (!p->mhd && p->n[0] >= 4096 && (rc = dalloc(p, &p->acc, 6 * c)) != PS_OK) return cleanup(rc);
    // 1D MHD from 2048 points: U^n and the accumulator in global scratch
    if (p->mhd && p->n[0] >= 2048 && (rc = dalloc(p, &p->acc, 16 * c)) != PS_OK) return cleanup(rc);
  } else {
    const bool mhd3 = p->mhd && p->nd == 3;
    const int ng = mhd3 ? 24 : p->mhd ? 16 : (p->nd == 3) ? 15 : 8;
    if ((rc = dalloc(p, &p->G, ng * c)) != PS_OK) return cleanup(rc);
    const size_t hplanes = mhd3 ? (size_t)3 * p->n[2] * p->n[1] : (size_t)2 * p->n[1];
    if (p->mhd && (rc = dalloc(p, &p->H, hplanes * nsolve * (p->n[0] / 2 + 1))) != PS_OK) return cleanup(rc);
    if (p->mhd && (d->mhd_resistivity != 0.0 || d->mhd_viscosity != 0.0) &&
        (rc = dalloc(p, &p->dif_buf, (mhd3 ? 18 : 12) * c)) != PS_OK)
      return cleanup(rc);
    if (p->nd == 3 && !mhd3 && (rc = dalloc(p, &p->AB, 10 * c)) != PS_OK) return cleanup(rc);
    if ((rc = dalloc(p, &p->acc, p->nc * c)) != PS_OK) return cleanup(rc);
    if ((rc = dalloc(p, &p->Us, p->nc * c)) != PS_OK) return cleanup(rc);
    if (split2d_grid(d) && (rc = dalloc(p, &p->R2, split2d_fields(d) * c)) != PS_OK) return cleanup(rc);
    p->split2d = split2d_grid(d);
    if (stage_buffer3d(d) && (rc = dalloc(p, &p->Us2, p->nc * c)) != PS_OK) return cleanup(rc);
  }
  p->av = av_params(d);
  if (p->nd == 2 && !lgl && !mr) {
    const int cap = p->mhd ? ((p->n[1] >= 1024) ? 8 : 16) : ((p->n[1] >= 1024) ? 4 : (p->n[1] >= 256) ? 8 : 16);
    p->tcols = ps::tile_cols_2d(p->n[0], p->n[1], nsolve, p->mhd);
    if (d->tile_cols != 0) {  // explicit choice (autotuner): 4, 8 or 16, at most the cap
      const int maxT = (p->n[1] >= 512) ? 8 : cap;
      if ((d->tile_cols != 4 && d->tile_cols != 8 && d->tile_cols != 16) || d->tile_cols > maxT)
        return cleanup(fail(PS_ERR_INVALID, "tile_cols %d not allowed here (4..%d, powers of two)", d->tile_cols,
                            maxT));
      p->tcols = d->tile_cols;
    }
  }
  if (d->av_mode != PS_AV_OFF && p->nd == 2 && (rc = dalloc(p, &p->av_buf, 21 * c)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->speed, nsolve)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->eref, nsolve)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->dt, nsolve)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->active, nsolve)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->steps_done, nsolve)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->status, 1)) != PS_OK) return cleanup(rc);
  if ((rc = dalloc(p, &p->ark_rej, nsolve)) != PS_OK || (rc = dalloc(p, &p->ark_ok, nsolve)) != PS_OK ||
      (rc = dalloc(p, &p->ark_err, nsolve)) != PS_OK || (rc = dalloc(p, &p->ark_scale, nsolve)) != PS_OK)
    return cleanup(rc);
  if (cudaMemset(p->ark_rej, 0, sizeof(int) * nsolve) != cudaSuccess)
    return cleanup(cuda_fail(cudaGetLastError(), "adaptive state"));
  if (cudaMemset(p->eref, 0, sizeof(float) * nsolve) != cudaSuccess ||
      cudaMemset(p->speed, 0, sizeof(float) * nsolve) != cudaSuccess ||
      cudaMemset(p->steps_done, 0, sizeof(int) * nsolve) != cudaSuccess ||
      cudaMemset(p->status, 0, sizeof(int)) != cudaSuccess)
    return cleanup(fail(PS_ERR_CUDA, "scalar initialisation failed"));
  if (lgl) {
    if ((rc = ps::lgl_setup(p)) != PS_OK) return cleanup(rc);
  } else if (mr) {
    if ((rc = ps::mr_setup(p)) != PS_OK) return cleanup(rc);
  } else if (p->nd >= 2 && !(p->mhd && p->nd == 3)) {
    if ((rc = make_map(&p->map_G_y, p->G, p, p->mhd ? 16 : (p->nd == 3) ? 15 : 8, 1)) != PS_OK)
      return cleanup(rc);
    if (p->nd == 3 && (rc = make_map(&p->map_AB_z, p->AB, p, 10, 2)) != PS_OK) return cleanup(rc);
    if ((rc = make_map(&p->map_acc, p->acc, p, p->nc, (p->nd == 3) ? 2 : 1)) != PS_OK) return cleanup(rc);
  }
  *out = p;
  return PS_OK;
}

}  // namespace

extern "C" {

const char* ps_last_error(void) { return g_err.c_str(); }

const char* ps_version(void) { return "phrike_gb300 0.2.0 (sm_103a)"; }

int ps_plan_desc_init(ps_plan_desc* d, int ndim) {
  if (!d) return fail(PS_ERR_INVALID, "null descriptor");
  memset(d, 0, sizeof(*d));
  d->ndim = ndim;
  for (int a = 0; a < 3; ++a) {
    d->n[a] = 1;
    d->length[a] = 1.0;
    d->basis[a] = PS_BASIS_FOURIER;
  }
  d->equations = PS_EQ_EULER;
  d->gamma = 1.4;
  d->dealias = 1;
  d->filter_enabled = 0;
  d->filter_p = 8;
  d->filter_alpha = 36.0;
  d->filter_interval = 1;
  d->cfl = (ndim == 1) ? 0.4 : (ndim == 2) ? 0.3 : 0.25;
  d->av_mode = PS_AV_OFF;
  d->av_nu_max = 1e-3;  // ArtificialViscosityConfig defaults (artificial_viscosity.py:55-63)
  d->av_s_ref = 1.0;
  d->av_s_min = 0.1;
  d->av_p = 2.0;
  d->av_epsilon = 1e-12;
  for (int c = 0; c < 5; ++c) d->av_weight[c] = 1.0;
  d->mhd_rho_min = 1e-10;
  d->mhd_p_min = 1e-12;
  d->mhd_cfl_diff = 1.0;
  const int walls[6] = {0, 1, 0, 0, 1, 0};  // density copy, momentum zero, energy copy
  for (int i = 0; i < 6; ++i) d->lgl_bc1d[i] = walls[i];
  d->mhd_project_substages = 1;
  d->mhd_divergence_clean = 1;
  return PS_OK;
}

int ps_batch_scratch_bytes(const ps_plan_desc* d, int nsolve, size_t* bytes) {
  int rc = validate(d);
  if (rc != PS_OK) return rc;
  if (!bytes) return fail(PS_ERR_INVALID, "null output");
  if (nsolve < 1) return fail(PS_ERR_INVALID, "nsolve must be >= 1");
  long cells = 1;
  for (int a = 0; a < d->ndim; ++a) cells *= d->n[a];
  size_t tables = 0;
  for (int a = 0; a < d->ndim; ++a) tables += (size_t)d->n[a] * (2 * sizeof(float) + 2 * sizeof(float2));
  if (is_lgl(d)) tables = ps::lgl_scratch_bytes(d, nsolve);
  if (is_mr(d)) {  // P, d and the twiddles W_N^q per axis
    tables = 0;
    for (int a = 0; a < d->ndim; ++a) tables += (size_t)d->n[a] * (2 * sizeof(float) + sizeof(float2));
  }
  size_t fields = scratch_fields(d->ndim, d->equations == PS_EQ_MHD);
  if (is_mr(d) && d->ndim == 1) fields += 6;  // stage input and increments
  if (split2d_grid(d)) fields += split2d_fields(d);  // the 2D right-hand side
  if (stage_buffer3d(d)) fields += 5;                // the second 3D stage input
  if (d->av_mode != PS_AV_OFF && d->ndim == 2) fields += 21;
  const bool mhd = d->equations == PS_EQ_MHD;
  if (d->ndim == 1 && !mhd && d->n[0] >= 4096) fields += 6;  // global U^n and accumulator
  if (d->ndim == 1 && mhd && d->n[0] >= 2048) fields += 16;
  if (mhd && d->ndim == 2 && (d->mhd_resistivity != 0.0 || d->mhd_viscosity != 0.0)) fields += 12;
  if (mhd && d->ndim == 3 && (d->mhd_resistivity != 0.0 || d->mhd_viscosity != 0.0)) fields += 18;
  *bytes = fields * (size_t)cells * sizeof(float) * nsolve + tables + 64 + 32 * (size_t)nsolve;
  return PS_OK;
}

int ps_plan_scratch_bytes(const ps_plan_desc* d, size_t* bytes) { return ps_batch_scratch_bytes(d, 1, bytes); }

int ps_plan_create(const ps_plan_desc* d, ps_plan* out) { return create(d, 1, out); }

int ps_batch_create(const ps_plan_desc* d, int nsolve, ps_plan* out) { return create(d, nsolve, out); }

int ps_plan_destroy(ps_plan p) {
  if (!p) return PS_OK;
  for (void* q : p->allocations) cudaFree(q);
  for (auto& r : p->launches) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  for (cudaEvent_t e : p->event_pool) cudaEventDestroy(e);
  delete p;
  return PS_OK;
}

int ps_plan_ncomp(ps_plan p) { return p ? p->nc : -1; }

int ps_plan_tile_cols(ps_plan p) { return (p && p->nd == 2 && !p->lgl) ? p->tcols : 0; }

int ps_plan_nsolve(ps_plan p) { return p ? p->nsolve : -1; }

int ps_plan_steps_done(ps_plan p, int* host_steps) {
  if (!p || !host_steps) return fail(PS_ERR_INVALID, "null argument");
  PS_CU(cudaMemcpy(host_steps, p->steps_done, sizeof(int) * p->nsolve, cudaMemcpyDeviceToHost), "steps read");
  return PS_OK;
}

int ps_plan_status(ps_plan p, int* status) {
  if (!p || !status) return fail(PS_ERR_INVALID, "null argument");
  int v = 0;
  PS_CU(cudaMemcpy(&v, p->status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
  *status = v;
  return PS_OK;
}

int ps_profile_enable(ps_plan p, int enable) {
  if (!p) return fail(PS_ERR_INVALID, "null plan");
  p->profiling = enable != 0;
  return PS_OK;
}

int ps_profile_collect(ps_plan p, int nkinds, int* launches, double* ms, double* bytes) {
  if (!p || nkinds < 1 || !launches || !ms || !bytes) return fail(PS_ERR_INVALID, "null argument");
  for (int k = 0; k < nkinds; ++k) {
    launches[k] = 0;
    ms[k] = 0.0;
    bytes[k] = 0.0;
  }
  for (auto& r : p->launches) {
    float t = 0.0f;
    cudaError_t e = cudaEventSynchronize(r.stop);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, r.start, r.stop);
    if (e != cudaSuccess) return cuda_fail(e, "profile events");
    if (r.kind < nkinds) {
      launches[r.kind] += 1;
      ms[r.kind] += t;
      bytes[r.kind] += r.bytes;
    }
    p->event_pool.push_back(r.start);
    p->event_pool.push_back(r.stop);
  }
  p->launches.clear();
  return PS_OK;
}

int ps_rhs(ps_plan p, const float* U, float* rhs, void* stream) {
  if (!p || !U || !rhs) return fail(PS_ERR_INVALID, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  if (p->lgl) return ps::lgl_rhs(p, U, rhs, s);
  if (p->mhd) {
    if (p->nd == 1) return mhd1d(p, const_cast<float*>(U), 0, 0.0, nullptr, nullptr, nullptr, rhs, s);
    if (p->nd == 3) return mhd3_stage(p, U, -1, U, rhs, 0.0, nullptr, nullptr, false, nullptr, nullptr, s, nullptr);
    if ((rc = xfirst_mhd(p, U, nullptr, s, nullptr)) != PS_OK) return rc;
    return last(p, -1, U, rhs, 0.0, nullptr, false, s, nullptr);
  }
  if (p->nd == 1) {
    if (p->av.mode != PS_AV_OFF || p->desc.gravity[0] != 0.0)
      return fail(PS_ERR_UNSUPPORTED, "1D ps_rhs covers the flux divergence only (no gravity or viscosity terms)");
    PS_CU(ps::launch_flux1d(U, p->cells, p->ss(3), p->nsolve, (float)p->desc.gamma, p->F1, s), "1D flux");
    return apply_op(p, 0, p->F1, rhs, 3, 1, -1.0f, s);
  }
  PS_CU(ps::launch_eref_set(U + (long)(p->nc - 1) * p->cells, p->ss(p->nc), p->nsolve, p->eref, s),
        "energy reference");
  if (p->av_buf && (rc = av_prepass(p, U, s, nullptr)) != PS_OK) return rc;
  if ((rc = xfirst(p, U, nullptr, nullptr, s, true)) != PS_OK) return rc;
  if (p->av_buf && (rc = av_apply(p, s)) != PS_OK) return rc;
  if (p->nd == 3 && (rc = ymid(p, s, nullptr)) != PS_OK) return rc;
  return last(p, -1, U, rhs, 0.0, nullptr, false, s, nullptr);
}

int ps_step_rk4(ps_plan p, float* U, double dt, const double* d_dt, void* stream) {
  return ps_run_steps(p, U, 1, dt, d_dt, stream);
}

int ps_run_steps(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, void* stream) {
  if (!p || !U) return fail(PS_ERR_INVALID, "null argument");
  if (nsteps < 0) return fail(PS_ERR_INVALID, "nsteps must be >= 0");
  if (nsteps == 0) return PS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (p->lgl) return ps::lgl_steps(p, U, nsteps, dt, d_dt, nullptr, nullptr, s);
  if (p->mhd) return steps_mhd(p, U, nsteps, dt, d_dt, nullptr, nullptr, s);
  if (p->nd == 1) return step_1d(p, U, nsteps, dt, d_dt, nullptr, nullptr, s);
  return steps_nd(p, U, nsteps, dt, d_dt, nullptr, nullptr, s);
}

int ps_run_cfl(ps_plan p, float* U, int nsteps, double* d_t, const double* d_tend, void* stream) {
  if (!p || !U || !d_t || !d_tend) return fail(PS_ERR_INVALID, "null argument");
  if (nsteps < 0) return fail(PS_ERR_INVALID, "nsteps must be >= 0");
  if (nsteps == 0) return PS_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (p->lgl) return ps::lgl_steps(p, U, nsteps, 0.0, nullptr, d_t, d_tend, s);
  if (p->mhd) return steps_mhd(p, U, nsteps, 0.0, nullptr, d_t, d_tend, s);
  if (p->nd == 1) return step_1d(p, U, nsteps, 0.0, nullptr, d_t, d_tend, s);
  return steps_nd(p, U, nsteps, 0.0, nullptr, d_t, d_tend, s);
}

void ps_adaptive_desc_init(ps_adaptive_desc* ad) {
  if (!ad) return;
  ad->method = PS_ARK_RK45;
  ad->rtol = 1e-6;
  ad->atol = 1e-8;
  ad->safety_factor = 0.9;
  ad->min_dt_factor = 0.1;
  ad->max_dt_factor = 5.0;
  ad->max_rejections = 10;
}

int ps_run_adaptive(ps_plan p, float* U, int nattempts, const ps_adaptive_desc* ad, double* d_t,
                    const double* d_tend, double* d_dt, const double* d_tout, int* d_counts, void* stream) {
  if (!p || !U || !ad || !d_t || !d_tend || !d_dt) return fail(PS_ERR_INVALID, "null argument");
  if (nattempts < 0) return fail(PS_ERR_INVALID, "nattempts must be >= 0");
  if (p->lgl) return fail(PS_ERR_UNSUPPORTED, "adaptive stepping is not supported on LGL grids");
  if (p->mr && p->nd == 1)
    return fail(PS_ERR_UNSUPPORTED, "1D adaptive stepping needs a power-of-two grid (8..4096)");
  ps::ArkTableau tab;
  if (ps::ark_tableau(ad->method, &tab) != 0) return fail(PS_ERR_INVALID, "unknown adaptive method %d", ad->method);
  if (!(ad->rtol >= 0.0) || !(ad->atol >= 0.0) || !(ad->safety_factor > 0.0) || !(ad->min_dt_factor > 0.0) ||
      !(ad->max_dt_factor >= ad->min_dt_factor))
    return fail(PS_ERR_INVALID, "adaptive tolerances and factors out of range");
  if (nattempts == 0) return PS_OK;
  const ps::ArkCtrl ctrl{ad->rtol, ad->atol, ad->safety_factor, ad->min_dt_factor, ad->max_dt_factor,
                         ad->max_rejections};
  cudaStream_t s = (cudaStream_t)stream;
  if (p->nd == 1) return run_adaptive_1d(p, U, nattempts, tab, ctrl, d_t, d_tend, d_dt, d_tout, d_counts, s);
  return run_adaptive_nd(p, U, nattempts, tab, ctrl, d_t, d_tend, d_dt, d_tout, d_counts, s);
}

int ps_adaptive_reset(ps_plan p, void* stream) {
  if (!p) return fail(PS_ERR_INVALID, "null argument");
  PS_CU(cudaMemsetAsync(p->ark_rej, 0, sizeof(int) * p->nsolve, (cudaStream_t)stream), "adaptive reset");
  return PS_OK;
}

int ps_derivative(ps_plan p, int axis, const float* f, float* out, int nf, void* stream) {
  if (!p || !f || !out) return fail(PS_ERR_INVALID, "null argument");
  if (axis < 0 || axis >= p->nd) return fail(PS_ERR_INVALID, "axis %d out of range", axis);
  if (nf < 1) return fail(PS_ERR_INVALID, "nfields must be >= 1");
  cudaStream_t s = (cudaStream_t)stream;
  if (p->lgl) return ps::lgl_derivative(p, axis, f, out, nf, s);
  const float* src = f;
  int rc;
  for (int a = 0; a < p->nd; ++a) {
    if ((rc = apply_op(p, a, src, out, nf, a == axis ? 1 : 0, 1.0f, s)) != PS_OK) return rc;
    src = out;
  }
  return PS_OK;
}

int ps_filter(ps_plan p, const float* f, float* out, int nf, void* stream) {
  if (!p || !f || !out) return fail(PS_ERR_INVALID, "null argument");
  if (nf < 1) return fail(PS_ERR_INVALID, "nfields must be >= 1");
  cudaStream_t s = (cudaStream_t)stream;
  if (p->lgl) return ps::lgl_filter(p, f, out, nf, s);
  const float* src = f;
  int rc;
  for (int a = 0; a < p->nd; ++a) {
    if ((rc = apply_op(p, a, src, out, nf, 0, 1.0f, s, true)) != PS_OK) return rc;
    src = out;
  }
  return PS_OK;
}

int ps_lgl_build(int n, double length, double* d_nodes, double* d_weights, double* d_D, void* stream) {
  if (n < 2) return fail(PS_ERR_INVALID, "LGL grids need at least 2 nodes (got %d)", n);
  if (!(length > 0.0)) return fail(PS_ERR_INVALID, "length must be positive");
  if (d_D != nullptr && (d_nodes == nullptr || d_weights == nullptr))
    return fail(PS_ERR_INVALID, "the differentiation matrix needs the node and weight arrays");
  if (d_nodes == nullptr && d_weights == nullptr) return PS_OK;
  PS_CU(ps::launch_lgl_build(n, length, d_nodes, d_weights, d_D, nullptr, (cudaStream_t)stream), "LGL build");
  return PS_OK;
}

int ps_apply_boundary_conditions(ps_plan p, float* U, void* stream) {
  if (!p || !U) return fail(PS_ERR_INVALID, "null argument");
  if (!p->lgl) return PS_OK;  // periodic Fourier grids have none
  if (p->nd == 1) {
    ps::Bc1D bc;
    for (int i = 0; i < 6; ++i) bc.c[i] = p->desc.lgl_bc1d[i];
    PS_CU(ps::launch_lgl1d_bc(U, p->n[0], p->ss(3), p->nsolve, bc, nullptr, (cudaStream_t)stream),
          "1D boundary conditions");
    return PS_OK;
  }
  PS_CU(ps::launch_lgl_bc(U, p->n[0], p->n[1], p->ss(4), p->nsolve, nullptr, (cudaStream_t)stream), "LGL walls");
  return PS_OK;
}

int ps_axis_op(ps_plan p, int axis, int op, const float* f, float* out, int nf, void* stream) {
  if (!p || !f || !out) return fail(PS_ERR_INVALID, "null argument");
  if (p->lgl) return fail(PS_ERR_UNSUPPORTED, "one-axis spectral operators need a Fourier plan");
  if (axis < 0 || axis >= p->nd) return fail(PS_ERR_INVALID, "axis %d out of range", axis);
  if (op < PS_OP_P || op > PS_OP_L) return fail(PS_ERR_INVALID, "op must be PS_OP_P, PS_OP_D or PS_OP_L");
  if (nf < 1) return fail(PS_ERR_INVALID, "nf must be >= 1");
  return apply_op(p, axis, f, out, nf, op, 1.0f, (cudaStream_t)stream);
}

int ps_project_solenoidal_3d(ps_plan p, float* Bx, float* By, float* Bz, void* stream) {
  if (!p || !Bx || !By || !Bz) return fail(PS_ERR_INVALID, "null argument");
  if (p->lgl || p->nd != 3 || p->H == nullptr)
    return fail(PS_ERR_UNSUPPORTED, "the 3D Helmholtz projection needs a 3D Fourier MHD plan");
  return project3(p, Bx, By, Bz, nullptr, p->cells, nullptr, (cudaStream_t)stream);
}

int ps_project_solenoidal(ps_plan p, float* Bx, float* By, void* stream) {
  if (!p || !Bx || !By) return fail(PS_ERR_INVALID, "null argument");
  if (p->lgl || p->nd != 2 || p->H == nullptr)
    return fail(PS_ERR_UNSUPPORTED, "the Helmholtz projection needs a 2D Fourier MHD plan");
  return project(p, Bx, By, nullptr, p->cells, nullptr, (cudaStream_t)stream);
}

int ps_project_state(ps_plan p, float* U, void* stream) {
  if (!p || !U) return fail(PS_ERR_INVALID, "null argument");
  if (!p->mhd) return fail(PS_ERR_UNSUPPORTED, "ps_project_state needs a PS_EQ_MHD plan");
  return project_state(p, U, nullptr, (cudaStream_t)stream);
}

int ps_max_wave_speed(ps_plan p, const float* U, float* d_out, void* stream) {
  if (!p || !U || !d_out) return fail(PS_ERR_INVALID, "null argument");
  if (p->mhd) {
    if (p->nd == 1)
      PS_CU(ps::launch_speed_mhd1d(U, p->cells, p->ss(8), p->nsolve, (float)p->desc.gamma, d_out,
                                   (cudaStream_t)stream),
            "max wave speed");
    else if (p->nd == 3)
      PS_CU(ps::launch_speed_mhd3(U, p->cells, p->ss(8), p->nsolve, (float)p->desc.gamma, d_out,
                                  (cudaStream_t)stream),
            "max wave speed");
    else
      PS_CU(ps::launch_speed_mhd(U, p->cells, p->ss(8), p->nsolve, (float)p->desc.gamma, d_out,
                                 (cudaStream_t)stream),
            "max wave speed");
    return PS_OK;
  }
  PS_CU(ps::launch_speed(p->nd, U, p->cells, p->ss(p->nc), p->nsolve, (float)p->desc.gamma, d_out,
                         (cudaStream_t)stream),
        "max wave speed");
  return PS_OK;
}

int ps_conserved(ps_plan p, const float* U, double* d_out, void* stream) {
  if (!p || !U || !d_out) return fail(PS_ERR_INVALID, "null argument");
  if (p->mhd) {
    PS_CU(ps::launch_conserved_mhd(U, p->cells, p->ss(8), p->nsolve, p->desc.gamma, d_out, (cudaStream_t)stream),
          "conserved sums");
    return PS_OK;
  }
  PS_CU(ps::launch_conserved(p->nd, U, p->cells, p->ss(p->nc), p->nsolve, p->desc.gamma, d_out,
                             (cudaStream_t)stream),
        "conserved sums");
  return PS_OK;
}

}  // extern "C"
