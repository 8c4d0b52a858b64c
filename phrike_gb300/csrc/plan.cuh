// Plan object shared by the translation units of the C ABI (ps_api.cu for
// Fourier grids, lgl_plan.cu for LGL x LGL grids), launch profiling and
// small host helpers.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "../../include/phrike_gb300.h"
#include "mixed_radix.cuh"
#include "pass_common.cuh"

struct ps_plan_s {
  ps_plan_desc desc;
  int nd = 0;
  int nsolve = 1;  // independent solves of the same grid (a batch)
  int n[3] = {1, 1, 1};
  long cells = 0;  // cells of one solve
  int nc = 0;
  // per-axis spectral tables (device): P, d, twf, twi
  float* P[3] = {nullptr, nullptr, nullptr};
  float* d[3] = {nullptr, nullptr, nullptr};
  float2* twf[3] = {nullptr, nullptr, nullptr};
  float2* twi[3] = {nullptr, nullptr, nullptr};
  // scratch, [nsolve][nfields][cells] each
  float* G = nullptr;    // x-pass outputs (2D: 8 fields, 3D: 15)
  float* AB = nullptr;   // 3D y-pass outputs (10 fields)
  float* acc = nullptr;  // RK accumulator (nc fields)
  float* Us = nullptr;   // stage input (nc fields)
  float* F1 = nullptr;   // 1D flux for ps_rhs (3 fields)
  // 2D Euler from 256 rows: the last pass writes the right-hand side R (4
  // fields) and an elementwise kernel applies the RK stage and the clamp
  bool split2d = false;
  float* R2 = nullptr;
  // 3D Euler with gravity: a second stage input (nc fields).  The last pass
  // reads the stage input for the gravity source one component pair at a
  // time while it writes the next stage input, so stages 1 and 2 must not
  // share the buffer: stage 1 writes Us2, stage 2 reads it.
  float* Us2 = nullptr;
  // per-solve device scalars
  float* speed = nullptr;  // CFL wave speed maxima
  float* eref = nullptr;   // E_ref of the energy-perturbation form
  double* dt = nullptr;    // step sizes (CFL runs)
  int* active = nullptr;   // 1 while a solve advances (CFL runs)
  int* steps_done = nullptr;
  int* status = nullptr;   // device status word (PS_STATUS_* bits set by kernels)
  // TMA tensor maps of the plan buffers and of the last state pointer seen
  CUtensorMap map_G_y{};    // G, y pencils
  CUtensorMap map_AB_z{};   // AB, z pencils (3D)
  CUtensorMap map_acc{};    // acc, last-pass pencils
  const float* map_U_ptr = nullptr;
  CUtensorMap map_U_last{};  // state, last-pass pencils
  long step_counter = 0;
  int tcols = 0;  // 2D: columns per strided-pass tile (0: the default for the pencil length)
  std::vector<void*> allocations;
  // launch profiling: CUDA events around every pass launch
  struct LaunchRec {
    int kind;
    double bytes;
    cudaEvent_t start, stop;
  };
  bool profiling = false;
  std::vector<LaunchRec> launches;
  std::vector<cudaEvent_t> event_pool;

  // LGL x LGL grids (PS_BASIS_LEGENDRE on both axes); index 0 = x, 1 = y
  bool lgl = false;
  int gemm = PS_GEMM_FP32;        // precision of the derivative contractions
  double* lgl_x[2] = {nullptr, nullptr};  // nodes (ascending), float64
  double* lgl_w[2] = {nullptr, nullptr};  // quadrature weights on [-1, 1]
  double* D64[2] = {nullptr, nullptr};    // differentiation matrices [n][n]
  float* D32[2] = {nullptr, nullptr};
  double* F64[2] = {nullptr, nullptr};    // nodal filter matrices (filter on)
  float* F32[2] = {nullptr, nullptr};
  double lgl_hmin = 0.0;                  // smallest node spacing (CFL)
  void* lgl_DT = nullptr;                 // 1D: D^T and the nodal filter transposed (float or double)
  void* lgl_FT = nullptr;
  // artificial viscosity (1D in the step kernel; 2D through av_buf, 21 fields per solve)
  ps::AVParams av{};
  float* av_buf = nullptr;
  // adaptive embedded RK: per-solve controller state and the stage slopes
  int* ark_rej = nullptr;    // consecutive rejections
  int* ark_ok = nullptr;     // attempt accepted
  float* ark_err = nullptr;  // max |U_high - U_low|
  float* ark_scale = nullptr;
  float* ark_K = nullptr;    // allocated on first use: stages x state (1D N >= 4096: + U^n)
  size_t ark_cap = 0;        // floats in ark_K
  // 2D ideal MHD (PS_EQ_MHD): half spectra of the Helmholtz projection
  bool mhd = false;
  float2* H = nullptr;                    // [nsolve][2][ny][nx/2+1]
  float* dif_buf = nullptr;               // explicit diffusion: per group T1, T2 (3 fields each)
  // tensor-core split-bf16 contractions: hi/lo planes and their TMA maps
  int pitch[2] = {0, 0};                  // bf16 row pitch along x / y (multiple of 8)
  void* Dsplit[2] = {nullptr, nullptr};   // [2][n][pitch] of D_x, D_y
  void* FX = nullptr;                     // [2][nsolve*4*ny][pitch_x] x flux
  void* FYT = nullptr;                    // [2][nsolve*4][nx][pitch_y] transposed y flux
  CUtensorMap map_FX{}, map_Dx{}, map_Dy{}, map_FYT{};
  int nt_x = 0, nt_y = 0;                 // N tiles of the two contractions

  // Fourier axes of any 5-smooth length (mixed-radix passes, mr_plan.cu)
  bool mr = false;
  ps::MrAxis mrax[3] = {};
  // point evaluation: 0 auto, 1 exact interpolant, 2 NUFFT (nufft.cu, tables made on first use)
  int tracer_method = 0;
  bool nu_ready = false;
  ps::MrAxis nu_axn[3] = {}, nu_axm[3] = {};
  float* nu_s[3] = {nullptr, nullptr, nullptr};
  float* nu_g = nullptr;    // [3][2Nz][2Ny][2Nx] oversampled grid (real part)
  float2* nu_t1 = nullptr;  // x resampled
  float2* nu_t2 = nullptr;  // x and y resampled (3D)

  ps::AxisOps ax(int a) const { return ps::AxisOps{P[a], d[a], twf[a], twi[a]}; }
  long ss(int nf) const { return (long)nf * cells; }  // solve stride of an nf-field buffer
  int rows() const { return (int)(cells / n[0]); }     // x-pencil rows of one solve
  // parabolic CFL cap of explicit MHD diffusion: cfl_diff / (max(eta, nu)
  // k^2_max), k^2_max = sum over axes of (pi n / L)^2 (solver.py:916-929,
  // 1018-1034); 0 when there is no diffusion
  double dt_diff() const {
    const double dif = fmax(desc.mhd_resistivity, desc.mhd_viscosity);
    if (!mhd || !(dif > 0.0)) return 0.0;
    double k2 = 0.0;
    for (int a = 0; a < nd; ++a) {
      const double km = M_PI * n[a] / desc.length[a];
      k2 += km * km;
    }
    return desc.mhd_cfl_diff / (dif * k2);
  }
  double hmin() const {                                 // smallest grid spacing (CFL)
    if (lgl) return lgl_hmin;
    double h = desc.length[0] / n[0];
    for (int a = 1; a < nd; ++a) h = fmin(h, desc.length[a] / n[a]);
    return h;
  }
};

namespace ps {

// Thread-local last error (ps_last_error): formats, records, returns `code`.
int errorf(int code, const char* fmt, ...);
int record_error(int code, const char* msg);

// Launch profiling: a ProfScope records a start event before a pass launch
// and, when it goes out of scope, the stop event with the kind and the
// algorithmic bytes of the pass.
inline cudaEvent_t take_event(ps_plan p) {
  if (!p->event_pool.empty()) {
    cudaEvent_t e = p->event_pool.back();
    p->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}



struct ProfScope {
  ps_plan p;
  cudaStream_t s;
  int kind;
  double bytes;
  cudaEvent_t start = nullptr;
  ProfScope(ps_plan p_, cudaStream_t s_, int kind_, double bytes_) : p(p_), s(s_), kind(kind_), bytes(bytes_) {
    if (p->profiling) {
      start = take_event(p);
      cudaEventRecord(start, s);
    }
  }
  ~ProfScope() {
    if (p->profiling && start) {
      cudaEvent_t stop = take_event(p);
      cudaEventRecord(stop, s);
      p->launches.push_back({kind, bytes, start, stop});
    }
  }
};


template <typename Tp>
int plan_alloc(ps_plan p, Tp** ptr, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(Tp));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return errorf(PS_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(Tp), cudaGetErrorString(e));
  }
  p->allocations.push_back(q);
  *ptr = static_cast<Tp*>(q);
  return PS_OK;
}

// LGL x LGL plans (lgl_plan.cu)
int lgl_validate(const ps_plan_desc* d);
size_t lgl_scratch_bytes(const ps_plan_desc* d, int nsolve);
int lgl_setup(ps_plan p);
int lgl_rhs(ps_plan p, const float* U, float* rhs, cudaStream_t s);
int lgl_steps(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
              cudaStream_t s);
int lgl_derivative(ps_plan p, int axis, const float* f, float* out, int nf, cudaStream_t s);
int lgl_filter(ps_plan p, const float* f, float* out, int nf, cudaStream_t s);

// Fourier plans on the mixed-radix passes (mr_plan.cu)
bool mr_axis_ok(int n);
int mr_setup(ps_plan p);
int mr_apply_op(ps_plan p, int axis, const float* in, float* out, int nf, int deriv, float scale, bool complement,
                const int* active, long ss_in, cudaStream_t s);
int mr_xfirst(ps_plan p, const float* U, float* Uw, float* speed, bool shift_in, const int* active, cudaStream_t s);
int mr_ymid(ps_plan p, const int* active, cudaStream_t s);
int mr_last(ps_plan p, int stage, const float* Un, float* out, double dt, const double* d_dt, bool filter_last,
            const int* active, cudaStream_t s);
int mr_steps_1d(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
                cudaStream_t s);

// NUFFT point evaluation (nufft.cu)
bool nufft_supported(const ps_plan_s* p);
int nufft_points(ps_plan p, const float* f, int nf, bool velocity, double* pos, double* prev, int np, int first,
                 double dt, float* out, cudaStream_t s);

}  // namespace ps
