// Fourier plans with axes of any 2^a 3^b 5^c length: tables, pass launches
// in the contracts of the power-of-two passes, and the 1D step loop.
#include <cuda_runtime.h>
#include <math.h>

#include <vector>

#include "mixed_radix.cuh"
#include "plan.cuh"
#include "reduce.cuh"

namespace ps {
namespace {

int cfail(cudaError_t e, const char* what) { return errorf(PS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); }

#define MR_CU(expr, what)                          \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return cfail(_e, what); \
  } while (0)

// Symbol tables of one axis in float64, stored as float (grid.py:47-63 mask
// and filter for any N: k = fftfreq(N) * N, cutoff N // 3, kmax = max |k|;
// wavenumbers 2 pi k / L, grid.py:255-257).  The derivative symbol is zero
// at the Nyquist index of even N (the reference keeps the real part of the
// inverse transform, which drops that term).  The mode numbers are the
// reference's float64 values fftfreq(N) * N = (k * (1/N)) * N, rounding
// included: for N that is not a power of two a mode k = N // 3 can come out
// one ulp above the cutoff and is then masked (N = 45: k = 15 gives
// 15.000000000000002), and the mask follows that.
void mr_tables(int N, double L, int dealias, int fon, int fp, double falpha, std::vector<float>& P,
               std::vector<float>& d, std::vector<float2>& tw) {
  P.resize(N);
  d.resize(N);
  tw.resize(N);
  const double val = 1.0 / (double)N;
  std::vector<double> kf(N);
  double kmax = 0.0;
  for (int k = 0; k < N; ++k) {
    const int kk = (2 * k <= N - 1) ? k : k - N;  // fftfreq ordering
    kf[k] = ((double)kk * val) * (double)N;
    kmax = fmax(kmax, fabs(kf[k]));
  }
  for (int k = 0; k < N; ++k) {
    const int kk = (2 * k <= N - 1) ? k : k - N;
    const double ak = fabs(kf[k]);
    double m = (!dealias || ak <= (double)(N / 3)) ? 1.0 : 0.0;
    if (fon) m *= exp(-falpha * pow(ak / (kmax > 1.0 ? kmax : 1.0), fp));
    P[k] = (float)(m / N);
    const double kphys = 2.0 * M_PI * kk / L;
    d[k] = (N % 2 == 0 && 2 * k == N) ? 0.0f : (float)(kphys * m / N);
    const double ang = -2.0 * M_PI * (double)k / N;
    tw[k] = make_float2((float)cos(ang), (float)sin(ang));
  }
}

MrGeom geom(const ps_plan_s* p, int axis, int extra_per_pencil) {
  long es = 1;
  for (int a = 0; a < axis; ++a) es *= p->n[a];
  return mr_geom(p->mrax[axis], es, p->cells / p->n[axis], extra_per_pencil);
}

}  // namespace

bool mr_axis_ok(int n) {
  int r[kMrMaxStages], nst = 0;
  return n >= 2 && n <= kMrMaxLen && mr_factor(n, r, &nst);
}

int mr_setup(ps_plan p) {
  p->mr = true;
  for (int a = 0; a < p->nd; ++a) {
    const int N = p->n[a];
    std::vector<float> P, d;
    std::vector<float2> tw;
    mr_tables(N, p->desc.length[a], p->desc.dealias, p->desc.filter_enabled, p->desc.filter_p, p->desc.filter_alpha,
              P, d, tw);
    int rc;
    if ((rc = plan_alloc(p, &p->P[a], N)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &p->d[a], N)) != PS_OK) return rc;
    if ((rc = plan_alloc(p, &p->twf[a], N)) != PS_OK) return rc;
    MR_CU(cudaMemcpy(p->P[a], P.data(), N * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    MR_CU(cudaMemcpy(p->d[a], d.data(), N * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    MR_CU(cudaMemcpy(p->twf[a], tw.data(), N * sizeof(float2), cudaMemcpyHostToDevice), "table upload");
    MrAxis& ax = p->mrax[a];
    int radix[kMrMaxStages];
    if (!mr_factor(N, radix, &ax.nst)) return errorf(PS_ERR_UNSUPPORTED, "axis %d: N=%d is not 5-smooth", a, N);
    ax.n = N;
    ax.rcode = 0;
    for (int s = 0; s < ax.nst; ++s) ax.rcode |= (unsigned long long)radix[s] << (4 * s);
    ax.ntp = (N + kMrDiv - 1) / kMrDiv;
    if (2 * ax.ntp > kMrThreads)  // two signals of one pencil per CTA at least
      return errorf(PS_ERR_UNSUPPORTED, "axis %d: N=%d needs more than %d threads per CTA", a, N, kMrThreads);
    ax.tw = p->twf[a];
    ax.P = p->P[a];
    ax.d = p->d[a];
  }
  return PS_OK;
}

int mr_apply_op(ps_plan p, int axis, const float* in, float* out, int nf, int deriv, float scale, bool complement,
                const int* active, long ss_in, cudaStream_t s) {
  MrOpArgs a{};
  a.in = in;
  a.out = out;
  a.nf = nf;
  a.fs = p->cells;
  a.ss_out = p->ss(nf);
  a.ss_in = (ss_in != 0) ? ss_in : a.ss_out;
  a.ax = p->mrax[axis];
  a.g = geom(p, axis, 0);
  a.deriv = deriv;
  a.scale = scale;
  a.kunit = (float)(2.0 * M_PI / p->desc.length[axis]);
  a.complement = complement ? 1 : 0;
  a.active = active;
  MR_CU(launch_mr_op(a, p->nsolve, s), "operator pass");
  return PS_OK;
}

int mr_xfirst(ps_plan p, const float* U, float* Uw, float* speed, bool shift_in, const int* active, cudaStream_t s) {
  MrXArgs a{};
  a.U = U;
  a.Uw = Uw;
  a.out = p->G;
  a.fs = p->cells;
  a.ssU = p->ss(p->nc);
  a.ssOut = p->ss(p->nd * p->nc);
  a.ax = p->mrax[0];
  a.g = geom(p, 0, 4 * p->nc * p->n[0]);
  a.nd = p->nd;
  a.gamma = (float)p->desc.gamma;
  a.speed = speed;
  a.eref = p->eref;
  a.active = active;
  a.shift_in = shift_in ? 1 : 0;
  MR_CU(launch_mr_x(a, p->nsolve, s), "x pass");
  return PS_OK;
}

int mr_ymid(ps_plan p, const int* active, cudaStream_t s) {
  MrY3Args a{};
  a.G = p->G;
  a.out = p->AB;
  a.fs = p->cells;
  a.ssG = p->ss(15);
  a.ssOut = p->ss(10);
  a.ax = p->mrax[1];
  a.g = geom(p, 1, 0);
  a.active = active;
  MR_CU(launch_mr_y3(a, p->nsolve, s), "y pass");
  return PS_OK;
}

int mr_last(ps_plan p, int stage, const float* Un, float* out, double dt, const double* d_dt, bool filter_last,
            const int* active, cudaStream_t s) {
  const int nc = p->nc, axis = p->nd - 1;
  MrLastArgs a{};
  if (p->nd == 3) {
    a.AB = p->AB;
    a.fa0 = 0;
    a.fb0 = 5;
    a.ssAB = p->ss(10);
  } else {
    a.AB = p->G;
    a.fa0 = 0;
    a.fb0 = nc;
    a.ssAB = p->ss(2 * nc);
  }
  a.acc = p->acc;
  a.out = out;
  a.Un = Un;
  a.Uin = (stage <= 0) ? Un : p->Us;
  a.fs = p->cells;
  a.ssAcc = a.ssOut = a.ssUn = p->ss(nc);
  a.ax = p->mrax[axis];
  a.g = geom(p, axis, 4 * nc * p->n[axis]);
  a.nd = p->nd;
  a.stage = stage;
  a.dt_dev = d_dt;
  a.dt = dt;
  a.gamma = (float)p->desc.gamma;
  a.rho_min = 1e-8f;  // _positivity_clamp_2d floors (solver.py:467); the 3D solver has no clamp
  a.p_min = 1e-10f;
  a.eref = p->eref;
  a.filter_last = filter_last ? 1 : 0;
  a.clamp = (p->nd == 2) ? 1 : 0;
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  a.gravity = 0;
  for (int d = 0; d < p->nd && d < 3; ++d) {
    a.grav[d] = (float)p->desc.gravity[d];
    if (p->desc.gravity[d] != 0.0) a.gravity = 1;
  }
  a.active = active;
  MR_CU(launch_mr_last(a, p->nsolve, s), "last pass");
  return PS_OK;
}

// 1D Euler steps on any-length grids, stage by stage: k_mr_line per stage
// (the whole-step kernel of the power-of-two plans holds its state in
// shared memory; here U^n is the caller's state and the stage input and the
// increments live in the plan scratch), then the filter P_x inside the RK
// step and once more at the cadence (solver.py:62-132, 259-269).  CFL mode:
// per-solve dt = cfl dx / max(|u| + a), clipped to the end time.
int mr_steps_1d(ps_plan p, float* U, int nsteps, double dt, const double* d_dt, double* d_t, const double* d_tend,
                cudaStream_t s) {
  int rc;
  const bool cfl = d_t != nullptr;
  const int* act = cfl ? p->active : nullptr;
  const double* dtp = cfl ? p->dt : d_dt;
  const long ssU = p->ss(3);
  float* E = U + 2 * p->cells;
  MR_CU(launch_eref_set(E, ssU, p->nsolve, p->eref, s), "energy reference");
  MR_CU(launch_energy_shift(E, p->cells, ssU, p->nsolve, p->eref, -1.0f, s), "energy shift");
  if (cfl) MR_CU(launch_fill_int(p->active, p->nsolve, 1, s), "active reset");
  MrLineArgs a{};
  a.Un = U;
  a.acc = p->acc;
  a.ss = ssU;
  a.ax = p->mrax[0];
  a.g = mr_geom(p->mrax[0], 1, 1, 0);
  a.gamma = (float)p->desc.gamma;
  a.rho_min = 1e-10f;  // _positivity_clamp floors (solver.py:32)
  a.p_min = 1e-12f;
  a.eref = p->eref;
  a.gx = (float)p->desc.gravity[0];
  a.rk2 = (p->desc.scheme == PS_SCHEME_RK2) ? 1 : 0;
  a.dt_dev = dtp;
  a.dt = dt;
  a.active = act;
  for (int it = 0; it < nsteps; ++it) {
    if (cfl) {
      MR_CU(launch_speed(1, U, p->cells, ssU, p->nsolve, (float)p->desc.gamma, p->speed, s, p->eref), "wave speed");
      MR_CU(launch_step_control(p->speed, p->desc.cfl, p->hmin(), d_t, d_tend, p->nsolve, p->dt, p->active, s),
            "step control");
    }
    for (int st = 0; st < 4; ++st) {
      if (a.rk2 && (st == 1 || st == 2)) continue;
      a.in = (st == 0) ? U : p->Us;
      a.out = (st < 3) ? p->Us : U;
      a.stage = st;
      ProfScope prof(p, s, PS_KIND_STEP1D, 4.0 * p->cells * p->nsolve * ((st == 0) ? 9 : (st == 3) ? 9 : 12));
      MR_CU(launch_mr_line(a, p->nsolve, s), "1D stage");
    }
    // filter inside the RK step, then again at the cadence
    if ((rc = mr_apply_op(p, 0, U, U, 3, 0, 1.0f, true, act, 0, s)) != PS_OK) return rc;
    if ((p->step_counter % p->desc.filter_interval) == 0 &&
        (rc = mr_apply_op(p, 0, U, U, 3, 0, 1.0f, true, act, 0, s)) != PS_OK)
      return rc;
    if (cfl) MR_CU(launch_step_advance(d_t, p->dt, p->speed, p->active, p->steps_done, p->nsolve, s), "advance");
    p->step_counter += 1;
  }
  MR_CU(launch_energy_shift(E, p->cells, ssU, p->nsolve, p->eref, 1.0f, s), "energy shift");
  return PS_OK;
}

}  // namespace ps
