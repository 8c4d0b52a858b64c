// Adaptive embedded Runge-Kutta on the device (adaptive.cu): tableaux, the
// per-solve attempt state and the cell-wise kernels of one attempt for the
// multi-pass (2D/3D, MHD) plans.  1D plans run whole attempt loops in
// k_ark1d (euler1d.cuh).
#pragma once
#include <cuda_runtime.h>

namespace ps {

// Embedded pair: stage matrix a (strictly lower), high- and low-order
// weights, and the order the controller uses (the embedded, low order).
struct ArkTableau {
  int stages;
  int order;
  double a[8][8];
  double bh[8];
  double bl[8];
};

// Step controller (adaptive.py:23-81) and its rejection limit (341-419)
struct ArkCtrl {
  double rtol, atol, safety, minf, maxf;
  int max_rej;
};

// 0 on success, -1 for an unknown method (PS_ARK_RK23 / RK45 / RK78)
int ark_tableau(int method, ArkTableau* tab);

// Per-solve state of the attempt loop.
struct ArkState {
  double* t;          // simulation time (advanced on acceptance)
  const double* tend;
  double* dtp;        // proposed step, replaced by dt_next after every attempt
  const double* tout; // nullable: a solve pauses once t + 1e-12 >= tout
  double* dt;         // the attempt's dt = min(dtp, tend - t)
  int* live;          // solve takes part in this attempt
  int* ok;            // attempt accepted (mask of the post-step operator)
  int* rej;           // consecutive rejections
  float* err;         // max |U_high - U_low|
  float* scale;       // max |U|
  int* counts;        // nullable [nsolve][2]: accepted, rejected attempts
  int nsolve;
};

// Coefficients of one linear combination: out = U + sum_j (dt * c[j]) K[idx[j]]
struct ArkComb {
  int m;
  int idx[8];
  double c[8];
};

cudaError_t launch_ark_begin(const ArkState& st, cudaStream_t s);
// max |U| per solve over n elements; the energy slice [ecomp*cells, +cells)
// adds eref[solve] (states in energy-perturbation form), eref nullable
cudaError_t launch_ark_scale(const float* U, long n, long ss, long cells, int ecomp, const float* eref,
                             const ArkState& st, cudaStream_t s);
cudaError_t launch_ark_stage(const float* U, const float* K, long kstride, float* out, long n, long ss,
                             const ArkComb& cmb, const ArkState& st, cudaStream_t s);
// W = U + dt sum bh_j K_j; err = max |dt sum (bh_j - bl_j) K_j|
cudaError_t launch_ark_final(const float* U, const float* K, long kstride, float* W, long n, long ss,
                             const ArkComb& high, const ArkComb& diff, const ArkState& st, cudaStream_t s);
cudaError_t launch_ark_decide(const ArkState& st, int order, const ArkCtrl& ctrl, cudaStream_t s);
// 2D MHD positivity clamp of accepted solves, in place (solver.py:956-964)
cudaError_t launch_ark_clamp_mhd(float* U, long cells, long ss, int nsolve, float gamma, float rho_min,
                                 float p_min, const int* mask, cudaStream_t s);

}  // namespace ps
