// TMA-fed strided pencil passes (pencils along y or z).
//
// Pencils along a strided axis need whole columns of the field.  Every
// input field tile ([N rows] x [T adjacent x columns], one 4-D tensor-map box
// per 256 rows) is streamed by the tensor memory accelerator into a ring of R
// shared-memory slots.  One elected thread issues the loads R tiles ahead of
// consumption; all threads wait on the slot's mbarrier (bounded), copy their
// pencil points out of shared memory and release the slot.  DRAM latency is
// thereby overlapped with the FFT work of earlier tiles instead of stalling
// the warps that need the data.
//
// Field buffers are described by 4-D tensor maps over [nf][Nz][Ny][Nx]
// float32 arrays, innermost first: dims {Nx, Ny, Nz, nf}.  Boxes are
// {T, min(N,256), 1, 1} for y pencils and {T, 1, min(N,256), 1} for z
// pencils; either lands in shared memory as rows of T floats.
#pragma once
#include "euler_passes.cuh"
#include "mhd_passes.cuh"
#include "tma.cuh"

namespace ps {

// resident CTAs per SM the register allocation must allow (about 512 threads)
template <int N, int T>
constexpr int tma_min_blocks() {
  return (512 / (Shape<N>::A * T)) > 0 ? (512 / (Shape<N>::A * T)) : 1;
}

template <int N, int T>
struct TileGeom {
  static constexpr int BOX = (N < 256) ? N : 256;  // rows per TMA box
  static constexpr int NBOX = N / BOX;
  static constexpr uint32_t BYTES = N * T * 4;
};

// Ring of R tile slots with one mbarrier each.  Tile i lives in slot i % R
// and completes phase (i / R) & 1 of that slot's barrier.
template <int N, int T, int R>
struct Ring {
  alignas(1024) float slot[R][N * T];
  uint64_t bar[R];
  int abort;
  int sched[64];  // tile schedule: map id * 256 + field within the solve
  int ntiles;
};

// Which axis the pencils run along (1 = y, 2 = z), and where the tile sits.
struct TileIssue {
  int axis;
  int x0;     // first column of the tile
  int outer;  // z (axis 1) or y (axis 2)
  // per map: field coordinate of this solve's first field (solve * fields per
  // solve); separate members, not an array, so they stay in registers
  int fb0, fb1, fb2;
};

// The (up to three) tensor maps a pass reads, as separate members so that no
// runtime-indexed array lands in local memory.
struct MapSet {
  const CUtensorMap* m0;
  const CUtensorMap* m1;
  const CUtensorMap* m2;
};

template <int N, int T, int R>
__device__ __forceinline__ void ring_issue(Ring<N, T, R>& rg, int i, const MapSet& maps, const TileIssue& ti) {
  using G = TileGeom<N, T>;
  const int s = i % R;
  const int code = rg.sched[i];
  const int mi = code >> 8;
  const CUtensorMap* m = (mi == 0) ? maps.m0 : (mi == 1) ? maps.m1 : maps.m2;
  const int f = ((mi == 0) ? ti.fb0 : (mi == 1) ? ti.fb1 : ti.fb2) + (code & 255);
  mbar_arrive_expect_tx(&rg.bar[s], G::BYTES);
#pragma unroll
  for (int b = 0; b < G::NBOX; ++b) {
    float* dst = &rg.slot[s][b * G::BOX * T];
    if (ti.axis == 1) tma_load_4d(dst, m, ti.x0, b * G::BOX, ti.outer, f, &rg.bar[s]);
    else tma_load_4d(dst, m, ti.x0, ti.outer, b * G::BOX, f, &rg.bar[s]);
  }
}

// Consumer side of the ring.  `issued` lives in thread 0 only.
template <int N, int T, int R>
struct RingCursor {
  Ring<N, T, R>& rg;
  MapSet maps;
  TileIssue ti;
  int* status;
  int issued;  // thread 0: tiles issued so far

  __device__ void start() {
    if (threadIdx.x == 0) {
      issued = 0;
      while (issued < rg.ntiles && issued < R) ring_issue<N, T, R>(rg, issued++, maps, ti);
    }
  }
  // wait for tile i and return its slot
  __device__ const float* wait(int i) {
    const int s = i % R;
    if (!*(volatile int*)&rg.abort) {
      if (!mbar_wait(&rg.bar[s], (uint32_t)((i / R) & 1), status)) *(volatile int*)&rg.abort = 1;
    }
    return rg.slot[s];
  }
  // all threads are done with tiles <= i: refill freed slots
  __device__ void release(int i) {
    __syncthreads();
    if (threadIdx.x == 0 && !*(volatile int*)&rg.abort) {
      while (issued < rg.ntiles && issued <= i + R) ring_issue<N, T, R>(rg, issued++, maps, ti);
    }
  }
  // before exit: every issued tile must have landed (bounded waits)
  __device__ void drain(int consumed) {
    if (threadIdx.x == 0) {
      for (int i = consumed; i < issued; ++i) mbar_wait(&rg.bar[i % R], (uint32_t)((i / R) & 1), status);
    }
  }
};

template <int N, int T, int R>
__device__ __forceinline__ void ring_init(Ring<N, T, R>& rg) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < R; ++s) mbar_init(&rg.bar[s], 1);
    rg.abort = 0;
    fence_barrier_init();
  }
}

// pair (fa, fb) of this thread's pencil points from two tiles
template <int N, int T>
__device__ __forceinline__ void tile_pair(float2 (&v)[Shape<N>::B], const float* ta, const float* tb, int t,
                                          int p) {
  constexpr int A = Shape<N>::A;
#pragma unroll
  for (int n2 = 0; n2 < Shape<N>::B; ++n2) {
    const int r = (t + A * n2) * T + p;
    v[n2] = make_float2(ta[r], tb ? tb[r] : 0.0f);
  }
}

// w <- sign * (P[k] z1 + i d[k] z2) for two packed spectra in spectral layout.
// P and i*d are real-to-real operators, so they act on the real and imaginary
// halves of a packed pencil independently: with z1 = FFT(a_c + i a_c') and
// z2 = FFT(b_c + i b_c') the inverse transform of w holds
// P a_c + D b_c in its real part and P a_c' + D b_c' in its imaginary part.
template <int N, int T>
__device__ __forceinline__ void apply_pd(float2 (&w)[Shape<N>::B], const float2 (&z2)[Shape<N>::B],
                                         const Pencil<N, T, true>& pf, const AxisSmem<N>& ax, float sign) {
#pragma unroll
  for (int r = 0; r < Shape<N>::B; ++r) {
    const int k = pf.kidx(r);
    const float P = sign * ax.P[k], d = sign * ax.d[k];
    w[r] = make_float2(fmaf(P, w[r].x, -d * z2[r].y), fmaf(P, w[r].y, d * z2[r].x));
  }
}

template <int N, int T, int R>
struct TmaStridedSmem {
  AxisSmem<N> ax;
  float2 buf[Pencil<N, T, true>::BUF];
  Ring<N, T, R> ring;
};

// ---------------------------------------------------------------------------
// 3D y pass.  Map 0 = G buffer (15 fields: G, Hy, Hz).  Output via st.global.
// ---------------------------------------------------------------------------
struct YMidTArgs {
  float* out;      // 10 fields per solve [A(5), B(5)]
  long fs;
  long ssOut;      // solve stride of out (10 * cells)
  int nsolve;
  StridedGeom g;   // geometry of one solve; blockIdx.y runs over nsolve * g.nouter
  AxisOps ax;
  const int* active;
  int* status;
};

template <int N, int T, int R>
__global__ void __launch_bounds__(Shape<N>::A * T, tma_min_blocks<N, T>())
    k_ymid3_t(const __grid_constant__ CUtensorMap mG, YMidTArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(1024) unsigned char smem_tma[];
  auto& S = *reinterpret_cast<TmaStridedSmem<N, T, R>*>(smem_tma);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int col = blockIdx.x * T + p;
  const int sol = blockIdx.y / a.g.nouter;
  const int outer = blockIdx.y % a.g.nouter;
  if (a.active != nullptr && a.active[sol] == 0) return;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  ring_init(S.ring);
  if (threadIdx.x == 0) {
    // A pairs (c, c+1) for c = 0, 2: G_c, G_c+1, Hy_c, Hy_c+1; Hz pairs for
    // c = 0, 2; then G_4, Hz_4, Hy_4 for the merged last job
    const int order[15] = {0, 1, 5, 6, 2, 3, 7, 8, 10, 11, 12, 13, 4, 14, 9};
    for (int i = 0; i < 15; ++i) S.ring.sched[i] = order[i];
    S.ring.ntiles = 15;
  }
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const MapSet maps{&mG, &mG, &mG};
  RingCursor<N, T, R> rc{S.ring, maps, TileIssue{1, (int)(blockIdx.x * T), outer, sol * 15, 0, 0}, a.status, 0};
  rc.start();
  const long base = (long)sol * a.ssOut + (long)outer * a.g.os + col + (long)t * a.g.as;
  const long step = (long)A * a.g.as;
  const bool valid = col < a.g.ncol;
  int ti = 0;
#pragma unroll 1
  for (int c = 0; c < 4; c += 2) {
    float2 w[B], z2[B];
    tile_pair<N, T>(w, rc.wait(ti), rc.wait(ti + 1), t, p);       // G_c + i G_c+1
    tile_pair<N, T>(z2, rc.wait(ti + 2), rc.wait(ti + 3), t, p);  // Hy_c + i Hy_c+1
    ti += 4;
    rc.release(ti - 1);
    pf.fwd(w);
    pf.fwd(z2);
    apply_pd<N, T>(w, z2, pf, S.ax, 1.0f);
    pf.inv(w);
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[c * a.fs + base + n2 * step] = w[n2].x;
        a.out[(c + 1) * a.fs + base + n2 * step] = w[n2].y;
      }
    }
  }
#pragma unroll 1
  for (int c = 0; c < 4; c += 2) {  // Hz_c + i Hz_c+1
    float2 w[B];
    tile_pair<N, T>(w, rc.wait(ti), rc.wait(ti + 1), t, p);
    rc.release(ti + 1);
    ti += 2;
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const float s = S.ax.P[pf.kidx(r)];
      w[r].x *= s;
      w[r].y *= s;
    }
    pf.inv(w);
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[(5 + c) * a.fs + base + n2 * step] = w[n2].x;
        a.out[(6 + c) * a.fs + base + n2 * step] = w[n2].y;
      }
    }
  }
  {  // merged last job: FFT(G_4 + i Hz_4) and FFT(Hy_4); P on the first plus D on the
     // second gives A_4 = P_y G_4 + D_y Hy_4 (real part) and B_4 = P_y Hz_4 (imaginary)
    float2 w[B], z2[B];
    tile_pair<N, T>(w, rc.wait(ti), rc.wait(ti + 1), t, p);
    tile_pair<N, T>(z2, rc.wait(ti + 2), nullptr, t, p);
    rc.release(ti + 2);
    ti += 3;
    pf.fwd(w);
    pf.fwd(z2);
    apply_pd<N, T>(w, z2, pf, S.ax, 1.0f);
    pf.inv(w);
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[4 * a.fs + base + n2 * step] = w[n2].x;
        a.out[9 * a.fs + base + n2 * step] = w[n2].y;
      }
    }
  }
  rc.drain(ti);
}

// ---------------------------------------------------------------------------
// Last pass with TMA inputs.  Maps: 0 = a/b buffer (a_c at field fa0 + c, b_c
// at fb0 + c), 1 = U^n, 2 = accumulator.  Writes via st.global.
// ---------------------------------------------------------------------------
struct LastTArgs {
  int fa0, fb0;        // field offsets of a_0 and b_0 in map 0 (within a solve)
  int nfAB;            // fields per solve in map 0
  float* acc;          // accumulator (written)
  float* out;          // rhs / next stage input / new state
  long fs;
  long ssAcc, ssOut, ssUn;  // solve strides of acc, out and Un
  const int* active;   // per-solve flags (null: all active)
  int nsolve;
  StridedGeom g;       // geometry of one solve; blockIdx.y runs over nsolve * g.nouter
  int axis;            // 1: y pencils, 2: z pencils
  AxisOps ax;
  int stage;           // -1 rhs only, 0..3 RK4 stage
  const float* Un;     // U^n (global; used by the clamped variant)
  const double* dt_dev;  // per-solve step sizes (null: dt for every solve)
  double dt;
  float gamma;
  float rho_min, p_min;
  const float* eref;     // per-solve E_ref
  int filter_last;
  int* status;
  int mhd;             // 1: 2D ideal MHD (8 components, the PHYS = 1 kernel)
  int tcols;           // 2D: columns per tile (4, 8, 16; 0: default) = the maps' box width
  // constant gravity (solver.py:453-464, 1193-1206): rhs_m += rho g, rhs_E += g . m,
  // from the stage input Uin (same layout and solve stride as Un)
  const float* Uin;
  float grav[3];
  int gravity;
  int rk2;             // midpoint RK2 coefficients (stages 0 and 3 only)
  int rhs2d;           // 2D, stage -1: the unclamped instantiation writes the right-hand side
  int pair_groups;     // unclamped launches: gridDim.z groups of component pairs (0 or 1: one)
};

// Gravity source at one point of solve-local offset o (element index of
// component 0): adds rho g to the momenta and g . m to the energy of k.
template <int ND>
__device__ __forceinline__ void gravity_source(const LastTArgs& a, const float* uin, long o, long fs,
                                               float (&k)[ND + 2]) {
  const float rho = uin[o];
  float gm = 0.0f;
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    k[1 + d] = fmaf(rho, a.grav[d], k[1 + d]);
    gm = fmaf(a.grav[d], uin[o + (1 + d) * fs], gm);
  }
  k[ND + 1] += gm;
}

// Resident CTAs the register allocation must allow.  The clamped variants
// hold every component's right-hand side until the clamp: about 170
// registers (2D Euler) without spilling; MHD needs all 255.
template <int N, int T, bool CLAMP, int PHYS>
constexpr int clamp_min_blocks() {
  if (!CLAMP) return tma_min_blocks<N, T>();
  if (PHYS == 1) return 1;
  const int m = 65536 / (Shape<N>::A * T * 168);
  return m > 0 ? m : 1;
}

// PHYS 0: Euler (ND + 2 components, energy-perturbation clamp); PHYS 1: 2D
// ideal MHD (8 components, MHD clamp, mhd_passes.cuh).  FL: the launch may
// apply the last factor of the end-of-step filter (stage 3); the other
// launches run an instantiation without those two transforms, whose smaller
// code stays in the instruction cache.
template <int N, int T, int ND, bool CLAMP, int R, int PHYS = 0, bool FL = true>
__global__ void __launch_bounds__(Shape<N>::A * T, clamp_min_blocks<N, T, CLAMP, PHYS>())
    k_last_t(const __grid_constant__ CUtensorMap mAB, const __grid_constant__ CUtensorMap mU,
             const __grid_constant__ CUtensorMap mAcc, LastTArgs a) {
  constexpr int NC = (PHYS == 1) ? 8 : ND + 2;
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(1024) unsigned char smem_tma[];
  auto& S = *reinterpret_cast<TmaStridedSmem<N, T, R>*>(smem_tma);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int col = blockIdx.x * T + p;
  const int sol = blockIdx.y / a.g.nouter;
  const int outer = blockIdx.y % a.g.nouter;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const bool valid = col < a.g.ncol;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  ring_init(S.ring);
  const bool need_un = !CLAMP && a.stage >= 0 && a.stage != 3;
  const bool need_acc = !CLAMP && a.stage >= 1;
  // component pairs [c_lo, c_hi) of this CTA: all of them, or one of gridDim.z
  // equal groups (unclamped launches on grids with few column tiles)
  const int ppg = ((NC + 1) / 2 + (int)gridDim.z - 1) / (int)gridDim.z;
  const int c_lo = CLAMP ? 0 : 2 * ppg * (int)blockIdx.z;
  const int c_hi = CLAMP ? NC : min(NC, c_lo + 2 * ppg);
  if (threadIdx.x == 0) {
    int n = 0;
    for (int c = c_lo; c < c_hi; c += 2) {
      const int m = (c + 1 < NC) ? 2 : 1;
      for (int q = 0; q < m; ++q) S.ring.sched[n++] = a.fa0 + c + q;
      for (int q = 0; q < m; ++q) S.ring.sched[n++] = a.fb0 + c + q;
      if (need_un)
        for (int q = 0; q < m; ++q) S.ring.sched[n++] = 256 + c + q;
      if (need_acc)
        for (int q = 0; q < m; ++q) S.ring.sched[n++] = 512 + c + q;
    }
    S.ring.ntiles = n;
  }
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const MapSet maps{&mAB, &mU, &mAcc};
  RingCursor<N, T, R> rc{S.ring, maps,
                         TileIssue{a.axis, (int)(blockIdx.x * T), outer, sol * a.nfAB, sol * NC, sol * NC},
                         a.status, 0};
  rc.start();
  const long base = (long)outer * a.g.os + col + (long)t * a.g.as;  // within a solve
  const long step = (long)A * a.g.as;
  const float dt = (a.dt_dev != nullptr) ? (float)a.dt_dev[sol] : (float)a.dt;
  const RKCoef rk = rk_coef(a.stage < 0 ? 0 : a.stage, dt, a.rk2);
  const float pmin_shift = a.p_min - (a.gamma - 1.0f) * a.eref[sol];
  float* const acc_s = (a.acc != nullptr) ? a.acc + (long)sol * a.ssAcc : nullptr;
  float* const out_s = a.out + (long)sol * a.ssOut;
  const float* const un_s = a.Un + (long)sol * a.ssUn;
  auto addr = [&](int c, int n2) { return c * a.fs + base + n2 * step; };
  auto filter_pair = [&](float2 (&w)[B]) {  // complementary form
    float2 w0[B];
#pragma unroll
    for (int r = 0; r < B; ++r) w0[r] = w[r];
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const float q = (1.0f / N) - S.ax.P[pf.kidx(r)];
      w[r].x *= q;
      w[r].y *= q;
    }
    pf.inv(w);
#pragma unroll
    for (int r = 0; r < B; ++r) w[r] = make_float2(w0[r].x - w[r].x, w0[r].y - w[r].y);
  };
  int ti = 0;
  // -(P a_c + D b_c) for components (c, c+1), real and imaginary part
  auto rhs_pair = [&](int c, float2 (&w)[B]) {
    const bool two = c + 1 < NC;
    const int m = two ? 2 : 1;
    float2 z2[B];
    tile_pair<N, T>(w, rc.wait(ti), two ? rc.wait(ti + 1) : nullptr, t, p);
    tile_pair<N, T>(z2, rc.wait(ti + m), two ? rc.wait(ti + m + 1) : nullptr, t, p);
    ti += 2 * m;
    rc.release(ti - 1);
    pf.fwd(w);
    pf.fwd(z2);
    apply_pd<N, T>(w, z2, pf, S.ax, -1.0f);
    pf.inv(w);
  };

  if constexpr (!CLAMP) {
#pragma unroll 1
    for (int c = c_lo; c < c_hi; c += 2) {
      const bool two = c + 1 < NC;
      const int m = two ? 2 : 1;
      float2 w[B];
      rhs_pair(c, w);
      if constexpr (PHYS == 0) {
        if (a.gravity && valid) {  // components (c, c+1) of rho g / g . m
          const float* uin = a.Uin + (long)sol * a.ssUn;
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) {
            float kk[ND + 2];
#pragma unroll
            for (int q = 0; q < ND + 2; ++q) kk[q] = 0.0f;
            gravity_source<ND>(a, uin, addr(0, n2), a.fs, kk);
            w[n2].x += kk[c];
            if (two) w[n2].y += kk[c + 1];
          }
        }
      }
      if (a.stage < 0) {
        if (valid) {
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) {
            out_s[addr(c, n2)] = w[n2].x;
            if (two) out_s[addr(c + 1, n2)] = w[n2].y;
          }
        }
        continue;
      }
      const float* tu[2] = {nullptr, nullptr};
      const float* tacc[2] = {nullptr, nullptr};
      if (need_un) {
        for (int q = 0; q < m; ++q) tu[q] = rc.wait(ti + q);
        ti += m;
      }
      if (need_acc) {
        for (int q = 0; q < m; ++q) tacc[q] = rc.wait(ti + q);
        ti += m;
      }
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        const int r = (t + A * n2) * T + p;
        const float k[2] = {w[n2].x, w[n2].y};
        float res[2] = {0.0f, 0.0f};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (q == 1 && !two) break;
          if (a.stage == 3) {
            res[q] = fmaf(rk.wacc, k[q], tacc[q][r]);
          } else {
            const float un = tu[q][r];
            const float ac = fmaf(rk.wacc, k[q], (a.stage == 0) ? un : tacc[q][r]);
            if (valid) acc_s[addr(c + q, n2)] = ac;
            res[q] = fmaf(rk.wnext, k[q], un);
          }
        }
        w[n2] = make_float2(res[0], res[1]);
      }
      if (need_un || need_acc) rc.release(ti - 1);
      if (FL && a.stage == 3 && a.filter_last) filter_pair(w);
      if (valid) {
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          out_s[addr(c, n2)] = w[n2].x;
          if (two) out_s[addr(c + 1, n2)] = w[n2].y;
        }
      }
    }
  } else {
    float2 kk[(NC + 1) / 2][B];
    if constexpr (PHYS == 1) {
#pragma unroll
      for (int c = 0; c < NC; c += 2) rhs_pair(c, kk[c / 2]);
    } else {
    // one pencil-transform body for all pairs (a rolled loop; the switch keeps
    // kk in registers): unrolled, the pairs' FFTs overflow the instruction cache
#pragma unroll 1
    for (int c = 0; c < NC; c += 2) {
      float2 w[B];
      rhs_pair(c, w);
      switch (c / 2) {
#define PS_KK_SET(J)                                                    \
  case J:                                                               \
    if constexpr (J < (NC + 1) / 2) {                                   \
      _Pragma("unroll") for (int r = 0; r < B; ++r) kk[J][r] = w[r];    \
    }                                                                   \
    break;
        PS_KK_SET(0)
        PS_KK_SET(1)
        PS_KK_SET(2)
        PS_KK_SET(3)
#undef PS_KK_SET
        default:
          break;
      }
    }
    }
    if constexpr (PHYS == 0) {
      if (a.gravity && valid) {
        const float* uin = a.Uin + (long)sol * a.ssUn;
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
          float k[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) k[c] = (c & 1) ? kk[c / 2][n2].y : kk[c / 2][n2].x;
          gravity_source<ND>(a, uin, addr(0, n2), a.fs, k);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            if (c & 1) kk[c / 2][n2].y = k[c];
            else kk[c / 2][n2].x = k[c];
          }
        }
      }
    }
    if (a.stage < 0) {
      if (valid) {
#pragma unroll
        for (int c = 0; c < NC; c += 2)
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) {
            out_s[addr(c, n2)] = kk[c / 2][n2].x;
            if (c + 1 < NC) out_s[addr(c + 1, n2)] = kk[c / 2][n2].y;
          }
      }
    } else {
      constexpr int CH = (NC > 5) ? 2 : 4;  // positions per batch of epilogue loads
#pragma unroll
      for (int n0 = 0; n0 < B; n0 += CH) {
        float un[CH][NC], ac[CH][NC];
#pragma unroll
        for (int j = 0; j < CH; ++j)
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            un[j][c] = (valid && a.stage != 3) ? __ldg(un_s + addr(c, n0 + j)) : 0.0f;
            ac[j][c] = (valid && a.stage != 0) ? acc_s[addr(c, n0 + j)] : 0.0f;
          }
#pragma unroll
        for (int j = 0; j < CH; ++j) {
          const int n2 = n0 + j;
          float u[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            const float k = (c & 1) ? kk[c / 2][n2].y : kk[c / 2][n2].x;
            float res;
            if (a.stage == 3) {
              res = fmaf(rk.wacc, k, ac[j][c]);
            } else {
              ac[j][c] = fmaf(rk.wacc, k, (a.stage == 0) ? un[j][c] : ac[j][c]);
              res = fmaf(rk.wnext, k, un[j][c]);
            }
            u[c] = valid ? res : ((c == 0) ? 1.0f : 0.0f);
          }
          if constexpr (PHYS == 1) clamp_mhd(u, a.gamma, a.rho_min, a.p_min);
          else clamp_state<ND>(u, a.gamma, a.rho_min, pmin_shift);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            if (c & 1) kk[c / 2][n2].y = u[c];
            else kk[c / 2][n2].x = u[c];
          }
        }
        if (valid && a.stage != 3) {
#pragma unroll
          for (int j = 0; j < CH; ++j)
#pragma unroll
            for (int c = 0; c < NC; ++c) acc_s[addr(c, n0 + j)] = ac[j][c];
        }
      }
#pragma unroll 1
      for (int c = 0; c < NC; c += 2) {
        float2 w[B];
        switch (c / 2) {
#define PS_KK_GET(J)                                                    \
  case J:                                                               \
    if constexpr (J < (NC + 1) / 2) {                                   \
      _Pragma("unroll") for (int r = 0; r < B; ++r) w[r] = kk[J][r];    \
    }                                                                   \
    break;
          PS_KK_GET(0)
          PS_KK_GET(1)
          PS_KK_GET(2)
          PS_KK_GET(3)
#undef PS_KK_GET
          default:
            break;
        }
        if (FL && a.stage == 3 && a.filter_last) filter_pair(w);
        if (valid) {
#pragma unroll
          for (int n2 = 0; n2 < B; ++n2) {
            out_s[addr(c, n2)] = w[n2].x;
            if (c + 1 < NC) out_s[addr(c + 1, n2)] = w[n2].y;
          }
        }
      }
    }
  }
  rc.drain(ti);
}

// ---------------------------------------------------------------------------
// Strided one-axis operator (P, D or complementary P) with TMA inputs.
// Map 0 = input buffer (fields 0..nf-1).  in and out may alias: a tile is
// fully landed in shared memory before any point of it is written back.
// ---------------------------------------------------------------------------
struct OpTArgs {
  float* out;
  int nf;          // fields per solve (map fields per solve as well)
  long fs;
  long ss;         // solve stride of out
  const int* active;
  int nsolve;
  StridedGeom g;   // geometry of one solve; blockIdx.y runs over nsolve * g.nouter
  int axis;
  AxisOps ax;
  int deriv;       // 0 P, 1 D, 2 L (Laplacian factor), 3 raw second derivative (op_symbol)
  float scale;
  int complement;
  int* status;
  int tcols;       // columns per tile (4, 8, 16; 0: default) = the map's box width
  float kunit;     // 2 pi / L of the axis (deriv 2, 3)
};

template <int N, int T, int R>
__global__ void __launch_bounds__(Shape<N>::A * T, tma_min_blocks<N, T>())
    k_op_t(const __grid_constant__ CUtensorMap mIn, OpTArgs a) {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  using PF = Pencil<N, T, true>;
  extern __shared__ __align__(1024) unsigned char smem_tma[];
  auto& S = *reinterpret_cast<TmaStridedSmem<N, T, R>*>(smem_tma);
  const int p = threadIdx.x % T, t = threadIdx.x / T;
  const int col = blockIdx.x * T + p;
  const int sol = blockIdx.y / a.g.nouter;
  const int outer = blockIdx.y % a.g.nouter;
  if (a.active != nullptr && a.active[sol] == 0) return;
  const bool valid = col < a.g.ncol;
  PF pf{p, t, S.buf, S.ax.twf, S.ax.twi};
  ring_init(S.ring);
  if (threadIdx.x == 0) {
    for (int f = 0; f < a.nf; ++f) S.ring.sched[f] = f;
    S.ring.ntiles = a.nf;
  }
  load_axis<N>(S.ax, a.ax);
  __syncthreads();
  const MapSet maps{&mIn, &mIn, &mIn};
  RingCursor<N, T, R> rc{S.ring, maps, TileIssue{a.axis, (int)(blockIdx.x * T), outer, sol * a.nf, 0, 0},
                         a.status, 0};
  rc.start();
  const long base = (long)sol * a.ss + (long)outer * a.g.os + col + (long)t * a.g.as;
  const long step = (long)A * a.g.as;
  const bool comp = a.complement && !a.deriv;
  int ti = 0;
#pragma unroll 1
  for (int c = 0; c < a.nf; c += 2) {
    const bool two = c + 1 < a.nf;
    float2 w[B], w0[B];
    tile_pair<N, T>(w, rc.wait(ti), two ? rc.wait(ti + 1) : nullptr, t, p);
    rc.release(ti + (two ? 1 : 0));
    ti += two ? 2 : 1;
#pragma unroll
    for (int r = 0; r < B; ++r) w0[r] = w[r];
    pf.fwd(w);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      const int k = pf.kidx(r);
      if (comp) {
        const float s = (1.0f / N) - S.ax.P[k];
        w[r].x *= s;
        w[r].y *= s;
      } else {
        w[r] = op_symbol<N>(w[r], k, a.deriv, a.scale, a.kunit, S.ax.P, S.ax.d);
      }
    }
    pf.inv(w);
    if (comp) {
#pragma unroll
      for (int r = 0; r < B; ++r) w[r] = make_float2(w0[r].x - w[r].x, w0[r].y - w[r].y);
    }
    if (valid) {
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) {
        a.out[c * a.fs + base + n2 * step] = w[n2].x;
        if (two) a.out[(c + 1) * a.fs + base + n2 * step] = w[n2].y;
      }
    }
  }
  rc.drain(ti);
}

}  // namespace ps
