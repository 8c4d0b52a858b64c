// Host-side launchers of the pass kernels, one explicit instantiation set per
// pencil length (kern_n*.cu), dispatched at run time by ps::dispatch_n.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_set>

#include "euler1d.cuh"
#include "mhd1d.cuh"
#include "euler_passes.cuh"
#include "passes_tma.cuh"

namespace ps {

template <int N> cudaError_t launch_xfirst(int nd, const XFirstArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_op(bool strided, const OpArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_step1d(const Step1DArgs& a, int nsolve, cudaStream_t s);
template <int N> cudaError_t launch_ark1d(const Ark1DArgs& a, int nsolve, cudaStream_t s);
template <int N> cudaError_t launch_mhd1d(const Mhd1DArgs& a, int nsolve, cudaStream_t s);

// TMA strided passes: columns per tile and ring depth per pencil length
template <int N> struct TmaTile {
  static constexpr int T = (N >= 1024) ? 8 : 16;  // T * (N / 256) <= 32 for grouped pencils
  static constexpr int R = 4;
};
template <int N> cudaError_t launch_ymid3_t(const CUtensorMap& mG, const YMidTArgs& a, cudaStream_t s);
template <int N>
cudaError_t launch_last_t(int nd, const CUtensorMap& mAB, const CUtensorMap& mU, const CUtensorMap& mAcc,
                          const LastTArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_op_t(const CUtensorMap& mIn, const OpTArgs& a, cudaStream_t s);
// 2D ideal MHD: x pass and the three Helmholtz projection passes
template <int N> cudaError_t launch_xfirst_mhd(const MhdXArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_proj_xf(const ProjArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_proj_y(const ProjArgs& a, cudaStream_t s);
template <int N> cudaError_t launch_proj_xi(const ProjArgs& a, cudaStream_t s);

inline bool supported_n(int n) {
  return n == 8 || n == 16 || n == 32 || n == 64 || n == 128 || n == 256 || n == 512 || n == 1024;
}
// 1D plans (one CTA per solve, whole steps in shared memory) also take 2048 and 4096
inline bool supported_n_1d(int n) { return supported_n(n) || n == 2048 || n == 4096; }

// Calls f(std::integral_constant<int, N>) for the supported pencil length n.
template <typename F>
cudaError_t dispatch_n(int n, F&& f) {
  switch (n) {
    case 8: return f(std::integral_constant<int, 8>{});
    case 16: return f(std::integral_constant<int, 16>{});
    case 32: return f(std::integral_constant<int, 32>{});
    case 64: return f(std::integral_constant<int, 64>{});
    case 128: return f(std::integral_constant<int, 128>{});
    case 256: return f(std::integral_constant<int, 256>{});
    case 512: return f(std::integral_constant<int, 512>{});
    case 1024: return f(std::integral_constant<int, 1024>{});
    default: return cudaErrorInvalidValue;
  }
}

// As dispatch_n, with the 1D-only lengths 2048 and 4096 (kern_n2048.cu,
// kern_n4096.cu instantiate the 1D step kernel and the contiguous operator).
template <typename F>
cudaError_t dispatch_n_1d(int n, F&& f) {
  if (n == 2048) return f(std::integral_constant<int, 2048>{});
  if (n == 4096) return f(std::integral_constant<int, 4096>{});
  return dispatch_n(n, f);
}

// Dynamic shared memory above 48 KB needs an opt-in; every pass kernel also
// asks for the largest shared-memory carveout so that several CTAs fit per SM.
// Attributes are set once per kernel (the first launch, which must not be
// inside a stream capture); later launches, captured or not, skip the calls.
template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  static std::mutex mu;
  static std::unordered_set<const void*> done;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(reinterpret_cast<const void*>(kernel))) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess && bytes > 48 * 1024)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.insert(reinterpret_cast<const void*>(kernel));
  return e;
}

// Strided passes at tile width T (2D plans choose 4, 8 or 16 columns; 3D
// plans and the 1024-point pencils use TmaTile<N>::T only).
template <int NN, int T>
cudaError_t last_t_T(int nd, const CUtensorMap& mAB, const CUtensorMap& mU, const CUtensorMap& mAcc,
                     const LastTArgs& a, cudaStream_t s) {
  constexpr int R = TmaTile<NN>::R;
  const dim3 grid((a.g.ncol + T - 1) / T, a.g.nouter * a.nsolve);
  const size_t sm = sizeof(TmaStridedSmem<NN, T, R>);
  cudaError_t e;
  const bool fl = a.filter_last && a.stage == 3;  // the launch applies the last filter factor
  if (nd == 3) {
    if constexpr (T == TmaTile<NN>::T) {
      if (fl) {
        if ((e = set_smem(k_last_t<NN, T, 3, false, R>, sm)) != cudaSuccess) return e;
        k_last_t<NN, T, 3, false, R><<<grid, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
      } else {
        if ((e = set_smem(k_last_t<NN, T, 3, false, R, 0, false>, sm)) != cudaSuccess) return e;
        k_last_t<NN, T, 3, false, R, 0, false><<<grid, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
      }
    } else {
      return cudaErrorInvalidValue;
    }
  } else if (a.rhs2d && a.stage < 0) {
    // the right-hand side alone: the unclamped body holds one pair of
    // components at a time (fewer registers, more CTAs per SM); on grids with
    // few column tiles the pairs are split over gridDim.z
    const dim3 gz(grid.x, grid.y, a.pair_groups > 1 ? a.pair_groups : 1);
    if constexpr (NN >= 256) {
      if (a.mhd) {
        if ((e = set_smem(k_last_t<NN, T, 2, false, R, 1, false>, sm)) != cudaSuccess) return e;
        k_last_t<NN, T, 2, false, R, 1, false><<<gz, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
      } else {
        if ((e = set_smem(k_last_t<NN, T, 2, false, R, 0, false>, sm)) != cudaSuccess) return e;
        k_last_t<NN, T, 2, false, R, 0, false><<<gz, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
      }
    } else {
      return cudaErrorInvalidValue;
    }
  } else if (a.mhd) {
    if ((e = set_smem(k_last_t<NN, T, 2, true, R, 1>, sm)) != cudaSuccess) return e;
    k_last_t<NN, T, 2, true, R, 1><<<grid, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
  } else {
    if ((e = set_smem(k_last_t<NN, T, 2, true, R>, sm)) != cudaSuccess) return e;
    k_last_t<NN, T, 2, true, R><<<grid, Shape<NN>::A * T, sm, s>>>(mAB, mU, mAcc, a);
  }
  return cudaGetLastError();
}

template <int NN, int T>
cudaError_t op_t_T(const CUtensorMap& mIn, const OpTArgs& a, cudaStream_t s) {
  constexpr int R = TmaTile<NN>::R;
  const dim3 grid((a.g.ncol + T - 1) / T, a.g.nouter * a.nsolve);
  const size_t sm = sizeof(TmaStridedSmem<NN, T, R>);
  cudaError_t e;
  if ((e = set_smem(k_op_t<NN, T, R>, sm)) != cudaSuccess) return e;
  k_op_t<NN, T, R><<<grid, Shape<NN>::A * T, sm, s>>>(mIn, a);
  return cudaGetLastError();
}

// Calls f(std::integral_constant<int, T>) for the tile width of a launch.
template <int NN, typename F>
cudaError_t dispatch_tcols(int tcols, F&& f) {
  const int T = (tcols > 0) ? tcols : TmaTile<NN>::T;
  if (T == 4) return f(std::integral_constant<int, 4>{});
  if (T == 8) return f(std::integral_constant<int, 8>{});
  if constexpr (TmaTile<NN>::T == 16) {
    if (T == 16) return f(std::integral_constant<int, 16>{});
  }
  return cudaErrorInvalidValue;
}

// Pencils per CTA of the contiguous-pencil passes of 2D/3D plans: the largest
// of TC, TC/2 and TC/4 (never less than one full warp per CTA) whose grid
// still gives two CTAs per SM; at TC, small single solves leave most of the
// 152 SMs idle.  Each pencil's arithmetic is the same at every width, so the
// results do not depend on it.
constexpr int cmax_int(int a, int b) { return a > b ? a : b; }
template <int NN>
struct RowWidths {
  static constexpr int T0 = Tile<NN>::TC;
  static constexpr int TMIN = cmax_int(cmax_int(1, 32 / Shape<NN>::A), T0 / 4);
  static constexpr int T1 = cmax_int(T0 / 2, TMIN);
};
template <int NN, typename F>
cudaError_t dispatch_rows(long units, F&& f) {
  using W = RowWidths<NN>;
  if ((units + W::T0 - 1) / W::T0 >= 2L * 148) return f(std::integral_constant<int, W::T0>{});
  if ((units + W::T1 - 1) / W::T1 >= 2L * 148) return f(std::integral_constant<int, W::T1>{});
  return f(std::integral_constant<int, W::TMIN>{});
}

// Columns per CTA of the projection's y pass over the half spectra (strided
// pencils; the grouped 512/1024-point pencils keep T * N / 256 <= 32): the
// largest of 16, 8, 4 and 2 that gives two CTAs per SM.
template <int NN, typename F>
cudaError_t dispatch_proj_cols(long units, F&& f) {
  constexpr int TMAX = (NN >= 1024) ? 8 : 16;
  constexpr int TMIN = cmax_int(2, 32 / Shape<NN>::A);
  if constexpr (TMAX >= 16 && TMIN <= 16)
    if ((units + 15) / 16 >= 2L * 148) return f(std::integral_constant<int, 16>{});
  if constexpr (TMIN <= 8)
    if ((units + 7) / 8 >= 2L * 148 || TMIN == 8) return f(std::integral_constant<int, 8>{});
  if constexpr (TMIN <= 4)
    if ((units + 3) / 4 >= 2L * 148 || TMIN == 4) return f(std::integral_constant<int, 4>{});
  if constexpr (TMIN <= 2) return f(std::integral_constant<int, 2>{});
  return f(std::integral_constant<int, TMAX>{});
}

// Launchers of the 2D/3D pencil lengths, in four groups so that the largest
// lengths compile as four translation units in parallel: the x pass and the
// operator and y passes, the 1D whole-step kernels, the last pass (every
// stage / clamp / MHD variant), and the 2D MHD x pass with the Helmholtz
// projection.  PS_DEFINE_ALL_LAUNCHERS puts the four in one unit.
#define PS_DEFINE_LAUNCHERS(NN)                                                                       \
  template <>                                                                                         \
  cudaError_t launch_xfirst<NN>(int nd, const XFirstArgs& a, cudaStream_t s) {                        \
    return dispatch_rows<NN>(a.rows, [&](auto tw) -> cudaError_t {                                    \
      constexpr int T = decltype(tw)::value;                                                          \
      const dim3 grid((a.rows + T - 1) / T);                                                          \
      const dim3 block(Shape<NN>::A * T);                                                             \
      cudaError_t e;                                                                                  \
      if (nd == 3) {                                                                                  \
        const size_t sm = sizeof(XFirstSmem<NN, T, 3>);                                               \
        if ((e = set_smem(k_xfirst<NN, T, 3>, sm)) != cudaSuccess) return e;                          \
        k_xfirst<NN, T, 3><<<grid, block, sm, s>>>(a);                                                \
      } else {                                                                                        \
        const size_t sm = sizeof(XFirstSmem<NN, T, 2>);                                               \
        if ((e = set_smem(k_xfirst<NN, T, 2>, sm)) != cudaSuccess) return e;                          \
        k_xfirst<NN, T, 2><<<grid, block, sm, s>>>(a);                                                \
      }                                                                                               \
      return cudaGetLastError();                                                                      \
    });                                                                                               \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_op<NN>(bool strided, const OpArgs& a, cudaStream_t s) {                          \
    if (strided) return cudaErrorInvalidValue; /* strided axes use launch_op_t */                     \
    constexpr int T = Tile<NN>::TC;                                                                   \
    const dim3 grid((a.rows + T - 1) / T);                                                            \
    const size_t sm = sizeof(StridedSmem<NN, T, false>);                                              \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_op<NN, T, false>, sm)) != cudaSuccess) return e;                              \
    k_op<NN, T, false><<<grid, Shape<NN>::A * T, sm, s>>>(a);                                         \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_ymid3_t<NN>(const CUtensorMap& mG, const YMidTArgs& a, cudaStream_t s) {         \
    constexpr int T = TmaTile<NN>::T, R = TmaTile<NN>::R;                                             \
    const dim3 grid((a.g.ncol + T - 1) / T, a.g.nouter * a.nsolve);                                   \
    const size_t sm = sizeof(TmaStridedSmem<NN, T, R>);                                               \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_ymid3_t<NN, T, R>, sm)) != cudaSuccess) return e;                             \
    k_ymid3_t<NN, T, R><<<grid, Shape<NN>::A * T, sm, s>>>(mG, a);                                    \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_op_t<NN>(const CUtensorMap& mIn, const OpTArgs& a, cudaStream_t s) {             \
    return dispatch_tcols<NN>(a.tcols, [&](auto tc) { return op_t_T<NN, decltype(tc)::value>(mIn, a, s); });\
  }

#define PS_DEFINE_STEP1D_LAUNCHERS(NN)                                                                \
  template <>                                                                                         \
  cudaError_t launch_step1d<NN>(const Step1DArgs& a, int nsolve, cudaStream_t s) {                    \
    const size_t sm = sizeof(Step1DSmem<NN>);                                                         \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_step1d<NN>, sm)) != cudaSuccess) return e;                                    \
    k_step1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                 \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_ark1d<NN>(const Ark1DArgs& a, int nsolve, cudaStream_t s) {                      \
    const size_t sm = sizeof(Step1DSmem<NN>);                                                         \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_ark1d<NN>, sm)) != cudaSuccess) return e;                                     \
    k_ark1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                  \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_mhd1d<NN>(const Mhd1DArgs& a, int nsolve, cudaStream_t s) {                      \
    if constexpr (NN > 2048) {                                                                        \
      return cudaErrorInvalidValue; /* 1D MHD pencils up to 2048 points */                            \
    } else {                                                                                          \
      const size_t sm = sizeof(Mhd1DSmem<NN>);                                                        \
      cudaError_t e;                                                                                  \
      if ((e = set_smem(k_mhd1d<NN>, sm)) != cudaSuccess) return e;                                   \
      k_mhd1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                \
      return cudaGetLastError();                                                                      \
    }                                                                                                 \
  }

#define PS_DEFINE_LAST_LAUNCHERS(NN)                                                                  \
  template <>                                                                                         \
  cudaError_t launch_last_t<NN>(int nd, const CUtensorMap& mAB, const CUtensorMap& mU,                \
                                const CUtensorMap& mAcc, const LastTArgs& a, cudaStream_t s) {        \
    return dispatch_tcols<NN>(a.tcols, [&](auto tc) {                                                 \
      return last_t_T<NN, decltype(tc)::value>(nd, mAB, mU, mAcc, a, s);                              \
    });                                                                                               \
  }

#define PS_DEFINE_MHD_LAUNCHERS(NN)                                                                   \
  template <>                                                                                         \
  cudaError_t launch_xfirst_mhd<NN>(const MhdXArgs& a, cudaStream_t s) {                              \
    constexpr int T = Tile<NN>::TC;                                                                   \
    const int tiles = (a.rows + T - 1) / T;                                                           \
    int groups = 1; /* job groups: two CTAs per SM where the grid allows */                           \
    while (groups < 8 && (long)tiles * groups < 2L * 148) groups *= 2;                                \
    const size_t sm = sizeof(MhdXSmem<NN, T>);                                                        \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_xfirst_mhd<NN, T>, sm)) != cudaSuccess) return e;                             \
    k_xfirst_mhd<NN, T><<<dim3(tiles, groups), Shape<NN>::A * T, sm, s>>>(a);                         \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_proj_xf<NN>(const ProjArgs& a, cudaStream_t s) {                                 \
    return dispatch_rows<NN>((long)a.ny * a.nsolve, [&](auto tw) -> cudaError_t {                     \
      constexpr int T = decltype(tw)::value;                                                          \
      const size_t sm = sizeof(MhdXSmem<NN, T>);                                                      \
      cudaError_t e;                                                                                  \
      if ((e = set_smem(k_proj_xf<NN, T>, sm)) != cudaSuccess) return e;                              \
      const int tiles = (a.ny * a.nsolve + T - 1) / T;                                                \
      const int fgroups = (tiles < 2 * 148) ? 2 : 1; /* Bx and By in separate CTAs */                 \
      k_proj_xf<NN, T><<<dim3(tiles, fgroups), Shape<NN>::A * T, sm, s>>>(a);                         \
      return cudaGetLastError();                                                                      \
    });                                                                                               \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_proj_y<NN>(const ProjArgs& a, cudaStream_t s) {                                  \
    return dispatch_proj_cols<NN>((long)a.hx * a.nsolve, [&](auto tw) -> cudaError_t {                \
      constexpr int T = decltype(tw)::value;                                                          \
      const size_t sm = sizeof(ProjYSmem<NN, T>);                                                     \
      cudaError_t e;                                                                                  \
      if ((e = set_smem(k_proj_y<NN, T>, sm)) != cudaSuccess) return e;                               \
      k_proj_y<NN, T><<<dim3((a.hx + T - 1) / T, a.nsolve), Shape<NN>::A * T, sm, s>>>(a);            \
      return cudaGetLastError();                                                                      \
    });                                                                                               \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_proj_xi<NN>(const ProjArgs& a, cudaStream_t s) {                                 \
    return dispatch_rows<NN>((long)a.ny * a.nsolve, [&](auto tw) -> cudaError_t {                     \
      constexpr int T = decltype(tw)::value;                                                          \
      const size_t sm = sizeof(MhdXSmem<NN, T>);                                                      \
      cudaError_t e;                                                                                  \
      if ((e = set_smem(k_proj_xi<NN, T>, sm)) != cudaSuccess) return e;                              \
      k_proj_xi<NN, T><<<(a.ny * a.nsolve + T - 1) / T, Shape<NN>::A * T, sm, s>>>(a);                \
      return cudaGetLastError();                                                                      \
    });                                                                                               \
  }

#define PS_DEFINE_ALL_LAUNCHERS(NN) \
  PS_DEFINE_LAUNCHERS(NN)             \
  PS_DEFINE_STEP1D_LAUNCHERS(NN)      \
  PS_DEFINE_LAST_LAUNCHERS(NN)        \
  PS_DEFINE_MHD_LAUNCHERS(NN)

// Launchers of the 1D-only pencil lengths: the whole-step kernel and the
// contiguous operator (ps_derivative / ps_filter / 1D ps_rhs).
#define PS_DEFINE_LAUNCHERS_1D(NN)                                                                    \
  template <>                                                                                         \
  cudaError_t launch_op<NN>(bool strided, const OpArgs& a, cudaStream_t s) {                          \
    if (strided) return cudaErrorInvalidValue;                                                        \
    constexpr int T = Tile<NN>::TC;                                                                   \
    const dim3 grid((a.rows + T - 1) / T);                                                            \
    const size_t sm = sizeof(StridedSmem<NN, T, false>);                                              \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_op<NN, T, false>, sm)) != cudaSuccess) return e;                              \
    k_op<NN, T, false><<<grid, Shape<NN>::A * T, sm, s>>>(a);                                         \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_step1d<NN>(const Step1DArgs& a, int nsolve, cudaStream_t s) {                    \
    const size_t sm = sizeof(Step1DSmem<NN>);                                                         \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_step1d<NN>, sm)) != cudaSuccess) return e;                                    \
    k_step1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                 \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_ark1d<NN>(const Ark1DArgs& a, int nsolve, cudaStream_t s) {                      \
    const size_t sm = sizeof(Step1DSmem<NN>);                                                         \
    cudaError_t e;                                                                                    \
    if ((e = set_smem(k_ark1d<NN>, sm)) != cudaSuccess) return e;                                     \
    k_ark1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                  \
    return cudaGetLastError();                                                                        \
  }                                                                                                   \
  template <>                                                                                         \
  cudaError_t launch_mhd1d<NN>(const Mhd1DArgs& a, int nsolve, cudaStream_t s) {                      \
    if constexpr (NN > 2048) {                                                                        \
      return cudaErrorInvalidValue; /* 1D MHD pencils up to 2048 points */                            \
    } else {                                                                                          \
      const size_t sm = sizeof(Mhd1DSmem<NN>);                                                        \
      cudaError_t e;                                                                                  \
      if ((e = set_smem(k_mhd1d<NN>, sm)) != cudaSuccess) return e;                                   \
      k_mhd1d<NN><<<nsolve, Shape<NN>::A, sm, s>>>(a);                                                \
      return cudaGetLastError();                                                                      \
    }                                                                                                 \
  }

}  // namespace ps
