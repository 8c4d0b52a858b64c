// In-place Stockham FFTs of pencils in shared memory for runtime lengths
// 2^a 3^b 5^c (radix-4, 3, 5 and 2 stages), shared by the mixed-radix pass
// kernels (mixed_radix.cu) and the NUFFT resampling passes (nufft.cu).
#pragma once
#include <cuda_runtime.h>

#include "mixed_radix.cuh"

namespace ps {
namespace mrfft {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
// floor(j / d) for 0 <= j < 2^21, through the float reciprocal: (j + 1/2)
// (1/d) is within (j/d) 2^-22 of its exact value, less than the distance
// 1/(2d) to the nearest integer.
__device__ __forceinline__ int qdiv(int j, float inv_d) { return __float2int_rz(((float)j + 0.5f) * inv_d); }

// -i z for the forward transform, +i z for the inverse
__device__ __forceinline__ float2 rot(float2 z, bool inv) {
  return inv ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x);
}

// Small DFTs X_k = sum_n v_n exp(-+2 pi i k n / R), constants from their
// closed forms: sin(2 pi/3) = sqrt(3)/2; cos(2 pi/5) = (sqrt(5) - 1)/4,
// cos(4 pi/5) = -(sqrt(5) + 1)/4, sin(2 pi/5) = sqrt((5 + sqrt(5))/8),
// sin(4 pi/5) = sqrt((5 - sqrt(5))/8).
template <int R>
__device__ __forceinline__ void dft_small(float2 (&v)[R], bool inv);

template <>
__device__ __forceinline__ void dft_small<2>(float2 (&v)[2], bool) {
  const float2 a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}
template <>
__device__ __forceinline__ void dft_small<4>(float2 (&v)[4], bool inv) {
  const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  const float2 t2 = cadd(v[1], v[3]), t3 = rot(csub(v[1], v[3]), inv);
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}
template <>
__device__ __forceinline__ void dft_small<3>(float2 (&v)[3], bool inv) {
  constexpr float s3 = 0.86602540378443864676f;
  const float2 t = cadd(v[1], v[2]);
  const float2 u = rot(cscale(csub(v[1], v[2]), s3), inv);
  const float2 m = make_float2(fmaf(-0.5f, t.x, v[0].x), fmaf(-0.5f, t.y, v[0].y));
  v[0] = cadd(v[0], t);
  v[1] = cadd(m, u);
  v[2] = csub(m, u);
}
template <>
__device__ __forceinline__ void dft_small<5>(float2 (&v)[5], bool inv) {
  constexpr float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
  constexpr float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
  const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const float2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  const float2 x0 = v[0];
  const float2 a1 = make_float2(x0.x + fmaf(c1, t1.x, c2 * t2.x), x0.y + fmaf(c1, t1.y, c2 * t2.y));
  const float2 a2 = make_float2(x0.x + fmaf(c2, t1.x, c1 * t2.x), x0.y + fmaf(c2, t1.y, c1 * t2.y));
  const float2 b1 = rot(make_float2(fmaf(s1, t3.x, s2 * t4.x), fmaf(s1, t3.y, s2 * t4.y)), inv);
  const float2 b2 = rot(make_float2(fmaf(s2, t3.x, -s1 * t4.x), fmaf(s2, t3.y, -s1 * t4.y)), inv);
  v[0] = cadd(x0, cadd(t1, t2));
  v[1] = cadd(a1, b1);
  v[4] = csub(a1, b1);
  v[2] = cadd(a2, b2);
  v[3] = csub(a2, b2);
}

// One Stockham stage of radix R over one pencil, in two phases around a
// block barrier: every thread first reads and transforms its butterflies into
// registers (at most MJ of them: ntp >= n/16 keeps ceil(n / (R ntp)) <= MJ),
// then writes them back.  The register file v is shared by all radices so
// that the stage loop keeps one set of live values.
__host__ __device__ constexpr int mr_mj(int R) { return (kMrDiv + R - 1) / R; }
__host__ __device__ constexpr int mr_max(int a, int b) { return a > b ? a : b; }
constexpr int kMrV = mr_max(mr_max(2 * mr_mj(2), 3 * mr_mj(3)), mr_max(4 * mr_mj(4), 5 * mr_mj(5)));
constexpr int kMrJ = mr_mj(2);

template <int R, int MJ>
__device__ __forceinline__ void mr_read(const float2* buf, int n, int ns, const float2* tw, int tp,
                                        int ntp, bool act, bool inv, float2 (&v)[kMrV], int (&dst)[kMrJ]) {
  static_assert(MJ * R <= kMrV && MJ <= kMrJ, "stage register budget");
  const int nb = n / R;
  const int tstep = n / (ns * R);
  const float ins = 1.0f / (float)ns;
#pragma unroll
  for (int jj = 0; jj < MJ; ++jj) {
    const int j = tp + jj * ntp;
    dst[jj] = -1;
    if (act && j < nb) {
      const int k = j - qdiv(j, ins) * ns;
      float2 x[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        x[r] = buf[j + r * nb];
        if (r > 0) {
          const float2 w = tw[k * r * tstep];
          x[r] = inv ? cmulc(x[r], w) : cmul(x[r], w);
        }
      }
      dft_small<R>(x, inv);
#pragma unroll
      for (int r = 0; r < R; ++r) v[jj * R + r] = x[r];
      dst[jj] = (j - k) * R + k;
    }
  }
}

template <int R, int MJ>
__device__ __forceinline__ void mr_write(float2* buf, int ns, const float2 (&v)[kMrV], const int (&dst)[kMrJ]) {
#pragma unroll
  for (int jj = 0; jj < MJ; ++jj)
    if (dst[jj] >= 0)
#pragma unroll
      for (int r = 0; r < R; ++r) buf[dst[jj] + r * ns] = v[jj * R + r];
}

// In-place transforms of npen pencils (pitch float2 apart) starting at base;
// unnormalised in both directions.  All threads of the block must call it.
__device__ __forceinline__ void mr_fft(float2* base, int pitch, int npen, const MrAxis& ax, bool inv) {
  const int q = threadIdx.x / ax.ntp, tp = threadIdx.x - q * ax.ntp;
  const bool act = q < npen;
  float2* buf = base + (long)(act ? q : 0) * pitch;
  float2 v[kMrV];
  int dst[kMrJ];
  __syncthreads();
  int ns = 1;
#pragma unroll 1
  for (int s = 0; s < ax.nst; ++s) {
    const int R = (int)((ax.rcode >> (4 * s)) & 15u);
    if (R == 4) mr_read<4, mr_mj(4)>(buf, ax.n, ns, ax.tw, tp, ax.ntp, act, inv, v, dst);
    else if (R == 3) mr_read<3, mr_mj(3)>(buf, ax.n, ns, ax.tw, tp, ax.ntp, act, inv, v, dst);
    else if (R == 5) mr_read<5, mr_mj(5)>(buf, ax.n, ns, ax.tw, tp, ax.ntp, act, inv, v, dst);
    else mr_read<2, mr_mj(2)>(buf, ax.n, ns, ax.tw, tp, ax.ntp, act, inv, v, dst);
    __syncthreads();
    if (R == 4) mr_write<4, mr_mj(4)>(buf, ns, v, dst);
    else if (R == 3) mr_write<3, mr_mj(3)>(buf, ns, v, dst);
    else if (R == 5) mr_write<5, mr_mj(5)>(buf, ns, v, dst);
    else mr_write<2, mr_mj(2)>(buf, ns, v, dst);
    __syncthreads();
    ns *= R;
  }
}

}  // namespace mrfft
}  // namespace ps
