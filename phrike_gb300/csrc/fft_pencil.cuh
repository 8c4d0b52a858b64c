// Register-resident pencil FFTs for the pseudo-spectral pass kernels.
//
// A pencil of N = A*B complex points is owned by A threads.  The forward
// transform is a two-step (four-step without the explicit transpose pass)
// decomposition:
//   input layout    : thread t holds x[t + A*n2],         n2 = 0..B-1
//   step 1          : B-point DFT in registers, twiddle W_N^{t*k2}
//   exchange        : one shared-memory transpose
//   step 2          : B/A A-point DFTs per thread
//   spectral layout : register j*A+k1 of thread t holds X[(t + A*j) + B*k1]
// The inverse runs the same steps backwards and returns to the input layout,
// so a forward/multiply/inverse round trip never reorders data in memory.
//
// All in-register DFTs are radix-2 decimation-in-time with compile-time
// twiddles; the constants are produced at compile time by a Taylor series
// after octant reduction (see ct_cos2pi / ct_sin2pi).
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

namespace ps {

// ---------------------------------------------------------------- constexpr trig
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int n = 1; n < 16; ++n) {
    term *= -x * x / double((2 * n) * (2 * n + 1));
    sum += term;
  }
  return sum;
}
constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n < 16; ++n) {
    term *= -x * x / double((2 * n - 1) * (2 * n));
    sum += term;
  }
  return sum;
}
// cos/sin of 2*pi*num/den, reduced to [0, pi/4] by octant with exact integer
// arithmetic on the residual.
constexpr void cs2pi(long num, long den, double& c, double& s) {
  long r = ((num % den) + den) % den;
  long q = (8 * r) / den;                                     // octant 0..7
  double phi = kPi * double(8 * r - q * den) / double(4 * den);        // [0, pi/4)
  double psi = kPi * double((q + 1) * den - 8 * r) / double(4 * den);  // pi/4 - phi
  double Cp = taylor_cos(phi), Sp = taylor_sin(phi);
  double Cq = taylor_cos(psi), Sq = taylor_sin(psi);
  switch (q) {
    case 0: c = Cp; s = Sp; break;
    case 1: c = Sq; s = Cq; break;
    case 2: c = -Sp; s = Cp; break;
    case 3: c = -Cq; s = Sq; break;
    case 4: c = -Cp; s = -Sp; break;
    case 5: c = -Sq; s = -Cq; break;
    case 6: c = Sp; s = -Cp; break;
    default: c = Cq; s = -Sq; break;
  }
}
constexpr double ct_cos2pi(long num, long den) { double c = 0, s = 0; cs2pi(num, den, c, s); return c; }
constexpr double ct_sin2pi(long num, long den) { double c = 0, s = 0; cs2pi(num, den, c, s); return s; }

// ---------------------------------------------------------------- static_for
template <int I, int E, typename F>
__device__ __forceinline__ void sfor(F&& f) {
  if constexpr (I < E) {
    f(std::integral_constant<int, I>{});
    sfor<I + 1, E>(f);
  }
}

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }
constexpr int bitrev(int i, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
  return r;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}

// d * exp(-+ 2 pi i J / M)   (forward sign -, inverse sign +)
template <int M, int J, bool INV>
__device__ __forceinline__ float2 twmul(float2 d) {
  if constexpr (J == 0) {
    return d;
  } else if constexpr (4 * J == M) {
    return INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  } else if constexpr (8 * J == M) {
    constexpr float r = 0.70710678118654752440f;
    return INV ? make_float2((d.x - d.y) * r, (d.y + d.x) * r)
               : make_float2((d.x + d.y) * r, (d.y - d.x) * r);
  } else if constexpr (8 * J == 3 * M) {
    constexpr float r = 0.70710678118654752440f;
    return INV ? make_float2((-d.x - d.y) * r, (d.x - d.y) * r)
               : make_float2((d.y - d.x) * r, (-d.y - d.x) * r);
  } else {
    constexpr float c = (float)ct_cos2pi(J, M);
    constexpr float s = (float)ct_sin2pi(J, M);
    return INV ? make_float2(fmaf(d.x, c, -d.y * s), fmaf(d.y, c, d.x * s))
               : make_float2(fmaf(d.x, c, d.y * s), fmaf(d.y, c, -d.x * s));
  }
}

// Radix-2 decimation-in-time butterfly a, b -> a + W b, a - W b with the
// compile-time twiddle W = exp(-+ 2 pi i J / M) = c + i s.  A nontrivial W
// is applied as W b = w * u with u = b + i tau b (two FMAs) and the scale w
// folded into the butterfly (four FMAs): six instructions instead of the
// eight of a complex multiply and two complex adds.  tau = s/c, w = c when
// |c| >= |s|, else tau = c/s, w = s, so |tau| <= 1.
template <int M, int J, bool INV>
__device__ __forceinline__ void bfly_dit(float2& a, float2& b) {
  const float2 x = a;
  if constexpr (J == 0 || 4 * J == M) {
    const float2 wb = twmul<M, J, INV>(b);
    a = cadd(x, wb);
    b = csub(x, wb);
  } else {
    constexpr double cd = ct_cos2pi(J, M);
    constexpr double sd = INV ? ct_sin2pi(J, M) : -ct_sin2pi(J, M);
    constexpr bool by_c = (cd < 0 ? -cd : cd) >= (sd < 0 ? -sd : sd);
    constexpr float tau = by_c ? float(sd / cd) : float(cd / sd);
    constexpr float w = by_c ? float(cd) : float(sd);
    float2 u;
    if constexpr (by_c) u = make_float2(fmaf(-tau, b.y, b.x), fmaf(tau, b.x, b.y));
    else u = make_float2(fmaf(tau, b.x, -b.y), fmaf(tau, b.y, b.x));
    a = make_float2(fmaf(w, u.x, x.x), fmaf(w, u.y, x.y));
    b = make_float2(fmaf(-w, u.x, x.x), fmaf(-w, u.y, x.y));
  }
}

// In-register DFT of L points starting at v[OFF]; natural order in and out.
// Radix-2 decimation in time: the bit-reversed input order is a compile-time
// renaming of registers, then log2(L) butterfly stages.
template <int L, bool INV, int OFF = 0, int CAP>
__device__ __forceinline__ void dft(float2 (&v)[CAP]) {
  if constexpr (L > 1) {
    constexpr int LOG = ilog2(L);
    float2 tmp[L];
    sfor<0, L>([&](auto ic) { tmp[decltype(ic)::value] = v[OFF + bitrev(decltype(ic)::value, LOG)]; });
    sfor<0, L>([&](auto ic) { v[OFF + decltype(ic)::value] = tmp[decltype(ic)::value]; });
    sfor<0, LOG>([&](auto sc) {
      constexpr int h = 1 << decltype(sc)::value;
      sfor<0, L / (2 * h)>([&](auto gc) {
        constexpr int start = OFF + decltype(gc)::value * 2 * h;
        sfor<0, h>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          bfly_dit<2 * h, j, INV>(v[start + j], v[start + j + h]);
        });
      });
    });
  }
}

// ---------------------------------------------------------------- pencil shapes
template <int N> struct Shape;
template <> struct Shape<8> { static constexpr int A = 2, B = 4; };
template <> struct Shape<16> { static constexpr int A = 4, B = 4; };
template <> struct Shape<32> { static constexpr int A = 4, B = 8; };
template <> struct Shape<64> { static constexpr int A = 8, B = 8; };
template <> struct Shape<128> { static constexpr int A = 8, B = 16; };
template <> struct Shape<256> { static constexpr int A = 16, B = 16; };
// N > 256: G = N/256 groups of 16 threads (see PencilGrp)
template <> struct Shape<512> { static constexpr int A = 32, B = 16; };
template <> struct Shape<1024> { static constexpr int A = 64, B = 16; };
template <> struct Shape<2048> { static constexpr int A = 128, B = 16; };  // 1D plans only
template <> struct Shape<4096> { static constexpr int A = 256, B = 16; };

// Exchange-buffer layout for T pencils.  Element (q, s) of pencil p, with
// q in [0,B) and s in [0,A).  In the contiguous-lane layout (the A threads of
// a pencil are adjacent lanes) each pencil owns a padded block; in the strided
// layout (lanes run over pencils) pencils are interleaved innermost.  Both are
// bank-conflict free for the access patterns below.
//
// WSYNC: every pencil's threads sit in one warp and every warp is full
// (contiguous layout, A <= 32, A*T a multiple of 32), so the exchanges only
// need a warp barrier; warps then run their transforms independently.
template <int N, int T, bool STRIDED, bool WSYNC = false>
struct PencilBase {
  static constexpr int A = Shape<N>::A;
  static constexpr int B = Shape<N>::B;
  static constexpr int J = B / A;
  static_assert(B % A == 0, "pencil shape needs B multiple of A");
  // contiguous layout: rows of A + 2 elements once A >= 16, so that a thread's
  // A consecutive elements start on a 16-byte boundary and move as 128-bit
  // words (conflict-free: eight lanes cover the 32 banks); A + 1 below
  static constexpr int PAD = STRIDED ? 0 : (A >= 16 ? 2 : 1);
  static constexpr bool VEC = !STRIDED && A >= 16;
  // contiguous layout: pencil blocks of B*(A+1) float2, rounded up to = A
  // (mod 16) when A < 16, so that the pencils sharing a warp fall on
  // different banks (A lanes x 8 bytes each)
  static constexpr int PBLK0 = B * (A + PAD);
  static constexpr int PBLK = (STRIDED || A >= 16) ? PBLK0 : PBLK0 + (((A - PBLK0 % 16) % 16) + 16) % 16;
  static constexpr int BUF = STRIDED ? T * B * A : T * PBLK;  // float2 elements
  static_assert(!WSYNC || (!STRIDED && A <= 32 && (A * T) % 32 == 0), "warp barrier needs warp-local pencils");

  static __device__ __forceinline__ void bar() {
    if constexpr (WSYNC) __syncwarp();
    else __syncthreads();
  }

  int p;   // pencil within the tile
  int t;   // thread within the pencil
  float2* buf;
  const float2* twf;  // [B][A]: W_N^{n1 k2}
  const float2* twi;  // [A][B]: W_N^{-n1 k2}

  __device__ __forceinline__ int xi(int q, int s) const {
    if constexpr (STRIDED) return (q * A + s) * T + p;
    else return p * PBLK + q * (A + PAD) + s;
  }
  // spectral index of register r = j*A + k1
  __device__ __forceinline__ int kidx(int r) const { return t + A * (r / A) + B * (r % A); }

  __device__ __forceinline__ void fwd(float2 (&v)[B]) const {
    dft<B, false>(v);
    sfor<1, B>([&](auto kc) {
      constexpr int k2 = decltype(kc)::value;
      v[k2] = cmul(v[k2], twf[k2 * A + t]);
    });
    bar();
    sfor<0, B>([&](auto kc) {
      constexpr int k2 = decltype(kc)::value;
      buf[xi(k2, t)] = v[k2];
    });
    bar();
    sfor<0, J>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (VEC) {
        const float4* src = reinterpret_cast<const float4*>(buf + xi(t + A * j, 0));
        sfor<0, A / 2>([&](auto hc) {
          constexpr int h = decltype(hc)::value;
          const float4 w = src[h];
          v[j * A + 2 * h] = make_float2(w.x, w.y);
          v[j * A + 2 * h + 1] = make_float2(w.z, w.w);
        });
      } else {
        sfor<0, A>([&](auto nc) {
          constexpr int n1 = decltype(nc)::value;
          v[j * A + n1] = buf[xi(t + A * j, n1)];
        });
      }
      dft<A, false, j * A>(v);
    });
  }

  __device__ __forceinline__ void inv(float2 (&v)[B]) const {
    sfor<0, J>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      dft<A, true, j * A>(v);
      sfor<1, A>([&](auto nc) {
        constexpr int n1 = decltype(nc)::value;
        v[j * A + n1] = cmul(v[j * A + n1], twi[n1 * B + t + A * j]);
      });
    });
    bar();
    sfor<0, J>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (VEC) {
        float4* dst = reinterpret_cast<float4*>(buf + xi(t + A * j, 0));
        sfor<0, A / 2>([&](auto hc) {
          constexpr int h = decltype(hc)::value;
          dst[h] = make_float4(v[j * A + 2 * h].x, v[j * A + 2 * h].y, v[j * A + 2 * h + 1].x,
                               v[j * A + 2 * h + 1].y);
        });
      } else {
        sfor<0, A>([&](auto nc) {
          constexpr int n1 = decltype(nc)::value;
          buf[xi(t + A * j, n1)] = v[j * A + n1];
        });
      }
    });
    bar();
    sfor<0, B>([&](auto kc) {
      constexpr int k2 = decltype(kc)::value;
      v[k2] = buf[xi(k2, t)];
    });
    dft<B, true>(v);
  }

  // vn[r] = X[-k(r) mod N] for a pencil in spectral layout.
  __device__ __forceinline__ void negk(const float2 (&v)[B], float2 (&vn)[B]) const {
    bar();
    sfor<0, B>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      buf[xi(t + A * (r / A), r % A)] = v[r];
    });
    bar();
    sfor<0, B>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      constexpr int k1 = r % A;
      const int k2 = t + A * (r / A);
      const int q = (k2 == 0) ? 0 : (B - k2);
      const int s = (k2 == 0) ? ((A - k1) % A) : (A - 1 - k1);
      vn[r] = buf[xi(q, s)];
    });
  }
};

// Pencils of N = G * 256 points (G = 2 or 4).  Pencil thread t' = G*t + g
// (t in [0,16), group g in [0,G)) holds positions t' + 16G*n2, i.e. point
// t + 16*n2 of the decimated sub-pencil x_g[m] = x[G*m + g].  The forward
// transform runs the 256-point PencilBase transform on every sub-pencil,
// multiplies S_g[k] by W_N^{g k} and finishes with a G-point DFT across the
// groups (radix-2 decimation in frequency over warp shuffles: every group of
// a pencil lives in the same warp).  Group g then holds
// X[k + 256 * bitrev(g)], k = t + 16 r.  The inverse runs the same steps in
// reverse (decimation in time with conjugate twiddles).
//
// Tables (N entries each, shared layout): twf/twi[0..255] are the 256-point
// sub-pencil twiddles, twf[256*g + k] = W_N^{g k} and twi[256*g + k] =
// W_N^{-g k} for g = 1..G-1, k < 256.
template <int N, int T, bool STRIDED>
struct PencilGrp {
  static constexpr int G = N / 256;
  static constexpr int A = Shape<N>::A;  // 16 * G
  static constexpr int B = Shape<N>::B;  // 16
  static constexpr int LG = ilog2(G);
  // a pencil of A <= 32 threads is one full warp: its sub-pencils exchange within it
  using Sub = PencilBase<256, T * G, STRIDED, (!STRIDED && A <= 32 && (A * T) % 32 == 0)>;
  static constexpr int BUF = Sub::BUF;
  static_assert(!STRIDED || T * G <= 32, "all groups of a pencil must share a warp");

  int p;   // pencil within the tile
  int t;   // pencil thread t' = G * t_sub + g
  float2* buf;
  const float2* twf;
  const float2* twi;

  __device__ __forceinline__ int g() const { return t % G; }
  __device__ __forceinline__ int ts() const { return t / G; }
  __device__ __forceinline__ Sub sub() const { return Sub{p * G + g(), ts(), buf, twf, twi}; }
  // lane distance between groups g and g ^ 1 of the same pencil thread
  __device__ __forceinline__ int lane_step() const { return STRIDED ? T : 1; }
  __device__ __forceinline__ int kidx(int r) const {
    return ts() + 16 * r + 256 * bitrev(g(), LG);
  }

  __device__ __forceinline__ void fwd(float2 (&v)[B]) const {
    sub().fwd(v);
    const int gg = g(), t0 = ts();
    if (gg > 0) {
#pragma unroll
      for (int r = 0; r < B; ++r) v[r] = cmul(v[r], twf[256 * gg + t0 + 16 * r]);
    }
    // G-point DFT across the groups, decimation in frequency
#pragma unroll
    for (int h = G / 2; h >= 1; h /= 2) {
      const int lane_x = h * lane_step();
      const bool upper = (gg & h) != 0;
      const int j = gg % h;  // position inside the 2h block
      float c = 1.0f, sn = 0.0f;
      if (h == 2) {  // W_4^{j}
        c = (j == 0) ? 1.0f : 0.0f;
        sn = (j == 0) ? 0.0f : -1.0f;
      } else if (h > 2) {  // W_{2h}^{j} = exp(-i pi j / h)
        sincospif((float)j / (float)h, &sn, &c);
        sn = -sn;
      }
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, v[r].x, lane_x),
                                     __shfl_xor_sync(0xffffffffu, v[r].y, lane_x));
        if (!upper) {
          v[r] = cadd(v[r], o);
        } else {
          const float2 d = csub(o, v[r]);  // lower - upper
          v[r] = make_float2(d.x * c - d.y * sn, d.x * sn + d.y * c);
        }
      }
    }
  }

  __device__ __forceinline__ void inv(float2 (&v)[B]) const {
    const int gg = g(), t0 = ts();
    // G-point inverse DFT across the groups, decimation in time (bit-reversed in)
#pragma unroll
    for (int h = 1; h <= G / 2; h *= 2) {
      const int lane_x = h * lane_step();
      const bool upper = (gg & h) != 0;
      const int j = gg % h;
      float c = 1.0f, sn = 0.0f;
      if (h == 2) {  // conj(W_4^{j})
        c = (j == 0) ? 1.0f : 0.0f;
        sn = (j == 0) ? 0.0f : 1.0f;
      } else if (h > 2) {  // conj(W_{2h}^{j}) = exp(+i pi j / h)
        sincospif((float)j / (float)h, &sn, &c);
      }
#pragma unroll
      for (int r = 0; r < B; ++r) {
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, v[r].x, lane_x),
                                     __shfl_xor_sync(0xffffffffu, v[r].y, lane_x));
        // lower holds x[i], upper holds x[i+h]; t = x[i+h] * w
        const float2 up = upper ? v[r] : o;
        const float2 lo = upper ? o : v[r];
        const float2 tw = make_float2(up.x * c - up.y * sn, up.x * sn + up.y * c);
        v[r] = upper ? csub(lo, tw) : cadd(lo, tw);
      }
    }
    if (gg > 0) {
#pragma unroll
      for (int r = 0; r < B; ++r) v[r] = cmul(v[r], twi[256 * gg + t0 + 16 * r]);
    }
    sub().inv(v);
  }
};

template <int N, int T, bool STRIDED>
using Pencil = typename std::conditional<
    (N > 256), PencilGrp<N, T, STRIDED>,
    PencilBase<N, T, STRIDED, (!STRIDED && Shape<N>::A <= 32 && (Shape<N>::A * T) % 32 == 0)>>::type;

}  // namespace ps
