// Shared-memory FFT core for pencils of one axis (device code).
//
// Algorithm: Stockham auto-sort FFT (decimation in time), mixed radix
// 2/3/4/5/7/8/9/16 (9 and 16 as 3x3 and 4x4 in registers),
// in the formulation of Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors" (SC'08): for each stage of radix R with span
// Ns (product of the radices already applied),
//     v[r] = x[j + r*m/R] * W_m^(k*r*m/(Ns*R)),  k = j mod Ns,
//     v    = DFT_R(v),
//     y[(j/Ns)*Ns*R + k + r*Ns] = v[r].
// P pencils of length m live in shared memory as buf[e*P + p] (element-major) so
// that consecutive threads touch consecutive pencils.  Stages ping-pong between
// two shared-memory buffers, one butterfly in registers per thread at a time and
// one barrier per stage.
//
// Lengths with a prime factor above 7 use Bluestein's algorithm (L. Bluestein,
// "A linear filtering approach to the computation of the discrete Fourier
// transform", 1970): X = w . IDFT_m(DFT_m(x . w) . DFT_m(conj w))/m with the chirp
// w[j] = exp(-pi i j^2/n) and m >= 2n-1 a 2/3/5/7-smooth length.
//
// Both directions are unnormalised (FFTW convention): forward uses exp(-2 pi i/m),
// inverse exp(+2 pi i/m).
#pragma once

#include "musg_internal.h"

namespace musg {

// Exact division of small non-negative integers by a runtime divisor without the
// integer-division instruction sequence: q0 = trunc(n * rcp(d)) in FP32 is within one
// of n/d for 0 <= n < 2^22 (the relative error of the product is below 2^-23 and
// n/d < 2^22), and one remainder correction makes it exact.
struct FDiv {
  int d;
  float inv;
  // IEEE division (no fast-math): the correctly rounded reciprocal
  __device__ __forceinline__ explicit FDiv(int d_) : d(d_), inv(1.0f / (float)d_) {}
  __device__ __forceinline__ int div(int n, int &r) const {
    int q = __float2int_rz(__int2float_rn(n) * inv);
    r = n - q * d;
    if (r < 0) {
      q -= 1;
      r += d;
    } else if (r >= d) {
      q += 1;
      r -= d;
    }
    return q;
  }
  __device__ __forceinline__ int div(int n) const {
    int r;
    return div(n, r);
  }
};

template <typename T> __device__ __forceinline__ T cadd(T a, T b) { return T{a.x + b.x, a.y + b.y}; }
template <typename T> __device__ __forceinline__ T csub(T a, T b) { return T{a.x - b.x, a.y - b.y}; }
template <typename T> __device__ __forceinline__ T cmul(T a, T b) {
  return T{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename T> __device__ __forceinline__ T mul_mi(T a) {
  return INV ? T{-a.y, a.x} : T{a.y, -a.x};
}

// -------------------------------------------------------------- small DFTs
template <int R, bool INV, typename T> struct Dft;

template <bool INV, typename T> struct Dft<2, INV, T> {
  static __device__ __forceinline__ void run(T *v) {
    T a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV, typename T> struct Dft<4, INV, T> {
  static __device__ __forceinline__ void run(T *v) {
    T t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    T t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <bool INV, typename T> struct Dft<8, INV, T> {
  static __device__ __forceinline__ void run(T *v) {
    using R = decltype(v[0].x);
    const R s = R(0.7071067811865475244008);
    T e[4] = {v[0], v[2], v[4], v[6]};
    T o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV, T>::run(e);
    Dft<4, INV, T>::run(o);
    // o[k] *= W8^k  (W8 = exp(-+ i pi/4))
    T o1 = INV ? T{s * (o[1].x - o[1].y), s * (o[1].x + o[1].y)}
               : T{s * (o[1].x + o[1].y), s * (o[1].y - o[1].x)};
    T o2 = mul_mi<INV>(o[2]);
    T o3 = INV ? T{-s * (o[3].x + o[3].y), s * (o[3].x - o[3].y)}
               : T{s * (o[3].y - o[3].x), -s * (o[3].x + o[3].y)};
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};

template <bool INV, typename T> struct Dft<3, INV, T> {
  static __device__ __forceinline__ void run(T *v) {
    using R = decltype(v[0].x);
    const R c = R(-0.5), s = R(0.8660254037844386467637);
    T t = cadd(v[1], v[2]);
    T d = csub(v[1], v[2]);
    T m = T{v[0].x + c * t.x, v[0].y + c * t.y};
    // i*s*d: forward y1 = m - i s d, inverse y1 = m + i s d
    T isd = T{-s * d.y, s * d.x};
    v[0] = cadd(v[0], t);
    v[1] = INV ? cadd(m, isd) : csub(m, isd);
    v[2] = INV ? csub(m, isd) : cadd(m, isd);
  }
};

// cos/sin(2 pi j / P) for the odd prime radices (j < P, folded to immediates once
// the loops below are unrolled)
template <int P> struct PrimeCS;
template <> struct PrimeCS<5> {
  static __device__ __forceinline__ double c(int j) {
    return j == 0 ? 1.0 : (j == 1 || j == 4) ? 0.3090169943749474241023 : -0.8090169943749474241023;
  }
  static __device__ __forceinline__ double s(int j) {
    return j == 0 ? 0.0 : j == 1 ? 0.9510565162951535721164 : j == 2 ? 0.5877852522924731291687
           : j == 3 ? -0.5877852522924731291687 : -0.9510565162951535721164;
  }
};
template <> struct PrimeCS<7> {
  static __device__ __forceinline__ double c(int j) {
    return j == 0 ? 1.0 : (j == 1 || j == 6) ? 0.623489801858733530525
           : (j == 2 || j == 5) ? -0.2225209339563144042889 : -0.9009688679024191262361;
  }
  static __device__ __forceinline__ double s(int j) {
    return j == 0 ? 0.0 : j == 1 ? 0.7818314824680298087084 : j == 2 ? 0.9749279121818236070181
           : j == 3 ? 0.4338837391175581204758 : j == 4 ? -0.4338837391175581204758
           : j == 5 ? -0.9749279121818236070181 : -0.7818314824680298087084;
  }
};

// odd prime radix P via the symmetric pair decomposition
//   y[k]   = x0 + sum_q a_q cos(2 pi kq/P) -+ i sum_q b_q sin(2 pi kq/P)
//   y[P-k] = x0 + sum_q a_q cos(2 pi kq/P) +- i sum_q b_q sin(2 pi kq/P)
// with a_q = x_q + x_{P-q}, b_q = x_q - x_{P-q}
template <int P, bool INV, typename T> struct DftPrime {
  static __device__ __forceinline__ void run(T *v) {
    using R = decltype(v[0].x);
    constexpr int H = (P - 1) / 2;
    T a[H], b[H];
#pragma unroll
    for (int q = 0; q < H; ++q) {
      a[q] = cadd(v[q + 1], v[P - 1 - q]);
      b[q] = csub(v[q + 1], v[P - 1 - q]);
    }
    const T x0 = v[0];
    T y0 = x0;
#pragma unroll
    for (int q = 0; q < H; ++q) y0 = cadd(y0, a[q]);
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      T re = x0, im = T{R(0), R(0)};
#pragma unroll
      for (int q = 1; q <= H; ++q) {
        const R c = R(PrimeCS<P>::c((k * q) % P)), s = R(PrimeCS<P>::s((k * q) % P));
        re.x += c * a[q - 1].x;
        re.y += c * a[q - 1].y;
        im.x += s * b[q - 1].x;
        im.y += s * b[q - 1].y;
      }
      const T iim = T{-im.y, im.x};
      v[k] = INV ? cadd(re, iim) : csub(re, iim);
      v[P - k] = INV ? csub(re, iim) : cadd(re, iim);
    }
    v[0] = y0;
  }
};

// cos/sin(2 pi j / N) for the composite radices 16 and 9 (j < N)
template <int N> struct CompCS;
template <> struct CompCS<16> {
  static __device__ __forceinline__ double c(int j) {
    constexpr double a = 0.9238795325112867561282, b = 0.7071067811865475244008, g = 0.3826834323650897717285;
    return j == 0 ? 1.0 : j == 1 ? a : j == 2 ? b : j == 3 ? g : j == 4 ? 0.0 : j == 5 ? -g : j == 6 ? -b
           : j == 7 ? -a : j == 8 ? -1.0 : j == 9 ? -a : j == 10 ? -b : j == 11 ? -g : j == 12 ? 0.0
           : j == 13 ? g : j == 14 ? b : a;
  }
  static __device__ __forceinline__ double s(int j) { return c((j + 12) & 15); }  // sin x = cos(x - pi/2)
};
template <> struct CompCS<9> {
  static __device__ __forceinline__ double c(int j) {
    return j == 0 ? 1.0 : (j == 1 || j == 8) ? 0.7660444431189780352024 : (j == 2 || j == 7) ? 0.1736481776669303488517
           : (j == 3 || j == 6) ? -0.5 : -0.9396926207859083840541;
  }
  static __device__ __forceinline__ double s(int j) {
    return j == 0 ? 0.0 : j == 1 ? 0.6427876096865393263226 : j == 2 ? 0.9848077530122080593667
           : j == 3 ? 0.8660254037844386467637 : j == 4 ? 0.3420201433256687330441
           : j == 5 ? -0.3420201433256687330441 : j == 6 ? -0.8660254037844386467637
           : j == 7 ? -0.9848077530122080593667 : -0.6427876096865393263226;
  }
};

// composite radix N = N1 * N2 in registers (Cooley-Tukey): N2 DFTs of length N1 over
// the stride-N2 subsequences, twiddles W_N^(n2 k1), then N1 DFTs of length N2
template <int N1, int N2, bool INV, typename T> struct DftComposite {
  static __device__ __forceinline__ void run(T *v) {
    using R = decltype(v[0].x);
    constexpr int N = N1 * N2;
    T a[N2][N1];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) {
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) a[n2][n1] = v[N2 * n1 + n2];
      Dft<N1, INV, T>::run(a[n2]);
#pragma unroll
      for (int k1 = 1; k1 < N1; ++k1) {
        const int j = (n2 * k1) % N;
        if (j == 0) continue;
        const R c = R(CompCS<N>::c(j)), sn = R(CompCS<N>::s(j));
        const T w = INV ? T{c, sn} : T{c, -sn};
        a[n2][k1] = cmul(a[n2][k1], w);
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
      T b[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) b[n2] = a[n2][k1];
      Dft<N2, INV, T>::run(b);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) v[k1 + N1 * k2] = b[k2];
    }
  }
};

template <bool INV, typename T> struct Dft<16, INV, T> {
  static __device__ __forceinline__ void run(T *v) { DftComposite<4, 4, INV, T>::run(v); }
};
template <bool INV, typename T> struct Dft<9, INV, T> {
  static __device__ __forceinline__ void run(T *v) { DftComposite<3, 3, INV, T>::run(v); }
};

template <bool INV, typename T> struct Dft<5, INV, T> {
  static __device__ __forceinline__ void run(T *v) { DftPrime<5, INV, T>::run(v); }
};
template <bool INV, typename T> struct Dft<7, INV, T> {
  static __device__ __forceinline__ void run(T *v) { DftPrime<7, INV, T>::run(v); }
};

// -------------------------------------------------------------- one stage
// out-of-place: reads src, writes dst (both P pencils of length m, element-major)
template <typename R, int RAD, bool INV>
__device__ __forceinline__ void fft_stage(const typename V2<R>::T *__restrict__ src,
                                          typename V2<R>::T *__restrict__ dst, int P, int m, int Ns,
                                          const typename V2<R>::T *__restrict__ tw) {
  using T = typename V2<R>::T;
  const int nb = m / RAD;
  const int total = nb * P;
  const int tws = m / (Ns * RAD);
  const FDiv fP(P), fNs(Ns);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int p, k;
    const int j = fP.div(t, p);
    fNs.div(j, k);
    T v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[r] = src[(j + r * nb) * P + p];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < RAD; ++r) {
        T w = __ldg(&tw[k * r * tws]);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    Dft<RAD, INV, T>::run(v);
    const int o = ((j - k) * RAD + k) * P + p;
#pragma unroll
    for (int r = 0; r < RAD; ++r) dst[o + r * Ns * P] = v[r];
  }
  __syncthreads();
}

// All stages of a plan; data starts in a, b is scratch of the same size.  Returns
// the buffer that holds the result.
template <typename R, bool INV>
__device__ __forceinline__ typename V2<R>::T *fft_stages(typename V2<R>::T *a, typename V2<R>::T *b, int P,
                                                          const AxisPlanD<R> &ap) {
  using T = typename V2<R>::T;
  int Ns = 1;
  unsigned long long code = ap.rcode;
  T *src = a, *dst = b;
  for (int s = 0; s < ap.nst; ++s, code >>= 5) {
    const int rad = (int)(code & 31ull);
    switch (rad) {
      case 2: fft_stage<R, 2, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 3: fft_stage<R, 3, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 4: fft_stage<R, 4, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 5: fft_stage<R, 5, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 7: fft_stage<R, 7, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 9: fft_stage<R, 9, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      case 8: fft_stage<R, 8, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
      default: fft_stage<R, 16, INV>(src, dst, P, ap.m, Ns, ap.tw); break;
    }
    Ns *= rad;
    T *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// Length-n DFT of P pencils held in a[e*P + p], e < n.  a and b each hold ap.m*P
// entries; returns the buffer (a or b) with the result in its first n*P entries.
// The caller synchronises after writing a; this routine ends with a barrier.
template <typename R, bool INV>
__device__ __forceinline__ typename V2<R>::T *fft_run(typename V2<R>::T *a, typename V2<R>::T *b, int P,
                                                       const AxisPlanD<R> &ap) {
  using T = typename V2<R>::T;
  if (!ap.blu) return fft_stages<R, INV>(a, b, P, ap);
  const int n = ap.n, m = ap.m;
  const int tot = m * P;
  const FDiv fP(P);
  // x . w (conj(x) for the inverse: IDFT(x) = conj(DFT(conj x))), zero padded
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int e = fP.div(i);
    if (e < n) {
      T x = a[i];
      if (INV) x.y = -x.y;
      a[i] = cmul(x, __ldg(&ap.chirp[e]));
    } else {
      a[i] = T{R(0), R(0)};
    }
  }
  __syncthreads();
  T *c = fft_stages<R, false>(a, b, P, ap);
  T *d = (c == a) ? b : a;
  for (int i = threadIdx.x; i < tot; i += blockDim.x) c[i] = cmul(c[i], __ldg(&ap.bf[fP.div(i)]));
  __syncthreads();
  c = fft_stages<R, true>(c, d, P, ap);
  for (int i = threadIdx.x; i < n * P; i += blockDim.x) {
    T x = cmul(c[i], __ldg(&ap.chirp[fP.div(i)]));
    if (INV) x.y = -x.y;
    c[i] = x;
  }
  __syncthreads();
  return c;
}

}  // namespace musg
