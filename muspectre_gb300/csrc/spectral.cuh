// Spectral passes of the FFT-Galerkin operator (device code + launchers).
//
// A real field is stored as component planes [c][pixel] (pixels row-major, last
// index fastest); its half spectrum as [c][k] complex with the last axis halved to
// n/2+1.  One transform = one pass per axis:
//
//   last axis   (pass "last"):  r2c / c2r of rows, two real rows packed into one
//                               complex FFT (x + i y); fused prologue / epilogue
//                               (tangent K:dF, CG vector updates, dot products)
//   middle axis (pass "axis"):  c2c of strided pencils, 3-D only
//   first axis  (pass "green"): c2c of strided pencils with all components of a
//                               k-point in one block, so that the Green operator
//                               (projection_small_strain.cc:56-86,
//                               projection_finite_strain_fast.cc:61-87) is applied
//                               between the forward and the inverse transform.
//
// The CG operator of one iteration is therefore: last(fwd, prologue) -> axis(fwd)
// -> green -> axis(inv) -> last(inv, epilogue), the projection of
// src/fft/projection_default.cc:54-63 with the tangent contraction of
// src/cell/cell_base.cc:182-188 fused into the first pass.
#pragma once

#include "fft_device.cuh"

namespace musg {

enum Prologue : int { PRO_PLAIN = 0, PRO_TANGENT = 1, PRO_CG = 2 };
enum Epilogue : int { EPI_PLAIN = 0, EPI_CG = 1 };
enum GreenMode : int { GM_SMALL = 0, GM_FINITE = 1, GM_FWD = 2, GM_INV = 3 };

// ------------------------------------------------------------ reductions
template <typename R> struct Acc {
  R s = R(0), c = R(0);
  // Neumaier's compensated summation (Neumaier 1974)
  __device__ __forceinline__ void add(R x) {
    R t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
template <> struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};

// sum of v over the block, result valid in thread 0
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = (l < nw) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// ------------------------------------------------------------ tangents
// small strain, isotropic: lam tr(e) I + mu (e + e^T)
template <int D, typename R>
__device__ __forceinline__ void tangent_small(const R *e, R lam, R mu, R *out) {
  R tr = R(0);
#pragma unroll
  for (int i = 0; i < D; ++i) tr += e[i + D * i];
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) out[i + D * j] = mu * (e[i + D * j] + e[j + D * i]) + (i == j ? lam * tr : R(0));
}

// finite strain, PK2/Green-Lagrange isotropic law linearised:
// K:dF = dF S + F (lam tr(A) I + mu (A + A^T)),  A = F^T dF
// (materials_toolbox.hh:313-350 contracted with dF)
template <int D, typename R>
__device__ __forceinline__ void tangent_finite(const R *dF, const R *F, const R *S, R lam, R mu, R *out) {
  R A[D * D];
#pragma unroll
  for (int n = 0; n < D; ++n)
#pragma unroll
    for (int s = 0; s < D; ++s) {
      R a = R(0);
#pragma unroll
      for (int j = 0; j < D; ++j) a += F[j + D * s] * dF[j + D * n];
      A[s + D * n] = a;
    }
  R tr = R(0);
#pragma unroll
  for (int i = 0; i < D; ++i) tr += A[i + D * i];
  R B[D * D];
#pragma unroll
  for (int m = 0; m < D; ++m)
#pragma unroll
    for (int r = 0; r < D; ++r) B[r + D * m] = mu * (A[r + D * m] + A[m + D * r]) + (r == m ? lam * tr : R(0));
#pragma unroll
  for (int m = 0; m < D; ++m)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      R v = R(0);
#pragma unroll
      for (int n = 0; n < D; ++n) v += dF[i + D * n] * S[n + D * m];
#pragma unroll
      for (int r = 0; r < D; ++r) v += F[i + D * r] * B[r + D * m];
      out[i + D * m] = v;
    }
}

// j-independent Kirchhoff tangent (materials_toolbox.hh:374-410 as written):
// K(i,m,j,n) = K'(i,m,n)  =>  (K:dF)(i,m) = sum_n K'(i,m,n) sum_j dF(j,n)
template <int D, typename R>
__device__ __forceinline__ void tangent_kprime(const R *dF, const R *Kp, R *out) {
  R cs[D];
#pragma unroll
  for (int n = 0; n < D; ++n) {
    R v = R(0);
#pragma unroll
    for (int j = 0; j < D; ++j) v += dF[j + D * n];
    cs[n] = v;
  }
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    R v = R(0);
#pragma unroll
    for (int n = 0; n < D; ++n) v += Kp[c + D * D * n] * cs[n];
    out[c] = v;
  }
}

template <int D, int TK, typename R>
__device__ __forceinline__ void apply_tangent(const TangentData<R> &td, long long px, long long npx,
                                              const R *in, R *out) {
  constexpr int D2 = D * D;
  int kind = TK;
  if constexpr (TK == TK_MIXED) kind = td.law_kind[td.mat[px]];
  if constexpr (TK == TK_SMALL) {
    tangent_small<D, R>(in, td.lam[px], td.mu[px], out);
  } else if (kind == TK_FINITE) {
    R F[D2], S[D2];
#pragma unroll
    for (int c = 0; c < D2; ++c) F[c] = td.F[c * npx + px];
#pragma unroll
    for (int c = 0; c < D2; ++c) S[c] = td.S[c * npx + px];
    tangent_finite<D, R>(in, F, S, td.lam[px], td.mu[px], out);
  } else {
    R Kp[D2 * D];
#pragma unroll
    for (int c = 0; c < D2 * D; ++c) Kp[c] = td.Kp[c * npx + px];
    tangent_kprime<D, R>(in, Kp, out);
  }
}

// ------------------------------------------------------------ pass "last"
template <typename R> struct LastArgs {
  AxisPlanD<R> ap;
  int L, H, G, ncomp;
  long long nrows, npx, nk;
  typename V2<R>::T *spec;
  const R *in;
  R *out;
  R scale;
  const CGState *st;
  const R *r;
  R *p;
  R *Ap;
  double *partial;
  TangentData<R> td;
};

// forward: real rows -> half spectra.  D is the tensor dimension for the tangent
// prologues (0 for PRO_PLAIN).
template <typename R, int PRO, int D, int TK>
__global__ void __launch_bounds__(kPassThreads) k_last_fwd(const LastArgs<R> a) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (PRO == PRO_CG && !a.st->active) return;
  const int L = a.L, G = a.G, nc = a.ncomp, G2 = G >> 1;
  const int P = nc * G2;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long row0 = (long long)blockIdx.x * G;
  R *bufr = reinterpret_cast<R *>(buf);
  if constexpr (PRO == PRO_PLAIN) {
    for (int idx = threadIdx.x; idx < nc * G * L; idx += blockDim.x) {
      const int c = idx / (G * L);
      const int rem = idx - c * G * L;
      const int g = rem / L, e = rem - g * L;
      const long long row = row0 + g;
      R v = R(0);
      if (row < a.nrows) v = a.in[(long long)c * a.npx + row * L + e] * a.scale;
      bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)] = v;
    }
  } else {
    constexpr int D2 = D * D;
    const bool first = (PRO == PRO_CG) ? (a.st->iter == 0) : false;
    const R beta = (PRO == PRO_CG) ? R(a.st->beta) : R(0);
    for (int idx = threadIdx.x; idx < G * L; idx += blockDim.x) {
      const int g = idx / L, e = idx - g * L;
      const long long row = row0 + g;
      R out[D2];
      if (row < a.nrows) {
        const long long px = row * L + e;
        R v[D2];
        if (PRO == PRO_CG) {
#pragma unroll
          for (int c = 0; c < D2; ++c) {
            const long long o = (long long)c * a.npx + px;
            R pv = -a.r[o];
            if (!first) pv += beta * a.p[o];
            a.p[o] = pv;
            v[c] = pv;
          }
        } else {
#pragma unroll
          for (int c = 0; c < D2; ++c) v[c] = a.in[(long long)c * a.npx + px];
        }
        apply_tangent<D, TK, R>(a.td, px, a.npx, v, out);
      } else {
#pragma unroll
        for (int c = 0; c < D2; ++c) out[c] = R(0);
      }
#pragma unroll
      for (int c = 0; c < D2; ++c) bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)] = out[c];
    }
  }
  __syncthreads();
  const T *res = fft_run<R, false>(buf, buf2, P, a.ap);
  // unpack the two real spectra: X = (Z_k + conj Z_{L-k})/2, Y = -i (Z_k - conj Z_{L-k})/2
  const int H = a.H;
  for (int idx = threadIdx.x; idx < nc * G * H; idx += blockDim.x) {
    const int c = idx / (G * H);
    const int rem = idx - c * G * H;
    const int gr = rem / H, k = rem - gr * H;
    const long long row = row0 + gr;
    if (row >= a.nrows) continue;
    const int q = c * G2 + (gr >> 1);
    const int kn = (k == 0) ? 0 : L - k;
    const T z = res[k * P + q], zn = res[kn * P + q];
    T o;
    if ((gr & 1) == 0) o = T{R(0.5) * (z.x + zn.x), R(0.5) * (z.y - zn.y)};
    else o = T{R(0.5) * (z.y + zn.y), R(-0.5) * (z.x - zn.x)};
    a.spec[(long long)c * a.nk + row * H + k] = o;
  }
}

// inverse: half spectra -> real rows.  PLAIN writes out = scale*x; CG writes Ap
// and the block sums of p.Ap.
template <typename R, int EPI, int D>
__global__ void __launch_bounds__(kPassThreads) k_last_inv(const LastArgs<R> a) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (EPI == EPI_CG && !a.st->active) return;
  const int L = a.L, G = a.G, nc = a.ncomp, G2 = G >> 1, H = a.H;
  const int P = nc * G2;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long row0 = (long long)blockIdx.x * G;
  const bool even = (L & 1) == 0;
  for (int idx = threadIdx.x; idx < nc * G2 * H; idx += blockDim.x) {
    const int c = idx / (G2 * H);
    const int rem = idx - c * G2 * H;
    const int g2 = rem / H, k = rem - g2 * H;
    const long long rx = row0 + 2 * g2, ry = rx + 1;
    T X = T{R(0), R(0)}, Y = T{R(0), R(0)};
    if (rx < a.nrows) X = a.spec[(long long)c * a.nk + rx * H + k];
    if (ry < a.nrows) Y = a.spec[(long long)c * a.nk + ry * H + k];
    const bool selfconj = (k == 0) || (even && 2 * k == L);
    if (selfconj) { X.y = R(0); Y.y = R(0); }  // c2r uses the real part only
    const int q = c * G2 + g2;
    buf[k * P + q] = T{X.x - Y.y, X.y + Y.x};
    if (!selfconj) buf[(L - k) * P + q] = T{X.x + Y.y, Y.x - X.y};
  }
  __syncthreads();
  const R *bufr = reinterpret_cast<const R *>(fft_run<R, true>(buf, buf2, P, a.ap));
  if constexpr (EPI == EPI_PLAIN) {
    for (int idx = threadIdx.x; idx < nc * G * L; idx += blockDim.x) {
      const int c = idx / (G * L);
      const int rem = idx - c * G * L;
      const int g = rem / L, e = rem - g * L;
      const long long row = row0 + g;
      if (row < a.nrows) a.out[(long long)c * a.npx + row * L + e] = a.scale * bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)];
    }
  } else {
    constexpr int D2 = D * D;
    Acc<R> acc;
    for (int idx = threadIdx.x; idx < G * L; idx += blockDim.x) {
      const int g = idx / L, e = idx - g * L;
      const long long row = row0 + g;
      if (row >= a.nrows) continue;
      const long long px = row * L + e;
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        const R v = bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)];
        const long long o = (long long)c * a.npx + px;
        a.Ap[o] = v;
        acc.add(a.p[o] * v);
      }
    }
    const double bs = block_sum(acc.value());
    if (threadIdx.x == 0) a.partial[blockIdx.x] = bs;
  }
}

// ------------------------------------------------------------ pass "axis"
template <typename R> struct AxisArgs {
  AxisPlanD<R> ap;
  int nax, T, ntiles;
  long long se, inner, sb;
  typename V2<R>::T *spec;
  const CGState *st;
};

template <typename R, bool INV>
__global__ void __launch_bounds__(kPassThreads) k_axis(const AxisArgs<R> a) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (a.st && !a.st->active) return;
  const int tile = blockIdx.x % a.ntiles;
  const long long batch = blockIdx.x / a.ntiles;
  const int Tt = a.T;
  T *buf2 = buf + (size_t)Tt * a.ap.m;
  T *base = a.spec + batch * a.sb;
  const long long pos0 = (long long)tile * Tt;
  for (int idx = threadIdx.x; idx < a.nax * Tt; idx += blockDim.x) {
    const int e = idx / Tt, t = idx - e * Tt;
    const long long pos = pos0 + t;
    buf[idx] = (pos < a.inner) ? base[e * a.se + pos] : T{R(0), R(0)};
  }
  __syncthreads();
  const T *res = fft_run<R, INV>(buf, buf2, Tt, a.ap);
  for (int idx = threadIdx.x; idx < a.nax * Tt; idx += blockDim.x) {
    const int e = idx / Tt, t = idx - e * Tt;
    const long long pos = pos0 + t;
    if (pos < a.inner) base[e * a.se + pos] = res[idx];
  }
}

// ------------------------------------------------------------ pass "green"
template <typename R> struct GreenArgs {
  AxisPlanD<R> ap;
  int n0, T, ncomp, n1, nh;
  long long Rr, nk;
  typename V2<R>::T *spec;
  const R *xi0, *xi1, *xi2;
  int nyq0, nyq1, nyq2;
  R norm;
  const CGState *st;
};

template <typename R, int MODE, int D>
__global__ void __launch_bounds__(kPassThreads) k_green(const GreenArgs<R> a) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (a.st && !a.st->active) return;
  const int Tt = a.T, nc = a.ncomp, n0 = a.n0;
  const int P = nc * Tt;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long rho0 = (long long)blockIdx.x * Tt;
  for (int idx = threadIdx.x; idx < nc * n0 * Tt; idx += blockDim.x) {
    const int t = idx % Tt;
    const int rest = idx / Tt;
    const int e = rest % n0, c = rest / n0;
    const long long rho = rho0 + t;
    buf[e * P + c * Tt + t] = (rho < a.Rr) ? a.spec[(long long)c * a.nk + e * a.Rr + rho] : T{R(0), R(0)};
  }
  __syncthreads();
  T *cur = buf;
  if (MODE != GM_INV) cur = fft_run<R, false>(buf, buf2, P, a.ap);
  if constexpr (MODE == GM_SMALL || MODE == GM_FINITE) {
    constexpr int D2 = D * D;
    for (int idx = threadIdx.x; idx < n0 * Tt; idx += blockDim.x) {
      const int e = idx / Tt, t = idx - e * Tt;
      const long long rho = rho0 + t;
      if (rho >= a.Rr) continue;
      int k1, k2 = 0;
      if (D == 3) {
        k1 = (int)(rho / a.nh);
        k2 = (int)(rho - (long long)k1 * a.nh);
      } else {
        k1 = (int)rho;
      }
      R xi[D];
      xi[0] = a.xi0[e];
      xi[1] = a.xi1[k1];
      if (D == 3) xi[D - 1] = a.xi2[k2];
      bool zero = (e == 0 && k1 == 0 && k2 == 0) || e == a.nyq0 || k1 == a.nyq1 || (D == 3 && k2 == a.nyq2);
      T f[D2];
#pragma unroll
      for (int c = 0; c < D2; ++c) f[c] = cur[e * P + c * Tt + t];
      T o[D2];
      if (zero) {
#pragma unroll
        for (int c = 0; c < D2; ++c) o[c] = T{R(0), R(0)};
      } else {
        R n2 = R(0);
#pragma unroll
        for (int d = 0; d < D; ++d) n2 += xi[d] * xi[d];
        const R inv = R(1) / sqrt(n2);
#pragma unroll
        for (int d = 0; d < D; ++d) xi[d] *= inv;
        if (MODE == GM_FINITE) {
          // f <- (f xi) xi^T   (projection_finite_strain_fast.cc:79-85)
#pragma unroll
          for (int i = 0; i < D; ++i) {
            T fx = T{R(0), R(0)};
#pragma unroll
            for (int j = 0; j < D; ++j) {
              fx.x += f[i + D * j].x * xi[j];
              fx.y += f[i + D * j].y * xi[j];
            }
#pragma unroll
            for (int j = 0; j < D; ++j) o[i + D * j] = T{fx.x * xi[j] * a.norm, fx.y * xi[j] * a.norm};
          }
        } else {
          // Ghat f = 1/2 (xi a^T + a xi^T) - xi xi^T (xi^T f xi),  a = (f + f^T) xi
          // (the contraction of projection_small_strain.cc:64-77 with f)
          T av[D];
          T s = T{R(0), R(0)};
#pragma unroll
          for (int i = 0; i < D; ++i) {
            T v = T{R(0), R(0)};
#pragma unroll
            for (int j = 0; j < D; ++j) {
              v.x += (f[i + D * j].x + f[j + D * i].x) * xi[j];
              v.y += (f[i + D * j].y + f[j + D * i].y) * xi[j];
              s.x += xi[i] * f[i + D * j].x * xi[j];
              s.y += xi[i] * f[i + D * j].y * xi[j];
            }
            av[i] = v;
          }
#pragma unroll
          for (int j = 0; j < D; ++j)
#pragma unroll
            for (int i = 0; i < D; ++i) {
              const R xx = xi[i] * xi[j];
              o[i + D * j] = T{(R(0.5) * (xi[i] * av[j].x + av[i].x * xi[j]) - xx * s.x) * a.norm,
                               (R(0.5) * (xi[i] * av[j].y + av[i].y * xi[j]) - xx * s.y) * a.norm};
            }
        }
      }
#pragma unroll
      for (int c = 0; c < D2; ++c) cur[e * P + c * Tt + t] = o[c];
    }
    __syncthreads();
  }
  if (MODE != GM_FWD) cur = fft_run<R, true>(cur, cur == buf ? buf2 : buf, P, a.ap);
  for (int idx = threadIdx.x; idx < nc * n0 * Tt; idx += blockDim.x) {
    const int t = idx % Tt;
    const int rest = idx / Tt;
    const int e = rest % n0, c = rest / n0;
    const long long rho = rho0 + t;
    if (rho < a.Rr) a.spec[(long long)c * a.nk + e * a.Rr + rho] = cur[e * P + c * Tt + t];
  }
}

}  // namespace musg
