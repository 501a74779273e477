// Register-resident pencil FFT passes for power-of-two lengths 16..256 (device code).
//
// A length M = R1 * R2 (R2 divides R1) transform is the two-stage Stockham network of
// fft_device.cuh with a fixed thread mapping instead of a loop over butterflies:
//   stage 1: lane y < Y = M / R1 holds x[y + Y r] (r < R1) in registers straight from
//            global memory, applies DFT_R1 and writes slot y R1 + r of its pencil in
//            shared memory;
//   stage 2: after one barrier, lane y takes the butterflies j = y + Y b (b < R1 / R2):
//            inputs slot j + R1 r (r < R2), twiddles W_M^(j r), DFT_R2, giving X[j + R1 r],
//            stored straight to global memory (or kept for the Green operator).
// The unnormalised inverse is the adjoint network in mirror order: IDFT_R2 of
// X[j + R1 r] followed by the conjugate twiddles, written back to the same slots; one
// barrier; IDFT_R1 of slots y R1 + r gives x[y + Y r].  Every index is a compile-time
// constant or a multiply-add of the thread coordinates, the radices are unrolled, and
// shared memory holds one buffer (no ping-pong), so a block keeps more pencils in
// flight than the generic path.
//
// Thread block: (T pencils of a tile, Y lanes, NC components); the pencils of a tile are
// T consecutive positions of the contiguous inner extent, so a warp reads and writes
// rows of T consecutive complex values.
#pragma once

#include "spectral.cuh"

namespace musg {

template <int M> struct RegPlan;
template <> struct RegPlan<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct RegPlan<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct RegPlan<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct RegPlan<128> { static constexpr int R1 = 16, R2 = 8; };
template <> struct RegPlan<256> { static constexpr int R1 = 16, R2 = 16; };

template <int M> struct RegFft {
  static constexpr int R1 = RegPlan<M>::R1, R2 = RegPlan<M>::R2;
  static constexpr int Y = M / R1;
  static constexpr int NB = R1 / R2;
  static_assert(R1 * R2 == M && R1 % R2 == 0 && Y == R2, "two-stage plan");
};

inline bool reg_fft_length(int m) { return m == 16 || m == 32 || m == 64 || m == 128 || m == 256; }

// stage-2 twiddle W_M^(j r) (j < R1, r < R2, so j r < M) from the block's shared
// copy of the plan's table (stage_twiddles)
template <bool CONJ, typename T>
__device__ __forceinline__ T reg_tw(const T *tw, int idx) {
  T w = tw[idx];
  if (CONJ) w.y = -w.y;
  return w;
}

// copy the plan's twiddle table W_M^k (k < M) into shared memory, by the whole block;
// a barrier must separate it from the first reg_tw.  Per-thread loads of the table
// from global memory (L1 hits) made the stage-2 butterflies wait on the load pipe:
// the last-axis inverse ran 63.5 us with them and 49.2 us with the shared copy.
template <int M, typename T>
__device__ __forceinline__ void stage_twiddles(T *dst, const T *__restrict__ src) {
  for (int k = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); k < M;
       k += blockDim.x * blockDim.y * blockDim.z)
    dst[k] = src[k];
}

// ------------------------------------------------------------ middle-axis pass
// pencils along axis 1 of [c][k0][k1][k2h]: AxisArgs as for k_axis, blockIdx.x =
// tile + ntiles * slab, blockIdx.z = problem of a batched launch
template <typename R, int M, bool INV>
__global__ void __launch_bounds__(512) k_axis_reg(const AxisArgs<R> a0) {
  dep_wait();
  using T = typename V2<R>::T;
  using F = RegFft<M>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  AxisArgs<R> a = a0;
  if (a0.batch) {
    a.spec = a0.batch[blockIdx.z].spec;
    a.st = a0.batch[blockIdx.z].st;
  }
  if (a.st && !a.st->active) return;
  const int Tt = blockDim.x, t = threadIdx.x, y = threadIdx.y;
  T *tws = buf + (size_t)Tt * M;  // after the tile
  stage_twiddles<M>(tws, a.ap.tw);
  const int tile = blockIdx.x % a.ntiles;
  const long long slab = blockIdx.x / a.ntiles;
  const long long pos = (long long)tile * Tt + t;
  const bool ok = pos < a.inner;
  T *base = a.spec + slab * a.sb + pos;
  const long long se = a.se;
  if (!INV) {
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = ok ? base[(y + F::Y * r) * se] : T{R(0), R(0)};
    Dft<F::R1, false, T>::run(v);
#pragma unroll
    for (int r = 0; r < F::R1; ++r) buf[(y * F::R1 + r) * Tt + t] = v[r];
    __syncthreads();
#pragma unroll
    for (int b = 0; b < F::NB; ++b) {
      const int j = y + F::Y * b;
      T w[F::R2];
#pragma unroll
      for (int r = 0; r < F::R2; ++r) w[r] = buf[(j + F::R1 * r) * Tt + t];
#pragma unroll
      for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], reg_tw<false>(tws, j * r));
      Dft<F::R2, false, T>::run(w);
      if (ok) {
#pragma unroll
        for (int r = 0; r < F::R2; ++r) base[(j + F::R1 * r) * se] = w[r];
      }
    }
  } else {
    __syncthreads();  // the twiddle copy
#pragma unroll
    for (int b = 0; b < F::NB; ++b) {
      const int j = y + F::Y * b;
      T w[F::R2];
#pragma unroll
      for (int r = 0; r < F::R2; ++r) w[r] = ok ? base[(j + F::R1 * r) * se] : T{R(0), R(0)};
      Dft<F::R2, true, T>::run(w);
#pragma unroll
      for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], reg_tw<true>(tws, j * r));
#pragma unroll
      for (int r = 0; r < F::R2; ++r) buf[(j + F::R1 * r) * Tt + t] = w[r];
    }
    __syncthreads();
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = buf[(y * F::R1 + r) * Tt + t];
    Dft<F::R1, true, T>::run(v);
    if (ok) {
#pragma unroll
      for (int r = 0; r < F::R1; ++r) base[(y + F::Y * r) * se] = v[r];
    }
  }
}

// ------------------------------------------------------------ Green pass
// first-axis forward FFT, Green operator, first-axis inverse FFT on the spectrum
// [c][k0][rho] (rho = k1 * nh + k2 in 3-D, k1 in 2-D).  Finite strain couples the D
// components of one row i of the tensor only: blockIdx.y = i, threadIdx.z = j picks
// component i + D j.  Small strain couples all D^2: threadIdx.z = component,
// gridDim.y = 1.  blockIdx.z = problem of a batched launch.  Shared memory:
// slot-major [slot][z][t], NC * T pencils of M entries.
template <typename R, int M, int MODE, int D>
__global__ void __launch_bounds__(384, 2) k_green_reg(const GreenArgs<R> a0) {
  dep_wait();
  using T = typename V2<R>::T;
  using F = RegFft<M>;
  static_assert(MODE == GM_SMALL || MODE == GM_FINITE, "projection modes only");
  constexpr int NC = MODE == GM_FINITE ? D : D * D;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  GreenArgs<R> a = a0;
  if (a0.batch) {
    a.spec = a0.batch[blockIdx.z].spec;
    a.st = a0.batch[blockIdx.z].st;
  }
  if (a.st && !a.st->active) return;
  const int Tt = blockDim.x, t = threadIdx.x, y = threadIdx.y, z = threadIdx.z;
  const int P = NC * Tt;
  const int comp = MODE == GM_FINITE ? (int)blockIdx.y + D * z : z;
  const long long rho = (long long)blockIdx.x * Tt + t;
  const bool ok = rho < a.Rr;
  T *base = a.spec + (long long)comp * a.nk + rho;
  const long long se = a.Rr;
  T *col = buf + z * Tt + t;  // this thread's pencil: slot s at col[s * P]
  T *tws = buf + (size_t)P * M;  // after the tile
  stage_twiddles<M>(tws, a.ap.tw);
  {
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = ok ? base[(y + F::Y * r) * se] : T{R(0), R(0)};
    Dft<F::R1, false, T>::run(v);
#pragma unroll
    for (int r = 0; r < F::R1; ++r) col[(y * F::R1 + r) * P] = v[r];
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < F::NB; ++b) {
    const int j = y + F::Y * b;
    T w[F::R2];
#pragma unroll
    for (int r = 0; r < F::R2; ++r) w[r] = col[(j + F::R1 * r) * P];
#pragma unroll
    for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], reg_tw<false>(tws, j * r));
    Dft<F::R2, false, T>::run(w);
#pragma unroll
    for (int r = 0; r < F::R2; ++r) col[(j + F::R1 * r) * P] = w[r];  // X[j + R1 r], own slots
  }
  __syncthreads();
  // Green operator on the k-points (e, rho) of this tile: e strided over the Y*NC
  // threads of column t
  if (ok) {
    int k1, k2 = 0;
    if (D == 3) {
      k1 = (int)(rho / a.nh);
      k2 = (int)(rho - (long long)k1 * a.nh);
    } else {
      k1 = (int)rho;
    }
    const R x1 = a.xi1[k1], x2 = D == 3 ? a.xi2[k2] : R(0);
    T *tc = buf + t;
    for (int e = y + F::Y * z; e < M; e += F::Y * NC) {
      R xi[D];
      xi[0] = a.xi0[e];
      xi[1] = x1;
      if (D == 3) xi[D - 1] = x2;
      T f[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) f[c] = tc[e * P + c * Tt];
      if (!unit_xi<D>(xi, e, k1, k2, a.nyq0, a.nyq1, a.nyq2)) {
#pragma unroll
        for (int c = 0; c < NC; ++c) f[c] = T{R(0), R(0)};
      } else if (MODE == GM_FINITE) {
        green_finite_row<D>(f, xi, a.norm);
      } else {
        T o[NC];
        green_small<D>(f, o, xi, a.norm);
#pragma unroll
        for (int c = 0; c < NC; ++c) f[c] = o[c];
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) tc[e * P + c * Tt] = f[c];
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < F::NB; ++b) {
    const int j = y + F::Y * b;
    T w[F::R2];
#pragma unroll
    for (int r = 0; r < F::R2; ++r) w[r] = col[(j + F::R1 * r) * P];
    Dft<F::R2, true, T>::run(w);
#pragma unroll
    for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], reg_tw<true>(tws, j * r));
#pragma unroll
    for (int r = 0; r < F::R2; ++r) col[(j + F::R1 * r) * P] = w[r];
  }
  __syncthreads();
  {
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = col[(y * F::R1 + r) * P];
    Dft<F::R1, true, T>::run(v);
    if (ok) {
#pragma unroll
      for (int r = 0; r < F::R1; ++r) base[(y + F::Y * r) * se] = v[r];
    }
  }
}

// ------------------------------------------------------------ last-axis passes
// Real rows of length L = M along the contiguous axis, two rows (2 g2, 2 g2 + 1) of one
// component packed as the real and imaginary parts of one complex pencil.  Thread
// block (Y lanes, Q = ncomp * G/2 pencils): lanes are the fastest thread index so that
// a warp reads and writes consecutive entries of a row.  A pencil sits in shared memory
// with slot s at position s + s / R1 (one pad entry per R1 slots), which keeps the
// stride-R1 accesses of stage 1 free of bank conflicts.
template <int M> struct LastLayout {
  static constexpr int R1 = RegFft<M>::R1;
  static constexpr int PS = M + M / R1;  // entries per pencil
  static __device__ __forceinline__ int pos(int s) { return s + s / R1; }
};

// forward with the CG prologue of the FP32 inner solve (PRO_CGF): p = -r + beta p
// (p = -r on the first iteration), v = K:p per pixel, spectrum of v, and the per-warp
// sums of p.v (cg_alpha finishes alpha = r.r / p.(K:p) from them).  FP32 only.
// At most 72 registers (blocks of up to 512 threads still fit): the pass is bound by
// load latency, and at 82 registers only five blocks of 144 threads shared an SM; six
// took the 128^3 pass from 84.3 to 79.1 us (no spills for the isotropic tangents).
template <int M, int D, int TK>
__global__ void __maxnreg__(72) k_last_fwd_reg(const LastArgs<float> a0) {
  dep_wait();
  using R = float;
  using T = float2;
  using F = RegFft<M>;
  using Lay = LastLayout<M>;
  constexpr int D2 = D * D;
  constexpr int L = M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  R *bufr = reinterpret_cast<R *>(smem_raw);
  LastArgs<float> a = a0;
  a.bind();
  if (!a.st->active) return;
  const int G = a.G, G2 = G >> 1, H = a.H;
  const int tid = threadIdx.x + blockDim.x * threadIdx.y, nth = blockDim.x * blockDim.y;
  T *tws = buf + (size_t)a.ncomp * G2 * Lay::PS;  // after the pencils
  stage_twiddles<M>(tws, a.ap.tw);
  const long long row0 = (long long)blockIdx.x * G;
  const bool first = a.st->iter == 0;
  const R beta = R(a.st->beta);
  Acc<R> pkp;
  for (int idx = tid; idx < G * L; idx += nth) {
    const int g = idx / L, e = idx % L;  // L is a power of two
    const long long row = row0 + g;
    R out[D2];
    if (row < a.nrows) {
      const long long px = row * L + e;
      R rv[D2], pv[D2], v[D2];
      TangentLocal<D, TK, R> tl;
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        const long long o = (long long)c * a.npx + px;
        rv[c] = a.r[o];
        pv[c] = first ? R(0) : a.p[o];
      }
      tl.load(a.td, px, a.npx);
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        v[c] = first ? -rv[c] : -rv[c] + beta * pv[c];
        a.p[(long long)c * a.npx + px] = v[c];
      }
      tl.apply(v, out);
      R q = R(0);  // p.(K:p) of the pixel, then one compensated add
#pragma unroll
      for (int c = 0; c < D2; ++c) q += v[c] * out[c];
      pkp.add(q);
    } else {
#pragma unroll
      for (int c = 0; c < D2; ++c) out[c] = R(0);
    }
#pragma unroll
    for (int c = 0; c < D2; ++c) bufr[2 * ((c * G2 + (g >> 1)) * Lay::PS + Lay::pos(e)) + (g & 1)] = out[c];
  }
  __syncthreads();
  const int y = threadIdx.x, q = threadIdx.y;
  T *col = buf + q * Lay::PS;
  T v[F::R1];
#pragma unroll
  for (int r = 0; r < F::R1; ++r) v[r] = col[Lay::pos(y + F::Y * r)];
  __syncthreads();
  Dft<F::R1, false, T>::run(v);
#pragma unroll
  for (int r = 0; r < F::R1; ++r) col[Lay::pos(y * F::R1 + r)] = v[r];
  __syncthreads();
#pragma unroll
  for (int b = 0; b < F::NB; ++b) {
    const int j = y + F::Y * b;
    T w[F::R2];
#pragma unroll
    for (int r = 0; r < F::R2; ++r) w[r] = col[Lay::pos(j + F::R1 * r)];
#pragma unroll
    for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], reg_tw<false>(tws, j * r));
    Dft<F::R2, false, T>::run(w);
#pragma unroll
    for (int r = 0; r < F::R2; ++r) col[Lay::pos(j + F::R1 * r)] = w[r];
  }
  __syncthreads();
  // unpack the two real spectra: X = (Z_k + conj Z_{L-k})/2, Y = -i (Z_k - conj Z_{L-k})/2
  const int c = q / G2, g2 = q - c * G2;
  const long long rx = row0 + 2 * g2, ry = rx + 1;
  T *sx = a.spec + (long long)c * a.nk + rx * H;
  for (int k = y; k < H; k += F::Y) {
    const int kn = (k == 0) ? 0 : L - k;
    const T z = col[Lay::pos(k)], zn = col[Lay::pos(kn)];
    if (rx < a.nrows) sx[k] = T{R(0.5) * (z.x + zn.x), R(0.5) * (z.y - zn.y)};
    if (ry < a.nrows) sx[H + k] = T{R(0.5) * (z.y + zn.y), R(-0.5) * (z.x - zn.x)};
  }
  warp_partial(pkp.value(), a.partial + (size_t)blockIdx.x * warps_per_block());
}

// the epilogue of the FP32 inner solve's inverse pass (EPI_CGF) for the entries o of
// rows x and y of a lane (ok: the row exists): Ap = v (stored only for operator
// checks), r += alpha Ap; returns the new r.r of the two entries
__device__ __forceinline__ float cgf_pair(const LastArgs<float> &a, long long ox, long long oy, bool okx, bool oky,
                                          float alpha, float rx, float ry, float2 v) {
  float q = 0.f;
  if (okx) {
    if (a.Ap) a.Ap[ox] = v.x;
    const float rn = rx + alpha * v.x;
    a.r[ox] = rn;
    q += rn * rn;
  }
  if (oky) {
    if (a.Ap) a.Ap[oy] = v.y;
    const float rn = ry + alpha * v.y;
    a.r[oy] = rn;
    q += rn * rn;
  }
  return q;
}

// inverse with the CG epilogue of the FP32 inner solve (EPI_CGF): c2r of the rows,
// r += alpha Ap, partial[block] = sum of the new r.r over the block's rows, and the
// last block to finish sets beta and the loop condition.  The r entries of a lane's
// outputs are loaded before the transform, after its spectrum entries, so that they
// are in flight with the transform.  FP32 only.
template <int M, int D>
__global__ void __launch_bounds__(384, 2) k_last_inv_reg(const LastArgs<float> a0) {
  dep_wait();
  using R = float;
  using T = float2;
  using F = RegFft<M>;
  using Lay = LastLayout<M>;
  constexpr int L = M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  LastArgs<float> a = a0;
  a.bind();
  if (!a.st->active) return;
  const int G = a.G, G2 = G >> 1, H = a.H;
  const int y = threadIdx.x, q = threadIdx.y;
  const int c = q / G2, g2 = q - c * G2;
  const long long row0 = (long long)blockIdx.x * G;
  const long long rx = row0 + 2 * g2, ry = rx + 1;
  const bool okx = rx < a.nrows, oky = ry < a.nrows;
  const long long ox = (long long)c * a.npx + rx * L, oy = ox + L;
  const T *sx = a.spec + (long long)c * a.nk + rx * H;
  T *col = buf + q * Lay::PS;
  T *tws = buf + (size_t)a.ncomp * G2 * Lay::PS;  // after the pencils
  stage_twiddles<M>(tws, a.ap.tw);
  // every spectrum entry of the lane first (the transform needs them), then p (the
  // epilogue needs it), so the spectrum loads are not queued behind the p loads
  T w[F::NB][F::R2];
#pragma unroll
  for (int b = 0; b < F::NB; ++b) {
    const int j = y + F::Y * b;
#pragma unroll
    for (int r = 0; r < F::R2; ++r) {
      const int k = j + F::R1 * r;
      const bool hi = k >= H;
      const int kk = hi ? L - k : k;
      T x = okx ? sx[kk] : T{R(0), R(0)};
      T z = oky ? sx[H + kk] : T{R(0), R(0)};
      if (hi) {
        x.y = -x.y;
        z.y = -z.y;
      }
      if (k == 0 || 2 * k == L) {  // c2r uses the real part of self-conjugate bins only
        x.y = R(0);
        z.y = R(0);
      }
      w[b][r] = T{x.x - z.y, x.y + z.x};
    }
  }
  R px[F::R1], py[F::R1];  // the r entries of the lane's outputs
#pragma unroll
  for (int r = 0; r < F::R1; ++r) {
    px[r] = okx ? a.r[ox + y + F::Y * r] : R(0);
    py[r] = oky ? a.r[oy + y + F::Y * r] : R(0);
  }
  __syncthreads();  // the twiddle copy
#pragma unroll
  for (int b = 0; b < F::NB; ++b) {
    const int j = y + F::Y * b;
    Dft<F::R2, true, T>::run(w[b]);
#pragma unroll
    for (int r = 1; r < F::R2; ++r) w[b][r] = cmul(w[b][r], reg_tw<true>(tws, j * r));
#pragma unroll
    for (int r = 0; r < F::R2; ++r) col[Lay::pos(j + F::R1 * r)] = w[b][r];
  }
  __syncthreads();
  T v[F::R1];
#pragma unroll
  for (int r = 0; r < F::R1; ++r) v[r] = col[Lay::pos(y * F::R1 + r)];
  Dft<F::R1, true, T>::run(v);
  Acc<R> acc;
  const R alpha = R(a.st->alpha);
#pragma unroll
  for (int r = 0; r < F::R1; ++r) {
    const int e = y + F::Y * r;
    acc.add(cgf_pair(a, ox + e, oy + e, okx, oky, alpha, px[r], py[r], v[r]));
  }
  const double bs = block_sum(acc.value());
  if (y == 0 && q == 0) a.partial[blockIdx.x] = bs;
  CGState *st = const_cast<CGState *>(a.st);
  if (cg_last_block(st)) cg_beta_step(st, a.partial, gridDim.x);
}

}  // namespace musg
