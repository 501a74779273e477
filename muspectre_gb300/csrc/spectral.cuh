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

// PRO_CG / EPI_CG: the reference's CG iteration (solver_cg.cc:76-97) split over the
// passes: the last pass writes Ap and finishes alpha = r.r / p.Ap, and cg_update then
// applies x += alpha p, r += alpha Ap and finishes beta.  PRO_CGF / EPI_CGF (the FP32
// inner solve of the mixed-precision path): p stays in the range of the projection
// G (x0 = 0, rhs = G(-P)), and G is self-adjoint and idempotent, so p.Ap =
// p.G(K:p) = p.(K:p); the forward pass forms K:p per pixel anyway and writes per-warp
// sums of p.(K:p) (no block barrier, ticket or memory fence in its many short blocks),
// cg_alpha finishes alpha in one block, and cg_update_x applies x += alpha p.  The
// inverse pass applies r += alpha Ap straight from its registers and finishes beta,
// so Ap is never stored: per iteration the field traffic drops from 19 to 16
// field-sized passes plus the tangent data.
enum Prologue : int { PRO_PLAIN = 0, PRO_TANGENT = 1, PRO_CG = 2, PRO_CGF = 3 };
enum Epilogue : int { EPI_PLAIN = 0, EPI_CG = 1, EPI_CGF = 2 };
enum GreenMode : int { GM_SMALL = 0, GM_FINITE = 1, GM_FWD = 2, GM_INV = 3 };

// independent global loads each thread keeps in flight in the staging loops
constexpr int kLoadBatch = 8;

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

// sum of v over the block (1-, 2- or 3-D, any number of threads), result valid in
// the thread of linear index 0.  A partial last warp shuffles among its existing lanes
// only (lanes past the block's end do not exist, so the mask names just the others and
// their values are never added); whole warps add in the same order as a full tree.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  const int nth = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int w = tid >> 5, l = tid & 31;
  const int nl = min(32, nth - (w << 5));
  const unsigned mask = nl == 32 ? 0xffffffffu : ((1u << nl) - 1u);
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(mask, v, o);
    if (l + o < nl) v += t;
  }
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    const int nw = (nth + 31) >> 5;
    v = (l < nw) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(mask, v, o);
      if (l + o < nl) v += t;
    }
  }
  return v;
}

// sum of v over the calling warp, written by its first lane to out[w] (w = the warp's
// index in the block); a partial last warp shuffles among its existing lanes only.
// No block barrier: for the per-warp partial sums of short-lived blocks.
__device__ __forceinline__ void warp_partial(double v, double *out) {
  const int nth = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int w = tid >> 5, l = tid & 31;
  const int nl = min(32, nth - (w << 5));
  const unsigned mask = nl == 32 ? 0xffffffffu : ((1u << nl) - 1u);
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_down_sync(mask, v, o);
    if (l + o < nl) v += t;
  }
  if (l == 0) out[w] = v;
}
__device__ __forceinline__ int warps_per_block() { return (blockDim.x * blockDim.y * blockDim.z + 31) >> 5; }

// ------------------------------------------------------------ CG scalar steps
// The kernel that produces a dot product's partial sums also finishes it: every block
// writes partial[blockIdx.x], and the block that finishes last (counted with the
// state's ticket) sums all gridDim.x partials in a fixed order and updates the state.
// Deterministic like a separate reduction kernel, without its launch.
__device__ __forceinline__ int lin_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int lin_nth() { return blockDim.x * blockDim.y * blockDim.z; }

// call by the whole block after thread 0 wrote this block's partial sum; nblk = the
// problem's blocks (gridDim.x, or a problem's share of a grouped launch)
__device__ __forceinline__ bool cg_last_block(CGState *st, int nblk) {
  __shared__ int last;
  __syncthreads();
  if (lin_tid() == 0) {
    __threadfence();
    last = atomicAdd(&st->ticket, 1) == nblk - 1;
  }
  __syncthreads();
  return last != 0;
}
__device__ __forceinline__ bool cg_last_block(CGState *st) { return cg_last_block(st, (int)gridDim.x); }

// Grouped launches: problems of different grids in one launch, the blocks of problem b
// being [blk0[b], blk0[b+1]) of a one-dimensional grid; b by binary search
__device__ __forceinline__ int group_problem(const int *blk0, int B) {
  int lo = 0, hi = B;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (blk0[mid] <= (int)blockIdx.x) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double sum_partials_fresh(const double *partial, int n) {
  // eight independent loads in flight per thread; each thread still adds its entries
  // in index order, so the sum is the same as one load at a time (tens of thousands of
  // per-warp partials took one 1024-thread block 11.5 us, serialised on L2 latency)
  const int nth = lin_nth();
  int i = lin_tid();
  double v = 0.0;
  for (; i + 7 * nth < n; i += 8 * nth) {
    double t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) t[u] = __ldcg(partial + i + u * nth);
#pragma unroll
    for (int u = 0; u < 8; ++u) v += t[u];
  }
  for (; i < n; i += nth) v += __ldcg(partial + i);
  return block_sum(v);
}

// alpha = r.r / p.Ap (solver_cg.cc:81)
__device__ __forceinline__ void cg_alpha_step(CGState *st, const double *partial, int n) {
  const double pAp = sum_partials_fresh(partial, n);
  if (lin_tid() == 0) {
    st->pAp = pAp;
    st->alpha = st->rdr / pAp;
    st->ticket = 0;
  }
}

// beta = new r.r / old r.r (solver_cg.cc:86-88) and the loop condition of the next
// iteration; a non-finite residual fails the comparison and ends the loop, as in the
// reference
__device__ __forceinline__ void cg_beta_step(CGState *st, const double *partial, int n) {
  const double nr = sum_partials_fresh(partial, n);
  if (lin_tid() == 0) {
    st->beta = nr / st->rdr;
    st->rdr = nr;
    st->iter += 1;
    st->counter += 1;
    if (!(st->iter < st->maxiter && st->rdr > st->tol2)) st->active = 0;
    st->ticket = 0;
  }
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
  // B is symmetric: the (m, r) entry repeats the (r, m) one bit for bit
  R B[D * D];
#pragma unroll
  for (int m = 0; m < D; ++m)
#pragma unroll
    for (int r = 0; r <= m; ++r) {
      const R b = mu * (A[r + D * m] + A[m + D * r]) + (r == m ? lam * tr : R(0));
      B[r + D * m] = b;
      B[m + D * r] = b;
    }
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

// per-material stiffness C (T4 layout (i + D j) + D^2 (k + D l)), MaterialLinearElasticGeneric
// (material_linear_elastic_generic.hh): small strain dP = C:de; finite strain
// dP = dF S + F (C:(F^T dF)) (the PK2/Green-Lagrange law linearised,
// materials_toolbox.hh:313-350 contracted with dF)
template <int D, typename R>
__device__ __forceinline__ void tangent_generic_small(const R *e, const R *__restrict__ C, R *out) {
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    R v = R(0);
#pragma unroll
    for (int q = 0; q < D * D; ++q) v += __ldg(&C[c + D * D * q]) * e[q];
    out[c] = v;
  }
}
template <int D, typename R>
__device__ __forceinline__ void tangent_generic_finite(const R *dF, const R *F, const R *S, const R *__restrict__ C,
                                                       R *out) {
  R A[D * D];
#pragma unroll
  for (int n = 0; n < D; ++n)
#pragma unroll
    for (int s = 0; s < D; ++s) {
      R a = R(0);
#pragma unroll
      for (int j = 0; j < D; ++j) a += F[j + D * s] * dF[j + D * n];
      A[s + D * n] = a;  // (F^T dF)(s, n)
    }
  R B[D * D];
  tangent_generic_small<D, R>(A, C, B);
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

// Tangent data of one pixel, loaded into registers before anything is stored so that
// all of a pixel's global loads are in flight together.
template <int D, int TK, typename R> struct TangentLocal {
  static constexpr int D2 = D * D;
  static constexpr bool kFinite = (TK == TK_FINITE || TK == TK_MIXED || TK == TK_FISO || TK == TK_GFINITE);
  static constexpr bool kGeneric = (TK == TK_GSMALL || TK == TK_GFINITE);
  static constexpr bool kKprime = (TK == TK_KPRIME || TK == TK_MIXED);
  int kind;
  R lam, mu;
  R F[kFinite ? D2 : 1], S[kFinite ? D2 : 1];
  R Kp[kKprime ? D2 * D : 1];
  const R *Cm = nullptr;
  const R *Kt = nullptr;  // TK_FULL: this pixel's first tangent entry (planes npx apart)
  long long kstride = 0;

  __device__ __forceinline__ void load(const TangentData<R> &td, long long px, long long npx) {
    kind = TK;
    if constexpr (TK == TK_FULL) {
      // the D^4 entries are read while they are applied (apply), not held in registers
      Kt = td.Kt + px;
      kstride = npx;
      return;
    }
    if constexpr (TK == TK_MIXED) kind = td.law_kind[td.mat[px]];
    if constexpr (kGeneric) Cm = td.C + (size_t)td.mat[px] * (D2 * D2);
    if constexpr (TK == TK_SMALL || (kFinite && !kGeneric)) {
      lam = td.lam[px];
      mu = td.mu[px];
    }
    if constexpr (kFinite) {
      if (TK == TK_FINITE || TK == TK_FISO || TK == TK_GFINITE || kind == TK_FINITE) {
#pragma unroll
        for (int c = 0; c < D2; ++c) F[c] = td.F[c * npx + px];
        if constexpr (TK != TK_FISO) {
#pragma unroll
          for (int c = 0; c < D2; ++c) S[c] = td.S[c * npx + px];
        }
      }
    }
    if constexpr (kKprime) {
      if (TK == TK_KPRIME || kind == TK_KPRIME) {
#pragma unroll
        for (int c = 0; c < D2 * D; ++c) Kp[c] = td.Kp[c * npx + px];
      }
    }
  }

  // the FP32 copy of F holds H = F - I (exact where F is near I); form F, and for
  // TK_FISO the PK2 stress S = lam tr(E) I + 2 mu E with E = (H + H^T + H^T H)/2
  // (materials_toolbox.hh:139-148, 661-663)
  __device__ __forceinline__ void finish() {
    if constexpr (kFinite && sizeof(R) == 4) {
      if constexpr (TK == TK_FISO) {
        // E and S are symmetric: each (j, i) entry repeats the (i, j) one bit for bit
        R E[D2];
        R tr = R(0);
#pragma unroll
        for (int j = 0; j < D; ++j)
#pragma unroll
          for (int i = 0; i <= j; ++i) {
            R hh = R(0);
#pragma unroll
            for (int k = 0; k < D; ++k) hh += F[k + D * i] * F[k + D * j];
            const R e = R(0.5) * (F[i + D * j] + F[j + D * i] + hh);
            E[i + D * j] = e;
            E[j + D * i] = e;
          }
#pragma unroll
        for (int i = 0; i < D; ++i) tr += E[i + D * i];
#pragma unroll
        for (int j = 0; j < D; ++j)
#pragma unroll
          for (int i = 0; i <= j; ++i) {
            const R sv = R(2) * mu * E[i + D * j] + (i == j ? lam * tr : R(0));
            S[i + D * j] = sv;
            S[j + D * i] = sv;
          }
      }
      if (TK != TK_MIXED || kind == TK_FINITE) {
#pragma unroll
        for (int i = 0; i < D; ++i) F[i + D * i] += R(1);
      }
    }
  }

  __device__ __forceinline__ void apply(const R *in, R *out) {
    finish();
    if constexpr (TK == TK_SMALL) {
      tangent_small<D, R>(in, lam, mu, out);
    } else if constexpr (TK == TK_FINITE || TK == TK_FISO) {
      tangent_finite<D, R>(in, F, S, lam, mu, out);
    } else if constexpr (TK == TK_GSMALL) {
      tangent_generic_small<D, R>(in, Cm, out);
    } else if constexpr (TK == TK_GFINITE) {
      tangent_generic_finite<D, R>(in, F, S, Cm, out);
    } else if constexpr (TK == TK_KPRIME) {
      tangent_kprime<D, R>(in, Kp, out);
    } else if constexpr (TK == TK_FULL) {
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        R v = R(0);
#pragma unroll
        for (int q = 0; q < D2; ++q) v += Kt[(long long)(c + D2 * q) * kstride] * in[q];
        out[c] = v;
      }
    } else {
      if (kind == TK_FINITE) tangent_finite<D, R>(in, F, S, lam, mu, out);
      else tangent_kprime<D, R>(in, Kp, out);
    }
  }
};

// ------------------------------------------------------------ pass "last"
// Per-problem pointers of a batched launch: problem b = blockIdx.y of a grid that
// covers a batch of same-shape RVEs (or right-hand sides) in one launch per stage.
template <typename R> struct ProblemPtrs {
  typename V2<R>::T *spec;
  const CGState *st;
  R *r;
  R *x;
  R *p;
  R *Ap;
  double *partial;
  TangentData<R> td;
};

template <typename R> struct LastArgs {
  AxisPlanD<R> ap;
  int L, H, G, ncomp;
  long long nrows, npx, nk;
  typename V2<R>::T *spec;
  const R *in;
  R *out;
  R scale;
  const CGState *st;
  R *r;
  R *x;   // the CG iterate (not read by the pass kernels; kept with the problem's pointers)
  R *p;
  R *Ap;  // EPI_CGF: stored only when set (operator checks)
  double *partial;
  TangentData<R> td;
  const ProblemPtrs<R> *batch;  // null: a single problem
  __device__ __forceinline__ void bind() {
    if (!batch) return;
    const ProblemPtrs<R> &q = batch[blockIdx.y];
    spec = q.spec;
    st = q.st;
    r = q.r;
    x = q.x;
    p = q.p;
    Ap = q.Ap;
    partial = q.partial;
    td = q.td;
  }
};

// forward: real rows -> half spectra.  D is the tensor dimension for the tangent
// prologues (0 for PRO_PLAIN).  bid: this block among the problem's blocks.
template <typename R, int PRO, int D, int TK>
__device__ __forceinline__ void last_fwd_body(const LastArgs<R> &a, long long bid) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  constexpr bool kCG = PRO == PRO_CG || PRO == PRO_CGF;
  if (kCG && !a.st->active) return;
  const int L = a.L, G = a.G, nc = a.ncomp, G2 = G >> 1;
  Acc<R> pkp;  // PRO_CGF: partial sum of p.(K:p)
  const int P = nc * G2;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long row0 = bid * G;
  R *bufr = reinterpret_cast<R *>(buf);
  const FDiv fGL(G * L), fL(L);
  if constexpr (PRO == PRO_PLAIN) {
    const int total = nc * G * L;
    for (int i0 = threadIdx.x; i0 < total; i0 += kLoadBatch * blockDim.x) {
      R v[kLoadBatch];
      int dst[kLoadBatch];
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int idx = i0 + u * blockDim.x;
        dst[u] = -1;
        v[u] = R(0);
        if (idx < total) {
          int rem, e;
          const int c = fGL.div(idx, rem);
          const int g = fL.div(rem, e);
          const long long row = row0 + g;
          if (row < a.nrows) v[u] = a.in[(long long)c * a.npx + row * L + e];
          dst[u] = 2 * (e * P + c * G2 + (g >> 1)) + (g & 1);
        }
      }
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u)
        if (dst[u] >= 0) bufr[dst[u]] = v[u] * a.scale;
    }
  } else {
    constexpr int D2 = D * D;
    const bool first = kCG ? (a.st->iter == 0) : false;
    const R beta = kCG ? R(a.st->beta) : R(0);
    for (int idx = threadIdx.x; idx < G * L; idx += blockDim.x) {
      int e;
      const int g = fL.div(idx, e);
      const long long row = row0 + g;
      R out[D2];
      if (row < a.nrows) {
        const long long px = row * L + e;
        R v[D2];
        TangentLocal<D, TK, R> tl;
        if (kCG) {
          R rv[D2], pv[D2];
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
        } else {
#pragma unroll
          for (int c = 0; c < D2; ++c) v[c] = a.in[(long long)c * a.npx + px];
          tl.load(a.td, px, a.npx);
        }
        tl.apply(v, out);
        if (PRO == PRO_CGF) {
          R q = R(0);  // p.(K:p) of the pixel, then one compensated add
#pragma unroll
          for (int c = 0; c < D2; ++c) q += v[c] * out[c];
          pkp.add(q);
        }
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
  const FDiv fGH(G * H), fH(H);
  for (int idx = threadIdx.x; idx < nc * G * H; idx += blockDim.x) {
    int rem, k;
    const int c = fGH.div(idx, rem);
    const int gr = fH.div(rem, k);
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
  if constexpr (PRO == PRO_CGF) warp_partial(pkp.value(), a.partial + (size_t)bid * warps_per_block());
}

template <typename R, int PRO, int D, int TK>
__global__ void __launch_bounds__(kPassThreads) k_last_fwd(const LastArgs<R> a0) {
  dep_wait();
  LastArgs<R> a = a0;
  a.bind();
  last_fwd_body<R, PRO, D, TK>(a, blockIdx.x);
}

template <typename R, int PRO, int D, int TK>
__global__ void __launch_bounds__(kPassThreads) k_last_fwd_g(const LastArgs<R> *tab, const int *blk0, int B) {
  dep_wait();
  const int b = group_problem(blk0, B);
  const LastArgs<R> a = tab[b];
  last_fwd_body<R, PRO, D, TK>(a, blockIdx.x - blk0[b]);
}

// inverse: half spectra -> real rows.  PLAIN writes out = scale*x; CG writes Ap
// and the block sums of p.Ap.
template <typename R, int EPI, int D>
__device__ __forceinline__ void last_inv_body(const LastArgs<R> &a, long long bid, int nblk) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (EPI != EPI_PLAIN && !a.st->active) return;
  const int L = a.L, G = a.G, nc = a.ncomp, G2 = G >> 1, H = a.H;
  const int P = nc * G2;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long row0 = bid * G;
  const bool even = (L & 1) == 0;
  const int total = nc * G2 * H;
  const FDiv fG2H(G2 * H), fH(H), fGL(G * L), fL(L);
  for (int i0 = threadIdx.x; i0 < total; i0 += kLoadBatch * blockDim.x) {
    T X[kLoadBatch], Y[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = i0 + u * blockDim.x;
      X[u] = T{R(0), R(0)};
      Y[u] = T{R(0), R(0)};
      if (idx < total) {
        int rem, k;
        const int c = fG2H.div(idx, rem);
        const int g2 = fH.div(rem, k);
        const long long rx = row0 + 2 * g2, ry = rx + 1;
        if (rx < a.nrows) X[u] = a.spec[(long long)c * a.nk + rx * H + k];
        if (ry < a.nrows) Y[u] = a.spec[(long long)c * a.nk + ry * H + k];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = i0 + u * blockDim.x;
      if (idx >= total) continue;
      int rem, k;
      const int c = fG2H.div(idx, rem);
      const int g2 = fH.div(rem, k);
      T x = X[u], y = Y[u];
      const bool selfconj = (k == 0) || (even && 2 * k == L);
      if (selfconj) { x.y = R(0); y.y = R(0); }  // c2r uses the real part only
      const int q = c * G2 + g2;
      buf[k * P + q] = T{x.x - y.y, x.y + y.x};
      if (!selfconj) buf[(L - k) * P + q] = T{x.x + y.y, y.x - x.y};
    }
  }
  __syncthreads();
  const R *bufr = reinterpret_cast<const R *>(fft_run<R, true>(buf, buf2, P, a.ap));
  if constexpr (EPI == EPI_PLAIN) {
    for (int idx = threadIdx.x; idx < nc * G * L; idx += blockDim.x) {
      int rem, e;
      const int c = fGL.div(idx, rem);
      const int g = fL.div(rem, e);
      const long long row = row0 + g;
      if (row < a.nrows) a.out[(long long)c * a.npx + row * L + e] = a.scale * bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)];
    }
  } else {
    constexpr int D2 = D * D;
    Acc<R> acc;
    const R alpha = EPI == EPI_CGF ? R(a.st->alpha) : R(0);
    for (int idx = threadIdx.x; idx < G * L; idx += blockDim.x) {
      int e;
      const int g = fL.div(idx, e);
      const long long row = row0 + g;
      if (row >= a.nrows) continue;
      const long long px = row * L + e;
      R q = R(0);
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        const R v = bufr[2 * (e * P + c * G2 + (g >> 1)) + (g & 1)];
        const long long o = (long long)c * a.npx + px;
        if constexpr (EPI == EPI_CG) {
          a.Ap[o] = v;
          acc.add(a.p[o] * v);
        } else {
          if (a.Ap) a.Ap[o] = v;
          const R rn = a.r[o] + alpha * v;
          a.r[o] = rn;
          q += rn * rn;
        }
      }
      if constexpr (EPI == EPI_CGF) acc.add(q);
    }
    const double bs = block_sum(acc.value());
    if (threadIdx.x == 0) a.partial[bid] = bs;
    CGState *st = const_cast<CGState *>(a.st);
    if (cg_last_block(st, nblk)) {
      if constexpr (EPI == EPI_CG) cg_alpha_step(st, a.partial, nblk);
      else cg_beta_step(st, a.partial, nblk);
    }
  }
}

template <typename R, int EPI, int D>
__global__ void __launch_bounds__(kPassThreads) k_last_inv(const LastArgs<R> a0) {
  dep_wait();
  LastArgs<R> a = a0;
  a.bind();
  last_inv_body<R, EPI, D>(a, blockIdx.x, (int)gridDim.x);
}

template <typename R, int EPI, int D>
__global__ void __launch_bounds__(kPassThreads) k_last_inv_g(const LastArgs<R> *tab, const int *blk0, int B) {
  dep_wait();
  const int b = group_problem(blk0, B);
  const LastArgs<R> a = tab[b];
  last_inv_body<R, EPI, D>(a, blockIdx.x - blk0[b], blk0[b + 1] - blk0[b]);
}

// ------------------------------------------------------------ pass "axis"
template <typename R> struct AxisArgs {
  AxisPlanD<R> ap;
  int nax, T, ntiles;
  long long se, inner, sb;
  typename V2<R>::T *spec;
  const CGState *st;
  const ProblemPtrs<R> *batch;
};

template <typename R, bool INV>
__device__ __forceinline__ void axis_body(const AxisArgs<R> &a, long long bid) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (a.st && !a.st->active) return;
  const int tile = (int)(bid % a.ntiles);
  const long long batch = bid / a.ntiles;
  const int Tt = a.T;
  T *buf2 = buf + (size_t)Tt * a.ap.m;
  T *base = a.spec + batch * a.sb;
  const long long pos0 = (long long)tile * Tt;
  const int total = a.nax * Tt;
  const FDiv fT(Tt);
  for (int i0 = threadIdx.x; i0 < total; i0 += kLoadBatch * blockDim.x) {
    T v[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = i0 + u * blockDim.x;
      v[u] = T{R(0), R(0)};
      if (idx < total) {
        int t;
        const int e = fT.div(idx, t);
        const long long pos = pos0 + t;
        if (pos < a.inner) v[u] = base[e * a.se + pos];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = i0 + u * blockDim.x;
      if (idx < total) buf[idx] = v[u];
    }
  }
  __syncthreads();
  const T *res = fft_run<R, INV>(buf, buf2, Tt, a.ap);
  for (int idx = threadIdx.x; idx < a.nax * Tt; idx += blockDim.x) {
    int t;
    const int e = fT.div(idx, t);
    const long long pos = pos0 + t;
    if (pos < a.inner) base[e * a.se + pos] = res[idx];
  }
}

template <typename R, bool INV>
__global__ void __launch_bounds__(kPassThreads) k_axis(const AxisArgs<R> a0) {
  dep_wait();
  AxisArgs<R> a = a0;
  if (a0.batch) {
    a.spec = a0.batch[blockIdx.y].spec;
    a.st = a0.batch[blockIdx.y].st;
  }
  axis_body<R, INV>(a, blockIdx.x);
}

template <typename R, bool INV>
__global__ void __launch_bounds__(kPassThreads) k_axis_g(const AxisArgs<R> *tab, const int *blk0, int B) {
  dep_wait();
  const int b = group_problem(blk0, B);
  const AxisArgs<R> a = tab[b];
  axis_body<R, INV>(a, blockIdx.x - blk0[b]);
}

// ------------------------------------------------------------ Green operators
// 1 / sqrt(n2): FP64 correctly rounded division of the square root (parity path);
// FP32 the rsqrtf intrinsic (2 ulp, far inside the FP32 operator's rounding)
__device__ __forceinline__ double inv_sqrt(double n2) { return 1.0 / sqrt(n2); }
__device__ __forceinline__ float inv_sqrt(float n2) { return rsqrtf(n2); }

// unit wave vector of k-point (xi0[e], xi1[k1], xi2[k2]); false where the operator
// is zero (the zero mode, and every Nyquist index under the even-grid extension)
template <int D, typename R>
__device__ __forceinline__ bool unit_xi(R *xi, int e, int k1, int k2, int nyq0, int nyq1, int nyq2) {
  if ((e == 0 && k1 == 0 && k2 == 0) || e == nyq0 || k1 == nyq1 || (D == 3 && k2 == nyq2)) return false;
  R n2 = R(0);
#pragma unroll
  for (int d = 0; d < D; ++d) n2 += xi[d] * xi[d];
  const R inv = inv_sqrt(n2);
#pragma unroll
  for (int d = 0; d < D; ++d) xi[d] *= inv;
  return true;
}

// finite strain, one row i of f: f_i. <- (f_i. xi) xi^T / N
// (projection_finite_strain_fast.cc:79-85)
template <int D, typename T, typename R>
__device__ __forceinline__ void green_finite_row(T *row, const R *xi, R norm) {
  T fx = T{R(0), R(0)};
#pragma unroll
  for (int j = 0; j < D; ++j) {
    fx.x += row[j].x * xi[j];
    fx.y += row[j].y * xi[j];
  }
#pragma unroll
  for (int j = 0; j < D; ++j) row[j] = T{fx.x * xi[j] * norm, fx.y * xi[j] * norm};
}

// small strain: Ghat f = 1/2 (xi a^T + a xi^T) - xi xi^T (xi^T f xi) with a = (f + f^T) xi,
// the contraction of the operator of projection_small_strain.cc:64-77 with f, / N
template <int D, typename T, typename R>
__device__ __forceinline__ void green_small(const T *f, T *o, const R *xi, R norm) {
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
      o[i + D * j] = T{(R(0.5) * (xi[i] * av[j].x + av[i].x * xi[j]) - xx * s.x) * norm,
                       (R(0.5) * (xi[i] * av[j].y + av[i].y * xi[j]) - xx * s.y) * norm};
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
  const ProblemPtrs<R> *batch;
};

template <typename R, int MODE, int D>
__device__ __forceinline__ void green_body(const GreenArgs<R> &a, long long bid) {
  using T = typename V2<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf = reinterpret_cast<T *>(smem_raw);
  if (a.st && !a.st->active) return;
  const int Tt = a.T, nc = a.ncomp, n0 = a.n0;
  const int P = nc * Tt;
  T *buf2 = buf + (size_t)P * a.ap.m;
  const long long rho0 = bid * Tt;
  const int total = nc * n0 * Tt;
  const FDiv fT(Tt), fn0(n0);
  for (int i0 = threadIdx.x; i0 < total; i0 += kLoadBatch * blockDim.x) {
    T v[kLoadBatch];
    int dst[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int idx = i0 + u * blockDim.x;
      v[u] = T{R(0), R(0)};
      dst[u] = -1;
      if (idx < total) {
        int t, e;
        const int rest = fT.div(idx, t);
        const int c = fn0.div(rest, e);
        const long long rho = rho0 + t;
        if (rho < a.Rr) v[u] = a.spec[(long long)c * a.nk + e * a.Rr + rho];
        dst[u] = e * P + c * Tt + t;
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u)
      if (dst[u] >= 0) buf[dst[u]] = v[u];
  }
  __syncthreads();
  T *cur = buf;
  if (MODE != GM_INV) cur = fft_run<R, false>(buf, buf2, P, a.ap);
  if constexpr (MODE == GM_SMALL || MODE == GM_FINITE) {
    constexpr int D2 = D * D;
    const FDiv fnh(a.nh);
    for (int idx = threadIdx.x; idx < n0 * Tt; idx += blockDim.x) {
      int t;
      const int e = fT.div(idx, t);
      const long long rho = rho0 + t;
      if (rho >= a.Rr) continue;
      int k1, k2 = 0;
      if (D == 3) {
        k1 = fnh.div((int)rho, k2);
      } else {
        k1 = (int)rho;
      }
      R xi[D];
      xi[0] = a.xi0[e];
      xi[1] = a.xi1[k1];
      if (D == 3) xi[D - 1] = a.xi2[k2];
      T f[D2];
#pragma unroll
      for (int c = 0; c < D2; ++c) f[c] = cur[e * P + c * Tt + t];
      T o[D2];
      if (!unit_xi<D>(xi, e, k1, k2, a.nyq0, a.nyq1, a.nyq2)) {
#pragma unroll
        for (int c = 0; c < D2; ++c) o[c] = T{R(0), R(0)};
      } else {
        if (MODE == GM_FINITE) {
#pragma unroll
          for (int i = 0; i < D; ++i) {
            T row[D];
#pragma unroll
            for (int j = 0; j < D; ++j) row[j] = f[i + D * j];
            green_finite_row<D>(row, xi, a.norm);
#pragma unroll
            for (int j = 0; j < D; ++j) o[i + D * j] = row[j];
          }
        } else {
          green_small<D>(f, o, xi, a.norm);
        }
      }
#pragma unroll
      for (int c = 0; c < D2; ++c) cur[e * P + c * Tt + t] = o[c];
    }
    __syncthreads();
  }
  if (MODE != GM_FWD) cur = fft_run<R, true>(cur, cur == buf ? buf2 : buf, P, a.ap);
  for (int idx = threadIdx.x; idx < nc * n0 * Tt; idx += blockDim.x) {
    int t, e;
    const int rest = fT.div(idx, t);
    const int c = fn0.div(rest, e);
    const long long rho = rho0 + t;
    if (rho < a.Rr) a.spec[(long long)c * a.nk + e * a.Rr + rho] = cur[e * P + c * Tt + t];
  }
}

template <typename R, int MODE, int D>
__global__ void __launch_bounds__(kPassThreads) k_green(const GreenArgs<R> a0) {
  dep_wait();
  GreenArgs<R> a = a0;
  if (a0.batch) {
    a.spec = a0.batch[blockIdx.y].spec;
    a.st = a0.batch[blockIdx.y].st;
  }
  green_body<R, MODE, D>(a, blockIdx.x);
}

template <typename R, int MODE, int D>
__global__ void __launch_bounds__(kPassThreads) k_green_g(const GreenArgs<R> *tab, const int *blk0, int B) {
  dep_wait();
  const int b = group_problem(blk0, B);
  const GreenArgs<R> a = tab[b];
  green_body<R, MODE, D>(a, blockIdx.x - blk0[b]);
}

}  // namespace musg
