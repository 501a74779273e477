// Conjugate-gradient vector and scalar kernels (src/solver/solver_cg.cc:54-110).
//
// The loop runs on the device: the CGState holds the FP64 scalars (r.r, alpha,
// beta, the iteration count and an `active` flag).  Every kernel of an iteration
// returns at once when `active` is 0, so a CUDA graph holding several iterations
// can be replayed past convergence without changing the result.  Dot products are
// reduced in two deterministic stages (fixed block partition, then the last block to
// finish sums the partials in a fixed order), so a rerun gives bit-identical scalars.  FP32 vectors are
// accumulated with Neumaier-compensated FP32 sums per thread and FP64 across
// threads and blocks.
#include <algorithm>
#include <cstdint>

#include "spectral.cuh"

namespace musg {

constexpr int kRedThreads = 256;
constexpr int kRedMaxBlocks = 2048;

int reduce_blocks(long long n) {
  long long b = (n + kRedThreads * 8 - 1) / (kRedThreads * 8);
  if (b < 1) b = 1;
  if (b > kRedMaxBlocks) b = kRedMaxBlocks;
  return (int)b;
}

// deterministic sum of nparts doubles by one block
__device__ __forceinline__ double sum_partials(const double *partial, int nparts) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += partial[i];
  return block_sum(v);
}

template <typename R>
__global__ void k_cg_init(const double *__restrict__ rhs, R *__restrict__ r, R *__restrict__ x, long long n,
                          double *partial, double *partial2) {
  Acc<R> acc;
  double acc2 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double b = rhs[i];
    const R rv = R(-b);
    r[i] = rv;
    x[i] = R(0);
    acc.add(rv * rv);
    acc2 += b * b;
  }
  const double s1 = block_sum(acc.value());
  if (threadIdx.x == 0) partial[blockIdx.x] = s1;
  __syncthreads();
  const double s2 = block_sum(acc2);
  if (threadIdx.x == 0) partial2[blockIdx.x] = s2;
}

__global__ void k_cg_init_scalars(CGState *st, const double *partial, const double *partial2, int nparts,
                                  double tol, int maxiter) {
  const double rdr = sum_partials(partial, nparts);
  __syncthreads();
  const double rhs2 = sum_partials(partial2, nparts);
  if (threadIdx.x == 0) {
    st->rdr = rdr;
    st->rhs_norm2 = rhs2;
    st->tol2 = tol * tol * rhs2;
    st->alpha = st->beta = st->pAp = 0.0;
    st->iter = 0;
    st->maxiter = maxiter;
    st->ticket = 0;
    // solver_cg.cc:76-77: i < maxiter && (rdr > tol2 || i == 0)
    st->active = maxiter > 0 ? 1 : 0;
  }
}

template <typename R>
void cg_init(CGState *st, const double *rhs, R *r, R *x, long long n, double tol, int maxiter, double *partial,
             double *partial2, cudaStream_t s) {
  const int nb = reduce_blocks(n);
  k_cg_init<R><<<nb, kRedThreads, 0, s>>>(rhs, r, x, n, partial, partial2);
  MUSG_CHECK_LAUNCH();
  k_cg_init_scalars<<<1, 1024, 0, s>>>(st, partial, partial2, nb, tol, maxiter);
  MUSG_CHECK_LAUNCH();
}

// x += alpha p, r += alpha Ap, partial sums of r.r.  16-byte vectors (float4 /
// double2) over one wave of blocks; the scalar tail (n not a multiple of the vector
// width) goes to block 0.  Solo and batched launches share this body, so a problem
// gives bit-identical scalars in both.
template <typename R> struct Vec16;
template <> struct Vec16<float> { using T = float4; static constexpr int W = 4; };
template <> struct Vec16<double> { using T = double2; static constexpr int W = 2; };

template <typename R>
__device__ __forceinline__ double cg_update_body(R alpha, R *__restrict__ x, R *__restrict__ r,
                                                 const R *__restrict__ p, const R *__restrict__ Ap, long long n) {
  using V = typename Vec16<R>::T;
  constexpr int W = Vec16<R>::W;
  Acc<R> acc;
  const long long nv = n / W;
  V *xv = reinterpret_cast<V *>(x);
  V *rv = reinterpret_cast<V *>(r);
  const V *pv = reinterpret_cast<const V *>(p);
  const V *av = reinterpret_cast<const V *>(Ap);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x) {
    V xi = xv[i], ri = rv[i];
    const V pi = pv[i], ai = av[i];
    R *xs = reinterpret_cast<R *>(&xi);
    R *rs = reinterpret_cast<R *>(&ri);
    const R *ps = reinterpret_cast<const R *>(&pi);
    const R *as = reinterpret_cast<const R *>(&ai);
#pragma unroll
    for (int u = 0; u < W; ++u) {
      xs[u] += alpha * ps[u];
      rs[u] = rs[u] + alpha * as[u];
      acc.add(rs[u] * rs[u]);
    }
    xv[i] = xi;
    rv[i] = ri;
  }
  if (blockIdx.x == 0) {
    for (long long i = nv * W + threadIdx.x; i < n; i += blockDim.x) {
      x[i] += alpha * p[i];
      const R v = r[i] + alpha * Ap[i];
      r[i] = v;
      acc.add(v * v);
    }
  }
  return block_sum(acc.value());
}

template <typename R>
__global__ void k_cg_update(CGState *__restrict__ st, R *__restrict__ x, R *__restrict__ r,
                            const R *__restrict__ p, const R *__restrict__ Ap, long long n, double *partial) {
  dep_wait();
  if (!st->active) return;
  const double bs = cg_update_body<R>(R(st->alpha), x, r, p, Ap, n);
  if (threadIdx.x == 0) partial[blockIdx.x] = bs;
  if (cg_last_block(st)) cg_beta_step(st, partial, gridDim.x);
}

int update_blocks(long long n) {
  static int nsm[64] = {0};
  int dev = 0;
  MUSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) dev = 0;
  if (nsm[dev] == 0) MUSG_CUDA(cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev));
  const long long need = (n / 2 + kRedThreads - 1) / kRedThreads;
  return (int)std::max<long long>(1, std::min<long long>(need, std::min(8LL * nsm[dev], (long long)kRedMaxBlocks)));
}

inline bool aligned16(const void *q) { return ((uintptr_t)q & 15u) == 0; }

template <typename R>
void cg_update(CGState *st, R *x, R *r, const R *p, const R *Ap, long long n, double *partial, cudaStream_t s) {
  if (!(aligned16(x) && aligned16(r) && aligned16(p) && aligned16(Ap)))
    throw Error(MUSG_ERR_ARGUMENT, "CG vectors must be 16-byte aligned");
  launch_pdl(k_cg_update<R>, dim3(update_blocks(n)), dim3(kRedThreads), 0, s, st, x, r, p, Ap, n, partial);
  MUSG_CHECK_LAUNCH();
}

// The part of a CG iteration of the FP32 inner solve that its spectral passes leave
// out: cg_alpha sets alpha = r.r / p.(K:p) from the forward pass's nparts partial sums
// (one block per problem, a fixed order), and cg_update_x applies x += alpha p.  Both
// run between the forward pass (which writes p and the sums) and the inverse pass
// (which may end the loop), so they are gated by the loop flag like them.
template <typename R> __device__ __forceinline__ void update_x_body(R alpha, R *x, const R *p, long long n) {
  using V = typename Vec16<R>::T;
  constexpr int W = Vec16<R>::W;
  const long long nv = n / W;
  V *xv = reinterpret_cast<V *>(x);
  const V *pv = reinterpret_cast<const V *>(p);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nv; i += (long long)gridDim.x * blockDim.x) {
    V xi = xv[i];
    const V pi = pv[i];
    R *xs = reinterpret_cast<R *>(&xi);
    const R *ps = reinterpret_cast<const R *>(&pi);
#pragma unroll
    for (int u = 0; u < W; ++u) xs[u] += alpha * ps[u];
    xv[i] = xi;
  }
  if (blockIdx.x == 0)
    for (long long i = nv * W + threadIdx.x; i < n; i += blockDim.x) x[i] += alpha * p[i];
}

// alpha = r.r / p.(K:p) of problem blockIdx.x (a table of states and partial arrays,
// or one state and array; nparts < 0: each problem's own count from the table)
__global__ void k_cg_alpha(CGState *st, const double *partial, const BatchVec<float> *tab, int nparts) {
  dep_wait();
  CGState *s = tab ? tab[blockIdx.x].st : st;
  const double *part = tab ? tab[blockIdx.x].partial : partial;
  if (nparts < 0) nparts = tab[blockIdx.x].nparts;
  if (!s->active) return;
  const double pAp = sum_partials_fresh(part, nparts);
  if (threadIdx.x == 0) {
    s->pAp = pAp;
    s->alpha = s->rdr / pAp;
  }
}

template <typename R> __global__ void k_cg_update_x(const CGState *st, R *x, const R *p, long long n) {
  dep_wait();
  if (!st->active) return;
  update_x_body<R>(R(st->alpha), x, p, n);
}

template <typename R>
void cg_update_x(const CGState *st, R *x, const R *p, long long n, const double *partial, int nparts,
                 cudaStream_t s) {
  if (!(aligned16(x) && aligned16(p))) throw Error(MUSG_ERR_ARGUMENT, "CG vectors must be 16-byte aligned");
  launch_pdl(k_cg_alpha, dim3(1), dim3(1024), 0, s, const_cast<CGState *>(st), partial,
             (const BatchVec<float> *)nullptr, nparts);
  MUSG_CHECK_LAUNCH();
  launch_pdl(k_cg_update_x<R>, dim3(update_blocks(n)), dim3(kRedThreads), 0, s, st, x, p, n);
  MUSG_CHECK_LAUNCH();
}

template <typename R> __global__ void k_cg_update_x_b(const BatchVec<R> *tab, long long n) {
  dep_wait();
  const BatchVec<R> q = tab[blockIdx.y];
  if (!q.st->active) return;
  update_x_body<R>(R(q.st->alpha), q.x, q.p, q.n);  // the problem's own length (n: the largest)
  (void)n;
}

template <typename R> void cg_update_x_batch(const BatchVec<R> *tab, long long n, int nparts, int B, cudaStream_t s) {
  launch_pdl(k_cg_alpha, dim3(B), dim3(1024), 0, s, (CGState *)nullptr, (const double *)nullptr,
             (const BatchVec<float> *)tab, nparts);
  MUSG_CHECK_LAUNCH();
  launch_pdl(k_cg_update_x_b<R>, dim3(update_blocks(n), B), dim3(kRedThreads), 0, s, tab, n);
  MUSG_CHECK_LAUNCH();
}

template void cg_update_x<float>(const CGState *, float *, const float *, long long, const double *, int,
                                 cudaStream_t);
template void cg_update_x_batch<float>(const BatchVec<float> *, long long, int, int, cudaStream_t);

// ------------------------------------------------------------------ batched
template <typename R>
__global__ void k_cg_update_b(const BatchVec<R> *tab, long long n) {
  dep_wait();
  const BatchVec<R> q = tab[blockIdx.y];
  if (!q.st->active) return;
  const double bs = cg_update_body<R>(R(q.st->alpha), q.x, q.r, q.p, q.Ap, q.n);  // n: the largest
  (void)n;
  if (threadIdx.x == 0) q.partial[blockIdx.x] = bs;
  if (cg_last_block(q.st)) cg_beta_step(q.st, q.partial, gridDim.x);
}

template <typename R> void cg_update_batch(const BatchVec<R> *tab, long long n, int B, cudaStream_t s) {
  launch_pdl(k_cg_update_b<R>, dim3(update_blocks(n), B), dim3(kRedThreads), 0, s, tab, n);
  MUSG_CHECK_LAUNCH();
}

template void cg_update_batch<double>(const BatchVec<double> *, long long, int, cudaStream_t);
template void cg_update_batch<float>(const BatchVec<float> *, long long, int, cudaStream_t);

// ------------------------------------------------------------------ dots
template <typename Ra, typename Rb>
__global__ void k_dot(const Ra *__restrict__ a, const Rb *__restrict__ b, long long n, double *partial) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  const double bs = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = bs;
}

__global__ void k_sum_to(const double *partial, int nparts, double *out) {
  const double v = sum_partials(partial, nparts);
  if (threadIdx.x == 0) *out = v;
}

template <typename Ra, typename Rb>
void dot_device(const Ra *a, const Rb *b, long long n, double *partial, double *out, cudaStream_t s) {
  const int nb = reduce_blocks(n);
  k_dot<Ra, Rb><<<nb, kRedThreads, 0, s>>>(a, b, n, partial);
  MUSG_CHECK_LAUNCH();
  k_sum_to<<<1, 1024, 0, s>>>(partial, nb, out);
  MUSG_CHECK_LAUNCH();
}

// F += x; partial sums of x.x and F.F (after the update)
template <typename R>
__global__ void k_newton_update(double *__restrict__ F, const R *__restrict__ x, long long n, double *partial,
                                int nparts) {
  double axx = 0.0, aff = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double xv = (double)x[i];
    const double f = F[i] + xv;
    F[i] = f;
    axx += xv * xv;
    aff += f * f;
  }
  const double s1 = block_sum(axx);
  if (threadIdx.x == 0) partial[blockIdx.x] = s1;
  __syncthreads();
  const double s2 = block_sum(aff);
  if (threadIdx.x == 0) partial[nparts + blockIdx.x] = s2;
}

// the input of the next residual's FP32 projection: d = rhs - (P - Pk) (the previous
// residual minus the stress change since), and the new stress kept: Pk = P
__global__ void k_residual_input(const double *__restrict__ rhs, const double *__restrict__ P,
                                 double *__restrict__ Pk, float *__restrict__ d, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = P[i];
    d[i] = (float)(rhs[i] - (v - Pk[i]));
    Pk[i] = v;
  }
}

// line-search trial F = F0 + lam x; partial sums of x.x (the full Newton increment)
// and F.F
template <typename R>
__global__ void k_newton_trial(double *__restrict__ F, const double *__restrict__ F0, const R *__restrict__ x,
                               double lam, long long n, double *partial, int nparts) {
  double axx = 0.0, aff = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double xv = (double)x[i];
    const double f = F0[i] + lam * xv;
    F[i] = f;
    axx += xv * xv;
    aff += f * f;
  }
  const double s1 = block_sum(axx);
  if (threadIdx.x == 0) partial[blockIdx.x] = s1;
  __syncthreads();
  const double s2 = block_sum(aff);
  if (threadIdx.x == 0) partial[nparts + blockIdx.x] = s2;
}

__global__ void k_sum2_to(const double *partial, int nparts, double *out) {
  const double a = sum_partials(partial, nparts);
  __syncthreads();
  const double b = sum_partials(partial + nparts, nparts);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

void residual_input(const double *rhs, const double *P, double *Pk, float *d, long long n, cudaStream_t s) {
  k_residual_input<<<reduce_blocks(n), kRedThreads, 0, s>>>(rhs, P, Pk, d, n);
  MUSG_CHECK_LAUNCH();
}

template <typename R>
void newton_update(double *F, const R *x, long long n, double *partial, double *out, cudaStream_t s) {
  const int nb = reduce_blocks(n);
  k_newton_update<R><<<nb, kRedThreads, 0, s>>>(F, x, n, partial, nb);
  MUSG_CHECK_LAUNCH();
  k_sum2_to<<<1, 1024, 0, s>>>(partial, nb, out);
  MUSG_CHECK_LAUNCH();
}

template <typename R>
void newton_trial(double *F, const double *F0, const R *x, double lam, long long n, double *partial, double *out,
                  cudaStream_t s) {
  const int nb = reduce_blocks(n);
  k_newton_trial<R><<<nb, kRedThreads, 0, s>>>(F, F0, x, lam, n, partial, nb);
  MUSG_CHECK_LAUNCH();
  k_sum2_to<<<1, 1024, 0, s>>>(partial, nb, out);
  MUSG_CHECK_LAUNCH();
}

// per-component means of a field [ncomp][npx]: deterministic block sums, then one
// block per component in a fixed order
__global__ void k_plane_sums(const double *__restrict__ f, long long npx, double *partial) {
  const double *fc = f + (long long)blockIdx.y * npx;
  double v = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npx; i += (long long)gridDim.x * blockDim.x)
    v += fc[i];
  const double bs = block_sum(v);
  if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = bs;
}

__global__ void k_plane_finish(const double *partial, int nparts, double scale, double *out) {
  const double v = sum_partials(partial + blockIdx.x * nparts, nparts);
  if (threadIdx.x == 0) out[blockIdx.x] = v * scale;
}

void plane_means(const double *f, int ncomp, long long npx, double *partial, double *out, cudaStream_t s) {
  const int nb = std::min(reduce_blocks(npx), 1024);
  k_plane_sums<<<dim3(nb, ncomp), kRedThreads, 0, s>>>(f, npx, partial);
  MUSG_CHECK_LAUNCH();
  k_plane_finish<<<ncomp, 1024, 0, s>>>(partial, nb, 1.0 / (double)npx, out);
  MUSG_CHECK_LAUNCH();
}

template <typename Rd, typename Rs>
__global__ void k_convert(Rd *__restrict__ dst, const Rs *__restrict__ src, long long n, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = Rd((double)src[i] * scale);
}

template <typename Rd, typename Rs>
void convert(Rd *dst, const Rs *src, long long n, double scale, cudaStream_t s) {
  k_convert<Rd, Rs><<<reduce_blocks(n), kRedThreads, 0, s>>>(dst, src, n, scale);
  MUSG_CHECK_LAUNCH();
}

template void cg_init<double>(CGState *, const double *, double *, double *, long long, double, int, double *,
                              double *, cudaStream_t);
template void cg_init<float>(CGState *, const double *, float *, float *, long long, double, int, double *, double *,
                             cudaStream_t);
template void cg_update<double>(CGState *, double *, double *, const double *, const double *, long long,
                                double *, cudaStream_t);
template void cg_update<float>(CGState *, float *, float *, const float *, const float *, long long, double *,
                               cudaStream_t);
template void dot_device<double, double>(const double *, const double *, long long, double *, double *, cudaStream_t);
template void dot_device<float, float>(const float *, const float *, long long, double *, double *, cudaStream_t);
template void newton_update<double>(double *, const double *, long long, double *, double *, cudaStream_t);
template void newton_update<float>(double *, const float *, long long, double *, double *, cudaStream_t);
template void newton_trial<double>(double *, const double *, const double *, double, long long, double *, double *,
                                   cudaStream_t);
template void newton_trial<float>(double *, const double *, const float *, double, long long, double *, double *,
                                  cudaStream_t);
template void convert<double, double>(double *, const double *, long long, double, cudaStream_t);
template void convert<float, double>(float *, const double *, long long, double, cudaStream_t);
template void convert<double, float>(double *, const float *, long long, double, cudaStream_t);

}  // namespace musg
