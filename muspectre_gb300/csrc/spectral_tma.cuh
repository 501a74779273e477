// Green pass (first-axis FFT, Green operator, inverse first-axis FFT) fed by the Tensor
// Memory Accelerator: a persistent FP32 kernel whose blocks walk tiles of T pencils,
// each tile brought into shared memory by one cp.async.bulk.tensor copy issued by one
// thread while the block transforms the previous tile (two buffers, one mbarrier each).
//
// The register Green kernel (k_green_reg) loads a tile into registers, transforms it
// and stores it.  Here the next tile is in flight during the whole transform of the
// current one, so no thread holds load registers or waits on HBM latency; what bounds
// the pass is then instruction issue (two FFTs per element), which the shared twiddle
// table, the shared xi_0 and the compile-time tile width below reduce.
//
// Tile layout.  The tensor map splits the pencil index e = e_lo + Y e_hi (Y = M / R1
// lanes) into two dimensions ordered (rho, row group, component, e_hi, e_lo), so the
// copy writes element (e, c, t) of the tile to shared slot s = e_lo R1 + e_hi, position
// s P + c T + t (P = NC T): lane y's first-stage inputs x[y + Y r] (r < R1) sit in its
// own slots y R1 + r, the slots the first stage writes its outputs to, so the forward
// transform starts in place without an extra barrier.  From there on the pass is the
// register kernel's: DFT_R2 stage, Green operator on natural-order frequencies, the
// adjoint inverse network, and the inverse first stage stores x[y + Y r] to global
// memory straight from registers.
//
// Per block, once: the twiddle table W_M^k and the first-axis wave numbers xi_0 are
// copied into shared memory (the persistent block reuses them for every tile), and the
// tile width TT is a compile-time constant, so every shared-memory offset of the
// transform is an immediate.
//
// Bounded waits.  A block waits for a tile's copy by polling the mbarrier with a
// wall-clock limit (kWaitLimitNs); if it runs out, the block records the fault in
// g_wait_fault, marks the CG state inactive, waits (with the same limit) for the
// other copy it has in flight, and returns.  The host reads the word (stream-ordered,
// wait_fault_word) after every CG solve, clears it and raises MUSG_ERR_RUNTIME.
#pragma once

#include <cuda.h>
#include <algorithm>
#include <cstdint>

#include "spectral_reg.cuh"

namespace musg {

// included by spectral_tma.cu only (whole-program compilation: one definition there)
static __device__ unsigned int g_wait_fault;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

// dynamic shared memory of k_green_tma: two tiles, two mbarriers + the fault flag
// (32 bytes), the twiddle table (m complex) and xi_0 (m reals)
inline size_t k_green_tma_smem(int m, int nc, int T) {
  return (size_t)2 * m * nc * T * sizeof(float2) + 32 + (size_t)m * sizeof(float2) + (size_t)m * sizeof(float);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// poll until the phase of the given parity completed or the wall-clock limit ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  unsigned long long limit_ns = kWaitLimitNs) {
  const unsigned long long t0 = global_ns();
  for (unsigned i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && global_ns() - t0 > limit_ns) return false;
  }
}

// Self-test of the bounded wait: one thread waits on an mbarrier that nothing arrives
// at, gives up after limit_ns, records the fault word like the pass kernels do, and
// the kernel exits (no copy is in flight).
__global__ void k_wait_probe(unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, limit_ns)) atomicOr(&g_wait_fault, 1u);
}
// generic-proxy accesses of shared memory before this point are ordered before the
// async-proxy (TMA) accesses issued after it
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                            int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
      : "memory");
}

// Tile t of ntiles = ntr * NG: row group g = t / ntr (finite strain: row i of F, else
// 0), rho tile t % ntr.  Thread block (TT, Y, NC) as k_green_reg with T = TT.
template <int M, int MODE, int D, int TT>
__global__ void __launch_bounds__(384, 2) k_green_tma(const GreenArgs<float> a, const __grid_constant__ CUtensorMap tm) {
  dep_wait();
  using R = float;
  using T = float2;
  using F = RegFft<M>;
  static_assert(MODE == GM_SMALL || MODE == GM_FINITE, "projection modes only");
  constexpr int NC = MODE == GM_FINITE ? D : D * D;
  constexpr int NG = MODE == GM_FINITE ? D : 1;
  constexpr int P = NC * TT;
  constexpr int tile_elems = M * P;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  if (a.st && !a.st->active) return;
  const int t = threadIdx.x, y = threadIdx.y, z = threadIdx.z;
  T *bufs = reinterpret_cast<T *>(tma_smem);
  uint64_t *bars = reinterpret_cast<uint64_t *>(tma_smem + (size_t)2 * tile_elems * sizeof(T));
  int &s_fault = *reinterpret_cast<int *>(bars + 2);
  T *tw = reinterpret_cast<T *>(bars + 4);
  R *xi0 = reinterpret_cast<R *>(tw + M);
  const int tid = lin_tid(), nth = lin_nth();
  const long long ntr = (a.Rr + TT - 1) / TT;
  const long long ntiles = ntr * NG;
  constexpr uint32_t bytes = (uint32_t)tile_elems * (uint32_t)sizeof(T);
  auto issue = [&](long long tile, int s) {
    const int g = (int)(tile / ntr);
    const int x = (int)((tile - (long long)g * ntr) * TT);
    mbar_expect_tx(&bars[s], bytes);
    tma_load_5d(bufs + (size_t)s * tile_elems, &tm, &bars[s], x, g, 0, 0, 0);
  };
  bool pending[2] = {false, false};  // thread 0: copies in flight per buffer
  if (tid == 0) {
    s_fault = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  for (int k = tid; k < M; k += nth) {
    tw[k] = a.ap.tw[k];
    xi0[k] = a.xi0[k];
  }
  __syncthreads();
  long long tile = blockIdx.x;
  if (tid == 0) {
    if (tile < ntiles) {
      issue(tile, 0);
      pending[0] = true;
    }
    if (tile + gridDim.x < ntiles) {
      issue(tile + gridDim.x, 1);
      pending[1] = true;
    }
  }
  for (int it = 0; tile < ntiles; ++it, tile += gridDim.x) {
    const int s = it & 1;
    const uint32_t parity = (uint32_t)((it >> 1) & 1);
    if (tid == 0) {
      if (mbar_wait_bounded(&bars[s], parity)) {
        pending[s] = false;
      } else {
        s_fault = 1;
      }
    }
    __syncthreads();
    if (s_fault) {
      if (tid == 0) {
        atomicOr(&g_wait_fault, 1u);
        if (a.st) const_cast<CGState *>(a.st)->active = 0;
        const uint32_t par1 = (uint32_t)(((it + 1) >> 1) & 1);
        if (pending[s ^ 1]) (void)mbar_wait_bounded(&bars[s ^ 1], par1);
      }
      return;
    }
    (void)mbar_try_wait(&bars[s], parity);  // this thread's own acquire of the completed copy
    const int g = (int)(tile / ntr);
    const long long rho = (tile - (long long)g * ntr) * TT + t;
    const bool ok = rho < a.Rr;
    const int comp = MODE == GM_FINITE ? g + D * z : z;
    T *buf = bufs + (size_t)s * tile_elems;
    T *col = buf + z * TT + t + y * F::R1 * P;  // this lane's first-stage slots
    {
      T v[F::R1];
#pragma unroll
      for (int r = 0; r < F::R1; ++r) v[r] = col[r * P];
      Dft<F::R1, false, T>::run(v);
#pragma unroll
      for (int r = 0; r < F::R1; ++r) col[r * P] = v[r];
    }
    __syncthreads();
    T *cj = buf + z * TT + t;
#pragma unroll
    for (int b = 0; b < F::NB; ++b) {
      const int j = y + F::Y * b;
      T *c2 = cj + j * P;
      T w[F::R2];
#pragma unroll
      for (int r = 0; r < F::R2; ++r) w[r] = c2[F::R1 * r * P];
#pragma unroll
      for (int r = 1; r < F::R2; ++r) w[r] = cmul(w[r], tw[j * r]);
      Dft<F::R2, false, T>::run(w);
#pragma unroll
      for (int r = 0; r < F::R2; ++r) c2[F::R1 * r * P] = w[r];
    }
    __syncthreads();
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
        xi[0] = xi0[e];
        xi[1] = x1;
        if (D == 3) xi[D - 1] = x2;
        T f[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) f[c] = tc[e * P + c * TT];
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
        for (int c = 0; c < NC; ++c) tc[e * P + c * TT] = f[c];
      }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < F::NB; ++b) {
      const int j = y + F::Y * b;
      T *c2 = cj + j * P;
      T w[F::R2];
#pragma unroll
      for (int r = 0; r < F::R2; ++r) w[r] = c2[F::R1 * r * P];
      Dft<F::R2, true, T>::run(w);
#pragma unroll
      for (int r = 1; r < F::R2; ++r) {
        const T u = tw[j * r];
        w[r] = cmul(w[r], T{u.x, -u.y});
      }
#pragma unroll
      for (int r = 0; r < F::R2; ++r) c2[F::R1 * r * P] = w[r];
    }
    __syncthreads();
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = col[r * P];
    __syncthreads();  // every thread is done with this buffer
    if (tid == 0 && tile + 2 * (long long)gridDim.x < ntiles) {
      fence_proxy_async_smem();
      issue(tile + 2 * (long long)gridDim.x, s);
      pending[s] = true;
    }
    Dft<F::R1, true, T>::run(v);
    if (ok) {
      T *base = a.spec + (long long)comp * a.nk + rho;
#pragma unroll
      for (int r = 0; r < F::R1; ++r) base[(long long)(y + F::Y * r) * a.Rr] = v[r];
    }
  }
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Last-axis inverse with the CG epilogue (the pass k_last_inv_reg computes: r += alpha Ap,
// new r.r), fed by
// bulk copies: a persistent block walks tiles of G rows; one thread stages the next
// tile's half spectra (per component the G rows are G*H contiguous complex values: one
// cp.async.bulk of G*H*8 bytes each) while the block transforms the current tile.  A
// lane reads all its spectrum entries of the tile into registers first, so after one
// barrier the tile's stage doubles as the transform's exchange buffer and a block
// needs two stages only.  The r entries are loaded from global memory at the start of
// each tile (they are needed in the epilogue).  Each block sums the new r.r over its
// tiles into one partial sum; the last block to finish sets beta.  A batched launch
// (a.batch) runs problem blockIdx.y with its own pointers, state and partial sums, in
// the same order as a single-problem launch, so batched and solo results agree bit for
// bit.  Dynamic shared memory: k_last_inv_tma_smem bytes.
inline size_t last_inv_tma_stage(int m, int nc, int G) {
  const size_t spec = (size_t)nc * G * (m / 2 + 1) * sizeof(float2);
  const size_t xchg = (size_t)nc * (G / 2) * (m + m / (m == 16 ? 4 : (m == 32 || m == 64) ? 8 : 16)) * sizeof(float2);
  return (std::max(spec, xchg) + 15) / 16 * 16;
}
inline size_t k_last_inv_tma_smem(int m, int nc, int G) {
  return 2 * last_inv_tma_stage(m, nc, G) + 32 + (size_t)m * sizeof(float2);
}

template <int M, int D, bool BATCH>
__global__ void __maxnreg__(96) k_last_inv_tma(const LastArgs<float> a0, unsigned stage_bytes) {
  dep_wait();
  // a batched launch binds problem blockIdx.y's pointers; a single problem reads its
  // arguments straight from the parameter space (no register copy, no spill at the
  // 96-register cap)
  LastArgs<float> ab;
  if constexpr (BATCH) {
    ab = a0;
    ab.bind();
  }
  const LastArgs<float> &a = BATCH ? ab : a0;
  using R = float;
  using T = float2;
  using F = RegFft<M>;
  using Lay = LastLayout<M>;
  constexpr int L = M;
  constexpr int NC = D * D;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  if (!a.st->active) return;
  const int G = a.G, G2 = G >> 1, H = a.H;
  const int y = threadIdx.x, q = threadIdx.y;
  const int c = q / G2, g2 = q - c * G2;
  const int tid = lin_tid();
  uint64_t *bars = reinterpret_cast<uint64_t *>(tma_smem + 2 * (size_t)stage_bytes);
  int &s_fault = *reinterpret_cast<int *>(bars + 2);
  T *tw = reinterpret_cast<T *>(bars + 4);  // W_M^k, k < M
  const long long ntiles = (a.nrows + G - 1) / G;
  auto issue = [&](long long tile, int s) {
    const long long row0 = tile * G;
    const long long rows = a.nrows - row0 < G ? a.nrows - row0 : G;
    const uint32_t bytes = (uint32_t)(rows * H * (long long)sizeof(T));
    unsigned char *dst = tma_smem + (size_t)s * stage_bytes;
    mbar_expect_tx(&bars[s], bytes * NC);
    for (int cc = 0; cc < NC; ++cc)
      bulk_load(dst + (size_t)cc * G * H * sizeof(T), a.spec + (long long)cc * a.nk + row0 * H, bytes, &bars[s]);
  };
  bool pending[2] = {false, false};
  if (tid == 0) {
    s_fault = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  for (int k = tid; k < M; k += lin_nth()) tw[k] = a.ap.tw[k];
  __syncthreads();
  long long tile = blockIdx.x;
  if (tid == 0) {
    if (tile < ntiles) {
      issue(tile, 0);
      pending[0] = true;
    }
    if (tile + gridDim.x < ntiles) {
      issue(tile + gridDim.x, 1);
      pending[1] = true;
    }
  }
  Acc<R> acc;
  const R alpha = R(a.st->alpha);
  for (int it = 0; tile < ntiles; ++it, tile += gridDim.x) {
    const int s = it & 1;
    const uint32_t parity = (uint32_t)((it >> 1) & 1);
    const long long row0 = tile * G;
    const long long rx = row0 + 2 * g2, ry = rx + 1;
    const bool okx = rx < a.nrows, oky = ry < a.nrows;
    const long long ox = (long long)c * a.npx + rx * L, oy = ox + L;
    R px[F::R1], py[F::R1];  // the r entries of the lane's outputs
#pragma unroll
    for (int r = 0; r < F::R1; ++r) {
      px[r] = okx ? a.r[ox + y + F::Y * r] : R(0);
      py[r] = oky ? a.r[oy + y + F::Y * r] : R(0);
    }
    if (tid == 0) {
      if (mbar_wait_bounded(&bars[s], parity)) {
        pending[s] = false;
      } else {
        s_fault = 1;
      }
    }
    __syncthreads();
    if (s_fault) {
      if (tid == 0) {
        atomicOr(&g_wait_fault, 1u);
        const_cast<CGState *>(a.st)->active = 0;
        const uint32_t par1 = (uint32_t)(((it + 1) >> 1) & 1);
        if (pending[s ^ 1]) (void)mbar_wait_bounded(&bars[s ^ 1], par1);
      }
      return;
    }
    (void)mbar_try_wait(&bars[s], parity);
    T *stage = reinterpret_cast<T *>(tma_smem + (size_t)s * stage_bytes);
    const T *sx = stage + ((size_t)c * G + 2 * g2) * H;
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
    __syncthreads();  // the stage now serves as the exchange buffer
    T *col = stage + q * Lay::PS;
#pragma unroll
    for (int b = 0; b < F::NB; ++b) {
      const int j = y + F::Y * b;
      Dft<F::R2, true, T>::run(w[b]);
#pragma unroll
      for (int r = 1; r < F::R2; ++r) {
        const T u = tw[j * r];
        w[b][r] = cmul(w[b][r], T{u.x, -u.y});
      }
#pragma unroll
      for (int r = 0; r < F::R2; ++r) col[Lay::pos(j + F::R1 * r)] = w[b][r];
    }
    __syncthreads();
    T v[F::R1];
#pragma unroll
    for (int r = 0; r < F::R1; ++r) v[r] = col[Lay::pos(y * F::R1 + r)];
    __syncthreads();  // every thread is done with this stage
    if (tid == 0 && tile + 2 * (long long)gridDim.x < ntiles) {
      fence_proxy_async_smem();
      issue(tile + 2 * (long long)gridDim.x, s);
      pending[s] = true;
    }
    Dft<F::R1, true, T>::run(v);
#pragma unroll
    for (int r = 0; r < F::R1; ++r) {
      const int e = y + F::Y * r;
      acc.add(cgf_pair(a, ox + e, oy + e, okx, oky, alpha, px[r], py[r], v[r]));
    }
  }
  const double bs = block_sum(acc.value());
  if (tid == 0) a.partial[blockIdx.x] = bs;
  CGState *st = const_cast<CGState *>(a.st);
  if (cg_last_block(st)) cg_beta_step(st, a.partial, gridDim.x);
}

}  // namespace musg
