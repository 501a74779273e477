// Host launchers of the spectral passes, instantiated once per precision by
// spectral_f64.cu and spectral_f32.cu.
#pragma once

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <set>
#include <vector>

#include "spectral.cuh"
#include "spectral_reg.cuh"

namespace musg {

// The FP32 Green pass through the TMA-fed persistent kernel (spectral_tma.cu) for a
// tile of Tt pencils; false (nothing launched) when the spectrum, the tile or the
// driver does not qualify, and the caller launches the register kernel instead.
bool launch_green_tma(Spectral &sp, int mode, const GreenArgs<float> &a, int Tt, cudaStream_t s);
// The FP32 last-axis inverse with the CG epilogue through the bulk-copy-fed
// persistent kernel (spectral_tma.cu) for tiles of G rows; returns its number of
// blocks (= partial sums), or 0 (nothing launched) when the shape does not qualify.
int launch_last_inv_tma(Spectral &sp, const LastArgs<float> &a, int G, cudaStream_t s, int B = 1);

namespace {

int optin_smem() {
  static int v = 0;
  if (v == 0) {
    int dev = 0;
    MUSG_CUDA(cudaGetDevice(&dev));
    int b = 0;
    MUSG_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    v = b - 2048;  // room for the static shared memory of the reductions
  }
  return v;
}

// raise the dynamic shared-memory limit of a kernel once (keyed by its address)
template <typename K> void allow_smem(K kernel) {
  static std::mutex mu;
  static std::set<const void *> done;
  const void *key = (const void *)kernel;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(key)) return;
  MUSG_CUDA(cudaFuncSetAttribute(key, cudaFuncAttributeMaxDynamicSharedMemorySize, optin_smem()));
  done.insert(key);
}

struct Cfg {
  int per;       // rows per block (last pass) or tile (axis / green passes)
  int blocks;
  size_t smem;
  int threads;
};

template <typename R> constexpr int prec_index() { return sizeof(R) == 8 ? 0 : 1; }

// shared memory per block: two ping-pong buffers of (pencils x m) complex values
template <typename R> Cfg last_cfg(const Spectral &sp) {
  const AxisPlan &ap = sp.ax[sp.g.dim - 1];
  const long per_pair = (long)sp.ncomp * ap.m;
  const long eb = 2 * sizeof(typename V2<R>::T);
  const long target = sp.tune_bytes[prec_index<R>()][0];
  long g2 = std::min(std::max(1L, target / (per_pair * eb)), (long)optin_smem() / (per_pair * eb));
  if (g2 < 1) throw Error(MUSG_ERR_ARGUMENT, "last-axis FFT too long for one thread block");
  g2 = std::min<long>(g2, 16);
  g2 = std::min<long>(g2, (sp.g.nrows + 1) / 2);
  Cfg c;
  c.per = (int)(2 * g2);
  c.blocks = (int)((sp.g.nrows + c.per - 1) / c.per);
  c.smem = (size_t)(g2 * per_pair * eb);
  c.threads = sp.tune_threads[prec_index<R>()][0];
  return c;
}

template <typename R> Cfg axis_cfg(const Spectral &sp, int axis, long long inner, long long nbatch) {
  const AxisPlan &ap = sp.ax[axis];
  const long eb = 2 * sizeof(typename V2<R>::T);
  const long target = sp.tune_bytes[prec_index<R>()][1];
  long T = std::min(std::max(1L, target / (ap.m * eb)), (long)optin_smem() / (ap.m * eb));
  if (T < 1) throw Error(MUSG_ERR_ARGUMENT, "FFT axis too long for one thread block");
  T = std::min<long>(T, 32);
  T = std::min<long>(T, inner);
  // balance the tiles over the inner extent (65 -> 22 + 22 + 21, not 32 + 32 + 1)
  const long nt = (inner + T - 1) / T;
  T = (inner + nt - 1) / nt;
  Cfg c;
  c.per = (int)T;
  const long long ntiles = (inner + T - 1) / T;
  c.blocks = (int)(ntiles * nbatch);
  c.smem = (size_t)(T * ap.m * eb);
  c.threads = sp.tune_threads[prec_index<R>()][1];
  return c;
}

template <typename R> Cfg green_cfg(const Spectral &sp, long long Rr) {
  const AxisPlan &ap = sp.ax[0];
  const long per = (long)sp.ncomp * ap.m;
  const long eb = 2 * sizeof(typename V2<R>::T);
  const long target = sp.tune_bytes[prec_index<R>()][2];
  long T = std::min(std::max(1L, target / (per * eb)), (long)optin_smem() / (per * eb));
  if (T < 1) throw Error(MUSG_ERR_ARGUMENT, "first-axis FFT too long for one thread block");
  T = std::min<long>(T, 32);
  T = std::min<long>(T, Rr);
  Cfg c;
  c.per = (int)T;
  c.blocks = (int)((Rr + T - 1) / T);
  c.smem = (size_t)(T * per * eb);
  c.threads = sp.tune_threads[prec_index<R>()][2];
  return c;
}

template <typename R> typename V2<R>::T *spec_of(Spectral &sp);
template <> inline double2 *spec_of<double>(Spectral &sp) { return (double2 *)sp.spec64; }
template <> inline float2 *spec_of<float>(Spectral &sp) {
  sp.ensure32();
  return (float2 *)sp.spec32;
}
template <typename R> const R *xi_of(const Spectral &sp, int d);
template <> inline const double *xi_of<double>(const Spectral &sp, int d) { return (const double *)sp.xi64[d]; }
template <> inline const float *xi_of<float>(const Spectral &sp, int d) { return (const float *)sp.xi32[d]; }

template <typename R> LastArgs<R> last_args(Spectral &sp, const Cfg &c) {
  LastArgs<R> a{};
  a.ap = sp.ax[sp.g.dim - 1].device<R>();
  a.L = sp.g.nlast();
  a.H = sp.g.nh;
  a.G = c.per;
  a.ncomp = sp.ncomp;
  a.nrows = sp.g.nrows;
  a.npx = sp.g.npx;
  a.nk = sp.g.nk;
  a.spec = spec_of<R>(sp);
  return a;
}

template <typename R, int PRO, int D, int TK>
void launch_fwd(const LastArgs<R> &a, const Cfg &c, cudaStream_t s, int B = 1) {
  auto k = k_last_fwd<R, PRO, D, TK>;
  allow_smem(k);
  launch_pdl(k, dim3(c.blocks, B), dim3(c.threads), c.smem, s, a);
  MUSG_CHECK_LAUNCH();
}

template <typename R, int PRO>
void dispatch_fwd(int dim, int tk, const LastArgs<R> &a, const Cfg &c, cudaStream_t s, int B = 1) {
  if (PRO == PRO_PLAIN) {
    launch_fwd<R, PRO_PLAIN, 0, TK_PLAIN>(a, c, s, B);
    return;
  }
#define MUSG_FWD_CASE(DD, TT) \
  if (dim == DD && tk == TT) { launch_fwd<R, PRO, DD, TT>(a, c, s, B); return; }
  MUSG_FWD_CASE(2, TK_SMALL) MUSG_FWD_CASE(2, TK_FINITE) MUSG_FWD_CASE(2, TK_KPRIME) MUSG_FWD_CASE(2, TK_MIXED)
  MUSG_FWD_CASE(3, TK_SMALL) MUSG_FWD_CASE(3, TK_FINITE) MUSG_FWD_CASE(3, TK_KPRIME) MUSG_FWD_CASE(3, TK_MIXED)
  MUSG_FWD_CASE(2, TK_GSMALL) MUSG_FWD_CASE(2, TK_GFINITE) MUSG_FWD_CASE(3, TK_GSMALL) MUSG_FWD_CASE(3, TK_GFINITE)
  MUSG_FWD_CASE(2, TK_FULL) MUSG_FWD_CASE(3, TK_FULL)
  if (sizeof(R) == 4) {
    MUSG_FWD_CASE(2, TK_FISO) MUSG_FWD_CASE(3, TK_FISO)
  }
#undef MUSG_FWD_CASE
  throw Error(MUSG_ERR_ARGUMENT, "unsupported tangent kind");
}

template <typename R, int EPI, int D>
void launch_inv(const LastArgs<R> &a, const Cfg &c, cudaStream_t s, int B = 1) {
  auto k = k_last_inv<R, EPI, D>;
  allow_smem(k);
  launch_pdl(k, dim3(c.blocks, B), dim3(c.threads), c.smem, s, a);
  MUSG_CHECK_LAUNCH();
}

// register-resident passes (spectral_reg.cuh): lanes per pencil of a length
int reg_lanes(int m) { return m == 16 || m == 32 ? 4 : m == 256 ? 16 : 8; }
int RegLanesR1(int m) { return m == 16 ? 4 : (m == 32 || m == 64) ? 8 : 16; }
bool reg_axis(const AxisPlan &p) { return !p.blu && p.m == p.n && reg_fft_length(p.n); }

// tile of T pencils from the tuned shared-memory target, at most tmax, balanced over
// the inner extent
long reg_tile(long target, long per_pencil, long tmax, long long inner) {
  long T = std::max(1L, std::min(tmax, target / per_pencil));
  T = std::min<long>(T, (long)optin_smem() / per_pencil - 1);  // room for the twiddle table
  T = std::max(1L, std::min<long>(T, inner));
  const long nt = (long)((inner + T - 1) / T);
  return (long)((inner + nt - 1) / nt);
}

template <typename R, bool INV>
void launch_axis_reg(int m, const AxisArgs<R> &a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
#define MUSG_AXR(M)                   \
  case M: {                           \
    auto k = k_axis_reg<R, M, INV>;   \
    allow_smem(k);                    \
    launch_pdl(k, grid, block, smem, s, a);   \
    break;                            \
  }
  switch (m) {
    MUSG_AXR(16) MUSG_AXR(32) MUSG_AXR(64) MUSG_AXR(128) MUSG_AXR(256)
    default: throw Error(MUSG_ERR_ARGUMENT, "no register FFT of this length");
  }
#undef MUSG_AXR
  MUSG_CHECK_LAUNCH();
}

template <typename R, int MODE, int D>
void launch_green_reg(int m, const GreenArgs<R> &a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
#define MUSG_GRR(M)                          \
  case M: {                                  \
    auto k = k_green_reg<R, M, MODE, D>;     \
    allow_smem(k);                           \
    launch_pdl(k, grid, block, smem, s, a);          \
    break;                                   \
  }
  switch (m) {
    MUSG_GRR(16) MUSG_GRR(32) MUSG_GRR(64) MUSG_GRR(128) MUSG_GRR(256)
    default: throw Error(MUSG_ERR_ARGUMENT, "no register FFT of this length");
  }
#undef MUSG_GRR
  MUSG_CHECK_LAUNCH();
}

// last-axis register kernels (FP32 CG passes): rows per block G = 2 G2 with the
// block (Y lanes, ncomp G2 pencils) a whole number of warps and at most 384 threads;
// G = 0 when the axis or the shape does not allow them
// Rows per block of the register last-axis passes (two rows share one complex
// transform, so G is even; a block is Y lanes x ncomp components x G/2 row pairs).
// Measured on 128^3 finite-strain cells (9 components, Y = 8): the forward pass is
// fastest at 144 threads (77 us; 78-86 us at 72, 216, 288 threads, 92 us at 360) and
// the inverse at 216 (70 us; 74 us at 288, 77 at 144, 91 at 72).  Small blocks keep
// more of them resident between the stage barriers; the rule takes the most row
// pairs whose block stays within those thread counts.  0 = no register path.
template <typename R> int last_reg_rows(const Spectral &sp, bool inv) {
  if (sizeof(R) != 4) return 0;
  const AxisPlan &ap = sp.ax[sp.g.dim - 1];
  if (!reg_axis(ap)) return 0;
  const int m = ap.m, Y = reg_lanes(m), nc = sp.ncomp;
  const long ps = (long)(m + m / RegLanesR1(m));
  const long per_g2 = (long)nc * ps * (long)sizeof(typename V2<R>::T);
  const long target = inv ? 224 : 160, bound = inv ? 384 : 512;  // launch bounds of the kernels
  const long th1 = (long)Y * nc;
  if (th1 > bound || per_g2 + (long)m * (long)sizeof(float2) > optin_smem()) return 0;
  long g2 = std::max(1L, target / th1);
  g2 = std::min<long>(g2, (sp.g.nrows + 1) / 2);
  g2 = std::min<long>(g2, (optin_smem() - (long)m * (long)sizeof(float2)) / per_g2);  // + twiddle table
  return (int)(2 * g2);
}

template <int D, int TK>
void launch_fwd_reg(int m, const LastArgs<float> &a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
#define MUSG_LFR(M)                           \
  case M: {                                   \
    auto k = k_last_fwd_reg<M, D, TK>;        \
    allow_smem(k);                            \
    launch_pdl(k, grid, block, smem, s, a);           \
    break;                                    \
  }
  switch (m) {
    MUSG_LFR(16) MUSG_LFR(32) MUSG_LFR(64) MUSG_LFR(128) MUSG_LFR(256)
    default: throw Error(MUSG_ERR_ARGUMENT, "no register FFT of this length");
  }
#undef MUSG_LFR
  MUSG_CHECK_LAUNCH();
}

template <int D>
void launch_inv_reg(int m, const LastArgs<float> &a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
#define MUSG_LIR(M)                           \
  case M: {                                   \
    auto k = k_last_inv_reg<M, D>;            \
    allow_smem(k);                            \
    launch_pdl(k, grid, block, smem, s, a);           \
    break;                                    \
  }
  switch (m) {
    MUSG_LIR(16) MUSG_LIR(32) MUSG_LIR(64) MUSG_LIR(128) MUSG_LIR(256)
    default: throw Error(MUSG_ERR_ARGUMENT, "no register FFT of this length");
  }
#undef MUSG_LIR
  MUSG_CHECK_LAUNCH();
}

// the two CG last-axis passes through the register kernels; returns the number of
// partial sums (blocks)
template <typename R>
int last_cg_reg(Spectral &sp, int tkind, LastArgs<R> a, int G, bool inv, cudaStream_t s, int B) {
  if constexpr (sizeof(R) != 4) {
    throw Error(MUSG_ERR_RUNTIME, "register last-axis passes are FP32 only");
  } else {
    const int m = sp.ax[sp.g.dim - 1].m, Y = reg_lanes(m);
    const int nc = sp.ncomp, G2 = G / 2;
    const int blocks = (int)((sp.g.nrows + G - 1) / G);
    const long ps = m + m / RegLanesR1(m);
    a.G = G;
    const dim3 grid(blocks, B), block(Y, nc * G2);
    const int wpb = (Y * nc * G2 + 31) / 32;  // warps per block (the forward pass's partial sums per block)
    const size_t smem = ((size_t)nc * G2 * ps + m) * sizeof(float2);  // pencils + twiddle table
    if (!inv) {
#define MUSG_FR(DD, TT) \
  if (sp.g.dim == DD && tkind == TT) { launch_fwd_reg<DD, TT>(m, a, grid, block, smem, s); return blocks * wpb; }
      MUSG_FR(2, TK_SMALL) MUSG_FR(2, TK_FINITE) MUSG_FR(2, TK_KPRIME) MUSG_FR(2, TK_MIXED) MUSG_FR(2, TK_FISO)
      MUSG_FR(3, TK_SMALL) MUSG_FR(3, TK_FINITE) MUSG_FR(3, TK_KPRIME) MUSG_FR(3, TK_MIXED) MUSG_FR(3, TK_FISO)
      MUSG_FR(2, TK_GSMALL) MUSG_FR(2, TK_GFINITE) MUSG_FR(3, TK_GSMALL) MUSG_FR(3, TK_GFINITE)
      MUSG_FR(2, TK_FULL) MUSG_FR(3, TK_FULL)
#undef MUSG_FR
      throw Error(MUSG_ERR_ARGUMENT, "unsupported tangent kind");
    }
    {
      const int nb = launch_last_inv_tma(sp, a, G, s, B);
      if (nb) return nb;
    }
    if (sp.g.dim == 2) launch_inv_reg<2>(m, a, grid, block, smem, s);
    else launch_inv_reg<3>(m, a, grid, block, smem, s);
    return blocks;
  }
}

template <typename R>
void run_axis(Spectral &sp, bool inv, const CGState *st, cudaStream_t s, const ProblemPtrs<R> *batch = nullptr,
              int B = 1) {
  // 3-D only: pencils along axis 1 of [c][k0][k1][k2h]
  const long long inner = sp.g.nh;
  const long long nbatch = (long long)sp.ncomp * sp.g.n[0];
  if (reg_axis(sp.ax[1])) {
    using T = typename V2<R>::T;
    const int m = sp.ax[1].m, Y = reg_lanes(m);
    const long Tt = reg_tile(sp.tune_bytes[prec_index<R>()][1], (long)m * sizeof(T), std::min(32, 512 / Y), inner);
    AxisArgs<R> a{};
    a.ap = sp.ax[1].device<R>();
    a.nax = m;
    a.T = (int)Tt;
    a.ntiles = (int)((inner + Tt - 1) / Tt);
    a.se = sp.g.nh;
    a.inner = inner;
    a.sb = (long long)sp.g.n[1] * sp.g.nh;
    a.spec = spec_of<R>(sp);
    a.st = st;
    a.batch = batch;
    const dim3 grid((unsigned)(a.ntiles * nbatch), 1, B), block((unsigned)Tt, Y, 1);
    const size_t smem = (size_t)(Tt + 1) * m * sizeof(T);  // tile + twiddle table
    if (inv) launch_axis_reg<R, true>(m, a, grid, block, smem, s);
    else launch_axis_reg<R, false>(m, a, grid, block, smem, s);
    return;
  }
  const Cfg c = axis_cfg<R>(sp, 1, inner, nbatch);
  AxisArgs<R> a{};
  a.ap = sp.ax[1].device<R>();
  a.nax = sp.g.n[1];
  a.T = c.per;
  a.ntiles = (int)((inner + c.per - 1) / c.per);
  a.se = sp.g.nh;
  a.inner = inner;
  a.sb = (long long)sp.g.n[1] * sp.g.nh;
  a.spec = spec_of<R>(sp);
  a.st = st;
  a.batch = batch;
  if (inv) {
    auto k = k_axis<R, true>;
    allow_smem(k);
    launch_pdl(k, dim3(c.blocks, B), dim3(c.threads), c.smem, s, a);
  } else {
    auto k = k_axis<R, false>;
    allow_smem(k);
    launch_pdl(k, dim3(c.blocks, B), dim3(c.threads), c.smem, s, a);
  }
  MUSG_CHECK_LAUNCH();
}

template <typename R>
void run_green(Spectral &sp, int mode, const CGState *st, cudaStream_t s, const ProblemPtrs<R> *batch = nullptr,
               int B = 1) {
  const int dim = sp.g.dim;
  const long long Rr = sp.g.nk / sp.g.n[0];
  const Cfg c = green_cfg<R>(sp, Rr);
  GreenArgs<R> a{};
  a.ap = sp.ax[0].device<R>();
  a.n0 = sp.g.n[0];
  a.T = c.per;
  a.ncomp = sp.ncomp;
  a.n1 = sp.g.n[1];
  a.nh = sp.g.nh;
  a.Rr = Rr;
  a.nk = sp.g.nk;
  a.spec = spec_of<R>(sp);
  a.xi0 = xi_of<R>(sp, 0);
  a.xi1 = xi_of<R>(sp, 1);
  a.xi2 = dim == 3 ? xi_of<R>(sp, 2) : nullptr;
  auto nyq = [&](int d) { return (sp.allow_even && sp.g.n[d] % 2 == 0) ? sp.g.n[d] / 2 : -1; };
  a.nyq0 = nyq(0);
  a.nyq1 = nyq(1);
  a.nyq2 = dim == 3 ? nyq(2) : -1;
  a.norm = R(1.0 / (double)sp.g.npx);
  a.st = st;
  a.batch = batch;
  if (reg_axis(sp.ax[0]) && (mode == GM_SMALL || mode == GM_FINITE)) {
    using T = typename V2<R>::T;
    const int m = sp.ax[0].m, Y = reg_lanes(m);
    const int nc = mode == GM_FINITE ? dim : dim * dim;
    const int tmax = std::min(32, 384 / (Y * nc));  // k_green_reg: at most 384 threads
    if (tmax >= 1) {
      const long Tt = reg_tile(sp.tune_bytes[prec_index<R>()][2], (long)nc * m * sizeof(T), tmax, Rr);
      a.T = (int)Tt;
      if constexpr (sizeof(R) == 4) {
        if (!batch && B == 1 && launch_green_tma(sp, mode, a, (int)Tt, s)) return;
      }
      const dim3 grid((unsigned)((Rr + Tt - 1) / Tt), mode == GM_FINITE ? dim : 1, B), block((unsigned)Tt, Y, nc);
      const size_t smem = (size_t)(nc * Tt + 1) * m * sizeof(T);  // tile + twiddle table
      if (mode == GM_FINITE && dim == 2) launch_green_reg<R, GM_FINITE, 2>(m, a, grid, block, smem, s);
      else if (mode == GM_FINITE) launch_green_reg<R, GM_FINITE, 3>(m, a, grid, block, smem, s);
      else if (dim == 2) launch_green_reg<R, GM_SMALL, 2>(m, a, grid, block, smem, s);
      else launch_green_reg<R, GM_SMALL, 3>(m, a, grid, block, smem, s);
      return;
    }
  }
#define MUSG_GREEN(MODE, DD)                                     \
  {                                                              \
    auto k = k_green<R, MODE, DD>;                               \
    allow_smem(k);                                               \
    launch_pdl(k, dim3(c.blocks, B), dim3(c.threads), c.smem, s, a);        \
  }
  if (mode == GM_FWD) MUSG_GREEN(GM_FWD, 2)
  else if (mode == GM_INV) MUSG_GREEN(GM_INV, 2)
  else if (mode == GM_SMALL && dim == 2) MUSG_GREEN(GM_SMALL, 2)
  else if (mode == GM_SMALL && dim == 3) MUSG_GREEN(GM_SMALL, 3)
  else if (mode == GM_FINITE && dim == 2) MUSG_GREEN(GM_FINITE, 2)
  else if (mode == GM_FINITE && dim == 3) MUSG_GREEN(GM_FINITE, 3)
  else throw Error(MUSG_ERR_ARGUMENT, "unsupported projection");
#undef MUSG_GREEN
  MUSG_CHECK_LAUNCH();
}

int green_mode_of(const Spectral &sp) {
  if (sp.proj_kind == MUSG_PROJ_SMALL_STRAIN) return GM_SMALL;
  if (sp.proj_kind == MUSG_PROJ_FINITE_STRAIN_FAST || sp.proj_kind == MUSG_PROJ_FINITE_STRAIN) return GM_FINITE;
  throw Error(MUSG_ERR_PROJECTION, "no projection operator attached to this spectral workspace");
}

}  // namespace

template <typename R>
void spectral_forward(Spectral &sp, const R *in, R scale, cudaStream_t s) {
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.in = in;
  a.scale = scale;
  dispatch_fwd<R, PRO_PLAIN>(sp.g.dim, TK_PLAIN, a, c, s);
  if (sp.g.dim == 3) run_axis<R>(sp, false, nullptr, s);
  run_green<R>(sp, GM_FWD, nullptr, s);
}

template <typename R>
void spectral_inverse(Spectral &sp, R *out, R scale, cudaStream_t s) {
  run_green<R>(sp, GM_INV, nullptr, s);
  if (sp.g.dim == 3) run_axis<R>(sp, true, nullptr, s);
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.out = out;
  a.scale = scale;
  launch_inv<R, EPI_PLAIN, 0>(a, c, s);
}

template <typename R>
void spectral_project(Spectral &sp, const R *in, R *out, R in_scale, cudaStream_t s) {
  const int gm = green_mode_of(sp);
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.in = in;
  a.out = out;
  a.scale = in_scale;
  dispatch_fwd<R, PRO_PLAIN>(sp.g.dim, TK_PLAIN, a, c, s);
  if (sp.g.dim == 3) run_axis<R>(sp, false, nullptr, s);
  run_green<R>(sp, gm, nullptr, s);
  if (sp.g.dim == 3) run_axis<R>(sp, true, nullptr, s);
  a.scale = R(1);
  launch_inv<R, EPI_PLAIN, 0>(a, c, s);
}

template <typename R>
int cg_operator(Spectral &sp, int tkind, const TangentData<R> &td, const CGState *st, R *r, R *x, R *p,
                R *Ap, double *partial, cudaStream_t s, cudaEvent_t *ev) {
  // FP32 (the mixed path's inner solve): the fused iteration; FP64: the reference's
  constexpr int kPro = sizeof(R) == 4 ? PRO_CGF : PRO_CG;
  constexpr int kEpi = sizeof(R) == 4 ? EPI_CGF : EPI_CG;
  const int gm = green_mode_of(sp);
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.st = st;
  a.r = r;
  a.x = x;
  a.p = p;
  a.Ap = Ap;
  a.partial = partial;
  a.td = td;
  int k = 0;
  auto mark = [&]() {
    if (ev) MUSG_CUDA(cudaEventRecord(ev[k++], s));
  };
  const int gfwd = last_reg_rows<R>(sp, false), ginv = last_reg_rows<R>(sp, true);
  const bool greg = gfwd && ginv;
  mark();
  int nfwd = c.blocks * ((c.threads + 31) / 32);  // the forward pass's per-warp partial sums
  if (greg) nfwd = last_cg_reg<R>(sp, tkind, a, gfwd, false, s, 1);
  else dispatch_fwd<R, kPro>(sp.g.dim, tkind, a, c, s);
  mark();
  if constexpr (sizeof(R) == 4) {
    // alpha, and x += alpha p, between the forward pass and the one that may end the loop
    cg_update_x<R>(st, x, p, sp.g.npx * sp.ncomp, partial, nfwd, s);
    mark();
  }
  if (sp.g.dim == 3) {
    run_axis<R>(sp, false, st, s);
    mark();
  }
  run_green<R>(sp, gm, st, s);
  mark();
  if (sp.g.dim == 3) {
    run_axis<R>(sp, true, st, s);
    mark();
  }
  int nb;
  if (greg) {
    nb = last_cg_reg<R>(sp, tkind, a, ginv, true, s, 1);
  } else {
    if (sp.g.dim == 2) launch_inv<R, kEpi, 2>(a, c, s);
    else launch_inv<R, kEpi, 3>(a, c, s);
    nb = c.blocks;
  }
  mark();
  return nb;
}

static_assert(sizeof(ProblemPtrs<float>) == sizeof(ProblemPtrsHost) &&
                  sizeof(ProblemPtrs<double>) == sizeof(ProblemPtrsHost),
              "host image of the batch table");

template <typename R>
int cg_operator_batch(Spectral &sp, int tkind, const ProblemPtrs<R> *tab, const BatchVec<R> *xtab, int B,
                      cudaStream_t s) {
  constexpr int kPro = sizeof(R) == 4 ? PRO_CGF : PRO_CG;
  constexpr int kEpi = sizeof(R) == 4 ? EPI_CGF : EPI_CG;
  const int gm = green_mode_of(sp);
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.batch = tab;
  const int gfwd = last_reg_rows<R>(sp, false), ginv = last_reg_rows<R>(sp, true);
  const bool greg = gfwd && ginv;
  int nfwd = c.blocks * ((c.threads + 31) / 32);
  if (greg) nfwd = last_cg_reg<R>(sp, tkind, a, gfwd, false, s, B);
  else dispatch_fwd<R, kPro>(sp.g.dim, tkind, a, c, s, B);
  if constexpr (sizeof(R) == 4) cg_update_x_batch<R>(xtab, sp.g.npx * sp.ncomp, nfwd, B, s);
  if (sp.g.dim == 3) run_axis<R>(sp, false, nullptr, s, tab, B);
  run_green<R>(sp, gm, nullptr, s, tab, B);
  if (sp.g.dim == 3) run_axis<R>(sp, true, nullptr, s, tab, B);
  if (greg) return last_cg_reg<R>(sp, tkind, a, ginv, true, s, B);
  if (sp.g.dim == 2) launch_inv<R, kEpi, 2>(a, c, s, B);
  else launch_inv<R, kEpi, 3>(a, c, s, B);
  return c.blocks;
}

template <typename R>
void tangent_operator(Spectral &sp, int tkind, const TangentData<R> &td, const R *in, R *out, cudaStream_t s) {
  const int gm = green_mode_of(sp);
  const Cfg c = last_cfg<R>(sp);
  LastArgs<R> a = last_args<R>(sp, c);
  a.in = in;
  a.out = out;
  a.scale = R(1);
  a.td = td;
  dispatch_fwd<R, PRO_TANGENT>(sp.g.dim, tkind, a, c, s);
  if (sp.g.dim == 3) run_axis<R>(sp, false, nullptr, s);
  run_green<R>(sp, gm, nullptr, s);
  if (sp.g.dim == 3) run_axis<R>(sp, true, nullptr, s);
  launch_inv<R, EPI_PLAIN, 0>(a, c, s);
}

// ------------------------------------------------------------------ grouped launches
// Device tables of one grouped operator: per pass the problems' arguments and the
// prefix sums of their blocks; one shared-memory size (the largest) and one block
// size (the first problem's tuned one) per pass.
struct GroupedOp {
  int dim = 0, tkind = 0, gm = 0, B = 0, prec = 0;
  int threads[3] = {0, 0, 0};
  size_t smem[3] = {0, 0, 0};
  int total[3] = {0, 0, 0};       // blocks of the last-axis, middle-axis and Green launches
  std::vector<int> fwd_parts;     // per problem: the forward pass's per-warp partial sums
  DevBuf last, axisf, axisi, green, blk;  // argument tables; blk: 3 x (B + 1) prefix sums
};

template <typename T> void upload_vec(DevBuf &d, const std::vector<T> &v) {
  d.alloc(v.size() * sizeof(T));
  MUSG_CUDA(cudaMemcpy(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

template <typename R> GroupedOp *grouped_op_create(const std::vector<GroupProblem> &probs, int tkind) {
  auto op = std::make_unique<GroupedOp>();
  const int B = (int)probs.size();
  Spectral &s0 = *probs[0].sp;
  op->dim = s0.g.dim;
  op->tkind = tkind;
  op->gm = green_mode_of(s0);
  op->B = B;
  op->prec = sizeof(R) == 8 ? 0 : 1;
  std::vector<LastArgs<R>> last(B);
  std::vector<AxisArgs<R>> axf(B), axi(B);
  std::vector<GreenArgs<R>> grn(B);
  std::vector<int> blk(3 * (B + 1), 0);
  op->fwd_parts.resize(B);
  for (int b = 0; b < B; ++b) {
    Spectral &sp = *probs[b].sp;
    if (sp.g.dim != op->dim || green_mode_of(sp) != op->gm || sp.ncomp != s0.ncomp)
      throw Error(MUSG_ERR_ARGUMENT, "a grouped operator needs one dimension, projection and component count");
    for (int k = 0; k < 3; ++k) {  // one block size per launch: the first problem's
      sp.tune_threads[op->prec][k] = s0.tune_threads[op->prec][k];
      sp.tune_bytes[op->prec][k] = s0.tune_bytes[op->prec][k];
    }
    // last axis
    const Cfg c = last_cfg<R>(sp);
    LastArgs<R> a = last_args<R>(sp, c);
    a.st = probs[b].st;
    a.r = static_cast<R *>(probs[b].r);
    a.x = static_cast<R *>(probs[b].x);
    a.p = static_cast<R *>(probs[b].p);
    a.Ap = static_cast<R *>(probs[b].Ap);
    a.partial = probs[b].partial;
    memcpy(&a.td, probs[b].td, sizeof(a.td));
    last[b] = a;
    blk[b + 1] = blk[b] + c.blocks;
    op->fwd_parts[b] = c.blocks * ((c.threads + 31) / 32);
    op->smem[0] = std::max(op->smem[0], c.smem);
    op->threads[0] = c.threads;
    // middle axis (3-D): the generic kernel's arguments of run_axis
    if (op->dim == 3) {
      const long long inner = sp.g.nh, nbatch = (long long)sp.ncomp * sp.g.n[0];
      const Cfg ca = axis_cfg<R>(sp, 1, inner, nbatch);
      AxisArgs<R> x{};
      x.ap = sp.ax[1].device<R>();
      x.nax = sp.g.n[1];
      x.T = ca.per;
      x.ntiles = (int)((inner + ca.per - 1) / ca.per);
      x.se = sp.g.nh;
      x.inner = inner;
      x.sb = (long long)sp.g.n[1] * sp.g.nh;
      x.spec = spec_of<R>(sp);
      x.st = probs[b].st;
      axf[b] = x;
      axi[b] = x;
      blk[(B + 1) + b + 1] = blk[(B + 1) + b] + ca.blocks;
      op->smem[1] = std::max(op->smem[1], ca.smem);
      op->threads[1] = ca.threads;
    }
    // first axis and the Green operator: the generic kernel's arguments of run_green
    const long long Rr = sp.g.nk / sp.g.n[0];
    const Cfg cg = green_cfg<R>(sp, Rr);
    GreenArgs<R> g{};
    g.ap = sp.ax[0].device<R>();
    g.n0 = sp.g.n[0];
    g.T = cg.per;
    g.ncomp = sp.ncomp;
    g.n1 = sp.g.n[1];
    g.nh = sp.g.nh;
    g.Rr = Rr;
    g.nk = sp.g.nk;
    g.spec = spec_of<R>(sp);
    g.xi0 = xi_of<R>(sp, 0);
    g.xi1 = xi_of<R>(sp, 1);
    g.xi2 = op->dim == 3 ? xi_of<R>(sp, 2) : nullptr;
    auto nyq = [&](int d) { return (sp.allow_even && sp.g.n[d] % 2 == 0) ? sp.g.n[d] / 2 : -1; };
    g.nyq0 = nyq(0);
    g.nyq1 = nyq(1);
    g.nyq2 = op->dim == 3 ? nyq(2) : -1;
    g.norm = R(1.0 / (double)sp.g.npx);
    g.st = probs[b].st;
    grn[b] = g;
    blk[2 * (B + 1) + b + 1] = blk[2 * (B + 1) + b] + cg.blocks;
    op->smem[2] = std::max(op->smem[2], cg.smem);
    op->threads[2] = cg.threads;
  }
  for (int k = 0; k < 3; ++k) op->total[k] = blk[k * (B + 1) + B];
  upload_vec(op->last, last);
  if (op->dim == 3) {
    upload_vec(op->axisf, axf);
    upload_vec(op->axisi, axi);
  }
  upload_vec(op->green, grn);
  upload_vec(op->blk, blk);
  return op.release();
}

template <typename R, int PRO, int D, int TK>
void launch_fwd_g(const GroupedOp &op, cudaStream_t s) {
  auto k = k_last_fwd_g<R, PRO, D, TK>;
  allow_smem(k);
  launch_pdl(k, dim3(op.total[0]), dim3(op.threads[0]), op.smem[0], s, op.last.as<const LastArgs<R>>(),
             op.blk.as<const int>(), op.B);
  MUSG_CHECK_LAUNCH();
}

template <typename R>
void grouped_op_run(GroupedOp *op, const BatchVec<R> *xtab, long long nmax, int B, cudaStream_t s) {
  constexpr int kPro = sizeof(R) == 4 ? PRO_CGF : PRO_CG;
  constexpr int kEpi = sizeof(R) == 4 ? EPI_CGF : EPI_CG;
  const int dim = op->dim, tk = op->tkind, Bp = op->B + 1;
  const int *blk = op->blk.as<const int>();
  // last-axis forward with the CG prologue
#define MUSG_FWDG_CASE(DD, TT) \
  if (dim == DD && tk == TT) { launch_fwd_g<R, kPro, DD, TT>(*op, s); goto fwd_done; }
  MUSG_FWDG_CASE(2, TK_SMALL) MUSG_FWDG_CASE(2, TK_FINITE) MUSG_FWDG_CASE(2, TK_KPRIME) MUSG_FWDG_CASE(2, TK_MIXED)
  MUSG_FWDG_CASE(3, TK_SMALL) MUSG_FWDG_CASE(3, TK_FINITE) MUSG_FWDG_CASE(3, TK_KPRIME) MUSG_FWDG_CASE(3, TK_MIXED)
  MUSG_FWDG_CASE(2, TK_GSMALL) MUSG_FWDG_CASE(2, TK_GFINITE) MUSG_FWDG_CASE(3, TK_GSMALL) MUSG_FWDG_CASE(3, TK_GFINITE)
  MUSG_FWDG_CASE(2, TK_FULL) MUSG_FWDG_CASE(3, TK_FULL)
  if constexpr (sizeof(R) == 4) {
    MUSG_FWDG_CASE(2, TK_FISO) MUSG_FWDG_CASE(3, TK_FISO)
  }
#undef MUSG_FWDG_CASE
  throw Error(MUSG_ERR_ARGUMENT, "unsupported tangent kind");
fwd_done:
  // FP32: alpha from each problem's own partial sums (nparts < 0), x += alpha p
  if constexpr (sizeof(R) == 4) cg_update_x_batch<R>(xtab, nmax, -1, B, s);
  if (dim == 3) {
    auto k = k_axis_g<R, false>;
    allow_smem(k);
    launch_pdl(k, dim3(op->total[1]), dim3(op->threads[1]), op->smem[1], s, op->axisf.as<const AxisArgs<R>>(),
               blk + Bp, op->B);
    MUSG_CHECK_LAUNCH();
  }
  {
#define MUSG_GREENG(MODE, DD)                                                                                   \
  {                                                                                                             \
    auto k = k_green_g<R, MODE, DD>;                                                                            \
    allow_smem(k);                                                                                              \
    launch_pdl(k, dim3(op->total[2]), dim3(op->threads[2]), op->smem[2], s, op->green.as<const GreenArgs<R>>(), \
               blk + 2 * Bp, op->B);                                                                            \
  }
    if (op->gm == GM_SMALL && dim == 2) MUSG_GREENG(GM_SMALL, 2)
    else if (op->gm == GM_SMALL) MUSG_GREENG(GM_SMALL, 3)
    else if (dim == 2) MUSG_GREENG(GM_FINITE, 2)
    else MUSG_GREENG(GM_FINITE, 3)
#undef MUSG_GREENG
    MUSG_CHECK_LAUNCH();
  }
  if (dim == 3) {
    auto k = k_axis_g<R, true>;
    allow_smem(k);
    launch_pdl(k, dim3(op->total[1]), dim3(op->threads[1]), op->smem[1], s, op->axisi.as<const AxisArgs<R>>(),
               blk + Bp, op->B);
    MUSG_CHECK_LAUNCH();
  }
  {
    auto k = dim == 2 ? k_last_inv_g<R, kEpi, 2> : k_last_inv_g<R, kEpi, 3>;
    allow_smem(k);
    launch_pdl(k, dim3(op->total[0]), dim3(op->threads[0]), op->smem[0], s, op->last.as<const LastArgs<R>>(), blk,
               op->B);
    MUSG_CHECK_LAUNCH();
  }
}

// Autotuner: candidate (threads, shared-memory target) per pass, each timed with
// CUDA events over `reps` launches on a scratch field; the fastest is kept.
template <typename R> void spectral_autotune(Spectral &sp, cudaStream_t s, int effort) {
  const int pi = prec_index<R>();
  const long long n = (long long)sp.g.npx * sp.ncomp;
  R *field = nullptr;
  MUSG_CUDA(cudaMalloc(&field, (size_t)n * sizeof(R)));
  MUSG_CUDA(cudaMemsetAsync(field, 0, (size_t)n * sizeof(R), s));
  cudaEvent_t e0, e1;
  MUSG_CUDA(cudaEventCreate(&e0));
  MUSG_CUDA(cudaEventCreate(&e1));
  const int reps = effort >= 2 ? 5 : 3;
  const int threads[] = {128, 256, 512};
  const long bytes[] = {16384, 32768, 49152, 73728, 110592, 225280};
  const int gm = sp.proj_kind >= 0 ? green_mode_of(sp) : GM_FWD;
  try {
    for (int pass = 0; pass < 3; ++pass) {
      if (pass == 1 && sp.g.dim != 3) continue;
      float best = 1e30f;
      int bt = sp.tune_threads[pi][pass];
      long bb = sp.tune_bytes[pi][pass];
      // the register-resident passes take their block shape from the tile alone:
      // sweep tiles of T pencils directly (the shared-memory target of T pencils)
      const bool reg = (pass == 1 && reg_axis(sp.ax[1])) || (pass == 2 && reg_axis(sp.ax[0]) && gm != GM_FWD);
      std::vector<long> cand(bytes, bytes + sizeof(bytes) / sizeof(bytes[0]));
      if (reg) {
        const int m = sp.ax[pass == 1 ? 1 : 0].m;
        const long nc = pass == 1 ? 1 : (gm == GM_FINITE ? sp.g.dim : (long)sp.g.dim * sp.g.dim);
        const long pencil = nc * m * (long)sizeof(typename V2<R>::T);
        cand.clear();
        for (long T : {4L, 8L, 12L, 16L, 24L, 32L}) cand.push_back(T * pencil);
      }
      for (int th : threads)
        for (long by : cand) {
          if (reg && th != threads[0]) continue;
          sp.tune_threads[pi][pass] = th;
          sp.tune_bytes[pi][pass] = by;
          float tot = 0;
          for (int r = -1; r < reps; ++r) {
            MUSG_CUDA(cudaEventRecord(e0, s));
            if (pass == 0) {
              const Cfg c = last_cfg<R>(sp);
              LastArgs<R> a = last_args<R>(sp, c);
              a.in = field;
              a.out = field;
              a.scale = R(1);
              dispatch_fwd<R, PRO_PLAIN>(sp.g.dim, TK_PLAIN, a, c, s);
              launch_inv<R, EPI_PLAIN, 0>(a, c, s);
            } else if (pass == 1) {
              run_axis<R>(sp, false, nullptr, s);
            } else {
              run_green<R>(sp, gm, nullptr, s);
            }
            MUSG_CUDA(cudaEventRecord(e1, s));
            MUSG_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            MUSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (r >= 0) tot += ms;
          }
          if (tot < best) {
            best = tot;
            bt = th;
            bb = by;
          }
        }
      sp.tune_threads[pi][pass] = bt;
      sp.tune_bytes[pi][pass] = bb;
    }
  } catch (...) {
    cudaFree(field);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaFree(field);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
}

#define MUSG_INSTANTIATE_SPECTRAL(R)                                                               \
  template void spectral_forward<R>(Spectral &, const R *, R, cudaStream_t);                      \
  template void spectral_inverse<R>(Spectral &, R *, R, cudaStream_t);                            \
  template void spectral_project<R>(Spectral &, const R *, R *, R, cudaStream_t);                 \
  template int cg_operator<R>(Spectral &, int, const TangentData<R> &, const CGState *, R *, R *,  \
                              R *, R *, double *, cudaStream_t, cudaEvent_t *);                    \
  template void tangent_operator<R>(Spectral &, int, const TangentData<R> &, const R *, R *,       \
                                    cudaStream_t);                                                 \
  template void spectral_autotune<R>(Spectral &, cudaStream_t, int);                               \
  template int cg_operator_batch<R>(Spectral &, int, const ProblemPtrs<R> *, const BatchVec<R> *, int,         \
                                    cudaStream_t);                                                             \
  template GroupedOp *grouped_op_create<R>(const std::vector<GroupProblem> &, int);                         \
  template void grouped_op_run<R>(GroupedOp *, const BatchVec<R> *, long long, int, cudaStream_t);

}  // namespace musg
