// Internal declarations shared by the CUDA translation units and the host API of
// libmusg.  Nothing here is part of the C ABI (include/musg.h is).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/musg.h"

namespace musg {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};


// Runs f, maps an exception to a status code and the calling thread's last-error
// message (the C-ABI convention of every musg_* entry point)
int guarded(const std::function<void()> &f);

#define MUSG_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      throw ::musg::Error(e_ == cudaErrorMemoryAllocation ? MUSG_ERR_MEMORY          \
                                                          : MUSG_ERR_CUDA,           \
                          std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

// kernels launched by the library in this process (graph replays add their nodes)
extern std::atomic<unsigned long long> g_launches;

#define MUSG_CHECK_LAUNCH()                 \
  do {                                      \
    ::musg::g_launches.fetch_add(1);        \
    MUSG_CUDA(cudaGetLastError());          \
  } while (0)

// Programmatic dependent launch: a kernel launched with launch_pdl may be scheduled
// while the previous kernel of its stream finishes (its launch overlaps that tail);
// it calls dep_wait() before it reads anything, which returns once the previous grid
// has completed and its memory is visible.  No kernel here triggers early, so the
// previous grid's blocks have all exited before any block of the next one runs.
#ifdef __CUDACC__
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  MUSG_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}
#endif

template <typename R> struct V2;
template <> struct V2<float> { using T = float2; };
template <> struct V2<double> { using T = double2; };

constexpr int kMaxStages = 12;  // 5 bits per stage in AxisPlanD::rcode
constexpr int kMaxMaterials = 256;
// MaterialHyperElastoPlastic1 mode (MatParams::logm_mode) with the consistent tangent
constexpr int kHep1Consistent = 2;

// ---------------------------------------------------------------- FFT plans
// Device view of a 1-D FFT plan for one axis.  A length-n transform runs as a
// Stockham mixed-radix FFT of length m (m == n), or, when n has a prime factor
// above 7, as Bluestein's chirp-z algorithm over a 2/3/5/7-smooth m >= 2n-1.
template <typename R> struct AxisPlanD {
  int n;
  int m;
  int nst;
  int blu;
  unsigned long long rcode;  // radix of stage s in bits [5s, 5s+5)
  const typename V2<R>::T *tw;    // m entries: exp(-2 pi i j / m)
  const typename V2<R>::T *chirp; // n entries: exp(-pi i j^2 / n)     (Bluestein)
  const typename V2<R>::T *bf;    // m entries: DFT_m(conj chirp)/m     (Bluestein)
};

struct AxisPlan {
  int n = 0, m = 0, nst = 0, blu = 0;
  int radix[kMaxStages] = {0};
  // device tables, double and float copies
  void *tw64 = nullptr, *chirp64 = nullptr, *bf64 = nullptr;
  void *tw32 = nullptr, *chirp32 = nullptr, *bf32 = nullptr;
  void build(int n);
  void release();
  template <typename R> AxisPlanD<R> device() const;
};

// ---------------------------------------------------------------- geometry
struct Geom {
  int dim = 0;
  int n[3] = {1, 1, 1};     // real grid, row-major, n[dim-1] is the last axis
  int nh = 0;               // n_last/2 + 1
  long long npx = 0;        // pixels
  long long nk = 0;         // hermitian k-points
  long long nrows = 0;      // npx / n_last
  int nlast() const { return n[dim - 1]; }
};

// Per-pixel tangent representation used by the CG operator (pass A prologue).
enum TangentKind : int {
  TK_PLAIN = 0,   // no tangent: input field copied (FFT engine / projection)
  TK_SMALL = 1,   // small strain, isotropic: dP = lam tr(dF) I + mu (dF + dF^T)
  TK_FINITE = 2,  // finite strain, isotropic PK2/GL: dP = dF S + F (lam tr(A) I + mu (A + A^T)), A = F^T dF
  TK_KPRIME = 3,  // j-independent Kirchhoff tangent: dP(i,m) = sum_n K'(i,m,n) sum_j dF(j,n)
  TK_MIXED = 4,   // per-pixel choice between TK_FINITE and TK_KPRIME by material law
  TK_FISO = 5,    // TK_FINITE with S rebuilt from F per application (isotropic LE1/LE3/LE4)
  TK_GSMALL = 6,  // small strain, per-material stiffness C (MaterialLinearElasticGeneric): dP = C:de
  TK_GFINITE = 7, // finite strain, per-material C: dP = dF S + F (C:(F^T dF))
  TK_FULL = 8,    // stored per-pixel tangent K(i,m,j,n) (D^4 planes): dP = K:dF (the consistent
                  // elasto-plastic tangent, and the elastic pixels of a cell that has it)
};

// A caller's stop flag (a host int another thread may set): nonzero ends a running
// solve at its next check with MUSG_ERR_RUNTIME "cancelled while running".
inline void check_stop(const int *flag) {
  if (flag && __atomic_load_n(flag, __ATOMIC_RELAXED) != 0) throw Error(MUSG_ERR_RUNTIME, "cancelled while running");
}

// Device data the CG operator reads (precision R).
template <typename R> struct TangentData {
  const R *lam = nullptr;   // [npx]
  const R *mu = nullptr;    // [npx]
  const R *F = nullptr;     // [D*D][npx]  (finite strain): F in FP64, F - I in FP32
  const R *S = nullptr;     // [D*D][npx] PK2 stress (finite strain, isotropic)
  const R *Kp = nullptr;    // [D^3][npx]  (Kirchhoff tangent)
  const uint8_t *mat = nullptr;      // [npx] material index (TK_MIXED, C)
  const uint8_t *law_kind = nullptr; // [kMaxMaterials]: TK_FINITE or TK_KPRIME (TK_MIXED)
  const R *C = nullptr;     // [nmat][D^4] stiffness per material (TK_GSMALL / TK_GFINITE)
  const R *Kt = nullptr;    // [D^4][npx] per-pixel tangent planes, entry (i + D m) + D^2 (j + D n) (TK_FULL)
};

// CG scalar state, resident on the device (all FP64).
struct CGState {
  double rdr;        // r.r of the current residual
  double rhs_norm2;  // rhs.rhs
  double tol2;       // tol^2 * rhs.rhs
  double alpha, beta, pAp;
  int iter;          // iterations of this solve
  int maxiter;
  int active;        // 1 while the loop runs
  int ticket;        // blocks of the running kernel that have written their partial sum
  unsigned long long counter;  // cumulative iterations (SolverBase::counter)
};

// ---------------------------------------------------------------- spectral ops
// Workspace + plans for one grid; one instance per cell / FFT engine / projection.
struct Spectral {
  Geom g;
  int ncomp = 0;            // components per pixel
  int proj_kind = -1;       // MUSG_PROJ_* (-1: none)
  bool allow_even = false;
  double lengths[3] = {1, 1, 1};
  AxisPlan ax[3];
  // per-axis xi_d(k) = fftfreq_d(k)/L_d over the hermitian index range, FP64 and FP32
  void *xi64[3] = {nullptr, nullptr, nullptr};
  void *xi32[3] = {nullptr, nullptr, nullptr};
  void *spec64 = nullptr;   // [ncomp][nk] complex double
  void *spec32 = nullptr;   // [ncomp][nk] complex float
  bool want32 = false;
  // launch shapes per precision (0: FP64, 1: FP32) and pass (0: last, 1: axis,
  // 2: green): threads per block and the shared memory a block aims for; set by
  // the defaults below or by spectral_autotune
  int tune_threads[2][3] = {{256, 256, 256}, {256, 256, 256}};
  long tune_bytes[2][3] = {{73728, 49152, 73728}, {73728, 49152, 73728}};
  // TMA descriptor of the FP32 spectrum for the Green pass (an opaque CUtensorMap,
  // encoded on first use for the tile width and mode below) and its persistent grid
  unsigned char green_tmap[128] = {};
  const void *green_tmap_spec = nullptr;
  int green_tmap_T = 0, green_tmap_mode = -1, green_tmap_grid = 0;
  void init(int dim, const int *res, int ncomp, int proj_kind, const double *lengths,
            bool allow_even, bool want32);
  void ensure32();
  void release();
};

// Device word set by a kernel whose bounded wait on an asynchronous copy ran out
// (spectral_tma.cuh); its device address, for a stream-ordered read by the host
unsigned *wait_fault_word();
// one block that waits on an mbarrier nothing arrives at, bounded by limit_ns
// (self-test of the bounded waits: it sets the fault word and exits)
void wait_probe(unsigned long long limit_ns, cudaStream_t s);

// Launch configuration limits of the pass kernels
constexpr int kPassThreads = 512;

// Pass launchers (spectral_*.cu).  All run on `stream`.
//  fwd: real field [ncomp][npx] (scaled) -> spectrum (r2c over all axes)
//  inv: spectrum -> real field (c2r, unnormalised, scaled)
//  project: real -> real through the Green operator of sp.proj_kind
template <typename R>
void spectral_forward(Spectral &sp, const R *in, R scale, cudaStream_t s);
template <typename R>
void spectral_inverse(Spectral &sp, R *out, R scale, cudaStream_t s);
template <typename R>
void spectral_project(Spectral &sp, const R *in, R *out, R in_scale, cudaStream_t s);

// CG operator application with the iteration's vector work fused into its passes.
// FP64 (the reference's order): p = -r + beta p (or p = -r on the first iteration),
// Ap = G(K:p), and alpha = r.r / p.Ap in the state (last block of the last pass);
// cg_update completes the iteration.  FP32 (the mixed path's inner solve): the whole
// iteration: the first pass writes the block sums of p.(K:p), cg_update_x sets
// alpha = r.r / p.(K:p) and applies x += alpha p, the last pass r += alpha Ap, beta
// and the loop condition; x is not
// read in FP64, and Ap is written in FP32 only when non-null.  Returns the number of
// partial sums written by the last pass.  ev (optional): an event is recorded before
// the first and after every kernel
template <typename R>
int cg_operator(Spectral &sp, int tkind, const TangentData<R> &td, const CGState *st,
                R *r, R *x, R *p, R *Ap, double *partial, cudaStream_t s,
                cudaEvent_t *ev = nullptr);
// plain operator (no CG state): out = G(K:in)
template <typename R>
void tangent_operator(Spectral &sp, int tkind, const TangentData<R> &td, const R *in,
                      R *out, cudaStream_t s);
// batched CG operator over B same-shape problems (one launch per pass; problem b
// is blockIdx.y); tab is a device array of B ProblemPtrs (spectral.cuh), whose host
// image is ProblemPtrsHost
template <typename R> struct ProblemPtrs;
struct ProblemPtrsHost {
  void *spec;
  const CGState *st;
  void *r;
  void *x;
  void *p;
  void *Ap;
  double *partial;
  unsigned char td[sizeof(TangentData<double>)];
};
template <typename R> struct BatchVec;
template <typename R>
int cg_operator_batch(Spectral &sp, int tkind, const ProblemPtrs<R> *tab, const BatchVec<R> *xtab, int B,
                      cudaStream_t s);
// Grouped CG operator over problems of different grids (the same dimension,
// projection and tangent kind): one launch per pass for all of them, problem b
// owning a contiguous range of the one-dimensional grid (generic pass kernels, whose
// plans and sizes are runtime values).  The per-problem arguments live in device
// tables built once; run launches one CG iteration's passes (FP32: with cg_alpha /
// cg_update_x over xtab between the forward and the middle passes).
struct GroupProblem {
  Spectral *sp;
  const CGState *st;
  void *r, *x, *p, *Ap;
  double *partial;
  unsigned char td[sizeof(TangentData<double>)];
};
struct GroupedOp;
template <typename R> GroupedOp *grouped_op_create(const std::vector<GroupProblem> &probs, int tkind);
void grouped_op_destroy(GroupedOp *op);
// partial sums the grouped forward pass writes for problem b (its blocks x warps)
int grouped_op_fwd_partials(const GroupedOp *op, int b);
template <typename R>
void grouped_op_run(GroupedOp *op, const BatchVec<R> *xtab, long long nmax, int B, cudaStream_t s);
// Times candidate launch shapes of each pass on this grid (CUDA events) and keeps
// the fastest (FFT_PlanFlags::measure / patient); fp32 selects the FP32 passes.
template <typename R> void spectral_autotune(Spectral &sp, cudaStream_t s, int effort);

// ---------------------------------------------------------------- CG kernels (cg.cu)
int reduce_blocks(long long n);
// per-component means of a field [ncomp][npx] into out[ncomp] (device); partial
// holds ncomp * 1024 doubles
void plane_means(const double *f, int ncomp, long long npx, double *partial, double *out, cudaStream_t s);
// blocks (= partial sums) of cg_update / cg_update_batch for n entries
int update_blocks(long long n);
template <typename R>
void cg_init(CGState *st, const double *rhs, R *r, R *x, long long n, double tol,
             int maxiter, double *partial, double *partial2, cudaStream_t s);
template <typename R>
void cg_update(CGState *st, R *x, R *r, const R *p, const R *Ap, long long n,
               double *partial, cudaStream_t s);
// batched variants: per-problem pointer tables (device arrays of B entries)
template <typename R> struct BatchVec {
  CGState *st;
  R *x;
  R *r;
  const R *p;
  const R *Ap;
  double *partial;
  long long n;  // entries of the problem's vectors
  int nparts;   // the forward pass's partial sums of the problem (grouped launches)
};
template <typename R>
void cg_update_batch(const BatchVec<R> *tab, long long n, int B, cudaStream_t s);
// alpha from the forward pass's nparts block sums of p.(K:p) and x += alpha p of the
// FP32 inner solve's iteration, launched between its forward and inverse passes
// (solo / batched; a batch's problems have nparts sums each in their partial arrays)
template <typename R>
void cg_update_x(const CGState *st, R *x, const R *p, long long n, const double *partial, int nparts,
                 cudaStream_t s);
template <typename R> void cg_update_x_batch(const BatchVec<R> *tab, long long n, int nparts, int B, cudaStream_t s);
// FP64 dot of a with b over n entries into *out_device (deterministic)
template <typename Ra, typename Rb>
void dot_device(const Ra *a, const Rb *b, long long n, double *partial, double *out,
                cudaStream_t s);
// y += x (promoting), with the dots x.x and y.y (after the update) into out[0], out[1]
// d = (float)(rhs - (P - Pk)), Pk = P: the FP32 input of the mixed path's
// incremental Newton residual
void residual_input(const double *rhs, const double *P, double *Pk, float *d, long long n, cudaStream_t s);
template <typename R>
void newton_update(double *F, const R *x, long long n, double *partial, double *out,
                   cudaStream_t s);
// line-search trial F = F0 + lam x, with x.x and F.F into out[0], out[1]
template <typename R>
void newton_trial(double *F, const double *F0, const R *x, double lam, long long n, double *partial, double *out,
                  cudaStream_t s);
template <typename Rd, typename Rs>
void convert(Rd *dst, const Rs *src, long long n, double scale, cudaStream_t s);

// ---------------------------------------------------------------- materials (materials.cu)
struct MatParams {
  int law;
  int logm_mode;            // HEP1: 0 projector sum (reference), 1 spectral, 2 spectral with the
                            // consistent Kirchhoff->PK1 tangent (kHep1Consistent)
  double lam, mu, K, tau_y0, H;
};

struct MaterialArgs {
  int dim, form;
  long long npx;
  const double *F;          // [D*D][npx]
  double *P;                // [D*D][npx]
  const uint8_t *mat;       // [npx]
  const MatParams *params;  // [nmat]
  const double *lam, *mu;   // [npx] (elastic laws)
  const double *eig;        // [D*D][npx] eigenstrain (LE2), may be null
  const double *Ctab;       // [nmat][D^4] stiffness of MaterialLinearElasticGeneric materials
  // HEP1 state, two buffers each; cur selects the current one
  double *Fprev[2], *be[2], *eps[2];
  int cur;
  // tangent outputs in CG precision (float or double, one of them set)
  double *S64, *Kp64, *Fc64;
  float *S32, *Kp32, *Fc32;
  double *Kfull;            // optional full tangent, AoS [npx][D^4] (API)
  double *Kt64;             // TK_FULL: tangent planes [D^4][npx] in the CG precision (one set)
  float *Kt32;
  int *nonfinite;           // device flag set when a non-finite stress appears
  int has_hep;              // any MaterialHyperElastoPlastic1 pixel in the cell
};
void material_evaluate(const MaterialArgs &a, cudaStream_t s);
void add_macro(double *F, const double *delta_dev, int ncomp, long long npx, cudaStream_t s);
void fill_uniform(double *F, const double *value_dev, int ncomp, long long npx, cudaStream_t s);
// per-pixel Lame planes from the material index and the per-material parameters
void fill_lame(const uint8_t *mat, const MatParams *params, double *lam, double *mu, long long npx, cudaStream_t s);

// AoS (host layout, pixel-major) <-> SoA (component planes) on the device
void aos_to_soa(const double *aos, double *soa, int ncomp, long long npx, cudaStream_t s);
void soa_to_aos(const double *soa, double *aos, int ncomp, long long npx, cudaStream_t s);
void soa_to_aos_complex(const double2 *soa, double2 *aos, int ncomp, long long nk, cudaStream_t s);
void aos_to_soa_complex(const double2 *aos, double2 *soa, int ncomp, long long nk, cudaStream_t s);

// measured FP64 FMA throughput of the current device, TFLOP/s (probe.cu)
double fp64_fma_tflops(cudaStream_t s);

// allocation-free projection on caller device buffers (noalloc.cu)
void noalloc_project(int dim, const int *resolutions, const double *lengths, int kind, int flags,
                     const double *in_device, double *out_device, cudaStream_t s);

// simple device buffer
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  void alloc(size_t b);
  void release();
  template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
  ~DevBuf() { release(); }
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
};

}  // namespace musg
