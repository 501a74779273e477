// Allocation-free projection: musg_projection_apply_noalloc (include/musg.h).
//
// Some callers cannot allocate device memory: code running inside a caller-owned
// memory pool or arena that forbids cudaMalloc/cudaFree, allocation-free real-time
// or embedded loops, or hosts that hand the library their own device buffers and
// nothing else.  This entry point applies the same Green-operator projection as
// musg_projection_apply, but on caller device buffers, and keeps every temporary
// (the component-plane copy of the field, the half spectrum, the FFT twiddle /
// Bluestein tables and the wave-vector tables) in one file-scope device array of
// kNoAllocScratchBytes.  It calls no cudaMalloc, cudaFree or allocating library
// routine, on the device or the host.
//
// Properties a caller must know:
//  * The array is part of the library image: every GPU that loads libmusg's device
//    code holds kNoAllocScratchBytes (64 MiB) for it until the process exits.  Under
//    CUDA's lazy module loading (the default since CUDA 12.2) that memory is
//    committed when the module is first used on the device, at the latest by the
//    first call here; if a caller's pool has taken the device memory by then, that
//    first call fails with MUSG_ERR_CUDA (out of memory).  Callers that reserve the
//    device memory for a pool should make one call (any small grid) before they do,
//    or run with CUDA_MODULE_LOADING=EAGER.
//  * Grids whose temporaries do not fit are rejected with MUSG_ERR_ARGUMENT before
//    anything is looked up or launched.
//  * The first call on a device looks the array's device address up
//    (cudaGetSymbolAddress) and caches it; make that first call before any CUDA
//    stream capture.
//  * All calls share the one array and it keeps the previous call's contents.
//    Every region is fully written before it is read, so nothing needs clearing;
//    but calls that overlap on the GPU (different streams, or concurrent host
//    threads) race on the array and must be serialised by the caller.
//  * The work is enqueued on `cuda_stream`; the call returns before it finishes.
#include <cmath>
#include <mutex>

#include "musg_internal.h"

namespace musg {
namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// the device address of the array for the current device (host code must not use
// the symbol itself: on the host it only names a stand-in)
void *scratch_address() {
  int dev = 0;
  MUSG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) throw Error(MUSG_ERR_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    MUSG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = p;
  }
  return g_noalloc_addr[dev];
}

// radices of a 2/3/5/7-smooth length (the policy of the allocating plans); false
// when another prime divides n
bool factor_fixed(int n, int *rad, int &nst) {
  nst = 0;
  int k = 0;
  while (n % 2 == 0) { n /= 2; ++k; }
  auto push = [&](int r) {
    if (nst < kMaxStages) rad[nst] = r;
    ++nst;
  };
  while (k > 0) {
    if (k >= 4 && k != 5 && k != 6) { push(16); k -= 4; }
    else if (k == 6) { push(8); push(8); k = 0; }
    else if (k == 5) { push(8); push(4); k = 0; }
    else if (k == 3) { push(8); k = 0; }
    else if (k == 2) { push(4); k = 0; }
    else { push(2); k = 0; }
  }
  while (n % 9 == 0) { push(9); n /= 9; }
  for (int r : {3, 5, 7})
    while (n % r == 0) { push(r); n /= r; }
  return n == 1 && nst <= kMaxStages;
}

int smooth_ge(int v) {
  for (int m = v;; ++m) {
    int t = m;
    for (int r : {2, 3, 5, 7})
      while (t % r == 0) t /= r;
    if (t == 1) return m;
  }
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// twiddles exp(-2 pi i j/m), Bluestein chirp exp(-pi i (j^2 mod 2n)/n) and the wave
// vector table fftfreq(n)[k]/L of one axis
__global__ void k_fill_axis(double2 *tw, int m, double2 *chirp, int n, double *xi, int len, double length) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m || j < n || j < len; j += gridDim.x * blockDim.x) {
    if (j < m) {
      double s, c;
      sincospi(-2.0 * (double)j / (double)m, &s, &c);
      tw[j] = make_double2(c, s);
    }
    if (chirp && j < n) {
      const long long q = ((long long)j * j) % (2LL * n);
      double s, c;
      sincospi(-(double)q / (double)n, &s, &c);
      chirp[j] = make_double2(c, s);
    }
    if (j < len) {
      const int N = (n - 1) / 2 + 1;
      const double f = j < N ? (double)j : (double)(-(n / 2) + j - N);
      xi[j] = f / length;
    }
  }
}

// Bluestein filter DFT_m(b)/m, b[t] = conj(chirp[|t|]) on the circle of length m,
// by a direct DFT with Kahan-compensated sums (one output per thread)
__global__ void k_fill_bluestein(const double2 *chirp, int n, double2 *bf, int m) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  double sr = 0, cr = 0, si = 0, ci = 0;
  for (int t = 0; t < m; ++t) {
    int a = -1;
    if (t < n) a = t;
    else if (t > m - n) a = m - t;
    if (a < 0) continue;
    const double2 w = chirp[a];
    const double br = w.x, bi = -w.y;
    const long long q = ((long long)t * k) % m;
    double s, c;
    sincospi(-2.0 * (double)q / (double)m, &s, &c);
    const double tr = br * c - bi * s, ti = br * s + bi * c;
    double y = tr - cr, u = sr + y;
    cr = (u - sr) - y;
    sr = u;
    y = ti - ci;
    u = si + y;
    ci = (u - si) - y;
    si = u;
  }
  bf[k] = make_double2(sr / m, si / m);
}

}  // namespace

void noalloc_project(int dim, const int *resolutions, const double *lengths, int kind, int flags,
                     const double *in_device, double *out_device, cudaStream_t s) {
  if (dim != 2 && dim != 3) throw Error(MUSG_ERR_ARGUMENT, "only 2- and 3-dimensional grids are supported");
  if (!resolutions || !in_device || !out_device) throw Error(MUSG_ERR_ARGUMENT, "null argument");
  if (kind < 0 || kind > 2) throw Error(MUSG_ERR_ARGUMENT, "unknown projection kind");
  const bool allow_even = (flags & MUSG_FLAG_ALLOW_EVEN) != 0;
  for (int d = 0; d < dim; ++d) {
    if (resolutions[d] < 1) throw Error(MUSG_ERR_ARGUMENT, "resolutions must be positive");
    if (!allow_even && resolutions[d] % 2 == 0)
      throw Error(MUSG_ERR_PROJECTION, "Only an odd number of gridpoints in each direction is supported");
  }
  // the workspace is described in place: plans and views into the static array,
  // no allocation (Spectral::init is not used; nothing here is ever released)
  Spectral sp;
  sp.g.dim = dim;
  sp.g.npx = 1;
  for (int d = 0; d < dim; ++d) {
    sp.g.n[d] = resolutions[d];
    sp.g.npx *= resolutions[d];
    sp.lengths[d] = lengths ? lengths[d] : 1.0;
  }
  sp.g.nh = sp.g.n[dim - 1] / 2 + 1;
  sp.g.nrows = sp.g.npx / sp.g.n[dim - 1];
  sp.g.nk = sp.g.nrows * sp.g.nh;
  sp.ncomp = dim * dim;
  sp.proj_kind = kind;
  sp.allow_even = allow_even;
  const long long nb_dof = sp.g.npx * sp.ncomp;
  // the field copy and the half spectrum alone bound every axis length well below
  // what the FFT plans can factorise, so reject oversized grids before planning
  const double need0 = (double)nb_dof * sizeof(double) + (double)sp.ncomp * (double)sp.g.nk * sizeof(double2);
  if (need0 > (double)kNoAllocScratchBytes)
    throw Error(MUSG_ERR_ARGUMENT, "grid too large for the allocation-free projection: its field copy and half "
                                   "spectrum alone need " + std::to_string((long long)need0) +
                                       " bytes of scratch, the maximum is " + std::to_string(kNoAllocScratchBytes) +
                                       " (64 MiB)");

  // layout of the array: [field planes][half spectrum][per axis: tw, chirp, bf, xi]
  size_t off = 0;
  const size_t off_soa = off;
  off += align256((size_t)nb_dof * sizeof(double));
  const size_t off_spec = off;
  off += align256((size_t)sp.ncomp * sp.g.nk * sizeof(double2));
  size_t off_tw[3], off_chirp[3], off_bf[3], off_xi[3];
  for (int d = 0; d < dim; ++d) {
    AxisPlan &ap = sp.ax[d];
    ap.n = sp.g.n[d];
    if (factor_fixed(ap.n, ap.radix, ap.nst)) {
      ap.blu = 0;
      ap.m = ap.n;
    } else {
      ap.blu = 1;
      ap.m = smooth_ge(2 * ap.n - 1);
      if (!factor_fixed(ap.m, ap.radix, ap.nst)) throw Error(MUSG_ERR_ARGUMENT, "FFT length too large");
    }
    off_tw[d] = off;
    off += align256((size_t)ap.m * sizeof(double2));
    off_chirp[d] = off;
    off += ap.blu ? align256((size_t)ap.n * sizeof(double2)) : 0;
    off_bf[d] = off;
    off += ap.blu ? align256((size_t)ap.m * sizeof(double2)) : 0;
    off_xi[d] = off;
    off += align256((size_t)((d == dim - 1) ? sp.g.nh : sp.g.n[d]) * sizeof(double));
  }
  if (off > kNoAllocScratchBytes)
    throw Error(MUSG_ERR_ARGUMENT, "grid too large for the allocation-free projection: it needs " + std::to_string(off) +
                                       " bytes of scratch, the maximum is " + std::to_string(kNoAllocScratchBytes) +
                                       " (64 MiB)");

  unsigned char *base = static_cast<unsigned char *>(scratch_address());
  double *soa = reinterpret_cast<double *>(base + off_soa);
  sp.spec64 = base + off_spec;
  for (int d = 0; d < dim; ++d) {
    AxisPlan &ap = sp.ax[d];
    ap.tw64 = base + off_tw[d];
    ap.chirp64 = ap.blu ? base + off_chirp[d] : nullptr;
    ap.bf64 = ap.blu ? base + off_bf[d] : nullptr;
    sp.xi64[d] = base + off_xi[d];
    const int len = (d == dim - 1) ? sp.g.nh : sp.g.n[d];
    const int work = std::max(ap.m, std::max(ap.n, len));
    k_fill_axis<<<(work + 255) / 256, 256, 0, s>>>((double2 *)ap.tw64, ap.m, (double2 *)ap.chirp64, ap.n,
                                                   (double *)sp.xi64[d], len, sp.lengths[d]);
    MUSG_CHECK_LAUNCH();
    if (ap.blu) {
      k_fill_bluestein<<<(ap.m + 127) / 128, 128, 0, s>>>((const double2 *)ap.chirp64, ap.n, (double2 *)ap.bf64,
                                                          ap.m);
      MUSG_CHECK_LAUNCH();
    }
  }
  aos_to_soa(in_device, soa, sp.ncomp, sp.g.npx, s);
  spectral_project<double>(sp, soa, soa, 1.0, s);
  soa_to_aos(soa, out_device, sp.ncomp, sp.g.npx, s);
}

}  // namespace musg
