// Host side of the FFT plans and spectral workspaces.
//
// Twiddles are computed in long double from their definition exp(-2 pi i j/m)
// and rounded once to double and to float; the Bluestein filter DFT_m(conj w)/m is
// formed on the host by a direct DFT with compensated (Kahan) summation.
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <vector>

#include "musg_internal.h"

namespace musg {

std::atomic<unsigned long long> g_launches{0};

void DevBuf::alloc(size_t b) {
  release();
  if (b == 0) return;
  MUSG_CUDA(cudaMalloc(&p, b));
  bytes = b;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

namespace {

// radices of a 2/3/5/7-smooth length; returns false when another prime divides n
bool factorize(int n, std::vector<int> &out) {
  out.clear();
  int k = 0;
  while (n % 2 == 0) { n /= 2; ++k; }
  // powers of two: radix 16 as long as possible, the remainder as balanced 8/4
  while (k > 0) {
    if (k >= 4 && k != 5 && k != 6) { out.push_back(16); k -= 4; }
    else if (k == 6) { out.push_back(8); out.push_back(8); k = 0; }
    else if (k == 5) { out.push_back(8); out.push_back(4); k = 0; }
    else if (k == 3) { out.push_back(8); k = 0; }
    else if (k == 2) { out.push_back(4); k = 0; }
    else { out.push_back(2); k = 0; }
  }
  while (n % 9 == 0) { out.push_back(9); n /= 9; }
  for (int r : {3, 5, 7})
    while (n % r == 0) { out.push_back(r); n /= r; }
  return n == 1;
}

int smooth_at_least(int v) {
  for (int m = v;; ++m) {
    int t = m;
    for (int r : {2, 3, 5, 7})
      while (t % r == 0) t /= r;
    if (t == 1) return m;
  }
}

const long double kPi = 3.141592653589793238462643383279502884L;

void *upload(const void *host, size_t bytes) {
  void *d = nullptr;
  MUSG_CUDA(cudaMalloc(&d, bytes));
  MUSG_CUDA(cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice));
  return d;
}

template <typename T2, typename R>
void *upload_complex(const std::vector<std::complex<long double>> &v) {
  std::vector<T2> h(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    h[i].x = static_cast<R>(v[i].real());
    h[i].y = static_cast<R>(v[i].imag());
  }
  return upload(h.data(), h.size() * sizeof(T2));
}

}  // namespace

void AxisPlan::build(int n_) {
  release();
  n = n_;
  std::vector<int> rad;
  if (factorize(n, rad)) {
    blu = 0;
    m = n;
  } else {
    blu = 1;
    if (n > (1 << 28)) throw Error(MUSG_ERR_ARGUMENT, "FFT length too large");
    m = smooth_at_least(2 * n - 1);
    factorize(m, rad);
  }
  if ((int)rad.size() > kMaxStages) throw Error(MUSG_ERR_ARGUMENT, "FFT length too large");
  nst = (int)rad.size();
  for (int s = 0; s < nst; ++s) radix[s] = rad[s];

  std::vector<std::complex<long double>> tw(m);
  for (int j = 0; j < m; ++j) {
    long double a = -2.0L * kPi * (long double)j / (long double)m;
    tw[j] = {cosl(a), sinl(a)};
  }
  tw64 = upload_complex<double2, double>(tw);
  tw32 = upload_complex<float2, float>(tw);
  if (blu) {
    std::vector<std::complex<long double>> w(n);
    for (int j = 0; j < n; ++j) {
      long long q = ((long long)j * j) % (2LL * n);
      long double a = -kPi * (long double)q / (long double)n;
      w[j] = {cosl(a), sinl(a)};
    }
    // b[t] = conj(w[|t|]) on the circle of length m
    std::vector<std::complex<double>> b(m, {0.0, 0.0});
    for (int t = 0; t < n; ++t) b[t] = std::conj(std::complex<double>((double)w[t].real(), (double)w[t].imag()));
    for (int t = 1; t < n; ++t) b[m - t] = b[t];
    std::vector<std::complex<long double>> bf(m);
    std::vector<std::complex<double>> twd(m);
    for (int j = 0; j < m; ++j) twd[j] = {(double)tw[j].real(), (double)tw[j].imag()};
    for (int k = 0; k < m; ++k) {
      // Kahan-compensated sum_t b[t] exp(-2 pi i t k / m)
      double sr = 0, sc = 0, ir = 0, ic = 0;
      long long idx = 0;
      for (int t = 0; t < m; ++t) {
        if (b[t].real() != 0.0 || b[t].imag() != 0.0) {
          std::complex<double> term = b[t] * twd[idx];
          double y = term.real() - sc;
          double tt = sr + y;
          sc = (tt - sr) - y;
          sr = tt;
          y = term.imag() - ic;
          tt = ir + y;
          ic = (tt - ir) - y;
          ir = tt;
        }
        idx += k;
        if (idx >= m) idx -= m;
      }
      bf[k] = {(long double)sr / m, (long double)ir / m};
    }
    chirp64 = upload_complex<double2, double>(w);
    chirp32 = upload_complex<float2, float>(w);
    bf64 = upload_complex<double2, double>(bf);
    bf32 = upload_complex<float2, float>(bf);
  }
}

void AxisPlan::release() {
  for (void **p : {&tw64, &chirp64, &bf64, &tw32, &chirp32, &bf32}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
}

template <> AxisPlanD<double> AxisPlan::device<double>() const {
  AxisPlanD<double> d{};
  d.n = n; d.m = m; d.nst = nst; d.blu = blu;
  d.rcode = 0;
  for (int s = 0; s < nst; ++s) d.rcode |= (unsigned long long)radix[s] << (5 * s);
  d.tw = (const double2 *)tw64;
  d.chirp = (const double2 *)chirp64;
  d.bf = (const double2 *)bf64;
  return d;
}

template <> AxisPlanD<float> AxisPlan::device<float>() const {
  AxisPlanD<float> d{};
  d.n = n; d.m = m; d.nst = nst; d.blu = blu;
  d.rcode = 0;
  for (int s = 0; s < nst; ++s) d.rcode |= (unsigned long long)radix[s] << (5 * s);
  d.tw = (const float2 *)tw32;
  d.chirp = (const float2 *)chirp32;
  d.bf = (const float2 *)bf32;
  return d;
}

// fftfreq(n)[k]/L (src/fft/fft_utils.cc:41-56)
static double fft_freq(int n, int k) {
  int N = (n - 1) / 2 + 1;
  return k < N ? (double)k : (double)(-(n / 2) + k - N);
}

void Spectral::init(int dim, const int *res, int ncomp_, int proj_kind_, const double *lengths_,
                    bool allow_even_, bool want32_) {
  release();
  if (dim != 2 && dim != 3) throw Error(MUSG_ERR_ARGUMENT, "only 2- and 3-dimensional grids are supported");
  g.dim = dim;
  g.npx = 1;
  for (int d = 0; d < 3; ++d) g.n[d] = 1;
  for (int d = 0; d < dim; ++d) {
    if (res[d] < 1) throw Error(MUSG_ERR_ARGUMENT, "resolutions must be positive");
    g.n[d] = res[d];
    g.npx *= res[d];
    lengths[d] = lengths_ ? lengths_[d] : 1.0;
  }
  g.nh = g.n[dim - 1] / 2 + 1;
  g.nrows = g.npx / g.n[dim - 1];
  g.nk = g.nrows * g.nh;
  ncomp = ncomp_;
  proj_kind = proj_kind_;
  allow_even = allow_even_;
  want32 = want32_;
  for (int d = 0; d < dim; ++d) ax[d].build(g.n[d]);
  // xi tables over the hermitian index range of each axis
  for (int d = 0; d < dim; ++d) {
    int len = (d == dim - 1) ? g.nh : g.n[d];
    std::vector<double> h(len);
    std::vector<float> hf(len);
    for (int k = 0; k < len; ++k) {
      h[k] = fft_freq(g.n[d], k) / lengths[d];
      hf[k] = (float)h[k];
    }
    xi64[d] = upload(h.data(), len * sizeof(double));
    xi32[d] = upload(hf.data(), len * sizeof(float));
  }
  MUSG_CUDA(cudaMalloc(&spec64, (size_t)ncomp * g.nk * sizeof(double2)));
  if (want32) ensure32();
}

void Spectral::ensure32() {
  want32 = true;
  if (!spec32) MUSG_CUDA(cudaMalloc(&spec32, (size_t)ncomp * g.nk * sizeof(float2)));
}

void Spectral::release() {
  for (auto &a : ax) a.release();
  for (int d = 0; d < 3; ++d) {
    if (xi64[d]) cudaFree(xi64[d]);
    if (xi32[d]) cudaFree(xi32[d]);
    xi64[d] = xi32[d] = nullptr;
  }
  if (spec64) cudaFree(spec64);
  if (spec32) cudaFree(spec32);
  spec64 = spec32 = nullptr;
}

}  // namespace musg
