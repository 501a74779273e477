// Per-pixel constitutive evaluation (FP64), the device counterpart of
// MaterialMuSpectre::compute_stresses_worker (src/materials/material_muSpectre_base.hh:292-401)
// for MaterialLinearElastic1-4 and MaterialHyperElastoPlastic1.
//
// One thread per pixel reads F from component planes, looks its material up in a
// small parameter table (uint8 material index per pixel) and writes P plus what the
// CG operator needs to apply the tangent (S and F for the finite-strain elastic laws,
// the j-independent Kirchhoff tangent K' for HyperElastoPlastic1), in the CG
// precision.  A full D^4 tangent is written only when the API asks for it.
#include <cmath>

#include "musg_internal.h"

namespace musg {

namespace {

constexpr int kMatThreads = 128;

template <int D> struct M {
  double a[D * D];  // column-major: (i, j) at i + D*j
  __device__ __forceinline__ double &operator()(int i, int j) { return a[i + D * j]; }
  __device__ __forceinline__ double operator()(int i, int j) const { return a[i + D * j]; }
};

template <int D> __device__ __forceinline__ M<D> mul(const M<D> &A, const M<D> &B) {
  M<D> C;
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) v += A(i, k) * B(k, j);
      C(i, j) = v;
    }
  return C;
}

template <int D> __device__ __forceinline__ M<D> mul_bt(const M<D> &A, const M<D> &B) {  // A B^T
  M<D> C;
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) v += A(i, k) * B(j, k);
      C(i, j) = v;
    }
  return C;
}

template <int D> __device__ __forceinline__ double trace(const M<D> &A) {
  double t = 0.0;
#pragma unroll
  for (int i = 0; i < D; ++i) t += A(i, i);
  return t;
}

// inverse by cofactors (closed form, as Eigen's fixed-size inverse)
__device__ __forceinline__ M<2> inv(const M<2> &A) {
  M<2> R;
  const double det = A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
  R(0, 0) = A(1, 1) / det;
  R(1, 1) = A(0, 0) / det;
  R(0, 1) = -A(0, 1) / det;
  R(1, 0) = -A(1, 0) / det;
  return R;
}
__device__ __forceinline__ M<3> inv(const M<3> &A) {
  M<3> C;
  C(0, 0) = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
  C(0, 1) = A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2);
  C(0, 2) = A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1);
  C(1, 0) = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
  C(1, 1) = A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0);
  C(1, 2) = A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2);
  C(2, 0) = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
  C(2, 1) = A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1);
  C(2, 2) = A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
  const double det = A(0, 0) * C(0, 0) + A(0, 1) * C(1, 0) + A(0, 2) * C(2, 0);
#pragma unroll
  for (int k = 0; k < 9; ++k) C.a[k] /= det;
  return C;
}

// Cyclic Jacobi eigen-decomposition of a symmetric matrix (C.G.J. Jacobi 1846; the
// rotation of H. Rutishauser, "The Jacobi method for real symmetric matrices",
// Numer. Math. 9, 1966): A = V diag(w) V^T, eigenvalues sorted ascending (the
// order Eigen's SelfAdjointEigenSolver returns them in).
template <int D> __device__ __forceinline__ void sym_eig(const M<D> &A0, double *w, M<D> &V) {
  M<D> A = A0;
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) V(i, j) = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 32; ++sweep) {
    double off = 0.0, scale = 0.0;
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int i = 0; i < D; ++i) {
        if (i < j) off += A(i, j) * A(i, j);
        scale += A(i, j) * A(i, j);
      }
    if (off <= 1e-36 * scale || off == 0.0) break;
#pragma unroll
    for (int p = 0; p < D - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < D; ++q) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        // A <- J^T A J with J the rotation in the (p, q) plane
#pragma unroll
        for (int k = 0; k < D; ++k) {
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
          const double vkp = V(k, p), vkq = V(k, q);
          V(k, p) = c * vkp - s * vkq;
          V(k, q) = s * vkp + c * vkq;
        }
      }
  }
#pragma unroll
  for (int i = 0; i < D; ++i) w[i] = A(i, i);
  // sort ascending (insertion sort, swapping eigenvector columns along)
  for (int i = 1; i < D; ++i)
    for (int j = i; j > 0 && w[j] < w[j - 1]; --j) {
      const double tw = w[j];
      w[j] = w[j - 1];
      w[j - 1] = tw;
      for (int k = 0; k < D; ++k) {
        const double tv = V(k, j);
        V(k, j) = V(k, j - 1);
        V(k, j - 1) = tv;
      }
    }
}

// log(T) by the projector sum of src/common/eigen_tools.hh:209-322:
//   sum_i log(l_i) prod_{j != i, j = D-1..0} (T - l_j I)/(l_i - l_j)
template <int D> __device__ __forceinline__ M<D> logm_projector(const M<D> &T) {
  double w[D];
  M<D> V;
  sym_eig<D>(T, w, V);
  M<D> out;
#pragma unroll
  for (int k = 0; k < D * D; ++k) out.a[k] = 0.0;
#pragma unroll
  for (int i = D - 1; i >= 0; --i) {
    M<D> Pi;
    bool have = false;
#pragma unroll
    for (int j = D - 1; j >= 0; --j) {
      if (j == i) continue;
      M<D> fac;
      const double d = 1.0 / (w[i] - w[j]);
#pragma unroll
      for (int c = 0; c < D; ++c)
#pragma unroll
        for (int r = 0; r < D; ++r) fac(r, c) = d * (T(r, c) - (r == c ? w[j] : 0.0));
      Pi = have ? mul<D>(fac, Pi) : fac;
      have = true;
    }
    const double l = log(w[i]);
#pragma unroll
    for (int k = 0; k < D * D; ++k) out.a[k] += l * Pi.a[k];
  }
  return out;
}

// log(T) = V diag(log w) V^T from an eigen-decomposition T = V diag(w) V^T
template <int D> __device__ __forceinline__ M<D> log_from_eig(const double *w, const M<D> &V) {
  M<D> out;
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) v += V(i, k) * log(w[k]) * V(j, k);
      out(i, j) = v;
    }
  return out;
}

// first divided difference of log at eigenvalues a, b: (log a - log b) / (a - b), and
// 1/b at a = b; log1p keeps it accurate when a and b are close (Daleckii-Krein
// derivative of the matrix logarithm in its eigenbasis)
__device__ __forceinline__ double log_divdiff(double a, double b) {
  const double x = (a - b) / b;
  return x == 0.0 ? 1.0 / b : log1p(x) / (a - b);
}

// exp(T) = sum_i e^{w_i} v_i v_i^T  (src/common/eigen_tools.hh:329-341)
template <int D> __device__ __forceinline__ M<D> expm_sym(const M<D> &T) {
  double w[D];
  M<D> V;
  sym_eig<D>(T, w, V);
  M<D> out;
#pragma unroll
  for (int k = 0; k < D * D; ++k) out.a[k] = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double e = exp(w[k]);
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int i = 0; i < D; ++i) out(i, j) += e * V(i, k) * V(j, k);
  }
  return out;
}

template <typename R> __device__ __forceinline__ void store(R *p, long long o, double v) { p[o] = (R)v; }

// one entry (index c + D^2 q of the T4 layout) of a pixel's full tangent into the API's
// AoS array and the CG operator's planes (TK_FULL), whichever are set
__device__ __forceinline__ void put_tangent(const MaterialArgs &a, long long px, int d4, int idx, double v) {
  if (a.Kfull) a.Kfull[px * d4 + idx] = v;
  if (a.Kt64) a.Kt64[(long long)idx * a.npx + px] = v;
  if (a.Kt32) a.Kt32[(long long)idx * a.npx + px] = (float)v;
}

// HEP: the cell has MaterialHyperElastoPlastic1 pixels.  Without them the elasto-plastic
// branch (eigen-solves, logm/expm) is compiled out, which keeps the elastic laws at a
// fraction of its registers (164 with it), so more blocks are resident.
template <int D, bool HEP>
__global__ void __launch_bounds__(kMatThreads) k_material(const MaterialArgs a, int cur) {
  constexpr int D2 = D * D;
  const long long px = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (px >= a.npx) return;
  const long long N = a.npx;
  M<D> F;
#pragma unroll
  for (int c = 0; c < D2; ++c) F.a[c] = a.F[c * N + px];
  const MatParams mp = a.params[a.mat[px]];
  M<D> P;
  const bool finite = (a.form == MUSG_FINITE_STRAIN);
  if (!HEP || mp.law != MUSG_LAW_HEP1) {
    const double lam = a.lam[px], mu = a.mu[px];
    // strain measure: infinitesimal (small) or Green-Lagrange (finite)
    M<D> E;
    if (finite) {
#pragma unroll
      for (int j = 0; j < D; ++j)
#pragma unroll
        for (int i = 0; i < D; ++i) {
          double v = 0.0;
#pragma unroll
          for (int k = 0; k < D; ++k) v += F(k, i) * F(k, j);
          E(i, j) = 0.5 * (v - (i == j ? 1.0 : 0.0));
        }
    } else {
      E = F;
    }
    if (mp.law == MUSG_LAW_LE2 && a.eig) {
#pragma unroll
      for (int c = 0; c < D2; ++c) E.a[c] -= a.eig[c * N + px];
    }
    // LE1/LE2: tr(E) lam I + 2 mu E (materials_toolbox.hh:661-663);
    // LE3/LE4: C:E with C = lam Itrac + 2 mu Isymm (tensmult)
    M<D> S;
    const double tr = trace<D>(E);
    const bool tens = (mp.law == MUSG_LAW_LE3 || mp.law == MUSG_LAW_LE4);
    const bool generic = (mp.law == MUSG_LAW_GENERIC);
    const double *C = generic ? a.Ctab + (size_t)a.mat[px] * (D2 * D2) : nullptr;
    if (generic) {
      // MaterialLinearElasticGeneric: S = C:E (tensmult, material_linear_elastic_generic.hh)
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < D2; ++q) v += C[c + D2 * q] * E.a[q];
        S.a[c] = v;
      }
    } else {
#pragma unroll
      for (int j = 0; j < D; ++j)
#pragma unroll
        for (int i = 0; i < D; ++i)
          S(i, j) = (tens ? mu * (E(i, j) + E(j, i)) : 2.0 * mu * E(i, j)) + (i == j ? lam * tr : 0.0);
    }
    if (finite) {
      P = mul<D>(F, S);  // PK1 = F S (materials_toolbox.hh:313-322)
#pragma unroll
      for (int c = 0; c < D2; ++c) {
        if (a.S64) store(a.S64, c * N + px, S.a[c]);
        if (a.S32) store(a.S32, c * N + px, S.a[c]);
      }
    } else {
      P = S;
    }
    if (a.Kfull || a.Kt64 || a.Kt32) {
#pragma unroll
      for (int l = 0; l < D; ++l)
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
          for (int j = 0; j < D; ++j)
#pragma unroll
            for (int i = 0; i < D; ++i) {
              double v;
              if (generic) {
                // small strain: K = C; finite: K(i,j,k,l) = d_ik S(j,l) + sum_rs F(i,r) C(r,j,l,s) F(k,s)
                // (materials_toolbox.hh:313-350)
                if (finite) {
                  v = (i == k ? S(j, l) : 0.0);
#pragma unroll
                  for (int r = 0; r < D; ++r)
#pragma unroll
                    for (int s2 = 0; s2 < D; ++s2) v += F(i, r) * C[(r + D * j) + D2 * (l + D * s2)] * F(k, s2);
                } else {
                  v = C[(i + D * j) + D2 * (k + D * l)];
                }
              } else if (finite) {
                // K(i,j,k,l) = d_ik S(j,l) + lam F(i,j) F(k,l) + mu (F(i,l) F(k,j) + d_jl (F F^T)(i,k))
                double ffT = 0.0;
#pragma unroll
                for (int r = 0; r < D; ++r) ffT += F(i, r) * F(k, r);
                v = (i == k ? S(j, l) : 0.0) + lam * F(i, j) * F(k, l) + mu * (F(i, l) * F(k, j) + (j == l ? ffT : 0.0));
              } else {
                v = lam * (i == j && k == l ? 1.0 : 0.0) + mu * ((i == k && j == l ? 1.0 : 0.0) + (i == l && j == k ? 1.0 : 0.0));
              }
              put_tangent(a, px, D2 * D2, (i + D * j) + D2 * (k + D * l), v);
            }
    }
  } else {
    // MaterialHyperElastoPlastic1 (material_hyper_elasto_plastic1.hh:228-309)
    const int old = 1 - cur;
    M<D> Fp, be;
#pragma unroll
    for (int c = 0; c < D2; ++c) {
      Fp.a[c] = a.Fprev[old][c * N + px];
      be.a[c] = a.be[old][c * N + px];
    }
    const double eps_old = a.eps[old][px];
    const M<D> Fpi = inv(Fp);
    const M<D> f = mul<D>(F, Fpi);
    const M<D> be_star = mul_bt<D>(mul<D>(f, be), f);
    const bool consistent = mp.logm_mode == kHep1Consistent;
    double w[D];
    M<D> V;
    M<D> ln_be;
    if (mp.logm_mode == 0) {
      ln_be = logm_projector<D>(be_star);
    } else {
      sym_eig<D>(be_star, w, V);  // kept for the consistent tangent
      ln_be = log_from_eig<D>(w, V);
    }
    const double lam = mp.lam, mu = mp.mu;
    M<D> tau_star;
    const double trl = trace<D>(ln_be);
#pragma unroll
    for (int k = 0; k < D2; ++k) tau_star.a[k] = 0.5 * (2.0 * mu * ln_be.a[k]);
#pragma unroll
    for (int i = 0; i < D; ++i) tau_star(i, i) += 0.5 * trl * lam;
    M<D> tau_d = tau_star;
    const double trt = trace<D>(tau_star);
#pragma unroll
    for (int i = 0; i < D; ++i) tau_d(i, i) -= trt / D;
    double dd = 0.0;
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int i = 0; i < D; ++i) dd += tau_d(i, j) * tau_d(j, i);
    const double tau_eq = sqrt(3 * .5 * dd);
    M<D> Nst;
    // the consistent mode takes N = 0 for a deviator-free tau* (e.g. F = I), where the
    // reference's 0/0 gives NaN; N only enters multiplied by dgamma = 0 there
    const bool no_flow = consistent && !(tau_eq > 0.0);
#pragma unroll
    for (int k = 0; k < D2; ++k) Nst.a[k] = no_flow ? 0.0 : 3 * .5 * tau_d.a[k] / tau_eq;
    double phi = tau_eq - mp.tau_y0 - mp.H * eps_old;
    phi = (phi < 0.0) ? 0.0 : phi;  // std::max(phi, 0.) keeps a NaN
    const double dgamma = phi / (mp.H + 3 * mu);
    M<D> tau;
#pragma unroll
    for (int k = 0; k < D2; ++k) tau.a[k] = tau_star.a[k] - 2 * dgamma * mu * Nst.a[k];
    // state update: F_prev.current() = F; be.current() = exp(ln_be - 2 dgamma N);
    // eps_p.current() += dgamma (accumulates over evaluations, as upstream)
#pragma unroll
    for (int k = 0; k < D2; ++k) ln_be.a[k] -= 2 * dgamma * Nst.a[k];
    const M<D> be_new = expm_sym<D>(ln_be);
#pragma unroll
    for (int c = 0; c < D2; ++c) {
      a.Fprev[cur][c * N + px] = F.a[c];
      a.be[cur][c * N + px] = be_new.a[c];
    }
    // the reference adds dgamma to the current buffer's stale contents on every
    // evaluation (...plastic1.hh:262); the consistent mode writes eps_old + dgamma, so
    // that a repeated evaluation (a line-search trial) leaves the same state
    a.eps[cur][px] = consistent ? eps_old + dgamma : a.eps[cur][px] + dgamma;
    // material tangent C = alpha Itrac + beta Isymm + gamma N (x) N
    double al, bt, gm;
    if (phi > 0.0) {
      const double a0 = dgamma * mu / tau_eq;
      const double a1 = mu / (mp.H + 3 * mu);
      al = mp.K / 2. - mu / 3 + a0 * mu;
      bt = (1 - 3 * a0) * mu;
      gm = 2 * mu * (a0 - a1);
    } else {
      al = 0.5 * lam;  // C = 1/2 C_T4(lam, mu) (material_hyper_elasto_plastic1.cc:62)
      bt = mu;
      gm = 0.0;
    }
    // Kirchhoff -> PK1 (materials_toolbox.hh:374-410): P = tau F^-T,
    // K'(i,m,n) = sum_r Finv(i,r) sum_s C(r,m,n,s)
    const M<D> Fi = inv(F);
    P = mul_bt<D>(tau, Fi);
    if (consistent) {
      // The consistent tangent (opt-in; the reference converts with the j-independent
      // K' below): K(i,m,j,n) = dP(i,m)/dF(j,n) with P = tau F^-T, so
      //   dP = dtau F^-T - P dF^T F^-T,   i.e. the second term is -P(i,n) Finv(m,j);
      //   dtau = C : d ln(be*)  (C as above, the derivative of tau in ln be*);
      //   d ln(be*) = V [g o (V^T dbe* V)] V^T with g(p,q) = log_divdiff(w_p, w_q);
      //   dbe* = dF Mb + (dF Mb)^T, Mb = F_prev^-1 be_old f^T (be* = f be_old f^T, f = F F_prev^-1).
      // Column (j, n) is the response to dF = e_j e_n^T.
      const M<D> Mb = mul_bt<D>(mul<D>(Fpi, be), f);
      const M<D> MV = mul<D>(Mb, V);
      M<D> Gd, Nt;
#pragma unroll
      for (int q = 0; q < D; ++q)
#pragma unroll
        for (int p = 0; p < D; ++p) {
          Gd(p, q) = p == q ? 1.0 / w[p] : log_divdiff(w[p], w[q]);
          double v = 0.0;
#pragma unroll
          for (int b = 0; b < D; ++b)
#pragma unroll
            for (int c2 = 0; c2 < D; ++c2) v += V(b, p) * Nst(b, c2) * V(c2, q);
          Nt(p, q) = v;
        }
#pragma unroll 1
      for (int n = 0; n < D; ++n)
#pragma unroll 1
        for (int j = 0; j < D; ++j) {
          M<D> sm;
          double trs = 0.0, nsv = 0.0;
#pragma unroll
          for (int q = 0; q < D; ++q)
#pragma unroll
            for (int p = 0; p < D; ++p) {
              const double t = V(j, p) * MV(n, q) + MV(n, p) * V(j, q);
              const double sv = Gd(p, q) * t;
              sm(p, q) = sv;
              nsv += Nt(p, q) * sv;
              if (p == q) trs += sv;
            }
          const M<D> dl = mul_bt<D>(mul<D>(V, sm), V);
          M<D> dtau;
#pragma unroll
          for (int k = 0; k < D2; ++k) dtau.a[k] = bt * dl.a[k] + gm * nsv * Nst.a[k];
#pragma unroll
          for (int i = 0; i < D; ++i) dtau(i, i) += al * trs;
#pragma unroll
          for (int m = 0; m < D; ++m)
#pragma unroll
            for (int i = 0; i < D; ++i) {
              double v = -P(i, n) * Fi(m, j);
#pragma unroll
              for (int r = 0; r < D; ++r) v += dtau(i, r) * Fi(m, r);
              put_tangent(a, px, D2 * D2, (i + D * m) + D2 * (j + D * n), v);
            }
        }
    } else {
    double ns[D];
#pragma unroll
    for (int n = 0; n < D; ++n) {
      double v = 0.0;
#pragma unroll
      for (int s = 0; s < D; ++s) v += Nst(n, s);
      ns[n] = v;
    }
    double Kp[D2 * D];
#pragma unroll
    for (int n = 0; n < D; ++n)
#pragma unroll
      for (int m = 0; m < D; ++m)
#pragma unroll
        for (int i = 0; i < D; ++i) {
          double v = 0.0;
#pragma unroll
          for (int r = 0; r < D; ++r) {
            const double cs = al * (r == m ? 1.0 : 0.0) + 0.5 * bt * ((r == n ? 1.0 : 0.0) + (m == n ? 1.0 : 0.0)) +
                              gm * Nst(r, m) * ns[n];
            v += Fi(i, r) * cs;
          }
          Kp[(i + D * m) + D2 * n] = v;
        }
#pragma unroll
    for (int c = 0; c < D2 * D; ++c) {
      if (a.Kp64) store(a.Kp64, c * N + px, Kp[c]);
      if (a.Kp32) store(a.Kp32, c * N + px, Kp[c]);
    }
    if (a.Kfull || a.Kt64 || a.Kt32) {
#pragma unroll
      for (int n = 0; n < D; ++n)
#pragma unroll
        for (int j = 0; j < D; ++j)
#pragma unroll
          for (int c = 0; c < D2; ++c) put_tangent(a, px, D2 * D2, c + D2 * (j + D * n), Kp[c + D2 * n]);
    }
    }  // reference tangent
  }
  bool bad = false;
#pragma unroll
  for (int c = 0; c < D2; ++c) {
    a.P[c * N + px] = P.a[c];
    if (!isfinite(P.a[c])) bad = true;
  }
  if (bad && a.nonfinite) atomicOr(a.nonfinite, 1);
  if (finite) {
#pragma unroll
    for (int c = 0; c < D2; ++c) {
      if (a.Fc32) store(a.Fc32, c * N + px, F.a[c] - ((c % (D + 1)) == 0 ? 1.0 : 0.0));  // H = F - I
      if (a.Fc64) store(a.Fc64, c * N + px, F.a[c]);
    }
  }
}

__global__ void k_add_macro(double *F, const double *delta, int nc, long long npx) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nc * npx; i += (long long)gridDim.x * blockDim.x)
    F[i] += delta[i / npx];
}

__global__ void k_fill_uniform(double *F, const double *v, int nc, long long npx) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nc * npx; i += (long long)gridDim.x * blockDim.x)
    F[i] = v[i / npx];
}

// AoS [p][c] <-> SoA [c][p] through a shared-memory tile (coalesced both ways)
template <typename T>
__global__ void k_aos_to_soa(const T *__restrict__ aos, T *__restrict__ soa, int nc, long long npx) {
  __shared__ T tile[32 * 33];
  const long long p0 = (long long)blockIdx.x * 32;
  for (int c0 = 0; c0 < nc; c0 += 32) {
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
      const int pl = i / 32, cl = i % 32;
      const long long p = p0 + pl;
      if (p < npx && c0 + cl < nc) tile[pl * 33 + cl] = aos[p * nc + c0 + cl];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
      const int cl = i / 32, pl = i % 32;
      const long long p = p0 + pl;
      if (p < npx && c0 + cl < nc) soa[(long long)(c0 + cl) * npx + p] = tile[pl * 33 + cl];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void k_soa_to_aos(const T *__restrict__ soa, T *__restrict__ aos, int nc, long long npx) {
  __shared__ T tile[32 * 33];
  const long long p0 = (long long)blockIdx.x * 32;
  for (int c0 = 0; c0 < nc; c0 += 32) {
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
      const int cl = i / 32, pl = i % 32;
      const long long p = p0 + pl;
      if (p < npx && c0 + cl < nc) tile[pl * 33 + cl] = soa[(long long)(c0 + cl) * npx + p];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
      const int pl = i / 32, cl = i % 32;
      const long long p = p0 + pl;
      if (p < npx && c0 + cl < nc) aos[p * nc + c0 + cl] = tile[pl * 33 + cl];
    }
    __syncthreads();
  }
}

int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 65535LL * 16) b = 65535LL * 16;
  return (int)(b < 1 ? 1 : b);
}

__global__ void k_fill_lame(const uint8_t *__restrict__ mat, const MatParams *__restrict__ params, double *lam,
                            double *mu, long long npx) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx; p += (long long)gridDim.x * blockDim.x) {
    const MatParams &q = params[mat[p]];
    lam[p] = q.lam;
    mu[p] = q.mu;
  }
}

}  // namespace

void fill_lame(const uint8_t *mat, const MatParams *params, double *lam, double *mu, long long npx, cudaStream_t s) {
  k_fill_lame<<<grid_for(npx, 256), 256, 0, s>>>(mat, params, lam, mu, npx);
  MUSG_CHECK_LAUNCH();
}

void material_evaluate(const MaterialArgs &a, cudaStream_t s) {
  const int nb = (int)((a.npx + kMatThreads - 1) / kMatThreads);
  if (a.dim == 2) {
    if (a.has_hep) k_material<2, true><<<nb, kMatThreads, 0, s>>>(a, a.cur);
    else k_material<2, false><<<nb, kMatThreads, 0, s>>>(a, a.cur);
  } else {
    if (a.has_hep) k_material<3, true><<<nb, kMatThreads, 0, s>>>(a, a.cur);
    else k_material<3, false><<<nb, kMatThreads, 0, s>>>(a, a.cur);
  }
  MUSG_CHECK_LAUNCH();
}

void add_macro(double *F, const double *delta_dev, int ncomp, long long npx, cudaStream_t s) {
  k_add_macro<<<grid_for(ncomp * npx, 256), 256, 0, s>>>(F, delta_dev, ncomp, npx);
  MUSG_CHECK_LAUNCH();
}

void fill_uniform(double *F, const double *value_dev, int ncomp, long long npx, cudaStream_t s) {
  k_fill_uniform<<<grid_for(ncomp * npx, 256), 256, 0, s>>>(F, value_dev, ncomp, npx);
  MUSG_CHECK_LAUNCH();
}

void aos_to_soa(const double *aos, double *soa, int ncomp, long long npx, cudaStream_t s) {
  k_aos_to_soa<double><<<(int)((npx + 31) / 32), 256, 0, s>>>(aos, soa, ncomp, npx);
  MUSG_CHECK_LAUNCH();
}

void soa_to_aos(const double *soa, double *aos, int ncomp, long long npx, cudaStream_t s) {
  k_soa_to_aos<double><<<(int)((npx + 31) / 32), 256, 0, s>>>(soa, aos, ncomp, npx);
  MUSG_CHECK_LAUNCH();
}

void soa_to_aos_complex(const double2 *soa, double2 *aos, int ncomp, long long nk, cudaStream_t s) {
  k_soa_to_aos<double2><<<(int)((nk + 31) / 32), 256, 0, s>>>(soa, aos, ncomp, nk);
  MUSG_CHECK_LAUNCH();
}

void aos_to_soa_complex(const double2 *aos, double2 *soa, int ncomp, long long nk, cudaStream_t s) {
  k_aos_to_soa<double2><<<(int)((nk + 31) / 32), 256, 0, s>>>(aos, soa, ncomp, nk);
  MUSG_CHECK_LAUNCH();
}

}  // namespace musg
