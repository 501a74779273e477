"""CPU oracle for the µSpectre Newton-CG homogenization path (FP64, NumPy/SciPy).

TEST INFRASTRUCTURE ONLY.  This module restates, in NumPy, the algorithm of the
reference µSpectre code for the FFT-Galerkin Newton-CG loop.  Only the test suite,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import it,
and only as the checker / the timed CPU baseline.  The product (``muspectre_gb300``)
never calls it: it runs on the GPU through ``libmusg.so`` and fails loudly when that
library is missing.

Every function cites the reference file:line it follows (paths relative to the
µSpectre source tree).  Conventions of the reference that are kept here:

* Pixels are row-major, last index fastest (``src/common/ccoord_operations.hh:151-192``).
* A field vector is pixel-major (AoS): pixel ``p``, component ``i + D*j`` of a 2nd-order
  tensor ``A(i,j)`` (Eigen column-major) sits at ``p*D*D + i + D*j``.  A 4th-order
  tangent sits at ``(i + D*j) + D*D*(k + D*l)`` (``src/common/T4_map_proxy.hh:84-105``).
* Inside this module tensors are NumPy arrays indexed naturally: ``A[p, i, j]`` and
  ``K[p, i, j, k, l]``; :func:`t2_from_vec` / :func:`t2_to_vec` convert.
* All arithmetic is FP64 (``Real = double``, ``src/common/common.hh:69-70``).

Parity pinning: this restatement is checked against every known-answer test the
reference ships for this path (see ``tests/test_oracle_*.py`` and
``tests/golden/``); the reference itself cannot be compiled here (Eigen, FFTW and
Boost.Test are absent), so there is no ``oracle/_ref`` binary.

Two third-party pieces of arithmetic are restated from their published definitions:
FFTW's unnormalised r2c/c2r transforms (``numpy``/``scipy.fft`` ``rfftn``/``irfftn`` with
the same conventions) and Eigen's ``SelfAdjointEigenSolver::computeDirect`` (replaced by
LAPACK ``eigh``; eigenvalues in ascending order, as Eigen returns them).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

try:  # scipy.fft gives multithreaded pocketfft; numpy.fft is the fallback
    import scipy.fft as _sfft
except Exception:  # pragma: no cover
    _sfft = None

# ---------------------------------------------------------------------------
# enums (src/common/common.hh:142-153)
FINITE_STRAIN = 0
SMALL_STRAIN = 1

#: number of threads the FFTs of this module may use (CPU baseline raises it)
FFT_WORKERS = 1


class ProjectionError(RuntimeError):
    """src/fft/projection_base.hh (ProjectionError)."""


class SolverError(RuntimeError):
    """src/solver/solver_common.hh:80-83."""


class ConvergenceError(SolverError):
    """src/solver/solver_common.hh:86-88."""


# ---------------------------------------------------------------------------
# coordinates (src/common/ccoord_operations.hh)

def hermitian_sizes(res: Sequence[int]) -> List[int]:
    """ccoord_operations.hh:64-68 -- last axis halved to n/2+1."""
    res = list(res)
    return res[:-1] + [res[-1] // 2 + 1]


def get_ccoord(res: Sequence[int], index: int) -> List[int]:
    """ccoord_operations.hh:151-164 (row-major, last index fastest)."""
    out = [0] * len(res)
    factor = 1
    for i in range(len(res) - 1, -1, -1):
        out[i] = index // factor % res[i]
        factor *= res[i]
    return out


def get_index(res: Sequence[int], ccoord: Sequence[int]) -> int:
    """ccoord_operations.hh:179-192."""
    idx, factor = 0, 1
    for i in range(len(res) - 1, -1, -1):
        idx += ccoord[i] * factor
        factor *= res[i]
    return idx


def fft_freqs(n: int, length: float = 1.0) -> np.ndarray:
    """fft_utils.cc:41-56 -- numpy-style fftfreq(n)*n, divided by the length."""
    out = np.empty(n)
    N = (n - 1) // 2 + 1
    for i in range(N):
        out[i] = i
    for i in range(N, n):
        out[i] = -(n // 2) + i - N
    return out / length


# ---------------------------------------------------------------------------
# tensor layout helpers

def t2_from_vec(vec: np.ndarray, dim: int) -> np.ndarray:
    """flat AoS field (p*D*D + i + D*j) -> array [p, i, j]."""
    return np.ascontiguousarray(vec.reshape(-1, dim, dim).transpose(0, 2, 1))


def t2_to_vec(arr: np.ndarray) -> np.ndarray:
    """array [p, i, j] -> flat AoS field."""
    return np.ascontiguousarray(arr.transpose(0, 2, 1)).reshape(-1)


def t4_from_vec(vec: np.ndarray, dim: int) -> np.ndarray:
    """flat AoS tangent ((i+D j) + D^2 (k + D l)) -> array [p, i, j, k, l]."""
    return np.ascontiguousarray(vec.reshape(-1, dim, dim, dim, dim).transpose(0, 4, 3, 2, 1))


def t4_to_vec(arr: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(arr.transpose(0, 4, 3, 2, 1)).reshape(-1)


# ---------------------------------------------------------------------------
# materials toolbox (src/materials/materials_toolbox.hh)

def lame_lambda(E, nu):
    """materials_toolbox.hh:504-512: λ = Eν/((1+ν)(1-2ν))."""
    return E * nu / ((1 + nu) * (1 - 2 * nu))


def lame_mu(E, nu):
    """materials_toolbox.hh:491-499: μ = E/(2(1+ν))."""
    return E / (2 * (1 + nu))


def bulk_K(E, nu):
    """materials_toolbox.hh:517-525: K = E/(3(1-2ν))."""
    return E / (3 * (1 - 2 * nu))


def young_from_K_mu(K, mu):
    """materials_toolbox.hh (Converter<Young, Bulk, Shear>): 9KG/(3K+G)."""
    return 9 * K * mu / (3 * K + mu)


def poisson_from_K_mu(K, mu):
    """materials_toolbox.hh (Converter<Poisson, Bulk, Shear>): (3K-2G)/(2(3K+G))."""
    return (3 * K - 2 * mu) / (2 * (3 * K + mu))


def itrac(dim):
    """tensor_algebra.hh:262-266: outer(I, I), I_ijkl = δij δkl."""
    I = np.eye(dim)
    return np.einsum('ij,kl->ijkl', I, I)


def isymm(dim):
    """tensor_algebra.hh:283-287: ½(outer_under(I,I) + outer_over(I,I))."""
    I = np.eye(dim)
    return 0.5 * (np.einsum('ik,jl->ijkl', I, I) + np.einsum('il,jk->ijkl', I, I))


def hooke_C(lam, mu, dim):
    """materials_toolbox.hh:638-652: C = λ Itrac + 2μ Isymm.  lam/mu may be arrays
    (one per pixel); the result then has a leading pixel axis."""
    lam = np.asarray(lam, dtype=float)
    mu = np.asarray(mu, dtype=float)
    return lam[..., None, None, None, None] * itrac(dim) + 2 * mu[..., None, None, None, None] * isymm(dim)


def hooke_stress(lam, mu, E):
    """materials_toolbox.hh:661-663: S = tr(E) λ I + 2μ E  (E: [p, i, j])."""
    dim = E.shape[-1]
    lam = np.asarray(lam, dtype=float).reshape(-1, 1, 1)
    mu = np.asarray(mu, dtype=float).reshape(-1, 1, 1)
    tr = np.trace(E, axis1=-2, axis2=-1)[:, None, None]
    return tr * lam * np.eye(dim) + 2 * mu * E


def green_lagrange(F):
    """materials_toolbox.hh:139-148: E = ½(FᵀF - I)."""
    dim = F.shape[-1]
    return 0.5 * (np.einsum('pki,pkj->pij', F, F) - np.eye(dim))


def tensmult(K, dF):
    """tensor_algebra.hh:234-259: dp(i,j) = Σ_kl K(i,j,k,l) df(k,l)."""
    return np.einsum('pijkl,pkl->pij', K, dF)


def pk1_from_pk2(F, S, C):
    """materials_toolbox.hh:313-350 (PK1_stress<PK2, GreenLagrange>):
    P = F S,  K(i,m,j,n) = δij S(m,n) + Σ_rs F(i,r) C(r,m,n,s) F(j,s)."""
    dim = F.shape[-1]
    I = np.eye(dim)
    if C.ndim == 4:
        K = np.einsum('pir,rmns,pjs->pimjn', F, C, F, optimize=True)
    else:
        K = np.einsum('pir,prmns,pjs->pimjn', F, C, F, optimize=True)
    K = K + np.einsum('ij,pmn->pimjn', I, S)
    P = np.einsum('pij,pjk->pik', F, S)
    return P, K


def pk1_from_kirchhoff(F, tau, C):
    """materials_toolbox.hh:374-410 (PK1_stress<Kirchhoff, Gradient>), as written:
    P = τ F⁻ᵀ,  K(i,m,j,n) = Σ_r F⁻¹(i,r) Σ_s C(r,m,n,s)   (independent of j)."""
    dim = F.shape[-1]
    Finv = np.linalg.inv(F)
    if C.ndim == 4:
        Cs = C.sum(axis=3)[None]  # Σ_s C(r,m,n,s)
    else:
        Cs = C.sum(axis=4)
    Kp = np.einsum('pir,prmn->pimn', Finv, Cs)  # K'(i,m,n)
    K = np.broadcast_to(Kp[:, :, :, None, :], (F.shape[0], dim, dim, dim, dim)).copy()
    P = np.einsum('pij,pkj->pik', tau, Finv)
    return P, K


# ---------------------------------------------------------------------------
# matrix functions (src/common/eigen_tools.hh:209-341)

def logm_projector(T):
    """eigen_tools.hh:209-322: log(T) = Σ_i log(λ_i) Π_{j≠i} (T - λ_j I)/(λ_i - λ_j),
    product taken for j = D-1 down to 0 (Proj<dim,i,j> recursion).  Eigenvalues in
    ascending order (Eigen computeDirect; here LAPACK eigh).  Repeated eigenvalues give
    non-finite entries, exactly like the formula in the reference."""
    dim = T.shape[-1]
    eigs = np.linalg.eigvalsh(T)
    I = np.eye(dim)
    out = np.zeros_like(T)
    with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
        for i in range(dim - 1, -1, -1):
            Pi = None
            for j in range(dim - 1, -1, -1):
                if j == i:
                    continue
                fac = (1.0 / (eigs[:, i] - eigs[:, j]))[:, None, None] * (T - eigs[:, j][:, None, None] * I)
                Pi = fac if Pi is None else np.einsum('pij,pjk->pik', fac, Pi)
            if Pi is None:
                Pi = np.broadcast_to(I, T.shape)
            out = out + np.log(eigs[:, i])[:, None, None] * Pi
    return out


def logm_spectral(T):
    """log(T) = V diag(log λ) Vᵀ (well defined for repeated eigenvalues)."""
    w, V = np.linalg.eigh(T)
    return np.einsum('pik,pk,pjk->pij', V, np.log(w), V)


def expm_sym(T):
    """eigen_tools.hh:329-341: exp(T) = Σ_i e^{λ_i} v_i v_iᵀ (symmetric T)."""
    w, V = np.linalg.eigh(T)
    return np.einsum('pik,pk,pjk->pij', V, np.exp(w), V)


# ---------------------------------------------------------------------------
# materials

class Material:
    """MaterialBase (src/materials/material_base.hh:53-168): a name and a pixel list."""

    law = ''

    def __init__(self, name: str, dim: int):
        self.name = name
        self.dim = dim
        self.pixels: List[int] = []

    def size(self):
        return len(self.pixels)

    def initialise(self):
        pass

    def save_history_variables(self):
        pass

    def evaluate(self, F, form):
        raise NotImplementedError


class MaterialLinearElastic1(Material):
    """material_linear_elastic1.{hh,cc}: GL strain / PK2 stress, constant λ, μ
    (ctor .cc:40-48; law .hh:166-194)."""

    law = 'le1'

    def __init__(self, name, dim, young, poisson):
        super().__init__(name, dim)
        self.young, self.poisson = young, poisson
        self.lam = lame_lambda(young, poisson)
        self.mu = lame_mu(young, poisson)
        self.C = hooke_C(self.lam, self.mu, dim)

    def add_pixel(self, index):
        self.pixels.append(int(index))

    def _lam_mu(self, n):
        return np.full(n, self.lam), np.full(n, self.mu)

    def _strain_shift(self, n):
        return None

    def evaluate(self, F, form):
        """material_muSpectre_base.hh:292-401 (compute_stresses_worker)."""
        n = F.shape[0]
        lam, mu = self._lam_mu(n)
        C = hooke_C(lam, mu, self.dim)
        shift = self._strain_shift(n)
        # LE1/LE2 evaluate Hooke's law directly (…1.hh:166-194); LE3/LE4 contract the
        # stiffness tensor (…3.hh:186-187, …4.hh:190-210)
        law = (lambda E_: tensmult(C, E_)) if self.law in ('le3', 'le4') else (lambda E_: hooke_stress(lam, mu, E_))
        if form == SMALL_STRAIN:
            eps = F if shift is None else F - shift
            return law(eps), C.copy()
        E = green_lagrange(F)
        if shift is not None:
            E = E - shift
        return pk1_from_pk2(F, law(E), C)


# Voigt index map of voigt_conversion.hh:118-125 (sym_mat)
VOIGT_SYM = {2: np.array([[0, 2], [2, 1]]), 3: np.array([[0, 5, 4], [5, 1, 3], [4, 3, 2]])}


def stiffness_from_voigt(C_voigt, dim):
    """material_linear_elastic_generic.cc:40-66: C(i,j,k,l) = C_voigt(sym(i,j), sym(k,l))."""
    Cv = np.asarray(C_voigt, dtype=float)
    vs = 3 if dim == 2 else 6
    if Cv.shape != (vs, vs):
        raise RuntimeError("The stiffness tensor should be input as a %d × %d Matrix in Voigt notation. "
                           "You supplied a %d × %d matrix" % (vs, vs, Cv.shape[0], Cv.shape[1]))
    s = VOIGT_SYM[dim]
    return Cv[s[:, :, None, None], s[None, None, :, :]]


class MaterialLinearElasticGeneric(Material):
    """material_linear_elastic_generic.{hh,cc}: GL strain / PK2 stress with a constant
    stiffness tensor given in Voigt notation; S = C:E (tensmult), tangent C."""

    law = 'generic'

    def __init__(self, name, dim, C_voigt):
        super().__init__(name, dim)
        self.C = stiffness_from_voigt(C_voigt, dim)

    def add_pixel(self, index):
        self.pixels.append(int(index))

    def evaluate(self, F, form):
        n = F.shape[0]
        C = np.broadcast_to(self.C, (n,) + self.C.shape).copy()
        if form == SMALL_STRAIN:
            return tensmult(C, F), C
        return pk1_from_pk2(F, tensmult(C, green_lagrange(F)), C)


class MaterialLinearElastic2(MaterialLinearElastic1):
    """material_linear_elastic2.{hh,cc}: LE1 applied to (E - E_eig), per-pixel
    eigenstrain (add_pixel .cc:57-64; law .hh:179-201)."""

    law = 'le2'

    def __init__(self, name, dim, young, poisson):
        super().__init__(name, dim, young, poisson)
        self.eig: List[np.ndarray] = []

    def add_pixel(self, index, eigenstrain=None):
        if eigenstrain is None:
            raise RuntimeError("this material needs pixels with and eigenstrain")
        self.pixels.append(int(index))
        self.eig.append(np.array(eigenstrain, dtype=float).reshape(self.dim, self.dim))

    def _strain_shift(self, n):
        return np.array(self.eig).reshape(n, self.dim, self.dim)


class MaterialLinearElastic3(MaterialLinearElastic1):
    """material_linear_elastic3.{hh,cc}: per-pixel stiffness C built from (E, ν)
    (add_pixel .cc:58-68); stress = C:E (tensmult)."""

    law = 'le3'

    def __init__(self, name, dim):
        Material.__init__(self, name, dim)
        self.E: List[float] = []
        self.nu: List[float] = []

    def add_pixel(self, index, young=None, poisson=None):
        if young is None or poisson is None:
            raise RuntimeError("this material needs pixels with Youngs modulus and Poisson ratio.")
        self.pixels.append(int(index))
        self.E.append(float(young))
        self.nu.append(float(poisson))

    def _lam_mu(self, n):
        E, nu = np.array(self.E), np.array(self.nu)
        return lame_lambda(E, nu), lame_mu(E, nu)


class MaterialLinearElastic4(MaterialLinearElastic3):
    """material_linear_elastic4.{hh,cc}: per-pixel λ, μ stored as scalar fields
    (add_pixel .cc:63-73; law .hh:190-210, C = compute_C_T4(λ, μ), σ = C:E)."""

    law = 'le4'


class MaterialHyperElastoPlastic1(Material):
    """material_hyper_elasto_plastic1.{hh,cc}: finite-strain J2 plasticity after
    Geers 2003, Kirchhoff stress w.r.t. the placement gradient.

    State fields (statefield.hh:322-326): each of F_prev, be_prev, eps_p holds two
    buffers; ``current`` is buffer ``idx`` and ``old`` is buffer ``1-idx``;
    ``cycle()`` only swaps the index.  ``eps_p.current() += Δγ`` runs on every
    evaluation (…plastic1.hh:262), so it accumulates on top of stale contents, as in
    the reference.
    """

    law = 'hep1'

    def __init__(self, name, dim, young, poisson, tau_y0, H, logm_mode='projector', tangent='reference'):
        super().__init__(name, dim)
        self.young, self.poisson = young, poisson
        self.lam = lame_lambda(young, poisson)
        self.mu = lame_mu(young, poisson)
        self.K = bulk_K(young, poisson)
        self.tau_y0, self.H = tau_y0, H
        # .cc:62: C = ½ C_T4(λ, μ) (Geers 2003 eq. 18)
        self.C = 0.5 * hooke_C(self.lam, self.mu, dim)
        if tangent not in ('reference', 'consistent'):
            raise ValueError(tangent)
        # the consistent tangent (an extension, see evaluate_consistent) needs the spectral logm
        self.tangent = tangent
        self.logm_mode = 'spectral' if tangent == 'consistent' else logm_mode
        self._idx = 0
        self.F_prev = self.be_prev = self.eps_p = None

    def add_pixel(self, index):
        self.pixels.append(int(index))

    def initialise(self):
        """.cc:76-84: zero-initialised local fields; current(F_prev)=current(be)=I; cycle."""
        n, d = len(self.pixels), self.dim
        self.F_prev = np.zeros((2, n, d, d))
        self.be_prev = np.zeros((2, n, d, d))
        self.eps_p = np.zeros((2, n))
        self.F_prev[self._idx][:] = np.eye(d)
        self.be_prev[self._idx][:] = np.eye(d)
        self.save_history_variables()

    def save_history_variables(self):
        """.cc:68-73 -> StateField::cycle (index rotation, no copy)."""
        self._idx = 1 - self._idx

    # current/old accessors
    def _cur(self, f):
        return f[self._idx]

    def _old(self, f):
        return f[1 - self._idx]

    def stress_n_internals(self, F):
        """…plastic1.hh:228-271."""
        d = self.dim
        I = np.eye(d)
        with np.errstate(divide='ignore', invalid='ignore', over='ignore'):
            f = np.einsum('pij,pjk->pik', F, np.linalg.inv(self._old(self.F_prev)))
            be_star = np.einsum('pij,pjk,plk->pil', f, self._old(self.be_prev), f)
            if self.logm_mode == 'projector':
                ln_be = logm_projector(be_star)
            else:
                ln_be = logm_spectral(be_star)
            tau_star = 0.5 * hooke_stress(np.full(F.shape[0], self.lam), np.full(F.shape[0], self.mu), ln_be)
            tr = np.trace(tau_star, axis1=1, axis2=2)
            tau_d = tau_star - (tr / d)[:, None, None] * I
            tau_eq = np.sqrt(3 * 0.5 * np.einsum('pij,pji->p', tau_d, tau_d))
            N = 3 * 0.5 * tau_d / tau_eq[:, None, None]
            if self.tangent == 'consistent':
                # a deviator-free Kirchhoff stress (e.g. F = I) has no flow direction; the
                # consistent mode takes N = 0 there (N only enters multiplied by Δγ = 0 or
                # the plastic-only tangent term), where the reference's 0/0 gives NaN
                N = np.where((tau_eq > 0)[:, None, None], N, 0.0)
            phi = np.maximum(tau_eq - self.tau_y0 - self.H * self._old(self.eps_p), 0.0)
            phi = np.where(np.isnan(tau_eq), np.nan, phi)  # std::max(NaN, 0) keeps NaN
            dgamma = phi / (self.H + 3 * self.mu)
            tau = tau_star - 2 * (dgamma * self.mu)[:, None, None] * N
            self._cur(self.F_prev)[:] = F
            ln_be = ln_be - 2 * dgamma[:, None, None] * N
            self._cur(self.be_prev)[:] = expm_sym(ln_be) if np.all(np.isfinite(ln_be)) else _expm_guard(ln_be)
            if self.tangent == 'consistent':
                # the consistent mode writes εp.cur = εp.old + Δγ (every evaluation, so a
                # repeated evaluation leaves the same state); the reference adds Δγ to the
                # current buffer's stale contents (…plastic1.hh:262), kept in the other modes
                self._cur(self.eps_p)[:] = self._old(self.eps_p) + dgamma
            else:
                self._cur(self.eps_p)[:] += dgamma
        is_plastic = phi > 0
        return tau, tau_eq, dgamma, N, is_plastic

    def evaluate_stress_tangent_kirchhoff(self, F):
        """…plastic1.hh:284-309: Kirchhoff stress and its tangent."""
        d = self.dim
        tau, tau_eq, dgamma, N, plastic = self.stress_n_internals(F)
        n = F.shape[0]
        C = np.broadcast_to(self.C, (n, d, d, d, d)).copy()
        if np.any(plastic):
            with np.errstate(divide='ignore', invalid='ignore'):
                a0 = dgamma * self.mu / tau_eq
            a1 = self.mu / (self.H + 3 * self.mu)
            Cp = ((self.K / 2. - self.mu / 3 + a0 * self.mu)[:, None, None, None, None] * itrac(d)
                  + ((1 - 3 * a0) * self.mu)[:, None, None, None, None] * isymm(d)
                  + (2 * self.mu * (a0 - a1))[:, None, None, None, None] * np.einsum('pij,pkl->pijkl', N, N))
            C[plastic] = Cp[plastic]
        return tau, C

    def evaluate(self, F, form):
        if form != FINITE_STRAIN:
            raise RuntimeError("MaterialHyperElastoPlastic1 needs the finite-strain formulation")
        if self.tangent == 'consistent':
            return self.evaluate_consistent(F)
        tau, C = self.evaluate_stress_tangent_kirchhoff(F)
        return pk1_from_kirchhoff(F, tau, C)

    def evaluate_consistent(self, F):
        """Stress as in stress_n_internals (…plastic1.hh:228-271, spectral logm) and the
        consistent tangent K(i,m,j,n) = dP(i,m)/dF(j,n) of P = τ F⁻ᵀ -- an extension: the
        reference converts with the j-independent K' of materials_toolbox.hh:374-410.

        With f = F F_prev⁻¹, be* = f be_old fᵀ = V diag(w) Vᵀ and the Kirchhoff tangent
        C = α Itrac + β Isymm + γ N⊗N of …plastic1.hh:294-308 (the derivative of τ in
        ln be*):
          dbe*     = dF Mb + (dF Mb)ᵀ,  Mb = F_prev⁻¹ be_old fᵀ
          d ln be* = V [g ∘ (Vᵀ dbe* V)] Vᵀ,  g(p,q) = (ln w_p - ln w_q)/(w_p - w_q), 1/w_p at p = q
                     (the Daleckii-Krein formula for the derivative of the matrix logarithm)
          dτ       = C : d ln be*
          dP       = dτ F⁻ᵀ - P dFᵀ F⁻ᵀ
        Column (j, n) of K is dP for dF = e_j e_nᵀ."""
        d = self.dim
        n = F.shape[0]
        Fp = self._old(self.F_prev).copy()
        be_old = self._old(self.be_prev).copy()
        tau, tau_eq, dgamma, N, plastic = self.stress_n_internals(F)
        Fpi = np.linalg.inv(Fp)
        f = np.einsum('pij,pjk->pik', F, Fpi)
        be_star = np.einsum('pij,pjk,plk->pil', f, be_old, f)
        w, V = np.linalg.eigh(be_star)
        Mb = np.einsum('pij,pjk,plk->pil', Fpi, be_old, f)
        MV = np.einsum('pij,pjk->pik', Mb, V)
        a_, b_ = w[:, :, None], w[:, None, :]
        with np.errstate(divide='ignore', invalid='ignore'):
            x = (a_ - b_) / b_
            g = np.where(x == 0, 1.0 / b_, np.log1p(x) / (a_ - b_))
        idx = np.arange(d)
        g[:, idx, idx] = 1.0 / w
        Nt = np.einsum('pbi,pbc,pcj->pij', V, N, V)
        with np.errstate(divide='ignore', invalid='ignore'):
            a0 = dgamma * self.mu / tau_eq
        a1 = self.mu / (self.H + 3 * self.mu)
        al = np.where(plastic, self.K / 2. - self.mu / 3 + a0 * self.mu, 0.5 * self.lam)
        bt = np.where(plastic, (1 - 3 * a0) * self.mu, self.mu)
        gm = np.where(plastic, 2 * self.mu * (a0 - a1), 0.0)
        Fi = np.linalg.inv(F)
        P = np.einsum('pij,pkj->pik', tau, Fi)
        I = np.eye(d)
        K = np.zeros((n, d, d, d, d))
        for j in range(d):
            for nn in range(d):
                t = V[:, j, :, None] * MV[:, nn, None, :] + MV[:, nn, :, None] * V[:, j, None, :]
                sm = g * t
                trs = np.einsum('pii->p', sm)
                nsv = np.einsum('pij,pij->p', Nt, sm)
                dl = np.einsum('pik,pkl,pjl->pij', V, sm, V)
                dtau = bt[:, None, None] * dl + (gm * nsv)[:, None, None] * N + (al * trs)[:, None, None] * I
                K[:, :, :, j, nn] = np.einsum('pir,pmr->pim', dtau, Fi) - P[:, :, nn, None] * Fi[:, None, :, j]
        return P, K


def _expm_guard(ln_be):
    """expm of a batch that may hold non-finite entries: NaN where not finite."""
    out = np.full_like(ln_be, np.nan)
    ok = np.all(np.isfinite(ln_be), axis=(1, 2))
    if np.any(ok):
        out[ok] = expm_sym(ln_be[ok])
    return out


# ---------------------------------------------------------------------------
# FFT engine (src/fft/fftw_engine.cc:53-158, src/fft/fft_engine_base.cc:40-70)

def _rfftn(a, axes):
    if _sfft is not None:
        return _sfft.rfftn(a, axes=axes, workers=FFT_WORKERS)
    return np.fft.rfftn(a, axes=axes)


def _irfftn(a, s, axes):
    if _sfft is not None:
        return _sfft.irfftn(a, s=s, axes=axes, workers=FFT_WORKERS)
    return np.fft.irfftn(a, s=s, axes=axes)


class FFTEngine:
    """FFTWEngine: batched (howmany = nb_components) unnormalised r2c / c2r over
    interleaved components (istride = howmany, idist = 1, fftw_engine.cc:65-77).
    Real field: N_px*nb_comp values, AoS.  Workspace: N_h*nb_comp complex, AoS."""

    def __init__(self, resolutions, nb_components):
        self.res = list(resolutions)
        self.nb = int(nb_components)
        self.fourier_res = hermitian_sizes(self.res)

    def normalisation(self):
        """fft_engine_base.cc:49: 1/N_px."""
        return 1.0 / float(np.prod(self.res))

    def fft(self, vec):
        a = np.asarray(vec, dtype=float).reshape(*self.res, self.nb)
        out = _rfftn(a, axes=tuple(range(len(self.res))))
        return out.reshape(-1)

    def ifft(self, work):
        w = np.asarray(work, dtype=complex).reshape(*self.fourier_res, self.nb)
        out = _irfftn(w, s=self.res, axes=tuple(range(len(self.res))))
        return out.reshape(-1) * float(np.prod(self.res))


# ---------------------------------------------------------------------------
# projections (src/fft/projection_*.cc)

SMALL, FINITE_FAST, FINITE_FULL = 'small', 'finite_fast', 'finite_full'


def unit_xi_grid(res, lengths):
    """fft_utils.hh:109-129 over the hermitian grid: ξ/‖ξ‖ with ξ_d = freq_d/L_d.
    Returns xi[k..., d] (the zero mode is left as 0 instead of NaN; the reference
    overwrites its operator there with 0, projection_small_strain.cc:82-84)."""
    dim = len(res)
    fres = hermitian_sizes(res)
    freqs = [fft_freqs(res[d], lengths[d])[:fres[d]] for d in range(dim)]
    grids = np.meshgrid(*freqs, indexing='ij')
    xi = np.stack(grids, axis=-1)
    nrm = np.sqrt(np.sum(xi * xi, axis=-1))
    with np.errstate(divide='ignore', invalid='ignore'):
        uxi = xi / nrm[..., None]
    uxi[nrm == 0] = 0.0
    return uxi


def nyquist_mask(res):
    """Even-grid extension (not in the reference, which rejects even grids):
    True at every hermitian k-point with a Nyquist index on some axis."""
    fres = hermitian_sizes(res)
    masks = []
    for d, n in enumerate(res):
        m = np.zeros(fres[d], dtype=bool)
        if n % 2 == 0:
            m[n // 2] = True
        masks.append(m)
    grids = np.meshgrid(*masks, indexing='ij')
    out = np.zeros(fres, dtype=bool)
    for g in grids:
        out |= g
    return out


class Projection:
    """ProjectionSmallStrain / ProjectionFiniteStrainFast / ProjectionFiniteStrain.

    * small strain (projection_small_strain.cc:56-86):
      Ĝ_ijlm = ½(ξi δjl ξm + ξi δjm ξl + ξj δil ξm + ξj δim ξl) − ξi ξj ξl ξm
    * finite strain fast (projection_finite_strain_fast.cc:61-87): f ← (f ξ) ξᵀ
    * finite strain full (projection_finite_strain.cc:62-95): Ĝ = I ⊗̲ ξξᵀ
    apply (projection_default.cc:54-63): f̂ ← (1/N) Ĝ f̂, with f̂ = r2c(f), f = c2r(f̂).

    The apply uses the contracted form of each operator (identical maths, no D⁴ table);
    :meth:`get_operator` materialises Ĝ exactly as the reference stores it.
    """

    def __init__(self, resolutions, lengths, kind, allow_even=False):
        self.res = list(resolutions)
        self.lengths = [float(x) for x in lengths]
        self.dim = len(self.res)
        self.kind = kind
        self.allow_even = allow_even
        if not allow_even:
            for r in self.res:
                if r % 2 == 0:
                    raise ProjectionError("Only an odd number of gridpoints in each direction is supported")
        self.engine = FFTEngine(self.res, self.dim * self.dim)
        self.xi = unit_xi_grid(self.res, self.lengths)
        self.mask = nyquist_mask(self.res) if allow_even else None

    def formulation(self):
        return SMALL_STRAIN if self.kind == SMALL else FINITE_STRAIN

    def _apply_hat(self, fh):
        """fh[k..., i, j] complex -> G fh (without the 1/N factor)."""
        xi = self.xi
        if self.kind == SMALL:
            a = np.einsum('...ij,...j->...i', fh + np.swapaxes(fh, -1, -2), xi)
            s = np.einsum('...i,...ij,...j->...', xi, fh, xi)
            out = 0.5 * (xi[..., :, None] * a[..., None, :] + a[..., :, None] * xi[..., None, :]) \
                - xi[..., :, None] * xi[..., None, :] * s[..., None, None]
        else:
            fx = np.einsum('...ij,...j->...i', fh, xi)
            out = fx[..., :, None] * xi[..., None, :]
        if self.mask is not None:
            out[self.mask] = 0
        return out

    def apply(self, vec):
        """Returns the projected field (flat AoS vector)."""
        d = self.dim
        f = t2_from_vec(np.asarray(vec, dtype=float), d).reshape(*self.res, d, d)
        axes = tuple(range(d))
        fh = _rfftn(f, axes=axes)
        fh = self._apply_hat(fh)
        out = _irfftn(fh, s=self.res, axes=axes)
        return t2_to_vec(out.reshape(-1, d, d))

    def get_operator(self):
        """Reference storage of the operator, one column per hermitian k-point:
        small/finite_full -> (D^4, N_h) with row (i+Dj) + D^2 (l+Dm);
        finite_fast -> (D, N_h) unit wave vectors."""
        d = self.dim
        xi = self.xi.reshape(-1, d)
        if self.kind == FINITE_FAST:
            return xi.T.copy()
        I = np.eye(d)
        if self.kind == SMALL:
            G = 0.5 * (np.einsum('pi,jl,pm->pijlm', xi, I, xi) + np.einsum('pi,jm,pl->pijlm', xi, I, xi)
                       + np.einsum('pj,il,pm->pijlm', xi, I, xi) + np.einsum('pj,im,pl->pijlm', xi, I, xi)) \
                - np.einsum('pi,pj,pl,pm->pijlm', xi, xi, xi, xi)
        else:
            G = np.einsum('ik,pj,pl->pijkl', I, xi, xi)  # outer_under(I, ξξᵀ)
        if self.mask is not None:
            G[self.mask.reshape(-1)] = 0
        return t4_to_vec(G).reshape(-1, d ** 4).T.copy()


# ---------------------------------------------------------------------------
# cell (src/cell/cell_base.cc)

class Cell:
    """CellBase<D,D> with the projection chosen by make_cell (cell_factory.hh:59-105):
    finite strain -> ProjectionFiniteStrainFast, small strain -> ProjectionSmallStrain."""

    def __init__(self, resolutions, lengths, formulation, allow_even=False):
        self.res = list(resolutions)
        self.dim = len(self.res)
        self.lengths = list(lengths)
        self.form = formulation
        kind = FINITE_FAST if formulation == FINITE_STRAIN else SMALL
        self.projection = Projection(self.res, self.lengths, kind, allow_even=allow_even)
        self.n_px = int(np.prod(self.res))
        d2 = self.dim * self.dim
        self.F = np.zeros(self.n_px * d2)
        self.P = np.zeros(self.n_px * d2)
        self.K = None
        self.materials: List[Material] = []
        self.initialised = False

    # -- API ---------------------------------------------------------------
    def nb_dof(self):
        return self.n_px * self.dim * self.dim

    def add_material(self, mat):
        self.materials.append(mat)
        return mat

    def check_material_coverage(self):
        """cell_base.cc:486-526."""
        owner = np.full(self.n_px, -1)
        for m_id, mat in enumerate(self.materials):
            for p in mat.pixels:
                if owner[p] != -1:
                    raise RuntimeError("Pixel %s is already assigned to material '%s' and cannot be reassigned to material '%s"
                                       % (get_ccoord(self.res, p), self.materials[owner[p]].name, mat.name))
                owner[p] = m_id
        if np.any(owner < 0):
            raise RuntimeError("The following pixels have were not assigned a material: ...")

    def initialise(self):
        """cell_base.cc:445-454."""
        self.check_material_coverage()
        for mat in self.materials:
            mat.initialise()
        self.initialised = True

    def set_uniform_strain(self, strain):
        """cell_base.cc:110-112."""
        F = np.broadcast_to(np.asarray(strain, dtype=float), (self.n_px, self.dim, self.dim))
        self.F = t2_to_vec(F.copy())

    def evaluate_stress_tangent(self):
        """cell_base.cc:129-146 (+ material_muSpectre_base.hh:292-401 per material)."""
        if not self.initialised:
            self.initialise()
        d = self.dim
        Fa = t2_from_vec(self.F, d)
        P = np.zeros_like(Fa)
        K = np.zeros((self.n_px, d, d, d, d))
        for mat in self.materials:
            idx = np.asarray(mat.pixels, dtype=np.int64)
            if idx.size == 0:
                continue
            Pm, Km = mat.evaluate(Fa[idx], self.form)
            P[idx] = Pm
            K[idx] = Km
        self.P = t2_to_vec(P)
        self.K = K
        return self.P, K

    def directional_stiffness(self, dF_vec):
        """cell_base.cc:150-192: dP = K:δF (tensmult) then project."""
        d = self.dim
        dP = tensmult(self.K, t2_from_vec(dF_vec, d))
        return self.projection.apply(t2_to_vec(dP))

    evaluate_projected_directional_stiffness = directional_stiffness

    def apply_projection(self, vec):
        """cell_base.cc:202-208."""
        return self.projection.apply(vec)

    def save_history_variables(self):
        """cell_base.cc:458-462."""
        for mat in self.materials:
            mat.save_history_variables()


# ---------------------------------------------------------------------------
# solvers (src/solver/)

@dataclass
class OptimizeResult:
    """solver_common.hh:50-67."""
    grad: np.ndarray
    stress: np.ndarray
    success: bool
    status: int
    message: str
    nb_it: int
    nb_fev: int


class SolverCG:
    """solver_cg.cc:54-110 -- Nocedal Alg. 5.2, x0 = 0, forced first iteration,
    stop on ‖r‖² ≤ tol²‖b‖², ConvergenceError otherwise; counter never reset."""

    def __init__(self, cell, tol, maxiter, verbose=False):
        self.cell, self.tol, self.maxiter, self.verbose = cell, float(tol), int(maxiter), verbose
        self.counter = 0
        self.converged = False
        self.history: List[int] = []  # CG iterations of each solve (diagnostic)

    def initialise(self):
        pass

    def get_counter(self):
        return self.counter

    def get_maxiter(self):
        return self.maxiter

    def get_tol(self):
        return self.tol

    def reset_counter(self):
        self.counter = 0

    def name(self):
        return "CG"

    def solve(self, rhs):
        x = np.zeros_like(rhs)
        r = self.cell.evaluate_projected_directional_stiffness(x) - rhs
        p = -r
        self.converged = False
        rdr = float(r @ r)
        rhs_norm2 = float(rhs @ rhs)
        tol2 = self.tol ** 2 * rhs_norm2
        i = 0
        while i < self.maxiter and (rdr > tol2 or i == 0):
            Ap = self.cell.evaluate_projected_directional_stiffness(p)
            alpha = rdr / float(p @ Ap)
            x += alpha * p
            r += alpha * Ap
            new_rdr = float(r @ r)
            beta = new_rdr / rdr
            rdr = new_rdr
            p = -r + beta * p
            i += 1
            self.counter += 1
        self.history.append(i)
        if rdr < tol2:
            self.converged = True
        else:
            raise ConvergenceError("Conjugate gradient has not converged. After %d steps, the solver  FAILED with  |r|/|b| = %g, cg_tol = %g"
                                   % (self.counter, math.sqrt(rdr / rhs_norm2) if rhs_norm2 > 0 else float('nan'), self.tol))
        return x


def check_symmetry(eps, rel_tol=1e-8):
    """solver_common.cc:39-43."""
    eps = np.asarray(eps, dtype=float)
    n = np.linalg.norm(eps)
    return bool(rel_tol >= np.linalg.norm(eps - eps.T) / n if n > 0 else True) or rel_tol >= n


def _line_search(cell, incrF, nr):
    """Backtracking (Armijo) line search on the norm of the projected residual G(-P),
    an extension of newton_cg (off by default): F = F0 + λ δF with λ = 1, 1/2, …, the
    first λ whose residual norm is below (1 - 1e-4 λ) times the current one, or
    λ = 1/1024.  Returns the projected residual at the accepted point and its norm
    (the next Newton iteration starts from this evaluation)."""
    F0 = cell.F.copy()
    lam = 1.0
    while True:
        cell.F = F0 + lam * incrF
        P, _ = cell.evaluate_stress_tangent()
        rhs = cell.apply_projection(-P)
        n2 = math.sqrt(float(rhs @ rhs))
        if n2 < (1.0 - 1e-4 * lam) * nr or lam <= 1.0 / 1024:
            return rhs, n2
        lam *= 0.5


def newton_cg(cell, load_steps, solver, newton_tol, equil_tol, verbose=0, line_search=False):
    """solvers.cc:44-217.  ``load_steps``: one D×D matrix or a list of them.
    Returns a list of OptimizeResult for a list input, one result otherwise.
    ``line_search`` (an extension, off by default) damps each Newton increment by
    :func:`_line_search`; the convergence test still measures the full increment δF,
    and a load step takes at most min(maxiter, 100) Newton iterations."""
    single = isinstance(load_steps, np.ndarray) and load_steps.ndim == 2
    steps = [np.asarray(load_steps, dtype=float)] if single else [np.asarray(s, dtype=float) for s in load_steps]
    d = cell.dim
    solver.initialise()
    if cell.form == FINITE_STRAIN:
        cell.set_uniform_strain(np.eye(d))
        for s in steps:
            if s.shape != (d, d):
                raise SolverError("Load increments need to be given in %d×%d matrices" % (d, d))
    elif cell.form == SMALL_STRAIN:
        cell.set_uniform_strain(np.zeros((d, d)))
        for s in steps:
            if s.shape != (d, d):
                raise SolverError("Load increments need to be given in %d×%d matrices" % (d, d))
            if not check_symmetry(s):
                raise SolverError("all Δε must be symmetric!")
    else:
        raise SolverError("Unknown strain measure")

    results = []
    previous = np.zeros((d, d))
    for macro in steps:
        Fa = t2_from_vec(cell.F, d)
        Fa += macro - previous
        cell.F = t2_to_vec(Fa)
        message = "Has not converged"
        incr_norm, grad_norm = 2 * newton_tol, 1.0
        stress_norm = 2 * equil_tol
        state = {'conv': False, 'msg': message}

        def convergence_test():
            incr_test = incr_norm / grad_norm <= newton_tol
            stress_test = stress_norm < equil_tol
            if incr_test:
                state['msg'] = "Residual  tolerance reached"
            elif stress_test:
                state['msg'] = "Reached stress divergence tolerance"
            state['conv'] = incr_test or stress_test
            return state['conv']

        newt_iter = 0
        evaluated = False
        newton_max = min(solver.get_maxiter(), 100) if line_search else solver.get_maxiter()
        while newt_iter < newton_max and not state['conv']:
            if not evaluated:
                P, _ = cell.evaluate_stress_tangent()
                rhs = -P
                rhs = cell.apply_projection(rhs)
                stress_norm = math.sqrt(float(rhs @ rhs))
            evaluated = False
            if convergence_test():
                break
            incrF = solver.solve(rhs)
            if line_search:
                rhs, stress_norm = _line_search(cell, incrF, stress_norm)
                evaluated = True
            else:
                cell.F = cell.F + incrF
            incr_norm = math.sqrt(float(incrF @ incrF))
            grad_norm = math.sqrt(float(cell.F @ cell.F))
            if verbose > 0:
                print("at Newton step %d, |δF|/|ΔF| = %.17g, tol = %g" % (newt_iter, incr_norm / grad_norm, newton_tol))
            convergence_test()
            newt_iter += 1
        previous = macro
        conv = convergence_test()
        results.append(OptimizeResult(cell.F.copy().reshape(-1, 1), cell.P.copy().reshape(-1, 1), conv, int(conv),
                                      state['msg'], newt_iter, solver.get_counter()))
        cell.save_history_variables()
    return results[0] if single else results


def de_geus(cell, load_steps, solver, newton_tol, equil_tol, verbose=0, line_search=False):
    """solvers.cc:220-408: Newton-Krylov of de Geus et al. (2017).  Per load step the
    first Newton iteration solves K δF = -G(K:ΔF̄) at the previous equilibrium
    (:343-355) and then applies ΔF̄ + δF; later iterations are those of newton_cg
    (``line_search`` as there, for the iterations after the first)."""
    single = isinstance(load_steps, np.ndarray) and load_steps.ndim == 2
    steps = [np.asarray(load_steps, dtype=float)] if single else [np.asarray(s, dtype=float) for s in load_steps]
    d = cell.dim
    solver.initialise()
    if cell.form == FINITE_STRAIN:
        cell.set_uniform_strain(np.eye(d))
        for s in steps:
            if s.shape != (d, d):
                raise SolverError("Load increments need to be given in %d×%d matrices" % (d, d))
    elif cell.form == SMALL_STRAIN:
        cell.set_uniform_strain(np.zeros((d, d)))
        for s in steps:
            if s.shape != (d, d):
                raise SolverError("Load increments need to be given in %d×%d matrices" % (d, d))
            if not check_symmetry(s):
                raise SolverError("all Δε must be symmetric!")
    else:
        raise SolverError("Unknown strain measure")

    results = []
    previous = np.zeros((d, d))
    for macro in steps:
        incr_norm, grad_norm = 2 * newton_tol, 1.0
        stress_norm = 2 * equil_tol
        state = {'conv': False, 'msg': "Has not converged"}

        def convergence_test():
            incr_test = incr_norm / grad_norm <= newton_tol
            stress_test = stress_norm < equil_tol
            if incr_test:
                state['msg'] = "Residual  tolerance reached"
            elif stress_test:
                state['msg'] = "Reached stress divergence tolerance"
            state['conv'] = incr_test or stress_test
            return state['conv']

        newt_iter = 0
        evaluated = False
        newton_max = min(solver.get_maxiter(), 100) if line_search else solver.get_maxiter()
        while newt_iter < newton_max and not state['conv']:
            if not evaluated:
                P, _ = cell.evaluate_stress_tangent()
            if newt_iter == 0:
                DeltaF = t2_to_vec(np.broadcast_to(macro - previous, (cell.n_px, d, d)).copy())
                rhs = -cell.evaluate_projected_directional_stiffness(DeltaF)
                stress_norm = math.sqrt(float(rhs @ rhs))
                if convergence_test():
                    break
                incrF = solver.solve(rhs)
                cell.F = cell.F + DeltaF
                cell.F = cell.F + incrF
            else:
                if not evaluated:
                    rhs = cell.apply_projection(-P)
                    stress_norm = math.sqrt(float(rhs @ rhs))
                evaluated = False
                if convergence_test():
                    break
                incrF = solver.solve(rhs)
                if line_search:
                    rhs, stress_norm = _line_search(cell, incrF, stress_norm)
                    evaluated = True
                else:
                    cell.F = cell.F + incrF
            incr_norm = math.sqrt(float(incrF @ incrF))
            grad_norm = math.sqrt(float(cell.F @ cell.F))
            if verbose > 0:
                print("at Newton step %d, |δF|/|ΔF| = %.17g, tol = %g" % (newt_iter, incr_norm / grad_norm, newton_tol))
            convergence_test()
            newt_iter += 1
        previous = macro
        conv = convergence_test()
        results.append(OptimizeResult(cell.F.copy().reshape(-1, 1), cell.P.copy().reshape(-1, 1), conv, int(conv),
                                      state['msg'], newt_iter, solver.get_counter()))
        cell.save_history_variables()
    return results[0] if single else results


def homogenised(vec, dim):
    """Pixel mean of a flat AoS field as a D×D matrix (FP64)."""
    return t2_from_vec(np.asarray(vec, dtype=float).reshape(-1), dim).mean(axis=0)
