"""Pin the CPU oracle against the known answers of the reference's own tests.

Each test names the reference test it restates.  The fixtures under ``tests/golden``
were written by ``tests/golden/make_golden.py`` from the reference tree.
"""
import itertools
import json
import os

import numpy as np
import pytest

from oracle import muspectre_oracle as o

GOLD = os.path.join(os.path.dirname(__file__), 'golden')
TOL = 1e-14 * 100  # tests/tests.hh:63


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_fftfreq_kat():
    """test_fft_utils.cc:43-84."""
    d = _load('fftfreq_kat.json')
    for case in d['cases']:
        assert np.abs(o.fft_freqs(case['n'], case['length']) - case['freqs']).sum() == 0.0
    for case in d['xi_cases']:
        xi = np.array([o.fft_freqs(n, L)[c] for n, L, c in zip(case['res'], case['lengths'], case['ccoord'])])
        assert np.linalg.norm(xi - case['xi']) < TOL
        uxi = xi / np.linalg.norm(xi)
        assert abs(uxi @ xi - np.linalg.norm(xi)) < np.linalg.norm(xi) * TOL


def test_hermitian_and_index_helpers():
    """ccoord_operations.hh:64-68,151-192."""
    assert o.hermitian_sizes([6, 4]) == [6, 3]
    assert o.hermitian_sizes([5, 5, 5]) == [5, 5, 3]
    res = [3, 4, 5]
    for i in range(60):
        assert o.get_index(res, o.get_ccoord(res, i)) == i
    assert o.get_ccoord(res, 1) == [0, 0, 1]


def test_expm_kat():
    """header_test_eigen_tools.cc:42-62."""
    d = _load('expm_kat.json')
    out = o.expm_sym(np.array(d['input'])[None])[0]
    assert np.linalg.norm(out - np.array(d['output'])) < d['tol']


def test_logm_inverse_of_expm():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((20, 3, 3)) * 0.3
    A = A + A.transpose(0, 2, 1)
    L = o.logm_projector(o.expm_sym(A))
    assert np.max(np.abs(L - A)) < 1e-10
    assert np.max(np.abs(o.logm_spectral(o.expm_sym(A)) - A)) < 1e-12


def test_hep1_kat():
    """test_material_hyper_elasto_plastic1.cc:85-339: elastic then plastic step on one
    pixel, Kirchhoff stress, bₑ, εₚ and the material tangent."""
    d = _load('hep1_kat.json')
    K, mu = d['K'], d['mu']
    E = o.young_from_K_mu(K, mu)
    nu = o.poisson_from_K_mu(K, mu)
    mat = o.MaterialHyperElastoPlastic1('Name', 3, E, nu, d['tau_y0'], d['H'])
    mat.add_pixel(0)
    # the test sets current() to I / I / 0 then cycles (same as initialise())
    mat.initialise()
    F = np.eye(3)[None].copy()
    for step in d['steps']:
        F[0, 0, 1] = step['F01']
        tau, C = mat.evaluate_stress_tangent_kirchhoff(F)
        assert np.linalg.norm(tau[0] - np.array(step['tau'])) < d['tol']
        assert np.linalg.norm(mat._cur(mat.be_prev)[0] - np.array(step['be'])) < d['tol']
        assert abs(step['eps_p'] - mat._cur(mat.eps_p)[0]) < d['tol']
        C_rows = o.t4_to_vec(C).reshape(9, 9).T  # T4 matrix (row i+3j, column k+3l)
        assert np.linalg.norm(C_rows - np.array(step['C4_rows'])) < d['tol']
        mat.save_history_variables()


def test_le4_response_kat():
    """test_material_linear_elastic4.cc:69-100."""
    for dim in (2, 3):
        E = np.zeros((1, dim, dim))
        E[0, 0, 0] = 0.001
        E[0, 1, 0] = E[0, 0, 1] = 0.005
        mat = o.MaterialLinearElastic4('name', dim)
        mat.add_pixel(0, 10.0, 0.3)
        lam, mu = o.lame_lambda(10.0, 0.3), o.lame_mu(10.0, 0.3)
        s, _ = mat.evaluate(E, o.SMALL_STRAIN)
        s = s[0]
        assert abs(s[0, 0] - (lam * E[0, 0, 0] + 2 * mu * E[0, 0, 0])) < TOL
        assert abs(s[0, 1] - 2 * mu * E[0, 0, 1]) < TOL
        assert abs(s[1, 0] - 2 * mu * E[0, 0, 1]) < TOL
        assert abs(s[1, 1] - lam * E[0, 0, 0]) < TOL
        if dim == 3:
            assert abs(s[2, 2] - lam * E[0, 0, 0]) < TOL


@pytest.mark.parametrize('dim', [2, 3])
@pytest.mark.parametrize('form', [o.FINITE_STRAIN, o.SMALL_STRAIN])
def test_cell_simple_evaluation(dim, form):
    """test_cell_base.cc:119-170: LE1 at F = I (finite) / ε = 0 (small) gives
    objective_hooke_explicit(λ, μ, I) exactly: P = 0 and K = C."""
    res = [3] * dim
    cell = o.Cell(res, [1.0] * dim, form)
    mat = cell.add_material(o.MaterialLinearElastic1('hard', dim, 210e9, .33))
    for i in range(cell.n_px):
        mat.add_pixel(i)
    cell.set_uniform_strain(np.eye(dim) if form == o.FINITE_STRAIN else np.zeros((dim, dim)))
    P, K = cell.evaluate_stress_tangent()
    assert np.all(P == 0)
    C = o.hooke_C(o.lame_lambda(210e9, .33), o.lame_mu(210e9, .33), dim)
    assert np.all(K == C)


def _laminate_cell(dim=2):
    res = [3] * dim
    cell = o.Cell(res, [1.0] * dim, o.SMALL_STRAIN)
    hard = cell.add_material(o.MaterialLinearElastic1('hard', dim, 2 * 2.0, .33))
    soft = cell.add_material(o.MaterialLinearElastic1('soft', dim, 2.0, .33))
    for i in range(cell.n_px):
        (hard if o.get_ccoord(res, i)[0] < 1 else soft).add_pixel(i)
    return cell, res


def test_laminate_patch():
    """test_solver_newton_cg.cc:218-323 (SolverCG): uniaxial and pure-shear patch tests
    on a 3×3 laminate with contrast 2; exact layer strains to 1e-12."""
    cell, res = _laminate_cell()
    factor = 1 / 2 * 1 / 3 + 1. - 1 / 3.
    eps_soft = 1.0 / factor
    eps_hard = eps_soft / 2
    for load, pattern in ((np.array([[1., 0], [0, 0]]), np.array([[1., 0], [0, 0]])),
                          (np.array([[0, 1.], [1., 0]]), np.array([[0, 1.], [1., 0]]))):
        solver = o.SolverCG(cell, 1e-8, 2 * 10)
        r = o.newton_cg(cell, load, solver, 1e-5, 1e-10, 0)
        F = o.t2_from_vec(cell.F, 2)
        for i in range(cell.n_px):
            ref = (eps_hard if o.get_ccoord(res, i)[0] < 1 else eps_soft) * pattern
            assert np.linalg.norm(F[i] - ref) <= TOL
        assert r.success



def test_laminate_patch_de_geus():
    """test_solver_newton_cg.cc:218-323 with de_geus (the pure-shear case there runs
    de_geus, :310-323): exact layer strains to 1e-12 for both load patterns."""
    cell, res = _laminate_cell()
    factor = 1 / 2 * 1 / 3 + 1. - 1 / 3.
    eps_soft = 1.0 / factor
    eps_hard = eps_soft / 2
    for pattern in (np.array([[1., 0], [0, 0]]), np.array([[0, 1.], [1., 0]])):
        solver = o.SolverCG(cell, 1e-8, 2 * 10)
        r = o.de_geus(cell, pattern, solver, 1e-5, 1e-10, 0)
        F = o.t2_from_vec(cell.F, 2)
        for i in range(cell.n_px):
            ref = (eps_hard if o.get_ccoord(res, i)[0] < 1 else eps_soft) * pattern
            assert np.linalg.norm(F[i] - ref) <= TOL
        assert r.success


def test_de_geus_first_step_is_the_increment_response():
    """solvers.cc:343-355: the first de Geus iteration solves K dF = -G(K:DF) at the
    previous equilibrium; on a linear cell de_geus and newton_cg reach the same
    strain field."""
    cell, res = _laminate_cell()
    load = np.array([[0.3, 0.1], [0.1, -0.2]])
    rg = o.de_geus(cell, load, o.SolverCG(cell, 1e-12, 40), 1e-8, 0.0, 0)
    Fg = cell.F.copy()
    rn = o.newton_cg(cell, load, o.SolverCG(cell, 1e-12, 40), 1e-8, 0.0, 0)
    assert rg.success and rn.success
    assert np.abs(Fg - cell.F).max() < 1e-10

def test_le4_homogeneous_solve():
    """python_material_linear_elastic4_test.py:63-86: σ = 2μΔε on a homogeneous 7×7."""
    cell = o.Cell([7, 7], [2.3, 3.9], o.SMALL_STRAIN)
    mat = cell.add_material(o.MaterialLinearElastic4('material', 2))
    for i in range(cell.n_px):
        mat.add_pixel(i, 10., 0.3)
    Del0 = np.array([[0, 0.025], [0.025, 0]])
    solver = o.SolverCG(cell, 1e-6, 100)
    r = o.newton_cg(cell, Del0, solver, 1e-6, 1e-6, 0)
    mu = 10. / (2 * 1.3)
    stress = 2 * mu * Del0
    assert np.linalg.norm(r.stress.reshape(-1, 4) - stress.reshape(1, 4)) < 1e-8


GOOSE = np.load(os.path.join(GOLD, 'goose_projection.npz'))


@pytest.mark.parametrize('ndim', [2, 3])
@pytest.mark.parametrize('kind', ['small', 'finite_fast', 'finite_full'])
def test_projection_vs_goose(ndim, kind):
    """python_projection_tests.py:99-130 (test_projection_result), 1e-12·N tolerance."""
    gkind = 'small' if kind == 'small' else 'finite'
    strain_g = GOOSE['%s_%dd_strain' % (gkind, ndim)]
    b_g = GOOSE['%s_%dd_result' % (gkind, ndim)]
    shape = [5] * ndim
    proj = o.Projection(shape, shape, kind)
    tol = 1e-12 * np.prod(shape)
    strain_mu = np.zeros((*shape, ndim, ndim))
    for ijk in itertools.product(range(5), repeat=ndim):
        strain_mu[ijk] = strain_g[(slice(None), slice(None), *ijk)].T
    # the reference binding takes a (D², N) array whose column is the pixel's
    # row-major D×D block; as an Eigen (column-major) matrix that block is its transpose
    vec = strain_mu.reshape(-1, ndim * ndim).reshape(-1)
    b_mu = proj.apply(vec).reshape(*shape, ndim, ndim)
    for ijk in itertools.product(range(5), repeat=ndim):
        err = np.linalg.norm(b_mu[ijk].T - b_g[(slice(None), slice(None), *ijk)])
        assert err < tol


@pytest.mark.parametrize('ndim', [2, 3])
@pytest.mark.parametrize('kind', ['small', 'finite_full'])
def test_ghat_vs_goose(ndim, kind):
    """python_projection_tests.py:63-97 (test_CompareGhat4) incl. its index shuffle."""
    gkind = 'small' if kind == 'small' else 'finite'
    refG = GOOSE['%s_%dd_ghat4' % (gkind, ndim)]
    shape = [5] * ndim
    proj = o.Projection(shape, shape, kind)
    d2 = ndim * ndim
    refG = refG.reshape(d2, d2, -1)
    mspG = proj.get_operator()
    msp_sizes = o.hermitian_sizes(shape)
    order = np.arange(d2).reshape(ndim, ndim).T.reshape(-1)
    tol = 1e-12 * np.prod(shape)
    for i in range(int(np.prod(msp_sizes))):
        coord = o.get_ccoord(msp_sizes, i)
        ref_id = o.get_index(shape, coord)
        msp_g = mspG[:, i].reshape(d2, d2)[order, :]
        assert np.linalg.norm(refG[:, :, ref_id] - msp_g) < tol


def test_projection_rejects_even():
    """projection_small_strain.cc:46-51 / test_projection_finite.cc:71-77."""
    with pytest.raises(o.ProjectionError):
        o.Projection([4, 5], [1., 1.], 'small')
    with pytest.raises(o.ProjectionError):
        o.Cell([5, 6], [1., 1.], o.FINITE_STRAIN)


@pytest.mark.parametrize('res', [[4, 4, 4], [6, 6, 6], [8, 8, 8], [6, 5]])
@pytest.mark.parametrize('kind', ['small', 'finite_fast'])
def test_even_extension_idempotent_hermitian(res, kind):
    """Even-grid extension (Ĝ = 0 at Nyquist points): G(Gf) = Gf and real output."""
    rng = np.random.default_rng(0)
    dim = len(res)
    proj = o.Projection(res, [1.0] * dim, kind, allow_even=True)
    f = rng.standard_normal(int(np.prod(res)) * dim * dim)
    if kind == 'small':
        fa = o.t2_from_vec(f, dim)
        f = o.t2_to_vec(0.5 * (fa + fa.transpose(0, 2, 1)))
    g1 = proj.apply(f)
    g2 = proj.apply(g1)
    assert np.linalg.norm(g2 - g1) < 1e-12 * np.linalg.norm(g1)


def test_fft_engine_vs_numpy():
    """python_fft_tests.py:60-101 at [6, 4] (even sizes are fine for the engine)."""
    rng = np.random.default_rng(1)
    res = [6, 4]
    eng = o.FFTEngine(res, 4)
    tol = 1e-14 * np.prod(res)
    in_arr = rng.random([*res, 2, 2])
    out_ref = np.fft.rfftn(in_arr, axes=(0, 1))
    out = eng.fft(in_arr.reshape(-1))
    assert np.linalg.norm(out_ref.reshape(-1) - out) < tol
    cres = o.hermitian_sizes(res)
    c = rng.random([*cres, 2, 2]) + 1j * rng.random([*cres, 2, 2])
    ref = np.fft.irfftn(c, s=res, axes=(0, 1))
    back = eng.ifft(c.reshape(-1)) * eng.normalisation()
    assert np.linalg.norm(ref.reshape(-1) - back) < tol


def test_cg_counter_cumulative_and_forced_iteration():
    """solver_cg.cc:76-77 (forced first iteration) and solvers.cc:208-210 (nb_fev is
    the cumulative CG count)."""
    cell, _ = _laminate_cell()
    solver = o.SolverCG(cell, 1e-8, 20)
    r1 = o.newton_cg(cell, [np.array([[0.01, 0], [0, 0]]), np.array([[0.02, 0], [0, 0]])], solver, 1e-5, 1e-10, 0)
    assert r1[1].nb_fev >= r1[0].nb_fev
    assert r1[1].nb_fev == sum(solver.history)


def test_cg_convergence_error():
    """solver_cg.cc:99-108: ConvergenceError when maxiter is reached."""
    res = [5, 5]
    cell = o.Cell(res, [1.0, 1.0], o.SMALL_STRAIN)
    rng = np.random.default_rng(2)
    mat = cell.add_material(o.MaterialLinearElastic4('m', 2))
    for i in range(cell.n_px):
        mat.add_pixel(i, float(rng.uniform(1, 10)), 0.3)
    solver = o.SolverCG(cell, 1e-10, 1)
    with pytest.raises(o.ConvergenceError):
        o.newton_cg(cell, np.array([[1., 0], [0, 0]]), solver, 1e-5, 1e-10, 0)


def test_small_strain_rejects_asymmetric_load():
    """solvers.cc:117-124."""
    cell, _ = _laminate_cell()
    with pytest.raises(o.SolverError):
        o.newton_cg(cell, np.array([[0, 1.], [0, 0]]), o.SolverCG(cell, 1e-8, 20), 1e-5, 1e-10, 0)



@pytest.mark.parametrize('dim', [2, 3])
def test_generic_stiffness_from_voigt(dim):
    """test_material_linear_elastic_generic.cc (C_test): the Voigt matrix of an isotropic
    law with lambda = 2, mu = 1.5 gives Hooke's C_T4."""
    lam, mu = 2.0, 1.5
    vs = 3 if dim == 2 else 6
    Cv = np.zeros((vs, vs))
    Cv[:dim, :dim] = lam
    Cv[:dim, :dim] += 2 * mu * np.eye(dim)
    Cv[dim:, dim:] += mu * np.eye(vs - dim)
    mat = o.MaterialLinearElasticGeneric('material', dim, Cv)
    assert np.linalg.norm(mat.C - o.hooke_C(lam, mu, dim)) < 1e-14
    with pytest.raises(RuntimeError):
        o.MaterialLinearElasticGeneric('bad', dim, np.zeros((vs + 1, vs)))
