"""MaterialLinearElasticGeneric (material_linear_elastic_generic.{hh,cc}) on the GPU.

* stress and full tangent per pixel against the oracle, in cells that mix an
  anisotropic generic material with LE1 and LE2, both formulations, 2-D and 3-D;
* the README-size 2-D solve and a two-step 3-D solve against the oracle (criteria of
  test_gpu_parity.py);
* an isotropic Voigt matrix reproduces MaterialLinearElastic1;
* the mixed-precision solve within 1e-6 of FP64, and one FP32 CG-operator application
  within 1e-5 of FP64 (register and generic pass lengths).
"""
import numpy as np
import pytest

from oracle import muspectre_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def rel(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def voigt_spd(dim, seed, scale=10.0):
    rng = np.random.default_rng(seed)
    vs = 3 if dim == 2 else 6
    A = rng.standard_normal((vs, vs))
    return scale * (A @ A.T / vs + np.eye(vs))


def isotropic_voigt(dim, lam, mu_):
    vs = 3 if dim == 2 else 6
    Cv = np.zeros((vs, vs))
    Cv[:dim, :dim] = lam
    Cv[:dim, :dim] += 2 * mu_ * np.eye(dim)
    Cv[dim:, dim:] += mu_ * np.eye(vs - dim)
    return Cv


def _pair(mu, res, form, seed):
    """Same microstructure in the oracle and on the GPU: generic / LE1 / LE2 owners."""
    rng = np.random.default_rng(seed)
    d = len(res)
    n = int(np.prod(res))
    ocell = o.Cell(res, [1.0] * d, form)
    gcell = mu.Cell(res, [1.0] * d, mu.Formulation(form))
    owner = rng.integers(0, 3, n)
    Cv = voigt_spd(d, seed)
    idx = np.flatnonzero(owner == 0)
    om = ocell.add_material(o.MaterialLinearElasticGeneric('g', d, Cv))
    for i in idx:
        om.add_pixel(i)
    getattr(mu.material, 'MaterialLinearElasticGeneric_%dd' % d).make(gcell, 'g', Cv).add_pixels(idx)
    idx = np.flatnonzero(owner == 1)
    om = ocell.add_material(o.MaterialLinearElastic1('a', d, 3.0, 0.3))
    for i in idx:
        om.add_pixel(i)
    getattr(mu.material, 'MaterialLinearElastic1_%dd' % d).make(gcell, 'a', 3.0, 0.3).add_pixels(idx)
    idx = np.flatnonzero(owner == 2)
    eig = rng.standard_normal((idx.size, d, d)) * 1e-3
    eig = 0.5 * (eig + eig.transpose(0, 2, 1))
    om = ocell.add_material(o.MaterialLinearElastic2('b', d, 7.0, 0.25))
    for i, e in zip(idx, eig):
        om.add_pixel(i, e)
    getattr(mu.material, 'MaterialLinearElastic2_%dd' % d).make(gcell, 'b', 7.0, 0.25).add_pixels(idx, eig)
    return ocell, gcell


@pytest.mark.parametrize('res', [[7, 5], [5, 3, 7]])
@pytest.mark.parametrize('form', [o.SMALL_STRAIN, o.FINITE_STRAIN])
def test_generic_stress_tangent_vs_oracle(mu, res, form):
    ocell, gcell = _pair(mu, res, form, 3)
    d = len(res)
    n = ocell.n_px
    rng = np.random.default_rng(4)
    F = rng.standard_normal((n, d, d)) * 0.05
    if form == o.FINITE_STRAIN:
        F += np.eye(d)
    ocell.F = o.t2_to_vec(F)
    P, K = ocell.evaluate_stress_tangent()
    gP, gK = gcell.evaluate_stress_tangent(o.t2_to_vec(F).reshape(n, -1).T, return_tangent=True)
    assert rel(gP.T.reshape(-1), P) < 1e-13
    assert rel(gK.T.reshape(-1), o.t4_to_vec(K)) < 1e-13
    dF = rng.standard_normal((d * d, n))
    ref = ocell.directional_stiffness(dF.T.reshape(-1))
    assert rel(gcell.directional_stiffness(dF).T.reshape(-1), ref) < 1e-12


def test_generic_solve_2d_vs_oracle(mu):
    ocell, gcell = _pair(mu, [21, 19], o.SMALL_STRAIN, 8)
    D = np.array([[0.01, 0.004], [0.004, -0.002]])
    ro = o.newton_cg(ocell, D, o.SolverCG(ocell, 1e-8, 400), 1e-5, 0.0, 0)
    rg = mu.solvers.newton_cg(gcell, D, mu.solvers.SolverCG(gcell, 1e-8, 400), 1e-5, 0.0)
    assert (rg.nb_it, rg.nb_fev) == (ro.nb_it, ro.nb_fev)
    assert rel(rg.grad, ro.grad) < 1e-10
    assert rel(rg.stress, ro.stress) < 1e-10


def test_generic_solve_3d_two_steps(mu):
    ocell, gcell = _pair(mu, [9, 7, 11], o.FINITE_STRAIN, 9)
    steps = [np.diag([0.01, 0, 0]), np.diag([0.02, -0.004, 0])]
    ro = o.newton_cg(ocell, steps, o.SolverCG(ocell, 1e-8, 500), 1e-6, 0.0, 0)
    rg = mu.solvers.newton_cg(gcell, steps, mu.solvers.SolverCG(gcell, 1e-8, 500), 1e-6, 0.0)
    for a, b in zip(rg, ro):
        assert a.success and b.success
        assert a.nb_it == b.nb_it
        assert abs(a.nb_fev - b.nb_fev) <= max(1, 0.01 * b.nb_fev)
        assert rel(a.grad, b.grad) < 1e-9


def test_isotropic_generic_equals_le1(mu):
    E, nu = 5.0, 0.3
    lam, shear = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    out = []
    for generic in (False, True):
        cell = mu.Cell([9, 9, 9], [1., 1., 1.], mu.Formulation.finite_strain)
        inside = np.zeros(729, bool)
        inside[::3] = True
        mu.material.MaterialLinearElastic1_3d.make(cell, 'hard', 50.0, 0.3).add_pixels(inside)
        if generic:
            mu.material.MaterialLinearElasticGeneric_3d.make(cell, 'soft', isotropic_voigt(3, lam, shear)).add_pixels(
                ~inside)
        else:
            mu.material.MaterialLinearElastic1_3d.make(cell, 'soft', E, nu).add_pixels(~inside)
        r = mu.solvers.newton_cg(cell, np.diag([0.02, 0, 0]), mu.solvers.SolverCG(cell, 1e-10, 500), 1e-8, 0.0)
        out.append(r)
    assert abs(out[0].nb_it - out[1].nb_it) <= 1
    assert rel(out[1].stress, out[0].stress) < 1e-8


@pytest.mark.parametrize('res', [[32, 32, 32], [15, 9, 10]])
def test_generic_mixed_precision(mu, res):
    d = len(res)
    out = {}
    for prec in ('fp64', 'mixed'):
        cell = mu.Cell(res, [1.0] * d, mu.Formulation.finite_strain, allow_even=True)
        n = cell.nb_pixels
        inside = np.random.default_rng(2).random(n) < 0.3
        mu.material.MaterialLinearElasticGeneric_3d.make(cell, 'g', voigt_spd(3, 5, 100.0)).add_pixels(inside)
        mu.material.MaterialLinearElastic1_3d.make(cell, 'm', 3.0, 0.3).add_pixels(~inside)
        r = mu.solvers.newton_cg(cell, np.diag([0.01, 0, 0]), mu.solvers.SolverCG(cell, 1e-8, 3000, precision=prec),
                                 1e-8, 0.0)
        assert r.success, r.message
        out[prec] = cell
    hm, h64 = out['mixed'].homogenised_stress(), out['fp64'].homogenised_stress()
    assert rel(hm, h64) < 1e-6
    # one FP32 CG-operator application against FP64
    cell = out['fp64']
    rng = np.random.default_rng(3)
    dF = rng.standard_normal((9, cell.nb_pixels))
    ref = cell.cg_operator(dF, 'fp64')
    assert rel(cell.directional_stiffness(dF), ref) < 1e-12
    assert rel(cell.cg_operator(dF, 'mixed'), ref) < 1e-5
