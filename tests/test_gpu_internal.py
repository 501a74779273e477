"""Internal fields and checkpoints.

* get_globalised_internal_real_array: the reference's tests
  (python_binding_tests.py:133-150 eigenstrain globalisation; test_cell_base.cc:
  229-331 managed and globalised fields, missing names) restated on the GPU cell,
  plus the HEP1 state fields against the oracle after two evaluations.
* checkpoint / restore: a cell rebuilt from a checkpoint continues with bit-identical
  results (elasto-plastic history included).
"""
import numpy as np
import pytest

import oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def test_eigenstrain_globalisation(mu):
    """python_binding_tests.py:133-139: globalised == the per-pixel input."""
    rng = np.random.default_rng(0)
    cell = mu.Cell([5, 7], [1., 1.], mu.Formulation.finite_strain)
    mat = mu.material.MaterialLinearElastic2_2d.make(cell, 'eigen', 210e9, .33)
    eig = rng.random((cell.nb_pixels, 2, 2))
    for p, pixel in enumerate(cell):
        mat.add_pixel(pixel, eig[p])
    g = cell.get_globalised_internal_real_array('Eigenstrain')
    assert g.shape == (4, cell.nb_pixels)
    assert np.array_equal(g, eig.transpose(0, 2, 1).reshape(-1, 4).T)


def test_eigenstrain_globalisation_constant(mu):
    """python_binding_tests.py:141-150: two LE2 materials, all ones."""
    cell = mu.Cell([5, 7], [1., 1.], mu.Formulation.finite_strain)
    m2 = mu.material.MaterialLinearElastic2_2d.make(cell, 'eigen', 210e9, .33)
    m3 = mu.material.MaterialLinearElastic2_2d.make(cell, 'eigen2', 120e9, .33)
    for i, pixel in enumerate(cell):
        (m2 if i % 2 == 0 else m3).add_pixel(pixel, np.ones((2, 2)))
    g = cell.get_globalised_internal_real_array('Eigenstrain')
    assert np.linalg.norm(g - 1) == 0


def test_lame_and_stiffness_fields(mu):
    """LE4's Lamé fields and LE3's stiffness tensor, zero at LE1 pixels."""
    rng = np.random.default_rng(1)
    cell = mu.Cell([3, 5, 7], [1., 1., 1.], mu.Formulation.small_strain)
    n = cell.nb_pixels
    owner = rng.integers(0, 3, n)
    E, nu = rng.uniform(1, 10, n), rng.uniform(0.2, 0.4, n)
    mu.material.MaterialLinearElastic1_3d.make(cell, 'a', 3.0, .3).add_pixels(np.flatnonzero(owner == 0))
    i3, i4 = np.flatnonzero(owner == 1), np.flatnonzero(owner == 2)
    mu.material.MaterialLinearElastic3_3d.make(cell, 'b').add_pixels(i3, E[i3], nu[i3])
    mu.material.MaterialLinearElastic4_3d.make(cell, 'c').add_pixels(i4, E[i4], nu[i4])
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    shear = E / (2 * (1 + nu))
    gl = cell.get_globalised_internal_real_array('local first Lame constant')
    gm = cell.get_globalised_internal_real_array('local second Lame constant(shear modulus)')
    assert gl.shape == (1, n)
    np.testing.assert_allclose(gl[0, i4], lam[i4], rtol=1e-14)
    np.testing.assert_allclose(gm[0, i4], shear[i4], rtol=1e-14)
    assert not np.any(gl[0, owner != 2]) and not np.any(gm[0, owner != 2])
    C = cell.get_globalised_internal_real_array('local stiffness tensor')
    assert C.shape == (81, n)
    d = np.eye(3)
    for p in i3[:5]:
        ref = (lam[p] * np.einsum('ij,kl->ijkl', d, d)
               + shear[p] * (np.einsum('ik,jl->ijkl', d, d) + np.einsum('il,jk->ijkl', d, d)))
        # T4 layout: entry (i + 3 j) + 9 (k + 3 l)
        np.testing.assert_allclose(C[:, p], ref.transpose(3, 2, 1, 0).reshape(-1), rtol=1e-13)
    assert not np.any(C[:, owner != 1])


def test_missing_field_and_managed_arrays(mu):
    """test_cell_base.cc:229-243 and :316-319."""
    cell = mu.Cell([3, 3], [1., 1.], mu.Formulation.finite_strain)
    mu.material.MaterialLinearElastic1_2d.make(cell, 'a', 1.0, .3).add_pixels(np.arange(9))
    with pytest.raises(RuntimeError, match='does not exist in any of the materials'):
        cell.get_globalised_internal_real_array('wrong_name')
    with pytest.raises(RuntimeError, match='does not exist'):
        cell.get_globalised_internal_real_array('Eigenstrain')   # no LE2 material here
    a = cell.get_managed_real_array('aaa', 5)
    assert a.shape == (5, cell.size)
    a[:] = 3.0
    assert np.all(cell.get_managed_real_array('aaa', 5) == 3.0)
    with pytest.raises(RuntimeError):
        cell.get_managed_real_array('aaa', 6)


def _hep_pair(mu):
    import test_gpu_parity as tp
    return tp._random_cell_pair(mu, [5, 3, 3], o.FINITE_STRAIN, 7, laws=('hep1', 'hep1', 'le1'))


def _random_F(rng, n, scale):
    return np.eye(3)[None] + scale * rng.standard_normal((n, 3, 3))


def test_hep1_state_fields_match_oracle(mu):
    """The elasto-plastic state after two evaluations (with a history cycle between
    them) equals the oracle's, sub-field by sub-field."""
    ocell, gcell, rng = _hep_pair(mu)
    n = gcell.nb_pixels
    for k in range(2):
        F = _random_F(rng, n, 0.02 * (k + 1))
        ocell.F = o.t2_to_vec(F)
        ocell.evaluate_stress_tangent()
        gcell.evaluate_stress_tangent(o.t2_to_vec(F).reshape(n, -1).T)
        if k == 0:
            ocell.save_history_variables()
            gcell.save_history_variables()
    prefixes = {'cumulated plastic flow εₚ': 'eps_p', 'Previous placement gradient Fᵗ': 'F_prev',
                'Previous left Cauchy-Green deformation bₑᵗ': 'be_prev'}
    for name, attr in prefixes.items():
        for sub in range(2):
            g = gcell.get_globalised_internal_real_array('%s, sub_field index %d' % (name, sub))
            ref = np.zeros_like(g)
            for m in ocell.materials:
                if isinstance(m, o.MaterialHyperElastoPlastic1):
                    v = getattr(m, attr)[sub]
                    for j, p in enumerate(m.pixels):
                        ref[:, p] = v[j] if v.ndim == 1 else v[j].T.reshape(-1)
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(g - ref).max() <= 1e-10 * scale, (name, sub)


def test_checkpoint_round_trip(mu):
    """Evaluate, cycle, checkpoint; a rebuilt cell restored from the image gives the
    same stress and state as the original at the next evaluation (bit-identical)."""
    _, ga, rng = _hep_pair(mu)
    _, gb, _ = _hep_pair(mu)
    n = ga.nb_pixels
    F1, F2 = _random_F(rng, n, 0.03), _random_F(rng, n, 0.04)
    v1, v2 = o.t2_to_vec(F1).reshape(n, -1).T, o.t2_to_vec(F2).reshape(n, -1).T
    ga.evaluate_stress_tangent(v1)
    ga.save_history_variables()
    image = ga.checkpoint()
    Pa = ga.evaluate_stress_tangent(v2)
    gb.restore(image)
    Pb = gb.evaluate_stress_tangent(v2)
    assert np.array_equal(Pa, Pb)
    name = 'cumulated plastic flow εₚ, sub_field index 0'
    assert np.array_equal(ga.get_globalised_internal_real_array(name), gb.get_globalised_internal_real_array(name))
    assert np.array_equal(ga.get_strain(), gb.get_strain())
    # a checkpoint does not load into a cell of another shape
    other = mu.Cell([5, 3, 5], [1., 1., 1.], mu.Formulation.finite_strain)
    mu.material.MaterialLinearElastic1_3d.make(other, 'a', 1.0, .3).add_pixels(np.arange(75))
    with pytest.raises(RuntimeError):
        other.restore(image)
