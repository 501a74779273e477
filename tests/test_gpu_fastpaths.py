"""Register-resident FFT passes (power-of-two axis lengths 16..256).

The mixed-precision CG runs its last-axis, middle-axis and Green passes through the
register kernels whenever an axis length is 16, 32, 64, 128 or 256 (and the FP64
path does for its middle-axis and Green passes).  Each case below reaches them with
a different tangent kind, dimension or length, and checks the mixed solve against
the FP64 solve of the same cell: homogenised stress within 1e-6 relative (the FP64
path itself is pinned to the oracle by test_gpu_parity.py).  Both solves run to a
Newton tolerance of 1e-8, so that their difference measures the FP32 operator and
not where each run stopped.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def _inclusions(res, seed, nsph=5):
    rng = np.random.default_rng(seed)
    d = len(res)
    pts = np.stack(np.meshgrid(*[np.arange(n) for n in res], indexing='ij'), -1).reshape(-1, d).astype(float)
    inside = np.zeros(len(pts), dtype=bool)
    n = np.array(res, dtype=float)
    for _ in range(nsph):
        c = rng.uniform(0, 1, d) * n
        r = rng.uniform(0.1, 0.25) * n.min()
        dd = np.abs(pts - c)
        dd = np.minimum(dd, n - dd)
        inside |= (dd * dd).sum(1) < r * r
    return inside


def _build(mu, case):
    res, form, law = case['res'], case['form'], case['law']
    d = len(res)
    cell = mu.Cell(res, [1.0] * d, form, allow_even=True)
    inside = _inclusions(res, case.get('seed', 1))
    mat = mu.material
    if law == 'le1':
        getattr(mat, 'MaterialLinearElastic1_%dd' % d).make(cell, 'incl', 210e9, .3).add_pixels(inside)
        getattr(mat, 'MaterialLinearElastic1_%dd' % d).make(cell, 'matrix', 3e9, .3).add_pixels(~inside)
    elif law == 'le2':
        getattr(mat, 'MaterialLinearElastic1_%dd' % d).make(cell, 'incl', 210e9, .3).add_pixels(inside)
        eig = np.zeros((int((~inside).sum()), d * d))
        eig[:, 0] = 1e-3
        getattr(mat, 'MaterialLinearElastic2_%dd' % d).make(cell, 'matrix', 3e9, .3).add_pixels(
            np.flatnonzero(~inside), eig)
    elif law == 'le4':
        rng = np.random.default_rng(5)
        npx = int(np.prod(res))
        E = np.exp(rng.normal(np.log(1e9), 0.8, npx))
        nu = rng.uniform(0.2, 0.4, npx)
        getattr(mat, 'MaterialLinearElastic4_%dd' % d).make(cell, 'm').add_pixels(np.arange(npx), E, nu)
    elif law == 'hep1':
        mat.MaterialHyperElastoPlastic1_3d.make(cell, 'a', 70e9, .33, 1e8, 5e8).add_pixels(inside)
        mat.MaterialHyperElastoPlastic1_3d.make(cell, 'b', 200e9, .3, 2e8, 1e9).add_pixels(~inside)
    elif law == 'hep1+le1':
        mat.MaterialHyperElastoPlastic1_3d.make(cell, 'plastic', 70e9, .33, 1e8, 5e8).add_pixels(inside)
        mat.MaterialLinearElastic1_3d.make(cell, 'matrix', 200e9, .3).add_pixels(~inside)
    cell.initialise()
    return cell


CASES = {
    'finite_le1_32c': dict(res=[32, 32, 32], form=0, law='le1'),          # S rebuilt from F - I
    'finite_le2_32c': dict(res=[32, 32, 32], form=0, law='le2'),          # stored S (eigenstrain)
    'small_le4_32c': dict(res=[32, 32, 32], form=1, law='le4'),           # small-strain Green, 9 components
    'finite_le1_2d': dict(res=[128, 64], form=0, law='le1'),              # 2-D: last axis 64, Green 128
    'small_le1_2d': dict(res=[64, 256], form=1, law='le1'),               # 2-D: last axis 256
    'finite_le1_16x32x256': dict(res=[16, 32, 256], form=0, law='le1'),   # lengths 16 / 32 / 256
    'finite_le1_256x16x16': dict(res=[256, 16, 16], form=0, law='le1'),   # Green over 256
}


def _hom(r, d):
    return r.stress.reshape(-1, d, d).mean(0)


@pytest.mark.parametrize('name', sorted(CASES))
def test_mixed_matches_fp64_on_register_paths(mu, name):
    case = CASES[name]
    d = len(case['res'])
    load = np.zeros((d, d))
    load[0, 0] = 0.01
    if case['form'] == 1:
        load[0, 1] = load[1, 0] = 0.004
    steps = [load]
    out = {}
    for prec in ('fp64', 'mixed'):
        cell = _build(mu, case)
        rs = mu.solvers.newton_cg(cell, steps, mu.solvers.SolverCG(cell, 1e-8, 3000, precision=prec), 1e-8, 0.0)
        assert all(r.success for r in rs), (prec, [r.message for r in rs])
        out[prec] = rs
    for a, b in zip(out['mixed'], out['fp64']):
        ha, hb = _hom(a, d), _hom(b, d)
        err = np.linalg.norm(ha - hb) / np.linalg.norm(hb)
        assert err < 1e-6, (name, err)


def test_fp64_projection_idempotent_register_lengths(mu):
    """Projection of a compatible field is the identity, at register lengths, in the
    FP64 engine (middle-axis and Green register kernels in FP64)."""
    for res in ([16, 32, 64], [128, 16, 16], [256, 16, 32]):
        proj = mu.fft.ProjectionFiniteStrainFast_3d(res, [1., 1., 1.], allow_even=True)
        rng = np.random.default_rng(0)
        f = rng.normal(size=(9, int(np.prod(res))))
        g1 = proj.apply_projection(f)
        g2 = proj.apply_projection(g1)
        assert np.abs(g2 - g1).max() <= 1e-12 * np.abs(g1).max()


OPERATOR_CASES = {
    'finite_le1_32c': dict(res=[32, 32, 32], form=0, law='le1'),
    'finite_le2_32c': dict(res=[32, 32, 32], form=0, law='le2'),
    'small_le4_32c': dict(res=[32, 32, 32], form=1, law='le4'),
    'finite_hep1_16c': dict(res=[16, 16, 16], form=0, law='hep1'),         # Kirchhoff tangent K'
    'finite_hep1_le1_16c': dict(res=[16, 16, 16], form=0, law='hep1+le1'),  # per-pixel tangent kind
    'finite_le1_2d': dict(res=[128, 64], form=0, law='le1'),
    'small_le1_2d_256': dict(res=[64, 256], form=1, law='le1'),
    'finite_le1_16x32x256': dict(res=[16, 32, 256], form=0, law='le1'),
    'finite_le1_256x16x16': dict(res=[256, 16, 16], form=0, law='le1'),
    'finite_le1_generic': dict(res=[15, 9, 10], form=0, law='le1'),         # generic (non power-of-two) passes
    'small_le1_generic': dict(res=[24, 20, 18], form=1, law='le1'),
    'finite_hep1_le1_generic': dict(res=[9, 7, 12], form=0, law='hep1+le1'),
    # qualification rules of the TMA-fed kernels: an odd row count keeps the register
    # last-axis inverse; an odd k-plane count keeps the register Green kernel
    'finite_le1_odd_rows': dict(res=[9, 7, 16], form=0, law='le1'),
    'finite_le1_odd_planes': dict(res=[16, 7, 32], form=0, law='le1'),
    'small_le1_tma_both': dict(res=[32, 16, 32], form=1, law='le1'),
}


@pytest.mark.parametrize('name', sorted(OPERATOR_CASES))
def test_fp32_cg_operator_matches_fp64(mu, name):
    """One application of the CG operator G(K:dF) at an evaluated tangent: the FP64
    CG kernels agree with Cell::evaluate_projected_directional_stiffness to 1e-12,
    and the FP32 operator of the mixed solver with them to 1e-5 (relative, 2-norm)."""
    case = OPERATOR_CASES[name]
    d = len(case['res'])
    cell = _build(mu, case)
    n = cell.nb_pixels
    rng = np.random.default_rng(11)
    F = np.tile(np.eye(d).reshape(-1, 1), (1, n)) + 0.01 * rng.normal(size=(d * d, n))
    if case['form'] == 1:
        F = 0.01 * rng.normal(size=(d * d, n))
        F = 0.5 * (F + F.reshape(d, d, n).transpose(1, 0, 2).reshape(d * d, n))
    cell.evaluate_stress_tangent(F)
    dF = rng.normal(size=(d * d, n))
    ref = cell.directional_stiffness(dF)
    op64 = cell.cg_operator(dF, 'fp64')
    op32 = cell.cg_operator(dF, 'mixed')
    nrm = np.linalg.norm(ref)
    assert np.linalg.norm(op64 - ref) <= 1e-12 * nrm
    assert np.linalg.norm(op32 - ref) <= 1e-5 * nrm, np.linalg.norm(op32 - ref) / nrm
