"""The oracle's consistent elasto-plastic tangent (an extension of the reference,
which converts the Kirchhoff tangent with the j-independent K' of
materials_toolbox.hh:374-410): central finite differences of P(F) reproduce
K = dP/dF, K is major-symmetric, and with the backtracking line search the oracle's
newton_cg solves the two-phase Voronoi ramp that the reference method does not."""
import numpy as np

from oracle import muspectre_oracle as o


def _material(E=200e9, nu=0.3, tau_y0=200e6, H=1e9, n=6):
    m = o.MaterialHyperElastoPlastic1('m', 3, E, nu, tau_y0, H, tangent='consistent')
    for i in range(n):
        m.add_pixel(i)
    m.initialise()
    return m


def _fd_error(mat, F, h=1e-7):
    P, K = mat.evaluate(F, o.FINITE_STRAIN)
    err = 0.0
    for j in range(3):
        for n in range(3):
            E = np.zeros((3, 3))
            E[j, n] = h
            Pp, _ = mat.evaluate(F + E, o.FINITE_STRAIN)
            Pm, _ = mat.evaluate(F - E, o.FINITE_STRAIN)
            err = max(err, np.abs((Pp - Pm) / (2 * h) - K[:, :, :, j, n]).max() / np.abs(K).max())
    sym = np.abs(K - K.transpose(0, 3, 4, 1, 2)).max() / np.abs(K).max()
    return err, sym


def test_consistent_tangent_finite_differences():
    rng = np.random.default_rng(0)
    for tau_y0 in (200e6, 1e12):  # plastic, then elastic
        mat = _material(tau_y0=tau_y0)
        F = np.eye(3) + 0.004 * rng.standard_normal((6, 3, 3))
        F[0] = np.diag([1.003, 1.0, 1.0])  # repeated eigenvalues of be*
        mat.evaluate(F, o.FINITE_STRAIN)
        mat.save_history_variables()
        for _ in range(2):  # with history: F_prev, be_old != I
            F = F + 0.003 * rng.standard_normal((6, 3, 3))
            err, sym = _fd_error(mat, F)
            assert err < 1e-7, err
            assert sym < 1e-12, sym
            plastic = mat.stress_n_internals(F)[4]
            assert plastic.all() if tau_y0 < 1e9 else not plastic.any()
            mat.save_history_variables()


def test_consistent_mode_state_update_is_idempotent():
    """A repeated evaluation (a line-search trial) leaves the same εp: the consistent
    mode writes εp.cur = εp.old + Δγ instead of adding to stale contents."""
    mat = _material()
    F = np.broadcast_to(np.diag([1.004, 0.999, 0.999]), (6, 3, 3)).copy()
    mat.evaluate(F, o.FINITE_STRAIN)
    e1 = mat._cur(mat.eps_p).copy()
    mat.evaluate(F, o.FINITE_STRAIN)
    assert np.array_equal(mat._cur(mat.eps_p), e1) and e1.max() > 0


def _voronoi_cell(w):
    oc = o.Cell(w['res'], w['lengths'], o.FINITE_STRAIN)
    for ph, mask in (('A', w['phaseA']), ('B', ~w['phaseA'])):
        p = w[ph]
        m = oc.add_material(o.MaterialHyperElastoPlastic1(ph, 3, p['E'], p['nu'], p['tau_y0'], p['H'],
                                                          tangent='consistent'))
        m.pixels = list(np.flatnonzero(mask))
    return oc


def test_projected_operator_finite_differences():
    """G(K:dF) is the derivative of the projected residual G(P(F)) on a heterogeneous
    two-phase cell (both phases plastic)."""
    from muspectre_gb300 import workloads
    w = workloads.voronoi(n=7, nseeds=5, nsteps=20)
    oc = _voronoi_cell(w)
    oc.initialise()
    rng = np.random.default_rng(1)
    F0 = np.broadcast_to(np.eye(3) + w['steps'][0], (oc.n_px, 3, 3)).copy() + 1e-3 * rng.standard_normal((oc.n_px, 3, 3))
    oc.F = o.t2_to_vec(F0)
    oc.evaluate_stress_tangent()
    dF = oc.apply_projection(rng.standard_normal(oc.nb_dof()))
    Jd = oc.directional_stiffness(dF)
    h = 1e-7
    oc.F = o.t2_to_vec(F0) + h * dF
    Pp, _ = oc.evaluate_stress_tangent()
    oc.F = o.t2_to_vec(F0) - h * dF
    Pm, _ = oc.evaluate_stress_tangent()
    fd = oc.apply_projection((Pp - Pm) / (2 * h))
    assert np.linalg.norm(fd - Jd) < 1e-7 * np.linalg.norm(Jd)


def test_voronoi_ramp_solves_with_line_search():
    """The 64³ elasto-plastic workload's material and load path on a 9³ Voronoi of 8
    grains, first 4 of the 20 steps: every step converges with the line search; without
    it the first step's Newton iterates diverge (the CG gives up)."""
    from muspectre_gb300 import workloads
    w = workloads.voronoi(n=9, nseeds=8, nsteps=20)
    oc = _voronoi_cell(w)
    rs = o.newton_cg(oc, w['steps'][:4], o.SolverCG(oc, 1e-8, 3000), 1e-6, 0.0, 0, line_search=True)
    assert all(r.success for r in rs)
    s11 = [o.homogenised(r.stress, 3)[0, 0] for r in rs]
    assert all(b > a for a, b in zip(s11, s11[1:]))
    oc2 = _voronoi_cell(w)
    try:
        o.newton_cg(oc2, w['steps'][:1], o.SolverCG(oc2, 1e-8, 2000), 1e-6, 0.0, 0)
        diverged = False
    except o.ConvergenceError:
        diverged = True
    assert diverged


def test_consistent_mode_at_identity_is_finite():
    """At F = I the trial Kirchhoff stress has no deviator: the reference's flow
    direction is 0/0 (NaN); the consistent mode takes N = 0 there, so P = 0 and the
    tangent is the elastic one (what de_geus evaluates first)."""
    mat = _material()
    F = np.broadcast_to(np.eye(3), (6, 3, 3)).copy()
    P, K = mat.evaluate(F, o.FINITE_STRAIN)
    assert np.all(P == 0.0)
    assert np.all(np.isfinite(K))
    lam, mu = mat.lam, mat.mu
    # the elastic tangent at F = I: lam tr(dF) I + mu (dF + dF^T)
    for j in range(3):
        for n in range(3):
            dF = np.zeros((3, 3))
            dF[j, n] = 1.0
            ref = lam * np.trace(dF) * np.eye(3) + mu * (dF + dF.T)
            assert np.allclose(K[0, :, :, j, n], ref, rtol=1e-12, atol=1e-3)
