"""Seeded synthetic microstructures for the benchmark configurations.

All generators are pure NumPy (PCG64 via ``default_rng``); the same arrays feed the
GPU path and the CPU oracle.  Pixel centres sit at integer coordinates; inclusions
use the periodic minimum-image distance.

* ``readme_disc``   51×51 small strain, LE1 hard disc (E 10e9) in a soft matrix
                    (E 70e9), ν .33, lengths 7×5, Δε = sym([[0,0],[0,.03]]).
* ``spheres``       n³ finite strain, LE1: ``nsph`` spheres, centres U[0,n)³,
                    radii U[4,12]·n/128 voxels, E 210e9 inside / 3e9 outside, ν .3,
                    ΔF = 0.02 e1⊗e1 (default n = 128, 40 spheres).
* ``lognormal``     n³ small strain, LE4: E = exp(N(ln 1e9, 0.8)), ν ~ U[.2, .4],
                    six unit symmetric load cases.
* ``voronoi``       n³ finite strain, two HEP1 phases on a periodic Voronoi of
                    ``nseeds`` grains, F11 ramped to 1.05 in ``nsteps`` steps.
"""
from __future__ import annotations

import numpy as np


def grid_coords(res):
    return np.stack(np.meshgrid(*[np.arange(n) for n in res], indexing='ij'), -1).reshape(-1, len(res))


def readme_disc():
    res = [51, 51]
    center = np.array([r // 2 for r in res])
    hard = np.linalg.norm(center - grid_coords(res), axis=1) < res[0] // 5
    Del0 = np.array([[0., 0.], [0., 0.03]])
    Del0 = 0.5 * (Del0 + Del0.T)
    return dict(res=res, lengths=[7., 5.], hard=hard, E_hard=10e9, E_soft=70e9, nu=0.33, load=Del0,
                cg_tol=1e-8, maxiter=401, newton_tol=1e-5, equil_tol=2.0)


def spheres(n=128, nsph=40, seed=2024):
    rng = np.random.default_rng(seed)
    res = [n, n, n]
    pts = grid_coords(res).astype(np.float64)
    inside = np.zeros(n ** 3, dtype=bool)
    scale = n / 128.0
    for _ in range(nsph):
        c = rng.uniform(0, n, 3)
        r = rng.uniform(4, 12) * scale
        d = np.abs(pts - c)
        d = np.minimum(d, n - d)
        inside |= (d * d).sum(1) < r * r
    load = np.zeros((3, 3))
    load[0, 0] = 0.02
    return dict(res=res, lengths=[1., 1., 1.], inside=inside, E_incl=210e9, E_matrix=3e9, nu=0.3, load=load,
                cg_tol=1e-8, maxiter=4000, newton_tol=1e-6, equil_tol=0.0, seed=seed)


def lognormal(n=256, seed=7):
    rng = np.random.default_rng(seed)
    npx = n ** 3
    E = np.exp(rng.normal(np.log(1e9), 0.8, npx))
    nu = rng.uniform(0.2, 0.4, npx)
    loads = []
    for (i, j) in ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)):
        e = np.zeros((3, 3))
        e[i, j] += 0.5
        e[j, i] += 0.5
        loads.append(e)
    return dict(res=[n, n, n], lengths=[1., 1., 1.], E=E, nu=nu, loads=loads, cg_tol=1e-7, maxiter=4000,
                newton_tol=1e-6, equil_tol=0.0, seed=seed)


def voronoi(n=64, nseeds=32, nsteps=20, seed=11):
    rng = np.random.default_rng(seed)
    res = [n, n, n]
    seeds = rng.uniform(0, n, (nseeds, 3))
    phase_of_grain = rng.random(nseeds) < 0.5
    pts = grid_coords(res).astype(np.float64)
    best = np.full(n ** 3, np.inf)
    grain = np.zeros(n ** 3, dtype=np.int64)
    for g, s in enumerate(seeds):
        d = np.abs(pts - s)
        d = np.minimum(d, n - d)
        dd = (d * d).sum(1)
        closer = dd < best
        best[closer] = dd[closer]
        grain[closer] = g
    phaseA = phase_of_grain[grain]
    steps = []
    for k in range(1, nsteps + 1):
        D = np.zeros((3, 3))
        D[0, 0] = 0.05 * k / nsteps
        steps.append(D)
    return dict(res=res, lengths=[1., 1., 1.], phaseA=phaseA,
                A=dict(E=200e9, nu=0.3, tau_y0=200e6, H=1e9), B=dict(E=70e9, nu=0.33, tau_y0=100e6, H=0.5e9),
                steps=steps, cg_tol=1e-8, maxiter=4000, newton_tol=1e-6, equil_tol=0.0, seed=seed)


def build_spheres_cell(mu, w, allow_even=True, flags=None):
    """The GPU cell; ``flags`` = FFT_PlanFlags (default: measure, i.e. autotuned launch
    shapes, as the reference's demonstrators plan with FFTW_MEASURE)."""
    cell = mu.Cell(w['res'], w['lengths'], mu.Formulation.finite_strain, allow_even=allow_even)
    mu.material.MaterialLinearElastic1_3d.make(cell, 'inclusions', w['E_incl'], w['nu']).add_pixels(w['inside'])
    mu.material.MaterialLinearElastic1_3d.make(cell, 'matrix', w['E_matrix'], w['nu']).add_pixels(~w['inside'])
    cell.initialise(mu.FFT_PlanFlags.measure if flags is None else flags)
    return cell


def build_spheres_oracle(o, w, allow_even=True):
    cell = o.Cell(w['res'], w['lengths'], o.FINITE_STRAIN, allow_even=allow_even)
    for name, E, mask in (('inclusions', w['E_incl'], w['inside']), ('matrix', w['E_matrix'], ~w['inside'])):
        m = cell.add_material(o.MaterialLinearElastic1(name, 3, E, w['nu']))
        m.pixels = list(np.flatnonzero(mask))
    cell.initialise()
    return cell
