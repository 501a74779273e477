"""Continuous-batching request server for homogenization solves.

Requests (one RVE each: grid, formulation, microstructure, load path) arrive over
time.  ``Server`` admits a request when a lane is free and its estimated device
footprint fits the HBM budget next to everything already admitted; requests of the
same shape that are waiting together are taken as one batch
(``batch.BatchSolver``: one launch per CG pass for all of them).  Each lane is a host
thread whose cells run on their own CUDA streams, so admitted requests overlap on
the device; the C library releases the GIL inside every call.  Fields and plastic
state stay on the device for all load steps of a request; memory returns to the
budget when the request completes.  Latency = completion - arrival.

Every request is computed by the same deterministic kernels whether it runs alone
or in the mix (per-request reductions in a fixed order), which
``tests/test_gpu_serving.py`` checks.
"""
from __future__ import annotations

import heapq
import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import batch as _batch
from . import solvers as _solvers
from .cell import Cell, Formulation


@dataclass
class Request:
    """One homogenization solve.  ``phase``: material index per pixel (row-major);
    ``materials``: per index (law, params) with law 'le1' (E, nu), 'le4' (per-pixel
    arrays E, nu over the phase's pixels) or 'hep1' (E, nu, tau_y0, H)."""
    rid: int
    res: List[int]
    formulation: int
    phase: np.ndarray
    materials: List[tuple]
    steps: List[np.ndarray]
    arrival: float = 0.0
    lengths: Optional[List[float]] = None

    def shape_key(self):
        kinds = tuple(sorted({m[0] == 'hep1' for m in self.materials}))
        return (tuple(self.res), int(self.formulation), kinds, len(self.steps))


@dataclass
class Result:
    rid: int
    success: bool
    message: str
    nb_it: int
    nb_fev: int
    stress: np.ndarray          # homogenised PK1 / Cauchy stress of the last step (D×D)
    latency: float
    batched_with: int = 1


def estimate_bytes(res, formulation, has_hep, precision='mixed'):
    """Device memory of one admitted request (fields, spectra, tangent data, CG
    vectors, state), as the library allocates it."""
    npx = int(np.prod(res))
    d = len(res)
    d2 = d * d
    nk = npx // res[-1] * (res[-1] // 2 + 1)
    b = 3 * d2 * npx * 8 + d2 * nk * 16 + 2 * d2 * npx * 8 + npx * (1 + 16) + (1 << 20)
    if formulation == Formulation.finite_strain:
        b += 2 * d2 * npx * 8
    if has_hep:
        b += 38 * npx * 8 + d2 * d * npx * 8
    if precision == 'mixed':
        b += npx * 8 + d2 * nk * 8 + 4 * d2 * npx * 4
        if formulation == Formulation.finite_strain:
            b += 2 * d2 * npx * 4
        if has_hep:
            b += d2 * d * npx * 4
    else:
        b += 4 * d2 * npx * 8
    return int(b)


def build_cell(req, flags=0):
    import muspectre_gb300 as mu
    d = len(req.res)
    cell = Cell(req.res, req.lengths or [1.0] * d, Formulation(req.formulation), allow_even=True)
    for k, (law, params) in enumerate(req.materials):
        mask = req.phase == k
        if not np.any(mask):
            continue
        if law == 'le1':
            getattr(mu.material, 'MaterialLinearElastic1_%dd' % d).make(cell, 'm%d' % k, *params).add_pixels(mask)
        elif law == 'le4':
            E, nu = params
            getattr(mu.material, 'MaterialLinearElastic4_%dd' % d).make(cell, 'm%d' % k).add_pixels(
                np.flatnonzero(mask), E, nu)
        elif law == 'hep1':
            getattr(mu.material, 'MaterialHyperElastoPlastic1_%dd' % d).make(cell, 'm%d' % k, *params).add_pixels(mask)
        else:
            raise ValueError('unknown law ' + law)
    cell.initialise(flags)
    return cell


def solve_alone(req, tol=1e-8, maxiter=2000, newton_tol=1e-6, precision='mixed'):
    """The reference point of the serving test: the request on its own."""
    cell = build_cell(req)
    d = len(req.res)
    try:
        rs = _solvers.newton_cg(cell, list(req.steps), _solvers.SolverCG(cell, tol, maxiter, precision=precision),
                                newton_tol, 0.0)
        r = rs[-1]
        return Result(req.rid, r.success, r.message, r.nb_it, r.nb_fev,
                      r.stress.reshape(-1, d, d).transpose(0, 2, 1).mean(0), 0.0)
    except _solvers.ConvergenceError as e:
        return Result(req.rid, False, str(e)[:63], 0, 0, np.full((d, d), np.nan), 0.0)


class Server:
    """Admission by HBM budget, lanes on separate streams, same-shape batching."""

    def __init__(self, hbm_budget_bytes, lanes=4, max_batch=8, precision='mixed', tol=1e-8, maxiter=2000,
                 newton_tol=1e-6):
        self.budget = int(hbm_budget_bytes)
        self.lanes = int(lanes)
        self.max_batch = int(max_batch)
        self.precision = precision
        self.tol, self.maxiter, self.newton_tol = tol, maxiter, newton_tol
        self.in_use = 0
        self.peak_in_use = 0
        self.queue: deque = deque()
        self.results: Dict[int, Result] = {}
        self.cv = threading.Condition()
        self.closed = False
        self.admitted_batches = 0
        self._threads: List[threading.Thread] = []

    # ------------------------------------------------------------------ client side
    def submit(self, req: Request):
        with self.cv:
            req.arrival = time.perf_counter()
            self.queue.append(req)
            self.cv.notify_all()

    def close(self):
        with self.cv:
            self.closed = True
            self.cv.notify_all()

    def start(self):
        for i in range(self.lanes):
            t = threading.Thread(target=self._lane, name='musg-lane-%d' % i, daemon=True)
            t.start()
            self._threads.append(t)

    def join(self):
        for t in self._threads:
            t.join()

    # ------------------------------------------------------------------ lanes
    def _footprint(self, req):
        has_hep = any(m[0] == 'hep1' for m in req.materials)
        return estimate_bytes(req.res, req.formulation, has_hep, self.precision)

    def _take(self):
        """Next admissible group: the oldest request that fits the budget, plus the
        waiting requests of the same shape that also fit (continuous batching)."""
        for i, req in enumerate(self.queue):
            fp = self._footprint(req)
            if self.in_use + fp > self.budget and self.in_use > 0:
                continue
            group = [req]
            used = fp
            key = req.shape_key()
            for other in list(self.queue)[i + 1:]:
                if len(group) >= self.max_batch:
                    break
                if other.shape_key() == key and self.in_use + used + fp <= self.budget:
                    group.append(other)
                    used += fp
            for g in group:
                self.queue.remove(g)
            self.in_use += used
            self.peak_in_use = max(self.peak_in_use, self.in_use)
            return group, used
        return None, 0

    def _lane(self):
        while True:
            with self.cv:
                while True:
                    group, used = self._take()
                    if group is not None:
                        break
                    if self.closed and not self.queue:
                        return
                    self.cv.wait(0.05)
            try:
                self._run(group)
            finally:
                with self.cv:
                    self.in_use -= used
                    self.cv.notify_all()

    def _run(self, group):
        d = len(group[0].res)
        cells = [build_cell(r) for r in group]
        res = []
        if len(group) == 1:
            req = group[0]
            try:
                rs = _solvers.newton_cg(cells[0], list(req.steps),
                                        _solvers.SolverCG(cells[0], self.tol, self.maxiter, precision=self.precision),
                                        self.newton_tol, 0.0)
                res.append(rs[-1])
            except _solvers.ConvergenceError as e:
                res.append(_solvers.OptimizeResult(np.empty((0, 1)), np.empty((0, 1)), False, 0, str(e)[:63], 0, 0))
        else:
            steps = np.stack([np.stack(r.steps) for r in group])
            bs = _batch.BatchSolver(cells, self.tol, self.maxiter, precision=self.precision)
            out = bs.newton_cg(steps, self.newton_tol, 0.0)
            res = [o[-1] for o in out]
            self.admitted_batches += 1
        now = time.perf_counter()
        for req, r in zip(group, res):
            st = r.stress.reshape(-1, d, d).transpose(0, 2, 1).mean(0) if r.stress.size else np.full((d, d), np.nan)
            result = Result(req.rid, r.success, r.message, r.nb_it, r.nb_fev, st, now - req.arrival, len(group))
            with self.cv:
                self.results[req.rid] = result


def c5_request(rid, seed, small=False):
    """BASELINE config 5 request drawn from its own seed: 2-D (64..1024, 2/3/5-smooth)
    or 3-D (32..160, 2/3/5-smooth); small or finite strain; LE1/LE4, or HEP1 with 1-10
    load steps (finite strain only); 1-60 spheres; E ~ U[1e9, 300e9], nu ~ U[0.2, 0.4];
    symmetric macro strain entries ~ U[-0.02, 0.02].  ``small`` caps the sizes (tests)."""
    rng = np.random.default_rng(seed)
    smooth = lambda lo, hi: [n for n in range(lo, hi + 1) if _smooth235(n)]
    d = 2 if rng.random() < 0.5 else 3
    if d == 2:
        sizes = smooth(64, 160 if small else 1024)
    else:
        sizes = smooth(32, 40 if small else 160)
    n = int(rng.choice(sizes))
    res = [n] * d
    hep = rng.random() < 0.2
    form = Formulation.finite_strain if (hep or rng.random() < 0.5) else Formulation.small_strain
    nsph = int(rng.integers(1, 61))
    pts = np.stack(np.meshgrid(*[np.arange(n)] * d, indexing='ij'), -1).reshape(-1, d).astype(np.float64)
    inside = np.zeros(n ** d, dtype=bool)
    for _ in range(nsph):
        c = rng.uniform(0, n, d)
        r = rng.uniform(0.03, 0.15) * n
        dd = np.abs(pts - c)
        dd = np.minimum(dd, n - dd)
        inside |= (dd * dd).sum(1) < r * r
    phase = inside.astype(np.int64)
    mats = []
    for k in range(2):
        E, nu = float(rng.uniform(1e9, 300e9)), float(rng.uniform(0.2, 0.4))
        if hep:
            mats.append(('hep1', (E, nu, E * 1e-3, E * 5e-3)))
        elif rng.random() < 0.5:
            mats.append(('le1', (E, nu)))
        else:
            cnt = int((phase == k).sum())
            mats.append(('le4', (rng.uniform(0.5, 1.5, cnt) * E, np.full(cnt, nu))))
    eps = rng.uniform(-0.02, 0.02, (d, d))
    eps = 0.5 * (eps + eps.T)
    nsteps = int(rng.integers(1, 11)) if hep else 1
    steps = [eps * (k + 1) / nsteps for k in range(nsteps)]
    return Request(rid, res, int(form), phase, mats, steps)


def _smooth235(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def run_stream(requests, rate_hz, server):
    """Feed requests with Poisson arrivals (exponential gaps at rate_hz), wait for all."""
    rng = np.random.default_rng(12345)
    server.start()
    t0 = time.perf_counter()
    for req in requests:
        server.submit(req)
        if rate_hz > 0:
            time.sleep(float(rng.exponential(1.0 / rate_hz)))
    server.close()
    server.join()
    wall = time.perf_counter() - t0
    lat = np.array([r.latency for r in server.results.values()])
    ok = sum(r.success for r in server.results.values())
    return {'requests': len(requests), 'succeeded': int(ok), 'wall_s': wall, 'solves_per_s': len(requests) / wall,
            'p50_ms': float(np.percentile(lat, 50) * 1e3), 'p99_ms': float(np.percentile(lat, 99) * 1e3),
            'peak_hbm_bytes': server.peak_in_use, 'batches': server.admitted_batches}
