"""Benchmark: RVE solves/s of the Newton-CG homogenization on GB300.

Workload (one "step" = one complete newton_cg solve): 128³ voxels, finite strain,
MaterialLinearElastic1 with 40 seeded spherical inclusions (radii U[4,12] voxels,
periodic wrap; E 210e9 in the spheres, 3e9 in the matrix, ν .3), applied
F = I + 0.02 e1⊗e1, CG tol 1e-8, Newton tol 1e-6.  128 is even, so the cell uses
the even-grid extension (Green operator zero at Nyquist k-points); the reference
rejects even grids.

value   mixed precision (FP32 inner CG / FFT / projection / tangent, FP64 Newton
        level) solves/s with the microstructure resident in HBM (every field on the
        device; 151 MB per field > 129 MB L2, so no L2 flush is needed between steps)
e2e     the same solve through the public API from host buffers: cell construction
        (host -> device upload of the microstructure), newton_cg, and the homogenised
        stress read back (device -> host), wall clock
fp64    the plain FP64 method on the same input, with the homogenised-stress error
        of the mixed result against it
roofline   the dominant kernel of one CG iteration, algorithmic bytes / CUDA-event
        duration against the measured HBM copy bandwidth
cpu_baseline  the NumPy/SciPy oracle (the reference's algorithm restated on the CPU)
        on a bounded sample of the same workload, all host cores for its FFTs

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Newton steps and CG iterations of a complete FP64 oracle solve of the 128^3 workload
# (the reference's algorithm on the CPU), measured with
#   python bench.py --impl reference --ref-full --steps 1 --warmup 0
# The reference arm and the CPU baseline time a bounded sample (the Newton-level work
# once, REF_SAMPLE_CG_ITERS CG iterations per step) and scale it by these counts.
REF_NEWTON_STEPS = 4
REF_CG_ITERS = 530
REF_SAMPLE_CG_ITERS = 8
# at or below this resolution the reference arm times complete oracle solves instead
REF_FULL_SOLVE_MAX_N = 48


def metric_name(n):
    """The metric both arms report (the driver divides one arm's value by the other's)."""
    return 'RVE solves/s (Newton-CG, %d^3 finite-strain LE1, 40 spheres)' % n


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--n', type=int, default=128)
    ap.add_argument('--fp64-steps', type=int, default=2)
    ap.add_argument('--e2e-steps', type=int, default=2)
    ap.add_argument('--cpu-cg-iters', type=int, default=REF_SAMPLE_CG_ITERS)
    ap.add_argument('--ref-full', action='store_true',
                    help='reference arm: complete oracle solves at any resolution (prints their counts)')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-extra', action='store_true', help='skip the other workloads (configs) of the metric')
    ap.add_argument('--configs', default='readme,lognormal,voronoi,serving',
                    help='the other workloads to run (comma list of readme, lognormal, voronoi, serving)')
    ap.add_argument('--only', default='all', choices=['all', 'mixed'],
                    help="'mixed': the mixed-precision solves only (for profiler launch lists)")
    return ap.parse_args()


def dist_init(args):
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    FIELDS = 'index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,' \
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,' \
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap'

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '100'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(',')]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower().startswith('active'):
                        reasons.add(nm)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled'], 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(mx), 'reasons': sorted(reasons),
                'samples': len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def algorithmic_bytes(name, npx, nk, d2, s, tm):
    """Bytes one launch of a CG-iteration kernel must move (per RHS)."""
    u = npx * d2 * s        # one real field
    spec = nk * d2 * 2 * s  # one half spectrum
    return {
        'last_axis_fwd_tangent': 3 * u + tm * npx + spec,  # r, p_old -> p; tangent data; spectrum out
        'axis1_fwd': 2 * spec,
        'green_axis0': 2 * spec,
        'axis1_inv': 2 * spec,
        'last_axis_inv_dot': spec + 2 * u,                 # spectrum in; p in; Ap out
        'cg_update': 6 * u,                                # x, p, r, Ap in; x, r out
        'last_axis_fwd_tangent_alpha': 3 * u + tm * npx + spec,  # the same, and p.(K:p) -> alpha
        'cg_update_x': 3 * u,                              # x, p in; x out
        'last_axis_inv_update_r': spec + 2 * u,            # spectrum, r in; r out
    }.get(name, 0)


def fp64_flops(name, npx, nk, res, d2=9):
    """Floating-point operations of one launch of an FP64 CG-iteration kernel (finite-strain
    LE1 tangent), counted as 5 m log2 m per complex transform of length m (two real rows
    share one; 2 more per real entry to unpack), about 200 per pixel for dP = K:dF from F
    and S, 100 per k-point for the Green operator of a row triple, 2 per vector entry
    per axpy or dot."""
    L, n1, n0 = res[2], res[1], res[0]
    last = d2 * (2.5 * np.log2(L) + 2.0)
    return {
        'last_axis_fwd_tangent': npx * (last + 200 + 2 * d2),
        'axis1_fwd': nk * d2 * 5 * np.log2(n1),
        'green_axis0': nk * (d2 * 10 * np.log2(n0) + 100),
        'axis1_inv': nk * d2 * 5 * np.log2(n1),
        'last_axis_inv_dot': npx * (last + 2 * d2),
        'cg_update': npx * d2 * 6,
    }.get(name, 0.0)


def measured_traffic(kernel, n):
    """DRAM bytes (read + write) per launch of a CG-iteration kernel from the committed
    ncu capture of this workload (profiles/traffic_spheres128_mixed.json), or None."""
    path = os.path.join(ROOT, 'profiles', 'traffic_spheres128_mixed.json')
    if n != 128 or not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)['bytes_per_launch'].get(kernel)


class CpuSample:
    """The oracle (NumPy/SciPy, FP64, all host cores for its FFTs) on the full-size
    workload: the Newton-level work (one material evaluation and the residual
    projection) timed once, then CG iterations timed on demand; a solve is scaled from
    them by the FP64 method's Newton and CG counts."""

    def __init__(self, w):
        from oracle import muspectre_oracle as o
        from muspectre_gb300 import workloads
        self.o = o
        o.FFT_WORKERS = os.cpu_count() or 1
        self.cell = workloads.build_spheres_oracle(o, w)
        self.res = w['res']
        d = 3
        F = np.broadcast_to(np.eye(d) + w['load'], (self.cell.n_px, d, d)).copy()
        self.cell.F = o.t2_to_vec(F)
        t0 = time.perf_counter()
        P, _ = self.cell.evaluate_stress_tangent()
        self.rhs = -self.cell.apply_projection(P)
        self.t_newton = time.perf_counter() - t0

    def cg_iteration_seconds(self, nit=1):
        solver = self.o.SolverCG(self.cell, 0.0, nit)
        t0 = time.perf_counter()
        try:
            solver.solve(self.rhs)
        except self.o.ConvergenceError:
            pass  # tol 0: runs exactly nit iterations
        return (time.perf_counter() - t0) / max(nit, 1)

    def describe(self, t_cg, newton_steps, cg_iters, nit):
        t_solve = newton_steps * self.t_newton + cg_iters * t_cg
        return {'solves_per_s': 1.0 / t_solve, 'pxit_per_s': self.cell.n_px / t_cg, 't_cg_iter_s': t_cg,
                't_newton_step_s': self.t_newton, 'cores': self.o.FFT_WORKERS,
                'sample': 'material evaluation + residual projection once and %d CG iteration(s) at %d^3 (FP64), '
                          'scaled to %d Newton steps and %d CG iterations per solve'
                          % (nit, self.res[0], newton_steps, cg_iters)}


def cpu_baseline(w, nit):
    """One bounded CPU sample of the workload (see CpuSample), scaled by the oracle's
    own Newton and CG counts of a complete solve."""
    smp = CpuSample(w)
    return smp.describe(smp.cg_iteration_seconds(nit), REF_NEWTON_STEPS, REF_CG_ITERS, nit)


def hom_err(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def readme_config(mu, workloads):
    """README example (51x51 small strain), FP64: the reference's own CPU-runnable case."""
    import torch
    w = workloads.readme_disc()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cell = mu.SystemFactory(w['res'], w['lengths'], mu.Formulation.small_strain)
        mu.material.MaterialLinearElastic1_2d.make(cell, 'hard', w['E_hard'], w['nu']).add_pixels(w['hard'])
        mu.material.MaterialLinearElastic1_2d.make(cell, 'soft', w['E_soft'], w['nu']).add_pixels(~w['hard'])
        r = mu.solvers.newton_cg(cell, w['load'], mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter']),
                                 w['newton_tol'], w['equil_tol'])
        hs = cell.homogenised_stress()
        times.append(time.perf_counter() - t0)
    return {'ms_per_solve': 1e3 * statistics.median(times[1:]), 'newton_steps': r.nb_it,
            'cg_iters': r.nb_fev, 'success': bool(r.success),
            'hom_stress': [float(x) for x in hs.reshape(-1)],
            'includes': 'cell construction, upload, solve, homogenised stress'}


def lognormal_config(mu, workloads, peak, n=256, repeats=3):
    """n^3 small-strain LE4 (lognormal E), six unit load cases batched as right-hand
    sides of one microstructure (one launch per CG pass for all six).  Mixed precision:
    a first (untimed) solve captures the CUDA graphs, then the median of `repeats` warm
    solves; FP64: one batched solve of the same cells; per load case the
    homogenised-stress error of the mixed result against the FP64 one.  px.it/s counts
    pixels x CG iterations x right-hand sides; its roofline fraction uses the CG
    iteration's algorithmic bytes (16 field passes + the Lame planes per px.it, FP32),
    so the Newton-level FP64 work makes it a lower bound."""
    import torch
    w = workloads.lognormal(n)
    cells = []
    for _ in w['loads']:
        c = mu.Cell(w['res'], w['lengths'], mu.Formulation.small_strain, allow_even=True)
        mu.material.MaterialLinearElastic4_3d.make(c, 'm').add_pixels(np.arange(c.nb_pixels), w['E'], w['nu'])
        c.initialise(mu.FFT_PlanFlags.measure)
        cells.append(c)
    loads = np.stack(w['loads'])[:, None]
    npx = cells[0].nb_pixels
    bs = mu.batch.BatchSolver(cells, w['cg_tol'], w['maxiter'], precision='mixed')
    res = bs.newton_cg(loads, w['newton_tol'], w['equil_tol'], return_stress=False)  # graph capture, warm-up
    c_prev = [r[0].nb_fev for r in res]
    times, per_solve = [], []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = bs.newton_cg(loads, w['newton_tol'], w['equil_tol'], return_stress=False)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        per_solve = [r[0].nb_fev - p for r, p in zip(res, c_prev)]  # cumulative counters
        c_prev = [r[0].nb_fev for r in res]
    hm = [r[0].hom_stress for r in res]
    del bs
    b64 = mu.batch.BatchSolver(cells, w['cg_tol'], w['maxiter'], precision='fp64')
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r64 = b64.newton_cg(loads, w['newton_tol'], w['equil_tol'], return_stress=False)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    errs = [hom_err(a, b[0].hom_stress) for a, b in zip(hm, r64)]
    dt = statistics.median(times)
    pxit = npx * sum(per_solve) / dt
    bpx = 16 * 9 * 4 + 8  # FP32 fields per px.it of the fused CG iteration + lambda, mu
    return {'seconds_median': dt, 'seconds_all': times, 'rhs_solves_per_s': len(cells) / dt,
            'cg_iters_per_rhs': per_solve, 'newton_steps': [r[0].nb_it for r in res],
            'pxit_per_s': pxit, 'cg_bytes_per_pxit': bpx,
            'roofline_frac_lower_bound': pxit * bpx / (peak * 1e9),
            'success': all(r[0].success for r in res), 'fp64_seconds': t64,
            'fp64_cg_iters_per_rhs': [r[0].nb_fev for r in r64],
            'stress_rel_err_vs_fp64_per_rhs': errs, 'stress_rel_err_vs_fp64_max': max(errs),
            'includes': 'warm batched solves (graphs captured by an untimed first solve), cells resident'}


def voronoi_config(mu, workloads, n=64):
    """n^3 two-phase HyperElastoPlastic1 on a periodic Voronoi of 32 grains, F11 ramped to
    1.05 in 20 load steps with the state on the device.  The reference method
    (projector logm, j-independent Kirchhoff tangent) ends in ConvergenceError at the
    first step; solved here with the consistent tangent and newton_cg's line search
    (both opt-in extensions): FP64 return mapping, FP32 inner CG (mixed), against the
    same solve in FP64 (the homogenised-stress error at every step)."""
    import torch
    w = workloads.voronoi(n)

    def cell_for(tangent):
        c = mu.Cell(w['res'], w['lengths'], mu.Formulation.finite_strain, allow_even=True)
        for ph, mask in (('A', w['phaseA']), ('B', ~w['phaseA'])):
            p = w[ph]
            mu.material.MaterialHyperElastoPlastic1_3d.make(c, ph, p['E'], p['nu'], p['tau_y0'], p['H'],
                                                           tangent=tangent).add_pixels(mask)
        c.initialise(mu.FFT_PlanFlags.measure)
        return c

    out = {}
    c = cell_for('reference')
    try:
        mu.solvers.newton_cg(c, w['steps'], mu.solvers.SolverCG(c, w['cg_tol'], 400, precision='mixed'),
                             w['newton_tol'], w['equil_tol'], return_fields=False)
        out['reference_method_status'] = 'solved'
    except mu.ConvergenceError as e:
        out['reference_method_status'] = 'ConvergenceError: ' + str(e)[:80]
    del c
    res = {}
    for prec in ('mixed', 'fp64'):
        c = cell_for('consistent')
        s = mu.solvers.SolverCG(c, w['cg_tol'], 1000, precision=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = mu.solvers.newton_cg(c, w['steps'], s, w['newton_tol'], w['equil_tol'], return_fields=False,
                                  line_search=True)
        torch.cuda.synchronize()
        res[prec] = (time.perf_counter() - t0, rs)
        del c, s
    tm, rm = res['mixed']
    t64, r64 = res['fp64']
    errs = [hom_err(a.hom_stress, b.hom_stress) for a, b in zip(rm, r64)]
    out.update({'solves_per_s': 1.0 / tm, 'seconds': tm, 'load_steps': len(rm),
                'success': all(r.success for r in rm),
                'newton_steps_per_load_step': [r.nb_it for r in rm], 'cg_iters_total': rm[-1].nb_fev,
                'fp64_seconds': t64, 'fp64_newton_steps_per_load_step': [r.nb_it for r in r64],
                'fp64_cg_iters_total': r64[-1].nb_fev, 'speedup_vs_fp64': t64 / tm,
                'stress_rel_err_vs_fp64_max': max(errs), 'stress_rel_err_vs_fp64_last': errs[-1],
                'hom_stress_11_mpa': [float(r.hom_stress[0, 0]) / 1e6 for r in rm],
                'method': 'consistent Kirchhoff->PK1 tangent, spectral logm, Armijo line search (extensions)'})
    return out


def serving_config(mu, nreq=2000, lanes=4, max_batch=8, budget=96 << 30, sweep_n=400, sample=20,
                   window_s=75.0, sweep_window_s=20.0, sample_budget_s=45.0, sample_max_cost=96 ** 3,
                   sample_timeout_s=10.0, sweep=(0.5, 1.0, 2.0, 4.0, 8.0)):
    """The serving stream: nreq seeded requests of mixed size, formulation, law and
    load path through the continuous-batching server (mixed precision).  Capacity: all
    nreq submitted at once (open loop, far past saturation) and a measurement window
    of window_s: then the requests still waiting are cancelled and the running ones
    stopped, so the leg stays within minutes (their counts are reported; throughput
    counts succeeded requests over the wall time).  Rate sweep: Poisson arrivals at
    the `sweep` multiples of that capacity for sweep_window_s each (from the first
    sweep_n requests), each on a fresh server, ended the same way (succeeded solves/s, p50/p99
    latency of the succeeded ones).  Accuracy: a seeded sample of up to `sample`
    served requests, among those whose cost (pixels x load steps, x30 for the
    elasto-plastic law) is at most sample_max_cost (an FP64 solve takes up to ~40x the
    mixed one), solved again alone in FP64 (the plain method, whose parity with the
    oracle the tests pin; each stopped after sample_timeout_s), within
    sample_budget_s; the homogenised-stress error of
    the served mixed result against it."""
    from muspectre_gb300 import serving
    t0 = time.perf_counter()
    reqs = [serving.c5_request(i, 1000 + i) for i in range(nreq)]
    t_gen = time.perf_counter() - t0
    srv = serving.Server(budget, lanes=lanes, max_batch=max_batch, precision='mixed')
    cap = serving.run_stream(reqs, rate_hz=0, server=srv, deadline_s=window_s, stop_running=True)
    mixed = dict(srv.results)
    del srv
    progress('serving capacity window: %d succeeded, %d cancelled, %.1f s' % (cap['succeeded'], cap['cancelled'],
                                                                             cap['wall_s']))
    capacity = cap['succeeded_per_s']
    rates = sweep
    sweep = []
    for f in rates:
        s2 = serving.Server(budget, lanes=lanes, max_batch=max_batch, precision='mixed')
        st = serving.run_stream(reqs[:sweep_n], rate_hz=f * capacity, server=s2, seed=77,
                                deadline_s=sweep_window_s, stop_running=True)
        sweep.append({'offered_hz': f * capacity, 'succeeded_per_s': st['succeeded_per_s'],
                      'p50_ms': st['p50_ms_succeeded'], 'p99_ms': st['p99_ms_succeeded'],
                      'succeeded': st['succeeded'], 'cancelled': st['cancelled'], 'offered': st['offered'],
                      'stopped_running': sum(1 for r in s2.results.values() if 'while running' in r.message),
                      'wall_s': st['wall_s'], 'batches': st['batches']})
        del s2
        progress('serving sweep at %.3g/s: %.3g succeeded/s' % (f * capacity, st['succeeded_per_s']))
    rng = np.random.default_rng(7)
    order = [int(i) for i in rng.permutation(nreq)]
    errs, skipped = {}, 0
    t1 = time.perf_counter()
    for i in order:
        if len(errs) >= sample or time.perf_counter() - t1 > sample_budget_s:
            break
        m = mixed.get(i)
        if m is None or not m.success:
            continue
        rq = reqs[i]
        cost = int(np.prod(rq.res)) * len(rq.steps) * (30 if any(mm[0] == 'hep1' for mm in rq.materials) else 1)
        if cost > sample_max_cost:
            skipped += 1
            continue
        r64 = serving.solve_alone(reqs[i], precision='fp64', timeout_s=sample_timeout_s)
        if r64.success:
            errs[i] = hom_err(m.stress, r64.stress)
    laws = [sorted({m[0] for m in r.materials}) for r in reqs]
    svc = np.array([r.service for r in mixed.values() if r.success]) if mixed else np.zeros(1)
    cap.update({'arrivals': 'all %d submitted at once (open loop); after %g s the waiting ones are cancelled and '
                'the running ones stopped' % (nreq, window_s), 'lanes': lanes, 'max_batch': max_batch,
                'hbm_budget_bytes': budget, 'request_generation_s': t_gen,
                'elasto_plastic_requests': sum('hep1' in l for l in laws),
                'stopped_running': sum(1 for r in mixed.values() if 'while running' in r.message),
                'service_ms_succeeded': {'p50': float(np.percentile(svc, 50) * 1e3),
                                         'p99': float(np.percentile(svc, 99) * 1e3)},
                'rate_sweep': sweep,
                'fp64_sample': {'requests': sorted(errs), 'compared': len(errs),
                                'rule': 'seeded order, pixels x load steps (x30 elasto-plastic) <= %d'
                                        % sample_max_cost,
                                'skipped_for_cost': skipped,
                                'stress_rel_err_max': max(errs.values()) if errs else None,
                                'stress_rel_err_median': float(np.median(list(errs.values()))) if errs else None,
                                'within_1e-6': sum(e <= 1e-6 for e in errs.values())}})
    return cap


def progress(msg):
    print('[bench] ' + msg, file=sys.stderr, flush=True)


def extra_configs(mu, workloads, peak, which):
    """The other workloads of the metric, each measured on this GPU (N=1 only)."""
    out = {}
    for key, name, fn in (('readme', 'readme_51x51_fp64', lambda: readme_config(mu, workloads)),
                          ('lognormal', 'lognormal256_le4_6rhs_mixed', lambda: lognormal_config(mu, workloads, peak)),
                          ('voronoi', 'voronoi64_hep1_20steps', lambda: voronoi_config(mu, workloads)),
                          ('serving', 'serving_stream_mixed', lambda: serving_config(mu))):
        if key not in which:
            continue
        t0 = time.perf_counter()
        out[name] = fn()
        progress('%s: %.1f s' % (name, time.perf_counter() - t0))
    return out


def run_reference(args, rank, world):
    """The reference's algorithm on the host CPU (the oracle; the C++ reference needs
    Eigen and FFTW, absent here), same workload and metric.  Up to 48^3 (or with
    --ref-full) one step is one complete newton_cg solve; above, one step is a timed
    sample of REF_SAMPLE_CG_ITERS CG iterations (after the Newton-level work, timed
    once), and the value is the solve rate that sample gives at the oracle's counts."""
    if rank != 0:
        return
    from muspectre_gb300 import workloads
    w = workloads.spheres(args.n)
    vals, step_ms = [], []
    info = None
    if args.n <= REF_FULL_SOLVE_MAX_N or args.ref_full:
        from oracle import muspectre_oracle as o
        o.FFT_WORKERS = os.cpu_count() or 1
        counts = None
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            oc = workloads.build_spheres_oracle(o, w)
            r = o.newton_cg(oc, w['load'], o.SolverCG(oc, w['cg_tol'], w['maxiter']), w['newton_tol'],
                            w['equil_tol'], 0)
            dt = time.perf_counter() - t0
            counts = (r.nb_it, r.nb_fev)
            if step >= args.warmup:
                vals.append(1.0 / dt)
                step_ms.append(1e3 * dt)
        info = {'cores': o.FFT_WORKERS, 'sample': 'complete solves at %d^3 (FP64): %d Newton steps, %d CG iterations'
                % (args.n, counts[0], counts[1]), 'value_kind': 'timed complete solves'}
    else:
        smp = CpuSample(w)  # the cell and one Newton-level evaluation, timed once
        nit = args.cpu_cg_iters
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            info = smp.describe(smp.cg_iteration_seconds(nit), REF_NEWTON_STEPS, REF_CG_ITERS, nit)
            if step >= args.warmup:
                vals.append(info['solves_per_s'])
                step_ms.append(1e3 * (time.perf_counter() - t0))
        info['value_kind'] = ('scaled from a timed sample: one step = %d CG iterations; a complete solve does not fit '
                              'the run, so ms_per_step is the sample\'s time, not 1/value' % nit)
        if args.n != 128:
            info['sample'] += ' (Newton and CG counts of the 128^3 workload)'
    v = statistics.median(vals)
    line = {'impl': 'reference', 'metric': metric_name(args.n), 'value': v,
            'unit': 'solves/s', 'higher_is_better': True, 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': statistics.median(step_ms), 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic (seeded spheres, seed %d)' % w['seed'],
            'config': {'workload': 'spheres%d_finite_le1' % args.n, 'resolution': w['res'], 'nb_spheres': 40,
                       'cg_tol': w['cg_tol'], 'newton_tol': w['newton_tol'], 'formulation': 'finite_strain'},
            'value_kind': info['value_kind'],
            'cpu_baseline': {'value': v, 'unit': 'solves/s', 'cores': info['cores'], 'kind': 'port',
                             'sample': info['sample']},
            'e2e': {'value': v, 'unit': 'solves/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_init(args)
    if args.impl == 'reference':
        run_reference(args, rank, world)
        return
    import torch
    import muspectre_gb300 as mu
    from muspectre_gb300 import workloads
    torch.cuda.set_device(local)
    mu._lib.lib().musg_set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
        pg = dist
    stream = torch.cuda.Stream()

    w = workloads.spheres(args.n)
    cell = workloads.build_spheres_cell(mu, w)
    cell.set_stream(stream.cuda_stream)
    npx = cell.nb_pixels
    mixed = mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter'], precision='mixed')
    fp64 = mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter'], precision='fp64')

    def solve(solver):
        return mu.solvers.newton_cg(cell, w['load'], solver, w['newton_tol'], w['equil_tol'], return_fields=False)

    def barrier():
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    # ---------------- mixed precision, device resident (the headline)
    for _ in range(args.warmup):
        solve(mixed)
    lat = []
    c0 = mixed.get_counter()
    barrier()
    l0 = mu._lib.launch_count()
    with Clocks(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            e_a = torch.cuda.Event(enable_timing=True)
            e_b = torch.cuda.Event(enable_timing=True)
            e_a.record(stream)
            r = solve(mixed)
            e_b.record(stream)
            lat.append((e_a, e_b))
        ev1.record(stream)
        barrier()
    launches = mu._lib.launch_count() - l0
    clocks = clk.summary()
    t_ms = ev0.elapsed_time(ev1)
    lat_ms = [a.elapsed_time(b) for a, b in lat]
    cg_per_solve = (mixed.get_counter() - c0) / args.steps
    newton_mixed = r.nb_it
    # replicas: every rank solves its own RVE; all solves over the slowest rank's time
    from muspectre_gb300 import replicas
    value, t_s, _ = replicas.aggregate_throughput(args.steps, t_ms / 1000.0)
    t_ms = t_s * 1000.0
    stress_mixed = None

    # per-kernel profile of one CG iteration (mixed) + roofline
    prof = mixed.profile(5)
    peak, peak_kind = measured_peaks()
    d2 = 9
    nk = (npx // w['res'][-1]) * (w['res'][-1] // 2 + 1)
    # algorithmic tangent data per pixel: F - I (FP32) and a 1-byte material index (the
    # kernel reads per-pixel lambda, mu planes instead, 8 bytes; the operator rebuilds S)
    tm = 4 * 9 + 1
    kern = {}
    for name, ms in prof.items():
        b = algorithmic_bytes(name, npx, nk, d2, 4, tm)
        kern[name] = {'ms': ms, 'gbs': (b / (ms * 1e-3) / 1e9) if ms > 0 and b else None, 'bytes': b}
    tot = sum(v['ms'] for v in kern.values())
    dom = max(kern, key=lambda k: kern[k]['ms'])
    roof = {'bound': 'hbm', 'kernel': dom, 'achieved': kern[dom]['gbs'], 'peak': peak, 'unit': 'GB/s',
            'frac': (kern[dom]['gbs'] / peak) if kern[dom]['gbs'] else None, 'traffic': measured_traffic(dom, args.n),
            'peak_source': peak_kind, 'share': kern[dom]['ms'] / tot if tot else None,
            'iteration_ms': tot,
            'iteration_gbs': sum(v['bytes'] for v in kern.values()) / (tot * 1e-3) / 1e9 if tot else None,
            'kernels': kern}
    if args.only == 'mixed':
        if rank == 0:
            print(json.dumps({'metric': 'RVE solves/s (mixed only)', 'value': value, 'unit': 'solves/s',
                              'ms_per_step': t_ms / args.steps, 'cg_iters_per_solve': cg_per_solve,
                              'gpu_launches': launches, 'launch_shapes': cell.tuning(),
                              'kernels': {k: [round(v['ms'] * 1e3, 1), round(v['gbs'] or 0)] for k, v in kern.items()},
                              'iteration_us': round(tot * 1e3, 1)}), flush=True)
        return

    progress('mixed: %.2f solves/s' % value)
    # ---------------- FP64 method on the same input
    fp64_lat = []
    for i in range(1 + args.fp64_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = mu.solvers.newton_cg(cell, w['load'], fp64, w['newton_tol'], w['equil_tol'], return_fields=(i == 0))
        torch.cuda.synchronize()
        if i == 0:
            stress64 = r64.stress
        else:
            fp64_lat.append(time.perf_counter() - t0)
    rm = mu.solvers.newton_cg(cell, w['load'], mixed, w['newton_tol'], w['equil_tol'])
    stress_mixed = rm.stress
    h64 = stress64.reshape(-1, 3, 3).mean(0)
    hm = stress_mixed.reshape(-1, 3, 3).mean(0)
    err = float(np.linalg.norm(hm - h64) / np.linalg.norm(h64))
    fp64_sps = 1.0 / statistics.median(fp64_lat)
    fp64_cg = r64.nb_fev  # cumulative counter: divide by solves done with this solver
    fp64_cg_per_solve = fp64_cg / (1 + args.fp64_steps)
    # the FP64 kernels against the measured FP64 FMA throughput (their bound)
    fp64_peak = mu._lib.probe_fp64_fma()
    prof64 = fp64.profile(5)
    k64 = {}
    for name, ms in prof64.items():
        fl = fp64_flops(name, npx, nk, w['res'])
        k64[name] = {'ms': ms, 'tflops': fl / (ms * 1e-3) / 1e12 if ms > 0 else None,
                     'frac_of_fp64_fma': (fl / (ms * 1e-3) / 1e12) / fp64_peak if ms > 0 else None,
                     'gbs': algorithmic_bytes(name, npx, nk, d2, 8, 8 * 18) / (ms * 1e-3) / 1e9 if ms > 0 else None}

    progress('fp64: %.3f solves/s' % fp64_sps)
    # ---------------- end to end through the public API from host buffers
    e2e_t = []
    h2d = npx  # the material index byte per pixel (the Lame planes are filled on the device from it)
    d2h = d2 * 8             # the homogenised stress (the metric's result)
    for i in range(args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c2 = workloads.build_spheres_cell(mu, w)
        s2 = mu.solvers.SolverCG(c2, w['cg_tol'], w['maxiter'], precision='mixed')
        r2 = mu.solvers.newton_cg(c2, w['load'], s2, w['newton_tol'], w['equil_tol'], return_fields=False)
        hs = c2.homogenised_stress()
        torch.cuda.synchronize()
        if i > 0:
            e2e_t.append(time.perf_counter() - t0)
        del s2, c2
    e2e_v = world / statistics.median(e2e_t)

    line = {
        'metric': metric_name(args.n),
        'value': value, 'unit': 'solves/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_ms / args.steps, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32-mixed (f64 Newton)', 'data': 'synthetic (seeded spheres, seed %d)' % w['seed'],
        'config': {'workload': 'spheres%d_finite_le1' % args.n, 'resolution': w['res'], 'nb_spheres': 40,
                   'formulation': 'finite_strain', 'cg_tol': w['cg_tol'], 'newton_tol': w['newton_tol'],
                   'even_grid_extension': True, 'l2': 'fields 151 MB > L2, no flush', 'parallelism': 'replicas'},
        'latency_ms': {'p50': float(np.percentile(lat_ms, 50)), 'p99': float(np.percentile(lat_ms, 99))},
        'newton_steps': newton_mixed, 'cg_iters_per_solve': cg_per_solve,
        'pxit_per_s': value * npx * cg_per_solve / world * world,
        'fp64': {'solves_per_s': fp64_sps, 'cg_iters_per_solve': fp64_cg_per_solve, 'newton_steps': r64.nb_it,
                 'fp64_fma_peak_tflops': fp64_peak, 'peak_source': 'measured (probe kernel of FMA chains)',
                 'kernels': k64},
        'speedup_vs_fp64': value / world / fp64_sps,
        'stress_rel_err_vs_fp64': err,
        'roofline': roof,
        'clocks': clocks,
        'gpu_launches': launches,
        'launch_shapes': cell.tuning(),
        'e2e': {'value': e2e_v, 'unit': 'solves/s', 'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h},
    }
    if rank == 0 and world == 1 and not args.no_extra:
        line['configs'] = extra_configs(mu, workloads, peak, args.configs.split(','))
    if rank == 0 and not args.no_cpu:
        t0 = time.perf_counter()
        cb = cpu_baseline(w, args.cpu_cg_iters)
        progress('cpu baseline: %.1f s' % (time.perf_counter() - t0))
        line['cpu_baseline'] = {'value': cb['solves_per_s'], 'unit': 'solves/s', 'cores': cb['cores'], 'kind': 'port',
                                'sample': cb['sample'], 'pxit_per_s': cb['pxit_per_s']}
    if pg:
        pg.barrier()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == '__main__':
    main()
