"""bench.py's JSON line for the reference arm (the oracle on the host CPU, no GPU): the
keys the benchmark contract names, on a tiny grid where each step is a complete solve."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), '--impl', 'reference', '--n', '8',
                          '--steps', '2', '--warmup', '1'], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'scaling',
                'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e'):
        assert key in line, key
    assert line['impl'] == 'reference' and line['unit'] == 'solves/s' and line['higher_is_better'] is True
    assert line['value'] > 0 and line['steps'] == 2 and line['warmup'] == 1
    assert line['config']['workload'] == 'spheres8_finite_le1' and line['config']['resolution'] == [8, 8, 8]
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['cores'] >= 1 and 'complete solves' in cb['sample'] and cb['value'] == line['value']
    e2e = line['e2e']
    assert e2e['value'] == line['value'] and e2e['h2d_bytes_per_step'] == 0 and e2e['d2h_bytes_per_step'] == 0


def test_reference_arm_metric_matches_ours():
    """Both arms print one metric string, so that their values can be divided."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.metric_name(128) == 'RVE solves/s (Newton-CG, 128^3 finite-strain LE1, 40 spheres)'
    src = open(os.path.join(ROOT, 'bench.py')).read()
    assert src.count("'metric': metric_name(args.n)") == 2


def test_scaled_sample_matches_complete_solves():
    """The reference arm's method at 128^3 (no complete solve fits the run): the
    Newton-level work timed once plus a timed sample of 8 CG iterations, scaled by the
    Newton and CG counts of a complete solve.  At 32^3 and 48^3, where a complete
    oracle solve takes seconds, the scaled estimate of the solve time is within 35%
    of the faster of two timed complete solves (measured: within 4% on an idle host)."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    from muspectre_gb300 import workloads
    from oracle import muspectre_oracle as o
    saved = o.FFT_WORKERS
    o.FFT_WORKERS = os.cpu_count() or 1
    try:
        for n in (32, 48):
            w = workloads.spheres(n)
            t_full = []
            for _ in range(2):  # the second solve runs with warm FFT plans and caches
                t0 = time.perf_counter()
                oc = workloads.build_spheres_oracle(o, w)
                r = o.newton_cg(oc, w['load'], o.SolverCG(oc, w['cg_tol'], w['maxiter']), w['newton_tol'],
                                w['equil_tol'], 0)
                t_full.append(time.perf_counter() - t0)
            t_full = min(t_full)
            smp = bench.CpuSample(w)
            est = smp.describe(smp.cg_iteration_seconds(bench.REF_SAMPLE_CG_ITERS), r.nb_it, r.nb_fev,
                               bench.REF_SAMPLE_CG_ITERS)
            ratio = t_full * est['solves_per_s']
            assert 0.65 < ratio < 1.35, (n, t_full, 1.0 / est['solves_per_s'])
    finally:
        o.FFT_WORKERS = saved


def test_fused_iteration_bytes():
    """The algorithmic bytes bench.py counts for the mixed CG iteration (its roofline
    numerator): six passes moving 8 fields and 8 half spectra plus the tangent data, i.e.
    16u + T_m with the half spectrum counted as a field (within 2/N at 128^3), against
    19u + T_m for the unfused iteration (forward, update, three FFT passes, inverse)."""
    sys.path.insert(0, ROOT)
    import bench
    n = 128
    npx, nk, d2, s = n ** 3, n * n * (n // 2 + 1), 9, 4
    u = npx * d2 * s
    tm = 4 * 9 + 1
    fused = ['last_axis_fwd_tangent_alpha', 'cg_update_x', 'axis1_fwd', 'green_axis0', 'axis1_inv',
             'last_axis_inv_update_r']
    unfused = ['last_axis_fwd_tangent', 'axis1_fwd', 'green_axis0', 'axis1_inv', 'last_axis_inv_dot', 'cg_update']
    b_fused = sum(bench.algorithmic_bytes(k, npx, nk, d2, s, tm) for k in fused)
    b_unfused = sum(bench.algorithmic_bytes(k, npx, nk, d2, s, tm) for k in unfused)
    assert abs(b_fused - (16 * u + tm * npx)) <= 2 / n * 16 * u
    assert abs(b_unfused - (19 * u + tm * npx)) <= 2 / n * 19 * u
