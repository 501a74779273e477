"""The C++ API header (include/muspectre_gb300.hh): a program written against it
compiles and links with libmusg.so, maps status codes onto the reference's exception
types, and (on a GPU) solves the README example with the same counts and homogenised
stress as the Python API."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, 'muspectre_gb300')


@pytest.fixture(scope='module')
def example(tmp_path_factory):
    from muspectre_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp('cpp') / 'api_example')
    cmd = ['g++', '-std=c++17', '-O1', '-Wall', '-I', os.path.join(ROOT, 'include'),
           os.path.join(ROOT, 'tests', 'cpp', 'api_example.cc'), '-L', PKG, '-lmusg', '-Wl,-rpath,' + PKG, '-o', exe]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    return exe


def test_cpp_api_builds_and_maps_errors(example):
    p = subprocess.run([example, 'cpu'], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert 'ProjectionError' in p.stdout


@pytest.mark.gpu
def test_cpp_api_readme_example(example):
    import muspectre_gb300 as mu
    from muspectre_gb300 import workloads
    p = subprocess.run([example, 'gpu'], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    first, second = p.stdout.strip().splitlines()[:2]
    ok, nb_it, nb_fev, *s = first.split()
    assert second == 'ConvergenceError'
    w = workloads.readme_disc()
    cell = mu.SystemFactory(w['res'], w['lengths'], mu.Formulation.small_strain)
    mu.material.MaterialLinearElastic1_2d.make(cell, 'hard', w['E_hard'], w['nu']).add_pixels(w['hard'])
    mu.material.MaterialLinearElastic1_2d.make(cell, 'soft', w['E_soft'], w['nu']).add_pixels(~w['hard'])
    r = mu.solvers.newton_cg(cell, w['load'], mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter']),
                             w['newton_tol'], w['equil_tol'])
    assert int(ok) == int(r.success) == 1
    assert (int(nb_it), int(nb_fev)) == (r.nb_it, r.nb_fev)
    hs = cell.homogenised_stress()
    cs = np.array([float(x) for x in s]).reshape(2, 2).T
    assert np.abs(cs - hs).max() <= 1e-12 * np.abs(hs).max()
