"""CPU checks of the drop-in boundary: libmusg.so loads without a GPU, exports every
symbol include/musg.h declares, and reports errors with the reference's exception
types where no device is needed."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope='module')
def lib():
    from muspectre_gb300 import build as b
    b.build()
    from muspectre_gb300 import _lib
    return _lib


def declared_symbols():
    src = open(os.path.join(ROOT, 'include', 'musg.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\b(musg_[a-z0-9_]+)\s*\(', src)))


def test_header_symbols_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    handle = ctypes.CDLL(lib.LIB_PATH)
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, missing
    # and the ctypes binding declares every one of them
    assert set(names) <= set(lib._SIGNATURES), set(names) - set(lib._SIGNATURES)


def test_device_count_without_gpu(lib):
    assert lib.device_count() >= 0


def test_even_grid_projection_error_without_gpu(lib):
    import muspectre_gb300 as mu
    with pytest.raises(mu.ProjectionError):
        mu.Cell([4, 5], [1., 1.], mu.Formulation.small_strain)
    with pytest.raises(mu.ProjectionError):
        mu.fft.ProjectionSmallStrain_3d([4, 5, 5], [1., 1., 1.])


def test_missing_library_fails_loudly(lib, monkeypatch):
    from muspectre_gb300 import _lib
    monkeypatch.setattr(_lib, '_lib', None)
    monkeypatch.setattr(_lib, 'LIB_PATH', '/nonexistent/libmusg.so')
    with pytest.raises(RuntimeError, match='not built'):
        _lib.lib()


def test_python_api_surface():
    import muspectre_gb300 as mu
    for name in ['Cell', 'CellFactory', 'SystemFactory', 'Formulation', 'get_hermitian_sizes',
                 'get_domain_ccoord', 'get_domain_index']:
        assert hasattr(mu, name)
    for d in (2, 3):
        for n in (1, 2, 3, 4):
            assert hasattr(mu.material, 'MaterialLinearElastic%d_%dd' % (n, d))
        assert hasattr(mu.material, 'MaterialHyperElastoPlastic1_%dd' % d)
        for p in ('ProjectionSmallStrain', 'ProjectionFiniteStrain', 'ProjectionFiniteStrainFast'):
            assert hasattr(mu.fft, '%s_%dd' % (p, d))
    assert hasattr(mu.solvers, 'SolverCG') and hasattr(mu.solvers, 'newton_cg')
    assert mu.get_hermitian_sizes([6, 4]) == [6, 3]
    # Cell::get_communicator: the single-rank stub (communicator.hh:107-125)
    comm = mu.Communicator()
    assert (comm.rank(), comm.size(), comm.sum(2.5)) == (0, 1, 2.5)
    assert hasattr(mu.CellBase, 'get_communicator')
    assert mu.get_domain_index([3, 4, 5], mu.get_domain_ccoord([3, 4, 5], 37)) == 37
