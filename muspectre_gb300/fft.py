"""FFT engines and projections (language_bindings/python/muSpectre/fft.py,
bind_py_fftengine.cc:57-107, bind_py_projections.cc:71-201).

Arrays follow the reference binding: the real field is (nb_components, nb_pixels),
the workspace (nb_components, nb_hermitian) complex, the last axis halved to n/2+1.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .cell import Formulation, get_hermitian_sizes

fft_engines = [('fftw', False), ('cuda', False)]


class FFTEngine:
    """FFTEngineBase<D> on the GPU: unnormalised r2c / c2r, normalisation() = 1/N."""

    def __init__(self, resolutions, nb_components):
        self.resolutions = [int(r) for r in resolutions]
        self.dim = len(self.resolutions)
        self.nb_components = int(nb_components)
        self.nb_pixels = int(np.prod(self.resolutions))
        self.fourier_resolutions = get_hermitian_sizes(self.resolutions)
        self.nb_fourier = int(np.prod(self.fourier_resolutions))
        h = C.c_void_p()
        r = np.array(self.resolutions, dtype=np.int32)
        L.check(L.lib().musg_fft_create(self.dim, L.iptr(r), self.nb_components, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_fft_destroy(h)
            except Exception:
                pass
            self._h = None

    def initialise(self, flags=0):
        pass

    def normalisation(self):
        return 1.0 / self.nb_pixels

    def get_subdomain_resolutions(self):
        return list(self.resolutions)

    def get_subdomain_locations(self):
        return [0] * self.dim

    def get_fourier_resolutions(self):
        return list(self.fourier_resolutions)

    def get_fourier_locations(self):
        return [0] * self.dim

    def get_domain_resolutions(self):
        return list(self.resolutions)

    def fft(self, array):
        """(nb_components, N) real -> (nb_components, N_h) complex."""
        a = np.asarray(array, dtype=np.float64)
        v = np.ascontiguousarray(a.reshape(self.nb_components, self.nb_pixels).T).reshape(-1)
        out = np.empty(self.nb_fourier * self.nb_components, dtype=np.complex128)
        L.check(L.lib().musg_fft_forward(self._h, L.dptr(v), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.nb_fourier, self.nb_components).T

    def ifft(self, array):
        """(nb_components, N_h) complex -> (nb_components, N) real (unnormalised)."""
        a = np.asarray(array, dtype=np.complex128)
        v = np.ascontiguousarray(a.reshape(self.nb_components, self.nb_fourier).T).reshape(-1)
        out = np.empty(self.nb_pixels * self.nb_components)
        L.check(L.lib().musg_fft_inverse(self._h, v.ctypes.data_as(C.POINTER(C.c_double)), L.dptr(out)))
        return out.reshape(self.nb_pixels, self.nb_components).T


def FFT(resolutions, nb_components, fft='fftw', communicator=None):
    """muSpectre.fft.FFT (fft.py:63-113)."""
    if fft not in ('fftw', 'cuda', 'gpu'):
        raise KeyError("Unknown FFT engine '{}'.".format(fft))
    if len(resolutions) not in (2, 3):
        raise ValueError('{}-d transforms are not supported'.format(len(resolutions)))
    if communicator is not None:
        raise ValueError("FFT engine '{}' does not support parallel execution.".format(fft))
    return FFTEngine(resolutions, nb_components)


_KINDS = {'small': L.PROJ_SMALL_STRAIN, 'finite_fast': L.PROJ_FINITE_STRAIN_FAST, 'finite': L.PROJ_FINITE_STRAIN}


class ProjectionBase:
    """ProjectionBase<D,D> (projection_base.hh:99-161) on the GPU."""

    kind = 'small'

    def __init__(self, resolutions, lengths, fft='fftw', communicator=None, allow_even=False, _kind=None):
        if _kind is not None:
            self.kind = _kind
        self.resolutions = [int(r) for r in resolutions]
        self.dim = len(self.resolutions)
        self.lengths = [float(x) for x in lengths]
        self.nb_pixels = int(np.prod(self.resolutions))
        h = C.c_void_p()
        r = np.array(self.resolutions, dtype=np.int32)
        ln = np.array(self.lengths, dtype=np.float64)
        L.check(L.lib().musg_projection_create(self.dim, L.iptr(r), L.dptr(ln), _KINDS[self.kind],
                                               L.FLAG_ALLOW_EVEN if allow_even else 0, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_projection_destroy(h)
            except Exception:
                pass
            self._h = None

    def initialise(self, flags=0):
        pass

    def get_formulation(self):
        return Formulation.small_strain if self.kind == 'small' else Formulation.finite_strain

    def get_subdomain_resolutions(self):
        return list(self.resolutions)

    def get_subdomain_locations(self):
        return [0] * self.dim

    def get_domain_resolutions(self):
        return list(self.resolutions)

    def get_domain_lengths(self):
        return list(self.lengths)

    def get_strain_shape(self):
        return [self.dim, self.dim]

    def apply_projection(self, field):
        """(D², N) array in, projected (D², N) array out (bind_py_projections.cc:150-169)."""
        d2 = self.dim * self.dim
        a = np.asarray(field, dtype=np.float64)
        if a.shape != (d2, self.nb_pixels):
            raise RuntimeError('Expected input array of shape ({}, {}), but input array has shape ({}).'.format(
                d2, self.nb_pixels, ', '.join(str(s) for s in a.shape)))
        v = np.ascontiguousarray(a.T).reshape(-1)
        L.check(L.lib().musg_projection_apply(self._h, L.dptr(v)))
        return v.reshape(self.nb_pixels, d2).T

    def get_operator(self):
        rows, cols = C.c_longlong(0), C.c_longlong(0)
        L.check(L.lib().musg_projection_get_operator(self._h, None, C.byref(rows), C.byref(cols)))
        out = np.empty(rows.value * cols.value)
        L.check(L.lib().musg_projection_get_operator(self._h, L.dptr(out), C.byref(rows), C.byref(cols)))
        return out.reshape(cols.value, rows.value).T


def _proj_class(name, kind):
    return type(name, (ProjectionBase,), {'kind': kind})


ProjectionSmallStrain_2d = _proj_class('ProjectionSmallStrain_2d', 'small')
ProjectionSmallStrain_3d = _proj_class('ProjectionSmallStrain_3d', 'small')
ProjectionFiniteStrain_2d = _proj_class('ProjectionFiniteStrain_2d', 'finite')
ProjectionFiniteStrain_3d = _proj_class('ProjectionFiniteStrain_3d', 'finite')
ProjectionFiniteStrainFast_2d = _proj_class('ProjectionFiniteStrainFast_2d', 'finite_fast')
ProjectionFiniteStrainFast_3d = _proj_class('ProjectionFiniteStrainFast_3d', 'finite_fast')


def Projection(resolutions, lengths, formulation=Formulation.finite_strain, fft='fftw', communicator=None,
               allow_even=False, _kind=None):
    """muSpectre.fft.Projection (fft.py:116-151): FiniteStrainFast for finite strain,
    SmallStrain for small strain."""
    kind = _kind or ('finite_fast' if Formulation(int(formulation)) == Formulation.finite_strain else 'small')
    return _proj_class('Projection', kind)(resolutions, lengths, allow_even=allow_even)
