"""Materials (language_bindings/python/bind_py_material.cc:57-155).

``MaterialLinearElastic{1,2,3,4}_{2,3}d.make(cell, name, ...)`` and
``add_pixel(pixel, ...)`` as in the reference, plus a vectorised ``add_pixels`` that
takes linear pixel indices or a boolean mask (the per-pixel call costs one Python
call per pixel, as upstream).  ``MaterialHyperElastoPlastic1_{2,3}d`` is provided as
well (the reference does not bind it to Python).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .cell import get_domain_index


class _Material:
    law = 0
    per_pixel = 0  # values per pixel (LE2: D*D, LE3/LE4: 2)

    def __init__(self, cell, name, params):
        self.cell = cell
        self.name = name
        self.dim = cell.dim
        p = np.asarray(params, dtype=np.float64) if params else np.zeros(1)
        idx = C.c_int(-1)
        L.check(L.lib().musg_material_create(cell.handle, self.law, name.encode(), L.dptr(p), len(params or []),
                                             C.byref(idx)))
        self._id = idx.value
        self._pending_idx = []
        self._pending_val = []
        self._count = 0
        cell._register(self)

    def _stride(self):
        return self.per_pixel if self.law != L.LAW_LE2 else self.dim * self.dim

    def _flush(self):
        if not self._pending_idx:
            return
        idx = self._pending_idx[0] if len(self._pending_idx) == 1 else np.concatenate(self._pending_idx)
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        vals = None
        if self._stride():
            vals = np.ascontiguousarray(np.concatenate(self._pending_val).astype(np.float64))
        self._pending_idx, self._pending_val = [], []
        L.check(L.lib().musg_material_add_pixels(self.cell.handle, self._id, L.llptr(idx), idx.size, L.dptr(vals),
                                                 self._stride()))

    def _add(self, indices, values=None):
        if self.cell.is_initialised():
            raise RuntimeError('cannot add pixels to an initialised cell')
        indices = np.atleast_1d(np.asarray(indices, dtype=np.int64))
        if np.any(indices < 0) or np.any(indices >= self.cell.nb_pixels):
            raise ValueError('pixel index out of range')
        self._pending_idx.append(indices)
        if self._stride():
            v = np.asarray(values, dtype=np.float64).reshape(indices.size, self._stride())
            self._pending_val.append(v.reshape(-1))
        self._count += indices.size

    def _index(self, pixel):
        return get_domain_index(self.cell.resolutions, pixel)

    def add_pixels(self, pixels):
        """Vectorised add_pixel: ``pixels`` is an array of linear (row-major) pixel
        indices or a boolean mask over the grid."""
        p = np.asarray(pixels)
        if p.dtype == bool:
            p = np.flatnonzero(p.reshape(-1))
        self._add(p)

    def size(self):
        return self._count


class _LE1(_Material):
    law = L.LAW_LE1

    @classmethod
    def make(cls, cell, name, Young, Poisson):
        """MaterialLinearElastic1::make (bind_py_material.cc:57-76)."""
        return cls(cell, name, [Young, Poisson])

    def add_pixel(self, pixel):
        self._add([self._index(pixel)])


class _LE2(_Material):
    law = L.LAW_LE2

    @classmethod
    def make(cls, cell, name, Young, Poisson):
        return cls(cell, name, [Young, Poisson])

    def add_pixel(self, pixel, eigenstrain=None):
        """material_linear_elastic2.cc:57-64: D×D eigenstrain per pixel."""
        if eigenstrain is None:
            raise RuntimeError('this material needs pixels with and eigenstrain')
        e = np.asarray(eigenstrain, dtype=np.float64).reshape(self.dim, self.dim)
        self._add([self._index(pixel)], e.T.reshape(1, -1))  # column-major

    def add_pixels(self, pixels, eigenstrains):
        p = np.asarray(pixels)
        if p.dtype == bool:
            p = np.flatnonzero(p.reshape(-1))
        e = np.asarray(eigenstrains, dtype=np.float64).reshape(p.size, self.dim, self.dim)
        self._add(p, e.transpose(0, 2, 1).reshape(p.size, -1))


class _LE3(_Material):
    law = L.LAW_LE3
    per_pixel = 2

    def __init__(self, cell, name):
        super().__init__(cell, name, [])

    @classmethod
    def make(cls, cell, name):
        return cls(cell, name)

    def add_pixel(self, pixel, Young=None, Poisson=None):
        if Young is None or Poisson is None:
            raise RuntimeError('this material needs pixels with Youngs modulus and Poisson ratio.')
        self._add([self._index(pixel)], np.array([[Young, Poisson]]))

    def add_pixels(self, pixels, Young, Poisson):
        p = np.asarray(pixels)
        if p.dtype == bool:
            p = np.flatnonzero(p.reshape(-1))
        E = np.broadcast_to(np.asarray(Young, dtype=np.float64).reshape(-1), (p.size,))
        nu = np.broadcast_to(np.asarray(Poisson, dtype=np.float64).reshape(-1), (p.size,))
        self._add(p, np.stack([E, nu], axis=1))


class _LE4(_LE3):
    law = L.LAW_LE4


class _HEP1(_Material):
    law = L.LAW_HEP1

    @classmethod
    def make(cls, cell, name, Young, Poisson, tau_y0, H, logm='projector', tangent='reference'):
        """MaterialHyperElastoPlastic1(name, E, ν, τ_y0, H)
        (material_hyper_elasto_plastic1.cc:41-65).  ``logm='projector'`` is the
        reference formula (non-finite on repeated eigenvalues); ``'spectral'`` uses
        V log(Λ) Vᵀ, identical for distinct eigenvalues.

        ``tangent='reference'`` converts the Kirchhoff tangent to PK1 as the reference
        does (materials_toolbox.hh:374-410, independent of j); ``'consistent'`` (an
        extension, off by default) stores the exact dP/dF of P = τ F⁻ᵀ through the
        derivative of the spectral logm, so that Newton-CG converges on heterogeneous
        elasto-plastic cells.  It implies ``logm='spectral'`` and writes
        εp.cur = εp.old + Δγ (the reference adds Δγ to stale contents)."""
        if tangent not in ('reference', 'consistent'):
            raise ValueError("tangent must be 'reference' or 'consistent'")
        mode = 2 if tangent == 'consistent' else {'projector': 0, 'spectral': 1}[logm]
        return cls(cell, name, [Young, Poisson, tau_y0, H, float(mode)])

    def add_pixel(self, pixel):
        self._add([self._index(pixel)])


class _Generic(_Material):
    law = L.LAW_GENERIC

    @classmethod
    def make(cls, cell, name, C_voigt):
        """MaterialLinearElasticGeneric(name, C_voigt) (material_linear_elastic_generic.cc:40-66):
        a constant stiffness tensor given as a Voigt matrix (3 × 3 in 2-D, 6 × 6 in 3-D,
        order xx, yy, [zz,] then yz, xz, xy).  The reference exposes it in C++ only."""
        C = np.asarray(C_voigt, dtype=np.float64)
        return cls(cell, name, list(C.reshape(-1)))

    def add_pixel(self, pixel):
        self._add([self._index(pixel)])


MaterialLinearElastic1_2d = type('MaterialLinearElastic1_2d', (_LE1,), {})
MaterialLinearElastic1_3d = type('MaterialLinearElastic1_3d', (_LE1,), {})
MaterialLinearElastic2_2d = type('MaterialLinearElastic2_2d', (_LE2,), {})
MaterialLinearElastic2_3d = type('MaterialLinearElastic2_3d', (_LE2,), {})
MaterialLinearElastic3_2d = type('MaterialLinearElastic3_2d', (_LE3,), {})
MaterialLinearElastic3_3d = type('MaterialLinearElastic3_3d', (_LE3,), {})
MaterialLinearElastic4_2d = type('MaterialLinearElastic4_2d', (_LE4,), {})
MaterialLinearElastic4_3d = type('MaterialLinearElastic4_3d', (_LE4,), {})
MaterialHyperElastoPlastic1_2d = type('MaterialHyperElastoPlastic1_2d', (_HEP1,), {})
MaterialHyperElastoPlastic1_3d = type('MaterialHyperElastoPlastic1_3d', (_HEP1,), {})
MaterialLinearElasticGeneric_2d = type('MaterialLinearElasticGeneric_2d', (_Generic,), {})
MaterialLinearElasticGeneric_3d = type('MaterialLinearElasticGeneric_3d', (_Generic,), {})
