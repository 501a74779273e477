"""Cells: the device-resident counterpart of µSpectre's CellBase<D,D>.

Python mirror of ``_muSpectre.CellFactory`` / ``CellBase{2,3}d``
(language_bindings/python/bind_py_cell.cc:86-202) over the C ABI.  Arrays follow the
reference binding: fields are (D², nb_pixels) arrays whose column p holds pixel p's
tensor entries in Eigen column-major order; flat vectors are pixel-major.
"""
from __future__ import annotations

import ctypes as C
import enum
from typing import List, Sequence

import numpy as np

from . import _lib as L


class Formulation(enum.IntEnum):
    """src/common/common.hh:149-153."""
    finite_strain = 0
    small_strain = 1


class FFT_PlanFlags(enum.IntEnum):
    """src/common/common.hh:142-146."""
    estimate = 0
    measure = 1
    patient = 2


def get_hermitian_sizes(full_sizes: Sequence[int]) -> List[int]:
    """ccoord_operations.hh:64-68."""
    s = list(full_sizes)
    return s[:-1] + [s[-1] // 2 + 1]


def get_domain_ccoord(resolutions: Sequence[int], i: int) -> List[int]:
    """ccoord_operations.hh:151-164 (bind_py_common.cc:84-95)."""
    out = [0] * len(resolutions)
    for d in range(len(resolutions) - 1, -1, -1):
        out[d] = int(i % resolutions[d])
        i //= resolutions[d]
    return out


def get_domain_index(sizes: Sequence[int], ccoord: Sequence[int]) -> int:
    """ccoord_operations.hh:179-192 (bind_py_common.cc:99-106)."""
    idx, f = 0, 1
    for d in range(len(sizes) - 1, -1, -1):
        idx += int(ccoord[d]) * f
        f *= sizes[d]
    return idx


class Communicator:
    """The single-rank communicator (src/common/communicator.hh:107-125, the build
    without MPI): a cell runs on one GPU; independent cells on other GPUs need no
    exchange (replicas)."""

    def rank(self):
        return 0

    def size(self):
        return 1

    def sum(self, arg):
        return arg


class CellBase:
    """CellBase<D,D> on the GPU (src/cell/cell_base.hh:241-526).

    The projection follows make_cell (cell_factory.hh:59-86): finite strain uses
    ProjectionFiniteStrainFast, small strain ProjectionSmallStrain.  Even
    resolutions raise ProjectionError like the reference unless ``allow_even=True``
    (extension: the Green operator is zero at every Nyquist k-point).
    """

    def __init__(self, resolutions, lengths=None, formulation=Formulation.finite_strain, allow_even=False):
        res = [int(r) for r in resolutions]
        self.dim = len(res)
        if self.dim not in (2, 3):
            raise ValueError('{}-d cells are not supported'.format(self.dim))
        self.resolutions = res
        self.lengths = [float(x) for x in (lengths if lengths is not None else [1.0] * self.dim)]
        self.formulation = Formulation(int(formulation))
        self.allow_even = bool(allow_even)
        h = C.c_void_p()
        r = np.array(res, dtype=np.int32)
        ln = np.array(self.lengths, dtype=np.float64)
        L.check(L.lib().musg_cell_create(self.dim, L.iptr(r), L.dptr(ln), int(self.formulation),
                                         L.FLAG_ALLOW_EVEN if allow_even else 0, C.byref(h)))
        self._h = h
        self.nb_pixels = int(np.prod(res))
        self.nb_dof = self.nb_pixels * self.dim * self.dim
        self._materials = []
        self._initialised = False
        self._has_tangent = False

    # -- lifetime --------------------------------------------------------------
    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_cell_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    # -- reference API ---------------------------------------------------------
    def __len__(self):
        return self.nb_pixels

    @property
    def size(self):
        return self.nb_pixels

    def __iter__(self):
        for i in range(self.nb_pixels):
            yield get_domain_ccoord(self.resolutions, i)

    def get_nb_dof(self):
        return self.nb_dof

    def get_formulation(self):
        return self.formulation

    def get_communicator(self):
        """Cell::get_communicator (cell_base.hh:124, 502-503): one rank."""
        return Communicator()

    def get_strain_shape(self):
        return [self.dim, self.dim]

    def get_subdomain_resolutions(self):
        return list(self.resolutions)

    def get_subdomain_locations(self):
        return [0] * self.dim

    def get_domain_resolutions(self):
        return list(self.resolutions)

    def get_domain_lengths(self):
        return list(self.lengths)

    def set_stream(self, stream_handle):
        """Run this cell's kernels on an external CUDA stream (an integer handle)."""
        L.check(L.lib().musg_cell_set_stream(self._h, C.c_void_p(int(stream_handle))))

    def _register(self, mat):
        self._materials.append(mat)
        return mat

    def _flush(self):
        for m in self._materials:
            m._flush()

    def initialise(self, flags=FFT_PlanFlags.estimate):
        """CellBase::initialise (cell_base.cc:445-454)."""
        if self._initialised:
            return
        self._flush()
        L.check(L.lib().musg_cell_initialise(self._h, int(flags)))
        self._initialised = True

    def is_initialised(self):
        return self._initialised

    def _as_field(self, v):
        a = np.asarray(v, dtype=np.float64)
        d2 = self.dim * self.dim
        if a.ndim == 2 and a.shape == (d2, self.nb_pixels):
            return np.ascontiguousarray(a.T).reshape(-1)
        if a.size == self.nb_dof:
            return np.ascontiguousarray(a.reshape(-1))
        raise RuntimeError('need array of shape ({}, {}) but got {}.'.format(d2, self.nb_pixels, a.shape))

    def _to_array(self, flat):
        return flat.reshape(self.nb_pixels, self.dim * self.dim).T

    def tuning(self):
        """Launch shapes of the spectral passes {precision: {pass: (threads, smem bytes)}}."""
        t = np.zeros(6, dtype=np.int32)
        b = np.zeros(6, dtype=np.int64)
        L.check(L.lib().musg_cell_tuning(self._h, L.iptr(t), L.llptr(b)))
        names = ('last_axis', 'middle_axis', 'green')
        return {prec: {names[k]: (int(t[3 * p + k]), int(b[3 * p + k])) for k in range(3)}
                for p, prec in enumerate(('fp64', 'fp32'))}

    def set_uniform_strain(self, strain):
        """CellBase::set_uniform_strain (cell_base.cc:110-112)."""
        m = np.asarray(strain, dtype=np.float64).reshape(self.dim, self.dim)
        L.check(L.lib().musg_cell_set_uniform_strain(self._h, L.dptr(L.f64(m.T.reshape(-1)))))

    def get_strain_vector(self):
        self.initialise()
        out = np.empty(self.nb_dof)
        L.check(L.lib().musg_cell_get_strain(self._h, L.dptr(out)))
        return out

    def set_strain_vector(self, v):
        L.check(L.lib().musg_cell_set_strain(self._h, L.dptr(self._as_field(v))))

    def get_stress_vector(self):
        out = np.empty(self.nb_dof)
        L.check(L.lib().musg_cell_get_stress(self._h, L.dptr(out)))
        return out

    def get_strain(self):
        """(D², N) strain array (bind_py_cell.cc:176-178)."""
        return self._to_array(self.get_strain_vector())

    def get_stress(self):
        return self._to_array(self.get_stress_vector())

    def evaluate_stress_tangent(self, strain=None, return_tangent=False):
        """bind_py_cell.cc:181-194 (strain given) / Cell::evaluate_stress_tangent
        (cell_base.cc:129-146).  Returns (P, K) as (D², N) and (D⁴, N) arrays when
        ``return_tangent`` is set, else P."""
        self.initialise()
        if strain is not None:
            self.set_strain_vector(strain)
        P = np.empty(self.nb_dof)
        K = np.empty(self.nb_dof * self.dim * self.dim) if return_tangent else None
        L.check(L.lib().musg_cell_evaluate_stress_tangent(self._h, L.dptr(P), L.dptr(K) if K is not None else None))
        self._has_tangent = True
        if return_tangent:
            return self._to_array(P), K.reshape(self.nb_pixels, -1).T
        return self._to_array(P)

    def evaluate_stress(self):
        return self.evaluate_stress_tangent()

    def project(self, field):
        """bind_py_cell.cc:155-173: G applied to a (D², N) array."""
        self.initialise()
        v = self._as_field(field).copy()
        L.check(L.lib().musg_cell_apply_projection(self._h, L.dptr(v)))
        return self._to_array(v)

    def apply_projection(self, vec):
        """Cell::apply_projection on a flat vector (returns the projected copy)."""
        self.initialise()
        v = L.f64(np.asarray(vec).reshape(-1)).copy()
        L.check(L.lib().musg_cell_apply_projection(self._h, L.dptr(v)))
        return v

    def directional_stiffness(self, dF):
        """bind_py_cell.cc:131-153: G(K:δF) for a (D², N) array.  Before any tangent
        was evaluated the reference works on a zero tangent, so this returns zeros."""
        self.initialise()
        v = self._as_field(dF)
        if not self._has_tangent:
            return np.zeros((self.dim * self.dim, self.nb_pixels))
        out = np.empty(self.nb_dof)
        L.check(L.lib().musg_cell_directional_stiffness(self._h, L.dptr(v), L.dptr(out)))
        return self._to_array(out)

    def evaluate_projected_directional_stiffness(self, dF_vec):
        """Cell::evaluate_projected_directional_stiffness (cell_base.cc:150-192) on a
        flat vector."""
        v = L.f64(np.asarray(dF_vec).reshape(-1))
        out = np.empty(self.nb_dof)
        L.check(L.lib().musg_cell_directional_stiffness(self._h, L.dptr(v), L.dptr(out)))
        return out

    def cg_operator(self, dF, precision='fp64'):
        """G(K:dF) for a (D², N) array through the kernels of one CG iteration, in FP64
        or in the FP32 operator of the mixed-precision solver (an extension for
        checking the mixed path; needs an evaluated tangent)."""
        self.initialise()
        v = self._as_field(dF)
        out = np.empty(self.nb_dof)
        prec = {'fp64': L.PRECISION_FP64, 'mixed': L.PRECISION_MIXED}[precision]
        L.check(L.lib().musg_cell_cg_operator(self._h, prec, L.dptr(v), L.dptr(out)))
        return self._to_array(out)

    def get_globalised_internal_real_array(self, unique_name):
        """CellBase::get_globalised_internal_real_array (cell_base.cc:370-436): the
        internal field of the materials that have it, zeros elsewhere, as a
        (nb_components, nb_pixels) array.  RuntimeError when no material has it."""
        self.initialise()
        name = unique_name.encode('utf-8')
        nc = C.c_int(0)
        L.check(L.lib().musg_cell_get_internal(self._h, name, None, 0, C.byref(nc)))
        out = np.empty(self.nb_pixels * nc.value)
        L.check(L.lib().musg_cell_get_internal(self._h, name, L.dptr(out), out.size, C.byref(nc)))
        return out.reshape(self.nb_pixels, nc.value).T

    def get_managed_real_array(self, unique_name, nb_components):
        """CellBase::get_managed_real_array (cell_base.cc:419-427): a cell-owned
        (nb_components, nb_pixels) array, created on first use; asking again with
        another number of components raises RuntimeError (cell_base.cc:354-363)."""
        managed = self.__dict__.setdefault('_managed', {})
        a = managed.get(unique_name)
        if a is None:
            a = managed[unique_name] = np.zeros((int(nb_components), self.nb_pixels))
        elif a.shape[0] != int(nb_components):
            raise RuntimeError("Field '{}' already exists and it has {} components. You asked for a field with "
                               "{}components.".format(unique_name, a.shape[0], nb_components))
        return a

    def checkpoint(self):
        """The cell's device state (strain, stress, elasto-plastic state) as bytes, for
        restore() into a cell built the same way (an extension of the reference)."""
        self.initialise()
        n = C.c_ulonglong(0)
        L.check(L.lib().musg_cell_checkpoint_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        L.check(L.lib().musg_cell_checkpoint_save(self._h, buf, n))
        return buf.raw

    def restore(self, image):
        """Load a checkpoint() image; the next solve continues from its state."""
        self.initialise()
        buf = C.create_string_buffer(bytes(image), len(image))
        L.check(L.lib().musg_cell_checkpoint_load(self._h, buf, len(image)))
        self._has_tangent = False

    def homogenised_stress(self):
        """Pixel mean of the stress field (D×D), reduced on the device."""
        out = np.empty(self.dim * self.dim)
        L.check(L.lib().musg_cell_homogenised_stress(self._h, L.dptr(out)))
        return out.reshape(self.dim, self.dim).T

    def save_history_variables(self):
        L.check(L.lib().musg_cell_save_history_variables(self._h))

    def get_projection(self):
        from .fft import Projection
        kind = 'small' if self.formulation == Formulation.small_strain else 'finite_fast'
        return Projection(self.resolutions, self.lengths, self.formulation, allow_even=self.allow_even,
                          _kind=kind)


class CellBase2d(CellBase):
    pass


class CellBase3d(CellBase):
    pass


def CellFactory(resolutions, lengths=None, formulation=Formulation.finite_strain, allow_even=False):
    """_muSpectre.CellFactory (bind_py_cell.cc:86-98): make_cell<D,D>."""
    cls = CellBase2d if len(resolutions) == 2 else CellBase3d
    return cls(resolutions, lengths, formulation, allow_even=allow_even)


#: the README calls the factory ``SystemFactory``
SystemFactory = CellFactory


def Cell(resolutions, lengths=None, formulation=Formulation.finite_strain, fft='fftw', communicator=None,
         allow_even=False):
    """muSpectre.Cell (language_bindings/python/muSpectre/__init__.py:54-103).  The GPU
    engine accepts ``fft='fftw'`` (and ``'cuda'``) for a drop-in; there is one rank."""
    if fft not in ('fftw', 'cuda', 'gpu'):
        raise KeyError("Unknown FFT engine '{}'.".format(fft))
    if communicator is not None:
        raise ValueError("FFT engine '{}' does not support parallel execution.".format(fft))
    return CellFactory(resolutions, lengths, formulation, allow_even=allow_even)
