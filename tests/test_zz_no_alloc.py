"""The allocation-free projection entry point (musg_projection_apply_noalloc).

It serves callers that cannot allocate device memory themselves or through the
library -- a caller-owned pool or arena that forbids cudaMalloc, or an
allocation-free real-time loop -- and hand in their own device buffers.  This test
calls it through the C ABI on device buffers, twice in a row for every case, and
compares it with the allocating musg_projection_apply at the projection tests'
tolerance (1e-13 relative).  On the second call of every case the device's free
memory (cudaMemGetInfo) is read right before and after the call and must not
change: the call allocates nothing.  It also checks that a grid too large for the
fixed scratch array is rejected with a clear error.  The file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (dim, resolutions, lengths, projection kind, flags)
CASES = [
    (2, [51, 51], [7., 5.], 0, 0),           # small strain, Bluestein axis (51 = 3·17)
    (3, [15, 17, 9], [1., 1.3, .7], 1, 0),   # finite strain (fast), Bluestein axis 17
    (3, [16, 16, 16], [1., 1., 1.], 0, 1),   # small strain, even grid extension
    (2, [34, 21], [2., 1.], 2, 1),           # finite strain (full operator), even axis
]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_noalloc_projection_matches_allocating_entry_point():
    torch = pytest.importorskip('torch')
    from muspectre_gb300 import _lib as L
    lib = L.lib()
    if L.device_count() < 1:
        pytest.fail('no CUDA device visible')
    rng = np.random.default_rng(1234)
    stream = torch.cuda.current_stream()
    for call in range(2):
        for dim, res, lengths, kind, flags in CASES:
            r = np.array(res, dtype=np.int32)
            ln = np.array(lengths, dtype=np.float64)
            nb_dof = int(np.prod(res)) * dim * dim
            f = rng.standard_normal(nb_dof)
            # the existing, allocating entry point on host buffers
            h = C.c_void_p()
            L.check(lib.musg_projection_create(dim, L.iptr(r), L.dptr(ln), kind, flags, C.byref(h)))
            ref = f.copy()
            L.check(lib.musg_projection_apply(h, L.dptr(ref)))
            L.check(lib.musg_projection_destroy(h))
            # the allocation-free one on device buffers
            d_in = torch.from_numpy(f).to('cuda')
            d_out = torch.full_like(d_in, float('nan'))
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            L.check(lib.musg_projection_apply_noalloc(dim, L.iptr(r), L.dptr(ln), kind, flags,
                                                      C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                                      C.c_void_p(stream.cuda_stream)))
            stream.synchronize()
            free1 = torch.cuda.mem_get_info()[0]
            if call == 1:
                assert free1 == free0, ('device memory changed across the call', res, free0, free1)
            got = d_out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert rel(got, ref) < 1e-13, (call, res)


def test_noalloc_rejects_oversized_grid():
    torch = pytest.importorskip('torch')
    from muspectre_gb300 import _lib as L
    lib = L.lib()
    buf = torch.zeros(16, dtype=torch.float64, device='cuda')
    r = np.array([256, 256, 256], dtype=np.int32)
    ln = np.ones(3)
    rc = lib.musg_projection_apply_noalloc(3, L.iptr(r), L.dptr(ln), 0, 1, C.c_void_p(buf.data_ptr()),
                                           C.c_void_p(buf.data_ptr()), C.c_void_p(0))
    assert rc == L.ERR_ARGUMENT
    assert b'maximum' in lib.musg_last_error()
    assert torch.all(buf == 0)
