"""GPU test of lymph_error_l2_noalloc, the L2-error entry point that
allocates no device memory (its partial sums live in a static device array).

It is meant for callers that cannot allocate device memory when they need
the norm.  The test gives it device copies of a real problem's modal mass
matrices and coefficients (allocated here by the test through the CUDA
runtime, as such a caller would hold them) and checks that two calls in a
row agree with the context path lymph_error_l2 on the same data: both
paths call the same device functions (the per-polyhedron body and the
fixed-order sum in common.cuh), so they must agree to the last bit.  It also
checks the size limit.  The file is named to be collected last.
"""
import ctypes
import glob
from ctypes import byref, c_double, c_void_p

import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ["libcudart.so", "libcudart.so.13", "libcudart.so.12"] + sorted(
            glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class DeviceArray:
    """A device copy of a float64 numpy array, owned by the test."""

    def __init__(self, rt, host):
        self.rt = rt
        host = np.ascontiguousarray(host, dtype=np.float64)
        self.ptr = c_void_p()
        assert rt.cudaMalloc(byref(self.ptr), ctypes.c_size_t(host.nbytes)) == 0
        assert rt.cudaMemcpy(self.ptr, host.ctypes.data_as(c_void_p), ctypes.c_size_t(host.nbytes), 1) == 0

    def free(self):
        self.rt.cudaFree(self.ptr)


@pytest.mark.parametrize("p", [2, 4])
def test_noalloc_l2_matches_context_path_twice(require_gpu, p):
    rt = _cudart()
    m = M.cube(3, bc="reference", agglomeration="bfs", seed=0, group=(4, 12), jitter=0.2)
    with MatrixFree(m, p, 1e-3) as g:
        g.MAKE_MATRICES_FREE()
        g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
        g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
        g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
        g.FIRST_TIME_STEP_MATRIX_FREE(0.0)
        g.run_steps(g.dt, 1.0, max_steps=5)
        g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_UEX, _lib.SLOT_UEX, 0.01)
        expected = g.COMPUTE_ERROR_L2_MATRIX_FREE(_lib.SLOT_UN, _lib.SLOT_UEX)
        mass = g.mass(1)
        uh = g.get_state(_lib.SLOT_UN)
        uex = g.get_state(_lib.SLOT_UEX)
        Np, n_poly = g.Np, g.n_poly
    bufs = [DeviceArray(rt, a) for a in (mass, uh, uex)]
    lib = _lib.load()
    try:
        for _ in range(2):
            out = c_double(-1.0)
            rc = lib.lymph_error_l2_noalloc(bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, n_poly, Np, byref(out))
            assert rc == 0, lib.lymph_last_error()
            assert expected > 0 and out.value == expected, (out.value, expected)
        # sizes beyond the static scratch are refused with a message
        out = c_double()
        rc = lib.lymph_error_l2_noalloc(bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, 262145, Np, byref(out))
        assert rc == _lib.LYMPH_ERR_INVALID and b"262144" in lib.lymph_last_error()
    finally:
        for b in bufs:
            b.free()
