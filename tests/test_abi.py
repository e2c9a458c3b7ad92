"""C ABI: the library builds, loads without a GPU, exports every symbol the
header declares, and reports errors as status codes."""
import ctypes as C

import numpy as np
import pytest


def test_exports_every_declared_symbol(lib):
    from ubootgl_gb300 import _lib as L
    names = L.declared_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bad_arguments_are_status_codes(lib):
    from ubootgl_gb300 import _lib as L
    h = C.c_void_p()
    flag = np.ones((16, 4), np.float32)
    assert lib.ubg_create(L.fptr(flag), 4, 16, 1.0, 1e-4, C.byref(h)) == -1  # EINVAL
    assert b">= 8" in lib.ubg_last_error()
    assert lib.ubg_create(None, 16, 16, 1.0, 1e-4, C.byref(h)) == -1
    o = L.Options()
    assert lib.ubg_default_options(C.byref(o)) == 0
    assert (o.vcycles, o.solver_mode, o.use_graph) == (2, 0, 1)


def test_no_cpu_fallback_without_gpu(lib):
    """Without a CUDA device the library refuses work instead of computing
    on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ubootgl_gb300 import _lib as L
    h = C.c_void_p()
    flag = np.ones((16, 16), np.float32)
    assert lib.ubg_create(L.fptr(flag), 16, 16, 1.0, 1e-4, C.byref(h)) == -2  # ECUDA
    assert b"no CUDA device" in lib.ubg_last_error()


def test_server_arguments_without_gpu(lib):
    """The step server's host-side checks: bad modes and limits are status
    codes, and a server with no sessions starts and stops without a GPU."""
    h = C.c_void_p()
    assert lib.ubg_server_create(1 << 20, 0, C.byref(h)) == -1  # max_active < 1
    assert lib.ubg_server_create(1 << 20, 4, C.byref(h)) == 0
    try:
        assert lib.ubg_server_set_mode(h, 7) == -1
        assert lib.ubg_server_set_mode(h, 0) == 0  # UBG_SERVE_STREAMS
        assert lib.ubg_server_set_mode(h, 1) == 0  # UBG_SERVE_FUSED
        assert lib.ubg_server_set_fuse_cells(h, -1) == -1
        assert lib.ubg_server_set_fuse_cells(h, 1 << 16) == 0
        r = C.c_uint64()
        assert lib.ubg_server_submit(h, 12345, 1, 0.5, C.byref(r)) == -1  # unknown session
        assert lib.ubg_server_close(h, 12345) == -1
        assert lib.ubg_server_drain(h) == 0
    finally:
        assert lib.ubg_server_destroy(h) == 0
