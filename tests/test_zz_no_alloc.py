"""fsibe_coftxy_static: the forward transform for callers that must not allocate device memory
(their device memory belongs to a pool, or they cannot afford cudaFree's device-wide
synchronisation).  It must give the same packed coefficients as the context-based entry point
fsibe_fft_forward, call after call, using only its file-scope scratch.  Collected last so a
stop-at-first-failure run has executed every other test before it."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel
from fsibe_2d_gb300 import make_params

pytestmark = pytest.mark.gpu


def test_static_scratch_transform_matches_fft_forward_twice():
    torch = pytest.importorskip("torch")
    import fsibe_2d_gb300 as F
    lib = F.library()
    fn = lib.fsibe_coftxy_static
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    fn.restype = C.c_int
    rng = np.random.default_rng(17)
    # two calls in a row: different sizes and contents, both through the shared scratch
    for nx, ny in ((256, 256), (128, 64)):
        f = rng.standard_normal((ny, nx))
        run = F.Run(make_params(nx=nx, ny=ny, ns=16))
        ref = run.coftxy(f)
        run.close()
        fd = torch.from_numpy(f).to("cuda")
        out = torch.full_like(fd, float("nan"))
        st = fn(fd.data_ptr(), out.data_ptr(), nx, ny, None)
        torch.cuda.synchronize()
        assert st == 0, lib.fsibe_last_error(None)
        assert rel(out.cpu().numpy(), ref) < 1e-13
        # the defining property: once its kernels are loaded (the call above), further calls
        # take no device memory at all
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for _ in range(5):
            assert fn(fd.data_ptr(), out.data_ptr(), nx, ny, None) == 0
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        assert rel(out.cpu().numpy(), ref) < 1e-13


def test_static_scratch_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    import fsibe_2d_gb300 as F
    lib = F.library()
    fn = lib.fsibe_coftxy_static
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    fn.restype = C.c_int
    x = torch.zeros(512 * 256, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    assert fn(x.data_ptr(), y.data_ptr(), 512, 256, None) == 8  # FSIBE_ERR_UNSUPPORTED
    assert b"65536" in lib.fsibe_last_error(None)
