"""tsdfl_resample_systematic_static (static scratch, no allocation) against
tsdfl_resample_systematic_device (context workspace), both through the C ABI.

Collected last on purpose and self-contained: passes alone in a fresh process
and after the other tests.  Results must be identical (bit-exact particles and
counts) on two calls in a row with different weights and draws.
"""
import ctypes as C

import numpy as np
import pytest

from tsdf_localization_gb300 import Context, TsdflError, _native as N

pytestmark = pytest.mark.gpu

STATIC_MAX = 1 << 18


def _particles(m, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(m, 7)).astype(np.float32)
    w = rng.random(m) ** 3
    p[:, 6] = (w / w.sum()).astype(np.float32)
    return p


def _run(torch, lib, fn, ctx, d_in, m, u0, cap):
    out = torch.full((cap, 7), -1.0, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    N.check(fn(ctx.handle, C.c_void_p(d_in.data_ptr()), m, np.float32(u0), C.c_void_p(out.data_ptr()), cap,
               C.c_void_p(cnt.data_ptr())))
    ctx.sync()
    return out.cpu().numpy(), int(cnt.item())


def test_static_scratch_matches_device_form():
    torch = pytest.importorskip("torch")
    lib = N.lib()
    ctx = Context(0)
    try:
        for call, (m, seed) in enumerate([(100_000, 1), (STATIC_MAX, 2)]):
            p = _particles(m, seed)
            u0 = float(np.float32(np.random.default_rng(seed + 10).random() / m))
            d_in = torch.from_numpy(p).cuda()
            cap = 2 * m + 16
            ref, n_ref = _run(torch, lib, lib.tsdfl_resample_systematic_device, ctx, d_in, m, u0, cap)
            got, n_got = _run(torch, lib, lib.tsdfl_resample_systematic_static, ctx, d_in, m, u0, cap)
            assert n_ref > 0 and n_got == n_ref, f"call {call}: count {n_got} != {n_ref}"
            assert np.array_equal(got[:n_got], ref[:n_ref]), f"call {call}: resampled particles differ"
            assert np.all(got[n_got:] == -1.0)
    finally:
        ctx.close()


def test_static_scratch_rejects_oversize():
    torch = pytest.importorskip("torch")
    lib = N.lib()
    ctx = Context(0)
    try:
        m = STATIC_MAX + 1
        d_in = torch.zeros((m, 7), dtype=torch.float32, device="cuda")
        out = torch.zeros((16, 7), dtype=torch.float32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        rc = lib.tsdfl_resample_systematic_static(ctx.handle, C.c_void_p(d_in.data_ptr()), m, np.float32(0.0),
                                                  C.c_void_p(out.data_ptr()), 16, C.c_void_p(cnt.data_ptr()))
        assert rc == N.TSDFL_ERR_UNSUPPORTED
        assert "static scratch limit" in lib.tsdfl_last_error().decode()
        with pytest.raises(TsdflError):
            N.check(rc)
    finally:
        ctx.close()


def _resample_ws(lib, ctx):
    rs = C.c_size_t()
    N.check(lib.tsdfl_ctx_workspace_bytes(ctx.handle, None, C.byref(rs)))
    return rs.value


def test_static_scratch_allocates_nothing():
    """On a fresh context, with every buffer allocated beforehand: the static
    form runs first (its first call only loads kernels and looks the scratch
    up); the context's resampling workspace stays at zero bytes through both
    static calls, and the second leaves the device's free memory exactly where
    it was.  The device form called afterwards grows that workspace, which
    shows the check would see it."""
    torch = pytest.importorskip("torch")
    lib = N.lib()
    ctx = Context(0)
    try:
        m = 200_000
        p1, p2 = _particles(m, 5), _particles(m, 6)
        d1, d2 = torch.from_numpy(p1).cuda(), torch.from_numpy(p2).cuda()
        cap = 2 * m + 16
        out = torch.zeros((cap, 7), dtype=torch.float32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()

        def call(fn, d_in, u0):
            N.check(fn(ctx.handle, C.c_void_p(d_in.data_ptr()), m, np.float32(u0), C.c_void_p(out.data_ptr()), cap,
                       C.c_void_p(cnt.data_ptr())))
            ctx.sync()

        assert _resample_ws(lib, ctx) == 0
        call(lib.tsdfl_resample_systematic_static, d1, 1.0e-6)
        free0 = torch.cuda.mem_get_info()[0]
        call(lib.tsdfl_resample_systematic_static, d2, 2.0e-6)
        assert torch.cuda.mem_get_info()[0] == free0
        assert _resample_ws(lib, ctx) == 0
        n_static = int(cnt.item())
        got = out[:n_static].cpu().numpy()
        call(lib.tsdfl_resample_systematic_device, d2, 2.0e-6)
        assert _resample_ws(lib, ctx) > 0
        assert int(cnt.item()) == n_static and np.array_equal(out[:n_static].cpu().numpy(), got)
    finally:
        ctx.close()
