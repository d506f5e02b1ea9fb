"""faz_resolve_eb_noalloc (the entry point that allocates nothing) against
the error bound that faz_compress_device_payload resolves for the same field.

Both reduce the field's range on the device and apply the same formula, so
the bound and the range must agree bit for bit.  Two calls run back to back
with different fields, the second much smaller than the first, so a stale
partial left in the shared scratch array by the first call would show up in
the second call's range.  This file is collected last on purpose: it must
pass both alone in a fresh process and after every other test.
"""
import ctypes

import numpy as np
import pytest

import faz_gb300 as F

pytestmark = pytest.mark.gpu

NOALLOC_MAX_VALUES = 1 << 28
FAZ_ERR_ARG = -1


def _noalloc(conf, t):
    import torch
    s = conf.to_struct()
    dt = F.FAZ_FLOAT if t.dtype == torch.float32 else F.FAZ_DOUBLE
    st = torch.cuda.current_stream(t.device).cuda_stream
    rc = F.library().faz_resolve_eb_noalloc(ctypes.byref(s), dt, ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(st))
    return rc, F.Config.from_struct(s)


def _existing(conf, t):
    _, c = F.compress_payload_device(conf, t)
    return c


def _field(shape, dtype, seed, scale, shift):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn(shape, generator=g, device="cuda", dtype=torch.float64) * scale + shift
    return x.to(dtype).contiguous()


def _conf(shape, mode):
    conf = F.Config(*shape)
    conf.cmprAlgo = F.ALGO_INTERP
    conf.errorBoundMode = mode
    conf.relErrorBound = 1e-3
    conf.absErrorBound = 2e-3
    conf.psnrErrorBound = 70.0
    return conf


def _bits(v):
    return np.float64(v).view(np.uint64)


@pytest.mark.parametrize("dtype_name,mode", [("float32", F.EB_REL), ("float64", F.EB_PSNR),
                                             ("float32", F.EB_ABS_AND_REL), ("float64", F.EB_ABS_OR_REL)])
def test_noalloc_matches_compress_two_calls(dtype_name, mode):
    import torch
    dtype = getattr(torch, dtype_name)
    cases = [((200, 300, 400), 11, 40.0, -7.0), ((50, 60, 70), 12, 0.25, 3.0)]
    for shape, seed, scale, shift in cases:
        x = _field(shape, dtype, seed, scale, shift)
        rc, got = _noalloc(_conf(shape, mode), x)
        assert rc == 0, F.library().faz_last_error().decode()
        want = _existing(_conf(shape, mode), x)
        assert got.errorBoundMode == F.EB_ABS
        assert _bits(got.absErrorBound) == _bits(want.absErrorBound)
        assert _bits(got.rng) == _bits(want.rng)
        # the range is max - min of the field in its own type
        xr = x.double()
        assert got.rng == float((x.max() - x.min()).item())
        assert got.rng == pytest.approx(float(xr.max() - xr.min()), rel=1e-6)


def test_noalloc_rejects_fields_beyond_limit():
    import torch
    x = torch.zeros(16, device="cuda", dtype=torch.float32)
    conf = _conf((NOALLOC_MAX_VALUES + 1,), F.EB_REL)
    rc, _ = _noalloc(conf, x)  # rejected before any device work
    assert rc == FAZ_ERR_ARG
    assert "no-allocation limit" in F.library().faz_last_error().decode()
