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
    conf.l2normErrorBound = 0.5
    return conf


def _bits(v):
    return np.float64(v).view(np.uint64)


@pytest.mark.parametrize("dtype_name,mode", [("float32", F.EB_REL), ("float64", F.EB_PSNR),
                                             ("float32", F.EB_ABS_AND_REL), ("float64", F.EB_ABS_OR_REL),
                                             ("float32", F.EB_L2NORM), ("float64", F.EB_ABS)])
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
        if mode in (F.EB_L2NORM, F.EB_ABS):
            continue  # neither mode reads the field's range
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


@pytest.mark.parametrize("n", [3 * 65536, 3 * 65536 + 1, NOALLOC_MAX_VALUES])
def test_noalloc_partial_count_at_tile_boundaries(n):
    """1-D fields of exactly k tiles of 65536 values, one value more, and the
    largest field accepted (2^28 values, all 4096 partials in use).  The
    extremes sit in the last tile, so a partial count one short would miss
    them.  A large field runs first, so stale partials would also show."""
    import torch
    big = _field((NOALLOC_MAX_VALUES // 2,), torch.float32, 21, 100.0, 0.0)
    rc, _ = _noalloc(_conf((big.numel(),), F.EB_REL), big)
    assert rc == 0, F.library().faz_last_error().decode()
    del big
    x = _field((n,), torch.float32, 22, 1.0, 0.0)
    x[-1] = 50.0
    x[-2] = -60.0
    rc, got = _noalloc(_conf((n,), F.EB_REL), x)
    assert rc == 0, F.library().faz_last_error().decode()
    assert got.rng == float((x.max() - x.min()).item()) == float(np.float32(50.0) - np.float32(-60.0))
    assert _bits(got.absErrorBound) == _bits(1e-3 * got.rng)


def test_noalloc_refuses_what_compress_refuses():
    """A num that does not match dims, and a constant field (bound 0), are
    refused as faz_compress refuses them; conf stays unchanged."""
    import torch
    x = torch.full((10, 20), 3.0, device="cuda", dtype=torch.float32)
    conf = _conf((10, 20), F.EB_REL)
    s = conf.to_struct()
    s.num = 10 * 20 + 1
    dt = F.FAZ_FLOAT
    st = torch.cuda.current_stream().cuda_stream
    rc = F.library().faz_resolve_eb_noalloc(ctypes.byref(s), dt, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(st))
    assert rc == FAZ_ERR_ARG
    assert "num does not match dims" in F.library().faz_last_error().decode()
    rc, got = _noalloc(_conf((10, 20), F.EB_REL), x)
    assert rc == FAZ_ERR_ARG
    assert "positive and finite" in F.library().faz_last_error().decode()
    assert got.errorBoundMode == F.EB_REL
