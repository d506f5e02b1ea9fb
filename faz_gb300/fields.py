"""Seeded synthetic scientific fields (no public dataset is used).

Spectral Gaussian random fields with a power-law spectrum P(k) ~ k^slope:
white noise is filtered in Fourier space by |k|^(slope/2), with per-axis
correlation-length scaling (anisotropy), optional white noise (as a fraction
of the field's standard deviation), optional sparse spikes and optional
piecewise-constant regions, then min-max scaled to [lo, hi].
"""
import numpy as np


def _spectral_numpy(shape, slope, aniso, seed):
    rng = np.random.default_rng(seed)
    white = rng.standard_normal(shape)
    spec = np.fft.rfftn(white)
    grids = []
    for ax, n in enumerate(shape):
        f = np.fft.rfftfreq(n) if ax == len(shape) - 1 else np.fft.fftfreq(n)
        grids.append(f * float(aniso[ax]))
    k2 = np.zeros(spec.shape)
    for ax, g in enumerate(grids):
        sh = [1] * len(shape)
        sh[ax] = len(g)
        k2 = k2 + g.reshape(sh) ** 2
    k = np.sqrt(k2)
    k.flat[0] = 1.0
    amp = k ** (slope / 2.0)
    amp.flat[0] = 0.0
    field = np.fft.irfftn(spec * amp, s=shape)
    return field, rng


def _bumps(shape, rng_uniform, count, xp):
    """Sum of `count` smooth Gaussian bumps on the unit cube of `shape`, with
    centres, widths (0.1..0.3 of the extent) and signed amplitudes (0.5..2)
    drawn from rng_uniform(lo, hi, n)."""
    grids = xp.meshgrid(*[xp.linspace(0.0, 1.0, n) for n in shape], indexing="ij")
    out = 0.0
    for _ in range(count):
        c = rng_uniform(0.0, 1.0, len(shape))
        w = float(rng_uniform(0.1, 0.3, 1)[0])
        a = float(rng_uniform(0.5, 2.0, 1)[0]) * (1 if rng_uniform(0.0, 1.0, 1)[0] < 0.5 else -1)
        r2 = sum((g - float(ci)) ** 2 for g, ci in zip(grids, c))
        out = out + a * xp.exp(-r2 / (2 * w * w))
    return out


def spectral_field(shape, slope=-3.0, aniso=None, noise=0.01, seed=0, lo=-50.0, hi=80.0,
                   spikes=0.0, piecewise=0, bumps=0, dtype=np.float32, device=None):
    """Seeded field of `shape` (slowest axis first).  `bumps` > 0 adds that many
    smooth Gaussian bumps as a background, at three times the spectral part's
    standard deviation.

    device=None builds on the CPU with numpy; a torch device string builds it
    there with torch.fft (used for the large benchmark fields).
    """
    shape = tuple(int(s) for s in shape)
    aniso = tuple(aniso) if aniso is not None else (1.0,) * len(shape)
    if device is not None:
        return _spectral_torch(shape, slope, aniso, noise, seed, lo, hi, spikes, piecewise, dtype, device, bumps)
    field, rng = _spectral_numpy(shape, slope, aniso, seed)
    sd = field.std()
    if bumps > 0:
        field = field + 3 * sd * _bumps(shape, lambda a, b, n: rng.uniform(a, b, n), bumps, np)
    if noise > 0:
        field = field + rng.standard_normal(shape) * (noise * sd)
    if piecewise > 0:
        field = _piecewise(field, rng, piecewise)
    fmin, fmax = field.min(), field.max()
    field = (field - fmin) / (fmax - fmin if fmax > fmin else 1.0) * (hi - lo) + lo
    if spikes > 0:
        n = field.size
        m = int(n * spikes)
        idx = rng.choice(n, size=m, replace=False)
        field.flat[idx] = rng.uniform(lo, hi, size=m)
    return field.astype(dtype)


def _piecewise(field, rng, regions):
    shape = field.shape
    out = field.copy()
    for _ in range(regions):
        sl = []
        for n in shape:
            a = int(rng.integers(0, max(1, n - 1)))
            b = int(min(n, a + max(1, n // 4)))
            sl.append(slice(a, b))
        out[tuple(sl)] = float(out[tuple(sl)].mean())
    return out


def _spectral_torch(shape, slope, aniso, noise, seed, lo, hi, spikes, piecewise, dtype, device, bumps=0):
    import torch
    g = torch.Generator(device=device).manual_seed(int(seed))
    white = torch.randn(shape, generator=g, device=device, dtype=torch.float32)
    spec = torch.fft.rfftn(white)
    del white
    k2 = None
    for ax, n in enumerate(shape):
        if ax == len(shape) - 1:
            f = torch.fft.rfftfreq(n, device=device)
        else:
            f = torch.fft.fftfreq(n, device=device)
        f = (f * float(aniso[ax])) ** 2
        sh = [1] * len(shape)
        sh[ax] = f.numel()
        f = f.reshape(sh)
        k2 = f if k2 is None else k2 + f
    k = torch.sqrt(k2)
    k.view(-1)[0] = 1.0
    amp = k.pow(slope / 2.0)
    amp.view(-1)[0] = 0.0
    spec.mul_(amp)
    del amp, k, k2
    field = torch.fft.irfftn(spec, s=shape)
    del spec
    sd = field.std()
    if bumps > 0:
        def uni(a, b, n):
            return (torch.rand(n, generator=g, device=device) * (b - a) + a).cpu().numpy()

        class _TorchNs:
            meshgrid = staticmethod(torch.meshgrid)
            exp = staticmethod(torch.exp)

            @staticmethod
            def linspace(a, b, n):
                return torch.linspace(a, b, n, device=device)
        field.add_(_bumps(shape, uni, bumps, _TorchNs) * (3 * sd))
    if noise > 0:
        field.add_(torch.randn(shape, generator=g, device=device) * (noise * sd))
    for _ in range(int(piecewise)):
        # a box of a quarter of each extent set to its mean
        sl = []
        for n in shape:
            a = int(torch.randint(0, max(1, n - 1), (1,), generator=g, device=device).item())
            sl.append(slice(a, min(n, a + max(1, n // 4))))
        box = field[tuple(sl)]
        box.fill_(box.mean())
    fmin, fmax = field.min(), field.max()
    span = (fmax - fmin) if fmax > fmin else torch.ones_like(fmax)
    field.sub_(fmin).div_(span).mul_(hi - lo).add_(lo)
    if spikes > 0:
        n = field.numel()
        m = int(n * spikes)
        idx = torch.randint(0, n, (m,), generator=g, device=device)
        vals = torch.rand((m,), generator=g, device=device) * (hi - lo) + lo
        field.view(-1)[idx] = vals
    tdt = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
    return field.to(tdt)
