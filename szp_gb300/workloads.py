"""Seeded synthetic fields for the benchmark configurations and the tests.

No dataset ships with the reference; these stand in for the fields its
examples read from disk:

* ``walk``        1-D random walk, Gaussian steps sigma=0.01 plus sin(2*pi*i/4096)
* ``fourier3d``   N^3 field, 16 random Fourier modes (|k| in [1,32], amplitude
                  ~ |k|^(-5/3)) plus Gaussian noise sigma=1e-3, flattened
                  row-major (x fastest)
* ``laplace_zero_patches``  2-D Laplace(0, 1e-3) field with seeded rectangular
                  zero patches until 40% of the 32-element blocks are zero
* ``bitcount_sweep`` / ``specials``  edge-case arrays for the parity tests

numpy versions serve the tests; ``fourier3d_torch`` / ``walk_torch`` build
the full-size fields directly in device memory for bench.py.
"""
import numpy as np


def walk(n, rng):
    steps = rng.normal(0.0, 0.01, n)
    i = np.arange(n, dtype=np.float64)
    return (np.cumsum(steps) + np.sin(2 * np.pi * i / 4096.0)).astype(np.float32)


def _modes(rng, count=16, kmax=32):
    ks, amps, phases = [], [], []
    while len(ks) < count:
        k = rng.integers(-kmax, kmax + 1, size=3)
        norm = float(np.sqrt((k * k).sum()))
        if 1.0 <= norm <= kmax:
            ks.append(k)
            amps.append(norm ** (-5.0 / 3.0))
            phases.append(rng.uniform(0, 2 * np.pi))
    return np.array(ks), np.array(amps), np.array(phases)


def fourier3d(N, rng, noise=1e-3):
    ks, amps, phases = _modes(rng)
    r = np.arange(N, dtype=np.float64)
    f = np.zeros((N, N, N), dtype=np.float64)  # [z, y, x]
    for k, a, ph in zip(ks, amps, phases):
        arg = (2 * np.pi / N) * (k[0] * r[None, None, :] + k[1] * r[None, :, None] + k[2] * r[:, None, None])
        f += a * np.sin(arg + ph)
    f += rng.normal(0.0, noise, f.shape)
    return f.astype(np.float32)


def laplace_zero_patches(ny, nx, rng, scale=1e-3, zero_frac=0.4, L=32):
    f = rng.laplace(0.0, scale, (ny, nx)).astype(np.float32)
    n = ny * nx

    def zero_blocks(a):
        flat = a.ravel()[1:]
        nb = flat.size // L
        if nb == 0:
            return 1.0
        return float((flat[: nb * L].reshape(nb, L) == 0).all(axis=1).mean())

    while zero_blocks(f) < zero_frac:
        h = int(rng.integers(1, max(2, ny // 4)))
        w = min(nx, int(rng.integers(max(L, nx // 16), max(L + 1, nx // 2))))
        y0 = int(rng.integers(0, ny - h + 1))
        x0 = int(rng.integers(0, nx - w + 1))
        f[y0:y0 + h, x0:x0 + w] = 0.0
    assert f.size == n
    return f


# Smallest max giving each bit count on glibc's log2f (x86-64, checked against
# the reference build): thresholds where (int)log2f(m)+1 exceeds the true width.
QUIRK_THRESHOLDS = [2097151, 4194302, 8388603, 16777205, 33554410, 67108819, 134217637, 268435273,
                    536870545, 1073741089, 2147482177, 4294964353]


def _pair(target):
    """floats (-a, b) with b - (-a) == target exactly (eb = 1)."""
    b = np.float32(min(target // 2, 2147483520))
    a = np.float32(target - int(b))
    return -float(a), float(b), int(b) + int(a)


def bitcount_sweep(rng, L=32, dtype=np.float32):
    """Blocks whose max |delta| sweeps every bit count 0..33 (eb = 1)."""
    out = [0.0]
    targets = [0]
    for bc in range(1, 34):
        targets.append(3 << (bc - 2) if bc >= 2 else 1)
    for t in QUIRK_THRESHOLDS:
        targets += [t - 2, t - 1, t, t + 1]
    for t in targets:
        blk = np.zeros(L, dtype=np.float64)
        if t:
            a, b, got = _pair(t)
            j = int(rng.integers(0, L - 2))
            blk[j], blk[j + 1] = a, b
            # random small jitter elsewhere for sign-bitmap coverage
            mask = rng.random(L) < 0.5
            mask[j:j + 3] = False
            blk[mask] = rng.integers(-3, 4, mask.sum())
        out.extend(blk.tolist())
    out.extend(rng.integers(-100, 100, 17).tolist())  # ragged tail
    return np.array(out, dtype=dtype)


def walk64(n, rng):
    """The walk in float64 (no rounding to float32)."""
    steps = rng.normal(0.0, 0.01, n)
    i = np.arange(n, dtype=np.float64)
    return np.cumsum(steps) + np.sin(2 * np.pi * i / 4096.0)


def specials64(rng, n=2000):
    """float64 walk with NaN, +-inf, huge, denormal, -0.0, max-double entries and
    values whose quantized product leaves the int32 range."""
    x = walk64(n, rng) * 10.0
    idx = rng.choice(np.arange(1, n), size=48, replace=False)
    vals = [np.nan, np.inf, -np.inf, 3.0e9 * 1e-3, -3.0e9 * 1e-3, 4.9e-324, 1e-310, -0.0, 1.7e308, -1.7e308,
            2147483.0, 2147483.6469]
    for k, i in enumerate(idx):
        x[i] = vals[k % len(vals)]
    return x


def specials(rng, n=2000):
    """Walk with NaN, +-inf, huge, denormal, -0.0 and max-float entries."""
    x = walk(n, rng) * np.float32(10.0)
    idx = rng.choice(np.arange(1, n), size=40, replace=False)
    vals = [np.nan, np.inf, -np.inf, 3.0e9 * 1e-3, -3.0e9 * 1e-3, 1e-42, -0.0, 3.4e38, -3.4e38, 2147483.0]
    for k, i in enumerate(idx):
        x[i] = np.float32(vals[k % len(vals)])
    return x.astype(np.float32)


# ---------------------------------------------------------------- device ---

def walk_torch(n, seed, device="cuda"):
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    steps = torch.randn(n, generator=g, device=device, dtype=torch.float64) * 0.01
    i = torch.arange(n, device=device, dtype=torch.float64)
    return (torch.cumsum(steps, 0) + torch.sin(2 * np.pi * i / 4096.0)).to(torch.float32)


def fourier3d_torch(N, seed, device="cuda", noise=1e-3):
    import torch
    rng = np.random.default_rng(seed)
    ks, amps, phases = _modes(rng)
    r = torch.arange(N, device=device, dtype=torch.float64) * (2 * np.pi / N)
    f = torch.zeros((N, N, N), device=device, dtype=torch.float32)
    for k, a, ph in zip(ks, amps, phases):
        ax = (k[0] * r).view(1, 1, N)
        ay = (k[1] * r).view(1, N, 1)
        az = (k[2] * r + ph).view(N, 1, 1)
        f += (a * torch.sin(ax + ay + az)).to(torch.float32)
    g = torch.Generator(device=device).manual_seed(seed + 1)
    f += torch.randn(f.shape, generator=g, device=device, dtype=torch.float32) * noise
    return f.reshape(-1)
