"""Seeded synthetic scalar fields for tests and benchmarks.

The reference ships no data set; its only usage example samples an analytic
sphere (DMC_CUDA/DMC_CUDA/src/dmc.cu:2215-2306, commented out).  These
generators make the benchmark workloads: a noisy sphere SDF, a sum of Gaussian
blobs, 4-octave lattice value noise quantised to uint16 and gyroids.  Every
field is indexed [z, y, x] (x fastest, the reference's Array3D layout,
utils.hpp:38), with integer point coordinates.

They are plain torch tensor code (device memory plumbing, not the extraction
path) and run on the CPU or a GPU.  The same seed gives the same parameters on
both; sample values computed on different devices may differ in the last bit,
so parity checks always hand one array to both sides.
"""
import math

import numpy as np
import torch


def _gen(seed):
    g = torch.Generator(device="cpu")
    g.manual_seed(int(seed))
    return g


def _axis(n, device):
    return torch.arange(n, device=device, dtype=torch.float32)


def sphere_sdf(n=64, radius=20.0, centre=None, noise=0.01, seed=1, device="cpu"):
    """Signed distance to a sphere plus uniform noise in [-noise, noise]."""
    if centre is None:
        centre = (n - 1) / 2.0
    a = _axis(n, device) - centre
    d = torch.sqrt(a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2) - radius
    if noise:
        u = torch.rand((n, n, n), generator=_gen(seed), dtype=torch.float32) * (2 * noise) - noise
        d = d + u.to(device)
    return d.contiguous()


def blob_params(dims, count=32, sigma=(8.0, 32.0), amp=(0.5, 1.5), seed=2):
    nx, ny, nz = dims
    g = _gen(seed)
    c = torch.rand((count, 3), generator=g, dtype=torch.float64) * torch.tensor([nx - 1, ny - 1, nz - 1], dtype=torch.float64)
    s = sigma[0] + torch.rand(count, generator=g, dtype=torch.float64) * (sigma[1] - sigma[0])
    a = amp[0] + torch.rand(count, generator=g, dtype=torch.float64) * (amp[1] - amp[0])
    return c, s, a


def gaussian_blobs(dims=(512, 512, 512), count=32, sigma=(8.0, 32.0), amp=(0.5, 1.5), seed=2,
                   device="cpu", out=None, slab=16):
    """Sum of ``count`` Gaussian blobs a*exp(-|p-c|^2 / (2 s^2)), float32."""
    nx, ny, nz = dims
    c, s, a = blob_params(dims, count, sigma, amp, seed)
    if out is None:
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=device)
    xs, ys = _axis(nx, device), _axis(ny, device)
    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        zs = torch.arange(z0, z1, device=device, dtype=torch.float32)
        acc = torch.zeros((z1 - z0, ny, nx), dtype=torch.float32, device=device)
        for i in range(count):
            k = float(-0.5 / (s[i] * s[i]))
            ex = torch.exp(k * (xs - float(c[i, 0])) ** 2)
            ey = torch.exp(k * (ys - float(c[i, 1])) ** 2)
            ez = torch.exp(k * (zs - float(c[i, 2])) ** 2)
            acc += float(a[i]) * ez[:, None, None] * ey[None, :, None] * ex[None, None, :]
        out[z0:z1] = acc
    return out


def _hash01(ix, iy, iz, salt):
    """Integer lattice hash -> uniform [0, 1).  A 32-bit multiply/xorshift mix
    (the "lowbias32" finaliser) evaluated in int64 with explicit masking."""
    M = 0xFFFFFFFF
    h = (ix * 0x8DA6B343) ^ (iy * 0xD8163841) ^ (iz * 0xCB1AB31F) ^ (salt * 0x165667B1)
    h = h & M
    h = h ^ (h >> 16)
    h = (h * 0x7FEB352D) & M
    h = h ^ (h >> 15)
    h = (h * 0x846CA68B) & M
    h = h ^ (h >> 16)
    return (h >> 8).to(torch.float32) * (1.0 / 16777216.0)


def value_noise_u16(dims=(1024, 1024, 1024), octaves=4, base_period=128, persistence=0.5, seed=3,
                    device="cpu", out=None, slab=8):
    """4-octave lattice value noise (period base_period / 2^o, amplitude
    persistence^o, smoothstep-weighted trilinear), normalised by the amplitude
    sum and quantised with round(v * 65535).

    Returns a torch.int16 tensor [z, y, x] that holds the uint16 bit patterns
    (torch has no general uint16 arithmetic); ``as_u16_numpy`` views it as
    numpy uint16."""
    nx, ny, nz = dims
    if out is None:
        out = torch.empty((nz, ny, nx), dtype=torch.int16, device=device)
    amps = [persistence ** o for o in range(octaves)]
    norm = sum(amps)
    xs = torch.arange(nx, device=device, dtype=torch.int64)
    ys = torch.arange(ny, device=device, dtype=torch.int64)

    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        zs = torch.arange(z0, z1, device=device, dtype=torch.int64)
        acc = torch.zeros((z1 - z0, ny, nx), dtype=torch.float32, device=device)
        for o in range(octaves):
            p = max(1, base_period >> o)
            salt = int(seed) * 16 + o

            def split(v):
                i0 = torch.div(v, p, rounding_mode="floor")
                t = (v - i0 * p).to(torch.float32) / p
                return i0, t * t * (3.0 - 2.0 * t)

            ix, tx = split(xs)
            iy, ty = split(ys)
            iz, tz = split(zs)
            IX, IY, IZ = ix[None, None, :], iy[None, :, None], iz[:, None, None]
            TX, TY, TZ = tx[None, None, :], ty[None, :, None], tz[:, None, None]
            v = 0.0
            for dz in (0, 1):
                wz = TZ if dz else 1.0 - TZ
                for dy in (0, 1):
                    wy = TY if dy else 1.0 - TY
                    for dx in (0, 1):
                        wx = TX if dx else 1.0 - TX
                        v = v + wz * wy * wx * _hash01(IX + dx, IY + dy, IZ + dz, salt)
            acc += amps[o] * v
        q = torch.round(acc * (65535.0 / norm)).clamp_(0, 65535).to(torch.int32)
        out[z0:z1] = (q - (q >= 32768).to(torch.int32) * 65536).to(torch.int16)
    return out


def as_u16_numpy(t):
    """View an int16 tensor holding uint16 bit patterns as a numpy uint16 array."""
    return t.detach().cpu().contiguous().numpy().view(np.uint16)


def gyroid(dims, freq, noise=0.02, seed=4, device="cpu"):
    """sin(fx)cos(fy) + sin(fy)cos(fz) + sin(fz)cos(fx) plus Gaussian noise."""
    nx, ny, nz = dims
    x = _axis(nx, device)[None, None, :] * freq
    y = _axis(ny, device)[None, :, None] * freq
    z = _axis(nz, device)[:, None, None] * freq
    v = torch.sin(x) * torch.cos(y) + torch.sin(y) * torch.cos(z) + torch.sin(z) * torch.cos(x)
    if noise:
        v = v + noise * torch.randn((nz, ny, nx), generator=_gen(seed), dtype=torch.float32).to(device)
    return v.contiguous()


def uneven_batch_specs(count=256, lo=16, hi=256, seed=5):
    """Per-volume (dims, frequency, isovalue) of the batched workload: dims
    log-uniform in [lo, hi] per axis, f uniform in [0.05, 0.4] rad/voxel plus
    N(0, 0.02), isovalue uniform in [-0.5, 0.5]."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        d = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), 3))).astype(int)
        d = np.clip(d, lo, hi)
        f = float(rng.uniform(0.05, 0.4) + rng.normal(0.0, 0.02))
        iso = float(rng.uniform(-0.5, 0.5))
        specs.append(dict(dims=(int(d[0]), int(d[1]), int(d[2])), freq=f, iso=iso, seed=1000 + i))
    return specs


def served_pool_specs(count=64, lo=32, hi=512, seed=9, size_tilt=1.4):
    """Per-volume recipe of the serving pool: dims log-uniform in [lo, hi] per
    axis; field kind uniform over blobs (float32), lattice noise (uint16) and
    gyroid (float32).  Blobs keep 32 centres, sigma 8-32, amplitude 0.5-1.5;
    noise keeps 4 octaves and persistence 0.5 with a base period of 32 voxels
    (most pool volumes are far smaller than 1024); gyroid frequency uniform in
    [0.05, 0.4] rad/voxel.

    Size tilt: a plain log-uniform draw gives a pool of about 1.1 GB on
    average, while the served configuration asks for about 6 GB.  Each drawn
    dims triple is therefore kept with probability (points / hi^3)^size_tilt
    and redrawn otherwise: the dims stay log-uniform in shape, with the upper
    tail weighted.  size_tilt = 1.4 puts the expected pool at about 6 GB
    (0: the plain draw)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        while True:
            d = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), 3))).astype(int)
            d = np.clip(d, lo, hi)
            if size_tilt <= 0 or rng.uniform() < (float(np.prod(d)) / float(hi) ** 3) ** size_tilt:
                break
        kind = ("blobs", "noise", "gyroid")[int(rng.integers(0, 3))]
        specs.append(dict(dims=(int(d[0]), int(d[1]), int(d[2])), kind=kind,
                          freq=float(rng.uniform(0.05, 0.4)), seed=2000 + i))
    return specs


def make_pool_volume(spec, device="cuda"):
    """One serving-pool volume from served_pool_specs (float32, or int16 holding uint16 bits)."""
    if spec["kind"] == "blobs":
        return gaussian_blobs(spec["dims"], seed=spec["seed"], device=device)
    if spec["kind"] == "noise":
        return value_noise_u16(spec["dims"], base_period=32, seed=spec["seed"], device=device)
    return gyroid(spec["dims"], spec["freq"], seed=spec["seed"], device=device)
