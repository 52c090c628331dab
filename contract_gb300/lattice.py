"""Lattice geometry and seeded synthetic propagators on the device.

Site order is PyQUDA's even/odd layout ``[2][Lt][Lz][Ly][Lx/2]``:
``site = (((p*Lt + t)*Lz + z)*Ly + y)*(Lx/2) + xh`` with ``x = 2*xh + ((p+t+z+y) & 1)``.
"""


def _torch():
    import torch
    return torch


def volume(latt):
    lx, ly, lz, lt = latt
    return lx * ly * lz * lt


def time_of_site(latt, device="cpu"):
    """t coordinate of every site, int64 [V]."""
    torch = _torch()
    lx, ly, lz, lt = latt
    half = lx * ly * lz // 2
    return (torch.arange(volume(latt), device=device) // half) % lt


def synthetic_propagator(latt, seed, mass, source_t=0, dtype=None, device="cuda"):
    """Unit-variance complex Gaussian entries times exp(-mass*|t - t0|) (periodic distance).

    Generated on ``device`` with a seeded torch generator, shape [V, 4, 4, 3, 3].
    """
    torch = _torch()
    dtype = dtype or torch.complex128
    lx, ly, lz, lt = latt
    v = volume(latt)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    rdt = torch.float64 if dtype == torch.complex128 else torch.float32
    re = torch.randn((v, 144), generator=g, device=device, dtype=rdt)
    im = torch.randn((v, 144), generator=g, device=device, dtype=rdt)
    p = torch.complex(re, im) * (0.5 ** 0.5)
    t = time_of_site(latt, device=device)
    dt = (t - source_t).abs()
    dt = torch.minimum(dt, lt - dt)
    p *= torch.exp(-mass * dt.to(rdt))[:, None]
    return p.reshape(v, 4, 4, 3, 3).to(dtype)
