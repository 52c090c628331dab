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


def coherent_propagator(latt, seed, mass, coherent_seed=0, source_t=0, dtype=None, device="cuda"):
    """A propagator that carries a signal: exp(-mass*|t - t0|) * (W + G(x)).

    W is one seeded spin-colour matrix shared by every site (unit-variance
    complex Gaussian entries, from ``coherent_seed``) -- the coherent part a
    wall source gives a propagator -- and G(x) the site noise of
    ``synthetic_propagator``.  Timeslice sums of contractions of such fields
    grow like the spatial volume while their noise grows like its square root,
    so |C_t| exceeds the spread of the site values sigma_t and a relative
    error per timeslice is well conditioned.
    """
    torch = _torch()
    dtype = dtype or torch.complex128
    noise = synthetic_propagator(latt, seed, 0.0, source_t, torch.complex128, device).reshape(-1, 144)
    g = torch.Generator(device="cpu")
    g.manual_seed(int(coherent_seed))
    w = torch.complex(torch.randn(144, generator=g, dtype=torch.float64),
                      torch.randn(144, generator=g, dtype=torch.float64)) * (0.5 ** 0.5)
    lx, ly, lz, lt = latt
    t = time_of_site(latt, device=device)
    dt = (t - source_t).abs()
    dt = torch.minimum(dt, lt - dt)
    p = (noise + w.to(device)[None, :]) * torch.exp(-mass * dt.to(torch.float64))[:, None]
    return p.reshape(-1, 4, 4, 3, 3).to(dtype)


def shifted_triple(p):
    """(P - 1, P, P + 1): three distinct propagators from one, as the
    reference's baryon example builds them from one inversion
    (``baryon_2pt.py:66-70``)."""
    return p - 1, p.clone(), p + 1
