"""FP64 numpy einsum oracle for every contraction (test infrastructure only).

Semantics follow CLQCD/contract:

* meson two-point: ``C(x) = Tr[(g5 Gij) S1(x) (g5 Gkl) S2(x)^dagger]`` over spin
  and colour -- the quantity ``meson_local`` accumulates in
  ``include/meson.cuh:33-50`` (coefficients from ``gamma_gamma5_data<true>``).
* baryon two-point: the ``doc/contract.py:6,20`` einsum strings, extended to the
  six contraction types of ``include/contract_enum.h:1-20`` (propagator index
  strings as in ``baryon_2pt.py:31-41``), with the Gamma_mn operand indexed
  ``nm`` exactly as in ``doc/contract.py``.
* general projector: the same strings with the Gamma_mn operand replaced by
  ``project_mn.reshape(4, 4)`` (``include/baryon_general.cuh:66,83``).
* diquark: ``include/diquark.cuh:33-57``.
* sequential: the in-place gradient dC(x)/dP_slot(x)
  (``include/baryon_sequential.cuh:36-163``).

Propagators are arrays ``[V, 4, 4, 3, 3]`` (sink spin, source spin, sink
colour, source colour), complex128, PyQUDA site order.
"""
import numpy as np

from .gamma import GAMMA, G5, epsilon

EPS = epsilon().astype(np.float64)

# contract_enum.h:1-8 -- value -> propagator index strings (i, j, n operands)
BARYON_TYPES = {
    0: ("IK_JL_NM", "ikad", "jlbe", "mncf"),
    1: ("IK_JM_NL", "ikad", "jnbe", "mlcf"),
    2: ("IL_JK_NM", "ilad", "jkbe", "mncf"),
    3: ("IL_JM_NK", "ilad", "jnbe", "mkcf"),
    4: ("IM_JK_NL", "inad", "jkbe", "mlcf"),
    5: ("IM_JL_NK", "inad", "jlbe", "mkcf"),
}
TYPE1 = (0, 2)  # Pn contracts with itself through Gamma_mn
TYPE2 = (1, 3, 4, 5)

SEQ_I, SEQ_J, SEQ_N = 0, 1, 2


def _as_sites(p):
    p = np.asarray(p)
    return p.reshape(-1, 4, 4, 3, 3)


def meson_two_point(p1, p2, gamma_ij, gamma_kl):
    m1 = G5 @ GAMMA[gamma_ij]
    m2 = G5 @ GAMMA[gamma_kl]
    return np.einsum("ji,xikad,kl,xjlad->x", m1, _as_sites(p1), m2, np.conj(_as_sites(p2)), optimize=True)


def meson_all_source(p1, p2, gamma_ij):
    return np.stack([meson_two_point(p1, p2, gamma_ij, g) for g in range(16)])


def meson_all_sink(p1, p2, gamma_kl):
    return np.stack([meson_two_point(p1, p2, g, gamma_kl) for g in range(16)])


def meson_all_gamma(p1, p2):
    """All 16x16 (Gamma_ij, Gamma_kl) pairs per site: [16, 16, V]."""
    t = np.einsum("xikad,xjlad->xikjl", _as_sites(p1), np.conj(_as_sites(p2)), optimize=True)
    g5g = np.einsum("ab,gbc->gac", G5, GAMMA)
    return np.einsum("Aji,xikjl,Bkl->ABx", g5g, t, g5g, optimize=True)


def meson_product_l1(p1, p2, latt):
    """Error scale for momentum-projected meson pairs: per timeslice, the
    largest sum_x |T(x)| over the 256 spin-colour products
    T[i][j][k][l](x) = sum_c S1[i][k][c] conj(S2[j][l][c]) that every Gamma
    pair is a signed sum of: [1, Lt, 1].  An FP32 projection sums terms of
    this size.  With one field in both slots the diagonal products are
    positive at every site, so at nonzero momentum the projection cancels
    terms of this size and its rounding is relative to it, not to |C| or to
    sigma of the pairs."""
    t = np.einsum("xikad,xjlad->ijklx", _as_sites(p1), np.conj(_as_sites(p2)), optimize=True).reshape(256, -1)
    return timeslice_sum(np.abs(t), latt).real.max(axis=0)[None, :, None]


def _baryon_subscripts(contract_type):
    _, si, sj, sn = BARYON_TYPES[int(contract_type)]
    return si, sj, sn


def baryon_general(pi, pj, pn, contract_type, gamma_ij, gamma_kl, w_nm):
    """Baryon two-point with an arbitrary 4x4 operand in the Gamma_mn slot."""
    si, sj, sn = _baryon_subscripts(contract_type)
    sub = f"abc,def,ij,kl,nm,x{si},x{sj},x{sn}->x"
    return np.einsum(sub, EPS, EPS, GAMMA[gamma_ij], GAMMA[gamma_kl], np.asarray(w_nm, dtype=np.complex128),
                     _as_sites(pi), _as_sites(pj), _as_sites(pn), optimize=True)


def baryon_two_point(pi, pj, pn, contract_type, gamma_ij, gamma_kl, gamma_mn):
    return baryon_general(pi, pj, pn, contract_type, gamma_ij, gamma_kl, GAMMA[gamma_mn])


def baryon_general_two_point(pi, pj, pn, contract_type, gamma_ij, gamma_kl, project_mn):
    """``project_mn`` is the flat 16-entry complex array passed to the C ABI."""
    w = np.asarray(project_mn, dtype=np.complex128).reshape(4, 4)
    return baryon_general(pi, pj, pn, contract_type, gamma_ij, gamma_kl, w)


def baryon_diquark(pi, pj, gamma_ij, gamma_kl):
    d = np.einsum("abc,def,ij,kl,xikbe,xjmcf->xmlad", EPS, EPS, GAMMA[gamma_ij], GAMMA[gamma_kl],
                  _as_sites(pi), _as_sites(pj), optimize=True)
    s = np.diag(G5).real
    return np.conj(d) * s[None, :, None, None, None] * s[None, None, :, None, None]


def baryon_sequential(pi, pj, pn, contract_type, sequential_type, gamma_ij, gamma_kl, gamma_mn):
    """Return dC(x)/dP_slot(x), shaped like a propagator (the value written in place)."""
    si, sj, sn = _baryon_subscripts(contract_type)
    ops = [(f"x{si}", _as_sites(pi)), (f"x{sj}", _as_sites(pj)), (f"x{sn}", _as_sites(pn))]
    out_sub, _ = ops[int(sequential_type)]
    rest = [o for k, o in enumerate(ops) if k != int(sequential_type)]
    sub = "abc,def,ij,kl,nm," + ",".join(s for s, _ in rest) + "->" + out_sub
    return np.einsum(sub, EPS, EPS, GAMMA[gamma_ij], GAMMA[gamma_kl], GAMMA[gamma_mn], *[a for _, a in rest],
                     optimize=True)


# ---------------------------------------------------------------------------
# Lattice geometry (PyQUDA even/odd order) and the per-timeslice / momentum
# reductions the caller performs on the per-site output.
# ---------------------------------------------------------------------------

def eo_coords(latt):
    """Coordinates of every site in PyQUDA even/odd order.

    ``latt = (Lx, Ly, Lz, Lt)``; site index
    ``(((p*Lt + t)*Lz + z)*Ly + y)*(Lx/2) + xh`` with ``x = 2*xh + ((p+t+z+y) & 1)``.
    Returns int64 arrays (x, y, z, t) of length V.
    """
    lx, ly, lz, lt = latt
    p, t, z, y, xh = np.meshgrid(np.arange(2), np.arange(lt), np.arange(lz), np.arange(ly), np.arange(lx // 2),
                                 indexing="ij")
    x = 2 * xh + ((p + t + z + y) & 1)
    return x.ravel(), y.ravel(), z.ravel(), t.ravel()


def timeslice_sum(per_site, latt):
    """Sum a per-site field [..., V] over the spatial volume: [..., Lt]."""
    lx, ly, lz, lt = latt
    a = np.asarray(per_site)
    a = a.reshape(a.shape[:-1] + (2, lt, lz * ly * lx // 2))
    return a.sum(axis=(-1, -3))


def momentum_list(nmax):
    """All integer momenta n in {-nmax..nmax}^3, x fastest."""
    r = np.arange(-nmax, nmax + 1)
    nz, ny, nx = np.meshgrid(r, r, r, indexing="ij")
    return np.stack([nx.ravel(), ny.ravel(), nz.ravel()], axis=1)


def momentum_project(per_site, latt, moms):
    """``sum_x exp(+i 2 pi n.x / L) T(x)`` per timeslice: [..., P, Lt].

    Phases are built from the exact integer ``(n.x) mod L`` per direction.
    """
    lx, ly, lz, lt = latt
    x, y, z, t = eo_coords(latt)
    moms = np.asarray(moms)
    ang = 2 * np.pi * (np.outer(moms[:, 0], x) % lx / lx + np.outer(moms[:, 1], y) % ly / ly
                       + np.outer(moms[:, 2], z) % lz / lz)
    ph = np.exp(1j * ang)  # [P, V]
    a = np.asarray(per_site)
    lead = a.shape[:-1]
    a2 = a.reshape(-1, a.shape[-1])
    out = np.zeros((a2.shape[0], len(moms), lt), dtype=np.complex128)
    for tt in range(lt):
        sel = t == tt
        out[:, :, tt] = a2[:, sel] @ ph[:, sel].T
    return out.reshape(lead + (len(moms), lt))


def make_propagator(latt, seed, mass, source_t=0, dtype=np.complex128):
    """Synthetic propagator: unit-variance complex Gaussian x exp(-mass*|t - t0|).

    Shape [V, 4, 4, 3, 3] in PyQUDA even/odd order.  ``|t - t0|`` is the
    periodic distance on the time axis.
    """
    lx, ly, lz, lt = latt
    v = lx * ly * lz * lt
    rng = np.random.default_rng(seed)
    re = rng.standard_normal((v, 144))
    im = rng.standard_normal((v, 144))
    p = (re + 1j * im) / np.sqrt(2.0)
    _, _, _, t = eo_coords(latt)
    dt = np.abs(t - source_t)
    dt = np.minimum(dt, lt - dt)
    p *= np.exp(-mass * dt)[:, None]
    return p.reshape(v, 4, 4, 3, 3).astype(dtype)
