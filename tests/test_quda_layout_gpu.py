"""Propagators in QUDA's native device order <-> PyQUDA even/odd order, and the
in-place change of spin basis, on the GPU through the C ABI.

The QUDA side of these tests is a numpy restatement of QUDA's native
colour-spinor order (twelve fields, one per source spin-colour, each
[parity][chunk][stride][16 bytes]); QUDA itself is not available here, so the
order is pinned to that restatement, not to QUDA's own code."""
import numpy as np
import pytest

from oracle import einsum_oracle as eo

pytestmark = pytest.mark.gpu


def quda_fields_numpy(prop, latt, stride):
    """The 12 QUDA native-order fields of an even/odd propagator [V, 4, 4, 3, 3],
    as flat complex arrays of 2 * 12 * stride entries (pads zero).

    Field f = 3 k + d holds, for parity p and checkerboard site x, the sink
    spin-colour vector v[3 s + c] = P[p V/2 + x][s][k][c][d]; complex128 keeps
    one entry per 16-byte chunk (FLOAT2), complex64 two (FLOAT4):
    field[p][chunk][x][entries of the chunk]."""
    v = prop.shape[0]
    half = v // 2
    epc = 1 if prop.dtype == np.complex128 else 2  # entries per 16-byte chunk
    nq = 12 // epc
    out = []
    for k in range(4):
        for d in range(3):
            vec = prop[:, :, k, :, d].reshape(2, half, 12)  # [p][x][3 s + c]
            f = np.zeros((2, nq, stride, epc), dtype=prop.dtype)
            f[:, :, :half, :] = vec.reshape(2, half, nq, epc).transpose(0, 2, 1, 3)
            out.append(f.reshape(-1))
    return out


def _prop(latt, seed, dtype):
    p = eo.make_propagator(latt, seed, 0.2)
    return p.astype(dtype)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("latt,pad", [((4, 2, 2, 4), 0), ((6, 2, 2, 3), 5), ((8, 4, 2, 6), 3), ((2, 1, 1, 1), 1)])
def test_quda_round_trip_bit_exact(dtype, latt, pad):
    import torch

    from contract_gb300 import api
    p = _prop(latt, 31, dtype)
    half = p.shape[0] // 2
    stride = half + pad
    dev = torch.from_numpy(p).cuda()
    fields = api.to_quda(dev, latt, stride)
    want = quda_fields_numpy(p, latt, stride)
    for f, w in zip(fields, want):
        assert np.array_equal(f.cpu().numpy(), w)
    back = api.from_quda(fields, latt, stride)
    assert np.array_equal(back.cpu().numpy(), p)
    # fields written on the host in QUDA's order, read on the device
    host_fields = [torch.from_numpy(w).cuda() for w in want]
    got = api.from_quda(host_fields, latt, stride)
    assert np.array_equal(got.cpu().numpy(), p)


def test_quda_conversion_feeds_a_contraction(c_oracle):
    """QUDA fields -> even/odd -> a baryon two-point, against the oracle on the
    original propagators."""
    import torch

    from contract_gb300 import api
    latt = (4, 2, 2, 4)
    props = [_prop(latt, s, np.complex128) for s in (1, 2, 3)]
    stride = 32 + 7  # V/2 = 32, seven pad sites
    conv = [api.from_quda([torch.from_numpy(w).cuda() for w in quda_fields_numpy(p, latt, stride)], latt, stride)
            for p in props]
    got = api.baryon(*conv, 1, 5, 5, gamma_mn=8).cpu().numpy()
    ref = c_oracle.baryon_two_point(*props, 1, 5, 5, 8)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def _unitary(seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-14), (np.complex64, 2e-6)])
def test_spin_rotation_against_numpy(dtype, tol):
    import torch

    from contract_gb300 import api
    latt = (4, 2, 2, 4)
    p = _prop(latt, 7, dtype)
    u = _unitary(3)
    ref = np.einsum("st,vtkcd,uk->vsucd", u, p.astype(np.complex128), u.conj())
    dev = torch.from_numpy(p).cuda()
    api.rotate_spin_basis(dev, u)
    got = dev.cpu().numpy()
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    api.rotate_spin_basis(dev, u.conj().T)  # and back
    assert np.abs(dev.cpu().numpy() - p).max() <= 2 * tol * np.abs(p).max()


def _pion(p, gam):
    """Per-site Tr[G P G P^dagger] over spin and colour."""
    return np.einsum("st,vtkcd,kl,vslcd->v", gam, p, gam, p.conj())


def test_spin_rotation_to_a_dirac_pauli_basis():
    """A sparse basis change (two nonzeros per row: the uniform zero-skipping
    branch), U = the g4 eigenbasis of the DeGrand-Rossi set, checked on g4
    first, then applied to a propagator; a pion trace is the same in both
    bases."""
    import torch

    from contract_gb300 import api
    g = eo.GAMMA
    g4 = g[8]
    g5 = g[1] @ g[2] @ g[4] @ g4
    r = 1 / np.sqrt(2)
    u = np.array([[r, 0, r, 0], [0, r, 0, r], [r, 0, -r, 0], [0, r, 0, -r]], dtype=np.complex128)
    assert np.allclose(u @ u.conj().T, np.eye(4))
    assert np.allclose(u @ g4 @ u.conj().T, np.diag([1, 1, -1, -1]))
    latt = (4, 2, 2, 4)
    p = _prop(latt, 9, np.complex128)
    dev = torch.from_numpy(p).cuda()
    api.rotate_spin_basis(dev, u)
    ref = np.einsum("st,vtkcd,uk->vsucd", u, p, u.conj())
    pr = dev.cpu().numpy()
    assert np.abs(pr - ref).max() <= 1e-14 * np.abs(ref).max()
    a, b = _pion(p, g5), _pion(pr, u @ g5 @ u.conj().T)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
