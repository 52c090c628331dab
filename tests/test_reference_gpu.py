"""The drop-in entry points against the reference's own CUDA kernels, on the
same GPU, on identical device inputs, at the baryon benchmark's full size.

The reference kernels are the reference's CUDA translation units compiled
unmodified to sm_103a cubins (``make -C oracle refgpu``) and launched through
the driver API exactly as the reference's host code launches them
(``oracle/ref_gpu.py``).  Inputs: the 24^3 x 64 propagators u, u, d of the
baryon benchmark (seeded complex Gaussian x exp(-m|t|), complex128, PyQUDA
even/odd order).  Every per-site output must agree to 1e-12 of its largest
value: both sides are FP64 and differ only in summation order.
"""
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12
LATT = (24, 24, 24, 64)
V = 24 * 24 * 24 * 64


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference cubins not built (make -C oracle refgpu REF=<CLQCD/contract checkout>)")
    return ref_gpu.ReferenceGPU(0)


@pytest.fixture(scope="module")
def env(ref):
    import torch

    from contract_gb300 import build
    build.build()
    from contract_gb300 import pycontract
    from contract_gb300.lattice import synthetic_propagator
    pycontract.init(0)
    u = synthetic_propagator(LATT, 1000, 0.25, device="cuda:0")
    u2 = u.clone()
    d = synthetic_propagator(LATT, 3000, 0.30, device="cuda:0")
    torch.cuda.synchronize()
    return pycontract, (u, u2, d)


def _rel(a, b):
    import torch
    torch.cuda.synchronize()
    scale = b.abs().max().item()
    assert scale > 0
    return (a - b).abs().max().item() / scale


def _proj():
    from contract_gb300 import api
    return api.projector_plus_minus()


def test_baryon_general_two_point_all_types(ref, env):
    """The benchmark's twelve calls: six types x (1 +- g4)/2 with C g5."""
    import torch
    pc, (u, u2, d) = env
    ours = torch.empty(V, dtype=torch.complex128, device="cuda:0")
    theirs = torch.empty_like(ours)
    for t in range(6):
        for w, proj in enumerate(_proj()):
            pc.baryon_general_two_point(ours, u, u2, d, t, V, 5, 5, proj)
            torch.cuda.synchronize()
            ref.baryon_general_two_point(theirs.data_ptr(), u.data_ptr(), u2.data_ptr(), d.data_ptr(), t, V, 5, 5,
                                         proj)
            assert _rel(ours, theirs) < TOL, (t, w)


def test_baryon_two_point_all_types(ref, env):
    import torch
    pc, (u, u2, d) = env
    ours = torch.empty(V, dtype=torch.complex128, device="cuda:0")
    theirs = torch.empty_like(ours)
    for t in range(6):
        for gmn in (8, 15):
            pc.baryon_two_point(ours, u, u2, d, t, V, 5, 5, gmn)
            torch.cuda.synchronize()
            ref.baryon_two_point(theirs.data_ptr(), u.data_ptr(), u2.data_ptr(), d.data_ptr(), t, V, 5, 5, gmn)
            assert _rel(ours, theirs) < TOL, (t, gmn)


def test_meson_two_point_and_all_gamma(ref, env):
    import torch
    pc, (u, _, d) = env
    ours = torch.empty(V, dtype=torch.complex128, device="cuda:0")
    theirs = torch.empty_like(ours)
    for gij, gkl in ((15, 15), (5, 5), (8, 3)):
        pc.meson_two_point(ours, u, d, V, gij, gkl)
        torch.cuda.synchronize()
        ref.meson_two_point(theirs.data_ptr(), u.data_ptr(), d.data_ptr(), V, gij, gkl)
        assert _rel(ours, theirs) < TOL, (gij, gkl)
    ours16 = torch.empty((16, V), dtype=torch.complex128, device="cuda:0")
    theirs16 = torch.empty_like(ours16)
    pc.meson_all_source_two_point([ours16[g] for g in range(16)], u, d, V, 5)
    torch.cuda.synchronize()
    ref.meson_all_source_two_point([theirs16[g].data_ptr() for g in range(16)], u.data_ptr(), d.data_ptr(), V, 5)
    assert _rel(ours16, theirs16) < TOL
    pc.meson_all_sink_two_point([ours16[g] for g in range(16)], u, d, V, 15)
    torch.cuda.synchronize()
    ref.meson_all_sink_two_point([theirs16[g].data_ptr() for g in range(16)], u.data_ptr(), d.data_ptr(), V, 15)
    assert _rel(ours16, theirs16) < TOL


def test_diquark(ref, env):
    import torch
    pc, (u, _, d) = env
    ours = torch.empty_like(u)
    theirs = torch.empty_like(u)
    pc.baryon_diquark(ours, u, d, V, 5, 5)
    torch.cuda.synchronize()
    ref.baryon_diquark(theirs.data_ptr(), u.data_ptr(), d.data_ptr(), V, 5, 5)
    assert _rel(ours, theirs) < TOL


@pytest.mark.parametrize("contract_type", [0, 1])
def test_sequential_all_slots(ref, env, contract_type):
    """In-place sequential source for each slot; the other two buffers are read only."""
    import torch
    pc, (u, u2, d) = env
    for slot in range(3):
        ours = [u, u2, d]
        theirs = [u, u2, d]
        ours[slot] = torch.zeros_like(u)
        theirs[slot] = torch.zeros_like(u)
        pc.baryon_sequential_two_point(*ours, contract_type, slot, V, 5, 5, 8)
        torch.cuda.synchronize()
        ref.baryon_sequential_two_point(*(x.data_ptr() for x in theirs), contract_type, slot, V, 5, 5, 8)
        assert _rel(ours[slot], theirs[slot]) < TOL, slot
        del ours, theirs
