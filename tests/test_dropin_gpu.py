"""Every contract.h entry point, called through the C ABI on the GPU, against
the golden fixtures computed by the reference's own per-site arithmetic."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 kernels; only the summation order differs from the reference


@pytest.fixture(scope="module")
def pc():
    from contract_gb300 import build
    build.build()
    from contract_gb300 import pycontract
    pycontract.init(0)
    return pycontract


@pytest.fixture(scope="module")
def dev(golden):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(golden[k])).cuda() for k in ("pi", "pj", "pn")}


def _np(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_meson_two_point(pc, dev, golden):
    import torch
    v = dev["pi"].shape[0]
    out = torch.empty(v, dtype=torch.complex128, device="cuda")
    for a in range(16):
        for b in range(16):
            pc.meson_two_point(out, dev["pi"], dev["pj"], v, a, b)
            assert rel_err(_np(out), golden["meson"][a, b]) < TOL, (a, b)


def test_meson_all_source_and_sink(pc, dev, golden):
    import torch
    v = dev["pi"].shape[0]
    out = torch.empty((16, v), dtype=torch.complex128, device="cuda")
    pc.meson_all_source_two_point([out[g] for g in range(16)], dev["pi"], dev["pj"], v, 5)
    assert rel_err(_np(out), golden["meson_all_source"]) < TOL
    pc.meson_all_sink_two_point([out[g] for g in range(16)], dev["pi"], dev["pj"], v, 10)
    assert rel_err(_np(out), golden["meson_all_sink"]) < TOL
    for g in range(16):
        pc.meson_all_source_two_point([out[k] for k in range(16)], dev["pi"], dev["pj"], v, g)
        assert rel_err(_np(out), golden["meson"][g]) < TOL
        pc.meson_all_sink_two_point([out[k] for k in range(16)], dev["pi"], dev["pj"], v, g)
        assert rel_err(_np(out), golden["meson"][:, g]) < TOL


def test_baryon_two_point(pc, dev, golden):
    import torch
    v = dev["pi"].shape[0]
    out = torch.empty(v, dtype=torch.complex128, device="cuda")
    for g, (gij, gkl) in enumerate(golden["baryon_gammas"]):
        for t in range(6):
            for gmn in range(16):
                pc.baryon_two_point(out, dev["pi"], dev["pj"], dev["pn"], t, v, int(gij), int(gkl), gmn)
                assert rel_err(_np(out), golden["baryon"][g, t, gmn]) < TOL, (gij, gkl, t, gmn)


def test_baryon_general_two_point(pc, dev, golden):
    import torch
    v = dev["pi"].shape[0]
    out = torch.empty(v, dtype=torch.complex128, device="cuda")
    for p, proj in enumerate(golden["projectors"]):
        for t in range(6):
            pc.baryon_general_two_point(out, dev["pi"], dev["pj"], dev["pn"], t, v, 5, 5, proj)
            assert rel_err(_np(out), golden["general"][p, t]) < TOL, (p, t)


def test_baryon_diquark(pc, dev, golden):
    import torch
    n = golden["diquark"].shape[1]
    pi, pj = dev["pi"][:n].contiguous(), dev["pj"][:n].contiguous()
    out = torch.empty_like(pi)
    for k, (a, b) in enumerate(golden["diquark_gammas"]):
        pc.baryon_diquark(out, pi, pj, n, int(a), int(b))
        assert rel_err(_np(out), golden["diquark"][k]) < TOL, (a, b)


def test_baryon_sequential_two_point(pc, dev, golden):
    n = golden["sequential"].shape[3]
    for g, gmn in enumerate(golden["seq_gmn"]):
        for t in range(6):
            for s in range(3):
                bufs = [dev[k][:n].clone() for k in ("pi", "pj", "pn")]
                pc.baryon_sequential_two_point(*bufs, t, s, n, 5, 5, int(gmn))
                assert rel_err(_np(bufs[s]), golden["sequential"][g, t, s]) < TOL, (gmn, t, s)
                for k in range(3):  # the other two slots are untouched
                    if k != s:
                        assert np.array_equal(_np(bufs[k]), golden[("pi", "pj", "pn")[k]][:n])


def test_invalid_sequential_type_is_noop(pc, dev):
    import torch
    n = 4
    bufs = [dev[k][:n].clone() for k in ("pi", "pj", "pn")]
    before = [b.clone() for b in bufs]
    lib = pc._L()
    lib.contract_set_error_mode(0)
    lib.baryon_sequential_two_point(*[b.data_ptr() for b in bufs], 0, 5, n, 5, 5, 8)
    torch.cuda.synchronize()
    for a, b in zip(bufs, before):
        assert torch.equal(a, b)
    lib.contract_set_error_mode(1)
