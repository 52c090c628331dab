"""Batched meson momentum projection and the mixed batch (baryon items and
meson items in three launches: two persistent kernels and one combined
finalisation), on lattices of uneven extents, against per-item calls and the
FP64 oracle; CUDA-graph replay; per-extent tile-shape tuning."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err
from oracle import einsum_oracle as eo

pytestmark = pytest.mark.gpu

TOL_C64_TIMESLICE = 1e-6  # |got - ref| <= 1e-6 max(|ref|, sigma), as for the per-call mixed forms
MESON_LATTS = [(4, 4, 4, 8), (6, 4, 4, 6), (4, 4, 4, 8), (10, 4, 4, 2), (4, 4, 16, 16)]  # every extent >= 3
BARYON_LATTS = [(4, 4, 4, 8), (4, 2, 2, 6), (6, 4, 2, 4)]


class MesonItem(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("correl", ctypes.c_void_p),
                ("lattice", ctypes.c_int * 4)]


class BaryonItem(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("propag_n", ctypes.c_void_p),
                ("correl", ctypes.c_void_p), ("lattice", ctypes.c_int * 4)]


@pytest.fixture(scope="module")
def lib():
    from contract_gb300 import _lib, build, pycontract
    build.build()
    pycontract.init(0)
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    return lib


def c64(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda().to(torch.complex64)


def moms_arg(moms):
    m = np.ascontiguousarray(np.asarray(moms, dtype=np.int32))
    return m, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def meson_set(same=False, seed=300):
    """Meson items: host propagators, device complex64 copies, outputs."""
    import torch
    moms = eo.momentum_list(1)
    out = []
    for k, latt in enumerate(MESON_LATTS):
        pi = eo.make_propagator(latt, seed + 2 * k, 0.2)
        pj = pi if same else eo.make_propagator(latt, seed + 2 * k + 1, 0.25)
        a = c64(pi)
        b = a if same else c64(pj)
        o = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        out.append({"latt": latt, "pi": pi, "pj": pj, "a": a, "b": b, "out": o})
    return moms, out


def baryon_set(seed=400):
    import torch
    out = []
    for k, latt in enumerate(BARYON_LATTS):
        ps = [eo.make_propagator(latt, seed + 3 * k + s, 0.1 + 0.1 * s) for s in range(3)]
        dev = [c64(p) for p in ps]
        o = torch.full((6, 2, latt[3]), float("nan"), dtype=torch.complex128, device="cuda")
        out.append({"latt": latt, "ps": ps, "dev": dev, "out": o})
    return out


def meson_items(ms):
    arr = (MesonItem * len(ms))()
    for k, m in enumerate(ms):
        arr[k].propag_i, arr[k].propag_j = m["a"].data_ptr(), m["b"].data_ptr()
        arr[k].correl = m["out"].data_ptr()
        arr[k].lattice = (ctypes.c_int * 4)(*m["latt"])
    return arr


def baryon_items(bs):
    arr = (BaryonItem * len(bs))()
    for k, b in enumerate(bs):
        arr[k].propag_i, arr[k].propag_j, arr[k].propag_n = (x.data_ptr() for x in b["dev"])
        arr[k].correl = b["out"].data_ptr()
        arr[k].lattice = (ctypes.c_int * 4)(*b["latt"])
    return arr


def per_call_meson(lib, m, moms):
    import torch
    ref = torch.empty_like(m["out"])
    mm, mp = moms_arg(moms)
    v = m["pi"].shape[0]
    lib.contract_meson_all_gamma_momentum(ref.data_ptr(), m["a"].data_ptr(), m["b"].data_ptr(), v,
                                          (ctypes.c_int * 4)(*m["latt"]), mp, len(moms), 1)
    return ref.cpu().numpy()


def check_meson_oracle(m, moms, got):
    site = eo.meson_all_gamma(m["pi"], m["pj"]).reshape(256, -1)
    ref = eo.momentum_project(site, m["latt"], moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, m["latt"]).real).T[None]
    l1 = eo.meson_product_l1(m["pi"], m["pj"], m["latt"]) if m["pi"] is m["pj"] else 0.0
    err = np.abs(got - ref) / np.maximum(np.maximum(np.abs(ref), sig), l1)
    assert err.max() < TOL_C64_TIMESLICE, (m["latt"], err.max())


@pytest.mark.parametrize("same", [False, True])
def test_meson_momentum_batch_matches_per_call(lib, same):
    """Every item of one batched launch equals its own per-call projection
    (same kernel arithmetic, so bit for bit) and the FP64 oracle."""
    import torch
    moms, ms = meson_set(same)
    mm, mp = moms_arg(moms)
    lib.contract_clear_error()
    lib.contract_meson_all_gamma_momentum_batch(meson_items(ms), len(ms), mp, len(moms), 1)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    for m in ms:
        got = m["out"].cpu().numpy()
        assert np.array_equal(got, per_call_meson(lib, m, moms)), m["latt"]
        check_meson_oracle(m, moms, got)
    assert lib.contract_check_device() == 0


def test_mixed_batch_and_graph_replay(lib):
    """Baryon and meson items of one mixed call against per-item calls and the
    oracle, directly and replayed from a CUDA graph."""
    import torch

    from contract_gb300 import api
    pp = np.ascontiguousarray(api.projector_plus_minus())
    moms, ms = meson_set(False, seed=500)
    bs = baryon_set()
    mm, mp = moms_arg(moms)
    barr, marr = baryon_items(bs), meson_items(ms)

    def call():
        lib.contract_batch_mixed(barr, len(bs), 5, 5, 2, pp.ctypes.data, marr, len(ms), mp, len(moms), 1)

    def check():
        for b in bs:
            got = b["out"].cpu().numpy()
            # the per-call pass runs the same site arithmetic, but its chunks of
            # sites (and so its FP32 partial sums) fall differently
            ref = api.baryon_all_types(*b["dev"], 5, 5, pp, latt=b["latt"]).cpu().numpy()
            assert rel_err(got, ref) < 1e-6, b["latt"]
            # and the oracle on the original FP64 propagators (sigma-normalised, per timeslice)
            site = np.array([[eo.baryon_general_two_point(*b["ps"], t, 5, 5, pp[w]) for w in range(2)]
                             for t in range(6)])
            oref = eo.timeslice_sum(site, b["latt"])
            sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, b["latt"]).real)
            assert (np.abs(got - oref) / np.maximum(np.abs(oref), sig)).max() < TOL_C64_TIMESLICE
        for m in ms:
            got = m["out"].cpu().numpy()
            assert np.array_equal(got, per_call_meson(lib, m, moms)), m["latt"]
            check_meson_oracle(m, moms, got)

    lib.contract_clear_error()
    call()
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    check()
    # graph: warm-up on the capture stream, then capture and replay
    for x in bs + ms:
        x["out"].fill_(float("nan"))
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        lib.contract_set_stream(s.cuda_stream)
        call()
    torch.cuda.current_stream().wait_stream(s)
    for x in bs + ms:
        x["out"].fill_(float("nan"))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        lib.contract_set_stream(torch.cuda.current_stream().cuda_stream)
        call()
    lib.contract_set_stream(None)
    g.replay()
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    check()
    assert lib.contract_check_device() == 0


def test_mixed_batch_tunes_per_extent(lib):
    """With autotuning on, every lattice class of each kind is timed alone and
    the launch takes the shape with the least total; the report names each
    class's best shape and the batch's choice, and the results stay right."""
    import torch

    from contract_gb300 import api
    pp = np.ascontiguousarray(api.projector_plus_minus())
    moms, ms = meson_set(True, seed=700)
    bs = baryon_set(seed=800)
    mm, mp = moms_arg(moms)
    lib.contract_set_autotune(1)
    try:
        lib.contract_clear_error()
        lib.contract_batch_mixed(baryon_items(bs), len(bs), 5, 5, 2, pp.ctypes.data, meson_items(ms), len(ms), mp,
                                 len(moms), 1)
        torch.cuda.synchronize()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    finally:
        lib.contract_set_autotune(0)
    buf = ctypes.create_string_buffer(1 << 16)
    lib.contract_autotune_report(buf, len(buf))
    rep = buf.value.decode()
    for latt in set(BARYON_LATTS):
        assert "batch=baryon,nproj=2,same=0,latt=" + ",".join(map(str, latt)) in rep, rep
    for latt in set(MESON_LATTS):
        assert "batch=meson_momentum,nmom=27,same=1,latt=" + ",".join(map(str, latt)) in rep, rep
    assert "batch=baryon,nproj=2,same=0,batch=" in rep and "batch=meson_momentum,nmom=27,same=1,batch=" in rep
    for b in bs:
        ref = api.baryon_all_types(*b["dev"], 5, 5, pp, latt=b["latt"]).cpu().numpy()
        assert rel_err(b["out"].cpu().numpy(), ref) < TOL_C64_TIMESLICE
    for m in ms:
        check_meson_oracle(m, moms, m["out"].cpu().numpy())


def test_meson_batch_rejects_mismatched_plans(lib):
    """n = +-2 are one group on L = 4 and two on L = 6: the plans' structures
    differ, and the batch refuses the call before any launch."""
    import torch
    moms = np.array([[2, 0, 0], [-2, 0, 0], [0, 0, 0]], dtype=np.int32)
    ms = []
    for latt in ((4, 4, 4, 4), (6, 4, 4, 4)):
        p = c64(eo.make_propagator(latt, 9, 0.2))
        ms.append({"latt": latt, "a": p, "b": p, "out": torch.zeros((3, latt[3], 256), dtype=torch.complex128,
                                                                     device="cuda")})
    mm, mp = moms_arg(moms)
    lib.contract_clear_error()
    lib.contract_meson_all_gamma_momentum_batch(meson_items(ms), 2, mp, 3, 1)
    assert lib.contract_last_error() == 1 and b"another structure" in lib.contract_last_error_message()
    lib.contract_clear_error()
    lib.contract_meson_all_gamma_momentum_batch(meson_items(ms), 2, mp, 3, 0)  # complex128: not batched
    assert lib.contract_last_error() == 1 and b"CONTRACT_C64" in lib.contract_last_error_message()
    lib.contract_clear_error()
