"""The CPU oracles against the reference's own arithmetic (golden fixtures
produced by tests/golden/make_golden.py from the host-compiled reference)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import einsum_oracle as eo
from oracle import gamma as gm
from oracle import lib as L

TOL = 1e-12


def test_gamma_tables_bit_exact(golden):
    t = gm.tables()
    assert np.array_equal(t["index"], golden["gamma_index"])
    for k in ("data", "data_t", "g_g5", "g5_g_t"):
        assert np.array_equal(t[k], golden["gamma_" + k]), k


def test_c_oracle_gamma_tables(golden, c_oracle):
    idx, data = L.c_gamma_tables()
    assert np.array_equal(idx, golden["gamma_index"])
    assert np.array_equal(data, golden["gamma_data"])


def test_gamma_group_structure():
    g = gm.GAMMA
    for n in range(16):
        assert np.allclose(g[n] @ g[n].conj().T, np.eye(4))  # unitary
        p, ph = gm.perm_phase(g[n])
        assert np.array_equal(p[p], np.arange(4))  # involutive permutation
        assert set(np.round(ph, 12)) <= {1, -1, 1j, -1j}
    assert np.allclose(gm.G5, np.diag([1, 1, -1, -1]))


@pytest.mark.parametrize("impl", ["einsum", "c"])
def test_meson(golden, impl, c_oracle):
    pi, pj = golden["pi"], golden["pj"]
    for a in range(16):
        for b in range(16):
            got = eo.meson_two_point(pi, pj, a, b) if impl == "einsum" else c_oracle.meson_two_point(pi, pj, a, b)
            assert rel_err(got, golden["meson"][a, b]) < TOL, (a, b)


def test_meson_all(golden, c_oracle):
    pi, pj = golden["pi"], golden["pj"]
    assert rel_err(c_oracle.meson_all_source(pi, pj, 5), golden["meson_all_source"]) < TOL
    assert rel_err(c_oracle.meson_all_sink(pi, pj, 10), golden["meson_all_sink"]) < TOL
    assert rel_err(eo.meson_all_source(pi, pj, 5), golden["meson_all_source"]) < TOL
    assert rel_err(eo.meson_all_gamma(pi, pj)[:, 10], golden["meson_all_sink"]) < TOL


@pytest.mark.parametrize("impl", ["einsum", "c"])
def test_baryon(golden, impl, c_oracle):
    pi, pj, pn = golden["pi"], golden["pj"], golden["pn"]
    for g, (gij, gkl) in enumerate(golden["baryon_gammas"]):
        for t in range(6):
            for gmn in range(16):
                f = eo.baryon_two_point if impl == "einsum" else c_oracle.baryon_two_point
                got = f(pi, pj, pn, t, int(gij), int(gkl), gmn)
                assert rel_err(got, golden["baryon"][g, t, gmn]) < TOL, (gij, gkl, t, gmn)


@pytest.mark.parametrize("impl", ["einsum", "c"])
def test_baryon_general(golden, impl, c_oracle):
    pi, pj, pn = golden["pi"], golden["pj"], golden["pn"]
    for p, proj in enumerate(golden["projectors"]):
        for t in range(6):
            f = eo.baryon_general_two_point if impl == "einsum" else c_oracle.baryon_general_two_point
            assert rel_err(f(pi, pj, pn, t, 5, 5, proj), golden["general"][p, t]) < TOL, (p, t)


@pytest.mark.parametrize("impl", ["einsum", "c"])
def test_diquark(golden, impl, c_oracle):
    n = golden["diquark"].shape[1]
    pi, pj = golden["pi"][:n], golden["pj"][:n]
    for k, (a, b) in enumerate(golden["diquark_gammas"]):
        f = eo.baryon_diquark if impl == "einsum" else c_oracle.baryon_diquark
        assert rel_err(f(pi, pj, int(a), int(b)), golden["diquark"][k]) < TOL, (a, b)


@pytest.mark.parametrize("impl", ["einsum", "c"])
def test_sequential(golden, impl, c_oracle):
    n = golden["sequential"].shape[3]
    pi, pj, pn = golden["pi"][:n], golden["pj"][:n], golden["pn"][:n]
    for g, gmn in enumerate(golden["seq_gmn"]):
        for t in range(6):
            for s in range(3):
                f = eo.baryon_sequential if impl == "einsum" else c_oracle.baryon_sequential
                got = f(pi, pj, pn, t, s, 5, 5, int(gmn))
                assert rel_err(got, golden["sequential"][g, t, s]) < TOL, (gmn, t, s)


def test_sequential_euler_identity(golden, c_oracle):
    """C is trilinear: sum over one propagator's entries of P * dC/dP equals C."""
    pi, pj, pn = golden["pi"], golden["pj"], golden["pn"]
    for t in range(6):
        c = c_oracle.baryon_two_point(pi, pj, pn, t, 5, 13, 8)
        for s, p in enumerate((pi, pj, pn)):
            d = c_oracle.baryon_sequential(pi, pj, pn, t, s, 5, 13, 8)
            lhs = np.einsum("xikad,xikad->x", p.reshape(-1, 4, 4, 3, 3), d.reshape(-1, 4, 4, 3, 3))
            assert rel_err(lhs, c) < 1e-12


def test_reference_host_build_matches_golden(golden):
    """Only where the reference sources were available to build oracle/_ref."""
    ref = L.ref_oracle()
    if ref is None:
        pytest.skip("oracle/_ref/libcontract_ref.so not built here (reference sources absent)")
    pi, pj, pn = golden["pi"], golden["pj"], golden["pn"]
    assert rel_err(ref.meson_two_point(pi, pj, 7, 12), golden["meson"][7, 12]) == 0.0
    assert rel_err(ref.baryon_two_point(pi, pj, pn, 3, 5, 5, 8), golden["baryon"][0, 3, 8]) == 0.0


def test_timeslice_and_momentum_helpers():
    latt = (4, 2, 2, 6)
    x, y, z, t = eo.eo_coords(latt)
    assert len(x) == 4 * 2 * 2 * 6
    # every coordinate appears exactly once
    lin = ((t * 2 + z) * 2 + y) * 4 + x
    assert np.array_equal(np.sort(lin), np.arange(len(lin)))
    f = np.arange(len(x)).astype(np.complex128)
    ts = eo.timeslice_sum(f, latt)
    assert np.allclose(ts, [f[t == k].sum() for k in range(6)])
    mp = eo.momentum_project(f, latt, [[0, 0, 0], [1, 0, 0]])
    assert np.allclose(mp[0], ts)
    ph = np.exp(2j * np.pi * x / 4)
    assert np.allclose(mp[1], [(f * ph)[t == k].sum() for k in range(6)])
