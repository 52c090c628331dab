"""GPU kernels against the C oracle on seeded lattices larger than the golden
fixtures: ragged tails, odd volumes, both precisions, per-site and
per-timeslice outputs, and the fused all-types kernel."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import einsum_oracle as eo

pytestmark = pytest.mark.gpu
TOL_C128 = 1e-12           # plain form (FP64 throughout)
# Mixed form (complex64 storage, FP32 arithmetic, FP64 timeslice reduction):
# |got_t - ref_t| <= 1e-6 * max(|ref_t|, sigma_t), sigma_t = sqrt(sum_{x in t} |ref(x)|^2).
# On timeslices with a signal (|ref_t| >= sigma_t) this is the plain 1e-6
# relative bound; with the i.i.d. Gaussian test propagators every timeslice is
# a zero-mean random walk of site values, and sigma_t is its natural scale.
TOL_C64_TIMESLICE = 1e-6
# Tensor-core momentum projection (CONTRACT_C64_TC): each operand is split
# into three bf16 terms (24 significant bits) and every term pair down to
# second order is kept (the terms dropped are of order 2^-24 of a product),
# with FP32 accumulation drained to round-to-nearest registers every 12 MMAs;
# the error bound is that of the other mixed forms, relative to max(|C_t|, sigma_t).
TOL_C64_TC = 1e-6
# Mixed momentum projection with one field in both propagator slots: relative
# to max(|C|, sigma, L1), L1 the largest per-timeslice sum of |T(x)| over the
# spin-colour products (oracle.einsum_oracle.meson_product_l1).  The diagonal
# products are then positive at every site: an FP32 projection to nonzero
# momentum cancels terms of size L1, and at zero momentum the Gamma pairs with
# opposite signs on the diagonal cancel them (in the FP32 sums, and in the
# product -> pair map, which is compensated).  Measured on the test lattices:
# 1.2-4.0e-7 of L1.
TOL_C64_COHERENT = 1e-6

LATT = (4, 4, 4, 8)


@pytest.fixture(scope="module")
def props():
    pi = eo.make_propagator(LATT, 21, 0.25)
    pj = eo.make_propagator(LATT, 22, 0.25)
    pn = eo.make_propagator(LATT, 23, 0.30)
    return pi, pj, pn


@pytest.fixture(scope="module")
def api():
    from contract_gb300 import build
    build.build()
    from contract_gb300 import api, pycontract
    pycontract.init(0)
    return api


def cuda(a, c64=False):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t.to(torch.complex64) if c64 else t


def per_t_rel(got, ref, site):
    """max_t |got_t - ref_t| / max(|ref_t|, sigma_t) for per-site values `site` [..., V]."""
    got, ref = np.asarray(got), np.asarray(ref)
    sigma = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, LATT).real)
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), sigma)))


def test_ragged_volumes(api, props, c_oracle):
    """Volumes that are not multiples of any tile (the reference needs volume % 4 == 0)."""
    from contract_gb300 import pycontract as pc
    for v in (1, 3, 37, 129, 200):
        pi, pj, pn = [p[:v] for p in props]
        got = pc.baryonTwoPoint(cuda(pi), cuda(pj), cuda(pn), 1, 5, 5, 8).cpu().numpy()
        assert rel_err(got, c_oracle.baryon_two_point(pi, pj, pn, 1, 5, 5, 8)) < TOL_C128, v
        got = pc.mesonTwoPoint(cuda(pi), cuda(pj), 15, 15).cpu().numpy()
        assert rel_err(got, c_oracle.meson_two_point(pi, pj, 15, 15)) < TOL_C128, v


def test_mixed_ragged_volumes_and_gammas(api, props, c_oracle):
    """complex64 per-site values through the drop-in functions on ragged volumes
    and a sweep of gamma selectors (including phased and diagonal ones), against
    the FP64 oracle relative to the largest value."""
    from contract_gb300 import pycontract as pc
    for v in (1, 3, 37, 129, 200):
        pi, pj, pn = [p[:v] for p in props]
        got = pc.baryonTwoPoint(cuda(pi, True), cuda(pj, True), cuda(pn, True), 1, 5, 5, 8).cpu().numpy()
        assert rel_err(got, c_oracle.baryon_two_point(pi, pj, pn, 1, 5, 5, 8)) < 1e-6, v
        got = pc.mesonTwoPoint(cuda(pi, True), cuda(pj, True), 15, 15).cpu().numpy()
        assert rel_err(got, c_oracle.meson_two_point(pi, pj, 15, 15)) < 1e-6, v
    pi, pj, pn = [p[:96] for p in props]
    a, b, c = cuda(pi, True), cuda(pj, True), cuda(pn, True)
    for gij, gkl in ((5, 5), (13, 13), (0, 15), (3, 10), (15, 6), (9, 12)):
        got = pc.mesonTwoPoint(a, b, gij, gkl).cpu().numpy()
        assert rel_err(got, c_oracle.meson_two_point(pi, pj, gij, gkl)) < 1e-6, (gij, gkl)
        got = pc.baryonDiquark(a, b, gij, gkl).cpu().numpy().astype(np.complex128)
        assert rel_err(got, c_oracle.baryon_diquark(pi, pj, gij, gkl)) < 1e-6, (gij, gkl)
        for t in range(6):
            for gmn in (0, 8, 15):
                got = pc.baryonTwoPoint(a, b, c, t, gij, gkl, gmn).cpu().numpy()
                ref = c_oracle.baryon_two_point(pi, pj, pn, t, gij, gkl, gmn)
                assert rel_err(got, ref) < 1e-6, (gij, gkl, t, gmn)
    # a dense projector (the materialised-N' triangle and the loop form) for every type
    rng = np.random.default_rng(29)
    dense = (rng.standard_normal(16) + 1j * rng.standard_normal(16)) / 4
    for t in range(6):
        got = api.baryon(a, b, c, t, 5, 5, project_mn=dense).cpu().numpy()
        assert rel_err(got, c_oracle.baryon_general_two_point(pi, pj, pn, t, 5, 5, dense)) < 1e-6, t
    # the all-sink meson (all 16 Gamma_ij at one Gamma_kl), per site
    for gkl in (5, 10):
        got = pc.mesonAllSinkTwoPoint(a, b, gkl).cpu().numpy()
        assert rel_err(got, c_oracle.meson_all_sink(pi, pj, gkl)) < 1e-6, gkl


def test_low_rank_projectors(api, props, c_oracle):
    """Projectors of rank 2 ((1 +- g4)/2) and rank 1 (polarised) through the
    per-call general two-point, every type, phased and unphased gammas, both
    precisions, against the FP64 oracle; the triangle types take the factored
    form (r colour wedges per spin pair)."""
    from contract_gb300 import _lib
    from contract_gb300.pycontract import gamma_matrices
    lib = _lib.lib()
    g, e = gamma_matrices(), np.eye(4)
    projs = [(e + g[8]) / 2, (e - g[8]) / 2, (e + g[8]) @ (e - 1j * g[3]) / 4, (e - g[8]) @ (e + 1j * g[3]) / 4,
             np.outer([0.5, 0, -1j, 0.25], [1, 2j, 0, -0.5])]  # last: factors not all of one modulus
    pi, pj, pn = [p[:200] for p in props]
    dev = {prec: [cuda(p, prec) for p in (pi, pj, pn)] for prec in (False, True)}
    for w, rank in zip(projs, (2, 2, 1, 1, 1)):
        w = np.ascontiguousarray(w.reshape(16))
        assert lib.contract_projector_rank(w.ctypes.data) == rank
        for gij, gkl in ((5, 5), (13, 10)):
            for t in range(6):
                ref = c_oracle.baryon_general_two_point(pi, pj, pn, t, gij, gkl, w)
                got = api.baryon(*dev[False], t, gij, gkl, project_mn=w).cpu().numpy()
                assert rel_err(got, ref) < TOL_C128, (rank, gij, gkl, t)
                got = api.baryon(*dev[True], t, gij, gkl, project_mn=w).cpu().numpy()
                assert rel_err(got, ref) < 1e-6, (rank, gij, gkl, t)


def test_empty_volume(api):
    import torch
    from contract_gb300 import pycontract as pc
    z = torch.empty((0, 4, 4, 3, 3), dtype=torch.complex128, device="cuda")
    assert pc.mesonTwoPoint(z, z, 5, 5).numel() == 0
    assert pc.baryonTwoPoint(z, z, z, 0, 5, 5, 8).numel() == 0


def test_baryon_all_types_all_gammas_c128(api, props, c_oracle):
    from contract_gb300 import pycontract as pc
    pi, pj, pn = props
    a, b, c = cuda(pi), cuda(pj), cuda(pn)
    for gij, gkl in ((5, 5), (13, 13), (0, 15), (3, 10)):
        for t in range(6):
            for gmn in (0, 8, 4, 15):
                got = pc.baryonTwoPoint(a, b, c, t, gij, gkl, gmn).cpu().numpy()
                assert rel_err(got, c_oracle.baryon_two_point(pi, pj, pn, t, gij, gkl, gmn)) < TOL_C128


def test_meson_all_per_timeslice(api, props, c_oracle):
    pi, pj, _ = props
    got = api.meson_all_timeslice(cuda(pi), cuda(pj), LATT, 5, source=True).cpu().numpy()
    site = c_oracle.meson_all_source(pi, pj, 5)
    ref = eo.timeslice_sum(site, LATT)
    assert rel_err(got, ref) < TOL_C128
    got64 = api.meson_all_timeslice(cuda(pi, True), cuda(pj, True), LATT, 5, source=True).cpu().numpy()
    for g in range(16):
        assert per_t_rel(got64[g], ref[g], site[g]) < TOL_C64_TIMESLICE, g


def test_baryon_timeslice_both_precisions(api, props, c_oracle):
    pi, pj, pn = props
    pp = api.projector_plus_minus()
    for t in range(6):
        site = c_oracle.baryon_general_two_point(pi, pj, pn, t, 5, 5, pp[0])
        ref = eo.timeslice_sum(site, LATT)
        got = api.baryon(cuda(pi), cuda(pj), cuda(pn), t, 5, 5, project_mn=pp[0], latt=LATT).cpu().numpy()
        assert rel_err(got, ref) < TOL_C128, t
        got64 = api.baryon(cuda(pi, True), cuda(pj, True), cuda(pn, True), t, 5, 5, project_mn=pp[0],
                           latt=LATT).cpu().numpy()
        assert per_t_rel(got64, ref, site) < TOL_C64_TIMESLICE, t


def test_fused_all_types(api, props, c_oracle):
    pi, pj, pn = props
    pp = api.projector_plus_minus()
    ref = np.zeros((6, 2, LATT[3]), np.complex128)
    ref_site = np.zeros((6, 2, pi.shape[0]), np.complex128)
    for t in range(6):
        for w in range(2):
            ref_site[t, w] = c_oracle.baryon_general_two_point(pi, pj, pn, t, 5, 5, pp[w])
            ref[t, w] = eo.timeslice_sum(ref_site[t, w], LATT)
    got = api.baryon_all_types(cuda(pi), cuda(pj), cuda(pn), 5, 5, pp, latt=LATT).cpu().numpy()
    assert rel_err(got, ref) < TOL_C128
    got_site = api.baryon_all_types(cuda(pi), cuda(pj), cuda(pn), 5, 5, pp).cpu().numpy()
    assert rel_err(got_site, ref_site) < TOL_C128
    got1 = api.baryon_all_types(cuda(pi), cuda(pj), cuda(pn), 5, 5, pp[:1], latt=LATT).cpu().numpy()
    assert rel_err(got1[:, 0], ref[:, 0]) < TOL_C128
    got64 = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT).cpu().numpy()
    for t in range(6):
        for w in range(2):
            assert per_t_rel(got64[t, w], ref[t, w], ref_site[t, w]) < TOL_C64_TIMESLICE, (t, w)


def test_fused_all_types_phased_projectors(api, props, c_oracle):
    """Both fused forms with (1 +- i g1 g2)/2: two gamma-basis terms whose spin
    phases are not all +1, the path the (1 +- g4)/2 projectors skip."""
    from contract_gb300.pycontract import gamma_matrices
    pi, pj, pn = props
    g12 = gamma_matrices()[3]
    e = np.eye(4)
    pp = np.stack([((e + 1j * g12) / 2).reshape(16), ((e - 1j * g12) / 2).reshape(16)])
    ref = np.zeros((6, 2, LATT[3]), np.complex128)
    ref_site = np.zeros((6, 2, pi.shape[0]), np.complex128)
    for t in range(6):
        for w in range(2):
            ref_site[t, w] = c_oracle.baryon_general_two_point(pi, pj, pn, t, 5, 5, pp[w])
            ref[t, w] = eo.timeslice_sum(ref_site[t, w], LATT)
    got = api.baryon_all_types(cuda(pi), cuda(pj), cuda(pn), 5, 5, pp, latt=LATT).cpu().numpy()
    assert rel_err(got, ref) < TOL_C128
    got64 = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT).cpu().numpy()
    for t in range(6):
        for w in range(2):
            assert per_t_rel(got64[t, w], ref[t, w], ref_site[t, w]) < TOL_C64_TIMESLICE, (t, w)


def test_fused_all_types_one_and_four_term_projectors(api, props, c_oracle):
    """The fused forms' general branch: a one-term projector (g4) and the
    polarised (1 + g4)(1 - i g1 g2)/4, four gamma-basis terms."""
    from contract_gb300.pycontract import gamma_matrices
    pi, pj, pn = props
    g = gamma_matrices()
    e = np.eye(4)
    pol = ((e + g[8]) @ (e - 1j * g[3]) / 4).reshape(16)
    pp = np.stack([g[8].reshape(16), pol])
    ref = np.zeros((6, 2, LATT[3]), np.complex128)
    ref_site = np.zeros((6, 2, pi.shape[0]), np.complex128)
    for t in range(6):
        for w in range(2):
            ref_site[t, w] = c_oracle.baryon_general_two_point(pi, pj, pn, t, 5, 5, pp[w])
            ref[t, w] = eo.timeslice_sum(ref_site[t, w], LATT)
    for w in range(2):  # one projector per call
        got = api.baryon_all_types(cuda(pi), cuda(pj), cuda(pn), 5, 5, pp[w:w + 1], latt=LATT).cpu().numpy()
        assert rel_err(got[:, 0], ref[:, w]) < TOL_C128
        got64 = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp[w:w + 1],
                                     latt=LATT).cpu().numpy()
        for t in range(6):
            assert per_t_rel(got64[t, 0], ref[t, w], ref_site[t, w]) < TOL_C64_TIMESLICE, (t, w)


def test_fused_all_types_one_low_rank_projector(api, props, c_oracle):
    """One projector of rank 2 ((1 +- g4)/2) or rank 1 (polarised) through the
    fused pass, which takes the factored triangle form for it: per timeslice
    and per site, two fields and one field for P_i and P_j, phased gammas,
    both precisions, against the FP64 oracle."""
    from contract_gb300.pycontract import gamma_matrices
    pi, pj, pn = props
    g, e = gamma_matrices(), np.eye(4)
    for w in ((e + g[8]) / 2, (e - g[8]) / 2, (e + g[8]) @ (e - 1j * g[3]) / 4):
        w = np.ascontiguousarray(w.reshape(1, 16))
        for gij, gkl, one_field in ((5, 5, False), (5, 5, True), (13, 10, False)):
            b = pi if one_field else pj
            site = np.array([c_oracle.baryon_general_two_point(pi, b, pn, t, gij, gkl, w[0]) for t in range(6)])
            ref = eo.timeslice_sum(site, LATT)
            for c64 in (False, True):
                da, dn = cuda(pi, c64), cuda(pn, c64)
                db = da if one_field else cuda(pj, c64)
                got = api.baryon_all_types(da, db, dn, gij, gkl, w, latt=LATT).cpu().numpy()[:, 0]
                if c64:
                    for t in range(6):
                        assert per_t_rel(got[t], ref[t], site[t]) < TOL_C64_TIMESLICE, (gij, gkl, one_field, t)
                else:
                    assert rel_err(got, ref) < TOL_C128, (gij, gkl, one_field)
                    got = api.baryon_all_types(da, db, dn, gij, gkl, w).cpu().numpy()[:, 0]  # per site
                    assert rel_err(got, site) < TOL_C128, (gij, gkl, one_field)


def test_fused_same_field_c128(api, props, c_oracle):
    """complex128 with one pointer for P_i and P_j: the one-pass shared-wedge form
    (and, for Gamma_ij = g5, whose permutation has fixed points, the merged
    one-pass form), one and two projectors, against the oracle."""
    pi, _, pn = props
    pp = api.projector_plus_minus()
    a, c = cuda(pi), cuda(pn)
    for gij, gkl in ((5, 5), (15, 5)):
        ref = np.zeros((6, 2, LATT[3]), np.complex128)
        for t in range(6):
            for w in range(2):
                ref[t, w] = eo.timeslice_sum(c_oracle.baryon_general_two_point(pi, pi, pn, t, gij, gkl, pp[w]), LATT)
        got = api.baryon_all_types(a, a, c, gij, gkl, pp, latt=LATT).cpu().numpy()
        assert rel_err(got, ref) < TOL_C128, (gij, gkl)
        got1 = api.baryon_all_types(a, a, c, gij, gkl, pp[:1], latt=LATT).cpu().numpy()
        assert rel_err(got1[:, 0], ref[:, 0]) < TOL_C128, (gij, gkl)


def test_fused_same_field_for_i_and_j(api, props, c_oracle):
    """P_i and P_j passed as one pointer (the u quark of a proton): the complex64
    fused pass evaluates one triangle pass instead of two; per call, in a batch
    and from host memory it matches the two-pass result on a copy."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi, _, pn = props
    pp = np.ascontiguousarray(api.projector_plus_minus())
    a, c = cuda(pi, True), cuda(pn, True)
    same = api.baryon_all_types(a, a, c, 5, 5, pp, latt=LATT).cpu().numpy()
    two = api.baryon_all_types(a, a.clone(), c, 5, 5, pp, latt=LATT).cpu().numpy()
    # the one-pass form and the two-pass form on a copy agree to FP32 rounding;
    # every entry is checked against the oracle on its own scale below
    assert np.abs(same - two).max() <= 1e-6 * np.abs(two).max()
    # one projector; phased gammas; a dense projector (the two-pass general form)
    rng = np.random.default_rng(17)
    dense = (rng.standard_normal(16) + 1j * rng.standard_normal(16)).reshape(1, 16)
    # (15: g5 is diagonal, a Gamma_ij permutation with fixed points -> the merged one-pass form)
    for gij, gkl, projs in ((5, 5, pp[:1]), (13, 10, pp), (5, 5, dense), (15, 5, pp), (0, 13, pp)):
        s1 = api.baryon_all_types(a, a, c, gij, gkl, projs, latt=LATT).cpu().numpy()
        t1 = api.baryon_all_types(a, a.clone(), c, gij, gkl, projs, latt=LATT).cpu().numpy()
        # some types vanish identically for one field (e.g. with Gamma_ij = g5): their
        # FP32 values are rounding noise, measured on the scale of the case's
        # largest per-timeslice spread
        sites = np.array([[c_oracle.baryon_general_two_point(pi, pi, pn, t, gij, gkl, projs[w])
                           for w in range(projs.shape[0])] for t in range(6)])
        ref = eo.timeslice_sum(sites, LATT)
        scale = np.sqrt(eo.timeslice_sum(np.abs(sites) ** 2, LATT).real).max(axis=(0, 1))
        for got in (s1, t1):
            err = np.abs(got - ref) / np.maximum(np.abs(ref), scale)
            assert err.max() < TOL_C64_TIMESLICE, (gij, gkl, err.max())
    for t in range(6):
        for w in range(2):
            site = c_oracle.baryon_general_two_point(pi, pi, pn, t, 5, 5, pp[w])
            assert per_t_rel(same[t, w], eo.timeslice_sum(site, LATT), site) < TOL_C64_TIMESLICE, (t, w)
    # batched: every item with one field for P_i and P_j
    items, outs, refs = [], [], []
    for k, latt in enumerate(BATCH_LATTS):
        u = cuda(eo.make_propagator(latt, 200 + k, 0.2), True)
        d = cuda(eo.make_propagator(latt, 300 + k, 0.3), True)
        items.append((u, u, d, latt))
        refs.append(api.baryon_all_types(u, u, d, 5, 5, pp, latt=latt).cpu().numpy())
        outs.append(torch.full((6, 2, latt[3]), float("nan"), dtype=torch.complex128, device="cuda"))
    arr = _batch_items(items, outs, lib)
    lib.contract_baryon_all_types_batch(arr, len(outs), 5, 5, 2, pp.ctypes.data, 1)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    for out, ref in zip(outs, refs):
        assert rel_err(out.cpu().numpy(), ref) < 1e-12
    # the same batch with P_j a copy of P_i: the two-pass batched form
    items2 = [(u, u.clone(), d, latt) for (u, _, d, latt) in items]
    outs2 = [torch.full_like(o, float("nan")) for o in outs]
    arr2 = _batch_items(items2, outs2, lib)
    lib.contract_baryon_all_types_batch(arr2, len(outs2), 5, 5, 2, pp.ctypes.data, 1)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    for out, out2 in zip(outs, outs2):
        a2, b2 = out.cpu().numpy(), out2.cpu().numpy()
        assert np.abs(a2 - b2).max() <= 1e-6 * np.abs(b2).max()
    # from host memory, P_j the same host buffer as P_i (copied once)
    hu = torch.from_numpy(np.ascontiguousarray(pi)).pin_memory()
    hd = torch.from_numpy(np.ascontiguousarray(pn)).pin_memory()
    hout = torch.empty((6, 2, LATT[3]), dtype=torch.complex128).pin_memory()
    lib.contract_baryon_all_types_host(hout.data_ptr(), hu.data_ptr(), hu.data_ptr(), hd.data_ptr(), pi.shape[0], 5, 5,
                                       2, pp.ctypes.data, 1, (ctypes.c_int * 4)(*LATT))
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    assert np.abs(hout.numpy() - same).max() <= 1e-6 * np.abs(same).max()
    api.check_device()


def test_mixed_field_ops(api, props, c_oracle):
    """complex64 diquark/sequential fields: elementwise error at FP32 level."""
    import torch
    from contract_gb300 import pycontract as pc
    pi, pj, pn = [p[:64] for p in props]
    ref = c_oracle.baryon_diquark(pi, pj, 5, 5)
    got = pc.baryonDiquark(cuda(pi, True), cuda(pj, True), 5, 5).to(torch.complex128).cpu().numpy()
    assert rel_err(got, ref) < 1e-6
    for t in range(6):
        for s in range(3):
            ref = c_oracle.baryon_sequential(pi, pj, pn, t, s, 5, 5, 8)
            bufs = [cuda(p, True) for p in (pi, pj, pn)]
            pc.baryonSequentialTwoPoint(*bufs, t, s, 5, 5, 8)
            assert rel_err(bufs[s].to(torch.complex128).cpu().numpy(), ref) < 1e-6, (t, s)


def test_precision_conversion_roundtrip(api, props):
    import torch
    pi = cuda(props[0])
    lo = api.to_c64(pi)
    assert torch.equal(lo, pi.to(torch.complex64))
    assert torch.equal(api.to_c128(lo), lo.to(torch.complex128))


def test_timeslice_deterministic(api, props):
    pi, pj, pn = props
    pp = api.projector_plus_minus()
    a = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT)
    b = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT)
    assert np.array_equal(a.cpu().numpy(), b.cpu().numpy())


def test_device_status_clean(api):
    api.check_device()


def test_autotuned_variants_agree(api, props, c_oracle):
    """Every tile-shape variant the autotuner can pick computes the same result."""
    import ctypes
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi, pj, pn = props
    pp = api.projector_plus_minus()
    ref = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT).cpu().numpy()
    lib.contract_set_autotune(1)
    try:
        got = api.baryon_all_types(cuda(pi, True), cuda(pj, True), cuda(pn, True), 5, 5, pp, latt=LATT).cpu().numpy()
        t = api.baryon(cuda(pi, True), cuda(pj, True), cuda(pn, True), 1, 5, 5, gamma_mn=8, latt=LATT).cpu().numpy()
    finally:
        lib.contract_set_autotune(0)
    assert rel_err(got, ref) < 1e-6
    site = c_oracle.baryon_two_point(pi, pj, pn, 1, 5, 5, 8)
    assert per_t_rel(t, eo.timeslice_sum(site, LATT), site) < TOL_C64_TIMESLICE
    buf = ctypes.create_string_buffer(4096)
    assert lib.contract_autotune_report(buf, len(buf)) >= 2


@pytest.mark.parametrize("latt", [(4, 4, 4, 4), (6, 2, 4, 3), (2, 3, 3, 2)])
def test_meson_all_gamma_momentum(api, latt, c_oracle):
    """All 16 x 16 meson pairs projected to momenta, both precisions, against
    the FP64 oracle (per-site all-gamma values, then the explicit phase sum)."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi = eo.make_propagator(latt, 31, 0.2)
    pj = eo.make_propagator(latt, 32, 0.2)
    moms = eo.momentum_list(1)
    if latt[0] == 6:
        moms = np.concatenate([moms, [[2, -1, 1], [3, 0, 0]]])
    site = eo.meson_all_gamma(pi, pj).reshape(256, -1)            # [256, V]
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)  # [P, Lt, 256]
    v = pi.shape[0]
    lat = (ctypes.c_int * 4)(*latt)
    m = np.ascontiguousarray(moms.astype(np.int32))
    # sigma per (p, t, gamma pair): root-sum-square of the site terms
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]  # [1, Lt, 256]
    for prec in (0, 1, 2):
        out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        a, b = cuda(pi, prec >= 1), cuda(pj, prec >= 1)
        lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), v, lat,
                                              m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), prec)
        got = out.cpu().numpy()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        if prec == 0:
            assert rel_err(got, ref) < TOL_C128
        else:
            err = np.abs(got - ref) / np.maximum(np.abs(ref), sig)
            assert err.max() < (TOL_C64_TIMESLICE if prec == 1 else TOL_C64_TC)
    api.check_device()


@pytest.mark.parametrize("latt", [(6, 6, 2, 3), (10, 4, 2, 2), (4, 4, 16, 16)])
def test_meson_momentum_fused_tiles(api, latt):
    """The fused complex64 projection (site values and X/Y transforms in one
    kernel): rows that cross 16-site tiles, a partial last tile per plane, and
    more (t, z) planes than SMs, so that CTAs walk several planes."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi = eo.make_propagator(latt, 61, 0.2)
    pj = eo.make_propagator(latt, 62, 0.25)
    moms = eo.momentum_list(1)
    site = eo.meson_all_gamma(pi, pj).reshape(256, -1)
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
    m = np.ascontiguousarray(moms.astype(np.int32))
    a, b = cuda(pi, True), cuda(pj, True)
    out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
    lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), pi.shape[0],
                                          (ctypes.c_int * 4)(*latt),
                                          m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), 1)
    got = out.cpu().numpy()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    assert (np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max() < TOL_C64_TIMESLICE
    api.check_device()


@pytest.mark.parametrize("latt", [(6, 6, 2, 3), (10, 4, 2, 2), (4, 4, 16, 16)])
def test_meson_momentum_same_field(api, latt):
    """One field for both propagators (a pion): the fused complex64 kernel forms
    136 of the 256 spin-colour products and the rest by Hermitian symmetry; it
    matches the oracle and the general form run on a copy of the field.  The
    error is measured against max(|C|, sigma, L1), L1 the largest per-timeslice
    sum of |T(x)| over the spin-colour products: the diagonal products of one
    field are positive at every site, an FP32 projection to nonzero momentum
    cancels terms of that size (up to 15x the pairs' sigma on these lattices),
    and its rounding reaches every pair, in the general form as much as in
    this one.  Tolerance TOL_C64_COHERENT of that scale."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi = eo.make_propagator(latt, 71, 0.2)
    moms = eo.momentum_list(1)
    site = eo.meson_all_gamma(pi, pi).reshape(256, -1)
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
    scale = np.maximum(np.maximum(np.abs(ref), sig), eo.meson_product_l1(pi, pi, latt))
    m = np.ascontiguousarray(moms.astype(np.int32))
    a = cuda(pi, True)
    got = {}
    for name, b in (("same", a), ("copy", a.clone())):
        out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), pi.shape[0],
                                              (ctypes.c_int * 4)(*latt),
                                              m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), 1)
        got[name] = out.cpu().numpy()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        err = (np.abs(got[name] - ref) / scale).max()
        assert err < TOL_C64_COHERENT, (name, err)
    assert np.abs(got["same"] - got["copy"]).max() <= 1e-6 * np.abs(got["copy"]).max()
    api.check_device()


def test_meson_momentum_many_z_groups(api):
    """Ten +nz/-nz groups for one (nx, ny) pair: the finalize runs two passes over
    its groups, each staging the projected products for the Gamma-pair combination."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    latt = (4, 4, 20, 2)
    moms = np.array([[0, 0, n] for n in range(-9, 11)], dtype=np.int32)  # nz = 10 is its own negative
    pi = eo.make_propagator(latt, 71, 0.2)
    pj = eo.make_propagator(latt, 72, 0.3)
    site = eo.meson_all_gamma(pi, pj).reshape(256, -1)
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
    for prec, tol in ((0, TOL_C128), (1, TOL_C64_TIMESLICE)):
        a, b = cuda(pi, prec >= 1), cuda(pj, prec >= 1)
        out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), pi.shape[0],
                                              (ctypes.c_int * 4)(*latt),
                                              moms.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), prec)
        got = out.cpu().numpy()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        if prec == 0:
            assert rel_err(got, ref) < tol
        else:
            assert (np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max() < tol
    api.check_device()


def test_fused_variants_forced(tmp_path):
    """Every compiled tile-shape variant of the fused all-types pass (complex64:
    shared-wedge, merged and two-loop forms, two and one projector, two fields
    and one field for P_i and P_j; complex128: the shared-wedge shapes), forced
    through a tune cache, against the FP64 oracle.  Each case uses its own lattice shape, so that each tune
    key fixes one variant."""
    import ctypes
    import json
    import os
    import subprocess
    import sys
    from contract_gb300 import _lib, build
    build.build()
    lib = _lib.lib()
    cache = tmp_path / "tune.txt"
    lines, cases, names = [], [], []
    for prec, nproj, same in ((1, 2, False), (1, 1, False), (1, 2, True), (1, 1, True), (0, 2, False),
                              (0, 1, False)):
        aux = nproj + (4 if same else 0)
        buf = ctypes.create_string_buffer(4096)
        n = lib.contract_variant_names(3, prec, aux, buf, len(buf))  # op 3: the fused all-types pass
        vnames = buf.value.decode().split()
        assert n == len(vnames) >= (7 if prec == 1 else 3), (n, vnames)
        for v, name in enumerate(vnames):
            latt = (4, 2, 2 + 2 * same, 2 + v) if nproj == 2 else (2, 4, 2 + 2 * same, 2 + v)
            vol = int(np.prod(latt))
            key = f"kind=3,prec={prec},aux={aux},volume={vol},lt={latt[3]},half={vol // latt[3] // 2}"
            lines.append(f"{key}\t{v} {name} 1.0\n")
            cases.append([list(latt), nproj, same, prec])
            names.append(name)
    cache.write_text("".join(lines))
    env = dict(os.environ, CONTRACT_TUNE_CACHE=str(cache), CONTRACT_AUTOTUNE="0")
    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fused_variants_child.py")
    res = subprocess.run([sys.executable, child, json.dumps(cases)], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    for name in set(names):
        assert name in out["report"], (name, out["report"])
    for name, case, err in zip(names, cases, out["errors"]):
        assert err < (TOL_C64_TIMESLICE if case[3] == 1 else TOL_C128), (name, case, err)


def test_baryon_variants_forced(tmp_path):
    """Every compiled tile-shape variant of the per-call baryon two-point, in
    complex64 and complex128 -- loop form; triangle form with a gamma
    projector; triangle form with N' materialised, for a dense projector;
    triangle form with a projector of rank <= 2, for (1 + g4)/2 and for a
    polarised projector -- forced through a tune cache, against the FP64 oracle.
    Each case uses its own lattice shape, so that each tune key fixes one
    variant."""
    import ctypes
    import json
    import os
    import subprocess
    import sys
    from contract_gb300 import _lib, build
    build.build()
    lib = _lib.lib()
    cache = tmp_path / "tune.txt"
    lines, cases, names = [], [], []
    for prec in (1, 0):
        for c, (op, aux, ctype, kind) in enumerate(((1, 0, 0, "g4"), (2, 0, 1, "g4"), (2, 1, 4, "dense"),
                                                    (2, 1, 3, "dense"), (2, 2, 4, "pp"), (2, 2, 5, "pol"))):
            buf = ctypes.create_string_buffer(4096)
            n = lib.contract_variant_names(op, prec, aux, buf, len(buf))
            vnames = buf.value.decode().split()
            assert n == len(vnames) >= 4, (op, prec, aux, vnames)
            for v, name in enumerate(vnames):
                latt = (4, 2 + 2 * c, 2, 3 + v)  # one lattice shape per (case, variant); the key holds prec
                vol = int(np.prod(latt))
                key = f"kind={op},prec={prec},aux={aux},volume={vol},lt={latt[3]},half={vol // latt[3] // 2}"
                lines.append(f"{key}\t{v} {name} 1.0\n")
                cases.append([list(latt), ctype, kind, prec])
                names.append((op, aux, name))
    cache.write_text("".join(lines))
    env = dict(os.environ, CONTRACT_TUNE_CACHE=str(cache), CONTRACT_AUTOTUNE="0")
    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "baryon_variants_child.py")
    res = subprocess.run([sys.executable, child, json.dumps(cases)], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    for (_, _, name) in set(names):
        assert name in out["report"], (name, out["report"])
    for name, case, err in zip(names, cases, out["errors"]):
        assert err < (TOL_C64_TIMESLICE if case[3] == 1 else TOL_C128), (name, case, err)


def test_site_variants_forced(tmp_path):
    """Every compiled tile-shape variant of the meson (one Gamma pair,
    all-source, all-sink), diquark and sequential-source kernels, in complex64
    and complex128, forced through a tune cache, against the FP64 oracle.
    Each case uses its own lattice shape, so that each tune key fixes one
    variant."""
    import ctypes
    import json
    import os
    import subprocess
    import sys
    from contract_gb300 import _lib, build
    build.build()
    lib = _lib.lib()
    cache = tmp_path / "tune.txt"
    lines, cases, names = [], [], []
    # (op, tune kind, aux, contract type, sequential slot); sequential aux = 3 (loop types) + slot
    ops = (("meson", 0, 0, 0, 0), ("meson_all_source", 6, 1, 0, 0), ("meson_all_sink", 6, 0, 0, 0),
           ("diquark", 4, 0, 0, 0), ("sequential", 5, 5, 0, 2), ("sequential", 5, 0, 1, 0))
    for prec in (1, 0):
        for c, (op, kind, aux, ctype, slot) in enumerate(ops):
            buf = ctypes.create_string_buffer(4096)
            n = lib.contract_variant_names(kind, prec, aux, buf, len(buf))
            vnames = buf.value.decode().split()
            assert n == len(vnames) >= 3, (op, prec, vnames)
            per_site = op in ("diquark", "sequential")
            for v, name in enumerate(vnames):
                latt = (4, 2, 2 + 2 * c, 3 + v)  # one lattice shape per (case, variant); the key holds prec
                vol = int(np.prod(latt))
                lt, half = (0, 0) if per_site else (latt[3], vol // latt[3] // 2)
                lines.append(f"kind={kind},prec={prec},aux={aux},volume={vol},lt={lt},half={half}\t{v} {name} 1.0\n")
                cases.append([op, list(latt), prec, ctype, slot])
                names.append(name)
    cache.write_text("".join(lines))
    env = dict(os.environ, CONTRACT_TUNE_CACHE=str(cache), CONTRACT_AUTOTUNE="0")
    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "site_variants_child.py")
    res = subprocess.run([sys.executable, child, json.dumps(cases)], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    for name in set(names):
        assert name in out["report"], (name, out["report"])
    # complex64: the inputs rounded to complex64 against FP64 ones, relative to the largest value
    for name, case, err in zip(names, cases, out["errors"]):
        assert err < (2e-6 if case[2] == 1 else TOL_C128), (name, case, err)


def test_momentum_variants_forced(tmp_path):
    """Each tile-shape variant of the momentum projection, forced through a tune
    cache: tensor-core work units of 192 k-steps (six units per timeslice on
    24x24x16) and 64 (eighteen units), the three-kernel complex64 form, and the
    fused kernel with 16 site warps (on rows of 32 sites: the aligned path), for
    two fields and for one field passed twice."""
    import json
    import os
    import subprocess
    import sys
    cache = tmp_path / "tune.txt"
    lines = []
    for latt, aux, variant, name in [((24, 24, 16, 2), 2, 2, "tc.unit192"), ((24, 24, 16, 1), 2, 1, "tc.unit64"),
                                     ((8, 8, 8, 2), 1, 1, "three-kernel"), ((32, 4, 16, 2), 1, 2, "fused.site16.xy8"),
                                     ((32, 4, 16, 3), 5, 2, "fused.site16.xy8")]:
        v = int(np.prod(latt))
        key = f"kind=7,prec=1,aux={aux},volume={v},lt={latt[3]},half={v // latt[3] // 2}"
        lines.append(f"{key}\t{variant} {name} 1.0\n")
    cache.write_text("".join(lines))
    env = dict(os.environ, CONTRACT_TUNE_CACHE=str(cache), CONTRACT_AUTOTUNE="0")
    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "momentum_variants_child.py")
    res = subprocess.run([sys.executable, child], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    out = json.loads(res.stdout.strip().splitlines()[-1])
    for name in ("tc.unit192", "tc.unit64", "three-kernel", "fused.site16.xy8"):
        assert name in out["report"], out["report"]
    assert "aux=5" in out["report"], out["report"]
    tc192, tc64, three, site16, site16_same = out["errors"]
    assert tc192 < TOL_C64_TC and tc64 < TOL_C64_TC, (tc192, tc64)
    assert three < TOL_C64_TIMESLICE and site16 < TOL_C64_TIMESLICE
    assert site16_same < TOL_C64_COHERENT, site16_same


def test_momentum_tensor_cores_two_momentum_groups(api):
    """CONTRACT_C64_TC with 147 momenta (two groups of 128 GEMM rows) on a
    lattice whose timeslice (6 x 6 x 4 = 144 sites) spans 18 k-steps."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    latt = (6, 6, 4, 2)
    pi = eo.make_propagator(latt, 41, 0.2)
    pj = eo.make_propagator(latt, 42, 0.3)
    r3, r1 = np.arange(-3, 4), np.arange(-1, 2)
    moms = np.stack(np.meshgrid(r3, r3, r1, indexing="ij"), -1).reshape(-1, 3)
    assert len(moms) == 147
    site = eo.meson_all_gamma(pi, pj).reshape(256, -1)
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
    out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
    m = np.ascontiguousarray(moms.astype(np.int32))
    a, b = cuda(pi, True), cuda(pj, True)  # keep both alive across the call
    lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(),
                                          pi.shape[0], (ctypes.c_int * 4)(*latt),
                                          m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), 2)
    got = out.cpu().numpy()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    err = np.abs(got - ref) / np.maximum(np.abs(ref), sig)
    assert err.max() < TOL_C64_TC
    api.check_device()


BATCH_LATTS = [(4, 4, 4, 8), (4, 2, 2, 6), (6, 4, 2, 4), (2, 2, 2, 2)]


def _batch_items(props_by_item, outs, lib_mod):
    from contract_gb300 import _lib  # noqa: F401
    import ctypes

    class Item(ctypes.Structure):
        _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("propag_n", ctypes.c_void_p),
                    ("correl", ctypes.c_void_p), ("lattice", ctypes.c_int * 4)]

    arr = (Item * len(outs))()
    for k, ((a, b, c, latt), out) in enumerate(zip(props_by_item, outs)):
        arr[k].propag_i, arr[k].propag_j, arr[k].propag_n = a.data_ptr(), b.data_ptr(), c.data_ptr()
        arr[k].correl = out.data_ptr()
        arr[k].lattice = (ctypes.c_int * 4)(*latt)
    return arr


@pytest.mark.parametrize("c64", [False, True])
def test_batched_work_queue_and_cuda_graph(api, c64):
    """One persistent launch over items on lattices of different extents
    matches per-item calls, directly and replayed from a CUDA graph."""
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pp = np.ascontiguousarray(api.projector_plus_minus())
    items, outs, refs = [], [], []
    for k, latt in enumerate(BATCH_LATTS):
        ps = [cuda(eo.make_propagator(latt, 100 + 3 * k + s, 0.1 + 0.1 * s), c64) for s in range(3)]
        items.append((*ps, latt))
        refs.append(api.baryon_all_types(*ps, 5, 5, pp, latt=latt).cpu().numpy())
        outs.append(torch.full((6, 2, latt[3]), float("nan"), dtype=torch.complex128, device="cuda"))
    arr = _batch_items(items, outs, lib)
    prec = 1 if c64 else 0
    lib.contract_baryon_all_types_batch(arr, len(outs), 5, 5, 2, pp.ctypes.data, prec)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    # complex64: the per-item calls may run another tile shape (autotuned), so
    # the FP32 partial sums group differently
    tol = 1e-6 if c64 else 1e-12
    for out, ref in zip(outs, refs):
        assert rel_err(out.cpu().numpy(), ref) < tol
    # capture the same launch in a CUDA graph and replay it
    for out in outs:
        out.fill_(float("nan"))
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        lib.contract_set_stream(s.cuda_stream)
        lib.contract_baryon_all_types_batch(arr, len(outs), 5, 5, 2, pp.ctypes.data, prec)  # warm-up
    torch.cuda.current_stream().wait_stream(s)
    for out in outs:
        out.fill_(float("nan"))
    with torch.cuda.graph(g):
        lib.contract_set_stream(torch.cuda.current_stream().cuda_stream)
        lib.contract_baryon_all_types_batch(arr, len(outs), 5, 5, 2, pp.ctypes.data, prec)
    lib.contract_set_stream(None)
    g.replay()
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    for out, ref in zip(outs, refs):
        assert rel_err(out.cpu().numpy(), ref) < tol
    api.check_device()


@pytest.mark.parametrize("c64", [False, True])
def test_batched_one_low_rank_projector(api, c_oracle, c64):
    """The batched launch with one projector of rank 2 ((1 + g4)/2 alone: the
    factored triangle form) over items of different extents, with two fields
    and with one field for P_i and P_j, against per-item calls and, for the
    first item, the FP64 oracle."""
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    w = np.ascontiguousarray(api.projector_plus_minus()[:1])
    tol = 1e-6 if c64 else 1e-12
    for one_field in (False, True):
        items, outs, refs, host = [], [], [], []
        for k, latt in enumerate(BATCH_LATTS):
            hp = [eo.make_propagator(latt, 200 + 3 * k + s, 0.1 + 0.1 * s) for s in range(3)]
            if one_field:
                hp[1] = hp[0]
            ps = [cuda(a, c64) for a in hp]
            if one_field:
                ps[1] = ps[0]
            items.append((*ps, latt))
            host.append(hp)
            refs.append(api.baryon_all_types(*ps, 5, 5, w, latt=latt).cpu().numpy())
            outs.append(torch.full((6, 1, latt[3]), float("nan"), dtype=torch.complex128, device="cuda"))
        arr = _batch_items(items, outs, lib)
        lib.contract_baryon_all_types_batch(arr, len(outs), 5, 5, 1, w.ctypes.data, 1 if c64 else 0)
        torch.cuda.synchronize()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        for out, ref in zip(outs, refs):
            assert rel_err(out.cpu().numpy(), ref) < tol, one_field
        latt = BATCH_LATTS[0]
        site = np.array([c_oracle.baryon_general_two_point(*host[0], t, 5, 5, w[0]) for t in range(6)])
        assert rel_err(outs[0].cpu().numpy()[:, 0], eo.timeslice_sum(site, latt)) < (1e-5 if c64 else 1e-12)
    api.check_device()


@pytest.mark.parametrize("c64", [False, True])
def test_sequential_sink_timeslice(api, props, c_oracle, c64):
    """Sequential source at t_sink: dC/dP on that timeslice, zero elsewhere."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pi, pj, pn = props
    v = pi.shape[0]
    _, _, _, tt = eo.eo_coords(LATT)
    lat = (ctypes.c_int * 4)(*LATT)
    for ct, slot, t_sink in ((1, 2, 3), (0, 0, 7), (4, 1, 0)):
        ref = c_oracle.baryon_sequential(pi, pj, pn, ct, slot, 5, 5, 8)
        ref[tt != t_sink] = 0
        bufs = [cuda(p, c64) for p in (pi, pj, pn)]
        lib.contract_sequential_sink(*[b.data_ptr() for b in bufs], ct, slot, v, lat, t_sink, 5, 5, 8, 1 if c64 else 0)
        got = bufs[slot].to(torch.complex128).cpu().numpy()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        assert np.count_nonzero(got[tt != t_sink]) == 0
        assert rel_err(got, ref) < (1e-6 if c64 else TOL_C128), (ct, slot, t_sink)


@pytest.mark.parametrize("c64", [False, True])
@pytest.mark.parametrize("latt", [(4, 4, 4, 8), (6, 2, 2, 5)])
def test_all_types_from_host_buffers(api, c64, latt):
    """contract_baryon_all_types_host (timeslice chunks copied from pinned host
    memory on two streams, contracted as they arrive) against the device call;
    Lt = 5 leaves a short last chunk."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    pp = np.ascontiguousarray(api.projector_plus_minus())
    ps = [eo.make_propagator(latt, 60 + s, 0.2 + 0.05 * s) for s in range(3)]
    v = ps[0].shape[0]
    lat = (ctypes.c_int * 4)(*latt)
    prec = 1 if c64 else 0
    dev = [cuda(x, c64) for x in ps]
    ref = torch.empty((6, 2, latt[3]), dtype=torch.complex128, device="cuda")
    lib.contract_baryon_all_types(ref.data_ptr(), *(x.data_ptr() for x in dev), v, 5, 5, 2, pp.ctypes.data, prec, lat)
    host = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in ps]
    out = torch.full((6, 2, latt[3]), float("nan"), dtype=torch.complex128).pin_memory()
    for _ in range(2):  # the second call reuses the staging buffers and streams
        lib.contract_baryon_all_types_host(out.data_ptr(), *(h.data_ptr() for h in host), v, 5, 5, 2,
                                           pp.ctypes.data, prec, lat)
    lib.contract_check_device()
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    assert rel_err(out.numpy(), ref.cpu().numpy()) < (1e-6 if c64 else 1e-12)


def test_pycontract_matrix_operands_as_in_reference_example(api, props):
    """pycontract.baryonTwoPoint called as the reference's example does
    (baryon_2pt.py:72-92): C g4 g5 and C g5 as 4x4 matrices (decomposed into a
    basis index and a phase) and the projector (1 - g4)/2 (sent through the
    general-projector path), against an einsum over the same matrices."""
    from contract_gb300 import pycontract as pc
    G = pc.gamma_matrices()
    C = G[2] @ G[8]
    cg_a, cg_b, proj = C @ G[8] @ G[15], C @ G[15], (G[0] - G[8]) / 2
    pi, pj, pn = props
    for t in (pc.BaryonContractType.IN_JK_ML, pc.BaryonContractType.IK_JL_MN):
        got = pc.baryonTwoPoint(cuda(pi), cuda(pj), cuda(pn), t, cg_a, cg_b, proj).cpu().numpy()
        si, sj, sn = eo._baryon_subscripts(int(t))
        ref = np.einsum(f"abc,def,ij,kl,nm,x{si},x{sj},x{sn}->x", eo.EPS, eo.EPS, cg_a, cg_b, proj,
                        eo._as_sites(pi), eo._as_sites(pj), eo._as_sites(pn), optimize=True)
        assert rel_err(got, ref) < TOL_C128


def test_momentum_grouping_edge_cases(api):
    """Momentum lists that stress the +n / -n pairing of the Z transform:
    duplicates, nz = +-Lz/2 (its own negative mod Lz), a lone -nz, and nx
    beyond Lx/2; all three forms against the explicit phase sum."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    latt = (4, 4, 4, 2)
    moms = np.array([[0, 0, 2], [0, 0, -2], [0, 0, 2], [1, 0, 0], [-1, 0, 0], [0, 0, 0], [0, 0, 0],
                     [0, 1, -1], [3, 2, 1], [-3, 2, 5]], dtype=np.int32)
    pi = eo.make_propagator(latt, 51, 0.2)
    pj = eo.make_propagator(latt, 52, 0.3)
    site = eo.meson_all_gamma(pi, pj).reshape(256, -1)
    ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
    sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
    m = np.ascontiguousarray(moms)
    for prec, tol in ((0, TOL_C128), (1, TOL_C64_TIMESLICE), (2, TOL_C64_TC)):
        a, b = cuda(pi, prec >= 1), cuda(pj, prec >= 1)
        out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), pi.shape[0],
                                              (ctypes.c_int * 4)(*latt),
                                              m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), prec)
        got = out.cpu().numpy()
        assert lib.contract_last_error() == 0, lib.contract_last_error_message()
        if prec == 0:
            assert rel_err(got, ref) < tol
        else:
            assert (np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max() < tol
    api.check_device()


@pytest.mark.parametrize("c64", [False, True])
def test_layout_conversion_lexicographic_even_odd(api, c64):
    """contract_convert_layout: lexicographic -> even/odd matches the
    oracle's site coordinates exactly, and the round trip is the identity."""
    import ctypes
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    latt = (6, 2, 4, 3)
    lx, ly, lz, lt = latt
    v = lx * ly * lz * lt
    rng = np.random.default_rng(7)
    lex = (rng.standard_normal((v, 144)) + 1j * rng.standard_normal((v, 144))).astype(np.complex128)
    x, y, z, t = eo.eo_coords(latt)
    want = lex[((t * lz + z) * ly + y) * lx + x]  # site e of the even/odd order
    prec = 1 if c64 else 0
    src = cuda(lex, c64)
    dst = torch.full_like(src, float("nan"))
    back = torch.full_like(src, float("nan"))
    lat = (ctypes.c_int * 4)(*latt)
    lib.contract_convert_layout(dst.data_ptr(), src.data_ptr(), lat, 1, prec)
    lib.contract_convert_layout(back.data_ptr(), dst.data_ptr(), lat, 0, prec)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0, lib.contract_last_error_message()
    ref = want.astype(np.complex64) if c64 else want
    assert np.array_equal(dst.cpu().numpy(), ref)
    assert torch.equal(back, src)

