"""The allocation-free entry point (contract_baryon_all_types_noalloc).

It exists for callers that cannot let the library call cudaMalloc -- a host
framework whose pool allocator owns the free device memory, a latency-critical
loop that cannot take cudaMalloc's implicit synchronisation, or a host that
requires an allocation-free contraction library.  Its per-timeslice partial
sums live in a fixed static device array, so its output must match the
allocating entry point (contract_baryon_all_types) on every call.

This file is collected last on purpose: a failure here leaves every other
test already run.  It also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LATT = (12, 12, 12, 16)
TOL_C128 = 1e-12  # same kernels, same reduction order: agreement is expected to be exact
TOL_C64 = 1e-6    # relative to the largest |value|, as for the other mixed-form tests


@pytest.fixture(scope="module")
def env():
    import torch

    from contract_gb300 import _lib, api, build
    from contract_gb300.lattice import synthetic_propagator
    build.build()
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    lib.contract_clear_error()
    torch.cuda.set_device(0)
    lib.init(0)
    props = [synthetic_propagator(LATT, s, m, device="cuda:0") for s, m in ((41, 0.25), (42, 0.25), (43, 0.3))]
    return lib, api, props


def _call_noalloc(lib, out, props, projs, prec, latt):
    lat = (ctypes.c_int * 4)(*latt)
    v = props[0].numel() // 144
    return lib.contract_baryon_all_types_noalloc(out.data_ptr(), props[0].data_ptr(), props[1].data_ptr(),
                                                 props[2].data_ptr(), v, 5, 5, projs.shape[0], projs.ctypes.data,
                                                 prec, lat)


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_allocating_entry_point_twice(env, prec):
    import torch
    lib, api, props = env
    if prec == 1:
        props = [api.to_c64(p) for p in props]
    projs = np.ascontiguousarray(api.projector_plus_minus())
    ref = api.baryon_all_types(*props, 5, 5, projs, latt=LATT)
    torch.cuda.synchronize()
    ref_np = ref.cpu().numpy()
    tol = TOL_C128 if prec == 0 else TOL_C64
    for call in range(2):  # the static scratch keeps the previous call's contents
        out = torch.full_like(ref, float("nan"))
        rc = _call_noalloc(lib, out, props, projs, prec, LATT)
        assert rc == 0, lib.contract_last_error_message()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got)), call
        assert np.abs(got - ref_np).max() / np.abs(ref_np).max() <= tol, call
    assert lib.contract_check_device() == 0


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_one_field_and_one_projector(env, prec):
    """The forms the allocating entry point picks by its arguments, run against
    the static scratch: one field passed as both P_i and P_j (the one-pass
    form), and a single projector."""
    import torch
    lib, api, props = env
    if prec == 1:
        props = [api.to_c64(p) for p in props]
    projs = np.ascontiguousarray(api.projector_plus_minus())
    tol = TOL_C128 if prec == 0 else TOL_C64
    cases = [([props[0], props[0], props[2]], projs), (props, np.ascontiguousarray(projs[:1])),
             ([props[0], props[0], props[2]], np.ascontiguousarray(projs[1:]))]
    for k, (trip, pj) in enumerate(cases):
        ref = api.baryon_all_types(*trip, 5, 5, pj, latt=LATT)
        torch.cuda.synchronize()
        ref_np = ref.cpu().numpy()
        for call in range(2):
            out = torch.full_like(ref, float("nan"))
            rc = _call_noalloc(lib, out, trip, pj, prec, LATT)
            assert rc == 0, lib.contract_last_error_message()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got)), (k, call)
            assert np.abs(got - ref_np).max() / np.abs(ref_np).max() <= tol, (k, call)
    assert lib.contract_check_device() == 0


def test_noalloc_rejects_lattices_beyond_the_static_scratch(env):
    """2 x 1 x 1 x 16384: one site per half-timeslice, so 32768 partial records
    of (at least 3) consumer warps x 12 outputs x 16 bytes -- more than the
    16 MiB array holds for every tile shape.  Real buffers of the right size are
    passed; the call must refuse before any launch."""
    import torch
    lib, api, _ = env
    latt = (2, 1, 1, 16384)
    v = 2 * 16384
    props = [torch.zeros((v, 4, 4, 3, 3), dtype=torch.complex64, device="cuda:0") for _ in range(3)]
    projs = np.ascontiguousarray(api.projector_plus_minus())
    out = torch.zeros((6, 2, latt[3]), dtype=torch.complex128, device="cuda:0")
    lib.contract_clear_error()
    rc = _call_noalloc(lib, out, props, projs, 1, latt)
    assert rc == 1
    assert b"static scratch" in lib.contract_last_error_message()
    lib.contract_clear_error()
    # the allocating entry point handles the same lattice
    api.baryon_all_types(*props, 5, 5, projs, latt=latt)
    torch.cuda.synchronize()
    assert lib.contract_last_error() == 0


def test_noalloc_needs_a_lattice(env):
    import torch
    lib, api, props = env
    projs = np.ascontiguousarray(api.projector_plus_minus())
    out = torch.zeros((6, 2, 16), dtype=torch.complex128, device="cuda:0")
    v = props[0].numel() // 144
    lib.contract_clear_error()
    rc = lib.contract_baryon_all_types_noalloc(out.data_ptr(), props[0].data_ptr(), props[1].data_ptr(),
                                               props[2].data_ptr(), v, 5, 5, 2, projs.ctypes.data, 0, None)
    assert rc == 1 and b"needs a lattice" in lib.contract_last_error_message()
    lib.contract_clear_error()
