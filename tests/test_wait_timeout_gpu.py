"""The site kernels' bounded waits, made to run out on purpose.

Every mbarrier wait of the site engines gives up after a wall-time limit,
sets the timeout bit of the device status word, waits (bounded again) for
the copies it may still have in flight, and returns.  Here the producer is
told to withhold the copies of one tile (contract_test_withhold_chunk), so
nothing ever completes that tile's barrier: the consumers' wait must run out
within the short limit set for the test, contract_check_device() must report
CONTRACT_ERROR_DEVICE_TIMEOUT, and the next call on the same context must
give the normal result.  Nothing faults, traps or spins without a limit.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
CONTRACT_ERROR_DEVICE_TIMEOUT = 3
LATT = (8, 8, 8, 8)
LIMIT_NS = 50_000_000  # 50 ms per wait


@pytest.fixture(scope="module")
def env():
    import torch

    from contract_gb300 import _lib, api, build
    from contract_gb300.lattice import synthetic_propagator
    build.build()
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    lib.init(0)
    props = [api.to_c64(synthetic_propagator(LATT, s, 0.3, device="cuda:0")) for s in (71, 72, 73)]
    torch.cuda.synchronize()
    return lib, api, props


def _timed_out(lib, run):
    lib.contract_clear_error()
    lib.contract_set_wait_limit(LIMIT_NS)
    lib.contract_test_withhold_chunk(0)
    try:
        t0 = time.monotonic()
        run()
        rc = lib.contract_check_device()
        elapsed = time.monotonic() - t0
        msg = lib.contract_last_error_message()
    finally:
        lib.contract_test_withhold_chunk(-1)
        lib.contract_set_wait_limit(0)
        lib.contract_clear_error()
    return rc, msg, elapsed


def test_scalar_kernel_wait_runs_out_and_context_recovers(env):
    import torch
    lib, api, props = env
    pp = np.ascontiguousarray(api.projector_plus_minus())
    ref = api.baryon_all_types(*props, 5, 5, pp, latt=LATT).cpu().numpy()
    out = torch.zeros((6, 2, LATT[3]), dtype=torch.complex128, device="cuda:0")
    rc, msg, elapsed = _timed_out(lib, lambda: api.baryon_all_types(*props, 5, 5, pp, latt=LATT, out=out))
    assert rc == CONTRACT_ERROR_DEVICE_TIMEOUT, (rc, msg)
    assert b"timed out" in msg
    assert elapsed < 20.0
    again = api.baryon_all_types(*props, 5, 5, pp, latt=LATT).cpu().numpy()
    assert lib.contract_check_device() == 0
    assert np.array_equal(again, ref)  # fixed reduction order: the same bits as before


def test_field_kernel_wait_runs_out_and_context_recovers(env):
    import torch
    lib, api, props = env
    v = props[0].shape[0]
    ref = torch.empty_like(props[0])
    lib.contract_diquark(ref.data_ptr(), props[0].data_ptr(), props[1].data_ptr(), v, 5, 5, 1)
    assert lib.contract_check_device() == 0
    out = torch.zeros_like(props[0])
    rc, msg, elapsed = _timed_out(lib, lambda: lib.contract_diquark(out.data_ptr(), props[0].data_ptr(),
                                                                    props[1].data_ptr(), v, 5, 5, 1))
    assert rc == CONTRACT_ERROR_DEVICE_TIMEOUT, (rc, msg)
    assert elapsed < 20.0
    again = torch.empty_like(props[0])
    lib.contract_diquark(again.data_ptr(), props[0].data_ptr(), props[1].data_ptr(), v, 5, 5, 1)
    assert lib.contract_check_device() == 0
    assert torch.equal(again, ref)
