"""Child process of test_parity_gpu.test_site_variants_forced: runs the meson
(one Gamma pair, all-source, all-sink), diquark and sequential-source kernels
on small lattices whose tune-cache entries (written by the parent into
CONTRACT_TUNE_CACHE) force one tile-shape variant each, in complex64 or
complex128, and prints, as one JSON line, each run's error against the FP64
oracle relative to the largest reference value, with the tuner's report."""
import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import einsum_oracle as eo  # noqa: E402
from oracle import lib as L  # noqa: E402


def main():
    import torch

    from contract_gb300 import _lib
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    # [[op name, lattice, precision: 1 complex64, 0 complex128, contract type, sequential slot], ...]
    cases = json.loads(sys.argv[1])
    oracle = L.c_oracle()
    errs = []
    for k, (op, latt, prec, ctype, slot) in enumerate(cases):
        latt = tuple(latt)
        v = int(np.prod(latt))
        props = [eo.make_propagator(latt, 500 + 3 * k + s, 0.2 + 0.05 * s) for s in range(3)]
        dtype = torch.complex64 if prec == 1 else torch.complex128
        dev = [torch.from_numpy(p).cuda().to(dtype) for p in props]
        lat = (ctypes.c_int * 4)(*latt)
        if op == "meson":
            out = torch.full((latt[3],), float("nan"), dtype=torch.complex128, device="cuda")
            lib.contract_meson(out.data_ptr(), dev[0].data_ptr(), dev[1].data_ptr(), v, 15, 13, prec, lat)
            ref = eo.timeslice_sum(oracle.meson_two_point(props[0], props[1], 15, 13), latt)
        elif op in ("meson_all_source", "meson_all_sink"):
            out = torch.full((16, latt[3]), float("nan"), dtype=torch.complex128, device="cuda")
            ptrs = (ctypes.c_void_p * 16)(*[out[g].data_ptr() for g in range(16)])
            source = op == "meson_all_source"
            lib.contract_meson_all(ptrs, dev[0].data_ptr(), dev[1].data_ptr(), v, 5, int(source), prec, lat)
            site = (oracle.meson_all_source if source else oracle.meson_all_sink)(props[0], props[1], 5)
            ref = eo.timeslice_sum(site, latt)
        elif op == "diquark":
            out = torch.full_like(dev[0], float("nan"))
            lib.contract_diquark(out.data_ptr(), dev[0].data_ptr(), dev[1].data_ptr(), v, 5, 5, prec)
            ref = oracle.baryon_diquark(props[0], props[1], 5, 5)
        else:  # sequential: the selected slot is overwritten
            lib.contract_sequential(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), ctype, slot, v, 5, 5, 8,
                                    prec)
            out = dev[slot]
            ref = oracle.baryon_sequential(*props, ctype, slot, 5, 5, 8)
        torch.cuda.synchronize()
        if lib.contract_last_error():
            raise RuntimeError(lib.contract_last_error_message().decode())
        got = out.cpu().numpy().astype(np.complex128).reshape(np.shape(ref))
        errs.append(float(np.abs(got - ref).max() / np.abs(ref).max()))
    buf = ctypes.create_string_buffer(16384)
    lib.contract_autotune_report(buf, len(buf))
    print(json.dumps({"errors": errs, "report": buf.value.decode()}))


if __name__ == "__main__":
    main()
