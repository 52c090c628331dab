"""Child process of test_parity_gpu.test_fused_variants_forced: runs the fused
all-types pass (complex64 or complex128) on small lattices whose tune-cache
entries (written by the parent into CONTRACT_TUNE_CACHE) force one tile-shape
variant each, and prints, as one JSON line, each run's per-timeslice error
against the FP64 oracle (complex64: relative to max(|C_t|, sigma_t);
complex128: to the largest |C_t|)."""
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

    from contract_gb300 import _lib, api
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    # [[latt, nproj, one field for P_i and P_j, precision: 1 complex64, 0 complex128], ...]
    cases = json.loads(sys.argv[1])
    oracle = L.c_oracle()
    pp = api.projector_plus_minus()
    g4 = np.asarray(eo.GAMMA[8]).reshape(1, 16)
    errs = []
    for k, (latt, nproj, same, prec) in enumerate(cases):
        latt = tuple(latt)
        projs = pp if nproj == 2 else g4  # (1 +- g4)/2: two gamma-basis terms; g4: one
        props = [eo.make_propagator(latt, 500 + 3 * k + s, 0.25) for s in range(3)]
        if same:
            props[1] = props[0]
        site = np.array([[oracle.baryon_general_two_point(*props, t, 5, 5, projs[w]) for w in range(nproj)]
                         for t in range(6)])
        ref = eo.timeslice_sum(site, latt)
        sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real)
        dev = [torch.from_numpy(p).cuda().to(torch.complex64 if prec == 1 else torch.complex128) for p in props]
        if same:
            dev[1] = dev[0]
        got = api.baryon_all_types(*dev, 5, 5, projs, latt=latt).cpu().numpy()
        if lib.contract_last_error():
            raise RuntimeError(lib.contract_last_error_message().decode())
        if prec == 1:
            errs.append(float((np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max()))
        else:
            errs.append(float(np.abs(got - ref).max() / np.abs(ref).max()))
    buf = np.zeros(16384, np.uint8)
    lib.contract_autotune_report(buf.ctypes.data, len(buf))
    print(json.dumps({"errors": errs, "report": bytes(buf).split(b"\0")[0].decode()}))


if __name__ == "__main__":
    main()
