"""Child process of test_parity_gpu.test_baryon_variants_forced: runs the
per-call baryon two-point (loop and triangle forms, complex64 or complex128) on small
lattices whose tune-cache entries (written by the parent into
CONTRACT_TUNE_CACHE) force one tile-shape variant each, and prints, as one
JSON line, each run's per-timeslice error against the FP64 oracle (complex64:
relative to max(|C_t|, sigma_t); complex128: to the largest |C_t|), with the
tuner's report."""
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

    from contract_gb300 import _lib, api
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    from contract_gb300.pycontract import gamma_matrices
    # [[latt, contract_type, projector: "g4", "pp", "pol" or "dense", precision: 1 complex64, 0 complex128], ...]
    cases = json.loads(sys.argv[1])
    oracle = L.c_oracle()
    rng = np.random.default_rng(17)
    g, e = gamma_matrices(), np.eye(4)
    projs = {"pp": np.ascontiguousarray(api.projector_plus_minus()[0]),  # (1 + g4)/2: rank 2
             "pol": np.ascontiguousarray(((e + g[8]) @ (e - 1j * g[3]) / 4).reshape(16)),  # rank 1
             "dense": np.ascontiguousarray((rng.standard_normal(16) + 1j * rng.standard_normal(16)) / 4)}
    errs = []
    for k, (latt, ctype, kind, prec) in enumerate(cases):
        use_proj = kind != "g4"
        proj = projs.get(kind)
        latt = tuple(latt)
        props = [eo.make_propagator(latt, 300 + 3 * k + s, 0.2 + 0.05 * s) for s in range(3)]
        dtype = torch.complex64 if prec == 1 else torch.complex128
        dev = [torch.from_numpy(p).cuda().to(dtype) for p in props]
        out = torch.full((latt[3],), float("nan"), dtype=torch.complex128, device="cuda")
        lib.contract_baryon(out.data_ptr(), *(d.data_ptr() for d in dev), ctype, props[0].shape[0], 5, 5, 8,
                            proj.ctypes.data if use_proj else None, prec, (ctypes.c_int * 4)(*latt))
        got = out.cpu().numpy()
        if lib.contract_last_error():
            raise RuntimeError(lib.contract_last_error_message().decode())
        site = (oracle.baryon_general_two_point(*props, ctype, 5, 5, proj) if use_proj
                else oracle.baryon_two_point(*props, ctype, 5, 5, 8))
        ref = eo.timeslice_sum(site, latt)
        sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real)
        if prec == 1:  # relative to max(|C_t|, sigma_t)
            errs.append(float((np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max()))
        else:  # complex128: relative to the largest |C_t|
            errs.append(float(np.abs(got - ref).max() / np.abs(ref).max()))
    buf = ctypes.create_string_buffer(16384)
    lib.contract_autotune_report(buf, len(buf))
    print(json.dumps({"errors": errs, "report": buf.value.decode()}))


if __name__ == "__main__":
    main()
