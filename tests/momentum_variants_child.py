"""Child process of test_parity_gpu.test_momentum_variants_forced: runs the
all-gamma momentum projection with tile-shape variants forced through a tune
cache (CONTRACT_TUNE_CACHE, written by the parent) and prints, as one JSON line,
the error of each run against the FP64 oracle relative to max(|C|, sigma)."""
import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import einsum_oracle as eo  # noqa: E402

# (lattice, precision mode, one field for both propagators); the parent's
# cache fixes each one's variant
CASES = [((24, 24, 16, 2), 2, False), ((24, 24, 16, 1), 2, False), ((8, 8, 8, 2), 1, False),
         ((32, 4, 16, 2), 1, False), ((32, 4, 16, 3), 1, True)]


def main():
    import torch
    from contract_gb300 import _lib
    lib = _lib.lib()
    lib.contract_set_error_mode(1)
    moms = np.ascontiguousarray(eo.momentum_list(1).astype(np.int32))
    errs = []
    for k, (latt, prec, same) in enumerate(CASES):
        pi = eo.make_propagator(latt, 81 + k, 0.2)
        pj = pi if same else eo.make_propagator(latt, 91 + k, 0.3)
        site = eo.meson_all_gamma(pi, pj).reshape(256, -1)
        ref = eo.momentum_project(site, latt, moms).transpose(1, 2, 0)
        sig = np.sqrt(eo.timeslice_sum(np.abs(site) ** 2, latt).real).T[None]
        # one field: the coherent products set the error scale (meson_product_l1)
        sig = np.maximum(sig, eo.meson_product_l1(pi, pj, latt)) if same else sig
        a = torch.from_numpy(pi).cuda().to(torch.complex64)
        b = a if same else torch.from_numpy(pj).cuda().to(torch.complex64)
        out = torch.full((len(moms), latt[3], 256), float("nan"), dtype=torch.complex128, device="cuda")
        lib.contract_meson_all_gamma_momentum(out.data_ptr(), a.data_ptr(), b.data_ptr(), pi.shape[0],
                                              (ctypes.c_int * 4)(*latt),
                                              moms.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(moms), prec)
        got = out.cpu().numpy()
        if lib.contract_last_error():
            raise RuntimeError(lib.contract_last_error_message().decode())
        errs.append(float((np.abs(got - ref) / np.maximum(np.abs(ref), sig)).max()))
    buf = ctypes.create_string_buffer(8192)
    lib.contract_autotune_report(buf, len(buf))
    print(json.dumps({"errors": errs, "report": buf.value.decode()}))


if __name__ == "__main__":
    main()
