"""Generate the golden fixtures in this directory from the reference itself.

The outputs come from ``oracle/_ref/libcontract_ref.so``: the reference's own
per-site device functions (CLQCD/contract ``include/*.cuh``) compiled as host
C++ by ``make -C oracle ref``.  Run from the repository root, where the
reference sources are available:

    make -C oracle all ref REF=<path to CLQCD/contract>
    python tests/golden/make_golden.py

Inputs are seeded synthetic propagators (``oracle.einsum_oracle.make_propagator``)
on a 2x2x2x4 lattice, stored alongside the outputs so the fixtures do not
depend on the generator staying unchanged.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import einsum_oracle as eo  # noqa: E402
from oracle import lib as L  # noqa: E402

LATT = (2, 2, 2, 4)  # Lx, Ly, Lz, Lt
V = 2 * 2 * 2 * 4
V_FIELD = 4  # sites kept for the field-valued outputs (diquark, sequential)


def projectors():
    """Flat project_mn arrays: (1 + g4)/2, (1 - g4)/2 and a seeded dense one."""
    g4 = eo.GAMMA[8]
    p_plus = ((np.eye(4) + g4) / 2).reshape(16)
    p_minus = ((np.eye(4) - g4) / 2).reshape(16)
    rng = np.random.default_rng(7)
    dense = (rng.standard_normal(16) + 1j * rng.standard_normal(16))
    return np.stack([p_plus, p_minus, dense]).astype(np.complex128)


def main():
    ref = L.ref_oracle()
    if ref is None:
        raise SystemExit("oracle/_ref/libcontract_ref.so not built (make -C oracle ref)")
    pi = eo.make_propagator(LATT, seed=11, mass=0.25)
    pj = eo.make_propagator(LATT, seed=12, mass=0.25)
    pn = eo.make_propagator(LATT, seed=13, mass=0.30)

    tables = L.ref_gamma_tables()

    meson = np.zeros((16, 16, V), np.complex128)
    for a in range(16):
        for b in range(16):
            meson[a, b] = ref.meson_two_point(pi, pj, a, b)
    meson_all_source = ref.meson_all_source(pi, pj, 5)
    meson_all_sink = ref.meson_all_sink(pi, pj, 10)

    baryon_gammas = np.array([(5, 5), (13, 9)], np.int64)
    baryon = np.zeros((len(baryon_gammas), 6, 16, V), np.complex128)
    for g, (gij, gkl) in enumerate(baryon_gammas):
        for t in range(6):
            for gmn in range(16):
                baryon[g, t, gmn] = ref.baryon_two_point(pi, pj, pn, t, int(gij), int(gkl), gmn)

    proj = projectors()
    general = np.zeros((len(proj), 6, V), np.complex128)
    for p in range(len(proj)):
        for t in range(6):
            general[p, t] = ref.baryon_general_two_point(pi, pj, pn, t, 5, 5, proj[p])

    fi, fj, fn = pi[:V_FIELD], pj[:V_FIELD], pn[:V_FIELD]
    diquark_gammas = np.array([(g, 5) for g in range(16)] + [(5, 0), (5, 15), (3, 12)], np.int64)
    diquark = np.stack([ref.baryon_diquark(fi, fj, int(a), int(b)) for a, b in diquark_gammas])

    seq_gmn = np.array([8, 3], np.int64)
    sequential = np.zeros((len(seq_gmn), 6, 3, V_FIELD, 4, 4, 3, 3), np.complex128)
    for g, gmn in enumerate(seq_gmn):
        for t in range(6):
            for s in range(3):
                sequential[g, t, s] = ref.baryon_sequential(fi, fj, fn, t, s, 5, 5, int(gmn))

    np.savez_compressed(
        os.path.join(HERE, "reference_small.npz"),
        latt=np.array(LATT), pi=pi, pj=pj, pn=pn,
        gamma_index=tables["index"], gamma_data=tables["data"], gamma_data_t=tables["data_t"],
        gamma_g_g5=tables["g_g5"], gamma_g5_g_t=tables["g5_g_t"],
        meson=meson, meson_all_source=meson_all_source, meson_all_sink=meson_all_sink,
        baryon_gammas=baryon_gammas, baryon=baryon,
        projectors=proj, general=general,
        diquark_gammas=diquark_gammas, diquark=diquark,
        seq_gmn=seq_gmn, sequential=sequential,
    )
    print("wrote", os.path.join(HERE, "reference_small.npz"))


if __name__ == "__main__":
    main()
