"""DeGrand-Rossi gamma algebra for the oracle (test infrastructure only).

The reference encodes its 16 gamma matrices as hand-written switch tables
(``include/gamma.cuh:41-127`` of CLQCD/contract).  Here the same 16 matrices
are *derived* from the four Euclidean gamma matrices of the DeGrand-Rossi
basis (the basis used by QUDA/PyQUDA):

    Gamma(n) = g1^(n&1) g2^((n>>1)&1) g3^((n>>2)&1) g4^((n>>3)&1)

so that ``Gamma(15) = g5 = diag(1, 1, -1, -1)``.  ``tests/test_gamma.py``
checks the derived tables bit-exactly against the reference's own switch
tables (host-compiled from ``gamma.cuh``) and the committed golden copy.
"""
import numpy as np

NS = 4
NC = 3

_I = 1j
G1 = np.array([[0, 0, 0, _I], [0, 0, _I, 0], [0, -_I, 0, 0], [-_I, 0, 0, 0]], dtype=np.complex128)
G2 = np.array([[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]], dtype=np.complex128)
G3 = np.array([[0, 0, _I, 0], [0, 0, 0, -_I], [-_I, 0, 0, 0], [0, _I, 0, 0]], dtype=np.complex128)
G4 = np.array([[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]], dtype=np.complex128)


def gamma(n: int) -> np.ndarray:
    """Return the 4x4 matrix Gamma(n), n in 0..15."""
    if not 0 <= n < 16:
        raise ValueError(f"gamma index {n} out of range")
    m = np.eye(4, dtype=np.complex128)
    for bit, g in enumerate((G1, G2, G3, G4)):
        if (n >> bit) & 1:
            m = m @ g
    return m


GAMMA = np.stack([gamma(n) for n in range(16)])
G5 = GAMMA[15]


def perm_phase(m: np.ndarray):
    """Decompose a one-nonzero-per-row 4x4 matrix into (perm[4], phase[4]).

    ``m[r, perm[r]] == phase[r]`` and every other entry is zero.
    """
    perm = np.full(4, -1, dtype=np.int64)
    phase = np.zeros(4, dtype=np.complex128)
    for r in range(4):
        nz = np.nonzero(np.abs(m[r]) > 0.5)[0]
        if len(nz) != 1:
            raise ValueError("matrix is not a signed permutation")
        perm[r] = nz[0]
        phase[r] = m[r, nz[0]]
    return perm, phase


def tables():
    """Index/phase tables of Gamma, Gamma^T, (Gamma g5) and (g5 Gamma)^T.

    Returns a dict of arrays shaped [16, 4]:
      ``index``       column of the single nonzero entry of row r
      ``data``        Gamma[r, index[r]]
      ``data_t``      (Gamma^T)[r, index[r]]  (= Gamma[index[r], r])
      ``g_g5``        (Gamma g5)[r, index[r]]
      ``g5_g_t``      ((g5 Gamma)^T)[r, index[r]]
    These are the quantities the reference's ``gamma_index``, ``gamma_data``
    and ``gamma_gamma5_data`` return (``gamma.cuh:58-127,225-271``).
    """
    out = {k: [] for k in ("index", "data", "data_t", "g_g5", "g5_g_t")}
    for n in range(16):
        g = GAMMA[n]
        p, ph = perm_phase(g)
        out["index"].append(p)
        out["data"].append(ph)
        out["data_t"].append(perm_phase(g.T)[1])
        out["g_g5"].append(perm_phase(g @ G5)[1])
        out["g5_g_t"].append(perm_phase((G5 @ g).T)[1])
    return {k: np.array(v) for k, v in out.items()}


def epsilon() -> np.ndarray:
    """Levi-Civita tensor eps[a, b, c] (int, 3x3x3)."""
    e = np.zeros((3, 3, 3), dtype=np.int64)
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        e[a, b, c] = 1
        e[a, c, b] = -1
    return e
