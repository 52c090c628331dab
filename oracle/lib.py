"""ctypes loaders for the compiled CPU oracles (test infrastructure only).

``C``   -- ``oracle/_ref/liboracle.so``, the plain-C restatement
           (``contract_oracle.c``), built by ``make -C oracle`` on any host.
``REF`` -- ``oracle/_ref/libcontract_ref.so``, the reference's own per-site
           functions compiled as host C++ (``make -C oracle ref``); ``None``
           when the reference sources were not available to build it.

Both take/return numpy complex128 arrays shaped like the C ABI's buffers.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def build(ref=False):
    """Compile the C oracle (and the reference host build when ``ref``)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"] + (["ref"] if ref else []), check=True)


def _load(name):
    path = os.path.join(OUT, name)
    if not os.path.exists(path):
        return None
    try:
        return ctypes.CDLL(path)
    except OSError:  # built for another host architecture
        return None


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


class _Lib:
    """Uniform numpy front end over either compiled oracle."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.prefix = prefix

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def meson_two_point(self, pi, pj, gamma_ij, gamma_kl):
        pi, pj = _c(pi), _c(pj)
        v = pi.size // 144
        out = np.zeros(v, np.complex128)
        self._f("meson_two_point")(_p(out), _p(pi), _p(pj), ctypes.c_size_t(v), gamma_ij, gamma_kl)
        return out

    def meson_all_source(self, pi, pj, gamma_ij):
        pi, pj = _c(pi), _c(pj)
        v = pi.size // 144
        out = np.zeros((16, v), np.complex128)
        self._f("meson_all_source")(_p(out), _p(pi), _p(pj), ctypes.c_size_t(v), gamma_ij)
        return out

    def meson_all_sink(self, pi, pj, gamma_kl):
        pi, pj = _c(pi), _c(pj)
        v = pi.size // 144
        out = np.zeros((16, v), np.complex128)
        self._f("meson_all_sink")(_p(out), _p(pi), _p(pj), ctypes.c_size_t(v), gamma_kl)
        return out

    def baryon_two_point(self, pi, pj, pn, contract_type, gamma_ij, gamma_kl, gamma_mn):
        pi, pj, pn = _c(pi), _c(pj), _c(pn)
        v = pi.size // 144
        out = np.zeros(v, np.complex128)
        rc = self._f("baryon_two_point")(_p(out), _p(pi), _p(pj), _p(pn), int(contract_type), ctypes.c_size_t(v),
                                         gamma_ij, gamma_kl, gamma_mn)
        if rc not in (0, None) and self.prefix == "ref_":
            raise ValueError("bad contraction selector")
        return out

    def baryon_general_two_point(self, pi, pj, pn, contract_type, gamma_ij, gamma_kl, project_mn):
        pi, pj, pn = _c(pi), _c(pj), _c(pn)
        proj = _c(np.asarray(project_mn).reshape(16))
        v = pi.size // 144
        out = np.zeros(v, np.complex128)
        name = "baryon_general_two_point" if self.prefix == "ref_" else "baryon_general"
        self._f(name)(_p(out), _p(pi), _p(pj), _p(pn), int(contract_type), ctypes.c_size_t(v), gamma_ij, gamma_kl,
                      _p(proj))
        return out

    def baryon_diquark(self, pi, pj, gamma_ij, gamma_kl):
        pi, pj = _c(pi), _c(pj)
        v = pi.size // 144
        out = np.zeros_like(pi)
        self._f("baryon_diquark")(_p(out), _p(pi), _p(pj), ctypes.c_size_t(v), gamma_ij, gamma_kl)
        return out

    def baryon_sequential(self, pi, pj, pn, contract_type, sequential_type, gamma_ij, gamma_kl, gamma_mn):
        """Return the overwritten slot (inputs are copied, not modified)."""
        bufs = [_c(pi).copy(), _c(pj).copy(), _c(pn).copy()]
        v = bufs[0].size // 144
        name = "baryon_sequential_two_point" if self.prefix == "ref_" else "baryon_sequential"
        self._f(name)(_p(bufs[0]), _p(bufs[1]), _p(bufs[2]), int(contract_type), int(sequential_type),
                      ctypes.c_size_t(v), gamma_ij, gamma_kl, gamma_mn)
        return bufs[int(sequential_type)]


def c_oracle():
    lib = _load("liboracle.so")
    return _Lib(lib, "oracle_") if lib is not None else None


def ref_oracle():
    lib = _load("libcontract_ref.so")
    if lib is None or not hasattr(lib, "ref_meson_two_point"):
        return None
    return _Lib(lib, "ref_")


def ref_gamma_tables():
    """The reference's own gamma switch tables, or None if not built."""
    lib = _load("libcontract_ref.so")
    if lib is None:
        return None
    idx = np.zeros(64, np.int32)
    bufs = [np.zeros(64, np.complex128) for _ in range(4)]
    lib.ref_gamma_tables(_p(idx), *[_p(b) for b in bufs])
    names = ("data", "data_t", "g_g5", "g5_g_t")
    out = {"index": idx.reshape(16, 4).astype(np.int64)}
    out.update({n: b.reshape(16, 4) for n, b in zip(names, bufs)})
    return out


def c_gamma_tables():
    lib = _load("liboracle.so")
    idx = np.zeros(64, np.int32)
    data = np.zeros(64, np.complex128)
    lib.oracle_gamma_tables(_p(idx), _p(data))
    return idx.reshape(16, 4).astype(np.int64), data.reshape(16, 4)
