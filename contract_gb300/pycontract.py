"""Python binding of libcontract.so, mirroring the ``pycontract`` plugin.

CLQCD/contract's Python binding is generated by ``pyquda_plugins`` from
``contract.h`` (README.md:13) and is used as ``pycontract.baryonTwoPoint(...)``
with ``pycontract.BaryonContractType`` (baryon_2pt.py:30,92,108).  This module
offers the same two layers on top of the C ABI:

* the C entry points under their C names, taking device pointers (ints) or
  CUDA tensors, ``volume`` and integer selectors -- exactly the ABI;
* camelCase helpers on CUDA tensors (``mesonTwoPoint``, ``baryonTwoPoint``,
  ...) that allocate the output, accept gamma matrices as integers or as 4x4
  matrices (a phase times a basis element; for the Gamma_mn slot any 4x4
  projector) and return tensors.

Errors raise ``ContractError``: importing this module switches the library to
its recording error mode instead of the reference's exit-on-error.
"""
import ctypes
import enum

import numpy as np

from . import _lib

_L = _lib.lib


class ContractError(RuntimeError):
    pass


class BaryonContractType(enum.IntEnum):
    """contract_enum.h:1-20 (values and aliases)."""
    IK_JL_NM = 0
    IK_JM_NL = 1
    IL_JK_NM = 2
    IL_JM_NK = 3
    IM_JK_NL = 4
    IM_JL_NK = 5
    AD_BE_CF = 0
    AD_BF_CE = 1
    AE_BD_CF = 2
    AE_BF_CD = 3
    AF_BD_CE = 4
    AF_BE_CD = 5
    IK_JL_MN = 0
    IK_JN_ML = 1
    IL_JK_MN = 2
    IL_JN_MK = 3
    IN_JK_ML = 4
    IN_JL_MK = 5


class BaryonSequentialType(enum.IntEnum):
    """contract_enum.h:22-26."""
    SEQUENTIAL_I = 0
    SEQUENTIAL_J = 1
    SEQUENTIAL_N = 2


CONTRACT_C128 = 0
CONTRACT_C64 = 1
CONTRACT_C64_TC = 2  # momentum projection on the tensor cores (split bf16)
_ERRORS_RECORD = 1


def _lib_record():
    lib = _L()
    lib.contract_set_error_mode(_ERRORS_RECORD)
    return lib


def _check(lib):
    code = lib.contract_last_error()
    if code:
        msg = lib.contract_last_error_message().decode()
        lib.contract_clear_error()
        raise ContractError(f"libcontract error {code}: {msg}")


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"expected a device pointer or tensor, got {type(x).__name__}")


def _ptr_array(ptrs):
    arr = (ctypes.c_void_p * 16)()
    if len(ptrs) != 16:
        raise ValueError("need 16 output pointers")
    for k, p in enumerate(ptrs):
        arr[k] = _ptr(p)
    return arr


def _complex_host(values, n):
    a = np.ascontiguousarray(np.asarray(values, dtype=np.complex128).reshape(n))
    return a


# ------------------------------------------------------------ C entry points --

def init(device: int):
    lib = _lib_record()
    lib.init(int(device))
    _check(lib)


def meson_two_point(correl, propag_i, propag_j, volume, gamma_ij, gamma_kl):
    lib = _lib_record()
    lib.meson_two_point(_ptr(correl), _ptr(propag_i), _ptr(propag_j), int(volume), int(gamma_ij), int(gamma_kl))
    _check(lib)


def meson_all_source_two_point(correl, propag_i, propag_j, volume, gamma_ij):
    lib = _lib_record()
    lib.meson_all_source_two_point(_ptr_array(correl), _ptr(propag_i), _ptr(propag_j), int(volume), int(gamma_ij))
    _check(lib)


def meson_all_sink_two_point(correl, propag_i, propag_j, volume, gamma_kl):
    lib = _lib_record()
    lib.meson_all_sink_two_point(_ptr_array(correl), _ptr(propag_i), _ptr(propag_j), int(volume), int(gamma_kl))
    _check(lib)


def baryon_diquark(diquark, propag_i, propag_j, volume, gamma_ij, gamma_kl):
    lib = _lib_record()
    lib.baryon_diquark(_ptr(diquark), _ptr(propag_i), _ptr(propag_j), int(volume), int(gamma_ij), int(gamma_kl))
    _check(lib)


def baryon_two_point(correl, propag_i, propag_j, propag_n, contract_type, volume, gamma_ij, gamma_kl, gamma_mn):
    lib = _lib_record()
    lib.baryon_two_point(_ptr(correl), _ptr(propag_i), _ptr(propag_j), _ptr(propag_n), int(contract_type),
                         int(volume), int(gamma_ij), int(gamma_kl), int(gamma_mn))
    _check(lib)


def baryon_general_two_point(correl, propag_i, propag_j, propag_n, contract_type, volume, gamma_ij, gamma_kl,
                             project_mn):
    lib = _lib_record()
    proj = _complex_host(project_mn, 16)
    lib.baryon_general_two_point(_ptr(correl), _ptr(propag_i), _ptr(propag_j), _ptr(propag_n), int(contract_type),
                                 int(volume), int(gamma_ij), int(gamma_kl), proj.ctypes.data)
    _check(lib)


def baryon_sequential_two_point(propag_i, propag_j, propag_n, contract_type, sequential_type, volume, gamma_ij,
                                gamma_kl, gamma_mn):
    lib = _lib_record()
    lib.baryon_sequential_two_point(_ptr(propag_i), _ptr(propag_j), _ptr(propag_n), int(contract_type),
                                    int(sequential_type), int(volume), int(gamma_ij), int(gamma_kl), int(gamma_mn))
    _check(lib)


# -------------------------------------------------------------- gamma algebra --

def gamma_table():
    """(perm[16, 4], phase[16, 4]) with Gamma(n)[r, perm[n, r]] = i**phase[n, r]."""
    lib = _L()
    perm = (ctypes.c_int * 64)()
    phase = (ctypes.c_int * 64)()
    lib.contract_gamma_table(perm, phase)
    return np.array(perm[:]).reshape(16, 4), np.array(phase[:]).reshape(16, 4)


def gamma_matrices():
    """The 16 gamma matrices as a [16, 4, 4] complex128 array."""
    perm, phase = gamma_table()
    g = np.zeros((16, 4, 4), np.complex128)
    for n in range(16):
        for r in range(4):
            g[n, r, perm[n, r]] = 1j ** phase[n, r]
    return g


def _as_matrix(g):
    if hasattr(g, "matrix"):  # PyQUDA Gamma / Polarize objects
        g = g.matrix
    if hasattr(g, "get"):  # cupy
        g = g.get()
    if hasattr(g, "detach"):
        g = g.detach().cpu().numpy()
    return np.asarray(g, dtype=np.complex128).reshape(4, 4)


def decompose_gamma(g):
    """Return (index, phase) with g == phase * Gamma(index); g an int or a 4x4 matrix.

    Raises ValueError if g is not a unit-modulus multiple of a basis element.
    """
    if isinstance(g, (int, np.integer)) or (hasattr(g, "__index__") and not hasattr(g, "shape")):
        return int(g), 1.0 + 0.0j
    m = _as_matrix(g)
    for n, b in enumerate(gamma_matrices()):
        c = np.vdot(b.ravel(), m.ravel()) / 4.0  # <Gamma(n), m> / 4
        if abs(abs(c) - 1.0) < 1e-12 and np.allclose(m, c * b, atol=1e-12):
            return n, complex(c)
    raise ValueError("matrix is not a phase times a gamma basis element")


# ------------------------------------------------------------ tensor helpers --

def _torch():
    import torch
    return torch


def _check_prop(p, name):
    torch = _torch()
    if not isinstance(p, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not p.is_cuda:
        raise ValueError(f"{name} must live on a CUDA device")
    if p.dtype not in (torch.complex128, torch.complex64):
        raise TypeError(f"{name} must be complex128 (or complex64 for the mixed form)")
    if not p.is_contiguous() or p.numel() % 144:
        raise ValueError(f"{name} must be contiguous with a multiple of 144 entries per site")
    return p.numel() // 144


def _volume(*props):
    vols = {_check_prop(p, f"propag_{k}") for k, p in enumerate(props)}
    if len(vols) != 1:
        raise ValueError("propagators have different volumes")
    if len({p.dtype for p in props}) != 1:
        raise ValueError("propagators have different dtypes")
    return vols.pop()


def mesonTwoPoint(propag_i, propag_j, gamma_ij, gamma_kl):
    """Per-site meson two-point, [V] complex128."""
    torch = _torch()
    v = _volume(propag_i, propag_j)
    (a, ca), (b, cb) = decompose_gamma(gamma_ij), decompose_gamma(gamma_kl)
    out = torch.empty(v, dtype=torch.complex128, device=propag_i.device)
    if propag_i.dtype == torch.complex128:
        meson_two_point(out, propag_i, propag_j, v, a, b)
    else:
        lib = _lib_record()
        lib.contract_meson(_ptr(out), _ptr(propag_i), _ptr(propag_j), v, a, b, CONTRACT_C64, None)
        _check(lib)
    return out if ca * cb == 1 else out * (ca * cb)


def _meson_all(propag_i, propag_j, gamma, source):
    torch = _torch()
    v = _volume(propag_i, propag_j)
    g, c = decompose_gamma(gamma)
    out = torch.empty((16, v), dtype=torch.complex128, device=propag_i.device)
    ptrs = [out[k] for k in range(16)]
    if propag_i.dtype == torch.complex128:
        (meson_all_source_two_point if source else meson_all_sink_two_point)(ptrs, propag_i, propag_j, v, g)
    else:
        lib = _lib_record()
        lib.contract_meson_all(_ptr_array(ptrs), _ptr(propag_i), _ptr(propag_j), v, g, int(source), CONTRACT_C64,
                               None)
        _check(lib)
    return out if c == 1 else out * c


def mesonAllSourceTwoPoint(propag_i, propag_j, gamma_ij):
    """[16, V]: all Gamma_kl for a fixed Gamma_ij."""
    return _meson_all(propag_i, propag_j, gamma_ij, True)


def mesonAllSinkTwoPoint(propag_i, propag_j, gamma_kl):
    """[16, V]: all Gamma_ij for a fixed Gamma_kl."""
    return _meson_all(propag_i, propag_j, gamma_kl, False)


def baryonDiquark(propag_i, propag_j, gamma_ij, gamma_kl):
    """Diquark field shaped like the propagators (complex conjugation makes it
    antilinear in the gamma phases, handled here)."""
    torch = _torch()
    v = _volume(propag_i, propag_j)
    (a, ca), (b, cb) = decompose_gamma(gamma_ij), decompose_gamma(gamma_kl)
    out = torch.empty_like(propag_i)
    lib = _lib_record()
    prec = CONTRACT_C128 if propag_i.dtype == torch.complex128 else CONTRACT_C64
    lib.contract_diquark(_ptr(out), _ptr(propag_i), _ptr(propag_j), v, a, b, prec)
    _check(lib)
    c = np.conj(ca * cb)
    return out if c == 1 else out * c


def _projector(gamma_mn):
    """(gamma index, phase, None) for a basis multiple, else (0, 1, flat project_mn)."""
    try:
        g, c = decompose_gamma(gamma_mn)
        return g, c, None
    except ValueError:
        return 0, 1.0, _complex_host(_as_matrix(gamma_mn), 16)


def baryonTwoPoint(propag_i, propag_j, propag_m, contract_type, gamma_ij, gamma_kl, gamma_mn):
    """Per-site baryon two-point [V]; gamma_mn may be any 4x4 matrix (general projector)."""
    torch = _torch()
    v = _volume(propag_i, propag_j, propag_m)
    (a, ca), (b, cb) = decompose_gamma(gamma_ij), decompose_gamma(gamma_kl)
    gmn, cmn, proj = _projector(gamma_mn)
    out = torch.empty(v, dtype=torch.complex128, device=propag_i.device)
    prec = CONTRACT_C128 if propag_i.dtype == torch.complex128 else CONTRACT_C64
    lib = _lib_record()
    lib.contract_baryon(_ptr(out), _ptr(propag_i), _ptr(propag_j), _ptr(propag_m), int(contract_type), v, a, b, gmn,
                        None if proj is None else proj.ctypes.data, prec, None)
    _check(lib)
    c = ca * cb * cmn
    return out if c == 1 else out * c


def baryonSequentialTwoPoint(propag_i, propag_j, propag_m, contract_type, sequential_type, gamma_ij, gamma_kl,
                             gamma_mn):
    """Overwrite the selected propagator in place with dC/dP; returns it."""
    torch = _torch()
    v = _volume(propag_i, propag_j, propag_m)
    (a, ca), (b, cb), (g, cg) = decompose_gamma(gamma_ij), decompose_gamma(gamma_kl), decompose_gamma(gamma_mn)
    prec = CONTRACT_C128 if propag_i.dtype == torch.complex128 else CONTRACT_C64
    lib = _lib_record()
    lib.contract_sequential(_ptr(propag_i), _ptr(propag_j), _ptr(propag_m), int(contract_type), int(sequential_type),
                            v, a, b, g, prec)
    _check(lib)
    target = (propag_i, propag_j, propag_m)[int(sequential_type)]
    c = ca * cb * cg
    if c != 1:
        target.mul_(c)
    return target
