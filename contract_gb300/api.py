"""Extension API on CUDA tensors: per-timeslice sums, all baryon types in one
pass, the mixed complex64 form and precision conversion.

Propagators: contiguous CUDA tensors of ``V*144`` complex entries in PyQUDA
even/odd order (any shape with 144 trailing entries per site).  complex128
selects the plain form, complex64 the mixed form (FP32 arithmetic, FP64
timeslice reduction).  ``latt = (Lx, Ly, Lz, Lt)``.  Results are complex128.
"""
import ctypes

import numpy as np

from . import _lib
from .pycontract import (CONTRACT_C128, CONTRACT_C64, _check, _complex_host, _lib_record, _ptr, _ptr_array, _volume,
                         decompose_gamma)


def _torch():
    import torch
    return torch


def _prec(p):
    return CONTRACT_C128 if p.dtype == _torch().complex128 else CONTRACT_C64


def _latt(latt):
    a = (ctypes.c_int * 4)(*[int(x) for x in latt])
    return a


def _gamma_int(g):
    n, c = decompose_gamma(g)
    if c != 1:
        raise ValueError("pass bare gamma indices (or unit-phase basis matrices) to the extension API")
    return n


def to_c64(p):
    """complex128 propagator -> new complex64 tensor (device conversion kernel)."""
    torch = _torch()
    v = _volume(p)
    out = torch.empty(p.shape, dtype=torch.complex64, device=p.device)
    lib = _lib_record()
    lib.contract_convert_precision(_ptr(out), _ptr(p), v, 1)
    _check(lib)
    return out


def to_c128(p):
    torch = _torch()
    v = _volume(p)
    out = torch.empty(p.shape, dtype=torch.complex128, device=p.device)
    lib = _lib_record()
    lib.contract_convert_precision(_ptr(out), _ptr(p), v, 0)
    _check(lib)
    return out


def meson_timeslice(propag_i, propag_j, latt, gamma_ij, gamma_kl):
    """Zero-momentum meson correlator per timeslice: [Lt]."""
    torch = _torch()
    v = _volume(propag_i, propag_j)
    out = torch.empty(int(latt[3]), dtype=torch.complex128, device=propag_i.device)
    lib = _lib_record()
    lib.contract_meson(_ptr(out), _ptr(propag_i), _ptr(propag_j), v, _gamma_int(gamma_ij), _gamma_int(gamma_kl),
                       _prec(propag_i), _latt(latt))
    _check(lib)
    return out


def meson_all_timeslice(propag_i, propag_j, latt, fixed_gamma, source=True):
    """[16, Lt]: all Gamma_kl (source=True) or all Gamma_ij for a fixed partner."""
    torch = _torch()
    v = _volume(propag_i, propag_j)
    out = torch.empty((16, int(latt[3])), dtype=torch.complex128, device=propag_i.device)
    lib = _lib_record()
    lib.contract_meson_all(_ptr_array([out[k] for k in range(16)]), _ptr(propag_i), _ptr(propag_j), v,
                           _gamma_int(fixed_gamma), int(bool(source)), _prec(propag_i), _latt(latt))
    _check(lib)
    return out


def baryon(propag_i, propag_j, propag_n, contract_type, gamma_ij, gamma_kl, gamma_mn=None, project_mn=None,
           latt=None):
    """Baryon two-point per site ([V], latt None) or per timeslice ([Lt])."""
    torch = _torch()
    v = _volume(propag_i, propag_j, propag_n)
    n_out = v if latt is None else int(latt[3])
    out = torch.empty(n_out, dtype=torch.complex128, device=propag_i.device)
    proj = None if project_mn is None else _complex_host(project_mn, 16)
    gmn = 0 if gamma_mn is None else _gamma_int(gamma_mn)
    if proj is None and gamma_mn is None:
        raise ValueError("give gamma_mn or project_mn")
    lib = _lib_record()
    lib.contract_baryon(_ptr(out), _ptr(propag_i), _ptr(propag_j), _ptr(propag_n), int(contract_type), v,
                        _gamma_int(gamma_ij), _gamma_int(gamma_kl), gmn, None if proj is None else proj.ctypes.data,
                        _prec(propag_i), None if latt is None else _latt(latt))
    _check(lib)
    return out


def baryon_all_types(propag_i, propag_j, propag_n, gamma_ij, gamma_kl, projectors, latt=None, out=None):
    """All six contraction types for 1 or 2 projectors in one pass.

    Returns [6, nproj, Lt] (latt given) or [6, nproj, V], types in
    BaryonContractType order.
    """
    torch = _torch()
    v = _volume(propag_i, propag_j, propag_n)
    projs = np.ascontiguousarray(np.asarray(projectors, dtype=np.complex128).reshape(-1, 16))
    nproj = projs.shape[0]
    n_out = v if latt is None else int(latt[3])
    if out is None:
        out = torch.empty((6, nproj, n_out), dtype=torch.complex128, device=propag_i.device)
    lib = _lib_record()
    lib.contract_baryon_all_types(_ptr(out), _ptr(propag_i), _ptr(propag_j), _ptr(propag_n), v,
                                  _gamma_int(gamma_ij), _gamma_int(gamma_kl), nproj, projs.ctypes.data,
                                  _prec(propag_i), None if latt is None else _latt(latt))
    _check(lib)
    return out


def _quda_fields(fields, latt, stride, dtype):
    torch = _torch()
    if len(fields) != 12:
        raise ValueError("a propagator is 12 QUDA colour-spinor fields (source spin k, colour d: field 3k + d)")
    half = int(np.prod([int(x) for x in latt])) // 2
    stride = int(stride) if stride else half
    need = 2 * 12 * stride  # complex entries per field: [2][chunks][stride][16 B]
    for f in fields:
        if not isinstance(f, torch.Tensor) or not f.is_cuda or not f.is_contiguous() or f.dtype != dtype:
            raise TypeError(f"QUDA fields must be contiguous CUDA tensors of {dtype}")
        if f.numel() < need:
            raise ValueError(f"QUDA field holds {f.numel()} complex entries, needs {need}")
    arr = (ctypes.c_void_p * 12)(*[f.data_ptr() for f in fields])
    return arr, stride


def from_quda(fields, latt, stride=0, out=None):
    """Propagator [V, 4, 4, 3, 3] in PyQUDA even/odd order from QUDA's 12
    native-order colour-spinor fields (complex128: FLOAT2 order; complex64:
    FLOAT4 order), each [2][chunks][stride][16 bytes]."""
    torch = _torch()
    dtype = fields[0].dtype
    arr, stride = _quda_fields(fields, latt, stride, dtype)
    v = int(np.prod([int(x) for x in latt]))
    if out is None:
        out = torch.empty((v, 4, 4, 3, 3), dtype=dtype, device=fields[0].device)
    lib = _lib_record()
    lib.contract_convert_from_quda(_ptr(out), arr, _latt(latt), stride,
                                   CONTRACT_C128 if dtype == torch.complex128 else CONTRACT_C64)
    _check(lib)
    return out


def to_quda(propag, latt, stride=0):
    """The 12 QUDA native-order colour-spinor fields of a PyQUDA even/odd
    propagator; each field is a flat tensor of 2 * 12 * stride complex entries
    whose pad sites (beyond V/2 in each parity) are zero."""
    torch = _torch()
    v = _volume(propag)
    half = v // 2
    stride = int(stride) if stride else half
    fields = [torch.zeros(2 * 12 * stride, dtype=propag.dtype, device=propag.device) for _ in range(12)]
    arr, stride = _quda_fields(fields, latt, stride, propag.dtype)
    lib = _lib_record()
    lib.contract_convert_to_quda(arr, _ptr(propag), _latt(latt), stride, _prec(propag))
    _check(lib)
    return fields


def rotate_spin_basis(propag, rotation):
    """In place P -> U P U^dagger on both spin indices (U: 4 x 4 complex)."""
    v = _volume(propag)
    u = np.ascontiguousarray(np.asarray(rotation, dtype=np.complex128).reshape(4, 4))
    lib = _lib_record()
    lib.contract_rotate_spin_basis(_ptr(propag), v, u.ctypes.data, _prec(propag))
    _check(lib)
    return propag


def set_stream(stream):
    """Queue library work on a torch.cuda.Stream (or raw cudaStream_t int); None = legacy default."""
    lib = _lib.lib()
    handle = None if stream is None else (stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
    lib.contract_set_stream(handle)


def check_device():
    """Synchronise and raise if a kernel reported an error through the device status word."""
    lib = _lib_record()
    lib.contract_check_device()
    _check(lib)


def projector_plus_minus():
    """(1 + g4)/2 and (1 - g4)/2 as a [2, 16] complex array (Gamma(8) = g4)."""
    from .pycontract import gamma_matrices
    g4 = gamma_matrices()[8]
    e = np.eye(4)
    return np.stack([((e + g4) / 2).reshape(16), ((e - g4) / 2).reshape(16)])
