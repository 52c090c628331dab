"""The reference's own CUDA kernels, run on this GPU (test infrastructure only).

``make -C oracle refgpu REF=<checkout>`` compiles each of the reference's CUDA
translation units (``lib/meson/*.cu``, ``lib/baryon/*.cu``) unmodified into an
sm_103a cubin under ``oracle/_ref/gpu/``.  A cubin holds device code only, so it
loads on any host (the aarch64 GPU machine as well as this x86 container) through
the CUDA driver API.  This module loads those cubins with ``libcuda`` via
ctypes and replays the reference's host-side launch for each ``contract.h``
entry point:

* the argument struct of each op is packed as the reference declares it
  (``MesonArgs`` ``include/meson.cuh:17-31``, ``MesonAllArgs``
  ``include/meson_all.cuh:17-30``, ``BaryonArgs`` ``include/baryon.cuh:16-32``,
  ``BaryonGeneralArgs`` ``include/baryon_general.cuh:16-35`` with its
  ``alignas(16)`` ``Complex<double>`` projector (``include/complex.cuh:13``),
  ``DiquarkArgs`` ``include/diquark.cuh:16-30``, ``BaryonSequentialArgs``
  ``include/baryon_sequential.cuh:19-34``);
* it is copied into the module's ``__constant__ target::buffer``
  (``include/kernel.cuh:49``, ``:180``) with a synchronous host->device copy,
  as ``cudaMemcpyToSymbol`` does in ``lib/target/runtime_api_cuda.cpp:31-32``;
* the template kernel ``contract::kernel<Kernel, Args>`` (``include/kernel.cuh:159-171``)
  is launched on the legacy default stream with
  ``grid = (volume * 16 + 63) / 64`` blocks of 64 threads (``include/kernel.cuh:173-177``;
  every op uses BLOCK_SIZE 64 and TILE_SIZE 16), after the reference's
  ``volume % 4`` check (e.g. ``lib/baryon/baryon.cu:10-13``).

Kernels are found by their Itanium-mangled names, built from the template
arguments the reference's dispatch switches instantiate (``lib/baryon/baryon.cu:25-45``
and the like).  Pointers are raw device addresses (ints), as in ``contract.h``.
Nothing here is used by the library: tests and ``bench.py``'s reference legs
call it to compare with, and time beside, the library on identical inputs.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN_DIR = os.path.join(HERE, "_ref", "gpu")
UNITS = ("meson", "meson_all", "baryon", "baryon_general", "diquark", "baryon_sequential_i",
         "baryon_sequential_j", "baryon_sequential_n")
TILES_PER_BLOCK = 4   # BLOCK_SIZE 64 / TILE_SIZE 16 in every op header
BLOCK = 64
BUFFER_SYMBOL = b"_ZN6target6bufferE"


def available():
    """True when every reference cubin has been built."""
    return all(os.path.exists(os.path.join(CUBIN_DIR, u + ".cubin")) for u in UNITS)


def _src(n):
    return f"{len(n)}{n}"


def _mangle(kernel, args, targs, enum):
    # void contract::kernel<contract::K<contract::A<targs>>, contract::A<targs>>()
    # S3_ / S4_ refer back to A<targs>; the enum type BaryonContractType adds one substitution.
    back = "S4_" if enum else "S3_"
    return f"_ZN8contract6kernelINS_{_src(kernel)}INS_{_src(args)}I{targs}EEEE{back}EEvv".encode()


def _ctype(t):
    return f"L18BaryonContractType{int(t)}E"


def kernel_name(op, contract_type=0, gamma=0, seq=None):
    if op == "meson":
        return _mangle("MesonKernel", "MesonArgs", "d", False)
    if op == "meson_all_source":
        return _mangle("MesonAllSourceKernel", "MesonAllArgs", "d", False)
    if op == "meson_all_sink":
        return _mangle("MesonAllSinkKernel", "MesonAllArgs", "d", False)
    if op == "baryon":
        return _mangle("BaryonKernel", "BaryonArgs", f"d{_ctype(contract_type)}Li{int(gamma)}E", True)
    if op == "baryon_general":
        return _mangle("BaryonGeneralKernel", "BaryonGeneralArgs", f"d{_ctype(contract_type)}", True)
    if op == "diquark":
        return _mangle("DiquarkKernel", "DiquarkArgs", f"Li{int(gamma)}Ed", False)
    if op == "sequential":
        return _mangle(f"BaryonSequential{'IJN'[seq]}Kernel", "BaryonSequentialArgs",
                       f"d{_ctype(contract_type)}Li{int(gamma)}E", True)
    raise ValueError(op)


# ---------------------------------------------------------------- arg structs --

class MesonArgs(ctypes.Structure):
    _fields_ = [("correl", ctypes.c_void_p), ("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p),
                ("gamma_ij", ctypes.c_int), ("gamma_kl", ctypes.c_int)]


class MesonAllArgs(ctypes.Structure):
    _fields_ = [("correl", ctypes.c_void_p * 16), ("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p),
                ("gamma", ctypes.c_int)]


class BaryonArgs(ctypes.Structure):
    _fields_ = [("correl", ctypes.c_void_p), ("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p),
                ("propag_n", ctypes.c_void_p), ("gamma_ij", ctypes.c_int), ("gamma_kl", ctypes.c_int)]


class BaryonGeneralArgs(ctypes.Structure):
    # 40 bytes of pointers and ints, then the 16-byte aligned projector at offset 48
    _fields_ = [("correl", ctypes.c_void_p), ("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p),
                ("propag_n", ctypes.c_void_p), ("gamma_ij", ctypes.c_int), ("gamma_kl", ctypes.c_int),
                ("_pad", ctypes.c_char * 8), ("project_mn", ctypes.c_double * 32)]


class DiquarkArgs(ctypes.Structure):
    _fields_ = [("diquark", ctypes.c_void_p), ("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p),
                ("gamma_ij", ctypes.c_int), ("gamma_kl", ctypes.c_int)]


class BaryonSequentialArgs(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("propag_n", ctypes.c_void_p),
                ("gamma_ij", ctypes.c_int), ("gamma_kl", ctypes.c_int)]


assert ctypes.sizeof(MesonArgs) == 32 and ctypes.sizeof(BaryonArgs) == 40
assert ctypes.sizeof(MesonAllArgs) == 152 and ctypes.sizeof(BaryonGeneralArgs) == 304
assert BaryonGeneralArgs.project_mn.offset == 48


# ------------------------------------------------------------------ driver API --

class CudaError(RuntimeError):
    pass


class ReferenceGPU:
    """Loaded reference cubins on one device (the primary context torch also uses)."""

    def __init__(self, device=0):
        if not available():
            raise FileNotFoundError(f"reference cubins missing in {CUBIN_DIR} (make -C oracle refgpu REF=...)")
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.cu.cuDeviceGet(ctypes.byref(dev), int(device)), "cuDeviceGet")
        self.ctx = ctypes.c_void_p()
        self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self.modules, self.buffers, self.funcs = {}, {}, {}
        with self:
            for u in UNITS:
                mod = ctypes.c_void_p()
                path = os.path.join(CUBIN_DIR, u + ".cubin").encode()
                self._check(self.cu.cuModuleLoad(ctypes.byref(mod), path), f"cuModuleLoad {u}")
                dptr, size = ctypes.c_uint64(), ctypes.c_size_t()
                self._check(self.cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(size), mod, BUFFER_SYMBOL),
                            f"constant buffer of {u}")
                self.modules[u] = mod
                self.buffers[u] = (dptr.value, size.value)

    # context management: push the primary context around every driver call
    def __enter__(self):
        self._check(self.cu.cuCtxPushCurrent_v2(self.ctx), "cuCtxPushCurrent")
        return self

    def __exit__(self, *exc):
        old = ctypes.c_void_p()
        self.cu.cuCtxPopCurrent_v2(ctypes.byref(old))

    def _check(self, rc, what):
        if rc != 0:
            msg = ctypes.c_char_p()
            self.cu.cuGetErrorString(rc, ctypes.byref(msg))
            raise CudaError(f"{what}: CUDA driver error {rc} ({(msg.value or b'?').decode()})")

    def _func(self, unit, name):
        key = (unit, name)
        if key not in self.funcs:
            fn = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), self.modules[unit], name),
                        f"kernel {name.decode()} in {unit}")
            self.funcs[key] = fn
        return self.funcs[key]

    def _launch(self, unit, name, args, volume):
        """The reference's contract_launch_kernel: constant-buffer copy, then the launch."""
        volume = int(volume)
        if volume % TILES_PER_BLOCK != 0:
            raise ValueError("Volume must be a multiple of TILES_PER_BLOCK")
        if volume == 0:
            return
        grid = (volume * 16 + BLOCK - 1) // BLOCK
        with self:
            fn = self._func(unit, name)
            dptr, size = self.buffers[unit]
            assert ctypes.sizeof(args) <= size
            self._check(self.cu.cuMemcpyHtoD_v2(ctypes.c_uint64(dptr), ctypes.byref(args),
                                                ctypes.c_size_t(ctypes.sizeof(args))), "constant buffer copy")
            self._check(self.cu.cuLaunchKernel(fn, grid, 1, 1, BLOCK, 1, 1, 0, None, None, None), "cuLaunchKernel")

    def synchronize(self):
        with self:
            self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    # ------------------------------------------------ contract.h entry points --
    # Same argument order and meaning as include/contract.h:15-27.

    def meson_two_point(self, correl, propag_i, propag_j, volume, gamma_ij, gamma_kl):
        a = MesonArgs(correl, propag_i, propag_j, gamma_ij, gamma_kl)
        self._launch("meson", kernel_name("meson"), a, volume)

    def _meson_all(self, op, correl16, propag_i, propag_j, volume, gamma):
        a = MesonAllArgs((ctypes.c_void_p * 16)(*correl16), propag_i, propag_j, gamma)
        self._launch("meson_all", kernel_name(op), a, volume)

    def meson_all_source_two_point(self, correl16, propag_i, propag_j, volume, gamma_ij):
        self._meson_all("meson_all_source", correl16, propag_i, propag_j, volume, gamma_ij)

    def meson_all_sink_two_point(self, correl16, propag_i, propag_j, volume, gamma_kl):
        self._meson_all("meson_all_sink", correl16, propag_i, propag_j, volume, gamma_kl)

    def baryon_diquark(self, diquark, propag_i, propag_j, volume, gamma_ij, gamma_kl):
        if not 0 <= gamma_ij < 16:
            return  # the reference's switch has no default action (lib/baryon/diquark.cu:38)
        a = DiquarkArgs(diquark, propag_i, propag_j, 0, gamma_kl)
        self._launch("diquark", kernel_name("diquark", gamma=gamma_ij), a, volume)

    def baryon_two_point(self, correl, propag_i, propag_j, propag_n, contract_type, volume, gamma_ij, gamma_kl,
                         gamma_mn):
        if not (0 <= contract_type < 6 and 0 <= gamma_mn < 16):
            raise ValueError("invalid contract_type or gamma_mn")
        a = BaryonArgs(correl, propag_i, propag_j, propag_n, gamma_ij, gamma_kl)
        self._launch("baryon", kernel_name("baryon", contract_type, gamma_mn), a, volume)

    def baryon_general_two_point(self, correl, propag_i, propag_j, propag_n, contract_type, volume, gamma_ij,
                                 gamma_kl, project_mn):
        if not 0 <= contract_type < 6:
            raise ValueError("invalid contract_type")
        a = BaryonGeneralArgs(correl, propag_i, propag_j, propag_n, gamma_ij, gamma_kl)
        flat = [float(v) for z in project_mn for v in (complex(z).real, complex(z).imag)]
        a.project_mn = (ctypes.c_double * 32)(*flat)
        self._launch("baryon_general", kernel_name("baryon_general", contract_type), a, volume)

    def baryon_sequential_two_point(self, propag_i, propag_j, propag_n, contract_type, sequential_type, volume,
                                    gamma_ij, gamma_kl, gamma_mn):
        if not (0 <= contract_type < 6 and 0 <= gamma_mn < 16):
            raise ValueError("invalid contract_type or gamma_mn")
        if sequential_type not in (0, 1, 2):
            return  # lib/contract.cpp:60 (default: break)
        a = BaryonSequentialArgs(propag_i, propag_j, propag_n, gamma_ij, gamma_kl)
        unit = "baryon_sequential_" + "ijn"[sequential_type]
        self._launch(unit, kernel_name("sequential", contract_type, gamma_mn, seq=sequential_type), a, volume)


# --------------------------------------------------------------- timing leg --

def time_baryon_general_sequence(latt, steps, warmup):
    """The reference's kernels on the baryon benchmark's twelve calls
    (six types x (1 +- g4)/2, C g5 = Gamma(5)) over seeded complex128
    propagators u, u, d -- the same values as the library's benchmark inputs.
    Returns ms per twelve-call sequence (CUDA events on the legacy stream)."""
    import numpy as np
    import torch

    from contract_gb300.lattice import synthetic_propagator
    ref = ReferenceGPU(0)
    v = int(np.prod(latt))
    u = synthetic_propagator(latt, 1000, 0.25, device="cuda:0")
    u2 = u.clone()
    d = synthetic_propagator(latt, 3000, 0.30, device="cuda:0")
    from .gamma import GAMMA
    e, g4 = np.eye(4), GAMMA[8]
    projs = [((e + g4) / 2).reshape(16), ((e - g4) / 2).reshape(16)]
    out = torch.empty(v, dtype=torch.complex128, device="cuda:0")

    def seq():
        for t in range(6):
            for p in projs:
                ref.baryon_general_two_point(out.data_ptr(), u.data_ptr(), u2.data_ptr(), d.data_ptr(), t, v, 5, 5, p)

    for _ in range(warmup):
        seq()
    ref.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        seq()
    e1.record()
    e1.synchronize()
    ref.synchronize()
    return e0.elapsed_time(e1) / steps


def main():
    import argparse
    import json
    import sys
    ap = argparse.ArgumentParser(description="time the reference's GPU kernels on the baryon benchmark")
    ap.add_argument("--lattice", default="24,24,24,64")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=1)
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    latt = tuple(int(x) for x in a.lattice.split(","))
    ms = time_baryon_general_sequence(latt, a.steps, a.warmup)
    print(json.dumps({"lattice": list(latt), "calls": 12, "ms_per_sequence": ms, "ms_per_call": ms / 12,
                      "kernels": "reference BaryonGeneralKernel x 6 types, sm_103a cubins, driver-API launch"}))


if __name__ == "__main__":
    main()
