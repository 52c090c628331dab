"""The C-ABI library without a GPU: it loads, exports every declared symbol,
carries the reference's enum values and gamma tables, and rejects invalid
calls the way the reference does."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib():
    from contract_gb300 import build
    build.build()
    from contract_gb300 import _lib
    return _lib.lib()


def declared_functions():
    names = set()
    for h in ("contract.h", "contract_gb300.h"):
        src = open(os.path.join(INCLUDE, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:void|int|size_t|const char|void \*)\s*\*?\s*(\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert {"init", "meson_two_point", "meson_all_source_two_point", "meson_all_sink_two_point", "baryon_diquark",
            "baryon_two_point", "baryon_general_two_point", "baryon_sequential_two_point"} <= names
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert names <= exported
    # nothing but the C ABI leaks out of the library
    assert exported == names, sorted(exported - names)


def test_python_signatures_cover_the_headers():
    from contract_gb300 import _lib
    assert declared_functions() == set(_lib.SIGNATURES)


def test_enum_values_match_contract_enum():
    from contract_gb300.pycontract import BaryonContractType as T, BaryonSequentialType as S
    src = open(os.path.join(INCLUDE, "contract_enum.h")).read()
    body = src[src.index("typedef enum {"):src.index("} BaryonContractType;")]
    values = {}
    nxt = 0
    for name, val in re.findall(r"(\w+)\s*(?:=\s*(\w+))?\s*,", body):
        values[name] = values[val] if val else nxt
        nxt = values[name] + 1
    assert values["IM_JL_NK"] == 5 and values["IN_JK_ML"] == 4 and values["AF_BE_CD"] == 5
    for name, v in values.items():
        assert T[name] == v, name
    assert (S.SEQUENTIAL_I, S.SEQUENTIAL_J, S.SEQUENTIAL_N) == (0, 1, 2)


def test_enum_header_include_twice(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "contract_enum.h"\n#include "contract_enum.h"\n#include "contract_gb300.h"\n'
                   "int main(void) { return IN_JL_MK == 5 ? 0 : 1; }\n")
    r = subprocess.run(["gcc", "-std=c11", "-I", INCLUDE, str(src), "-o", str(tmp_path / "t")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(tmp_path / "t")]).returncode == 0


def test_gamma_table_bit_exact(lib, golden):
    perm = (ctypes.c_int * 64)()
    phase = (ctypes.c_int * 64)()
    lib.contract_gamma_table(perm, phase)
    perm = np.array(perm[:]).reshape(16, 4)
    val = 1j ** np.array(phase[:]).reshape(16, 4)
    assert np.array_equal(perm, golden["gamma_index"])
    assert np.array_equal(np.round(val, 15), golden["gamma_data"])


def test_decompose_gamma():
    from contract_gb300 import pycontract as pc
    g = pc.gamma_matrices()
    c_g5 = g[2] @ g[8] @ g[15]  # C g5 = g2 g4 g5
    n, c = pc.decompose_gamma(c_g5)
    assert n == 5 and c == 1
    n, c = pc.decompose_gamma(-1j * g[13])
    assert n == 13 and abs(c + 1j) < 1e-15
    with pytest.raises(ValueError):
        pc.decompose_gamma((np.eye(4) + g[8]) / 2)


def test_projector_rank(lib):
    """Projectors that the triangle kernels factor as sum_r x_r y_r^T (rank <= 2,
    elimination with an exactly zero remainder) and those they apply as N' = W N."""
    from contract_gb300 import pycontract as pc
    g = pc.gamma_matrices()
    e = np.eye(4)

    def rank(w):
        buf = np.ascontiguousarray(np.asarray(w, np.complex128).reshape(16))
        return lib.contract_projector_rank(buf.ctypes.data)

    assert rank((e + g[8]) / 2) == 2 and rank((e - g[8]) / 2) == 2
    assert rank((e + g[8]) @ (e - 1j * g[3]) / 4) == 1
    assert rank((e - g[8]) @ (e + 1j * g[3]) / 4) == 1
    x, y = np.array([0.5, 0, -1j, 0.25]), np.array([1, 2j, 0, -0.5])
    assert rank(np.outer(x, y)) == 1
    assert rank(e) == 0 and rank(g[5]) == 0 and rank(np.zeros((4, 4))) == 0
    rng = np.random.default_rng(3)
    assert rank(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))) == 0
    assert lib.contract_projector_rank(None) == 0
    nan = (e + g[8]) / 2
    nan[3, 0] = np.nan  # a zero entry of the rank-2 projector: the factors would drop it
    assert rank(nan) == 0


def _run(code):
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT,
                          env=dict(os.environ, PYTHONPATH=ROOT))


def test_invalid_selector_exits_like_reference():
    # baryon.cu:61-63 of the reference: "Error: Invalid contract_type value %d" then exit(-1).
    r = _run("from contract_gb300 import _lib; L=_lib.lib(); "
             "L.baryon_two_point(None,None,None,None,7,0,5,5,8); print('survived')")
    assert r.returncode == 255 and "survived" not in r.stdout
    assert "Invalid contract_type value 7" in r.stderr
    r = _run("from contract_gb300 import _lib; L=_lib.lib(); "
             "L.baryon_two_point(None,None,None,None,1,0,5,5,16); print('survived')")
    assert r.returncode == 255 and "Invalid gamma_mn value 16" in r.stderr


def test_silent_noops_like_reference():
    # diquark.cu:40 and contract.cpp:60 of the reference ignore these selectors.
    r = _run("from contract_gb300 import _lib; L=_lib.lib(); "
             "L.baryon_diquark(None,None,None,0,17,5); "
             "L.baryon_sequential_two_point(None,None,None,0,3,0,5,5,8); print('survived')")
    assert r.returncode == 0 and "survived" in r.stdout


def test_record_mode_reports_errors(lib):
    lib.contract_set_error_mode(1)
    try:
        lib.contract_clear_error()
        lib.baryon_two_point(None, None, None, None, 9, 0, 5, 5, 8)
        assert lib.contract_last_error() == 1
        assert b"Invalid contract_type value 9" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lib.meson_two_point(None, None, None, 16, 5, 5)
        assert lib.contract_last_error() == 1 and b"NULL" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lat = (ctypes.c_int * 4)(3, 2, 2, 4)  # odd Lx
        lib.contract_meson(None, None, None, 0, 5, 5, 0, lat)
        assert lib.contract_last_error() == 1 and b"Lx even" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lib.contract_baryon_all_types(None, None, None, None, 0, 5, 5, 3, None, 0, None)
        assert lib.contract_last_error() == 1
        lib.contract_clear_error()
    finally:
        lib.contract_set_error_mode(0)


def test_pycontract_raises_on_invalid(lib):
    from contract_gb300 import pycontract as pc
    with pytest.raises(pc.ContractError, match="Invalid gamma_kl"):
        pc.meson_two_point(0, 0, 0, 0, 3, 99)
    lib.contract_set_error_mode(0)


def test_workspace_bytes(lib):
    lat = (ctypes.c_int * 4)(24, 24, 24, 64)
    b = lib.contract_workspace_bytes(lat, 12)
    assert b >= 884736 // 16 * 12 * 16  # one partial per (at least) 16-site tile


def test_misaligned_pointer_rejected(lib):
    lib.contract_set_error_mode(1)
    try:
        lib.contract_clear_error()
        lib.meson_two_point(0x1008, 0x2000, 0x3000, 4, 5, 5)
        assert lib.contract_last_error() == 1 and b"16-byte aligned" in lib.contract_last_error_message()
        lib.contract_clear_error()
    finally:
        lib.contract_set_error_mode(0)


def test_batch_validation_without_gpu(lib):
    lib.contract_set_error_mode(1)
    try:
        lib.contract_clear_error()
        lib.contract_baryon_all_types_batch(None, 200, 5, 5, 2, None, 1)
        assert lib.contract_last_error() == 1 and b"nitems" in lib.contract_last_error_message()
        lib.contract_clear_error()
    finally:
        lib.contract_set_error_mode(0)


def test_quda_conversion_argument_checks(lib):
    lib.contract_set_error_mode(1)
    try:
        lat = (ctypes.c_int * 4)(4, 2, 2, 4)
        fields = (ctypes.c_void_p * 12)(*[0x100000 * (k + 1) for k in range(12)])
        lib.contract_clear_error()
        lib.contract_convert_from_quda(0x10000000, fields, lat, 15, 0)  # stride below V/2 = 16
        assert lib.contract_last_error() == 1 and b"stride" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lib.contract_convert_to_quda(None, 0x10000000, lat, 0, 0)
        assert lib.contract_last_error() == 1 and b"fields is NULL" in lib.contract_last_error_message()
        lib.contract_clear_error()
        fields[3] = fields[2] + 256  # overlaps field 2 (each field is 2 x 12 x 16 x 16 bytes)
        lib.contract_convert_from_quda(0x10000000, fields, lat, 0, 0)
        assert lib.contract_last_error() == 1 and b"overlap" in lib.contract_last_error_message()
        lib.contract_clear_error()
        fields[3] = 0x100008  # misaligned
        lib.contract_convert_to_quda(fields, 0x10000000, lat, 0, 1)
        assert lib.contract_last_error() == 1 and b"16-byte aligned" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lib.contract_rotate_spin_basis(0x10000000, 16, None, 0)
        assert lib.contract_last_error() == 1 and b"rotation is NULL" in lib.contract_last_error_message()
        lib.contract_clear_error()
    finally:
        lib.contract_set_error_mode(0)


class _MesonItem(ctypes.Structure):
    _fields_ = [("propag_i", ctypes.c_void_p), ("propag_j", ctypes.c_void_p), ("correl", ctypes.c_void_p),
                ("lattice", ctypes.c_int * 4)]


def test_mixed_batch_validation_without_gpu(lib):
    """The batched meson / mixed calls reject bad arguments on the host, before any
    CUDA call (the pointers here are never dereferenced)."""
    moms = np.array([[2, 0, 0], [-2, 0, 0], [0, 0, 0]], dtype=np.int32)
    mp = moms.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    items = (_MesonItem * 2)()
    for k, latt in enumerate(((4, 4, 4, 4), (6, 4, 4, 4))):
        items[k].propag_i = items[k].propag_j = 0x100000 * (k + 1)
        items[k].correl = 0x1000000 * (k + 1)
        items[k].lattice = (ctypes.c_int * 4)(*latt)
    lib.contract_set_error_mode(1)
    try:
        lib.contract_clear_error()
        lib.contract_meson_all_gamma_momentum_batch(items, 2, mp, 3, 0)
        assert lib.contract_last_error() == 1 and b"CONTRACT_C64" in lib.contract_last_error_message()
        lib.contract_clear_error()
        lib.contract_batch_mixed(None, 0, 5, 5, 2, None, items, 200, mp, 3, 1)
        assert lib.contract_last_error() == 1 and b"item counts" in lib.contract_last_error_message()
        lib.contract_clear_error()
        # n = +-2 form one group on L = 4 and two on L = 6
        lib.contract_meson_all_gamma_momentum_batch(items, 2, mp, 3, 1)
        assert lib.contract_last_error() == 1 and b"another structure" in lib.contract_last_error_message()
        lib.contract_clear_error()
        items[1].lattice = (ctypes.c_int * 4)(66, 4, 4, 4)
        lib.contract_meson_all_gamma_momentum_batch(items, 2, mp, 3, 1)
        assert lib.contract_last_error() == 1 and b"up to 64" in lib.contract_last_error_message()
        lib.contract_clear_error()
        items[1].propag_i = 0x100008  # misaligned
        items[1].lattice = (ctypes.c_int * 4)(4, 4, 4, 4)
        lib.contract_meson_all_gamma_momentum_batch(items, 2, mp, 3, 1)
        assert lib.contract_last_error() == 1 and b"16-byte aligned" in lib.contract_last_error_message()
        lib.contract_clear_error()
    finally:
        lib.contract_set_error_mode(0)
