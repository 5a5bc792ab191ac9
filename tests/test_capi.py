"""The C ABI library builds, loads and exports every entry point the header
declares; host-only entry points run without a GPU."""
import ctypes
import os
import re
import shutil

import pytest

import cases
from dadi_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "dadi_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dgb_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    declared = header_functions()
    assert declared, "no declarations parsed"
    assert sorted(_lib.EXPORTS) == declared
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(lib):
    assert lib.dgb_abi_version() == 1
    assert lib.dgb_status_string(0) == b"ok"
    assert b"workspace" in lib.dgb_status_string(_lib.DGB_ERR_WORKSPACE)


def test_struct_layout():
    assert ctypes.sizeof(_lib.PForm) == 32
    assert ctypes.sizeof(_lib.Settings) == 40
    assert ctypes.sizeof(_lib.Inst2D) == 16 + 9 * 32 + 8


def _c_layout(tmp_path, struct, fields):
    """sizeof(struct) and offsetof(struct, f) for each field, from the header
    compiled by the host C compiler."""
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dadi_gb300.h"',
             'int main(void) {', '    printf("%%zu\\n", sizeof(%s));' % struct]
    lines += ['    printf("%%zu\\n", offsetof(%s, %s));' % (struct, f) for f in fields]
    lines += ['    return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    return int(out[0]), [int(v) for v in out[1:]]


@pytest.mark.parametrize("struct,dtype,cfields", [
    ("dgb_extrap_item", "EX_ITEM", ["fs", "x", "out", "data", "ll", "ll_multinom", "scale",
                                    "ngrids", "size", "mask_corners", "pad_"]),
    ("dgb_fs_item2d", "FS_ITEM", ["phi", "xx", "d1x", "d2x", "d1y", "d2y", "out", "L", "n1",
                                  "n2", "pad_"]),
    ("dgb_item2d", "ITEM2D_DTYPE", ["L", "masks", "xx_off", "out_off", "sched"]),
])
def test_record_dtypes_match_header(tmp_path, struct, dtype, cfields):
    """The numpy record types the host fills match the C structs byte for
    byte (size and every field offset)."""
    if shutil.which("gcc") is None:
        pytest.skip("no host C compiler")
    from dadi_gb300 import batch, epilogue
    dt = getattr(epilogue, dtype, None) or getattr(batch, dtype)
    size, offs = _c_layout(tmp_path, struct, cfields)
    assert dt.itemsize == size
    assert [dt.fields[n][1] for n in dt.names] == offs


@pytest.mark.parametrize("struct,ctype", [("dgb_settings", "Settings"), ("dgb_pform", "PForm"),
                                          ("dgb_instnd", "InstND"), ("dgb_itemnd", "ItemND"),
                                          ("dgb_seednd", "SeedND"),
                                          ("dgb_itemnd_adj", "ItemNDAdj")])
def test_ctypes_structs_match_header(tmp_path, struct, ctype):
    """The ctypes structures passed by reference match the C structs (size
    and every field offset)."""
    if shutil.which("gcc") is None:
        pytest.skip("no host C compiler")
    cls = getattr(_lib, ctype)
    names = [f[0] for f in cls._fields_]
    size, offs = _c_layout(tmp_path, struct, names)
    assert ctypes.sizeof(cls) == size
    assert [getattr(cls, n).offset for n in names] == offs


def test_inst2d_dtype_matches_header(tmp_path):
    """batch.INST_DTYPE (the dgb_inst2d records the host fills) matches the C
    struct."""
    if shutil.which("gcc") is None:
        pytest.skip("no host C compiler")
    from dadi_gb300 import batch
    cf = ["T", "initial_t", "nu", "m12", "m21", "gamma", "h", "theta0", "frozen_mask",
          "nomut_mask"]
    size, offs = _c_layout(tmp_path, "dgb_inst2d", cf)
    dt = batch.INST_DTYPE
    assert dt.itemsize == size
    assert [dt.fields[n][1] for n in dt.names] == offs


def test_count_steps_matches_python_schedule(lib):
    from dadi_gb300 import batch
    draws = cases.im_draws(16)
    insts = batch.im_instances(draws)
    steps = batch.count_steps(insts)
    for p, n in zip(draws, steps):
        s, nu1, nu2, T, m12, m21 = p
        t, k = 0.0, 0
        a = lambda t: s * (nu1 / s) ** (t / T)
        b = lambda t: (1 - s) * (nu2 / (1 - s)) ** (t / T)
        while t < T:
            dt = min(1e-3 / max(0.25 / a(t), m12), 1e-3 / max(0.25 / b(t), m21))
            t = t + min(dt, T - t)
            k += 1
        assert abs(k - n) <= 1
