"""CPU: the C-ABI library loads and exports every function declared in include/*.h, and the
host-side argument checks behave like the reference's (fpa_dispatch.h:179-182)."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import cubigfloat_gb300 as fpa
from cubigfloat_gb300 import build as fpa_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*\b([a-z_][a-z0-9_]*)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    fpa_build.build()
    return fpa.lib()


def test_header_declares_reference_api():
    names = declared_functions()
    ref16 = ["fpa_init", "fpa_clear", "fpa_copy_array_to_device", "fpa_copy_array_to_host", "fpa_set_ui",
             "fpa_set_si", "fpa_set_float", "fpa_set_double", "fpa_set", "fpa_sgn", "fpa_cmp", "fpa_neg",
             "fpa_add", "fpa_sub", "fpa_mul", "fpa_div", "fpa_sqrt"]
    for n in ref16:
        assert n in names


def test_library_exports_all_declared(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", fpa.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        getattr(lib, n)


def test_enum_and_struct_layout():
    assert (fpa.fpa_round_truncate, fpa.fpa_round_ties_away_from_zero) == (0, 4)
    assert (fpa.fpa_success, fpa.fpa_math_error, fpa.fpa_invalid_precisions, fpa.fpa_invalid_counts) == (0, 1, 2, 3)
    assert ctypes.sizeof(fpa.fpa_s) == 24
    assert fpa.fpa_s.gpu_exps.offset == 8 and fpa.fpa_s.gpu_limbs.offset == 16


def test_argument_checks_without_device(lib):
    P = ctypes.byref
    a, b, r = fpa.fpa_s(5, 1024, None, None), fpa.fpa_s(6, 1024, None, None), fpa.fpa_s(5, 1024, None, None)
    assert lib.fpa_add(P(r), P(a), P(b), 3) == fpa.fpa_invalid_counts
    b.count = 5; b.precision = 2048
    assert lib.fpa_mul(P(r), P(a), P(b), 3) == fpa.fpa_invalid_precisions
    x = fpa.fpa_s()
    assert lib.fpa_init(P(x), 10, 1000) == fpa.fpa_invalid_precisions
    assert lib.fpa_init(P(x), 10, 16416) == fpa.fpa_invalid_precisions
    assert lib.fpa_gb300_num_configs() == 20
    c128 = lib.fpa_gb300_get_config(128)       # the autotuned table's choice, or the default (4)
    assert 0 <= c128 < 20 and np.prod(fpa.configs()[c128]) >= 128
    assert lib.fpa_gb300_get_config(513) == -1


def test_configs_cover_all_precisions(lib):
    cfgs = fpa.configs()
    for n in range(1, 513):
        c = fpa.get_config(n)
        g, k, r = cfgs[c]
        assert g * k * r >= max(n, 4)


def test_c_caller_compiles_and_links(lib, tmp_path):
    """A plain C program written against include/fpa.h (the reference caller's flow,
    fpa_test.c:283-306) compiles with gcc and links against libfpa_gb300.so."""
    import c_build
    exe = c_build.build(tmp_path)
    assert os.path.exists(exe)
