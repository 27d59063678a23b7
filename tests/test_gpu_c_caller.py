"""GPU: the drop-in fpa.h API called from a compiled C program (tests/c_caller/fpa_caller.c,
gcc against include/fpa.h and libfpa_gb300.so), following the reference's own test driver
(fpa_init -> fpa_copy_array_to_device -> operation -> fpa_copy_array_to_host -> fpa_clear,
fpa_test.c:283-306), checked bit-exact against the oracle.  The second test mirrors the
reference driver's own matrix of counts and precisions (fpa_test.c:384-390: mul 10^6 at
2048 bits and 10^5 at 5120, div 10^6 at 1024 and 10^5 at 2048, sqrt 10^6 at 1024 and 10^5
at 5120, ties to even) on operands of the reference generator's pattern (tests.c:173-181,
815-830)."""
import os

import numpy as np
import pytest

import c_build
import oracle
from cubigfloat_gb300 import workloads as W
from helpers import mismatches

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return c_build.build(tmp_path_factory.mktemp("c_caller"))


def _operands(op, n, count, seed):
    rng = np.random.default_rng(seed)
    ae, al = W.reference_style_bulk(rng, count, n, signs=(op != 4))
    be, bl = W.reference_style_bulk(rng, count, n)
    return ae, al, be, bl


@pytest.mark.parametrize("op", range(5))
@pytest.mark.parametrize("n", (1, 32, 129))
def test_c_caller_every_op_and_mode(exe, tmp_path, op, n):
    ae, al, be, bl = _operands(op, n, 3000, 10 * op + n)
    for mode in range(5):
        got = c_build.run(exe, tmp_path, op, n, mode, ae, al, be, bl)
        exp = oracle.run(op, n, mode, ae, al, be, bl, threads=THREADS)
        bad = mismatches(exp[0], exp[1], got[0], got[1])
        assert bad.size == 0, (op, n, mode, bad[:5])


# (op, count, precision) of the reference driver's main() (fpa_test.c:384-390)
REFERENCE_MATRIX = [(2, 1000000, 2048), (2, 100000, 5120), (3, 1000000, 1024), (3, 100000, 2048),
                    (4, 1000000, 1024), (4, 100000, 5120)]


@pytest.mark.parametrize("case", REFERENCE_MATRIX, ids=lambda c: f"op{c[0]}_{c[1]}x{c[2]}")
def test_reference_driver_matrix(exe, tmp_path, case):
    op, count, precision = case
    n = precision // 32
    ae, al, be, bl = _operands(op, n, count, 1000 + op + n)
    got = c_build.run(exe, tmp_path, op, n, 3, ae, al, be, bl)
    exp = oracle.run(op, n, 3, ae, al, be, bl, threads=THREADS)
    bad = mismatches(exp[0], exp[1], got[0], got[1])
    assert bad.size == 0, (case, bad.size, bad[:5])
