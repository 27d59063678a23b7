"""GPU parity of the non-arithmetic fpa.h entry points through the C ABI, bit-exact against
the oracle (itself pinned to MPFR by tests/test_conversions_oracle.py):
fpa_set_ui / fpa_set_si / fpa_set_float / fpa_set_double, fpa_set (precision change in all
five modes), fpa_sgn, fpa_cmp, fpa_neg, at 1, 2, 32, 128 and 512 limbs, on edge values
(0, 1, INT64_MIN, UINT64_MAX, +-0.0, subnormals, +-inf, NaNs, ties at 32 bits) and every
special class; and the stream-ordered forms (fpa_copy_array_to_device_async,
fpa_copy_array_to_host_async, fpa_op_async on a non-default stream) against the
synchronous fpa.h calls."""
import ctypes

import numpy as np
import pytest

import conv_cases as CC
import cubigfloat_gb300 as fpa
import oracle
from helpers import mismatches

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SETTERS = {"ui": (fpa.fpa_set_ui, CC.uint_values), "si": (fpa.fpa_set_si, CC.int_values),
           "float": (fpa.fpa_set_float, lambda s: CC.float_bits(s).view(np.float32)),
           "double": (fpa.fpa_set_double, lambda s: CC.double_bits(s).view(np.float64))}


@pytest.fixture(scope="module", autouse=True)
def device_errors_clear():
    fpa.device_errors()
    yield
    assert fpa.device_errors() == 0


def _array(e, l, n):
    A = fpa.FpaArray(len(e), 32 * n)
    assert A.to_device(e, l) == fpa.fpa_success
    return A


@pytest.mark.parametrize("n", CC.SIZES)
@pytest.mark.parametrize("kind", list(SETTERS))
def test_set_values(kind, n):
    fn, gen = SETTERS[kind]
    v = gen(100 + n)
    R = fpa.FpaArray(len(v), 32 * n)
    assert fn(R, v) == fpa.fpa_success
    got = R.to_host()
    exp = oracle.set_values(kind, n, v)
    bad = mismatches(exp[0], exp[1], got[0], got[1])
    assert bad.size == 0, (kind, n, v[bad[:5]], exp[0][bad[:5]], got[0][bad[:5]])


@pytest.mark.parametrize("count", (1, 2, 255, 257))
def test_set_counts(count):
    """Ragged counts: every element written, none past the end (fpa_warp_set.h's per-warp
    bound is `warp > count`, one past the end; here the bound is exact)."""
    v = CC.int_values(7, count=max(count, 24))[:count]
    R = fpa.FpaArray(count + 1, 64)
    guard = np.full(count + 1, 0xDEADBEEF, np.uint32)
    assert R.to_device(guard, np.zeros((count + 1, 2), np.uint32)) == fpa.fpa_success
    R.s.count = count                                  # write only the first `count`
    assert fpa.fpa_set_si(R, v) == fpa.fpa_success
    R.s.count = count + 1
    e, l = R.to_host()
    oe, ol = oracle.set_values("si", 2, v)
    assert mismatches(oe, ol, e[:count], l[:count]).size == 0
    assert e[count] == 0xDEADBEEF


@pytest.mark.parametrize("pair", CC.PREC_PAIRS, ids=str)
def test_set_prec(pair):
    nx, nr = pair
    xe, xl = CC.prec_sources(200 + nx + nr, nx, nr)
    xe = np.concatenate([xe, CC.CLASSES])
    xl = np.concatenate([xl, np.zeros((CC.CLASSES.size, nx), np.uint32)])
    X = _array(xe, xl, nx)
    R = fpa.FpaArray(len(xe), 32 * nr)
    for mode in range(5):
        assert fpa.fpa_set(R, X, mode) == fpa.fpa_success
        got = R.to_host()
        exp = oracle.set_prec(nr, nx, mode, xe, xl)
        bad = mismatches(exp[0], exp[1], got[0], got[1])
        assert bad.size == 0, (pair, mode, bad[:5])


def test_set_prec_overflow():
    from cubigfloat_gb300 import workloads as W
    xe = np.array([W.exp_word(0x7FFFFFFF - W.BIAS, 0), W.exp_word(0x7FFFFFFF - W.BIAS, 1)], np.uint32)
    xl = np.full((2, 2), 0xFFFFFFFF, np.uint32)
    X = _array(xe, xl, 2)
    R = fpa.FpaArray(2, 32)
    for mode in range(5):
        assert fpa.fpa_set(R, X, mode) == fpa.fpa_success
        e, _ = R.to_host()
        assert list(e) == list(oracle.set_prec(1, 2, mode, xe, xl)[0])


@pytest.mark.parametrize("n", CC.SIZES)
def test_sgn_cmp_neg(n):
    xe, xl = CC.numbers(300 + n, n)
    X = _array(xe, xl, n)
    r = torch.full((len(xe),), 99, dtype=torch.int32, device="cuda")
    assert fpa.fpa_sgn(r.data_ptr(), X) == fpa.fpa_success
    assert (r.cpu().numpy() == oracle.sgn(xe)).all()
    R = fpa.FpaArray(len(xe), 32 * n)
    assert fpa.fpa_neg(R, X) == fpa.fpa_success
    got = R.to_host()
    exp = oracle.neg(n, xe, xl)
    assert mismatches(exp[0], exp[1], got[0], got[1]).size == 0
    ae, al, be, bl = CC.compare_pairs(400 + n, n)
    A, B = _array(ae, al, n), _array(be, bl, n)
    r = torch.full((len(ae),), 99, dtype=torch.int32, device="cuda")
    assert fpa.fpa_cmp(r.data_ptr(), A, B) == fpa.fpa_success
    exp = oracle.cmp(n, ae, al, be, bl)
    got = r.cpu().numpy()
    assert (got == exp).all(), np.nonzero(got != exp)[0][:5]


def test_argument_checks():
    """Counts first, then precisions (fpa_dispatch.h:128-173)."""
    A, B, C = fpa.FpaArray(4, 64), fpa.FpaArray(5, 64), fpa.FpaArray(4, 96)
    r = torch.zeros(8, dtype=torch.int32, device="cuda")
    assert fpa.fpa_cmp(r.data_ptr(), A, B) == fpa.fpa_invalid_counts
    assert fpa.fpa_cmp(r.data_ptr(), A, C) == fpa.fpa_invalid_precisions
    assert fpa.fpa_neg(B, A) == fpa.fpa_invalid_counts
    assert fpa.fpa_neg(C, A) == fpa.fpa_invalid_precisions
    assert fpa.fpa_set(B, A, 3) == fpa.fpa_invalid_counts
    assert fpa.fpa_set(C, A, 3) == fpa.fpa_success       # a precision change is the point of fpa_set


@pytest.mark.parametrize("op", ("mul", "div", "sqrt", "add"))
def test_async_forms_match_sync(op):
    """Operands in pinned host memory copied with fpa_copy_array_to_device_async, the
    operation by fpa_op_async and the result by fpa_copy_array_to_host_async, all on one
    non-default stream, give the same numbers as the synchronous fpa.h calls."""
    from cubigfloat_gb300 import workloads as W
    n, count = 128, 1000
    (ae, al), (be, bl) = W.workload_4096(op if op != "add" else "mul", 77, count=count, n=n)
    code = fpa.OPS[op]
    A, B, R = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    L = fpa.lib()
    vp = ctypes.c_void_p
    pin = [torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).pin_memory() for x in (ae, al, be, bl)]
    out = [torch.zeros(count, dtype=torch.int32).pin_memory(), torch.zeros(count * n, dtype=torch.int32).pin_memory()]
    s = torch.cuda.Stream()
    assert L.fpa_copy_array_to_device_async(A.ref, vp(pin[0].data_ptr()), vp(pin[1].data_ptr()),
                                            vp(s.cuda_stream)) == 0
    assert L.fpa_copy_array_to_device_async(B.ref, vp(pin[2].data_ptr()), vp(pin[3].data_ptr()),
                                            vp(s.cuda_stream)) == 0
    assert L.fpa_op_async(code, R.ref, A.ref, B.ref, 3, vp(s.cuda_stream)) == 0
    assert L.fpa_copy_array_to_host_async(R.ref, vp(out[0].data_ptr()), vp(out[1].data_ptr()),
                                          vp(s.cuda_stream)) == 0
    s.synchronize()
    got_e, got_l = out[0].numpy().view(np.uint32), out[1].numpy().view(np.uint32).reshape(count, n)
    # synchronous fpa.h path
    A2, B2, R2 = fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n), fpa.FpaArray(count, 32 * n)
    assert A2.to_device(ae, al) == 0 and B2.to_device(be, bl) == 0
    fn = {"mul": fpa.fpa_mul, "div": fpa.fpa_div, "add": fpa.fpa_add}.get(op)
    assert (fn(R2, A2, B2, 3) if fn else fpa.fpa_sqrt(R2, A2, 3)) == 0
    exp_e, exp_l = R2.to_host()
    assert mismatches(exp_e, exp_l, got_e, got_l).size == 0
    oe, ol = oracle.run(code, n, 3, ae, al, be, bl, threads=8)
    assert mismatches(oe, ol, got_e, got_l).size == 0
