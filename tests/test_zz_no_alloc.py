"""GPU: fpa_batch_run_noalloc, the batched run that allocates nothing.

Some callers must not allocate GPU memory where they compute: a serving loop whose latency
budget cannot absorb cudaMalloc / cudaFree (which may synchronize the device), or a host
application that hands all device memory to its own allocator up front.  They call this
entry point with device buffers they already own, and its working memory is a fixed device
array inside the library.  This test calls it through the C ABI twice in a row, on two
different mixed batches, and requires each result to equal what the allocating entry point
(fpa_batch_create + fpa_batch_run) produces for the same inputs, bit for bit, with the
error word clear after each call.  It also checks that a batch larger than the fixed array
is rejected.  The file is collected last so that a run stopping at the first failure has
run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import cubigfloat_gb300 as fpa
from cubigfloat_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FPA_NOALLOC_MAX_OPS = 4096


def _lib():
    L = fpa.lib()
    vp = ctypes.c_void_p
    L.fpa_batch_run_noalloc.restype = ctypes.c_int
    L.fpa_batch_run_noalloc.argtypes = [vp, ctypes.c_uint32, vp, vp, vp, vp, vp, vp, vp]
    L.fpa_batch_noalloc_errors.restype = ctypes.c_uint32
    L.fpa_batch_noalloc_errors.argtypes = [vp]
    return L


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _same_values(descs, exp, got):
    ee, el = exp
    ge, gl = got
    if not np.array_equal(ee, ge):
        return False
    for i in np.nonzero(ee > 8)[0]:
        o, n = int(descs["r_off"][i]), int(descs["limbs"][i])
        if not np.array_equal(el[o:o + n], gl[o:o + n]):
            return False
    return True


def test_noalloc_matches_allocating_batch_on_two_calls():
    L = _lib()
    for seed in (31, 32):
        descs, ae, al, be, bl, total = W.mixed(seed, 3000, min_bits=32, max_bits=16384)
        descs["mode"] = np.random.default_rng(seed).integers(0, 5, size=len(descs))
        d_ae, d_al, d_be, d_bl = _dev(ae), _dev(al), _dev(be), _dev(bl)
        ins = (d_ae.data_ptr(), d_al.data_ptr(), d_be.data_ptr(), d_bl.data_ptr())
        # the allocating entry point
        ref_e = torch.zeros(len(descs), dtype=torch.int32, device="cuda")
        ref_l = torch.zeros(total, dtype=torch.int32, device="cuda")
        b = fpa.Batch(descs)
        assert b.run(ref_e.data_ptr(), ref_l.data_ptr(), *ins) == fpa.fpa_success
        torch.cuda.synchronize()
        b.destroy()
        # the entry point that allocates nothing
        got_e = torch.zeros(len(descs), dtype=torch.int32, device="cuda")
        got_l = torch.zeros(total, dtype=torch.int32, device="cuda")
        d = np.ascontiguousarray(descs)
        rc = L.fpa_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), len(descs), got_e.data_ptr(),
                                     got_l.data_ptr(), *ins, None)
        assert rc == fpa.fpa_success
        torch.cuda.synchronize()
        assert L.fpa_batch_noalloc_errors(None) == 0
        assert _same_values(descs, (_host(ref_e), _host(ref_l)), (_host(got_e), _host(got_l)))


def test_noalloc_rejects_more_than_its_maximum():
    L = _lib()
    descs, *_ = W.mixed(5, FPA_NOALLOC_MAX_OPS + 1, min_bits=256, max_bits=512)
    d = np.ascontiguousarray(descs)
    rc = L.fpa_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), len(descs), None, None, None, None, None,
                                 None, None)
    assert rc == fpa.fpa_invalid_counts
    # the rejected call touched nothing: the error word of the last batch is still readable and clear
    assert L.fpa_batch_noalloc_errors(None) == 0
