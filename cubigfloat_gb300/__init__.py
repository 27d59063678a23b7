"""Python mirror of the fpa.h C API, bound to libfpa_gb300.so with ctypes.

The names, argument order and result codes follow the reference's public header
(fpa.h:8-63): `FpaArray` plays the role of `fpa_t` (fpa_init / fpa_clear /
fpa_copy_array_to_device / fpa_copy_array_to_host), and `fpa_add`, `fpa_mul`, ... take
(r, a, b, mode) and return an `fpa_result` code.  There is no CPU fallback: importing
this module fails loudly if the CUDA library has not been built.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfpa_gb300.so")

# fpa.h:8-10
fpa_round_truncate, fpa_round_up, fpa_round_down, fpa_round_ties_to_even, fpa_round_ties_away_from_zero = range(5)
MODES = (fpa_round_truncate, fpa_round_up, fpa_round_down, fpa_round_ties_to_even, fpa_round_ties_away_from_zero)
# fpa.h:12-17 (+ fpa_device_error)
fpa_success, fpa_math_error, fpa_invalid_precisions, fpa_invalid_counts, fpa_device_error = range(5)
# fpa_gb300.h
OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_SQRT = range(5)
OPS = {"add": OP_ADD, "sub": OP_SUB, "mul": OP_MUL, "div": OP_DIV, "sqrt": OP_SQRT}

BIAS = 0x3FFFFFF3


class fpa_s(ctypes.Structure):
    """fpa.h:19-26"""
    _fields_ = [("count", ctypes.c_uint32), ("precision", ctypes.c_uint32),
                ("gpu_exps", ctypes.c_void_p), ("gpu_limbs", ctypes.c_void_p)]


class FpaError(RuntimeError):
    pass


class ServerJobOpts(ctypes.Structure):
    """fpa_gb300.h: fpa_server_job_opts"""
    _fields_ = [("a_from", ctypes.c_int64), ("b_from", ctypes.c_int64), ("keep", ctypes.c_uint32),
                ("copy_out", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    """fpa_gb300.h: fpa_server_config"""
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_batch_ops", ctypes.c_uint32), ("batching", ctypes.c_int)]


_lib = None


def lib():
    """Load libfpa_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FpaError(f"CUDA library missing: {LIB_PATH} (run cubigfloat_gb300.build.build())")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(fpa_s)
    u32, u64, i32, vp = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p
    sig = {
        "fpa_init": (i32, [P, u32, u32]),
        "fpa_clear": (i32, [P]),
        "fpa_copy_array_to_device": (i32, [P, vp, vp]),
        "fpa_copy_array_to_host": (i32, [P, vp, vp]),
        "fpa_set_ui": (i32, [P, vp]),
        "fpa_set_si": (i32, [P, vp]),
        "fpa_set_float": (i32, [P, vp]),
        "fpa_set_double": (i32, [P, vp]),
        "fpa_set": (i32, [P, P, i32]),
        "fpa_sgn": (i32, [vp, P]),
        "fpa_cmp": (i32, [vp, P, P]),
        "fpa_neg": (i32, [P, P]),
        "fpa_add": (i32, [P, P, P, i32]),
        "fpa_sub": (i32, [P, P, P, i32]),
        "fpa_mul": (i32, [P, P, P, i32]),
        "fpa_div": (i32, [P, P, P, i32]),
        "fpa_sqrt": (i32, [P, P, i32]),
        "fpa_gb300_fma": (i32, [P, P, P, P, i32]),
        "fpa_gb300_elementwise": (i32, [i32, u32, u64, i32, vp, vp, vp, vp, vp, vp, vp]),
        "fpa_op_async": (i32, [i32, P, P, P, i32, vp]),
        "fpa_copy_array_to_device_async": (i32, [P, vp, vp, vp]),
        "fpa_copy_array_to_host_async": (i32, [P, vp, vp, vp]),
        "fpa_gb300_device_errors": (u32, []),
        "fpa_gb300_num_configs": (i32, []),
        "fpa_gb300_config_shape": (i32, [i32, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u32)]),
        "fpa_gb300_set_config": (i32, [u32, i32]),
        "fpa_gb300_get_config": (i32, [u32]),
        "fpa_gb300_version": (ctypes.c_char_p, []),
        "fpa_gb300_measure_imad_peak": (i32, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
        "fpa_gb300_measure_product_peak": (i32, [ctypes.POINTER(ctypes.c_double)]),
        "fpa_batch_create": (i32, [ctypes.POINTER(vp), vp, u64]),
        "fpa_batch_run": (i32, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "fpa_batch_capture": (i32, [vp, vp, vp, vp, vp, vp, vp]),
        "fpa_batch_graph_launch": (i32, [vp, vp]),
        "fpa_batch_info": (i32, [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]),
        "fpa_batch_destroy": (i32, [vp]),
        "fpa_gb300_set_op_config": (i32, [i32, u32, i32]),
        "fpa_gb300_get_op_config": (i32, [i32, u32]),
        "fpa_gb300_set_karatsuba_limbs": (i32, [u32]),
        "fpa_gb300_get_karatsuba_limbs": (u32, []),
        "fpa_server_create": (i32, [ctypes.POINTER(vp), ctypes.POINTER(ServerConfig)]),
        "fpa_server_submit": (ctypes.c_int64, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp]),
        "fpa_server_wait": (i32, [vp, ctypes.c_int64, ctypes.c_int64]),
        "fpa_server_job_times": (i32, [vp, ctypes.c_int64, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                       ctypes.POINTER(u64)]),
        "fpa_server_release": (i32, [vp, ctypes.c_int64]),
        "fpa_server_stats": (i32, [vp, ctypes.POINTER(u64)]),
        "fpa_server_create_resident": (i32, [ctypes.POINTER(vp), ctypes.POINTER(ServerConfig), u64]),
        "fpa_server_submit_ex": (ctypes.c_int64, [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp,
                                                  ctypes.POINTER(ServerJobOpts)]),
        "fpa_server_read": (i32, [vp, ctypes.c_int64, vp, vp]),
        "fpa_server_costs": (i32, [vp, ctypes.POINTER(u64)]),
        "fpa_server_destroy": (i32, [vp]),
        "fpa_gb300_dot": (i32, [u32, u64, u32, i32, vp, vp, vp, vp, vp, vp, vp]),
        "fpa_gb300_newton_sqrt": (i32, [u32, u64, u32, i32, vp, vp, vp, vp, vp]),
        "fpa_gb300_autotune": (i32, [i32, u32, u32, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_double)]),
        "fpa_gb300_load_tuning": (i32, [ctypes.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class FpaArray:
    """An fpa_t: `count` numbers of `precision` bits in device memory."""

    def __init__(self, count, precision):
        self.s = fpa_s()
        rc = lib().fpa_init(ctypes.byref(self.s), count, precision)
        if rc != fpa_success:
            raise FpaError(f"fpa_init({count}, {precision}) -> {rc}")
        self._live = True

    @property
    def count(self):
        return self.s.count

    @property
    def precision(self):
        return self.s.precision

    @property
    def limbs(self):
        return self.s.precision // 32

    @property
    def ref(self):
        return ctypes.byref(self.s)

    def to_device(self, exps, limbs):
        exps = np.ascontiguousarray(exps, dtype=np.uint32)
        limbs = np.ascontiguousarray(limbs, dtype=np.uint32)
        assert exps.size == self.count and limbs.size == self.count * self.limbs
        return lib().fpa_copy_array_to_device(self.ref, _ptr(exps), _ptr(limbs))

    def to_host(self):
        exps = np.zeros(self.count, dtype=np.uint32)
        limbs = np.zeros((self.count, self.limbs), dtype=np.uint32)
        rc = lib().fpa_copy_array_to_host(self.ref, _ptr(exps), _ptr(limbs))
        if rc != fpa_success:
            raise FpaError(f"fpa_copy_array_to_host -> {rc}")
        return exps, limbs

    def clear(self):
        if self._live:
            lib().fpa_clear(self.ref)
            self._live = False

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass


def fpa_add(r, a, b, mode):
    return lib().fpa_add(r.ref, a.ref, b.ref, mode)


def fpa_sub(r, a, b, mode):
    return lib().fpa_sub(r.ref, a.ref, b.ref, mode)


def fpa_mul(r, a, b, mode):
    return lib().fpa_mul(r.ref, a.ref, b.ref, mode)


def fpa_div(r, a, b, mode):
    return lib().fpa_div(r.ref, a.ref, b.ref, mode)


def fpa_sqrt(r, x, mode):
    return lib().fpa_sqrt(r.ref, x.ref, mode)


def fpa_fma(r, a, b, c, mode):
    """fpa_gb300_fma: r = RND(a*b + c) with one rounding."""
    return lib().fpa_gb300_fma(r.ref, a.ref, b.ref, c.ref, mode)


def fpa_neg(r, a):
    return lib().fpa_neg(r.ref, a.ref)


def fpa_set(r, x, mode):
    return lib().fpa_set(r.ref, x.ref, mode)


def fpa_set_ui(r, values):
    v = np.ascontiguousarray(values, dtype=np.uint64)
    return lib().fpa_set_ui(r.ref, _ptr(v))


def fpa_set_si(r, values):
    v = np.ascontiguousarray(values, dtype=np.int64)
    return lib().fpa_set_si(r.ref, _ptr(v))


def fpa_set_float(r, values):
    v = np.ascontiguousarray(values, dtype=np.float32)
    return lib().fpa_set_float(r.ref, _ptr(v))


def fpa_set_double(r, values):
    v = np.ascontiguousarray(values, dtype=np.float64)
    return lib().fpa_set_double(r.ref, _ptr(v))


def fpa_sgn(r_dev_ptr, x):
    """r_dev_ptr: device address of `count` int32 results."""
    return lib().fpa_sgn(ctypes.c_void_p(r_dev_ptr), x.ref)


def fpa_cmp(r_dev_ptr, a, b):
    return lib().fpa_cmp(ctypes.c_void_p(r_dev_ptr), a.ref, b.ref)


def elementwise(op, precision, count, mode, r_exps, r_limbs, a_exps, a_limbs, b_exps=0, b_limbs=0, stream=0):
    """fpa_gb300_elementwise on raw device addresses (ints)."""
    v = ctypes.c_void_p
    return lib().fpa_gb300_elementwise(op, precision, count, mode, v(r_exps), v(r_limbs), v(a_exps), v(a_limbs),
                                       v(b_exps), v(b_limbs), v(stream))


def device_errors():
    return lib().fpa_gb300_device_errors()


def dot(precision, count, length, mode, r_exps, r_limbs, x_exps, x_limbs, y_exps, y_limbs, stream=0):
    """fpa_gb300_dot on raw device addresses."""
    v = ctypes.c_void_p
    return lib().fpa_gb300_dot(precision, count, length, mode, v(r_exps), v(r_limbs), v(x_exps), v(x_limbs),
                               v(y_exps), v(y_limbs), v(stream))


def newton_sqrt(precision, count, iters, mode, y_exps, y_limbs, x_exps, x_limbs, stream=0):
    """fpa_gb300_newton_sqrt on raw device addresses (y updated in place)."""
    v = ctypes.c_void_p
    return lib().fpa_gb300_newton_sqrt(precision, count, iters, mode, v(y_exps), v(y_limbs), v(x_exps),
                                       v(x_limbs), v(stream))


def configs():
    out = []
    for c in range(lib().fpa_gb300_num_configs()):
        g, k, r = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        lib().fpa_gb300_config_shape(c, ctypes.byref(g), ctypes.byref(k), ctypes.byref(r))
        out.append((g.value, k.value, r.value))
    return out


def set_config(limbs, cfg):
    return lib().fpa_gb300_set_config(limbs, cfg)


def get_config(limbs):
    return lib().fpa_gb300_get_config(limbs)


def measure_imad_peak():
    """(mad.lo.u32/s, mad.hi.u32/s) measured on the current GPU."""
    lo, hi = ctypes.c_double(), ctypes.c_double()
    rc = lib().fpa_gb300_measure_imad_peak(ctypes.byref(lo), ctypes.byref(hi))
    if rc != fpa_success:
        raise FpaError(f"fpa_gb300_measure_imad_peak -> {rc}")
    return lo.value, hi.value


def measure_product_peak():
    """Limb products per second (mad.lo.cc / madc.hi.cc / addc into 96-bit columns, the
    product kernels' instruction triple) measured on the current GPU."""
    p = ctypes.c_double()
    rc = lib().fpa_gb300_measure_product_peak(ctypes.byref(p))
    if rc != fpa_success:
        raise FpaError(f"fpa_gb300_measure_product_peak -> {rc}")
    return p.value


def set_op_config(op, limbs, cfg):
    return lib().fpa_gb300_set_op_config(op, limbs, cfg)


def get_op_config(op, limbs):
    return lib().fpa_gb300_get_op_config(op, limbs)


def set_karatsuba_limbs(limbs):
    """fpa_mul takes one Karatsuba level from `limbs` limbs up (0 = never)."""
    return lib().fpa_gb300_set_karatsuba_limbs(limbs)


def get_karatsuba_limbs():
    return lib().fpa_gb300_get_karatsuba_limbs()


# fpa_gb300.h: fpa_batch_desc (32 bytes)
BATCH_DESC = np.dtype([("op", "u1"), ("mode", "u1"), ("limbs", "<u2"), ("reserved", "<u4"),
                       ("r_off", "<u8"), ("a_off", "<u8"), ("b_off", "<u8")])


class Batch:
    """fpa_batch_t: a planned mixed batch (descriptors are a BATCH_DESC array)."""

    def __init__(self, descs):
        descs = np.ascontiguousarray(descs, dtype=BATCH_DESC)
        self.count = descs.size
        self.h = ctypes.c_void_p()
        rc = lib().fpa_batch_create(ctypes.byref(self.h), descs.ctypes.data_as(ctypes.c_void_p), self.count)
        if rc != fpa_success:
            raise FpaError(f"fpa_batch_create -> {rc}")

    def run(self, r_exps, r_limbs, a_exps, a_limbs, b_exps=0, b_limbs=0, stream=0):
        v = ctypes.c_void_p
        return lib().fpa_batch_run(self.h, v(r_exps), v(r_limbs), v(a_exps), v(a_limbs), v(b_exps), v(b_limbs),
                                   v(stream))

    def capture(self, r_exps, r_limbs, a_exps, a_limbs, b_exps=0, b_limbs=0):
        v = ctypes.c_void_p
        return lib().fpa_batch_capture(self.h, v(r_exps), v(r_limbs), v(a_exps), v(a_limbs), v(b_exps), v(b_limbs))

    def graph_launch(self, stream=0):
        return lib().fpa_batch_graph_launch(self.h, ctypes.c_void_p(stream))

    def info(self):
        t = (ctypes.c_uint32 * 3)()
        k = ctypes.c_uint32()
        lib().fpa_batch_info(self.h, t, ctypes.byref(k))
        return list(t), k.value

    def destroy(self):
        if self.h:
            lib().fpa_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """fpa_server_t: request loop with continuous batching (batching=True) or plain
    per-job launches (batching=False)."""

    def __init__(self, hbm_budget_bytes=1 << 30, max_inflight=4, max_batch_ops=0, batching=True, resident_bytes=0):
        cfg = ServerConfig(hbm_budget_bytes, max_inflight, max_batch_ops, 1 if batching else 0)
        self.h = ctypes.c_void_p()
        rc = lib().fpa_server_create_resident(ctypes.byref(self.h), ctypes.byref(cfg), resident_bytes)
        if rc != fpa_success:
            raise FpaError(f"fpa_server_create_resident -> {rc}")
        self._keep = {}

    def submit(self, precision, ops, modes, a_exps, a_limbs, b_exps=None, b_limbs=None, a_from=0, b_from=0,
               keep=False, copy_out=True):
        """Submit one job; returns (job_id, (r_exps, r_limbs)) whose arrays are filled when
        the job completes (None when copy_out is False).  a_from / b_from: job ids whose kept
        results are the operands (the host operands are then ignored and may be None);
        keep: keep this job's result on the device for later jobs and read()."""
        ops = np.ascontiguousarray(ops, dtype=np.uint8)
        count = ops.size
        modes = np.ascontiguousarray(modes, dtype=np.uint8) if modes is not None else None
        arrs = [np.ascontiguousarray(x, dtype=np.uint32) if x is not None else None
                for x in (a_exps, a_limbs, b_exps, b_limbs)]
        r_e = np.zeros(count, dtype=np.uint32) if copy_out else None
        r_l = np.zeros(count * (precision // 32), dtype=np.uint32) if copy_out else None
        p = lambda x: x.ctypes.data_as(ctypes.c_void_p) if x is not None else None
        opts = ServerJobOpts(a_from, b_from, 1 if keep else 0, 1 if copy_out else 0)
        jid = lib().fpa_server_submit_ex(self.h, precision, count, p(ops), p(modes), p(arrs[0]), p(arrs[1]),
                                         p(arrs[2]), p(arrs[3]), p(r_e), p(r_l), ctypes.byref(opts))
        if jid <= 0:
            raise FpaError(f"fpa_server_submit_ex -> {-jid}")
        self._keep[jid] = (ops, modes, arrs, r_e, r_l, precision, count)
        return jid, (r_e, r_l)

    def read(self, jid):
        """A kept result, copied to host memory (waits for the job)."""
        precision, count = self._keep[jid][5], self._keep[jid][6]
        r_e = np.zeros(count, dtype=np.uint32)
        r_l = np.zeros(count * (precision // 32), dtype=np.uint32)
        rc = lib().fpa_server_read(self.h, jid, r_e.ctypes.data_as(ctypes.c_void_p),
                                   r_l.ctypes.data_as(ctypes.c_void_p))
        if rc != fpa_success:
            raise FpaError(f"fpa_server_read -> {rc}")
        return r_e, r_l

    def costs(self):
        """Nanoseconds summed over all batches: host packing, host-to-device, kernels, device-to-host."""
        c = (ctypes.c_uint64 * 4)()
        lib().fpa_server_costs(self.h, c)
        return dict(zip(["pack_ns", "h2d_ns", "device_ns", "d2h_ns"], list(c)))

    def wait(self, jid, timeout_ms=-1):
        return lib().fpa_server_wait(self.h, jid, timeout_ms)

    def times(self, jid):
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        lib().fpa_server_job_times(self.h, jid, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def release(self, jid):
        rc = lib().fpa_server_release(self.h, jid)
        if rc == fpa_success:
            self._keep.pop(jid, None)
        return rc

    def stats(self):
        s = (ctypes.c_uint64 * 6)()
        lib().fpa_server_stats(self.h, s)
        return dict(zip(["jobs", "ops", "batches", "peak_bytes", "failed", "budget_bytes"], list(s)))

    def destroy(self):
        if self.h:
            lib().fpa_server_destroy(self.h)
            self.h = ctypes.c_void_p()
        self._keep.clear()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
