"""ctypes binding of the C ABI in ``include/sdemc.h`` (``lib/libsdemc.so``).

This is the only place Python touches the native library.  There is no CPU
fallback: if the library is missing or no CUDA device is present, every call
raises.  Device buffers are torch tensors; only raw pointers, sizes and the
current CUDA stream cross the boundary.
"""
import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libsdemc.so")

MAX_DIM = 8
CHOL_LEN = 36
MARK_PARAMS = 12
CHUNK_PATHS = 32

# status codes
OK, EINVAL, EUNSUPPORTED, ENOMEM, ETIMEOUT, ECUDA, EOVERFLOW = range(7)
# enums (mirror include/sdemc.h)
NOISE_DIAG, NOISE_INDEP_SHARED, NOISE_INDEP_PAIR = 0, 1, 2
GRID_ADAPTED, GRID_UNIFORM = 0, 1
MARK_NONE, MARK_LOGNORMAL, MARK_INVCDF = 0, 1, 2
JUMP_COMMON, JUMP_ONE_ASSET = 0, 1
MODEL_AFFINE, MODEL_HESTON, MODEL_ASIAN = 0, 1, 2
(PAYOFF_EUROCALL, PAYOFF_EUROPUT, PAYOFF_BINARY_AON, PAYOFF_BASKET_ARITH, PAYOFF_BASKET_GEO,
 PAYOFF_RAINBOW, PAYOFF_DIGITAL, PAYOFF_BESTOF, PAYOFF_ASIANCALL, PAYOFF_HESTON_RAINBOW) = range(10)
CFG_EXACT_EULER = 1
INST_PAYOFF_AT_NOMINAL_STEP = 1

_f8 = ctypes.c_float * MAX_DIM


class SdemcInst(ctypes.Structure):
    """Mirror of ``sdemc_inst`` (field order and types must match the header)."""
    _fields_ = [
        ("dim", ctypes.c_int32), ("noise", ctypes.c_int32), ("grid", ctypes.c_int32),
        ("num_steps", ctypes.c_int32), ("mark", ctypes.c_int32), ("jump_target", ctypes.c_int32),
        ("exact_jumps", ctypes.c_int32), ("payoff", ctypes.c_int32), ("payoff_log", ctypes.c_int32),
        ("flags", ctypes.c_int32), ("stream_id", ctypes.c_uint32), ("model", ctypes.c_uint32),
        ("seed", ctypes.c_uint64), ("path_offset", ctypes.c_uint64), ("num_paths", ctypes.c_int64),
        ("T", ctypes.c_float), ("h", ctypes.c_float), ("rate", ctypes.c_float),
        ("inv_rate", ctypes.c_float), ("strike", ctypes.c_float), ("payoff_scale", ctypes.c_float),
        ("discount", ctypes.c_float), ("disc_rate", ctypes.c_float), ("reserved0", ctypes.c_int32 * 2),
        ("x0", _f8), ("drift_a", _f8), ("drift_b", _f8), ("diff_s", _f8), ("diff_q", _f8),
        ("diff2_s", _f8), ("diff2_q", _f8), ("jump_g", _f8), ("jump_k", _f8), ("jump_cdf", _f8),
        ("chol", ctypes.c_float * CHOL_LEN), ("mark_p", ctypes.c_float * MARK_PARAMS),
    ]

    def copy(self):
        c = SdemcInst()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(SdemcInst))
        return c

    def to_bytes(self):
        return ctypes.string_at(ctypes.byref(self), ctypes.sizeof(SdemcInst))


class SdemcCvWeights(ctypes.Structure):
    """Mirror of ``sdemc_cv_weights``: the served control variate's weight parameters."""
    _fields_ = [("comp", _f8), ("inv_comp", _f8), ("scale_over_k", ctypes.c_float), ("inv_sig", ctypes.c_float),
                ("drift", ctypes.c_float), ("T", ctypes.c_float), ("comp_j2", ctypes.c_float),
                ("inv_comp_j2", ctypes.c_float), ("agg", ctypes.c_int32), ("wkind", ctypes.c_int32),
                ("jumps", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class SdemcCfg(ctypes.Structure):
    _fields_ = [("block_threads", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
                ("interleave", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("timeout_ns", ctypes.c_int64)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_PROTOS = {
    "sdemc_abi_version": (_I, []),
    "sdemc_inst_size": (ctypes.c_size_t, []),
    "sdemc_inst_offsets": (_I, [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_I)]),
    "sdemc_last_error": (_I, [ctypes.c_char_p, ctypes.c_size_t]),
    "sdemc_device_sms": (_I, [ctypes.POINTER(_I)]),
    "sdemc_price_scratch_bytes": (ctypes.c_size_t, [_P]),
    "sdemc_price": (_I, [_P, _P, _P, ctypes.c_size_t, _P, _P, _P]),
    "sdemc_price_chunks": (_I, [_P, _P, _P, ctypes.c_size_t, _P, _P]),
    "sdemc_reduce_chunks": (_I, [_P, ctypes.c_int64, _I, _P, _P]),
    "sdemc_batch_plan_bytes": (ctypes.c_size_t, [_I]),
    "sdemc_batch_plan": (_I, [_P, _I, _P, ctypes.c_size_t]),
    "sdemc_batch_scratch_bytes": (ctypes.c_size_t, [_P]),
    "sdemc_price_batch": (_I, [_P, _P, _P, ctypes.c_size_t, _P, _P, _P, _I, _P]),
    "sdemc_cv_nparams": (_I, [_I]),
    "sdemc_cv_forward": (_I, [_I, _P, _P, _P, _P, _P, _P, ctypes.c_int64, _I, ctypes.c_float, _P, _P, _P]),
    "sdemc_cv_backward": (_I, [_I, _P, _P, _P, _P, _P, ctypes.c_int64, _I, ctypes.c_float, _P, _P, _I, _P, _P]),
    "sdemc_adam_step": (_I, [_P, _P, _P, _P, _I, _I, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, _P]),
    "sdemc_adam_bias": (_I, [_I, ctypes.c_float, ctypes.c_float, _P]),
    "sdemc_adam_step_dev": (_I, [_P, _P, _P, _P, _I, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, _P]),
    "sdemc_batch_autotune": (_I, [_P, _P, _P, ctypes.c_size_t, _P, _P, _P, _I, _P, _I, _I, _P, _P, _P, _P, _P]),
    "sdemc_cv_backward_tc": (_I, [_I, _P, _P, _P, _P, _P, ctypes.c_int64, _I, ctypes.c_float, _P, _P, _I, _P, _P,
                                  _P]),
    "sdemc_cv_forward_tc_scratch_bytes": (ctypes.c_size_t, [ctypes.c_int64, _I]),
    "sdemc_cv_forward_tc": (_I, [_I, _P, _P, _P, _P, _P, _P, ctypes.c_int64, _I, ctypes.c_float, _P, _P,
                                 ctypes.c_size_t, _P, _P]),
    "sdemc_price_cv_scratch_bytes": (ctypes.c_size_t, [_P]),
    "sdemc_price_cv": (_I, [_P, _P, ctypes.c_float, _P, ctypes.c_size_t, _P, _P, _P]),
    "sdemc_price_f64": (_I, [_P, _P, ctypes.c_size_t, _P, _P]),
    "sdemc_price_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "sdemc_price_noalloc": (_I, [_P, _P, _P, _P, _P]),
    "sdemc_replay": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sdemc_materialise": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _I, _P, _P, _P, _I, _P, _P]),
    "sdemc_mlmc_scratch_bytes": (ctypes.c_size_t, [_P]),
    "sdemc_mlmc_level": (_I, [_P, _I, _I, ctypes.c_float, ctypes.c_float, _P, _P, ctypes.c_size_t,
                              _P, _P, _P]),
    "sdemc_mlmc_terminals": (_I, [_P, _I, _I, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P]),
    "sdemc_mlmc_replay": (_I, [_P, _I, _I, ctypes.c_float, ctypes.c_float, _I, _I, _I, _I, _P, _P,
                               _P, _P, _P, _P, _P, _P]),
    "sdemc_mlmc_paths": (_I, [_P, _I, _I, ctypes.c_float, ctypes.c_float, _I, _I, _P, _P, _P, _P, _P, _P]),
    "sdemc_mlmc_replay_paths": (_I, [_P, _I, _I, ctypes.c_float, ctypes.c_float, _I, _I, _I, _I, _P, _P, _P,
                                     _P, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "sdemc_serve_cv_weights": (_I, [_P, _P]),
    "sdemc_serve_cv_paths": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _I, _P, _I, _P, _P]),
    "sdemc_server_create": (_I, [_P, ctypes.POINTER(_P)]),
    "sdemc_server_admit": (_I, [_P, _P]),
    "sdemc_server_poll": (_I, [_P, _P, _I, ctypes.POINTER(_I), ctypes.c_int64]),
    "sdemc_server_stats_get": (_I, [_P, _P]),
    "sdemc_server_destroy": (_I, [_P]),
    "sdemc_serve_sizes": (_I, [ctypes.POINTER(ctypes.c_size_t), _I]),
    "sdemc_philox": (_I, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                          ctypes.c_uint32, _I, _P, _P]),
    "sdemc_fp32_probe": (_I, [_I, _P, _I, ctypes.POINTER(ctypes.c_double), _P]),
    "sdemc_mufu_probe": (_I, [_I, _P, _I, ctypes.POINTER(ctypes.c_double), _P]),
    "sdemc_wait_probe": (_I, [_I, _P, _P]),
}
EXPORTED = tuple(_PROTOS)

_lib = None
_lock = threading.Lock()


def load():
    """Load the native library (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("sde_mc_gb300 native library missing at %s; build it with "
                               "`python -m sde_mc_gb300.build` (there is no CPU fallback)" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.sdemc_abi_version() != 1 or lib.sdemc_inst_size() != ctypes.sizeof(SdemcInst):
            raise RuntimeError("libsdemc ABI mismatch: header size %d vs ctypes %d" %
                               (lib.sdemc_inst_size(), ctypes.sizeof(SdemcInst)))
        _lib = lib
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().sdemc_last_error(buf, 512)
    return buf.value.decode(errors="replace")


_EXC = {EINVAL: ValueError, EUNSUPPORTED: NotImplementedError, ENOMEM: MemoryError,
        ETIMEOUT: TimeoutError, ECUDA: RuntimeError, EOVERFLOW: IndexError}


def check(rc, what="sdemc"):
    if rc != OK:
        raise _EXC.get(rc, RuntimeError)("%s failed (status %d): %s" % (what, rc, last_error()))


def status_error(st, what):
    """Raise for a device-side status word read back from a kernel."""
    st = int(st)
    if st == OK:
        return
    if st == ETIMEOUT:
        raise TimeoutError("%s: a bounded tensor-core wait gave up; every output of that launch, and of any "
                           "tensor-core launch that ran on the device at the same time, is void and must be "
                           "discarded" % what)
    if st & EOVERFLOW == EOVERFLOW:
        raise IndexError("%s: a path needed more steps/jumps than its storage or iteration cap "
                         "(the reference raises IndexError when its pre-drawn jump times run out)" % what)
    raise RuntimeError("%s: device status %d" % (what, st))


def require_cuda(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError("sde_mc_gb300 runs on a CUDA GPU (sm_103a) only; no CUDA device is "
                           "available and there is no CPU fallback")
    load()
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    dev = torch.device(device)
    if dev.type != "cuda":
        return torch.device("cuda", torch.cuda.current_device())
    return dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream_handle(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def byref(s):
    return ctypes.byref(s) if s is not None else None


# ------------------------------------------------------------ scratch -----
class ScratchPool:
    """Caller-owned scratch (torch memory) per (device, stream), grown on demand.

    The library never allocates; kernels that need per-chunk partials get a
    slice of this buffer.  The first 4 bytes hold the device status word, which
    must start at zero and is cleared by the reduction kernel after each use.
    """

    def __init__(self):
        self._bufs = {}

    def get(self, nbytes, device):
        key = (device.index, torch.cuda.current_stream(device).cuda_stream)
        buf = self._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            size = max(int(nbytes), 1 << 16)
            size = 1 << (size - 1).bit_length()
            buf = torch.zeros(size, dtype=torch.uint8, device=device)
            self._bufs[key] = buf
        return buf


SCRATCH = ScratchPool()


def abi_offsets():
    lib = load()
    n = _I(0)
    check(lib.sdemc_inst_offsets(None, ctypes.byref(n)), "sdemc_inst_offsets")
    arr = (ctypes.c_size_t * n.value)()
    check(lib.sdemc_inst_offsets(arr, ctypes.byref(n)), "sdemc_inst_offsets")
    return list(arr)


def ctypes_offsets():
    return [getattr(SdemcInst, f[0]).offset for f in SdemcInst._fields_]
