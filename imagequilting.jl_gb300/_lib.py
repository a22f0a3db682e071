"""ctypes binding of libiqgpu.so (declarations in include/iqgpu.h).

The library is built in-tree by build.py. There is no CPU fallback: without the library,
every call raises IQError.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libiqgpu.so")

IQ_OK = 0
IQ_ERR_ARG = 1
IQ_ERR_CUDA = 2
IQ_ERR_ALLOC = 3
IQ_ERR_NOPATTERN = 4
IQ_ERR_CUTCAP = 5
IQ_ERR_STATE = 6
IQ_ERR_LIMIT = 7
IQ_F32 = 0
IQ_F64 = 1
PATHS = {"raster": 0, "dilation": 1, "random": 2}

c_i64p = ctypes.POINTER(ctypes.c_int64)


class IQError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libiqgpu error %d: %s" % (code, msg))
        self.code = code


class SimParams(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("tilesize", ctypes.c_int64 * 3),
                ("simsize", ctypes.c_int64 * 3), ("overlap", ctypes.c_double * 3),
                ("tol", ctypes.c_double), ("path", ctypes.c_int32), ("nreal", ctypes.c_int32),
                ("debug", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("real0", ctypes.c_int64)]


class HardData(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("coords", ctypes.c_void_p), ("values", ctypes.c_void_p)]


class SoftData(ctypes.Structure):
    _fields_ = [("aux", ctypes.c_void_p), ("auxsize", ctypes.c_int64 * 3),
                ("auxti", ctypes.c_void_p)]


# name -> (restype, argtypes); mirrors include/iqgpu.h
SIGNATURES = {
    "iq_version": (ctypes.c_int, []),
    "iq_last_error": (ctypes.c_char_p, []),
    "iq_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "iq_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "iq_ctx_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "iq_ties": (ctypes.c_int, [ctypes.c_void_p, c_i64p]),
    "iq_lp_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, c_i64p, ctypes.c_uint64]),
    "iq_lp_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, c_i64p]),
    "iq_lp_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, c_i64p, ctypes.c_void_p,
                                        ctypes.c_int64]),
    "iq_lp_embed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_i64p, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "iq_lp_loss_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_void_p, c_i64p, c_i64p, ctypes.c_void_p,
                                       ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_void_p]),
    "iq_lp_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "iq_lp_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "iq_set_ti": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                 c_i64p]),
    "iq_simulate": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SimParams),
                                   ctypes.POINTER(HardData), ctypes.c_int32,
                                   ctypes.POINTER(SoftData), ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "iq_fastdistance": (ctypes.c_int, [ctypes.c_void_p, c_i64p, ctypes.c_int32, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "iq_pick": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                               ctypes.POINTER(ctypes.c_void_p), ctypes.c_double, ctypes.c_uint64,
                               ctypes.c_int64, ctypes.c_int64, c_i64p, c_i64p, c_i64p,
                               ctypes.POINTER(ctypes.c_double), ctypes.c_int64]),
    "iq_pick_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_double,
                                       ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, c_i64p,
                                       c_i64p, c_i64p, ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int64, ctypes.c_void_p]),
    "iq_graphcut": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int32, c_i64p, ctypes.c_int32, ctypes.c_void_p]),
    "iq_finddisabled": (ctypes.c_int, [ctypes.c_void_p, c_i64p, ctypes.c_void_p]),
    "iq_genpath": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int32, c_i64p, ctypes.c_int32,
                                  ctypes.c_int64, c_i64p, c_i64p]),
    "iq_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "iq_profile_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p,
                                      ctypes.POINTER(ctypes.c_double), c_i64p,
                                      ctypes.POINTER(ctypes.c_double)]),
    "iq_ctx_launches": (ctypes.c_int64, [ctypes.c_void_p]),
    "iq_set_option": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64]),
}

_lib = None


def load():
    """Load libiqgpu.so (raises IQError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise IQError(-1, "libiqgpu.so is missing: build it with __graft_entry__.build() "
                              "or imagequilting.jl_gb300/build.py")
        lib = ctypes.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def check(rc):
    if rc != IQ_OK:
        msg = load().iq_last_error()
        raise IQError(rc, msg.decode() if msg else "")
    return rc


def i64arr(values):
    return (ctypes.c_int64 * len(values))(*[int(v) for v in values])
