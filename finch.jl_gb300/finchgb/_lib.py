"""ctypes binding of libfinchgb.so, the C ABI declared in include/finchgb.h.

This is the same binding a Julia `ccall` layer makes: plain pointers, sizes
and int status codes.  There is no CPU fallback: if
the shared library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_size_t, c_uint, c_uint64, c_void_p, c_char_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_native" / "libfinchgb.so"

# fgb_status
OK, EINVAL, ENOMEM, ETIMEOUT, ECUDA, EUNSUPPORTED, EBUSY, ECANCELLED = range(8)
STATUS_NAMES = {0: "OK", 1: "EINVAL", 2: "ENOMEM", 3: "ETIMEOUT", 4: "ECUDA", 5: "EUNSUPPORTED",
                6: "EBUSY", 7: "ECANCELLED"}
# fgb_dtype
NONE, F64, F32, BF16, I32, I64, BOOL = -1, 0, 1, 2, 3, 4, 5
# fgb_semiring
PLUS_TIMES, MIN_PLUS, MAX_PLUS, OR_AND = 0, 1, 2, 3
# fgb_orient
CSR, CSC = 0, 1
# flags
ACCUMULATE, FINCH_ORDER, FMA, NO_FMA = 0x1, 0x2, 0x4, 0x8
# fgb_ewise_op
EW_MUL, EW_ADD = 0, 1
# fgb_combine
COMBINE_ADD, COMBINE_OR, COMBINE_MIN, COMBINE_MAX, COMBINE_LAST = range(5)


class FinchGBError(RuntimeError):
    """A libfinchgb call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"[{STATUS_NAMES.get(status, status)}] {message}")


class FgbSpmmTuning(ctypes.Structure):
    _fields_ = [("lanes", c_int32), ("variant", c_int32), ("path", c_int64), ("bands", c_int32),
                ("reserved", c_int32)]


class FgbSddmmTuning(ctypes.Structure):
    _fields_ = [("lanes", c_int32), ("variant", c_int32), ("chunk", c_int64), ("slab", c_int64),
                ("bands", c_int32), ("reserved", c_int32)]


class FgbCgOptions(ctypes.Structure):
    _fields_ = [("rtol", c_double), ("max_iter", c_int64), ("chunk", c_int32),
                ("precision", c_int32), ("replace_every", c_int64), ("accumulate", c_int32),
                ("reserved", c_int32)]


class FgbCgResult(ctypes.Structure):
    _fields_ = [("iterations", c_int64), ("replacements", c_int64),
                ("true_rel_residual", c_double), ("seconds", c_double), ("converged", c_int32),
                ("compact_index", c_int32)]


class FgbPlanDesc(ctypes.Structure):
    _fields_ = [("op", c_int32), ("semiring", c_int32), ("dtype", c_int32), ("flags", c_uint),
                ("A", c_void_p), ("in0", c_void_p), ("in1", c_void_p), ("out", c_void_p),
                ("ld_in0", c_int64), ("ld_in1", c_int64), ("ld_out", c_int64), ("k", c_int64)]


class FgbPlanInfo(ctypes.Structure):
    _fields_ = [("lanes", c_int32), ("bands", c_int32), ("path", c_int64),
                ("tuned_ms", c_double), ("first_candidate_ms", c_double),
                ("candidates", c_int32), ("from_cache", c_int32), ("panels", c_int32),
                ("variant", c_int32), ("launches", c_int32), ("reserved", c_int32)]


class FgbServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", c_size_t), ("max_inflight", c_int32), ("rows_per_item", c_int32),
                ("blocks_per_sm", c_int32), ("idle_exit_us", c_int32), ("mode", c_int32),
                ("reserved", c_int32)]


class FgbRequest(ctypes.Structure):
    _fields_ = [("op", c_int32), ("matrix", c_int32), ("matrix_b", c_int32), ("nk", c_int32),
                ("input", c_void_p), ("output", c_void_p)]


class FgbServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_uint64), ("completed", c_uint64), ("launches", c_uint64),
                ("batches_published", c_uint64), ("pool_used", c_uint64), ("admit_ns", c_uint64),
                ("scan_ns", c_uint64), ("finish_ns", c_uint64), ("iterations", c_uint64),
                ("queue_ns", c_uint64), ("service_ns", c_uint64)]


SERVER_CLASSES = 10  # FGB_SERVER_CLASSES


class FgbServerClassShape(ctypes.Structure):
    _fields_ = [("matrices", c_int32), ("lanes", c_int32), ("rows_per_item", c_int32), ("reserved", c_int32),
                ("ms", c_double), ("ms_default", c_double)]


class FgbServerTuning(ctypes.Structure):
    _fields_ = [("cls", FgbServerClassShape * SERVER_CLASSES)]


class FgbSparse(ctypes.Structure):
    _fields_ = [("nrows", c_int64), ("ncols", c_int64), ("nnz", c_int64), ("orient", c_int32),
                ("index_base", c_int32), ("ptr_t", c_int32), ("idx_t", c_int32),
                ("val_t", c_int32), ("reserved", c_int32), ("ptr", c_void_p), ("idx", c_void_p),
                ("val", c_void_p)]


# name -> (restype, argtypes); every symbol include/*.h declares.
SIGNATURES: dict[str, tuple] = {
    "fgb_version": (c_int, []),
    "fgb_gather_ceiling": (c_int, [c_void_p, c_int64, c_int32, c_int64, POINTER(c_double), c_void_p]),
    "fgb_last_error": (c_char_p, []),
    "fgb_ctx_create": (c_int, [c_int, POINTER(c_void_p)]),
    "fgb_ctx_destroy": (c_int, [c_void_p]),
    "fgb_ctx_stream": (c_void_p, [c_void_p]),
    "fgb_ctx_num_sms": (c_int, [c_void_p]),
    "fgb_ctx_device_error": (c_int, [c_void_p, POINTER(c_int)]),
    "fgb_malloc": (c_int, [c_void_p, c_size_t, POINTER(c_void_p)]),
    "fgb_free": (c_int, [c_void_p, c_void_p]),
    "fgb_host_alloc": (c_int, [c_void_p, c_size_t, POINTER(c_void_p)]),
    "fgb_host_free": (c_int, [c_void_p, c_void_p]),
    "fgb_upload": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "fgb_download": (c_int, [c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "fgb_stream_sync": (c_int, [c_void_p, c_void_p]),
    "fgb_narrow_index": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_void_p]),
    "fgb_transpose": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_void_p, c_void_p, c_void_p]),
    "fgb_coo_assemble": (c_int, [c_void_p, c_int64, c_int64, c_int64, c_int, c_void_p, c_void_p, c_int,
                                 c_int, c_void_p, c_int, POINTER(FgbSparse), POINTER(c_int64),
                                 c_void_p]),
    "fgb_spmv": (c_int, [c_void_p, c_int, POINTER(FgbSparse), c_void_p, c_int, c_void_p, c_int,
                         c_uint, c_void_p]),
    "fgb_spmm": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_int64, c_int64, c_void_p,
                         c_int64, c_int, c_uint, c_void_p]),
    "fgb_spmm_ex": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_int64, c_int64, c_void_p,
                            c_int64, c_int, c_uint, POINTER(FgbSpmmTuning), c_void_p]),
    "fgb_spmm_noalloc": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_int64, c_int64,
                                 c_void_p, c_int64, c_int, c_uint, c_void_p]),
    "fgb_sddmm": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_int64, c_void_p, c_int64,
                          c_int64, c_void_p, c_int, c_uint, c_void_p]),
    "fgb_sddmm_ex": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_int64, c_void_p, c_int64,
                             c_int64, c_void_p, c_int, c_uint, POINTER(FgbSddmmTuning), c_void_p]),
    "fgb_spgemm_symbolic": (c_int, [c_void_p, POINTER(FgbSparse), POINTER(FgbSparse), c_void_p,
                                    POINTER(c_int64), c_void_p]),
    "fgb_spgemm_numeric": (c_int, [c_void_p, POINTER(FgbSparse), POINTER(FgbSparse), c_int, c_uint,
                                   POINTER(FgbSparse), c_void_p]),
    "fgb_ewise_count": (c_int, [c_void_p, c_int, POINTER(FgbSparse), POINTER(FgbSparse), c_void_p,
                                POINTER(c_int64), c_void_p]),
    "fgb_ewise_fill": (c_int, [c_void_p, c_int, POINTER(FgbSparse), POINTER(FgbSparse), c_void_p,
                               c_void_p, c_void_p, c_void_p]),
    "fgb_ewise_reduce": (c_int, [c_void_p, c_int, POINTER(FgbSparse), POINTER(FgbSparse), c_void_p,
                                 c_int64, c_void_p, c_int, c_uint, c_void_p]),
    "fgb_dense_dot": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fgb_dense_axpby": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_int, c_void_p]),
    "fgb_dense_map": (c_int, [c_void_p, c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p,
                              c_void_p]),
    "fgb_dense_affine": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "fgb_reduce_minmax": (c_int, [c_void_p, c_int, c_int, POINTER(FgbSparse), c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "fgb_sparse_scale": (c_int, [c_void_p, POINTER(FgbSparse), c_int, c_int, c_int, c_void_p, c_int, c_int,
                                 c_void_p, c_int, c_void_p, c_void_p, c_void_p, POINTER(c_int64),
                                 POINTER(c_int64), c_void_p]),
    "fgb_scalar_op": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fgb_spgemm_dense": (c_int, [c_void_p, POINTER(FgbSparse), POINTER(FgbSparse), c_int, c_uint, c_void_p,
                                 c_int64, c_void_p]),
    "fgb_sparse_to_dense": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_void_p, c_int64, c_void_p]),
    "fgb_spmm_semiring": (c_int, [c_void_p, c_int, POINTER(FgbSparse), c_void_p, c_int64, c_int64, c_void_p,
                                  c_int64, c_int, c_uint, c_void_p]),
    "fgb_bfs_pull": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_void_p, c_void_p, c_int, c_int64,
                             c_int64, c_void_p, c_void_p]),
    "fgb_or_count": (c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fgb_minby_map": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p]),
    "fgb_minby_relax": (c_int, [c_void_p, POINTER(FgbSparse), c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_int64, c_void_p]),
    "fgb_cg_solve": (c_int, [c_void_p, POINTER(FgbSparse), POINTER(FgbSparse), c_void_p, c_void_p,
                             POINTER(FgbCgOptions), POINTER(FgbCgResult), c_void_p]),
    "fgb_panels_create": (c_int, [c_void_p, POINTER(FgbSparse), c_int32, POINTER(c_void_p)]),
    "fgb_panels_spmm": (c_int, [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_void_p, c_int64,
                                c_int, c_uint, POINTER(FgbSpmmTuning), c_void_p]),
    "fgb_panels_destroy": (c_int, [c_void_p]),
    "fgb_plan_create": (c_int, [c_void_p, POINTER(FgbPlanDesc), c_int32, POINTER(c_void_p)]),
    "fgb_plan_execute": (c_int, [c_void_p, c_void_p]),
    "fgb_plan_info_get": (c_int, [c_void_p, POINTER(FgbPlanInfo)]),
    "fgb_plan_destroy": (c_int, [c_void_p]),
    "fgb_random_csr": (c_int, [c_void_p, c_uint64, c_int64, c_int64, c_double, c_int, c_void_p,
                               c_void_p, c_void_p, POINTER(c_int64), c_void_p]),
    "fgb_server_create": (c_int, [c_void_p, POINTER(FgbServerConfig), POINTER(c_void_p)]),
    "fgb_server_register": (c_int, [c_void_p, POINTER(FgbSparse), POINTER(c_int32)]),
    "fgb_server_submit": (c_int, [c_void_p, POINTER(FgbRequest), POINTER(c_uint64)]),
    "fgb_server_wait": (c_int, [c_void_p, c_uint64, c_int32, POINTER(c_double)]),
    "fgb_server_submit_batch": (c_int, [c_void_p, POINTER(FgbRequest), c_int32, POINTER(c_uint64),
                                        POINTER(c_int32)]),
    "fgb_server_wait_batch": (c_int, [c_void_p, POINTER(c_uint64), c_int32, c_int32,
                                      POINTER(c_double)]),
    "fgb_server_tune": (c_int, [c_void_p, c_int32, POINTER(FgbServerTuning)]),
    "fgb_server_set_tuning": (c_int, [c_void_p, POINTER(FgbServerTuning)]),
    "fgb_server_stats_get": (c_int, [c_void_p, POINTER(FgbServerStats)]),
    "fgb_server_destroy": (c_int, [c_void_p]),
}

# fgb_request_op / fgb_serve_mode
REQ_SPMV, REQ_SPMM, REQ_MASKED_MUL = 0, 1, 2
SERVE_BATCHED, SERVE_PER_CALL = 0, 1

# fgb_map_op
MAP_ADD, MAP_SUB, MAP_MUL, MAP_DIV, MAP_MIN, MAP_MAX = range(6)
AXIS_ROW, AXIS_COL = 0, 1

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def load() -> ctypes.CDLL:
    """Loads libfinchgb.so (built in-tree); raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise FinchGBError(ECUDA, f"libfinchgb.so not built ({LIB_PATH}); run "
                                          "__graft_entry__.build() -- there is no CPU fallback")
            L = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    msg = load().fgb_last_error()
    return msg.decode() if msg else ""


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise FinchGBError(status, f"{what}: {last_error()}" if what else last_error())


def call(name: str, *args) -> None:
    """Calls an entry point and raises FinchGBError on a non-zero status."""
    check(getattr(load(), name)(*args), name)
