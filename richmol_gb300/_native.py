"""ctypes binding of librichmol_gb300.so (C ABI in include/richmol_gb300.h).

The shared library is built in-tree (``richmol_gb300/lib``) by ``build_library``
for sm_103a. There is no CPU fallback: if the library or a CUDA device is
missing, every GPU entry point raises.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_DIR = os.path.join(PKG, "lib")
LIB_PATH = os.path.join(LIB_DIR, "librichmol_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
SOURCES = [os.path.join(PKG, "csrc", f) for f in ("kr_step.cu", "kr_batch.cu", "kr_batch_simt.cu", "kr_batch_tc.cu",
                                                        "kr_batch_zr.cu", "kr_expv.cu")]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

KR_OK, KR_ERR_ARG, KR_ERR_CUDA, KR_ERR_MAXORDER, KR_ERR_TIMEOUT, KR_ERR_UNSUPPORTED = range(6)
KR_K_COMPLEX, KR_K_REAL, KR_K_IMAG = 0, 1, 2
KR_MAXCART = 9
KR_MAXPART = 4096
KR_PART_INLINE = 16  # parts whose field coefficients go as kernel parameters
KR_STEP_SKIP_KRYLOV = 1
KR_MATVEC_TENSOR, KR_MATVEC_FP32, KR_MATVEC_TENSOR_TMEM, KR_MATVEC_FP32_REG = 0, 1, 2, 3
KR_SEG_F64, KR_SEG_F32_MATVEC = 0, 1
KR_PREC_F64, KR_PREC_DF = 0, 1
# bytes of per-step field input that travel host -> device (the field
# coefficients, scales and thresholds of kr_set_field, passed as kernel
# parameters): int npart (padded to 8) + 16 x 9 complex + 16 complex + 16 double
FIELD_COEF_BYTES = 8 + KR_PART_INLINE * KR_MAXCART * 16 + KR_PART_INLINE * 16 + KR_PART_INLINE * 8

EXPORTED = [
    "kr_ctx_create", "kr_ctx_destroy", "kr_last_error", "kr_op_create", "kr_op_destroy", "kr_op_check",
    "kr_set_field", "kr_set_field_schedule", "kr_set_field_step",
    "kr_matvec", "kr_step", "kr_sync_status", "kr_op_launch_count", "kr_op_work",
    "kr_probe_fp64", "kr_probe_fp32", "kr_probe_mma", "kr_probe_mma_ta", "kr_probe_wait", "kr_step_static", "kr_static_scratch_bytes",
    "kr_batch_create", "kr_batch_destroy", "kr_batch_load", "kr_batch_store", "kr_batch_step", "kr_batch_sync",
    "kr_batch_korder", "kr_batch_expect", "kr_batch_launch_count", "kr_batch_matvec", "kr_batch_apply", "kr_batch_set_matvec",
    "kr_batch_populations",
    "kr_expv", "kr_op_norm1", "kr_observables",
    "kr_seg_create", "kr_seg_destroy", "kr_seg_step", "kr_seg_launch_count", "kr_seg_set_precision",
    "kr_op_set_precision", "kr_batch_expect_dev",
]


class KrylovError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"[kr status {code}] {msg}")
        self.code = code


def build_library(verbose=False, nvcc="nvcc"):
    """Compiles the CUDA sources (one process per translation unit, in
    parallel) and links richmol_gb300/lib/librichmol_gb300.so."""
    os.makedirs(LIB_DIR, exist_ok=True)
    common = [nvcc, *ARCH_FLAGS, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
    if verbose:
        common.insert(1, "-Xptxas=-v")
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(LIB_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen([*common, "-c", "-o", obj, src], stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    out, failed = [], False
    for pr in procs:
        o, _ = pr.communicate()
        out.append(o)
        failed |= pr.returncode != 0
    if failed:
        raise RuntimeError("nvcc failed:\n" + "".join(out))
    tmp = LIB_PATH + ".tmp"
    res = subprocess.run([nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB_PATH)
    return "".join(out) + res.stdout + res.stderr


class kr_op_desc(ctypes.Structure):
    P = ctypes.c_void_p
    _fields_ = [
        ("nslab_out", ctypes.c_int32), ("nslab_in", ctypes.c_int32),
        ("out_dm", P), ("out_dk", P), ("out_off", P),
        ("in_dm", P), ("in_dk", P), ("in_off", P),
        ("dim_out", ctypes.c_int64), ("dim_in", ctypes.c_int64),
        ("nk", ctypes.c_int32),
        ("k_off", P), ("k_rows", P), ("k_cols", P), ("k_type", P),
        ("k_data", P), ("k_data_len", ctypes.c_int64),
        ("nm", ctypes.c_int32),
        ("m_rows", P), ("m_width", P), ("m_ncart", P), ("m_col_off", P), ("m_val_off", P),
        ("m_col", P), ("m_col_len", ctypes.c_int64),
        ("m_val", P), ("m_val_len", ctypes.c_int64),
        ("npart", ctypes.c_int32),
        ("nmf", ctypes.c_int32), ("mf_group", P), ("mf_part", P),
        ("nterm", ctypes.c_int32), ("t_out", P), ("t_in", P), ("t_k", P), ("t_mf", P),
        ("maxorder", ctypes.c_int32),
        ("out_stride", P), ("in_stride", P),
    ]


_lib = None
_lib_lock = threading.Lock()


def lib():
    """Loads the library once; raises if it has not been built."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run richmol_gb300._native.build_library() "
                              "(or __graft_entry__.build()) first; there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
        L.kr_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.kr_ctx_create.restype = ctypes.c_int
        L.kr_ctx_destroy.argtypes = [vp]
        L.kr_ctx_destroy.restype = None
        L.kr_last_error.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
        L.kr_last_error.restype = ctypes.c_int
        L.kr_op_create.argtypes = [vp, ctypes.POINTER(kr_op_desc), ctypes.POINTER(vp)]
        L.kr_op_create.restype = ctypes.c_int
        L.kr_op_destroy.argtypes = [vp]
        L.kr_op_destroy.restype = None
        L.kr_op_check.argtypes = [ctypes.POINTER(kr_op_desc), ctypes.c_char_p, ctypes.c_size_t]
        L.kr_op_check.restype = ctypes.c_int
        L.kr_set_field.argtypes = [vp, vp, vp, vp, vp]
        L.kr_set_field.restype = ctypes.c_int
        L.kr_set_field_schedule.argtypes = [vp, i32, vp, vp, vp, vp]
        L.kr_set_field_schedule.restype = ctypes.c_int
        L.kr_set_field_step.argtypes = [vp, i32, vp]
        L.kr_set_field_step.restype = ctypes.c_int
        L.kr_matvec.argtypes = [vp, vp, vp, i64, vp]
        L.kr_matvec.restype = ctypes.c_int
        L.kr_step.argtypes = [vp, vp, i64, vp, dbl, dbl, dbl, ctypes.c_uint32, vp, vp]
        L.kr_step.restype = ctypes.c_int
        L.kr_sync_status.argtypes = [vp, vp]
        L.kr_sync_status.restype = ctypes.c_int
        L.kr_op_launch_count.argtypes = [vp]
        L.kr_op_launch_count.restype = i64
        L.kr_op_work.argtypes = [vp, ctypes.POINTER(dbl), ctypes.POINTER(dbl)]
        L.kr_op_work.restype = ctypes.c_int
        L.kr_step_static.argtypes = [vp, vp, i64, vp, dbl, dbl, dbl, ctypes.c_uint32, vp, vp]
        L.kr_step_static.restype = ctypes.c_int
        L.kr_static_scratch_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
        L.kr_static_scratch_bytes.restype = ctypes.c_int
        L.kr_batch_create.argtypes = [vp, i64, i32, ctypes.POINTER(vp)]
        L.kr_batch_create.restype = ctypes.c_int
        L.kr_batch_destroy.argtypes = [vp]
        L.kr_batch_destroy.restype = None
        L.kr_batch_load.argtypes = [vp, vp, vp]
        L.kr_batch_load.restype = ctypes.c_int
        L.kr_batch_store.argtypes = [vp, vp, vp]
        L.kr_batch_store.restype = ctypes.c_int
        L.kr_batch_step.argtypes = [vp, vp, vp, dbl, dbl, dbl, ctypes.POINTER(i32), vp]
        L.kr_batch_step.restype = ctypes.c_int
        L.kr_batch_sync.argtypes = [vp, ctypes.POINTER(i32), vp]
        L.kr_batch_sync.restype = ctypes.c_int
        L.kr_batch_korder.argtypes = [vp, vp, vp]
        L.kr_batch_korder.restype = ctypes.c_int
        L.kr_batch_expect.argtypes = [vp, vp, vp, vp]
        L.kr_batch_expect.restype = ctypes.c_int
        L.kr_batch_expect_dev.argtypes = [vp, vp, vp, vp, vp]
        L.kr_batch_expect_dev.restype = ctypes.c_int
        L.kr_batch_populations.argtypes = [vp, vp, vp]
        L.kr_batch_populations.restype = ctypes.c_int
        L.kr_batch_set_matvec.argtypes = [vp, i32]
        L.kr_batch_set_matvec.restype = ctypes.c_int
        L.kr_batch_apply.argtypes = [vp, vp, vp, vp, vp]
        L.kr_batch_apply.restype = ctypes.c_int
        L.kr_seg_create.argtypes = [vp, i32, vp, ctypes.POINTER(vp)]
        L.kr_seg_create.restype = ctypes.c_int
        L.kr_seg_destroy.argtypes = [vp]
        L.kr_seg_destroy.restype = None
        L.kr_seg_step.argtypes = [vp, vp, vp, dbl, dbl, dbl, vp, vp]
        L.kr_seg_step.restype = ctypes.c_int
        L.kr_seg_launch_count.argtypes = [vp]
        L.kr_seg_launch_count.restype = i64
        L.kr_seg_set_precision.argtypes = [vp, i32]
        L.kr_seg_set_precision.restype = ctypes.c_int
        L.kr_op_set_precision.argtypes = [vp, i32]
        L.kr_op_set_precision.restype = ctypes.c_int
        L.kr_batch_matvec.argtypes = [vp, vp, vp]
        L.kr_batch_matvec.restype = ctypes.c_int
        L.kr_batch_launch_count.argtypes = [vp]
        L.kr_batch_launch_count.restype = i64
        L.kr_probe_fp32.argtypes = [vp, ctypes.POINTER(dbl)]
        L.kr_probe_fp32.restype = ctypes.c_int
        L.kr_expv.argtypes = [vp, vp, vp, dbl, i32, dbl, dbl, vp, vp]
        L.kr_expv.restype = ctypes.c_int
        L.kr_op_norm1.argtypes = [vp, ctypes.POINTER(dbl), vp]
        L.kr_op_norm1.restype = ctypes.c_int
        L.kr_observables.argtypes = [vp, vp, i64, vp, vp, ctypes.POINTER(dbl), vp]
        L.kr_observables.restype = ctypes.c_int
        L.kr_probe_mma.argtypes = [vp, vp, vp, vp]
        L.kr_probe_mma.restype = ctypes.c_int
        L.kr_probe_mma_ta.argtypes = [vp, vp, vp, vp]
        L.kr_probe_mma_ta.restype = ctypes.c_int
        L.kr_probe_wait.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(dbl)]
        L.kr_probe_wait.restype = ctypes.c_int
        L.kr_probe_fp64.argtypes = [vp, ctypes.POINTER(dbl)]
        L.kr_probe_fp64.restype = ctypes.c_int
        _lib = L
        return L


def last_error(ctx=None):
    buf = ctypes.create_string_buffer(1024)
    lib().kr_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code, ctx=None):
    if code != KR_OK:
        raise KrylovError(code, last_error(ctx))


def ptr(a):
    """Address of a contiguous numpy array or torch tensor."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous
        return a.ctypes.data
    assert a.is_contiguous()
    return a.data_ptr()
