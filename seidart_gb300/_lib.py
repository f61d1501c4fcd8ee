"""ctypes binding of ``libseidart_gb300.so`` (the C ABI in include/seidart_gb300.h).

The library is built in-tree by ``seidart_gb300.build``.  There is no
fallback: if the shared library is missing or does not load, every solver call
raises :class:`LibraryMissingError`.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libseidart_gb300.so"

SEISMIC2, SEISMIC25, ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C = 1, 2, 3, 4, 5
KIND_NAMES = {SEISMIC2: "seismic2", SEISMIC25: "seismic25", ELECTROMAG2: "electromag2", ELECTROMAG25: "electromag25",
              ELECTROMAG2C: "electromag2c"}
KIND_BY_NAME = {v: k for k, v in KIND_NAMES.items()}

SFD_OK, SFD_ERR_BAD_ARG, SFD_ERR_STATE, SFD_ERR_CUDA, SFD_ERR_UNSTABLE, SFD_ERR_TIMEOUT = 0, -1, -2, -3, -4, -5

# Every exported symbol of include/seidart_gb300.h
EXPORTS = (
    "sfd_version", "sfd_last_error", "sfd_model_planes", "sfd_num_fields", "sfd_num_channels",
    "sfd_num_memory", "sfd_state_bytes", "sfd_create", "sfd_set_model", "sfd_set_model_ids", "sfd_set_cpml", "sfd_set_cpml2d",
    "sfd_set_source", "sfd_set_stress_source", "sfd_set_source_wavelet", "sfd_set_cpml_params", "sfd_share_model", "sfd_set_receivers", "sfd_reset", "sfd_set_field", "sfd_get_field",
    "sfd_get_field_async", "sfd_encode_field_i16",
    "sfd_get_memory", "sfd_run", "sfd_status", "sfd_get_traces", "sfd_traces_device", "sfd_field_device", "sfd_launch_half",
    "sfd_on_chip", "sfd_set_wait_limit", "sfd_test_stall_waits",
    "sfd_destroy", "sfd_checkpoint_bytes", "sfd_checkpoint_save", "sfd_checkpoint_load", "sfd_run_checkpointed", "sfd_adjoint_record",
    "sfd_adjoint_bytes",
    "sfd_adjoint_begin", "sfd_adjoint_segment", "sfd_adjoint_gradient", "sfd_batch_scratch_bytes", "sfd_batch_create", "sfd_batch_set_tiling", "sfd_batch_run",
    "sfd_batch_status", "sfd_batch_set_wait_limit", "sfd_batch_test_stall_waits", "sfd_batch_destroy", "sfd_electromag2_run_static",
)


class LibraryMissingError(RuntimeError):
    pass


class SfdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class UnstableError(SfdError):
    pass


class SfdConfig(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("npml", C.c_int32), ("nstep", C.c_int32), ("nrec", C.c_int32), ("flags", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
    ]


class SfdCpmlParams(C.Structure):
    _fields_ = [
        ("sig_max", C.c_double * 3), ("alpha_max", C.c_double), ("kappa_max", C.c_double),
        ("NP", C.c_double), ("NPA", C.c_double), ("mode", C.c_int32),
    ]


WAVELETS = {"gaus0": 0, "gaus1": 1, "gaus2": 2}

_lock = threading.Lock()
_lib = None


def _declare(lib):
    P = C.c_void_p
    i32, i64, sz = C.c_int32, C.c_int64, C.c_size_t
    dp, fp, ip = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int32)
    sig = {
        "sfd_version": (i32, []),
        "sfd_last_error": (C.c_char_p, []),
        "sfd_model_planes": (i32, [i32]),
        "sfd_num_fields": (i32, [i32]),
        "sfd_num_channels": (i32, [i32]),
        "sfd_num_memory": (i32, [i32]),
        "sfd_state_bytes": (i32, [C.POINTER(SfdConfig), C.POINTER(sz)]),
        "sfd_create": (i32, [C.POINTER(SfdConfig), P, sz, P, C.POINTER(P)]),
        "sfd_set_model": (i32, [P, dp, i64]),
        "sfd_set_model_ids": (i32, [P, P, i32, dp, i64]),
        "sfd_set_cpml": (i32, [P, dp, i64]),
        "sfd_set_cpml2d": (i32, [P, dp, i64]),
        "sfd_set_source": (i32, [P, i32, i32, i32, dp, i32, i32]),
        "sfd_set_stress_source": (i32, [P, i32, i32, i32, dp, i32, i32]),
        "sfd_set_source_wavelet": (i32, [P, i32, i32, i32, i32, i32, C.c_double, C.c_double, dp, i32]),
        "sfd_set_cpml_params": (i32, [P, C.POINTER(SfdCpmlParams)]),
        "sfd_set_receivers": (i32, [P, ip, i32]),
        "sfd_share_model": (i32, [P, P]),
        "sfd_reset": (i32, [P]),
        "sfd_set_field": (i32, [P, i32, fp, i64]),
        "sfd_get_field": (i32, [P, i32, fp, i64]),
        "sfd_get_field_async": (i32, [P, i32, P, i64]),
        "sfd_encode_field_i16": (i32, [P, i32, P, P]),
        "sfd_get_memory": (i32, [P, i32, fp, i64]),
        "sfd_run": (i32, [P, i64]),
        "sfd_status": (i32, [P, C.POINTER(i64), dp]),
        "sfd_get_traces": (i32, [P, fp, i64]),
        "sfd_traces_device": (P, [P]),
        "sfd_field_device": (i32, [P, i32, C.POINTER(P), C.POINTER(i64)]),
        "sfd_launch_half": (i32, [P, i32, i32]),
        "sfd_on_chip": (i32, [P, ip, ip]),
        "sfd_set_wait_limit": (i32, [P, i64]),
        "sfd_test_stall_waits": (i32, [P, i32]),
        "sfd_destroy": (i32, [P]),
        "sfd_electromag2_run_static": (i32, [C.POINTER(SfdConfig), dp, dp, i32, i32, dp, ip, fp, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def lib():
    """Load (once) and return the CUDA library; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise LibraryMissingError(
                    f"{LIB_PATH} is not built; run `python -m seidart_gb300.build` (CUDA toolkit required)")
            try:
                handle = C.CDLL(str(LIB_PATH))
            except OSError as e:
                raise LibraryMissingError(f"cannot load {LIB_PATH}: {e}") from e
            _declare(handle)
            _lib = handle
        return _lib


def check(code: int) -> None:
    if code == SFD_OK:
        return
    msg = lib().sfd_last_error().decode(errors="replace")
    if code == SFD_ERR_UNSTABLE:
        raise UnstableError(code, msg)
    raise SfdError(code, msg)
