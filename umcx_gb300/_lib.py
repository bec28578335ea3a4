"""ctypes binding of libumcx_gb300.so (include/umcx_gpu.h, include/umcx_host.h).

The library is built in-tree by umcx_gb300.build into umcx_gb300/_build/.  Loading fails loudly when it is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libumcx_gb300.so"

UMCX_OK, UMCX_ERR_INPUT, UMCX_ERR_CUDA, UMCX_ERR_TIMEOUT, UMCX_ERR_NODEV = 0, 1, 2, 3, 4
OUT_FLUENCE_RATE, OUT_FLUENCE, OUT_ENERGY = 0, 1, 2
SRC_TYPES = ["pencil", "isotropic", "cone", "disk", "planar", "fourier"]
DET_ID, DET_PPATH, DET_EXITPOS, DET_EXITDIR = 1, 4, 16, 32
LABEL_DET = 0x80
SIM_STRICT_MATH = 0x1
SIM_FP32_ACCUM = 0x2
ACTION_RUN, ACTION_DUMPJSON, ACTION_DUMPMASK, ACTION_HELP = 0, 1, 2, 3


class Sim(C.Structure):
    """umcx_sim (MCX_param of the reference plus the kernel's own inputs)."""

    _fields_ = [
        ("dim", C.c_uint32 * 4),
        ("nphoton", C.c_uint64),
        ("photon_offset", C.c_uint64),
        ("tstart", C.c_float),
        ("tend", C.c_float),
        ("rtstep", C.c_float),
        ("unitinmm", C.c_float),
        ("isreflect", C.c_int32),
        ("issavevol", C.c_int32),
        ("issavedet", C.c_int32),
        ("savedetflag", C.c_int32),
        ("mediumnum", C.c_int32),
        ("outputtype", C.c_int32),
        ("detnum", C.c_int32),
        ("srctype", C.c_int32),
        ("maxdetphotons", C.c_uint32),
        ("flags", C.c_uint32),
        ("seeds", C.c_uint32 * 4),
        ("srcpos", C.c_float * 4),
        ("srcdir", C.c_float * 4),
        ("srcparam1", C.c_float * 4),
        ("srcparam2", C.c_float * 4),
    ]

    def copy(self) -> "Sim":
        s = Sim()
        C.memmove(C.byref(s), C.byref(self), C.sizeof(Sim))
        return s


class Result(C.Structure):
    _fields_ = [
        ("energy_escape", C.c_double),
        ("energy_total", C.c_double),
        ("detected", C.c_uint64),
        ("saved", C.c_uint64),
        ("launched", C.c_uint64),
        ("steps", C.c_uint64),
        ("crossings", C.c_uint64),
        ("scatters", C.c_uint64),
        ("reflections", C.c_uint64),
        ("capped", C.c_uint64),
        ("kernel_ms", C.c_float),
        ("total_ms", C.c_float),
        ("status", C.c_int32),
        ("block_size", C.c_int32),
        ("grid_size", C.c_int32),
        ("reserved", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class Tuning(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("blocks_per_sm", C.c_int32), ("aggregation", C.c_int32),
                ("budget_ms", C.c_int32), ("grid_size", C.c_int32), ("reserved", C.c_int32)]


class Peaks(C.Structure):
    _fields_ = [("fp32_fma_per_s", C.c_double), ("sfu_per_s", C.c_double), ("l2_atomic_per_s", C.c_double),
                ("sm_count", C.c_int32), ("sm_clock_khz", C.c_int32)]


class Adjoint(C.Structure):
    _fields_ = [("readings", C.c_void_p), ("dread_dmua", C.c_void_p), ("dread_dmus", C.c_void_p),
                ("dflu_dmua", C.c_void_p), ("dflu_dmus", C.c_void_p), ("jacobian", C.c_void_p),
                ("records", C.c_uint64), ("replay_mismatch", C.c_uint64), ("replay_ms", C.c_float),
                ("reserved", C.c_int32)]


assert C.sizeof(Sim) == 168, C.sizeof(Sim)

class ShapeOp(C.Structure):
    _fields_ = [("kind", C.c_int32), ("tag", C.c_int32), ("present", C.c_uint32), ("f", C.c_float * 8),
                ("reserved", C.c_int32)]


class Domain(C.Structure):
    _fields_ = [("dim", C.c_uint32 * 3), ("fill", C.c_int32), ("ops", C.POINTER(ShapeOp)), ("nops", C.c_int32),
                ("mediumnum", C.c_int32), ("volume", C.c_void_p), ("detpos", C.c_void_p), ("detnum", C.c_int32),
                ("reserved", C.c_int32)]


assert C.sizeof(ShapeOp) == 48, C.sizeof(ShapeOp)

UMCX_JOB_DEVICE_LABELS = 1
SHAPE_SPHERE, SHAPE_BOX, SHAPE_XLAYER, SHAPE_YLAYER, SHAPE_ZLAYER, SHAPE_CYLINDER = range(6)
SHAPE_HAS_TAG, SHAPE_HAS_SIZE0, SHAPE_HAS_HI = 0x1, 0x2, 0x10

ABI_VERSION = 4  # UMCX_ABI_VERSION of include/umcx_gpu.h that these signatures follow

_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_U8P = C.POINTER(C.c_uint8)

# (name, restype, argtypes) of every exported entry point declared in include/*.h
SIGNATURES = [
    ("umcx_abi_version", C.c_int, []),
    ("umcx_device_checks", C.c_int, []),
    ("umcx_create", C.c_int, [C.POINTER(_P), C.c_int]),
    ("umcx_destroy", None, [_P]),
    ("umcx_last_error", C.c_char_p, [_P]),
    ("umcx_set_tuning", C.c_int, [_P, C.POINTER(Tuning)]),
    ("umcx_seeds_from_rngseed", C.c_int, [C.c_int32, C.POINTER(C.c_uint32)]),
    ("umcx_detp_columns", C.c_int, [C.POINTER(Sim)]),
    ("umcx_gpu_forward", C.c_int, [_P, C.POINTER(Sim), _P, _P, _P, _P, _P, C.POINTER(Result)]),
    ("umcx_gpu_forward_device", C.c_int, [_P, C.POINTER(Sim), _P, _P, _P, _P, _P, _P, C.POINTER(Result)]),
    ("umcx_gpu_forward_adjoint", C.c_int, [_P, C.POINTER(Sim), _P, _P, _P, _P, _P, C.POINTER(Result)]),
    ("umcx_gpu_backward", C.c_int, [_P, C.POINTER(Adjoint)]),
    ("umcx_batch_create", C.c_int, [_P, C.c_int, C.POINTER(Sim), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p), C.POINTER(_P)]),
    ("umcx_batch_run", C.c_int, [_P, C.POINTER(Result)]),
    ("umcx_batch_get", C.c_int, [_P, C.c_int, _P, _P, C.POINTER(Result)]),
    ("umcx_batch_set_tuning", C.c_int, [_P, C.POINTER(Tuning)]),
    ("umcx_batch_destroy", None, [_P]),
    ("umcx_batch_labels", C.c_void_p, [_P, C.c_int]),
    ("umcx_gpu_build_labels", C.c_int, [_P, C.POINTER(Domain), _P]),
    ("umcx_autotune", C.c_int, [_P, C.POINTER(Sim), _P, _P, _P, _P, _P, C.c_double, C.POINTER(Tuning),
                                C.POINTER(C.c_float)]),
    ("umcx_gpu_rng_dump", C.c_int, [_P, C.POINTER(C.c_uint32), C.c_uint64, C.c_uint32, C.c_uint32, _P]),
    ("umcx_measure_peaks", C.c_int, [C.c_int, C.POINTER(Peaks)]),
    ("umcx_gpu_forward_noalloc", C.c_int, [C.c_int, C.POINTER(Sim), _P, _P, _P, _P, _P, _P, C.POINTER(Result)]),
    ("MCX_run_cmd", C.c_int, [C.POINTER(C.c_char_p), C.c_int]),
    ("MCX_run_json", C.c_int, [C.c_char_p]),
    ("umcx_main", C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
    ("umcx_job_from_args", C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(C.c_char_p)]),
    ("umcx_job_from_json", C.c_int, [C.POINTER(_P), C.c_char_p]),
    ("umcx_job_from_args_ex", C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(C.c_char_p), C.c_uint32]),
    ("umcx_job_build_labels", C.c_int, [_P, _P, _P]),
    ("umcx_job_free", None, [_P]),
    ("umcx_job_error", C.c_char_p, [_P]),
    ("umcx_job_action", C.c_int, [_P]),
    ("umcx_job_console", C.c_char_p, [_P]),
    ("umcx_job_config_json", C.c_char_p, [_P, C.c_int]),
    ("umcx_job_sim", C.POINTER(Sim), [_P]),
    ("umcx_job_labels", _U8P, [_P]),
    ("umcx_job_media", _FP, [_P]),
    ("umcx_job_detpos", _FP, [_P]),
    ("umcx_job_isnormalized", C.c_int, [_P]),
    ("umcx_job_tuning", C.c_int, [_P, C.POINTER(Tuning)]),
    ("umcx_job_normalizer", C.c_float, [_P, C.c_double]),
    ("umcx_job_domain_dims", C.c_int, [_P, C.POINTER(C.c_uint32)]),
    ("umcx_job_domain_int32", C.c_int, [_P, _P, C.c_size_t]),
    ("umcx_job_dump_mask", C.c_int, [_P, C.c_char_p]),
    ("umcx_job_write_outputs", C.c_int, [_P, _P, _P, C.POINTER(Result), C.c_int]),
]

_lib = None


def load() -> C.CDLL:
    """Load libumcx_gb300.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m umcx_gb300.build` first")
        lib = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.umcx_abi_version() != ABI_VERSION:
            raise RuntimeError(f"{LIB_PATH} has ABI {lib.umcx_abi_version()}, these bindings {ABI_VERSION}: rebuild it")
        _lib = lib
    return _lib


def check(rc: int, ctx=None, what: str = "") -> None:
    if rc != UMCX_OK:
        msg = load().umcx_last_error(ctx).decode() if ctx else ""
        raise RuntimeError(f"{what} failed with status {rc}: {msg}")
