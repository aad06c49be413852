"""ctypes binding of libphono_gpu.so (include/phono.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every call raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libphono_gpu.so"

PHONO_OK = 0
ERRORS = {-1: "PHONO_ERR_ARG", -2: "PHONO_ERR_CUDA", -3: "PHONO_ERR_NOMEM", -4: "PHONO_ERR_STATE",
          -5: "PHONO_ERR_NUMERIC", -6: "PHONO_ERR_TIMEOUT"}

PRECISIONS = {"f64": 0, "f32k": 1, "f64v": 2}
BATCH_PERSISTENT, BATCH_STREAMS = 0, 1  # phono_batch_set_mode
SURFACE_MODES = {"reference": 0, "corrected": 1}
BCS = {"absorbing": 0, "reference": 0, "rigid": 1}
SOURCE_MODES = {"line": 0, "wall": 1}
FIELDS = {"ux": 0, "uy": 1, "uz": 2, "ux_old": 3, "uy_old": 4, "uz_old": 5,
          "vx": 6, "vy": 7, "vz": 8, "cx": 9, "cy": 10, "cz": 11}

# exported symbols of include/phono.h (checked by the CPU test suite)
EXPORTS = ["phono_create", "phono_set_source", "phono_step", "phono_steps_done", "phono_reset",
           "phono_set_materials", "phono_stream", "phono_sync",
           "phono_read_surface", "phono_download", "phono_upload", "phono_elem_size", "phono_energy",
           "phono_energy_static", "phono_batch_create", "phono_batch_add", "phono_batch_remove",
           "phono_batch_remaining", "phono_batch_step", "phono_batch_sync", "phono_batch_last_step_ms",
           "phono_batch_destroy", "phono_batch_set_mode", "phono_set_tiling", "phono_set_segments", "phono_footprint", "phono_set_steps_done",
           "phono_upload_surface", "phono_set_lattice", "phono_set_inclusions", "phono_download_materials",
           "phono_test_wait_timeout", "phono_time_kernels",
           "phono_last_step_ms", "phono_destroy", "phono_last_error", "phono_abi_version"]


class PhonoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class PhonoDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("fdx", ctypes.c_void_p), ("fdy", ctypes.c_void_p), ("fdz", ctypes.c_void_p),
        ("sdx", ctypes.c_void_p), ("sdy", ctypes.c_void_p), ("sdz", ctypes.c_void_p),
        ("mat", ctypes.c_void_p), ("table", ctypes.c_void_p), ("nmat", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("precision", ctypes.c_int), ("surface_mode", ctypes.c_int), ("bc", ctypes.c_int),
        ("source_mode", ctypes.c_int), ("max_steps", ctypes.c_int), ("record_every", ctypes.c_int),
        ("tile_j", ctypes.c_int), ("x_segment", ctypes.c_int),
    ]


class PhonoEnergyDense(ctypes.Structure):
    """phono_energy_dense of include/phono.h: caller-owned dense device arrays."""
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("precision", ctypes.c_int),
        ("ux", ctypes.c_void_p), ("uy", ctypes.c_void_p), ("uz", ctypes.c_void_p),
        ("vx", ctypes.c_void_p), ("vy", ctypes.c_void_p), ("vz", ctypes.c_void_p),
        ("mat", ctypes.c_void_p), ("table", ctypes.c_void_p),
        ("fdx", ctypes.c_void_p), ("fdy", ctypes.c_void_p), ("fdz", ctypes.c_void_p),
        ("sdx", ctypes.c_void_p), ("sdy", ctypes.c_void_p), ("sdz", ctypes.c_void_p),
        ("dt", ctypes.c_double), ("nmat", ctypes.c_int),
    ]


class PhonoLattice(ctypes.Structure):
    """phono_lattice of include/phono.h: a lattice of cylindrical holes."""
    _fields_ = [
        ("pitch", ctypes.c_int), ("ncx", ctypes.c_int), ("ncy", ctypes.c_int),
        ("radius", ctypes.c_void_p), ("kind", ctypes.c_void_p), ("depth", ctypes.c_int), ("host", ctypes.c_int),
    ]


class PhonoInclusions(ctypes.Structure):
    """phono_inclusions of include/phono.h: the reference's inclusion list (Grid.targets)."""
    _fields_ = [
        ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p), ("n", ctypes.c_int),
        ("tx", ctypes.c_void_p), ("ty", ctypes.c_void_p), ("tz", ctypes.c_void_p), ("tr", ctypes.c_void_p),
        ("id", ctypes.c_void_p), ("inside", ctypes.c_int), ("host", ctypes.c_int),
    ]


ENERGY_STATIC_MAX_NX = 8192

_lib = None


def load(path: Path | None = None):
    """Load the library (once); raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with phonomena_gb300.build.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(str(p))
    vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "phono_create": (ci, [ctypes.POINTER(PhonoDesc), ctypes.POINTER(vp)]),
        "phono_set_source": (ci, [vp, vp, ci]),
        "phono_step": (ci, [vp, ci]),
        "phono_steps_done": (ci, [vp]),
        "phono_reset": (ci, [vp]),
        "phono_set_materials": (ci, [vp, vp, vp, ci]),
        "phono_stream": (vp, [vp]),
        "phono_sync": (ci, [vp]),
        "phono_read_surface": (ci, [vp, ci, ci, vp]),
        "phono_download": (ci, [vp, ci, vp, ctypes.c_size_t]),
        "phono_upload": (ci, [vp, ci, vp, ctypes.c_size_t]),
        "phono_elem_size": (ci, [vp]),
        "phono_energy": (ci, [vp, vp]),
        "phono_energy_static": (ci, [ctypes.POINTER(PhonoEnergyDense), vp, vp]),
        "phono_batch_create": (ci, [ci, ci, ci, ctypes.POINTER(vp)]),
        "phono_batch_add": (ci, [vp, vp, ci]),
        "phono_batch_remove": (ci, [vp, ci]),
        "phono_batch_remaining": (ci, [vp, ci]),
        "phono_batch_step": (ci, [vp, ci]),
        "phono_batch_sync": (ci, [vp]),
        "phono_batch_last_step_ms": (ci, [vp, ctypes.POINTER(ctypes.c_float)]),
        "phono_batch_destroy": (None, [vp]),
        "phono_batch_set_mode": (ci, [vp, ci, ci]),
        "phono_set_tiling": (ci, [vp, ci, ci]),
        "phono_set_segments": (ci, [vp, ci, vp, ci]),
        "phono_set_steps_done": (ci, [vp, ci]),
        "phono_upload_surface": (ci, [vp, ci, ci, vp]),
        "phono_set_lattice": (ci, [vp, ctypes.POINTER(PhonoLattice), vp, ci]),
        "phono_set_inclusions": (ci, [vp, ctypes.POINTER(PhonoInclusions), vp, ci]),
        "phono_download_materials": (ci, [vp, vp, ctypes.c_size_t]),
        "phono_test_wait_timeout": (ci, [vp, ci, ci]),
        "phono_time_kernels": (ci, [vp, ci, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
        "phono_footprint": (ci, [ci, ci, ci, ci, ci, ci, ctypes.POINTER(ctypes.c_size_t)]),
        "phono_last_step_ms": (ci, [vp, ctypes.POINTER(ctypes.c_float)]),
        "phono_destroy": (None, [vp]),
        "phono_last_error": (ctypes.c_char_p, []),
        "phono_abi_version": (ci, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != PHONO_OK:
        msg = _lib.phono_last_error().decode(errors="replace") if _lib is not None else ""
        raise PhonoError(rc, msg)
    return rc
