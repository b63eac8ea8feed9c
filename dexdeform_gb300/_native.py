"""ctypes binding of libdexmpm.so (include/dexmpm.h).

The library is the only compute path: if it is missing, or no CUDA device is
present, every entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import c_bool, POINTER, c_char_p, c_float, c_int, c_int32, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libdexmpm.so")

OK, ERR_ARG, ERR_LAUNCH, ERR_OUT_OF_GRID, ERR_TOO_MANY_BODIES = 0, 1, 2, 4, 8
MAX_BODIES = 32
FLAG_EXACT_CAPSULE_GRAD = 1
STATE_PLANES = 24
TAPE_PLANES = 33  # DEXMPM_TAPE_PLANES: SVD (24) + stress (9) per particle
PX, PV, PF, PC = 0, 3, 6, 15


class DexError(RuntimeError):
    pass


class DexEnv(ctypes.Structure):
    _fields_ = [("p_off", c_int32), ("n", c_int32), ("blk_off", c_int32), ("body_off", c_int32),
                ("gx", c_int32), ("gy", c_int32), ("gz", c_int32), ("n_bodies", c_int32),
                ("dx", c_float), ("inv_dx", c_float), ("dt", c_float), ("ground_friction", c_float),
                ("gravity", c_float * 3), ("ground_height", c_float)]


class DexBatch(ctypes.Structure):
    _fields_ = [("n_envs", c_int32), ("n_particles", c_int32), ("n_tiles", c_int32), ("n_blocks", c_int32),
                ("n_bodies", c_int32), ("tile_size", c_int32), ("grid_ctas", c_int32), ("flags", c_int32),
                ("n_slots", c_int32), ("pad0", c_int32), ("pad1", c_int32), ("pad2", c_int32),
                ("envs", c_void_p), ("tiles", c_void_p), ("block_env", c_void_p), ("mass", c_void_p),
                ("vol", c_void_p), ("mu_lam_yield", c_void_p), ("grid", c_void_p), ("vout", c_void_p),
                ("vout_grad", c_void_p), ("in_grad", c_void_p), ("block_flag", c_void_p),
                ("block_list", c_void_p), ("block_count", c_void_p), ("done_counter", c_void_p),
                ("body_shape", c_void_p), ("error", c_void_p), ("block_xyz", c_void_p)]


class DexSegment(ctypes.Structure):
    _fields_ = [("other", c_void_p), ("other_stride", c_int32), ("offset", c_int32), ("count", c_int32),
                ("pad", c_int32)]


SEGMENTS_GATHER, SEGMENTS_SCATTER, SEGMENTS_SCATTER_ADD = 0, 1, 2


class DexSortWork(ctypes.Structure):
    _fields_ = [("cell_count", c_void_p), ("cell_start", c_void_p), ("block_total", c_void_p),
                ("block_base", c_void_p), ("block_flag", c_void_p), ("block_list", c_void_p), ("rank", c_void_p),
                ("key", c_void_p), ("partial", c_void_p), ("counters", c_void_p)]


SORT_CHUNK = 4096  # DEXMPM_SORT_CHUNK


def sort_partials(n_blocks: int) -> int:
    return (n_blocks + SORT_CHUNK - 1) // SORT_CHUNK


assert ctypes.sizeof(DexEnv) == 64

P = c_void_p
_REF_SIGS = {
    "compute_svd": [P] * 6 + [c_float, c_int, P],
    "compute_svd_grad": [P] * 11 + [c_float, c_int, P],
    "p2g": [P] * 10 + [P, P, c_float, c_float, c_float, P, P, P, c_int, P],
    "p2g_grad": [P] * 10 + [P, P, c_float, c_float, c_float] + [P] * 13 + [c_int, P],
    "grid_op_v2": [P] * 11 + [c_float] * 4 + [P, P, c_int, P],
    "grid_op_v2_grad": [P] * 17 + [c_float] * 4 + [P, P, P, c_int, P],
    "g2p": [P, P, P, c_float, c_float, c_float, P, P, c_float, P, P, c_int, P],
    "g2p_grad": [P, P, P, c_float, c_float, c_float, P, P, c_float, P, P, c_int, P, P, P, P, P, P],
    "compute_dist": [P] * 6 + [c_int] + [P] * 4 + [c_int, c_int, P],
    "particle2mass": [P, P, P, P, c_float, c_float, P, P, P, P, c_int, c_int, c_int, P],
    "particle_sdf": [P] * 5 + [c_int, P, c_float] + [P] * 3 + [c_int, P],
    "render": [P] * 13 + [c_float, P, c_int, c_bool, P, c_int, c_int, c_float, c_int, P, P],
}
_BATCH_SIGS = {
    "dexmpm_reset": [POINTER(DexBatch), P],
    "dexmpm_clear_slots": [POINTER(DexBatch), c_int, c_int, P],
    "dexmpm_p2g": [POINTER(DexBatch), c_int, P, P, P, P],
    "dexmpm_grid_op": [POINTER(DexBatch), c_int, c_int, P, P, P],
    "dexmpm_g2p": [POINTER(DexBatch), c_int, P, P, P],
    "dexmpm_g2p2g": [POINTER(DexBatch), c_int, c_int, P, P, P, P, P],
    "dexmpm_substep": [POINTER(DexBatch), c_int, c_int, P, P, P, P, P, P],
    "dexmpm_substep_grad": [POINTER(DexBatch), c_int, P, P, P, P, P, P, P, P, P, P],
    "dexmpm_g2p_grad": [POINTER(DexBatch), c_int, P, P, P, P, P],
    "dexmpm_grid_op_grad": [POINTER(DexBatch), c_int, P, P, P, P, P],
    "dexmpm_p2g_grad": [POINTER(DexBatch), c_int, P, P, P, P, P],
    "dexmpm_p2g_g2p_grad": [POINTER(DexBatch), c_int, c_int, P, P, P, P, P, P, P],
    "dexmpm_get_error": [POINTER(DexBatch), POINTER(c_int32), P],
    "dexmpm_substep_noalloc": [POINTER(DexEnv), P, P, P, P, P, P, P, P, P, P],
    "dexmpm_sort": [POINTER(DexBatch), POINTER(DexSortWork), P, P, P, P],
    "dexmpm_permute": [P, P, P, c_int, c_int, c_int, P],
    "dexmpm_copy_segments": [P, c_int, c_int, P, c_int, c_int, c_int, P],
    "dexmpm_abi_get_error": [POINTER(c_int32)],
}

# every symbol include/dexmpm.h declares
EXPORTED = sorted(list(_REF_SIGS) + list(_BATCH_SIGS) + ["dexmpm_version"])

_lib = None


def lib_available() -> bool:
    return os.path.isfile(LIB_PATH)


def load(path: str = LIB_PATH):
    """Load libdexmpm.so and declare its prototypes (no CUDA call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(path):
        raise DexError(f"{path} is missing; build it with `python -m dexdeform_gb300.build`")
    L = ctypes.CDLL(path)
    for name, args in {**_REF_SIGS, **_BATCH_SIGS}.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = c_int
    L.dexmpm_version.restype = c_char_p
    L.dexmpm_version.argtypes = []
    _lib = L
    return L


def check(rc: int, what: str):
    if rc != OK:
        raise DexError(f"{what} failed with status {rc}")


def require_cuda():
    import torch
    if not torch.cuda.is_available():
        raise DexError("a CUDA device is required: libdexmpm.so has no CPU path")


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return c_void_p(s.cuda_stream)


def ptr(t) -> c_void_p:
    return c_void_p(t.data_ptr()) if t is not None else c_void_p(0)
