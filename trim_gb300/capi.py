"""ctypes binding of the C ABI in include/trim_gb300.h.

The product path: every call goes into the in-tree libtrim_gb300.so (built by
trim_gb300/buildlib.py).  There is no fallback -- if the library is missing the
import fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_lib", "libtrim_gb300.so")
HEADER = os.path.join(ROOT, "include", "trim_gb300.h")

TN_OK = 0
TN_ERR = {1: "ARG", 2: "OOM", 3: "TIMEOUT", 4: "CUDA", 5: "SHAPE", 6: "LABEL", 7: "UNSUPPORTED", 8: "NOBLOCK", 9: "FILE"}
MODE_FP64, MODE_SPLIT, MODE_FAST_BF16, MODE_FAST_TF32 = 0, 1, 2, 3
MODE_TC_ONLY, MODE_TC_FUSED, MODE_TC_TILED = 0x100, 0x200, 0x400
MODES = {"fp64": MODE_FP64, "split": MODE_SPLIT, "bf16": MODE_FAST_BF16, "tf32": MODE_FAST_TF32,
         "split_tc": MODE_SPLIT | MODE_TC_ONLY, "bf16_tc": MODE_FAST_BF16 | MODE_TC_ONLY,
         # every sector on the tensor cores, in one form
         "split_fused": MODE_SPLIT | MODE_TC_ONLY | MODE_TC_FUSED,
         "split_tiled": MODE_SPLIT | MODE_TC_ONLY | MODE_TC_TILED,
         "bf16_fused": MODE_FAST_BF16 | MODE_TC_ONLY | MODE_TC_FUSED,
         "bf16_tiled": MODE_FAST_BF16 | MODE_TC_ONLY | MODE_TC_TILED,
         "tf32_tc": MODE_FAST_TF32 | MODE_TC_ONLY}


class TnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[TN_ERR_{TN_ERR.get(code, code)}] {msg}")
        self.code = code


class SectorGemm(C.Structure):
    _fields_ = [("M", C.c_int64), ("N", C.c_int64), ("K", C.c_int64),
                ("a_off", C.c_int64), ("b_off", C.c_int64), ("c_off", C.c_int64)]


class SvdSector(C.Structure):
    _fields_ = [("M", C.c_int64), ("N", C.c_int64), ("a_off", C.c_int64), ("u_off", C.c_int64),
                ("s_off", C.c_int64), ("vt_off", C.c_int64)]


class EighSector(C.Structure):
    _fields_ = [("N", C.c_int64), ("a_off", C.c_int64), ("e_off", C.c_int64), ("v_off", C.c_int64)]


_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64
_IP = C.POINTER(C.c_int)
_I64P = C.POINTER(C.c_int64)
_DP = C.c_void_p  # double* (host or device) passed as address

_PROTOS = {
    "tn_last_error": (C.c_char_p, []),
    "tn_version": (_I, []),
    "tn_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "tn_ctx_destroy": (_I, [_P]),
    "tn_ctx_set_stream": (_I, [_P, _P]),
    "tn_ctx_sync": (_I, [_P]),
    "tn_ctx_launch_count": (_I, [_P, _I64P]),
    "tn_prof_enable": (_I, [_P, _I]),
    "tn_prof_read": (_I, [_P, _I, C.c_char_p, C.POINTER(C.c_double), _I64P, C.POINTER(C.c_double), C.POINTER(C.c_double), _IP]),
    "tn_sectormap_build": (_I, [_P, _I, _IP, _IP, _IP, _IP, C.POINTER(_P)]),
    "tn_sectormap_query": (_I, [_P, _I64P, _IP, _IP]),
    "tn_sectormap_blocks": (_I, [_P, _IP, _I64P, _I64P, _I64P]),
    "tn_sectormap_destroy": (_I, [_P]),
    "tn_permute": (_I, [_P, _P, _P, _IP, _DP, _DP]),
    "tn_plan_check_permute": (_I, [_P, _P, _IP, _DP, _DP, _I64P]),
    "tn_permute_c128": (_I, [_P, _P, _P, _IP, _DP, _DP]),
    "tn_tensor_add_gate": (_I, [_P, _I, _IP]),
    "tn_add_gate_c128": (_I, [_P, _P, _I, _IP, _DP]),
    "tn_transpose_c128": (_I, [_P, _P, _P, _I, _DP, _DP]),
    "tn_plan_check_permute_c128": (_I, [_P, _P, _IP, _DP, _DP, _I64P]),
    "tn_plan_check_views": (_I, [_P, _P, _IP, _DP, _DP, _IP]),
    "tn_contract_sectors": (_I, [_P, _I, _I, C.POINTER(SectorGemm), _DP, _DP, _DP]),
    "tn_autotune": (_I, [_P, _I, _I64P]),
    "tn_contract_sectors_fp64_noalloc": (_I, [_P, _I, C.POINTER(SectorGemm), _DP, _DP, _DP]),
    "tn_svd_sectors": (_I, [_P, _I, C.POINTER(SvdSector), _DP, _DP, _DP, _DP, _IP]),
    "tn_svd_plan": (_I, [_I64, _I64, _I, _IP, _IP, _IP, _I64P]),
    "tn_eigh_sectors": (_I, [_P, _I, C.POINTER(EighSector), _DP, _DP, _DP, _IP]),
    "tn_truncate_sectors": (_I, [_P, _I, _I64P, _I64P, _DP, _I64, _I64P, C.POINTER(C.c_double)]),
    "tn_tensor_svd_truncate": (_I, [_P, _I64, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P), C.POINTER(C.c_double)]),
    "tn_tensor_create": (_I, [_P, _I, _IP, _IP, _IP, _IP, C.POINTER(_P)]),
    "tn_tensor_destroy": (_I, [_P]),
    "tn_tensor_copy": (_I, [_P, C.POINTER(_P)]),
    "tn_tensor_set_elem": (_I, [_P, _DP, _I64]),
    "tn_tensor_set_elem_async": (_I, [_P, _DP, _I64]),
    "tn_tensor_get_elem": (_I, [_P, _DP, _I64]),
    "tn_tensor_device_elem": (_I, [_P, C.POINTER(_P), _I64P]),
    "tn_tensor_set_elem_device": (_I, [_P, _DP, _I64]),
    "tn_tensor_set_label": (_I, [_P, _I, _IP]),
    "tn_tensor_put_block": (_I, [_P, _IP, _I64, _I64, _I, _DP, _I64]),
    "tn_contract_sectors_loop": (_I, [_P, _I, _I, _P, _DP, _DP, _DP]),
    "tn_tensor_load": (_I, [_P, C.c_char_p, _P]),
    "tn_tensor_save": (_I, [_P, C.c_char_p]),
    "tn_batch_create": (_I, [_I, _P, _P, _P]),
    "tn_batch_destroy": (_I, [_P]),
    "tn_batch_put": (_I, [_P, _I, _P, _P]),
    "tn_batch_launch": (_I, [_P, _I]),
    "tn_batch_capture": (_I, [_P, _I]),
    "tn_batch_replay": (_I, [_P]),
    "tn_batch_output": (_I, [_P, _I, _P]),
    "tn_batch_sectors": (_I, [_P, _I, _P, _IP]),
    "tn_tensor_is_diagonal": (_I, [_P, _IP]),
    "tn_tensor_get_labels": (_I, [_P, _IP, _IP]),
    "tn_tensor_bonds": (_I, [_P, _IP, _IP, _IP, _IP, _IP, _I]),
    "tn_tensor_sectormap": (_I, [_P, C.POINTER(_P)]),
    "tn_tensor_permute": (_I, [_P, _I, _IP, _I]),
    "tn_tensor_transpose": (_I, [_P]),
    "tn_tensor_combine_bond": (_I, [_P, _I, _IP]),
    "tn_contract": (_I, [_P, _P, _I, _I, C.POINTER(_P)]),
    "tn_otimes": (_I, [_P, _P, _I, C.POINTER(_P)]),
    "tn_contract_batch": (_I, [_I, C.POINTER(_P), C.POINTER(_P), _I, C.POINTER(_P)]),
    "tn_tensor_scale": (_I, [_P, C.c_double]),
    "tn_network_create": (_I, [_P, C.c_char_p, C.POINTER(_P)]),
    "tn_network_destroy": (_I, [_P]),
    "tn_network_put_tensor": (_I, [_P, C.c_char_p, _P]),
    "tn_network_launch": (_I, [_P, _I, C.POINTER(_P)]),
    "tn_network_tree": (_I, [_P, C.c_char_p, _I]),
    "tn_network_capture": (_I, [_P, _I]),
    "tn_network_replay": (_I, [_P]),
    "tn_network_bind_host_input": (_I, [_P, C.c_char_p, _DP, _I64]),
    "tn_network_bind_host_output": (_I, [_P, _DP, _I64]),
    "tn_network_output": (_I, [_P, C.POINTER(_P)]),
}

_lib = None


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(tn_\w+)\s*\(", text, flags=re.M)))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"trim_gb300 extension not built: {LIB_PATH} missing (run trim_gb300/buildlib.py)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != TN_OK:
        msg = lib().tn_last_error()
        raise TnError(rc, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def int_array(vals):
    vals = list(vals)
    return (C.c_int * max(1, len(vals)))(*vals)


def pack_bonds(bonds):
    """bonds: [(btype, [(u1, prt, prtf, deg), ...]), ...] -> ctypes arrays."""
    btype = int_array([b[0] for b in bonds])
    nq = int_array([len(b[1]) for b in bonds])
    q, d = [], []
    for _, runs in bonds:
        for (u, p, f, dg) in runs:
            q += [u, p, f]
            d.append(dg)
    return len(bonds), btype, nq, int_array(q), int_array(d)
