"""ctypes binding of the C-ABI in include/mibm.h.

The same binding drives two shared libraries with identical exports: the
product library ``libmibm.so`` (CUDA, sm_103a) and, in the test suite only,
the CPU oracle.  Constants are parsed from the header so that the Python side
cannot drift from the C side.
"""
from __future__ import annotations

import ctypes as C
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(_HERE)
HEADER = os.path.join(ROOT, "include", "mibm.h")


def _parse_enums(path: str) -> dict[str, int]:
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out: dict[str, int] = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", text, flags=re.S):
        val = -1
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, v = (s.strip() for s in item.split("="))
                val = int(v, 0)
            else:
                name = item
                val += 1
            out[name] = val
    return out


ENUMS = _parse_enums(HEADER)
globals().update(ENUMS)

#: exported function name -> (restype, argtypes)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_longlong)
SIGNATURES: dict[str, tuple] = {
    "mibm_context_create_": (C.c_int, []),
    "mibm_context_bind_": (C.c_int, [_I]),
    "mibm_context_destroy_": (C.c_int, [_I]),
    "mibm_last_status_": (C.c_int, []),
    "mibm_last_message": (C.c_char_p, []),
    "mibm_set_grid_": (None, [_I, _I, _I, _D, _D, _D]),
    "mibm_set_mesh_sizes_": (None, [_I, _I, _I]),
    "mibm_register_field_": (None, [_I, C.c_void_p]),
    "mibm_register_mesh_": (None, [_I, C.c_void_p]),
    "mibm_register_scalar_": (None, [_I, C.c_void_p]),
    "mibm_register_int_": (None, [_I, C.c_void_p]),
    "mibm_init_": (None, []),
    "mibm_sync_from_host_": (None, [_L]),
    "mibm_sync_to_host_": (None, [_L]),
    "mibm_device_count_": (C.c_int, []),
    "mibm_launch_count_": (C.c_ulonglong, []),
    "mibm_select_device_": (C.c_int, [_I]),
    "mibm_timer_mark_": (None, [_I]),
    "mibm_timer_ms_": (C.c_double, [_I, _I]),
    "mibm_profile_": (None, [_I]),
    "mibm_profile_count_": (C.c_int, []),
    "mibm_profile_get_": (C.c_int, [_I, C.c_char_p, _I, _D, C.POINTER(C.c_longlong)]),
    "mibm_solxi_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p]),
    "mibm_set_precision_": (None, [_I, _I]),
    "mibm_set_tma_": (None, [_I]),
    "mibm_set_fused_uvw_": (None, [_I]),
    "mibm_bounds_check_": (C.c_int, []),
    "mibm_bounds_selftest_": (C.c_int, []),
    "mibm_set_graphs_": (None, [_I]),
    "mibm_autotune_": (C.c_int, []),
    "mibm_autotune_get_": (C.c_int, [C.c_void_p]),
    "mibm_autotune_save_": (C.c_int, [C.c_char_p]),
    "mibm_autotune_load_": (C.c_int, [C.c_char_p]),
    "mibm_batch_create_": (C.c_int, [C.c_void_p, _I]),
    "mibm_batch_step_": (C.c_int, [_I, _I]),
    "mibm_batch_destroy_": (C.c_int, [_I]),
    "mibm_batch_add_": (C.c_int, [_I, _I]),
    "mibm_batch_remove_": (C.c_int, [_I, _I]),
    "mibm_batch_set_launch_": (C.c_int, [_I, _I]),
    "mibm_divergence_max_": (C.c_double, []),
    "mibm_set_remesh_callback_": (None, [C.c_void_p, C.c_void_p]),
    "mibm_pin_host_": (C.c_int, [_I]),
    "mibm_remesh_count_": (C.c_int, []),
    "mibm_remesh_mesh": (C.c_int, [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 11 + [C.c_double, C.c_void_p]),
    "mibm_remesh_builtin_": (C.c_int, [C.c_void_p]),
    "mibm_remesh_stats_": (C.c_int, [C.c_void_p]),
    "mibm_diagnostics_": (C.c_int, [C.c_void_p]),
    "mibm_set_diagnostics_": (None, [_I]),
    "mibm_diagnostics_get_": (C.c_int, [C.c_void_p]),
    "solxi_": (None, [_D]),
    "solxj_": (None, [_D]),
    "solxk_": (None, [C.c_void_p, _D]),
    "interp_": (None, [C.c_void_p, C.c_void_p, _I, _I, _I, _I, _I, _I]),
    "mibm_hit_modes_": (C.c_int, []),
    "mibm_hit_bhat_": (None, [C.c_void_p, _I]),
    "mibm_hit_rng_": (None, [C.c_void_p, _I]),
    "mibm_selftest_": (C.c_int, []),
}
VOID_ROUTINES = [
    "tschem_", "hdnl1_", "hdnl2_", "hdnl3_", "hdnlte_", "invtr1_", "invtr2_", "invtr3_",
    "invtrte_", "divg_", "phcalc_", "updvp_", "prcalc_", "findcentroidindices_",
    "mlsweight_", "mlsforce_", "velforce_", "tempforce_", "findprobeindices_",
    "mls_heatflux_", "apply_stefancondition_", "tagcells_", "particle_", "cfl_", "get_dt_",
    "tagcells_initial_", "calchitrandomforce_", "calcabc_hitforce_", "mibm_linear_hit_force_",
    "mls_structloads_", "update_part_pos_",
]
for _n in VOID_ROUTINES:
    SIGNATURES[_n] = (None, [])


#: C type of the host remesher passed to mibm_set_remesh_callback_
REMESH_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)


def header_symbols() -> list[str]:
    """Every function name declared in include/mibm.h."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"typedef[^;]*;", "", text)
    return re.findall(r"\b([a-z_][a-z0-9_]*)\s*\((?:[^;{]*?)\)\s*;", text)


class Lib:
    """A loaded library exporting the mibm C-ABI."""

    def __init__(self, path: str):
        self.path = path
        self.dll = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(self.dll, name)
            fn.restype = res
            fn.argtypes = args
        self._extra()

    def _extra(self) -> None:
        pass

    def __getattr__(self, name):
        return getattr(self.dll, name)

    def profile(self) -> dict[str, tuple[float, int]]:
        """Per-kernel totals of the bound context: name -> (ms, launches)."""
        out = {}
        n = self.dll.mibm_profile_count_()
        buf = C.create_string_buffer(128)
        for i in range(n):
            ms, cnt = C.c_double(), C.c_longlong()
            self.dll.mibm_profile_get_(C.byref(C.c_int(i)), buf, C.byref(C.c_int(128)), C.byref(ms), C.byref(cnt))
            out[buf.value.decode()] = (ms.value, cnt.value)
        return out

    def check(self, what: str = "") -> None:
        st = self.dll.mibm_last_status_()
        if st != 0:
            msg = self.dll.mibm_last_message()
            raise RuntimeError(f"{os.path.basename(self.path)}: {what} failed with status {st}: "
                               f"{msg.decode() if msg else ''}")


def ref_int(v: int):
    return C.byref(C.c_int(int(v)))


def ref_double(v: float):
    return C.byref(C.c_double(float(v)))


def ref_ll(v: int):
    return C.byref(C.c_longlong(int(v)))
