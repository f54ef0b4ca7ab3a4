"""ctypes binding of liba2c_gpp.so (include/a2c_gpp.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "liba2c_gpp.so"

A2C_OK = 0
A2C_ERR_INVALID = 1
A2C_ERR_CUDA = 2
A2C_ERR_NOMEM = 3
A2C_ERR_NEIGHBOR_OVERFLOW = 4
A2C_ERR_NONFINITE = 5
A2C_ERR_STATE = 6
A2C_ERR_TIMEOUT = 7
A2C_ERR_NO_DEVICE = 8
A2C_ERR_LISTS_STALE = 9

A2C_FP64 = 0
A2C_MIXED = 1

A2C_PAIRS_BOTH_SIDES = 0
A2C_PAIRS_ONCE = 1

LIST_PDPD, LIST_PDH, LIST_HPD, LIST_HH, LIST_HH1 = range(5)

CONVERGED_GATOL = 3
CONVERGED_STALLED = 6
DIVERGED_MAXITS = -2
DIVERGED_NAN = -4
DIVERGED_MAXFCN = -5
DIVERGED_LS_FAILURE = -6


class GppParams(C.Structure):
    _fields_ = [
        ("nPd", C.c_int), ("nH", C.c_int),
        ("T", C.c_double), ("QWp", C.c_double), ("eps", C.c_double), ("rc", C.c_double), ("a_Pd", C.c_double),
        ("box", C.c_double * 3), ("periodic", C.c_int * 3),
        ("coe_Pd", C.c_double * 4), ("coe_H", C.c_double * 4),
        ("precision", C.c_int), ("device", C.c_int),
    ]


class LbfgsParams(C.Structure):
    _fields_ = [
        ("m", C.c_int), ("max_it", C.c_int), ("max_fev", C.c_int), ("max_ls", C.c_int),
        ("gatol", C.c_double), ("c1", C.c_double), ("init_step", C.c_double), ("sigma_lb", C.c_double),
        ("f_noise", C.c_double), ("polish", C.c_int), ("stall_window", C.c_int), ("stall_rtol", C.c_double),
        ("max_step", C.c_double),
    ]


class LatticeSpec(C.Structure):
    _fields_ = [
        ("ncell", C.c_int * 3), ("a", C.c_double), ("periodic", C.c_int * 3),
        ("pos_std", C.c_double), ("sigma_lo", C.c_double), ("sigma_hi", C.c_double),
        ("x_mode", C.c_int), ("x_center", C.c_double), ("x_half", C.c_double),
        ("x_matrix", C.c_double), ("x_nucleus", C.c_double), ("nucleus_radius", C.c_double),
        ("interface_width", C.c_double), ("xLb", C.c_double), ("xUb", C.c_double),
        ("seed", C.c_uint64),
    ]


class SnapshotDesc(C.Structure):
    _fields_ = [("prefix", C.c_char_p), ("format", C.c_int), ("precision", C.c_int), ("axes", C.c_double * 9),
                ("origin", C.c_double * 3), ("periodic", C.c_int * 3), ("lattice_id", C.c_int)]


class Input(C.Structure):
    _fields_ = [("T", C.c_double), ("nu", C.c_double), ("Qm", C.c_double), ("t_subsurf", C.c_double),
                ("mubd", C.c_double), ("eps", C.c_double), ("rc", C.c_double), ("potential_file", C.c_char * 256),
                ("dt", C.c_double), ("max_time", C.c_double), ("cfl", C.c_double), ("max_its", C.c_int),
                ("output_format", C.c_int), ("output_precision", C.c_int), ("output_frequency", C.c_int),
                ("output_interval", C.c_double), ("output_prefix", C.c_char * 256),
                ("output_solution", C.c_char * 256), ("lattice_axes", C.c_double * 9),
                ("lattice_origin", C.c_double * 3), ("lattice_periodic", C.c_int * 3), ("n_assignments", C.c_int),
                ("n_used", C.c_int)]


class Geometry(C.Structure):
    _fields_ = [("type", C.c_int), ("order", C.c_int), ("inclusion", C.c_int), ("exterior", C.c_int),
                ("p", C.c_double * 12)]


class SiteGroup(C.Structure):
    _fields_ = [("l", C.c_double * 3), ("materialid", C.c_int), ("tag", C.c_int), ("atomic_frequency", C.c_double),
                ("mean_displacement", C.c_double * 3), ("x", C.c_double)]


class LatticeDesc(C.Structure):
    _fields_ = [("abc", C.c_double * 9), ("origin", C.c_double * 3), ("periodic", C.c_int * 3),
                ("dmin", C.c_double), ("nsites", C.c_int), ("sites", C.POINTER(SiteGroup)), ("ngeom", C.c_int),
                ("geoms", C.POINTER(Geometry))]


class Region(C.Structure):
    _fields_ = [("lattice_id", C.c_int), ("materialid", C.c_int), ("siteid", C.c_int), ("tag", C.c_int),
                ("atomic_frequency", C.c_double), ("mean_displacement", C.c_double * 3), ("x", C.c_double),
                ("ngeom", C.c_int), ("geoms", C.POINTER(Geometry))]


class LatticeSites(C.Structure):
    _fields_ = [("capacity", C.c_int64), ("count", C.c_int64), ("q", C.c_void_p), ("q0", C.c_void_p),
                ("l", C.c_void_p), ("siteid", C.c_void_p), ("matid", C.c_void_p), ("tag", C.c_void_p),
                ("sigma", C.c_void_p), ("x", C.c_void_p)]


class DmdParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("nu", C.c_double), ("Qm", C.c_double), ("xLb", C.c_double),
                ("xUb", C.c_double), ("x_bd", C.c_double), ("gamma_bd", C.c_double), ("lbfgs", LbfgsParams),
                ("neighbor_update", C.c_int), ("host_steps", C.c_int)]


_lib = None

P = C.c_void_p
D = C.c_double
I = C.c_int


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA evaluator has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    sig = {
        "a2c_gpp_default_params": (None, [C.POINTER(GppParams)]),
        "a2c_lbfgs_default_params": (None, [C.POINTER(LbfgsParams)]),
        "a2c_status_string": (C.c_char_p, [I]),
        "a2c_gpp_create": (I, [C.POINTER(GppParams), C.POINTER(P)]),
        "a2c_gpp_destroy": (I, [P]),
        "a2c_gpp_stream": (P, [P]),
        "a2c_gpp_set_precision": (I, [P, I]),
        "a2c_gpp_synchronize": (I, [P]),
        "a2c_gpp_set_threads_per_site": (I, [P, I]),
        "a2c_gpp_set_pair_mode": (I, [P, I]),
        "a2c_gpp_set_neighbor_lists": (I, [P] * 13),
        "a2c_gpp_get_pair_mode": (I, [P, C.POINTER(C.c_int)]),
        "a2c_gpp_set_occupancy": (I, [P, P]),
        "a2c_gpp_get_occupancy": (I, [P, P]),
        "a2c_gpp_set_state": (I, [P, P]),
        "a2c_gpp_get_state": (I, [P, P]),
        "a2c_gpp_build_neighbors": (I, [P, P, C.POINTER(I)]),
        "a2c_gpp_neighbor_total": (I, [P, I, C.POINTER(C.c_int64)]),
        "a2c_gpp_set_neighbor_skin": (I, [P, D]),
        "a2c_snapshot_begin": (I, [C.POINTER(SnapshotDesc)]),
        "a2c_input_read": (I, [C.c_char_p, C.POINTER(Input), C.c_char_p, I]),
        "a2c_input_apply": (I, [C.POINTER(Input), C.POINTER(GppParams)]),
        "a2c_input_lattice": (I, [C.c_char_p, I, C.POINTER(LatticeDesc), C.POINTER(SiteGroup), I,
                                  C.POINTER(Geometry), I, C.c_char_p, I]),
        "a2c_lattice_build": (I, [C.POINTER(LatticeDesc), C.POINTER(LatticeSites), C.c_char_p, I]),
        "a2c_lattice_conflicts": (I, [P, C.c_int64, P, C.c_int64, D, P, C.POINTER(C.c_int64)]),
        "a2c_lattice_apply_region": (I, [C.POINTER(Region), C.POINTER(LatticeSites), C.c_char_p, I]),
        "a2c_snapshot_write_lattice": (I, [C.POINTER(SnapshotDesc), I, D, C.POINTER(LatticeSites), P,
                                           C.POINTER(C.c_char_p), I]),
        "a2c_input_regions": (I, [C.c_char_p, C.POINTER(Region), I, C.POINTER(Geometry), I, C.POINTER(C.c_int),
                                  C.c_char_p, I]),
        "a2c_input_material_names": (I, [C.c_char_p, P, I, I, C.POINTER(C.c_int), C.c_char_p, I]),
        "a2c_snapshot_write": (I, [C.POINTER(SnapshotDesc), I, D, I, I, P, P, P, P, P, P]),
        "a2c_gpp_snapshot_async": (I, [P, C.POINTER(SnapshotDesc), I, D, P, P, P, P]),
        "a2c_gpp_snapshot_wait": (I, [P]),
        "a2c_gpp_update_neighbors": (I, [P, P, C.POINTER(I), C.POINTER(I)]),
        "a2c_gpp_get_neighbors": (I, [P, I, P, P]),
        "a2c_gpp_get_shell_counts": (I, [P, P]),
        "a2c_gpp_eval": (I, [P, P, C.POINTER(D), P]),
        "a2c_gpp_eval_device": (I, [P, P, P, P]),
        "a2c_gpp_profile_eval": (I, [P, P, P, P, P]),
        "a2c_gpp_get_density": (I, [P, P]),
        "a2c_gpp_bounds": (I, [P, P, P]),
        "a2c_gpp_eam_eval": (I, [P, I, P, C.c_int64, P]),
        "a2c_gpp_minimize": (I, [P, P, C.POINTER(LbfgsParams), C.POINTER(D), C.POINTER(I), C.POINTER(I),
                                 C.POINTER(D), C.POINTER(I)]),
        "a2c_gpp_chem_potential": (I, [P, D, P, P]),
        "a2c_gpp_minimize_stats": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(D)]),
        "a2c_gpp_apply_dirichlet": (I, [P, P, I, D, D, P, P]),
        "a2c_gpp_diffuse": (I, [P, D, D, D, D, D, P, P, P]),
        "a2c_gpp_macro_results": (I, [P, P, P, I, C.POINTER(D), C.POINTER(D)]),
        "a2c_lattice_fcc": (I, [C.POINTER(LatticeSpec), P, P, P]),
        "a2c_lattice_fcc_device": (I, [C.POINTER(LatticeSpec), P, P, P, P]),
        "a2c_gpp_peak_flops": (I, [I, I, C.POINTER(D)]),
        "a2c_gpp_dmd_run": (I, [P, P, P, P, P, P, I, P, I, C.POINTER(DmdParams), I, P, P, P, P]),
        "a2c_restart_write": (I, [C.c_char_p, I, I, P, P, P, P, I, D]),
        "a2c_restart_read": (I, [C.c_char_p, I, I, D, D, P, P, P, P]),
        "a2c_gpp_batch_create": (I, [C.POINTER(GppParams), I, C.POINTER(C.c_void_p)]),
        "a2c_gpp_batch_destroy": (I, [P]),
        "a2c_gpp_batch_info": (I, [P, C.POINTER(I), C.POINTER(C.c_int64)]),
        "a2c_gpp_batch_set_occupancy": (I, [P, P]),
        "a2c_gpp_batch_build_neighbors": (I, [P, P, C.POINTER(I)]),
        "a2c_gpp_batch_set_threads_per_site": (I, [P, I]),
        "a2c_gpp_batch_set_graphs": (I, [P, I]),
        "a2c_gpp_batch_eval": (I, [P, P, P, P]),
        "a2c_gpp_batch_minimize": (I, [P, P, C.POINTER(LbfgsParams), P, P, P, P, P, P, P]),
        "a2c_gpp_batch_stats": (I, [P, C.POINTER(I), C.POINTER(D)]),
        "a2c_gpp_batch_autotune": (I, [P, P, I, C.POINTER(I), P]),
        "a2c_gpp_autotune": (I, [P, I, C.POINTER(I), P]),
        "a2c_gpp_set_tile": (I, [P, I, I, I]),
        "a2c_gpp_get_tile": (I, [P, P]),
        "a2c_gpp_autotune_tile": (I, [P, I, P, P]),
        "a2c_gpp_batch_set_tile": (I, [P, I, I, I]),
        "a2c_gpp_batch_get_tile": (I, [P, P]),
        "a2c_gpp_batch_autotune_tile": (I, [P, P, I, P, P]),
        "a2c_gpp_set_minimizer": (I, [P, I]),
        "a2c_eam_analytic": (I, [I, P, C.c_int64, P, P]),
        "a2c_mixed_table_eval": (I, [I, P, C.c_int64, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names of the C ABI functions this binding expects the library to export."""
    return ["a2c_gpp_default_params", "a2c_lbfgs_default_params", "a2c_status_string", "a2c_gpp_create",
            "a2c_gpp_destroy", "a2c_gpp_stream", "a2c_gpp_set_precision", "a2c_gpp_synchronize",
            "a2c_gpp_set_threads_per_site", "a2c_gpp_set_pair_mode", "a2c_gpp_get_pair_mode", "a2c_gpp_set_neighbor_lists",
            "a2c_gpp_set_occupancy",
            "a2c_gpp_get_occupancy", "a2c_gpp_set_state", "a2c_gpp_get_state", "a2c_gpp_build_neighbors",
            "a2c_gpp_neighbor_total", "a2c_gpp_set_neighbor_skin", "a2c_gpp_update_neighbors", "a2c_snapshot_begin", "a2c_input_read", "a2c_input_apply",
            "a2c_input_lattice", "a2c_lattice_build", "a2c_lattice_conflicts", "a2c_lattice_apply_region",
            "a2c_input_regions", "a2c_snapshot_write_lattice", "a2c_input_material_names",
            "a2c_snapshot_write", "a2c_gpp_snapshot_async", "a2c_gpp_snapshot_wait", "a2c_gpp_get_neighbors", "a2c_gpp_get_shell_counts", "a2c_gpp_eval",
            "a2c_gpp_eval_device", "a2c_gpp_profile_eval", "a2c_gpp_get_density", "a2c_gpp_eam_eval", "a2c_gpp_bounds", "a2c_gpp_minimize",
            "a2c_gpp_chem_potential", "a2c_gpp_minimize_stats", "a2c_gpp_apply_dirichlet", "a2c_gpp_diffuse", "a2c_gpp_macro_results",
            "a2c_lattice_fcc", "a2c_gpp_peak_flops", "a2c_gpp_dmd_run", "a2c_restart_write", "a2c_restart_read",
            "a2c_gpp_batch_create", "a2c_gpp_batch_destroy", "a2c_gpp_batch_info", "a2c_gpp_batch_set_occupancy",
            "a2c_gpp_batch_build_neighbors", "a2c_gpp_batch_set_threads_per_site", "a2c_gpp_batch_set_graphs",
            "a2c_gpp_batch_eval", "a2c_gpp_batch_minimize", "a2c_gpp_batch_stats", "a2c_gpp_batch_autotune",
            "a2c_gpp_autotune", "a2c_gpp_set_minimizer", "a2c_eam_analytic", "a2c_mixed_table_eval",
            "a2c_lattice_fcc_device", "a2c_gpp_set_tile", "a2c_gpp_get_tile", "a2c_gpp_autotune_tile",
            "a2c_gpp_batch_set_tile", "a2c_gpp_batch_get_tile", "a2c_gpp_batch_autotune_tile"]


class A2CError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = lib().a2c_status_string(status).decode()
        super().__init__(f"{where}: status {status} ({msg})")
        self.status = status


def check(status: int, where: str) -> None:
    if status != A2C_OK:
        raise A2CError(status, where)


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays crossing the C ABI must be contiguous"
    return a.ctypes.data
