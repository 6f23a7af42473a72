"""Loader and ctypes declarations of libemcgpu (include/emcgpu.h).

The engine lives in the shared library built from viennaemc_gb300/csrc/ for
sm_103a.  There is no fallback: if the library cannot be built or loaded the
import of the engine API raises.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_PATH = os.path.join(PKG, "libemcgpu.so")
SOURCES = ["emcg_core.cu", "emcg_bulk.cu", "emcg_device.cu", "emcg_poisson.cu", "emcg_p2p.cu"]
HEADERS = ["emcg_common.cuh", "emcg_host.h", "emcg_model.h", "emcg_poisson.cuh", "emcg_rates.cuh",
           "emcg_p2p.cuh", "emcg_exp.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

MAX_VALLEYS, MAX_DEG, MAX_MECH, MAX_NF, MAX_REGIONS = 4, 8, 32, 8, 16
MAX_TABLESETS = MAX_VALLEYS * MAX_REGIONS
FP64, FP32 = 0, 1
(MECH_ACOUSTIC, MECH_ZERO_IV_ABS, MECH_ZERO_IV_EMI, MECH_FIRST_IV_ABS, MECH_FIRST_IV_EMI,
 MECH_COULOMB) = range(6)
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "timeout",
          -4: "not converged", -5: "out of table", -6: "replay mismatch", -7: "capacity"}


class EmcgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(INCLUDE, "emcgpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libemcgpu.so for sm_103a (translation units in parallel)."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = _nvcc()
    objdir = os.path.join(PKG, "_build")
    os.makedirs(objdir, exist_ok=True)
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
             f"-I{CSRC}"]
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(objdir, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{out}")
        if verbose and out:
            print(out)
    tmp = LIB_PATH + ".tmp"
    subprocess.run([nvcc, ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class ValleyDesc(C.Structure):
    _fields_ = [("deg", C.c_int32), ("pad_", C.c_int32), ("rel_mass", C.c_double * 3),
                ("particle_mass", C.c_double), ("alpha", C.c_double), ("bottom", C.c_double),
                ("rot", (C.c_double * 9) * MAX_DEG)]


class MechDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("valley", C.c_int32), ("final_valley", C.c_int32),
                ("n_final", C.c_int32), ("shift", C.c_double), ("coulomb_sc2", C.c_double),
                ("final_sub", (C.c_int32 * MAX_NF) * MAX_DEG)]


class TablesetDesc(C.Structure):
    _fields_ = [("valley", C.c_int32), ("region", C.c_int32), ("n_tables", C.c_int32),
                ("pad_", C.c_int32), ("mech", C.c_int32 * MAX_MECH), ("tau_max", C.c_double)]


SURFACE_SPECULAR, SURFACE_CONSTANT, SURFACE_ROUGHNESS = 0, 1, 2  # emcg_model_desc.surface_kind


class ModelDesc(C.Structure):
    _fields_ = [("n_valleys", C.c_int32), ("n_mechs", C.c_int32), ("n_tablesets", C.c_int32),
                ("n_levels", C.c_int32), ("max_energy", C.c_double), ("grain_tau", C.c_double),
                ("valleys", C.POINTER(ValleyDesc)), ("mechs", C.POINTER(MechDesc)),
                ("tablesets", C.POINTER(TablesetDesc)), ("tables", C.POINTER(C.c_double)),
                ("region_doping", C.c_double * MAX_REGIONS), ("grain", C.c_int32),
                ("grain_pad_", C.c_int32), ("grain_transmission", C.c_double),
                ("surface_kind", C.c_int32 * 4), ("surface_param", C.c_double * 4)]


class EnsembleDesc(C.Structure):
    _fields_ = [("model", C.c_int32), ("pad_", C.c_int32), ("capacity", C.c_int64),
                ("field", C.c_double * 3), ("charge", C.c_double), ("field_dir", C.c_double * 3),
                ("box", C.c_double * 3), ("dt", C.c_double), ("seed", C.c_uint64),
                ("stream", C.c_uint32), ("flags", C.c_uint32)]


class StateF32Desc(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_float)) for n in
                ("kx", "ky", "kz", "px", "py", "pz", "energy", "tau", "grain_tau")] + \
               [("meta", C.POINTER(C.c_uint32)), ("n", C.c_int64)]


class StateDesc(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in
                ("kx", "ky", "kz", "px", "py", "pz", "energy", "tau", "grain_tau")] + \
               [(n, C.POINTER(C.c_int32)) for n in ("valley", "sub", "region")] + \
               [("n", C.c_int64)]


_lib = None


def lib():
    """Load libemcgpu (building it first if its sources are newer)."""
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    i32, i64, u32, d, vp = C.c_int32, C.c_int64, C.c_uint32, C.c_double, C.c_void_p
    P = C.POINTER
    L.emcg_last_error.restype = C.c_char_p
    L.emcg_version.restype = i32
    L.emcg_bulk_create.restype = i32
    L.emcg_bulk_create.argtypes = [P(ModelDesc), i32, P(EnsembleDesc), i32, i32, P(vp)]
    L.emcg_destroy.restype = i32
    L.emcg_destroy.argtypes = [vp]
    L.emcg_bulk_update_ensemble.restype = i32
    L.emcg_bulk_update_ensemble.argtypes = [vp, i32, P(EnsembleDesc)]
    L.emcg_set_state.restype = i32
    L.emcg_set_state.argtypes = [vp, i32, P(StateDesc)]
    L.emcg_get_state.restype = i32
    L.emcg_get_state.argtypes = [vp, i32, P(StateDesc)]
    L.emcg_set_state_f32.restype = i32
    L.emcg_set_state_f32.argtypes = [vp, i32, P(StateF32Desc)]
    L.emcg_get_state_f32.restype = i32
    L.emcg_get_state_f32.argtypes = [vp, i32, P(StateF32Desc)]
    L.emcg_bulk_step_from_host.restype = i32
    L.emcg_bulk_step_from_host.argtypes = [vp, i32, P(StateF32Desc), i32, u32, P(C.c_double)]
    L.emcg_num_particles.restype = i64
    L.emcg_num_particles.argtypes = [vp, i32]
    L.emcg_bulk_init.restype = i32
    L.emcg_bulk_init.argtypes = [vp, i32, i64, P(i64), P(i64), P(d), d]
    L.emcg_bulk_step.restype = i32
    L.emcg_bulk_step.argtypes = [vp, i32, u32, P(d)]
    L.emcg_set_replay.restype = i32
    L.emcg_set_replay.argtypes = [vp, P(C.c_uint64), i64, P(i64), i64]
    L.emcg_last_kernel_ms.restype = i32
    L.emcg_last_kernel_ms.argtypes = [vp, P(d)]
    L.emcg_set_launch.restype = i32
    L.emcg_set_launch.argtypes = [vp, i32, i32]
    L.emcg_get_launch.restype = i32
    L.emcg_get_launch.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.emcg_set_scatter_mode.restype = i32
    L.emcg_set_scatter_mode.argtypes = [vp, i32]
    L.emcg_set_pass_actions.restype = i32
    L.emcg_set_pass_actions.argtypes = [vp, i32]
    L.emcg_get_pass_actions.restype = i32
    L.emcg_get_pass_actions.argtypes = [vp, C.POINTER(i32)]
    L.emcg_set_occupancy.restype = i32
    L.emcg_set_occupancy.argtypes = [vp, i32]
    L.emcg_host_alloc.restype = i32
    L.emcg_host_alloc.argtypes = [i64, C.POINTER(vp)]
    L.emcg_host_free.restype = i32
    L.emcg_host_free.argtypes = [vp]
    L.emcg_drift_kat.restype = i32
    L.emcg_drift_kat.argtypes = [vp, i32, i64, P(i32), P(d), P(d), P(d), P(d), P(d)]
    L.emcg_grain_kat.restype = i32
    L.emcg_grain_kat.argtypes = [vp, i64, P(d), u32]
    for name, args in _EXTRA_DECLS:
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype = i32
            fn.argtypes = args


_EXTRA_DECLS: list = []


def check(status: int) -> None:
    if status != 0:
        msg = lib().emcg_last_error().decode(errors="replace")
        raise EmcgError(status, msg)


# ---- device engine ---------------------------------------------------------------
PM_NGP, PM_CIC, PM_NEC, PM_NEC_VWD = 0, 1, 2, 3
CONTACT_OHMIC, CONTACT_SCHOTTKY, CONTACT_GATE = 0, 1, 2
GRID_POTENTIAL, GRID_EX, GRID_EY, GRID_NRPART, GRID_CONC = range(5)


class DeviceDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("hx", C.c_double), ("hy", C.c_double),
                ("max_x", C.c_double), ("max_y", C.c_double), ("width", C.c_double),
                ("temperature", C.c_double), ("ni", C.c_double), ("eps_r", C.c_double),
                ("doping", C.POINTER(C.c_double)), ("region", C.POINTER(C.c_int32)),
                ("boundary_contact", C.POINTER(C.c_int32) * 4), ("n_contacts", C.c_int32),
                ("pad_", C.c_int32), ("contact_type", C.POINTER(C.c_int32)),
                ("contact_voltage", C.POINTER(C.c_double)),
                ("contact_param", C.POINTER(C.c_double))]


class DeviceConfig(C.Structure):
    _fields_ = [("pm_scheme", C.c_int32), ("tau_region_is_valley", C.c_int32),
                ("capacity", C.c_int64), ("dt", C.c_double), ("charge", C.c_double),
                ("carriers_per_particle", C.c_double), ("seed", C.c_uint64),
                ("stream", C.c_uint32), ("poisson_max_cycles", C.c_int32),
                ("poisson_rtol", C.c_double), ("poisson_smooth", C.c_int32),
                ("poisson_fp32", C.c_int32), ("round_expected", C.c_int32),
                ("pad_", C.c_int32), ("poisson_update_tol", C.c_double)]


def _i32p():
    return C.POINTER(C.c_int32)


_EXTRA_DECLS.extend([
    ("emcg_device_create", [C.POINTER(ModelDesc), C.POINTER(DeviceDesc), C.POINTER(DeviceConfig),
                            C.c_int32, C.POINTER(C.c_void_p)]),
    ("emcg_device_set_grid", [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    ("emcg_device_get_grid", [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    ("emcg_device_poisson", [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                             C.POINTER(C.c_int32)]),
    ("emcg_device_efield", [C.c_void_p]),
    ("emcg_device_surface_kat", [C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.c_uint32]),
    ("emcg_device_move", [C.c_void_p, C.c_uint32, C.POINTER(C.c_int32)]),
    ("emcg_device_contacts", [C.c_void_p, C.c_uint32, C.POINTER(C.c_int32)]),
    ("emcg_device_assign", [C.c_void_p]),
    ("emcg_device_step", [C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_int32)]),
    ("emcg_device_init", [C.c_void_p, C.c_int32, C.c_int32]),
    ("emcg_device_set_replay", [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64), C.c_int64,
                                C.POINTER(C.c_int64), C.c_int64]),
    ("emcg_device_timing", [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("emcg_device_poisson_counts", [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("emcg_device_poisson_mode", [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    ("emcg_device_set_poisson_cluster", [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    ("emcg_device_set_poisson", [C.c_void_p, C.c_double, C.c_int32, C.c_double]),
    ("emcg_device_step_many", [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_uint32,
                               C.POINTER(C.POINTER(C.c_int32))]),
    ("emcg_bulk_set_graph", [C.c_void_p, C.c_int32]),
    ("emcg_bulk_autotune", [C.c_void_p, C.c_int32, C.c_uint32, C.POINTER(C.c_int32),
                            C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("emcg_poisson_solve_noalloc", [C.POINTER(DeviceDesc), C.c_void_p, C.c_void_p, C.c_int32,
                                    C.c_int32, C.c_double, C.c_int32, C.c_void_p,
                                    C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    ("emcg_update_rates", [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]),
    ("emcg_get_rates", [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("emcg_p2p_coulomb", [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_int32,
                          C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    ("emcg_bulk_set_coulomb", [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_int32]),
    ("emcg_bulk_set_fixed_charges", [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64]),
    ("emcg_bulk_get_coulomb", [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
])
