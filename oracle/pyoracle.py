"""ctypes bindings for the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the engine in viennaemc_gb300/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

ACOUSTIC, ZERO_IV_ABS, ZERO_IV_EMI, FIRST_IV_ABS, FIRST_IV_EMI, COULOMB = range(6)
RNG_MT, RNG_PHILOX, RNG_REPLAY, RNG_PHILOX32 = range(4)

_lib = None


def build(force: bool = False) -> None:
    """Compile liboracle.so with the Makefile beside this file."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


class Particles(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in
                ("kx", "ky", "kz", "px", "py", "pz", "E", "tau", "gtau")] + \
               [(n, C.POINTER(C.c_int32)) for n in ("valley", "sub", "region")] + \
               [("n", C.c_int64)]


class Rng(C.Structure):
    _fields_ = [("mode", C.c_int32), ("stream", C.c_uint32), ("seed", C.c_uint64),
                ("mt", C.c_uint64 * 312), ("mt_idx", C.c_int32), ("pad_", C.c_int32),
                ("words", C.POINTER(C.c_uint64)), ("nwords", C.c_int64), ("pos", C.c_int64),
                ("rec", C.POINTER(C.c_uint64)), ("rec_cap", C.c_int64), ("rec_n", C.c_int64),
                ("rec_overflow", C.c_int32), ("pad2_", C.c_int32)]


def _declare(L):
    d, i32, i64, u32, u64, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_void_p
    P = C.POINTER
    L.oc_model_new.restype = vp
    L.oc_model_new.argtypes = [d, d, d, d, d, i32, d]
    L.oc_model_free.argtypes = [vp]
    L.oc_add_valley.restype = i32
    L.oc_add_valley.argtypes = [vp, P(d), d, i32, d, d]
    L.oc_set_frame.restype = i32
    L.oc_set_frame.argtypes = [vp, i32, i32, P(d), P(d), P(d)]
    L.oc_add_mech.restype = i32
    L.oc_add_mech.argtypes = [vp, i32, i32, i32, d, d, i32, P(i32), P(i32), i32]
    L.oc_set_region_doping.restype = i32
    L.oc_set_region_doping.argtypes = [vp, i32, d]
    L.oc_set_grain.restype = i32
    L.oc_set_grain.argtypes = [vp, d, d]
    L.oc_set_surface.restype = i32
    L.oc_set_surface.argtypes = [vp, i32, i32, d]
    L.oc_build_tables.restype = i32
    L.oc_build_tables.argtypes = [vp]
    for fn in ("oc_get_raw_table", "oc_get_norm_table"):
        getattr(L, fn).restype = i32
        getattr(L, fn).argtypes = [vp, i32, i32, i32, P(d)]
    L.oc_set_raw_tables.restype = i32
    L.oc_set_raw_tables.argtypes = [vp, i32, i32, P(d)]
    L.oc_p2p_pair.restype = None
    L.oc_p2p_pair.argtypes = [d, d, d, d, d, d, d, d, d, P(d)]
    L.oc_p2p_coulomb.restype = i32
    L.oc_p2p_coulomb.argtypes = [P(d), P(d), C.c_int64, d, d, i32, P(d), P(d), i32]
    L.oc_bulk_run_coulomb.restype = i32
    L.oc_bulk_run_coulomb.argtypes = [vp, vp, d, d, P(d), P(d), P(d), P(d), P(d), C.c_int64, d, d,
                                      i32, C.c_uint64, C.c_uint32, C.c_uint32, i32, i32, P(d)]
    L.oc_n_tables.restype = i32
    L.oc_n_tables.argtypes = [vp, i32, i32]
    L.oc_table_mech.restype = i32
    L.oc_table_mech.argtypes = [vp, i32, i32, i32]
    L.oc_get_tau.restype = d
    L.oc_get_tau.argtypes = [vp, i32, i32]
    L.oc_valley_consts.argtypes = [vp, i32, P(d)]
    L.oc_valley_rot.argtypes = [vp, i32, P(d)]
    L.oc_energy.restype = d
    L.oc_energy.argtypes = [vp, i32, P(d)]
    L.oc_norm_wave_vec.restype = d
    L.oc_norm_wave_vec.argtypes = [vp, i32, d]
    L.oc_velocity.argtypes = [vp, i32, i32, P(d), d, P(d)]
    L.oc_drift.argtypes = [vp, d, P(d), P(d), i32, i32, P(d), i32, P(d)]
    L.oc_mt_seed.argtypes = [P(Rng), u64]
    L.oc_mt_next.restype = u64
    L.oc_mt_next.argtypes = [P(Rng)]
    L.oc_philox4x32_10.argtypes = [P(u32), P(u32), P(u32)]
    L.oc_canonical.restype = d
    L.oc_canonical.argtypes = [u64]
    L.oc_bulk_step.restype = i32
    L.oc_bulk_step.argtypes = [vp, P(Particles), d, P(d), P(d), P(Rng), u32, P(i64)]
    L.oc_bulk_run_philox.restype = i32
    L.oc_bulk_run_philox.argtypes = [vp, P(Particles), d, P(d), P(d), P(d), u64, u32, u32,
                                     i32, i32, P(d), i32]
    L.oc_observables.argtypes = [vp, P(Particles), P(d), P(d)]
    L.oc_bulk_init.restype = i64
    L.oc_bulk_init.argtypes = [vp, P(d), P(d), d, P(Rng), P(Particles), i64]
    L.oc_init_particle.argtypes = [vp, P(i64), P(i64), P(d), i32, i32, d, P(Rng),
                                   P(Particles), i64, i32]
    if hasattr(L, "oc_device_declare"):
        pass


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def lptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def darr(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


STATE_F = ("kx", "ky", "kz", "px", "py", "pz", "E", "tau", "gtau")
STATE_I = ("valley", "sub", "region")


class State:
    """Structure-of-arrays particle state held in numpy (float64 / int32)."""

    def __init__(self, n: int):
        for f in STATE_F:
            setattr(self, f, np.zeros(n, np.float64))
        for f in STATE_I:
            setattr(self, f, np.zeros(n, np.int32))
        self.n = n

    @classmethod
    def from_dict(cls, d: dict) -> "State":
        n = len(d["E"])
        s = cls(n)
        for f in STATE_F:
            getattr(s, f)[:] = d[f]
        for f in STATE_I:
            getattr(s, f)[:] = d[f]
        return s

    def to_dict(self) -> dict:
        return {f: getattr(self, f).copy() for f in STATE_F + STATE_I}

    def copy(self) -> "State":
        return State.from_dict(self.to_dict())

    def resize(self, n: int) -> "State":
        s = State(n)
        m = min(n, self.n)
        for f in STATE_F + STATE_I:
            getattr(s, f)[:m] = getattr(self, f)[:m]
        return s

    def cstruct(self) -> Particles:
        p = Particles()
        for f in STATE_F:
            setattr(p, f, dptr(getattr(self, f)))
        for f in STATE_I:
            setattr(p, f, iptr(getattr(self, f)))
        p.n = self.n
        return p


class RngState:
    def __init__(self, mode=RNG_MT, seed=0, stream=0):
        self.r = Rng()
        self.r.mode = mode
        self.r.seed = seed
        self.r.stream = stream
        self._keep = []
        if mode == RNG_MT:
            lib().oc_mt_seed(C.byref(self.r), seed)

    def load_mt(self, words):
        """Load a libstdc++ mt19937_64 text state (312 words + index)."""
        for i in range(312):
            self.r.mt[i] = int(words[i])
        self.r.mt_idx = int(words[312])

    def set_replay(self, words: np.ndarray):
        w = np.ascontiguousarray(words, dtype=np.uint64)
        self._keep.append(w)
        self.r.mode = RNG_REPLAY
        self.r.words = uptr(w)
        self.r.nwords = len(w)
        self.r.pos = 0

    def start_record(self, cap: int):
        buf = np.zeros(cap, np.uint64)
        self._rec = buf
        self.r.rec = uptr(buf)
        self.r.rec_cap = cap
        self.r.rec_n = 0
        self.r.rec_overflow = 0

    def recorded(self) -> np.ndarray:
        assert not self.r.rec_overflow, "record buffer overflow"
        return self._rec[: self.r.rec_n].copy()


class Model:
    """Oracle model: valleys, mechanisms and rate tables."""

    def __init__(self, temperature=300.0, rho=2329.0, vsound=9040.0, epsR=11.8,
                 Ni=1.45e16, n_levels=1000, max_energy=1.0):
        self.h = lib().oc_model_new(temperature, rho, vsound, epsR, Ni, n_levels, max_energy)
        self.n_levels = n_levels
        self.max_energy = max_energy
        self.temperature = temperature
        self.nV = 0

    def __del__(self):
        try:
            lib().oc_model_free(self.h)
        except Exception:
            pass

    def add_valley(self, rel_mass, particle_mass, deg, alpha, bottom=0.0, frames=None):
        v = lib().oc_add_valley(self.h, dptr(darr(rel_mass)), particle_mass, deg, alpha, bottom)
        assert v >= 0
        if frames:
            for s, (a, b, c) in enumerate(frames):
                assert lib().oc_set_frame(self.h, v, s, dptr(darr(a)), dptr(darr(b)),
                                          dptr(darr(c))) == 0
        self.nV += 1
        return v

    def add_mech(self, kind, valley, regions, p0=0.0, p1=0.0, final_valley=None,
                 final_sub=None):
        fs = np.zeros(1, np.int32) if final_sub is None else \
            np.ascontiguousarray(np.asarray(final_sub, np.int32))
        nF = 0 if final_sub is None else fs.shape[1]
        regs = np.ascontiguousarray(np.asarray(regions, np.int32))
        fv = valley if final_valley is None else final_valley
        idx = lib().oc_add_mech(self.h, kind, valley, fv, p0, p1, nF, iptr(fs.reshape(-1)),
                                iptr(regs), len(regs))
        assert idx >= 0
        return idx

    def set_region_doping(self, region, doping):
        assert lib().oc_set_region_doping(self.h, region, doping) == 0

    def set_surface(self, boundary, kind, param):
        """A surface mechanism at one device boundary (XMIN 0 .. YMAX 3): kind
        SURFACE_CONSTANT (specularity) or SURFACE_ROUGHNESS (height [m])."""
        assert lib().oc_set_surface(self.h, boundary, kind, param) == 0

    def set_grain(self, transmission_prob, scatter_rate):
        """emcGrainScatterMechanism(transmissionProb, scatterRate) on the type
        (include/emcGrainScatterMechanism.hpp:27-29)."""
        assert lib().oc_set_grain(self.h, transmission_prob, scatter_rate) == 0

    def build_tables(self):
        assert lib().oc_build_tables(self.h) == 0

    def n_tables(self, valley, region):
        return lib().oc_n_tables(self.h, valley, region)

    def raw_table(self, valley, region, t):
        out = np.zeros(self.n_levels)
        assert lib().oc_get_raw_table(self.h, valley, region, t, dptr(out)) == 0
        return out

    def norm_table(self, valley, region, t):
        out = np.zeros(self.n_levels)
        assert lib().oc_get_norm_table(self.h, valley, region, t, dptr(out)) == 0
        return out

    def set_raw_tables(self, valley, region, raw):
        """reinitScatterTables with the rates raw (n_tables x n_levels)."""
        a = np.ascontiguousarray(np.asarray(raw, np.float64).reshape(-1))
        assert a.size == self.n_tables(valley, region) * self.n_levels
        assert lib().oc_set_raw_tables(self.h, valley, region, dptr(a)) == 0

    def tau(self, valley, region):
        return lib().oc_get_tau(self.h, valley, region)

    def valley_consts(self, v):
        out = np.zeros(8)
        lib().oc_valley_consts(self.h, v, dptr(out))
        return out

    # ---- dynamics -------------------------------------------------------
    def bulk_step(self, st: State, dt, force, box, rng: RngState, step, offsets=None):
        p = st.cstruct()
        off = None
        if offsets:
            off = np.zeros(st.n + 1, np.int64)
        rc = lib().oc_bulk_step(self.h, C.byref(p), dt, dptr(darr(force)), dptr(darr(box)),
                                C.byref(rng.r), step, lptr(off) if off is not None else None)
        return rc, off

    def bulk_run_philox(self, st: State, dt, force, box, field_dir, seed, stream, step0,
                        n_steps, n_threads=0, want_obs=True, words32=False):
        """words32: draw as the engine's float source (one 32-bit word per draw)."""
        p = st.cstruct()
        obs = np.zeros((n_steps, self.nV, 3)) if want_obs else None
        rc = lib().oc_bulk_run_philox(self.h, C.byref(p), dt, dptr(darr(force)), dptr(darr(box)),
                                      dptr(darr(field_dir)), seed, stream, step0, n_steps,
                                      n_threads, dptr(obs) if want_obs else None, int(words32))
        assert rc == 0, rc
        return obs

    def bulk_run_coulomb(self, st: State, dt, charge, field, box, field_dir, fixed_pos,
                         fixed_q, eps_r, inv_cutoff, images, seed, stream, step0, n_steps,
                         n_threads=0, want_obs=True):
        """FMMBulkParticleHandler's loop: Coulomb sums, then a step with
        per-particle forces, n_steps times (Philox)."""
        p = st.cstruct()
        obs = np.zeros((n_steps, self.nV, 3)) if want_obs else None
        fp = np.ascontiguousarray(np.asarray(fixed_pos, np.float64).reshape(3, -1))
        fq = np.ascontiguousarray(np.asarray(fixed_q, np.float64).reshape(-1))
        rc = lib().oc_bulk_run_coulomb(self.h, C.byref(p), dt, charge, dptr(darr(field)),
                                       dptr(darr(box)), dptr(darr(field_dir)),
                                       dptr(fp.reshape(-1)), dptr(fq), fq.size, eps_r,
                                       inv_cutoff, images, seed, stream, step0, n_steps,
                                       n_threads, dptr(obs) if want_obs else None)
        assert rc == 0, rc
        return obs

    def observables(self, st: State, field_dir):
        out = np.zeros((self.nV, 3))
        p = st.cstruct()
        lib().oc_observables(self.h, C.byref(p), dptr(darr(field_dir)), dptr(out))
        return out

    def bulk_init(self, max_pos, spacing, doping, rng: RngState, cap=1 << 22):
        st = State(cap)
        p = st.cstruct()
        n = lib().oc_bulk_init(self.h, dptr(darr(max_pos)), dptr(darr(spacing)), doping,
                               C.byref(rng.r), C.byref(p), cap)
        assert n >= 0
        return st.resize(int(n))


# ---- canonical silicon models (restated from the reference example) ----------
SI_FRAMES = [((1, 0, 0), (0, 1, 0), (0, 0, 1)),
             ((0, 1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (0, 1, 0), (1, 0, 0))]
F_SUB = [[1, 1, 2, 2], [0, 0, 2, 2], [0, 0, 1, 1]]
G_SUB = [[0], [1], [2]]
ME = 9.11e-31
KB, Q = 1.38066e-23, 1.60219e-19
JACOBONI = [("G1", False, 140., 0.5e10), ("G2", False, 215., 0.8e10),
            ("G3", False, 720., 11.e10), ("F1", True, 220., 0.3e10),
            ("F2", True, 550., 2.0e10), ("F3", True, 685., 2.0e10)]


SURFACE_SPECULAR, SURFACE_CONSTANT, SURFACE_ROUGHNESS = 0, 1, 2


def silicon_model(name="jacoboni", temperature=300.0, n_levels=1000, max_energy=1.0,
                  mt=None, regions=(0,), coulomb=False, grain=None) -> Model:
    """Oracle twin of the silicon models used by the reference harness;
    grain: (transmission probability, scatter rate [1/s]) of a grain
    mechanism."""
    m = Model(temperature=temperature, n_levels=n_levels, max_energy=max_energy)
    if grain is not None:
        m.set_grain(*grain)
    if mt is None:
        mt = 0.196 if name == "refbulk" else 0.19
    m.add_valley([0.916, mt, mt], ME, 3, 0.5, 0.0, SI_FRAMES)
    regs = list(regions)
    if name == "refbulk":
        m.add_mech(ACOUSTIC, 0, regs, 9.0)
        for kind in (ZERO_IV_ABS, ZERO_IV_EMI):
            m.add_mech(kind, 0, regs, 5.23e10, 0.06, 0, F_SUB)
        for kind in (ZERO_IV_ABS, ZERO_IV_EMI):
            m.add_mech(kind, 0, regs, 5.23e10, 0.06, 0, G_SUB)
        for kind in (FIRST_IV_ABS, FIRST_IV_EMI):
            m.add_mech(kind, 0, regs, 2.5, 0.023, 0, F_SUB)
        for kind in (FIRST_IV_ABS, FIRST_IV_EMI):
            m.add_mech(kind, 0, regs, 4.0, 0.018, 0, G_SUB)
    elif name == "jacoboni":
        m.add_mech(ACOUSTIC, 0, regs, 9.0)
        for _, isF, theta, D in JACOBONI:
            e = KB * theta / Q
            fs = F_SUB if isF else G_SUB
            m.add_mech(ZERO_IV_ABS, 0, regs, D, e, 0, fs)
            m.add_mech(ZERO_IV_EMI, 0, regs, D, e, 0, fs)
    else:
        raise ValueError(name)
    if coulomb:
        m.add_mech(COULOMB, 0, regs, 11.8)
    m.build_tables()
    return m


# ---- reference harness output -------------------------------------------------
def parse_ref(text: str) -> dict:
    out = {}
    for line in text.splitlines():
        parts = line.split()
        if len(parts) < 2:
            continue
        key, n = parts[0], int(parts[1])
        vals = parts[2:2 + n]
        if key.startswith("name_") or "_name_v" in key:
            out[key] = vals[0] if vals else ""
        elif vals and (vals[0].startswith("0x") or vals[0].startswith("-0x")
                       or "p" in vals[0] or vals[0] in ("inf", "-inf", "nan")):
            out[key] = np.array([float.fromhex(v) for v in vals])
        else:
            out[key] = np.array([int(v) for v in vals], dtype=np.uint64 if key.startswith("mt")
                                else np.int64)
    return out


def run_ref(*args) -> dict:
    if not os.path.exists(REF_DRIVER):
        raise FileNotFoundError("reference harness not built (make -C oracle ref)")
    # the reference writes its table files into the working directory: run it
    # in a scratch directory under oracle/_ref/ and remove that afterwards
    import shutil
    import tempfile
    base = os.path.join(HERE, "_ref", "scratch")
    os.makedirs(base, exist_ok=True)
    work = tempfile.mkdtemp(dir=base)
    try:
        r = subprocess.run([REF_DRIVER] + [str(a) for a in args], check=True,
                           capture_output=True, text=True, cwd=work)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    return parse_ref(r.stdout)


def state_from_ref(d: dict, tag: str) -> State:
    return State.from_dict({f: d[f"{tag}_{f}"] for f in STATE_F + STATE_I})


# ---- device (2-D) path ----------------------------------------------------------
NGP, CIC, NEC, NEC_VWD = 0, 1, 2, 3


class DevDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("hx", C.c_double), ("hy", C.c_double),
                ("maxX", C.c_double), ("maxY", C.c_double), ("width", C.c_double),
                ("T", C.c_double), ("Ni", C.c_double), ("epsR", C.c_double),
                ("doping", C.POINTER(C.c_double)), ("region", C.POINTER(C.c_int32)),
                ("bnd", C.POINTER(C.c_int32) * 4), ("nContacts", C.c_int32), ("pad_", C.c_int32),
                ("ctype", C.POINTER(C.c_int32)), ("cvolt", C.POINTER(C.c_double)),
                ("cpar", C.POINTER(C.c_double))]


def _declare_dev(L):
    d, i32, i64, u32, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint32, C.c_void_p
    P = C.POINTER
    L.oc_dev_debye.restype = d
    L.oc_dev_debye.argtypes = [P(DevDesc)]
    L.oc_dev_cell_volume.restype = d
    L.oc_dev_cell_volume.argtypes = [P(DevDesc)]
    L.oc_dev_contact_idx.restype = i32
    L.oc_dev_contact_idx.argtypes = [P(DevDesc), i32, i32]
    L.oc_dev_is_reservoir.restype = i32
    L.oc_dev_is_reservoir.argtypes = [P(DevDesc), i32, i32]
    L.oc_dev_efield.argtypes = [P(DevDesc), P(d), P(d), P(d)]
    L.oc_dev_efield_pm.argtypes = [P(DevDesc), C.c_int32, P(d), P(d), P(d)]
    L.oc_dev_assign.argtypes = [P(DevDesc), i32, P(d), P(d), i64, d, P(d)]
    L.oc_dev_force.argtypes = [P(DevDesc), i32, P(d), P(d), d, d, d, P(d)]
    L.oc_dev_move.restype = i32
    L.oc_dev_move.argtypes = [vp, P(DevDesc), i32, P(Particles), P(d), P(d), d, d, P(Rng), u32,
                              P(i32), P(i64)]
    L.oc_dev_exp_nr.argtypes = [P(DevDesc), P(d), i32]
    L.oc_dev_contacts.restype = i64
    L.oc_dev_contacts.argtypes = [vp, P(DevDesc), P(Particles), i64, P(d), d, P(Rng), u32, P(i32),
                                  i32]
    L.oc_dev_concentration.argtypes = [P(DevDesc), P(d), P(d)]
    L.oc_dev_init_potential.argtypes = [P(DevDesc), P(d)]
    L.oc_dev_sor.restype = i64
    L.oc_dev_sor.argtypes = [P(DevDesc), P(d), P(d), d, d, i32, i64]
    L.oc_dev_init.restype = i64
    L.oc_dev_init.argtypes = [vp, P(DevDesc), P(d), i32, d, P(Rng), P(Particles), i64, i32]


class Device:
    """Flattened 2-D device for the oracle (arrays kept alive here)."""

    def __init__(self, nx, ny, hx, hy, width, doping, region, bnd, ctype, cvolt, cpar,
                 T=300.0, Ni=1.45e16, epsR=11.8):
        L = lib()
        if not hasattr(L, "_dev_declared"):
            _declare_dev(L)
            L._dev_declared = True
        self.nx, self.ny = nx, ny
        self.doping = darr(doping)
        self.region = np.ascontiguousarray(np.asarray(region, np.int32))
        self.bnd = [np.ascontiguousarray(np.asarray(b, np.int32)) for b in bnd]
        self.ctype = np.ascontiguousarray(np.asarray(ctype, np.int32))
        self.cvolt = darr(cvolt)
        self.cpar = darr(cpar).reshape(-1)
        d = DevDesc()
        d.nx, d.ny, d.hx, d.hy = nx, ny, hx, hy
        d.maxX, d.maxY = hx * (nx - 1), hy * (ny - 1)
        d.width, d.T, d.Ni, d.epsR = width, T, Ni, epsR
        d.doping, d.region = dptr(self.doping), iptr(self.region)
        for b in range(4):
            d.bnd[b] = iptr(self.bnd[b])
        d.nContacts = len(self.ctype)
        d.ctype, d.cvolt, d.cpar = iptr(self.ctype), dptr(self.cvolt), dptr(self.cpar)
        self.d = d

    def set_max(self, maxX, maxY):
        self.d.maxX, self.d.maxY = maxX, maxY

    @property
    def L(self):
        return lib()

    def efield(self, pot, scheme=NGP):
        Ex = np.zeros(self.nx * self.ny)
        Ey = np.zeros(self.nx * self.ny)
        self.L.oc_dev_efield_pm(C.byref(self.d), scheme, dptr(darr(pot)), dptr(Ex), dptr(Ey))
        return Ex, Ey

    def sor(self, pot, conc=None, omega=1.8, acc=1e-4, reset=True, max_sweeps=10 ** 7):
        pot = darr(pot).copy()
        c = dptr(darr(conc)) if conc is not None else None
        n = self.L.oc_dev_sor(C.byref(self.d), dptr(pot), c, omega, acc, int(reset), max_sweeps)
        return pot, n

    def assign(self, scheme, st, nrC=1.0):
        g = np.zeros(self.nx * self.ny)
        self.L.oc_dev_assign(C.byref(self.d), scheme, dptr(st.px), dptr(st.py), st.n, nrC, dptr(g))
        return g

    def concentration(self, nr):
        c = np.zeros(self.nx * self.ny)
        self.L.oc_dev_concentration(C.byref(self.d), dptr(darr(nr)), dptr(c))
        return c

    def exp_nr(self, round_counts=False):
        e = np.zeros(self.nx * self.ny)
        self.L.oc_dev_exp_nr(C.byref(self.d), dptr(e), int(round_counts))
        return e

    def move(self, model, scheme, st, Ex, Ey, dt, rng, step, charge=-1.60219e-19, offsets=False):
        p = st.cstruct()
        netto = np.zeros(max(len(self.ctype), 1), np.int32)
        off = np.zeros(st.n + 1, np.int64) if offsets else None
        rc = self.L.oc_dev_move(model.h, C.byref(self.d), scheme, C.byref(p), dptr(darr(Ex)),
                                dptr(darr(Ey)), dt, charge, C.byref(rng.r), step, iptr(netto),
                                lptr(off) if off is not None else None)
        st.n = int(p.n)
        return rc, netto, off

    def contacts(self, model, st, cap, expnr, rng, step, nrC=1.0, tau_region_is_valley=False):
        """st must have capacity `cap` allocated (State.resize)."""
        p = st.cstruct()
        p.n = st.n
        remInj = np.zeros(max(len(self.ctype), 1), np.int32)
        n = self.L.oc_dev_contacts(model.h, C.byref(self.d), C.byref(p), cap, dptr(darr(expnr)),
                                   nrC, C.byref(rng.r), step, iptr(remInj),
                                   int(tau_region_is_valley))
        assert n >= 0, n
        st.n = int(n)
        return remInj

    def init_particles(self, model, rng, pot=None, round_counts=False, nrC=1.0, cap=1 << 20,
                       tau_region_is_valley=False):
        st = State(cap)
        p = st.cstruct()
        n = self.L.oc_dev_init(model.h, C.byref(self.d), dptr(darr(pot)) if pot is not None
                               else None, int(round_counts), nrC, C.byref(rng.r), C.byref(p), cap,
                               int(tau_region_is_valley))
        assert n >= 0
        return st.resize(int(n))


def truncate(st: State, n: int) -> State:
    """View of the first n particles (copy)."""
    return st.resize(n)


# ---- particle-particle Coulomb (FMM handlers, direct sum) -------------------------
def p2p_pair(t, qt, s, qs, inv_cutoff=1e9):
    """NonMutualParticles for one pair: (force x, y, z, potential)."""
    out = np.zeros(4)
    lib().oc_p2p_pair(t[0], t[1], t[2], qt, s[0], s[1], s[2], qs, inv_cutoff, dptr(out))
    return out


def p2p_coulomb(pos, q, inv_cutoff=1e9, box=0.0, images=0, threads=0):
    """Direct Coulomb sums: pos (3, n), q (n,) -> force (3, n), potential (n,)."""
    p = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(3, -1))
    qq = np.ascontiguousarray(np.asarray(q, np.float64))
    n = qq.size
    f = np.zeros((3, n))
    pot = np.zeros(n)
    assert lib().oc_p2p_coulomb(dptr(p.reshape(-1)), dptr(qq), n, inv_cutoff, box, images,
                                dptr(f.reshape(-1)), dptr(pot), threads) == 0
    return f, pot
