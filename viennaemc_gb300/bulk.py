"""Bulk ensembles on the GPU engine.

BulkParticleHandler mirrors basicBulkParticleHandler
(examples/bulkSimulation/basicBulkParticleHandler.hpp:43-614): same names,
argument meaning and observables, with the particle state resident on the
GPU.  BulkBatch advances many uneven ensembles (different fields,
temperatures, particle counts) together in one launch.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .physics import Electron, thermal_voltage

STATE_F = ("kx", "ky", "kz", "px", "py", "pz", "energy", "tau", "grain_tau")
STATE_I = ("valley", "sub", "region")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class ParticleState:
    """Host structure-of-arrays particle state (float64 / int32).

    pinned: the arrays live in one page-locked block (emcg_host_alloc), so
    uploads and downloads run at the full host-link rate."""

    def __init__(self, n: int, pinned: bool = False):
        self.n = int(n)
        self._block = None
        if pinned and self.n:
            lib = L.lib()
            nb = self.n * (8 * len(STATE_F) + 4 * len(STATE_I))
            p = C.c_void_p()
            L.check(lib.emcg_host_alloc(nb, C.byref(p)))
            self._block = p
            self._finalizer = weakref.finalize(self, lib.emcg_host_free, p)
            raw = np.ctypeslib.as_array((C.c_uint8 * nb).from_address(p.value))
            off = 0
            for f in STATE_F:
                setattr(self, f, raw[off:off + 8 * self.n].view(np.float64))
                off += 8 * self.n
            for f in STATE_I:
                setattr(self, f, raw[off:off + 4 * self.n].view(np.int32))
                off += 4 * self.n
            for f in STATE_F + STATE_I:
                getattr(self, f)[:] = 0
            return
        for f in STATE_F:
            setattr(self, f, np.zeros(self.n, np.float64))
        for f in STATE_I:
            setattr(self, f, np.zeros(self.n, np.int32))

    @classmethod
    def from_arrays(cls, **kw) -> "ParticleState":
        n = len(kw["energy"])
        s = cls(n)
        for f in STATE_F + STATE_I:
            if f in kw:
                getattr(s, f)[:] = kw[f]
        return s

    def desc(self) -> L.StateDesc:
        d = L.StateDesc()
        for f in STATE_F:
            setattr(d, f, _dp(getattr(self, f)))
        for f in STATE_I:
            setattr(d, f, _ip(getattr(self, f)))
        d.n = self.n
        return d


class ParticleStateF32:
    """Host particle state in the float engine's own layout (emcg_state_f32):
    float fields and meta = valley | subvalley << 8 | region << 16, 40 bytes a
    particle; pinned: one page-locked block (emcg_host_alloc)."""

    def __init__(self, n: int, pinned: bool = False):
        self.n = int(n)
        nb = self.n * (4 * len(STATE_F) + 4)
        if pinned and self.n:
            lib = L.lib()
            p = C.c_void_p()
            L.check(lib.emcg_host_alloc(nb, C.byref(p)))
            self._finalizer = weakref.finalize(self, lib.emcg_host_free, p)
            raw = np.ctypeslib.as_array((C.c_uint8 * nb).from_address(p.value))
            raw[:] = 0
        else:
            raw = np.zeros(max(nb, 1), np.uint8)
        for k, f in enumerate(STATE_F):
            setattr(self, f, raw[4 * k * self.n:4 * (k + 1) * self.n].view(np.float32))
        self.meta = raw[4 * len(STATE_F) * self.n:nb].view(np.uint32)
        # the fields are views of one block and stay put: the descriptor is
        # built once (a step call then costs no ctypes conversions)
        d = L.StateF32Desc()
        for f in STATE_F:
            setattr(d, f, getattr(self, f).ctypes.data_as(C.POINTER(C.c_float)))
        d.meta = self.meta.ctypes.data_as(C.POINTER(C.c_uint32))
        d.n = self.n
        self._desc = d

    def __setattr__(self, k, val):
        if k in STATE_F + ("meta",) and "_desc" in self.__dict__:
            raise AttributeError(f"{k} is a view of the state's block: assign in place "
                                 f"({k}[:] = ...)")
        object.__setattr__(self, k, val)

    @classmethod
    def from_state(cls, st: "ParticleState", pinned: bool = False) -> "ParticleStateF32":
        s = cls(st.n, pinned)
        for f in STATE_F:
            getattr(s, f)[:] = getattr(st, f)
        s.meta[:] = (np.asarray(st.valley, np.uint32) | (np.asarray(st.sub, np.uint32) << 8) |
                     (np.asarray(st.region, np.uint32) << 16))
        return s

    def desc(self) -> L.StateF32Desc:
        return self._desc


def update_rates(lib, h, model: int, raw, particle_type) -> object:
    """emcg_update_rates: raw is a host array, a CUDA float64 tensor (device
    rates), or None (refill from the particle type's mechanisms).  Returns
    what must stay alive until the next step call (a device tensor)."""
    if raw is None:
        raw = particle_type.raw_rates()
    if hasattr(raw, "is_cuda") and raw.is_cuda:
        import torch
        if raw.dtype != torch.float64 or not raw.is_contiguous():
            raise ValueError("device rates must be a contiguous float64 tensor")
        torch.cuda.current_stream(raw.device).synchronize()  # complete before the call
        L.check(lib.emcg_update_rates(h, model, C.c_void_p(raw.data_ptr()), 1))
        return raw
    a = np.ascontiguousarray(np.asarray(raw, np.float64).reshape(-1))
    want = particle_type.scatterHandler.fill_size()
    if a.size != want:
        raise ValueError(f"rates: {a.size} values, the model's tables hold {want}")
    L.check(lib.emcg_update_rates(h, model, a.ctypes.data_as(C.c_void_p), 0))
    return None


def get_rates(lib, h, model: int, particle_type):
    """emcg_get_rates: (tables in the raw layout, tau per table set)."""
    n = particle_type.scatterHandler.fill_size()
    nts = len(particle_type.scatterHandler.table_mechs)
    tables, tau = np.zeros(max(n, 1)), np.zeros(max(nts, 1))
    L.check(lib.emcg_get_rates(h, model, tables.ctypes.data_as(C.c_void_p),
                               tau.ctypes.data_as(C.c_void_p)))
    return tables[:n], tau[:nts]


def _normalize(v):
    s = 0.0
    for x in v:
        s += x * x
    n = math.sqrt(s)
    return [float(x) for x in v] if n == 0 else [x / n for x in v]


@dataclass
class EnsembleSpec:
    """One bulk ensemble: the model it uses, its particle count and field."""
    model: int
    n_particles: int
    field_strength: float
    field_dir: tuple
    box: tuple
    dt: float
    seed: int
    stream: int = 0
    temperature: float = 300.0
    # the double engine draws as the float engine (EMCG_ENS_FLOAT_DRAWS)
    float_draws: bool = False


class BulkBatch:
    """Several bulk ensembles advanced together on one GPU.

    models: list of Electron particle types (e.g. one per temperature).
    precision: "fp64" (parity engine) or "fp32" (throughput engine).
    """

    def __init__(self, models, ensembles, precision="fp64", capacity_slack=0):
        self._lib = L.lib()
        self.models = list(models)
        self.specs = list(ensembles)
        self.precision = L.FP64 if precision in ("fp64", L.FP64) else L.FP32
        self._mdesc = [m.model_desc() for m in self.models]
        marr = (L.ModelDesc * len(self._mdesc))(*self._mdesc)
        self._marr = marr
        self.nVmax = max(m.getNrValleys() for m in self.models)
        earr = (L.EnsembleDesc * len(self.specs))()
        for i, sp in enumerate(self.specs):
            self._fill_ens(earr[i], sp, sp.n_particles + capacity_slack)
        self._earr = earr
        h = C.c_void_p()
        L.check(self._lib.emcg_bulk_create(marr, len(self._mdesc), earr, len(self.specs),
                                           self.precision, C.byref(h)))
        self.h = h
        self.step_index = 0

    def _fill_ens(self, d, sp: EnsembleSpec, capacity: int):
        pt = self.models[sp.model]
        dirn = _normalize(sp.field_dir)  # basicBulkParticleHandler.hpp:100-101
        d.model = sp.model
        d.capacity = capacity
        for i in range(3):
            d.field[i] = dirn[i] * sp.field_strength
            d.field_dir[i] = dirn[i]
            d.box[i] = sp.box[i]
        d.charge = pt.getCharge()
        d.dt = sp.dt
        d.seed = sp.seed
        d.stream = sp.stream
        d.flags = 1 if sp.float_draws else 0

    def close(self):
        if getattr(self, "h", None):
            self._lib.emcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- particles -----------------------------------------------------------
    def init_particles(self, ens: int, n: int | None = None, coords=None, extent=None,
                       spacing=None):
        """GPU initial particles (emcElectron::generateInitialParticle)."""
        sp = self.specs[ens]
        n = sp.n_particles if n is None else int(n)
        Vt = thermal_voltage(sp.temperature)
        if coords is None:
            L.check(self._lib.emcg_bulk_init(self.h, ens, n, None, None, None, Vt))
        else:
            c = np.ascontiguousarray(np.asarray(coords, np.int64).reshape(-1, 3))
            ext = np.ascontiguousarray(np.asarray(extent, np.int64))
            spc = np.ascontiguousarray(np.asarray(spacing, np.float64))
            L.check(self._lib.emcg_bulk_init(
                self.h, ens, len(c), c.ctypes.data_as(C.POINTER(C.c_int64)),
                ext.ctypes.data_as(C.POINTER(C.c_int64)), _dp(spc), Vt))

    def set_state(self, ens: int, st: ParticleState):
        d = st.desc()
        L.check(self._lib.emcg_set_state(self.h, ens, C.byref(d)))

    def set_state_f32(self, ens: int, st: ParticleStateF32):
        """Upload in the float engine's own layout (emcg_set_state_f32)."""
        L.check(self._lib.emcg_set_state_f32(self.h, ens, C.byref(st.desc())))

    def get_state_f32(self, ens: int, out: ParticleStateF32 | None = None) -> ParticleStateF32:
        n = self.num_particles(ens)
        out = out if out is not None and out.n == n else ParticleStateF32(n)
        d = out.desc()
        L.check(self._lib.emcg_get_state_f32(self.h, ens, C.byref(d)))
        return out

    def get_state(self, ens: int) -> ParticleState:
        n = self._lib.emcg_num_particles(self.h, ens)
        st = ParticleState(n)
        d = st.desc()
        L.check(self._lib.emcg_get_state(self.h, ens, C.byref(d)))
        return st

    def num_particles(self, ens: int) -> int:
        return int(self._lib.emcg_num_particles(self.h, ens))

    def update_ensemble(self, ens: int, spec: EnsembleSpec):
        d = L.EnsembleDesc()
        self._fill_ens(d, spec, self._earr[ens].capacity)
        L.check(self._lib.emcg_bulk_update_ensemble(self.h, ens, C.byref(d)))
        self.specs[ens] = spec
        self._earr[ens] = d

    # ---- dynamics ------------------------------------------------------------
    def set_launch(self, block_threads=0, steps_per_launch=0, min_blocks=0, queued=None,
                   pass_actions=None):
        L.check(self._lib.emcg_set_launch(self.h, block_threads, steps_per_launch))
        if min_blocks:
            L.check(self._lib.emcg_set_occupancy(self.h, min_blocks))
        if queued is not None:
            L.check(self._lib.emcg_set_scatter_mode(self.h, int(queued)))
        if pass_actions is not None:
            L.check(self._lib.emcg_set_pass_actions(self.h, int(pass_actions)))

    def launch(self) -> dict:
        """Block size of the last launch and the steps-per-launch setting."""
        blk, per = C.c_int32(), C.c_int32()
        L.check(self._lib.emcg_get_launch(self.h, C.byref(blk), C.byref(per)))
        return {"block_threads": blk.value, "steps_per_launch": per.value}

    def pass_actions(self) -> int:
        """Free flights per drift pass of the warp-asynchronous kernel."""
        n = C.c_int32()
        L.check(self._lib.emcg_get_pass_actions(self.h, C.byref(n)))
        return n.value

    def set_graph(self, enable: bool = True):
        """Replay each launch of steps from an instantiated CUDA graph."""
        L.check(self._lib.emcg_bulk_set_graph(self.h, int(enable)))

    def autotune(self, trial_steps: int = 50, step0: int | None = None) -> dict:
        """Time each candidate launch shape on trial_steps steps, in a forward
        and a backward pass over the shapes (the steps advance the ensembles,
        like warm-up steps), and keep the fastest."""
        s0 = self.step_index if step0 is None else int(step0)
        used, blk, mb, q = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        L.check(self._lib.emcg_bulk_autotune(self.h, int(trial_steps), s0, C.byref(used),
                                             C.byref(blk), C.byref(mb), C.byref(q)))
        self.step_index = s0 + used.value
        return {"block_threads": blk.value, "min_blocks": mb.value, "queued": q.value,
                "pass_actions": self.pass_actions(), "steps_used": used.value}

    def step(self, n_steps: int = 1, observables: bool = True, step0: int | None = None):
        """Advance all ensembles; returns sums [ens, step, valley, {E, v.dir, count}]."""
        s0 = self.step_index if step0 is None else int(step0)
        obs = np.zeros((len(self.specs), n_steps, self.nVmax, 3)) if observables else None
        L.check(self._lib.emcg_bulk_step(self.h, n_steps, s0, _dp(obs) if observables else None))
        self.step_index = s0 + n_steps
        return obs

    def step_from_host(self, ens: int, st: ParticleStateF32, n_steps: int = 1,
                       observables: bool = True, step0: int | None = None):
        """set_state_f32(ens, st) then step(n_steps) in one call
        (emcg_bulk_step_from_host): with st in page-locked memory the first
        launch reads the start state from host memory, the upload overlapping
        the steps."""
        s0 = self.step_index if step0 is None else int(step0)
        obs = np.zeros((len(self.specs), n_steps, self.nVmax, 3)) if observables else None
        L.check(self._lib.emcg_bulk_step_from_host(self.h, ens, C.byref(st.desc()), n_steps, s0,
                                                   _dp(obs) if observables else None))
        self.step_index = s0 + n_steps
        return obs

    def reinit_scatter_tables(self, model: int = 0, raw=None):
        """emcScatterHandler::reinitScatterTables (include/emcScatterHandler.hpp:
        100-108) of model `model` on the GPU, before the next step: raw are the
        refilled rates (host array, or CUDA float64 tensor), None refills them
        from the model's mechanisms now."""
        self._rates_keep = update_rates(self._lib, self.h, model, raw, self.models[model])

    def get_rates(self, model: int = 0):
        """The engine's normalised tables (raw layout) and tau per table set."""
        return get_rates(self._lib, self.h, model, self.models[model])

    def set_coulomb(self, eps_r, inv_cutoff=1e9, images=0, enable=True):
        """Particle-particle Coulomb steps (FMMBulkParticleHandler,
        examples/bulkSimulationFMM): each step sums the Coulomb force of every
        ensemble's particles and fixed charges on its particles, then moves
        them with force = charge x field - (ke / eps_r) x sum."""
        L.check(self._lib.emcg_bulk_set_coulomb(self.h, int(enable), float(eps_r),
                                                float(inv_cutoff), int(images)))

    def set_fixed_charges(self, ens: int, pos, q):
        """Charges of ensemble ens that do not move (donors): pos (3, n), q (n,)."""
        p = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(3, -1))
        qq = np.ascontiguousarray(np.asarray(q, np.float64).reshape(-1))
        if p.shape[1] != qq.size:
            raise ValueError("pos and q disagree in n")
        self._fixed_keep = (p, qq)
        L.check(self._lib.emcg_bulk_set_fixed_charges(self.h, ens, p.ctypes.data_as(C.c_void_p),
                                                      qq.ctypes.data_as(C.c_void_p), qq.size))

    def get_coulomb(self, ens: int):
        """(force sums (3, n), potential sums (n,)) of the last Coulomb step."""
        n = self.num_particles(ens)
        f, p = np.zeros((3, n)), np.zeros(n)
        L.check(self._lib.emcg_bulk_get_coulomb(self.h, ens, f.ctypes.data_as(C.c_void_p),
                                                p.ctypes.data_as(C.c_void_p)))
        return f, p

    def set_replay(self, words, offsets):
        w = np.ascontiguousarray(np.asarray(words, np.uint64))
        o = np.ascontiguousarray(np.asarray(offsets, np.int64))
        self._replay_keep = (w, o)
        L.check(self._lib.emcg_set_replay(self.h, w.ctypes.data_as(C.POINTER(C.c_uint64)),
                                          len(w), o.ctypes.data_as(C.POINTER(C.c_int64)),
                                          len(o)))

    def last_kernel_ms(self) -> float:
        ms = C.c_double()
        L.check(self._lib.emcg_last_kernel_ms(self.h, C.byref(ms)))
        return ms.value

    @staticmethod
    def averages(obs_sums: np.ndarray, n_particles) -> dict:
        """Per-step getAvgEnergy / getAvgDriftVelocity /
        getValleyOccupationProbability from observable sums."""
        cnt = obs_sums[..., 2]
        with np.errstate(invalid="ignore", divide="ignore"):
            avgE = np.where(cnt > 0, obs_sums[..., 0] / np.maximum(cnt, 1), 0.0)
            avgV = np.where(cnt > 0, obs_sums[..., 1] / np.maximum(cnt, 1), 0.0)
        n = np.asarray(n_particles, np.float64).reshape(-1, *([1] * (cnt.ndim - 1)))
        occ = np.where(n > 0, cnt / np.maximum(n, 1), 0.0)
        return {"energy": avgE, "drift_velocity": avgV, "occupation": occ}


class BulkParticleHandler:
    """basicBulkParticleHandler (examples/bulkSimulation/basicBulkParticleHandler.hpp)
    for one electron type on the GPU.

    handler = BulkParticleHandler(maxPos, particleType, fieldDir, fieldStrength, seed)
    handler.generateInitialParticles(spacing, doping)    # node-based counts
    handler.moveParticles(dt)                            # one time step
    handler.getAvgEnergy(0), getAvgDriftVelocity(0), getValleyOccupationProbability(0)
    """

    def __init__(self, max_pos, particle_type: Electron, field_dir, field_strength=0.0,
                 seed=0, temperature=300.0, precision="fp64", capacity=None, dt=1e-15):
        if seed == 0:  # the reference draws a wall-clock seed for 0 (:110-115)
            import time
            seed = time.time_ns() & 0xFFFFFFFFFFFFFFFF
        self.max_pos = tuple(float(x) for x in max_pos)
        self.type = particle_type
        self.field_dir = _normalize(field_dir)
        self.field_strength = float(field_strength)
        self.seed = int(seed)
        self.temperature = float(temperature)
        self.dt = float(dt)
        self.precision = precision
        self._capacity = capacity
        self._batch = None
        self._last = None
        self.n = 0

    def _spec(self, n):
        return EnsembleSpec(0, n, self.field_strength, tuple(self.field_dir), self.max_pos,
                            self.dt, self.seed, 0, self.temperature)

    def _ensure(self, n):
        cap = max(self._capacity or 0, n)
        if self._batch is None or self._batch._earr[0].capacity < cap:
            if self._batch is not None:
                self._batch.close()
            self._batch = BulkBatch([self.type], [self._spec(cap)], self.precision)
        return self._batch

    def generateInitialParticles(self, spacing=None, doping=None, n=None):
        """Initial particles.  With (spacing, doping): the reference's node-based
        count doping * cellVolume (half per boundary dimension), the
        fractional part drawn at random (:143-159); with n: n particles uniform
        in the box."""
        if n is not None:
            b = self._ensure(int(n))
            b.init_particles(0, int(n))
            self.n = int(n)
            return
        ext = [int(round(mp / h)) + 1 for mp, h in zip(self.max_pos, spacing)]
        cell = 1.0
        for h in spacing:
            cell = cell * h
        rng = np.random.default_rng(self.seed)
        coords = []
        for z in range(ext[2]):
            for y in range(ext[1]):
                for x in range(ext[0]):
                    nr = doping
                    for c, e in zip((x, y, z), ext):
                        if c == 0 or c == e - 1:
                            nr *= 0.5
                    nr = nr * cell
                    while nr >= 1:
                        coords.append((x, y, z))
                        nr -= 1
                    if rng.random() < nr:
                        coords.append((x, y, z))
        b = self._ensure(len(coords))
        b.init_particles(0, coords=coords, extent=ext, spacing=spacing)
        self.n = len(coords)

    def resetAppliedFieldStrength(self, strength):
        self.field_strength = float(strength)
        if self._batch is not None:
            self._batch.update_ensemble(0, self._spec(self._batch.specs[0].n_particles))

    def getAppliedField(self):
        return [d * self.field_strength for d in self.field_dir]

    def getNrParticles(self, idx_type=0):
        return self.n

    def moveParticles(self, dt, n_steps=1):
        """Advance by n_steps steps of dt; returns per-step averages."""
        b = self._batch
        if dt != self.dt:
            self.dt = float(dt)
            b.update_ensemble(0, self._spec(b.specs[0].n_particles))
        obs = b.step(n_steps)
        self._last = BulkBatch.averages(obs, [self.n])
        return self._last

    def reinitScatterTables(self, raw=None):
        """The particle type's scatterHandler.reinitScatterTables() on the GPU
        (before any particle exists: on the host model the engine is built
        from)."""
        if raw is None:  # refill on the host model too, so a rebuilt engine agrees
            h = self.type.scatterHandler
            h.reinitScatterTables()
            raw = np.concatenate([h.raw[k].reshape(-1) for k in sorted(h.table_mechs)]) \
                if h.table_mechs else np.zeros(0)
        if self._batch is not None:
            self._batch.reinit_scatter_tables(0, raw)

    def getAvgEnergy(self, idx_type=0):
        return self._current()["energy"]

    def getAvgDriftVelocity(self, idx_type=0):
        return self._current()["drift_velocity"]

    def getValleyOccupationProbability(self, idx_type=0):
        return self._current()["occupation"]

    def _current(self):
        if self._last is None:
            raise RuntimeError("observables are produced by moveParticles")
        return {k: v[0, -1] for k, v in self._last.items()}

    def get_state(self):
        return self._batch.get_state(0)

    def set_state(self, st: ParticleState):
        self._ensure(st.n).set_state(0, st)
        self.n = st.n

    def deleteParticles(self):
        if self._batch is not None:
            self._batch.set_state(0, ParticleState(0))
        self.n = 0


class FMMBulkParticleHandler(BulkParticleHandler):
    """FMMBulkParticleHandler (examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp)
    on the GPU: bulk electrons with particle-particle Coulomb forces, the
    donors as fixed charges.  The FMM's sums are formed directly on the GPU
    in every step; images is the number of periodic copies of the box on each
    side (scalFMM's periodicity parameter repeats the box in its own way; this
    sums over (2 images + 1)^3 boxes).

    handler = FMMBulkParticleHandler(maxPos, electronType, fieldDir, fieldStrength,
                                     images, eps_r=11.8, doping=1e24)
    handler.generateInitialParticles(spacing)      # electrons and donors
    handler.executeFMM(); handler.moveParticles(dt)
    handler.getAvgEnergy(0), getAvgDriftVelocity(0), getValleyOccupationProbability(0)
    """

    def __init__(self, max_pos, particle_type: Electron, field_dir, field_strength=0.0,
                 images=0, eps_r=11.8, doping=0.0, inv_cutoff=1e9, seed=0,
                 temperature=300.0, precision="fp64", capacity=None, dt=1e-16):
        super().__init__(max_pos, particle_type, field_dir, field_strength, seed, temperature,
                         precision, capacity, dt)
        self.images = int(images)
        self.eps_r = float(eps_r)
        self.doping = float(doping)
        self.inv_cutoff = float(inv_cutoff)
        self.donors = np.zeros((3, 0))

    def generateInitialParticles(self, spacing=None, doping=None, n=None):
        """Electrons (the node-based counts of the doping, or n uniform) and as
        many donors as electrons, uniform in the box (addParticle with the
        reference's initParticlePos, :155-176, :446-460)."""
        super().generateInitialParticles(spacing, self.doping if doping is None else doping, n)
        rs = np.random.default_rng(self.seed + 1)
        self.donors = rs.random((3, self.n)) * np.asarray(self.max_pos)[:, None]
        self._apply()

    def _apply(self):
        b = self._batch
        b.set_fixed_charges(0, self.donors, np.full(self.donors.shape[1], -self.type.getCharge()))
        b.set_coulomb(self.eps_r, self.inv_cutoff, self.images)

    def set_state(self, st: ParticleState):
        super().set_state(st)
        self._apply()

    def getNrRepeatedBoxes(self):
        return (2 * self.images + 1) ** 3

    def executeFMM(self):
        """The Coulomb sums run inside each step (moveParticles)."""

    def resetForcesAndPotential(self):
        """Nothing to reset: the sums are formed afresh in every step."""

    def rearrangeTree(self):
        """No tree: the direct sums need no arrangement."""

    def getCoulomb(self):
        """Force and potential sums of the last step (container values)."""
        return self._batch.get_coulomb(0)
