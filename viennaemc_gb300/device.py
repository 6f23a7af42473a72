"""2-D device simulations on the GPU engine.

Device mirrors emcDevice (include/emcDevice.hpp) with its doping profile
(include/emcDopingProfile.hpp) and surface (include/emcSurface.hpp): the same
grid, region and contact bookkeeping, built on the host.
DeviceSimulation mirrors emcSimulation (include/emcSimulation.hpp): the
equilibrium characteristics, performEMCStep and the terminal-current
bookkeeping of emcSimulationResults (include/emcSimulationResults.hpp), with
every per-step stage running in libemcgpu.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from . import results as R
from .bulk import ParticleState, get_rates, update_rates
from .physics import Material, thermal_voltage

XMIN, XMAX, YMIN, YMAX = range(4)  # emcBoundaryPos (include/emcBoundaryPos.hpp:13-20)
OHMIC, SCHOTTKY, GATE = L.CONTACT_OHMIC, L.CONTACT_SCHOTTKY, L.CONTACT_GATE
NGP, CIC, NEC, NEC_VWD = L.PM_NGP, L.PM_CIC, L.PM_NEC, L.PM_NEC_VWD


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class Device:
    """2-D emcDevice: box [0, maxPos] with fixed spacing, doping regions and
    contacts on the four boundaries."""

    def __init__(self, material: Material, max_pos, spacing, temperature=300.0):
        self.material = material
        self.max_pos = (float(max_pos[0]), float(max_pos[1]))
        self.spacing = (float(spacing[0]), float(spacing[1]))
        self.temperature = float(temperature)
        self.width = 1e-6  # include/emcDevice.hpp:63
        # maxPosToExtent (include/emcUtil.hpp:98-110)
        self.nx = int(round(self.max_pos[0] / self.spacing[0])) + 1
        self.ny = int(round(self.max_pos[1] / self.spacing[1])) + 1
        n = self.nx * self.ny
        self.doping = np.full(n, material.Ni)           # emcDopingProfile(ext, Ni, Ni)
        self.region = np.full(n, -1, np.int32)
        self.region_doping = {-1: material.Ni}
        self.n_regions = 0
        self.bnd = [np.full(self.ny, -1, np.int32), np.full(self.ny, -1, np.int32),
                    np.full(self.nx, -1, np.int32), np.full(self.nx, -1, np.int32)]
        self.contacts = []  # (type, voltage, (epsOx, thickness, barrier))

    # ---- geometry -------------------------------------------------------------
    def setDeviceWidth(self, w):
        self.width = float(w)

    def getThermalVoltage(self):
        return thermal_voltage(self.temperature)

    def getCellVolume(self):
        v = 1.0
        v = v * self.spacing[0]
        v = v * self.spacing[1]
        return v * self.width

    def posToCoord(self, pos):
        return [int(round(p / h)) for p, h in zip(pos, self.spacing)]

    # ---- doping (include/emcDopingProfile.hpp:74-81, 161-207) ---------------------
    def addConstantDopingRegion(self, min_pos, max_pos, doping):
        lo, hi = self.posToCoord(min_pos), self.posToCoord(max_pos)
        ext = (self.nx, self.ny)
        for d in range(2):
            lo[d] = min(ext[d], max(0, lo[d]))
            hi[d] = min(ext[d], max(0, hi[d]))
            if hi[d] < lo[d]:
                lo[d], hi[d] = hi[d], lo[d]
        r = self.n_regions
        for y in range(lo[1], min(hi[1], self.ny - 1) + 1):
            for x in range(lo[0], min(hi[0], self.nx - 1) + 1):
                self.region[y * self.nx + x] = r
                self.doping[y * self.nx + x] = doping
        self.region_doping[r] = float(doping)
        self.n_regions += 1
        return r

    # ---- contacts (include/emcSurface.hpp:199-222, 380-409) ----------------------
    def _surface_coord(self, bp, pos):
        return int(round(pos / (self.spacing[1] if bp // 2 == 0 else self.spacing[0])))

    def _on_boundary(self, x, y, b):
        return (x == 0, x == self.nx - 1, y == 0, y == self.ny - 1)[b]

    def _add_contact(self, bp, ctype, voltage, min_pos, max_pos, par=(0.0, 0.0, 0.0)):
        idx = len(self.contacts)
        lo = self._surface_coord(bp, min_pos[0])
        hi = self._surface_coord(bp, max_pos[0])
        n = len(self.bnd[bp])
        if not (0 <= lo < n and 0 <= hi < n):
            raise ValueError("contact position out of bounds")
        self.bnd[bp][lo:hi + 1] = idx
        if ctype in (OHMIC, SCHOTTKY):  # updateAllOccurences
            for c in range(lo, hi + 1):
                if bp // 2 == 0:
                    x, y = (0 if bp == XMIN else self.nx - 1), c
                else:
                    x, y = c, (0 if bp == YMIN else self.ny - 1)
                for b2 in range(4):
                    if self._on_boundary(x, y, b2):
                        self.bnd[b2][y if b2 < 2 else x] = idx
        self.contacts.append((ctype, float(voltage), tuple(float(p) for p in par)))
        return idx

    def addOhmicContact(self, boundary, voltage, min_pos, max_pos):
        return self._add_contact(boundary, OHMIC, voltage, min_pos, max_pos)

    def addGateContact(self, boundary, voltage, min_pos, max_pos, eps_oxide, thickness,
                       barrier):
        return self._add_contact(boundary, GATE, voltage, min_pos, max_pos,
                                 (eps_oxide, thickness, barrier))

    def getDopingRegionDoping(self, r):
        return self.region_doping.get(int(r), self.material.Ni)

    # ---- engine descriptor -------------------------------------------------------
    def desc(self) -> L.DeviceDesc:
        if np.any(self.region < 0):
            bad = int(np.argmax(self.region < 0))
            raise ValueError("Doping regions must be added to every discrete grid point "
                             f"(missing at node {bad})")  # emcSimulation.hpp:234-256
        d = L.DeviceDesc()
        d.nx, d.ny = self.nx, self.ny
        d.hx, d.hy = self.spacing
        d.max_x, d.max_y = self.max_pos
        d.width, d.temperature = self.width, self.temperature
        d.ni, d.eps_r = self.material.Ni, self.material.epsR
        self._dop = np.ascontiguousarray(self.doping, np.float64)
        self._reg = np.ascontiguousarray(self.region, np.int32)
        d.doping, d.region = _dp(self._dop), _ip(self._reg)
        self._bnd = [np.ascontiguousarray(b, np.int32) for b in self.bnd]
        for b in range(4):
            d.boundary_contact[b] = _ip(self._bnd[b])
        nc = len(self.contacts)
        self._ct = np.array([c[0] for c in self.contacts] or [0], np.int32)
        self._cv = np.array([c[1] for c in self.contacts] or [0.0])
        self._cp = np.array([p for c in self.contacts for p in c[2]] or [0.0, 0.0, 0.0])
        d.n_contacts = nc
        d.contact_type, d.contact_voltage, d.contact_param = _ip(self._ct), _dp(self._cv), \
            _dp(self._cp)
        return d


class DeviceSimulation:
    """emcSimulation on the GPU engine.

    sim = DeviceSimulation(device, electron_type, scheme=CIC, dt=1e-16, ...)
    sim.calcEquilibriumCharacteristics()
    sim.performEMCStep() / sim.execute(n_steps)
    sim.current()  # average terminal current per contact [A]
    """

    def __init__(self, device: Device, particle_type, scheme=NGP, dt=1e-16, seed=1,
                 capacity=None, precision="fp64", carriers_per_particle=1.0,
                 potential_init=False, round_counts=False, tau_region_is_valley=False,
                 poisson_rtol=1e-8, poisson_max_cycles=60, poisson_fp32=True, poisson_smooth=0,
                 stream=0, poisson_update_tol=0.0):
        self._lib = L.lib()
        self.device = device
        self.type = particle_type
        self.dt = float(dt)
        self.nc = len(device.contacts)
        self.potential_init = potential_init
        self.round_counts = round_counts
        self.carriers = float(carriers_per_particle)
        if capacity is None:
            vol = device.getCellVolume()
            capacity = int(1.6 * max(np.sum(np.abs(device.doping)), 1.0) * vol) + 4096
        self._md = particle_type.model_desc(region_doping=device.getDopingRegionDoping)
        self._dd = device.desc()
        cfg = L.DeviceConfig()
        cfg.pm_scheme = scheme
        cfg.tau_region_is_valley = int(tau_region_is_valley)
        cfg.capacity = int(capacity)
        cfg.dt = self.dt
        cfg.charge = particle_type.getCharge()
        cfg.carriers_per_particle = self.carriers
        cfg.seed = seed
        cfg.stream = stream
        cfg.poisson_max_cycles = poisson_max_cycles
        cfg.poisson_rtol = poisson_rtol
        cfg.poisson_smooth = poisson_smooth
        cfg.poisson_fp32 = int(poisson_fp32)
        # electronVWD rounds both the initial and the expected contact counts
        cfg.round_expected = int(round_counts)
        cfg.poisson_update_tol = float(poisson_update_tol)
        self.cfg = cfg
        self.precision = L.FP64 if precision in ("fp64", L.FP64) else L.FP32
        h = C.c_void_p()
        L.check(self._lib.emcg_device_create(C.byref(self._md), C.byref(self._dd),
                                             C.byref(cfg), self.precision, C.byref(h)))
        self.h = h
        self.step_index = 0
        self.netto = []
        self.transient_steps = 0
        # emcSimulationResults: averages, netto counts and current per step
        self.results = R.SimulationResults(
            device.nx, device.ny, device.getThermalVoltage(), device.material.Ni,
            self.carriers * particle_type.getCharge() / self.dt,
            getattr(particle_type, "getName", lambda: "Electrons")())
        self.poisson_info = None

    def close(self):
        if getattr(self, "h", None):
            self._lib.emcg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- scatter tables --------------------------------------------------------
    def reinitScatterTables(self, raw=None):
        """The particle type's scatterHandler.reinitScatterTables()
        (include/emcScatterHandler.hpp:100-108) on the GPU, before the next
        step: raw are the refilled rates (host array or CUDA float64 tensor);
        None refills them from the mechanisms now."""
        self._rates_keep = update_rates(self._lib, self.h, 0, raw, self.type)

    def get_rates(self):
        """The engine's normalised tables (raw layout) and tau per table set."""
        return get_rates(self._lib, self.h, 0, self.type)

    # ---- grids -----------------------------------------------------------------
    def get_grid(self, which):
        out = np.zeros(self.device.nx * self.device.ny)
        L.check(self._lib.emcg_device_get_grid(self.h, which, _dp(out)))
        return out

    def set_grid(self, which, values):
        v = np.ascontiguousarray(values, np.float64)
        L.check(self._lib.emcg_device_set_grid(self.h, which, _dp(v)))

    potential = property(lambda self: self.get_grid(L.GRID_POTENTIAL))
    concentration = property(lambda self: self.get_grid(L.GRID_CONC))

    # ---- stages ----------------------------------------------------------------
    def poisson(self, equilibrium=False, reset_bc=True):
        rel, cyc = C.c_double(), C.c_int32()
        L.check(self._lib.emcg_device_poisson(self.h, int(equilibrium), int(reset_bc),
                                              C.byref(rel), C.byref(cyc)))
        self.poisson_info = (rel.value, cyc.value)
        return self.poisson_info

    def efield(self):
        L.check(self._lib.emcg_device_efield(self.h))

    def surface_kat(self, boundary, k, pos, step=0):
        """scatterParticleAtBoundary at one boundary for independent particles
        (k: n x 3, pos: n x 2); returns the new (k, pos)."""
        kk = np.ascontiguousarray(np.asarray(k, np.float64).T).copy()
        pp = np.ascontiguousarray(np.asarray(pos, np.float64).T).copy()
        L.check(self._lib.emcg_device_surface_kat(self.h, int(boundary), kk.shape[1], _dp(kk),
                                                  _dp(pp), int(step)))
        return kk.T.copy(), pp.T.copy()

    def move(self, step=None):
        netto = np.zeros(max(self.nc, 1), np.int32)
        s = self.step_index if step is None else step
        L.check(self._lib.emcg_device_move(self.h, s, _ip(netto)))
        return netto[:self.nc]

    def contacts(self, step=None):
        ri = np.zeros(max(self.nc, 1), np.int32)
        s = self.step_index if step is None else step
        L.check(self._lib.emcg_device_contacts(self.h, s, _ip(ri)))
        return ri[:self.nc]

    def assign(self):
        L.check(self._lib.emcg_device_assign(self.h))

    def init_particles(self):
        L.check(self._lib.emcg_device_init(self.h, int(self.potential_init),
                                           int(self.round_counts)))

    def set_replay(self, phase, words, offsets):
        w = np.ascontiguousarray(np.asarray(words, np.uint64))
        o = np.ascontiguousarray(np.asarray(offsets, np.int64))
        self._rk = getattr(self, "_rk", {})
        self._rk[phase] = (w, o)
        L.check(self._lib.emcg_device_set_replay(
            self.h, phase, w.ctypes.data_as(C.POINTER(C.c_uint64)), len(w),
            o.ctypes.data_as(C.POINTER(C.c_int64)), len(o)))

    # ---- particles ---------------------------------------------------------------
    def num_particles(self):
        return int(self._lib.emcg_num_particles(self.h, 0))

    def get_state(self) -> ParticleState:
        st = ParticleState(self.num_particles())
        d = st.desc()
        L.check(self._lib.emcg_get_state(self.h, 0, C.byref(d)))
        return st

    def set_state(self, st: ParticleState):
        d = st.desc()
        L.check(self._lib.emcg_set_state(self.h, 0, C.byref(d)))

    # ---- emcSimulation -------------------------------------------------------------
    def calcEquilibriumCharacteristics(self):
        """include/emcSimulation.hpp:139-146"""
        self.poisson(equilibrium=True, reset_bc=True)
        self.efield()
        self.init_particles()
        self.assign()

    def performEMCStep(self, n_steps=1):
        """include/emcSimulation.hpp:164-193 (non-FMM branch), n_steps times."""
        netto = np.zeros((n_steps, max(self.nc, 1)), np.int32)
        L.check(self._lib.emcg_device_step(self.h, n_steps, self.step_index, _ip(netto)))
        self._record(netto[:, :self.nc])
        return netto[:, :self.nc]

    def _record(self, rows):
        for r in rows:
            if self.step_index >= self.transient_steps:  # updateCurrent: non-transient steps
                self.results.update_current(r)
            self.netto.append(r)
            self.step_index += 1

    @staticmethod
    def performEMCStepMany(sims, n_steps=1):
        """performEMCStep on several simulations at once (e.g. a bias sweep):
        the library steps each on its own stream from its own host thread.
        Every simulation must be at the same step index."""
        sims = list(sims)
        if not sims:
            return []
        s0 = sims[0].step_index
        if any(x.step_index != s0 for x in sims):
            raise ValueError("simulations of a batch must be at the same step")
        lib = sims[0]._lib
        outs = [np.zeros((n_steps, max(x.nc, 1)), np.int32) for x in sims]
        hs = (C.c_void_p * len(sims))(*[x.h.value for x in sims])
        ptrs = (C.POINTER(C.c_int32) * len(sims))(*[_ip(o) for o in outs])
        L.check(lib.emcg_device_step_many(hs, len(sims), n_steps, s0, ptrs))
        res = []
        for x, o in zip(sims, outs):
            x._record(o[:, :x.nc])
            res.append(o[:, :x.nc])
        return res

    def execute(self, n_steps, transient_steps=0, steps_for_avg=0, output_prefix=None):
        """emcSimulation::execute (include/emcSimulation.hpp:106-127): equilibrium,
        n_steps steps, the potential and concentration averaged over the last
        steps_for_avg steps, the current over the steps after transient_steps.
        With output_prefix the reference's files are written: the "Eq"
        results, then the current table, averages and the "Final" particles."""
        self.transient_steps = int(transient_steps)
        self.calcEquilibriumCharacteristics()
        if output_prefix is not None:
            R.ensure_dir(output_prefix)
            self.writeCurrentResultsToFiles(output_prefix, "Eq")
        steps_for_avg = min(int(steps_for_avg), n_steps)
        first = n_steps - steps_for_avg
        if first > 0:
            self.performEMCStep(first)
        for _ in range(steps_for_avg):
            self.performEMCStep(1)
            self.results.update_average(self.potential, self.concentration)
        if output_prefix is not None:
            self.writeFinalResults(output_prefix)
        return np.array(self.netto[-n_steps:]) if n_steps else np.zeros((0, self.nc), np.int32)

    # ---- output (emcSimulation.hpp:222-230) ---------------------------------------
    def writeCurrentResultsToFiles(self, prefix, suffix):
        """Potential, concentration, E field and particles now, as the reference
        writes them."""
        self.results.write_current_results(prefix, suffix, self.potential, self.concentration,
                                           self.get_grid(L.GRID_EX), self.get_grid(L.GRID_EY))
        self.print(prefix, suffix)

    def writeFinalResults(self, prefix):
        """Current table, averaged concentration and potential, final particles."""
        self.results.write_final_results(prefix, self.dt, self.transient_steps * self.dt)
        self.print(prefix, "Final")

    def print(self, prefix, suffix):
        """emcBasicParticleHandler::print: the particle dump."""
        R.write_particles(f"{prefix}{self.results.name}{suffix}.txt", self.device.max_pos,
                          self.get_state())

    def timing(self):
        a, b = C.c_double(), C.c_double()
        L.check(self._lib.emcg_device_timing(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def poisson_mode(self, mode=-1):
        """Select (1 cluster, 0 multi-launch) or query (-1) the Poisson execution;
        returns the CTAs per cluster in use (0: multi-launch)."""
        cs = C.c_int32()
        L.check(self._lib.emcg_device_poisson_mode(self.h, int(mode), C.byref(cs)))
        return cs.value

    def set_poisson_cluster(self, max_ctas=0):
        """Bound the CTAs of the single-launch Poisson cluster (0: none);
        returns the cluster size in use (0: multi-launch path)."""
        cs = C.c_int32()
        L.check(self._lib.emcg_device_set_poisson_cluster(self.h, int(max_ctas), C.byref(cs)))
        return cs.value

    def set_poisson(self, rtol=None, max_cycles=None, update_tol=None):
        """Poisson settings: relative-residual target, Newton-step limit, and the
        reference SOR's update tolerance in volts (0: off)."""
        L.check(self._lib.emcg_device_set_poisson(
            self.h, -1.0 if rtol is None else float(rtol),
            -1 if max_cycles is None else int(max_cycles),
            -1.0 if update_tol is None else float(update_tol)))

    def poisson_counts(self):
        """(V-cycles, solves) of the last performEMCStep call."""
        a, b = C.c_int64(), C.c_int64()
        L.check(self._lib.emcg_device_poisson_counts(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def current(self, transient_steps=0):
        """Average current per contact [A]: netto particles per step times
        carriers * charge / dt (emcSimulationResults::updateCurrent, :125-150)."""
        nt = np.array(self.netto[transient_steps:], np.float64)
        if len(nt) == 0:
            return np.zeros(self.nc)
        return nt.mean(axis=0) * self.carriers * self.type.getCharge() / self.dt
