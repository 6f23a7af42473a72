"""Host-side band and scattering model: valleys, scatter mechanisms, rate
tables and the particle type that owns them.

Mirrors the reference classes whose tables the engine consumes:
  emcNonParabolicAnisotropValley   include/ValleyTypes/emcNonParabolicAnistropValley.hpp
  emcAcousticScatterMechanism      include/ScatterMechanisms/emcAcousticScatterMechanism.hpp
  emcZeroOrderInterValley*         include/ScatterMechanisms/emcZeroOrderInterValleyScatterMechanism.hpp
  emcFirstOrderInterValley*        include/ScatterMechanisms/emcFirstOrderInterValleyScatterMechanism.hpp
  emcCoulombScatterMechanism       include/ScatterMechanisms/emcCoulombScatterMechanism.hpp
  emcScatterHandler (tables)       include/emcScatterHandler.hpp
  emcElectron / emcParticleType    include/ParticleType/
Rates are evaluated with the same scalar libm calls and operation order as the
reference so that the tables match the reference's doubles.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

# include/emcConstants.hpp:12-24
PI = 3.14159265358979323846
Q = 1.60219e-19
KB = 1.38066e-23
HBAR = 1.05459e-34
EPS0 = 8.85419e-12
ME = 9.11e-31


@dataclass
class Material:
    """include/emcMaterial.hpp:13-38"""
    epsR: float
    rho: float
    Ni: float
    velSound: float
    bandGap: float


def silicon_material() -> Material:
    """examples/SiliconFunctions.hpp:15-19, 242-244"""
    return Material(11.8, 2329.0, 1.45e16, 9040.0, 1.15)


def thermal_voltage(T: float) -> float:
    """include/emcDevice.hpp:87 (kB / q * T)"""
    return KB / Q * T


def _normalize(d):
    s = 0.0
    for x in d:
        s += x * x
    n = math.sqrt(s)
    return list(d) if n == 0.0 else [x / n for x in d]


class NonParabolicAnisotropValley:
    """Kane non-parabolic valley with anisotropic masses (:22-204)."""

    def __init__(self, rel_mass, particle_mass, deg, alpha, bottom=0.0):
        self.rel_mass = [float(x) for x in rel_mass]
        self.particle_mass = float(particle_mass)
        self.deg = int(deg)
        self.alpha = float(alpha)
        self.bottom = float(bottom)
        ident = [1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0]
        self.rot = [list(ident) for _ in range(self.deg)]
        dos = 1.0
        for m in self.rel_mass:
            dos = dos * m
        self.eff_mass_dos = math.pow(dos, 1.0 / 3.0) * self.particle_mass  # :185-188
        acc = 0.0
        for m in self.rel_mass:
            acc += 1.0 / m
        self.eff_mass_cond = 3.0 * self.particle_mass / acc  # :190-193
        self.vogt = [math.sqrt(self.eff_mass_cond / (m * self.particle_mass))
                     for m in self.rel_mass]  # :198-204

    def setSubValleyEllipseCoordSystem(self, sub, d1, d2, d3):
        """:68-80 -- rows of the rotation are the normalised axes"""
        if not 0 <= sub < self.deg:
            raise ValueError("Using invalid subvalley index.")
        dot = lambda a, b: a[0] * b[0] + a[1] * b[1] + a[2] * b[2]  # noqa: E731
        if dot(d1, d2) != 0 or dot(d1, d3) != 0 or dot(d2, d3) != 0:
            raise ValueError("The given coordinate system for a subvalley is not orthogonal")
        self.rot[sub] = _normalize(d1) + _normalize(d2) + _normalize(d3)

    def getEffMassDOS(self, energy=0.0):
        return self.eff_mass_dos * math.pow(1 + 2 * self.alpha * energy, 3.0)

    def getEffMassCond(self, energy=0.0):
        return self.eff_mass_cond * (1 + 2 * energy * self.alpha)

    def getGamma(self, energy):
        return energy * (1 + self.alpha * energy)

    def getNormWaveVec(self, energy):
        return math.sqrt(2 * self.eff_mass_cond * self.getGamma(energy) * Q) / HBAR

    def getEnergy(self, k):
        sq = 0.0
        for x in k:
            sq += x * x
        g = HBAR * HBAR * sq / (self.eff_mass_cond * Q)
        return g / (1 + math.sqrt(1 + 2 * self.alpha * g))

    def desc(self) -> L.ValleyDesc:
        d = L.ValleyDesc()
        d.deg = self.deg
        for i in range(3):
            d.rel_mass[i] = self.rel_mass[i]
        d.particle_mass = self.particle_mass
        d.alpha = self.alpha
        d.bottom = self.bottom
        for s in range(self.deg):
            for i in range(9):
                d.rot[s][i] = self.rot[s][i]
        return d


class ScatterMechanism:
    """Base of the mechanisms (include/ScatterMechanisms/emcScatterMechanism.hpp:17-53)."""
    kind = -1

    def __init__(self, idx_valley: int):
        self.idx_valley = int(idx_valley)
        self.valleys: list = []

    def getScatterRate(self, energy: float, region: int) -> float:  # pragma: no cover
        raise NotImplementedError

    def getName(self) -> str:  # pragma: no cover
        raise NotImplementedError

    def desc(self, particle_type) -> L.MechDesc:
        d = L.MechDesc()
        d.kind = self.kind
        d.valley = self.idx_valley
        d.final_valley = self.idx_valley
        return d


class AcousticScatterMechanism(ScatterMechanism):
    """Intravalley acoustic phonons, elastic and isotropic (:68-127)."""
    kind = L.MECH_ACOUSTIC

    def __init__(self, idx_valley, sigma, temperature, rho, vel_sound):
        super().__init__(idx_valley)
        cL = rho * math.pow(vel_sound, 2.0)
        self.scatter_const = (math.sqrt(2.0 * Q) * math.pow(sigma * Q, 2.0) * KB * temperature /
                              (PI * cL * math.pow(HBAR, 4.0)))

    def getName(self):
        return "Acoustic"

    def getScatterRate(self, energy, region=0):
        v = self.valleys[self.idx_valley]
        md, alpha, g = v.getEffMassDOS(), v.alpha, v.getGamma(energy)
        return self.scatter_const * math.pow(md, 3.0 / 2.0) * math.sqrt(g) * (2 * alpha * energy + 1.0)


def _nr_phonons(ph_energy, temperature):
    return 1.0 / (math.exp(Q * ph_energy / (KB * temperature)) - 1.0)


class _InterValley(ScatterMechanism):
    absorption = True
    first_order = False

    def __init__(self, name_suffix, idx_valley, final_sub, def_pot, phonon_energy, temperature,
                 rho, idx_final_valley=None):
        super().__init__(idx_valley)
        self.name_suffix = name_suffix
        self.final_sub = {int(k): [int(x) for x in v] for k, v in dict(final_sub).items()}
        self.nF = len(self.final_sub[0])
        self.idx_final_valley = idx_valley if idx_final_valley is None else int(idx_final_valley)
        self.phonon_energy = float(phonon_energy)
        nF = float(self.nF)
        if self.first_order:  # emcFirstOrderInterValleyScatterMechanism.hpp:11-20
            r = (nF * math.sqrt(2.0) * math.pow(Q, 5.0 / 2.0) * math.pow(def_pot, 2.0) /
                 (PI * rho * math.pow(HBAR, 4.0) * phonon_energy))
        else:  # emcZeroOrderInterValleyScatterMechanism.hpp:12-21
            r = (nF * math.sqrt(Q) * math.pow(def_pot / HBAR, 2.0) * Q /
                 (PI * rho * phonon_energy * math.sqrt(2.0)))
        n = _nr_phonons(phonon_energy, temperature)
        self.scatter_const = r * n if self.absorption else r * (n + 1)

    @property
    def delta_valley(self):
        return (self.valleys[self.idx_final_valley].bottom -
                self.valleys[self.idx_valley].bottom)

    def getName(self):
        order = "First" if self.first_order else "Zero"
        kind = "Absorption" if self.absorption else "Emission"
        return f"{order}InterValley{kind}{self.name_suffix}"

    def getScatterRate(self, energy, region=0):
        vi, vf = self.valleys[self.idx_valley], self.valleys[self.idx_final_valley]
        dv = vf.bottom - vi.bottom
        ef = (energy + self.phonon_energy - dv) if self.absorption else \
            (energy - self.phonon_energy - dv)
        if ef > 0:
            md, alpha = vf.getEffMassDOS(), vf.alpha
            if self.first_order:
                g, gf = vi.getGamma(energy), vf.getGamma(ef)
                return (self.scatter_const * math.pow(md, 5.0 / 2.0) * math.sqrt(gf) *
                        (2 * alpha * ef + 1.0) * (g + gf))
            g = vf.getGamma(ef)
            return self.scatter_const * math.pow(md, 3.0 / 2.0) * math.sqrt(g) * (2 * alpha * ef + 1.0)
        return 0.0

    def desc(self, particle_type):
        d = super().desc(particle_type)
        d.final_valley = self.idx_final_valley
        d.n_final = self.nF
        dv = self.delta_valley
        # absorption: energy += (phononEnergy - deltaValley); emission: -= (ph + dv)
        d.shift = (self.phonon_energy - dv) if self.absorption else -(self.phonon_energy + dv)
        deg = particle_type.valleys[self.idx_valley].deg
        for s in range(deg):
            for f in range(self.nF):
                d.final_sub[s][f] = self.final_sub[s][f]
        return d


class ZeroOrderInterValleyAbsorptionScatterMechanism(_InterValley):
    kind = L.MECH_ZERO_IV_ABS
    absorption, first_order = True, False


class ZeroOrderInterValleyEmissionScatterMechanism(_InterValley):
    kind = L.MECH_ZERO_IV_EMI
    absorption, first_order = False, False


class FirstOrderInterValleyAbsorptionScatterMechanism(_InterValley):
    kind = L.MECH_FIRST_IV_ABS
    absorption, first_order = True, True


class FirstOrderInterValleyEmissionScatterMechanism(_InterValley):
    kind = L.MECH_FIRST_IV_EMI
    absorption, first_order = False, True


class CoulombScatterMechanism(ScatterMechanism):
    """Brooks-Herring ionised-impurity scattering (:11-60)."""
    kind = L.MECH_COULOMB

    def __init__(self, idx_valley, epsR, temperature, region_doping):
        super().__init__(idx_valley)
        eps = EPS0 * epsR
        Vt = thermal_voltage(temperature)
        self.sc1 = math.sqrt(2 * Q) * math.pow(KB * temperature, 2.0) / (PI * math.pow(HBAR, 4.0))
        self.sc2 = 8 * eps * Vt / (HBAR * HBAR)
        self.region_doping = region_doping  # callable region -> net doping

    def getName(self):
        return "Coulomb"

    def getScatterRate(self, energy, region=0):
        doping = math.fabs(self.region_doping(region))
        v = self.valleys[self.idx_valley]
        md, mc, alpha, g = v.getEffMassDOS(), v.getEffMassCond(), v.alpha, v.getGamma(energy)
        return (self.sc1 * math.pow(md, 3.0 / 2.0) / doping * math.sqrt(g) *
                (2 * alpha * energy + 1.0) / (1 + (self.sc2 * mc * g / doping)))

    def desc(self, particle_type):
        d = super().desc(particle_type)
        d.coulomb_sc2 = self.sc2
        return d


class ScatterHandler:
    """Rate tables per (valley, region) (include/emcScatterHandler.hpp:47-289)."""

    def __init__(self, n_levels=1000, max_energy=4.0):
        self.n_levels = int(n_levels)
        self.max_energy = float(max_energy)
        self.dE = self.max_energy / self.n_levels
        self.mechanisms: list = []
        self.table_mechs: dict = {}  # (valley, region) -> [mechanism index]
        self.raw: dict = {}
        self.norm: dict = {}
        self.tau: dict = {}
        self.grainScatterMech = None
        self.grainTau = 1.0  # include/emcScatterHandler.hpp:61-62
        self.surfaceScatterMechanisms = [None] * 4  # per boundary, :63-65, 114-124

    def setGrainScatterMechanism(self, mech):
        self.grainScatterMech = mech

    def getGrainTau(self):
        return self.grainTau

    def addScatterMechanism(self, mech, regions):
        idx = len(self.mechanisms)
        self.mechanisms.append(mech)
        for r in regions:
            self.table_mechs.setdefault((mech.idx_valley, int(r)), []).append(idx)

    def _fill(self, key):
        """fillScatterTables (:220-235) for one (valley, region) table set: the
        rate of each of its mechanisms at (level + 1) dE."""
        v, r = key
        dE, L_ = self.dE, self.n_levels
        rows = []
        for mi in self.table_mechs[key]:
            m = self.mechanisms[mi]
            rows.append([m.getScatterRate((l + 1) * dE, r) for l in range(L_)])
        return np.array(rows, dtype=np.float64).reshape(len(rows), L_)

    def fill_rates(self) -> np.ndarray:
        """The refilled rates of every table set in key order, table-major and
        concatenated: the raw layout the engine's rate-table rebuild takes."""
        chunks = [self._fill(key).reshape(-1) for key in sorted(self.table_mechs)]
        return np.concatenate(chunks) if chunks else np.zeros(0)

    def fill_size(self) -> int:
        """Number of rates in the concatenated raw layout."""
        return sum(len(m) for m in self.table_mechs.values()) * self.n_levels

    def reinitScatterTables(self):
        """reinitScatterTables (:100-108): refill and renormalise, no files."""
        self.raw.clear()
        self.norm.clear()
        self.tau.clear()
        self.initScatterTables()

    def initScatterTables(self):
        """fillScatterTables + renormalizeTables (:220-235, :248-273)"""
        for key in sorted(self.table_mechs):
            rows = self.table_mechs[key]
            raw = self._fill(key)
            self.raw[key] = raw
            if len(rows) == 0:
                self.tau[key] = 2e-15
                self.norm[key] = raw
                continue
            cum = np.cumsum(raw, axis=0)  # sequential in table order, exact like std::plus
            mx = float(cum[-1].max())
            self.norm[key] = cum / mx
            self.tau[key] = 1.0 / mx
        if self.grainScatterMech is not None:  # :233-234
            self.grainTau = 1.0 / self.grainScatterMech.getScatterRate()

    def getTau(self, region, valley):
        return self.tau.get((valley, region), 2e-15)


class GrainScatterMechanism:
    """emcGrainScatterMechanism (include/emcGrainScatterMechanism.hpp:16-80):
    grains met at a mean rate; a particle is transmitted (new direction in the
    hemisphere of k) with the transmission probability, else reflected (the
    opposite hemisphere), |k| kept.  The scattering itself runs in the engine
    (grainScatter); this holds its two parameters."""

    def __init__(self, transmissionProb=0.5, scatterRate=1e14):
        self.transmissionProb = float(transmissionProb)
        self.scatterRate = float(scatterRate)

    def getScatterRate(self):
        return self.scatterRate


class ConstantSurfaceScatterMechanism:
    """emcConstantSurfaceScatterMechanism (include/SurfaceScatterMechanisms/
    emcConstantSurfaceScatterMechanism.hpp): at its boundary a particle is
    reflected specularly with the specularity parameter's probability, else
    diffusely (polar angle asin(sqrt(u)) from the inward normal).  max_pos is
    the reference constructor's; the engine takes the device's extent."""

    kind = L.SURFACE_CONSTANT

    def __init__(self, specularityParam, max_pos=None):
        self.param = float(specularityParam)


class MomentumDependentSurfaceScatterMechanism:
    """emcMomentumDependentSurfaceScatterMechanism (include/
    SurfaceScatterMechanisms/emcMomentumDependentSurfaceScatterMechanism.hpp):
    diffuse with probability 1 - exp(-(2 h k_perp)^2) for roughness height h
    [m], else specular."""

    kind = L.SURFACE_ROUGHNESS

    def __init__(self, roughnessHeight, max_pos=None):
        self.param = float(roughnessHeight)


class Electron:
    """Electron particle type (include/ParticleType/emcElectron.hpp:15-105):
    valleys + scatter handler; charge -q, mass m0."""

    def __init__(self, n_levels=1000, max_energy=4.0):
        self.valleys: list = []
        self.scatterHandler = ScatterHandler(n_levels, max_energy)

    def getName(self):
        return "Electrons"

    def getMass(self):
        return ME

    def getCharge(self):
        return -Q

    def getNrValleys(self):
        return len(self.valleys)

    def addValley(self, valley):
        if valley.deg < 1 or valley.alpha < 0:
            raise ValueError("invalid valley")
        self.valleys.append(valley)

    def addScatterMechanism(self, regions, mech):
        if not 0 <= mech.idx_valley < len(self.valleys):
            raise ValueError("Used index for Valley is invalid.")
        mech.valleys = self.valleys
        self.scatterHandler.addScatterMechanism(mech, regions)

    def initScatterTables(self):
        self.scatterHandler.initScatterTables()

    def setGrainScatterMechanism(self, mech):
        """emcParticleType::setGrainScatterMechanism (emcParticleType.hpp:134-138);
        the grain free-flight constant follows at the next table build."""
        self.scatterHandler.setGrainScatterMechanism(mech)

    def getGrainTau(self):
        return self.scatterHandler.getGrainTau()

    def setSurfaceScatterMechanism(self, boundary, mech):
        """emcParticleType::setSurfaceScatterMechanism(boundaryPosition,
        mechanism) (emcParticleType.hpp:155-166); boundary 0..3 = XMIN, XMAX,
        YMIN, YMAX.  Used by device simulations."""
        if not 0 <= int(boundary) < 4:
            raise ValueError("boundary must be XMIN, XMAX, YMIN or YMAX")
        self.scatterHandler.surfaceScatterMechanisms[int(boundary)] = mech

    def getTau(self, valley, region):
        return self.scatterHandler.getTau(region, valley)

    def raw_rates(self) -> np.ndarray:
        """The rates of the scatter tables refilled now from the mechanisms
        (fillScatterTables without renormalisation), in the layout of the
        engine's rate-table rebuild."""
        return self.scatterHandler.fill_rates()

    # ---- engine descriptor -------------------------------------------------
    def model_desc(self, region_doping=None):
        """emcg_model_desc of this particle type; keeps the backing buffers
        alive on the returned object (attribute `_keep`)."""
        h = self.scatterHandler
        if not h.norm:
            self.initScatterTables()
        nV = len(self.valleys)
        va = (L.ValleyDesc * nV)(*[v.desc() for v in self.valleys])
        nM = len(h.mechanisms)
        ma = (L.MechDesc * max(nM, 1))(*[m.desc(self) for m in h.mechanisms])
        keys = sorted(h.table_mechs)
        ta = (L.TablesetDesc * max(len(keys), 1))()
        chunks = []
        for i, key in enumerate(keys):
            t = ta[i]
            t.valley, t.region = key
            mechs = h.table_mechs[key]
            t.n_tables = len(mechs)
            for j, mi in enumerate(mechs):
                t.mech[j] = mi
            t.tau_max = h.tau[key]
            chunks.append(h.norm[key].reshape(-1))
        tables = np.ascontiguousarray(np.concatenate(chunks) if chunks else np.zeros(1))
        d = L.ModelDesc()
        d.n_valleys, d.n_mechs, d.n_tablesets = nV, nM, len(keys)
        d.n_levels, d.max_energy, d.grain_tau = h.n_levels, h.max_energy, h.getGrainTau()
        if h.grainScatterMech is not None:
            d.grain, d.grain_transmission = 1, h.grainScatterMech.transmissionProb
        for b, sm in enumerate(h.surfaceScatterMechanisms):
            if sm is not None:
                d.surface_kind[b], d.surface_param[b] = sm.kind, sm.param
        d.valleys, d.mechs, d.tablesets = va, ma, ta
        d.tables = tables.ctypes.data_as(C.POINTER(C.c_double))
        for r in range(L.MAX_REGIONS):
            d.region_doping[r] = region_doping(r) if region_doping else 1.45e16
        d._keep = (va, ma, ta, tables)
        return d


# ---- silicon (examples/SiliconFunctions.hpp) ----------------------------------
SI_FRAMES = [((1, 0, 0), (0, 1, 0), (0, 0, 1)),
             ((0, 1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (0, 1, 0), (1, 0, 0))]
FINAL_G = {0: [0], 1: [1], 2: [2]}
FINAL_F = {0: [1, 1, 2, 2], 1: [0, 0, 2, 2], 2: [0, 0, 1, 1]}

# Intervalley phonons of Jacoboni & Reggiani, Rev. Mod. Phys. 55, 645 (1983),
# silicon: (name, f-type, phonon temperature [K], coupling [eV/m]); used as
# zero-order couplings in the bulk benchmark model.
JACOBONI_SI = [("G1", False, 140., 0.5e10), ("G2", False, 215., 0.8e10),
               ("G3", False, 720., 11.e10), ("F1", True, 220., 0.3e10),
               ("F2", True, 550., 2.0e10), ("F3", True, 685., 2.0e10)]


def add_x_valley(pt: Electron, mt: float = 0.196, ml: float = 0.916, alpha: float = 0.5):
    """Silicon::addXValley (:249-261): three paired Delta valleys."""
    v = NonParabolicAnisotropValley([ml, mt, mt], pt.getMass(), 3, alpha)
    for s, (a, b, c) in enumerate(SI_FRAMES):
        v.setSubValleyEllipseCoordSystem(s, a, b, c)
    pt.addValley(v)
    return v


def silicon_electron(model: str = "jacoboni", temperature: float = 300.0, n_levels: int = 1000,
                     max_energy: float = 1.0, regions=(0,), mt=None, coulomb: bool = False,
                     region_doping=None, zero_order=True, first_order=True,
                     grain=None) -> Electron:
    """Silicon electrons with one of two mechanism sets:

    "refbulk":  the reference bulk example (acoustic + zero-order f/g at 60 meV
                + first-order f/g; m_t = 0.196), SiliconFunctions.hpp:224-333.
    "jacoboni": acoustic (9 eV) + 3 g + 3 f zero-order phonons of the
                Jacoboni-Reggiani table; m_t = 0.19.

    grain: (transmission probability, scatter rate [1/s]) of a grain
    mechanism (GrainScatterMechanism), none by default.
    """
    mat = silicon_material()
    pt = Electron(n_levels, max_energy)
    add_x_valley(pt, mt if mt is not None else (0.196 if model == "refbulk" else 0.19))
    regs = list(regions)
    pt.addScatterMechanism(regs, AcousticScatterMechanism(0, 9.0, temperature, mat.rho,
                                                          mat.velSound))
    if model == "refbulk":
        if zero_order:
            for fs, sfx in ((FINAL_F, "F"), (FINAL_G, "G")):
                pt.addScatterMechanism(regs, ZeroOrderInterValleyAbsorptionScatterMechanism(
                    sfx, 0, fs, 5.23e10, 0.06, temperature, mat.rho))
                pt.addScatterMechanism(regs, ZeroOrderInterValleyEmissionScatterMechanism(
                    sfx, 0, fs, 5.23e10, 0.06, temperature, mat.rho))
        if first_order:
            for fs, sfx, D, e in ((FINAL_F, "F", 2.5, 0.023), (FINAL_G, "G", 4.0, 0.018)):
                pt.addScatterMechanism(regs, FirstOrderInterValleyAbsorptionScatterMechanism(
                    sfx, 0, fs, D, e, temperature, mat.rho))
                pt.addScatterMechanism(regs, FirstOrderInterValleyEmissionScatterMechanism(
                    sfx, 0, fs, D, e, temperature, mat.rho))
    elif model == "jacoboni":
        for name, isF, theta, D in JACOBONI_SI:
            e = KB * theta / Q
            fs = FINAL_F if isF else FINAL_G
            pt.addScatterMechanism(regs, ZeroOrderInterValleyAbsorptionScatterMechanism(
                name, 0, fs, D, e, temperature, mat.rho))
            pt.addScatterMechanism(regs, ZeroOrderInterValleyEmissionScatterMechanism(
                name, 0, fs, D, e, temperature, mat.rho))
    else:
        raise ValueError(model)
    if coulomb:
        if region_doping is None:
            raise ValueError("Coulomb scattering needs region_doping")
        pt.addScatterMechanism(regs, CoulombScatterMechanism(0, mat.epsR, temperature,
                                                             region_doping))
    if grain is not None:
        pt.setGrainScatterMechanism(GrainScatterMechanism(*grain))
    pt.initScatterTables()
    return pt
