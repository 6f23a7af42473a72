"""Results and output files of a device simulation.

Mirrors emcSimulationResults (include/emcSimulationResults.hpp): the
potential and concentration averaged over the last steps, the netto particle
count per step and contact, and the current averaged over the non-transient
steps so far.  The writers produce the reference's files byte for byte:

- grids (include/emcOutput.hpp:13-56 and emcGrid::print,
  include/emcGrid.hpp:143-165): the extent, then one line per y with the values
  of that row, x fastest;
- the current table (include/emcOutput.hpp:58-76): per step the time, the
  netto counts, then the currents of every contact;
- the particle dump (emcBasicParticleHandler::print,
  include/ParticleHandler/emcBasicParticleHandler.hpp:193-214).

Numbers are formatted as a C++ ostream formats them by default (six
significant digits, %g).
"""
from __future__ import annotations

import os

import numpy as np


def fmt(v) -> str:
    """A number as std::ostream << v writes it (default float formatting)."""
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return "%g" % float(v)


def grid_text(values, nx: int, ny: int) -> str:
    v = np.asarray(values, np.float64).reshape(ny, nx)
    rows = [" ".join(fmt(x) for x in v[y]) for y in range(ny)]
    return f"{nx} {ny}\n" + "\n".join(rows) + "\n"


def write_grid(path: str, values, nx: int, ny: int) -> None:
    with open(path, "w") as f:
        f.write(grid_text(values, nx, ny))


def current_text(netto, current, step_time: float, start_time: float) -> str:
    lines = []
    for s in range(1, len(current) + 1):
        t = start_time + s * step_time
        parts = [fmt(t)] + [fmt(int(n)) for n in netto[s - 1]] + [fmt(c) for c in current[s - 1]]
        lines.append(" ".join(parts) + "\n")
    return "".join(lines)


def particles_text(max_pos, st, moved: bool = True) -> str:
    """st: ParticleState-like with px, py, kx, ky, kz, energy, sub, valley, tau."""
    out = [f"{fmt(max_pos[0])} {fmt(max_pos[1])}\n"]
    n = len(st.px)
    for i in range(n):
        line = f"{i} {fmt(st.px[i])} {fmt(st.py[i])}"
        if moved:
            line += (f" {fmt(st.kx[i])} {fmt(st.ky[i])} {fmt(st.kz[i])} {fmt(st.energy[i])}"
                     f" {fmt(int(st.sub[i]))} {fmt(int(st.valley[i]))} {fmt(st.tau[i])}")
        out.append(line + ("\n" if i < n - 1 else ""))
    return "".join(out)


class SimulationResults:
    """emcSimulationResults for one particle type on a 2-D device.

    thermal_voltage, ni: the device's (undoNormalizeVoltage / undoNormalizeDoping);
    current_factor: carriers per particle x charge / step time
    (emcSimulationResults.hpp:63-66).
    """

    def __init__(self, nx: int, ny: int, thermal_voltage: float, ni: float,
                 current_factor: float, type_name: str = "Electrons"):
        self.nx, self.ny = nx, ny
        self.Vt, self.Ni = thermal_voltage, ni
        self.factor = current_factor
        self.name = type_name
        self.avg_pot = np.zeros(nx * ny)
        self.avg_conc = np.zeros(nx * ny)
        self.n_avg = 0
        self.netto = []
        self.current = []
        self.netto_sum = None

    def update_average(self, pot, conc) -> None:
        """updateAverageCharacteristics (:80-87): pot normalised (phi / Vt),
        conc normalised (n / Ni)."""
        self.avg_pot += np.asarray(pot, np.float64)
        self.avg_conc += np.asarray(conc, np.float64)
        self.n_avg += 1

    def update_current(self, netto_row) -> None:
        """updateCurrent (:125-150) with netto = removed - (injected - deleted)."""
        row = np.asarray(netto_row, np.int64)
        if self.netto_sum is None:
            self.netto_sum = np.zeros(len(row))
        self.netto.append(row.copy())
        self.netto_sum = self.netto_sum + row.astype(np.float64)
        n = len(self.netto)
        self.current.append(self.netto_sum / n * self.factor)

    def write_current_results(self, prefix: str, suffix: str, pot, conc, ex, ey) -> None:
        """writeCurrentResults (:152-172)."""
        write_grid(f"{prefix}Potential{suffix}.txt", np.asarray(pot) * self.Vt, self.nx, self.ny)
        write_grid(f"{prefix}{self.name}Conc{suffix}.txt", np.asarray(conc) * self.Ni,
                   self.nx, self.ny)
        write_grid(f"{prefix}EFieldX{suffix}.txt", ex, self.nx, self.ny)
        write_grid(f"{prefix}EFieldY{suffix}.txt", ey, self.nx, self.ny)

    def write_final_results(self, prefix: str, step_time: float, start_time: float) -> None:
        """writeFinalResults (:174-201): the current table and the averaged
        concentration and potential."""
        with open(f"{prefix}{self.name}Current.txt", "w") as f:
            f.write(current_text(self.netto, self.current, step_time, start_time))
        n = max(self.n_avg, 1)
        write_grid(f"{prefix}{self.name}ConcAvg.txt", self.avg_conc / n * self.Ni,
                   self.nx, self.ny)
        write_grid(f"{prefix}PotentialAvg.txt", self.avg_pot / n * self.Vt, self.nx, self.ny)


def write_particles(path: str, max_pos, st, moved: bool = True) -> None:
    with open(path, "w") as f:
        f.write(particles_text(max_pos, st, moved))


def ensure_dir(prefix: str) -> None:
    d = os.path.dirname(prefix)
    if d:
        os.makedirs(d, exist_ok=True)
