"""Output layer against the reference's own files (tests/golden/output_*,
written by the reference's emcSimulationResults and emcBasicParticleHandler
after the last step of the device golden cases): the same data through
viennaemc_gb300.results must give the same bytes."""
import os

import numpy as np
import pytest

from conftest import golden

HERE = os.path.join(os.path.dirname(__file__), "golden")
CASES = [("device_resistor_ngp.npz", "output_resistor_ngp"),
         ("device_mosfet_necvwd.npz", "output_mosfet_necvwd")]


def _ref(dirname, f):
    with open(os.path.join(HERE, dirname, f)) as fh:
        return fh.read()


class _State:
    def __init__(self, g, s):
        self.px, self.py = g[f"s{s}_px"], g[f"s{s}_py"]
        self.kx, self.ky, self.kz = g[f"s{s}_kx"], g[f"s{s}_ky"], g[f"s{s}_kz"]
        self.energy, self.tau = g[f"s{s}_E"], g[f"s{s}_tau"]
        self.sub, self.valley = g[f"s{s}_sub"], g[f"s{s}_valley"]


@pytest.mark.parametrize("case,outdir", CASES)
def test_output_files_match_reference(tmp_path, case, outdir):
    from viennaemc_gb300 import results as R
    g = golden(case)
    geom = g["geom"]
    nx, ny = int(round(geom[0] / geom[2])) + 1, int(round(geom[1] / geom[3])) + 1
    Vt, ni = float(geom[7]), 1.45e16
    steps = int(g["params"][2])
    dt = float(g["params"][1])
    factor = 1.0 * -1.60219e-19 / dt
    res = R.SimulationResults(nx, ny, Vt, ni, factor)
    for s in range(1, steps + 1):
        res.update_current(g[f"netto{s}"])
        res.update_average(g[f"pot{s}"], g[f"conc{s}"])
        assert np.array_equal(res.current[-1], g[f"cur{s}"])
    prefix = str(tmp_path) + "/"
    res.write_current_results(prefix, "Step", g[f"pot{steps}"], g[f"conc{steps}"],
                              g[f"ex{steps}"], g[f"ey{steps}"])
    res.write_final_results(prefix, dt, 0.0)
    R.write_particles(prefix + "ElectronsStep.txt", (geom[0], geom[1]), _State(g, steps))
    ref_files = sorted(os.listdir(os.path.join(HERE, outdir)))
    assert sorted(os.listdir(tmp_path)) == ref_files
    for f in ref_files:
        ours = open(os.path.join(tmp_path, f)).read()
        assert ours == _ref(outdir, f), f
