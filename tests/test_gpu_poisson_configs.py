"""Poisson on the configuration grids against the reference's SOR.

The 2-D resistor (201 x 101 nodes) and the n-MOSFET (401 x 201 nodes, gate
with its Robin term) are solved by the single-launch cluster solve that the
device step uses there: float multigrid V-cycles distributed over the CTAs of
a cluster, inside double Newton steps, to a relative residual of 1e-10.  The
oracle's restatement of the reference's SOR (include/PoissonSolver/
emcSORSolver.hpp:49-197), run to an update below 1e-12 V, gives the same
potential within 1e-7 thermal voltages: equilibrium from asinh(C/2), then
non-equilibrium with a concentration 5 % off equilibrium at random.  A
non-finite concentration ends both solve forms with EMCG_ERR_NONCONVERGED.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-7  # thermal voltages


def _oracle_device(oracle, dev):
    ct = np.array([c[0] for c in dev.contacts], np.int32)
    cv = np.array([c[1] for c in dev.contacts], np.float64)
    cp = np.array([p for c in dev.contacts for p in c[2]], np.float64).reshape(-1, 3)
    od = oracle.Device(dev.nx, dev.ny, dev.spacing[0], dev.spacing[1], dev.width, dev.doping,
                       dev.region, dev.bnd, ct, cv, cp)
    od.set_max(*dev.max_pos)
    return od


def _config_sim(grid, fp32=True):
    import bench
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    if grid == "resistor_201x101":
        dev = bench.resistor_device(D, P)
    else:
        dev = bench.mosfet_device(D, P, 0.5)
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0,
                            regions=list(range(dev.n_regions)), coulomb=True,
                            region_doping=dev.getDopingRegionDoping, first_order=False)
    sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=5, precision="fp32",
                             poisson_rtol=1e-10, poisson_max_cycles=200, poisson_fp32=fp32)
    return dev, sim


@pytest.mark.parametrize("grid,fp32", [("resistor_201x101", True), ("resistor_201x101", False),
                                       ("mosfet_401x201", True)])
def test_config_grid_solve_matches_converged_sor(engine, oracle, grid, fp32):
    from viennaemc_gb300 import _lib as L
    dev, sim = _config_sim(grid, fp32)
    assert sim.poisson_mode() > 1  # the cluster solve, distributed over several CTAs
    od = _oracle_device(oracle, dev)
    pot0 = np.arcsinh(0.5 * dev.doping / dev.material.Ni)
    sim.set_grid(L.GRID_POTENTIAL, pot0)
    rel, _ = sim.poisson(equilibrium=True, reset_bc=True)
    eq = sim.potential
    ref_eq, n_eq = od.sor(pot0, None, 1.8, 1e-12, True)
    assert rel <= 1e-10 and n_eq > 0
    assert np.max(np.abs(eq - ref_eq)) <= TOL, np.max(np.abs(eq - ref_eq))
    rs = np.random.default_rng(3)
    conc = np.exp(ref_eq) * (1 + 0.05 * rs.standard_normal(ref_eq.size))
    sim.set_grid(L.GRID_CONC, conc)
    rel, cyc = sim.poisson(equilibrium=False, reset_bc=True)
    ne = sim.potential
    ref_ne, n_ne = od.sor(ref_eq, conc, 1.8, 1e-12, True)
    assert rel <= 1e-10 and cyc > 0 and n_ne > 100
    assert np.max(np.abs(ne - ref_ne)) <= TOL, np.max(np.abs(ne - ref_ne))
    sim.close()


@pytest.mark.parametrize("mode", [1, 0])
def test_non_finite_concentration_is_reported(engine, mode):
    """A NaN in the concentration: the residual maxima would drop it (fmax),
    so it is counted as an infinite residual and the solve ends as not
    converged, in the cluster (1) and the multi-launch (0) form; the handle
    stays usable."""
    from viennaemc_gb300 import _lib as L
    dev, sim = _config_sim("resistor_201x101")
    sim.poisson_mode(mode)
    pot0 = np.arcsinh(0.5 * dev.doping / dev.material.Ni)
    sim.set_grid(L.GRID_POTENTIAL, pot0)
    sim.poisson(equilibrium=True, reset_bc=True)
    eq = sim.potential
    conc = np.exp(eq)
    conc[dev.nx * 50 + 100] = np.nan
    sim.set_grid(L.GRID_CONC, conc)
    with pytest.raises(L.EmcgError) as ei:
        sim.poisson(equilibrium=False, reset_bc=True)
    assert ei.value.status == -4 and "non-finite" in str(ei.value)
    sim.set_grid(L.GRID_POTENTIAL, eq)
    sim.set_grid(L.GRID_CONC, np.exp(eq))
    rel, _ = sim.poisson(equilibrium=False, reset_bc=True)
    assert rel <= 1e-10
    sim.close()
