"""emcg_poisson_solve_noalloc against emcg_device_poisson.

The no-allocation entry point solves the same equation with the same float
multigrid inside double Newton / defect correction, but builds its levels in
its fixed device array from the caller's description on every call; the two
agree up to the rounding of the level coefficients.  Two calls in a row
(equilibrium from asinh(C/2), then non-equilibrium with the reference's
step-1 concentration) check that a call does not depend on what the previous
call left in the array.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from test_gpu_device import _sim
from test_oracle_device_golden import DEVICE_CASES

pytestmark = pytest.mark.gpu
TOL = 1e-8  # thermal voltages; both solvers stop at a relative residual of 1e-10
RTOL, MAX_CYCLES, SMOOTH = 1e-10, 200, 2


def _noalloc(desc, pot, conc, reset_bc=1):
    import torch
    from viennaemc_gb300 import _lib as L
    d_pot = torch.tensor(np.asarray(pot), dtype=torch.float64, device="cuda")
    d_conc = None if conc is None else torch.tensor(np.asarray(conc), dtype=torch.float64,
                                                    device="cuda")
    torch.cuda.synchronize()
    rel, cyc = C.c_double(), C.c_int32()
    s = L.lib().emcg_poisson_solve_noalloc(
        C.byref(desc), C.c_void_p(d_pot.data_ptr()),
        None if d_conc is None else C.c_void_p(d_conc.data_ptr()), reset_bc, SMOOTH, RTOL,
        MAX_CYCLES, None, C.byref(rel), C.byref(cyc))
    return s, d_pot.cpu().numpy(), rel.value, cyc.value


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_noalloc_matches_allocating_solver(engine, case):
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    sim, dev, pt = _sim(engine, g, case, poisson_rtol=RTOL, poisson_fp32=True,
                        poisson_max_cycles=MAX_CYCLES, poisson_smooth=SMOOTH)
    desc = dev.desc()
    # the allocating entry point, twice
    sim.set_grid(L.GRID_POTENTIAL, g["pot_init"])
    rel_a1, cyc_a1 = sim.poisson(equilibrium=True, reset_bc=True)
    eq_a = sim.potential.copy()
    sim.set_grid(L.GRID_POTENTIAL, g["pot_eq"])
    sim.set_grid(L.GRID_CONC, g["conc0"])
    rel_a2, cyc_a2 = sim.poisson(equilibrium=False, reset_bc=True)
    ne_a = sim.potential.copy()
    sim.close()
    # the no-allocation entry point, twice
    s1, eq_n, rel_n1, cyc_n1 = _noalloc(desc, g["pot_init"], None)
    L.check(s1)
    s2, ne_n, rel_n2, cyc_n2 = _noalloc(desc, g["pot_eq"], g["conc0"])
    L.check(s2)
    assert max(rel_a1, rel_a2, rel_n1, rel_n2) <= RTOL
    # same iteration up to rounding (a uniform resistor starts at its equilibrium: 0 cycles)
    assert abs(cyc_n1 - cyc_a1) <= 1 and abs(cyc_n2 - cyc_a2) <= 1, (cyc_n1, cyc_a1, cyc_n2, cyc_a2)
    assert cyc_n2 > 0
    assert np.max(np.abs(eq_n - eq_a)) <= TOL, np.max(np.abs(eq_n - eq_a))
    assert np.max(np.abs(ne_n - ne_a)) <= TOL, np.max(np.abs(ne_n - ne_a))
    # a repeated call gives the same bits: nothing carries over between calls
    s3, eq_n2, _, cyc_n3 = _noalloc(desc, g["pot_init"], None)
    L.check(s3)
    assert cyc_n3 == cyc_n1 and np.array_equal(eq_n2, eq_n)


def test_noalloc_rejects_oversize_grid(engine):
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    from viennaemc_gb300.physics import silicon_material
    dev = D.Device(silicon_material(), (399e-9, 399e-9), (1e-9, 1e-9))  # 400 x 400 nodes
    dev.addConstantDopingRegion((0, 0), (399e-9, 399e-9), 1e24)
    dev.addOhmicContact(D.XMIN, 0.0, (0,), (399e-9,))
    desc = dev.desc()
    assert desc.nx * desc.ny > 131072
    pot = np.full(desc.nx * desc.ny, 0.25)
    s, out, _, _ = _noalloc(desc, pot, None)
    assert s == -1  # EMCG_ERR_ARG
    assert "no-allocation" in L.lib().emcg_last_error().decode()
    assert np.array_equal(out, pot)


def test_noalloc_reports_non_finite_concentration(engine):
    """A NaN in the caller's concentration ends the solve as not converged
    (the residual maxima would otherwise drop it)."""
    from viennaemc_gb300 import _lib as L
    g = golden(DEVICE_CASES[0])
    sim, dev, pt = _sim(engine, g, DEVICE_CASES[0])
    desc = dev.desc()
    conc = np.array(g["conc0"], np.float64)
    conc[len(conc) // 2] = np.nan
    s, _, _, _ = _noalloc(desc, g["pot_eq"], conc)
    assert s == -4 and "non-finite" in L.lib().emcg_last_error().decode()
    s, _, rel, _ = _noalloc(desc, g["pot_eq"], g["conc0"])
    L.check(s)
    assert rel <= RTOL
    sim.close()
