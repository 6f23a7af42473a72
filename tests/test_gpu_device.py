"""Device engine on the GPU against the reference's device runs and the oracle.

Replay: the FP64 engine consumes the reference's own random words (move and
injection phases, attributed per particle) from the reference's state before
each step and must land on the reference's state after it (1e-12 relative),
with the same netto contact counts.  Poisson: the multigrid / defect-correction
solver against the reference's SOR iteration run to 1e-12 V.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden
from test_oracle_device_golden import (DEVICE_CASES, _host_device, _oracle_device, _oracle_model,
                                       flavour, surfaces)

pytestmark = pytest.mark.gpu
RTOL = 1e-12
FIELDS_F = ("kx", "ky", "kz", "px", "py", "E", "tau", "gtau")
ENG = {"E": "energy", "gtau": "grain_tau"}


def _electron(engine, dev, grain=None, surface=()):
    """The harness's particle type: acoustic, Coulomb, zero-order f/g
    absorption/emission, in that registration order, 4 eV tables; grain: a
    grain mechanism (transmission probability, scatter rate); surface: the
    fixture's surface mechanisms (boundary, kind, parameter)."""
    from viennaemc_gb300 import physics as P
    mat = P.silicon_material()
    pt = P.Electron(1000, 4.0)
    P.add_x_valley(pt, 0.196)
    regs = list(range(dev.n_regions))
    pt.addScatterMechanism(regs, P.AcousticScatterMechanism(0, 9.0, 300.0, mat.rho, mat.velSound))
    pt.addScatterMechanism(regs, P.CoulombScatterMechanism(0, mat.epsR, 300.0,
                                                           dev.getDopingRegionDoping))
    for fs, sfx in ((P.FINAL_F, "F"), (P.FINAL_G, "G")):
        pt.addScatterMechanism(regs, P.ZeroOrderInterValleyAbsorptionScatterMechanism(
            sfx, 0, fs, 5.23e10, 0.06, 300.0, mat.rho))
        pt.addScatterMechanism(regs, P.ZeroOrderInterValleyEmissionScatterMechanism(
            sfx, 0, fs, 5.23e10, 0.06, 300.0, mat.rho))
    if grain is not None:
        pt.setGrainScatterMechanism(P.GrainScatterMechanism(*grain))
    for b, kind, par in surface:
        cls = (P.ConstantSurfaceScatterMechanism if kind == 1
               else P.MomentumDependentSurfaceScatterMechanism)
        pt.setSurfaceScatterMechanism(b, cls(par))
    pt.initScatterTables()
    return pt


def _sim(engine, g, case, precision="fp64", seed=1, grain=None, **kw):
    from viennaemc_gb300 import device as D
    scheme, pot_init, vwd = flavour(g)
    dev = _host_device(g, pot_init)
    pt = _electron(engine, dev, grain, surfaces(g))
    return D.DeviceSimulation(dev, pt, scheme=scheme, dt=float(g["params"][1]),
                              seed=seed, capacity=1 << 15, precision=precision,
                              potential_init=pot_init, round_counts=vwd,
                              tau_region_is_valley=vwd, **kw), dev, pt


def _engine_state(engine, g, s):
    kw = {ENG.get(f, f): g[f"s{s}_{f}"] for f in FIELDS_F}
    kw["pz"] = np.zeros(len(g[f"s{s}_E"]))
    kw.update({f: g[f"s{s}_{f}"] for f in ("valley", "sub", "region")})
    return engine.ParticleState.from_arrays(**kw)


def _assert_state(st, g, s, rtol=RTOL):
    assert st.n == len(g[f"s{s}_E"]), (s, st.n)
    for f in FIELDS_F:
        a, b = getattr(st, ENG.get(f, f)), g[f"s{s}_{f}"]
        err = np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)
        assert err <= rtol, (s, f, err)
    for f in ("valley", "sub", "region"):
        assert np.array_equal(getattr(st, f), g[f"s{s}_{f}"]), (s, f)


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_efield_matches_reference(engine, case):
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    sim, dev, pt = _sim(engine, g, case)
    for s in (1, 2):
        sim.set_grid(L.GRID_POTENTIAL, g[f"pot{s}"])
        sim.efield()
        ex, ey = sim.get_grid(L.GRID_EX), sim.get_grid(L.GRID_EY)
        scale = max(np.abs(g[f"ex{s}"]).max(), np.abs(g[f"ey{s}"]).max())
        assert np.max(np.abs(ex - g[f"ex{s}"])) <= RTOL * scale
        assert np.max(np.abs(ey - g[f"ey{s}"])) <= RTOL * scale
    sim.close()


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_replayed_step_matches_reference(engine, case):
    """move + contacts from the reference's state and random words."""
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    sim, dev, pt = _sim(engine, g, case)
    for s in range(1, int(g["params"][2]) + 1):
        sim.set_state(_engine_state(engine, g, s - 1))
        sim.set_grid(L.GRID_EX, g[f"ex{s}"])
        sim.set_grid(L.GRID_EY, g[f"ey{s}"])
        sim.set_replay(0, g[f"move_words{s}"], g[f"move_offsets{s}"])
        netto = sim.move(step=s)
        w = g[f"inject_words{s}"]
        per = 9  # 2 position + 7 particle draws per injected electron
        sim.set_replay(1, w, np.arange(0, len(w) + 1, per, dtype=np.int64))
        rem_inj = sim.contacts(step=s)
        assert np.array_equal(netto - rem_inj, g[f"netto{s}"]), s
        _assert_state(sim.get_state(), g, s)
    sim.close()


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_assignment_and_concentration_match_reference(engine, case):
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    sim, dev, pt = _sim(engine, g, case)
    for s in (0, 1, 3):
        sim.set_state(_engine_state(engine, g, s))
        sim.assign()
        nr, conc = sim.get_grid(L.GRID_NRPART), sim.get_grid(L.GRID_CONC)
        assert np.allclose(nr, g[f"nr{s}"], rtol=1e-12, atol=1e-12)
        assert np.allclose(conc, g[f"conc{s}"], rtol=1e-12, atol=0)
    sim.close()


@pytest.mark.parametrize("case", DEVICE_CASES)
@pytest.mark.parametrize("fp32", [True, False])
def test_poisson_matches_converged_sor(engine, oracle, case, fp32):
    """Equilibrium and non-equilibrium potentials: multigrid + double
    refinement to 1e-10 relative residual vs the reference's SOR to 1e-12 V."""
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    sim, dev, pt = _sim(engine, g, case, poisson_rtol=1e-10, poisson_fp32=fp32,
                      poisson_max_cycles=200)
    odev = _oracle_device(oracle, g)
    # equilibrium from the initial guess asinh(C/2)
    sim.set_grid(L.GRID_POTENTIAL, g["pot_init"])
    rel, cyc = sim.poisson(equilibrium=True, reset_bc=True)
    ref, sweeps = odev.sor(g["pot_init"], None, 1.8, 1e-12, True)
    assert sweeps > 0 and rel <= 1e-10
    assert np.max(np.abs(sim.potential - ref)) <= 1e-7, np.max(np.abs(sim.potential - ref))
    # non-equilibrium with the reference's concentration of step 1
    sim.set_grid(L.GRID_POTENTIAL, g["pot_eq"])
    sim.set_grid(L.GRID_CONC, g["conc0"])
    rel, cyc = sim.poisson(equilibrium=False, reset_bc=True)
    ref, sweeps = odev.sor(g["pot_eq"], g["conc0"], 1.8, 1e-12, True)
    assert sweeps > 0 and rel <= 1e-10
    assert np.max(np.abs(sim.potential - ref)) <= 1e-7, np.max(np.abs(sim.potential - ref))
    sim.close()


@pytest.mark.parametrize("case,grain", [(c, None) for c in DEVICE_CASES] +
                         [(DEVICE_CASES[0], (0.4, 5e14)), (DEVICE_CASES[1], (0.6, 5e14))])
def test_philox_step_matches_oracle(engine, oracle, case, grain):
    """Same potential, same Philox counters: E field, move, contacts and
    assignment of the FP64 engine equal the oracle's (1e-12); also with a
    grain mechanism (emcBasicParticleHandler.hpp:131-138), the grain timers
    set below one step so that most particles meet a grain."""
    from viennaemc_gb300 import _lib as L
    g = golden(case)
    seed, stream = 0xBEEF, 0
    sim, dev, pt = _sim(engine, g, case, seed=seed, grain=grain)
    odev = _oracle_device(oracle, g)
    m, regs = _oracle_model(oracle, g)
    if grain is not None:
        m.set_grain(*grain)
    scheme, _, vwd = flavour(g)
    dt = float(g["params"][1])
    cur = oracle.State.from_dict({f: g[f"s0_{f}"] for f in oracle.STATE_F + oracle.STATE_I})
    if grain is not None:
        cur.gtau[:] = np.linspace(0.05, 0.95, cur.n) * dt
    cur = cur.resize(1 << 15)
    cur.n = len(g["s0_E"])
    est = _engine_state(engine, g, 0)
    if grain is not None:
        est.grain_tau[:] = cur.gtau[:cur.n]
    sim.set_state(est)
    rng = oracle.RngState(oracle.RNG_PHILOX, seed, stream)
    expnr = odev.exp_nr(vwd)
    for s in range(1, 4):
        sim.set_grid(L.GRID_POTENTIAL, g[f"pot{s}"])
        sim.efield()
        Ex, Ey = odev.efield(g[f"pot{s}"], scheme)
        netto = sim.move(step=s)
        rem_inj = sim.contacts(step=s)
        rc, onet, _ = odev.move(m, scheme, cur, Ex, Ey, dt, rng, s)
        ori = odev.contacts(m, cur, 1 << 15, expnr, rng, s, tau_region_is_valley=vwd)
        assert np.array_equal(netto, onet) and np.array_equal(rem_inj, ori)
        st = sim.get_state()
        assert st.n == cur.n
        for f in FIELDS_F:
            a, b = getattr(st, ENG.get(f, f)), getattr(cur, f)[:cur.n]
            assert np.max(np.abs(a - b)) <= RTOL * max(np.abs(b).max(), 1e-300), (s, f)
        sim.assign()
        nr = odev.assign(scheme, cur.resize(cur.n))
        assert np.allclose(sim.get_grid(L.GRID_NRPART), nr, rtol=1e-12, atol=1e-12)
    sim.close()


@pytest.mark.parametrize("case", [DEVICE_CASES[0], "device_resistor_surface.npz"])
def test_full_device_steps_run_and_conserve_count(engine, case):
    """performEMCStep end to end (Poisson -> E -> move -> contacts -> assign),
    FP64 and FP32, also with surface mechanisms (the move kernels' surface
    instances): particle count changes only by the contact flux."""
    g = golden(case)
    for precision in ("fp64", "fp32"):
        sim, dev, pt = _sim(engine, g, case, precision=precision, seed=3)
        sim.calcEquilibriumCharacteristics()
        n0 = sim.num_particles()
        netto = sim.performEMCStep(20)
        n1 = sim.num_particles()
        assert n1 == n0 - int(netto.sum())
        assert np.all(np.isfinite(sim.potential))
        sim.close()


def test_device_step_equals_its_stages(engine):
    """performEMCStep (one compaction per step, the Poisson solve enqueued)
    gives what its stages called one by one give: Poisson, E field, move
    (compacting), contacts (compacting), assignment -- same potential, same
    particles bit for bit, same contact counts, FP64 and FP32."""
    g = golden(DEVICE_CASES[0])
    K = 6
    for precision in ("fp64", "fp32"):
        a, _, _ = _sim(engine, g, DEVICE_CASES[0], precision=precision, seed=3)
        b, _, _ = _sim(engine, g, DEVICE_CASES[0], precision=precision, seed=3)
        a.calcEquilibriumCharacteristics()
        b.calcEquilibriumCharacteristics()
        s0 = b.step_index
        net_a = a.performEMCStep(K)
        rows = []
        for s in range(K):
            b.poisson(equilibrium=False, reset_bc=(s == 0))
            b.efield()
            n = b.move(step=s0 + s)
            ri = b.contacts(step=s0 + s)
            b.assign()
            rows.append(n - ri)
        assert np.array_equal(net_a, np.array(rows)), precision
        assert np.array_equal(a.potential, b.potential), precision
        sa, sb = a.get_state(), b.get_state()
        for f in ("kx", "ky", "kz", "energy", "px", "py", "tau", "valley", "sub", "region"):
            assert np.array_equal(getattr(sa, f), getattr(sb, f)), (precision, f)
        a.close()
        b.close()


def _resistor_201x101(scale=1):
    from viennaemc_gb300 import device as D
    from viennaemc_gb300.physics import silicon_material
    lx, ly = 100e-9 * scale, 50e-9 * scale
    dev = D.Device(silicon_material(), (lx, ly), (0.5e-9, 0.5e-9))
    dev.setDeviceWidth(1e-4)
    dev.addConstantDopingRegion((0, 0), (lx, ly), 1e24)
    dev.addOhmicContact(D.XMAX, 0.0, (0,), (ly,))
    dev.addOhmicContact(D.XMIN, 0.5, (0,), (ly,))
    return dev


# resistor_401x201: a CTA's band of the finest level holds more nodes than the
# register-held sweeps take, so those sweeps run one phase per half sweep
@pytest.mark.parametrize("case", DEVICE_CASES + ["resistor_201x101", "resistor_401x201"])
def test_poisson_cluster_equals_multilaunch(engine, case):
    """The single-launch cluster solve and the one-launch-per-phase solve
    evaluate the same expressions on the same values: same cycles, same
    potential (1e-13 thermal voltages)."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    if case.startswith("resistor_"):
        from viennaemc_gb300 import physics as P
        dev = _resistor_201x101(2 if case == "resistor_401x201" else 1)
        pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                                coulomb=True, region_doping=dev.getDopingRegionDoping)
        sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=5, precision="fp32",
                                 poisson_rtol=1e-10, poisson_max_cycles=200)
        pot0 = np.arcsinh(0.5 * dev.doping / dev.material.Ni)
        rs = np.random.default_rng(1)
        conc = np.exp(pot0) * (1 + 0.05 * rs.standard_normal(pot0.size))
    else:
        g = golden(case)
        sim, dev, pt = _sim(engine, g, case, precision="fp32", poisson_rtol=1e-10,
                            poisson_max_cycles=200)
        pot0, conc = g["pot_init"], g["conc0"]
    assert sim.poisson_mode() >= 1
    if case.startswith("resistor_"):
        assert sim.poisson_mode() > 1  # distributed over several CTAs
    out = {}
    for mode in (1, 0):
        sim.poisson_mode(mode)
        sim.set_grid(L.GRID_POTENTIAL, pot0)
        r1 = sim.poisson(equilibrium=True, reset_bc=True)
        eq = sim.potential
        sim.set_grid(L.GRID_CONC, conc)
        r2 = sim.poisson(equilibrium=False, reset_bc=True)
        out[mode] = (r1, r2, eq, sim.potential)
    sim.close()
    a, b = out[1], out[0]
    assert a[0][1] == b[0][1] and a[1][1] == b[1][1], (a[0], b[0], a[1], b[1])
    assert max(a[0][0], a[1][0]) <= 1e-10
    assert np.max(np.abs(a[2] - b[2])) <= 1e-13 * max(1.0, np.abs(b[2]).max())
    assert np.max(np.abs(a[3] - b[3])) <= 1e-13 * max(1.0, np.abs(b[3]).max())


@pytest.mark.parametrize("case", ["resistor_201x101", "resistor_401x201"])
def test_poisson_cluster_size_does_not_change_the_solve(engine, case):
    """Clusters of 16, 14, 12, 10 or 8 CTAs (the sizes a batch of engines may
    be given so that all their solves fit at once) split the rows differently
    but evaluate the same expressions: the same Newton steps and potential
    (1e-13 thermal voltages) as the 16-CTA solve.  On 401 x 201, 12 CTAs fit
    in shared memory only with bands a row apart between levels (their
    restrictions and prolongations reach a neighbour's rows); 10 and 8 do
    not fit."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    dev = _resistor_201x101(2 if case == "resistor_401x201" else 1)
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                            coulomb=True, region_doping=dev.getDopingRegionDoping)
    sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=5, precision="fp32",
                             poisson_rtol=1e-10, poisson_max_cycles=200)
    pot0 = np.arcsinh(0.5 * dev.doping / dev.material.Ni)
    rs = np.random.default_rng(2)
    conc = np.exp(pot0) * (1 + 0.05 * rs.standard_normal(pot0.size))
    out = {}
    for cap in (16, 14, 12, 10, 8):
        cs = sim.set_poisson_cluster(cap)
        if cs == 0 or cs in out:  # the layout does not fit, or the size was run
            continue
        sim.set_grid(L.GRID_POTENTIAL, pot0)
        r1 = sim.poisson(equilibrium=True, reset_bc=True)
        eq = sim.potential
        sim.set_grid(L.GRID_CONC, conc)
        r2 = sim.poisson(equilibrium=False, reset_bc=True)
        out[cs] = (r1[1], r2[1], eq, sim.potential, r1[0], r2[0])
    assert sim.set_poisson_cluster(0) == 16
    for bad in (-1, 17):
        with pytest.raises(engine._lib.EmcgError):
            sim.set_poisson_cluster(bad)
    assert sim.poisson_mode() == 16
    sim.close()
    assert sorted(out) == ([12, 14, 16] if case == "resistor_401x201" else [8, 10, 12, 14, 16])
    a = out[16]
    for cs, b in out.items():
        assert b[:2] == a[:2], (cs, b[:2], a[:2])
        assert max(b[4], b[5]) <= 1e-10
        for k in (2, 3):
            assert np.max(np.abs(b[k] - a[k])) <= 1e-13 * max(1.0, np.abs(a[k]).max()), cs


def test_step_many_equals_separate_steps(engine):
    """Stepping two engines concurrently gives what stepping each alone gives."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    g = golden(DEVICE_CASES[1])
    runs = []
    for batch in (False, True):
        sims = []
        for seed in (5, 6):
            sim, dev, pt = _sim(engine, g, DEVICE_CASES[1], precision="fp32", seed=seed)
            sim.calcEquilibriumCharacteristics()
            sims.append(sim)
        if batch:
            nets = D.DeviceSimulation.performEMCStepMany(sims, 4)
        else:
            nets = [s.performEMCStep(4) for s in sims]
        runs.append([(n, s.potential, s.num_particles()) for n, s in zip(nets, sims)])
        for s in sims:
            s.close()
    for (na, pa, ca), (nb, pb, cb) in zip(*runs):
        assert np.array_equal(na, nb) and ca == cb
        assert np.allclose(pa, pb, rtol=1e-9, atol=1e-9)


def test_step_many_plans_clusters_for_the_batch(engine):
    """Eight engines on 201 x 101 grids (16-CTA Poisson clusters alone; the
    device holds seven of those at once) stepped as one batch, which plans
    clusters of a size the device holds eight of: every engine lands where it
    lands stepped alone (same contact counts, particles and potential), and
    each engine's own 16-CTA plan is back after the batch."""
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    dev = _resistor_201x101()
    dev.setDeviceWidth(2e-6)  # about 1e4 electrons
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                            coulomb=True, region_doping=dev.getDopingRegionDoping)
    runs = []
    for batch in (False, True):
        sims = []
        for seed in range(8):
            sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=20 + seed,
                                     precision="fp32", poisson_rtol=1e-8)
            sim.calcEquilibriumCharacteristics()
            assert sim.poisson_mode() == 16
            sims.append(sim)
        if batch:
            nets = D.DeviceSimulation.performEMCStepMany(sims, 3)
            assert all(s.poisson_mode() == 16 for s in sims)
        else:
            nets = [s.performEMCStep(3) for s in sims]
        runs.append([(n, s.potential, s.num_particles()) for n, s in zip(nets, sims)])
        for s in sims:
            s.close()
    for (na, pa, ca), (nb, pb, cb) in zip(*runs):
        assert np.array_equal(na, nb) and ca == cb
        assert np.max(np.abs(pa - pb)) <= 1e-13 * np.abs(pb).max()


def test_execute_writes_reference_output_files(engine, tmp_path):
    """execute() with an output prefix writes the reference's file set: grids
    with their extent, the particle dump, the current table over the
    non-transient steps (the same writers are byte-checked against the
    reference's files in test_results_output.py)."""
    g = golden(DEVICE_CASES[0])
    sim, dev, pt = _sim(engine, g, DEVICE_CASES[0], precision="fp32", seed=9)
    prefix = str(tmp_path / "out") + "/"
    netto = sim.execute(12, transient_steps=2, steps_for_avg=4, output_prefix=prefix)
    n = sim.num_particles()
    sim.close()
    names = sorted(os.listdir(tmp_path / "out"))
    assert names == sorted(["PotentialEq.txt", "ElectronsConcEq.txt", "EFieldXEq.txt",
                            "EFieldYEq.txt", "ElectronsEq.txt", "ElectronsCurrent.txt",
                            "ElectronsConcAvg.txt", "PotentialAvg.txt", "ElectronsFinal.txt"])
    for f in ("PotentialEq.txt", "ElectronsConcAvg.txt", "PotentialAvg.txt"):
        lines = open(tmp_path / "out" / f).read().splitlines()
        assert lines[0] == f"{dev.nx} {dev.ny}" and len(lines) == dev.ny + 1
        assert all(len(l.split()) == dev.nx for l in lines[1:])
    parts = open(tmp_path / "out" / "ElectronsFinal.txt").read().split("\n")
    assert len(parts) == n + 1 and all(len(p.split()) == 10 for p in parts[1:])
    cur = np.loadtxt(tmp_path / "out" / "ElectronsCurrent.txt")
    assert cur.shape == (10, 1 + 2 * len(dev.contacts))
    nt = netto[2:].astype(np.float64)
    factor = -1.60219e-19 / float(g["params"][1])
    expect = np.cumsum(nt, axis=0) / np.arange(1, 11)[:, None] * factor
    assert np.allclose(cur[:, 1:1 + len(dev.contacts)], nt)
    assert np.allclose(cur[:, 1 + len(dev.contacts):], expect, rtol=1e-5)


def test_poisson_update_rule_matches_between_paths(engine):
    """The reference SOR's rule (stop once an update moves no potential by more
    than 1e-4 V) stops both executions at the same Newton step with the same
    potential, earlier than the residual rule."""
    from viennaemc_gb300 import _lib as L
    g = golden(DEVICE_CASES[1])
    sim, dev, pt = _sim(engine, g, DEVICE_CASES[1], precision="fp32", poisson_rtol=1e-12,
                        poisson_max_cycles=200)
    out = {}
    for mode in (1, 0):
        sim.poisson_mode(mode)
        sim.set_poisson(update_tol=1e-4)
        sim.set_grid(L.GRID_POTENTIAL, g["pot_eq"])
        sim.set_grid(L.GRID_CONC, g["conc0"])
        rel, cyc = sim.poisson(equilibrium=False, reset_bc=True)
        out[mode] = (cyc, sim.potential)
        sim.set_poisson(update_tol=0.0)
        sim.set_grid(L.GRID_POTENTIAL, g["pot_eq"])
        rel2, cyc2 = sim.poisson(equilibrium=False, reset_bc=True)
        assert cyc2 > cyc and rel2 <= 1e-12
    sim.close()
    assert out[1][0] == out[0][0]
    assert np.max(np.abs(out[1][1] - out[0][1])) <= 1e-12 * np.abs(out[0][1]).max()


def test_initial_particles_beyond_capacity_are_rejected(engine):
    """A capacity below the device's initial particle count is an argument
    error with a message, not a silent truncation."""
    g = golden(DEVICE_CASES[0])
    sim, dev, pt = _sim(engine, g, DEVICE_CASES[0], precision="fp32")
    sim.close()
    from viennaemc_gb300 import device as D
    small = D.DeviceSimulation(dev, pt, scheme=D.NGP, dt=1e-15, seed=1, capacity=100,
                               precision="fp32")
    small.poisson(equilibrium=True, reset_bc=True)
    with pytest.raises(engine._lib.EmcgError) as ei:
        small.init_particles()
    assert ei.value.status == -1 and "capacity" in str(ei.value)
    small.close()


def test_step_reports_a_solve_that_missed_its_target(engine):
    """The device step checks its enqueued Poisson solve at the end of the
    step: a Newton-step limit too small for the target is reported there."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    dev = _resistor_201x101()
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                            coulomb=True, region_doping=dev.getDopingRegionDoping)
    sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=5, precision="fp32",
                             poisson_rtol=1e-8, poisson_max_cycles=60)
    sim.calcEquilibriumCharacteristics()
    sim.performEMCStep(2)
    sim.set_poisson(rtol=1e-30, max_cycles=1)
    with pytest.raises(L.EmcgError):
        sim.performEMCStep(1)
    sim.set_poisson(rtol=1e-8, max_cycles=60)
    sim.performEMCStep(2)  # the handle stays usable
    assert sim.num_particles() > 0
    sim.close()


def test_deposition_is_reproducible_bit_for_bit(engine):
    """The 201 x 101 resistor with about 5e5 electrons (CIC, FP32), 20 steps
    from the same seed, twice: the deposition sums fixed-point weights with
    integer atomics, so the assigned charge, the concentration and the
    potential are equal bit for bit, whatever order the atomics ran in; and
    the assigned charge equals a host sum of the same particles' CIC weights
    to within float rounding."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    out = []
    for _ in range(2):
        dev = _resistor_201x101()
        pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                                coulomb=True, region_doping=dev.getDopingRegionDoping)
        sim = D.DeviceSimulation(dev, pt, scheme=D.CIC, dt=1e-16, seed=77, precision="fp32",
                                 poisson_rtol=1e-8, poisson_max_cycles=60)
        sim.calcEquilibriumCharacteristics()
        sim.performEMCStep(20)
        out.append((sim.get_grid(L.GRID_NRPART), sim.concentration, sim.potential,
                    sim.get_state()))
        sim.close()
    (nr, conc, pot, st), (nr2, conc2, pot2, _) = out
    assert st.n > 400000
    assert np.array_equal(nr, nr2) and np.array_equal(conc, conc2) and np.array_equal(pot, pot2)
    # the reference's CIC weights (the lower node gets w = pos / h - floor,
    # emcCICScheme.hpp:30-66) summed on the host
    h = 0.5e-9
    px, py = st.px.astype(np.float32), st.py.astype(np.float32)
    fx, fy = px * np.float32(1.0 / h), py * np.float32(1.0 / h)  # as the float engine
    mx, my = np.floor(fx).astype(int), np.floor(fy).astype(int)
    wx, wy = (fx - mx).astype(np.float64), (fy - my).astype(np.float64)
    ref = np.zeros((101, 201))
    for dx, dy, w in ((0, 0, wx * wy), (1, 0, (1 - wx) * wy), (0, 1, wx * (1 - wy)),
                      (1, 1, (1 - wx) * (1 - wy))):
        x, y = mx + dx, my + dy
        ok = (x >= 0) & (x < 201) & (y >= 0) & (y < 101)
        np.add.at(ref, (y[ok], x[ok]), w[ok])
    # the float engine forms its weights in float
    assert np.allclose(nr.reshape(101, 201), ref, rtol=0, atol=2e-6), \
        np.abs(nr.reshape(101, 201) - ref).max()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_surface_mechanisms_reference_kat(engine, precision):
    """The reference's surface-scattering test (tests/testSurfaceScatterMechanisms/
    testSurfaceScatterMechanisms.cpp:16-118) through the engine's boundary
    routine, 1000 particles per case, on a 2-D device of the same 1 um extent
    (the z positions of the 3-D original drop out): a smooth surface
    (specularity 1) reflects, a rough one (specularity 0) and a
    momentum-dependent one at |2 h k_perp| = 6 scatter diffusely into the
    device, a boundary without mechanism reflects; |k| is kept."""
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    mat = P.silicon_material()
    dev = D.Device(mat, (1e-6, 1e-6), (1e-7, 1e-7))
    dev.addConstantDopingRegion((0, 0), (1e-6, 1e-6), 1e22)
    pt = P.silicon_electron("jacoboni", n_levels=1000, max_energy=4.0)
    pt.setSurfaceScatterMechanism(D.YMAX, P.ConstantSurfaceScatterMechanism(1.0))
    pt.setSurfaceScatterMechanism(D.XMIN, P.ConstantSurfaceScatterMechanism(0.0))
    pt.setSurfaceScatterMechanism(D.XMAX, P.MomentumDependentSurfaceScatterMechanism(3e-10))
    sim = D.DeviceSimulation(dev, pt, scheme=D.NGP, dt=1e-15, seed=1, capacity=1 << 12,
                             precision=precision)
    n, mx = 1000, 1e-6
    rtol = 1e-10 if precision == "fp64" else 1e-6

    def run(b, k0, p0):
        k, p = sim.surface_kat(b, np.tile(k0, (n, 1)), np.tile(p0, (n, 1)))
        assert np.allclose(np.linalg.norm(k, axis=1), np.linalg.norm(k0), rtol=rtol, atol=0)
        return k, p

    # YMAX, smooth: specular
    k, p = run(D.YMAX, [1, 1, 1], [1e-6, 1.1e-6])
    assert np.all(k[:, 1] < 0) and np.all(k[:, 0] == 1) and np.all(k[:, 2] == 1)
    assert np.allclose(p[:, 1], 2 * mx - 1.1e-6, rtol=rtol)
    assert np.allclose(p[:, 0], 1e-6, rtol=rtol)
    # XMIN, rough: diffuse into the device
    k, p = run(D.XMIN, [-1, 1, 1], [-0.1e-6, 1e-6])
    assert np.all(k[:, 0] > 0) and np.all(k[:, 1] != 1) and np.all(k[:, 2] != 1)
    assert np.allclose(p[:, 0], 0.1e-6, rtol=rtol) and np.allclose(p[:, 1], 1e-6, rtol=rtol)
    # XMAX, momentum-dependent: diffuse (1 - exp(-36))
    k, p = run(D.XMAX, [1e10, 1e10, 1e10], [1.1e-6, 5e-7])
    assert np.all(k[:, 0] < 0) and np.all(k[:, 1] != 1e10) and np.all(k[:, 2] != 1e10)
    assert np.allclose(p[:, 0], 2 * mx - 1.1e-6, rtol=rtol)
    assert np.allclose(p[:, 1], 5e-7, rtol=rtol)
    # XMIN, far outside in both directions: diffuse, then every coordinate back
    # inside with k pointing inwards
    k, p = run(D.XMIN, [-1, -1, -1], [-0.1, -0.1])
    assert np.all(k[:, 0] > 0) and np.all(k[:, 1] > 0)
    assert np.allclose(p, 0.1, rtol=rtol)
    # YMIN, no mechanism: plain reflection
    k, p = run(D.YMIN, [1, -1, 1], [5e-7, -0.1])
    assert np.all(k[:, 1] > 0) and np.all(k[:, 0] == 1) and np.all(k[:, 2] == 1)
    assert np.allclose(p[:, 1], 0.1, rtol=rtol) and np.allclose(p[:, 0], 5e-7, rtol=rtol)
    # the diffuse directions: a cosine law about the inward normal (mean of
    # cos(theta) = 2/3 for the constant mechanism)
    k, _ = run(D.XMIN, [-1, 1, 1], [-0.1e-6, 1e-6])
    ct = k[:, 0] / np.linalg.norm(k, axis=1)
    assert abs(ct.mean() - 2 / 3) < 0.03, ct.mean()
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_grid_layout_through_the_field(engine, precision):
    """The grid index layout of the reference's tests/testGrid (x fastest,
    neighbours at +-1 and +-nx) seen through the E field
    (include/PMSchemes/emcEFieldCalculation.hpp:13-81): with the potential
    phi = y nx + x (thermal voltages), the interior field is -Vt / hx and
    -nx Vt / hy; at the ohmic contacts (XMIN, XMAX) the normal field repeats
    the neighbour's, at the artificial boundaries (YMIN, YMAX) it is 0."""
    from viennaemc_gb300 import _lib as L
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    dev = D.Device(P.silicon_material(), (20e-9, 10e-9), (1e-9, 2e-9))
    dev.addConstantDopingRegion((0, 0), (20e-9, 10e-9), 1e24)
    dev.addOhmicContact(D.XMIN, 0.0, (0,), (10e-9,))
    dev.addOhmicContact(D.XMAX, 0.1, (0,), (10e-9,))
    pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0)
    sim = D.DeviceSimulation(dev, pt, scheme=D.NGP, dt=1e-15, seed=1, capacity=1 << 12,
                             precision=precision)
    nx, ny = dev.nx, dev.ny
    assert (nx, ny) == (21, 6)
    sim.set_grid(L.GRID_POTENTIAL, np.arange(nx * ny, dtype=float))
    sim.efield()
    ex = sim.get_grid(L.GRID_EX).reshape(ny, nx)
    ey = sim.get_grid(L.GRID_EY).reshape(ny, nx)
    Vt = dev.getThermalVoltage()
    rtol = 1e-12 if precision == "fp64" else 1e-6
    assert np.allclose(ex[:, 1:-1], -Vt / 1e-9, rtol=rtol, atol=0)
    assert np.allclose(ey[1:-1, :], -nx * Vt / 2e-9, rtol=rtol, atol=0)
    assert np.allclose(ex[:, 0], ex[:, 1], rtol=rtol) and np.allclose(ex[:, -1], ex[:, -2], rtol=rtol)
    assert np.all(ey[0, 1:-1] == 0) and np.all(ey[-1, 1:-1] == 0)
    sim.close()
