"""Device-path oracle and host device builder against the reference's own
device runs (tests/golden/device_*.npz, written by make_golden.py from the
reference's emcSimulation): every stage bit-exact."""
import numpy as np
import pytest

from conftest import golden

DEVICE_CASES = ["device_resistor_ngp.npz", "device_mosfet_cic.npz", "device_resistor_nec.npz",
                "device_mosfet_necvwd.npz", "device_resistor_surface.npz"]


def flavour(g):
    """(PM scheme, potential-based initial counts, electronVWD) of a fixture:
    resistor NGP, MOSFET CIC, resistor with the NEC scheme, and the mosfet2D
    example's NEC-VWD scheme with its electronVWD particle type (rounded counts,
    tau drawn with the valley as the region); the NGP resistor with surface
    mechanisms on its artificial boundaries.  Scheme numbers are shared by the
    oracle and the engine."""
    kind = str(g["kind"])
    scheme = {"resistor": 0, "mosfet": 1, "resistor_nec": 2, "mosfet_vwd": 3,
              "resistor_surface": 0}[kind]
    return scheme, kind.startswith("mosfet"), kind == "mosfet_vwd"


def _oracle_device(oracle, g):
    geom = g["geom"]
    nx, ny = int(round(geom[0] / geom[2])) + 1, int(round(geom[1] / geom[3])) + 1
    dev = oracle.Device(nx, ny, geom[2], geom[3], geom[4], g["doping"], g["region"],
                        [g[f"bnd{b}"] for b in range(4)], g["ctype"], g["cvolt"],
                        g["cpar"].reshape(-1, 3))
    dev.set_max(geom[0], geom[1])
    return dev


def _oracle_model(oracle, g):
    nreg = int(g["region"].max()) + 1
    m = oracle.Model(n_levels=1000, max_energy=4.0)
    m.add_valley([0.916, 0.196, 0.196], oracle.ME, 3, 0.5, 0.0, oracle.SI_FRAMES)
    regs = list(range(nreg))
    for r in regs:
        m.set_region_doping(r, g["doping"][g["region"] == r][0])
    m.add_mech(oracle.ACOUSTIC, 0, regs, 9.0)
    m.add_mech(oracle.COULOMB, 0, regs, 11.8)
    for fs in (oracle.F_SUB, oracle.G_SUB):
        m.add_mech(oracle.ZERO_IV_ABS, 0, regs, 5.23e10, 0.06, 0, fs)
        m.add_mech(oracle.ZERO_IV_EMI, 0, regs, 5.23e10, 0.06, 0, fs)
    for b, kind, par in surfaces(g):
        m.set_surface(b, kind, par)
    m.build_tables()
    return m, regs


def surfaces(g):
    """(boundary, kind, parameter) of the fixture's surface mechanisms; the
    kinds are shared by the oracle and the engine (0 specular, 1 constant
    specularity, 2 momentum-dependent roughness)."""
    return [(int(b), int(k), float(p)) for b, k, p in g["surface"]] if "surface" in g else []


def _state(oracle, g, s):
    return oracle.State.from_dict({f: g[f"s{s}_{f}"] for f in oracle.STATE_F + oracle.STATE_I})


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_device_pipeline_matches_reference(oracle, case):
    g = golden(case)
    dev = _oracle_device(oracle, g)
    m, regs = _oracle_model(oracle, g)
    for r in regs:
        assert np.array_equal(m.raw_table(0, r, 1), g["raw_coulomb"][r])
    for t in range(6):
        assert np.array_equal(m.raw_table(0, 0, t), g["raw_r0"][t])
    scheme, pot_init, vwd = flavour(g)
    seed, dt, steps, acc, width = g["params"]
    pot, _ = dev.sor(g["pot_init"], None, 1.8, acc, True)
    assert np.array_equal(pot, g["pot_eq"])
    Ex, Ey = dev.efield(pot, scheme)
    assert np.array_equal(Ex, g["ex_eq"]) and np.array_equal(Ey, g["ey_eq"])
    rng = oracle.RngState(oracle.RNG_MT, 0)
    rng.load_mt(g["mt_pre"])
    st = dev.init_particles(m, rng, pot if pot_init else None, round_counts=vwd,
                            tau_region_is_valley=vwd)
    s0 = _state(oracle, g, 0)
    for f in oracle.STATE_F + oracle.STATE_I:
        assert np.array_equal(getattr(st, f), getattr(s0, f)), f
    assert np.array_equal(dev.exp_nr(vwd), g["expnr"])
    nr = dev.assign(scheme, st)
    assert np.array_equal(nr, g["nr0"])
    conc = dev.concentration(nr)
    assert np.array_equal(conc, g["conc0"])
    cur = st.resize(1 << 16)
    cur.n = st.n
    for s in range(1, int(steps) + 1):
        pot, _ = dev.sor(pot, conc, 1.8, acc, s == 1)
        assert np.array_equal(pot, g[f"pot{s}"])
        Ex, Ey = dev.efield(pot, scheme)
        assert np.array_equal(Ex, g[f"ex{s}"]) and np.array_equal(Ey, g[f"ey{s}"])
        rc, netto, _ = dev.move(m, scheme, cur, Ex, Ey, dt, rng, s)
        assert rc == 0
        rem_inj = dev.contacts(m, cur, 1 << 16, dev.exp_nr(vwd), rng, s,
                               tau_region_is_valley=vwd)
        assert np.array_equal(netto - rem_inj, g[f"netto{s}"])
        ref = _state(oracle, g, s)
        assert cur.n == ref.n
        for f in oracle.STATE_F + oracle.STATE_I:
            assert np.array_equal(getattr(cur, f)[:cur.n], getattr(ref, f)), (s, f)
        nr = dev.assign(scheme, cur.resize(cur.n))
        conc = dev.concentration(nr)
        assert np.array_equal(nr, g[f"nr{s}"]) and np.array_equal(conc, g[f"conc{s}"])


def _host_device(g, mos):
    from viennaemc_gb300 import device as D
    from viennaemc_gb300.physics import silicon_material
    geom = g["geom"]
    dev = D.Device(silicon_material(), (geom[0], geom[1]), (geom[2], geom[3]))
    dev.setDeviceWidth(geom[4])
    if mos:
        dev.addConstantDopingRegion((0, 8e-9), (30e-9, 20e-9), -1e24)
        dev.addConstantDopingRegion((0, 0), (10e-9, 8e-9), 1e26)
        dev.addConstantDopingRegion((10e-9, 0), (20e-9, 8e-9), -1e24)
        dev.addConstantDopingRegion((20e-9, 0), (30e-9, 8e-9), 1e26)
        dev.addOhmicContact(D.YMAX, 0, (0,), (30e-9,))
        dev.addOhmicContact(D.YMIN, 0, (0,), (10e-9,))
        dev.addGateContact(D.YMIN, 1.0, (10e-9,), (20e-9,), 3.9, 1.2e-9, 1.15 / 2.0)
        dev.addOhmicContact(D.YMIN, 0.5, (20e-9,), (30e-9,))
    else:
        dev.addConstantDopingRegion((0, 0), (geom[0], geom[1]), 1e25)
        dev.addOhmicContact(D.XMAX, 0, (0,), (geom[1],))
        dev.addOhmicContact(D.XMIN, 0.1, (0,), (geom[1],))
    return dev


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_host_device_builder_matches_reference(case):
    g = golden(case)
    dev = _host_device(g, flavour(g)[1])
    assert np.array_equal(dev.doping, g["doping"])
    assert np.array_equal(dev.region, g["region"])
    for b in range(4):
        assert np.array_equal(dev.bnd[b], g[f"bnd{b}"]), b
    assert [c[0] for c in dev.contacts] == list(g["ctype"])
    assert np.array_equal([c[1] for c in dev.contacts], g["cvolt"])
    assert np.array_equal(np.array([p for c in dev.contacts for p in c[2]]), g["cpar"])
    assert dev.getCellVolume() == g["geom"][5]
    assert dev.getThermalVoltage() == g["geom"][7]


@pytest.mark.parametrize("case", DEVICE_CASES)
def test_host_coulomb_tables_match_reference(case):
    from viennaemc_gb300 import physics
    g = golden(case)
    dev = _host_device(g, flavour(g)[1])
    regs = list(range(dev.n_regions))
    pt = physics.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=regs,
                                  coulomb=True, region_doping=dev.getDopingRegionDoping,
                                  first_order=False)
    # the reference harness registers Coulomb second; compare by name
    h = pt.scatterHandler
    for r in regs:
        names = [h.mechanisms[i].getName() for i in h.table_mechs[(0, r)]]
        ci = names.index("Coulomb")
        assert np.array_equal(h.raw[(0, r)][ci], g["raw_coulomb"][r])
