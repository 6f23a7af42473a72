"""Rate-table rebuild (emcScatterHandler::reinitScatterTables,
include/emcScatterHandler.hpp:100-108) on the GPU.

Pinned to the reference's own rebuild with rates that change: the fixture
holds an acoustic + hot-phonon Froehlich absorption/emission table set before
and after the reference advanced its phonon bath and called
reinitScatterTables (tests/golden/make_golden.py, part "reinit").

* CPU: the oracle's renormalisation against the fixture, bit for bit; the
  host model's refill layout;
* GPU: the engine's rebuild from host and from device rates against the
  fixture, bit for bit (FP64) and to float rounding of the same doubles
  (FP32); a run whose tables are swapped mid-way equals a run built on the
  new tables, and the FP64 engine matches the oracle across the swap; bad
  rates are refused (host) or reported at the next call (device) and leave
  the tables as they were.
"""
import numpy as np
import pytest

from conftest import golden

G = "reinit_hot_phonon.npz"


def _oracle_holder(oracle, n_levels, max_energy):
    """An oracle model with one (valley 0, region 0) set of three tables; the
    mechanisms only fix the table count, the rates are replaced."""
    m = oracle.Model(n_levels=n_levels, max_energy=max_energy)
    m.add_valley([0.916, 0.19, 0.19], oracle.ME, 3, 0.5, 0.0, oracle.SI_FRAMES)
    m.add_mech(oracle.ACOUSTIC, 0, [0], 9.0)
    m.add_mech(oracle.ZERO_IV_ABS, 0, [0], 5.23e10, 0.06, 0, oracle.G_SUB)
    m.add_mech(oracle.ZERO_IV_EMI, 0, [0], 5.23e10, 0.06, 0, oracle.G_SUB)
    m.build_tables()
    return m


def test_oracle_rebuild_matches_reference(oracle):
    """renormalizeTables on the reference's refilled rates, before and after
    the phonon bath moved: the oracle lands on the reference's tables and tau
    bit for bit."""
    g = golden(G)
    nL, maxE = int(g["params"][0]), float(g["params"][1])
    m = _oracle_holder(oracle, nL, maxE)
    assert not np.array_equal(g["init_norm"], g["re_norm"])
    for tag in ("init", "re"):
        m.set_raw_tables(0, 0, g[f"{tag}_raw"])
        for t in range(g[f"{tag}_raw"].shape[0]):
            assert np.array_equal(m.norm_table(0, 0, t), g[f"{tag}_norm"][t]), (tag, t)
        assert m.tau(0, 0) == g[f"{tag}_tau"][0], tag


def test_numpy_restatement_matches_reference():
    """The host mirror's renormalisation (cumulative sum in table order, divided
    by the maximum of the last row) gives the reference's bits."""
    g = golden(G)
    for tag in ("init", "re"):
        cum = np.cumsum(g[f"{tag}_raw"], axis=0)
        mx = cum[-1].max()
        assert np.array_equal(cum / mx, g[f"{tag}_norm"])
        assert 1.0 / mx == g[f"{tag}_tau"][0]


def test_host_refill_layout():
    """fill_rates concatenates the table sets in key order, table-major; the
    host reinit reproduces the tables of the first initialisation."""
    from viennaemc_gb300 import physics as P
    pt = P.silicon_electron("jacoboni", regions=(0, 1))
    h = pt.scatterHandler
    assert len(h.table_mechs) == 2
    raw = pt.raw_rates()
    keys = sorted(h.table_mechs)
    want = np.concatenate([h.raw[k].reshape(-1) for k in keys])
    assert raw.size == h.fill_size() and np.array_equal(raw, want)
    norm0 = {k: h.norm[k].copy() for k in keys}
    tau0 = dict(h.tau)
    h.reinitScatterTables()
    for k in keys:
        assert np.array_equal(h.norm[k], norm0[k]) and h.tau[k] == tau0[k]


# ---- GPU ---------------------------------------------------------------------

def _three_table_type(engine, n_levels, max_energy):
    """Engine particle type with one (0, 0) set of three tables."""
    from viennaemc_gb300 import physics as P
    mat = P.silicon_material()
    pt = P.Electron(n_levels, max_energy)
    P.add_x_valley(pt, 0.19)
    pt.addScatterMechanism([0], P.AcousticScatterMechanism(0, 9.0, 300.0, mat.rho,
                                                           mat.velSound))
    pt.addScatterMechanism([0], P.ZeroOrderInterValleyAbsorptionScatterMechanism(
        "G", 0, P.FINAL_G, 5.23e10, 0.06, 300.0, mat.rho))
    pt.addScatterMechanism([0], P.ZeroOrderInterValleyEmissionScatterMechanism(
        "G", 0, P.FINAL_G, 5.23e10, 0.06, 300.0, mat.rho))
    pt.initScatterTables()
    return pt


def _bulk(engine, pt, precision, n=4000, seed=5, init=True):
    spec = engine.EnsembleSpec(0, n, 1e6, (1, 0, 0), (1e-6,) * 3, 1e-15, seed, 0, 300.0)
    b = engine.BulkBatch([pt], [spec], precision)
    if init:
        b.init_particles(0)
    return b


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_rebuild_matches_reference(engine, precision):
    """Host rates in, the engine's tables and tau out: the reference's bits
    (FP64), or those doubles rounded to float (FP32)."""
    g = golden(G)
    nL, maxE = int(g["params"][0]), float(g["params"][1])
    b = _bulk(engine, _three_table_type(engine, nL, maxE), precision)
    cast = (lambda a: a) if precision == "fp64" else \
        (lambda a: np.asarray(a, np.float32).astype(np.float64))
    for tag in ("re", "init", "re"):
        b.reinit_scatter_tables(0, g[f"{tag}_raw"])
        tables, tau = b.get_rates(0)
        assert np.array_equal(tables, cast(g[f"{tag}_norm"].reshape(-1))), tag
        assert tau[0] == cast(g[f"{tag}_tau"])[0], tag
    b.step(5)  # the engine runs on the rebuilt tables
    b.close()


@pytest.mark.gpu
def test_gpu_rebuild_from_device_rates(engine):
    """Rates already on the GPU (a CUDA tensor) give the same tables."""
    import torch
    g = golden(G)
    nL, maxE = int(g["params"][0]), float(g["params"][1])
    b = _bulk(engine, _three_table_type(engine, nL, maxE), "fp64")
    raw = torch.tensor(g["re_raw"].reshape(-1), dtype=torch.float64, device="cuda")
    b.reinit_scatter_tables(0, raw)
    tables, tau = b.get_rates(0)
    assert np.array_equal(tables, g["re_norm"].reshape(-1))
    assert tau[0] == g["re_tau"][0]
    b.close()


@pytest.mark.gpu
def test_gpu_bad_rates_leave_tables(engine):
    """A non-finite host rate is refused before any launch; device rates whose
    maximum is zero are reported by the next call and change nothing."""
    import torch
    g = golden(G)
    nL, maxE = int(g["params"][0]), float(g["params"][1])
    b = _bulk(engine, _three_table_type(engine, nL, maxE), "fp64")
    before, tau0 = b.get_rates(0)
    bad = g["re_raw"].copy()
    bad[1, 17] = np.nan
    with pytest.raises(engine._lib.EmcgError) as ei:
        b.reinit_scatter_tables(0, bad)
    assert ei.value.status == -1
    with pytest.raises(ValueError):
        b.reinit_scatter_tables(0, g["re_raw"][:2])  # wrong size
    zeros = torch.zeros(bad.size, dtype=torch.float64, device="cuda")
    b.reinit_scatter_tables(0, zeros)
    with pytest.raises(engine._lib.EmcgError) as ei:
        b.get_rates(0)
    assert ei.value.status == -1
    after, tau1 = b.get_rates(0)
    assert np.array_equal(after, before) and tau1[0] == tau0[0]
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,graph,mode", [("fp64", False, 0), ("fp32", False, 2),
                                                  ("fp32", True, 2), ("fp32", True, 0)])
def test_swap_mid_run_equals_run_on_new_tables(engine, precision, graph, mode):
    """Tables swapped between steps: from then on the run is the same as one
    whose model was built on the new tables (same Philox streams), bit for
    bit, with and without graph replay."""
    from viennaemc_gb300 import physics as P
    pa = P.silicon_electron("jacoboni", temperature=300.0)
    pb = P.silicon_electron("jacoboni", temperature=200.0)
    runs, st0 = [], None
    for swap in (True, False):
        b = _bulk(engine, pa if swap else pb, precision, n=6000, seed=9, init=False)
        b.set_launch(256, 10, queued=mode)
        b.set_graph(graph)
        if st0 is None:  # both runs start from the same particles
            b.init_particles(0)
            st0 = b.get_state(0)
        else:
            b.set_state(0, st0)
        if swap:
            b.step(5, step0=100)  # a graph exists before the swap
            b.set_state(0, st0)
            b.reinit_scatter_tables(0, pb.raw_rates())
        o = b.step(30, step0=0)
        runs.append((o, b.get_state(0)))
        b.close()
    (oa, sa), (ob, sb) = runs
    for f in ("kx", "ky", "kz", "energy", "tau", "px"):
        assert np.array_equal(getattr(sa, f), getattr(sb, f)), f
    assert np.array_equal(sa.valley, sb.valley) and np.array_equal(sa.sub, sb.sub)
    assert np.array_equal(oa[..., 2], ob[..., 2])


@pytest.mark.gpu
def test_fp64_swap_matches_oracle(engine, oracle):
    """FP64 engine and oracle, same Philox stream, tables of 300 K for 40 steps
    then of 200 K for 40 steps: states agree to 1e-12 (last-ulp branch flips
    counted)."""
    from viennaemc_gb300 import physics as P
    m = oracle.silicon_model("jacoboni", temperature=300.0)
    m200 = oracle.silicon_model("jacoboni", temperature=200.0)
    nT = m.n_tables(0, 0)
    raw200 = np.stack([m200.raw_table(0, 0, t) for t in range(nT)])
    pt = P.silicon_electron("jacoboni", temperature=300.0)
    pt200 = P.silicon_electron("jacoboni", temperature=200.0)
    assert np.array_equal(pt200.raw_rates(), raw200.reshape(-1))
    rng = oracle.RngState(oracle.RNG_MT, 31)
    st = m.bulk_init([2e-6] * 3, [2e-7] * 3, 4e20, rng)
    seed, stream, field = 0xABCDEF, 2, 1e6
    spec = engine.EnsembleSpec(0, st.n, field, (-1, 0, 0), (2e-6,) * 3, 1e-15, seed, stream)
    b = engine.BulkBatch([pt], [spec], "fp64")
    kw = {"energy": st.E, "grain_tau": st.gtau}
    kw.update({f: getattr(st, f) for f in ("kx", "ky", "kz", "px", "py", "pz", "tau",
                                            "valley", "sub", "region")})
    b.set_state(0, engine.ParticleState.from_arrays(**kw))
    b.step(40, step0=0)
    b.reinit_scatter_tables(0, raw200)
    b.step(40, step0=40)
    got = b.get_state(0)
    b.close()
    ref = st.copy()
    force = [1.60219e-19 * field, 0, 0]
    m.bulk_run_philox(ref, 1e-15, force, [2e-6] * 3, [-1.0, 0, 0], seed, stream, 0, 40,
                      n_threads=1, want_obs=False)
    m.set_raw_tables(0, 0, raw200)
    m.bulk_run_philox(ref, 1e-15, force, [2e-6] * 3, [-1.0, 0, 0], seed, stream, 40, 40,
                      n_threads=1, want_obs=False)
    bad = np.zeros(st.n, bool)
    for fe, fo in (("kx", "kx"), ("ky", "ky"), ("kz", "kz"), ("energy", "E"), ("tau", "tau"),
                   ("px", "px")):
        a, r = getattr(got, fe), getattr(ref, fo)
        bad |= np.abs(a - r) > 1e-12 * np.max(np.abs(r))
    bad |= (got.valley != ref.valley) | (got.sub != ref.sub)
    assert bad.sum() <= max(1, st.n // 1000), bad.sum()


@pytest.mark.gpu
def test_device_engine_rebuild_equals_engine_on_new_tables(engine):
    """Device engine (41 x 21 resistor, CIC, FP64): tables rebuilt on the GPU
    right after creation give the same equilibrium, steps and contact counts
    as an engine built on those tables (the acoustic rates scaled by 0.7)."""
    from viennaemc_gb300 import device as D
    from viennaemc_gb300 import physics as P
    from viennaemc_gb300.physics import silicon_material

    def resistor():
        dev = D.Device(silicon_material(), (20e-9, 10e-9), (0.5e-9, 0.5e-9))
        dev.setDeviceWidth(1e-5)
        dev.addConstantDopingRegion((0, 0), (20e-9, 10e-9), 1e24)
        dev.addOhmicContact(D.XMAX, 0.0, (0,), (10e-9,))
        dev.addOhmicContact(D.XMIN, 0.2, (0,), (10e-9,))
        return dev

    def electron(dev, acoustic_scale):
        pt = P.silicon_electron("refbulk", n_levels=1000, max_energy=4.0, regions=[0],
                                coulomb=True, region_doping=dev.getDopingRegionDoping)
        h = pt.scatterHandler
        for key in sorted(h.table_mechs):
            raw = h.raw[key].copy()
            raw[0] *= acoustic_scale  # table 0 is the acoustic mechanism
            cum = np.cumsum(raw, axis=0)
            mx = cum[-1].max()
            h.raw[key], h.norm[key], h.tau[key] = raw, cum / mx, 1.0 / mx
        return pt

    runs = []
    for rebuild in (True, False):
        dev = resistor()
        pt_new = electron(dev, 0.7)
        sim = D.DeviceSimulation(dev, electron(dev, 1.0) if rebuild else pt_new, scheme=D.CIC,
                                 dt=1e-16, seed=11, precision="fp64")
        if rebuild:
            h = pt_new.scatterHandler  # its raw rates were scaled by hand, not refilled
            sim.reinitScatterTables(np.concatenate([h.raw[k].reshape(-1)
                                                    for k in sorted(h.table_mechs)]))
            tables, tau = sim.get_rates()
            h = pt_new.scatterHandler
            keys = sorted(h.table_mechs)
            assert np.array_equal(tables, np.concatenate([h.norm[k].reshape(-1) for k in keys]))
            assert np.array_equal(tau, [h.tau[k] for k in keys])
        sim.calcEquilibriumCharacteristics()
        netto = sim.performEMCStep(10)
        runs.append((netto, sim.get_state(), sim.potential))
        sim.close()
    (na, sa, pa), (nb, sb, pb) = runs
    # CIC deposits fractional charges with double atomics, whose order varies:
    # potentials and states agree to rounding, not bit for bit
    # (a particle whose path branched on a last-ulp difference is counted)
    assert np.array_equal(na, nb) and len(sa.kx) == len(sb.kx)
    bad = sa.valley != sb.valley
    for f in ("kx", "ky", "energy", "px"):
        a, b = getattr(sa, f), getattr(sb, f)
        bad |= np.abs(a - b) > 1e-9 * np.abs(b).max()
    assert bad.sum() <= max(1, len(sa.kx) // 200), bad.sum()
    assert np.allclose(pa, pb, rtol=1e-6, atol=1e-6)
