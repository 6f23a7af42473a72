"""Bulk steps with particle-particle Coulomb forces: FMMBulkParticleHandler
(examples/bulkSimulationFMM) on the GPU.

Each step sums the Coulomb force of an ensemble's electrons and fixed donors
on its electrons (the direct sums that replace executeFMM) and moves the
electrons one step with force = charge x field - (ke / eps_r) x sum.

* FP64 engine against the oracle's loop (oracle Coulomb sums, oracle per-
  particle-force steps) on the same Philox stream: states agree to 1e-10,
  bar a few last-ulp branch flips;
* the sums the engine used equal the oracle's sums over the same positions;
* FP32 runs, argument checks, and switching the interaction off.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q = 1.60219e-19
EPS_R = 11.8


def _setup(engine, oracle, n_el=1200, box=1e-7, seed=17, grain=None):
    m = oracle.silicon_model("jacoboni", grain=grain)
    rng = oracle.RngState(oracle.RNG_MT, seed)
    # 1.2e24 m^-3 electrons on a (box / 8) grid
    st = m.bulk_init([box] * 3, [box / 8] * 3, n_el / box ** 3, rng)
    rs = np.random.default_rng(seed)
    nd = st.n
    fixed = rs.random((3, nd)) * box
    fq = np.full(nd, Q)  # ionised donors
    return m, st, fixed, fq


def _engine_state(engine, st):
    kw = {"energy": st.E, "grain_tau": st.gtau}
    kw.update({f: getattr(st, f) for f in ("kx", "ky", "kz", "px", "py", "pz", "tau",
                                            "valley", "sub", "region")})
    return engine.ParticleState.from_arrays(**kw)


def _batch(engine, n, box, precision, seed=321, stream=2, field=1e6, grain=None):
    pt = engine.physics.silicon_electron("jacoboni", grain=grain)
    spec = engine.EnsembleSpec(0, n, field, (1, 0, 0), (box,) * 3, 1e-15, seed, stream)
    return engine.BulkBatch([pt], [spec], precision)


@pytest.mark.parametrize("grain", [None, (0.5, 3e14)])
def test_fp64_coulomb_steps_match_oracle(engine, oracle, grain):
    """Also with a grain mechanism (grain events in the per-particle-force
    steps of the Coulomb kernel)."""
    box = 1e-7
    m, st, fixed, fq = _setup(engine, oracle, grain=grain)
    assert st.n > 800
    b = _batch(engine, st.n, box, "fp64", grain=grain)
    b.set_state(0, _engine_state(engine, st))
    b.set_fixed_charges(0, fixed, fq)
    b.set_coulomb(EPS_R, 1e9, 0)
    obs = b.step(12, step0=0)
    got = b.get_state(0)
    b.close()
    ref = st.copy()
    oobs = m.bulk_run_coulomb(ref, 1e-15, -Q, [1e6, 0, 0], [box] * 3, [1.0, 0, 0], fixed, fq,
                              EPS_R, 1e9, 0, 321, 2, 0, 12, n_threads=1)
    bad = (got.valley != ref.valley) | (got.sub != ref.sub)
    for fe, fo in (("kx", "kx"), ("ky", "ky"), ("kz", "kz"), ("energy", "E"), ("px", "px"),
                   ("py", "py"), ("tau", "tau")):
        a, r = getattr(got, fe), getattr(ref, fo)
        bad |= np.abs(a - r) > 1e-10 * np.max(np.abs(r))
    assert bad.sum() <= max(2, st.n // 200), bad.sum()
    assert np.allclose(obs[0, :, 0, 2], oobs[:, 0, 2])
    assert np.allclose(obs[0, :, 0, 0], oobs[:, 0, 0], rtol=1e-6)


def test_coulomb_sums_equal_oracle_over_the_same_positions(engine, oracle):
    box = 1e-7
    m, st, fixed, fq = _setup(engine, oracle, seed=5)
    for precision, tol in (("fp64", 1e-12), ("fp32", 1e-4)):
        b = _batch(engine, st.n, box, precision)
        b.set_state(0, _engine_state(engine, st))
        b.set_fixed_charges(0, fixed, fq)
        b.set_coulomb(EPS_R)
        pos0 = b.get_state(0)  # the positions the first step starts from
        b.step(1)
        f, p = b.get_coulomb(0)
        b.close()
        src = np.concatenate([np.stack([pos0.px, pos0.py, pos0.pz]), fixed], axis=1)
        q = np.concatenate([np.full(st.n, -Q), fq])
        fo, po_ = oracle.p2p_coulomb(src, q, 1e9)
        rel = np.max(np.abs(f - fo[:, :st.n])) / np.max(np.abs(fo[:, :st.n]))
        assert rel <= tol, (precision, rel)
        assert np.max(np.abs(p - po_[:st.n])) / np.max(np.abs(po_[:st.n])) <= tol


def test_fp32_coulomb_steps_and_switching_off(engine, oracle):
    box = 1e-7
    m, st, fixed, fq = _setup(engine, oracle, seed=8)
    b = _batch(engine, st.n, box, "fp32")
    b.set_state(0, _engine_state(engine, st))
    b.set_fixed_charges(0, fixed, fq)
    b.set_coulomb(EPS_R, 1e9, 1)  # one shell of periodic copies
    o = b.step(30)
    assert np.all(np.isfinite(o)) and np.all(o[0, :, 0, 2] == st.n)
    b.set_coulomb(EPS_R, enable=False)
    o2 = b.step(10)
    assert np.all(np.isfinite(o2)) and np.all(o2[0, :, 0, 2] == st.n)
    b.close()


def test_coulomb_argument_checks(engine):
    pt = engine.physics.silicon_electron("jacoboni")
    spec = engine.EnsembleSpec(0, 100, 1e6, (1, 0, 0), (1e-7, 1e-7, 2e-7), 1e-15, 1, 0)
    b = engine.BulkBatch([pt], [spec], "fp32")
    with pytest.raises(engine._lib.EmcgError):
        b.set_coulomb(EPS_R, 1e9, 1)  # periodic copies of a box that is not cubic
    with pytest.raises(engine._lib.EmcgError):
        b.set_coulomb(-1.0)
    with pytest.raises(engine._lib.EmcgError):
        b.get_coulomb(0)  # no Coulomb step yet
    with pytest.raises(ValueError):
        b.set_fixed_charges(0, np.zeros((3, 4)), np.zeros(3))
    b.close()


def test_fmm_bulk_handler_mirror(engine):
    """The handler mirror: electrons from the doping, as many fixed donors,
    the Coulomb interaction on, the reference's call sequence."""
    pt = engine.physics.silicon_electron("jacoboni")
    h = engine.FMMBulkParticleHandler((1e-7,) * 3, pt, (1, 0, 0), 1e6, images=0,
                                      eps_r=EPS_R, doping=1e24, seed=4, precision="fp32",
                                      dt=1e-16)
    h.generateInitialParticles(spacing=(1e-8,) * 3)
    assert 500 < h.getNrParticles(0) < 1500 and h.donors.shape[1] == h.getNrParticles(0)
    assert h.getNrRepeatedBoxes() == 1
    for _ in range(3):
        h.executeFMM()
        h.moveParticles(1e-16)
        h.resetForcesAndPotential()
        h.rearrangeTree()
    f, p = h.getCoulomb()
    assert f.shape == (3, h.getNrParticles(0)) and np.all(np.isfinite(f))
    assert np.isfinite(h.getAvgEnergy(0)).all() and h.getValleyOccupationProbability(0)[0] == 1
