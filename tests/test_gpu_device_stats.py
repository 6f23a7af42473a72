"""Terminal current of the device engine against the reference algorithm,
over 16 seeds.

The reference's device step (emcSimulation::performEMCStep,
include/emcSimulation.hpp:164-193: SOR Poisson, E field, drift and scatter,
ohmic contacts, assignment) is run by the oracle's restatement with the
reference's own random-number engine, std::mt19937_64 seeded 1..16 -- the
oracle is bit-identical to the reference on the device fixtures -- on the
fixtures' 21 x 11-node resistor (Nd 1e25, 0.1 V, NGP, dt 1 fs), Poisson
converged (SOR to 1e-9 V).  The engine runs the same device on its Philox
streams, seeds 1..16, in FP64 and in FP32, Poisson to a relative residual of
1e-10.  Observable: the netto particle flow per step at each contact, the
quantity emcSimulationResults::updateCurrent turns into the terminal current
(include/emcSimulationResults.hpp:125-150), averaged over 400 steps after
100.  The 16-seed means must agree within 3 sigma of their difference: FP64
engine against the reference algorithm, FP32 engine against the FP64 engine.
"""
import numpy as np
import pytest

from conftest import golden
from test_gpu_device import _sim
from test_oracle_device_golden import _oracle_device, _oracle_model

pytestmark = pytest.mark.gpu
CASE = "device_resistor_ngp.npz"
SEEDS, WARM, K = range(1, 17), 100, 400


def _reference_flow(oracle, g):
    dev = _oracle_device(oracle, g)
    m, _ = _oracle_model(oracle, g)
    dt = float(g["params"][1])
    out = []
    for seed in SEEDS:
        rng = oracle.RngState(oracle.RNG_MT, seed)
        pot, _ = dev.sor(g["pot_init"], None, 1.8, 1e-9, True)
        st = dev.init_particles(m, rng, None)
        conc = dev.concentration(dev.assign(0, st))
        cur = st.resize(1 << 14)
        cur.n = st.n
        tot = np.zeros(2)
        for s in range(1, WARM + K + 1):
            pot, _ = dev.sor(pot, conc, 1.8, 1e-9, s == 1)
            Ex, Ey = dev.efield(pot, 0)
            rc, netto, _ = dev.move(m, 0, cur, Ex, Ey, dt, rng, s)
            assert rc == 0
            ri = dev.contacts(m, cur, 1 << 14, dev.exp_nr(False), rng, s)
            if s > WARM:
                tot += netto - ri
            conc = dev.concentration(dev.assign(0, cur.resize(cur.n)))
        out.append(tot / K)
    return np.array(out)


def _engine_flow(engine, g, precision):
    out = []
    for seed in SEEDS:
        sim, _, _ = _sim(engine, g, CASE, precision=precision, seed=seed, poisson_rtol=1e-10,
                         poisson_max_cycles=200)
        sim.calcEquilibriumCharacteristics()
        netto = sim.performEMCStep(WARM + K)
        out.append(netto[WARM:].mean(axis=0))
        sim.close()
    return np.array(out)


def _agree(a, b):
    ma, mb = a.mean(axis=0), b.mean(axis=0)
    se = np.sqrt(a.var(axis=0, ddof=1) / len(a) + b.var(axis=0, ddof=1) / len(b))
    return np.abs(ma - mb), 3 * se


def test_device_current_matches_reference_16_seeds(engine, oracle):
    g = golden(CASE)
    ref = _reference_flow(oracle, g)
    f64 = _engine_flow(engine, g, "fp64")
    f32 = _engine_flow(engine, g, "fp32")
    # the current is well resolved: its mean is far above its sampling error
    assert np.all(np.abs(ref.mean(axis=0)) > 20 * ref.std(axis=0, ddof=1) / 4)
    d, lim = _agree(f64, ref)
    assert np.all(d <= lim), ("fp64 vs reference", f64.mean(0), ref.mean(0), lim)
    d, lim = _agree(f32, f64)
    assert np.all(d <= lim), ("fp32 vs fp64", f32.mean(0), f64.mean(0), lim)
    # particles are conserved on average: what leaves at one contact enters at the other
    for x in (ref, f64, f32):
        tot = x.sum(axis=1)
        assert abs(tot.mean()) <= 3 * tot.std(ddof=1) / 4 + 0.05
