"""The CPU oracle against vectors produced by the reference itself.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py from
the reference's own classes (oracle/_ref/ref_driver).  Every check here is
bit-exact: the oracle restates the reference operation by operation.
"""
import numpy as np
import pytest

from conftest import BULK_CASES, case_grain, case_model, golden

pytestmark = []


def test_mt19937_64_matches_reference(oracle):
    g = golden("mt19937_64.npz")
    r = oracle.RngState(oracle.RNG_MT, 5489)
    L = oracle.lib()
    import ctypes as C
    words = np.array([L.oc_mt_next(C.byref(r.r)) for _ in range(len(g["words"]))], np.uint64)
    assert np.array_equal(words, g["words"])


def test_mt19937_64_standard_value(oracle):
    # the C++ standard fixes the 10000th output of a default-seeded mt19937_64
    import ctypes as C
    r = oracle.RngState(oracle.RNG_MT, 5489)
    L = oracle.lib()
    for _ in range(9999):
        L.oc_mt_next(C.byref(r.r))
    assert L.oc_mt_next(C.byref(r.r)) == 9981545732273789042


def test_canonical_map_matches_libstdcxx(oracle):
    g = golden("mt19937_64.npz")
    L = oracle.lib()
    u = np.array([L.oc_canonical(int(w)) for w in g["words"]])
    dlog = u * (1.0 - 1e-6) + 1e-6
    expect = np.where(np.arange(len(u)) % 2 == 1, dlog, u)
    assert np.array_equal(expect, g["canon"])


def test_canonical_clamps_below_one(oracle):
    L = oracle.lib()
    assert L.oc_canonical(0xFFFFFFFFFFFFFFFF) == np.nextafter(1.0, 0.0)
    assert L.oc_canonical(0) == 0.0


@pytest.mark.parametrize("ctr,key,expect", [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
])
def test_philox4x32_10_known_answers(oracle, ctr, key, expect):
    # known-answer vectors of the Random123 distribution (kat_vectors)
    import ctypes as C
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    oracle.lib().oc_philox4x32_10(c, k, o)
    assert tuple(o) == expect


@pytest.mark.parametrize("case", BULK_CASES)
def test_rate_tables_match_reference(oracle, case):
    g = golden(case)
    name, T, nL, maxE, mt = case_model(g)
    m = oracle.silicon_model(name, temperature=T, n_levels=nL, max_energy=maxE, mt=mt,
                            grain=case_grain(g))
    assert m.n_tables(0, 0) == g["raw"].shape[0]
    for t in range(g["raw"].shape[0]):
        assert np.array_equal(m.raw_table(0, 0, t), g["raw"][t]), t
    cum = np.cumsum(g["raw"], axis=0)
    norm = cum / cum[-1].max()
    for t in range(g["raw"].shape[0]):
        assert np.array_equal(m.norm_table(0, 0, t), norm[t])
    assert m.tau(0, 0) == g["tau"][0]


@pytest.mark.parametrize("case", BULK_CASES)
def test_initial_particles_match_reference(oracle, case):
    g = golden(case)
    name, T, nL, maxE, mt = case_model(g)
    box, h, doping, seed = g["params"][3:7]
    m = oracle.silicon_model(name, temperature=T, n_levels=nL, max_energy=maxE, mt=mt,
                            grain=case_grain(g))
    rng = oracle.RngState(oracle.RNG_MT, int(seed))
    st = m.bulk_init([box] * 3, [h] * 3, doping, rng)
    assert st.n == len(g["s0_E"])
    for f in oracle.STATE_F + oracle.STATE_I:
        assert np.array_equal(getattr(st, f), g[f"s0_{f}"]), f
    mt_state = np.array(list(rng.r.mt), np.uint64)
    assert np.array_equal(mt_state, g["mt0"][:312]) and rng.r.mt_idx == g["mt0"][312]


def _state(oracle, g, s):
    return oracle.State.from_dict({f: g[f"s{s}_{f}"] for f in oracle.STATE_F + oracle.STATE_I})


@pytest.mark.parametrize("case", BULK_CASES)
@pytest.mark.parametrize("mode", ["mt", "replay"])
def test_trajectories_match_reference(oracle, case, mode):
    g = golden(case)
    name, T, nL, maxE, mt = case_model(g)
    m = oracle.silicon_model(name, temperature=T, n_levels=nL, max_energy=maxE, mt=mt,
                            grain=case_grain(g))
    dt, box = float(g["dt"]), float(g["box"])
    force = -oracle.Q * g["applied_field"]
    steps = g["offsets"].shape[0]
    cur = _state(oracle, g, 0)
    if mode == "mt":
        rng = oracle.RngState(oracle.RNG_MT, 0)
        rng.load_mt(g["mt0"])
    else:
        rng = oracle.RngState(oracle.RNG_MT, 0)
        rng.set_replay(g["words"])
    for s in range(1, steps + 1):
        rc, _ = m.bulk_step(cur, dt, force, [box] * 3, rng, s)
        assert rc == 0
        ref = _state(oracle, g, s)
        for f in oracle.STATE_F + oracle.STATE_I:
            assert np.array_equal(getattr(cur, f), getattr(ref, f)), (s, f)
        obs = m.observables(cur, g["field_dir"])
        assert np.array_equal(obs.reshape(-1), g[f"obs{s}"]), s
    if mode == "replay":
        assert rng.r.pos == len(g["words"])


@pytest.mark.parametrize("case", BULK_CASES)
def test_word_attribution_is_contiguous(case):
    g = golden(case)
    off = g["offsets"]
    assert off[0, 0] == 0 and off[-1, -1] == len(g["words"])
    assert np.all(np.diff(off, axis=1) >= 0)
    assert np.array_equal(off[1:, 0], off[:-1, -1])


def test_drift_known_answers_reference_kat(oracle):
    """Inputs and tolerances of the reference's tests/testParticleMovement:
    analytic free flight from k = 0 in isotropic and anisotropic valleys."""
    hbar = 1.05459e-34
    me = 9.11e-31
    dT = 1e-12
    frames = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((0, 1, 0), (1, 0, 0), (0, 0, 1)),
              ((0, 0, 1), (0, 1, 0), (1, 0, 0)), ((-1, 1, 1), (1, 1, 0), (1, -1, 2)),
              ((1, 1, 1), (-1, 1, 0), (-1, -1, 2)), ((-1, -1, 1), (1, 0, 1), (-1, 2, 1))]

    def expected(force, eff):
        mc = 3.0 / sum(1.0 / m for m in eff)
        k = [f * dT * np.sqrt(mc / m) / hbar for f, m in zip(force, eff)]
        pos = [kn / 2.0 * dT / np.sqrt(m * mc) * hbar for kn, m in zip(k, eff)]
        return np.array(k), np.array(pos)

    def to_cs(d1, d2, d3, v):
        return np.array([np.dot(d, v) / np.linalg.norm(d) for d in (d1, d2, d3)])

    def from_cs(d1, d2, d3, v):
        return sum(np.array(d, float) / np.linalg.norm(d) * v[i] for i, d in enumerate((d1, d2, d3)))

    import ctypes as C
    L = oracle.lib()
    # isotropic: masses (1, 1, 1), 6 subvalleys with identity frames
    m = oracle.Model()
    m.add_valley([1, 1, 1], me, 6, 0.5)
    force = [1e-19, 5e-19, 1e-20]
    ek, ep = expected(force, [1, 1, 1])
    for sub in range(6):
        k = np.zeros(3)
        E = np.zeros(1)
        pos = np.zeros(3)
        L.oc_drift(m.h, dT, oracle.dptr(k), oracle.dptr(E), 0, sub, oracle.dptr(pos), 3,
                   oracle.dptr(np.array(force)))
        assert np.all(np.abs(pos - ep) <= 1e-9) and np.all(np.abs(k - ek) <= 1e-9)
    # anisotropic: masses (0.1, 0.5, 1) in six rotated frames
    m2 = oracle.Model()
    m2.add_valley([0.1, 0.5, 1], me, 6, 0.5, 0.0, frames)
    force = np.array([1e-17, 1e-17, 1e-17])
    for sub, (d1, d2, d3) in enumerate(frames):
        k = np.zeros(3)
        E = np.zeros(1)
        pos = np.full(3, 1e-7)
        L.oc_drift(m2.h, dT, oracle.dptr(k), oracle.dptr(E), 0, sub, oracle.dptr(pos), 3,
                   oracle.dptr(force))
        ek, ep = expected(to_cs(d1, d2, d3, force), [0.1, 0.5, 1])
        ek = from_cs(d1, d2, d3, ek)
        ep = from_cs(d1, d2, d3, ep) + 1e-7
        eE = L.oc_energy(m2.h, 0, oracle.dptr(np.ascontiguousarray(ek)))
        assert np.all(np.abs(k - ek) <= 1e-5), sub
        assert np.all(np.abs(pos - ep) <= 1e-10), sub
        assert abs(E[0] - eE) <= 1e-10
