"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_driver (the reference's own classes compiled from its
headers by `make -C oracle ref`, which needs the reference tree) and stores:

  bulk_<case>.npz   raw rate tables and tau of the (valley, region)
                    set, the reference's initial particles, its mt19937_64 state
                    after initialisation, particle states after each of the
                    first steps, per-step observables, and the per-particle
                    attribution of the reference's random words for each step
                    (offsets into `words`, recorded by the oracle while it
                    reproduced the reference bit for bit).
  mt19937_64.npz    first words of std::mt19937_64(5489) and canonical maps.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

# (name, model, T, nLevels, maxE, box, spacing, doping, seed, field, dir, dt, steps, mt)
CASES = [
    ("jacoboni_300K", "jacoboni", 300.0, 1000, 1.0, 5e-7, 1e-7, 6e20, 12345, 1e6,
     (-1, 0, 0), 1e-15, 24, 0.19),
    ("refbulk_300K", "refbulk", 300.0, 1000, 1.0, 5e-7, 1e-7, 6e20, 777, 1e6,
     (-1, 0, 0), 5e-16, 24, 0.196),
    ("jacoboni_77K_111", "jacoboni", 77.0, 2000, 2.0, 5e-7, 1e-7, 6e20, 4242, 1e7,
     (1, 1, 1), 1e-15, 24, 0.19),
]


def make_bulk(case):
    (name, model, T, nL, maxE, box, h, doping, seed, field, dirn, dt, steps, mt) = case
    d = po.run_ref("bulk", model, T, nL, maxE, box, h, doping, seed, field, *dirn, dt, steps, mt)
    m = po.silicon_model(model, temperature=T, n_levels=nL, max_energy=maxE, mt=mt)
    nT = m.n_tables(0, 0)
    raw = np.stack([d[f"raw_v0_r0_t{t}"] for t in range(nT)])
    norm = np.stack([d[f"norm_v0_r0_t{t}"] for t in range(nT)])
    names = np.array([d[f"name_v0_r0_t{t}"] for t in range(nT)])
    # normalised tables are cumsum(raw) / max, checked against the reference here
    cum = np.cumsum(raw, axis=0)
    assert np.array_equal(cum / cum[-1].max(), norm)
    out = {"raw": raw, "names": names, "tau": d["tau_v0_r0"],
           "applied_field": d["appliedField"], "field_dir": d["appliedFieldDir"],
           "mt0": d["mt0"], "dt": np.array(dt), "box": np.array(box),
           "params": np.array([T, nL, maxE, box, h, doping, seed, field, dt, steps, mt])}
    st = po.state_from_ref(d, "s0")
    for f in po.STATE_F + po.STATE_I:
        out[f"s0_{f}"] = getattr(st, f)
    # replay the reference's stream through the oracle, recording attribution
    rng = po.RngState(po.RNG_MT, 0)
    rng.load_mt(d["mt0"])
    force = -po.Q * d["appliedField"]
    cur = st.copy()
    words, offs = [], []
    base = 0
    for s in range(1, steps + 1):
        rng.start_record(1 << 20)
        rc, off = m.bulk_step(cur, dt, force, [box] * 3, rng, s, offsets=True)
        assert rc == 0
        w = rng.recorded()
        words.append(w)
        offs.append(off + base)
        base += len(w)
        ref = po.state_from_ref(d, f"s{s}")
        for f in po.STATE_F + po.STATE_I:
            a, b = getattr(cur, f), getattr(ref, f)
            assert np.array_equal(a, b), f"oracle diverged from reference: step {s} {f}"
            out[f"s{s}_{f}"] = b
        out[f"obs{s}"] = d[f"obs{s}"]
    out["obs0"] = d["obs0"]
    out["words"] = np.concatenate(words).astype(np.uint64)
    out["offsets"] = np.stack(offs).astype(np.int64)  # [steps, n+1] into words
    np.savez_compressed(os.path.join(HERE, f"bulk_{name}.npz"), **out)
    print(f"bulk_{name}: n={st.n} steps={steps} words={len(out['words'])} tables={nT}")


def make_mt():
    d = po.run_ref("mt", 5489, 2000)
    np.savez_compressed(os.path.join(HERE, "mt19937_64.npz"), words=d["mt"], canon=d["canon"])
    print("mt19937_64: 2000 words")


if __name__ == "__main__":
    po.build(force=True)
    make_mt()
    for c in CASES:
        make_bulk(c)
