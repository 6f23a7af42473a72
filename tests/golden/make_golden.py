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
  p2p_cutoff.npz    the reference's particle-particle pair kernel with the 1 nm
                    cutoff (FP2PRCutoff.hpp), summed directly over 256 particles.
  reinit_hot_phonon.npz
                    rates, normalised tables and tau of an acoustic + hot-phonon
                    Froehlich absorption/emission set before and after the
                    reference's reinitScatterTables, with the phonon bath
                    advanced in between (the rates change).

Run from the repository root:  python tests/golden/make_golden.py [part ...]
(parts: mt bulk device output reinit p2p; default all).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

# (name, model, T, nLevels, maxE, box, spacing, doping, seed, field, dir, dt, steps, mt
#  [, grain mechanism (transmission probability, scatter rate [1/s])])
CASES = [
    ("jacoboni_300K", "jacoboni", 300.0, 1000, 1.0, 5e-7, 1e-7, 6e20, 12345, 1e6,
     (-1, 0, 0), 1e-15, 24, 0.19),
    ("refbulk_300K", "refbulk", 300.0, 1000, 1.0, 5e-7, 1e-7, 6e20, 777, 1e6,
     (-1, 0, 0), 5e-16, 24, 0.196),
    ("jacoboni_77K_111", "jacoboni", 77.0, 2000, 2.0, 5e-7, 1e-7, 6e20, 4242, 1e7,
     (1, 1, 1), 1e-15, 24, 0.19),
    # an emcGrainScatterMechanism: a grain every 5 fs on average, half of the
    # particles transmitted, half reflected
    ("jacoboni_300K_grain", "jacoboni", 300.0, 1000, 1.0, 5e-7, 1e-7, 6e20, 2468, 1e6,
     (-1, 0, 0), 1e-15, 24, 0.19, (0.5, 2e14)),
]


def make_bulk(case):
    (name, model, T, nL, maxE, box, h, doping, seed, field, dirn, dt, steps, mt) = case[:14]
    grain = case[14] if len(case) > 14 else None
    d = po.run_ref("bulk", model, T, nL, maxE, box, h, doping, seed, field, *dirn, dt, steps, mt,
                   *(grain or ()))
    m = po.silicon_model(model, temperature=T, n_levels=nL, max_energy=maxE, mt=mt, grain=grain)
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
    if grain is not None:
        out["grain"] = np.array(grain, dtype=np.float64)
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


# (name, kind, seed, dt, steps, SOR accuracy [V], device width [m])
DEVICE_CASES = [("resistor_ngp", "resistor", 42, 1e-15, 3, 1e-4, 3e-7),
                ("mosfet_cic", "mosfet", 7, 1e-15, 3, 1e-4, 3e-8),
                ("resistor_nec", "resistor_nec", 42, 1e-15, 3, 1e-4, 3e-7),
                ("mosfet_necvwd", "mosfet_vwd", 7, 1e-15, 3, 1e-4, 3e-8),
                ("resistor_surface", "resistor_surface", 4242, 4e-15, 6, 1e-4, 3e-7)]

# surface mechanisms of a harness device kind: (boundary XMIN 0 .. YMAX 3,
# oracle kind, parameter), as the harness sets them
DEVICE_SURFACES = {"resistor_surface": [(2, po.SURFACE_CONSTANT, 0.3),
                                        (3, po.SURFACE_ROUGHNESS, 0.5e-9)]}


def device_flavour(kind):
    """PM scheme, potential-based initial counts, electronVWD (rounded counts,
    tau drawn with the valley as the region) of a harness device kind."""
    scheme = {"resistor": po.NGP, "mosfet": po.CIC, "resistor_nec": po.NEC,
              "mosfet_vwd": po.NEC_VWD, "resistor_surface": po.NGP}[kind]
    return scheme, kind.startswith("mosfet"), kind == "mosfet_vwd"


def device_of(d):
    g = d["geom"]
    nx, ny = int(round(g[0] / g[2])) + 1, int(round(g[1] / g[3])) + 1
    dev = po.Device(nx, ny, g[2], g[3], g[4], d["doping"], d["region"],
                    [d[f"bnd{b}"] for b in range(4)], d["ctype"], d["cvolt"],
                    d["cpar"].reshape(-1, 3))
    dev.set_max(g[0], g[1])
    return dev


def device_model(d, kind=""):
    """Oracle model of the device harness: acoustic, Coulomb and zero-order f/g
    intervalley phonons on every doping region (4 eV tables), and the kind's
    surface mechanisms."""
    nreg = int(d["region"].max()) + 1
    m = po.Model(n_levels=1000, max_energy=4.0)
    m.add_valley([0.916, 0.196, 0.196], po.ME, 3, 0.5, 0.0, po.SI_FRAMES)
    regs = list(range(nreg))
    for r in regs:
        m.set_region_doping(r, d["doping"][d["region"] == r][0])
    m.add_mech(po.ACOUSTIC, 0, regs, 9.0)
    m.add_mech(po.COULOMB, 0, regs, 11.8)
    for fs in (po.F_SUB, po.G_SUB):
        m.add_mech(po.ZERO_IV_ABS, 0, regs, 5.23e10, 0.06, 0, fs)
        m.add_mech(po.ZERO_IV_EMI, 0, regs, 5.23e10, 0.06, 0, fs)
    for b, sk, par in DEVICE_SURFACES.get(kind, []):
        m.set_surface(b, sk, par)
    m.build_tables()
    return m, regs


def make_device(case):
    name, kind, seed, dt, steps, acc, width = case
    d = po.run_ref("device", kind, seed, dt, steps, acc, width)
    dev = device_of(d)
    m, regs = device_model(d, kind)
    for r in regs:
        for t in range(6):
            assert np.array_equal(m.raw_table(0, r, t), d[f"raw_v0_r{r}_t{t}"])
    out = {k: d[k] for k in ("doping", "region", "bnd0", "bnd1", "bnd2", "bnd3", "ctype",
                             "cvolt", "cpar", "geom", "pot_init", "pot_eq", "ex_eq", "ey_eq",
                             "mt_pre", "mt0", "nr0", "conc0", "expnr")}
    out["raw_r0"] = np.stack([d[f"raw_v0_r0_t{t}"] for t in range(6)])
    out["raw_coulomb"] = np.stack([d[f"raw_v0_r{r}_t1"] for r in regs])
    out["params"] = np.array([seed, dt, steps, acc, width])
    out["kind"] = np.array(kind)
    if kind in DEVICE_SURFACES:
        out["surface"] = np.array(DEVICE_SURFACES[kind], dtype=np.float64)
    scheme, pot_init, vwd = device_flavour(kind)
    pot, _ = dev.sor(d["pot_init"], None, 1.8, acc, True)
    assert np.array_equal(pot, d["pot_eq"])
    Ex, Ey = dev.efield(pot, scheme)
    assert np.array_equal(Ex, d["ex_eq"]) and np.array_equal(Ey, d["ey_eq"])
    rng = po.RngState(po.RNG_MT, 0)
    rng.load_mt(d["mt_pre"])
    st = dev.init_particles(m, rng, pot if pot_init else None, round_counts=vwd,
                            tau_region_is_valley=vwd)
    for f in po.STATE_F + po.STATE_I:
        assert np.array_equal(getattr(st, f), d[f"s0_{f}"])
        out[f"s0_{f}"] = d[f"s0_{f}"]
    expnr = dev.exp_nr(vwd)
    assert np.array_equal(expnr, d["expnr"])
    conc = dev.concentration(dev.assign(scheme, st))
    cap = 1 << 16
    cur = st.resize(cap)
    cur.n = st.n
    for s in range(1, steps + 1):
        pot, _ = dev.sor(pot, conc, 1.8, acc, s == 1)
        Ex, Ey = dev.efield(pot, scheme)
        assert np.array_equal(pot, d[f"pot{s}"]) and np.array_equal(Ex, d[f"ex{s}"])
        assert np.array_equal(Ey, d[f"ey{s}"])
        n_before = cur.n
        rng.start_record(1 << 20)
        rc, netto, off = dev.move(m, scheme, cur, Ex, Ey, dt, rng, s, offsets=True)
        assert rc == 0
        out[f"move_words{s}"] = rng.recorded()
        out[f"move_offsets{s}"] = off
        out[f"move_n{s}"] = np.array([n_before, cur.n])
        rng.start_record(1 << 20)
        rem_inj = dev.contacts(m, cur, cap, expnr, rng, s, tau_region_is_valley=vwd)
        out[f"inject_words{s}"] = rng.recorded()
        out[f"netto{s}"] = d[f"netto{s}"]
        assert np.array_equal(netto - rem_inj, d[f"netto{s}"])
        for f in po.STATE_F + po.STATE_I:
            assert np.array_equal(getattr(cur, f)[:cur.n], d[f"s{s}_{f}"]), (s, f)
            out[f"s{s}_{f}"] = d[f"s{s}_{f}"]
        nr = dev.assign(scheme, cur.resize(cur.n))
        conc = dev.concentration(nr)
        assert np.array_equal(nr, d[f"nr{s}"]) and np.array_equal(conc, d[f"conc{s}"])
        for k in ("pot", "ex", "ey", "nr", "conc", "cur"):
            out[f"{k}{s}"] = d[f"{k}{s}"]
    np.savez_compressed(os.path.join(HERE, f"device_{name}.npz"), **out)
    print(f"device_{name}: {dev.nx}x{dev.ny} n0={st.n} steps={steps}")


def make_output(case, outdir_name):
    """The reference's own output files after the device case's last step
    (potential, concentration and E field with suffix "Step", the particle dump,
    the step-averaged potential and concentration, the current table)."""
    import shutil
    import tempfile
    name, kind, seed, dt, steps, acc, width = case
    dst = os.path.join(HERE, outdir_name)
    scratch = os.path.join(ROOT, "oracle", "_ref", "scratch")
    os.makedirs(scratch, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="emc_out_", dir=scratch)
    po.run_ref("device", kind, seed, dt, steps, acc, width, tmp)
    os.makedirs(dst, exist_ok=True)
    for f in sorted(os.listdir(tmp)):
        shutil.copy(os.path.join(tmp, f), os.path.join(dst, f))
    shutil.rmtree(tmp)
    print(f"{outdir_name}: {sorted(os.listdir(dst))}")


P2P_CASE = (256, 5e-8, 11)  # particles, cube edge [m], seed


def make_p2p():
    """The reference's 1 nm cutoff pair kernel over 256 particles (every
    target summed over every other particle in index order), and one mutual
    call per consecutive pair."""
    n, box, seed = P2P_CASE
    d = po.run_ref("p2p", n, box, seed)
    out = {k: d[k] for k in ("x", "y", "z", "q", "fx", "fy", "fz", "pot", "mutual")}
    out["params"] = np.array(P2P_CASE, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "p2p_cutoff.npz"), **out)
    print(f"p2p_cutoff: {n} particles in a {box:g} m cube")


REINIT_CASE = (1000, 1.0, 20000, 1e-13)  # levels, max energy [eV], emissions, bath dt [s]


def make_reinit():
    nL, maxE, nEm, dtb = REINIT_CASE
    d = po.run_ref("reinit", nL, maxE, nEm, dtb)
    out = {"params": np.array(REINIT_CASE, dtype=np.float64)}
    for tag in ("init", "re"):
        nT = len([k for k in d if k.startswith(f"{tag}_raw_v0_r0_t")])
        raw = np.stack([d[f"{tag}_raw_v0_r0_t{t}"] for t in range(nT)])
        norm = np.stack([d[f"{tag}_norm_v0_r0_t{t}"] for t in range(nT)])
        out[f"{tag}_raw"], out[f"{tag}_norm"] = raw, norm
        out[f"{tag}_tau"] = d[f"{tag}_tau_v0_r0"]
        out[f"{tag}_meanNq"] = d[f"{tag}_meanNq"]
        out["names"] = np.array([d[f"{tag}_name_v0_r0_t{t}"] for t in range(nT)])
    assert not np.array_equal(out["init_raw"], out["re_raw"]), "the rates did not change"
    np.savez_compressed(os.path.join(HERE, "reinit_hot_phonon.npz"), **out)
    print(f"reinit_hot_phonon: {out['init_raw'].shape} tables, tau "
          f"{out['init_tau'][0]:.4e} -> {out['re_tau'][0]:.4e}")


def make_mt():
    d = po.run_ref("mt", 5489, 2000)
    np.savez_compressed(os.path.join(HERE, "mt19937_64.npz"), words=d["mt"], canon=d["canon"])
    print("mt19937_64: 2000 words")


if __name__ == "__main__":
    po.build(force=True)
    parts = set(sys.argv[1:]) or {"mt", "bulk", "device", "output", "reinit", "p2p"}
    if "mt" in parts:
        make_mt()
    if "bulk" in parts:
        for c in CASES:
            make_bulk(c)
    if "device" in parts:
        for c in DEVICE_CASES:
            make_device(c)
    if "output" in parts:
        make_output(DEVICE_CASES[0], "output_resistor_ngp")
        make_output(DEVICE_CASES[3], "output_mosfet_necvwd")
    if "reinit" in parts:
        make_reinit()
    if "p2p" in parts:
        make_p2p()
