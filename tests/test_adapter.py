"""The C++ drop-in adapter (include/emcgpu_reference.hpp), compiled with the
reference's headers where the reference tree is present (it is not on GPU
hosts; oracle/Makefile names where it is):

* against the Python host builder: the same engine descriptor from the
  reference's own mechanism classes and device;
* the plugins of the reference's interfaces under its stock emcSimulation,
  run against a recording stand-in of libemcgpu: the reference's step loop
  calls the engine in the reference's order and the engine's results reach
  the reference's results and output files.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden


def _reference_tree():
    out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"],
                         capture_output=True, text=True)
    return out.stdout.strip() if out.returncode == 0 else ""


REF = _reference_tree()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")),
                    reason="reference headers not available")
def test_adapter_descriptor_matches_host_builder(tmp_path):
    from viennaemc_gb300 import _lib, physics
    lib = _lib.build()
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", f"-I{REF}/include", f"-I{ROOT}/include",
                    os.path.join(ROOT, "tests", "adapter", "adapter_check.cpp"), "-o", str(exe),
                    f"-L{os.path.dirname(lib)}", "-lemcgpu",
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    pt = physics.silicon_electron("jacoboni")
    d = pt.model_desc()
    counts = [int(x) for x in out[0].split()[1:]]
    assert counts == [d.n_valleys, d.n_mechs, d.n_tablesets, d.n_levels]
    assert float.fromhex(out[1].split()[1]) == d.tablesets[0].tau_max
    for i in range(3):
        rm = float.fromhex(out[2 + i].split()[1])
        assert abs(rm - d.valleys[0].rel_mass[i]) <= 1e-14 * rm
    for m in range(d.n_mechs):
        kind, nf, shift, fs = out[5 + m].split()[1:]
        assert int(kind) == d.mechs[m].kind and int(nf) == d.mechs[m].n_final
        assert abs(float.fromhex(shift) - d.mechs[m].shift) <= 1e-15
        if d.mechs[m].n_final:
            assert int(fs) == d.mechs[m].final_sub[1][0]
    tab = np.ctypeslib.as_array(d.tables, shape=(d.n_mechs * d.n_levels,))
    for line in out[5 + d.n_mechs:]:
        if line.startswith("table"):
            i, v = line.split()[1:]
            assert float.fromhex(v) == tab[int(i)]
    # the grain mechanism: descriptor fields as the Python builder sets them
    g = physics.silicon_electron("jacoboni", grain=(0.3, 2e14)).model_desc()
    flag, prob, gtau = [l for l in out if l.startswith("grain ")][0].split()[1:]
    assert (int(flag), float.fromhex(prob), float.fromhex(gtau)) == \
        (g.grain, g.grain_transmission, g.grain_tau)
    sf = [l for l in out if l.startswith("surface ")][0].split()[1:]
    pt2 = physics.silicon_electron("jacoboni")
    pt2.setSurfaceScatterMechanism(2, physics.ConstantSurfaceScatterMechanism(0.3))
    pt2.setSurfaceScatterMechanism(3, physics.MomentumDependentSurfaceScatterMechanism(0.5e-9))
    g2 = pt2.model_desc()
    assert [int(x) for x in sf[:4]] == list(g2.surface_kind) == [0, 0, 1, 2]
    assert [float.fromhex(x) for x in sf[4:]] == list(g2.surface_param)
    flag, gtau = [l for l in out if l.startswith("nograin ")][0].split()[1:]
    assert (int(flag), float.fromhex(gtau)) == (d.grain, d.grain_tau) == (0, 1.0)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")),
                    reason="reference headers not available")
def test_adapter_device_desc_matches_host_device(tmp_path):
    """emcgpu::DeviceDesc built from the reference's emcDevice equals the Python
    host builder's descriptor for the same gated device."""
    from viennaemc_gb300 import _lib
    from viennaemc_gb300 import device as D
    from viennaemc_gb300.physics import Material
    lib = _lib.build()
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", f"-I{REF}/include", f"-I{ROOT}/include",
                    os.path.join(ROOT, "tests", "adapter", "adapter_check.cpp"), "-o", str(exe),
                    f"-L{os.path.dirname(lib)}", "-lemcgpu",
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    mat = Material(11.8, 2329., 1.45e16, 9040., 1.15)
    dev = D.Device(mat, (30e-9, 20e-9), (1e-9, 1e-9))
    dev.setDeviceWidth(3e-8)
    dev.addConstantDopingRegion((0, 8e-9), (30e-9, 20e-9), -1e24)
    dev.addConstantDopingRegion((0, 0), (10e-9, 8e-9), 1e26)
    dev.addConstantDopingRegion((10e-9, 0), (20e-9, 8e-9), -1e24)
    dev.addConstantDopingRegion((20e-9, 0), (30e-9, 8e-9), 1e26)
    dev.addOhmicContact(D.YMAX, 0, (0,), (30e-9,))
    dev.addOhmicContact(D.YMIN, 0, (0,), (10e-9,))
    dev.addGateContact(D.YMIN, 1.0, (10e-9,), (20e-9,), 3.9, 1.2e-9, 1.15 / 2.0)
    dev.addOhmicContact(D.YMIN, 0.5, (20e-9,), (30e-9,))
    d = dev.desc()
    head = [l for l in out if l.startswith("dev ")][0].split()[1:]
    assert (int(head[0]), int(head[1])) == (d.nx, d.ny)
    vals = [float.fromhex(x) for x in head[2:]]
    ref = [d.hx, d.hy, d.max_x, d.max_y, d.width, d.temperature, d.ni, d.eps_r]
    assert np.allclose(vals, ref, rtol=1e-15, atol=0)
    nodes = [l.split()[1:] for l in out if l.startswith("node ")]
    assert len(nodes) == d.nx * d.ny
    for i, dop, reg in nodes:
        assert float.fromhex(dop) == d.doping[int(i)] and int(reg) == d.region[int(i)]
    for l in out:
        if l.startswith("bnd "):
            b, c, k = map(int, l.split()[1:])
            assert k == d.boundary_contact[b][c], (b, c)
    cts = [l.split()[1:] for l in out if l.startswith("contact ")]
    assert len(cts) == d.n_contacts
    for k, t, v, p0, p1, p2 in cts:
        k = int(k)
        assert int(t) == d.contact_type[k] and float.fromhex(v) == d.contact_voltage[k]
        assert [float.fromhex(p) for p in (p0, p1, p2)] == list(d.contact_param[3 * k:3 * k + 3])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")),
                    reason="reference headers not available")
def test_adapter_raw_rates_match_host_refill(tmp_path):
    """ModelBuilder::rawRates (the reference mechanisms refilled, as the C++
    reinitScatterTables passes them to emcg_update_rates) equals the host
    model's refill bit for bit, in the same layout."""
    from viennaemc_gb300 import _lib, physics
    lib = _lib.build()
    exe = tmp_path / "adapter_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", f"-I{REF}/include", f"-I{ROOT}/include",
                    os.path.join(ROOT, "tests", "adapter", "adapter_check.cpp"), "-o", str(exe),
                    f"-L{os.path.dirname(lib)}", "-lemcgpu",
                    f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    raw = physics.silicon_electron("jacoboni").raw_rates()
    n = int([l for l in out if l.startswith("rawcount")][0].split()[1])
    assert n == raw.size
    lines = [l.split() for l in out if l.startswith("raw ")]
    assert len(lines) == (n + 88) // 89
    for _, i, v in lines:
        assert float.fromhex(v) == raw[int(i)], i


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include")),
                    reason="reference headers not available")
def test_stock_emcsimulation_runs_on_the_gpu_plugins(tmp_path):
    """emcSimulation<T, emcDevice<T, 2>, GpuPoissonSolver, GpuParticleHandler,
    GpuPMScheme> compiles (its static_asserts accept the plugin bases) and its
    execute() runs through the plugins (tests/adapter/emcsim_plugins.cpp, the
    fixtures' 21 x 11-node resistor, seed 42, 6 steps of which 2 transient).
    Against the recording stand-in (tests/adapter/stub_emcgpu.cpp):
    - the engine is created once, with the NGP scheme, the step time, the seed
      and the particle type's charge;
    - the initial particles are the reference's own (its counts and random
      stream through addParticle): the particle dump of the plugin handler
      equals the reference's initial electrons of the fixture;
    - every step calls Poisson (reset only in the first), the field, move,
      contacts and assignment in emcSimulation::performEMCStep's order, with
      the step counter advancing;
    - the concentration the solver hands over is the reference's own
      (updateCurrentParticleConcentrations of the engine's 2 particles per
      node), and the potentials follow the engine's values;
    - the current file carries the engine's netto counts (removed 3 - c minus
      injected c + 1) and the reference's running current."""
    stub = tmp_path / "stub"
    stub.mkdir()
    inc = os.path.join(ROOT, "include")
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", "-shared", "-fPIC", f"-I{inc}",
                    os.path.join(ROOT, "tests", "adapter", "stub_emcgpu.cpp"), "-o",
                    str(stub / "libemcgpu.so")], check=True)
    exe = tmp_path / "emcsim_plugins"
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", f"-I{REF}/include", f"-I{inc}",
                    os.path.join(ROOT, "tests", "adapter", "emcsim_plugins.cpp"), "-o", str(exe),
                    f"-L{stub}", "-lemcgpu", f"-Wl,-rpath,{stub}"], check=True)
    log = tmp_path / "calls.txt"
    env = dict(os.environ, EMCG_STUB_LOG=str(log))
    subprocess.run([str(exe), "res", "6"], cwd=tmp_path, env=env, check=True,
                   capture_output=True)
    calls = [l.split() for l in log.read_text().splitlines()]
    create = [c for c in calls if c[0] == "create"]
    assert len(create) == 1
    kv = dict(x.split("=") for x in create[0][4:])
    assert create[0][1:4] == ["21", "11", "2"] and kv["pm"] == "0" and kv["seed"] == "42"
    assert float.fromhex(kv["dt"]) == 1e-15 and float.fromhex(kv["charge"]) == -1.60219e-19
    # the initial electrons: the reference's own (tests/golden, seed 42)
    g = golden("device_resistor_ngp.npz")
    states = [c for c in calls if c[0] == "state"]
    assert len(states) == 1 and int(states[0][2]) == len(g["s0_E"])
    dump = np.loadtxt(tmp_path / "resElectronsEq.txt", skiprows=1)
    assert dump.shape[0] == len(g["s0_E"])
    for col, f in ((1, "px"), (2, "py"), (3, "kx"), (4, "ky"), (5, "kz"), (6, "E"), (9, "tau")):
        assert np.allclose(dump[:, col], g[f"s0_{f}"], rtol=6e-6, atol=0), f  # 6 digits
    assert np.array_equal(dump[:, 7].astype(int), g["s0_sub"])
    # the step loop, in performEMCStep's order
    seq = [c[0] if c[0] not in ("poisson", "move", "contacts", "set", "get") else " ".join(c[:2])
           + (" " + c[2] if c[0] == "poisson" else "") for c in calls]
    first = seq.index("move 0")
    step = ["set 0", "set 4", "poisson 0 1", "get 0", "set 0", "efield", "get 1", "get 2",
            "move 0", "contacts 0", "assign", "get 3"]
    assert seq[first - 8:first + 4] == step
    for s in range(1, 6):
        i = seq.index(f"move {s}")
        assert seq[i - 8:i + 4] == [x.replace("poisson 0 1", "poisson 0 0")
                                    .replace("move 0", f"move {s}")
                                    .replace("contacts 0", f"contacts {s}") for x in step]
    assert "move 6" not in seq
    # the concentration from 2 particles per node, interior node 118
    conc = [float.fromhex(c[3]) for c in calls if c[:2] == ["set", "4"]]
    assert len(conc) == 6 and np.allclose(conc, 2 / (1e-9 * 1e-9 * 3e-7) / 1.45e16, rtol=1e-12)
    # the current file: time, netto per contact, running current per contact
    cur = np.loadtxt(tmp_path / "resElectronsCurrent.txt")
    assert cur.shape == (4, 5)
    assert np.array_equal(cur[:, 1:3], np.tile([2, 0], (4, 1)))
    assert np.allclose(cur[:, 3], 2 * -1.60219e-19 / 1e-15, rtol=1e-5) and np.all(cur[:, 4] == 0)
