"""The C++ drop-in adapter (include/emcgpu_reference.hpp) against the Python
host builder: compiled with the reference's headers where the reference tree
is present (it is not on GPU hosts), it must produce the same engine
descriptor from the reference's own mechanism classes."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

REF = os.environ.get("VIENNAEMC_INCLUDE", "/root/reference")


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
