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
