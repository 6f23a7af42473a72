"""Host-side checks that need no GPU: the C ABI library loads and exports every
entry point of include/emcgpu.h, rejects invalid arguments before touching
the device, and the host model builder reproduces the reference's tables."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import BULK_CASES, ROOT, case_grain, case_model, golden


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "emcgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const char \*|int32_t|int64_t)\s*\n?\s*(emcg_\w+)\(",
                                 txt, re.M)))


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ("emcg_bulk_create", "emcg_bulk_step", "emcg_set_replay", "emcg_destroy",
              "emcg_last_error", "emcg_set_state", "emcg_get_state", "emcg_bulk_init"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from viennaemc_gb300 import _lib
    path = _lib.build()
    lib = C.CDLL(path)
    for s in header_symbols():
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True,
                         text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(header_symbols()) <= exported


@pytest.mark.parametrize("case", BULK_CASES)
def test_host_model_builder_matches_reference_tables(case):
    from viennaemc_gb300 import physics
    g = golden(case)
    name, T, nL, maxE, mt = case_model(g)
    pt = physics.silicon_electron(name, temperature=T, n_levels=nL, max_energy=maxE, mt=mt,
                                  grain=case_grain(g))
    raw = pt.scatterHandler.raw[(0, 0)]
    assert np.array_equal(raw, g["raw"])
    assert pt.getTau(0, 0) == g["tau"][0]
    names = [m.getName() for m in pt.scatterHandler.mechanisms]
    assert names == [str(x) for x in g["names"]]
    # the grain mechanism: the reference's initial particles draw their grain
    # timers with 1 / rate (mean of the fixture's s0 timers within 3 sigma)
    d = pt.model_desc()
    grain = case_grain(g)
    if grain is None:
        assert (d.grain, d.grain_tau) == (0, 1.0)
    else:
        assert (d.grain, d.grain_transmission, d.grain_tau) == (1, grain[0], 1.0 / grain[1])
        gt = g["s0_gtau"]
        assert abs(gt.mean() - d.grain_tau) < 3 * d.grain_tau / np.sqrt(len(gt))


def _desc(**over):
    from viennaemc_gb300 import physics
    pt = physics.silicon_electron("jacoboni")
    d = pt.model_desc()
    for k, v in over.items():
        setattr(d, k, v)
    return pt, d


def _create(models, ens, prec=0):
    from viennaemc_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    n_models = len(models)
    marr = (_lib.ModelDesc * max(n_models, 1))(*models)
    earr = (_lib.EnsembleDesc * max(len(ens), 1))(*ens)
    st = L.emcg_bulk_create(marr, n_models, earr, len(ens), prec, C.byref(h))
    return st, L.emcg_last_error().decode()


def _ens(**over):
    from viennaemc_gb300 import _lib
    e = _lib.EnsembleDesc()
    e.model, e.capacity, e.charge, e.dt, e.seed = 0, 16, -1.60219e-19, 1e-15, 1
    for i in range(3):
        e.box[i] = 5e-7
        e.field_dir[i] = 1.0 if i == 0 else 0.0
    for k, v in over.items():
        setattr(e, k, v)
    return e


@pytest.mark.parametrize("bad,msg", [
    (dict(n_valleys=0), "n_valleys"),
    (dict(n_levels=0), "n_levels"),
    (dict(max_energy=-1.0), "max_energy"),
    (dict(grain_tau=0.0), "grain_tau"),
    (dict(grain=2), "grain must be 0 or 1"),
    (dict(surface_kind=(C.c_int32 * 4)(0, 0, 3, 0)), "surface_kind"),
    (dict(surface_kind=(C.c_int32 * 4)(0, 0, 0, 2)), "roughness height"),
    (dict(grain=1, grain_transmission=float("nan")), "grain_transmission"),
])
def test_create_rejects_bad_model_without_gpu(bad, msg):
    pt, d = _desc(**bad)
    st, err = _create([d], [_ens()])
    assert st == -1 and msg in err


def test_create_rejects_bad_ensembles_and_precision():
    pt, d = _desc()
    st, err = _create([d], [_ens(model=3)])
    assert st == -1 and "model" in err
    st, err = _create([d], [_ens(dt=0.0)])
    assert st == -1 and "dt" in err
    st, err = _create([d], [_ens()], prec=7)
    assert st == -1 and "precision" in err


def test_create_rejects_mechanism_of_another_valley():
    pt, d = _desc()
    d.mechs[3].valley = 1  # valley 1 does not exist
    st, err = _create([d], [_ens()])
    assert st == -1 and "valley" in err


def test_create_rejects_bad_final_subvalley():
    pt, d = _desc()
    d.mechs[1].final_sub[0][0] = 7  # valley has 3 subvalleys
    st, err = _create([d], [_ens()])
    assert st == -1 and "final subvalley" in err


def test_null_handle_calls_fail_cleanly():
    from viennaemc_gb300 import _lib
    L = _lib.lib()
    assert L.emcg_bulk_step(None, 1, 0, None) == -1
    assert L.emcg_destroy(None) == 0
    assert L.emcg_num_particles(None, 0) == -1


def test_model_descriptor_layout():
    from viennaemc_gb300 import physics
    pt = physics.silicon_electron("jacoboni")
    d = pt.model_desc()
    assert d.n_valleys == 1 and d.n_mechs == 13 and d.n_tablesets == 1
    ts = d.tablesets[0]
    assert ts.n_tables == 13 and list(ts.mech)[:13] == list(range(13))
    nT, nL = 13, d.n_levels
    tab = np.ctypeslib.as_array(d.tables, shape=(nT * nL,)).reshape(nT, nL)
    assert np.array_equal(tab, pt.scatterHandler.norm[(0, 0)])
    # intervalley energy shifts: absorption +hw, emission -hw
    for i, m in enumerate(pt.scatterHandler.mechanisms[1:], start=1):
        sign = 1 if m.absorption else -1
        assert d.mechs[i].shift == sign * m.phonon_energy


def test_bulk_handler_field_and_observable_averaging():
    from viennaemc_gb300.bulk import BulkBatch
    sums = np.zeros((1, 2, 1, 3))
    sums[0, :, 0] = [[3.0, -6.0, 3.0], [0.0, 0.0, 0.0]]
    a = BulkBatch.averages(sums, [3])
    assert a["energy"][0, 0, 0] == 1.0 and a["drift_velocity"][0, 0, 0] == -2.0
    assert a["occupation"][0, 0, 0] == 1.0 and a["energy"][0, 1, 0] == 0.0


def test_float_state_fields_are_fixed_views():
    """ParticleStateF32 builds its C descriptor once: its fields are views of
    one block, written in place; rebinding a field is refused (the descriptor
    would point at the old array)."""
    from viennaemc_gb300.bulk import STATE_F, ParticleStateF32
    st = ParticleStateF32(5)
    st.kx[:] = np.arange(5, dtype=np.float32)
    st.meta[:] = 7
    d = st.desc()
    assert C.cast(d.kx, C.c_void_p).value == st.kx.ctypes.data
    assert C.cast(d.meta, C.c_void_p).value == st.meta.ctypes.data and d.n == 5
    assert d.kx[4] == 4.0 and d.meta[2] == 7
    for f in STATE_F + ("meta",):
        with pytest.raises(AttributeError, match="in place"):
            setattr(st, f, np.zeros(5, np.float32))
    st.note = "other attributes stay free"


def test_step_from_host_checks_arguments_without_gpu():
    """emcg_bulk_step_from_host refuses a NULL handle or state before any
    CUDA call."""
    from viennaemc_gb300 import _lib as L
    lib = L.lib()
    assert lib.emcg_bulk_step_from_host(None, 0, None, 1, 0, None) == -1


def test_poisson_exp_is_accurate(tmp_path):
    """The Poisson residual's table-driven exp (emcg_exp.h, Tang's method)
    agrees with libm's exp to about one unit in the last place over the range
    it serves, and hands overflow, underflow and NaN to the library."""
    exe = tmp_path / "exp_check"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT}/viennaemc_gb300/csrc",
                    f"{ROOT}/tests/native/exp_check.cpp", "-o", str(exe)], check=True)
    worst, _, specials = subprocess.run([str(exe)], check=True, capture_output=True,
                                        text=True).stdout.split()
    assert float(worst) < 5e-16 and specials == "1"


# the frames of the reference's tests/testValleyCoordinateTransformation: an
# X valley with 6 subvalleys and an L valley with 8 (the last repeats the sixth)
X_FRAMES = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((-1, 0, 0), (0, 1, 0), (0, 0, 1)),
            ((0, 1, 0), (1, 0, 0), (0, 0, 1)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
            ((0, 0, 1), (0, 1, 0), (1, 0, 0)), ((0, 0, -1), (0, 1, 0), (1, 0, 0))]
L_FRAMES = [((1, 1, 1), (-1, 1, 0), (-1, -1, 2)), ((-1, -1, -1), (-1, 1, 0), (-1, -1, 2)),
            ((-1, 1, 1), (1, 1, 0), (1, -1, 2)), ((1, -1, 1), (1, 1, 0), (-1, 1, 2)),
            ((1, 1, -1), (1, 0, 1), (-1, 2, 1)), ((-1, -1, 1), (1, 0, 1), (-1, 2, 1)),
            ((-1, 1, -1), (1, 1, 0), (-1, 1, 2)), ((-1, -1, 1), (1, 0, 1), (-1, 2, 1))]
VALLEY_FRAMES = {"X": ((0.9, 0.1, 0.1), 0.5, X_FRAMES), "L": ((0.8, 0.2, 0.2), 0.3, L_FRAMES)}


@pytest.mark.parametrize("name", sorted(VALLEY_FRAMES))
def test_valley_coordinate_transformation_known_answers(name):
    """tests/testValleyCoordinateTransformation of the reference: the ellipse
    coordinates of (1, 2, 3) are its inner products with the subvalley's
    normalised axes, and the way back gives (1, 2, 3) again (1e-9)."""
    from viennaemc_gb300 import physics
    masses, alpha, frames = VALLEY_FRAMES[name]
    v = physics.NonParabolicAnisotropValley(list(masses), 9.11e-31, len(frames), alpha)
    for s, (a, b, c) in enumerate(frames):
        v.setSubValleyEllipseCoordSystem(s, a, b, c)
    vec = np.array([1.0, 2.0, 3.0])
    for s, dirs in enumerate(frames):
        R = np.array(v.rot[s]).reshape(3, 3)
        ell = R @ vec
        for i, d in enumerate(dirs):
            d = np.array(d, float) / np.linalg.norm(d)
            assert abs(ell[i] - vec @ d) <= 1e-9
        assert np.all(np.abs(R.T @ ell - vec) <= 1e-9)
    with pytest.raises(ValueError):  # the reference refuses axes that are not orthogonal
        v.setSubValleyEllipseCoordSystem(0, (1, 0, 0), (1, 1, 0), (0, 0, 1))


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct of include/emcgpu.h that the Python host fills has the
    header's size and field offsets (a C program compiled against the header
    prints them)."""
    import subprocess
    from viennaemc_gb300 import _lib
    pairs = {"emcg_valley_desc": _lib.ValleyDesc, "emcg_mech_desc": _lib.MechDesc,
             "emcg_tableset_desc": _lib.TablesetDesc, "emcg_model_desc": _lib.ModelDesc,
             "emcg_ensemble_desc": _lib.EnsembleDesc, "emcg_state": _lib.StateDesc,
             "emcg_state_f32": _lib.StateF32Desc, "emcg_device_desc": _lib.DeviceDesc,
             "emcg_device_config": _lib.DeviceConfig}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "emcgpu.h"',
             "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        cname, f, v = line.split()
        got[(cname, f)] = int(v)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
