import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libemcgpu")
    if not config.option.basetemp:  # keep test scratch files inside the repository
        config.option.basetemp = os.path.join(ROOT, ".pytest_tmp")


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


BULK_CASES = ["bulk_jacoboni_300K.npz", "bulk_refbulk_300K.npz", "bulk_jacoboni_77K_111.npz",
              "bulk_jacoboni_300K_grain.npz"]


def case_model(g: dict):
    """(model name, temperature, levels, max energy, mt) of a bulk fixture."""
    T, nL, maxE, box, h, doping, seed, field, dt, steps, mt = g["params"]
    name = "refbulk" if g["raw"].shape[0] == 9 else "jacoboni"
    return name, float(T), int(nL), float(maxE), float(mt)


def case_grain(g: dict):
    """(transmission probability, scatter rate) of the fixture's grain
    mechanism, None without one."""
    return tuple(float(x) for x in g["grain"]) if "grain" in g else None


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


_gpu = None


def gpu_available() -> bool:
    global _gpu
    if _gpu is None:
        try:
            import torch
            _gpu = bool(torch.cuda.is_available())
        except Exception:
            _gpu = False
    return _gpu


@pytest.fixture(scope="session")
def engine():
    """The engine package; fails loudly if libemcgpu cannot be built/loaded."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    import viennaemc_gb300 as v
    v._lib.lib()
    return v
