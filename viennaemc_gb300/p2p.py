"""Particle-particle Coulomb sums of the FMM particle handlers on the GPU.

emcFMMParticleHandler (include/ParticleHandler/emcFMMParticleHandler.hpp) and
FMMBulkParticleHandler (examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp)
let scalFMM compute, for every particle, the Coulomb force and potential of
all other particles; the pair term has a 1 nm cutoff
(include/ParticleHandler/FMM/FP2PRCutoff.hpp:18-100).  coulomb() evaluates
those sums directly on the GPU (the FMM's exact value) and returns scalFMM's
container values; force_on_particles() applies the handlers' Coulomb factor.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L

EPS0 = 8.85419e-12                # include/emcConstants.hpp:21
KE = 1.0 / (4 * math.pi * EPS0)   # :27, [V m / C]


def coulomb(pos, charge, inv_cutoff=1e9, box=0.0, images=0, precision="fp64",
            return_ms=False):
    """pos (3, n) [m], charge (n,) [C] -> force (3, n), potential (n,):
    sum_j -q_i q_j d / r^3 and sum_j q_j / r (container values)."""
    p = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(3, -1))
    q = np.ascontiguousarray(np.asarray(charge, np.float64).reshape(-1))
    n = q.size
    if p.shape[1] != n:
        raise ValueError("pos and charge disagree in n")
    f = np.zeros((3, n))
    pot = np.zeros(n)
    ms = C.c_double()
    prec = L.FP64 if precision in ("fp64", L.FP64) else L.FP32
    L.check(L.lib().emcg_p2p_coulomb(p.ctypes.data_as(C.c_void_p), q.ctypes.data_as(C.c_void_p),
                                     n, float(inv_cutoff), float(box), int(images), prec,
                                     f.ctypes.data_as(C.c_void_p),
                                     pot.ctypes.data_as(C.c_void_p), C.byref(ms)))
    return (f, pot, ms.value) if return_ms else (f, pot)


def force_on_particles(pos, charge, eps_r, inv_cutoff=1e9, box=0.0, images=0,
                       precision="fp64"):
    """The particle-particle Coulomb force on each particle [N], as
    FMMBulkParticleHandler::getForceAtParticle applies it (:433-440):
    -(ke / eps_r) times the container force."""
    f, _ = coulomb(pos, charge, inv_cutoff, box, images, precision)
    return -(KE / eps_r) * f
