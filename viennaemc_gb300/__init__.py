"""sm_103a engine for the ViennaEMC per-particle hot path.

The compute path is libemcgpu (CUDA, built from csrc/ for sm_103a, C ABI in
include/emcgpu.h).  This package is the host side: the band/scattering model
that produces the rate tables (physics), and mirrors of the reference's
handlers on top of the C ABI (bulk, device).
"""
from . import _lib
from .physics import (Electron, NonParabolicAnisotropValley, AcousticScatterMechanism,
                      ZeroOrderInterValleyAbsorptionScatterMechanism,
                      ZeroOrderInterValleyEmissionScatterMechanism,
                      FirstOrderInterValleyAbsorptionScatterMechanism,
                      FirstOrderInterValleyEmissionScatterMechanism, CoulombScatterMechanism,
                      GrainScatterMechanism, ConstantSurfaceScatterMechanism,
                      MomentumDependentSurfaceScatterMechanism, silicon_electron, silicon_material, thermal_voltage)
from .bulk import (BulkBatch, BulkParticleHandler, EnsembleSpec, FMMBulkParticleHandler,
                   ParticleState, ParticleStateF32)

build = _lib.build
__all__ = ["Electron", "NonParabolicAnisotropValley", "AcousticScatterMechanism",
           "ZeroOrderInterValleyAbsorptionScatterMechanism",
           "ZeroOrderInterValleyEmissionScatterMechanism",
           "FirstOrderInterValleyAbsorptionScatterMechanism",
           "FirstOrderInterValleyEmissionScatterMechanism", "CoulombScatterMechanism",
           "GrainScatterMechanism", "ConstantSurfaceScatterMechanism",
           "MomentumDependentSurfaceScatterMechanism", "silicon_electron", "silicon_material", "thermal_voltage", "BulkBatch",
           "BulkParticleHandler", "EnsembleSpec", "FMMBulkParticleHandler", "ParticleState",
           "build"]
