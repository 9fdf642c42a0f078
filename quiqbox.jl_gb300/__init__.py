"""GB300-native (sm_103a) integral and Hartree–Fock path of Quiqbox.jl.

The CUDA library ``_build/libquiqbox_gb300.so`` implements the Gaussian-orbital
integrals (Boys function, overlap, kinetic, nuclear attraction, electron
repulsion), a fused ERI + J/K build with no stored ERI tensor, and the RHF/UHF
SCF driver, behind the C ABI of include/quiqbox_gb300.h.  This package is the
host-side mirror of the reference's Julia API on top of that ABI.
"""
from .basis import (PrimitiveOrb, CompositeOrb, NuclearCluster, FlatBasis, genGaussTypeOrb,  # noqa: F401
                    genGaussTypeOrbSeq, nucRepulsion, flatten, prepareSpinConfiguration,
                    cartesian_components, norm_factor, basis_set_names, NUCLEAR_CHARGE)
from .api import (overlaps, overlap, elecKinetics, elecKinetic, nucAttractions, nucAttraction,  # noqa: F401
                  coreHamiltonian, elecRepulsions, elecRepulsion, elecRepulsion_list, jk, SCFconfig,
                  HFconfig, HFfinalInfo, runHartreeFock, RCHartreeFock, UOHartreeFock, fp64_peak, fp64_dmma_peak, device_info,
                  computeBoysSequence, computeBoysFunc, multipoleMoments, multipoleMoment,
                  runHartreeFockBatched, BatchSCFConfig, BatchSCFResult, jk_autotune, diis_coefficients,
                  DimensionMismatch, DomainError)
from ._lib import Context, load as load_library, LIB_PATH, EXPORTED  # noqa: F401
from .differentiation import GaussShell, rhf_energy_gradient, rhf_energy  # noqa: F401
