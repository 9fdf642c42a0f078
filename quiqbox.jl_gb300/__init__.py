"""GB300-native integral + Hartree–Fock path of Quiqbox.jl (placeholder; API filled in below)."""
from .basis import (PrimitiveOrb, CompositeOrb, NuclearCluster, genGaussTypeOrb,  # noqa: F401
                    genGaussTypeOrbSeq, nucRepulsion, flatten, FlatBasis,
                    prepareSpinConfiguration, cartesian_components, norm_factor)
