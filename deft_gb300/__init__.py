"""deft_gb300: GB300-native (sm_103a) FMT functional + conjugate-gradient hot
path of deft (droundy/deft), behind a C ABI (include/deft_gb300.h) with a
Python mirror of the reference's Functional / Grid / Minimizer API."""
from .api import (  # noqa: F401
    ChemicalPotential,
    ConjugateGradient,
    Context,
    ExternalPotential,
    Functional,
    Grid,
    GridDescription,
    HardSpheresWBnotensor,
    IdealGas,
    Lattice,
    EffectivePotentialToDensity,
    MaxIter,
    Minimizer,
    OfEffectivePotential,
    Precision,
    PreconditionedConjugateGradient,
    QuadraticLineMinimizer,
    SecantLineMinimizer,
    constrain,
    default_context,
    find_chemical_potential,
)
from ._lib import DeftError, LIB_PATH  # noqa: F401
