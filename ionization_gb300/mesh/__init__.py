"""Mesh time-evolution API (same names as ionization.mesh)."""

from .data import (  # noqa: F401
    DATA_NAME_TO_DATASTORE_TYPE,
    DEFAULT_DATASTORE_TYPES,
    Data,
    Datastore,
    DirectionalRadialProbabilityCurrent,
    Fields,
    InnerProducts,
    InternalEnergyExpectationValue,
    Norm,
    NormBySphericalHarmonic,
    NormWithinRadius,
    RExpectationValue,
    TotalEnergyExpectationValue,
    ZExpectationValue,
)
from .evolution_methods import (  # noqa: F401
    AlternatingDirectionImplicit,
    EvolutionMethod,
    FourierSplitOperator,
    SplitInteractionOperator,
)
from .mesh_operators import (  # noqa: F401
    CylindricalSliceLengthGaugeOperators,
    DotOperator,
    KineticEnergyDerivation,
    LineLengthGaugeOperators,
    LineVelocityGaugeOperators,
    MeshOperator,
    MeshOperators,
    RectangleLengthGaugeOperators,
    SphericalHarmonicLengthGaugeOperators,
    SphericalHarmonicVelocityGaugeOperators,
    SphericalSliceLengthGaugeOperators,
    SumOfOperators,
    TDMAOperator,
    add_to_diagonal_sparse_matrix_diagonal,
    apply_operators_sequentially,
)
from .meshes import (  # noqa: F401
    CylindricalSliceMesh,
    LineMesh,
    QuantumMesh,
    RectangleMesh,
    SphericalHarmonicMesh,
    SphericalSliceMesh,
    WrappingDirection,
)
from .sims import (  # noqa: F401
    CylindricalSliceSpecification,
    LineSpecification,
    MeshSimulation,
    MeshSpecification,
    RectangleSpecification,
    SphericalHarmonicSimulation,
    SphericalHarmonicSpecification,
    SphericalSliceSpecification,
)
