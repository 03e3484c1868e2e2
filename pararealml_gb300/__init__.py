"""GB300-native (sm_103a) FDM and Parareal engine with PararealML's interface.

The problem-definition classes mirror ``pararealml``'s public API so that
problems written for the reference construct unchanged; the operators
(``pararealml_gb300.operators.fdm.FDMOperator``,
``pararealml_gb300.operators.parareal.PararealOperator``) run on the GPU
through the C ABI of ``libprml_gb300.so`` and also accept the reference's
own problem objects.
"""

from .boundary_condition import (
    BoundaryCondition,
    CauchyBoundaryCondition,
    ConstantBoundaryCondition,
    ConstantFluxBoundaryCondition,
    ConstantValueBoundaryCondition,
    DirichletBoundaryCondition,
    NeumannBoundaryCondition,
    vectorize_bc_function,
)
from .constrained_problem import ConstrainedProblem
from .constraint import Constraint, apply_constraints_along_last_axis
from .differential_equation import (
    LHS,
    BurgersEquation,
    CahnHilliardEquation,
    ConvectionDiffusionEquation,
    DifferentialEquation,
    DiffusionEquation,
    NavierStokesEquation,
    PopulationGrowthEquation,
    ShallowWaterEquation,
    SymbolicEquationSystem,
    Symbols,
    WaveEquation,
)
from .initial_condition import (
    ConstantInitialCondition,
    ContinuousInitialCondition,
    DiscreteInitialCondition,
    GaussianInitialCondition,
    InitialCondition,
    vectorize_ic_function,
)
from .initial_value_problem import InitialValueProblem
from .mesh import CoordinateSystem, Mesh
from .operator import Operator, discretize_time_domain
from .solution import Solution

__version__ = "0.1.0"
