"""fastode_gb300: the Rosenbrock integrator of fastode (davidfillmore/
Fast-ODE-Atmospheric-Chem) rebuilt as hand-written sm_103a CUDA for GB300.

Drop-in surface (same names, arguments and results as the reference's
fastode package): ``Algorithm``, ``Memory``, ``Counts``, ``ROS3``, ``RODAS3``,
``Mechanism``, ``ChemSystem``, ``quantize``. Batched device-resident driver:
``Batch``. Everything numerical runs on the GPU; the package has no CPU
integrator.
"""
from .tableaus import ROS3, RODAS3, Tableau
from .counts import Counts
from .chem import Mechanism, ChemSystem
from .solvers import Algorithm, BackwardEuler, Memory, RestartingLoop, quantize

__all__ = ["ROS3", "RODAS3", "Tableau", "Counts", "Mechanism", "ChemSystem", "Algorithm", "BackwardEuler", "RestartingLoop", "Memory",
           "quantize"]
