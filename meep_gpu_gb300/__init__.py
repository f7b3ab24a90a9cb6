"""meep_gpu_gb300: a GB300-native FDTD stepping engine behind the ``meep_gpu`` driver API.

``FdtdDriver`` takes the same configuration calls as the reference's driver
(``meep_gpu/driver.py``) and steps the simulation with two fused sm_103a kernels per
step in ``libmeepgb.so`` (C ABI: ``include/meepgb.h``). There is no CPU stepping path.
"""

from .conductivity import AbsorberLayer
from .dft import DFTMonitor, FluxDftData, FluxMonitor, FluxPlaneDft
from .dispersion import DRUDE, LORENTZ, Susceptibility
from .driver import FdtdCancelled, FdtdDivergence, FdtdDriver
from .grid import Grid, Mirror, Unsupported
from .pml import PML

__all__ = ["FdtdDriver", "FdtdCancelled", "FdtdDivergence", "Susceptibility", "LORENTZ",
           "DRUDE", "Grid", "PML", "FluxMonitor", "DFTMonitor", "Unsupported", "AbsorberLayer",
           "FluxDftData", "FluxPlaneDft", "Mirror"]
__version__ = "0.1.0"
