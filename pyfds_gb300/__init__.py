"""pyfds_gb300: GB300-native time stepping for pyfds fields.

The public names match the reference package (``import pyfds_gb300 as fds`` in place
of ``import pyfds as fds``): fields, materials, boundaries, outputs and material
regions keep their constructors and attributes, while ``simulate()`` and
``sim_step()`` run as fused CUDA kernels on the GPU (see ``include/fds_capi.h``).
"""
from . import fields, gfx, regions  # noqa: F401
from .acoustic_flow import *  # noqa: F401,F403
from .acoustics import *  # noqa: F401,F403
from .coupled_fields import *  # noqa: F401,F403
from .coupling import *  # noqa: F401,F403
from .gfx import *  # noqa: F401,F403
from .nonlinear_acoustics import *  # noqa: F401,F403
from .regions import *  # noqa: F401,F403
from .thermal import *  # noqa: F401,F403

__version__ = "0.1.0"
