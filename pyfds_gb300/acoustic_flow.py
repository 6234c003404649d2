"""Acoustic field in a moving medium (pyfds/acoustic_flow.py:13-57).

``AcousticFlow2D`` is ``Acoustic2D`` plus a flow along x: after every step, each row
y whose shift period ``flow_t_deltas[y] = int(dx / flow[y] / dt)`` divides the step
moves one cell in +x in pressure and both velocities (its first cell becomes 0).
On the GPU the shift is a kernel between the pressure update and the next step's
pressure boundaries (``FDS_FLAG_FLOW`` in include/fds_capi.h), so ``simulate()`` still
runs every step of a chunk in one library call.
"""
import logging as lo
import warnings as wn

import numpy as np

from . import _capi
from .acoustics import Acoustic2D

__all__ = [
    'AcousticFlow2D',
]

logger = lo.getLogger('pyfds')


class AcousticFlow2D(Acoustic2D):
    """Two-dimensional acoustic field with a medium moving along x
    (pyfds/acoustic_flow.py:13-47)."""

    def __init__(self, flow, *args, **kwargs):
        """Args:
            flow: flow velocity along x (scalar, or a vector of length y_samples).
            *args, **kwargs: the Acoustic2D constructor arguments.
        """
        super().__init__(*args, **kwargs)
        if isinstance(flow, (list, np.ndarray)) and len(flow) == self.y.samples:
            self.flow = np.asarray(flow)
        elif isinstance(flow, (float, int)):
            self.flow = np.ones(self.y.samples) * flow
        else:
            raise ValueError('Flow must either be scalar or a vector with length of y_samples.')
        # step period of the shift per row (same expression as the reference; a row at
        # rest divides by zero and gets a saturated period: shifted at step 0 only)
        with np.errstate(divide='ignore', invalid='ignore'):
            self.flow_t_deltas = (self.x.increment / self.flow / self.t.increment).astype(int)
        if np.any(self.flow_t_deltas == 1) or np.any(self.flow_t_deltas == 0):
            wn.warn('Flow velocity may be to high. Consider reducing t_delta.', stacklevel=2)
            logger.warning('Flow velocity may be to high. Consider reducing t_delta.')

    def _stag_flags(self):
        return super()._stag_flags() | _capi.FLAG_FLOW

    def _flow_periods(self):
        return np.asarray(self.flow_t_deltas, dtype=np.int64)

    def sim_step(self):
        """Simulate one step: the Acoustic2D step, then the flow shift of this step
        (pyfds/acoustic_flow.py:44-47), in one library call."""
        if not self.matrices_assembled:
            self.assemble_matrices()
        if self._engine().run(self.step, 1, cache_tables=True):
            self._engine().report_nonfinite(self.step + 1)

    _gpu_sim_step = sim_step

    def apply_flow(self):
        """The flow shift of the current step alone, on the device state
        (pyfds/acoustic_flow.py:49-57)."""
        if not self.matrices_assembled:
            self.assemble_matrices()
        self._engine().flow_shift(self.step)
