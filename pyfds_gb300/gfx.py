"""Headless field snapshots in place of the reference's live animation
(pyfds/gfx.py:14-406).

The reference animates a component with matplotlib in a second process and can
encode the frames with ffmpeg. Neither exists where this package runs (no graphics
stack), so ``Animator1D`` / ``Animator2D`` keep the constructor, its checks and
``field_as_matrix`` and turn ``start_simulation`` into a headless recorder: the
field advances ``steps_per_frame`` steps per chunk on the GPU and each frame (the
observed component) is copied device to device into one frame tensor, with no host
round trip per frame. ``save_video=True`` writes the frames and their times to an
``.npz`` file instead of a video. Plot windows (``show_setup``, ``plot_region``) are
not available.
"""
import numpy as np

from . import fields as fld
from ._engine import require_cuda

__all__ = ['Animator', 'Animator1D', 'Animator2D']


class Animator:
    """Frame recorder of one field component (pyfds/gfx.py:14-127, headless)."""

    def __init__(self, field, observed_component=None, steps_per_frame=10, scale=1,
                 frame_delay=1e-2, save_video=False, video_file_name='pyfds_vid.mp4'):
        self.field = field
        self.field_components = {name: getattr(self.field, name) for name in dir(self.field)
                                 if isinstance(getattr(self.field, name), fld.FieldComponent)}
        if observed_component:
            if observed_component in self.field_components.keys():
                self.observed_component = observed_component
            else:
                raise KeyError('Field component {} not found in given field.'
                               .format(observed_component))
        else:
            self.observed_component = list(self.field_components.keys())[0]
        self.steps_per_frame = int(steps_per_frame)
        if isinstance(scale, (list, tuple, np.ndarray)) and len(scale) == 2:
            self.scale = scale
        elif isinstance(scale, (float, int)):
            self.scale = (-scale, scale)
        else:
            raise ValueError('Scale must either be scalar or a 2 element vector.')
        self.frame_delay = frame_delay
        self.save_video = save_video
        self.video_file_name = video_file_name
        self.frames = None       # device tensor [frames, points] (float64)
        self.frame_times = []    # simulated time of each frame

    def _frame_shape(self):
        return (self.field.num_points,)

    def start_simulation(self):
        """Run ``int(t.samples / steps_per_frame)`` chunks of ``steps_per_frame`` steps
        (the reference's ``_sim_function``, pyfds/gfx.py:72-86) and record the observed
        component after each chunk. Returns the frame tensor."""
        torch = require_cuda()
        f = self.field
        n_frames = int(f.t.samples / self.steps_per_frame)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.frames = torch.empty((n_frames,) + self._frame_shape(), dtype=torch.float64,
                                  device=dev)
        self.frame_times = []
        for k in range(n_frames):
            f.simulate(self.steps_per_frame)
            self.frames[k].view(-1).copy_(self._device_values())
            self.frame_times.append(float(f.t.vector[f.step - 1]))
        if self.save_video:
            name = self.video_file_name
            if not name.endswith('.npz'):
                name = name.rsplit('.', 1)[0] + '.npz'
            np.savez_compressed(name, frames=self.frames.cpu().numpy(),
                                times=np.asarray(self.frame_times),
                                component=self.observed_component)
        return self.frames

    def _device_values(self):
        """The observed component as a float64 device tensor (no host copy)."""
        f = self.field
        eng = f._engine() if hasattr(f, '_engine') else None
        name = self.observed_component
        comp = getattr(f, name)
        if eng is None or name not in eng.buffers or getattr(comp, '_where', 'host') == 'host':
            torch = require_cuda()
            return torch.as_tensor(np.asarray(comp.values, dtype=np.float64), device='cuda')
        return eng.device_values(name)

    def show_setup(self, halt=True):
        raise NotImplementedError('plot windows need a graphics stack; this package records '
                                  'frames headless (start_simulation)')

    def plot_region(self, region):
        raise NotImplementedError('plot windows need a graphics stack')


class Animator1D(Animator):
    """Frames of a 1-D field (pyfds/gfx.py:129-242, headless)."""


class Animator2D(Animator):
    """Frames of a 2-D field as [y][x] matrices (pyfds/gfx.py:244-404, headless)."""

    def _frame_shape(self):
        return (self.field.y.samples, self.field.x.samples)

    def field_as_matrix(self, component=None):
        """A field component (the observed one by default) as a [y][x] matrix
        (pyfds/gfx.py:301-314)."""
        if component is None:
            component = getattr(self.field, self.observed_component).values
        return np.reshape(component, (self.field.y.samples, self.field.x.samples))


# SI prefixes of the axis labels, by factor (the standard table, as pyfds/gfx.py:422-440
# uses it: yocto to yotta in steps of 10^3)
prefixes = {float('1e%d' % (3 * k)): p
            for k, p in zip(range(-8, 9), ('y', 'z', 'a', 'f', 'p', 'n', 'µ', 'm', '',
                                           'k', 'M', 'G', 'T', 'P', 'E', 'Z', 'Y'))}


def get_prefix(value):
    """Metric prefix for an axis whose largest value is ``value`` (pyfds/gfx.py:406-419):
    the smallest factor with ``value / factor < 1000``, the largest factor if none
    qualifies (including NaN). Returns ``(prefix, factor)``."""
    factors = sorted(prefixes)
    factor = next((f for f in factors if value / f < 1e3), factors[-1])
    return prefixes[factor], factor
