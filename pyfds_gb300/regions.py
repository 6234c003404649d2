"""Regions, boundaries, outputs and material regions (pyfds/regions.py API).

These are host-side descriptions. A field compiles its components' boundaries
and outputs into device tables (``pyfds_gb300._tables``) before each launch, so the
objects keep the reference's mutable, list-based interface: append to
``component.boundaries`` / ``component.outputs``, change ``boundary.value`` or
``boundary.additive`` between runs.
"""
import numpy as np

__all__ = [
    'Boundary', 'MaterialRegion', 'Output',
]


class Region:
    """Point indices plus metadata (pyfds/regions.py:8-24)."""

    def __init__(self, indices, name=''):
        self.indices = indices
        self.name = name


class PointRegion(Region):
    """Region given by individual points (pyfds/regions.py:27-40)."""

    def __init__(self, indices, coordinates, name=''):
        super().__init__(indices, name)
        self.point_coordinates = coordinates


class LineRegion(Region):
    """Region along a line of points (pyfds/regions.py:43-56)."""

    def __init__(self, indices, coordinates, name=''):
        super().__init__(indices, name)
        self.line_coordinates = coordinates


class RectRegion(Region):
    """Rectangular block of points (pyfds/regions.py:59-72)."""

    def __init__(self, indices, coordinates, name=''):
        super().__init__(indices, name)
        self.rect_coordinates = coordinates


class TriRegion(Region):
    """Triangular set of points (pyfds/regions.py:75-88)."""

    def __init__(self, indices, coordinates, name=''):
        super().__init__(indices, name)
        self.tri_coordinates = coordinates


class EllipseRegion(Region):
    """Elliptic set of points (pyfds/regions.py:91-103)."""

    def __init__(self, indices, centre, radii, name=''):
        super().__init__(indices, name)
        self.centre = centre
        self.radii = radii


class Boundary:
    """Values written to a component every step: sources and fixed values
    (pyfds/regions.py:106-145).

    ``value`` is a scalar, a signal (``value[step]`` is broadcast to every point;
    a 2-D array gives one row per step), or a list with one signal per point.
    ``additive`` multiplies the old value: ``new = additive * old + value``.
    """

    def __init__(self, region, value=0, additive=False):
        self.region = region
        self.value = value
        self.additive = additive

    def apply(self, old_values, step):
        """Host-side evaluation of the boundary for one step (used by
        ``FieldComponent.apply_bounds`` on a stand-alone component; fields apply
        their boundaries on the GPU inside the time-step kernel)."""
        if np.ndim(self.value) == 0:
            return self.additive * old_values + self.value
        if isinstance(self.value, np.ndarray):
            return self.additive * old_values + self.value[step]
        return [self.additive * old_values[k] + sig[step] for k, sig in enumerate(self.value)]


class Output:
    """Values recorded from a component every step (pyfds/regions.py:148-165).

    ``signals[k]`` is the list of samples of the k-th point of the region. The
    samples a GPU call records arrive as a float64 block on the host; lists that
    exist grow at once, new ones are built when ``signals`` is next read (building
    Python lists of millions of samples costs more than the call's copy; a caller
    that never reads them does not pay for it).
    """

    def __init__(self, region):
        self.region = region
        self._signals = []
        self._pending = []  # host blocks [points, steps] not yet in the lists

    @property
    def signals(self):
        if self._pending:
            pending, self._pending = self._pending, []
            for rows in pending:
                if not self._signals:
                    self._signals = [r.tolist() for r in rows]
                else:
                    for sig, r in zip(self._signals[:len(rows)], rows):
                        sig.extend(r.tolist())
        return self._signals

    @signals.setter
    def signals(self, value):
        self._pending = []
        self._signals = value

    def _record(self, rows):
        """Append the samples of a GPU call: one row per point, as in ``signals``.
        Lists that exist grow in place at once (a caller may hold them); new ones
        are built when ``signals`` is read."""
        if self._signals:
            for sig, r in zip(self._signals[:len(rows)], rows):
                sig.extend(r.tolist())
        else:
            self._pending.append(rows)

    @property
    def mean_signal(self):
        """Mean over all points of the region, per step."""
        return np.mean(np.asarray(self.signals), axis=0)


class MaterialRegion:
    """Material(s) assigned to a region (pyfds/regions.py:168-180)."""

    def __init__(self, region, material):
        self.region = region
        self.materials = [material]
