"""Fields, dimensions and field components (pyfds/fields.py API) on a GB300.

``Field.simulate`` / ``sim_step`` of the staggered fields run on the GPU through
``pyfds_gb300._engine``: one fused CUDA launch per step, boundaries and outputs
handled inside it. The geometry API (dimensions, index/position conversion,
region factories), material lookup and the DIA operator builders keep the
reference's behaviour; the operator builders return scipy matrices for
inspection, the time stepping itself is matrix-free.
"""
import logging as lo

import numpy as np

from . import regions as reg

logger = lo.getLogger('pyfds')


class Field:
    """Base class for all fields (pyfds/fields.py:9-127)."""

    def __init__(self):
        self.material_regions = []
        self.step = 0
        self.matrices_assembled = False
        self.t = None

    @property
    def num_points(self):
        raise NotImplementedError

    def get_index(self, position):
        raise NotImplementedError

    def material_vector(self, mat_parameter):
        """Per-point value of one material parameter; later material regions
        overwrite earlier ones (pyfds/fields.py:34-57)."""
        param_found = False
        mat_vector = np.zeros(self.num_points)
        for mat_reg in self.material_regions:
            for mat in mat_reg.materials:
                if hasattr(mat, mat_parameter):
                    mat_vector[_as_index(mat_reg.region.indices)] = getattr(mat, mat_parameter)
                    param_found = True
        if not param_found:
            raise KeyError('Material parameter {} not found in set materials.')
        return mat_vector

    def assemble_matrices(self):
        raise NotImplementedError

    def sim_step(self):
        raise NotImplementedError

    def _fused_path(self):
        """True when ``sim_step`` is this package's own GPU step (not overridden by a
        subclass), so that ``simulate`` may run many steps per call."""
        own = getattr(type(self), '_gpu_sim_step', None)
        return own is not None and type(self).sim_step is own

    def simulate(self, num_steps=None):
        """Run ``num_steps`` steps (``self.t.samples`` by default), pyfds/fields.py:67-95.

        A subclass that overrides ``sim_step`` is stepped one ``sim_step`` at a
        time, as in the reference; otherwise the steps run as one GPU call per
        chunk (one chunk unless progress is logged, which is reported per chunk).
        """
        if not num_steps:
            num_steps = self.t.samples
            progress_logger = ProgressLogger(num_steps)
        else:
            progress_logger = None

        if not self.matrices_assembled:
            self.assemble_matrices()
            logger.info('Matrices created.')

        logger.info('Starting simulation of {} steps.'.format(num_steps))

        start_step = self.step
        if self._fused_path():
            chunks = [num_steps]
            if progress_logger and logger.isEnabledFor(lo.INFO):
                edges = sorted({int(round(num_steps * k / 20)) for k in range(21)})
                chunks = [b - a for a, b in zip(edges[:-1], edges[1:]) if b > a]
            for n in chunks:
                # tables are reused while the boundaries, outputs and tiling are
                # unchanged (a fingerprint with content checksums) and cover the steps
                diverged = self._engine().run(self.step, n, cache_tables=True)
                if progress_logger:
                    progress_logger.log(self.step + n - 1)
                self.step += n
                if diverged:
                    self._engine().report_nonfinite(self.step)
        else:
            while self.step < start_step + num_steps:
                self.sim_step()
                if progress_logger:
                    progress_logger.log(self.step)
                self.step += 1

        logger.info('Simulation of {} steps completed.'.format(num_steps))

    def get_point_region(self, position, name=''):
        return reg.PointRegion([self.get_index(position)], position, name=name)

    def add_material_region(self, *args, **kwargs):
        new_material_region = reg.MaterialRegion(*args, **kwargs)
        self.material_regions.append(new_material_region)
        logger.info('Material region {} added.'.format(new_material_region.region.name))

    def reset(self):
        """Zero every component but keep boundaries and outputs (pyfds/fields.py:121-127)."""
        for name in dir(self):
            if isinstance(getattr(self, name), FieldComponent):
                getattr(self, name).values = np.zeros_like(getattr(self, name).values)
        self.step = 0


def _as_index(indices):
    if isinstance(indices, np.ndarray):
        return indices
    return np.asarray(indices, dtype=np.int64)


def _first_derivative(n, factors, variant, step):
    import scipy.sparse as sp
    if factors is None:
        factors = np.array(1).repeat(n)
    if variant == 'forward':
        return sp.dia_matrix((np.array([-factors, factors]), [0, step]), shape=(n, n))
    elif variant == 'central':
        return sp.dia_matrix((np.array([-factors / 2, factors / 2]), [-step, step]), shape=(n, n))
    elif variant == 'backward':
        return sp.dia_matrix((np.array([-factors, factors]), [-step, 0]), shape=(n, n))
    raise ValueError('Unknown difference quotient variant {}.'.format(variant))


def _second_derivative(n, factors, step):
    import scipy.sparse as sp
    if factors is None:
        factors = np.array(1).repeat(n)
    return sp.dia_matrix((np.array([factors, -2 * factors, factors]), [-step, 0, step]),
                         shape=(n, n))


class Field1D(Field):
    """One-dimensional field (pyfds/fields.py:130-241)."""

    def __init__(self, x_samples, x_delta, t_samples, t_delta, material):
        super().__init__()
        self.x = Dimension(x_samples, x_delta)
        self.t = Dimension(t_samples, t_delta)
        self.add_material_region(self.get_line_region((0, max(self.x.vector)), name='main'),
                                 material)

    @property
    def num_points(self):
        return self.x.samples

    @property
    def _nx(self):
        return self.x.samples

    @property
    def _ny(self):
        return 1

    def d_x(self, factors=None, variant='forward'):
        """DIA matrix of the first x derivative times per-point factors."""
        return _first_derivative(self.num_points, factors, variant, 1)

    def d_x2(self, factors=None):
        """DIA matrix of the second x derivative times per-point factors."""
        return _second_derivative(self.num_points, factors, 1)

    def get_index(self, position):
        return self.x.get_index(position)

    def get_position(self, index):
        return self.x.vector[index]

    def get_line_region(self, position, name=''):
        """Inclusive line (start, end) in x coordinates."""
        return reg.LineRegion(list(range(self.get_index(position[0]),
                                         self.get_index(position[1]) + 1)),
                              position, name=name)


class Field2D(Field):
    """Two-dimensional field with flat index ``x + y * x.samples`` (pyfds/fields.py:244-533)."""

    def __init__(self, x_samples, x_delta, y_samples, y_delta, t_samples, t_delta, material):
        super().__init__()
        self.x = Dimension(x_samples, x_delta)
        self.y = Dimension(y_samples, y_delta)
        self.t = Dimension(t_samples, t_delta)
        self.add_material_region(self.get_rect_region(
            (0, 0, max(self.x.vector), max(self.y.vector)), name='main'), material)

    @property
    def num_points(self):
        return self.x.samples * self.y.samples

    @property
    def _nx(self):
        return self.x.samples

    @property
    def _ny(self):
        return self.y.samples

    def d_x(self, factors=None, variant='forward'):
        return _first_derivative(self.num_points, factors, variant, 1)

    def d_y(self, factors=None, variant='forward'):
        return _first_derivative(self.num_points, factors, variant, self.x.samples)

    def d_x2(self, factors=None):
        return _second_derivative(self.num_points, factors, 1)

    def d_y2(self, factors=None):
        return _second_derivative(self.num_points, factors, self.x.samples)

    def get_index(self, position):
        return self.x.get_index(position[0]) + self.y.get_index(position[1]) * self.x.samples

    def get_position(self, index):
        return self.x.vector[index % self.x.samples], self.y.vector[int(index / self.x.samples)]

    def _positions(self, idx):
        idx = np.asarray(idx)
        return (self.x.vector[idx % self.x.samples],
                self.y.vector[(idx / self.x.samples).astype(np.int64)])

    def get_line_region(self, position, name=''):
        """Line of points from (start_x, start_y) to (end_x, end_y), inclusive."""
        nx = self.x.samples
        start_idx = self.get_index(position[:2])
        end_idx = self.get_index(position[2:])
        x_diff = start_idx % nx - end_idx % nx
        y_diff = int(start_idx / nx) - int(end_idx / nx)
        num_points = max(np.abs([x_diff, y_diff]))
        point_indices = []
        for ii in range(num_points + 1):
            x_position = start_idx % nx - np.round(ii / num_points * x_diff)
            y_position = int(start_idx / nx) - np.round(ii / num_points * y_diff)
            point_indices.append(int(x_position + nx * y_position))
        return reg.LineRegion(point_indices, position, name=name)

    def get_rect_region(self, position, name=''):
        """Rectangle (origin_x, origin_y, size_x, size_y), inclusive; indices ordered
        x-major then y, as the reference lists them."""
        x_start = self.x.get_index(position[0])
        y_start = self.y.get_index(position[1])
        x_end = self.x.get_index(position[0] + position[2])
        y_end = self.y.get_index(position[1] + position[3])
        x_start, x_end = min(x_start, x_end), max(x_start, x_end)
        y_start, y_end = min(y_start, y_end), max(y_start, y_end)
        xs = np.arange(x_start, x_end + 1, dtype=np.int64)
        ys = np.arange(y_start, y_end + 1, dtype=np.int64)
        indices = (xs[:, None] + ys[None, :] * self.x.samples).reshape(-1)
        return reg.RectRegion(indices, position, name)

    def get_tri_region(self, position, name=''):
        """Points inside the triangle (p0x, p0y, p1x, p1y, p2x, p2y), inclusive."""
        if (position[2] - position[0]) * (position[5] - position[1]) - \
                (position[3] - position[1]) * (position[4] - position[0]) > 0:
            position = (position[0], position[1], position[4], position[5],
                        position[2], position[3])
        p = position
        corner = (self.get_index(p[:2]), self.get_index(p[2:4]), self.get_index(p[4:]))
        ii = np.arange(min(corner), max(corner) + 1)
        px, py = self._positions(ii)
        e01 = (px - p[0]) * (p[3] - p[1]) - (py - p[1]) * (p[2] - p[0])
        e12 = (px - p[2]) * (p[5] - p[3]) - (py - p[3]) * (p[4] - p[2])
        e20 = (px - p[4]) * (p[1] - p[5]) - (py - p[5]) * (p[0] - p[4])
        inside = (e01 >= 0) & (e12 >= 0) & (e20 >= 0)
        return reg.TriRegion(ii[inside].tolist(), position, name)

    def get_ellipse_region(self, centre, radii, name=''):
        """Points inside the ellipse with the given centre and half axes."""
        if np.isscalar(radii):
            radii = (radii, radii)
        lo_i = self.get_index((centre[0], centre[1] - radii[1]))
        hi_i = self.get_index((centre[0], centre[1] + radii[1]))
        ii = np.arange(lo_i, hi_i)
        px, py = self._positions(ii)
        inside = (centre[0] - px) ** 2 / radii[0] ** 2 + (centre[1] - py) ** 2 / radii[1] ** 2 <= 1
        return reg.EllipseRegion(ii[inside].tolist(), centre, radii, name)


class Dimension:
    """A space or time axis (pyfds/fields.py:536-571)."""

    def __init__(self, samples, increment):
        self.samples = int(samples)
        self.increment = increment
        self.snap_radius = np.finfo(float).eps * 10

    @property
    def vector(self):
        return np.arange(start=0, stop=self.samples) * self.increment

    def get_index(self, value):
        """Index of the sample within an absolute 10-eps snap radius of ``value``."""
        index, = np.where(np.abs(self.vector - value) <= self.snap_radius)
        assert len(index) < 2, "Multiple points found within snap radius of given value."
        assert len(index) > 0, "No point found within snap radius of given value."
        return int(index[0])


class FieldComponent:
    """One component of a field (pyfds/fields.py:574-633).

    ``values`` is a float64 numpy array as in the reference. Inside a field that has
    run on the GPU the device copy is authoritative; reading ``values`` copies it to
    the host, and the host copy (which the caller may modify in place) is uploaded
    again before the next launch. Assigning ``values`` replaces the state.
    """

    def __init__(self, num_points):
        self._values = np.zeros(num_points)
        self._engine = None
        self._name = None
        self._where = "host"  # host | device | both
        self.boundaries = []
        self.outputs = []

    def _attach(self, engine, name):
        self._engine = engine
        self._name = name

    @property
    def values(self):
        if self._where == "device":
            self._values = self._engine.download(self._name)
        if self._engine is not None:
            self._where = "host"
        return self._values

    @values.setter
    def values(self, value):
        self._values = value
        self._where = "host"

    def apply_bounds(self, step):
        """Apply the boundaries to ``values`` on the host (stand-alone components;
        a field applies them on the GPU inside its time step)."""
        for bound in self.boundaries:
            idx = _as_index(bound.region.indices)
            self.values[idx] = bound.apply(self.values[idx], step=step)

    def write_outputs(self):
        """Record ``values`` at every output point on the host (stand-alone components)."""
        vals = self.values
        for output in self.outputs:
            if not output.signals:
                output.signals = [[vals[index]] for index in output.region.indices]
            else:
                for index, signal in zip(output.region.indices, output.signals):
                    signal.append(vals[index])

    def add_boundary(self, *args, **kwargs):
        new_bound = reg.Boundary(*args, **kwargs)
        self.boundaries.append(new_bound)
        logger.info('Boundary {} added.'.format(new_bound.region.name))

    def add_output(self, *args, **kwargs):
        new_output = reg.Output(*args, **kwargs)
        self.outputs.append(new_output)
        logger.info('Output region {} added.'.format(new_output.region.name))

    def __getstate__(self):
        st = self.__dict__.copy()
        st["_values"] = np.array(self.values, dtype=np.float64, copy=True)
        st["_engine"] = None
        st["_where"] = "host"
        return st


class ProgressLogger:
    """Logs progress in percent at a fixed increment (pyfds/fields.py:636-668)."""

    def __init__(self, num_steps, log_increment=5, logger_instance=None):
        self.num_steps = num_steps
        self.log_increment = log_increment
        self.logger = logger_instance if logger_instance else logger
        self._last_message_at = None

    def log(self, current_step):
        pct = int(current_step / self.num_steps * 100)
        if int(current_step / self.num_steps * 100 % self.log_increment) == 0 and \
                self._last_message_at != pct:
            self.logger.info('Simulating. {} % completed.'.format(pct))
            self._last_message_at = pct
