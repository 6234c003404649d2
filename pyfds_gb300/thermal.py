"""Thermal fields (pyfds/thermal.py API), time-stepped on the GPU."""
import logging as lo

import numpy as np

from . import _capi
from . import fields as fld
from ._stag import StagField

__all__ = [
    'Thermal1D', 'Thermal2D', 'Thermal3DAxi', 'ThermalMaterial'
]

logger = lo.getLogger('pyfds')


class Thermal1D(StagField, fld.Field1D):
    """One-dimensional thermal field: temperature and heat flux (pyfds/thermal.py:12-51)."""

    _stag_family = _capi.FAMILY_THERMAL
    _stag_components = ('temperature', 'heat_flux')

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        fld.Field1D.__init__(self, *args, **kwargs)
        self._init_gpu(precision, exact, tile)
        self.temperature = fld.FieldComponent(self.num_points)
        self.heat_flux = fld.FieldComponent(self.num_points)

    def _coefficients(self):
        # factors of pyfds/thermal.py:29-38, same expression order
        dt, dx = self.t.increment, self.x.increment
        rho = self.material_vector('density')
        cp = self.material_vector('heat_capacity')
        kx = self.material_vector('thermal_conductivity_x')
        return {"kx": dt / dx / rho / cp, "bx": 1 / dx * kx}, 0

    @property
    def a_t_q(self):
        return self._operator('a_t_q', lambda: self.d_x(
            factors=self.t.increment / self.x.increment / self.material_vector('density')
            / self.material_vector('heat_capacity')))

    @property
    def a_q_t(self):
        return self._operator('a_q_t', lambda: self.d_x(
            factors=1 / self.x.increment * self.material_vector('thermal_conductivity_x'),
            variant='backward'))


class Thermal2D(StagField, fld.Field2D):
    """Two-dimensional thermal field (pyfds/thermal.py:54-107)."""

    _stag_family = _capi.FAMILY_THERMAL
    _stag_components = ('temperature', 'heat_flux_x', 'heat_flux_y')

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        fld.Field2D.__init__(self, *args, **kwargs)
        self._init_gpu(precision, exact, tile)
        self.temperature = fld.FieldComponent(self.num_points)
        self.heat_flux_x = fld.FieldComponent(self.num_points)
        self.heat_flux_y = fld.FieldComponent(self.num_points)

    def _radii(self):
        return None

    def _coefficients(self):
        # factors of pyfds/thermal.py:75-90 (and :144-159 for the axisymmetric field)
        dt, dx, dy = self.t.increment, self.x.increment, self.y.increment
        rho = self.material_vector('density')
        cp = self.material_vector('heat_capacity')
        kx = self.material_vector('thermal_conductivity_x')
        ky = self.material_vector('thermal_conductivity_y')
        hx = dt / dx / rho / cp
        flags = _capi.FLAG_HAS_V
        coefs = {"ky": dt / dy / rho / cp, "bx": 1 / dx * kx, "by": 1 / dy * ky}
        r = self._radii()
        if r is not None:
            flags |= _capi.FLAG_AXI
            coefs["rx"] = self.x.vector + dx / 2
            if self.exact:
                hx = hx / r
        coefs["kx"] = hx
        return coefs, flags

    @property
    def a_t_qx(self):
        r = self._radii()
        return self._operator('a_t_qx', lambda: self.d_x(
            factors=self.t.increment / self.x.increment / self.material_vector('density')
            / self.material_vector('heat_capacity') / (1 if r is None else r)))

    @property
    def a_t_qy(self):
        return self._operator('a_t_qy', lambda: self.d_y(
            factors=self.t.increment / self.y.increment / self.material_vector('density')
            / self.material_vector('heat_capacity')))

    @property
    def a_qx_t(self):
        return self._operator('a_qx_t', lambda: self.d_x(
            factors=1 / self.x.increment * self.material_vector('thermal_conductivity_x'),
            variant='backward'))

    @property
    def a_qy_t(self):
        return self._operator('a_qy_t', lambda: self.d_y(
            factors=1 / self.y.increment * self.material_vector('thermal_conductivity_y'),
            variant='backward'))


class Thermal3DAxi(Thermal2D):
    """Axisymmetric thermal field; x is the radius, y the axis (pyfds/thermal.py:110-176)."""

    def _radii(self):
        """Radius of each heat-flux point, x + dx/2 (pyfds/thermal.py:132-142)."""
        return np.tile(self.x.vector, self.y.samples) + self.x.increment / 2


class ThermalMaterial:
    """Thermal material parameters; conductivity scalar or (x, y) (pyfds/thermal.py:179-211)."""

    def __init__(self, heat_capacity, density, thermal_conductivity):
        self.heat_capacity = heat_capacity
        self.density = density
        self.thermal_conductivity_x = None
        self.thermal_conductivity_y = None
        self.thermal_conductivity = thermal_conductivity

    @property
    def thermal_conductivity(self):
        return self.thermal_conductivity_x, self.thermal_conductivity_y

    @thermal_conductivity.setter
    def thermal_conductivity(self, value):
        if isinstance(value, (list, tuple, np.ndarray)) and len(value) == 2:
            self.thermal_conductivity_x = value[0]
            self.thermal_conductivity_y = value[1]
        elif isinstance(value, (float, int)):
            self.thermal_conductivity_x = value
            self.thermal_conductivity_y = value
        else:
            raise ValueError('Thermal conductivity must either be scalar or a 2 element vector.')
