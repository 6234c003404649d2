"""Linear acoustic fields (pyfds/acoustics.py API), time-stepped on the GPU."""
import numpy as np

from . import _capi
from . import fields as fld
from ._stag import StagField, summed_absorption

__all__ = [
    'Acoustic1D', 'Acoustic2D', 'Acoustic3DAxi', 'AcousticMaterial',
]


class _AcousticBase(StagField):
    _stag_family = _capi.FAMILY_ACOUSTIC

    def is_stable(self):
        """CFL check with 1 % headroom, absorption not accounted for
        (pyfds/acoustics.py:54-63, 130-139, 227-236)."""
        inc = self.x.increment if not hasattr(self, 'y') else min(self.x.increment,
                                                                  self.y.increment)
        return np.all(self.material_vector('sound_velocity') < 0.99 * inc / self.t.increment)


class Acoustic1D(_AcousticBase, fld.Field1D):
    """One-dimensional acoustic field: pressure and velocity (pyfds/acoustics.py:9-63)."""

    _stag_components = ('pressure', 'velocity')

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        fld.Field1D.__init__(self, *args, **kwargs)
        self._init_gpu(precision, exact, tile)
        self.pressure = fld.FieldComponent(self.num_points)
        self.velocity = fld.FieldComponent(self.num_points)

    def _coefficients(self):
        # factors of pyfds/acoustics.py:27-38, same expression order
        dt, dx = self.t.increment, self.x.increment
        c = self.material_vector('sound_velocity')
        rho = self.material_vector('density')
        mu = self.material_vector('absorption_coef')
        coefs = {"kx": dt / dx * c ** 2 * rho, "bx": dt / dx / rho}
        flags = 0
        a = dt / dx ** 2 * mu / rho
        if np.any(a != 0):
            flags |= _capi.FLAG_ABSORB
            coefs.update(summed_absorption(self.x.samples, False, a, None))
        return coefs, flags

    @property
    def a_p_v(self):
        return self._operator('a_p_v', lambda: self.d_x(
            factors=self.t.increment / self.x.increment * self.material_vector('sound_velocity')
            ** 2 * self.material_vector('density')))

    @property
    def a_v_p(self):
        return self._operator('a_v_p', lambda: self.d_x(
            factors=self.t.increment / self.x.increment / self.material_vector('density'),
            variant='backward'))

    @property
    def a_v_v(self):
        return self._operator('a_v_v', lambda: self.d_x2(
            factors=self.t.increment / self.x.increment ** 2
            * self.material_vector('absorption_coef') / self.material_vector('density')))


class Acoustic2D(_AcousticBase, fld.Field2D):
    """Two-dimensional acoustic field (pyfds/acoustics.py:66-139)."""

    _stag_components = ('pressure', 'velocity_x', 'velocity_y')

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        fld.Field2D.__init__(self, *args, **kwargs)
        self._init_gpu(precision, exact, tile)
        self.pressure = fld.FieldComponent(self.num_points)
        self.velocity_x = fld.FieldComponent(self.num_points)
        self.velocity_y = fld.FieldComponent(self.num_points)

    def _coefficients(self):
        # factors of pyfds/acoustics.py:89-109, same expression order
        dt, dx, dy = self.t.increment, self.x.increment, self.y.increment
        c = self.material_vector('sound_velocity')
        rho = self.material_vector('density')
        mu = self.material_vector('absorption_coef')
        coefs = {"kx": dt / dx * c ** 2 * rho, "ky": dt / dy * c ** 2 * rho,
                 "bx": dt / dx / rho, "by": dt / dy / rho}
        flags = _capi.FLAG_HAS_V
        ax = dt / dx ** 2 * mu / rho
        ay = dt / dy ** 2 * mu / rho
        if np.any(ax != 0) or np.any(ay != 0):
            flags |= _capi.FLAG_ABSORB
            coefs.update(summed_absorption(self.x.samples, True, ax, ay))
        return coefs, flags

    def _absorption_operator(self):
        return (self.d_x2(factors=(self.t.increment / self.x.increment ** 2
                                   * self.material_vector('absorption_coef')
                                   / self.material_vector('density')))
                + self.d_y2(factors=(self.t.increment / self.y.increment ** 2
                                     * self.material_vector('absorption_coef')
                                     / self.material_vector('density')))).todia()

    @property
    def a_p_vx(self):
        return self._operator('a_p_vx', lambda: self.d_x(
            factors=self.t.increment / self.x.increment * self.material_vector('sound_velocity')
            ** 2 * self.material_vector('density')))

    @property
    def a_p_vy(self):
        return self._operator('a_p_vy', lambda: self.d_y(
            factors=self.t.increment / self.y.increment * self.material_vector('sound_velocity')
            ** 2 * self.material_vector('density')))

    @property
    def a_vx_p(self):
        return self._operator('a_vx_p', lambda: self.d_x(
            factors=self.t.increment / self.x.increment / self.material_vector('density'),
            variant='backward'))

    @property
    def a_vy_p(self):
        return self._operator('a_vy_p', lambda: self.d_y(
            factors=self.t.increment / self.y.increment / self.material_vector('density'),
            variant='backward'))

    @property
    def a_vx_vx(self):
        return self._operator('a_vx_vx', self._absorption_operator)

    @property
    def a_vy_vy(self):
        return self.a_vx_vx


class Acoustic3DAxi(_AcousticBase, fld.Field2D):
    """Axisymmetric acoustic field; x is the radius, y the axis (pyfds/acoustics.py:142-236)."""

    _stag_components = ('pressure', 'velocity_x', 'velocity_y')

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        fld.Field2D.__init__(self, *args, **kwargs)
        self._init_gpu(precision, exact, tile)
        self.pressure = fld.FieldComponent(self.num_points)
        self.velocity_x = fld.FieldComponent(self.num_points)
        self.velocity_y = fld.FieldComponent(self.num_points)

    def _radii(self):
        """Radius of each velocity point, x + dx/2 (pyfds/acoustics.py:166-176)."""
        return np.tile(self.x.vector, self.y.samples) + self.x.increment / 2

    def _coefficients(self):
        # factors of pyfds/acoustics.py:178-203, same expression order
        dt, dx, dy = self.t.increment, self.x.increment, self.y.increment
        c = self.material_vector('sound_velocity')
        rho = self.material_vector('density')
        mu = self.material_vector('absorption_coef')
        r = self._radii()
        kx = dt / dx * c ** 2 * rho
        if self.exact:
            # a_p_vx keeps the 1/r factor and the step multiplies v_x by r
            kx = kx / r
        coefs = {"kx": kx, "ky": dt / dy * c ** 2 * rho, "bx": dt / dx / rho,
                 "by": dt / dy / rho, "rx": self.x.vector + dx / 2}
        flags = _capi.FLAG_HAS_V | _capi.FLAG_AXI
        ax = dt / dx ** 2 * mu / rho
        ay = dt / dy ** 2 * mu / rho
        if np.any(mu != 0):
            flags |= _capi.FLAG_ABSORB
            central = dt / dx * mu / rho / r
            coefs.update(summed_absorption(self.x.samples, True, ax, ay, central))
            coefs["ex"] = dt * mu / rho
        return coefs, flags

    def _absorption_operator(self):
        return (self.d_x2(factors=(self.t.increment / self.x.increment ** 2
                                   * self.material_vector('absorption_coef')
                                   / self.material_vector('density')))
                + self.d_y2(factors=(self.t.increment / self.y.increment ** 2
                                     * self.material_vector('absorption_coef')
                                     / self.material_vector('density')))
                + self.d_x(factors=(self.t.increment / self.x.increment
                                    * self.material_vector('absorption_coef')
                                    / self.material_vector('density') / self._radii()),
                           variant='central')).todia()

    @property
    def a_p_vx(self):
        return self._operator('a_p_vx', lambda: self.d_x(
            factors=self.t.increment / self.x.increment * self.material_vector('sound_velocity')
            ** 2 * self.material_vector('density') / self._radii()))

    @property
    def a_p_vy(self):
        return self._operator('a_p_vy', lambda: self.d_y(
            factors=self.t.increment / self.y.increment * self.material_vector('sound_velocity')
            ** 2 * self.material_vector('density')))

    @property
    def a_vx_p(self):
        return self._operator('a_vx_p', lambda: self.d_x(
            factors=self.t.increment / self.x.increment / self.material_vector('density'),
            variant='backward'))

    @property
    def a_vy_p(self):
        return self._operator('a_vy_p', lambda: self.d_y(
            factors=self.t.increment / self.y.increment / self.material_vector('density'),
            variant='backward'))

    @property
    def a_vx_vx(self):
        return self._operator('a_vx_vx', self._absorption_operator)

    @property
    def a_vy_vy(self):
        return self.a_vx_vx


class AcousticMaterial:
    """Acoustic material parameters (pyfds/acoustics.py:239-286)."""

    def __init__(self, sound_velocity, density,
                 shear_viscosity=0, bulk_viscosity=0,
                 thermal_conductivity=0, isobaric_heat_cap=1, isochoric_heat_cap=1,
                 absorption_coef=None):
        self.sound_velocity = sound_velocity
        self.density = density
        self.shear_viscosity = shear_viscosity
        self.bulk_viscosity = bulk_viscosity
        self.thermal_conductivity = thermal_conductivity
        self.isobaric_heat_cap = isobaric_heat_cap
        self.isochoric_heat_cap = isochoric_heat_cap
        self._absorption_coef = absorption_coef

    @property
    def absorption_coef(self):
        """mu = 4/3 shear + bulk + kappa (cp - cv) / (cp cv), unless set explicitly
        (a falsy explicit value falls back to the computed one, as in the reference)."""
        if not self._absorption_coef:
            return (4 / 3 * self.shear_viscosity + self.bulk_viscosity
                    + self.thermal_conductivity
                    * (self.isobaric_heat_cap - self.isochoric_heat_cap)
                    / (self.isobaric_heat_cap * self.isochoric_heat_cap))
        return self._absorption_coef

    @absorption_coef.setter
    def absorption_coef(self, value):
        self._absorption_coef = value
