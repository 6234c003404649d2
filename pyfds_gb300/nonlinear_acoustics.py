"""Nonlinear 1-D acoustic fields (pyfds/nonlinear_acoustics.py API), time-stepped on
the GPU by ``fds_nl1d_run`` (include/fds_capi.h): one launch runs every step of a
``simulate`` chunk."""
import ctypes as C

import numpy as np

from . import _capi, _tables
from . import acoustics as ac
from . import fields as fld
from ._engine import StagEngine, require_cuda
from ._stag import StagField

__all__ = [
    'IdealGas1D', 'Acoustic2ndOrder1D', 'AcousticMaterial2ndOrder',
]


class _NlEngine(StagEngine):
    """StagEngine whose launch is the nonlinear 1-D step (same buffers and tables,
    bucketed per tile of ``tile_cells`` cells: one CTA per tile)."""

    @staticmethod
    def tile_cells(n):
        """64 cells per CTA (spreads the FP64 work over SMs), more for fields above
        512 tiles so that every CTA stays resident."""
        return 64 * max(1, -(-n // (64 * 512)))

    def _geometry(self, batched=False):
        n = self.field.num_points
        return _tables.TileGeometry(n, 1, self.tile_cells(n), 1, False, 0)

    def launch(self, plan):
        torch = require_cuda()
        f = self.field
        prob = _capi.FdsNl1dProblem()
        prob.kind = f._nl_kind
        prob.flags = f._nl_flags() | (_capi.FLAG_EXACT if f.exact else 0)
        prob.n = f.num_points
        prob.tile_x = plan["geo"].tx
        prob.f1 = f._nl_scalars["f1"]
        prob.fc = f._nl_scalars["fc"]
        for name in ("a", "rho0", "e1", "e2"):
            setattr(prob, name, self.coef_tensors[name].data_ptr())
        if getattr(self, "_sync", None) is None:
            self._sync = torch.zeros(1, dtype=torch.int32, device=self.coef_tensors["a"].device)
        prob.sync = self._sync.data_ptr()
        prob.status = self.status.data_ptr() if self.status is not None else None
        names = f._stag_components
        state = _capi.FdsStagState()
        for k in range(3):
            cur, nxt = self.buffers[names[k]]
            state.cur[k] = cur.data_ptr()
            state.nxt[k] = nxt.data_ptr()
        lib = _capi.load()
        code = lib.fds_nl1d_run(C.byref(prob), C.byref(state), C.byref(plan["tstruct"]),
                                plan["step0"], plan["nsteps"],
                                C.c_void_p(torch.cuda.current_stream().cuda_stream))
        _capi.check(code)
        self.launches += 1
        for k, name in enumerate(names):
            bufs = self.buffers[name]
            if state.cur[k] != bufs[0].data_ptr():
                bufs.reverse()
            getattr(f, name)._where = "device"
        self._last = plan


class _Nonlinear1D(StagField, fld.Field1D):
    """Shared part of the nonlinear 1-D fields. Their constructors accept the
    ``precision`` ("f64" only), ``exact`` and ``tile`` keywords of the other fields;
    ``tile`` is ignored (one CTA steps the whole field)."""
    _stag_family = _capi.FAMILY_ACOUSTIC  # every component carries state
    _stag_components = ('pressure', 'velocity', 'density')
    _nl_kind = None

    def _init_nonlinear(self, precision, exact):
        if precision != 'f64':
            raise ValueError("nonlinear 1-D fields run in precision='f64' only")
        self._init_gpu(precision, exact, None)
        self.pressure = fld.FieldComponent(self.num_points)
        self.velocity = fld.FieldComponent(self.num_points)
        self.density = fld.FieldComponent(self.num_points)

    def _engine(self):
        if self._eng is None:
            self._eng = _NlEngine(self)
        return self._eng

    def _common_coefficients(self):
        # factors of pyfds/nonlinear_acoustics.py:41-52, same expression order
        dt, dx = self.t.increment, self.x.increment
        n = self.x.samples
        f1 = (dt / dx * np.ones(n))[0]
        fc = ((dt / dx / 2) * np.ones(n) / 2)[0]
        self._nl_scalars = {"f1": float(f1), "fc": float(fc)}
        return {"a": dt / dx ** 2 * self.material_vector('absorption_coef'),
                "rho0": self.material_vector('density')}

    # reference-style operators, for inspection
    @property
    def a_d_v(self):
        return self._operator('a_d_v', lambda: self.d_x(
            factors=(self.t.increment / self.x.increment * np.ones(self.x.samples))))

    @property
    def a_v_p(self):
        return self._operator('a_v_p', lambda: self.d_x(
            factors=(self.t.increment / self.x.increment) * np.ones(self.x.samples),
            variant='backward'))

    @property
    def a_v_v(self):
        return self._operator('a_v_v', lambda: self.d_x2(
            factors=(self.t.increment / self.x.increment ** 2
                     * self.material_vector('absorption_coef'))))

    @property
    def a_v_v2(self):
        return self._operator('a_v_v2', lambda: self.d_x(
            factors=(self.t.increment / self.x.increment / 2) * np.ones(self.x.samples),
            variant='central'))

    @property
    def stat_density(self):
        return self.material_vector('density') if self.matrices_assembled else None


class IdealGas1D(_Nonlinear1D):
    """One-dimensional nonlinear acoustic field in an ideal gas
    (pyfds/nonlinear_acoustics.py:10-104)."""

    _nl_kind = _capi.NL1D_IDEAL_GAS

    def __init__(self, convective=True, nl_state=True, *args, precision='f64', exact=False,
                 tile=None, **kwargs):
        fld.Field1D.__init__(self, *args, **kwargs)
        self.convective = convective
        self.nl_state = nl_state
        self._init_nonlinear(precision, exact)

    def _nl_flags(self):
        return ((_capi.NL1D_CONVECTIVE if self.convective else 0)
                | (_capi.NL1D_NL_STATE if self.nl_state else 0))

    def _coefficients(self):
        coefs = self._common_coefficients()
        rho0 = coefs["rho0"]
        c = self.material_vector('sound_velocity')
        gamma = (self.material_vector('isobaric_heat_cap')
                 / self.material_vector('isochoric_heat_cap'))
        if self.nl_state:
            coefs["e1"] = rho0 * c ** 2 / gamma
            coefs["e2"] = gamma
        else:
            coefs["e1"] = c ** 2
            coefs["e2"] = np.zeros_like(c)
        return coefs, 0

    @property
    def sound_velocity(self):
        return self.material_vector('sound_velocity') if self.matrices_assembled else None

    @property
    def heat_cap_ratio(self):
        if not self.matrices_assembled:
            return None
        return (self.material_vector('isobaric_heat_cap')
                / self.material_vector('isochoric_heat_cap'))

    def is_stable(self):
        """CFL check with 1 % headroom (pyfds/nonlinear_acoustics.py:92-104)."""
        return np.all(self.material_vector('sound_velocity')
                      < 0.99 * self.x.increment / self.t.increment)


class Acoustic2ndOrder1D(_Nonlinear1D):
    """One-dimensional nonlinear acoustic field, second-order state equation
    (pyfds/nonlinear_acoustics.py:107-163)."""

    _nl_kind = _capi.NL1D_SECOND_ORDER

    def __init__(self, *args, precision='f64', exact=False, tile=None, **kwargs):
        if not (hasattr(kwargs['material'], 'd_rho_p')
                and hasattr(kwargs['material'], 'd_rho2_p')):
            raise RuntimeError('Material with properties d_rho_p and d_rho2_p is required for '
                               '2nd order nonlinear acoustic simulation.')
        fld.Field1D.__init__(self, *args, **kwargs)
        self._init_nonlinear(precision, exact)

    def _nl_flags(self):
        return _capi.NL1D_CONVECTIVE

    def _coefficients(self):
        coefs = self._common_coefficients()
        coefs["e1"] = self.material_vector('d_rho_p')
        coefs["e2"] = self.material_vector('d_rho2_p') / 2
        return coefs, 0

    @property
    def d_rho_p(self):
        return self.material_vector('d_rho_p') if self.matrices_assembled else None

    @property
    def d_rho2_p(self):
        return self.material_vector('d_rho2_p') if self.matrices_assembled else None


class AcousticMaterial2ndOrder(ac.AcousticMaterial):
    """Acoustic material with the first and second derivative of pressure with
    respect to density (pyfds/nonlinear_acoustics.py:166-190)."""

    def __init__(self, d_rho_p=None, d_rho2_p=0, *args, **kwargs):
        super().__init__(*args, **kwargs)
        if not d_rho_p:
            # as in the reference: the attribute lookup goes through the class, where
            # sound_velocity is not defined (it is set per instance)
            self.d_rho_p = super().sound_velocity ** 2
        else:
            self.d_rho_p = d_rho_p
        self.d_rho2_p = d_rho2_p
