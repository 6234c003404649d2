"""Predefined coupled fields (pyfds/coupled_fields.py API)."""
import ctypes as C

import numpy as np

from . import _capi
from . import acoustics as ac
from . import coupling as cp
from . import thermal as th
from ._engine import require_cuda

__all__ = [
    'ThermoAcoustic1D',
]


class ThermoAcoustic1D(cp.SynchronizedFields):
    """Acoustic and thermal 1-D co-simulation: viscous losses of the acoustic field
    heat the thermal field (pyfds/coupled_fields.py:10-65)."""

    def __init__(self, x_samples, x_delta, t_samples, t_delta,
                 thermal_material, acoustic_material, stepping=1, **field_kwargs):
        """Args as in the reference; ``field_kwargs`` (e.g. ``exact=True``) go to both
        field constructors."""
        acoustic_field = ac.Acoustic1D(x_samples, x_delta, t_samples, t_delta, acoustic_material,
                                       **field_kwargs)
        thermal_field = th.Thermal1D(x_samples, x_delta, t_samples, t_delta, thermal_material,
                                     **field_kwargs)
        acoustic_loss = cp.BoundaryCoupling(
            source_component=acoustic_field.velocity,
            target_component=thermal_field.temperature,
            transfer_function=self._loss_coupling,
            additive=True,
            accumulate=True if stepping > 1 else False,
            stepping=stepping)
        super().__init__([acoustic_field, thermal_field], [acoustic_loss])
        self._loss = acoustic_loss
        self._coupling_vectors = None
        self.get_index = acoustic_field.get_index
        self.get_position = acoustic_field.get_position
        self.get_line_region = acoustic_field.get_line_region

    def _loss_coupling(self, velocity):
        """Heat per step from the velocity gradient: mu / (rho_th c_th) (dv/dx)^2 dt, the
        derivative formed with the acoustic field's a_v_p without its density factor."""
        velocity_derivative = self.fields[0].a_v_p.dot(
            velocity * self.fields[0].material_vector('density'))
        return self.fields[0].material_vector('absorption_coef') \
            / self.fields[1].material_vector('density') \
            / self.fields[1].material_vector('heat_capacity') \
            * velocity_derivative ** 2 * self.t.increment

    # ------------------------------------------------------------ native stepping
    def _native_path(self):
        """True while the coupling is the built-in loss coupling and both fields are
        plain float64 GPU fields: then simulate() runs every step of a chunk in one
        library call (fds_thermoacoustic_run)."""
        loss = self._loss
        if self.interactions != [loss] or loss.additive is not True:
            return False
        if getattr(loss.transfer_function, '__func__', None) is not ThermoAcoustic1D._loss_coupling \
                or getattr(loss.transfer_function, '__self__', None) is not self:
            return False
        if loss.source_component is not self.fields[0].velocity or \
                loss.target_component is not self.fields[1].temperature:
            return False
        for f in self.fields:
            if f.precision != 'f64' or not f._fused_path() or 'material_vector' in vars(f):
                return False
        return True

    def simulate(self, num_steps=None):
        """Field.simulate (pyfds/fields.py:67-95); on the native path all steps of the
        call run in the library, with the same result as stepping one by one."""
        if not self._native_path():
            return super().simulate(num_steps)
        if not num_steps:
            num_steps = self.t.samples
        if not self.matrices_assembled:
            self.assemble_matrices()
        diverged = self._run_native(self.step, int(num_steps))
        self.step = self.step + int(num_steps)
        for eng in diverged:
            eng.report_nonfinite(self.step)

    def _run_native(self, step0, n):
        torch = require_cuda()
        acf, thf = self.fields
        ea, et = acf._engine(), thf._engine()
        pa = ea.prepare(step0, n, cache_tables=True)
        pt = et.prepare(step0, n, cache_tables=True)
        dev = ea.coef_tensors["bx"].device
        key = (acf._coef_version, thf._coef_version)
        if self._coupling_vectors is None or self._coupling_vectors[0] != key:
            g = acf.material_vector('absorption_coef') / thf.material_vector('density') \
                / thf.material_vector('heat_capacity')
            rho = acf.material_vector('density')
            self._coupling_vectors = (key, torch.from_numpy(np.ascontiguousarray(g)).to(dev),
                                      torch.from_numpy(np.ascontiguousarray(rho)).to(dev))
        _, g_t, rho_t = self._coupling_vectors
        acc_host = self._loss.accumulated_transfer
        empty = C.c_int32(1 if np.ndim(acc_host) == 0 and acc_host == 0 else 0)
        acc = torch.zeros(acf.num_points, dtype=torch.float64, device=dev)
        if not empty.value:
            acc.copy_(torch.from_numpy(np.broadcast_to(np.asarray(acc_host, dtype=np.float64),
                                                       (acf.num_points,)).copy()))
        states = []
        for eng, f in ((ea, acf), (et, thf)):
            st = _capi.FdsStagState()
            for k, name in enumerate(f._stag_components):
                cur, nxt = eng.buffers[name]
                st.cur[k] = cur.data_ptr()
                st.nxt[k] = nxt.data_ptr()
            states.append(st)
        lib = _capi.load()
        code = lib.fds_thermoacoustic_run(
            C.byref(pa["prob"]), C.byref(states[0]), C.byref(pa["tstruct"]),
            C.byref(pt["prob"]), C.byref(states[1]), C.byref(pt["tstruct"]),
            C.c_void_p(g_t.data_ptr()), C.c_void_p(rho_t.data_ptr()),
            C.c_void_p(acc.data_ptr()), C.byref(empty), float(self.t.increment),
            int(self._loss.stepping), 1 if self._loss.accumulate else 0, int(step0), int(n),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
        _capi.check(code)
        diverged = []
        for eng, f, st, plan in ((ea, acf, states[0], pa), (et, thf, states[1], pt)):
            for k, name in enumerate(f._stag_components):
                bufs = eng.buffers[name]
                if st.cur[k] != bufs[0].data_ptr():
                    bufs.reverse()
                getattr(f, name)._where = "device"
            eng._last = plan
            if eng.finish(plan):
                diverged.append(eng)
        if self._loss.accumulate:
            self._loss.accumulated_transfer = 0 if empty.value else acc.cpu().numpy()
        return diverged
