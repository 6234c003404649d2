"""Coupling API (pyfds/coupling.py): the behaviour the reference's own tests check
(test/test_coupling.py), on this package's classes (CPU: no time stepping)."""
import numpy as np
import pytest

import pyfds_gb300 as fds


def _thermal():
    return fds.Thermal1D(t_delta=1, t_samples=1, x_delta=1, x_samples=3,
                         material=fds.ThermalMaterial(1, 1, 1))


def test_synchronized_fields_structure():
    acs = fds.Acoustic1D(t_delta=1, t_samples=1, x_delta=1, x_samples=3,
                         material=fds.AcousticMaterial(400, 1))
    ths = _thermal()
    with pytest.raises(RuntimeError):
        fds.SynchronizedFields([acs, acs], [])
    cpl = fds.SynchronizedFields([acs, ths], [])
    for comp in (acs.velocity, acs.pressure, ths.temperature, ths.heat_flux):
        assert comp in vars(cpl).values()
    assert len(cpl.material_regions) == 2
    cpl.assemble_matrices()
    assert acs.matrices_assembled and ths.matrices_assembled and cpl.matrices_assembled
    cpl.step = 4
    assert acs.step == ths.step == cpl.step == 4


def test_boundary_coupling():
    comp1 = fds.fields.FieldComponent(num_points=12)
    comp1.values = 2 * np.ones(12)
    comp2 = fds.fields.FieldComponent(num_points=12)
    comp2.values = np.ones(12)
    fds.BoundaryCoupling(comp1, comp2, lambda x: x ** 2).apply(0)
    assert np.allclose(comp2.values, 5)
    accu = fds.BoundaryCoupling(comp1, comp2, lambda x: x, False, True, 3)
    for s in (1, 2, 3, 4):
        accu.apply(s)
    assert np.allclose(comp2.values, 6)


def test_material_coupling_stepping_and_threshold():
    base = np.array([[-1, 1, 0], [0, -1, 1], [0, 0, -1]])
    ths1 = _thermal()
    ths1.assemble_matrices()
    assert np.allclose(ths1.a_t_q.toarray(), base)
    comp1 = fds.fields.FieldComponent(num_points=3)
    comp1.values = np.ones(3)
    cs = fds.MaterialCoupling(comp1, ths1, 'density', lambda x: 1 + x ** 2, stepping=2)
    assert np.allclose(ths1.material_vector('density'), 2)
    assert np.allclose(ths1.material_vector('thermal_conductivity_x'), 1)
    cs.apply(0)
    assert np.allclose(ths1.a_t_q.toarray(), base / 2)
    comp1.values = 2 * np.ones(3)
    cs.apply(1)
    assert np.allclose(ths1.a_t_q.toarray(), base / 2)
    cs.apply(2)
    assert np.allclose(ths1.a_t_q.toarray(), base / 5)
    comp1.values = np.zeros(3)
    ths2 = _thermal()
    ct = fds.MaterialCoupling(comp1, ths2, 'density', lambda x: 1 + x ** 2,
                              rel_change_threshold=0.4)
    ct.apply(0)
    assert np.allclose(ths2.a_t_q.toarray(), base)
    comp1.values = np.ones(3)
    ct.apply(1)
    assert np.allclose(ths2.a_t_q.toarray(), base / 2)
    comp1.values = 1.5 * np.ones(3)
    ct.apply(2)
    assert np.allclose(ths2.a_t_q.toarray(), base / 2)
