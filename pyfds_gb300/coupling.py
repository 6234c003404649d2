"""Coupled fields (pyfds/coupling.py API).

``SynchronizedFields`` steps several fields of the same resolution in lockstep and
applies interactions after every step; ``BoundaryCoupling`` feeds a transfer
function of one component into another, the ``MaterialCoupling`` family scales a
material parameter of a field by a transfer function of a component and
re-assembles that field's coefficients. Each field's step runs on the GPU; an
interaction reads and writes the components' ``values`` (host copies that are
uploaded again before the next launch), so user-supplied transfer functions keep
working on numpy arrays exactly as in the reference.
"""
import logging as lo

import numpy as np

from . import fields as fld

__all__ = [
    'SynchronizedFields', 'BoundaryCoupling', 'MaterialCoupling', 'MaterialCouplingExponential',
    'MaterialCouplingPowerLaw',
]

logger = lo.getLogger('pyfds')


class SynchronizedFields(fld.Field):
    """Fields with the same time stepping, advanced together (pyfds/coupling.py:14-87)."""

    def __init__(self, fields, interactions):
        self.fields = fields
        self.interactions = interactions
        # the components of every field are reachable from here (as in the reference,
        # for the animation helpers); identically named components cannot be coupled
        for field in self.fields:
            for name, value in vars(field).items():
                if isinstance(value, fld.FieldComponent):
                    if not hasattr(self, name):
                        setattr(self, name, value)
                    else:
                        raise RuntimeError("Coupling of fields with identically named components "
                                           "is currently not possible")
        self.t = self.fields[0].t
        self.x = self.fields[0].x
        if hasattr(self.fields[0], 'y'):
            self.y = self.fields[0].y

    @property
    def step(self):
        """The step of the first field."""
        return self.fields[0].step

    @step.setter
    def step(self, value):
        for field in self.fields:
            field.step = value

    @property
    def num_points(self):
        return self.fields[0].num_points

    @property
    def material_regions(self):
        """Material regions of every field (read only: add regions to the fields)."""
        regions = []
        for field in self.fields:
            regions += field.material_regions
        return regions

    def assemble_matrices(self):
        for field in self.fields:
            field.assemble_matrices()

    @property
    def matrices_assembled(self):
        return all([field.matrices_assembled for field in self.fields])

    def sim_step(self):
        """One step of every field, then every interaction (pyfds/coupling.py:81-87)."""
        for field in self.fields:
            field.sim_step()
        for interaction in self.interactions:
            interaction.apply(self.step)


class BoundaryCoupling:
    """Feeds ``transfer_function(source.values)`` into a target component
    (pyfds/coupling.py:90-140): added to it or replacing it, every ``stepping``
    steps, optionally accumulated over the steps in between."""

    def __init__(self, source_component, target_component, transfer_function,
                 additive=True, accumulate=False, stepping=1):
        self.source_component = source_component
        self.target_component = target_component
        self.transfer_function = transfer_function
        self.additive = additive
        self.accumulate = accumulate
        self.stepping = stepping
        self.accumulated_transfer = 0

    def apply(self, step):
        if self.accumulate is True:
            self.accumulated_transfer += self.transfer_function(self.source_component.values)
        if step % self.stepping == 0:
            if self.accumulate is False:
                transfer = self.transfer_function(self.source_component.values)
            else:
                transfer = self.accumulated_transfer
                self.accumulated_transfer = 0
            if self.additive is True:
                self.target_component.values += transfer
            else:
                self.target_component.values = transfer


class MaterialCoupling:
    """Scales a material parameter of ``target_field`` by
    ``transfer_function(source.values)`` (pyfds/coupling.py:143-206). The field's
    ``material_vector`` is replaced by one that applies the factor; coefficients are
    re-assembled every ``stepping`` steps when the factors moved by more than
    ``rel_change_threshold`` (always when it is None)."""

    def __init__(self, source_component, target_field, target_parameter,
                 transfer_function, rel_change_threshold=None, stepping=1):
        self.source_component = source_component
        self.target_field = target_field
        self.target_parameter = target_parameter
        self.transfer_function = transfer_function
        self.rel_change_threshold = rel_change_threshold
        self.stepping = stepping
        self.last_used_factors = 0
        self.target_field.static_material_vector = self.target_field.material_vector
        self.target_field.material_vector = self._material_vector

    def _material_vector(self, mat_parameter):
        if mat_parameter == self.target_parameter:
            return self.target_field.static_material_vector(mat_parameter) \
                * self.transfer_function(self.source_component.values)
        return self.target_field.static_material_vector(mat_parameter)

    def apply(self, step):
        if step % self.stepping == 0:
            transfer_factors = self.transfer_function(self.source_component.values)
            rel_change = max(abs((transfer_factors - self.last_used_factors) / transfer_factors))
            if self.rel_change_threshold is None or rel_change > self.rel_change_threshold:
                # assemble_matrices reads the replaced material_vector
                self.target_field.assemble_matrices()
                self.last_used_factors = transfer_factors
                if self.rel_change_threshold is not None:
                    logger.info(f"Relative change in parameters is {rel_change}.")
                    logger.info(f"Matrices reassembled in step {step}.")


class MaterialCouplingExponential(MaterialCoupling):
    """Factor a + (1 - a) exp(b q) (pyfds/coupling.py:209-254)."""

    def __init__(self, source_component, target_field, target_parameter, a, b,
                 rel_change_threshold=None, stepping=1):
        self.a = a
        self.b = b
        super().__init__(source_component=source_component, target_field=target_field,
                         target_parameter=target_parameter,
                         transfer_function=self.transfer_function,
                         rel_change_threshold=rel_change_threshold, stepping=stepping)

    def transfer_function(self, values):
        return self.a + (1 - self.a) * np.exp(self.b * values)


class MaterialCouplingPowerLaw(MaterialCoupling):
    """Factor 1 + factor q^power (pyfds/coupling.py:257-300)."""

    def __init__(self, source_component, target_field, target_parameter, power, factor,
                 rel_change_threshold=None, stepping=1):
        self.power = power
        self.factor = factor
        super().__init__(source_component=source_component, target_field=target_field,
                         target_parameter=target_parameter,
                         transfer_function=self.transfer_function,
                         rel_change_threshold=rel_change_threshold, stepping=stepping)

    def transfer_function(self, values):
        return 1 + self.factor * values ** self.power
