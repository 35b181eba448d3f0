"""SIMP penaliser bookkeeping (the reference's src/penalizers.py:7-46).

The device evaluates r(x) = m + x^p (1 - m) inside the kernels; this object
keeps the reference's host-side contract (penalisation must be set before
use, ``ValueError`` otherwise) and evaluates r and r' on host or torch data.
"""
from __future__ import annotations


class ElasticPenalizer:
    """Solid isotropic material penalisation with minimum m = 1e-6."""

    def __init__(self):
        self.penalization: float | None = None
        self.minimum = 1e-6

    def set_penalization(self, penalization: float):
        self.penalization = penalization

    def assert_has_penalization(self):
        if self.penalization is None:
            raise ValueError("You must set penalization before calling penalizer")
        return self.penalization

    def __call__(self, rho):
        p, m = self.assert_has_penalization(), self.minimum
        return m + rho ** p * (1 - m)

    def derivative(self, rho):
        p, m = self.assert_has_penalization(), self.minimum
        return p * rho ** (p - 1) * (1 - m)


class FluidPenalizer(ElasticPenalizer):
    """Brinkman inverse permeability alpha(rho) = a_max + (a_min - a_max) rho (1 + q) / (rho + q)
    with a_min = 2.5 / 100^2 and a_max = 2.5 / 0.01^2 (the reference's src/penalizers.py:49-67);
    the device evaluates it inside the fluid kernels."""

    def __init__(self):
        super().__init__()
        self.minimum = 2.5 / 100 ** 2
        self.maximum = 2.5 / 0.01 ** 2

    def __call__(self, rho):
        q, mini, maxi = self.assert_has_penalization(), self.minimum, self.maximum
        return maxi + (mini - maxi) * rho * (1 + q) / (rho + q)

    def derivative(self, rho):
        q, mini, maxi = self.assert_has_penalization(), self.minimum, self.maximum
        return (mini - maxi) * q * (1 + q) / (rho + q) ** 2
