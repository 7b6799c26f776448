"""Symbolic derivative placeholder (derivative.py:6-26)."""
from sympy import Symbol

__all__ = ['DDerivative']


class DDerivative(Symbol):
    """A Symbol standing for a partial derivative of a field.

    ``fd[a]`` holds the finite-difference approximation of accuracy ``a``
    (filled by Field.populate_derivatives); ``var`` is the index symbol the
    derivative is taken along and ``order`` the derivative order."""

    def __new__(cls, name, *args, **kwargs):
        return Symbol.__new__(cls, name)

    def __init__(self, name, var, order, max_accuracy):
        self.var = var
        self.order = order
        self.max_accuracy = max_accuracy
        self.fd = [None] * (max_accuracy + 1)
