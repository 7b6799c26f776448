"""Symbol carrying a value, a C type and a constness flag (variable.py:6-21)."""
from sympy import Symbol

__all__ = ['Variable']


class Variable(Symbol):
    """A SymPy Symbol with the extra information the code generators need:
    ``value`` (its numeric value), ``type`` (C type string) and ``constant``
    (whether its value may be folded into generated code)."""

    def __new__(cls, name, *args, **kwargs):
        return Symbol.__new__(cls, name)

    def __init__(self, name, value=0, type='int', constant=False):
        self.type = type
        self.constant = constant
        self.value = value
