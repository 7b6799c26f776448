"""opesci-fd API on a GB300-native CUDA backend.

Star-exports the modelling API like the reference package
(opesci/__init__.py:1-8): fields, derivatives, grids, code printer, FD helpers
and the SymPy names model scripts use."""
from .variable import *  # noqa: F401,F403
from .fields import *  # noqa: F401,F403
from .derivative import *  # noqa: F401,F403
from .staggeredgrid import *  # noqa: F401,F403
from .codeprinter import *  # noqa: F401,F403
from .util import *  # noqa: F401,F403
from .regulargrid import *  # noqa: F401,F403
from sympy import symbols, Eq, sqrt, pi, cos, sin, Float  # noqa: F401

__version__ = '0.1.0+gb300'
