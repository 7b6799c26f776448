"""C / CUDA expression printer (restates opesci/codeprinter.py on SymPy 1.14's
C99 printer).  Conventions kept from the reference (codeprinter.py:13-63):
Indexed -> a[i][j][k], Rational p/q -> p.0F/q.0F, Mod -> (a)%(b), Float with
an F suffix in scientific/fixed notation chosen by mpmath."""
from sympy import Eq
from sympy.printing.c import C99CodePrinter
from mpmath.libmp import to_str, prec_to_dps

__all__ = ['CodePrinter', 'ccode', 'ccode_eq']


class CodePrinter(C99CodePrinter):
    """C99 printer with the reference's array and literal conventions."""

    _default_settings = dict(C99CodePrinter._default_settings, full_prec='auto')

    def __init__(self, settings=None):
        super().__init__(settings or {})

    def _print_Indexed(self, expr):
        return self._print(expr.base.label) + ''.join(
            '[' + self._print(x) + ']' for x in expr.indices)

    def _print_Rational(self, expr):
        return '%d.0F/%d.0F' % (int(expr.p), int(expr.q))

    def _print_Mod(self, expr):
        return '%'.join('(' + ccode(x) + ')' for x in expr.args)

    def _print_Float(self, expr):
        prec = expr._prec
        dps = 0 if prec < 5 else prec_to_dps(expr._prec)
        full_prec = self._settings.get("full_prec", "auto")
        if full_prec is True:
            strip = False
        elif full_prec is False:
            strip = True
        else:
            strip = self._print_level > 1
        rv = to_str(expr._mpf_, dps, strip_zeros=strip, max_fixed=-2, min_fixed=2)
        if rv.startswith('-.0'):
            rv = '-0.' + rv[3:]
        elif rv.startswith('.0'):
            rv = '0.' + rv[2:]
        return rv + 'F'

    def _print_Pi(self, expr):
        return 'M_PI'

    def _print_Pow(self, expr):
        # keep pow(x, 2.0) style of the reference output for float exponents
        return super()._print_Pow(expr)

    def _print_Symbol(self, expr):
        return expr.name

    def _print_Variable(self, expr):
        # opesci Variable is a Symbol subclass; SymPy's printer would treat
        # the class name as its codegen AST Variable
        return expr.name

    def _print_DDerivative(self, expr):
        return expr.name


def ccode(expr, **settings):
    """C code of an expression, or an assignment for an Eq."""
    if isinstance(expr, Eq):
        return ccode_eq(expr)
    return CodePrinter(settings).doprint(expr, None)


def ccode_eq(eq, **settings):
    """``lhs = rhs`` for an equation."""
    return (CodePrinter(settings).doprint(eq.lhs, None) + ' = '
            + CodePrinter(settings).doprint(eq.rhs, None))
