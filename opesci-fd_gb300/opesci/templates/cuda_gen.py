"""CUDA code generation for the sweep arithmetic.

The stress and velocity updates are printed from the solved symbolic kernels
(StaggeredGrid.kernel_sympy: expanded, constant-folded, media resolved) with
the same C printer as the reference's generator (codeprinter.py:13-82), then
turned into a device function by two substitutions:

  * every floating literal becomes K[i] (i in order of appearance);
  * every array reference f[_t][x+a][y+b][z+c] becomes A(F_f, a, b, c) and
    every media reference m[x][y][z] becomes A.m(M_m).

Term order, operator order and the arithmetic of the reference's C
expression are therefore kept; only the literal values move to a run-time
table.  SymPy orders the terms of these kernels by their array parts, so the
printed structure depends on the space order and the media mode, not on dt,
spacing or media values; each model's structure is checked against the
signature of the generated header before its table is used.

``python -m opesci.templates.cuda_gen`` (from opesci-fd_gb300/) regenerates
csrc/generated/sweeps_gen.cuh, ghosts_gen.cuh (the space-order-4 Levander
ghost expressions) and signatures.json for space orders 2-8 with constant and
heterogeneous media.
"""
import contextlib
import hashlib
import json
import math
import os
import re
from fractions import Fraction

import numpy as np

from ..codeprinter import ccode

_LIT = re.compile(r'(?<![\w\]\.])(\d+\.\d*(?:e[+-]?\d+)?)F')
_ARR = re.compile(r'\b(U|V|W|Txx|Tyy|Tzz|Txy|Tyz|Txz)\[_t[01]\]\[x(?: ([+-]) (\d+))?\]\[y(?: ([+-]) (\d+))?\]\[z(?: ([+-]) (\d+))?\]')
_MED = re.compile(r'\b(lambda|mu12|mu13|mu23|mu|beta1|beta2|beta3)\[x\]\[y\]\[z\]')
_FIELD = {'U': 'F_U', 'V': 'F_V', 'W': 'F_W', 'Txx': 'F_TXX', 'Tyy': 'F_TYY', 'Tzz': 'F_TZZ',
          'Txy': 'F_TXY', 'Tyz': 'F_TYZ', 'Txz': 'F_TXZ'}
_MEDIA = {'lambda': 'M_LAM', 'mu': 'M_MU', 'mu12': 'M_MU12', 'mu13': 'M_MU13', 'mu23': 'M_MU23',
          'beta1': 'M_B1', 'beta2': 'M_B2', 'beta3': 'M_B3'}

STRESS_ORDER = ['Txx', 'Tyy', 'Tzz', 'Txy', 'Tyz', 'Txz']
VELOCITY_ORDER = ['U', 'V', 'W']


def decimal_to_f32(text):
    """Nearest float32 to a decimal string, ties to even — what a C compiler
    does with the literal ``textF``."""
    q = Fraction(text)
    f = np.float32(float(q))
    best = None
    for c in (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))):
        d = abs(Fraction(float(c)) - q)
        key = (d, int(np.frombuffer(np.float32(c).tobytes(), dtype=np.uint32)[0]) & 1)
        if best is None or key < best[0]:
            best = (key, c)
    return np.float32(best[1])


def _sub_arrays(text):
    def arr(m):
        f = _FIELD[m.group(1)]
        offs = []
        for sgn, val in ((m.group(2), m.group(3)), (m.group(4), m.group(5)), (m.group(6), m.group(7))):
            offs.append('0' if sgn is None else ('-' if sgn == '-' else '') + val)
        return 'A(%s, %s)' % (f, ', '.join(offs))
    text = _ARR.sub(arr, text)
    text = _MED.sub(lambda m: 'A.m(%s)' % _MEDIA[m.group(1)], text)
    return text


def kernel_text(grid, fields):
    """(device-expression texts, literal strings) of the update kernels of
    ``fields`` in the grid's current switches."""
    grid.create_const_dict()
    exprs, lits = [], []
    for f in fields:
        s = ccode(grid.kernel_sympy(f))
        parts = []
        pos = 0
        for m in _LIT.finditer(s):
            parts.append(s[pos:m.start()])
            parts.append('K[%d]' % len(lits))
            lits.append(m.group(1))
            pos = m.end()
        parts.append(s[pos:])
        body = _sub_arrays(''.join(parts))
        if '[' in body.replace('K[', '').replace('A(', ''):
            raise ValueError('unsupported array reference in kernel of %s: %s' % (f.label, body[:200]))
        exprs.append(body)
    return exprs, lits


def signature(exprs):
    canon = '\n'.join(re.sub(r'K\[\d+\]', 'K', e) for e in exprs)
    return hashlib.sha1(canon.encode()).hexdigest()[:16]


@contextlib.contextmanager
def default_form(grid):
    """The grid's update and ghost expressions printed with the expand and
    eval_const switches on (their defaults), whatever the grid's own
    switches.  The device kernels are built for that printed form; with the
    switches off the reference prints the same update unexpanded or with
    named constants, which rounds differently (by ~1e-7 relative)."""
    saved = (grid.expand, grid.eval_const)
    grid.expand, grid.eval_const = True, True
    try:
        yield grid
    finally:
        grid.expand, grid.eval_const = saved


def model_tables(grid):
    """sweep_tables of the grid in its own printed form when the prebuilt
    kernels evaluate it, else in the default form: (tables, own_form)."""
    key = 'so%d_%s' % (grid.order[1], 'het' if grid.read else 'const')
    pre = prebuilt_signatures().get(key)
    tabs = sweep_tables(grid)
    if pre is not None and pre['stress'] == tabs['stress'][0] and pre['velocity'] == tabs['velocity'][0]:
        return tabs, True
    if grid.expand and grid.eval_const:
        return tabs, True
    with default_form(grid):
        return sweep_tables(grid), False


def model_ghost_table(grid):
    """ghost_table of the grid, in the default printed form when its expand
    or eval_const switch is off."""
    if grid.expand and grid.eval_const:
        return ghost_table(grid)
    with default_form(grid):
        return ghost_table(grid)


def sweep_tables(grid):
    """Run-time coefficient tables and structure signatures of a solved
    StaggeredGrid: {'stress': (sig, float32 array), 'velocity': (...)}."""
    by = {f.label.name: f for f in grid.fields}
    out = {}
    for kind, order in (('stress', STRESS_ORDER), ('velocity', VELOCITY_ORDER)):
        exprs, lits = kernel_text(grid, [by[n] for n in order])
        out[kind] = (signature(exprs), np.array([decimal_to_f32(t) for t in lits], dtype=np.float32))
    return out


def _unit_grid(space_order):
    """Heterogeneous model with dt = 1 and unit spacing: its literals are the
    exact rationals r_i of the update expressions (K_i = r_i dt / h)."""
    from ..models import elastic_grid
    return elastic_grid((13.0, 13.0, 13.0), (13, 13, 13), 1.0, 10.0, space_order=space_order,
                        read=True, rho_file='r', vp_file='p', vs_file='s', analytic=False,
                        free_surface=False)


def het_tables(space_order, dt, h):
    """Literal tables of the heterogeneous update expressions for isotropic
    spacing h and time step dt, from the stored unit tables: every literal of
    these expressions is a rational times dt/h.  Returns float32 (ks, kv)."""
    sig = prebuilt_signatures()['so%d_het' % space_order]
    f = float(dt) / float(h)
    ks = np.array([np.float32(float(r) * f) for r in sig['unit_stress']], dtype=np.float32)
    kv = np.array([np.float32(float(r) * f) for r in sig['unit_velocity']], dtype=np.float32)
    return ks, kv


def _variant_grid(space_order, hetero):
    from ..models import elastic_grid
    if hetero:
        return elastic_grid((130.0, 130.0, 130.0), (13, 13, 13), 7e-4, 7e-3, space_order=space_order,
                            read=True, rho_file='r', vp_file='p', vs_file='s', analytic=False,
                            free_surface=False)
    return elastic_grid((1.0, 1.0, 1.0), (13, 13, 13), 3e-3, 3e-2, space_order=space_order,
                        analytic=False, free_surface=False)


def split_terms(expr):
    """The top-level terms of a printed sum, left to right: [(op, term)] with
    op '' for the first term (which may carry a unary sign) and '+'/'-' for
    the rest.  Rejoining them gives the expression back exactly."""
    out, depth, start, op = [], 0, 0, ''
    i = 0
    while i < len(expr):
        c = expr[i]
        if c in '([':
            depth += 1
        elif c in ')]':
            depth -= 1
        elif depth == 0 and expr[i:i + 3] in (' + ', ' - ') and i > start:
            out.append((op, expr[start:i]))
            op = expr[i + 1]
            start = i + 3
            i += 3
            continue
        i += 1
    out.append((op, expr[start:]))
    back = out[0][1] + ''.join(' %s %s' % (o, t) for o, t in out[1:])
    if back != expr:
        raise RuntimeError('term split does not reproduce the expression')
    return out


def interleaved_lines(exprs, indent='    '):
    """Statements evaluating the sums ``exprs`` into out[0..n-1] with their
    accumulation chains interleaved term by term: chain i is still
    ((t0 op t1) op t2) ... in its printed order, so every result rounds
    exactly as the single expression does, while the independent chains sit
    side by side for the instruction scheduler."""
    terms = [split_terms(e) for e in exprs]
    lines = ['%sC o%d = %s;' % (indent, i, t[0][1]) for i, t in enumerate(terms)]
    for k in range(1, max(len(t) for t in terms)):
        for i, t in enumerate(terms):
            if k < len(t):
                lines.append('%so%d = o%d %s %s;' % (indent, i, i, t[k][0], t[k][1]))
    lines += ['%sout[%d] = o%d;' % (indent, i, i) for i in range(len(terms))]
    return lines


def sequential_lines(exprs, indent='    '):
    """One statement per output, each sum as printed."""
    return ['%sout[%d] = %s;' % (indent, i, e) for i, e in enumerate(exprs)]


# Space orders whose sweeps are emitted with interleaved chains: measured on
# the GB300 at 512^3, interleaving shortened the space-order-4 velocity sweep
# (1.331 -> 1.315 ms) and lengthened the space-order-8 sweeps (2.45 -> 2.53 ms
# stress, 2.00 -> 2.09 ms velocity), whose long chains already overlap.
INTERLEAVE_MAX_ORDER = 4


def generate_headers(outdir):
    """Write sweeps_gen.cuh and signatures.json for all prebuilt variants."""
    os.makedirs(outdir, exist_ok=True)
    sigs = {}
    lines = ['// GENERATED by opesci/templates/cuda_gen.py from the symbolic kernels of',
             '// StaggeredGrid (expanded, constant-folded, media resolved); do not edit.',
             '// Each function evaluates the reference generator\'s C expression of the',
             '// update with its literals taken from the table K; up to space order 4',
             '// the sums of the outputs are interleaved term by term (each chain in',
             '// its printed order).',
             '#pragma once', '#include "ofd_common.cuh"', '', 'namespace ofd {', '',
             'template <int R, int HET> struct GenSweep { static constexpr bool ok = false; };', '']
    for so in (2, 4, 6, 8):
        for het in (0, 1):
            g = _variant_grid(so, het)
            by = {f.label.name: f for f in g.fields}
            se, sl = kernel_text(g, [by[n] for n in STRESS_ORDER])
            ve, vl = kernel_text(g, [by[n] for n in VELOCITY_ORDER])
            key = 'so%d_%s' % (so, 'het' if het else 'const')
            sigs[key] = {'stress': signature(se), 'velocity': signature(ve),
                         'nk_stress': len(sl), 'nk_velocity': len(vl)}
            if het:
                ug = _unit_grid(so)
                uby = {f.label.name: f for f in ug.fields}
                use, usl = kernel_text(ug, [uby[n] for n in STRESS_ORDER])
                uve, uvl = kernel_text(ug, [uby[n] for n in VELOCITY_ORDER])
                if signature(use) != sigs[key]['stress'] or signature(uve) != sigs[key]['velocity']:
                    raise RuntimeError('unit-step structure differs for %s' % key)
                sigs[key]['unit_stress'] = usl
                sigs[key]['unit_velocity'] = uvl
            lines.append('template <> struct GenSweep<%d, %d> {' % (so // 2, het))
            lines.append('  static constexpr bool ok = true;')
            lines.append('  static constexpr int NK_STRESS = %d, NK_VELOCITY = %d;' % (len(sl), len(vl)))
            lines.append('  template <typename C, class Acc, class KT>')
            lines.append('  __device__ __forceinline__ static void stress(const Acc &A, const KT &K, C out[6]) {')
            lines += interleaved_lines(se) if so <= INTERLEAVE_MAX_ORDER else sequential_lines(se)
            lines.append('  }')
            lines.append('  template <typename C, class Acc, class KT>')
            lines.append('  __device__ __forceinline__ static void velocity(const Acc &A, const KT &K, C out[3]) {')
            lines += interleaved_lines(ve) if so <= INTERLEAVE_MAX_ORDER else sequential_lines(ve)
            lines.append('  }')
            lines.append('};')
            lines.append('')
    lines += kmap_lines(sigs)
    lines.append('}  // namespace ofd')
    with open(os.path.join(outdir, 'sweeps_gen.cuh'), 'w') as f:
        f.write('\n'.join(lines) + '\n')
    generate_ghost_header(outdir, sigs)
    sigs['so4_het']['unit_ghost'] = het_ghost_units()
    with open(os.path.join(outdir, 'signatures.json'), 'w') as f:
        json.dump(sigs, f, indent=1, sort_keys=True)
    return sigs


def kmap_lines(sigs):
    """C++ of KMap<R, STRESS>: for the heterogeneous expressions, the index of
    each literal among the distinct rationals of its unit table.  A table
    K_i = r_i dt / h (isotropic spacing) has equal values wherever the r_i
    are equal, so K can be held as those few distinct values."""
    lines = ['// Literal index -> index among the distinct unit rationals of the',
             '// heterogeneous expression (tables K_i = r_i dt / h repeat a few values).',
             'template <int R, bool STRESS> struct KMap { static constexpr bool ok = false; };', '']
    for so in (2, 4, 6, 8):
        key = 'so%d_het' % so
        if key not in sigs:
            continue
        for kind, stress in (('unit_stress', 'true'), ('unit_velocity', 'false')):
            uniq, idx = [], []
            for t in sigs[key][kind]:
                q = Fraction(t)
                if q not in uniq:
                    uniq.append(q)
                idx.append(uniq.index(q))
            lines.append('template <> struct KMap<%d, %s> {' % (so // 2, stress))
            lines.append('  static constexpr bool ok = true;')
            lines.append('  static constexpr int NU = %d, NK = %d;' % (len(uniq), len(idx)))
            lines.append('  __host__ __device__ static constexpr int at(int i) {')
            lines.append('    constexpr int m[%d] = {%s};' % (len(idx), ', '.join(str(i) for i in idx)))
            lines.append('    return m[i];')
            lines.append('  }')
            lines.append('};')
            lines.append('')
    return lines


def prebuilt_signatures():
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                        'csrc', 'generated', 'signatures.json')
    with open(path) as f:
        return json.load(f)




# ----------------------------------------------------------------- ghosts
#
# The Levander free-surface ghosts of space order 4 (fields.py:192-381,
# applied by staggeredgrid.py:754-864) are printed the same way: the
# expanded, constant-folded ghost equations of the frontend (transform_bc,
# media resolved in read mode) become device expressions with their literals
# in a run-time table KG.  Array references are given as offsets from the
# ghost row's point on the boundary plane b (b = m on the lower face,
# dim - m - 1 on the upper), so the text does not depend on the grid size:
#   F[_tL][i][j][k] -> A(F_F, L, ox, oy, oz),  med[i][j][k] -> A.m(M_med, ox, oy, oz).
# pow(m, 2) of the reference's C (a double result, which makes the rest of
# the sum double in C) becomes ofd_pow2(m), the exact double square.
# Every expression is a case of a switch over (component, face normal, side).

_GARR = re.compile(r'\b(U|V|W|Txx|Tyy|Tzz|Txy|Tyz|Txz)\[_t([01])\]\[([^\]]+)\]\[([^\]]+)\]\[([^\]]+)\]')
_GMED = re.compile(r'\b(lambda|mu12|mu13|mu23|mu|beta1|beta2|beta3)\[([^\]]+)\]\[([^\]]+)\]\[([^\]]+)\]')
_GPOW = re.compile(r'pow\((A\.m\([^()]*\)), 2\)')
GHOST_STRESS = ['Txx', 'Tyy', 'Tzz']
GHOST_VEL = ['U', 'V', 'W']


def _ghost_offsets(idx, d, b):
    """Offsets (ox, oy, oz) of three printed indices; axis d holds a plane
    number (relative to b), the others loop variables with offsets."""
    out = []
    for axis, t in enumerate(idx):
        t = t.strip()
        if axis == d:
            if not re.fullmatch(r'\d+', t):
                raise ValueError('unexpected face-normal index %r' % t)
            out.append(int(t) - b)
            continue
        m = re.fullmatch(r'([xyz])(?: ([+-]) (\d+))?', t)
        if not m or 'xyz'.index(m.group(1)) != axis:
            raise ValueError('unexpected in-plane index %r on axis %d' % (t, axis))
        out.append(0 if m.group(2) is None else (int(m.group(3)) if m.group(2) == '+' else -int(m.group(3))))
    return out


def _ghost_rhs(grid, field, d, side):
    """(lhs, rhs) C texts of the ghost equations of ``field`` on face
    (d, side), media resolved in read mode."""
    from ..codeprinter import ccode_eq
    out = []
    for bc in grid.transform_bc(field, d + 1, side):
        if grid.read:
            bc = grid.resolve_media_params(bc)
        s = ccode_eq(bc).replace('[_t + 1]', '[_t1]').replace('[_t]', '[_t0]')
        lhs, rhs = s.split(' = ', 1)
        out.append((lhs, rhs))
    return out


def ghost_text(grid):
    """(cases, literal strings): cases = [(kind, comp, d, side, device text)]
    for the Levander ghosts of a space-order-4 grid with free surfaces on all
    faces; kind 'stress' (normal-stress recompute) or 'velocity'."""
    grid.create_const_dict()
    m = grid.margin.value
    dims = [dd.value for dd in grid.dim]
    by = {f.label.name: f for f in grid.fields}
    cases, lits = [], []

    def device(rhs, d, b):
        parts, pos = [], 0
        for mm in _LIT.finditer(rhs):
            parts.append(rhs[pos:mm.start()])
            parts.append('K[%d]' % len(lits))
            lits.append(mm.group(1))
            pos = mm.end()
        parts.append(rhs[pos:])
        t = ''.join(parts)
        t = _GARR.sub(lambda a: 'A(%s, %s, %s)' % (_FIELD[a.group(1)], a.group(2),
                                                 ', '.join(str(v) for v in _ghost_offsets(a.group(3, 4, 5), d, b))), t)
        t = _GMED.sub(lambda a: 'A.m(%s, %s)' % (_MEDIA[a.group(1)],
                                               ', '.join(str(v) for v in _ghost_offsets(a.group(2, 3, 4), d, b))), t)
        t = _GPOW.sub(lambda a: 'ofd_pow2(%s)' % a.group(1), t)
        if '[' in t.replace('K[', '') or 'pow(' in t:
            raise ValueError('unsupported reference in ghost expression: %s' % t[:200])
        return t

    for ci, name in enumerate(GHOST_STRESS):
        for d in range(3):
            if d == ci:
                continue
            for side in range(2):
                eqs = _ghost_rhs(grid, by[name], d, side)
                if len(eqs) != 1:
                    raise ValueError('expected one recompute equation for %s on face %d/%d' % (name, d, side))
                b = m if side == 0 else dims[d] - m - 1
                cases.append(('stress', ci, d, side, device(eqs[0][1], d, b)))
    for d in range(3):
        for ci, name in enumerate(GHOST_VEL):
            for side in range(2):
                eqs = _ghost_rhs(grid, by[name], d, side)
                if len(eqs) != 1:
                    raise ValueError('expected one ghost equation for %s on face %d/%d' % (name, d, side))
                b = m if side == 0 else dims[d] - m - 1
                cases.append(('velocity', ci, d, side, device(eqs[0][1], d, b)))
    return cases, lits


def ghost_signature(cases):
    canon = '\n'.join('%s %d %d %d %s' % (k, c, d, s, re.sub(r'K\[\d+\]', 'K', t)) for k, c, d, s, t in cases)
    return hashlib.sha1(canon.encode()).hexdigest()[:16]


def ghost_table(grid):
    """(signature, float32 literal table) of a space-order-4 grid's
    Levander ghost expressions, or None when the grid has other ghosts."""
    if grid.order[1] != 4:
        return None
    fs = getattr(grid, 'free_surface', {})
    if len(fs) != 6 or any(v != 'levander' for v in fs.values()):
        return None
    cases, lits = ghost_text(grid)
    return ghost_signature(cases), np.array([decimal_to_f32(t) for t in lits], dtype=np.float32)


def _ghost_variant_grid(hetero):
    from ..models import elastic_grid
    if hetero:
        return elastic_grid((130.0, 130.0, 130.0), (13, 13, 13), 7e-4, 7e-3, space_order=4,
                            read=True, rho_file='r', vp_file='p', vs_file='s', analytic=False,
                            free_surface=True)
    return elastic_grid((1.0, 1.0, 1.0), (13, 13, 13), 3e-3, 3e-2, space_order=4,
                        analytic=False, free_surface=True)


def generate_ghost_header(outdir, sigs):
    """ghosts_gen.cuh: GenGhost4<HET>::stress / ::velocity, and the ghost
    signatures into ``sigs`` (so4_het / so4_const: 'ghost', 'nk_ghost')."""
    lines = ['// GENERATED by opesci/templates/cuda_gen.py from the Levander ghost equations',
             '// of StaggeredGrid at space order 4 (expanded, constant-folded, media',
             '// resolved); do not edit.  Each case evaluates the reference generator\'s C',
             '// expression of one ghost value with its literals taken from the table K;',
             '// A(F, level, ox, oy, oz) is the field at level t0 (0) or t1 (1) at an offset',
             '// from the ghost row\'s point on the boundary plane, A.m(M, ox, oy, oz) a medium.',
             '#pragma once', '#include "ofd_common.cuh"', '', 'namespace ofd {', '',
             '// the exact double square of a float (pow(float, 2) of the reference\'s C++)',
             '__device__ __forceinline__ double ofd_pow2(float v) { return (double)v * (double)v; }', '',
             'template <int HET> struct GenGhost4 { static constexpr bool ok = false; };', '']
    for het in (0, 1):
        g = _ghost_variant_grid(het)
        cases, lits = ghost_text(g)
        key = 'so4_%s' % ('het' if het else 'const')
        sigs.setdefault(key, {})['ghost'] = ghost_signature(cases)
        sigs[key]['nk_ghost'] = len(lits)
        lines.append('template <> struct GenGhost4<%d> {' % het)
        lines.append('  static constexpr bool ok = true;')
        lines.append('  static constexpr int NK = %d;' % len(lits))
        for kind in ('stress', 'velocity'):
            lines.append('  // %s ghost of component c on face normal d, side (0 lower, 1 upper)' %
                         ('normal-stress recompute' if kind == 'stress' else 'velocity'))
            lines.append('  template <class Acc, class KT>')
            lines.append('  __device__ %sstatic float %s(int c, int d, int side, const Acc &A, const KT &K) {' % ('__forceinline__ ' if kind == 'velocity' else '', kind))
            lines.append('    switch (c * 6 + d * 2 + side) {')
            for k, c, d, side, t in cases:
                if k == kind:
                    lines.append('      case %d: return (float)(%s);' % (c * 6 + d * 2 + side, t))
            lines.append('    }')
            lines.append('    return 0.f;')
            lines.append('  }')
        lines.append('};')
        lines.append('')
    lines.append('}  // namespace ofd')
    with open(os.path.join(outdir, 'ghosts_gen.cuh'), 'w') as f:
        f.write('\n'.join(lines) + '\n')


def _het_ghost_grid(dt, h):
    from ..models import elastic_grid
    return elastic_grid((h * 13, h * 13, h * 13), (13, 13, 13), dt, dt * 10, space_order=4, read=True,
                        rho_file='r', vp_file='p', vs_file='s', analytic=False, free_surface=True)


def het_ghost_units():
    """Each literal of the heterogeneous space-order-4 ghost expressions is a
    monomial r dt^a h^b (isotropic spacing h): [str(r), a, b] per literal,
    from the tables at (dt, h) = (1, 1), (2, 1) and (1, 2); checked against
    a table at (7e-4, 10)."""
    _, l1 = ghost_text(_het_ghost_grid(1.0, 1.0))
    _, l2 = ghost_text(_het_ghost_grid(2.0, 1.0))
    _, l3 = ghost_text(_het_ghost_grid(1.0, 2.0))
    _, l4 = ghost_text(_het_ghost_grid(7e-4, 10.0))
    out = []
    for a, b, c, d in zip(l1, l2, l3, l4):
        ra, rb, rc = Fraction(a), Fraction(b), Fraction(c)
        ea = math.log2(float(rb / ra))
        eh = math.log2(float(rc / ra))
        if abs(ea - round(ea)) > 1e-9 or abs(eh - round(eh)) > 1e-9:
            raise RuntimeError('ghost literal is not a monomial in dt and h')
        pred = float(ra) * 7e-4 ** round(ea) * 10.0 ** round(eh)
        if abs(pred / float(Fraction(d)) - 1) > 1e-13:
            raise RuntimeError('ghost literal check failed')
        out.append([a, int(round(ea)), int(round(eh))])
    return out


def het_ghost_table(dt, h):
    """Literal table of the heterogeneous space-order-4 Levander ghost
    expressions for isotropic spacing h and time step dt, from the stored
    monomials (the same values the frontend prints for that grid)."""
    units = prebuilt_signatures()['so4_het']['unit_ghost']
    return np.array([np.float32(float(Fraction(r)) * float(dt) ** a * float(h) ** b) for r, a, b in units],
                    dtype=np.float32)


if __name__ == '__main__':
    here = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    print(generate_headers(os.path.join(here, 'csrc', 'generated')))
