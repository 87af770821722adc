"""Arithmetic-expression evaluator for refractive-index and mask formulas (oracle side).

TEST INFRASTRUCTURE ONLY: part of the CPU oracle, never imported by the product.

The reference evaluates the index strings (``no``, ``ne``, ``ne_imag``, ``nhost``, ``nin``,
``nout``; variable ``lambda`` in µm) and the mask formula (variables ``x``, ``y``, ``z``)
with muParser (BeamPropagationSolver/src/PhysicsLib/PhysicsCoefficients.cpp:27-103,
BeamPropagationSolver/src/UtilitiesLib/VectorField.cpp:72-76). muParser is a third-party
dependency that is absent here (unpinned in conda_recipe/recipe.yaml); this module restates
the subset of its published grammar that the Nemaktis Python front end produces:
numbers, variables, ``+ - * / ^`` (``^`` right-associative, binding tighter than unary
minus), parentheses, comparisons, ``&& ||``, the ternary ``?:``, the constants ``_pi`` and
``_e`` and muParser's built-in functions. Values may be Python floats or numpy arrays.
"""
import math
import re

import numpy as np

_TOKEN = re.compile(
    r"\s*(?:(?P<num>(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)|(?P<name>[A-Za-z_][A-Za-z_0-9]*)"
    r"|(?P<op>\|\||&&|<=|>=|==|!=|[-+*/^(),<>?:]))")

_FUNCS = {
    "sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin, "acos": np.arccos,
    "atan": np.arctan, "sinh": np.sinh, "cosh": np.cosh, "tanh": np.tanh,
    "asinh": np.arcsinh, "acosh": np.arccosh, "atanh": np.arctanh,
    "log2": np.log2, "log10": np.log10, "log": np.log, "ln": np.log, "exp": np.exp,
    "sqrt": np.sqrt, "sign": np.sign, "rint": np.rint, "abs": np.abs,
}
_VARFUNCS = {"min": np.minimum.reduce, "max": np.maximum.reduce}
_CONSTS = {"_pi": math.pi, "_e": math.e}


class ExprError(ValueError):
    pass


def _tokenize(s):
    pos, out = 0, []
    s = s.rstrip()
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m or m.end() == pos:
            raise ExprError("unexpected character in expression: %r" % s[pos:])
        pos = m.end()
        for kind in ("num", "name", "op"):
            if m.group(kind) is not None:
                out.append((kind, m.group(kind)))
    return out


class _Parser:
    def __init__(self, tokens, env):
        self.t, self.i, self.env = tokens, 0, env

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if tok[0] is None or (val is not None and tok[1] != val):
            raise ExprError("expected %r" % val)
        self.i += 1
        return tok

    def parse(self):
        v = self.ternary()
        if self.i != len(self.t):
            raise ExprError("unexpected token %r" % (self.t[self.i][1],))
        return v

    def ternary(self):
        c = self.lor()
        if self.peek()[1] == "?":
            self.take("?")
            a = self.ternary()
            self.take(":")
            b = self.ternary()
            return np.where(np.asarray(c) != 0, a, b) if isinstance(c, np.ndarray) else (a if c else b)
        return c

    def lor(self):
        v = self.land()
        while self.peek()[1] == "||":
            self.take()
            w = self.land()
            v = np.logical_or(v != 0, w != 0) * 1.0
        return v

    def land(self):
        v = self.cmp()
        while self.peek()[1] == "&&":
            self.take()
            w = self.cmp()
            v = np.logical_and(v != 0, w != 0) * 1.0
        return v

    def cmp(self):
        v = self.add()
        ops = {"<": np.less, ">": np.greater, "<=": np.less_equal, ">=": np.greater_equal,
               "==": np.equal, "!=": np.not_equal}
        while self.peek()[1] in ops:
            op = self.take()[1]
            v = ops[op](v, self.add()) * 1.0
        return v

    def add(self):
        v = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            w = self.mul()
            v = v + w if op == "+" else v - w
        return v

    def mul(self):
        v = self.unary()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            w = self.unary()
            v = v * w if op == "*" else v / w
        return v

    def unary(self):
        if self.peek()[1] == "-":
            self.take()
            return -self.unary()
        if self.peek()[1] == "+":
            self.take()
            return self.unary()
        return self.power()

    def power(self):
        base = self.primary()
        if self.peek()[1] == "^":
            self.take()
            return np.power(base, self.unary())
        return base

    def primary(self):
        kind, val = self.peek()
        if kind == "num":
            self.take()
            return float(val)
        if kind == "name":
            self.take()
            if self.peek()[1] == "(":
                self.take("(")
                args = [self.ternary()]
                while self.peek()[1] == ",":
                    self.take(",")
                    args.append(self.ternary())
                self.take(")")
                if val in _FUNCS and len(args) == 1:
                    return _FUNCS[val](args[0])
                if val in _VARFUNCS:
                    return _VARFUNCS[val](np.broadcast_arrays(*[np.asarray(a, float) for a in args]))
                if val == "sum":
                    return sum(args)
                if val == "avg":
                    return sum(args) / len(args)
                raise ExprError("unknown function %r" % val)
            if val in self.env:
                return self.env[val]
            if val in _CONSTS:
                return _CONSTS[val]
            raise ExprError("unknown variable %r" % val)
        if val == "(":
            self.take("(")
            v = self.ternary()
            self.take(")")
            return v
        raise ExprError("unexpected token %r" % (val,))


def evaluate(expr, **env):
    """Evaluate ``expr`` with the given variables (scalars or numpy arrays)."""
    tokens = _tokenize(str(expr))
    if not tokens:
        raise ExprError("empty expression")
    v = _Parser(tokens, env).parse()
    if isinstance(v, np.ndarray) and v.ndim == 0:
        return float(v)
    return v
