"""A UFL-shaped front end for the run-time compiled DG forms.

dune-fem writes schemes in UFL (python/dune/models/integrands/ufl.py lowers
a UFL form to the C++ of an integrands class).  This module accepts forms
written the same way over the structured-grid DG spaces of this package,
for example

    u, v, x = TrialFunction(1), TestFunction(1), SpatialCoordinate()
    a = inner((1 + u[0]**2) * grad(u)[0, :], grad(v)[0, :]) * dx \
        + (u[0]**3 - sin(x[0])) * v[0] * dx
    form = to_form(a, dirichlet=[x[0] * x[1]])

and lowers them to the pointwise pieces of integrands.Form: the coefficient
of grad v in the dx terms becomes the diffusive flux F(x, u, grad u), the
coefficient of v the source s(x, u, grad u), and the DG face terms are the
interior-penalty ones Form builds from F (with A = dF/d grad u by dual
numbers).  A convective flux with its wave speed and Dirichlet data are
given as expressions too.

What is supported: the trial function u (components u[m]), its gradient
grad(u)[m, k], the spatial coordinate x[k], grad(e) and div(E) of
coefficient expressions in x and u (symbolic, by the chain rule; e.g. a
manufactured right-hand side -div(eps grad(exact) - b exact)), numbers and
Constant, + - * /
and ** (numeric or integer exponents), exp, log, sqrt, sin, cos, tan, tanh,
sinh, cosh, atan, abs, max_value / min_value, conditional(cond, a, b) with
lt / gt / le / ge, inner / dot over component lists, and the facet normal
n[k] in a wave speed.  The form must be linear in the test function v.

A form of dx terms alone gets its face terms generated (above).  A form
with facet integrals gives them itself, as UFL does
(python/dune/models/integrands/ufl.py lowers the same three integrals):
  - over interior facets, `* dS`, with restrictions e('+') / e('-') of
    u, grad u, v, grad v and the normal (n('+') is the outward normal of
    the '+' cell, n('-') = -n('+')), jump(e) = e('+') - e('-'),
    jump(e, n) = e('+') n('+') + e('-') n('-') and avg(e);
  - over boundary facets, `* ds`, with u, grad u, v, grad v and n;
  - FacetSize(): avg(CellVolume) / FacetArea on interior facets and
    CellVolume / FacetArea on boundary facets (the cell width normal to the
    face on these grids); those two ratios may also be written as in UFL.
A dS integrand must not change when '+' and '-' are exchanged (as on any
mesh, where the choice is arbitrary): each cell takes the v('+') part with
itself as '+'.  Such a form is lowered to the raw interior / skeleton /
boundary bodies of integrands.Form; periodic faces are interior facets.
"""
import numbers

import integrands


class Expr:
    """A scalar expression tree; cpp() is its CUDA C++ text in the form
    kernels' names (u[m], g[m][k], x[k])."""

    def __add__(self, o):
        return _bin("+", self, o)

    def __radd__(self, o):
        return _bin("+", o, self)

    def __sub__(self, o):
        return _bin("-", self, o)

    def __rsub__(self, o):
        return _bin("-", o, self)

    def __mul__(self, o):
        if isinstance(o, (VLinear, Vector)):
            return o.__rmul__(self)
        return _bin("*", self, o)

    def __rmul__(self, o):
        return _bin("*", o, self)

    def __truediv__(self, o):
        return _bin("/", self, o)

    def __rtruediv__(self, o):
        return _bin("/", o, self)

    def __neg__(self):
        return Op("-", (self,))

    def __abs__(self):
        return Op("fabs", (self,))

    def __pow__(self, p):
        if isinstance(p, numbers.Integral) and 1 <= p <= 16:
            return Op("ipow%d" % p, (self,))
        return Op("pow", (self, _wrap(p)))

    def __lt__(self, o):
        return Cond("<", self, _wrap(o))

    def __gt__(self, o):
        return Cond(">", self, _wrap(o))

    def __le__(self, o):
        return Cond("<=", self, _wrap(o))

    def __ge__(self, o):
        return Cond(">=", self, _wrap(o))

    def __call__(self, side):
        """The restriction e('+') or e('-') to one side of an interior facet."""
        return self.restrict(_side(side))

    def restrict(self, side):
        return self

    def leaves(self):
        return []


def _side(side):
    if side not in ("+", "-"):
        raise ValueError("ufl: restrict with '+' or '-'")
    return side


class Num(Expr):
    def __init__(self, v):
        self.v = float(v)

    def cpp(self):
        return repr(self.v)


class Constant(Num):
    """A named constant (its value is compiled into the kernel)."""

    def __init__(self, v, name=None):
        super().__init__(v)
        self.name = name


class Leaf(Expr):
    def __init__(self, text):
        self.text = text

    def cpp(self):
        return self.text

    def restrict(self, side):
        t = self.text
        if t.startswith("u[") or t.startswith("g["):
            return Leaf(t[0] + ("L" if side == "+" else "R") + t[1:])
        if t.startswith("uL[") or t.startswith("uR[") or t.startswith("gL[") or t.startswith("gR["):
            raise ValueError("ufl: %s is restricted already" % t)
        if t.startswith("n[") and side == "-":
            return Op("-", (self,))
        return self  # x[k], the facet size

    def leaves(self):
        return [self.text]


class Op(Expr):
    _FN = {"exp", "log", "sqrt", "sin", "cos", "tan", "tanh", "sinh", "cosh", "atan", "fabs", "pow", "max", "min"}

    def __init__(self, op, args):
        self.op, self.args = op, args

    def restrict(self, side):
        return Op(self.op, tuple(a.restrict(side) for a in self.args))

    def leaves(self):
        return [t for a in self.args for t in a.leaves()]

    def cpp(self):
        a = [x.cpp() for x in self.args]
        if self.op in "+-*/" and len(a) == 2:
            return "(%s %s %s)" % (a[0], self.op, a[1])
        if self.op == "-":
            return "(-%s)" % a[0]
        if self.op.startswith("ipow"):
            return "ipow<%s>(D(%s))" % (self.op[4:], a[0])
        if self.op in ("max", "min"):
            return "%s(D(%s), D(%s))" % (self.op, a[0], a[1])
        if self.op == "pow":
            return "pow(D(%s), %s)" % (a[0], a[1])
        return "%s(%s)" % (self.op, ", ".join(a))


class Cond(Expr):
    def __init__(self, op, a, b):
        self.op, self.a, self.b = op, a, b

    def restrict(self, side):
        return Cond(self.op, self.a.restrict(side), self.b.restrict(side))

    def leaves(self):
        return self.a.leaves() + self.b.leaves()

    def cpp(self):
        return "(%s %s %s)" % (self.a.cpp(), self.op, self.b.cpp())


class Conditional(Expr):
    def __init__(self, c, a, b):
        self.c, self.a, self.b = c, a, b

    def restrict(self, side):
        return Conditional(self.c.restrict(side), self.a.restrict(side), self.b.restrict(side))

    def leaves(self):
        return self.c.leaves() + self.a.leaves() + self.b.leaves()

    def cpp(self):
        return "(%s ? D(%s) : D(%s))" % (self.c.cpp(), self.a.cpp(), self.b.cpp())


def _wrap(v):
    if isinstance(v, Expr):
        return v
    if isinstance(v, numbers.Real):
        return Num(v)
    raise TypeError("ufl: cannot use %r in an expression" % (v,))


def _is(e, v):
    return isinstance(e, Num) and not isinstance(e, Constant) and e.v == v


def _bin(op, a, b):
    a, b = _wrap(a), _wrap(b)
    if op == "*" and _is(b, 1.0):
        return a
    if op == "*" and _is(a, 1.0):
        return b
    return Op(op, (a, b))


def _fn(name):
    def f(a):
        return Op(name, (_wrap(a),))
    return f


exp, log, sqrt, sin, cos, tan = _fn("exp"), _fn("log"), _fn("sqrt"), _fn("sin"), _fn("cos"), _fn("tan")
tanh, sinh, cosh, atan = _fn("tanh"), _fn("sinh"), _fn("cosh"), _fn("atan")


def max_value(a, b):
    return Op("max", (_wrap(a), _wrap(b)))


def min_value(a, b):
    return Op("min", (_wrap(a), _wrap(b)))


def conditional(c, a, b):
    if not isinstance(c, Cond):
        raise TypeError("ufl: conditional needs a comparison (lt, gt, le, ge or <, >, <=, >=)")
    return Conditional(c, _wrap(a), _wrap(b))


def lt(a, b):
    return Cond("<", _wrap(a), _wrap(b))


def gt(a, b):
    return Cond(">", _wrap(a), _wrap(b))


def le(a, b):
    return Cond("<=", _wrap(a), _wrap(b))


def ge(a, b):
    return Cond(">=", _wrap(a), _wrap(b))


class Vector:
    """A list of expressions (a gradient row, a coefficient vector)."""

    def __init__(self, items):
        self.items = list(items)

    def __len__(self):
        return len(self.items)

    def __getitem__(self, k):
        return self.items[k]

    def __mul__(self, s):
        return Vector([e * s for e in self.items])

    def __rmul__(self, s):
        return Vector([s * e for e in self.items])

    def __add__(self, o):
        return Vector([a + b for a, b in zip(self.items, o.items)])

    def __sub__(self, o):
        return Vector([a - b for a, b in zip(self.items, o.items)])

    def __neg__(self):
        return Vector([-a for a in self.items])

    def __call__(self, side):
        return Vector([e(side) for e in self.items])


def as_vector(items):
    return Vector([_wrap(e) if not isinstance(e, VLinear) else e for e in items])


# ---- the test function and forms linear in it ---------------------------------

class VLinear:
    """sum_m c_v[m] v_m + sum_{m,k} c_g[m][k] dv_m/dx_k (c: expressions)."""

    def __init__(self, terms=None):
        self.terms = dict(terms or {})  # ("v", m) or ("g", m, k) -> Expr

    def _scale(self, s):
        return VLinear({k: _wrap(s) * c for k, c in self.terms.items()})

    def __mul__(self, s):
        if isinstance(s, (VLinear, Vector)):
            raise ValueError("ufl: the form is not linear in the test function")
        if isinstance(s, Measure):
            return s.__rmul__(self)
        return self._scale(s)

    __rmul__ = _scale

    def __truediv__(self, s):
        return self._scale(1.0 / _wrap(s) if not isinstance(s, numbers.Real) else 1.0 / s)

    def __add__(self, o):
        if isinstance(o, Integrals):
            return Integrals(dx=self) + o
        if not isinstance(o, VLinear):
            raise ValueError("ufl: a sum of terms linear and not linear in the test function")
        t = dict(self.terms)
        for k, c in o.terms.items():
            t[k] = t[k] + c if k in t else c
        return VLinear(t)

    def __sub__(self, o):
        if isinstance(o, Integrals):
            return Integrals(dx=self) - o
        return self + (-1.0) * o

    def __neg__(self):
        return self._scale(-1.0)

    def __call__(self, side):
        side = _side(side)
        out = {}
        for key, c in self.terms.items():
            if len(key[0]) > 1:
                raise ValueError("ufl: the test function is restricted already")
            out[(key[0] + side,) + key[1:]] = c.restrict(side)
        return VLinear(out)

    def restricted(self):
        return any(len(k[0]) > 1 for k in self.terms)

    def __eq__(self, rhs):
        return Equation(self, rhs)

    __hash__ = None


class TestFunction:
    """v of the DG space with `components` components: v[m]."""

    def __init__(self, components=1):
        self.components = components

    def __getitem__(self, m):
        return VLinear({("v", m): Num(1.0)})


class TrialFunction:
    """u, the unknown of a (possibly nonlinear) form: u[m]."""

    def __init__(self, components=1):
        self.components = components

    def __getitem__(self, m):
        return Leaf("u[%d]" % m)


class SpatialCoordinate:
    def __getitem__(self, k):
        return Leaf("x[%d]" % k)


class _Grad:
    def __init__(self, f):
        self.f = f

    def __getitem__(self, idx):
        m, k = idx
        if isinstance(self.f, TestFunction):
            if isinstance(k, slice):
                return Vector([VLinear({("g", m, kk): Num(1.0)}) for kk in range(3)])
            return VLinear({("g", m, k): Num(1.0)})
        if isinstance(k, slice):
            return Vector([Leaf("g[%d][%d]" % (m, kk)) for kk in range(3)])
        return Leaf("g[%d][%d]" % (m, k))


# ---- derivatives of coefficient expressions ---------------------------------------

def _zero(e):
    return isinstance(e, Num) and not isinstance(e, Constant) and e.v == 0.0


def _sum(a, b):
    if _zero(a):
        return b
    if _zero(b):
        return a
    return Op("+", (a, b))


def _prod(a, b):
    if _zero(a) or _zero(b):
        return Num(0.0)
    return _bin("*", a, b)


def _diff(e, var):
    """d e / d var for var "x[k]" or "u[m]", by the chain rule over the tree.
    Gradients of u inside e would need second derivatives: refused."""
    if isinstance(e, Num):
        return Num(0.0)
    if isinstance(e, Leaf):
        t = e.text
        if t == var:
            return Num(1.0)
        if t.startswith("g") or t[:2] in ("uL", "uR"):
            raise ValueError("ufl: grad of an expression needs it in x and u only (not grad u, not restricted)")
        return Num(0.0)
    if isinstance(e, (Cond,)):
        return Num(0.0)
    if isinstance(e, Conditional):  # almost everywhere
        return Conditional(e.c, _diff(e.a, var), _diff(e.b, var))
    if not isinstance(e, Op):
        raise TypeError("ufl: cannot differentiate %r" % (e,))
    a = e.args
    da = [_diff(x, var) for x in a]
    op = e.op
    if op == "+" and len(a) == 2:
        return _sum(da[0], da[1])
    if op == "-" and len(a) == 2:
        return _sum(da[0], _prod(Num(-1.0), da[1])) if not _zero(da[1]) else da[0]
    if op == "-":
        return Num(0.0) if _zero(da[0]) else Op("-", (da[0],))
    if op == "*":
        return _sum(_prod(da[0], a[1]), _prod(a[0], da[1]))
    if op == "/":
        num = _sum(_prod(da[0], a[1]), _prod(Num(-1.0), _prod(a[0], da[1])))
        return Num(0.0) if _zero(num) else Op("/", (num, Op("*", (a[1], a[1]))))
    if all(_zero(d) for d in da):
        return Num(0.0)
    x, dx = a[0], da[0]
    if op == "exp":
        return _prod(Op("exp", (x,)), dx)
    if op == "log":
        return Op("/", (dx, x))
    if op == "sqrt":
        return Op("/", (dx, Op("*", (Num(2.0), Op("sqrt", (x,))))))
    if op == "sin":
        return _prod(Op("cos", (x,)), dx)
    if op == "cos":
        return _prod(Op("-", (Op("sin", (x,)),)), dx)
    if op == "tan":
        return _prod(Op("+", (Num(1.0), Op("ipow2", (Op("tan", (x,)),)))), dx)
    if op == "tanh":
        return _prod(Op("-", (Num(1.0), Op("ipow2", (Op("tanh", (x,)),)))), dx)
    if op == "sinh":
        return _prod(Op("cosh", (x,)), dx)
    if op == "cosh":
        return _prod(Op("sinh", (x,)), dx)
    if op == "atan":
        return Op("/", (dx, Op("+", (Num(1.0), Op("ipow2", (x,))))))
    if op == "fabs":
        return Conditional(Cond(">=", x, Num(0.0)), dx, Op("-", (dx,)))
    if op.startswith("ipow"):
        n = int(op[4:])
        base = Num(float(n)) if n == 1 else _prod(Num(float(n)), Op("ipow%d" % (n - 1), (x,)) if n > 2 else x)
        return _prod(base, dx)
    if op == "pow":
        if not isinstance(a[1], Num) or not _zero(da[1]):
            raise ValueError("ufl: grad of pow needs a constant exponent")
        return _prod(_prod(a[1], Op("pow", (x, Num(a[1].v - 1.0)))), dx)
    if op in ("max", "min"):
        pick = Cond(">=" if op == "max" else "<=", a[0], a[1])
        return Conditional(pick, da[0], da[1])
    raise ValueError("ufl: cannot differentiate %s" % op)


def _total_grad(e, components):
    """d e / d x_k along the solution: the partial in x_k plus
    sum_m d e / d u_m * g[m][k]."""
    e = _wrap(e)
    out = []
    for k in range(3):
        d = _diff(e, "x[%d]" % k)
        for m in range(components):
            du = _diff(e, "u[%d]" % m)
            d = _sum(d, _prod(du, Leaf("g[%d][%d]" % (m, k))))
        out.append(d)
    return Vector(out)


def grad(f, components=4):
    """grad(u)[m, k] = du_m/dx_k (grad(u)[m, :] is the row as a vector); of a
    coefficient expression e(x, u) the vector of its total derivatives
    d e / d x_k (e may depend on u[m], m < components, but not on grad u)."""
    if isinstance(f, (TestFunction, TrialFunction)):
        return _Grad(f)
    if isinstance(f, Expr):
        return _total_grad(f, components)
    raise TypeError("ufl: grad of a test or trial function or of an expression")


def div(f, components=4):
    """sum_k d f_k / d x_k of a vector of expressions."""
    if not isinstance(f, Vector) or len(f) != 3:
        raise TypeError("ufl: div of a vector of three expressions")
    out = Num(0.0)
    for k in range(3):
        out = _sum(out, _total_grad(f[k], components)[k])
    return out


def inner(a, b):
    if isinstance(a, Vector) and isinstance(b, Vector):
        if len(a) != len(b):
            raise ValueError("ufl: inner of vectors of different lengths")
        s = a[0] * b[0]
        for i in range(1, len(a)):
            s = s + a[i] * b[i]
        return s
    return a * b


dot = inner


class Measure:
    def __init__(self, name):
        self.name = name

    def __rmul__(self, integrand):
        if not isinstance(integrand, VLinear):
            raise ValueError("ufl: the integrand must be linear in the test function")
        leaves = [t for c in integrand.terms.values() for t in c.leaves()]
        restricted = [t for t in leaves if t[:2] in ("uL", "uR", "gL", "gR")]
        facet = [t for t in leaves if t.startswith("n[") or t == _FACET_SIZE]
        if self.name == "dx":
            if integrand.restricted() or restricted or facet:
                raise ValueError("ufl: restrictions, normals and facet sizes belong to dS / ds terms")
            return integrand
        if self.name == "dS":
            unrestricted = [t for t in leaves if t[:2] in ("u[", "g[")]
            if unrestricted or not integrand.restricted() or any(len(k[0]) == 1 for k in integrand.terms):
                raise ValueError("ufl: restrict u, grad u and v with ('+') / ('-') in dS terms")
            return Integrals(dS=integrand)
        if integrand.restricted() or restricted:
            raise ValueError("ufl: no restrictions in ds terms")
        return Integrals(ds=integrand)


class Integrals:
    """A form with facet integrals: its dx, dS and ds integrands."""

    def __init__(self, dx=None, dS=None, ds=None):
        self.parts = {"dx": dx or VLinear(), "dS": dS or VLinear(), "ds": ds or VLinear()}

    @staticmethod
    def of(a):
        if isinstance(a, Integrals):
            return a
        if isinstance(a, VLinear):
            return Integrals(dx=a)
        raise ValueError("ufl: add forms (integrands times a measure)")

    def __add__(self, o):
        o = Integrals.of(o)
        return Integrals(**{k: self.parts[k] + o.parts[k] for k in self.parts})

    __radd__ = __add__

    def __sub__(self, o):
        o = Integrals.of(o)
        return Integrals(**{k: self.parts[k] - o.parts[k] for k in self.parts})

    def __rsub__(self, o):
        return Integrals.of(o) - self

    def __neg__(self):
        return Integrals(**{k: -p for k, p in self.parts.items()})

    def __eq__(self, rhs):
        return Equation(self, rhs)

    __hash__ = None


_FACET_SIZE = "(1.0 / sigma)"


def FacetSize():
    """avg(CellVolume)/FacetArea on interior facets, CellVolume/FacetArea on
    boundary facets: the cell width normal to the face.  The form kernels
    pass sigma = penalty / h_F to the face terms; a form that uses the facet
    size runs with penalty 1 (FormOperator sets it), so h_F = 1 / sigma."""
    return Leaf(_FACET_SIZE)


class _MeshQuantity:
    """CellVolume / FacetArea of the uniform structured grid: only their
    ratio, the facet size, is an expression here (UFL's
    avg(CellVolume(space)) / FacetArea(space) and CellVolume(space) /
    FacetArea(space), which are the same on these grids)."""

    def __init__(self, kind):
        self.kind = kind

    def __call__(self, side):
        _side(side)
        return self  # the cells of a uniform grid all have the same volume

    def __truediv__(self, o):
        if self.kind == "volume" and isinstance(o, _MeshQuantity) and o.kind == "area":
            return FacetSize()
        raise ValueError("ufl: CellVolume and FacetArea are supported as CellVolume / FacetArea only")


def CellVolume(space=None):
    return _MeshQuantity("volume")


def FacetArea(space=None):
    return _MeshQuantity("area")


def jump(e, n=None):
    """e('+') - e('-'), or e('+') n('+') + e('-') n('-') with a normal."""
    if n is None:
        return e("+") - e("-")
    if not isinstance(n, FacetNormal):
        raise TypeError("ufl: jump(e, n) takes the FacetNormal")
    np_, nm = n("+"), n("-")
    return Vector([e("+") * np_[k] + e("-") * nm[k] for k in range(3)])


def avg(e):
    """(e('+') + e('-')) / 2."""
    if isinstance(e, _MeshQuantity):
        return e
    return 0.5 * (e("+") + e("-"))


dx = Measure("dx")
ds = Measure("ds")
dS = Measure("dS")


def _body(v, side=""):
    """Statements assigning s[m] and F[m][k] from the coefficients of v_m and
    dv_m/dx_k (of the restriction `side` of v, if given)."""
    out = []
    for key, c in sorted(v.terms.items(), key=lambda kv: repr(kv[0])):
        kind = key[0]
        if kind == "g" + side:
            out.append("F[%d][%d] = F[%d][%d] + D(%s);" % (key[1], key[2], key[1], key[2], c.cpp()))
        elif kind == "v" + side:
            out.append("s[%d] = s[%d] + D(%s);" % (key[1], key[1], c.cpp()))
    return "\n".join(out)


def to_form(a, components=1, advection=None, wavespeed=None, dirichlet=None, symmetry=1):
    """integrands.Form of the form `a` (linear in the test function).

    dx terms alone: flux F[m][k] = coefficient of dv_m/dx_k, source s[m] =
    coefficient of v_m, with the face terms generated; advection: per
    component a list of three expressions (Fa[m][k]), wavespeed: an
    expression (may use n[k]), dirichlet: one expression of x per component
    (None: natural boundary).

    With dS / ds terms: the raw interior, skeleton and boundary bodies of
    the three integrals (the skeleton from the v('+') part, the cell itself
    being '+'); advection, wavespeed and dirichlet are then part of the
    integrals and not given here."""
    if isinstance(a, Integrals):
        if not (a.parts["dS"].terms or a.parts["ds"].terms):
            a = a.parts["dx"]
        else:
            if advection is not None or wavespeed is not None or dirichlet is not None or symmetry != 1:
                raise ValueError("ufl: with facet integrals give the face terms in the form itself")
            interior = _body(a.parts["dx"])
            skeleton = _body(a.parts["dS"], "+")
            boundary = _body(a.parts["ds"])
            form = integrands.Form(components=components, interior=interior, skeleton=skeleton, boundary=boundary)
            form.unit_penalty = _FACET_SIZE in skeleton or _FACET_SIZE in boundary
            return form
    if not isinstance(a, VLinear):
        raise ValueError("ufl: a must be a form (an integrand linear in v times a measure)")
    flux, source = [], []
    for key, c in sorted(a.terms.items(), key=lambda kv: repr(kv[0])):
        if key[0] == "g":
            flux.append("F[%d][%d] = F[%d][%d] + D(%s);" % (key[1], key[2], key[1], key[2], c.cpp()))
        else:
            source.append("s[%d] = s[%d] + D(%s);" % (key[1], key[1], c.cpp()))
    adv = None
    if advection is not None:
        adv = "\n".join("Fa[%d][%d] = D(%s);" % (m, k, _wrap(e).cpp())
                        for m, row in enumerate(advection) for k, e in enumerate(row) if row is not None)
    ws = _wrap(wavespeed).cpp() if wavespeed is not None else None
    dirich = None
    if dirichlet is not None:
        dirich = "using D = R;\n" + "\n".join("gD[%d] = R(%s);" % (m, _wrap(e).cpp()) for m, e in enumerate(dirichlet))
    return integrands.Form(components=components, flux="\n".join(flux) or None, source="\n".join(source) or None,
                           advection=adv, wavespeed=ws, dirichlet=dirich, symmetry=symmetry)


class FacetNormal:
    """n[k], the outward normal of the face, for the wave speed of a
    convective flux and in ds terms; n('+') / n('-') as vectors in dS
    terms."""

    def __getitem__(self, k):
        return Leaf("n[%d]" % k)

    def __call__(self, side):
        return Vector([Leaf("n[%d]" % k).restrict(_side(side)) for k in range(3)])

    def vector(self):
        return Vector([Leaf("n[%d]" % k) for k in range(3)])


# ---- spaces, boundary conditions and schemes in dune.fem's shape -------------------

class Equation:
    """a == b: the form a(u, v) - b(v), set to zero by a scheme."""

    def __init__(self, lhs, rhs):
        self.lhs, self.rhs = lhs, rhs

    def residual(self):
        if isinstance(self.rhs, numbers.Real) and self.rhs == 0:
            return self.lhs
        return self.lhs - self.rhs


class DGSpace:
    """A discontinuous Legendre space of order `order` with `dimRange`
    components on a structured grid of `cells` (the counterpart of
    dune.fem.space.dglegendre over a YaspGrid; the dofs are laid out as
    dune-fem lays out a non-hierarchical Legendre DG space)."""

    def __init__(self, cells, order, dimRange=1, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0),
                 periodic=(0, 0, 0), precision=None):
        import gbfem
        self.cells, self.order, self.dimRange = tuple(int(c) for c in cells), int(order), int(dimRange)
        self.lower, self.upper, self.periodic = tuple(lower), tuple(upper), tuple(periodic)
        self.precision = gbfem.F64 if precision is None else precision
        self.size = self.dimRange * (self.order + 1) ** 3 * self.cells[0] * self.cells[1] * self.cells[2]

    @property
    def zero(self):
        import gbfem
        z = gbfem.DeviceArray(self.size, self.precision)
        z.clear()
        return z


def dglegendre(cells, order, dimRange=1, **kwargs):
    """DGSpace(cells, order, dimRange, lower=, upper=, periodic=, precision=)."""
    return DGSpace(cells, order, dimRange, **kwargs)


class DirichletBC:
    """Dirichlet data g on the non-periodic boundary: one expression of x per
    component (or one expression for a scalar space).  DG spaces take it
    weakly, through the interior-penalty boundary terms (the form's
    dirichlet); the counterpart of dune.ufl.DirichletBC in a DG scheme."""

    def __init__(self, space, value):
        self.space = space
        self.value = list(value) if isinstance(value, (list, tuple, Vector)) else [value]


def galerkin(integrands, space=None, solver=None, parameters=None, quad_points=0, penalty=None):
    """A scheme for `integrands`: an Equation (a == b, a == 0), or a list of
    one Equation and at most one DirichletBC, as dune.fem.scheme.galerkin
    takes them (python/dune/fem/scheme/__init__.py).  The form is compiled
    at run time (integrands.FormOperator) on `space` (or the DirichletBC's);
    solver: the linear method ("cg", "gmres", "bicgstab", ...), stored as
    "linear.method" in the fem.solver parameters.  Returns a gbfem.Scheme:
    scheme(u, w), scheme.solve(target=, rightHandSide=)."""
    import gbfem
    import integrands as _integrands
    items = list(integrands) if isinstance(integrands, (list, tuple)) else [integrands]
    eqs = [e for e in items if isinstance(e, Equation)]
    bcs = [e for e in items if isinstance(e, DirichletBC)]
    if len(eqs) != 1 or len(bcs) > 1 or len(eqs) + len(bcs) != len(items):
        raise ValueError("galerkin: one equation (a == b) and at most one DirichletBC")
    space = space if space is not None else (bcs[0].space if bcs else None)
    if not isinstance(space, DGSpace):
        raise ValueError("galerkin: a DGSpace (dglegendre) is needed")
    residual = eqs[0].residual()
    has_faces = isinstance(residual, Integrals) and (residual.parts["dS"].terms or residual.parts["ds"].terms)
    if bcs and has_faces:
        raise ValueError("galerkin: a form with its own facet integrals gives its boundary terms itself")
    if bcs and len(bcs[0].value) != space.dimRange:
        raise ValueError("galerkin: one Dirichlet expression per component")
    form = to_form(residual, components=space.dimRange, dirichlet=bcs[0].value if bcs else None)
    op = _integrands.FormOperator(form, space.cells, space.order, quad_points=quad_points,
                                  precision=space.precision, penalty=penalty, periodic=space.periodic,
                                  lower=space.lower, upper=space.upper)
    prm = dict(parameters or {})
    if solver is not None:
        prm["linear.method"] = solver
    scheme = gbfem.Scheme(op, prm)
    scheme.form = form
    return scheme
