"""Orthotope Machine graphs built in Python and run on the GPU.

The builder mirrors the reference's Builder monad
(Language/Paraiso/OM/Builder/Internal.hs): ``load``, ``store``, ``shift``,
``imm``, the arithmetic operators, ``reduce``, ``broadcast``,
``load_index``, ``load_size`` and ``cast`` create the nodes of one kernel's
dataflow graph, in the order and with the types the Haskell builder gives
them:

* a Python number next to a value becomes an ``imm`` of that value's type
  and realm (``fromInteger`` / ``fromRational'``);
* ``v ** n`` with an integer ``n`` multiplies by repeated squaring, as the
  builder's ``(^)``; ``v.pow_t(y)`` is ``exp(log v * y)``, the default of
  ``(**)``; ``pow_(v, y)`` is the ``Pow`` node (``(^/)``);
* comparisons give ``bool`` values; ``select(c, a, b)`` is ``Arith Select``.

``OM.to_text()`` serialises the machine in the line format that
``om_create_graph`` (include/om_gb300.h) compiles into CUDA kernels.
"""
from __future__ import annotations

import math

TYPES = ("int", "float", "double", "bool")
Int, Float, Double, Bool = TYPES


class OMGraphError(ValueError):
    pass


class Static:
    def __init__(self, om: "OM", index: int, name: str, realm: str, typ: str):
        self.om, self.index, self.name, self.realm, self.type = om, index, name, realm, typ


class Value:
    """A node of a kernel's dataflow graph (realm 'array' or 'scalar')."""

    def __init__(self, kernel: "Kernel", node: int, realm: str, typ: str):
        self.k, self.node, self.realm, self.type = kernel, node, realm, typ

    # -- helpers
    def _lift(self, other) -> "Value":
        if isinstance(other, Value):
            if other.k is not self.k:
                raise OMGraphError("values of different kernels")
            return other
        return self.k.imm(other, self.type, self.realm)

    def _bin(self, op: str, other, rtype=None, swap=False) -> "Value":
        o = self._lift(other)
        a, b = (o, self) if swap else (self, o)
        if a.realm != b.realm:
            raise OMGraphError(f"{op}: realms differ ({a.realm}, {b.realm}); use broadcast")
        if a.type != b.type:
            raise OMGraphError(f"{op}: types differ ({a.type}, {b.type}); use cast")
        return self.k._arith(op, rtype or a.type, a.realm, [a, b])

    # -- arithmetic (Additive, Ring, Field, IntegralDomain)
    def __add__(self, o): return self._bin("add", o)
    def __radd__(self, o): return self._bin("add", o, swap=True)
    def __sub__(self, o): return self._bin("sub", o)
    def __rsub__(self, o): return self._bin("sub", o, swap=True)
    def __mul__(self, o): return self._bin("mul", o)
    def __rmul__(self, o): return self._bin("mul", o, swap=True)
    def __truediv__(self, o): return self._bin("div", o)
    def __rtruediv__(self, o): return self._bin("div", o, swap=True)
    def __floordiv__(self, o): return self._bin("div", o)     # IntegralDomain div
    def __mod__(self, o): return self._bin("mod", o)
    def __neg__(self): return self.k._arith("neg", self.type, self.realm, [self])

    def __pow__(self, n):
        """Integer power by repeated squaring, as the builder's (^)."""
        if not isinstance(n, int) or n < 0:
            raise OMGraphError("v ** n takes a non-negative int; use pow_t or pow_")
        if n == 0:
            return self.k.imm(1, self.type, self.realm)
        if n == 1:
            return self

        def f(x, m):
            if m == 1:
                return x
            h = m // 2
            y = f(x, h)
            sq = y * y
            return x * sq if m - 2 * h > 0 else sq
        return f(self, n)

    def pow_t(self, y) -> "Value":
        """(**) of the Transcendental class: exp (log x * y)."""
        return exp(log(self) * self._lift(y))

    # -- comparisons (bool results)
    def __lt__(self, o): return self._bin("lt", o, Bool)
    def __le__(self, o): return self._bin("le", o, Bool)
    def __gt__(self, o): return self._bin("gt", o, Bool)
    def __ge__(self, o): return self._bin("ge", o, Bool)
    def eq(self, o): return self._bin("eq", o, Bool)
    def ne(self, o): return self._bin("ne", o, Bool)

    # -- Boolean
    def __and__(self, o): return self._bin("and", o)
    def __or__(self, o): return self._bin("or", o)
    def __invert__(self): return self.k._arith("not", self.type, self.realm, [self])

    def __bool__(self):
        raise OMGraphError("an OM value has no truth value; use select")

    __hash__ = object.__hash__


def _unary(op):
    def f(v: Value) -> Value:
        return v.k._arith(op, v.type, v.realm, [v])
    f.__name__ = op
    return f


sqrt, exp, log, sin, cos, tan = (_unary(o) for o in ("sqrt", "exp", "log", "sin", "cos", "tan"))
asin, acos, atan = (_unary(o) for o in ("asin", "acos", "atan"))
abs_, signum, recip = _unary("abs"), _unary("signum"), _unary("inv")


def atan2(y: Value, x) -> Value:
    return y._bin("atan2", x)


def max_(a: Value, b) -> Value:
    return a._bin("max", b)


def min_(a: Value, b) -> Value:
    return a._bin("min", b)


def pow_(a: Value, b) -> Value:
    return a._bin("pow", b)


def select(c: Value, a, b) -> Value:
    """Arith Select.  Literal branches become imms of the other branch's type,
    or (both literal) int for Python ints and double otherwise."""
    if c.type != Bool:
        raise OMGraphError("select: condition must be bool")
    if not isinstance(a, Value) and not isinstance(b, Value):
        typ = Int if isinstance(a, int) and isinstance(b, int) else Double
        a = c.k.imm(a, typ, c.realm)
    ref = a if isinstance(a, Value) else b
    a, b = ref._lift(a), ref._lift(b)
    if a.type != b.type or not (c.realm == a.realm == b.realm):
        raise OMGraphError("select: branches must share type and realm with the condition")
    return c.k._arith("select", a.type, a.realm, [c, a, b])


def cast(v: Value, typ: str) -> Value:
    if typ not in TYPES:
        raise OMGraphError(f"unknown type {typ}")
    return v.k._arith("cast", typ, v.realm, [v])


class Kernel:
    def __init__(self, om: "OM", name: str):
        self.om, self.name = om, name
        self.lines: list[str] = []
        self.n = 0
        self.stores: set[str] = set()

    def _new(self, text: str, realm: str, typ: str) -> Value:
        node = self.n
        self.n += 1
        self.lines.append(f"{node} {text.split(' ', 1)[0]} {realm} {typ}"
                          + (" " + text.split(" ", 1)[1] if " " in text else ""))
        return Value(self, node, realm, typ)

    def _arith(self, op: str, typ: str, realm: str, args: list[Value]) -> Value:
        return self._new(op + " " + " ".join(str(a.node) for a in args), realm, typ)

    # -- builder verbs
    def load(self, s: Static) -> Value:
        return self._new(f"load {s.name}", s.realm, s.type)

    def store(self, s: Static, v) -> None:
        if not isinstance(v, Value):
            v = self.imm(v, s.type, s.realm)
        if v.realm != s.realm or v.type != s.type:
            raise OMGraphError(f"store {s.name}: {v.realm} {v.type} into {s.realm} {s.type}")
        self.lines.append(f"store {s.name} {v.node}")
        self.stores.add(s.name)

    def imm(self, x, typ: str, realm: str = "array") -> Value:
        if typ == Bool:
            lit = "1" if x else "0"
        elif typ == Int:
            if int(x) != x:
                raise OMGraphError(f"imm {x!r} is not an int")
            lit = str(int(x))
        else:
            lit = float(x).hex()
        return self._new(f"imm {lit}", realm, typ)

    def shift(self, v: Value, vec) -> Value:
        vec = tuple(int(a) for a in (vec if isinstance(vec, (tuple, list)) else (vec,)))
        if len(vec) != self.om.ndim or v.realm != "array":
            raise OMGraphError("shift: an array value and one offset per axis")
        return self._new(f"shift {v.node} " + " ".join(map(str, vec)), "array", v.type)

    def load_index(self, axis: int) -> Value:
        return self._new(f"loadindex {int(axis)}", "array", Int)

    def load_size(self, axis: int) -> Value:
        return self._new(f"loadsize {int(axis)}", "scalar", Int)

    def reduce(self, op: str, v: Value) -> Value:
        if op not in ("sum", "min", "max") or v.realm != "array":
            raise OMGraphError("reduce sum|min|max of an array value")
        return self._new(f"reduce {op} {v.node}", "scalar", v.type)

    def broadcast(self, v: Value) -> Value:
        if v.realm != "scalar":
            raise OMGraphError("broadcast of a scalar value")
        return self._new(f"broadcast {v.node}", "array", v.type)

    def bind(self, v: Value) -> Value:
        return v

    def manifest(self, v: Value) -> Value:
        """Anot.add Alloc.Manifest <?> v: the value is computed once per
        kernel run into an array that later uses read (at any shift), instead
        of being recomputed where it is used (Alloc.Delayed).  The values are
        the same either way."""
        if v.realm != "array":
            raise OMGraphError("manifest of an array value")
        self.lines.append(f"manifest {v.node}")
        return v

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


class OM:
    """An Orthotope Machine: statics and named kernels over an n-D mesh."""

    def __init__(self, name: str, size, boundary: str = "cyclic"):
        self.name = name
        self.size = tuple(int(s) for s in size)
        if not 1 <= len(self.size) <= 3 or min(self.size) < 1:
            raise OMGraphError("size: 1 to 3 positive extents")
        if boundary not in ("cyclic", "open"):
            raise OMGraphError("boundary: 'cyclic' or 'open'")
        self.boundary = boundary
        self.ndim = len(self.size)
        self.statics: list[Static] = []
        self.kernels: list[Kernel] = []

    def _static(self, name, realm, typ) -> Static:
        if typ not in TYPES:
            raise OMGraphError(f"unknown type {typ}")
        if any(s.name == name for s in self.statics):
            raise OMGraphError(f"duplicate static {name}")
        s = Static(self, len(self.statics), name, realm, typ)
        self.statics.append(s)
        return s

    def static_array(self, name: str, typ: str) -> Static:
        return self._static(name, "array", typ)

    def static_scalar(self, name: str, typ: str) -> Static:
        return self._static(name, "scalar", typ)

    def kernel(self, name: str) -> Kernel:
        k = Kernel(self, name)
        self.kernels.append(k)
        return k

    def to_text(self) -> str:
        out = [f"om {self.name} {self.ndim} " + " ".join(map(str, self.size)) + f" {self.boundary}"]
        out += [f"static {s.name} {s.realm} {s.type}" for s in self.statics]
        for k in self.kernels:
            out.append(f"kernel {k.name}")
            out += k.lines
            out.append("end")
        return "\n".join(out) + "\n"


PI = math.pi

_CTYPE = {Int: "int", Float: "float", Double: "double", Bool: "bool"}


def emit_header(om: OM) -> str:
    """The C++ class the reference's generator prints for this machine
    (Language/Paraiso/Generator/PlanTrans.hs:51-277): a default constructor,
    the om_size / om_memory_size / margin accessors, a reference accessor per
    Scalar static, a container and an element accessor per Array static and
    a method per kernel -- here over the C ABI, with the graph compiled for
    the GPU when the object is constructed (include/om_shim.hpp)."""
    idx = ", ".join(f"int i{a}" for a in range(om.ndim))
    args = ", ".join(f"i{a}" for a in range(om.ndim)) + (", 0" if om.ndim == 1 else "")
    arrays = [s for s in om.statics if s.realm == "array"]
    out = [f"// {om.name}.hpp -- generated from an omgraph machine; the GB300 runtime runs it.",
           "#pragma once", "", '#include "om_shim.hpp"', "",
           f"class {om.name} : public om_shim::machine {{", " public:"]
    init = "".join(f", {s.name}_(h_, \"{s.name}\")" for s in arrays)
    out.append(f"  {om.name}() : om_shim::machine(graph()){init} {{}}")
    out.append("")
    for s in om.statics:
        t = _CTYPE[s.type]
        if s.realm == "scalar":
            st = "int" if s.type == Bool else t
            out.append(f"  {st} &{s.name}() {{ return scalar<{st}>(\"{s.name}\"); }}")
        else:
            out.append(f"  om_shim::host_array<{t}> &{s.name}() {{ return {s.name}_; }}")
            out.append(f"  {t} &{s.name}({idx}) {{ return element<{t}>(\"{s.name}\", {args}); }}")
    out.append("")
    for k in om.kernels:
        out.append(f"  void {k.name}() {{ run(\"{k.name}\"); }}")
    out += ["", "  static const char *graph() {", '    return R"OMGRAPH(' + om.to_text() +
            ')OMGRAPH";', "  }", "", " private:"]
    for s in arrays:
        out.append(f"  om_shim::host_array<{_CTYPE[s.type]}> {s.name}_;")
    out.append("};")
    return "\n".join(out) + "\n"
