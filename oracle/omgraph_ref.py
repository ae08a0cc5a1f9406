"""CPU oracle (test infrastructure) for Orthotope Machine graphs in the text
format of paraiso_gb300/omgraph.py: a numpy restatement of what the
reference's generator makes of an OM graph.

* Valid regions (Language/Paraiso/Optimization/BoundaryAnalysis.hs:33-94):
  Load -> the full array; Shift v -> the input's region moved by v, cut to
  the full array; Imm, LoadIndex, LoadSize, Reduce, Broadcast -> infinite;
  Arith -> intersection of its inputs; Store -> its input's region.
* Margins (Language/Paraiso/Generator/OMTrans.hs:103-120): open axes take the
  intersection of every array store's region; cyclic axes have none.
* A stored array is a manifest computed on its value's region and zero
  elsewhere, copied into the static when the kernel ends
  (PlanTrans.hs:243-258); loads inside a kernel see the statics as they
  were when it began.
* Reduce runs over the whole manifest (margins included), so cells outside
  the region contribute zeros (PlanTrans.hs:712-720).
* `shift v x` at cell c reads x[c - v] (PlanTrans.hs:561-562); LoadIndex
  is the memory coordinate minus the lower margin, wrapped on cyclic axes
  (PlanTrans.hs:455-466).
* Arithmetic follows C on the OM's types (int32 wraps, integer division
  truncates, std::max/std::min argument order).
"""
from __future__ import annotations

import math

import numpy as np

NP = {"int": np.int32, "float": np.float32, "double": np.float64, "bool": np.bool_}
INF = None  # an open end of an interval


def parse(text: str) -> dict:
    lines = [l.split() for l in text.splitlines() if l.strip() and not l.startswith("#")]
    head = lines[0]
    assert head[0] == "om"
    ndim = int(head[2])
    om = {"name": head[1], "ndim": ndim, "size": tuple(int(x) for x in head[3:3 + ndim]),
          "boundary": head[3 + ndim], "statics": {}, "order": [], "kernels": {}}
    cur = None
    for w in lines[1:]:
        if w[0] == "static":
            om["statics"][w[1]] = (w[2], w[3])
            om["order"].append(w[1])
        elif w[0] == "kernel":
            cur = []
            om["kernels"][w[1]] = cur
        elif w[0] == "end":
            cur = None
        elif w[0] == "manifest":
            continue   # an allocation choice: the values are the same
        else:
            cur.append(w)
    return om


# a region: per axis (lo, hi); lo = None (-inf) or offset from the lower
# edge, hi = None (+inf) or offset from the upper edge (<= 0 when cut)
def _full(nd):
    return tuple((0, 0) for _ in range(nd))


def _inf(nd):
    return tuple((INF, INF) for _ in range(nd))


def _meet(a, b):
    out = []
    for (l1, h1), (l2, h2) in zip(a, b):
        lo = l2 if l1 is INF else (l1 if l2 is INF else max(l1, l2))
        hi = h2 if h1 is INF else (h1 if h2 is INF else min(h1, h2))
        out.append((lo, hi))
    return tuple(out)


def _shift(reg, vec):
    moved = tuple((None if lo is INF else lo + v, None if hi is INF else hi + v)
                  for (lo, hi), v in zip(reg, vec))
    return _meet(moved, _full(len(vec)))


def regions(om: dict, kernel) -> dict:
    nd = om["ndim"]
    reg = {}
    for w in kernel:
        if w[0] == "store":
            continue
        node, op = int(w[0]), w[1]
        args = w[4:]
        if op in ("imm", "loadindex", "loadsize", "reduce", "broadcast") or w[2] == "scalar":
            reg[node] = _inf(nd)
        elif op == "load":
            reg[node] = _full(nd)
        elif op == "shift":
            reg[node] = _shift(reg[int(args[0])], [int(x) for x in args[1:]])
        else:
            r = _inf(nd)
            for a in args:
                r = _meet(r, reg[int(a)])
            reg[node] = r
    return reg


def margins(om: dict):
    nd = om["ndim"]
    if om["boundary"] == "cyclic":
        return [0] * nd, [0] * nd
    united = _inf(nd)
    for kern in om["kernels"].values():
        reg = regions(om, kern)
        for w in kern:
            if w[0] == "store" and om["statics"][w[1]][0] == "array":
                united = _meet(united, reg[int(w[2])])
    lower = [0 if lo is INF else lo for lo, _ in united]
    upper = [0 if hi is INF else -hi for _, hi in united]
    return lower, upper


class Machine:
    """Statics of an OM graph in memory-sized numpy arrays ([.., y, x])."""

    def __init__(self, text: str):
        self.om = parse(text)
        self.lm, self.um = margins(self.om)
        self.ms = [n + a + b for n, a, b in zip(self.om["size"], self.lm, self.um)]
        self.shape = tuple(reversed(self.ms))
        self.values = {}
        for name in self.om["order"]:
            realm, typ = self.om["statics"][name]
            self.values[name] = (np.zeros(self.shape, NP[typ]) if realm == "array"
                                 else NP[typ](0))

    def _mask(self, reg):
        m = np.ones(self.shape, bool)
        if self.om["boundary"] == "cyclic":
            return m   # cyclic axes: every cell is computed (OMTrans.hs:103-116)
        for ax, (lo, hi) in enumerate(reg):
            n = self.ms[ax]
            a = 0 if lo is INF else lo
            b = n if hi is INF else n + hi
            idx = np.arange(n)
            sel = (idx >= a) & (idx < b)
            shape = [1] * len(self.shape)
            shape[len(self.shape) - 1 - ax] = n
            m &= sel.reshape(shape)
        return m

    def run(self, kname: str) -> None:
        om = self.om
        kern = om["kernels"][kname]
        reg = regions(om, kern)
        val = {}
        new = {}
        with np.errstate(all="ignore"):
            for w in kern:
                if w[0] == "store":
                    name, v = w[1], val[int(w[2])]
                    realm, typ = om["statics"][name]
                    if realm == "array":
                        m = self._mask(reg[int(w[2])])
                        new[name] = np.where(m, np.broadcast_to(v, self.shape), 0).astype(NP[typ])
                    else:
                        new[name] = NP[typ](v)
                    continue
                node, op, realm, typ = int(w[0]), w[1], w[2], w[3]
                args = w[4:]
                t = NP[typ]
                a = [val[int(x)] for x in args] if op not in (
                    "load", "imm", "loadindex", "loadsize", "shift", "reduce") else None
                if op == "load":
                    r = self.values[args[0]]
                    r = r.copy() if realm == "array" else r
                elif op == "imm":
                    lit = args[0]
                    x = float.fromhex(lit) if typ in ("float", "double") else int(lit)
                    r = np.full(self.shape, x, t) if realm == "array" else t(x)
                elif op == "loadindex":
                    ax = int(args[0])
                    idx = np.arange(self.ms[ax], dtype=np.int64) - self.lm[ax]
                    shape = [1] * len(self.shape)
                    shape[len(self.shape) - 1 - ax] = self.ms[ax]
                    r = np.broadcast_to(idx.reshape(shape), self.shape).astype(np.int32)
                elif op == "loadsize":
                    r = np.int32(om["size"][int(args[0])])
                elif op == "shift":
                    x = val[int(args[0])]
                    r = x
                    for ax, v in enumerate(int(s) for s in args[1:]):
                        # shift v reads x[c - v]; out-of-array cells lie
                        # outside the region (open) or wrap (cyclic)
                        r = np.roll(r, v, axis=len(self.shape) - 1 - ax)
                elif op == "reduce":
                    x = val[int(args[1])]
                    m = self._mask(reg[int(args[1])])
                    man = np.where(m, x, 0).astype(t)
                    if args[0] == "sum":
                        if typ in ("float", "double"):
                            r = t(math.fsum(man.astype(np.float64).ravel()))
                        else:
                            r = t(man.astype(np.int64).sum())
                    elif args[0] == "min":
                        r = man.min()
                    else:
                        r = man.max()
                elif op == "broadcast":
                    r = np.full(self.shape, val[int(args[0])], t)
                else:
                    r = _arith(op, t, typ, a)
                if realm == "array" and np.ndim(r) == 0:
                    r = np.full(self.shape, r, t)
                val[node] = r
        self.values.update(new)


def _cdiv(a, b, t):
    if np.issubdtype(t, np.integer):
        a64, b64 = np.asarray(a, np.int64), np.asarray(b, np.int64)
        q = np.abs(a64) // np.abs(b64)
        return (np.where((a64 < 0) ^ (b64 < 0), -q, q)).astype(t)
    return (np.asarray(a, t) / np.asarray(b, t)).astype(t)


def _arith(op, t, typ, a):
    f = {
        "add": lambda x, y: x + y, "sub": lambda x, y: x - y, "mul": lambda x, y: x * y,
        "neg": lambda x: -x, "not": lambda x: np.logical_not(x),
        "and": lambda x, y: np.logical_and(x, y), "or": lambda x, y: np.logical_or(x, y),
        "eq": lambda x, y: x == y, "ne": lambda x, y: x != y, "lt": lambda x, y: x < y,
        "le": lambda x, y: x <= y, "gt": lambda x, y: x > y, "ge": lambda x, y: x >= y,
        "select": lambda c, x, y: np.where(c, x, y),
        "max": lambda x, y: np.where(x < y, y, x), "min": lambda x, y: np.where(y < x, y, x),
        "abs": np.abs, "signum": np.sign, "sqrt": np.sqrt, "exp": np.exp, "log": np.log,
        "sin": np.sin, "cos": np.cos, "tan": np.tan, "asin": np.arcsin, "acos": np.arccos,
        "atan": np.arctan, "atan2": np.arctan2, "pow": np.power,
    }
    if op == "div":
        return _cdiv(a[0], a[1], t)
    if op == "inv":
        return _cdiv(t(1), a[0], t)
    if op == "mod":
        x, y = np.asarray(a[0], np.int64), np.asarray(a[1], np.int64)
        return (x - _cdiv(x, y, np.int64) * y).astype(t)
    if op == "cast":
        x = np.asarray(a[0])
        if np.issubdtype(t, np.integer) and x.dtype.kind == "f":
            return np.trunc(x).astype(t)
        return x.astype(t)
    return np.asarray(f[op](*a)).astype(t)
