"""Builder of PC formula tapes (the node format of include/pirgpu.h, enum pc_kind).

lala-pc builds its PC propagators as trees of pc::Term and pc::Formula objects
(include/lala/terms.hpp, formula.hpp) through factory functions such as
Term::make_add or Formula::make_leq.  Here the same factories append nodes to
a flat tape, children before parents, and return the new node's index:

    t = Tape()
    x, y = t.var(0), t.var(1)
    t.prop(t.leq(t.add(x, y), t.constant(5)))     # x + y <= 5
    ctx.pc_tell(*t.arrays())

A tape is an int32 array of shape (n, 4): kind, a, b, c per node.
"""
import numpy as np

# terms (Term's alternatives, terms.hpp:572-589)
VAR, CONST, FORMULA, NEG, ABS, ADD, SUB, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, NADD, NMUL = range(16)
# formulas (Formula's alternatives, formula.hpp:905-920)
PVAR, NVAR, TRUE, FALSE, LEQ, GT, EQ, NEQ, AND, OR, EQUIV, IMPLY, XOR = range(16, 29)
ARG = 29
AE = 30  # a formula of the store itself (AbstractElement): items TELL / NTELL / ASK / NASK
TELL, NTELL, ASK, NASK, ASK_OUT, NASK_OUT = range(31, 37)
NUM_KINDS = 37
MAX_DEPTH = 64  # PC_MAX_DEPTH

TERMS = frozenset(range(0, 16))
FORMULAS = frozenset(list(range(16, 29)) + [AE])
ITEMS = frozenset(range(31, 37))
BINARY_TERMS = {ADD: "+", SUB: "-", MUL: "*", TDIV: "tdiv", FDIV: "fdiv", CDIV: "cdiv", EDIV: "ediv",
                MIN: "min", MAX: "max"}
NEGATED = {LEQ: GT, GT: LEQ, EQ: NEQ, NEQ: EQ}

INF = 2**31 - 1
MINF = -2**31


class Tape:
    """A growing tape of PC nodes and the roots of its propagators."""

    def __init__(self):
        self.nodes = []
        self.roots = []

    def _add(self, kind, a=0, b=0, c=0):
        self.nodes.append((kind, int(a), int(b), int(c)))
        return len(self.nodes) - 1

    def kind(self, n):
        return self.nodes[n][0]

    # -- terms ----------------------------------------------------------
    def var(self, x):
        return self._add(VAR, x)

    def constant(self, lb, ub=None):
        return self._add(CONST, lb, lb if ub is None else ub)

    def formula(self, f):
        """A formula used as a term: its truth value 0/1."""
        assert self.kind(f) in FORMULAS
        return self._add(FORMULA, f)

    def neg(self, t):
        return self._add(NEG, t)

    def abs(self, t):
        return self._add(ABS, t)

    def binary(self, kind, x, y):
        assert kind in BINARY_TERMS
        return self._add(kind, x, y)

    def add(self, x, y):
        return self._add(ADD, x, y)

    def sub(self, x, y):
        return self._add(SUB, x, y)

    def mul(self, x, y):
        return self._add(MUL, x, y)

    def tdiv(self, x, y):
        return self._add(TDIV, x, y)

    def fdiv(self, x, y):
        return self._add(FDIV, x, y)

    def cdiv(self, x, y):
        return self._add(CDIV, x, y)

    def ediv(self, x, y):
        return self._add(EDIV, x, y)

    def min(self, x, y):
        return self._add(MIN, x, y)

    def max(self, x, y):
        return self._add(MAX, x, y)

    def _nary(self, kind, terms):
        terms = list(terms)
        assert terms
        first = len(self.nodes)
        for t in terms:
            self._add(ARG, t)
        return self._add(kind, first, len(terms))

    def nadd(self, terms):
        return self._nary(NADD, terms)

    def nmul(self, terms):
        return self._nary(NMUL, terms)

    # -- formulas -------------------------------------------------------
    def pvar(self, x):
        return self._add(PVAR, x)

    def nvar(self, x):
        return self._add(NVAR, x)

    def true(self):
        return self._add(TRUE)

    def false(self):
        return self._add(FALSE)

    def leq(self, l, r):
        return self._add(LEQ, l, r)

    def gt(self, l, r):
        return self._add(GT, l, r)

    def eq(self, l, r):
        return self._add(EQ, l, r)

    def neq(self, l, r):
        return self._add(NEQ, l, r)

    def conj(self, f, g):
        return self._add(AND, f, g)

    def disj(self, f, g):
        return self._add(OR, f, g)

    def equiv(self, f, g):
        return self._add(EQUIV, f, g)

    def imply(self, f, g):
        return self._add(IMPLY, f, g)

    def xor(self, f, g):
        return self._add(XOR, f, g)

    def abstract_element(self, tell=(), not_tell=(), ask=(), not_ask=(), ask_out=(), not_ask_out=()):
        """A formula of the store itself (AbstractElement, formula.hpp:14-78):
        each list holds (var, lb, ub) items; ask = every `ask` item's variable
        inside its interval and every `ask_out` item's variable outside it,
        deduce = meet every `tell` item (nask / contradeduce: the `not_`
        lists)."""
        first = len(self.nodes)
        for kind, items in ((TELL, tell), (NTELL, not_tell), (ASK, ask), (NASK, not_ask), (ASK_OUT, ask_out),
                            (NASK_OUT, not_ask_out)):
            for v, lb, ub in items:
                self._add(kind, v, lb, ub)
        return self._add(AE, first, len(self.nodes) - first)

    # -- propagators ----------------------------------------------------
    def prop(self, f):
        assert self.kind(f) in FORMULAS
        self.roots.append(f)
        return f

    def arrays(self):
        """(tape (n, 4) int32, roots int32)."""
        t = np.array(self.nodes, np.int32).reshape(-1, 4)
        return t, np.array(self.roots, np.int32)
