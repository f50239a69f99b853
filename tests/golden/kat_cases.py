"""Known-answer cases of lala-pc's PIR tests (tests/pir_test.cpp), as instances.

Each case states the variables, the ternary propagators and, per step, the
bounds the reference test expects before and after the Gauss-Seidel fixpoint
(`deduce_and_test`, tests/pir_test.cpp:54-73), whether the store must fail
(`deduce_and_test_bot`, :75-89) and whether the element is extractable (every
propagator entailed and not failed; `test_extract`, :31-52).

The reference builds its instances from FlatZinc through lala-core's
ternarizer (not vendored).  Here each formula is written directly as PIR
propagators `x = y <op> z`; constants become singleton variables, `a - b` is
ADD with permuted roles (`a = t + b`), `-a` is MUL by the constant -1, a
strict comparison is a reified LEQ with a false constant, and boolean
and/or/not are MIN/MAX/ADD over 0/1 variables.  The propagator count is the
one the reference test asserts wherever that decomposition has the same size
(`num`); only the bounds of the variables the test names are compared.

Expected values are transcribed from the test source (file:line on each case).
Cases that need lala-core's set/element ternarization (ReifiedIn :190-211,
ElementConstraint1 :569-582, InConstraint1 :608-623) are not reproduced.
"""

INF = 2**31 - 1
MINF = -2**31
TOP = (MINF, INF)

ADD, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, EQ, LEQ = range(10)
OPNAMES = ["ADD", "MUL", "TDIV", "FDIV", "CDIV", "EDIV", "MIN", "MAX", "EQ", "LEQ"]


class Model:
    """Variables (name -> index, initial bounds) and propagators."""

    def __init__(self):
        self.names, self.lb, self.ub, self.props = [], [], [], []
        self.index = {}

    def var(self, name, lb=MINF, ub=INF):
        self.index[name] = len(self.names)
        self.names.append(name)
        self.lb.append(lb)
        self.ub.append(ub)
        return name

    def c(self, v):
        """Singleton variable holding the constant v (a ternarizer constant)."""
        name = "__C%d" % v
        if name not in self.index:
            self.var(name, v, v)
        return name

    def fresh(self, lb=MINF, ub=INF):
        return self.var("__T%d" % len(self.names), lb, ub)

    def prop(self, op, x, y, z):
        self.props.append((op, x, y, z))


class Step:
    def __init__(self, num, before, after=None, ua=False, bot=False, bounds=(), props=()):
        self.num = num              # expected number of propagators
        self.before = before        # bounds of the first len(before) vars
        self.after = before if after is None else after
        self.ua = ua                # extractable after the fixpoint
        self.bot = bot              # the fixpoint must fail
        self.bounds = list(bounds)  # tells before this step: (var, lb, ub) meets
        self.props = list(props)    # tells before this step: new propagators


class Case:
    def __init__(self, name, ref, build, steps):
        self.name, self.ref, self.build, self.steps = name, ref, build, steps


CASES = []


def case(name, ref, steps):
    def deco(fn):
        CASES.append(Case(name, ref, fn, steps))
        return fn
    return deco


# ---------------------------------------------------------------- linear ----
@case("TernaryProblem", "tests/pir_test.cpp:175-182",
      [Step(1, [(0, 10), (0, 10), (5, 5)], [(0, 5), (0, 5), (5, 5)])])
def _(m):
    m.var("x", 0, 10); m.var("y", 0, 10); m.var("z", 5, 5)
    m.prop(ADD, "z", "x", "y")


@case("ReifiedEquality", "tests/pir_test.cpp:184-188",
      [Step(1, [(0, 1), TOP])])
def _(m):
    m.var("x"); m.var("y")
    m.prop(EQ, "x", "y", m.c(2))


@case("AddEquality", "tests/pir_test.cpp:213-220",
      [Step(1, [(0, 10), (0, 10)], [(0, 5), (0, 5)])])
def _(m):
    m.var("x", 0, 10); m.var("y", 0, 10)
    m.prop(ADD, m.c(5), "x", "y")


@case("TemporalConstraint1Flat", "tests/pir_test.cpp:222-230",
      [Step(1, [(0, 10), (0, 10), (MINF, 5)], [(0, 5), (0, 5), (0, 5)])])
def _(m):
    m.var("x", 0, 10); m.var("y", 0, 10); m.var("z", MINF, 5)
    m.prop(ADD, "z", "x", "y")


def _sum_le(lo, hi, bound_lb, bound_ub):
    def build(m):
        m.var("x", lo, hi); m.var("y", lo, hi)
        t = m.fresh(bound_lb, bound_ub)
        m.prop(ADD, t, "x", "y")
    return build


for _name, _ref, _lo, _hi, _blb, _bub, _after, _ua in [
    ("TemporalConstraint1", ":232-238", 0, 10, MINF, 5, [(0, 5), (0, 5)], False),
    ("TemporalConstraint2", ":241-247", 0, 10, 6, INF, None, False),
    ("TemporalConstraint3", ":250-256", 0, 3, 6, INF, [(3, 3), (3, 3)], True),
    ("TemporalConstraint4", ":259-265", 0, 3, 5, INF, [(2, 3), (2, 3)], False),
    ("TemporalConstraint5", ":268-274", 0, 4, 5, 5, [(1, 4), (1, 4)], False),
]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _sum_le(_lo, _hi, _blb, _bub),
                      [Step(1, [(_lo, _hi), (_lo, _hi)], _after, _ua)]))


def _diff(bound_lb, bound_ub):
    def build(m):
        m.var("x", 0, 10); m.var("y", 0, 10)
        t = m.fresh(bound_lb, bound_ub)      # t = x - y, i.e. x = t + y
        m.prop(ADD, "x", t, "y")
    return build


for _name, _ref, _blb, _bub, _after, _ua in [
    ("TemporalConstraint6", ":276-283", MINF, 5, None, False),
    ("TemporalConstraint7", ":285-292", MINF, -10, [(0, 0), (10, 10)], True),
    ("TemporalConstraint8", ":294-301", 5, INF, [(5, 10), (0, 5)], False),
    ("TemporalConstraint9", ":303-310", MINF, -5, [(0, 5), (5, 10)], False),
]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _diff(_blb, _bub),
                      [Step(1, [(0, 10), (0, 10)], _after, _ua)]))


@case("TemporalConstraint10", "tests/pir_test.cpp:312-319",
      [Step(2, [(0, 10), (0, 10)], [(0, 5), (5, 10)])])
def _(m):
    m.var("x", 0, 10); m.var("y", 0, 10)
    t = m.fresh()
    m.prop(ADD, t, m.c(-5), "y")          # t = -5 + y
    m.prop(LEQ, m.c(1), "x", t)           # x <= t


def _sum3(lo, hi, bound):
    def build(m):
        m.var("x", lo, hi); m.var("y", lo, hi); m.var("z", lo, hi)
        t1 = m.fresh()
        t2 = m.fresh(MINF, bound)
        m.prop(ADD, t1, "x", "y")
        m.prop(ADD, t2, t1, "z")
    return build


CASES.append(Case("TopProp", "tests/pir_test.cpp:321-329", _sum3(3, 10, 8),
                  [Step(2, [(3, 10)] * 3, bot=True)]))
CASES.append(Case("TernaryAdd2", "tests/pir_test.cpp:331-339", _sum3(3, 10, 9),
                  [Step(2, [(3, 10)] * 3, [(3, 3)] * 3, True)]))
CASES.append(Case("TernaryAdd3", "tests/pir_test.cpp:341-349", _sum3(3, 10, 10),
                  [Step(2, [(3, 10)] * 3, [(3, 4)] * 3)]))
CASES.append(Case("TernaryAdd4", "tests/pir_test.cpp:351-359", _sum3(-2, 2, -5),
                  [Step(2, [(-2, 2)] * 3, [(-2, -1)] * 3)]))


def _pb(cx, cy, cz):
    """cx*x + cy*y + cz*z <= 2 over booleans; coefficient 1 is not multiplied."""
    def build(m):
        for v in "xyz":
            m.var(v, 0, 1)
        terms = []
        for coef, v in ((cx, "x"), (cy, "y"), (cz, "z")):
            if coef == 1:
                terms.append(v)
            elif coef == -1:
                t = m.fresh(); m.prop(MUL, t, m.c(-1), v); terms.append(t)
            else:
                t = m.fresh(); m.prop(MUL, t, m.c(coef), v); terms.append(t)
        a1 = m.fresh()
        m.prop(ADD, a1, terms[0], terms[1])
        a2 = m.fresh(MINF, 2)
        m.prop(ADD, a2, a1, terms[2])
    return build


CASES.append(Case("PseudoBoolean1", "tests/pir_test.cpp:361-369", _pb(2, 1, 3),
                  [Step(4, [(0, 1)] * 3, [(0, 1), (0, 1), (0, 0)])]))
CASES.append(Case("PseudoBoolean2", "tests/pir_test.cpp:371-383", _pb(2, 5, 3),
                  [Step(5, [(0, 1)] * 3, [(0, 1), (0, 0), (0, 0)])]))
CASES.append(Case("PseudoBoolean3", "tests/pir_test.cpp:385-393", _pb(3, 5, 3),
                  [Step(5, [(0, 1)] * 3, [(0, 0)] * 3, True)]))
CASES.append(Case("PseudoBoolean4", "tests/pir_test.cpp:395-403", _pb(-1, 1, 3),
                  [Step(4, [(0, 1)] * 3)]))


def _neg(xlo, xhi, yv, rel):
    """-x rel y with y a fixed variable; rel in {le, ge, gt}."""
    def build(m):
        m.var("x", xlo, xhi); m.var("y", yv, yv)
        n = m.fresh()
        m.prop(MUL, n, m.c(-1), "x")
        if rel == "le":
            m.prop(LEQ, m.c(1), n, "y")
        elif rel == "ge":
            m.prop(LEQ, m.c(1), "y", n)
        else:  # n > y  <=>  not (n <= y)
            m.prop(LEQ, m.c(0), n, "y")
    return build


for _name, _ref, _xlo, _xhi, _yv, _rel, _after, _bot in [
    ("NegationOp1", ":405-413", -4, 3, 2, "le", [(-2, 3), (2, 2)], False),
    ("NegationOp2", ":415-423", -4, 3, -2, "le", [(2, 3), (-2, -2)], False),
    ("NegationOp3", ":425-433", 0, 3, -2, "le", [(2, 3), (-2, -2)], False),
    ("NegationOp4", ":435-443", -4, -3, 4, "le", None, False),
    ("NegationOp5", ":445-453", -4, 3, -2, "ge", [(-4, 2), (-2, -2)], False),
    ("NegationOp6", ":455-463", -4, 3, 2, "gt", [(-4, -3), (2, 2)], False),
    ("NegationOp7", ":465-473", -4, 3, 5, "ge", None, True),
]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _neg(_xlo, _xhi, _yv, _rel),
                      [Step(2, [(_xlo, _xhi), (_yv, _yv)], _after, bot=_bot)]))


def _resource(xlo, xhi, ylo, yhi, k1, k2):
    """b <=> (x - y <= k1 /\\ y - x <= k2)."""
    def build(m):
        m.var("x", xlo, xhi); m.var("y", ylo, yhi); m.var("b", 0, 1)
        t1, r1, t2, r2 = m.fresh(), m.fresh(), m.fresh(), m.fresh()
        m.prop(ADD, "x", t1, "y")          # t1 = x - y
        m.prop(LEQ, r1, t1, m.c(k1))
        m.prop(ADD, "y", t2, "x")          # t2 = y - x
        m.prop(LEQ, r2, t2, m.c(k2))
        m.prop(MIN, "b", r1, r2)           # b = r1 /\ r2
    return build


CASES.append(Case("ResourceConstraint1", "tests/pir_test.cpp:475-487",
                  _resource(5, 10, 9, 15, 0, 2),
                  [Step(5, [(5, 10), (9, 15), (0, 1)]),
                   Step(5, [(5, 10), (9, 15), (1, 1)], [(7, 10), (9, 12), (1, 1)],
                        bounds=[("b", 1, 1)])]))
CASES.append(Case("ResourceConstraint2", "tests/pir_test.cpp:489-500",
                  _resource(1, 2, 0, 2, 2, -1),
                  [Step(5, [(1, 2), (0, 2), (0, 1)]),
                   Step(5, [(1, 2), (0, 2), (0, 0)], [(1, 2), (1, 2), (0, 0)],
                        bounds=[("b", 0, 0)])]))


@case("Strict1", "tests/pir_test.cpp:502-506", [Step(1, [(1, 10)], bot=True)])
def _(m):
    m.var("x", 1, 10); m.var("y", 10, 10)
    m.prop(LEQ, m.c(0), "x", "y")          # x > y  <=>  not (x <= y)


@case("Strict2", "tests/pir_test.cpp:508-512", [Step(1, [(1, 10)], [(1, 9)], True)])
def _(m):
    m.var("x", 1, 10); m.var("y", 10, 10)
    m.prop(LEQ, m.c(0), "y", "x")          # x < y  <=>  not (y <= x)


@case("Strict3", "tests/pir_test.cpp:514-518", [Step(5, [(1, 10)], [(1, 9)], True)])
def _(m):
    m.var("x", 1, 10); m.var("y", 10, 10)
    nb1, b1, nb2, b2 = m.fresh(), m.fresh(), m.fresh(), m.fresh()
    m.prop(LEQ, nb1, "y", "x")             # nb1 = (y <= x), b1 = x < y = 1 - nb1
    m.prop(ADD, m.c(1), b1, nb1)
    m.prop(LEQ, nb2, "x", "y")             # nb2 = (x <= y), b2 = x > y = 1 - nb2
    m.prop(ADD, m.c(1), b2, nb2)
    m.prop(MAX, m.c(1), b1, b2)            # b1 \/ b2


def _eq(xlo, xhi, ylo, yhi):
    def build(m):
        m.var("x", xlo, xhi); m.var("y", ylo, yhi)
        m.prop(EQ, m.c(1), "x", "y")
    return build


for _name, _ref, _y, _after in [
    ("EqualConstraint1", ":520-524", (9, 10), [(9, 10), (9, 10)]),
    ("EqualConstraint2", ":526-530", (1, 2), [(1, 2), (1, 2)]),
    ("EqualConstraint3", ":532-536", (0, 11), [(1, 10), (1, 10)]),
    ("EqualConstraint4", ":538-542", (5, 11), [(5, 10), (5, 10)]),
]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _eq(1, 10, *_y),
                      [Step(1, [(1, 10), _y], _after)]))


def _ne(yv):
    def build(m):
        m.var("x", 1, 10); m.var("y", yv, yv)
        m.prop(EQ, m.c(0), "x", "y")
    return build


def _ne_const(m):
    m.var("x", 1, 10)
    m.prop(EQ, m.c(0), "x", m.c(10))


CASES.append(Case("NotEqualConstraint1", "tests/pir_test.cpp:544-548", _ne_const,
                  [Step(1, [(1, 10)], [(1, 9)], True)]))
CASES.append(Case("NotEqualConstraint2", "tests/pir_test.cpp:550-554", _ne(10),
                  [Step(1, [(1, 10), (10, 10)], [(1, 9), (10, 10)], True)]))
CASES.append(Case("NotEqualConstraint3", "tests/pir_test.cpp:556-560", _ne(1),
                  [Step(1, [(1, 10), (1, 1)], [(2, 10), (1, 1)], True)]))
CASES.append(Case("NotEqualConstraint4", "tests/pir_test.cpp:562-566", _ne_const,
                  [Step(1, [(1, 10)], [(1, 9)], True)]))


def _xor(lo, hi):
    def build(m):
        m.var("x", lo, hi); m.var("y", lo, hi)
        b1, b2 = m.fresh(), m.fresh()
        m.prop(EQ, b1, "x", m.c(5))
        m.prop(EQ, b2, "y", m.c(5))
        m.prop(ADD, m.c(1), b1, b2)       # b1 xor b2
    return build


CASES.append(Case("XorConstraint1", "tests/pir_test.cpp:585-594", _xor(MINF, INF),
                  [Step(3, [TOP, TOP]),
                   Step(3, [(1, 1), TOP], [(1, 1), (5, 5)], True, bounds=[("x", 1, 1)])]))
CASES.append(Case("XorConstraint2", "tests/pir_test.cpp:596-605", _xor(1, 5),
                  [Step(3, [(1, 5), (1, 5)]),
                   Step(3, [(1, 5), (5, 5)], [(1, 4), (5, 5)], True, bounds=[("y", 5, 5)])]))


# ------------------------------------------------------------- min / max ----
def _minmax(op):
    def build(m):
        m.var("x", 0, 4); m.var("y", 2, 5); m.var("z", 0, 10)
        m.prop(op, "z", "x", "y")
    return build


CASES.append(Case("MinConstraint1", "tests/pir_test.cpp:625-640", _minmax(MIN), [
    Step(1, [(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (0, 4)]),
    Step(1, [(0, 4), (2, 5), (0, 3)], bounds=[("z", MINF, 3)]),
    Step(1, [(0, 1), (2, 5), (0, 3)], [(0, 1), (2, 5), (0, 1)], bounds=[("x", MINF, 1)]),
    Step(1, [(0, 0), (2, 5), (0, 1)], [(0, 0), (2, 5), (0, 0)], True, bounds=[("x", MINF, 0)]),
]))
CASES.append(Case("MinConstraint2", "tests/pir_test.cpp:642-654", _minmax(MIN), [
    Step(1, [(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (0, 4)]),
    Step(1, [(0, 4), (2, 5), (0, 3)], bounds=[("z", MINF, 3)]),
    Step(1, [(4, 4), (2, 5), (0, 3)], [(4, 4), (2, 3), (2, 3)], bounds=[("x", 4, 4)]),
]))
CASES.append(Case("MaxConstraint1", "tests/pir_test.cpp:670-685", _minmax(MAX), [
    Step(1, [(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (2, 5)]),
    Step(1, [(0, 4), (2, 5), (2, 3)], [(0, 3), (2, 3), (2, 3)], bounds=[("z", MINF, 3)]),
    Step(1, [(0, 1), (2, 3), (2, 3)], bounds=[("x", MINF, 1)]),
    Step(1, [(0, 1), (2, 2), (2, 3)], [(0, 1), (2, 2), (2, 2)], True, bounds=[("y", 2, 2)]),
]))
CASES.append(Case("MaxConstraint2", "tests/pir_test.cpp:687-696", _minmax(MAX), [
    Step(1, [(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (2, 5)]),
    Step(1, [(0, 4), (2, 5), (5, 5)], [(0, 4), (5, 5), (5, 5)], True, bounds=[("z", 5, INF)]),
]))


@case("MinConstraint3", "tests/pir_test.cpp:656-668", [
    Step(1, [TOP, (0, 1), (0, 1)], [TOP, (1, 1), (1, 1)], True),
    Step(2, [TOP, (1, 1), (1, 1)], [(MINF, 5), (1, 1), (1, 1)], True,
         props=[(LEQ, "b1", "x", "__C5")]),
    Step(3, [(MINF, 5), (1, 1), (1, 1)], [(5, 5), (1, 1), (1, 1)], True,
         props=[(LEQ, "b2", "__C5", "x")]),
])
def _(m):
    m.var("x"); m.var("b1", 0, 1); m.var("b2", 0, 1)
    m.prop(MIN, m.c(1), "b1", "b2")
    m.c(5)


@case("MaxConstraint3", "tests/pir_test.cpp:698-709", [
    Step(1, [TOP, (0, 1), (0, 1)], [TOP, (0, 0), (0, 0)], True),
    Step(2, [TOP, (0, 0), (0, 0)], [(6, INF), (0, 0), (0, 0)], True,
         props=[(LEQ, "b1", "x", "__C5")]),
    Step(3, [(6, INF), (0, 0), (0, 0)], [(6, 6), (0, 0), (0, 0)], True,
         props=[(LEQ, "b2", "__C7", "x")]),
])
def _(m):
    m.var("x"); m.var("b1", 0, 1); m.var("b2", 0, 1)
    m.prop(MAX, m.c(0), "b1", "b2")
    m.c(5); m.c(7)


# --------------------------------------------------------- bool clauses ----
def _clause(m):
    """bool_clause([x1, x2], [y1, y2]): x1 \\/ x2 \\/ not y1 \\/ not y2."""
    for v in ("x1", "x2", "y1", "y2"):
        m.var(v, 0, 1)
    ny1, ny2, m1, m2 = m.fresh(), m.fresh(), m.fresh(), m.fresh()
    m.prop(ADD, m.c(1), ny1, "y1")
    m.prop(ADD, m.c(1), ny2, "y2")
    m.prop(MAX, m1, "x1", "x2")
    m.prop(MAX, m2, ny1, ny2)
    m.prop(MAX, m.c(1), m1, m2)


B4 = [(0, 1)] * 4
CASES.append(Case("BooleanClause1", "tests/pir_test.cpp:711-719", _clause, [
    Step(5, B4),
    Step(5, [(1, 1), (0, 1), (0, 1), (0, 1)], bounds=[("x1", 1, 1)])]))
CASES.append(Case("BooleanClause2", "tests/pir_test.cpp:721-729", _clause, [
    Step(5, B4),
    Step(5, [(0, 1), (0, 1), (0, 0), (0, 1)], bounds=[("y1", 0, 0)])]))
CASES.append(Case("BooleanClause3", "tests/pir_test.cpp:731-743", _clause, [
    Step(5, B4),
    Step(5, [(0, 0), (0, 1), (0, 1), (0, 1)], bounds=[("x1", 0, 0)]),
    Step(5, [(0, 0), (0, 0), (0, 1), (0, 1)], bounds=[("x2", 0, 0)]),
    Step(5, [(0, 0), (0, 0), (1, 1), (0, 1)], [(0, 0), (0, 0), (1, 1), (0, 0)], True,
         bounds=[("y1", 1, 1)])]))
CASES.append(Case("BooleanClause4", "tests/pir_test.cpp:745-757", _clause, [
    Step(5, B4),
    Step(5, [(0, 0), (0, 1), (0, 1), (0, 1)], bounds=[("x1", 0, 0)]),
    Step(5, [(0, 0), (0, 1), (1, 1), (0, 1)], bounds=[("y1", 1, 1)]),
    Step(5, [(0, 0), (0, 1), (1, 1), (1, 1)], [(0, 0), (1, 1), (1, 1), (1, 1)], True,
         bounds=[("y2", 1, 1)])]))


# ------------------------------------------------------------ int_times ----
def _times(x, y, z):
    def build(m):
        m.var("x", *x); m.var("y", *y); m.var("z", *z)
        m.prop(MUL, "z", "x", "y")         # int_times(x, y, z): z = x * y
    return build


B3 = [(0, 1)] * 3
CASES.append(Case("IntTimes1", "tests/pir_test.cpp:759-771", _times((0, 1), (0, 1), (0, 1)), [
    Step(1, B3),
    Step(1, [(1, 1), (0, 1), (0, 1)], bounds=[("x", 1, 1)]),
    Step(1, [(1, 1), (1, 1), (0, 1)], [(1, 1)] * 3, True, bounds=[("y", 1, 1)])]))
CASES.append(Case("IntTimes2", "tests/pir_test.cpp:773-783", _times((0, 1), (0, 1), (0, 1)), [
    Step(1, B3),
    Step(1, [(0, 1), (0, 1), (1, 1)], [(1, 1)] * 3, True, bounds=[("z", 1, 1)])]))
CASES.append(Case("IntTimes3", "tests/pir_test.cpp:785-793", _times((0, 0), (0, 1), (0, 1)), [
    Step(1, [(0, 0), (0, 1), (0, 1)], [(0, 0), (0, 1), (0, 0)], True)]))
CASES.append(Case("IntTimes4", "tests/pir_test.cpp:795-803", _times((0, 1), (0, 0), (0, 1)), [
    Step(1, [(0, 1), (0, 0), (0, 1)], [(0, 1), (0, 0), (0, 0)], True)]))
CASES.append(Case("IntTimes5", "tests/pir_test.cpp:805-813", _times((1, 2), (0, 1), (0, 0)), [
    Step(1, [(1, 2), (0, 1), (0, 0)], [(1, 2), (0, 0), (0, 0)], True)]))
CASES.append(Case("IntTimes6", "tests/pir_test.cpp:815-823", _times((0, 1), (1, 2), (0, 0)), [
    Step(1, [(0, 1), (1, 2), (0, 0)], [(0, 0), (1, 2), (0, 0)], True)]))


# ------------------------------------------------------------- division ----
@case("IntDiv1", "tests/pir_test.cpp:825-835", [
    Step(1, B3, [(0, 1), (1, 1), (0, 1)]),
    Step(1, [(1, 1), (1, 1), (0, 1)], [(1, 1)] * 3, True, bounds=[("x", 1, 1)])])
def _(m):
    m.var("x", 0, 1); m.var("y", 0, 1); m.var("z", 0, 1)
    m.prop(TDIV, "z", "x", "y")            # int_div(x, y, z): z = x / y


def _div0y2(op):
    def build(m):
        m.var("y", 0, 1)
        m.prop(op, m.c(0), "y", m.c(2))    # int_?div(y, 2, 0): 0 = y / 2
    return build


for _name, _ref, _op in [("IntTDiv0y2", ":837-845", TDIV), ("IntFDiv0y2", ":847-855", FDIV),
                         ("IntEDiv0y2", ":857-865", EDIV)]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _div0y2(_op), [
        Step(1, [(0, 1)]),
        Step(1, [(1, 1)], ua=True, bounds=[("y", 1, 1)])]))
CASES.append(Case("IntCDiv0y2", "tests/pir_test.cpp:867-873", _div0y2(CDIV), [
    Step(1, [(0, 1)], [(0, 0)], True)]))


def _div1(op):
    def build(m):
        m.var("x", 2, 10); m.var("y", -25, 25); m.var("z", -2, 3)
        m.prop(op, "x", "y", "z")          # int_?div(y, z, x): x = y / z
    return build


for _name, _ref, _op, _ylo in [("IntEDiv1", ":875-883", EDIV, -20), ("IntCDiv1", ":885-893", CDIV, -20),
                               ("IntTDiv1", ":895-903", TDIV, -21), ("IntFDiv1", ":905-913", FDIV, -21)]:
    CASES.append(Case(_name, "tests/pir_test.cpp" + _ref, _div1(_op), [
        Step(1, [(2, 10), (-25, 25), (-2, 3)], [(2, 10), (_ylo, 25), (-2, 3)])]))


@case("IntAbs1", "tests/pir_test.cpp:915-922", [
    Step(3, [(-15, 5), (-10, 10)], [(-10, 5), (0, 10)])])
def _(m):
    m.var("x", -15, 5); m.var("y", -10, 10)
    n = m.fresh()
    m.prop(MUL, n, m.c(-1), "x")          # n = -x
    m.prop(MAX, "y", "x", n)               # y = max(x, -x)
    m.prop(LEQ, m.c(1), m.c(0), "y")       # 0 <= y


# ------------------------------------------------------- infinite domains ----
def _inf(m):
    m.var("x"); m.var("b", 0, 1)
    m.prop(LEQ, "b", "x", m.c(5))          # b = (x <= 5)


CASES.append(Case("InfiniteDomain1", "tests/pir_test.cpp:924-934", _inf, [
    Step(1, [TOP, (0, 1)]),
    Step(1, [TOP, (1, 1)], [(MINF, 5), (1, 1)], True, bounds=[("b", 1, 1)])]))
CASES.append(Case("InfiniteDomain2", "tests/pir_test.cpp:936-946", _inf, [
    Step(1, [TOP, (0, 1)]),
    Step(1, [TOP, (0, 0)], [(6, INF), (0, 0)], True, bounds=[("b", 0, 0)])]))


def build_case(c):
    """Instantiate a case: returns the Model (initial bounds and propagators)."""
    m = Model()
    c.build(m)
    return m
