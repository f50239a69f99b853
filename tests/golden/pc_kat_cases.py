"""Known-answer cases of lala-pc's PC tests (tests/pc_test.cpp), as FlatZinc.

Each case is (name, pc_test.cpp line, FlatZinc model, steps).  A step is
(tell, num, before, after, extractable, changed): `tell` is FlatZinc told
into the model before the step (interpret_must_succeed, or None for the
first step); the rest restates one deduce_and_test call
(tests/pc_test.cpp:85-105): the propagator count, the bounds of the user
variables (declaration order) before and after the Gauss-Seidel fixpoint,
is_extractable() after it, and the loop's has_changed.  BOT as `after`
means the store must become empty (is_bot()).

The reference compiles the FlatZinc with lala-parsing into formulas that
PC interprets (pc.hpp:505-605); here include/pirgpu_fzn_pc.hpp does.
Expected values are transcribed from the test source.

AE_CASES restate the AbstractElement tests (:714-764), whose two comparisons
are typed for the store (tests/pc_test.cpp:709-712), so that PC keeps each as
an AbstractElement (formula.hpp:14-78) holding the store's tell / ask of the
comparison and of its negation, combined by `nbool_equiv` (read as <=>, which
the expected values require).  `x >= 5`: tell / ask x in [5, inf), negation
x in (-inf, 4].  `x == 5`: tell / ask x in [5, 5]; its negation x != 5 has no
interval tell (no holes) and asks that 5 is not in x.  A step is
(store meets, before, after, extractable, changed); BOT as `after`: the store
becomes empty.
"""

INF = 2**31 - 1
MINF = -2**31
TOP = (MINF, INF)
BOT = "bot"

XY10 = ("var int: x; var int: y; constraint int_ge(x, 0); constraint int_le(x, 10);"
        " constraint int_ge(y, 0); constraint int_le(y, 10);")
XY3 = ("var int: x; var int: y; constraint int_ge(x, 0); constraint int_le(x, 3);"
       " constraint int_ge(y, 0); constraint int_le(y, 3);")


def xyz(lo, hi):
    return ("var int: x; var int: y; var int: z; " +
            " ".join("constraint int_ge(%s, %d); constraint int_le(%s, %d);" % (v, lo, v, hi) for v in "xyz"))


def one(before, after=None, ua=False, changed=None, num=1, tell=None):
    if after is None:
        after = before
        changed = False if changed is None else changed
    elif changed is None:
        changed = True
    return (tell, num, before, after, ua, changed)


CASES = [
    ("AddEquality", 114, XY10 + " constraint int_plus(x, y, 5);",
     [one([(0, 10), (0, 10)], [(0, 5), (0, 5)])]),
    ("TemporalConstraint1Flat", 123,
     "var int: x; var int: y; var int: z; constraint int_ge(x, 0); constraint int_le(x, 10);"
     " constraint int_ge(y, 0); constraint int_le(y, 10); constraint int_le(z, 5); constraint int_plus(x, y, z);",
     [one([(0, 10), (0, 10), (MINF, 5)], [(0, 5), (0, 5), (0, 5)])]),
    ("TemporalConstraint1", 132, XY10 + " constraint int_le(int_plus(x, y), 5);",
     [one([(0, 10), (0, 10)], [(0, 5), (0, 5)])]),
    ("TemporalConstraint2", 141, XY10 + " constraint int_gt(int_plus(x, y), 5);",
     [one([(0, 10), (0, 10)])]),
    ("TemporalConstraint3", 150, XY3 + " constraint int_gt(int_plus(x, y), 5);",
     [one([(0, 3), (0, 3)], [(3, 3), (3, 3)], ua=True)]),
    ("TemporalConstraint4", 159, XY3 + " constraint int_ge(int_plus(x, y), 5);",
     [one([(0, 3), (0, 3)], [(2, 3), (2, 3)])]),
    ("TemporalConstraint5", 168,
     "var int: x; var int: y; constraint int_ge(x, 0); constraint int_le(x, 4);"
     " constraint int_ge(y, 0); constraint int_le(y, 4); constraint int_eq(int_plus(x, y), 5);",
     [one([(0, 4), (0, 4)], [(1, 4), (1, 4)])]),
    ("TemporalConstraint6", 177, XY10 + " constraint int_le(int_minus(x, y), 5);",
     [one([(0, 10), (0, 10)])]),
    ("TemporalConstraint7", 186, XY10 + " constraint int_le(int_minus(x, y), -10);",
     [one([(0, 10), (0, 10)], [(0, 0), (10, 10)], ua=True)]),
    ("TemporalConstraint8", 195, XY10 + " constraint int_ge(int_minus(x, y), 5);",
     [one([(0, 10), (0, 10)], [(5, 10), (0, 5)])]),
    ("TemporalConstraint9", 204, XY10 + " constraint int_le(int_minus(x, y), -5);",
     [one([(0, 10), (0, 10)], [(0, 5), (5, 10)])]),
    ("TemporalConstraint10", 213, XY10 + " constraint int_le(x, int_plus(-5, y));",
     [one([(0, 10), (0, 10)], [(0, 5), (5, 10)])]),
    ("TopProp", 222, xyz(3, 10) + " constraint int_le(int_plus(int_plus(x, y),z), 8);",
     [one([(3, 10)] * 3, BOT)]),
    ("TernaryAdd2", 233, xyz(3, 10) + " constraint int_le(int_plus(int_plus(x, y),z), 9);",
     [one([(3, 10)] * 3, [(3, 3)] * 3, ua=True)]),
    ("TernaryAdd3", 243, xyz(3, 10) + " constraint int_le(int_plus(int_plus(x, y),z), 10);",
     [one([(3, 10)] * 3, [(3, 4)] * 3)]),
    ("TernaryAdd4", 253, xyz(-2, 2) + " constraint int_le(int_plus(int_plus(x, y),z), -5);",
     [one([(-2, 2)] * 3, [(-2, -1)] * 3)]),
    ("PseudoBoolean1", 263,
     xyz(0, 1) + " constraint int_le(int_plus(int_plus(int_times(2,x), y),int_times(3,z)), 2);",
     [one([(0, 1)] * 3, [(0, 1), (0, 1), (0, 0)])]),
    ("PseudoBoolean2", 273,
     xyz(0, 1) + " constraint int_le(int_plus(int_plus(int_times(2,x), int_times(5,y)),int_times(3,z)), 2);",
     [one([(0, 1)] * 3, [(0, 1), (0, 0), (0, 0)], ua=True)]),
    ("PseudoBoolean3", 283,
     xyz(0, 1) + " constraint int_le(int_plus(int_plus(int_times(3,x), int_times(5,y)),int_times(3,z)), 2);",
     [one([(0, 1)] * 3, [(0, 0)] * 3, ua=True)]),
    ("PseudoBoolean4", 293,
     xyz(0, 1) + " constraint int_le(int_plus(int_plus(int_neg(x), y),int_times(3,z)), 2);",
     [one([(0, 1)] * 3)]),
    ("NegationOp1", 303, "var int: x; constraint int_ge(x, -4); constraint int_le(x, 3);"
     " constraint int_le(int_neg(x), 2);", [one([(-4, 3)], [(-2, 3)], ua=True)]),
    ("NegationOp2", 311, "var int: x; constraint int_ge(x, -4); constraint int_le(x, 3);"
     " constraint int_le(int_neg(x), -2);", [one([(-4, 3)], [(2, 3)], ua=True)]),
    ("NegationOp3", 319, "var int: x; constraint int_ge(x, 0); constraint int_le(x, 3);"
     " constraint int_le(int_neg(x), -2);", [one([(0, 3)], [(2, 3)], ua=True)]),
    ("NegationOp4", 327, "var int: x; constraint int_ge(x, -4); constraint int_le(x, -3);"
     " constraint int_le(int_neg(x), 4);", [one([(-4, -3)], ua=True)]),
    ("NegationOp5", 335, "var int: x; constraint int_ge(x, -4); constraint int_le(x, 3);"
     " constraint int_ge(int_neg(x), -2);", [one([(-4, 3)], [(-4, 2)], ua=True)]),
    ("NegationOp6", 343, "var int: x; constraint int_ge(x, -4); constraint int_le(x, 3);"
     " constraint int_gt(int_neg(x), 2);", [one([(-4, 3)], [(-4, -3)], ua=True)]),
    ("NegationOp7", 351, "var int: x; constraint int_ge(x, -4); constraint int_le(x, 3);"
     " constraint int_ge(int_neg(x), 5);", [one([(-4, 3)], BOT)]),
    ("ResourceConstraint1", 360,
     "var int: x; var int: y; var int: b; constraint int_ge(x, 5); constraint int_le(x, 10);"
     " constraint int_ge(y, 9); constraint int_le(y, 15); constraint int_ge(b, 0); constraint int_le(b, 1);"
     " constraint int_eq(b, bool_and(int_le(int_minus(x, y), 0), int_le(int_minus(y, x), 2)));",
     [one([(5, 10), (9, 15), (0, 1)]),
      one([(5, 10), (9, 15), (1, 1)], [(7, 10), (9, 12), (1, 1)], tell="constraint int_eq(b, 1);")]),
    ("ResourceConstraint2", 373,
     "var int: x; var int: y; var int: b; constraint int_ge(x, 1); constraint int_le(x, 2);"
     " constraint int_ge(y, 0); constraint int_le(y, 2); constraint int_ge(b, 0); constraint int_le(b, 1);"
     " constraint int_eq(b, bool_and(int_le(int_minus(x, y), 2), int_le(int_minus(y, x), -1)));",
     [one([(1, 2), (0, 2), (0, 1)]),
      one([(1, 2), (0, 2), (0, 0)], [(1, 2), (1, 2), (0, 0)], tell="constraint int_eq(b, 0);")]),
    ("NotEqualConstraint1", 386, "var 1..10: x; constraint int_ne(x, 10);",
     [one([(1, 10)], [(1, 9)], ua=True)]),
    ("NotEqualConstraint2", 392, "var 1..10: x; var 10..10: y; constraint int_ne(x, y);",
     [one([(1, 10), (10, 10)], [(1, 9), (10, 10)], ua=True)]),
    ("NotEqualConstraint3", 398, "var 1..10: x; constraint bool_not(int_eq(x, 10));",
     [one([(1, 10)], [(1, 9)], ua=True)]),
    ("ElementConstraint1", 405,
     "array[1..3] of int: a = [10, 11, 12]; var 1..3: b; var 10..12: c; constraint array_int_element(b, a, c);",
     [one([(1, 3), (10, 12)], num=3),
      one([(1, 3), (10, 11)], [(1, 2), (10, 11)], num=3, tell="constraint int_le(c, 11);"),
      one([(1, 2), (11, 11)], [(2, 2), (11, 11)], num=3, ua=True, tell="constraint int_ge(c, 11);")]),
    ("XorConstraint1", 422, "var int: x; var int: y; constraint bool_xor(int_eq(x, 5), int_eq(y, 5));",
     [one([TOP, TOP]),
      one([(1, 1), TOP], [(1, 1), (5, 5)], ua=True, tell="constraint int_eq(x, 1);")]),
    ("XorConstraint2", 433, "var 1..5: x; var 1..5: y; constraint bool_xor(int_eq(x, 5), int_eq(y, 5));",
     [one([(1, 5), (1, 5)]),
      one([(1, 5), (5, 5)], [(1, 4), (5, 5)], ua=True, tell="constraint int_eq(y, 5);")]),
    ("InConstraint1", 469, "var {1, 3}: x; var 2..3: y;",
     [one([(1, 3), (2, 3)]),
      one([(1, 3), (2, 3)], [(3, 3), (3, 3)], num=2, ua=True, tell="constraint int_eq(x, y);")]),
    ("MinConstraint1", 479, "var 0..4: x; var 2..5: y; var 0..10: z; constraint int_min(x, y, z);",
     [one([(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (0, 4)]),
      one([(0, 4), (2, 5), (0, 3)], tell="constraint int_le(z, 3);"),
      one([(0, 1), (2, 5), (0, 3)], [(0, 1), (2, 5), (0, 1)], tell="constraint int_le(x, 1);"),
      one([(0, 0), (2, 5), (0, 1)], [(0, 0), (2, 5), (0, 0)], ua=True, tell="constraint int_le(x, 0);")]),
    ("MinConstraint2", 496, "var 0..4: x; var 2..5: y; var 0..10: z; constraint int_min(x, y, z);",
     [one([(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (0, 4)]),
      one([(0, 4), (2, 5), (0, 3)], tell="constraint int_le(z, 3);"),
      one([(4, 4), (2, 5), (0, 3)], [(4, 4), (2, 3), (2, 3)], tell="constraint int_eq(x, 4);")]),
    ("MinConstraint3", 510, "var int: x; var 0..1: b1; var 0..1: b2; constraint int_min(b1, b2, 1);",
     [one([TOP, (0, 1), (0, 1)], [TOP, (1, 1), (1, 1)], ua=True),
      one([TOP, (1, 1), (1, 1)], [(MINF, 5), (1, 1), (1, 1)], num=2, ua=True,
          tell="constraint int_eq(b1, int_le(x, 5));"),
      one([(MINF, 5), (1, 1), (1, 1)], [(5, 5), (1, 1), (1, 1)], num=3, ua=True,
          tell="constraint int_eq(b2, int_ge(x, 5));")]),
    ("MaxConstraint1", 524, "var 0..4: x; var 2..5: y; var 0..10: z; constraint int_max(x, y, z);",
     [one([(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (2, 5)]),
      one([(0, 4), (2, 5), (2, 3)], [(0, 3), (2, 3), (2, 3)], tell="constraint int_le(z, 3);"),
      one([(0, 1), (2, 3), (2, 3)], tell="constraint int_le(x, 1);"),
      one([(0, 1), (2, 2), (2, 3)], [(0, 1), (2, 2), (2, 2)], ua=True, tell="constraint int_eq(y, 2);")]),
    ("MaxConstraint2", 541, "var 0..4: x; var 2..5: y; var 0..10: z; constraint int_max(x, y, z);",
     [one([(0, 4), (2, 5), (0, 10)], [(0, 4), (2, 5), (2, 5)]),
      one([(0, 4), (2, 5), (5, 5)], [(0, 4), (5, 5), (5, 5)], ua=True, tell="constraint int_ge(z, 5);")]),
    ("MaxConstraint3", 551, "var int: x; var 0..1: b1; var 0..1: b2; constraint int_max(b1, b2, 0);",
     [one([TOP, (0, 1), (0, 1)], [TOP, (0, 0), (0, 0)], ua=True),
      one([TOP, (0, 0), (0, 0)], [(6, INF), (0, 0), (0, 0)], num=2, ua=True,
          tell="constraint int_eq(b1, int_le(x, 5));"),
      one([(6, INF), (0, 0), (0, 0)], [(6, 6), (0, 0), (0, 0)], num=3, ua=True,
          tell="constraint int_eq(b2, int_ge(x, 7));")]),
    ("BooleanClause1", 564,
     "array[1..2] of var bool: x; array[1..2] of var bool: y; constraint bool_clause(x, y);",
     [one([(0, 1)] * 4),
      one([(1, 1), (0, 1), (0, 1), (0, 1)], ua=True, tell="constraint int_eq(x[1], true);")]),
    ("BooleanClause2", 574,
     "array[1..2] of var bool: x; array[1..2] of var bool: y; constraint bool_clause(x, y);",
     [one([(0, 1)] * 4),
      one([(0, 1), (0, 1), (0, 0), (0, 1)], ua=True, tell="constraint int_eq(y[1], false);")]),
    ("BooleanClause3", 584,
     "array[1..2] of var bool: x; array[1..2] of var bool: y; constraint bool_clause(x, y);",
     [one([(0, 1)] * 4),
      one([(0, 0), (0, 1), (0, 1), (0, 1)], tell="constraint int_eq(x[1], false);"),
      one([(0, 0), (0, 0), (0, 1), (0, 1)], tell="constraint int_eq(x[2], false);"),
      one([(0, 0), (0, 0), (1, 1), (0, 1)], [(0, 0), (0, 0), (1, 1), (0, 0)], ua=True,
          tell="constraint int_eq(y[1], true);")]),
    ("BooleanClause4", 598,
     "array[1..2] of var bool: x; array[1..2] of var bool: y; constraint bool_clause(x, y);",
     [one([(0, 1)] * 4),
      one([(0, 0), (0, 1), (0, 1), (0, 1)], tell="constraint int_eq(x[1], false);"),
      one([(0, 0), (0, 1), (1, 1), (0, 1)], tell="constraint int_eq(y[1], true);"),
      one([(0, 0), (0, 1), (1, 1), (1, 1)], [(0, 0), (1, 1), (1, 1), (1, 1)], ua=True,
          tell="constraint int_eq(y[2], true);")]),
    ("IntTimes1", 612, "var 0..1: x; var 0..1: y; var 0..1: z; constraint int_times(x,y,z);",
     [one([(0, 1)] * 3),
      one([(1, 1), (0, 1), (0, 1)], tell="constraint int_eq(x, 1);"),
      one([(1, 1), (1, 1), (0, 1)], [(1, 1)] * 3, ua=True, tell="constraint int_eq(y, 1);")]),
    ("IntTimes2", 626, "var 0..1: x; var 0..1: y; var 0..1: z; constraint int_times(x,y,z);",
     [one([(0, 1)] * 3),
      one([(0, 1), (0, 1), (1, 1)], [(1, 1)] * 3, ua=True, tell="constraint int_eq(z, 1);")]),
    ("IntTimes3", 638, "var 0..0: x; var 0..1: y; var 0..1: z; constraint int_times(x, y, z);",
     [one([(0, 0), (0, 1), (0, 1)], [(0, 0), (0, 1), (0, 0)], ua=True)]),
    ("IntTimes4", 648, "var 0..1: x; var 0..0: y; var 0..1: z; constraint int_times(x, y, z);",
     [one([(0, 1), (0, 0), (0, 1)], [(0, 1), (0, 0), (0, 0)], ua=True)]),
    ("IntTimes5", 658, "var 1..2: x; var 0..1: y; var 0..0: z; constraint int_times(x, y, z);",
     [one([(1, 2), (0, 1), (0, 0)], [(1, 2), (0, 0), (0, 0)], ua=True)]),
    ("IntTimes6", 668, "var 0..1: x; var 1..2: y; var 0..0: z; constraint int_times(x, y, z);",
     [one([(0, 1), (1, 2), (0, 0)], [(0, 0), (1, 2), (0, 0)], ua=True)]),
    ("IntDiv1", 678, "var 0..1: x; var 0..1: y; var 0..1: z; constraint int_div(x,y,z);",
     [one([(0, 1)] * 3, [(0, 1), (1, 1), (0, 1)]),
      one([(1, 1), (1, 1), (0, 1)], [(1, 1)] * 3, ua=True, tell="constraint int_eq(x, 1);")]),
    ("IntDiv2", 690, "var 0..1: y; constraint int_div(y,2,0);",
     [one([(0, 1)], ua=True),
      one([(1, 1)], ua=True, tell="constraint int_eq(y, 1);")]),
    ("IntAbs1", 700, "var -15..5: x; var -10..10: y; constraint int_abs(x, y);",
     [one([(-15, 5), (-10, 10)], [(-10, 5), (0, 10)])]),
    ("InfiniteDomain1", 766, "var int: x; var bool: b; constraint int_eq(b, int_le(x,5));",
     [one([TOP, (0, 1)]),
      one([TOP, (1, 1)], [(MINF, 5), (1, 1)], ua=True, tell="constraint int_eq(b, 1);")]),
    ("InfiniteDomain2", 778, "var int: x; var bool: b; constraint int_eq(b, int_le(x,5));",
     [one([TOP, (0, 1)]),
      one([TOP, (0, 0)], [(6, INF), (0, 0)], ua=True, tell="constraint int_eq(b, 0);")]),
]


AE_CASES = [
    ("AbstractElement1", 714, "ge_le",
     [([], [(0, 10), (0, 10)], [(0, 10), (0, 10)], False, False),
      ([(0, 5, 5)], [(5, 5), (0, 10)], [(5, 5), (0, 5)], True, True)]),
    ("AbstractElement2", 725, "ge_le",
     [([], [(0, 10), (0, 10)], [(0, 10), (0, 10)], False, False),
      ([(0, 4, 4)], [(4, 4), (0, 10)], [(4, 4), (6, 10)], True, True)]),
    ("AbstractElement3", 736, "eq_eq",
     [([], [(0, 10), (0, 10)], [(0, 10), (0, 10)], False, False),
      ([(1, 6, 6)], [(0, 10), (6, 6)], [(0, 10), (6, 6)], False, False),
      ([(0, 5, 5)], [(5, 5), (6, 6)], BOT, False, True)]),
    ("AbstractElement4", 751, "eq_eq",
     [([], [(0, 10), (0, 10)], [(0, 10), (0, 10)], False, False),
      ([(1, 4, 4)], [(0, 10), (4, 4)], [(0, 10), (4, 4)], False, False),
      ([(0, 5, 5)], [(5, 5), (4, 4)], BOT, False, True)]),
]
