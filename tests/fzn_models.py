"""FlatZinc models for the front-end tests (written for these tests; the
expected bounds of the known-answer cases are those of lala-pc's
tests/pir_test.cpp for the same models)."""


def send_more_money():
    letters = "SENDMORY"
    s = "".join("var 0..9: %s;\n" % c for c in letters)
    s += "constraint int_ne(S, 0);\nconstraint int_ne(M, 0);\n"
    for i in range(len(letters)):
        for j in range(i + 1, len(letters)):
            s += "constraint int_ne(%s, %s);\n" % (letters[i], letters[j])
    coef = [1000, 100, 10, 1, 1000, 100, 10, 1, -10000, -1000, -100, -10, -1]
    terms = ["S", "E", "N", "D", "M", "O", "R", "E", "M", "O", "N", "E", "Y"]
    s += "constraint int_lin_eq([%s], [%s], 0);\nsolve satisfy;\n" % (
        ", ".join(map(str, coef)), ", ".join(terms))
    return s, list(letters)


def queens(n):
    s = "array [1..%d] of var 1..%d: q :: output_array([1..%d]);\n" % (n, n, n)
    for i in range(1, n + 1):
        for j in range(i + 1, n + 1):
            s += "constraint int_ne(q[%d], q[%d]);\n" % (i, j)
            s += "constraint int_lin_ne([1, -1], [q[%d], q[%d]], %d);\n" % (i, j, j - i)
            s += "constraint int_lin_ne([1, -1], [q[%d], q[%d]], %d);\n" % (i, j, i - j)
    s += "solve satisfy;\n"
    return s, ["q[%d]" % i for i in range(1, n + 1)]


TOP = (-2**31, 2**31 - 1)

# (name, [model text, then the texts told after it], the user variables,
#  their bounds after the fixpoint of each step, extractable at the last step)
KATS = [
    ("TernaryProblem",
     ["var int: x; var int: y; var int: z; constraint int_ge(x, 0); constraint int_le(x, 10);"
      " constraint int_ge(y, 0); constraint int_le(y, 10); constraint int_ge(z, 5);"
      " constraint int_le(z, 5); constraint int_plus(x, y, z);"],
     ["x", "y", "z"], [[(0, 5), (0, 5), (5, 5)]]),
    ("ReifiedEquality", ["var int: x; var int: y; constraint int_eq(x, int_eq(y, 2));"],
     ["x", "y"], [[(0, 1), TOP]]),
    ("ReifiedIn", ["var {1, 2, 4, 5}: x; var bool: y; constraint set_in_reif(x, 2..2, y);"],
     ["x", "y"], [[(1, 5), (0, 1)]]),
    ("ElementConstraint1",
     ["array [1..3] of int: a = [10, 11, 12]; var 1..3: b; var 10..12: c;"
      " constraint array_int_element(b, a, c);",
      "constraint int_le(c, 11);", "constraint int_ge(c, 11);"],
     ["b", "c"], [[(1, 3), (10, 12)], [(1, 2), (10, 11)], [(2, 2), (11, 11)]]),
    ("XorConstraint1", ["var int: x; var int: y; constraint bool_xor(int_eq(x, 5), int_eq(y, 5));",
                        "constraint int_eq(x, 1);"],
     ["x", "y"], [[TOP, TOP], [(1, 1), (5, 5)]]),
    ("XorConstraint2", ["var 1..5: x; var 1..5: y; constraint bool_xor(int_eq(x, 5), int_eq(y, 5));",
                        "constraint int_eq(y, 5);"],
     ["x", "y"], [[(1, 5), (1, 5)], [(1, 4), (5, 5)]]),
    ("InConstraint1", ["var {1, 3}: x; var 2..3: y;", "constraint int_eq(x, y);"],
     ["x", "y"], [[(1, 3), (2, 3)], [(3, 3), (3, 3)]]),
    ("MinConstraint1", ["var 0..4: x; var 2..5: y; var 0..10: z; constraint int_min(x, y, z);"],
     ["x", "y", "z"], [[(0, 4), (2, 5), (0, 4)]]),
]


def magic_square3():
    """The 3 x 3 magic square: the numbers 1..9, every row, column and
    diagonal summing to 15.  It has 8 solutions (the rotations and
    reflections of one square).  Returns (FlatZinc text, cell names)."""
    cells = ["m%d%d" % (i, j) for i in range(3) for j in range(3)]
    lines = ["var 1..9: %s :: output_var;" % c for c in cells]
    lines.append("constraint fzn_all_different_int([%s]);" % ", ".join(cells))
    lines_of = [[(i, j) for j in range(3)] for i in range(3)] + [[(i, j) for i in range(3)] for j in range(3)]
    lines_of += [[(k, k) for k in range(3)], [(k, 2 - k) for k in range(3)]]
    for ln in lines_of:
        lines.append("constraint int_lin_eq([1, 1, 1], [%s], 15);" % ", ".join("m%d%d" % ij for ij in ln))
    lines.append("solve satisfy;")
    return "\n".join(lines), cells
