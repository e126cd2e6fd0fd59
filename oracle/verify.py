"""Exact-arithmetic re-check of certificate lines (a restatement of the reference's
independent gate, sieve/verify_covers.py:246-275, in unbounded Python integers).

TEST INFRASTRUCTURE ONLY: the GPU tests run every certificate the engine emits through it.

  RUNG p A r u       A = (p+r)/4, q = pA, u | q^2, u == -q (mod r), and
                     4/p = 1/A + 1/x + 1/y with x = (q+u)/r, y = q(q+u)/(ru) integers
  SOLVED p a c d k   m = 4acd-1, e = ck-a >= 1, p = mk - 4a^2 d, and
                     4/p = 1/(ade) + 1/(acdp) + 1/(cdep)
"""
from fractions import Fraction


def check_line(line):
    """(kind, ok) for one record line; SURVIVOR lines are never ok."""
    t = line.split()
    if not t:
        return None, True
    if t[0] == "RUNG":
        p, A, r, u = map(int, t[1:5])
        q = p * A
        x, rem = divmod(q + u, r)
        y, rem2 = divmod(q * (q + u), r * u)
        ok = (A == (p + r) // 4 and (q * q) % u == 0 and (q + u) % r == 0 and rem == 0 and rem2 == 0
              and Fraction(4, p) == Fraction(1, A) + Fraction(1, x) + Fraction(1, y))
        return "RUNG", ok
    if t[0] == "SOLVED":
        p, a, c, d, k = map(int, t[1:6])
        m = 4 * a * c * d - 1
        e = c * k - a
        ok = (e >= 1 and p == m * k - 4 * a * a * d
              and Fraction(4, p) == Fraction(1, a * d * e) + Fraction(1, a * c * d * p) + Fraction(1, c * d * e * p))
        return "SOLVED", ok
    if t[0] == "SURVIVOR":
        return "SURVIVOR", False
    return t[0], True


def check_text(text):
    """Counts of (RUNG, SOLVED, bad, SURVIVOR) over a scanner's output."""
    n_rung = n_solved = bad = surv = 0
    for line in text.splitlines():
        kind, ok = check_line(line)
        if kind == "RUNG":
            n_rung += 1
        elif kind == "SOLVED":
            n_solved += 1
        elif kind == "SURVIVOR":
            surv += 1
            continue
        if not ok:
            bad += 1
    return n_rung, n_solved, bad, surv
