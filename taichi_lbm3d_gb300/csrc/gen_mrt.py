"""Generate mrt_gen.cuh: the D3Q19 moment transforms of the reference's MRT
collision, unrolled for the fused kernels.

The reference multiplies by M and by fp32(inv(M)) as dense 19x19 FP32 products
accumulated left to right (LBM_3D_SinglePhase_Solver.py:226,241; the 2-phase
script's multiply_M and its inv_M loop, 2phase/lbm_solver_3d_2phase_sparse.py:232-239,
:341-344).  This generator keeps that order term by term but:

* drops terms whose coefficient is exactly zero (adding a signed zero to a
  non-zero partial sum leaves it unchanged);
* for M (entries 0, +-1, +-2) every product is exact, so each term is an
  add/sub or an exact fma by +-2;
* for inv(M) every column's non-zero entries are +-2^n times one of at most two
  "odd parts" (e.g. 1/36, 1/18 = 2*(1/36), 1/3): the product base*m[l] is rounded
  once per (column, odd part) and each term is that product scaled by +-2^n,
  which is exact, so the sum equals the reference's term by term.

Run:  python gen_mrt.py > mrt_gen.cuh
"""
from fractions import Fraction

M = [
    [1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [-1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [1, -2, -2, -2, -2, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, -2, 2, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, -2, 2, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
    [0, 0, 0, 0, 0, -2, 2, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
    [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
    [0, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
    [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, -1, -1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, -1, 1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1]]


def exact_inverse(A):
    n = len(A)
    a = [[Fraction(A[r][c]) for c in range(n)] + [Fraction(int(r == c)) for c in range(n)] for r in range(n)]
    for col in range(n):
        piv = next(r for r in range(col, n) if a[r][col] != 0)
        a[col], a[piv] = a[piv], a[col]
        d = a[col][col]
        a[col] = [x / d for x in a[col]]
        for r in range(n):
            if r != col and a[r][col] != 0:
                f = a[r][col]
                a[r] = [x - f * y for x, y in zip(a[r], a[col])]
    return [row[n:] for row in a]


def odd_part(q):
    """|q| = 2^e * o with o's numerator and denominator odd; return (o, e)."""
    q = abs(q)
    e = 0
    num, den = q.numerator, q.denominator
    while num % 2 == 0:
        num //= 2
        e += 1
    while den % 2 == 0:
        den //= 2
        e -= 1
    return Fraction(num, den), e


def coef(k):
    """Exact power-of-two coefficient literal."""
    return "(R)%r" % float(k)


def gen():
    inv = exact_inverse(M)
    out = []
    w = out.append
    w("// Generated by gen_mrt.py -- do not edit.  D3Q19 moment transforms of the")
    w("// reference MRT (literal left-to-right order, exact zero terms dropped).")
    w("#pragma once")
    w("")
    # ---- m = M * x
    w("template <typename R>")
    w("__host__ __device__ __forceinline__ void mrt_moments(const R* x, R* m) {")
    for r in range(19):
        terms = [(M[r][c], c) for c in range(19) if M[r][c] != 0]
        k0, c0 = terms[0]
        if k0 == 1:
            expr = "x[%d]" % c0
        elif k0 == -1:
            expr = "-x[%d]" % c0
        else:
            expr = "%s * x[%d]" % (coef(k0), c0)
        w("  { R a = %s;" % expr)
        for k, c in terms[1:]:
            if k == 1:
                w("    a = a + x[%d];" % c)
            elif k == -1:
                w("    a = a - x[%d];" % c)
            else:
                w("    a = lbm_fma(%s, x[%d], a);" % (coef(k), c))
        w("    m[%d] = a; }" % r)
    w("}")
    w("")
    # ---- f = inv(M) * m, factored by column odd parts
    w("template <typename R>")
    w("__host__ __device__ __forceinline__ void mrt_back(const R* m, R* f) {")
    prods = {}
    for c in range(19):
        fams = []
        for r in range(19):
            if inv[r][c] != 0:
                o, _ = odd_part(inv[r][c])
                if o not in fams:
                    fams.append(o)
        for fi, o in enumerate(fams):
            name = "p%d_%d" % (c, fi)
            prods[(c, o)] = name
            w("  const R %s = (R)(%d.0 / %d.0) * m[%d];  // odd part %s" % (name, o.numerator, o.denominator, c, o))
    for r in range(19):
        terms = [(inv[r][c], c) for c in range(19) if inv[r][c] != 0]
        first = True
        for q, c in terms:
            o, e = odd_part(q)
            k = (1 if q > 0 else -1) * (2.0 ** e)
            p = prods[(c, o)]
            if first:
                w("  { R a = %s * %s;" % (coef(k), p))
                first = False
            else:
                w("    a = lbm_fma(%s, %s, a);" % (coef(k), p))
        w("    f[%d] = a; }" % r)
    w("}")
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    import sys
    sys.stdout.write(gen())
