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

The deviation-form kernels use mrt_moments_fast / mrt_back_fast (gen_fast):
same transforms, cheaper, with no term-by-term parity requirement.

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




def gen_fast():
    """Transforms for the deviation-form kernels (no bit-parity requirement):
    M f from opposite-pair sums a_p = f_{2p+1} + f_{2p+2} and differences
    d_p = f_{2p+1} - f_{2p+2} with shared partial sums; inv(M) m from the exact
    inverses of its even (f0, a_p) and odd (d_p) blocks, as FMA chains."""
    inv = exact_inverse(M)
    out = []
    w = out.append
    # check the pair structure: rows use (c, c) or (c, -c) on every opposite pair
    even_rows, odd_rows = [], []
    for r in range(19):
        kinds = set()
        for p in range(9):
            x, y = M[r][2 * p + 1], M[r][2 * p + 2]
            if x == 0 and y == 0:
                continue
            kinds.add("a" if x == y else ("d" if x == -y else "?"))
        assert "?" not in kinds and len(kinds) <= 1, r
        (odd_rows if "d" in kinds else even_rows).append(r)
    w("template <typename R>")
    w("__host__ __device__ __forceinline__ void mrt_moments_fast(const R* f, R* m) {")
    for p in range(9):
        w("  const R a%d = f[%d] + f[%d], d%d = f[%d] - f[%d];" % (p, 2 * p + 1, 2 * p + 2, p, 2 * p + 1, 2 * p + 2))
    w("  const R sf = (a0 + a1) + a2, se1 = a3 + a4, se2 = a5 + a6, se3 = a7 + a8;")
    w("  const R e = (se1 + se2) + se3, a12 = a1 + a2, e12 = se1 + se2, a1m2 = a1 - a2, e1m2 = se1 - se2;")
    w("  const R d34p = d3 + d4, d34m = d3 - d4, d56p = d5 + d6, d56m = d5 - d6, d78p = d7 + d8, d78m = d7 - d8;")
    w("  m[0] = (f[0] + sf) + e;")
    w("  m[1] = e - f[0];")
    w("  m[2] = lbm_fma((R)-2, sf, f[0] + e);")
    w("  m[9] = lbm_fma((R)-2, se3, lbm_fma((R)2, a0, e12 - a12));")
    w("  m[10] = lbm_fma((R)-2, se3, lbm_fma((R)-2, a0, e12 + a12));")
    w("  m[11] = a1m2 + e1m2;")
    w("  m[12] = e1m2 - a1m2;")
    w("  m[13] = a3 - a4; m[14] = a7 - a8; m[15] = a5 - a6;")
    w("  m[3] = (d0 + d34p) + d56p;")
    w("  m[4] = lbm_fma((R)-2, d0, d34p + d56p);")
    w("  m[5] = (d1 + d34m) + d78p;")
    w("  m[6] = lbm_fma((R)-2, d1, d34m + d78p);")
    w("  m[7] = (d2 + d56m) + d78m;")
    w("  m[8] = lbm_fma((R)-2, d2, d56m + d78m);")
    w("  m[16] = d34p - d56p;")
    w("  m[17] = d78p - d34m;")
    w("  m[18] = d56m - d78m;")
    w("}")
    w("")
    # sanity of the hand-written moment expressions against M on random integers
    import random
    rnd = random.Random(5)
    for _ in range(20):
        f = [rnd.randint(-50, 50) for _ in range(19)]
        a = [f[2 * p + 1] + f[2 * p + 2] for p in range(9)]
        d = [f[2 * p + 1] - f[2 * p + 2] for p in range(9)]
        sf, se1, se2, se3 = a[0] + a[1] + a[2], a[3] + a[4], a[5] + a[6], a[7] + a[8]
        e, a12, e12, a1m2, e1m2 = se1 + se2 + se3, a[1] + a[2], se1 + se2, a[1] - a[2], se1 - se2
        d34p, d34m, d56p, d56m, d78p, d78m = d[3] + d[4], d[3] - d[4], d[5] + d[6], d[5] - d[6], d[7] + d[8], d[7] - d[8]
        m = [0] * 19
        m[0], m[1], m[2] = f[0] + sf + e, e - f[0], f[0] + e - 2 * sf
        m[9], m[10] = e12 - a12 + 2 * a[0] - 2 * se3, e12 + a12 - 2 * a[0] - 2 * se3
        m[11], m[12], m[13], m[14], m[15] = a1m2 + e1m2, e1m2 - a1m2, a[3] - a[4], a[7] - a[8], a[5] - a[6]
        m[3], m[4] = d[0] + d34p + d56p, d34p + d56p - 2 * d[0]
        m[5], m[6] = d[1] + d34m + d78p, d34m + d78p - 2 * d[1]
        m[7], m[8] = d[2] + d56m + d78m, d56m + d78m - 2 * d[2]
        m[16], m[17], m[18] = d34p - d56p, d78p - d34m, d56m - d78m
        ref = [sum(M[r][c] * f[c] for c in range(19)) for r in range(19)]
        assert m == ref, (m, ref)
    # inverse: even block (f0, a_0..a_8) and odd block (d_0..d_8) in terms of moments
    #   f0 = sum_k inv[0][k] m_k;  a_p = f_{2p+1} + f_{2p+2};  d_p = f_{2p+1} - f_{2p+2}
    w("template <typename R>")
    w("__host__ __device__ __forceinline__ void mrt_back_fast(const R* m, R* f) {")

    def chain(coefs, name):
        terms = [(c, k) for k, c in coefs if c != 0]
        first = True
        expr = None
        for c, k in terms:
            if first:
                expr = "(R)(%r) * m[%d]" % (float(c), k)
                first = False
            else:
                expr = "lbm_fma((R)(%r), m[%d], %s)" % (float(c), k, expr)
        w("  const R %s = %s;" % (name, expr if expr else "(R)0"))

    chain([(k, inv[0][k]) for k in range(19)], "f0")
    for p in range(9):
        s1, s2 = 2 * p + 1, 2 * p + 2
        # half sums / differences so that f = ha +- hd
        chain([(k, (inv[s1][k] + inv[s2][k]) / 2) for k in range(19)], "ha%d" % p)
        chain([(k, (inv[s1][k] - inv[s2][k]) / 2) for k in range(19)], "hd%d" % p)
    w("  f[0] = f0;")
    for p in range(9):
        w("  f[%d] = ha%d + hd%d; f[%d] = ha%d - hd%d;" % (2 * p + 1, p, p, 2 * p + 2, p, p))
    w("}")
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    import sys
    sys.stdout.write(gen())
    sys.stdout.write("\n")
    sys.stdout.write(gen_fast())
