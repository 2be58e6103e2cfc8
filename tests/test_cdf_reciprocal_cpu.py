"""The counting kernels' fixed-point reciprocal, restated in exact integer
arithmetic: for every CDF value C the count floor((C n - G) / Q) + 1 that
the kernels derive from a truncated high product by a fixed-point
reciprocal (with the exact 128-bit comparison near a boundary) equals the
big-integer definition.
This checks the error bounds the device code relies on (its windows around
the uniforms' grid) on random totals and on CDF values placed on and next
to the grid; the GPU tests then compare the kernels' counts with the same
definition."""
import random

M64 = (1 << 64) - 1


def exact_F(C, Q, n, G):
    X = C * n - G
    return 0 if X < 0 else min(n, X // Q + 1)


def settle(C, k, low, Q, G, n):
    m = k if low else k + 1
    ok = m < 0 or m * Q + G <= C * n
    if low:
        return k if ok else k - 1
    return k + 1 if ok else k


def usual_constants(Q, n, G):
    """s, m, g of the usual case, or None (s < 20)."""
    s = 32
    while s > 0 and (n << s) >= Q:
        s -= 1
    if s < 20:
        return None
    return s, ((n << s) << 64) // Q, (G << s) // Q


def F_usual(C, Q, n, G, s, m, g):
    if C >= Q:
        return n
    c1, c0, m1, m0 = C >> 32, C & 0xFFFFFFFF, m >> 32, m & 0xFFFFFFFF
    H = c1 * m1 + ((c1 * m0) >> 32) + ((c0 * m1) >> 32)  # three products
    B = H - g
    k, f = B >> s, B & ((1 << s) - 1)
    if (((B & 0xFFFFFFFF) + 6) & ((1 << s) - 1)) < 8:  # f < 2 or f >= 2^s - 6
        k = settle(C, k, f < 2, Q, G, n)
    return min(n, k + 1)


def F_general(C, Q, n, G):
    if C >= Q:
        return n
    z = 64 - Q.bit_length()
    Qs = Q << z
    rcp = ((1 << 128) - 1) // Qs - (1 << 64)
    assert 0 <= rcp <= M64
    gam = M64 if G >= Q else (G << 64) // Q
    Cs = C << z
    H = Cs + ((Cs * rcp) >> 64)
    assert H <= M64
    B = H * n - gam
    k, f = B >> 64, B & M64
    if f == 0 or f >= (1 << 64) - (4 * n + 8):
        k = settle(C, k, f == 0, Q, G, n)
    return min(n, k + 1)


def _cases(rng, Q, n, G):
    Cs = [rng.randint(0, Q) for _ in range(20)]
    for _ in range(20):
        j = rng.randint(0, n)
        c = (j * Q + G) // n
        Cs += [c + e for e in (-2, -1, 0, 1, 2) if 0 <= c + e <= Q]
    return Cs


def test_reciprocal_counts_match_the_definition():
    rng = random.Random(11)
    usual = 0
    for trial in range(1500):
        n = rng.randint(2, 1 << rng.randint(1, 31))
        if trial % 4 == 0:
            Q = n * rng.randint(1 << 20, 1 << 31)  # equal-weight-like totals
        else:
            Q = rng.randint(1, (1 << rng.randint(1, 63)) - 1)
        if Q >= 1 << 63:
            continue
        a = rng.getrandbits(32) if trial % 5 else 0
        G = -((-a * Q) // (1 << 32))  # ceil(a Q / 2^32), systematic
        for g in (G, 0):  # systematic, stratified (j* = floor(C n / Q))
            cst = usual_constants(Q, n, g)
            for C in _cases(rng, Q, n, g):
                want = exact_F(C, Q, n, g)
                assert F_general(C, Q, n, g) == want, (C, Q, n, g)
                if cst is not None:
                    usual += 1
                    assert F_usual(C, Q, n, g, *cst) == want, (C, Q, n, g)
    assert usual > 10000
