"""GF(2) polynomial helpers used to pin the xoroshiro128+ jump constant.

Polynomials are Python ints: bit k is the coefficient of x^k.
"""


def berlekamp_massey(bits):
    """Shortest LFSR for a GF(2) sequence; returns the connection polynomial C(x)."""
    c, b = 1, 1
    L, m = 0, 1
    for n, s in enumerate(bits):
        d = s
        for i in range(1, L + 1):
            d ^= ((c >> i) & 1) & bits[n - i]
        if d == 0:
            m += 1
        elif 2 * L <= n:
            t = c
            c ^= b << m
            L = n + 1 - L
            b = t
            m = 1
        else:
            c ^= b << m
            m += 1
    return c, L


def reciprocal(c, degree):
    """x^degree * C(1/x): the characteristic polynomial of the recurrence."""
    out = 0
    for i in range(degree + 1):
        if (c >> i) & 1:
            out |= 1 << (degree - i)
    return out


def polymod(a, p):
    dp = p.bit_length() - 1
    while a.bit_length() - 1 >= dp:
        a ^= p << (a.bit_length() - 1 - dp)
    return a


def polymulmod(a, b, p):
    out = 0
    while b:
        if b & 1:
            out ^= a
        b >>= 1
        a <<= 1
    return polymod(out, p)


def x_pow_2k_mod(k, p):
    """x^(2^k) mod p by k squarings."""
    r = polymod(2, p)
    for _ in range(k):
        r = polymulmod(r, r, p)
    return r
