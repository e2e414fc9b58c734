"""Generate hankel_tables.inc: coefficient tables of the device Hankel evaluator.

The device evaluates H_nu^(1)(x) = J_nu(x) + i Y_nu(x), nu in {0, 1}, for real x > 0 in
three regions (see hankel.cuh):

  x <  XA          ascending power series in q = x^2/4 (A&S 9.1.10, 9.1.11), Horner form;
  XA <= x < XC     piecewise Chebyshev expansions of J_nu and Y_nu on intervals of width W;
  x >= XC          Hankel asymptotic expansion (A&S 9.2.5-9.2.10), P and Q as polynomials
                   in 1/x^2 with coefficients (nu, m) / 2^m.

All coefficients are computed here with mpmath at 50 digits and written as C hex-float
literals.  Run:  python gen_hankel_tables.py  (writes hankel_tables.inc next to itself).
"""
import os
import mpmath as mp

mp.mp.dps = 50

XA = 3.0          # series below, Chebyshev pieces above
XC = 25.0         # asymptotic expansion from here on
W = 2.0           # width of a Chebyshev piece
DEG = 18          # degree of each Chebyshev piece
NSER = 16         # number of series terms
NASY = 10         # terms of P and of Q


def hexd(v):
    return float(v).hex()


def series_coeffs():
    a0, b0, a1, b1 = [], [], [], []
    H = mp.mpf(0)
    for k in range(NSER):
        if k > 0:
            H += mp.mpf(1) / k
        Hn = H + mp.mpf(1) / (k + 1)
        s = (-1) ** k
        a0.append(mp.mpf(s) / mp.factorial(k) ** 2)                       # J0 = sum a0_k q^k
        b0.append(-mp.mpf(2) / mp.pi * H * s / mp.factorial(k) ** 2)      # Y0 rest
        a1.append(mp.mpf(s) / (mp.factorial(k) * mp.factorial(k + 1)))    # J1 = (x/2) sum a1_k q^k
        b1.append(-(H + Hn) / mp.pi * s / (mp.factorial(k) * mp.factorial(k + 1)))  # Y1 rest (x/2) sum
    return a0, b0, a1, b1


def cheb_fit(f, a, b, deg):
    n = deg + 1
    nodes = [mp.cos(mp.pi * (j + mp.mpf(1) / 2) / n) for j in range(n)]
    vals = [f((b - a) / 2 * t + (a + b) / 2) for t in nodes]
    c = []
    for k in range(n):
        s = mp.fsum(vals[j] * mp.cos(mp.pi * k * (j + mp.mpf(1) / 2) / n) for j in range(n))
        c.append(s * 2 / n)
    c[0] /= 2
    return c


def asym_coeffs(nu):
    mu = 4 * nu * nu
    P, Q = [], []
    c = mp.mpf(1)
    P.append(c)
    for m in range(1, 2 * NASY + 1):
        c = c * (mu - (2 * m - 1) ** 2) / (4 * m) / 2   # (nu, m) / 2^m
        sgn = -1 if (m // 2) % 2 else 1
        (Q if m % 2 else P).append(sgn * c)
    return P[:NASY], Q[:NASY]


def main():
    out = []
    out.append("// Generated by gen_hankel_tables.py -- do not edit.")
    out.append(f"#define HK_XA {XA!r}")
    out.append(f"#define HK_XC {XC!r}")
    out.append(f"#define HK_W {W!r}")
    out.append(f"#define HK_DEG {DEG}")
    out.append(f"#define HK_NSER {NSER}")
    out.append(f"#define HK_NASY {NASY}")
    npieces = int(round((XC - XA) / W))
    out.append(f"#define HK_NPIECES {npieces}")
    a0, b0, a1, b1 = series_coeffs()
    for name, arr in (("hk_ser_a0", a0), ("hk_ser_b0", b0), ("hk_ser_a1", a1), ("hk_ser_b1", b1)):
        out.append(f"HK_TABLE double {name}[{NSER}] = {{" + ", ".join(hexd(v) for v in arr) + "};")
    maxerr = 0.0
    for nu in (0, 1):
        rows = []
        for p in range(npieces):
            a = mp.mpf(XA) + p * W
            b = a + W
            cj = cheb_fit(lambda x: mp.besselj(nu, x), a, b, DEG)
            cy = cheb_fit(lambda x: mp.bessely(nu, x), a, b, DEG)
            rows.append(cj + cy)
            # check the truncated expansion on a few points against mpmath
            for t in [mp.mpf(i) / 50 - 1 for i in range(101)]:
                x = (b - a) / 2 * t + (a + b) / 2
                T = [mp.mpf(1), t]
                for k in range(2, DEG + 1):
                    T.append(2 * t * T[-1] - T[-2])
                ej = mp.fsum(cj[k] * T[k] for k in range(DEG + 1)) - mp.besselj(nu, x)
                ey = mp.fsum(cy[k] * T[k] for k in range(DEG + 1)) - mp.bessely(nu, x)
                h = mp.sqrt(mp.besselj(nu, x) ** 2 + mp.bessely(nu, x) ** 2)
                maxerr = max(maxerr, float(abs(ej) / h), float(abs(ey) / h))
        flat = [hexd(v) for r in rows for v in r]
        out.append(f"HK_TABLE double hk_cheb{nu}[{npieces * 2 * (DEG + 1)}] = {{" + ", ".join(flat) + "};")
        P, Q = asym_coeffs(nu)
        out.append(f"HK_TABLE double hk_asyP{nu}[{NASY}] = {{" + ", ".join(hexd(v) for v in P) + "};")
        out.append(f"HK_TABLE double hk_asyQ{nu}[{NASY}] = {{" + ", ".join(hexd(v) for v in Q) + "};")
    out.append(f"// max truncation error of the Chebyshev pieces relative to |H|: {maxerr:.3e}")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hankel_tables.inc")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path, "max piece error", maxerr)


if __name__ == "__main__":
    main()
