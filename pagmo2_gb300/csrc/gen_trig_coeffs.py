"""Writes the fixed-point polynomial coefficients of trig_fixed.h.

sin(2 pi r) = r S(r^2) and cos(2 pi r) = 1 + r^2 H(r^2) for |r| <= 1/4, S and
H of degree 8 in z = r^2 on [0, 1/16], interpolated at the 9 Chebyshev nodes
of that interval in 60-digit arithmetic (mpmath), then rounded to Q55 integers
(value x 2^55). Prints the interpolation error of each fit (sup over a fine
grid: S 1.3e-18 of S >= 4, H 4.1e-19) and the two C arrays.

    python pagmo2_gb300/csrc/gen_trig_coeffs.py
"""
import mpmath as mp

mp.mp.dps = 60
DEG = 8
ZMAX = mp.mpf(1) / 16


def s_fn(z):
    if z == 0:
        return 2 * mp.pi
    r = mp.sqrt(z)
    return mp.sin(2 * mp.pi * r) / r


def h_fn(z):
    if z == 0:
        return -2 * mp.pi ** 2
    r = mp.sqrt(z)
    return (mp.cos(2 * mp.pi * r) - 1) / z


def interpolate(f):
    n = DEG + 1
    nodes = [ZMAX / 2 + ZMAX / 2 * mp.cos(mp.pi * (2 * i + 1) / (2 * n)) for i in range(n)]
    a = mp.matrix([[z ** j for j in range(n)] for z in nodes])
    c = mp.lu_solve(a, mp.matrix([f(z) for z in nodes]))
    return [c[j] for j in range(n)]


def main():
    for name, f in (("kS", s_fn), ("kH", h_fn)):
        c = interpolate(f)
        err = max(abs(sum(c[j] * z ** j for j in range(DEG + 1)) - f(z)) for z in [ZMAX * i / 4000 for i in range(4001)])
        q = [int(mp.nint(v * 2 ** 55)) for v in c]
        print(f"// interpolation error {mp.nstr(err, 3)}")
        print("constexpr int64_t " + ", ".join(f"{name}{j} = {v}LL" for j, v in enumerate(q)) + ";")


if __name__ == "__main__":
    main()
