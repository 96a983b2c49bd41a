"""Generate the FP32 polynomial coefficients used by ``spp_fp32.h``.

The device kernels and the CPU FP32 mirror must evaluate sin/cos/atan/log/exp
with *identical* arithmetic so that the two produce bit-identical trajectories.
CUDA's and libm's transcendental functions differ in their last bits, so this
project carries its own: Cody-Waite range reduction (Cody & Waite, "Software
Manual for the Elementary Functions", 1980) followed by a polynomial whose
coefficients are fitted here by weighted least squares on Chebyshev nodes
(relative-error weighting), then rounded to float32.

Run ``python gen_fp32_poly.py`` to print the constant block that is pasted into
``spp_fp32.h``.  The accuracy of the resulting functions is checked against
FP64 libm in ``tests/test_fp32_math.py``.
"""
import numpy as np


def cheb_nodes(a, b, n=4000):
    k = np.arange(n)
    x = np.cos(np.pi * (k + 0.5) / n)
    return 0.5 * (a + b) + 0.5 * (b - a) * x


def fit(xs, target, basis_pows, weight):
    A = np.stack([xs ** p for p in basis_pows], axis=1) * weight[:, None]
    c, *_ = np.linalg.lstsq(A, target * weight, rcond=None)
    return c


def f32(v):
    return float(np.float32(v))


def main():
    out = {}
    # sin(r) = r + r^3 * P(r^2), |r| <= pi/4 ; fit P on z=r^2
    r = cheb_nodes(1e-4, np.pi / 4)
    z = r * r
    P = fit(z, (np.sin(r) - r) / r ** 3, [0, 1, 2, 3], np.abs(r ** 3 / np.sin(r)))
    out["SIN"] = [f32(c) for c in P]
    # cos(r) = 1 - r^2/2 + r^4 * Q(r^2)
    Q = fit(z, (np.cos(r) - 1 + z / 2) / z ** 2, [0, 1, 2, 3], z ** 2 / np.cos(r))
    out["COS"] = [f32(c) for c in Q]
    # atan(t) = t + t^3 * A(t^2), |t| <= tan(pi/8)
    t = cheb_nodes(1e-4, np.sqrt(2) - 1)
    u = t * t
    Acoef = fit(u, (np.arctan(t) - t) / t ** 3, list(range(7)), np.abs(t ** 3 / np.arctan(t)))
    out["ATAN"] = [f32(c) for c in Acoef]
    # log(m) = 2 s + s^3 * R(s^2), s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)]
    smax = (np.sqrt(2) - 1) / (np.sqrt(2) + 1)
    s = cheb_nodes(1e-4, smax)
    w = s * s
    R = fit(w, (2 * np.arctanh(s) - 2 * s) / s ** 3, [0, 1, 2, 3], np.abs(s ** 3 / (2 * np.arctanh(s))))
    out["LOG"] = [f32(c) for c in R]
    # exp(r) = 1 + r + r^2 * E(r), |r| <= ln2/2
    rr = cheb_nodes(-np.log(2) / 2, np.log(2) / 2)
    E = fit(rr, (np.exp(rr) - 1 - rr) / rr ** 2, list(range(6)), rr ** 2 / np.exp(rr))
    out["EXP"] = [f32(c) for c in E]

    def hexf(v):
        return np.float32(v).view(np.uint32)

    for name, cs in out.items():
        for i, c in enumerate(cs):
            print(f"#define SPP_{name}_C{i} {c!r:>24}f  /* 0x{hexf(c):08x} */")
    # Cody-Waite splits of pi/2 and ln2 (leading parts keep 12 significant bits)
    def split(v, bits=12):
        m, e = np.frexp(v)
        hi = np.ldexp(np.round(np.ldexp(m, bits)), e - bits)
        return hi
    pio2 = np.pi / 2
    hi = split(pio2)
    mid = split(pio2 - hi)
    lo = f32(pio2 - hi - mid)
    print(f"#define SPP_PIO2_HI {f32(hi)!r}f\n#define SPP_PIO2_MID {f32(mid)!r}f\n#define SPP_PIO2_LO {lo!r}f")
    ln2 = np.log(2.0)
    lhi = split(ln2)
    print(f"#define SPP_LN2_HI {f32(lhi)!r}f\n#define SPP_LN2_LO {f32(ln2 - lhi)!r}f")


if __name__ == "__main__":
    main()
