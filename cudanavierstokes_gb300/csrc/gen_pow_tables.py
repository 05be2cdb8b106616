"""Generate pow_tables.h: the 64-entry tables of the FP64 power x^a used for the viscosity
law (pow_visc in cns_common.cuh), computed with 60-digit arithmetic (mpmath) and written as
exact hexadecimal double literals.

  kPowRcp[i]            r_i = 1 / c_i rounded to double, c_i = 1 + (i + 1/2) / 64
  kPowLnHi/Lo[i]        -ln(r_i) as a double-double (hi + lo)
  kPowExpHi/Lo[i]       2^(i/64) as a double-double
  POW_LN2_HI / LO       ln(2) split: hi with 42 significant bits (k * hi exact for the
                        binary exponents |k| < 2^11 of finite doubles), lo the rest
  POW_LN2_64_HI / LO    ln(2)/64 split: hi with 40 significant bits (j * hi exact for
                        |j| < 2^13), lo the rest

Run from this directory: python gen_pow_tables.py > pow_tables.h
"""
import mpmath

mpmath.mp.dps = 60


def dd(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def main():
    rcp, lnh, lnl, exh, exl = [], [], [], [], []
    for i in range(64):
        c = 1 + (mpmath.mpf(i) + mpmath.mpf("0.5")) / 64
        r = float(1 / c)
        rcp.append(r)
        h, l = dd(-mpmath.log(mpmath.mpf(r)))
        lnh.append(h); lnl.append(l)
        h, l = dd(mpmath.power(2, mpmath.mpf(i) / 64))
        exh.append(h); exl.append(l)

    def split(v, bits):
        m, e = mpmath.frexp(v)
        hi = float(mpmath.ldexp(mpmath.floor(mpmath.ldexp(m, bits)), e - bits))
        return hi, float(v - mpmath.mpf(hi))

    l2h, l2l = split(mpmath.log(2), 42)
    hi, lo = split(mpmath.log(2) / 64, 40)

    def arr(name, vals):
        body = ",\n".join("    " + ", ".join(v.hex() for v in vals[k:k + 4]) for k in range(0, 64, 4))
        return f"static __device__ const double {name}[64] = {{\n{body}}};\n"

    print("// pow_tables.h -- generated by gen_pow_tables.py (do not edit): the tables of the FP64")
    print("// power x^a of the viscosity law (pow_visc, cns_common.cuh).")
    print("#pragma once\n")
    print(f"#define POW_LN2_HI {l2h.hex()}")
    print(f"#define POW_LN2_LO {l2l.hex()}")
    print(f"#define POW_LN2_64_HI {hi.hex()}")
    print(f"#define POW_LN2_64_LO {lo.hex()}\n")
    for name, vals in (("kPowRcp", rcp), ("kPowLnHi", lnh), ("kPowLnLo", lnl), ("kPowExpHi", exh),
                       ("kPowExpLo", exl)):
        print(arr(name, vals))


if __name__ == "__main__":
    main()
