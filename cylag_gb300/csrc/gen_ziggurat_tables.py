"""Generate ziggurat_tables.h: the 128-layer normal ziggurat tables of
Marsaglia & Tsang (2000), built with the recurrence CyLag uses at import
(cylag/lsm/random_utils.pyx:118-146) and the host libm (math.exp/log/sqrt
call the C library).  Written as hexadecimal floats so that the device and
every host read the identical bits.

Usage: python cylag_gb300/csrc/gen_ziggurat_tables.py > cylag_gb300/csrc/ziggurat_tables.h
"""
import math


def tables():
    kn = [0] * 128
    wn = [0.0] * 128
    fn = [0.0] * 128
    m1 = 2147483648.0
    dn = 3.442619855899
    tn = dn
    vn = 9.91256303526217e-3
    q = vn / math.exp(-0.5 * dn * dn)
    kn[0] = int((dn / q) * m1) & 0xFFFFFFFF
    kn[1] = 0
    wn[0] = q / m1
    wn[127] = dn / m1
    fn[0] = 1.0
    fn[127] = math.exp(-0.5 * dn * dn)
    for i in range(126, 0, -1):
        dn = math.sqrt(-2.0 * math.log(vn / dn + math.exp(-0.5 * dn * dn)))
        kn[i + 1] = int((dn / tn) * m1) & 0xFFFFFFFF
        tn = dn
        fn[i] = math.exp(-0.5 * dn * dn)
        wn[i] = dn / m1
    return kn, wn, fn


def main():
    kn, wn, fn = tables()
    out = ["/* Generated by gen_ziggurat_tables.py -- do not edit. */",
           "#pragma once",
           "#define CG_ZIG_KN_INIT { \\"]
    out += ["    %du, \\" % v for v in kn] + ["}", "#define CG_ZIG_WN_INIT { \\"]
    out += ["    %s, \\" % v.hex() for v in wn] + ["}", "#define CG_ZIG_FN_INIT { \\"]
    out += ["    %s, \\" % v.hex() for v in fn] + ["}"]
    print("\n".join(out))


if __name__ == "__main__":
    main()
