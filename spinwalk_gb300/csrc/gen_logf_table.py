"""Generates sw_logf_table.h: the 64-entry reduction table of the library's float-float logf
candidate (sw_logf.h). Run once; the output is committed so host and device use identical
constants on every platform.

Bucket j covers the float bit patterns im in [0x3f400000 + j*2^17, 0x3f400000 + (j+1)*2^17),
i.e. the reduced argument m in [0.75, 1.5). For each bucket: invc = float(1/center), and
L = log(1/invc) split into float hi + float lo, computed with 60-digit mpmath. The bucket just
below 1.0 uses invc = 1, L = 0 exactly, so log(x) for x -> 1 has no cancellation.
"""
import os
import struct

import mpmath

mpmath.mp.dps = 60


def f32(x):
    return struct.unpack("<f", struct.pack("<f", float(x)))[0]


def bits2f(b):
    return struct.unpack("<f", struct.pack("<I", b))[0]


def main():
    rows = []
    for j in range(64):
        lo = bits2f(0x3F400000 + j * (1 << 17))
        hi = bits2f(0x3F400000 + (j + 1) * (1 << 17))
        if hi == 1.0:                      # bucket [0.9921875, 1): reduce by exactly 1
            invc, lhi, llo = 1.0, 0.0, 0.0
        else:
            c = (mpmath.mpf(lo) + mpmath.mpf(hi)) / 2
            invc = f32(1 / c)
            L = -mpmath.log(mpmath.mpf(invc))
            lhi = f32(L)
            llo = f32(L - mpmath.mpf(lhi))
        rows.append((invc, lhi, llo))
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "sw_logf_table.h"), "w") as f:
        f.write("// Generated by gen_logf_table.py -- do not edit.\n")
        f.write("// {invc, Lhi, Llo} per bucket of the reduced argument m in [0.75, 1.5).\n")
        f.write("#pragma once\n")
        f.write("#define SW_LOGF_TABLE_INIT { \\\n")
        for invc, lhi, llo in rows:
            f.write("    %s, %s, %s, \\\n" % (float.hex(invc) + "f", float.hex(lhi) + "f",
                                               float.hex(llo) + "f"))
        f.write("}\n")


if __name__ == "__main__":
    main()
