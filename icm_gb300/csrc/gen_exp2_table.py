"""Writes exp2_table.cuh: 2^(j/128), j = 0..127, as double-double pairs
(hi = the value rounded to double, lo = the remainder rounded to double),
computed at 60 significant digits.  The table is data for the leaf factor's
exponential (leafdiv.cuh); rerun this script to regenerate it."""
import os

import mpmath

mpmath.mp.dps = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rows = []
    for j in range(128):
        v = mpmath.power(2, mpmath.mpf(j) / 128)
        hi = float(v)
        lo = float(v - mpmath.mpf(hi))
        rows.append(f"    {{{hi.hex()}, {lo.hex()}}},   // 2^({j}/128)")
    body = "\n".join(rows)
    text = f"""// exp2_table.cuh -- 2^(j/128), j = 0..127, as double-double pairs {{hi, lo}}.
// Written by gen_exp2_table.py (60-digit arithmetic); do not edit by hand.
#pragma once

namespace icmg {{

__device__ static const double kExp2Tab[128][2] = {{
{body}
}};

}}  // namespace icmg
"""
    with open(os.path.join(HERE, "exp2_table.cuh"), "w") as f:
        f.write(text)


if __name__ == "__main__":
    main()
