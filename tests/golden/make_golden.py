"""Generates tests/golden/plan_multipass.npz.

The vectors come from the reference's own in-test 1D periodic reference loop,
test/test_paliwa_plan.cpp:114-139 (TEST transform_plan.multipass_sparse_values):
maximum level 6 (period 64), transform level 4 (spacing 4), input
1 + sin(0.7 i), every filter parity mask of 1..5 passes with coefficients
{-.5, 1, .125} on even pass indices and {0, 1, .25} on odd ones, and both
level orders {4,3,2,1} and {1,2,3,4}. The loop below restates those lines:

    for l in levels:
        stride = 1 << (maximum - l)
        for (offset, f) in filters:
            for i in range(offset * stride, period, 2 * stride):
                ref[i] = f0*ref[(i + period - stride) % period]
                         + f1*ref[i] + f2*ref[(i + stride) % period]

Run: python tests/golden/make_golden.py
"""
import math
import os

import numpy as np

MAXIMUM, LEVEL, PERIOD = 6, 4, 64


def filters_for(passes, mask):
    out = []
    for p in range(passes):
        off = 1 if mask & (1 << p) else 0
        co = (0.0, 1.0, 0.25) if p % 2 else (-0.5, 1.0, 0.125)
        out.append((off, co))
    return out


def reference_loop(inp, levels, filters):
    ref = list(inp)
    for l in levels:
        stride = 1 << (MAXIMUM - l)
        for off, f in filters:
            for i in range(off * stride, PERIOD, 2 * stride):
                ref[i] = (f[0] * ref[(i + PERIOD - stride) % PERIOD]
                          + f[1] * ref[i]
                          + f[2] * ref[(i + stride) % PERIOD])
    return ref


def main():
    inp = [1.0 + math.sin(i * 0.7) for i in range(PERIOD)]
    cases, outs = [], []
    for passes in range(1, 6):
        for mask in range(1 << passes):
            for order, levels in enumerate(([4, 3, 2, 1], [1, 2, 3, 4])):
                cases.append((passes, mask, order))
                outs.append(reference_loop(inp, levels,
                                           filters_for(passes, mask)))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        "plan_multipass.npz")
    np.savez_compressed(path, input=np.array(inp),
                        cases=np.array(cases, dtype=np.int64),
                        output=np.array(outs))
    print(path, len(cases))


if __name__ == "__main__":
    main()
