"""The drop-in C++ headers (include/paliwa/) against the reference itself.

tests/cpp/domains_probe.cpp includes paliwa_domains.hpp,
paliwa_dimensions.hpp and paliwa_utils.hpp by name and prints the results of
their index maps, domain operations and planner helpers for cases read from
its input; each line is compared with the same function of the reference's
own headers compiled here (oracle/_ref, through oracle/reference.py). Host
only; skipped where the reference checkout is absent.
"""
import os
import subprocess

import numpy as np
import pytest

import reference as R

pytestmark = pytest.mark.skipif(not R.available(),
                                reason="reference checkout not present")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    R.build()
    exe = str(tmp_path_factory.mktemp("probe") / "domains_probe")
    r = subprocess.run(
        ["g++", "-std=c++20", "-O1", "-I" + os.path.join(ROOT, "include"),
         os.path.join(ROOT, "tests", "cpp", "domains_probe.cpp"), "-o", exe],
        capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def run(lines):
        out = subprocess.run([exe], input="\n".join(lines) + "\n",
                             capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
        return out.stdout.split("\n")[:len(lines)]
    return run


def ints(s):
    return [int(x) for x in s.split()]


def test_index_maps(probe):
    rng = np.random.default_rng(31)
    cases, want = [], []
    for _ in range(400):
        n = int(rng.integers(1, 5))
        l = [int(rng.integers(0, 8)) for _ in range(n)]
        L = [x + int(rng.integers(0, 4)) for x in l]
        lb = [int(rng.integers(0, 9)) for _ in range(n)]
        for kind, cmd in ((0, "sdl"), (1, "shd")):
            cases.append(" ".join(map(str, [cmd, n] + l + L + lb)))
            f, e, s = R.level_domain(kind, l, L, lb)
            want.append(list(f) + list(e) + list(s))
        # the strided domain restricted to a box
        f, e, s = R.level_domain(0, l, L)
        bf = [int(rng.integers(0, 1 << x)) for x in L]
        be = [int(rng.integers(1, (1 << x) - b + 1)) for x, b in zip(L, bf)]
        cases.append(" ".join(map(str, ["rsd", n] + list(f) + list(e) +
                                  list(s) + bf + be)))
        rf, re_, rs = R.restrict_strided_with_discrete((f, e, s), bf, be)
        want.append(list(rf) + list(re_) + list(rs))
    got = probe(cases)
    for c, g, w in zip(cases, got, want):
        assert ints(g) == w, c


def test_dimensions_and_subspaces(probe):
    cases, want = [], []
    for n in (1, 2, 3, 7, 8, 64, 1000, 4096):
        cases.append(f"pui {n}")
        want.append(R.periodic_unit_interval(n))
    for lv in ((2, 1), (0, 3, 1), (1, 1, 1, 2), (3,), (0,)):
        cases.append(" ".join(map(str, ["ihs", len(lv)] + list(lv))))
        want.append(R.hierarchical_subspaces(lv))
    got = probe(cases)
    for c, g, w in zip(cases, got, want):
        if c.startswith("pui"):
            assert [float(x) for x in g.split()] == w, c
        else:
            assert [tuple(int(v) for v in t.strip(",").split(","))
                    for t in g.split()] == w, c


def test_planner_helpers(probe):
    rng = np.random.default_rng(37)
    cases, want = [], []
    for _ in range(300):
        period = 1 << int(rng.integers(1, 8))
        k = int(rng.integers(1, period + 1))
        idx = sorted(int(v) for v in rng.choice(period, k, replace=False))
        cases.append(" ".join(map(str, ["cpb", period, k] + idx)))
        want.append(list(R.covering_periodic_bounds(idx, period)))
    for _ in range(400):
        L = int(rng.integers(1, 9))
        level = int(rng.integers(1, L + 1))
        pl = int(rng.integers(1, level + 1))
        step = 1 << (L - pl + 1)
        first = ((int(rng.integers(0, 1 << L)) // step) * step +
                 int(rng.integers(0, 2)) * (step // 2)) % (1 << L)
        last = (first + int(rng.integers(0, 1 << L)) // step * step) % (1 << L)
        origin = int(rng.integers(0, 1 << level)) << (L - level)
        cases.append(f"pps {first} {last} {origin} {level} {L} {pl}")
        want.append([v for s in R.pole_pass_segments((first, last), origin,
                                                     level, L, pl) for v in s])
    for _ in range(300):
        P = 1 << int(rng.integers(1, 8))
        s0 = min(P, 1 << int(rng.integers(0, 3)))
        e0 = int(rng.integers(1, P // s0 + 1))
        f0 = int(rng.integers(0, P - (e0 - 1) * s0))
        b = (int(rng.integers(0, P)), int(rng.integers(0, P)))
        if rng.random() < 0.1:
            b = (-1, -1)
        cases.append(f"rpb {f0} 3 {e0} 2 {s0} 5 {b[0]} {b[1]} {P}")
        want.append([v for p in R.restrict_periodic_bounds_2d(
            (f0, 3), (e0, 2), (s0, 5), b, P) for t in p for v in t])
    for _ in range(200):
        L = int(rng.integers(1, 8))
        P = 1 << L
        nb = int(rng.integers(1, L + 2))
        bounds = []
        for h in range(nb):
            if rng.random() < 0.3:
                bounds.append((-1, -1))
                continue
            st = P if h == 0 else 2 << (L - h)
            off = 0 if h == 0 else 1 << (L - h)
            a = off + st * int(rng.integers(0, max(1, P // st)))
            c = off + st * int(rng.integers(0, max(1, P // st)))
            bounds.append((a % P, c % P))
        cases.append(" ".join(map(str, ["ftb", L, nb] +
                                  [v for b in bounds for v in b])))
        want.append(R.for_each_transform_index(bounds, L))
    for _ in range(300):
        L = int(rng.integers(1, 9))
        l = int(rng.integers(1, L + 1))
        lmin = int(rng.integers(0, l + 1))
        sp = 1 << (L - l)
        lf = int(rng.integers(0, 1 << l)) * sp
        le = int(rng.integers(1, (1 << L) - lf + 1))
        fwd = int(rng.integers(0, 2))
        w = ["hat", "biorthogonal", "fullweighting"][int(rng.integers(0, 3))]
        cases.append(f"rtd {fwd} {l} {lmin} {L} {lf} {le} {w}")
        try:
            want.append(R.required_transform_domain(fwd, l, lmin, L, lf, le, w))
        except RuntimeError:
            want.append("error")
    got = probe(cases)
    for c, g, w in zip(cases, got, want):
        if w == "error":
            assert g.startswith("error"), c
        elif c.startswith("rpb"):
            assert ints(g.replace("|", "")) == w, c
        elif c.startswith("pps"):
            assert [int(v) for t in g.split() for v in t.split(",")] == w, c
        else:
            assert ints(g) == w, c
