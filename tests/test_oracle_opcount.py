"""The exact arithmetic of one tet-substep, counted on the FP64 restatement.

oracle/opcount.cpp instantiates the oracle's scalar-generic body
(oracle/xfem_oracle_real.inc) on a counting scalar and runs one coupled tet
solve (SolveElement -> SolveElementMixed + EnergyXpbdConstrainSimultaneous,
XPBDFEM/Fem.cpp:437-564, XPBDFEM/Xpbd.h:123-215) and one vertex's predict and
finalize (XPBDFEM/Geo.cpp:307-344). The counts replace the survey's hand
count of about 440 FLOP per tet-substep in the roofline's compute figure.

Element arithmetic (the scalar R): per coupled Neo-Hookean solve 208 add/sub,
283 mul, 14 div = 505 FLOP (+3 comparisons); Yeoh 533. Position arithmetic
is double in the restatement and counted from the code: 9 subtractions for
the edge vectors and 12 additions for the update per tet; per vertex 18
(velocity, prediction, velocity update) plus 5 in R.
"""
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def counts(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("opcount") / "opcount")
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-w", "-I" + os.path.join(ROOT, "oracle"), "-o",
                    exe, os.path.join(ROOT, "oracle", "opcount.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.strip().splitlines():
        f = line.split()
        res[f[0]] = {f[i]: int(f[i + 1]) for i in range(1, len(f), 2)}
    return res


def test_tet_solve_counts(counts):
    nh, yeoh = counts["tet_solve_nh_coupled"], counts["tet_solve_yeoh_coupled"]
    assert (nh["add"], nh["mul"], nh["div"], nh["sqrt"]) == (208, 283, 14, 0)
    assert nh["flops"] == 505
    assert yeoh["flops"] == 533
    assert nh["cmp"] == 3 and yeoh["cmp"] == 4


def test_vertex_counts(counts):
    v = counts["vertex_predict_finalize"]
    assert v["flops"] == 5


def test_flops_per_tet_substep(counts):
    """On the 1.5M-tet mesh (V/T = 0.17592): 505 + 21 + 0.17592 (5 + 18)."""
    f = counts["tet_solve_nh_coupled"]["flops"] + 9 + 12 + 0.17592 * (counts["vertex_predict_finalize"]["flops"] + 18)
    assert abs(f - 530.05) < 0.01
