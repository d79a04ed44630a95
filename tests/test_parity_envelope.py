"""The parity bar itself (tests/parity.py), on the golden fixtures: every
build's own result passes, and planted deviations -- an iteration count
outside the branch's range, eigenvalues off by more than the bar -- fail,
including in a case where the reference's builds branch."""
import json
import os

import numpy as np
import pytest

from tests import parity

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(HERE, name + ".json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", ["lap20_k10", "bad_initial_block", "constraints_diag40",
                                  "fail_gevp", "wrong_constraints"])
def test_every_reference_build_passes(name):
    g = load(name)
    for r in parity.runs(g):
        parity.check(g, r["flag"], r["iterations"], r["lambda"])


def test_branching_case_bounds_iterations_by_the_branch_taken():
    g = load("bad_initial_block")  # two builds fail at setup, one converges in 40
    conv = [r for r in parity.runs(g) if r["flag"] == 0][0]
    with pytest.raises(AssertionError):
        parity.check(g, -1, 37, g["lambda"])  # a late failure is not a setup failure
    with pytest.raises(AssertionError):
        parity.check(g, 0, conv["iterations"] + 10, conv["lambda"])


def test_branching_case_still_checks_eigenvalues():
    g = load("bad_initial_block")
    conv = [r for r in parity.runs(g) if r["flag"] == 0][0]
    lam = np.array(conv["lambda"]) * (1 + 1e-7)
    with pytest.raises(AssertionError):
        parity.check(g, 0, conv["iterations"], lam)


def test_wrong_eigenvalues_fail_where_builds_agree():
    g = load("constraints_diag40")
    lam = np.array(g["lambda"])
    lam[1] *= 1 + 1e-8
    with pytest.raises(AssertionError):
        parity.check(g, g["flag"], g["iterations"], lam)
    with pytest.raises(AssertionError):
        parity.check(g, g["flag"], g["iterations"] + 3, g["lambda"])
