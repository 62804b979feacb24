"""The EAS enhancement mapping of the reference on distorted hexes, held by two
independent restatements: the oracle's entry-by-entry C++ element
(oracle/oracle.cpp) and a whole-matrix numpy one
(tests/golden/make_eas_distorted.py), both following
src/elements/solid_elements.cpp:1054-1206 with the row of J0^-1 as the mode
gradient (:1132-1134).  On these elements the textbook column form differs by
percents, so agreement to 1e-13 pins the reference's form."""
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import make_eas_distorted as ME  # noqa: E402


@pytest.fixture(scope="module")
def fixture():
    with open(os.path.join(GOLDEN, "eas_distorted_hex.json")) as fh:
        return json.load(fh)["cases"]


def test_fixture_is_the_numpy_restatement(fixture):
    for c in fixture:
        K = ME.eas_ke(np.array(c["xyz"]), c["E"], c["nu"])
        ref = np.array(c["ke"])
        assert np.abs(K - ref).max() <= 1e-14 * np.abs(ref).max(), c["name"]


def test_oracle_matches_numpy_restatement_on_distorted_hexes(oracle, fixture):
    for c in fixture:
        ref = np.array(c["ke"])
        K = oracle.chexa8_ke(np.array(c["xyz"]), c["E"], c["nu"], 0)
        assert np.abs(K - ref).max() <= 1e-13 * np.abs(ref).max(), c["name"]
        # the elements exercise the quirk: the textbook mapping is far off
        Kt = ME.eas_ke(np.array(c["xyz"]), c["E"], c["nu"], textbook=True)
        assert np.abs(Kt - ref).max() > 1e-3 * np.abs(ref).max()
        assert np.abs(K - Kt).max() > 1e-3 * np.abs(ref).max()
        # symmetric, and rigid translations in the null space
        assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
        for a in range(3):
            t = np.zeros(24)
            t[a::3] = 1.0
            assert np.abs(K @ t).max() <= 1e-9 * np.abs(K).max()
