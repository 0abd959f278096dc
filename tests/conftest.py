"""Shared test setup: import paths, the `gpu` marker and golden-case helpers."""
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(REPO, "doe-csfg-hackathon_gb300")
for p in (PKG_ROOT, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden", "gpp_golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


def unhex(pairs):
    if pairs is None:
        return None
    return np.array([complex(float.fromhex(a), float.fromhex(b)) for a, b in pairs])


def case_inputs(case):
    from gppsigma import workload as W
    if case["kind"] == "ramp":
        return W.ramp_inputs(*case["args"])
    return W.make_inputs(W.Shape(**case["shape"]), case["seed"])


def rel_err(got, want):
    """Per real/imaginary component relative error, max over the array.
    Components whose reference value is exactly zero are compared absolutely."""
    got = np.asarray(got, dtype=np.complex128).ravel()
    want = np.asarray(want, dtype=np.complex128).ravel()
    g = np.concatenate([got.real, got.imag])
    w = np.concatenate([want.real, want.imag])
    den = np.where(w == 0.0, 1.0, np.abs(w))
    return float(np.max(np.abs(g - w) / den)) if g.size else 0.0


@pytest.fixture(scope="session")
def golden_cases():
    return load_golden()
