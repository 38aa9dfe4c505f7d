"""Shared test set-up: the `gpu` marker, import paths and golden fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "late: a path whose first GPU run this is; runs last")


def pytest_collection_modifyitems(config, items):
    # tests marked late go after the others (stable order otherwise), so
    # that under -x a failure there hides no other result
    items.sort(key=lambda it: it.get_closest_marker("late") is not None)


def golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def golden_path(name):
    return os.path.join(GOLDEN, name)


def tables(kind):
    """(pair, rho, embed) fixture table files of a golden case family."""
    if kind == "lj":
        return (golden_path("lj.pt"),)
    if kind == "lj_f1":
        return (golden_path("lj_f1.pt"),)
    return tuple(golden_path(kind + ext) for ext in (".pt", ".rho", ".emb"))


@pytest.fixture
def gold():
    return golden
