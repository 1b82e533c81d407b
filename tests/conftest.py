import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    import torch
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def load_npz(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as d:
        return {k: d[k] for k in d.files}


def load_json(name):
    with open(os.path.join(GOLDEN, name + ".json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def kat():
    return load_json("kat")


@pytest.fixture(scope="session")
def ref_stats():
    return load_json("stats")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build as ob
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build", "libsdemc_oracle.so")):
        ob.build()
    from oracle import oracle
    return oracle
