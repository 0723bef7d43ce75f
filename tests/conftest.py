import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")
DATA = os.path.join(REPO, "g4hepem_gb300", "data")
T3 = os.path.join(DATA, "three_couples_0.7mm.json")
T16 = os.path.join(DATA, "random16_two_regions.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    assert O.build_port(), "could not build the CPU port (oracle/Makefile)"
    libs = {}

    def get(path):
        if path not in libs:
            libs[path] = O.PortLib().load(path)
        return libs[path]
    return get


@pytest.fixture(scope="session")
def ref():
    """The reference itself, where its sources are present (this container)."""
    from oracle import oracle as O
    if not os.path.isdir(O.reference_dir()) or not O.build_ref():
        pytest.skip("reference sources not available on this host")
    libs = {}

    def get(path):
        if path not in libs:
            libs[path] = O.RefLib().load(path)
        return libs[path]
    return get


@pytest.fixture(scope="session")
def native():
    from g4hepem_gb300 import build as B
    B.build()
    from g4hepem_gb300 import native as N
    N.lib()
    return N


@pytest.fixture(scope="session")
def gpu_ctx(native):
    if not has_gpu():
        pytest.skip("no GPU")
    ctxs = {}

    def get(path):
        if path not in ctxs:
            ctxs[path] = native.Context(path)
        return ctxs[path]
    yield get
    for c in ctxs.values():
        c.close()


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def golden_state(g, prefix, which="in"):
    from g4hepem_gb300.workload import STATE_FIELDS
    return {f: np.ascontiguousarray(g[f"{prefix}{which}_{f}"]) for f in STATE_FIELDS}


def golden_res(g, prefix):
    from g4hepem_gb300.native import OUT_FIELDS
    return {f: g[f"{prefix}res_{f}"] for f, _, _ in OUT_FIELDS}
