import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
METRICS = ["TV", "CN", "TM", "MSM", "MSV", "MSRV"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def fp():
    from fastpartitioner_gb300 import build
    build.build()
    import fastpartitioner_gb300
    return fastpartitioner_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_engine(fp):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    eng = fp.Engine(0)
    yield eng
    eng.close()


def golden_cases():
    return sorted(GOLDEN.glob("*.npz"))


def load_golden(path):
    """(Hypergraph, passes, Ks, npz) for one committed fixture."""
    import fastpartitioner_gb300 as fpk
    z = np.load(path)
    nov, noe, passes = (int(x) for x in z["dims"])
    hg = fpk.Hypergraph(nov, noe, z["vptr"], z["vnets"], z["nptr"], z["npins"], z["src"])
    return hg, passes, [int(k) for k in z["Ks"]], z
