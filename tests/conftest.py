import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden_energies():
    return json.loads((GOLDEN / "energies.json").read_text())


@pytest.fixture(scope="session")
def golden_tables():
    meta = json.loads((GOLDEN / "tables_digest.json").read_text())
    arrays = np.load(GOLDEN / "tables_small.npz")
    return meta, arrays


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def edlib():
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import _build, _capi
    _build.build()
    return _capi.load()


@pytest.fixture(scope="session")
def ed(edlib):
    import exact_diagonalization_for_fermionic_systems_with_gpu_gb300 as pkg
    return pkg


def philox_uniform(seed: int, n: int, scale: float = 1.0) -> np.ndarray:
    from oracle.oracle import philox_uniform as pu
    return pu(seed, n, scale)


def rel_err(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
