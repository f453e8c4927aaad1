import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpsat():
    from gpupsat_gb300 import _build
    _build.build()
    import gpupsat_gb300
    return gpupsat_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def bcp_golden():
    z = np.load(GOLDEN / "bcp_golden.npz")
    cases = []
    for i in range(int(z["n_cases"][0])):
        cases.append({k[len(f"c{i}_"):]: z[k] for k in z.files if k.startswith(f"c{i}_")})
    return cases


@pytest.fixture(scope="session")
def scan_golden():
    z = np.load(GOLDEN / "scan_golden.npz")
    cases = []
    for i in range(int(z["n_cases"][0])):
        cases.append({k[len(f"c{i}_"):]: z[k] for k in z.files if k.startswith(f"c{i}_")})
    return cases


@pytest.fixture(scope="session")
def preprocess_golden():
    z = np.load(GOLDEN / "preprocess_golden.npz")
    cases = []
    for i in range(int(z["n_cases"][0])):
        cases.append({k[len(f"p{i}_"):]: z[k] for k in z.files if k.startswith(f"p{i}_")})
    return cases


@pytest.fixture(scope="session")
def cuda_ok(gpsat):
    if gpsat.device_count() == 0:
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return True


def compare_bcp(a: dict, b: dict, trails=None, label=""):
    """Bit-exact comparison of two BCP result dicts (numpy)."""
    T = len(a["status"]) if trails is None else len(trails)
    idx = range(T) if trails is None else trails
    for j, t in enumerate(idx):
        ta = t if trails is None else j
        for key in ("status", "conflict", "stop", "n_impl"):
            assert a[key][ta] == b[key][t], f"{label} trail {t}: {key} {a[key][ta]} != {b[key][t]}"
        k = int(a["n_impl"][ta])
        assert np.array_equal(a["impl_lit"][ta, :k], b["impl_lit"][t, :k]), f"{label} trail {t}: implied literals"
        assert np.array_equal(a["impl_reason"][ta, :k], b["impl_reason"][t, :k]), f"{label} trail {t}: reasons"
