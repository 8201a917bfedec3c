import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    from clblm_gb300 import build as B
    B.build()
    from clblm_gb300 import capi
    return capi


GOLDEN = ROOT / "tests" / "golden"


@pytest.fixture(scope="session")
def mtckd():
    """The reference's MT_CKD H2O table, 0-3000 cm-1 (tests/golden)."""
    import numpy as np
    from clblm_gb300.capi_types import Continuum
    z = np.load(GOLDEN / "mtckd_h2o_0_3000.npz")
    wv = z["wavenumbers"]
    return Continuum(wv[0], wv[1] - wv[0], z["self_absco_ref"], z["for_absco_ref"], z["self_texp"],
                     float(z["ref_press"]), float(z["ref_temp"]))
