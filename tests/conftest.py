import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Builds the library and the oracle once if they are missing."""
    from cdmf_gb300 import _build
    from oracle import oracle
    if not os.path.exists(_build.LIB):
        _build.build()
    if not (os.path.exists(os.path.join(oracle.HERE, "liboracle_f32.so"))
            and os.path.exists(os.path.join(oracle.HERE, "liboracle_f64.so"))):
        oracle.build()
    yield


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    import numpy as np
    from cdmf_gb300.formats import RatingMatrix
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    R = RatingMatrix(int(z["m"]), int(z["n"]), z["csr_ptr"], z["csr_idx"], z["csr_val"], z["csc_ptr"],
                     z["csc_idx"], z["csc_val"], z["te_row"], z["te_col"], z["te_val"])
    return R, z
