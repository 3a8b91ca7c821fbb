import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on GB300)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        with np.load(GOLDEN / name) as z:
            return {k: z[k] for k in z.files}
    return load


@pytest.fixture(scope="session")
def parity_report():
    """A dict the parity tests record their measured agreement in; written
    at the end of the session to the JSON file named by $AJG_PARITY_REPORT
    (merged with what the file holds), when that is set."""
    rep = {}
    yield rep
    path = os.environ.get("AJG_PARITY_REPORT")
    if path and rep:
        old = json.loads(Path(path).read_text()) if os.path.exists(path) else {}
        old.update(rep)
        Path(path).write_text(json.dumps(old, indent=1, sort_keys=True) + "\n")
