import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"
# The reference checkout, when the environment names one (REF_DIR); tests
# that compile or run the reference's own sources skip without it.
REF_DIR = Path(os.environ["REF_DIR"]) if os.environ.get("REF_DIR") else None
HAVE_REF = REF_DIR is not None and (REF_DIR / "refgas.h").exists()
REF_SKIP = "reference sources absent (set REF_DIR to a reference checkout)"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_names():
    # engine cases; the other fixtures cover CSR ties and the text formats
    other = {"csr_ties", "text_formats", "ref_written_mtx"}
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if p.stem not in other)


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def libgas():
    from graphreduce_gb300.build import build, build_oracle
    from graphreduce_gb300 import _lib
    build()
    build_oracle(with_reference=HAVE_REF)
    return _lib.load()
