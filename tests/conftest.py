"""Shared pytest set-up: import paths, the gpu marker, golden fixtures."""

from __future__ import annotations

import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
GOLDEN_CASES = ["smoke6", "rand24", "circle256", "avg_offsets", "blob_frame"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # Enforced by the pytest-timeout plugin where it is installed.
    config.addinivalue_line("markers", "timeout(seconds): fail the test after this many seconds")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def problem_args(d: dict):
    """(src, mask, tgt, mask_on_src, mask_on_tgt, gradient) of a golden case."""
    return (d["src"], d["mask"], d["tgt"], tuple(int(v) for v in d["mask_on_src"]),
            tuple(int(v) for v in d["mask_on_tgt"]), str(d["gradient"]))


@pytest.fixture(params=GOLDEN_CASES)
def golden(request):
    return request.param, load_golden(request.param)
