import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libhx.so")


def _cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_ok():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def hx():
    """The libhx Python mirror, with libhx.so built in-tree if needed."""
    import hashinator_gb300 as hxmod
    from hashinator_gb300 import build
    if not hxmod.LIB_PATH.exists():
        build.build_lib()
    hxmod.lib()
    return hxmod


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.lib()
    return oracle


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def golden_extra_cases():
    """Edge-case fixtures (tests/golden/extra/), loaded as "extra/<name>"."""
    return sorted(f"extra/{p.stem}" for p in (GOLDEN / "extra").glob("*.npz"))


def load_golden(name):
    import numpy as np
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}
