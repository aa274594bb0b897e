import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a (GB300) device and the built library")


def _gpu_available() -> bool:
    try:
        import schnellfmm_gb300 as sg
        sg.load_library()
        e = sg.Engine()
        e.close()
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine():
    """Default engine: split-FP8 tensor-core path."""
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engine_bf16():
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_BF16)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engines(engine, engine_bf16, engine_fp32):
    return {"fp8": engine, "bf16": engine_bf16, "fp32": engine_fp32}


@pytest.fixture(scope="session")
def engine_fp32():
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.FP32)
    yield eng
    eng.close()
