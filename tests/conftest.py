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
    """Split-FP8 tensor-core engine on the counter sketch stream (the tests
    that compare with the oracle's counter stream use it; test_gpu_rng covers
    the default ChaCha8 stream)."""
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8, rng=sg.SketchRng.COUNTER)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engine_bf16():
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_BF16, rng=sg.SketchRng.COUNTER)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engines(engine, engine_bf16, engine_fp32):
    return {"fp8": engine, "bf16": engine_bf16, "fp32": engine_fp32}


@pytest.fixture(scope="session")
def engine_fp32():
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.FP32, rng=sg.SketchRng.COUNTER)
    yield eng
    eng.close()
