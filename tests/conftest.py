import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "swap-assembler_gb300", ROOT / "oracle", ROOT / "tests" / "golden", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def native_built():
    """Build the native library, the generator and the oracle once if missing."""
    pkg = ROOT / "swap-assembler_gb300"
    need = [pkg / "libswapgb.so", pkg / "libswgsynth.so", pkg / "bin" / "swap",
            ROOT / "oracle" / "build" / "liboracle.so"]
    if not all(p.exists() for p in need):
        import importlib.util
        spec = importlib.util.spec_from_file_location("swg_build", pkg / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        mod.build_oracle()
    return True
