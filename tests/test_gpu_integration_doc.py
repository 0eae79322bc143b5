"""The in-process ctypes stub that INTEGRATION.md points maintainers to
(sgfim/examples/ctypes_adapter_stub.py) runs against the built library and
returns what the Python front end returns."""
import importlib.util
import os

import pytest

from sgfim import datagen

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300", "sgfim", "examples", "ctypes_adapter_stub.py")


def test_integration_ctypes_stub(tmp_path):
    from sgfim.engine import Engine
    spec = importlib.util.spec_from_file_location("ctypes_adapter_stub", STUB)
    stub = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(stub)
    rows = datagen.regime_txns(3000, 8, 5, 4, 0.3, seed=12)
    path = tmp_path / "w.txt"
    path.write_text("".join(" ".join(str(int(x) + 1) for x in r) + "\n" for r in rows))
    got = stub.run_gb300(str(path), 120)
    assert got["ok"]
    with Engine() as eng:
        eng.load_fimi(str(path))
        want = eng.mine(120).as_dict()
    assert got["mfis"] == want and len(want) > 0
