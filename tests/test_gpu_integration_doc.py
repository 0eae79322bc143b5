"""The in-process ctypes stub printed in INTEGRATION.md runs as written against
the built library and returns what the Python front end returns."""
import os
import re

import numpy as np
import pytest

from sgfim import datagen

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integration_ctypes_stub(tmp_path):
    from sgfim import _lib
    from sgfim.engine import Engine
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = next(b for b in re.findall(r"```python\n(.*?)```", doc, re.S) if "def run_gb300" in b)
    code = block.replace('"<repo>/20261008-self-growing-evidence-agent_gb300/sgfim/_lib/libsgfim.so"',
                         repr(_lib.LIB_PATH))
    ns = {}
    exec(compile(code, "INTEGRATION.md", "exec"), ns)
    rows = datagen.regime_txns(3000, 8, 5, 4, 0.3, seed=12)
    path = tmp_path / "w.txt"
    path.write_text("".join(" ".join(str(int(x) + 1) for x in r) + "\n" for r in rows))
    got = ns["run_gb300"](str(path), 120)
    assert got["ok"]
    with Engine() as eng:
        eng.load_fimi(str(path))
        want = eng.mine(120).as_dict()
    assert got["mfis"] == want and len(want) > 0
