"""A live run of the CLI shims reproduces their recorded output
(tests/golden/shim_golden.json, made by tests/golden/make_shim_golden.py):
the same exit code, the same result-file name and, timing values aside, the
same bytes in the result file and on stdout (the dataset's path is stored as
"<fimi>")."""
import hashlib
import json
import os
import re
import subprocess
import sys

import pytest

from sgfim import results

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TIMED = re.compile(r"((?:computation|total|preprocessing)_time\(s\):|runtimePerStage\(s\):)[^\n]*")
STAGE_TIME = re.compile(r"(runtime:) [\d.eE+-]+")


def _untimed(text):
    return STAGE_TIME.sub(r"\1 <t>", TIMED.sub(r"\1 <t>", text))


def test_shims_reproduce_recorded_output(tmp_path):
    gold = json.load(open(os.path.join(HERE, "golden", "shim_golden.json")))
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_shim_golden import fimi_text
    text = fimi_text()
    assert hashlib.sha256(text.encode()).hexdigest() == gold["fimi_sha256"]
    fimi = str(tmp_path / gold["fimi_name"])
    with open(fimi, "w", encoding="utf-8") as f:
        f.write(text)
    for case in gold["cases"]:
        out = results.result_path(case["kind"], fimi, case["arg"])
        assert os.path.basename(out) == gold["fimi_name"] + case["results_name"]
        p = subprocess.run([os.path.join(results.LIB_DIR, results.SHIMS[case["kind"]]), fimi, case["arg"]],
                           capture_output=True)
        assert p.returncode == case["exit_code"]
        assert _untimed(p.stdout.decode("utf-8").replace(fimi, "<fimi>")) == _untimed(case["stdout"])
        with open(out, encoding="utf-8") as f:
            assert _untimed(f.read().replace(fimi, "<fimi>")) == _untimed(case["results_text"])
