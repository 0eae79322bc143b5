"""The reference's own engine adapter, unmodified, on the shims' output.

code/pipeline/engine_adapter.py runs CoParaCG_<engine>.exe <fimi> <thr> from
TENSORFIM_DIR and AnytimeMining.exe <fimi> <stages> (ANYFIM_EXE), then parses
the Results.txt they leave next to the dataset (engine_adapter.py:24-26,
70-131).  Pointing those two globals at the shims is the whole drop-in.  Here
the adapter is imported from the reference checkout named by SGFIM_REFERENCE
(skipped without it: the reference is not shipped with this project), its
globals are patched, and its run_tensorfim / run_anyfim drive executables
that replay the shims' recorded output for the dataset
(tests/golden/shim_golden.json; test_gpu_shims.py checks on a GPU that the
live shims print and write exactly those bytes).  The adapter's answers must
be the oracle's TensorFIM and AnyFIM sets.
"""
import importlib.util
import json
import os
import stat
import sys

import pytest

import oracle
from sgfim import datagen

HERE = os.path.dirname(os.path.abspath(__file__))

REPLAY = '''#!{python}
import json, sys
case = json.load(open({case_path!r}))
fimi = sys.argv[1]
assert sys.argv[2] == case["arg"], sys.argv
with open(fimi + case["results_name"], "w", encoding="utf-8") as f:
    f.write(case["results_text"].replace("<fimi>", fimi))
sys.stdout.write(case["stdout"].replace("<fimi>", fimi))
sys.exit(case["exit_code"])
'''


def _reference_adapter():
    ref = os.environ.get("SGFIM_REFERENCE")
    path = os.path.join(ref, "code", "pipeline", "engine_adapter.py") if ref else ""
    if not ref or not os.path.exists(path):
        pytest.skip("SGFIM_REFERENCE does not name a reference checkout")
    sys.dont_write_bytecode = True
    spec = importlib.util.spec_from_file_location("reference_engine_adapter", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _replay_exe(tmp_path, name, case):
    case_path = tmp_path / (name + ".json")
    case_path.write_text(json.dumps(case))
    exe = tmp_path / name
    exe.write_text(REPLAY.format(python=sys.executable, case_path=str(case_path)))
    exe.chmod(exe.stat().st_mode | stat.S_IXUSR)
    return str(exe)


def test_reference_adapter_on_shim_output(tmp_path):
    ea = _reference_adapter()
    gold = json.load(open(os.path.join(HERE, "golden", "shim_golden.json")))
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_shim_golden import fimi_text
    data = tmp_path / "data"
    data.mkdir()
    fimi = str(data / gold["fimi_name"])
    with open(fimi, "w", encoding="utf-8") as f:
        f.write(fimi_text())
    cases = {c["kind"]: c for c in gold["cases"]}
    bins = tmp_path / "bin"
    bins.mkdir()
    ea.TENSORFIM_DIR = str(bins)
    _replay_exe(bins, "CoParaCG_bmma.exe", cases["tensorfim"])
    ea.ANYFIM_EXE = _replay_exe(bins, "AnytimeMining.exe", cases["anyfim"])

    rows1 = [[x + 1 for x in r] for r in datagen.regime_txns(4000, 8, 5, 4, 0.3, seed=12).tolist()]
    r = ea.run_tensorfim("bmma", fimi, float(cases["tensorfim"]["arg"]))
    assert r["ok"] and r["comp_times"] and r["tot_times"]
    assert r["mfis"] == oracle.tensorfim_mfis(rows1, 0.03)
    a = ea.run_anyfim(fimi, int(cases["anyfim"]["arg"]))
    assert a["ok"]
    want = oracle.anyfim_stages(rows1, 12)
    assert {k: dict(v) for k, v in a["stages"].items()} == want
    assert a["meta"]["MFIsNumPerStage"] == [len(want[k]) for k in sorted(want)]
