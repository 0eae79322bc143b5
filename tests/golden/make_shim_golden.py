"""Record the CLI shims' output on a fixed FIMI file (run on a GPU machine).

    python tests/golden/make_shim_golden.py        # writes tests/golden/shim_golden.json

The dataset is the seeded 4,000-transaction, 8-sensor x 5-bin workload of
tests/test_gpu_mining.py (1-based ids).  For `sgfim_tensorfim <fimi> 0.03`
and `sgfim_anytime <fimi> 12` the file stores the argv, the exit code, the
stdout and the Results.txt each one wrote, named as the engines name it.
tests/test_gpu_shims.py checks that a live run of the shims reproduces these
bytes (timing values and the dataset's path aside); tests/test_reference_adapter.py
feeds them to the reference's own engine_adapter.run_tensorfim / run_anyfim.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300"))

from sgfim import datagen, results  # noqa: E402

CASES = [("tensorfim", "0.03"), ("anyfim", "12")]


def fimi_text():
    rows = datagen.regime_txns(4000, 8, 5, 4, 0.3, seed=12)
    return "".join(" ".join(str(x + 1) for x in sorted(r.tolist())) + "\n" for r in rows)


def run_case(kind, arg, fimi):
    out = results.result_path(kind, fimi, arg)
    if os.path.exists(out):
        os.remove(out)
    p = subprocess.run([os.path.join(results.LIB_DIR, results.SHIMS[kind]), fimi, arg], capture_output=True)
    with open(out, encoding="utf-8") as f:
        text = f.read()
    # the dataset's path appears in the output; it is stored as "<fimi>"
    return {"kind": kind, "arg": arg, "exit_code": p.returncode,
            "stdout": p.stdout.decode("utf-8").replace(fimi, "<fimi>"),
            "results_name": os.path.basename(out)[len("d.txt"):], "results_text": text.replace(fimi, "<fimi>")}


def main():
    text = fimi_text()
    with tempfile.TemporaryDirectory() as tmp:
        fimi = os.path.join(tmp, "d.txt")
        with open(fimi, "w", encoding="utf-8") as f:
            f.write(text)
        cases = [run_case(k, a, fimi) for k, a in CASES]
    gold = {"fimi_sha256": hashlib.sha256(text.encode()).hexdigest(), "fimi_name": "d.txt", "cases": cases}
    with open(os.path.join(HERE, "shim_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)


if __name__ == "__main__":
    main()
