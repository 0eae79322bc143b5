"""Results.txt files of the CLI shims, and running the shims.

The pipeline scrapes the engines' result files and stdout with four regular
expressions (code/pipeline/engine_adapter.py:29-33); the shims
(csrc/cli_tensorfim.cpp, csrc/cli_anytime.cpp) write exactly that format,
so the patterns below are the interface and are kept character for
character.  ``read_results`` classifies each line once: a stage header opens
a stage, a record adds an itemset to the open stage (or to the single
TensorFIM list), and a "key: v1, v2, ..." header line of an AnyFIM file is
kept as a list of numbers.  ``run_shim`` runs a shim on a FIMI file and
returns the file it wrote, parsed, with the timings printed on stdout.
"""
from __future__ import annotations

import os
import re
import subprocess
from dataclasses import dataclass, field

# the record, stage-header and timing patterns of the engines' output (interface)
RECORD = re.compile(r"^\d+th:\s+\d+\s+\{\s*([^}]*)\}\s+support:\s+\S+\s+frequency:\s+(\d+)")
STAGE_HEADER = re.compile(r"^=+ (\d+)th stage MFIs Number: (\d+) =+")
COMPUTATION_TIME = re.compile(r"computation_time\(s\):\s*([\d.eE+-]+)")
TOTAL_TIME = re.compile(r"total_time\(s\):\s*([\d.eE+-]+)")

# AnyFIM header arrays and the type of their values
_ARRAYS = {"runtimePerStage(s)": float, "supportThrePerStage": float, "frequencyThrePerStage": float,
           "MFIsNumPerStage": int, "itemsNumPerStage": int, "dimensionPerStage": int,
           "preprocessing_time(s)": float}

SHIMS = {"tensorfim": "sgfim_tensorfim", "anyfim": "sgfim_anytime"}
LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")


@dataclass
class ResultsFile:
    sets: dict = field(default_factory=dict)      # TensorFIM: {frozenset(ids): frequency}
    stages: dict = field(default_factory=dict)    # AnyFIM: {k: [(frozenset(ids), frequency), ...]}
    arrays: dict = field(default_factory=dict)    # AnyFIM header arrays
    computation_s: float | None = None
    total_s: float | None = None

    def cumulative(self):
        """{k: every itemset reported in stages 1..k}."""
        out, seen = {}, set()
        for k in sorted(self.stages):
            seen |= {s for s, _ in self.stages[k]}
            out[k] = set(seen)
        return out


def _numbers(body, cast):
    return [cast(tok.rstrip(",")) for tok in body.split() if tok.strip(",")]


def read_results(path):
    """Parse a TensorFIM or AnyFIM Results.txt (the kind follows from its stage headers)."""
    res = ResultsFile()
    stage = None
    with open(path, encoding="utf-8", errors="replace") as f:
        for raw in f:
            line = raw.strip()
            head = STAGE_HEADER.match(line)
            if head:
                stage = res.stages.setdefault(int(head.group(1)), [])
                continue
            rec = RECORD.match(line)
            if rec:
                itemset = frozenset(int(x) for x in rec.group(1).split())
                if stage is None:
                    res.sets[itemset] = int(rec.group(2))
                else:
                    stage.append((itemset, int(rec.group(2))))
                continue
            key, sep, body = line.partition(":")
            if sep and key in _ARRAYS:
                res.arrays[key] = _numbers(body, _ARRAYS[key])
    return res


def timings(text):
    """(computation_s, total_s) of the last timing lines in a shim's stdout, None when absent."""
    c, t = COMPUTATION_TIME.findall(text), TOTAL_TIME.findall(text)
    return (float(c[-1]) if c else None), (float(t[-1]) if t else None)


def result_path(kind, fimi_path, arg):
    """Where a shim writes its file: next to the dataset, named as the engines name it."""
    if kind == "tensorfim":
        return f"{fimi_path}-{float(arg):.6f}=Results.txt"
    return f"{fimi_path}-{int(arg)}-stages=Results.txt"


def run_shim(kind, fimi_path, arg, timeout=3600, lib_dir=LIB_DIR):
    """Run a CLI shim (kind "tensorfim": arg = relative threshold; "anyfim": arg =
    number of stages) and return its parsed ResultsFile, or None when it wrote none."""
    out = result_path(kind, fimi_path, arg)
    if os.path.exists(out):
        os.remove(out)
    p = subprocess.run([os.path.join(lib_dir, SHIMS[kind]), fimi_path, str(arg)], capture_output=True,
                       timeout=timeout)
    if not os.path.exists(out):
        return None
    res = read_results(out)
    res.computation_s, res.total_s = timings(p.stdout.decode("utf-8", errors="replace"))
    return res
