"""The engine's FIMI parser (csrc/io.cpp parse_fimi_file, the restatement of
readTransSetFile, kernel_bitmap.cu:205-233) on the CPU: a small harness built
against io.cpp prints the parsed transactions, which must equal the oracle's
byte-by-byte restatement on edge cases (empty lines, CRLF, tabs, letters,
negative ids, a last line without a newline, blank-only tails) and on a file
of more than 1 MB, which the parser cuts into line-aligned slices parsed by
several threads.  An id above 32 bits is an error."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "20261008-self-growing-evidence-agent_gb300", "csrc")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

HARNESS = r"""
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
namespace sg {
int parse_fimi_file(const char *path, std::vector<uint64_t> &row_ptr, std::vector<uint32_t> &items, std::string &err);
}
int main(int argc, char **argv) {
    std::vector<uint64_t> rp;
    std::vector<uint32_t> it;
    std::string err;
    const int rc = sg::parse_fimi_file(argv[1], rp, it, err);
    std::printf("%d\n", rc);
    if (rc) return 0;
    for (size_t r = 0; r + 1 < rp.size(); ++r) {
        for (uint64_t k = rp[r]; k < rp[r + 1]; ++k) std::printf(k == rp[r] ? "%u" : " %u", it[k]);
        std::printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def parser(tmp_path_factory):
    if shutil.which("g++") is None or not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    d = tmp_path_factory.mktemp("fimi")
    (d / "main.cpp").write_text(HARNESS)
    exe = d / "parse"
    lib = os.path.join(CUDA, "lib64")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", f"-I{CUDA}/include", f"-I{CSRC}", str(d / "main.cpp"),
                    os.path.join(CSRC, "io.cpp"), f"-L{lib}", f"-Wl,-rpath,{lib}", "-lcudart", "-o", str(exe)],
                   check=True, timeout=180)

    def run(path):
        out = subprocess.run([str(exe), str(path)], capture_output=True, text=True, timeout=120, check=True).stdout
        lines = out.split("\n")
        rc = int(lines[0])
        rows = [[int(x) for x in ln.split()] for ln in lines[1:-1]]
        return rc, rows
    return run


CASES = {
    "plain": b"1 2 3\n4 5\n",
    "empty_lines": b"\n\n1\n\n2 3\n\n",
    "crlf_tabs": b"1\t2\r\n3  4 \r\n\t5\r\n",
    "negatives": b"1 -2 3\n-4\n5-6 7\n--8 9\n",
    "letters": b"a1b2 c\nxyz\n3,4;5\n",
    "no_final_newline": b"1 2\n3 4",
    "final_blank_tail": b"1 2\n   \t",
    "final_negative_only": b"1\n-5",
    "leading_zeros": b"007 0 00\n",
    "empty_file": b"",
    "only_newlines": b"\n\n\n",
    "max_id": b"4294967294 1\n",
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_parser_matches_byte_rules(parser, tmp_path, name):
    p = tmp_path / f"{name}.txt"
    p.write_bytes(CASES[name])
    rc, rows = parser(p)
    assert rc == 0
    assert rows == oracle.parse_fimi(str(p))


def test_parser_large_file_parallel_slices(parser, tmp_path):
    rng = np.random.default_rng(3)
    seps = [b" ", b"  ", b"\t", b" - 7 ", b",", b"\r"]
    lines = []
    for i in range(150_000):
        k = int(rng.integers(0, 9))
        ids = rng.integers(0, 5000, k)
        parts = [str(int(x)).encode() for x in ids]
        lines.append(seps[i % len(seps)].join(parts))
    data = b"\n".join(lines)   # no final newline: the last line counts when it holds an item
    assert len(data) > (1 << 20)
    p = tmp_path / "big.txt"
    p.write_bytes(data)
    rc, rows = parser(p)
    assert rc == 0
    assert rows == oracle.parse_fimi(str(p))


def test_parser_rejects_ids_above_32_bits(parser, tmp_path):
    p = tmp_path / "big_id.txt"
    p.write_bytes(b"1 4294967295\n")
    rc, _ = parser(p)
    assert rc != 0
