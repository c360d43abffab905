"""The reference-side bindings INTEGRATION.md gives a maintainer compile
against include/fastpart.h: the shared wrapper header, the per-metric
partition_gpu_wrapper shims, MSM's partition_gpu, and the BFS-ordering and
CN-thinning fragments (placed in a function that declares the variables the
reference's drivers hold there, with the drivers' types).  The "driver fix"
blocks are compiled in place, inside the drivers, by test_dropin_drivers.py."""
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")

# the drivers' variables the fragments use (TV/tv.cpp, CN/cn.cpp)
FRAGMENT_PRELUDE = """#include <cstdlib>
#include "fastpart.h"
void fragment(int nov, int noe, long long pins, unsigned int* row_ptr, unsigned int* col_ind,
              unsigned int* row_ptr_inv, unsigned int* col_ind_inv, int* src_nodes, int* ordering,
              fp_hypergraph full, int THINMEAN, int THINMIN, fp_ctx* ctx, int K, int REFI_ITER, int* part_vec) {
"""


def cpp_blocks():
    return re.findall(r"```(?:cpp|c\+\+)\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S)


def compile_ok(path, inc):
    res = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-Wall", "-Werror", "-Wno-unused-variable",
                          "-Wno-unused-but-set-variable", "-I", str(ROOT / "include"), "-I", str(inc), str(path)],
                         capture_output=True, text=True)
    return res.returncode == 0, res.stderr[-3000:]


def test_every_binding_block_compiles(tmp_path):
    blocks = cpp_blocks()
    assert len(blocks) >= 8
    common = [b for b in blocks if "fp_wrapper_refine(int metric" in b]
    assert len(common) == 1
    (tmp_path / "fp_wrapper_common.h").write_text("#pragma once\n" + common[0])
    n_units = n_fragments = 0
    for i, b in enumerate(blocks):
        if b is common[0] or b.startswith("// driver fix "):
            continue
        src = tmp_path / f"block{i}.cpp"
        if "#include" in b:                       # a whole translation unit
            src.write_text(b)
            n_units += 1
        else:                                      # a fragment of a driver's function
            src.write_text(FRAGMENT_PRELUDE + b + "\n}\n")
            n_fragments += 1
        ok, err = compile_ok(src, tmp_path)
        assert ok, f"INTEGRATION.md block {i} does not compile:\n{b[:400]}\n{err}"
    assert n_units >= 5 and n_fragments >= 2
