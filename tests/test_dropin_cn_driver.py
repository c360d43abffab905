"""The drop-in, end to end: the reference's own CN driver (CN/cn.cpp with
CN/partition.cpp and shared/, from the staging copy oracle/Makefile keeps) is
built with the CN shim of INTEGRATION.md in place of gpu_partition.cu and
linked against libfastpart.so.  Here (no GPU) it must link and run its CPU
path unchanged, and with -g report the library's error instead of crashing;
the GPU comparison (-g 1 against the CPU refinement) runs with the GPU tests."""
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = ROOT / "oracle" / "_ref" / "src"
CFLAGS = ["-O2", "-std=c++11", "-fopenmp", "-ffp-contract=off", "-w"]


def shim_sources(tmp):
    blocks = re.findall(r"```(?:cpp|c\+\+)\n(.*?)```", (ROOT / "INTEGRATION.md").read_text(), re.S)
    common = [b for b in blocks if "fp_wrapper_refine(int metric" in b]
    cn = [b for b in blocks if "FP_METRIC_CN, row_ptr" in b]
    assert len(common) == 1 and len(cn) == 1
    (tmp / "fp_wrapper_common.h").write_text("#pragma once\n" + common[0])
    (tmp / "cn_fp_wrapper.cpp").write_text(cn[0])
    return tmp / "cn_fp_wrapper.cpp"


@pytest.fixture(scope="session")
def cn_driver(fp, tmp_path_factory):
    """Path of the reference CN driver linked against libfastpart.so."""
    if not (SRC / "CN" / "cn.cpp").exists() or shutil.which("g++") is None:
        pytest.skip("reference CN driver sources not staged (oracle/_ref/src)")
    tmp = tmp_path_factory.mktemp("cn_driver")
    shim = shim_sources(tmp)
    lib = fp.library_path()
    exe = tmp / "cn_gb300"
    cmd = ["g++", *CFLAGS, "-I", str(SRC / "CN"), "-I", str(SRC / "shared"), "-I", str(ROOT / "include"),
           "-I", str(tmp), str(SRC / "CN" / "cn.cpp"), str(SRC / "CN" / "partition.cpp"),
           str(SRC / "shared" / "metric.cpp"), str(SRC / "shared" / "utils.cpp"),
           str(SRC / "shared" / "hypergraph_rw.cpp"), str(shim), "-L", str(lib.parent), "-lfastpart",
           f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe


def run_driver(exe, hg_path, K, passes, gpu):
    res = subprocess.run([str(exe), "-f", str(hg_path), "-k", str(K), "-r", "1", "-i", str(passes), "-g", str(gpu)],
                         capture_output=True, text=True, timeout=600, cwd=hg_path.parent)
    return res


def after_lines(text):
    return re.findall(r"^After Refinement (TV|CN|TM|MGM|MGV|MGAV) : (-?\d+)$", text, re.M)


def test_reference_cn_driver_links_and_runs(fp, cn_driver, tmp_path):
    """The CPU path of the linked driver runs as the reference's does; -g without
    a usable device reports the library's status and the driver completes."""
    import torch
    hg = fp.generate(fp.GenSpec.zipf(3000, 2500, 2.1, 2, 120, beta=1.2, seed=71))
    path = tmp_path / "g.hg"
    fp.write_patohlike(hg, path)
    cpu = run_driver(cn_driver, path, 8, 3, 0)
    assert cpu.returncode == 0, cpu.stderr[-2000:]
    assert len(after_lines(cpu.stdout)) == 6
    if not torch.cuda.is_available():
        gpu = run_driver(cn_driver, path, 8, 3, 1)
        assert gpu.returncode == 0, gpu.stderr[-2000:]
        assert "fastpart:" in gpu.stderr
