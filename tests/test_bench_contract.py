"""Host-side pieces of bench.py that need no GPU: the workload table, the
roofline traffic read from the committed ncu summary, and the algorithmic-byte
model the roofline divides by."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
bench = pytest.importorskip("bench")


def test_workloads_are_named_by_shape_and_complete():
    need = {"nov", "noe", "alpha", "lo", "hi", "beta", "weight_rule", "K", "eps", "passes", "seed"}
    assert "zipf4m" in bench.WORKLOADS
    for name, w in bench.WORKLOADS.items():
        assert need <= set(w), name
        assert w["K"] >= 2 and w["passes"] >= 1 and w["eps"] > 1.0, name
    z = bench.WORKLOADS["zipf4m"]
    assert (z["nov"], z["noe"], z["K"], z["passes"]) == (4_194_304, 4_194_304, 256, 10)
    s = bench.WORKLOADS["zipf16m_k1024"]
    assert (s["nov"], s["noe"], s["K"], s["hi"], s["alpha"]) == (16_777_216, 8_388_608, 1024, 100_000, 1.9)
    assert bench.metrics_for(s, "") == ["TM", "MSRV"]
    assert bench.metrics_for(z, "") == bench.METRICS and bench.metrics_for(z, "TV,CN") == ["TV", "CN"]


def test_traffic_comes_from_the_committed_summary():
    """The dominant kernel's DRAM traffic per full-size launch comes from the
    ncu summary under profiles/ (one line per metric of the kernel); it is not
    claimed for reduced-scale runs or for kernels and metrics the summaries do
    not cover."""
    t = bench.measured_traffic("spec_ldg_kernel", "zipf4m", 1, ["TV", "MSV", "MSRV"])
    assert isinstance(t, int) and t > 0
    text = (ROOT / "profiles" / "engines_dram_l2_zipf4m.md").read_text()
    per = [int(line.split()[-1]) for line in text.splitlines() if line.strip().startswith("traffic: spec_ldg_kernel")]
    assert len(per) == 3 and t == int(sum(per) / 3)
    assert bench.measured_traffic("spec_ldg_kernel", "zipf4m", 2, ["TV"]) is None
    assert bench.measured_traffic("spec_cn_kernel", "zipf4m", 1, ["CN"]) is None
    assert bench.measured_traffic("spec_ldg_kernel", "uniform16k", 1, ["TV"]) is None


def test_every_metric_maps_to_a_kernel():
    assert set(bench.KERNEL_OF) == set(bench.METRICS)
    assert set(bench.KERNEL_OF.values()) == {"spec_ldg_kernel", "spec_cn_kernel", "spec_msg_kernel"}


@pytest.fixture(scope="module")
def small_hg():
    import fastpartitioner_gb300 as fp
    return fp.generate(fp.GenSpec.zipf(2000, 2000, 2.1, 2, 200, beta=1.5, weight_rule=1, seed=3))


def test_algorithmic_bytes_model(small_hg):
    """Positive, grows with the moved vertices, and orders the metrics by what
    they read: CN reads only the two-part nets' pins, the volume and message
    metrics read more than TV."""
    hg = small_hg
    K = 16
    rng = np.random.default_rng(0)
    ln = rng.integers(1, 4, size=hg.noe).astype(np.int32)
    none = np.zeros(hg.nov, bool)
    some = rng.random(hg.nov) < 0.3
    tv0 = bench.algorithmic_bytes("TV", hg, ln, none, K)
    tv1 = bench.algorithmic_bytes("TV", hg, ln, some, K)
    assert 0 < tv0 < tv1
    assert bench.algorithmic_bytes("MSV", hg, ln, none, K) > tv0
    assert bench.algorithmic_bytes("TM", hg, ln, none, K) > bench.algorithmic_bytes("MSV", hg, ln, none, K)
    cn = bench.algorithmic_bytes("CN", hg, ln, none, K)
    sizes = np.diff(hg.nptr).astype(np.int64)
    assert cn == 4 * (hg.noe + 1) + 8 * hg.noe + int(np.sum(8 * sizes[ln == 2]))


def _reference_line(monkeypatch, capsys, available):
    import json
    import oracle
    if available and not oracle.reference_available():
        pytest.skip("reference harness not built (reference sources unavailable)")
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    if not available:
        monkeypatch.setattr(oracle, "reference_available", lambda *a: False)
    # one host thread: the reference's sequential partition(); its OpenMP path
    # is racy on instances this small (runs end with SIGSEGV)
    monkeypatch.setattr(bench.os, "cpu_count", lambda: 1)
    args = bench.argparse.Namespace(config="zipf4m", metrics="TV,CN", scale=256, passes=0, cpu_passes=1, warmup=1,
                                    steps=2)
    bench.run_reference_arm(args)
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(lines) == 1
    return json.loads(lines[0])


@pytest.mark.parametrize("available", [True, False], ids=["reference", "port"])
def test_reference_arm_line(monkeypatch, capsys, available):
    """bench.py --impl reference on a tiny sample: one JSON line with the
    contract's keys, the same metric and unit as the GPU arm, an e2e with no
    host-device bytes and a cpu_baseline describing the run."""
    line = _reference_line(monkeypatch, capsys, available)
    need = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}
    assert need <= set(line)
    assert line["impl"] == "reference" and line["unit"] == "pins/s" and line["higher_is_better"] is True
    assert line["metric"] == bench.METRIC and line["value"] > 0 and line["steps"] == 2
    cb = line["cpu_baseline"]
    assert cb["kind"] == ("reference" if available else "port") and cb["value"] == line["value"]
    assert cb["cores"] >= 1 and "vertices" in cb["sample"] and "schedule of each of TV,CN" in cb["sample"]
    # the same workload string as the GPU arm, and no product library in the process's work
    w = bench.WORKLOADS["zipf4m"]
    assert line["config"]["workload"].startswith("zipf4m: 16384 vertices, 16384 nets")
    assert set(line["config"]["per_metric_pins_per_s"]) == {"TV", "CN"}
    assert line["e2e"] == {"value": line["value"], "unit": "pins/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_run_ended_by_a_signal_is_retried(monkeypatch, capsys):
    """A reference run that a signal ends is run again and counted; a run that
    fails with an exit status is not retried."""
    import oracle
    if not oracle.reference_available():
        pytest.skip("reference harness not built (reference sources unavailable)")
    real = oracle.run_reference_file
    calls = {"n": 0}

    def flaky(*a, **k):
        calls["n"] += 1
        if calls["n"] == 2:
            raise oracle.ReferenceRunError(-11, "reference run failed (-11)")
        return real(*a, **k)

    monkeypatch.setattr(oracle, "run_reference_file", flaky)
    line = _reference_line(monkeypatch, capsys, True)
    assert line["cpu_baseline"]["crashed_runs_retried"] == 1 and line["value"] > 0

    def failing(*a, **k):
        raise oracle.ReferenceRunError(3, "reference run failed (3)")

    monkeypatch.setattr(oracle, "run_reference_file", failing)
    with pytest.raises(oracle.ReferenceRunError):
        bench.run_reference_retrying(oracle, None, 8, "TV", 1, 1)


def test_reference_arm_loads_no_product_library(tmp_path):
    """The reference arm draws its instance with the oracle's generator: the
    process never imports the product package nor maps libfastpart.so."""
    import subprocess
    code = ("import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--scale', '256', '--metrics', 'TV', "
            "'--steps', '1', '--warmup', '0']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'fastpartitioner_gb300' not in sys.modules, 'product package imported'; "
            "assert 'libfastpart' not in maps, 'product library mapped'")
    res = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    import json
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
