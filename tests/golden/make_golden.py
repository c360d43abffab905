"""Generates tests/golden/*.npz from the reference itself.

Each fixture holds one small seeded instance (both CSRs and the sources) and, for
every (metric, K) case, the reference's own results -- produced by running the
reference's partition() (compiled from its sources by oracle/Makefile into
oracle/_ref/) through oracle/ref_harness.cpp:

  part_vec_init / part_vec     part vector after the stream / after refinement
  ep_len / lists               per-net part counts and the concatenated ordered
                               part lists after refinement
  metrics_init / metrics_final the six printed metric values (TV CN TM MGM MGV MGAV)

Usage (needs oracle/_ref, i.e. the reference sources):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import fastpartitioner_gb300 as fp  # noqa: E402
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
METRICS = ["TV", "CN", "TM", "MSM", "MSV", "MSRV"]

# name -> (generator spec, K values, passes)
CASES = {
    "colnet_600_s0": (fp.GenSpec.column_net(600, 600, 2, 16, seed=0), [2, 4, 8], 5),
    "colnet_600_s7": (fp.GenSpec.column_net(600, 600, 2, 8, seed=7), [3, 8], 4),
    "colnet_256_s3": (fp.GenSpec.column_net(256, 256, 2, 6, seed=3), [2, 16], 6),
    "zipf_800_s1": (fp.GenSpec.zipf(800, 800, 2.1, 2, 200, beta=1.5, seed=1), [4, 16], 5),
    "zipf_500_s2": (fp.GenSpec.zipf(500, 500, 1.9, 2, 100, beta=0.0, seed=2), [8, 32], 5),
    # sparse, high-K cases: the ones where MSM finds moves
    "zipf_400_s0": (fp.GenSpec.zipf(400, 400, 2.5, 2, 50, seed=0), [32, 64], 4),
    "colnet_300_s1": (fp.GenSpec.column_net(300, 300, 2, 3, seed=1), [8, 16, 64], 4),
}


def make(name: str, spec, Ks, passes) -> Path:
    hg = fp.generate(spec)
    arrays = {"vptr": hg.vptr, "vnets": hg.vnets, "nptr": hg.nptr, "npins": hg.npins, "src": hg.src,
              "dims": np.array([hg.nov, hg.noe, passes], np.int64), "Ks": np.array(Ks, np.int64)}
    for m in METRICS:
        for K in Ks:
            r = oracle.run_reference(hg, K, m, passes)
            key = f"{m}_{K}"
            arrays[f"{key}_part_vec_init"] = r["part_vec_init"].astype(np.int32)
            arrays[f"{key}_part_vec"] = r["part_vec"].astype(np.int32)
            arrays[f"{key}_ep_len"] = r["ep_len"].astype(np.int32)
            arrays[f"{key}_lists"] = r["lists"].astype(np.int32)
            arrays[f"{key}_metrics_init"] = np.array([r["metrics_init"][k] for k in oracle.OUTPUT_ORDER], np.int64)
            arrays[f"{key}_metrics_final"] = np.array([r["metrics_final"][k] for k in oracle.OUTPUT_ORDER], np.int64)
    path = OUT / f"{name}.npz"
    np.savez_compressed(path, **arrays)
    return path


def main():
    if not oracle.reference_available():
        oracle.build()
    if not oracle.reference_available():
        raise SystemExit("oracle/_ref is not built: the reference sources are needed")
    for name, (spec, Ks, passes) in CASES.items():
        p = make(name, spec, Ks, passes)
        print(f"{p.name}: {p.stat().st_size} bytes")


if __name__ == "__main__":
    main()
