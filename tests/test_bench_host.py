"""Host-side pieces of bench.py that need no GPU: the committed DRAM-traffic
summary per kernel and storage, the argument surface, and the ensemble's
weight files."""

import json
import os

import bench


def test_traffic_summary_has_both_hot_kernels():
    rows = json.load(open(os.path.join(bench.ROOT, "profiles", "k_step_traffic.json")))
    keys = {(r.get("kernel"), r["storage"]) for r in rows}
    for storage in ("f32", "f32dev", "f16dev", "bf16dev"):
        assert ("k_step_pipe", storage) in keys
    for storage in ("f32", "f32dev"):
        assert ("k_step2", storage) in keys
    for r in rows:
        # one launch moves about one read and one write of the lattice
        per_cell = r["dram_bytes_per_launch"] / r["cells"]
        full = 72 if r["storage"] in ("f32", "f32dev") else 36
        assert 0.85 * full < per_cell < 1.05 * full
        assert "ncu" in r["source"] and "--clock-control none" in r["source"]


def test_profiled_traffic_scales_by_cells_and_picks_the_kernel():
    one, row1 = bench.profiled_traffic("f32", "cavity", 8192 * 8192, "k_step_pipe")
    two, row2 = bench.profiled_traffic("f32", "cavity", 8192 * 8192, "k_step2")
    assert row1["kernel"] == "k_step_pipe" and row2["kernel"] == "k_step2"
    assert abs(one / (8192 * 8192) - row1["dram_bytes_per_launch"] / row1["cells"]) < 1e-9
    assert two is not None and abs(two - one) < 0.1 * one
    assert bench.profiled_traffic("f64", "cavity", 100) == (None, None)


def test_arguments_and_extras():
    a = bench.parse([])
    assert (a.nx, a.ny, a.storage, a.boundary, a.gpus, a.copy_streams) == (8192, 8192, "f32", "cavity", 1, 1)
    assert set(a.extras.split(",")) == {"operator_path", "fp16_store", "warm_start"}
    assert bench.parse(["--no-extras"]).no_extras


def test_ensemble_weight_files_share_the_split():
    import numpy as np
    files = bench.weight_files()
    assert files[0] == bench.WEIGHTS and len(files) == 5
    held = [json.loads(str(np.load(f, allow_pickle=True)["meta"]))["held_out_re"] for f in files]
    assert all(h == held[0] for h in held)
