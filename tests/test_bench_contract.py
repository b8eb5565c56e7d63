"""The reference arm of bench.py on the CPU: one JSON line with the
contract's keys, timed on the oracle's CG (the reference's CPU path is not
runnable), no host<->device bytes, and the GPU leg reported unavailable
when there is no GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(__import__("torch").cuda.is_available(), reason="CPU-only check")
def test_reference_arm_json_line():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "solve_hbm_gbs" and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("poisson7_128^3")
    assert "unavailable" in d["reference_gpu_kernels"]


def test_streamed_bytes_per_format():
    """The algorithmic bytes bench.py credits each column format with: 12 B
    per stored FP64 entry with 32-bit columns, 9 with one-byte codes (plus
    the 128-byte offset table), 10 with 16-bit deltas; the FP64 solver loops
    read the 32-bit columns whatever compact copy exists; every coded or
    delta variant of a fast or mixed kernel in the launch table carries the
    bytes of its own format."""
    sys.path.insert(0, ROOT)
    import bench
    n, S = 2_097_152, 14_614_528
    slices = (n + 31) // 32 + 1
    assert bench.iter_matrix_bytes("sell", n, 0, S) == 12 * S + 4 * slices
    assert bench.iter_matrix_bytes("sell8", n, 0, S) == 9 * S + 4 * slices + 128
    assert bench.iter_matrix_bytes("sell16", n, 0, S) == 10 * S + 4 * slices
    for fmt in ("sell8", "sell16"):
        assert bench.iter_matrix_bytes(fmt, n, 0, S, fp64_loop=True) == 12 * S + 4 * slices
    nnz = 14_581_760
    assert bench.iter_matrix_bytes("csr", n, nnz, nnz) == 12 * nnz + 4 * (n + 1)
    t = bench._launch_bytes(n, 6_242_304, nnz, S, 65_536)
    for name, (formula, val) in t.items():
        if "Msell" in formula and (name.startswith("k_f_") or name.startswith("k_mx_")):
            # the format is the kernel's last template argument (the first for
            # k_mx_residual)
            if name.startswith("k_mx_residual"):
                fmt1 = name.replace("<1, ", "<@, ")
            elif name.startswith("k_f_mr_spmv"):
                fmt1 = name[:-2] + "@>" if name.endswith(", 1>") else name
            else:
                fmt1 = name.replace("<1>", "<@>")
            if "@" not in fmt1:
                continue
            for fmt, tag in (("2", "Msell8"), ("3", "Msell16")):
                other = fmt1.replace("@", fmt)
                assert other in t, other
                assert tag in t[other][0] and t[other][1] < val
