"""The reference arm of bench.py runs on the host cores alone, so its JSON line is checked here.

`bench.py --impl reference` times the CPU restatement of the reference engine on a fixed sample
of the ensemble.  Its line must carry the benchmark contract's keys with the GPU arm's metric,
unit, direction and workload `config` (both arms build it with `ensemble_config`), an `e2e`
object without host-device copies, and a `cpu_baseline` that describes this very run.  Under a
two-rank launch, rank 0 alone prints.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


def _run(launcher=()):
    cmd = [sys.executable, *launcher, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "0"]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_line_follows_the_contract():
    out = _run()
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["metric"] == "particle-steps/s" and line["unit"] == "particle-steps/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    # the workload config is the GPU arm's: ensemble_config over the configured ensemble
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tissue-forge_gb300"))
    import bench
    from tfg import configs
    ns, _ = configs.ensemble_sizes(256)
    assert line["config"] == bench.ensemble_config(256, 1, int(np.sum(ns)))


def test_reference_arm_under_two_ranks_prints_one_line():
    """Launched like the multi-GPU runs (torchrun, gloo here), rank 0 alone times the sample
    and prints; the other rank exits 0 without output."""
    launcher = ("-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                "--master-port", str(_free_port()))
    out = _run(launcher)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["config"]["sims_all_ranks"] == 512
