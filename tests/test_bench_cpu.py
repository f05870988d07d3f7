"""The bench's CPU legs and bookkeeping, without a GPU: the reference arm's JSON line, the bounded
CPU-baseline sample and the algorithmic bytes behind roofline.achieved."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                          "single_256", "--steps", "2", "--warmup", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("single 256x256")


def test_cpu_baseline_sample_is_bounded_and_described():
    import bench
    worlds, seeds, _ = bench.workload("single_256")
    rate, cores, sample = bench.cpu_leg(worlds, seeds, min_seconds=0.3)
    assert rate > 0 and cores >= 1
    gens = int(sample.split(" generation")[0])
    assert gens >= 1 and "%d threads" % cores in sample


def test_algorithmic_bytes():
    import bench
    from auto_gb300 import configs
    one = configs.single_4096()
    assert bench.alg_bytes_per_gen([one]) == 12.0 * 4096 * 4096
    multi = configs.multichannel()
    assert bench.alg_bytes_per_gen([multi]) == (8.0 * 3 + 4.0 * 9) * 1024 * 1024  # 20 B per channel-cell
    ws = configs.batched(8)
    assert bench.alg_bytes_per_gen(ws) == sum(12.0 * w.width * w.height for w in ws)


def test_reference_arm_under_torchrun_prints_once():
    """Under torchrun (two gloo ranks here) rank 0 alone times the reference arm and prints its line;
    the other rank exits 0 without work."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--config", "single_256", "--steps", "1", "--warmup", "0",
                          "--gpus", "2"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
