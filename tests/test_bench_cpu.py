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


# The fields of the reference's results/*.jsonl record, in order, with their types: `Sample` in
# crates/auto-cli/src/bench.rs:39-55 (String x 4, u32 x 2, u64 x 2, f64 x 3, u32 x 2, f64).
SAMPLE_FIELDS = [("id", str), ("tag", str), ("adapter", str), ("checks", str), ("width", int), ("height", int),
                 ("cells", int), ("memory_bytes", int), ("steps_per_second", float),
                 ("generations_per_second", float), ("cells_per_second", float), ("batch_steps", int),
                 ("batches", int), ("spread", float)]


class _FakeSim:
    """Stands in for Sim in the harness: each step of `batch` generations takes batch * 0.5 ms."""
    cells_per_step = 65536
    memory_bytes = 1234567

    def __init__(self):
        self.stepped = 0

    def step(self, n):
        import time
        self.stepped += n
        time.sleep(n * 0.0005)

    def wait(self):
        pass


def test_jsonl_sample_has_exactly_the_reference_fields(tmp_path):
    """bench.append_reference_sample writes one record with the reference's Sample fields, in its
    order and types, and the record's rates agree with each other."""
    import bench
    from auto_gb300 import configs
    path = tmp_path / "gpu.jsonl"
    sim = _FakeSim()
    w = configs.single_256()
    bench.append_reference_sample(str(path), sim, [w], {}, "fp32", seconds=0.3)
    lines = path.read_text().splitlines()
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert list(rec) == [f for f, _ in SAMPLE_FIELDS]
    for f, t in SAMPLE_FIELDS:
        assert isinstance(rec[f], t) and not isinstance(rec[f], bool), (f, rec[f])
    assert rec["width"] == w.width and rec["height"] == w.height and rec["cells"] == sim.cells_per_step
    assert rec["memory_bytes"] == sim.memory_bytes and rec["checks"] == "Safe"
    assert rec["generations_per_second"] == rec["steps_per_second"]
    assert abs(rec["cells_per_second"] - rec["steps_per_second"] * rec["cells"]) < 1e-6 * rec["cells_per_second"]


def test_reference_rate_grows_the_batch_to_20ms_and_takes_the_median():
    """crates/auto-cli/src/bench.rs:112-166: the batch grows until one submit takes >= 20 ms, then
    batches run for the measuring time and the median rate is reported."""
    import bench
    sim = _FakeSim()
    median, spread, batch, nb = bench.reference_rate(sim, seconds=0.3, warmup=4)
    assert batch * 0.0005 >= 0.02 * 0.8  # the submit that ended the search took about 20 ms or more
    assert nb >= 3 and 0.0 <= spread < 1.0
    assert 0.5 / 0.0005 * 0.5 < median <= 1.0 / 0.0005  # about 2000 generations/s, sleep overhead aside
