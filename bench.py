"""Lenia cell-updates/s on one GB300 (and N independent replicas under torchrun).

One bench step = one ``lenia_step(ctx, G)`` call: G generations (default 64, one CUDA-graph replay)
of every world in the workload.  The default workload is the metric's own: 384 uneven worlds
(sides 128..1024, per-world R, mu, sigma, dt) batched in one context; ``--config single_4096`` runs
the single 4096x4096 world with a three-shell R=52 kernel, ``--config multichannel`` the 3-channel
1024x1024 world with 9 kernels.

Printed JSON (one line, rank 0):
  value   cell-updates/s with the state resident in HBM, from CUDA events on the engine stream
          around the K timed bench steps, max over ranks
  e2e     the same metric through the public C ABI with host buffers: every bench step writes
          every world's state from a pinned host buffer (lenia_write_states_async), runs G
          generations and reads every state back into another (lenia_read_states_async); the
          copies overlap the neighbouring steps' generations.  blocking_value: the same with the
          blocking calls (lenia_write_states / lenia_read_states)
  roofline  12 algorithmic bytes per cell-update (state read and written, one complex f32
          half-spectrum value) over the event-timed generation time, against the measured HBM
          copy bandwidth; traffic = DRAM bytes per generation from an ncu capture of one
          graph replay with warm caches (``--profile-window``, summarised by ``--traffic-from``)
  cpu_baseline  the CPU restatement of the reference step on the host cores, bounded sample
  clocks  SM clock and throttle reasons sampled with nvidia-smi during the timed region
  gpu_launches  kernel launches in the timed region (two per size class per generation)

``--impl reference`` times the reference's step as restated on the CPU (the reference itself is
Rust + WGSL on Vulkan and cannot run here) on all host cores, on the same workload.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Lenia cell-updates/s on 1 GB300, batched TC vs plain FP32, at ≤1e-4 vs FP64"
UNIT = "cell-updates/s"
ALG_BYTES_PER_UPDATE = 12.0  # state read + write (8 B) + one f32 complex half-spectrum of the kernel (4 B)


def alg_bytes_per_gen(worlds):
    """Algorithmic bytes of one generation: (8 C + 4 K) H W per world -- every channel's state read and
    written once, plus one f32 complex half-spectrum (4 B per cell) per kernel.  12 B per cell-update
    for one channel and one kernel; 20 B per channel-cell for 3 channels and 9 kernels."""
    return sum((8.0 * w.channels + 4.0 * len(w.kernels)) * w.width * w.height for w in worlds)
PUBLISHED_REF = {"lenia_4096x4096_R13": 3.174e8, "hardware": "AMD RX 7900 XT (wgpu/Vulkan)",
                 "source": "results/gpu.jsonl:81"}


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="batched", choices=["batched", "single_4096", "single_256", "multichannel"])
    p.add_argument("--path", default="fp32", choices=["fp32", "tf32", "bf16x3", "radix2"])
    p.add_argument("--gens", type=int, default=64, help="generations per bench step")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--tc-rows", action="store_true",
                   help="tensor-core paths: run the row pass on the tensor cores too where it applies (after "
                        "autotuning, which otherwise keeps the faster row pass per class)")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default launch variants instead of timing both per size class")
    p.add_argument("--jsonl", default=None, help="also append a sample in the reference's results/*.jsonl format")
    p.add_argument("--no-paths", action="store_true", help="skip timing the other step paths side by side")
    p.add_argument("--grids", action="store_true",
                   help="the reference's own published programs and grids, measured its way: one line per grid")
    p.add_argument("--only-side", type=int, default=0,
                   help="keep only the workload's worlds of this side (a size class alone, e.g. for a profile)")
    p.add_argument("--max-worlds", type=int, default=0, help="keep at most this many of the workload's worlds")
    p.add_argument("--variants", default=None, metavar="COL,ROW",
                   help="with --profile-window: pin every class's column and row launch variants (lenia_set_variants) "
                        "after any autotuning, e.g. 1,0")
    p.add_argument("--profile-window", action="store_true",
                   help="set up, autotune and warm up the workload, then run exactly one bench step (one graph "
                        "replay) between cudaProfilerStart and cudaProfilerStop and exit: for ncu "
                        "--profile-from-start off")
    p.add_argument("--traffic-from", default=None, metavar="CSV",
                   help="summarise an ncu --csv capture of --profile-window (dram__bytes_read.sum, "
                        "dram__bytes_write.sum, gpu__time_duration.sum) into profiles/traffic.json and exit")
    p.add_argument("--traffic-graph", action="store_true",
                   help="with --traffic-from: the capture profiled the whole graph replay as one workload (ncu "
                        "--graph-profiling graph), so concurrent branches and lanes ran as in the timed run")
    return p.parse_args(argv)


# ----------------------------------------------------------------------------- distributed plumbing

def pin_gpu():
    """Under torchrun, show each rank only its own GPU (CUDA_VISIBLE_DEVICES), before any CUDA use.

    The engine library carries its own CUDA runtime, so a torch.cuda.set_device call would not
    choose its device; with one visible GPU per process, every runtime in the process uses the
    rank's GPU as device 0.  Returns the GPU's index among all GPUs (for nvidia-smi)."""
    if int(os.environ.get("WORLD_SIZE", "1")) <= 1 or "LOCAL_RANK" not in os.environ:
        return 0
    local = int(os.environ["LOCAL_RANK"])
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    ids = [x.strip() for x in vis.split(",") if x.strip()] if vis else []
    phys = ids[local] if local < len(ids) else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = phys
    return int(phys) if phys.isdigit() else local


class Dist:
    """torchrun plumbing: barrier and max over ranks (NCCL on GPUs, gloo without)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.torch = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            self.torch = torch
            if torch.cuda.is_available():
                # one visible GPU per rank after pin_gpu(); the rank's own index otherwise
                torch.cuda.set_device(0 if torch.cuda.device_count() == 1 else self.local)
                self.device = "cuda"
            dist.init_process_group("nccl" if self.device == "cuda" else "gloo")

    def barrier(self):
        if self.world > 1:
            self.torch.distributed.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([v], dtype=self.torch.float64, device=self.device)
        self.torch.distributed.all_reduce(t, op=self.torch.distributed.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.world == 1:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=self.device)
        self.torch.distributed.all_reduce(t, op=self.torch.distributed.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.torch.distributed.destroy_process_group()


def device_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except Exception:
        pass


# ----------------------------------------------------------------------------- clocks

REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]


class Clocks:
    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(REASONS, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- workloads

def workload(name, only_side=0, max_worlds=0):
    """(worlds, seeds, config) of a named workload, optionally cut to one size class and / or its first
    max_worlds worlds (the config then says so)."""
    worlds, seeds, cfg = _workload(name)
    if only_side or max_worlds:
        keep = [i for i, w in enumerate(worlds) if not only_side or w.width == only_side]
        keep = keep[:max_worlds] if max_worlds else keep
        worlds, seeds = [worlds[i] for i in keep], [seeds[i] for i in keep]
        cfg = dict(cfg, workload=cfg["workload"] + " -- subset: %d world(s)%s" % (
            len(worlds), " of side %d" % only_side if only_side else ""))
    return worlds, seeds, cfg


def _workload(name):
    import auto_gb300 as ag
    from auto_gb300 import configs
    if name == "single_4096":
        w = configs.single_4096()
        return [w], [configs.SEED_4096], {"workload": "single 4096x4096 world, R=52, beta=[1,.5,.25], mu=.26, "
                                                       "sigma=.036, dt=.05, 16 U[0,1] 256^2 patches (seed 1)"}
    if name == "single_256":
        return [configs.single_256()], [configs.SEED_256], {"workload": "single 256x256 world, R=13 (seed 0)"}
    if name == "multichannel":
        return [configs.multichannel()], [configs.SEED_MULTI], {"workload": "3 channels x 1024^2, 9 kernels"}
    ws = configs.batched(384)
    return ws, list(range(len(ws))), {"workload": "384 uneven worlds, sides 128..1024, per-world R/mu/sigma/dt"}


def shard(worlds, rank, nranks):
    """Indices of the worlds rank `rank` runs: largest first, each to the least-loaded rank, so
    every rank gets a near-equal share of the cells (deterministic on every rank)."""
    load = [0] * nranks
    mine = []
    order = sorted(range(len(worlds)), key=lambda i: (-worlds[i].cells_per_step, i))
    for i in order:
        r = min(range(nranks), key=lambda k: (load[k], k))
        load[r] += worlds[i].cells_per_step
        if r == rank:
            mine.append(i)
    return sorted(mine)


def seed_all(sim, worlds, seeds):
    for i, (w, s) in enumerate(zip(worlds, seeds)):
        sim.seed_patches(i, s, w.seed.patches)


# ----------------------------------------------------------------------------- CPU leg

def cpu_leg(worlds, seeds, min_seconds=10.0):
    """The reference's f32 step restated in C (oracle/lenia_oracle.c) on all host cores: a bounded
    sample of the workload, at least `min_seconds` of timed CPU work, cycling through the workload's
    one-channel power-of-two worlds one generation at a time.  With several worlds every core steps
    whole worlds of its own (one thread each); one world runs its rows and columns over all cores.
    Returns (cell-updates/s, cores, sample description)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle.oracle import RefF32
    cores = os.cpu_count() or 1
    ref = RefF32(threads=cores)
    todo = [(w, s) for w, s in zip(worlds, seeds)
            if w.channels == 1 and (w.width & (w.width - 1)) == 0 and (w.height & (w.height - 1)) == 0]
    if not todo:
        return None, cores, "no world the restated reference step supports"
    per_world = len(todo) > 1
    batch = cores if per_world else 1
    prepared = {}
    cells = 0
    t_total = 0.0
    steps_done = 0
    i = 0
    pool = ThreadPoolExecutor(max_workers=cores) if per_world else None

    def step_one(j):
        w = todo[j][0]
        st, spectra = prepared[j]
        prepared[j][0] = ref.step(w, st, steps=1, spectra=spectra, threads=1 if per_world else cores)
        return w.width * w.height

    while t_total < min_seconds:
        js = [(i + k) % len(todo) for k in range(min(batch, len(todo)))]
        for j in js:
            if j not in prepared:  # initial state and kernel spectrum, outside the timed region
                w, s = todo[j]
                prepared[j] = [ref.seed_patches(w.width, w.height, s, w.seed.patches), ref.spectra(w)]
        t0 = time.perf_counter()
        done = sum(pool.map(step_one, js)) if pool else step_one(js[0])
        t_total += time.perf_counter() - t0
        cells += done
        steps_done += len(js)
        i = (i + len(js)) % len(todo)
    if pool:
        pool.shutdown()
    sample = ("%d generation(s) over %d of the workload's world(s) (one-channel, power-of-two sides), %.1f s "
              "of wall time, %d threads (%s)" % (steps_done, min(len(todo), steps_done), t_total, cores,
                                                 "a world per thread" if per_world else
                                                 "the world's rows and columns over the threads"))
    return cells / t_total, cores, sample


def run_reference(args, dist):
    worlds, seeds, cfg = workload(args.config, args.only_side, args.max_worlds)
    if dist.rank != 0:
        return
    from oracle.oracle import RefF32
    cores = os.cpu_count() or 1
    ref = RefF32(threads=cores)
    pot = [(w, s) for w, s in zip(worlds, seeds) if w.channels == 1 and (w.width & (w.width - 1)) == 0]
    # one bench step = one generation of as many worlds as fit in ~2 s of CPU work
    prepared = []
    for w, s in pot:
        prepared.append((w, ref.seed_patches(w.width, w.height, s, w.seed.patches), ref.spectra(w)))
        if sum(x[0].width * x[0].height for x in prepared) >= 4096 * 4096:
            break

    # Several worlds: every host core steps whole worlds of its own, one thread each (the oracle
    # releases the GIL), which keeps all cores busy on small worlds where threading one world's rows
    # and columns does not; one world: its rows and columns over all cores.
    from concurrent.futures import ThreadPoolExecutor
    per_world = len(prepared) > 1
    pool = ThreadPoolExecutor(max_workers=cores) if per_world else None

    def step_one(i):
        w, st, sp = prepared[i]
        prepared[i] = (w, ref.step(w, st, steps=1, spectra=sp, threads=1 if per_world else cores), sp)
        return w.width * w.height

    def one():
        if pool:
            return sum(pool.map(step_one, range(len(prepared))))
        return sum(step_one(i) for i in range(len(prepared)))

    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    cells = 0
    for _ in range(args.steps):
        cells += one()
    dt = time.perf_counter() - t0
    if pool:
        pool.shutdown()
    value = cells / dt
    cfg.update({"path": "cpu restatement of spectral.rs (radix-2 Stockham, f32)", "gens_per_step": 1})
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": cfg,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": "%d world(s) one generation per step, %d threads (%s); the reference (Rust + "
                                      "WGSL on Vulkan) cannot build or run on this box" % (
                                          len(prepared), cores, "a world per thread" if per_world else
                                          "the world's rows and columns over the threads")},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ----------------------------------------------------------------------------- our arm

TRAFFIC_JSON = os.path.join(ROOT, "profiles", "traffic.json")


def read_traffic():
    try:
        return json.load(open(TRAFFIC_JSON))
    except Exception:
        return {}


_UNIT_SCALE = {"byte": 1.0, "kbyte": 1e3, "mbyte": 1e6, "gbyte": 1e9, "kibyte": 1024.0, "mibyte": 1024.0 ** 2,
               "gibyte": 1024.0 ** 3, "nsecond": 1e-9, "usecond": 1e-6, "msecond": 1e-3, "second": 1.0,
               "ns": 1e-9, "us": 1e-6, "ms": 1e-3}


def parse_ncu_csv(path):
    """Per-launch metrics of an ``ncu --csv`` log: a list of (kernel name, {metric: value in bytes or
    seconds}) in launch order."""
    import csv
    rows = []
    with open(path, newline="") as f:
        lines = [l for l in f if l.startswith('"')]  # drop ncu's own ==PROF== lines
    launches = {}
    order = []
    for r in csv.DictReader(lines):
        lid = r.get("ID")
        if lid is None or r.get("Metric Name") is None:
            continue
        if lid not in launches:
            launches[lid] = (r.get("Kernel Name", ""), {})
            order.append(lid)
        try:
            v = float(r["Metric Value"].replace(",", ""))
        except ValueError:
            continue
        v *= _UNIT_SCALE.get((r.get("Metric Unit") or "byte").strip().lower(), 1.0)
        launches[lid][1][r["Metric Name"]] = v
    for lid in order:
        rows.append(launches[lid])
    return rows


def summarise_traffic(csv_path, config, path, gens, graph=False):
    """DRAM bytes per generation of one graph replay (``--profile-window``): every launch's
    dram__bytes_read.sum + dram__bytes_write.sum summed and divided by the generations the replay
    ran, with the share of each kernel family.  With ``graph`` the capture holds one result, the
    whole replay profiled as one workload.  Written to profiles/traffic.json under
    "<config>/<path>"."""
    rows = parse_ncu_csv(csv_path)
    if not rows:
        raise SystemExit("no launches in %s" % csv_path)
    fam = {}
    total_b = total_t = 0.0
    for name, m in rows:
        b = m.get("dram__bytes_read.sum", 0.0) + m.get("dram__bytes_write.sum", 0.0)
        t = m.get("gpu__time_duration.sum", 0.0)
        # the kernel's own name: no return type, namespaces or template arguments
        key = name.split("(")[0].split("<")[0].replace("void ", "").split("::")[-1].strip()
        f = fam.setdefault(key, {"launches": 0, "dram_bytes": 0.0, "time_s": 0.0})
        f["launches"] += 1
        f["dram_bytes"] += b
        f["time_s"] += t
        total_b += b
        total_t += t
    for f in fam.values():
        f["share_of_bytes"] = f["dram_bytes"] / total_b if total_b else None
        f["share_of_time"] = f["time_s"] / total_t if total_t else None
    data = read_traffic()
    key = "%s/%s" % (config, path)
    data[key] = total_b / gens
    details = data.setdefault("details", {})
    details[key] = {"results": len(rows), "generations": gens, "dram_bytes_per_generation": total_b / gens,
                    "cache": "warm (ncu --cache-control none, one graph replay after warm-up)",
                    "profiled": ("the whole graph replay as one workload (ncu --graph-profiling graph): branches and "
                                 "lanes concurrent as in the timed run") if graph else
                                ("every launch on its own (ncu serialises them: a graph's concurrent lanes run one "
                                 "after another)"),
                    "kernels": fam}
    data["note"] = ("DRAM bytes per generation: dram__bytes_read.sum + dram__bytes_write.sum over one graph "
                    "replay, divided by its generations; command in profiles/traffic.md")
    with open(TRAFFIC_JSON, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    return data[key], details[key]


def profile_window(args, dist):
    """One bench step between cudaProfilerStart / cudaProfilerStop, after the same set-up,
    autotuning and warm-up as the timed run, for ``ncu --profile-from-start off``."""
    import torch
    from auto_gb300 import Sim
    worlds, seeds, cfg = workload(args.config, args.only_side, args.max_worlds)
    sim = Sim(worlds, seed=0, path=args.path)
    seed_all(sim, worlds, seeds)
    if not args.no_autotune:
        sim.autotune()
    if args.tc_rows:
        sim.set_tc_rows(True)
    if args.variants:
        vc, vr = (int(x) for x in args.variants.split(","))
        sim.set_variants(vc, vr)
    for _ in range(args.warmup):
        sim.step(args.gens)
    sim.wait()
    torch.cuda.init()
    torch.cuda.profiler.start()
    sim.step(args.gens)
    sim.wait()
    torch.cuda.profiler.stop()
    sim.close()
    print(json.dumps({"profile_window": args.config, "path": args.path, "generations": args.gens}))


def run_ours(args, dist):
    import auto_gb300 as ag
    from auto_gb300 import Sim

    worlds, seeds, cfg = workload(args.config, args.only_side, args.max_worlds)
    scaling = "weak"
    if dist.world > 1 and len(worlds) > 1:
        # several worlds: split them across ranks (total work fixed); one world: every rank a replica
        idx = shard(worlds, dist.rank, dist.world)
        worlds, seeds = [worlds[i] for i in idx], [seeds[i] for i in idx]
        scaling = "strong"
    sim = Sim(worlds, seed=0, path=args.path)
    seed_all(sim, worlds, seeds)
    if not args.no_autotune:
        sim.autotune()  # the engine's autotuner: times every launch variant per size class
    if args.tc_rows:
        sim.set_tc_rows(True)
    # launch shape per size class after autotuning: variants (column: 0/1 scalar at 64/128 registers,
    # 2 paired; row: 0/1), chunks of worlds run back to back through L2, rows per row item, the
    # cluster-resident step, and whether the row pass runs on the tensor cores
    variants = {"%dx%d" % wh: {"column": v["column_variant"], "row": v["row_variant"], "chunks": v["chunks"],
                               "worlds": v["worlds"], "chunk_budget_mib": v["chunk_budget_mib"],
                               "rows_per_row_item": v["rows_per_row_item"], "resident": v["resident"],
                               "resident_variant": v["resident_variant"], "tc_rows": v["tc_rows"],
                               "tc_column_variant": v["tc_column_variant"], "persistent": v["persistent"],
                               "lanes": v["lanes"]}
                for wh, v in sim.shapes().items()}
    G = args.gens
    cells = sim.cells_per_step
    for _ in range(args.warmup):
        sim.step(G)
    sim.wait()
    device_sync()
    dist.barrier()
    device_sync()
    clocks = Clocks(getattr(dist, "gpu_index", dist.local))
    clocks.start()
    ms = sim.step_timed(args.steps * G)
    device_sync()
    dist.barrier()
    device_sync()
    clk = clocks.stop()
    ms = dist.max(ms)
    total_cells = dist.sum(cells)
    value = total_cells * G * args.steps / (ms * 1e-3)
    ms_per_gen = ms / (args.steps * G)

    # per-kernel breakdown (event-timed launches on the engine stream, right after the timed region)
    prof = sim.profile(5)
    col_ms, row_ms, step_ms = [float(x) for x in prof]
    # per size class: its launches timed alone, and its cell-updates/s at that time
    class_cells = {}
    for w in worlds:
        class_cells[(w.width, w.height)] = class_cells.get((w.width, w.height), 0) + w.channels * w.width * w.height
    classes = {}
    if len(class_cells) > 1 and args.path != "radix2":
        # per class, alone: column and row launches each under events (serial), and the class as the
        # step graph runs it (chunks on their lanes), which gives its rate
        for (cw, ch), (cms, rms, gms) in sorted(sim.profile_classes(3).items()):
            n = class_cells[(cw, ch)]
            v = variants.get("%dx%d" % (cw, ch), {})
            classes["%dx%d" % (cw, ch)] = {"worlds": sum(1 for w in worlds if (w.width, w.height) == (cw, ch)),
                                           "column_ms": cms, "row_ms": rms, "graph_ms": gms,
                                           "cell_updates_per_s": n / (gms * 1e-3) if gms > 0 else None,
                                           "launch_variant": v}
    nclasses = len({(w.width, w.height) for w in worlds})
    # per size class (per chunk of a chunked class) and generation: one column and one row launch; the
    # tensor-core paths add the FP32 column launch for each channel's first tile group (sizes 256..4096)
    tc_sizes = (256, 512, 1024, 2048, 4096)
    shapes = sim.shapes()
    launches_per_gen = sum((3 if args.path in ("tf32", "bf16x3") and h in tc_sizes else 2) *
                           max(1, shapes.get((wd, h), {}).get("chunks", 1))  # a chunked class: per chunk
                           for (wd, h) in {(w.width, w.height) for w in worlds}
                           if not shapes.get((wd, h), {}).get("resident") and shapes.get((wd, h), {}).get("persistent", -1) < 0)
    # a cluster-resident or persistent class is one launch per bench step (all G generations)
    launches_per_step_resident = sum(1 for v in shapes.values() if v.get("resident") or v.get("persistent", -1) >= 0)
    if args.path == "radix2":
        n = worlds[0].width
        lg = int(np.log2(n))
        launches_per_gen = len(worlds) * (1 + 2 * lg + 1 + len(worlds[0].kernels) * (2 + 2 * lg) + 1)

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    achieved = alg_bytes_per_gen(worlds) / (ms_per_gen * 1e-3) / 1e9
    traffic = read_traffic().get("%s/%s" % (args.config, args.path))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "peak_source": peak_src,
                "what": "whole step (column + row launch) as the unit: (8 C + 4 K) H W bytes per world-generation "
                        "(12 B per cell-update at C = K = 1) over the event-timed "
                        "generation time",
                "kernels": {"column_ms": col_ms, "row_ms": row_ms, "step_ms_serial": step_ms,
                            "column_share": col_ms / step_ms if step_ms else None,
                            "column_own_bytes_per_cell": 8.0 + 1.0, "row_own_bytes_per_cell": 16.0,
                            "column_gbs": cells * 9.0 / (col_ms * 1e-3) / 1e9 if col_ms else None,
                            "row_gbs": cells * 16.0 / (row_ms * 1e-3) / 1e9 if row_ms else None}}

    e2e = None
    if not args.no_e2e:
        import torch
        # every world's state in pinned host buffers, world after world: the steps' input and result
        n = sum(w.channels * w.height * w.width for w in worlds)
        a_in = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        a_out = torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        sim.read_states(a_in)
        L = sim._L
        from auto_gb300._lib import check, fptr
        # Every bench step uploads every state, runs G generations and downloads every state,
        # through the public C ABI.  Streamed: the copies run on the engine's copy stream and
        # overlap the generations of the neighbouring steps.
        sim.write_states_async(a_in)  # staging buffers allocated outside the timed region
        sim.read_states_async(a_out)
        sim.wait()
        device_sync()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            check(L.lenia_write_states_async(sim._ctx, fptr(a_in), a_in.size), sim._ctx)
            check(L.lenia_step(sim._ctx, G), sim._ctx)
            check(L.lenia_read_states_async(sim._ctx, fptr(a_out), a_out.size), sim._ctx)
        sim.wait()
        device_sync()
        t_e2e = dist.max(time.perf_counter() - t0)
        # the same with blocking copies, each step waiting for its own download
        device_sync()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            check(L.lenia_write_states(sim._ctx, fptr(a_in), a_in.size), sim._ctx)
            check(L.lenia_step(sim._ctx, G), sim._ctx)
            check(L.lenia_read_states(sim._ctx, fptr(a_out), a_out.size), sim._ctx)
        device_sync()
        t_block = dist.max(time.perf_counter() - t0)
        e2e = {"value": total_cells * G * args.steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": a_in.nbytes,
               "d2h_bytes_per_step": a_out.nbytes, "gens_per_step": G,
               "copies": "streamed: lenia_write_states_async / lenia_read_states_async overlap the steps",
               "blocking_value": total_cells * G * args.steps / t_block}

    # every step path on the same workload, side by side (event-timed, state resident)
    paths = {}
    if not args.no_paths:
        for pth in ("fp32", "bf16x3", "tf32", "radix2"):
            if pth == args.path:
                paths[pth] = {"value": value, "ms_per_generation": ms_per_gen}
                continue
            if pth == "radix2" and any(w.channels != 1 or (w.width & (w.width - 1)) or (w.height & (w.height - 1))
                                       for w in worlds):
                paths[pth] = {"value": None, "why": "the radix-2 path runs one-channel power-of-two worlds only"}
                continue
            with Sim(worlds, seed=0, path=pth) as other:
                seed_all(other, worlds, seeds)
                if not args.no_autotune:
                    other.autotune()
                g = G if pth != "radix2" else 4
                other.step(g)
                other.wait()
                reps = max(2, min(args.steps, 20)) if pth != "radix2" else 5
                t_ms = other.step_timed(reps * g)
                t_ms = dist.max(t_ms)
                paths[pth] = {"value": dist.sum(other.cells_per_step) * g * reps / (t_ms * 1e-3),
                              "ms_per_generation": t_ms / (reps * g)}
        if not any(w.channels != 1 or len(w.kernels) != 1 for w in worlds):
            # the tensor-core step with every row pass it can take on the tensor cores, and with every row
            # pass on the FP32 CUDA cores (the autotuned bf16x3 entry chooses per class)
            for name, on in (("bf16x3_tc_rows", True), ("bf16x3_fp32_rows", False)):
                with Sim(worlds, seed=0, path="bf16x3") as other:
                    seed_all(other, worlds, seeds)
                    if not args.no_autotune:
                        other.autotune()
                    other.set_tc_rows(on)
                    tc_classes = ["%dx%d" % k for k, v in other.shapes().items() if v["tc_rows"]]
                    other.step(G)
                    other.wait()
                    reps = max(2, min(args.steps, 20))
                    t_ms = dist.max(other.step_timed(reps * G))
                    paths[name] = {"value": dist.sum(other.cells_per_step) * G * reps / (t_ms * 1e-3),
                                   "ms_per_generation": t_ms / (reps * G),
                                   "tc_row_classes": tc_classes}
        if paths.get("fp32", {}).get("value") and paths.get("radix2", {}).get("value"):
            paths["fp32_over_radix2"] = paths["fp32"]["value"] / paths["radix2"]["value"]
        if paths.get("bf16x3", {}).get("value") and paths.get("radix2", {}).get("value"):
            paths["bf16x3_over_radix2"] = paths["bf16x3"]["value"] / paths["radix2"]["value"]
        if paths.get("bf16x3", {}).get("value") and paths.get("fp32", {}).get("value"):
            paths["bf16x3_over_fp32"] = paths["bf16x3"]["value"] / paths["fp32"]["value"]
        if len(worlds) > 1 and args.path != "radix2":
            # the same worlds one at a time, each alone in its own context (every k-th world, up to 48)
            pick = list(range(0, len(worlds), max(1, len(worlds) // 48)))[:48]
            one_ms, one_cells = 0.0, 0
            for i in pick:
                with Sim(worlds[i], seed=0, path=args.path) as one:
                    seed_all(one, [worlds[i]], [seeds[i]])
                    if not args.no_autotune:
                        one.autotune()
                    one.step(G)
                    one.wait()
                    one_ms += one.step_timed(2 * G)
                    one_cells += one.cells_per_step * 2 * G
            one_value = one_cells / (one_ms * 1e-3)
            paths["one_at_a_time"] = {"value": one_value, "worlds": len(pick),
                                      "what": "each sampled world alone in a context, %d generations each, "
                                              "summed cell-updates over summed event time" % (2 * G)}
            paths["batched_over_one_at_a_time"] = value / one_value

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        v, cores, sample = cpu_leg(worlds, seeds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    if dist.rank == 0:
        cfg.update({"path": args.path + ("+tc_rows" if args.tc_rows and args.path in ("bf16x3", "tf32") else ""),
                    "gens_per_step": G, "cells_per_generation": cells, "worlds": len(worlds),
                    "l2": "no flush: per-generation working set (state + half-spectrum + kernel spectrum) "
                          "exceeds the 129 MB L2" if cells >= 4096 * 4096 else "no flush",
                    "parallelism": ("replicas" if scaling == "weak" else "worlds sharded") if dist.world > 1
                    else "single"})
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": scaling,
               "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg, "roofline": roofline,
               "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": (launches_per_gen * G + launches_per_step_resident) * args.steps,
               "launch_variants": variants, "classes": classes, "branch_split": {"cells": sim.branch_split[0], "each_own_branch": sim.branch_split[1]},
               "paths": paths,
               "ms_per_generation": ms_per_gen, "reference_published": PUBLISHED_REF}
        print(json.dumps(out))
    if args.jsonl and dist.rank == 0:
        append_reference_sample(args.jsonl, sim, worlds, cfg, args.path)
    sim.close()


def reference_rate(sim, seconds=2.0, warmup=32):
    """Steps/s measured the reference's way (crates/auto-cli/src/bench.rs:112-166): warm up, grow the
    batch until one submit takes >= 20 ms, then run batches for `seconds`; returns the median rate,
    the 10-90% spread, the batch and the number of batches."""
    sim.step(warmup)
    sim.wait()
    batch = 1
    while True:
        t = time.perf_counter()
        sim.step(batch)
        sim.wait()
        dt = time.perf_counter() - t
        if dt >= 0.02 or batch >= 1 << 16:
            break
        want = int(math.ceil(batch * 0.025 / max(dt, 1e-5)))
        batch = min(max(want, batch + 1), batch * 8, 1 << 16)
    rates = []
    start = time.perf_counter()
    while time.perf_counter() - start < seconds or len(rates) < 3:
        t = time.perf_counter()
        sim.step(batch)
        sim.wait()
        rates.append(batch / (time.perf_counter() - t))
    rates.sort()
    median = rates[len(rates) // 2]
    spread = (rates[len(rates) * 9 // 10] - rates[len(rates) // 10]) / median
    return median, spread, batch, len(rates)


def append_reference_sample(path, sim, worlds, cfg, impl_path, seconds=2.0):
    """One record in the reference's results/*.jsonl format (crates/auto-cli/src/bench.rs:39-55),
    measured its way (reference_rate)."""
    median, spread, batch, nb = reference_rate(sim, seconds=seconds)
    cells = int(sim.cells_per_step)
    w0 = worlds[0]
    rec = {"id": w0.id if len(worlds) == 1 else "batched", "tag": impl_path, "adapter": "NVIDIA GB300 (CUDA, sm_103a)",
           "checks": "Safe", "width": int(w0.width), "height": int(w0.height), "cells": cells,
           "memory_bytes": int(sim.memory_bytes), "steps_per_second": float(median),
           "generations_per_second": float(median), "cells_per_second": float(median * cells),
           "batch_steps": int(batch), "batches": int(nb), "spread": float(spread)}
    with open(path, "a") as f:
        f.write(json.dumps(rec) + "\n")


# The reference's published rows for its own programs (results/gpu.jsonl:78-91, RX 7900 XT,
# wgpu/Vulkan): program, side, cells/s.
REFERENCE_GRIDS = [("lenia", 512, 6.337e8), ("lenia", 1024, 6.834e8), ("lenia", 2048, 6.272e8),
                   ("lenia", 4096, 3.174e8), ("lenia", 8192, 1.571e8), ("smoothlife", 1024, 4.561e8),
                   ("smoothlife", 4096, 2.119e8), ("mnca", 1024, 4.560e8), ("mnca", 4096, 2.135e8)]


def run_grids(args, dist):
    """One JSON line per published grid: the same program and size here, measured the reference's
    way, next to the reference's own number.  The lenia program starts from U[0,1] patches instead
    of the reference's Orbium tiling (an FFT step's speed does not depend on the state's values);
    SmoothLife and MNCA use their own on-device seeds."""
    import auto_gb300 as ag
    from auto_gb300 import Sim
    if dist.rank != 0:
        return
    for prog, side, published in REFERENCE_GRIDS:
        world = {"lenia": ag.lenia, "smoothlife": ag.smoothlife, "mnca": ag.mnca}[prog](side, side)
        with Sim(world, seed=1, path=args.path) as sim:
            if prog == "lenia":
                q = side // 4
                sim.seed_patches(0, 1, [(q, q, side // 2, side // 2)])
            if not args.no_autotune:
                sim.autotune()
            rate, spread, batch, nb = reference_rate(sim)
            cells = sim.cells_per_step
        print(json.dumps({"grid": "%s %dx%d" % (prog, side, side), "path": args.path,
                          "cells_per_second": rate * cells, "steps_per_second": rate, "spread": spread,
                          "batch_steps": batch, "batches": nb,
                          "reference_published": published, "over_reference": rate * cells / published,
                          "reference_hardware": "AMD RX 7900 XT (wgpu/Vulkan)"}), flush=True)


def main():
    args = parse()
    gpu = pin_gpu()
    dist = Dist()
    dist.gpu_index = gpu
    try:
        if args.traffic_from:
            per_gen, det = summarise_traffic(args.traffic_from, args.config, args.path, args.gens, args.traffic_graph)
            print(json.dumps({"traffic_per_generation": per_gen, "details": det}))
        elif args.profile_window:
            profile_window(args, dist)
        elif args.impl == "reference":
            run_reference(args, dist)
        elif args.grids:
            run_grids(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
