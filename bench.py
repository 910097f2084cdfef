#!/usr/bin/env python
"""Throughput of the GB300 membrane MD step: bead-steps/s on one GB300.

Workload (default): the flat tensionless bilayer of 20,000 three-bead lipids
(60,000 beads) at 3.45 lipids/sigma^2, z box 15 sigma, constant-tension MC
barostat on (deltaLXY 0.01, tension 0), Langevin gamma 1, kT 3, dt 0.02,
mixed precision.  Seeded synthetic input built in the reference generator's
geometry, equilibrated for 1,000 untimed steps.

One bench step = 80 MD loop iterations (MD.cpp:335-729), ten barostat
periods of resizeRate 8, on the device-resident state, launched as one CUDA
graph per period; L2 is flushed (256 MiB write) between timed steps and every
step is bracketed by CUDA events on the library's stream.  `e2e` runs the same
metric through the C ABI with host buffers: per e2e step the state is
uploaded, 48 iterations are advanced, the energies are measured and the state
is read back.

`roofline` is the whole MD step against HBM: 176 algorithmic bytes per
bead-step (x and v FP64 read and write, the 16-byte position mirror written
and read, the int64 force accumulator written and read) times the measured
bead-steps/s, over the measured copy bandwidth.  `kernels` gives the same
figure for the pair pass + integrator alone, timed per launch with CUDA
events, and `issue` the instruction-issue bound of the step from the warp
instructions the committed ncu capture counted.  `force_err` is the mixed
form's force error against the oracle's FP64 forces on the bench's own state.

Other workloads (--workload): vesicle5k (15,000-bead vesicle, no barostat),
batch64 (64 independent bilayers of 1,000-8,000 lipids and tension 0-1, one
handle, one set of launches per step), sphere80k (240,001-bead vesicle with a
continuum sphere) and adjoint10k (gradient of a 200-step window of a
30,000-bead bilayer: forward, recompute and backward passes).  Under torchrun
every rank runs its own copy of the workload (weak scaling, no data-path
collective), except batch64, whose 64 replicas are split across the ranks
(strong scaling).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload bilayer20k|vesicle5k|batch64|sphere80k|adjoint10k]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG_BYTES_PER_BEAD_STEP = 176  # x,v FP64 r/w 96 + position mirror w/r 32 + force accumulator w/r 48
METRIC = "bead-steps/s on 1 GB300 (mixed precision)"
UNIT = "bead-steps/s"
E2E_INTERVAL = 48  # six barostat periods: one e2e step = upload, 48 MD steps, energies, download
PERIOD = 8         # MD steps of one barostat period (resizeRate, MD.cpp:67)
STEP_MD = 10 * PERIOD  # MD steps per bench step (20 bench steps take over 100 ms)
SMS = 152          # GB300 streaming multiprocessors
ISSUE_PER_SM_CLK = 4  # warp instructions issued per SM and clock (four schedulers)
# DRAM bytes and warp instructions per bead and MD step of the mixed step,
# summed over every kernel of the step with its launches per MD step, from ncu
# captures of the workload (metrics dram__bytes_read.sum, dram__bytes_write.sum,
# smsp__inst_executed.sum per kernel).  "warm": one pass per launch with the
# caches as the previous kernels left them (--cache-control none), the traffic
# of the bench's L2-resident loop; "cold": every launch after an L2 flush, each
# kernel's whole working set from DRAM (an upper bound).  The commands and the
# per-kernel tables are in profiles/step_traffic_warm_bilayer60k.md and
# profiles/step_traffic_bilayer60k.md.  Traffic is a named constant because ncu
# cannot run inside the timed region.
STEP_PROFILE = {
    "bilayer20k": {"dram_bytes_per_bead_step": 54.0, "dram_bytes_per_bead_step_cold": 773.0,
                   "warp_inst_per_bead_step": 618.0,
                   "source": "profiles/step_traffic_warm_bilayer60k.md (ncu --cache-control none: the bench's "
                             "L2-resident loop; traffic and instructions) and profiles/step_traffic_bilayer60k.md "
                             "(ncu, caches flushed per launch: an upper bound on traffic)"},
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# Verlet-list skin per workload.  The list lives a whole number of steps,
# mostly two, at kT 3 and dt 0.02: it is rebuilt once the fastest bead has
# moved skin/2, about 0.19 sigma per step at 60,000 beads and more for more
# beads (the largest of more Maxwell draws).  The smallest skin that still
# keeps two steps is the fastest: 0.42 for the 15,000- and 60,000-bead
# systems; the 240,001-bead vesicle and the 64-replica batch (up to 480,000
# beads) rebuild after one step too often at 0.42 and keep the library's 0.5.
SKIN_DEFAULT = {"bilayer20k": 0.42, "vesicle5k": 0.42}


def workload(args, rank, tmpdir, world=1):
    """(paths, systems, config) of the benchmarked workload for one rank.
    The config dict describes the whole job and is the same in both arms."""
    import softmold_gb300 as smd
    from softmold_gb300.scaling import replica_range
    if args.workload == "bilayer20k":
        path = os.path.join(tmpdir, f"bench{rank}.mpd")
        smd.synth_bilayer(path, 1000 + rank, 20000, 3.45, 15.0, 0.01, 0.0)
        cfg = {"workload": "flat tensionless bilayer, 20,000 3-bead lipids (60,000 beads), 3.45/sigma^2, "
                           "z 15 sigma, MC barostat deltaLXY 0.01 tension 0, kT 3, gamma 1, dt 0.02"}
        paths = [path]
    elif args.workload == "vesicle5k":
        path = os.path.join(tmpdir, f"bench{rank}.mpd")
        smd.synth_vesicle(path, 1000 + rank, 5000, 3.45, 60.0)
        cfg = {"workload": "vesicle, 5,000 3-bead lipids (15,000 beads), 60^3 box, kT 3, gamma 1, dt 0.02"}
        paths = [path]
    elif args.workload == "sphere80k":
        path = os.path.join(tmpdir, f"bench{rank}.mpd")
        # sphere radius 5, surface 2 sigma outside the outer heads; head well Umin -10.  The table's
        # inner polynomial keeps beads out only while (Umax - Umin)/6 > ~2.3 |Umin|: heads Umax 300
        # (barrier ~+530 at 1 sigma inside the surface), tails Umax 100 (soft repulsion, no well)
        smd.synth_vesicle_sphere(path, 1000 + rank, 80000, 3.45, 190.0, 5.0, -10.0, 300.0, 2.0, 100.0)
        cfg = {"workload": "vesicle of 80,000 3-bead lipids (240,001 beads with the sphere), 190^3 box, one "
                           "continuum sphere R 5 sigma 2 sigma outside the outer heads (head Umin -10 Umax 300, "
                           "tail Umax 100, range 2), kT 3, gamma 1, dt 0.02"}
        paths = [path]
    elif args.workload == "adjoint10k":
        path = os.path.join(tmpdir, f"bench{rank}.mpd")
        smd.synth_bilayer(path, 1000 + rank, 10000, 3.45, 15.0, 0.0, 0.0)
        cfg = {"workload": "adjoint of a 200-step window (checkpoints every 20) of a flat bilayer of 10,000 "
                           "3-bead lipids (30,000 beads), box fixed, kT 3, gamma 1, dt 0.02"}
        paths = [path]
    elif args.workload == "batch64":
        # the same 64 replicas for every job size; under torchrun each rank
        # advances its share (replica_range) and the job's total is fixed
        rng = np.random.default_rng(64)
        lipids = rng.integers(1000, 8001, size=64)
        tensions = rng.uniform(0.0, 1.0, size=64)
        paths = []
        for k in replica_range(64, rank, world):
            path = os.path.join(tmpdir, f"bench{rank}_{k}.mpd")
            smd.synth_bilayer(path, 5000 + k, int(lipids[k]), 3.45, 15.0, 0.01, float(tensions[k]))
            paths.append(path)
        cfg = {"workload": "64 independent flat bilayers in one batch, 3-bead lipids per replica uniform in "
                           "[1000, 8000] (seeded), tension uniform in [0, 1], own seed and box each, z 15 sigma, "
                           "MC barostat deltaLXY 0.01, kT 3, gamma 1, dt 0.02",
               "replicas": 64, "lipids_per_replica": [int(x) for x in lipids]}
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    return paths, [smd.read_mpd(p) for p in paths], cfg


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region: NVML
    (read-only queries through ctypes) every 20 ms, else nvidia-smi every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReasons bits
    REASONS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
               "hw_thermal_slowdown": 0x40, "hw_power_brake_slowdown": 0x80}

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.nvml = None
        self.lines = []
        self.samples = []  # (sm_mhz, sm_max_mhz, reason bits)
        self.halt = threading.Event()

    def _nvml_open(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return False
        if lib.nvmlInit_v2() != 0:
            return False
        h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.dev), C.byref(h)) != 0:
            return False
        self.reason_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.nvml, self.handle, self.C = lib, h, C
        return True

    def _nvml_loop(self):
        C, lib, h = self.C, self.nvml, self.handle
        sm, smax, bits = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.halt.is_set():
            if (lib.nvmlDeviceGetClockInfo(h, 1, C.byref(sm)) == 0 and
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(smax)) == 0 and
                    self.reason_fn(h, C.byref(bits)) == 0):
                self.samples.append((float(sm.value), float(smax.value), int(bits.value)))
            self.halt.wait(0.02)

    def start(self):
        if self._nvml_open():
            self.t = threading.Thread(target=self._nvml_loop, daemon=True)
            self.t.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def started(self):
        return bool(self.samples or self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.nvml is not None:
            self.halt.set()
            self.t.join(timeout=2)
            self.nvml.nvmlShutdown()
            sm = [s[0] for s in self.samples]
            reasons = sorted({k for s in self.samples for k, b in self.REASONS.items() if s[2] & b})
            return {"sm_mhz": statistics.median(sm) if sm else None,
                    "sm_max_mhz": max(s[1] for s in self.samples) if sm else None,
                    "reasons": reasons, "samples": len(sm), "source": "nvml, 20 ms"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def oracle_time(path, threads, steps):
    """Seconds of `steps` MD steps of the oracle's restatement of the
    reference loop (oracle/md_oracle.cpp) on .mpd `path`, timed in a fresh
    Python process that loads nothing but the oracle: inside this process,
    beside torch's OpenMP runtime and the CUDA context, the same loop runs
    about 30 % slower (10.4 M against 14.2 M bead-steps/s on the 60,000-bead
    bilayer, 16 Arm cores)."""
    code = ("import ctypes as C, sys\n"
            "lib = C.CDLL(sys.argv[1])\n"
            "lib.orc_md_time.argtypes = [C.c_char_p, C.c_int, C.c_int]\n"
            "lib.orc_md_time.restype = C.c_double\n"
            "print(lib.orc_md_time(sys.argv[2].encode(), int(sys.argv[3]), int(sys.argv[4])))\n")
    lib = os.path.join(ROOT, "oracle", "_build", "libsmd_oracle.so")
    r = subprocess.run([sys.executable, "-c", code, lib, path[:-4], str(threads), str(steps)], capture_output=True,
                       text=True, env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
    try:
        t = float(r.stdout.strip().splitlines()[-1])
    except (ValueError, IndexError):
        t = -1.0
    if r.returncode != 0 or t < 0:
        raise RuntimeError(f"the oracle could not run {path}: {r.stderr[-300:]}")
    return t


def cpu_baseline(path, threads, target_s=12.0):
    """The oracle's restatement of the reference MD loop on the host cores."""
    t = oracle_time(path, threads, 4)
    steps = max(4, int(4 * target_s / max(t, 1e-3)))
    return steps, oracle_time(path, threads, steps)


def melt_on_host(path, threads, steps):
    """Runs the oracle's MD loop (the reference `MD` restated) on the host for
    `steps` untimed steps from the workload's lattice start and leaves the
    final state in the .mpd, so that the reference arm samples the same kind
    of state as the GPU arm (which equilibrates on the device)."""
    import re
    import subprocess
    d, base = os.path.split(path)
    txt = open(path).read()
    dt = float(re.search(r"^deltaT\s+(\S+)", txt, re.M).group(1))
    t_end = repr(steps * dt)
    for key in ("finalTime", "storeInterval", "measureInterval"):
        txt = re.sub(rf"^{key}\s+\S+", f"{key} {t_end}", txt, flags=re.M)
    open(path, "w").write(txt)
    exe = os.path.join(ROOT, "oracle", "_build", "md_oracle")
    r = subprocess.run([exe, base[:-4], str(threads)], cwd=d, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
    if r.returncode != 0:
        raise RuntimeError(f"the oracle could not run {path}: {r.stdout[-300:]} {r.stderr[-300:]}")


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm (the oracle port of
    MD.cpp, built here) on all host threads, same workload, config and
    metric; one bench step is a sample of STEP_MD MD steps."""
    if rank != 0:
        return
    from softmold_gb300 import build
    build.build_oracle()
    with tempfile.TemporaryDirectory() as tmp:
        paths, ms, cfg = workload(args, 0, tmp)
        threads = os.cpu_count() or 1
        # melt the lattice start on the host, as the GPU arm does on the device
        # (up to 1,000 steps, at most 2.5e8 bead-steps for the whole workload)
        n_all = sum(len(m.type) for m in ms)
        melt = max(100, min(1000, int(2.5e8 / n_all)))
        for p_ in paths:
            melt_on_host(p_, threads, melt)
        import ctypes as C
        lib = C.CDLL(os.path.join(ROOT, "oracle", "_build", "libsmd_oracle.so"))
        lib.orc_md_time.argtypes = [C.c_char_p, C.c_int, C.c_int]
        lib.orc_md_time.restype = C.c_double
        # one bench step: STEP_MD MD steps of the system, or of one replica of
        # a batch in turn (replicas are independent: bead-steps and times add)
        for k in range(args.warmup):
            lib.orc_md_time(paths[k % len(paths)][:-4].encode(), threads, 2)
        total, units = 0.0, 0
        for k in range(args.steps):
            j = k % len(paths)
            total += lib.orc_md_time(paths[j][:-4].encode(), threads, STEP_MD)
            units += len(ms[j].type) * STEP_MD
        value = units / total
        n = sum(len(m.type) for m in ms)
        what = f"the {n}-bead workload" if len(ms) == 1 else f"replicas of the {len(ms)}-replica batch in turn"
        sample = f"{args.steps} samples of {STEP_MD} MD steps of {what}, after {melt} untimed steps from the lattice start"
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)


def oracle_forces(ms, pos, boxes):
    """The oracle's FP64 conservative forces (CellOpt::computeForce +
    Blob::doChainForce + doBeadForce restated in oracle/smd_oracle.cpp) of
    every replica at the given state, in input order: the checker behind
    force_err."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_binding import Oracle
    orc = Oracle()
    out, base = [], 0
    for m, b in zip(ms, boxes):
        n = len(m.type)
        g = {"pos": np.ascontiguousarray(pos[base:base + n]), "type": m.type, "box": b, "cutoff": m.cutoff,
             "n_types": m.n_types, "fconst": m.fconst, "chain_blocks": m.chain_blocks,
             "chain_consts": m.chain_consts}
        if m.sphere_index is not None and len(m.sphere_index):
            g["sphere_index"], g["sphere_consts"] = m.sphere_index, m.sphere_consts
        out.append(orc.forces(g))
        base += n
    return np.concatenate(out)


def bench_adjoint(args, s, stream, n, cfg, world, rank, dist):
    """One bench step = smd_adjoint over a 200-step window, checkpoints every
    20 (forward, recompute and backward passes); value = beads x window steps
    per second of that call."""
    import torch
    T, ck = 200, 20
    for _ in range(args.warmup):
        s.adjoint(T, ck, segment_local=True)
    torch.cuda.synchronize()
    times, grads = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = s.adjoint(T, ck, segment_local=True)
        times.append(time.perf_counter() - t0)
        grads.append(r["grad"].tolist())
    tot = sum(times)
    if rank == 0:
        print(json.dumps({
            "metric": "adjoint bead-steps/s on 1 GB300 (mixed, 200-step window, checkpoint every 20)",
            "value": n * T * args.steps / tot, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair terms, f64 adjoint", "data": "synthetic",
            "config": cfg, "segment_local_grad_last": grads[-1],
            "note": "host wall clock around smd_adjoint (it synchronises); the reference has no adjoint"}),
            flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


def profile_run(args):
    """The workload kernel by kernel, for ncu (which cannot see the kernel
    nodes of graphs with conditional nodes): the default launch
    configuration (8 lanes per bead, the flat list build with 128 threads),
    1,001 equilibration steps, then args.profile_run steps."""
    import softmold_gb300 as smd
    from softmold_gb300 import build
    build.build_library()
    tmp = tempfile.mkdtemp(prefix="smd_prof_")
    _, ms, _ = workload(args, 0, tmp)
    s = smd.System(ms if len(ms) > 1 else ms[0], precision=smd.MIXED, skin=args.skin)
    s.use_graphs(False)
    s.set_tuning(8, 0)
    s.prepare()
    s.advance(1001)
    r0 = s.rebuilds()
    s.advance(args.profile_run)
    print(f"rebuilds {s.rebuilds() - r0} in {args.profile_run} steps; launches {s.launches()}")
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="bilayer20k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--skin", type=float, default=None,
                    help="Verlet-list skin in sigma (default: per workload, SKIN_DEFAULT)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the step kernels one by one (for profilers that cannot see kernels in graphs)")
    ap.add_argument("--profile-run", type=int, default=0, metavar="STEPS",
                    help="for ncu: equilibrate the workload kernel by kernel with the default launch "
                         "configuration, run STEPS more MD steps and exit (no timing, no JSON line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.skin is None:
        args.skin = SKIN_DEFAULT.get(args.workload, 0.5)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.profile_run:
        return profile_run(args)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import softmold_gb300 as smd
    from softmold_gb300 import build
    from softmold_gb300.scaling import job_throughput
    build.build_library()

    tmp = tempfile.mkdtemp(prefix="smd_bench_")
    paths, ms, cfg = workload(args, rank, tmp, world)
    m = ms if len(ms) > 1 else ms[0]
    n = sum(len(x.type) for x in ms)
    stream = torch.cuda.Stream()
    s = smd.System(m, precision=smd.MIXED, skin=args.skin)
    s.set_stream(stream.cuda_stream)
    if args.no_graphs:
        s.use_graphs(False)
    s.prepare()
    s.advance(1001)  # equilibration from the lattice start (untimed); leaves step % PERIOD == 1

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    K, W = args.steps, args.warmup
    if args.workload == "adjoint10k":
        return bench_adjoint(args, s, stream, n, cfg, world, rank, dist)

    def timed_loop(sys_, steps):
        """`steps` bench steps of STEP_MD MD steps each, L2 flushed before each."""
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        l0 = sys_.timing()[2]
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.zero_()
                starts[k].record(stream)
                sys_.advance(STEP_MD, asynchronous=True)
                ends[k].record(stream)
        torch.cuda.synchronize()
        sys_.sync()
        launches = sys_.timing()[2] - l0
        ms_ = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        return sum(ms_), launches

    timed_loop(s, W)
    rebuilds0 = s.rebuilds()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    t_wait = time.time()
    while not sampler.started() and time.time() - t_wait < 5:  # sampler start-up outside the timed region
        time.sleep(0.05)
    torch.cuda.nvtx.range_push("timed")
    total_ms, launches = timed_loop(s, K)
    torch.cuda.nvtx.range_pop()
    clocks = sampler.stop()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    rebuilds = s.rebuilds() - rebuilds0
    last_disp, slack = s.list_state()
    value, _, max_s = job_throughput(n * STEP_MD * K, total_ms / 1e3, dist, "cuda")
    max_ms = 1e3 * max_s
    # per-launch times of the pair and integrate passes (profiling mode records
    # events around every step, so it launches kernel by kernel, untimed here)
    s.profile(True)
    timed_loop(s, min(K, 4))
    kernel_ms, kernel_launches, _ = s.timing()
    s.profile(False)

    # FP64 plain form on the same state
    pos, vel = s.state()
    boxes = [s.box(r) for r in range(len(ms))]  # the boxes of this state (the e2e run below moves them on)
    offs = np.cumsum([0] + [len(x.type) for x in ms])
    for r in range(len(ms)):
        q = pos[offs[r]:offs[r + 1]]
        if not (np.isfinite(q).all() and (q >= 0).all() and (q <= boxes[r]).all()):
            raise RuntimeError(f"replica {r} left its box: the run blew up (bead-steps/s not reported)")
    p = smd.System(m, precision=smd.PLAIN_FP64, skin=args.skin)
    p.set_stream(stream.cuda_stream)
    for r in range(len(ms)):
        p.set_box(boxes[r], r)
    p.set_state(pos, vel)
    f_plain = p.forces()
    f_mixed = s.forces()
    p.prepare()
    p.advance(1)  # step % PERIOD == 1, where a barostat period starts
    kp = min(K, 3)
    timed_loop(p, 1)
    plain_ms, _ = timed_loop(p, kp)
    plain_value, _, _ = job_throughput(n * STEP_MD * kp, plain_ms / 1e3, dist, "cuda")
    p.close()

    # end to end through the C ABI with host buffers
    hp = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    hv = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    hp[:], hv[:] = s.state()
    e2e_t = []
    for k in range(args.e2e_steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.set_state(hp, hv)
        s.advance(E2E_INTERVAL)
        e = s.energy()
        s.state(hp, hv)
        t1 = time.perf_counter()
        if k >= 2:
            e2e_t.append(t1 - t0)
    e2e_value, _, _ = job_throughput(n * E2E_INTERVAL, statistics.mean(e2e_t), dist, "cuda")
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(hp.nbytes + hv.nbytes),
           "d2h_bytes_per_step": int(hp.nbytes + hv.nbytes + 32),
           "md_steps_per_e2e_step": E2E_INTERVAL, "potential_last": e[0]["pair"] + e[0]["bonded"]}

    # the whole step against HBM (176 algorithmic bytes per bead-step), and
    # the pair + integrate passes alone from their per-launch CUDA events
    peak, peak_kind = load_peaks()
    us_md_step = max_ms * 1e3 / (K * STEP_MD)
    achieved = value * ALG_BYTES_PER_BEAD_STEP / 1e9
    prof = STEP_PROFILE.get(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": prof["dram_bytes_per_bead_step"] * n if prof else None,
                "traffic_cold": prof["dram_bytes_per_bead_step_cold"] * n if prof else None,
                "traffic_per": "MD step, every kernel of the step (DRAM read + write); traffic with the caches "
                               "as the step leaves them, traffic_cold with L2 flushed before every launch",
                "alg_bytes_per_bead_step": ALG_BYTES_PER_BEAD_STEP, "alg_bytes_per_md_step": ALG_BYTES_PER_BEAD_STEP * n,
                "kernel": "the whole MD step (every kernel, list builds and barostat passes included)",
                "peak_source": f"{peak_kind} hbm_gbs"}
    kernels = None
    if kernel_launches:
        avg_us = 1e3 * kernel_ms / kernel_launches
        kernels = {"k_force + k_integ": {
            "avg_us_per_md_step": avg_us, "achieved_gbs": ALG_BYTES_PER_BEAD_STEP * n / (avg_us * 1e3),
            "frac": ALG_BYTES_PER_BEAD_STEP * n / (avg_us * 1e3) / peak, "launch_pairs": kernel_launches,
            "share_of_step": avg_us / us_md_step}}
    issue = None
    if prof and clocks.get("sm_mhz"):
        inst = prof["warp_inst_per_bead_step"] * n  # per MD step
        bound_us = inst / (SMS * ISSUE_PER_SM_CLK * clocks["sm_mhz"] * 1e6) * 1e6
        issue = {"warp_inst_per_md_step": inst, "issue_peak_warp_inst_per_s": SMS * ISSUE_PER_SM_CLK * clocks["sm_mhz"] * 1e6,
                 "bound_us_per_md_step": bound_us, "measured_us_per_md_step": us_md_step,
                 "frac": bound_us / us_md_step, "source": prof["source"]}

    base = None
    force_err = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        f_ref = oracle_forces(ms, pos, boxes)
        fscale = np.abs(f_ref).max()
        force_err = {"max": float(np.abs(f_mixed - f_ref).max() / fscale),
                     "rms": float(np.sqrt(np.mean((f_mixed - f_ref) ** 2)) / fscale),
                     "plain_max": float(np.abs(f_plain - f_ref).max() / fscale),
                     "reference": "FP64 oracle (the reference's computeForce + doChainForce + doBeadForce restated) "
                                  "on the bench's final state, relative to max |F|"}
        threads = os.cpu_count() or 1
        # equilibrated state of (a sample of) the replicas, timed one after another
        sample = range(len(ms)) if len(ms) == 1 else range(0, len(ms), 16)
        units, secs = 0, 0.0
        for r in sample:
            ck = os.path.join(tmp, f"cpu{r}.mpd")
            a, b = offs[r], offs[r + 1]
            smd.mpd_update_state(paths[r], ck, pos[a:b], vel[a:b], boxes[r], 0.0)
            st, t_ = cpu_baseline(ck, threads, target_s=12.0 / len(sample))
            units += (b - a) * st
            secs += t_
        what = (f"the same {n}-bead system" if len(ms) == 1 else
                f"replicas {list(sample)} of the batch ({sum(offs[r + 1] - offs[r] for r in sample)} beads) "
                f"one after another")
        base = {"value": units / secs, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"MD steps of {what} (equilibrated state), oracle port of MD.cpp with OpenMP"}
    s.close()
    if rank == 0:
        run = {"beads_per_gpu": n, "md_steps_per_bench_step": STEP_MD, "us_per_md_step": us_md_step,
               "l2": "flushed (256 MiB write) between timed steps", "skin": args.skin,
               "parallelism": (f"replicas split over {world} ranks" if args.workload == "batch64" and world > 1
                               else f"replicas x{world}"),
               "list_rebuilds_per_md_step": rebuilds / (K * STEP_MD), "last_max_displacement": last_disp}
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": max_ms / K, "higher_is_better": True,
            "scaling": "strong" if args.workload == "batch64" and world > 1 else "weak", "vs_baseline": None,
            "dtype": "f32+i64 fixed-point forces, f64 integrate", "data": "synthetic", "config": cfg, "run": run,
            "roofline": roofline, "kernels": kernels, "issue": issue, "cpu_baseline": base, "e2e": e2e,
            "clocks": clocks, "gpu_launches": launches,
            "plain_fp64": {"value": plain_value, "ms_per_step": plain_ms / kp,
                           "mixed_speedup": value / plain_value},
            "force_err": force_err,
        }), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
