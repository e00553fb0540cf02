"""Benchmark: 2.5D space-charge macroparticle-kicks/s on the FODO workload
(1e6 protons at 1 GeV, 128x128x64 grid, 40 TEAPOT FODO cells with 4 SC
nodes each = 160 SC kicks per turn), plain FP64 form by default.

One step = one turn of the lattice over the whole bunch (160 kicks).
  value  : device-timed throughput with the bunch resident in HBM; the L2
           (129 MB > the 48 MB bunch) is flushed by writing a 512 MiB buffer
           before every timed step.
  e2e    : the same metric through the reference-facing API with host
           buffers: per step, upload the coordinates from pinned host memory,
           Lattice.trackBunch, download the coordinates to pinned memory.
  --impl reference : the CPU restatement of the reference algorithm
           (oracle/, all host threads as MPI-rank-like slices) on a bounded
           sample of the same workload.
Multi-GPU (torchrun): independent replicas, one bunch per rank (the path
has no data-path collective in a one-GPU-per-bunch layout).
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "py-orbit_gb300"))

N_PARTICLES = 1_000_000
GRID = (128, 128, 64)
CELLS = 40
METRIC = "2.5D SC macroparticle-kicks/s, 1M particles 128x128 grid, vs FP64 plain form"
# CPU legs (the oracle on the host cores): the whole FODO bunch, one turn per
# step (the same configuration as the GPU arm); the large ring's 1.6e7
# particles take minutes per turn on the host, so it times a 1e6 sample.
CPU_SAMPLE_RING = 1_000_000
L2_NOTE = "GPU arm: flushed (512 MiB write) before each timed step"

# Algorithmic HBM bytes per particle of each particle kernel: the fused pass
# reads and writes x, xp, y, yp, z, dE; the deposit and the extrema scan
# read x, y, z; the stand-alone kick reads x, y, z, xp, yp and writes xp, yp.
ALG_BYTES = {"pass_kick_maps": 96, "pass_maps": 96, "deposit": 24, "extrema": 24, "kick": 56}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="plain", choices=["plain", "fp32", "learned", "learned-fp32"],
                    help="learned: the plain form with the trained denoiser closure, 1e5 particles by default; "
                         "learned-fp32: the same closure on the FP32 field form")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--error-turns", type=int, default=100,
                    help="turns of the rms-emittance and tune-shift error report of a non-plain form")
    ap.add_argument("--workload", default="fodo", choices=["fodo", "batched", "ring"],
                    help="fodo: one 1e6-particle bunch (default); batched: the 64-bunch scan; "
                         "ring: the large ring, 1.6e7 particles, 256x256x128")
    ap.add_argument("--members", type=int, default=64, help="bunches of the batched scan")
    ap.add_argument("--no-report", action="store_true",
                    help="skip the secondary reports (learned form: plain at equal density and force noise, emittance growth; "
                         "fp32 form: error report; batched: one-program-per-bunch comparison)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(v, dist, device="cuda"):
    """The largest v over the ranks (the slowest replica sets the job's
    time); v itself without a process group."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def measured_bf16_tflops():
    """The measured dense bf16 GEMM rate (burst), or None."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("bf16_tflops")
    return None


# Algorithmic FP64 operations per particle, counted from the reference
# formulas (each +, -, *, / is one operation; per-element constants that the
# reference computes once per call are not counted):
#   SC kick (SpaceChargeCalc2p5D.cc:104-119 with Grid2D::calcGradient and
#   Grid1D::getValue): indices and fractions 14, weights 16, derivative
#   weights 12, two 9-point sums 54, line density 12, factor 1, kicks 4 = 113
#   deposit (Grid2D::binValue + Grid1D::binValue): 14 + 16 + 27 + 12 = 69
#   maps (teapotbase.cc): drift 22, quad1 16, quad2/bend2 25, quad fringe 70,
#   bend1 18, bend3 20, bend4 14, bend fringe 16, multp 4 + 3 per pole,
#   rotatexy 12, wrap 2, kick 3
SC_KICK_FLOPS = 113
DEPOSIT_FLOPS = 69
MAP_FLOPS = {1: 22, 2: 16, 3: 25, 4: 70, 5: 70, 6: 18, 7: 25, 8: 20, 9: 14, 10: 16, 11: 16, 12: 7, 13: 60,
             14: 60, 15: 12, 16: 2, 17: 3, 18: 20, 19: 30, 20: 60}


# FP64-pipe instructions per particle (thread level: DFMA, DMUL, DADD, the
# conversions and compares) that the kernels execute on this workload,
# counted by ncu (sm__inst_executed_pipe_fp64.sum x 32 / particles, 4e6
# particles, the multiplies of the drift, quad fringe and bend maps on the
# integer pipes): the fused pass alternates the {kick, quad1, quad2 (the
# two back-to-back quad2 of the reference schedule merged), quad1,
# fringe-out} segment (56.1) and the {kick, drift, fringe-in} segment
# (38.1); the deposit runs 6.3 (one FMA per coordinate and the fixed-point
# conversions; weights and sums are integer).
FP64_INST_PER_PARTICLE = {"pass_kick_maps": (56.09 + 38.09) / 2, "deposit": 6.26}


def pass_flops_per_turn(ops):
    """FP64 operations per particle of all fused passes of one turn."""
    total = 0
    for code, ints, dbls in ops:
        if code == 32:
            total += SC_KICK_FLOPS
        else:
            f = MAP_FLOPS.get(code, 0)
            if code == 12 and ints:
                f = 4 + 3 * int(ints[0])
            total += f
    return total


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# The single-bunch workloads: coordinates, lattice, intensity, description.
WL = {"name": "fodo", "n": N_PARTICLES, "intensity": 1e14, "kicks": 160,
      "desc": "FODO 40 cells x 4 SC nodes"}


def wl_coords(n, seed):
    from orbit_gb300 import workloads as W
    return W.c5_coords(n, seed=seed) if WL["name"] == "ring" else W.c2_coords(n, seed=seed)


def wl_lattice(calc):
    from orbit_gb300 import workloads as W
    with quiet():
        return W.ring_lattice(calc) if WL["name"] == "ring" else W.fodo_lattice(calc, cells=CELLS)


def set_workload(name):
    global GRID
    if name == "ring":
        GRID = (256, 256, 128)
        WL.update({"name": "ring", "n": 16_000_000, "intensity": 1e14, "kicks": 129,
                   "desc": "large ring: 32 cells, 300 TEAPOT elements (sector bends 2pi/32, FODO quads, "
                           "sextupoles k2=+-2), 129 SC nodes; KV 6 mm/1 mrad, parabolic 250 m"})


def build_workload(n, form, seed):
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    soa = wl_coords(n, seed)
    bunch = W.make_bunch(soa, WL["intensity"] / n)
    calc = SpaceChargeCalc2p5D(*GRID, form={"learned": "plain", "learned-fp32": "fp32"}.get(form, form))
    if form in ("learned", "learned-fp32"):
        from orbit_gb300.denoiser import default_network
        calc.setDenoiser(default_network(size=GRID[0]), 10, 1e-3)
    lat = wl_lattice(calc)
    return soa, bunch, calc, lat


# Multiply-adds x 2 of one 128 x 128 forward pass of the denoiser: the 14
# 3x3 convolutions (H W 9 cin cout each) and the 1x1 output.
DENOISER_GFLOP_128 = 2 * sum(h * h * 9 * ci * co for h, ci, co in (
    (128, 1, 16), (128, 16, 16), (64, 16, 32), (64, 32, 32), (32, 32, 64), (32, 64, 64), (16, 64, 64), (16, 64, 64),
    (32, 128, 64), (32, 64, 64), (64, 96, 32), (64, 32, 32), (128, 48, 16), (128, 16, 16))) * 1e-9 + 2 * 128 * 128 * 16e-9


def learned_report(calc, ms_per_turn, n, n_equal=10_000_000, turns=10, form="plain"):
    """The learned form against the plain form at two particle counts: equal
    density noise (1e7, the network's training targets) and equal force
    noise (n times the network's measured gain in force error on 96 held-out
    synthetic beams, which is far below its gain in density error: the
    force weights beam-scale noise by 1/k^2 and a single snapshot cannot
    tell that noise from beam structure).  Reports one turn's time of the
    plain form at both counts (CUDA graphs, bunch resident) and the
    rms-emittance growth over `turns` turns of plain n_equal, plain n and
    learned n on the same lattice."""
    import numpy as np
    import torch
    from bunch import BunchTwissAnalysis
    from orbit_gb300 import workloads as W
    from orbit_gb300.denoiser import default_network, evaluate, make_pairs
    from spacecharge import SpaceChargeCalc2p5D

    def em(b):
        tw = BunchTwissAnalysis()
        tw.analyzeBunch(b)
        return np.array([tw.getEmittance(0), tw.getEmittance(1)])

    def setup(npart, with_net):
        b = W.make_bunch(W.c2_coords(npart, seed=77), W.C2_MACROSIZE * (N_PARTICLES / npart))
        c = SpaceChargeCalc2p5D(*GRID, form=form if with_net else "plain")
        if with_net:
            c.setDenoiser(default_network(), 10, 1e-3)
        with quiet():
            lat = W.fodo_lattice(c, cells=CELLS)
        return b, c, lat

    def plain_turn_ms(npart):
        b, c, lat = setup(npart, False)
        lat.trackBunchTurns(b, 1)  # records and captures
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lat.trackBunchTurns(b, 3)
        b._device_bunch().sync()
        return (time.perf_counter() - t0) / 3 * 1e3

    X, T, _ = make_pairs(96, seed=999)
    ev = evaluate(default_network(max_batch=16), X, T, force=True)
    del X, T
    n_force = int(round(n * ev["gain_force"]))
    plain_force_ms = plain_turn_ms(n_force)
    plain_equal_ms = plain_turn_ms(n_equal)
    growth = {}
    for name, npart, with_net in (("plain_%d" % n_equal, n_equal, False), ("plain_%d" % n, n, False),
                                  ("learned_%d" % n, n, True)):
        b, c, lat = setup(npart, with_net)
        e0 = em(b)
        lat.trackBunchTurns(b, turns)
        growth[name] = (em(b) / e0).tolist()
        if with_net:
            state = c.getDenoiserState()
    ref = np.array(growth["plain_%d" % n_equal])
    return {"equal_density_noise_particles": n_equal, "plain_equal_density_noise_ms_per_turn": plain_equal_ms,
            "speedup_vs_plain_equal_density_noise": plain_equal_ms / ms_per_turn,
            "network_gain": {k: ev[k] for k in ("gain", "gain_force", "gain_by_k", "k_bands")},
            "equal_force_noise_particles": n_force, "plain_equal_force_noise_ms_per_turn": plain_force_ms,
            "speedup_vs_plain_equal_force_noise": plain_force_ms / ms_per_turn,
            "emittance_growth_turns": turns, "emittance_growth": growth,
            "growth_dev_learned": (np.array(growth["learned_%d" % n]) / ref - 1).tolist(),
            "growth_dev_plain_same_n": (np.array(growth["plain_%d" % n]) / ref - 1).tolist(),
            "check": state, "check_this_run": calc.getDenoiserState(),
            "network_shape": "4-level conv encoder-decoder, 302,561 parameters, BF16 weights, shipped training"}


def ring_learned_report(calc, ms_per_turn, n, turns=100, form="fp32"):
    """The learned form on the large ring (the shipped convolutional
    network on the 256 x 256 grid) against the plain form at the ring's
    1.6e7 particles: one turn's time of each, and the rms-emittance growth
    over `turns` turns of plain 1.6e7, plain n and learned n (same beam,
    same lattice)."""
    import numpy as np
    import torch
    from bunch import BunchTwissAnalysis
    from orbit_gb300 import workloads as W
    from orbit_gb300.denoiser import default_network
    from spacecharge import SpaceChargeCalc2p5D

    def em(b):
        tw = BunchTwissAnalysis()
        tw.analyzeBunch(b)
        return np.array([tw.getEmittance(0), tw.getEmittance(1)])

    def setup(npart, with_net):
        b = W.make_bunch(W.c5_coords(npart, seed=78), WL["intensity"] / npart)
        c = SpaceChargeCalc2p5D(*GRID, form=form if with_net else "plain")
        if with_net:
            c.setDenoiser(default_network(size=GRID[0]), 10, 1e-3)
        with quiet():
            lat = W.ring_lattice(c)
        return b, c, lat

    b, c, lat = setup(WL["n"], False)
    lat.trackBunchTurns(b, 1)  # records and captures
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat.trackBunchTurns(b, 2)
    b._device_bunch().sync()
    plain_ms = (time.perf_counter() - t0) / 2 * 1e3
    growth, state = {}, None
    for name, npart, with_net in (("plain_%d" % WL["n"], WL["n"], False), ("plain_%d" % n, n, False),
                                  ("learned_%d" % n, n, True)):
        b, c, lat = setup(npart, with_net)
        e0 = em(b)
        lat.trackBunchTurns(b, turns)
        growth[name] = (em(b) / e0).tolist()
        if with_net:
            state = c.getDenoiserState()
    ref = np.array(growth["plain_%d" % WL["n"]])
    return {"plain_particles": WL["n"], "plain_ms_per_turn": plain_ms,
            "speedup_vs_plain_same_beam": plain_ms / ms_per_turn,
            "emittance_growth_turns": turns, "emittance_growth": growth,
            "growth_dev_learned": (np.array(growth["learned_%d" % n]) / ref - 1).tolist(),
            "growth_dev_plain_same_n": (np.array(growth["plain_%d" % n]) / ref - 1).tolist(),
            "check": state, "check_this_run": calc.getDenoiserState(),
            "network_shape": "the shipped 128 x 128-trained convolutional network run on the 256 x 256 grid"}


def cpu_reference_rate(n_sample, turns, warmup, threads):
    """Times the CPU restatement of the reference (oracle) on a sample of the
    FODO workload; returns (kicks/s, seconds per turn, kicks per turn)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from orbit_gb300 import workloads as W
    from orbit.teapot.recording import BunchRecorder
    from orbit.lattice import AccActionsContainer
    soa = wl_coords(n_sample, 99)

    class _Calc:  # records SC nodes without a GPU calculator
        def trackBunch(self, bunch, length, boundary=None):
            bunch._record_sc(self, length)

    lat = wl_lattice(_Calc())
    bunch = W.make_bunch(soa, WL["intensity"] / n_sample)
    rec = BunchRecorder(bunch)
    cont = AccActionsContainer()
    cont.addAction(lambda p: p["node"].track(p), AccActionsContainer.BODY)
    lat.trackActions(cont, {"bunch": rec, "useCharge": 1})
    ops = rec.ops
    kicks_per_turn = sum(1 for o in ops if o[0] == 32)
    s = bunch.getSyncParticle()
    sync = O.make_sync(beta=s.beta(), gamma=s.gamma(), momentum=s.momentum(), macrosize=bunch.macroSize())
    sc = [O.OracleSC(*GRID)]
    a = soa.copy()
    for _ in range(warmup):
        O.run_program(ops, 1, a, sync, sc, nthreads=threads)
    times = []
    for _ in range(turns):
        t0 = time.perf_counter()
        rc = O.run_program(ops, 1, a, sync, sc, nthreads=threads)
        times.append(time.perf_counter() - t0)
        if rc != 0:
            raise RuntimeError("oracle status %d" % rc)
    total = sum(times)
    return n_sample * kicks_per_turn * turns / total, total / turns, kicks_per_turn


def cpu_sample_n(n):
    """Particles of the CPU legs: the GPU arm's whole bunch, except on the
    large ring (a 1e6 sample of its 1.6e7)."""
    return min(n, CPU_SAMPLE_RING) if WL["name"] == "ring" else n


def bench_config(n, kicks_per_turn, form, world):
    """The workload description shared by both arms (same keys, same values
    where both run the same configuration)."""
    return {"workload": "%s, %d particles, grid %dx%dx%d, one turn per step" % (WL["desc"], n, *GRID),
            "form": form, "particles": n, "grid": list(GRID), "kicks_per_step": kicks_per_turn, "l2": L2_NOTE,
            "parallelism": "replicas" if world > 1 else "single"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = cpu_sample_n(WL["n"])
    rate, per_turn, kpt = cpu_reference_rate(n, args.steps, args.warmup, threads)
    ms_per_step = per_turn * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "macroparticle-kicks/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 4D waterbag rms 4 mm/0.8 mrad, z~N(0,10 m), dE~N(0,1 MeV))",
        "config": bench_config(n, kpt, "plain", 1),
        "cpu_baseline": {"value": rate, "unit": "macroparticle-kicks/s", "cores": threads, "kind": "port",
                         "sample": "%d particles x 1 turn (%d SC kicks) per step, %d threads as rank slices "
                                   "(the reference's MPI decomposition); the restatement reproduces the compiled "
                                   "reference bit for bit at one thread" % (n, kpt, threads)},
        "e2e": {"value": rate, "unit": "macroparticle-kicks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    torch.cuda.init()
    # the learned forms run at 1/100 (FODO, the network's training ratio) or
    # 1/40 (the ring's 256 x 256 grid: the same particles per cell as the
    # 1e5 training inputs on 128 x 128) of the plain form's particles
    n_learned = 100_000 if WL["name"] == "fodo" else WL["n"] // 40
    n = args.n if args.n else (n_learned if args.form.startswith("learned") else WL["n"])
    TRAFFIC.n = n
    soa, bunch, calc, lat = build_workload(n, args.form, seed=1000 + rank)
    prog = lat.fusedProgram(bunch)
    dev = bunch._device_bunch()
    stream = torch.cuda.ExternalStream(dev.stream_ptr())
    kicks_per_turn = sum(1 for o in prog.ops if o[0] == 32)
    # per-kernel times of one eager turn (CUDA events on the bunch's stream);
    # first, because it drops the captured graphs, which the warm-up turns
    # then capture again outside the timed region
    prof = prog.device.profile(dev)
    bunch._device_modified()
    for _ in range(max(args.warmup, 1)):
        prog.run(bunch, 1)
    launches_per_turn = prog.launches_per_turn()
    from orbit_gb300 import device_peaks
    fp64_peak, copy_gbs = device_peaks()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        dev.sync()
        if dist is not None:
            dist.barrier()

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    step_ms = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        prog.device.enqueue(dev, 1)
        e1.record(stream)
        dev.sync()
        step_ms.append(e0.elapsed_time(e1))
    wall = time.perf_counter() - wall0
    barrier()
    clk = clocks.stop()
    bunch._device_modified()
    total_ms = max_over_ranks(sum(step_ms), dist)
    kicks = world * n * kicks_per_turn * args.steps
    value = kicks / (total_ms * 1e-3)

    # ---- end to end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pin_in = torch.empty((6, n), dtype=torch.float64, pin_memory=True).numpy()
        pin_out = torch.empty((6, n), dtype=torch.float64, pin_memory=True).numpy()
        pin_in[...] = soa
        e2e_ms = []
        for i in range(args.steps + 1):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            bunch.setCoordinates(pin_in, copy=False)
            lat.trackBunch(bunch)
            bunch.getCoordinates(out=pin_out)
            t1 = time.perf_counter()
            if i > 0:  # the first call re-records and re-captures the graphs
                e2e_ms.append((t1 - t0) * 1e3)
        tot = max_over_ranks(sum(e2e_ms), dist)
        e2e = {"value": world * n * kicks_per_turn * len(e2e_ms) / (tot * 1e-3), "unit": "macroparticle-kicks/s",
               "h2d_bytes_per_step": int(pin_in.nbytes), "d2h_bytes_per_step": int(pin_out.nbytes),
               "ms_per_step": tot / len(e2e_ms)}

    if rank != 0:
        return
    # ---- roofline of the dominant kernel (largest share of the eager turn)
    hbm_peak, peak_kind = measured_peaks()
    turn_ms = sum(v[0] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    name, (dom_ms, dom_launches) = dom
    per_launch_ms = dom_ms / dom_launches
    alg_bytes = ALG_BYTES.get(name, 0) * n
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9 if alg_bytes else None
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if achieved else None, "traffic": TRAFFIC.get((args.form, name)),
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "kernel_ms_per_launch": per_launch_ms, "share_of_turn": dom_ms / turn_ms,
                "kernels": {k: {"ms": v[0], "launches": v[1], "share": v[0] / turn_ms} for k, v in prof.items()}}
    if name == "learn_network":
        # the learned forms: the network's 3x3 layers run on the tensor cores
        # (TF32, half the BF16 rate); the bound is its FLOPs per forward over
        # the forward's time (one 128 x 128 image per kick: latency-bound)
        bf16 = measured_bf16_tflops()
        tf32_peak = bf16 / 2.0 if bf16 else 1900.0 / 2.0
        tflops = DENOISER_GFLOP_128 * (GRID[0] * GRID[1] / 16384.0) * 1e-3 / (per_launch_ms * 1e-3)
        roofline.update({"bound": "tensor", "achieved": tflops, "peak": tf32_peak, "unit": "TFLOP/s",
                         "frac": tflops / tf32_peak, "traffic": None,
                         "peak_source": "half the measured bf16 GEMM rate (MEASURED_PEAKS.json bf16_tflops)"
                         if bf16 else "half the fallback 1.9 PFLOP/s bf16"})
    if args.form in ("plain", "fp32") and name in ("pass_kick_maps", "pass_maps"):
        # The fused pass keeps the maps in FP64 (both forms) and is bound by
        # the FP64 pipe, not by HBM: its roof is the FP64 rate.  Algorithmic
        # work = the reference's FP64 operation count of every map and SC
        # kick the passes of one turn apply (FLOP-counting each +, -, *, /
        # of teapotbase.cc and of the kick formulas), over the passes' time,
        # against the DFMA rate measured in this process (2 FLOP per DFMA;
        # MEASURED_PEAKS.json has no FP64 figure).  The deposit, gradient
        # and extrema run on the integer pipes here, so the pass does the
        # reference's work in fewer FP64 instructions than its count / 2
        # and can read above 1.0.
        hbm = dict(roofline)
        hbm.pop("kernels", None)
        pass_ms = sum(v[0] for k, v in prof.items() if k in ("pass_kick_maps", "pass_maps"))
        flops_turn = pass_flops_per_turn(prog.ops) * float(n)
        tflops = flops_turn / (pass_ms * 1e-3) / 1e12
        roofline.update({
            "bound": "fp64", "kernel": "fused pass (kick + maps + extrema), all launches of one turn",
            "achieved": tflops, "peak": fp64_peak, "unit": "TFLOP/s", "frac": tflops / fp64_peak,
            "peak_source": "measured in this run (orbit_device_peaks: independent DFMA chains on every SM, "
                           "2 FLOP per DFMA); MEASURED_PEAKS.json carries no FP64 figure",
            "alg_flops_per_particle_turn": pass_flops_per_turn(prog.ops),
            "alg_count": "reference operation count of the SC kick (113 per particle) and of each map "
                         "(teapotbase.cc), bench.py MAP_FLOPS",
            "hbm": {"achieved": hbm["achieved"], "peak": hbm["peak"], "unit": "GB/s", "frac": hbm["frac"],
                    "traffic": hbm["traffic"], "alg_bytes_per_particle": ALG_BYTES[name],
                    "peak_source": hbm["peak_source"]}})
        # counted FP64 instructions (ncu) of the passes and of the deposit
        # against the live DFMA instruction rate
        peak_inst = fp64_peak / 2 * 1e12
        from orbit_gb300 import device_mul_rates
        m_fp64, m_int, m_mix = device_mul_rates()
        fp = {"peak_inst_per_s": peak_inst,
              "mul_rates_gmul_s": {"fp64_pipe": m_fp64, "integer_pipes": m_int, "both": m_mix,
                                   "note": "correctly rounded binary64 multiplies measured in this run; the maps' "
                                           "drift, quad-fringe and bend multiplies run on the integer pipes"}}
        for kname, ipp in FP64_INST_PER_PARTICLE.items():
            k_ms, k_l = prof.get(kname, (0.0, 0))
            if k_ms > 0 and args.form == "plain" and WL["name"] == "fodo":
                rate = ipp * n * k_l / (k_ms * 1e-3)
                fp[kname] = {"fp64_inst_per_particle": ipp, "achieved_inst_per_s": rate, "frac": rate / peak_inst}
        roofline["fp64_pipe"] = fp
    # how often the Poisson solver grid was reshaped (Green spectrum rebuilt)
    kicks_done, green_done = calc._calc.counters()
    green_rate = green_done / kicks_done if kicks_done else None
    learned = None
    if args.form.startswith("learned") and WL["name"] == "ring":
        learned = {} if args.no_report else ring_learned_report(calc, ms_per_turn=total_ms / args.steps, n=n,
                                                                  form="fp32" if args.form == "learned-fp32" else "plain")
    elif args.form.startswith("learned"):
        learned = {} if args.no_report else learned_report(calc, ms_per_turn=total_ms / args.steps, n=n,
                                                             form="fp32" if args.form == "learned-fp32" else "plain")
        # the network's arithmetic rate (TF32 tensor-core MMAs on BF16 weights)
        net_ms, net_l = prof.get("learn_network", (0.0, 0))
        if net_ms > 0:
            gflop = DENOISER_GFLOP_128 * (GRID[0] * GRID[1] / 16384.0)
            tflops = gflop / (net_ms / net_l)
            bf16_peak = measured_bf16_tflops()
            learned["network"] = {"gflop_per_forward": gflop, "ms_per_forward": net_ms / net_l,
                                  "achieved_tflops": tflops,
                                  "tensor_peak_tflops": bf16_peak / 2.0 if bf16_peak else None,
                                  "tensor_frac": tflops / (bf16_peak / 2.0) if bf16_peak else None,
                                  "note": "3x3 layers on the tensor cores (tcgen05 kind::tf32, FP32 accumulation "
                                          "in TMEM), one 128 x 128 image per kick, latency-bound; peak = half the "
                                          "measured bf16 GEMM rate (TF32 runs at half the BF16 rate); per-launch "
                                          "times of the eager profile"}
    form_err = None
    if args.form == "fp32" and args.error_turns > 0 and not args.no_report:
        # accuracy of the reduced-precision form against the FP64 plain form
        # on the same bunch (outside the timed region)
        from orbit_gb300 import workloads as W
        from orbit_gb300.form_report import form_error
        from spacecharge import SpaceChargeCalc2p5D

        def make_lattice(form):
            with quiet():
                return W.fodo_lattice(None if form is None else SpaceChargeCalc2p5D(*GRID, form=form), cells=CELLS)

        form_err = form_error(soa, bunch.macroSize(), make_lattice, args.form, turns=args.error_turns)
    cpu = None
    if not args.no_cpu and world == 1:
        threads = os.cpu_count() or 1
        ncpu = cpu_sample_n(n)
        rate, per_turn, kpt = cpu_reference_rate(ncpu, 1, 0, threads)
        cpu = {"value": rate, "unit": "macroparticle-kicks/s", "cores": threads, "kind": "port",
               "sample": "%d particles x 1 turn (%d SC kicks), %d threads as rank slices" % (ncpu, kpt, threads),
               "same_config": ncpu == n}
    line = {
        "metric": METRIC, "value": value, "unit": "macroparticle-kicks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"plain": "f64", "fp32": "f32-field/f64-coords",
                  "learned": "f64 + bf16-weight network (tf32 tensor-core MMA, f32 accumulation)",
                  "learned-fp32": "f32-field/f64-coords + bf16-weight network (tf32 tensor-core MMA, f32 accumulation)"
                  }[args.form],
        "data": "synthetic (seeded 4D waterbag rms 4 mm/0.8 mrad, z~N(0,10 m), dE~N(0,1 MeV))",
        "config": bench_config(n, kicks_per_turn, args.form, world),
        "green_rebuilds_per_kick": green_rate,
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": launches_per_turn * args.steps, "wall_s": wall,
    }
    if form_err is not None:
        line["form_error_vs_fp64"] = form_err
    if learned is not None:
        line["learned"] = learned
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# DRAM traffic per particle per launch, dram__bytes_read.sum +
# dram__bytes_write.sum from one ncu capture of a 4e6-particle run of this
# benchmark (bunch larger than L2); scaled to the bench's particle count.
TRAFFIC_PER_PARTICLE = {("plain", "pass_kick_maps"): 88.9, ("plain", "deposit"): 24.75}


class _Traffic(dict):
    n = N_PARTICLES

    def get(self, key, default=None):
        if WL["name"] != "fodo":  # captured on the FODO workload only
            return None
        v = TRAFFIC_PER_PARTICLE.get(key)
        return None if v is None else v * self.n


TRAFFIC = _Traffic()


def build_scan(members, cells=CELLS):
    """The batched scan: [(soa, bunch, lattice)] per member."""
    from orbit_gb300 import workloads as W
    from spacecharge import SpaceChargeCalc2p5D
    out = []
    for k, (n, grid, k1, intensity) in enumerate(W.c3_scan(members)):
        soa = W.c3_coords(n, seed=7000 + k)
        b = W.make_bunch(soa, intensity / n)
        with quiet():
            lat = W.fodo_lattice(SpaceChargeCalc2p5D(*grid), cells=cells, kq=k1)
        out.append((soa, b, lat))
    return out


def run_batched(args):
    """The 64-bunch scan: one step = one turn of every bunch through its
    own 40-cell FODO lattice, all bunches in one batch (orbit_batch_*)."""
    import torch
    rank, world, local = dist_env()
    dist = None
    if world > 1:  # replicas: every rank runs the whole scan on its own GPU
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist
    torch.cuda.init()
    from orbit_gb300.batch import BunchBatch
    scan = build_scan(args.members)
    bb = BunchBatch([(b, lat) for _, b, lat in scan])
    n_tot = sum(soa.shape[1] for soa, _, _ in scan)
    bb.trackTurns(max(args.warmup, 1))  # the first turn autotunes, the rest replays the graphs
    kicks_per_turn = sum(1 for o in scan[0][2].fusedProgram(scan[0][1]).ops if o[0] == 32)
    stream = torch.cuda.ExternalStream(bb._batch.stream_ptr())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    bb.sync()
    if dist is not None:
        dist.barrier()
    clocks.start()
    step_ms = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bb.enqueueTurns(1)
        e1.record(stream)
        bb.sync()
        step_ms.append(e0.elapsed_time(e1))
    wall = time.perf_counter() - wall0
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(step_ms), dist)
    value = world * n_tot * kicks_per_turn * args.steps / (total_ms * 1e-3)
    # the same bunches tracked one program each (each bunch on its own
    # stream, so the programs overlap as far as the GPU lets them)
    def unbatched_turn():
        for _, b, lat in scan:
            lat.fusedProgram(b).device.enqueue(b._device_bunch(), 1)
            b._device_modified()
        for _, b, _ in scan:
            b._device_bunch().sync()

    unb_ms = None
    if not args.no_report:
        unbatched_turn()  # records the programs and captures their graphs
        unb_turns = 2
        t0 = time.perf_counter()
        for _ in range(unb_turns):
            unbatched_turn()
        unb_ms = (time.perf_counter() - t0) * 1e3 / unb_turns
    # end to end: upload every bunch from pinned host memory, one turn,
    # download every bunch
    e2e = None
    if not args.no_e2e:
        pins = []
        for soa, b, _ in scan:
            pi = torch.empty(soa.shape, dtype=torch.float64, pin_memory=True).numpy()
            po = torch.empty(soa.shape, dtype=torch.float64, pin_memory=True).numpy()
            pi[...] = soa
            pins.append((pi, po))
        e2e_ms = []
        for i in range(min(args.steps, 3) + 1):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for (pi, _), (_, b, _) in zip(pins, scan):
                b.setCoordinates(pi, copy=False)
            bb.trackTurns(1)
            for (_, po), (_, b, _) in zip(pins, scan):
                b.getCoordinates(out=po)
            t1 = time.perf_counter()
            if i > 0:  # the first call re-records the programs and recaptures the graphs
                e2e_ms.append((t1 - t0) * 1e3)
        tot = max_over_ranks(sum(e2e_ms), dist)
        e2e = {"value": world * n_tot * kicks_per_turn * len(e2e_ms) / (tot * 1e-3), "unit": "macroparticle-kicks/s",
               "h2d_bytes_per_step": int(sum(p[0].nbytes for p in pins)),
               "d2h_bytes_per_step": int(sum(p[1].nbytes for p in pins)), "ms_per_step": tot / len(e2e_ms)}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    prof = bb.profile()
    hbm_peak, peak_kind = measured_peaks()
    turn_ms = sum(v[0] for v in prof.values())
    # per grid class: particles, and the achieved bandwidth of its kick
    # passes (96 B per particle) and deposits (24 B per particle)
    per_class = {}
    for soa, b, lat in scan:
        calc = lat.fusedProgram(b).calcs[0]
        g = "%dx%dx%d" % (calc._calc.nx, calc._calc.ny, calc._calc.nz)
        per_class[g] = per_class.get(g, 0) + soa.shape[1]
    kinds = {}
    for g, npart in per_class.items():
        for stage, nbytes in (("batch_pass_", 96.0), ("batch_deposit_", 24.0)):
            ms, launches = prof.get(stage + g, (0.0, 0))
            if ms > 0:
                kinds[stage + g] = {"ms": ms, "launches": launches, "particles": npart,
                                    "achieved_gbs": nbytes * npart * kicks_per_turn / (ms * 1e-3) / 1e9}
    # the dominant stage over all classes: the kick passes
    pass_ms = sum(v[0] for k, v in prof.items() if k.startswith("batch_pass_") and k != "batch_pass_maps")
    achieved = 96.0 * n_tot * kicks_per_turn / (pass_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": "batch_pass (kick + maps + extrema, all classes)", "achieved": achieved,
                "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "share_of_turn": pass_ms / turn_ms, "per_class": kinds,
                "kernels": {k: {"ms": v[0], "launches": v[1], "share": v[0] / turn_ms} for k, v in prof.items()}}
    cpu = None
    if not args.no_cpu and world == 1:
        threads = os.cpu_count() or 1
        rate, per_turn, kpt = cpu_reference_rate(N_PARTICLES, 1, 0, threads)
        cpu = {"value": rate, "unit": "macroparticle-kicks/s", "cores": threads, "kind": "port",
               "sample": "%d particles x 1 turn of the 128x128x64 FODO lattice (%d SC kicks), %d threads"
                         % (N_PARTICLES, kpt, threads)}
    classes = bb.classes()
    line = {
        "metric": METRIC, "value": value, "unit": "macroparticle-kicks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian 6D bunches of the scan)",
        "config": {"workload": "batched scan: %d bunches, %d particles in all (log-uniform 5e4-2e6), "
                               "intensity 1e12-2e14, k1 0.3-0.7, grids 64x64x32/128x128x64/256x256x64, "
                               "40-cell FODO x 4 SC nodes, one turn per step" % (len(scan), n_tot),
                   "particles": n_tot, "members": len(scan), "kicks_per_step": kicks_per_turn,
                   "classes": classes, "l2": "flushed (512 MiB write) before each timed step; inputs > L2",
                   "unbatched_ms_per_turn": unb_ms, "parallelism": "replicas" if world > 1 else "single"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": bb.launchesPerTurn() * args.steps, "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    set_workload(args.workload)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
