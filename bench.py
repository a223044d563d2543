"""Benchmark of the probe-particle AFM hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload slab_molecule]
                    [--impl ours|reference] [--cpu-budget S] [--no-cpu-baseline]

One step = one full pass of the reference CPU pipeline's work on the workload: the
Lennard-Jones + point-charge force field with the Fmax clamps and FF = FFLJ + Q*FFel
(one fused kernel), the relaxed scan with FIRE at every pixel and height, and Fz -> Δf
(fused into the relaxation kernel).  Default workload: the 2000-atom slab + 60-atom
molecule, 800x800x500 grid, 512x512x40 scan (the large single system).

Printed (rank 0, one JSON line): value = relaxed pixel-heights per second of the whole
step with the atoms already in device memory; e2e = the same metric through the public
host API (ppafm_gb300.HighLevel.Pipeline with host atoms in and host fzs/positions/Δf
out, copies inside the timed region); roofline of the dominant kernel (force field,
float32-FMA bound) against an FFMA peak measured in the same process; the CPU baseline
(the reference pipeline on this host's cores, bounded sample, extrapolated).

Multi-GPU (torchrun, N > 1): every rank relaxes its own independent system (weak scaling,
no collective on the data path); value = all ranks' pixel-heights / max rank time.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "relaxed pixel-z points/s & FF grid-pt·atoms/s; FIRE iters/pixel at 1e-4 eV/Å"
UNIT = "pixel-z/s"
FLOPS_LJ_PAIR = 26  # float32 flops per atom-point pair, FMA = 2 (LJ only)
FLOPS_LJC_PAIR = 30  # LJ + Coulomb sharing r^2
FLOPS_TIP_CHARGE_PAIR = 20  # one AFMulator tip charge on one atom (FF.cl evalLJC_QZs_noPos)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="slab_molecule", choices=["slab_molecule", "small_molecule", "density_overlap", "molecule_batch", "afmulator"])
    ap.add_argument("--nmol", type=int, default=256)
    ap.add_argument("--no-learned", action="store_true", help="molecule_batch: skip the learned warm start")
    ap.add_argument("--train-steps", type=int, default=480000, help="molecule_batch: Adam steps of the warm-start network (outside the timed region)")
    ap.add_argument("--tuning", default=None, help="molecule_batch launch shape 'ctas_per_sm,tile_w,tile_h,chunk' (default: autotuned)")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--relax-tps", type=int, default=0, help="lanes per stroke of the single-system relaxation (1, 2, 4, 8; 0 = library default)")
    ap.add_argument("--no-extras", action="store_true", help="default workload: skip the other workloads added to the line (the 256-molecule batch with its per-molecule loop and learned warm start, the small molecule, the density-overlap route, the AFMulator)")
    return ap.parse_args()


def dist_env():
    from ppafm_gb300.ranks import dist_env as env

    return env()


def make_workload(name, seed, scale):
    from ppafm_gb300 import workloads

    return getattr(workloads, name)(seed=seed, scale=scale)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
        sm, smax, reasons = [], [], set()
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": float(max(smax)) if smax else None, "reasons": sorted(reasons), "samples": len(sm)}


def read_profile_traffic(kernel, workload):
    """DRAM bytes per launch of a kernel from its committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def read_measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def ffma_peak_tflops(torch, lib, check, tptr, stream_handle):
    """FP32 FMA peak of this GPU measured now: dependent FFMA chains on every SM."""
    import ctypes

    scratch = torch.zeros(1024, device="cuda")
    cnt = ctypes.c_longlong(0)
    iters = 20000
    for _ in range(2):
        check(lib.ppgpu_ffma_peak(tptr(scratch), iters, ctypes.byref(cnt), stream_handle()))
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        check(lib.ppgpu_ffma_peak(tptr(scratch), iters, ctypes.byref(cnt), stream_handle()))
        b.record()
        b.synchronize()
        t = a.elapsed_time(b) * 1e-3
        best = max(best, 2.0 * cnt.value / t / 1e12)
    return best


class PointChargeJob:
    """LJ + point-charge force field (one fused kernel), relaxed scan + Δf."""

    def __init__(self, w, relax, HL, torch):
        self.w = w
        self.torch = torch
        self.HL = HL
        self.pl = HL.Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], w, relax=relax, want_iters=False)
        self.npts = int(np.prod(self.pl.gridN))
        self.natoms = self.pl.natoms
        self.nch = self.pl.ncharged
        self.ff_name = "ff_kernel<LJC> (force field)" if self.pl.Q != 0.0 else "ff_kernel<LJ> (force field)"
        self.launches_per_step = 2
        self.pinned_slots(2)
        self.host_in = {k: np.asarray(w[k]).copy() for k in ("Zs", "Rs", "Qs")}

    def pinned_slots(self, n):
        """n pinned host buffers for the atom records of steps in flight."""
        self.rec_pinned = [self.torch.empty(self.pl.atoms.shape, dtype=self.pl.atoms.dtype, pin_memory=True) for _ in range(n)]

    def e2e_host(self, slot=0):
        """Host prep of one step (PBC images, LJ mixing, packing into pinned slot `slot`);
        returns the bytes e2e_h2d copies."""
        from ppafm_gb300.device import pack_atoms

        pl = self.pl
        Rs0, cLJs, kqq = self.HL.prepare_atoms(self.host_in["Zs"], self.host_in["Rs"], self.host_in["Qs"], pl.lvec, self.w)
        rec, _, _ = pack_atoms(Rs0, cLJs, kqq if pl.Q != 0.0 else None, device="cpu")
        pin = self.rec_pinned[slot]
        pin.copy_(rec)
        return int(pin.numel() * pin.element_size())

    def e2e_h2d(self, slot=0):
        """H2D of the atom records of pinned slot `slot` (on the current stream)."""
        self.pl.atoms.copy_(self.rec_pinned[slot], non_blocking=True)

    def ff_roofline(self, t_ff, peak_fp32):
        if self.pl.Q != 0.0:
            flops = self.npts * ((self.natoms - self.nch) * FLOPS_LJ_PAIR + self.nch * FLOPS_LJC_PAIR)
        else:
            flops = self.npts * self.natoms * FLOPS_LJ_PAIR
        achieved = flops / t_ff / 1e12
        return {"bound": "fp32", "kernel": self.ff_name, "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s", "frac": achieved / peak_fp32 if peak_fp32 else None, "peak_source": "FFMA microbenchmark measured in this run (MEASURED_PEAKS.json has no FP32 figure)", "flops_per_launch": flops}

    def config(self):
        return {"atoms": len(self.w["Zs"]), "atoms_with_images": self.natoms, "charged_atoms_with_images": self.nch}

    def extra(self, t_ff):
        return {"ff_grid_pt_atoms_per_s": self.npts * self.natoms / t_ff}


class OverlapJob:
    """FFT density-overlap route: Pauli + Hartree force field (cuFFT + fused k-space
    kernels), relaxed scan + Δf.  Inputs of a step: the three density grids."""

    def __init__(self, w, relax, HL, torch):
        self.w = w
        self.torch = torch
        self.pl = HL.DensityOverlapPipeline.from_workload(w, relax=relax, want_iters=False)
        self.npts = int(np.prod(self.pl.gridN))
        self.launches_per_step = 13  # 2 copies, 2 x (sums + power), 2 x (2 R2C, spectra, C2R x4, pack), R2C + poisson + C2R, relax (cuFFT launches counted as one each)
        self.host = [torch.empty(self.pl.gridN, dtype=torch.float32, pin_memory=True) for _ in range(3)]
        for h, d in zip(self.host, (self.pl.rho_s, self.pl.rho_q, self.pl.rho_t)):
            h.copy_(d)

    def pinned_slots(self, n):
        """The density grids stay in one pinned set: every step copies the same host arrays."""

    def e2e_host(self, slot=0):
        """Nothing to prepare: the density grids are pinned host arrays; returns their bytes."""
        return int(sum(h.numel() * h.element_size() for h in self.host))

    def e2e_h2d(self, slot=0):
        """H2D of the three density grids (on the current stream)."""
        for h, d in zip(self.host, (self.pl.rho_s, self.pl.rho_q, self.pl.rho_t)):
            d.copy_(h, non_blocking=True)
        return int(sum(h.numel() * h.element_size() for h in self.host))

    def ff_roofline(self, t_ff, peak_fp32):
        return None

    def config(self):
        return {"atoms": len(self.w["Zs"]), "fft": "float32 complex (cuFFT R2C/C2R)", "A_pauli": self.w["Apauli"], "B_pauli": self.w["Bpauli"]}

    def extra(self, t_ff):
        return {}


def cpu_batch_sample(systems, budget_s, seed=0):
    """The reference pipeline on the host cores for 4 molecules of the batch (each sampled by
    oracle/cpu_baseline.py), as pixel-heights per second."""
    try:
        from oracle import cpu_baseline

        picks = systems[:: max(1, len(systems) // 4)][:4]
        tot_s, tot_pz, info = 0.0, 0.0, None
        for m in picks:
            s = cpu_baseline.sample_pipeline(m, budget_s=budget_s / len(picks), seed=seed)
            tot_s += s["total_s"]
            tot_pz += s["pixel_z_per_s"] * s["total_s"]
            info = s
        return {"value": tot_pz / tot_s, "unit": UNIT, "cores": info["cores"], "kind": info["kind"], "sample": f"{len(picks)} of {len(systems)} molecules, each: " + info["sample"]}
    except Exception as e:  # the baseline is reported, never fatal
        return {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}


class BatchBench:
    """256-molecule batch: one persistent launch (force fields + relaxed scans + df of every
    molecule) replayed from a CUDA graph, launch shape from the autotuner.  Also times the
    plain GPU form (one HighLevel.Pipeline per molecule) for comparison."""

    def __init__(self, systems, relax, HL, torch, tuning=None):
        from ppafm_gb300 import batch as BT

        self.w = systems[0]
        self.systems = systems
        self.torch = torch
        self.HL = HL
        if tuning is None:
            self.tuning, self.tune_ms = BT.autotune(systems, self.w, relax, reps=2)
        else:
            self.tuning, self.tune_ms = tuple(tuning), None
        self.pl = BT.BatchPipeline(systems, self.w, relax=relax, want_ppos=True, tuning=self.tuning, out_sets=2)
        self.pl.capture()
        self.units = self.pl.pixel_z
        self.npts = int(sum(np.prod(s["n"]) for s in self.pl.systems))
        self.pairs = int(sum(np.prod(s["n"]) * s["natoms"] for s in self.pl.systems))
        self.launches_per_step = 1
        self.BT = BT
        self.relax = relax
        # two slots of pinned inputs and outputs and of device outputs (pipelined end-to-end
        # steps); the output copies run on their own stream
        self.pin_out = [[{k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in s["out"].items()} for s in self.pl.systems] for _ in range(2)]
        self.rec_pin = [[torch.empty(s["rec"].shape, dtype=s["rec"].dtype, pin_memory=True) for s in self.pl.systems] for _ in range(2)]
        self._done = [None, None]
        self._k = 0
        self.d2h_stream = torch.cuda.Stream()

    def step(self):
        self.pl.replay()

    def e2e_step(self):
        """Public API end to end, pipelined: host atoms of every molecule -> packed records in
        pinned slot k % 2 (H2D, in stream order: the launch before reads the records) -> the
        batched launch into device output set k % 2 -> those outputs to pinned slot k % 2 on
        the copy stream while the next launch writes the other set.  The host prepares step k
        while the GPU runs step k-1, waiting only for step k-2's outputs before it reuses
        their slots."""
        from ppafm_gb300.device import pack_atoms

        torch = self.torch
        st = torch.cuda.current_stream()
        slot = self._k % 2
        if self._done[slot] is not None:
            self._done[slot].synchronize()
        h2d = 0
        for s, w, pin in zip(self.pl.systems, self.systems, self.rec_pin[slot]):
            Rs0, cLJs, kqq = self.HL.prepare_atoms(w["Zs"], w["Rs"], w["Qs"], w["lvec"], self.w)
            rec, _, _ = pack_atoms(Rs0, cLJs, kqq, device="cpu")
            pin.copy_(rec)
            h2d += rec.numel() * rec.element_size()
        for s, pin in zip(self.pl.systems, self.rec_pin[slot]):
            s["rec"].copy_(pin, non_blocking=True)
        if self._done[slot] is not None:
            st.wait_event(self._done[slot])  # device output set `slot` has been copied out
        self.pl.replay(slot)
        ran = torch.cuda.Event()
        ran.record(st)
        d2h = 0
        ds = self.d2h_stream
        with torch.cuda.stream(ds):
            ds.wait_event(ran)
            for s, pin in zip(self.pl.systems, self.pin_out[slot]):
                for k, v in s["outs"][slot].items():
                    pin[k].copy_(v, non_blocking=True)
                    d2h += v.numel() * v.element_size()
            self._done[slot] = torch.cuda.Event()
            self._done[slot].record(ds)
        self._k += 1
        return h2d, d2h

    def e2e_drain(self):
        """The current stream waits for the output copies still in flight."""
        self.torch.cuda.current_stream().wait_stream(self.d2h_stream)

    def learned(self, args, plain_loop_ms, steps=480000, lr=1e-3):
        """Config-4 line: train the warm-start network on plain-FIRE pairs of a held-out batch
        (every 4th stroke of 256 other molecules: ~21M pairs; Adam, batch 8192, cosine-decayed
        learning rate, z error weighted 10x), then
        time the height-synchronous batched run with it (CUDA graph) against plain FIRE."""
        import torch

        from ppafm_gb300 import workloads
        from ppafm_gb300.warmstart import WarmStartNet, generate_pairs

        held = workloads.molecule_batch(seed=args.seed + 1000, nmol=args.nmol, scale=args.scale)
        t0 = time.perf_counter()
        X, T = generate_pairs(held, self.w, self.relax, stride=4, tuning=self.tuning)
        torch.cuda.synchronize()
        t_gen = time.perf_counter() - t0
        net = WarmStartNet(seed=0)
        t0 = time.perf_counter()
        log = net.train(X, T, steps=steps, batch=8192, lr=lr, log_every=steps // 3, schedule="cosine")
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t0
        npairs = int(X.shape[0])
        del X, T, held
        pl = self.BT.BatchPipeline(self.systems, self.w, relax=self.relax, want_ppos=False, want_iters=True, tuning=self.tuning)

        def its():
            return np.concatenate([pl.outputs(j)["iters"].cpu().numpy().ravel() for j in range(len(self.systems))])

        def dfs():
            return [pl.outputs(j)["df"].cpu().numpy().copy() for j in range(len(self.systems))]

        pl.run()
        torch.cuda.synchronize()
        it_plain, df_plain = its(), dfs()
        ms = {}
        clocks = ClockSampler(torch.cuda.current_device())
        clocks.start()
        for name, fn in (("learned", lambda: pl.run_layered(net)), ("layered_plain", lambda: pl.run_layered(None))):
            g = pl.capture(fn)
            g.replay()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(args.steps):
                g.replay()
            b.record()
            b.synchronize()
            ms[name] = a.elapsed_time(b) / args.steps
            if name == "learned":
                it_l, df_l = its(), dfs()
        clk = clocks.stop()
        dd = np.concatenate([np.abs(x - y).ravel() for x, y in zip(df_l, df_plain)])
        net.close()
        pl.close()
        return {
            "clocks": clk,
            "ms_per_step": ms["learned"],
            "value": self.units / (ms["learned"] * 1e-3),
            "speedup_vs_plain_gpu_loop": plain_loop_ms / ms["learned"],
            "layered_plain_ms_per_step": ms["layered_plain"],
            "fire_iters_per_pixel_z": {"plain_mean": float(it_plain.mean()), "plain_p99": float(np.percentile(it_plain, 99)), "learned_mean": float(it_l.mean()), "learned_p99": float(np.percentile(it_l, 99))},
            "df_vs_plain_fire": {"frac_over_0.1Hz": float((dd > 0.1).mean()), "p99.9_Hz": float(np.quantile(dd, 0.999)), "max_Hz": float(dd.max())},
            "training": {"pairs": npairs, "steps": steps, "batch": 8192, "lr": lr, "schedule": "cosine", "loss_weights": [1.0, 1.0, 10.0], "generate_s": t_gen, "train_s": t_train, "loss": log},
        }

    def plain_ms(self, reps=3):
        """The per-molecule loop (best of reps, CUDA events) and the clocks seen meanwhile."""
        pls = self.BT.plain_loop(self.systems, self.w, self.relax)
        torch = self.torch
        for p in pls:
            p.run()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        best = float("inf")
        clocks = ClockSampler(torch.cuda.current_device())
        clocks.start()
        for _ in range(reps):
            a.record()
            for p in pls:
                p.run()
            b.record()
            b.synchronize()
            best = min(best, a.elapsed_time(b))
        self.plain_clocks = clocks.stop()
        return best


def run_batch(args, rank, world, local):
    import torch

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import _lib, workloads

    torch.cuda.set_device(local)
    L = _lib.load()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    systems = workloads.molecule_batch(seed=args.seed + rank, nmol=args.nmol, scale=args.scale)
    w = systems[0]
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    tuning = [int(x) for x in args.tuning.split(",")] if args.tuning else None
    job = BatchBench(systems, relax, HL, torch, tuning=tuning)
    st = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        job.step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for a, b in ev:
        a.record(st)
        job.step()
        b.record(st)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    t_step = sum(a.elapsed_time(b) * 1e-3 for a, b in ev)
    iters = job.pl.iterations()
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    # end to end
    for _ in range(max(1, args.warmup)):
        job.e2e_step()
    barrier()
    torch.cuda.synchronize()  # the first timed step's host work falls inside the interval
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(args.steps):
        h2d, d2h = job.e2e_step()
    job.e2e_drain()
    b.record(st)
    b.synchronize()
    t_e2e = a.elapsed_time(b) * 1e-3
    from ppafm_gb300.ranks import max_over_ranks

    t_step_max, t_e2e_max = max_over_ranks([t_step, t_e2e], device="cuda")
    K = args.steps
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return None
    plain = job.plain_ms()
    learned = None
    if not args.no_learned:
        learned = job.learned(args, plain, steps=args.train_steps)
    peak = ffma_peak_tflops(torch, L, _lib.check, _lib.tptr, _lib.stream_handle)
    flops = job.pairs * FLOPS_LJC_PAIR
    line = {
        "metric": METRIC,
        "value": job.units * world * K / t_step_max,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_step_max / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {
            "workload": "molecule_batch",
            "molecules": len(systems),
            "atoms": [int(min(len(s["Zs"]) for s in systems)), int(max(len(s["Zs"]) for s in systems))],
            "grid_points": job.npts,
            "pixel_z": job.units,
            "scan_per_molecule": list(job.pl.systems[0]["scan_shape"]),
            "fire": relax,
            "tuning": {"ctas_per_sm": job.tuning[0], "tile": [job.tuning[1], job.tuning[2]], "chunk": job.tuning[3]},
            "l2": "inputs larger than L2 (force fields %.2f GB)" % (job.npts * 16 / 1e9),
            "parallelism": f"replicas x{world}",
        },
        "plain_gpu_loop": {"ms_per_step": plain, "value": job.units / (plain * 1e-3), "speedup_of_batched": plain / (1e3 * t_step_max / K), "clocks": job.plain_clocks},
        "learned_warm_start": learned,
        "fire_iters_per_pixel_z": iters / job.units,
        "e2e": {"value": job.units * world * K / t_e2e_max, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": job.launches_per_step * K,
        "roofline": {
            "bound": "fp32",
            "kernel": "batch_kernel (force-field phase + relaxation phase, one launch)",
            "achieved": flops / (t_step_max / K) / 1e12,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": flops / (t_step_max / K) / 1e12 / peak if peak else None,
            "peak_source": "FFMA microbenchmark measured in this run; achieved counts only the force-field flops over the whole step",
            "flops_per_launch": flops,
            "traffic": read_profile_traffic("batch_kernel", "molecule_batch") if (args.nmol, args.scale) == (256, 1.0) else None,
        },
        "cpu_baseline": None,
        "clocks": clk,
        "wall_s": wall,
    }
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_batch_sample(systems, args.cpu_budget)
    if world > 1:
        torch.distributed.destroy_process_group()
    return line


def run_ours(args, rank, world, local):
    import torch

    from ppafm_gb300 import HighLevel as HL
    from ppafm_gb300 import _lib

    torch.cuda.set_device(local)
    L = _lib.load()
    if args.relax_tps:
        _lib.check(L.ppgpu_set_relax_tps(args.relax_tps))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = make_workload(args.workload, args.seed + rank, args.scale)
    relax = dict(maxIters=w["maxIters"], convF2=w["convF2"], dt=w["dt"], damping=w["damping"])
    job = (OverlapJob if args.workload == "density_overlap" else PointChargeJob)(w, relax, HL, torch)
    pl = job.pl
    nx, ny, nz = pl.scan_shape
    units = nx * ny * nz
    npts = job.npts
    st = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---------------- device-resident steps, pipelined: step k+1's force field runs while step
    # k's relaxation finishes (force-field grids and output sets in flight,
    # HighLevel.StepPipeline).  A force field that fits in L2 is flushed from it before every
    # timed step's relaxation: 256 MB written on the relaxation stream once the step's force
    # field is done, so the relaxation reads its grid from DRAM, not from the L2 lines its
    # producer left.
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda") if npts * 16 < 129e6 else None
    NSLOT = 3  # grids, device output sets and pinned host slots in flight
    sp = HL.StepPipeline(pl, nbuf=NSLOT)
    flush_l2 = (lambda: flush.zero_()) if flush is not None else None

    def device_step(timing=None):
        return sp.step(timing=timing, before_relax=flush_l2)

    for _ in range(args.warmup):
        device_step()
    sp.wait_idle()
    torch.cuda.synchronize()
    pl.counter.zero_()
    timing = []
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    ev_a = torch.cuda.Event(enable_timing=True)
    ev_b = torch.cuda.Event(enable_timing=True)
    ev_a.record(st)
    sp.start_after(ev_a)
    for _ in range(args.steps):
        device_step(timing)
    sp.wait_idle(st)
    ev_b.record(st)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    t_ff = [e[0].elapsed_time(e[1]) * 1e-3 for e in timing]
    t_rx = [e[2].elapsed_time(e[3]) * 1e-3 for e in timing]
    t_step = ev_a.elapsed_time(ev_b) * 1e-3
    iters_total = int(pl.counter.item())
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))

    # ---------------- end to end through the host API.  Every step copies its own inputs in
    # and its outputs out, through pinned slot k % NSLOT, on two more streams: the inputs of step
    # k go in once step k-1's force field has read its inputs, the outputs of step k come out
    # once its relaxation is done (step k+NSLOT's relaxation, which writes the same device
    # output set, waits for that copy); the host prepares step k while the GPU works and waits
    # only for step k-NSLOT's outputs before reusing their pinned slot.  Force fields and
    # relaxations are pipelined as above.
    out0 = sp.outs[0]
    pin_out = [{k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in out0.items()} for _ in range(NSLOT)]
    job.pinned_slots(NSLOT)
    cs = torch.cuda.Stream()  # host -> device
    ds = torch.cuda.Stream()  # device -> host
    done = [None] * NSLOT
    last = {"ff": None}
    h2d = [0]
    kstep = [0]

    def e2e_step():
        slot = kstep[0] % NSLOT
        if done[slot] is not None:
            done[slot].synchronize()
        h2d[0] = job.e2e_host(slot)
        with torch.cuda.stream(cs):
            if last["ff"] is not None:
                cs.wait_event(last["ff"])
            job.e2e_h2d(slot)
            inputs_in = torch.cuda.Event()
            inputs_in.record(cs)
        j, out, ff_done, rx_done = sp.step(after=inputs_in, before_relax=flush_l2)
        last["ff"] = ff_done
        with torch.cuda.stream(ds):
            ds.wait_event(rx_done)
            for k, v in out.items():
                pin_out[slot][k].copy_(v, non_blocking=True)
            done[slot] = torch.cuda.Event()
            done[slot].record(ds)
        sp.release(j, done[slot])
        kstep[0] += 1

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    sp.start_after(a)
    cs.wait_event(a)
    ds.wait_event(a)
    for _ in range(args.steps):
        e2e_step()
    sp.wait_idle(st)
    st.wait_stream(ds)  # the last outputs are on the host before the interval ends
    b.record(st)
    b.synchronize()
    barrier()
    t_e2e = a.elapsed_time(b) * 1e-3
    d2h = int(sum(v.numel() * v.element_size() for v in pin_out[0].values()))

    # ---------------- max over ranks
    from ppafm_gb300.ranks import max_over_ranks

    t_step_max, t_e2e_max = max_over_ranks([t_step, t_e2e], device="cuda")
    K = args.steps
    value = units * world * K / t_step_max
    e2e_value = units * world * K / t_e2e_max

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return None

    # ---------------- roofline of the dominant kernel
    t_ff_avg = float(np.mean(t_ff))
    t_rx_avg = float(np.mean(t_rx))
    if t_ff_avg >= t_rx_avg and job.ff_roofline(t_ff_avg, 1.0) is not None:
        peak = ffma_peak_tflops(torch, L, _lib.check, _lib.tptr, _lib.stream_handle)
        roof = job.ff_roofline(t_ff_avg, peak)
        roof["traffic"] = read_profile_traffic("ff_kernel", args.workload)
    else:
        # relaxation: gathers of 8 float4 corners per FIRE iteration + 32 B out per pixel-z
        peaks = read_measured_peaks()
        hbm = peaks.get("hbm_gbs")
        moved = 128.0 * iters_total / K + 32.0 * units
        achieved = moved / t_rx_avg / 1e9
        roof = {"bound": "hbm", "kernel": "relax_kernel<scan> (FIRE + fused df)", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if hbm else None, "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm else "fallback 6800 GB/s", "bytes_per_launch": moved, "traffic": read_profile_traffic("relax_kernel", args.workload)}
        if not hbm:
            roof["peak"] = 6800.0
            roof["frac"] = achieved / 6800.0

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            from oracle import cpu_baseline

            s = cpu_baseline.sample_pipeline(w, budget_s=args.cpu_budget)
            cpu = {"value": s["pixel_z_per_s"], "unit": UNIT, "cores": s["cores"], "cpu_model": s.get("cpu_model"), "kind": s["kind"], "sample": s["sample"], "seconds_full_job": s["seconds_full_job"]}
            if "ff_pairs_per_s" in s:
                cpu["ff_grid_pt_atoms_per_s"] = s["ff_pairs_per_s"]
        except Exception as e:  # the baseline is reported, never fatal
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}

    config = {"workload": args.workload}
    config.update(job.config())
    config.update(
        {
            "grid": list(pl.gridN),
            "scan": [nx, ny, nz],
            "fire": relax,
            "probe": {"klat": w["klat"], "krad": w["krad"], "r0": list(w["r0Probe"]), "Q": w["charge"]},
            "df": {"f0": w["f0Cantilever"], "k": w["kCantilever"], "A": w["Amplitude"]},
            "l2": ("inputs larger than L2 (force field %.2f GB)" if npts * 16 >= 129e6 else "force field %.2f GB fits in L2: 256 MB written before every step's relaxation (after its force field) to flush it") % (npts * 16 / 1e9),
            "relax_lanes_per_stroke": args.relax_tps or 1,
            "steps": "pipelined: step k+1's force field runs while step k's relaxation finishes (three force-field grids and output sets in flight, relaxations on a higher-priority stream); stage_ms are each kernel's own event-timed duration on its stream",
            "parallelism": f"replicas x{world}",
        }
    )
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_step_max / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": config,
    }
    line.update(job.extra(t_ff_avg))
    line.update(
        {
            "fire_iters_per_pixel_z": iters_total / (units * K),
            "stage_ms": {"force_field": 1e3 * t_ff_avg, "relax_and_df": 1e3 * t_rx_avg},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d[0], "d2h_bytes_per_step": d2h},
            "gpu_launches": job.launches_per_step * K,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
            "wall_s": wall,
        }
    )
    if world > 1:
        torch.distributed.destroy_process_group()
    return line


def run_reference(args, rank, world):
    if rank != 0:
        return None
    if args.workload == "afmulator":
        return {"impl": "reference", "unavailable": "the reference's AFMulator runs on OpenCL, which has no runtime here; the afmulator line's cpu_baseline times the C restatement of its kernels instead"}
    from oracle import cpu_baseline

    if args.workload == "molecule_batch":
        from ppafm_gb300 import workloads

        systems = workloads.molecule_batch(seed=args.seed, nmol=args.nmol, scale=args.scale)
        vals = [cpu_batch_sample(systems, args.cpu_budget / 2, seed=i) for i in range(args.warmup + args.steps)][args.warmup :]
        v = float(np.median([x["value"] for x in vals]))
        from ppafm_gb300 import common as C

        units = 0
        for m in systems:
            xT, yT, zT, _ = C.prepareScanGrids(m["scanMin"], m["scanMax"], m["scanStep"], m["r0Probe"])
            units += len(xT) * len(yT) * len(zT)
        return {
            "impl": "reference",
            "metric": METRIC,
            "value": v,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1e3 * units / v,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": "molecule_batch", "molecules": len(systems), "parallelism": "host cores"},
            "cpu_baseline": dict(vals[-1], value=v),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
    w = make_workload(args.workload, args.seed, args.scale)
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        s = cpu_baseline.sample_pipeline(w, budget_s=args.cpu_budget / 2, seed=i)
        if i >= args.warmup:
            vals.append(s["pixel_z_per_s"])
            info = s
    v = float(np.median(vals))
    from ppafm_gb300 import common as C

    xT, yT, zT, _ = C.prepareScanGrids(w["scanMin"], w["scanMax"], w["scanStep"], w["r0Probe"])
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * len(xT) * len(yT) * len(zT) / v,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "grid": list(w["gridN"]), "scan": [len(xT), len(yT), len(zT)], "parallelism": "host cores"},
        "ff_grid_pt_atoms_per_s": info["ff_pairs_per_s"],
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"], "cpu_model": info.get("cpu_model"), "kind": info["kind"], "sample": info["sample"], "seconds_full_job": info["seconds_full_job"]},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_afmulator(args, rank, world, local):
    """The AFMulator's point-charge route the way the ML generators drive it: for each molecule
    of a seeded set (the first args.nmol // 4 molecules of the batch workload), the scan window
    follows the molecule, its force field (LJ + four tip charges) is made on a grid around the
    window and the tilted-stroke relaxation + z convolution writes its image into one device
    buffer; the images go to the host once per step (GeneratorAFMtrainer, sim_type LJ+PC).
    A step is one batch.  The inputs are host molecules by design (the generator packs every
    molecule's atoms), so the step is end to end; value and e2e are that one measurement.  The
    two kernels' durations come from a second pass that brackets each image's launches with
    CUDA events.  The generator runs the AFMulator in its overlap mode (each image's force field
    beside the previous image's relaxation)."""
    import torch

    from ppafm_gb300 import _lib, workloads
    from ppafm_gb300.AFMulator import AFMulator
    from ppafm_gb300.ml.Generator import GeneratorAFMtrainer

    torch.cuda.set_device(local)
    L = _lib.load()
    nmol = max(1, args.nmol // 4)
    mols = workloads.molecule_batch(seed=args.seed + rank, nmol=nmol, scale=args.scale)
    samples = [{"xyzs": np.asarray(m["Rs"], np.float64), "Zs": np.asarray(m["Zs"]), "qs": np.asarray(m["Qs"], np.float64)} for m in mols]
    kw = dict(pixPerAngstrome=10, scan_dim=(128, 128, 30), scan_window=((0.0, 0.0, 7.0), (16.0, 16.0, 10.0)), df_steps=10)
    afm = AFMulator(**kw)
    seen = []
    record = [False]

    class Trainer(GeneratorAFMtrainer):
        def on_afm_start(self):
            if record[0]:
                d = self.sample_dict
                seen.append((self.scan_window, d["xyzs"], d["Zs"], d["qs"], d["REAs"]))

    tr = Trainer(afm, [], samples, sim_type="LJ+PC", batch_size=nmol, iZPPs=[8], Qs=[[-10, 20, -10, 0]], QZs=[[0.1, 0, -0.1, 0]])
    for _ in range(args.warmup):
        for _ in tr:
            pass
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    clocks = ClockSampler(local)
    clocks.start()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record(st)
    for _ in range(args.steps):
        for _ in tr:
            pass
    b.record(st)
    b.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    t_step = a.elapsed_time(b) * 1e-3 / args.steps
    nx, ny, nz = kw["scan_dim"]
    units = nmol * nx * ny * nz
    # kernel pass: each image's force field and relaxation bracketed by events (in the
    # AFMulator's plain mode: one stream, so the events bracket the two kernels)
    record[0] = True
    for _ in tr:
        pass
    afm.set_overlap(False)
    torch.cuda.synchronize()
    out = torch.empty((nx, ny, nz - kw["df_steps"] + 1), dtype=torch.float32, device="cuda")

    def images(timing=None):
        for sw, xyzs, Zs, qs, REAs in seen:
            afm.setScanWindow(sw, kw["scan_dim"], df_steps=kw["df_steps"])
            afm.setLvec()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)] if timing is not None else None
            if e:
                e[0].record(st)
            afm.prepareFF(xyzs, Zs, qs, REAs=REAs)
            if e:
                e[1].record(st)
            afm.evalAFM(out=out)
            if e:
                e[2].record(st)
                timing.append(e)

    ev = []
    images(ev)
    torch.cuda.synchronize()
    t_ff = float(np.mean([e[0].elapsed_time(e[1]) for e in ev])) * 1e-3
    t_rx = float(np.mean([e[1].elapsed_time(e[2]) for e in ev])) * 1e-3
    afm.counter.zero_()
    images()
    iters = int(afm.counter.item())
    _lib.check(L.ppgpu_device_status(_lib.stream_handle()))
    npts = int(np.prod(afm.nDim))
    # the dominant kernel is the force field (ff_kernel<QZS>, FP32-FMA bound).  Work per
    # atom-point pair in FF.cl's form (FMA = 2): LJ 26 flops, each nonzero tip charge 20
    # (offset 1, r^2 5, R2SAFE 1, 1/r^2 1, energy 2, force factor 1, charge weight 3,
    # accumulation 6): 86 for the three-charge tip
    nq = int(np.count_nonzero(afm.Qs))
    flops = float(np.mean([npts * len(z) for _, _, z, _, _ in seen])) * (FLOPS_LJ_PAIR + FLOPS_TIP_CHARGE_PAIR * nq)
    peak = ffma_peak_tflops(torch, L, _lib.check, _lib.tptr, _lib.stream_handle)
    achieved = flops / t_ff / 1e12
    roof = {"bound": "fp32", "kernel": "ff_kernel<QZS> (LJ + point-charge tip force field)", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None, "peak_source": "FFMA microbenchmark measured in this run (MEASURED_PEAKS.json has no FP32 figure)", "flops_per_launch": flops, "flops_per_pair": FLOPS_LJ_PAIR + FLOPS_TIP_CHARGE_PAIR * nq, "traffic": read_profile_traffic("ff_kernel", "afmulator")}
    if rank != 0:
        return None
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            from oracle import oracle as O
            from ppafm_gb300 import species

            FFp = np.array([(r[0], r[1], r[2]) for r in species.loadSpecies()])
            nthreads = os.cpu_count() or 1
            picks = seen[: max(1, min(4, len(seen)))]
            t0c = time.perf_counter()
            for sw, xyzs, Zs, qs, REAs in picks:
                O.AFMulator(FFp, **{**kw, "scan_window": sw}).eval(xyzs, Zs, qs, REAs=REAs, nthreads=nthreads)
            tc = (time.perf_counter() - t0c) / len(picks)
            from oracle.cpu_baseline import cpu_model

            cpu = {"value": nx * ny * nz / tc, "unit": UNIT, "cores": nthreads, "cpu_model": cpu_model(), "kind": "port", "sample": f"{len(picks)} of {len(seen)} molecules through the oracle's float32 C restatement of the OpenCL kernels (evalLJC_QZs_noPos, relaxStrokesTilted, convolveZ), OpenMP over grid points and pixels; the reference's own path is OpenCL, which does not run here"}
        except Exception as exc:  # the baseline is reported, never fatal
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {exc}"}
    return {
        "metric": METRIC,
        "value": units / t_step,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "afmulator", "molecules": nmol, "scan": list(kw["scan_dim"]), "force_field_grid": [int(x) for x in afm.nDim], "route": "LJ + point-charge tip (Qs -10, 20, -10 e at QZ 0.1, 0, -0.1 A)", "df_steps": kw["df_steps"], "l2": "every image has its own force field (%.0f MB) and scan window" % (npts * 16 / 1e6), "parallelism": f"replicas x{world}"},
        "images_per_s": nmol / t_step,
        "stage_ms": {"force_field": 1e3 * t_ff, "relax_and_df": 1e3 * t_rx},
        "fire_iters_per_pixel_z": iters / units,
        "e2e": {"value": units / t_step, "unit": UNIT, "h2d_bytes_per_step": int(sum(len(s["Zs"]) * 48 for s in samples)), "d2h_bytes_per_step": int(nmol * nx * ny * (nz - kw["df_steps"] + 1) * 4)},
        "gpu_launches": 2 * nmol * args.steps,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
        "wall_s": wall,
    }


def extra_batch(args, rank, world, local):
    """The 256-molecule batch measured in the default run (its own line's main figures): the
    batched persistent launch, the plain per-molecule loop and the learned warm start, each
    timed with CUDA events and with the clocks sampled meanwhile."""
    import copy

    a = copy.copy(args)
    a.workload = "molecule_batch"
    a.steps = EXTRA_BATCH_STEPS
    a.warmup = max(3, min(args.warmup, 3))
    a.cpu_budget = args.cpu_budget / 2
    line = run_batch(a, rank, world, local)
    if line is None:
        return None
    keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "e2e", "fire_iters_per_pixel_z", "plain_gpu_loop", "learned_warm_start", "clocks", "cpu_baseline", "gpu_launches")
    out = {k: line[k] for k in keep if k in line}
    out["config"] = line["config"]
    out["roofline"] = {k: line["roofline"][k] for k in ("kernel", "achieved", "peak", "unit", "frac")}
    return out


# Timed steps of the single-system extras: enough for the timed region to span many clock samples
# (a step of these workloads takes 2-4 ms; an AFMulator step is one batch of 64 images).
EXTRA_STEPS = {"small_molecule": 400, "density_overlap": 300, "afmulator": 5}
# Timed steps of the 256-molecule batch in the default run (~0.22 s each): its end-to-end loop
# starts from an idle GPU, so the first step's host preparation and the last step's output copy
# fall inside the timed region; ten steps keep them a small part of it.
EXTRA_BATCH_STEPS = 10


def extra_single(args, rank, world, local, workload):
    """A single-system workload measured in the default run with its own CUDA-event timing,
    clock samples, roofline and a shorter CPU-baseline sample: the small molecule (config 0),
    the density-overlap FFT route (config 3) and the AFMulator."""
    import copy

    a = copy.copy(args)
    a.workload = workload
    a.steps = EXTRA_STEPS[workload]
    a.warmup = 3
    a.cpu_budget = args.cpu_budget / 4
    line = (run_afmulator if workload == "afmulator" else run_ours)(a, rank, world, local)
    if line is None:
        return None
    keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "e2e", "stage_ms", "images_per_s", "fire_iters_per_pixel_z", "clocks", "cpu_baseline", "gpu_launches", "config")
    out = {k: line[k] for k in keep if k in line}
    out["roofline"] = {k: line["roofline"][k] for k in ("kernel", "bound", "achieved", "peak", "unit", "frac", "traffic") if k in line["roofline"]}
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "molecule_batch":
        line = run_batch(args, rank, world, local)
    elif args.workload == "afmulator":
        line = run_afmulator(args, rank, world, local)
    else:
        line = run_ours(args, rank, world, local)
        if line is not None and args.workload == "slab_molecule" and world == 1 and not args.no_extras:
            extras = {"molecule_batch": extra_batch(args, rank, world, local)}
            for wl in ("small_molecule", "density_overlap", "afmulator"):
                extras[wl] = extra_single(args, rank, world, local, wl)
            line["extra_workloads"] = extras
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
