"""Many systems in one persistent launch, and the autotuner of its launch shape.

The reference's batched caller, ``ml/Generator.py:68-144``, loops over molecules and runs
the simulator once per molecule.  ``BatchPipeline`` runs the same work -- per system the
Lennard-Jones + point-charge force field (FF = FFLJ + Q*FFel with the clamp, fused), the
relaxed scan and Δf -- for a whole batch as one persistent kernel over a packed work list
(``ppgpu_batch_run``), optionally replayed from a CUDA graph.

The launch shape (CTAs per SM, the pixel-tile shape that orders the strokes, strokes per
warp chunk) is chosen by ``autotune``: it times every candidate on the batch itself and
caches the winner per GPU and batch signature in ``_lib/autotune.json``.
"""

import ctypes
import hashlib
import json
import os
import time

import numpy as np
import torch

from . import common as PPU
from ._lib import LIB_PATH, BatchJob, check, lib, stream_handle
from .device import pack_atoms
from .HighLevel import Fmax_DEFAULT, _get, prepare_atoms, tip_vector

DEFAULT_TUNING = (2, 8, 4, 64)
CANDIDATES = [(c, tw, th, ch) for c in (1, 2) for (tw, th) in ((32, 1), (8, 4), (4, 8), (16, 2)) for ch in (32, 64, 128)]
TUNING_CACHE = os.path.join(os.path.dirname(LIB_PATH), "autotune.json")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class BatchPipeline:
    """A batch of systems: each a dict with Zs, Rs, Qs, lvec (orthogonal cell), gridN and
    its scan (scanMin, scanMax, scanStep).  Probe, FIRE and Δf settings come from
    ``parameters`` (shared by the batch).  Buffers stay in device memory; ``run()`` is one
    launch (plus a counter reset), ``capture()`` records it in a CUDA graph.
    out_sets > 1 keeps that many sets of output buffers (``systems[j]["outs"][slot]``), each
    with its own launch handle and graph (``run(slot=...)``, ``replay(slot)``,
    ``outputs(j, slot)``), so one set can be copied to the host while the next run writes
    another; force fields and atom records are shared."""

    def __init__(self, systems, parameters, relax=None, with_df=True, want_ppos=True, want_iters=False, tuning=None, FFparams=None, device="cuda", out_sets=1):
        self.p = parameters
        self.device = device
        self.Q = float(_get(parameters, "charge", 0.0))
        self.prm = tip_vector(parameters, relax)
        self.tuning = tuple(tuning) if tuning is not None else DEFAULT_TUNING
        dz = _get(parameters, "scanStep")[2]
        self.W = None
        if with_df:
            units = 16.0217656
            W = PPU.get_df_weight(_get(parameters, "Amplitude", 1.0), dz=dz)
            self.W = np.ascontiguousarray(W * units * _get(parameters, "f0Cantilever") / _get(parameters, "kCantilever"), dtype=np.float64)
        self.systems = []
        self._keep = []
        jobs = (BatchJob * len(systems))()
        for j, w in enumerate(systems):
            lvec = np.asarray(w["lvec"], dtype=np.float64)
            n = tuple(int(x) for x in w["gridN"])
            Rs0, cLJs, kqq = prepare_atoms(w["Zs"], w["Rs"], w["Qs"], lvec, parameters, FFparams)
            rec, natoms, nch = pack_atoms(Rs0, cLJs, kqq if self.Q != 0.0 else None, device=device)
            FE = torch.empty(int(np.prod(n)) * 4, dtype=torch.float32, device=device)
            scan = w if "scanMin" in w else parameters
            xT, yT, zT, lvecScan = PPU.prepareScanGrids(_get(scan, "scanMin"), _get(scan, "scanMax"), _get(scan, "scanStep"), _get(parameters, "r0Probe"))
            if abs(_get(scan, "scanStep")[2] - dz) > 1e-12 and self.W is not None:
                raise ValueError("systems of one batch share the z step (the df weights)")
            xs = np.ascontiguousarray(xT - lvec[0, 0])
            ys = np.ascontiguousarray(yT - lvec[0, 1])
            zs = np.ascontiguousarray(zT[::-1] - lvec[0, 2])
            nx, ny, nz = len(xs), len(ys), len(zs)

            def new_out():
                o = {"fzs": torch.empty((nx, ny, nz), dtype=torch.float32, device=device)}
                if want_ppos:
                    o["ppos"] = torch.empty((nx, ny, nz, 3), dtype=torch.float32, device=device)
                if want_iters:
                    o["iters"] = torch.empty((nx, ny, nz), dtype=torch.int32, device=device)
                if self.W is not None:
                    o["df"] = torch.empty((nx, ny, nz - len(self.W) + 1), dtype=torch.float32, device=device)
                return o

            outs = [new_out() for _ in range(max(1, int(out_sets)))]
            out = outs[0]
            J = jobs[j]
            J.FE = FE.data_ptr()
            J.atoms = rec.data_ptr()
            J.natoms = natoms
            J.ncharged = nch
            for k in range(3):
                J.n[k] = n[k]
                J.pos_offset[k] = lvec[0, k]
            cell = np.ascontiguousarray(lvec[1:4]).reshape(-1)
            for k in range(9):
                J.cell[k] = cell[k]
            J.nx, J.ny, J.nz = nx, ny, nz
            J.xs, J.ys, J.zs = _dp(xs), _dp(ys), _dp(zs)
            J.fzs = out["fzs"].data_ptr()
            J.ppos = out["ppos"].data_ptr() if "ppos" in out else None
            J.df = out["df"].data_ptr() if "df" in out else None
            J.iters = out["iters"].data_ptr() if "iters" in out else None
            self._keep += [xs, ys, zs, rec]
            self.systems.append(dict(FE=FE, rec=rec, n=n, lvec=lvec, natoms=natoms, ncharged=nch, out=out, outs=outs, scan_shape=(nx, ny, nz), lvecScan=lvecScan))
        self._jobs = [jobs]
        for slot in range(1, len(self.systems[0]["outs"]) if self.systems else 1):
            js = (BatchJob * len(systems))()
            ctypes.memmove(js, jobs, ctypes.sizeof(jobs))
            for j, sysd in enumerate(self.systems):
                o = sysd["outs"][slot]
                js[j].fzs = o["fzs"].data_ptr()
                js[j].ppos = o["ppos"].data_ptr() if "ppos" in o else None
                js[j].df = o["df"].data_ptr() if "df" in o else None
                js[j].iters = o["iters"].data_ptr() if "iters" in o else None
            self._jobs.append(js)
        if torch.device(device).type == "cuda":
            torch.cuda.current_stream().synchronize()  # the atom records are on the device before any stream runs
        tun = np.ascontiguousarray(self.tuning, dtype=np.int32)
        W = self.W if self.W is not None else np.zeros(1)
        self.handles = []
        for js in self._jobs:
            h = ctypes.c_void_p()
            self.handles.append(h)
            check(lib().ppgpu_batch_create(ctypes.cast(js, ctypes.c_void_p), len(systems), _dp(np.ascontiguousarray(self.prm, dtype=np.float64)), self.Q, Fmax_DEFAULT, 0 if self.W is None else len(self.W), _dp(W), tun.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.byref(h)))
        self.handle = self.handles[0]
        info = (ctypes.c_longlong * 4)()
        check(lib().ppgpu_batch_info(self.handle, info))
        self.ff_items, self.strokes, self.ctas, _ = list(info)
        self.graphs = [None] * len(self.handles)
        self.graph = None

    # --------------------------------------------------------------- running
    def run(self, stream=None, slot=0):
        check(lib().ppgpu_batch_run(self.handles[slot], stream_handle(stream)))

    def run_layered(self, net=None, record=None, stream=None):
        """Height-synchronous run: with a WarmStartNet the learned warm start, without it plain
        FIRE (same results as run()).  record = (stride, X, T) stores training pairs."""
        mlp = net.handle if net is not None else None
        stride, X, T = record if record is not None else (0, None, None)
        check(lib().ppgpu_batch_run_layered(self.handle, mlp, int(stride), None if X is None else ctypes.c_void_p(X.data_ptr()), None if T is None else ctypes.c_void_p(T.data_ptr()), stream_handle(stream)))

    def capture(self, fn=None):
        """Records one run (or fn(), e.g. lambda: self.run_layered(net)) in a CUDA graph;
        replay() launches it.  Without fn, every output set gets its graph (replay(slot))."""
        if fn is None:
            for slot in range(len(self.handles)):
                self.graphs[slot] = self._capture(lambda: self.run(slot=slot))
            self.graph = self.graphs[0]
            return self.graph
        self.graph = self._capture(fn)
        self.graphs[0] = self.graph
        return self.graph

    def _capture(self, fn):
        torch.cuda.synchronize()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            fn()  # warm-up outside the capture (lazy module loading, first-use buffers)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            fn()
        return graph

    def replay(self, slot=0):
        if self.graphs[slot] is None:
            self.capture()
        self.graphs[slot].replay()

    def iterations(self):
        v = ctypes.c_ulonglong(0)
        check(lib().ppgpu_batch_iterations(self.handle, ctypes.byref(v), stream_handle()))
        return int(v.value)

    @property
    def pixel_z(self):
        return int(sum(np.prod(s["scan_shape"]) for s in self.systems))

    def outputs(self, j, slot=0):
        return self.systems[j]["outs"][slot]

    def close(self):
        for h in getattr(self, "handles", []):
            if h is not None and h.value:
                lib().ppgpu_batch_destroy(h)
        self.handles = []
        self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ autotuner


def _signature(systems):
    h = hashlib.sha1()
    for w in systems:
        h.update(np.asarray(w["gridN"], dtype=np.int64).tobytes())
        h.update(np.int64(len(w["Zs"])).tobytes())
        for k in ("scanMin", "scanMax", "scanStep"):
            if k in w:
                h.update(np.asarray(w[k], dtype=np.float64).tobytes())
    return f"{len(systems)}:{h.hexdigest()[:16]}"


def _load_cache():
    try:
        with open(TUNING_CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time_pipeline(pl, reps):
    pl.run()  # warm-up
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(reps):
        a.record()
        pl.run()
        b.record()
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def autotune(systems, parameters, relax=None, candidates=None, reps=2, use_cache=True, verbose=False):
    """Times every candidate (CTAs per SM, tile width, tile height, chunk) on this batch and
    returns (best tuning, {tuning: ms}).  Results are cached per GPU and batch signature."""
    key = f"{torch.cuda.get_device_name()}|{_signature(systems)}"
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        return tuple(cache[key]["best"]), {tuple(json.loads(k)): v for k, v in cache[key]["ms"].items()}
    cands = list(candidates or CANDIDATES)
    times = {}
    for c in cands:
        pl = BatchPipeline(systems, parameters, relax=relax, want_ppos=False, tuning=c)
        times[tuple(c)] = _time_pipeline(pl, reps)
        pl.close()
        if verbose:
            print("autotune", c, "%.3f ms" % times[tuple(c)], flush=True)
    best = min(times, key=times.get)
    if use_cache:
        cache = _load_cache()
        cache[key] = {"best": list(best), "ms": {json.dumps(list(k)): v for k, v in times.items()}, "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        try:
            with open(TUNING_CACHE, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return best, times


def plain_loop(systems, parameters, relax=None):
    """The same work one system at a time through HighLevel.Pipeline (the plain GPU form the
    batched launch is measured against).  Returns the list of pipelines (built, not run)."""
    from .HighLevel import Pipeline

    out = []
    for w in systems:
        params = dict(parameters)
        for k in ("scanMin", "scanMax", "scanStep"):
            if k in w:
                params[k] = w[k]
        out.append(Pipeline(w["Zs"], w["Rs"], w["Qs"], w["lvec"], w["gridN"], params, relax=relax, want_ppos=False))
    return out
