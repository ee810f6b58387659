"""Benchmark of the GB300 lattice Boltzmann time step.

Workload (one GPU): a batch of seeded 1024x1024 pore images of the multi-block
configuration (disk radii U[6,40], porosity U[0.5,0.7], 3-level quadtree,
Kn U[0.01,1]); the batch is sized so that its state is larger than L2.
A bench step is one coarse time step of every image of the batch.

  value     MLUPS over the batch, device-timed with CUDA events around K steps
            replayed from CUDA graphs (state resident in HBM)
  e2e       MLUPS through the public C ABI with pinned host buffers: per image
            (two host threads, each context on its own stream) the equilibrium
            state is uploaded (mgpu_set_equilibrium), K steps run with the
            reference's per-step residual and break test (mgpu_run), and the
            per-cell fields are read back (mgpu_download_cells); the median of 5
            such runs
  roofline  the finest-level step kernel: 72 B per lattice update (9 FP32
            populations read + 9 written) over its CUDA-event launch time;
            batch_achieved / batch_frac: the same 72 B per update at the
            batch's own rate (value)
  timing    the K-step window is timed repeatedly until the windows cover
            --min-seconds (at least 3); value is the median window
  steady_state  config2_steady images (1024^2, two levels, on which the
            reference's scheme has a steady state), each run from rest to a
            relative permeability change below 1e-6 over 1000 steps: steps,
            GPU seconds, permeability
  steady_batch  (--steady-batch N) N config4_steady images as one batch to
            the same criterion
  config3   the adsorption step of config 3 (512^2 Shan-Chen image), MLUPS
            over --adsorption-steps steps (the --adsorption run's line)
  cpu_baseline  the FP64 CPU oracle (a restatement of the reference's step)
            on the host cores, on a bounded sample of the same workload, with
            all threads and with one

--impl reference times that CPU implementation alone, as the reference arm.
--properties N times the pore-property pipeline (skeleton, distance transforms,
local pore size, Kn) on one seeded N x N disk image instead: the GPU kernels
through mgpu_pore_properties_gpu (host buffers in and out) against the host
code of mgpu_pore_properties, and checks that both agree bit for bit.
Multi-GPU (torchrun): every rank runs its own batch (weak scaling, no
collective on the data path).
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_LU = 72.0
# host threads of the end-to-end leg, each stepping its share of the images in
# turn: two large images in flight at once share the L2 best (config 2, 1 / 2 / 4
# threads: 9.2 / 8.9 / 8.4 k MLUPS; single-block 1024^2: 13.7 / 16.9 / 12.0 k)
E2E_THREADS = 2
E2E_REPEATS = 5
WORKLOAD = "config2: 1024x1024 seeded disk images (r U[6,40], porosity U[0.5,0.7]), 3-level quadtree, Kn U[0.01,1]"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._th = None

    def start(self):
        # one nvidia-smi in loop mode (a sample every 25 ms), read line by line
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "25"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return

        def run():
            for line in self._proc.stdout:
                if self._stop.is_set():
                    break
                line = line.strip()
                if line:
                    self.rows.append([v.strip() for v in line.split(",")])

        self._th = threading.Thread(target=run, daemon=True)
        self._th.start()
        time.sleep(0.3)  # nvidia-smi is up and sampling before the timed region starts
        self.rows.clear()

    def stop(self):
        self._stop.set()
        if getattr(self, "_proc", None) is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._th:
            self._th.join(timeout=10)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 2 + i and "Active" in r[2 + i]
                          and "Not" not in r[2 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


WORKLOADS = {
    "config2": WORKLOAD,
    "single1024": "1024x1024 seeded disk images (r U[6,40], porosity 0.6), single block, Kn 0.1",
    "config4": "config4: seeded disk images of side {128..2048}, porosity U[0.45,0.75], 1-3 levels, "
               "log-uniform Kn in [0.01, 2], stepped together (uneven sizes and depths)",
}


def lpt_partition(costs, world):
    """Greedy longest-processing-time split of independent images over ranks:
    the costliest image first, each to the rank with the least work so far
    (the lowest rank on ties).  Returns each rank's image indices, ascending."""
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def rank_images(count, rank, world, workload="config2"):
    """This rank's images.  Equal-cost workloads: rank r takes images
    r*count .. r*count+count-1; config 4 (sides 128-2048): the count*world
    images are split by the greedy LPT rule on their pixel counts, so that the
    slowest rank, which sets the job's time, has as little as possible."""
    if workload != "config4" or world == 1:
        return make_images(count, rank * count, workload)
    from mantiis_gb300 import workloads

    costs = [float(workloads.config4_side(i)) ** 2 for i in range(count * world)]
    mine = lpt_partition(costs, world)[rank]
    return [workloads.config4(i) for i in mine]


def make_images(count, offset, workload="config2"):
    from mantiis_gb300 import workloads

    if workload == "single1024":
        return [dict(workloads.image(1024, 6, 40, 0.6, 0.1, 5000 + offset + i), levels=1) for i in range(count)]
    if workload == "config4":
        return [workloads.config4(offset + i) for i in range(count)]
    return [dict(workloads.config2(offset + i), levels=3) for i in range(count)]


def params_for(img, plain_path=-1):
    from mantiis_gb300 import default_params

    if img.get("levels", 3) == 1:
        return default_params(multiblock=0, dx=img["dx"], plain_path=plain_path)
    return default_params(multiblock=1, max_allowed_level=img["levels"], dx=img["dx"], edge_fine=1,
                          plain_path=plain_path)


def oracle_grid(img):
    """Grid tables of a benchmark image from the oracle's own restatement of the
    reference's grid construction (oracle/grid_oracle.cpp): the CPU legs run no
    product code."""
    from oracle.pygrid import GridTables

    levels = img.get("levels", 3)
    return GridTables(img["pore"], img["kn"], img["locpore"], multiblock=levels > 1, max_allowed_level=levels,
                      edge_fine=levels > 1 and img.get("edge_fine", 1), dx=img["dx"])


def cpu_oracle_rate(grid, dx, seconds, threads):
    """MLUPS of the FP64 oracle on one image's grid, steps sized to ~`seconds`."""
    from oracle.pyoracle import for_grid

    lu = grid.lattice_updates()
    o = for_grid(grid, sim="transport", dx=dx, threads=threads)
    t0 = time.perf_counter()
    o.run(1)
    t1 = time.perf_counter()
    per = max(t1 - t0, 1e-6)
    steps = max(2, int(seconds / per))
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    return lu * steps / dt / 1e6, steps, dt, lu


def loaded_product_libraries():
    """Shared objects of this repository's package mapped into this process."""
    try:
        maps = Path("/proc/self/maps").read_text()
    except OSError:
        return None
    pkg = str(ROOT / "mantiis_gb300")
    return sorted({ln.split()[-1] for ln in maps.splitlines() if ln.split()[-1].startswith(pkg)})


def job_rate(lu_local, ms_local, steps, dist=None, device="cpu"):
    """Whole-job MLUPS over all ranks (weak scaling: every rank steps its own
    images): the lattice updates of all ranks over the slowest rank's time.
    Returns (MLUPS, max ms, lattice updates per step of the job)."""
    ms, lu = float(ms_local), float(lu_local)
    if dist:
        import torch

        t_ms = torch.tensor([ms], dtype=torch.float64, device=device)
        t_lu = torch.tensor([lu], dtype=torch.float64, device=device)
        dist.all_reduce(t_ms, op=dist.ReduceOp.MAX)
        dist.all_reduce(t_lu, op=dist.ReduceOp.SUM)
        ms, lu = float(t_ms.item()), float(t_lu.item())
    return lu * steps / (ms / 1e3) / 1e6, ms, lu


STEADY_WORKLOAD = ("config2_steady: 1024x1024 seeded disk images (r U[6,40], porosity U[0.5,0.7], void x edges), "
                   "2-level quadtree, Kn U[0.01,0.02]")


STEADY_BATCH_WORKLOAD = ("config4_steady: seeded disk images of side {128..2048} (r n/256..n/32, porosity "
                         "U[0.45,0.75], void x edges), 1-2 levels, log-uniform Kn in [0.01, 0.12] single block, "
                         "Kn U[0.01,0.02] x min(1024/n, 2) with two levels; all images in one batch")


def steady_batch_leg(count, stream, chunk=1000, tol=1e-6, max_steps=100000):
    """The config-4 set in its steady variant: `count` images of uneven size and
    depth stepped together as one batch until every image's permeability
    changes by less than `tol` (relative) over `chunk` steps; a settled image
    leaves the batch (the others go on in a batch of their own).  GPU time with
    CUDA events around the run."""
    import torch

    from mantiis_gb300 import Batch, workloads
    from mantiis_gb300.surrogate import make_solvers, run_batch_to_steady

    # the images and their contexts are made on all host cores (8x4 plain-cell
    # tiles fixed: surrogate.make_solvers)
    t_setup = time.perf_counter()
    imgs = workloads.generate(workloads.config4_steady, range(count))
    sol = make_solvers(imgs, concurrent=1)
    t_setup = time.perf_counter() - t_setup
    for s in sol:
        s.set_stream(stream.cuda_stream)
    b = Batch(sol)
    b.set_stream(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = {}
    steps, k = run_batch_to_steady(b, chunk=chunk, tol=tol, max_steps=max_steps, stats=stats)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    done = int(steps.max())
    lu = float(sum(s.info["lu_per_step"] for s in sol))
    out = {"workload": STEADY_BATCH_WORKLOAD, "images": count, "host_setup_seconds": t_setup,
           "criterion": f"relative permeability change below {tol:g} over {chunk} steps; a settled image "
                        f"leaves the batch",
           "settled": int((steps < max_steps).sum()), "coarse_steps": done, "gpu_seconds": ms / 1e3,
           "mlups": stats["lu"] / (ms / 1e3) / 1e6, "lu_done": stats["lu"], "batches": stats["batches"],
           "lu_if_all_stepped_to_the_end": lu * done, "lu_per_step": lu,
           "sides": [int(im["pore"].shape[0]) for im in imgs], "levels": [int(im["levels"]) for im in imgs],
           "steps_to_settle": [int(v) for v in steps], "permeability": [float(v) for v in k],
           "positive": int((np.asarray(k) > 0).sum()), "finite": bool(np.isfinite(k).all())}
    b.close()
    for s in sol:
        s.close()
    return out


def steady_state_leg(count, stream, chunk=500, tol=1e-6, max_steps=200000):
    """Images on which the reference's multi-block scheme has a steady state,
    each run from rest until its permeability changes by less than `tol`
    (relative) over 1000 steps, one after another: coarse steps, GPU time
    (CUDA events around every chunk of the run, checks included) and the
    permeability of each."""
    import torch

    from mantiis_gb300 import Solver, default_params, workloads

    out = []
    for i in range(count):
        img = workloads.config2_steady(i)
        p = default_params(multiblock=1, max_allowed_level=img["levels"], dx=img["dx"], edge_fine=1)
        s = Solver(img["pore"], img["kn"], img["locpore"], p)
        s.set_stream(stream.cuda_stream)
        hist, steps, ms = [s.observables()["permeability"]], 0, 0.0
        settled = False
        while steps < max_steps and not settled:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.advance_graph(chunk)
            k = s.observables()["permeability"]  # waits for the chunk
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
            steps += chunk
            hist.append(k)
            span = 1000 // chunk
            settled = (len(hist) > span and np.isfinite(k) and k != 0
                       and abs(k - hist[-1 - span]) <= tol * abs(k))
        out.append({"image": i, "steps": steps, "settled": bool(settled), "gpu_seconds": ms / 1e3,
                    "permeability": k, "mlups": s.info["lu_per_step"] * steps / (ms / 1e3) / 1e6,
                    "kn_mean": img["kn_mean"], "cells": s.n_cells})
        s.close()
    return {"workload": STEADY_WORKLOAD, "criterion": f"relative permeability change below {tol:g} over 1000 steps",
            "images": out, "gpu_seconds_total": sum(o["gpu_seconds"] for o in out)}


def run_reference(args, rank, world):
    """The CPU arm: the FP64 oracle restatement of the reference step on all host
    cores.  A step is one sample of n coarse steps of image 0, n sized so that the
    whole run (warm-up and K samples) stays within about --ref-budget seconds."""
    if rank != 0:
        return
    from oracle.pygrid import config2_image
    from oracle.pyoracle import for_grid

    # image 0 of the GPU arm's batch (stored as bits in oracle/data); its Kn
    # field, grid tables and unit system from the oracle's own code
    img = config2_image(0)
    threads = os.cpu_count() or 1
    g = oracle_grid(img)
    lu = g.lattice_updates()
    o = for_grid(g, sim="transport", dx=img["dx"], threads=threads)
    t0 = time.perf_counter()
    o.run(1)
    per = max(time.perf_counter() - t0, 1e-6)
    n = max(1, int(args.ref_budget / ((args.steps + args.warmup) * per)))
    for _ in range(args.warmup):
        o.run(n)
    rates = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.run(n)
        rates.append(lu * n / (time.perf_counter() - t0) / 1e6)
    o.close()
    rate = float(np.median(rates))
    line = {
        "impl": "reference", "metric": "MLUPS", "value": rate, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "images": 1, "n": 1024, "levels": 3},
        "cpu_baseline": {"value": rate, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"image 0, {n} coarse step(s) per step (median of {args.steps}), FP64 oracle "
                                   f"restatement of the reference step (oracle/lbm_oracle.cpp) on the oracle's own "
                                   f"grid tables (oracle/grid_oracle.cpp), OpenMP {threads} threads"},
        "e2e": {"value": rate, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "product_libraries_loaded": loaded_product_libraries(),
    }
    print(json.dumps(line))


def adsorption_leg(steps, warmup, engine):
    """Config 3 (Shan-Chen adsorption, 512x512 seeded disk image, porosity 0.6,
    psi = rho0 (1 - exp(-rho/rho0)), G = -4.5, G_ads = -0.5, rho = 0.5 +- 1e-3):
    MLUPS of the two-pass adsorption step with the per-step density residual,
    device-timed over `steps` steps, and the roofline of the step (80 B per
    update: 72 B of populations and the psi plane written and read)."""
    import torch

    from mantiis_gb300 import SIM_ADSORPTION, Solver, default_params
    from mantiis_gb300.workloads import config3

    img = config3(0)
    # the common-convention constants in the reference's force convention
    p = default_params(dx=img["dx"], simulation=SIM_ADSORPTION, rho_init=0.5, fbody=0.0, psi_form=1, rho_psi=0.5,
                       g_ff=-4.5 / 18, g_fs=3 * -0.5, check_every=1)
    stream = torch.cuda.Stream()
    s = Solver(img["pore"], img["kn"], img["locpore"], p)
    s.set_stream(stream.cuda_stream)
    s.set_engine(engine)
    rng = np.random.default_rng(3000)
    rho = 0.5 + rng.uniform(-1e-3, 1e-3, s.n_cells)
    s.set_equilibrium(rho, np.zeros_like(rho), np.zeros_like(rho))
    s.advance(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.advance(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = s.info["lu_per_step"]
    mass = float(s.observables()["mass"])
    s.close()
    peak, peak_kind = peaks()
    achieved = 80.0 * cells * steps / (ms / 1e3) / 1e9
    return {
        "metric": "MLUPS", "value": cells * steps / (ms / 1e3) / 1e6, "unit": "MLUPS", "n_gpus": 1,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps, "higher_is_better": True,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "config3: 512x512 seeded disk image, porosity 0.6, Shan-Chen adsorption, "
                               "exponential psi (rho0 0.5), G -4.5, G_ads -0.5, rho 0.5 +- 1e-3",
                   "cells": cells, "l2": "state L2-resident (one 512^2 image)",
                   "engine": "one cooperative launch per call (grid barriers between passes)" if engine
                   else "launches per pass, pairs of steps from a CUDA graph"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "kernel": "adsorption step (" + ("k_ads_persistent" if engine else
                                                      "k_ads_psi + k_ads_step") + ")",
                     "bytes_per_unit": 80.0},
        "mass_after": mass,
    }


def run_adsorption(args):
    print(json.dumps(adsorption_leg(args.steps, args.warmup, args.ads_engine)))


def run_conv(args):
    """The warm-start network's 3x3 convolutions at its layer sizes (8 images;
    32..256 channels at 128^2..16^2 pixels, as the encoder-decoder's levels):
    device time per call of the CUDA-core kernels and of the tcgen05 implicit
    GEMMs, forward (bias + ReLU), data gradient and weight gradient, median of
    `--steps` calls after `--warmup`; FLOP = 2 * 9 * cin * cout * pixels."""
    import torch

    from mantiis_gb300.surrogate import _ptr, cnn_lib

    L = cnn_lib()
    torch.manual_seed(0)
    stream = torch.cuda.current_stream()
    s = C.c_void_p(stream.cuda_stream)
    layers = [(8, 32, 32, 128), (8, 64, 64, 64), (8, 128, 128, 32), (8, 256, 256, 16)]
    out = []
    for n, cin, cout, hw in layers:
        x = torch.randn(n, cin, hw, hw, device="cuda")
        dy = torch.randn(n, cout, hw, hw, device="cuda")
        w = torch.randn(cout * cin * 9, device="cuda") * (2.0 / (9 * cin)) ** 0.5
        w16 = torch.empty(w.numel(), dtype=torch.int16, device="cuda")
        L.cnn_to_bf16(_ptr(w), _ptr(w16), w.numel(), s)
        b = torch.zeros(cout, device="cuda")
        y = torch.empty(n, cout, hw, hw, device="cuda")
        dx = torch.empty_like(x)
        dw = torch.zeros(cout * cin * 9, device="cuda")
        db = torch.zeros(cout, device="cuda")
        calls = {
            "forward_cuda_cores": lambda: L.cnn_conv3x3_forward(_ptr(x), _ptr(w16), _ptr(b), _ptr(y), n, cin, cout,
                                                                hw, hw, 1, s),
            "forward_tcgen05": lambda: L.cnn_conv3x3_forward_tc(_ptr(x), _ptr(w16), _ptr(b), _ptr(y), n, cin, cout,
                                                                hw, hw, 1, s),
            "data_grad_cuda_cores": lambda: L.cnn_conv3x3_backward_data(_ptr(dy), _ptr(w16), _ptr(dx), n, cin, cout,
                                                                        hw, hw, s),
            "data_grad_tcgen05": lambda: L.cnn_conv3x3_backward_data_tc(_ptr(dy), _ptr(w16), _ptr(dx), n, cin, cout,
                                                                        hw, hw, s),
            "weight_grad_cuda_cores": lambda: L.cnn_conv3x3_backward_weight(_ptr(x), _ptr(dy), _ptr(dw), _ptr(db), n,
                                                                            cin, cout, hw, hw, s),
            "weight_grad_tcgen05": lambda: L.cnn_conv3x3_backward_weight_tc(_ptr(x), _ptr(dy), _ptr(dw), _ptr(db),
                                                                            n, cin, cout, hw, hw, s),
        }
        flop = 2.0 * 9 * cin * cout * n * hw * hw
        row = {"images": n, "cin": cin, "cout": cout, "pixels": hw * hw, "gflop": flop / 1e9}
        for name, fn in calls.items():
            for _ in range(args.warmup):
                if fn() != 0:
                    raise RuntimeError(f"{name} failed")
            times = []
            for _ in range(args.steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            ms = float(np.median(times))
            row[name] = {"us": ms * 1e3, "tflops": flop / (ms / 1e3) / 1e12}
        if L.cnn_tc_error() != 0:
            raise RuntimeError("a tensor-core wait ran out")
        out.append(row)
    peak = None
    try:
        peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("bf16_tflops")
    except (OSError, ValueError):
        pass
    print(json.dumps({"metric": "conv3x3_tflops", "unit": "TFLOP/s", "layers": out, "bf16_peak_tflops": peak,
                      "note": "BF16 operands, FP32 accumulation; the tcgen05 path splits each FP32 activation "
                              "into two BF16 parts (two MMAs per product)"}))


def run_properties(args):
    from mantiis_gb300 import generate_disks, pore_properties, pore_properties_gpu

    n = args.properties
    pore = generate_disks(n, max(2, n // 64), max(4, n // 16), 0.6, 5, open_x_edges=True)
    for _ in range(args.warmup):
        pore_properties_gpu(pore[: min(n, 256), : min(n, 256)].copy(), 1e-9, 5e-9)
    times = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        lp, kn, iters = pore_properties_gpu(pore, 1e-9, 5e-9, return_iterations=True)
        times.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    lp_h, kn_h = pore_properties(pore, 1e-9, 5e-9)
    host_s = time.perf_counter() - t0
    print(json.dumps({
        "metric": "pore_properties_ms", "value": round(1e3 * float(np.median(times)), 3), "unit": "ms",
        "higher_is_better": False, "steps": len(times), "warmup": args.warmup,
        "config": {"workload": f"one {n}x{n} seeded disk image (r U[{max(2, n // 64)},{max(4, n // 16)}], "
                               "porosity 0.6, void x edges)", "thinning_iterations": int(iters)},
        "host_ms": round(1e3 * host_s, 1), "host_cores": 1,
        "bit_equal": bool(np.array_equal(lp, lp_h) and np.array_equal(kn, kn_h)),
        "gpu_launches": 2 * 16 * int(-(-iters // 16)) + 9,
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--images", type=int, default=4)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--ref-budget", type=float, default=150.0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--min-seconds", type=float, default=0.5,
                    help="repeat the timed K-step window until the windows cover this much time")
    ap.add_argument("--steady-images", type=int, default=4,
                    help="images of the steady-state leg (0 = skip it)")
    ap.add_argument("--engine", type=int, default=0, choices=[0, 1],
                    help="batch engine: 0 per-image launches on concurrent streams, 1 one persistent launch per step")
    ap.add_argument("--steady-batch", type=int, default=0,
                    help="also run this many config4_steady images to steady state as one batch")
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--properties", type=int, default=0, metavar="N")
    ap.add_argument("--conv", action="store_true",
                    help="time the warm-start network's convolutions (CUDA cores and tcgen05) instead")
    ap.add_argument("--adsorption", action="store_true", help="time the config-3 adsorption step instead")
    ap.add_argument("--adsorption-steps", type=int, default=2000,
                    help="steps of the config-3 adsorption leg of the headline run (0 = skip it)")
    ap.add_argument("--ads-engine", type=int, default=1, choices=[0, 1],
                    help="adsorption engine: 1 one cooperative launch per call, 0 launches per pass")
    # plain-cell kernels: -1 times all three at creation (autotune); a fixed
    # path keeps profiled runs, whose timings the profiler distorts, on one path
    ap.add_argument("--plain-path", type=int, default=-1, choices=[-1, 0, 1, 2])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.properties:
        run_properties(args)
        return
    if args.conv:
        run_conv(args)
        return
    if args.adsorption:
        run_adsorption(args)
        return

    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from mantiis_gb300 import Batch, Solver

    imgs = rank_images(args.images, rank, world, args.workload)
    # a dedicated (non-default) stream: every context enqueues on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    solvers = []
    for img in imgs:
        p_img = params_for(img, args.plain_path)
        p_img.concurrent = 1  # the batch and the end-to-end leg step several images at once
        s = Solver(img["pore"], img["kn"], img["locpore"], p_img)
        s.set_stream(stream.cuda_stream)
        solvers.append(s)
    lu_step = float(sum(s.info["lu_per_step"] for s in solvers))
    state_mb = sum(s.info["device_bytes"] for s in solvers) / 1e6

    # all images step together: one launch per phase over the batch, two
    # coarse steps per CUDA graph (captured during the warm-up)
    batch = Batch(solvers)
    batch.set_stream(stream.cuda_stream)
    batch.set_engine(args.engine, 0)
    warm = args.warmup + (args.warmup % 2)
    batch.advance(warm)
    torch.cuda.synchronize()
    K = args.steps + (args.steps % 2)
    clk = ClockSampler(local)
    clk.start()
    # the K-step window is timed again and again until the windows cover at
    # least --min-seconds (and at least 3 windows), so that the clock sampler
    # sees the GPU under load; the median window is reported
    windows, total_ms, launches = [], 0.0, 0
    while len(windows) < 3 or total_ms < 1e3 * args.min_seconds:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = batch.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.advance(K)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = batch.launches - l0
        windows.append(e0.elapsed_time(e1))
        total_ms += windows[-1]
    clocks = clk.stop()
    ms = float(np.median(windows))
    value, ms, lu_job = job_rate(lu_step, ms, K, dist, "cuda")

    finite = all(np.isfinite(o["mean_ux"]) for o in batch.observables())
    batch.close()

    # roofline: finest-level step kernel of image 0 on a separate context
    prof = Solver(imgs[0]["pore"], imgs[0]["kn"], imgs[0]["locpore"], params_for(imgs[0], args.plain_path))
    prof.set_stream(stream.cuda_stream)
    prof.advance(2)
    lvl1 = prof.level_info(1)
    plain_kernels = {0: "k_phase_plain", 1: "k_phase_plain_tma + k_phase_plain", 2: "k_phase_plain8"}[
        prof.info["plain_path"]]
    reps = 200
    prof.step_level(1, 10)
    torch.cuda.synchronize()
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    prof.step_level(1, reps)
    r1.record(stream)
    torch.cuda.synchronize()
    k_ms = r0.elapsed_time(r1) / reps
    peak, peak_kind = peaks()
    achieved = BYTES_PER_LU * lvl1["active"] / (k_ms / 1e3) / 1e9
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get("level1_substep_bytes")
        except Exception:
            traffic = None
    prof.close()

    # end to end through the public API with host buffers: the images on
    # E2E_THREADS host threads, each context on its own stream (contexts are
    # independent and single-threaded);
    # per image the equilibrium state is uploaded, Ke steps run with the per-step
    # residual and break test, and the cell fields are read back
    def e2e_leg(Ke):
        """Per image (on E2E_THREADS host threads, each context on its own
        stream): upload of the initial state, Ke steps with the per-step residual
        and break test, read-back of the cell fields; None when Ke is 0 (for
        profiled runs, whose multi-threaded host calls the profiler serialises)."""
        if Ke <= 0:
            return None
        e2e_streams = [torch.cuda.Stream() for _ in solvers]
        # (the contexts were created with concurrent=1: two of them step at once)
        for s, st in zip(solvers, e2e_streams):
            s.set_stream(st.cuda_stream)

        # pinned host buffers per image: the initial state and the fields read back
        pinned = []
        for s in solvers:
            n = s.n_cells
            buf = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
                   for k in ("rho", "ux", "uy", "out_rho", "out_ux", "out_uy")}
            buf["rho"][:] = s.info["rho_in"]
            buf["ux"][:] = 0.0
            buf["uy"][:] = 0.0
            pinned.append(buf)

        def e2e_image(i, steps):
            s, b = solvers[i], pinned[i]
            n = s.n_cells
            s.set_equilibrium(b["rho"], b["ux"], b["uy"])
            s.run(steps)
            s.cells(out={"rho": b["out_rho"], "ux": b["out_ux"], "uy": b["out_uy"]})
            return 3 * n * 8, 3 * n * 8 + steps * 4 * 8

        from concurrent.futures import ThreadPoolExecutor

        with ThreadPoolExecutor(min(len(solvers), E2E_THREADS)) as ex:
            # untimed: plans, checkpoint buffers and the two-step residual graph
            list(ex.map(lambda i: e2e_image(i, 5), range(len(solvers))))
            torch.cuda.synchronize()
            # the whole leg (upload, Ke steps, download of every image) is timed
            # E2E_REPEATS times from the same initial state; the median is reported,
            # since one ~60 ms host-timed run is exposed to host-side hiccups
            e2e_runs = []
            for _ in range(E2E_REPEATS):
                t0 = time.perf_counter()
                moved = list(ex.map(lambda i: e2e_image(i, Ke), range(len(solvers))))
                torch.cuda.synchronize()
                e2e_runs.append(time.perf_counter() - t0)
            e2e_s = float(np.median(e2e_runs))
        h2d = sum(m[0] for m in moved)
        d2h = sum(m[1] for m in moved)
        e2e = lu_step * Ke / e2e_s / 1e6
        return {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": h2d / Ke, "d2h_bytes_per_step": d2h / Ke,
                "steps": Ke, "seconds": e2e_s, "repeats": len(e2e_runs),
                "seconds_min_max": [min(e2e_runs), max(e2e_runs)]}

    e2e_obj = e2e_leg(args.e2e_steps)

    steady = None
    if rank == 0 and args.steady_images > 0:
        steady = steady_state_leg(args.steady_images, stream)
    steady_batch = None
    if rank == 0 and args.steady_batch > 0:
        steady_batch = steady_batch_leg(args.steady_batch, stream)

    # config 3 beside the headline: the adsorption step of one 512^2 image
    config3 = None
    if rank == 0 and args.adsorption_steps > 0:
        config3 = adsorption_leg(args.adsorption_steps, 10, args.ads_engine)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        og = oracle_grid(imgs[0])
        rate, steps, dt, lu = cpu_oracle_rate(og, imgs[0]["dx"], args.cpu_seconds, threads)
        rate1, steps1, dt1, _ = cpu_oracle_rate(og, imgs[0]["dx"], args.cpu_seconds / 2, 1)
        cpu = {"value": rate, "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": f"image 0 of the batch, {steps} coarse steps ({dt:.1f} s), FP64 oracle restatement of the "
                         f"reference step (oracle/lbm_oracle.cpp) on the oracle's own grid tables "
                         f"(oracle/grid_oracle.cpp), OpenMP {threads} threads; stepping only (the grid and the "
                         f"initial state are built before the timed steps)",
               "value_1_thread": rate1, "sample_1_thread": f"{steps1} coarse steps ({dt1:.1f} s), 1 thread"}

    if rank == 0:
        line = {
            "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": warm,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "images_per_gpu": len(imgs),
                       "n": [int(im["pore"].shape[0]) for im in imgs] if args.workload == "config4" else 1024,
                       "levels": [int(im["levels"]) for im in imgs] if args.workload == "config4" else imgs[0]["levels"],
                       "lu_per_step_per_gpu": lu_step, "device_state_mb_per_gpu": round(state_mb, 1),
                       "l2": "inputs larger than L2 (state of the batch > 129 MB)",
                       "graph": ("one CUDA graph of 2 coarse steps for the whole batch, images on L2-sized concurrent "
                                 "streams" if args.engine == 0 else
                                 "one CUDA graph of 2 coarse steps for the whole batch, one persistent launch per step"),
                       "state_finite_after_timed_steps": finite,
                       **({} if finite else {"state_note": "the reference's multi-block scheme diverges on these "
                                                           "images (its FP64 restatement too); the step's work "
                                                           "and timing do not depend on the values"})},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": f"level-1 substep ({plain_kernels} + k_phase_special)", "units_per_launch": lvl1["active"],
                         "bytes_per_unit": BYTES_PER_LU, "ms_per_launch": k_ms,
                         # the whole batch step: 72 B per lattice update at the bench's own rate
                         "batch_achieved": BYTES_PER_LU * value / 1e3, "batch_frac": BYTES_PER_LU * value / 1e3 / peak},
            "timing": {"windows": len(windows), "window_steps": K, "ms_min": min(windows), "ms_max": max(windows),
                       "seconds_timed": total_ms / 1e3},
            "steady_state": steady,
            **({"steady_batch": steady_batch} if steady_batch else {}),
            **({"config3": {k: config3[k] for k in ("value", "unit", "ms_per_step", "steps", "roofline", "config",
                                                    "mass_after")}} if config3 else {}),
            "cpu_baseline": cpu,
            "e2e": e2e_obj,
            "clocks": clocks,
            "gpu_launches": int(launches),
        }
        print(json.dumps(line))
    for s in solvers:
        s.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
