"""Benchmark: particle-steps/s of the TRISTAN-MP hot path on one GB300.

Workload (default `value`): the 2D two-stream/Weibel box of 1024 x 1024
cells, 3rd-order shapes, 16 particles per cell per species (33.5 M
particles), 4 filter passes, FP64 Gauss-law / energy / momentum diagnostics
every lap. A "step" is one full lap of the main loop: field advance, push,
Esirkepov deposit, periodic wrap, current fold, filter, add_current, tile
sort and the diagnostics. Inputs are seeded synthetic plasmas with the
reference setup's shapes (tristan_gb300.setups); the particle arrays (~2 GB)
are far larger than the 129 MB L2, so no flush is needed between laps.

The same line carries, with the same fields, `c3`: the 3D Weibel box of
256^3 cells at order 2 (134 M particles), the configuration the 3D targets
are stated on; `ensemble`: 64 seeded 2D boxes, batched fixed point against
the plain form; and `shock`: the 2D pair shock on 8192 x 512 cells.

Arms:
  default           the GB300 C-ABI library; prints one JSON line with the
                    FP32 deposit form as `value` (each tile's exact
                    fixed-point sums rounded once to FP32 and added with
                    FP32 global atomics), the int64 fixed-point form beside
                    it, the dominant kernel's roofline, the CPU baseline,
                    the end-to-end figure, the Gauss-law residuals and the
                    SM clocks.
  --impl reference  the reference algorithm on the host cores: the OpenMP
                    build of the CPU restatement (the reference is Fortran
                    with MPI, and no Fortran compiler is installed, so the
                    reference itself cannot be built).

Multi-GPU: the path does not shard (one domain, no collectives); N ranks
run N independent replicas and `value` sums them (weak scaling).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

METRIC = "particle-steps/s (push+deposit+fields), batched/fixed-pt vs plain, same GB300"
UNIT = "particle-steps/s"
DEFAULT_WORKLOAD = "twostream2d_1024_o3"
C3_WORKLOAD = "weibel3d_256_o2"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-c3", action="store_true", help="leave out the 3D order-2 record of the default line")
    ap.add_argument("--no-fixed", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--host-parts", type=int, default=0,
                    help="parts per species of the end-to-end lap (0: by size)")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--sort-every", type=int, default=0, help="0: chosen by the autotuner")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tile", type=int, nargs=3, default=None,
                    help="tile shape of the single-domain workloads (with --no-autotune)")
    ap.add_argument("--ppc0", type=float, default=None,
                    help="particles per cell of both species together (profiling the field kernels on the "
                         "full grid with few particles)")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-shock", action="store_true")
    ap.add_argument("--shock-steps", type=int, default=100)
    ap.add_argument("--shock-sort-every", type=int, default=4,
                    help="tile sort cadence of the shock run (injected particles ride the tail kernel between sorts)")
    ap.add_argument("--ens-boxes", type=int, default=64)
    ap.add_argument("--ens-steps", type=int, default=40)
    ap.add_argument("--ens-tile", type=int, nargs=2, default=None,
                    help="tile shape of the ensemble (with --no-autotune)")
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws, local):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws, impl):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if impl == "gb300" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples during the timed region (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        time.sleep(0.25)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(workload, form):
    """per-launch DRAM bytes of the tile kernel from the committed ncu summary"""
    try:
        with open(os.path.join(ROOT, "profiles", "tile_kernel_traffic.json")) as f:
            d = json.load(f)
        return d.get(workload, {}).get(form)
    except Exception:
        return None


def committed_instructions(workload, form):
    """warp instructions per launch of the tile kernel from the committed ncu summary"""
    try:
        with open(os.path.join(ROOT, "profiles", "tile_kernel_traffic.json")) as f:
            d = json.load(f)
        return d.get("warp_instructions", {}).get(workload, {}).get(form)
    except Exception:
        return None


def tile_kernel_bytes(cfg, n_particles, fixed):
    """algorithmic bytes of one push+deposit launch: per particle read
    cell+offsets+u+ch (32 B) and write cell+offsets+u (28 B); per cell the
    gathered E,B (24 B) and the flushed current (12 B, 24 B fixed point)"""
    return 60.0 * n_particles + (24.0 + (24.0 if fixed else 12.0)) * cfg.ncells


# the two deposit forms, as they are: both sum a tile's FP32 Esirkepov
# contributions exactly in a fixed-point shared-memory window
DEPOSIT_FP32 = ("fp32: exact fixed-point tile window, each tile sum rounded once to FP32 and added with "
                "FP32 global atomics")
DEPOSIT_FIXED = "int64 fixed point (bit-reproducible)"


def run_form(cfg, ions, lecs, warmup, steps, fixed, device, ws, local, clocks=False):
    from tristan_gb300.gpu import GpuSim
    cfg.fixed = int(fixed)
    sim = GpuSim(cfg, device=device)
    sim.set_particles(ions, lecs)
    w = max(warmup, 3)
    sim.step(w)
    sim.synchronize()
    sim.enable_timing(True)
    barrier(ws, local)
    sim.synchronize()
    if clocks:
        with ClockSampler(device) as cs:
            ms = sim.step_timed(steps)
        clk = cs.summary()
    else:
        ms = sim.step_timed(steps)
        clk = None
    phases = sim.phase_times()
    kps = sim.kernels_per_step()
    hist = sim.diag_history(min(w + steps, 1024))
    sim.close()
    return ms, phases, kps, clk, hist


def run_e2e(cfg, ions, lecs, e2e_steps, host_parts, device):
    from tristan_gb300.gpu import GpuSim, SYNC_ALL, SYNC_B, SYNC_E, SYNC_PARTICLES
    cfg.fixed = 0
    sim = GpuSim(cfg, device=device, pinned=True)
    sim.set_particles(ions, lecs, upload=False)
    sim.set_host_parts(host_parts)
    up = SYNC_E | SYNC_B | SYNC_PARTICLES
    sim.sync_from_host(SYNC_ALL)
    sim.step_host(1)
    h2d, d2h = sim.host_bytes(up), sim.host_bytes(SYNC_ALL)
    huge = sim.host_huge_fraction()
    # one tg_step_host call per lap: E, B and the records up, the lap,
    # everything back, as the reference's main loop would drive it
    laps = []
    # the interpreter's cyclic garbage collector stays off while the laps
    # are timed (a collection pass is the harness's pause, not the lap's)
    gc_was = gc.isenabled()
    gc.disable()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        sim.step_host(1)
        laps.append((time.perf_counter() - t1) * 1e3)
    dt = time.perf_counter() - t0
    if gc_was:
        gc.enable()
    sim.close()
    return dt, h2d, d2h, huge, laps


def copy_only_ms(h2d, d2h, device, reps=3):
    """the same bytes moved between page-locked host memory and the device
    with nothing else running, both directions at once (one stream each):
    the link's bound for one end-to-end step. The host buffers come from the
    same allocator as GpuSim's pinned host arrays (anonymous memory advised
    for huge pages, then cudaHostRegister), so both see the same kind of
    pages. Returns (ms, share of the buffers on huge pages)."""
    import ctypes
    import torch
    from tristan_gb300 import gpu
    dev = torch.device("cuda", device)
    rt = gpu._cudart_lib()
    rt.cudaMemcpyAsync.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                   ctypes.c_void_p]
    rt.cudaMemcpyAsync.restype = ctypes.c_int
    hu = gpu._host_array(h2d, np.uint8, True)
    hd = gpu._host_array(d2h, np.uint8, True)
    hu[:] = 1
    hd[:] = 1
    huge = gpu.huge_page_fraction([hu, hd])
    for a in (hu, hd):
        if rt.cudaHostRegister(a.ctypes.data, a.nbytes, 0) != 0:
            raise RuntimeError("cudaHostRegister failed")
    du = torch.empty(h2d, dtype=torch.uint8, device=dev)
    dd = torch.empty(d2h, dtype=torch.uint8, device=dev)
    s_up, s_down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    try:
        for r in range(reps + 1):
            if r == 1:
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
            if rt.cudaMemcpyAsync(du.data_ptr(), hu.ctypes.data, h2d, 1, s_up.cuda_stream) != 0:
                raise RuntimeError("cudaMemcpyAsync failed")
            if rt.cudaMemcpyAsync(hd.ctypes.data, dd.data_ptr(), d2h, 2, s_down.cuda_stream) != 0:
                raise RuntimeError("cudaMemcpyAsync failed")
        torch.cuda.synchronize(dev)
        ms = (time.perf_counter() - t0) / reps * 1e3
    finally:
        torch.cuda.synchronize(dev)
        for a in (hu, hd):
            rt.cudaHostUnregister(a.ctypes.data)
    del du, dd
    return ms, huge


def cpu_baseline(cfg, ions, lecs, steps):
    """the OpenMP CPU restatement on the host cores: one warm-up lap, then
    `steps` timed laps; the oracle's FP64 diagnostics after the warm-up lap
    and after the last lap (outside the timed region)"""
    import oracle
    oracle.build()
    cfg.fixed = 0
    sim = oracle.OracleSim(cfg, openmp=True)
    sim.set_particles(ions, lecs)
    sim.step(1)
    d_first = sim.diagnostics()
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    d_last = sim.diagnostics()
    return dt, sim.lib.to_num_threads(), d_first, d_last


def species_density_norm(cfg, nions, nlecs):
    """|rho_s|_2 of one species' mean charge density over the interior
    cells (unit particle weights, as the loaders make them)"""
    ncell = cfg.interior_cells
    return (abs(cfg.qi) * nions + abs(cfg.qe) * nlecs) / (2.0 * ncell) * (ncell ** 0.5)


def hist_residual(hist, lap):
    """(relative, absolute) Gauss residual of 1-based `lap` from a diag
    history whose first record is lap 1"""
    if lap < 1 or lap > len(hist) or hist[lap - 1][1] <= 0:
        return None, None
    r2, p2 = hist[lap - 1][0], hist[lap - 1][1]
    return float(np.sqrt(r2 / p2)), float(np.sqrt(r2))


def measure_workload(name, args, ws, rank, local, steps, warmup, e2e_steps, cpu_steps, sort_every, autotune):
    """One single-domain workload: the FP32 form timed by CUDA events with
    the SM clocks sampled (value), the fixed-point form, the end-to-end lap
    through tg_step_host, the fused kernel's roofline, the CPU baseline and
    the Gauss-law residuals. Returns the fields of a bench line."""
    from tristan_gb300 import setups
    device = local
    cfg = setups.make_config(name, diag_every=1, sort_every=max(sort_every, 1))
    if args.ppc0:
        cfg.ppc0 = float(args.ppc0)
    if args.tile and not autotune:
        cfg.tile = tuple(args.tile)
    ions, lecs = setups.load_beams(cfg, seed=123457 + rank)
    setups.with_capacity(cfg, len(ions), len(lecs))
    n_p = len(ions) + len(lecs)
    tuned = None
    if autotune:
        # tile shape and re-sort cadence for this plasma (before any timing)
        from tristan_gb300.gpu import autotune as tune
        best, table = tune(cfg, ions, lecs, laps=2, device=local)
        tuned = {"tile": list(cfg.tile), "sort_every": cfg.sort_every, "best_ms_per_lap": best,
                 "candidates": int(len(table))}
    grid = [cfg.nx, cfg.ny] + ([cfg.nz] if cfg.dims == 3 else [])
    config = {"workload": name, "grid": grid, "order": cfg.order, "particles": n_p,
              "ppc_per_species": int(cfg.ppc0 // 2), "ntimes": cfg.ntimes, "deposit": DEPOSIT_FP32,
              "diagnostics": "fp64 gauss/energy/momentum every lap", "sort_every": cfg.sort_every,
              "tile": list(cfg.tile), "autotuned": tuned,
              "l2": "inputs larger than L2 (particle arrays %.1f GB), no flush" % (n_p * 44 / 1e9)}
    ms, phases, kps, clk, hist = run_form(cfg, ions, lecs, warmup, steps, False, device, ws, local, clocks=True)
    ms = allreduce_max(ms, ws, args.impl)
    value = ws * n_p * steps / (ms / 1e3)
    fixed = None
    if not args.no_fixed:
        ms_f, ph_f, _, _, _ = run_form(cfg, ions, lecs, warmup, steps, True, device, ws, local)
        ms_f = allreduce_max(ms_f, ws, args.impl)
        fixed = {"value": ws * n_p * steps / (ms_f / 1e3), "ms_per_step": ms_f / steps,
                 "particle_kernel_ms": ph_f["particles"], "deposit": DEPOSIT_FIXED}
    dt_e2e, h2d, d2h, huge_lap, lap_ms = run_e2e(cfg, ions, lecs, e2e_steps, args.host_parts, device)
    ms_e2e = dt_e2e / e2e_steps * 1e3
    ms_link, huge_link = copy_only_ms(h2d, d2h, device)
    e2e = {"value": ws * n_p * e2e_steps / dt_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": ms_e2e,
           "link": {"bound": "host link (NVLink-C2C), both directions at once",
                    "copy_only_ms": ms_link, "achieved_gbs": (h2d + d2h) / ms_e2e / 1e6,
                    "peak_gbs": (h2d + d2h) / ms_link / 1e6, "frac": ms_link / ms_e2e,
                    # the host link moves fewer bytes per second from base
                    # pages when both directions run; the kernel grants
                    # huge pages as free memory allows
                    "host_huge_page_share": {"lap_arrays": huge_lap, "copy_buffers": huge_link}},
           # the lap cannot take less than the longer of its copies and its
           # device-resident lap (the two overlap part by part)
           "lap_bound_ms": max(ms_link, ms / steps), "frac_of_lap_bound": max(ms_link, ms / steps) / ms_e2e,
           "mode": "one tg_step_host call per lap: E, B, particle records up; the lap; fields, "
                   "records, counts down (each species in parts: a part is sorted and pushed as soon "
                   "as it is in, and goes home while later parts arrive)",
           "host_parts": args.host_parts or "by size",
           # each lap's host wall-clock (the value above is their mean)
           "lap_ms": [round(v, 3) for v in lap_ms], "lap_ms_median": statistics.median(lap_ms)}
    peak, peak_kind = measured_peak_hbm()
    t_kernel = phases["particles"] / 1e3
    alg = tile_kernel_bytes(cfg, n_p, False)
    achieved = alg / t_kernel / 1e9 if t_kernel > 0 else None
    roofline = {"kernel": "k_tiles<%d,%d> (fused push + Esirkepov deposit + wrap)" % (cfg.dims, cfg.order),
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                "traffic": committed_traffic(name, "fp32"),
                "algorithmic_bytes_per_launch": alg, "launch_ms": phases["particles"]}
    # the bound the kernel actually sits at: instruction issue (one warp
    # instruction per clock per SM sub-partition, 4 per SM, at the SM clock
    # sampled during the timed laps)
    ninst = committed_instructions(name, "fp32")
    if ninst and t_kernel > 0 and clk and clk.get("sm_mhz"):
        issue_peak = 152 * 4 * clk["sm_mhz"] * 1e6
        roofline["issue"] = {"achieved": ninst / t_kernel, "peak": issue_peak, "unit": "warp-instructions/s",
                             "frac": ninst / t_kernel / issue_peak, "instructions_per_launch": ninst,
                             "peak_basis": "152 SMs x 4 issue slots x median SM clock under load"}
    total_laps = max(warmup, 3) + steps
    last = min(total_laps, len(hist))
    r_last, a_last = hist_residual(hist, last)
    norm_s = species_density_norm(cfg, len(ions), len(lecs))
    gauss = {"definition": "|div E - F^ntimes(rho)|_2 / |F^ntimes(rho)|_2 over the interior, FP64 on the "
                           "device; vs_species_density: the same numerator over one species' mean charge "
                           "density",
             "lap": last, "residual": r_last,
             "residual_vs_species_density": (a_last / norm_s) if a_last is not None else None}
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and cpu_steps > 0:
        dt_cpu, cores, d1, dN = cpu_baseline(cfg, ions, lecs, cpu_steps)
        cpu = {"value": n_p * cpu_steps / dt_cpu, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cpu_steps} full laps of the workload (after 1 warm-up lap) on the OpenMP "
                         "CPU restatement; the Fortran reference cannot be built (no Fortran compiler)"}
        # the reference arithmetic's own residual on the same plasma: the
        # oracle's FP32 laps against the device's at the same lap
        g1, _ = hist_residual(hist, 1)
        gN, _ = hist_residual(hist, 1 + cpu_steps)
        gauss["reference_arithmetic"] = {
            "laps": [1, 1 + cpu_steps], "oracle": [d1["gauss_residual"], dN["gauss_residual"]],
            "gpu": [g1, gN],
            "note": "the same residual in the CPU restatement of the reference's FP32 arithmetic: the "
                    "floor is the rounding of each Esirkepov contribution and carry, not the GPU path"}
    d = hist[-1] if len(hist) else None
    return {"value": value, "ms_per_step": ms / steps, "config": config, "fixed_point": fixed,
            "phase_ms_per_lap": phases, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": kps * steps, "gauss": gauss,
            "gauss_residual_last_lap": (float(np.sqrt(d[0] / d[1])) if d is not None and d[1] > 0 else None)}


def run_ensemble(args, device):
    """The 64-box ensemble: the batched fixed-point form (one launch per
    phase for all boxes, graph-replayed) against the plain form (one
    single-domain context per box, all resident, each lap stepped box after
    box through tg_step and timed by the host clock around the whole loop,
    so the host gaps between boxes count), both on the same seeded boxes,
    tile shape and sort cadence; no diagnostics in the timed laps of either.
    Particle-steps/s are aggregated over all boxes. The CPU baseline runs
    the OpenMP restatement box after box (one timed lap each) and sums."""
    from tristan_gb300 import setups
    from tristan_gb300.gpu import EnsembleSim, GpuSim, ensemble_autotune
    t0 = time.perf_counter()
    cfgs, table = setups.ensemble_configs(nbox=args.ens_boxes, seed=20240607)
    parts = setups.load_ensemble(cfgs)
    t_load = time.perf_counter() - t0
    counts = [len(i) + len(l) for i, l in parts]
    n_p = sum(counts)
    # autotune on a sample of boxes: the two largest of each shape order
    sample = []
    for o in (1, 2, 3):
        idx = sorted((b for b, c in enumerate(cfgs) if c.order == o), key=lambda b: -counts[b])[:2]
        sample += idx
    tuned = None
    if not args.no_autotune and sample:
        scfg = [cfgs[b] for b in sample]
        best, tab = ensemble_autotune(scfg, [parts[b] for b in sample], laps=1, device=device)
        for c in cfgs:
            c.tile, c.sort_every = scfg[0].tile, scfg[0].sort_every
        tuned = {"tile": list(scfg[0].tile), "sort_every": scfg[0].sort_every, "sample_boxes": sample,
                 "best_ms_per_lap_on_sample": best, "candidates": int(len(tab))}
    elif args.ens_tile:
        for c in cfgs:
            c.tile, c.sort_every = (args.ens_tile[0], args.ens_tile[1], 1), max(args.sort_every, 1)
    se = cfgs[0].sort_every
    warm = max(args.warmup, 2 * se)
    K = max(2 * se, args.ens_steps // (2 * se) * (2 * se))

    def batched(fixed):
        for c in cfgs:
            c.fixed = int(fixed)
        e = EnsembleSim(cfgs, device=device)
        for b, (ions, lecs) in enumerate(parts):
            e.set_particles(b, ions, lecs)
        e.sync_from_host()
        e.step(warm)
        e.synchronize()
        ms = e.step_timed(K)
        res, res_s = 0.0, 0.0
        for b in range(e.nbox):
            d = e.diagnostics(b)
            res = max(res, d["gauss_residual"])
            res_s = max(res_s, d["gauss_abs"] / species_density_norm(cfgs[b], len(parts[b][0]), len(parts[b][1])))
        kps = e.kernels_per_step()
        e.close()
        return ms, res, res_s, kps

    if args.workload == "ensemble64" and args.no_fixed:
        # profiling: the batched fixed-point form alone
        ms_bf, _, _, kps = batched(True)
        return {"batched_fixed": {"value": n_p * K / (ms_bf / 1e3), "ms_per_step": ms_bf / K}}

    def plain(fixed):
        """(host wall-clock ms of K laps of every box, the sum of each box's
        own device time for K laps)"""
        sims = []
        try:
            for b, c in enumerate(cfgs):
                c.fixed = int(fixed)
                g = GpuSim(c, device=device)
                g.set_particles(*parts[b])
                g.step(warm)
                sims.append(g)
            for g in sims:
                g.synchronize()
            t0 = time.perf_counter()
            for _ in range(K):
                for g in sims:
                    g.step(1)
            for g in sims:
                g.synchronize()
            wall = (time.perf_counter() - t0) * 1e3
            dev = sum(g.step_timed(K) for g in sims)
        finally:
            for g in sims:
                g.close()
        return wall, dev

    ms_bf, res_bf, res_bf_s, kps = batched(True)
    ms_b32, res_b32, res_b32_s, _ = batched(False)
    wall_pf, dev_pf = plain(True)
    wall_p32, dev_p32 = plain(False)
    rate = lambda ms: n_p * K / (ms / 1e3)
    orders = {o: sum(1 for c in cfgs if c.order == o) for o in (1, 2, 3)}
    cpu = None
    if not args.no_cpu:
        import oracle
        oracle.build()
        t_cpu, threads = 0.0, 1
        for b, c in enumerate(cfgs):
            c.fixed = 0
            sim = oracle.OracleSim(c, openmp=True)
            sim.set_particles(*parts[b])
            sim.step(1)
            t1 = time.perf_counter()
            sim.step(1)
            t_cpu += time.perf_counter() - t1
            threads = sim.lib.to_num_threads()
            del sim
        cpu = {"value": n_p / t_cpu, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one lap of every box (after one warm-up lap each) on the OpenMP CPU restatement, "
                         "box after box, summed"}
    return {
        "workload": "ensemble of %d periodic 2D boxes (seeded sides, plasmas, shape orders)" % len(cfgs),
        "boxes": len(cfgs), "particles": n_p, "cells": int(sum(c.nx * c.ny for c in cfgs)),
        "boxes_per_order": orders, "seed": 20240607, "steps": K, "warmup": warm,
        "tile": list(cfgs[0].tile), "sort_every": se, "autotuned": tuned,
        "batched_fixed": {"value": rate(ms_bf), "ms_per_step": ms_bf / K, "gauss_residual_max": res_bf,
                          "gauss_residual_vs_species_density_max": res_bf_s},
        "batched_fp32": {"value": rate(ms_b32), "ms_per_step": ms_b32 / K, "gauss_residual_max": res_b32,
                         "gauss_residual_vs_species_density_max": res_b32_s},
        "plain_fp32": {"value": rate(wall_p32), "ms_per_step": wall_p32 / K,
                       "device_only": {"value": rate(dev_p32), "ms_per_step": dev_p32 / K},
                       "form": "one single-domain context per box, all resident; each lap every box's tg_step "
                               "in turn, host wall-clock around the loop (device_only: the boxes' own device "
                               "times summed, no host gaps)"},
        "plain_fixed": {"value": rate(wall_pf), "ms_per_step": wall_pf / K,
                        "device_only": {"value": rate(dev_pf), "ms_per_step": dev_pf / K}},
        "batched_fixed_over_plain_fp32": wall_p32 / ms_bf,
        "batched_fixed_over_plain_fixed": wall_pf / ms_bf,
        "batched_fixed_over_plain_fixed_device_only": dev_pf / ms_bf,
        "cpu_baseline": cpu,
        "kernels_per_step": kps, "host_load_s": t_load,
    }


def run_shock(args, device):
    """The 2D pair shock on 8192 x 512 cells (order 3, 16 per cell per
    species upstream, gamma0 = 15, sigma = 0.1): the initial half-box load
    drawn on the device, then laps with the reflecting wall, conductor and
    moving injector running as kernels inside the lap (graph-replayed; the
    particles injected between two tile sorts are moved by the tail kernel).
    particle-steps/s use the mean particle count of the timed laps."""
    from tristan_gb300 import setups
    from tristan_gb300.gpu import GpuSim, SYNC_ALL
    se = max(1, args.shock_sort_every)
    cfg = setups.make_config("shock2d_8192x512_o3", sort_every=se)
    sh, fields, region = setups.shock_params(cfg)
    K = max(2 * se, args.shock_steps // (2 * se) * (2 * se))
    warm = max(2 * se, max(args.warmup, 4) // (2 * se) * (2 * se))
    cfg.maxhlf = setups.shock_capacity(cfg, K + warm, sh)
    g = GpuSim(cfg, device=device)
    g.set_fields(**fields)
    g.sync_from_host(SYNC_ALL)
    g.shock_init(sh)
    t0 = time.perf_counter()
    g.inject_region(*region)
    g.synchronize()
    t_load = time.perf_counter() - t0
    n_load = sum(g.counts())
    g.step(warm)
    g.synchronize()
    n0 = sum(g.counts())
    ms = g.step_timed(K)
    n1 = sum(g.counts())
    st = g.shock_state()
    kps = g.kernels_per_step()
    g.close()
    mean_n = 0.5 * (n0 + n1)
    return {"workload": "shock2d_8192x512_o3", "grid": [cfg.nx, cfg.ny], "order": cfg.order,
            "ppc_per_species_upstream": int(cfg.ppc0 // 2), "steps": K, "warmup": warm,
            "value": mean_n * K / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / K,
            "particles_initial_load": n_load, "particles_timed": [n0, n1],
            "device_load_s": t_load, "xinject2": st["xinject2"], "walloc": st["walloc"],
            "kernels_per_step": kps, "deposit": DEPOSIT_FP32, "sort_every": se,
            "hooks": "reflecting wall + zigzag, conductor, moving injector (jump-ahead Park-Miller)"}


def main():
    args = parse()
    ws, rank, local = dist_setup(args)
    __graft_entry__.load_package()
    if args.workload == "shock2d_8192x512_o3":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, "workload": args.workload,
                              "shock": run_shock(args, local)}), flush=True)
        return
    if args.workload == "ensemble64":
        # the ensemble alone (its numbers also ride on the default line)
        if rank == 0:
            ens = run_ensemble(args, local)
            print(json.dumps({"metric": METRIC, "unit": UNIT, "workload": "ensemble64", "ensemble": ens}),
                  flush=True)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        from tristan_gb300 import setups
        import oracle
        oracle.build()
        cfg = setups.make_config(args.workload, diag_every=1, sort_every=max(args.sort_every, 1))
        ions, lecs = setups.load_beams(cfg, seed=123457 + rank)
        setups.with_capacity(cfg, len(ions), len(lecs))
        n_p = len(ions) + len(lecs)
        grid = [cfg.nx, cfg.ny] + ([cfg.nz] if cfg.dims == 3 else [])
        config = {"workload": args.workload, "grid": grid, "order": cfg.order, "particles": n_p,
                  "ppc_per_species": int(cfg.ppc0 // 2), "ntimes": cfg.ntimes, "deposit": DEPOSIT_FP32,
                  "diagnostics": "fp64 gauss/energy/momentum every lap", "sort_every": cfg.sort_every,
                  "tile": list(cfg.tile), "autotuned": None,
                  "l2": "inputs larger than L2 (particle arrays %.1f GB), no flush" % (n_p * 44 / 1e9)}
        cfg.fixed = 0
        sim = oracle.OracleSim(cfg, openmp=True)
        sim.set_particles(ions, lecs)
        sim.step(max(args.warmup, 0))
        t0 = time.perf_counter()
        sim.step(args.steps)
        dt = time.perf_counter() - t0
        cores = sim.lib.to_num_threads()
        value = n_p * args.steps / dt
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{args.steps} full laps of the workload, OpenMP CPU restatement "
                                           "(the reference Fortran cannot be built: no Fortran compiler)"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    main_line = measure_workload(args.workload, args, ws, rank, local, args.steps, args.warmup, args.e2e_steps,
                                 args.cpu_steps, args.sort_every, args.impl == "gb300" and not args.no_autotune
                                 and args.sort_every == 0)
    c3 = None
    if args.workload == DEFAULT_WORKLOAD and not args.no_c3:
        # the 3D order-2 target configuration (134 M particles): the same
        # record, fewer laps (about 45 ms each)
        c3 = measure_workload(C3_WORKLOAD, args, ws, rank, local, min(args.steps, 10), 3, 2,
                              min(args.cpu_steps, 2), args.sort_every,
                              args.impl == "gb300" and not args.no_autotune and args.sort_every == 0)
    ens = None
    if rank == 0 and not args.no_ensemble:
        ens = run_ensemble(args, local)
    shock = None
    if rank == 0 and not args.no_shock:
        shock = run_shock(args, local)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": main_line["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main_line["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    for k in ("config", "fixed_point", "phase_ms_per_lap", "roofline", "cpu_baseline", "e2e", "clocks",
              "gpu_launches", "gauss", "gauss_residual_last_lap"):
        line[k] = main_line[k]
    line["c3"] = c3
    line["ensemble"] = ens
    line["shock"] = shock
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
