"""Benchmark of the PIC/DSMC time step: particle-steps/s on one GB300.

Workload (the FP64 form): 200 mm cube at h = 2 mm
(6.0e6 tets, 1.03e6 nodes), 1e7 Ti+ from a 20 mm disk (Thompson energies,
cosine-law directions), Ar 0.5 Pa VHS, dt = 5e-9 s, Poisson every 10 steps,
re-sort every 20. Synthetic, seeded inputs (no dataset is involved).

value: alive-particle steps processed in the K timed steps / device time of
those steps (CUDA events on the library's stream), inputs resident in HBM.
e2e:   the same metric through the C ABI with host buffers: upload of the
particle state from pinned memory, K steps with the per-step stats read
(the reference's stop check), download of the particles and surface counters.
roofline: the fused step kernel (push + walk + collide + settle), algorithmic
bytes = 112 B per alive particle + 152 B per occupied tet, over its
CUDA-event time; peak from MEASURED_PEAKS.json.
cpu_baseline / --impl reference: the FP64 CPU oracle (OpenMP restatement of
the reference step; the reference itself does not build here) on a bounded
sample of the same workload, all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "particle-steps/s @1e7 ptcl: mixed vs FP64 GPU at \u22641% deposit L1; grad/fwd cost"
UNIT = "particle-steps/s"


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def dist_info():
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names[1:], parts[5:9]):
                if val.lower() in ("active", "0x1", "1"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# dram__bytes_read.sum + dram__bytes_write.sum of the step kernel and its walk kernel per alive
# particle, workload 1 geometry, one ncu --set full capture at 4e6 particles (FP64: 229.1 + 151.4
# MB for k_step64, 71.27 + 1.472 MB for k_walk_queue64; mixed: 128.2 + 40.67 MB for k_step32,
# 53.52 + 1.419 MB for k_walk_queue32)
STEP_TRAFFIC_B = {
    "64": (453.2e6 / 4e6, "ncu capture of k_step64 + k_walk_queue64 at 4e6 particles, scaled by particles"),
    "32": (223.8e6 / 4e6, "ncu capture of k_step32 + k_walk_queue32 at 4e6 particles, scaled by particles"),
}
# The resource that binds the step kernels is not HBM: the FP64 form's step is
# FP64-issue-bound (GB300 issues about 2 FP64 thread-ops per clock per SM),
# the FP32 form's is memory-latency-bound. Pipe utilisation from the same
# captures (sm__pipe_fp64_cycles_active, % of peak sustained active).
STEP_BINDING = {
    "64": {"resource": "fp64 pipe", "k_step64": 0.783, "k_walk_queue64": 0.589,
           "source": "ncu --set full, k_step64 + k_walk_queue64 at 4e6 particles"},
    "32": {"resource": "memory latency (long-scoreboard stalls; fp64 pipe 0 in k_step32)",
           "k_step32_issue_active": 0.434, "k_step32_warps_active": 0.482,
           "source": "ncu --set full, k_step32 + k_walk_queue32 at 4e6 particles"},
}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback 6.8 TB/s"


def build_workload(args):
    from start_gb300.workloads import workload1, workload3

    if args.workload == 3:
        # jittered 200 x 200 x 100 mm box with two plate electrodes, VSS argon 2 Pa
        n = args.particles if args.particles != 10_000_000 else 50_000_000
        w = workload3(n_particles=n, seed=0, steps=args.warmup + args.steps)
    else:
        w = workload1(n_particles=args.particles, cells=args.cells, seed=0, steps=args.warmup + args.steps)
    w.params["precision"] = 1 if args.precision == "mixed" else 0
    w.params["preconditioner"] = {"jacobi": 0, "amg": 1, "amg32": 2}[args.precond]
    if args.resort_every is not None:
        w.params["resort_every"] = args.resort_every
    return w


def cpu_sample(w, n_sample, steps, warmup=0, threads=None, want_state=False, timed_threads=None):
    """Times the CPU oracle on the first n_sample particles of the workload:
    one untimed deposit + cold solve and `warmup` untimed steps, then `steps`
    timed steps of the full loop (deposit + warm PCG every poisson_every
    steps, push/walk/collide/settle every step), as the GPU arm does.
    timed_threads: thread count of the timed steps only (the untimed ones use
    `threads`)."""
    import oracle

    prev = oracle.get_threads()
    if threads:
        oracle.set_threads(threads)
    t0 = time.perf_counter()
    o = oracle.Oracle(w.mesh, w.params)
    t_setup = time.perf_counter() - t0
    o.set_particles(w.pos[:n_sample], w.vel[:n_sample])
    if warmup > 0:
        o.run(warmup, raise_on_nonconvergence=False)
    s0 = o.stats()["particle_steps"]
    if timed_threads:
        oracle.set_threads(timed_threads)
    t0 = time.perf_counter()
    o.run(steps, raise_on_nonconvergence=False)
    dt = time.perf_counter() - t0
    st = o.stats()
    info = dict(setup_s=t_setup, timed_s=dt, particle_steps=st["particle_steps"] - s0, threads=oracle.get_threads())
    if want_state:
        info["state"] = {"counts": o.triangle_counts(), "stats": st, "tet": o.particles()["tet"]}
    o.close()
    oracle.set_threads(prev)
    return (st["particle_steps"] - s0) / dt, info


def cpu_sample_desc(w, n_sample, steps, warmup):
    who = "all" if n_sample >= len(w.pos) else f"{n_sample} of"
    return (f"{who} {len(w.pos)} particles on the full mesh, {warmup} untimed + {steps} timed full-loop steps "
            f"(deposit + warm PCG every {w.params['poisson_every']} steps, push/walk/collide/settle every step)")


def host_cpu():
    """CPU model string, logical cores and OMP_NUM_THREADS of this host."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        import platform

        model = platform.processor() or platform.machine()
    return {"cpu_model": model, "nproc": os.cpu_count(), "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS")}


def surface_bins(mesh, patch=0.01):
    """Bin of each surface triangle: its surface tag x patch-sized squares."""
    lo = mesh.nodes.min(0)
    n = int(np.ceil(float(np.max(mesh.nodes.max(0) - lo)) / patch))
    ij = np.floor((mesh.triangle_centroids() - lo) / patch).astype(np.int64).clip(0, n - 1)
    key = mesh.tri_tag.astype(np.int64) * n ** 3 + (ij * np.array([n * n, n, 1])).sum(1)
    return np.unique(key, return_inverse=True)[1]


def chi2_two_sample(a, b):
    """Chi-square two-sample test of two histograms (bins empty in both dropped)."""
    from scipy import stats

    a, b = np.asarray(a, float), np.asarray(b, float)
    keep = (a + b) > 0
    a, b = a[keep], b[keep]
    if len(a) < 2 or a.sum() == 0 or b.sum() == 0:
        return None, 0, None
    k1, k2 = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = float(np.sum((k1 * a - k2 * b) ** 2 / (a + b)))
    dof = len(a) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def compare_forms(ref, other):
    """Errors of one GPU state against another after the same steps: L1 error
    of the surface histogram over triangles, landing-position RMS over the
    particles settled in both, and the potential's max error."""
    cr, co = ref["counts"].astype(float), other["counts"].astype(float)
    both = ((ref["flags"] & 1) != 0) & ((other["flags"] & 1) != 0)
    d = other["pos"][both] - ref["pos"][both]
    return {"l1_hist_error": float(np.abs(co - cr).sum() / max(cr.sum(), 1.0)),
            "landing_rms_m": float(np.sqrt(np.mean(np.sum(d * d, axis=1)))) if both.any() else None,
            "landed_in_both": int(both.sum()),
            "phi_max_rel_error": float(np.max(np.abs(other["phi"] - ref["phi"])) /
                                       max(float(np.max(np.abs(ref["phi"]))), 1e-300)),
            "settled_ref": int(cr.sum()), "settled_other": int(co.sum())}


def gpu_state(eng):
    p = eng.particles()
    return {"counts": eng.triangle_counts(), "pos": p["pos"], "flags": p["flags"], "tet": p["tet"],
            "phi": eng.potential(), "stats": eng.stats()}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    w = build_workload(args)
    n_sample = min(args.cpu_sample or len(w.pos), len(w.pos))
    steps = args.cpu_steps or args.steps
    v, info = cpu_sample(w, n_sample, steps, args.warmup)
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * info["timed_s"] / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded workload generator)",
        "config": config_dict(args, w),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": info.get("threads"), "kind": "port",
                         "sample": cpu_sample_desc(w, n_sample, steps, args.warmup), "timed_s": info["timed_s"],
                         **host_cpu()},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference itself needs CGAL/Trilinos/Gmsh (absent); the timed CPU path is the FP64 "
                "OpenMP oracle port of its step",
    }
    print(json.dumps(line))
    return 0


def grad_leg(args, local):
    """Gradient of the smoothed landing objective (the 100 mm electrode cube at
    h = 4 mm, 1e6 Ti+, 300 steps, argon 1 Pa HS with collision events frozen,
    checkpoints every 32 steps): cost of forward + backward against one plain
    forward pass (set particles, electrode solve, 300 particle steps).

    Two configurations: the one the gradient is timed on (top electrode at
    +500 V turning the ions back onto z = 0, target the centre of the bottom
    face), and the configuration as stated (six potentials uniform in
    [-100, 100] V drawn with seed 1, target the centre of the z = 100 mm face),
    where almost no ion lands within 300 steps. On the first, central
    differences of the live forward pass (h = 1e-3 V, 1e-4 rad) are set against
    the pathwise gradient: their gap is the contribution of the per-cell field
    jumps that the pathwise derivative leaves out."""
    import torch

    from start_gb300.adjoint import LandingProblem

    V = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 500.0])
    a0 = np.deg2rad(30.0)
    lp = LandingProblem(n_particles=args.grad_particles, steps=300, collisions=True)
    e = lp.engine

    def plain_forward(Vx):
        e.set_dirichlet(lp.dirichlet_values(Vx))
        x0, v0, _, _ = lp.initial_state(a0)
        e.set_particles(x0, v0)
        e.solve(np.zeros(lp.mesh.n_nodes))
        e.process(lp.steps)
        e.synchronize()

    def timed(f, reps=3):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = f()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3, out

    def measure(Vx, target):
        lp.target = np.asarray(target, float)
        plain_forward(Vx)
        lp.forward(Vx, a0)
        if lp._last[2] > 0:
            lp.backward()  # warm-up (allocations, graphs)
        t_plain, _ = timed(lambda: plain_forward(Vx))
        t_fwd, J = timed(lambda: lp.forward(Vx, a0))
        n_landed = int(lp._last[2])
        if n_landed == 0:  # nothing to differentiate: J = 0 for every parameter near these
            return {"electrodes_V": np.asarray(Vx).tolist(), "target": lp.target.tolist(), "J": J,
                    "n_landed": 0, "plain_forward_ms": t_plain, "grad_forward_ms": t_fwd}
        t_bwd, (dV, da, iters) = timed(lp.backward)
        return {"electrodes_V": np.asarray(Vx).tolist(), "target": lp.target.tolist(), "J": J,
                "n_landed": n_landed, "dJ_dV": dV.tolist(), "dJ_dalpha": da, "adjoint_cg_iters": iters,
                "plain_forward_ms": t_plain, "grad_forward_ms": t_fwd, "backward_ms": t_bwd,
                "cost_ratio": (t_fwd + t_bwd) / t_plain}

    out = {"workload": "cube100mm_h4mm_1e6ptcl_grad", "n_particles": int(args.grad_particles), "steps": 300,
           "checkpoint_every": lp.every, "half_angle_deg": 30.0, "sigma_m": lp.sigma,
           "timing": "host wall clock, median of 3, synchronised"}
    out.update(measure(V, (0.05, 0.05, 0.0)))
    # the same with the recovered field's gradient in the backward pass
    e.grad_field_gradient(True)
    fg = measure(V, (0.05, 0.05, 0.0))
    e.grad_field_gradient(False)
    out["field_gradient"] = {k: fg[k] for k in ("dJ_dV", "dJ_dalpha", "grad_forward_ms", "backward_ms", "cost_ratio")}
    if not args.no_grad_fd:
        grads = {"pathwise": (out["dJ_dV"], out["dJ_dalpha"]), "field_gradient": (fg["dJ_dV"], fg["dJ_dalpha"])}
        out["live_fd"] = live_fd_gaps(lp, V, a0, grads, ((1e-3, 1e-4), (1.0, 1e-2)))
        # 400 steps without gas: every ion lands, so J's count does not change
        # under the perturbation, and no collision decision can flip; only
        # the per-cell field's jumps separate the live map from the gradients
        lq = LandingProblem(n_particles=args.grad_particles, steps=400, collisions=False)
        lq.target = np.array([0.05, 0.05, 0.0])
        gq = {}
        for name, on in (("pathwise", False), ("field_gradient", True)):
            lq.engine.grad_field_gradient(on)
            lq.forward(V, a0)
            dVq, daq, _ = lq.backward()
            gq[name] = (dVq.tolist(), daq)
        out["live_fd_400steps_no_gas"] = live_fd_gaps(lq, V, a0, gq, ((1.0, 1e-2),))
        out["live_fd_400steps_no_gas"]["n_landed"] = int(lq._last[2])
        lq.close()
    V_stated = np.random.default_rng(1).uniform(-100.0, 100.0, 6)
    out["as_stated"] = measure(V_stated, (0.05, 0.05, 0.1))
    lp.close()
    return out


def live_fd_gaps(lp, V, a0, grads, steps):
    """Central differences of the live forward pass (nothing frozen) against
    each gradient in grads ({name: (dJ/dV, dJ/dalpha)}), at each (h_V, h_rad)
    in steps. Small steps see few of the jumps the gradients leave out
    (pushes that change cell, collision decisions that flip, ions that land or
    not by the last step), each of which moves J by about 1/N; larger steps
    average over many."""
    res = {"note": "relative gap = max |fd - gradient| / max |fd| (potentials), |fd - gradient| / |fd| (alpha)"}
    for hv, ha in steps:
        fd = []
        for f in range(len(V)):
            dv = np.zeros(len(V))
            dv[f] = hv
            fd.append((lp.forward(V + dv, a0) - lp.forward(V - dv, a0)) / (2 * hv))
        fd = np.array(fd)
        fd_a = (lp.forward(V, a0 + ha) - lp.forward(V, a0 - ha)) / (2 * ha)
        r = {"dJ_dV": fd.tolist(), "dJ_dalpha": fd_a}
        for name, (dV, da) in grads.items():
            r[f"rel_gap_V_{name}"] = float(np.max(np.abs(fd - np.asarray(dV))) / np.max(np.abs(fd)))
            r[f"rel_gap_alpha_{name}"] = abs(fd_a - da) / abs(fd_a)
        res[f"h_{hv:g}V_{ha:g}rad"] = r
    return res


def config_dict(args, w):
    return {"workload": w.name, "n_particles": int(len(w.pos)), "n_tets": int(w.mesh.n_tets),
            "n_nodes": int(w.mesh.n_nodes), "n_triangles": int(w.mesh.n_triangles),
            "collision_model": {1: "HS", 2: "VHS", 3: "VSS"}.get(w.params["collision_model"], "none"),
            "poisson_every": w.params["poisson_every"],
            "resort_every": w.params["resort_every"], "dt": w.params["dt"], "precision": args.precision,
            "preconditioner": args.precond,
            "l2_policy": f"inputs larger than L2 (particles {len(w.pos) * 56 / 1e6:.0f} MB, "
                         f"mesh {w.mesh.n_tets * 200 / 1e9:.1f} GB)",
            "timed_steps_start_at": args.warmup}


def timed_steps(eng, stream, steps):
    """Device time (CUDA events on the library's stream) of `steps` steps of
    spg_run, with the alive-particle steps they processed."""
    import torch

    s0 = eng.stats()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    eng.run(steps, raise_on_nonconvergence=False)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    s1 = eng.stats()
    return ev0.elapsed_time(ev1), s1["particle_steps"] - s0["particle_steps"], s0, s1


def pinned_io(w):
    import torch

    n = len(w.pos)
    pos_h = torch.from_numpy(w.pos).pin_memory().numpy()
    vel_h = torch.from_numpy(w.vel).pin_memory().numpy()
    out = {"pos": torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy(),
           "vel": torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy(),
           "tet": torch.empty(n, dtype=torch.int32).pin_memory().numpy(),
           "flags": torch.empty(n, dtype=torch.int32).pin_memory().numpy().view(np.uint32)}
    return pos_h, vel_h, out


def e2e_leg(eng, w, steps, reference_calls):
    """A whole job through the C ABI with pinned host buffers: upload, `steps`
    steps with the per-step stats read (the reference's stop check), download
    of particles and counters; host wall clock. reference_calls: the steps go
    through the reference-named calls (spg_gather -> spg_solve every
    poisson_every steps with the density left on the GPU, spg_process every
    step), as the C++ shim's time loop makes them; otherwise spg_run(1)."""
    import torch

    pos_h, vel_h, out = pinned_io(w)
    every = w.params["poisson_every"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.set_particles(pos_h, vel_h)  # returns after the upload and the location
    t_up = time.perf_counter()
    s_start = eng.stats()["particle_steps"]
    t_first = None
    for k in range(steps):
        if reference_calls:
            if k % every == 0:
                eng.gather(want_rho=False)
                eng.solve(rho=None, want_phi=False, raise_on_nonconvergence=False)
            st = eng.process(1)  # returns the step's stats (D2H)
        else:
            st = eng.run(1, raise_on_nonconvergence=False)
        if t_first is None:
            t_first = time.perf_counter()
        if st["n_alive"] == 0:
            break
    t_steps = time.perf_counter()
    counts = eng.triangle_counts()
    eng.particles(out=out)  # D2H straight into the pinned arrays
    torch.cuda.synchronize()
    t_end = time.perf_counter()
    t = t_end - t0
    phases = {"upload_locate_ms": 1e3 * (t_up - t0), "first_step_ms": 1e3 * (t_first - t_up),
              "other_steps_ms": 1e3 * (t_steps - t_first), "download_ms": 1e3 * (t_end - t_steps)}
    ps = eng.stats()["particle_steps"] - s_start
    h2d = (pos_h.nbytes + vel_h.nbytes) / steps
    d2h = (sum(a.nbytes for a in out.values()) + counts.nbytes) / steps + 96
    calls = ("spg_set_particles; spg_gather(NULL) + spg_solve(NULL) every poisson_every steps, spg_process(1) "
             "every step; spg_get_triangle_counts, spg_get_particles" if reference_calls else
             "spg_set_particles; spg_run(1) per step; spg_get_triangle_counts, spg_get_particles")
    return {"value": ps / t, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "seconds": t,
            "phases_ms": phases, "calls": calls, "note": "job-level: upload, K steps from step 0 (cold first Poisson solve), "
                                    "per-step stats read, download; host wall clock"}


def run_gpu(args):
    import torch

    from start_gb300 import StartPIC

    rank, world, local = dist_info()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    W, K = args.warmup, args.steps
    w = build_workload(args)
    w.params["device"] = local
    eng = StartPIC(w.mesh, w.params)
    setup_ms = eng.setup_times()  # FEM set-up on the GPU, host mesh work, AMG hierarchy
    eng.set_particles(w.pos, w.vel)
    stream = torch.cuda.ExternalStream(eng.stream_ptr(), device=local)
    eng.run(W)
    eng.synchronize()
    # The timed steps run without the per-phase event profiler; the same steps
    # are then replayed from a checkpoint (bit-exact) with it for the breakdown.
    snap = eng.checkpoint()
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    ms, ps, st0, st1 = timed_steps(eng, stream, K)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    eng.restore(snap)
    del snap
    eng.profile_enable(True)
    eng.run(K, raise_on_nonconvergence=False)
    prof = eng.profile()
    eng.profile_enable(False)
    assert eng.stats()["particle_steps"] == st1["particle_steps"]
    state64 = gpu_state(eng)  # after W + K steps: parity against the oracle and the mixed form
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        c = torch.tensor([float(ps)], device="cuda")
        torch.distributed.all_reduce(c)
        ps = int(c.item())
    value = ps / (ms / 1e3)
    peak, peak_src = measured_peak()
    sfx = "32" if args.precision == "mixed" else "64"
    phases = {
        "step": (f"k_step{sfx} + k_walk_queue{sfx} (push, move, collide, walk, settle)", prof["step_ms"],
                 prof["step_bytes"], prof["step_launches"]),
        "pcg": ("PCG iterations (SELL-32 SpMV + dots, updates"
                + (", AMG V-cycle)" if args.precond != "jacobi" else ")"), prof["pcg_ms"], prof["pcg_bytes"],
                prof["pcg_iters"]),
        "deposit": (f"k_deposit{sfx} (fixed-point P1 deposit)", prof["deposit_ms"], prof["deposit_bytes"],
                    prof["deposit_launches"]),
    }
    dom = max(phases, key=lambda k: phases[k][1])
    name, dms, dbytes, dl = phases[dom]
    bw = dbytes / (dms / 1e3) / 1e9 if dms > 0 else None
    traffic, traffic_src = args.traffic, "--traffic" if args.traffic else None
    binding = None
    if traffic is None and dom == "step" and args.workload == 1:
        # DRAM bytes (read + write) of the step kernel pair per alive particle from one ncu capture
        # of the same geometry at 4e6 particles, scaled by the particles one launch processes
        per_particle, src = STEP_TRAFFIC_B[sfx]
        traffic, traffic_src = per_particle * ps / max(1, K), src
        binding = STEP_BINDING[sfx]
    roof = {"kernel": name, "phase": dom, "bound": "hbm", "achieved": bw, "peak": peak, "unit": "GB/s",
            "frac": (bw / peak) if bw else None, "traffic": traffic, "traffic_source": traffic_src,
            "peak_source": peak_src, "bytes_per_launch": dbytes / max(1, dl), "ms_per_launch": dms / max(1, dl)}
    if binding:
        roof["binding"] = binding
    for k, (nm, ms_k, b_k, l_k) in phases.items():
        roof[f"{k}_GBps"] = b_k / (ms_k / 1e3) / 1e9 if ms_k > 0 else None
    breakdown = {k: prof[k] for k in ("step_ms", "deposit_ms", "pcg_ms", "efield_ms", "sort_ms")}
    breakdown["pcg_iters"] = prof["pcg_iters"]
    breakdown["pcg_GBps"] = prof["pcg_bytes"] / (prof["pcg_ms"] / 1e3) / 1e9 if prof["pcg_ms"] > 0 else None
    breakdown["deposit_GBps"] = (prof["deposit_bytes"] / (prof["deposit_ms"] / 1e3) / 1e9
                                 if prof["deposit_ms"] > 0 else None)
    breakdown["occupied_tets"] = prof["occupied_tets"]

    # the configured run length of the mixed-form comparison (1,000 steps):
    # both forms continue from their W + K state, untimed
    acc_steps = max(args.accuracy_steps, W + K)
    state64_long = None
    if not args.no_mixed and not args.no_accuracy and acc_steps > W + K:
        eng.run(acc_steps - W - K, raise_on_nonconvergence=False)
        state64_long = gpu_state(eng)

    e2e = e2e_ref = None
    if not args.no_e2e:
        e2e = e2e_leg(eng, w, K, reference_calls=False)
        e2e_ref = e2e_leg(eng, w, K, reference_calls=True)
    eng.close()

    mixed = None
    if not args.no_mixed:
        # The mixed-precision form on the same inputs and steps: throughput,
        # and its errors against the FP64 form after the same W + K steps and
        # after the configured 1,000 steps.
        wm = build_workload(args)
        wm.params["device"] = local
        wm.params["precision"] = 1
        em = StartPIC(wm.mesh, wm.params)
        em.set_particles(wm.pos, wm.vel)
        sm_ = torch.cuda.ExternalStream(em.stream_ptr(), device=local)
        em.run(W)
        em.synchronize()
        msnap = em.checkpoint()
        mms, mps, _, _ = timed_steps(em, sm_, K)
        em.restore(msnap)
        em.profile_enable(True)
        em.run(K, raise_on_nonconvergence=False)
        mp = em.profile()
        em.profile_enable(False)
        mstate = gpu_state(em)
        # the same steps one launch per step (no segments): time and identity
        em.restore(msnap)
        del msnap
        em.set_step_segments(1)
        sms_, sps_, _, _ = timed_steps(em, sm_, K)
        sstate = gpu_state(em)
        em.set_step_segments(32)
        single = {"ms_per_step": sms_ / K, "value": sps_ / (sms_ / 1e3),
                  "identical_to_segments": bool(all(np.array_equal(mstate[k], sstate[k])
                                                    for k in ("counts", "pos", "flags", "tet", "phi"))
                                                and mstate["stats"] == sstate["stats"])}
        cmp_short = compare_forms(state64, mstate)
        mval = mps / (mms / 1e3)
        mixed = {"value": mval, "unit": UNIT, "ms_per_step": mms / K, "speedup_vs_fp64": mval / value,
                 "l1_hist_error_vs_fp64": cmp_short["l1_hist_error"],
                 "landing_rms_m_vs_fp64": cmp_short["landing_rms_m"], "landed_in_both": cmp_short["landed_in_both"],
                 "phi_max_rel_error_vs_fp64": cmp_short["phi_max_rel_error"],
                 "settled_fp64": cmp_short["settled_ref"], "settled_mixed": cmp_short["settled_other"],
                 "compared_after_steps": W + K,
                 "breakdown_ms": {k: mp[k] for k in ("step_ms", "deposit_ms", "pcg_ms", "efield_ms", "sort_ms")},
                 "pcg_iters": mp["pcg_iters"],
                 "step_GBps": mp["step_bytes"] / (mp["step_ms"] / 1e3) / 1e9 if mp["step_ms"] > 0 else None,
                 "step_GBps_note": ("algorithmic bytes of one step per particle-step (the state read and "
                                    "written, the occupied tets' records); the segmented step moves the "
                                    "state once per segment, so this effective rate exceeds its DRAM "
                                    "traffic (profiles/k_seg32_w1_4e6ptcl.md)"),
                 "pcg_GBps": mp["pcg_bytes"] / (mp["pcg_ms"] / 1e3) / 1e9 if mp["pcg_ms"] > 0 else None,
                 "gpu_launches": mp["kernel_launches"],
                 "one_launch_per_step": single,
                 "dtype": ("f32 state/push/V-cycle, f64 PCG SpMV + vectors + sums" if args.precond != "jacobi"
                           else "f32 state/push/SpMV, f64 refinement + sums")}
        if state64_long is not None:
            em.run(acc_steps - W - K, raise_on_nonconvergence=False)
            acc = compare_forms(state64_long, gpu_state(em))
            acc["steps"] = acc_steps
            acc["bar"] = "l1_hist_error <= 0.01"
            acc["pass"] = acc["l1_hist_error"] <= 0.01
            mixed["accuracy_full_run"] = acc
        em.close()

    fp64_amg = None
    if not args.no_fp64_amg and args.precond == "amg32" and args.precision == "fp64":
        # FP64 throughout: the same FP64 step with the V-cycle in FP64 too
        wa = build_workload(args)
        wa.params["device"] = local
        wa.params["preconditioner"] = 1
        ea = StartPIC(wa.mesh, wa.params)
        ea.set_particles(wa.pos, wa.vel)
        sa = torch.cuda.ExternalStream(ea.stream_ptr(), device=local)
        ea.run(W)
        ams, aps, _, ast1 = timed_steps(ea, sa, K)
        cmp_a = compare_forms(state64, gpu_state(ea))
        aval = aps / (ams / 1e3)
        fp64_amg = {"value": aval, "unit": UNIT, "ms_per_step": ams / K, "preconditioner": "amg (FP64 V-cycle)",
                    "cg_iters_total": ast1["cg_iters_total"], "l1_hist_error_vs_amg32": cmp_a["l1_hist_error"],
                    "phi_max_rel_error_vs_amg32": cmp_a["phi_max_rel_error"]}
        if mixed:
            mixed["speedup_vs_fp64_amg"] = mixed["value"] / aval
        ea.close()

    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        n_sample = min(args.cpu_sample or len(w.pos), len(w.pos))
        steps = args.cpu_steps or K
        full = n_sample == len(w.pos) and steps == K
        v, info = cpu_sample(w, n_sample, steps, W, want_state=full)
        cpu = {"value": v, "unit": UNIT, "cores": info["threads"], "kind": "port",
               "sample": cpu_sample_desc(w, n_sample, steps, W), "timed_s": info["timed_s"],
               "setup_s": info["setup_s"], **host_cpu()}
        if full:
            # the headline run against the oracle on the identical workload and steps
            so = info["state"]
            inv = surface_bins(w.mesh, 0.01)
            chi2, dof, p = chi2_two_sample(np.bincount(inv, weights=state64["counts"].astype(float)),
                                           np.bincount(inv, weights=so["counts"].astype(float)))
            cg_, co_ = state64["stats"]["collisions"], so["stats"]["collisions"]
            parity = {"vs": "FP64 CPU oracle, same workload and seeds", "steps": W + K,
                      "gpu_preconditioner": args.precond, "oracle_solver": "Jacobi PCG",
                      "chi2_p": p, "chi2": chi2, "chi2_dof": dof, "bins": "surface tag x 10 mm squares",
                      "collisions_gpu": int(cg_), "collisions_oracle": int(co_),
                      "collisions_ratio": cg_ / co_ if co_ else None,
                      "settled_gpu": int(state64["counts"].sum()), "settled_oracle": int(so["counts"].sum()),
                      "identical_tet_fraction": float(np.mean(state64["tet"] == so["tet"])),
                      "bars": "chi2_p > 0.01, collisions within 5 %"}
            parity["pass"] = bool(p is not None and p > 0.01 and abs(cg_ - co_) <= 0.05 * max(co_, 1))
        if not args.no_cpu1:
            # one core, a bounded sample: a tenth of the particles, W untimed
            # steps on all cores (the cold solve), then 10 timed steps with one
            # warm solve on one core
            n1 = min(len(w.pos), max(1, len(w.pos) // 10))
            v1, i1 = cpu_sample(w, n1, 10, W, timed_threads=1)
            cpu["one_core"] = {"value": v1, "unit": UNIT, "cores": i1["threads"],
                               "sample": cpu_sample_desc(w, n1, 10, W), "timed_s": i1["timed_s"]}

    grad = None
    if not args.no_grad and rank == 0:
        grad = grad_leg(args, local)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded workload generator)", "config": config_dict(args, w),
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "e2e_reference_calls": e2e_ref, "clocks": clk,
            "gpu_launches": prof["kernel_launches"], "breakdown_ms": breakdown, "parity": parity,
            "mixed": mixed, "fp64_amg": fp64_amg, "grad": grad,
            "alive_particles": {"start": st0["n_alive"], "end": st1["n_alive"]},
            "setup_ms": setup_ms,
            "cg_iters_last": st1["cg_iters_last"],
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", type=int, default=1, choices=[1, 3],
                    help="1: 200 mm Kuhn cube, 1e7 ions (headline); 3: jittered plate box, 5e7 ions")
    ap.add_argument("--particles", type=int, default=10_000_000)
    ap.add_argument("--cells", type=int, default=100)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--precond", default="amg32", choices=["jacobi", "amg", "amg32"],
                    help="Poisson PCG preconditioner (both forms)")
    ap.add_argument("--resort-every", type=int, default=None,
                    help="steps between tet re-sorts of the particles (default: the workload's)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="particles in the CPU sample (0: all)")
    ap.add_argument("--cpu-steps", type=int, default=0, help="timed CPU steps (0: --steps)")
    ap.add_argument("--no-grad", action="store_true", help="skip the gradient leg")
    ap.add_argument("--grad-particles", type=int, default=1_000_000)
    ap.add_argument("--no-grad-fd", action="store_true", help="skip the live-map finite differences")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the untimed FP64-vs-mixed comparison over the configured run length")
    ap.add_argument("--accuracy-steps", type=int, default=1000, help="steps of that comparison")
    ap.add_argument("--no-fp64-amg", action="store_true", help="skip the FP64-V-cycle leg")
    ap.add_argument("--no-cpu1", action="store_true", help="skip the one-core CPU sample")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per launch of the step kernel, if captured")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
