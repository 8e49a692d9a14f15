"""Benchmark of the per-step SPH hot path on GB300.

A "step" is one global-timestep leapfrog step (step_leapfrog.f90:91-760) of
the whole particle set: tree build, density h-rho iterations, EOS, force
pair loop (with any velocity iterations) and the kick-drift-kick update.

Default workload: the Sedov blast set, 128^3 = 2,097,152 particles on a
jittered lattice in a periodic [-0.5,0.5)^3 box (seeded synthetic input; no
public dataset exists for this path). Its working set (~1 GB) is far larger
than the 129 MB L2, so no L2 flush is needed between steps.

Lines (one JSON line from rank 0):
  * our arm (default --precision both): the FP64 form and the mixed form run
    on the same input; value = particle-steps/s of the mixed form with inputs
    resident in HBM (device time from CUDA events on the library's stream),
    with the FP64 form's rate, their ratio and the mixed form's acceleration
    error beside it; e2e = each form through the C ABI with pinned host
    buffers (state upload, step, state download per step); momentum and
    energy conservation over the timed steps; roofline of the dominant
    kernel; cpu_baseline from the CPU oracle on the same steps;
  * beside them (`configs`): the other benchmark configurations - hydro 64^3
    (one evaluation + 10 steps), ideal MHD 128^3, the self-gravitating cloud
    of 2^21 particles - each in both forms with conservation and both forms'
    errors against the FP64 oracle on every particle, and the Sedov set's
    full 200 steps in both forms;
  * beside them (Sedov workloads): individual timesteps on the same set, one
    dtmax interval (dtmax = 2^5 x the first global dt), against the global
    scheme stepping every particle at the smallest bin's dt;
  * --impl reference: the CPU oracle (C++ OpenMP restatement of the reference
    Fortran; the reference cannot be compiled here) on all host cores.

Multi-GPU: the path runs as independent replicas (one per rank).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, 1 GB300: mixed vs FP64 at stated error; adjoint/forward ratio"
UNIT = "particle-steps/s"
# force pair loop, leaf-staged gather model (bytes): neighbour record read once
# per leaf trial entry, own record read + results written per particle
R_NB_FORCE = 72
R_OWN_FORCE = 72 + 40
# mixed form: positions FP64 (24 B), the rest of the neighbour record FP32
R_NB_FORCE_MIXED = 24 + 24
R_OWN_FORCE_MIXED = 24 + 64 + 40
# DRAM bytes (read + write) per particle of one k_force_mixed launch, from the
# ncu capture of the Sedov 96^3 case (profiles/pair_kernels_sedov96.md),
# scaled to the launch by the particle count
TRAFFIC_PER_PARTICLE_MIXED = (203.11e6 + 71.06e6) / 884736
TRAFFIC_SOURCE = ("scaled: ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_force_mixed launch on "
                  "Sedov 96^3 (profiles/pair_kernels_sedov96.md) x npart / 884,736")
# floating-point operations per particle of one force launch: thread-level
# SASS counts from ncu on the Sedov 96^3 case (profiles/flop_counts_sedov96.md;
# FP32 fadd + fmul + 2 ffma, FP64 dadd + dmul + 2 dfma), scaled to a launch by
# the particle count (the neighbours per particle do not depend on it)
FLOPS_PER_PARTICLE = {
    "k_force_mixed": {"fp32": (3759926183 + 3865459352 + 2 * 1511419870) / 884736, "fp64": 242924786 / 884736},
    "k_force": {"fp64": (1451552236 + 2536837906 + 2 * 1784275018) / 884736,
                "fp32": (1537615966 + 2704518873 + 2 * 948633950) / 884736},
}
# pipe peaks of one GB300 at its 2.07 GHz maximum SM clock: 152 SMs x 128 FP32
# or 2 FP64 lanes x 2 flops (an FMA-chain probe reaches 86 % and 95 % of them)
PEAK_TFLOPS = {"fp32": 152 * 128 * 2 * 2.07e9 / 1e12, "fp64": 152 * 2 * 2 * 2.07e9 / 1e12}
# the binding pipe of each force kernel as ncu sees it on the Sedov 96^3 case
# (profiles/flop_counts_sedov96.md, profiles/pair_kernels_sedov96.md): an FP64
# warp instruction holds the FP64 pipe whatever its active lanes, so the
# thread-level flop fraction understates the plain kernel's use of it
NCU_PIPES = {"k_force": {"fp64_pipe_active": 0.853, "issue_active": 0.117},
             "k_force_mixed": {"fp64_pipe_active": 0.326, "fma_pipe_active": 0.213, "issue_active": 0.541}}


def flop_roofline(kernel: str, n: int, ms_per_launch: float) -> dict:
    """Flop roofline of one force launch: the kernel's arithmetic pipe (FP32
    for the mixed form, FP64 for the plain path) against its peak."""
    fl = FLOPS_PER_PARTICLE[kernel]
    pipe = "fp32" if kernel == "k_force_mixed" else "fp64"
    out = {"kernel": kernel, "pipe": pipe, "unit": "TFLOP/s", "peak_source": "nominal (SM count x lanes x clock)"}
    for k, per in fl.items():
        out[k] = {"flops_per_launch": per * n, "achieved": per * n / (ms_per_launch / 1e3) / 1e12,
                  "peak": PEAK_TFLOPS[k]}
        out[k]["frac"] = out[k]["achieved"] / PEAK_TFLOPS[k]
    out["frac"] = out[pipe]["frac"]
    out["ncu_pipes"] = dict(NCU_PIPES[kernel], source="ncu, Sedov 96^3 launch (profiles/)")
    out["scaled_from"] = "ncu thread-level op counts of one Sedov 96^3 launch (profiles/), x npart / 884,736"
    return out


def workload(name: str):
    from phantom_gb300 import setups as S
    if name.startswith("sedov") and name.endswith("cd"):
        # the reference's default build: Cullen & Dehnen switch (nalpha = 3)
        n1d = int(name[5:-2] or 128)
        cfg, x, v, B = S.sedov(n1d)
        cfg = dict(cfg, nalpha=3, alpha=0.0, alphamax=1.0)
        return (f"sedov {n1d}^3 jittered lattice, periodic, gamma=5/3, hfact=1.2, C_cour=0.3, "
                "Cullen-Dehnen switch (alpha 0..1)"), (cfg, x, v, B)
    if name.startswith("sedov"):
        n1d = int(name[5:] or 128)
        return f"sedov {n1d}^3 jittered lattice, periodic, gamma=5/3, hfact=1.2, C_cour=0.3", S.sedov(n1d)
    if name == "hydro64":
        return "adiabatic hydro 64^3 jittered lattice, periodic, alpha=1 beta=2 alphau=1", S.hydro_lattice(64)
    if name == "mhd128":
        return "ideal MHD 128^3 jittered lattice with cleaning", S.mhd_vortex(128)
    if name.startswith("cloud"):
        n = {"cloud2m": 2 ** 21, "cloud256k": 2 ** 18, "cloud64k": 2 ** 16}.get(name)
        if n is None:
            raise SystemExit(f"unknown workload {name}")
        return (f"self-gravitating isothermal cloud, {n} particles uniform in a unit sphere, cs=0.2, "
                "Omega=0.5, theta=0.5 quadrupole tree gravity, open boundaries"), S.gravity_cloud(n)
    raise SystemExit(f"unknown workload {name}")


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("PH_BENCH_BACKEND", "") != "gloo" else "gloo"
        dist.init_process_group(backend=backend)
        return dist, rank, ws
    return None, 0, 1


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0])); smax = max(smax, float(f[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def cpu_oracle_rate(cfg, x, v, B, nthreads: int, nsteps: int = 1, warmup: int = 0):
    """Time the CPU oracle (OpenMP over leaf cells) on nsteps full leapfrog
    steps of the same particle set, after one untimed derivs and warmup
    untimed steps (so that the steps timed are the GPU arm's first ones)."""
    from oracle import oracle as O
    O.build()
    o = O.Oracle(cfg, nthreads=nthreads)
    o.set_particles(x, v, B)
    dt = o.derivs(1, 0.0)
    t = 0.0
    for _ in range(warmup):
        dtn, _, dterr = o.step(t, dt); t += dt; dt = min(dtn, dterr)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        dtn, its, dterr = o.step(t, dt)
        t += dt
        dt = min(dtn, dterr)
    el = time.perf_counter() - t0
    o.close()
    return len(x) * nsteps / el, el


def run_reference(args, dist, rank, ws):
    if rank != 0:
        return 0
    desc, (cfg, x, v, B) = workload(args.workload)
    nthreads = os.cpu_count() or 1
    from oracle import oracle as O
    O.build()
    o = O.Oracle(cfg, nthreads=nthreads)
    o.set_particles(x, v, B)
    dt = o.derivs(1, 0.0)
    t = 0.0
    for _ in range(args.warmup):
        dtn, _, dterr = o.step(t, dt); t += dt; dt = min(dtn, dterr)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dtn, _, dterr = o.step(t, dt); t += dt; dt = min(dtn, dterr)
    el = time.perf_counter() - t0
    n = len(x)
    value = n * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": desc, "npart": n, "precision": "fp64",
                   "parallelism": "openmp-cells"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} full leapfrog steps of the {n}-particle set"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def conservation_drift(c0, c1, pscale):
    """Momentum and energy conservation between two ph_conservation records
    (energies.f90:65-852: totmom :706, etot = ekin + etherm + emag + epot
    :691): the change of each momentum component against the scale of the
    momentum sum (sum m |v|, its rounding scale), and the relative change of
    the total energy."""
    e0 = float(c0[3] + c0[4] + c0[5] + c0[6])
    e1 = float(c1[3] + c1[4] + c1[5] + c1[6])
    dp = float(np.abs(np.asarray(c1[:3]) - np.asarray(c0[:3])).max())
    return {"momentum_start": [float(v) for v in c0[:3]], "momentum_end": [float(v) for v in c1[:3]],
            "momentum_change_over_sum_m_abs_v": dp / max(pscale, 1e-300),
            "etot_start": e0, "etot_end": e1, "etot_rel_change": abs(e1 - e0) / max(abs(e0), 1e-300),
            "components_end": {"ekin": float(c1[3]), "etherm": float(c1[4]), "emag": float(c1[5]),
                               "epot": float(c1[6])}}


def sum_m_abs_v(ctx, cfg):
    _, v, _ = ctx.download()
    return float(cfg["massoftype"] * np.abs(v[:, :3]).sum())


def time_arm(args, dist, ws, cfg, x, v, B, prec, local, e2e=True, steps=None, warmup=None, tune=True):
    """Warm-up, then K timed leapfrog steps with the state resident in HBM
    (device time from the library's CUDA events), momentum and energy
    conservation over those steps, then optionally the same K steps end to
    end through the C ABI with pinned host buffers."""
    import torch
    from phantom_gb300 import capi
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    n = len(x)
    ctx = capi.Context(cfg, precision=prec)
    if args.force_sym is not None:
        ctx.set_tune(force_sym=args.force_sym)
    ctx.upload(x, v, B)
    # warps per block of the pair and walk kernels tuned on this particle set
    # (no result changes; the leaf size stays the reference's minpart = 10)
    tuned = ctx.autotune() if (tune and not args.no_autotune) else ctx.tune()
    dt = ctx.derivs(1, 0.0)
    if cfg.get("nalpha", 0):
        ctx.alpha_initial()  # initial.F90:736-742
    t = 0.0
    for _ in range(warmup):
        dtn, _, dterr = ctx.step(t, dt); t += dt; dt = min(dtn, dterr)

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()
    mhd = bool(cfg["mhd"])
    snap = [pinned((n, 4), torch.float64), pinned((n, 4), torch.float64),
            pinned((n, 4), torch.float64) if mhd else None, pinned((n, 4), torch.float64),
            pinned((n, 4), torch.float64) if mhd else None, pinned(n, torch.float32)]
    ctx.download_state(*snap)
    t_snap, dt_snap = t, dt
    c0 = ctx.conservation()
    p0 = sum_m_abs_v(ctx, cfg)
    torch.cuda.synchronize(); barrier(dist)
    l0 = ctx.launches()
    dev_ms, kforce_ms, ktotal = 0.0, 0.0, np.zeros(8)
    trial_sum, pairs, its_tot = 0, 0, 0
    with ClockSampler(local) as clk:
        w0 = time.perf_counter()
        for _ in range(steps):
            dtn, its, dterr = ctx.step(t, dt)
            tm = ctx.timings()
            wc = ctx.work_counters()
            dev_ms += tm[7]; ktotal += tm; kforce_ms += tm[4]
            trial_sum += int(wc[0]); pairs += int(wc[2]); its_tot += its
            t += dt; dt = min(dtn, dterr)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    launches = ctx.launches() - l0
    barrier(dist)
    c1 = ctx.conservation()
    cons = conservation_drift(c0, c1, max(p0, sum_m_abs_v(ctx, cfg)))
    cons.update({"steps": steps, "t_start": t_snap, "t_end": t})
    dev_s = reduce_max(dist, dev_ms / 1e3)
    out = {"value": n * ws * steps / dev_s, "ms_per_step": dev_s * 1e3 / steps,
           "wall_ms_per_step": 1e3 * wall / steps, "launches": launches, "clocks": clk.summary(),
           "phases": (ktotal / steps).tolist(), "kforce_ms": kforce_ms, "its": its_tot,
           "trial_sum": trial_sum, "pairs": pairs, "tune": tuned, "conservation": cons}
    if e2e:
        host = [None if a is None else torch.from_numpy(a.copy()).pin_memory().numpy() for a in snap]
        # per step: xyzh, vxyzu, fxyzu (+ Bevol, dBevol) as (4,N) float64 and div v float32, each way
        out["h2d"] = out["d2h"] = n * 4 * 8 * (3 + (2 if mhd else 0)) + n * 4
        t, dt = t_snap, dt_snap
        barrier(dist)
        e0 = time.perf_counter()
        for _ in range(steps):
            ctx.upload_state(*host)
            dtn, its, dterr = ctx.step(t, dt)
            ctx.download_state(*host)
            t += dt; dt = min(dtn, dterr)
        e2e_s = reduce_max(dist, time.perf_counter() - e0)
        out["e2e"] = n * ws * steps / e2e_s
    ctx.close()
    return out


def time_eval_steps(cfg, x, v, B, prec, nsteps=10, reps=3):
    """One density + force evaluation then nsteps leapfrog steps from the
    initial state (the hydro 64^3 benchmark's definition), device time from
    the library's events: the median of reps runs after one untimed run."""
    from phantom_gb300 import capi
    n = len(x)
    ctx = capi.Context(cfg, precision=prec)
    runs = []
    for r in range(reps + 1):
        ctx.upload(x, v, B)
        dt = ctx.derivs(1, 0.0)
        tm = ctx.timings()
        ms = float(tm[0] + tm[1] + tm[2])
        c0 = ctx.conservation()
        p0 = sum_m_abs_v(ctx, cfg)
        t = 0.0
        its_tot = 0
        for _ in range(nsteps):
            dtn, its, dterr = ctx.step(t, dt)
            ms += float(ctx.timings()[7])
            its_tot += its
            t += dt; dt = min(dtn, dterr)
        cons = conservation_drift(c0, ctx.conservation(), max(p0, sum_m_abs_v(ctx, cfg)))
        if r > 0:
            runs.append((ms, its_tot, cons))
    ctx.close()
    runs.sort(key=lambda q: q[0])
    ms, its_tot, cons = runs[len(runs) // 2]
    cons.update({"steps": nsteps})
    return {"value": n * nsteps / (ms / 1e3), "ms_total": ms, "ms_per_step": ms / nsteps,
            "velocity_iterations_per_step": its_tot / nsteps, "conservation": cons,
            "definition": f"particle-steps/s = N x {nsteps} / (one derivs + {nsteps} leapfrog steps), median of {reps}"}


def flip_neighbourhood(cfg, xyzh, h, flipped):
    """Particles within the kernel reach of a flipped particle k
    (r < 2 max(h_k, h_j)): the forces a different h of k moves."""
    from scipy.spatial import cKDTree
    box = None
    pos = xyzh[:, :3]
    if cfg["periodic"]:
        box = np.array([cfg["xmax"] - cfg["xmin"], cfg["ymax"] - cfg["ymin"], cfg["zmax"] - cfg["zmin"]])
        pos = np.mod(pos - np.array([cfg["xmin"], cfg["ymin"], cfg["zmin"]]), box)
    tree = cKDTree(pos, boxsize=box)
    hmax = float(h.max())
    near = np.zeros(len(h), bool)
    for k in np.nonzero(flipped)[0]:
        cand = np.asarray(tree.query_ball_point(pos[k], 2.0 * hmax * 1.01), dtype=np.int64)
        d = pos[cand] - pos[k]
        if box is not None:
            d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(axis=1))
        near[cand[r < 2.0 * np.maximum(h[k], h[cand]) * 1.01]] = True
    return near


def oracle_errors(cfg, x, v, B, nthreads):
    """One derivs (tree, density, force) from the same state on the FP64
    oracle, the GPU FP64 path and the GPU mixed form, over every particle:
    max over particles of |a - a_oracle| / max |a_oracle| per component of
    fxyzu (and dB/dt with MHD), the largest relative difference of h, and the
    number of particles whose h differs by more than 1e-6 (a Newton-Raphson
    stopping test decided differently within the FP32 rounding of the mixed
    form's density sums, at the reference's tolh)."""
    from oracle import oracle as O
    from phantom_gb300 import capi
    t0 = time.perf_counter()
    o = O.Oracle(cfg, nthreads=nthreads)
    o.set_particles(x, v, B)
    o.derivs(1, 0.0)
    fo = o.get_force()
    ho_x = o.get_particles()[0]
    ho = ho_x[:, 3].copy()
    o.close()
    t_oracle = time.perf_counter() - t0
    ncomp = 3 if cfg["isothermal"] else 4
    res = {"oracle_derivs_s": t_oracle, "oracle_threads": nthreads,
           "measure": "max_i |f_i - f_oracle,i| / max_i |f_oracle,i| per component"}
    for prec, name in ((capi.PH_PREC_FP64, "fp64"), (capi.PH_PREC_MIXED, "mixed")):
        ctx = capi.Context(cfg, precision=prec)
        ctx.upload(x, v, B)
        ctx.derivs(1, 0.0)
        fg = ctx.force(2, 0.0)
        hg = ctx.download()[0][:, 3]
        ctx.close()

        def rel(a, b):
            s = float(np.abs(b).max())
            return 0.0 if s == 0.0 else float(np.abs(a - b).max() / s)
        e = {"fxyzu": [rel(fg["fxyzu"][:, c], fo["fxyzu"][:, c]) for c in range(ncomp)]}
        if cfg["mhd"]:
            e["dBevol"] = [rel(fg["dBevol"][:, c], fo["dBevol"][:, c]) for c in range(4)]
        if cfg["gravity"]:
            e["poten"] = rel(fg["poten"].astype(np.float64), fo["poten"].astype(np.float64))
        dh = np.abs(hg / ho - 1.0)
        e["h_max_rel"] = float(dh.max())
        flipped = dh > 1e-6
        e["particles_h_differ_1e-6"] = int(flipped.sum())
        e["accel_max_rel"] = max(e["fxyzu"][:3])
        if flipped.any():
            # the same measure over the particles outside the kernel reach of
            # every particle whose h-rho solve stopped one iteration apart
            keep = ~flip_neighbourhood(cfg, ho_x, ho, flipped)
            e["outside_flip_neighbourhoods"] = {
                "particles": int(keep.sum()),
                "fxyzu": [float(np.abs(fg["fxyzu"][keep, c] - fo["fxyzu"][keep, c]).max()
                                / max(np.abs(fo["fxyzu"][:, c]).max(), 1e-300)) for c in range(ncomp)]}
            if cfg["mhd"]:
                e["outside_flip_neighbourhoods"]["dBevol"] = [
                    float(np.abs(fg["dBevol"][keep, c] - fo["dBevol"][keep, c]).max()
                          / max(np.abs(fo["dBevol"][:, c]).max(), 1e-300)) for c in range(4)]
        res[name] = e
    return res


def mixed_error(cfg, x, v, B):
    """Error of the mixed form against the FP64 path on the full particle
    set: one derivs (tree, density, force) from the same state in each form;
    max over particles of |a_mixed - a_fp64| / max |a_fp64| per component (and
    du/dt), and the largest relative error of h. At the reference's tolh a
    cell whose h-rho iteration stops one Newton-Raphson step apart in the two
    forms keeps an h difference inside the tolerance band; the same measure
    with both forms converged to tolh = 1e-7 isolates the arithmetic error."""
    from phantom_gb300 import capi

    def one(c):
        res = {}
        for prec in (capi.PH_PREC_FP64, capi.PH_PREC_MIXED):
            ctx = capi.Context(c, precision=prec)
            ctx.upload(x, v, B)
            ctx.derivs(1, 0.0)
            f = ctx.force(2, 0.0)["fxyzu"]
            xo, _, _ = ctx.download()
            res[prec] = (f, xo[:, 3].copy())
            ctx.close()
        (f64, h64), (fmx, hmx) = res[capi.PH_PREC_FP64], res[capi.PH_PREC_MIXED]
        acc = max(float(np.abs(fmx[:, k] - f64[:, k]).max() / max(np.abs(f64[:, k]).max(), 1e-300))
                  for k in range(3))
        da = np.linalg.norm(fmx[:, :3] - f64[:, :3], axis=1) / max(np.linalg.norm(f64[:, :3], axis=1).max(), 1e-300)
        du = (float(np.abs(fmx[:, 3] - f64[:, 3]).max() / np.abs(f64[:, 3]).max())
              if np.abs(f64[:, 3]).max() > 0 else 0.0)
        dh = np.abs(hmx / h64 - 1.0)
        return acc, float(np.sqrt(np.mean(da ** 2))), du, float(dh.max()), int((dh > 1e-6).sum())

    acc, rms, du, dh, nflip = one(cfg)
    tight = dict(cfg); tight["tolh"] = 1.0e-7
    acc_c, rms_c, du_c, dh_c, _ = one(tight)
    return {"accel_max_rel": acc, "accel_rms_rel": rms, "dudt_max_rel": du, "h_max_rel": dh,
            "particles_h_differ_1e-6": nflip, "tolh": cfg["tolh"],
            "converged_tolh_1e-7": {"accel_max_rel": acc_c, "accel_rms_rel": rms_c, "dudt_max_rel": du_c,
                                    "h_max_rel": dh_c},
            "reference": "FP64 GPU path on the same input (matches the FP64 oracle to 1e-10 on the test sets)",
            "target": 1.0e-5}


def adjoint_ratio(n1d: int = 128, reps: int = 3):
    """Cost of the adjoint of one derivs evaluation (ph_adjoint: tree,
    density and force lists recomputed at the uploaded state, then the two
    adjoint pair passes) over the forward derivs evaluation (tree, density,
    force), device time from the library's CUDA events, on the adiabatic
    hydro lattice (alpha=1, beta=2, alpha_u=1) at n1d^3 particles. Both FP64."""
    from phantom_gb300 import capi, setups as S
    cfg, x, v, B = S.hydro_lattice(n1d)
    n = len(x)
    w = np.random.default_rng(0).standard_normal((n, 4))
    out = {"workload": f"hydro lattice {n1d}^3 ({n} particles)", "target": 3.0,
           "gradients": "d(sum w . fxyzu)/d(x, v, u) of one derivs; rollouts chain one adjoint per force evaluation"}
    for prec, name in ((capi.PH_PREC_FP64, "fp64"), (capi.PH_PREC_MIXED, "mixed")):
        ctx = capi.Context(cfg, precision=prec)
        fw, bw = [], []
        for r in range(reps + 1):
            ctx.upload(x, v, B)
            ctx.derivs(1, 0.0)
            tm = ctx.timings()
            f_ms = tm[0] + tm[1] + tm[2]
            ctx.upload(x, v, B)
            ctx.adjoint(w)
            a_ms = ctx.timings()[7]
            if r > 0:
                fw.append(f_ms); bw.append(a_ms)
        ctx.close()
        f, a = statistics.median(fw), statistics.median(bw)
        out[name] = {"forward_ms": f, "adjoint_ms": a, "ratio": a / f}
    out["ratio"] = out["fp64"]["ratio"]
    return out


def rollout_adjoint_timing(n1d: int = 128, nsteps: int = 16, ckpt: int = 4, reps: int = 2):
    """The benchmark's adjoint configuration: the adiabatic hydro lattice
    (alpha=1, beta=2, alpha_u=1) at n1d^3 particles, L = sum w . a after a
    16-step leapfrog rollout (fixed timestep: the first derivs' dt), w ~ N(0,1)
    seeded, checkpoints every 4 steps, through ph_rollout_adjoint on the
    device: the reverse pass (segment recomputes from the checkpoints and one
    adjoint per force evaluation) over the forward rollout (one derivs and
    the steps), device time from the library's events, median of reps, for
    the precision form (the configuration's) and the FP64 form."""
    from phantom_gb300 import capi, setups as S
    cfg, x, v, B = S.hydro_lattice(n1d)
    n = len(x)
    w = np.zeros((n, 4))
    w[:, :3] = np.random.default_rng(0).standard_normal((n, 3))
    out = {"workload": f"hydro lattice {n1d}^3 ({n} particles), alpha=1 beta=2 alphau=1",
           "steps": nsteps, "checkpoint_every": ckpt, "target": 3.0,
           "definition": "reverse pass (segment recomputes + adjoints) / forward rollout (derivs + steps)"}
    for prec, name in ((capi.PH_PREC_MIXED, "mixed"), (capi.PH_PREC_FP64, "fp64")):
        ctx = capi.Context(cfg, precision=prec)
        ctx.upload(x, v, B)
        dt = ctx.derivs(1, 0.0)
        fw, bw, adj, rec = [], [], [], []
        for r in range(reps + 1):
            ctx.upload(x, v, B)
            ctx.rollout_adjoint([dt] * nsteps, w, ckpt=ckpt)
            tm = ctx.timings()
            if r > 0:
                fw.append(tm[0]); bw.append(tm[1]); adj.append(tm[2]); rec.append(tm[3])
        ctx.close()
        f, b = statistics.median(fw), statistics.median(bw)
        out[name] = {"forward_ms": f, "reverse_ms": b, "reverse_adjoints_ms": statistics.median(adj),
                     "reverse_recompute_ms": statistics.median(rec), "ratio": b / f}
    out["ratio"] = out["mixed"]["ratio"]
    return out


def revtree_timing(cfg, x, v, B, reps=5):
    """revtree (tree refit, kdtree.F90:1851-2037) against maketree on the same
    particle set: device times of the refit and of the full build (median of
    reps), as the reference's kdtree test reports their ratio."""
    import statistics
    from phantom_gb300 import capi
    ctx = capi.Context(cfg)
    ctx.upload(x, v, B)
    mk, rv = [], []
    for _ in range(reps + 1):
        ctx.build_tree()
        mk.append(ctx.timings()[0])
    xw, _, _ = ctx.download()
    for _ in range(reps + 1):
        ctx.revtree(xw)
        rv.append(ctx.timings()[0])
    ctx.close()
    mk, rv = statistics.median(mk[1:]), statistics.median(rv[1:])
    return {"maketree_ms": mk, "revtree_ms": rv, "ratio": rv / mk}


def ind_timing(cfg, x, v, B, prec, global_ms_per_step, nbins=5, max_sub=512):
    """Individual timesteps on the same particle set: dtmax = 2^nbins times
    the global step of the first derivs, so the blast's particles spread over
    the bins while the cold background sits in the lowest. One dtmax interval
    untimed, then one timed (device time of each substep from the library's
    events). The global scheme advances the same interval in 2^nbinmax steps
    of every particle at global_ms_per_step each."""
    from phantom_gb300 import capi
    ctx = capi.Context(cfg, precision=prec)
    ctx.upload(x, v, B)
    dt0 = ctx.derivs(1, 0.0)
    ctx.close()
    dtmax = dt0 * 2 ** nbins
    c2 = dict(cfg, ind_timesteps=1, dtmax=dtmax)
    ctx = capi.Context(c2, precision=prec)
    ctx.upload(x, v, B)
    ctx.derivs(1, 0.0)
    if cfg.get("nalpha", 0):
        ctx.alpha_initial()
    ctx.ind_init(0.0)
    t = 0.0
    for _ in range(max_sub):  # warm-up interval
        t, _ = ctx.ind_substep(t)
        if ctx.ind_counters()[1] == 0:
            break
    nb_start = ctx.ind_counters()[0]
    dev_ms, nupd, nsub = 0.0, 0, 0
    l0 = ctx.launches()
    for _ in range(max_sub):
        t, na = ctx.ind_substep(t)
        dev_ms += float(ctx.timings()[7])
        nupd += na
        nsub += 1
        if ctx.ind_counters()[1] == 0:
            break
    launches = ctx.launches() - l0
    b, _, (nbinmax, _, _) = ctx.ind_state()
    hist = np.bincount(b.astype(np.int64), minlength=nbinmax + 1).tolist()
    ctx.close()
    n = len(x)
    glob_ms = (2 ** nb_start) * global_ms_per_step
    return {"workload": f"same particle set, ind_timesteps=1, dtmax = 2^{nbins} x first global dt ({dtmax:.3e})",
            "precision": "mixed" if prec == capi.PH_PREC_MIXED else "fp64",
            "substeps": nsub, "nbinmax": nb_start, "bins_at_end": hist, "particle_updates": nupd,
            "updates_per_particle": nupd / n, "ms_interval": dev_ms, "ms_per_substep": dev_ms / max(nsub, 1),
            "particle_updates_per_s": nupd / max(dev_ms / 1e3, 1e-12), "gpu_launches": launches,
            "global_ms_same_interval": glob_ms, "speedup_vs_global": glob_ms / max(dev_ms, 1e-12)}


def config_block(args, cfg, x, v, B, local, nthreads, eval_steps=None):
    """One benchmark configuration beside the headline: the FP64 and mixed
    rates on the same input (device time), conservation over the timed steps,
    and both forms' errors against the FP64 oracle on every particle."""
    from phantom_gb300 import capi
    out = {"npart": len(x)}
    for prec, name in ((capi.PH_PREC_FP64, "fp64"), (capi.PH_PREC_MIXED, "mixed")):
        if eval_steps:
            out[name] = time_eval_steps(cfg, x, v, B, prec, nsteps=eval_steps)
        else:
            r = time_arm(args, None, 1, cfg, x, v, B, prec, local, e2e=False, tune=False)
            out[name] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "gpu_launches": r["launches"],
                         "velocity_iterations_per_step": r["its"] / args.steps, "clocks": r["clocks"],
                         "k_force_ms_per_step": r["phases"][4], "conservation": r["conservation"],
                         "steps": args.steps, "warmup": args.warmup}
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    if not args.no_cpu:
        out["error_vs_oracle"] = oracle_errors(cfg, x, v, B, nthreads)
    return out


def run_ours(args, dist, rank, ws):
    import torch
    from phantom_gb300 import capi
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.adjoint_only:
        if rank == 0:
            print(json.dumps({"adjoint": adjoint_ratio(args.adjoint_n1d),
                              "adjoint_rollout": rollout_adjoint_timing(args.adjoint_n1d)}), flush=True)
        return 0
    desc, (cfg, x, v, B) = workload(args.workload)
    n = len(x)
    precs = {"fp64": [capi.PH_PREC_FP64], "mixed": [capi.PH_PREC_MIXED],
             "both": [capi.PH_PREC_FP64, capi.PH_PREC_MIXED]}[args.precision]
    arms = {}
    for prec in precs:
        arms[prec] = time_arm(args, dist, ws, cfg, x, v, B, prec, local, e2e=True)
    hp = precs[-1]
    h = arms[hp]
    mixed = hp == capi.PH_PREC_MIXED
    # ---- roofline of the dominant kernel (force pair loop), hbm model
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    nlaunch = max(h["its"], 1)  # one force evaluation per velocity iteration
    kf_per = h["kforce_ms"] / nlaunch / 1e3
    rnb, rown = (R_NB_FORCE_MIXED, R_OWN_FORCE_MIXED) if mixed else (R_NB_FORCE, R_OWN_FORCE)
    bytes_per_launch = (h["trial_sum"] / nlaunch) * rnb + n * rown
    achieved = bytes_per_launch / max(kf_per, 1e-12) / 1e9
    traffic = TRAFFIC_PER_PARTICLE_MIXED * n if (mixed and args.workload.startswith("sedov")) else None
    roof = {"bound": "hbm", "kernel": "k_force_mixed" if mixed else "k_force", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "traffic_source": TRAFFIC_SOURCE if traffic is not None else None,
            "peak_source": "measured" if peaks else "fallback",
            "model": f"leaf-staged gather: {rnb} B x trial entries + {rown} B x particles per launch",
            "algorithmic_bytes_per_launch": bytes_per_launch,
            "ms_per_launch": kf_per * 1e3, "launches_per_step": h["its"] / args.steps}
    flop_roof = flop_roofline("k_force_mixed" if mixed else "k_force", n, kf_per * 1e3)
    nth = os.cpu_count() or 1
    # ---- CPU baseline: oracle port on the host cores, a bounded sample of the
    # timed steps (the same warm-up, then the first steps the GPU arm times)
    cpu = None
    if rank == 0 and not args.no_cpu:
        ks = min(args.steps, args.cpu_steps)
        rate, el = cpu_oracle_rate(cfg, x, v, B, nth, nsteps=ks, warmup=args.warmup)
        cpu = {"value": rate, "unit": UNIT, "cores": nth, "kind": "port",
               "sample": (f"steps {args.warmup + 1}..{args.warmup + ks} of the same {n}-particle set (after one "
                          f"untimed derivs and {args.warmup} untimed steps, as the GPU arm), FP64, {el:.1f} s")}
    ph = h["phases"]
    line = {
        "metric": METRIC, "value": h["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": h["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": desc, "npart": n,
                   "precision": "mixed" if mixed else "fp64", "parallelism": f"replicas{ws}",
                   "launch": {k: h["tune"][k] for k in ("minpart", "dens_warps", "force_warps", "walk_warps")},
                   "l2": "working set >> 129 MB L2 (no flush needed)"},
        "e2e": {"value": h["e2e"], "unit": UNIT, "h2d_bytes_per_step": h["h2d"], "d2h_bytes_per_step": h["d2h"]},
        "roofline": roof,
        "flop_roofline": flop_roof,
        "cpu_baseline": cpu,
        "gpu_launches": h["launches"],
        "clocks": h["clocks"],
        "conservation": h["conservation"],
        "phases_ms_per_step": {"tree": ph[0], "density": ph[1], "force": ph[2], "integrate": ph[3],
                               "k_force": ph[4], "k_density": ph[5], "walks": ph[6], "step_total": ph[7]},
        "wall_ms_per_step": h["wall_ms_per_step"],
        "velocity_iterations_per_step": h["its"] / args.steps,
        "pairs_per_step": h["pairs"] / args.steps,
        "adjoint_over_forward": None,
    }
    if cpu:
        line["vs_cpu"] = {"mixed_device": h["value"] / cpu["value"] if mixed else None,
                          "mixed_e2e": h["e2e"] / cpu["value"] if mixed else None,
                          "note": "GPU rates over the CPU oracle's FP64 rate on the same steps"}
    if args.precision == "both" and ws == 1:
        line["revtree"] = revtree_timing(cfg, x, v, B)
    if not args.no_ind and args.workload.startswith("sedov") and ws == 1:
        line["individual_timesteps"] = ind_timing(cfg, x, v, B, hp, h["ms_per_step"])
    if args.precision == "both" and not args.no_adjoint and ws == 1:
        adj = adjoint_ratio(args.adjoint_n1d)
        ro = rollout_adjoint_timing(args.adjoint_n1d)
        line["adjoint_over_forward"] = ro["ratio"]
        line["adjoint"] = adj
        line["adjoint_rollout"] = ro
    if len(precs) == 2:
        f = arms[capi.PH_PREC_FP64]
        f_per_ms = f["kforce_ms"] / max(f["its"], 1)
        line["fp64"] = {"value": f["value"], "ms_per_step": f["ms_per_step"], "gpu_launches": f["launches"],
                        "clocks": f["clocks"], "k_force_ms_per_step": f["phases"][4],
                        "e2e": {"value": f["e2e"], "unit": UNIT, "h2d_bytes_per_step": f["h2d"],
                                "d2h_bytes_per_step": f["d2h"]},
                        "conservation": f["conservation"],
                        "velocity_iterations_per_step": f["its"] / args.steps,
                        "flop_roofline": flop_roofline("k_force", n, f_per_ms)}
        if cpu:
            line["vs_cpu"]["fp64_device"] = f["value"] / cpu["value"]
            line["vs_cpu"]["fp64_e2e"] = f["e2e"] / cpu["value"]
        line["mixed_over_fp64"] = h["value"] / f["value"]
        line["mixed_error"] = mixed_error(cfg, x, v, B)
        if ws == 1 and not args.no_configs:
            # the other benchmark configurations, and the headline set's full
            # step count, beside the headline line
            cfgs = {}
            if not args.no_cpu:
                cfgs[args.workload] = {"error_vs_oracle": oracle_errors(cfg, x, v, B, nth)}
            if args.workload == "sedov128":
                full = {}
                for prec, name in ((capi.PH_PREC_FP64, "fp64"), (capi.PH_PREC_MIXED, "mixed")):
                    r = time_arm(args, None, 1, cfg, x, v, B, prec, local, e2e=False, steps=200, warmup=0,
                                 tune=False)
                    full[name] = {"value": r["value"], "ms_per_step": r["ms_per_step"],
                                  "velocity_iterations_per_step": r["its"] / 200,
                                  "conservation": r["conservation"], "clocks": r["clocks"]}
                full["mixed_over_fp64"] = full["mixed"]["value"] / full["fp64"]["value"]
                full["definition"] = "the configuration's 200 steps from the initial derivs (device time)"
                cfgs["sedov128_200steps"] = full
            for name, es in (("hydro64", 10), ("mhd128", None), ("cloud2m", None)):
                if name == args.workload:
                    continue
                d, (c2, x2, v2, B2) = workload(name)
                blk = config_block(args, c2, x2, v2, B2, local, nth, eval_steps=es)
                blk["description"] = d
                cfgs[name] = blk
                del x2, v2, B2
            line["configs"] = cfgs
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sedov128")
    ap.add_argument("--precision", default="both", choices=["fp64", "mixed", "both"],
                    help="both (default): FP64 and mixed arms on the same input; the line's value is the mixed arm")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward measurement")
    ap.add_argument("--adjoint-n1d", type=int, default=128, help="hydro lattice size of the adjoint measurement")
    ap.add_argument("--adjoint-only", action="store_true", help="only the adjoint/forward measurement")
    ap.add_argument("--no-ind", action="store_true", help="skip the individual-timestep measurement")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other benchmark configurations and the 200-step run beside the headline")
    ap.add_argument("--cpu-steps", type=int, default=8, help="steps of the CPU-baseline sample (at most --steps)")
    ap.add_argument("--force-sym", type=int, default=None, choices=[0, 1],
                    help="FP64 force without self-gravity: 1 evaluates each unordered pair once (the library's "
                         "default), 0 from each side")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default warps per block instead of tuning them on the workload")
    args = ap.parse_args()
    dist, rank, ws = dist_init()
    rc = run_reference(args, dist, rank, ws) if args.impl == "reference" else run_ours(args, dist, rank, ws)
    if dist is not None:
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
