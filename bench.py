"""Benchmark of the grid-erosion step on GB300.

Workload (the metric's configuration): a 4096 x 4096 FP32 world, 6-octave
simplex fBm heightmap (base frequency 1/128, lacunarity 2, gain 0.5, seed 0)
scaled to [0, 64]; dt 0.02, G 9.81, Kc 0.1, Ks = Kd = 0.05, Ke 0.015;
thermal erosion with talus tan 0.65 and slippage 0.3; Bernoulli rain of 0.5
with p = 0.001 per cell and step from Philox4x32-10.  Data are synthetic
(seeded noise).  One bench "step" is one erosion step of the whole grid; the
metric is cell-steps per second.  The 9 carried fields (604 MB) exceed the
129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is the fused kernel with fields resident in
HBM; `plain_value` the per-pass kernels; `e2e` goes through the C ABI with
pinned host buffers (upload of the initial fields and download of the
result inside the timed region).  `--impl reference` times the CPU
restatement of the reference's passes (the reference itself is GLSL/OpenGL
and cannot run without a graphics stack).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "hydro-gen_gb300"))

N_GRID = 4096
BYTES_PER_CELL_STEP = 72  # 9 FP32 fields (rock, water, sediment, 4 fluxes, u, v) read + written
METRIC = "cell-steps/s fused vs per-pass at 4096²"
UNIT = "cell-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_GRID)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the adjoint and batch measurements")
    ap.add_argument("--extra", choices=["particles", "render", "two_layer", "terrain", "adjoint", "adjoint_thermal",
                                        "batch", "batch_class", "config1", "fp64_error", "fit_study", "large",
                                        "fd_check"],
                    default=None,
                    help="run only this extra measurement (--steps timed steps or frames, --warmup warm-up) "
                         "and print its JSON; for profiling captures")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(dist, value, device):
    """The job's time for replicas: the slowest rank's (weak scaling)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world_size, cells, steps, seconds):
    """Cell-steps per second of the whole job: every rank advances its own
    world of `cells` cells by `steps` steps within `seconds`."""
    return world_size * cells * steps / seconds


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic_per_cell_step():
    """DRAM bytes per cell-step of the fused kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "fused_step_config2.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_cell_step:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        time.sleep(0.15)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(n_sample=1024, budget_s=12.0):
    """The float oracle (CPU restatement of the reference passes), all host
    threads, on an n_sample^2 world with the same physics and rain."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    w = O.OracleWorld(n_sample, 32)
    w.set("rock", O.fbm(n_sample))
    s, o = O.workload("config2")
    w.step(s, o, 1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        w.step(s, o, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s and steps >= 3:
            break
    return {"value": steps * n_sample * n_sample / el, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"{n_sample}x{n_sample} world, same physics and rain, {steps} steps in {el:.1f} s "
                      f"(float oracle, OpenMP over rows)"}


def fd_check(H, torch, w, tape, reset, b0, target, n, nsteps, g, dks, db0, cells=64, eps=(1e-3, 1e-5), seed=0,
             reference_adjoint=False):
    """The GPU adjoint's gradients at the fit's starting point (uniform Ks
    0.05, the initial rock) against central finite differences of the FP64
    reference forward on `cells` random cells (fixed seed), for both the
    per-cell Ks and the initial rock, at each step size in `eps`.  The FP64
    differences run on all host cores (each perturbed forward only where it
    differs from an unperturbed one run in lockstep, bit for bit the full
    forward).  Relative error |g - fd| / max(|fd|, 1e-2 max|g|): the floor
    keeps cells whose gradient is ~0 (deposition, where Ks has no effect)
    from dividing by noise.  The scheme is piecewise smooth (dissolve or
    deposit, clamps, maxima), and over 256 steps a difference of 1e-3
    straddles a switch at a share of the cells, so 1e-5 is reported beside
    it.  With reference_adjoint the FP64 reference adjoint of the same loss
    (minutes of host time) is compared too: with the FD and with the GPU
    over every cell."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    ks = np.full((n, n), 0.05, np.float32)
    w.upload("ks", ks)
    reset()
    tape.forward()
    loss = H.mse(w, target.data_ptr(), g.data_ptr())
    tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
    w.sync()
    gk, gb = dks.cpu().numpy().astype(np.float64), db0.cpu().numpy().astype(np.float64)
    tgt = target.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(seed)
    pick = rng.choice(n * n, size=cells, replace=False)
    out = {"cells": cells, "seed": seed, "loss": loss, "fd_cores": O.num_threads(), "tolerance": 1e-3,
           "relative_error": "|g - fd| / max(|fd|, 1e-2 max|g|)"}

    def compare(grad, fdv):
        gv = grad.flat[pick]
        rel = np.abs(gv - fdv) / np.maximum(np.abs(fdv), 1e-2 * np.abs(grad).max())
        return {"within_tol": int(np.sum(rel <= 1e-3)), "max_rel": float(rel.max()),
                "median_rel": float(np.median(rel))}

    fds = {}
    for e in eps:
        t0 = time.perf_counter()
        fd = O.fd_ref(O.settings_config1(), 0.01, 1, b0.astype(np.float64), ks, tgt, nsteps,
                      np.concatenate([pick, pick]), np.array([0] * cells + [1] * cells), e)
        fds[e] = fd
        out[f"eps_{e:g}"] = {"fd_seconds": time.perf_counter() - t0, "gpu_ks": compare(gk, fd[:cells]),
                             "gpu_rock0": compare(gb, fd[cells:])}
    if reference_adjoint:
        t0 = time.perf_counter()
        _, rk, rb = O.adjoint_ref(O.settings_config1(), 0.01, 1, b0.astype(np.float64), ks, tgt, nsteps)
        out["reference_adjoint_seconds"] = time.perf_counter() - t0
        for e, fd in fds.items():
            out[f"eps_{e:g}"]["fp64_adjoint_ks"] = compare(rk, fd[:cells])
            out[f"eps_{e:g}"]["fp64_adjoint_rock0"] = compare(rb, fd[cells:])
        out["gpu_vs_fp64_adjoint_rel_l2"] = {"ks": float(np.linalg.norm(gk - rk) / np.linalg.norm(rk)),
                                             "rock0": float(np.linalg.norm(gb - rb) / np.linalg.norm(rb))}
    w.sync()
    return out


def bench_adjoint(H, torch, n=1024, nsteps=256, ckpt=32, reps=3, fd_cells=64, fit_kw=None, reference_adjoint=False):
    """Forward + adjoint of the inverse-erosion workload: 1024^2, config-1
    physics, per-cell Ks = 0.05 exp(0.5 n(x)) from 3-octave simplex noise,
    MSE to a target, gradients for Ks and the initial rock; then fit_iters
    iterations of the native descent (hg_inverse_fit) on both."""
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config1")
    w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    ks_true = w.download("ks")
    w.step(nsteps, H.MODE_FUSED)
    target = torch.empty((n, n), dtype=torch.float32, device="cuda")
    w.download_device("rock", target.data_ptr())
    w.init_heightmap(H.noise(seed=0))
    b0 = w.download("rock")
    g = torch.empty_like(target)
    dks = torch.empty_like(target)
    db0 = torch.empty_like(target)
    tape = H.Tape(w, nsteps, ckpt)
    stream = torch.cuda.ExternalStream(w.stream)

    def reset():
        w.upload("rock", b0)
        for f in ("water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"):
            w.upload(f, np.zeros((n, n), np.float32))
        w.step_count = 0

    fwd_ms, all_ms = [], []
    for r in range(reps + 1):
        reset()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        tape.forward()
        e1.record(stream)
        H.mse(w, target.data_ptr(), g.data_ptr())
        tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
        e2.record(stream)
        e2.synchronize()
        if r:
            fwd_ms.append(e0.elapsed_time(e1))
            all_ms.append(e0.elapsed_time(e2))
    f, a = statistics.median(fwd_ms), statistics.median(all_ms)
    cs = n * n * nsteps
    fd = (fd_check(H, torch, w, tape, reset, b0, target, n, nsteps, g, dks, db0, cells=fd_cells,
                   reference_adjoint=reference_adjoint) if fd_cells else None)
    # the fit itself (hg_inverse_fit) from uniform Ks = 0.05 and the true
    # initial rock
    fit = bench_fit(H, torch, w, target, ks_true, b0, n, nsteps, ckpt, **(fit_kw or {}))
    return {"workload": f"inverse erosion {n}x{n}, {nsteps} steps, per-cell Ks, checkpoints every {ckpt}",
            "forward_cell_steps_per_s": cs / (f / 1e3), "fwd_adjoint_cell_steps_per_s": cs / (a / 1e3),
            "fwd_adjoint_over_forward_time": a / f, "ms_forward": f, "ms_fwd_adjoint": a,
            "fd_check": fd, "fit": fit}


def bench_fit(H, torch, w, target, ks_true, b0, n, nsteps, ckpt, iters=100, chunk=10, ks_step=0.01,
              rock_step=0.0, decay=1.0):
    """The inverse-erosion fit of the 1024^2 workload through hg_inverse_fit:
    from uniform Ks = 0.05 (and the true initial rock), `iters` iterations
    in calls of `chunk`, the largest per-iteration change multiplied by
    `decay` after each call (1: a fixed step; on this workload a fixed step
    of 0.01 lowered the loss and the Ks error further in 100 iterations than
    steps shrinking by 0.8 or 0.9 per call).  Reports the loss of every iteration, and
    after every call the relative L2 error of the fitted Ks against the
    target's Ks field, over all cells and over the cells where the first
    gradient moved Ks (erosion happens there; elsewhere the loss does not
    depend on Ks and Ks keeps its start value), and the RMS error of the
    initial rock (height units)."""
    ks = torch.full((n, n), 0.05, dtype=torch.float32, device="cuda")
    b0_dev = torch.from_numpy(b0).cuda()
    b0_true = b0_dev.clone()
    kt = torch.from_numpy(ks_true).cuda().double()
    losses, norms, curve = [], [], []
    moved = None
    ms = 0.0
    step_k, step_b = ks_step, rock_step
    for c0 in range(0, iters, chunk):
        k = min(chunk, iters - c0)
        fs = H.fit_settings(nsteps=nsteps, ckpt_every=ckpt, iters=k, ks_step=step_k, rock_step=step_b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        l, g = H.inverse_fit(w, target.data_ptr(), ks.data_ptr(), b0_dev.data_ptr(), fs, grad_norms=True)
        ms += (time.perf_counter() - t0) * 1e3
        losses += l
        norms += g
        if moved is None:
            moved = ks != 0.05
        d = ks.double() - kt
        curve.append({"iter": c0 + k, "ks_step": step_k, "loss": l[-1],
                      "ks_rel_err": float(d.norm() / kt.norm()),
                      "ks_rel_err_eroding": float(d[moved].norm() / kt[moved].norm()) if bool(moved.any()) else None,
                      "rock0_rms_err": float((b0_dev.double() - b0_true.double()).pow(2).mean().sqrt())})
        step_k *= decay
        step_b *= decay
    d0 = torch.full_like(kt, 0.05) - kt
    return {"iters": iters, "chunk": chunk, "ks_step": ks_step, "rock_step": rock_step, "decay": decay,
            "ms_per_iter": ms / iters, "losses": losses, "grad_norms": norms,
            "ks_rel_err_start": float(d0.norm() / kt.norm()),
            "ks_rel_err_start_eroding": float(d0[moved].norm() / kt[moved].norm()) if bool(moved.any()) else None,
            "eroding_cells": int(moved.sum()), "curve": curve,
            "ks_rel_err": curve[-1]["ks_rel_err"], "ks_rel_err_eroding": curve[-1]["ks_rel_err_eroding"],
            "rock0_rms_err": curve[-1]["rock0_rms_err"],
            "loss_first": losses[0], "loss_last": losses[-1]}


def bench_adjoint_workload(H, torch, n=N_GRID, nsteps=500, reps=2):
    """Forward + adjoint at the metric's workload (4096^2, Bernoulli rain,
    talus slippage, its 500 steps) with a per-cell Ks field: nsteps taped
    steps from the initial heightmap, checkpoint interval chosen from free
    memory (the steps beyond one segment are recomputed in the backward),
    MSE to a target, gradients for Ks and the initial rock."""
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config2")
    w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    b0 = w.download("rock")
    target = torch.from_numpy(b0).cuda().mul_(0.999)
    g = torch.empty_like(target)
    dks = torch.empty_like(target)
    db0 = torch.empty_like(target)
    tape = H.Tape(w, nsteps, H.HG_AUTO)
    stream = torch.cuda.ExternalStream(w.stream)
    res = []
    for r in range(reps + 1):
        w.upload("rock", b0)
        for f in ("water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"):
            w.upload(f, np.zeros((n, n), np.float32))
        w.step_count = 0
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        tape.forward()
        e1.record(stream)
        H.mse(w, target.data_ptr(), g.data_ptr())
        tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
        e2.record(stream)
        e2.synchronize()
        if r:
            res.append((e0.elapsed_time(e1), e0.elapsed_time(e2)))
    f = statistics.median(x[0] for x in res)
    a = statistics.median(x[1] for x in res)
    out = {"workload": f"{n}x{n} Bernoulli rain + talus slippage, per-cell Ks, {nsteps} steps",
           "ckpt_every": tape.ckpt_every, "recomputed_steps": nsteps - tape.ckpt_every, "ms_forward": f,
           "ms_fwd_adjoint": a, "fwd_adjoint_over_forward_time": a / f,
           "fwd_adjoint_cell_steps_per_s": n * n * nsteps / (a / 1e3),
           "gradient_finite": bool(torch.isfinite(dks).all() and torch.isfinite(db0).all())}
    tape.close()
    w.close()
    return out


def bench_large(H, torch, n=8192, fwd_steps=2000, adj_steps=512, nbatch=16, bn=1024, bsteps=256):
    """The large workload: 8192^2, uniform-rain physics with talus slippage
    (tan 0.65, rate 0.3): 2000 forward steps; forward + adjoint over 512
    steps with the checkpoint interval chosen from free memory; and 16
    independent 1024^2 forward + adjoint tapes (256 steps, checkpoints every
    32) on their own streams."""
    def physics(w):
        H.configure(w, "config1")
        s = H.settings_config1()
        s.Kspeed[0] = 0.3
        w.set_erosion(s)

    def events(stream):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        return e

    out = {"workload": f"{n}x{n}, config-1 physics + thermal (tan 0.65, rate 0.3)"}
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    physics(w)
    st = torch.cuda.ExternalStream(w.stream)
    w.step(10, H.MODE_FUSED)
    w.sync()
    e0, e1 = events(st)
    e0.record(st)
    w.step(fwd_steps, H.MODE_FUSED)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    cs = n * n * fwd_steps / (ms / 1e3)
    out["forward"] = {"steps": fwd_steps, "ms_per_step": ms / fwd_steps, "cell_steps_per_s": cs,
                      "algorithmic_GBs": cs * BYTES_PER_CELL_STEP / 1e9}
    # forward + adjoint over 512 steps from the eroded state
    target = torch.empty((n, n), dtype=torch.float32, device="cuda")
    w.download_device("rock", target.data_ptr())
    target.mul_(0.999)
    g = torch.empty_like(target)
    dks = torch.empty_like(target)
    db0 = torch.empty_like(target)
    w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
    tape = H.Tape(w, adj_steps, H.HG_AUTO)
    torch.cuda.synchronize()
    e0, e1 = events(st)
    e2 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    tape.forward()
    e1.record(st)
    H.mse(w, target.data_ptr(), g.data_ptr())
    tape.backward(g.data_ptr(), dks.data_ptr(), db0.data_ptr())
    e2.record(st)
    e2.synchronize()
    f, a = e0.elapsed_time(e1), e0.elapsed_time(e2)
    out["fwd_adjoint"] = {"steps": adj_steps, "ckpt_every": tape.ckpt_every,
                          "recomputed_steps": adj_steps - tape.ckpt_every, "ms_forward": f, "ms_fwd_adjoint": a,
                          "fwd_adjoint_over_forward_time": a / f,
                          "fwd_adjoint_cell_steps_per_s": n * n * adj_steps / (a / 1e3),
                          "gradient_finite": bool(torch.isfinite(dks).all() and torch.isfinite(db0).all())}
    tape.close()
    w.close()
    # 16 independent 1024^2 tapes, each on its own stream
    ws, tapes, tg = [], [], []
    for k in range(nbatch):
        x = H.World(bn)
        x.init_heightmap(H.noise(seed=100 + k))
        physics(x)
        x.init_ks_field(H.noise(seed=200 + k, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
        t = torch.empty((bn, bn), dtype=torch.float32, device="cuda")
        x.download_device("rock", t.data_ptr())
        t.mul_(0.999)
        ws.append(x)
        tg.append((t, torch.empty_like(t), torch.empty_like(t)))
        tapes.append(H.Tape(x, bsteps, 32))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for tp in tapes:
        tp.forward()
    for x, tp, (t, gg, dk) in zip(ws, tapes, tg):
        H.mse(x, t.data_ptr(), gg.data_ptr())
        tp.backward(gg.data_ptr(), dk.data_ptr(), None)
    for x in ws:
        x.sync()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    out["batched_adjoint"] = {"terrains": nbatch, "side": bn, "steps": bsteps, "seconds": el,
                              "fwd_adjoint_cell_steps_per_s": nbatch * bn * bn * bsteps / el}
    for tp in tapes:
        tp.close()
    for x in ws:
        x.close()
    out["gradient_error_vs_fp64"] = ("checked at 64^2 and 128^2 against the FP64 reference adjoint "
                                     "(tests/test_gpu_adjoint.py): <= 1.5e-4 relative L2, thermal on and off")
    return out


def bench_config1(H, torch, n=256, nsteps=1000, reps=3, cpu=True):
    """Config 1 as the workloads define it: 256^2, uniform rain 0.01 every
    step, thermal off, 1000 steps; per-pass and fused kernels (CUDA events,
    median of three runs), and the float and FP64 oracles on the host."""
    out = {"workload": f"config1 {n}x{n}, {nsteps} steps", "steps": nsteps}
    for name, mode in (("plain", H.MODE_PLAIN), ("fused", H.MODE_FUSED)):
        times = []
        for r in range(reps + 1):
            w = H.World(n)
            w.init_heightmap(H.noise(seed=0))
            H.configure(w, "config1")
            w.sync()
            stream = torch.cuda.ExternalStream(w.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            w.step(nsteps, mode)
            e1.record(stream)
            e1.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
            w.close()
        ms = statistics.median(times)
        out[name] = {"ms_per_run": ms, "cell_steps_per_s": n * n * nsteps / (ms / 1e3)}
    if not cpu:
        return out
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    s, o = O.workload("config1")
    for prec in (32, 64):
        ow = O.OracleWorld(n, prec)
        ow.set("rock", O.fbm(n))
        t0 = time.perf_counter()
        ow.step(s, o, nsteps)
        el = time.perf_counter() - t0
        out[f"cpu_fp{prec}"] = {"value": n * n * nsteps / el, "unit": "cell-steps/s", "cores": O.num_threads(),
                                "kind": "port", "sample": f"the full run, {el:.2f} s"}
    return out


def bench_fp64_error(H, torch):
    """Rock error of the GPU's float result against the FP64 oracle at each
    workload's own size: max and 99.9th percentile of |d rock| / (rock
    range), and the cells above the workload's bar (1e-4 at 100 steps, 1e-3
    at 500 and 1000).  The FP64 oracle runs on all host cores (4096^2 x 500
    steps and 8192^2 x 100 steps take minutes), so this is an extra, not
    part of the default line."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    def err(w, ow):
        g = w.download("rock").astype(np.float64)
        r = ow.get("rock")
        e = np.abs(g - r) / (r.max() - r.min())
        return e

    def row(e, bar):
        return {"max": float(e.max()), "p99_9": float(np.quantile(e, 0.999)), "bar": bar,
                "cells_above_bar": int(np.sum(e > bar)), "cells": int(e.size), "holds": bool(e.max() <= bar)}

    def run(name, n, cfg, checkpoints, ks=False, thermal=False, init_seed=0):
        w = H.World(n)
        w.init_heightmap(H.noise(seed=init_seed))
        H.configure(w, cfg)
        s, o = O.workload(cfg)
        if thermal:  # config-1 physics with the large workload's talus slippage
            es = H.settings_config1()
            es.Kspeed[0] = 0.3
            es.Kalpha[0] = float(np.arctan(0.65))
            w.set_erosion(es)
            s.Kspeed[0] = 0.3
            s.Kalpha[0] = float(np.arctan(0.65))
        ow = O.OracleWorld(n, 64)
        ow.set("rock", w.download("rock"))
        if ks:
            w.init_ks_field(H.noise(seed=7, octaves=3, frequency=1.0 / 256), 0.05, 0.5)
            ow.set_ks(w.download("ks"))
        out, done, t0 = {"grid": n}, 0, time.perf_counter()
        for k in checkpoints:
            w.step(k - done, H.MODE_FUSED)
            ow.step(s, o, k - done)
            done = k
            out[f"steps_{k}"] = row(err(w, ow), 1e-4 if k <= 100 else 1e-3)
        out["oracle_s"] = time.perf_counter() - t0
        w.close()
        res[name] = out

    res = {"oracle_cores": O.num_threads()}
    run("config1_256", 256, "config1", (100, 1000))
    run("config2_256", 256, "config2", (100, 500))
    run("config4_1024_per_cell_ks", 1024, "config1", (256,), ks=True)
    run("config2_4096", 4096, "config2", (100, 500))
    run("config5_8192_thermal", 8192, "config1", (100,), thermal=True)
    return res


def bench_batch(H, torch, count=64, nsteps=200, warmup=16):
    """64 terrains of sides drawn from {256, 512, 1024, 2048} with their own
    seeds and parameters, stepped three ways: each terrain's own fused
    launches, one table launch per kernel for all terrains (tile height and
    graph replay fixed to the table's tuned choice), and the batch API's
    autotuned form (the faster of the two)."""
    ts = H.config3_terrains(count=count, seed=0)
    ws = [H.make_config3_world(t, terrain_id=i) for i, t in enumerate(ts)]
    cells = sum(t["n"] ** 2 for t in ts)
    out = {"workload": f"{count} terrains, sides from {{256,512,1024,2048}}, {cells} cells", "steps": nsteps}

    def timed(b, mode):
        b.step(warmup, mode)
        b.sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.step(nsteps, mode)
        b.sync()
        torch.cuda.synchronize()
        return cells * nsteps / (time.perf_counter() - t0)

    b = H.Batch(ws)
    out["per_terrain_cell_steps_per_s"] = timed(b, H.MODE_FUSED_PER_WORLD)
    out["autotuned_cell_steps_per_s"] = timed(b, H.MODE_FUSED)
    th, graph, ms = b.tuning()
    per_world, ms_pw = b.launch_form()
    out["tuned"] = {"form": "per_terrain" if per_world else "one_launch", "tile": [64, th], "graph": graph,
                    "one_launch_ms_per_step": ms, "per_terrain_ms_per_step": ms_pw}
    b.close()
    for i, (w, t) in enumerate(zip(ws, ts)):
        w.set_options(H.options(H.RAIN_BERNOULLI, p=0.001, seed=t["seed"], terrain_id=i, tile=(64, th),
                                graph=graph))
    b = H.Batch(ws)
    out["one_launch_cell_steps_per_s"] = timed(b, H.MODE_FUSED)
    b.close()
    out["one_launch_over_per_terrain"] = out["one_launch_cell_steps_per_s"] / out["per_terrain_cell_steps_per_s"]
    for w in ws:
        w.close()
    out["size_classes"] = batch_size_classes(H, torch)
    single = out["size_classes"]["4096"]["per_terrain_ps_per_cell_step"]  # the single-world kernels
    out["one_launch_over_single_world_rate"] = out["one_launch_cell_steps_per_s"] * single * 1e-12
    return out


CLASS_TERRAINS = {256: 128, 512: 64, 1024: 16, 2048: 4, 4096: 1}


def batch_size_classes(H, torch, nsteps=100, warmup=16, sides=(256, 512, 1024, 2048, 4096)):
    """The per-cell cost of each terrain size of the ragged batch on its own:
    a batch of equal terrains per side (config-2 physics, Bernoulli rain,
    64 x 16 tiles, graph replay) as one table launch and as each terrain's own
    launches; at 4096² one world, whose own launches are the single-world
    kernels.  ps per cell-step."""
    out = {}
    for side in sides:
        count = CLASS_TERRAINS.get(side, 1)
        ws = []
        for i in range(count):
            w = H.World(side)
            w.init_heightmap(H.noise(seed=i))
            H.configure(w, "config2")
            w.set_options(H.options(H.RAIN_BERNOULLI, p=0.001, seed=i, terrain_id=i, tile=(64, 16), graph=1))
            ws.append(w)
        cells = count * side * side
        b = H.Batch(ws)
        row = {"terrains": count}
        for key, mode in (("one_launch", H.MODE_FUSED), ("per_terrain", H.MODE_FUSED_PER_WORLD)):
            b.step(warmup, mode)
            b.sync()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.step(nsteps, mode)
            b.sync()
            torch.cuda.synchronize()
            row[key + "_ps_per_cell_step"] = 1e12 * (time.perf_counter() - t0) / (nsteps * cells)
        b.close()
        for w in ws:
            w.close()
        out[str(side)] = row
    return out


def bench_batch_sharded(H, torch, dist, rank, world_size, device, count=64, nsteps=200, warmup=16):
    """The ragged 64-terrain workload split over the job's ranks by area
    (hydrogen.shard_by_area, no data exchange): each rank steps its share as
    one autotuned batch; the job's time is the slowest rank's (strong
    scaling: the total work is fixed)."""
    ts = H.config3_terrains(count=count, seed=0)
    owner = H.shard_by_area([t["n"] for t in ts], world_size)
    mine = [i for i in range(count) if owner[i] == rank]
    ws = [H.make_config3_world(ts[i], terrain_id=i) for i in mine]
    cells = sum(t["n"] ** 2 for t in ts)
    loads = [sum(ts[i]["n"] ** 2 for i in range(count) if owner[i] == r) for r in range(world_size)]
    b = H.Batch(ws) if ws else None
    if b:
        b.step(warmup, H.MODE_FUSED)
        b.sync()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    if b:
        b.step(nsteps, H.MODE_FUSED)
        b.sync()
    torch.cuda.synchronize()
    el = max_over_ranks(dist, time.perf_counter() - t0, device)
    if b:
        b.close()
    for w in ws:
        w.close()
    return {"workload": f"{count} terrains, sides from {{256,512,1024,2048}}, {cells} cells, split by area",
            "ranks": world_size, "scaling": "strong", "steps": nsteps, "cell_steps_per_s": cells * nsteps / el,
            "largest_over_mean_load": max(loads) / (cells / world_size)}


def bench_two_layer(H, torch, n=4096, nsteps=100, warmup=10, cpu_budget_s=6.0, cpu_n=1024):
    """The reference's own model: a two-layer (rock + dirt) world from its
    terrain generator with its default grid settings (src/state.cpp:81-92:
    Kconv 0.001, slippage 0.5 / 2.0, so both talus layers and smoothing run)
    and uniform rain of 0.01 every step; the fused three-kernel step and the
    per-pass kernels.  The float oracle steps a 1024^2 world of the same
    model on the host."""
    s = H.ErosionSettings()
    H.check(H.lib.hg_default_erosion_settings(H.ctypes.byref(s)))
    cells = n * n
    peak, kind = peaks()
    out = {"workload": f"{n}x{n} two-layer world (reference terrain), reference grid defaults, uniform rain 0.01",
           "steps": nsteps}
    for name, mode in (("plain", H.MODE_PLAIN), ("fused", H.MODE_FUSED)):
        w = H.World(n, layers=2)
        w.init_reference_heightmap(H.map_settings(hmap_dims=(n, n)))
        w.set_erosion(s)
        w.set_rain(H.rain_uniform(0.01, 1))
        w.set_options(H.options(H.RAIN_UNIFORM))
        w.step(warmup, mode)
        w.sync()
        stream = torch.cuda.ExternalStream(w.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = H.lib.hg_launch_count()
        e0.record(stream)
        w.step(nsteps, mode)
        e1.record(stream)
        e1.synchronize()
        launches = H.lib.hg_launch_count() - l0
        ms = e0.elapsed_time(e1) / nsteps
        w.close()
        achieved = 88.0 * cells / (ms / 1e3) / 1e9  # 11 fields x 4 B x (read + write)
        out[name] = {"ms_per_step": ms, "cell_steps_per_s": cells / (ms / 1e3), "launches_per_step": launches / nsteps,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                  "frac": achieved / peak, "algorithmic_bytes_per_cell_step": 88,
                                  "peak_source": f"{kind} hbm_gbs"}}
    out["fused_vs_plain"] = out["plain"]["ms_per_step"] / out["fused"]["ms_per_step"]
    if cpu_budget_s <= 0:
        return out
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    rock, dirt = O.ref_heightmap(H.map_settings(hmap_dims=(cpu_n, cpu_n)), cpu_n)
    ow = O.OracleWorld(cpu_n, 32)
    ow.set("rock", rock)
    ow.set("dirt", dirt)
    os_, oo = O.erosion_from(s), O.options(1, 1, 0.01)
    ow.step(os_, oo, 1)
    k, t0 = 0, time.perf_counter()
    while True:
        ow.step(os_, oo, 1)
        k += 1
        if time.perf_counter() - t0 >= cpu_budget_s and k >= 2:
            break
    cel = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": k * cpu_n * cpu_n / cel, "unit": "cell-steps/s", "cores": O.num_threads(),
                           "kind": "port", "sample": f"{cpu_n}x{cpu_n} world of the same model, {k} steps in "
                           f"{cel:.1f} s (float oracle, OpenMP over rows)"}
    return out


def bench_terrain(H, torch, n=4096, reps=5, cpu_budget_s=4.0, cpu_n=512):
    """The reference's terrain generator (glsl/heightmap.glsl, default map
    settings: 8 octaves of derivative-damped gradient noise with domain warp)
    on a 4096^2 two-layer world; the oracle generates a 512^2 map."""
    w = H.World(n, layers=2)
    ms_ = H.map_settings(hmap_dims=(n, n))
    w.init_reference_heightmap(ms_)
    w.sync()
    stream = torch.cuda.ExternalStream(w.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        w.init_reference_heightmap(ms_)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    w.close()
    out = {"workload": f"reference terrain generator, {n}x{n}, default map settings", "ms": ms,
           "cells_per_s": n * n / (ms / 1e3)}
    if cpu_budget_s <= 0:
        return out
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    m2 = H.map_settings(hmap_dims=(cpu_n, cpu_n))
    k, t0 = 0, time.perf_counter()
    while True:
        O.ref_heightmap(m2, cpu_n)
        k += 1
        if time.perf_counter() - t0 >= cpu_budget_s:
            break
    cel = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": k * cpu_n * cpu_n / cel, "unit": "cells/s", "cores": O.num_threads(),
                           "kind": "port", "sample": f"{cpu_n}x{cpu_n} map, {k} maps in {cel:.1f} s (float oracle, "
                           "OpenMP over rows)"}
    return out


def bench_particles(H, torch, n=1024, count=262144, nsteps=200, warmup=10, cpu_budget_s=6.0):
    """Droplet erosion (the reference's "particle" erosion type and default
    particle_count 262144) on a 1024^2 two-layer world from the reference's
    terrain generator with its particle defaults; the float oracle's
    sequential restatement times a few steps of the same world on the host."""
    w = H.World(n, layers=2)
    ms = H.map_settings(hmap_dims=(n, n))
    w.init_reference_heightmap(ms)
    w.particles_init(count)
    s = H.settings_particles()
    w.set_erosion(s)
    w.set_options(H.options(H.RAIN_UNIFORM, seed=11))
    rock0, dirt0 = w.download("rock"), w.download("dirt")
    w.step(warmup, H.MODE_PARTICLES)
    w.sync()
    torch.cuda.synchronize()
    l0 = H.lib.hg_launch_count()
    t0 = time.perf_counter()
    w.step(nsteps, H.MODE_PARTICLES)
    w.sync()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    launches = H.lib.hg_launch_count() - l0
    w.close()
    out = {"workload": f"{n}x{n} two-layer world (reference terrain), {count} droplets, particle defaults, "
                       "thermal both layers + smoothing", "steps": nsteps,
           "droplet_steps_per_s": count * nsteps / el, "ms_per_step": 1e3 * el / nsteps,
           "launches_per_step": launches / nsteps}
    if cpu_budget_s <= 0:
        return out
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    ow = O.OracleWorld(n, 32)
    ow.set("rock", rock0)
    ow.set("dirt", dirt0)
    ow.particles_init(count)
    os_, oo = O.erosion_from(s), O.options(1, 1, 0.0, seed=11)
    ow.particle_step(os_, oo, 1)
    k, t0 = 0, time.perf_counter()
    while True:
        ow.particle_step(os_, oo, 1)
        k += 1
        if time.perf_counter() - t0 >= cpu_budget_s and k >= 2:
            break
    cel = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": count * k / cel, "unit": "droplet-steps/s", "cores": O.num_threads(),
                           "kind": "port", "sample": f"same world, {k} steps in {cel:.1f} s (droplets in id "
                           "order on one core, grid passes OpenMP)"}
    return out


def bench_render(H, torch, n=1024, width=1920, height=1080, frames=20, warmup=3, cpu_budget_s=6.0):
    """The headless ray-marcher on a 1024^2 two-layer world from the
    reference's terrain generator with a lake (water filled to height 96, the
    reference's WATER_HEIGHT), 1920x1080 from inside the map over the lake; the
    float oracle renders a 192x108 image of the same view on the host."""
    w = H.World(n, layers=2)
    ms = H.map_settings(hmap_dims=(n, n))
    w.init_reference_heightmap(ms)
    rock, dirt = w.download("rock"), w.download("dirt")
    ground = rock + dirt
    w.upload("water", np.where(ground < 96.0, 96.0 - ground, 0.0).astype(np.float32))
    cam = H.camera((150.0, 170.0, 150.0), (1.0, -0.35, 1.0), aspect=width / height)
    img = torch.empty(width * height * 4, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(w.stream)

    def frame():
        H.check(H.lib.hg_render_device(w.h, H.ctypes.byref(cam), width, height, img.data_ptr(), None))

    for _ in range(warmup):
        frame()
    w.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(frames):
        frame()
    e1.record(stream)
    e1.synchronize()
    dev_ms = e0.elapsed_time(e1) / frames
    host = np.empty((height, width, 4), np.uint8)
    t0 = time.perf_counter()
    for _ in range(frames):
        H.check(H.lib.hg_render(w.h, H.ctypes.byref(cam), width, height, host.ctypes.data, None))
    e2e_ms = 1e3 * (time.perf_counter() - t0) / frames
    fields = {k: w.download(k) for k in ("rock", "dirt", "water", "sediment", "sediment_dirt")}
    w.close()
    mpix = width * height / 1e6
    out = {"workload": f"{width}x{height} frame of a {n}x{n} two-layer world with a lake", "frames": frames,
           "ms_per_frame": dev_ms, "mpixels_per_s": mpix / (dev_ms / 1e3),
           "e2e": {"ms_per_frame": e2e_ms, "mpixels_per_s": mpix / (e2e_ms / 1e3),
                   "d2h_bytes_per_frame": width * height * 4},
           }
    if cpu_budget_s <= 0:
        return out
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cw, ch = width // 10, height // 10
    k, t0 = 0, time.perf_counter()
    while True:
        O.render(fields, n, cam, cw, ch, ms.max_height, n)
        k += 1
        if time.perf_counter() - t0 >= cpu_budget_s:
            break
    cel = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": k * cw * ch / 1e6 / cel, "unit": "Mpixel/s", "cores": O.num_threads(),
                           "kind": "port", "sample": f"{cw}x{ch} image of the same view, {k} frames in {cel:.1f} s "
                           "(float oracle, OpenMP over rows)"}
    return out


def run_reference(args, rank):
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    n = args.n
    w = O.OracleWorld(n, 32)
    w.set("rock", O.fbm(n))
    s, o = O.workload("config2")
    w.step(s, o, args.warmup)
    t0 = time.perf_counter()
    w.step(s, o, args.steps)
    el = time.perf_counter() - t0
    v = args.steps * n * n / el
    sample = (f"each step is one erosion step of the whole {n}x{n} world, same init, physics and rain as the "
              f"GPU arm (float CPU restatement of the GLSL passes; the reference's GL path needs a graphics "
              f"stack, unavailable on this box)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"config2 erosion {n}x{n} FP32, thermal on, Bernoulli rain p=0.001",
                       "grid": n, "parallelism": "single GPU" if args.gpus == 1 else f"replicas x{args.gpus}",
                       "l2": "inputs larger than L2 (9 fields x 4 B x n^2)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world_size, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    import hydrogen as H

    torch.cuda.set_device(local)
    if args.extra is not None:
        if rank == 0:
            budget = 0.0 if args.no_cpu_baseline else 6.0
            if args.extra == "particles":
                out = bench_particles(H, torch, nsteps=args.steps, warmup=args.warmup, cpu_budget_s=budget)
            elif args.extra == "two_layer":
                out = bench_two_layer(H, torch, nsteps=args.steps, warmup=args.warmup, cpu_budget_s=budget)
            elif args.extra == "terrain":
                out = bench_terrain(H, torch, reps=args.steps, cpu_budget_s=budget)
            elif args.extra == "config1":
                out = bench_config1(H, torch, cpu=budget > 0)
            elif args.extra == "fd_check":  # the default line's check plus the FP64 reference adjoint
                out = bench_adjoint(H, torch, reps=1, fit_kw=dict(iters=1, chunk=1),
                                    reference_adjoint=True)["fd_check"]
            elif args.extra == "large":
                out = bench_large(H, torch)
            elif args.extra == "fp64_error":
                out = bench_fp64_error(H, torch)
            elif args.extra == "fit_study":  # fit schedules on the inverse workload
                out = {}
                for name, kw in (("ks_fixed_0.01", dict(ks_step=0.01, decay=1.0)),
                                 ("ks_0.01_decay_0.8", dict(ks_step=0.01, decay=0.8)),
                                 ("ks_0.005_decay_0.9", dict(ks_step=0.005, decay=0.9)),
                                 ("ks_rock_0.01_0.02_decay_0.8", dict(ks_step=0.01, rock_step=0.02, decay=0.8))):
                    r = bench_adjoint(H, torch, reps=1, fd_cells=0, fit_kw=kw)["fit"]
                    out[name] = {k: v for k, v in r.items() if k not in ("losses", "grad_norms")}
                    out[name]["losses_every_10"] = r["losses"][::10] + [r["losses"][-1]]
            elif args.extra == "adjoint":  # --steps reversed steps, --warmup timed repetitions
                out = bench_adjoint(H, torch, nsteps=args.steps, ckpt=min(32, args.steps),
                                    reps=max(1, args.warmup))
            elif args.extra == "batch":  # --steps timed steps, --warmup warm-up steps
                out = bench_batch(H, torch, nsteps=args.steps, warmup=args.warmup)
            elif args.extra == "batch_class":  # one size class of the batch: --n side
                out = batch_size_classes(H, torch, nsteps=args.steps, warmup=args.warmup, sides=(args.n,))
            elif args.extra == "adjoint_thermal":  # --n grid, --steps taped steps, --warmup repetitions
                out = bench_adjoint_workload(H, torch, n=args.n, nsteps=args.steps, reps=max(1, args.warmup))
            else:
                out = bench_render(H, torch, frames=args.steps, warmup=args.warmup, cpu_budget_s=budget)
            print(json.dumps(out), flush=True)
        return
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n = args.n
    cells = n * n
    w = H.World(n)
    w.init_heightmap(H.noise(seed=0))
    H.configure(w, "config2")
    w.set_options(H.options(H.RAIN_BERNOULLI, p=0.001, seed=0, terrain_id=rank))
    init = {f: w.download(f) for f in ("rock",)}
    stream = torch.cuda.ExternalStream(w.stream)

    def timed(mode, steps, warmup):
        # the first fused call of >= 8 steps runs the autotuner (8 ordinary
        # steps): warming up with at least that many keeps it out of the
        # timed region
        w.step(max(warmup, 8) if mode == H.MODE_FUSED else warmup, mode)
        w.sync()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = H.lib.hg_launch_count()
        e0.record(stream)
        w.step(steps, mode)
        e1.record(stream)
        e1.synchronize()
        launches = H.lib.hg_launch_count() - l0
        barrier()
        ms = max_over_ranks(dist, e0.elapsed_time(e1), "cuda")
        return ms, launches

    # per-pass kernels (denominator of the fused-vs-plain ratio)
    plain_steps = min(args.steps, 100)
    plain_ms, _ = timed(H.MODE_PLAIN, plain_steps, max(3, args.warmup // 4))
    # fused kernel: the headline
    w.upload("rock", init["rock"])
    for f in ("water", "sediment", "flux_l", "flux_r", "flux_t", "flux_b"):
        w.upload(f, init["rock"] * 0)
    w.step_count = 0
    with Clocks(local) as clk:
        fused_ms, launches = timed(H.MODE_FUSED, args.steps, args.warmup)
    tuned = w.tuning()
    # the roofline unit is one fused step: the k_hydro + k_transport pair
    # (two launches) that moves the step's 72 B per cell
    fused_step_ms = fused_ms / args.steps

    value = job_throughput(world_size, cells, args.steps, fused_ms / 1e3)
    plain_value = job_throughput(world_size, cells, plain_steps, plain_ms / 1e3)

    # e2e: C ABI with pinned host buffers, copies inside the timed region.
    # The workload's input is its initial heightmap (water, sediment and
    # flux start at zero, set on the device as the reference's texture
    # creation does); its result is read back as rock, water and sediment.
    rock_host = torch.from_numpy(init["rock"]).pin_memory()
    outs = {f: torch.empty((n, n), dtype=torch.float32).pin_memory() for f in ("rock", "water", "sediment")}
    barrier()
    t0 = time.perf_counter()
    H.check(H.lib.hg_init_heightmap_host(w.h, H.ctypes.c_void_p(rock_host.data_ptr())))
    t1 = time.perf_counter()  # returns once its copy is done
    w.step(args.steps, H.MODE_FUSED)
    w.sync()
    t2 = time.perf_counter()
    for f, t in outs.items():
        H.check(H.lib.hg_world_download(w.h, H.FIELDS[f], t.data_ptr()))
    barrier()
    t3 = time.perf_counter()
    e2e_s = max_over_ranks(dist, t3 - t0, "cuda")
    h2d = cells * 4 / args.steps
    d2h = 3 * cells * 4 / args.steps
    # the copies' own rates from pinned memory (the host link bounds them:
    # about 210 GB/s up and 190 GB/s down on GB300, whatever the copy form;
    # the upload's time includes zeroing the other fields on the device)
    copy_rates = {"h2d_gbs": cells * 4 / (t1 - t0) / 1e9, "d2h_gbs": 3 * cells * 4 / (t3 - t2) / 1e9}
    # the ragged batch split over the ranks: every rank takes part, rank 0 reports
    sharded = None
    if world_size > 1 and not args.no_extras:
        w.close()
        sharded = bench_batch_sharded(H, torch, dist, rank, world_size, "cuda")

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    achieved = BYTES_PER_CELL_STEP * cells / (fused_step_ms / 1e3) / 1e9
    tpc = profiled_traffic_per_cell_step()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": fused_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded simplex fBm terrain, Philox rain)",
        "config": {"workload": f"config2 erosion {n}x{n} FP32, thermal on, Bernoulli rain p=0.001",
                   "grid": n, "parallelism": f"replicas x{world_size}" if world_size > 1 else "single GPU",
                   "l2": "inputs larger than L2 (9 fields x 4 B x n^2)"},
        "plain_value": plain_value, "fused_vs_plain": value / plain_value,
        "plain_ms_per_step": plain_ms / plain_steps,
        "pct_hbm_peak": 100.0 * achieved / peak,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "kernel": "fused step = k_hydro + k_transport launch pair (50 % / 50 % of its time, ncu "
                               "launch list); achieved = 72 B x cells / ms per step",
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "traffic": tpc * cells if tpc else None,
                     "algorithmic_bytes_per_step": BYTES_PER_CELL_STEP * cells},
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "tuned": {"tile": [64, tuned[0]], "graph": bool(tuned[1]), "tuning_ms_per_step": list(tuned[2])},
        "e2e": {"value": job_throughput(world_size, cells, args.steps, e2e_s), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, **copy_rates},
    }
    # the extras and the CPU baseline are single-GPU measurements: the N = 1
    # line carries them, replica lines (N > 1) do not hold N GPUs for them
    single = world_size == 1
    cpu = 0.0 if args.no_cpu_baseline else 6.0
    if not args.no_extras and single:
        line["fwd_adjoint"] = bench_adjoint(H, torch)
        line["fwd_adjoint_4096"] = bench_adjoint_workload(H, torch)
        line["batch"] = bench_batch(H, torch)
        line["config1"] = bench_config1(H, torch, cpu=cpu > 0)
        line["large"] = bench_large(H, torch)
        line["two_layer"] = bench_two_layer(H, torch, cpu_budget_s=cpu)
        line["terrain"] = bench_terrain(H, torch, cpu_budget_s=cpu * 2.0 / 3.0)
        line["particles"] = bench_particles(H, torch, cpu_budget_s=cpu)
        line["render"] = bench_render(H, torch, cpu_budget_s=cpu)
    if sharded is not None:
        line["batch_sharded"] = sharded
    if not args.no_cpu_baseline and single:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
