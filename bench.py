"""Benchmark: RK4 node-steps/s of the OLDG field step on one GB300.

Workload (default): the 3D periodic uniform forest, P = 3, E = 4, roots = 16
(4096 blocks of 16^3, 256^3 = 16.8M nodes), the standing sine mode with
wavenumbers (1, 2, 3), dt = 0.5 h/(P+1), h = 1/256. A step is one RK4 step
of the whole forest (4 fused stage launches replayed from a CUDA graph);
the value is the median of --repeats timed regions of exactly --steps steps.

Arms: the plain FP64 path (the drop-in) and the FP32-field path with FP64
energy/time and compensated (two-sum) RK accumulation, the headline
`value`. Both run 100 steps from the same initial data outside the timed
region to state the L2 / Linf error against the exact solution and against
the FP64 run, and the energy drift. Beside them the line carries the other
configurations as sub-objects: the 512-problem 2D ensemble (`batched`), the
nested reflecting box (`nested`), the thirteen-patch benchmark ball
(`ball13`), the 2D quarter-period box (`c1`) and the seven-patch ball
(`ball7`, and at the reference's own plane wave `ball7_reference_wave`),
each with both precisions, and the kernels around the stage kernel with
their achieved bandwidth (`aux_kernels`).

--impl reference times the reference's CPU data flow (oracle/refcpu.c, a C
restatement held to the oracle; all host threads) on the same 256^3 box;
the reference itself is Julia and is not installed on this machine.

Under torchrun (N > 1) every rank runs an independent replica (the path
does not shard on one box: replicas only), a barrier brackets each timed
region, and the time is the max over ranks.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "treewaveoldg.jl_gb300"))
sys.path.insert(0, ROOT)

METRIC = "node-steps/s on 1 GB300: mixed-precision batched vs plain FP64, at equal L2 error"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--roots", type=int, default=16)
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--arms", default="f64,f32c",
                    help="comma list of the precisions to run; the headline needs f32c (profiling runs one)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="leave out the nested box, the benchmark ball and the small configurations")
    ap.add_argument("--repeats", type=int, default=10,
                    help="timed regions of exactly --steps steps each; the median is the value")
    ap.add_argument("--ball-roots", default="4,4,44",
                    help="ball13: the roots (n, m, m') of the thirteen-patch ball (the benchmark ball's 4,4,44; "
                         "a smaller m' for profiling)")
    ap.add_argument("--nested-roots", type=int, default=8,
                    help="nested: the roots per side (8: the configuration's 1408 blocks in L2; 24: 38,016 blocks, "
                         "19.5M nodes, beyond L2)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (untimed, before the warm-up) and run the default launch layouts")
    ap.add_argument("--workload", default="box256", choices=["box256", "nested", "batched", "c1", "ball", "ball13",
                                                             "transfer"],
                    help="box256: the 256^3 periodic box (the headline); nested: the 3D reflecting box with "
                         "three nested refinement levels (P=3, E=2, roots=8) and a Gaussian pulse; batched: the "
                         "512-problem 2D ensemble alone; c1: the 2D "
                         "periodic P=4, E=2, roots=8 box to a quarter period at CFL 0.25; ball: the seven-patch "
                         "ball, P=3, E=2, roots=(4,4), plane wave with Dirichlet sphere, to t=6; ball13: the "
                         "reference's benchmark ball, thirteen patches, roots (4,4,44), E=4, P=3, Lc=4, Rm=12, "
                         "R1=100, radiative sphere (19.1M nodes); transfer: the projection of two particles' "
                         "density onto the nodes over the first run's window (box of side 5, h_e = 1/8, P=3, E=4, "
                         "ell = 1e-3, R2 = 2.5)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region: the sampler is started
    and seen to report before the region begins, samples every 10 ms, and,
    for a region shorter than that, keeps the first sample after it."""

    def __init__(self, index):
        self.index = index
        self.samples = []            # (time, fields)
        self._p = None
        self.t0 = self.t1 = None

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "10"]
        try:
            self._p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            deadline = time.time() + 5
            while not self.samples and time.time() < deadline and self._p.poll() is None:
                time.sleep(0.005)
        except OSError:
            self._p = None
        self.t0 = time.time()
        return self

    def _read(self):
        for line in self._p.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def __exit__(self, *a):
        self.t1 = time.time()
        if self._p is not None:
            deadline = self.t1 + 1
            while not any(t >= self.t1 for t, _ in self.samples) and time.time() < deadline \
                    and self._p.poll() is None:
                time.sleep(0.005)
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        inside = [f for t, f in self.samples if self.t0 <= t <= self.t1]
        trailing = 0
        if not inside:
            after = [f for t, f in self.samples if t > self.t1][:1]
            inside, trailing = after, len(after)
        ok = [s for s in inside if len(s) >= 7]
        sm = [float(s[0]) for s in ok if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in ok if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in ok for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(ok) - trailing, "trailing_samples": trailing,
                "interval_ms": 10}


WORKLOAD = "box256"
TUNE = True
KERNEL_NAMES = {1: "stage3r_kernel", 2: "stage_kernel_c", 3: "stage_kernel"}
# algorithmic bytes per node-step: 34 words (+4 compensation words for f32c)
BYTES_NS = {"f64": 272.0, "f32c": 152.0}


def box_problem(twoldg, workload, roots, precision):
    """The 256^3 periodic box (P = 3, E = 4) or the nested reflecting box."""
    dtype = np.float64 if precision == "f64" else np.float32
    if workload == "nested":
        forest = twoldg.wave_forest(dtype, 3, 3, 2, roots=roots, reflecting=True,
                                    refined=twoldg.nested_cubes(3, 1 / 8, 3))
    else:
        forest = twoldg.wave_forest(dtype, 3, 3, 4, roots=roots)
    p = twoldg.WaveProblem(forest, twoldg.Element(dtype, 3), precision=precision)
    return forest, p


def box_initial(workload, x, var, T):
    if workload == "nested":
        r2 = sum((x[d] - T(0.5)) ** 2 for d in range(3))
        u = np.exp(-r2 / T(0.05) ** 2).astype(T)
        return u if var == 1 else np.zeros_like(u)
    twopi = T(2 * math.pi)
    u = np.sin(twopi * x[0]) * np.sin(twopi * T(2) * x[1]) * np.sin(twopi * T(3) * x[2])
    return u if var == 1 else np.zeros_like(u)


def c2_initial(x, var, T):
    return box_initial("box256", x, var, T)


def box_exact(workload, x, var, t, T):
    if workload == "nested":
        return None  # no closed form: errors are stated against the FP64 run
    om = 2 * math.pi * math.sqrt(14.0)
    s = np.sin(2 * math.pi * x[0]) * np.sin(4 * math.pi * x[1]) * np.sin(6 * math.pi * x[2])
    return (math.cos(om * t) * s if var == 1 else -om * math.sin(om * t) * s).astype(T)


def timed_regions(twoldg, torch, p, u, dt, steps, repeats, clocks_index, t0=0.0):
    """`repeats` timed regions of exactly `steps` RK4 steps each, every one
    bracketed by a barrier and a device synchronisation and timed with CUDA
    events on the library's own stream (max over ranks), the clock sampler
    running through all of them. An untimed call of `steps` steps at t0
    comes first: it captures the step graphs that a call of that length
    launches, so that no capture falls in a timed region (the regions start
    at t0 + steps dt). Returns (per-region ms, clock summary)."""
    lib = twoldg._lib.lib()
    ptr = ctypes.c_void_p(u.data_ptr())
    stream = torch.cuda.ExternalStream(lib.twoldg_stream(p.handle))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ptr, t0, dt, steps))
    torch.cuda.synchronize()
    times = []
    with Clocks(clocks_index) as clk:
        for r in range(repeats):
            barrier()
            torch.cuda.synchronize()
            ev0.record(stream)
            twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ptr, t0 + (r + 1) * steps * dt, dt, steps))
            ev1.record(stream)
            ev1.synchronize()
            torch.cuda.synchronize()
            times.append(max_over_ranks(ev0.elapsed_time(ev1)))
    return times, clk.summary()


def run_arm(twoldg, torch, precision, roots, steps, warmup, clocks_index, workload=None, repeats=10):
    workload = workload or WORKLOAD
    T = np.float64 if precision == "f64" else np.float32
    forest, p = box_problem(twoldg, workload, roots, precision)
    u0 = twoldg.initial_state(p, lambda x, var: box_initial(workload, x, var, T))
    dt = 0.5 * forest.minimum_spacing() / 4
    lib = twoldg._lib.lib()
    u = u0.clone()
    ptr = ctypes.c_void_p(u.data_ptr())
    torch.cuda.synchronize()
    layout = p.autotune(u, dt) if TUNE else {}
    twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ptr, 0.0, dt, warmup))
    p.synchronize()
    times, clocks = timed_regions(twoldg, torch, p, u, dt, steps, repeats, clocks_index)
    ms = float(np.median(times))
    # per-stage launch durations (the four stages launched one by one with
    # events between them, outside the step's graph)
    st = (ctypes.c_float * 4)()
    prof = []
    for _ in range(5):
        twoldg._lib.check(lib.twoldg_profile_step(p.handle, ptr, dt, st))
        prof.append(list(st))
    stage_ms = np.min(np.array(prof), axis=0)
    return dict(forest=forest, p=p, u0=u0, dt=dt, ms=ms, region_ms=times, stage_ms=stage_ms, clocks=clocks,
                nodes=p.state_words // 2, layout=layout, workload=workload, u=u)


def accuracy(twoldg, torch, arm, nsteps, ref64=None):
    p, T = arm["p"], arm["p"].dtype.type
    workload = arm["workload"]
    u = arm["u0"].clone()
    if p.precision == "f32c":
        twoldg._lib.check(twoldg._lib.lib().twoldg_reset_compensation(p.handle))
    e0 = twoldg.wave_energy(p, u)
    integ = twoldg.wave_integrator(p, u, 0.0, nsteps * arm["dt"], arm["dt"], alias_u0=True)
    integ.nsteps = nsteps
    integ.solve()
    e1 = twoldg.wave_energy(p, u)
    t = nsteps * arm["dt"]
    out = dict(energy_drift=abs(e1 - e0) / e0, steps=nsteps)
    if workload != "nested":
        ue = p.to_device(p.fill_at_nodes(lambda x, var: box_exact(workload, x, var, t, T)))
        out.update(l2=twoldg.quadrature_norm(p, u, 2, ref=ue), linf=twoldg.quadrature_norm(p, u, math.inf, ref=ue))
    if ref64 is not None:
        r = ref64.to(u.dtype)
        out["l2_vs_fp64"] = twoldg.quadrature_norm(p, u, 2, ref=r)
        out["linf_vs_fp64"] = twoldg.quadrature_norm(p, u, math.inf, ref=r)
    return out, u


def aux_kernels(twoldg, arm, hbm, reps=5):
    """Achieved HBM bandwidth of the kernels around the stage kernel, one
    launch each, timed with CUDA events on the library's stream
    (twoldg_profile_kernels; least of `reps`), against their algorithmic
    bytes: the face export reads P+1 planes per face and writes two
    (u's face node and the own element's part of its wide derivative), the
    energy reads u and v (2 words a node), the norm of u - ref reads both
    states (4), the indicator's peak reads u (1), the modal indicator reads u
    (1) and writes one word per element, the truncation reads and writes v
    (2). Coarse-fine ghosts (nested forests only) are reported as time."""
    lib = twoldg._lib.lib()
    p, u = arm["p"], arm["u"]
    W = 8 if p.precision == "f64" else 4
    forest = arm["forest"]
    N, D, P = forest.N, forest.D, 3
    nb, nodes = len(forest.leaves), arm["nodes"]
    F = N ** (D - 1)
    ms = (ctypes.c_float * 7)()
    best = [math.inf] * 7
    for _ in range(reps):
        twoldg._lib.check(lib.twoldg_profile_kernels(p.handle, ctypes.c_void_p(u.data_ptr()), ms, 7))
        best = [min(a, b) for a, b in zip(best, ms)]
    E = N // (P + 1)
    alg = {"export_faces_kernel": W * nb * 2 * D * F * (P + 1 + 2),
           "energy_kernel": W * nodes * 2, "norm_kernel": W * nodes * 4, "maxabs_kernel": W * nodes,
           "mode_staged_kernel": W * (nodes + nb * E ** D), "truncate_kernel": W * nodes * 2}
    names = ["export_faces_kernel", "cf_ghost_kernel", "energy_kernel", "norm_kernel", "maxabs_kernel",
             "mode_staged_kernel", "truncate_kernel"]
    out = {}
    for k, name in enumerate(names):
        t = best[k]
        if name in alg:
            gbs = alg[name] / (t / 1e3) / 1e9
            out[name] = {"us": t * 1e3, "algorithmic_bytes": alg[name], "achieved_gbs": gbs, "frac": gbs / hbm}
        elif t > 0:
            out[name] = {"us": t * 1e3, "bound": "latency (coarse-fine face planes only)"}
    return out


def box_object(twoldg, torch, workload, roots, steps, warmup, accuracy_steps, repeats, clocks_index, hbm):
    """Both arms of a box workload, as a sub-object of the bench line: value
    (FP32 + compensated), FP64 beside it, the roofline, accuracy against the
    FP64 run and the energy drift, and the auxiliary kernels' bandwidth."""
    arms = {prec: run_arm(twoldg, torch, prec, roots, steps, warmup, clocks_index, workload, repeats)
            for prec in ("f64", "f32c")}
    acc64, u64 = accuracy(twoldg, torch, arms["f64"], accuracy_steps)
    acc32 = accuracy(twoldg, torch, arms["f32c"], accuracy_steps, ref64=u64)[0]
    out = {}
    for prec, a in arms.items():
        mps = a["ms"] / steps
        ach = BYTES_NS[prec] * a["nodes"] / (mps / 1e3) / 1e9
        out[prec] = {"value": a["nodes"] * steps / (a["ms"] / 1e3), "ms_per_step": mps,
                     "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm},
                     "stage_ms": [float(x) for x in a["stage_ms"]], "clocks": a["clocks"],
                     "aux_kernels": aux_kernels(twoldg, a, hbm)}
    out["f64"]["accuracy"], out["f32c"]["accuracy"] = acc64, acc32
    out["f64"]["layout"], out["f32c"]["layout"] = arms["f64"]["layout"], arms["f32c"]["layout"]
    out["nodes"] = arms["f32c"]["nodes"]
    out["blocks"] = len(arms["f32c"]["forest"].leaves)
    out["steps"], out["repeats"] = steps, repeats
    out["speedup_f32c_vs_f64"] = out["f32c"]["value"] / out["f64"]["value"]
    return out


def e2e(twoldg, torch, arm, steps):
    """The same metric through the public API with host buffers: every step
    copies its input state from pinned host memory to the device, takes one
    RK4 step there and copies the result back to pinned host memory. A ring
    of NB device buffers lets a step's upload, the previous step's RK4 step
    and the download before it run at once (separate copy streams, ordered by
    events against the library's stream): with two, a buffer's upload, step
    and download form a chain that the next use of it waits on, and with
    three the host link (both directions at once) bounds the step; the last
    result read back is checked against a plain step."""
    NB = 3
    p = arm["p"]
    lib = twoldg._lib.lib()
    host_in = arm["u0"].cpu().pin_memory()
    host_out = [torch.empty_like(host_in).pin_memory() for _ in range(NB)]
    dev = [torch.empty_like(arm["u0"]) for _ in range(NB)]
    dt = arm["dt"]
    compute = torch.cuda.ExternalStream(lib.twoldg_stream(p.handle))
    cin, cout = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(NB)]
    ev_done = [torch.cuda.Event() for _ in range(NB)]
    ev_out = [torch.cuda.Event() for _ in range(NB)]

    def step(k):
        b = k % NB
        with torch.cuda.stream(cin):
            if k >= NB:
                cin.wait_event(ev_out[b])        # that buffer's last download is done
            dev[b].copy_(host_in, non_blocking=True)
            ev_in[b].record(cin)
        compute.wait_event(ev_in[b])
        twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ctypes.c_void_p(dev[b].data_ptr()), 0.0, dt, 1))
        ev_done[b].record(compute)
        with torch.cuda.stream(cout):
            cout.wait_event(ev_done[b])
            host_out[b].copy_(dev[b], non_blocking=True)
            ev_out[b].record(cout)

    for k in range(NB):                          # capture every buffer's step graph
        step(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        step(k)
    torch.cuda.synchronize()
    sec = max_over_ranks(time.perf_counter() - t0)
    check = arm["u0"].clone()
    twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ctypes.c_void_p(check.data_ptr()), 0.0, dt, 1))
    p.synchronize()
    if not torch.equal(check.cpu(), host_out[(steps - 1) % NB]):
        raise RuntimeError("the pipelined end-to-end step differs from a plain step")
    nbytes = dev[0].numel() * dev[0].element_size()
    return dict(value=arm["nodes"] * steps / sec * world(), unit="node-steps/s",
                h2d_bytes_per_step=nbytes, d2h_bytes_per_step=nbytes, pipelined="%d device buffers" % NB)


def batched(twoldg, torch, steps, warmup, accuracy_steps, n=512, repeats=5):
    """The batched ensemble: n 2D periodic problems of uneven P, E and roots
    (seeded), all stepped by one graph launch per RK4 step; FP64 and FP32 +
    compensated node-steps/s, and the L2 difference of the two after
    accuracy_steps steps relative to the FP64 state's L2 norm."""
    out = {}
    states = {}
    for prec in ("f64", "f32c"):
        dtype = np.float64 if prec == "f64" else np.float32
        members = twoldg.sine_ensemble(n, seed=0, dtype=dtype)
        b = twoldg.Batch([(f, P) for f, P, _ in members], precision=prec)
        u0 = twoldg.fill_batch(b, members)
        dts = [0.5 * f.minimum_spacing() / (P + 1) for f, P, _ in members]
        u = u0.clone()
        if TUNE:
            out.setdefault("layout", {}).update(b.autotune(u, dts))
        # warm-up, then one untimed call of the timed region's length, which
        # captures its step graphs (a batch takes up to 16 steps a graph)
        b.rk4_step(u, dts, warmup)
        b.rk4_step(u, dts, steps)
        b.synchronize()
        stream = b.stream()
        arr = (ctypes.c_double * len(dts))(*[float(x) for x in dts])
        regions = []
        for _ in range(repeats):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            twoldg._lib.check(twoldg._lib.lib().twoldg_batch_rk4_step(b._h, ctypes.c_void_p(u.data_ptr()), arr,
                                                                      steps))
            e1.record(stream)
            e1.synchronize()
            regions.append(e0.elapsed_time(e1))
        sec = float(np.median(regions)) / 1e3
        ach = BYTES_NS[prec] * b.nodes * steps / sec / 1e9
        out[prec] = {"value": b.nodes * steps / sec, "ms_per_step": sec * 1e3 / steps,
                     "achieved_gbs": ach, "region_ms": regions,
                     "timing": "median of %d timed regions of %d RK4 steps (CUDA events on the batch's stream)"
                               % (repeats, steps)}
        if accuracy_steps:
            v = u0.clone()
            b.rk4_step(v, dts, accuracy_steps)
            b.synchronize()
            states[prec] = v.double()
        out["members"] = n
        out["nodes"] = b.nodes
        out["shapes"] = len({(P, f.N) for f, P, _ in members})
    if accuracy_steps:
        d = states["f32c"] - states["f64"]
        out["l2_f32c_vs_f64_rel"] = float(torch.linalg.norm(d) / torch.linalg.norm(states["f64"]))
        out["accuracy_steps"] = accuracy_steps
    out["speedup_f32c_vs_f64"] = out["f32c"]["value"] / out["f64"]["value"]
    return out


# --- the small configurations: whole runs to t_end, FP64 against FP32 + compensated ---------
def small_problem(twoldg, prec, workload=None):
    """(problem, u0, dt, nsteps, t_end, exact(t) -> device state) of the c1 or
    ball workload; ball_ref is the seven-patch ball at the reference's own
    plane wave, k = (1.1, -0.7, 0.5), to t = 1 (src/sevenpatch.jl:84-117)."""
    workload = workload or WORKLOAD
    T = np.float64 if prec == "f64" else np.float32
    if workload == "c1":
        forest = twoldg.wave_forest(T, 2, 4, 2, roots=8)
        p = twoldg.WaveProblem(forest, twoldg.Element(T, 4), precision=prec)
        u0 = twoldg.initial_state(p, twoldg.wave_exact(2, 1.0, 1, 0.0, T))
        t_end, cfl = 0.25 * 2 * math.pi / twoldg.wave_omega(2, 1.0, 1), 0.25

        def exact(t):
            return p.to_device(p.fill_at_nodes(twoldg.wave_exact(2, 1.0, 1, t, T)))
    else:
        forest, geo = twoldg.sevenpatch_forest(T, 3, 2, roots=(4, 4), Lc=1.0, R1=3.0)
        k = np.array([1.1, -0.7, 0.5])
        if workload == "ball_ref":
            wave = twoldg.PlaneWave(k, 0.3)
            t_end, cfl = 1.0, 0.5
        else:
            wave = twoldg.PlaneWave(2 * math.pi * k / np.linalg.norm(k), 0.3)
            t_end, cfl = 6.0, 0.5
        p = twoldg.WaveProblem(forest, twoldg.Element(T, 3), geometry=geo, boundary=wave, precision=prec)
        u0 = twoldg.initial_state(p, twoldg.sevenpatch_exact(geo, wave, 0.0))

        def exact(t):
            return p.to_device(p.fill_at_nodes(twoldg.sevenpatch_exact(geo, wave, t)))
    nsteps = int(math.ceil(T(t_end) / twoldg.oldg_timestep(p, cfl)))
    dt = float(T(T(t_end) / T(nsteps)))
    return p, u0, dt, nsteps, float(T(t_end)), exact


SMALL_NAMES = {
    "c1": "2D periodic box, P=4, E=2, roots=8 (6400 nodes), sin(2 pi x) sin(2 pi y) to a quarter period at CFL 0.25",
    "ball": "seven-patch ball, P=3, E=2, roots=(4,4), Lc=1, R1=3 (%d nodes), plane wave |k|=2 pi along "
            "(1.1,-0.7,0.5), phi=0.3, Dirichlet sphere, to t=6 at CFL 0.5",
    "ball_ref": "seven-patch ball, P=3, E=2, roots=(4,4), Lc=1, R1=3 (%d nodes), the reference's plane wave "
                "k=(1.1,-0.7,0.5), phi=0.3, Dirichlet sphere, to t=1 at CFL 0.5",
}


def small_run(twoldg, torch, workload, reps):
    """Both arms of a small configuration: node-steps/s of the whole run to
    t_end (CUDA events on the library's stream, least of `reps` runs after a
    warm-up run), the L2 and Linf errors against the exact solution and
    against the FP64 run, and the energy drift."""
    lib = twoldg._lib.lib()
    arms, final = {}, {}
    for prec in ("f64", "f32c"):
        p, u0, dt, nsteps, t_end, exact = small_problem(twoldg, prec, workload)
        u = u0.clone()
        layout = p.autotune(u, dt) if TUNE else {}
        stream = torch.cuda.ExternalStream(lib.twoldg_stream(p.handle))
        best = math.inf
        for rep in range(1 + reps):
            u = u0.clone()
            if prec == "f32c":
                twoldg._lib.check(lib.twoldg_reset_compensation(p.handle))
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ctypes.c_void_p(u.data_ptr()), 0.0, dt, nsteps))
            ev1.record(stream)
            ev1.synchronize()
            if rep > 0:
                best = min(best, ev0.elapsed_time(ev1))
        nodes = p.state_words // 2
        ue = exact(t_end)
        e0, e1 = twoldg.wave_energy(p, u0, t=0.0), twoldg.wave_energy(p, u, t=t_end)
        arms[prec] = {"value": nodes * nsteps / (best / 1e3), "ms_per_step": best / nsteps, "nsteps": nsteps,
                      "nodes": nodes, "layout": layout,
                      "l2": twoldg.quadrature_norm(p, u, 2, ref=ue),
                      "l2u": twoldg.quadrature_norm(p, u, 2, vars=(1,), ref=ue),
                      "l2v": twoldg.quadrature_norm(p, u, 2, vars=(2,), ref=ue),
                      "linf": twoldg.quadrature_norm(p, u, math.inf, ref=ue),
                      "energy_drift": abs(e1 - e0) / abs(e0)}
        final[prec] = (p, u)
    p32, u32 = final["f32c"]
    r = final["f64"][1].to(u32.dtype)
    arms["f32c"]["l2_vs_fp64"] = twoldg.quadrature_norm(p32, u32, 2, ref=r)
    arms["f32c"]["linf_vs_fp64"] = twoldg.quadrature_norm(p32, u32, math.inf, ref=r)
    name = SMALL_NAMES[workload]
    if "%d" in name:
        name = name % arms["f32c"]["nodes"]
    return {"workload": name, "fp64": arms["f64"], "f32c": arms["f32c"],
            "speedup_f32c_vs_f64": arms["f32c"]["value"] / arms["f64"]["value"],
            "l2_flush": "none: the state fits in L2 (a whole run to t_end is timed)"}


def small_config(args, twoldg, torch):
    res = small_run(twoldg, torch, WORKLOAD, max(1, args.steps // 50))
    head = res["f32c"]
    line = {"metric": METRIC, "value": head["value"], "unit": "node-steps/s", "n_gpus": 1,
            "steps": head["nsteps"], "warmup": 1, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": res["workload"], "precision": "f32c", "l2_flush": res["l2_flush"]},
            "fp64": res["fp64"], "f32c": res["f32c"], "speedup_vs_fp64": res["speedup_f32c_vs_f64"],
            "roofline": None, "gpu_launches": None}
    print(json.dumps(line))


def ball13_run(twoldg, torch, roots, steps, warmup, repeats=3):
    """The reference's benchmark ball (bin/ball_benchmark.jl): the
    thirteen-patch ball of 4672 blocks of 16^3 (roots (4, 4, 44), Lc = 4,
    Rm = 12, R1 = 100), P = 3, Sommerfeld's radiative sphere, truncation on,
    the state sin(1), sin(2), ... truncated; `repeats` timed regions of
    `steps` RK4 steps at cfl 1/2 with CUDA events on the library's stream,
    FP64 and FP32 + compensated, and the FP32 run's L2 distance from the FP64
    one and the two energies after the warm-up, priming and timed steps."""
    lib = twoldg._lib.lib()
    forest, geo = twoldg.thirteenpatch_forest(np.float64, 3, 4, roots=roots, Lc=4.0, Rm=12.0, R1=100.0)
    hbm, _ = peaks()
    arms, final = {}, {}
    for prec in ("f64", "f32c"):
        T = np.float64 if prec == "f64" else np.float32
        p = twoldg.WaveProblem(forest, twoldg.Element(T, 3), geometry=geo, boundary=twoldg.RadiativeBoundary(),
                               precision=prec)
        u = torch.from_numpy(np.sin(np.arange(1, p.state_words + 1, dtype=np.float64)).astype(T)).cuda()
        twoldg.truncate_state(u, p)
        e0 = twoldg.wave_energy(p, u, t=0.0)
        dt = float(twoldg.oldg_timestep(p, 0.5))
        ptr = ctypes.c_void_p(u.data_ptr())
        torch.cuda.synchronize()
        twoldg._lib.check(lib.twoldg_rk4_step(p.handle, ptr, 0.0, dt, warmup))
        p.synchronize()
        times, clocks = timed_regions(twoldg, torch, p, u, dt, steps, repeats, 0, t0=warmup * dt)
        ms = float(np.median(times))
        nodes = p.state_words // 2
        st = (ctypes.c_float * 4)()
        v = u.clone()
        twoldg._lib.check(lib.twoldg_profile_step(p.handle, ctypes.c_void_p(v.data_ptr()), dt, st))
        t1 = (warmup + (repeats + 1) * steps) * dt
        mps = ms / steps
        ach = BYTES_NS[prec] * nodes / (mps / 1e3) / 1e9
        arms[prec] = {"value": nodes * steps / (ms / 1e3), "ms_per_step": mps,
                      "ns_per_node_step": mps * 1e6 / nodes, "stage_ms": [float(x) for x in st],
                      "nodes": nodes, "dt": dt, "clocks": clocks,
                      "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                                   "note": "the flat step's algorithmic bytes (the minimum RK4 data flow); the full metric reads "
                                           "fluxes and sqrt(g) besides"},
                      "energy0": e0, "energy": twoldg.wave_energy(p, u, t=t1)}
        final[prec] = (p, u)
    p32, u32 = final["f32c"]
    r = final["f64"][1].to(torch.float32)
    arms["f32c"]["l2_vs_fp64"] = float(twoldg.quadrature_norm(p32, u32, 2, ref=r))
    arms["f32c"]["energy_vs_fp64"] = abs(arms["f32c"]["energy"] - arms["f64"]["energy"]) / arms["f64"]["energy"]
    return {"workload": "the benchmark ball: thirteen-patch, roots %s, E=4, P=3, Lc=4, Rm=12, R1=100 (%d blocks "
                        "of 16^3, %d nodes), Sommerfeld radiative sphere, truncation on, state sin(1..n) truncated, "
                        "cfl 1/2" % (roots, forest.nleaves(), arms["f32c"]["nodes"]),
            "fp64": arms["f64"], "f32c": arms["f32c"], "steps": steps, "repeats": repeats,
            "speedup_f32c_vs_f64": arms["f32c"]["value"] / arms["f64"]["value"],
            "reference_h200_ns_per_node_step": {"f64": 2.84, "f32": 1.92, "source": "CODE.md:5108-5122"},
            "gpu_launches_per_step": 9}


def ball_benchmark(args, twoldg, torch):
    roots = tuple(int(x) for x in args.ball_roots.split(","))
    res = ball13_run(twoldg, torch, roots, args.steps, args.warmup, repeats=1)
    head = res["f32c"]
    line = {"metric": METRIC, "value": head["value"], "unit": "node-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": res["workload"], "precision": "f32c", "l2_flush": "inputs larger than L2"},
            "fp64": res["fp64"], "f32c": res["f32c"], "speedup_vs_fp64": res["speedup_f32c_vs_f64"],
            "reference_h200_ns_per_node_step": res["reference_h200_ns_per_node_step"],
            "clocks": head["clocks"], "roofline": head["roofline"], "gpu_launches": 1 + 9 * args.steps}
    print(json.dumps(line))


def transfer_setup(twoldg, T=np.float64, hdiv=8):
    """The first run's transfer (bin/projection.jl, CODE.md "Quadrature"): two
    opposite charges Q = +-sqrt(0.005), ell = 1e-3, on a circle of diameter 1
    at v = 0.2, moved off the element corners by (0.31, 0.17, 0.43) h_e, in a
    periodic box of side 5 with h_e = 1/hdiv, P = 3, E = 4; the source's ball
    is the window's, R2 = 2.5 about the centre."""
    roots = 5 * hdiv // 4
    forest = twoldg.wave_forest(T, 3, 3, 4, roots=roots, L=5.0)
    p = twoldg.WaveProblem(forest, twoldg.Element(T, 3))
    he = 1.0 / hdiv
    c = np.array([2.5, 2.5, 2.5])
    off = np.array([0.31, 0.17, 0.43]) * he
    q = math.sqrt(0.005)
    parts = [twoldg.ParticleSupport(c + np.array([0.5, 0, 0]) + off, (0.0, 0.2, 0.0), 1e-3, charge=q),
             twoldg.ParticleSupport(c - np.array([0.5, 0, 0]) + off, (0.0, -0.2, 0.0), 1e-3, charge=-q)]
    return p, parts, (c, 2.5)


def transfer_benchmark(args, twoldg, torch, record=True):
    """Projections of the first run's two particles: the library's plan (host),
    then K projections of their density (evaluated in the kernels) and of a
    caller's values at the plan's points, each timed alone with CUDA events on
    the library's stream and L2 flushed in between; the far rule's oracle on a
    sample of elements for the CPU baseline."""
    lib = twoldg._lib.lib()
    p, parts, ball = transfer_setup(twoldg)
    t0 = time.perf_counter()
    plan = twoldg.TransferPlan(p, parts, ball)
    plan_s = time.perf_counter() - t0
    # the plan for moved particles, as an inspiral's right-hand side redoes it
    # at every stage: the pair turned about the centre by 1e-3 rad per update
    upd = []
    for k in range(1, 8):
        ang = 1e-3 * k
        rot = np.array([[math.cos(ang), -math.sin(ang), 0], [math.sin(ang), math.cos(ang), 0], [0, 0, 1]])
        moved = [twoldg.ParticleSupport(ball[0] + rot @ (np.array(s.z) - ball[0]), rot @ np.array(s.v), s.ell,
                                        charge=s.charge) for s in parts]
        t0 = time.perf_counter()
        plan.update(moved)
        upd.append(time.perf_counter() - t0)
    plan.update(parts)
    c = plan.counts
    stream = torch.cuda.ExternalStream(lib.twoldg_stream(p.handle))
    du = p.statevector()
    xs = plan.points()
    r = ((xs - 2.5) ** 2).sum(0).sqrt()
    values = (torch.cos(3 * r) * torch.exp(-r)).contiguous()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    times = {"density": [], "values": []}
    for kind in ("density", "values"):
        for it in range(args.warmup + args.steps):
            flush.fill_(float(it))
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            if kind == "density":
                twoldg._lib.check(lib.twoldg_project_density(plan._h, ctypes.c_void_p(du.data_ptr()), -1.0, 2))
            else:
                twoldg._lib.check(lib.twoldg_project_values(plan._h, ctypes.c_void_p(values.data_ptr()),
                                                            ctypes.c_void_p(du.data_ptr()), -1.0, 2))
            ev1.record(stream)
            ev1.synchronize()
            if it >= args.warmup:
                times[kind].append(ev0.elapsed_time(ev1))
    ms = {k: float(np.median(v)) for k, v in times.items()}
    # the pairing of each particle's (grad rho, rho) with a field (the
    # inspiral's force), host-visible latency: the first after the particles
    # move builds the supports' compact rule and the kernel's moments, every
    # later one gathers, sums and copies 8 numbers back
    t0 = time.perf_counter()
    plan.pairing(du, 1, True)
    pair_first = time.perf_counter() - t0
    pair = []
    for _ in range(20):
        t0 = time.perf_counter()
        plan.pairing(du, 1, True)
        pair.append(time.perf_counter() - t0)
    # algorithmic bytes of the values path: each point's value read once, the
    # touched elements' nodes read and written, the nested rule's points and
    # weights read
    M = 64
    elems = c["far_elements"] + c["graded_elements"] + c["near_elements"]
    alg = 8 * c["points"] + 2 * 8 * M * elems + 4 * 8 * c["near_points"]
    hbm, peak_kind = peaks()
    out = {"workload": "first-run window: 2 particles (Q = +-sqrt(0.005), ell = 1e-3, v = 0.2, off the corners), "
                       "box of side 5, h_e = 1/8, P=3, E=4 (%d blocks of 16^3), ball R2 = 2.5" % p.nblocks,
           "counts": c, "plan_ms": plan_s * 1e3, "plan_update_ms": float(np.median(upd)) * 1e3,
           "host_threads": os.cpu_count(), "projection_ms": ms,
           "points_per_s": {k: c["points"] / (v / 1e3) for k, v in ms.items()},
           "values_roofline": {"bound": "hbm", "achieved": alg / (ms["values"] / 1e3) / 1e9, "peak": hbm,
                               "unit": "GB/s", "frac": alg / (ms["values"] / 1e3) / 1e9 / hbm,
                               "algorithmic_bytes": alg, "peak_kind": peak_kind},
           "gpu_launches_per_projection": 3,
           "pairing_ms": {"first_after_update": pair_first * 1e3, "steady": float(np.median(pair)) * 1e3}}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = transfer_cpu_sample(p, parts, ball, plan)
    plan.close()
    return out


def transfer_cpu_sample(p, parts, ball, plan):
    """The oracle's projection of the same density on a sample (200 far-rule
    elements and one nested-rule element, the particle's own), scaled by the
    plan's element counts to one projection; one host thread."""
    from oracle import transfer as OT
    f = p.forest
    mesh = OT.Mesh([[f.block_extent(k)[d][0] for d in range(3)] for k in f.leaves],
                   [f.spacing(k) for k in f.leaves], 3, 4)
    t = OT.Tables(3)

    def S(X):
        return sum(OT.particle_density(X, s.z, s.v, s.ell, s.charge) for s in parts)

    blocks = list(range(mesh.nblocks))[::97][:8]
    elems = [(b, e) for b in blocks for e in [(0, 0, 0), (1, 2, 3), (3, 3, 3), (2, 1, 0)]]
    elems = (elems * 8)[:200]
    t0 = time.perf_counter()
    for b, e in elems:
        lo, hi = mesh.element_box(b, e)
        OT.tensor_rule(S, t.far, lo, hi, 3)
    far_s = (time.perf_counter() - t0) / len(elems)
    s0 = parts[0]
    he = 0.125
    lo = [math.floor(s0.z[d] / he) * he for d in range(3)]
    hi = [x + he for x in lo]
    sup = OT.Support(s0.z, s0.v, s0.ell)
    t0 = time.perf_counter()
    OT.nested_rule(lambda X: S(X)[:, None] * t.element_basis(lo, hi, X), sup, t, lo, hi, 3)
    near_s = time.perf_counter() - t0
    c = plan.counts
    total = far_s * (c["far_elements"] + c["graded_elements"]) + near_s * c["near_elements"]
    return {"value": 1.0 / total, "unit": "projections/s", "cores": 1, "kind": "port",
            "sample": "the oracle's far rule on 200 elements and its nested rule on the particle's own element, "
                      "scaled by the plan's counts (far and graded elements at the far rule's cost, near elements "
                      "at the particle's element's)", "seconds_per_projection": total}


# --- multi-rank plumbing (replicas) -------------------------------------------
_dist = None


def world():
    return int(os.environ.get("WORLD_SIZE", "1"))


def rank():
    return int(os.environ.get("RANK", "0"))


def init_dist(torch):
    global _dist
    if world() > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        _dist = dist


def barrier():
    if _dist is not None:
        _dist.barrier()


def max_over_ranks(x):
    if _dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], device="cuda" if torch.cuda.is_available() else "cpu")
    _dist.all_reduce(t, op=_dist.ReduceOp.MAX)
    return float(t.item())


# --- CPU baseline: the reference's CPU data flow, restated (oracle/refcpu.c) ----
# The reference's own published CPU rates for this box: one EPYC 7532 core
# steps it in 2.35 s (7.1e6 node-steps/s, CODE.md:5026), 64 cores in 72.1 ms
# (2.3e8, CODE.md:5013-5026; 4.23 ns per node-step, CODE.md:5077).
PUBLISHED_CPU = {"per_core": 16777216 / 2.35, "cores_64": 16777216 / 0.0721,
                 "source": "reference CODE.md:5013-5026 (EPYC 7532, Julia 1.13, threads pinned)"}


def _c2_cpu_state(forest):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cases import state_from
    return state_from(forest, 3, lambda x, var: c2_initial(x, var, np.float64))


class CpuBox:
    """The 256^3 box on the reference's CPU data flow (FP64, OpenMP over
    blocks on every host thread), stepped in place."""

    def __init__(self, roots=16):
        from oracle import refcpu
        import twoldg
        self.refcpu = refcpu
        self.forest = twoldg.wave_forest(np.float64, 3, 3, 4, roots=roots)
        self.r = refcpu.RefCPU(self.forest, 3)
        self.u = self.r.truncate(_c2_cpu_state(self.forest))
        self.dt = 0.5 * self.forest.minimum_spacing() / 4
        self.nodes = len(self.forest.leaves) * self.forest.N ** 3

    def step(self, n=1):
        t0 = time.perf_counter()
        self.r.rk4(self.u, self.dt, n, inplace=True)
        return time.perf_counter() - t0


def per_core_rate(steps=3):
    """One host thread on an 8^3-block sample of the box (2.1M nodes, the same
    16^3 blocks), in node-steps/s."""
    from oracle import refcpu
    n = refcpu.threads()
    refcpu.set_threads(1)
    try:
        box = CpuBox(roots=8)
        box.step(1)
        sec = box.step(steps)
        return box.nodes * steps / sec
    finally:
        refcpu.set_threads(n)


def cpu_sample(steps=5):
    """The CPU baseline on the benchmark's own forest: `steps` RK4 steps of the
    whole 256^3 box on every host thread, and the rate of one thread."""
    box = CpuBox()
    box.step(1)  # warm-up (page-in, thread pool)
    sec = box.step(steps)
    cores = box.refcpu.threads()
    return dict(value=box.nodes * steps / sec, unit="node-steps/s", cores=cores, kind="port",
                per_core=per_core_rate(), same_config=True, published=PUBLISHED_CPU,
                sample="%d RK4 step(s) of the whole 3D P=3 E=4 periodic box (4096 blocks of 16^3, %d nodes), "
                       "FP64, the reference's CPU data flow (oracle/refcpu.c: scatter, ghost fill, gradient pass, "
                       "ghost fill, Laplacian pass; rank-one truncation; fused RK4 broadcasts), OpenMP over "
                       "blocks; per_core: one thread on an 8^3-block sample" % (steps, box.nodes))


def reference_arm(args):
    if rank() != 0:
        return
    import torch  # noqa: F401
    box = CpuBox()
    for _ in range(args.warmup):
        box.step(1)
    times = [box.step(1) for _ in range(args.steps)]
    value = box.nodes / float(np.median(times))
    cores = box.refcpu.threads()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "node-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "ms_per_step": float(np.median(times)) * 1e3,
            "config": {"workload": "3D periodic uniform forest, P=3, E=4, roots=16 (4096 blocks of 16^3, %d nodes), "
                                   "standing sine mode (1,2,3), dt=0.5h/(P+1); each step one RK4 step of the whole "
                                   "box (median over the steps)" % box.nodes},
            "cpu_baseline": {"value": value, "unit": "node-steps/s", "cores": cores, "kind": "port",
                             "same_config": True, "published": PUBLISHED_CPU,
                             "sample": "one RK4 step of the whole 256^3 box per step, FP64, the reference's CPU "
                                       "data flow restated in C (oracle/refcpu.c), OpenMP over blocks on %d "
                                       "threads" % cores},
            "e2e": {"value": value, "unit": "node-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (Julia + TreeAMR + CUDA.jl) cannot run on this machine; its CPU data flow is "
                    "timed through a C restatement held to the oracle at 1e-12 (tests/test_refcpu.py)"}
    print(json.dumps(line))


def traffic_from_profiles(precision):
    """DRAM bytes per stage launch measured by ncu for this workload
    (profiles/stage_kernel_traffic.txt: "<precision> <bytes>" lines)."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2 and parts[0] == precision:
                return float(parts[1])
    return None


def main():
    args = parse()
    global WORKLOAD, TUNE
    WORKLOAD = args.workload
    TUNE = not args.no_tune
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch
    import twoldg
    init_dist(torch)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    twoldg.build()
    if WORKLOAD in ("c1", "ball"):
        small_config(args, twoldg, torch)
        return
    if WORKLOAD == "ball13":
        ball_benchmark(args, twoldg, torch)
        return
    if WORKLOAD == "transfer":
        tr = transfer_benchmark(args, twoldg, torch)
        ms = tr["projection_ms"]["values"]
        line = {"metric": "projections/s (a caller's source at every point of the first run's window: 10.95M "
                          "points, far, graded and nested rules)",
                "value": 1e3 / ms, "unit": "projections/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": tr["workload"], "l2_flush": "64 MB written between "
                                                "projections"},
                "transfer": tr, "roofline": tr["values_roofline"], "gpu_launches": 3 * args.steps}
        if "cpu_baseline" in tr:
            line["cpu_baseline"] = tr["cpu_baseline"]
        print(json.dumps(line))
        return
    if WORKLOAD == "batched":
        hbm, _ = peaks()
        bat = batched(twoldg, torch, args.steps, args.warmup, args.accuracy_steps)
        head = bat["f32c"]
        line = {"metric": METRIC, "value": head["value"], "unit": "node-steps/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "the batched ensemble: %d 2D periodic problems, P 2-5, E 2/4, roots 4-16 "
                                       "(seeded), %d nodes in %d shapes, FP32 fields + compensated RK4"
                                       % (bat["members"], bat["nodes"], bat["shapes"]), "precision": "f32c",
                           "l2_flush": "inputs larger than L2 (state %.0f MB + stage scratch)" % (bat["nodes"] * 8 / 1e6)},
                "batched": bat,
                "roofline": {"bound": "hbm", "achieved": head["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                             "frac": head["achieved_gbs"] / hbm},
                "gpu_launches": None}
        print(json.dumps(line))
        return
    if WORKLOAD == "nested":
        hbm, _ = peaks()
        obj = box_object(twoldg, torch, "nested", args.nested_roots, args.steps, args.warmup, args.accuracy_steps,
                         args.repeats, local, hbm)
        head = obj["f32c"]
        state_mb = obj["nodes"] * 2 * 4 / 1e6
        line = {"metric": METRIC, "value": head["value"], "unit": "node-steps/s", "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "3D reflecting box, nested cubes 1/8, 1/4, 1/2 (3 levels), P=3, E=2, roots=%d "
                                       "(%d blocks, %d nodes), Gaussian pulse, FP32 fields + compensated RK4"
                                       % (args.nested_roots, obj["blocks"], obj["nodes"]), "precision": "f32c",
                           "l2_flush": "none: the state fits in L2" if state_mb < 64 else
                                       "inputs larger than L2 (state %.0f MB + stage scratch)" % state_mb},
                "nested": obj, "roofline": head["roofline"], "clocks": head["clocks"],
                "gpu_launches": None}
        print(json.dumps(line))
        return
    arms = {}
    wanted = args.arms.split(",")
    for prec in ("f64", "f32c"):
        if prec in wanted:
            arms[prec] = run_arm(twoldg, torch, prec, args.roots, args.steps, args.warmup, local,
                                 repeats=args.repeats)
    if set(wanted) != {"f64", "f32c"}:
        # a partial run (profiling): report the arms' times only
        if rank() == 0:
            print(json.dumps({k: {"ms_per_step": v["ms"] / args.steps, "stage_ms": [float(x) for x in v["stage_ms"]],
                                  "layout": v["layout"]} for k, v in arms.items()}))
        return
    acc64, u64 = (None, None) if args.accuracy_steps == 0 else accuracy(twoldg, torch, arms["f64"], args.accuracy_steps)
    acc32 = None if args.accuracy_steps == 0 else accuracy(twoldg, torch, arms["f32c"], args.accuracy_steps,
                                                           ref64=u64)[0]
    # at least 20 pipelined steps: with fewer, filling and draining the
    # two-buffer pipeline is a visible share of the timed region
    ee = None if args.no_e2e else e2e(twoldg, torch, arms["f32c"], max(20, args.steps))
    bat = None if args.no_batched else batched(twoldg, torch, max(10, args.steps // 4), args.warmup,
                                               args.accuracy_steps)
    hbm, peak_kind = peaks()
    head = arms["f32c"]
    nodes = head["nodes"]
    mps = head["ms"] / args.steps
    value = nodes / (mps / 1e3) * world()
    v64 = nodes / (arms["f64"]["ms"] / args.steps / 1e3) * world()
    # the stage kernel's average launch over the timed region: a step is its
    # four launches back to back in the step's graph (and one face export per
    # rk4_step call), so a launch averages a quarter of a step
    achieved = BYTES_NS["f32c"] * nodes / (mps / 1e3) / 1e9
    ach64 = BYTES_NS["f64"] * nodes / (arms["f64"]["ms"] / args.steps / 1e3) / 1e9
    stage = head["stage_ms"]
    traffic = traffic_from_profiles("f32c")
    chosen = next(iter(head["layout"].values()), {"kernel": 1})
    kname = "%s (3D, P=3, E=4, float, compensated)" % KERNEL_NAMES.get(chosen["kernel"], "stage3r_kernel")
    line = {
        "metric": METRIC, "value": value, "unit": "node-steps/s", "n_gpus": world(), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3D periodic uniform forest, P=3, E=4, roots=%d (%d blocks of 16^3, %d nodes), "
                               "standing sine mode (1,2,3), dt=0.5h/(P+1), FP32 fields + compensated RK4"
                               % (args.roots, len(head["forest"].leaves), nodes),
                   "precision": "f32c", "parallelism": "replicas" if world() > 1 else "single",
                   "l2_flush": "inputs larger than L2 (state %.0f MB + stage scratch)" % (nodes * 8 / 1e6),
                   "timing": "median of %d timed regions of exactly %d RK4 steps each (CUDA events on the "
                             "library's stream, barrier and synchronisation around each)" % (args.repeats, args.steps)},
        "region_ms": head["region_ms"],
        "fp64": {"value": v64, "ms_per_step": arms["f64"]["ms"] / args.steps, "region_ms": arms["f64"]["region_ms"],
                 "stage_ms": [float(x) for x in arms["f64"]["stage_ms"]],
                 "roofline_frac": ach64 / hbm, "layout": arms["f64"]["layout"],
                 "aux_kernels": aux_kernels(twoldg, arms["f64"], hbm),
                 "bound": "the FP64 pipe, not HBM (ncu: 84% FP64-pipe activity per stage, "
                          "profiles/stage3r_f64_256cube.md); roofline_frac is the HBM fraction"},
        "speedup_vs_fp64": value / v64,
        "accuracy": {"fp64": acc64, "f32c": acc32},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_kind": peak_kind, "kernel": kname, "layout": head["layout"],
                     "achieved_from": "the timed region: 152 B/node-step x nodes / ms_per_step, i.e. the minimum RK4 "
                                      "data flow's algorithmic bytes per stage launch over the average launch (a "
                                      "quarter step)",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per stage launch, "
                                       "profiles/stage3r_f32c_256cube.md",
                     "stage_ms": [float(x) for x in stage],
                     "stage_ms_source": "twoldg_profile_step: the four stages launched one by one outside the "
                                        "step's graph with events between them; their sum exceeds the graph's step "
                                        "by the launch gaps the graph removes"},
        "aux_kernels": aux_kernels(twoldg, head, hbm),
        "clocks": head["clocks"],
        "e2e": ee,
        "batched": bat,
        "gpu_launches": args.repeats * (1 + 4 * args.steps),
    }
    if not args.no_extra:
        line["nested"] = box_object(twoldg, torch, "nested", 8, 100, args.warmup, args.accuracy_steps, 5, local, hbm)
        line["nested"]["workload"] = ("3D reflecting box, nested cubes 1/8, 1/4, 1/2 (3 levels), P=3, E=2, roots=8 "
                                      "(8^3 blocks), Gaussian pulse exp(-r^2/0.05^2), dt=0.5h_min/(P+1); the state "
                                      "fits in L2, so the roofline bounds it from above only")
        # the same refinement at a size beyond L2 (roots 24: 38016 blocks,
        # 19.5M nodes, like the 256^3 box), where HBM bounds the refined path
        line["nested_large"] = box_object(twoldg, torch, "nested", 24, 20, args.warmup, min(20, args.accuracy_steps),
                                          3, local, hbm)
        line["nested_large"]["workload"] = ("the nested box's refinement (nested cubes 1/8, 1/4, 1/2, P=3, E=2) on "
                                            "roots=24: 38016 blocks, 19.5M nodes, state beyond L2")
        line["ball13"] = ball13_run(twoldg, torch, (4, 4, 44), 20, args.warmup, repeats=3)
        line["c1"] = small_run(twoldg, torch, "c1", 2)
        line["ball7"] = small_run(twoldg, torch, "ball", 2)
        line["ball7_reference_wave"] = small_run(twoldg, torch, "ball_ref", 1)
    if rank() == 0 and world() == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(5)
    if rank() == 0:
        print(json.dumps(line))
    if _dist is not None:
        _dist.destroy_process_group()


if __name__ == "__main__":
    main()
