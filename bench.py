"""Benchmark: PD-IPC cloth steps/s on GB300 (512x512 cloth onto an icosphere).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp32|fp64|mixed] [--config c1|c0]

One step = PdIpcSimulator::run(frame) on the 512x512 workload: prediction,
outer CCD iterations (each 20 local-global iterations of 15 Chebyshev-Jacobi
R2 sweeps, CCD, contact), velocity update.  `value` is device time from CUDA
events recorded on the library's own stream around every step (L2 flushed
between steps); `e2e` is wall time through the C ABI with host buffers: the
initial state uploaded from host memory (pdipc_set_state), then per step
BaseSimulator::animate (step + postRun copy of all positions to host memory).  With torchrun
(N > 1) every rank steps an independent replica on its own GPU (the path does
not shard: "replicas only"); the value is all replicas' steps over the slowest
rank's time.

--impl reference times the CPU restatement of the reference algorithm (the
reference has no CPU path; its CUDA kernels, built for the host under an
emulation of the CUDA execution model, pin the restatement but would time the
emulation, not an implementation) on every host core: whole
steps 0..K-1 of the same workload with the reference's stopping rule, in the
R2-operator form and FP64 (in the reference's FP32 the stopping rule never
fires at 512x512, so FP64 is the CPU's fastest convergent arithmetic and runs
the same outer-iteration counts as the GPU's mixed mode); steps that would
start after --ref-budget-s are not run and `steps` says how many ran.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pd-ipc-armadillodemo_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "512x512 cloth PD-IPC steps/sec: mixed/batched vs plain GPU vs CPU at <=1e-4 m err"
UNIT = "steps/s"


def workload(name: str, scene_path: str | None = None):
    from pdipc import scenes
    if scene_path:
        import pdipc
        return pdipc.read_scene(scene_path)
    return {"c0": scenes.config0, "c1": scenes.config1, "c2": scenes.config2, "c4": scenes.config4}[name](seed=0)


def workload_desc(sc, prec: str) -> str:
    if len(sc.cloths) != 1 or sc.solids or not sc.statics:
        nt = sum(v.T.shape[0] for v in sc.solids)
        nf = sum(c.F.shape[0] for c in sc.cloths)
        return (f"{sc.name}: {len(sc.cloths)} cloths ({nf} f), {len(sc.solids)} tet models ({nt} tets), "
                f"{sc.n_sim} simulated v, {len(sc.statics)} fixed meshes ({sc.n_total - sc.n_sim} v); "
                f"dt {sc.dt:g} s, {sc.lg_iterations} PD iterations x 15 Chebyshev-Jacobi R2 sweeps, "
                f"dhat {sc.dhat:g} m, kappa {sc.kappa:g}; {prec}")
    c = sc.cloths[0]
    s = sc.statics[0]
    n = int(round(c.X.shape[0] ** 0.5))
    return (f"{n}x{n} cloth ({c.X.shape[0]} v / {c.F.shape[0]} f, 1 m, alternating diagonals, +/-1e-4 m jitter, "
            f"seed 0, 2 corners pinned) onto a fixed icosphere ({s.X.shape[0]} v / {s.F.shape[0]} f, r 0.3 m, "
            f"0.5 m below); dt 1/240 s, {sc.lg_iterations} PD iterations x 15 Chebyshev-Jacobi R2 sweeps, "
            f"dhat {sc.dhat:g} m, kappa {sc.kappa:g}; {prec}")


# ---------------------------------------------------------------------------- distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws: int, backend: str):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value: float, device=None) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_steps_per_s(world_size: int, steps: int, max_ms: float) -> float:
    """Whole-job throughput of independent replicas: every rank steps its own
    copy of the workload, the job ends with the slowest rank."""
    return world_size * steps / (max_ms * 1e-3)


def cloth_energy(sc, X, V) -> float:
    """Energy of the simulated cloths in a state (J): kinetic (lumped masses,
    density x one third of the adjacent triangles' rest area), gravitational
    potential along y, and the stretch energy 1/2 k_stretch (l - l0)^2 over the
    mesh edges (rest lengths from the cloth's initial positions)."""
    e, off = 0.0, 0
    for c in sc.cloths:
        n = c.X.shape[0]
        x, v = X[off:off + n], V[off:off + n]
        a = np.linalg.norm(np.cross(c.X[c.F[:, 1]] - c.X[c.F[:, 0]], c.X[c.F[:, 2]] - c.X[c.F[:, 0]]), axis=1) / 2
        m = np.zeros(n)
        for k in range(3):
            np.add.at(m, c.F[:, k], c.density * a / 3.0)
        ed = np.unique(np.sort(np.concatenate([c.F[:, [0, 1]], c.F[:, [1, 2]], c.F[:, [2, 0]]]), axis=1), axis=0)
        l0 = np.linalg.norm(c.X[ed[:, 0]] - c.X[ed[:, 1]], axis=1)
        ln = np.linalg.norm(x[ed[:, 0]] - x[ed[:, 1]], axis=1)
        e += 0.5 * float(np.sum(m[:, None] * v * v)) - sc.gravity * float(np.sum(m * x[:, 1]))
        e += 0.5 * c.k_stretch * float(np.sum((ln - l0) ** 2))
        off += n
    return e


def nvtx_push(name: str):
    """Open an NVTX push/pop range on this thread (`ncu --nvtx --nvtx-include
    "<name>/"` then profiles only launches inside it); returns its pop."""
    try:
        import torch.cuda.nvtx as nvtx
        nvtx.range_push(name)
        return nvtx.range_pop
    except Exception:
        return lambda: None


def barrier(dist, device=None):
    if dist is None:
        return
    if device is not None:
        dist.barrier(device_ids=[device.index])
    else:
        dist.barrier()


# ---------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region.

    nvidia-smi starts (and its NVML session comes up, which can hold up the
    process's CUDA calls for a while) before the timed region: __enter__
    returns once the first sample has arrived.  Only samples stamped between
    mark_start() and mark_end() count (the one right after the region too,
    when the region is shorter than the sampling period)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self.t_start = self.t_end = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.time() + 10.0
            while not self.lines and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def mark_start(self):
        self.t_start = datetime.datetime.now()

    def mark_end(self):
        self.t_end = datetime.datetime.now()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        # a region shorter than the sampling period: wait (briefly) for the
        # first sample stamped after its start
        deadline = time.time() + 0.6
        while self.proc and self.t_start is not None and time.time() < deadline and self.proc.poll() is None:
            if any(self._stamp(ln) is not None and self._stamp(ln) >= self.t_start for ln in list(self.lines)):
                break
            time.sleep(0.01)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    @staticmethod
    def _stamp(ln: str):
        try:
            return datetime.datetime.strptime(ln.split(",")[0].strip(), "%Y/%m/%d %H:%M:%S.%f")
        except ValueError:
            return None

    def _in_region(self) -> list[list[str]]:
        rows = []
        for ln in list(self.lines):
            parts = [p.strip() for p in ln.split(",")]
            ts = self._stamp(ln)
            if len(parts) < 10 or ts is None:
                continue
            rows.append((ts, parts[1:]))
        if self.t_start is None or self.t_end is None:
            return [p for _, p in rows]
        inside = [p for ts, p in rows if self.t_start <= ts <= self.t_end]
        if not inside:  # a region shorter than the period: the first sample after its start
            after = [p for ts, p in rows if ts >= self.t_start]
            inside = after[:1]
        return inside

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for parts in self._in_region():
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------- helpers
def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(prec: str):
    """DRAM bytes per launch of the persistent PD solve from the committed ncu
    summary, if present."""
    p = os.path.join(ROOT, "profiles", f"pd_persistent_c1_{prec}.md")
    try:
        for ln in open(p):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":", 1)[1])
    except OSError:
        pass
    return None


def oracle_whole_steps(scene, prec: str, threads: int, max_steps: int, budget_s: float, warmup: int = 0):
    """The oracle (the reference's algorithm restated on the CPU, its R2-operator
    form) stepping the workload from its initial state with the reference's
    stopping rule: whole steps, timed one by one, until `max_steps` steps or
    `budget_s` seconds.  Nothing is extrapolated: the figures cover the steps
    that ran."""
    from oracle.oracle import FORM_R2, Oracle
    t0 = time.perf_counter()
    orc = Oracle(scene, prec, FORM_R2, threads=threads)
    t_init = time.perf_counter() - t0
    x0, v0 = scene.initial_positions(), np.zeros((scene.n_sim, 3))
    for _ in range(warmup):
        orc.step(1)
    if warmup:
        orc.set_state(x0, v0)
    times, outers = [], []
    while len(times) < max_steps and sum(times) < budget_s:
        t0 = time.perf_counter()
        orc.step(1)
        times.append(time.perf_counter() - t0)
        outers.append(int(orc.stats()["last_outer_iters"]))
    orc.close()
    n, total = len(times), float(sum(times))
    return {"steps": n, "seconds": total, "init_s": t_init, "outers": outers,
            "steps_per_s": n / total, "s_per_outer_iteration": total / max(sum(outers), 1)}


def oracle_fp32_outer(scene, threads: int):
    """Seconds per outer iteration of the oracle in the reference's own FP32
    arithmetic (R2-operator form): one outer iteration of step 0.  At this size
    the reference's absolute stopping rule never fires in FP32, so its steps run
    the 30-iteration cap; this figure prices one iteration of that."""
    from oracle.oracle import FORM_R2, Oracle
    orc = Oracle(scene, "fp32", FORM_R2, threads=threads, fixed_outer=1)
    t0 = time.perf_counter()
    orc.step(1)
    dt = time.perf_counter() - t0
    orc.close()
    return dt


def cpu_reference_sample(scene, threads: int, max_steps: int = 3, budget_s: float = 20.0):
    """cpu_baseline of the GPU arm: the first whole steps of the same workload on
    the host cores (FP64 R2-operator form of the oracle, the reference's stopping
    rule), plus the price of one FP32 outer iteration."""
    r = oracle_whole_steps(scene, "fp64", threads, max_steps, budget_s)
    fp32_outer = oracle_fp32_outer(scene, threads)
    return {"value": r["steps_per_s"], "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"steps 0..{r['steps'] - 1} of the same workload run in full ({r['seconds']:.1f} s; outer "
                       f"iterations {r['outers']}, the reference's stopping rule), the reference's R2-operator "
                       f"algorithm restated on the CPU in FP64, {threads} threads, init {r['init_s']:.1f} s "
                       f"untimed. FP64 is the CPU's fastest convergent arithmetic here: in the reference's FP32 "
                       f"the absolute rule |dx|^2 < 1e-5 never fires at 512x512 and every step runs the "
                       f"30-iteration cap at {fp32_outer:.2f} s per outer iteration"),
            "s_per_outer_iteration": r["s_per_outer_iteration"],
            "outer_iterations_per_step": float(np.mean(r["outers"])),
            "fp32_s_per_outer_iteration": fp32_outer}


# ---------------------------------------------------------------------------- arms
def run_ours(args):
    import torch
    import pdipc

    ws, rank, local = dist_env()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = init_dist(ws, "nccl")
    sc = workload(args.config, args.scene)
    # config 2 (independent instances) shards: each rank steps its run of the
    # instance table, balanced by cumulative vertex count; a single cloth runs
    # a replica per rank
    partitioned = args.config == "c2" and ws > 1 and not args.scene
    if partitioned:
        from pdipc import scenes as _sc
        first = pdipc.partition_instances([c.X.shape[0] for c in sc.cloths], ws)
        sc = _sc.instance_slice(sc, int(first[rank]), int(first[rank + 1]))
    # the launch configuration is chosen by the library's autotuner at
    # initialize (untimed), unless --no-autotune
    sim = pdipc.Simulator(sc, args.precision, device=local, autotune=0 if args.no_autotune else 1,
                          instance_stop=instance_stop(args))
    tuning = sim.tuning()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    sim.step(args.warmup)                    # captures the graph, grows candidate buffers
    sim.reset()
    torch.cuda.synchronize()

    # Timed run through the public API with host buffers: the initial state is
    # uploaded from host memory (set_state), then every step is animate() =
    # run + postRun (positions to host).  `value` sums the device time of the
    # steps (CUDA events on the library's stream); `e2e` is the wall time of the
    # same calls, host<->device copies included.
    x_init = sc.initial_positions()
    v_init = np.zeros((sc.n_sim, 3))
    out = np.empty((sim.n_total, 3), np.float64)
    barrier(dist, dev)
    dev_ms, launches, outers = 0.0, 0, []
    pd_ms, pd_solves, ccd_ms, contact_ms = 0.0, 0, 0.0, 0.0
    flush.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.set_state(x_init, v_init)
    e2e_wall = time.perf_counter() - t0
    range_pop = nvtx_push("timed")           # lets a profiler select the timed launches
    with ClockSampler(local) as clk:
        clk.mark_start()
        for _ in range(args.steps):
            flush.zero_()                    # L2 flush between timed steps (256 MB write)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sim.animate(out)
            e2e_wall += time.perf_counter() - t0
            st = sim.stats()
            dev_ms += st["device_ms"]
            launches += st["kernel_launches"]
            outers.append(st["last_outer_iters"])
            pd_ms += st["pd_solve_ms"]
            pd_solves += st["pd_solves"]
            ccd_ms += st["ccd_ms"]
            contact_ms += st["contact_ms"]
        torch.cuda.synchronize()
        clk.mark_end()
    range_pop()
    barrier(dist, dev)
    dev_ms_max = max_over_ranks(dist, dev_ms, dev)
    e2e_max = max_over_ranks(dist, e2e_wall, dev)
    st_end = sim.stats()
    x_end = out.copy()
    v_end = sim.velocities().copy()

    # the contact phase of the same run: advance untimed to step
    # `contact_start`, then time `contact_steps` steps the same way
    contact = None
    if args.contact_steps > 0 and not args.scene:
        done = args.steps
        if done < args.contact_start:
            sim.step(args.contact_start - done)
            done = args.contact_start
        c_ms, c_outers, c_pd, c_ccd, c_ct = 0.0, [], 0.0, 0.0, 0.0
        for _ in range(args.contact_steps):
            flush.zero_()
            torch.cuda.synchronize()
            sim.step(1)
            st = sim.stats()
            c_ms += st["device_ms"]
            c_outers.append(st["last_outer_iters"])
            c_pd += st["pd_solve_ms"]
            c_ccd += st["ccd_ms"]
            c_ct += st["contact_ms"]
        k = args.contact_steps
        contact = {"steps_timed": f"{done}..{done + k - 1} (after {done} steps from the initial state)",
                   "value": round(k / (c_ms * 1e-3), 4), "unit": UNIT, "ms_per_step": round(c_ms / k, 3),
                   "outer_iterations_per_step": float(np.mean(c_outers)),
                   "ms_per_outer_iteration": round(c_ms / max(sum(c_outers), 1), 4),
                   "active_contacts_last": int(sim.stats()["active_contacts"]),
                   "step_breakdown_ms": {"pd_solve": round(c_pd / k, 3), "ccd": round(c_ccd / k, 3),
                                         "contact": round(c_ct / k, 3),
                                         "rest": round((c_ms - c_pd - c_ccd - c_ct) / k, 3)}}

    # plain FP64 GPU form over the same steps: its speed, the position error of
    # this run after them, and the one-step error of this mode started from the
    # FP64 run's own state every 10 steps
    fp64 = None
    if args.precision != "fp64" and args.fp64_steps > 0:
        k64 = min(args.fp64_steps, args.steps)
        ref = pdipc.Simulator(sc, "fp64", device=local, instance_stop=instance_stop(args))
        ref.step(args.warmup)
        ref.reset()
        ms64, outers64, one_step = 0.0, [], []
        for k in range(k64):
            probe = k % 10 == 0
            if probe:
                sim.set_state(ref.positions(), ref.velocities())
                sim.step(1)
                x_probe = sim.positions()
            flush.zero_()
            torch.cuda.synchronize()
            ref.step(1)
            ms64 += ref.stats()["device_ms"]
            outers64.append(ref.stats()["last_outer_iters"])
            if probe:
                one_step.append((k, float(np.abs(x_probe - ref.positions()).max())))
        err = float(np.abs(x_end - ref.positions()).max()) if k64 == args.steps else None
        energy = None
        if k64 == args.steps and not args.scene:
            e_mine = cloth_energy(sc, x_end[:sc.n_sim], v_end)
            e_ref = cloth_energy(sc, ref.positions()[:sc.n_sim], ref.velocities())
            energy = {"this_mode_J": e_mine, "fp64_J": e_ref, "abs_err_J": abs(e_mine - e_ref),
                      "rel_err": abs(e_mine - e_ref) / max(abs(e_ref), 1e-300),
                      "definition": "kinetic + gravitational potential + 1/2 k_stretch (l - l0)^2 over mesh edges "
                                    "of the simulated cloths after the timed steps"}
        fp64 = {"value": round(k64 / (ms64 * 1e-3), 4), "unit": UNIT, "steps": k64,
                "ms_per_step": round(ms64 / k64, 3),
                "outer_iterations_per_step": {"mean": float(np.mean(outers64)), "max": int(max(outers64))},
                "max_position_err_m_after_steps": err,
                "energy_after_steps": energy,
                "one_step_err_m_from_fp64_state": {"max": max(e for _, e in one_step),
                                                   "at_steps": [k for k, _ in one_step],
                                                   "values": [float("%.3g" % e) for _, e in one_step]},
                "note": "the trajectory error after many steps is bounded below by the FP64 path's own "
                        "sensitivity once contact starts (an FP64 run perturbed by 1e-9 m departs by mm "
                        "within 50 steps at this size: bench.py --accuracy-study); the one-step error "
                        "from the same state is the precision mode's own contribution"}
        ref.close()
        del ref

    # the reference's own arithmetic on the GPU over the same steps: FP32 in
    # every kernel, the reference's stopping rule (which never fires at this
    # size in FP32, so its steps run the outer-iteration cap)
    fp32 = None
    if args.precision != "fp32" and args.fp32_steps > 0:
        k32 = min(args.fp32_steps, args.steps)
        g32 = pdipc.Simulator(sc, "fp32", device=local, instance_stop=instance_stop(args))
        g32.step(args.warmup)
        g32.reset()
        ms32, outers32 = 0.0, []
        for _ in range(k32):
            flush.zero_()
            torch.cuda.synchronize()
            g32.step(1)
            ms32 += g32.stats()["device_ms"]
            outers32.append(g32.stats()["last_outer_iters"])
        # the local step of the per-sweep path in the reference's arithmetic (FP32
        # state: the algorithmic bytes' sizes), timed alone like local_alone
        lms32, lb32 = g32.local_timing(400)
        pk, _ = measured_peak_hbm()
        fp32 = {"value": round(k32 / (ms32 * 1e-3), 4), "unit": UNIT, "steps": k32,
                "ms_per_step": round(ms32 / k32, 3),
                "outer_iterations_per_step": {"mean": float(np.mean(outers32)), "max": int(max(outers32))},
                "ms_per_outer_iteration": round(ms32 / max(sum(outers32), 1), 4),
                "local_alone": {"kernel": "k_local_aq + k_local_rhs_sweep (FP32 state), 400 back to back",
                                "bytes_per_launch": lb32, "ms_per_launch": round(lms32, 6),
                                "achieved": round(lb32 / (lms32 * 1e-3) / 1e9, 1),
                                "frac": round(lb32 / (lms32 * 1e-3) / 1e9 / pk, 4)}}
        g32.close()
        del g32

    # roofline of the dominant kernel: the PD solve of an outer iteration (one
    # persistent launch), timed by the library's events around each solve over
    # the timed steps; and one J sweep launched alone, for comparison
    pd_bytes = float(st_end["pd_solve_bytes"])
    pd_ms_per = pd_ms / max(pd_solves, 1)
    peak, peak_kind = measured_peak_hbm()
    achieved = pd_bytes / (pd_ms_per * 1e-3) / 1e9
    sim.set_state(x_end)
    sweep_ms, sweep_bytes = sim.sweep_timing(400)
    sweep_gbs = sweep_bytes / (sweep_ms * 1e-3) / 1e9
    local_ms, local_bytes = sim.local_timing(400)
    local_gbs = local_bytes / (local_ms * 1e-3) / 1e9
    pd_kernel = {3: "k_pd_persistent (cooperative, matrix values and the iterate's band in shared memory, "
                    "halo by bulk copies)",
                 2: "k_pd_persistent (cooperative, matrix values in shared memory)",
                 1: "k_pd_persistent (cooperative, matrix from L2)",
                 0: "PD solve as a CUDA graph of per-sweep kernels"}[st_end["pd_path"]]
    state_bytes = 16 if args.precision == "fp32" else 32

    # replicas: every rank's steps count; a partitioned batch: the ranks
    # together advance the one batch, which is done when the slowest rank is
    value = aggregate_steps_per_s(1 if partitioned else ws, args.steps, dev_ms_max)
    e2e = aggregate_steps_per_s(1 if partitioned else ws, args.steps, e2e_max * 1e3)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    mean_outer = float(np.mean(outers))
    traffic = profiled_traffic(args.precision) if args.config == "c1" and not args.scene else None
    res = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "strong" if partitioned else "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "fp64": "f64",
                  "mixed": "f32 (local step, residual terms, sweeps) + f64 (state, CCD/contact refinement)"}[
            args.precision], "data": "synthetic (seeded generator; no public dataset for this path)",
        "config": run_config(sc, args, ws),
        "run": {"outer_iterations_per_step": {"mean": mean_outer, "min": int(min(outers)), "max": int(max(outers))},
                "ms_per_outer_iteration": round(dev_ms_max / max(sum(outers), 1), 4),
                "vertices_sim": sim.n_sim, "vertices_total": sim.n_total,
                "patch_pairs": st_end["patch_pairs"], "pt_candidates": st_end["pt_candidates"],
                "ee_candidates": st_end["ee_candidates"], "device_bytes": st_end["device_bytes"],
                "l2_flush": "256 MB written between timed steps"},
        "element_updates_per_s": round(sim.n_sim * sc.lg_iterations * float(np.sum(outers)) / (dev_ms / 1e3), 1),
        "gpu_launches": int(launches),
        "step_breakdown_ms": {"pd_solve": round(pd_ms / args.steps, 3), "ccd": round(ccd_ms / args.steps, 3),
                              "contact": round(contact_ms / args.steps, 3),
                              "rest": round((dev_ms - pd_ms - ccd_ms - contact_ms) / args.steps, 3),
                              "note": "per timed step, CUDA events on the library's stream"},
        "e2e": {"value": round(e2e, 4), "unit": UNIT,
                "h2d_bytes_per_step": int(round((sim.n_total + sc.n_sim) * state_bytes / args.steps)),
                "d2h_bytes_per_step": int(sim.n_total * state_bytes + 8 * round(mean_outer) + 48),
                "note": "wall time of the timed run itself: set_state of the initial positions/velocities "
                        "from host memory once, then animate() per step (step + copy of every position to "
                        "host); the state stays on the device between steps, as in the reference"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": None if traffic is None else round(traffic),
                     "kernel": pd_kernel, "launches_timed": int(pd_solves),
                     "bytes_per_launch": round(pd_bytes), "ms_per_launch": round(pd_ms_per, 4),
                     "bytes_rule": "per vertex and local-global iteration: local step 16 d + 68, 2 x cheby sweeps "
                                   "of 8 n + 28, (cheby - 1) x 12 Chebyshev reads (FP32 sizes)",
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                     "sweep_alone": {"kernel": "one weighted-Jacobi sweep launch (SELL-32) timed alone",
                                     "bytes_per_launch": int(sweep_bytes), "ms_per_launch": round(sweep_ms, 6),
                                     "achieved": round(sweep_gbs, 1), "frac": round(sweep_gbs / peak, 4)},
                     "local_alone": {"kernel": "the local step alone: curvature kernel + right-hand-side kernel "
                                               "with the first sweep fused (k_local_aq_rel + k_local_residual in "
                                               "the mixed mode), 400 back to back",
                                     "bytes_per_launch": int(local_bytes), "ms_per_launch": round(local_ms, 6),
                                     "achieved": round(local_gbs, 1), "frac": round(local_gbs / peak, 4),
                                     "bytes_rule": "per vertex: 16 d + 68 (local step) + 8 n + 28 (fused sweep)"}},
        "clocks": clk.summary(),
    }
    res["tuning"] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in tuning.items()}
    if fp64 is not None:
        res["fp64_gpu"] = fp64
    if fp32 is not None:
        res["fp32_gpu"] = fp32
    if contact is not None:
        res["contact_phase"] = contact
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_reference_sample(sc, os.cpu_count() or 1, args.cpu_steps, args.cpu_budget_s)
        cb = res["cpu_baseline"]
        res["per_outer_iteration"] = {
            "gpu_ms": res["run"]["ms_per_outer_iteration"],
            "cpu_fp64_r2_ms": round(cb["s_per_outer_iteration"] * 1e3, 2),
            "gpu_fp32_ms": fp32["ms_per_outer_iteration"] if fp32 else None,
            "cpu_fp32_r2_ms": round(cb["fp32_s_per_outer_iteration"] * 1e3, 2),
            "note": "the same outer iteration (20 local-global iterations of 15 Chebyshev R2 steps, CCD, "
                    "contact) priced on each side; the GPU mixed mode and the CPU FP64 run stop after the same "
                    "outer-iteration counts (equal to the FP64 oracle's step for step)"}
    print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def instance_stop(args) -> int:
    """1 when the run uses per-instance stopping (each independent instance of
    a batch takes the reference's stopping rule on its own vertices)."""
    if args.instance_stop == "auto":
        return int(args.config == "c2" and not args.scene)
    return int(args.instance_stop == "on")


def run_config(sc, args, ws: int) -> dict:
    """The `config` object, identical in both arms for the same arguments."""
    return {"workload": workload_desc(sc, args.precision), "steps_timed": f"0..{args.steps - 1}",
            "stopping_rule": ("per instance (each model's own |dx|^2 < 1e-5)" if instance_stop(args)
                              else "the reference's: one test over the scene's vertices (|dx|^2 < 1e-5)"),
            "parallelism": ((f"instance table partitioned over {ws} ranks by cumulative vertex count"
                             if args.config == "c2" and not args.scene else "replicas only")
                            if ws > 1 else "single GPU"),
            "l2": "working set above L2 (about 1 GB at 512x512, more than any cache on either side); the GPU "
                  "arm also writes 256 MB between timed steps"}


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm, R2-operator
    form, restated on the CPU) on every host thread, stepping the same workload
    from the same initial state with the reference's stopping rule.  Whole
    steps, timed one by one; steps past the time budget are not run, and
    `steps` reports how many were."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    sc = workload(args.config, args.scene)
    threads = os.cpu_count() or 1
    r = oracle_whole_steps(sc, "fp64", threads, args.steps, args.ref_budget_s, warmup=min(args.warmup, 1))
    n = r["steps"]
    value = r["steps_per_s"]
    sample = (f"steps 0..{n - 1} of {args.steps} run in full ({r['seconds']:.1f} s; outer iterations per step "
              f"{r['outers']}, the reference's stopping rule |dx|^2 < 1e-5, cap 30), the reference's R2-operator "
              f"algorithm restated on the CPU in FP64 (at 512x512 the rule never fires in FP32, so FP64 is the "
              f"CPU's fastest convergent arithmetic), {threads} threads; init {r['init_s']:.1f} s and "
              f"{min(args.warmup, 1)} warm-up step untimed")
    res = {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": ws,
           "steps": n, "warmup": args.warmup, "ms_per_step": round(1e3 / value, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded generator; no public dataset for this path)",
           "config": run_config(sc, args, ws),
           "run": {"outer_iterations_per_step": {"mean": float(np.mean(r["outers"])), "min": int(min(r["outers"])),
                                                 "max": int(max(r["outers"]))},
                   "s_per_outer_iteration": round(r["s_per_outer_iteration"], 4),
                   "steps_requested": args.steps},
           "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(res), flush=True)


def run_accuracy_study(args):
    """Position error of the chosen precision mode against the FP64 form along
    the same run, next to the FP64 form's own sensitivity: a second FP64 run
    whose simulated vertices start perturbed by a seeded uniform 1e-9 m."""
    import pdipc
    ws, rank, local = dist_env()
    if rank != 0:
        return
    sc = workload(args.config, args.scene)
    a = pdipc.Simulator(sc, "fp64", device=local)
    b = pdipc.Simulator(sc, "fp64", device=local)
    c = pdipc.Simulator(sc, args.precision, device=local)
    x = b.positions()
    x[:sc.n_sim] += np.random.default_rng(1).uniform(-1e-9, 1e-9, (sc.n_sim, 3))
    b.set_state(x)
    rows = []
    for k in range(args.steps):
        oa = []
        for sim in (a, b, c):
            sim.step(1)
            oa.append(sim.stats()["last_outer_iters"])
        if (k + 1) % 10 == 0 or k + 1 == args.steps:
            xa = a.positions()[:sc.n_sim]
            rows.append({"step": k + 1, "active_contacts": a.stats()["active_contacts"],
                         "fp64_vs_fp64_perturbed_1e-9_m": float(np.abs(xa - b.positions()[:sc.n_sim]).max()),
                         f"{args.precision}_vs_fp64_m": float(np.abs(xa - c.positions()[:sc.n_sim]).max()),
                         "outer_iterations_fp64_fp64p_mode": oa})
    print(json.dumps({"study": "accuracy", "workload": workload_desc(sc, args.precision), "rows": rows}),
          flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp32", "fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=100)
    ap.add_argument("--config", default="c1", choices=["c1", "c0", "c2", "c4"],
                    help="c1 is the benchmark workload; the others are for reference measurements")
    ap.add_argument("--scene", default=None,
                    help="a reference-format config.xml to run instead of --config (reference measurement)")
    ap.add_argument("--fp32-steps", type=int, default=100,
                    help="steps of the FP32 GPU form (the reference's arithmetic) timed beside the headline")
    ap.add_argument("--contact-start", type=int, default=50,
                    help="first step of the contact-phase window timed after the headline run")
    ap.add_argument("--contact-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="run the built-in launch configuration")
    ap.add_argument("--instance-stop", choices=["auto", "on", "off"], default="auto",
                    help="per-instance stopping rule (pdipc_params.instance_stop); auto: on for the batch of "
                         "independent drops (config c2), off otherwise")
    ap.add_argument("--cpu-steps", type=int, default=3, help="whole steps in the GPU arm's cpu_baseline sample")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--ref-budget-s", type=float, default=300.0,
                    help="the reference arm stops starting new steps after this many seconds of stepping")
    ap.add_argument("--accuracy-study", action="store_true",
                    help="print the error-vs-FP64 table of the precision mode instead of the bench line")
    args = ap.parse_args(argv)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.accuracy_study:
        run_accuracy_study(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
