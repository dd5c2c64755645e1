"""Throughput benchmark of the per-RK-stage RHS + time update (DOF-stage updates/s).

Workload: double Mach reflection, [0,4]x[0,1]x[0,0.0167], 240x60x1 cells, N=3 (921,600 DoFs),
synthetic inputs generated in code (IC, BCs and seeded noise of the configuration). One step =
one RK4(3)5[3R+]N time step (5 RHS evaluations + register updates + the CFL min-reduction).
DOF-stage updates/s = DoFs * 5 * steps / time.

Forms measured: the plain FP64 form; the mixed form (flux differencing, surface fluxes and the
indicator in FP32; the state, the metric terms, the 1/det J scaling, the three RK registers and
their accumulation in FP64) with the modal troubled-cell sensor and with the learned one (trained
weights in plens_gb300/sensor_weights.bin); and, for comparison, the mixed_r32 form (FP32 RK
registers and FP32 metric images) with the learned sensor. `value` is the mixed form with the
learned sensor (the modal one when no weights are shipped).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: one process per GPU (torchrun), each rank advances its own replica of the workload
(the path does not need a collective on one GPU: "replicas only"); the max of the per-rank
times over the ranks is the job time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DOF-stage updates/s: FP32+learned sensor vs FP64 plain, GB300, rho L1 err<=1e-4"
UNIT = "DOF-stage/s"
# Algorithmic bytes of one DOF-stage through the volume kernel, averaged over the five RK4 stages.
# FP64 and MIXED forms: U read and written 80, two RK registers read 80 (stages 3-5; one at stage
# 2, none at stage 1; the reference's update, which copies its registers down every stage
# (dgsem/plens.cc:4353-4400), moves more, and the count keeps two reads throughout), one
# written 40 at stages 1-4 (the last stage's dt*R is read by no later stage and is not written),
# Ja and detJ (the MIXED form: Ja and 1/detJ) 80: 280 - 40/5 = 272. MIXED_R32 form: the registers hold dt*R in FP32 (2 x 20
# read, 20 written at stages 1-4) and the kernel reads the FP32 images of Ja and detJ (40):
# 80 + 40 + 16 + 40 = 176.
BYTES_PER_DOF_STAGE = {"plain": 272, "modal": 272, "learned": 272, "learned_r32": 176}
# What the MIXED form's volume kernel actually reads and writes per DOF-stage at N = 3, averaged
# over the five stages (it reads no register where the stage's coefficient is zero, and it moves
# the FP32 state image and the face values, which the algorithmic count leaves out): 80 (state)
# + 56 + 32 (registers) + 36 + 8 (Ja image, 1/detJ) + 40 (state image) + 30 (face values).
MOVED_BYTES_MIXED = 282
WORKLOAD = "double Mach reflection 240x60x1 cells, N=3, 921600 DoFs, RK4(3)5[3R+]N, HLLC + Chandrashekhar"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profile(name: str):
    """DRAM bytes per launch of the volume kernel from the committed ncu summary, if present."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class _Nvml:
    """Read-only NVML queries through ctypes (the library the driver installs): SM clock, its
    maximum and the active clock-event (throttle) reasons of one GPU."""

    SW_POWER_CAP, HW_SLOWDOWN, SW_THERMAL, HW_THERMAL = 0x4, 0x8, 0x20, 0x40

    def __init__(self, index: int):
        import ctypes
        self.C = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sm_clock(self) -> int:
        v = self.C.c_uint()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, self.C.byref(v))  # NVML_CLOCK_SM
        return v.value

    def sm_max(self) -> int:
        v = self.C.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, self.C.byref(v))
        return v.value

    def reasons(self) -> int:
        v = self.C.c_ulonglong()
        self.reasons_fn(self.h, self.C.byref(v))
        return v.value


class ClockSampler:
    """Clock / throttle sampling during the timed region: NVML polled every 2 ms from a thread
    (the timed regions are tens of milliseconds), else nvidia-smi at its 200 ms period."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.thread = None
        self.samples = []
        self.nvml = None
        try:
            self.nvml = _Nvml(gpu_index)
            self.max_mhz = self.nvml.sm_max()
        except Exception:
            self.nvml = None
        self.path = None if self.nvml else Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def _poll(self):
        while not self.stop.is_set():
            try:
                self.samples.append((self.nvml.sm_clock(), self.nvml.reasons()))
            except Exception:
                pass
            self.stop.wait(0.002)

    def __enter__(self):
        if self.nvml is not None:
            import threading
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.thread is not None:
            self.stop.set()
            self.thread.join(timeout=5)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            if not self.samples:
                return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "source": "nvml"}
            names = ((_Nvml.HW_SLOWDOWN, "hw_slowdown"), (_Nvml.HW_THERMAL, "hw_thermal_slowdown"),
                     (_Nvml.SW_THERMAL, "sw_thermal_slowdown"), (_Nvml.SW_POWER_CAP, "sw_power_cap"))
            reasons = sorted({n for _, r in self.samples for bit, n in names if r & bit})
            return {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                    "reasons": reasons, "samples": len(self.samples), "source": "nvml, 2 ms"}
        try:
            rows = [r.split(",") for r in self.path.read_text().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def _rel_l1(X, ref):
    d = np.abs(X - ref)
    a = np.abs(ref)
    return [float(d[0].sum() / a[0].sum()), float(d[1:4].sum() / max(a[1:4].sum(), 1e-300)),
            float(d[4].sum() / a[4].sum())]


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device) -> float:
    """Job time = max over ranks (all_reduce MAX); identity on one process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def _sensor_weights():
    p = ROOT / "plens_gb300" / "sensor_weights.bin"
    if p.exists():
        w = np.fromfile(p, dtype=np.float32)
        from plens_gb300.api import MLP_N_PARAMS
        if w.size == MLP_N_PARAMS:
            return w
    return None


# the mesh-size arguments of each workload's builder, in the order --mesh gives them
MESH_ARGS = {"dmr": ("nx", "ny"), "sod": ("n",), "cylinder": ("n_radial", "n_azimuthal"), "shock_vortex": ("n",)}


def _spec(workload: str, precision: str, sensor: str, mesh: tuple = ()):
    """The workload's specification; `mesh` replaces its cell counts (a smaller case of the same
    workload, for profiles that must fit a few GB)."""
    from plens_gb300 import configs
    size = dict(zip(MESH_ARGS[workload], mesh))
    if workload == "dmr":
        return configs.dmr(precision=precision, sensor=sensor, end_time=1e9, **size)
    if workload == "sod":
        return configs.sod(precision=precision, sensor=sensor, end_time=1e9, **size)
    if workload == "cylinder":
        return configs.cylinder(precision=precision, sensor=sensor, **size)
    if workload == "shock_vortex":
        return configs.shock_vortex(precision=precision, sensor=sensor, **size)
    raise ValueError(workload)


def _form_case(workload: str, precision: str, sensor: str, cache: dict | None = None, mesh: tuple = ()):
    """The workload's Case with the form's precision and sensor. With a cache, the mesh, metric
    terms and initial state are built once per workload and only the two parameters change."""
    from plens_gb300 import configs
    if cache is None:
        return configs.make_case(_spec(workload, precision, sensor, mesh))
    if workload not in cache:
        cache[workload] = configs.make_case(_spec(workload, "fp64", "modal"))
    case = cache[workload]
    from plens_gb300.api import PRECISIONS
    case.params.precision = PRECISIONS[precision]
    case.params.sensor = 1 if sensor == "learned" else 0
    return case


def measure_form(precision: str, sensor: str, steps: int, warmup: int, device_index: int, weights=None,
                 workload: str = "dmr", cache: dict | None = None, tensor_cores: bool | None = None, e2e: bool = True,
                 indicator_tc: bool | None = None, mesh: tuple = ()):
    import torch

    from plens_gb300.api import GpuSolver, PlensError

    case = _form_case(workload, precision, sensor, cache, mesh)
    U0 = case.initial_state()
    g = GpuSolver(case)
    if sensor == "learned":
        g.set_sensor_weights(weights)
        if tensor_cores is not None:
            g.set_sensor_tensor_cores(tensor_cores)
    elif indicator_tc is not None:
        g.set_indicator_tensor_cores(indicator_tc)
    g.set_state(U0, 0.0)
    g.advance(warmup)
    stream = torch.cuda.ExternalStream(g.stream, device=torch.device("cuda", device_index))
    launches0 = g.kernel_launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    # timed region: the steps as the library runs them (each step a replayed CUDA graph)
    with ClockSampler(device_index) as cs:
        ev0.record(stream)
        g.advance_async(steps)
        ev1.record(stream)
        g.synchronize()
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = g.kernel_launches - launches0
    # the same number of steps again with the library's CUDA events around every volume-kernel
    # launch (eager launches), for the kernel's own duration
    g.set_kernel_timing(True)
    g.advance_async(steps)
    g.synchronize()
    vol_ms, vol_n = g.kernel_timing()
    g.set_kernel_timing(False)
    stats = g.sensor_stats() if sensor == "learned" else None
    try:  # the compacted troubled-cell list of the last RHS (mixed forms)
        lo_cells = int(len(g.troubled_cells()))
    except PlensError:
        lo_cells = None
    Ug = g.get_state()

    if not e2e:
        g.close()
        return {"case": case, "ms": ms, "launches": launches, "vol_ms": vol_ms, "vol_n": vol_n,
                "clocks": cs.summary(), "stats": stats, "U": Ug, "lo_cells": lo_cells}
    # end to end through the C ABI with pinned host buffers: per step a state goes host -> device,
    # one step runs, the new state comes back. (1) plens_gpu_advance_states: a sequence of states,
    # the transfers on copy streams beside the steps; (2) the serial loop set_state -> advance(1)
    # -> get_state, each call synchronous.
    pin_in = torch.empty((5, case.n_dofs), dtype=torch.float64).pin_memory()
    pin_in.numpy()[:] = Ug
    pin_out = torch.empty((5, case.n_dofs), dtype=torch.float64).pin_memory()
    t_state = g.get_time()[0]
    e2e_steps = max(3, steps)
    g.advance_states([pin_in.numpy()], [pin_out.numpy()], t_state, 1)  # copy streams and buffers made
    barrier()
    t0 = time.perf_counter()
    g.advance_states([pin_in.numpy()] * e2e_steps, [pin_out.numpy()] * e2e_steps, t_state, 1)
    t_e2e = time.perf_counter() - t0
    serial_steps = max(3, min(steps, 20))
    barrier()
    t0 = time.perf_counter()
    for _ in range(serial_steps):
        g.set_state(pin_in.numpy())
        g.advance(1)
        g.get_state(pin_out.numpy())
    t_serial = time.perf_counter() - t0
    g.close()
    return {
        "case": case, "ms": ms, "launches": launches, "vol_ms": vol_ms, "vol_n": vol_n,
        "clocks": cs.summary(), "stats": stats, "U": Ug, "e2e_s": t_e2e, "e2e_steps": e2e_steps,
        "serial_s": t_serial, "serial_steps": serial_steps, "bytes_state": 5 * case.n_dofs * 8,
    }


def cpu_baseline(max_seconds: float = 20.0, steps_cap: int | None = None):
    """The oracle (FP64 C++/OpenMP restatement of the reference's CPU path) on the host cores,
    on whole RK steps of the same workload, bounded to about max_seconds."""
    from oracle.pyoracle import Oracle, max_threads
    from plens_gb300 import configs

    case = configs.make_case(configs.dmr(end_time=1e9))
    o = Oracle(case)
    o.set_state(case.initial_state(), 0.0)
    t0 = time.perf_counter()
    o.advance(1)
    t1 = time.perf_counter() - t0
    n = max(1, int(max_seconds / max(t1, 1e-3)))
    if steps_cap:
        n = min(n, steps_cap)
    t0 = time.perf_counter()
    o.advance(n)
    dt = time.perf_counter() - t0
    dofstage = case.n_dofs * 5 * n
    return {"value": dofstage / dt, "unit": UNIT, "cores": max_threads(), "kind": "port",
            "sample": f"{n} RK4 step(s) of the full 921600-DoF workload after 1 warm-up step, {dt:.2f} s"}


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return
    cb = cpu_baseline(max_seconds=float(os.environ.get("PLENS_REF_SECONDS", "30")))
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference CPU/MPI path unavailable here (deal.II/PETSc/p4est/MPI absent); "
                "timed: the FP64 C++/OpenMP restatement of its per-stage RHS and update",
    }
    print(json.dumps(line), flush=True)


# per configuration: the accuracy window of the FP32 forms against the FP64 form (the config's own
# run length where it fits in minutes, else a stated window), and the full-size window in which the
# FP64 form is compared with the oracle
WORKLOADS = {
    "sod": {"acc_steps": 100, "acc_end": None, "oracle_steps": 100, "note": "config run length: 100 steps"},
    # the config runs to t = 0.2, but every form (FP64 included, as the FP64 oracle) stops there
    # on the positivity assertion first: the window is fixed, and `horizon` reports where the FP32
    # form stops
    "dmr": {"acc_steps": 1000, "acc_end": None, "oracle_steps": 100, "windows": [100, 300, 1000],
            "note": "first 100, 300 and 1000 steps (the config's t = 0.2 is not reached, see horizon)",
            "horizon": 0.2},
    "cylinder": {"acc_steps": 1000, "acc_end": None, "oracle_steps": 10,
                 "note": "first 1000 of the config's 20000 steps", "full_run_steps": 20000},
    "shock_vortex": {"acc_steps": 20, "acc_end": None, "oracle_steps": 1,
                     "note": "first 20 of the config's 500 steps"},
}


def run_workload_report(args):
    """One JSON line per configuration: DOF-stage/s of the FP64 plain form, the FP32 form with
    the modal and with the learned sensor, and the oracle on the host cores; the relative L1
    errors of the FP32 forms against the FP64 form over the configuration's accuracy window, and
    of the FP64 form against the oracle over a full-size window."""
    import torch

    from oracle.pyoracle import Oracle, max_threads
    from plens_gb300 import configs
    from plens_gb300.api import GpuSolver, PlensError

    torch.cuda.set_device(0)
    wl = WORKLOADS[args.workload]
    acc_steps = args.accuracy_steps or wl["acc_steps"]
    end = wl["acc_end"] if wl["acc_end"] is not None else 1e300
    weights = _sensor_weights()
    forms = [("fp64_plain", "fp64", "modal"), ("fp32_modal", "mixed", "modal")]
    if weights is not None:
        forms += [("fp32_learned", "mixed", "learned"), ("fp32_r32_learned", "mixed_r32", "learned")]
    out = {"workload": args.workload, "accuracy_window": wl["note"] if not args.accuracy_steps else f"{acc_steps} steps"}
    states = {}
    windows = [acc_steps] if args.accuracy_steps else wl.get("windows", [acc_steps])
    cache = {}
    for name, prec, sensor in forms:
        r = measure_form(prec, sensor, args.steps, args.warmup, 0, weights, workload=args.workload, cache=cache)
        nd = r["case"].n_dofs
        out[name] = {"dof_stage_per_s": nd * 5 * args.steps / (r["ms"] / 1e3), "ms_per_step": r["ms"] / args.steps,
                     "volume_kernel_ms": r["vol_ms"] / max(r["vol_n"], 1), "n_dofs": nd, "clocks": r["clocks"]}
    # accuracy: every form from the initial condition, states kept at each window; the FP64 form
    # once more from an initial density perturbed by 1e-12 (relative) measures how fast the flow
    # itself amplifies a perturbation over the same windows
    runs = [(n, p_, s_, False) for n, p_, s_ in forms] + [("fp64_perturbed_1e-12", "fp64", "modal", True)]
    for name, prec, sensor, perturb in runs:
        case = _form_case(args.workload, prec, sensor, cache)
        g = GpuSolver(case)
        if sensor == "learned":
            g.set_sensor_weights(weights)
        U0 = case.initial_state()
        if perturb:
            rng = np.random.default_rng(7)
            U0[0] *= 1 + 1e-12 * rng.uniform(-1, 1, U0.shape[1])
        g.set_state(U0, case.start_time)
        t0 = time.perf_counter()
        rec = out.setdefault(name, {})
        try:
            done = 0
            for w in windows:
                g.advance(w - done, end)
                done = w
                states[(name, w)] = g.get_state()
            t, n, _ = g.get_time()
            rec["accuracy_run"] = {"steps": n, "seconds": time.perf_counter() - t0, "t_end": t}
        except PlensError as e:
            rec["accuracy_run"] = {"error": str(e)}
        if sensor == "learned":
            st = g.sensor_stats()
            st["fallback_rate"] = st["fallbacks"] / max(st["judged"] * case.n_cells, 1)
            rec["accuracy_run"]["sensor_stats"] = st
        g.close()
    for name in ("fp32_modal", "fp32_learned", "fp32_r32_learned", "fp64_perturbed_1e-12"):
        for w in windows:
            if (name, w) in states and ("fp64_plain", w) in states:
                out[name].setdefault("rel_l1_vs_fp64", {})[f"{w}_steps"] = dict(
                    zip(("rho", "momentum", "rhoE"), _rel_l1(states[(name, w)], states[("fp64_plain", w)])))
    if wl.get("horizon"):
        # how far the FP32 modal form gets towards the configuration's end time
        case = _form_case(args.workload, "mixed", "modal", cache)
        g = GpuSolver(case)
        g.set_state(case.initial_state(), case.start_time)
        t0 = time.perf_counter()
        h = {"end_time": wl["horizon"]}
        try:
            for _ in range(200):
                g.advance(500, wl["horizon"])
                t, n, dt = g.get_time()
                if t >= wl["horizon"] or time.perf_counter() - t0 > 120:
                    break
            h["reached"] = True
        except PlensError as e:
            h["reached"] = False
            h["error"] = str(e)
        t, n, dt = g.get_time()
        h.update({"t": t, "steps": n, "last_dt": dt, "seconds": time.perf_counter() - t0})
        out["horizon_fp32_modal"] = h
        g.close()
    if wl.get("full_run_steps"):
        # the configuration's whole run in the headline form (mixed, learned sensor where weights
        # are shipped): completion, time, the judge's outcome
        sensor = "learned" if weights is not None else "modal"
        case = _form_case(args.workload, "mixed", sensor, cache)
        g = GpuSolver(case)
        if sensor == "learned":
            g.set_sensor_weights(weights)
        g.set_state(case.initial_state(), case.start_time)
        t0 = time.perf_counter()
        run = {"form": f"mixed + {sensor}", "steps_asked": wl["full_run_steps"]}
        try:
            g.advance(wl["full_run_steps"])
            run["completed"] = True
        except PlensError as e:
            run["completed"] = False
            run["error"] = str(e)
        t, n, dt = g.get_time()
        run.update({"steps": n, "t": t, "last_dt": dt, "seconds": time.perf_counter() - t0,
                    "dof_stage_per_s": case.n_dofs * 5 * n / max(time.perf_counter() - t0, 1e-9)})
        if sensor == "learned":
            run["sensor_stats"] = g.sensor_stats()
        out["full_run"] = run
        g.close()
    # the FP64 form against the oracle at full size
    case = _form_case(args.workload, "fp64", "modal", cache)
    o = Oracle(case)
    o.set_state(case.initial_state(), case.start_time)
    t0 = time.perf_counter()
    o.advance(wl["oracle_steps"])
    dt = time.perf_counter() - t0
    g = GpuSolver(case)
    g.set_state(case.initial_state(), case.start_time)
    g.advance(wl["oracle_steps"])
    out["fp64_vs_oracle"] = {"steps": wl["oracle_steps"],
                             "rel_l1": dict(zip(("rho", "momentum", "rhoE"), _rel_l1(g.get_state(), o.get_state()[0])))}
    g.close()
    out["cpu_oracle"] = {"dof_stage_per_s": case.n_dofs * 5 * wl["oracle_steps"] / dt, "cores": max_threads(),
                         "steps": wl["oracle_steps"], "seconds": dt}
    print(json.dumps(out), flush=True)


# z boundaries and z resolution of the double Mach reflection: the variants of the horizon study
HORIZON_VARIANTS = {
    "periodic": dict(z_bc="periodic"),                  # the configuration: one periodic cell across z
    "periodic_no_noise": dict(z_bc="periodic", noise=0.0),  # the same without the seeded density noise
    "symmetry": dict(z_bc="symmetry"),                  # the reference's own z boundaries
    "periodic_2_cells": dict(z_bc="periodic", nz=2),    # two periodic cells across z
    "plens_2d": dict(z_bc="periodic", plens_2d=True),   # the reference's PLENS_2D switch
}


def run_horizon(args):
    """How far the double Mach reflection gets towards t = 0.2 with each z treatment, and how the
    flow's z-dependence grows on the way: every 100 steps the max |rho w| over max |rho u|, and the
    largest spread of rho and of rho E across the P z-layers of a cell (relative to their maxima).
    One JSON line per variant; on a positivity failure, the first failing dof with its cell, node,
    z-layer and location."""
    import torch

    from plens_gb300 import configs
    from plens_gb300.api import GpuSolver, PositivityError

    torch.cuda.set_device(0)
    prec = args.horizon_precision
    for name in args.horizon.split(","):
        case = configs.make_case(configs.dmr(precision=prec, **HORIZON_VARIANTS[name]))
        P = case.degree + 1
        P2, P3 = P * P, P ** 3

        def zstats(U):
            Ur = U.reshape(5, case.n_cells, P, P2)
            spread = lambda a: float((a.max(axis=1) - a.min(axis=1)).max() / np.abs(a).max())  # noqa: E731
            return {"w_rel": float(np.abs(U[3]).max() / np.abs(U[1:4]).max()), "rho_z_spread": spread(Ur[0]),
                    "rhoE_z_spread": spread(Ur[4])}

        g = GpuSolver(case)
        g.set_state(case.initial_state(), 0.0)
        t0 = time.perf_counter()
        hist, out = [], {"variant": name, "precision": prec, "end_time": 0.2}
        while True:
            try:
                g.advance(100, 0.2)
            except PositivityError as e:
                t, n, _ = g.get_time()
                xyz = case.dof_xyz()[:, e.dof]
                out["failed"] = {"t": t, "steps": n, "dof": e.dof, "cell": e.dof // P3, "node": e.dof % P3,
                                 "z_layer": (e.dof % P3) // P2, "xyz": [float(v) for v in xyz]}
                break
            t, n, _ = g.get_time()
            hist.append(dict(t=t, steps=n, **zstats(g.get_state())))
            if t >= 0.2 or time.perf_counter() - t0 > 300:
                out["reached"] = t >= 0.2
                break
        out["seconds"] = time.perf_counter() - t0
        out["history"] = hist
        g.close()
        print(json.dumps(out), flush=True)


FORMS = {"plain": ("fp64", "modal"), "modal": ("mixed", "modal"), "learned": ("mixed", "learned"),
         "modal_r32": ("mixed_r32", "modal"), "learned_r32": ("mixed_r32", "learned")}


def run_single_form(args):
    """One form on one workload (the double Mach reflection unless --workload names another):
    device time per step, the volume kernel's mean launch time and, with a troubled-cell list,
    the troubled cells of the last RHS (no end-to-end pass, no accuracy comparison)."""
    import torch

    torch.cuda.set_device(0)
    prec, sensor = FORMS[args.form]
    r = measure_form(prec, sensor, args.steps, args.warmup, 0, _sensor_weights() if sensor == "learned" else None,
                     workload=args.workload or "dmr",
                     tensor_cores=False if args.sensor_cuda_cores else None, e2e=False,
                     indicator_tc=False if args.indicator_cuda_cores else None, mesh=args.mesh)
    nd = r["case"].n_dofs
    vol = r["vol_ms"] / max(r["vol_n"], 1)
    print(json.dumps({"form": args.form, "workload": args.workload or "dmr", "mesh": list(args.mesh),
                      "n_cells": r["case"].n_cells,
                      "precision": prec, "sensor": sensor, "steps": args.steps,
                      "indicator_cuda_cores": args.indicator_cuda_cores,
                      "ms_per_step": r["ms"] / args.steps, "dof_stage_per_s": nd * 5 * args.steps / (r["ms"] / 1e3),
                      "volume_kernel_ms": vol, "gpu_launches": r["launches"], "clocks": r["clocks"],
                      "troubled_cells": r["lo_cells"],
                      "troubled_fraction": (r["lo_cells"] / r["case"].n_cells) if r["lo_cells"] is not None else None,
                      "sensor_stats": r["stats"]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="", choices=["", "sod", "dmr", "cylinder", "shock_vortex"],
                    help="per-configuration report (throughput of every form, accuracy after --accuracy-steps) "
                         "instead of the benchmark line")
    ap.add_argument("--accuracy-steps", type=int, default=0, help="override the accuracy window (steps)")
    ap.add_argument("--sensor-cuda-cores", action="store_true",
                    help="the learned sensor's network on the CUDA cores (the default at degree 3 is the fused "
                         "tensor-core kernel)")
    ap.add_argument("--indicator-cuda-cores", action="store_true",
                    help="the modal indicator's change of basis on the CUDA cores (mixed forms, degree 3; "
                         "the default there is the tensor-core form)")
    ap.add_argument("--horizon", default="", help="comma-separated DMR z variants: " + ",".join(HORIZON_VARIANTS))
    ap.add_argument("--horizon-precision", default="mixed", choices=["fp64", "mixed", "mixed_r32"])
    ap.add_argument("--form", default="", choices=["", "plain", "modal", "learned", "modal_r32", "learned_r32"],
                    help="time one form only and print its numbers (a short run for profiling) instead of "
                         "the benchmark line")
    ap.add_argument("--mesh", default="",
                    help="with --form: comma-separated cell counts replacing the workload's ("
                         + "; ".join(f"{w}: {','.join(a)}" for w, a in MESH_ARGS.items()) + ")")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    args.mesh = tuple(int(v) for v in args.mesh.split(",")) if args.mesh else ()
    if args.mesh and not args.form:
        ap.error("--mesh applies to --form runs only")
    if len(args.mesh) > len(MESH_ARGS[args.workload or "dmr"]):
        ap.error(f"--mesh: {args.workload or 'dmr'} takes {len(MESH_ARGS[args.workload or 'dmr'])} count(s)")
    if args.impl == "reference":
        run_reference(args)
        return
    if args.horizon:
        run_horizon(args)
        return
    if args.form:
        run_single_form(args)
        return
    if args.workload:
        run_workload_report(args)
        return

    import torch
    import torch.distributed as dist

    ws, rank, local = _dist()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    device = torch.device("cuda", local if ws > 1 else 0)

    import __graft_entry__
    if not (ROOT / "plens_gb300" / "lib" / "libplens_gpu.so").exists():
        if rank == 0:
            __graft_entry__.build()
        barrier()

    weights = _sensor_weights()
    cache = {}
    plain = measure_form("fp64", "modal", args.steps, args.warmup, device.index, cache=cache)
    modal = measure_form("mixed", "modal", args.steps, args.warmup, device.index, cache=cache)
    learned = (measure_form("mixed", "learned", args.steps, args.warmup, device.index, weights, cache=cache,
                            tensor_cores=False if args.sensor_cuda_cores else None)
               if weights is not None else None)
    learned_r32 = (measure_form("mixed_r32", "learned", args.steps, args.warmup, device.index, weights, cache=cache,
                                tensor_cores=False if args.sensor_cuda_cores else None)
                   if weights is not None else None)
    fast = learned if learned is not None else modal
    fast_sensor = "learned" if learned is not None else "modal"

    case = plain["case"]
    nd = case.n_dofs
    job = {}
    for k, r in (("plain", plain), ("modal", modal), ("learned", learned), ("learned_r32", learned_r32)):
        if r is None:
            continue
        t = max_over_ranks(r["ms"] / 1e3, device)
        te = max_over_ranks(r["e2e_s"], device)
        ts = max_over_ranks(r["serial_s"], device)
        job[k] = {"value": nd * 5 * args.steps * ws / t, "ms_per_step": 1e3 * t / args.steps,
                  "e2e": nd * 5 * r["e2e_steps"] * ws / te,
                  "e2e_serial_calls": nd * 5 * r["serial_steps"] * ws / ts,
                  "volume_kernel_ms": r["vol_ms"] / max(r["vol_n"], 1),
                  "bytes_per_dof_stage": BYTES_PER_DOF_STAGE[k],
                  "achieved_gbs": BYTES_PER_DOF_STAGE[k] * nd / (r["vol_ms"] / max(r["vol_n"], 1) / 1e3) / 1e9}
    # accuracy of the FP32 forms against the plain FP64 form after the same steps
    job["modal"]["rel_l1_vs_fp64_plain"] = dict(zip(("rho", "momentum", "rhoE"), _rel_l1(modal["U"], plain["U"])))
    if learned is not None:
        for k, r in (("learned", learned), ("learned_r32", learned_r32)):
            job[k]["rel_l1_vs_fp64_plain"] = dict(zip(("rho", "momentum", "rhoE"), _rel_l1(r["U"], plain["U"])))
            job[k]["sensor_stats"] = r["stats"]

    if rank != 0:
        return
    peak, peak_kind = _peaks()
    hd = job["learned"] if learned is not None else job["modal"]
    achieved = hd["achieved_gbs"]
    line = {
        "metric": METRIC,
        "value": hd["value"],
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": hd["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 flux differencing, surface fluxes, indicator; f64 state, metric terms, 1/detJ scaling, "
                 "RK registers and their accumulation",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": f"mixed FP32 + {fast_sensor} sensor"
                   + (" (network on the CUDA cores)" if args.sensor_cuda_cores and learned is not None else
                      " (fused tensor-core sensor and modal indicator)"),
                   "l2": "working set per step > L2 (state, 3 registers, metrics, face buffers ~ 0.5 GB)",
                   "parallelism": f"replicas x{ws}"},
        "forms": {
            "fp64_plain": job["plain"],
            "fp32_modal_sensor": job["modal"],
            "fp32_learned_sensor": job.get("learned"),
            "fp32_r32_learned_sensor": dict(job["learned_r32"], dtype="f32 flux differencing, f32 RK registers and "
                                            "metric images, f64 state") if "learned_r32" in job else None,
            "multiple_headline_over_fp64_plain": hd["value"] / job["plain"]["value"],
        },
        "roofline": {
            "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind, "kernel": f"k_volume_mx (mixed form, {fast_sensor} sensor)",
            "traffic": _traffic_from_profile("k_volume_mx_dmr.md"),
            "note": "achieved: algorithmic 272 B per DOF-stage (FP64 state r/w 80, two FP64 registers read "
                    "80, one written 40 at stages 1-4 (none at the last stage, whose dt*R no stage reads), "
                    "Ja and 1/detJ 80) x 921600 DoFs per launch / mean CUDA-event launch time of the "
                    "kernel-timing pass; traffic: ncu DRAM bytes of a stage-1 launch from "
                    "profiles/k_volume_mx_dmr.md",
            "moved_bytes_per_dof_stage": MOVED_BYTES_MIXED,
            "achieved_moved": MOVED_BYTES_MIXED * achieved / BYTES_PER_DOF_STAGE["learned"],
            "moved_note": "what the kernel reads and writes per DOF-stage, averaged over the five stages: FP64 "
                          "state r/w 80; FP64 registers read 56 (none at stage 1, one at stage 2, two at "
                          "stages 3-5) and written 32; the FP32 rounding of Ja 36 (an image made once, the "
                          "values of rounding the FP64 Ja) and FP64 1/detJ 8; the FP32 state image r/w 40; "
                          "the FP32 face values 30",
        },
        "e2e": {"value": hd["e2e"], "unit": UNIT, "h2d_bytes_per_step": fast["bytes_state"],
                "d2h_bytes_per_step": fast["bytes_state"],
                "how": "plens_gpu_advance_states over a sequence of one-step members from page-locked host "
                       "buffers (host -> device copy, one step, device -> host copy per member; the copies run "
                       "on copy streams beside the steps)",
                "serial_calls": hd["e2e_serial_calls"]},
        "gpu_launches": fast["launches"],
        "clocks": fast["clocks"],
    }
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"] = cpu_baseline(max_seconds=15.0)
    print(json.dumps(line), flush=True)
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
