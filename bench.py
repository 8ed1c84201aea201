#!/usr/bin/env python3
"""Benchmark of the compact3d channel time step on GB300: grid-point-substeps/s.

One "step" is one call of GETUP (compact3d.f:879-960) on the whole channel; the reference
is single-stage AB2/Crank-Nicolson, so one substep is one step and the metric is
N1M*N2M*N3M * steps / second.

Arms
  default (ours)     the CUDA library through its C-ABI, on the workload named by
                     --workload (default channel384: 384 x 257 x 384 points, Re_tau ~550),
                     in the FP32-mixed form (--form), with the plain FP64 form measured in
                     the same run for comparison and the relative L2 error of the mixed form
                     against the FP64 form after the same steps.
                     Further sections of the same JSON line: "batched" (32 uneven
                     channels as one CUDA graph per ensemble step, against the same
                     channels stepped one after another in FP64) and "les" (the
                     wall-modelled LES workload les128 in both forms, with the mixed
                     form's wall stress, bulk velocity and velocity error against FP64
                     after --les-steps steps) and "operators" (each compact operator, y
                     stencil and the Poisson solve alone on the 256 x 193 x 256 field,
                     FP64 and mixed, with GB/s against the HBM peak).
  --impl reference   the reference's CPU path on all host cores, on the same whole grid: the
                     reference's own routines (compact3d.f translated to C with its OpenMP
                     loops, oracle/ref.py) where a translation is present, else the FP64
                     OpenMP restatement of the step (oracle/).

Multi-GPU: under torchrun every rank advances its own channel (independent replicas, no
collective on the data path); the time is the max over ranks and ``value`` the sum of all
ranks' points / that time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from compact3d_gb300 import ic  # noqa: E402
from compact3d_gb300.grid import C3D_FP64, C3D_MIXED, C3D_MIXED_IR, WORKLOADS, make_grid  # noqa: E402

METRIC = "grid-pt-substeps/s on 1 GB300: FP32-mixed & batched vs FP64, at stated L2 err"
UNIT = "grid-pt-substeps/s"


# ------------------------------------------------------------------------------------
# distributed plumbing (only when launched by torchrun with WORLD_SIZE > 1)
# ------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------
class Clocks:
    """SM clock, power and throttle reasons sampled every 10 ms during the timed region.

    NVML is read through ctypes (libnvidia-ml.so.1, the driver's own library; reading
    changes no setting).  The device is found by the CUDA device's UUID, so the index
    mapping of CUDA_VISIBLE_DEVICES does not matter.  Without NVML, ``nvidia-smi -lms``
    samples instead (200 ms apart)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, gpu: int, interval_s: float = 0.01):
        self.gpu = gpu
        self.interval = interval_s
        self.proc = None
        self.path = None
        self.nv = None
        self.thread = None
        try:
            self._nvml_open()
        except Exception:
            self.nv = None

    def _nvml_open(self):
        import ctypes
        import torch
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit")
        uuid = "GPU-" + str(torch.cuda.get_device_properties(self.gpu).uuid)
        h = ctypes.c_void_p()
        if nv.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h)) != 0:
            raise RuntimeError("nvmlDeviceGetHandleByUUID")
        self.h = h
        self.nv = nv
        self.reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))   # NVML_CLOCK_SM = 1
        self.max_mhz = float(mx.value)

    def _sample_loop(self):
        import ctypes
        mhz, mw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_flag:
            ok = self.nv.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(mhz)) == 0
            self.nv.nvmlDeviceGetPowerUsage(self.h, ctypes.byref(mw))
            self.reasons_fn(self.h, ctypes.byref(rs))
            if ok:
                self.rows.append((float(mhz.value), mw.value / 1e3, int(rs.value)))
            time.sleep(self.interval)

    def start(self):
        if self.nv is not None:
            import threading
            self.rows = []
            self.stop_flag = False
            self.thread = threading.Thread(target=self._sample_loop, daemon=True)
            self.thread.start()
            return
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.thread is not None:
            self.stop_flag = True
            self.thread.join()
            self.thread = None
            rows = self.rows
            if not rows:
                return None
            reasons = sorted({k for r in rows for k, b in self.BITS.items() if r[2] & b})
            return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": self.max_mhz,
                    "power_w_max": max(r[1] for r in rows), "reasons": reasons, "samples": len(rows),
                    "source": f"NVML every {self.interval * 1e3:.0f} ms"}
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi every 200 ms"}


class L2Flush:
    """Overwrites a 512 MB device buffer (4x the 129 MB L2) between timed iterations of
    the workloads whose working set fits in L2; the channel stream is idle meanwhile."""

    def __init__(self, device: int):
        import torch
        self.torch = torch
        self.buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")

    def __call__(self):
        self.buf.add_(1.0)
        self.torch.cuda.synchronize()


def host_link_gbs(device: int, nbytes: int = 1 << 30):
    """Copy rate of the host link in each direction (GB/s): one pinned 1 GiB buffer
    copied to and from the device with cudaMemcpyAsync, best of three, CUDA events."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=f"cuda:{device}")
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = None
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            dst.copy_(src, non_blocking=True)
            b.record()
            b.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / best / 1e6
    del h, d
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_for(workload: str, form: str, kernel: str):
    """DRAM bytes per launch of `kernel` from a committed ncu summary, if there is one."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(f"{workload}/{form}/{kernel}")
    return None if e is None else float(e["bytes_per_launch"])


# ------------------------------------------------------------------------------------
# CPU reference (oracle restatement of the reference's OpenMP path)
# ------------------------------------------------------------------------------------
def _mem_available_gb() -> float:
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


# host memory the reference's own routines need on channel384 (static arrays of the
# compile-time extents, about 24 GB resident), with a margin
REF_MEM_GB = 48.0


def cpu_reference(workload: str, steps: int, warmup: int):
    """Time the reference's CPU path on the whole `workload` grid, on all host cores:
    `warmup` untimed steps, then exactly `steps` timed steps (host wall clock).

    The reference's own routines run when they are available: compact3d.f translated to C
    with its !$OMP PARALLEL DO loops kept (oracle/f77c.py, oracle/ref.py; FFTW replaced by
    oracle/fftw_shim.c), which needs a translation made where the reference source is and
    REF_MEM_GB of available host memory.  Otherwise the OpenMP oracle restatement of the
    same step runs.  Returns (rate in pt-steps/s, seconds per step, cores, kind, sample)."""
    os.environ.setdefault("OMP_STACKSIZE", "64M")   # before any OpenMP runtime starts
    import oracle
    from oracle import ref
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    g, dt = make_grid(workload)
    U, P, HH = ic.perturbed_laminar(g)
    o = oracle.Oracle(g, threads=cores)
    o.project(U)
    use_ref = ref.available(g.n1, g.n2, g.n3, omp=True) and _mem_available_gb() >= REF_MEM_GB
    if use_ref:
        del o
        runner = ref.RefChannel(g, omp=True)
        kind, what = "reference", ("the reference's own GETUP (compact3d.f translated to C with its OpenMP loops, "
                                   "FFTW replaced by the DFT it documents)")
    else:
        runner = o
        kind, what = "port", "the OpenMP oracle restatement of GETUP"
    pg = pg3 = 0.0
    n = 1
    for _ in range(warmup):
        pg, pg3 = runner.getup(U, P, HH, n, dt, pg, pg3)
        n += 1
    steps = max(1, steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        pg, pg3 = runner.getup(U, P, HH, n, dt, pg, pg3)
        n += 1
    t = time.perf_counter() - t0
    rate = g.points * steps / t
    sample = (f"{steps} timed steps (after {warmup} untimed) of {what} on the whole {workload} grid, "
              f"{g.n1m}x{g.n2m}x{g.n3m} cells, FP64, {cores} OpenMP threads")
    return rate, t / steps, cores, kind, sample


def workload_config(args, g, dt, form):
    """The `config` object both arms print for the workload."""
    return dict(workload=f"{args.workload}: {g.n1m}x{g.n2m + 1}x{g.n3m} points "
                         f"(cells {g.n1m}x{g.n2m}x{g.n3m}), RE={g.re}, dt={dt}, "
                         + (f"y tanh-stretched beta={g.cks}" if g.wmodel == 0 else "uniform y"),
                form=form, cells=[g.n1m, g.n2m, g.n3m])


FORMS = {"mixed": C3D_MIXED, "fp64": C3D_FP64, "mixed_ir": C3D_MIXED_IR}


def make_channel(lib, g, form, U, P, HH):
    ch = lib.Channel(g, FORMS[form])
    ch.upload(U, P, HH)
    ch.project()
    ch.set_presg(0.0, 0.0)
    return ch


def run_ours(args, D: Dist):
    from compact3d_gb300 import lib
    lib.check(lib.load().c3d_set_device(D.local), "c3d_set_device")
    g, dt = make_grid(args.workload)
    U0, P0, HH0 = ic.perturbed_laminar(g, seed=ic.SEED0 + D.rank)
    pts = g.points
    K, W = args.steps, args.warmup

    # ---- main form, device-resident (value) ----
    ch = make_channel(lib, g, args.form, U0, P0, HH0)
    if args.schedule:
        ch.set_schedule(json.loads(args.schedule))
        schedule = ch.get_schedule()
    else:
        schedule = ch.autotune() if not args.no_tune else ch.get_schedule()
    n = 1
    for _ in range(W):
        ch.step_async(n, dt)
        n += 1
    ch.sync()
    launches_per_step = ch.last_step_stats()[1]
    clocks = Clocks(D.local)
    field_bytes = 8 * g.n1m * (g.n2m + 2) * g.n3m
    small = field_bytes < 2 * 129e6   # a field smaller than twice L2: flush it between steps
    flush = L2Flush(D.local) if small else None
    D.barrier()
    clocks.start()
    if small:
        ms = 0.0
        for _ in range(K):
            flush()
            ch.timer_start()
            ch.step_async(n, dt)
            n += 1
            ms += ch.timer_stop()
    else:
        ch.timer_start()
        for _ in range(K):
            ch.step_async(n, dt)
            n += 1
        ms = ch.timer_stop()
    ck = clocks.stop()
    D.barrier()
    ms_max = D.max(ms)
    total_pts = D.sum(pts)
    value = total_pts * K / (ms_max / 1e3)
    res = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=D.world, steps=K, warmup=W,
               ms_per_step=ms_max / K, higher_is_better=True, scaling="weak", vs_baseline=None,
               dtype="f64" if args.form == "fp64" else "f32+f64 mixed", data="synthetic")
    res["config"] = workload_config(args, g, dt, args.form)
    res["config"]["l2_policy"] = (f"L2 flushed (512 MB written) before every timed step, each step timed alone; "
                                  f"each FP64 field is {field_bytes / 1e6:.0f} MB" if small else
                                  f"inputs larger than L2: each FP64 field is {field_bytes / 1e6:.0f} MB")
    res["config"]["parallelism"] = f"replicas x{D.world}"
    res["gpu_launches"] = launches_per_step * K
    res["schedule"] = schedule
    if ck:
        res["clocks"] = ck

    # ---- per-kernel profile (separate short run, CUDA events around each launch) ----
    ch.profile(True)
    for _ in range(2):
        ch.step_async(n, dt)
        n += 1
    ch.sync()
    prof = ch.profile_read()
    ch.profile(False)
    dom = max(prof, key=lambda e: e["ms"])
    peak, kind = peaks()
    avg_ms = dom["ms"] / dom["launches"]
    achieved = dom["bytes"] / (avg_ms / 1e3) / 1e9
    res["roofline"] = dict(bound="hbm", kernel=dom["name"], achieved=achieved, peak=peak,
                           unit="GB/s", frac=achieved / peak, peak_kind=kind,
                           traffic=traffic_for(args.workload, args.form, dom["name"]),
                           alg_bytes_per_launch=dom["bytes"], avg_launch_ms=avg_ms)
    step_ms = sum(e["ms"] for e in prof) / 2
    # whole step against the five-pass plane-fused schedule's algorithmic bytes per
    # grid-point-substep (264 B mixed, 320 B FP64), and the bytes the kernels of this
    # build are specified to move per point
    b_alg = 320.0 if args.form == "fp64" else 264.0
    step_gbs = value / D.world * b_alg / 1e9
    res["step_roofline"] = dict(bytes_per_point=b_alg, achieved=step_gbs, peak=peak, unit="GB/s",
                                frac=step_gbs / peak, peak_kind=kind,
                                kernel_bytes_per_point=sum(e["bytes"] for e in prof) / 2 / pts)
    res["kernels"] = {e["name"]: dict(ms=e["ms"] / e["launches"], share=e["ms"] / (2 * step_ms),
                                      gbs=e["bytes"] / (e["ms"] / e["launches"] / 1e3) / 1e9)
                      for e in prof}

    # ---- FP64 form in the same run, and the mixed form's error against it ----
    if args.form != "fp64" and not args.no_fp64:
        c64 = make_channel(lib, g, "fp64", U0, P0, HH0)
        if not args.no_tune:
            c64.autotune()
        m = 1
        for _ in range(W):
            c64.step_async(m, dt)
            m += 1
        c64.sync()
        k64 = max(2, min(K, args.fp64_steps))
        c64.timer_start()
        for _ in range(k64):
            c64.step_async(m, dt)
            m += 1
        ms64 = D.max(c64.timer_stop())
        res["fp64"] = dict(value=total_pts * k64 / (ms64 / 1e3), ms_per_step=ms64 / k64, steps=k64)
        # the other mixed variant (with / without the pressure refinement step)
        other = "mixed_ir" if args.form == "mixed" else "mixed"
        co = make_channel(lib, g, other, U0, P0, HH0)
        if not args.no_tune:
            co.autotune()
        m = 1
        for _ in range(W):
            co.step_async(m, dt)
            m += 1
        co.sync()
        co.timer_start()
        for _ in range(K):
            co.step_async(m, dt)
            m += 1
        mso = D.max(co.timer_stop())
        res[other] = dict(value=total_pts * K / (mso / 1e3), ms_per_step=mso / K, steps=K)
        co.close()
        c64.close()
        res["err_vs_fp64"] = error_study(lib, g, dt, U0, P0, HH0, args.err_steps, floor=not args.no_floor)

    # ---- end to end through the host-array drop-in (c3d_getup) ----
    if not args.no_e2e:
        from compact3d_gb300 import lib as L
        # the driver's arrays in page-locked memory from c3d_host_alloc (an array pinned
        # after the fact keeps whatever physical pages it has; after another process has
        # used and freed tens of GB of host memory those transfer far below the link rate)
        U, P, HH = (L.host_array(a.shape) for a in (U0, P0, HH0))
        U[...], P[...], HH[...] = U0, P0, HH0
        ce = lib.Channel(g, FORMS[args.form])
        ce.upload(U, P, HH)
        ce.project()
        ce.download(U, P, HH)
        pg = pg3 = 0.0
        m = 1
        for _ in range(min(W, 2)):
            pg, pg3 = ce.getup(U, P, HH, m, dt, pg, pg3)
            m += 1
        # The host memory behind the link is shared with the machine's other tenants: a
        # window of getups now and then runs at half the link rate although the pages and
        # the path are unchanged, so the figure is the median of several timed windows and
        # every window is listed.
        ke = max(2, min(K, args.e2e_steps))
        wins = []
        for _ in range(max(1, args.e2e_windows)):
            D.barrier()
            t0 = time.perf_counter()
            for _ in range(ke):
                pg, pg3 = ce.getup(U, P, HH, m, dt, pg, pg3)
                m += 1
            wins.append(D.max(time.perf_counter() - t0))
        te = statistics.median(wins)
        bytes_io = U.nbytes + P.nbytes + HH.nbytes
        link = host_link_gbs(D.local)
        # Floor of a getup: every input byte must cross the link before the step can finish
        # and every output byte after it starts, and the step hides behind the transfers
        # (HH moves while the step runs), so in / h2d rate + out / d2h rate.
        floor_ms = bytes_io / link["h2d"] / 1e6 + bytes_io / link["d2h"] / 1e6
        e2e_ms = te / ke * 1e3
        res["e2e"] = dict(value=total_pts * ke / te, unit=UNIT, h2d_bytes_per_step=bytes_io,
                          d2h_bytes_per_step=bytes_io, steps=ke, ms_per_step=e2e_ms,
                          link_gbs={k: round(v, 1) for k, v in link.items()},
                          floor_ms=floor_ms, frac_of_floor=floor_ms / e2e_ms,
                          windows_ms_per_step=[round(w / ke * 1e3, 2) for w in wins],
                          path="c3d_getup: Fortran-layout host arrays in page-locked memory (c3d_host_alloc) by DMA through a device "
                               "staging area on a copy stream, U/P then HH in, HH out from the end of xB "
                               "while the step runs, U/P out after it")
        ce.close()
        for a in (U, P, HH):
            L.host_free(a)
    ch.close()

    # ---- batched ensemble (configs with many independent channels) ----
    if not args.no_batch:
        res["batched"] = run_batched(args, D)

    # ---- wall-modelled LES ----
    if not args.no_les:
        res["les"] = run_les(args, D)

    # ---- operators one at a time (compact derivatives, y stencils, Poisson) ----
    if not args.no_ops:
        res["operators"] = run_operators(args, D)

    # ---- the rows after the step: plane statistics, checkpoint, a second wall model ----
    if not args.no_next:
        res["next_rows"] = run_next(args, D, g, dt, U0, P0, HH0)

    # ---- CPU baseline (rank 0, N=1 only) ----
    if D.rank == 0 and D.world == 1 and not args.no_cpu:
        rate, _, cores, kind, sample = cpu_reference(args.workload, steps=2, warmup=1)
        res["cpu_baseline"] = dict(value=rate, unit=UNIT, cores=cores, kind=kind, sample=sample)
    return with_summary(res)


def with_summary(res: dict) -> dict:
    """Orders the line so that the long per-kernel and per-section tables come first and a
    compact summary of every form's headline figure comes last (the end of the line is
    what a truncated log keeps)."""
    big = ("kernels", "schedule", "operators", "next_rows", "les", "batched", "err_vs_fp64")
    out = {k: v for k, v in res.items() if k not in big}
    tail = {k: res[k] for k in big if k in res}
    summ = dict(mixed=res["value"], ms_per_step=res["ms_per_step"])
    for k in ("fp64", "mixed_ir"):
        if k in res:
            summ[k] = res[k]["value"]
    b = res.get("batched")
    if b:
        summ["batched"] = b["value"]
        for k in ("streams_form", "mixed_sequential", "fp64_sequential"):
            if k in b:
                summ["batched_" + k] = b[k]["value"]
    e = res.get("err_vs_fp64")
    if e and "mixed" in e:
        summ["err_vs_fp64"] = {k: e["mixed"][k] for k in ("u", "v", "w", "p", "p_mean", "p_fluct", "divmax", "bulk_rel",
                                                           "wsm_rel")}
        summ["err_vs_fp64"]["steps"] = e["steps"]
    l_ = res.get("les")
    if l_:
        summ["les128_ms"] = {f: l_[f]["ms_per_step"] for f in ("mixed", "fp64") if f in l_}
    for k in ("roofline", "step_roofline"):
        if k in res:
            summ[k + "_frac"] = res[k]["frac"]
    if "e2e" in res:
        summ["e2e"] = res["e2e"]["value"]
    if "cpu_baseline" in res:
        summ["cpu_baseline"] = res["cpu_baseline"]["value"]
    out.update(tail)
    out["summary"] = summ
    return out


def flow_stats(U, g):
    """Plane statistics of a velocity field (host array U(0:M1,0:M2,0:M3,3)): the mean
    streamwise profile and the RMS profiles of u', v', w' and the shear stress <u'v'>, all
    at the cell centres j = 1..N2M (v averaged from the two faces)."""
    n1, n2, n3 = g.n1m, g.n2m, g.n3m
    u = U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0]
    v = 0.5 * (U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 1] + U[1:n1 + 1, 2:n2 + 2, 1:n3 + 1, 1])
    w = U[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2]
    um = u.mean(axis=(0, 2))
    up, vp, wp = u - um[None, :, None], v - v.mean(axis=(0, 2))[None, :, None], w - w.mean(axis=(0, 2))[None, :, None]
    return dict(mean_u=um, urms=np.sqrt((up ** 2).mean(axis=(0, 2))), vrms=np.sqrt((vp ** 2).mean(axis=(0, 2))),
                wrms=np.sqrt((wp ** 2).mean(axis=(0, 2))), uv=(up * vp).mean(axis=(0, 2)))


def error_study(lib, g, dt, U0, P0, HH0, steps: int, floor: bool = True):
    """Error of the mixed form against the FP64 GPU form after `steps` steps from the same
    start: relative L2 of u, v, w (interiors) and of P, max |div u|, bulk velocity
    FLOW1/ALY, plane-mean wall shear WSM(1), PRESG, and the relative L2 of the mean profile
    and of the RMS and shear-stress profiles.  With `floor`, the same figures for an FP64
    run whose start was perturbed by 1e-15 max|U| (projected): the chaotic growth of a
    round-off-sized difference, below which no form can be compared."""
    n1, n2, n3 = g.n1m, g.n2m, g.n3m

    def rl(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    runs = {"mixed": make_channel(lib, g, "mixed", U0, P0, HH0), "fp64": make_channel(lib, g, "fp64", U0, P0, HH0),
            "mixed_ir": make_channel(lib, g, "mixed_ir", U0, P0, HH0)}
    if floor:
        rng = np.random.default_rng(ic.SEED0 + 77)
        Up = U0 + 1e-15 * float(np.abs(U0).max()) * rng.standard_normal(U0.shape)
        runs["fp64_perturbed"] = make_channel(lib, g, "fp64", np.asfortranarray(Up), P0, HH0)
    for s in range(1, steps + 1):
        for c in runs.values():
            c.step_async(s, dt)
    fields = {k: c.download() for k, c in runs.items()}
    diags = {k: c.diagnose() for k, c in runs.items()}
    presg = {k: c.get_presg() for k, c in runs.items()}
    for c in runs.values():
        c.close()
    Uf, Pf, _ = fields["fp64"]
    sf = flow_stats(Uf, g)
    out = dict(steps=steps, reference="FP64 GPU form (per step within 1e-10 of the FP64 oracle)")
    for name in [k for k in runs if k != "fp64"]:
        Um, Pm, _ = fields[name]
        sm = flow_stats(Um, g)
        d = diags[name]
        out[name] = dict(
            u=rl(Um[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], Uf[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0]),
            v=rl(Um[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1], Uf[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1]),
            w=rl(Um[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], Uf[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2]),
            p=rl(Pm[:n1, :n2, :n3], Pf[:n1, :n2, :n3]),
            # P split into its plane means (the kx = kz = 0 Poisson mode) and the rest
            p_mean=rl(Pm[:n1, :n2, :n3].mean(axis=(0, 2)), Pf[:n1, :n2, :n3].mean(axis=(0, 2))),
            p_fluct=rl(Pm[:n1, :n2, :n3] - Pm[:n1, :n2, :n3].mean(axis=(0, 2))[None, :, None],
                       Pf[:n1, :n2, :n3] - Pf[:n1, :n2, :n3].mean(axis=(0, 2))[None, :, None]),
            divmax=d["divmax"], bulk=d["flow1"] / g.aly, wsm=float(d["wsm"][0]), presg=presg[name][0],
            mean_u=rl(sm["mean_u"], sf["mean_u"]),
            rms=rl(np.concatenate([sm[k] for k in ("urms", "vrms", "wrms", "uv")]),
                   np.concatenate([sf[k] for k in ("urms", "vrms", "wrms", "uv")])))
        out[name]["bulk_rel"] = abs(out[name]["bulk"] - diags["fp64"]["flow1"] / g.aly) / abs(diags["fp64"]["flow1"] / g.aly)
        out[name]["wsm_rel"] = abs(out[name]["wsm"] - float(diags["fp64"]["wsm"][0])) / abs(float(diags["fp64"]["wsm"][0]))
    out["fp64"] = dict(divmax=diags["fp64"]["divmax"], bulk=diags["fp64"]["flow1"] / g.aly,
                       wsm=float(diags["fp64"]["wsm"][0]), presg=presg["fp64"][0])
    return out


def run_next(args, D: Dist, g, dt, U0, P0, HH0):
    """ENERGY's plane statistics and a checkpoint write + read on the main workload (mixed
    form), and the LES step with the algebraic wall models WERNER, MARUSIC1 and PIOMELLI and
    with the scale-dependent SGS model on les128 (mixed form)."""
    import shutil
    import tempfile
    from compact3d_gb300 import lib
    out = {}
    ch = make_channel(lib, g, "mixed", U0, P0, HH0)
    ch.step(1, dt, 0.0, 0.0)
    ch.plane_stats()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        ch.plane_stats()
    ms = (time.perf_counter() - t0) / reps * 1e3
    # two passes over the plane: u, v, w, P (double-float) and u, v, w again
    alg = 7 * 8.0 * g.points
    out["plane_stats"] = dict(ms_per_call=ms, alg_bytes=alg, gbs=alg / ms / 1e6, values_per_plane=29,
                              note="FP64 arithmetic on the double-float state; host-timed call incl. copy-out")
    ch.plane_spectra()
    t0 = time.perf_counter()
    for _ in range(2):
        ch.plane_spectra()
    ms_sp = (time.perf_counter() - t0) / 2 * 1e3
    out["plane_spectra"] = dict(ms_per_call=ms_sp, tables="XSPCTR, ZSPCTR, RXX, RZZ, RXY (3 components)",
                                note="FP64 FFTs of every x and z line of the three components, the plane statistics "
                                     "for VM/VRMS, host-timed call incl. copy-out")
    # particles: one step of 1M particles in the channel (host arrays in and out)
    rng = np.random.default_rng(5)
    npar = 1_000_000
    Dp = 0.0002 / 0.05
    par = np.column_stack([rng.uniform(0, g.alx, npar), rng.uniform(0.5 * Dp, 2.0 - 0.5 * Dp, npar),
                           rng.uniform(0, g.alz, npar), rng.normal(0.5, 0.2, npar), rng.normal(0, 0.05, npar),
                           rng.normal(0, 0.05, npar)])
    ch.particles_advance(par, dt)
    t0 = time.perf_counter()
    for _ in range(3):
        ch.particles_advance(par, dt)
    ms_p = (time.perf_counter() - t0) / 3 * 1e3
    out["particles"] = dict(particles=npar, ms_per_step=ms_p, particles_per_s=npar / ms_p * 1e3,
                            note="CALC_UX_4RK + BC_PAR on the device (4 interpolations of u, v, w per particle, FP64), "
                                 "host arrays copied in and out inside the timing")
    d = tempfile.mkdtemp(prefix="c3d_ckpt_")
    try:
        path = os.path.join(d, "ckpt.bin")
        t0 = time.perf_counter()
        ch.checkpoint_write(path, 1, dt, 0.0, 0.0)
        tw = time.perf_counter() - t0
        nbytes = os.path.getsize(path)
        r = lib.Channel(g, FORMS["mixed"])
        t0 = time.perf_counter()
        r.checkpoint_read(path)
        tr = time.perf_counter() - t0
        r.close()
        out["checkpoint"] = dict(bytes=nbytes, write_ms=tw * 1e3, read_ms=tr * 1e3,
                                 write_gbs=nbytes / tw / 1e9, read_gbs=nbytes / tr / 1e9,
                                 note="file in a temporary directory of the host; includes device packing, copies, fwrite/fread")
    finally:
        shutil.rmtree(d, ignore_errors=True)
    ch.close()
    for key, over, label in (("les_werner", dict(wmodel=4), "SGSCS + WALLMODEL_WERNER (WMODEL 4)"),
                             ("les_marusic", dict(wmodel=3), "SGSCS + MARUSIC1 (WMODEL 3)"),
                             ("les_piomelli", dict(wmodel=5), "SGSCS + PIOMELLI (WMODEL 5)"),
                             ("les_sgssd", dict(files=3), "SGSSD (FILES 3) + WALLMODEL_INSTANT"),
                             ("les_iwmles", dict(wmodel=2), "SGSCS + WALLMODEL_IWMLES_SMOOTH (WMODEL 2), "
                                                            "model updates every fifth step inside the timed steps")):
        gl, dtl = make_grid("les128", **over)
        Ul, Pl, Hl = ic.loglaw(gl, 2000.0, amp=0.05, seed=ic.SEED0 + 3000 + D.rank)
        c = make_channel(lib, gl, "mixed", Ul, Pl, Hl)
        if not args.no_tune:
            c.autotune()
        flush = L2Flush(D.local)
        n = 1
        for _ in range(max(3, args.warmup)):
            c.step_async(n, dtl)
            n += 1
        c.sync()
        K = args.steps
        msl = 0.0
        for _ in range(K):
            flush()
            c.timer_start()
            c.step_async(n, dtl)
            n += 1
            msl += c.timer_stop()
        msl = D.max(msl)
        out[key] = dict(workload=f"les128, {label}, mixed form, L2 flushed per step",
                        value=D.sum(gl.points) * K / (msl / 1e3), unit=UNIT, ms_per_step=msl / K, steps=K,
                        wsm=float(c.get_wsm()[0]))
        c.close()
    return out


def run_les(args, D: Dist):
    """The wall-modelled LES workload (les128: 128 x 65 x 128 points, 8pi x 2 x 3pi,
    Re_tau ~2000, SGSCS + WALLMODEL_INSTANT, seeded log-law start with a 5% perturbation):
    grid-pt-substeps/s of the mixed and FP64 forms, and after `les_steps` steps from the
    same start the mixed form's wall stress WSM(1), bulk velocity and velocity error
    against the FP64 form."""
    from compact3d_gb300 import lib
    g, dt = make_grid("les128")
    U0, P0, HH0 = ic.loglaw(g, 2000.0, amp=0.05, seed=ic.SEED0 + 3000 + D.rank)
    out = dict(workload=f"les128: {g.n1m}x{g.n2m + 1}x{g.n3m} points, 8pi x 2 x 3pi, uniform y, "
                        f"RE={g.re} (Re_tau ~2000), dt={dt}, SGSCS + WALLMODEL_INSTANT, log-law start + 5%",
               l2_policy="L2 flushed (512 MB written) before every timed step; each step timed alone")
    flush = L2Flush(D.local)
    for form in ("mixed", "fp64"):
        ch = make_channel(lib, g, form, U0, P0, HH0)
        if not args.no_tune:
            ch.autotune()
        n = 1
        for _ in range(max(3, args.warmup)):
            ch.step_async(n, dt)
            n += 1
        ch.sync()
        K = args.steps
        ms = 0.0
        for _ in range(K):   # the working set is about L2-sized: flush before every step
            flush()
            ch.timer_start()
            ch.step_async(n, dt)
            n += 1
            ms += ch.timer_stop()
        ms = D.max(ms)
        out[form] = dict(value=D.sum(g.points) * K / (ms / 1e3), unit=UNIT, ms_per_step=ms / K, steps=K,
                         kernels_per_step=ch.last_step_stats()[1])
        ch.close()
    ns = args.les_steps
    if ns > 0:
        runs = {f: make_channel(lib, g, f, U0, P0, HH0) for f in ("mixed", "fp64")}
        hist = {f: [] for f in runs}
        every = max(1, ns // 10)
        for s_ in range(1, ns + 1):
            for c in runs.values():
                c.step_async(s_, dt)
            if s_ % every == 0 or s_ == ns:
                for f, c in runs.items():
                    d = c.diagnose()
                    hist[f].append((s_, float(c.get_wsm()[0]), d["flow1"] / g.aly))
        Um, _, _ = runs["mixed"].download()
        Uf, _, _ = runs["fp64"].download()
        n1, n2, n3 = g.n1m, g.n2m, g.n3m

        def rl(a, b):
            return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        wm, wf = hist["mixed"][-1][1], hist["fp64"][-1][1]
        bm, bf = hist["mixed"][-1][2], hist["fp64"][-1][2]
        out["err_vs_fp64"] = dict(
            steps=ns, u=rl(Um[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0], Uf[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 0]),
            v=rl(Um[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1], Uf[1:n1 + 1, 2:n2 + 1, 1:n3 + 1, 1]),
            w=rl(Um[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2], Uf[1:n1 + 1, 1:n2 + 1, 1:n3 + 1, 2]),
            wall_stress_mixed=wm, wall_stress_fp64=wf, wall_stress_rel=abs(wm - wf) / abs(wf),
            bulk_mixed=bm, bulk_fp64=bf, bulk_rel=abs(bm - bf) / abs(bf),
            history=dict(step=[h[0] for h in hist["fp64"]],
                         wall_stress_mixed=[h[1] for h in hist["mixed"]],
                         wall_stress_fp64=[h[1] for h in hist["fp64"]]))
        for c in runs.values():
            c.close()
    return out


def run_operators(args, D: Dist):
    """The isolated operators on the field256 workload (256 x 193 x 256 points, seeded
    band-limited input): for each operator the FP64 and mixed time per application,
    algorithmic GB/s (operand read + result written; the Poisson solve also moves the
    half spectrum through its five passes) against the measured HBM peak, and the mixed
    result's relative L2 error against the FP64 result."""
    from compact3d_gb300 import lib
    g, _ = make_grid("field256")
    U, _P = ic.band_limited(g, seed=ic.SEED0 + 4000 + D.rank)
    F = np.asfortranarray(U[..., 0])
    peak, kind = peaks()
    N = g.points
    K = max(5, args.steps)
    chans = {f: lib.Channel(g, C3D_MIXED if f == "mixed" else C3D_FP64) for f in ("fp64", "mixed")}
    out = dict(workload=f"field256: {g.n1m}x{g.n2m + 1}x{g.n3m} points, band-limited |k| <= N/3 in x, z, "
                        f"smooth random y profile", peak_gbs=peak, peak_kind=kind, applications=K, ops={})
    flush = L2Flush(D.local)
    out["l2_policy"] = "L2 flushed (512 MB written) before every timed application; each timed alone"
    for name, op in lib.OPS.items():
        row = {}
        res = {}
        for form, ch in chans.items():
            R = 4 if form == "mixed" else 8
            ch.op_set(F)
            ch.op_apply(op, 3)
            ch.sync()
            ms = 0.0
            for _ in range(K):
                flush()
                ch.timer_start()
                ch.op_apply(op, 1)
                ms += ch.timer_stop()
            ms = D.max(ms) / K
            alg = N * (10 * R + 8) if name == "POISSON" else N * 2 * R
            gbs = alg / (ms / 1e3) / 1e9
            row[form] = dict(ms=ms, gbs=gbs, frac=gbs / peak, alg_bytes=alg)
            res[form] = ch.op_get()
        j0 = 2 if name == "DY1" else 1
        a = res["mixed"][1:g.n1m + 1, j0:g.n2m + 1, 1:g.n3m + 1]
        b = res["fp64"][1:g.n1m + 1, j0:g.n2m + 1, 1:g.n3m + 1]
        row["mixed_rel_l2_vs_fp64"] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        out["ops"][name] = row
    for c in chans.values():
        c.close()
    return out


def ensemble_grids(nchan: int, seed: int, precision: int):
    """The batched ensemble workload: grids drawn uniformly from Nx, Nz in {48,64,96,128}
    and Ny in {33,49,65,97} points, Re_bulk uniform in [3000, 12000] (RE = 3/4 Re_bulk),
    domain 4pi x 2 x 4/3 pi, tanh stretching beta = 2, dt = 0.002."""
    from compact3d_gb300.grid import Grid
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nchan):
        nx = int(rng.choice([48, 64, 96, 128]))
        nz = int(rng.choice([48, 64, 96, 128]))
        ny = int(rng.choice([33, 49, 65, 97]))
        reb = float(rng.uniform(3000.0, 12000.0))
        g = Grid(n1m=nx, n2m=ny - 1, n3m=nz, alx=4 * math.pi, aly=2.0, alz=4 * math.pi / 3, re=0.75 * reb,
                 cks=2.0, precision=precision)
        out.append(g)
    return out, 0.002


def run_batched(args, D: Dist):
    """Aggregate grid-point-substeps/s of the ensemble as one CUDA graph (mixed form), and
    of the same channels stepped one after another in the plain FP64 form."""
    from compact3d_gb300 import lib
    grids, dt = ensemble_grids(args.nchan, ic.SEED0 + 1000 + D.rank, C3D_MIXED)
    ics = [ic.perturbed_laminar(g, seed=ic.SEED0 + 2000 + i) for i, g in enumerate(grids)]
    pts = sum(g.points for g in grids)
    b = lib.Batch(grids)
    for ch, (U, P, HH) in zip(b.channels, ics):
        ch.upload(U, P, HH)
        ch.project()
        if not args.no_tune:
            ch.autotune()   # per grid shape, cached (the streams form runs the tuned schedules)
    n = len(grids)
    dts = [dt] * n
    K = args.steps
    tot = D.sum(pts)
    step = 1
    timed = {}
    for form in ("worklist", "streams"):
        b.set_form(form)
        p, p3 = [0.0] * n, [0.0] * n
        for _ in range(max(3, args.warmup)):
            p, p3 = b.step(step, dts, p, p3)
            step += 1
        D.barrier()
        t0 = time.perf_counter()
        dev_ms = 0.0
        for _ in range(K):
            p, p3 = b.step(step, dts, p, p3)
            step += 1
            dev_ms += b.last_step_stats()[0]
        wall = D.max(time.perf_counter() - t0)
        dev_ms = D.max(dev_ms)
        timed[form] = (dev_ms, wall, b.last_step_stats()[1])
    b.close()
    dev_ms, wall, launches = timed["worklist"]
    out = dict(value=tot * K / (dev_ms / 1e3), unit=UNIT, channels=n, points=pts, steps=K,
               ms_per_step=dev_ms / K, wall_value=tot * K / wall, kernels_per_step=launches,
               form="mixed, work-list form: one launch per pass and kernel group over all channels, "
                    "one CUDA graph per ensemble step",
               workload="32 channels: Nx,Nz in {48,64,96,128}, Ny in {33,49,65,97}, "
                        "Re_bulk in [3000,12000], seeded")
    sm, sw, sl = timed["streams"]
    out["streams_form"] = dict(value=tot * K / (sm / 1e3), ms_per_step=sm / K, kernels_per_step=sl,
                               form="each channel's own tuned step on its own stream, one CUDA graph")
    # the same channels, one after another: plain FP64, and the mixed form without the
    # graph (so that the batching gain and the precision gain can be told apart)
    for key, prec, k_seq in (("fp64_sequential", C3D_FP64, max(2, min(K, args.fp64_steps))),
                             ("mixed_sequential", C3D_MIXED, max(2, min(K, 20)))):
        t_seq = 0.0
        for i, g in enumerate(grids):
            c = lib.Channel(g, prec)
            U, P, HH = ics[i]
            c.upload(U, P, HH)
            c.project()
            if not args.no_tune:
                c.autotune()
            c.set_presg(0.0, 0.0)
            for s_ in range(1, 3):
                c.step_async(s_, dt)
            c.sync()
            c.timer_start()
            for s_ in range(k_seq):
                c.step_async(3 + s_, dt)
            t_seq += c.timer_stop()
            c.close()
        t_seq = D.max(t_seq)
        out[key] = dict(value=tot * k_seq / (t_seq / 1e3), ms_per_step=t_seq / k_seq, steps=k_seq)
    return out


def run_reference(args, D: Dist):
    """The reference arm: the reference's CPU path (see cpu_reference) on the host cores, on
    the same workload grid as the GPU arm, every step a full GETUP."""
    if D.rank != 0:
        return None
    K, W = args.steps, args.warmup
    rate, s_per_step, cores, kind, sample = cpu_reference(args.workload, steps=K, warmup=W)
    g, dt = make_grid(args.workload)
    res = dict(impl="reference", metric=METRIC, value=rate, unit=UNIT, n_gpus=D.world, steps=K,
               warmup=W, ms_per_step=s_per_step * 1e3, higher_is_better=True,
               scaling="weak", vs_baseline=None, dtype="f64", data="synthetic",
               config=workload_config(args, g, dt, "fp64-cpu"))
    res["cpu_baseline"] = dict(value=rate, unit=UNIT, cores=cores, kind=kind, sample=sample)
    res["e2e"] = dict(value=rate, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200 for the GPU arm, 20 for the CPU reference arm)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="channel384", choices=sorted(WORKLOADS))
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64", "mixed_ir"])
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--err-steps", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--e2e-windows", type=int, default=7, help="timed windows of --e2e-steps getups (median reported)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-floor", action="store_true")
    ap.add_argument("--no-les", action="store_true")
    ap.add_argument("--no-ops", action="store_true")
    ap.add_argument("--no-next", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--schedule", default="", help="JSON launch schedule for the main channel instead of autotuning")
    ap.add_argument("--les-steps", type=int, default=200)
    ap.add_argument("--nchan", type=int, default=32)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20 if args.impl == "reference" else 200
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    D = Dist()
    res = run_reference(args, D) if args.impl == "reference" else run_ours(args, D)
    if D.rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    D.close()


if __name__ == "__main__":
    main()
