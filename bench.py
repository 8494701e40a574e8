#!/usr/bin/env python3
"""Benchmark of the GB300 shot-profile migration: shot*omega*depth-steps per second.

Workload (default "survey64"): the 2-D PSPI survey -- velocity 500 x 1024 at 10 m
(seeded Gaussian random field), 64 shots with receiver apertures of 200..800
traces, nt=1500 at 2 ms, 5-50 Hz (271 frequencies), 8 reference velocities,
padx=padt=2 (2048-point rows). One step = one migration of the whole survey
(8,672,000 units: 64 shots x 271 frequencies x 500 depth steps).

  value  units/s with the traces already in device memory (wem_migrate_device),
         CUDA events on the library's stream around exactly K steps;
  e2e    the same through the public C ABI with host buffers (wem_migrate): the
         H2D copy of the traces, all kernels and the D2H copy of the image;
  roofline  the depth-recursion kernel: algorithmic FLOPs per unit x units / its
         event-timed duration;
  cpu_baseline  the reference's CPU algorithm on this machine's host cores on a
         bounded sample (one shot of the survey, all its frequencies).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--workload split1]
Under torchrun each rank migrates its own copy of the survey (weak scaling); no
collective is on the data path.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "seismic.jl_gb300"))

import numpy as np  # noqa: E402


def survey(workload: str, rank: int, born: str = "gpu"):
    """The workload's synthetic survey. The 2-D PSPI surveys carry Born data of a seeded 1 %
    random reflectivity: born="gpu" models every shot with the library's reference forward
    operator; born="cpu" (the reference arm) models only the shot its CPU sample migrates,
    with the oracle's port of the reference's forward operator on the host cores."""
    from wemgpu import synth
    if workload == "survey64":
        c = synth.config1(seed=1001 + rank)
        wl = ("2-D PSPI survey: 64 shots, 500x1024 grid @10 m, nref=8, 5-50 Hz, nt=1500, padx=padt=2, "
              "Born data of a 1% random reflectivity")
    elif workload == "survey8":
        c = synth.config1(seed=1001 + rank, nshot=8)
        wl = ("2-D PSPI survey subset for profiling: 8 shots, 500x1024 grid @10 m, nref=8, 5-50 Hz, nt=1500, "
              "Born data")
    elif workload == "survey3d":
        c = synth.config3(seed=1003 + rank)
        wl = "3-D PSPI: 1 shot, 300x256x256 grid @12.5 m, nref=6, 3-60 Hz, nt=2000, padx=padt=2 (512x512 planes)"
    elif workload == "survey3d_band":
        c = synth.config3(seed=1003 + rank)
        c["params"] = dict(c["params"], fmax=float(c["params"]["fmin"]) + 12.0)
        wl = ("3-D PSPI for profiling: 1 shot, 300x256x256 grid @12.5 m, nref=6, 3-15 Hz, nt=2000, padx=padt=2 "
              "(512x512 planes)")
    elif workload == "lsm32":
        c = synth.config4(seed=1004 + rank)
        c["params"] = dict(c["params"], interp="linear")
        wl = ("2-D least-squares PSPI migration: 32 shots, 300x512 grid @10 m, nref=8, 5-45 Hz, nt=1500, "
              "20 CG iterations over the exact modelling/migration pair")
    elif workload == "angles8":
        c = synth.config1(seed=1001 + rank, nshot=8)
        wl = ("2-D source incidence angles (compute_angles): 8 shots, 500x1024 grid @10 m, 5-50 Hz of the "
              "unpadded 1500-sample axis")
    elif workload == "split1":
        c = synth.config0(seed=1000 + rank)
        wl = "2-D split-step: 1 shot, 200x256 grid @10 m, 3 layers, 5-60 Hz, nt=1000, padx=padt=2"
    elif workload == "elastic8":
        c = synth.config4(seed=1004 + rank, nshot=8)
        c["params"] = dict(c["params"], fmax=30.0)
        wl = ("2-D elastic migration (ewem): 8 shots, 300x512 grid @10 m, vs = vp/1.8 with a 5% seeded wobble, "
              "5-30 Hz, nt=1500, padx=padt=2, x and z components on every cell")
    elif workload == "elastic3d":
        c = synth.small_case3d(1006 + rank, nx=128, ny=128, nz=60, nt=500, nshot=2, pspi=0, fmax=25.0, padx=2)
        c["params"] = dict(c["params"], fmin=5.0)
        wl = ("3-D elastic migration (ewem, nmy > 1): 2 shots, 60x128x128 grid @10 m, vs = vp/1.8 with a 5% "
              "seeded wobble, 5-25 Hz, nt=500, padx=padt=2 (256x256 planes), x and z components on every cell")
    else:
        raise SystemExit(f"unknown workload {workload}")
    if workload in ("survey64", "survey8", "angles8"):
        c = born_data_port_shot(c) if born == "cpu" else synth.with_born_data(c)
    return c, wl


def cpu_sample_shots(nshot: int, k: int = 4) -> list[int]:
    """The shots the CPU legs time: k evenly spaced ones."""
    k = min(k, nshot)
    return [int((2 * i + 1) * nshot // (2 * k)) for i in range(k)]


def born_data_port_shot(c: dict) -> dict:
    """The CPU sample's shots (cpu_sample_shots) with Born data of the same seeded
    reflectivity as synth.with_born_data, modelled by the oracle's port of the reference's
    forward operator (wem.c:252-281) on the host cores; the other shots keep their traces."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from wemgpu import Shots, synth
    O.build()
    p, shots = c["params"], c["shots"]
    nmx, nz = int(p["nmx"]), int(p["nz"])
    m = synth.random_reflectivity(nmx * 7919 + nz, nmx, nz)
    data = shots.data.copy()
    for s in cpu_sample_shots(shots.nshot):
        full = O.wem_port(dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s])), c["vel"], c["wav"], m=m, adj=False,
                          nthreads=os.cpu_count() or 1)
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        data[lo:hi] = full[shots.trace_cell[lo:hi]]
    out = dict(c)
    out["shots"] = Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell, data)
    return out


def band(p: dict):
    """Number of frequencies the reference processes (wem.c:79-89, float arithmetic)."""
    f32 = np.float32
    nt, padt, dt = int(p["nt"]), int(p["padt"]), f32(p["dt"])
    ntfft = int(f32(2 * padt) * f32(nt) / f32(2))
    nw = ntfft // 2 + 1
    fmax, fmin = f32(p["fmax"]), f32(p["fmin"])
    ifmax = int(f32(int(fmax)) * dt * f32(ntfft) + f32(1)) if fmax * dt * f32(ntfft) + f32(1) < nw else nw
    ifmin = int(f32(int(fmin)) * dt * f32(ntfft)) if fmin * dt * f32(ntfft) + f32(1) < ifmax else 0
    return ifmax - ifmin


def band_elastic(p: dict):
    """Frequencies of the reference's elastic migration (ewem.c:44-57: ntfft = 2 truncf(padt nt/2),
    ifmax = trunc(fmax dt ntfft) + 1, float products)."""
    f32 = np.float32
    nt, padt, dt = int(p["nt"]), int(p["padt"]), f32(p["dt"])
    ntfft = 2 * int(math.trunc(float(f32(f32(padt) * f32(nt)) / f32(2))))
    nw = ntfft // 2 + 1
    prod = f32(f32(p["fmax"]) * dt * f32(ntfft))
    ifmax = int(math.trunc(float(prod))) + 1 if prod + f32(1) < nw else nw
    prodn = f32(f32(p["fmin"]) * dt * f32(ntfft))
    ifmin = int(math.trunc(float(prodn))) if prodn + f32(1) < ifmax else 0
    return ifmax - ifmin


def flops_per_unit(p: dict) -> float:
    """Algorithmic FLOPs of one (shot, frequency, depth step): source and receiver
    continuation plus the imaging condition, 5 N log2 N per complex FFT, with
    N = nkx (2-D) or nkx*nky (3-D) and n = nmx*nmy.
    PSPI:  per wavefield 5N log2N + R (6N + 5N log2N) + 8n;  unit = 2 F + 3n.
    Split-step: per wavefield 2 * 5N log2N + 6N + 14n;     unit = 2 F + 3n."""
    nmy = int(p.get("nmy", 1))
    n = int(p["nmx"]) * nmy
    N = int(p["padx"]) * int(p["nmx"]) * (int(p["padx"]) * nmy if nmy > 1 else 1)
    lg = math.log2(N)
    if int(p.get("pspi", 1)):
        R = int(p["nref"])
        F = 5 * N * lg + R * (6 * N + 5 * N * lg) + 8 * n
    else:
        F = 2 * 5 * N * lg + 6 * N + 14 * n
    return 2 * F + 3 * n


def inverse_transforms_per_step(p: dict, vel: np.ndarray, paired: bool, direct_sums: bool = True) -> float:
    """Mean inverse transforms per wavefield step of the 2-D PSPI depth kernel over the
    depth steps: one per reference some point takes its wavefield from; in the paired
    form of the nearest-lower mode (interp=ref) one per two references whose every taker
    keeps the real part only, and one per reference taken whole somewhere. The selection
    restates the float arithmetic of wem.c:40-70."""
    f32 = np.float32
    nref, nmx = int(p["nref"]), int(p["nmx"])
    vel = np.asarray(vel, f32).reshape(-1, int(p["nz"]))
    total = 0
    for iz in range(vel.shape[1]):
        v = vel[:, iz]
        vmin = f32(v[:nmx].min())
        vmax = f32(max(v[nmx - 1], v.max()))
        ir = np.arange(nref, dtype=f32)
        vref = vmin + ir * (vmax - vmin) / (f32(nref) - f32(1))
        if vmax > vmin + f32(10):
            i = np.maximum(((f32(nref - 1) * (v - vmin)) / (vmax - vmin)).astype(np.int64), 0)  # 3-D: v < vmin
            i1 = np.where(i > nref - 2, nref - 1, i)
            i2 = np.where(i > nref - 2, nref - 1, i + 1)
        else:
            i1 = i2 = np.zeros(v.shape, np.int64)
        interp = (vref[i2] - vref[i1]).astype(np.float64) > 10.0
        used = set(i1.tolist())
        if p.get("interp", "ref") == "linear":
            used |= set((i1[interp] + 1).tolist())
            total += len(used)
            continue
        if not paired:
            total += len(used)
            continue
        if direct_sums and 1 <= np.count_nonzero(~interp) <= 4:  # whole points by direct sums, every reference paired
            total += (len(used) + 1) // 2
            continue
        whole = set(i1[~interp].tolist())
        ro = len(used - whole)
        total += len(whole) + ro // 2 + ro % 2
    return total / vel.shape[1]


def tensor_flops_per_unit(p: dict) -> float:
    """Tensor-core FLOPs one (shot, frequency, depth step) executes in split16 mode: every
    radix-16 pass of a 2048-sample row is M=128 x N=32 x K=32 per product and the radix-8
    pass two M=128 x N=16 x K=16 products, with 3 products (hi*hi, lo*hi, hi*lo) each;
    (1 + R) transforms per wavefield (PSPI) or 2 (split-step), 2 wavefields."""
    per_fft = 3 * (2 * (2 * 128 * 32 * 32) + 2 * (2 * 128 * 16 * 16))
    nfft = 1 + int(p["nref"]) if int(p.get("pspi", 1)) else 2
    return 2.0 * nfft * per_fft


def accuracy(c: dict, ctx_factory, nsample: int = 4) -> dict:
    """Relative L2 image error of `nsample` evenly spaced shots of the survey, stacked, over
    the full band and every depth step, against the oracle's FP64 operator, for FP32 and
    split16 (the contract's 1e-4 bar); beside them the reference's own FP32 arithmetic (the
    port, bit-identical to the compiled reference) against the same FP64 image -- the floor."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from wemgpu import synth
    from wemgpu.api import Shots
    O.build()
    p = dict(c["params"])
    shots = c["shots"]
    which = cpu_sample_shots(shots.nshot, nsample)
    offs, cells, data = [0], [], []
    for s in which:
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        cells.append(shots.trace_cell[lo:hi])
        data.append(shots.data[lo:hi])
        offs.append(offs[-1] + hi - lo)
    sub = Shots(shots.sx[which], shots.sy[which], np.asarray(offs, np.int64), np.concatenate(cells),
                np.concatenate(data))
    q = {k_: v for k_, v in p.items() if k_ != "precision"}
    ncell = int(p["nmx"]) * int(p.get("nmy", 1))
    cores = os.cpu_count() or 1
    want = ref32 = None
    t0 = time.perf_counter()
    for s in which:
        d = synth.shot_gather_full(shots, s, ncell)
        qs = dict(q, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        w = O.wem_fp64(qs, c["vel"], c["wav"], d=d, adj=True, nthreads=cores).astype(np.float64)
        r = O.wem_port(qs, c["vel"], c["wav"], d=d, adj=True, nthreads=cores).astype(np.float64)
        want = w if want is None else want + w
        ref32 = r if ref32 is None else ref32 + r
    el = time.perf_counter() - t0
    nw = np.linalg.norm(want)
    out = {"sample": f"shots {which} stacked, {band(p)} frequencies ({p['fmin']:g}-{p['fmax']:g} Hz) x "
                     f"{p['nz']} depth steps (the oracle took {el:.0f} s on {cores} cores)",
           "oracle": "FP64 restatement of wem.c",
           "rel_l2_reference_fp32": float(np.linalg.norm(ref32 - want) / nw)}
    for prec in ("fp32", "split16"):
        ctx = ctx_factory()
        try:
            m = ctx.prepare(dict(q, precision=prec), c["vel"], c["wav"]).migrate(sub)
        except Exception as e:  # split16 is built for 2048-point rows only
            out[f"rel_l2_{prec}"] = f"not run: {e}"
            continue
        finally:
            ctx.close()
        out[f"rel_l2_{prec}"] = float(np.linalg.norm(m - want) / nw)
        out[f"rel_l2_{prec}_vs_reference_fp32"] = float(np.linalg.norm(m - ref32) / np.linalg.norm(ref32))
    return out


def bytes_per_unit_3d(p: dict, planes: float | None = None) -> float:
    """Device-memory bytes of one 3-D (shot, frequency, depth step) in the three-pass
    design (the padded x-y plane does not fit in shared memory): with n = nmx*nmy,
    M = nmx*nky rows kept after the y transform and R planes per wavefield (one per
    reference, or fewer with paired planes), both wavefields: pass A reads U (2n) and
    writes Y (2M); pass B reads Y (2M) and writes C (2RM); pass C reads C (2RM) and
    writes U (2n); 8 bytes per complex sample."""
    nmy = int(p["nmy"])
    n = int(p["nmx"]) * nmy
    M = int(p["nmx"]) * int(p["padx"]) * nmy
    R = planes if planes is not None else (int(p["nref"]) if int(p.get("pspi", 1)) else 1)
    return 8.0 * (4 * n + 4 * M + 4 * R * M)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.first = ""

    def start(self):
        """Starts the sampler and waits (at most 2 s) for its first sample, so that a timed
        region shorter than the 200 ms period still has the sample taken as it begins."""
        import select
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            ready, _, _ = select.select([self.proc.stdout], [], [], 2.0)
            if ready:
                self.first = self.proc.stdout.readline()
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        out = self.first + (out or "")
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


KERNEL_SOURCES = ("wem_fft.cuh", "wem_step.cuh", "wem_kernels.cuh", "wem_kernels.cu", "wem_tc.cuh", "wem_3d.cu",
                  "wem_internal.h")


ELASTIC_SOURCES = KERNEL_SOURCES + ("wem_elastic.cuh", "wem_elastic.cu")
TRAFFIC_SOURCES = {"elastic8": ELASTIC_SOURCES}  # workloads whose kernels have sources of their own


def kernel_source_sha(names=KERNEL_SOURCES) -> str:
    """sha256 (first 16 hex digits) of the device-code sources the depth kernels are built from."""
    import hashlib
    h = hashlib.sha256()
    for name in names:
        with open(os.path.join(ROOT, "seismic.jl_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def recorded_traffic(workload: str):
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the depth
    kernel for a workload, from the committed ncu summary (profiles/dram_traffic.json).
    A record whose kernel-source hash differs from the current kernel sources is returned
    with "stale": True (its bytes describe an older kernel)."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            rec = json.load(f).get(workload)
    except Exception:
        return None
    if rec is None:
        return None
    rec = dict(rec)
    rec["stale"] = rec.get("kernel_source_sha") != kernel_source_sha(TRAFFIC_SOURCES.get(workload, KERNEL_SOURCES))
    return rec


_FP32_PEAK = {}


def fp32_peak(device: int):
    """FP32 FMA throughput measured on this GPU in this run (wem_measure_fp32_peak)."""
    if device not in _FP32_PEAK:
        from wemgpu._lib import measure_fp32_peak
        _FP32_PEAK[device] = measure_fp32_peak(device)
    return _FP32_PEAK[device]


def executed_flops_per_unit(p: dict, vel, paired: bool) -> tuple[float, float, float]:
    """FLOPs one (shot, frequency, depth step) executes in the 2-D PSPI depth kernel (as
    opposed to the algorithmic count of flops_per_unit): the forward transform, the inverse
    transforms actually run (references no point uses skipped; two real parts per transform
    in the paired form), a phase multiply per used reference and the selection; both
    wavefields plus the imaging. Returns (flops, inverse transforms, used references)."""
    nmx = int(p["nmx"])
    N = int(p["padx"]) * nmx
    lg = math.log2(N)
    x = inverse_transforms_per_step(p, vel, paired)
    r_used = inverse_transforms_per_step(p, vel, False)
    F = 5 * N * lg * (1 + x) + 6 * N * r_used + 8 * nmx
    return 2 * F + 3 * nmx, x, r_used


def accuracy_sample(c: dict, kept: dict, ctx_factory) -> dict:
    """Relative L2 image error of the GPU migration against the CPU leg's own image (the
    reference's FP32 arithmetic, the port bit-identical to the compiled reference) on the
    CPU leg's shots and band: for the 3-D survey, whose FP64 oracle would take minutes more."""
    from wemgpu.api import Shots
    shots, which = c["shots"], kept["which"]
    offs, cells, data = [0], [], []
    for s in which:
        lo, hi = int(shots.trace_offset[s]), int(shots.trace_offset[s + 1])
        cells.append(shots.trace_cell[lo:hi])
        data.append(shots.data[lo:hi])
        offs.append(offs[-1] + hi - lo)
    sub = Shots(shots.sx[which], shots.sy[which], np.asarray(offs, np.int64), np.concatenate(cells),
                np.concatenate(data))
    q = {k_: v for k_, v in kept["params"].items() if k_ != "precision"}
    ctx = ctx_factory()
    try:
        m = ctx.prepare(q, c["vel"], c["wav"]).migrate(sub).astype(np.float64)
    finally:
        ctx.close()
    ref = kept["image"]
    return {"sample": f"the CPU leg's shots {which}, {band(q)} frequencies ({q['fmin']:g}-{q['fmax']:g} Hz) x "
                      f"{q['nz']} depth steps",
            "oracle": "the port of the reference's C (its FP32 arithmetic)",
            "rel_l2_fp32_vs_reference_fp32": float(np.linalg.norm(m - ref) / np.linalg.norm(ref))}


def cpu_baseline(c, nsample: int = 4, which=None, keep=None):
    """The reference's CPU algorithm on `nsample` evenly spaced shots of the survey (every
    frequency; about 20-25 s on the GPU host's cores), all host cores, one shot at a time as
    the Julia wrapper calls it. oracle/_ref (the reference's own C core) when it was built
    on this machine, else the oracle port of it. `which` picks the shots instead. `keep`, a
    dict, receives the stacked CPU image, the parameters and the shots it was made with."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from wemgpu import synth
    O.build()
    p = dict(c["params"])
    shots = c["shots"]
    if which is None:
        which = cpu_sample_shots(shots.nshot, nsample)
    cores = os.cpu_count() or 1
    kind = "reference" if O.ref_available() else "port"
    nf_all = band(p)
    if int(p.get("nmy", 1)) > 1:
        # a 3-D depth step costs ~1000x a 2-D one: the sample is the lowest 17 frequencies
        # (the band edge is (int)fmax, wem.c:86), about one per host core
        p["fmax"] = float(p["fmin"]) + 2.0
    dt = 0.0
    img = None
    for s in which:
        q = dict(p, sx=float(shots.sx[s]), sy=float(shots.sy[s]))
        d = synth.shot_gather_full(shots, s, int(p["nmx"]) * int(p.get("nmy", 1)))
        t0 = time.perf_counter()
        if kind == "reference":
            m = O.wem_ref(q, c["vel"], c["wav"], d=d, adj=True)
            cores = O.omp_threads()
        else:
            m = O.wem_port(q, c["vel"], c["wav"], d=d, adj=True, nthreads=cores)
        dt += time.perf_counter() - t0
        if keep is not None:
            img = np.asarray(m, np.float64) if img is None else img + m
    if keep is not None:
        keep.update(image=img, params=p, which=list(which))
    units = len(which) * band(p) * int(p["nz"])
    return {"value": units / dt, "unit": "shot*omega*depth-steps/s", "cores": cores, "kind": kind,
            "sample": f"shots {which} of {shots.nshot}, {band(p)} of {nf_all} frequencies x {p['nz']} depth steps "
                      f"({units} units) in {dt:.1f} s"}


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    c, wl = survey(args.workload, 0, born="cpu")
    p = c["params"]
    nf = band(p)
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        # one shot per step, cycling over the CPU sample's shots (their apertures differ)
        sample = cpu_sample_shots(c["shots"].nshot)
        info = cpu_baseline(c, which=[sample[i % len(sample)]])
        if i >= args.warmup:
            vals.append(info["value"])
    v = statistics.mean(vals)
    info["value"] = v
    line = {"impl": "reference", "metric": "shot*omega*depth-steps/s", "value": v, "unit": "shot*omega*depth-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * (nf * int(p["nz"])) / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": wl, "step": "one shot of the survey on the host cores, cycling over 4 evenly "
                                                "spaced shots"},
            "cpu_baseline": info,
            "e2e": {"value": v, "unit": "shot*omega*depth-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_elastic(args, c, wl, rank, world, local):
    """Elastic migration of every shot (wem_elastic; the reference's ewem, src/Imaging/c/ewem.c).
    A unit is one shot * frequency * depth step (the source step and the receiver's
    separation, two potential continuations and recombination). One step = all shots."""
    import torch
    import wemgpu
    from wemgpu import synth
    p, shots = c["params"], c["shots"]
    nmx, nmy, nz, nt = int(p["nmx"]), int(p.get("nmy", 1)), int(p["nz"]), int(p["nt"])
    ncell = nmx * nmy
    rng = np.random.default_rng(2005 + rank)
    vp = c["vel"]
    vs = (vp / 1.8 * (1.0 + 0.05 * rng.standard_normal(vp.shape))).astype(np.float32)
    uz = np.stack([synth.shot_gather_full(shots, s, ncell) for s in range(shots.nshot)])
    ux = (0.5 * np.roll(uz, 3, axis=2)).astype(np.float32)
    sx = np.asarray(shots.sx, np.float32)
    sy = np.asarray(shots.sy, np.float32)
    nf = band_elastic(p)
    units = len(sx) * nf * nz
    for _ in range(args.warmup):
        wemgpu.elastic(p, vp, vs, c["wav"], sx, sy, ux=ux, uz=uz, adj=True, device=local)
    sampler = ClockSampler(local)
    torch.cuda.synchronize()
    sampler.start()
    dev_ms, wall = [], []
    L = wemgpu.lib()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        wemgpu.elastic(p, vp, vs, c["wav"], sx, sy, ux=ux, uz=uz, adj=True, device=local)
        wall.append(time.perf_counter() - t0)
        dev_ms.append(float(L.wem_elastic_last_ms()))
    clocks = sampler.stop()
    ms = statistics.mean(dev_ms)
    nkx = int(p["padx"]) * nmx
    npl = nkx * (int(p["padx"]) * nmy if nmy > 1 else 1)  # samples of a padded row (2-D) or plane (3-D)
    lg = math.log2(npl)
    # algorithmic FLOPs per unit: the source step (2 transforms) and the receiver's separation,
    # two continuations and recombination (10 transforms), 5 N log2 N each, plus ~60 per sample
    fl = 12 * 5 * npl * lg + 60 * npl
    ach = units * fl / (ms / 1000.0) / 1e12
    fp32_meas = fp32_peak(local)
    tr = recorded_traffic("elastic8") if args.fmax is None and nmy == 1 else None
    traffic = tr.get("bytes_per_launch") if tr and not tr["stale"] else None
    if nmy > 1:
        # per depth step: 3 spectra once, then 6 plane passes (3 row, 3 column) per step and 2 reductions
        launches = 3 + 6 * nz + 2 + 2
        kern = "3-D plane passes (wem_e3_rows_kernel, wem_e3_cols_kernel) + spectra + reductions, whole step"
    else:
        # 3 spectra (wavelet, x, z), the tables, the depth kernel, 2 image reductions
        launches = 7
        kern = "wem_ewem_kernel + tables + spectra + reductions, whole step"
    line = {"metric": "shot*omega*depth-steps/s", "value": world * units / (ms / 1000.0),
            "unit": "shot*omega*depth-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "gpu_launches": args.steps * launches,
            "config": {"workload": wl, "units_per_step_per_gpu": units, "shots": len(sx), "frequencies": nf,
                       "depth_steps": nz, "nkx": nkx, "plane": npl, "l2": "inputs larger than L2"},
            "e2e": {"value": world * units / statistics.mean(wall), "unit": "shot*omega*depth-steps/s",
                    "h2d_bytes_per_step": int(ux.nbytes + uz.nbytes), "d2h_bytes_per_step": int(2 * ncell * nz * 4)},
            "roofline": {"bound": "fp32", "achieved": ach, "peak": fp32_meas, "unit": "TFLOP/s",
                         "frac": ach / fp32_meas, "traffic": traffic,
                         "peak_source": "FP32 FMA probe (wem_measure_fp32_peak), measured in this run",
                         "kernel": kern, "ms_per_launch": ms,
                         "flops_per_unit": fl, "traffic_kernel": "wem_ewem_kernel (DRAM bytes of one launch)"},
            "clocks": clocks}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU leg: the oracle's FP64 restatement (NumPy, one thread) on one shot, 2 Hz of the band
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import ewem_np as E
        q = dict(p, sx=float(sx[len(sx) // 2]), sy=float(sy[len(sx) // 2]), fmax=float(p["fmin"]) + 2.0)
        nq = band_elastic(q)
        s0 = len(sx) // 2
        t0 = time.perf_counter()
        want = (E.ewem3d if nmy > 1 else E.ewem)(q, vp, vs, c["wav"], ux=ux[s0], uz=uz[s0], adj=True)
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nq * nz / el, "unit": "shot*omega*depth-steps/s", "cores": 1, "kind": "port",
                                "sample": f"1 shot, {nq} frequencies x {nz} depth steps in {el:.1f} s "
                                          "(NumPy FP64 restatement, one thread)"}
        got = wemgpu.elastic(q, vp, vs, c["wav"], [q["sx"]], [q["sy"]], ux=ux[s0:s0 + 1], uz=uz[s0:s0 + 1], adj=True,
                             device=local)
        line["accuracy"] = {"rel_l2_p_vs_fp64": float(np.linalg.norm(got[0] - want[0]) / np.linalg.norm(want[0])),
                            "rel_l2_s_vs_fp64": float(np.linalg.norm(got[1] - want[2]) / np.linalg.norm(want[2])),
                            "sample": "the CPU leg's shot and band"}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_angles(args, c, wl, rank, world, local):
    """Source-side incidence angles of every shot (wem_angles; the reference's
    compute_angles, wem.c:566-992). A unit is one shot * frequency * depth step of the
    angle computation (frequencies of the unpadded time axis). One step = all shots."""
    import torch
    import wemgpu
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    p, shots = c["params"], c["shots"]
    ctx = wemgpu.Context(local)
    sx = np.asarray(shots.sx, np.float32)
    nt, dt = int(p["nt"]), float(p["dt"])
    nf = band(dict(p, padt=1))
    units = len(sx) * nf * int(p["nz"])
    for _ in range(args.warmup):
        ctx.angles(p, c["vel"], c["wav"], sx)
    sampler = ClockSampler(local)
    torch.cuda.synchronize()
    sampler.start()
    dev_ms, wall = [], []
    launches = 0  # this library's kernels
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ax, ay = ctx.angles(p, c["vel"], c["wav"], sx)
        wall.append(time.perf_counter() - t0)
        ms_k, nk = ctx.last_timing()
        dev_ms.append(ms_k)
        launches += nk
    clocks = sampler.stop()
    ms = statistics.mean(dev_ms)
    line = {"metric": "shot*omega*depth-steps/s", "value": world * units / (ms / 1000.0),
            "unit": "shot*omega*depth-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "gpu_launches": launches,
            "config": {"workload": wl, "units_per_step_per_gpu": units, "shots": len(sx), "frequencies": nf,
                       "depth_steps": int(p["nz"]), "l2": "inputs larger than L2 (wavefields of every frequency)"},
            "e2e": {"value": world * units / statistics.mean(wall), "unit": "shot*omega*depth-steps/s",
                    "h2d_bytes_per_step": int(c["vel"].nbytes + c["wav"].nbytes),
                    "d2h_bytes_per_step": int(ax.nbytes + ay.nbytes)},
            "clocks": clocks}
    # roofline of the whole angle step on the CUDA cores: the reference's algorithmic FLOPs
    # per unit (one shot, frequency and depth row): the split-step source step (two row
    # transforms, ~20 per sample) and its share of the derivatives -- one forward and four
    # inverse transforms of the nmx x nz volume per frequency (wem.c:829-992), 5 N log2 N each
    nmx_a, nz_a = int(p["nmx"]), int(p["nz"])
    fl = 10 * nmx_a * math.log2(nmx_a) + 20 * nmx_a + 25 * nmx_a * math.log2(nmx_a * nz_a)
    ach = units * fl / (ms / 1000.0) / 1e12
    fp32_meas = fp32_peak(local)
    tr = recorded_traffic("elastic8") if args.fmax is None else None
    traffic = tr.get("bytes_per_launch") if tr and not tr["stale"] else None
    line["roofline"] = {"bound": "fp32", "achieved": ach, "peak": fp32_meas, "unit": "TFLOP/s",
                        "frac": ach / fp32_meas, "traffic": None,
                        "peak_source": "FP32 FMA probe (wem_measure_fp32_peak), measured in this run",
                        "kernel": "wem_angles_* kernels (extrapolation, derivative convolutions, accumulation), whole step",
                        "ms_per_launch": ms, "flops_per_unit": fl}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU leg: the oracle's FP64 restatement of compute_angles on one shot, 2 Hz of the band
        import angles_np as A
        q = dict(p, sx=float(sx[len(sx) // 2]), fmax=float(p["fmin"]) + 2.0)
        nq = band(dict(q, padt=1))
        t0 = time.perf_counter()
        want, _ = A.compute_angles(q, c["vel"], c["wav"])
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nq * int(p["nz"]) / el, "unit": "shot*omega*depth-steps/s", "cores": 1,
                                "kind": "port", "sample": f"1 shot, {nq} frequencies x {p['nz']} depth steps in {el:.1f} s "
                                                          "(NumPy FP64 restatement, one thread)"}
        got, _ = ctx.angles(q, c["vel"], c["wav"], [q["sx"]])
        g0 = got[0].astype(np.float64)
        live = np.abs(want) > 1e-3
        # the sign (side of arrival) is ill-conditioned where the two sides carry equal energy;
        # the reference's own FP32 result flips a few such points against FP64 too
        line["accuracy"] = {"rel_l2_vs_fp64": float(np.linalg.norm(g0 - want) / np.linalg.norm(want)),
                            "rel_l2_of_magnitude_vs_fp64": float(np.linalg.norm(np.abs(g0) - np.abs(want))
                                                                 / np.linalg.norm(want)),
                            "sign_flips": int(np.count_nonzero(np.sign(g0[live]) != np.sign(want[live]))),
                            "points": int(live.sum()), "sample": "the CPU leg's shot and band"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    return 0


def run_lsm(args, ctx, c, wl, units, dev, rank, world, dist):
    """The least-squares workload: Born data of a seeded reflectivity (1 % of the cells, N(0,1)), then CG
    (Scales 1987) from zero over wem_model(exact) / wem_migrate. One step = one CG solve."""
    import torch
    from wemgpu import Shots
    from wemgpu.cg import conjugate_gradients, dot_test, least_squares_migration
    p, shots = c["params"], c["shots"]
    rng = np.random.default_rng(2004)
    m_true = np.zeros((int(p["nmx"]), int(p["nz"])), np.float32)
    k = m_true.size // 100
    m_true.flat[rng.choice(m_true.size, k, replace=False)] = rng.standard_normal(k).astype(np.float32)
    d_obs = ctx.model(shots, m_true, exact=True)
    geo = lambda d: Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell, np.ascontiguousarray(d, np.float32))
    fwd = lambda m: ctx.model(shots, np.asarray(m, np.float32), exact=True)
    adj = lambda r: ctx.migrate(geo(r))
    a, b = dot_test(fwd, adj, rng.standard_normal(m_true.shape).astype(np.float32),
                    rng.standard_normal(d_obs.shape).astype(np.float32))
    # value: CG with the data, residual and image vectors resident in device memory
    # (wem_model_device / wem_migrate_device on torch tensors, float64 inner products on the
    # device); e2e: the same CG through the host-buffer calls (wem_model / wem_migrate)
    ntr, nt = d_obs.shape
    nm = m_true.shape
    cur = torch.cuda.current_stream(dev)

    launches = [0]

    def fwd_dev(m_t):
        d_t = torch.empty((ntr, nt), dtype=torch.float32, device=dev)
        cur.synchronize()  # the library runs on its own stream
        ctx.model_device(shots, m_t.data_ptr(), d_t.data_ptr(), exact=True)
        launches[0] += ctx.last_timing()[1]
        return d_t

    def adj_dev(r_t):
        m_t = torch.empty(nm, dtype=torch.float32, device=dev)
        cur.synchronize()
        ctx.migrate_device(shots, r_t.data_ptr(), m_t.data_ptr())
        launches[0] += ctx.last_timing()[1]
        return m_t

    inner_dev = lambda x, y: float(torch.dot(x.reshape(-1).double(), y.reshape(-1).double()))
    d_obs_t = torch.from_numpy(d_obs).to(dev)
    for _ in range(args.warmup):
        conjugate_gradients(d_obs_t, fwd_dev, adj_dev, niter=2, inner_fn=inner_dev)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.synchronize()
    sampler.start()
    t0 = time.perf_counter()
    costs = None
    launches[0] = 0
    for _ in range(args.steps):
        m_est_t, costs = conjugate_gradients(d_obs_t, fwd_dev, adj_dev, niter=20, inner_fn=inner_dev)
    torch.cuda.synchronize()
    el = (time.perf_counter() - t0) / args.steps
    clocks = sampler.stop()
    m_est = m_est_t.cpu().numpy()
    # e2e: the host-buffer least-squares call (traces in from pinned host memory once, the
    # image out once), after one untimed call
    obs = geo(d_obs)
    least_squares_migration(ctx, obs, niter=2)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    m_e2e, costs_e2e = least_squares_migration(ctx, obs, niter=20)
    el_e2e = time.perf_counter() - t1
    # and CG over the per-application host-buffer calls (wem_model / wem_migrate), every
    # operator application copying its input in and its output out
    conjugate_gradients(d_obs, fwd, adj, niter=2)
    t1 = time.perf_counter()
    _, costs_host = conjugate_gradients(d_obs, fwd, adj, niter=20)
    el_host = time.perf_counter() - t1
    napply = 2 * 20 + 1
    err = float(np.linalg.norm(m_est - m_true) / np.linalg.norm(m_true))
    line = {"metric": "shot*omega*depth-steps/s", "value": world * napply * units / el, "unit": "shot*omega*depth-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": wl, "units_per_operator": units, "operator_applications_per_step": napply,
                       "l2": "inputs larger than L2",
                       "cg": "vectors in device memory (value); e2e: least_squares_migration on host traces"},
            "e2e": {"value": world * napply * units / el_e2e, "unit": "shot*omega*depth-steps/s",
                    "h2d_bytes_per_step": int(d_obs.nbytes), "d2h_bytes_per_step": int(m_e2e.nbytes)},
            "gpu_launches": launches[0],
            "host_operator_calls": {"value": world * napply * units / el_host, "unit": "shot*omega*depth-steps/s",
                                    "h2d_bytes_per_step": int(napply * (shots.data.nbytes + m_true.nbytes) // 2),
                                    "d2h_bytes_per_step": int(napply * (shots.data.nbytes + m_true.nbytes) // 2)},
            "cg": {"misfit": [float(x) for x in costs], "misfit_e2e": [float(x) for x in costs_e2e],
                   "misfit_host_buffers": [float(x) for x in costs_host],
                   "dot_test": [a, b], "dot_rel": abs(a - b) / abs(a), "model_rel_err": err},
            "clocks": clocks}
    # roofline of the operator pair: the algorithmic FP32 work of every application (the
    # migration's count per unit; the exact modelling does the same transforms) over the
    # device-resident solve's time, against the contract's bf16 peak and the nominal FP32 peak
    fl = flops_per_unit(p)
    ach = napply * units * fl / el / 1e12
    fp32_meas = fp32_peak(dev.index if dev.index is not None else 0)
    line["roofline"] = {"bound": "fp32", "achieved": ach, "peak": fp32_meas, "unit": "TFLOP/s",
                        "frac": ach / fp32_meas, "traffic": None,
                        "peak_source": "FP32 FMA probe (wem_measure_fp32_peak), measured in this run",
                        "kernel": "wem_migrate_kernel + wem_model_kernel (41 operator applications)",
                        "ms_per_launch": 1000.0 * el / napply, "flops_per_unit": fl}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU leg: the reference's algorithm for one operator application (the migration
        # of one shot, every frequency) on the host cores; the Born modelling costs the same
        # transforms per unit
        line["cpu_baseline"] = cpu_baseline(c)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="survey64",
                    choices=["survey64", "survey8", "survey3d", "survey3d_band", "split1", "lsm32", "angles8",
                             "elastic8", "elastic3d"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "split16"],
                    help="split16: the FFTs' DFT stages on the tensor cores (split fp16 operands)")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the image-error check against the FP64 oracle")
    ap.add_argument("--fmax", type=float, default=None,
                    help="upper band edge in Hz instead of the workload's (smaller cases for profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.warmup < 3:
        args.warmup = 3

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import wemgpu
    if not os.path.exists(wemgpu.LIB_PATH):
        raise SystemExit("shotwem.so is not built: python -c 'import __graft_entry__ as g; g.build()'")
    c, wl = survey(args.workload, rank)
    if args.fmax is not None:
        c["params"] = dict(c["params"], fmax=float(args.fmax))
        wl += f" [band cut to {c['params']['fmin']:g}-{args.fmax:g} Hz]"
    if args.workload == "angles8":
        return run_angles(args, c, wl, rank, world, local)
    if args.workload in ("elastic8", "elastic3d"):
        return run_elastic(args, c, wl, rank, world, local)
    if args.precision != "fp32":
        c["params"] = dict(c["params"], precision=args.precision)
        wl += f" [{args.precision}: DFT stages on the tensor cores, split fp16 hi+lo operands, fp32 accumulation]"
    p, shots = c["params"], c["shots"]
    nf, nz, nshot = band(p), int(p["nz"]), shots.nshot
    units = nshot * nf * nz
    ctx = wemgpu.Context(local).prepare(p, c["vel"], c["wav"])
    d_dev = torch.from_numpy(np.ascontiguousarray(shots.data)).to(dev)
    m_dev = torch.empty((int(p["nmx"]) * int(p.get("nmy", 1)), nz), dtype=torch.float32, device=dev)  # [nmx*nmy][nz]
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)

    if args.workload == "lsm32":
        return run_lsm(args, ctx, c, wl, units, dev, rank, world, dist)
    for _ in range(args.warmup):
        ctx.migrate_device(shots, d_dev.data_ptr(), m_dev.data_ptr(), sync=True)
    kernels_per_step = ctx.last_timing()[1]

    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kms = []
    ev0.record(stream)
    for _ in range(args.steps):
        ctx.migrate_device(shots, d_dev.data_ptr(), m_dev.data_ptr(), sync=True)
        kms.append(ctx.last_kernel_times())
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    launch = ctx.last_launch() if int(p.get("nmy", 1)) == 1 else None
    elapsed = ev0.elapsed_time(ev1) / 1000.0
    t = torch.tensor([elapsed], dtype=torch.float64, device=dev)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    elapsed = float(t.item())
    value = world * units * args.steps / elapsed

    # end to end through the public API with host buffers: the traces in pinned host memory
    # (the contract's e2e), and beside it from ordinary pageable memory (what a caller that
    # does not pin gets: the library stages the copy through its own pinned slots)
    from wemgpu import Shots
    pinned = torch.from_numpy(np.ascontiguousarray(shots.data)).pin_memory()
    shots_pinned = Shots(shots.sx, shots.sy, shots.trace_offset, shots.trace_cell, pinned.numpy())
    img = np.zeros((int(p["nmx"]) * int(p.get("nmy", 1)), nz), np.float32)

    def e2e_time(sv):
        ts = []
        for _ in range(max(1, args.e2e_steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = ctx.migrate(sv)
            ts.append(time.perf_counter() - t0)
        return statistics.mean(ts), out
    e2e_s, img = e2e_time(shots_pinned)
    e2e_page_s, _ = e2e_time(shots)
    te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if dist:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_s = float(te.item())
    h2d = int(shots.data.nbytes)
    d2h = int(img.nbytes)

    mig_ms = statistics.mean(k[1] for k in kms)
    fl = flops_per_unit(p)
    achieved = units * fl / (mig_ms / 1000.0) / 1e12
    peaks, src = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_nominal = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    fp32_meas = fp32_peak(local)
    prec = p.get("precision", "fp32")
    tr = recorded_traffic(args.workload if prec == "fp32" else f"{args.workload}_{prec}")
    traffic = tr.get("bytes_per_launch") if tr and not tr["stale"] else None

    # The FP32 form runs on the CUDA cores: its bound is the FP32 FMA rate measured in this
    # run. achieved/frac count the algorithmic FLOPs; the *_executed fields count what the
    # kernel runs (skipped references, paired inverse transforms).
    roof = {"bound": "fp32", "achieved": achieved, "peak": fp32_meas, "unit": "TFLOP/s",
            "frac": achieved / fp32_meas, "traffic": traffic,
            "peak_source": "FP32 FMA probe (wem_measure_fp32_peak), measured in this run",
            "kernel": "wem_migrate_kernel", "ms_per_launch": mig_ms,
            "flops_per_unit": fl, "fp32_nominal_tflops": fp32_nominal}
    if tr and tr["stale"]:
        roof["traffic_note"] = "the recorded ncu capture is of older kernel sources; not reported"
    if int(p.get("pspi", 1)) and int(p.get("nmy", 1)) == 1:
        paired = (launch or {}).get("form") == "fp32-paired"
        fe, xinv, rused = executed_flops_per_unit(p, c["vel"], paired)
        roof.update({"inverse_transforms_per_wavefield_step": xinv, "references_used_per_depth_step": rused,
                     "flops_per_unit_executed": fe, "achieved_executed": units * fe / (mig_ms / 1000.0) / 1e12,
                     "frac_executed": units * fe / (mig_ms / 1000.0) / 1e12 / fp32_meas})
    if p.get("precision", "fp32") == "split16":
        tf = tensor_flops_per_unit(p)
        tach = units * tf / (mig_ms / 1000.0) / 1e12
        # timed inside a launch of about a second: the sustained tensor peak applies
        tpeak = float(peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1700.0)))
        roof = {"bound": "tensor", "achieved": tach, "peak": tpeak, "unit": "TFLOP/s", "frac": tach / tpeak,
                "traffic": traffic, "peak_source": f"bf16 dense sustained, {src}",
                "kernel": "wem_migrate_kernel (split16: DFT stages on tcgen05)", "ms_per_launch": mig_ms,
                "tensor_flops_per_unit": tf, "flops_per_unit": fl, "algorithmic_tflops": achieved,
                "fp32_peak_measured": fp32_meas, "fp32_frac_algorithmic": achieved / fp32_meas}
    if int(p.get("nmy", 1)) > 1:
        # 3-D: three passes over device memory per depth step; their bytes bound it (the
        # planes per wavefield the run uses: paired planes in the nearest-lower mode)
        paired3 = int(p.get("pspi", 1)) and p.get("interp", "ref") == "ref" and \
            os.environ.get("WEM_PAIRED", "1") != "0" and int(p["nref"]) <= 16
        sums3 = int(p["padx"]) * int(p["nmx"]) <= 512 and int(p["padx"]) * int(p["nmy"]) <= 512 and \
            os.environ.get("WEM_DIRECT_SUMS", "1") != "0"
        planes = inverse_transforms_per_step(p, c["vel"], bool(paired3), direct_sums=sums3) \
            if int(p.get("pspi", 1)) else 1.0
        bu = bytes_per_unit_3d(p, planes)
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        gbs = units * bu / (mig_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                "traffic": traffic, "peak_source": f"HBM copy, {src}",
                "kernel": "wem3d_rows_fwd + wem3d_cols + wem3d_rows_inv (all depth steps)",
                "ms_per_launch": mig_ms, "bytes_per_unit": bu, "flops_per_unit": fl,
                "fp32_tflops": achieved, "fp32_peak_measured": fp32_meas,
                "fp32_frac": achieved / fp32_meas}
        if tr and tr["stale"]:
            roof["traffic_note"] = "the recorded ncu capture is of older kernel sources; not reported"
    line = {
        "metric": "shot*omega*depth-steps/s", "value": value, "unit": "shot*omega*depth-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if p.get("precision", "fp32") == "fp32" else "f16x2-split/f32",
        "data": "synthetic (seeded)",
        "config": {"workload": wl, "units_per_step_per_gpu": units, "shots": nshot, "frequencies": nf,
                   "depth_steps": nz, "pspi": int(p["pspi"]), "nref": int(p["nref"]), "nkx": int(p["padx"]) * int(p["nmx"]),
                   "interp": p.get("interp", "ref"), "l2": "inputs larger than L2 (traces, spectra, image accumulators)",
                   "parallelism": f"replicas x{world}, shots sharded by rank",
                   "depth_kernel_launch": launch},
        "e2e": {"value": world * units / e2e_s, "unit": "shot*omega*depth-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "host_buffers": "traces in pinned host memory",
                "pageable_value": world * units / e2e_page_s},
        "gpu_launches": kernels_per_step * args.steps,
        "roofline": roof,
        "kernel_ms": {"spectra": statistics.mean(k[0] for k in kms), "extrapolate": mig_ms,
                      "reduce": statistics.mean(k[2] for k in kms)},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU leg: the reference's algorithm timed on the host cores, and the image
        # error measured against the FP64 oracle
        kept = {}
        line["cpu_baseline"] = cpu_baseline(c, keep=kept)
        if not args.no_accuracy:
            if int(p.get("nmy", 1)) == 1:
                line["accuracy"] = accuracy(c, lambda: wemgpu.Context(local))
            else:
                line["accuracy"] = accuracy_sample(c, kept, lambda: wemgpu.Context(local))
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
