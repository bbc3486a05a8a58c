"""Benchmark of the GB300 ExaMiniMD hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload lj4m|lj32k|snapw] [--precision mixed|fp64]

Metric: atom-steps/s (ExaMiniMD's own definition, N * nsteps / time,
examinimd.cpp:286-289).  A step is one MD timestep of the full hot path --
NVE half kick + drift, CommSerial halo refresh (or, every 20th step,
exchange + sorted binning + six-phase halo + binning + CSR neighbour
build), zeroed forces, the LJ force, final half kick -- driven by the
re-hosted ExaMiniMD loop on the GB300 modules.

Workload (default): "LJ-4M", fcc lattice at reduced density 0.8442,
100x100x100 unit cells = 4,000,000 atoms, eps = sigma = 1, r_c = 2.5,
skin 0.3, rebuild every 20 steps, CSR full list, NVE dt 0.005, velocities
from ExaMiniMD's "loop geom" generator at T* = 1.44 (uniform draws: the
reference has no Gaussian option).  Synthetic input generated in-process.

* value: device throughput with the system resident in HBM; K timed steps
  between CUDA events on the library's stream, barrier + synchronize on
  both sides, max over ranks; N>1 runs independent replicas (weak scaling,
  no data-path collective -- CommSerial has no inter-GPU exchange).
* e2e: the same step driven through the C ABI with host buffers -- every
  step uploads x, v, f from pinned host memory (emd_system_update), runs
  the step and downloads x, v, f (emd_system_get).
* roofline: the dominant kernel's algorithmic bytes per launch (CSR row
  entries + row metadata + own position + force read/write) over its mean
  CUDA-event duration measured inside the timed region, against the
  measured HBM copy bandwidth.
* cpu_baseline: the CPU oracle (a restatement of ExaMiniMD's serial
  algorithm, OpenMP over atoms) on this host's cores, a bounded sample of
  the same workload.
* accuracy (mixed form, after the timed region): forces of the final state
  against the FP64 drop-in on the same positions (RMS and max |dF| over the
  RMS force), and the NVE total-energy drift of both forms over
  --drift-steps further steps, per 1000 steps.
* snap_w: the SNAP-W workload (bcc tungsten, 128,000 atoms, 2J = 8) through
  the same driver in both forms, device-timed, with the mixed-form force
  error at step 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "lj4m": dict(cells=100, desc="LJ-4M: fcc rho*=0.8442 100^3 cells = 4,000,000 atoms, rc 2.5, skin 0.3, "
                                 "rebuild every 20, CSR full list, NVE dt 0.005"),
    "lj32k": dict(cells=20, desc="LJ-32k: fcc rho*=0.8442 20^3 cells = 32,000 atoms, rc 2.5, skin 0.3, "
                                 "rebuild every 20, CSR full list, NVE dt 0.005"),
    "snapw": dict(cells=40, desc="SNAP-W: bcc W a=3.1803 A, 40^3 cells = 128,000 atoms, twojmax 8, synthetic "
                                 "coefficients (seed 20261203), 300 K, dt 0.5 fs, rebuild every step, full list"),
}
METRIC = "atom-steps/s"

SNAP_DESC = ("SNAP-W: bcc W a=3.1803 A, 40^3 cells = 128,000 atoms, metal units, mass 183.84, twojmax 8, rcutfac "
             "4.73442, rfac0 0.99363, rmin0 0, 56 coefficients (beta0 = -8, beta1..55 ~ N(0, 0.1), seed 20261203), "
             "300 K loop-geom velocities, dt 0.5 fs, newton on, skin 1.0, neighbour rebuild every step, full list")


def snap_files(work: str) -> tuple[str, str]:
    """Synthetic tungsten coefficient file and the shipped W.snapparam values."""
    import numpy as np
    beta = np.concatenate([[-8.0], np.random.default_rng(20261203).normal(0.0, 0.1, 55)])
    coeff, param = os.path.join(work, "W.synth.snapcoeff"), os.path.join(work, "W.snapparam")
    with open(coeff, "w") as fp:
        fp.write("1 56\nW 0.5 1\n" + "".join(f"{float(b)!r}\n" for b in beta))
    with open(param, "w") as fp:
        fp.write("rcutfac 4.73442\ntwojmax 8\nrfac0 0.99363\nrmin0 0\ndiagonalstyle 3\nbzeroflag 0\n"
                 "quadraticflag 0\n")
    return coeff, param


def snap_deck_text(cells: int, steps: int, coeff: str, param: str) -> str:
    return f"""units metal
timestep 0.0005
atom_style atomic
newton on
lattice bcc 3.1803
region box block 0 {cells} 0 {cells} 0 {cells}
create_box 1 box
create_atoms 1 box
mass 1 183.84
pair_style snap
pair_coeff * * {coeff} W {param} W
neighbor 1.0 bin
neigh_modify once no every 1 delay 0 check yes
velocity all create 300.0 4928459 loop geom
fix 1 all nve
thermo 0
run {steps}
"""


def deck_text(cells: int, steps: int, mass=1.0, temp=1.44, thermo: int = 0) -> str:
    return f"""units lj
atom_style atomic
newton off
lattice fcc 0.8442
region box block 0 {cells} 0 {cells} 0 {cells}
create_box 1 box
create_atoms 1 box
mass 1 {mass}
velocity all create {temp} 87287 loop geom
pair_style lj/cut 2.5
pair_coeff 1 1 1.0 1.0 2.5
neighbor 0.3 bin
neigh_modify delay 0 every 20 check no
fix 1 all nve
thermo {thermo}
run {steps}
"""


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return dict(hbm_gbs=float(d["hbm_gbs"]), src="measured")
    return dict(hbm_gbs=6800.0, src="fallback")


def fp_pipe_peaks(device: int) -> dict:
    """FP64 and FP32 (non-tensor) arithmetic peaks of this GPU, measured as
    cuBLAS DGEMM and SGEMM (TF32 off) throughput, best of three, in GFLOP/s:
    the denominators of the SNAP roofline (MEASURED_PEAKS.json holds HBM and
    bf16 tensor figures only)."""
    import torch
    out = {}
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for name, dt, n in (("fp64", torch.float64, 4096), ("fp32", torch.float32, 8192)):
            a = torch.randn(n, n, dtype=dt, device=device)
            b = torch.randn(n, n, dtype=dt, device=device)
            torch.matmul(a, b)
            torch.cuda.synchronize()
            best = 1e30
            for _ in range(3):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b)
                e1.record()
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            out[name] = 2.0 * n ** 3 / (best * 1e-3) / 1e9
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    out["how"] = "torch.matmul DGEMM 4096^3 and SGEMM 8192^3 (TF32 off), best of 3, CUDA events"
    return out


def snap_inside_mean(ctx, n_local: int, rcutsq: float) -> float:
    """Mean number of neighbours inside the SNAP cutoff, from the device's
    positions and full list."""
    import numpy as np
    nl_, ng_ = ctx.info()[:2]
    st = ctx.get(0, nl_ + ng_, fields=("x",))
    x = st["x"]
    num = np.empty(max(n_local, 1), np.int32)
    from examinimd_gb300._lib import _ip
    assert ctx.lib.emd_neigh_get(ctx.h, _ip(num), None) == 0
    total = int(num[:n_local].sum())
    ent = np.empty(max(total, 1), np.int32)
    assert ctx.lib.emd_neigh_get(ctx.h, None, _ip(ent)) == 0
    i = np.repeat(np.arange(n_local), num[:n_local])
    d = x[ent[:total]] - x[i]
    return float(np.count_nonzero(np.einsum("ij,ij->i", d, d) < rcutsq)) / n_local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_pg(ws, use_cuda):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("nccl" if use_cuda else "gloo")
    return dist


def reduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ CPU arm
def cpu_sample(cells: int, steps: int, warmup: int, threads: int | None = None) -> dict:
    """Times the CPU oracle (serial algorithm of ExaMiniMD, OpenMP over atoms)."""
    from oracle.orc import Oracle
    from tests import mdloop
    threads = threads or os.cpu_count() or 1
    setup = mdloop.LJSetup(cells)
    t0 = time.perf_counter()
    state = mdloop.make_lattice(setup, threads)
    o = Oracle(threads)
    mdloop.init(o, setup, state)
    t_init = time.perf_counter() - t0
    n = o.info()[0]
    for s in range(1, warmup + 1):
        mdloop.step(o, setup, s)
    t1 = time.perf_counter()
    for s in range(warmup + 1, warmup + steps + 1):
        mdloop.step(o, setup, s)
    dt = time.perf_counter() - t1
    return dict(value=n * steps / dt, n=n, steps=steps, seconds=dt, init_s=t_init, threads=threads)


def run_reference_arm(a, ws, rank):
    if rank != 0:
        return
    wl = WORKLOADS[a.workload]
    steps = max(1, min(a.steps, 20))
    warm = min(a.warmup, 5)
    r = cpu_sample(wl["cells"], steps, warm)
    sample = (f"{wl['desc']}; CPU oracle port of ExaMiniMD's serial algorithm, {r['threads']} OpenMP threads; "
              f"{warm} warm-up + {steps} timed steps of the full {r['n']}-atom system (bounded sample), init "
              f"{r['init_s']:.1f}s excluded")
    line = {"metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": ws, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 * r["seconds"] / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (fcc lattice, loop-geom velocities)",
            "config": {"workload": a.workload, "atoms": r["n"], "neigh": "CSR full", "precision": "fp64",
                       "l2": "working set > L2"},
            "impl": "reference",
            "cpu_baseline": {"value": r["value"], "unit": METRIC, "cores": r["threads"], "kind": "port",
                             "sample": sample},
            "e2e": {"value": r["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    emit(line)


# ------------------------------------------------------------------ GPU arm
def algorithmic_bytes_per_atom(precision: str, mean_row: float) -> float:
    """Bytes one atom's force evaluation must move from DRAM: its list entries
    (4 B each), its row metadata (count 4 B; FP64 CSR also the row start),
    its own position and one fetch of its copy as somebody's neighbour
    (cell-sorted gathers: FP32 float4 16 B each for mixed, double4 32 B each
    for FP64), and the force write (24 B; the zeroing is folded in)."""
    if precision == "mixed":
        return 4.0 * mean_row + 4.0 + 16.0 + 16.0 + 24.0
    return 4.0 * mean_row + 8.0 + 32.0 + 32.0 + 24.0


def run_gpu_arm(a, ws, rank, local):
    import numpy as np
    import torch

    from examinimd_gb300 import MD

    dist = init_pg(ws, True)
    torch.cuda.set_device(local)
    wl = WORKLOADS[a.workload]
    snap = a.workload == "snapw"
    tmp = tempfile.mkdtemp(prefix="emdbench_")
    deck = os.path.join(tmp, "in.deck")
    with open(deck, "w") as fp:
        if snap:
            fp.write(snap_deck_text(wl["cells"], a.steps, *snap_files(tmp)))
        else:
            fp.write(deck_text(wl["cells"], a.steps))
    md = MD(["-il", deck, "--quiet", "--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
             "--comm-type", "SERIAL", "--precision", a.precision, "--device", str(local)])
    ctx = md.ctx
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    N = md.info()["N"]
    # warm-up (complete rebuild cycles so the timed region starts right after a build)
    md.run(a.warmup)
    ctx.synchronize()
    kname = (f"snap_{a.precision}" if snap else
             ("lj_full_mixed" if a.precision == "mixed" else "lj_full_fp64"))
    # in the timed region only the dominant kernel is bracketed by events
    # (two per launch; the other launches are counted): the per-kernel
    # breakdown comes from a separate pass below
    ctx.timing(True)
    ctx.timing_only(kname)
    ctx.timing_reset()
    clocks = ClockSampler(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    e0.record(stream)
    md.run(a.steps)
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    ms_max = reduce_max(dist, ms)
    rep = ctx.timing_report()
    launches = sum(c for _, c in rep.values())
    value = ws * N * a.steps / (ms_max * 1e-3)
    kms, kn = rep.get(kname, (0.0, 0))
    # per-kernel breakdown: every launch bracketed, over one more rebuild cycle
    # (20 steps; 3 for SNAP, which rebuilds every step) after the timed region
    ctx.timing_only(None)
    ctx.timing_reset()
    md.run(3 if snap else 20)
    ctx.synchronize()
    rep_all = ctx.timing_report()
    ctx.timing(False)

    # dominant kernel roofline
    nl = md.info()["N_local"]
    mean_row = float(md_row_mean(ctx, nl))
    peaks = load_peaks()
    if snap:
        # bound by the FP64 pipe (the Wigner-U recursion stays FP64 in both
        # forms); no measured FP64 peak exists to divide by
        roof = {"kernel": kname, "bound": "fp64", "achieved": None, "peak": None, "unit": "GFLOP/s",
                "frac": None, "traffic": None, "mean_row": mean_row, "launch_ms": (kms / kn) if kn else None,
                "note": "FP64-pipe bound (ncu sm__inst_executed_pipe_fp64); DRAM traffic negligible"}
    else:
        bytes_launch = algorithmic_bytes_per_atom(a.precision, mean_row) * nl
        achieved = bytes_launch / (kms / kn * 1e-3) / 1e9 if kn else None
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            ent = json.load(open(tpath)).get(f"{kname}@{a.workload}")
            if ent:
                traffic = ent.get("bytes_per_launch")
        roof = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": (achieved / peaks["hbm_gbs"]) if achieved else None, "traffic": traffic,
                "peak_source": peaks["src"], "bytes_per_launch": bytes_launch, "mean_row": mean_row,
                "launch_ms": (kms / kn) if kn else None}
        if a.precision == "fp64" and kn:
            # the FP64 drop-in is bound by the FP64 pipe: 8 operations per listed
            # pair (difference, r^2, test) and 13 more inside the cutoff (1/r^2,
            # r^-6, the force, the sums); the inside fraction is the volume
            # ratio (rc / (rc + skin))^3 of the two cutoffs
            pk = fp_pipe_peaks(local)
            inside = (2.5 / 2.8) ** 3
            flops = nl * mean_row * (8.0 + 13.0 * inside)
            got = flops / (kms / kn * 1e-3) / 1e9
            roof["fp64_pipe"] = {"achieved": got, "peak": pk["fp64"], "unit": "GFLOP/s", "frac": got / pk["fp64"],
                                 "flops_per_launch": flops, "peak_how": pk["how"]}
    kernels = {k: {"ms": v[0], "launches": v[1], "share": v[0] / max(1e-12, sum(x[0] for x in rep_all.values()))}
               for k, v in sorted(rep_all.items(), key=lambda kv: -kv[1][0])}

    # e2e through the C ABI with host buffers (pinned), copies inside the timed region
    e2e_steps = max(1, min(a.steps, a.e2e_steps))
    hx = torch.empty((nl, 3), dtype=torch.float64, pin_memory=True).numpy()
    hv = torch.empty((nl, 3), dtype=torch.float64, pin_memory=True).numpy()
    hf = torch.empty((nl, 3), dtype=torch.float64, pin_memory=True).numpy()
    lib = ctx.lib
    from examinimd_gb300._lib import _dp
    st = lib.emd_system_get(ctx.h, 0, nl, _dp(hx), _dp(hv), _dp(hf), None, None, None)
    assert st == 0
    barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # every step: x, v, f uploaded from the pinned host arrays, one ExaMiniMD
    # step, x, v, f read back into them (x's read-back overlaps the force; each
    # field's upload for the next step follows its read-back)
    md.run_host(e2e_steps, hx, hv, hf)
    ctx.synchronize()
    t_e2e = reduce_max(dist, time.perf_counter() - t0)
    barrier(dist)
    e2e = {"value": ws * N * e2e_steps / t_e2e, "unit": METRIC, "h2d_bytes_per_step": int(nl * 72),
           "d2h_bytes_per_step": int(nl * 72), "steps": e2e_steps,
           "path": "emd_md_run_host: per step x,v,f pinned H2D, one ExaMiniMD step, x,v,f D2H (x's read-back "
                   "overlapping the force, f's the final integration; each H2D of the next step queued behind "
                   "the same field's D2H, so the two directions overlap; the step starts in two row chunks)"}
    T, pe, ke = md.thermo(recompute=True)

    extra = {}
    if not a.no_fp64 and a.workload.startswith("lj") and a.precision == "mixed":
        extra["fp64"] = fp64_block(local, wl["cells"], a.fp64_steps, 3)
        extra["fp64"]["mixed_over_fp64"] = value / ws / extra["fp64"]["value"]
    if not a.no_thermo and a.workload.startswith("lj") and a.precision == "mixed":
        extra["thermo10"] = thermo_block(local, wl["cells"], a.thermo_steps, 5)
        extra["thermo10"]["relative_to_thermo0"] = extra["thermo10"]["value"] / (value / ws)
    if not a.no_accuracy and a.workload.startswith("lj") and a.precision == "mixed":
        extra["accuracy"] = lj_accuracy(md, wl["cells"], a.drift_steps, local)
    if not a.no_snap and a.workload == "lj4m":
        extra["snap_w"] = snap_measure(local, a.snap_steps, max(2, a.snap_steps // 5), 3,
                                       with_cpu=(rank == 0 and not a.no_cpu))
    if not a.no_batch and a.workload == "lj4m":
        extra["batched_lj"] = batch_measure(local, a.batch_steps, 8, 20)
    if not a.no_fit and a.workload == "lj4m":
        extra["fit_gradients"] = fit_measure(local, a.fit_evals)
    if rank == 0 and not a.no_cpu and not snap:
        try:
            r = cpu_sample(WORKLOADS["lj4m"]["cells"] if a.workload == "lj4m" else wl["cells"], a.cpu_steps, 1)
            extra["cpu_baseline"] = {
                "value": r["value"], "unit": METRIC, "cores": r["threads"], "kind": "port",
                "sample": (f"CPU oracle port of ExaMiniMD's serial algorithm (OpenMP over atoms), same {r['n']}-atom "
                           f"workload, 1 warm-up + {r['steps']} timed steps incl. one neighbour rebuild per 20; "
                           f"init excluded")}
        except Exception as e:  # the baseline must not take the GPU line down
            extra["cpu_baseline"] = {"value": None, "unit": METRIC, "cores": os.cpu_count(), "kind": "port",
                                     "sample": f"failed: {e}"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64" if a.precision == "mixed" else "f64",
                "data": ("synthetic (bcc W lattice, synthetic SNAP coefficients, loop-geom velocities)" if snap
                         else "synthetic (fcc lattice, ExaMiniMD loop-geom velocities)"),
                "config": {"workload": a.workload, "desc": wl["desc"], "atoms_per_gpu": N, "precision": a.precision,
                           "neigh": "CSR full", "parallelism": f"replicas{ws}",
                           "l2": ("compute-bound (SNAP); inputs re-read every step, no flush" if snap else
                                  "working set (positions, forces, 1.2 GB neighbour list) > 129 MB L2; no flush")},
                "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "thermo_end": {"T": T, "PE_per_atom": pe, "KE_per_atom": ke}, "kernels": kernels}
        line.update(extra)
        emit(line)
    md.close()
    if dist is not None:
        dist.destroy_process_group()


def by_id(st: dict, key: str):
    import numpy as np
    order = np.argsort(st["id"])
    return st[key][order]


def force_error(f, f_ref) -> dict:
    """RMS and max of |dF| over the RMS of |F_ref| (per-atom relative errors
    are unbounded where the net force nearly cancels)."""
    import numpy as np
    err = np.linalg.norm(f - f_ref, axis=1)
    scale = float(np.sqrt(np.mean(np.linalg.norm(f_ref, axis=1) ** 2)))
    return {"rms_rel": float(np.sqrt(np.mean(err ** 2)) / scale), "max_rel": float(err.max() / scale),
            "force_scale_rms": scale}


def lj_accuracy(md, cells: int, drift_steps: int, device: int) -> dict:
    """Mixed-form accuracy at full size, from the state the timed run ended in:
    forces against the FP64 drop-in on the same positions, and the NVE total
    energy drift of both forms over `drift_steps` further steps."""
    from examinimd_gb300 import Context, EMD_PREC_FP64
    from tests import mdloop
    ctx = md.ctx
    nl = md.info()["N_local"]
    st = ctx.get(0, nl)
    setup = mdloop.LJSetup(cells)
    ref = Context(device)
    mdloop.init(ref, setup, st, precision=EMD_PREC_FP64)
    nr = ref.info()[0]
    out = force_error(by_id(st, "f"), by_id(ref.get(0, nr), "f"))
    N = float(nr)

    def e_ref():
        return (ref.lj_energy() + 0.5 * ref.thermo_mv2()) / N
    T, pe, ke = md.thermo(recompute=True)
    e0m, e0r = pe + ke, e_ref()
    t0 = time.perf_counter()
    md.run(drift_steps)
    t_m = time.perf_counter() - t0
    T, pe, ke = md.thermo(recompute=True)
    e1m = pe + ke
    t0 = time.perf_counter()
    for s_ in range(1, drift_steps + 1):
        mdloop.step(ref, setup, s_)
    ref.synchronize()
    t_r = time.perf_counter() - t0
    e1r = e_ref()
    ref.close()
    out.update({"energy_drift_steps": drift_steps,
                "energy_drift_rel_mixed": (e1m - e0m) / abs(e0m) * 1000.0 / drift_steps,
                "energy_drift_rel_fp64": (e1r - e0r) / abs(e0r) * 1000.0 / drift_steps,
                "drift_units": "relative change of total energy per 1000 steps",
                "E0_per_atom": e0r, "drift_wall_s": {"mixed": t_m, "fp64": t_r}})
    return out


def snap_accuracy(md, device: int, cells: int, coeff: str, param: str, steps_done: int) -> dict:
    """Mixed-form SNAP forces of the state the run ended in against the FP64
    drop-in on the same positions."""
    from examinimd_gb300 import Context, EMD_PREC_FP64
    from tests import mdloop
    from tests.golden.decks import read_snap_files
    nl = md.info()["N_local"]
    st = md.ctx.get(0, nl)
    setup = mdloop.SnapSetup(cells, cells, cells, read_snap_files(coeff, param), a=3.1803, mass=183.84,
                             lattice_style=2, dt=0.0005)
    ref = Context(device)
    mdloop.init(ref, setup, st, precision=EMD_PREC_FP64)
    out = force_error(by_id(st, "f"), by_id(ref.get(0, ref.info()[0]), "f"))
    ref.close()
    out["state"] = f"after {steps_done} mixed-form steps from the 300 K lattice"
    return out


def snap_cpu_sample(coeff: str, param: str, cells: int = 20, steps: int = 20, threads: int | None = None) -> dict:
    """The CPU oracle's SNAP (the reference formulation, OpenMP over atoms on
    every host core) on a bcc cells^3 sample of the SNAP-W workload, timed per
    atom-step."""
    from oracle.orc import Oracle
    from tests import mdloop
    from tests.golden.decks import read_snap_files
    setup = mdloop.SnapSetup(cells, cells, cells, read_snap_files(coeff, param), a=3.1803, mass=183.84,
                             lattice_style=2, dt=0.0005)
    state = mdloop.make_lattice(setup)
    threads = threads or os.cpu_count() or 1
    o = Oracle(threads)
    mdloop.init(o, setup, state)
    n = o.info()[0]
    t0 = time.perf_counter()
    for s_ in range(1, steps + 1):
        mdloop.step(o, setup, s_)
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"CPU oracle (ExaMiniMD's SNAP formulation, OpenMP over atoms with a force buffer per thread), "
                      f"bcc {cells}^3 = {n} atoms of the SNAP-W workload, {steps} steps (neighbour rebuild every "
                      f"step), {dt:.1f} s"}


def snap_measure(local: int, steps_mixed: int, steps_fp64: int, warm: int, cells: int = 40,
                 with_cpu: bool = True) -> dict:
    """SNAP-W through the driver in both forms: device-timed atom-steps/s, the
    SNAP kernel's share, and the mixed-form force error at step 0."""
    import torch

    from examinimd_gb300 import MD
    tmp = tempfile.mkdtemp(prefix="emdsnap_")
    coeff, param = snap_files(tmp)
    peaks = fp_pipe_peaks(local)
    res, acc = {}, None
    for prec, steps in (("mixed", steps_mixed), ("fp64", steps_fp64)):
        deck = os.path.join(tmp, f"in.snap.{prec}")
        with open(deck, "w") as fp:
            fp.write(snap_deck_text(cells, steps, coeff, param))
        md = MD(["-il", deck, "--quiet", "--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
                 "--comm-type", "SERIAL", "--precision", prec, "--device", str(local)])
        ctx = md.ctx
        stream = torch.cuda.ExternalStream(ctx.stream, device=local)
        md.run(warm)
        ctx.synchronize()
        ctx.timing(True)
        ctx.timing_reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        md.run(steps)
        e1.record(stream)
        ctx.synchronize()
        ms = e0.elapsed_time(e1)
        rep = ctx.timing_report()
        ctx.timing(False)
        kname = f"snap_{prec}"
        kms, kn = rep.get(kname, (0.0, 0))
        N = md.info()["N"]
        res[prec] = {"value": N * steps / (ms * 1e-3), "unit": METRIC, "ms_per_step": ms / steps, "steps": steps,
                     "warmup": warm, "kernel": kname, "kernel_ms_per_launch": (kms / kn) if kn else None,
                     "kernel_share": kms / max(1e-12, sum(v[0] for v in rep.values())),
                     "gpu_launches": sum(c for _, c in rep.values())}
        if prec == "mixed":
            acc = snap_accuracy(md, local, cells, coeff, param, warm + steps)
        # roofline: operations of the kernel's own formulation (snap_flops)
        # against the measured FP64 and FP32 pipe peaks
        if kn:
            from examinimd_gb300.snap_flops import snap_flops
            rc = 2.0 * 0.5 * 4.73442  # 2 radius rcutfac of the synthetic W coefficients
            nin = snap_inside_mean(ctx, md.info()["N_local"], rc * rc)
            fl = snap_flops(8, nin)
            t = kms / kn * 1e-3
            n_loc = md.info()["N_local"]
            f64, f32 = fl["fp64"][prec] * n_loc, fl["fp32"][prec] * n_loc
            t_roof = max(f64 / (peaks["fp64"] * 1e9), f32 / (peaks["fp32"] * 1e9))
            res[prec]["roofline"] = {
                "bound": "fp64" if prec == "fp64" else "fp64+fp32 (max of the two pipe times)",
                "flops_per_atom": fl["total"], "fp64_flops_per_atom": fl["fp64"][prec],
                "fp32_flops_per_atom": fl["fp32"][prec], "ninside_mean": nin,
                "achieved_gflops": fl["total"] * n_loc / t / 1e9, "peak_fp64_gflops": peaks["fp64"],
                "peak_fp32_gflops": peaks["fp32"], "frac": t_roof / t,
                "how": "examinimd_gb300/snap_flops.py counts the kernel's loops; peaks " + peaks["how"]}
        md.close()
    res["speedup_mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    res["accuracy"] = acc
    res["energy_drift"] = snap_drift(local, coeff, param)
    if with_cpu:
        res["cpu_baseline"] = snap_cpu_sample(coeff, param)
    res["config"] = SNAP_DESC
    return res


def timed_lj(local: int, cells: int, precision: str, steps: int, warm: int, thermo: int = 0,
             only: tuple = ()) -> dict:
    """One LJ run of the benchmark deck through the driver, device-timed with
    CUDA events on the library's stream; returns the run's figures and the
    per-kernel report (the MD object is closed).  `only`: the kernels whose
    launches get events (the others are counted)."""
    import torch

    from examinimd_gb300 import MD
    tmp = tempfile.mkdtemp(prefix="emdlj_")
    deck = os.path.join(tmp, "in.deck")
    with open(deck, "w") as fp:
        fp.write(deck_text(cells, warm + steps, thermo=thermo))
    md = MD(["-il", deck, "--quiet", "--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL", "--comm-type",
             "SERIAL", "--precision", precision, "--device", str(local)])
    ctx = md.ctx
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    md.run(warm)
    ctx.synchronize()
    ctx.timing(True)
    ctx.timing_only(list(only) or None)
    ctx.timing_reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    md.run(steps)
    e1.record(stream)
    ctx.synchronize()
    ms = e0.elapsed_time(e1)
    rep = ctx.timing_report()
    ctx.timing(False)
    N, nl = md.info()["N"], md.info()["N_local"]
    mean_row = float(md_row_mean(ctx, nl))
    md.close()
    return {"value": N * steps / (ms * 1e-3), "ms_per_step": ms / steps, "steps": steps, "warmup": warm,
            "atoms": N, "n_local": nl, "mean_row": mean_row, "report": rep,
            "gpu_launches": sum(c for _, c in rep.values())}


def fp64_block(local: int, cells: int, steps: int, warm: int) -> dict:
    """The FP64 drop-in on the same LJ workload: throughput and the roofline
    of its force kernel (bound by the FP64 pipe)."""
    r = timed_lj(local, cells, "fp64", steps, warm, only=("lj_full_fp64",))
    kms, kn = r["report"].get("lj_full_fp64", (0.0, 0))
    out = {k: r[k] for k in ("value", "ms_per_step", "steps", "warmup", "atoms", "gpu_launches")}
    out["unit"] = METRIC
    if kn:
        pk = fp_pipe_peaks(local)
        inside = (2.5 / 2.8) ** 3
        flops = r["n_local"] * r["mean_row"] * (8.0 + 13.0 * inside)
        t = kms / kn * 1e-3
        bytes_launch = algorithmic_bytes_per_atom("fp64", r["mean_row"]) * r["n_local"]
        out["roofline"] = {"kernel": "lj_full_fp64", "bound": "fp64", "launch_ms": kms / kn,
                           "achieved": flops / t / 1e9, "peak": pk["fp64"], "unit": "GFLOP/s",
                           "frac": flops / t / 1e9 / pk["fp64"], "flops_per_launch": flops,
                           "hbm_gbs": bytes_launch / t / 1e9, "peak_how": pk["how"],
                           "note": "8 FP64 operations per listed pair and 13 more inside the cutoff"}
    return out


def thermo_block(local: int, cells: int, steps: int, warm: int, every: int = 10) -> dict:
    """The mixed form with a thermo evaluation every `every` steps (ExaMiniMD's
    LJ-32k deck prints thermo every 10): on those steps the force call also
    runs the mixed-precision energy kernel over the same rows
    (emd_lj_request_energy)."""
    r = timed_lj(local, cells, "mixed", steps, warm, thermo=every,
                 only=("lj_full_mixed", "lj_energy_mixed", "lj_pos_remainder"))
    rep = r["report"]
    out = {k: r[k] for k in ("value", "ms_per_step", "steps", "warmup", "atoms", "gpu_launches")}
    out.update(unit=METRIC, thermo_every=every,
               kernels_ms_per_launch={k: v[0] / v[1] for k, v in rep.items()
                                      if v[1] and k.startswith(("lj_full", "lj_energy", "lj_pos"))})
    return out


def shipped_w_files(work: str) -> tuple[str, str]:
    """ExaMiniMD's shipped W.snapcoeff / W.snapparam numbers (kept in the
    golden fixture tests/golden/snap_W_sc.npz), written back as files."""
    import numpy as np

    from tests.golden.decks import write_snap_files
    g = np.load(os.path.join(ROOT, "tests", "golden", "snap_W_sc.npz"))
    snap = dict(elem=str(g["snap_elem"]), radius=float(g["snap_radius"]), weight=float(g["snap_weight"]),
                beta=list(g["snap_beta"]), params=dict(zip([str(k) for k in g["snap_param_keys"]],
                                                           [str(v) for v in g["snap_param_vals"]])))
    write_snap_files(work, dict(coeff="W.shipped.snapcoeff", param="W.shipped.snapparam"), snap)
    return os.path.join(work, "W.shipped.snapcoeff"), os.path.join(work, "W.shipped.snapparam")


def snap_drift(local: int, coeff: str, param: str, cells: int = 16, steps: int = 1000, every: int = 25) -> dict:
    """NVE total-energy drift of SNAP in both forms: the SNAP energy (with the
    1.25e5 / r^12 term of the reference's repulsion) plus the kinetic energy,
    both in FP64, sampled every `every` steps of a bcc cells^3 W system from
    the 300 K lattice (dt 0.5 fs); drift = slope of a least-squares line
    through the samples, relative to |E0|, per 1000 steps.  Two coefficient
    sets: the workload's synthetic one, whose random coefficients make the
    lattice unstable (the temperature runs away, so the drift is the
    integrator's on a violent trajectory, the same in both forms), and
    ExaMiniMD's shipped W fit, a physical tungsten model."""
    import numpy as np

    from examinimd_gb300 import MD
    tmp = tempfile.mkdtemp(prefix="emdsnapdrift_")
    out = {"steps": steps, "sample_every": every, "dt_ps": 0.0005,
           "units": "relative change of total energy per 1000 steps (least-squares slope)"}
    sets = (("synthetic_beta", coeff, param), ("shipped_W", *shipped_w_files(tmp)))
    for label, cf, pf in sets:
        res = {}
        for prec in ("mixed", "fp64"):
            deck = os.path.join(tmp, f"in.snap.{label}.{prec}")
            with open(deck, "w") as fp:
                fp.write(snap_deck_text(cells, steps, cf, pf))
            md = MD(["-il", deck, "--quiet", "--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
                     "--comm-type", "SERIAL", "--precision", prec, "--device", str(local)])
            t0 = time.perf_counter()
            es, ts, temps = [], [], []
            for s_ in range(0, steps + 1, every):
                if s_ > 0:
                    md.run(every)
                T, pe, ke = md.thermo(recompute=True)
                es.append(pe + ke)
                ts.append(s_)
                temps.append(T)
            wall = time.perf_counter() - t0
            out["atoms"] = md.info()["N"]
            md.close()
            e = np.array(es)
            slope = np.polyfit(np.array(ts, float), e, 1)[0]
            res[prec] = {"drift_per_1000": slope * 1000.0 / abs(e[0]), "E0_per_atom": float(e[0]),
                         "end_to_end_per_1000": (e[-1] - e[0]) / abs(e[0]) * 1000.0 / steps,
                         "T_start": temps[0], "T_end": temps[-1], "T_max": max(temps), "wall_s": wall}
        out[label] = res
    return out


def fit_measure(local: int, evals: int) -> dict:
    """Force-matching gradient throughput: the 64 bcc W configurations (16 to
    1,024 atoms) with targets from a hidden beta*, and the 16 fcc LJ
    configurations with hidden (eps, sigma); one evaluation is the loss and its
    gradient (FP64 forward of every configuration, then the adjoint kernels)
    through the torch harness."""
    import numpy as np
    import torch
    from examinimd_gb300 import fit
    ncoef = fit.ncoeffall_for(8)
    scfg = [fit.SnapConfig(x, box, fit.W_PARAMS, device=local) for x, box in fit.snap_config_set(64)]
    lcfg = [fit.LJConfig(x, box, device=local) for x, box in fit.lj_config_set(16)]
    with torch.no_grad():
        Es, Fs = fit.SnapEnergyForces.apply(torch.tensor(fit.synthetic_beta(20261203, ncoef)), scfg)
        El, Fl = fit.LJEnergyForces.apply(torch.tensor([1.05, 0.98], dtype=torch.float64), lcfg)
    out = {}
    for name, cfgs, p0, fn, Er, Fr, wE in (
            ("snap", scfg, fit.synthetic_beta(7, ncoef), fit.SnapEnergyForces, Es, Fs, 1e-2),
            ("lj", lcfg, np.array([1.0, 1.0]), fit.LJEnergyForces, El, Fl, 1e-3)):
        def step():
            p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
            E, F = fn.apply(p, cfgs)
            fit.loss_fn(E, F, Er, Fr, w_E=wE, w_F=1.0).backward()
            return p.grad
        step()  # warm-up (contexts, tables, lists)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(evals):
            g = step()
        t = time.perf_counter() - t0
        atoms = sum(c.n for c in cfgs)
        out[name] = {"gradient_evals_per_s": evals / t, "configs": len(cfgs), "atoms": atoms,
                     "atom_evals_per_s": atoms * evals / t, "grad_norm": float(g.norm()),
                     "how": "wall time of loss + backward through torch.autograd (FP64 forward of every "
                            "configuration, then the adjoint; SNAP: the adjoint reads the U_tot and Z its "
                            "forward kept), each configuration on its own context"}
    for c in scfg + lcfg:
        c.close()
    return out


def batch_ensemble(nsys=256, seed=20261204, rho=0.8442, temp=1.44):
    """256 fcc LJ systems, N_k log-uniform in [500, 20000] realised as
    round((N_k / 4)^(1/3)) cubic cells, lattice positions, Gaussian velocities
    at temp with zero net momentum per system."""
    import numpy as np
    from examinimd_gb300 import fit
    rng = np.random.default_rng(seed)
    a = (4.0 / rho) ** (1.0 / 3.0)
    target = np.exp(rng.uniform(np.log(500.0), np.log(20000.0), nsys))
    cells = np.maximum(5, np.round((target / 4.0) ** (1.0 / 3.0)).astype(int))
    xs, vs, boxes = [], [], []
    for c in cells:
        x = fit.lattice("fcc", a, int(c))
        v = rng.normal(0.0, np.sqrt(temp), size=x.shape)
        v -= v.mean(axis=0)
        xs.append(x)
        vs.append(v)
        boxes.append([c * a] * 3)
    return cells, np.array([len(x) for x in xs]), np.array(boxes), np.concatenate(xs), np.concatenate(vs)


def batch_measure(local: int, steps: int, loop_sample: int, loop_steps: int) -> dict:
    """The batched ensemble: tuned shape, `steps` steps in CUDA graphs, device-timed;
    beside it the same systems looped one at a time through the FP64 drop-in
    driver (a sample of `loop_sample` sizes, `loop_steps` steps each)."""
    import numpy as np
    import torch

    from examinimd_gb300 import MD, Batch
    cells, ns, boxes, x, v = batch_ensemble()
    t0 = time.perf_counter()
    b = Batch(ns, boxes, x, v)
    t_create = time.perf_counter() - t0
    threads, spl = b.tune(40)
    stream = torch.cuda.ExternalStream(b.stream, device=local)
    mv2, pe = b.thermo()
    e0 = 0.5 * mv2 + pe
    e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e_a.record(stream)
    b.run(steps)
    e_b.record(stream)
    torch.cuda.synchronize()
    ms = e_a.elapsed_time(e_b)
    mv2, pe = b.thermo()
    e1 = 0.5 * mv2 + pe
    drift = np.abs(e1 - e0) / np.abs(e0) * 1000.0 / steps
    b.close()
    total = int(ns.sum())
    value = total * steps / (ms * 1e-3)
    # looping the FP64 single-system drop-in over a spread of the same sizes
    tmp = tempfile.mkdtemp(prefix="emdloop_")
    pick = np.unique(np.quantile(cells, np.linspace(0, 1, loop_sample), method="nearest"))
    loop_atoms, loop_ms = 0, 0.0
    for c in pick:
        deck = os.path.join(tmp, f"in.lj{c}")
        with open(deck, "w") as fp:
            fp.write(deck_text(int(c), loop_steps))
        md = MD(["-il", deck, "--quiet", "--precision", "fp64", "--device", str(local)])
        s = torch.cuda.ExternalStream(md.ctx.stream, device=local)
        md.run(3)
        md.ctx.synchronize()
        a1, a2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t1 = time.perf_counter()
        a1.record(s)
        md.run(loop_steps)
        a2.record(s)
        md.ctx.synchronize()
        wall = (time.perf_counter() - t1) * 1e3
        loop_ms += max(wall, a1.elapsed_time(a2))
        loop_atoms += md.info()["N"] * loop_steps
        md.close()
    loop_rate = loop_atoms / (loop_ms * 1e-3)
    return {"value": value, "unit": METRIC, "systems": int(len(ns)), "atoms": total, "steps": steps,
            "ms": ms, "atoms_min": int(ns.min()), "atoms_max": int(ns.max()),
            "shape": {"form": "phased (one launch per phase over all systems)" if spl == 0 else
                      "persistent (one CTA per system)", "threads_per_cta": threads, "steps_per_launch": spl,
                      "chosen_by": "emd_batch_tune (40 steps)"},
            "create_s": t_create, "energy_drift_rel_per_1000_max": float(drift.max()),
            "looped_fp64": {"value": loop_rate, "unit": METRIC, "sizes_cells": [int(c) for c in pick],
                            "steps_each": loop_steps,
                            "how": "ExaMiniMD driver, FP64 drop-in, one system at a time (wall time incl. launches)"},
            "speedup_vs_looped_fp64": value / loop_rate,
            "config": "256 fcc LJ systems, rho* 0.8442, N log-uniform in [500, 20000] (seed 20261204), T* 1.44 "
                      "Gaussian velocities, rc 2.5, skin 0.3, every 20, mixed form, CUDA-graph step loop, tuned form"}


def md_row_mean(ctx, nl) -> float:
    """Mean CSR row length from the list's own row counts."""
    import numpy as np
    num = np.empty(max(nl, 1), np.int32)
    from examinimd_gb300._lib import _ip
    st = ctx.lib.emd_neigh_get(ctx.h, _ip(num), None)
    if st != 0:
        return 0.0
    return float(num[:nl].mean())


_JSON_FD = None


def emit(line: dict) -> None:
    """The one JSON line, on the process's original stdout."""
    os.write(_JSON_FD if _JSON_FD is not None else 1, (json.dumps(line) + "\n").encode())


def main():
    global _JSON_FD
    # anything else written to stdout (the library's own prints, buffered C
    # stdio flushed at exit) goes to stderr, so stdout carries one JSON line
    sys.stdout.flush()
    _JSON_FD = os.dup(1)
    os.dup2(2, 1)
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: 1000 LJ steps (about 0.8 s of timed work at LJ-4M, 50 rebuild
    # cycles and several 200 ms clock samples inside the timed region), 20 SNAP
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lj4m", choices=list(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cells", type=int, default=None, help="override the lattice size (profiling cases)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=60)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the full-size force-error / drift check")
    ap.add_argument("--drift-steps", type=int, default=1000)
    ap.add_argument("--no-snap", action="store_true", help="skip the SNAP-W measurement")
    ap.add_argument("--snap-steps", type=int, default=20)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--batch-steps", type=int, default=500)
    ap.add_argument("--no-fit", action="store_true", help="skip the fitting-gradient measurement")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 drop-in sub-block")
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--no-thermo", action="store_true", help="skip the thermo-every-10 sub-block")
    ap.add_argument("--thermo-steps", type=int, default=100)
    ap.add_argument("--fit-evals", type=int, default=5)
    a = ap.parse_args()
    if a.steps is None:
        a.steps = 20 if a.workload == "snapw" else 1000
    if a.warmup < 3:
        sys.exit("--warmup must be >= 3")
    if a.cells:
        kind = "SNAP bcc W" if a.workload == "snapw" else "LJ fcc rho*=0.8442"
        WORKLOADS[a.workload] = dict(cells=a.cells, desc=f"{kind} {a.cells}^3 cells (profiling case)")
    ws, rank, local = dist_env()
    if a.impl == "reference":
        run_reference_arm(a, ws, rank)
        return
    run_gpu_arm(a, ws, rank, local)


if __name__ == "__main__":
    main()
