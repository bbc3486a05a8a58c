"""Benchmark of the GB300 ExaMiniMD hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload lj4m|lj32k] [--precision mixed|fp64]

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
}
METRIC = "atom-steps/s"


def deck_text(cells: int, steps: int, mass=1.0, temp=1.44) -> str:
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
thermo 0
run {steps}
"""


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return dict(hbm_gbs=float(d["hbm_gbs"]), src="measured")
    return dict(hbm_gbs=6800.0, src="fallback")


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
    warm = max(0, min(a.warmup, 2))
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
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def algorithmic_bytes_per_atom(precision: str, mean_row: float) -> float:
    """Bytes one atom's force evaluation must move: its CSR row entries (4 B
    each), row metadata (length + start, 8 B), its own position (FP32 float4
    16 B for mixed, double4 32 B for FP64), the force read + write (48 B)."""
    pos = 16.0 if precision == "mixed" else 32.0
    return 4.0 * mean_row + 8.0 + pos + 48.0


def run_gpu_arm(a, ws, rank, local):
    import numpy as np
    import torch

    from examinimd_gb300 import MD

    dist = init_pg(ws, True)
    torch.cuda.set_device(local)
    wl = WORKLOADS[a.workload]
    tmp = tempfile.mkdtemp(prefix="emdbench_")
    deck = os.path.join(tmp, "in.lj")
    with open(deck, "w") as fp:
        fp.write(deck_text(wl["cells"], a.steps))
    md = MD(["-il", deck, "--quiet", "--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
             "--comm-type", "SERIAL", "--precision", a.precision, "--device", str(local)])
    ctx = md.ctx
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    N = md.info()["N"]
    # warm-up (complete rebuild cycles so the timed region starts right after a build)
    md.run(a.warmup)
    ctx.synchronize()
    ctx.timing(True)
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
    ctx.timing(False)
    launches = sum(c for _, c in rep.values())
    value = ws * N * a.steps / (ms_max * 1e-3)

    # dominant kernel roofline
    kname = "lj_full_mixed" if a.precision == "mixed" else "lj_full_fp64"
    kms, kn = rep.get(kname, (0.0, 0))
    nl = md.info()["N_local"]
    mean_row = float(md_row_mean(ctx, nl))
    bytes_launch = algorithmic_bytes_per_atom(a.precision, mean_row) * nl
    peaks = load_peaks()
    achieved = bytes_launch / (kms / kn * 1e-3) / 1e9 if kn else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath))
        ent = tj.get(f"{kname}@{a.workload}")
        if ent:
            traffic = ent.get("bytes_per_launch")
    roof = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None, "traffic": traffic,
            "peak_source": peaks["src"], "bytes_per_launch": bytes_launch, "mean_row": mean_row,
            "launch_ms": (kms / kn) if kn else None}
    kernels = {k: {"ms": v[0], "launches": v[1], "share": v[0] / max(1e-12, sum(x[0] for x in rep.values()))}
               for k, v in sorted(rep.items(), key=lambda kv: -kv[1][0])}

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
    for _ in range(e2e_steps):
        n_now = md.info()["N_local"]
        assert lib.emd_system_update(ctx.h, 0, n_now, _dp(hx), _dp(hv), _dp(hf)) == 0
        md.run(1)
        assert lib.emd_system_get(ctx.h, 0, n_now, _dp(hx), _dp(hv), _dp(hf), None, None, None) == 0
    ctx.synchronize()
    t_e2e = reduce_max(dist, time.perf_counter() - t0)
    barrier(dist)
    e2e = {"value": ws * N * e2e_steps / t_e2e, "unit": METRIC, "h2d_bytes_per_step": int(nl * 72),
           "d2h_bytes_per_step": int(nl * 72), "steps": e2e_steps,
           "path": "emd_system_update (x,v,f pinned H2D) + one ExaMiniMD step + emd_system_get (x,v,f D2H)"}
    T, pe, ke = md.thermo(recompute=True)

    extra = {}
    if rank == 0 and not a.no_cpu:
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
                "data": "synthetic (fcc lattice, ExaMiniMD loop-geom velocities)",
                "config": {"workload": a.workload, "desc": wl["desc"], "atoms_per_gpu": N, "precision": a.precision,
                           "neigh": "CSR full", "parallelism": f"replicas{ws}",
                           "l2": "working set (positions, forces, 1.2 GB neighbour list) > 129 MB L2; no flush"},
                "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "thermo_end": {"T": T, "PE_per_atom": pe, "KE_per_atom": ke}, "kernels": kernels}
        line.update(extra)
        print(json.dumps(line), flush=True)
    md.close()
    if dist is not None:
        dist.destroy_process_group()


def md_row_mean(ctx, nl) -> float:
    """Mean CSR row length from the list's own row counts."""
    import numpy as np
    num = np.empty(max(nl, 1), np.int32)
    from examinimd_gb300._lib import _ip
    st = ctx.lib.emd_neigh_get(ctx.h, _ip(num), None)
    if st != 0:
        return 0.0
    return float(num[:nl].mean())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lj4m", choices=list(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cells", type=int, default=None, help="override the lattice size (profiling cases)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args()
    if a.warmup < 3:
        sys.exit("--warmup must be >= 3")
    if a.cells:
        WORKLOADS[a.workload] = dict(cells=a.cells, desc=f"LJ fcc rho*=0.8442 {a.cells}^3 cells (profiling case)")
    ws, rank, local = dist_env()
    if a.impl == "reference":
        run_reference_arm(a, ws, rank)
        return
    run_gpu_arm(a, ws, rank, local)


if __name__ == "__main__":
    main()
