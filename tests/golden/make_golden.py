"""Regenerates the golden fixtures in tests/golden/ from ExaMiniMD itself.

Requires the ExaMiniMD source tree (--ref, or $EXAMINIMD_SRC as
oracle/build.py resolves it) and builds it against the serial Kokkos shim
(oracle/Makefile.ref).  For every case it runs

  * ref_examinimd -il DECK ... --dumpbinary EVERY DIR  (the reference's own
    binary dumps: id, type, q, x, v, f of the owned atoms), and
  * ref_probe OUT DECK ...  (the reference's binning, ghosts, neighbour rows
    and initial forces right after ExaMiniMD::init),

and stores the selected steps plus the thermo lines in CASE.npz.  For the
DIGEST_CASES (too large for array fixtures) it stores SHA-256 digests of the
same arrays, the dump arrays in the reference's atom order, in
CASE.digest.json.

    python tests/golden/make_golden.py [--ref SRC] [--only CASE]
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.decks import CASES, DIGEST_CASES, digest, read_snap_files, snap_elements, write_case  # noqa: E402


def read_probe(path: str) -> dict:
    out = {}
    with open(path, "rb") as fp:
        while True:
            head = fp.read(32)
            if len(head) < 32:
                break
            name = head.split(b"\0")[0].decode()
            t = fp.read(1).decode()
            (n,) = struct.unpack("q", fp.read(8))
            dt = np.int32 if t == "i" else np.float64
            out[name] = np.frombuffer(fp.read(n * np.dtype(dt).itemsize), dtype=dt).copy()
    return out


def read_dump(path: str) -> dict:
    with open(path, "rb") as fp:
        (n,) = struct.unpack("i", fp.read(4))
        idv = np.frombuffer(fp.read(4 * n), np.int32).copy()
        typ = np.frombuffer(fp.read(4 * n), np.int32).copy()
        q = np.frombuffer(fp.read(8 * n), np.float64).copy()
        x = np.frombuffer(fp.read(24 * n), np.float64).reshape(n, 3).copy()
        v = np.frombuffer(fp.read(24 * n), np.float64).reshape(n, 3).copy()
        f = np.frombuffer(fp.read(24 * n), np.float64).reshape(n, 3).copy()
    return dict(id=idv, type=typ, q=q, x=x, v=v, f=f)


def parse_thermo(stdout: str) -> np.ndarray:
    rows = []
    on = False
    for line in stdout.splitlines():
        if line.startswith("#Timestep"):
            on = True
            continue
        if on:
            m = re.match(r"^(\d+) (\S+) (\S+) (\S+) ", line)
            if m:
                rows.append([float(m.group(i)) for i in range(1, 5)])
            elif line.strip() == "":
                if rows:
                    break
    return np.array(rows)


def make_digest(exe: str, probe: str, name: str, case: dict) -> None:
    """Digests of an LJ case's dumps (kept steps), probe arrays and thermo."""
    import json
    work = tempfile.mkdtemp(prefix="golden_")
    try:
        deck, args = write_case(case, work)
        dump_dir = os.path.join(work, "dump")
        os.makedirs(dump_dir)
        r = subprocess.run([exe, "-il", deck] + args + ["--dumpbinary", str(case["dump_every"]), dump_dir],
                           cwd=work, capture_output=True, text=True, check=True)
        pr = os.path.join(work, "probe.bin")
        subprocess.run([probe, pr, "-il", deck] + args, cwd=work, capture_output=True, text=True, check=True)
        P = read_probe(pr)
        out = dict(case=name, probe={k: digest(v) for k, v in P.items()},
                   probe_counts=[int(v) for v in P["counts"]], probe_nbin=[int(v) for v in P["nbin"]],
                   neigh_total=int(P["num_neighs"].sum()), thermo=parse_thermo(r.stdout).tolist(), steps={})
        for step in case["keep_steps"]:
            d = read_dump(os.path.join(dump_dir, f"output.{step:010d}.000"))
            out["steps"][str(step)] = {k: digest(v) for k, v in d.items()}
        path = os.path.join(HERE, f"{name}.digest.json")
        with open(path, "w") as fp:
            json.dump(out, fp, indent=1)
        print(f"{name}: digests of {len(case['keep_steps'])} dumps, N={P['counts'][0]}, ghosts={P['counts'][1]}")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="ExaMiniMD source tree (default: $EXAMINIMD_SRC)")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    sys.path.insert(0, ROOT)
    from oracle.build import build_reference, reference_source  # noqa: E402

    a.ref = a.ref or reference_source()
    exe = build_reference(a.ref)
    if exe is None:
        sys.exit(f"ExaMiniMD sources not found under {a.ref}")
    probe = os.path.join(os.path.dirname(exe), "ref_probe")
    for name, case in DIGEST_CASES.items():
        if a.only and name != a.only:
            continue
        make_digest(exe, probe, name, case)
    for name, case in CASES.items():
        if a.only and name != a.only:
            continue
        work = tempfile.mkdtemp(prefix="golden_")
        try:
            snap = None
            if case["kind"] == "snap":
                sd = os.path.join(a.ref, "input", "snap")
                if "synthetic_second" in case:
                    # the shipped Ta06A numbers as element A, a seeded variant as element B
                    base = read_snap_files(os.path.join(sd, "Ta06A.snapcoeff"), os.path.join(sd, case["param"]))
                    sp = case["synthetic_second"]
                    rng = np.random.default_rng(sp["seed"])
                    beta_b = [b * sp["scale"] + float(rng.normal(0.0, 0.01)) for b in base["beta"]]
                    snap = dict(elements=[dict(name="A", radius=base["radius"], weight=base["weight"],
                                               beta=base["beta"]),
                                          dict(name="B", radius=sp["radius"], weight=sp["weight"], beta=beta_b)],
                                params=base["params"])
                else:
                    snap = read_snap_files(os.path.join(sd, case["coeff"]), os.path.join(sd, case["param"]))
            deck, args = write_case(case, work, snap)
            dump_dir = os.path.join(work, "dump")
            os.makedirs(dump_dir)
            r = subprocess.run([exe, "-il", deck] + args + ["--dumpbinary", str(case["dump_every"]), dump_dir],
                               cwd=work, capture_output=True, text=True, check=True)
            thermo = parse_thermo(r.stdout)
            pr = os.path.join(work, "probe.bin")
            subprocess.run([probe, pr, "-il", deck] + args, cwd=work, capture_output=True, text=True, check=True)
            P = read_probe(pr)
            data = {f"probe_{k}": v for k, v in P.items()}
            data["thermo"] = thermo
            for step in case["keep_steps"]:
                d = read_dump(os.path.join(dump_dir, f"output.{step:010d}.000"))
                for k, v in d.items():
                    data[f"s{step}_{k}"] = v
            data["keep_steps"] = np.array(case["keep_steps"], np.int32)
            if snap is not None:
                elems = snap_elements(snap)
                data["snap_elem"] = np.array(elems[0]["name"])
                data["snap_radius"] = np.array(elems[0]["radius"])
                data["snap_weight"] = np.array(elems[0]["weight"])
                data["snap_beta"] = np.array(elems[0]["beta"])
                data["snap_elems"] = np.array([e["name"] for e in elems])
                data["snap_radii"] = np.array([e["radius"] for e in elems])
                data["snap_weights"] = np.array([e["weight"] for e in elems])
                data["snap_betas"] = np.array([e["beta"] for e in elems])
                data["snap_param_keys"] = np.array(list(snap["params"].keys()))
                data["snap_param_vals"] = np.array(list(snap["params"].values()))
            out = os.path.join(HERE, f"{name}.npz")
            np.savez_compressed(out, **data)
            print(f"{name}: {os.path.getsize(out) / 1024:.1f} KiB, N={len(data['s0_id'])}, "
                  f"ghosts={P['counts'][1]}, thermo rows={len(thermo)}")
        finally:
            shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
