"""Floating-point operation count of one SNAP force evaluation, per atom.

The count enumerates the loops of the GB300 kernel (`csrc/snap_kernel.cuh`)
for a given twojmax and number of inside neighbours, phase by phase, with one
operation per add, subtract or multiply (a fused multiply-add counts two) and
one per square root, division or transcendental call.  It counts the
formulation the kernel runs (the adjoint form with reverse-mode pair forces),
which needs fewer operations than the reference's
(compute_ui / compute_zi / compute_duidrj / compute_dbidrj, sna_impl.hpp).

`snap_flops(twojmax, ninside)` returns a dict of per-atom counts by phase and
by arithmetic type for each precision form:

- B, the U_tot recursion and its sums, is FP64 in both forms;
- the per-neighbour scalars are FP64 in both forms;
- C (Z and Y) and D (the pair forces) are FP32 in the mixed form and FP64 in
  the FP64 form; the FP64 tail of D (repulsion, scatter, sum for i) is FP64.
"""
from __future__ import annotations


def _triples(J: int):
    """Full (j1 >= j2, j) triples of the Z contraction (SNA::build_indexlist)."""
    for j1 in range(J + 1):
        for j2 in range(j1 + 1):
            for j in range(abs(j1 - j2), min(J, j1 + j2) + 1, 2):
                yield j1, j2, j


def _nh(j: int) -> int:
    """Elements of the half layer of j (mb <= j / 2)."""
    return (j + 1) * (j // 2 + 1)


def z_loop_counts(J: int) -> tuple[int, int, int]:
    """(jobs, outer iterations, inner iterations) of the Z contraction."""
    jobs = outer = inner = 0
    for j1, j2, j in _triples(J):
        for mb in range(j // 2 + 1):
            for ma in range(j + 1):
                jobs += 1
                ma1lo = max(0, (2 * ma - j - j2 + j1) // 2)
                ma1hi = min(j1, (2 * ma - j + j2 + j1) // 2)
                mb1lo = max(0, (2 * mb - j - j2 + j1) // 2)
                mb1hi = min(j1, (2 * mb - j + j2 + j1) // 2)
                na, nb = max(0, ma1hi - ma1lo + 1), max(0, mb1hi - mb1lo + 1)
                outer += na
                inner += na * nb
    return jobs, outer, inner


def snap_flops(twojmax: int, ninside: float) -> dict:
    """Per-atom operation counts of one force evaluation (see the module doc)."""
    J, n = twojmax, float(ninside)
    half = sum(_nh(j) for j in range(1, J + 1))  # half-layer elements, layers 1..J
    nyh = sum(_nh(j) for j in range(J + 1))
    # per-neighbour scalars (mixed form's closed forms; the FP64 form's
    # reference formulas are within a few operations of it): r, two sincos,
    # two divisions, a, b and their twelve derivatives, the switching function
    # and the r^-12 repulsion
    scalars = n * 80.0
    # B: 14 per element per neighbour (two complex multiply-adds), the layer
    # sums (2 per neighbour per element incl. layer 0) and the 1/f scaling
    b_stage = n * 14.0 * half + n * 2.0 * nyh + 4.0 * nyh
    # C: Z (complex product 6, CG scale 2, accumulate 2 per inner; 4 per
    # outer), Y (4 per job, 2 for the w / f scale per element)
    jobs, outer, inner = z_loop_counts(J)
    c_stage = 10.0 * inner + 4.0 * outer + 4.0 * jobs + 2.0 * nyh
    # D (reverse mode), per neighbour: forward 14 + 4 (Phi) per half element,
    # adjoint 18 per half element and 16 per gathered layer-(j-1) element,
    # then the pair force (3 components of about ten) and the lane sums
    gathered = sum(j * (j // 2 + 1) for j in range(2, J + 1))
    d_sweeps = n * (18.0 * half + 18.0 * half + 16.0 * gathered + 31.0 + 3 * 31.0)
    d_tail = n * (3.0 + 3.0 + 12.0)  # repulsion add, scatter, sum for i (FP64)
    total = scalars + b_stage + c_stage + d_sweeps + d_tail
    return {
        "twojmax": J,
        "ninside": n,
        "phases": {"scalars": scalars, "B": b_stage, "C": c_stage, "D": d_sweeps + d_tail},
        "total": total,
        "fp64": {"mixed": scalars + b_stage + d_tail, "fp64": total},
        "fp32": {"mixed": c_stage + d_sweeps, "fp64": 0.0},
    }


__all__ = ["snap_flops", "z_loop_counts"]
