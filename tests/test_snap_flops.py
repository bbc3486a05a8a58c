"""The SNAP operation counter used by bench.py's SNAP roofline (CPU)."""
from examinimd_gb300.snap_flops import snap_flops, z_loop_counts


def test_z_loop_counts_match_the_kernel_tables():
    # 2J = 8: 125 full triples, 2386 Z jobs (the kernel's job table), and
    # the inner/outer trip counts of compute_zi's loops over them
    assert z_loop_counts(8) == (2386, 9028, 41889)
    # 2J = 2: triples (0,0,0) (1,0,1) (1,1,0) (1,1,2) (2,0,2) (2,1,1) (2,2,0)
    # (2,2,2), half grids of 1, 2, 1, 6, 6, 2, 1, 6 elements
    assert z_loop_counts(2)[0] == 25


def test_phases_add_up_and_split_by_form():
    d = snap_flops(8, 26)
    assert abs(sum(d["phases"].values()) - d["total"]) < 1e-6 * d["total"]
    assert abs(d["fp64"]["mixed"] + d["fp32"]["mixed"] - d["total"]) < 1e-6 * d["total"]
    assert d["fp64"]["fp64"] == d["total"] and d["fp32"]["fp64"] == 0.0
    # the adjoint formulation: well under the reference formulation's ~1.8 MFLOP
    assert 0.5e6 < d["total"] < 1.0e6
    # linear in the neighbour count except for the per-atom Z / Y contraction
    assert snap_flops(8, 52)["total"] - d["total"] > 0
