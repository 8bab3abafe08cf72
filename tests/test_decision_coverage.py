"""CPU check of the decision-branch frames of tests/test_gpu_decisions.py:
on the oracle, each frame takes the branch it is named for, and together
they take every branch the GPU parity suite has to compare -- a non-zero
deblock level search outcome at 8 and 10 bits, cdef_bits 1, 2 and 3, a
restoration plane mixing WIENER and NONE units and a plane of type NONE."""
import pytest

from test_gpu_decisions import BRANCHES, frame, lr_mixed, lr_plane_none


@pytest.mark.parametrize("case", BRANCHES, ids=[c[0] for c in BRANCHES])
def test_frame_takes_its_branch(oracle, case):
    name, args, taken = case
    d = oracle.filter_stage(frame(*args))[0]
    assert taken(d), d


def test_branch_coverage_complete(oracle):
    seen = {"lf8": False, "lf10": False, "bits": set(), "mixed": False, "none": False}
    for name, args, _ in BRANCHES:
        d = oracle.filter_stage(frame(*args))[0]
        if d["lf"][0] > 0 and args[5] <= 5:
            seen["lf10" if args[3] == 10 else "lf8"] = True
        seen["bits"].add(d["cdef_bits"])
        seen["mixed"] |= lr_mixed(d)
        seen["none"] |= lr_plane_none(d)
    assert seen["lf8"] and seen["lf10"] and seen["mixed"] and seen["none"]
    assert {1, 2, 3} <= seen["bits"]


def test_oracle_trace_lines(oracle, tmp_path):
    """The oracle's trace has the reference's line kinds in order: the
    deblock climb, the CDEF rows and pick, then the restoration units."""
    path = str(tmp_path / "t.txt")
    oracle.trace(path)
    try:
        oracle.filter_stage(frame(11, 256, 192, 8, 30, 4, "cosine"))
    finally:
        oracle.trace(None)
    lines = open(path).read().splitlines()
    kinds = [l.split()[0] for l in lines]
    assert kinds[0] == "DLF_TRY" and "DLF_PICK" in kinds
    assert kinds.index("RS_CDEF_FB") > kinds.index("DLF_PICK")
    assert kinds.index("LRNONE") > kinds.index("RS_CDEF_PICK")
    assert all(l.startswith("DLF_TRY plane=0 lvl0=") for l in lines[:2])
