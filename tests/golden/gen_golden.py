"""Generate the committed golden fixtures from the reference's own tests and
captures. Run once, in a checkout that has the reference project at
REF_ROOT; the outputs under tests/golden/ are what the test suite reads, so
nothing at test time needs the reference.

Sources (paths relative to the reference project):
  rust/crates/svtav1-dsp/src/quant_tables.rs             AC/DC qlookup, 8-bit
  rust/crates/svtav1-encoder/src/bd10_qlookup_tables.rs  AC/DC qlookup, 10-bit
  rust/crates/svtav1-encoder/tests/data/c_dgd_g64_q{20,40}_p6.bin
        post-CDEF 64x64 luma recons dumped from instrumented C SVT-AV1
  rust/docs/captures/gradient_{64x64,128x128}_q{20,40,55}_p6.lrdbg.txt
        per-unit C dumps of the Wiener search (LRNONE/LRWNSOLVE/...)
  rust/docs/captures/m0m5_config_dlf.txt
        C deblock-level hill-climb traces (DLFDBG SEARCH/TRY/STEP/PICK)
  rust/crates/svtav1-encoder/src/cdef.rs (tests)           finish_rd / qp anchors
  rust/crates/svtav1-encoder/src/deblock.rs (tests)        closed-form levels
  rust/crates/svtav1-encoder/src/restoration.rs (tests)    RD constants
  rust/crates/svtav1-encoder/src/pd0.rs (doc comment)      lambda anchors
  rust/crates/svtav1-dsp/src/superres.rs                  normative upscale filter (64 x 8)

Usage: python tests/golden/gen_golden.py [REF_ROOT]
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _table(path, name):
    s = open(path).read()
    i = s.index(name)
    j = s.index("[", s.index("=", i))
    k = s.index("];", j)
    nums = [int(x) for x in re.findall(r"-?\d+", s[j + 1:k])]
    assert len(nums) == 256, (name, len(nums))
    return nums


def _ints(s):
    s = re.sub(r"(?<=\d)[ui](8|16|32|64|size)\b", "", s)  # drop Rust literal suffixes
    return [int(x.replace("_", "")) for x in re.findall(r"-?\d[\d_]*", s)]


def parse_lrdbg(path):
    """Parse one C LR capture into per-plane records."""
    planes = {}
    for line in open(path):
        line = line.strip()
        m = re.match(r"(LR[A-Z]+) (.*)", line)
        if not m:
            continue
        tag, rest = m.groups()
        kv = dict(re.findall(r"(\w+)=(\[[^\]]*\]|\S+)", rest))
        p = int(kv["plane"])
        rec = planes.setdefault(p, {})
        if tag == "LRNONE":
            rec["lim"] = _ints(kv["lim"])
            rec["sse_none"] = int(kv["sse"])
        elif tag == "LRWNSOLVE":
            win = int(kv["win"])
            rec["win"] = win
            # C prints the whole WIENER_WIN-sized vd/hd arrays; only the
            # first `win` entries are written by the solver.
            rec["vd"] = _ints(kv["vd"])[:win]
            rec["hd"] = _ints(kv["hd"])[:win]
            rec["v"] = _ints(kv["v"])
            rec["h"] = _ints(kv["h"])
        elif tag == "LRWNSCORE":
            rec["score"] = int(kv["score"])
        elif tag == "LRWNSEG":
            rec["sse_wn"] = int(kv["sse_wn"])
        elif tag == "LRWNFIN":
            rec["fin"] = {
                "sse_none": int(kv["sse_none"]), "sse_wn": int(kv["sse_wn"]),
                "bits_none": int(kv["bits_none"]), "bits_wn": int(kv["bits_wn"]),
                "cnt_bits": int(kv["cnt_bits"]), "rdmult": int(kv["rdmult"]),
                "cost_none": float(kv["cost_none"]), "cost_wn": float(kv["cost_wn"]),
                "pick": int(kv["pick"]), "refv": _ints(kv["refv"]), "refh": _ints(kv["refh"]),
            }
        elif tag == "LRBEST":
            rec["frame_rtype"] = int(kv["frame_rtype"])
    return planes


def parse_dlf(path):
    cells = []
    cur = None
    for line in open(path):
        line = line.strip()
        m = re.match(r"## DLF search: (\S+)", line)
        if m:
            cur = {"cell": m.group(1), "tries": [], "steps": []}
            cells.append(cur)
            continue
        if cur is None or not line.startswith("DLFDBG"):
            continue
        kv = dict(re.findall(r"(\w+)=(\[[^\]]*\]|\S+)", line))
        if "DLFDBG SEARCH" in line:
            cur["conv_th"] = int(kv["conv_th"])
        elif "DLFDBG TRY" in line:
            cur["tries"].append([int(kv["lvl0"]), int(kv["err"])])
        elif "DLFDBG STEP" in line:
            cur["steps"].append({"mid": int(kv["mid"]), "step": int(kv["step"]), "bias": int(kv["bias"])})
        elif "DLFDBG PICK" in line:
            cur["pick"] = int(kv["filt_best"])
            cur["best_err"] = int(kv["best_err"])
    return cells


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    crates = os.path.join(ref, "rust", "crates")
    caps = os.path.join(ref, "rust", "docs", "captures")
    out = {}

    out["tables"] = {
        "dc8": _table(os.path.join(crates, "svtav1-dsp/src/quant_tables.rs"), "DC_QLOOKUP_8"),
        "ac8": _table(os.path.join(crates, "svtav1-dsp/src/quant_tables.rs"), "AC_QLOOKUP_8"),
        "dc10": _table(os.path.join(crates, "svtav1-encoder/src/bd10_qlookup_tables.rs"),
                       "pub static DC_QLOOKUP_10"),
        "ac10": _table(os.path.join(crates, "svtav1-encoder/src/bd10_qlookup_tables.rs"),
                       "pub static AC_QLOOKUP_10"),
    }

    sr = open(os.path.join(crates, "svtav1-dsp/src/superres.rs")).read()
    i = sr.index("RESIZE_FILTER_NORMATIVE")
    j = sr.index("= [", sr.index("pub static RESIZE_FILTER_NORMATIVE"))
    body = sr[j + 3:sr.index("];", j)]
    taps = [int(x) for x in re.findall(r"-?\d+", body)]
    assert len(taps) == 64 * 8, len(taps)
    out["tables"]["superres_filter"] = [taps[k * 8:(k + 1) * 8] for k in range(64)]

    # Wiener captures. The two 64x64 cells carry their C recon inputs.
    lr = {}
    for size in ("64x64", "128x128"):
        for q in (20, 40, 55):
            name = "gradient_%s_q%d_p6" % (size, q)
            lr[name] = parse_lrdbg(os.path.join(caps, name + ".lrdbg.txt"))
    out["lr_captures"] = lr
    for q in (20, 40):
        src = os.path.join(crates, "svtav1-encoder/tests/data/c_dgd_g64_q%d_p6.bin" % q)
        shutil.copyfile(src, os.path.join(HERE, "c_dgd_g64_q%d_p6.bin" % q))

    out["dlf_traces"] = parse_dlf(os.path.join(caps, "m0m5_config_dlf.txt"))

    # Unit-test anchors, extracted from the reference test bodies.
    cdef_src = open(os.path.join(crates, "svtav1-encoder/src/cdef.rs")).read()
    fin = []
    body = cdef_src[cdef_src.index("fn finish_rd_matches_c_captures"):]
    body = body[:body.index("\n    }\n")]
    for blk in re.finditer(r"let (m\d+) = \[(.*?)\];", body, re.S):
        rows = re.findall(r"row\(\s*\[([^\]]*)\],\s*(\[[^\]]*\]|uvrow)", blk.group(2))
        uvrow = _ints(re.search(r"let uvrow = \[([^\]]*)\]", body).group(1))
        rr = []
        for y, uv in rows:
            rr.append(_ints(y) + (uvrow if uv == "uvrow" else _ints(uv)))
        call = re.search(r"finish_cdef_rd\(&%s, (\d+), (\d+)\),\s*\((\d+), alloc::vec!\[(\d+)\], alloc::vec!\[(\d+)\]\)"
                         % blk.group(1), body)
        n_cand, qidx, bits, l0, l1 = (int(x) for x in call.groups())
        fin.append({"rows": rr, "n_cand": n_cand, "qindex": qidx, "bits": bits, "lev0": [l0], "lev1": [l1]})
    out["cdef_finish"] = fin

    qp = []
    for m in re.finditer(r"pick_cdef_params_key_frame\((\d+), (\d+), false\);\s*assert_eq!\(\s*\(\w+\.damping, \w+\.y_strength, \w+\.uv_strength\),\s*\((\d+), (\d+), (\d+)\)",
                         cdef_src):
        qp.append([int(x) for x in m.groups()])
    ys = re.search(r"for \(q, want_y\) in \[\((\d+)u8, (\d+)u8\), \((\d+), (\d+)\), \((\d+), (\d+)\), \((\d+), (\d+)\), \((\d+), (\d+)\)\]",
                   cdef_src)
    luma_y = [[int(ys.group(i)), int(ys.group(i + 1))] for i in range(1, 11, 2)]
    damp = [[int(a), int(b)] for a, b in
            re.findall(r"pick_cdef_params_key_frame\((\d+), 8, false\)\.damping, (\d+)\)", cdef_src)]
    y52 = [[int(a), int(b), int(c)] for a, b, c in
           re.findall(r"pick_cdef_params_key_frame\((\d+), (\d+), false\)\.y_strength, (\d+)\);", cdef_src)]
    out["cdef_qp"] = {"full": qp, "luma_y_bd8": luma_y, "damping_bd8": damp, "y_strength": y52}

    dbk = open(os.path.join(crates, "svtav1-encoder/src/deblock.rs")).read()
    out["deblock_key_bd8"] = [[int(a)] + _ints(b) for a, b in
                              re.findall(r"pick_filter_levels_key_frame\((\d+), 8\)\.levels,\s*\[([^\]]*)\]", dbk)]

    rst = open(os.path.join(crates, "svtav1-encoder/src/restoration.rs")).read()
    out["restore_cost"] = _ints(re.search(r"wiener_restore_cost\(\), \[([^\]]*)\]", rst).group(1))
    out["rdcost_dbl"] = [[int(a), int(b), int(c), int(d), float(e)] for a, b, c, d, e in
                         re.findall(r"rdcost_dbl\((\d+), (\d+) >> (\d+), (\d+)\), ([\d.]+)\)", rst)]

    pd0 = open(os.path.join(crates, "svtav1-encoder/src/pd0.rs")).read()
    m = re.search(r"Instrumented: (\d+) / (\d+) / (\d+) at\s*/// qindex (\d+)/(\d+)/(\d+)", pd0)
    out["lambda_8bit_unweighted"] = [[int(m.group(4)), int(m.group(1))], [int(m.group(5)), int(m.group(2))],
                                     [int(m.group(6)), int(m.group(3))]]

    dsp_r = open(os.path.join(crates, "svtav1-dsp/src/restoration.rs")).read()
    out["count_units"] = [[int(a), int(b), int(c)] for a, b, c in
                          re.findall(r"count_units_in_tile\((\d+), (\d+)\), (\d+)\)", dsp_r)]

    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
