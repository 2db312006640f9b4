"""The committed GB300 tuning file (fft_demo_gb300/tuning/gb300.json) names
only tile variants and four-step splits the library builds (CPU: the
kernel registration units and the JSON are read as text, no GPU needed).

Keys: "precision/pass kind/log2 pass length" -> tile (0 small, 1 big, 2 mid,
3 narrow) and "split/precision/log2 n" -> log2 of the column-pass length."""
import json
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "fft_demo_gb300", "csrc")
PATH = os.path.join(REPO, "fft_demo_gb300", "tuning", "gb300.json")

F16, SPLIT = 0, 1
ROW, COL, ROWT = 0, 1, 2
TILES = {"kTileSmall": 0, "kTileBig": 1, "kTileMid": 2, "kTileNarrow": 3}
# registration function -> (precision, pass kind) of its table argument(s)
TABLES = {
    "register_row_kernels": {"tab": (F16, ROW)},
    "register_col_kernels": {"tab": (F16, COL)},
    "register_rowt_kernels": {"tab": (F16, ROWT)},
    "register_split_row_kernels": {"tab": (SPLIT, ROW)},
    "register_split_col_kernels": {"tab": (SPLIT, COL)},
    "register_split_rowt_kernels": {"tab": (SPLIT, ROWT)},
    "register_split_mid_kernels": {"row": (SPLIT, ROW), "col": (SPLIT, COL), "rowt": (SPLIT, ROWT)},
    "register_f16_narrow_kernels": {"row": (F16, ROW), "col": (F16, COL), "rowt": (F16, ROWT)},
    "register_split_pf_kernels": {"row": (SPLIT, ROW), "col": (SPLIT, COL), "rowt": (SPLIT, ROWT)},
}


def built_variants():
    """(precision, kind, log2 L) -> set of tiles registered in kernels_*.cu."""
    out = {}
    seen = set()
    for fname in sorted(os.listdir(CSRC)):
        if not (fname.startswith("kernels_") and fname.endswith(".cu")):
            continue
        src = open(os.path.join(CSRC, fname)).read()
        for fm in re.finditer(r"void (register_\w+)\(([^)]*)\) \{(.*?)\n\}", src, re.S):
            name, body = fm.group(1), fm.group(3)
            if name not in TABLES:
                continue
            seen.add(name)
            for m in re.finditer(r"fill_(?:pf_|split_pf_|split_)?entry<(\d+),[^>]*>\((\w+), (kTile\w+)\)", body):
                prec, kind = TABLES[name][m.group(2)]
                logl = int(m.group(1)).bit_length() - 1
                out.setdefault((prec, kind, logl), set()).add(TILES[m.group(3)])
    assert seen == set(TABLES), set(TABLES) - seen
    return out


def test_registration_parsed():
    b = built_variants()
    # spot checks against the kernel files
    assert 3 in b[(F16, ROW, 12)] and 2 in b[(F16, ROW, 13)] and 3 not in b.get((F16, ROW, 13), set())
    assert 2 in b[(SPLIT, ROW, 12)] and 2 in b[(SPLIT, COL, 9)] and 2 not in b.get((SPLIT, ROWT, 7), set())
    assert 3 in b[(SPLIT, ROW, 10)] and 3 in b[(SPLIT, COL, 10)] and 3 not in b.get((SPLIT, ROWT, 7), set())


def test_tuning_file_names_built_variants():
    data = json.load(open(PATH))
    assert list(data) == ["NVIDIA GB300"]
    built = built_variants()
    entries = data["NVIDIA GB300"]
    assert entries
    for key, val in entries.items():
        parts = key.split("/")
        if parts[0] == "split":
            prec, logn = int(parts[1]), int(parts[2])
            assert prec in (F16, SPLIT) and 15 <= logn <= 24, key
            pass_max = 12 if prec == F16 else 11
            a = int(val)
            assert 4 <= a and 4 <= logn - a <= pass_max, (key, val)
            assert (prec, COL, a) in built and (prec, ROWT, logn - a) in built, (key, val)
        else:
            prec, kind, logl = (int(p) for p in parts)
            assert int(val) in built.get((prec, kind, logl), set()), (key, val)


def test_autotuner_pass_chain_matches_plan_rule():
    """autotune.passes_of (the passes the tuner times) follows the plan's
    built-in rule in capi.cu: single pass up to 2^14 (FP16) / 2^13 (split),
    else a column pass of 2^a and a transposing pass of 2^(log n - a) with
    a = min(log n / 2, 10), raised until the row pass is <= 2^12 / 2^11."""
    from fft_demo_gb300 import FP16, SPLIT_FP32
    from fft_demo_gb300.autotune import passes_of, PASS_COL, PASS_ROW, PASS_ROWT
    assert passes_of(1 << 14, FP16) == [(PASS_ROW, 14)]
    assert passes_of(1 << 15, FP16) == [(PASS_COL, 7), (PASS_ROWT, 8)]
    assert passes_of(1 << 20, FP16) == [(PASS_COL, 10), (PASS_ROWT, 10)]
    assert passes_of(1 << 24, FP16) == [(PASS_COL, 12), (PASS_ROWT, 12)]
    assert passes_of(1 << 13, SPLIT_FP32) == [(PASS_ROW, 13)]
    assert passes_of(1 << 14, SPLIT_FP32) == [(PASS_COL, 7), (PASS_ROWT, 7)]
    assert passes_of(1 << 22, SPLIT_FP32) == [(PASS_COL, 11), (PASS_ROWT, 11)]
    assert passes_of(1 << 20, SPLIT_FP32, split=9) == [(PASS_COL, 9), (PASS_ROWT, 11)]
    assert passes_of(0, FP16, dims=2, shape2d=(1024, 512)) == [(PASS_ROW, 9), (PASS_COL, 10)]
    # the same constants in the plan code
    src = open(os.path.join(CSRC, "capi.cu")).read()
    assert "const int single_max = precision == TCFFT_FP16 ? kMaxLogL : 13;" in src
    assert "const int pass_max = precision == TCFFT_FP16 ? 12 : 11;" in src
    assert "int a = logn / 2 < 10 ? logn / 2 : 10;" in src
    assert "constexpr int kMaxLogL = 14;" in open(os.path.join(CSRC, "passes.cuh")).read()
