"""The row-schedule autotuner: fits csrc/sched_table.h from timings on the GPU.

Every BSR product (K in FP64; each level's A, prolongation and restriction in FP32) runs with one
of two row schedules (csrc/spmv_row.cuh): a warp per block row, or five block rows per warp.
The two add a row's blocks in different orders and group the fused reductions of the
conjugate-gradient products differently, so the library takes the schedule from a committed
table - a function of the operator's mean blocks per row - and never from a timing at run time. This
script makes that table: it assembles the workloads below with the library's timing log on
(SVXG_TUNE_LOG=1, set before the library loads), collects both schedules' times for every
operator, and for each kind of operator picks the bound on mean blocks per row (five rows per
warp at or below it) that minimizes the summed time over all of them.

    python -m opus_destruct_2_gb300.autotune [--write] [--out summary.txt]

--write rewrites csrc/sched_table.h; the library must then be rebuilt (__graft_entry__.build()).
"""
from __future__ import annotations

import argparse
import ctypes
import os
import sys

KINDS = ("K (FP64)", "A (FP32)", "prolongation (FP32)", "restriction (FP32)")


class TuneEntry(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("level", ctypes.c_int32), ("rows", ctypes.c_int64),
                ("blocks", ctypes.c_int64), ("ms_warp_row", ctypes.c_float), ("ms_group_row", ctypes.c_float)]


def collect(workloads=None):
    """[(kind, level, rows, blocks, ms_warp_row, ms_group_row)] over every operator assembled."""
    if "opus_destruct_2_gb300" in sys.modules and getattr(sys.modules["opus_destruct_2_gb300"], "_lib", None):
        raise RuntimeError("the library is loaded already: run the autotuner in a fresh process")
    os.environ["SVXG_TUNE_LOG"] = "1"
    from . import StressProblem, load_library, synth
    from .graph import StressOptions, default_materials

    L = load_library()
    L.svxg_debug_tune_log.restype = ctypes.c_int32
    L.svxg_debug_tune_log.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                      ctypes.POINTER(ctypes.c_int32)]
    mats = default_materials()
    if workloads is None:
        workloads = [synth.city_graph(lots_x=4, lots_y=4, seed=5)[:2], synth.city_graph(lots_x=8, lots_y=8, seed=2)[:2],
                     synth.tower_graph(storeys=10, seed=1)[:2]]
        workloads += [g[:2] for g in synth.batch_graphs(24, median=600, hi=20000, seed=11)]
    rows = []
    for nodes, bonds in workloads:
        G = StressProblem(nodes, bonds, mats)
        if not G.assemble(StressOptions()):
            continue
        cnt = ctypes.c_int32(0)
        L.svxg_debug_tune_log(G._h, None, 0, ctypes.byref(cnt))
        buf = (TuneEntry * max(cnt.value, 1))()
        L.svxg_debug_tune_log(G._h, buf, cnt.value, ctypes.byref(cnt))
        rows += [(e.kind, e.level, e.rows, e.blocks, e.ms_warp_row, e.ms_group_row) for e in buf[:cnt.value]]
        del G
    return rows


def fit(rows):
    """Per kind: (bound, summed ms with it, ms all warp-row, ms all group-row, ms of the best per operator)."""
    out = {}
    for k in range(4):
        ops = [(b / r, w, g) for kind, _, r, b, w, g in rows if kind == k and r > 0]
        if not ops:
            continue
        cands = sorted({0.0} | {m for m, _, _ in ops} | {1e9})
        best = None
        for t in cands:
            tot = sum(g if m <= t else w for m, w, g in ops)
            if best is None or tot < best[1] - 1e-9:
                best = (t, tot)
        out[k] = (best[0], best[1], sum(w for _, w, _ in ops), sum(g for _, _, g in ops),
                  sum(min(w, g) for _, w, g in ops), len(ops))
    return out


def write_table(bounds, path=None):
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "sched_table.h")
    vals = [bounds.get(k, 8.0) for k in range(4)]
    text = open(path).read()
    start = text.index("constexpr double kGroupRowMaxMean[4] = {")
    end = text.index("};", start) + 2
    lit = ", ".join(f"{v:.4g}" if v < 1e8 else "1e9" for v in vals)
    text = text[:start] + f"constexpr double kGroupRowMaxMean[4] = {{{lit}}};" + text[end:]
    with open(path, "w") as f:
        f.write(text)
    return path


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--write", action="store_true", help="rewrite csrc/sched_table.h")
    ap.add_argument("--out", default=None, help="also write the summary to this file")
    a = ap.parse_args(argv)
    rows = collect()
    res = fit(rows)
    lines = [f"{len(rows)} operators timed (three products per schedule each)",
             "kind | operators | bound (mean blocks/row) | ms chosen | ms all warp-row | ms all group-row | ms best each"]
    for k, (t, tot, w, g, b, n) in sorted(res.items()):
        lines.append(f"{KINDS[k]} | {n} | {t:.4g} | {tot:.3f} | {w:.3f} | {g:.3f} | {b:.3f}")
    lines.append("per operator: kind level rows blocks mean ms_warp_row ms_group_row")
    for kind, lev, r, bl, w, g in rows:
        lines.append(f"{kind} {lev} {r} {bl} {bl / max(r, 1):.2f} {w:.4f} {g:.4f}")
    text = "\n".join(lines)
    print(text)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")
    if a.write:
        print("wrote", write_table({k: v[0] for k, v in res.items()}))


if __name__ == "__main__":
    main()
