"""Autotuner of the aggregation's launch shape on the GPU it runs on.

The aggregation (sgm_kernel) runs bands of R image rows per CTA; R sets the number of work items, the wavefront
lag between bands and how many row warps share an SM. The library's planner predicts a good R from a model of
the persistent schedule; this tuner measures instead. For each class (d-stride dp, padded height bucket) it
times the aggregation stage of a representative synthetic rig at every band height that fits the SM (median of
several computes, CUDA events around the stage), and writes the fastest R per class as a C++ table:

    python -m sister_gb300.autotune --out sister_gb300/csrc/tuned_gb300.h

The table is compiled into the library; sgm_plan uses it on a 152-SM device and falls back to the model for
geometries outside the table's classes (or with SISTER_TUNE_SGM_ROWS set).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import sys
import time

# (dp, lower and upper bound of the padded height Hp of the class, representative rig w x h x dc)
CLASSES = [
    (64, 0, 768, (480, 352, 64)), (64, 768, 1536, (1024, 768, 64)), (64, 1536, 1 << 30, (1920, 1600, 64)),
    (128, 0, 768, (640, 480, 128)), (128, 768, 1536, (1280, 960, 128)), (128, 1536, 1 << 30, (2048, 1600, 128)),
    (192, 0, 1024, (640, 480, 192)), (192, 1024, 1792, (1280, 1008, 192)), (192, 1792, 1 << 30, (2048, 1600, 192)),
    (256, 0, 1024, (640, 480, 256)), (256, 1024, 1792, (1920, 1080, 256)), (256, 1792, 1 << 30, (2448, 2048, 256)),
    (384, 0, 1536, (1024, 720, 320)), (384, 1536, 1 << 30, (2048, 1600, 384)),
    (512, 0, 2048, (1280, 960, 512)), (512, 2048, 1 << 30, (2448, 2048, 512)),
]


def time_rows(ctx, rows: int, reps: int) -> float:
    import sister_gb300 as sg

    ctx.tune_set(sg.TUNE_SGM_ROWS, rows)
    ctx.compute_device(ctx._out_ptr)
    ctx.synchronize()
    ms = []
    for _ in range(reps):
        ctx.compute_device(ctx._out_ptr)
        agg = [t for name, t in ctx.profile_read() if name == "aggregate"]
        if agg:
            ms.append(agg[0])
    ctx.synchronize()
    return statistics.median(ms)


def tune(device: int = 0, reps: int = 5, classes=CLASSES, log=print):
    import torch
    import sister_gb300 as sg
    from sister_gb300 import synth

    results = []
    for dp, lo, hi, (w, h, dc) in classes:
        views, _ = synth.make_rig(w, h, max(dc // 9, 2), max(dc - 16, 8), seed=77, tiles=10)
        dev = [torch.from_numpy(v).cuda(device) for v in views]
        out = torch.empty((h, w), dtype=torch.int16, device="cuda:%d" % device)
        ctx = sg.Context(device)
        ctx.load_views_device([t.data_ptr() for t in dev], w, h, w, 1)
        ctx.set_max_disparity(dc)
        ctx._out_ptr = out.data_ptr()
        ctx.profile(True)
        model_rows = ctx.tune_get(sg.TUNE_SGM_ROWS)
        times = {}
        for rows in range(2, 17):
            ctx.tune_set(sg.TUNE_SGM_ROWS, rows)
            if ctx.tune_get(sg.TUNE_SGM_ROWS) != rows:  # does not fit the SM: the planner clamped it
                continue
            times[rows] = time_rows(ctx, rows, reps)
        best = min(times, key=times.get)
        ctx.close()
        del dev, out
        torch.cuda.empty_cache()
        rec = {"dp": dp, "hp_lo": lo, "hp_hi": hi, "rig": [w, h, dc], "best_rows": best, "best_ms": times[best],
               "model_rows": model_rows, "model_ms": times.get(model_rows), "ms_by_rows": times}
        log(json.dumps(rec))
        results.append(rec)
    return results


def write_header(results, path: str, device_name: str):
    lines = [
        "// Generated by python -m sister_gb300.autotune on %s (%s). Do not edit by hand." % (device_name,
                                                                                           time.strftime("%Y-%m-%d")),
        "// Fastest measured band height of the aggregation per (d-stride, padded height) class; sgm_plan uses it on",
        "// a 152-SM device. Columns: dp, padded height range [lo, hi), rows per band; measured ms of the",
        "// representative rig at the best and at the model's band height in the trailing comment.",
        "#pragma once",
        "namespace sister {",
        "struct TunedRows {",
        "    int dp, hp_lo, hp_hi, rows;",
        "};",
        "constexpr TunedRows kTunedRows[] = {",
    ]
    for r in results:
        lines.append("    {%d, %d, %d, %d}, // %dx%dx%d: %.3f ms (model R=%d: %s ms)" % (
            r["dp"], r["hp_lo"], min(r["hp_hi"], 1 << 30), r["best_rows"], *r["rig"], r["best_ms"],
            r["model_rows"], "%.3f" % r["model_ms"] if r["model_ms"] else "n/a"))
    lines += ["    {0, 0, 0, 0}, // end", "};", "} // namespace sister", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default=None, help="write the C++ table here")
    ap.add_argument("--json", default=None, help="write the measurements here")
    args = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    from sister_gb300 import build

    build.build()
    torch.cuda.set_device(args.device)
    res = tune(args.device, args.reps)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(res, f, indent=1)
    if args.out:
        write_header(res, args.out, torch.cuda.get_device_name(args.device))


if __name__ == "__main__":
    main()
