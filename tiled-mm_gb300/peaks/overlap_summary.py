"""Summary of a copy/compute timeline written by overlap_trace.cpp: per marked call, the
device time the copy engines (H2D, D2H) and the kernels were busy (union of their intervals),
how much of the copy time ran under kernels, and per-stream busy time.

    python tiled-mm_gb300/peaks/overlap_summary.py gpurun_out/trace_native4096.csv"""
from __future__ import annotations

import csv
import sys
from collections import defaultdict


def union(iv):
    iv = sorted(iv)
    out = []
    for s, e in iv:
        if out and s <= out[-1][1]:
            out[-1][1] = max(out[-1][1], e)
        else:
            out.append([s, e])
    return out


def length(u):
    return sum(e - s for s, e in u)


def intersect(u, v):
    i = j = 0
    total = 0
    while i < len(u) and j < len(v):
        s, e = max(u[i][0], v[j][0]), min(u[i][1], v[j][1])
        if e > s:
            total += e - s
        if u[i][1] < v[j][1]:
            i += 1
        else:
            j += 1
    return total


def clip(iv, lo, hi):
    return [(max(s, lo), min(e, hi)) for s, e in iv if e > lo and s < hi]


def summarise(path: str) -> str:
    rows = list(csv.DictReader(open(path)))
    marks = sorted((int(r["start_ns"]), r["name"]) for r in rows if r["what"] == "mark")
    begins = {name.split()[1]: t for t, name in marks if name.startswith("begin")}
    ends = {name.split()[1]: t for t, name in marks if name.startswith("end")}
    acts = [r for r in rows if r["what"] in ("kernel", "memcpy")]
    lines = ["| call | span ms | kernels busy ms | H2D busy ms | D2H busy ms | copies busy ms | copies under "
             "kernels ms | copy time hidden | H2D GB/s while busy |",
             "|---|---|---|---|---|---|---|---|---|"]
    per_stream_total = defaultdict(float)
    for key in sorted(begins, key=int):
        lo, hi = begins[key], ends.get(key)
        if hi is None:
            continue
        kern = union(clip([(int(r["start_ns"]), int(r["end_ns"])) for r in acts if r["what"] == "kernel"], lo, hi))
        h2d_iv = [(int(r["start_ns"]), int(r["end_ns"])) for r in acts if r["what"] == "memcpy" and r["name"] == "H2D"]
        h2d = union(clip(h2d_iv, lo, hi))
        d2h = union(clip([(int(r["start_ns"]), int(r["end_ns"])) for r in acts
                          if r["what"] == "memcpy" and r["name"] == "D2H"], lo, hi))
        cp = union(h2d + d2h)
        h2d_bytes = sum(int(r["bytes"]) for r in acts if r["what"] == "memcpy" and r["name"] == "H2D"
                        and lo <= int(r["start_ns"]) < hi)
        inside = [r for r in acts if lo <= int(r["start_ns"]) < hi]
        span = (max(int(r["end_ns"]) for r in inside) - min(int(r["start_ns"]) for r in inside)) if inside else 0
        for r in inside:
            per_stream_total[(r["stream"], r["what"] if r["what"] == "kernel" else r["name"])] += (
                int(r["end_ns"]) - int(r["start_ns"]))
        hidden = intersect(kern, cp) / length(cp) if cp else 0.0
        lines.append(f"| {key} | {span / 1e6:.2f} | {length(kern) / 1e6:.2f} | {length(h2d) / 1e6:.2f} | "
                     f"{length(d2h) / 1e6:.2f} | {length(cp) / 1e6:.2f} | {intersect(kern, cp) / 1e6:.2f} | "
                     f"{hidden:.1%} | {h2d_bytes / max(length(h2d), 1):.1f} |")
    lines.append("")
    lines.append("| stream | activity | busy ms (sum over the marked calls) |")
    lines.append("|---|---|---|")
    for (stream, what), ns in sorted(per_stream_total.items(), key=lambda x: (int(x[0][0]), x[0][1])):
        lines.append(f"| {stream} | {what} | {ns / 1e6:.2f} |")
    return "\n".join(lines)


if __name__ == "__main__":
    print(summarise(sys.argv[1]))
