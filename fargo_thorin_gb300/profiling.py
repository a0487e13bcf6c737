"""Summaries of ncu output for the profile notes.

``python -m fargo_thorin_gb300.profiling launches <csv>`` reads the CSV log of
``ncu --metrics gpu__time_duration.sum --csv --log-file <csv> ...`` and prints
a markdown table of launches, total time, share and average per kernel.
``python -m fargo_thorin_gb300.profiling raw <csv>`` reads
``ncu -i <rep> --page raw --csv`` output and prints the metrics used for the
roofline (DRAM bytes, throughput, FP64 pipe, warps, registers) per launch.
"""
import collections
import csv
import sys

_SCALE_TO_US = {"ns": 1e-3, "nsecond": 1e-3, "us": 1.0, "usecond": 1.0, "ms": 1e3, "msecond": 1e3,
                "s": 1e6, "second": 1e6}


def _rows(path):
    rows = list(csv.reader(open(path)))
    h = next(i for i, r in enumerate(rows) if "Kernel Name" in r)
    return rows[h], rows[h + 1:]


def launch_table(path, top=40):
    hdr, data = _rows(path)
    ki, mi, ui = hdr.index("Kernel Name"), hdr.index("Metric Value"), hdr.index("Metric Unit")
    tot, cnt = collections.Counter(), collections.Counter()
    for r in data:
        if len(r) <= mi or not r[mi]:
            continue
        us = float(r[mi].replace(",", "")) * _SCALE_TO_US[r[ui]]
        name = r[ki].split("(")[0].replace("void ", "")
        tot[name] += us
        cnt[name] += 1
    total = sum(tot.values())
    out = [f"{sum(cnt.values())} launches, {total / 1e3:.2f} ms summed (cold-cache, serialised).", "",
           "| kernel | launches | total ms | share | avg us |", "|---|---:|---:|---:|---:|"]
    for k, v in tot.most_common(top):
        out.append(f"| {k} | {cnt[k]} | {v / 1e3:.3f} | {100 * v / total:.1f}% | {v / cnt[k]:.1f} |")
    return "\n".join(out)


RAW_METRICS = ("gpu__time_duration.sum", "dram__bytes_read.sum", "dram__bytes_write.sum",
               "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed", "dram__cycles_active.avg.pct_of_peak_sustained_elapsed",
               "sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active",
               "sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active",
               "sm__warps_active.avg.pct_of_peak_sustained_active", "launch__registers_per_thread",
               "launch__grid_size", "launch__block_size")


def raw_table(path):
    rows = list(csv.reader(open(path)))
    hdr, units = rows[0], rows[1]
    cols = [(m, hdr.index(m)) for m in RAW_METRICS if m in hdr]
    ki = hdr.index("Kernel Name")
    out = ["| kernel | " + " | ".join(f"{m} ({units[i]})" for m, i in cols) + " |",
           "|---|" + "---:|" * len(cols)]
    for r in rows[2:]:
        out.append(f"| {r[ki].split('(')[0]} | " + " | ".join(r[i] for _, i in cols) + " |")
    return "\n".join(out)


if __name__ == "__main__":
    kind, path = sys.argv[1], sys.argv[2]
    print(launch_table(path) if kind == "launches" else raw_table(path))
