"""Shape-bucket autotuner for the split-precision energy path.

Below 16 virtuals, and below 64 (a,i) columns (nocc*nvirt), fragments run
in FP64 (slice count 0, fixed rules in the library).  For
each larger virtual-space bucket it runs representative seeded fragments on the
GPU four ways -- the plain FP64 kernel (the reference values), the split
kernel with one residual slice on the paired kernel (three products per
element pair) and on the one-CTA kernel (four: more accurate), and with two
residual slices -- and picks the cheapest form whose worst pair-energy
relative error over the sample stays below half of the 1e-7 target (a 2x
margin for fragments not in the sample): one slice if the one-CTA run
qualifies (with the bucket held to the one-CTA kernel unless the paired run
qualifies too), else two.  Every run forces its kernel, so an installed
kernel table does not enter the measurement.  It also records the split
kernel's time per bucket.

For every bucket that runs one residual slice it then picks the energy
kernel, i.e. the tile shape: the one-CTA kernel (128 x 128 tiles, four
products per element pair) or the paired-CTA kernel (256 x 128 tiles on a
pair of SMs sharing the B operand, three products, a dummy CTA when an
occupied index has no partner).  It times both on a grid of occupied
counts and auxiliary sizes at the bucket's middle virtual count, each shape
replicated in one graph-launched batch plan until the launch does about
2 ms of work (CUDA events, best of three), and fits per-bucket thresholds
(paired kernel where nocc >= min_nocc and NBA >= min_nba) that minimise the
summed time over the grid.  Isolated shapes do not settle it: in a batch
the two kernels run as separate persistent launches over a mixed queue, so
the fitted table, uniform tables and "one-CTA kernel only" are then timed
on a seeded mixed batch of 128 uneven fragments (nocc U[8,64], nvirt
U[64,512], NBA U[256,2048]) and the fastest table is kept.

The tables are installed in the library with ``apply``
(rimp2_set_split_buckets, rimp2_set_split_kernel_rule) and can be saved as
JSON.  Every number it uses is measured on the GPU it runs on.

    python -m rimp2_gpu_gb300.autotune --out rimp2_gpu_gb300/tuning/split_buckets.json
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import api

TARGET = 1e-7
FP64_BELOW = 16  # fixed FP64 tier (slice count 0) below this many virtuals
BUCKET_EDGES = [64, 128, 192, 256, 384]          # nvirt_min of each bucket
BUCKET_TOP = [128, 192, 256, 384, 513]


def _sample(lo, hi):
    """Fragments at the bucket's low edge (fewest (a,b) terms per pair: the
    worst case for averaging), middle and top, with few and many occupied
    orbitals and short and long auxiliary spaces."""
    nv = [lo, lo + 1, (lo + hi) // 2, hi - 1]
    return [(o, v, b) for v in nv for (o, b) in ((8, 256), (40, 512), (16, 2048))]


SAMPLE = {lo: _sample(lo, hi) for lo, hi in zip(BUCKET_EDGES, BUCKET_TOP)}
# the top bucket also covers the production fragment shapes the reference's
# generator lists (generate.F90:48-53,65-70: nvirt 741/1041, nocc 59/99, NBA 2173)
SAMPLE[BUCKET_EDGES[-1]] += [(59, 741, 2173), (99, 1041, 2173)]


def _run(nocc, nvirt, NBA, seed):
    import torch
    st = torch.cuda.Stream()
    s = st.cuda_stream
    with torch.cuda.stream(st):
        dC = torch.empty(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
        deo = torch.empty(nocc, dtype=torch.float64, device="cuda")
        dev = torch.empty(nvirt, dtype=torch.float64, device="cuda")
        out = {k: (torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                   torch.zeros(1, dtype=torch.float64, device="cuda")) for k in (0, "1p", "1o", 2)}
    api.gen_fragment_dev(seed, nocc, nvirt, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(),
                         stream=s)
    E, T = out[0]
    api.energy_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), E.data_ptr(),
                   T.data_ptr(), precision=api.PREC_FP64, stream=s)
    res = {}
    old = os.environ.get("RIMP2_PAIR_KERNEL")
    try:
        # one residual slice on the paired kernel (three products), on the
        # one-CTA kernel (four products), two residual slices (one-CTA);
        # forced, so that no installed kernel table enters the measurement
        for key, ns in (("1p", 1), ("1o", 1), (2, 2)):
            os.environ["RIMP2_PAIR_KERNEL"] = "1" if key == "1p" else "0"
            E2, T2 = out[key]
            args = (nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), E2.data_ptr(),
                    T2.data_ptr())
            api.energy_split_dev(*args, nslices=ns, stream=s)  # warm
            st.synchronize()
            t0 = time.perf_counter()
            api.energy_split_dev(*args, nslices=ns, stream=s)
            st.synchronize()
            res[key] = {"ms": (time.perf_counter() - t0) * 1e3}
            if old is None:
                os.environ.pop("RIMP2_PAIR_KERNEL", None)
            else:
                os.environ["RIMP2_PAIR_KERNEL"] = old
    finally:
        if old is None:
            os.environ.pop("RIMP2_PAIR_KERNEL", None)
        else:
            os.environ["RIMP2_PAIR_KERNEL"] = old
    api.sync_status(s)
    ref = E.cpu().numpy()
    for ns in ("1p", "1o", 2):
        e = out[ns][0].cpu().numpy()
        res[ns]["pair_max"] = float(np.max(np.abs(e - ref) / np.abs(ref)))
        res[ns]["total"] = abs(out[ns][1].item() - T.item()) / abs(T.item())
    return res


KGRID_NOCC = [4, 8, 12, 16, 32]
KGRID_NBA = [256, 512, 1024, 2048, 4096]
NEVER = 1 << 30  # a threshold no fragment reaches
KWORK = 2.0e12   # effective FLOP per timed launch (about 2 ms of work)


def _time_kernels(nocc, nvirt, NBA, seed):
    """Milliseconds per graph launch of a batch of `copies` fragments of one
    shape (one residual slice), one-CTA and paired kernel."""
    import torch
    eff = 2.0 * NBA * (nocc * nvirt) ** 2
    copies = int(max(1, min(64, round(KWORK / eff))))
    st = torch.cuda.Stream()
    s = st.cuda_stream
    with torch.cuda.stream(st):
        dC = torch.empty(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
        deo = torch.empty(nocc, dtype=torch.float64, device="cuda")
        dev = torch.empty(nvirt, dtype=torch.float64, device="cuda")
        outs = [(torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                 torch.zeros(1, dtype=torch.float64, device="cuda")) for _ in range(copies)]
    api.gen_fragment_dev(seed, nocc, nvirt, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(),
                         stream=s)
    frags = [(nocc, nvirt, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), E.data_ptr(),
              T.data_ptr()) for E, T in outs]
    res = {}
    old = os.environ.get("RIMP2_PAIR_KERNEL")
    try:
        for kern, name in (("0", "one"), ("1", "pair")):
            os.environ["RIMP2_PAIR_KERNEL"] = kern
            plan = api.BatchPlan(frags, nslices=[1] * copies, graph=True, stream=s)
            plan.execute(stream=s)
            best = float("inf")
            for _ in range(3):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(st)
                plan.execute(stream=s)
                e1.record(st)
                st.synchronize()
                best = min(best, e0.elapsed_time(e1))
            api.sync_status(s)
            plan.close()
            res[name] = best
    finally:
        if old is None:
            os.environ.pop("RIMP2_PAIR_KERNEL", None)
        else:
            os.environ["RIMP2_PAIR_KERNEL"] = old
    res["copies"] = copies
    return res


def _fit_rule(grid):
    """Thresholds (min_nocc, min_nba) minimising the summed time of the grid
    when the paired kernel runs exactly where nocc >= min_nocc and NBA >=
    min_nba."""
    cn = sorted({g["nocc"] for g in grid}) + [NEVER]
    cb = sorted({g["NBA"] for g in grid}) + [NEVER]
    best = None
    for mo in cn:
        for mb in cb:
            t = sum(g["pair_ms"] if (g["nocc"] >= mo and g["NBA"] >= mb) else g["one_ms"]
                    for g in grid)
            if best is None or t < best[0] - 1e-9:
                best = (t, mo, mb)
    return best


def _grid_rule(buckets, seed):
    """Per-bucket thresholds fitted to the grid of isolated shapes."""
    rule = []
    for k, b in enumerate(buckets):
        if b["nslices"] != 1:
            continue
        lo = b["nvirt_min"]
        hi = BUCKET_TOP[BUCKET_EDGES.index(lo)] if lo in BUCKET_EDGES else lo + 128
        nv = (lo + hi) // 2
        grid = []
        for n, nocc in enumerate(KGRID_NOCC):
            for m, NBA in enumerate(KGRID_NBA):
                r = _time_kernels(nocc, nv, NBA, seed + 1000 * k + 10 * n + m)
                grid.append({"nocc": nocc, "nvirt": nv, "NBA": NBA, "copies": r["copies"],
                             "one_ms": r["one"], "pair_ms": r["pair"]})
        t, mo, mb = _fit_rule(grid)
        rule.append({"nvirt_min": lo, "min_nocc": mo, "min_nba": mb,
                     "grid_ms_chosen": t,
                     "grid_ms_one_only": sum(g["one_ms"] for g in grid),
                     "grid_ms_pair_only": sum(g["pair_ms"] for g in grid), "grid": grid})
    if rule:  # below the first one-slice bucket (an explicit nslices = 1)
        first = dict(rule[0], nvirt_min=0)
        first.pop("grid", None)
        first["note"] = "thresholds of the first measured bucket"
        rule.insert(0, first)
    return rule


MIX_N, MIX_SEED = 128, 7  # the mixed batch the kernel table is chosen on


def mixed_batch_shapes(n=MIX_N, seed=MIX_SEED):
    """Uneven fragments: nocc ~ U[8,64], nvirt ~ U[64,512], NBA ~ U[256,2048]."""
    g = np.random.Generator(np.random.Philox(seed))
    return list(zip(g.integers(8, 65, n).tolist(), g.integers(64, 513, n).tolist(),
                    g.integers(256, 2049, n).tolist()))


def _time_mixed_batch(candidates, seed=123):
    """Milliseconds per graph launch of one mixed batch under each candidate
    kernel table (best of three after two warm-up launches)."""
    import torch
    st = torch.cuda.Stream()
    s = st.cuda_stream
    bufs, desc = [], []
    with torch.cuda.stream(st):
        for f, (nocc, nvirt, NBA) in enumerate(mixed_batch_shapes()):
            d = dict(C=torch.empty(NBA * nvirt * nocc, dtype=torch.float64, device="cuda"),
                     eo=torch.empty(nocc, dtype=torch.float64, device="cuda"),
                     ev=torch.empty(nvirt, dtype=torch.float64, device="cuda"),
                     E=torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                     T=torch.zeros(1, dtype=torch.float64, device="cuda"))
            api.gen_fragment_dev(seed + f, nocc, nvirt, NBA, d["C"].data_ptr(), d["eo"].data_ptr(),
                                 d["ev"].data_ptr(), stream=s)
            bufs.append(d)
            desc.append((nocc, nvirt, NBA, d["C"].data_ptr(), d["eo"].data_ptr(),
                         d["ev"].data_ptr(), d["E"].data_ptr(), d["T"].data_ptr()))
    st.synchronize()
    out = {}
    for name, table in candidates.items():
        api.set_split_kernel_rule([x["nvirt_min"] for x in table], [x["min_nocc"] for x in table],
                                  [x["min_nba"] for x in table])
        plan = api.BatchPlan(desc, graph=True, stream=s)
        for _ in range(2):
            plan.execute(stream=s)
        best = float("inf")
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            plan.execute(stream=s)
            e1.record(st)
            st.synchronize()
            best = min(best, e0.elapsed_time(e1))
        api.sync_status(s)
        plan.close()
        out[name] = best
    return out


def tune_kernels(buckets, seed=91):
    """Energy-kernel table for the one-residual-slice buckets: thresholds
    fitted per bucket to isolated shapes, then that table and uniform
    tables timed on a mixed batch of uneven fragments, whose graph-launched
    persistent groups are what a batch runs; the fastest table is kept."""
    forced = sorted(b["nvirt_min"] for b in buckets if b.get("one_cta_only"))
    grid = _grid_rule([b for b in buckets if not b.get("one_cta_only")], seed)
    strip = lambda t: [{k: x[k] for k in ("nvirt_min", "min_nocc", "min_nba")} for x in t]  # noqa: E731
    edges = sorted({0} | {b["nvirt_min"] for b in buckets})

    def with_forced(table):
        """The candidate's thresholds at every bucket edge, the one-CTA
        kernel only in buckets whose one-slice form is accurate enough only
        with its four products."""
        out = []
        for lo in edges:
            r = max((x for x in table if x["nvirt_min"] <= lo), key=lambda x: x["nvirt_min"])
            never = lo in forced
            out.append(dict(nvirt_min=lo, min_nocc=NEVER if never else r["min_nocc"],
                            min_nba=NEVER if never else r["min_nba"]))
        return out

    cands = {"grid_fit": with_forced(strip(grid)),
             "one_cta_only": with_forced([dict(nvirt_min=0, min_nocc=NEVER, min_nba=NEVER)])}
    for mo in (8, 10, 16, 24):
        for mb in (512, 1024, 1536):
            cands[f"nocc>={mo},NBA>={mb}"] = with_forced([dict(nvirt_min=0, min_nocc=mo,
                                                               min_nba=mb)])
    times = _time_mixed_batch(cands)
    best = min(times, key=times.get)
    table = [dict(x, chosen_by=best) for x in cands[best]]
    return table, {"chosen": best, "one_cta_only_buckets": forced,
                   "mixed_batch": {"fragments": MIX_N, "seed": MIX_SEED,
                                                     "shapes": "nocc U[8,64], nvirt U[64,512], "
                                                               "NBA U[256,2048]"},
                   "batch_ms": times, "grid_fit": grid}


def tune(seed=77):
    table = []
    for k, lo in enumerate(BUCKET_EDGES):
        worst = {"1p": 0.0, "1o": 0.0, 2: 0.0}
        ms = {"1p": 0.0, "1o": 0.0, 2: 0.0}
        for n, (nocc, nvirt, NBA) in enumerate(SAMPLE[lo]):
            r = _run(nocc, nvirt, NBA, seed + 100 * k + n)
            for ns in ("1p", "1o", 2):
                worst[ns] = max(worst[ns], r[ns]["pair_max"], r[ns]["total"])
                ms[ns] += r[ns]["ms"]
        # one residual slice performs 3 (paired) or 4 (one-CTA) products per
        # element pair, two slices 6: one slice wherever the one-CTA kernel
        # meets the margin, held to that kernel unless the paired one does too
        okp, oko = worst["1p"] <= TARGET / 2, worst["1o"] <= TARGET / 2
        pick = 1 if oko else 2
        table.append({"nvirt_min": lo if k else FP64_BELOW, "nslices": pick,
                      "one_cta_only": bool(pick == 1 and not okp),
                      "worst_rel_err": {"1_paired": worst["1p"], "1_one_cta": worst["1o"],
                                        "2": worst[2]},
                      "split_ms": {"1_paired": ms["1p"], "1_one_cta": ms["1o"], "2": ms[2]},
                      "sample": SAMPLE[lo]})
    fixed = {"nvirt_min": 0, "nslices": 0,
             "rule": f"fragments with fewer than {FP64_BELOW} virtuals run in FP64: a pair "
                     "energy of a few g^2 terms has nothing to average the split form's "
                     "FP32-accumulated correction against; the library also sends every "
                     "fragment with nocc*nvirt < 64 to FP64 (its FP32 epilogue rounding "
                     "leaves 2-5e-8 on such pair energies)"}
    rule, sel = tune_kernels(table)
    return {"target": TARGET, "margin": 0.5, "buckets": [fixed] + table,
            "kernel_rule": rule, "kernel_rule_selection": sel}


def apply(table):
    b = table["buckets"]
    api.set_split_buckets([x["nvirt_min"] for x in b], [x["nslices"] for x in b])
    r = table.get("kernel_rule")
    if r:
        api.set_split_kernel_rule([x["nvirt_min"] for x in r], [x["min_nocc"] for x in r],
                                  [x["min_nba"] for x in r])


def load(path):
    with open(path) as f:
        t = json.load(f)
    apply(t)
    return t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--kernels-only", default=None, metavar="TABLE",
                    help="keep the slice counts of this JSON table, re-measure the kernel rule")
    a = ap.parse_args()
    if a.kernels_only:
        with open(a.kernels_only) as f:
            t = json.load(f)
        apply(t)  # the slice counts the batch runs with
        t["kernel_rule"], t["kernel_rule_selection"] = tune_kernels(
            [x for x in t["buckets"] if x["nvirt_min"] > 0])
    else:
        t = tune()
    apply(t)
    txt = json.dumps(t, indent=1)
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        with open(a.out, "w") as f:
            f.write(txt + "\n")
    print(txt)


if __name__ == "__main__":
    main()
