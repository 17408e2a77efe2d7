"""Shape-bucket autotuner for the split-precision energy path.

Below 16 virtuals, and below 64 (a,i) columns (nocc*nvirt), fragments run
in FP64 (slice count 0, fixed rules in the library).  For
each larger virtual-space bucket it runs representative seeded fragments on the
GPU three ways -- the plain FP64 kernel (the reference values) and the split
kernel with one and with two residual slices -- and picks the cheapest slice
count whose worst pair-energy relative error over the sample stays below
half of the 1e-7 target (a 2x margin for fragments not in the sample).  It
also records the split kernel's time per bucket.  The table is installed in
the library with ``apply`` (rimp2_set_split_buckets) and can be saved as
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
                   torch.zeros(1, dtype=torch.float64, device="cuda")) for k in (0, 1, 2)}
    api.gen_fragment_dev(seed, nocc, nvirt, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(),
                         stream=s)
    E, T = out[0]
    api.energy_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), E.data_ptr(),
                   T.data_ptr(), precision=api.PREC_FP64, stream=s)
    res = {}
    for ns in (1, 2):
        E2, T2 = out[ns]
        args = (nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), E2.data_ptr(),
                T2.data_ptr())
        api.energy_split_dev(*args, nslices=ns, stream=s)  # warm
        st.synchronize()
        t0 = time.perf_counter()
        api.energy_split_dev(*args, nslices=ns, stream=s)
        st.synchronize()
        res[ns] = {"ms": (time.perf_counter() - t0) * 1e3}
    api.sync_status(s)
    ref = E.cpu().numpy()
    for ns in (1, 2):
        e = out[ns][0].cpu().numpy()
        res[ns]["pair_max"] = float(np.max(np.abs(e - ref) / np.abs(ref)))
        res[ns]["total"] = abs(out[ns][1].item() - T.item()) / abs(T.item())
    return res


def tune(seed=77):
    table = []
    for k, lo in enumerate(BUCKET_EDGES):
        worst = {1: 0.0, 2: 0.0}
        ms = {1: 0.0, 2: 0.0}
        for n, (nocc, nvirt, NBA) in enumerate(SAMPLE[lo]):
            r = _run(nocc, nvirt, NBA, seed + 100 * k + n)
            for ns in (1, 2):
                worst[ns] = max(worst[ns], r[ns]["pair_max"], r[ns]["total"])
                ms[ns] += r[ns]["ms"]
        pick = 1 if worst[1] <= TARGET / 2 else 2
        table.append({"nvirt_min": lo if k else FP64_BELOW, "nslices": pick,
                      "worst_rel_err": {"1": worst[1], "2": worst[2]},
                      "split_ms": {"1": ms[1], "2": ms[2]}, "sample": SAMPLE[lo]})
    fixed = {"nvirt_min": 0, "nslices": 0,
             "rule": f"fragments with fewer than {FP64_BELOW} virtuals run in FP64: a pair "
                     "energy of a few g^2 terms has nothing to average the split form's "
                     "FP32-accumulated correction against; the library also sends every "
                     "fragment with nocc*nvirt < 64 to FP64 (its FP32 epilogue rounding "
                     "leaves 2-5e-8 on such pair energies)"}
    return {"target": TARGET, "margin": 0.5, "buckets": [fixed] + table}


def apply(table):
    b = table["buckets"]
    api.set_split_buckets([x["nvirt_min"] for x in b], [x["nslices"] for x in b])


def load(path):
    with open(path) as f:
        t = json.load(f)
    apply(t)
    return t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
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
