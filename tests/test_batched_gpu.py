"""Batched uneven fragments: one persistent launch over a device work queue,
optionally replayed from a CUDA graph.  Each fragment's pair and total
energies are checked against the CPU oracle: FP64 path 1e-11 relative,
split path 1e-7 relative."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

# uneven shapes in the range of the batched workload (nocc 8-64, nvirt 64-512,
# NBA 256-2048), kept small enough for the oracle
SHAPES = [(8, 64, 256), (11, 200, 300), (5, 130, 777), (16, 96, 384), (3, 257, 129), (9, 64, 1024)]


@pytest.fixture(scope="module")
def frags():
    out = []
    for k, (nocc, nvirt, NBA) in enumerate(SHAPES):
        Ca, eo, ev = O.gen_fragment(500 + k, nocc, nvirt, NBA)
        Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
        out.append((Ca, eo, ev, Epr, Er))
    return out


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 1e-7)])
def test_energy_batched_host_api(frags, prec, tol):
    from rimp2_gpu_gb300 import api
    res = api.energy_batched([(f[0], f[1], f[2]) for f in frags], precision=prec)
    for (Ep, E), f in zip(res, frags):
        rel = np.abs(Ep - f[3]) / np.abs(f[3])
        assert rel.max() <= tol, rel.max()
        assert abs(E - f[4]) <= tol * abs(f[4])


@pytest.mark.parametrize("nslices", [None, [0, 1, 2, 0, 1, 0], [0] * len(SHAPES)],
                         ids=["buckets", "mixed", "fp64"])
def test_batch_plan_graph_replay(frags, nslices):
    """Slice count 0 puts a fragment in the plain FP64 persistent launch: its
    energies must meet the FP64 bar (1e-11), the split ones 1e-7."""
    import torch
    from rimp2_gpu_gb300 import api
    dev = []
    for Ca, eo, ev, _, _ in frags:
        nocc, nvirt, NBA = eo.size, ev.size, Ca.shape[0]
        t = dict(C=torch.from_numpy(Ca.ravel(order="F")).cuda(), eo=torch.from_numpy(eo).cuda(),
                 ev=torch.from_numpy(ev).cuda(),
                 E=torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                 T=torch.zeros(1, dtype=torch.float64, device="cuda"))
        dev.append((nocc, nvirt, NBA, t))
    desc = [(n, v, b, t["C"].data_ptr(), t["eo"].data_ptr(), t["ev"].data_ptr(), t["E"].data_ptr(),
             t["T"].data_ptr()) for n, v, b, t in dev]
    st = torch.cuda.Stream()
    plan = api.BatchPlan(desc, nslices=nslices, graph=True, stream=st.cuda_stream)
    results = []
    ns = nslices or [1] * len(SHAPES)
    expect_launches = sum(3 if k == 0 else 5 for k in set(ns))
    for rep in range(3):
        for _, _, _, t in dev:
            t["E"].zero_()
            t["T"].zero_()
        torch.cuda.synchronize()
        n0 = api.kernel_launch_count()
        plan.execute(stream=st.cuda_stream)
        if nslices is not None:
            assert api.kernel_launch_count() - n0 == expect_launches
        st.synchronize()
        api.sync_status(st.cuda_stream)
        results.append([(t["E"].cpu().numpy().copy(), t["T"].item()) for _, _, _, t in dev])
    plan.close()
    for rep in range(1, 3):  # deterministic replays
        for (Ea, Ta), (Eb, Tb) in zip(results[0], results[rep]):
            np.testing.assert_array_equal(Ea, Eb)
            assert Ta == Tb
    for (Ep, E), f, (n, _, _, _), k in zip(results[0], frags, dev, ns):
        tol = 1e-11 if k == 0 else 1e-7
        Ep = Ep.reshape(n, n, order="F")
        assert (np.abs(Ep - f[3]) / np.abs(f[3])).max() <= tol
        assert abs(E - f[4]) <= tol * abs(f[4])


def test_bucket_table_roundtrip():
    from rimp2_gpu_gb300 import api
    api.set_split_buckets([0, 128], [2, 1])
    assert api.split_nslices(100, 4, 64) == 2 and api.split_nslices(200, 4, 64) == 1
    from rimp2_gpu_gb300 import autotune
    import os
    t = autotune.load(os.path.join(os.path.dirname(api.__file__), "tuning", "split_buckets.json"))
    assert t["buckets"][0]["nvirt_min"] == 0
    for b in t["buckets"]:
        assert api.split_nslices(max(b["nvirt_min"], 1), 4, 64) == b["nslices"]


def test_batch_plan_all_four_groups():
    """One plan with a fragment in each launch group: paired-CTA kernel
    (one residual slice; the kernel table set to nocc >= 10, NBA >= 1024
    here), one-CTA kernel with one and with two residual slices, and plain
    FP64 -- one persistent launch sequence per group, every fragment against
    the oracle."""
    import os
    import torch
    from rimp2_gpu_gb300 import api, autotune
    api.set_split_kernel_rule([0], [10], [1024])
    try:
        _all_four_groups(api, torch)
    finally:
        autotune.load(os.path.join(os.path.dirname(api.__file__), "tuning", "split_buckets.json"))


def _all_four_groups(api, torch):
    shapes = [(12, 256, 1024, 1), (11, 200, 300, 1), (5, 130, 777, 2), (8, 64, 256, 0)]
    dev, ref = [], []
    for k, (nocc, nvirt, NBA, _) in enumerate(shapes):
        Ca, eo, ev = O.gen_fragment(800 + k, nocc, nvirt, NBA)
        ref.append(O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True))
        dev.append(dict(C=torch.from_numpy(Ca.ravel(order="F")).cuda(),
                        eo=torch.from_numpy(eo).cuda(), ev=torch.from_numpy(ev).cuda(),
                        E=torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                        T=torch.zeros(1, dtype=torch.float64, device="cuda")))
    desc = [(n, v, b, t["C"].data_ptr(), t["eo"].data_ptr(), t["ev"].data_ptr(), t["E"].data_ptr(),
             t["T"].data_ptr()) for (n, v, b, _), t in zip(shapes, dev)]
    plan = api.BatchPlan(desc, nslices=[s[3] for s in shapes], graph=True)
    n0 = api.kernel_launch_count()
    plan.execute()
    torch.cuda.synchronize()
    api.sync_status()
    assert api.kernel_launch_count() - n0 == 3 + 5 + 5 + 5
    plan.close()
    for (n, _, _, ns), t, (Epr, Er) in zip(shapes, dev, ref):
        tol = 1e-11 if ns == 0 else 1e-7
        Ep = t["E"].cpu().numpy().reshape(n, n, order="F")
        assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= tol
        assert abs(t["T"].item() - Er) <= tol * abs(Er)


@pytest.mark.parametrize("prec,tol", [(0, 1e-11), (1, 1e-7)])
def test_energy_batched_packed_pinned(prec, tol):
    """Packed host input in pinned memory through rimp2_energy_batched's
    overlapped copies (per launch group on the copy stream, each group's
    kernels waiting for its own fragments).  Split form: every launch group
    present -- paired kernel (the kernel table set to nocc >= 10, NBA >= 1024
    here), one-CTA kernel with one and with two residual slices, and plain
    FP64 (nocc * nvirt < 64); FP64 form: all in the plain launch.  The two
    paired-kernel fragments fall in different plans (the host call divides
    that group by volume so that its first half starts while the second half
    is copied)."""
    import os
    import torch
    from rimp2_gpu_gb300 import api, autotune
    shapes = [(12, 256, 1024), (11, 200, 300), (5, 130, 777), (8, 64, 256), (2, 20, 100),
              (10, 192, 1024)]
    data = [O.gen_fragment(900 + k, *s) for k, s in enumerate(shapes)]
    ref = [O.pair_energies(v, n, b, Ca, eo, ev, blocked=True)
           for (n, v, b), (Ca, eo, ev) in zip(shapes, data)]
    ca = torch.empty(sum(n * v * b for n, v, b in shapes), dtype=torch.float64, pin_memory=True)
    cav, o = ca.numpy(), 0
    for Ca, _, _ in data:
        cav[o:o + Ca.size] = Ca.ravel(order="F")
        o += Ca.size
    eo = np.concatenate([d[1] for d in data])
    ev = np.concatenate([d[2] for d in data])
    api.set_split_kernel_rule([0], [10], [1024])
    try:
        assert [api.split_nslices(v, n, b) for n, v, b in shapes] == [1, 1, 1, 2, 0, 1]
        assert [api.split_kernel_for(v, n, b) for n, v, b in shapes] == [2, 1, 1, 1, 0, 2]
        res = api.energy_batched_packed([s[0] for s in shapes], [s[1] for s in shapes],
                                        [s[2] for s in shapes], cav, eo, ev, precision=prec)
    finally:
        autotune.load(os.path.join(os.path.dirname(api.__file__), "tuning", "split_buckets.json"))
    for (n, v, b), (Ep, E), (Epr, Er) in zip(shapes, res, ref):
        bar = 1e-11 if prec == 0 or api.split_nslices(v, n, b) == 0 else tol
        assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= bar
        assert abs(E - Er) <= bar * abs(Er)
    with pytest.raises(ValueError):
        api.energy_batched_packed([s[0] for s in shapes], [s[1] for s in shapes],
                                  [s[2] for s in shapes], cav[:-1], eo, ev, precision=prec)


def test_batch_graph_overlap_forms_bitwise(frags, monkeypatch):
    """The batch graph with the launch groups in sequence (default) and with
    the next group's slicing on a side branch (RIMP2_BATCH_OVERLAP=1) runs
    the same kernels on the same items: the energies agree bit for bit."""
    import torch
    from rimp2_gpu_gb300 import api
    out = []
    for ov in ("0", "1"):
        monkeypatch.setenv("RIMP2_BATCH_OVERLAP", ov)
        dev = []
        for Ca, eo, ev, _, _ in frags:
            nocc, nvirt, NBA = eo.size, ev.size, Ca.shape[0]
            dev.append((nocc, nvirt, NBA, dict(
                C=torch.from_numpy(Ca.ravel(order="F")).cuda(), eo=torch.from_numpy(eo).cuda(),
                ev=torch.from_numpy(ev).cuda(),
                E=torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
                T=torch.zeros(1, dtype=torch.float64, device="cuda"))))
        desc = [(n, v, b, t["C"].data_ptr(), t["eo"].data_ptr(), t["ev"].data_ptr(),
                 t["E"].data_ptr(), t["T"].data_ptr()) for n, v, b, t in dev]
        plan = api.BatchPlan(desc, nslices=[0, 1, 2, 0, 1, 0], graph=True)
        plan.execute()
        torch.cuda.synchronize()
        api.sync_status()
        plan.close()
        out.append([(t["E"].cpu().numpy(), t["T"].item()) for _, _, _, t in dev])
    for (a, ta), (b, tb) in zip(*out):
        assert np.array_equal(a, b) and ta == tb
