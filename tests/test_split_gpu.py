"""Split-precision (tcgen05, FP16 Ozaki slices) energies against FP64.

Bar: every pair energy and the total within 1e-7 relative of the FP64
values, with the slice count the library picks for the shape; with two
residual slices the contraction error is negligible and what remains is the
FP32 epilogue's rounding (bar 3e-8).  Errors are printed
for the record.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(16, 96, 384), (8, 64, 256), (5, 130, 200), (3, 300, 77), (12, 256, 1024),
          (2, 128, 64), (1, 1, 1)]


@pytest.fixture(scope="module")
def api():
    from rimp2_gpu_gb300 import api as A
    return A


def dev_energy(api, Ca, eo, ev, nslices):
    import torch
    NBA, nvirt, nocc = Ca.shape
    dC = torch.from_numpy(Ca.ravel(order="F")).cuda()
    deo, dev = torch.from_numpy(eo).cuda(), torch.from_numpy(ev).cuda()
    dE = torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda")
    dT = torch.zeros(1, dtype=torch.float64, device="cuda")
    api.energy_split_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(),
                         dE.data_ptr(), dT.data_ptr(), nslices=nslices)
    torch.cuda.synchronize()
    return dE.cpu().numpy().reshape(nocc, nocc, order="F"), dT.item()


@pytest.mark.parametrize("nocc,nvirt,NBA", SHAPES)
def test_split_energy_within_1e7(api, nocc, nvirt, NBA):
    Ca, eo, ev = O.gen_fragment(200 + nvirt, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    Ep, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    rel = np.abs(Ep - Epr) / np.abs(Epr)
    tot = abs(E - Er) / abs(Er)
    ns = api.lib().rimp2_split_nslices(nvirt, nocc, NBA)
    print(f"\nsplit nocc={nocc} nvirt={nvirt} NBA={NBA} nslices={ns}: pair max {rel.max():.2e} "
          f"mean {rel.mean():.2e} total {tot:.2e}")
    # (1, 1, 1) runs in the FP64 tier (fewer than 64 (a,i) columns); every
    # split call is held to the same 1e-7 bar
    assert rel.max() <= 1e-7
    assert tot <= 1e-7


@pytest.mark.parametrize("nocc,nvirt,NBA", SHAPES[:4])
def test_split_two_slices_tight(api, nocc, nvirt, NBA):
    Ca, eo, ev = O.gen_fragment(300 + nvirt, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    for ns in (1, 2):
        Ep, E = dev_energy(api, Ca, eo, ev, ns)
        rel = np.abs(Ep - Epr) / np.abs(Epr)
        print(f"\nnslices={ns} nocc={nocc} nvirt={nvirt} NBA={NBA}: pair max {rel.max():.2e} "
              f"total {abs(E - Er) / abs(Er):.2e}")
        if ns == 2:  # contraction error negligible; FP32 epilogue rounding remains
            assert rel.max() <= 3e-8


def test_split_exact_integer_part(api):
    """Columns that are exact small integers times a power of two are sliced
    with zero residual, so the split energy must equal FP64 to rounding of
    the FP32 epilogue only (no contraction error at all)."""
    nocc, nvirt, NBA = 3, 40, 96
    rng = np.random.default_rng(0)
    Ca = np.asfortranarray(rng.integers(-40, 41, size=(NBA, nvirt, nocc)).astype(np.float64) / 1024)
    eo = np.sort(rng.uniform(-1.5, -0.3, nocc))
    ev = np.sort(rng.uniform(0.1, 3.0, nvirt))
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev)
    Ep, E = dev_energy(api, Ca, eo, ev, 1)
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-7
    assert abs(E - Er) <= 1e-7 * abs(Er)


def test_device_generator_matches_oracle(api):
    import torch
    nocc, nvirt, NBA = 5, 33, 70
    Ca, eo, ev = O.gen_fragment(9, nocc, nvirt, NBA)
    dC = torch.zeros(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
    deo = torch.zeros(nocc, dtype=torch.float64, device="cuda")
    dev = torch.zeros(nvirt, dtype=torch.float64, device="cuda")
    api.gen_fragment_dev(9, nocc, nvirt, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_allclose(dC.cpu().numpy(), Ca.ravel(order="F"), rtol=1e-13, atol=1e-17)
    np.testing.assert_allclose(deo.cpu().numpy(), eo, rtol=1e-15)
    np.testing.assert_allclose(dev.cpu().numpy(), ev, rtol=1e-15)


@pytest.mark.parametrize("nslices", [1, 2])
def test_split_large_K_exactness_bound(api, nslices):
    """NBA = 8192 (above the 4096 of the large configuration): the per-column
    scale must shrink so that ||S0||^2 <= 2^24 still holds; energies stay
    within the bar."""
    nocc, nvirt, NBA = 2, 128, 8192
    Ca, eo, ev = O.gen_fragment(77, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    Ep, E = dev_energy(api, Ca, eo, ev, nslices)
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-7


@pytest.mark.parametrize("nocc,nvirt,NBA,noE,nvE", [(8, 96, 256, 3, 24), (16, 200, 512, 5, 40),
                                                   (12, 256, 1024, 4, 64), (5, 130, 300, 5, 130)])
def test_split_eos_energy_vs_fp64(nocc, nvirt, NBA, noE, nvE):
    """Split-form local-orbital fragment energies within 1e-7 of the FP64
    fused form (random orthonormal local blocks; the last case has
    noccEOS = nocc and nvirtEOS = nvirt)."""
    from oracle import oracle as O
    from rimp2_gpu_gb300 import api
    Ca, eo, ev = O.gen_fragment(40 + nocc, nocc, nvirt, NBA)

    def q(m, k, s):
        return np.asfortranarray(np.linalg.qr(O.gen_matrix(40 + nocc, s, m, m))[0][:, :k])
    U = (q(nocc, noE, 1), q(nvirt, nvirt, 2), q(nocc, nocc, 3), q(nvirt, nvE, 4))
    ref = api.energy_eos(nvirt, nocc, noE, nvE, NBA, Ca, eo, ev, *U, precision=api.PREC_FP64)
    got = api.energy_eos(nvirt, nocc, noE, nvE, NBA, Ca, eo, ev, *U, precision=api.PREC_SPLIT)
    for r, g in zip(ref, got):
        assert abs(g - r) <= 1e-7 * abs(r), (g, r)


def test_split_eos_identity_is_canonical():
    from oracle import oracle as O
    from rimp2_gpu_gb300 import api
    nocc, nvirt, NBA = 9, 160, 640
    Ca, eo, ev = O.gen_fragment(77, nocc, nvirt, NBA)
    Io, Iv = np.eye(nocc, order="F"), np.eye(nvirt, order="F")
    eocc, evir = api.energy_eos(nvirt, nocc, nocc, nvirt, NBA, Ca, eo, ev, Io, Iv, Io, Iv,
                                precision=api.PREC_SPLIT)
    _, E = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    assert abs(eocc - E) <= 1e-7 * abs(E) and abs(evir - E) <= 1e-7 * abs(E)


# (nocc, nvirt, NBA): odd and even nocc (dummy second CTA), nocc = 1, a single
# and a ragged last virtual tile, K not a multiple of 64
PAIR_SHAPES = [(16, 96, 384), (7, 300, 77), (1, 130, 200), (2, 128, 64), (33, 256, 1000),
               (12, 256, 1024), (5, 17, 96)]


@pytest.fixture
def kernel_choice(monkeypatch):
    def use(v):
        monkeypatch.setenv("RIMP2_PAIR_KERNEL", v)
    return use


@pytest.mark.parametrize("nocc,nvirt,NBA", PAIR_SHAPES)
def test_pair_kernel_within_1e7(api, kernel_choice, nocc, nvirt, NBA):
    """The paired-CTA (cta_group::2) energy kernel against the FP64 oracle,
    and against the one-CTA kernel on the same slices (one residual slice)."""
    Ca, eo, ev = O.gen_fragment(500 + nvirt + nocc, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    kernel_choice("1")
    Ep, E = dev_energy(api, Ca, eo, ev, 1)
    kernel_choice("0")
    Ep1, E1 = dev_energy(api, Ca, eo, ev, 1)
    rel = np.abs(Ep - Epr) / np.abs(Epr)
    print(f"\npair kernel nocc={nocc} nvirt={nvirt} NBA={NBA}: pair max {rel.max():.2e} "
          f"total {abs(E - Er) / abs(Er):.2e}; vs one-CTA {abs(E - E1) / abs(E1):.2e}")
    assert rel.max() <= 1e-7
    assert abs(E - Er) <= 1e-7 * abs(Er)
    assert (np.abs(Ep - Ep1) / np.abs(Ep1)).max() <= 1e-7


# valid counts of the last 128-wide virtual block (zero-padded columns in
# its tiles): one, around the 16-column steps, half, and one short of full
SHORT_BLOCK = [1, 15, 16, 17, 40, 64, 65, 100, 112, 113, 127]


@pytest.mark.parametrize("rem", SHORT_BLOCK)
def test_short_last_block_both_kernels(api, kernel_choice, rem):
    """Fragments whose last 128-wide virtual block holds `rem` valid columns,
    against the CPU oracle: with one residual slice (nvirt = 256 + rem, in
    the one-slice bucket) on the paired kernel and on the one-CTA kernel --
    off-diagonal tile pairs with one short block and the short diagonal
    pair -- and with two residual slices on the one-CTA kernel beside one
    full block (128 + rem) and alone (rem >= 16)."""
    nocc, NBA = 7, 200
    runs = [(256 + rem, "1", 1), (256 + rem, "0", 1), (128 + rem, "0", 2)]
    if rem >= 16:
        runs.append((rem, "0", 2))
    ref = {}
    for nvirt, kern, ns in runs:
        if nvirt not in ref:
            Ca, eo, ev = O.gen_fragment(1100 + nvirt, nocc, nvirt, NBA)
            ref[nvirt] = (Ca, eo, ev) + O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
        Ca, eo, ev, Epr, Er = ref[nvirt]
        kernel_choice(kern)
        Ep, E = dev_energy(api, Ca, eo, ev, ns)
        assert api.last_split_kernel() == (2 if kern == "1" else 1)
        rel = np.abs(Ep - Epr) / np.abs(Epr)
        assert rel.max() <= 1e-7, (nvirt, kern, ns, rel.max())
        assert abs(E - Er) <= 1e-7 * abs(Er)


def test_pair_kernel_batched(api, kernel_choice):
    """Uneven fragments through one paired-CTA launch (graph-captured plan)."""
    import torch
    shapes = [(9, 200, 300), (16, 96, 384), (4, 257, 130), (1, 64, 64), (21, 128, 512)]
    kernel_choice("1")
    frags, bufs = [], []
    for k, (nocc, nvirt, NBA) in enumerate(shapes):
        Ca, eo, ev = O.gen_fragment(900 + k, nocc, nvirt, NBA)
        d = [torch.from_numpy(Ca.ravel(order="F")).cuda(), torch.from_numpy(eo).cuda(),
             torch.from_numpy(ev).cuda(), torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda"),
             torch.zeros(1, dtype=torch.float64, device="cuda")]
        bufs.append((Ca, eo, ev, d))
        frags.append((nocc, nvirt, NBA) + tuple(x.data_ptr() for x in d))
    plan = api.BatchPlan(frags, nslices=[1] * len(frags), graph=True)
    plan.execute()
    torch.cuda.synchronize()
    for (nocc, nvirt, NBA), (Ca, eo, ev, d) in zip(shapes, bufs):
        Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
        Ep = d[3].cpu().numpy().reshape(nocc, nocc, order="F")
        assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-7
        assert abs(d[4].item() - Er) <= 1e-7 * abs(Er)
    plan.close()


def test_kernel_choice_is_reported(api, kernel_choice):
    """One-residual-slice fragments run the kernel the table picks (set here
    to the paired kernel for nocc >= 10 and NBA >= 1024), the rest the
    one-CTA kernel; the environment overrides the choice and the library
    says which kernel ran."""
    import os
    from rimp2_gpu_gb300 import autotune
    api.set_split_kernel_rule([0], [10], [1024])
    try:
        _kernel_choice_checks(api, kernel_choice)
    finally:
        autotune.load(os.path.join(os.path.dirname(api.__file__), "tuning", "split_buckets.json"))


def _kernel_choice_checks(api, kernel_choice):
    small = O.gen_fragment(31, 6, 200, 256)
    big = O.gen_fragment(32, 32, 130, 1024)
    kernel_choice("")
    dev_energy(api, *small, 1)
    assert api.last_split_kernel() == 1
    dev_energy(api, *big, 1)
    assert api.last_split_kernel() == 2
    kernel_choice("0")
    dev_energy(api, *big, 1)
    assert api.last_split_kernel() == 1
    kernel_choice("1")
    dev_energy(api, *small, 1)
    assert api.last_split_kernel() == 2
    dev_energy(api, *small, 2)  # two residual slices: one-CTA kernel only
    assert api.last_split_kernel() == 1


@pytest.mark.parametrize("nocc,nvirt,NBA", [(33, 256, 1000), (9, 200, 512)])
def test_pair_kernel_host_streamed(api, kernel_choice, nocc, nvirt, NBA):
    """The host-pointer split call copies Calpha in occupied chunks and runs
    the paired kernel on each chunk's pair items as the chunk lands."""
    Ca, eo, ev = O.gen_fragment(700 + nocc, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    kernel_choice("1")
    Ep, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert api.last_split_kernel() == 2
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-7
    assert abs(E - Er) <= 1e-7 * abs(Er)


@pytest.mark.parametrize("pair", ["0", "1"])
def test_streamed_slicing_placement_bitwise(api, kernel_choice, monkeypatch, pair):
    """The host call slices each occupied chunk on its own stream beside the
    previous chunk's energy kernel; with RIMP2_STREAM_SLICE=0 it slices on
    the energy stream between the launches.  The same kernels compute the
    same items and reduce them in the same order: the energies must agree
    bit for bit, and with the oracle within 1e-7."""
    nocc, nvirt, NBA = 40, 200, 640  # seven chunks: 4, 6, 9, 13, 19, 28, 40 occupied indices
    Ca, eo, ev = O.gen_fragment(880, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    kernel_choice(pair)
    Ep1, E1 = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    monkeypatch.setenv("RIMP2_STREAM_SLICE", "0")
    Ep0, E0 = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert np.array_equal(Ep1, Ep0) and E1 == E0
    assert (np.abs(Ep1 - Epr) / np.abs(Epr)).max() <= 1e-7
    assert abs(E1 - Er) <= 1e-7 * abs(Er)


def test_pair_kernel_long_K_against_oracle(api, kernel_choice):
    """A long auxiliary space on the paired-CTA kernel (one residual slice,
    forced: the kernel table starts it at nocc >= 16 for this bucket):
    nocc=12, nvirt=512, NBA=4096, 64 K chunks per product chain, the regime
    of the large single fragment.  Every pair energy against the CPU oracle
    (the alpha loop of RIMP2.F90:395-405 restated, with the MP2 energy),
    split at 1e-7 and the plain FP64 kernel at 1e-11, in the manner of the
    reference's own Debug self-check (RIMP2.F90:253-367)."""
    nocc, nvirt, NBA = 12, 512, 4096
    kernel_choice("1")
    Ca, eo, ev = O.gen_fragment(61, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    Ep, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert api.last_split_kernel() == 2, "expected the paired-CTA kernel"
    rel = np.abs(Ep - Epr) / np.abs(Epr)
    print(f"\nlong K paired kernel: pair max {rel.max():.2e} total {abs(E - Er) / abs(Er):.2e}")
    assert rel.max() <= 1e-7
    assert abs(E - Er) <= 1e-7 * abs(Er)
    Ep64, E64 = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_FP64)
    assert (np.abs(Ep64 - Epr) / np.abs(Epr)).max() <= 1e-11
    assert abs(E64 - Er) <= 1e-11 * abs(Er)


def test_rcp_denom_error_bound():
    """The split epilogue's reciprocal of an energy denominator (rcp.approx
    refined by one Newton-Raphson step) against CUDA's correctly rounded
    __frcp_rn and against numpy's 1/d rounded to float32, over the whole
    denominator range of the synthetic fragments, Delta in [-9, -0.8]
    (occupied energies in [-1.5, -0.3], virtual in [0.1, 3.0]).  Bound: at
    most 1 ulp from the correctly rounded value, at least 99% of the values
    exact, and no one-sided drift (mean signed difference below 0.01 ulp), so
    a fragment whose denominators are all equal accumulates no bias."""
    import ctypes as C
    from rimp2_gpu_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(5)
    lo, hi = np.float32(-9.0), np.float32(-0.8)
    # every float in a few dense windows, plus uniform samples of the range
    dense = [np.arange(0, 1 << 16, dtype=np.int64) + b for b in
             (hi.view(np.int32).astype(np.int64), np.float32(-1.0).view(np.int32).astype(np.int64),
              np.float32(-2.0).view(np.int32).astype(np.int64),
              np.float32(-4.0).view(np.int32).astype(np.int64))]
    d = np.concatenate([np.concatenate(dense).astype(np.int32).view(np.float32),
                        rng.uniform(lo, hi, 1 << 20).astype(np.float32), [lo, hi]])
    d = np.ascontiguousarray(d[(d >= lo) & (d <= hi)], dtype=np.float32)
    r = np.empty_like(d)
    ref = np.empty_like(d)
    fp = C.POINTER(C.c_float)
    st = L.rimp2_selftest_rcp_denom(len(d), d.ctypes.data_as(fp), r.ctypes.data_as(fp),
                                    ref.ctypes.data_as(fp))
    assert st == 0, L.rimp2_last_error_string()
    ref_np = (1.0 / d.astype(np.float64)).astype(np.float32)
    assert np.array_equal(ref, ref_np)  # __frcp_rn is the correctly rounded reciprocal
    ulp = np.spacing(np.abs(ref)).astype(np.float64)
    diff = (r.astype(np.float64) - ref.astype(np.float64)) / ulp
    print(f"\nrcp_denom over {len(d)} denominators: max {np.abs(diff).max():.0f} ulp, "
          f"exact {np.mean(diff == 0):.4%}, mean signed {diff.mean():+.2e} ulp")
    assert np.abs(diff).max() <= 1.0
    assert np.mean(diff == 0) >= 0.99
    assert abs(diff.mean()) < 0.01
