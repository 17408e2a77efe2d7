"""AO front end on the GPU (FP64): AO->MO transform, metric Cholesky and the
triangular solve that forms Calpha, against the CPU oracle (1e-10 relative
to the largest element), and the energy built on it."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def t(a):
    import torch
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()


def close(x, ref, rel):
    err = np.abs(x - ref).max() / np.abs(ref).max()
    assert err <= rel, err


@pytest.mark.parametrize("NBA,nbas,nocc", [(96, 40, 4), (130, 50, 5), (64, 24, 3)])
def test_calpha_from_ao_vs_oracle(NBA, nbas, nocc):
    from rimp2_gpu_gb300 import api
    nvirt = nbas - nocc
    ao = O.gen_ao3c(3, NBA, nbas)
    V = O.gen_metric(3, NBA)
    Cm = O.gen_mo(3, nbas)
    B = O.ao2mo(NBA, nbas, nocc, nvirt, ao, Cm)
    L = O.cholesky(V)
    ref = O.trsm_lower(L, B.reshape(NBA, -1, order="F")).reshape(B.shape, order="F")
    got = api.calpha_from_ao(NBA, nbas, nocc, nvirt, ao, V, Cm)
    close(got, ref, 1e-10)
    # energy on top of it (split path) within the energy bar of FP64
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, ref, np.sort(np.linspace(-1.2, -0.4, nocc)),
                              np.sort(np.linspace(0.2, 2.5, nvirt)))
    Ep, E = api.energy(nvirt, nocc, NBA, np.asfortranarray(got), np.sort(np.linspace(-1.2, -0.4, nocc)),
                       np.sort(np.linspace(0.2, 2.5, nvirt)), precision=api.PREC_SPLIT)
    assert abs(E - Er) <= 1e-7 * abs(Er)


def test_device_ao_generators_match_oracle():
    import torch
    from rimp2_gpu_gb300 import api
    NBA, nbas = 70, 33
    dao = torch.zeros(NBA * nbas * nbas, dtype=torch.float64, device="cuda")
    dV = torch.zeros(NBA * NBA, dtype=torch.float64, device="cuda")
    api.gen_ao_dev(5, NBA, nbas, dao.data_ptr(), dV.data_ptr())
    torch.cuda.synchronize()
    close(dao.cpu().numpy(), O.gen_ao3c(5, NBA, nbas).ravel(order="F"), 1e-14)
    close(dV.cpu().numpy(), O.gen_metric(5, NBA).ravel(order="F"), 1e-13)


@pytest.mark.parametrize("n,m", [(200, 37), (64, 5), (1, 3), (1100, 130)])
def test_cholesky_and_solve_blocks(n, m):
    """Several 64-blocks plus a ragged one, exactly one block, a 1x1 metric,
    and a metric of 18 blocks (the panel GEMM and the lower-triangle trailing
    update at many sizes)."""
    import torch
    from rimp2_gpu_gb300 import api
    V = O.gen_metric(8, n)
    dV = t(V)
    api.cholesky_dev(n, dV.data_ptr())
    torch.cuda.synchronize()
    L = dV.cpu().numpy().reshape(n, n, order="F")
    close(L, O.cholesky(V), 1e-12)
    assert np.all(np.triu(L, 1) == 0)
    Bm = O.gen_matrix(8, 9, n, m)
    dB, dX = t(Bm), torch.zeros(n * m, dtype=torch.float64, device="cuda")
    api.trsm_lower_dev(n, m, dV.data_ptr(), dB.data_ptr(), dX.data_ptr())
    torch.cuda.synchronize()
    close(dX.cpu().numpy().reshape(n, m, order="F"), O.trsm_lower(L, Bm), 1e-11)


def test_cholesky_rejects_indefinite_metric():
    import torch
    from rimp2_gpu_gb300 import api, _lib
    n = 70
    V = O.gen_metric(8, n)
    V[65, 65] = -5.0  # a negative pivot in the second block
    dV = t(V)
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.cholesky_dev(n, dV.data_ptr())
    assert ei.value.status == 1 and "positive definite" in str(ei.value)
    torch.cuda.synchronize()


@pytest.mark.parametrize("NBA,nbas,nocc", [(96, 40, 4), (300, 130, 13), (200, 77, 7)])
def test_split_ao2mo_matches_fp64(NBA, nbas, nocc):
    """AO->MO on the tensor cores (exact-integer FP16 slices, two residual
    slices) against the FP64 front end on the same inputs: Calpha within
    1e-8 of its largest element (the FP64 solve by the metric's Cholesky
    factor amplifies the transform's ~1e-10 rounding a few times), energies
    within 1e-7."""
    import torch
    from rimp2_gpu_gb300 import api
    nvirt = nbas - nocc
    dao = torch.zeros(NBA * nbas * nbas, dtype=torch.float64, device="cuda")
    dV = torch.zeros(NBA * NBA, dtype=torch.float64, device="cuda")
    api.gen_ao_dev(11, NBA, nbas, dao.data_ptr(), dV.data_ptr())
    dC = t(O.gen_mo(11, nbas))
    out64 = torch.zeros(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
    outsp = torch.zeros_like(out64)
    api.calpha_from_ao_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dV.data_ptr(), dC.data_ptr(),
                           out64.data_ptr())
    api.calpha_from_ao_split_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dV.data_ptr(),
                                 dC.data_ptr(), outsp.data_ptr())
    torch.cuda.synchronize()
    a, b = outsp.cpu().numpy(), out64.cpu().numpy()
    close(a, b, 1e-8)
    eo = np.sort(np.linspace(-1.3, -0.4, nocc))
    ev = np.sort(np.linspace(0.2, 2.8, nvirt))
    Ca64 = b.reshape(NBA, nvirt, nocc, order="F")
    Casp = np.asfortranarray(a.reshape(NBA, nvirt, nocc, order="F"))
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, np.asfortranarray(Ca64), eo, ev, blocked=True)
    Ep, E = api.energy(nvirt, nocc, NBA, Casp, eo, ev, precision=api.PREC_SPLIT)
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-7
    assert abs(E - Er) <= 1e-7 * abs(Er)


@pytest.mark.parametrize("NBA,nbas,nocc", [(75, 37, 4), (200, 130, 13), (130, 201, 80),
                                           (96, 70, 7), (180, 230, 85)])
def test_split_ao2mo_transform_vs_fp64(NBA, nbas, nocc):
    """The AO->MO transform alone, tensor-core form against the FP64 form on
    the same inputs, within 1e-8 of the largest element (measured 1.4-5.9e-9,
    the fused first half and the sliced one alike): odd NBA (rows not
    16-byte aligned), nbas not a multiple of the 8-row mu tile nor of the
    64-wide K chunk, 16 to 80 occupied columns in the fused first half, and
    nocc = 85 beyond it (the sliced first half)."""
    import torch
    from rimp2_gpu_gb300 import api
    nvirt = nbas - nocc
    dao = torch.zeros(NBA * nbas * nbas, dtype=torch.float64, device="cuda")
    dV = torch.zeros(NBA * NBA, dtype=torch.float64, device="cuda")
    api.gen_ao_dev(13, NBA, nbas, dao.data_ptr(), dV.data_ptr())
    dC = t(O.gen_mo(13, nbas))
    o64 = torch.zeros(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
    osp = torch.zeros_like(o64)
    api.ao2mo_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dC.data_ptr(), o64.data_ptr(),
                  split=False)
    api.ao2mo_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dC.data_ptr(), osp.data_ptr(),
                  split=True)
    torch.cuda.synchronize()
    api.sync_status()
    a, b = osp.cpu().numpy(), o64.cpu().numpy()
    err = np.abs(a - b).max() / np.abs(b).max()
    print(f"\nsplit AO->MO NBA={NBA} nbas={nbas} nocc={nocc}: {err:.2e} of the largest element")
    assert err <= 1e-8


@pytest.mark.parametrize("NBA,nbas,nocc", [(75, 37, 4), (130, 201, 80)])
def test_split_ao2mo_sliced_first_half(monkeypatch, NBA, nbas, nocc):
    """The sliced first half (AO slicer + persistent split GEMM), which the
    library takes beyond 80 occupied orbitals, forced at shapes the fused
    kernel would take: same bar against the FP64 transform."""
    import torch
    from rimp2_gpu_gb300 import api
    monkeypatch.setenv("RIMP2_AO_FUSED", "0")
    nvirt = nbas - nocc
    dao = torch.zeros(NBA * nbas * nbas, dtype=torch.float64, device="cuda")
    dV = torch.zeros(NBA * NBA, dtype=torch.float64, device="cuda")
    api.gen_ao_dev(17, NBA, nbas, dao.data_ptr(), dV.data_ptr())
    dC = t(O.gen_mo(17, nbas))
    o64 = torch.zeros(NBA * nvirt * nocc, dtype=torch.float64, device="cuda")
    osp = torch.zeros_like(o64)
    api.ao2mo_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dC.data_ptr(), o64.data_ptr(),
                  split=False)
    api.ao2mo_dev(NBA, nbas, nocc, nvirt, dao.data_ptr(), dC.data_ptr(), osp.data_ptr(),
                  split=True)
    torch.cuda.synchronize()
    api.sync_status()
    a, b = osp.cpu().numpy(), o64.cpu().numpy()
    assert np.abs(a - b).max() / np.abs(b).max() <= 1e-8
