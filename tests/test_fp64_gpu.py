"""Parity of the FP64 GPU path (C-ABI) with the CPU oracle.

Tolerances: pair and total energies 1e-11 relative, amplitudes 1e-12
absolute; every other array within 1e-12 relative to its largest element
(different but exact-to-rounding FP64 summation orders on the two sides),
and the reference's own 1e-10 absolute check (RIMP2.F90:262) for the
constant fixtures.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from rimp2_gpu_gb300 import api as A
    return A


def close(x, ref, rel=1e-12):
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(x - ref).max() / scale
    assert err <= rel, f"max rel-to-max error {err:.3e} > {rel:g}"


def test_energy_cfg1_golden(api, golden):
    g = golden("energy_cfg1.npz")
    nocc, nvirt, NBA = int(g["nocc"]), int(g["nvirt"]), int(g["NBA"])
    Ca, eo, ev = O.gen_fragment(int(g["seed"]), nocc, nvirt, NBA)
    Ep, E, t = api.energy(nvirt, nocc, NBA, Ca, eo, ev, amplitudes=True)
    rel = np.abs(Ep - g["Epair"]) / np.abs(g["Epair"])
    assert rel.max() <= 1e-11, rel.max()
    assert abs(E - float(g["Etot"])) <= 1e-11 * abs(float(g["Etot"]))
    assert np.abs(t[:, :, :8, :2] - g["t_slice"]).max() <= 1e-12


@pytest.mark.parametrize("nocc,nvirt,NBA", [(1, 1, 1), (3, 17, 5), (5, 64, 64), (7, 65, 129),
                                            (4, 130, 33), (2, 200, 300)])
def test_energy_ragged_vs_oracle(api, nocc, nvirt, NBA):
    Ca, eo, ev = O.gen_fragment(100 + nocc, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    Ep, E, t = api.energy(nvirt, nocc, NBA, Ca, eo, ev, amplitudes=True)
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-11
    assert abs(E - Er) <= 1e-11 * abs(Er)
    tr = O.amplitudes(nvirt, nocc, NBA, Ca, eo, ev)
    assert np.abs(t - tr).max() <= 1e-12
    # permutation symmetry of the amplitudes: t(a,i,b,j) = t(b,j,a,i)
    # (the two orderings come from two tensor-op tiles: equal to rounding)
    np.testing.assert_allclose(t, t.transpose(2, 3, 0, 1), rtol=1e-14, atol=1e-18)


def test_energy_dev_pointer_form(api):
    import torch
    nocc, nvirt, NBA = 6, 70, 90
    Ca, eo, ev = O.gen_fragment(21, nocc, nvirt, NBA)
    Epr, Er = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
    dC = torch.from_numpy(Ca.ravel(order="F")).cuda()
    deo, dev = torch.from_numpy(eo).cuda(), torch.from_numpy(ev).cuda()
    dE = torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda")
    dT = torch.zeros(1, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    api.energy_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(), dE.data_ptr(),
                   dT.data_ptr(), stream=s)
    torch.cuda.synchronize()
    Ep = dE.cpu().numpy().reshape(nocc, nocc, order="F")
    assert (np.abs(Ep - Epr) / np.abs(Epr)).max() <= 1e-11
    assert abs(dT.item() - Er) <= 1e-11 * abs(Er)


def test_subroutines_golden(api, golden):
    g = golden("small_general.npz")
    nvirt, nocc, noccEOS, nvirtEOS, NBA = (int(g[k]) for k in
                                           ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA"))
    F = lambda k: np.asfortranarray(g[k])  # noqa: E731
    Ca, eo, ev = F("Calpha"), F("EVocc"), F("EVvirt")
    tocc = O.fzeros(nocc, noccEOS, nvirt, nvirt)
    api.calc_toccA(nvirt, nocc, noccEOS, NBA, Ca, eo, ev, tocc, F("UoccEOST"))
    close(tocc, g["tocc"])
    tvirt = O.fzeros(nocc, nocc, nvirtEOS, nvirt)
    api.calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, Ca, eo, ev, tvirt, F("UvirtEOST"))
    close(tvirt, g["tvirt"])
    djik = O.fzeros(nvirt, nocc, nocc, noccEOS)
    api.calc_gen4DimFO(NBA, Ca, nvirt, nocc, F("Y"), nocc, noccEOS, djik)
    close(djik, g["djik"])
    outs = api.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Ca, eo, ev, F("UoccEOST"),
                         F("UvirtT"), F("UoccT"), F("UvirtEOST"))
    for name, arr in zip(("toccEOS", "tvirtEOS", "goccEOS", "gvirtEOS"), outs):
        close(arr, g[name])


def test_subroutines_each_vs_oracle(api):
    nvirt, nocc, noccEOS, nvirtEOS, NBA = 19, 6, 4, 5, 23
    Ca, eo, ev = O.gen_fragment(31, nocc, nvirt, NBA)
    UvT = O.gen_matrix(31, 11, nvirt, nvirt)
    UoT = O.gen_matrix(31, 12, nocc, nocc)
    # toccB / tvirtB on random intermediates
    t3 = np.asfortranarray(O.gen_matrix(31, 20, noccEOS * noccEOS * nvirt, nvirt).reshape(
        noccEOS, noccEOS, nvirt, nvirt, order="F"))
    a, r = O.fzeros(nvirt, noccEOS, nvirt, noccEOS), O.fzeros(nvirt, noccEOS, nvirt, noccEOS)
    api.calc_toccB(nvirt, noccEOS, t3, UvT, a)
    O.calc_toccB(nvirt, noccEOS, t3, UvT, r)
    close(a, r)
    v3 = np.asfortranarray(O.gen_matrix(31, 21, nocc * nocc * nvirtEOS, nvirtEOS).reshape(
        nocc, nocc, nvirtEOS, nvirtEOS, order="F"))
    a, r = O.fzeros(nvirtEOS, nocc, nvirtEOS, nocc), O.fzeros(nvirtEOS, nocc, nvirtEOS, nocc)
    api.calc_tvirtB(nvirtEOS, nocc, v3, UoT, a)
    O.calc_tvirtB(nvirtEOS, nocc, v3, UoT, r)
    close(a, r)
    # TransAlpha1 / TransAlpha2
    a, r = O.fzeros(NBA, nvirt, nocc), O.fzeros(NBA, nvirt, nocc)
    api.TransAlpha1(nvirt, nocc, NBA, UvT, Ca, a)
    O.transalpha1(nvirt, nocc, NBA, UvT, Ca, r)
    close(a, r)
    UvE = O.gen_matrix(31, 13, nvirt, nvirtEOS)
    a, r = O.fzeros(NBA, nvirtEOS, nocc), O.fzeros(NBA, nvirtEOS, nocc)
    api.TransAlpha2(nocc, nvirt, nvirtEOS, NBA, UvE, Ca, a)
    O.transalpha2(nocc, nvirt, nvirtEOS, NBA, UvE, Ca, r)
    close(a, r)
    # gocc / gvirt
    a, r = O.fzeros(nvirt, nocc, nvirt, nocc), O.fzeros(nvirt, nocc, nvirt, nocc)
    api.calc_gocc(nvirt, nocc, NBA, Ca, a)
    O.calc_gocc(nvirt, nocc, NBA, Ca, r)
    close(a, r)
    api.calc_gvirt(nvirt, nocc, NBA, Ca, a)
    close(a, r)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_dgemm(api, ta, tb):
    M, N, K = 37, 23, 71
    A = O.gen_matrix(1, 1, *((M, K) if ta == "N" else (K, M)))
    B = O.gen_matrix(1, 2, *((K, N) if tb == "N" else (N, K)))
    Cg = O.gen_matrix(1, 3, M + 3, N)
    Cr = Cg.copy(order="F")
    lda, ldb = A.shape[0], B.shape[0]
    api.dgemm(ta, tb, M, N, K, 0.7, A, lda, B, ldb, -1.3, Cg, M + 3)
    O.dgemm(ta, tb, M, N, K, 0.7, A, lda, B, ldb, -1.3, Cr, M + 3)
    close(Cg, Cr, 1e-13)


@pytest.mark.parametrize("k", [0, 1])
def test_steps5to8_reference_known_answers(api, k):
    """The reference's own fixtures and its 1e-10 check (RIMP2.GPU.F90:349-422)."""
    from tests.test_oracle import SIZES, closed_forms
    nvirt, nocc, noccEOS, nvirtEOS, NBA = SIZES[k]
    arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    outs = api.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, *arrs)
    exp = closed_forms(nvirt, nocc, NBA)
    for name, arr in zip(("toccEOS", "tvirtEOS", "goccEOS", "gvirtEOS"), outs):
        assert np.abs(arr - exp[name]).max() <= 1e-10, name


@pytest.mark.parametrize("k", [0, 1])
def test_first_order_reference_known_answers(api, k):
    """The driver's first-order block (RIMP2.F90:172-251) on generate.F90's
    first-order inputs, with the reference's 1e-10 check (RIMP2.F90:337,355)
    against the closed forms."""
    from tests.test_oracle import SIZES, first_order_closed_forms
    nvirt, nocc, noccEOS, nvirtEOS, NBA = SIZES[k]
    Ca, _, _, UoE, UvT, UoT, UvE = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    occ, vv = O.gen_kat_fo(NBA, nvirt, nocc, nocc)
    djik, blad = api.first_order(nvirt, nocc, noccEOS, nvirtEOS, nocc, NBA, Ca, occ, vv, UoE, UvT,
                                 UoT, UvE)
    d_exp, b_exp = first_order_closed_forms(nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc)
    assert np.abs(djik - d_exp).max() <= 1e-10
    assert np.abs(blad - b_exp).max() <= 1e-10


def test_first_order_golden_general(api, golden):
    """Random non-unitary matrices, nocctot != nocc with a separate UoccallT."""
    g = golden("first_order.npz")
    nv, no, ne, ve, nb, nt = (int(g[k]) for k in ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA",
                                                 "nocctot"))
    A = {k: np.asfortranarray(g[k]) for k in ("Calpha", "CalphaOcc", "CalphaVV", "UoccEOST",
                                              "UvirtT", "UoccT", "UoccallT", "UvirtEOST")}
    djik, blad = api.first_order(nv, no, ne, ve, nt, nb, A["Calpha"], A["CalphaOcc"],
                                 A["CalphaVV"], A["UoccEOST"], A["UvirtT"], A["UoccT"],
                                 A["UvirtEOST"], UoccallT=A["UoccallT"])
    close(djik, g["djik"])
    close(blad, g["blad"])


def test_first_order_rejects_nocc_above_nvirt(api):
    from rimp2_gpu_gb300 import _lib
    nv, no, ne, ve, nb = 3, 4, 2, 2, 5
    z = lambda *s: np.zeros(s, order="F")  # noqa: E731
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.first_order(nv, no, ne, ve, no, nb, z(nb, nv, no), z(nb, no, no), z(nb, nv, nv),
                        z(no, ne), z(nv, nv), z(no, no), z(nv, ve))
    assert ei.value.status == 1


def test_energy_eos_golden_general(api, golden):
    """Fused local-orbital fragment energies against the energies contracted
    from the reference's own Step 5-8 arrays (random non-unitary U)."""
    g = golden("small_general.npz")
    n = {k: int(g[k]) for k in ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA")}
    A = [np.asfortranarray(g[k]) for k in ("Calpha", "EVocc", "EVvirt", "UoccEOST", "UvirtT",
                                           "UoccT", "UvirtEOST")]
    eocc, evir = api.energy_eos(n["nvirt"], n["nocc"], n["noccEOS"], n["nvirtEOS"], n["NBA"], *A)
    ro, rv = O.energy_eos_from_arrays(g["toccEOS"], g["goccEOS"], g["tvirtEOS"], g["gvirtEOS"])
    assert abs(eocc - ro) <= 1e-11 * abs(ro), (eocc, ro)
    assert abs(evir - rv) <= 1e-11 * abs(rv), (evir, rv)


def test_energy_eos_fragment_vs_oracle_arrays(api):
    """nocc=16, nvirt=96, NBA=384 with orthonormal local-orbital blocks
    (noccEOS=5, nvirtEOS=24): oracle Steps 5-8 arrays contracted in FP64."""
    nocc, nvirt, NBA, noE, nvE = 16, 96, 384, 5, 24
    Ca, eo, ev = O.gen_fragment(21, nocc, nvirt, NBA)
    q = lambda m, k, s: np.asfortranarray(np.linalg.qr(O.gen_matrix(21, s, m, m))[0][:, :k])  # noqa
    UoE, UvT, UoT, UvE = q(nocc, noE, 30), q(nvirt, nvirt, 31), q(nocc, nocc, 32), q(nvirt, nvE, 33)
    tE, vE, gE, gvE = O.steps5to8(nvirt, nocc, noE, nvE, NBA, Ca, eo, ev, UoE, UvT, UoT, UvE)
    ro, rv = O.energy_eos_from_arrays(tE, gE, vE, gvE)
    eocc, evir = api.energy_eos(nvirt, nocc, noE, nvE, NBA, Ca, eo, ev, UoE, UvT, UoT, UvE)
    assert abs(eocc - ro) <= 1e-11 * abs(ro), (eocc, ro)
    assert abs(evir - rv) <= 1e-11 * abs(rv), (evir, rv)


def test_energy_eos_identity_is_canonical(api):
    nocc, nvirt, NBA = 7, 65, 129
    Ca, eo, ev = O.gen_fragment(22, nocc, nvirt, NBA)
    Io, Iv = np.eye(nocc, order="F"), np.eye(nvirt, order="F")
    eocc, evir = api.energy_eos(nvirt, nocc, nocc, nvirt, NBA, Ca, eo, ev, Io, Iv, Io, Iv)
    _, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev)
    assert abs(eocc - E) <= 1e-12 * abs(E) and abs(evir - E) <= 1e-12 * abs(E)


def test_get_dev_mem(api):
    total, free = api.get_dev_mem()
    assert total > 200e9 and 0 < free <= total


def test_fault_injection_alloc(api, monkeypatch):
    from rimp2_gpu_gb300 import _lib
    monkeypatch.setenv("RIMP2_FAULT_INJECT", "alloc")
    Ca, eo, ev = O.gen_fragment(2, 2, 8, 8)
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.energy(8, 2, 8, Ca, eo, ev)
    assert ei.value.status == 3
    monkeypatch.delenv("RIMP2_FAULT_INJECT")
    Ep, E = api.energy(8, 2, 8, Ca, eo, ev)  # the library stays usable
    assert np.isfinite(E)


def test_fault_injection_launch(api, monkeypatch):
    from rimp2_gpu_gb300 import _lib
    Ca, eo, ev = O.gen_fragment(3, 2, 8, 8)
    monkeypatch.setenv("RIMP2_FAULT_INJECT", "launch")
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.energy(8, 2, 8, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert ei.value.status == 2 and "injected" in str(ei.value)
    monkeypatch.delenv("RIMP2_FAULT_INJECT")
    Ep, E = api.energy(8, 2, 8, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert np.isfinite(E)


def test_bounded_wait_gives_up_and_library_recovers(api):
    """A device wait on a barrier nothing completes must end by its clock
    budget with RIMP2_ERR_TIMEOUT (no hang, no trap), and the next call works."""
    st = api.lib().rimp2_selftest_bounded_wait(2_000_000, None)  # ~1 ms of SM clock
    assert st == 5, api.last_error()
    assert "bounded wait" in api.last_error()
    Ca, eo, ev = O.gen_fragment(4, 3, 40, 50)
    Epr, Er = O.pair_energies(40, 3, 50, Ca, eo, ev)
    Ep, E = api.energy(40, 3, 50, Ca, eo, ev, precision=api.PREC_SPLIT)
    assert abs(E - Er) <= 1e-7 * abs(Er)
