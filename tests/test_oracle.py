"""CPU oracle pinned against the reference's own known answers (no GPU)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

# closed forms of the constant fixtures (generate.F90:77-128):
# every element of each output equals one constant
C_CONST = 0.00124235636 + 0.01010101 + 0.014321
D_CONST = 2 * (1.934321 - 1.91321)
U1, UV, UO, W = 0.030321 + 0.101121, 0.021321 + 0.01321, 0.032321 + 0.01521, 0.023321 + 0.01421
SIZES = [(74, 10, 4, 15, 273), (104, 20, 4, 15, 373)]  # generate.F90:41-46, 58-63


def closed_forms(nvirt, nocc, NBA):
    c = C_CONST
    return dict(
        toccEOS=NBA * c * c / D_CONST * (nocc * U1) ** 2 * (nvirt * UV) ** 2,
        tvirtEOS=NBA * c * c / D_CONST * (nvirt * W) ** 2 * (nocc * UO) ** 2,
        goccEOS=NBA * (c * nocc * U1 * nvirt * UV) ** 2,
        gvirtEOS=NBA * (c * nocc * UO * nvirt * W) ** 2)


def test_philox_known_answers():
    # Random123 published known-answer vectors for philox4x32-10
    assert O.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert O.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2) == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert O.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                           [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


@pytest.mark.parametrize("k", [0, 1])
def test_reference_known_answers(k, golden):
    nvirt, nocc, noccEOS, nvirtEOS, NBA = SIZES[k]
    arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    outs = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, *arrs)
    exp = closed_forms(nvirt, nocc, NBA)
    g = golden("kat.npz")
    for name, arr in zip(("toccEOS", "tvirtEOS", "goccEOS", "gvirtEOS"), outs):
        # the reference's own check: |diff| > 1e-10 => stop 'ERROR3' (RIMP2.F90:262)
        assert np.abs(arr - exp[name]).max() <= 1e-10, name
        np.testing.assert_array_equal(np.array([arr.min(), arr.max()]), g[f"file{k+1}_{name}"])


# first-order fixture inputs CalphaOcc/CalphaVV(A,B,C) = A*X + B*Y + C*Z
# (generate.F90:258,304); djik and blad are constants with closed forms
FX, FY, FZ = 0.01124235636, 0.01011111, 0.16422


def first_order_closed_forms(nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot):
    c = C_CONST
    sa = FX * NBA * (NBA + 1) / 2
    # djik: Calpha3 = nvirt*UV*c*nocc*U1 (RIMP2.F90:182,186); Calpha4(alpha) =
    # U1*UO*nocctot*nocc*(alpha X + Y (nocc+1)/2 + Z (nocctot+1)/2) (:197,201)
    djik = (nvirt * UV * c * nocc * U1) * U1 * UO * nocctot * nocc * (
        sa + NBA * (FY * (nocc + 1) / 2 + FZ * (nocctot + 1) / 2))
    # blad: Calpha3 = nvirt*W*c*nocc*UO (:220,225); the CalphaVV DGEMM sums
    # k = 1..nocc (:232-235): Calpha4(alpha) = W*UV*nocc*nvirt*(alpha X +
    # Y (nvirt+1)/2 + Z (nocc+1)/2) (:242)
    blad = (nvirt * W * c * nocc * UO) * W * UV * nocc * nvirt * (
        sa + NBA * (FY * (nvirt + 1) / 2 + FZ * (nocc + 1) / 2))
    return djik, blad


@pytest.mark.parametrize("k", [0, 1])
def test_first_order_known_answers(k, golden):
    """The driver's first_order block on generate.F90's first-order inputs
    matches the closed forms within the reference's 1e-10 (RIMP2.F90:337,355)."""
    nvirt, nocc, noccEOS, nvirtEOS, NBA = SIZES[k]
    arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    Ca, _, _, UoE, UvT, UoT, UvE = arrs
    occ, vv = O.gen_kat_fo(NBA, nvirt, nocc, nocc)
    djik, blad = O.first_order(nvirt, nocc, noccEOS, nvirtEOS, nocc, NBA, Ca, occ, vv, UoE, UvT,
                               UoT, UvE)
    d_exp, b_exp = first_order_closed_forms(nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc)
    assert np.abs(djik - d_exp).max() <= 1e-10
    assert np.abs(blad - b_exp).max() <= 1e-10
    g = golden("first_order.npz")
    np.testing.assert_array_equal(np.array([djik.min(), djik.max()]), g[f"file{k+1}_djik"])
    np.testing.assert_array_equal(np.array([blad.min(), blad.max()]), g[f"file{k+1}_blad"])


def test_first_order_einsum_restatement(golden):
    """The oracle's first-order sequence against an independent numpy
    restatement of RIMP2.F90:177-248, with random non-unitary matrices and
    nocctot != nocc, and against the committed fixture."""
    g = golden("first_order.npz")
    nv, no, ne, ve, nb, nt = (int(g[k]) for k in ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA",
                                                 "nocctot"))
    A = {k: np.asfortranarray(g[k]) for k in ("Calpha", "CalphaOcc", "CalphaVV", "UoccEOST",
                                              "UvirtT", "UoccT", "UoccallT", "UvirtEOST")}
    djik, blad = O.first_order(nv, no, ne, ve, nt, nb, A["Calpha"], A["CalphaOcc"], A["CalphaVV"],
                               A["UoccEOST"], A["UvirtT"], A["UoccT"], A["UvirtEOST"],
                               UoccallT=A["UoccallT"])
    Ca = A["Calpha"]
    c2 = np.einsum("xbj,jl->xbl", Ca, A["UoccEOST"])                     # :182
    c3 = np.einsum("nm,xnl->xml", A["UvirtT"], c2)                       # :186 TransAlpha2
    c2b = np.einsum("xbm,mk->xbk", A["CalphaOcc"], A["UoccallT"])        # :197
    c4 = np.einsum("bl,xbk->xlk", A["UoccEOST"], c2b)                    # :201
    d_ref = np.einsum("xab,xcd->abcd", c3, c4)                           # :207
    c2 = np.einsum("xbj,jk->xbk", Ca, A["UoccT"])                        # :220
    c3 = np.einsum("bm,xbk->xmk", A["UvirtEOST"], c2)                    # :225
    Uview = A["UvirtT"].ravel(order="F")[:no * nv].reshape(no, nv, order="F")  # K = ldb = nocc
    c2b = np.einsum("xbk,kn->xbn", A["CalphaVV"][:, :, :no], Uview)     # :232-235
    c4 = np.einsum("bm,xbn->xmn", A["UvirtEOST"], c2b)                   # :242
    b_ref = np.einsum("xab,xcd->abcd", c3, c4)                           # :248
    np.testing.assert_allclose(djik, d_ref, rtol=1e-12, atol=1e-13 * np.abs(d_ref).max())
    np.testing.assert_allclose(blad, b_ref, rtol=1e-12, atol=1e-13 * np.abs(b_ref).max())
    np.testing.assert_allclose(djik, g["djik"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(blad, g["blad"], rtol=1e-13, atol=1e-15)


def test_golden_small_general_reproduces(golden):
    g = golden("small_general.npz")
    n = {k: int(g[k]) for k in ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA")}
    outs = O.steps5to8(n["nvirt"], n["nocc"], n["noccEOS"], n["nvirtEOS"], n["NBA"],
                       *(np.asfortranarray(g[k]) for k in ("Calpha", "EVocc", "EVvirt", "UoccEOST",
                                                           "UvirtT", "UoccT", "UvirtEOST")))
    for name, arr in zip(("toccEOS", "tvirtEOS", "goccEOS", "gvirtEOS"), outs):
        np.testing.assert_allclose(arr, g[name], rtol=1e-13, atol=1e-15)


def test_generator_matches_golden(golden):
    g = golden("energy_cfg1.npz")
    Ca, eo, ev = O.gen_fragment(int(g["seed"]), int(g["nocc"]), int(g["nvirt"]), int(g["NBA"]))
    np.testing.assert_allclose(Ca[:64, 0, 0], g["calpha_head"], rtol=1e-14)
    assert abs(Ca.sum() - g["calpha_sum"]) < 1e-10
    np.testing.assert_allclose(eo, g["EVocc"], rtol=1e-15)
    # synthetic distributions named by the workload definition
    assert np.all(np.diff(eo) >= 0) and eo.min() >= -1.5 and eo.max() <= -0.3
    assert np.all(np.diff(ev) >= 0) and ev.min() >= 0.1 and ev.max() <= 3.0


def test_energy_blocked_equals_faithful():
    Ca, eo, ev = O.gen_fragment(3, 6, 33, 57)
    Ep1, E1 = O.pair_energies(33, 6, 57, Ca, eo, ev)
    Ep2, E2 = O.pair_energies(33, 6, 57, Ca, eo, ev, blocked=True)
    np.testing.assert_allclose(Ep2, Ep1, rtol=1e-13)
    assert abs(E1 - E2) <= 1e-13 * abs(E1)
    assert E1 < 0 and np.all(np.diag(Ep1) < 0)


def test_energy_from_reference_arrays_identity():
    """With U = I (noccEOS=nocc, nvirtEOS=nvirt) the occupied-partitioned
    energy built from the reference's toccEOS/goccEOS and the virtual-
    partitioned one from tvirtEOS/gvirtEOS both equal the canonical E."""
    nvirt, nocc, NBA = 12, 4, 29
    Ca, eo, ev = O.gen_fragment(5, nocc, nvirt, NBA)
    I_o, I_v = np.eye(nocc, order="F"), np.eye(nvirt, order="F")
    tE, vE, gE, gvE = O.steps5to8(nvirt, nocc, nocc, nvirt, NBA, Ca, eo, ev, I_o, I_v, I_o, I_v)
    # toccEOS(a,i,b,j); exchange swaps a<->b
    e_occ = np.einsum("aibj,aibj->", tE, 2 * gE - gE.transpose(2, 1, 0, 3))
    e_vir = np.einsum("aibj,aibj->", vE, 2 * gvE - gvE.transpose(0, 3, 2, 1))
    _, E = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev)
    assert abs(e_occ - E) <= 1e-13 * abs(E)
    assert abs(e_vir - E) <= 1e-13 * abs(E)


def fused_eos_numpy(Ca, eo, ev, Uo, Uv):
    """sum_ij,ab g_ij^ab/D (2 gt_ij^ab - gt_ij^ba) with gt from Calpha
    projected by Po = Uo Uo^T and Pv = Uv Uv^T (plain numpy)."""
    Po, Pv = Uo @ Uo.T, Uv @ Uv.T
    Ct = np.einsum("ac,xck,ki->xai", Pv, Ca, Po)
    g = np.einsum("xai,xbj->iajb", Ca, Ca)
    gt = np.einsum("xai,xbj->iajb", Ct, Ct)
    D = eo[:, None, None, None] + eo[None, None, :, None] - ev[None, :, None, None] - \
        ev[None, None, None, :]
    return float(np.sum(g / D * (2 * gt - gt.transpose(0, 3, 2, 1))))


def test_fused_eos_energy_equals_reference_arrays(golden):
    """The fused local-orbital energy (projected Calpha) equals the energy
    contracted from the reference's own Step 5-8 arrays, for random
    non-unitary U (golden case): both partitionings."""
    g = golden("small_general.npz")
    A = {k: np.asarray(g[k]) for k in ("Calpha", "EVocc", "EVvirt", "UoccEOST", "UvirtT", "UoccT",
                                       "UvirtEOST")}
    e_occ, e_vir = O.energy_eos_from_arrays(g["toccEOS"], g["goccEOS"], g["tvirtEOS"],
                                            g["gvirtEOS"])
    f_occ = fused_eos_numpy(A["Calpha"], A["EVocc"], A["EVvirt"], A["UoccEOST"], A["UvirtT"])
    f_vir = fused_eos_numpy(A["Calpha"], A["EVocc"], A["EVvirt"], A["UoccT"], A["UvirtEOST"])
    assert abs(f_occ - e_occ) <= 1e-12 * abs(e_occ)
    assert abs(f_vir - e_vir) <= 1e-12 * abs(e_vir)


def test_amplitudes_match_tocca_with_identity():
    nvirt, nocc, NBA = 9, 3, 17
    Ca, eo, ev = O.gen_fragment(7, nocc, nvirt, NBA)
    tocc = O.fzeros(nocc, nocc, nvirt, nvirt)
    O.calc_toccA(nvirt, nocc, nocc, NBA, Ca, eo, ev, tocc, np.eye(nocc, order="F"))
    t = O.amplitudes(nvirt, nocc, NBA, Ca, eo, ev)  # t(a,i,b,j)
    np.testing.assert_array_equal(t, tocc.transpose(2, 0, 3, 1))


def test_datafile_roundtrip(tmp_path):
    """Calpha{1,2}.data record layout (generate.F90:75-128,333-336)."""
    nvirt, nocc, noccEOS, nvirtEOS, NBA = 7, 3, 2, 4, 11
    arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    outs = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, *arrs)
    p = str(tmp_path / "Calpha1.data")
    O.write_datafile(p, nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc, *arrs, outs[0], outs[1], outs[3],
                     outs[2])
    back = O.read_datafile(p)
    assert (back["nvirt"], back["nocc"], back["NBA"]) == (nvirt, nocc, NBA)
    np.testing.assert_array_equal(back["Calpha"], arrs[0])
    np.testing.assert_array_equal(back["goccEOS"], outs[2])
    np.testing.assert_array_equal(back["gvirtEOS"], outs[3])
    # header record: 4-byte marker 24, six int32, marker 24
    raw = open(p, "rb").read(32)
    assert np.frombuffer(raw[:4], np.int32)[0] == 24
    assert list(np.frombuffer(raw[4:28], np.int32)) == [nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc]


def test_cholesky_trsm_front_end():
    NBA, nbas, nocc = 24, 10, 2
    nvirt = nbas - nocc
    ao = O.gen_ao3c(2, NBA, nbas)
    np.testing.assert_array_equal(ao, ao.transpose(0, 2, 1))
    V = O.gen_metric(2, NBA)
    L = O.cholesky(V)
    np.testing.assert_allclose(L @ L.T, V, rtol=1e-12, atol=1e-12)
    Cm = O.gen_mo(2, nbas)
    np.testing.assert_allclose(Cm.T @ Cm, np.eye(nbas), atol=1e-12)
    B = O.ao2mo(NBA, nbas, nocc, nvirt, ao, Cm)
    ref = np.einsum("xmn,ma,ni->xai", ao, Cm[:, nocc:], Cm[:, :nocc])
    np.testing.assert_allclose(B, ref, rtol=1e-11, atol=1e-13)
    X = O.trsm_lower(L, B.reshape(NBA, -1, order="F")).reshape(B.shape, order="F")
    # Calpha^T Calpha = B^T V^-1 B
    G = np.einsum("xai,xbj->aibj", X, X)
    G2 = np.einsum("xai,xy,ybj->aibj", B, np.linalg.inv(V), B)
    np.testing.assert_allclose(G, G2, rtol=1e-9, atol=1e-12)
