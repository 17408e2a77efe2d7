"""Generate the committed golden fixtures under tests/golden/ with the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py

Each .npz holds the seeded inputs and the oracle outputs of one small case,
so GPU parity tests compare against fixed vectors without regenerating
inputs (the generators use libm, whose last bits may differ across hosts).

  small_general.npz : Steps 5-8 of RIMP2.F90:71-170 with random, non-unitary
                      rotation matrices (ragged sizes nvirt=21, nocc=5,
                      noccEOS=3, nvirtEOS=7, NBA=37), plus toccA/tvirtA
                      intermediates and the first-order gen4DimFO product.
  energy_cfg1.npz   : MP2 pair energies, total and a slice of amplitudes for
                      nocc=16, nvirt=96, NBA=384 (seed 1; the reference-sized
                      CPU-runnable fragment).  Calpha itself is regenerated
                      from the seed at test time and checked against the
                      stored checksums.
  kat.npz           : outputs of the constant-valued fixtures of
                      generate.F90:77-128 at both shipped sizes.
  first_order.npz   : the driver's first-order block (RIMP2.F90:172-251):
                      djik and blad of a small case with random non-unitary
                      matrices and nocctot != nocc (a separate UoccallT), and
                      the min/max of djik and blad from the generate.F90
                      first-order fixture inputs (:254-260,300-306) at both
                      shipped sizes (every element is the same constant).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402


def small_general():
    nvirt, nocc, noccEOS, nvirtEOS, NBA = 21, 5, 3, 7, 37
    seed = 11
    Ca, eo, ev = O.gen_fragment(seed, nocc, nvirt, NBA)
    UoE = O.gen_matrix(seed, 10, nocc, noccEOS)
    UvT = O.gen_matrix(seed, 11, nvirt, nvirt)
    UoT = O.gen_matrix(seed, 12, nocc, nocc)
    UvE = O.gen_matrix(seed, 13, nvirt, nvirtEOS)
    tE, vE, gE, gvE = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Ca, eo, ev, UoE, UvT, UoT, UvE)
    tocc = O.fzeros(nocc, noccEOS, nvirt, nvirt)
    O.calc_toccA(nvirt, nocc, noccEOS, NBA, Ca, eo, ev, tocc, UoE)
    tvirt = O.fzeros(nocc, nocc, nvirtEOS, nvirt)
    O.calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, Ca, eo, ev, tvirt, UvE)
    # first-order product gen4DimFO(NBA, X(NBA,nvirt,nocc), Y(NBA,nocc,noccEOS))
    Y = np.asfortranarray(Ca[:, :nocc, :noccEOS])
    djik = O.fzeros(nvirt, nocc, nocc, noccEOS)
    O.calc_gen4DimFO(NBA, Ca, nvirt, nocc, Y, nocc, noccEOS, djik)
    np.savez_compressed(os.path.join(HERE, "small_general.npz"), nvirt=nvirt, nocc=nocc,
                        noccEOS=noccEOS, nvirtEOS=nvirtEOS, NBA=NBA, Calpha=Ca, EVocc=eo,
                        EVvirt=ev, UoccEOST=UoE, UvirtT=UvT, UoccT=UoT, UvirtEOST=UvE, toccEOS=tE,
                        tvirtEOS=vE, goccEOS=gE, gvirtEOS=gvE, tocc=tocc, tvirt=tvirt, Y=Y,
                        djik=djik)


def energy_cfg1():
    nocc, nvirt, NBA, seed = 16, 96, 384, 1
    Ca, eo, ev = O.gen_fragment(seed, nocc, nvirt, NBA)
    Ep, E = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev)
    t = O.amplitudes(nvirt, nocc, NBA, Ca, eo, ev)
    np.savez_compressed(os.path.join(HERE, "energy_cfg1.npz"), nocc=nocc, nvirt=nvirt, NBA=NBA,
                        seed=seed, calpha_sum=Ca.sum(), calpha_abssum=np.abs(Ca).sum(),
                        calpha_head=Ca[:64, 0, 0].copy(), EVocc=eo, EVvirt=ev, Epair=Ep, Etot=E,
                        t_slice=np.asfortranarray(t[:, :, :8, :2]))


def kat():
    out = {}
    for k, (nvirt, nocc, noccEOS, nvirtEOS, NBA) in enumerate([(74, 10, 4, 15, 273),
                                                                (104, 20, 4, 15, 373)], 1):
        arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
        tE, vE, gE, gvE = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, *arrs)
        for name, a in zip(("toccEOS", "tvirtEOS", "goccEOS", "gvirtEOS"), (tE, vE, gE, gvE)):
            # every element is the same closed-form constant: keep min/max
            out[f"file{k}_{name}"] = np.array([a.min(), a.max()])
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **out)


def first_order():
    nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot = 21, 5, 3, 7, 37, 8
    seed = 12
    Ca = O.gen_calpha(seed, NBA, nvirt, nocc)
    occ = O.gen_matrix(seed, 20, NBA * nocc, nocctot).reshape(NBA, nocc, nocctot, order="F")
    vv = O.gen_matrix(seed, 21, NBA * nvirt, nvirt).reshape(NBA, nvirt, nvirt, order="F")
    UoE = O.gen_matrix(seed, 10, nocc, noccEOS)
    UvT = O.gen_matrix(seed, 11, nvirt, nvirt)
    UoT = O.gen_matrix(seed, 12, nocc, nocc)
    UoA = O.gen_matrix(seed, 14, nocctot, nocctot)
    UvE = O.gen_matrix(seed, 13, nvirt, nvirtEOS)
    occ, vv = np.asfortranarray(occ), np.asfortranarray(vv)
    djik, blad = O.first_order(nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA, Ca, occ, vv, UoE, UvT,
                               UoT, UvE, UoccallT=UoA)
    out = dict(nvirt=nvirt, nocc=nocc, noccEOS=noccEOS, nvirtEOS=nvirtEOS, NBA=NBA, nocctot=nocctot,
               Calpha=Ca, CalphaOcc=occ, CalphaVV=vv, UoccEOST=UoE, UvirtT=UvT, UoccT=UoT,
               UoccallT=UoA, UvirtEOST=UvE, djik=djik, blad=blad)
    for k, (nvirt, nocc, noccEOS, nvirtEOS, NBA) in enumerate([(74, 10, 4, 15, 273),
                                                                (104, 20, 4, 15, 373)], 1):
        Ca, eo, ev, UoE, UvT, UoT, UvE = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
        occ, vv = O.gen_kat_fo(NBA, nvirt, nocc, nocc)
        d, b = O.first_order(nvirt, nocc, noccEOS, nvirtEOS, nocc, NBA, Ca, occ, vv, UoE, UvT, UoT,
                             UvE)
        out[f"file{k}_djik"] = np.array([d.min(), d.max()])
        out[f"file{k}_blad"] = np.array([b.min(), b.max()])
    np.savez_compressed(os.path.join(HERE, "first_order.npz"), **out)


if __name__ == "__main__":
    small_general()
    energy_cfg1()
    first_order()
    kat()
    print("golden fixtures written to", HERE)
