"""CPU emulation of the split-precision products (no GPU): the slicing of
the energy kernels restated in numpy (power-of-two column scales, S0 an
integer with ||S0||_2 <= 2^12, R1 and V = fp16(C s) rounded to FP16), the
contractions done in float64 so that only the slicing error remains.

Checks the argument for the paired kernel's three-product form: folding
R1a S0b + R1a R1b into R1a V leaves a same-column bias on g_ii(a,a) that the
per-column correction sum_k R1 (V - S0 - R1) removes, after which the pair
energies are as close to FP64 as with the exact four products."""
import numpy as np

from oracle import oracle as O


def slices(C):
    K = C.shape[0]
    mx = np.abs(C).max(axis=0)
    nrm = np.sqrt((C * C).sum(axis=0))
    e = np.floor(np.log2(np.minimum(2047.5 / mx, (4096.0 - 0.5 * np.sqrt(K)) / nrm)))
    while True:
        S0 = np.rint(C * 2.0 ** e)
        bad = (S0 * S0).sum(axis=0) > 2 ** 24
        if not bad.any():
            break
        e[bad] -= 1
    X = C * 2.0 ** e
    S0 = np.rint(X)
    R1 = (X - S0).astype(np.float16).astype(np.float64)
    V = X.astype(np.float16).astype(np.float64)
    return S0, R1, V, 2.0 ** (-e)


def pair_energies(G, eo, ev, nocc, nvirt):
    G4 = G.reshape(nocc, nvirt, nocc, nvirt)  # [i, a, j, b]
    E = np.empty((nocc, nocc))
    for i in range(nocc):
        for j in range(nocc):
            g = G4[i, :, j, :]
            D = eo[i] + eo[j] - ev[:, None] - ev[None, :]
            E[i, j] = (g * (2 * g - g.T) / D).sum()
    return E


def test_three_product_form_with_diagonal_correction():
    worst = {"4": 0.0, "3": 0.0, "3c": 0.0}
    diag_bias = {"3": 0.0, "3c": 0.0}
    for nocc, nvirt, NBA, seed in [(4, 128, 2048, 1), (3, 256, 1024, 2), (5, 96, 512, 3)]:
        Ca, eo, ev = O.gen_fragment(seed, nocc, nvirt, NBA)
        C = np.asarray(Ca).reshape(NBA, nvirt * nocc, order="F")
        E0 = pair_energies(C.T @ C, eo, ev, nocc, nvirt)
        S0, R1, V, inv = slices(C)
        sc = np.outer(inv, inv)
        G4 = (S0.T @ S0 + S0.T @ R1 + R1.T @ S0 + R1.T @ R1) * sc
        G3 = (S0.T @ S0 + S0.T @ R1 + R1.T @ V) * sc
        G3c = G3.copy()
        d = (R1 * (V - S0 - R1)).sum(axis=0)
        idx = np.arange(G3.shape[0])
        G3c[idx, idx] -= d * inv * inv
        for key, G in (("4", G4), ("3", G3), ("3c", G3c)):
            rel = np.abs(pair_energies(G, eo, ev, nocc, nvirt) - E0) / np.abs(E0)
            worst[key] = max(worst[key], rel.max())
            if key in diag_bias:
                diag_bias[key] = max(diag_bias[key], np.diag(rel).max())
    print(f"\nworst pair error: four products {worst['4']:.2e}, three {worst['3']:.2e}, "
          f"three + correction {worst['3c']:.2e}")
    assert worst["4"] < 1e-7 and worst["3c"] < 1e-7
    # the correction removes most of the i=j bias and lands near the exact form
    assert diag_bias["3c"] < 0.6 * diag_bias["3"]
    assert worst["3c"] <= 1.5 * worst["4"] + 5e-9
