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


def _f32(bits):
    return np.array([bits], dtype=np.uint32).view(np.float32)[0]


def split_f32_emulated(x, e):
    """The device split of a double x with |x 2^e| < 2^22 (split_f32 in
    split_kernels.cu) restated step by step in numpy float32: f_hi from the
    top 24 significant bits (bit moves only), f_lo from the next 23 bits via
    the 2^23 magic constant, q = round(f_hi) via 1.5 * 2^23, r = (f_hi - q)
    + f_lo, the sign of x applied to both; below 2^-40 of the scaled unit,
    zeros and subnormals give q = r = 0."""
    b = int(np.array([x], dtype=np.float64).view(np.uint64)[0])
    hi, lo = b >> 32, b & 0xFFFFFFFF
    sgn = hi & 0x80000000
    ed = (hi >> 20) & 0x7FF
    E = ed - 1023 + e
    if ed == 0 or E < -40:
        return np.float32(0.0), np.float32(0.0)
    frac23 = ((hi << 3) | (lo >> 29)) & 0x7FFFFF
    fhi = _f32(((E + 127) << 23) | frac23)
    lo23 = np.float32(_f32(0x4B000000 | ((lo >> 6) & 0x7FFFFF)) - np.float32(8388608.0))
    flo = np.float32(lo23 * _f32((E - 46 + 127) << 23))
    qm = np.float32(np.float32(fhi + np.float32(12582912.0)) - np.float32(12582912.0))
    rm = np.float32(np.float32(fhi - qm) + flo)
    return (-qm, -rm) if sgn else (qm, rm)


def test_fp32_split_of_doubles_against_exact_arithmetic():
    """q is an integer within the bound, q + r equals x 2^e to 2^-25 of |r|
    plus the 2^-37 dropped below f_lo (checked in exact rationals), and
    |r| <= 1/2 whenever |x 2^e| >= 1 (round half to even)."""
    from fractions import Fraction
    rng = np.random.default_rng(3)
    for bound in (511.5, 2047.5):
        for _ in range(4000):
            e = int(rng.integers(-60, 60))
            mag = float(rng.choice([rng.uniform(0, bound), 10 ** rng.uniform(-14, np.log10(bound)),
                                    bound, 0.5, 1.5, 2.5]))
            x = np.ldexp(min(mag, bound), -e) * (1 if rng.random() < 0.5 else -1)
            q, r = split_f32_emulated(x, e)
            v = Fraction(float(x)) * Fraction(2) ** e
            assert float(q) == int(q) and abs(q) <= bound + 0.5
            err = abs(Fraction(float(q)) + Fraction(float(r)) - v)
            assert err <= Fraction(abs(float(r))) * Fraction(1, 2 ** 24) + Fraction(1, 2 ** 36)
            if abs(v) >= 1:
                assert abs(Fraction(float(r))) <= Fraction(1, 2) + Fraction(1, 2 ** 20)


def col_scale_exponent_emulated(mx, ss, K):
    """The slicers' column exponent in integer and FP32 arithmetic (numpy
    float32 operations are correctly rounded, like the kernel's sqrtf and
    division)."""
    if mx == 0.0:
        return 0
    b = int(np.float64(mx).view(np.uint64))
    ed = b >> 52
    if ed == 0:
        return 100
    e1 = (10 if (b & ((1 << 52) - 1)) <= (0xFFE00 << 32) else 9) - (ed - 1023)
    e2 = 127
    ss = np.float32(ss)
    if ss > 0:
        f = np.float32
        r = (f(4096.0) - f(0.5) * np.sqrt(f(K))) / np.sqrt(ss) * f(0.99999905)
        e2 = int((int(np.float32(r).view(np.uint32)) >> 23) & 0xFF) - 127
    return max(-100, min(100, min(e1, e2)))


def test_column_exponent_without_fp64_math():
    """The integer/FP32 exponent keeps |C 2^e| <= 2047.5 exactly and the
    column norm within 4096 - sqrt(K)/2, and is the FP64 formula's exponent
    or one below it (the FP32 margin)."""
    rng = np.random.default_rng(11)
    lower = 0
    for t in range(3000):
        K = int(rng.integers(1, 5000))
        scale = 10.0 ** rng.uniform(-15, 15)  # squares within FP32 range
        C = rng.standard_normal(K) * scale
        if t % 3 == 0:  # a dominant element with mantissa near 2 - 2^-11
            m = float(rng.choice([2 - 2.0 ** -11, np.nextafter(2 - 2.0 ** -11, 2), 1.0, 1.9995]))
            C[int(rng.integers(K))] = np.ldexp(m, int(np.floor(np.log2(scale))) + 4)
        mx = float(np.abs(C).max())
        ss = float(np.float32((C * C).sum()))
        nrm = np.sqrt(ss) * (1.0 + 1e-6)
        lim = min(2047.5 / mx, (4096.0 - 0.5 * np.sqrt(K)) / nrm)
        e_old = max(-100, min(100, int(np.floor(np.log2(lim)))))
        e = col_scale_exponent_emulated(mx, ss, K)
        assert mx * 2.0 ** e <= 2047.5
        assert np.sqrt((C * C).sum()) * 2.0 ** e <= 4096.0 - 0.5 * np.sqrt(K)
        assert e_old - 1 <= e <= e_old
        # the FP64 formula's 2047.5 / mx rounds up to a power of two for a
        # mantissa just above 2 - 2^-11, where its exponent breaks the bound
        lower += e < e_old and mx * 2.0 ** e_old <= 2047.5
    assert lower < 10  # the FP32 margin costs a bit only near a power of two
    assert col_scale_exponent_emulated(0.0, 0.0, 64) == 0
    assert col_scale_exponent_emulated(np.float64(1e-310), 0.0, 64) == 100
