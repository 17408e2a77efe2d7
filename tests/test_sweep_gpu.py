"""Seeded sweep over small ragged fragment shapes (1 <= nocc <= 20,
1 <= nvirt <= 260, 1 <= NBA <= 700, plus the tiniest split shapes: nocc 1-3
with 16 <= nvirt <= 63), each checked against the CPU oracle: single-fragment
FP64 (1e-11 relative per pair and total) and split (1e-7 on every shape; the
library sends fragments with fewer than 64 (a,i) columns to its FP64 tier),
and the same shapes as one batch through the host batched call in both
precisions."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

_g = np.random.Generator(np.random.Philox(2024))
SHAPES = [(int(o), int(v), int(b)) for o, v, b in zip(_g.integers(1, 21, 20),
                                                         _g.integers(1, 261, 20),
                                                         _g.integers(1, 701, 20))]
SHAPES += [(1, 1, 1), (1, 129, 1), (20, 1, 700), (2, 257, 65)]
# nocc in {1,2,3}, 16 <= nvirt <= 63: either side of the 64-column FP64 tier
_t = np.random.Generator(np.random.Philox(2025))
SHAPES += [(o, int(v), int(b)) for o in (1, 2, 3)
           for v, b in zip(_t.integers(16, 64, 3), _t.integers(32, 701, 3))]


@pytest.fixture(scope="module")
def cases():
    out = []
    for k, (nocc, nvirt, NBA) in enumerate(SHAPES):
        Ca, eo, ev = O.gen_fragment(900 + k, nocc, nvirt, NBA)
        Ep, E = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
        out.append((Ca, eo, ev, Ep, E))
    return out


def _tol_split(nocc, nvirt):
    return 1e-7


def _check(Ep, E, ref_Ep, ref_E, tol):
    rel = np.abs(Ep - ref_Ep) / np.abs(ref_Ep)
    assert rel.max() <= tol, rel.max()
    assert abs(E - ref_E) <= tol * abs(ref_E)


@pytest.mark.parametrize("k", range(len(SHAPES)))
def test_sweep_single_fragment(cases, k):
    from rimp2_gpu_gb300 import api
    Ca, eo, ev, ref_Ep, ref_E = cases[k]
    NBA, nvirt, nocc = Ca.shape
    Ep, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_FP64)
    _check(Ep, E, ref_Ep, ref_E, 1e-11)
    Ep, E = api.energy(nvirt, nocc, NBA, Ca, eo, ev, precision=api.PREC_SPLIT)
    _check(Ep, E, ref_Ep, ref_E, _tol_split(nocc, nvirt))


@pytest.mark.parametrize("prec", [0, 1])
def test_sweep_as_one_batch(cases, prec):
    from rimp2_gpu_gb300 import api
    res = api.energy_batched([(c[0], c[1], c[2]) for c in cases], precision=prec)
    for (Ep, E), c, (nocc, nvirt, _) in zip(res, cases, SHAPES):
        _check(Ep, E, c[3], c[4], 1e-11 if prec == 0 else _tol_split(nocc, nvirt))
