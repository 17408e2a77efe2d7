"""The allocation-free FP64 energy entry point, through the C-ABI.

Callers such as a Fortran/OpenACC driver that already owns the device memory
cannot let the library allocate; rimp2_energy_fp64_noalloc_dev works out of a
fixed device array instead.  Its energies must match the CPU oracle and the
regular FP64 entry point (the 1e-11 relative tolerance of the FP64 parity
tests) on two calls in a row, the second reusing the array left by the first,
and the second call must leave the device's free memory unchanged.  Collected
last so that a failure here never hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).ravel(order="F")).cuda()


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    from rimp2_gpu_gb300 import _lib, api
    L = _lib.lib()
    cases = [(7, 96, 200, 41), (4, 130, 77, 42)]
    for nocc, nvirt, NBA, seed in cases:
        Ca, eo, ev = O.gen_fragment(seed, nocc, nvirt, NBA)
        dC = _dev(Ca.reshape(-1, order="F"))
        deo, dev = _dev(eo), _dev(ev)
        ref_E = torch.zeros(nocc * nocc, dtype=torch.float64, device="cuda")
        ref_T = torch.zeros(1, dtype=torch.float64, device="cuda")
        api.energy_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(), dev.data_ptr(),
                       ref_E.data_ptr(), ref_T.data_ptr(), precision=api.PREC_FP64)
        torch.cuda.synchronize()
        Er = ref_E.cpu().numpy()
        Tr = ref_T.item()
        Eo, To = O.pair_energies(nvirt, nocc, NBA, Ca, eo, ev, blocked=True)
        Eo = np.asarray(Eo).ravel(order="F")
        for call in range(2):
            dE = torch.full((nocc * nocc,), np.nan, dtype=torch.float64, device="cuda")
            dT = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            free0 = api.get_dev_mem()[1]
            st = L.rimp2_energy_fp64_noalloc_dev(nvirt, nocc, NBA, dC.data_ptr(), deo.data_ptr(),
                                                 dev.data_ptr(), dE.data_ptr(), dT.data_ptr(),
                                                 None)
            assert st == 0, L.rimp2_last_error_string()
            torch.cuda.synchronize()
            free1 = api.get_dev_mem()[1]
            if call == 1:
                assert free1 == free0, f"device free memory moved by {free0 - free1} bytes"
            E = dE.cpu().numpy()
            rel = np.abs(E - Er) / np.abs(Er)
            assert rel.max() <= 1e-11, (call, rel.max())
            assert abs(dT.item() - Tr) <= 1e-11 * abs(Tr), call
            rel_o = np.abs(E - Eo) / np.abs(Eo)
            assert rel_o.max() <= 1e-11, ("oracle", call, rel_o.max())
            assert abs(dT.item() - To) <= 1e-11 * abs(To), ("oracle total", call)


def test_noalloc_rejects_fragments_above_its_limit():
    import torch
    from rimp2_gpu_gb300 import _lib
    L = _lib.lib()
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    # nocc=512, nvirt=2048: 131328 pairs x 528 tile pairs of partials >> 16 MiB
    st = L.rimp2_energy_fp64_noalloc_dev(2048, 512, 64, p, p, p, p, p, None)
    assert st == 1
    assert b"limit" in L.rimp2_last_error_string()
