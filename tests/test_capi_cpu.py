"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol the header declares, validates arguments before touching the device,
and reports the absence of a GPU as a status instead of falling back."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "rimp2_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rimp2_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from rimp2_gpu_gb300 import _lib
    L = _lib.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
        assert s in _lib.SIGNATURES, f"{s} missing from the ctypes signature table"


def test_version_and_error_string():
    from rimp2_gpu_gb300 import _lib
    assert b"sm_103a" in _lib.lib().rimp2_version()
    assert isinstance(_lib.lib().rimp2_last_error_string(), bytes)


def test_argument_validation_before_device():
    from rimp2_gpu_gb300 import api, _lib
    Ca = np.zeros((4, 3, 2), order="F")
    eo, ev = np.zeros(2), np.zeros(3)
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.energy(3, 2, 4, Ca, eo, ev, precision=7)
    assert ei.value.status == 1 and "precision" in str(ei.value)
    i = lambda v: C.byref(C.c_int(v))  # noqa: E731
    st = _lib.lib().rimp2_calc_tocca(i(0), i(2), i(2), i(4), None, None, None, None, None)
    assert st == 1
    assert b"bad dims" in _lib.lib().rimp2_last_error_string()


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU status path")
def test_no_gpu_reports_status_not_fallback():
    from rimp2_gpu_gb300 import api, _lib
    Ca = np.zeros((4, 3, 2), order="F")
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.energy(3, 2, 4, Ca, np.zeros(2), np.zeros(3))
    assert ei.value.status == 4


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from rimp2_gpu_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(ImportError):
        _lib.lib()


def test_product_does_not_import_oracle():
    pkg = os.path.join(ROOT, "rimp2_gpu_gb300")
    for dp, _, fs in os.walk(pkg):
        for f in fs:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".F90")):
                txt = open(os.path.join(dp, f)).read()
                assert "oracle" not in txt.replace("the oracle is", ""), f


def test_default_buckets_match_committed_tuning_table():
    import json
    from rimp2_gpu_gb300 import api
    t = json.load(open(os.path.join(ROOT, "rimp2_gpu_gb300", "tuning", "split_buckets.json")))
    for b in t["buckets"]:
        for nv in (b["nvirt_min"], b["nvirt_min"] + 1):
            assert api.split_nslices(max(nv, 1), 8, 256) == b["nslices"] or any(
                c["nvirt_min"] <= nv and c["nvirt_min"] > b["nvirt_min"] for c in t["buckets"])
        assert b["worst_rel_err"][str(b["nslices"])] <= t["target"] * t["margin"]
