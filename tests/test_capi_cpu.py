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


def test_batched_packed_input_validation():
    """The packed batched call checks its packing on the host (sizes against
    the fragment dimensions) and the library checks the dimensions before it
    touches a device."""
    from rimp2_gpu_gb300 import api, _lib
    nocc, nvirt, nba = [2, 3], [4, 5], [6, 7]
    ca = np.zeros(2 * 4 * 6 + 3 * 5 * 7)
    eo, ev = np.zeros(5), np.zeros(9)
    with pytest.raises(ValueError):
        api.energy_batched_packed(nocc, nvirt, nba, ca[:-1], eo, ev)
    with pytest.raises(ValueError):
        api.energy_batched_packed(nocc, nvirt, nba, ca, eo[:-1], ev)
    with pytest.raises(ValueError):
        api.energy_batched_packed(nocc, nvirt[:1], nba, ca, eo, ev)
    with pytest.raises(_lib.Rimp2Error) as ei:  # zero dimension: status 1 before the device
        api.energy_batched_packed([2, 0], [4, 5], [6, 7], np.zeros(48), np.zeros(2), np.zeros(9))
    assert ei.value.status == 1 and "bad dims" in str(ei.value)


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
        if b["nslices"] == 0:  # the fixed FP64 tier
            assert "rule" in b
            continue
        # one slice: the one-CTA kernel (four products) met the margin, and
        # the paired kernel (three) too unless the bucket is held to the
        # one-CTA kernel by the kernel table
        if b["nslices"] == 1:
            keys = ["1_one_cta"] + ([] if b.get("one_cta_only") else ["1_paired"])
        else:
            keys = [str(b["nslices"])]
        for key in keys:
            assert b["worst_rel_err"][key] <= t["target"] * t["margin"]
        if b.get("one_cta_only"):
            for nv in (b["nvirt_min"], b["nvirt_min"] + 1):
                assert api.split_kernel_for(nv, 64, 4096) == 1


def _raw_records(path):
    """Split a Fortran unformatted sequential file into its records."""
    out, b = [], open(path, "rb").read()
    p = 0
    while p < len(b):
        n = int(np.frombuffer(b, np.int32, 1, p)[0])
        out.append(b[p + 4:p + 4 + n])
        assert int(np.frombuffer(b, np.int32, 1, p + 4 + n)[0]) == n
        p += 8 + n
    return out


def test_datafile_reads_oracle_written_file(tmp_path):
    """The library reads a Calpha{1,2}.data file written in the record order
    of generate.F90:75-128,333-336 by the oracle."""
    from oracle import oracle as O
    from rimp2_gpu_gb300 import api
    nvirt, nocc, noccEOS, nvirtEOS, NBA = 7, 3, 2, 4, 11
    arrs = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    outs = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, *arrs)
    path = str(tmp_path / "Calpha1.data")
    O.write_datafile(path, nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc, *arrs, outs[0], outs[1],
                     outs[3], outs[2])
    d = api.read_datafile(path)
    assert (d["nvirt"], d["nocc"], d["noccEOS"], d["nvirtEOS"], d["NBA"], d["nocctot"]) == \
        (nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc)
    for name, a in zip(("Calpha", "EVocc", "EVvirt", "UoccEOST", "UvirtT", "UoccT", "UvirtEOST"),
                       arrs):
        np.testing.assert_array_equal(d[name], a)
    np.testing.assert_array_equal(d["toccEOS"], outs[0])
    np.testing.assert_array_equal(d["tvirtEOS"], outs[1])
    np.testing.assert_array_equal(d["goccEOS"], outs[2])
    np.testing.assert_array_equal(d["gvirtEOS"], outs[3])
    # inputs only: the known-answer records are skipped
    d2 = api.read_datafile(path, known_answers=False)
    assert "toccEOS" not in d2
    np.testing.assert_array_equal(d2["Calpha"], arrs[0])


def test_datafile_first_order_roundtrip_and_layout(tmp_path):
    """First-order files: CalphaOcc/CalphaVV after UvirtEOST and djik/blad
    after goccEOS (generate.F90:262,308,333-339); the library writes them
    and reads them back, and the raw records are in that order."""
    from oracle import oracle as O
    from rimp2_gpu_gb300 import api
    nvirt, nocc, noccEOS, nvirtEOS, NBA = 9, 4, 2, 3, 13
    Ca, eo, ev, UoE, UvT, UoT, UvE = O.gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS)
    occ, vv = O.gen_kat_fo(NBA, nvirt, nocc, nocc)
    tE, vE, gE, gvE = O.steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Ca, eo, ev, UoE, UvT, UoT,
                                  UvE)
    djik, blad = O.first_order(nvirt, nocc, noccEOS, nvirtEOS, nocc, NBA, Ca, occ, vv, UoE, UvT,
                               UoT, UvE)
    arrays = dict(nvirt=nvirt, nocc=nocc, noccEOS=noccEOS, nvirtEOS=nvirtEOS, NBA=NBA,
                  nocctot=nocc, Calpha=Ca, EVocc=eo, EVvirt=ev, UoccEOST=UoE, UvirtT=UvT,
                  UoccT=UoT, UvirtEOST=UvE, CalphaOcc=occ, CalphaVV=vv, toccEOS=tE,
                  tvirtEOS=vE, gvirtEOS=gvE, goccEOS=gE, djik=djik, blad=blad)
    path = str(tmp_path / "Calpha2.data")
    api.write_datafile(path, arrays, first_order=True)
    recs = _raw_records(path)
    assert len(recs) == 16
    np.testing.assert_array_equal(np.frombuffer(recs[0], np.int32),
                                  [nvirt, nocc, noccEOS, nvirtEOS, NBA, nocc])
    order = ["Calpha", "EVocc", "EVvirt", "UoccEOST", "UvirtT", "UoccT", "UvirtEOST", "CalphaOcc",
             "CalphaVV", "toccEOS", "tvirtEOS", "gvirtEOS", "goccEOS", "djik", "blad"]
    for rec, name in zip(recs[1:], order):
        np.testing.assert_array_equal(np.frombuffer(rec, np.float64),
                                      np.asarray(arrays[name]).ravel(order="F"))
    d = api.read_datafile(path, first_order=True)
    for name in order:
        np.testing.assert_array_equal(d[name], arrays[name])


def test_datafile_rejects_bad_files(tmp_path):
    from rimp2_gpu_gb300 import api, _lib
    good = tmp_path / "ok.data"
    Ca = np.zeros((5, 3, 2), order="F")
    arrays = dict(nvirt=3, nocc=2, noccEOS=1, nvirtEOS=1, NBA=5, nocctot=2, Calpha=Ca,
                  EVocc=np.zeros(2), EVvirt=np.zeros(3), UoccEOST=np.zeros((2, 1)),
                  UvirtT=np.zeros((3, 3)), UoccT=np.zeros((2, 2)), UvirtEOST=np.zeros((3, 1)))
    api.write_datafile(str(good), arrays)
    d = api.read_datafile(str(good), known_answers=False)
    assert d["Calpha"].shape == (5, 3, 2)
    with pytest.raises(_lib.Rimp2Error):  # known answers requested but absent
        api.read_datafile(str(good))
    b = bytearray(good.read_bytes())
    bad = tmp_path / "bad.data"
    bad.write_bytes(bytes(b[:len(b) - 10]))  # truncated
    with pytest.raises(_lib.Rimp2Error):
        api.read_datafile(str(bad), known_answers=False)
    b[32] ^= 0xFF  # corrupt the Calpha record's length marker
    bad.write_bytes(bytes(b))
    with pytest.raises(_lib.Rimp2Error) as ei:
        api.read_datafile(str(bad), known_answers=False)
    assert ei.value.status == 1
    with pytest.raises(_lib.Rimp2Error):
        api.read_datafile(str(tmp_path / "missing.data"))


def test_split_kernel_report_before_any_launch():
    """The kernel-choice report is a host-side read: 0 in a fresh process
    before any split launch."""
    import subprocess
    import sys
    out = subprocess.run([sys.executable, "-c", "from rimp2_gpu_gb300 import api; "
                          "print(api.last_split_kernel())"], cwd=ROOT, capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "0"


def test_fortran_module_matches_header():
    """Every bind(C) interface of the Fortran module names a function that
    include/rimp2_gpu.h declares and the library exports, with the same
    number of arguments (the module cannot be compiled here: no Fortran
    compiler in this run)."""
    import ctypes
    import re
    hdr = open(os.path.join(ROOT, "include", "rimp2_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|long long|const char\s*\*)\s*(rimp2_\w+)\s*\(([^)]*)\)\s*;", hdr):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    f90 = open(os.path.join(ROOT, "rimp2_gpu_gb300", "fortran", "rimp2_gpu_interfaces.F90")).read()
    f90 = re.sub(r"&\s*\n\s*&?", " ", f90)  # join continuation lines
    found = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"",
                       f90, flags=re.I)
    assert len(found) == f90.count("bind(C, name=")
    lib = ctypes.CDLL(os.path.join(ROOT, "rimp2_gpu_gb300", "librimp2_gpu_gb300.so"))
    for fname, args, cname in found:
        assert cname in protos, f"{cname} is not declared in rimp2_gpu.h"
        nargs = 0 if not args.strip() else args.count(",") + 1
        assert nargs == protos[cname], f"{cname}: {nargs} Fortran arguments, {protos[cname]} in C"
        assert hasattr(lib, cname), f"{cname} is not exported"


def test_kernel_rule_table(monkeypatch):
    """The energy-kernel table of the one-residual-slice split form is a
    host-side lookup: per virtual bucket, the paired-CTA kernel where nocc
    and NBA reach the bucket's thresholds; two-slice shapes run the one-CTA
    kernel, tiny ones the FP64 tier; the environment overrides the table."""
    from rimp2_gpu_gb300 import api, _lib
    monkeypatch.delenv("RIMP2_PAIR_KERNEL", raising=False)
    api.set_split_buckets([0, 16, 128, 192], [0, 2, 2, 1])
    try:
        api.set_split_kernel_rule([0, 256], [10, 4], [1024, 512])
        assert api.split_kernel_for(200, 12, 1024) == 2
        assert api.split_kernel_for(200, 8, 2048) == 1   # nocc below the first bucket's 10
        assert api.split_kernel_for(200, 12, 512) == 1   # NBA below 1024
        assert api.split_kernel_for(300, 4, 512) == 2    # second bucket
        assert api.split_kernel_for(300, 3, 4096) == 1
        assert api.split_kernel_for(100, 40, 4096) == 1  # two residual slices: one-CTA only
        assert api.split_kernel_for(8, 4, 4096) == 0     # FP64 tier
        monkeypatch.setenv("RIMP2_PAIR_KERNEL", "1")
        assert api.split_kernel_for(300, 3, 64) == 2
        monkeypatch.setenv("RIMP2_PAIR_KERNEL", "0")
        assert api.split_kernel_for(200, 12, 1024) == 1
        monkeypatch.delenv("RIMP2_PAIR_KERNEL")
        for bad in (([0, 0], [10, 4], [1024, 512]), ([0], [0], [1024]), ([0], [10], [0])):
            with pytest.raises(_lib.Rimp2Error):
                api.set_split_kernel_rule(*bad)
    finally:
        from rimp2_gpu_gb300 import autotune
        autotune.load(os.path.join(ROOT, "rimp2_gpu_gb300", "tuning", "split_buckets.json"))


def test_kernel_rule_fit():
    """The autotuner keeps the thresholds that minimise the summed time of
    its grid, and 'never' when the paired kernel wins nowhere."""
    from rimp2_gpu_gb300 import autotune as A
    grid = [{"nocc": o, "NBA": b, "one_ms": 1.0,
             "pair_ms": 0.8 if (o >= 12 and b >= 2048) else 1.3}
            for o in A.KGRID_NOCC for b in A.KGRID_NBA]
    t, mo, mb = A._fit_rule(grid)
    assert (mo, mb) == (12, 2048)
    assert abs(t - (len(grid) - 0.2 * 3 * 2)) < 1e-9
    for g in grid:
        g["pair_ms"] = 2.0
    _, mo, mb = A._fit_rule(grid)
    assert mo == A.NEVER or mb == A.NEVER


def test_tuned_tables_match_library_defaults():
    """The library's built-in tables are the committed autotuner output."""
    import json
    import subprocess
    import sys
    t = json.load(open(os.path.join(ROOT, "rimp2_gpu_gb300", "tuning", "split_buckets.json")))
    code = ("from rimp2_gpu_gb300 import api\n"
            "import json, sys\n"
            "t = json.loads(sys.argv[1])\n"
            "for b in t['buckets']:\n"
            "    assert api.split_nslices(max(b['nvirt_min'], 64), 4, 64) == b['nslices'] or "
            "b['nvirt_min'] < 16, b\n"
            "rules = t.get('kernel_rule', [])\n"
            "for k, r in enumerate(rules):\n"
            "    if r['nvirt_min'] == 0 and len(rules) > 1: continue\n"
            "    nv = max(r['nvirt_min'], 192)\n"
            "    if k + 1 < len(rules) and nv >= rules[k + 1]['nvirt_min']: continue\n"
            "    if api.split_nslices(nv, 64, 4096) != 1: continue\n"
            "    mo, mb = r['min_nocc'], r['min_nba']\n"
            "    if mo < 65536 and mb < 65536:\n"
            "        assert api.split_kernel_for(nv, mo, mb) == 2, r\n"
            "    if mo > 1 and mo < 65536:\n"
            "        assert api.split_kernel_for(nv, mo - 1, max(mb, 1) if mb < 65536 else 64) == 1, r\n"
            "    if mb > 1 and mb < 65536:\n"
            "        assert api.split_kernel_for(nv, max(mo, 64) if mo < 65536 else 64, mb - 1) == 1, r\n")
    out = subprocess.run([sys.executable, "-c", code, json.dumps(t)], cwd=ROOT,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
