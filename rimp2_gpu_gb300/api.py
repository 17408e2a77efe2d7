"""Python mirror of the reference's subroutine interface, over the C-ABI.

Every function keeps the argument list of the RIMP2.F90 subroutine it
replaces (januseriksen/rimp2_gpu, file:line in each docstring); arrays are
numpy ``float64`` in Fortran order with the reference's explicit shapes and
outputs are written in place, as the Fortran ``intent(inout)`` dummies are.
A failing call raises :class:`Rimp2Error` carrying the library's status and
message; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Rimp2Error, call, lib  # noqa: F401

_dp = C.POINTER(C.c_double)

PREC_FP64 = 0
PREC_SPLIT = 1


def _i(v):
    return C.byref(C.c_int(int(v)))


def _a(x, name, shape=None, writable=False):
    if not isinstance(x, np.ndarray) or x.dtype != np.float64:
        raise TypeError(f"{name} must be a float64 numpy array")
    if not (x.flags.f_contiguous or x.ndim <= 1):
        raise ValueError(f"{name} must be Fortran-ordered")
    if shape is not None and x.size != int(np.prod(shape)):
        raise ValueError(f"{name} has {x.size} elements, expected shape {tuple(shape)}")
    if writable and not x.flags.writeable:
        raise ValueError(f"{name} must be writable")
    return x.ctypes.data_as(_dp)


def calc_toccA(nvirt, nocc, noccEOS, NBA, Calpha, EVocc, EVvirt, tocc, UoccEOST):
    """RIMP2_calc_toccA (RIMP2.F90:381-417)."""
    call("rimp2_calc_tocca", _i(nvirt), _i(nocc), _i(noccEOS), _i(NBA),
         _a(Calpha, "Calpha", (NBA, nvirt, nocc)), _a(EVocc, "EVocc", (nocc,)),
         _a(EVvirt, "EVvirt", (nvirt,)), _a(tocc, "tocc", (nocc, noccEOS, nvirt, nvirt), True),
         _a(UoccEOST, "UoccEOST", (nocc, noccEOS)))


def calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, Calpha, EVocc, EVvirt, tvirt, UvirtEOST):
    """RIMP2_calc_tvirtA (RIMP2.F90:419-453)."""
    call("rimp2_calc_tvirta", _i(nvirt), _i(nocc), _i(nvirtEOS), _i(NBA),
         _a(Calpha, "Calpha", (NBA, nvirt, nocc)), _a(EVocc, "EVocc", (nocc,)),
         _a(EVvirt, "EVvirt", (nvirt,)), _a(tvirt, "tvirt", (nocc, nocc, nvirtEOS, nvirt), True),
         _a(UvirtEOST, "UvirtEOST", (nvirt, nvirtEOS)))


def calc_toccB(nvirt, noccEOS, tocc, UvirtT, toccEOS):
    """RIMP2_calc_toccB (RIMP2.F90:456-481)."""
    call("rimp2_calc_toccb", _i(nvirt), _i(noccEOS),
         _a(tocc, "tocc", (noccEOS, noccEOS, nvirt, nvirt)), _a(UvirtT, "UvirtT", (nvirt, nvirt)),
         _a(toccEOS, "toccEOS", (nvirt, noccEOS, nvirt, noccEOS), True))


def calc_tvirtB(nvirtEOS, nocc, tvirt, UoccT, tvirtEOS):
    """RIMP2_calc_tvirtB (RIMP2.F90:483-508)."""
    call("rimp2_calc_tvirtb", _i(nvirtEOS), _i(nocc),
         _a(tvirt, "tvirt", (nocc, nocc, nvirtEOS, nvirtEOS)), _a(UoccT, "UoccT", (nocc, nocc)),
         _a(tvirtEOS, "tvirtEOS", (nvirtEOS, nocc, nvirtEOS, nocc), True))


def TransAlpha1(nvirt, noccEOS, nba, UvirtT, AlphaCD4, AlphaCD5):
    """RIMP2_TransAlpha1 (RIMP2.F90:510-533)."""
    call("rimp2_transalpha1", _i(nvirt), _i(noccEOS), _i(nba), _a(UvirtT, "UvirtT", (nvirt, nvirt)),
         _a(AlphaCD4, "AlphaCD4", (nba, nvirt, noccEOS)),
         _a(AlphaCD5, "AlphaCD5", (nba, nvirt, noccEOS), True))


def TransAlpha2(n2, n1, n3, nba, U, AlphaCD4, AlphaCD5):
    """RIMP2_TransAlpha2 (RIMP2.F90:536-560)."""
    call("rimp2_transalpha2", _i(n2), _i(n1), _i(n3), _i(nba), _a(U, "U", (n1, n3)),
         _a(AlphaCD4, "AlphaCD4", (nba, n1, n2)), _a(AlphaCD5, "AlphaCD5", (nba, n3, n2), True))


def calc_gocc(nvirt, noccEOS, NBA, Calpha3, goccEOS):
    """RIMP2_calc_gocc (RIMP2.F90:562-587)."""
    call("rimp2_calc_gocc", _i(nvirt), _i(noccEOS), _i(NBA),
         _a(Calpha3, "Calpha3", (NBA, nvirt, noccEOS)),
         _a(goccEOS, "goccEOS", (nvirt, noccEOS, nvirt, noccEOS), True))


def calc_gvirt(nvirtEOS, nocc, NBA, Calpha3, gvirtEOS):
    """RIMP2_calc_gvirt (RIMP2.F90:589-614)."""
    call("rimp2_calc_gvirt", _i(nvirtEOS), _i(nocc), _i(NBA),
         _a(Calpha3, "Calpha3", (NBA, nvirtEOS, nocc)),
         _a(gvirtEOS, "gvirtEOS", (nvirtEOS, nocc, nvirtEOS, nocc), True))


def calc_gen4DimFO(NBA, Calpha3, n1, n2, Calpha4, n3, n4, djik):
    """RIMP2_calc_gen4DimFO (RIMP2.F90:616-641)."""
    call("rimp2_calc_gen4dimfo", _i(NBA), _a(Calpha3, "Calpha3", (NBA, n1, n2)), _i(n1), _i(n2),
         _a(Calpha4, "Calpha4", (NBA, n3, n4)), _i(n3), _i(n4),
         _a(djik, "djik", (n1, n2, n3, n4), True))


def dgemm(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    """Column-major DGEMM as called at RIMP2.F90:79,87,110,118,137,160."""
    call("rimp2_dgemm", transa.encode(), transb.encode(), _i(m), _i(n), _i(k),
         C.byref(C.c_double(alpha)), _a(A, "A"), _i(lda), _a(B, "B"), _i(ldb),
         C.byref(C.c_double(beta)), _a(Cm, "C", writable=True), _i(ldc))


def steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Calpha, EVocc, EVvirt, UoccEOST, UvirtT, UoccT,
              UvirtEOST):
    """Driver Steps 5-8 (RIMP2.F90:71-170) on the GPU; returns
    (toccEOS, tvirtEOS, goccEOS, gvirtEOS)."""
    f = lambda *s: np.zeros(s, dtype=np.float64, order="F")  # noqa: E731
    toccEOS = f(nvirt, noccEOS, nvirt, noccEOS)
    tvirtEOS = f(nvirtEOS, nocc, nvirtEOS, nocc)
    goccEOS = f(nvirt, noccEOS, nvirt, noccEOS)
    gvirtEOS = f(nvirtEOS, nocc, nvirtEOS, nocc)
    call("rimp2_steps5to8", _i(nvirt), _i(nocc), _i(noccEOS), _i(nvirtEOS), _i(NBA),
         _a(Calpha, "Calpha", (NBA, nvirt, nocc)), _a(EVocc, "EVocc"), _a(EVvirt, "EVvirt"),
         _a(UoccEOST, "UoccEOST"), _a(UvirtT, "UvirtT"), _a(UoccT, "UoccT"),
         _a(UvirtEOST, "UvirtEOST"), _a(toccEOS, "toccEOS", writable=True),
         _a(tvirtEOS, "tvirtEOS", writable=True), _a(goccEOS, "goccEOS", writable=True),
         _a(gvirtEOS, "gvirtEOS", writable=True))
    return toccEOS, tvirtEOS, goccEOS, gvirtEOS


def first_order(nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA, Calpha, CalphaOcc, CalphaVV,
                UoccEOST, UvirtT, UoccT, UvirtEOST, UoccallT=None):
    """First-order property integrals of the driver (RIMP2.F90:172-251) on
    the GPU; returns (djik, blad).  UoccallT defaults to UoccT, as the driver
    passes it (RIMP2.F90:197)."""
    if UoccallT is None:
        UoccallT = UoccT
    f = lambda *s: np.zeros(s, dtype=np.float64, order="F")  # noqa: E731
    djik = f(nvirt, noccEOS, noccEOS, nocctot)
    blad = f(nvirtEOS, nocc, nvirtEOS, nvirt)
    call("rimp2_first_order", _i(nvirt), _i(nocc), _i(noccEOS), _i(nvirtEOS), _i(nocctot), _i(NBA),
         _a(Calpha, "Calpha", (NBA, nvirt, nocc)),
         _a(CalphaOcc, "CalphaOcc", (NBA, nocc, nocctot)),
         _a(CalphaVV, "CalphaVV", (NBA, nvirt, nvirt)), _a(UoccEOST, "UoccEOST", (nocc, noccEOS)),
         _a(UvirtT, "UvirtT", (nvirt, nvirt)), _a(UoccT, "UoccT", (nocc, nocc)),
         _a(UoccallT, "UoccallT", (nocctot, nocctot)), _a(UvirtEOST, "UvirtEOST", (nvirt, nvirtEOS)),
         _a(djik, "djik", writable=True), _a(blad, "blad", writable=True))
    return djik, blad


def energy_eos(nvirt, nocc, noccEOS, nvirtEOS, NBA, Calpha, EVocc, EVvirt, UoccEOST, UvirtT,
               UoccT, UvirtEOST, precision=PREC_FP64):
    """Fused DEC fragment energies (Eocc, Evirt) for general local orbitals
    from the inputs of Steps 5-8 (C-ABI rimp2_energy_eos); FP64 or split."""
    eo_ = C.c_double()
    ev_ = C.c_double()
    call("rimp2_energy_eos", _i(nvirt), _i(nocc), _i(noccEOS), _i(nvirtEOS), _i(NBA),
         _a(Calpha, "Calpha", (NBA, nvirt, nocc)), _a(EVocc, "EVocc", (nocc,)),
         _a(EVvirt, "EVvirt", (nvirt,)), _a(UoccEOST, "UoccEOST", (nocc, noccEOS)),
         _a(UvirtT, "UvirtT", (nvirt, nvirt)), _a(UoccT, "UoccT", (nocc, nocc)),
         _a(UvirtEOST, "UvirtEOST", (nvirt, nvirtEOS)), C.pointer(eo_), C.pointer(ev_),
         _i(precision))
    return eo_.value, ev_.value


DATAFILE_RECORDS = ("Calpha", "EVocc", "EVvirt", "UoccEOST", "UvirtT", "UoccT", "UvirtEOST",
                    "CalphaOcc", "CalphaVV", "toccEOS", "tvirtEOS", "gvirtEOS", "goccEOS",
                    "djik", "blad")
_FIRST_ORDER_ONLY = {"CalphaOcc", "CalphaVV", "djik", "blad"}


def _datafile_shapes(nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot):
    return dict(Calpha=(NBA, nvirt, nocc), EVocc=(nocc,), EVvirt=(nvirt,),
                UoccEOST=(nocc, noccEOS), UvirtT=(nvirt, nvirt), UoccT=(nocc, nocc),
                UvirtEOST=(nvirt, nvirtEOS), CalphaOcc=(NBA, nocc, nocctot),
                CalphaVV=(NBA, nvirt, nvirt), toccEOS=(nvirt, noccEOS, nvirt, noccEOS),
                tvirtEOS=(nvirtEOS, nocc, nvirtEOS, nocc),
                gvirtEOS=(nvirtEOS, nocc, nvirtEOS, nocc),
                goccEOS=(nvirt, noccEOS, nvirt, noccEOS), djik=(nvirt, noccEOS, noccEOS, nocctot),
                blad=(nvirtEOS, nocc, nvirtEOS, nvirt))


def read_datafile(path, first_order=False, known_answers=True):
    """Read a Calpha{1,2}.data file (C-ABI rimp2_datafile_read); returns a
    dict of the header dimensions and Fortran-ordered arrays.  With
    known_answers=False the test records (toccEOS on) are skipped."""
    h = (C.c_int * 6)()
    call("rimp2_datafile_header", str(path).encode(), h)
    dims = dict(zip(("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA", "nocctot"), list(h)))
    shapes = _datafile_shapes(**dims)
    out = dict(dims)
    ptrs = (C.c_void_p * len(DATAFILE_RECORDS))()
    for k, name in enumerate(DATAFILE_RECORDS):
        if name in _FIRST_ORDER_ONLY and not first_order:
            continue
        if k >= 9 and not known_answers:
            continue
        a = np.zeros(shapes[name], dtype=np.float64, order="F")
        out[name] = a
        ptrs[k] = a.ctypes.data
    call("rimp2_datafile_read", str(path).encode(), 1 if first_order else 0, ptrs)
    return out


def write_datafile(path, arrays, first_order=False):
    """Write a Calpha{1,2}.data file from a dict holding the header
    dimensions and the arrays (C-ABI rimp2_datafile_write)."""
    dims = [int(arrays[k]) for k in ("nvirt", "nocc", "noccEOS", "nvirtEOS", "NBA", "nocctot")]
    shapes = _datafile_shapes(*dims)
    ptrs = (C.c_void_p * len(DATAFILE_RECORDS))()
    keep = []
    for k, name in enumerate(DATAFILE_RECORDS):
        a = arrays.get(name)
        if a is None:
            continue
        a = np.asfortranarray(a, dtype=np.float64)
        if a.size != int(np.prod(shapes[name])):
            raise ValueError(f"{name} has {a.size} elements, expected {shapes[name]}")
        keep.append(a)
        ptrs[k] = a.ctypes.data
    call("rimp2_datafile_write", str(path).encode(), (C.c_int * 6)(*dims),
         1 if first_order else 0, ptrs)


def energy(nvirt, nocc, NBA, Calpha, EVocc, EVvirt, precision=PREC_FP64, amplitudes=False):
    """MP2 pair energies and total from host arrays (C-ABI rimp2_energy).
    Returns (Epair[nocc,nocc], Etot[, tamp(nvirt,nocc,nvirt,nocc)])."""
    Ep = np.zeros((nocc, nocc), dtype=np.float64, order="F")
    Et = np.zeros(1, dtype=np.float64)
    t = np.zeros((nvirt, nocc, nvirt, nocc), dtype=np.float64, order="F") if amplitudes else None
    call("rimp2_energy", _i(nvirt), _i(nocc), _i(NBA), _a(Calpha, "Calpha", (NBA, nvirt, nocc)),
         _a(EVocc, "EVocc", (nocc,)), _a(EVvirt, "EVvirt", (nvirt,)), _a(Ep, "Epair", writable=True),
         _a(Et, "Etot", writable=True), (_a(t, "tamp", writable=True) if t is not None else None),
         _i(precision))
    return (Ep, float(Et[0]), t) if amplitudes else (Ep, float(Et[0]))


def energy_dev(nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot, dtamp=0,
               precision=PREC_FP64, stream=0):
    """Device-pointer form (integers are raw device addresses, e.g.
    ``torch.Tensor.data_ptr()``); stream-ordered, no synchronisation."""
    call("rimp2_energy_dev", nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot, dtamp or None,
         precision, stream or None)


def energy_split_dev(nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot, nslices=1,
                     stream=0):
    """Split-precision energy with an explicit residual-slice count."""
    call("rimp2_energy_split_dev", nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot,
         nslices, stream or None)


def energy_batched(frags, precision=PREC_FP64):
    """frags: list of (Calpha, EVocc, EVvirt) numpy arrays of uneven sizes.
    Returns a list of (Epair, Etot).  The fragments are packed into one
    array first (a host copy); energy_batched_packed takes packed input."""
    nocc = [f[1].size for f in frags]
    nvirt = [f[2].size for f in frags]
    nba = [f[0].shape[0] for f in frags]
    ca = np.concatenate([np.asfortranarray(f[0]).ravel(order="F") for f in frags])
    eo = np.concatenate([f[1] for f in frags])
    ev = np.concatenate([f[2] for f in frags])
    return energy_batched_packed(nocc, nvirt, nba, ca, eo, ev, precision)


def energy_batched_packed(nocc, nvirt, nba, ca, eo, ev, precision=PREC_FP64):
    """Batched energies of fragments packed back to back in host memory:
    ``ca`` holds each fragment's Calpha(NBA, nvirt, nocc) (column-major) in
    turn, ``eo``/``ev`` their occupied/virtual orbital energies.  The library
    copies fragment by fragment, launch group by launch group, and each
    group's kernels wait only for its own copies: with ``ca`` in pinned
    memory (e.g. a ``torch.empty(..., pin_memory=True)`` tensor's numpy
    view) the transfer of later groups overlaps the kernels of earlier ones.
    Returns a list of (Epair, Etot)."""
    nocc = np.ascontiguousarray(nocc, dtype=np.int32)
    nvirt = np.ascontiguousarray(nvirt, dtype=np.int32)
    nba = np.ascontiguousarray(nba, dtype=np.int32)
    nf = len(nocc)
    if not (len(nvirt) == len(nba) == nf):
        raise ValueError("nocc, nvirt and nba must have one entry per fragment")
    sizes = nba.astype(np.int64) * nvirt * nocc
    off = lambda v: np.concatenate([[0], np.cumsum(v)[:-1]]).astype(np.int64)  # noqa: E731
    if ca.size != int(sizes.sum()) or eo.size != int(nocc.sum()) or ev.size != int(nvirt.sum()):
        raise ValueError("packed Calpha / orbital energies do not match the fragment sizes")
    ca_off, eo_off, ev_off = off(sizes), off(nocc), off(nvirt)
    ep_off = off(nocc.astype(np.int64) ** 2)
    Ep = np.zeros(int((nocc.astype(np.int64) ** 2).sum()), dtype=np.float64)
    Et = np.zeros(nf, dtype=np.float64)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    lp = lambda a: a.ctypes.data_as(C.POINTER(C.c_longlong))  # noqa: E731
    call("rimp2_energy_batched", _i(nf), ip(nocc), ip(nvirt), ip(nba), _a(ca, "Calpha"), lp(ca_off),
         _a(eo, "EVocc"), lp(eo_off), _a(ev, "EVvirt"), lp(ev_off), _a(Ep, "Epair", writable=True),
         lp(ep_off), _a(Et, "Etot", writable=True), _i(precision))
    out = []
    for f in range(nf):
        n = int(nocc[f])
        out.append((Ep[ep_off[f]:ep_off[f] + n * n].reshape((n, n), order="F"), float(Et[f])))
    return out


def gen_fragment_dev(seed, nocc, nvirt, NBA, dCalpha=0, dEVocc=0, dEVvirt=0, stream=0):
    """Generate a seeded synthetic fragment directly in device memory."""
    call("rimp2_gen_fragment_dev", seed, nocc, nvirt, NBA, dCalpha or None, dEVocc or None,
         dEVvirt or None, stream or None)


class BatchPlan:
    """Batched energies of many device-resident fragments: one persistent
    launch per group (paired-CTA kernel, one-CTA kernel with one or two
    residual slices, plain FP64) draining a device work queue, optionally
    captured once as a CUDA graph (C-ABI rimp2_batch_plan_*).  ``frags`` is
    a list of (nocc, nvirt, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot)
    with device addresses; ``nslices`` per fragment is 1 or 2 (split form)
    or 0 (plain FP64), None for the shape-bucket table; outputs are written
    at every ``execute``."""

    def __init__(self, frags, nslices=None, graph=True, stream=0):
        n = len(frags)
        ia = lambda k: (C.c_int * n)(*[int(f[k]) for f in frags])  # noqa: E731
        pa = lambda k: (C.c_void_p * n)(*[int(f[k]) for f in frags])  # noqa: E731
        self._keep = [ia(0), ia(1), ia(2), pa(3), pa(4), pa(5), pa(6), pa(7)]
        ns = (C.c_int * n)(*nslices) if nslices is not None else None
        self._keep.append(ns)
        self._plan = C.c_void_p()
        # C order: (plan, nfrag, nocc[], nvirt[], NBA[], Calpha[], EVocc[], EVvirt[], Epair[],
        # Etot[], nslices[], use_graph, stream)
        call("rimp2_batch_plan_create", C.byref(self._plan), n, self._keep[0], self._keep[1],
             self._keep[2], self._keep[3], self._keep[4], self._keep[5], self._keep[6],
             self._keep[7], ns, 1 if graph else 0, stream or None)

    def execute(self, stream=0):
        call("rimp2_batch_plan_execute", self._plan, stream or None)

    def close(self):
        if self._plan:
            call("rimp2_batch_plan_destroy", self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_split_buckets(nvirt_min, nslices):
    """Install a shape-bucket table for the split form's slice count."""
    n = len(nvirt_min)
    call("rimp2_set_split_buckets", n, (C.c_int * n)(*nvirt_min), (C.c_int * n)(*nslices))


def split_nslices(nvirt, nocc, NBA):
    return lib().rimp2_split_nslices(nvirt, nocc, NBA)


def set_split_kernel_rule(nvirt_min, min_nocc, min_nba):
    """Install the energy-kernel table of the one-residual-slice split form
    (paired-CTA kernel where nocc >= min_nocc and NBA >= min_nba)."""
    n = len(nvirt_min)
    call("rimp2_set_split_kernel_rule", n, (C.c_int * n)(*nvirt_min), (C.c_int * n)(*min_nocc),
         (C.c_int * n)(*min_nba))


def split_kernel_for(nvirt, nocc, NBA):
    """0 FP64 tier, 1 one-CTA kernel, 2 paired-CTA kernel for this shape."""
    return int(lib().rimp2_split_kernel_for(nvirt, nocc, NBA))


def calpha_from_ao(NBA, nbas, nocc, nvirt, ao, V, Cmo):
    """Calpha(NBA,nvirt,nocc) from AO three-centre integrals, metric and MO
    coefficients (FP64 Cholesky + triangular solve on the GPU)."""
    out = np.zeros((NBA, nvirt, nocc), dtype=np.float64, order="F")
    call("rimp2_calpha_from_ao", _i(NBA), _i(nbas), _i(nocc), _i(nvirt),
         _a(ao, "ao", (NBA, nbas, nbas)), _a(V, "V", (NBA, NBA)), _a(Cmo, "Cmo", (nbas, nbas)),
         _a(out, "Calpha", writable=True))
    return out


def calpha_from_ao_dev(NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha, stream=0):
    call("rimp2_calpha_from_ao_dev", NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha,
         stream or None)


def calpha_from_ao_split_dev(NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha, stream=0):
    """AO->MO transform on the tensor cores (split precision), FP64 Cholesky/solve."""
    call("rimp2_calpha_from_ao_split_dev", NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha,
         stream or None)


def ao2mo_dev(NBA, nbas, nocc, nvirt, dao, dCmo, dout, split=True, stream=0):
    """(alpha|a i) from (alpha|mu nu) and the MO coefficients, device pointers."""
    call("rimp2_ao2mo_dev", NBA, nbas, nocc, nvirt, dao, dCmo, dout, 1 if split else 0,
         stream or None)


def cholesky_dev(n, dV, stream=0):
    call("rimp2_cholesky_dev", n, dV, stream or None)


def trsm_lower_dev(n, m, dL, dB, dX, stream=0):
    call("rimp2_trsm_lower_dev", n, m, dL, dB, dX, stream or None)


def gen_ao_dev(seed, NBA, nbas, dao=0, dV=0, stream=0):
    call("rimp2_gen_ao_dev", seed, NBA, nbas, dao or None, dV or None, stream or None)


def get_dev_mem():
    """(total, free) device memory in bytes (replaces get_dev_mem, cuda_api.cu:5-8)."""
    t = C.c_size_t()
    f = C.c_size_t()
    call("rimp2_get_dev_mem", C.byref(t), C.byref(f))
    return t.value, f.value


def sync_status(stream=0):
    """Synchronise and raise if an earlier device-pointer call failed on the GPU."""
    call("rimp2_sync_status", stream or None)


def set_timing(on=True):
    call("rimp2_set_timing", 1 if on else 0)


def last_timing():
    """(slicing_ms, energy_kernel_ms, reduction_ms) of the last split call."""
    a = (C.c_float * 4)()
    call("rimp2_last_timing", a)
    return tuple(a[:3])


def last_split_kernel():
    """Energy kernel of the last split launch: 0 none, 1 one-CTA, 2 paired-CTA."""
    return int(lib().rimp2_last_split_kernel())


def probe_fp64_peak():
    """Measured FP64 DMMA throughput (TFLOP/s) of the current GPU."""
    v = C.c_double()
    call("rimp2_probe_fp64_peak", C.byref(v))
    return v.value


def kernel_launch_count():
    return lib().rimp2_kernel_launch_count()


def last_error():
    return lib().rimp2_last_error_string().decode(errors="replace")
