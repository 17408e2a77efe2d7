"""ctypes front end of the CPU oracle (``rimp2_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, always as the checker.  The
product library never imports this module.

Every routine mirrors one subroutine of the reference program RIMP2.F90
(januseriksen/rimp2_gpu) with the same argument list and the same
column-major (Fortran) array layout; numpy arrays passed here must be
``float64`` in Fortran order.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "rimp2_oracle.c")
_OUT = os.path.join(_HERE, "_build", "librimp2_oracle.so")
_lock = threading.Lock()
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, no FMA contraction, no fast-math)."""
    os.makedirs(os.path.dirname(_OUT), exist_ok=True)
    if not force and os.path.exists(_OUT) and os.path.getmtime(_OUT) >= os.path.getmtime(_SRC):
        return _OUT
    tmp = _OUT + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, _SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _OUT)
    return _OUT


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            L = C.CDLL(path)
            i, d, u64, u32 = C.c_int, C.c_double, C.c_uint64, C.c_uint32
            sig = {
                "orc_calc_toccA": [i, i, i, i, _dp, _dp, _dp, _dp, _dp],
                "orc_calc_tvirtA": [i, i, i, i, _dp, _dp, _dp, _dp, _dp],
                "orc_calc_toccB": [i, i, _dp, _dp, _dp],
                "orc_calc_tvirtB": [i, i, _dp, _dp, _dp],
                "orc_transalpha1": [i, i, i, _dp, _dp, _dp],
                "orc_transalpha2": [i, i, i, i, _dp, _dp, _dp],
                "orc_calc_gocc": [i, i, i, _dp, _dp],
                "orc_calc_gvirt": [i, i, i, _dp, _dp],
                "orc_gen4dimfo": [i, _dp, i, i, _dp, i, i, _dp],
                "orc_dgemm": [C.c_char, C.c_char, i, i, i, d, _dp, i, _dp, i, d, _dp, i],
                "orc_steps5to8": [i, i, i, i, i] + [_dp] * 11,
                "orc_first_order": [i] * 6 + [_dp] * 10,
                "orc_gen_kat_fo": [i] * 4 + [_dp] * 2,
                "orc_pair_energies": [i, i, i, _dp, _dp, _dp, _dp, _ip, i],
                "orc_pair_energies_blocked": [i, i, i, _dp, _dp, _dp, _dp, _ip, i],
                "orc_amplitudes": [i, i, i, _dp, _dp, _dp, _dp],
                "orc_philox4x32_10": [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)],
                "orc_uniform": [u64, u32, u64],
                "orc_normal": [u64, u32, u64],
                "orc_gen_calpha": [u64, i, i, i, _dp],
                "orc_gen_eps": [u64, i, i, _dp, _dp],
                "orc_gen_calpha_slabs": [u64, i, i, _ip, i, _dp],
                "orc_gen_matrix": [u64, u32, i, i, _dp],
                "orc_gen_kat": [i, i, i, i, i] + [_dp] * 7,
                "orc_write_datafile": [C.c_char_p] + [i] * 6 + [_dp] * 11,
                "orc_read_header": [C.c_char_p, C.POINTER(C.c_int32)],
                "orc_read_datafile": [C.c_char_p] + [_dp] * 11,
                "orc_gen_ao3c": [u64, i, i, _dp],
                "orc_gen_metric": [u64, i, _dp],
                "orc_gen_mo": [u64, i, _dp],
                "orc_ao2mo": [i, i, i, i, _dp, _dp, _dp],
                "orc_cholesky": [i, _dp],
                "orc_trsm_lower": [i, i, _dp, _dp],
                "orc_num_threads": [],
                "orc_set_num_threads": [i],
            }
            ret = {"orc_pair_energies": d, "orc_pair_energies_blocked": d, "orc_uniform": d,
                   "orc_normal": d, "orc_steps5to8": i, "orc_first_order": i, "orc_write_datafile": i,
                   "orc_read_header": i, "orc_read_datafile": i, "orc_cholesky": i,
                   "orc_num_threads": i}
            for name, args in sig.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = ret.get(name, None)
            _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim <= 1), "need float64 F-order"
    return a.ctypes.data_as(_dp)


def fzeros(*shape):
    return np.zeros(shape, dtype=np.float64, order="F")


# --- RIMP2.F90 subroutines ---------------------------------------------------

def calc_toccA(nvirt, nocc, noccEOS, NBA, Calpha, EVocc, EVvirt, tocc, UoccEOST):
    """RIMP2_calc_toccA (RIMP2.F90:381-417)."""
    lib().orc_calc_toccA(nvirt, nocc, noccEOS, NBA, _p(Calpha), _p(EVocc), _p(EVvirt), _p(tocc),
                         _p(UoccEOST))


def calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, Calpha, EVocc, EVvirt, tvirt, UvirtEOST):
    """RIMP2_calc_tvirtA (RIMP2.F90:419-453)."""
    lib().orc_calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, _p(Calpha), _p(EVocc), _p(EVvirt), _p(tvirt),
                          _p(UvirtEOST))


def calc_toccB(nvirt, noccEOS, tocc, UvirtT, toccEOS):
    """RIMP2_calc_toccB (RIMP2.F90:456-481)."""
    lib().orc_calc_toccB(nvirt, noccEOS, _p(tocc), _p(UvirtT), _p(toccEOS))


def calc_tvirtB(nvirtEOS, nocc, tvirt, UoccT, tvirtEOS):
    """RIMP2_calc_tvirtB (RIMP2.F90:483-508)."""
    lib().orc_calc_tvirtB(nvirtEOS, nocc, _p(tvirt), _p(UoccT), _p(tvirtEOS))


def transalpha1(nvirt, noccEOS, nba, UvirtT, AlphaCD4, AlphaCD5):
    """RIMP2_TransAlpha1 (RIMP2.F90:510-533)."""
    lib().orc_transalpha1(nvirt, noccEOS, nba, _p(UvirtT), _p(AlphaCD4), _p(AlphaCD5))


def transalpha2(n2, n1, n3, nba, U, AlphaCD4, AlphaCD5):
    """RIMP2_TransAlpha2 (RIMP2.F90:536-560)."""
    lib().orc_transalpha2(n2, n1, n3, nba, _p(U), _p(AlphaCD4), _p(AlphaCD5))


def calc_gocc(nvirt, noccEOS, NBA, Calpha3, goccEOS):
    """RIMP2_calc_gocc (RIMP2.F90:562-587)."""
    lib().orc_calc_gocc(nvirt, noccEOS, NBA, _p(Calpha3), _p(goccEOS))


def calc_gvirt(nvirtEOS, nocc, NBA, Calpha3, gvirtEOS):
    """RIMP2_calc_gvirt (RIMP2.F90:589-614)."""
    lib().orc_calc_gvirt(nvirtEOS, nocc, NBA, _p(Calpha3), _p(gvirtEOS))


def calc_gen4DimFO(NBA, Calpha3, n1, n2, Calpha4, n3, n4, djik):
    """RIMP2_calc_gen4DimFO (RIMP2.F90:616-641)."""
    lib().orc_gen4dimfo(NBA, _p(Calpha3), n1, n2, _p(Calpha4), n3, n4, _p(djik))


def dgemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, Cm, ldc):
    """Column-major dgemm as called at RIMP2.F90:79,87,110,118,137,160."""
    lib().orc_dgemm(ta.encode(), tb.encode(), M, N, K, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm),
                    ldc)


def steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, Calpha, EVocc, EVvirt, UoccEOST, UvirtT, UoccT,
              UvirtEOST):
    """Driver Steps 5-8 (RIMP2.F90:71-170); returns (toccEOS, tvirtEOS, goccEOS, gvirtEOS)."""
    toccEOS = fzeros(nvirt, noccEOS, nvirt, noccEOS)
    tvirtEOS = fzeros(nvirtEOS, nocc, nvirtEOS, nocc)
    goccEOS = fzeros(nvirt, noccEOS, nvirt, noccEOS)
    gvirtEOS = fzeros(nvirtEOS, nocc, nvirtEOS, nocc)
    rc = lib().orc_steps5to8(nvirt, nocc, noccEOS, nvirtEOS, NBA, _p(Calpha), _p(EVocc), _p(EVvirt),
                             _p(UoccEOST), _p(UvirtT), _p(UoccT), _p(UvirtEOST), _p(toccEOS),
                             _p(tvirtEOS), _p(goccEOS), _p(gvirtEOS))
    if rc:
        raise MemoryError("oracle steps5to8 allocation failed")
    return toccEOS, tvirtEOS, goccEOS, gvirtEOS


# --- energies ----------------------------------------------------------------

def first_order(nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA, Calpha, CalphaOcc, CalphaVV,
                UoccEOST, UvirtT, UoccT, UvirtEOST, UoccallT=None):
    """First-order block of the driver (RIMP2.F90:172-251): (djik, blad)."""
    if UoccallT is None:
        UoccallT = UoccT
    djik = fzeros(nvirt, noccEOS, noccEOS, nocctot)
    blad = fzeros(nvirtEOS, nocc, nvirtEOS, nvirt)
    rc = lib().orc_first_order(nvirt, nocc, noccEOS, nvirtEOS, nocctot, NBA, _p(Calpha),
                               _p(CalphaOcc), _p(CalphaVV), _p(UoccEOST), _p(UvirtT), _p(UoccT),
                               _p(UoccallT), _p(UvirtEOST), _p(djik), _p(blad))
    if rc:
        raise MemoryError("oracle first_order allocation failed")
    return djik, blad


def energy_eos_from_arrays(toccEOS, goccEOS, tvirtEOS, gvirtEOS):
    """Fragment energies from the reference's Step 5-8 arrays (restated MP2
    expression in the local basis; the reference computes no energy):
    Eocc = sum toccEOS(aL,iL,bL,jL) (2 goccEOS(aL,iL,bL,jL) - goccEOS(bL,iL,aL,jL)),
    Evirt = sum tvirtEOS(aL,iL,bL,jL) (2 gvirtEOS(aL,iL,bL,jL) - gvirtEOS(aL,jL,bL,iL)).
    Compensated (fsum) over all elements."""
    import math
    xo = toccEOS * (2.0 * goccEOS - np.transpose(goccEOS, (2, 1, 0, 3)))
    xv = tvirtEOS * (2.0 * gvirtEOS - np.transpose(gvirtEOS, (0, 3, 2, 1)))
    return math.fsum(xo.ravel()), math.fsum(xv.ravel())


def _pairs_arg(pairs):
    if pairs is None:
        return None, 0, None
    arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    return arr.ctypes.data_as(_ip), arr.shape[0], arr


def pair_energies(nvirt, nocc, NBA, Calpha, EVocc, EVvirt, pairs=None, blocked=False):
    """MP2 pair energies e_ij (nocc x nocc, symmetric) and the total
    E = sum_ij e_ij, FP64 with compensated sums.  ``pairs`` restricts the work
    to a list of (i, j) pairs (other entries of Epair stay NaN)."""
    Ep = np.full((nocc, nocc), np.nan, dtype=np.float64, order="F")
    pp, n, keep = _pairs_arg(pairs)
    f = lib().orc_pair_energies_blocked if blocked else lib().orc_pair_energies
    tot = f(nvirt, nocc, NBA, _p(Calpha), _p(EVocc), _p(EVvirt), _p(Ep), pp, n)
    del keep
    return Ep, tot


def amplitudes(nvirt, nocc, NBA, Calpha, EVocc, EVvirt):
    """Canonical amplitudes t(a,i,b,j) = g_ij(a,b) / D."""
    t = fzeros(nvirt, nocc, nvirt, nocc)
    lib().orc_amplitudes(nvirt, nocc, NBA, _p(Calpha), _p(EVocc), _p(EVvirt), _p(t))
    return t


# --- generators --------------------------------------------------------------

def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def gen_calpha(seed, NBA, nvirt, nocc):
    a = fzeros(NBA, nvirt, nocc)
    lib().orc_gen_calpha(seed, NBA, nvirt, nocc, _p(a))
    return a


def gen_calpha_slabs(seed, NBA, nvirt, occ):
    """Calpha(:,:,occ) of a fragment, generated for a subset of occupied indices."""
    occ = np.ascontiguousarray(np.asarray(occ, dtype=np.int32))
    out = fzeros(NBA, nvirt, occ.size)
    lib().orc_gen_calpha_slabs(seed, NBA, nvirt, occ.ctypes.data_as(_ip), occ.size, _p(out))
    return out


def gen_eps(seed, nocc, nvirt):
    eo = np.zeros(nocc)
    ev = np.zeros(nvirt)
    lib().orc_gen_eps(seed, nocc, nvirt, _p(eo), _p(ev))
    return eo, ev


def gen_matrix(seed, stream, n1, n2):
    U = fzeros(n1, n2)
    lib().orc_gen_matrix(seed, stream, n1, n2, _p(U))
    return U


def gen_fragment(seed, nocc, nvirt, NBA):
    """Calpha, EVocc, EVvirt of one synthetic fragment."""
    Ca = gen_calpha(seed, NBA, nvirt, nocc)
    eo, ev = gen_eps(seed, nocc, nvirt)
    return Ca, eo, ev


def gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS):
    """Constant-valued fixtures of generate.F90:77-128."""
    Ca = fzeros(NBA, nvirt, nocc)
    eo = np.zeros(nocc)
    ev = np.zeros(nvirt)
    UoE = fzeros(nocc, noccEOS)
    UvT = fzeros(nvirt, nvirt)
    UoT = fzeros(nocc, nocc)
    UvE = fzeros(nvirt, nvirtEOS)
    lib().orc_gen_kat(NBA, nvirt, nocc, noccEOS, nvirtEOS, _p(Ca), _p(eo), _p(ev), _p(UoE), _p(UvT),
                      _p(UoT), _p(UvE))
    return Ca, eo, ev, UoE, UvT, UoT, UvE


def gen_kat_fo(NBA, nvirt, nocc, nocctot):
    """First-order fixture inputs of generate.F90:254-260,300-306."""
    occ = fzeros(NBA, nocc, nocctot)
    vv = fzeros(NBA, nvirt, nvirt)
    lib().orc_gen_kat_fo(NBA, nvirt, nocc, nocctot, _p(occ), _p(vv))
    return occ, vv


def write_datafile(path, nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot, Calpha, EVocc, EVvirt,
                   UoccEOST, UvirtT, UoccT, UvirtEOST, toccEOS, tvirtEOS, gvirtEOS, goccEOS):
    rc = lib().orc_write_datafile(path.encode(), nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot,
                                  _p(Calpha), _p(EVocc), _p(EVvirt), _p(UoccEOST), _p(UvirtT),
                                  _p(UoccT), _p(UvirtEOST), _p(toccEOS), _p(tvirtEOS),
                                  _p(gvirtEOS), _p(goccEOS))
    if rc:
        raise OSError(f"write_datafile({path}) failed")


def read_datafile(path):
    h = (C.c_int32 * 6)()
    if lib().orc_read_header(path.encode(), h):
        raise OSError(f"bad header in {path}")
    nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot = list(h)
    arrs = dict(Calpha=fzeros(NBA, nvirt, nocc), EVocc=np.zeros(nocc), EVvirt=np.zeros(nvirt),
                UoccEOST=fzeros(nocc, noccEOS), UvirtT=fzeros(nvirt, nvirt),
                UoccT=fzeros(nocc, nocc), UvirtEOST=fzeros(nvirt, nvirtEOS),
                toccEOS=fzeros(nvirt, noccEOS, nvirt, noccEOS),
                tvirtEOS=fzeros(nvirtEOS, nocc, nvirtEOS, nocc),
                gvirtEOS=fzeros(nvirtEOS, nocc, nvirtEOS, nocc),
                goccEOS=fzeros(nvirt, noccEOS, nvirt, noccEOS))
    rc = lib().orc_read_datafile(path.encode(), *[_p(v) for v in arrs.values()])
    if rc:
        raise OSError(f"read_datafile({path}) failed rc={rc}")
    arrs.update(nvirt=nvirt, nocc=nocc, noccEOS=noccEOS, nvirtEOS=nvirtEOS, NBA=NBA,
                nocctot=nocctot)
    return arrs


# --- AO front end --------------------------------------------------------------

def gen_ao3c(seed, NBA, nbas):
    a = fzeros(NBA, nbas, nbas)
    lib().orc_gen_ao3c(seed, NBA, nbas, _p(a))
    return a


def gen_metric(seed, NBA):
    V = fzeros(NBA, NBA)
    lib().orc_gen_metric(seed, NBA, _p(V))
    return V


def gen_mo(seed, nbas):
    Cm = fzeros(nbas, nbas)
    lib().orc_gen_mo(seed, nbas, _p(Cm))
    return Cm


def ao2mo(NBA, nbas, nocc, nvirt, ao, Cmo):
    out = fzeros(NBA, nvirt, nocc)
    lib().orc_ao2mo(NBA, nbas, nocc, nvirt, _p(ao), _p(Cmo), _p(out))
    return out


def cholesky(V):
    L = np.array(V, dtype=np.float64, order="F", copy=True)
    rc = lib().orc_cholesky(L.shape[0], _p(L))
    if rc:
        raise np.linalg.LinAlgError(f"metric not positive definite at pivot {rc - 1}")
    return np.tril(L)


def trsm_lower(L, B):
    X = np.array(B, dtype=np.float64, order="F", copy=True)
    n = L.shape[0]
    lib().orc_trsm_lower(n, X.size // n, _p(np.asfortranarray(L)), _p(X))
    return X


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(n):
    lib().orc_set_num_threads(n)
