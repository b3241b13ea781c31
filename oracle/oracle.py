"""ctypes binding of the CPU restatement (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker.  It builds
``oracle/liboracle.so`` from ``bertha_oracle.cpp`` on first use.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = os.path.join(_HERE, "bertha_oracle.cpp")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        d, i, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        L.orc_boys.argtypes = [d, i, P]
        L.orc_rints.argtypes = [P, d, i, P]
        L.orc_cart_index.argtypes = [i, i, i]
        L.orc_eq_pair.argtypes = [i, i, d, P, i, i, d, P, i, P]
        L.orc_fock_layout.argtypes = [i, P, P, P, P, i, i, i, P, P]
        L.orc_clmfast.argtypes = [i, P, P, P, P, i, i, i, i, i, i, P, i, P, P, i]
        L.orc_eri_quartet.argtypes = [P, P, P, i, i, P]
        L.orc_eq_pair_q.argtypes = [i, i, d, P, i, i, d, P, i, i, i, P]
        L.orc_breit_kernel.argtypes = [P, d, i, i, i, i, P]
        L.orc_bii_quartet.argtypes = [P, P, P, i, i, i, P]
        L.orc_brtfast.argtypes = [i, P, P, P, P, i, i, i, i, i, i, P, i, P, i]
        L.orc_oneel.argtypes = [i, P, P, P, P, i, i, i, P, P, P, P, P, i]
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ntuv(L):
    return (L + 1) * (L + 2) * (L + 3) // 6


def boys(T, lam):
    F = np.zeros(lam + 1)
    lib().orc_boys(float(T), int(lam), _p(F))
    return F


def rints(qp, alpha, lam):
    R = np.zeros(ntuv(lam))
    q = np.ascontiguousarray(qp, dtype=np.float64)
    lib().orc_rints(_p(q), float(alpha), int(lam), _p(R))
    return R


def cart_index(t, u, v):
    return lib().orc_cart_index(t, u, v)


def eq_pair(ka, mqa, ea, A, kb, mqb, eb, B, small):
    """E-coefficients of one primitive spinor pair; mqa, mqb are signed 2m."""
    la = -ka - 1 if ka < 0 else ka
    lb = -kb - 1 if kb < 0 else kb
    out = np.zeros(2 * ntuv(la + lb + 2 + 2))
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    n = lib().orc_eq_pair(ka, mqa, ea, _p(A), kb, mqb, eb, _p(B), int(small), _p(out))
    return out[: 2 * n].view(np.complex128).copy()


def eq_pair_q(ka, mqa, ea, A, kb, mqb, eb, B, sa, sb, iq):
    """psi_a^+ sigma_iq psi_b E-coefficients (iq 0 unit, 1..3 x, y, z) for
    components sa, sb (0 large, 1 small); LS carries i, SL carries -i."""
    la = -ka - 1 if ka < 0 else ka
    lb = -kb - 1 if kb < 0 else kb
    out = np.zeros(2 * ntuv(la + lb + 2 + 2))
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    n = lib().orc_eq_pair_q(ka, mqa, ea, _p(A), kb, mqb, eb, _p(B), int(sa), int(sb),
                            int(iq), _p(out))
    return out[: 2 * n].view(np.complex128).copy()


def breit_kernel(qp, alpha, t, u, v, gaunt=False):
    """3x3 Breit kernel W_ij at Hermite index (t,u,v), PRE = 1."""
    q = np.ascontiguousarray(qp, dtype=np.float64)
    out = np.zeros(9)
    lib().orc_breit_kernel(_p(q), float(alpha), int(t), int(u), int(v), int(gaunt), _p(out))
    return out.reshape(3, 3)


def bii_quartet(xyz4, l4, ex4, t1, t2, gaunt=False):
    """Breit integrals of one primitive quartet (t = 0 LS, 1 SL), shaped as
    eri_quartet's result."""
    xyz4 = np.ascontiguousarray(xyz4, dtype=np.float64)
    l4 = np.ascontiguousarray(l4, dtype=np.int32)
    ex4 = np.ascontiguousarray(ex4, dtype=np.float64)
    nl = [2 * l + 1 for l in l4]
    out = np.zeros(2 * 16 * int(np.prod(nl)))
    n = lib().orc_bii_quartet(_p(xyz4), _p(l4), _p(ex4), int(t1), int(t2), int(gaunt),
                              _p(out))
    assert n == 16 * int(np.prod(nl))
    return out.view(np.complex128).reshape(nl + [16])


def eri_quartet(xyz4, l4, ex4, t1, t2):
    """All spinor integrals of one primitive quartet.

    Returns an array [lab_a, lab_b, lab_c, lab_d, 16] (complex), labels in the
    order kappa=l (|m| ascending) then kappa=-l-1 (|m| ascending); the last
    index is 8*sa+4*sb+2*sc+sd with s=1 for m>0.
    """
    xyz4 = np.ascontiguousarray(xyz4, dtype=np.float64)
    l4 = np.ascontiguousarray(l4, dtype=np.int32)
    ex4 = np.ascontiguousarray(ex4, dtype=np.float64)
    nl = [2 * l + 1 for l in l4]
    out = np.zeros(2 * 16 * int(np.prod(nl)))
    n = lib().orc_eri_quartet(_p(xyz4), _p(l4), _p(ex4), int(t1), int(t2), _p(out))
    assert n == 16 * int(np.prod(nl))
    return out.view(np.complex128).reshape(nl + [16])


def _basis_arrays(basis):
    xyz = np.ascontiguousarray(basis.xyz, dtype=np.float64)
    lmax = np.ascontiguousarray(basis.lmax, dtype=np.int32)
    nfn = np.ascontiguousarray(basis.nfn, dtype=np.int32)
    ex = np.ascontiguousarray(basis.ex, dtype=np.float64)
    return xyz, lmax, nfn, ex


def fock_layout(basis):
    xyz, lmax, nfn, ex = _basis_arrays(basis)
    maxl1, maxbs = ex.shape[1], ex.shape[2]
    nk = 2 * (maxl1 - 1) + 2
    lrge = np.full((basis.ncnt, nk, 28), -1, dtype=np.int32)
    nskp = ctypes.c_int(0)
    ndim = lib().orc_fock_layout(basis.ncnt, _p(xyz), _p(lmax), _p(nfn), _p(ex),
                                 maxl1, maxbs, int(basis.hmlt == 0), _p(lrge),
                                 ctypes.byref(nskp))
    return ndim, nskp.value, lrge


def clmfast(basis, dent, ilev, racah1=True):
    """Multi-centre Coulomb Fock build (INTSYM off): returns (GDIR, GXCH)."""
    xyz, lmax, nfn, ex = _basis_arrays(basis)
    maxl1, maxbs = ex.shape[1], ex.shape[2]
    nd = dent.shape[0]
    D = np.asfortranarray(dent, dtype=np.complex128)
    gd = np.zeros((nd, nd), dtype=np.complex128, order="F")
    gx = np.zeros((nd, nd), dtype=np.complex128, order="F")
    lib().orc_clmfast(basis.ncnt, _p(xyz), _p(lmax), _p(nfn), _p(ex), maxl1, maxbs,
                      int(basis.hmlt), int(basis.isym), int(ilev), int(racah1),
                      _p(D), nd, _p(gd), _p(gx), nd)
    return gd, gx


def brtfast(basis, dent, ilev, racah1=True, gaunt=False):
    """Closed-shell multi-centre Breit exchange matrix BXCH."""
    xyz, lmax, nfn, ex = _basis_arrays(basis)
    maxl1, maxbs = ex.shape[1], ex.shape[2]
    nd = dent.shape[0]
    D = np.asfortranarray(dent, dtype=np.complex128)
    bx = np.zeros((nd, nd), dtype=np.complex128, order="F")
    lib().orc_brtfast(basis.ncnt, _p(xyz), _p(lmax), _p(nfn), _p(ex), maxl1, maxbs,
                      int(basis.isym), int(ilev), int(racah1), int(gaunt), _p(D), nd,
                      _p(bx), nd)
    return bx


def oneel(basis, znuc, xi):
    """One-electron matrices (OVLP, HNUC, HKIN) of ONEEL; xi[c] is the
    Gaussian nuclear exponent of centre c (0 for a point nucleus)."""
    xyz, lmax, nfn, ex = _basis_arrays(basis)
    maxl1, maxbs = ex.shape[1], ex.shape[2]
    nd = basis.ndim
    z = np.ascontiguousarray(znuc, dtype=np.float64)
    x = np.ascontiguousarray(xi, dtype=np.float64)
    out = [np.zeros((nd, nd), dtype=np.complex128, order="F") for _ in range(3)]
    lib().orc_oneel(basis.ncnt, _p(xyz), _p(lmax), _p(nfn), _p(ex), maxl1, maxbs,
                    int(basis.hmlt), _p(z), _p(x), _p(out[0]), _p(out[1]), _p(out[2]), nd)
    return tuple(out)


class QuartetOracle:
    """Oracle digestion of explicit shell-quartet lists (batch types 1, 5)."""

    def __init__(self, basis):
        L = lib()
        P, i, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        L.orc_ctx_new.argtypes = [i, P, P, P, P, i, i, i]
        L.orc_ctx_new.restype = P
        L.orc_ctx_free.argtypes = [P]
        L.orc_ctx_prepare.argtypes = [P, P, ll, i, i]
        L.orc_ctx_quartets.argtypes = [P, P, ll, i, i, P, i, P, P, i, i]
        L.orc_ndim.argtypes = [P, P]
        xyz, lmax, nfn, ex = _basis_arrays(basis)
        self._keep = (xyz, lmax, nfn, ex)
        self.h = L.orc_ctx_new(basis.ncnt, _p(xyz), _p(lmax), _p(nfn), _p(ex),
                               ex.shape[1], ex.shape[2], int(basis.hmlt))
        ns = ctypes.c_int()
        self.ndim = L.orc_ndim(self.h, ctypes.byref(ns))
        self.nskp = ns.value

    def prepare(self, quart, t1, t2):
        q = np.ascontiguousarray(quart, dtype=np.int32)
        return lib().orc_ctx_prepare(self.h, _p(q), q.shape[0], int(t1), int(t2))

    def digest(self, quart, t1, t2, dent, gd, gx, nthreads=1):
        q = np.ascontiguousarray(quart, dtype=np.int32)
        assert gd.flags.f_contiguous and gx.flags.f_contiguous
        D = np.asfortranarray(dent, dtype=np.complex128)
        lib().orc_ctx_quartets(self.h, _p(q), q.shape[0], int(t1), int(t2), _p(D),
                               D.shape[0], _p(gd), _p(gx), gd.shape[0], int(nthreads))

    def close(self):
        if self.h:
            lib().orc_ctx_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
