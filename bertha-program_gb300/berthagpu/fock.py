"""Host mirror of the reference's Fock-build interface for this path.

``FockBuilder`` plays the part of EQSAVE + CLMFAST + BRTFAST
(bertha-scf.f:5287, 5401, 5441): construction uploads the basis and
generates the E-coefficients on the GPU; ``clmfast(dent, ilev)`` returns
(GDIR, GXCH) and ``brtfast(dent, ilev)`` returns BXCH, overwritten as the
reference does.  Errors raise BerthaGPUError (the reference STOPs).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import BerthaGPUError, check, check_batch, lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class FockBuilder:
    def __init__(self, basis, racah1=True, gaunt=False):
        self.basis = basis
        self._ctx = ctypes.c_void_p()
        xyz = np.ascontiguousarray(basis.xyz, dtype=np.float64)
        nkap = np.ascontiguousarray(basis.nkap, dtype=np.int32)
        nfn = np.ascontiguousarray(basis.nfn, dtype=np.int32)
        ex = np.ascontiguousarray(basis.ex, dtype=np.float64)
        mel, mbs = nfn.shape[1] - 1, ex.shape[2]
        flags = (0 if racah1 else _lib.FLAG_NO_RACAH1) | (_lib.FLAG_GAUNT if gaunt else 0)
        rc = lib().bertha_gpu_init(ctypes.byref(self._ctx), basis.ncnt, _p(xyz), _p(nkap),
                                   _p(nfn), mel, _p(ex), mbs, int(basis.hmlt),
                                   int(basis.isym), flags)
        if rc != 0:
            msg = lib().bertha_gpu_last_error(None)
            raise BerthaGPUError(rc, msg.decode() if msg else "")
        nd, ns = ctypes.c_int(), ctypes.c_int()
        check(lib().bertha_gpu_dims(self._ctx, ctypes.byref(nd), ctypes.byref(ns)), self._ctx)
        self.ndim, self.nskp = nd.value, ns.value
        self.precision = "fp64"

    def set_precision(self, prec):
        """'fp64' (drop-in), 'df32' (split precision on the FP32 pipes),
        'tc32' (3xTF32 contractions on the tensor cores) or 'auto' (per
        angular class the fastest kernel within the error budget, chosen on
        the first build)."""
        check(lib().bertha_gpu_set_precision(self._ctx, _lib.PREC[prec]), self._ctx)
        self.precision = prec

    def set_error_budget(self, eh):
        """Energy error (Eh) the 'auto' tuner may spend on tensor-core
        classes per Coulomb build."""
        check(lib().bertha_gpu_set_error_budget(self._ctx, float(eh)), self._ctx)

    def set_screening(self, threshold):
        """Schwarz threshold on Q_ab*Q_cd (0 = off, the reference default)."""
        check(lib().bertha_gpu_set_screening(self._ctx, float(threshold)), self._ctx)

    def set_list_limits(self, cache_quartets=0, chunk_quartets=0):
        """Quartet-list memory: cached up to cache_quartets, streamed in chunks
        of chunk_quartets above (0: library defaults)."""
        check(lib().bertha_gpu_set_list_limits(self._ctx, int(cache_quartets),
                                               int(chunk_quartets)), self._ctx)

    def close(self):
        if self._ctx:
            lib().bertha_gpu_free(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def shells(self):
        n = len(self.basis.shells())
        cnt = np.zeros(n, np.int32); l = np.zeros(n, np.int32); ib = np.zeros(n, np.int32)
        ns = ctypes.c_int()
        check(lib().bertha_gpu_shells(self._ctx, ctypes.byref(ns), _p(cnt), _p(l), _p(ib)), self._ctx)
        return cnt[: ns.value], l[: ns.value], ib[: ns.value]

    def layout(self):
        lrge = np.full(self.basis.ncnt * (2 * _lib.MAX_L + 2) * 28, -1, dtype=np.int32)
        check(lib().bertha_gpu_layout(self._ctx, _p(lrge)), self._ctx)
        return lrge.reshape(self.basis.ncnt, 2 * _lib.MAX_L + 2, 28)

    def clmfast(self, dent, ilev):
        """CALL CLMFAST on host arrays: returns (GDIR, GXCH)."""
        n = self.ndim
        D = np.asfortranarray(dent, dtype=np.complex128)
        if D.shape != (n, n):
            raise BerthaGPUError(_lib.BG_ERR_ARG, f"density shape {D.shape} != ({n},{n})")
        gd = np.zeros((n, n), dtype=np.complex128, order="F")
        gx = np.zeros((n, n), dtype=np.complex128, order="F")
        check(lib().bertha_gpu_clmfast(self._ctx, _p(D), n, int(ilev), _p(gd), _p(gx), n),
              self._ctx)
        return gd, gx

    def brtfast(self, dent, ilev):
        """CALL BRTFAST on host arrays: returns BXCH (closed shell)."""
        n = self.ndim
        D = np.asfortranarray(dent, dtype=np.complex128)
        if D.shape != (n, n):
            raise BerthaGPUError(_lib.BG_ERR_ARG, f"density shape {D.shape} != ({n},{n})")
        bx = np.zeros((n, n), dtype=np.complex128, order="F")
        check(lib().bertha_gpu_brtfast(self._ctx, _p(D), n, int(ilev), _p(bx), n), self._ctx)
        return bx

    def brtfast_device(self, d_dent, d_bxch, ilev, ld, stream=0):
        check(lib().bertha_gpu_brtfast_device(self._ctx, ctypes.c_void_p(d_dent), ld, int(ilev),
                                              ctypes.c_void_p(d_bxch), ld,
                                              ctypes.c_void_p(stream)), self._ctx)

    def oneel(self, znuc, xi):
        """CALL OVRLP + ONEEL: returns (OVLP, HNUC, HKIN)."""
        n = self.ndim
        z = np.ascontiguousarray(znuc, dtype=np.float64)
        x = np.ascontiguousarray(xi, dtype=np.float64)
        if z.shape != (self.basis.ncnt,) or x.shape != (self.basis.ncnt,):
            raise BerthaGPUError(_lib.BG_ERR_ARG, "znuc and xi need one value per centre")
        out = [np.zeros((n, n), dtype=np.complex128, order="F") for _ in range(3)]
        check(lib().bertha_gpu_oneel(self._ctx, _p(z), _p(x), _p(out[0]), _p(out[1]),
                                     _p(out[2]), n), self._ctx)
        return tuple(out)

    def oneel_device(self, znuc, xi, d_ovlp, d_hnuc, d_hkin, ld, stream=0):
        z = np.ascontiguousarray(znuc, dtype=np.float64)
        x = np.ascontiguousarray(xi, dtype=np.float64)
        check(lib().bertha_gpu_oneel_device(self._ctx, _p(z), _p(x), ctypes.c_void_p(d_ovlp),
                                            ctypes.c_void_p(d_hnuc), ctypes.c_void_p(d_hkin),
                                            ld, ctypes.c_void_p(stream)), self._ctx)

    def clmfast_device(self, d_dent, d_gdir, d_gxch, ilev, ld, stream=0):
        """Device-resident build: pointers are integers (e.g. tensor.data_ptr())."""
        check(lib().bertha_gpu_clmfast_device(self._ctx, ctypes.c_void_p(d_dent), ld, int(ilev),
                                              ctypes.c_void_p(d_gdir), ctypes.c_void_p(d_gxch),
                                              ld, ctypes.c_void_p(stream)), self._ctx)

    def quartets(self, d_quart, nq, t1, t2, d_dent, d_gdir, d_gxch, ld, stream=0):
        check(lib().bertha_gpu_quartets(self._ctx, ctypes.c_void_p(d_quart), int(nq), int(t1),
                                        int(t2), ctypes.c_void_p(d_dent), ld,
                                        ctypes.c_void_p(d_gdir), ctypes.c_void_p(d_gxch), ld,
                                        ctypes.c_void_p(stream)), self._ctx)

    def quartets_segments(self, d_quart, seg, lclass, t1, t2, d_dent, d_gdir, d_gxch, ld,
                          stream=0):
        """Explicit list grouped by angular class: seg (nseg+1 offsets) and
        lclass (nseg x 4 angular momenta) are host arrays."""
        sg = np.ascontiguousarray(seg, dtype=np.int64)
        lc = np.ascontiguousarray(lclass, dtype=np.int32)
        check(lib().bertha_gpu_quartets_segments(
            self._ctx, ctypes.c_void_p(d_quart), len(sg) - 1, _p(sg), _p(lc), int(t1), int(t2),
            ctypes.c_void_p(d_dent), ld, ctypes.c_void_p(d_gdir), ctypes.c_void_p(d_gxch), ld,
            ctypes.c_void_p(stream)), self._ctx)

    def tuning_record(self, breit=False):
        """The autotuner's last record, one dict per segment (class and
        bound decade): comp, class (l_a, l_b, l_c, l_d), quartets, kernel
        chosen, sample ms and estimated energy error per kernel."""
        n = ctypes.c_int()
        check(lib().bertha_gpu_tuning_record(self._ctx, int(breit), 0, None, None,
                                             ctypes.byref(n)), self._ctx)
        info = np.zeros(4 * max(n.value, 1), np.int32)
        vals = np.zeros(6 * max(n.value, 1), np.float64)
        check(lib().bertha_gpu_tuning_record(self._ctx, int(breit), n.value, _p(info), _p(vals),
                                             ctypes.byref(n)), self._ctx)
        rows = []
        for i in range(n.value):
            k = int(info[4 * i + 1])
            rows.append({"comp": int(info[4 * i]),
                         "class": ((k >> 6) & 3, (k >> 4) & 3, (k >> 2) & 3, k & 3),
                         "quartets": int(info[4 * i + 2]), "kind": int(info[4 * i + 3]),
                         "ms": [float(x) for x in vals[6 * i:6 * i + 3]],
                         "err": [float(x) for x in vals[6 * i + 3:6 * i + 6]]})
        return rows

    def breit_stats(self):
        """Kernel use of the last Breit build: FP64 and tensor-core quartets, runs."""
        nq = (ctypes.c_longlong * 3)()
        r = ctypes.c_int()
        check(lib().bertha_gpu_breit_kernel_stats(self._ctx, nq, ctypes.byref(r)), self._ctx)
        return {"fp64_quartets": nq[0], "tc32_quartets": nq[2], "runs": r.value}

    def launches(self):
        return int(lib().bertha_gpu_launches(self._ctx))

    def auto_stats(self):
        """Under precision 'auto' (or 'tc32'): quartets on the FP64, split and
        tensor-core kernels, runs (launches per build)."""
        nq = (ctypes.c_longlong * 3)()
        r = ctypes.c_int()
        check(lib().bertha_gpu_kernel_stats(self._ctx, nq, ctypes.byref(r)), self._ctx)
        return {"fp64_quartets": nq[0], "df32_quartets": nq[1], "tc32_quartets": nq[2],
                "runs": r.value}


class FockBatch:
    """Batched CLMFAST over independent instances (one FockBuilder each, all
    with the same Hamiltonian, shape and RACAH1 flag): one kernel launch per
    component class for every instance.  ``moff``/``ld`` place instance k's
    matrices at complex element moff[k] + i + ld[k]*j of the device arrays;
    the default packs them one after another with ld = NDIM.  The builders
    may be closed once the batch exists."""

    def __init__(self, builders, moff=None, ld=None):
        n = len(builders)
        arr = (ctypes.c_void_p * n)(*[b.ctx.value for b in builders])
        self.ndim = [b.ndim for b in builders]
        if moff is None:
            moff = np.concatenate([[0], np.cumsum([d * d for d in self.ndim])[:-1]])
        if ld is None:
            ld = self.ndim
        self.moff = np.ascontiguousarray(moff, dtype=np.int64)
        self.ld = np.ascontiguousarray(ld, dtype=np.int32)
        self._b = ctypes.c_void_p()
        rc = lib().bertha_gpu_batch_create(ctypes.byref(self._b), n, arr, _p(self.moff),
                                           _p(self.ld))
        check_batch(rc, None)
        self.n = n

    def set_precision(self, prec):
        check_batch(lib().bertha_gpu_batch_set_precision(self._b, _lib.PREC[prec]), self._b)

    def set_error_budget(self, eh):
        check_batch(lib().bertha_gpu_batch_set_error_budget(self._b, float(eh)), self._b)

    def clmfast_device(self, d_dent, d_gdir, d_gxch, ilev=3, stream=0):
        check_batch(lib().bertha_gpu_batch_clmfast_device(
            self._b, ctypes.c_void_p(d_dent), int(ilev), ctypes.c_void_p(d_gdir),
            ctypes.c_void_p(d_gxch), ctypes.c_void_p(stream)), self._b)

    def quartets(self):
        return int(lib().bertha_gpu_batch_quartets(self._b))

    def auto_stats(self):
        nq = (ctypes.c_longlong * 3)()
        r = ctypes.c_int()
        check_batch(lib().bertha_gpu_batch_kernel_stats(self._b, nq, ctypes.byref(r)), self._b)
        return {"fp64_quartets": nq[0], "df32_quartets": nq[1], "tc32_quartets": nq[2],
                "runs": r.value}

    def launches(self):
        return int(lib().bertha_gpu_batch_launches(self._b))

    def close(self):
        if self._b:
            lib().bertha_gpu_batch_free(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
