"""Closed-shell Dirac-Hartree-Fock SCF driver on the GPU.

Mirrors the structure of the reference's HFSCF (bertha-scf.f:5097-6680)
for a closed-shell molecule: the one-electron matrices once (OVRLP + ONEEL,
:5345-5346), then per iteration the two-electron Fock build (CLMFAST :5401,
BRTFAST :5441 for DHFB/DHFQ), the Fock matrix
F = HNUC + HKIN + GDIR - GXCH - BXCH (:5518), the energies of ENRGIES
(:3698; E = ENUC + sum_ij D_ij (H_ij + G_ij/2), elementwise as the
reference sums), DIIS extrapolation (:3883), the generalized eigenproblem
F C = S C E (ZHEGV, :5557) and DENSTY (:3580, D_ij = sum_occ conj(C_i) C_j
over the lowest NOCC positive-energy states).  Everything stays on the
device: the Fock build through the library's device entry points, the
linear algebra (eigensolver, DIIS) through torch on the same stream, FP64.
The reference's stage progression (ILEV 1..3), level shifting and damping
only change the path to convergence; this driver starts from the
bare-nucleus guess and runs every iteration at stage 3.
"""
import time

import numpy as np

from . import deck
from .fock import FockBuilder

CLIGHT = 137.035999084


def nuclear_repulsion(basis):
    """ENUC of NUCGEOM (bertha-scf.f:2549-2573): point charges."""
    e = 0.0
    z = basis.znuc
    for i in range(basis.ncnt):
        for j in range(i):
            e += z[i] * z[j] / float(np.linalg.norm(basis.xyz[i] - basis.xyz[j]))
    return e


class GPUBackend:
    """Fock-build backend on the library's device entry points.  Buffers are
    row-major tensors holding column-major matrices, so each matrix is the
    transposed view of its buffer."""

    def __init__(self, basis, precision="fp64", screen=1e-12, breit=None, racah1=False,
                 torch=None):
        self.t = torch
        self.basis = basis
        self.breit = (basis.hmlt >= deck.HMLT["DHFB"]) if breit is None else bool(breit)
        self.fb = FockBuilder(basis, racah1=racah1)
        self.fb.set_precision(precision)
        self.fb.set_screening(screen)
        self.n = self.fb.ndim
        self.device = "cuda"
        self.bufs = [self._mat() for _ in range(4)]

    def _mat(self):
        return self.t.zeros((self.n, self.n), dtype=self.t.complex128, device="cuda")

    def _stream(self):
        return self.t.cuda.current_stream().cuda_stream

    def oneel(self):
        b = self.basis
        S, V, T = self._mat(), self._mat(), self._mat()
        xi = deck.nuclear_exponents(b.znuc, b.anuc)
        self.fb.oneel_device(b.znuc, xi, S.data_ptr(), V.data_ptr(), T.data_ptr(), self.n,
                             self._stream())
        return S.T.contiguous(), V.T.contiguous(), T.T.contiguous()

    def fock(self, D):
        """G = GDIR - GXCH (- BXCH) for the density D (reference convention)."""
        bd, bj, bk, bb = self.bufs
        sp = self._stream()
        bd.copy_(D.T)
        self.fb.clmfast_device(bd.data_ptr(), bj.data_ptr(), bk.data_ptr(), 3, self.n, sp)
        G = (bj - bk).T
        if self.breit:
            self.fb.brtfast_device(bd.data_ptr(), bb.data_ptr(), 3, self.n, sp)
            G = G - bb.T
        return G

    def sync(self):
        self.t.cuda.synchronize()

    def close(self):
        self.fb.close()


class DHFSCF:
    """The SCF loop over a backend providing oneel() and fock(D)."""

    def __init__(self, basis, nocc, precision="fp64", screen=1e-12, breit=None, racah1=False,
                 torch=None, backend=None):
        if torch is None:
            import torch as _t
            torch = _t
        self.torch = torch
        self.basis = basis
        self.nocc = int(nocc)
        self.backend = backend or GPUBackend(basis, precision, screen, breit, racah1, torch)
        self.n = self.backend.n

    def run(self, max_iter=60, etol=1e-9, ndiis=8, shift=0.5, verbose=False):
        """Iterate to |dE| < etol.  shift: LEVSHFT's virtual-space level shift
        SHLV in Eh (the H2O deck's stage-3 value 0.5), applied from the second
        iteration on; it moves the path, not the converged solution."""
        t = self.torch
        be = self.backend
        dev = be.device
        t0 = time.perf_counter()
        S, V, T = be.oneel()
        H1 = V + T
        enuc = nuclear_repulsion(self.basis)
        # orthogonaliser X = S^-1/2 over the non-singular subspace
        s, U = t.linalg.eigh(S)
        keep = s > 1e-10 * s.max()
        X = U[:, keep] / t.sqrt(s[keep])[None, :]
        be.sync()
        t_one = time.perf_counter() - t0

        def solve(F):
            e, Cp = t.linalg.eigh(X.conj().T @ F @ X)
            C = X @ Cp
            nneg = int((e < -CLIGHT * CLIGHT).sum().item())
            occ = C[:, nneg:nneg + self.nocc]
            # DENSTY: D_ij = sum_occ conj(C_i) C_j
            return e, nneg, occ.conj() @ occ.T, C

        eps, nneg, D, C = solve(H1)
        hist_F, hist_E = [], []
        energy, last = None, None
        iters, t_fock, t_lin = [], 0.0, 0.0
        for it in range(1, max_iter + 1):
            ti = time.perf_counter()
            G = be.fock(D)
            be.sync()
            tf = time.perf_counter()
            t_fock += tf - ti
            F = H1 + G
            # ENRGIES on the density that built F
            energy = enuc + float(t.sum(D * (H1 + 0.5 * G)).real.item())
            if shift and it > 1:
                # LEVSHFT (:3641): F += SHLV sum_vir (S c_v)(S c_v)^+ over the
                # positive-energy virtuals of the last diagonalisation
                A = S @ C[:, nneg + self.nocc:]
                F = F + shift * (A @ A.conj().T)
            # DIIS on the commutator F P S - S P F, P = D^T
            P = D.T
            err = F @ P @ S - S @ P @ F
            hist_F.append(F)
            hist_E.append(err)
            if len(hist_F) > ndiis:
                hist_F.pop(0)
                hist_E.pop(0)
            m = len(hist_F)
            if m > 1:
                B = t.zeros((m + 1, m + 1), dtype=t.float64, device=dev)
                for i in range(m):
                    for j in range(i + 1):
                        v = t.sum(hist_E[i].conj() * hist_E[j]).real
                        B[i, j] = v
                        B[j, i] = v
                B[m, :m] = -1.0
                B[:m, m] = -1.0
                rhs = t.zeros(m + 1, dtype=t.float64, device=dev)
                rhs[m] = -1.0
                w = t.linalg.solve(B, rhs)
                F = sum(w[i] * hist_F[i] for i in range(m))
            eps, nneg, D, C = solve(F)
            be.sync()
            t_lin += time.perf_counter() - tf
            de = None if last is None else energy - last
            iters.append({"iter": it, "energy": energy, "de": de,
                          "err": float(err.abs().max().item()),
                          "s": time.perf_counter() - ti})
            if verbose:
                print(iters[-1], flush=True)
            if last is not None and abs(de) < etol:
                break
            last = energy
        return {"energy": energy, "enuc": enuc, "iterations": len(iters),
                "converged": bool(iters and iters[-1]["de"] is not None
                                  and abs(iters[-1]["de"]) < etol),
                "oneel_s": t_one, "fock_s": t_fock, "linalg_s": t_lin,
                "wall_s": t_one + t_fock + t_lin, "history": iters,
                "orbital_energies": eps[nneg:nneg + self.nocc].cpu().numpy().tolist()}

    def close(self):
        self.backend.close()
