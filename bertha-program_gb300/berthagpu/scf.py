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
The reference's stage progression (ILEV 1..3 with a level shift per
stage, :6038-6110) is available as `stages`; without it every iteration
runs at stage 3.  Stages, level shifts and the start only change the path
to convergence, not the converged solution.
"""
import time

import numpy as np

from . import deck, wfn
from .fock import FockBatch, FockBuilder

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
        self.ilev = 3  # integral inclusion level of the Coulomb builds
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
        self.fb.clmfast_device(bd.data_ptr(), bj.data_ptr(), bk.data_ptr(), self.ilev, self.n,
                               sp)
        G = (bj - bk).T
        if self.breit:
            # multi-centre Breit quartets from ILEV 3 on, as BRTFAST (:17231)
            self.fb.brtfast_device(bd.data_ptr(), bb.data_ptr(), self.ilev, self.n, sp)
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

    def run(self, max_iter=60, etol=1e-9, ndiis=8, shift=0.5, mom=0, verbose=False,
            guess=None, wfn_out=None, return_density=False, dtol=None, dc_first=None,
            stages=None):
        """Iterate to |dE| < etol and, with dtol, until the largest change of
        a density-matrix element between iterations is below dtol too, so
        that a converged energy does not depend on where a slowly drifting
        iteration happened to stop.  (The DIIS error F P S - S P F, whose
        largest element is recorded as "err", is no stopping test: for a
        heavy atom its rounding floor sits near 1e-5 from Fock elements near
        2c^2, and in the orthonormal basis the near-singular directions of
        the kinetically balanced overlap magnify it further.)
        dc_first: with a Breit Hamiltonian, iterate without the Breit term
        until |dE| < dc_first, then add it (DIIS restarted): the Breit
        interaction is a small correction, and the cheaper Dirac-Coulomb
        iterations take the density most of the way.
        shift: LEVSHFT's virtual-space level shift
        SHLV in Eh (the H2O deck's stage-3 value 0.5), applied from the second
        iteration on; it moves the path, not the converged solution.
        mom: from this iteration on (0: never) the occupied spinors are the
        positive-energy eigenvectors that overlap most with the previous
        occupied space (maximum overlap) instead of the lowest ones, which
        stops occupations from flipping between near-degenerate levels.
        guess: None for the bare-nucleus start (diagonalised H1), a density
        matrix (NDIM x NDIM), (EIGN, COEF) of a wavefunction file (DENSTY of
        its occupied states) or "atomic" (superposed atomic densities, see
        atomic_guess).  wfn_out: write the last eigenvalues and eigenvectors
        as a `.wfn` file (virtual eigenvalues without the level shift, as
        HFSCF writes them).
        stages: HFSCF's integral inclusion levels before the last one, as
        (ilev, shift, tol, max_iter) tuples, e.g. ((1, 3.0, 1e-8, 12),
        (2, 1.0, 5e-11, 15)): iterate with the Coulomb build at ILEV ilev
        and level shift `shift` until the weighted energy difference
        |dE| / (|E| + 1) falls below tol (HFSCF's ENRGLV1 = 1e-8 and
        ENRGLV2 = 5e-11, :5167-5168) or the stage has run max_iter
        iterations, then move to the next stage with a fresh DIIS subspace;
        the last stage is ILEV 3 with `shift`, where the convergence tests
        apply."""
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

        state = {"occ": None}

        def solve(F, use_mom=False):
            e, Cp = t.linalg.eigh(X.conj().T @ F @ X)
            C = X @ Cp
            nneg = int((e < -CLIGHT * CLIGHT).sum().item())
            if use_mom and state["occ"] is not None:
                # projections of the positive-energy eigenvectors on the
                # previous occupied space, S-metric
                P = state["occ"].conj().T @ (S @ C[:, nneg:])
                w = (P.abs() ** 2).sum(0)
                idx = t.sort(t.topk(w, self.nocc).indices).values + nneg
                occ = C[:, idx]
            else:
                idx = t.arange(nneg, nneg + self.nocc, device=C.device)
                occ = C[:, nneg:nneg + self.nocc]
            state["occ"] = occ
            vmask = t.ones(C.shape[1], dtype=t.bool, device=C.device)
            vmask[:nneg] = False
            vmask[idx] = False
            state["vir"] = C[:, vmask]
            # DENSTY: D_ij = sum_occ conj(C_i) C_j
            return e, nneg, occ.conj() @ occ.T, C

        if guess is None:
            eps, nneg, D, C = solve(H1)
        else:
            if isinstance(guess, str) and guess == "atomic":
                guess = atomic_guess(self.basis, torch=t,
                                     backend_factory=getattr(be, "atom_factory", None))
            if isinstance(guess, tuple):
                eign, coef = guess
                nskp = int((np.asarray(eign) < -CLIGHT * CLIGHT).sum())
                guess = wfn.density(coef, nskp, self.nocc)
            D = t.as_tensor(np.asarray(guess), dtype=t.complex128, device=dev)
            eps, nneg, C = None, 0, None
        hist_F, hist_E = [], []
        energy, last = None, None
        iters, t_fock, t_lin = [], 0.0, 0.0
        staged = bool(dc_first) and getattr(be, "breit", False)
        if staged:
            be.breit = False
        plan = [tuple(st) for st in (stages or ())]
        si, n_stage = 0, 0

        def enter_stage():
            be.ilev = plan[si][0] if si < len(plan) else 3
            return plan[si][1] if si < len(plan) else shift

        cur_shift = enter_stage()
        for it in range(1, max_iter + 1):
            ti = time.perf_counter()
            G = be.fock(D)
            be.sync()
            tf = time.perf_counter()
            t_fock += tf - ti
            F = H1 + G
            # ENRGIES on the density that built F
            energy = enuc + float(t.sum(D * (H1 + 0.5 * G)).real.item())
            if cur_shift and it > 1 and "vir" in state:
                # LEVSHFT (:3641): F += SHLV sum_vir (S c_v)(S c_v)^+ over the
                # positive-energy virtuals of the last diagonalisation
                A = S @ state["vir"]
                F = F + cur_shift * (A @ A.conj().T)
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
            D_old = D
            eps, nneg, D, C = solve(F, use_mom=bool(mom) and it >= mom)
            ddens = float((D - D_old).abs().max().item())
            be.sync()
            t_lin += time.perf_counter() - tf
            de = None if last is None else energy - last
            iters.append({"iter": it, "energy": energy, "de": de, "ddens": ddens,
                          "err": float(err.abs().max().item()),
                          "breit": bool(getattr(be, "breit", False)),
                          "ilev": int(getattr(be, "ilev", 3)), "shift": cur_shift,
                          "s": time.perf_counter() - ti})
            if verbose:
                print(iters[-1], flush=True)
            if si < len(plan):
                # HFSCF's stage test (:6038-6098) on the weighted energy
                # difference
                n_stage += 1
                if ((de is not None and abs(de) / (abs(energy) + 1.0) < plan[si][2])
                        or n_stage >= plan[si][3]):
                    si, n_stage = si + 1, 0
                    cur_shift = enter_stage()
                    hist_F, hist_E = [], []
                    last = None
                else:
                    last = energy
                continue
            if staged and not be.breit:
                if last is not None and abs(de) < dc_first:
                    # the Breit term from the next build on
                    be.breit = True
                    hist_F, hist_E = [], []
                    energy = None
                last = energy
                continue
            if (last is not None and abs(de) < etol
                    and (dtol is None or ddens < dtol)):
                break
            last = energy
        if staged:
            be.breit = True
        final_stage = si >= len(plan)
        be.ilev = 3
        if wfn_out:
            n = self.n
            e = eps.cpu().numpy().copy()
            Cn = C.cpu().numpy()
            if cur_shift and len(iters) > 1:
                vir = np.ones(len(e), bool)
                vir[:nneg] = False
                occ_e = sorted(e[nneg:])[:self.nocc]
                vir &= ~np.isin(e, occ_e)
                e[vir] -= cur_shift
            # the orthogonaliser may drop near-singular directions: pad to
            # NDIM records with zero vectors
            eign = np.zeros(n)
            coef = np.zeros((n, n), dtype=np.complex128)
            eign[:len(e)] = e
            coef[:, :Cn.shape[1]] = Cn
            wfn.write_wfn(wfn_out, eign, coef)
        out = {"energy": energy, "enuc": enuc, "iterations": len(iters),
               "converged": bool(iters and iters[-1]["de"] is not None
                                 and abs(iters[-1]["de"]) < etol
                                 and (dtol is None or iters[-1]["ddens"] < dtol)
                                 and (not staged or iters[-1]["breit"])
                                 and final_stage),
               "density_change": iters[-1]["ddens"] if iters else None,
               "commutator": iters[-1]["err"] if iters else None,
               "oneel_s": t_one, "fock_s": t_fock, "linalg_s": t_lin,
               "wall_s": t_one + t_fock + t_lin, "history": iters,
               "orbital_energies": eps[nneg:nneg + self.nocc].cpu().numpy().tolist()}
        if return_density:
            out["density"] = D
        return out

    def energy_at(self, D):
        """ENRGIES' total energy of the density D (NDIM x NDIM, device) with
        this backend's Fock build: one build, no iteration.  Two precisions'
        energies at one converged density measure the precision's effect on
        the energy apart from where each SCF stops."""
        t = self.torch
        S, V, T = self.backend.oneel()
        H1 = V + T
        G = self.backend.fock(D)
        self.backend.sync()
        return nuclear_repulsion(self.basis) + float(t.sum(D * (H1 + 0.5 * G)).real.item())

    def close(self):
        self.backend.close()


def atomic_guess(basis, torch=None, backend_factory=None, max_iter=25, etol=1e-6, nelec=None):
    """Starting density of a molecule from SCFs of its atoms (the role of the
    atomic wavefunctions the reference reads from bertha-atomic): for every
    centre, a Dirac-Coulomb SCF of the centre's own basis functions with
    NOCC = Z spinors occupied (maximum-overlap occupation, so that an odd
    electron count keeps one spinor of its Kramers pair), its density placed
    on the centre's rows and columns of the molecular layout (FOCKIND).
    Centres with the same charge and exponents share one atomic SCF.
    backend_factory(atom) makes the Fock-build backend of an atom (default:
    the GPU library).  nelec: electrons per centre instead of Z (the
    electron counts of a deck's atomic configurations, e.g. an ion's)."""
    if torch is None:
        import torch as _t
        torch = _t
    hm = "NORL" if basis.hmlt == deck.HMLT["NORL"] else "DHFR"
    cache, dens = {}, []
    for c in range(basis.ncnt):
        z = int(round(float(basis.znuc[c])))
        if z <= 0:
            dens.append(None)
            continue
        atom = wfn.atom_of_centre(basis, c, hmlt=hm)
        ne = z if nelec is None else int(nelec[c])
        key = (z, ne, atom.ex.tobytes(), atom.nfn.tobytes())
        if key not in cache:
            be = backend_factory(atom) if backend_factory else None
            s = DHFSCF(atom, nocc=ne, screen=1e-12, racah1=False, torch=torch, backend=be)
            r = s.run(max_iter=max_iter, etol=etol, mom=2, return_density=True)
            s.close()
            cache[key] = r["density"].cpu().numpy()
        dens.append(cache[key])
    return wfn.embed_atomic_densities(basis, dens)


class BatchedDHFSCF:
    """Closed-shell DHF SCF of many independent instances at once (atoms
    and ions of different basis sizes), every step batched on the GPU.

    The instances' matrices are padded to the largest NDIM N and held as
    [n, N, N] tensors; the two-electron build is one FockBatch call (one
    kernel launch per component class for all instances), captured once as
    a CUDA graph and replayed every iteration.  Per instance the loop is the
    one of DHFSCF (HFSCF's order: Fock build, ENRGIES, LEVSHFT, DIIS, ZHEGV,
    DENSTY).  Padding rows and columns carry S = 1 and a large positive
    diagonal in F, so they form eigenvectors of their own that are never
    occupied; near-singular overlap directions are shifted out the same way.
    """

    PAD = 1.0e4

    def __init__(self, bases, nocc, precision="fp64", screen=1e-12, racah1=False, torch=None,
                 graph=True):
        if torch is None:
            import torch as _t
            torch = _t
        t = self.torch = torch
        self.bases = list(bases)
        self.nocc = [int(x) for x in nocc]
        n = self.n = len(self.bases)
        builders = [FockBuilder(b, racah1=racah1) for b in self.bases]
        for fb in builders:
            fb.set_precision(precision)
            fb.set_screening(screen)
        self.ndim = [fb.ndim for fb in builders]
        N = self.N = max(self.ndim)
        z = dict(dtype=t.complex128, device="cuda")
        S, V, T = (t.zeros((n, N, N), **z) for _ in range(3))
        st = t.cuda.current_stream().cuda_stream
        for k, (b, fb) in enumerate(zip(self.bases, builders)):
            xi = deck.nuclear_exponents(b.znuc, b.anuc)
            fb.oneel_device(b.znuc, xi, S[k].data_ptr(), V[k].data_ptr(), T[k].data_ptr(), N, st)
        self.batch = FockBatch(builders, moff=[k * N * N for k in range(n)], ld=[N] * n)
        for fb in builders:
            fb.close()
        # column-major buffers -> matrices
        self.S = S.transpose(1, 2).contiguous()
        self.H1 = (V + T).transpose(1, 2).contiguous()
        idx = t.arange(N, device="cuda")
        nd = t.tensor(self.ndim, device="cuda")
        inside = idx[None, :] < nd[:, None]                      # [n, N]
        self.block = (inside[:, :, None] & inside[:, None, :]).to(t.float64)
        pad = (~inside).to(t.complex128)
        self.S = self.S + t.diag_embed(pad)
        self.H1 = self.H1 + self.PAD * t.diag_embed(pad)
        self.enuc = t.tensor([nuclear_repulsion(b) for b in self.bases], dtype=t.float64,
                             device="cuda")
        self.bufs = [t.zeros((n, N, N), **z) for _ in range(3)]
        self.graph = None
        self.precision = precision
        if graph:
            bd, bj, bk = self.bufs
            s = t.cuda.Stream()
            s.wait_stream(t.cuda.current_stream())
            with t.cuda.stream(s):
                # first call: quartet lists and scratch (host work, allocation)
                self.batch.clmfast_device(bd.data_ptr(), bj.data_ptr(), bk.data_ptr(), 3,
                                          s.cuda_stream)
            s.synchronize()
            g = t.cuda.CUDAGraph()
            with t.cuda.graph(g, stream=s):
                self.batch.clmfast_device(bd.data_ptr(), bj.data_ptr(), bk.data_ptr(), 3,
                                          t.cuda.current_stream().cuda_stream)
            self.graph = g

    def fock(self, D):
        """G = GDIR - GXCH of every instance for the densities D [n, N, N]."""
        bd, bj, bk = self.bufs
        bd.copy_(D.transpose(1, 2))
        if self.graph is not None:
            self.graph.replay()
        else:
            self.batch.clmfast_device(bd.data_ptr(), bj.data_ptr(), bk.data_ptr(), 3,
                                      self.torch.cuda.current_stream().cuda_stream)
        return (bj - bk).transpose(1, 2)

    def quartets(self):
        return self.batch.quartets()

    def run(self, max_iter=60, etol=1e-9, ndiis=8, shift=0.5, mom=0, verbose=False):
        """As DHFSCF.run for every instance at once (mom: maximum-overlap
        occupation from that iteration on, per instance)."""
        t = self.torch
        n, N = self.n, self.N
        t0 = time.perf_counter()
        S, H1 = self.S, self.H1
        s, U = t.linalg.eigh(S)
        keep = s > 1e-10 * s.max(dim=1, keepdim=True).values
        X = U * t.where(keep, s.clamp_min(1e-300).rsqrt(), t.zeros_like(s))[:, None, :]
        drop = t.diag_embed((~keep).to(t.complex128)) * self.PAD
        Xh = X.conj().transpose(1, 2)
        nocc = t.tensor(self.nocc, device="cuda")
        col = t.arange(N, device="cuda")[None, :]
        c2 = CLIGHT * CLIGHT

        state = {"occ": None}

        def solve(F, use_mom=False):
            e, Cp = t.linalg.eigh(Xh @ F @ X + drop)
            C = X @ Cp
            nneg = (e < -c2).sum(dim=1, keepdim=True)
            # positive-energy eigenvectors (padding and dropped directions
            # sit at PAD)
            pos = (col >= nneg) & (e < 0.5 * self.PAD)
            if use_mom and state["occ"] is not None:
                # the NOCC positive-energy eigenvectors with the largest
                # projection on the previous occupied space, per instance
                w = ((state["occ"].conj().transpose(1, 2) @ (S @ C)).abs() ** 2).sum(1)
                w = t.where(pos, w, t.full_like(w, -1.0))
                rank = t.argsort(t.argsort(-w, dim=1), dim=1)
                occb = rank < nocc[:, None]
            else:
                occb = (col >= nneg) & (col < nneg + nocc[:, None])
            occ = occb.to(t.complex128)
            vir = (pos & ~occb).to(t.complex128)
            Co = C * occ[:, None, :]
            state["occ"] = Co
            # DENSTY: D_ij = sum_occ conj(C_i) C_j
            return e, Co.conj() @ Co.transpose(1, 2), C * vir[:, None, :], nneg

        eps, D, Cv, nneg = solve(H1)
        t.cuda.synchronize()
        t_one = time.perf_counter() - t0
        hist_F, hist_E = [], []
        last = None
        done = t.zeros(n, dtype=t.bool, device="cuda")
        iters, t_fock, t_lin = [], 0.0, 0.0
        energy = None
        for it in range(1, max_iter + 1):
            ti = time.perf_counter()
            G = self.fock(D)
            t.cuda.synchronize()
            tf = time.perf_counter()
            t_fock += tf - ti
            F = H1 + G
            energy = self.enuc + (D * (H1 + 0.5 * G) * self.block).sum(dim=(1, 2)).real
            if shift and it > 1:
                A = S @ Cv
                F = F + shift * (A @ A.conj().transpose(1, 2))
            P = D.transpose(1, 2)
            err = F @ P @ S - S @ P @ F
            hist_F.append(F)
            hist_E.append(err)
            if len(hist_F) > ndiis:
                hist_F.pop(0)
                hist_E.pop(0)
            m = len(hist_F)
            if m > 1:
                Es = t.stack(hist_E, 1).reshape(n, m, -1)
                B = t.zeros((n, m + 1, m + 1), dtype=t.float64, device="cuda")
                B[:, :m, :m] = (Es.conj() @ Es.transpose(1, 2)).real
                # scale-invariant regularisation for instances already converged
                tr = B[:, :m, :m].diagonal(dim1=1, dim2=2).mean(1).clamp_min(1e-300)
                B[:, :m, :m] += 1e-14 * tr[:, None, None] * t.eye(m, device="cuda")
                B[:, m, :m] = -1.0
                B[:, :m, m] = -1.0
                rhs = t.zeros((n, m + 1), dtype=t.float64, device="cuda")
                rhs[:, m] = -1.0
                w = t.linalg.solve(B, rhs)[:, :m].to(t.complex128)
                F = (t.stack(hist_F, 1) * w[:, :, None, None]).sum(1)
            eps, D, Cv, nneg = solve(F, use_mom=bool(mom) and it >= mom)
            t.cuda.synchronize()
            t_lin += time.perf_counter() - tf
            de = None if last is None else energy - last
            if de is not None:
                done = de.abs() < etol
            iters.append({"iter": it, "max_abs_de": None if de is None else float(de.abs().max()),
                          "converged": int(done.sum()), "s": time.perf_counter() - ti})
            if verbose:
                print(iters[-1], flush=True)
            if bool(done.all()):
                break
            last = energy
        return {"energy": energy.cpu().numpy().tolist(),
                "converged": done.cpu().numpy().tolist(),
                "iterations": len(iters), "oneel_s": t_one, "fock_s": t_fock,
                "linalg_s": t_lin, "wall_s": t_one + t_fock + t_lin,
                "quartets_per_build": self.quartets(), "history": iters}

    def close(self):
        self.graph = None
        self.batch.close()
