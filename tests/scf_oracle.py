"""SCF backends on the oracle (test infrastructure): one-electron matrices and
Fock builds of the CPU restatement, as torch CPU tensors, for the DHFSCF
loop of berthagpu.scf.  OracleBackend builds by the MD route throughout
(RACAH1 off, as the GPU library does); ReferenceRouteBackend by the
reference's default route (CLMFAST with RACAH1 on plus COULOMB1 per
centre)."""
import numpy as np
import torch

from berthagpu import deck
from oracle import oracle as orc


class OracleBackend:
    device = "cpu"

    def __init__(self, basis, racah1=False, breit=False):
        self.basis = basis
        self.racah1 = racah1
        self.breit = breit
        self.n = basis.ndim
        self.ilev = 3

    def oneel(self):
        b = self.basis
        xi = deck.nuclear_exponents(b.znuc, b.anuc)
        return tuple(torch.from_numpy(np.ascontiguousarray(m)) for m in orc.oneel(b, b.znuc, xi))

    def fock(self, D):
        d = np.asfortranarray(D.numpy())
        gd, gx = orc.clmfast(self.basis, d, self.ilev, racah1=self.racah1)
        g = gd - gx
        if self.breit:
            g = g - orc.brtfast(self.basis, d, self.ilev, racah1=self.racah1)
        return torch.from_numpy(np.ascontiguousarray(g))

    def sync(self):
        pass

    def close(self):
        pass


def _racah_part(args):
    from oracle import racah1
    atom, dent, lrge, pairs = args
    return racah1.coulomb1(atom, dent, lrge, pairs=set(pairs))


class ReferenceRouteBackend:
    """Fock builds of the reference's default route on the CPU, for
    berthagpu.scf.DHFSCF: G = GDIR - GXCH with the multi-centre terms of
    the oracle's CLMFAST (RACAH1 on: one-centre quartets skipped) and the
    one-centre terms of the Racah restatement of COULOMB1, each centre's
    block digested in its atomic layout and placed by FOCKIND."""
    device = "cpu"

    def __init__(self, basis, pool, torch):
        from berthagpu import wfn
        self.t = torch
        self.basis = basis
        self.n = basis.ndim
        self.ilev = 3
        self.pool = pool
        self.atoms = [wfn.atom_of_centre(basis, c, hmlt="DHFR") for c in range(basis.ncnt)]
        self.idx = [wfn.centre_index_map(basis, c, a) for c, a in enumerate(self.atoms)]
        self.lrge = [wfn.fock_layout(a)[0] for a in self.atoms]

    def oneel(self):
        from berthagpu import deck
        from oracle import oracle as orc
        b = self.basis
        xi = deck.nuclear_exponents(b.znuc, b.anuc)
        return tuple(self.t.from_numpy(np.ascontiguousarray(m))
                     for m in orc.oneel(b, b.znuc, xi))

    def _one_centre(self, c, d):
        atom = self.atoms[c]
        nk = 2 * int(atom.lmax[0]) + 1
        pairs = sorted(((a, b) for a in range(1, nk + 1) for b in range(1, nk + 1)),
                       key=lambda p: -(p[0] + p[1]))
        nw = self.pool._max_workers
        chunks = [pairs[k::nw] for k in range(nw)]
        jobs = [(atom, d, self.lrge[c], ch) for ch in chunks if ch]
        gd = np.zeros_like(d)
        gx = np.zeros_like(d)
        for rd, rx in self.pool.map(_racah_part, jobs):
            gd += rd
            gx += rx
        return gd, gx

    def fock(self, D):
        from oracle import oracle as orc
        d = np.asfortranarray(D.numpy())
        gd, gx = orc.clmfast(self.basis, d, self.ilev, racah1=True)
        gd, gx = np.array(gd), np.array(gx)
        for c in range(self.basis.ncnt):
            ix = np.ix_(self.idx[c], self.idx[c])
            rd, rx = self._one_centre(c, np.ascontiguousarray(d[ix]))
            gd[ix] += rd
            gx[ix] += rx
        return self.t.from_numpy(np.ascontiguousarray(gd - gx))

    def sync(self):
        pass

    def close(self):
        pass
