"""SCF backend on the oracle (test infrastructure): one-electron matrices and
Fock builds of the CPU restatement, as torch CPU tensors, for the DHFSCF
loop of berthagpu.scf."""
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
