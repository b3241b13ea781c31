"""Run one Fock build of a built-in case or a BERTHA deck and print timings.

  python -m berthagpu.run --case tlf --build breit --screen 1e-12
  python -m berthagpu.run --deck input/H2O.inp --build coulomb --precision df32

Cases: h2o, tlf, tlf-small, c6h6.  The density is a seeded random Hermitian
one (DENSTY form); the output is one JSON line with the wall time of each
call through the host-array entry points and the energy terms
1/2 sum_ij D_ij G_ij of the matrices built (ENRGIES' convention).
"""
import argparse
import json
import time

import numpy as np

from . import deck
from .fock import FockBuilder

CASES = {"h2o": deck.h2o_basis, "tlf": deck.tlf_basis, "tlf-small": deck.tlf_small_basis,
         "c6h6": deck.c6h6_basis}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    g = p.add_mutually_exclusive_group(required=True)
    g.add_argument("--case", choices=sorted(CASES))
    g.add_argument("--deck")
    p.add_argument("--build", choices=["coulomb", "breit", "both"], default="coulomb")
    p.add_argument("--precision", choices=["fp64", "df32"], default="fp64")
    p.add_argument("--ilev", type=int, default=3)
    p.add_argument("--screen", type=float, default=0.0)
    p.add_argument("--repeat", type=int, default=1)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-racah1", action="store_true")
    p.add_argument("--gaunt", action="store_true")
    a = p.parse_args(argv)
    b = CASES[a.case]() if a.case else deck.read_deck(a.deck)
    if a.build != "coulomb" and b.hmlt < deck.HMLT["DHFR"]:
        b = dataclasses_replace(b, deck.HMLT["DHFB"])
    dent = deck.density(b, seed=a.seed, real=b.isym != 0)
    out = {"case": a.case or a.deck, "ndim": b.ndim, "shells": len(b.shells()),
           "isym": int(b.isym), "build": a.build, "precision": a.precision,
           "ilev": a.ilev, "screen": a.screen}
    t0 = time.perf_counter()
    fb = FockBuilder(b, racah1=not a.no_racah1, gaunt=a.gaunt)
    fb.set_precision(a.precision)
    fb.set_screening(a.screen)
    out["init_s"] = time.perf_counter() - t0
    if a.build in ("coulomb", "both"):
        ts = []
        for _ in range(a.repeat):
            t0 = time.perf_counter()
            gd, gx = fb.clmfast(dent, a.ilev)
            ts.append(time.perf_counter() - t0)
        out["coulomb_s"] = ts
        out["energy_j_eh"] = float(0.5 * np.sum(dent * gd).real)
        out["energy_k_eh"] = float(0.5 * np.sum(dent * gx).real)
    if a.build in ("breit", "both"):
        ts = []
        for _ in range(a.repeat):
            t0 = time.perf_counter()
            bx = fb.brtfast(dent, a.ilev)
            ts.append(time.perf_counter() - t0)
        out["breit_s"] = ts
        out["energy_bx_eh"] = float(0.5 * np.sum(dent * bx).real)
    fb.close()
    print(json.dumps(out), flush=True)


def dataclasses_replace(b, hmlt):
    return deck.Basis(xyz=b.xyz, lmax=b.lmax, nfn=b.nfn, ex=b.ex, hmlt=hmlt, isym=b.isym,
                      znuc=b.znuc, name=b.name)


if __name__ == "__main__":
    main()
