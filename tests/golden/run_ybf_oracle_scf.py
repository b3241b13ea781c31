"""The oracle's own Dirac-Coulomb SCF of YbF+ (the deck of the golden
fixture ybf_plus_388.json), by the reference's default route: CLMFAST's
multi-centre terms with RACAH1 on (oracle/bertha_oracle.cpp) plus
COULOMB1's one-centre terms of every centre (oracle/racah1.py), as HFSCF
calls them (bertha-scf.f:5401-5421).  The SCF path is the one of
tests/test_ybf_golden.py: atomic start from the deck's configurations,
HFSCF's stages with the deck's level shifts.

CPU only and slow: on 8 cores the atomic start takes about 30 minutes
and a stage-3 build 6-7 minutes, and 32 iterations took 3.1 hours with
stage 3 still oscillating at the mEh level, as the reference's own stage
3 did.  Prints every iteration; at the end writes ybf_plus_388_oracle.json
beside this file (the energy, the iterations and the occupied spinor
energies).

  python tests/golden/run_ybf_oracle_scf.py
"""
import json
import os
import sys
import time
from concurrent.futures import ProcessPoolExecutor
import multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "bertha-program_gb300"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)


def main():
    import torch

    import test_ybf_golden as T
    from berthagpu.scf import DHFSCF, atomic_guess
    from scf_oracle import ReferenceRouteBackend
    g = T._gold()
    b = T._basis(g)
    t0 = time.time()
    with ProcessPoolExecutor(max_workers=os.cpu_count() or 1,
                             mp_context=mp.get_context("spawn")) as pool:
        factory = lambda atom: ReferenceRouteBackend(atom, pool, torch)  # noqa: E731
        guess = atomic_guess(b, torch=torch, backend_factory=factory,
                             nelec=[c["nelec"] for c in g["centres"]])
        print(f"atomic start {time.time() - t0:.0f} s", flush=True)
        scf = DHFSCF(b, nocc=g["ncls"], torch=torch, backend=factory(b))
        sh = g["shifts"]
        r = scf.run(max_iter=50, etol=1e-7, shift=sh[2], guess=guess, verbose=True,
                    stages=((1, sh[0], 1e-8, 12), (2, sh[1], 5e-11, 15)))
    hist = r["history"]
    out = {"route": "CLMFAST (RACAH1 on) + COULOMB1, oracle restatements, FP64 CPU",
           "energy": r["energy"], "converged": r["converged"], "iterations": r["iterations"],
           "last_de": hist[-1]["de"], "density_change": hist[-1]["ddens"],
           "ilev": [h["ilev"] for h in hist], "energies": [h["energy"] for h in hist],
           "orbital_energies": r["orbital_energies"], "wall_s": time.time() - t0}
    with open(os.path.join(HERE, "ybf_plus_388_oracle.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("energy", "converged", "iterations", "wall_s")}))


if __name__ == "__main__":
    main()
