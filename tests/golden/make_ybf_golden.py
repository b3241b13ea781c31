"""Writes ybf_plus_388.json: the reference's own recorded Dirac-Coulomb SCF
of YbF+ at R = 3.88 bohr, as a golden fixture for the Fock-build chain.

Input (read from the reference tree, which must be present here; the
fixture travels without it):
- input/YbFplus_388.inp, the CARDIN deck: geometry, Gaussian nuclei,
  optimised Yb 26s26p15d8f and F 10s6p exponents, NCLS = 78, the atomic
  configurations (Yb 68 and F 10 electrons) and the stage level shifts;
- output/YbFplus_388_DHFP_HFSCF_scf.out, the log of that deck's run
  (HMLT DHFP: a Dirac-Coulomb SCF, Breit and QED added only after
  convergence, which leaves the recorded SCF energies those of the
  Dirac-Coulomb Hamiltonian).

Output: the deck's data, the energy terms ENRGIES printed at every
iteration (nucleus-nucleus, electron-nucleus, kinetic, Coulomb direct and
exchange, total) with the iteration's inclusion level, and the spinor
energies of the last two iterations.

  python tests/golden/make_ybf_golden.py /root/reference
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "bertha-program_gb300"))

from berthagpu import deck  # noqa: E402

DECK = "input/YbFplus_388.inp"
LOG = "output/YbFplus_388_DHFP_HFSCF_scf.out"
TERMS = {"Nucleus-nucleus": "enuc", "Electron-nucleus": "enuc_el", "Electron kinetic": "ekin",
         "Coulomb direct (closed)": "gdir", "Coulomb exchange (closed)": "gxch",
         "Molecule total": "total"}


def parse_log(text):
    its, cur = [], None
    spec = re.compile(r"^\s*(\d+)\s+(\d+) \((\w+)\s*\)\s+(\S+)\s+(-?\d+/2)\s+(-?\d+\.\d+)\s+(\d+\.\d+)\s*$")
    for line in text.splitlines():
        # the iteration's header (indented), not its convergence summary
        m = re.match(r"^\s{10,}Iteration number\s+(\d+)\s*$", line)
        if m:
            cur = {"iter": int(m.group(1)), "terms": {}, "spinors": []}
            its.append(cur)
            continue
        if cur is None:
            continue
        m = re.match(r"^ Integral inclusion level\s+(\d+)\s*$", line)
        if m:
            cur["ilev"] = int(m.group(1))
            continue
        m = spec.match(line)
        if m:
            cur["spinors"].append({"centre": int(m.group(2)), "term": m.group(4),
                                   "mj": m.group(5), "energy": float(m.group(6)),
                                   "population": float(m.group(7))})
            continue
        for label, key in TERMS.items():
            if line.startswith(" " + label) and key not in cur["terms"]:
                cur["terms"][key] = float(line.split()[-1])
    return [i for i in its if "total" in i["terms"]]


def main(ref):
    b, meta = deck.read_deck(os.path.join(ref, DECK))
    with open(os.path.join(ref, LOG)) as f:
        text = f.read()
    ndim = int(re.search(r"Fock matrix dimension:\s+(\d+)", text).group(1))
    clight = float(re.search(r"Speed of light:\s+(\S+)", text).group(1))
    its = parse_log(text)
    centres = []
    for c in range(b.ncnt):
        centres.append({"xyz": [float(x) for x in b.xyz[c]], "z": b.znuc[c], "mass": b.anuc[c],
                        "nelec": meta["nelec"][c],
                        "exponents": {str(l): [float(e) for e in b.ex[c, l, :b.nfn[c, l]]]
                                      for l in range(b.nfn.shape[1]) if b.nfn[c, l] > 0}})
    out = {"source": {"deck": DECK, "log": LOG},
           "hamiltonian_of_scf": "DHFR", "ndim": ndim, "speed_of_light": clight,
           "ncls": meta["ncls"], "shifts": list(meta["shifts"]), "start_stage": meta["ilev"],
           "centres": centres,
           "iterations": [{"iter": i["iter"], "ilev": i["ilev"], **i["terms"]} for i in its],
           "spinors_last": its[-1]["spinors"], "spinors_previous": its[-2]["spinors"]}
    with open(os.path.join(HERE, "ybf_plus_388.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"{len(its)} iterations, ndim {ndim}, last total {its[-1]['terms']['total']}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
