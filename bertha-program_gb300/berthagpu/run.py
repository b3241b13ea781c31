"""Run one Fock build of a built-in case or a BERTHA deck and print timings.

  python -m berthagpu.run --case tlf --build breit --screen 1e-12
  python -m berthagpu.run --deck input/H2O.inp --build coulomb --precision df32

Cases: h2o, tlf, tlf-small, c6h6.  The density is a seeded random Hermitian
one (DENSTY form); the output is one JSON line with the wall time of each
call through the host-array entry points and the energy terms
1/2 sum_ij D_ij G_ij of the matrices built (ENRGIES' convention).

Batched closed-shell atoms (one FockBatch launch per component class for
all of them), the Fock build timed on the device in both precisions and,
with --scf, the batched DHF SCF in both precisions:

  python -m berthagpu.run --atoms 96 [--zmax 86] [--scf]

Quartets of the ERI microbenchmark's distribution digested through the
class-segmented explicit-list entry point, optionally one angular class
(l_a l_b l_c l_d) of one component class, device time per repeat:

  python -m berthagpu.run --microbench 262144 --lclass 3333 --comp 1 1 --precision tc32
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
    g.add_argument("--atoms", type=int, help="batch of N seeded closed-shell atoms")
    g.add_argument("--microbench", type=int,
                   help="N quartets of the ERI microbenchmark's distribution")
    p.add_argument("--lclass", help="--microbench: one angular class, e.g. 3333")
    p.add_argument("--comp", type=int, nargs=2, default=None,
                   help="--microbench: one component class t1 t2 (0 large, 1 small)")
    p.add_argument("--zmax", type=int, default=86, help="largest Z drawn for --atoms")
    p.add_argument("--scf-only", action="store_true",
                   help="--atoms: only the batched SCF, in --precision")
    p.add_argument("--scf", action="store_true",
                   help="run the closed-shell DHF SCF (with --atoms: the batched SCF too)")
    p.add_argument("--nocc", type=int, default=0, help="--scf: occupied spinors (0: sum of Z)")
    p.add_argument("--no-breit", action="store_true", help="--scf: Dirac-Coulomb only")
    p.add_argument("--etol", type=float, default=1e-9, help="--scf: |dE| convergence, Eh")
    p.add_argument("--shift", type=float, default=0.5, help="--scf: level shift, Eh")
    p.add_argument("--mom", type=int, default=0,
                   help="--scf: maximum-overlap occupation from this iteration (0: aufbau)")
    p.add_argument("--ndiis", type=int, default=8, help="--scf: DIIS subspace size")
    p.add_argument("--max-iter", type=int, default=80, help="--scf: iteration limit")
    p.add_argument("--guess", choices=["bare", "atomic"], default="bare",
                   help="--scf: bare-nucleus start or superposed atomic densities")
    p.add_argument("--staged", action="store_true",
                   help="--scf: HFSCF's integral inclusion stages from ILEV 1 (a deck's "
                        "starting stage and level shifts when given)")
    p.add_argument("--stage-iter", type=int, default=15,
                   help="--staged: iteration limit of each stage before the last")
    p.add_argument("--dtol", type=float, default=None,
                   help="--scf: largest density-matrix change for convergence")
    p.add_argument("--wfn-in", help="--scf: start from this .wfn file")
    p.add_argument("--wfn-out", help="--scf: write the final eigenvectors as a .wfn file")
    p.add_argument("--build", choices=["coulomb", "breit", "both"], default="coulomb")
    p.add_argument("--precision", choices=["fp64", "df32", "auto", "tc32"], default="fp64")
    p.add_argument("--ilev", type=int, default=3)
    p.add_argument("--screen", type=float, default=0.0)
    p.add_argument("--repeat", type=int, default=1)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-racah1", action="store_true")
    p.add_argument("--gaunt", action="store_true")
    p.add_argument("--verbose", action="store_true", help="--scf: print every iteration")
    a = p.parse_args(argv)
    if a.atoms:
        print(json.dumps(atoms_main(a)), flush=True)
        return
    if a.microbench:
        print(json.dumps(microbench_main(a)), flush=True)
        return
    meta = {}
    if a.case:
        b = CASES[a.case]()
    else:
        b, meta = deck.read_deck(a.deck)
    if a.build != "coulomb" and b.hmlt < deck.HMLT["DHFR"]:
        b = dataclasses_replace(b, deck.HMLT["DHFB"])
    if a.scf:
        print(json.dumps(scf_main(a, b, meta)), flush=True)
        return
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
        if a.precision == "auto":
            out["auto"] = fb.auto_stats()
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


def microbench_main(a):
    """Explicit lists of the ERI microbenchmark (workloads.microbench_*),
    grouped by angular class, digested with bertha_gpu_quartets_segments;
    device time of each repeat by CUDA events."""
    import torch

    from . import workloads
    b = workloads.microbench_pool(seed=a.seed)
    raw = workloads.microbench_quartets(b, a.microbench, seed=a.seed)
    dent = deck.density(b, seed=a.seed)
    fb = FockBuilder(b)
    fb.set_precision(a.precision)
    n = fb.ndim
    D = torch.from_numpy(np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)).cuda()
    GD = torch.zeros(n, 2 * n, dtype=torch.float64, device="cuda")
    GX = torch.zeros_like(GD)
    jobs = []
    for cls, q in raw.items():
        if a.comp and tuple(cls) != tuple(a.comp):
            continue
        qs, seg, lcl = workloads.group_by_class(b, q)
        keep = [i for i in range(len(seg) - 1)
                if not a.lclass or "".join(str(int(x)) for x in lcl[i]) == a.lclass]
        if not keep:
            continue
        dq = torch.from_numpy(qs).cuda()
        jobs.append((cls, dq, seg, lcl, keep))
    st = torch.cuda.current_stream()
    times, nq = [], 0
    for r in range(a.repeat):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for cls, dq, seg, lcl, keep in jobs:
            for i in keep:
                fb.quartets_segments(dq[int(seg[i]):].data_ptr(), seg[i:i + 2] - seg[i],
                                     lcl[i:i + 1], cls[0], cls[1], D.data_ptr(), GD.data_ptr(),
                                     GX.data_ptr(), n, st.cuda_stream)
                if r == 0:
                    nq += int(seg[i + 1] - seg[i])
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    from . import _lib
    fb.close()
    return {"microbench": a.microbench, "lclass": a.lclass, "comp": a.comp,
            "precision": a.precision, "quartets": nq, "device_s": times,
            "quartets_per_s": nq / min(times), "device_status": _lib.device_status()}


def stage_plan(meta, shift, stage_iter):
    """HFSCF's stages before the last (:6038-6098) as DHFSCF.run's `stages`:
    from the deck's starting stage (ILEV, :519-536) up to stage 2, each with
    its level shift SHLEV and HFSCF's energy tolerance (ENRGLV1 = 1e-8,
    ENRGLV2 = 5e-11, :5167-5168), and the shift of stage 3."""
    shifts = meta.get("shifts") or (shift, shift, shift)
    tols = {1: 1e-8, 2: 5e-11}
    start = int(meta.get("ilev", 1))
    plan = [(lv, shifts[lv - 1], tols[lv], stage_iter) for lv in (1, 2) if lv >= start]
    return plan, shifts[2]


def scf_main(a, b, meta=None):
    """Closed-shell DHF SCF of one molecule on the GPU (every step on the
    device), FP64 or mixed precision as --precision says.  With a deck:
    NCLS occupied spinors, its atoms' electron counts for the atomic start
    and, with --staged, its stages and level shifts."""
    from .scf import DHFSCF
    meta = meta or {}
    if meta.get("open_shell"):
        raise SystemExit("open-shell decks (NOPN > 0) need QDIR/QXCH, which are not built; "
                         "the SCF driver is closed-shell")
    nocc = a.nocc or int(meta.get("ncls") or round(sum(b.znuc)))
    stages, shift = None, a.shift
    if a.staged:
        stages, shift = stage_plan(meta, a.shift, a.stage_iter)
    s = DHFSCF(b, nocc, precision=a.precision, screen=a.screen or 1e-12,
               breit=False if a.no_breit else None, racah1=False)
    guess = None
    t0 = time.perf_counter()
    if a.wfn_in:
        from . import wfn
        guess = wfn.read_wfn(a.wfn_in, b.ndim)
    elif a.guess == "atomic":
        from .scf import atomic_guess
        guess = atomic_guess(b, nelec=meta.get("nelec"))
    t_guess = time.perf_counter() - t0
    r = s.run(etol=a.etol, max_iter=a.max_iter, ndiis=a.ndiis, shift=shift, mom=a.mom,
              guess=guess, wfn_out=a.wfn_out, dtol=a.dtol, stages=stages, verbose=a.verbose)
    r["guess"] = "wfn" if a.wfn_in else a.guess
    r["guess_s"] = t_guess
    s.close()
    hist = r.pop("history")
    r["orbital_energies"] = r["orbital_energies"][-4:]
    r.update({"case": a.case or a.deck, "ndim": b.ndim, "nocc": nocc,
              "precision": a.precision, "breit": not a.no_breit and b.hmlt >= deck.HMLT["DHFB"],
              "screen": a.screen or 1e-12, "shift": shift, "mom": a.mom, "ndiis": a.ndiis,
              "stages": stages, "iter_s": [h["s"] for h in hist],
              "ilev": [h["ilev"] for h in hist],
              "energies": [h["energy"] for h in hist]})
    return r


def atoms_main(a):
    """Batched Fock builds (and SCF) of a seeded draw of closed-shell atoms."""
    import torch

    from .fock import FockBatch
    from .scf import BatchedDHFSCF

    zset = [z for z in deck.CLOSED_SHELL_ATOMS if z <= a.zmax]
    bases = deck.batched_atoms(a.atoms, seed=a.seed, zset=zset)
    zs = [int(b.znuc[0]) for b in bases]
    if a.scf_only:
        s = BatchedDHFSCF(bases, zs, precision=a.precision, screen=a.screen or 1e-12)
        r = s.run(etol=a.etol, max_iter=a.max_iter, mom=a.mom, shift=a.shift)
        s.close()
        hist = r.pop("history")
        e = r.pop("energy")
        conv = r.pop("converged")
        r.update({"atoms": a.atoms, "precision": a.precision, "converged": int(sum(conv)),
                  "iter_s": [h["s"] for h in hist],
                  "max_abs_de": [h["max_abs_de"] for h in hist],
                  "energy_by_z": {str(z): v for z, v in zip(zs, e)},
                  "unconverged_z": sorted({z for z, c in zip(zs, conv) if not c})})
        return r
    out = {"atoms": a.atoms, "z_drawn_from": zset, "z": zs,
           "ndim": [b.ndim for b in bases], "screen": a.screen or 1e-12}
    screen = a.screen or 1e-12
    dens = [np.asarray(deck.density(b, seed=a.seed + k, nocc=z, real=True))
            for k, (b, z) in enumerate(zip(bases, zs))]
    D = torch.from_numpy(np.concatenate([d.ravel(order="F") for d in dens])).cuda()
    for prec in ("fp64", "df32", "auto"):
        t0 = time.perf_counter()
        fbs = []
        for b in bases:
            fb = FockBuilder(b, racah1=False)
            fb.set_precision(prec)
            fb.set_screening(screen)
            fbs.append(fb)
        batch = FockBatch(fbs)
        for fb in fbs:
            fb.close()
        t_init = time.perf_counter() - t0
        J, K = torch.zeros_like(D), torch.zeros_like(D)
        t0 = time.perf_counter()
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3)
        torch.cuda.synchronize()
        t_first = time.perf_counter() - t0
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        nq = batch.quartets()
        Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
        ej, ek, off = [], [], 0
        for d in dens:
            n = d.shape[0]
            ej.append(float(0.5 * np.sum(d * Jh[off:off + n * n].reshape(n, n, order="F")).real))
            ek.append(float(0.5 * np.sum(d * Kh[off:off + n * n].reshape(n, n, order="F")).real))
            off += n * n
        out[prec] = {"init_s": t_init, "first_call_s": t_first, "device_s": ms / 1e3,
                     "quartets": nq, "quartets_per_s": nq / (ms / 1e3),
                     "launches": batch.launches(), "energy_j_eh": ej, "energy_k_eh": ek}
        if prec == "auto":
            out[prec]["auto"] = batch.auto_stats()
        batch.close()
    for prec in ("df32", "auto"):
        out[prec + "_energy_max_abs_err_eh"] = max(
            max(abs(x - y) for x, y in zip(out["fp64"]["energy_j_eh"], out[prec]["energy_j_eh"])),
            max(abs(x - y) for x, y in zip(out["fp64"]["energy_k_eh"], out[prec]["energy_k_eh"])))
    for prec in ("fp64", "df32", "auto"):
        for key in ("energy_j_eh", "energy_k_eh"):
            out[prec][key] = out[prec][key][:8]  # keep the line short
    if a.scf:
        res = {}
        for prec in ("fp64", "df32"):
            s = BatchedDHFSCF(bases, zs, precision=prec, screen=screen)
            r = s.run(etol=1e-9, max_iter=80)
            s.close()
            r.pop("history")
            res[prec] = r
        de = [abs(x - y) for x, y in zip(res["fp64"]["energy"], res["df32"]["energy"])]
        out["scf"] = {
            "fp64": {k: v for k, v in res["fp64"].items() if k != "energy"},
            "df32": {k: v for k, v in res["df32"].items() if k != "energy"},
            "energy_fp64_by_z": {str(z): e for z, e in zip(zs, res["fp64"]["energy"])},
            "df32_vs_fp64_max_abs_eh": max(de),
            "all_converged": all(res["fp64"]["converged"]) and all(res["df32"]["converged"])}
        for prec in ("fp64", "df32"):
            out["scf"][prec]["converged"] = int(sum(out["scf"][prec]["converged"]))
    return out


def dataclasses_replace(b, hmlt):
    return deck.Basis(xyz=b.xyz, lmax=b.lmax, nfn=b.nfn, ex=b.ex, hmlt=hmlt, isym=b.isym,
                      znuc=b.znuc, name=b.name)


if __name__ == "__main__":
    main()
